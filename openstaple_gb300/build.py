"""Builds the in-tree native libraries.

* ``openstaple_gb300/libostaple_gb300.so`` -- the CUDA hot path for sm_103a,
  compiled with nvcc (one translation unit per kernel family, compiled in
  parallel, linked as a plain shared library with a C ABI).
* ``openstaple_gb300/libostaple_gb300_bench.so`` -- the benchmark's
  measurement entry points (``csrc/bench/``), linked against the library.
* ``oracle/liboracle.so`` -- the CPU restatement used by the tests as the
  parity checker (plain C, gcc, OpenMP).
* ``oracle/_ref/libref_<dims>.so`` -- the reference's own C sources compiled
  per lattice size, only where the reference source tree is available.

Everything is rebuilt only when a source is newer than its output.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = ROOT / "_build"
LIB = PKG / "libostaple_gb300.so"
BENCH_LIB = PKG / "libostaple_gb300_bench.so"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "liboracle.so"
REF_OUT = ORACLE_DIR / "_ref"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
              "--expt-relaxed-constexpr", "-I", str(ROOT / "include")]

# lattice sizes for which the reference is compiled as a test oracle
REF_DIMS = [(4, 4, 4, 4), (8, 8, 8, 8), (4, 6, 8, 10), (16, 16, 16, 16)]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build openstaple_gb300")


def _newer(srcs, out: Path) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(s).stat().st_mtime > t for s in srcs)


def _run(cmd, cwd=None):
    p = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"command failed ({p.returncode}): {' '.join(map(str, cmd))}\n{p.stdout}")
    return p.stdout


def build_library(verbose: bool = False) -> Path:
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    sources = sorted(CSRC.glob("*.cu"))
    jobs = []
    objs = []
    for src in sources:
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if _newer([src, *headers], obj):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            outs = list(ex.map(_run, jobs))
        if verbose:
            for o in outs:
                if o.strip():
                    print(o)
    if jobs or _newer(objs, LIB):
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"])
    return LIB


def build_bench_library(verbose: bool = False) -> Path:
    nvcc = _nvcc()
    srcs = sorted((CSRC / "bench").glob("*.cu"))
    headers = list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    if _newer([*srcs, *headers, LIB], BENCH_LIB):
        _run([nvcc, *ARCH, *NVCC_FLAGS, "-shared", "-o", str(BENCH_LIB), *map(str, srcs),
              "-L", str(PKG), "-lostaple_gb300", "-Xlinker", "-rpath,$ORIGIN", "-lcudart"])
    return BENCH_LIB


def build_oracle(verbose: bool = False) -> Path:
    srcs = sorted(ORACLE_DIR.glob("*.c"))
    srcs = [s for s in srcs if s.name != "ref_harness.c"]
    hdrs = list(ORACLE_DIR.glob("*.h"))
    if srcs and _newer([*srcs, *hdrs], ORACLE_LIB):
        cc = os.environ.get("CC", "gcc")
        _run([cc, "-O3", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-o", str(ORACLE_LIB),
              *map(str, srcs), "-lm"])
    return ORACLE_LIB


def reference_root() -> Path | None:
    root = Path(os.environ.get("OSTAPLE_REFERENCE", "/root/reference"))
    return root if (root / "src" / "OpenAcc" / "fermion_matrix.c").exists() else None


def build_reference_oracles(dims=REF_DIMS, verbose: bool = False) -> list[Path]:
    ref = reference_root()
    if ref is None:
        return []
    mk = ORACLE_DIR / "Makefile.ref"

    def one(d):
        _run(["make", "-s", "-f", str(mk), f"REFROOT={ref}", "DIMS=" + " ".join(map(str, d))], cwd=str(ROOT))
        return REF_OUT / ("libref_" + "x".join(map(str, d)) + ".so")

    with cf.ThreadPoolExecutor(max_workers=min(len(dims), os.cpu_count() or 4)) as ex:
        return list(ex.map(one, dims))


def build_all(verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        futs = [ex.submit(build_library, verbose), ex.submit(build_oracle, verbose),
                ex.submit(build_reference_oracles, REF_DIMS, verbose)]
        for f in futs:
            f.result()
    build_bench_library(verbose)


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
    print("built", LIB)
