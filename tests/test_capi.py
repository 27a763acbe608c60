"""The C-ABI library loads on a CPU-only machine and exports every function
that include/*.h declares (no compute calls without a GPU)."""
import ctypes
import re
from pathlib import Path

from conftest import ROOT

HEADER_DECL = re.compile(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*\**\s*([A-Za-z_][A-Za-z0-9_]*)\s*\(",
                         re.M)


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        txt = h.read_text()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        txt = re.sub(r"#[^\n]*", "", txt)
        for m in HEADER_DECL.finditer(txt):
            n = m.group(1)
            if n not in ("if", "while", "for", "return", "sizeof", "struct", "typedef"):
                names.add(n)
    return sorted(names)


def test_header_declares_reference_entry_points():
    names = declared_functions()
    for ref_name in ["acc_Deo", "acc_Doe", "fermion_matrix_multiplication", "fermion_matrix_multiplication_shifted",
                     "ker_invert_openacc", "multishift_invert", "recombine_shifted_vec3_to_vec3",
                     "l2norm2_global", "real_scal_prod_global", "scal_prod_global"]:
        assert ref_name in names


def declared_in(header):
    return [n for n in declared_functions() if re.search(r"\b%s\s*\(" % n, (ROOT / "include" / header).read_text())]


def test_library_exports_every_declared_symbol(built):
    from openstaple_gb300.native import BENCH_LIB_PATH, LIB_PATH
    L = ctypes.CDLL(str(LIB_PATH))
    missing = [n for n in declared_in("ostaple_gb300.h") if not hasattr(L, n)]
    assert not missing, f"declared but not exported: {missing}"
    # the measurement entry points live in the benchmark library only
    LB = ctypes.CDLL(str(BENCH_LIB_PATH))
    bench = declared_in("ostaple_gb300_bench.h")
    assert sorted(bench) == ["ostaple_probe_fma_tflops", "ostaple_time_kernel"]
    assert all(hasattr(LB, n) for n in bench)
    assert not any(hasattr(L, n) for n in bench)
    # the weak inverter_tricks global is exported too
    assert ctypes.c_int.in_dll(L, "inverter_tricks") is not None


def test_init_without_gpu_fails_cleanly(built):
    """Without a device the library reports an error instead of crashing."""
    import pytest
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    from openstaple_gb300.native import lib
    L = lib()
    rc = L.ostaple_init(4, 4, 4, 4)
    assert rc != 0
    assert b"no CUDA device" in L.ostaple_last_error()
    L.ostaple_clear_error()
    # odd extents are rejected before touching the device
    assert L.ostaple_init(5, 4, 4, 4) == -6
    L.ostaple_clear_error()


def test_host_switches_without_a_gpu(built):
    """The launch-shape autotuner and the sloppy-link format are host state:
    they can be set and read back on a machine without a GPU."""
    from openstaple_gb300 import api
    from openstaple_gb300.native import lib
    L = lib()
    assert api.autotune_report() == ""          # nothing tuned in this process
    api.autotune(False)
    api.autotune(2 + 3)                          # forced candidate (tests)
    api.autotune(True)
    assert api.autotune_report() == ""
    prev = api.set_sloppy_links("f32")
    assert prev == "q16"                         # the default
    assert api.set_sloppy_links("q16") == "f32"
    assert L.ostaple_set_sloppy_links(1) == 1
    import pytest
    with pytest.raises(ValueError):
        api.set_sloppy_links("fp16")
