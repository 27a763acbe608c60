"""Generates the golden vectors under tests/golden/ from the reference's own
compiled C code (oracle/_ref, built by oracle/Makefile.ref from the reference
source tree) and copies the coefficients of the two rational approximations
used by the benchmark configurations out of the reference's .REMEZ files.

Run from the repository root where the reference source tree is available:

    python tests/golden/make_golden.py [/path/to/reference]

Inputs are regenerated from seeds by openstaple_gb300.fields, whose
counter-based generator is platform independent; the fixture also stores a
checksum of every input so a test can detect a generator change.
"""
from __future__ import annotations

import json
import re
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from openstaple_gb300 import build, fields as F  # noqa: E402
from oracle import Reference  # noqa: E402

HERE = Path(__file__).resolve().parent

# (dims, link seed, source seed, mass, link smearing eps)
CASES = [((4, 4, 4, 4), 11, 5, 0.1), ((4, 6, 8, 10), 12, 6, 0.05), ((8, 8, 8, 8), 13, 7, 0.1)]
APPROX_FILES = {
    "order8": "tools/test/ratapproxes/approx_-1_over_4_mlogerr_3.8_mloglm_6.2.REMEZ",
    "order19": "saved_approxs/approx_-1_over_4_order_19_mloglm_6.4.REMEZ",
}


def parse_remez(path: Path) -> dict:
    """Reads the reference's .REMEZ text format (rationalapprox.c:83-117)."""
    txt = path.read_text()
    num, den = map(int, re.search(r"\(x\)\^\((-?\d+)/(\d+)\)", txt).groups())
    order = int(re.search(r"Order:\s*(\d+)", txt).group(1))
    lmin = float(re.search(r"Lambda Min:\s*([-+0-9.eE]+)", txt).group(1))
    lmax = float(re.search(r"Lambda Max:\s*([-+0-9.eE]+)", txt).group(1))
    err = float(re.search(r"Error:\s*([-+0-9.eE]+)", txt).group(1))
    a0 = float(re.search(r"RA_a0 = ([-+0-9.eE]+)", txt).group(1))
    pairs = re.findall(r"RA_a\[(\d+)\] = ([-+0-9.eE]+), RA_b\[\d+\] = ([-+0-9.eE]+)", txt)
    a = [float(p[1]) for p in pairs]
    b = [float(p[2]) for p in pairs]
    assert len(a) == order
    return dict(exponent_num=num, exponent_den=den, order=order, lambda_min=lmin, lambda_max=lmax, error=err,
                a0=a0, a=a, b=b)


def checksum(x: np.ndarray) -> float:
    return float(np.sum(np.abs(x.astype(np.complex128)) ** 2))


def main(refroot: str) -> None:
    ref = Path(refroot)
    approx = {k: parse_remez(ref / v) for k, v in APPROX_FILES.items()}
    (HERE / "ratapprox.json").write_text(json.dumps(approx, indent=1))

    build.build_reference_oracles([c[0] for c in CASES])
    for dims, sl, ss, mass in CASES:
        r = Reference(dims)
        ph = r.phases()
        u = F.random_su3_links(dims, sl)
        v = F.gaussian_vec3(dims, ss)
        out = dict(dims=np.array(dims), link_seed=sl, src_seed=ss, mass=mass,
                   u_checksum=checksum(u), src_checksum=checksum(v))
        out["Deo"] = r.Deo(u, v, ph)
        out["Doe"] = r.Doe(u, v, ph)
        out["mdagm"] = r.mdagm(u, v, ph, mass, 0.0)
        out["mdagm_shift"] = r.mdagm(u, v, ph, mass, 0.37)
        st, n, x = r.cg(u, ph, mass, v, 1e-10, 10000, 0.0, 10000)
        out.update(cg_status=st, cg_iters=n, cg_x=x)
        ap = approx["order8"]
        # rescaled as rescale_rational_approximation() does for lambda_max = 64
        # (rationalapprox.c:145-194): scale = 1.05 * max
        mx = 64.0 * 1.05
        eps = mx ** (ap["exponent_num"] / ap["exponent_den"])
        a0 = ap["a0"] * eps
        a = np.array(ap["a"]) * mx * eps
        b = np.array(ap["b"]) * mx
        st, n, xs = r.cgm(u, ph, mass, a0, a, b, v, 1e-10, 10000)
        out.update(cgm_status=st, cgm_iters=n, cgm_xs=xs, cgm_recombined=r.recombine(xs, v, a0, a))
        # eigenvalue bounds (find_min_max.c:21-117) from the source as start vector
        mm, p, _ = r.find_min_max(u, ph, mass, v)
        mn, _, _ = r.find_min(u, ph, mass, v, mm[1])
        out.update(eig_minmax=mm, eig_p=p, eig_min=mn)
        tag = "x".join(map(str, dims))
        np.savez_compressed(HERE / f"dirac_{tag}.npz", **out)
        print("wrote", tag, "cg", out["cg_iters"], "cgm", out["cgm_iters"], "eig", mm, mn)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
