"""Generates the golden vectors under tests/golden/ from the reference's own
compiled C code (oracle/_ref, built by oracle/Makefile.ref from the reference
source tree) and copies the coefficients of the two rational approximations
used by the benchmark configurations out of the reference's .REMEZ files.

Run from the repository root where the reference source tree is available
(its path as the first argument, or in OSTAPLE_REFERENCE), optionally naming
the fixture groups to write (default: all):

    python tests/golden/make_golden.py /path/to/reference [dirac] [gauge] [config2] [hmc] [rhmc] [remez]

* dirac   -- dirac_<dims>.npz: D_eo/D_oe, M^+M, CG, CG-M, eigenvalue bounds;
* gauge   -- gauge_<dims>_e<eps>.npz: staples, Q_A, stout levels,
  exp(-Q_A)U, Lambda, Sigma, the force outer products, the backfield and TA
  steps and a whole fermion_force_soloopenacc with two pseudofermions;
* config2 -- config2_16x16x16x16.npz: the 16^4 benchmark configuration
  (2 stout steps of rho = 0.15, m = 0.05, order-8 CG-M to 1e-10 per shift,
  the rational fermion force), at sampled sites;
* hmc     -- hmc_<dims>.npz: the pure-gauge tree-level Symanzik HMC pieces
  (gauge staples and force, plaquette and rectangle sums, 1/2 tr P^2, the
  momentum kick, the link update, two multistep_2MN_gauge calls);
* rhmc    -- rhmc_md_4x4x4x4.npz: the reference's multistep_2MN_SOLOOPENACC
  (molecular dynamics with a two-pseudofermion flavour and stout smearing);
* remez   -- remez_reference.json: every .REMEZ file the reference ships in
  its current format (full-precision header), the outputs of its
  multiprecision Remez program, for the library's own generator to match.

Inputs are regenerated from seeds by openstaple_gb300.fields, whose
counter-based generator is platform independent; the fixture also stores a
checksum of every input so a test can detect a generator change.
"""
from __future__ import annotations

import json
import os
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
    "fi_1_over_8": "tools/test/ratapproxes/approx_1_over_8_mlogerr_8.1_mloglm_6.2.REMEZ",
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


def approx_rescaled(approx: dict, key: str, lam_max: float = 64.0):
    """(a0, a, b) of a mother approximation on [lambda_min, 1] rescaled as
    rescale_rational_approximation() does for lambda_max (rationalapprox.c:
    145-194): scale = 1.05 * lambda_max."""
    ap = approx[key]
    mx = lam_max * 1.05
    eps = mx ** (ap["exponent_num"] / ap["exponent_den"])
    return ap["a0"] * eps, np.array(ap["a"]) * mx * eps, np.array(ap["b"]) * mx


def write_dirac(approx: dict) -> None:
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
        a0, a, b = approx_rescaled(approx, "order8")
        st, n, xs = r.cgm(u, ph, mass, a0, a, b, v, 1e-10, 10000)
        out.update(cgm_status=st, cgm_iters=n, cgm_xs=xs, cgm_recombined=r.recombine(xs, v, a0, a))
        # eigenvalue bounds (find_min_max.c:21-117) from the source as start vector
        mm, p, _ = r.find_min_max(u, ph, mass, v)
        mn, _, _ = r.find_min(u, ph, mass, v, mm[1])
        out.update(eig_minmax=mm, eig_p=p, eig_min=mn)
        tag = "x".join(map(str, dims))
        np.savez_compressed(HERE / f"dirac_{tag}.npz", **out)
        print("wrote", tag, "cg", out["cg_iters"], "cgm", out["cgm_iters"], "eig", mm, mn)


# (dims, link seed, link eps, sampling stride): eps = 0.01 keeps every c1 of
# the Cayley-Hamilton exponential below 4e-3 (the series branch)
GAUGE_CASES = [((4, 4, 4, 4), 101, 0.3, 1), ((4, 4, 4, 4), 102, 0.01, 2), ((4, 6, 8, 10), 103, 0.05, 15)]
GAUGE_RHO = 0.15
SIGMA_SEED, XS_SEED, PHI_SEED, FORCE_MASS = 18, 40, 52, 0.1


def gauge_inputs(dims, link_seed, eps):
    """The inputs of a gauge fixture, regenerated from seeds: links, a
    Sigma' field, four shift solutions X_k, two pseudofermions."""
    u = F.random_su3_links(dims, link_seed, eps=eps)
    sig = F.random_su3_links(dims, SIGMA_SEED, eps=1.0) * 0.7
    xs = np.stack([F.gaussian_vec3(dims, XS_SEED + k) for k in range(4)])
    phis = np.stack([F.gaussian_vec3(dims, PHI_SEED + k) for k in range(2)])
    return u, sig, xs, phis


FORCE_A = [0.31, 0.21, 0.11, 0.07]


def alg_index(sh: int, sites: np.ndarray) -> np.ndarray:
    """Indices, within one direction of a tamat_soa/thmat_soa array viewed
    as 8*sizeh doubles (c01, c02, c12 complex, then two real diagonals;
    struct_c_def.h:47-60), of the entries that belong to the given sites."""
    parts = []
    for k in range(3):
        parts.append(np.stack([k * 2 * sh + 2 * sites, k * 2 * sh + 2 * sites + 1], axis=1).ravel())
    for k in range(2):
        parts.append(6 * sh + k * sh + sites)
    return np.concatenate(parts)


def write_gauge(approx: dict) -> None:
    build.build_reference_oracles(sorted({c[0] for c in GAUGE_CASES}))
    a0, a8, b8 = approx_rescaled(approx, "order8")
    for dims, sl, eps, stride in GAUGE_CASES:
        r = Reference(dims)
        ph = r.phases()
        u, sig, xs, phis = gauge_inputs(dims, sl, eps)
        sites = np.arange(0, r.sizeh, stride)
        aidx = alg_index(r.sizeh, sites)

        def smp(f):
            return np.ascontiguousarray(f[..., sites])

        stap = r.staples(u)
        qa = r.rho_ta(u, stap, GAUGE_RHO)
        levels = r.stout_levels(u, 2, GAUGE_RHO)
        lam = r.lambda_(sig, u, qa)
        out = dict(dims=np.array(dims), link_seed=sl, eps=eps, rho=GAUGE_RHO, stride=stride, sites=sites, alg_idx=aidx,
                   u_checksum=checksum(u), sig_checksum=checksum(sig), xs_checksum=checksum(xs),
                   phi_checksum=checksum(phis), force_mass=FORCE_MASS, force_a=np.array(FORCE_A),
                   md_a=a8, md_b=b8)

        def smp_alg(f):
            return np.ascontiguousarray(f[:, aidx])

        out["staples"] = smp(stap)
        out["qa"] = smp_alg(qa)
        out["stout1"] = smp(levels[:8, :2])
        out["stout2"] = smp(levels[8:, :2])
        out["exp_qa_u"] = smp(r.exp_times_conf(u, qa)[:, :2])
        out["lambda"] = smp_alg(lam)
        out["sigma"] = smp(r.sigma(lam, u, sig, qa, GAUGE_RHO))
        out["sigma_prime_to_sigma"] = smp(r.sigma_prime_to_sigma(sig, u, GAUGE_RHO))
        aux = r.force_outer(u, xs, ph, FORCE_A)
        out["force_outer"] = smp(aux)
        pip = r.backfield_times_force(ph, aux, np.zeros_like(aux))
        out["backfield"] = smp(pip)
        out["conf_force_ta"] = smp_alg(r.conf_times_force_ta(u, pip, r.tamat()))
        out["fermion_force"] = smp_alg(r.fermion_force(u, ph, FORCE_MASS, a8, b8, phis, 1e-12))
        tag = "x".join(map(str, dims)) + f"_e{eps:g}"
        np.savez_compressed(HERE / f"gauge_{tag}.npz", **out)
        print("wrote gauge", tag)


# the 16^4 benchmark configuration: seeded exp(0.3 i H) links, 2 stout steps
# rho = 0.15, m = 0.05, one Gaussian source, order-8 x^(-1/4) to 1e-10 per
# shift, the rational fermion force; stored at every CONFIG2_STRIDE-th site
CONFIG2 = dict(dims=(16, 16, 16, 16), link_seed=21, src_seed=22, mass=0.05, rho=0.15, steps=2, res=1e-10)
CONFIG2_STRIDE = 61


def write_config2(approx: dict) -> None:
    c = CONFIG2
    dims = c["dims"]
    build.build_reference_oracles([dims])
    r = Reference(dims)
    ph = r.phases()
    u = F.random_su3_links(dims, c["link_seed"])
    phi = F.gaussian_vec3(dims, c["src_seed"])
    a0, a, b = approx_rescaled(approx, "order8")
    levels = r.stout_levels(u, c["steps"], c["rho"])
    u2 = np.ascontiguousarray(levels[8:])
    st, n, xs = r.cgm(u2, ph, c["mass"], a0, a, b, phi, c["res"], 10000)
    rec = r.recombine(xs, phi, a0, a)
    ipdot = r.fermion_force(u, ph, c["mass"], a, b, phi[None], c["res"], steps=c["steps"], rho=c["rho"])
    sites = np.arange(0, r.sizeh, CONFIG2_STRIDE)
    out = dict(dims=np.array(dims), sites=sites, u_checksum=checksum(u), src_checksum=checksum(phi),
               a0=a0, a=a, b=b, cgm_status=st, cgm_iters=n,
               stout2=np.ascontiguousarray(levels[8:, :2][..., sites]),
               cgm_xs=np.ascontiguousarray(xs[..., sites]), recombined=np.ascontiguousarray(rec[..., sites]),
               xs_norm2=np.array([checksum(x) for x in xs]),
               alg_idx=alg_index(r.sizeh, sites),
               fermion_force=np.ascontiguousarray(ipdot[:, alg_index(r.sizeh, sites)]))
    out.update({k: v for k, v in c.items() if k not in ("dims",)})
    np.savez_compressed(HERE / "config2_16x16x16x16.npz", **out)
    print("wrote config2: cgm", n, "iterations, status", st)


# pure-gauge tree-level Symanzik HMC pieces: (dims, link seed, eps, stride)
HMC_CASES = [((4, 4, 4, 4), 501, 0.5, 1), ((4, 6, 8, 10), 502, 0.3, 15)]
HMC_MOM = (61, 3)                       # momenta (seed, stream) of fields.gauge_momenta
HMC_MD = dict(beta=3.75, no_md=3, gauge_scale=2, t=1.0, ncalls=2)


def write_hmc(approx: dict) -> None:
    build.build_reference_oracles(sorted({c[0] for c in HMC_CASES}))
    for dims, sl, eps, stride in HMC_CASES:
        r = Reference(dims)
        u = F.random_su3_links(dims, sl, eps=eps)
        mom = F.gauge_momenta(dims, *HMC_MOM)
        sites = np.arange(0, r.sizeh, stride)
        aidx = alg_index(r.sizeh, sites)

        def smp(f):
            return np.ascontiguousarray(f[..., sites])

        def smp_alg(f):
            return np.ascontiguousarray(f[:, aidx])

        ip = r.ipdot_gauge(u)
        md = HMC_MD
        u2, m2 = r.gauge_2mn(u, mom, md["beta"], md["no_md"], md["gauge_scale"], md["t"], md["ncalls"])
        out = dict(dims=np.array(dims), link_seed=sl, eps=eps, stride=stride, sites=sites, alg_idx=aidx,
                   mom_seed=HMC_MOM[0], mom_stream=HMC_MOM[1], u_checksum=checksum(u),
                   mom_checksum=float(np.sum(mom ** 2)),
                   staples=smp(r.gauge_staples(u)), ipdot=smp_alg(ip),
                   plaq_sum=r.plaquette_sum(u), rect_sum=r.rectangle_sum(u), mom_action=r.momenta_action(mom),
                   mom_sum_mult=smp_alg(r.mom_sum_mult(mom, ip, -0.02)),
                   mom_exp=smp(r.mom_exp_times_conf(u, mom, 0.05)[:, :2]),
                   deltas=r.md_deltas(md["beta"], md["no_md"], md["gauge_scale"], md["t"]),
                   md_u=smp(u2[:, :2]), md_mom=smp_alg(m2), **{f"md_{k}": v for k, v in md.items()})
        tag = "x".join(map(str, dims))
        np.savez_compressed(HERE / f"hmc_{tag}.npz", **out)
        print("wrote hmc", tag)


# molecular dynamics with fermions: one flavour, two pseudofermions chi,
# order-8 x^(-1/4) approx_md, stout 2 x 0.15
RHMC_MD = dict(dims=(4, 4, 4, 4), link_seed=701, eps=0.3, mom=(702, 0), chi_seeds=(703, 704), mass=0.1, res=1e-12,
               beta=3.75, no_md=2, gauge_scale=2, t=1.0, steps=2, rho=0.15)


def write_rhmc(approx: dict) -> None:
    c = RHMC_MD
    dims = c["dims"]
    build.build_reference_oracles([dims])
    r = Reference(dims)
    ph = r.phases()
    u = F.random_su3_links(dims, c["link_seed"], eps=c["eps"])
    mom = F.gauge_momenta(dims, *c["mom"])
    chis = np.stack([F.gaussian_vec3(dims, k) for k in c["chi_seeds"]])
    a0, a, b = approx_rescaled(approx, "order8")
    ur, mr = r.rhmc_md(u, mom, ph, c["mass"], a, b, chis, c["res"], c["beta"], c["no_md"], c["gauge_scale"], c["t"],
                       c["steps"], c["rho"])
    out = dict(u_checksum=checksum(u), mom_checksum=float(np.sum(mom ** 2)), chi_checksum=checksum(chis),
               a=a, b=b, md_u=np.ascontiguousarray(ur[:, :2]), md_mom=mr)
    out.update({k: np.array(v) for k, v in c.items()})
    np.savez_compressed(HERE / "rhmc_md_4x4x4x4.npz", **out)
    print("wrote rhmc md")


def write_remez(ref: Path) -> None:
    out = {}
    for path in sorted([*ref.glob("saved_approxs/*.REMEZ"), *ref.glob("tools/test/ratapproxes/*.REMEZ")]):
        txt = path.read_text()
        if not re.search(r"Lambda Min:\s*[-+0-9.]+e", txt):   # the older fixed-point header
            continue
        d = parse_remez(path)
        if d["error"] <= 0:
            continue
        out[str(path.relative_to(ref))] = d
    (HERE / "remez_reference.json").write_text(json.dumps(out, indent=1))
    print("wrote remez", len(out))


def main(refroot: str, groups) -> None:
    ref = Path(refroot)
    os.environ["OSTAPLE_REFERENCE"] = str(ref)
    approx = {k: parse_remez(ref / v) for k, v in APPROX_FILES.items()}
    (HERE / "ratapprox.json").write_text(json.dumps(approx, indent=1))
    if "dirac" in groups:
        write_dirac(approx)
    if "gauge" in groups:
        write_gauge(approx)
    if "config2" in groups:
        write_config2(approx)
    if "hmc" in groups:
        write_hmc(approx)
    if "remez" in groups:
        write_remez(ref)
    if "rhmc" in groups:
        write_rhmc(approx)


if __name__ == "__main__":
    args = sys.argv[1:]
    root = args.pop(0) if args and not args[0] in ("dirac", "gauge", "config2", "hmc", "rhmc", "remez") else os.environ.get(
        "OSTAPLE_REFERENCE")
    if not root:
        sys.exit("usage: make_golden.py /path/to/reference [dirac] [gauge] [config2] [hmc] [rhmc] [remez]")
    main(root, set(args) or {"dirac", "gauge", "config2", "hmc", "rhmc", "remez"})
