"""Pins the CPU oracle (oracle/ostaple_oracle.c) to the reference.

* against the golden vectors produced by the reference's own compiled C code
  (tests/golden/, made by tests/golden/make_golden.py);
* against the reference compiled from source (oracle/_ref) where it is
  available (this is skipped on machines without the reference tree).
"""
import numpy as np
import pytest

from conftest import load_golden, relerr
from openstaple_gb300 import fields as F

GOLDEN_TAGS = ["4x4x4x4", "4x6x8x10", "8x8x8x8"]


def _inputs(g):
    dims = tuple(int(d) for d in g["dims"])
    u = F.random_su3_links(dims, int(g["link_seed"]))
    v = F.gaussian_vec3(dims, int(g["src_seed"]))
    # the generator must still produce the fixture's inputs
    assert np.isclose(np.sum(np.abs(u) ** 2), float(g["u_checksum"]), rtol=1e-14)
    assert np.isclose(np.sum(np.abs(v) ** 2), float(g["src_checksum"]), rtol=1e-14)
    return dims, u, v


@pytest.mark.parametrize("tag", GOLDEN_TAGS)
def test_oracle_matches_golden_dirac(built, tag):
    from oracle import Oracle
    g = load_golden(tag)
    dims, u, v = _inputs(g)
    o = Oracle(dims)
    ph = o.phases()
    assert np.array_equal(ph, F.staggered_phases(dims))
    assert relerr(o.Deo(u, v, ph), g["Deo"]) <= 1e-15
    assert relerr(o.Doe(u, v, ph), g["Doe"]) <= 1e-15
    m = float(g["mass"])
    assert relerr(o.mdagm(u, v, ph, m * m), g["mdagm"]) <= 1e-14
    assert relerr(o.mdagm(u, v, ph, m * m + 0.37), g["mdagm_shift"]) <= 1e-14


@pytest.mark.parametrize("tag", GOLDEN_TAGS)
def test_oracle_matches_golden_solvers(built, tag):
    import json
    from conftest import GOLDEN
    from oracle import Oracle
    g = load_golden(tag)
    dims, u, v = _inputs(g)
    o = Oracle(dims)
    ph = o.phases()
    m = float(g["mass"])
    st, n, x = o.cg(u, ph, m, v, 1e-10)
    assert st == int(g["cg_status"]) == 1
    assert n == int(g["cg_iters"])
    assert relerr(x, g["cg_x"]) <= 1e-12
    ap = json.loads((GOLDEN / "ratapprox.json").read_text())["order8"]
    mx = 64.0 * 1.05
    eps = mx ** (ap["exponent_num"] / ap["exponent_den"])
    a0, a, b = ap["a0"] * eps, np.array(ap["a"]) * mx * eps, np.array(ap["b"]) * mx
    st, n, xs = o.cgm(u, ph, m, b, v, 1e-10)
    assert st == int(g["cgm_status"]) == 1
    assert n == int(g["cgm_iters"])
    assert relerr(xs, g["cgm_xs"]) <= 1e-12
    assert relerr(o.recombine(xs, v, a0, a), g["cgm_recombined"]) <= 1e-12


@pytest.mark.parametrize("tag", GOLDEN_TAGS)
def test_oracle_matches_golden_eigenvalue_bounds(built, tag):
    from oracle import Oracle
    g = load_golden(tag)
    dims, u, v = _inputs(g)
    o = Oracle(dims)
    ph = o.phases()
    m = float(g["mass"])
    mx, loops, p, _ = o.find_max(u, ph, m, v)
    assert loops > 1
    assert g["eig_minmax"][0] == m * m
    assert abs(mx - g["eig_minmax"][1]) <= 1e-13 * mx
    assert relerr(p, g["eig_p"]) <= 1e-12
    mn, _, _, _ = o.find_min(u, ph, m, v, mx)
    assert abs(mn - float(g["eig_min"])) <= 1e-12 * abs(mn)


REF_DIMS = [(4, 4, 4, 4), (8, 8, 8, 8), (4, 6, 8, 10)]


@pytest.mark.parametrize("dims", REF_DIMS)
def test_oracle_matches_compiled_reference(built, dims):
    from oracle import Oracle, Reference, ref_available
    if not ref_available(dims):
        pytest.skip("reference not compiled here (no reference source tree)")
    r, o = Reference(dims), Oracle(dims)
    ph = r.phases()
    assert np.array_equal(o.phases(), ph)
    u = F.random_su3_links(dims, 101)
    v = F.gaussian_vec3(dims, 102)
    # same arithmetic up to the compiler's FMA contraction choices
    assert relerr(o.Deo(u, v, ph), r.Deo(u, v, ph)) <= 2e-16
    assert relerr(o.Doe(u, v, ph), r.Doe(u, v, ph)) <= 2e-16
    # a generic (imaginary chemical potential) phase exercises the cos/sin path
    ph2 = r.phases(0.3)
    assert np.array_equal(o.phases(0.3), ph2)
    assert relerr(o.Deo(u, v, ph2), r.Deo(u, v, ph2)) <= 1e-15
    st1, n1, x1 = o.cg(u, ph, 0.05, v, 1e-10, restart=40)
    st2, n2, x2 = r.cg(u, ph, 0.05, v, 1e-10, restart=40)
    assert (st1, n1) == (st2, n2)
    assert relerr(x1, x2) <= 1e-12
    mm, p2, _ = r.find_min_max(u, ph, 0.05, v)
    mx, _, p1, _ = o.find_max(u, ph, 0.05, v)
    assert mm[0] == 0.05 * 0.05
    assert abs(mx - mm[1]) <= 1e-13 * mx
    assert relerr(p1, p2) <= 1e-12


def test_oracle_cg_max_iterations_failure(built):
    """max_cg exhaustion reports INVERTER_FAILURE like the reference."""
    from oracle import Oracle
    dims = (4, 4, 4, 4)
    o = Oracle(dims)
    ph = o.phases()
    u = F.random_su3_links(dims, 3)
    v = F.gaussian_vec3(dims, 4)
    st, n, _ = o.cg(u, ph, 0.1, v, 1e-10, max_cg=5, restart=5)
    assert st == 0 and n == 5


# ---- stout smearing and the fermion force chain ---------------------------
# Tolerances (relative, max-norm): 1e-14 for the staples, Q_A, the stout
# exponential and the outer products; 5e-14 for Lambda and the Sigma chain,
# whose Cayley-Hamilton derivative coefficients divide by (9u^2 - w^2)^2;
# 1e-12 for a whole force, which includes two multi-shift solves to 1e-12.

GAUGE_TAGS = ["4x4x4x4_e0.3", "4x4x4x4_e0.01", "4x6x8x10_e0.05"]


from conftest import load_gauge_fixture as _gauge_fixture  # noqa: E402
from conftest import sample_alg as _smp_alg  # noqa: E402
from conftest import sample_sites as _smp  # noqa: E402


@pytest.mark.parametrize("dims", REF_DIMS)
@pytest.mark.parametrize("eps", [0.3, 0.01])
def test_oracle_gauge_chain_matches_compiled_reference(built, dims, eps):
    """Staples, Q_A, two stout levels, exp(-Q_A) U, Lambda, Sigma, the
    Sigma' -> Sigma step, the outer products, the backfield and the TA
    projection: the oracle against the reference's own compiled C
    (stouting.c:27-1302, plaquettes.c:196-259, fermion_force_utilities.c:
    30-153).  eps = 0.01 puts every link in the c1 < 4e-3 series branch of
    the exponential (cayley_hamilton.h:67-72)."""
    from oracle import Oracle, Reference, ref_available
    if not ref_available(dims):
        pytest.skip("reference not compiled here (no reference source tree)")
    r, o = Reference(dims), Oracle(dims)
    u = F.random_su3_links(dims, 201, eps=eps)
    sig = F.random_su3_links(dims, 202, eps=1.0) * 0.7
    ph = r.phases()
    stap = r.staples(u)
    assert relerr(o.staples(u), stap) <= 1e-14
    qa = r.rho_ta(u, stap, 0.15)
    assert relerr(o.rho_ta(u, stap, 0.15), qa) <= 1e-14
    lv = r.stout_levels(u, 2, 0.15)
    l1 = o.stout(u, 0.15)
    assert relerr(l1[:, :2], lv[:8, :2]) <= 1e-14
    assert relerr(o.stout(l1, 0.15)[:, :2], lv[8:, :2]) <= 1e-14
    assert relerr(o.exp_times_conf(u, qa)[:, :2], r.exp_times_conf(u, qa)[:, :2]) <= 1e-14
    lam = r.lambda_(sig, u, qa)
    assert relerr(o.lambda_(sig, u, qa), lam) <= 5e-14
    assert relerr(o.sigma(lam, u, sig, qa, 0.15), r.sigma(lam, u, sig, qa, 0.15)) <= 5e-14
    assert relerr(o.sigma_prime_to_sigma(sig, u, 0.15), r.sigma_prime_to_sigma(sig, u, 0.15)) <= 5e-14
    xs = np.stack([F.gaussian_vec3(dims, 210 + k) for k in range(3)])
    a = [0.5, 0.25, 0.125]
    aux = r.force_outer(u, xs, ph, a)
    assert relerr(o.force_outer(u, xs, ph, a), aux) <= 1e-14
    pip = r.backfield_times_force(ph, aux, sig)
    assert relerr(o.backfield_times_force(ph, aux, sig), pip) <= 1e-14
    t0 = r.tamat()
    assert relerr(o.conf_times_force_ta(u, pip, t0), r.conf_times_force_ta(u, pip, t0)) <= 1e-14


def _oracle_force(o, u, ph, mass, a, b, phis, res, rho=0.15):
    """The fermion_force_soloopenacc chain (fermion_force.c:166-320) from
    oracle pieces: two stout levels, one CG-M per pseudofermion with
    approx_md, outer products, phases, Sigma' -> Sigma per level, -TA(U Sigma)."""
    u1 = o.stout(u, rho)
    u2 = o.stout(u1, rho)
    aux = o.su3()
    for phi in phis:
        st, n, xs = o.cgm(u2, ph, mass, b, np.ascontiguousarray(phi), res)
        assert st == 1
        aux += o.force_outer(u2, xs, ph, a)
    sig = o.backfield_times_force(ph, aux, np.zeros_like(aux))
    sig = o.sigma_prime_to_sigma(sig, u1, rho)
    sig = o.sigma_prime_to_sigma(sig, u, rho)
    return o.conf_times_force_ta(u, sig, o.tamat())


@pytest.mark.parametrize("dims", [(4, 4, 4, 4), (4, 6, 8, 10)])
def test_oracle_fermion_force_matches_compiled_reference(built, dims):
    """A whole fermion_force_soloopenacc (2 stout levels, two pseudofermions,
    order-8 approx_md) run by the reference's own compiled code against the
    oracle chain."""
    import json
    from conftest import GOLDEN
    from oracle import Oracle, Reference, ref_available
    if not ref_available(dims):
        pytest.skip("reference not compiled here (no reference source tree)")
    r, o = Reference(dims), Oracle(dims)
    ap = json.loads((GOLDEN / "ratapprox.json").read_text())["order8"]
    mx = 64.0 * 1.05
    e = mx ** (ap["exponent_num"] / ap["exponent_den"])
    a, b = np.array(ap["a"]) * mx * e, np.array(ap["b"]) * mx
    u = F.random_su3_links(dims, 221, eps=0.3)
    ph = r.phases()
    phis = np.stack([F.gaussian_vec3(dims, 222), F.gaussian_vec3(dims, 223)])
    ip_r = r.fermion_force(u, ph, 0.1, a, b, phis, 1e-12)
    assert relerr(_oracle_force(o, u, ph, 0.1, a, b, phis, 1e-12), ip_r) <= 1e-12


@pytest.mark.parametrize("tag", GAUGE_TAGS)
def test_oracle_matches_golden_gauge(built, tag):
    """The oracle against the gauge fixtures that the compiled reference
    wrote (tests/golden/make_golden.py), on every machine."""
    from oracle import Oracle
    g, dims, u, sig, xs, phis = _gauge_fixture(tag)
    o = Oracle(dims)
    ph = o.phases()
    rho = float(g["rho"])
    stap = o.staples(u)
    assert relerr(_smp(stap, g), g["staples"]) <= 1e-14
    qa = o.rho_ta(u, stap, rho)
    assert relerr(_smp_alg(qa, g), g["qa"]) <= 1e-14
    l1 = o.stout(u, rho)
    assert relerr(_smp(l1[:, :2], g), g["stout1"]) <= 1e-14
    assert relerr(_smp(o.stout(l1, rho)[:, :2], g), g["stout2"]) <= 1e-14
    assert relerr(_smp(o.exp_times_conf(u, qa)[:, :2], g), g["exp_qa_u"]) <= 1e-14
    lam = o.lambda_(sig, u, qa)
    assert relerr(_smp_alg(lam, g), g["lambda"]) <= 5e-14
    assert relerr(_smp(o.sigma(lam, u, sig, qa, rho), g), g["sigma"]) <= 5e-14
    assert relerr(_smp(o.sigma_prime_to_sigma(sig, u, rho), g), g["sigma_prime_to_sigma"]) <= 5e-14
    aux = o.force_outer(u, xs, ph, g["force_a"])
    assert relerr(_smp(aux, g), g["force_outer"]) <= 1e-14
    pip = o.backfield_times_force(ph, aux, np.zeros_like(aux))
    assert relerr(_smp(pip, g), g["backfield"]) <= 1e-14
    assert relerr(_smp_alg(o.conf_times_force_ta(u, pip, o.tamat()), g), g["conf_force_ta"]) <= 1e-14
    ip = _oracle_force(o, u, ph, float(g["force_mass"]), g["md_a"], g["md_b"], phis, 1e-12, rho)
    assert relerr(_smp_alg(ip, g), g["fermion_force"]) <= 1e-12


def test_oracle_matches_golden_config2(built):
    """The 16^4 benchmark configuration (2 stout steps of rho = 0.15,
    m = 0.05, order-8 CG-M to 1e-10 per shift, the rational force) against
    the compiled reference's outputs at sampled sites: same CG-M iteration
    count, solutions within 1e-12, force within 1e-11."""
    from conftest import GOLDEN
    from oracle import Oracle
    g = dict(np.load(GOLDEN / "config2_16x16x16x16.npz"))
    dims = tuple(int(d) for d in g["dims"])
    u = F.random_su3_links(dims, int(g["link_seed"]))
    phi = F.gaussian_vec3(dims, int(g["src_seed"]))
    assert np.isclose(np.sum(np.abs(u) ** 2), float(g["u_checksum"]), rtol=1e-14)
    assert np.isclose(np.sum(np.abs(phi) ** 2), float(g["src_checksum"]), rtol=1e-14)
    o = Oracle(dims, threads=8)
    ph = o.phases()
    rho, mass, res = float(g["rho"]), float(g["mass"]), float(g["res"])
    u1 = o.stout(u, rho)
    u2 = o.stout(u1, rho)
    assert relerr(_smp(u2[:, :2], g), g["stout2"]) <= 1e-14
    st, n, xs = o.cgm(u2, ph, mass, g["b"], phi, res)
    assert st == int(g["cgm_status"]) == 1
    assert n == int(g["cgm_iters"])
    assert relerr(_smp(xs, g), g["cgm_xs"]) <= 1e-12
    assert relerr(_smp(o.recombine(xs, phi, float(g["a0"]), g["a"]), g), g["recombined"]) <= 1e-12
    ip = _oracle_force(o, u, ph, mass, g["a"], g["b"], phi[None], res, rho)
    assert relerr(_smp_alg(ip, g), g["fermion_force"]) <= 1e-11


# ---- pure-gauge tree-level Symanzik HMC ------------------------------------
# Tolerances: 1e-14 relative (max-norm) for the staples, the force, the
# momentum kick and the link update; 1e-13 relative for the plaquette,
# rectangle and momentum sums; 1e-12 after two gauge multisteps (18 force
# evaluations and link updates in sequence).

HMC_TAGS = ["4x4x4x4", "4x6x8x10"]


def _hmc_fixture(tag):
    from conftest import GOLDEN
    g = dict(np.load(GOLDEN / f"hmc_{tag}.npz"))
    dims = tuple(int(d) for d in g["dims"])
    u = F.random_su3_links(dims, int(g["link_seed"]), eps=float(g["eps"]))
    mom = F.gauge_momenta(dims, int(g["mom_seed"]), int(g["mom_stream"]))
    assert np.isclose(np.sum(np.abs(u) ** 2), float(g["u_checksum"]), rtol=1e-14)
    assert np.isclose(np.sum(mom ** 2), float(g["mom_checksum"]), rtol=1e-14)
    return g, dims, u, mom


@pytest.mark.parametrize("dims", REF_DIMS)
def test_oracle_gauge_hmc_matches_compiled_reference(built, dims):
    """Staples and force of the tree-level Symanzik action, plaquette and
    rectangle sums, 1/2 tr P^2, the momentum kick, the link update and two
    gauge multisteps of the 2MN integrator: the oracle against the
    reference's own compiled ipdot_gauge.c, plaquettes.c, rectangles.c,
    su3_utilities.c, su3_measurements.c, md_integrator.c, md_parameters.c."""
    from oracle import Oracle, Reference, ref_available
    if not ref_available(dims):
        pytest.skip("reference not compiled here (no reference source tree)")
    r, o = Reference(dims), Oracle(dims)
    u = F.random_su3_links(dims, 601, eps=0.4)
    mom = F.gauge_momenta(dims, 602, 1)
    assert relerr(o.gauge_staples(u), r.gauge_staples(u)) <= 1e-14
    ip = r.ipdot_gauge(u)
    assert relerr(o.ipdot_gauge(u), ip) <= 1e-14
    assert abs(o.plaquette_sum(u) - r.plaquette_sum(u)) <= 1e-13 * abs(r.plaquette_sum(u))
    assert abs(o.rectangle_sum(u) - r.rectangle_sum(u)) <= 1e-13 * abs(r.rectangle_sum(u))
    assert abs(o.momenta_action(mom) - r.momenta_action(mom)) <= 1e-13 * r.momenta_action(mom)
    assert relerr(o.mom_sum_mult(mom, ip, -0.03), r.mom_sum_mult(mom, ip, -0.03)) <= 1e-14
    assert relerr(o.mom_exp_times_conf(u, mom, 0.05)[:, :2], r.mom_exp_times_conf(u, mom, 0.05)[:, :2]) <= 1e-14
    assert np.array_equal(o.md_deltas(3.75, 18, 4, 1.0), r.md_deltas(3.75, 18, 4, 1.0))
    uo, mo = o.gauge_2mn(u, mom, 3.75, 2, 3, 1.0, 2)
    ur, mr = r.gauge_2mn(u, mom, 3.75, 2, 3, 1.0, 2)
    assert relerr(uo[:, :2], ur[:, :2]) <= 1e-12
    assert relerr(mo, mr) <= 1e-12


@pytest.mark.parametrize("tag", HMC_TAGS)
def test_oracle_matches_golden_hmc(built, tag):
    from oracle import Oracle
    g, dims, u, mom = _hmc_fixture(tag)
    o = Oracle(dims)
    ip = o.ipdot_gauge(u)
    assert relerr(_smp(o.gauge_staples(u), g), g["staples"]) <= 1e-14
    assert relerr(_smp_alg(ip, g), g["ipdot"]) <= 1e-14
    assert abs(o.plaquette_sum(u) - float(g["plaq_sum"])) <= 1e-13 * abs(float(g["plaq_sum"]))
    assert abs(o.rectangle_sum(u) - float(g["rect_sum"])) <= 1e-13 * abs(float(g["rect_sum"]))
    assert abs(o.momenta_action(mom) - float(g["mom_action"])) <= 1e-13 * float(g["mom_action"])
    assert relerr(_smp_alg(o.mom_sum_mult(mom, ip, -0.02), g), g["mom_sum_mult"]) <= 1e-14
    assert relerr(_smp(o.mom_exp_times_conf(u, mom, 0.05)[:, :2], g), g["mom_exp"]) <= 1e-14
    uo, mo = o.gauge_2mn(u, mom, float(g["md_beta"]), int(g["md_no_md"]), int(g["md_gauge_scale"]),
                         float(g["md_t"]), int(g["md_ncalls"]))
    assert relerr(_smp(uo[:, :2], g), g["md_u"]) <= 1e-12
    assert relerr(_smp_alg(mo, g), g["md_mom"]) <= 1e-12


def test_oracle_fermion_md_matches_golden(built):
    """The reference's multistep_2MN_SOLOOPENACC (molecular dynamics with a
    two-pseudofermion flavour, stout 2 x 0.15) restated from oracle pieces:
    F(d0) [G F(d1) G F(d2)]^(no_md-1) G F(d1) G F(d0), F the fermion force
    kick and G one gauge multistep (md_integrator.c:502-742).  Links and
    momenta within 1e-12."""
    from conftest import GOLDEN
    from oracle import Oracle
    g = dict(np.load(GOLDEN / "rhmc_md_4x4x4x4.npz"))
    dims = tuple(int(d) for d in g["dims"])
    o = Oracle(dims)
    u = F.random_su3_links(dims, int(g["link_seed"]), eps=float(g["eps"]))
    mom = F.gauge_momenta(dims, *[int(v) for v in g["mom"]])
    chis = np.stack([F.gaussian_vec3(dims, int(k)) for k in g["chi_seeds"]])
    ph = o.phases()
    beta, no_md, gs, t = float(g["beta"]), int(g["no_md"]), int(g["gauge_scale"]), float(g["t"])
    d = o.md_deltas(beta, no_md, gs, t)
    mass, res, rho = float(g["mass"]), float(g["res"]), float(g["rho"])

    def F_(uu, mm, k):
        return o.mom_sum_mult(mm, _oracle_force(o, uu, ph, mass, g["a"], g["b"], chis, res, rho), d[k])

    def G_(uu, mm):
        return o.gauge_2mn(uu, mm, beta, no_md, gs, t, 1)

    mom = F_(u, mom, 0)
    for _ in range(1, no_md):
        u, mom = G_(u, mom)
        mom = F_(u, mom, 1)
        u, mom = G_(u, mom)
        mom = F_(u, mom, 2)
    u, mom = G_(u, mom)
    mom = F_(u, mom, 1)
    u, mom = G_(u, mom)
    mom = F_(u, mom, 0)
    assert relerr(u[:, :2], g["md_u"]) <= 1e-12
    assert relerr(mom, g["md_mom"]) <= 1e-12
