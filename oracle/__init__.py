"""Test oracle (checker only): ctypes bindings of

* ``oracle/liboracle.so`` -- the CPU restatement in ``ostaple_oracle.c``;
* ``oracle/_ref/libref_<dims>.so`` -- the reference's own C sources compiled
  per lattice size by ``Makefile.ref`` (present only where the reference
  source tree was available at build time).

Only the tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg
use this package.  The product never imports it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "liboracle.so"
REF_DIR = HERE / "_ref"

_P, _D, _I = C.c_void_p, C.c_double, C.c_int


def _p(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


class Oracle:
    """The CPU restatement (runtime geometry)."""

    _sig = {
        "orc_init": (_I, [_I, _I, _I, _I]),
        "orc_sizeh": (_I, []),
        "orc_set_threads": (None, [_I]),
        "orc_calc_phases": (None, [_P, _D]),
        "orc_Deo": (None, [_P, _P, _P, _P]),
        "orc_Doe": (None, [_P, _P, _P, _P]),
        "orc_mdagm": (None, [_P, _P, _P, _P, _P, _D]),
        "orc_norm2": (_D, [_P]),
        "orc_rdot": (_D, [_P, _P]),
        "orc_cg": (_I, [_P, _P, _D, _P, _P, _D, _I, _D, _I, C.POINTER(_I)]),
        "orc_cgm": (_I, [_P, _P, _D, _I, _P, _P, _P, _D, _I, C.POINTER(_I)]),
        "orc_recombine": (None, [_P, _P, _P, _I, _D, _P]),
        "orc_find_max": (_D, [_P, _P, _D, _P, _P, C.POINTER(_I)]),
        "orc_find_min": (_D, [_P, _P, _D, _P, _P, _D, C.POINTER(_I)]),
        "orc_staples": (None, [_P, _P]),
        "orc_rho_ta": (None, [_P, _P, _P, _D]),
        "orc_exp_times_conf": (None, [_P, _P, _P]),
        "orc_stout": (None, [_P, _P, _D]),
        "orc_lambda": (None, [_P, _P, _P, _P]),
        "orc_sigma": (None, [_P, _P, _P, _P, _D]),
        "orc_sigma_prime_to_sigma": (None, [_P, _P, _D]),
        "orc_force_outer": (None, [_P, _P, _P, _P, _I, _P]),
        "orc_backfield_times_force": (None, [_P, _P, _P]),
        "orc_conf_times_force_ta": (None, [_P, _P, _P]),
        "orc_gauge_staples": (None, [_P, _P]),
        "orc_ipdot_gauge": (None, [_P, _P]),
        "orc_plaquette_sum": (_D, [_P]),
        "orc_rectangle_sum": (_D, [_P]),
        "orc_momenta_action": (_D, [_P]),
        "orc_mom_sum_mult": (None, [_P, _P, _D]),
        "orc_mom_exp_times_conf": (None, [_P, _P, _D]),
        "orc_md_deltas": (None, [_D, _I, _I, _D, _P]),
        "orc_2mn_gauge": (None, [_P, _P, _D, _I, _I, _D, _I]),
    }

    def __init__(self, dims, threads: int = 1):
        if not ORACLE_LIB.exists():
            raise RuntimeError(f"{ORACLE_LIB} missing: run __graft_entry__.build()")
        self.L = C.CDLL(str(ORACLE_LIB))
        for n, (r, a) in self._sig.items():
            f = getattr(self.L, n)
            f.restype = r
            f.argtypes = a
        self.dims = tuple(dims)
        self.sizeh = self.L.orc_init(*self.dims)
        self.L.orc_set_threads(threads)

    def set_threads(self, n: int) -> None:
        self.L.orc_set_threads(n)

    def phases(self, im_chem_pot: float = 0.0) -> np.ndarray:
        ph = np.zeros((8, self.sizeh))
        self.L.orc_calc_phases(_p(ph), im_chem_pot)
        return ph

    def Deo(self, u, inp, ph):
        out = np.zeros((3, self.sizeh), np.complex128)
        self.L.orc_Deo(_p(u), _p(out), _p(inp), _p(ph))
        return out

    def Doe(self, u, inp, ph):
        out = np.zeros((3, self.sizeh), np.complex128)
        self.L.orc_Doe(_p(u), _p(out), _p(inp), _p(ph))
        return out

    def mdagm(self, u, inp, ph, m2):
        out = np.zeros((3, self.sizeh), np.complex128)
        tmp = np.zeros_like(out)
        self.L.orc_mdagm(_p(u), _p(out), _p(inp), _p(tmp), _p(ph), m2)
        return out

    def norm2(self, a) -> float:
        return self.L.orc_norm2(_p(a))

    def cg(self, u, ph, mass, b, res, max_cg=10000, shift=0.0, restart=10000, x0=None):
        x = np.zeros((3, self.sizeh), np.complex128) if x0 is None else x0.copy()
        n = C.c_int(0)
        st = self.L.orc_cg(_p(u), _p(ph), mass, _p(x), _p(b), res, max_cg, shift, restart, C.byref(n))
        return st, n.value, x

    def eo_inversion(self, u, ph, mass, in_e, in_o, res, max_cg=10000):
        """D (out_e, out_o) = (in_e, in_o) by even/odd reduction
        (Meas/ferm_meas.c:50-71): out_e = (M^+M)^-1 (m in_e - D_eo in_o) by
        the FP64 CG from a zero guess, out_o = (in_o - D_oe out_e) / m."""
        phi_e = mass * in_e - self.Deo(u, in_o, ph)
        st, n, out_e = self.cg(u, ph, mass, phi_e, res, max_cg=max_cg)
        out_o = (in_o - self.Doe(u, out_e, ph)) / mass
        return st, n, out_e, out_o

    def cgm(self, u, ph, mass, shifts, b, res, max_cg=10000):
        shifts = np.ascontiguousarray(shifts, dtype=np.float64)
        xs = np.zeros((len(shifts), 3, self.sizeh), np.complex128)
        n = C.c_int(0)
        st = self.L.orc_cgm(_p(u), _p(ph), mass, len(shifts), _p(shifts), _p(xs), _p(b), res, max_cg, C.byref(n))
        return st, n.value, xs

    def recombine(self, xs, b, a0, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        out = np.zeros((3, self.sizeh), np.complex128)
        self.L.orc_recombine(_p(xs), _p(b), _p(out), len(a), a0, _p(a))
        return out

    def find_max(self, u, ph, mass, p0):
        """(max, loops, p, r): power iteration from start vector p0."""
        p = np.ascontiguousarray(p0, dtype=np.complex128).copy()
        r = np.zeros_like(p)
        n = C.c_int(0)
        mx = self.L.orc_find_max(_p(u), _p(ph), mass, _p(p), _p(r), C.byref(n))
        return mx, n.value, p, r

    def find_min(self, u, ph, mass, p0, max_eig):
        p = np.ascontiguousarray(p0, dtype=np.complex128).copy()
        r = np.zeros_like(p)
        n = C.c_int(0)
        mn = self.L.orc_find_min(_p(u), _p(ph), mass, _p(p), _p(r), max_eig, C.byref(n))
        return mn, n.value, p, r

    # --- gauge part: su3[8] = complex (8,3,3,sizeh); tamat/thmat = float (8, 8*sizeh) ---
    def su3(self):
        return np.zeros((8, 3, 3, self.sizeh), np.complex128)

    def tamat(self):
        return np.zeros((8, 8 * self.sizeh))

    def staples(self, u):
        s = self.su3()
        self.L.orc_staples(_p(u), _p(s))
        return s

    def rho_ta(self, u, stap, rho):
        q = self.tamat()
        self.L.orc_rho_ta(_p(u), _p(stap), _p(q), rho)
        return q

    def stout(self, u, rho):
        out = u.copy()
        self.L.orc_stout(_p(u), _p(out), rho)
        return out

    def sigma_prime_to_sigma(self, sigma, u, rho):
        s = sigma.copy()
        self.L.orc_sigma_prime_to_sigma(_p(s), _p(u), rho)
        return s

    def lambda_(self, sp, u, qa):
        lam = self.tamat()
        self.L.orc_lambda(_p(lam), _p(sp), _p(u), _p(qa))
        return lam

    def sigma(self, lam, u, s, qa, rho):
        """Sigma from Sigma' (s) and Lambda (compute_sigma, stouting.c:1175-1302)."""
        out = np.ascontiguousarray(s).copy()
        self.L.orc_sigma(_p(np.ascontiguousarray(lam)), _p(u), _p(out), _p(np.ascontiguousarray(qa)), rho)
        return out

    def exp_times_conf(self, u, qa):
        out = u.copy()
        self.L.orc_exp_times_conf(_p(u), _p(np.ascontiguousarray(qa)), _p(out))
        return out

    def force_outer(self, u, xs, ph, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        aux = self.su3()
        self.L.orc_force_outer(_p(u), _p(aux), _p(xs), _p(ph), len(a), _p(a))
        return aux

    def backfield_times_force(self, ph, aux, pip):
        out = pip.copy()
        self.L.orc_backfield_times_force(_p(ph), _p(aux), _p(out))
        return out

    def conf_times_force_ta(self, u, sigma, ipdot):
        out = ipdot.copy()
        self.L.orc_conf_times_force_ta(_p(u), _p(sigma), _p(out))
        return out

    # --- pure-gauge tree-level Symanzik HMC ---
    def gauge_staples(self, u):
        s = self.su3()
        self.L.orc_gauge_staples(_p(u), _p(s))
        return s

    def plaquette_sum(self, u):
        return self.L.orc_plaquette_sum(_p(u))

    def rectangle_sum(self, u):
        return self.L.orc_rectangle_sum(_p(u))

    def momenta_action(self, mom):
        return self.L.orc_momenta_action(_p(np.ascontiguousarray(mom)))

    def mom_sum_mult(self, mom, ipdot, fact):
        out = np.ascontiguousarray(mom).copy()
        self.L.orc_mom_sum_mult(_p(out), _p(np.ascontiguousarray(ipdot)), fact)
        return out

    def mom_exp_times_conf(self, u, mom, delta):
        out = u.copy()
        self.L.orc_mom_exp_times_conf(_p(out), _p(np.ascontiguousarray(mom)), delta)
        return out

    def md_deltas(self, beta, no_md, gauge_scale, t):
        d = np.zeros(7)
        self.L.orc_md_deltas(beta, no_md, gauge_scale, t, _p(d))
        return d

    def gauge_2mn(self, u, mom, beta, no_md, gauge_scale, t, ncalls):
        """(U, P) after ncalls x multistep_2MN_gauge; a pure-gauge trajectory is 2 no_md calls."""
        uo, mo = u.copy(), np.ascontiguousarray(mom).copy()
        self.L.orc_2mn_gauge(_p(uo), _p(mo), beta, no_md, gauge_scale, t, ncalls)
        return uo, mo

    def ipdot_gauge(self, u):
        ip = self.tamat()
        self.L.orc_ipdot_gauge(_p(u), _p(ip))
        return ip


def ref_available(dims) -> bool:
    return (REF_DIR / ("libref_" + "x".join(map(str, dims)) + ".so")).exists()


class Reference:
    """The reference's own compiled C (one library per lattice size)."""

    _sig = {
        "ref_sizeh": (_I, []),
        "ref_dims": (None, [_P]),
        "ref_setup": (None, [_I]),
        "ref_set_restart": (None, [_I]),
        "ref_calc_phases": (None, [_P, _D, _D]),
        "ref_Deo": (None, [_P, _P, _P, _P]),
        "ref_Doe": (None, [_P, _P, _P, _P]),
        "ref_mdagm_shifted": (None, [_P, _P, _P, _P, _P, _D, _D]),
        "ref_l2norm2": (_D, [_P]),
        "ref_real_scal_prod": (_D, [_P, _P]),
        "ref_scal_prod": (None, [_P, _P, _P]),
        "ref_cg": (_I, [_P, _P, _D, _P, _P, _D, _I, _D, C.POINTER(_I)]),
        "ref_cgm": (_I, [_P, _P, _D, _I, _D, _P, _P, _P, _P, _D, _I, C.POINTER(_I)]),
        "ref_recombine": (None, [_P, _P, _P, _I, _D, _P]),
        "ref_find_min_max": (None, [_P, _P, _D, _P, _P, _P]),
        "ref_ra_read": (_I, [C.c_char_p, _P]),
        "ref_ra_save": (None, [C.c_char_p, _P]),
        "ref_ra_rescale": (None, [_P, _P, _P]),
        "ref_ra_renormalize": (None, [_P, _P]),
        "ref_ra_evaluate": (_D, [_P, _D]),
        "ref_ra_filename": (None, [_D, _I, _I, _D, _P]),
        "ref_find_min": (_D, [_P, _P, _D, _P, _P, _D]),
        "ref_stout_isotropic": (None, [_P, _P, _D]),
        "ref_staples": (None, [_P, _P]),
        "ref_rho_ta": (None, [_P, _P, _P, _D]),
        "ref_force_outer_products": (None, [_P, _P, _P, _P, _D, _I, _P]),
        "ref_backfield_times_force": (None, [_P, _P, _P]),
        "ref_sigma_prime_to_sigma": (None, [_P, _P, _D]),
        "ref_conf_times_force_ta": (None, [_P, _P, _P]),
        "ref_set_tamat_zero": (None, [_P]),
        "ref_exp_times_conf": (None, [_P, _P, _P]),
        "ref_lambda": (None, [_P, _P, _P, _P]),
        "ref_sigma": (None, [_P, _P, _P, _P, _D]),
        "ref_stout_wrapper": (None, [_P, _P, _I, _D]),
        "ref_fermion_force": (None, [_P, _P, _P, _P, _D, _I, _I, _P, _P, _P, _D, _I, _I, _D]),
        "ref_gauge_staples": (None, [_P, _P]),
        "ref_ipdot_gauge": (None, [_P, _P, _P]),
        "ref_plaquette_sum": (_D, [_P]),
        "ref_rectangle_sum": (_D, [_P]),
        "ref_momenta_action": (_D, [_P]),
        "ref_mom_sum_mult": (None, [_P, _P, _D]),
        "ref_mom_exp_times_conf": (None, [_P, _P, _D]),
        "ref_md_deltas": (None, [_D, _I, _I, _D, _P]),
        "ref_2mn_gauge": (None, [_P, _P, _D, _I, _I, _D, _I]),
        "ref_rhmc_md": (None, [_P, _P, _P, _D, _I, _I, _P, _P, _P, _D, _I, _D, _I, _I, _D, _I, _D]),
        "ref_write_ascii": (_I, [_P, C.c_char_p, _I, _P]),
        "ref_read_ascii": (_I, [_P, C.c_char_p]),
        "ref_write_ildg": (_I, [_P, C.c_char_p, _I, C.c_char_p]),
        "ref_read_ildg": (_I, [_P, C.c_char_p]),
        "ref_set_beta": (None, [_D]),
    }

    def __init__(self, dims):
        path = REF_DIR / ("libref_" + "x".join(map(str, dims)) + ".so")
        if not path.exists():
            raise RuntimeError(f"{path} not built (reference source tree unavailable?)")
        self.L = C.CDLL(str(path))
        for n, (r, a) in self._sig.items():
            f = getattr(self.L, n)
            f.restype = r
            f.argtypes = a
        self.L.ref_setup(0)
        self.dims = tuple(dims)
        self.sizeh = self.L.ref_sizeh()

    def phases(self, im_chem_pot=0.0):
        ph = np.zeros((8, self.sizeh))
        self.L.ref_calc_phases(_p(ph), im_chem_pot, 1.0)
        return ph

    def Deo(self, u, inp, ph):
        out = np.zeros((3, self.sizeh), np.complex128)
        self.L.ref_Deo(_p(u), _p(out), _p(inp), _p(ph))
        return out

    def Doe(self, u, inp, ph):
        out = np.zeros((3, self.sizeh), np.complex128)
        self.L.ref_Doe(_p(u), _p(out), _p(inp), _p(ph))
        return out

    def mdagm(self, u, inp, ph, mass, shift=0.0):
        out = np.zeros((3, self.sizeh), np.complex128)
        tmp = np.zeros_like(out)
        self.L.ref_mdagm_shifted(_p(u), _p(out), _p(inp), _p(tmp), _p(ph), mass, shift)
        return out

    def cg(self, u, ph, mass, b, res, max_cg=10000, shift=0.0, restart=10000, x0=None):
        x = np.zeros((3, self.sizeh), np.complex128) if x0 is None else x0.copy()
        n = C.c_int(0)
        self.L.ref_set_restart(restart)
        st = self.L.ref_cg(_p(u), _p(ph), mass, _p(x), _p(b), res, max_cg, shift, C.byref(n))
        return st, n.value, x

    def cgm(self, u, ph, mass, a0, a, shifts, b, res, max_cg=10000):
        a = np.ascontiguousarray(a, dtype=np.float64)
        shifts = np.ascontiguousarray(shifts, dtype=np.float64)
        xs = np.zeros((len(shifts), 3, self.sizeh), np.complex128)
        n = C.c_int(0)
        st = self.L.ref_cgm(_p(u), _p(ph), mass, len(shifts), a0, _p(a), _p(shifts), _p(xs), _p(b), res, max_cg,
                            C.byref(n))
        return st, n.value, xs

    def recombine(self, xs, b, a0, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        out = np.zeros((3, self.sizeh), np.complex128)
        self.L.ref_recombine(_p(xs), _p(b), _p(out), len(a), a0, _p(a))
        return out

    def find_min_max(self, u, ph, mass, p0):
        """(minmax[2], p, r) from find_min_max_eigenvalue_soloopenacc."""
        p = np.ascontiguousarray(p0, dtype=np.complex128).copy()
        r = np.zeros_like(p)
        mm = np.zeros(2)
        self.L.ref_find_min_max(_p(u), _p(ph), mass, _p(p), _p(r), _p(mm))
        return mm, p, r

    def find_min(self, u, ph, mass, p0, max_eig):
        p = np.ascontiguousarray(p0, dtype=np.complex128).copy()
        r = np.zeros_like(p)
        mn = self.L.ref_find_min(_p(u), _p(ph), mass, _p(p), _p(r), max_eig)
        return mn, p, r

    def su3(self):
        return np.zeros((8, 3, 3, self.sizeh), np.complex128)

    def tamat(self):
        return np.zeros((8, 8 * self.sizeh))

    def staples(self, u):
        s = self.su3()
        self.L.ref_staples(_p(u), _p(s))
        return s

    def rho_ta(self, u, stap, rho):
        q = self.tamat()
        self.L.ref_rho_ta(_p(u), _p(stap), _p(q), rho)
        return q

    def stout(self, u, rho):
        out = u.copy()
        self.L.ref_stout_isotropic(_p(u), _p(out), rho)
        return out

    def sigma_prime_to_sigma(self, sigma, u, rho):
        s = sigma.copy()
        self.L.ref_sigma_prime_to_sigma(_p(s), _p(u), rho)
        return s

    def force_outer(self, u, xs, ph, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        aux = self.su3()
        self.L.ref_force_outer_products(_p(u), _p(aux), _p(xs), _p(ph), 0.0, len(a), _p(a))
        return aux

    def backfield_times_force(self, ph, aux, pip):
        out = pip.copy()
        self.L.ref_backfield_times_force(_p(ph), _p(aux), _p(out))
        return out

    def conf_times_force_ta(self, u, sigma, ipdot):
        out = ipdot.copy()
        self.L.ref_conf_times_force_ta(_p(u), _p(sigma), _p(out))
        return out

    def exp_times_conf(self, u, qa):
        out = u.copy()
        self.L.ref_exp_times_conf(_p(u), _p(np.ascontiguousarray(qa)), _p(out))
        return out

    def lambda_(self, sp, u, qa):
        lam = self.tamat()
        self.L.ref_lambda(_p(lam), _p(np.ascontiguousarray(sp)), _p(u), _p(np.ascontiguousarray(qa)))
        return lam

    def sigma(self, lam, u, s, qa, rho):
        out = np.ascontiguousarray(s).copy()
        self.L.ref_sigma(_p(np.ascontiguousarray(lam)), _p(u), _p(out), _p(np.ascontiguousarray(qa)), rho)
        return out

    def stout_levels(self, u, steps, rho):
        """stout_wrapper: (steps*8, 3, 3, sizeh) smeared levels (rows 0-1 written)."""
        lv = np.zeros((8 * steps, 3, 3, self.sizeh), np.complex128)
        self.L.ref_stout_wrapper(_p(u), _p(lv), steps, rho)
        return lv

    def fermion_force(self, u, ph, mass, a, b, phis, res, steps=2, rho=0.15, max_cg=10000):
        """ipdot of fermion_force_soloopenacc for one flavour with len(phis)
        pseudofermions and approx_md = (a, b)."""
        a = np.ascontiguousarray(a, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        phis = np.ascontiguousarray(phis, dtype=np.complex128).reshape(-1, 3, self.sizeh)
        lv = np.zeros((8 * max(steps, 1), 3, 3, self.sizeh), np.complex128)
        ip = self.tamat()
        ph = np.ascontiguousarray(ph)
        self.L.ref_fermion_force(_p(u), _p(lv), _p(ip), _p(ph), mass, len(phis), len(a), _p(a), _p(b), _p(phis),
                                 res, max_cg, steps, rho)
        return ip

    # --- pure-gauge tree-level Symanzik HMC ---
    def gauge_staples(self, u):
        s = self.su3()
        self.L.ref_gauge_staples(_p(u), _p(s))
        return s

    def plaquette_sum(self, u):
        return self.L.ref_plaquette_sum(_p(u))

    def rectangle_sum(self, u):
        return self.L.ref_rectangle_sum(_p(u))

    def momenta_action(self, mom):
        return self.L.ref_momenta_action(_p(np.ascontiguousarray(mom)))

    def mom_sum_mult(self, mom, ipdot, fact):
        out = np.ascontiguousarray(mom).copy()
        self.L.ref_mom_sum_mult(_p(out), _p(np.ascontiguousarray(ipdot)), fact)
        return out

    def mom_exp_times_conf(self, u, mom, delta):
        out = u.copy()
        self.L.ref_mom_exp_times_conf(_p(out), _p(np.ascontiguousarray(mom)), delta)
        return out

    def md_deltas(self, beta, no_md, gauge_scale, t):
        d = np.zeros(7)
        self.L.ref_md_deltas(beta, no_md, gauge_scale, t, _p(d))
        return d

    def gauge_2mn(self, u, mom, beta, no_md, gauge_scale, t, ncalls):
        """(U, P) after ncalls x multistep_2MN_gauge; a pure-gauge trajectory is 2 no_md calls."""
        uo, mo = u.copy(), np.ascontiguousarray(mom).copy()
        self.L.ref_2mn_gauge(_p(uo), _p(mo), beta, no_md, gauge_scale, t, ncalls)
        return uo, mo

    def ipdot_gauge(self, u):
        ip = self.tamat()
        st = self.su3()
        self.L.ref_ipdot_gauge(_p(u), _p(st), _p(ip))
        return ip

    def rhmc_md(self, u, mom, ph, mass, a, b, chis, res, beta, no_md, gauge_scale, t, steps=2, rho=0.15,
                max_cg=10000):
        """(U, P) after the reference's multistep_2MN_SOLOOPENACC with one
        flavour of len(chis) pseudofermions and approx_md = (a, b)."""
        a = np.ascontiguousarray(a, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        chis = np.ascontiguousarray(chis, dtype=np.complex128).reshape(-1, 3, self.sizeh)
        uo, mo = u.copy(), np.ascontiguousarray(mom).copy()
        self.L.ref_rhmc_md(_p(uo), _p(mo), _p(np.ascontiguousarray(ph)), mass, len(chis), len(a), _p(a), _p(b),
                           _p(chis), res, max_cg, beta, no_md, gauge_scale, t, steps, rho)
        return uo, mo

    # --- configuration files (the reference's io.c) ---
    def write_ascii(self, u, path, traj, beta=0.0, phases=None):
        self.L.ref_set_beta(beta)
        return self.L.ref_write_ascii(_p(u), str(path).encode(), traj, None if phases is None else _p(phases))

    def read_ascii(self, path):
        u = self.su3()
        t = self.L.ref_read_ascii(_p(u), str(path).encode())
        return t, u

    def write_ildg(self, u, path, traj, text=""):
        return self.L.ref_write_ildg(_p(u), str(path).encode(), traj, text.encode())

    def read_ildg(self, path):
        u = self.su3()
        t = self.L.ref_read_ildg(_p(u), str(path).encode())
        return t, u
