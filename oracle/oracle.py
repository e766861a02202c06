"""ctypes front end of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py``; never by the product package.
The C++ restatement it wraps follows the reference file:line by file:line
(see the header of vca_oracle.cpp); parity against the reference binary is
unpinned because the reference cannot be built here.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from vca_gb300.config import VcaConfig

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liboracle.so")
_lib = None


def build(force: bool = False) -> str:
    src = os.path.join(_HERE, "vca_oracle.cpp")
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", _HERE, "liboracle.so"])
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB)
        P, I, D, L64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int64
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        lp = ctypes.POINTER(ctypes.c_int64)
        sig = {
            "orc_create": (P, [ctypes.POINTER(VcaConfig), dp, dp, L64, dp, dp]),
            "orc_destroy": (None, [P]),
            "orc_ns": (I, [P]),
            "orc_nsectors": (I, [P]),
            "orc_binomial": (L64, [I, I]),
            "orc_sector_info": (I, [P, I, ip, ip, lp, lp]),
            "orc_c_sector": (I, [P, I, I]),
            "orc_cdg_sector": (I, [P, I, I]),
            "orc_map": (L64, [P, I, I, lp, L64]),
            "orc_hxv": (I, [P, I, dp, dp]),
            "orc_spin_matrix": (L64, [P, I, I, lp, lp, dp, L64]),
            "orc_diag_elements": (I, [P, I, dp]),
            "orc_dense_h": (I, [P, I, dp]),
            "orc_lanczos_gs": (D, [P, I, dp, ip]),
            "orc_lanczos_tridiag": (I, [P, I, dp, I, dp, dp]),
            "orc_tql2": (I, [I, dp, dp, dp, dp]),
            "orc_tri_lowest": (D, [dp, dp, I, dp]),
            "orc_start_value": (D, [ctypes.c_uint64, I, L64]),
            "orc_diagonalize": (I, [P, ip]),
            "orc_sector_energies": (I, [P, dp]),
            "orc_state": (I, [P, I, ip, dp, dp]),
            "orc_egs": (D, [P]),
            "orc_build_gf": (I, [P]),
            "orc_gf_channel": (I, [P, I, I, I, I, I, I, I, dp, dp, dp, dp, I]),
            "orc_gf_cluster": (I, [P, dp, L64, dp]),
            "orc_delta_bath": (I, [P, D, D, dp]),
            "orc_sigma_g0": (I, [P, D, D, dp, dp]),
            "orc_observables": (I, [P, dp]),
            "orc_sum_kmesh": (D, [P, D]),
            "orc_gauss_legendre01": (I, [I, dp, dp]),
            "orc_frequency_integration": (D, [P]),
            "orc_solve": (D, [P, dp, dp]),
            "orc_solve_timed": (D, [P, dp, dp, dp]),
            "orc_chain_sample": (D, [P, I, I, I]),
            "orc_sum_kmesh_complex": (D, [P, D, D, dp]),
            "orc_contour_rule": (I, [D, D, D, I, dp, dp, I]),
            "orc_contour_integrand": (D, [P, D, D]),
            "orc_frequency_integration_finite_t": (D, [P]),
            "orc_thermal": (I, [P, dp, ip]),
            "orc_custom_observable": (D, [P, dp, I]),
            "orc_sum_observable_kmesh": (D, [P, D, D, dp, I, I]),
            "orc_set_threads": (I, [I]),
            "orc_lowest_pairs": (I, [P, I, I, dp, dp]),
            "orc_neigen": (I, [P, ip]),
            "orc_state_list_t0": (I, [dp, I, D, ip, dp, I]),
            "orc_state_list_finite_t": (I, [dp, I, ctypes.POINTER(VcaConfig), I, ip, I, dp, dp, ip]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if a is not None else None


def _c128(a):
    return None if a is None else np.asfortranarray(a, dtype=np.complex128)


def set_threads(n: int) -> int:
    return lib().orc_set_threads(int(n))


def gauss_legendre01(n: int):
    x = np.zeros(n)
    w = np.zeros(n)
    lib().orc_gauss_legendre01(n, _dp(x), _dp(w))
    return x, w


def contour_rule(R: float, beta: float, mu: float, ngl: int):
    """Nodes and weights of the fixed rule on the contour angle [0, pi]."""
    n = lib().orc_contour_rule(R, beta, mu, ngl, None, None, 0)
    th = np.zeros(n)
    w = np.zeros(n)
    lib().orc_contour_rule(R, beta, mu, ngl, _dp(th), _dp(w), n)
    return th, w


def tql2(d, e):
    n = len(d)
    d = np.ascontiguousarray(d, dtype=np.float64)
    e = np.ascontiguousarray(e, dtype=np.float64)
    w = np.zeros(n)
    z0 = np.zeros(n)
    r = lib().orc_tql2(n, _dp(d), _dp(e), _dp(w), _dp(z0))
    return w, z0, r


def tri_lowest(a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    s = np.zeros(len(a))
    th = lib().orc_tri_lowest(_dp(a), _dp(b), len(a), _dp(s))
    return th, s


class Oracle:
    """One oracle model: mirrors vca_init_solver + vca_solve state."""

    def __init__(self, cfg: VcaConfig, Hloc, Hk=None, bath_h=None, bath_v=None):
        self.L = lib()
        self.cfg = cfg.copy()
        self._Hloc = _c128(Hloc)
        self._Hk = _c128(Hk) if Hk is not None else None
        self._bh = _c128(bath_h)
        self._bv = _c128(bath_v)
        nk = self._Hk.shape[-1] if self._Hk is not None else 0
        self.h = self.L.orc_create(ctypes.byref(self.cfg), _dp(self._Hloc), _dp(self._Hk), nk,
                                   _dp(self._bh), _dp(self._bv))
        self.Ns = self.L.orc_ns(self.h)
        self.Nsectors = self.L.orc_nsectors(self.h)

    @classmethod
    def from_point(cls, pt):
        return cls(pt.cfg, pt.Hloc, pt.Hk, pt.bath_h, pt.bath_v)

    def __del__(self):
        try:
            if getattr(self, "h", None):
                self.L.orc_destroy(self.h)
                self.h = None
        except Exception:
            pass

    # ---- sectors -----------------------------------------------------
    def sector_info(self, isector: int):
        nu, nd = ctypes.c_int(), ctypes.c_int()
        du, dd = ctypes.c_int64(), ctypes.c_int64()
        self.L.orc_sector_info(self.h, isector, ctypes.byref(nu), ctypes.byref(nd), ctypes.byref(du),
                               ctypes.byref(dd))
        return nu.value, nd.value, du.value, dd.value

    def dim(self, isector: int) -> int:
        _, _, du, dd = self.sector_info(isector)
        return du * dd

    def c_sector(self, isector, spin):
        return self.L.orc_c_sector(self.h, isector, spin)

    def cdg_sector(self, isector, spin):
        return self.L.orc_cdg_sector(self.h, isector, spin)

    def sector_map(self, isector: int, spin: int) -> np.ndarray:
        n = self.L.orc_map(self.h, isector, spin, None, 0)
        out = np.zeros(n, dtype=np.int64)
        self.L.orc_map(self.h, isector, spin, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), n)
        return out

    # ---- Hamiltonian -------------------------------------------------
    def hxv(self, isector: int, v: np.ndarray) -> np.ndarray:
        v = np.ascontiguousarray(v, dtype=np.complex128)
        hv = np.zeros_like(v)
        self.L.orc_hxv(self.h, isector, _dp(v), _dp(hv))
        return hv

    def diag_elements(self, isector: int) -> np.ndarray:
        out = np.zeros(self.dim(isector), dtype=np.complex128)
        self.L.orc_diag_elements(self.h, isector, _dp(out))
        return out

    def spin_matrix(self, isector: int, spin: int):
        n = self.L.orc_spin_matrix(self.h, isector, spin, None, None, None, 0)
        r = np.zeros(n, dtype=np.int64)
        c = np.zeros(n, dtype=np.int64)
        v = np.zeros(n, dtype=np.complex128)
        lp = ctypes.POINTER(ctypes.c_int64)
        self.L.orc_spin_matrix(self.h, isector, spin, r.ctypes.data_as(lp), c.ctypes.data_as(lp), _dp(v), n)
        return r, c, v

    def dense_h(self, isector: int) -> np.ndarray:
        d = self.dim(isector)
        out = np.zeros((d, d), dtype=np.complex128, order="F")
        self.L.orc_dense_h(self.h, isector, _dp(out))
        return out

    def lanczos_gs(self, isector: int):
        d = self.dim(isector)
        psi = np.zeros(d, dtype=np.complex128)
        it = ctypes.c_int()
        e = self.L.orc_lanczos_gs(self.h, isector, _dp(psi), ctypes.byref(it))
        return e, psi, it.value

    def lanczos_tridiag(self, isector: int, v1: np.ndarray, nlanc: int):
        v1 = np.ascontiguousarray(v1, dtype=np.complex128)
        a = np.zeros(nlanc)
        b = np.zeros(nlanc)
        self.L.orc_lanczos_tridiag(self.h, isector, _dp(v1), nlanc, _dp(a), _dp(b))
        return a, b

    # ---- solve stages --------------------------------------------------
    def diagonalize(self, mask=None) -> int:
        m = None
        if mask is not None:
            m = np.ascontiguousarray(mask, dtype=np.int32)
            m = m.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        return self.L.orc_diagonalize(self.h, m)

    def sector_energies(self) -> np.ndarray:
        out = np.zeros(self.Nsectors)
        self.L.orc_sector_energies(self.h, _dp(out))
        return out

    def state(self, k: int, with_vector: bool = False):
        isec = ctypes.c_int()
        e = ctypes.c_double()
        self.L.orc_state(self.h, k, ctypes.byref(isec), ctypes.byref(e), None)
        vec = None
        if with_vector:
            vec = np.zeros(self.dim(isec.value), dtype=np.complex128)
            self.L.orc_state(self.h, k, ctypes.byref(isec), ctypes.byref(e), _dp(vec))
        return isec.value, e.value, vec

    def egs(self) -> float:
        return self.L.orc_egs(self.h)

    def build_gf(self):
        self.L.orc_build_gf(self.h)

    def gf_channel(self, il, jl, ispin, io, jo, istate, ichan, cap=4096):
        p = np.zeros(cap, dtype=np.complex128)
        w = np.zeros(cap, dtype=np.complex128)
        a = np.zeros(cap)
        b = np.zeros(cap)
        n = self.L.orc_gf_channel(self.h, il, jl, ispin, io, jo, istate, ichan, _dp(p), _dp(w), _dp(a),
                                  _dp(b), cap)
        if n < 0:
            return None
        return p[:n], w[:n], a[:n], b[:n]

    def gf_cluster(self, z) -> np.ndarray:
        z = np.ascontiguousarray(np.atleast_1d(z), dtype=np.complex128)
        c = self.cfg
        shape = (c.Nlat, c.Nlat, c.Nspin, c.Nspin, c.Norb, c.Norb, len(z))
        out = np.zeros(shape, dtype=np.complex128, order="F")
        self.L.orc_gf_cluster(self.h, _dp(z), len(z), _dp(out))
        return out

    def delta_bath(self, z: complex) -> np.ndarray:
        n = self.cfg.Nlat * self.cfg.Nspin * self.cfg.Norb
        out = np.zeros((n, n), dtype=np.complex128, order="F")
        self.L.orc_delta_bath(self.h, z.real, z.imag, _dp(out))
        return out

    def observables(self) -> dict:
        """dens, dens_up, dens_dw, docc, mag as (Nlat, Norb) arrays (vca_lanc_observables)."""
        c = self.cfg
        nimp = c.Nlat * c.Norb
        v = np.zeros(3 * nimp)
        self.L.orc_observables(self.h, _dp(v))
        # flat index = bit = iorb + ilat*Norb (imp_state_index)
        up, dw, dd = (v[q * nimp:(q + 1) * nimp].reshape(c.Nlat, c.Norb) for q in range(3))
        return {"dens": up + dw, "dens_up": up, "dens_dw": dw, "docc": dd, "mag": up - dw}

    def sigma_g0(self, z: complex):
        """(Sigma, G0) at z as lso N x N matrices (build_sigma_normal)."""
        c = self.cfg
        N = c.Nlat * c.Nspin * c.Norb
        sg = np.zeros(N * N, dtype=np.complex128)
        g0 = np.zeros(N * N, dtype=np.complex128)
        self.L.orc_sigma_g0(self.h, float(np.real(z)), float(np.imag(z)), _dp(sg), _dp(g0))
        return sg.reshape(N, N, order="F"), g0.reshape(N, N, order="F")

    def sum_kmesh(self, w: float) -> float:
        return self.L.orc_sum_kmesh(self.h, float(w))

    def frequency_integration(self) -> float:
        return self.L.orc_frequency_integration(self.h)

    def sum_kmesh_complex(self, z: complex) -> complex:
        im = ctypes.c_double()
        re = self.L.orc_sum_kmesh_complex(self.h, float(np.real(z)), float(np.imag(z)), ctypes.byref(im))
        return complex(re, im.value)

    def contour_integrand(self, R: float, theta: float) -> float:
        return self.L.orc_contour_integrand(self.h, float(R), float(theta))

    def frequency_integration_finite_t(self) -> float:
        return self.L.orc_frequency_integration_finite_t(self.h)

    def custom_observable(self, s) -> float:
        """One custom observable of the last solve; s (Nlat,Nlat,Nspin,Nspin,Norb,Norb[,Nk])."""
        s = np.asfortranarray(s, dtype=np.complex128)
        return self.L.orc_custom_observable(self.h, _dp(s), 1 if s.ndim == 7 else 0)

    def sum_observable_kmesh(self, z: complex, s, tail: bool) -> float:
        s = np.asfortranarray(s, dtype=np.complex128)
        return self.L.orc_sum_observable_kmesh(self.h, float(np.real(z)), float(np.imag(z)), _dp(s),
                                               1 if s.ndim == 7 else 0, 1 if tail else 0)

    def thermal(self) -> dict:
        """The fields of vca_thermal for the last solve."""
        d = np.zeros(7)
        i = np.zeros(4, dtype=np.int32)
        self.L.orc_thermal(self.h, _dp(d), i.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
        keys = ("zeta", "omega_prime", "e_min", "max_exc", "integration_R", "sum_part", "contour_part")
        out = dict(zip(keys, d.tolist()))
        out.update(nmax=int(i[0]), nstates_total=int(i[1]), contour_points=int(i[2]), finite_t=int(i[3]))
        return out

    def states(self):
        """[(sector, energy)] of the retained state list, in list order."""
        out = []
        k = 0
        while True:
            isec = ctypes.c_int()
            e = ctypes.c_double()
            if self.L.orc_state(self.h, k, ctypes.byref(isec), ctypes.byref(e), None) != 0:
                break
            out.append((isec.value, e.value))
            k += 1
        return out

    def lowest_pairs(self, isector: int, k: int):
        """The k lowest eigenpairs of a sector on the LANC_METHOD="arpack"
        path (dense below LANC_DIM_THRESHOLD): energies ascending and the
        vectors as columns."""
        D = self.dim(isector)
        e = np.zeros(max(k, 1))
        v = np.zeros((max(k, 1), D), dtype=np.complex128)
        n = self.L.orc_lowest_pairs(self.h, isector, k, _dp(e), _dp(v))
        return e[:n], v[:n].T.copy()

    def neigen(self) -> np.ndarray:
        """neigen_sector of every sector (LANC_METHOD="arpack")."""
        out = np.zeros(self.Nsectors, dtype=np.int32)
        self.L.orc_neigen(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
        return out

    def solve(self):
        egs = ctypes.c_double()
        oi = ctypes.c_double()
        sft = self.L.orc_solve(self.h, ctypes.byref(egs), ctypes.byref(oi))
        return sft, egs.value, oi.value

    def solve_timed(self):
        """solve() plus the wall seconds of its stages (diagonalisation,
        chains, frequency integration)."""
        egs = ctypes.c_double()
        oi = ctypes.c_double()
        st = np.zeros(3)
        sft = self.L.orc_solve_timed(self.h, ctypes.byref(egs), ctypes.byref(oi), _dp(st))
        return sft, egs.value, oi.value, st.tolist()

    def chain_sample(self, isector: int, nchains: int, nlanc: int) -> float:
        """Wall seconds of nchains chains of nlanc steps on sector isector run
        as the chain stage runs them (one per thread)."""
        return self.L.orc_chain_sample(self.h, isector, nchains, nlanc)


def state_list_t0(E, gs_threshold: float):
    """[(sector, energy)] the T=0 bookkeeping keeps for sector energies E."""
    E = np.ascontiguousarray(E, dtype=np.float64)
    sec = np.zeros(len(E), dtype=np.int32)
    en = np.zeros(len(E))
    n = lib().orc_state_list_t0(_dp(E), len(E), gs_threshold, sec.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                _dp(en), len(E))
    return list(zip(sec[:n].tolist(), en[:n].tolist()))


def state_list_finite_t(E, cfg: VcaConfig, nstates_total: int):
    """(sectors, zeta, emin, adjusted nstates_total) of the annealing sweeps."""
    E = np.ascontiguousarray(E, dtype=np.float64)
    sec = np.zeros(max(len(E), 1), dtype=np.int32)
    z, lo = ctypes.c_double(), ctypes.c_double()
    nt = ctypes.c_int()
    n = lib().orc_state_list_finite_t(_dp(E), len(E), ctypes.byref(cfg), nstates_total,
                                      sec.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(sec),
                                      ctypes.byref(z), ctypes.byref(lo), ctypes.byref(nt))
    return sec[:n].tolist(), z.value, lo.value, nt.value


def start_value(seed: int, isector: int, i: int) -> float:
    return lib().orc_start_value(seed, isector, i)
