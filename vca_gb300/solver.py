"""Python mirror of the reference's VCA module over the C-ABI.

The names follow ``VCA.f90:1-38`` / ``VCA_MAIN.f90:21-39`` of QcmPlab/VCA:
``vca_init_solver``, ``vca_solve``, ``vca_get_sft_potential``,
``vca_gf_cluster``, ``vca_get_gimp_matsubara``, ``vca_get_gimp_realaxis``.
Arrays are Fortran-ordered complex128 with the reference's shapes.  Errors the
reference turns into ``stop "..."`` raise :class:`VcaError` with the library's
message.  There is no CPU fallback: if ``libvca_gpu.so`` is missing or no GPU
is visible the calls raise.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

from . import search as _search
from .reshape import (vca_lso2nnn_reshape, vca_nn2so_reshape, vca_nnn2lso_reshape,  # noqa: F401
                      vca_rectangular_j2n_reshape, vca_rectangular_n2j_reshape, vca_so2nn_reshape)
from .config import VcaConfig, hloc_shape, bath_h_shape, bath_v_shape

_HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(_HERE, "libvca_gpu.so")
_lib = None

# exported symbols of include/vca_gpu.h
EXPORTS = [
    "vca_config_defaults", "vca_gpu_init", "vca_gpu_solve", "vca_gpu_solve_batch",
    "vca_gpu_get_sft_potential", "vca_gpu_get_energies", "vca_gpu_gf_cluster",
    "vca_gpu_get_gimp_matsubara", "vca_gpu_get_gimp_realaxis", "vca_gpu_get_state_count",
    "vca_gpu_get_state", "vca_gpu_get_sector_energies", "vca_gpu_get_gf_channel",
    "vca_gpu_sum_kmesh", "vca_gpu_finalize", "vca_gpu_last_error", "vca_gpu_sector_info",
    "vca_gpu_sector_map", "vca_gpu_set_hamiltonian", "vca_gpu_hxv", "vca_gpu_hxv_device",
    "vca_gpu_get_sigma_matsubara", "vca_gpu_get_sigma_realaxis", "vca_gpu_get_g0_matsubara",
    "vca_gpu_get_g0_realaxis", "vca_gpu_get_dens", "vca_gpu_get_dens_up", "vca_gpu_get_dens_dw",
    "vca_gpu_get_docc", "vca_gpu_get_mag",
    "vca_gpu_hxv_timed", "vca_gpu_hxv_alpha_noalloc", "vca_gpu_sector_row_order", "vca_gpu_upload_hk", "vca_gpu_solve_resident", "vca_gpu_kernel_launches",
    "vca_gpu_get_timings", "vca_gpu_synchronize", "vca_gpu_set_ql_max_iter", "vca_gpu_sector_bounds",
    "vca_gpu_set_omega_inverse_form", "vca_gpu_set_autotune", "vca_gpu_set_hop_pairing", "vca_gpu_set_chain_streams", "vca_gpu_set_stage_extra_tx",
    "vca_gpu_timer_start",
    "vca_gpu_timer_stop",
    "vca_gpu_arith_info", "vca_gpu_sum_kmesh_complex", "vca_gpu_get_thermal", "vca_gpu_custom_observable",
    "vca_gpu_save_gfprime", "vca_gpu_read_gfprime", "vca_gfm_write", "vca_gfm_read",
    "vca_gpu_print_impSigma", "vca_gpu_print_impG", "vca_gpu_print_impG0",
    "vca_state_list_t0", "vca_state_list_finite_t", "vca_pair_kpoints", "vca_contour_rule",
    "vca_tridiag_eig", "vca_herm_eig", "vca_gpu_sector_pairs", "vca_hop_schedule", "vca_hop_parity_order",
    "vca_read_impSigma", "vca_splot_read",
    "vca_mlp_config_defaults", "vca_mlp_init", "vca_mlp_finalize", "vca_mlp_param_count",
    "vca_mlp_get_params", "vca_mlp_set_params", "vca_mlp_set_data", "vca_mlp_loss_grad", "vca_mlp_train",
    "vca_mlp_predict", "vca_umma_gemm_check", "vca_umma_timeout_check",
]


class VcaThermal(ctypes.Structure):
    """Mirror of ``vca_thermal`` (include/vca_gpu.h)."""
    _fields_ = [
        ("zeta", ctypes.c_double),
        ("omega_prime", ctypes.c_double),
        ("e_min", ctypes.c_double),
        ("max_exc", ctypes.c_double),
        ("integration_R", ctypes.c_double),
        ("sum_part", ctypes.c_double),
        ("contour_part", ctypes.c_double),
        ("nmax", ctypes.c_int32),
        ("nstates_total", ctypes.c_int32),
        ("contour_points", ctypes.c_int32),
        ("finite_t", ctypes.c_int32),
    ]


class VcaError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def load(path: Optional[str] = None):
    """Load the C-ABI library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIBPATH
    if not os.path.exists(p):
        raise VcaError(-4, f"{p} is missing: run vca_gb300.build.build() (no CPU fallback)")
    L = ctypes.CDLL(p)
    dp = ctypes.POINTER(ctypes.c_double)
    i32, i64 = ctypes.c_int32, ctypes.c_int64
    vp = ctypes.c_void_p
    cfgp = ctypes.POINTER(VcaConfig)
    sig = {
        "vca_config_defaults": (None, [cfgp]),
        "vca_gpu_init": (ctypes.c_int, [cfgp, dp, dp]),
        "vca_gpu_solve": (ctypes.c_int, [dp, dp, i64, dp, dp, dp]),
        "vca_gpu_solve_batch": (ctypes.c_int, [i32, dp, i64, dp, i64, dp, i64, dp, i64, dp]),
        "vca_gpu_get_sft_potential": (ctypes.c_int, [dp]),
        "vca_gpu_get_energies": (ctypes.c_int, [dp, dp]),
        "vca_gpu_gf_cluster": (ctypes.c_int, [dp, i64, dp]),
        "vca_gpu_get_gimp_matsubara": (ctypes.c_int, [dp]),
        "vca_gpu_get_gimp_realaxis": (ctypes.c_int, [dp]),
        "vca_gpu_get_sigma_matsubara": (ctypes.c_int, [dp]),
        "vca_gpu_get_sigma_realaxis": (ctypes.c_int, [dp]),
        "vca_gpu_get_g0_matsubara": (ctypes.c_int, [dp]),
        "vca_gpu_get_g0_realaxis": (ctypes.c_int, [dp]),
        "vca_gpu_get_dens": (ctypes.c_int, [dp]),
        "vca_gpu_get_dens_up": (ctypes.c_int, [dp]),
        "vca_gpu_get_dens_dw": (ctypes.c_int, [dp]),
        "vca_gpu_get_docc": (ctypes.c_int, [dp]),
        "vca_gpu_get_mag": (ctypes.c_int, [dp]),
        "vca_gpu_get_state_count": (ctypes.c_int, [ctypes.POINTER(i32)]),
        "vca_gpu_get_state": (ctypes.c_int, [i32, ctypes.POINTER(i32), dp]),
        "vca_gpu_get_sector_energies": (ctypes.c_int, [dp, i32]),
        "vca_gpu_get_gf_channel": (ctypes.c_int, [i32, i32, i32, i32, i32, i32, i32,
                                                  ctypes.POINTER(i32), dp, dp, i32]),
        "vca_gpu_sum_kmesh": (ctypes.c_int, [dp, i64, dp]),
        "vca_gpu_sum_kmesh_complex": (ctypes.c_int, [dp, i64, dp]),
        "vca_gpu_get_thermal": (ctypes.c_int, [ctypes.POINTER(VcaThermal)]),
        "vca_gpu_custom_observable": (ctypes.c_int, [dp, i32, dp]),
        "vca_gpu_finalize": (ctypes.c_int, []),
        "vca_gpu_last_error": (ctypes.c_int, [ctypes.c_char_p, i32]),
        "vca_gpu_sector_info": (ctypes.c_int, [i32, ctypes.POINTER(i32), ctypes.POINTER(i32),
                                               ctypes.POINTER(i64), ctypes.POINTER(i64)]),
        "vca_gpu_sector_map": (ctypes.c_int, [i32, i32, ctypes.POINTER(i64), i64]),
        "vca_gpu_set_hamiltonian": (ctypes.c_int, [dp, dp, dp]),
        "vca_gpu_hxv": (ctypes.c_int, [i32, dp, dp]),
        "vca_gpu_hxv_device": (ctypes.c_int, [i32, vp, vp, i32]),
        "vca_gpu_hxv_timed": (ctypes.c_int, [i32, vp, vp, i32, i32, i32, dp]),
        "vca_gpu_hxv_alpha_noalloc": (ctypes.c_int, [i32, vp, vp, i32, vp]),
        "vca_gpu_sector_row_order": (ctypes.c_int, [i32, ctypes.POINTER(i64), i64]),
        "vca_gpu_upload_hk": (ctypes.c_int, [dp, i64]),
        "vca_gpu_solve_resident": (ctypes.c_int, [dp, dp, dp, dp]),
        "vca_gpu_kernel_launches": (i64, []),
        "vca_gpu_get_timings": (ctypes.c_int, [dp, i32]),
        "vca_gpu_synchronize": (ctypes.c_int, []),
        "vca_gpu_set_ql_max_iter": (ctypes.c_int, [i32]),
        "vca_gpu_sector_bounds": (ctypes.c_int, [dp, i32]),
        "vca_gpu_set_omega_inverse_form": (ctypes.c_int, [i32]),
        "vca_gpu_set_autotune": (ctypes.c_int, [i32]),
        "vca_gpu_set_hop_pairing": (ctypes.c_int, [i32]),
        "vca_gpu_set_chain_streams": (ctypes.c_int, [i32]),
        "vca_gpu_set_stage_extra_tx": (ctypes.c_int, [i32]),
        "vca_gpu_timer_start": (ctypes.c_int, []),
        "vca_gpu_timer_stop": (ctypes.c_int, [dp]),
        "vca_gpu_arith_info": (ctypes.c_int, [ctypes.POINTER(i32)] * 3),
        "vca_state_list_t0": (ctypes.c_int, [dp, i32, ctypes.c_double, ctypes.POINTER(i32), dp, i32,
                                             ctypes.POINTER(i32)]),
        "vca_state_list_finite_t": (ctypes.c_int, [dp, i32, cfgp, i32, ctypes.POINTER(i32), i32,
                                                   ctypes.POINTER(i32), dp, dp, ctypes.POINTER(i32)]),
        "vca_pair_kpoints": (ctypes.c_int, [dp, i64, i64, ctypes.POINTER(i64), dp, i64, ctypes.POINTER(i64)]),
        "vca_tridiag_eig": (ctypes.c_int, [i32, dp, dp, dp, dp]),
        "vca_hop_schedule": (ctypes.c_int, [i32, i32, i32, vp, vp, vp, i64, vp, vp, ctypes.POINTER(i64),
                                            ctypes.POINTER(i64)]),
        "vca_hop_parity_order": (ctypes.c_int, [i32, i32, vp, vp, vp]),
        "vca_gpu_sector_pairs": (ctypes.c_int, [i32, i32, dp, dp, ctypes.POINTER(i32)]),
        "vca_herm_eig": (ctypes.c_int, [i32, dp, dp, dp]),
        "vca_contour_rule": (ctypes.c_int, [ctypes.c_double, ctypes.c_double, ctypes.c_double, i32, dp, dp, i32,
                                            ctypes.POINTER(i32)]),
        "vca_gpu_print_impSigma": (ctypes.c_int, []),
        "vca_read_impSigma": (ctypes.c_int, []),
        "vca_splot_read": (ctypes.c_int, [ctypes.c_char_p, i64, dp, dp]),
        "vca_gpu_print_impG": (ctypes.c_int, []),
        "vca_gpu_print_impG0": (ctypes.c_int, []),
        "vca_gpu_save_gfprime": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, i32, i32]),
        "vca_gpu_read_gfprime": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, i32, i32]),
        "vca_gfm_write": (ctypes.c_int, [ctypes.c_char_p, i32, i64, ctypes.POINTER(i32), ctypes.POINTER(i32),
                                         ctypes.POINTER(i32), dp, dp]),
        "vca_gfm_read": (ctypes.c_int, [ctypes.c_char_p, i32, i64, ctypes.POINTER(i64), ctypes.POINTER(i32),
                                        ctypes.POINTER(i32), ctypes.POINTER(i32), dp, dp]),
    }
    fp = ctypes.POINTER(ctypes.c_float)
    u16p = ctypes.POINTER(ctypes.c_uint16)
    from .surrogate import MlpConfig
    sig.update({
        "vca_mlp_config_defaults": (None, [ctypes.POINTER(MlpConfig)]),
        "vca_mlp_init": (ctypes.c_int, [ctypes.POINTER(MlpConfig)]),
        "vca_mlp_finalize": (ctypes.c_int, []),
        "vca_mlp_param_count": (i64, []),
        "vca_mlp_get_params": (ctypes.c_int, [fp, i64]),
        "vca_mlp_set_params": (ctypes.c_int, [fp, i64]),
        "vca_mlp_set_data": (ctypes.c_int, [i32, dp, dp, dp, dp]),
        "vca_mlp_loss_grad": (ctypes.c_int, [dp, fp, i64]),
        "vca_mlp_train": (ctypes.c_int, [i32, dp]),
        "vca_mlp_predict": (ctypes.c_int, [i32, dp, dp, dp]),
        "vca_umma_gemm_check": (ctypes.c_int, [u16p, u16p, fp, i32, i32, i32]),
        "vca_umma_timeout_check": (ctypes.c_int, []),
    })
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _dp(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _c128(a, shape=None, name="array"):
    if a is None:
        return None
    a = np.asfortranarray(a, dtype=np.complex128)
    if shape is not None and tuple(a.shape) != tuple(shape):
        raise VcaError(-2, f"{name} has shape {a.shape}, expected {tuple(shape)}")
    return a


def check(rc: int):
    if rc != 0:
        buf = ctypes.create_string_buffer(1024)
        load().vca_gpu_last_error(buf, 1024)
        raise VcaError(rc, buf.value.decode(errors="replace"))


def library_defaults() -> VcaConfig:
    c = VcaConfig()
    load().vca_config_defaults(ctypes.byref(c))
    return c


class VcaSolver:
    """One solver context (the library keeps one global context, as the
    reference keeps module globals)."""

    def __init__(self, cfg: VcaConfig, bath_h=None, bath_v=None):
        self.L = load()
        self.cfg = cfg.copy()
        self.has_bath = bath_h is not None
        if self.has_bath:
            bath_h = _c128(bath_h, bath_h_shape(cfg), "bath_h")
            bath_v = _c128(bath_v, bath_v_shape(cfg), "bath_v")
        else:
            self.cfg.Nlat_bath = 0
            self.cfg.Norb_bath = 0
        check(self.L.vca_gpu_init(ctypes.byref(self.cfg), _dp(bath_h), _dp(bath_v)))

    # ---- vca_solve -----------------------------------------------------
    def solve(self, Hloc, Hk, bath_h=None, bath_v=None) -> float:
        c = self.cfg
        Hloc = _c128(Hloc, hloc_shape(c), "Hloc")
        Hk = _c128(Hk, None, "Hk")
        if Hk.shape[:6] != hloc_shape(c) or Hk.ndim != 7:
            raise VcaError(-2, f"Hk has shape {Hk.shape}, expected {hloc_shape(c)} + (Nk,)")
        if bath_h is not None:
            bath_h = _c128(bath_h, bath_h_shape(c), "bath_h")
            bath_v = _c128(bath_v, bath_v_shape(c), "bath_v")
        out = ctypes.c_double()
        check(self.L.vca_gpu_solve(_dp(Hloc), _dp(Hk), Hk.shape[6], _dp(bath_h), _dp(bath_v),
                                   ctypes.byref(out)))
        return out.value

    def solve_batch(self, Hloc_b, Hk, bath_h_b=None, bath_v_b=None) -> np.ndarray:
        c = self.cfg
        Hloc_b = np.asfortranarray(Hloc_b, dtype=np.complex128)
        B = Hloc_b.shape[-1]
        Hk = _c128(Hk)
        out = np.zeros(B)
        n_h = int(np.prod(hloc_shape(c)))
        bh = np.asfortranarray(bath_h_b, dtype=np.complex128) if bath_h_b is not None else None
        bv = np.asfortranarray(bath_v_b, dtype=np.complex128) if bath_v_b is not None else None
        check(self.L.vca_gpu_solve_batch(B, _dp(Hloc_b), n_h, _dp(Hk), Hk.shape[6],
                                         _dp(bh), int(np.prod(bath_h_shape(c))) if bh is not None else 0,
                                         _dp(bv), int(np.prod(bath_v_shape(c))) if bv is not None else 0,
                                         _dp(out)))
        return out

    def upload_hk(self, Hk):
        Hk = _c128(Hk)
        check(self.L.vca_gpu_upload_hk(_dp(Hk), Hk.shape[6]))

    def solve_resident(self, Hloc, bath_h=None, bath_v=None) -> float:
        c = self.cfg
        Hloc = _c128(Hloc, hloc_shape(c), "Hloc")
        if bath_h is not None:
            bath_h = _c128(bath_h, bath_h_shape(c), "bath_h")
            bath_v = _c128(bath_v, bath_v_shape(c), "bath_v")
        out = ctypes.c_double()
        check(self.L.vca_gpu_solve_resident(_dp(Hloc), _dp(bath_h), _dp(bath_v), ctypes.byref(out)))
        return out.value

    def timings(self, batched: bool = False):
        """Stage wall times (ms) of the last solve, or with batched=True of
        the last batched-form solve_batch (tables, search, eigenvectors,
        chains, Omega, closing plain solve)."""
        out = np.zeros(13)
        check(self.L.vca_gpu_get_timings(_dp(out), 13))
        return out[4:] if batched else out[:4]

    def sector_pairs(self, isector: int, k: int):
        """(energies, vectors as columns) of the k lowest eigenpairs of a
        sector as the "arpack" diagonalisation finds them."""
        _, _, du, dd = self.sector_info(isector)
        D = du * dd
        e = np.zeros(k)
        v = np.zeros(2 * k * D)
        n = ctypes.c_int32()
        check(self.L.vca_gpu_sector_pairs(isector, k, _dp(e), _dp(v), ctypes.byref(n)))
        nn = n.value
        return e[:nn], v.view(np.complex128).reshape(k, D)[:nn].T

    def chain_timings(self):
        """The last solve's chain stage: (start-vector ms, Lanczos-step ms,
        column batches)."""
        out = np.zeros(16)
        check(self.L.vca_gpu_get_timings(_dp(out), 16))
        return float(out[13]), float(out[14]), int(out[15])

    def arith_info(self):
        fx, F, G = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        check(self.L.vca_gpu_arith_info(ctypes.byref(fx), ctypes.byref(F), ctypes.byref(G)))
        return bool(fx.value), F.value, G.value

    def timer_start(self):
        check(self.L.vca_gpu_timer_start())

    def timer_stop(self) -> float:
        ms = ctypes.c_double()
        check(self.L.vca_gpu_timer_stop(ctypes.byref(ms)))
        return ms.value

    def synchronize(self):
        check(self.L.vca_gpu_synchronize())

    def sector_bounds(self) -> np.ndarray:
        """Lower bound of every sector's lowest energy (one-body ground energy)."""
        n = (self.Ns + 1) ** 2
        out = np.zeros(n)
        check(self.L.vca_gpu_sector_bounds(_dp(out), n))
        return out

    def set_autotune(self, on: bool):
        """Tune the batched chains' tile shape at first use (default on)."""
        check(self.L.vca_gpu_set_autotune(1 if on else 0))

    def set_stage_extra_tx(self, nbytes: int):
        """Test hook: make the chains' H x v bulk-copy wait run out (0 = off)."""
        check(self.L.vca_gpu_set_stage_extra_tx(int(nbytes)))

    def set_chain_streams(self, n: int):
        """Chain column groups in flight at a time (1 or 2, default 1)."""
        check(self.L.vca_gpu_set_chain_streams(int(n)))

    def set_hop_pairing(self, on: bool):
        """Pair the chains' kernel's hop parities per quarter warp (default
        on; applies to the next set_hamiltonian)."""
        check(self.L.vca_gpu_set_hop_pairing(1 if on else 0))

    def set_omega_inverse_form(self, on: bool):
        """T=0 k-sum through G'^-1 + M_k below w = 10 (default on)."""
        check(self.L.vca_gpu_set_omega_inverse_form(1 if on else 0))

    def set_ql_max_iter(self, n: int):
        """QL sweeps per eigenvalue allowed when chains become poles (default 60)."""
        check(self.L.vca_gpu_set_ql_max_iter(int(n)))

    def kernel_launches(self) -> int:
        return int(self.L.vca_gpu_kernel_launches())

    def sector_row_order(self, isector) -> np.ndarray:
        """Sector element index held in each batch row under hxv_variant 2."""
        _, _, du, dd = self.sector_info(isector)
        out = np.zeros(du * dd, dtype=np.int64)
        check(self.L.vca_gpu_sector_row_order(isector, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                              out.size))
        return out

    def hxv_alpha_noalloc(self, isector, d_v, d_hv, ncols, d_alpha):
        """Y = H X on device columns and alpha[c] = <x_c, H x_c> into the
        device array d_alpha, with no device allocation (static scratch)."""
        check(self.L.vca_gpu_hxv_alpha_noalloc(isector, ctypes.c_void_p(d_v), ctypes.c_void_p(d_hv), ncols,
                                               ctypes.c_void_p(d_alpha)))

    def hxv_timed(self, isector, d_v, d_hv, is_complex, ncols, reps) -> float:
        ms = ctypes.c_double()
        check(self.L.vca_gpu_hxv_timed(isector, ctypes.c_void_p(d_v), ctypes.c_void_p(d_hv), is_complex,
                                       ncols, reps, ctypes.byref(ms)))
        return ms.value

    def get_sft_potential(self) -> float:
        out = ctypes.c_double()
        check(self.L.vca_gpu_get_sft_potential(ctypes.byref(out)))
        return out.value

    def energies(self):
        egs, oi = ctypes.c_double(), ctypes.c_double()
        check(self.L.vca_gpu_get_energies(ctypes.byref(egs), ctypes.byref(oi)))
        return egs.value, oi.value

    def states(self):
        n = ctypes.c_int32()
        check(self.L.vca_gpu_get_state_count(ctypes.byref(n)))
        out = []
        for k in range(1, n.value + 1):
            s, e = ctypes.c_int32(), ctypes.c_double()
            check(self.L.vca_gpu_get_state(k, ctypes.byref(s), ctypes.byref(e)))
            out.append((s.value, e.value))
        return out

    def sector_energies(self) -> np.ndarray:
        ns = (self.Ns + 1) ** 2
        out = np.zeros(ns)
        check(self.L.vca_gpu_get_sector_energies(_dp(out), ns))
        return out

    @property
    def Ns(self) -> int:
        c = self.cfg
        return c.Nlat * c.Norb + c.Nlat_bath * c.Norb_bath

    def gf_channel(self, il, jl, ispin, io, jo, istate, ichan, cap=4096):
        n = ctypes.c_int32()
        p = np.zeros(cap, dtype=np.complex128)
        w = np.zeros(cap, dtype=np.complex128)
        check(self.L.vca_gpu_get_gf_channel(il, jl, ispin, io, jo, istate, ichan, ctypes.byref(n),
                                            _dp(p), _dp(w), cap))
        return p[: n.value], w[: n.value]

    def gf_cluster(self, z) -> np.ndarray:
        z = np.ascontiguousarray(np.atleast_1d(z), dtype=np.complex128)
        c = self.cfg
        out = np.zeros(hloc_shape(c) + (len(z),), dtype=np.complex128, order="F")
        check(self.L.vca_gpu_gf_cluster(_dp(z), len(z), _dp(out)))
        return out

    def gimp_matsubara(self) -> np.ndarray:
        out = np.zeros(hloc_shape(self.cfg) + (self.cfg.Lmats,), dtype=np.complex128, order="F")
        check(self.L.vca_gpu_get_gimp_matsubara(_dp(out)))
        return out

    def gimp_realaxis(self) -> np.ndarray:
        out = np.zeros(hloc_shape(self.cfg) + (self.cfg.Lreal,), dtype=np.complex128, order="F")
        check(self.L.vca_gpu_get_gimp_realaxis(_dp(out)))
        return out

    def _grid(self, fn, mats: bool) -> np.ndarray:
        L = self.cfg.Lmats if mats else self.cfg.Lreal
        out = np.zeros(hloc_shape(self.cfg) + (L,), dtype=np.complex128, order="F")
        check(fn(_dp(out)))
        return out

    def observables(self) -> dict:
        """vca_get_dens / _dens_up / _dens_dw / _docc / _mag: (Nlat, Norb) arrays."""
        out = {}
        for key in ("dens", "dens_up", "dens_dw", "docc", "mag"):
            a = np.zeros((self.cfg.Nlat, self.cfg.Norb), order="F")
            check(getattr(self.L, "vca_gpu_get_" + key)(_dp(a)))
            out[key] = a
        return out

    def sigma_matsubara(self) -> np.ndarray:
        """vca_get_sigma_matsubara: Sigma(i w_n), (Nlat,Nlat,Nspin,Nspin,Norb,Norb,Lmats)."""
        return self._grid(self.L.vca_gpu_get_sigma_matsubara, True)

    def sigma_realaxis(self) -> np.ndarray:
        return self._grid(self.L.vca_gpu_get_sigma_realaxis, False)

    def g0_matsubara(self) -> np.ndarray:
        return self._grid(self.L.vca_gpu_get_g0_matsubara, True)

    def g0_realaxis(self) -> np.ndarray:
        return self._grid(self.L.vca_gpu_get_g0_realaxis, False)

    def sum_kmesh(self, w) -> np.ndarray:
        w = np.ascontiguousarray(np.atleast_1d(w), dtype=np.float64)
        out = np.zeros(len(w))
        check(self.L.vca_gpu_sum_kmesh(_dp(w), len(w), _dp(out)))
        return out

    def sum_kmesh_complex(self, z) -> np.ndarray:
        """sum_kmesh_complex: (1/Lk) sum_k log det(...) at complex z (principal branch per k)."""
        z = np.ascontiguousarray(np.atleast_1d(z), dtype=np.complex128)
        out = np.zeros(len(z), dtype=np.complex128)
        check(self.L.vca_gpu_sum_kmesh_complex(_dp(z), len(z), _dp(out)))
        return out

    def custom_observable(self, s) -> float:
        """Value of one custom observable for the last solve: s has shape
        (Nlat,Nlat,Nspin,Nspin,Norb,Norb) (the same at every k) or
        (...,Nk) (k-dependent), as add_custom_observable takes it."""
        s = np.asfortranarray(s, dtype=np.complex128)
        kdep = 1 if s.ndim == 7 else 0
        if s.shape[:6] != hloc_shape(self.cfg):
            raise ValueError(f"s has shape {s.shape}, expected {hloc_shape(self.cfg)}[+ (Nk,)]")
        out = ctypes.c_double()
        check(self.L.vca_gpu_custom_observable(_dp(s), kdep, ctypes.byref(out)))
        return out.value

    # custom-observable registry with the reference's call sequence
    # (init_custom_observables, add_custom_observable, get_custom_observables,
    # clear_custom_observables, VCA_OBSERVABLES.f90:76-180)
    def init_custom_observables(self, n: int, nk: int):
        self._custom = {"asked": int(n), "nk": int(nk), "items": []}

    def add_custom_observable(self, name: str, s):
        if not getattr(self, "_custom", None):
            raise VcaError(-3, "add_custom_observable: custom observables not initialized")
        if len(self._custom["items"]) >= self._custom["asked"]:
            raise VcaError(-9, "add_custom_observable: too many observables given")
        s = np.asfortranarray(s, dtype=np.complex128)
        if s.ndim == 7 and s.shape[6] != self._custom["nk"]:
            raise ValueError("add_custom_observable: k-dependent s must have Nk matrices")
        self._custom["items"].append((name, s))

    def get_custom_observables(self) -> dict:
        if not getattr(self, "_custom", None):
            return {}
        return {name: self.custom_observable(s) for name, s in self._custom["items"]}

    def clear_custom_observables(self):
        self._custom = None

    def thermal(self) -> dict:
        """zeta, Omega', E_min, max_exc, contour radius, Matsubara and contour
        parts, nmax, the adapted LANC_NSTATES_TOTAL, contour nodes, finite_t."""
        t = VcaThermal()
        check(self.L.vca_gpu_get_thermal(ctypes.byref(t)))
        return {name: getattr(t, name) for name, _ in VcaThermal._fields_}

    # ---- parity hooks ------------------------------------------------------
    def sector_info(self, isector):
        a, b = ctypes.c_int32(), ctypes.c_int32()
        du, dd = ctypes.c_int64(), ctypes.c_int64()
        check(self.L.vca_gpu_sector_info(isector, ctypes.byref(a), ctypes.byref(b), ctypes.byref(du),
                                         ctypes.byref(dd)))
        return a.value, b.value, du.value, dd.value

    def sector_map(self, isector, spin) -> np.ndarray:
        _, _, du, dd = self.sector_info(isector)
        n = du if spin == 1 else dd
        out = np.zeros(n, dtype=np.int64)
        check(self.L.vca_gpu_sector_map(isector, spin, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), n))
        return out

    def set_hamiltonian(self, Hloc, bath_h=None, bath_v=None):
        c = self.cfg
        Hloc = _c128(Hloc, hloc_shape(c), "Hloc")
        if bath_h is not None:
            bath_h = _c128(bath_h, bath_h_shape(c), "bath_h")
            bath_v = _c128(bath_v, bath_v_shape(c), "bath_v")
        check(self.L.vca_gpu_set_hamiltonian(_dp(Hloc), _dp(bath_h), _dp(bath_v)))

    def hxv(self, isector, v) -> np.ndarray:
        v = np.ascontiguousarray(v, dtype=np.complex128)
        hv = np.zeros_like(v)
        check(self.L.vca_gpu_hxv(isector, _dp(v), _dp(hv)))
        return hv

    def save_gfprime(self, file: str = "gfprime", used: bool = False, use_formatted: bool = False,
                     suffix: Optional[str] = None):
        """save_gfprime (VCA_AUX_FUNX.f90:601-645): the pole tables of the
        last solve (or of the last read_gfprime) to file//suffix//".restart"
        (".used" when used); suffix None = the config's file_suffix."""
        sfx = None if suffix is None else suffix.encode()
        check(self.L.vca_gpu_save_gfprime(file.encode(), sfx, int(used), int(use_formatted)))
        return gfprime_path(file, used, self._suffix(suffix))

    def read_gfprime(self, file: str = "gfprime", used: bool = False, use_formatted: bool = False,
                     suffix: Optional[str] = None):
        """read_gfprime (VCA_AUX_FUNX.f90:651-697): the tables replace the
        solve's for gf_cluster and gf_channel until the next solve."""
        sfx = None if suffix is None else suffix.encode()
        check(self.L.vca_gpu_read_gfprime(file.encode(), sfx, int(used), int(use_formatted)))

    def _suffix(self, suffix: Optional[str]) -> str:
        return self.cfg.file_suffix.decode() if suffix is None else suffix

    def print_impSigma(self):
        """vca_print_impSigma (VCA_IO.f90:112-138): splot files of Sigma."""
        check(self.L.vca_gpu_print_impSigma())

    def read_impSigma(self):
        """vca_read_impSigma (VCA_IO.f90:208-239): Sigma from the impSigma
        splot files; the Sigma getters return it until the next solve."""
        check(self.L.vca_read_impSigma())

    def print_impG(self):
        """vca_print_impG (VCA_IO.f90:146-173): splot files of G'."""
        check(self.L.vca_gpu_print_impG())

    def print_impG0(self):
        """vca_print_impG0 (VCA_IO.f90:179-205): splot files of G0."""
        check(self.L.vca_gpu_print_impG0())

    def close(self):
        self.L.vca_gpu_finalize()


# ---- state-list logic of the solve (host only, no GPU needed) -------------
def state_list_t0(E, gs_threshold: float):
    """[(sector, energy)] the T=0 bookkeeping keeps (VCA_DIAG.f90:224-236)
    for every sector's lowest energy E (1-based sector order)."""
    E = np.ascontiguousarray(E, dtype=np.float64)
    cap = max(len(E), 1)
    sec = np.zeros(cap, dtype=np.int32)
    en = np.zeros(cap)
    n = ctypes.c_int32()
    i32p = ctypes.POINTER(ctypes.c_int32)
    check(load().vca_state_list_t0(_dp(E), len(E), gs_threshold, sec.ctypes.data_as(i32p), _dp(en), cap,
                                   ctypes.byref(n)))
    return list(zip(sec[:n.value].tolist(), en[:n.value].tolist()))


def tridiag_eig(d, e):
    """Eigenvalues (ascending) and eigenvectors (columns) of the symmetric
    tridiagonal matrix with diagonal d and off-diagonal e (host QL)."""
    d = np.ascontiguousarray(d, dtype=np.float64)
    n = len(d)
    e = np.ascontiguousarray(np.r_[e, 0.0][:max(n - 1, 1)], dtype=np.float64)
    w = np.zeros(n)
    Z = np.zeros(n * n)
    check(load().vca_tridiag_eig(n, _dp(d), _dp(e), _dp(w), _dp(Z)))
    return w, Z.reshape(n, n).T


def hop_schedule(cnt, hop, K: int = 1):
    """(sched words [rounds, 32], wround, wgrp [nwarps, 2K], conflicts): the
    paired-column kernel's bank schedule of one spin space (host)."""
    cnt = np.ascontiguousarray(cnt, dtype=np.int32)
    hop = np.ascontiguousarray(hop, dtype=np.uint32)  # [width, dim]
    dim = len(cnt)
    width = hop.shape[0]
    nw = (dim + 31) // 32
    wround = np.zeros(nw + 1, dtype=np.int32)
    wgrp = np.zeros(nw * 2 * K, dtype=np.int32)
    cap = int(nw * 2 * max(1, width) * 32)
    sched = np.zeros(cap, dtype=np.uint32)
    nr, nc = ctypes.c_int64(), ctypes.c_int64()
    vp_ = ctypes.c_void_p
    check(load().vca_hop_schedule(dim, width, K, vp_(cnt.ctypes.data), vp_(hop.ctypes.data), vp_(sched.ctypes.data),
                                  cap, vp_(wround.ctypes.data), vp_(wgrp.ctypes.data), ctypes.byref(nr),
                                  ctypes.byref(nc)))
    return sched[:nr.value * 32].reshape(nr.value, 32), wround, wgrp.reshape(nw, 2 * K), nc.value


def hop_parity_order(cnt, npos, rhop):
    """The chains' kernel's up hops re-ordered for bank pairing (host); rhop
    [width, dim] is modified in place and returned."""
    cnt = np.ascontiguousarray(cnt, dtype=np.int32)
    npos = np.ascontiguousarray(npos, dtype=np.int32)
    assert rhop.dtype == np.uint32 and rhop.flags["C_CONTIGUOUS"]
    vp_ = ctypes.c_void_p
    check(load().vca_hop_parity_order(len(cnt), rhop.shape[0], vp_(cnt.ctypes.data), vp_(npos.ctypes.data),
                                      vp_(rhop.ctypes.data)))
    return rhop


def herm_eig(A):
    """Eigenvalues (ascending) and eigenvectors (columns) of the Hermitian
    matrix A (host Jacobi)."""
    A = np.ascontiguousarray(A, dtype=np.complex128)
    n = A.shape[0]
    w = np.zeros(n)
    Z = np.zeros(2 * n * n)
    check(load().vca_herm_eig(n, _dp(A.view(np.float64)), _dp(w), _dp(Z)))
    return w, Z.view(np.complex128).reshape(n, n).T


def state_list_finite_t(E, cfg: VcaConfig, nstates_total: int):
    """(sectors in list order, zeta, E_min, adjusted LANC_NSTATES_TOTAL) of
    the annealing sweeps (VCA_DIAG.f90:78-256, vca_post_diag :357-451)."""
    E = np.ascontiguousarray(E, dtype=np.float64)
    cap = max(len(E), 1)
    sec = np.zeros(cap, dtype=np.int32)
    n, nt = ctypes.c_int32(), ctypes.c_int32()
    z, lo = ctypes.c_double(), ctypes.c_double()
    i32p = ctypes.POINTER(ctypes.c_int32)
    check(load().vca_state_list_finite_t(_dp(E), len(E), ctypes.byref(cfg), nstates_total, sec.ctypes.data_as(i32p),
                                         cap, ctypes.byref(n), ctypes.byref(z), ctypes.byref(lo), ctypes.byref(nt)))
    return sec[:n.value].tolist(), z.value, lo.value, nt.value


def pair_kpoints(Hk):
    """(representatives, weights) of the Omega k-sum for Hk of shape
    (...,Nk): conjugate pairs H_k' = conj(H_k) summed once with weight 2."""
    Hk = np.asfortranarray(Hk, dtype=np.complex128)
    Nk = Hk.shape[-1]
    nel = Hk.size // max(Nk, 1)
    reps = np.zeros(max(Nk, 1), dtype=np.int64)
    w = np.zeros(max(Nk, 1))
    n = ctypes.c_int64()
    check(load().vca_pair_kpoints(_dp(Hk), Nk, nel, reps.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), _dp(w),
                                  len(reps), ctypes.byref(n)))
    return reps[:n.value], w[:n.value]


def contour_rule(R: float, beta: float, mu: float, ngl: int):
    """Nodes and weights on [0, pi] of the contour rule at radius R."""
    n = ctypes.c_int32()
    check(load().vca_contour_rule(R, beta, mu, ngl, None, None, 0, ctypes.byref(n)))
    th = np.zeros(n.value)
    w = np.zeros(n.value)
    check(load().vca_contour_rule(R, beta, mu, ngl, _dp(th), _dp(w), n.value, ctypes.byref(n)))
    return th, w


# ---- GFmatrix restart files (host only, no GPU needed) --------------------
def gfprime_path(file: str = "gfprime", used: bool = False, suffix: str = "") -> str:
    """file//file_suffix//(".used" | ".restart") (VCA_AUX_FUNX.f90:615-617)."""
    return file + suffix + (".used" if used else ".restart")


def splot_name(name: str, ilat: int, jlat: int, iorb: int, jorb: int, ispin: int, matsubara: bool,
               suffix: str = "") -> str:
    """File of one element written by vca_print_impSigma / _impG / _impG0
    (VCA_IO.f90:125-128): name in impSigma, impG, impG0; indices 1-based."""
    return (f"{name}_Isite{ilat:04d}_Jsite{jlat:04d}_l{iorb}{jorb}_s{ispin}_"
            f"{'iw' if matsubara else 'realw'}{suffix}.vca")


def read_splot(path: str, n: Optional[int] = None):
    """x and the complex function of a splot file (columns x, Im, Re); n
    lines (default: the file's line count)."""
    if n is None:
        with open(path) as f:
            n = sum(1 for line in f if line.strip())
    x = np.zeros(n)
    y = np.zeros(n, dtype=np.complex128)
    check(load().vca_splot_read(path.encode(), n, _dp(x), _dp(y)))
    return x, y


def gfm_elements(cfg: VcaConfig):
    """(ilat, jlat, ispin, iorb, jorb), 1-based, in the order of the file's
    elements: the loops of save_gfprime, ilat outermost (VCA_AUX_FUNX.f90:
    627-641)."""
    return [(il, jl, s, io, jo)
            for il in range(1, cfg.Nlat + 1) for jl in range(1, cfg.Nlat + 1)
            for s in range(1, cfg.Nspin + 1)
            for io in range(1, cfg.Norb + 1) for jo in range(1, cfg.Norb + 1)]


def write_gfmatrix(path: str, table, formatted: bool = False):
    """Write a GFmatrix table: table[element][state][channel] = (poles,
    weights), complex arrays of equal length, elements in file order."""
    ns, nc, nx, P, W = [], [], [], [], []
    for el in table:
        ns.append(len(el))
        for st in el:
            nc.append(len(st))
            for p, w in st:
                p = np.asarray(p, dtype=np.complex128).ravel()
                w = np.asarray(w, dtype=np.complex128).ravel()
                if p.shape != w.shape:
                    raise VcaError(-9, "poles and weights differ in length")
                nx.append(len(p))
                P.append(p)
                W.append(w)
    i32p = ctypes.POINTER(ctypes.c_int32)
    a_ns, a_nc, a_nx = (np.array(v, dtype=np.int32) for v in (ns, nc, nx))
    a_p = np.ascontiguousarray(np.concatenate(P) if P else np.zeros(0, np.complex128))
    a_w = np.ascontiguousarray(np.concatenate(W) if W else np.zeros(0, np.complex128))
    check(load().vca_gfm_write(path.encode(), int(formatted), len(ns), a_ns.ctypes.data_as(i32p),
                               a_nc.ctypes.data_as(i32p), a_nx.ctypes.data_as(i32p), _dp(a_p), _dp(a_w)))


def read_gfmatrix(path: str, nelem: int, formatted: bool = False):
    """Read nelem elements of a GFmatrix file into
    table[element][state][channel] = (poles, weights)."""
    L = load()
    i32p = ctypes.POINTER(ctypes.c_int32)
    sizes = np.zeros(3, dtype=np.int64)
    check(L.vca_gfm_read(path.encode(), int(formatted), nelem, sizes.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                         None, None, None, None, None))
    ns = np.zeros(max(nelem, 1), np.int32)
    nc = np.zeros(max(int(sizes[0]), 1), np.int32)
    nx = np.zeros(max(int(sizes[1]), 1), np.int32)
    P = np.zeros(max(int(sizes[2]), 1), np.complex128)
    W = np.zeros(max(int(sizes[2]), 1), np.complex128)
    check(L.vca_gfm_read(path.encode(), int(formatted), nelem, sizes.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                         ns.ctypes.data_as(i32p), nc.ctypes.data_as(i32p), nx.ctypes.data_as(i32p), _dp(P), _dp(W)))
    table, a, b, x = [], 0, 0, 0
    for e in range(nelem):
        el = []
        for _ in range(ns[e]):
            st = []
            for _ in range(nc[a]):
                n = int(nx[b])
                st.append((P[x:x + n].copy(), W[x:x + n].copy()))
                x += n
                b += 1
            el.append(st)
            a += 1
        table.append(el)
    return table


# ---- functional interface with the reference's names ---------------------
_solver: Optional[VcaSolver] = None


def vca_init_solver(cfg: VcaConfig, bath_h=None, bath_v=None) -> VcaSolver:
    """vca_init_solver (VCA_MAIN.f90:51-76)."""
    global _solver
    _solver = VcaSolver(cfg, bath_h, bath_v)
    return _solver


def vca_solve(Hloc, Hk, bath_h=None, bath_v=None) -> float:
    """vca_solve (VCA_MAIN.f90:124-215): returns the SFT potential."""
    if _solver is None:
        raise VcaError(-3, "vca_init_solver has not been called")
    return _solver.solve(Hloc, Hk, bath_h, bath_v)


def _ctx() -> VcaSolver:
    if _solver is None:
        raise VcaError(-3, "vca_init_solver has not been called")
    return _solver


def vca_get_sft_potential() -> float:
    """vca_get_sft_potential (VCA_IO/get_sft_potential.f90:1-4)."""
    return _ctx().get_sft_potential()


def vca_gf_cluster(z) -> np.ndarray:
    """vca_gf_cluster (VCA_IO/gf_cluster.f90): G'(z), shape (...,len(z))."""
    return _ctx().gf_cluster(z)


# the other public names of module VCA (VCA.f90:1-38)
def vca_get_sigma_matsubara() -> np.ndarray:
    """vca_get_sigma_matsubara (VCA_IO/get_sigma_matsubara.f90)."""
    return _ctx().sigma_matsubara()


def vca_get_sigma_realaxis() -> np.ndarray:
    """vca_get_sigma_realaxis (VCA_IO/get_sigma_realaxis.f90)."""
    return _ctx().sigma_realaxis()


def vca_get_gimp_matsubara() -> np.ndarray:
    """vca_get_gimp_matsubara (VCA_IO/get_gimp_matsubara.f90)."""
    return _ctx().gimp_matsubara()


def vca_get_gimp_realaxis() -> np.ndarray:
    """vca_get_gimp_realaxis (VCA_IO/get_gimp_realaxis.f90)."""
    return _ctx().gimp_realaxis()


def observables_cluster() -> dict:
    """observables_cluster (VCA_OBSERVABLES.f90:70-74): dens, dens_up,
    dens_dw, docc and mag of the last solve, each (Nlat,Norb)."""
    return _ctx().observables()


def vca_get_dens() -> np.ndarray:
    """vca_get_dens (VCA_IO/get_dens.f90): (Nlat,Norb)."""
    return _ctx().observables()["dens"]


def vca_get_mag() -> np.ndarray:
    """vca_get_mag (VCA_IO/get_mag.f90): (Nlat,Norb)."""
    return _ctx().observables()["mag"]


def vca_get_docc() -> np.ndarray:
    """vca_get_docc (VCA_IO/get_docc.f90): (Nlat,Norb)."""
    return _ctx().observables()["docc"]


def init_custom_observables(N: int, Nk: int):
    """init_custom_observables (VCA_OBSERVABLES.f90:76-87)."""
    return _ctx().init_custom_observables(N, Nk)


def add_custom_observable(name: str, sij):
    """add_custom_observable, local or k-dependent (VCA_OBSERVABLES.f90:89-134)."""
    return _ctx().add_custom_observable(name, sij)


def get_custom_observables() -> dict:
    """get_custom_observables (VCA_OBSERVABLES.f90:137-165): name -> value."""
    return _ctx().get_custom_observables()


def clear_custom_observables():
    """clear_custom_observables (VCA_OBSERVABLES.f90:168-180)."""
    return _ctx().clear_custom_observables()


def vca_print_impSigma():
    """vca_print_impSigma (VCA_IO.f90:112-138)."""
    _ctx().print_impSigma()


def vca_read_impSigma():
    """vca_read_impSigma (VCA_IO.f90:208-239)."""
    _ctx().read_impSigma()


def vca_print_impG():
    """vca_print_impG (VCA_IO.f90:146-173)."""
    _ctx().print_impG()


def vca_print_impG0():
    """vca_print_impG0 (VCA_IO.f90:179-205)."""
    _ctx().print_impG0()


def save_gfprime(file: str = "gfprime", used: bool = False, use_formatted: bool = False):
    """save_gfprime (VCA_AUX_FUNX.f90:601-645)."""
    return _ctx().save_gfprime(file, used, use_formatted)


def read_gfprime(file: str = "gfprime", used: bool = False, use_formatted: bool = False):
    """read_gfprime (VCA_AUX_FUNX.f90:651-697)."""
    _ctx().read_gfprime(file, used, use_formatted)


# density searches (VCA_AUX_FUNX.f90:700-897); the SAVE state of the
# reference's module lives in search_state
search_state = _search.SearchState()


def search_chemical_potential(var: float, ntmp: float, converged: bool):
    """search_chemical_potential(var, ntmp, converged) -> (var, converged)."""
    return _search.search_chemical_potential(search_state, var, ntmp, converged)


def vca_search_variable(var: float, ntmp: float, converged: bool):
    """vca_search_variable(var, ntmp, converged) -> (var, converged)."""
    return _search.vca_search_variable(search_state, var, ntmp, converged)


def vca_get_cluster_dimension(with_bath: bool = False) -> int:
    """vca_get_cluster_dimension (VCA_AUX_FUNX.f90:97-114): Nspin * levels."""
    c = _ctx().cfg
    ns = c.Nlat * c.Norb + (c.Nlat_bath * c.Norb_bath if with_bath else 0)
    return c.Nspin * ns
