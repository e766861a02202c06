"""Input variables of the solver: a ctypes mirror of ``vca_config``.

Field names, meanings and defaults follow ``VCA_INPUT_VARS.f90:14-81`` and the
defaults set at ``VCA_INPUT_VARS.f90:112-172`` of QcmPlab/VCA.  The fields after
``verbose`` up to ``hxv_variant``, and ``contour_nodes``, have no counterpart
in the reference; they pin down what the reference leaves to SciFortran
(Lanczos stopping rule and start vector) or replaces (the adaptive QUADPACK
integrals of ``VCA_OMEGA.f90:132,172`` become fixed Gauss-Legendre rules).
``bandwidth`` is a module variable the reference's drivers assign
(``drivers/vca_hm_2dsquare.f90:72``).  The layout must match
``include/vca_gpu.h``.
"""
from __future__ import annotations

import ctypes

LANC_ARPACK = 0
LANC_LANCZOS = 1
ARITH_AUTO, ARITH_FP64, ARITH_FX = 0, 1, 2


class VcaConfig(ctypes.Structure):
    _fields_ = [
        ("Norb", ctypes.c_int32),
        ("Nspin", ctypes.c_int32),
        ("Nlat", ctypes.c_int32),
        ("Nlat_bath", ctypes.c_int32),
        ("Norb_bath", ctypes.c_int32),
        ("no_sector_screen", ctypes.c_int32),
        ("Uloc", ctypes.c_double * 5),
        ("Ust", ctypes.c_double),
        ("Jh", ctypes.c_double),
        ("Jx", ctypes.c_double),
        ("Jp", ctypes.c_double),
        ("xmu", ctypes.c_double),
        ("beta", ctypes.c_double),
        ("eps", ctypes.c_double),
        ("wini", ctypes.c_double),
        ("wfin", ctypes.c_double),
        ("hfmode", ctypes.c_int32),
        ("hfshift", ctypes.c_int32),
        ("Lmats", ctypes.c_int32),
        ("Lreal", ctypes.c_int32),
        ("lanc_method", ctypes.c_int32),
        ("lanc_niter", ctypes.c_int32),
        ("lanc_ngfiter", ctypes.c_int32),
        ("lanc_dim_threshold", ctypes.c_int32),
        ("lanc_nstates_sector", ctypes.c_int32),
        ("lanc_nstates_total", ctypes.c_int32),
        ("lanc_tolerance", ctypes.c_double),
        ("gs_threshold", ctypes.c_double),
        ("vca_gf_symmetric", ctypes.c_int32),
        ("vca_sparse_H", ctypes.c_int32),
        ("vca_twin", ctypes.c_int32),
        ("vca_sectors", ctypes.c_int32),
        ("vca_sectors_shift", ctypes.c_int32),
        ("verbose", ctypes.c_int32),
        ("omega_nodes", ctypes.c_int32),
        ("gs_check_every", ctypes.c_int32),
        ("omega_scale", ctypes.c_double),
        ("gs_residual_tol", ctypes.c_double),
        ("gf_beta_tol", ctypes.c_double),
        ("start_seed", ctypes.c_uint64),
        ("arith", ctypes.c_int32),
        ("hxv_variant", ctypes.c_int32),
        ("lanc_nstates_step", ctypes.c_int32),
        ("lanc_niter_spectrum", ctypes.c_int32),
        ("contour_nodes", ctypes.c_int32),
        ("sector_at_a_time", ctypes.c_int32),
        ("cutoff", ctypes.c_double),
        ("bandwidth", ctypes.c_double),
        ("gs_beta_tol", ctypes.c_double),
        ("print_sigma", ctypes.c_int32),
        ("print_impg", ctypes.c_int32),
        ("print_impg0", ctypes.c_int32),
        ("batch_loop", ctypes.c_int32),
        ("file_suffix", ctypes.c_char * 64),
    ]

    def copy(self) -> "VcaConfig":
        c = VcaConfig()
        ctypes.memmove(ctypes.byref(c), ctypes.byref(self), ctypes.sizeof(VcaConfig))
        return c

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if name == "Uloc" else v
        return out


def default_config(**overrides) -> VcaConfig:
    """Reference defaults (VCA_INPUT_VARS.f90:112-172) plus build defaults."""
    c = VcaConfig()
    c.Norb, c.Nspin, c.Nlat, c.Nlat_bath, c.Norb_bath = 1, 1, 1, 0, 0
    for i, u in enumerate([2.0, 0.0, 0.0, 0.0, 0.0]):
        c.Uloc[i] = u
    c.Ust = c.Jh = c.Jx = c.Jp = 0.0
    c.beta, c.xmu = 1000.0, 0.0
    c.hfmode, c.hfshift = 1, 1
    c.Lmats, c.Lreal = 5000, 5000
    c.wini, c.wfin, c.eps = -5.0, 5.0, 0.01
    c.vca_twin, c.vca_sectors, c.vca_sectors_shift = 0, 0, 1
    c.vca_sparse_H, c.vca_gf_symmetric = 1, 0
    c.lanc_method = LANC_ARPACK
    c.lanc_nstates_sector, c.lanc_nstates_total = 6, 1
    c.lanc_niter, c.lanc_ngfiter = 512, 200
    c.lanc_tolerance, c.lanc_dim_threshold = 1e-12, 256
    c.gs_threshold = 1e-9
    c.verbose = 3
    c.omega_nodes = 4096
    c.gs_check_every = 10
    c.omega_scale = 1.0
    c.gs_residual_tol = 1e-11
    c.gf_beta_tol = 1e-6
    c.gs_beta_tol = 1e-12
    c.start_seed = 20261203
    c.arith = ARITH_AUTO
    c.hxv_variant = 0
    c.lanc_nstates_step, c.lanc_niter_spectrum = 2, 10
    c.cutoff, c.bandwidth = 1e-9, 0.0
    c.contour_nodes = 24
    c.print_sigma = c.print_impg = c.print_impg0 = 0  # on in the reference (VCA_INPUT_VARS.f90:137-139)
    c.file_suffix = b""
    for k, v in overrides.items():
        if k == "Uloc":
            for i in range(5):
                c.Uloc[i] = v[i] if i < len(v) else 0.0
        elif not hasattr(c, k):
            raise KeyError(f"unknown input variable {k}")
        elif k == "file_suffix":
            c.file_suffix = v.encode() if isinstance(v, str) else v
        else:
            setattr(c, k, v)
    return c


def nlso(cfg: VcaConfig) -> int:
    return cfg.Nlat * cfg.Nspin * cfg.Norb


def hloc_shape(cfg: VcaConfig) -> tuple:
    """(Nlat,Nlat,Nspin,Nspin,Norb,Norb) as VCA_MAIN.f90:125."""
    return (cfg.Nlat, cfg.Nlat, cfg.Nspin, cfg.Nspin, cfg.Norb, cfg.Norb)


def bath_h_shape(cfg: VcaConfig) -> tuple:
    return (cfg.Nlat_bath, cfg.Nlat_bath, cfg.Nspin, cfg.Nspin, cfg.Norb_bath, cfg.Norb_bath)


def bath_v_shape(cfg: VcaConfig) -> tuple:
    return (cfg.Nlat, cfg.Nlat_bath, cfg.Nspin, cfg.Nspin, cfg.Norb, cfg.Norb_bath)
