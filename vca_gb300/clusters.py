"""Synthetic cluster inputs for the solver: t' (Hloc), H_k and the bath.

These restate the model recipes of the reference drivers (the reference ships
no dataset; its drivers build t' and H_k and call ``vca_solve``):

* 1D Hubbard chain     drivers/vca_hm_chain1d.f90:148-227
* 2D square cluster    drivers/vca_hm_2dsquare_bath.f90:154-269 (site index
                       ``indices2N``, :294-300)
* BHZ 2x2 cluster      drivers/vca_bhz_2d.f90:312-472

All arrays are complex128 in Fortran (column-major) order with the reference's
shapes: Hloc (Nlat,Nlat,Nspin,Nspin,Norb,Norb), Hk (...,Nk), bath_h
(Nlat_bath,Nlat_bath,Nspin,Nspin,Norb_bath,Norb_bath), bath_v
(Nlat,Nlat_bath,Nspin,Nspin,Norb,Norb_bath).  k-grids are laid out explicitly
(k = 2*pi*m/(N*L) in the reduced zone) instead of through DMFT_tools
TB_build_kgrid: H_k is an input of vca_solve, so only its values matter.
Random parameters come from numpy PCG64 with the seed given.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from .config import VcaConfig, default_config, LANC_LANCZOS

SEED = 20261203


@dataclass
class SolvePoint:
    """One vca_solve call: configuration plus its arrays."""
    cfg: VcaConfig
    Hloc: np.ndarray
    Hk: np.ndarray
    bath_h: Optional[np.ndarray] = None
    bath_v: Optional[np.ndarray] = None
    label: str = ""
    params: dict = field(default_factory=dict)

    @property
    def Nk(self) -> int:
        return self.Hk.shape[-1]


def _zeros(*shape):
    return np.zeros(shape, dtype=np.complex128, order="F")


def nnn2lso(a: np.ndarray) -> np.ndarray:
    """(Nlat,Nlat,Nspin,Nspin,Norb,Norb[,L]) -> (Nlso,Nlso[,L]), lso index
    is = iorb + (ilat-1)*Norb + (ispin-1)*Norb*Nlat (VCA_AUX_FUNX.f90:255-279)."""
    nlat, _, nsp, _, norb, _ = a.shape[:6]
    rest = a.shape[6:]
    # axes (ilat,jlat,is,js,io,jo) -> (io,ilat,is, jo,jlat,js) in Fortran order
    b = np.transpose(a, (4, 0, 2, 5, 1, 3) + tuple(range(6, a.ndim)))
    n = nlat * nsp * norb
    return np.reshape(b, (n, n) + rest, order="F")


def lso2nnn(m: np.ndarray, nlat: int, nspin: int, norb: int) -> np.ndarray:
    rest = m.shape[2:]
    b = np.reshape(m, (norb, nlat, nspin, norb, nlat, nspin) + rest, order="F")
    return np.asfortranarray(np.transpose(b, (1, 4, 2, 5, 0, 3) + tuple(range(6, b.ndim))))


def lanczos_cfg(**kw) -> VcaConfig:
    """Parity mode of the plain path: LANC_METHOD='lanczos', T=0, stored
    semantics, VCA_GF_SYMMETRIC=F."""
    base = dict(lanc_method=LANC_LANCZOS, lanc_nstates_total=1, vca_gf_symmetric=0, verbose=0)
    base.update(kw)
    return default_config(**base)


# ---------------------------------------------------------------------------
# 1D chain (config 1): Nlat sites, open cluster, boundary phase in H_k
# ---------------------------------------------------------------------------
def chain1d(tprime: float = 1.0, nlat: int = 4, U: float = 4.0, xmu: float = 2.0, t: float = 1.0,
            nk: int = 64, ngfiter: int = 100, omega_nodes: int = 4096, **cfgkw) -> SolvePoint:
    cfg = lanczos_cfg(Nlat=nlat, Norb=1, Nspin=1, Uloc=[U], hfmode=0, xmu=xmu,
                      lanc_ngfiter=ngfiter, omega_nodes=omega_nodes, **cfgkw)
    H = _zeros(nlat, nlat, 1, 1, 1, 1)
    for i in range(nlat):  # generate_tcluster (vca_hm_chain1d.f90:148-171)
        if i > 0:
            H[i, i - 1, 0, 0, 0, 0] = -tprime
        if i < nlat - 1:
            H[i, i + 1, 0, 0, 0, 0] = -tprime
    Hk = _zeros(nlat, nlat, 1, 1, 1, 1, nk)
    for m in range(nk):  # tk (vca_hm_chain1d.f90:204-227), k = 2 pi m/(nk*Nlat)
        kN = 2.0 * np.pi * m / nk  # k * Nlat
        for i in range(nlat):
            if i > 0:
                Hk[i, i - 1, 0, 0, 0, 0, m] = -t
            if i < nlat - 1:
                Hk[i, i + 1, 0, 0, 0, 0, m] = -t
        Hk[0, nlat - 1, 0, 0, 0, 0, m] += -t * np.exp(1j * kN)
        Hk[nlat - 1, 0, 0, 0, 0, 0, m] += -t * np.exp(-1j * kN)
    return SolvePoint(cfg, H, Hk, label=f"chain{nlat} t'={tprime:.4f}", params={"tprime": tprime})


# ---------------------------------------------------------------------------
# 2D square cluster Nx x Ny (configs 2, 5): site index N = Nx*(y-1)+x
# ---------------------------------------------------------------------------
def square_site(x: int, y: int, nx: int) -> int:
    return nx * y + x  # 0-based indices2N


def _square_hopping(nx, ny, nspin, t, H, spin_block=None):
    for s in range(nspin) if spin_block is None else [spin_block]:
        for x in range(nx):
            for y in range(ny):
                i = square_site(x, y, nx)
                for dx, dy in ((1, 0), (-1, 0), (0, 1), (0, -1)):
                    xx, yy = x + dx, y + dy
                    if 0 <= xx < nx and 0 <= yy < ny:
                        H[square_site(xx, yy, nx), i, s, s, 0, 0] = -t


def square(nx: int = 4, ny: int = 3, U: float = 8.0, xmu: float = 4.0, t: float = 1.0,
           tprime: Optional[float] = None, maf: float = 0.0, nspin: int = 2, nkx: int = 32,
           nky: int = 32, ngfiter: int = 200, omega_nodes: int = 8192, mu_shift: float = 0.0,
           cdw: float = 0.0, **cfgkw) -> SolvePoint:
    """Square Hubbard cluster with an antiferromagnetic Weiss field M on the
    cluster only: Hloc(i,i,s,s) += M*(-1)^(x+y)*(+1 up / -1 down), and
    optionally a staggered charge field cdw*(-1)^(x+y) on both spins (the
    surrogate's fourth input on a one-orbital cluster, where a uniform
    orbital energy would only repeat mu')."""
    nlat = nx * ny
    tp = t if tprime is None else tprime
    cfg = lanczos_cfg(Nlat=nlat, Norb=1, Nspin=nspin, Uloc=[U], hfmode=0, xmu=xmu,
                      lanc_ngfiter=ngfiter, omega_nodes=omega_nodes, **cfgkw)
    H = _zeros(nlat, nlat, nspin, nspin, 1, 1)
    _square_hopping(nx, ny, nspin, tp, H)
    for x in range(nx):
        for y in range(ny):
            i = square_site(x, y, nx)
            for s in range(nspin):
                sz = 1.0 if s == 0 else -1.0
                H[i, i, s, s, 0, 0] += -mu_shift + (maf * (-1) ** (x + y) * sz if nspin == 2 else 0.0)
                H[i, i, s, s, 0, 0] += cdw * (-1) ** (x + y)
    nk = nkx * nky
    Hk = _zeros(nlat, nlat, nspin, nspin, 1, 1, nk)
    base = _zeros(nlat, nlat, nspin, nspin, 1, 1)
    _square_hopping(nx, ny, nspin, t, base)
    ik = 0
    for a in range(nkx):
        for b in range(nky):
            kxN = 2.0 * np.pi * a / nkx  # kx*Nx, reduced zone
            kyN = 2.0 * np.pi * b / nky
            Hk[..., ik] = base
            for s in range(nspin):  # boundary terms (vca_hm_2dsquare_bath.f90:254-267)
                for y in range(ny):
                    i1, i2 = square_site(0, y, nx), square_site(nx - 1, y, nx)
                    Hk[i2, i1, s, s, 0, 0, ik] += -t * np.exp(1j * kxN)
                    Hk[i1, i2, s, s, 0, 0, ik] += -t * np.exp(-1j * kxN)
                for x in range(nx):
                    i1, i2 = square_site(x, 0, nx), square_site(x, ny - 1, nx)
                    Hk[i2, i1, s, s, 0, 0, ik] += -t * np.exp(1j * kyN)
                    Hk[i1, i2, s, s, 0, 0, ik] += -t * np.exp(-1j * kyN)
            ik += 1
    return SolvePoint(cfg, H, Hk, label=f"square{nx}x{ny} M={maf:.4f}",
                      params={"maf": maf, "tprime": tp, "mu_shift": mu_shift, "cdw": cdw})


# ---------------------------------------------------------------------------
# 2x2 cluster with 8 bath levels (config 3)
# ---------------------------------------------------------------------------
def bath_base(nb: int = 8, nlat: int = 4, seed: int = SEED):
    rng = np.random.Generator(np.random.PCG64(seed))
    A = rng.normal(0.0, 0.5, size=(nb, nb))
    h = (A + A.T) / np.sqrt(2.0)
    v = rng.uniform(-0.5, 0.5, size=(nlat, nb))
    return h, v


def square_bath(s_h: float = 1.0, s_v: float = 1.0, mu_prime: float = 2.0, U: float = 4.0,
                t: float = 1.0, nk1: int = 24, ngfiter: int = 200, omega_nodes: int = 4096,
                nb: int = 8, seed: int = SEED, **cfgkw) -> SolvePoint:
    nx = ny = 2
    nlat = 4
    xmu = U / 2.0
    cfg = lanczos_cfg(Nlat=nlat, Norb=1, Nspin=1, Nlat_bath=nb, Norb_bath=1, Uloc=[U], hfmode=0,
                      xmu=xmu, lanc_ngfiter=ngfiter, omega_nodes=omega_nodes, **cfgkw)
    h0, v0 = bath_base(nb, nlat, seed)
    pt = square(nx, ny, U=U, xmu=xmu, t=t, nspin=1, nkx=nk1, nky=nk1, ngfiter=ngfiter,
                omega_nodes=omega_nodes, mu_shift=(mu_prime - xmu))
    bh = _zeros(nb, nb, 1, 1, 1, 1)
    bh[:, :, 0, 0, 0, 0] = s_h * h0
    bv = _zeros(nlat, nb, 1, 1, 1, 1)
    bv[:, :, 0, 0, 0, 0] = s_v * v0
    return SolvePoint(cfg, pt.Hloc, pt.Hk, bh, bv, label=f"2x2+{nb}bath",
                      params={"s_h": s_h, "s_v": s_v, "mu_prime": mu_prime})


# ---------------------------------------------------------------------------
# BHZ two-orbital 2x2 cluster (config 4)
# ---------------------------------------------------------------------------
SX = np.array([[0, 1], [1, 0]], dtype=np.complex128)
SZ = np.array([[1, 0], [0, -1]], dtype=np.complex128)


def _t_m(mass):
    return mass * SZ


def _t_x(hop1, hop2, spin):  # vca_bhz_2d.f90:443-452
    sz = (-1.0) ** spin  # spinsign = spin+1 (1-based) -> (-1)^(spinsign+1)
    return -hop1 * SZ + 0.5 * sz * 1j * hop2 * SX


def _t_y(hop1, hop2):  # vca_bhz_2d.f90:454-462
    m = -hop1 * SZ
    m[0, 1] = -hop2 * 0.5
    m[1, 0] = hop2 * 0.5
    return m


def bhz(mass: float = 2.0, lam: float = 0.3, t: float = 1.0, U: float = 2.0, Jfrac: float = 0.25,
        delta: float = 0.0, nk1: int = 48, ngfiter: int = 200, omega_nodes: int = 4096,
        **cfgkw) -> SolvePoint:
    """BHZ 2x2 cluster.  The variational orbital splitting delta enters as an
    on-site orbital mixing delta*tau_x: a delta*tau_z term would only shift
    the mass M' and so is degenerate with it."""
    nx = ny = 2
    nlat, norb, nspin = 4, 2, 2
    J = Jfrac * U
    cfg = lanczos_cfg(Nlat=nlat, Norb=norb, Nspin=nspin, Uloc=[U, U], Ust=U - 2.0 * J, Jh=J,
                      hfmode=1, xmu=0.0, lanc_ngfiter=ngfiter, omega_nodes=omega_nodes, **cfgkw)

    def build(m_val, phase_x=None, phase_y=None, add_delta=0.0):
        H = _zeros(nlat, nlat, nspin, nspin, norb, norb)
        for s in range(nspin):  # generate_tcluster (vca_bhz_2d.f90:312-345)
            for x in range(nx):
                for y in range(ny):
                    i1 = square_site(x, y, nx)
                    H[i1, i1, s, s] = _t_m(m_val) + add_delta * SX
                    if x < nx - 1:
                        H[square_site(x + 1, y, nx), i1, s, s] = _t_x(t, lam, s)
                    if x > 0:
                        H[square_site(x - 1, y, nx), i1, s, s] = np.conj(_t_x(t, lam, s)).T
                    if y < ny - 1:
                        H[square_site(x, y + 1, nx), i1, s, s] = _t_y(t, lam)
                    if y > 0:
                        H[square_site(x, y - 1, nx), i1, s, s] = _t_y(t, lam).T
            if phase_x is not None:  # tk boundary terms (vca_bhz_2d.f90:380-393)
                for y in range(ny):
                    i1, i2 = square_site(0, y, nx), square_site(nx - 1, y, nx)
                    H[i2, i1, s, s] += np.conj(_t_x(t, lam, s)).T * np.exp(1j * phase_x)
                    H[i1, i2, s, s] += _t_x(t, lam, s) * np.exp(-1j * phase_x)
                for x in range(nx):
                    i1, i2 = square_site(x, 0, nx), square_site(x, ny - 1, nx)
                    H[i2, i1, s, s] += _t_y(t, lam).T * np.exp(1j * phase_y)
                    H[i1, i2, s, s] += _t_y(t, lam) * np.exp(-1j * phase_y)
        return H

    Hloc = build(mass, add_delta=delta)
    nk = nk1 * nk1
    Hk = _zeros(nlat, nlat, nspin, nspin, norb, norb, nk)
    ik = 0
    for a in range(nk1):
        for b in range(nk1):
            Hk[..., ik] = build(2.0, 2 * np.pi * a / nk1, 2 * np.pi * b / nk1)
            ik += 1
    return SolvePoint(cfg, Hloc, Hk, label="bhz2x2", params={"mass": mass, "delta": delta})


def batch_square_bath(B: int = 256, seed: int = SEED, **kw):
    """Config 3 batch: (s_h, s_v, mu') ~ U([0.5,1.5]x[0.5,1.5]x[1.5,2.5])."""
    rng = np.random.Generator(np.random.PCG64(seed + 3))
    pts = rng.uniform([0.5, 0.5, 1.5], [1.5, 1.5, 2.5], size=(B, 3))
    return [square_bath(s_h=p[0], s_v=p[1], mu_prime=p[2], **kw) for p in pts]


def batch_bhz(B: int = 1024, seed: int = SEED, **kw):
    """Config 4 batch: M' ~ U[1.5,2.5], delta ~ U[-0.2,0.2]."""
    rng = np.random.Generator(np.random.PCG64(seed + 4))
    pts = rng.uniform([1.5, -0.2], [2.5, 0.2], size=(B, 2))
    return [bhz(mass=p[0], delta=p[1], **kw) for p in pts]


# ---------------------------------------------------------------------------
# The stationary-point search problem of the surrogate: a 2x2 cluster stands
# in for the 4x4 one (whose single solve takes minutes), same inputs
# ---------------------------------------------------------------------------
SEARCH_PARAMS = ("tprime", "maf", "cdw")
SEARCH_LO = np.array([1.1, 0.2, -0.2])
SEARCH_HI = np.array([1.7, 0.55, 0.2])


def search_point(p, nkx: int = 8, ngfiter: int = 100, omega_nodes: int = 512) -> SolvePoint:
    """2x2 Hubbard cluster at half filling (U = 8, xmu = 4, Nspin = 2) with
    variational (t', M_AF, staggered charge field), 8x8 k-grid.  Omega has an
    interior stationary point in the box SEARCH_LO..SEARCH_HI near
    (1.35, 0.33, 0): a minimum in t' and M_AF, a maximum in the charge field.
    (A cluster mu' would enter Omega linearly here, with slope -<N> = -4, so
    it has no stationary point and is not searched.)"""
    return square(nx=2, ny=2, U=8.0, xmu=4.0, tprime=float(p[0]), maf=float(p[1]), cdw=float(p[2]), nspin=2,
                  nkx=nkx, nky=nkx, ngfiter=ngfiter, omega_nodes=omega_nodes)
