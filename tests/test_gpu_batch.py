"""The batched form of vca_gpu_solve_batch (many variational points per launch)
against a loop of plain vca_gpu_solve calls, and against the oracle's
fixtures at the full C3/C4 configurations.

Tolerances: Omega 1e-10 relative (the batched form runs in FP64; the loop
runs the default arithmetic, fixed point where it applies).  After a batch
the context holds the last point's solve, as a loop of vca_solve leaves it.
"""
import os

import numpy as np
import pytest

from vca_gb300 import clusters
from vca_gb300.solver import VcaSolver

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
E_TOL = 1e-10


def _rel(a, b):
    return abs(a - b) / max(1.0, abs(b))


def _stack(pts):
    Hl = np.stack([p.Hloc for p in pts], axis=-1)
    bh = np.stack([p.bath_h for p in pts], axis=-1) if pts[0].bath_h is not None else None
    bv = np.stack([p.bath_v for p in pts], axis=-1) if pts[0].bath_v is not None else None
    return Hl, bh, bv


def _small(name):
    rng = np.random.default_rng(len(name))
    if name == "bath2x2+4":
        return [clusters.square_bath(s_h=a, s_v=b, mu_prime=m, nb=4, nk1=6, ngfiter=60, omega_nodes=256)
                for a, b, m in rng.uniform([0.5, 0.5, 1.5], [1.5, 1.5, 2.5], size=(4, 3))]
    if name == "bhz":
        return [clusters.bhz(mass=m, delta=d, nk1=4, ngfiter=60, omega_nodes=256)
                for m, d in rng.uniform([1.5, -0.2], [2.5, 0.2], size=(4, 2))]
    if name == "square2x2_afm":
        return [clusters.square(nx=2, ny=2, U=8.0, xmu=4.0, maf=float(m), nspin=2, nkx=6, nky=6, ngfiter=80,
                                omega_nodes=256) for m in (0.0, 0.1, 0.2, 0.3)]
    if name == "chain4":
        return [clusters.chain1d(tprime=float(t), nlat=4, U=4.0, xmu=2.0, nk=16, ngfiter=100, omega_nodes=256)
                for t in (0.85, 0.95, 1.05, 1.15)]
    raise KeyError(name)


@pytest.mark.parametrize("name", ["bath2x2+4", "bhz", "square2x2_afm", "chain4"])
def test_batched_form_equals_a_loop_of_plain_solves(name):
    pts = _small(name)
    Hl, bh, bv = _stack(pts)
    s = VcaSolver(pts[0].cfg, pts[0].bath_h, pts[0].bath_v)
    om = s.solve_batch(Hl, pts[0].Hk, bh, bv)
    last = s.energies()
    ref = []
    for p in pts:
        r = VcaSolver(p.cfg, p.bath_h, p.bath_v)
        ref.append(r.solve(p.Hloc, p.Hk, p.bath_h, p.bath_v))
        e_last = r.energies()
    for a, b in zip(om, ref):
        assert _rel(a, b) < E_TOL, (name, a, b)
    assert _rel(last[0], e_last[0]) < E_TOL and _rel(last[1], e_last[1]) < E_TOL


def test_batch_loop_switch_gives_the_same_values():
    pts = _small("bhz")
    Hl, bh, bv = _stack(pts)
    cfg = pts[0].cfg.copy()
    cfg.batch_loop = 1
    a = VcaSolver(cfg).solve_batch(Hl, pts[0].Hk)
    b = VcaSolver(pts[0].cfg).solve_batch(Hl, pts[0].Hk)
    np.testing.assert_allclose(a, b, rtol=E_TOL, atol=0)


def test_sector_at_a_time_search_equals_the_batched_search():
    """The reference's loop over sectors (one Lanczos run per sector) and the
    batched multi-sector search give the same sector energies and Omega."""
    for pt in (_small("bath2x2+4")[0], _small("square2x2_afm")[2]):
        vals = []
        for mode in (0, 1):
            cfg = pt.cfg.copy()
            cfg.sector_at_a_time = mode
            s = VcaSolver(cfg, pt.bath_h, pt.bath_v)
            om = s.solve(pt.Hloc, pt.Hk, pt.bath_h, pt.bath_v)
            vals.append((om, s.sector_energies()))
        assert _rel(vals[0][0], vals[1][0]) < E_TOL
        np.testing.assert_allclose(vals[0][1], vals[1][1], rtol=1e-12, atol=1e-12)


def _fixture(name):
    return dict(np.load(os.path.join(GOLD, f"config_{name}.npz")))


@pytest.mark.parametrize("which", ["c3", "c4"])
def test_batched_full_configs_against_the_oracle(which):
    """Three points of the C3 (2x2 + 8 bath levels, 24x24 k, 200-step chains,
    4096 nodes) or C4 (BHZ 2x2, 48x48 k) batch: the first against the oracle's
    fixture (E_gs, the Omega integral and Omega at 1e-10, the ground-state
    sectors), all three against plain solves."""
    if which == "c3":
        pts = clusters.batch_square_bath(B=3)
        fx = _fixture("c3_p0")
    else:
        pts = clusters.batch_bhz(B=3)
        fx = _fixture("c4_p0")
    Hl, bh, bv = _stack(pts)
    s = VcaSolver(pts[0].cfg, pts[0].bath_h, pts[0].bath_v)
    om = s.solve_batch(Hl, pts[0].Hk, bh, bv)
    assert _rel(om[0], float(fx["sft"])) < E_TOL, (om[0], fx["sft"])
    p = pts[0]
    r = VcaSolver(p.cfg, p.bath_h, p.bath_v)
    plain0 = r.solve(p.Hloc, p.Hk, p.bath_h, p.bath_v)
    egs, oi = r.energies()
    assert _rel(plain0, float(fx["sft"])) < E_TOL
    assert _rel(egs, float(fx["egs"])) < E_TOL and _rel(oi, float(fx["omega_int"])) < E_TOL
    assert sorted(x[0] for x in r.states()) == sorted(int(v) for v in fx["states"])
    se = r.sector_energies()
    np.testing.assert_allclose(se, fx["sector_e"], rtol=E_TOL, atol=E_TOL)
    g = r.gf_cluster(1j * fx["wg"])
    np.testing.assert_allclose(g, fx["g"], rtol=0, atol=1e-8)
    for p, o in zip(pts[1:], om[1:]):
        r = VcaSolver(p.cfg, p.bath_h, p.bath_v)
        assert _rel(o, r.solve(p.Hloc, pts[0].Hk, p.bath_h, p.bath_v)) < E_TOL


@pytest.mark.parametrize("name", ["bath2x2+4", "bhz", "square2x2_afm", "chain4"])
def test_sector_bounds_are_below_every_sector_energy(name):
    """The one-body lower bound the batched form screens sectors with is at
    most each sector's lowest energy (plain solve, every sector searched)."""
    pt = _small(name)[1]
    s = VcaSolver(pt.cfg, pt.bath_h, pt.bath_v)
    s.solve(pt.Hloc, pt.Hk, pt.bath_h, pt.bath_v)
    e = s.sector_energies()
    b = s.sector_bounds()
    assert np.all(b <= e + 1e-9 * np.maximum(1.0, np.abs(e))), (b - e).max()


def test_screened_and_full_batched_searches_agree():
    """Screening skips (point, sector) searches; Omega is unchanged."""
    pts = clusters.batch_square_bath(B=3, nk1=6, ngfiter=60, omega_nodes=256)
    Hl, bh, bv = _stack(pts)
    vals, skipped = [], []
    for flag in (0, 1):
        cfg = pts[0].cfg.copy()
        cfg.no_sector_screen = flag
        s = VcaSolver(cfg, pts[0].bath_h, pts[0].bath_v)
        vals.append(s.solve_batch(Hl, pts[0].Hk, bh, bv))
        skipped.append(s.timings(batched=True)[6])
    np.testing.assert_allclose(vals[0], vals[1], rtol=E_TOL, atol=0)
    assert skipped[0] > 0 and skipped[1] == 0, skipped


def test_autotuned_and_fixed_chain_shapes_agree():
    """The chains' tile shape the autotuner picks changes only the order of
    the dot products' sums: Omega agrees with the fixed shape to 1e-12."""
    pts = _small("bhz")
    Hl, bh, bv = _stack(pts)
    vals, shapes = [], []
    for on in (True, False):
        s = VcaSolver(pts[0].cfg)
        s.set_autotune(on)
        vals.append(s.solve_batch(Hl, pts[0].Hk))
        shapes.append(tuple(s.timings(batched=True)[7:9]))
    np.testing.assert_allclose(vals[0], vals[1], rtol=1e-12, atol=0)
    assert shapes[1] == (64, 8)
    assert shapes[0][0] in (64, 256, 1024) and shapes[0][1] in (4, 8, 16)
