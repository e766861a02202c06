"""The solve's host-side state-list logic against the oracle's, without a
GPU: the library's vca_state_list_t0 / vca_state_list_finite_t (the replay
the solve runs on the batched search's sector energies) and the oracle's
restatement on thousands of seeded energy sets.

Energies are drawn in clusters around a few levels with offsets at and
around the thresholds (GS_THRESHOLD, 10*GS_THRESHOLD, the CUTOFF spread),
exact ties included.  The lists (sectors and order), zeta, E_min and the
adjusted LANC_NSTATES_TOTAL must be identical, bit for bit.
"""
import numpy as np
import pytest

from vca_gb300 import clusters
from vca_gb300.config import default_config
from vca_gb300.solver import state_list_finite_t, state_list_t0
from oracle import oracle as orc
from oracle.oracle import Oracle

OFFSETS = np.array([0.0, 0.0, 1e-10, 5e-10, 1e-9, 1.5e-9, 9e-9, 1e-8, 1.1e-8, 1e-7, 0.01, 0.3, 1.0, 4.0])


def energies(rng):
    n = int(rng.choice([1, 2, 9, 25, 81, 169, 289]))
    levels = rng.normal(scale=3.0, size=int(rng.integers(1, 4)))
    E = levels[rng.integers(0, len(levels), size=n)]
    E = E + rng.choice(OFFSETS, size=n) * rng.choice([-1.0, 1.0], size=n)
    return E


@pytest.mark.parametrize("seed", range(4))
def test_t0_list_matches_oracle(seed):
    rng = np.random.default_rng(1000 + seed)
    for _ in range(500):
        E = energies(rng)
        thr = float(rng.choice([1e-9, 1e-8, 0.0]))
        assert state_list_t0(E, thr) == orc.state_list_t0(E, thr)


@pytest.mark.parametrize("seed", range(4))
def test_finite_t_list_matches_oracle(seed):
    rng = np.random.default_rng(2000 + seed)
    for _ in range(300):
        E = energies(rng)
        cfg = default_config(beta=float(rng.choice([0.5, 3.0, 20.0, 200.0])),
                             cutoff=float(rng.choice([1e-9, 1e-6, 0.1])),
                             lanc_nstates_step=int(rng.integers(0, 4)),
                             lanc_niter_spectrum=int(rng.integers(1, 12)))
        nt = 2 * int(rng.integers(1, 6))
        got = state_list_finite_t(E, cfg, nt)
        ref = orc.state_list_finite_t(E, cfg, nt)
        assert got == ref, (E.tolist(), got, ref)


def test_replays_are_what_the_oracle_solve_keeps():
    """The oracle's pure replays on its own sector energies give the state
    lists of its solves (T=0 and finite T)."""
    pt = clusters.square(nx=2, ny=2, U=8.0, xmu=0.95, maf=0.0, nspin=1, nkx=4, nky=4, ngfiter=40,
                         omega_nodes=64)
    o = Oracle.from_point(pt)
    o.diagonalize()
    assert [s for s, _ in orc.state_list_t0(o.sector_energies(), pt.cfg.gs_threshold)] == [s for s, _ in o.states()]
    ft = clusters.square(nx=2, ny=2, U=8.0, xmu=4.0, maf=0.2, nspin=2, nkx=4, nky=4, ngfiter=40, omega_nodes=64)
    cfg = ft.cfg.copy()
    cfg.lanc_nstates_total, cfg.beta, cfg.bandwidth = 2, 8.0, 8.0
    ft.cfg = cfg
    o = Oracle.from_point(ft)
    o.diagonalize()
    sec, zeta, emin, nt = orc.state_list_finite_t(o.sector_energies(), cfg, 2)
    assert sec == [s for s, _ in o.states()] and nt == o.thermal()["nstates_total"]
    assert zeta == o.thermal()["zeta"] and emin == min(e for _, e in o.states())
