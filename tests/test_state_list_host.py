"""The solve's host-side state-list logic against the oracle's, without a
GPU: the library's vca_state_list_t0 / vca_state_list_finite_t (the replay
the solve runs on the batched search's sector energies) and the oracle's
restatement on thousands of seeded energy sets.

Energies are drawn in clusters around a few levels with offsets at and
around the thresholds (GS_THRESHOLD, 10*GS_THRESHOLD, the CUTOFF spread),
exact ties included.  The lists (sectors and order), zeta, E_min and the
adjusted LANC_NSTATES_TOTAL must be identical, bit for bit.

Also host logic of the Omega integral: the k-point pairing of the k-sum
(vca_pair_kpoints) against a brute-force pairing and known counts, and the
contour rule's nodes (vca_contour_rule) against the oracle's (1e-15).
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


def _brute_pairs(Hk):
    """Greedy pairing in k order by direct comparison (the reference sums
    every k; pairing is this library's, so the check is the property: each
    weight-2 representative has exactly one partner H_k' = conj(H_k))."""
    Nk = Hk.shape[-1]
    H = Hk.reshape(-1, Nk, order="F")
    tol = 1e-13 * (1.0 + np.abs(np.concatenate([H.real.ravel(), H.imag.ravel()])).max())
    used = np.zeros(Nk, bool)
    reps, wts = [], []
    for k in range(Nk):
        if used[k]:
            continue
        used[k] = True
        cand = [j for j in range(Nk) if not used[j]
                and np.all(np.abs(H[:, j].real - H[:, k].real) <= tol)
                and np.all(np.abs(H[:, j].imag + H[:, k].imag) <= tol)]
        reps.append(k)
        wts.append(2.0 if cand else 1.0)
        if cand:
            used[cand[0]] = True
    return np.array(reps), np.array(wts)


@pytest.mark.parametrize("make", [
    lambda: clusters.square(nx=4, ny=3, U=8.0, xmu=4.0, maf=0.1, nspin=2, nkx=32, nky=32, ngfiter=20,
                            omega_nodes=64),
    lambda: clusters.chain1d(tprime=1.0, nlat=4, U=4.0, xmu=2.0, nk=64, ngfiter=20, omega_nodes=64),
    lambda: clusters.bhz(mass=2.2, delta=0.1, nk1=12, ngfiter=20, omega_nodes=64),
    lambda: clusters.square_bath(nb=4, nk1=8, ngfiter=20, omega_nodes=64),
])
def test_kpoint_pairs_match_brute_force(make):
    from vca_gb300.solver import pair_kpoints
    pt = make()
    reps, w = pair_kpoints(pt.Hk)
    assert w.sum() == pt.Nk and np.all(np.diff(reps) > 0)
    if pt.Nk <= 256:
        r2, w2 = _brute_pairs(pt.Hk)
        # generic grids pair uniquely: the same representatives and weights
        np.testing.assert_array_equal(reps, r2)
        np.testing.assert_array_equal(w, w2)


def test_kpoint_pairs_known_counts_and_random():
    from vca_gb300.solver import pair_kpoints
    pt = clusters.square(nx=4, ny=3, U=8.0, xmu=4.0, maf=0.1, nspin=2, nkx=32, nky=32, ngfiter=20, omega_nodes=64)
    assert len(pair_kpoints(pt.Hk)[0]) == 514  # the benchmark grid: 514 of 1024 points
    rng = np.random.default_rng(4)
    H = rng.normal(size=(3, 3, 1, 1, 1, 1, 40)) + 1j * rng.normal(size=(3, 3, 1, 1, 1, 1, 40))
    reps, w = pair_kpoints(H)
    assert len(reps) == 40 and np.all(w == 1.0)  # no conjugate partners
    H[..., 7] = np.conj(H[..., 30])
    reps, w = pair_kpoints(H)
    assert len(reps) == 39 and w[list(reps).index(7)] == 2.0 and 30 not in reps


def test_contour_rule_matches_oracle():
    from vca_gb300.solver import contour_rule
    rng = np.random.default_rng(6)
    for _ in range(200):
        R = float(rng.uniform(1.0, 60.0))
        beta = float(rng.choice([0.5, 5.0, 40.0, 400.0]))
        mu = float(rng.uniform(-1.2, 1.2)) * R
        ngl = int(rng.choice([2, 8, 24]))
        th, w = contour_rule(R, beta, mu, ngl)
        th2, w2 = orc.contour_rule(R, beta, mu, ngl)
        assert len(th) == len(th2)
        np.testing.assert_allclose(th, th2, rtol=0, atol=1e-15)
        np.testing.assert_allclose(w, w2, rtol=0, atol=1e-15)
        assert abs(w.sum() - np.pi) < 1e-12 and np.all(np.diff(th) > 0)


def test_hooks_reject_bad_arguments():
    from vca_gb300.solver import VcaError
    with pytest.raises(VcaError) as e:
        state_list_finite_t(np.array([0.0, 1.0]), default_config(beta=1.0), 0)
    assert e.value.code == -9
    with pytest.raises(VcaError) as e:
        state_list_finite_t(np.array([0.0]), default_config(beta=1.0, cutoff=1.0), 2)
    assert e.value.code == -1
    assert state_list_finite_t(np.zeros(0), default_config(beta=1.0), 2)[0] == []
