"""GPU parity of the finite-temperature path (LANC_NSTATES_TOTAL > 1)
through the C-ABI against the CPU oracle.

Compared: the annealed state list (the same sectors, energies 1e-10
relative), zeta / Omega' (1e-10 relative), nmax, the contour radius and node
count (exact), the Matsubara and contour parts and the SFT potential (1e-10
relative), the complex integrand on the contour (1e-10), G'(z) (1e-8
absolute) and the Boltzmann-weighted observables (1e-10), plus the
carry-over of the adapted LANC_NSTATES_TOTAL into the next solve.

max_exc is the largest Ritz value of chains run without reorthogonalisation
from ground-state vectors that meet a 1e-11 residual, so it is set by
rounding: the oracle alone moves it by 1.9e-7 relative across Lanczos start
seeds on bhz_b10 (tests/test_oracle_finite_t.py measures this).  It enters
Omega only through nmax = int(2(|max_exc| + bandwidth) beta / pi) and the
radius R = 2 (nmax + 1) pi / beta, which are compared exactly; max_exc itself
is compared at MAX_EXC_TOL, and every model keeps the nmax argument further
than that tolerance from an integer, so that the exact comparison is sound.
"""
import numpy as np
import pytest

from vca_gb300 import clusters
from vca_gb300.clusters import nnn2lso
from vca_gb300.solver import VcaSolver
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

E_TOL = 1e-10
G_TOL = 1e-8
MAX_EXC_TOL = 1e-6


def _ft(pt, beta, bandwidth, nstates=2, **kw):
    cfg = pt.cfg.copy()
    cfg.lanc_nstates_total, cfg.beta, cfg.bandwidth = nstates, beta, bandwidth
    for k, v in kw.items():
        setattr(cfg, k, v)
    pt.cfg = cfg
    return pt


POINTS = {
    "atom_b2": lambda: _ft(clusters.chain1d(tprime=0.0, t=0.0, nlat=1, U=4.0, xmu=2.0, nk=4, ngfiter=8,
                                            omega_nodes=64), 2.0, 0.0),
    "chain2_u0": lambda: _ft(clusters.chain1d(tprime=1.0, nlat=2, U=0.0, xmu=0.0, nk=32, ngfiter=50,
                                              omega_nodes=64), 20.0, 4.0),
    "square2x2_b10": lambda: _ft(clusters.square(nx=2, ny=2, U=4.0, xmu=2.0, maf=0.0, nspin=1, nkx=6, nky=6,
                                                 ngfiter=60, omega_nodes=64), 10.0, 8.0),
    "square2x2_eps_b10": lambda: _split(_ft(clusters.square(nx=2, ny=2, U=4.0, xmu=2.0, maf=0.0, nspin=1, nkx=6,
                                                            nky=6, ngfiter=60, omega_nodes=64), 10.0, 8.0)),
    "square2x2_afm_b8": lambda: _ft(clusters.square(nx=2, ny=2, U=8.0, xmu=4.0, maf=0.2, nspin=2, nkx=4,
                                                    nky=4, ngfiter=60, omega_nodes=64), 8.0, 8.0),
    "bath2x2+2_b10": lambda: _ft(clusters.square_bath(nb=2, nk1=4, ngfiter=40, omega_nodes=64), 10.0, 8.0),
    # beta = 10: the annealing converges and trims; at beta = 6 the sweeps run
    # out with the cap cutting through a 4-fold degenerate level, where which
    # members stay follows the rounding of each run
    "bhz_b10": lambda: _ft(clusters.bhz(mass=2.2, delta=0.1, nk1=4, ngfiter=40, omega_nodes=64), 10.0, 8.0),
}


def _split(pt):
    """Site energies that lift the plaquette's symmetry degeneracies."""
    for i, e in enumerate((0.0, 0.07, -0.04, 0.02)):
        pt.Hloc[i, i, 0, 0, 0, 0] += e
        pt.Hk[i, i, 0, 0, 0, 0, :] += e
    return pt


def _degenerate_sector_ground_state(o, states, dmax=1200):
    """True when a listed sector's lowest level is degenerate: one Lanczos
    vector in that subspace is as good as another (the reference takes
    whichever its start vector leads to), so G' and the observables depend on
    the run while Omega, zeta and the energies do not."""
    for isec, _ in states:
        if 1 < o.dim(isec) <= dmax:
            w = np.linalg.eigvalsh(o.dense_h(isec))
            if w[1] - w[0] < 1e-8:
                return True
    return False


def _rel(a, b):
    return abs(a - b) / max(1.0, abs(b))


def _assert_nmax_away_from_edge(cfg, max_exc):
    """nmax is compared exactly only where a max_exc error of MAX_EXC_TOL
    cannot move the integer part of its argument."""
    x = 2.0 * (abs(max_exc) + cfg.bandwidth) * cfg.beta / np.pi
    dx = 2.0 * MAX_EXC_TOL * max(1.0, abs(max_exc)) * cfg.beta / np.pi
    edge = min(x - np.floor(x), np.ceil(x) - x)
    assert edge > 10 * dx, f"nmax argument {x} within {edge:.2e} of an integer: choose another model"


@pytest.mark.parametrize("name", list(POINTS))
def test_finite_t_solve_matches_oracle(name):
    pt = POINTS[name]()
    s = VcaSolver(pt.cfg, pt.bath_h, pt.bath_v)
    o = Oracle.from_point(pt)
    for rep in range(2):  # the second solve starts from the adapted list size
        sft = s.solve(pt.Hloc, pt.Hk, pt.bath_h, pt.bath_v)
        sft_ref, emin_ref, oi_ref = o.solve()
        # the same sectors with the same energies; the order inside a group of
        # degenerate states follows the rounding of each run's energies
        st, st_ref = sorted(s.states()), sorted(o.states())
        assert [x[0] for x in st] == [x[0] for x in st_ref], (rep, st, st_ref)
        for (_, e), (_, er) in zip(st, st_ref):
            assert _rel(e, er) < E_TOL
        t, tr = s.thermal(), o.thermal()
        assert t["finite_t"] == 1 and t["nstates_total"] == tr["nstates_total"]
        for key in ("zeta", "omega_prime", "e_min", "sum_part", "contour_part"):
            assert _rel(t[key], tr[key]) < E_TOL, (rep, key, t[key], tr[key])
        assert _rel(t["max_exc"], tr["max_exc"]) < MAX_EXC_TOL, (rep, t["max_exc"], tr["max_exc"])
        _assert_nmax_away_from_edge(pt.cfg, tr["max_exc"])
        assert t["nmax"] == tr["nmax"] and t["contour_points"] == tr["contour_points"]
        assert t["integration_R"] == tr["integration_R"]
        assert _rel(sft, sft_ref) < E_TOL, (rep, sft, sft_ref)
    # integrand on the contour and G' off the axis
    R = t["integration_R"]
    z = R * np.exp(1j * np.array([0.05, 1.2, 1.9, 3.1]))
    f = s.sum_kmesh_complex(z)
    fr = np.array([o.sum_kmesh_complex(x) for x in z])
    np.testing.assert_allclose(f, fr, rtol=0, atol=E_TOL)
    if _degenerate_sector_ground_state(o, st_ref):
        assert name == "square2x2_b10"  # the symmetric plaquette: N=3 doublets
        return
    zz = np.array([0.4j, 1.3 + 0.2j, 5.0j])
    np.testing.assert_allclose(s.gf_cluster(zz), o.gf_cluster(zz), rtol=0, atol=G_TOL)
    got, ref = s.observables(), o.observables()
    for key in ref:
        np.testing.assert_allclose(got[key], ref[key], rtol=0, atol=E_TOL, err_msg=f"{name} {key}")


def test_finite_t_u0_half_filling_is_the_lattice_value():
    pt = POINTS["chain2_u0"]()
    beta = pt.cfg.beta
    s = VcaSolver(pt.cfg)
    sft = s.solve(pt.Hloc, pt.Hk)
    Hk = nnn2lso(pt.Hk)
    ex = 2 * np.mean([-np.sum(np.logaddexp(0.0, -beta * np.linalg.eigvalsh(Hk[:, :, k]))) / beta
                      for k in range(pt.Nk)])
    assert abs(sft - ex) < 1e-12 + 10 * np.exp(-2.0 * beta), (sft, ex)


def test_finite_t_fixed_point_and_fp64_agree():
    vals = []
    for arith in (2, 1):
        pt = POINTS["square2x2_afm_b8"]()
        pt.cfg.arith = arith
        s = VcaSolver(pt.cfg)
        vals.append((s.solve(pt.Hloc, pt.Hk), s.thermal()["zeta"], s.arith_info()[0]))
    (a, za, fa), (b, zb, fb) = vals
    assert fa == 1 and fb == 0
    assert _rel(a, b) < E_TOL and _rel(za, zb) < E_TOL
