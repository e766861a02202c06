"""The surrogate-guided stationary-point search against the plain searches,
on the 2x2 cluster's (t', M_AF, charge field) box (vca_gb300/clusters.py
search_point): every Omega is a plain FP64 GPU solve, counted.

* The plain Newton search (central differences of plain solves) converges to
  the interior stationary point; the coordinate-wise Brent search (the
  drivers' one-parameter tool, cycled) reaches the same Omega (1e-9).
* The surrogate search reaches the plain stationary value within 1e-6 using
  at most a fifth of the coordinate-wise Brent search's solver calls and
  fewer than half of Newton's; every accepted point was re-solved plainly
  and the surrogate's error there is recorded.
* What the network gains: the best of the solves the surrogate search spent
  on its space-filling design is far from stationary (|dOmega| > 1e-4), and
  Newton stopped after as many solver calls as the surrogate search used is
  not within 1e-6 either.
"""
import numpy as np
import pytest

from vca_gb300 import clusters
from vca_gb300.solver import VcaSolver
from vca_gb300.surrogate import CountingSolver, coordinate_brent_search, newton_fd_search, surrogate_search

pytestmark = pytest.mark.gpu

LO, HI = clusters.SEARCH_LO, clusters.SEARCH_HI
P0 = 0.5 * (LO + HI)


@pytest.fixture(scope="module")
def solve():
    pt = clusters.search_point(P0)
    s = VcaSolver(pt.cfg)
    s.upload_hk(pt.Hk)
    yield lambda p: s.solve_resident(clusters.search_point(p).Hloc)
    s.close()


def test_surrogate_search_reaches_the_plain_stationary_point(solve):
    f_n = CountingSolver(solve)
    p_n, om_n, it = newton_fd_search(f_n, P0, LO, HI)
    assert it < 25
    f_b = CountingSolver(solve)
    p_b, om_b, _ = coordinate_brent_search(f_b, P0, LO, HI, ["min", "min", "max"])
    assert abs(om_b - om_n) < 1e-9
    f_s = CountingSolver(solve)
    p_s, om_s, hist = surrogate_search(f_s, LO, HI, P0, n_design=10, steps=4000)
    assert abs(om_s - om_n) < 1e-6, (om_s, om_n)
    assert 5 * f_s.calls <= f_b.calls, (f_s.calls, f_b.calls)
    assert 2 * f_s.calls < f_n.calls, (f_s.calls, f_n.calls)
    assert all(np.isfinite(h["surrogate_error"]) for h in hist)
    # the design alone, and Newton on the same budget, are not stationary
    design = [v for _, v in f_s.log[:11]]
    assert min(abs(v - om_n) for v in design) > 1e-4
    f_c = CountingSolver(solve)
    _, om_c, _ = newton_fd_search(f_c, P0, LO, HI, maxit=max(1, f_s.calls // 19))
    assert f_c.calls <= f_s.calls + 1 and abs(om_c - om_n) > 1e-6
