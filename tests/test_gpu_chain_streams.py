"""The Green's-function chains with two column groups in flight on two
streams and one group after another (the default): each group computes
exactly what it computes alone, and the groups store their chains in the
same order, so Omega and G'(z) must agree bit for bit.  Fixed-point (3x3
Hubbard) and FP64 (2x2 + 4 bath levels, chan2) models."""
import numpy as np
import pytest

from vca_gb300 import clusters
from vca_gb300.solver import VcaSolver

pytestmark = pytest.mark.gpu


def _points():
    yield "square3x3-fx", clusters.square(nx=3, ny=3, U=8.0, xmu=4.0, maf=0.2, nspin=2, nkx=4, nky=4,
                                          ngfiter=40, omega_nodes=128)
    pt = clusters.square_bath(nb=4, nk1=6, ngfiter=40, omega_nodes=128)
    cfg = pt.cfg.copy()
    cfg.vca_gf_symmetric = 1
    pt.cfg = cfg
    yield "bath2x2+4-f64", pt


@pytest.mark.parametrize("name,pt", list(_points()), ids=lambda x: x if isinstance(x, str) else "")
def test_two_chain_streams_change_no_result(name, pt):
    zs = np.array([0.3j, 1.0 + 0.5j, -2.0 + 0.1j])
    out = []
    for n in (1, 2):
        s = VcaSolver(pt.cfg, pt.bath_h, pt.bath_v)
        s.set_chain_streams(n)
        om = s.solve(pt.Hloc, pt.Hk, pt.bath_h, pt.bath_v)
        G = s.gf_cluster(zs)
        out.append((om, G, s.chain_timings()[2]))
        s.close()
    assert out[0][0] == out[1][0], (out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
    assert out[1][2] >= 2  # at least one pair of groups ran together
