"""Committed golden fixtures (tests/golden/make_golden.py): the oracle must keep
reproducing them (CPU), and the CUDA path must match them (GPU).
Tolerances: E_gs, Omega 1e-10 relative; G'(i w) 1e-8 absolute."""
import os

import numpy as np
import pytest

from vca_gb300 import clusters

HERE = os.path.dirname(os.path.abspath(__file__))
CH = np.load(os.path.join(HERE, "golden", "chain4.npz"))
SM = np.load(os.path.join(HERE, "golden", "small_models.npz"))
MM = np.load(os.path.join(HERE, "golden", "mid_models.npz"))


def chain_point(tp):
    return clusters.chain1d(tprime=float(tp), nlat=4, U=4.0, xmu=2.0, nk=64, ngfiter=100, omega_nodes=4096)


def small_points():
    return {
        "sq2x2": clusters.square(nx=2, ny=2, U=8.0, xmu=4.0, maf=0.2, nspin=2, nkx=6, nky=6, ngfiter=80,
                                 omega_nodes=1024),
        "bath": clusters.square_bath(nb=2, nk1=6, ngfiter=60, omega_nodes=1024),
        "bhz": clusters.bhz(mass=2.2, delta=0.1, nk1=4, ngfiter=60, omega_nodes=1024),
    }


def mid_points():
    """The points of mid_models.npz (as make_golden.mid_points)."""
    sq = clusters.square(nx=3, ny=3, U=8.0, xmu=4.0, maf=0.1, nspin=2, nkx=8, nky=8, ngfiter=100,
                         omega_nodes=2048)
    ft = clusters.square(nx=3, ny=3, U=8.0, xmu=4.0, maf=0.1, nspin=2, nkx=8, nky=8, ngfiter=80,
                         omega_nodes=256)
    c = ft.cfg.copy()
    c.lanc_nstates_total, c.beta, c.bandwidth = 2, 10.0, 8.0
    ft.cfg = c
    bath = clusters.square_bath(nb=6, nk1=6, ngfiter=80, omega_nodes=1024)
    return {"sq3x3": sq, "sq3x3_b10": ft, "bath6": bath}


def _rel(a, b):
    return abs(a - float(b)) / max(1.0, abs(float(b)))


def test_oracle_reproduces_mid_fixture():
    from oracle.oracle import Oracle
    pt = mid_points()["sq3x3"]
    o = Oracle.from_point(pt)
    sft, egs, _ = o.solve()
    assert _rel(sft, MM["sq3x3_sft"]) < 1e-12 and _rel(egs, MM["sq3x3_egs"]) < 1e-12
    assert np.abs(o.gf_cluster(1j * MM["wg"]) - MM["sq3x3_g"]).max() < 1e-12


@pytest.mark.parametrize("idx", [0, 10, 20])
def test_oracle_reproduces_chain_fixture(idx):
    from oracle.oracle import Oracle
    o = Oracle.from_point(chain_point(CH["tprime"][idx]))
    sft, egs, oi = o.solve()
    assert abs(egs - CH["egs"][idx]) < 1e-12 * abs(egs)
    assert abs(sft - CH["sft"][idx]) < 1e-12 * abs(sft)


@pytest.mark.gpu
def test_gpu_chain_sweep_matches_fixture():
    from vca_gb300.solver import VcaSolver
    s = None
    for i, tp in enumerate(CH["tprime"]):
        pt = chain_point(tp)
        if s is None:
            s = VcaSolver(pt.cfg)
        om = s.solve(pt.Hloc, pt.Hk)
        egs, oi = s.energies()
        assert abs(egs - CH["egs"][i]) <= 1e-10 * abs(CH["egs"][i])
        assert abs(om - CH["sft"][i]) <= 1e-10 * abs(CH["sft"][i]), (tp, om, CH["sft"][i])
        if abs(tp - 1.0) < 1e-12:
            np.testing.assert_allclose(s.sector_energies(), CH["sector_e_t1"], rtol=1e-10, atol=1e-10)
            g = s.gf_cluster(1j * CH["wg"])
            assert np.abs(g - CH["g_t1"]).max() < 1e-8


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["sq2x2", "bath", "bhz"])
def test_gpu_small_models_match_fixture(name):
    from vca_gb300.solver import VcaSolver
    pt = small_points()[name]
    s = VcaSolver(pt.cfg, pt.bath_h, pt.bath_v)
    om = s.solve(pt.Hloc, pt.Hk, pt.bath_h, pt.bath_v)
    egs, oi = s.energies()
    assert abs(egs - SM[name + "_egs"]) <= 1e-10 * abs(SM[name + "_egs"])
    assert abs(om - SM[name + "_sft"]) <= 1e-10 * abs(SM[name + "_sft"])
    g = s.gf_cluster(1j * SM["wg"])
    assert np.abs(g - SM[name + "_g"]).max() < 1e-8


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["sq3x3", "sq3x3_b10", "bath6"])
def test_gpu_mid_models_match_fixture(name):
    """Sectors larger than the oracle runs inside these tests: the 3x3 AFM
    cluster (up to 15,876 states; fixed point) at T=0 and at beta=10, and
    the 2x2 cluster with 6 bath levels (up to 63,504 states; FP64).  Every
    listed sector's lowest level is simple (gaps >= 0.22), so G' is a parity
    quantity too."""
    from vca_gb300.solver import VcaSolver
    pt = mid_points()[name]
    s = VcaSolver(pt.cfg, pt.bath_h, pt.bath_v)
    om = s.solve(pt.Hloc, pt.Hk, pt.bath_h, pt.bath_v)
    egs, _ = s.energies()
    assert _rel(egs, MM[name + "_egs"]) < 1e-10
    assert _rel(om, MM[name + "_sft"]) < 1e-10, (om, float(MM[name + "_sft"]))
    np.testing.assert_allclose(s.sector_energies(), MM[name + "_sector_e"], rtol=1e-10, atol=1e-10)
    assert np.abs(s.gf_cluster(1j * MM["wg"]) - MM[name + "_g"]).max() < 1e-8
    if name + "_states" in MM:
        t = s.thermal()
        assert sorted(x for x, _ in s.states()) == MM[name + "_states"].tolist()
        for key in ("zeta", "omega_prime", "max_exc", "sum_part", "contour_part"):
            assert _rel(t[key], MM[name + "_" + key]) < 1e-10, key
        assert t["nmax"] == int(MM[name + "_nmax"])
    s.close()
