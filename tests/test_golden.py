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


def chain_point(tp):
    return clusters.chain1d(tprime=float(tp), nlat=4, U=4.0, xmu=2.0, nk=64, ngfiter=100, omega_nodes=4096)


def small_points():
    return {
        "sq2x2": clusters.square(nx=2, ny=2, U=8.0, xmu=4.0, maf=0.2, nspin=2, nkx=6, nky=6, ngfiter=80,
                                 omega_nodes=1024),
        "bath": clusters.square_bath(nb=2, nk1=6, ngfiter=60, omega_nodes=1024),
        "bhz": clusters.bhz(mass=2.2, delta=0.1, nk1=4, ngfiter=60, omega_nodes=1024),
    }


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
