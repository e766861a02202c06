"""GPU parity of the custom observables (vca_gpu_custom_observable, the
reference's init/add/get_custom_observables, VCA_OBSERVABLES.f90:89-170,
335-500) through the C-ABI against the CPU oracle, at T=0 and at finite T,
for a k-independent and a k-dependent matrix: 1e-10 relative (absolute below
1).  Also the registry calls in the reference's order, and the U=0 band
occupation as a closed form."""
import numpy as np
import pytest

from vca_gb300 import clusters
from vca_gb300.clusters import nnn2lso
from vca_gb300.solver import VcaSolver, VcaError
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _ft(pt, beta, bandwidth):
    cfg = pt.cfg.copy()
    cfg.lanc_nstates_total, cfg.beta, cfg.bandwidth = 2, beta, bandwidth
    pt.cfg = cfg
    return pt


POINTS = {
    "chain4": lambda: clusters.chain1d(tprime=0.9, nlat=4, U=4.0, xmu=2.0, nk=16, ngfiter=100, omega_nodes=256),
    "square2x2_afm": lambda: clusters.square(nx=2, ny=2, U=8.0, xmu=4.0, maf=0.2, nspin=2, nkx=6, nky=6,
                                             ngfiter=80, omega_nodes=256),
    "bath2x2+4": lambda: clusters.square_bath(nb=4, nk1=6, ngfiter=60, omega_nodes=256, seed=11),
    "bhz_small": lambda: clusters.bhz(mass=2.2, delta=0.1, nk1=4, ngfiter=60, omega_nodes=256),
    "square2x2_afm_b8": lambda: _ft(clusters.square(nx=2, ny=2, U=8.0, xmu=4.0, maf=0.2, nspin=2, nkx=4, nky=4,
                                                    ngfiter=60, omega_nodes=64), 8.0, 8.0),
    "bath2x2+2_b10": lambda: _ft(clusters.square_bath(nb=2, nk1=4, ngfiter=40, omega_nodes=64), 10.0, 8.0),
}


def _close(a, b):
    return abs(a - b) <= TOL * max(1.0, abs(b))


@pytest.mark.parametrize("name", list(POINTS))
def test_custom_observable_matches_oracle(name):
    pt = POINTS[name]()
    s = VcaSolver(pt.cfg, pt.bath_h, pt.bath_v)
    s.solve(pt.Hloc, pt.Hk, pt.bath_h, pt.bath_v)
    o = Oracle.from_point(pt)
    o.solve()
    rng = np.random.default_rng(3)
    loc = np.asfortranarray(rng.normal(size=pt.Hloc.shape) + 1j * rng.normal(size=pt.Hloc.shape))
    kdep = np.asfortranarray(rng.normal(size=pt.Hk.shape) + 1j * rng.normal(size=pt.Hk.shape))
    for sm in (loc, kdep, pt.Hk):
        got, ref = s.custom_observable(sm), o.custom_observable(sm)
        assert _close(got, ref), (name, sm.ndim, got, ref)


def test_custom_observable_registry_and_u0_occupation():
    pt = clusters.square(nx=2, ny=2, U=0.0, xmu=0.37, nspin=2, nkx=4, nky=4, ngfiter=40, omega_nodes=1024)
    s = VcaSolver(pt.cfg)
    s.solve(pt.Hloc, pt.Hk)
    one = np.zeros(pt.Hloc.shape, complex, order="F")
    for i in range(pt.cfg.Nlat):
        for sp in range(pt.cfg.Nspin):
            one[i, i, sp, sp, 0, 0] = 1.0
    s.init_custom_observables(2, pt.Nk)
    s.add_custom_observable("n_tot", one)
    s.add_custom_observable("e_kin", pt.Hk)
    with pytest.raises(VcaError):
        s.add_custom_observable("third", one)
    vals = s.get_custom_observables()
    Hk = nnn2lso(pt.Hk)
    nocc = ekin = 0.0
    for k in range(pt.Nk):
        e = np.linalg.eigvalsh(Hk[:, :, k])
        nocc += np.sum(e < pt.cfg.xmu)
        ekin += np.sum(e[e < pt.cfg.xmu])
    assert abs(vals["n_tot"] - nocc / pt.Nk) < 1e-10
    assert abs(vals["e_kin"] - ekin / pt.Nk) < 1e-10
    s.clear_custom_observables()
    assert s.get_custom_observables() == {}
