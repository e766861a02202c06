"""The oracle's custom observables (VCA_OBSERVABLES.f90:335-500) pinned
against closed forms and scipy's QUADPACK.

* T=0, U=0: the VCA lattice Green's function is the exact one, so s = 1 gives
  the number of occupied bands and s_k = H_k the band energy below xmu,
  averaged over k, times (3 - Nspin) (the tail subtraction Tr[s]/(iw - 1.1)
  contributes Tr[s]/2 exactly);
* the integrand against a direct numpy evaluation of the reference formula;
* the fixed rule against adaptive QUADPACK on an interacting model;
* a k-independent s against the same matrix repeated at every k.
"""
import numpy as np
import pytest
import scipy.integrate

from vca_gb300 import clusters
from vca_gb300.clusters import nnn2lso
from oracle.oracle import Oracle


def _solved(pt):
    o = Oracle.from_point(pt)
    o.solve()
    return o


def test_t0_u0_occupation_and_band_energy():
    for pt in (clusters.chain1d(tprime=1.0, nlat=2, U=0.0, xmu=0.3, nk=32, ngfiter=50, omega_nodes=1024),
               clusters.square(nx=2, ny=2, U=0.0, xmu=0.37, nspin=2, nkx=4, nky=4, ngfiter=40, omega_nodes=1024)):
        o = _solved(pt)
        mu = pt.cfg.xmu
        Hk = nnn2lso(pt.Hk)
        mult = 3 - pt.cfg.Nspin
        nocc = ekin = 0.0
        for k in range(pt.Nk):
            e = np.linalg.eigvalsh(Hk[:, :, k])
            nocc += np.sum(e < mu)
            ekin += np.sum(e[e < mu])
        one = np.zeros(pt.Hloc.shape, complex, order="F")
        for i in range(pt.cfg.Nlat):
            for sp in range(pt.cfg.Nspin):
                one[i, i, sp, sp, 0, 0] = 1.0
        assert abs(o.custom_observable(one) - mult * nocc / pt.Nk) < 1e-10
        assert abs(o.custom_observable(pt.Hk) - mult * ekin / pt.Nk) < 1e-10


def test_integrand_direct_formula():
    pt = clusters.square_bath(nb=2, nk1=3, omega_nodes=64, ngfiter=40)
    o = _solved(pt)
    rng = np.random.default_rng(5)
    N = pt.cfg.Nlat * pt.cfg.Nspin * pt.cfg.Norb
    s = np.asfortranarray(rng.normal(size=pt.Hk.shape) + 1j * rng.normal(size=pt.Hk.shape))
    Hl = nnn2lso(pt.Hloc)
    Hk = nnn2lso(pt.Hk)
    S = nnn2lso(s)
    for z, tail in ((0.7j, True), (3.1j, True), (1.5 + 0.4j, False), (-6.0 + 2.0j, False)):
        Gi = np.linalg.inv(nnn2lso(o.gf_cluster(z)[..., 0]))
        D = o.delta_bath(z)
        f = 0.0
        for k in range(pt.Nk):
            G = np.linalg.inv(Gi - (Hk[:, :, k] - Hl - D))
            t = np.trace(S[:, :, k] @ G)
            if tail:
                t -= np.trace(S[:, :, k]) / (z - 1.1)
            f += t.real
        f /= pt.Nk
        assert abs(o.sum_observable_kmesh(z, s, tail) - f) < 1e-12 * max(1.0, abs(f)), (z, f)
    assert N == 4


def test_fixed_rule_against_qagi_and_local_vs_kdep():
    pt = clusters.square(nx=2, ny=2, U=4.0, xmu=2.0, maf=0.1, nspin=2, nkx=4, nky=4, ngfiter=60,
                         omega_nodes=2048)
    o = _solved(pt)
    rng = np.random.default_rng(9)
    a = rng.normal(size=pt.Hloc.shape) + 1j * rng.normal(size=pt.Hloc.shape)
    s = np.asfortranarray(a)
    val = o.custom_observable(s)
    q, _ = scipy.integrate.quad(lambda w: o.sum_observable_kmesh(1j * w, s, True), 0.0, np.inf, epsabs=1e-12,
                                epsrel=1e-12, limit=500)
    assert abs(val - (3 - pt.cfg.Nspin) * q / np.pi) < 1e-9
    sk = np.asfortranarray(np.repeat(s[..., None], pt.Nk, axis=6))
    assert abs(o.custom_observable(sk) - val) < 1e-12 * max(1.0, abs(val))
