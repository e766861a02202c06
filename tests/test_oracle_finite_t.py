"""The oracle's finite-temperature path (LANC_NSTATES_TOTAL > 1) pinned
against closed forms and scipy's QUADPACK.

* The state-list annealing (VCA_DIAG.f90:78-256, vca_post_diag :357-451):
  the single Hubbard site, whose four sector energies are known, walked
  through the sweeps by hand -- list contents, zeta taken before the trim,
  the adapted LANC_NSTATES_TOTAL and its carry-over to the next solve.
* Boltzmann weights of the chains and the observables: the atomic Green's
  function and occupations.
* Omega (VCA_OMEGA.f90:153-204): at U=0 and xmu=0 the Matsubara sum plus the
  contour integral reproduce the exact lattice grand potential; with xmu != 0
  the reference's fermi(w - xmu) moves the result off it, and the unshifted
  Fermi function restores it -- both checked.
* The fixed contour rule against adaptive QUADPACK on the same integrand.
"""
import numpy as np
import pytest
import scipy.integrate

from vca_gb300 import clusters
from vca_gb300.clusters import nnn2lso
from oracle import oracle as orc
from oracle.oracle import Oracle


def lattice_omega(pt, beta, mu):
    """-T sum_k sum_bands ln(1 + exp(-beta(e - mu))) per cluster, spin multiplicity 3 - Nspin."""
    Hk = nnn2lso(pt.Hk)
    tot = 0.0
    for k in range(pt.Nk):
        e = np.linalg.eigvalsh(Hk[:, :, k]) - mu
        tot -= np.sum(np.logaddexp(0.0, -beta * e)) / beta
    return (3 - pt.cfg.Nspin) * tot / pt.Nk


def atom(beta, nstates=2):
    """One Hubbard site, U=4, xmu=2, no lattice coupling (H_k = Hloc = 0):
    sectors 1..4 = (n_up,n_dw) = (0,0), (0,1), (1,0), (1,1) with energies
    0, -2, -2, 0."""
    return clusters.chain1d(tprime=0.0, t=0.0, nlat=1, U=4.0, xmu=2.0, nk=4, ngfiter=8, omega_nodes=64,
                            lanc_nstates_total=nstates, beta=beta, bandwidth=0.0)


def test_annealing_trims_after_convergence():
    o = Oracle.from_point(atom(20.0))
    sft, emin, oi = o.solve()
    # sweep 1 (cap 2): [(3,-2), (2,-2)], spread 1 -> cap 4; sweep 2: all four,
    # exp(-40) < cutoff -> converged; zeta over the four, then the two E=0
    # states are trimmed and the cap reset to max(2,2)+2
    assert o.states() == [(3, -2.0), (2, -2.0)]
    t = o.thermal()
    assert t["finite_t"] == 1 and t["nstates_total"] == 4
    assert t["zeta"] == pytest.approx(2.0 + 2.0 * np.exp(-40.0), rel=1e-15)
    assert t["omega_prime"] == pytest.approx(-2.0 - np.log(2.0) / 20.0, rel=1e-15)
    assert oi == 0.0  # H_k = Hloc: det(1) = 1 at every node
    assert sft == pytest.approx(-2.0 - np.log(2.0) / 20.0, rel=1e-15)
    # the adapted cap carries over: the next solve converges in its first sweep
    o.solve()
    assert o.states() == [(3, -2.0), (2, -2.0)] and o.thermal()["nstates_total"] == 4


def test_annealing_grows_until_the_sweeps_run_out():
    o = Oracle.from_point(atom(2.0, nstates=3))  # odd cap rounded up to 4 (VCA_SETUP.f90:172-175)
    o.solve()
    # exp(-4) > cutoff at every sweep: the list keeps all four states and the
    # cap grows by 2 per sweep, 4 + 2*10
    assert o.states() == [(3, -2.0), (2, -2.0), (4, 0.0), (1, 0.0)]
    t = o.thermal()
    assert t["nstates_total"] == 24
    z = 2.0 + 2.0 * np.exp(-4.0)
    assert t["zeta"] == pytest.approx(z, rel=1e-15)
    assert t["omega_prime"] == pytest.approx(-2.0 - np.log(z) / 2.0, rel=1e-15)
    # Boltzmann-weighted observables and Green's function of the atom
    obs = o.observables()
    assert obs["dens_up"][0, 0] == pytest.approx(0.5, abs=1e-15)
    assert obs["docc"][0, 0] == pytest.approx(np.exp(-4.0) / z, abs=1e-15)
    zz = np.array([0.3j, 1.7j, 0.4 + 0.2j])
    g = o.gf_cluster(zz)[0, 0, 0, 0, 0, 0]
    np.testing.assert_allclose(g, 0.5 / (zz + 2.0) + 0.5 / (zz - 2.0), atol=1e-14)


@pytest.mark.parametrize("beta", [20.0, 35.0])
def test_omega_u0_half_filling_is_the_lattice_value(beta):
    pt = clusters.chain1d(tprime=1.0, nlat=2, U=0.0, xmu=0.0, nk=32, ngfiter=50, omega_nodes=64,
                          lanc_nstates_total=2, beta=beta, bandwidth=4.0)
    o = Oracle.from_point(pt)
    sft, emin, oi = o.solve()
    # one state per sector: excited states inside a sector are missing, which
    # costs exp(-beta * 2) here (the in-sector gap is 2t)
    assert abs(sft - lattice_omega(pt, beta, 0.0)) < 1e-13 + 10 * np.exp(-2.0 * beta)
    t = o.thermal()
    assert t["nmax"] == ((lambda n: n // 2 if n % 2 == 0 else (n + 1) // 2)(
        int(2 * (abs(t["max_exc"]) + 4.0) * beta / np.pi)))
    assert t["integration_R"] == pytest.approx(2 * (t["nmax"] + 1) * np.pi / beta, rel=1e-15)


def test_fermi_shift_of_the_reference_contour():
    """The reference's contour uses fermi(w - xmu) while H already holds -xmu:
    with xmu != 0 its Omega leaves the lattice value; the same Matsubara sum
    with the unshifted fermi(w) on the contour gives it back."""
    beta, mu = 20.0, 0.5
    pt = clusters.chain1d(tprime=1.0, nlat=2, U=0.0, xmu=mu, nk=32, ngfiter=50, omega_nodes=64,
                          lanc_nstates_total=2, beta=beta, bandwidth=4.0)
    o = Oracle.from_point(pt)
    sft, emin, oi = o.solve()
    t = o.thermal()
    exact = lattice_omega(pt, beta, mu)
    assert abs(sft - exact) > 1e-5
    R = t["integration_R"]

    def f(th):
        w = R * np.exp(1j * th)
        x = beta * w
        fermi = 0.0 if x.real >= 100 else 1.0 / (np.exp(x) + 1.0)
        return ((1 / np.pi) * w * fermi * o.sum_kmesh_complex(w)).real

    val, _ = scipy.integrate.quad(f, 0.0, np.pi, points=[np.pi / 2], limit=400, epsabs=1e-14, epsrel=1e-14)
    fixed = t["omega_prime"] - (3 - pt.cfg.Nspin) * (t["sum_part"] + val)
    assert abs(fixed - exact) < 1e-11


def test_contour_rule_against_quadpack():
    pt = clusters.square(nx=2, ny=2, U=4.0, xmu=2.0, maf=0.0, nspin=1, nkx=4, nky=4, ngfiter=60,
                         omega_nodes=64)
    cfg = pt.cfg.copy()
    cfg.lanc_nstates_total, cfg.beta, cfg.bandwidth = 2, 10.0, 8.0
    pt.cfg = cfg
    o = Oracle.from_point(pt)
    o.solve()
    t = o.thermal()
    R = t["integration_R"]
    th0 = np.arccos(cfg.xmu / R)
    val, err = scipy.integrate.quad(lambda th: o.contour_integrand(R, th), 0.0, np.pi, points=[th0], limit=1000,
                                    epsabs=1e-14, epsrel=1e-14)
    assert abs(t["contour_part"] - val) < 1e-12, (t["contour_part"], val, err)
    th, w = orc.contour_rule(R, cfg.beta, cfg.xmu, cfg.contour_nodes)
    assert len(th) == t["contour_points"] and np.all(np.diff(th) > 0) and abs(w.sum() - np.pi) < 1e-13


def test_sum_kmesh_complex_direct_formula():
    pt = clusters.square_bath(nb=2, nk1=3, omega_nodes=64, ngfiter=40)
    o = Oracle.from_point(pt)
    o.diagonalize()
    o.build_gf()
    Hl = nnn2lso(pt.Hloc)
    Hk = nnn2lso(pt.Hk)
    for z in (0.3j, 2.0 + 0.5j, -7.0 + 1e-3j, 30.0 * np.exp(2.0j)):
        G = nnn2lso(o.gf_cluster(z)[..., 0])
        D = o.delta_bath(z)
        f = np.mean([np.log(np.linalg.det(np.eye(G.shape[0]) + (D + Hl - Hk[:, :, k]) @ G))
                     for k in range(pt.Nk)])
        got = o.sum_kmesh_complex(z)
        assert abs(got - f) < 1e-12 * max(1, abs(f)), (z, got, f)


@pytest.mark.parametrize("mu_frac", [0.05, 0.97, -0.97])
def test_contour_rule_with_the_fermi_step_near_the_ends(mu_frac):
    """The graded rule when the Fermi step sits near theta = 0 or pi (xmu
    close to +-R): against adaptive QUADPACK on a model integrand with the
    same Fermi factor and a smooth F(w)."""
    R, beta = 20.0, 15.0
    mu = mu_frac * R
    th, w = orc.contour_rule(R, beta, mu, 24)

    def f(t):
        z = R * np.exp(1j * t)
        x = beta * (z - mu)
        fermi = 0.0 if x.real >= 100 else 1.0 / (np.exp(x) + 1.0)
        F = np.log(1.0 + 3.0 / (z * z + 2.0 * z + 5.0))
        return ((1 / np.pi) * z * fermi * F).real

    rule = float(np.dot(w, [f(t) for t in th]))
    pts = [float(np.arccos(np.clip(mu / R, -1.0, 1.0)))]
    ref, _ = scipy.integrate.quad(f, 0.0, np.pi, points=pts, limit=2000, epsabs=1e-14, epsrel=1e-14)
    assert abs(rule - ref) < 1e-12, (mu_frac, rule, ref)


def test_max_exc_is_rounding_set_but_nmax_is_not():
    """max_exc is the largest Ritz value of the Green's-function chains,
    which run without reorthogonalisation from ground-state vectors that
    meet a 1e-11 residual, so its last digits follow the start vector.  On
    the finite-temperature BHZ test model the oracle alone, over six Lanczos
    start seeds, moves it by ~2e-7 relative (measured), while nmax and the
    contour radius -- the only ways it enters Omega -- and Omega itself stay
    put.  The GPU parity test compares max_exc at 1e-6 for this reason."""
    vals, nmax, R, sft = [], set(), set(), []
    for seed in (20261203, 1, 2, 3, 77, 991):
        pt = clusters.bhz(mass=2.2, delta=0.1, nk1=4, ngfiter=40, omega_nodes=64)
        cfg = pt.cfg.copy()
        cfg.lanc_nstates_total, cfg.beta, cfg.bandwidth, cfg.start_seed = 2, 10.0, 8.0, seed
        pt.cfg = cfg
        o = Oracle.from_point(pt)
        sft.append(o.solve()[0])
        t = o.thermal()
        vals.append(t["max_exc"])
        nmax.add(t["nmax"])
        R.add(t["integration_R"])
    v = np.array(vals)
    spread = (v.max() - v.min()) / abs(v[0])
    assert 1e-9 < spread < 1e-6, spread
    assert len(nmax) == 1 and len(R) == 1
    assert (max(sft) - min(sft)) / abs(sft[0]) < 1e-10
