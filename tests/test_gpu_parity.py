"""GPU parity: the CUDA path through the C-ABI against the CPU oracle.

Tolerances (from the parity targets of this path): Fock maps, sector tables
and matrix-element signs bit-exact; H x v to 1e-13 relative; ground-state
energies and Omega to 1e-10 relative; G'(i w) to 1e-8 absolute.
"""
import numpy as np
import pytest

from vca_gb300 import clusters
from vca_gb300.clusters import nnn2lso
from vca_gb300.solver import VcaSolver, VcaError
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

E_TOL = 1e-10
G_TOL = 1e-8


def _rng(seed=7):
    return np.random.default_rng(seed)


def _small_bath(nb=4, seed=11, **kw):
    return clusters.square_bath(nb=nb, nk1=6, ngfiter=60, omega_nodes=256, seed=seed, **kw)


POINTS = {
    "chain4": lambda: clusters.chain1d(tprime=0.9, nlat=4, U=4.0, xmu=2.0, nk=16, ngfiter=100,
                                       omega_nodes=256),
    "square2x2_afm": lambda: clusters.square(nx=2, ny=2, U=8.0, xmu=4.0, maf=0.2, nspin=2, nkx=6,
                                             nky=6, ngfiter=80, omega_nodes=256),
    "bath2x2+4": lambda: _small_bath(),
    # 8 sites: the column kernels run with many warps per CTA
    "square2x4_afm": lambda: clusters.square(nx=2, ny=4, U=8.0, xmu=4.0, maf=0.2, nspin=2, nkx=4,
                                             nky=4, ngfiter=60, omega_nodes=128),
    "bhz_small": lambda: clusters.bhz(mass=2.2, delta=0.1, nk1=4, ngfiter=60, omega_nodes=256),
}


@pytest.fixture(scope="module", params=list(POINTS))
def point(request):
    return POINTS[request.param]()


def test_sector_maps_bitexact(point):
    s = VcaSolver(point.cfg, point.bath_h, point.bath_v)
    o = Oracle.from_point(point)
    assert s.Ns == o.Ns
    for isec in range(1, o.Nsectors + 1):
        assert s.sector_info(isec) == o.sector_info(isec)
        for spin in (1, 2):
            np.testing.assert_array_equal(s.sector_map(isec, spin), o.sector_map(isec, spin))


def test_hxv_matches_oracle(point):
    s = VcaSolver(point.cfg, point.bath_h, point.bath_v)
    s.set_hamiltonian(point.Hloc, point.bath_h, point.bath_v)
    o = Oracle.from_point(point)
    rng = _rng()
    worst = 0.0
    for isec in range(1, o.Nsectors + 1):
        d = o.dim(isec)
        if d > 20000:
            continue
        v = rng.normal(size=d) + 1j * rng.normal(size=d)
        ref = o.hxv(isec, v)
        got = s.hxv(isec, v)
        scale = max(1.0, np.abs(ref).max())
        worst = max(worst, np.abs(got - ref).max() / scale)
    assert worst < 1e-13, worst


def test_solve_matches_oracle(point):
    s = VcaSolver(point.cfg, point.bath_h, point.bath_v)
    om = s.solve(point.Hloc, point.Hk, point.bath_h, point.bath_v)
    o = Oracle.from_point(point)
    ref, egs_ref, oi_ref = o.solve()
    egs, oi = s.energies()
    assert abs(egs - egs_ref) <= E_TOL * abs(egs_ref)
    # every sector's lowest eigenvalue
    se = s.sector_energies()
    so = o.sector_energies()
    np.testing.assert_allclose(se, so, rtol=E_TOL, atol=E_TOL)
    # ground-state list
    st = s.states()
    so_states = []
    k = 0
    while True:
        r = o.state(k) if k < 64 else None
        if r is None or r[0] <= 0:
            break
        so_states.append(r[:2])
        k += 1
    assert [x[0] for x in st] == [x[0] for x in so_states]
    np.testing.assert_allclose([x[1] for x in st], [x[1] for x in so_states], rtol=E_TOL)
    assert abs(om - ref) <= E_TOL * abs(ref), (om, ref)
    # cluster Green's function on the imaginary axis
    z = 1j * np.array([0.05, 0.3, 1.0, 3.0, 10.0])
    g = s.gf_cluster(z)
    go = o.gf_cluster(z)
    assert np.abs(g - go).max() < G_TOL, np.abs(g - go).max()


def test_sum_kmesh_matches_oracle():
    pt = POINTS["square2x2_afm"]()
    s = VcaSolver(pt.cfg)
    s.solve(pt.Hloc, pt.Hk)
    o = Oracle.from_point(pt)
    o.solve()
    w = np.array([0.01, 0.5, 2.0, 40.0, 1e4])
    f = s.sum_kmesh(w)
    fo = np.array([o.sum_kmesh(x) for x in w])
    np.testing.assert_allclose(f, fo, rtol=1e-10, atol=1e-12)


def test_shape_errors_raise():
    pt = POINTS["chain4"]()
    s = VcaSolver(pt.cfg)
    with pytest.raises(VcaError):
        s.solve(pt.Hloc[:2], pt.Hk)
    bad = pt.Hloc.copy()
    bad[0, 0, 0, 0, 0, 0] = np.nan
    with pytest.raises(VcaError) as ei:
        s.solve(bad, pt.Hk)
    assert ei.value.code == -7


@pytest.mark.parametrize("arith", [1, 2], ids=["fp64", "fx"])
@pytest.mark.parametrize("name", ["chain4", "square2x2_afm", "square2x4_afm"])
def test_fixed_point_and_fp64_paths_agree(name, arith):
    """Both arithmetic paths of a real Hamiltonian against the oracle."""
    pt = POINTS[name]()
    cfg = pt.cfg.copy()
    cfg.arith = arith
    s = VcaSolver(cfg)
    om = s.solve(pt.Hloc, pt.Hk)
    assert s.arith_info()[0] == (arith == 2)
    o = Oracle.from_point(pt)
    ref, egs_ref, _ = o.solve()
    egs, _ = s.energies()
    assert abs(egs - egs_ref) <= E_TOL * abs(egs_ref)
    assert abs(om - ref) <= E_TOL * abs(ref), (om, ref)
    np.testing.assert_allclose(s.sector_energies(), o.sector_energies(), rtol=E_TOL, atol=E_TOL)
    z = 1j * np.array([0.05, 0.3, 1.0, 3.0, 10.0])
    assert np.abs(s.gf_cluster(z) - o.gf_cluster(z)).max() < G_TOL


def test_gf_channel_poles_match_oracle():
    """Poles and weights of single channels (formed on demand from the stored
    chain tridiagonals) against the oracle's, compared as the pole sums
    sum_j w_j / (z - p_j) at points off the real axis (1e-8 absolute), and
    against the continued-fraction G'(z) of the solve for a diagonal element."""
    pt = POINTS["square2x2_afm"]()
    s = VcaSolver(pt.cfg)
    s.solve(pt.Hloc, pt.Hk)
    o = Oracle.from_point(pt)
    o.solve()
    z = np.array([0.3 + 0.1j, -1.0 + 1.0j, 2.0 + 5.0j])

    def psum(p, w):
        return (w[None, :] / (z[:, None] - p[None, :].real)).sum(axis=1)

    checked = 0
    for il, jl in ((1, 1), (1, 2), (2, 4)):
        for ispin in (1, 2):
            for ichan in (1, 2, 3, 4):
                if il == jl and ichan > 2:
                    continue
                p, w = s.gf_channel(il, jl, ispin, 1, 1, 1, ichan)
                ref = o.gf_channel(il, jl, ispin, 1, 1, 0, ichan)  # oracle states are 0-based
                assert ref is not None and len(p) == len(ref[0])
                assert np.abs(psum(p, w) - psum(ref[0], ref[1])).max() < G_TOL
                checked += 1
    assert checked == 20
    # diagonal element: particle + hole channels of the ground state = G'_11
    g = s.gf_cluster(z)[0, 0, 0, 0, 0, 0, :]
    tot = sum(psum(*s.gf_channel(1, 1, 1, 1, 1, 1, ch)) for ch in (1, 2))
    assert np.abs(g - tot).max() < 1e-10


def test_unconverged_ql_is_reported_not_returned():
    """With the QL cap forced to one sweep per eigenvalue the 80-step chains
    cannot converge: the pole request must fail with VCA_ERR_NUMERIC (-7)
    rather than return poles of an unfinished QL.  Restoring the default cap
    gives the poles back, equal to a fresh context's."""
    pt = POINTS["square2x2_afm"]()
    s = VcaSolver(pt.cfg)
    s.solve(pt.Hloc, pt.Hk)
    p0, w0 = s.gf_channel(1, 1, 1, 1, 1, 1, 1)
    s.set_ql_max_iter(1)
    with pytest.raises(VcaError) as ei:
        s.gf_channel(1, 1, 1, 1, 1, 1, 1)
    assert ei.value.code == -7 and "did not converge" in str(ei.value)
    s.set_ql_max_iter(60)
    p1, w1 = s.gf_channel(1, 1, 1, 1, 1, 1, 1)
    np.testing.assert_array_equal(p1, p0)
    np.testing.assert_array_equal(w1, w0)


@pytest.mark.parametrize("name", list(POINTS))
def test_sigma_and_g0_grids_match_oracle(name):
    """vca_get_sigma_matsubara/_realaxis and the G0 grids (build_sigma_normal)
    against the oracle on 40 Matsubara and 40 real-axis points."""
    pt = POINTS[name]()
    cfg = pt.cfg.copy()
    cfg.Lmats, cfg.Lreal = 40, 40
    s = VcaSolver(cfg, pt.bath_h, pt.bath_v)
    s.solve(pt.Hloc, pt.Hk, pt.bath_h, pt.bath_v)
    o = Oracle.from_point(pt)
    o.solve()
    c = cfg
    wm = np.pi / c.beta * (2 * np.arange(1, c.Lmats + 1) - 1)
    wr = np.linspace(c.wini, c.wfin, c.Lreal)
    # Matsubara axis: G', Sigma and G0 against the oracle.
    sig, g0, gimp = s.sigma_matsubara(), s.g0_matsubara(), s.gimp_matsubara()
    for q in range(0, c.Lmats, 7):
        z = 1j * wm[q]
        so, go = o.sigma_g0(z)
        gref = nnn2lso(o.gf_cluster(z)[..., 0])
        assert np.abs(nnn2lso(gimp[..., q]) - gref).max() < G_TOL, (name, z)
        assert np.abs(nnn2lso(sig[..., q]) - so).max() <= 1e-8 * (1.0 + np.abs(so).max()), (name, z)
        assert np.abs(nnn2lso(g0[..., q]) - go).max() <= 1e-10 * (1.0 + np.abs(go).max()), (name, z)
    # Real axis (eta = eps): G0 involves no Lanczos chain and is compared
    # with the oracle.  G' there is not a parity quantity at small eta: the
    # chains' unconverged high-energy Ritz values move with roundoff (without
    # reorthogonalisation, as in the reference), which on the imaginary axis
    # stays below 1e-8 but at eta = 0.01 reaches ~1e-3 near those poles.
    # Sigma is checked as G0^-1 - G'^-1 of the library's own G' and G0.
    sig, g0, gimp = s.sigma_realaxis(), s.g0_realaxis(), s.gimp_realaxis()
    for q in range(0, c.Lreal, 7):
        z = wr[q] + 1j * c.eps
        _, go = o.sigma_g0(z)
        gg = nnn2lso(g0[..., q])
        assert np.abs(gg - go).max() <= 1e-10 * (1.0 + np.abs(go).max()), (name, z)
        sref = np.linalg.inv(gg) - np.linalg.inv(nnn2lso(gimp[..., q]))
        assert np.abs(nnn2lso(sig[..., q]) - sref).max() <= 1e-9 * (1.0 + np.abs(sref).max()), (name, z)


@pytest.mark.parametrize("name", list(POINTS))
def test_observables_match_oracle(name):
    """vca_get_dens/_docc/_mag (vca_lanc_observables) against the oracle."""
    pt = POINTS[name]()
    s = VcaSolver(pt.cfg, pt.bath_h, pt.bath_v)
    s.solve(pt.Hloc, pt.Hk, pt.bath_h, pt.bath_v)
    o = Oracle.from_point(pt)
    o.solve()
    got, ref = s.observables(), o.observables()
    for key in ref:
        np.testing.assert_allclose(got[key], ref[key], rtol=0, atol=1e-10, err_msg=f"{name} {key}")


@pytest.mark.parametrize("name", ["chain4", "square2x2_afm", "bhz_small"])
def test_chan2_solve_matches_oracle(name):
    """VCA_GF_SYMMETRIC=T: two channels per off-diagonal element
    (lanc_build_gf_normal_mix_chan2, VCA_GF_NORMAL.f90:327-556) and the
    recombination with chan4 = 0."""
    pt = POINTS[name]()
    pt.cfg.vca_gf_symmetric = 1
    s = VcaSolver(pt.cfg, pt.bath_h, pt.bath_v)
    om = s.solve(pt.Hloc, pt.Hk, pt.bath_h, pt.bath_v)
    o = Oracle.from_point(pt)
    ref, _, _ = o.solve()
    assert abs(om - ref) <= E_TOL * abs(ref), (om, ref)
    z = np.array([0.2j, 1.0j, 0.7 + 0.3j])
    np.testing.assert_allclose(s.gf_cluster(z), o.gf_cluster(z), rtol=0, atol=G_TOL)
    p, w = s.gf_channel(1, 2, 1, 1, 1, 1, 1)
    assert len(p) > 0
    assert len(s.gf_channel(1, 2, 1, 1, 1, 1, 3)[0]) == 0  # no third channel


@pytest.mark.parametrize("name", ["bhz_small", "bath2x2+4", "square2x2_afm"])
def test_omega_inverse_form_equals_product_form(name):
    """The T=0 integrand as ln|det(G'^-1 + M_k)| + ln|det G'| below w = 10
    (the default) and as ln|det(1 + M_k G')| at every node give the same
    Omega and the same integrand."""
    pt = POINTS[name]()
    vals, f = [], []
    w = np.array([0.01, 0.3, 2.0, 9.0, 40.0])
    for on in (True, False):
        s = VcaSolver(pt.cfg, pt.bath_h, pt.bath_v)
        s.set_omega_inverse_form(on)
        vals.append(s.solve(pt.Hloc, pt.Hk, pt.bath_h, pt.bath_v))
        f.append(s.sum_kmesh(w))
    assert abs(vals[0] - vals[1]) < 1e-12 * max(1.0, abs(vals[1])), vals
    np.testing.assert_allclose(f[0], f[1], rtol=1e-12, atol=1e-13)
