"""The oracle (CPU restatement) pinned against independent constructions.

The reference has no tests or golden vectors and cannot be built here, so the
oracle is checked against: an independent numpy construction of the sector
Hamiltonian from the operator definitions, dense exact diagonalisation, the
Hubbard-dimer and U=0 closed forms, and scipy's LAPACK / QUADPACK.
"""
import itertools

import numpy as np
import pytest
import scipy.integrate
import scipy.linalg

from vca_gb300 import clusters
from vca_gb300.clusters import nnn2lso
from oracle import oracle as orc
from oracle.oracle import Oracle


# ---------------------------------------------------------------------------
# independent numpy restatement of the operator algebra (small Ns only)
# ---------------------------------------------------------------------------
def words(ns, n):
    return [w for w in range(1 << ns) if bin(w).count("1") == n]


def one_word_sign(w, pos):  # pos 0-based: (-1)^(set bits below pos)
    return -1.0 if bin(w & ((1 << pos) - 1)).count("1") % 2 else 1.0


def spin_matrix_np(ns, n, A):
    """H_sigma[target, source] = sum_{i!=j} A[i,j] c^dag_i c_j on words of popcount n."""
    ws = words(ns, n)
    idx = {w: k for k, w in enumerate(ws)}
    H = np.zeros((len(ws), len(ws)), dtype=complex)
    for s, w in enumerate(ws):
        for i in range(ns):
            for j in range(ns):
                if i == j or A[i, j] == 0:
                    continue
                if (w >> j) & 1 and not (w >> i) & 1:
                    sg1 = one_word_sign(w, j)
                    k1 = w & ~(1 << j)
                    sg2 = one_word_sign(k1, i)
                    H[idx[k1 | (1 << i)], s] += A[i, j] * sg1 * sg2
    return H


def amplitude_matrix(pt, sidx):
    c = pt.cfg
    L = c.Nlat * c.Norb
    ns = L + c.Nlat_bath * c.Norb_bath
    A = np.zeros((ns, ns), dtype=complex)
    for il, jl, io, jo in itertools.product(range(c.Nlat), range(c.Nlat), range(c.Norb), range(c.Norb)):
        A[io + il * c.Norb, jo + jl * c.Norb] = pt.Hloc[il, jl, sidx, sidx, io, jo]
    if pt.bath_h is not None:
        for a, b, oa, ob in itertools.product(range(c.Nlat_bath), range(c.Nlat_bath), range(c.Norb_bath),
                                              range(c.Norb_bath)):
            A[L + a * c.Norb_bath + oa, L + b * c.Norb_bath + ob] = pt.bath_h[a, b, sidx, sidx, oa, ob]
        for il, b, io, ob in itertools.product(range(c.Nlat), range(c.Nlat_bath), range(c.Norb),
                                               range(c.Norb_bath)):
            v = pt.bath_v[il, b, sidx, sidx, io, ob]
            A[io + il * c.Norb, L + b * c.Norb_bath + ob] = v
            A[L + b * c.Norb_bath + ob, io + il * c.Norb] = np.conj(v)
    np.fill_diagonal(A, 0)
    return A


SMALL = {
    "chain4": lambda: clusters.chain1d(tprime=0.9, nlat=4, U=4.0, xmu=2.0, nk=8, omega_nodes=128),
    "square2x2": lambda: clusters.square(nx=2, ny=2, U=6.0, xmu=3.0, maf=0.15, nspin=2, nkx=4, nky=4,
                                         omega_nodes=128),
    "bath2+2": lambda: clusters.square_bath(nb=2, nk1=4, omega_nodes=128, ngfiter=50),
    "bhz": lambda: clusters.bhz(nk1=2, omega_nodes=64, ngfiter=40),
}


@pytest.fixture(params=list(SMALL))
def small(request):
    return SMALL[request.param]()


def test_sector_tables():
    pt = clusters.chain1d(nlat=4, nk=2)
    o = Oracle.from_point(pt)
    assert o.Ns == 4 and o.Nsectors == 25
    total = 0
    for isec in range(1, 26):
        nu, nd, du, dd = o.sector_info(isec)
        assert isec == 1 + nd + nu * 5  # get_Sector (VCA_SETUP.f90:404-415)
        assert du == orc.lib().orc_binomial(4, nu) and dd == orc.lib().orc_binomial(4, nd)
        total += du * dd
        assert o.cdg_sector(isec, 1) == (1 + nd + (nu + 1) * 5 if nu < 4 else 0)
        assert o.c_sector(isec, 2) == (1 + (nd - 1) + nu * 5 if nd > 0 else 0)
        np.testing.assert_array_equal(o.sector_map(isec, 1), words(4, nu))
    assert total == 4 ** 4
    for n in range(17):  # binomial through FP64 rounding is exact up to Ns=16
        assert orc.lib().orc_binomial(16, n) == scipy.special.comb(16, n, exact=True)


def test_spin_matrices_match_operator_algebra(small):
    o = Oracle.from_point(small)
    c = small.cfg
    for isec in [1 + (o.Ns // 2) + (o.Ns // 2) * (o.Ns + 1), 1 + 1 + 2 * (o.Ns + 1)]:
        nu, nd, du, dd = o.sector_info(isec)
        for spin, n, sidx in ((1, nu, 0), (2, nd, c.Nspin - 1)):
            r, cc, v = o.spin_matrix(isec, spin)
            dim = du if spin == 1 else dd
            H = np.zeros((dim, dim), dtype=complex)
            np.add.at(H, (r, cc), v)
            Hn = spin_matrix_np(o.Ns, n, amplitude_matrix(small, sidx))
            np.testing.assert_array_equal(H, Hn)


def test_dense_hermitian_and_hxv(small):
    o = Oracle.from_point(small)
    rng = np.random.default_rng(3)
    for isec in range(1, o.Nsectors + 1):
        d = o.dim(isec)
        if d > 400:
            continue
        H = o.dense_h(isec)
        np.testing.assert_allclose(H, H.conj().T, atol=1e-14)
        v = rng.normal(size=d) + 1j * rng.normal(size=d)
        np.testing.assert_allclose(o.hxv(isec, v), H @ v, atol=1e-12)


def test_dimer_closed_form():
    for U in (0.5, 3.0, 8.0):
        # half filling (xmu = U/2): the N=2 singlet, E = (U - sqrt(U^2+16t^2))/2 - 2*xmu
        pt = clusters.chain1d(tprime=1.0, nlat=2, U=U, xmu=U / 2, nk=2, omega_nodes=32)
        o = Oracle.from_point(pt)
        o.diagonalize()
        assert abs(o.egs() - ((U - np.sqrt(U * U + 16)) / 2 - U)) < 1e-12


def test_lanczos_gs_matches_lapack(small):
    o = Oracle.from_point(small)
    for isec in range(1, o.Nsectors + 1):
        d = o.dim(isec)
        if d < 2 or d > 600:
            continue
        w, V = np.linalg.eigh(o.dense_h(isec))
        e, psi, it = o.lanczos_gs(isec)
        assert abs(e - w[0]) < 1e-11 * max(1, abs(w[0]))
        H = o.dense_h(isec)
        assert np.linalg.norm(H @ psi - e * psi) < 1e-9


def test_tql2_and_tridiagonal_lowest():
    rng = np.random.default_rng(5)
    for n in (1, 2, 7, 60, 200):
        d = rng.normal(size=n)
        e = np.r_[0.0, rng.normal(size=n - 1)]
        w, z0, r = orc.tql2(d, e)
        ww, V = scipy.linalg.eigh_tridiagonal(d, e[1:])
        assert r == 0
        np.testing.assert_allclose(w, ww, atol=1e-12)
        np.testing.assert_allclose(z0 ** 2, V[0] ** 2, atol=1e-12)
        th, s = orc.tri_lowest(d, e[1:])
        assert abs(th - ww[0]) < 1e-12
        assert min(np.linalg.norm(s - V[:, 0]), np.linalg.norm(s + V[:, 0])) < 1e-9


def test_gauss_legendre_nodes():
    for n in (8, 256, 4096):
        x, w = orc.gauss_legendre01(n)
        xr, wr = np.polynomial.legendre.leggauss(n)
        np.testing.assert_allclose(x, 0.5 * (xr + 1), atol=1e-14)
        # exact for monomials of degree < 2n (numpy's own weights drift ~1e-7 at n=4096)
        for k in (0, 1, 7, n, 2 * n - 1):
            assert abs((w * x ** k).sum() * (k + 1) - 1.0) < 1e-12


def _exact_gf(o, pt, z, ispin=1):
    """G_ij(z) by dense ED of the N+-1 sectors (T=0, one ground state)."""
    c = pt.cfg
    isec, e0, psi = o.state(0, with_vector=True)
    nu, nd, du, dd = o.sector_info(isec)
    L = c.Nlat * c.Norb
    out = np.zeros((L, L, len(z)), dtype=complex)

    def op_matrix(tsec, pos, dag):
        # matrix of c^dag_pos (dag) or c_pos from isec to tsec on spin `ispin`
        tnu, tnd, tdu, tdd = o.sector_info(tsec)
        mu_s, md_s = words(o.Ns, nu), words(o.Ns, nd)
        mu_t, md_t = words(o.Ns, tnu), words(o.Ns, tnd)
        iu = {w: k for k, w in enumerate(mu_t)}
        idd = {w: k for k, w in enumerate(md_t)}
        M = np.zeros((tdu * tdd, du * dd))
        for s in range(du * dd):
            wu, wd = mu_s[s % du], md_s[s // du]
            w = wu if ispin == 1 else wd
            occ = (w >> pos) & 1
            if occ == dag:
                continue
            sg = one_word_sign(w, pos)
            w2 = w ^ (1 << pos)
            t = (iu[w2] + idd[wd] * tdu) if ispin == 1 else (iu[wu] + idd[w2] * tdu)
            M[t, s] = sg
        return M

    for dag, fsec in ((1, o.cdg_sector(isec, ispin)), (0, o.c_sector(isec, ispin))):
        if not fsec:
            continue
        w, V = np.linalg.eigh(o.dense_h(fsec))
        amps = []
        for p in range(L):
            amps.append(V.conj().T @ (op_matrix(fsec, p, dag) @ psi))
        for i in range(L):
            for j in range(L):
                if dag:  # <c_i R c^dag_j>
                    num = np.conj(amps[i]) * amps[j]
                    out[i, j] += (num[None, :] / (z[:, None] - (w - e0)[None, :])).sum(1)
                else:    # <c^dag_j R' c_i>
                    num = np.conj(amps[j]) * amps[i]
                    out[i, j] += (num[None, :] / (z[:, None] + (w - e0)[None, :])).sum(1)
    return out


def test_gf_poles_match_dense_resolvent():
    pt = clusters.chain1d(tprime=0.8, nlat=4, U=4.0, xmu=2.0, nk=4, ngfiter=100, omega_nodes=64)
    o = Oracle.from_point(pt)
    o.diagonalize()
    o.build_gf()
    z = np.array([0.2j, 1.0j, 0.5 + 0.3j, 4.0j])
    g = o.gf_cluster(z)
    ge = _exact_gf(o, pt, z)
    for i in range(4):
        for j in range(4):
            np.testing.assert_allclose(g[i, j, 0, 0, 0, 0], ge[i, j], atol=1e-10)


def test_gf_chan2_matches_dense_resolvent():
    """VCA_GF_SYMMETRIC=T (two channels, lanc_build_gf_normal_mix_chan2,
    VCA_GF_NORMAL.f90:327-556): exact for a real symmetric model."""
    pt = clusters.chain1d(tprime=0.8, nlat=4, U=4.0, xmu=2.0, nk=4, ngfiter=100, omega_nodes=64)
    pt.cfg.vca_gf_symmetric = 1
    o = Oracle.from_point(pt)
    o.diagonalize()
    o.build_gf()
    z = np.array([0.2j, 1.0j, 0.5 + 0.3j])
    g = o.gf_cluster(z)
    ge = _exact_gf(o, pt, z)
    for i in range(4):
        for j in range(4):
            np.testing.assert_allclose(g[i, j, 0, 0, 0, 0], ge[i, j], atol=1e-10)
    assert o.gf_channel(1, 2, 1, 1, 1, 0, 3) is None or len(o.gf_channel(1, 2, 1, 1, 1, 0, 3)[0]) == 0


def test_omega_u0_closed_form():
    for pt, mu, sfac in (
        (clusters.chain1d(tprime=1.0, nlat=4, U=0.0, xmu=0.3, nk=32, omega_nodes=512), 0.3, 2.0),
        (clusters.square(nx=2, ny=2, U=0.0, xmu=0.37, nspin=2, nkx=4, nky=4, omega_nodes=512), 0.37, 1.0),
    ):
        o = Oracle.from_point(pt)
        sft, egs, oi = o.solve()
        Hk = nnn2lso(pt.Hk)
        ex = sfac * np.mean([np.minimum(np.linalg.eigvalsh(Hk[:, :, k]) - mu, 0).sum() for k in range(pt.Nk)])
        assert abs(sft - ex) < 1e-12 * abs(ex)


def test_sum_kmesh_direct_formula():
    pt = clusters.square_bath(nb=2, nk1=3, omega_nodes=64, ngfiter=40)
    o = Oracle.from_point(pt)
    o.diagonalize()
    o.build_gf()
    c = pt.cfg
    for w in (0.1, 1.3, 25.0):
        G = nnn2lso(o.gf_cluster(1j * w)[..., 0])
        D = o.delta_bath(1j * w)
        Hl = nnn2lso(pt.Hloc)
        Hk = nnn2lso(pt.Hk)
        f = np.mean([np.log(abs(np.linalg.det(np.eye(G.shape[0]) + (D + Hl - Hk[:, :, k]) @ G)))
                     for k in range(pt.Nk)])
        assert abs(o.sum_kmesh(w) - f) < 1e-12 * max(1, abs(f))
        # Delta_bath = V (z + mu - h)^-1 V^dag (VCA_BATH_FUNCTIONS.f90:127-150)
        h = nnn2lso(pt.bath_h)
        V = pt.bath_v[:, :, 0, 0, 0, 0]
        De = V @ np.linalg.inv((1j * w + c.xmu) * np.eye(h.shape[0]) - h) @ V.conj().T
        np.testing.assert_allclose(D, De, atol=1e-13)


def test_fixed_rule_against_qagi():
    pt = clusters.chain1d(tprime=1.05, nlat=4, U=4.0, xmu=2.0, nk=16, omega_nodes=1024)
    o = Oracle.from_point(pt)
    sft, egs, oi = o.solve()
    val, err = scipy.integrate.quad(o.sum_kmesh, 0.0, np.inf, epsabs=1e-13, epsrel=1e-13, limit=500)
    oi_q = 2.0 * val / np.pi
    assert abs(oi - oi_q) < 1e-10 * abs(egs), (oi, oi_q)


def test_oracle_sigma_known_answers():
    """build_sigma_normal restatement: Sigma = 0 at U = 0, and the half-filled
    Hubbard atom's Sigma(z) = U/2 + U^2/(4z)."""
    pt = clusters.chain1d(tprime=1.0, nlat=4, U=0.0, xmu=0.0, nk=8, ngfiter=100, omega_nodes=64)
    o = Oracle.from_point(pt)
    o.solve()
    for z in (0.3j, 1.7j, 0.5 + 0.05j):
        sg, g0 = o.sigma_g0(z)
        assert np.abs(sg).max() < 1e-12
    U = 4.0
    pt = clusters.chain1d(tprime=1.0, nlat=1, U=U, xmu=U / 2, nk=4, ngfiter=20, omega_nodes=64)
    o = Oracle.from_point(pt)
    o.solve()
    for z in (0.5j, 2.0j, 1.0 + 0.1j):
        sg, g0 = o.sigma_g0(z)
        assert abs(sg[0, 0] - (U / 2 + U * U / (4 * z))) < 1e-12
        assert abs(g0[0, 0] - 1.0 / (z + U / 2)) < 1e-14  # G0 = 1/(z + mu), Hloc = 0


def test_oracle_observables_known_answers():
    """vca_lanc_observables restatement: the half-filled Hubbard atom has two
    degenerate ground states (one electron, either spin, weight 1/2 each):
    dens 1, dens_up = dens_dw = 1/2, docc 0, mag 0; a half-filled 2x2 cluster
    holds N = 4 electrons and its AFM Weiss field gives a staggered mag."""
    pt = clusters.chain1d(tprime=1.0, nlat=1, U=4.0, xmu=2.0, nk=4, ngfiter=20, omega_nodes=64)
    o = Oracle.from_point(pt)
    o.solve()
    ob = o.observables()
    assert abs(ob["dens"][0, 0] - 1.0) < 1e-14 and abs(ob["dens_up"][0, 0] - 0.5) < 1e-14
    assert abs(ob["docc"][0, 0]) < 1e-14 and abs(ob["mag"][0, 0]) < 1e-14
    pt = clusters.square(nx=2, ny=2, U=8.0, xmu=4.0, maf=0.2, nspin=2, nkx=4, nky=4, ngfiter=40,
                         omega_nodes=64)
    o = Oracle.from_point(pt)
    o.solve()
    ob = o.observables()
    assert abs(ob["dens"].sum() - 4.0) < 1e-12
    m = ob["mag"][:, 0]
    assert m[0] < -0.5 and m[1] > 0.5 and m[2] > 0.5 and m[3] < -0.5  # (-1)^(x+y) pattern


def _exact_gf_avg(o, pt, z, ispin):
    """G_ij(z) on spin `ispin` from dense resolvents of the N+-1 sectors,
    averaged over every state of the T=0 list (weight 1/zeta):
    <g|c_i (z + E - H)^-1 c_j^dag|g> + <g|c_j^dag (z - E + H)^-1 c_i|g>, with
    positions p = iorb + ilat*Norb (0-based bits of the spin word,
    VCA_SETUP.f90:705-710)."""
    c = pt.cfg
    L = c.Nlat * c.Norb
    out = np.zeros((L, L, len(z)), dtype=complex)
    states = [o.state(k, with_vector=True) for k in range(len(o.states()))]
    for isec, e0, psi in states:
        nu, nd, du, dd = o.sector_info(isec)
        for dag, fsec in ((1, o.cdg_sector(isec, ispin)), (0, o.c_sector(isec, ispin))):
            if not fsec:
                continue
            tnu, tnd, tdu, tdd = o.sector_info(fsec)
            mu_s, md_s = words(o.Ns, nu), words(o.Ns, nd)
            mu_t, md_t = words(o.Ns, tnu), words(o.Ns, tnd)
            iu = {w: k for k, w in enumerate(mu_t)}
            idd = {w: k for k, w in enumerate(md_t)}
            Vp = np.zeros((tdu * tdd, L), dtype=complex)  # c^dag_p|g> or c_p|g>
            for p in range(L):
                for s in range(du * dd):
                    wu, wd = mu_s[s % du], md_s[s // du]
                    ww = wu if ispin == 1 else wd
                    if ((ww >> p) & 1) == dag:
                        continue
                    w2 = ww ^ (1 << p)
                    t = (iu[w2] + idd[wd] * tdu) if ispin == 1 else (iu[wu] + idd[w2] * tdu)
                    Vp[t, p] += one_word_sign(ww, p) * psi[s]
            H = o.dense_h(fsec)
            I = np.eye(len(H))
            for q, zq in enumerate(z):
                if dag:
                    X = np.linalg.solve((zq + e0) * I - H, Vp)
                    out[:, :, q] += Vp.conj().T @ X          # [i, j] = v_i^H R v_j
                else:
                    X = np.linalg.solve((zq - e0) * I + H, Vp)
                    out[:, :, q] += (Vp.conj().T @ X).T      # [i, j] = w_j^H R' w_i
    return out / len(states)


@pytest.mark.parametrize("make", [
    lambda: clusters.square_bath(nb=2, nk1=3, ngfiter=200, omega_nodes=64),
    lambda: clusters.bhz(mass=2.2, delta=0.1, nk1=2, ngfiter=400, omega_nodes=64),
    lambda: clusters.square(nx=2, ny=2, U=8.0, xmu=4.0, maf=0.2, nspin=2, nkx=2, nky=2, ngfiter=100,
                            omega_nodes=64),
])
def test_gf_bath_multiorbital_and_both_spins_match_dense_resolvent(make):
    """Every element of G' on both spins, against dense ED: a bath cluster
    (hybridisation in H), the two-orbital BHZ cluster (complex amplitudes)
    and the AFM plaquette (spin-dependent Weiss field)."""
    pt = make()
    o = Oracle.from_point(pt)
    o.diagonalize()
    o.build_gf()
    c = pt.cfg
    z = np.array([0.3j, 1.2 + 0.5j, 3.0j])
    g = o.gf_cluster(z)
    for sp in range(1, c.Nspin + 1):
        ge = _exact_gf_avg(o, pt, z, sp)
        for il in range(c.Nlat):
            for jl in range(c.Nlat):
                for io in range(c.Norb):
                    for jo in range(c.Norb):
                        got = g[il, jl, sp - 1, sp - 1, io, jo]
                        ref = ge[io + il * c.Norb, jo + jl * c.Norb]
                        assert np.abs(got - ref).max() < 1e-9, (sp, il, jl, io, jo, got, ref)


def test_oracle_is_deterministic_across_thread_counts():
    """The oracle's sums run in a fixed order (contiguous chunks, k order), so
    its results carry the same bits for any number of host threads."""
    from oracle import oracle as orc
    pt = SMALL["bath2+2"]()
    out = []
    n0 = orc.set_threads(0)  # 0 leaves the count as it is and returns it
    for nt in (1, 5):
        orc.set_threads(nt)
        o = Oracle.from_point(pt)
        sft, egs, oi = o.solve()
        e, psi, it = o.lanczos_gs(32)
        out.append((sft, egs, oi, e, it, psi.tobytes(), o.sum_kmesh_complex(0.7 + 0.2j)))
    orc.set_threads(n0)
    assert out[0] == out[1]


@pytest.mark.parametrize("hfmode", [0, 1])
def test_local_term_three_orbitals_matches_the_reference_formula(hfmode):
    """The diagonal of H (stored/H_cluster_local.f90) restated element by
    element in numpy for 2 sites x 3 orbitals, both spins with different
    orbital energies, Uloc per orbital, Ust, Jh and the HFMODE shifts."""
    from vca_gb300.config import default_config
    from vca_gb300.clusters import _zeros
    rng = np.random.default_rng(17 + hfmode)
    Nlat, Norb, Nspin = 2, 3, 2
    U = [3.0, 2.5, 2.0]
    Ust, Jh, xmu = 1.4, 0.35, 0.8
    cfg = default_config(Nlat=Nlat, Norb=Norb, Nspin=Nspin, Uloc=U, Ust=Ust, Jh=Jh, xmu=xmu,
                         hfmode=hfmode, lanc_method=1, lanc_nstates_total=1)
    Hloc = _zeros(Nlat, Nlat, Nspin, Nspin, Norb, Norb)
    eps = rng.normal(size=(Nlat, Nspin, Norb))
    for il in range(Nlat):
        for s in range(Nspin):
            for io in range(Norb):
                Hloc[il, il, s, s, io, io] = eps[il, s, io]
    Hk = np.asfortranarray(Hloc[..., None].copy())
    o = Oracle(cfg, Hloc, Hk)
    checked = 0
    for isec in range(1, o.Nsectors + 1):
        nu, nd, du, dd = o.sector_info(isec)
        if du * dd > 400:
            continue
        mu_, md_ = o.sector_map(isec, 1), o.sector_map(isec, 2)
        ref = np.zeros(du * dd)
        for i in range(du * dd):
            wu, wd = int(mu_[i % du]), int(md_[i // du])
            n = lambda w, il, io: float((w >> (io + il * Norb)) & 1)
            h = 0.0
            for il in range(Nlat):
                for io in range(Norb):
                    up, dw = n(wu, il, io), n(wd, il, io)
                    h += eps[il, 0, io] * up + eps[il, 1, io] * dw - xmu * (up + dw) + U[io] * up * dw
                    if hfmode:
                        h += -0.5 * U[io] * (up + dw) + 0.25 * U[io]
                    for jo in range(io + 1, Norb):
                        uj, dj = n(wu, il, jo), n(wd, il, jo)
                        h += Ust * (up * dj + uj * dw) + (Ust - Jh) * (up * uj + dw * dj)
                        if hfmode:
                            tot = up + dw + uj + dj
                            h += -0.5 * Ust * tot + 0.25 * Ust - 0.5 * (Ust - Jh) * tot + 0.25 * (Ust - Jh)
            ref[i] = h
        np.testing.assert_allclose(o.diag_elements(isec), ref, rtol=0, atol=1e-13)
        checked += 1
    assert checked > 20


@pytest.mark.parametrize("hfshift", [0, 1])
def test_local_term_with_bath_levels_and_the_hartree_shift(hfshift):
    """Bath levels in the diagonal (diag_hybr_bath.f90:6-10, HxV_local.f90:
    80-88): bath_h(l,l,s,s,o,o) on the bit Nlat*Norb + l*Norb_bath + o
    (getBathStride, VCA_SETUP.f90:341-349), minus xmu, with HFMODE and without
    HFSHIFT shifted by -(Uloc(o)/2 + Ust(Norb-1)/2 + (Ust-Jh)(Norb-1)/2)
    (vca_set_bath, VCA_BATH_SETUP.f90:127-134), Uloc indexed by the bath
    orbital as the reference does."""
    from vca_gb300.config import default_config
    from vca_gb300.clusters import _zeros
    rng = np.random.default_rng(5 + hfshift)
    Nlat, Norb, Nspin, Nlb, Nob = 2, 1, 2, 3, 1
    U, xmu = [3.0, 0.0, 0.0, 0.0, 0.0], 1.1
    cfg = default_config(Nlat=Nlat, Norb=Norb, Nspin=Nspin, Nlat_bath=Nlb, Norb_bath=Nob, Uloc=U, xmu=xmu,
                         hfmode=1, hfshift=hfshift, lanc_method=1, lanc_nstates_total=1)
    Hloc = _zeros(Nlat, Nlat, Nspin, Nspin, Norb, Norb)
    Hk = np.asfortranarray(Hloc[..., None].copy())
    bh = _zeros(Nlb, Nlb, Nspin, Nspin, Nob, Nob)
    A = rng.normal(size=(Nlb, Nlb))
    for s in range(Nspin):
        bh[:, :, s, s, 0, 0] = A + A.T + s * np.diag(rng.normal(size=Nlb))
    bv = np.asfortranarray(rng.uniform(-0.5, 0.5, size=(Nlat, Nlb, Nspin, Nspin, Norb, Nob)).astype(complex))
    for s1 in range(Nspin):
        for s2 in range(Nspin):
            if s1 != s2:
                bv[:, :, s1, s2] = 0.0
    o = Oracle(cfg, Hloc, Hk, bh, bv)
    shift = 0.0 if hfshift else 0.5 * U[0]
    for isec in range(1, o.Nsectors + 1):
        nu, nd, du, dd = o.sector_info(isec)
        mu_, md_ = o.sector_map(isec, 1), o.sector_map(isec, 2)
        ref = np.zeros(du * dd)
        for i in range(du * dd):
            wu, wd = int(mu_[i % du]), int(md_[i // du])
            h = 0.0
            for il in range(Nlat):
                up, dw = (wu >> il) & 1, (wd >> il) & 1
                h += -xmu * (up + dw) + U[0] * up * dw - 0.5 * U[0] * (up + dw) + 0.25 * U[0]
            for lb in range(Nlb):
                b = Nlat * Norb + lb * Nob
                up, dw = (wu >> b) & 1, (wd >> b) & 1
                h += (bh[lb, lb, 0, 0, 0, 0].real - shift) * up + (bh[lb, lb, 1, 1, 0, 0].real - shift) * dw
                h -= xmu * (up + dw)
            ref[i] = h
        np.testing.assert_allclose(o.diag_elements(isec), ref, rtol=0, atol=1e-13)


def test_delta_bath_is_the_reference_formula():
    """Delta(x) = V ((x + xmu) - h)^-1 V^dag in lso layout
    (delta_bath_freq_main, VCA_BATH_FUNCTIONS.f90:127-150), written with the
    reshapes of VCA_AUX_FUNX (the Python mirror's, themselves checked against
    the reference's index loops) and numpy's inverse; the bath as
    vca_set_bath leaves it, shifted under HFMODE without HFSHIFT."""
    from vca_gb300.reshape import vca_nnn2lso_reshape, vca_rectangular_n2j_reshape
    for hf in (0, 1):
        pt = clusters.square_bath(nb=4, nk1=3, ngfiter=20, omega_nodes=64, seed=13)
        c = pt.cfg.copy()
        c.hfmode, c.hfshift = hf, 0
        pt.cfg = c
        o = Oracle.from_point(pt)
        h = np.array(pt.bath_h, dtype=complex)
        if hf:
            for lb in range(c.Nlat_bath):
                for ob in range(c.Norb_bath):
                    for s in range(c.Nspin):
                        h[lb, lb, s, s, ob, ob] -= (0.5 * c.Uloc[ob] + 0.5 * c.Ust * (c.Norb - 1)
                                                    + 0.5 * (c.Ust - c.Jh) * (c.Norb - 1))
        hl = vca_nnn2lso_reshape(h, c.Nlat_bath, c.Nspin, c.Norb_bath)
        V = vca_rectangular_n2j_reshape(pt.bath_v, c.Nlat, c.Nlat_bath, c.Nspin, c.Nspin, c.Norb, c.Norb_bath)
        for x in (0.4j, 1.5 + 0.2j, -3.0 + 1.0j):
            ref = V @ np.linalg.inv((x + c.xmu) * np.eye(len(hl)) - hl) @ V.conj().T
            np.testing.assert_allclose(o.delta_bath(x), ref, rtol=0, atol=1e-13)


def test_timed_solve_and_chain_sample():
    """The oracle entries behind the CPU baseline: solve_timed gives the
    solve's Omega with non-negative stage times that sum to at most the
    wall time, and chain_sample runs one chain per thread on a sector."""
    import time
    from vca_gb300 import clusters
    from oracle.oracle import Oracle
    pt = clusters.square(nx=2, ny=2, U=8.0, xmu=4.0, maf=0.1, nspin=2, nkx=4, nky=4, ngfiter=40, omega_nodes=64)
    ref = Oracle.from_point(pt).solve()[0]
    t0 = time.perf_counter()
    om, _, _, st = Oracle.from_point(pt).solve_timed()
    wall = time.perf_counter() - t0
    assert om == ref
    assert len(st) == 3 and min(st) >= 0.0 and sum(st) <= wall + 1e-3
    o = Oracle.from_point(pt)
    isec = 1 + 2 + 2 * 5  # sector (2,2): 36 states
    dt = o.chain_sample(isec, 4, 20)
    assert 0.0 <= dt < 10.0
