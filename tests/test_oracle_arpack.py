"""The oracle's LANC_METHOD="arpack" path, the reference default
(VCA_DIAG.f90:98-111,153-170,220-236; vca_post_diag :395-451): several
eigenpairs per sector, Neigen = min(dim, neigen_sector).

* the multi-eigenpair solver (Lanczos with full reorthogonalisation above
  LANC_DIM_THRESHOLD) against numpy's dense eigh;
* T=0 with a degenerate ground level inside sectors (the 2x2 plaquette at
  U=8, three electrons: a doublet in each of the sectors (2,1) and (1,2)):
  the whole multiplet is kept (zeta = 4, where one state per sector keeps 2),
  and G'_ii(z) is the multiplet average, checked against an independent
  numpy resolvent evaluation  (1/zeta) sum_g [<g|c (z + E - H)^-1 c^dag|g> +
  <g|c^dag (z - E + H)^-1 c|g>];
* finite T at U=0: with every sector's excited states in the list the
  Omega of the annealed list is the exact lattice grand potential; one state
  per sector misses the in-sector excitations;
* finite T at U=4: with all states listed (two- and three-site chains), zeta,
  Omega', G'_ii(z) and G'_ij(z) equal the exact thermal Lehmann results (the
  Boltzmann weights of the chains, pesoBZ = norm2 e^{-beta(E_i-E_gs)}/zeta;
  the mixed channels and their recombination, with four channels and two).
"""
import numpy as np
import pytest

from vca_gb300 import clusters
from vca_gb300.clusters import nnn2lso
from vca_gb300.config import LANC_ARPACK, LANC_LANCZOS
from oracle.oracle import Oracle


def _with(pt, **kw):
    cfg = pt.cfg.copy()
    for k, v in kw.items():
        setattr(cfg, k, v)
    pt.cfg = cfg
    return pt


def test_lowest_pairs_match_dense_eigh():
    pt = _with(clusters.bhz(mass=2.2, delta=0.1, nk1=4, ngfiter=60, omega_nodes=256),
               lanc_method=LANC_ARPACK, lanc_dim_threshold=4)
    o = Oracle.from_point(pt)
    checked = 0
    for isec in range(1, o.Nsectors + 1):
        D = o.dim(isec)
        if not 100 <= D <= 900:
            continue
        e, v = o.lowest_pairs(isec, 6)
        w, Z = np.linalg.eigh(o.dense_h(isec))
        np.testing.assert_allclose(e, w[:6], rtol=0, atol=1e-10 * max(1.0, abs(w[0])))
        for j in range(6):
            gaps = np.abs(w - w[j])
            gaps[j] = np.inf
            if gaps.min() > 1e-6:  # a simple level: the vector up to a phase
                assert abs(abs(np.vdot(Z[:, j], v[:, j])) - 1.0) < 1e-9
        checked += 1
        if checked == 4:
            break
    assert checked == 4


def _plaquette(method, xmu=0.95):
    pt = clusters.square(nx=2, ny=2, U=8.0, xmu=xmu, maf=0.0, nspin=1, nkx=4, nky=4, ngfiter=100,
                         omega_nodes=256)
    return _with(pt, lanc_method=method)


def _apply(o, src, g, site, dag):
    """c^dag_{site,up} |g> (dag) or c_{site,up} |g> in the target sector:
    up word bit `site`, sign (-1)^(occupied up bits below it)."""
    tgt = o.cdg_sector(src, 1) if dag else o.c_sector(src, 1)
    mu_s, md_s = o.sector_map(src, 1), o.sector_map(src, 2)
    mu_t = o.sector_map(tgt, 1)
    rank = {int(w): r for r, w in enumerate(mu_t)}
    out = np.zeros(o.dim(tgt), dtype=np.complex128)
    for idw in range(len(md_s)):
        for iup, w in enumerate(mu_s):
            w = int(w)
            occ = (w >> site) & 1
            if occ == dag:
                continue
            sign = -1.0 if bin(w & ((1 << site) - 1)).count("1") % 2 else 1.0
            out[rank[w ^ (1 << site)] + idw * len(mu_t)] += sign * g[iup + idw * len(mu_s)]
    return tgt, out


def test_t0_keeps_the_whole_multiplet_and_averages_gf():
    o = Oracle.from_point(_plaquette(LANC_ARPACK))
    o.solve()
    st = o.states()
    assert sorted(s for s, _ in st) == [8, 8, 12, 12]
    assert o.thermal()["zeta"] == 4.0
    one = Oracle.from_point(_plaquette(LANC_LANCZOS))
    one.solve()
    assert sorted(s for s, _ in one.states()) == [8, 12] and one.thermal()["zeta"] == 2.0
    # independent multiplet average of G'_ii
    e0 = min(e for _, e in st)
    ground = []
    for isec in (8, 12):
        w, Z = np.linalg.eigh(o.dense_h(isec))
        ground += [(isec, Z[:, j]) for j in range(len(w)) if w[j] - e0 < 1e-9]
    assert len(ground) == 4
    zs = np.array([0.4j, 1.3 + 0.4j, -2.0 + 1.0j])
    G = o.gf_cluster(zs)
    for site in range(4):
        ref = np.zeros(len(zs), dtype=np.complex128)
        for isec, g in ground:
            for dag in (True, False):
                tgt, v = _apply(o, isec, g, site, dag)
                if tgt == 0 or not np.any(v):
                    continue
                Ht = o.dense_h(tgt)
                I = np.eye(len(v))
                for q, z in enumerate(zs):
                    A = (z + e0) * I - Ht if dag else (z - e0) * I + Ht
                    ref[q] += np.vdot(v, np.linalg.solve(A, v))
        ref /= len(ground)
        got = G[site, site, 0, 0, 0, 0, :]
        assert np.abs(got - ref).max() < 1e-10, (site, got, ref)


def _lattice_omega(pt, beta, mu):
    Hk = nnn2lso(pt.Hk)
    tot = 0.0
    for k in range(pt.Nk):
        e = np.linalg.eigvalsh(Hk[:, :, k]) - mu
        tot -= np.sum(np.logaddexp(0.0, -beta * e)) / beta
    return (3 - pt.cfg.Nspin) * tot / pt.Nk


def test_finite_t_u0_is_the_lattice_value_with_excited_states():
    beta = 3.0
    res = {}
    for method in (LANC_ARPACK, LANC_LANCZOS):
        pt = clusters.chain1d(tprime=1.0, nlat=2, U=0.0, xmu=0.0, nk=32, ngfiter=50, omega_nodes=64,
                              lanc_nstates_total=2, beta=beta, bandwidth=4.0)
        pt = _with(pt, lanc_method=method)
        o = Oracle.from_point(pt)
        sft, _, _ = o.solve()
        res[method] = (sft, o.thermal(), len(o.states()), o)
        exact = _lattice_omega(pt, beta, 0.0)
    sft, t, n, o = res[LANC_ARPACK]
    # every one of the 16 cluster states is in the list (the weight of the
    # highest is exp(-12) > CUTOFF)
    assert n == 16 and t["finite_t"] == 1
    assert abs(sft - exact) < 1e-10, (sft, exact)
    # the in-sector excitations carry exp(-beta * 2): one state per sector
    # (9 sectors) misses them
    sft1, _, n1, _ = res[LANC_LANCZOS]
    assert n1 == 9 and abs(sft1 - exact) > 1e-4
    # neigen_sector after the sweeps: each sector's count in the list + 1
    # (the list holds every state of every sector)
    ne = o.neigen()
    for isec in range(1, o.Nsectors + 1):
        assert ne[isec - 1] == o.dim(isec) + 1


def test_finite_t_gf_is_the_exact_thermal_average():
    """Interacting two-site chain (U=4) at beta=1 in the arpack method: the
    list holds all 16 cluster states, so G'_ii(z) must be the exact thermal
    Lehmann sum (1/Z) sum_m e^{-beta E_m} [<m|c (z+E_m-H)^-1 c^dag|m> +
    <m|c^dag (z-E_m+H)^-1 c|m>] over every eigenstate m of every sector,
    evaluated here with dense resolvents, and Omega' = -T ln Z."""
    beta = 1.0
    pt = clusters.chain1d(tprime=1.0, nlat=2, U=4.0, xmu=1.3, nk=8, ngfiter=50, omega_nodes=64,
                          lanc_nstates_total=2, beta=beta, bandwidth=4.0)
    pt = _with(pt, lanc_method=LANC_ARPACK, lanc_niter_spectrum=20)
    o = Oracle.from_point(pt)
    o.solve()
    assert len(o.states()) == 16
    eig = {isec: np.linalg.eigh(o.dense_h(isec)) for isec in range(1, o.Nsectors + 1)}
    e0 = min(w.min() for w, _ in eig.values())
    Z = sum(np.exp(-beta * (w - e0)).sum() for w, _ in eig.values())
    t = o.thermal()
    assert abs(t["zeta"] - Z) < 1e-12 * Z
    assert abs(t["omega_prime"] - (e0 - np.log(Z) / beta)) < 1e-12
    zs = np.array([0.5j, 1.1 + 0.3j, -0.7 + 2.0j])
    G = o.gf_cluster(zs)
    for site in range(2):
        ref = np.zeros(len(zs), dtype=np.complex128)
        for isec, (w, V) in eig.items():
            for m in range(len(w)):
                pm = np.exp(-beta * (w[m] - e0)) / Z
                for dag in (True, False):
                    tgt, v = _apply(o, isec, V[:, m], site, dag)
                    if tgt == 0 or not np.any(v):
                        continue
                    Ht = o.dense_h(tgt)
                    I = np.eye(len(v))
                    for q, z in enumerate(zs):
                        A = (z + w[m]) * I - Ht if dag else (z - w[m]) * I + Ht
                        ref[q] += pm * np.vdot(v, np.linalg.solve(A, v))
        assert np.abs(G[site, site, 0, 0, 0, 0, :] - ref).max() < 1e-10, site


@pytest.mark.parametrize("symmetric", [0, 1])
def test_finite_t_offdiagonal_gf_is_the_exact_thermal_average(symmetric):
    """The same thermal cluster, off-diagonal elements: G'_ij(z) = (1/Z)
    sum_m e^{-beta E_m} [<m|c_i (z+E_m-H)^-1 c_j^dag|m> + <m|c_j^dag
    (z-E_m+H)^-1 c_i|m>], which the chains reach through the mixed channels
    and the recombination 1/2[G^mix - (1 - i chan4)(G_ii + G_jj)]
    (VCA_GF_NORMAL.f90:89-101) -- with four channels (VCA_GF_SYMMETRIC=F) and
    with two (=T, a real model)."""
    beta = 1.0
    pt = clusters.chain1d(tprime=1.0, nlat=3, U=4.0, xmu=1.3, nk=8, ngfiter=80, omega_nodes=64,
                          lanc_nstates_total=2, beta=beta, bandwidth=4.0)
    pt = _with(pt, lanc_method=LANC_ARPACK, lanc_niter_spectrum=40, vca_gf_symmetric=symmetric)
    o = Oracle.from_point(pt)
    o.solve()
    assert len(o.states()) == 64
    eig = {isec: np.linalg.eigh(o.dense_h(isec)) for isec in range(1, o.Nsectors + 1)}
    e0 = min(w.min() for w, _ in eig.values())
    Z = sum(np.exp(-beta * (w - e0)).sum() for w, _ in eig.values())
    zs = np.array([0.5j, 1.1 + 0.3j])
    G = o.gf_cluster(zs)
    for i, j in ((0, 1), (1, 0), (0, 2)):
        ref = np.zeros(len(zs), dtype=np.complex128)
        for isec, (w, V) in eig.items():
            for m in range(len(w)):
                pm = np.exp(-beta * (w[m] - e0)) / Z
                if pm < 1e-300:
                    continue
                ti, vi = _apply(o, isec, V[:, m], i, True)
                tj, vj = _apply(o, isec, V[:, m], j, True)
                if ti and np.any(vi) and np.any(vj):
                    Ht = o.dense_h(ti)
                    for q, z in enumerate(zs):
                        ref[q] += pm * np.vdot(vi, np.linalg.solve((z + w[m]) * np.eye(len(vi)) - Ht, vj))
                ti, wi = _apply(o, isec, V[:, m], i, False)
                tj, wj = _apply(o, isec, V[:, m], j, False)
                if ti and np.any(wi) and np.any(wj):
                    Ht = o.dense_h(ti)
                    for q, z in enumerate(zs):
                        ref[q] += pm * np.vdot(wj, np.linalg.solve((z - w[m]) * np.eye(len(wi)) + Ht, wi))
        got = G[i, j, 0, 0, 0, 0, :]
        assert np.abs(got - ref).max() < 1e-10, (i, j, got, ref)
