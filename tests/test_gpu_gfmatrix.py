"""GPU: GFmatrix restart files through the C-ABI (vca_gpu_save_gfprime /
vca_gpu_read_gfprime, VCA_AUX_FUNX.f90:601-697).

* save: the file holds the oracle's impGmatrix -- every element, every state
  (in the GPU's list order, which inside a degenerate group follows each
  run's rounding), 2 or 4 channels, the same excitation counts (exact) --
  with pole sums
  equal to the oracle's at points off the real axis (1e-8, the G' parity
  tolerance), and exactly the tables vca_gpu_get_gf_channel lists;
* read into a fresh context (init, no solve): G'(z) from the loaded tables
  on the GPU equals the solve's continued fractions (1e-10) and the oracle's
  G' (1e-8); a file written from the oracle's tables gives the oracle's G'
  to 1e-12 (the same sums in the same order);
* the grid getters keep the solve's tables after a read, a solve drops the
  loaded tables, and a save of loaded tables writes them back unchanged.
"""
import numpy as np
import pytest

from vca_gb300 import clusters
from vca_gb300.solver import VcaError, VcaSolver, gfm_elements, gfprime_path
from oracle import gfmatrix as ogm
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

G_TOL = 1e-8
Z = np.array([0.3 + 0.1j, -1.0 + 1.0j, 2.0 + 5.0j, 0.7j])


def _ft(pt, beta, bandwidth):
    cfg = pt.cfg.copy()
    cfg.lanc_nstates_total, cfg.beta, cfg.bandwidth = 2, beta, bandwidth
    pt.cfg = cfg
    return pt


def _chan2(pt):
    pt.cfg.vca_gf_symmetric = 1
    return pt


POINTS = {
    "chain4": lambda: clusters.chain1d(tprime=0.9, nlat=4, U=4.0, xmu=2.0, nk=16, ngfiter=100, omega_nodes=256),
    "square2x2_afm": lambda: clusters.square(nx=2, ny=2, U=8.0, xmu=4.0, maf=0.2, nspin=2, nkx=6, nky=6,
                                             ngfiter=80, omega_nodes=256),
    "bath2x2+4": lambda: clusters.square_bath(nb=4, nk1=6, ngfiter=60, omega_nodes=256, seed=11),
    "bhz_small": lambda: clusters.bhz(mass=2.2, delta=0.1, nk1=4, ngfiter=60, omega_nodes=256),
    "square2x2_afm_b8": lambda: _ft(clusters.square(nx=2, ny=2, U=8.0, xmu=4.0, maf=0.2, nspin=2, nkx=4, nky=4,
                                                    ngfiter=60, omega_nodes=64), 8.0, 8.0),
    "chain4_chan2": lambda: _chan2(clusters.chain1d(tprime=0.9, nlat=4, U=4.0, xmu=2.0, nk=16, ngfiter=100,
                                                    omega_nodes=256)),
}


def psum(p, w):
    p = np.asarray(p, np.complex128)
    w = np.asarray(w, np.complex128)
    return (w[None, :] / (Z[:, None] - p[None, :])).sum(axis=1)


def _align(ref, states, ref_states):
    """The oracle's table with its states in the order of the GPU's list.
    Inside a group of degenerate states the list order follows each run's
    rounding; the Lanczos method keeps one state per sector, so the sector
    names the state."""
    assert sorted(x[0] for x in states) == sorted(x[0] for x in ref_states)
    pos = {sec: k for k, (sec, _) in enumerate(ref_states)}
    return [[el[pos[sec]] for sec, _ in states] for el in ref]


def _read(path, nelem, formatted):
    data = open(path, "rb").read()
    return ogm.decode_formatted(data.decode(), nelem) if formatted else ogm.decode_unformatted(data, nelem)


@pytest.mark.parametrize("name", list(POINTS))
def test_save_matches_oracle_and_read_gives_back_gf(tmp_path, name):
    pt = POINTS[name]()
    s = VcaSolver(pt.cfg, pt.bath_h, pt.bath_v)
    s.solve(pt.Hloc, pt.Hk, pt.bath_h, pt.bath_v)
    g_solve = s.gf_cluster(Z)
    o = Oracle.from_point(pt)
    o.solve()
    ref = _align(ogm.table_from_oracle(o, pt.cfg), s.states(), o.states())
    els = gfm_elements(pt.cfg)
    stem = str(tmp_path / "gfprime")
    for formatted in (False, True):
        path = s.save_gfprime(stem, used=formatted, use_formatted=formatted)
        assert path == gfprime_path(stem, formatted)
        t = _read(path, len(els), formatted)
        assert ogm.same_structure(t, ref), name
        worst = 0.0
        for el, er in zip(t, ref):
            for st, sr in zip(el, er):
                for (p, w), (pr, wr) in zip(st, sr):
                    if len(p):
                        worst = max(worst, np.abs(psum(p, w) - psum(pr, wr)).max())
        assert worst < G_TOL, (name, formatted, worst)
        # the file is what the channel getter lists
        for (il, jl, sp, io, jo), el in list(zip(els, t))[:: max(1, len(els) // 7)]:
            for k, st in enumerate(el):
                for ich, (p, w) in enumerate(st):
                    gp, gw = s.gf_channel(il, jl, sp, io, jo, k + 1, ich + 1)
                    assert np.array_equal(gp, p) and np.array_equal(gw, w)
    s.close()
    # a fresh context reads the file back: G' on the GPU from the poles
    r = VcaSolver(pt.cfg, pt.bath_h, pt.bath_v)
    for formatted in (False, True):
        r.read_gfprime(stem, used=formatted, use_formatted=formatted)
        g_read = r.gf_cluster(Z)
        assert np.abs(g_read - g_solve).max() < 1e-10, (name, formatted)
        assert np.abs(g_read - o.gf_cluster(Z)).max() < G_TOL, (name, formatted)
    r.close()


@pytest.mark.parametrize("name", ["chain4", "bhz_small", "square2x2_afm_b8"])
def test_read_of_oracle_tables_gives_the_oracle_gf(tmp_path, name):
    pt = POINTS[name]()
    o = Oracle.from_point(pt)
    o.solve()
    t = ogm.table_from_oracle(o, pt.cfg)
    stem = str(tmp_path / "orc")
    with open(gfprime_path(stem), "wb") as f:
        f.write(ogm.encode_unformatted(t))
    with open(gfprime_path(stem, True), "w") as f:
        f.write(ogm.encode_formatted(t))
    r = VcaSolver(pt.cfg, pt.bath_h, pt.bath_v)
    g_ref = o.gf_cluster(Z)
    for used in (False, True):
        r.read_gfprime(stem, used=used, use_formatted=used)
        g = r.gf_cluster(Z)
        assert np.abs(g - g_ref).max() <= 1e-12 * max(1.0, np.abs(g_ref).max()), (name, used)
        il, jl, sp, io, jo = gfm_elements(pt.cfg)[1]
        p, w = r.gf_channel(il, jl, sp, io, jo, 1, 1)
        assert ogm.bit_equal([[[(p, w)]]], [[[t[1][0][0]]]])
    r.close()


def test_loaded_tables_and_the_solve(tmp_path):
    pt = POINTS["square2x2_afm"]()
    cfg = pt.cfg.copy()
    cfg.Lmats, cfg.Lreal = 16, 16
    s = VcaSolver(cfg)
    with pytest.raises(VcaError) as e:
        s.save_gfprime(str(tmp_path / "none"))
    assert e.value.code == -3  # impGmatrix not allocated
    with pytest.raises(VcaError) as e:
        s.read_gfprime(str(tmp_path / "absent"))
    assert e.value.code == -10
    s.solve(pt.Hloc, pt.Hk)
    g0 = s.gf_cluster(Z)
    sig0, gm0 = s.sigma_matsubara(), s.gimp_matsubara()
    stem = str(tmp_path / "a")
    s.save_gfprime(stem)
    # tables of another point, loaded on top of this solve
    other = clusters.square(nx=2, ny=2, U=6.0, xmu=3.0, maf=0.0, nspin=2, nkx=6, nky=6, ngfiter=80,
                            omega_nodes=256)
    o = Oracle.from_point(other)
    o.solve()
    t = ogm.table_from_oracle(o, other.cfg)
    with open(gfprime_path(str(tmp_path / "b")), "wb") as f:
        f.write(ogm.encode_unformatted(t))
    s.read_gfprime(str(tmp_path / "b"))
    assert np.abs(s.gf_cluster(Z) - o.gf_cluster(Z)).max() < 1e-12
    # the grids of build_gf_normal stay the solve's
    assert np.abs(s.sigma_matsubara() - sig0).max() < 1e-12 and np.abs(s.gimp_matsubara() - gm0).max() < 1e-12
    # a save of the loaded tables writes them back unchanged
    s.save_gfprime(str(tmp_path / "c"))
    assert open(gfprime_path(str(tmp_path / "c")), "rb").read() == ogm.encode_unformatted(t)
    # the next solve drops them
    s.solve(pt.Hloc, pt.Hk)
    assert np.abs(s.gf_cluster(Z) - g0).max() < 1e-12
    s.save_gfprime(str(tmp_path / "d"))
    nel = len(gfm_elements(cfg))
    ta, td = (_read(gfprime_path(str(tmp_path / x)), nel, False) for x in ("a", "d"))
    assert ogm.same_structure(ta, td)
    for ea, ed in zip(ta, td):
        for sa, sd in zip(ea, ed):
            for (pa, wa), (pd, wd) in zip(sa, sd):
                if len(pa):
                    assert np.abs(psum(pa, wa) - psum(pd, wd)).max() < 1e-12
    s.close()
