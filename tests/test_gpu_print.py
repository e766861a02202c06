"""GPU: splot files of Sigma, G' and G0 (vca_print_impSigma / _impG /
_impG0, VCA_IO.f90:112-205) through the C-ABI.

* one file per spin-diagonal element and grid, with the reference's names
  (file_suffix included), columns x, Im, Re equal bit-exact to the getters'
  arrays (17 significant digits);
* PRINT_SIGMA / PRINT_IMPG / PRINT_IMPG0 print at the end of a solve;
* the restart files take the same file_suffix when none is passed.
"""
import os

import numpy as np
import pytest

from vca_gb300 import clusters
from vca_gb300.solver import VcaError, VcaSolver, gfprime_path, read_splot, splot_name

pytestmark = pytest.mark.gpu


def _point(**kw):
    pt = clusters.square(nx=2, ny=2, U=8.0, xmu=4.0, maf=0.2, nspin=2, nkx=4, nky=4, ngfiter=60, omega_nodes=128)
    cfg = pt.cfg.copy()
    cfg.Lmats, cfg.Lreal = 12, 9
    for k, v in kw.items():
        setattr(cfg, k, v)
    pt.cfg = cfg
    return pt


def _elements(c):
    return [(il, jl, io, jo, s) for il in range(1, c.Nlat + 1) for jl in range(1, c.Nlat + 1)
            for io in range(1, c.Norb + 1) for jo in range(1, c.Norb + 1) for s in range(1, c.Nspin + 1)]


def _check(s, c, name, getter, mats, suffix):
    arr = getter()
    x_ref = (np.pi / c.beta * (2 * np.arange(1, c.Lmats + 1) - 1)) if mats else np.linspace(c.wini, c.wfin, c.Lreal)
    for il, jl, io, jo, sp in _elements(c):
        x, y = read_splot(splot_name(name, il, jl, io, jo, sp, mats, suffix))
        np.testing.assert_allclose(x, x_ref, rtol=0, atol=1e-13)
        assert np.array_equal(y, arr[il - 1, jl - 1, sp - 1, sp - 1, io - 1, jo - 1, :]), (name, il, jl, sp)


def test_print_calls_write_the_getters_arrays(tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    pt = _point(file_suffix=b"_t")
    c = pt.cfg
    s = VcaSolver(c)
    with pytest.raises(VcaError) as e:
        s.print_impG()
    assert e.value.code == -3
    s.solve(pt.Hloc, pt.Hk)
    assert os.listdir(tmp_path) == []  # the flags are off
    s.print_impSigma()
    s.print_impG()
    s.print_impG0()
    n_el = c.Nlat ** 2 * c.Norb ** 2 * c.Nspin
    assert len(os.listdir(tmp_path)) == 3 * 2 * n_el
    for name, mg, rg in (("impSigma", s.sigma_matsubara, s.sigma_realaxis), ("impG", s.gimp_matsubara, s.gimp_realaxis),
                         ("impG0", s.g0_matsubara, s.g0_realaxis)):
        _check(s, c, name, mg, True, "_t")
        _check(s, c, name, rg, False, "_t")
    # restart files take the config's file_suffix
    assert s.save_gfprime("gfprime") == gfprime_path("gfprime", False, "_t")
    assert os.path.exists("gfprime_t.restart")
    s.close()


def test_print_flags_print_at_the_end_of_a_solve(tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    pt = _point(print_sigma=1, print_impg=0, print_impg0=1)
    c = pt.cfg
    s = VcaSolver(c)
    s.solve(pt.Hloc, pt.Hk)
    names = os.listdir(tmp_path)
    n_el = c.Nlat ** 2 * c.Norb ** 2 * c.Nspin
    assert len(names) == 2 * 2 * n_el
    assert not any(n.startswith("impG_") for n in names)
    _check(s, c, "impSigma", s.sigma_matsubara, True, "")
    _check(s, c, "impG0", s.g0_realaxis, False, "")
    s.close()


def test_read_impsigma_gives_the_printed_sigma_back(tmp_path, monkeypatch):
    """vca_read_impSigma (VCA_IO.f90:208-239): a fresh context reads the
    files of another and its Sigma getters return them, bit-exact, until a
    solve replaces them."""
    monkeypatch.chdir(tmp_path)
    pt = _point(file_suffix=b"_r")
    c = pt.cfg
    s = VcaSolver(c)
    s.solve(pt.Hloc, pt.Hk)
    sm, sr = s.sigma_matsubara(), s.sigma_realaxis()
    s.print_impSigma()
    s.close()
    r = VcaSolver(c)
    with pytest.raises(VcaError) as e:
        r.sigma_matsubara()
    assert e.value.code == -3
    r.read_impSigma()
    assert np.array_equal(r.sigma_matsubara(), sm) and np.array_equal(r.sigma_realaxis(), sr)
    # the solve recomputes Sigma from its own chains
    r.solve(pt.Hloc, pt.Hk)
    assert np.abs(r.sigma_matsubara() - sm).max() < 1e-12
    r.close()
    with pytest.raises(VcaError) as e:
        VcaSolver(_point(file_suffix=b"_none").cfg).read_impSigma()
    assert e.value.code == -10
