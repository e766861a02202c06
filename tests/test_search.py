"""The density searches of VCA_AUX_FUNX.f90:700-897 (host only):
search_chemical_potential walked by hand through its branches (step,
direction flip, threshold reduction, the niter guard), and run to
convergence on a smooth model density; vca_search_variable's secant step
(exact on a linear density in two calls) and its files."""
import math
import os

import numpy as np
import pytest

from vca_gb300 import solver
from vca_gb300.search import SearchState, search_chemical_potential, vca_search_variable


def test_chemical_potential_branches_by_hand():
    st = SearchState(nread=1.3, nerr=1e-4, ndelta=0.1, niter=5, write_files=False)
    # too few electrons: one step up, no flip
    var, conv = search_chemical_potential(st, 0.0, 1.0, True)
    assert (var, conv, st.nindex, st.ndelta) == (0.1, False, 1, 0.1)
    # too many: the direction flips, the step halves before it is taken
    var, conv = search_chemical_potential(st, var, 1.5, True)
    assert var == pytest.approx(0.05, abs=1e-17) and st.nindex == -1 and st.ndelta == 0.05
    # inside the threshold 1e-2 in a converged loop: no step, the threshold
    # drops a decade, the step halves again and the loop must go on
    var0 = var
    var, conv = search_chemical_potential(st, var, 1.305, True)
    assert var == var0 and st.nindex == 0 and not conv
    assert (st.nth_magnitude, st.count, st.ndelta) == (-3, 0, 0.025) and st.nth == pytest.approx(1e-3)
    # and once more down to NERR
    var, conv = search_chemical_potential(st, var, 1.3002, True)
    assert st.nth == 1e-4 and st.ndelta == 0.0125 and not conv
    # inside NERR: converged, no more reductions (nth is not above nerr)
    var, conv = search_chemical_potential(st, var, 1.30005, True)
    assert conv and st.nth == 1e-4 and st.nindex == 0
    assert [round(x[2], 12) for x in st.log] == [-0.3, 0.2, 0.005, 0.0002, 0.00005]


def test_niter_guard_with_the_default_zero():
    """niter is never read from the input file (0): the first call that does
    not converge switches the reductions off and restores 10^nth_magnitude_old."""
    st = SearchState(nread=1.0, write_files=False)
    var, conv = search_chemical_potential(st, 0.0, 0.5, True)
    assert not conv and not st.ireduce and st.nth == pytest.approx(1e-2)
    var, conv = search_chemical_potential(st, var, 1.0 + 5e-3, True)
    assert conv  # within the 1e-2 threshold, which no longer shrinks


def test_chemical_potential_converges_on_a_model_density():
    n = lambda mu: 2.0 / (1.0 + math.exp(-(mu - 1.0) / 0.3))
    st = SearchState(nread=1.3, nerr=1e-4, ndelta=0.1, niter=20, write_files=False)
    mu, conv = 0.0, False
    for _ in range(200):
        mu, conv = search_chemical_potential(st, mu, n(mu), True)
        if conv and st.nth <= st.nerr:
            break
    assert conv and st.nth == 1e-4 and abs(n(mu) - 1.3) <= 1e-4


def test_search_variable_secant_and_files(tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    (tmp_path / "var_compressibility.restart").write_text("  0.25D0\n")
    st = SearchState(nread=1.3, nerr=1e-10, ndelta=0.1, file_suffix="_x")
    dens = lambda v: 3.0 * v + 0.1
    v, conv = vca_search_variable(st, 0.2, dens(0.2), True)
    assert st.chich == 0.25 and v == pytest.approx(0.2 + 0.6 / 0.25) and not conv
    v, conv = vca_search_variable(st, v, dens(v), True)
    assert st.chich == pytest.approx(3.0) and abs(dens(v) - 1.3) < 1e-12
    v, conv = vca_search_variable(st, v, dens(v), True)
    assert conv
    lines = (tmp_path / "search_variable_iteration_info_x.ed").read_text().splitlines()
    assert lines[0] == "#var,ntmp,ndiff" and len(lines) == 4
    assert float((tmp_path / "var_compressibility.used").read_text()) == pytest.approx(3.0)


def test_module_level_names_share_one_state(tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    solver.search_state = SearchState(nread=2.0, write_files=True, niter=3)
    var, conv = solver.search_chemical_potential(0.0, 1.0, True)
    assert var == 0.1 and solver.search_state.count == 1
    assert os.path.exists("search_mu_iteration.ed")
    assert np.loadtxt("search_mu_iteration.ed").tolist() == [0.1, 1.0, -1.0]
