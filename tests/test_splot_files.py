"""The splot reader of vca_read_impSigma (VCA_IO.f90:208-239) without a GPU:
columns x, Im, Re in the forms a Fortran writer may use (E or D
exponents, comma or blank separators), bit-exact on 17-digit text, and
VCA_ERR_IO on a short or missing file."""
import numpy as np
import pytest

from vca_gb300 import solver
from vca_gb300.solver import VcaError, read_splot, splot_name


def test_reader_forms(tmp_path):
    p = tmp_path / "impSigma_Isite0001_Jsite0002_l11_s1_iw.vca"
    p.write_text("  0.314159265358979D+00,  -1.5D-01 ,  2.25\n 0.94247779607693797E+00 3e-1 -4\n")
    x, y = read_splot(str(p))
    np.testing.assert_array_equal(x, [0.314159265358979, 0.94247779607693797])
    np.testing.assert_array_equal(y, [2.25 - 0.15j, -4 + 0.3j])
    assert splot_name("impSigma", 1, 2, 1, 1, 1, True) == p.name


def test_round_trip_of_17_digit_text(tmp_path):
    rng = np.random.default_rng(2)
    x = rng.normal(size=50)
    y = rng.normal(size=50) * 10.0 ** rng.integers(-200, 200, size=50) + 1j * rng.normal(size=50)
    p = tmp_path / "f.vca"
    with open(p, "w") as f:
        for a, b in zip(x, y):
            f.write(f"{a:24.16E} {b.imag:24.16E} {b.real:24.16E}\n")
    x2, y2 = read_splot(str(p))
    assert np.array_equal(x2, x) and np.array_equal(y2, y)


def test_short_and_missing_files(tmp_path):
    p = tmp_path / "s.vca"
    p.write_text("1 2 3\n4 5\n")
    with pytest.raises(VcaError) as e:
        read_splot(str(p), 2)
    assert e.value.code == -10
    with pytest.raises(VcaError) as e:
        read_splot(str(tmp_path / "none.vca"), 1)
    assert e.value.code == -10
    solver.load().vca_gpu_finalize()
    assert solver.load().vca_read_impSigma() == -3
