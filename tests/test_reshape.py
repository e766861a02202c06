"""The reshapes of VCA_AUX_FUNX.f90:175-468 against the reference's index
loops written out element by element (1-based formulas as in the source),
with trailing axes, and their round trips; the library's own nnn2lso of the
synthetic inputs agrees."""
import numpy as np

from vca_gb300 import clusters
from vca_gb300.solver import (vca_lso2nnn_reshape, vca_nn2so_reshape, vca_nnn2lso_reshape,
                              vca_rectangular_j2n_reshape, vca_rectangular_n2j_reshape, vca_so2nn_reshape)


def test_rectangular_against_the_loops():
    rng = np.random.default_rng(1)
    Nlat, Nlat2, Nspin, Nspin2, Norb, Norb2 = 3, 2, 2, 1, 2, 3
    H = rng.normal(size=(Nlat * Nspin * Norb, Nlat2 * Nspin2 * Norb2, 4)) + 1j * rng.normal(
        size=(Nlat * Nspin * Norb, Nlat2 * Nspin2 * Norb2, 4))
    N = vca_rectangular_j2n_reshape(H, Nlat, Nlat2, Nspin, Nspin2, Norb, Norb2)
    for il in range(1, Nlat + 1):
        for jl in range(1, Nlat2 + 1):
            for isp in range(1, Nspin + 1):
                for jsp in range(1, Nspin2 + 1):
                    for io in range(1, Norb + 1):
                        for jo in range(1, Norb2 + 1):
                            i = io + (il - 1) * Norb + (isp - 1) * Norb * Nlat
                            j = jo + (jl - 1) * Norb2 + (jsp - 1) * Norb2 * Nlat2
                            assert np.array_equal(N[il - 1, jl - 1, isp - 1, jsp - 1, io - 1, jo - 1], H[i - 1, j - 1])
    assert np.array_equal(vca_rectangular_n2j_reshape(N, Nlat, Nlat2, Nspin, Nspin2, Norb, Norb2), H)


def test_square_and_so_forms():
    rng = np.random.default_rng(2)
    Nlat, Nspin, Norb = 2, 2, 3
    n = Nlat * Nspin * Norb
    H = rng.normal(size=(n, n))
    N = vca_lso2nnn_reshape(H, Nlat, Nspin, Norb)
    assert np.array_equal(vca_nnn2lso_reshape(N, Nlat, Nspin, Norb), H)
    assert np.array_equal(clusters.nnn2lso(N), H)
    S = rng.normal(size=(Nspin * Norb, Nspin * Norb, 5))
    M = vca_so2nn_reshape(S, Nspin, Norb)
    for isp in range(1, Nspin + 1):
        for jsp in range(1, Nspin + 1):
            for io in range(1, Norb + 1):
                for jo in range(1, Norb + 1):
                    i, j = io + (isp - 1) * Norb, jo + (jsp - 1) * Norb
                    assert np.array_equal(M[isp - 1, jsp - 1, io - 1, jo - 1], S[i - 1, j - 1])
    assert np.array_equal(vca_nn2so_reshape(M, Nspin, Norb), S)
