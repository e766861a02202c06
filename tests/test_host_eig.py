"""The host eigensolvers of the "arpack" diagonalisation (implicit QL on the
Ritz tridiagonal, cyclic Jacobi below LANC_DIM_THRESHOLD) through the C-ABI
against numpy's eigh.  No GPU."""
import numpy as np
import pytest

from vca_gb300.solver import herm_eig, tridiag_eig


@pytest.mark.parametrize("n,seed", [(1, 0), (2, 1), (7, 2), (60, 3), (300, 4)])
def test_tridiag_eig_matches_eigh(n, seed):
    rng = np.random.default_rng(seed)
    d = rng.normal(size=n)
    e = rng.normal(size=max(n - 1, 0))
    T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    w, Z = tridiag_eig(d, e)
    ref = np.linalg.eigvalsh(T)
    scale = max(1.0, np.abs(ref).max())
    np.testing.assert_allclose(w, ref, rtol=0, atol=1e-13 * scale * max(1, n) ** 0.5)
    np.testing.assert_allclose(Z.T @ Z, np.eye(n), atol=1e-12)
    np.testing.assert_allclose(T @ Z, Z * w, atol=1e-11 * scale)


def test_tridiag_eig_degenerate_and_split():
    # a split matrix (zero coupling) with a repeated eigenvalue
    d = np.array([1.0, 2.0, 1.0, 2.0, 3.0])
    e = np.array([0.5, 0.0, 0.5, 0.0])
    w, Z = tridiag_eig(d, e)
    T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    np.testing.assert_allclose(w, np.linalg.eigvalsh(T), atol=1e-14)
    np.testing.assert_allclose(T @ Z, Z * w, atol=1e-13)


@pytest.mark.parametrize("n,seed,cplx", [(1, 0, True), (5, 1, False), (16, 2, True), (64, 3, True)])
def test_herm_eig_matches_eigh(n, seed, cplx):
    rng = np.random.default_rng(seed)
    A = rng.normal(size=(n, n)) + (1j * rng.normal(size=(n, n)) if cplx else 0.0)
    A = A + A.conj().T
    w, Z = herm_eig(A)
    ref = np.linalg.eigvalsh(A)
    np.testing.assert_allclose(w, ref, rtol=0, atol=1e-12 * max(1.0, np.abs(ref).max()))
    np.testing.assert_allclose(Z.conj().T @ Z, np.eye(n), atol=1e-12)
    np.testing.assert_allclose(A @ Z, Z * w, atol=1e-11 * max(1.0, np.abs(ref).max()))


def test_herm_eig_multiplet():
    # a doubly degenerate level: the eigenvectors span its eigenspace
    rng = np.random.default_rng(7)
    Q, _ = np.linalg.qr(rng.normal(size=(6, 6)) + 1j * rng.normal(size=(6, 6)))
    lam = np.array([-1.0, -1.0, 0.5, 2.0, 2.0, 3.0])
    A = (Q * lam) @ Q.conj().T
    w, Z = herm_eig(A)
    np.testing.assert_allclose(w, lam, atol=1e-13)
    P = Z[:, :2] @ Z[:, :2].conj().T
    np.testing.assert_allclose(P, Q[:, :2] @ Q[:, :2].conj().T, atol=1e-12)
