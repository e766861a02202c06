"""Fixed-point column-batch H x v through the C-ABI on sectors large enough
that every kernel form runs with many warps per CTA.

The staged form (shared-memory up block, streamed down blocks) rounds the
exact int128 sum of every element once; the warp form rounds its up and down
halves separately, so the two agree to one unit of 2^-G.  Both must match
the oracle's FP64 H x v of the same fixed-point input to their output
rounding (tested at 1e-13 of the column scale).
"""
import numpy as np
import pytest

from vca_gb300 import clusters
from vca_gb300.solver import VcaSolver
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

SLAB = 8


def _point():
    return clusters.square(nx=3, ny=3, U=8.0, xmu=4.0, maf=0.2, nspin=2, nkx=4, nky=4, ngfiter=40,
                           omega_nodes=64)


def _to_slabs(a):
    """(D, m) row-major -> slab-major flat array (slabs of 8 columns)."""
    D, m = a.shape
    return np.ascontiguousarray(a.reshape(D, m // SLAB, SLAB).transpose(1, 0, 2)).reshape(-1)


def _from_slabs(flat, D, m):
    return flat.reshape(m // SLAB, D, SLAB).transpose(1, 0, 2).reshape(D, m)


def _fx_columns(D, m, F, seed):
    x = np.random.default_rng(seed).normal(size=(D, m))
    x /= np.linalg.norm(x, axis=0, keepdims=True)
    return np.rint(x * 2.0 ** F).astype(np.int64)


def _apply(pt, variant, isec, X, m):
    import torch
    cfg = pt.cfg.copy()
    cfg.hxv_variant = variant
    s = VcaSolver(cfg)
    s.set_hamiltonian(pt.Hloc)
    fx, F, G = s.arith_info()
    assert fx
    dX = torch.from_numpy(_to_slabs(X)).cuda()
    dY = torch.zeros_like(dX)
    s.hxv_timed(isec, dX.data_ptr(), dY.data_ptr(), 0, m, 1)
    torch.cuda.synchronize()
    Y = _from_slabs(dY.cpu().numpy(), X.shape[0], m)
    del s
    return Y, F, G


@pytest.mark.parametrize("m", [16, 40])
def test_staged_and_warp_forms_agree_and_match_oracle(m):
    pt = _point()
    Ns = 9
    nup, ndw = 5, 4
    isec = 1 + ndw + nup * (Ns + 1)
    probe = VcaSolver(pt.cfg)
    probe.set_hamiltonian(pt.Hloc)
    _, _, du, dd = probe.sector_info(isec)
    fx, F, G = probe.arith_info()
    del probe
    assert fx and du == 126 and dd == 126
    D = du * dd
    X = _fx_columns(D, m, F, seed=100 + m)
    Ys, F1, G1 = _apply(pt, 0, isec, X, m)
    Yw, F2, G2 = _apply(pt, 1, isec, X, m)
    assert (F1, G1) == (F2, G2) == (F, G)
    assert np.abs(Ys - Yw).max() <= 1
    o = Oracle.from_point(pt)
    worst = 0.0
    for c in range(m):
        ref = o.hxv(isec, X[:, c].astype(np.float64) * 2.0 ** -F).real
        for Y in (Ys, Yw):
            got = Y[:, c].astype(np.float64) * 2.0 ** -G
            worst = max(worst, np.abs(got - ref).max() / max(1.0, np.abs(ref).max()))
    assert worst < 1e-13, worst


def test_column_count_not_multiple_of_slab_rejected():
    import torch
    from vca_gb300.solver import VcaError
    pt = _point()
    s = VcaSolver(pt.cfg)
    s.set_hamiltonian(pt.Hloc)
    isec = 1 + 4 + 5 * 10
    _, _, du, dd = s.sector_info(isec)
    d = torch.zeros(du * dd * 24, dtype=torch.int64, device="cuda")
    with pytest.raises(VcaError):
        s.hxv_timed(isec, d.data_ptr(), d.data_ptr(), 0, 20, 1)


@pytest.mark.parametrize("m", [16, 40])
def test_position_ordered_form_matches_staged_form(m):
    """hxv_variant 2 (rows of the up role in hop-count order, the chains'
    layout) gives the staged form's output bit for bit, row-permuted: both
    round the same exact int128 sum once."""
    pt = _point()
    isec = 1 + 4 + 5 * 10
    probe = VcaSolver(pt.cfg)
    probe.set_hamiltonian(pt.Hloc)
    _, _, du, dd = probe.sector_info(isec)
    fx, F, G = probe.arith_info()
    order = probe.sector_row_order(isec)
    del probe
    D = du * dd
    assert sorted(order.tolist()) == list(range(D))
    X = _fx_columns(D, m, F, seed=300 + m)
    Ys, _, _ = _apply(pt, 0, isec, X, m)
    Yr, _, _ = _apply(pt, 2, isec, X[order], m)
    np.testing.assert_array_equal(Yr, Ys[order])


def test_single_vector_large_sector_matches_oracle():
    """One vector of a large sector (2x7 cluster, sector (7,7), D = 11.8M:
    the two-kernel staged single-vector form with two L2 row chunks) against
    the oracle's FP64 H x v of the same fixed-point input (the form rounds
    its up and down halves separately: 1e-13 of the vector scale)."""
    import torch
    pt = clusters.square(nx=7, ny=2, U=8.0, xmu=4.0, maf=0.0, nspin=1, nkx=2, nky=2, ngfiter=10,
                         omega_nodes=16)
    s = VcaSolver(pt.cfg)
    s.set_hamiltonian(pt.Hloc)
    isec = 1 + 7 + 7 * 15
    _, _, du, dd = s.sector_info(isec)
    assert du == dd == 3432
    fx, F, G = s.arith_info()
    assert fx
    D = du * dd
    x = np.random.default_rng(5).normal(size=D)
    x /= np.linalg.norm(x)
    X = np.rint(x * 2.0 ** F).astype(np.int64)
    dX = torch.from_numpy(X).cuda()
    dY = torch.zeros_like(dX)
    s.hxv_timed(isec, dX.data_ptr(), dY.data_ptr(), 0, 1, 1)
    torch.cuda.synchronize()
    got = dY.cpu().numpy().astype(np.float64) * 2.0 ** -G
    o = Oracle.from_point(pt)
    ref = o.hxv(isec, X.astype(np.float64) * 2.0 ** -F).real
    assert np.abs(got - ref).max() / max(1.0, np.abs(ref).max()) < 1e-13


def test_hop_pairing_changes_no_result():
    """The position-ordered kernel with its up hops re-ordered for bank
    pairing (the default) and in the plain sign-sorted order: the same
    exact sums, so the same output bit for bit."""
    import torch
    pt = _point()
    isec = 1 + 4 + 5 * 10
    m = 40
    out = []
    for on in (True, False):
        cfg = pt.cfg.copy()
        cfg.hxv_variant = 2
        s = VcaSolver(cfg)
        s.set_hop_pairing(on)
        s.set_hamiltonian(pt.Hloc)
        _, _, du, dd = s.sector_info(isec)
        fx, F, G = s.arith_info()
        D = du * dd
        X = _fx_columns(D, m, F, seed=77)
        order = s.sector_row_order(isec)
        dX = torch.from_numpy(_to_slabs(X[order])).cuda()
        dY = torch.zeros_like(dX)
        s.hxv_timed(isec, dX.data_ptr(), dY.data_ptr(), 0, m, 1)
        torch.cuda.synchronize()
        out.append(dY.cpu().numpy())
        s.close()
    np.testing.assert_array_equal(out[0], out[1])
