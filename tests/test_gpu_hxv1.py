"""Single-vector fixed-point H x v of large sectors (D >= 2^22): the
paired-column form (two columns per CTA interleaved in shared memory, hops
walked in a bank schedule, row-pair down streams) against the one-column
form (hxv_variant 1) and the oracle.

Both forms sum the same hops exactly in int64 and round the same int128 once
per half, so they agree bit for bit whatever order the schedule puts a row's
hops in.  The cases cover one and two hopping magnitudes, an odd DimDw (the
last CTA holds one column) and an odd DimUp (the down part keeps one row per
thread).
"""
import dataclasses

import numpy as np
import pytest

from vca_gb300 import clusters
from vca_gb300.solver import VcaSolver
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

NX, NY = 7, 2
NS = NX * NY


def _point(ty):
    pt = clusters.square(nx=NX, ny=NY, U=8.0, xmu=4.0, maf=0.3, nspin=2, nkx=2, nky=2, ngfiter=10,
                         omega_nodes=16)
    if ty == 1.0:
        return pt
    H = pt.Hloc.copy()
    for x in range(NX):  # vertical bonds (x,0)-(x,1) at a second magnitude
        i, j = x, NX + x
        for s in range(2):
            H[i, j, s, s, 0, 0] = -ty
            H[j, i, s, s, 0, 0] = -ty
    return dataclasses.replace(pt, Hloc=H)


def _hxv(pt, variant, isec, X):
    import torch
    cfg = pt.cfg.copy()
    cfg.hxv_variant = variant
    s = VcaSolver(cfg)
    s.set_hamiltonian(pt.Hloc)
    fx, F, G = s.arith_info()
    assert fx
    dX = torch.from_numpy(X).cuda()
    dY = torch.zeros_like(dX)
    s.hxv_timed(isec, dX.data_ptr(), dY.data_ptr(), 0, 1, 2)
    torch.cuda.synchronize()
    Y = dY.cpu().numpy()
    del s
    return Y, F, G


@pytest.mark.parametrize("ty,nup,ndw,oracle_check", [
    (1.0, 7, 7, False),   # one magnitude, DimUp = DimDw = 3432
    (0.7, 7, 6, True),    # two magnitudes, DimDw = 3003 odd
    (0.7, 6, 7, False),   # two magnitudes, DimUp = 3003 odd
])
def test_paired_column_form_matches_one_column_form(ty, nup, ndw, oracle_check):
    pt = _point(ty)
    isec = 1 + nup + ndw * (NS + 1)
    probe = VcaSolver(pt.cfg)
    probe.set_hamiltonian(pt.Hloc)
    _, _, du, dd = probe.sector_info(isec)
    fx, F, G = probe.arith_info()
    del probe
    D = du * dd
    assert D >= 1 << 22
    x = np.random.default_rng(17 + nup + 3 * ndw).normal(size=D)
    x /= np.linalg.norm(x)
    X = np.rint(x * 2.0 ** F).astype(np.int64)
    Yp, _, _ = _hxv(pt, 0, isec, X)
    Y1, _, _ = _hxv(pt, 1, isec, X)
    np.testing.assert_array_equal(Yp, Y1)
    if oracle_check:
        o = Oracle.from_point(pt)
        ref = o.hxv(isec, X.astype(np.float64) * 2.0 ** -F).real
        got = Yp.astype(np.float64) * 2.0 ** -G
        assert np.abs(got - ref).max() / max(1.0, np.abs(ref).max()) < 1e-13


def _slabs(X):
    D, m = X.shape
    return np.ascontiguousarray(X.reshape(D, m // 8, 8).transpose(1, 0, 2)).reshape(-1)


@pytest.mark.parametrize("ty,nup,ndw,m", [(1.0, 7, 7, 16), (0.7, 7, 6, 24)])
def test_slab_pair_form_matches_warp_form(ty, nup, ndw, m):
    """Column batches of a sector whose up block of one slab does not fit
    shared memory (2x7 cluster, DimUp 3432): the slab-pair form (16-byte
    column pairs through the bank schedule, chunked down streams, separate
    exact alpha partials) against the warp form (hxv_variant 1), Y and
    alpha = <x, Hx> bit for bit."""
    import torch
    pt = _point(ty)
    isec = 1 + nup + ndw * (NS + 1)
    out = {}
    for variant in (0, 1):
        cfg = pt.cfg.copy()
        cfg.hxv_variant = variant
        s = VcaSolver(cfg)
        s.set_hamiltonian(pt.Hloc)
        _, _, du, dd = s.sector_info(isec)
        fx, F, G = s.arith_info()
        assert fx
        D = du * dd
        x = np.random.default_rng(40 + m).normal(size=(D, m))
        x /= np.linalg.norm(x, axis=0, keepdims=True)
        dX = torch.from_numpy(_slabs(np.rint(x * 2.0 ** F).astype(np.int64))).cuda()
        dY = torch.zeros_like(dX)
        dA = torch.zeros(m, dtype=torch.float64, device="cuda")
        s.hxv_alpha_noalloc(isec, dX.data_ptr(), dY.data_ptr(), m, dA.data_ptr())
        torch.cuda.synchronize()
        out[variant] = (dY.cpu().numpy(), dA.cpu().numpy())
        del dX, dY, dA
        s.close()
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
