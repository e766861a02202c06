"""The allocation-free column H x v (vca_gpu_hxv_alpha_noalloc) through the
C-ABI against the existing entry point (vca_gpu_hxv_timed, one repetition)
on the same columns, three calls in a row: Y must equal the existing entry
point's Y (same kernels), and alpha[c] must equal <x_c, y_c> of the existing
entry point's output -- exactly summed in the fixed-point path (1e-14
relative after the conversion to double), 1e-13 relative in FP64.

Collected last on purpose: it must pass alone in a fresh process and after
every other test (its scratch address is looked up on the first call).
"""
import numpy as np
import pytest

from vca_gb300 import clusters
from vca_gb300.solver import VcaSolver, VcaError

pytestmark = pytest.mark.gpu

SLAB = 8
NS = 9
ISEC = 1 + 4 + 5 * (NS + 1)  # sector (5 up, 4 down) of the 3x3 cluster: 126 x 126


def _solver(arith, variant=0):
    pt = clusters.square(nx=3, ny=3, U=8.0, xmu=4.0, maf=0.2, nspin=2, nkx=4, nky=4, ngfiter=40,
                         omega_nodes=64)
    cfg = pt.cfg.copy()
    cfg.arith = arith
    cfg.hxv_variant = variant
    s = VcaSolver(cfg)
    s.set_hamiltonian(pt.Hloc)
    return s


def _columns(s, m, seed):
    _, _, du, dd = s.sector_info(ISEC)
    D = du * dd
    x = np.random.default_rng(seed).normal(size=(D, m))
    x /= np.linalg.norm(x, axis=0, keepdims=True)
    fx, F, G = s.arith_info()
    if fx:  # int64 fixed point, slab-major (slabs of 8 columns) once m >= 8
        X = np.rint(x * 2.0 ** F).astype(np.int64)
        if m >= SLAB:
            X = np.ascontiguousarray(X.reshape(D, m // SLAB, SLAB).transpose(1, 0, 2))
        return X.reshape(-1), D
    return np.ascontiguousarray(x).reshape(-1), D


def _rows(flat, D, m, fx):
    if fx and m >= SLAB:
        return flat.reshape(m // SLAB, D, SLAB).transpose(1, 0, 2).reshape(D, m)
    return flat.reshape(D, m)


@pytest.mark.parametrize("arith,m,variant", [(2, 8, 0), (2, 40, 0), (2, 40, 1), (2, 40, 2),
                                             (1, 8, 0), (1, 40, 0)],
                         ids=["fx-m8", "fx-m40", "fx-m40-warp", "fx-m40-rowperm", "fp64-m8", "fp64-m40"])
def test_noalloc_matches_existing_entry_point(arith, m, variant):
    """hxv_variant 1 (warp kernel) and 2 (row-permuted kernel) size and fill
    the partial-sum rows differently from the default staged kernel, so each
    is compared with the existing entry point.  Free device memory and
    torch's allocated bytes are recorded after a first call and must be
    unchanged by the next ones: the entry point allocates nothing."""
    import torch
    s = _solver(arith, variant)
    fx, F, G = s.arith_info()
    assert fx == (arith == 2)
    flat, D = _columns(s, m, seed=17 + m)
    dX = torch.from_numpy(flat).cuda()
    dYref = torch.zeros_like(dX)
    s.hxv_timed(ISEC, dX.data_ptr(), dYref.data_ptr(), 0, m, 1)
    s.synchronize()
    Yref = dYref.cpu().numpy()
    X = _rows(flat, D, m, fx)
    Yr = _rows(Yref, D, m, fx)
    if fx:
        exact = (X.astype(object) * Yr.astype(object)).sum(axis=0)
        aref = np.array([float(v) for v in exact]) * 2.0 ** -(F + G)
        rtol = 1e-14
    else:
        aref = (X * Yr).sum(axis=0)
        rtol = 1e-13
    dY = torch.full_like(dX, 7)
    dA = torch.full((m,), np.nan, dtype=torch.float64, device="cuda")
    mem = None
    for call in range(3):
        dY.fill_(7)
        dA.fill_(float("nan"))
        torch.cuda.synchronize()
        if call == 1:  # after the first call has looked up the scratch address
            mem = (torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated())
        s.hxv_alpha_noalloc(ISEC, dX.data_ptr(), dY.data_ptr(), m, dA.data_ptr())
        s.synchronize()
        if call >= 1:
            assert (torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated()) == mem
        np.testing.assert_array_equal(dY.cpu().numpy(), Yref)
        np.testing.assert_allclose(dA.cpu().numpy(), aref, rtol=rtol, atol=0.0)


def test_noalloc_rejects_batches_beyond_the_static_scratch():
    import torch
    s = _solver(2)
    # 126 partial rows x 4168 columns x 16 bytes > 8 MiB: rejected on the host
    # before any launch, so small buffers are never touched
    d = torch.zeros(64, dtype=torch.int64, device="cuda")
    a = torch.zeros(64, dtype=torch.float64, device="cuda")
    with pytest.raises(VcaError) as ei:
        s.hxv_alpha_noalloc(ISEC, d.data_ptr(), d.data_ptr(), 4168, a.data_ptr())
    assert ei.value.code == -9
    assert "static scratch" in str(ei.value)
