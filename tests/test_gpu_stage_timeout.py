"""The bounded wait of the chains' column H x v (the position-ordered
kernel stages its own block with one cp.async.bulk copy and waits on an
mbarrier for at most one second): with the test hook the barrier expects
more bytes than are copied, so the wait runs out without any fault; the
call returns VCA_ERR_TIMEOUT, and after the hook is cleared the same call
on the same context gives the normal result."""
import numpy as np
import pytest

from vca_gb300 import clusters
from vca_gb300.solver import VcaSolver, VcaError

pytestmark = pytest.mark.gpu

SLAB = 8


def test_stage_copy_timeout_is_reported_and_the_context_recovers():
    import torch
    pt = clusters.square(nx=3, ny=3, U=8.0, xmu=4.0, maf=0.2, nspin=2, nkx=4, nky=4, ngfiter=40,
                         omega_nodes=64)
    cfg = pt.cfg.copy()
    cfg.hxv_variant = 2  # the position-ordered kernel
    s = VcaSolver(cfg)
    s.set_hamiltonian(pt.Hloc)
    isec = 1 + 4 + 5 * 10  # sector (4 up, 5 down): 126 x 126
    _, _, du, dd = s.sector_info(isec)
    fx, F, _ = s.arith_info()
    assert fx
    D, m = du * dd, 16
    x = np.random.default_rng(3).normal(size=(D, m))
    x /= np.linalg.norm(x, axis=0, keepdims=True)
    X = np.rint(x * 2.0 ** F).astype(np.int64)
    X = np.ascontiguousarray(X.reshape(D, m // SLAB, SLAB).transpose(1, 0, 2)).reshape(-1)
    dX = torch.from_numpy(X).cuda()
    dY = torch.zeros_like(dX)
    s.hxv_timed(isec, dX.data_ptr(), dY.data_ptr(), 0, m, 1)
    torch.cuda.synchronize()
    ref = dY.cpu().numpy().copy()
    s.set_stage_extra_tx(16)
    with pytest.raises(VcaError) as ei:
        s.hxv_timed(isec, dX.data_ptr(), dY.data_ptr(), 0, m, 1)
    assert ei.value.code == -5  # VCA_ERR_TIMEOUT
    s.set_stage_extra_tx(0)
    dY.zero_()
    s.hxv_timed(isec, dX.data_ptr(), dY.data_ptr(), 0, m, 1)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dY.cpu().numpy(), ref)
    s.close()
