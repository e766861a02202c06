"""The surrogate network's GPU kernels against the CPU restatement.

* The tensor-core GEMM (tcgen05.mma, BF16 operands, FP32 accumulation)
  against numpy on the same BF16 values: one to sixteen K chunks, one to
  three row tiles, with and without accumulation into C.  Tolerance: the
  worst-case FP32 summation bound K * 2^-24 * sum_k |a_k b_k| per element
  (observed at K = 1024: about 2^-22 of that sum; a layout error gives
  errors of the order of the sum itself).
* Its bounded waits: a load barrier that is never completed makes the call
  return VCA_ERR_TIMEOUT, and the next GEMM on the same context is right.
* Loss and every parameter gradient of the Sobolev loss (values and input
  gradients) at given weights: against the restatement that rounds the
  GEMM operands to BF16 where the GPU does (1e-3 relative per parameter
  block) and against the float64 network (2e-2 relative per block, the
  BF16 operand error).
* Training: Adam on a smooth function with its gradient; the fitted values
  and input gradients at held-out points, and the GPU's input gradients
  against the restatement's tangents at the trained weights.
"""
import numpy as np
import pytest

from oracle import mlp

pytestmark = pytest.mark.gpu


def _bits(a):
    return (mlp.bf16_round(a).astype(np.float32).view(np.uint32) >> 16).astype(np.uint16)


@pytest.mark.parametrize("M,K", [(128, 64), (256, 128), (128, 1024), (384, 192)])
@pytest.mark.parametrize("acc", [False, True])
def test_umma_gemm_matches_numpy(M, K, acc):
    from vca_gb300.surrogate import umma_gemm_check
    rng = np.random.default_rng(M + K)
    A = mlp.bf16_round(rng.normal(size=(M, K)))
    B = mlp.bf16_round(rng.normal(size=(128, K)))
    C0 = rng.normal(size=(M, 128)).astype(np.float32) if acc else None
    got = umma_gemm_check(_bits(A), _bits(B), C0, accumulate=acc).astype(np.float64)
    ref = A @ B.T + (C0.astype(np.float64) if acc else 0.0)
    bound = (K + 1) * 2.0 ** -24 * (np.abs(A) @ np.abs(B).T + (np.abs(C0) if acc else 0.0)) + 1e-30
    assert np.all(np.abs(got - ref) <= bound), np.max(np.abs(got - ref) / bound)


def test_umma_bounded_wait_reports_timeout_and_context_survives():
    from vca_gb300.solver import VcaError, load
    from vca_gb300.surrogate import umma_gemm_check
    rc = load().vca_umma_timeout_check()
    assert rc == -5, rc
    with pytest.raises(VcaError):
        from vca_gb300.solver import check
        check(rc)
    rng = np.random.default_rng(1)
    A = mlp.bf16_round(rng.normal(size=(128, 64)))
    B = mlp.bf16_round(rng.normal(size=(128, 64)))
    got = umma_gemm_check(_bits(A), _bits(B)).astype(np.float64)
    assert np.abs(got - A @ B.T).max() < 1e-4


def _net(nin=4, **kw):
    from vca_gb300.surrogate import SurrogateNet
    return SurrogateNet(n_in=nin, capacity=512, **kw)


def _blocks(nin):
    o, _ = mlp.offsets(nin)
    return o


@pytest.mark.parametrize("S,lam,mixed", [(37, 0.7, False), (200, 1.0, False), (130, 0.0, False), (61, 1.3, True)])
def test_loss_and_gradients_match_oracle(S, lam, mixed):
    nin = 4
    rng = np.random.default_rng(S)
    x = rng.uniform(-1, 1, (S, nin))
    y = np.sin(x @ np.array([1.0, -0.5, 0.3, 0.8]))
    dy = np.cos(x)
    gw = np.where(rng.random(S) < 0.5, 0.0, rng.uniform(0.5, 2.0, S)) if mixed else None
    net = _net(nin, grad_weight=lam)
    p = mlp.init_params(nin, seed=S).astype(np.float32)
    net.set_params(p)
    net.set_data(x, y, dy, gw)
    if mixed:
        lam = lam * gw.astype(np.float32).astype(np.float64)
    loss, g = net.loss_grad()
    p64 = p.astype(np.float64)
    xs = x.astype(np.float32).astype(np.float64)  # the GPU holds x, y, dy in FP32
    ys = y.astype(np.float32).astype(np.float64)
    ds = dy.astype(np.float32).astype(np.float64)
    lb, gb = mlp.loss_grad(p64, xs, ys, ds, lam, bf16=True)
    l64, g64 = mlp.loss_grad(p64, xs, ys, ds, lam, bf16=False)
    assert abs(loss - lb) < 1e-4 * abs(lb), (loss, lb)
    assert abs(loss - l64) < 2e-2 * abs(l64), (loss, l64)
    for name, (a, s) in _blocks(nin).items():
        gg, rb, r64 = g[a:a + s].astype(np.float64), gb[a:a + s], g64[a:a + s]
        eb = np.linalg.norm(gg - rb) / np.linalg.norm(rb)
        e64 = np.linalg.norm(gg - r64) / np.linalg.norm(r64)
        assert eb < 1e-3, (name, eb)
        assert e64 < 2e-2, (name, e64)
    net.close()


def test_training_fits_values_and_gradients():
    nin = 3
    rng = np.random.default_rng(11)

    def fn(x):
        return 0.6 * x[:, 0] ** 2 - 0.4 * x[:, 1] ** 2 + 0.3 * x[:, 0] * x[:, 2] + 0.2 * np.sin(2 * x[:, 2])

    def dfn(x):
        return np.stack([1.2 * x[:, 0] + 0.3 * x[:, 2], -0.8 * x[:, 1], 0.3 * x[:, 0] + 0.4 * np.cos(2 * x[:, 2])],
                        axis=1)

    x = rng.uniform(-1, 1, (96, nin))
    net = _net(nin, grad_weight=1.0, lr=2e-3)
    net.set_data(x, fn(x), dfn(x))
    l0, _ = net.loss_grad()
    loss = net.train(3000)
    assert loss < 2e-3 * l0, (l0, loss)
    xt = rng.uniform(-0.8, 0.8, (64, nin))
    f, df = net.predict(xt)
    assert np.abs(f - fn(xt)).max() < 0.03
    assert np.abs(df - dfn(xt)).max() < 0.08
    # the GPU's input gradients are the restatement's tangents at the trained weights
    p = net.params().astype(np.float64)
    fr, gr, _ = mlp.forward(p, xt.astype(np.float32).astype(np.float64), bf16=True)
    np.testing.assert_allclose(f, fr, rtol=0, atol=2e-4 * max(1.0, np.abs(fr).max()))
    np.testing.assert_allclose(df, gr, rtol=0, atol=2e-4 * max(1.0, np.abs(gr).max()))
    net.close()
