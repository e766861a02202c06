"""The Omega surrogate: a small network trained on the GPU on Omega values and
gradients that the solver itself produces, used to propose candidates for
the stationary-point search.

The reference searches with scalar minimisers around ``vca_solve``
(``brent`` in drivers/vca_hm_chain1d.f90:104-108, ``fmin_bfgs``/``fmin`` in
drivers/vca_bhz_2d.f90:244-305); here the network proposes, and every
accepted point is re-solved by the plain solver, which is both judge and
fallback.

``SurrogateNet`` drives the C-ABI ``vca_mlp_*`` entry points (CUDA kernels in
vca_gb300/csrc/vca_mlp.cu, tensor-core GEMMs in vca_umma.cu); it scales the
parameter box to [-1, 1]^n and the targets to unit spread before training.
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np


class MlpConfig(ctypes.Structure):
    """Mirror of ``vca_mlp_config`` (include/vca_gpu.h)."""
    _fields_ = [
        ("n_in", ctypes.c_int32),
        ("capacity", ctypes.c_int32),
        ("seed", ctypes.c_uint64),
        ("lr", ctypes.c_double),
        ("beta1", ctypes.c_double),
        ("beta2", ctypes.c_double),
        ("adam_eps", ctypes.c_double),
        ("grad_weight", ctypes.c_double),
        ("weight_decay", ctypes.c_double),
    ]


def _lib():
    from .solver import load
    return load()


def _check(rc):
    from .solver import check
    check(rc)


def _dp(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def mlp_defaults() -> MlpConfig:
    c = MlpConfig()
    _lib().vca_mlp_config_defaults(ctypes.byref(c))
    return c


class SurrogateNet:
    """Raw network on already-scaled inputs (the C-ABI's units)."""

    def __init__(self, n_in: int = 4, capacity: int = 4096, seed: int = 20261203, **kw):
        self.L = _lib()
        c = mlp_defaults()
        c.n_in, c.capacity, c.seed = n_in, capacity, seed
        for k, v in kw.items():
            setattr(c, k, v)
        self.cfg = c
        _check(self.L.vca_mlp_init(ctypes.byref(c)))
        self.n_in = n_in
        self.nparams = int(self.L.vca_mlp_param_count())

    def close(self):
        self.L.vca_mlp_finalize()

    def params(self) -> np.ndarray:
        out = np.zeros(self.nparams, dtype=np.float32)
        _check(self.L.vca_mlp_get_params(_fp(out), out.size))
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(self.L.vca_mlp_set_params(_fp(p), p.size))

    def set_data(self, x, y, dy=None):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.ascontiguousarray(y, dtype=np.float64)
        dy = None if dy is None else np.ascontiguousarray(dy, dtype=np.float64)
        _check(self.L.vca_mlp_set_data(len(y), _dp(x), _dp(y), _dp(dy)))

    def loss_grad(self):
        loss = ctypes.c_double()
        g = np.zeros(self.nparams, dtype=np.float32)
        _check(self.L.vca_mlp_loss_grad(ctypes.byref(loss), _fp(g), g.size))
        return loss.value, g

    def train(self, steps: int) -> float:
        loss = ctypes.c_double()
        _check(self.L.vca_mlp_train(int(steps), ctypes.byref(loss)))
        return loss.value

    def predict(self, x, grad: bool = True):
        x = np.ascontiguousarray(np.atleast_2d(x), dtype=np.float64)
        n = x.shape[0]
        f = np.zeros(n)
        df = np.zeros((n, self.n_in)) if grad else None
        _check(self.L.vca_mlp_predict(n, _dp(x), _dp(f), _dp(df)))
        return (f, df) if grad else f


def umma_gemm_check(A_bits: np.ndarray, B_bits: np.ndarray, C: Optional[np.ndarray] = None,
                    accumulate: bool = False) -> np.ndarray:
    """C[M][128] (+)= A B^T on the tensor cores; A, B as bf16 bit patterns."""
    A_bits = np.ascontiguousarray(A_bits, dtype=np.uint16)
    B_bits = np.ascontiguousarray(B_bits, dtype=np.uint16)
    M, K = A_bits.shape
    out = np.zeros((M, 128), dtype=np.float32) if C is None else np.ascontiguousarray(C, dtype=np.float32).copy()
    u16 = ctypes.POINTER(ctypes.c_uint16)
    _check(_lib().vca_umma_gemm_check(A_bits.ctypes.data_as(u16), B_bits.ctypes.data_as(u16), _fp(out), M, K,
                                      1 if accumulate else 0))
    return out
