"""The Omega surrogate: a small network trained on the GPU on Omega values and
gradients that the solver itself produces, used to propose candidates for
the stationary-point search.

The reference searches with scalar minimisers around ``vca_solve``
(``brent`` in drivers/vca_hm_chain1d.f90:104-108, ``fmin_bfgs``/``fmin`` in
drivers/vca_bhz_2d.f90:244-305); here the network proposes, and every
accepted point is re-solved by the plain solver, which both decides and
stands in.

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

    def set_data(self, x, y, dy=None, gw=None):
        """gw[j]: weight of sample j's gradient term (None: 1 for every sample)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.ascontiguousarray(y, dtype=np.float64)
        dy = None if dy is None else np.ascontiguousarray(dy, dtype=np.float64)
        gw = None if gw is None else np.ascontiguousarray(gw, dtype=np.float64)
        _check(self.L.vca_mlp_set_data(len(y), _dp(x), _dp(y), _dp(dy), _dp(gw)))

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


# ---------------------------------------------------------------------------
# Stationary-point searches of Omega over a box of variational parameters
# ---------------------------------------------------------------------------
class CountingSolver:
    """Wraps a plain solve p -> Omega and counts the calls (the cost the
    searches are compared on)."""

    def __init__(self, solve):
        self.solve = solve
        self.calls = 0
        self.log = []

    def __call__(self, p):
        self.calls += 1
        v = float(self.solve(np.asarray(p, dtype=np.float64)))
        self.log.append((np.array(p, dtype=np.float64), v))
        return v


def newton_fd_search(f, p0, lo, hi, h_frac=1e-3, tol=1e-7, maxit=25):
    """The plain search: Newton's method on grad Omega = 0 with the gradient
    and Hessian from central differences of plain solves (1 + 2d + 2d(d-1)
    calls per iteration).  It finds saddle points as well as minima, which
    the drivers' minimisers (brent, fmin_bfgs) do not.  Stops when the
    Newton step is below tol of the box half-width in every coordinate."""
    lo, hi = np.asarray(lo, float), np.asarray(hi, float)
    d = len(lo)
    hw = 0.5 * (hi - lo)
    h = h_frac * hw
    p = np.array(p0, dtype=np.float64)
    E = np.eye(d)
    it = 0
    for it in range(1, maxit + 1):
        f0 = f(p)
        fp = np.array([f(p + h[i] * E[i]) for i in range(d)])
        fm = np.array([f(p - h[i] * E[i]) for i in range(d)])
        g = (fp - fm) / (2 * h)
        H = np.diag((fp - 2 * f0 + fm) / h ** 2)
        for i in range(d):
            for j in range(i + 1, d):
                a = f(p + h[i] * E[i] + h[j] * E[j])
                b = f(p + h[i] * E[i] - h[j] * E[j])
                c = f(p - h[i] * E[i] + h[j] * E[j])
                e = f(p - h[i] * E[i] - h[j] * E[j])
                H[i, j] = H[j, i] = (a - b - c + e) / (4 * h[i] * h[j])
        step = -np.linalg.solve(H, g)
        s = np.max(np.abs(step) / hw)
        if s > 0.5:  # damp long steps
            step *= 0.5 / s
        p = np.clip(p + step, lo, hi)
        if np.max(np.abs(step) / hw) < tol:
            break
    return p, f(p), it


def coordinate_brent_search(f, p0, lo, hi, kinds, xtol=1e-5, tol=1e-5, maxcycles=30):
    """The drivers' tool applied per variable: Brent's method on one
    parameter at a time (brent, drivers/vca_hm_chain1d.f90:104-108),
    minimising Omega along the variables of kind "min" and maximising it
    along those of kind "max", cycled until no parameter moves by more than
    tol of its box half-width."""
    import scipy.optimize
    lo, hi = np.asarray(lo, float), np.asarray(hi, float)
    p = np.array(p0, dtype=np.float64)
    hw = 0.5 * (hi - lo)
    cyc = 0
    for cyc in range(1, maxcycles + 1):
        moved = 0.0
        for i, kind in enumerate(kinds):
            sg = 1.0 if kind == "min" else -1.0

            def g(t, i=i, sg=sg):
                q = p.copy()
                q[i] = t
                return sg * f(q)
            r = scipy.optimize.minimize_scalar(g, bounds=(lo[i], hi[i]), method="bounded",
                                               options={"xatol": xtol * hw[i]})
            moved = max(moved, abs(r.x - p[i]) / hw[i])
            p[i] = r.x
        if moved < tol:
            break
    return p, f(p), cyc


class BoxSurrogate:
    """The network on a box of variational parameters: inputs scaled to
    [-1, 1]^d, Omega shifted and scaled to unit spread by the first fit, and
    its gradients scaled alike."""

    def __init__(self, lo, hi, seed=20261203, capacity=1024, **net_kw):
        self.lo, self.hi = np.asarray(lo, float), np.asarray(hi, float)
        self.d = len(self.lo)
        self.net = SurrogateNet(n_in=self.d, capacity=capacity, seed=seed, **net_kw)
        self.mu = self.sd = None

    def close(self):
        self.net.close()

    def x(self, P):
        return 2.0 * (np.atleast_2d(P) - self.lo) / (self.hi - self.lo) - 1.0

    def p(self, X):
        return self.lo + 0.5 * (np.atleast_2d(X) + 1.0) * (self.hi - self.lo)

    def fit(self, P, Om, dOm=None, steps=3000):
        """dOm[j]: the gradient at P[j] in parameter units, or a row of NaN
        where none was measured (that sample's gradient term is off)."""
        Om = np.asarray(Om, float)
        if self.mu is None:
            self.mu, self.sd = float(np.mean(Om)), float(max(np.std(Om), 1e-12))
        dy = gw = None
        if dOm is not None:
            dOm = np.asarray(dOm, float)
            have = np.all(np.isfinite(dOm), axis=1)
            dy = np.where(have[:, None], np.nan_to_num(dOm) * 0.5 * (self.hi - self.lo) / self.sd, 0.0)
            gw = have.astype(float)
        self.net.set_data(self.x(P), (Om - self.mu) / self.sd, dy, gw)
        return self.net.train(steps)

    def predict(self, P):
        f, df = self.net.predict(self.x(P))
        return self.mu + self.sd * f, df * self.sd * 2.0 / (self.hi - self.lo)

    def hessian_x(self, x, h=0.02):
        """The network's Hessian in scaled inputs: central differences of its
        exact input gradient (tangent rows), 2d points in one prediction."""
        d = self.d
        pts = np.vstack([x] + [x + h * e for e in np.eye(d)] + [x - h * e for e in np.eye(d)])
        _, g = self.net.predict(pts)
        H = (g[1:1 + d] - g[1 + d:]).T / (2 * h)
        return g[0], 0.5 * (H + H.T)

    def stationary(self, p_start, iters=40):
        """Newton on the network's input gradient from p_start."""
        x = self.x(p_start)[0]
        for _ in range(iters):
            g, H = self.hessian_x(x)
            step = -np.linalg.lstsq(H, g, rcond=None)[0]
            s = np.max(np.abs(step))
            if s > 0.25:
                step *= 0.25 / s
            x = np.clip(x + step, -1.0, 1.0)
            if s < 1e-6:
                break
        return self.p(x)[0]


def surrogate_search(f, lo, hi, p0, n_design=6, h_frac=1e-3, rounds=8, steps=3000, omega_tol=1e-7,
                     seed=20261203, grad_weight=1.0, **net_kw):
    """Surrogate-guided stationary-point search.

    The network is fitted to a space-filling design of plain solves (p0 and a
    Latin hypercube of n_design points, values only).  Each round proposes
    the network's stationary point (Newton on the network from the last
    proposal), re-solves it by the plain path together with its gradient
    from d forward differences of plain solves, adds that value and gradient
    to the training set (the Sobolev term), and refits.  The plain solver
    decides: the search stops when the measured gradient g at a proposal,
    through the network's curvature H there, puts it within
    |1/2 g^T H^-1 g| < omega_tol of the stationary value.  Returns the last
    verified point, its plain Omega, and per round the surrogate's error."""
    lo, hi = np.asarray(lo, float), np.asarray(hi, float)
    d = len(lo)
    hw = 0.5 * (hi - lo)
    rng = np.random.default_rng(seed)
    u = (np.argsort(rng.random((n_design, d)), axis=0) + rng.random((n_design, d))) / n_design
    P = [np.asarray(p0, float)] + [lo + ui * (hi - lo) for ui in u]
    Om = [f(q) for q in P]
    G = [np.full(d, np.nan) for _ in P]
    S = BoxSurrogate(lo, hi, seed=seed, grad_weight=grad_weight, **net_kw)
    history = []
    cand, om_c = P[0], Om[0]
    try:
        for r in range(rounds):
            S.fit(np.array(P), np.array(Om), np.array(G), steps=steps)
            cand = S.stationary(cand)
            pred, pgrad = S.predict(cand[None])
            om_c = f(cand)  # every accepted point is re-solved by the plain path
            h = h_frac * hw
            g = np.array([(f(np.clip(cand + h[i] * np.eye(d)[i], lo, hi)) - om_c) / h[i] for i in range(d)])
            _, Hx = S.hessian_x(S.x(cand)[0])
            gx = g * hw  # gradient in the scaled inputs
            try:
                est = abs(0.5 * gx @ np.linalg.solve(Hx * S.sd, gx))
            except np.linalg.LinAlgError:
                est = np.inf
            history.append({"point": cand.tolist(), "omega": om_c, "surrogate": float(pred[0]),
                            "surrogate_error": abs(float(pred[0]) - om_c),
                            "gradient": g.tolist(), "omega_gap_estimate": float(est)})
            P.append(cand)
            Om.append(om_c)
            G.append(g)
            if est < omega_tol:
                break
    finally:
        S.close()
    return cand, om_c, history
