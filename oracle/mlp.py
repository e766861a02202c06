"""CPU restatement of the Omega surrogate network -- test infrastructure only.

The surrogate (4 -> 128 -> 128 -> 128 -> 1, SiLU) has no counterpart in the
reference; this file is the checker of its GPU kernels (vca_gb300/csrc/
vca_mlp.cu): the forward pass, the forward-mode input tangents, the Sobolev
loss and its gradient with respect to every parameter, written out by hand
(no autograd) in float64.

With ``bf16=True`` the operands of the two 128 x 128 products are rounded
to bfloat16 (round to nearest even) at the points where the GPU rounds them:
W2 and W3, the activations and tangents entering each product, and the
back-propagated pre-activation gradients entering the backward products.
Everything else stays float64.  ``bf16=False`` is the exact-arithmetic
network the BF16 kernels approximate.

Parameter layout (flat, as vca_mlp_get_params): W1[128][n_in], b1[128],
W2[128][128], b2[128], W3[128][128], b3[128], w4[128], b4.
"""
from __future__ import annotations

import numpy as np

W = 128


def offsets(nin: int):
    o = {}
    k = 0
    for name, size in (("W1", W * nin), ("b1", W), ("W2", W * W), ("b2", W), ("W3", W * W), ("b3", W),
                       ("w4", W), ("b4", 1)):
        o[name] = (k, size)
        k += size
    return o, k


def unpack(p: np.ndarray, nin: int) -> dict:
    o, n = offsets(nin)
    assert p.size == n
    d = {k: np.asarray(p[a:a + s], dtype=np.float64) for k, (a, s) in o.items()}
    d["W1"] = d["W1"].reshape(W, nin)
    d["W2"] = d["W2"].reshape(W, W)
    d["W3"] = d["W3"].reshape(W, W)
    d["b4"] = float(d["b4"][0])
    return d


def pack(g: dict, nin: int) -> np.ndarray:
    o, n = offsets(nin)
    out = np.zeros(n)
    for k, (a, s) in o.items():
        out[a:a + s] = np.ravel(g[k])
    return out


def bf16_round(x: np.ndarray) -> np.ndarray:
    """Round to bfloat16 (nearest even) through float32, as __float2bfloat16_rn."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def silu3(z):
    sg = 1.0 / (1.0 + np.exp(-z))
    s = z * sg
    s1 = sg * (1.0 + z * (1.0 - sg))
    s2 = sg * (1.0 - sg) * (2.0 + z * (1.0 - 2.0 * sg))
    return s, s1, s2


def forward(p: np.ndarray, x: np.ndarray, bf16: bool = False, tangents: bool = True):
    """f[n] and, with tangents, df/dx [n][nin]; plus the intermediates."""
    nin = x.shape[1]
    P = unpack(p, nin)
    r = bf16_round if bf16 else (lambda a: a)
    W2, W3 = r(P["W2"]), r(P["W3"])
    z1 = x @ P["W1"].T + P["b1"]                       # [n][128]
    s, s1, s2 = silu3(z1)
    a1 = s
    zd1 = np.broadcast_to(P["W1"].T[:, None, :], (nin, x.shape[0], W))  # dz1/dx_d = W1[:, d]
    ad1 = s1[None] * zd1 if tangents else None
    z2 = r(a1) @ W2.T + P["b2"]
    zd2 = r(ad1) @ W2.T if tangents else None
    s, s1_2, s2_2 = silu3(z2)
    a2 = s
    ad2 = s1_2[None] * zd2 if tangents else None
    z3 = r(a2) @ W3.T + P["b3"]
    zd3 = r(ad2) @ W3.T if tangents else None
    s, s1_3, s2_3 = silu3(z3)
    a3 = s
    f = a3 @ P["w4"] + P["b4"]
    g = None
    if tangents:
        ad3 = s1_3[None] * zd3
        g = (ad3 @ P["w4"]).T                           # [n][nin]
    cache = dict(P=P, W2=W2, W3=W3, z1=z1, zd1=zd1, s1_1=silu3(z1)[1], s2_1=silu3(z1)[2], a1=a1, ad1=ad1,
                 z2=z2, zd2=zd2, s1_2=s1_2, s2_2=s2_2, a2=a2, ad2=ad2, z3=z3, zd3=zd3, s1_3=s1_3, s2_3=s2_3,
                 a3=a3)
    return f, g, cache


def loss_grad(p: np.ndarray, x: np.ndarray, y: np.ndarray, dy: np.ndarray, lam, bf16: bool = False):
    """Mean over samples of (f - y)^2 + lam_j |df/dx - dy|^2, and its gradient
    with respect to the flat parameters (reverse pass written out); lam is a
    scalar or one weight per sample."""
    n, nin = x.shape
    lam = np.broadcast_to(np.asarray(lam, dtype=np.float64), (n,))
    r = bf16_round if bf16 else (lambda a: a)
    f, g, c = forward(p, x, bf16=bf16)
    P = c["P"]
    res = f - y
    resd = g - dy
    loss = float(np.mean(res ** 2 + lam * np.sum(resd ** 2, axis=1)))
    e = 2.0 * res / n                                    # dL/df
    ed = (2.0 * lam[:, None] * resd / n).T               # dL/d(df/dx_d), [nin][n]
    # head: f = w4 . a3 + b4, g_d = w4 . (s'(z3) zd3_d)
    s3 = c["a3"]
    gw4 = e @ s3 + np.einsum("dn,dno->o", ed, c["s1_3"][None] * c["zd3"])
    gb4 = float(np.sum(e))
    w4 = P["w4"]
    gz3 = e[:, None] * w4[None] * c["s1_3"] + np.einsum("dn,dno->no", ed, w4[None, None] * c["zd3"]) * c["s2_3"]
    gzd3 = ed[:, :, None] * w4[None, None] * c["s1_3"][None]
    gb3 = gz3.sum(axis=0)
    GZ3, GZD3 = r(gz3), r(gzd3)
    gW3 = GZ3.T @ r(c["a2"]) + np.einsum("dno,dni->oi", GZD3, r(c["ad2"]))
    ga2 = GZ3 @ c["W3"]
    gad2 = GZD3 @ c["W3"]
    # layer 2 SiLU
    gz2 = ga2 * c["s1_2"] + np.sum(gad2 * c["zd2"], axis=0) * c["s2_2"]
    gzd2 = gad2 * c["s1_2"][None]
    gb2 = gz2.sum(axis=0)
    GZ2, GZD2 = r(gz2), r(gzd2)
    gW2 = GZ2.T @ r(c["a1"]) + np.einsum("dno,dni->oi", GZD2, r(c["ad1"]))
    ga1 = GZ2 @ c["W2"]
    gad1 = GZD2 @ c["W2"]
    # input layer SiLU; z1 = W1 x + b1, zd1_d = W1[:, d]
    gz1 = ga1 * c["s1_1"] + np.sum(gad1 * c["zd1"], axis=0) * c["s2_1"]
    gzd1 = gad1 * c["s1_1"][None]
    gb1 = gz1.sum(axis=0)
    gW1 = gz1.T @ x + gzd1.sum(axis=1).T
    grad = pack(dict(W1=gW1, b1=gb1, W2=gW2, b2=gb2, W3=gW3, b3=gb3, w4=gw4, b4=gb4), nin)
    return loss, grad


def init_params(nin: int, seed: int = 0, scale: float = 1.0) -> np.ndarray:
    """Glorot-uniform weights and small random biases (for tests)."""
    rng = np.random.default_rng(seed)
    P = {
        "W1": rng.uniform(-1, 1, (W, nin)) * np.sqrt(6.0 / (nin + W)) * scale,
        "b1": rng.normal(0, 0.1, W),
        "W2": rng.uniform(-1, 1, (W, W)) * np.sqrt(6.0 / (2 * W)) * scale,
        "b2": rng.normal(0, 0.1, W),
        "W3": rng.uniform(-1, 1, (W, W)) * np.sqrt(6.0 / (2 * W)) * scale,
        "b3": rng.normal(0, 0.1, W),
        "w4": rng.uniform(-1, 1, W) * np.sqrt(6.0 / (W + 1)) * scale,
        "b4": 0.05,
    }
    return pack(P, nin)
