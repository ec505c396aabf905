"""CPU oracle of the surrogate MLP (test infrastructure only: tests/ and the checker in
__graft_entry__.smoke() use it to check the GPU network; nothing in the product imports it).

The reference engine has no surrogate, so this oracle is pinned by mathematics instead of
reference vectors: `numeric_gradients` (central differences in float64) checks
`loss_and_gradients` in exact arithmetic (emulate=False), and the same code with
emulate=True rounds to BF16 exactly where the GPU does:

    weights        BF16 copies of the FP32 master weights feed every product
    activations    H_{l+1} = bf16(gelu(H_l W_l^T + b_l)), H_0 = bf16(x)
    output         Y = H_{L-1} W^T + b (FP32, not rounded)
    loss gradient  dY = bf16(2 (Y - T) / (B * out_dim))
    backward       dW_l = dZ_l^T H_l, db_l = sum_b dZ_l, dZ_{l-1} = bf16((dZ_l W_l) * gelu'(Z_{l-1}))

Products accumulate in float64 here and in FP32 on the tensor cores; the tests state the
tolerance that difference needs.  GELU is the exact x * Phi(x).
"""
from __future__ import annotations

import math

import numpy as np

_erf = np.vectorize(math.erf, otypes=[np.float64])


def bf16(x) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    rounded = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return rounded.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + _erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def layer_shapes(in_dim: int, hidden: int, hidden_layers: int, out_dim: int) -> list[tuple[int, int]]:
    """(out, in) of every layer."""
    dims = [in_dim] + [hidden] * hidden_layers + [out_dim]
    return [(dims[i + 1], dims[i]) for i in range(len(dims) - 1)]


def unflatten(flat: np.ndarray, shapes) -> list[tuple[np.ndarray, np.ndarray]]:
    """epi_mlp_get_params layout: per layer W (out x in, row-major) then b (out)."""
    out, o = [], 0
    for n, k in shapes:
        w = np.asarray(flat[o:o + n * k], dtype=np.float64).reshape(n, k)
        o += n * k
        b = np.asarray(flat[o:o + n], dtype=np.float64)
        o += n
        out.append((w, b))
    return out


def flatten(layers) -> np.ndarray:
    return np.concatenate([np.concatenate([w.ravel(), b]) for w, b in layers])


def forward(layers, x, emulate: bool = True):
    """Outputs and the cache (inputs H_l, pre-activations Z_l) of every layer."""
    r = bf16 if emulate else (lambda a: np.asarray(a, dtype=np.float64))
    h = r(x)
    hs, zs = [], []
    for i, (w, b) in enumerate(layers):
        hs.append(h)
        z = h @ r(w).T + np.asarray(b, dtype=np.float64)
        zs.append(z)
        if i + 1 < len(layers):
            h = r(gelu(z))
    return zs[-1], (hs, zs)


def loss_and_gradients(layers, x, t, emulate: bool = True):
    """Mean squared error over every output and its gradients (same structure as layers)."""
    r = bf16 if emulate else (lambda a: np.asarray(a, dtype=np.float64))
    y, (hs, zs) = forward(layers, x, emulate)
    B, out_dim = y.shape
    diff = y - np.asarray(t, dtype=np.float64)
    loss = float(np.mean(diff * diff))
    dz = r(2.0 * diff / (B * out_dim))
    grads = [None] * len(layers)
    for l in range(len(layers) - 1, -1, -1):
        w, _ = layers[l]
        grads[l] = (dz.T @ hs[l], dz.sum(axis=0))
        if l > 0:
            dz = r((dz @ r(w)) * gelu_grad(zs[l - 1]))
    return loss, grads


def numeric_gradients(layers, x, t, picks, eps: float = 1e-6):
    """Central differences of the exact loss at the (layer, 'w'|'b', index) picks."""
    out = []
    for l, kind, idx in picks:
        vals = []
        for sgn in (1.0, -1.0):
            pert = [(w.copy(), b.copy()) for w, b in layers]
            a = pert[l][0] if kind == "w" else pert[l][1]
            a[idx] += sgn * eps
            vals.append(loss_and_gradients(pert, x, t, emulate=False)[0])
        out.append((vals[0] - vals[1]) / (2.0 * eps))
    return np.array(out)


def adam_step(p, g, m, v, t: int, lr: float, beta1: float, beta2: float, eps: float):
    """Adam (Kingma & Ba 2015) with bias correction; returns new (p, m, v)."""
    m = beta1 * m + (1.0 - beta1) * g
    v = beta2 * v + (1.0 - beta2) * g * g
    mhat = m / (1.0 - beta1 ** t)
    vhat = v / (1.0 - beta2 ** t)
    return p - lr * mhat / (np.sqrt(vhat) + eps), m, v
