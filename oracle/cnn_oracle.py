"""CPU restatement of the self-learning effective model (float64 numpy).

TEST INFRASTRUCTURE ONLY: the checker of the CUDA training and inference
kernels; the product never calls it.

The model has no counterpart in the reference (whose sweep makes local
updates only, src/tU/phy_update.jl:256-267): a periodic three-layer
convolutional net over the slice x site HS field,

    x[c][t][j]  = [s(t, j) == c + 1]                       (4 one-hot channels)
    a1[o][t][j] = tanh(b1[o] + sum_{c,dy,dx} W1[o,c,dy,dx] x[c][t+dy-1][j+dx-1])
    a2[o][t][j] = tanh(b2[o] + sum_{c,dy,dx} W2[o,c,dy,dx] a1[c][t+dy-1][j+dx-1])
    y[t][j]     = b3 + sum_{c,dy,dx} W3[0,c,dy,dx] a2[c][t+dy-1][j+dx-1]
    F(s)        = sum_{t,j} y[t][j]

with indices periodic in t (mod Nt) and j (mod Ns), fitted to
2 log|det(P^H B(Theta,0) P)|.  Written from the definition with np.roll
(layer 3 is evaluated as a full convolution here, not through the
summed-kernel identity the CUDA kernels use).
"""
from __future__ import annotations

import numpy as np

CH = 16
SHAPES = [("W1", (CH, 4, 3, 3)), ("b1", (CH,)), ("W2", (CH, CH, 3, 3)), ("b2", (CH,)),
          ("W3", (1, CH, 3, 3)), ("b3", (1,))]
NPARAM = sum(int(np.prod(s)) for _, s in SHAPES)


def bf16(p):
    """Round float32 values to bfloat16 (round to nearest even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(p, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    out, o = {}, 0
    for name, shp in SHAPES:
        n = int(np.prod(shp))
        out[name] = np.asarray(p[o:o + n], dtype=np.float64).reshape(shp)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SHAPES])


def init_params(seed: int = 0):
    """He-style random initial weights (float32)."""
    rng = np.random.default_rng(seed)
    d = {"W1": rng.normal(0, 1 / 6, (CH, 4, 3, 3)), "b1": np.zeros(CH),
         "W2": rng.normal(0, 1 / 12, (CH, CH, 3, 3)), "b2": np.zeros(CH),
         "W3": rng.normal(0, 1 / 12, (1, CH, 3, 3)), "b3": np.zeros(1)}
    return pack(d).astype(np.float32)


def _shift(a, dy, dx):
    """a[..., t + dy - 1, j + dx - 1] (periodic)."""
    return np.roll(a, shift=(1 - dy, 1 - dx), axis=(-2, -1))


def _conv(W, b, a):
    """out[o] = b[o] + sum_{c,dy,dx} W[o,c,dy,dx] a[c][t+dy-1][j+dx-1]; a: (B, C, Nt, Ns)."""
    out = np.zeros((a.shape[0], W.shape[0]) + a.shape[2:])
    for dy in range(3):
        for dx in range(3):
            out += np.einsum("oc,bctj->botj", W[:, :, dy, dx], _shift(a, dy, dx))
    return out + b[None, :, None, None]


def _conv_T(W, d):
    """Adjoint of _conv in its input: da[c][t][j] = sum W[o,c,dy,dx] d[o][t-dy+1][j-dx+1]."""
    out = np.zeros((d.shape[0], W.shape[1]) + d.shape[2:])
    for dy in range(3):
        for dx in range(3):
            out += np.einsum("oc,botj->bctj", W[:, :, dy, dx], _shift(d, 2 - dy, 2 - dx))
    return out


def _wgrad(d, a):
    """dW[o,c,dy,dx] = sum_{b,t,j} d[b,o,t,j] a[b,c,t+dy-1,j+dx-1]."""
    g = np.zeros((d.shape[1], a.shape[1], 3, 3))
    for dy in range(3):
        for dx in range(3):
            g[:, :, dy, dx] = np.einsum("botj,bctj->oc", d, _shift(a, dy, dx))
    return g


def onehot(fields):
    f = np.asarray(fields).astype(np.int64) - 1
    return (f[:, None, :, :] == np.arange(4)[None, :, None, None]).astype(np.float64)


def forward(fields, params, round_bf16=True):
    """F(s_b) for fields (B, Nt, Ns) with values 1..4; returns (F, cache)."""
    p = unpack(bf16(params) if round_bf16 else np.asarray(params, dtype=np.float64))
    x = onehot(fields)
    a1 = np.tanh(_conv(p["W1"], p["b1"], x))
    a2 = np.tanh(_conv(p["W2"], p["b2"], a1))
    y = _conv(p["W3"], p["b3"], a2)
    return y.sum(axis=(1, 2, 3)), (p, x, a1, a2)


def grad(fields, dF, params, round_bf16=True):
    """Gradient of sum_b dF[b] F(s_b) with respect to the parameters (flat)."""
    _, (p, x, a1, a2) = forward(fields, params, round_bf16)
    B = x.shape[0]
    dy = np.broadcast_to(np.asarray(dF, dtype=np.float64)[:, None, None, None], (B, 1) + x.shape[2:])
    g = {"W3": _wgrad(dy, a2), "b3": np.array([dy.sum()])}
    dz2 = _conv_T(p["W3"], dy) * (1 - a2 ** 2)
    g["W2"] = _wgrad(dz2, a1)
    g["b2"] = dz2.sum(axis=(0, 2, 3))
    dz1 = _conv_T(p["W2"], dz2) * (1 - a1 ** 2)
    g["W1"] = _wgrad(dz1, x)
    g["b1"] = dz1.sum(axis=(0, 2, 3))
    return pack(g)


def adam_step(p, m, v, g, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (Kingma & Ba 2015) with bias correction."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v
