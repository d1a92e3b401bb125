"""Self-learning Monte Carlo for the t-U sweep: the effective model.

The effective model is a periodic three-layer convolutional net over the
slice x site HS field whose summed output F(s) is fitted to the fermion part
2 log|det(P^H B(Theta,0) P)| of the log-weight (``Sweeper.log_det``).  Its
training and inference run in the library's own CUDA kernels
(``kdq_cnn_forward``, ``kdq_cnn_grad``, ``kdq_cnn_train``).  The reference has
no counterpart (its sweep makes local updates only, src/tU/phy_update.jl:
256-267).

Configurations are passed as uint8 arrays (n_cfg, Nt, Ns) with values 1..4,
i.e. a t-U field ``s`` of shape (Ns, Nt) transposed (``cnn_fields``).
"""
from __future__ import annotations

import numpy as np

from . import _lib

NPARAM = 3057
CH = 16


def cnn_fields(s):
    """(n, Ns, Nt) t-U fields (or one (Ns, Nt) field) as (n, Nt, Ns) CNN input."""
    s = np.asarray(s, dtype=np.uint8)
    if s.ndim == 2:
        s = s[None]
    return np.ascontiguousarray(np.transpose(s, (0, 2, 1)))


def init_params(seed: int = 0, zero_output: bool = False) -> np.ndarray:
    """Random initial parameters (float32, NPARAM): N(0, 1/6) for W1,
    N(0, 1/12) for W2 and W3, zero biases.  ``zero_output`` starts the last
    layer at zero, so that the untrained F is the constant the standardised
    target is centred on (the summed output otherwise starts with a spread
    of order sqrt(Nt Ns) times the target's)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAM, dtype=np.float32)
    p[0:576] = rng.normal(0, 1 / 6, 576)
    p[592:2896] = rng.normal(0, 1 / 12, 2304)
    if not zero_output:
        p[2912:3056] = rng.normal(0, 1 / 12, 144)
    return p


def _shape(fields):
    f = np.ascontiguousarray(np.asarray(fields, dtype=np.uint8))
    if f.ndim != 3:
        raise ValueError("fields must be (n_cfg, Nt, Ns)")
    if f.size and (f.min() < 1 or f.max() > 4):
        raise ValueError("field values must be in 1..4")
    return f, f.shape


def _params(p):
    p = np.ascontiguousarray(np.asarray(p, dtype=np.float32))
    if p.shape != (NPARAM,):
        raise ValueError(f"params must hold {NPARAM} floats")
    return p


def cnn_forward(fields, params, device: int = 0) -> np.ndarray:
    """F(s_b) for every configuration (float64, n_cfg)."""
    f, (n, Nt, Ns) = _shape(fields)
    p = _params(params)
    out = np.empty(n)
    _lib.check(_lib.load().kdq_cnn_forward(f.ctypes.data, n, Nt, Ns, p.ctypes.data, out.ctypes.data, device))
    return out


def cnn_grad(fields, dF, params, device: int = 0) -> np.ndarray:
    """Gradient of sum_b dF[b] F(s_b) with respect to the parameters (float32)."""
    f, (n, Nt, Ns) = _shape(fields)
    p = _params(params)
    d = np.ascontiguousarray(np.asarray(dF, dtype=np.float64))
    if d.shape != (n,):
        raise ValueError("dF must hold one value per configuration")
    g = np.empty(NPARAM, dtype=np.float32)
    _lib.check(_lib.load().kdq_cnn_grad(f.ctypes.data, d.ctypes.data, n, Nt, Ns, p.ctypes.data, g.ctypes.data,
                                        device))
    return g


def cnn_train(fields, target, params, epochs: int, batch: int = 64, lr: float = 1e-3, seed: int = 0,
              device: int = 0):
    """Fit F to ``target`` (mean squared error, Adam); returns (params, loss per epoch)."""
    f, (n, Nt, Ns) = _shape(fields)
    p = _params(params).copy()
    y = np.ascontiguousarray(np.asarray(target, dtype=np.float64))
    if y.shape != (n,):
        raise ValueError("target must hold one value per configuration")
    loss = np.zeros(max(epochs, 1))
    _lib.check(_lib.load().kdq_cnn_train(f.ctypes.data, y.ctypes.data, n, Nt, Ns, epochs, batch, lr, seed,
                                         p.ctypes.data, loss.ctypes.data, device))
    return p, loss[:epochs]


def fit_effective_model(fields, logdet, epochs: int = 20, batch: int = 64, lr: float = 2e-3, seed: int = 0,
                        params=None, device: int = 0):
    """Train the effective model on configurations and their log|det|.

    The target 2 log|det| is standardised (mean mu, deviation sd) for the fit
    and the scale is folded back into the last layer afterwards, so that the
    returned parameters give F(s) ~ 2 log|det(P^H B P)| directly.  F sums
    Nt Ns outputs, so one Adam step moves it by about lr Nt Ns: the step
    size is lr scaled by min(1, 400 / (Nt Ns)).  Returns (params, loss per
    epoch in standardised units, (mu, sd)).
    """
    f, (n, Nt, Ns) = _shape(fields)
    t = 2.0 * np.asarray(logdet, dtype=np.float64)
    mu, sd = float(t.mean()), float(t.std()) or 1.0
    p0 = init_params(seed, zero_output=True) if params is None else _params(params).copy()
    lr_eff = lr * min(1.0, 400.0 / (Nt * Ns))
    p, loss = cnn_train(f, (t - mu) / sd, p0, epochs, batch, lr_eff, seed, device)
    p = p.astype(np.float64)
    p[2912:3056] *= sd                       # W3
    p[3056] = p[3056] * sd + mu / (Nt * Ns)  # b3
    return p.astype(np.float32), loss, (mu, sd)
