"""The effective model's CPU restatement (oracle/cnn_oracle.py): gradients
against central finite differences, the layer-3 summed-kernel identity the
CUDA kernels rely on, and bf16 rounding."""
import numpy as np

import cnn_oracle as N


def _fields(B, Nt, Ns, seed):
    return np.random.default_rng(seed).integers(1, 5, size=(B, Nt, Ns)).astype(np.uint8)


def test_gradient_matches_finite_differences():
    f = _fields(2, 5, 6, 1)
    p = N.init_params(3).astype(np.float64)
    p[N.NPARAM - 1] = 0.3
    dF = np.array([0.7, -1.3])
    g = N.grad(f, dF, p, round_bf16=False)
    rng = np.random.default_rng(0)
    for i in list(rng.choice(N.NPARAM, 40, replace=False)) + [N.NPARAM - 1, 576, 2896]:
        h = 1e-5
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        Fp, _ = N.forward(f, pp, round_bf16=False)
        Fm, _ = N.forward(f, pm, round_bf16=False)
        fd = float(dF @ (Fp - Fm)) / (2 * h)
        assert abs(fd - g[i]) < 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_layer3_sum_identity():
    # sum over a periodic domain of a linear 3x3 convolution = sum of its
    # input weighted by the kernel's tap sums (the CUDA kernels' layer 3)
    f = _fields(3, 7, 9, 2)
    p = N.init_params(5).astype(np.float64)
    F, (q, x, a1, a2) = N.forward(f, p, round_bf16=False)
    w3s = q["W3"][0].sum(axis=(1, 2))
    F2 = np.einsum("c,bctj->b", w3s, a2) + q["b3"][0] * 7 * 9
    np.testing.assert_allclose(F, F2, rtol=1e-12, atol=1e-12)


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 1e-3], dtype=np.float32)
    r = N.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == -2.5
    assert abs(r[4] - 1e-3) < 1e-3 * 2 ** -8
