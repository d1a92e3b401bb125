"""The effective model's CUDA kernels (through the C ABI) against the CPU
restatement: forward values, parameter gradients, one Adam step, and a fit
that lowers the loss.  FP32 accumulation with bf16 weights on the GPU, float64
with the same bf16-rounded weights in the oracle."""
import numpy as np
import pytest

import cnn_oracle as N
from kapdqmc_gb300 import slmc

pytestmark = pytest.mark.gpu


def _fields(B, Nt, Ns, seed):
    return np.random.default_rng(seed).integers(1, 5, size=(B, Nt, Ns)).astype(np.uint8)


@pytest.mark.parametrize("B,Nt,Ns", [(3, 20, 16), (2, 13, 162), (2, 200, 162), (1, 1, 3), (4, 7, 72)])
def test_forward_matches_oracle(B, Nt, Ns):
    f = _fields(B, Nt, Ns, Nt * Ns)
    p = slmc.init_params(1)
    p[3056] = 0.25
    got = slmc.cnn_forward(f, p)
    ref, _ = N.forward(f, p)
    scale = np.abs(ref).max() + Nt * Ns * 1e-3
    assert np.abs(got - ref).max() < 2e-5 * scale, (got, ref)


@pytest.mark.parametrize("B,Nt,Ns", [(3, 20, 16), (2, 13, 162), (5, 9, 72)])
def test_gradient_matches_oracle(B, Nt, Ns):
    f = _fields(B, Nt, Ns, 7 + Ns)
    p = slmc.init_params(2)
    dF = np.random.default_rng(3).normal(size=B)
    got = slmc.cnn_grad(f, dF, p).astype(np.float64)
    ref = N.grad(f, dF, p)
    err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert err < 1e-5, err
    assert np.abs(got - ref).max() < 1e-4 * np.abs(ref).max()


def test_one_adam_step_matches_oracle():
    f = _fields(8, 12, 16, 5)
    y = np.random.default_rng(6).normal(size=8)
    p0 = slmc.init_params(4)
    lr = 1e-3
    p1, loss = slmc.cnn_train(f, y, p0, epochs=1, batch=8, lr=lr, seed=0)
    F, _ = N.forward(f, p0)
    assert abs(loss[0] - np.mean((F - y) ** 2)) < 1e-5 * max(1.0, loss[0])
    g = N.grad(f, 2 * (F - y) / 8, p0)
    want, _, _ = N.adam_step(p0.astype(np.float64), 0.0, 0.0, g, 1, lr)
    # the first Adam step moves each parameter by lr * g / (|g| + eps): compare
    # where the gradient's sign is well determined, bound the rest by lr
    sure = np.abs(g) > 1e-3 * np.abs(g).max()
    assert np.abs(p1[sure] - want[sure]).max() < 1e-6
    assert np.abs(p1 - p0).max() <= lr * 1.001


def test_fit_lowers_loss_on_a_teacher_network():
    f = _fields(256, 16, 16, 9)
    teacher = slmc.init_params(11)
    y, _ = N.forward(f, teacher)
    p, loss = slmc.cnn_train(f, (y - y.mean()) / y.std(), slmc.init_params(12), epochs=40, batch=32,
                             lr=3e-3, seed=1)
    assert loss[-1] < 0.1 * loss[0], loss
