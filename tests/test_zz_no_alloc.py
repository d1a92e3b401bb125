"""kdq_grover_det_noalloc, the allocation-free Grover determinant.

It serves callers that cannot call cudaMalloc (work recorded into CUDA
graphs, loops that must not stall on the device synchronisation cudaMalloc
can cause, processes whose device memory is held by another allocator): the
caller hands over device buffers and the library takes its scratch from a
fixed device array.  Checked through the C ABI against the allocating entry
point kdq_grover_det and against the oracle's determinant of the Grover
matrix (numpy, independent of the CUDA kernel both entry points share), on
two calls in a row (the second sees the first call's leftovers in the
shared scratch).  This file is collected last so a failure here cannot hide
the other tests' results.
"""
import ctypes

import numpy as np
import pytest

import dqmc_oracle as O
from kapdqmc_gb300 import _lib
from kapdqmc_gb300.sweep import grover_det

pytestmark = pytest.mark.gpu

RTOL = 1e-10          # as the other Grover-determinant tests


def _pure_states(rng, Ns, n, cplx):
    out = []
    for _ in range(n):
        A = rng.normal(size=(Ns, Ns // 2)) + (1j * rng.normal(size=(Ns, Ns // 2)) if cplx else 0)
        Q = np.linalg.qr(A)[0]
        out.append(np.eye(Ns) - Q @ Q.conj().T)
    return np.array(out)


def _device_call(torch, lib, G1, G2, index, cplx):
    npairs, Ns = G1.shape[0], G1.shape[1]
    mats = []
    for a, b in zip(G1, G2):
        for m in (a, b):
            flat = np.ravel(m, order="F")
            mats.append(flat.astype(np.complex128).view(np.float64) if cplx else flat.real.astype(np.float64))
    dG = torch.from_numpy(np.concatenate(mats)).cuda()
    didx = torch.tensor(index, dtype=torch.int32).cuda()
    ddet = torch.full((2 * npairs,), -7.0, dtype=torch.float64).cuda()
    torch.cuda.synchronize()
    rc = lib.kdq_grover_det_noalloc(ctypes.c_void_p(dG.data_ptr()), Ns, int(cplx), npairs,
                                    ctypes.c_void_p(didx.data_ptr()), len(index),
                                    ctypes.c_void_p(ddet.data_ptr()), None)
    assert rc == _lib.KDQ_OK, lib.kdq_last_error(None)
    torch.cuda.synchronize()
    return ddet.cpu().numpy().view(np.complex128)


def test_noalloc_grover_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    rng = np.random.default_rng(17)
    cases = [(64, 6, list(range(1, 33)), True),          # 8x8 lattice, left half, complex
             (36, 9, [2, 3, 5, 7, 11, 13, 17, 19, 23], False)]
    for Ns, npairs, index, cplx in cases:
        G = _pure_states(rng, Ns, 2 * npairs, cplx)
        G1, G2 = G[0::2], G[1::2]
        want = grover_det(G1, G2, index)                  # allocating entry point
        oracle = np.array([O.grover_det(a, b, index) for a, b in zip(G1, G2)])
        np.testing.assert_allclose(want, oracle, rtol=RTOL, atol=1e-14)
        for _ in range(2):                                # the second call reuses the scratch
            got = _device_call(torch, lib, G1, G2, index, cplx)
            np.testing.assert_allclose(got, want, rtol=RTOL, atol=1e-14)
            np.testing.assert_allclose(got, oracle, rtol=RTOL, atol=1e-14)


def test_noalloc_rejects_requests_beyond_the_fixed_scratch():
    """A request beyond the fixed scratch is refused before any launch.  The
    buffers are real device allocations of the request's own size, so even a
    regression of the size check would read valid memory, not fault."""
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    Ns = nA = 64
    npairs = 64        # 64 pairs x 3 x 64^2 complex = 12 MiB of scratch > 8 MiB
    dG = torch.zeros(2 * npairs * Ns * Ns * 2, dtype=torch.float64, device="cuda")
    didx = torch.arange(1, nA + 1, dtype=torch.int32, device="cuda")
    ddet = torch.full((2 * npairs,), -7.0, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = lib.kdq_grover_det_noalloc(ctypes.c_void_p(dG.data_ptr()), Ns, 1, npairs,
                                    ctypes.c_void_p(didx.data_ptr()), nA,
                                    ctypes.c_void_p(ddet.data_ptr()), None)
    assert rc == _lib.KDQ_ERR_ARG
    assert b"maximum" in lib.kdq_last_error(None)
    torch.cuda.synchronize()
    assert torch.all(ddet == -7.0)                       # nothing was launched
