"""ctypes driver of the C restatement of the t-V, t-U and t-UV sweeps
(oracle/cport/kdq_cpu.c).

TEST INFRASTRUCTURE ONLY: the timed CPU baseline and its parity tests.  The
BLAS/LAPACK it calls come from the OpenBLAS bundled with numpy.
"""
from __future__ import annotations

import ctypes as C
import glob
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "cport" / "kdq_cpu.c"
LIB = HERE / "cport" / "libkdq_cpu.so"
_lib = None


def build(force=False):
    if force or not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-o", str(LIB), str(SRC), "-ldl", "-lm"], check=True)
    return LIB


def openblas_path():
    import numpy
    pats = [os.path.join(os.path.dirname(numpy.__file__), "..", "numpy.libs", "*openblas64*"),
            os.path.join(os.path.dirname(numpy.__file__), ".libs", "*openblas64*")]
    for p in pats:
        hits = sorted(glob.glob(p))
        if hits:
            return os.path.realpath(hits[0])
    raise FileNotFoundError("no ILP64 OpenBLAS bundled with numpy")


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        if lib.kdq_cpu_load_blas(openblas_path().encode()) != 0:
            raise RuntimeError("BLAS/LAPACK symbols not found in numpy's OpenBLAS")
        lib.kdq_cpu_tv_phy_update.restype = C.c_int
        lib.kdq_cpu_tu_phy_update.restype = C.c_int
        lib.kdq_cpu_tuv_phy_update.restype = C.c_int
        _lib = lib
    return _lib


def _p(a):
    return C.c_void_p(a.ctypes.data)


def tv_phy_update(model, s, sweeps, k, u, record=True, log=False):
    """Run the C restatement; returns (s, obs rows, accept log or None)."""
    lib = load()
    s = np.asfortranarray(np.array(s, dtype=np.uint8))
    flat_s = np.ascontiguousarray(np.ravel(s, order="F"))
    f = lambda m: np.ascontiguousarray(np.ravel(np.asarray(m, dtype=np.float64), order="F"))
    mats = [f(model.eK), f(model.eKinv), f(model.HalfeK), f(model.HalfeKinv), f(model.K), f(model.Pt)]
    UV = f(model.UV)
    bonds = np.ascontiguousarray(np.asarray(model.nnidx).transpose(1, 0, 2).reshape(-1, 2), dtype=np.int32)
    nodes = np.ascontiguousarray(model.nodes, dtype=np.int64)
    alpha, gamma, eta = (np.ascontiguousarray(x, dtype=np.float64) for x in (model.α, model.γ, model.η))
    k = np.ascontiguousarray(k, dtype=np.uint8)
    u = np.ascontiguousarray(u, dtype=np.float64)
    obs = np.zeros(max(sweeps, 1) * 10)
    acc = np.zeros(len(k), dtype=np.uint8) if log else None
    hc = int("HoneyComb" in model.Lattice)
    rc = lib.kdq_cpu_tv_phy_update(
        C.c_int(model.Ns), C.c_int(model.Nt), C.c_int(model.z), C.c_int(len(nodes)), _p(nodes), _p(alpha),
        _p(gamma), _p(eta), *(_p(m) for m in mats[:5]), C.c_double(model.Ht), _p(mats[5]), _p(bonds), _p(UV),
        C.c_int(model.site[0]), C.c_int(model.site[1]), C.c_int(hc), _p(flat_s), C.c_int(sweeps),
        C.c_int(int(record)), _p(k), _p(u), C.c_size_t(len(k)), _p(obs), _p(acc) if log else None)
    if rc != 0:
        raise RuntimeError(f"kdq_cpu_tv_phy_update failed with {rc}")
    s_out = flat_s.reshape(model.field_shape, order="F")
    return s_out, obs.reshape(-1, 10)[:sweeps], acc


def tu_phy_update(model, s, sweeps, k, u, record=True, log=False):
    """Run the C restatement of the t-U sweep; returns (s, obs rows (sweeps, 6), accept log or None)."""
    lib = load()
    s = np.asfortranarray(np.array(s, dtype=np.uint8))
    flat_s = np.ascontiguousarray(np.ravel(s, order="F"))
    z = lambda m: np.ascontiguousarray(np.ravel(np.asarray(m, dtype=np.complex128), order="F")).view(np.float64)
    mats = [z(model.eK), z(model.eKinv), z(model.HalfeK), z(model.HalfeKinv), z(model.K), z(model.Pt)]
    nodes = np.ascontiguousarray(model.nodes, dtype=np.int64)
    alpha, gamma, eta = (np.ascontiguousarray(x, dtype=np.float64) for x in (model.α, model.γ, model.η))
    k = np.ascontiguousarray(k, dtype=np.uint8)
    u = np.ascontiguousarray(u, dtype=np.float64)
    obs = np.zeros(max(sweeps, 1) * 6)
    acc = np.zeros(len(k), dtype=np.uint8) if log else None
    hc = int("HoneyComb" in model.Lattice)
    rc = lib.kdq_cpu_tu_phy_update(
        C.c_int(model.Ns), C.c_int(model.Nt), C.c_int(len(nodes)), _p(nodes), _p(alpha), _p(gamma), _p(eta),
        *(_p(m) for m in mats[:5]), C.c_double(model.Ht), _p(mats[5]), C.c_int(model.site[0]),
        C.c_int(model.site[1]), C.c_int(hc), _p(flat_s), C.c_int(sweeps), C.c_int(int(record)), _p(k), _p(u),
        C.c_size_t(len(k)), _p(obs), _p(acc) if log else None)
    if rc != 0:
        raise RuntimeError(f"kdq_cpu_tu_phy_update failed with {rc}")
    s_out = flat_s.reshape(model.field_shape, order="F")
    return s_out, obs.reshape(-1, 6)[:sweeps], acc


def tuv_phy_update(model, s, sweeps, k, u, record=True, log=False):
    """Run the C restatement of the t-UV sweep (complex or, for U < 0, the
    real branch); returns (s, obs rows (sweeps, 7), accept log or None)."""
    lib = load()
    s = np.asfortranarray(np.array(s, dtype=np.uint8))
    flat_s = np.ascontiguousarray(np.ravel(s, order="F"))
    z = lambda m: np.ascontiguousarray(np.ravel(np.asarray(m, dtype=np.complex128), order="F")).view(np.float64)
    mats = [z(model.eK), z(model.eKinv), z(model.HalfeK), z(model.HalfeKinv), z(model.K), z(model.Pt)]
    nn = np.asarray(model.nnidx)
    bonds = np.ascontiguousarray(np.stack([nn[:, :, 0].ravel(order="F"), nn[:, :, 1].ravel(order="F")], axis=1),
                                 dtype=np.int32)
    nodes = np.ascontiguousarray(model.nodes, dtype=np.int64)
    gamma, eta = (np.ascontiguousarray(x, dtype=np.float64) for x in (model.γ, model.η))
    k = np.ascontiguousarray(k, dtype=np.uint8)
    u = np.ascontiguousarray(u, dtype=np.float64)
    obs = np.zeros(max(sweeps, 1) * 7)
    acc = np.zeros(len(k), dtype=np.uint8) if log else None
    hc = int("HoneyComb" in model.Lattice)
    rc = lib.kdq_cpu_tuv_phy_update(
        C.c_int(model.Ns), C.c_int(model.Nt), C.c_int(len(nodes)), _p(nodes), _p(gamma), _p(eta),
        *(_p(m) for m in mats[:5]), C.c_double(model.Ht), C.c_double(model.U), C.c_double(model.V),
        C.c_double(model.a), C.c_int(0 if model.is_complex else 1), _p(mats[5]), _p(bonds), C.c_int(len(bonds)),
        C.c_int(model.site[0]), C.c_int(model.site[1]), C.c_int(hc), _p(flat_s), C.c_int(sweeps),
        C.c_int(int(record)), _p(k), _p(u), C.c_size_t(len(k)), _p(obs), _p(acc) if log else None)
    if rc != 0:
        raise RuntimeError(f"kdq_cpu_tuv_phy_update failed with {rc}")
    s_out = flat_s.reshape(model.field_shape, order="F")
    return s_out, obs.reshape(-1, 7)[:sweeps], acc
