"""Host-side mirror of the reference's sweep entry points over the CUDA library.

``phy_update(path, model, s, Sweeps, record)`` keeps the reference's
signature and semantics (returns the updated field, appends one CSV row per
sweep when recording); :class:`Sweeper` exposes the batched, resident form
(many chains per handle, device-resident state between calls).

References (KAPDQMC): src/tU/phy_update.jl:3-152, src/tV/phy_update.jl:1-188,
src/tUV/phy_update.jl:1-186, src/KAPDQMC.jl:12-28.
"""
from __future__ import annotations

import ctypes as C
import decimal
import math
import os
import threading

import numpy as np

from . import _lib
from .model import KIND_TU, KIND_TUV, KIND_TV

_LATTICE_ID = {"SQUARE45": 0, "SQUARE90": 1, "HoneyComb120": 2, "HoneyComb60": 3}
_CSV_LOCKS: dict = {}
_CSV_GUARD = threading.Lock()


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def _mat(m, as_complex):
    """Column-major matrix as a flat float64 buffer (interleaved if complex)."""
    m = np.asarray(m)
    flat = np.ravel(m, order="F")
    if as_complex:
        return np.ascontiguousarray(flat.astype(np.complex128)).view(np.float64)
    return np.ascontiguousarray(flat.real.astype(np.float64))


def model_desc(model):
    """kdq_model_desc for a model struct; returns (desc, keepalive)."""
    kind = model.kind
    gc = bool(model.is_complex)
    kmats = [model.eK, model.eKinv, model.HalfeK, model.HalfeKinv, model.K]
    kc = any(np.iscomplexobj(x) and np.any(np.imag(x) != 0) for x in kmats)
    keep = []

    def ptr(a):
        keep.append(a)
        return a.ctypes.data

    d = _lib.ModelDesc()
    d.kind = kind
    d.lattice = _LATTICE_ID[model.Lattice]
    d.site[0], d.site[1] = int(model.site[0]), int(model.site[1]) if len(model.site) > 1 else 1
    d.Ns, d.Nt = model.Ns, model.Nt
    d.z = 1 if kind == KIND_TU else int(model.nnidx.shape[1])
    d.g_complex, d.k_complex = int(gc), int(kc)
    nodes = _c(model.nodes, np.int64)
    d.n_nodes = len(nodes)
    d.nodes = ptr(nodes)
    d.alpha = ptr(_c(model.α, np.float64)) if kind != 2 else None
    d.gamma = ptr(_c(model.γ, np.float64))
    d.eta = ptr(_c(model.η, np.float64))
    d.a = float(getattr(model, "a", 0.0))
    d.Ht = float(model.Ht)
    d.U = float(getattr(model, "U", 0.0))
    d.V = float(getattr(model, "V", 0.0))
    d.eK, d.eKinv, d.HalfeK, d.HalfeKinv, d.K = (ptr(_mat(x, kc)) for x in kmats)
    d.Pt = ptr(_mat(model.Pt, gc))
    if kind != KIND_TU:
        b = np.asarray(model.nnidx).transpose(1, 0, 2).reshape(-1, 2)   # column-major bond order
        d.bonds = ptr(_c(b, np.int32))
    return d, keep


class Sweeper:
    """A batch of independent Markov chains of one model on one GPU."""

    def __init__(self, model, nchains: int = 1, device: int = 0):
        self.lib = _lib.load()
        self.model = model
        self.nchains = int(nchains)
        d, keep = model_desc(model)
        h = C.c_void_p()
        _lib.check(self.lib.kdq_create(C.byref(h), C.byref(d), self.nchains, device), None)
        del keep
        self.h = h
        self.n_obs = self.lib.kdq_n_obs(h)
        self.field_size = model.Nt * model.n_field

    # -- lifecycle ---------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.lib.kdq_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _ck(self, rc):
        _lib.check(rc, self.h)

    # -- state -------------------------------------------------------------
    def set_fields(self, s):
        """s: one field (model.field_shape) or a stack (nchains, *field_shape)."""
        s = np.asarray(s, dtype=np.uint8)
        if s.shape == tuple(self.model.field_shape):
            s = s[None]
        if s.shape[0] != self.nchains:
            raise ValueError(f"need {self.nchains} fields, got {s.shape[0]}")
        flat = np.concatenate([np.ravel(x, order="F") for x in s])
        flat = np.ascontiguousarray(flat)
        self._ck(self.lib.kdq_set_fields(self.h, flat.ctypes.data, flat.size))

    def get_fields(self):
        out = np.empty(self.nchains * self.field_size, dtype=np.uint8)
        self._ck(self.lib.kdq_get_fields(self.h, out.ctypes.data, out.size))
        shp = tuple(self.model.field_shape)
        return np.stack([out[c * self.field_size:(c + 1) * self.field_size].reshape(shp, order="F")
                         for c in range(self.nchains)])

    def set_rng(self, seed: int, sweep_offset: int = 0):
        self._ck(self.lib.kdq_set_rng(self.h, int(seed) & (2 ** 64 - 1), int(sweep_offset)))

    def set_tape(self, k, u):
        """Explicit proposal tape, arrays of shape (nchains, n)."""
        k = np.ascontiguousarray(np.asarray(k, dtype=np.uint8).reshape(self.nchains, -1))
        u = np.ascontiguousarray(np.asarray(u, dtype=np.float64).reshape(self.nchains, -1))
        self._keep_tape = (k, u)
        self._ck(self.lib.kdq_set_tape(self.h, k.ctypes.data, u.ctypes.data, k.shape[1]))

    # -- sweeps ------------------------------------------------------------
    def phy_update(self, sweeps: int, record=False):
        """Init from the fields + sweeps; returns obs (nchains, sweeps, n_obs) or None.

        record: 0/False none, 1/True as the reference, 2 the fast form of the
        same estimator (see kdq_phy_update)."""
        if record:
            obs = np.empty(self.nchains * sweeps * self.n_obs)
            self._ck(self.lib.kdq_phy_update(self.h, sweeps, int(record), obs.ctypes.data, obs.size))
            return obs.reshape(self.nchains, sweeps, self.n_obs)
        self._ck(self.lib.kdq_phy_update(self.h, sweeps, 0, None, 0))
        return None

    def init(self):
        self._ck(self.lib.kdq_init(self.h))

    def sweep(self, sweeps: int, record=False):
        self._ck(self.lib.kdq_sweep(self.h, sweeps, int(record)))

    def synchronize(self):
        self._ck(self.lib.kdq_synchronize(self.h))

    def get_obs(self, rows: int):
        obs = np.empty(self.nchains * rows * self.n_obs)
        self._ck(self.lib.kdq_get_obs(self.h, obs.ctypes.data, obs.size))
        return obs.reshape(self.nchains, rows, self.n_obs)

    def set_precision(self, mode: str):
        """"fp64" (default, the reference's arithmetic) or "mixed" (FP32 G,
        3xTF32 tensor-core kinetic products, delayed FP32 updates, FP64
        acceptance ratios, double-float QR and G recompute)."""
        code = {"fp64": 0, "mixed": 1}[mode]
        self._ck(self.lib.kdq_set_precision(self.h, code))
        self.precision = mode

    PHASES = ("wrap", "update", "measure", "block_product", "qr", "recompute", "cluster_moves", "ratio_windows")

    def enable_phase_timing(self, enable: bool = True):
        self._ck(self.lib.kdq_enable_phase_timing(self.h, int(bool(enable))))

    def phase_cycles(self) -> dict:
        out = np.zeros(8)
        self._ck(self.lib.kdq_get_phase_cycles(self.h, out.ctypes.data))
        return dict(zip(self.PHASES, out[:8].tolist()))

    def set_graphs(self, enable: bool):
        """Replay sweeps from a captured CUDA graph (default) or launch block by block."""
        self._ck(self.lib.kdq_set_graphs(self.h, int(bool(enable))))

    def set_sweep_launch(self, per_sweep: bool):
        """One launch per sweep (each chain's CTA runs all of the sweep's
        blocks) or, the default, one launch per stabilisation block."""
        self._ck(self.lib.kdq_set_sweep_launch(self.h, int(bool(per_sweep))))

    def set_tiles(self, rows: int):
        """Register-tile class of the sweep kernel (1, 3 or 6 row groups of 32 sites)."""
        self._ck(self.lib.kdq_set_tiles(self.h, int(rows)))

    @property
    def tiles(self) -> int:
        return self.lib.kdq_get_tiles(self.h)

    def autotune(self):
        """Time one sweep per valid tile class, keep the fastest, restore the
        fields and random-stream positions; returns (class, {class: ms})."""
        chosen = C.c_int32()
        ms = np.empty(3)
        self._ck(self.lib.kdq_autotune(self.h, C.byref(chosen), ms.ctypes.data, 3))
        return chosen.value, {r: float(t) for r, t in zip((1, 3, 6), ms) if t >= 0}

    @property
    def stream(self) -> int:
        return self.lib.kdq_stream(self.h) or 0

    # -- inspection --------------------------------------------------------
    def green(self, chain: int = 0):
        N = self.model.Ns
        gc = self.model.is_complex
        buf = np.empty(N * N * (2 if gc else 1))
        self._ck(self.lib.kdq_get_green(self.h, chain, buf.ctypes.data, buf.size))
        if gc:
            buf = buf.view(np.complex128)
        return buf.reshape(N, N, order="F")

    def stats(self):
        st = _lib.Stats()
        self._ck(self.lib.kdq_get_stats(self.h, C.byref(st)))
        return {f: getattr(st, f) for f, _ in st._fields_}

    def enable_accept_log(self, n_per_chain: int):
        self._acc_cap = int(n_per_chain)
        self._ck(self.lib.kdq_enable_accept_log(self.h, self._acc_cap))

    def accept_log(self):
        out = np.empty(self.nchains * self._acc_cap, dtype=np.uint8)
        self._ck(self.lib.kdq_get_accept_log(self.h, out.ctypes.data, out.size))
        return out.reshape(self.nchains, self._acc_cap)

    def grover_det(self, index):
        """Grover determinants of the chain pairs (0,1), (2,3), ... at their current slice."""
        idx = np.ascontiguousarray(np.asarray(index, dtype=np.int32))
        out = np.empty(2 * (self.nchains // 2))
        self._ck(self.lib.kdq_grover_det_chains(self.h, idx.ctypes.data, idx.size, out.ctypes.data))
        return out.view(np.complex128)

    def keep_middle_green(self, enable: bool = True):
        """Keep each chain's G at tau = Nt/2 during recording sweeps."""
        self._ck(self.lib.kdq_keep_middle_green(self.h, int(bool(enable))))

    def grover_det_middle(self, index):
        """Grover determinants of the chain pairs on their G at tau = Nt/2."""
        idx = np.ascontiguousarray(np.asarray(index, dtype=np.int32))
        out = np.empty(2 * (self.nchains // 2))
        self._ck(self.lib.kdq_grover_det_middle(self.h, idx.ctypes.data, idx.size, out.ctypes.data))
        return out.view(np.complex128)

    def log_det(self):
        """log|det(P^H B(Theta,0) P)| (n_chains,) and det/|det| (complex, n_chains,)
        of every chain's current fields, from the stabilised B chains."""
        ld = np.empty(self.nchains)
        ph = np.empty(2 * self.nchains)
        self._ck(self.lib.kdq_get_log_det(self.h, ld.ctypes.data, ph.ctypes.data, self.nchains))
        return ld, ph[0::2] + 1j * ph[1::2]

    def log_weight(self, fields=None):
        """Full log-weight log|W(s)| of every chain (see ``log_weight``)."""
        ld, _ = self.log_det()
        s = self.get_fields() if fields is None else fields
        return np.array([log_weight(self.model, s[c], ld[c]) for c in range(self.nchains)])

    def slmc_enable(self, params, moves_per_slice: int = 1, cluster_len: int = 32, eff_steps: int = 64):
        """Turn on the self-learning cluster moves (t-U) with the effective
        model ``params`` (see ``kapdqmc_gb300.slmc``); moves_per_slice=0 turns them off."""
        p = np.ascontiguousarray(np.asarray(params, dtype=np.float32))
        if p.shape != (3057,):
            raise ValueError("params must hold 3057 floats")
        self._ck(self.lib.kdq_slmc_enable(self.h, p.ctypes.data, moves_per_slice, cluster_len, eff_steps))

    def scee_enable(self, indexA, indexB, lam: float, nlam: int):
        """Regions (1-based sites), lambda and Nlambda of the coupled SCEE sweep."""
        a = np.ascontiguousarray(np.asarray(indexA, dtype=np.int32))
        b = np.ascontiguousarray(np.asarray(indexB, dtype=np.int32))
        self._ck(self.lib.kdq_scee_enable(self.h, a.ctypes.data, a.size, b.ctypes.data, b.size, float(lam), int(nlam)))

    def scee_run(self, sweeps: int):
        """Coupled SCEE sweeps of every replica pair; returns (n_pairs, sweeps + 1)
        rows as ctrl_SCEEicr writes them (lambda, then one estimator per sweep)."""
        npairs = self.nchains // 2
        out = np.empty(npairs * (sweeps + 1))
        self._ck(self.lib.kdq_scee_run(self.h, sweeps, out.ctypes.data, out.size))
        return out.reshape(npairs, sweeps + 1)

    def dop_enable(self, alpha: float, indexA, indexB, lam: float, nlam: int):
        """Angle, regions (1-based sites), lambda and Nlambda of the disorder-operator sweep."""
        a = np.ascontiguousarray(np.asarray(indexA, dtype=np.int32))
        b = np.ascontiguousarray(np.asarray(indexB, dtype=np.int32))
        self._ck(self.lib.kdq_dop_enable(self.h, float(alpha), a.ctypes.data, a.size, b.ctypes.data, b.size,
                                         float(lam), int(nlam)))

    def dop_run(self, sweeps: int):
        """Disorder-operator sweeps of every chain; returns (n_chains, sweeps + 1)
        rows as ctrl_SCDOPicr writes them."""
        out = np.empty(self.nchains * (sweeps + 1))
        self._ck(self.lib.kdq_dop_run(self.h, sweeps, out.ctypes.data, out.size))
        return out.reshape(self.nchains, sweeps + 1)

    def scee_green(self, chain: int, which: int):
        """Green's function `which` (0 Gt, 1 G0, 2 Gt0, 3 G0t) of one replica."""
        N = self.model.Ns
        cplx = self.model.is_complex
        out = np.empty((2 if cplx else 1) * N * N)
        self._ck(self.lib.kdq_scee_get_green(self.h, chain, which, out.ctypes.data, out.size))
        return (out.view(np.complex128) if cplx else out).reshape(N, N, order="F")

    def set_measure_full(self, enable: bool = True):
        """t-U and complex t-UV: 4 more columns after the reference's 6 or 7:
        honeycomb, CDW0, CDW1, SDW0, SDW1 with all terms; square lattices,
        the staggered charge structure factor at (pi, pi), 0, the staggered
        spin structure factor at (pi, pi), 0."""
        self._ck(self.lib.kdq_set_measure_full(self.h, int(bool(enable))))
        self.n_obs = self.lib.kdq_n_obs(self.h)

    def slmc_stats(self):
        """(proposed, accepted, no-change) cluster moves of the last call."""
        out = np.zeros(3, dtype=np.int64)
        self._ck(self.lib.kdq_get_slmc_stats(self.h, out.ctypes.data))
        return {"proposed": int(out[0]), "accepted": int(out[1]), "unchanged": int(out[2])}

    def drift(self, sweeps: int):
        n = sweeps * 2 * (len(self.model.nodes) - 1)
        out = np.empty(self.nchains * n)
        self._ck(self.lib.kdq_get_drift(self.h, out.ctypes.data, out.size))
        return out.reshape(self.nchains, n)


def log_weight(model, s, logdet: float) -> float:
    """log|W(s)| of one configuration from log|det(P^H B(Theta,0) P)|.

    W is the weight whose ratios the sweep accepts with: t-U and complex t-UV
    |det|^2 prod gamma[s] (src/tU/phy_update.jl:260-261, src/tUV/GreenMatrix.jl:
    73-89), t-V det prod gamma[s] (src/tV/GreenMatrix.jl:76-89 with
    src/tV/phy_update.jl:196-199), real t-UV det^2 prod gamma[s] e^{-(a+1) eta[s]}
    (src/tUV/phy_update.jl:192-197).
    """
    s = np.asarray(s).astype(np.int64).ravel() - 1
    loc = float(np.log(np.asarray(model.γ, dtype=float))[s].sum())
    if model.kind == KIND_TV:
        return loc + logdet
    if model.kind == KIND_TUV and not model.is_complex:
        loc -= (model.a + 1.0) * float(np.asarray(model.η, dtype=float)[s].sum())
    return loc + 2.0 * logdet


def grover_det(G1, G2, index, device: int = 0):
    """det(2 G1_A G2_A - G1_A - G2_A + I) for stacks of replica pairs.

    G1, G2: (npairs, Ns, Ns) or (Ns, Ns) arrays; index: 1-based sites of A.
    GroverMatrix! (src/public/GF.jl:101-109) and the det of get_ABGM!
    (src/tU/SCEE.jl:264-276).  Returns complex determinants (npairs,).
    """
    lib = _lib.load()
    G1 = np.asarray(G1)
    G2 = np.asarray(G2)
    if G1.ndim == 2:
        G1, G2 = G1[None], G2[None]
    gc = np.iscomplexobj(G1) or np.iscomplexobj(G2)
    npairs, Ns = G1.shape[0], G1.shape[1]
    mats = []
    for a, b in zip(G1, G2):
        mats += [_mat(a, gc), _mat(b, gc)]
    buf = np.ascontiguousarray(np.concatenate(mats))
    idx = np.ascontiguousarray(np.asarray(index, dtype=np.int32))
    out = np.empty(2 * npairs)
    _lib.check(lib.kdq_grover_det(buf.ctypes.data, Ns, int(gc), npairs, idx.ctypes.data, idx.size,
                                  out.ctypes.data, device), None)
    return out.view(np.complex128)



def julia_float(x) -> str:
    """A Float64 as Julia's ``print`` writes it (what ``writedlm`` puts in
    the reference's CSV files and ``$(x)`` in its file names): the shortest
    round-trip digits, written plainly when the decimal point falls within
    -4 < pt <= 6 digits of the first digit (whole values end in ".0"), else
    as d.ddde<exp> with no exponent padding ("1.0e-5", "1.234567e6").  Julia
    chooses this in Base.Ryu.writeshortest."""
    x = float(x)
    if math.isnan(x):
        return "NaN"
    if math.isinf(x):
        return "Inf" if x > 0 else "-Inf"
    if x == 0.0:
        return "-0.0" if math.copysign(1.0, x) < 0 else "0.0"
    sign, digits, exp = decimal.Decimal(repr(x)).as_tuple()   # repr: shortest round-trip digits
    full = "".join(map(str, digits))
    d = full.rstrip("0")
    exp += len(full) - len(d)                                    # trailing zeros move into the exponent
    olength = len(d)
    pt = exp + olength
    neg = "-" if sign else ""
    if -4 < pt <= 6 and not (pt >= olength and abs(math.fmod(abs(x) + 0.05, 10.0 ** (pt - olength)) - 0.05) > 0.05):
        if pt <= 0:
            return neg + "0." + "0" * (-pt) + d
        if pt >= olength:
            return neg + d + "0" * (pt - olength) + ".0"
        return neg + d[:pt] + "." + d[pt:]
    return neg + d[0] + "." + (d[1:] or "0") + "e" + str(pt - 1)

# ------------------------------------------------------------------------
# reference-shaped entry points
# ------------------------------------------------------------------------
def _csv_name(path, model):
    """File name scheme of the reference's CSV output.

    src/tU/phy_update.jl:12-27, src/tV/phy_update.jl:10-23,
    src/tUV/phy_update.jl:13-22 (the tV/tUV square case is named "□").
    """
    f = julia_float

    site = "[" + ", ".join(str(int(v)) for v in model.site) + "]"
    if model.kind == KIND_TU:
        name = {"SQUARE90": "□90", "SQUARE45": "□45", "HoneyComb60": "HC", "HoneyComb120": "HC120"}[model.Lattice]
        if model.Θquench == 0.0:
            return os.path.join(path, f"tUphy{name}_t{f(model.Ht)}U{f(model.Hu1)}size{site}Δt{f(model.Δt)}"
                                      f"Θ{f(model.Θrelax)}BS{model.BatchSize}.csv")
        return os.path.join(path, f"tUphy{name}_t{f(model.Ht)}U{f(model.Hu1)}_{f(model.Hu2)}size{site}"
                                  f"Δt{f(model.Δt)}Θ{f(model.Θrelax)}_{f(model.Θquench)}BS{model.BatchSize}.csv")
    name = {"SQUARE45": "□", "SQUARE90": "□", "HoneyComb60": "HC", "HoneyComb120": "HC120"}[model.Lattice]
    if model.kind == KIND_TV:
        if len(np.unique(model.α)) == 1:
            return os.path.join(path, f"tVphy{name}_t{f(model.Ht)}V{f(model.Hv1)}size{site}Δt{f(model.Δt)}"
                                      f"Θ{f(model.Θrelax)}BS{model.BatchSize}.csv")
        return os.path.join(path, f"tVphy{name}_t{f(model.Ht)}V{f(model.Hv1)}_{f(model.Hv2)}size{site}"
                                  f"Δt{f(model.Δt)}Θ{f(model.Θrelax)}_{f(model.Θquench)}BS{model.BatchSize}.csv")
    return os.path.join(path, f"tUVphy{name}_t{f(model.Ht)}U{f(model.U)}V{f(model.V)}size{site}"
                              f"Δt{f(model.Δt)}Θ{f(model.Θ)}BS{model.BatchSize}.csv")


def _append_csv(file, rows):
    """Append rows under a per-file lock (the reference's lock is per call,
    src/tU/phy_update.jl:4, so it never serialises concurrent callers)."""
    with _CSV_GUARD:
        lk = _CSV_LOCKS.setdefault(os.path.abspath(file), threading.Lock())
    with lk, open(file, "a") as io:
        for r in rows:
            io.write(",".join(julia_float(v) for v in np.ravel(r)) + "\n")


def _scee_csv_name(path, model, nlam):
    """src/tU/SCEE.jl:16-32, src/tV/SCEE.jl:16-32."""
    f = julia_float

    site = "[" + ", ".join(str(int(v)) for v in model.site) + "]"
    if model.kind == KIND_TUV:   # src/tUV/SCEE.jl:16-26
        name = {"SQUARE45": "□", "SQUARE90": "□", "HoneyComb60": "HC60", "HoneyComb120": "HC120"}[model.Lattice]
        return os.path.join(path, f"tUVSCEE{name}_t{f(model.Ht)}U{f(model.U)}V{f(model.V)}size{site}Δt{f(model.Δt)}"
                                  f"Θ{f(model.Θ)}N{nlam}BS{model.BatchSize}.csv")
    if model.kind == KIND_TV:
        name = {"SQUARE45": "□", "SQUARE90": "□", "HoneyComb60": "HC", "HoneyComb120": "HC120"}[model.Lattice]
        if len(np.unique(model.α)) == 1:
            return os.path.join(path, f"tVSCEE{name}_t{f(model.Ht)}V{f(model.Hv1)}size{site}Δt{f(model.Δt)}"
                                      f"Θ{f(model.Θrelax)}N{nlam}BS{model.BatchSize}.csv")
        return os.path.join(path, f"tVSCEE{name}_t{f(model.Ht)}V{f(model.Hv1)}_{f(model.Hv2)}size{site}Δt{f(model.Δt)}"
                                  f"Θ{f(model.Θrelax)}_{f(model.Θquench)}N{nlam}BS{model.BatchSize}.csv")
    name = {"SQUARE90": "□90", "SQUARE45": "□45", "HoneyComb60": "HC", "HoneyComb120": "HC120"}[model.Lattice]
    if model.Θquench == 0.0:
        return os.path.join(path, f"tUSCEE{name}_t{f(model.Ht)}U{f(model.Hu1)}size{site}Δt{f(model.Δt)}"
                                  f"Θ{f(model.Θrelax)}N{nlam}BS{model.BatchSize}.csv")
    return os.path.join(path, f"tUSCEE{name}_t{f(model.Ht)}U{f(model.Hu1)}_{f(model.Hu2)}size{site}Δt{f(model.Δt)}"
                              f"Θ{f(model.Θrelax)}_{f(model.Θquench)}N{nlam}BS{model.BatchSize}.csv")


def ctrl_SCEEicr(path, model, indexA, indexB, Sweeps: int, λ: float, Nλ: int, ss, record: bool, *,
                 seed=None, tape=None, device: int = 0):
    """Coupled incremental SCEE sweep of the replica pair(s) ``ss``
    (src/tU/SCEE.jl:1-211, src/tV/SCEE.jl:1-431, src/tUV/SCEE.jl:1-339):
    returns the updated fields.  ``ss`` is a pair
    [s1, s2] or a stack of pairs (n_pairs, 2, ...); with ``record`` one CSV row
    per pair (lambda, then the per-sweep estimator) is appended to the
    reference's file name under ``path`` and the rows are also returned."""

    ss = np.asarray(ss, dtype=np.uint8)
    single = ss.ndim == len(model.field_shape) + 1
    pairs = ss[None] if single else ss
    stack = pairs.reshape((-1,) + tuple(model.field_shape))
    with Sweeper(model, nchains=stack.shape[0], device=device) as sw:
        sw.set_fields(stack)
        if tape is not None:
            sw.set_tape(*tape)
        else:
            sw.set_rng(int.from_bytes(os.urandom(8), "little") if seed is None else seed)
        sw.scee_enable(indexA, indexB, λ, Nλ)
        O = sw.scee_run(Sweeps)
        out = sw.get_fields().reshape(pairs.shape)
    out = out[0] if single else out
    if record:
        if path:
            _append_csv(_scee_csv_name(path, model, Nλ), O)
        return out, O
    return out


def _dop_csv_name(path, model, nlam):
    """src/tU/disorder_operate.jl:15-31 (the quench variant keyed on a non-constant alpha profile)."""
    f = julia_float

    site = "[" + ", ".join(str(int(v)) for v in model.site) + "]"
    name = {"SQUARE90": "□90", "SQUARE45": "□45", "HoneyComb60": "HC", "HoneyComb120": "HC120"}[model.Lattice]
    if len(np.unique(model.α)) == 1:
        return os.path.join(path, f"tUSCDOP{name}_t{f(model.Ht)}U{f(model.Hu1)}size{site}Δt{f(model.Δt)}"
                                  f"Θ{f(model.Θrelax)}N{nlam}BS{model.BatchSize}.csv")
    return os.path.join(path, f"tUSCDOP{name}_t{f(model.Ht)}U{f(model.Hu1)}_{f(model.Hu2)}size{site}Δt{f(model.Δt)}"
                              f"Θ{f(model.Θrelax)}_{f(model.Θquench)}N{nlam}BS{model.BatchSize}.csv")


def ctrl_SCDOPicr(path, model, alpha: float, indexA, indexB, Sweeps: int, λ: float, Nλ: int, s, record: bool, *,
                  seed=None, tape=None, device: int = 0):
    """Disorder-operator sweep of the field(s) ``s`` (src/tU/disorder_operate.jl:
    1-247): returns the updated field(s); with ``record`` one CSV row per chain
    (lambda, then the per-sweep estimator) is appended under ``path`` and the
    rows are also returned."""
    if model.kind != KIND_TU:
        raise ValueError("ctrl_SCDOPicr is implemented for t-U")
    s = np.asarray(s, dtype=np.uint8)
    single = s.shape == tuple(model.field_shape)
    stack = s[None] if single else s
    with Sweeper(model, nchains=stack.shape[0], device=device) as sw:
        sw.set_fields(stack)
        if tape is not None:
            sw.set_tape(*tape)
        else:
            sw.set_rng(int.from_bytes(os.urandom(8), "little") if seed is None else seed)
        sw.dop_enable(alpha, indexA, indexB, λ, Nλ)
        O = sw.dop_run(Sweeps)
        out = sw.get_fields()
    out = out[0] if single else out
    if record:
        if path:
            _append_csv(_dop_csv_name(path, model, Nλ), O)
        return out, O
    return out


def phy_update(path, model, s, Sweeps: int, record: bool = False, *, seed=None, tape=None,
               device: int = 0, sweeper: Sweeper | None = None):
    """Sweep the HS field(s) ``s`` and return the updated field(s).

    ``s`` is one field in the reference's layout or a stack of fields (one
    per chain).  ``seed`` selects the Philox stream (default: time-based,
    like the reference's unseeded generator); ``tape=(k, u)`` gives an
    explicit proposal tape instead.  When ``record`` is true one CSV row per
    sweep (averaged over chains) is appended to the reference's file name
    under ``path`` and the per-chain rows are also returned as ``s, obs``.
    """
    s = np.asarray(s, dtype=np.uint8)
    single = s.shape == tuple(model.field_shape)
    stack = s[None] if single else s
    own = sweeper is None
    sw = sweeper or Sweeper(model, nchains=stack.shape[0], device=device)
    try:
        sw.set_fields(stack)
        if tape is not None:
            sw.set_tape(*tape)
        else:
            if seed is None:
                seed = int.from_bytes(os.urandom(8), "little")
            sw.set_rng(seed)
        obs = sw.phy_update(Sweeps, record)
        out = sw.get_fields()
    finally:
        if own:
            sw.close()
    out = out[0] if single else out
    if record:
        if path:   # the reference's columns; further columns are returned only
            _append_csv(_csv_name(path, model), obs.mean(axis=0)[..., :6 if model.kind == KIND_TU else None])
        return out, obs
    return out


class SweeperGroup:
    """Sweepers of different lattices, models or precisions on one GPU, swept
    together as one CUDA graph per sweep (``kdq_group_sweep``).  Each
    sweeper's results equal those of sweeping it alone."""

    def __init__(self, sweepers):
        self.lib = _lib.load()
        self.sweepers = list(sweepers)
        arr = (C.c_void_p * len(self.sweepers))(*[s.h.value for s in self.sweepers])
        g = C.c_void_p()
        _lib.check(self.lib.kdq_group_create(C.byref(g), arr, len(self.sweepers)), None)
        self.g = g

    def close(self):
        if getattr(self, "g", None):
            self.lib.kdq_group_destroy(self.g)
            self.g = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _ck(self, rc):
        if rc != _lib.KDQ_OK:
            msg = self.lib.kdq_group_last_error(self.g)
            raise _lib.KdqError(rc, msg.decode() if msg else "")

    def sweep(self, sweeps: int, record=False):
        self._ck(self.lib.kdq_group_sweep(self.g, int(sweeps), int(record)))

    def synchronize(self):
        self._ck(self.lib.kdq_group_synchronize(self.g))

    def phy_update(self, sweeps: int, record=False):
        """Init every sweeper from its fields, sweep all together; returns one
        obs array (nchains, sweeps, n_obs) per sweeper, or None."""
        for s in self.sweepers:
            s.init()
        self.sweep(sweeps, record)
        self.synchronize()
        if not record:
            return None
        return [s.get_obs(sweeps) for s in self.sweepers]
