"""Algorithmic operation counts of one sweep (roofline numerators).

Counts are real floating-point operations (a complex multiply-add is 8, a
real one 2; a complex x real multiply-add is 4) of the algorithm as the
sweep kernels perform it: the slice wraps, the local-update ratios and
rank-k updates, the thin-factor block products, the Householder
orthonormalisation, the G recompute and, when recording, the measurement
wraps.  The reference's dense bond-rotation GEMMs in t-V are not counted
(the rotations are O(N^2) 2x2 block operations).
"""
from __future__ import annotations

from .model import KIND_TU, KIND_TV


def _mac(model, left_complex: bool, right_complex: bool) -> int:
    if left_complex and right_complex:
        return 8
    if left_complex or right_complex:
        return 4
    return 2


def sweep_flops(model, accepted: float, record, k_complex: bool = False) -> dict:
    """FLOPs of one forward+backward sweep of one chain.

    ``accepted``: accepted proposals per chain-sweep (measured).
    """
    N, Nt, ns = model.Ns, model.Nt, model.Ns // 2
    gc = bool(model.is_complex)
    kc = bool(k_complex)
    mgk = _mac(model, gc, kc)                 # G (x) eK
    mgg = _mac(model, gc, gc)
    out = {}
    # two N^3 products per slice and direction
    wrap = 2 * N ** 3 * mgk
    rot = 0
    if model.kind == KIND_TV:
        rot = model.z * 14 * N * N           # 2x2 block rotations per slice
    out["wrap"] = 2 * Nt * (wrap + rot)
    # local updates: rank-k update of G per accepted proposal
    rank = 1 if model.kind == KIND_TU else 2
    out["update"] = accepted * (rank * N * N * mgg + N * rank * rank * mgg)
    # stabilisation: per node crossing (2 (NN-1) per sweep)
    nodes = list(model.nodes)
    n_cross = 2 * (len(nodes) - 1)
    thin = Nt * 2 * (N * N * ns * mgk + (model.z * 14 * N * ns // 2 if model.kind == KIND_TV else 0))
    hh = 2 * (2 * N * ns * ns - 2 * ns ** 3 // 3) * (mgg // 2)   # geqrf + orgqr (mgg/2 per op pair)
    getg = (ns * ns * N + ns ** 3 // 3 + ns * ns * N + N * N * ns) * mgg
    out["stabilise"] = thin + n_cross * (hh + getg)
    out["stabilise_qr_lu"] = n_cross * (hh + getg)     # FP64 (plain) or double-float (mixed)
    # of which the two products after the inverse, X = (BL BR)^-1 BL and BR X
    # (3xTF32 tensor tiles in the mixed sweep)
    out["recompute_products"] = n_cross * (ns * ns * N + N * N * ns) * mgg
    # of the local updates: the rank-k G updates themselves (the mixed sweep's
    # delayed flushes, 3xTF32 tensor tiles for a complex G)
    out["update_flush"] = accepted * rank * N * N * mgg
    if record == 2:
        # fast form: two products per measurement plus the factor pushes/pops
        # (each a slice matrix applied to L and to R)
        out["measure_kinetic"] = fast_factor_ops(model) * (wrap + rot)
        out["measure"] = out["measure_kinetic"] + measured_slices(model) * 2 * N ** 3 * mgg
    elif record:
        out["measure_kinetic"] = measure_wraps(model) * (wrap + rot) + measured_slices(model) * 2 * N ** 3 * mgk
        out["measure"] = out["measure_kinetic"]
    else:
        out["measure"] = out["measure_kinetic"] = 0
    parts = ("stabilise_qr_lu", "measure_kinetic", "recompute_products", "update_flush")
    out["total"] = sum(v for k, v in out.items() if k not in parts)
    return out


# FP32-pipe instructions per algorithmic flop of the double-float
# arithmetic of the mixed sweep's stabilisation: a real multiply-add (2
# flops) of its GEMMs and reflector dot products takes 12 FP32 operations
# (kdq_device.cuh, madd_lazy; 15 with a renormalisation per step).
DF_OPS_PER_FLOP = 6.0
# TF32 tensor products per FP32 product of the 3xTF32 split
TF32_PRODUCTS = 3


def mixed_roofline(fl: dict, tc_flush: bool = True) -> dict:
    """Work of one mixed-precision chain-sweep per pipe, in the units the
    pipe's peak is measured in: 'tensor' = TF32 tensor flops of the 3xTF32
    products (slice wraps, thin block products, measurement factors, the
    recompute's X and BR X products and, with tc_flush, the delayed rank-k
    flushes of G), 'fp32' = FP32-pipe flops of the double-float
    stabilisation (QR, BL BR and its inverse; 2 * DF_OPS_PER_FLOP per
    algorithmic flop, the peak counting an FMA as 2) plus the rest of the
    FP32 local updates and the measurement products."""
    flush = fl["update_flush"] if tc_flush else 0
    tensor = TF32_PRODUCTS * (fl["wrap"] + (fl["stabilise"] - fl["stabilise_qr_lu"]) + fl["measure_kinetic"]
                              + fl["recompute_products"] + flush)
    fp32 = (2 * DF_OPS_PER_FLOP * (fl["stabilise_qr_lu"] - fl["recompute_products"]) + fl["update"] - flush
            + (fl["measure"] - fl["measure_kinetic"]))
    return {"tensor": tensor, "fp32": fp32}


def _window(model):
    NN = len(model.nodes)
    Θidx = NN // 2 + 1
    nodes = list(model.nodes)
    fwd, bwd = [], []
    for k in range(1, NN):
        lo, hi = nodes[k - 1], nodes[k]
        if model.kind == KIND_TU:
            f_on = 0 <= Θidx - k <= 1
            b_on = 0 <= (k + 1) - Θidx <= 1
        else:
            f_on = abs(k - Θidx) <= 1
            b_on = abs(k + 1 - Θidx) <= 1
        if f_on:
            fwd += list(range(lo + 1, hi + 1))
        if b_on:
            bwd += [lt - 1 if model.kind == KIND_TV else lt for lt in range(hi, lo, -1)]
    return fwd + bwd


def measured_slices(model) -> int:
    return len(_window(model))


def measure_wraps(model) -> int:
    """Slices wrapped by the measurements of one sweep (each to Nt/2)."""
    half = model.Nt // 2
    n = 0
    for t0 in _window(model):
        n += (t0 - half) if 2 * t0 > model.Nt else (half - t0)
    return n


def fast_factor_ops(model) -> int:
    """Factor pushes + pops of the record == 2 measurement in one steady-state sweep.

    Replays the sweep order (every slice's fields change when it is updated)
    against the factor stack of the kernel's measure_fast."""
    Nt, half = model.Nt, model.Nt // 2
    NN = len(model.nodes)
    Θidx = NN // 2 + 1
    nodes = list(model.nodes)
    version = [0] * (Nt + 2)
    stack: list = []
    ops = 0

    def measure(t0):
        nonlocal stack, ops
        below = 2 * t0 <= Nt
        m = half - t0 if below else t0 - half
        target = [((half - q) if below else (half + 1 + q), 1 if below else -1) for q in range(m)]
        k = 0
        while k < min(len(stack), m) and stack[k] == (target[k][0], target[k][1], version[target[k][0]]):
            k += 1
        ops += (len(stack) - k if k else 0) + (m - k)
        stack = [(sl, o, version[sl]) for sl, o in target]

    def in_window(idx):
        if model.kind == KIND_TU:
            return None
        return abs(idx - Θidx) <= 1

    count_from = None
    for sweep in range(2):
        if sweep == 1:
            count_from = ops
        idx = 1
        for lt in range(1, Nt + 1):
            version[lt] += 1
            on = (0 <= Θidx - idx <= 1) if model.kind == KIND_TU else abs(idx - Θidx) <= 1
            if on:
                measure(lt)
            if lt in nodes:
                idx += 1
        for lt in range(Nt, 0, -1):
            version[lt] += 1
            on = (0 <= idx - Θidx <= 1) if model.kind == KIND_TU else abs(idx - Θidx) <= 1
            if on:
                measure(lt - 1 if model.kind == KIND_TV else lt)
            if lt - 1 in nodes:
                idx -= 1
    return ops - count_from
