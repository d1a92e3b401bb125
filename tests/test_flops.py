"""Operation counts behind the bench's roofline (kapdqmc_gb300/flops.py).

Known answers for a 16-site t-U lattice (Nt = 20, five nodes) worked out by
hand from the sweep's structure, and the bookkeeping identities of the
mixed sweep's per-pipe split: every algorithmic flop is assigned to exactly
one pipe.
"""
import pytest

import cases
from kapdqmc_gb300.flops import (DF_OPS_PER_FLOP, TF32_PRODUCTS, measure_wraps, measured_slices, mixed_roofline,
                                 sweep_flops)


def test_known_answers_t_u_16_sites():
    m = cases.tu_square()                  # N = 16, ns = 8, Nt = 20, NN = 5
    assert (m.Ns, m.Nt, len(m.nodes)) == (16, 20, 5)
    N, ns, Nt = 16, 8, 20
    fl = sweep_flops(m, accepted=10.0, record=2)
    # two N^3 products per slice and direction, complex G times real eK: 4 flops per multiply-add
    assert fl["wrap"] == 2 * Nt * 2 * N ** 3 * 4
    # rank-1 updates: N^2 complex multiply-adds per acceptance, plus the N-vector
    assert fl["update"] == 10 * (N * N * 8 + N * 8)
    assert fl["update_flush"] == 10 * N * N * 8
    # 2 (NN - 1) node crossings, each with X = (BL BR)^-1 BL and BR X
    assert fl["recompute_products"] == 8 * (ns * ns * N + N * N * ns) * 8
    assert fl["total"] == fl["wrap"] + fl["update"] + fl["stabilise"] + fl["measure"]


@pytest.mark.parametrize("make", [cases.tu_square, cases.tu_honeycomb, cases.c3, cases.tuv_honeycomb])
def test_mixed_pipe_split_accounts_for_every_flop(make):
    m = make()
    fl = sweep_flops(m, accepted=123.0, record=2)
    assert 0 < fl["recompute_products"] <= fl["stabilise_qr_lu"] <= fl["stabilise"]
    assert 0 < fl["update_flush"] <= fl["update"]
    assert 0 < fl["measure_kinetic"] <= fl["measure"]
    w = mixed_roofline(fl)
    tensor_flops = (fl["wrap"] + (fl["stabilise"] - fl["stabilise_qr_lu"]) + fl["measure_kinetic"]
                    + fl["recompute_products"] + fl["update_flush"])
    df_flops = fl["stabilise_qr_lu"] - fl["recompute_products"]
    fp32_flops = (fl["update"] - fl["update_flush"]) + (fl["measure"] - fl["measure_kinetic"])
    assert w["tensor"] == pytest.approx(TF32_PRODUCTS * tensor_flops)
    assert w["fp32"] == pytest.approx(2 * DF_OPS_PER_FLOP * df_flops + fp32_flops)
    # the three groups partition the algorithmic total
    assert tensor_flops + df_flops + fp32_flops == pytest.approx(fl["total"])
    # without tensor-core flushes the rank-k updates fall back to the FP32 pipe
    w0 = mixed_roofline(fl, tc_flush=False)
    assert w0["tensor"] == pytest.approx(w["tensor"] - TF32_PRODUCTS * fl["update_flush"])
    assert w0["fp32"] == pytest.approx(w["fp32"] + fl["update_flush"])


def test_measurement_window_counts():
    m = cases.tu_square()
    assert measured_slices(m) > 0
    assert measure_wraps(m) >= 0
    assert sweep_flops(m, 1.0, record=0)["measure"] == 0
