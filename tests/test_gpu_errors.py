"""Argument and state errors of the C ABI are reported as status codes with
a message (the reference raises Julia errors), and leave the handle usable."""
import numpy as np
import pytest

import cases
from kapdqmc_gb300 import Initial_s, slmc
from kapdqmc_gb300._lib import KdqError
from kapdqmc_gb300.sweep import Sweeper

pytestmark = pytest.mark.gpu


def test_scee_and_dop_argument_errors():
    m = cases.tu_honeycomb()
    with Sweeper(m, 3) as sw:
        sw.set_fields(np.stack([Initial_s(m, c) for c in range(3)]))
        with pytest.raises(KdqError, match="even number of chains"):
            sw.scee_enable([1, 2], [1], 0.5, 2)
        with pytest.raises(KdqError, match="region"):
            sw.dop_enable(0.5, list(range(1, m.Ns + 1)), [1], 0.5, 2)
        with pytest.raises(KdqError, match="out of range"):
            sw.dop_enable(0.5, [0, 1], [1], 0.5, 2)
        with pytest.raises(KdqError, match="lambda"):
            sw.dop_enable(0.5, [1, 2], [1], 1.5, 2)
        with pytest.raises(KdqError, match="must precede"):
            sw.scee_run(1)
        sw.set_rng(1)
        sw.phy_update(1, False)           # still usable


def test_model_restrictions():
    mv = cases.tv_honeycomb()
    with Sweeper(mv, 2) as sw:
        with pytest.raises(KdqError, match="disorder-operator"):
            sw.dop_enable(0.5, [1, 2], [1], 0.5, 2)
        with pytest.raises(KdqError, match="t-U only"):
            sw.slmc_enable(np.zeros(3057, np.float32), 1, 4, 8)
        with pytest.raises(KdqError, match="mixed precision"):
            sw.set_precision("mixed")
        with pytest.raises(KdqError, match="complex t-UV only"):
            sw.set_measure_full(True)
    with Sweeper(cases.tuv_honeycomb(U=-4.0, V=0.3), 2) as sw:     # real t-UV sweep
        with pytest.raises(KdqError, match="complex t-UV only"):
            sw.set_measure_full(True)


def test_slmc_argument_errors():
    m = cases.tu_square()
    with Sweeper(m, 1) as sw:
        p = slmc.init_params(0)
        with pytest.raises(KdqError, match="cluster_len"):
            sw.slmc_enable(p, 1, 9, 8)       # > Ns - 8 = 8
        bad = p.copy()
        bad[5] = np.nan
        with pytest.raises(KdqError, match="non-finite"):
            sw.slmc_enable(bad, 1, 4, 8)
        sw.slmc_enable(p, 0, 4, 8)           # off is always accepted


def test_cnn_argument_errors():
    with pytest.raises(ValueError):
        slmc.cnn_forward(np.zeros((1, 4, 4), np.uint8), slmc.init_params(0))   # values must be 1..4
    with pytest.raises(KdqError, match="Ns"):
        slmc.cnn_forward(np.ones((1, 4, 2), np.uint8), slmc.init_params(0))
