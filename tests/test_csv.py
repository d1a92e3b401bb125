"""The CSV side output of phy_update: the reference's file names and the
number format of Julia's writedlm, byte for byte.

File names: src/tU/phy_update.jl:12-27, src/tV/phy_update.jl:10-23,
src/tUV/phy_update.jl:13-22.  Rows: one ``writedlm(io, row, ',')`` per sweep
(src/tU/phy_update.jl:143-145, src/tV/phy_update.jl:178,
src/tUV/phy_update.jl:178), i.e. Julia's ``print`` of each Float64 joined
by commas.
"""
import os

import numpy as np
import pytest

import cases
from kapdqmc_gb300 import tU_Hubbard_Para
from kapdqmc_gb300.sweep import _append_csv, _csv_name, julia_float


# Julia 1.x `print(x)` of these Float64 values (Base.Ryu.writeshortest)
JULIA_PRINT = [
    (1.0, "1.0"), (0.0, "0.0"), (-0.0, "-0.0"), (10.0, "10.0"), (0.05, "0.05"),
    (0.1, "0.1"), (1e-4, "0.0001"), (1.234e-4, "0.0001234"), (1e-5, "1.0e-5"),
    (-1.2345678e-7, "-1.2345678e-7"), (100000.0, "100000.0"), (999999.0, "999999.0"),
    (123456.7, "123456.7"), (1e6, "1.0e6"), (1234567.0, "1.234567e6"), (1e16, "1.0e16"),
    (-87.123456789, "-87.123456789"), (5e-324, "5.0e-324"), (float("nan"), "NaN"),
    (float("inf"), "Inf"), (float("-inf"), "-Inf"), (1.0 / 3.0, "0.3333333333333333"),
]


@pytest.mark.parametrize("x,want", JULIA_PRINT)
def test_julia_float_format(x, want):
    assert julia_float(x) == want


def test_julia_float_round_trips():
    rng = np.random.default_rng(3)
    for x in np.concatenate([rng.normal(size=200) * 10.0 ** rng.integers(-12, 12, size=200),
                             rng.normal(size=50)]):
        assert float(julia_float(x)) == x


def test_file_names_follow_the_reference():
    tu = cases.tu_square()
    assert os.path.basename(_csv_name("/p", tu)) == "tUphy□45_t1.0U4.0size[2, 4]Δt0.1Θ1.0BS5.csv"
    hc = cases.tu_honeycomb()
    assert os.path.basename(_csv_name("/p", hc)) == "tUphyHC120_t1.0U4.0size[3, 3]Δt0.1Θ1.0BS5.csv"
    q = cases.tu_quench()
    assert os.path.basename(_csv_name("/p", q)) == "tUphyHC120_t1.0U0.0_3.8size[3, 3]Δt0.1Θ0.4_0.4BS10.csv"
    tv = cases.tv_honeycomb()
    assert os.path.basename(_csv_name("/p", tv)) == "tVphyHC120_t1.0V1.0size[3, 3]Δt0.1Θ1.0BS5.csv"
    tuv = cases.tuv_honeycomb()
    assert os.path.basename(_csv_name("/p", tuv)) == "tUVphyHC120_t1.0U4.0V0.5size[3, 3]Δt0.1Θ1.0BS5.csv"
    sq = cases.tuv_square()
    assert os.path.basename(_csv_name("/p", sq)) == "tUVphy□_t1.0U4.0V0.5size[2, 4]Δt0.1Θ1.0BS5.csv"
    c3 = tU_Hubbard_Para(Ht=1.0, Hu1=8.0, Hu2=8.0, Δt=0.05, Θrelax=8.0, Θquench=0.0,
                         Lattice="SQUARE45", site=[6, 12], BatchSize=8, Initial="H0")
    assert os.path.basename(_csv_name("/p", c3)) == "tUphy□45_t1.0U8.0size[6, 12]Δt0.05Θ8.0BS8.csv"


def test_rows_are_appended_in_writedlm_format(tmp_path):
    f = tmp_path / "out.csv"
    rows = np.array([[-12.5, 3.0, 1e-5, 0.25, 2e6, -0.0], [1.0, 2.0, 3.0, 4.0, 5.0, 6.0]])
    _append_csv(str(f), rows[:1])
    _append_csv(str(f), rows[1:])
    assert f.read_bytes() == "-12.5,3.0,1.0e-5,0.25,2.0e6,-0.0\n1.0,2.0,3.0,4.0,5.0,6.0\n".encode()
