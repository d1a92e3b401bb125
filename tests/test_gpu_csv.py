"""phy_update with record writes the reference's CSV file through the
Python wrapper: the reference's file name under ``path``, one writedlm row
per sweep with the reference's columns (src/tU/phy_update.jl:23-27,143-145:
Ek Eu CDW0 CDW1 SDW0 SDW1; src/tV/phy_update.jl:19-23,178: Ek Ev R0 R1;
src/tUV/phy_update.jl:22,178: Ek Eu Ev CDW0 CDW1 SDW0 SDW1), each the mean
over the call's chains, appended across calls."""
import os

import numpy as np
import pytest

import cases
from kapdqmc_gb300 import Initial_s
from kapdqmc_gb300.sweep import _csv_name, julia_float, phy_update

pytestmark = pytest.mark.gpu

NCOLS = {0: 6, 1: None, 2: 7}


@pytest.mark.parametrize("make", [cases.tu_honeycomb, cases.tv_honeycomb, cases.tuv_honeycomb],
                         ids=["tU", "tV", "tUV"])
def test_phy_update_appends_the_reference_csv(tmp_path, make):
    model = make()
    s = np.stack([Initial_s(model, 11 + c) for c in range(3)])
    lines = []
    for call in range(2):
        s, obs = phy_update(str(tmp_path), model, s, 2, True, seed=90 + call)
        ncol = NCOLS[model.kind]
        mean = obs.mean(axis=0)[:, :ncol]
        assert mean.shape[1] == (ncol or obs.shape[2])
        lines += [",".join(julia_float(v) for v in row) for row in mean]
    files = os.listdir(tmp_path)
    assert files == [os.path.basename(_csv_name(str(tmp_path), model))]
    text = (tmp_path / files[0]).read_text()
    assert text == "".join(ln + "\n" for ln in lines)
    assert all(np.isfinite([float(v) for ln in lines for v in ln.split(",")]))
