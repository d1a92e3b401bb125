"""The CUDA sweep (through the C ABI) against the committed golden fixtures.

Each fixture (tests/golden/sweep_*.json, written by make_golden.py) holds a
small model's initial fields, the Philox stream it consumes and the
oracle's results after two recorded sweeps.  The GPU must make the same
accept/reject decisions, end on the same fields, and match G to 1e-10 and
log|det| to 1e-9 (relative), and the measurement rows to the fixture's
``obs_tol``: 1e-9, or 1000 times the change the oracle's own rows show when
G is perturbed by 1e-15 before each measurement, where the wraps to
tau = Nt/2 amplify rounding more (t-V, real HS exponentials).  No oracle
code runs here.
"""
import json
from pathlib import Path

import numpy as np
import pytest

import cases
from kapdqmc_gb300.sweep import Sweeper

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
G_TOL = 1e-10
LD_TOL = 1e-9


@pytest.mark.parametrize("path", sorted(GOLDEN.glob("sweep_*.json")), ids=lambda p: p.stem)
def test_gpu_matches_golden_fixture(path):
    spec = json.loads(path.read_text())
    model = getattr(cases, spec["case"])()
    assert spec["chain"] == 0
    fields = np.array(spec["s"], dtype=np.uint8).reshape(model.field_shape, order="F")
    with Sweeper(model, 1) as sw:
        sw.set_fields(fields[None])
        sw.set_rng(spec["seed"])
        sw.enable_accept_log(spec["proposals"])
        obs = sw.phy_update(spec["sweeps"], True)
        s_out = sw.get_fields()[0]
        acc = sw.accept_log()[0].astype(bool)
        G = sw.green(0)
        ld, _ = sw.log_det()
    want = np.unpackbits(np.frombuffer(bytes.fromhex(spec["accepts_hex"]), np.uint8))[: spec["proposals"]]
    np.testing.assert_array_equal(acc, want.astype(bool))
    assert np.ravel(s_out, order="F").tolist() == spec["s_out"]
    ro = np.array(spec["obs"])
    err = np.abs(obs[0] - ro).max() / max(1.0, np.abs(ro).max())
    assert err < spec["obs_tol"], (err, spec["obs_tol"])
    Gw = np.array(spec["G_re"]) + (1j * np.array(spec["G_im"]) if spec["G_im"] is not None else 0)
    Gw = Gw.reshape(model.Ns, model.Ns, order="F")
    rel = np.linalg.norm(G - Gw) / np.linalg.norm(Gw)
    assert rel < G_TOL, rel
    assert abs(ld[0] - spec["log_det"]) < LD_TOL * max(1.0, abs(spec["log_det"]))
