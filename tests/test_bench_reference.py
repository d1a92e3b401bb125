"""The reference arm of bench.py on the host cores: the C restatement of the
reference sweep (t-UV: src/tUV/phy_update.jl:1-203; t-U, the default
workload: src/tU/phy_update.jl:3-267) timed on the workload, printing the
bench contract's JSON line; under torchrun only rank 0 runs and prints."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
ARGS = ["--impl", "reference", "--steps", "1", "--warmup", "3"]


def _bench(workload=None, env_extra=None):
    env = dict(os.environ)
    env.update(env_extra or {})
    extra = ["--workload", workload] if workload else []
    return subprocess.run([sys.executable, str(ROOT / "bench.py"), *ARGS, *extra], capture_output=True, text=True,
                          timeout=900, env=env, cwd=ROOT)


@pytest.mark.parametrize("workload,model,size", [("c4", "t-UV", "t-UV 8x8"), (None, "t-U", "t-U 12x12")],
                         ids=["tuv_8x8", "tu_12x12_default"])
def test_reference_arm_prints_the_contract_line(workload, model, size):
    r = _bench(workload)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference"
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["e2e"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == line["value"] and cb["cores"] >= 1
    assert model + " sweep" in cb["sample"]
    assert size in line["config"]["workload"]


def test_reference_arm_is_silent_on_other_ranks():
    r = _bench("c4", {"RANK": "1", "WORLD_SIZE": "2"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
