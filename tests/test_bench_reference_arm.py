"""The bench's reference arm on the host (no GPU): the C/OpenMP restatement timed for whole frames,
printing the contract's JSON line, and silent on ranks other than 0."""

import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _run(extra_env=None):
    env = dict(os.environ, **(extra_env or {}))
    cmd = [sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--cells", "6", "--steps", "1",
           "--warmup", "1"]
    return subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=300, cwd=ROOT)


def test_reference_arm_prints_the_contract_line():
    res = _run()
    assert res.returncode == 0, res.stderr[-2000:]
    line = json.loads(res.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["value"] > 0 and line["steps"] == 1 and line["warmup"] == 1 and line["higher_is_better"]
    assert line["config"]["workload"] == "hex8_block_6^3" and line["config"]["nodes"] == 7 ** 3
    base = line["cpu_baseline"]
    assert base["value"] == line["value"] and base["kind"] in ("port", "reference") and base["cores"] >= 1
    assert base["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_reference_arm_is_silent_off_rank_zero():
    res = _run({"RANK": "1", "WORLD_SIZE": "2"})
    assert res.returncode == 0, res.stderr[-2000:]
    assert res.stdout.strip() == ""
