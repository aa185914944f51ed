"""bench.py's one-line JSON output carries the keys its reader expects, in
both arms, at a small scale (the full workload is the bench's own run)."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _run(args, timeout):
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], capture_output=True, text=True,
                       timeout=timeout, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [x for x in r.stdout.strip().splitlines() if x.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    return json.loads(lines[0])


BASE_KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
             "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"}


def test_reference_arm_line(lib_built):
    line = _run(["--impl", "reference", "--scale", "0.02", "--steps", "1", "--warmup", "3"], 900)
    assert BASE_KEYS <= set(line)
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["config"]["workload"]
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0


@pytest.mark.gpu
def test_gpu_arm_line(lib_built):
    line = _run(["--scale", "0.05", "--sections", "none", "--no-cpu-baseline", "--steps", "1", "--warmup", "3"], 900)
    assert BASE_KEYS <= set(line) and "impl" not in line
    assert line["value"] > 0 and line["dtype"] == "int32" and line["gpu_launches"] > 0
    r = line["roofline"]
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and r["peak"] > 0
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    e = line["e2e"]
    assert e["value"] > 0 and e["h2d_bytes_per_step"] > 0 and e["d2h_bytes_per_step"] > 0
    assert {"sm_mhz", "sm_max_mhz", "reasons"} <= set(line["clocks"])
    assert line["per_op"] and all(op["ms_mean"] > 0 for op in line["per_op"])
    # the reference arm names the same workload, config for config
    ref = _run(["--impl", "reference", "--scale", "0.05", "--steps", "1", "--warmup", "3"], 900)
    assert ref["config"] == line["config"]
    assert (ref["metric"], ref["unit"], ref["higher_is_better"]) == (line["metric"], line["unit"],
                                                                      line["higher_is_better"])
