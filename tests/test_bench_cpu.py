"""The bench's reference arm (the oracle port timed on the host cores) keeps the JSON-line
contract: one line with the metric of the GPU arm, a cpu_baseline describing the run and an
e2e entry with no host-device traffic."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "3", "--warmup", "3"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config"):
        assert k in d, k
    assert d["steps"] == 3 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["unit"] == "particle-steps/s" and d["higher_is_better"] is True and d["value"] > 0
    assert d["config"]["workload"] == "es_pic_2049x1025_64M"
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"] and cb["kind"] in ("port", "reference")
    assert cb["cores"] >= 1 and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    ps = d["poisson"]
    assert ps["ms_per_solve"] > 0 and ps["newton_it"] >= 1 and ps["residual"] < 1e-5
    dj = d["dsmc"]
    assert dj["workload"] == "dsmc_jet_513x257_zr" and dj["value"] > 0
    assert dj["collisions_per_step"] > 0 and dj["dsmc_ms_per_step"] > 0
