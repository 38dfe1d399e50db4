"""`bench.py --impl reference`: the CPU arm's JSON line and its rank rule.

The reference arm times the FP64 oracle port of the reference's
back-projection (BPA_SAR.m:177-197, linear interpolation) on the host cores.
It runs here on the small workload (512 pulses x 1024 samples, 512^2 image,
one timed step, about 2 s on 8 cores): one JSON line carrying the contract's
keys, with `cpu_baseline` and `e2e` describing the same run (no host-device
copies); under torchrun every rank but 0 exits 0 without work or output.
"""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CMD = [sys.executable, "bench.py", "--impl", "reference", "--size", "small", "--steps", "1", "--warmup", "0"]


def run(env_extra):
    env = dict(os.environ, **env_extra)
    return subprocess.run(CMD, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)


def test_reference_line():
    out = run({"RANK": "0"})
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout
    d = json.loads(lines[0])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["metric"] == "BP Gpix*pulse/s" and d["unit"] == "Gpix*pulse/s"
    assert d["value"] > 0 and d["ms_per_step"] > 0 and d["higher_is_better"] is True
    assert d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 0 and d["vs_baseline"] is None
    assert "512 pulses x 1024 samples" in d["config"]["workload"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert cb["unit"] == d["unit"] and "pulses" in cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
    # the timed updates per step agree with the sampled tile and the rate
    w, h = d["config"]["sample_tile"]
    assert abs(w * h * 512 / (d["ms_per_step"] * 1e-3) / 1e9 - d["value"]) <= 1e-9 * d["value"] + 1e-12


def test_other_ranks_exit_quietly():
    out = run({"RANK": "1", "WORLD_SIZE": "2"})
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.strip() == ""
