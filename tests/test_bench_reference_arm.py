"""bench.py's reference arm on the host cores.

`bench.py --impl reference` times the restated reference CPU path (the oracle, test
infrastructure) on a fixed seeded point sample of the workload and prints one JSON line
with the contract's keys; launched as several ranks, only rank 0 does work and prints.
"""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(env_extra, *args):
    env = dict(os.environ, **env_extra)
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", *args],
                          capture_output=True, text=True, env=env, timeout=600, cwd=ROOT)


def _lines(out):
    return [json.loads(l) for l in out.splitlines() if l.startswith("{")]


def test_reference_arm_prints_the_contract_line():
    r = _run({}, "--steps", "2", "--warmup", "1", "--cpu-points", "24")
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _lines(r.stdout)
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference"
    assert d["metric"] == "walk-steps/s" and d["unit"] == "walk-steps/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 1
    assert d["config"]["workload"] == "mixed_wost_2d"
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert cb["sample"].startswith("fixed seeded sample of 24 of ")
    assert d["e2e"] == {"value": d["value"], "unit": "walk-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_works_on_rank_0_only():
    r = _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}, "--steps", "1", "--warmup", "1",
             "--cpu-points", "8")
    assert r.returncode == 0, r.stderr[-2000:]
    assert _lines(r.stdout) == []
