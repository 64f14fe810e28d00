"""bench.py's reference arm on the host cores (no GPU): the one JSON line of
the bench contract, the CUDA library left unmapped (the arm runs only the
oracle's C restatement of the reference's algorithm), and the other ranks of
a multi-rank launch exiting without work."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import json, sys
sys.argv = ["bench.py", "--impl", "reference", "--log2n", "16", "--steps", "2", "--warmup", "1"]
import bench
rc = bench.main()
maps = open("/proc/self/maps").read()
print("STATUS " + json.dumps({"rc": rc, "capssa_mapped": "libcapssa_gb300" in maps}))
"""


def _run(extra_env=None):
    env = dict(os.environ)
    env.update(extra_env or {})
    r = subprocess.run([sys.executable, "-c", SCRIPT], cwd=ROOT, env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    status = [json.loads(l[7:]) for l in r.stdout.splitlines() if l.startswith("STATUS ")]
    assert len(status) == 1
    return lines, status[0]


def test_reference_arm_prints_the_contract_line():
    lines, status = _run()
    assert status["rc"] == 0
    assert not status["capssa_mapped"]  # only the oracle ran
    assert len(lines) == 1
    d = lines[0]
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference"
    assert d["metric"] == d["unit"] == "Msuffixes/s"
    assert d["steps"] == 2 and d["warmup"] == 1 and d["n_gpus"] == 1
    assert d["higher_is_better"] is True and d["vs_baseline"] is None
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["config"]["n"] == 1 << 16 and "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": "Msuffixes/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_without_work():
    lines, status = _run({"RANK": "1", "LOCAL_RANK": "1", "WORLD_SIZE": "2"})
    assert status["rc"] == 0
    assert lines == []
