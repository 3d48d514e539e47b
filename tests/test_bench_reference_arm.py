"""bench.py's reference arm (the reference's CPU algorithm, the pinned oracle, on the host cores) prints the one JSON
line the benchmark contract asks for, with the metric, unit and workload of the GPU arm's line."""
import json
import os
import subprocess
import sys

from tests import oracle_tools as ot

KEYS = {"impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
        "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"}


def test_reference_arm_line(built):
    env = dict(os.environ, PYTHONPATH=ot.REPO)
    r = subprocess.run([sys.executable, os.path.join(ot.REPO, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], cwd=ot.REPO, env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert KEYS <= set(d), KEYS - set(d)
    assert d["impl"] == "reference" and d["metric"] == "pairs/s" and d["unit"] == "pairs/s" and d["value"] > 0
    assert d["higher_is_better"] is True and d["n_gpus"] == 1
    assert d["config"]["stars"] == 20000 and d["config"]["clusters"] == 4087
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
