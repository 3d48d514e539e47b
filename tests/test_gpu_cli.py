"""The drop-in phygas_screen CLI against the reference's own phygas_screen (compiled from its sources, outputs
committed as tests/golden/cli_*.txt.gz by tests/golden/make_golden.py) on a seeded synthetic workload: the same
stdout bytes for the default arguments, the chance-alignment control run and other chi2_max / n_samp / r_kernel, in
both precisions -- the screen, the control transform and the GPU row writer end to end."""
import gzip
import hashlib
import json
import os
import subprocess
import tempfile

import pytest

import phygas_gb300 as pg
from phygas_gb300 import synth

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
# the workload and cases of tests/golden/make_golden.py (CLI_STARS, CLI_CLUSTERS, CLI_SEED, CLI_CASES)
INFO = json.load(open(os.path.join(GOLDEN, "golden.json")))["cli"]
CASES = sorted(INFO)


def _expected(name):
    with gzip.open(os.path.join(GOLDEN, "cli_%s.txt.gz" % name), "rb") as f:
        return f.read()


def test_cli_fixtures_are_intact():
    """The committed reference outputs match the row counts and hashes recorded when they were made."""
    for name in CASES:
        out = _expected(name)
        assert out.count(b"\n") == INFO[name]["rows"] > 1000
        assert hashlib.sha1(out).hexdigest()[:12] == INFO[name]["sha1_12"]


@pytest.fixture(scope="module")
def workload(built):
    stars, clusters, seed = 64, 1000, 1005
    assert all(INFO[n]["workload"] == "synth screen %d stars %d clusters seed %d" % (stars, clusters, seed)
               for n in CASES)
    with tempfile.TemporaryDirectory() as d:
        yield synth.write_workload(d, "screen", stars, seed, clusters)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("name", CASES)
def test_cli_stdout_equals_reference_cli(workload, name, precision):
    cp, tp = workload
    env = dict(os.environ, PHYGAS_PRECISION=precision, PHYGAS_CHUNK="24")      # several chunks through the pipeline
    r = subprocess.run([pg.SCREEN_CLI, cp, tp] + INFO[name]["args"], env=env, stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, check=True)
    want = _expected(name)
    if r.stdout != want:
        got, exp = r.stdout.splitlines(), want.splitlines()
        diff = [(a, b) for a, b in zip(got, exp) if a != b][:3]
        pytest.fail("%s/%s: %d lines vs %d; first differences %r" % (name, precision, len(got), len(exp), diff))
