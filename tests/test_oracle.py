"""The oracle is pinned to the reference: raw values bit for bit, and the published row hashes."""
import gzip
import json
import os

import pytest

from tests import oracle_tools as ot

with open(os.path.join(ot.GOLDEN, "golden.json")) as f:
    GOLDEN_INFO = json.load(f)


@pytest.mark.parametrize("name", sorted(k[len("ref_dump_"):] for k in GOLDEN_INFO["commands"]
                                        if k.startswith("ref_dump_")))
def test_oracle_equals_reference_raw_values(golden, name):
    """oracle/dump_main.c on the oracle gives the reference build's output byte for byte (C99 hex floats)."""
    args = GOLDEN_INFO["commands"]["ref_dump_" + name].split()
    files = {"C": golden["clusters"], "S": golden["screen"], "P": golden["pulsar"]}
    out = ot.run([ot.ORACLE_DUMP] + [files.get(a, a) for a in args])
    with gzip.open(os.path.join(ot.GOLDEN, "ref_dump_%s.txt.gz" % name), "rt") as f:
        want = f.read()
    assert out == want


def test_published_hashes_recorded():
    for prof, (h, n) in ot.PUBLISHED.items():
        assert GOLDEN_INFO["published"][prof]["sha1_12"] == h
        assert GOLDEN_INFO["published"][prof]["rows"] == n
        rows = ot.golden_rows(prof)
        assert (ot.rows_hash(rows), len(rows)) == (h, n)


def test_oracle_screen_profile_hash(golden):
    """2,000 stars x 4,087 clusters: the published hash 3e860a4f0e51 (6,387 rows)."""
    slices = [(j, j + 125, 0, 4087) for j in range(0, 2000, 125)]
    rows = ot.wu_rows(golden["clusters"], golden["screen"], slices)
    assert (ot.rows_hash(rows), len(rows)) == ot.PUBLISHED["screen"]


def test_oracle_pulsar_profile_hash(golden):
    """1 pulsar x 4,087 clusters x 100 clones: the published hash 73bd8776bd66 (4,042 rows)."""
    step = 256
    slices = [(0, 1, i, min(i + step, 4087)) for i in range(0, 4087, step)]
    rows = ot.wu_rows(golden["clusters"], golden["pulsar"], slices)
    assert (ot.rows_hash(rows), len(rows)) == ot.PUBLISHED["pulsar"]
