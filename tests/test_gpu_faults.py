"""Failure paths of the pgx_* layer, made on the host: the context's N-th device allocation reports out-of-memory
(PHYGAS_FAIL_ALLOC_AT=N at pgx_open, the allocation never reaching the device).  The entry point that made it
returns PGX_E_NOMEM with a message; the context stays usable, and its next calls give the same results as a context
that never failed.  No GPU fault is made: the failure is a return code."""
import os
import tempfile

import numpy as np
import pytest

import phygas_gb300 as pg
from phygas_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def work(built):
    with tempfile.TemporaryDirectory() as d:
        cp, tp = synth.write_workload(d, "screen", 96, 1005)
        clusters, stars = pg.read_clusters(cp), pg.read_targets(tp)
    tmax = max(c.tmax_myr for c in clusters)
    draws = pg.draw_targets(stars)
    ti, ci = np.zeros(6, np.int32), np.arange(6, dtype=np.int32)
    batch = pg.draw_pair_batch(stars, ti, clusters, ci, 50)
    with pg.Context(0) as c:
        c.set_clusters(clusters)
        want = c.screen(*draws, tmax, 25.0, pg.PGX_MIXED)
        want_pair = c.pair(*batch)
    return dict(clusters=clusters, draws=draws, tmax=tmax, rows=want, batch=batch, res=want_pair)


def _ctx_failing_at(n):
    old = os.environ.get("PHYGAS_FAIL_ALLOC_AT")
    os.environ["PHYGAS_FAIL_ALLOC_AT"] = str(n)
    try:
        return pg.Context(0)
    finally:
        if old is None:
            os.environ.pop("PHYGAS_FAIL_ALLOC_AT", None)
        else:
            os.environ["PHYGAS_FAIL_ALLOC_AT"] = old


@pytest.mark.parametrize("n", [1, 2, 5, 9, 14, 20, 26])
def test_out_of_memory_is_reported_and_the_context_recovers(work, n):
    """The injected failure surfaces as PGX_E_NOMEM (GpuError "out of device memory ... injected") from whichever
    call made the n-th allocation -- the cluster table, the screen or the pair batch -- and the same calls then
    succeed on the same context with the results of a context that never failed."""
    ctx = _ctx_failing_at(n)
    failed = []
    try:
        for _ in range(2):
            try:
                ctx.set_clusters(work["clusters"])
                rows = ctx.screen(*work["draws"], work["tmax"], 25.0, pg.PGX_MIXED)
                res = ctx.pair(*work["batch"])
                break
            except pg.GpuError as e:
                assert "out of device memory" in str(e) and "injected" in str(e), e
                failed.append(str(e))
        else:
            pytest.fail("the calls failed twice")
        assert rows.tobytes() == work["rows"].tobytes()
        assert res.tobytes() == work["res"].tobytes()
    finally:
        ctx.close()
    assert len(failed) == 1, failed             # the n-th allocation failed once, the retry went through


def test_no_injection_without_the_variable(work):
    with pg.Context(0) as ctx:
        ctx.set_clusters(work["clusters"])
        rows = ctx.screen(*work["draws"], work["tmax"], 25.0, pg.PGX_MIXED)
    assert rows.tobytes() == work["rows"].tobytes()
