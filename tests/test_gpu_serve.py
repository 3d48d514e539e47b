"""The request loop (pgx_server_*): jobs that run together on several slots give exactly the results they give alone,
screen jobs give exactly pgx_screen's rows, pair jobs pgx_pair's results, and the device-memory budget limits how many
jobs run at once."""
import numpy as np
import pytest

import phygas_gb300 as pg
from tests import oracle_tools as ot

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def inputs(built):
    g = ot.golden_inputs()
    return pg.read_clusters(g["clusters"]), pg.read_targets(g["screen"]), pg.read_targets(g["pulsar"])


def _mix(clusters, stars, pulsars):
    return [(pg.PGX_JOB_SCREEN, stars[0:400], dict(precision=pg.PGX_MIXED)),
            (pg.PGX_JOB_CONTROL, stars[400:700], dict(precision=pg.PGX_MIXED)),
            (pg.PGX_JOB_PAIRS, pulsars[0:1], dict(n_clones=40)),
            (pg.PGX_JOB_SCREEN, stars[700:900], dict(precision=pg.PGX_FP64)),
            (pg.PGX_JOB_SCREEN, stars[900:1500], dict(precision=pg.PGX_MIXED, p_min=0.0))]


def test_same_results_alone_and_in_the_mix(inputs):
    clusters, stars, pulsars = inputs
    jobs = _mix(clusters, stars, pulsars)
    with pg.Server(clusters, slots=3) as srv:
        ids = [srv.submit(k, t, **kw) for k, t, kw in jobs]
        mixed = [srv.wait(i) for i in ids]
        rows0 = srv.rows(ids[0])
        pairs2 = srv.pairs(ids[2])
        st = srv.stats()
    assert all(r["status"] == 0 for r in mixed), mixed
    assert st["max_running"] >= 2 and st["finished"] == len(jobs)
    for r in mixed:
        assert r["t_submit"] <= r["t_start"] <= r["t_end"]
    with pg.Server(clusters, slots=1) as srv:
        alone = []
        for k, t, kw in jobs:
            alone.append(srv.wait(srv.submit(k, t, **kw)))
    for a, b in zip(mixed, alone):
        assert (a["digest"], a["n_out"], a["work"]) == (b["digest"], b["n_out"], b["work"])
    # the screen job's rows are pgx_screen's rows with p_r50 >= 0.001; the pair job's results pgx_pair's
    tmax = max(c.tmax_myr for c in clusters)
    with pg.Context(0) as ctx:
        ctx.set_clusters(clusters)
        want = ctx.screen(*pg.draw_targets(stars[0:400]), tmax, 25.0)
        want = want[want["p_r50"] >= 0.001]
        assert rows0.tobytes() == want.tobytes()
        ti, ci = pg.prefilter_pairs(pulsars[0:1], clusters)
        res = ctx.pair(*pg.draw_pair_batch(pulsars[0:1], ti, clusters, ci, 40, 0.05))
        assert np.array_equal(pairs2[1], ci) and pairs2[0].tobytes() == res.tobytes()


def test_memory_budget_admits_one_job_at_a_time(inputs):
    clusters, stars, _ = inputs
    with pg.Server(clusters, slots=3, hbm_budget_gb=1e-6) as srv:
        ids = [srv.submit(pg.PGX_JOB_SCREEN, stars[i * 200:(i + 1) * 200]) for i in range(4)]
        res = [srv.wait(i) for i in ids]
        st = srv.stats()
    assert all(r["status"] == 0 for r in res)
    assert st["max_running"] == 1
    order = sorted(res, key=lambda r: r["t_start"])
    assert all(a["t_end"] <= b["t_start"] for a, b in zip(order, order[1:]))


def test_bounded_wait_times_out_then_the_job_completes(inputs):
    """pgx_server_wait_for: PGX_E_TIMEOUT (TimeoutError) while a job runs, the result once it has finished."""
    clusters, stars, pulsars = inputs
    with pg.Server(clusters, slots=1) as srv:
        jid = srv.submit(pg.PGX_JOB_PAIRS, pulsars[0:1], n_clones=1000)
        with pytest.raises(TimeoutError):
            srv.wait(jid, timeout=0.001)
        done = srv.wait(jid)
        again = srv.wait(jid, timeout=0.001)
    assert done["status"] == 0 and done["n_out"] > 0
    assert again == done
