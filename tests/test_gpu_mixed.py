"""The mixed-precision screen: its FP32 error bounds hold, and its rows equal the FP64 screen's rows exactly (the FP32
work only decides what is certain; everything else is recomputed with the FP64 path's own functions)."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import phygas_gb300 as pg
from phygas_gb300 import synth
from tests import oracle_tools as ot

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(built):
    c = pg.Context(0)
    yield c
    c.close()


def _psd(rng, n, lo, hi, needle_frac):
    Q, _ = np.linalg.qr(rng.normal(size=(n, 3, 3)))
    lam = 10.0 ** rng.uniform(lo, hi, size=(n, 3))
    needle = rng.uniform(size=n) < needle_frac
    lam[needle, 1:] = 0.0                                   # rank-1 covariances: the worst conditioned
    S = np.einsum("nij,nj,nkj->nik", Q, lam, Q)
    return np.stack([S[:, 0, 0], S[:, 0, 1], S[:, 0, 2], S[:, 1, 1], S[:, 1, 2], S[:, 2, 2]], axis=1)


def random_points(n, seed):
    rng = np.random.default_rng(seed)
    t0 = np.column_stack([-8.122 + rng.uniform(-3, 3, n), rng.uniform(-3, 3, n), rng.uniform(-0.5, 0.5, n)])
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    c0 = t0 + d * (10.0 ** rng.uniform(-4.5, 0.3, n))[:, None]
    t1 = t0 + rng.normal(size=(n, 3)) * 0.05
    c1 = c0 + (t1 - t0) + rng.normal(size=(n, 3)) * (10.0 ** rng.uniform(-4, -1, n))[:, None]
    pos = np.concatenate([t0, c0, t1, c1], axis=1)
    S = np.concatenate([_psd(rng, n, -9, 0, 0.15), _psd(rng, n, -10, -3, 0.05)], axis=1)
    R2 = (10.0 ** rng.uniform(-3, -1.7, n)) ** 2
    return pos, S, R2


def test_fp32_draw_error_within_bound(ctx):
    """The FP32 draws of the mixed finish (fast log / cosine / reciprocal square root units with their documented
    worst-case errors) stay within their per-draw bound of the FP64 path's draws: 100,000 random pairs x 512 draws
    x 3 components, separations from 0.1 pc to 3 kpc, covariances from isotropic to needles, sigma 0.1 pc to 1 kpc."""
    rng = np.random.default_rng(5)
    n = 100_000
    m = rng.normal(size=(n, 3)) * (10.0 ** rng.uniform(-4, 0.5, n))[:, None]
    S = _psd(rng, n, -8, 0, 0.3)
    A = S[:, [0, 1, 2, 1, 3, 4, 2, 4, 5]].reshape(n, 3, 3)
    A += np.eye(3) * (1e-9 * (S[:, 0] + S[:, 3] + S[:, 5]))[:, None, None]
    C = np.linalg.cholesky(A)
    L = np.column_stack([C[:, 0, 0], C[:, 1, 0], C[:, 2, 0], C[:, 1, 1], C[:, 2, 1], C[:, 2, 2]])
    r50 = 10.0 ** rng.uniform(-3.5, -2, n)
    fin = np.column_stack([m, L, r50, r50 * 10.0 ** rng.uniform(0.3, 1, n)])
    seeds = rng.integers(0, 2**63, n, dtype=np.uint64) * np.uint64(2) + rng.integers(0, 2, n, dtype=np.uint64)
    ratio = ctx.check_draws(fin, seeds)
    print("draw error / bound: median %.3g, max %.3g" % (np.median(ratio), ratio.max()))
    assert np.all(np.isfinite(ratio)) and ratio.max() <= 1.0, np.sort(ratio)[-5:]


@pytest.mark.parametrize("cut", [25.0, 1e6])
def test_fp32_bounds_hold(ctx, cut):
    """2 million random points, 15 % with rank-1 (needle) star covariances: where the FP32 filter rejects a point
    by the trace bound, the FP64 path rejects it too or finds it above the cut; where its cheap pre-test skips a
    point, the FP64 value is at or above the cut; elsewhere lb <= chi2_64 <= ub (the FP64 path's computed value,
    adjugate rounding included)."""
    pos, S, R2 = random_points(2_000_000, 11 if cut == 25.0 else 12)
    v, lb, ub, rej = ctx.check_bounds(pos, S, R2, cut)
    r = rej == 1
    assert np.all(np.isinf(v[r]) | (v[r] > cut)), np.sort(v[r])[:5]
    sk = rej == 2
    assert np.all(np.isinf(v[sk]) | (v[sk] >= cut)), np.sort(v[sk])[:5]
    print("skipped by the cheap test %.3f" % sk.mean())
    ok = ~r & (v >= 0) & np.isfinite(v)
    lbv, ubv, vv = lb[ok].astype(np.float64), ub[ok].astype(np.float64), v[ok]
    bad = (lbv > vv) | (ubv < vv)
    assert not bad.any(), (np.flatnonzero(bad)[:5], lbv[bad][:5], vv[bad][:5], ubv[bad][:5])
    decided = np.isfinite(ubv)
    width = (ubv[decided] - lbv[decided]) / np.maximum(vv[decided], 1e-30)
    print("rejected %.3f, undecided %.4f, median relative width %.2e" % (r.mean(), 1 - decided.mean(),
                                                                         np.median(width)))
    assert decided.mean() > 0.5


def test_mixed_rows_identical_to_fp64(ctx, golden):
    """The reference's 2,000-star `screen` profile: every row of the mixed path equals the FP64 path's, bit for
    bit (chi2, argmin point, segment fraction, distances, sigma, speed, p_r50, p_rtot)."""
    clusters, stars = pg.read_clusters(golden["clusters"]), pg.read_targets(golden["screen"])
    ctx.set_clusters(clusters)
    ps0, sig, pre = pg.draw_targets(stars)
    tmax = max(c.tmax_myr for c in clusters)
    r64 = ctx.screen(ps0, sig, pre, tmax, 25.0, pg.PGX_FP64)
    r32 = ctx.screen(ps0, sig, pre, tmax, 25.0, pg.PGX_MIXED)
    st = ctx.stats()
    assert len(r64) == len(r32) > 100000
    assert r64.tobytes() == r32.tobytes()
    print("kept %d, candidates %d, rechecked draws %d" % (len(r32), st["candidates"], st["rechecked_draws"]))


def test_cli_control_run_mixed_equals_fp64(built):
    """The drop-in phygas_screen with the chance-alignment `control` switch (velocities of the star nt/2 lines
    away): identical stdout in both precisions, on 600 synthetic stars x 4,087 clusters."""
    with tempfile.TemporaryDirectory() as d:
        cp, tp = synth.write_workload(d, "screen", 600, 1002)
        outs = []
        for prec in ("fp64", "mixed"):
            env = dict(os.environ, PHYGAS_PRECISION=prec)
            outs.append(subprocess.run([pg.SCREEN_CLI, cp, tp, "25", "64", "2", "control"], env=env,
                                       stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, check=True).stdout)
    assert outs[0] == outs[1]
    assert len(outs[0].splitlines()) > 1000


def test_block_test_is_sound(built):
    """The filter's block test (one test for eight points of a pair; PHYGAS_SCAN_BLOCKS=1) on the tracks of 768
    synthetic stars x 4,087 clusters of the benchmark workload: every point of every block it settles has the FP64
    path's chi2 >= the cut (pgx_check_blocks evaluates each in FP64), at three cuts; and it settles blocks."""
    with tempfile.TemporaryDirectory() as d:
        cp, tp = synth.write_workload(d, "screen", 768, 1001)
        clusters, stars = pg.read_clusters(cp), pg.read_targets(tp)
    tmax = max(c.tmax_myr for c in clusters)
    old = os.environ.get("PHYGAS_SCAN_BLOCKS")
    os.environ["PHYGAS_SCAN_BLOCKS"] = "1"
    try:
        with pg.Context(0) as c:
            c.set_clusters(clusters)
            c.set_split(0)
            c.stage(*pg.draw_targets(stars))
            got = {cut: c.check_blocks(tmax, cut) for cut in (9.0, 25.0, 100.0)}
    finally:
        if old is None:
            os.environ.pop("PHYGAS_SCAN_BLOCKS", None)
        else:
            os.environ["PHYGAS_SCAN_BLOCKS"] = old
    for cut, r in got.items():
        assert r["violations"] == 0 and r["point_violations"] == 0, (cut, r)
        assert r["points"] > 0 and r["settled"] <= r["settleable"], (cut, r)
    assert got[25.0]["settled"] > 0.3 * got[25.0]["tested"], got


def test_block_test_changes_no_row(built):
    """The same chunk with the block test and with every point walked (PHYGAS_SCAN_BLOCKS=0): identical rows."""
    with tempfile.TemporaryDirectory() as d:
        cp, tp = synth.write_workload(d, "screen", 512, 1002)
        clusters, stars = pg.read_clusters(cp), pg.read_targets(tp)
    tmax = max(c.tmax_myr for c in clusters)
    draws = pg.draw_targets(stars)
    rows = {}
    old = os.environ.get("PHYGAS_SCAN_BLOCKS")
    try:
        for flag in ("1", "0"):
            os.environ["PHYGAS_SCAN_BLOCKS"] = flag
            with pg.Context(0) as c:
                c.set_clusters(clusters)
                rows[flag] = c.screen(*draws, tmax, 25.0, pg.PGX_MIXED)
                if flag == "1":
                    rows["fp64"] = c.screen(*draws, tmax, 25.0, pg.PGX_FP64)
    finally:
        if old is None:
            os.environ.pop("PHYGAS_SCAN_BLOCKS", None)
        else:
            os.environ["PHYGAS_SCAN_BLOCKS"] = old
    assert len(rows["1"]) > 1000
    assert rows["1"].tobytes() == rows["0"].tobytes() == rows["fp64"].tobytes()


def test_screen_autotuner_keeps_the_rows(built):
    """pgx_tune_screen times every launch shape of the block filter on the staged chunk and keeps the fastest; the
    rows after tuning are the rows before."""
    with tempfile.TemporaryDirectory() as d:
        cp, tp = synth.write_workload(d, "screen", 512, 1006)
        clusters, stars = pg.read_clusters(cp), pg.read_targets(tp)
    tmax = max(c.tmax_myr for c in clusters)
    with pg.Context(0) as c:
        c.set_clusters(clusters)
        draws = pg.draw_targets(stars)
        before = c.screen(*draws, tmax)
        c.stage(*draws)
        best, table = c.tune_screen(tmax)
        assert 0 <= best < len(table) and all(ms > 0 for _, ms in table)
        after = c.screen(*draws, tmax)
    assert before.tobytes() == after.tobytes()


def test_staged_filter_changes_no_row(built):
    """The block filter with each cluster's data copied into shared memory by bulk copies (PHYGAS_SCAN_TMA=1): the
    same rows as the filter reading the cluster table through the cache."""
    with tempfile.TemporaryDirectory() as d:
        cp, tp = synth.write_workload(d, "screen", 512, 1007)
        clusters, stars = pg.read_clusters(cp), pg.read_targets(tp)
    tmax = max(c.tmax_myr for c in clusters)
    draws = pg.draw_targets(stars)
    rows = {}
    old = os.environ.get("PHYGAS_SCAN_TMA")
    try:
        for flag in ("0", "1"):
            os.environ["PHYGAS_SCAN_TMA"] = flag
            with pg.Context(0) as c:
                c.set_clusters(clusters)
                rows[flag] = c.screen(*draws, tmax, 25.0, pg.PGX_MIXED)
    finally:
        if old is None:
            os.environ.pop("PHYGAS_SCAN_TMA", None)
        else:
            os.environ["PHYGAS_SCAN_TMA"] = old
    assert len(rows["0"]) > 1000
    assert rows["0"].tobytes() == rows["1"].tobytes()
