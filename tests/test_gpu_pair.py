"""GPU parity of the pair Monte Carlo: per-clone closest approaches, the warp-shuffle quantile reduction (bit-exact
on identical inputs), the 1 pulsar x 64 cluster x 200 clone x 400 step workload, and the reference's published row
hash on its own `pulsar` profile through the drop-in CLI."""
import ctypes as C
import gzip
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


def ref_pairs(name):
    with gzip.open(os.path.join(ot.GOLDEN, "ref_dump_%s.txt.gz" % name), "rt") as f:
        return ot.parse_pair_dump(f.read())


def test_reduction_bit_exact(built, golden):
    """ph_pair_reduce on the GPU, fed the reference's own per-clone results: the reference's PhResult bit for bit
    (sorted quantiles with linear interpolation, strict < fractions)."""
    L = pg.lib()
    L.ph_pair_reduce.argtypes = [C.POINTER(pg.PhCluster), C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                 C.POINTER(C.c_double), C.POINTER(pg.PhResult)]
    clusters = pg.read_clusters(golden["clusters"])
    for name in ("pair_pulsar", "pair_star"):
        for p in ref_pairs(name):
            cl = np.array(p["clones"]).reshape(-1, 3)
            b, t, v = (np.ascontiguousarray(cl[:, q]) for q in range(3))
            res = pg.PhResult()
            L.ph_pair_reduce(C.byref(clusters[p["cluster"]]), p["m"], pg._ptr(b), pg._ptr(t), pg._ptr(v),
                             C.byref(res))
            assert res.n == p["res"]["n"]
            for k, want in p["res"].items():
                assert getattr(res, k) == want, (name, p["cluster"], k)


def test_reduction_large_pairs(ctx):
    """Pairs of 1,000 (one warp, registers and shuffles), 3,000 clones (shared-memory sort) and more than 16,384
    (radix selection from global memory; the reference has no limit) reduce exactly like a sort on the host, ties
    included."""
    rng = np.random.default_rng(5)
    for m in (1, 31, 200, 1000, 1024, 1025, 3000, 16384, 16385, 70001):
        cl = np.abs(rng.normal(size=(3, m))) * np.array([[1e-3], [10.0], [0.05]])
        if m > 3000:                     # repeated values: ties at the order statistics
            cl[:, ::7] = cl[:, :1]
        b, t, v = cl
        L = pg.lib()
        L.ph_pair_reduce.argtypes = [C.POINTER(pg.PhCluster), C.c_int, C.POINTER(C.c_double),
                                     C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(pg.PhResult)]
        c = pg.PhCluster()
        c.r50_pc, c.rtot_pc = 0.5, 1.5
        res = pg.PhResult()
        L.ph_pair_reduce(C.byref(c), m, pg._ptr(np.ascontiguousarray(b)), pg._ptr(np.ascontiguousarray(t)),
                         pg._ptr(np.ascontiguousarray(v)), C.byref(res))
        O = C.CDLL(ot.ORACLE_LIB)
        O.ph_pair_reduce.argtypes = L.ph_pair_reduce.argtypes
        want = pg.PhResult()
        O.ph_pair_reduce(C.byref(c), m, pg._ptr(np.ascontiguousarray(b)), pg._ptr(np.ascontiguousarray(t)),
                         pg._ptr(np.ascontiguousarray(v)), C.byref(want))
        for k, _ in pg.PhResult._fields_:
            assert getattr(res, k) == getattr(want, k), (m, k)


def _check_pairs(res, clones, pairs, off):
    worst = 0.0
    for q, p in enumerate(pairs):
        o = p["res"]
        r = res[q]
        assert r["n"] == o["n"]
        for k in ("f_r50", "f_rtot"):
            assert abs(r[k] - o[k]) <= ot.PROB_TOL, (q, k, r[k], o[k])
        for k in ("d05", "d50", "d95", "t05", "t50", "t95", "v05", "v50", "v95"):
            worst = max(worst, ot.rel_err(r[k], o[k]) if o[k] else abs(r[k]))
        if clones is not None:
            ref = np.array(p["clones"])
            got = clones[:, off[q]:off[q + 1]].T
            assert np.all(np.abs(got[:, 0] - ref[:, 0]) <= ot.REL_TOL * ref[:, 0] + 1e-12), q
    return worst


def test_clones_match_oracle(ctx):
    """The reference's own clone draws traced on the GPU: closest approach, time and speed per clone and the
    quantiles within 1e-6 relative, fractions identical."""
    for name in ("pair_pulsar", "pair_star"):
        pairs = ref_pairs(name)
        off = np.concatenate([[0], np.cumsum([p["m"] for p in pairs])]).astype(np.int32)
        ps = np.concatenate([np.array(p["ps"]).ravel() for p in pairs])
        steps = np.array([p["steps"] for p in pairs], np.int32)
        dt = np.array([p["dt"] for p in pairs])
        cls = pg.read_clusters(ot.golden_inputs()["clusters"])
        r50 = np.array([cls[p["cluster"]].r50_pc for p in pairs])
        rt = np.array([cls[p["cluster"]].rtot_pc for p in pairs])
        res, clones = ctx.pair(off, ps, steps, dt, r50, rt, want_clones=True)
        worst = _check_pairs(res, clones, pairs, off)
        assert worst <= ot.REL_TOL, (name, worst)


def test_pair64_workload_matches_oracle(ctx):
    """1 synthetic pulsar x 64 clusters x 200 clones x 400 steps (the plain FP64 ph_pair configuration)."""
    with tempfile.TemporaryDirectory() as d:
        cp, tp = synth.write_workload(d, "pair64", 1, 1000)
        out = ot.run([ot.ORACLE_DUMP, "pair", cp, tp, "0", "0", "64", "200", "0.05"])
        pairs = ot.parse_pair_dump(out)
        targets, clusters = pg.read_targets(tp), pg.read_clusters(cp)
        off, ps, steps, dt, r50, rt = pg.pair_draws(targets, clusters, [(0, i) for i in range(64)], 200)
    assert all(s == 400 for s in steps)
    for q, p in enumerate(pairs):
        assert np.array_equal(ps[12 * off[q]:12 * off[q + 1]], np.array(p["ps"]).ravel())
    res, clones = ctx.pair(off, ps, steps, dt, r50, rt, want_clones=True)
    worst = _check_pairs(res, clones, pairs, off)
    assert worst <= ot.REL_TOL, worst
    st = ctx.stats()
    assert st["clone_steps"] == 64 * 200 * 400 and st["kernels"] >= 1


def test_pulsar_profile_published_hash_via_cli(built, golden):
    """phygas_cli (the drop-in CLI) on the reference's `pulsar` profile: the published hash 73bd8776bd66."""
    out = subprocess.run([pg.PAIR_CLI, golden["clusters"], golden["pulsar"], "100", "0.05"], stdout=subprocess.PIPE,
                         stderr=subprocess.PIPE, text=True, check=True).stdout
    rows = [" ".join(ln.split()[:15]) + "\n" for ln in out.splitlines()]
    gold = ot.golden_rows("pulsar")
    if (ot.rows_hash(rows), len(rows)) != ot.PUBLISHED["pulsar"]:
        diff = [(a, b) for a, b in zip(rows, gold) if a != b][:5]
        pytest.fail("rows %d vs %d; first differences %r" % (len(rows), len(gold), diff))


def test_every_launch_shape_gives_the_same_bits(ctx):
    """The autotuner's launch shapes (warps per block x clones per lane) of the graph-captured clone kernel give
    identical results on an uneven batch (clone counts 1..1000), the tuner keeps one shape, pgx_pair then reproduces
    its results, and the clones match the oracle's."""
    rng = np.random.default_rng(4)
    with tempfile.TemporaryDirectory() as d:
        cp, tp = synth.write_workload(d, "pair64", 2, 1000)
        targets, clusters = pg.read_targets(tp), pg.read_clusters(cp)
        ti = np.repeat(np.arange(2), 20).astype(np.int32)
        ci = rng.integers(0, len(clusters), 40).astype(np.int32)
        ncl = rng.choice([1, 31, 33, 200, 500, 1000], 40).astype(np.int32)
        ncl[7] = 500
        batch = pg.draw_pair_batch(targets, ti, clusters, ci, ncl, 0.05)
        checks = {q: ot.parse_pair_dump(ot.run([ot.ORACLE_DUMP, "pair", cp, tp, str(ti[q]), str(ci[q]),
                                                str(ci[q] + 1), str(ncl[q]), "0.05"]))[0] for q in (0, 7, 39)}
    best, table = ctx.tune_pair(*batch)
    assert 0 <= best < len(table) and all(t > 0 for _, _, _, t in table)
    res, clones = ctx.pair(*batch, want_clones=True)
    again = ctx.pair(*batch)
    assert res.tobytes() == again.tobytes()
    off = batch[0]
    for q, p in checks.items():
        assert off[q + 1] - off[q] == p["m"]
        ref = np.array(p["clones"])
        got = clones[:, off[q]:off[q + 1]].T
        assert np.all(np.abs(got - ref) <= ot.REL_TOL * np.abs(ref) + 1e-12), q
    print("launch shapes:", table, "chosen", table[best][:3])


def test_pipelined_pair_targets_and_capped_grid_give_the_same_bits(ctx):
    """pgx_pair_targets (host draws of each batch of pairs overlapping the GPU's tracing of the one before, in batches
    of 7 pairs here) gives the bits of pgx_draw_pair_batch + pgx_pair on the whole list, also with the persistent
    clone kernel capped at one block per SM (pgx_pair_blocks, the request loop's setting)."""
    rng = np.random.default_rng(5)
    with tempfile.TemporaryDirectory() as d:
        cp, tp = synth.write_workload(d, "pair64", 3, 1001)
        targets, clusters = pg.read_targets(tp), pg.read_clusters(cp)
    ti = rng.integers(0, 3, 40).astype(np.int32)
    ci = rng.integers(0, len(clusters), 40).astype(np.int32)
    ncl = rng.choice([0, 1, 33, 200, 1000, 1500], 40).astype(np.int32)
    want = ctx.pair(*pg.draw_pair_batch(targets, ti, clusters, ci, ncl, 0.05))
    got = ctx.pair_targets(targets, ti, clusters, ci, ncl, 0.05, batch_pairs=7)
    assert got.tobytes() == want.tobytes()
    st = ctx.stats()
    assert st["pairs"] == 40 and st["clones"] == int(ncl.sum())
    ctx.pair_blocks(1)
    try:
        assert ctx.pair_targets(targets, ti, clusters, ci, ncl, 0.05).tobytes() == want.tobytes()
    finally:
        ctx.pair_blocks(0)


def test_live_cap_gives_the_same_bits(ctx):
    """pgx_pair_blocks_while (the request loop's setting): batches launched while the flag is set keep to one block per
    SM, the others take the whole GPU; the results are the same bits either way, and after the flag changes between
    calls (both captured graphs in use)."""
    import ctypes
    rng = np.random.default_rng(6)
    with tempfile.TemporaryDirectory() as d:
        cp, tp = synth.write_workload(d, "pair64", 3, 1001)
        targets, clusters = pg.read_targets(tp), pg.read_clusters(cp)
    ti = rng.integers(0, 3, 30).astype(np.int32)
    ci = rng.integers(0, len(clusters), 30).astype(np.int32)
    ncl = rng.choice([0, 1, 64, 500, 1024], 30).astype(np.int32)
    batch = pg.draw_pair_batch(targets, ti, clusters, ci, ncl, 0.05)
    want = ctx.pair(*batch)
    busy = ctypes.c_int(1)
    ctx.pair_blocks_while(1, busy)
    try:
        for flag in (1, 0, 1, 0):
            busy.value = flag
            assert ctx.pair(*batch).tobytes() == want.tobytes(), flag
            assert ctx.pair_targets(targets, ti, clusters, ci, ncl, 0.05, batch_pairs=11).tobytes() == want.tobytes()
    finally:
        ctx.pair_blocks_while(0, None)
