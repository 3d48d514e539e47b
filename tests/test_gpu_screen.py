"""GPU parity of the screen: STM tracks, the chi2 scan, the 512-draw probabilities, the kept-pair sets, and the
reference's published row hash on its own `screen` profile -- for the FP64 path and the mixed-precision path."""
import numpy as np
import pytest

import phygas_gb300 as pg
from tests import oracle_tools as ot

pytestmark = pytest.mark.gpu
PRECISIONS = [pg.PGX_FP64, pg.PGX_MIXED]


@pytest.fixture(scope="module")
def ctx(built):
    c = pg.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def data(golden):
    return dict(clusters=pg.read_clusters(golden["clusters"]), stars=pg.read_targets(golden["screen"]))


def _tracks_close(got, ref, keyfn, n_points):
    worst = np.zeros(3)
    for (i, k), v in ref.items():
        g = got[keyfn(i, k)]
        v = np.array(v)
        worst[0] = max(worst[0], np.max(np.abs(g[:3] - v[:3])))                      # kpc
        worst[1] = max(worst[1], np.max(np.abs(g[3:6] - v[3:6]) / np.abs(v[3:6]).max()))
        worst[2] = max(worst[2], np.max(np.abs(g[6:] - v[6:])) / max(np.abs(v[6:]).max(), 1e-300))
    return worst


def test_stm_tracks_match_oracle(ctx, data, golden):
    """pgx_lin (nominal + 6 neighbour orbits in FP64, S = A Sigma0 A^T) against the oracle's ph_lin_cluster /
    ph_lin_target: positions within 1e-9 kpc, velocities and covariances within 1e-6 relative."""
    for which, objs, n in (("c", data["clusters"], 24), ("t", data["stars"], 3)):
        ref = ot.oracle_lin(golden["clusters"], golden["screen"], which, 0, n)
        if which == "c":
            ps0, sig = pg.draw_clusters(objs[:n])
            npts = np.array([int(np.ceil(o.tmax_myr / 0.5)) + 1 for o in objs[:n]], np.int32)
        else:
            ps0, sig, _ = pg.draw_targets(objs[:n])
            tmax = max(c.tmax_myr for c in data["clusters"])
            npts = np.full(n, int(np.ceil(tmax / 0.5)) + 1, np.int32)
        pos, vel, S = ctx.lin(ps0, sig, npts)
        start = np.concatenate([[0], np.cumsum(npts)[:-1]])
        got = {}
        for i in range(n):
            for k in range(npts[i]):
                r = start[i] + k
                got[(i, k)] = np.concatenate([pos[r], vel[r], S[r]])
        assert len(got) == len(ref)
        w = _tracks_close(got, ref, lambda i, k: (i, k), npts)
        assert w[0] < 1e-9 and w[1] < 1e-6 and w[2] < 1e-6, (which, w)


def _compare_rows(rows, ref, cut=25.0):
    got = {(int(r["star"]), int(r["cluster"])): r for r in rows}
    only_g = set(got) - set(ref)
    only_r = set(ref) - set(got)
    for key in only_g:
        assert abs(got[key]["chi2"] - cut) <= ot.REL_TOL * cut, ("extra pair", key, got[key]["chi2"])
    for key in only_r:
        assert abs(ref[key]["chi2"] - cut) <= ot.REL_TOL * cut, ("missing pair", key, ref[key]["chi2"])
    n_kb = 0
    worst = {}
    for key in set(got) & set(ref):
        g, o = got[key], ref[key]
        if g["kb"] != o["kb"]:
            n_kb += 1
            continue
        for f in ("chi2", "t_myr", "d_nom_pc", "sig_pc", "vrel_kms"):
            e = ot.rel_err(g[f], o[f]) if o[f] != 0 else abs(g[f])
            worst[f] = max(worst.get(f, 0.0), e)
        for f in ("p_r50", "p_rtot"):
            assert abs(g[f] - o[f]) <= ot.PROB_TOL, (key, f, g[f], o[f])
    return len(set(got) & set(ref)), n_kb, worst


@pytest.mark.parametrize("precision", PRECISIONS, ids=["fp64", "mixed"])
def test_screen_rows_match_oracle(ctx, data, golden, precision):
    """8 stars x 4,087 clusters: same kept pairs, chi2 / t / d / sigma / vrel within 1e-6 relative, identical
    p_r50 and p_rtot (counts out of 512), same argmin point."""
    ctx.set_clusters(data["clusters"])
    ps0, sig, pre = pg.draw_targets(data["stars"][:8])
    tmax = max(c.tmax_myr for c in data["clusters"])
    rows = ctx.screen(ps0, sig, pre, tmax, 25.0, precision)
    ref = ot.oracle_screen(golden["clusters"], golden["screen"], 0, 8)
    n, n_kb, worst = _compare_rows(rows, ref)
    assert n > 500
    assert n_kb == 0, n_kb
    for f, e in worst.items():
        assert e <= ot.REL_TOL, (f, e)


def boinc_rows(rows, data, p_min=0.001):
    out = []
    for r in rows:
        if r["p_r50"] < p_min:
            continue
        t, c = data["stars"][r["star"]], data["clusters"][r["cluster"]]
        out.append("%s %s %s %.3f %.3f %.2f %.2f %.4f %.4f %.2f\n" % (
            t.id.decode(), c.name.decode(), c.kind.decode(), r["chi2"], r["t_myr"], r["d_nom_pc"], r["sig_pc"],
            r["p_r50"], r["p_rtot"], r["vrel_kms"]))
    return out


@pytest.mark.parametrize("precision", PRECISIONS, ids=["fp64", "mixed"])
def test_screen_profile_published_hash(ctx, data, precision):
    """The reference's `screen` benchmark profile (2,000 stars x 4,087 clusters, PHYGAS 1 screen 25 64 2 0.001):
    the GPU rows hash to the published 3e860a4f0e51 (6,387 rows)."""
    ctx.set_clusters(data["clusters"])
    ps0, sig, pre = pg.draw_targets(data["stars"])
    tmax = max(c.tmax_myr for c in data["clusters"])
    rows = ctx.screen(ps0, sig, pre, tmax, 25.0, precision)
    lines = boinc_rows(rows, data)
    gold = ot.golden_rows("screen")
    if (ot.rows_hash(lines), len(lines)) != ot.PUBLISHED["screen"]:
        diff = [(a, b) for a, b in zip(lines, gold) if a != b][:5]
        pytest.fail("rows %d vs %d; first differences %r" % (len(lines), len(gold), diff))


def test_screen_into_page_locked_rows(ctx, golden):
    """pgx_screen_into writes the same rows as pgx_screen into a caller buffer (here page-locked, pgx_host_alloc);
    a buffer too small gives PGX_E_LIMIT with the row count, and the rows stay on the device for pgx_screen_fetch."""
    clusters, stars = pg.read_clusters(golden["clusters"]), pg.read_targets(golden["screen"])[:300]
    ctx.set_clusters(clusters)
    tmax = max(c.tmax_myr for c in clusters)
    a, b, c = pg.draw_targets(stars)
    want = ctx.screen(a, b, c, tmax)
    buf = pg.HostRows(len(want) + 10)
    got = ctx.screen_into(a, b, c, tmax, buf)
    assert got.tobytes() == want.tobytes()
    small = np.zeros(max(len(want) // 2, 1), pg.ROW_DTYPE)
    with pytest.raises(pg.GpuError, match="size limit"):
        ctx.screen_into(a, b, c, tmax, small)
    assert ctx.fetch(len(want)).tobytes() == want.tobytes()
    buf.close()


def test_screen_chunks_pipeline_matches_one_screen(ctx, golden):
    """pgx_screen_chunks (host draws, GPU screen and row copies overlapped, emit on the calling thread) gives each
    chunk's rows in order, equal to screening the whole list at once after renumbering the stars; the buffers it
    keeps serve a second call with other chunk sizes; a non-zero emit stops the run with an error."""
    clusters, stars = pg.read_clusters(golden["clusters"]), pg.read_targets(golden["screen"])[:300]
    ctx.set_clusters(clusters)
    tmax = max(c.tmax_myr for c in clusters)
    for prec in PRECISIONS:
        want = ctx.screen(*pg.draw_targets(stars), tmax, 25.0, prec)
        for chunk in (128, 37, 300):
            got, firsts = [], []

            def emit(first, rows):
                r = np.array(rows, copy=True)
                r["star"] += first
                firsts.append(first)
                got.append(r)
            ctx.screen_chunks(stars, chunk, tmax, emit, 25.0, prec)
            assert firsts == list(range(0, len(stars), chunk))
            assert np.concatenate(got).tobytes() == want.tobytes(), (prec, chunk)
    calls = []

    def stop(first, rows):
        calls.append(first)
        return 1 / 0
    with pytest.raises(ZeroDivisionError):
        ctx.screen_chunks(stars, 50, tmax, stop)
    assert calls == [0]
    assert len(ctx.screen(*pg.draw_targets(stars[:40]), tmax)) >= 0      # the context is still usable


def test_screen_chunks_ramp_up(ctx):
    """Against 4,087 clusters a chunk of more than about 1e7 star-cluster pairs is preceded by smaller ones: the first
    chunk of round(1e7 / 4,087) = 2,447 stars, each next one half again as large (integer halves), up to the chunk
    size.  A staged chunk of 9,000 stars is screened in parts that ramp up too (2,447, 4,282, 2,271).  The
    rows, in order and renumbered, equal one screen of the whole list unsplit, in both precisions."""
    from phygas_gb300 import synth
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        cp, tp = synth.write_workload(d, "screen", 9000, 1007)
        clusters, stars = pg.read_clusters(cp), pg.read_targets(tp)
    assert len(clusters) == 4087
    ctx.set_clusters(clusters)
    tmax = max(c.tmax_myr for c in clusters)
    draws = pg.draw_targets(stars)
    for prec in PRECISIONS:
        try:
            ctx.set_split(0)
            whole = ctx.screen(*draws, tmax, 25.0, prec)
        finally:
            ctx.set_split(8192)
        want = ctx.screen(*draws, tmax, 25.0, prec)
        assert ctx.stats()["parts"] == 3
        assert want.tobytes() == whole.tobytes(), prec
        for chunk, firsts_want in ((9000, [0, 2447, 6117]), (4000, [0, 2447, 6117]),
                                   (2000, [0, 2000, 4000, 6000, 8000])):
            got, firsts = [], []

            def emit(first, rows):
                r = np.array(rows, copy=True)
                r["star"] += first
                firsts.append(first)
                got.append(r)
            ctx.screen_chunks(stars, chunk, tmax, emit, 25.0, prec)
            assert firsts == firsts_want, (prec, chunk, firsts)
            assert np.concatenate(got).tobytes() == want.tobytes(), (prec, chunk)


def _lines(rows, stars, clusters, first=0):
    """the reference CLI's line for each row, formatted by Python (exact decimal rounding, as printf)"""
    out = []
    for r in rows:
        t, c = stars[first + int(r["star"])], clusters[int(r["cluster"])]
        out.append("%s %s %s %.3f %.3f %.2f %.2f %.4f %.4f %.2f %.3f %.3f\n" % (
            t.id.decode(), c.name.decode(), c.kind.decode(), r["chi2"], r["t_myr"], r["d_nom_pc"], r["sig_pc"],
            r["p_r50"], r["p_rtot"], r["vrel_kms"], c.age16, c.age84))
    return "".join(out).encode()


def test_screen_chunks_text_is_printf_of_the_rows(ctx, golden):
    """pgx_screen_chunks_text: each chunk's lines, formatted on the GPU, are byte for byte the printf text of the
    rows pgx_screen returns (Python's %-formatting rounds the exact binary value as the C library does)."""
    clusters, stars = pg.read_clusters(golden["clusters"]), pg.read_targets(golden["screen"])[:300]
    ctx.set_clusters(clusters)
    tmax = max(c.tmax_myr for c in clusters)
    rows = ctx.screen(*pg.draw_targets(stars), tmax)
    want = _lines(rows, stars, clusters)
    for chunk in (300, 64):
        got, counts = [], []

        def emit(first, text, n):
            got.append(bytes(text))
            counts.append(n)
        ctx.screen_chunks_text(stars, clusters, chunk, tmax, emit)
        assert sum(counts) == len(rows)
        assert b"".join(got) == want, chunk
    with pytest.raises(pg.GpuError):
        ctx.screen_chunks_text(stars, clusters[:10], 64, tmax, lambda *a: None)     # not the resident table


def test_split_chunk_equals_unsplit(ctx, golden):
    """A staged chunk of at least 8,192 stars is screened in parts (each part's orbits beside the previous part's
    screen, the two track slots in turn): its rows -- star indices across the parts, their order, every field --
    equal the same chunk screened whole through pgx_screen_chunks, in both precisions, for 2, 3 (uneven), 4 and 7
    parts."""
    from phygas_gb300 import synth
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        cp, tp = synth.write_workload(d, "screen", 9001, 1006, 1000)
        clusters, stars = pg.read_clusters(cp), pg.read_targets(tp)
    ctx.set_clusters(clusters)
    tmax = max(c.tmax_myr for c in clusters)
    draws = pg.draw_targets(stars)
    try:
        for prec in PRECISIONS:
            whole = []
            ctx.screen_chunks(stars, len(stars), tmax, lambda first, rows: whole.append(np.array(rows, copy=True)),
                              25.0, prec)
            assert len(whole) == 1 and len(whole[0]) > 10000
            for parts in (2, 3, 4, 7):
                ctx.set_split(8192, parts)
                split = ctx.screen(*draws, tmax, 25.0, prec)
                st = ctx.stats()
                assert split["star"].max() > len(stars) * (parts - 1) // parts      # rows from the last part
                assert split.tobytes() == whole[0].tobytes(), (prec, parts)
                assert st["kept"] == len(split) and st["pairs"] == len(stars) * len(clusters), (prec, parts)
    finally:
        ctx.set_split(8192, 0)
