"""CPU checks of libphygas_gb300: it loads without a GPU, exports every entry point its headers declare, its
records have the C layouts, and its host half (draws, seeds, readers, tracks, prefilter) equals the oracle bit for
bit -- the GPU stages then start from the reference's own inputs."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

import phygas_gb300 as pg
from tests import oracle_tools as ot

HEADERS = [os.path.join(ot.REPO, "include", h) for h in ("phygas.h", "phygas_gb300.h")]


def declared_symbols():
    names = set()
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names.update(re.findall(r"\b((?:ph|pgx)_\w+)\s*\(", text))
        names.update(re.findall(r"extern\s+(?:const\s+)?\w+\s+(\w+)\s*;", text))
    return sorted(names)


def test_library_loads_and_exports_every_declared_symbol(built):
    L = C.CDLL(pg.LIB_PATH)
    missing = [n for n in declared_symbols() if not hasattr(L, n)]
    assert not missing, missing
    assert len(declared_symbols()) >= 40


LAYOUT_PROBE = r"""
#include <stddef.h>
#include <stdio.h>
#include "phygas_gb300.h"
#define S(T) printf(#T " %zu\n", sizeof(T));
#define O(T, f) printf(#T "." #f " %zu\n", offsetof(T, f));
int main(void) {
  S(PhCluster) S(PhTarget) S(PhResult) S(PgxScreenRow) S(PgxStats) S(PhLin) S(PhTrack) S(PhScreen)
  O(PhCluster, kind) O(PhCluster, has_rv) O(PhCluster, r50_pc) O(PhCluster, tmax_myr)
  O(PhTarget, kind) O(PhTarget, has_rv) O(PhTarget, e_rv)
  O(PhResult, d05) O(PhResult, f_rtot) O(PgxScreenRow, sb) O(PgxScreenRow, vrel_kms)
  O(PgxStats, pairs) O(PgxStats, kernels)
  return 0;
}
"""


def test_record_layouts_match_bindings(built):
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "p.c"), os.path.join(d, "p")
        open(src, "w").write(LAYOUT_PROBE)
        subprocess.check_call(["gcc", "-I", os.path.join(ot.REPO, "include"), src, "-o", exe])
        got = dict(ln.split() for ln in subprocess.check_output([exe], text=True).splitlines())
    for name, cls in (("PhCluster", pg.PhCluster), ("PhTarget", pg.PhTarget), ("PhResult", pg.PhResult),
                      ("PgxScreenRow", pg.PgxScreenRow), ("PgxStats", pg.PgxStats)):
        assert int(got[name]) == C.sizeof(cls), name
    for key, val in got.items():
        if "." in key:
            t, f = key.split(".")
            assert getattr(getattr(pg, t), f).offset == int(val), key
    assert int(got["PgxScreenRow"]) == pg.ROW_DTYPE.itemsize
    assert int(got["PhResult"]) == pg.RESULT_DTYPE.itemsize


@pytest.fixture(scope="module")
def both(built):
    O = C.CDLL(ot.ORACLE_LIB)
    O.ph_init()
    return pg.lib(), O


def test_readers_identical(both, golden):
    P, O = both
    for path, T, fn in ((golden["clusters"], pg.PhCluster, "ph_read_clusters"),
                        (golden["screen"], pg.PhTarget, "ph_read_targets"),
                        (golden["pulsar"], pg.PhTarget, "ph_read_targets")):
        pa, pb = C.POINTER(T)(), C.POINTER(T)()
        na = getattr(P, fn)(path.encode(), C.byref(pa))
        getattr(O, fn).argtypes = [C.c_char_p, C.POINTER(C.POINTER(T))]
        nb = getattr(O, fn)(path.encode(), C.byref(pb))
        assert na == nb > 0
        for i in range(na):      # field by field: padding and the bytes after a name's NUL are undefined
            for f, ft in T._fields_:
                va, vb = getattr(pa[i], f), getattr(pb[i], f)
                if ft is C.c_double:
                    va, vb = np.float64(va).tobytes(), np.float64(vb).tobytes()
                assert va == vb, (path, i, f)


def test_seeds_identical(both):
    P, O = both
    O.ph_seed.restype = C.c_uint64
    O.ph_seed.argtypes = [C.c_char_p, C.c_char_p]
    for a, b in ((b"lin", b"SYN_00001"), (b"4000000000000000007", b"SYN_04086"), (b"", b""), (b"x" * 39, b"y")):
        assert P.ph_seed(a, b) == O.ph_seed(a, b)
        assert P.ph_seed(a, b) == pg.lib().ph_seed(a, b)


def test_target_draws_identical(both, golden):
    """ph_lin_target_init (64 draws + 6-D covariance) and the threaded batch draws: bit-identical to the oracle."""
    P, O = both
    stars = pg.read_targets(golden["screen"])[:64]
    ps0, sig, pre = pg.draw_targets(stars, 64, threads=4)
    O.ph_lin_target_init.argtypes = [C.POINTER(pg.PhTarget), C.c_int, C.c_uint64, C.POINTER(C.c_double),
                                     C.POINTER(C.c_double)]
    O.ph_seed.restype = C.c_uint64
    O.ph_seed.argtypes = [C.c_char_p, C.c_char_p]
    for j, t in enumerate(stars):
        a, s = np.zeros(6), np.zeros(36)
        O.ph_lin_target_init(C.byref(t), 64, O.ph_seed(b"lin", t.id), pg._ptr(a), pg._ptr(s))
        assert np.array_equal(a, ps0[j]) and np.array_equal(s, sig[j]), j
        assert pre[j] == pg.lib().pgx_seed_prefix(t.id)


def test_cluster_draws_identical(both, golden):
    """pgx_draw_clusters equals the oracle's draws (ph_sample_cluster) and its covariance arithmetic."""
    P, O = both

    class Rng(C.Structure):
        _fields_ = [("state", C.c_uint64)]

    class PS(C.Structure):
        _fields_ = [("v", C.c_double * 6)]

    O.ph_sample_cluster.argtypes = [C.POINTER(pg.PhCluster), C.POINTER(Rng), C.POINTER(PS)]
    O.ph_seed.restype = C.c_uint64
    O.ph_seed.argtypes = [C.c_char_p, C.c_char_p]
    clusters = pg.read_clusters(golden["clusters"])
    pick = [0, 1, 2, 5, 17, 400, 4086] + [i for i in range(4087) if not clusters[i].has_rv][:5]
    sel = (pg.PhCluster * len(pick))(*[clusters[i] for i in pick])
    ps0, sig = pg.draw_clusters(sel, 64, threads=3)
    for q, c in enumerate(sel):
        nom = PS()
        O.ph_sample_cluster(C.byref(c), None, C.byref(nom))
        g = Rng(O.ph_seed(b"lin", c.name))
        draws = []
        for _ in range(64):
            d = PS()
            if O.ph_sample_cluster(C.byref(c), C.byref(g), C.byref(d)) == 0:
                draws.append(list(d.v))
        cov = [[0.0] * 6 for _ in range(6)]
        for d in draws:
            e = [d[i] - nom.v[i] for i in range(6)]
            for a in range(6):
                for b in range(6):
                    cov[a][b] += e[a] * e[b]
        cov = [[v / len(draws) for v in row] for row in cov]
        assert list(nom.v) == list(ps0[q])
        assert np.array_equal(np.array(cov).ravel(), sig[q]), pick[q]


def test_pair_draws_identical(both, golden):
    """ph_pair_draw (clone start states, steps, dt): bit-identical, for the pulsar and for stars."""
    P, O = both
    clusters = pg.read_clusters(golden["clusters"])
    for tfile, js in ((golden["pulsar"], [0]), (golden["screen"], [3, 11])):
        targets = pg.read_targets(tfile)
        for j in js:
            for i in (0, 7, 123, 4000):
                t, c = targets[j], clusters[i]
                seed = P.ph_seed(t.id, c.name)
                out = []
                for L in (P, O):
                    L.ph_pair_draw.argtypes = [C.POINTER(pg.PhTarget), C.POINTER(pg.PhCluster), C.c_int,
                                               C.c_double, C.c_uint64, C.POINTER(C.c_double), C.POINTER(C.c_int),
                                               C.POINTER(C.c_double)]
                    ps, st, dt = np.zeros(12 * 50), C.c_int(), C.c_double()
                    m = L.ph_pair_draw(C.byref(t), C.byref(c), 50, 0.05, seed, pg._ptr(ps), C.byref(st),
                                       C.byref(dt))
                    out.append((m, st.value, dt.value, ps[:12 * m].tobytes()))
                assert out[0] == out[1], (j, i)


def test_tracks_and_prefilter_identical(both, golden):
    """ph_track_target / ph_track_cluster / ph_prefilter (host): identical tracks and decisions."""
    P, O = both

    class Track(C.Structure):
        _fields_ = [("n", C.c_int), ("pos", C.POINTER(C.c_double)), ("sig_pos", C.c_double),
                    ("sig_vel", C.c_double)]

    clusters = pg.read_clusters(golden["clusters"])
    pulsar = pg.read_targets(golden["pulsar"])[0]
    for L in (P, O):
        L.ph_track_target.argtypes = [C.POINTER(pg.PhTarget), C.c_double, C.c_int, C.c_uint64, C.POINTER(Track)]
        L.ph_track_cluster.argtypes = [C.POINTER(pg.PhCluster), C.c_int, C.c_uint64, C.POINTER(Track)]
        L.ph_prefilter.argtypes = [C.POINTER(Track), C.POINTER(Track), C.POINTER(pg.PhCluster)]
        L.ph_seed.restype = C.c_uint64
        L.ph_seed.argtypes = [C.c_char_p, C.c_char_p]
    tt = [Track(), Track()]
    for L, t in zip((P, O), tt):
        L.ph_track_target(C.byref(pulsar), 100.0, 32, L.ph_seed(b"track", pulsar.id), C.byref(t))
    assert tt[0].n == tt[1].n and (tt[0].sig_pos, tt[0].sig_vel) == (tt[1].sig_pos, tt[1].sig_vel)
    assert C.string_at(tt[0].pos, 24 * tt[0].n) == C.string_at(tt[1].pos, 24 * tt[1].n)
    for i in range(0, 4087, 97):
        c = clusters[i]
        ct = [Track(), Track()]
        dec = []
        for L, t, x in zip((P, O), ct, tt):
            L.ph_track_cluster(C.byref(c), 32, L.ph_seed(b"track", c.name), C.byref(t))
            dec.append(L.ph_prefilter(C.byref(x), C.byref(t), C.byref(c)))
        assert C.string_at(ct[0].pos, 24 * ct[0].n) == C.string_at(ct[1].pos, 24 * ct[1].n), i
        assert dec[0] == dec[1], i


def test_prefilter_pairs_matches_the_oracle(both, golden):
    """pgx_prefilter_pairs (threaded tracks + ph_prefilter) keeps exactly the pairs the oracle's tracks and prefilter
    keep, in (target, cluster) order, for the reference's pulsar against 600 of the golden clusters."""
    P, O = both

    class Track(C.Structure):
        _fields_ = [("n", C.c_int), ("pos", C.POINTER(C.c_double)), ("sig_pos", C.c_double),
                    ("sig_vel", C.c_double)]

    clusters = pg.read_clusters(golden["clusters"])[:600]
    targets = pg.read_targets(golden["pulsar"])[:2]
    ti, ci = pg.prefilter_pairs(targets, clusters)
    O.ph_track_target.argtypes = [C.POINTER(pg.PhTarget), C.c_double, C.c_int, C.c_uint64, C.POINTER(Track)]
    O.ph_track_cluster.argtypes = [C.POINTER(pg.PhCluster), C.c_int, C.c_uint64, C.POINTER(Track)]
    O.ph_prefilter.argtypes = [C.POINTER(Track), C.POINTER(Track), C.POINTER(pg.PhCluster)]
    O.ph_seed.restype = C.c_uint64
    O.ph_seed.argtypes = [C.c_char_p, C.c_char_p]
    tmax = max(c.tmax_myr for c in clusters)
    cts = []
    for c in clusters:
        t = Track()
        O.ph_track_cluster(C.byref(c), 32, O.ph_seed(b"track", c.name), C.byref(t))
        cts.append(t)
    want = []
    for j, tg in enumerate(targets):
        tt = Track()
        O.ph_track_target(C.byref(tg), tmax, 32, O.ph_seed(b"track", tg.id), C.byref(tt))
        want += [(j, i) for i, c in enumerate(clusters) if O.ph_prefilter(C.byref(tt), C.byref(cts[i]), C.byref(c))]
    assert list(zip(ti.tolist(), ci.tolist())) == want
    assert 0 < len(want) < 1200


def test_draw_pair_batch_matches_ph_pair_draw(both, golden):
    """pgx_draw_pair_batch: every pair's clones, steps and dt bit-identical to the oracle's ph_pair_draw with the
    pair's own clone count, packed back to back."""
    P, O = both
    clusters = pg.read_clusters(golden["clusters"])
    targets = list(pg.read_targets(golden["pulsar"])[:1]) + list(pg.read_targets(golden["screen"])[:3])
    rng = np.random.default_rng(2)
    ti = rng.integers(0, len(targets), 40).astype(np.int32)
    ci = rng.integers(0, len(clusters), 40).astype(np.int32)
    ncl = rng.choice([0, 1, 7, 33, 200], 40).astype(np.int32)
    off, ps, steps, dt, r50, rt = pg.draw_pair_batch(targets, ti, clusters, ci, ncl, 0.05)
    O.ph_pair_draw.argtypes = [C.POINTER(pg.PhTarget), C.POINTER(pg.PhCluster), C.c_int, C.c_double, C.c_uint64,
                               C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_double)]
    O.ph_seed.restype = C.c_uint64
    O.ph_seed.argtypes = [C.c_char_p, C.c_char_p]
    for q in range(40):
        t, c = targets[ti[q]], clusters[ci[q]]
        buf, st, d = np.zeros(12 * max(int(ncl[q]), 1)), C.c_int(), C.c_double()
        m = O.ph_pair_draw(C.byref(t), C.byref(c), int(ncl[q]), 0.05, O.ph_seed(t.id, c.name), pg._ptr(buf),
                           C.byref(st), C.byref(d))
        assert off[q + 1] - off[q] == m, q
        assert ps[12 * off[q]:12 * off[q + 1]].tobytes() == buf[:12 * m].tobytes(), q
        assert (steps[q], dt[q], r50[q], rt[q]) == (st.value, d.value, c.r50_pc, c.rtot_pc), q


def test_serving_stream_plan(built, golden):
    """phygas_serve's seeded Poisson stream (its `plan` mode needs no GPU): the same seed gives the same stream,
    inter-arrival times average 1/rate, chunk sizes stay in 1,000..20,000 stars (at most the file), and the job kinds
    come in about 40 / 20 / 40 % (screen / control / pulsar)."""
    import json
    args = [pg.SERVE_CLI, golden["clusters"], golden["screen"], golden["pulsar"], "3000", "2.0", "3", "mixed", "77",
            "plan"]
    a = subprocess.run(args, stdout=subprocess.PIPE, check=True, text=True).stdout
    b = subprocess.run(args, stdout=subprocess.PIPE, check=True, text=True).stdout
    assert a == b
    jobs = [json.loads(x) for x in a.splitlines()]
    t = np.array([j["arrive_s"] for j in jobs])
    assert np.all(np.diff(t) > 0) and abs(np.mean(np.diff(t)) - 0.5) < 0.05
    kinds = [j["kind"] for j in jobs]
    frac = {k: kinds.count(k) / len(kinds) for k in ("screen", "control", "pulsar")}
    assert abs(frac["screen"] - 0.4) < 0.04 and abs(frac["control"] - 0.2) < 0.04 and abs(frac["pulsar"] - 0.4) < 0.04
    n_stars = len(pg.read_targets(golden["screen"]))
    for j in jobs:
        if j["kind"] == "pulsar":
            assert j["n"] == 1
        else:
            assert min(1000, n_stars) <= j["n"] <= min(20000, n_stars) and j["first"] + j["n"] <= n_stars


def test_cluster_list_matches_whole_items(golden):
    """pgx_cluster_list (the stage-2 "clusters=" list, src/main_phygas_boinc.cpp:309-333): whole comma-separated
    items only, results in cluster order whatever the list's order, unknown names ignored."""
    clusters = pg.read_clusters(golden["clusters"])
    names = [clusters[i].name.decode() for i in (300, 5, 17)]
    assert pg.cluster_list(clusters, ",".join(names)).tolist() == [5, 17, 300]
    n5 = clusters[5].name.decode()
    assert pg.cluster_list(clusters, "x" + n5 + ",y" + n5 + "z," + n5 + "q").tolist() == []
    assert pg.cluster_list(clusters, "no_such_cluster," + n5).tolist() == [5]
    assert pg.cluster_list(clusters, "").tolist() == []


def test_readers_on_awkward_lines(both, tmp_path):
    """ph_read_clusters / ph_read_targets (reference src/phygas.c:462-506) on lines the reference skips or splits: a
    header, comments, blank and short lines, non-numbers, `nan` fields, trailing tokens (a stage-2 "clusters=" list),
    a line longer than its 1,024-byte buffer, no final newline; and a missing file (-1).  Same counts and records as
    the oracle's readers."""
    P, O = both
    cl = ["0 SYN_A m 218.2 -63.4 1016.5 30.5 -2.52 0.05 -0.59 0.05 1.019 3.987 3.2 8.3 54 90 135 100",
          "# a comment", "", "   ", "1 SHORT o 1 2 3",
          "2 SYN_B o 174.7 -64.8 1068.3 32.0 5.35 0.07 2.48 0.07 nan nan 7.3 16.7 2.3 3.8 5.7 5.7",
          "3 SYN_C o 174.7 -64.8 1068.3 32.0 5.35 0.07 2.48 0.07 nan 4.0 7.3 16.7 2.3 3.8 5.7 5.7 extra tokens",
          "4 SYN_D o x -64.8 1068.3 32.0 5.35 0.07 2.48 0.07 1 2 7.3 16.7 2.3 3.8 5.7 5.7",
          "5 SYN_E o 1 2 3 4 5 6 7 8 9 10 11 12 13 14 15 16 " + "9" * 1100,
          "6 SYN_LAST o 10 -5 500 5 1 0.1 2 0.1 -3.2 1.1 2 6 10 20 30 30"]
    tg = ["PHYGAS 1 pair 100 0.05",
          "JSYN0 P 104.8 4.06 0.0 0.0 1633.2 0.25 -20.37 0.32 -38.25 0.32 nan nan 79.95",
          "STAR1 S 10.0 -5.0 2.5 0.2 0.0 0.0 1.0 0.1 -2.0 0.1 12.0 1.5 clusters=SYN_A,SYN_B",
          "# STAR2 S 10 -5 2.5 0.2 0 0 1 0.1 -2 0.1 12 1.5", "STAR3 S 10 -5 2.5",
          "STAR4 S 10.0 -5.0 2.5 0.2 0.0 0.0 1.0 0.1 -2.0 0.1 nan 1.5",
          "X" * 1030 + " S 1 2 3 4 5 6 7 8 9 10 11 12",
          "STAR5 S 11.0 -6.0 2.0 0.2 0.0 0.0 1.0 0.1 -2.0 0.1 12.0 1.5"]
    for lines, T, fn in ((cl, pg.PhCluster, "ph_read_clusters"), (tg, pg.PhTarget, "ph_read_targets")):
        path = tmp_path / (fn + ".txt")
        path.write_text("\n".join(lines))                 # no final newline
        pa, pb = C.POINTER(T)(), C.POINTER(T)()
        getattr(P, fn).argtypes = getattr(O, fn).argtypes = [C.c_char_p, C.POINTER(C.POINTER(T))]
        na = getattr(P, fn)(str(path).encode(), C.byref(pa))
        nb = getattr(O, fn)(str(path).encode(), C.byref(pb))
        assert na == nb >= 3, (fn, na, nb)
        for i in range(na):
            for f, ft in T._fields_:
                va, vb = getattr(pa[i], f), getattr(pb[i], f)
                if ft is C.c_double:
                    va, vb = np.float64(va).tobytes(), np.float64(vb).tobytes()
                assert va == vb, (fn, i, f)
        missing = str(tmp_path / "no_such_file.txt").encode()
        assert getattr(P, fn)(missing, C.byref(pa)) == getattr(O, fn)(missing, C.byref(pb)) == -1


def test_track_starts_identical(both, golden):
    """pgh_track_starts (the host half of the GPU prefilter: each object's nominal start and its 32-draw spread) gives
    the oracle's ph_sample_* nominal point and ph_track_* sig_pos / sig_vel, bit for bit, for targets and clusters."""
    P, O = both

    class Track(C.Structure):
        _fields_ = [("n", C.c_int), ("pos", C.POINTER(C.c_double)), ("sig_pos", C.c_double),
                    ("sig_vel", C.c_double)]

    class PhaseSpace(C.Structure):
        _fields_ = [("pos", C.c_double * 3), ("vel", C.c_double * 3)]

    clusters = pg.read_clusters(golden["clusters"])[:200]
    targets = list(pg.read_targets(golden["pulsar"])[:3]) + list(pg.read_targets(golden["screen"])[:20])
    P.pgh_track_starts.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_double),
                                   C.POINTER(C.c_double)]
    O.ph_track_target.argtypes = [C.POINTER(pg.PhTarget), C.c_double, C.c_int, C.c_uint64, C.POINTER(Track)]
    O.ph_track_cluster.argtypes = [C.POINTER(pg.PhCluster), C.c_int, C.c_uint64, C.POINTER(Track)]
    O.ph_sample_target.argtypes = [C.POINTER(pg.PhTarget), C.c_void_p, C.POINTER(PhaseSpace)]
    O.ph_sample_cluster.argtypes = [C.POINTER(pg.PhCluster), C.c_void_p, C.POINTER(PhaseSpace)]
    O.ph_seed.restype = C.c_uint64
    O.ph_seed.argtypes = [C.c_char_p, C.c_char_p]
    tmax = max(c.tmax_myr for c in clusters)
    for objs, is_t in ((targets, True), (clusters, False)):
        arr = pg.as_array(objs, pg.PhTarget if is_t else pg.PhCluster)
        ps, sig = np.zeros(6 * len(objs)), np.zeros(2 * len(objs))
        P.pgh_track_starts(C.cast(arr, C.c_void_p) if is_t else None, None if is_t else C.cast(arr, C.c_void_p),
                           len(objs), 4, pg._ptr(ps), pg._ptr(sig))
        for i, o in enumerate(objs):
            nom, t = PhaseSpace(), Track()
            if is_t:
                O.ph_sample_target(C.byref(o), None, C.byref(nom))
                O.ph_track_target(C.byref(o), tmax, 32, O.ph_seed(b"track", o.id), C.byref(t))
            else:
                O.ph_sample_cluster(C.byref(o), None, C.byref(nom))
                O.ph_track_cluster(C.byref(o), 32, O.ph_seed(b"track", o.name), C.byref(t))
            want = np.array(list(nom.pos) + list(nom.vel))
            assert ps[6 * i:6 * i + 6].tobytes() == want.tobytes(), (is_t, i)
            assert sig[2 * i:2 * i + 2].tobytes() == np.array([t.sig_pos, t.sig_vel]).tobytes(), (is_t, i)
