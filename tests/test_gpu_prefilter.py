"""GPU parity of the prefilter (pgx_prefilter: the coarse tracks and every pair's segment tests on the GPU) against
the host code (pgx_prefilter_pairs, which tests/test_host_abi.py pins to the oracle, i.e. to the reference's
ph_track_target / ph_track_cluster / ph_prefilter, src/phygas.c:98-168): the same pairs in the same order, the GPU's
coarse tracks within 1e-9 kpc of the host's (the decisions keep a margin of 1e-7 kpc), pairs inside the margin
decided by the host, and the cluster tracks kept between calls."""
import ctypes as C
import os
import tempfile

import numpy as np
import pytest

import phygas_gb300 as pg
from phygas_gb300 import synth
from tests import oracle_tools as ot

pytestmark = pytest.mark.gpu


class Track(C.Structure):
    _fields_ = [("n", C.c_int), ("pos", C.POINTER(C.c_double)), ("sig_pos", C.c_double), ("sig_vel", C.c_double)]


class PhaseSpace(C.Structure):
    _fields_ = [("pos", C.c_double * 3), ("vel", C.c_double * 3)]


@pytest.fixture(scope="module")
def inputs(golden):
    clusters = pg.read_clusters(golden["clusters"])
    d = tempfile.mkdtemp(prefix="phygas_pref_")
    pp = os.path.join(d, "pulsars.txt")
    with open(pp, "w") as f:
        f.write("\n".join(synth.pulsars(24, 1007)) + "\n")
    targets = list(pg.read_targets(golden["pulsar"])[:4]) + list(pg.read_targets(pp)) \
        + list(pg.read_targets(golden["screen"])[:8])
    return clusters, targets


@pytest.fixture(scope="module")
def ctx():
    with pg.Context(0) as c:
        yield c


def _host_lib():
    L = pg.lib()
    L.ph_track_target.argtypes = [C.POINTER(pg.PhTarget), C.c_double, C.c_int, C.c_uint64, C.POINTER(Track)]
    L.ph_track_cluster.argtypes = [C.POINTER(pg.PhCluster), C.c_int, C.c_uint64, C.POINTER(Track)]
    L.ph_track_free.argtypes = [C.POINTER(Track)]
    L.ph_seed.restype = C.c_uint64
    L.ph_seed.argtypes = [C.c_char_p, C.c_char_p]
    L.ph_sample_target.argtypes = [C.POINTER(pg.PhTarget), C.c_void_p, C.POINTER(PhaseSpace)]
    L.ph_sample_cluster.argtypes = [C.POINTER(pg.PhCluster), C.c_void_p, C.POINTER(PhaseSpace)]
    return L


def test_coarse_tracks_match_the_host_within_the_margin(ctx, inputs):
    """pgx_tracks (GPU) against ph_track_target / ph_track_cluster (host, the reference's code): every point within
    1e-9 kpc, a hundredth of the margin the prefilter's decisions keep."""
    clusters, targets = inputs
    L = _host_lib()
    tmax = max(c.tmax_myr for c in clusters)
    objs = [("t", t) for t in targets[:12]] + [("c", clusters[i]) for i in range(0, len(clusters), 41)]
    ps, npts, want = [], [], []
    for kind, o in objs:
        nom, tr = PhaseSpace(), Track()
        if kind == "t":
            L.ph_sample_target(C.byref(o), None, C.byref(nom))
            L.ph_track_target(C.byref(o), tmax, 32, L.ph_seed(b"track", o.id), C.byref(tr))
        else:
            L.ph_sample_cluster(C.byref(o), None, C.byref(nom))
            L.ph_track_cluster(C.byref(o), 32, L.ph_seed(b"track", o.name), C.byref(tr))
        ps.append(list(nom.pos) + list(nom.vel))
        npts.append(tr.n)
        want.append(np.ctypeslib.as_array(tr.pos, (3 * tr.n,)).reshape(-1, 3).copy())
        L.ph_track_free(C.byref(tr))
    got = ctx.tracks(np.array(ps), np.array(npts, np.int32))
    want = np.concatenate(want)
    assert got.shape == want.shape
    dev = np.abs(got - want).max()
    assert dev < 1e-9, dev
    assert np.array_equal(got[0], want[0])          # the starts are the host's own values


def test_gpu_prefilter_keeps_the_host_pairs(ctx, inputs):
    """The same (target, cluster) pairs in the same order as pgx_prefilter_pairs, for 36 targets (the reference's
    pulsar, synthetic pulsars, stars) against the 4,087 clusters; few pairs need the host."""
    clusters, targets = inputs
    ti, ci = pg.prefilter_pairs(targets, clusters)
    gi, gc = ctx.prefilter(targets, clusters)
    st = ctx.stats()
    assert np.array_equal(ti, gi) and np.array_equal(ci, gc)
    assert 0 < len(ti) < len(targets) * len(clusters)
    assert st["prefilter_pairs"] == len(targets) * len(clusters)
    assert st["prefilter_rechecked"] <= 0.01 * st["prefilter_pairs"], st["prefilter_rechecked"]
    # a second call with the same clusters traces only the targets
    gi2, gc2 = ctx.prefilter(targets[:5], clusters)
    st2 = ctx.stats()
    assert st2["kernels"] < st["kernels"] and st2["body_steps"] < st["body_steps"]
    keep = ti < 5
    assert np.array_equal(gi2, ti[keep]) and np.array_equal(gc2, ci[keep])


def test_pairs_inside_the_margin_go_to_the_host(ctx, inputs):
    """With a margin of 1,000 kpc no pair can be decided on the GPU: the host decides every one, with the same
    result; with 5 kpc, about half."""
    clusters, targets = inputs
    ti, ci = pg.prefilter_pairs(targets[:6], clusters)
    got = {}
    try:
        for m in (1000.0, 5.0):
            ctx.prefilter_margin(m)
            got[m] = ctx.prefilter(targets[:6], clusters), ctx.stats()
    finally:
        ctx.prefilter_margin(1e-7)
    for m, ((gi, gc), st) in got.items():
        assert np.array_equal(ti, gi) and np.array_equal(ci, gc), m
    assert got[1000.0][1]["prefilter_rechecked"] == 6 * len(clusters)
    assert 0 < got[5.0][1]["prefilter_rechecked"] < 6 * len(clusters)


def test_edge_cases(ctx, inputs):
    clusters, targets = inputs
    gi, gc = ctx.prefilter([], clusters)
    assert len(gi) == 0 and len(gc) == 0
    gi, gc = ctx.prefilter(targets[:2], [])
    assert len(gi) == 0
    # other clusters than the ones held: the cluster side is traced again
    ti, ci = pg.prefilter_pairs(targets[:3], clusters[100:700])
    gi, gc = ctx.prefilter(targets[:3], clusters[100:700])
    assert np.array_equal(ti, gi) and np.array_equal(ci, gc)
    with pytest.raises(pg.GpuError):
        ctx.prefilter_margin(-1.0)


def test_stage2_pairs_with_lists(ctx, inputs):
    """pgx_pairs_with_lists (the reference BOINC pair mode's selection, src/main_phygas_boinc.cpp:445-447): a target
    with a "clusters=" list gets exactly the listed clusters in cluster order, the others the prefilter's pairs, all
    in target order."""
    clusters, targets = inputs
    tg = targets[:4]
    names = ",".join(clusters[i].name.decode() for i in (4000, 12, 733))
    lists = [None, names, "", "no_such_cluster"]
    ti, ci = ctx.pairs_with_lists(tg, lists, clusters)
    pti, pci = pg.prefilter_pairs([tg[0], tg[2]], clusters)
    want = [(0, int(c)) for t, c in zip(pti, pci) if t == 0] + [(1, 12), (1, 733), (1, 4000)] \
        + [(2, int(c)) for t, c in zip(pti, pci) if t == 1]
    assert list(zip(ti.tolist(), ci.tolist())) == want


def test_stage2_pairs_match_the_oracle_work_unit(ctx, inputs, golden):
    """The same selection against the oracle's work-unit runner (the reference BOINC app's pair-mode loop over
    "clusters=" lines, src/main_phygas_boinc.cpp:304-321, 445-447): the (target, cluster) pairs it runs, in its
    order, from a work unit with a list, an empty list (the prefilter decides), a list naming no cluster, and no
    list -- for stars and a pulsar."""
    import tempfile
    clusters, _ = inputs
    with open(golden["screen"]) as f:
        star_lines = [ln.rstrip("\n") for ln in f if ln.strip() and not ln.startswith(("#", "PHYGAS"))][:3]
    with open(golden["pulsar"]) as f:
        pulsar_lines = [ln.rstrip("\n") for ln in f if ln.strip() and not ln.startswith(("#", "PHYGAS"))][:1]
    names = ",".join(clusters[i].name.decode() for i in (4000, 12, 733, 2048))
    renamed = "X" + pulsar_lines[0]              # the same pulsar under another id (ids key the rows)
    lines = [star_lines[0] + " clusters=" + names, star_lines[1] + " clusters=", star_lines[2],
             renamed + " clusters=no_such_cluster", pulsar_lines[0]]
    with tempfile.TemporaryDirectory() as d:
        wu = os.path.join(d, "in")
        with open(wu, "w") as f:
            f.write("PHYGAS 1 pair 2 0.05\n" + "\n".join(lines) + "\n")
        out = ot.run([ot.ORACLE_WU, golden["clusters"], wu])
        tp = os.path.join(d, "targets")
        with open(tp, "w") as f:
            f.write("\n".join(ln.split(" clusters=")[0] for ln in lines) + "\n")
        targets = pg.read_targets(tp)
    lists = [ln.split(" clusters=")[1] if " clusters=" in ln else None for ln in lines]
    ti, ci = ctx.pairs_with_lists(targets, lists, clusters)
    index = {c.name.decode(): i for i, c in enumerate(clusters)}
    ids = {t.id.decode(): j for j, t in enumerate(targets)}
    assert len(ids) == len(targets)
    want = [(ids[row.split()[0]], index[row.split()[1]]) for row in out.splitlines()]
    got = list(zip(ti.tolist(), ci.tolist()))
    assert got == want
    assert {t for t, _ in got} == {0, 1, 2, 4}
