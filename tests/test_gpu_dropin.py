"""GPU parity of the drop-in per-pair API (include/phygas.h = the reference's src/phygas.h:80-135): every function a
program written against the reference calls, driven through identical ctypes calls on libphygas_gb300 (GPU) and on
the oracle library (the reference's CPU algorithm, pinned bit for bit to the reference):

  ph_lin_target / ph_lin_cluster   tracks: positions within 1e-9 kpc, velocities and S within 1e-6 relative
  ph_screen_chi2_cut / _chi2       on the same tracks: the same argmin point and segment fraction, chi2 bit for bit
                                   (the FP64 path keeps the reference's operation order); on each library's own
                                   tracks: the same kb, chi2 within 1e-6
  ph_screen_finish / ph_screen     identical p_r50 / p_rtot counts; t, d, sigma, vrel within 1e-6 relative
  ph_pair_clone / ph_pair          closest approaches within 1e-6 relative, identical fractions, including a pair of
                                   more than 16,384 clones (the GPU's selection path for large pairs)
"""
import ctypes as C

import numpy as np
import pytest

import phygas_gb300 as pg
from tests import oracle_tools as ot

pytestmark = pytest.mark.gpu


class Vec3(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double)]


class PhLin(C.Structure):
    _fields_ = [("n", C.c_int), ("pos", C.POINTER(Vec3)), ("vel", C.POINTER(Vec3)),
                ("S", C.POINTER(C.c_double * 6))]


class PhScreen(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("chi2", "t", "d_nom_pc", "sig_pc", "p_r50", "p_rtot", "vrel")]


_P = C.POINTER
API = [
    ("ph_init", None, []),
    ("ph_seed", C.c_uint64, [C.c_char_p, C.c_char_p]),
    ("ph_lin_target", None, [_P(pg.PhTarget), C.c_double, C.c_int, C.c_uint64, _P(PhLin)]),
    ("ph_lin_cluster", None, [_P(pg.PhCluster), C.c_int, C.c_uint64, _P(PhLin)]),
    ("ph_lin_free", None, [_P(PhLin)]),
    ("ph_screen_chi2_cut", C.c_double, [_P(PhLin), _P(PhLin), _P(pg.PhCluster), C.c_double, _P(C.c_int),
                                        _P(C.c_double)]),
    ("ph_screen_chi2", C.c_double, [_P(PhLin), _P(PhLin), _P(pg.PhCluster), _P(C.c_int), _P(C.c_double)]),
    ("ph_screen_finish", None, [_P(PhLin), _P(PhLin), _P(pg.PhCluster), C.c_uint64, C.c_double, C.c_int,
                                C.c_double, _P(PhScreen)]),
    ("ph_screen", None, [_P(PhLin), _P(PhLin), _P(pg.PhCluster), C.c_uint64, _P(PhScreen)]),
    ("ph_pair_draw", C.c_int, [_P(pg.PhTarget), _P(pg.PhCluster), C.c_int, C.c_double, C.c_uint64,
                               _P(C.c_double), _P(C.c_int), _P(C.c_double)]),
    ("ph_pair_clone", None, [_P(C.c_double), C.c_int, C.c_double, _P(C.c_double), _P(C.c_double),
                             _P(C.c_double)]),
    ("ph_pair", None, [_P(pg.PhTarget), _P(pg.PhCluster), C.c_int, C.c_double, C.c_uint64, _P(pg.PhResult)]),
]


def _bind(path):
    L = C.CDLL(path)
    for name, res, args in API:
        f = getattr(L, name)
        f.restype, f.argtypes = res, args
    L.ph_init()
    return L


@pytest.fixture(scope="module")
def libs(built):
    """(GPU library, oracle library), each with ph_screen_r = 2 (the screen profile's r_kernel)."""
    gpu, ora = _bind(pg.LIB_PATH), _bind(ot.ORACLE_LIB)
    for L in (gpu, ora):
        C.c_double.in_dll(L, "ph_screen_r").value = 2.0
    return gpu, ora


@pytest.fixture(scope="module")
def data(golden):
    clusters = pg.read_clusters(golden["clusters"])
    return dict(clusters=clusters, stars=pg.read_targets(golden["screen"]),
                pulsars=pg.read_targets(golden["pulsar"]), tmax=max(c.tmax_myr for c in clusters))


def _lin_arrays(l):
    n = l.n
    pos = np.ctypeslib.as_array(C.cast(l.pos, _P(C.c_double)), (n, 3)).copy()
    vel = np.ctypeslib.as_array(C.cast(l.vel, _P(C.c_double)), (n, 3)).copy()
    S = np.ctypeslib.as_array(C.cast(l.S, _P(C.c_double)), (n, 6)).copy()
    return pos, vel, S


def _assert_tracks_close(a, b, what):
    (pa, va, Sa), (pb, vb, Sb) = _lin_arrays(a), _lin_arrays(b)
    assert a.n == b.n, what
    assert np.max(np.abs(pa - pb)) < 1e-9, what
    assert np.max(np.abs(va - vb)) < 1e-6 * np.abs(vb).max(), what
    assert np.max(np.abs(Sa - Sb)) < 1e-6 * np.abs(Sb).max(), what


def _lins(L, data, stars, clusters):
    tl, cl = [], []
    for j in stars:
        t = data["stars"][j]
        out = PhLin()
        L.ph_lin_target(C.byref(t), data["tmax"], 64, L.ph_seed(b"lin", t.id), C.byref(out))
        tl.append(out)
    for i in clusters:
        c = data["clusters"][i]
        out = PhLin()
        L.ph_lin_cluster(C.byref(c), 64, L.ph_seed(b"lin", c.name), C.byref(out))
        cl.append(out)
    return tl, cl


# 3 stars x 40 clusters spread over the table: a few hundred pairs, a few dozen kept at chi2 < 25
STARS = [0, 3, 6]
CLUSTERS = list(range(0, 4087, 103))


@pytest.fixture(scope="module")
def tracks(libs, data):
    gpu, ora = libs
    t_g, c_g = _lins(gpu, data, STARS, CLUSTERS)
    t_o, c_o = _lins(ora, data, STARS, CLUSTERS)
    yield (t_g, c_g), (t_o, c_o)
    for L, (tl, cl) in ((gpu, (t_g, c_g)), (ora, (t_o, c_o))):
        for x in tl + cl:
            L.ph_lin_free(C.byref(x))


def test_lin_target_and_cluster(tracks):
    """ph_lin_target / ph_lin_cluster: the same point counts, the tracks within the track tolerances."""
    (t_g, c_g), (t_o, c_o) = tracks
    for q, (a, b) in enumerate(zip(t_g, t_o)):
        _assert_tracks_close(a, b, ("target", q))
    for q, (a, b) in enumerate(zip(c_g, c_o)):
        _assert_tracks_close(a, b, ("cluster", q))


def _chi2(L, t, c, cl, cut):
    kb, sb = C.c_int(), C.c_double()
    if cut is None:
        v = L.ph_screen_chi2(C.byref(t), C.byref(c), C.byref(cl), C.byref(kb), C.byref(sb))
    else:
        v = L.ph_screen_chi2_cut(C.byref(t), C.byref(c), C.byref(cl), cut, C.byref(kb), C.byref(sb))
    return v, kb.value, sb.value


def test_chi2_on_the_same_tracks(libs, data, tracks):
    """ph_screen_chi2_cut (cut 25) and ph_screen_chi2 (no cut) of every pair, both libraries given the oracle's
    tracks: the same chi2, kb and sb, bit for bit."""
    gpu, ora = libs
    _, (t_o, c_o) = tracks
    n_kept = 0
    for j, t in enumerate(t_o):
        for q, i in enumerate(CLUSTERS):
            cl = data["clusters"][i]
            for cut in (25.0, None):
                g = _chi2(gpu, t, c_o[q], cl, cut)
                o = _chi2(ora, t, c_o[q], cl, cut)
                assert g[1] == o[1], (j, i, cut, g, o)
                assert g[0] == o[0] or (np.isinf(g[0]) and np.isinf(o[0])), (j, i, cut, g, o)
                if g[0] < 25.0 and cut is not None:
                    n_kept += 1
                    assert g[2] == o[2], (j, i, g, o)
    assert n_kept > 5, n_kept


def test_chi2_on_own_tracks(libs, data, tracks):
    """Each library on its own tracks: the same kept pairs and argmin points, chi2 within 1e-6 relative."""
    gpu, ora = libs
    (t_g, c_g), (t_o, c_o) = tracks
    for j in range(len(STARS)):
        for q, i in enumerate(CLUSTERS):
            cl = data["clusters"][i]
            g = _chi2(gpu, t_g[j], c_g[q], cl, 25.0)
            o = _chi2(ora, t_o[j], c_o[q], cl, 25.0)
            if o[0] < 25.0 or g[0] < 25.0:
                assert g[1] == o[1], (j, i, g, o)
                assert ot.close_rel(g[0], o[0]), (j, i, g, o)


def _close_screen(g, o, what):
    assert g.p_r50 == o.p_r50 and g.p_rtot == o.p_rtot, (what, g.p_r50, o.p_r50, g.p_rtot, o.p_rtot)
    for f in ("chi2", "t", "d_nom_pc", "sig_pc", "vrel"):
        a, b = getattr(g, f), getattr(o, f)
        assert abs(a - b) <= ot.REL_TOL * abs(b) + 1e-12, (what, f, a, b)


def test_finish_and_screen(libs, data, tracks):
    """ph_screen_finish on the same tracks and arguments, and ph_screen end to end on each library's own tracks:
    identical probability counts, the other fields within 1e-6 relative."""
    gpu, ora = libs
    (t_g, c_g), (t_o, c_o) = tracks
    n = 0
    for j, jj in enumerate(STARS):
        for q, i in enumerate(CLUSTERS):
            cl = data["clusters"][i]
            chi2, kb, sb = _chi2(ora, t_o[j], c_o[q], cl, 25.0)
            if not chi2 < 25.0:
                continue
            seed = ora.ph_seed(data["stars"][jj].id, cl.name)
            g, o = PhScreen(), PhScreen()
            gpu.ph_screen_finish(C.byref(t_o[j]), C.byref(c_o[q]), C.byref(cl), seed, chi2, kb, sb, C.byref(g))
            ora.ph_screen_finish(C.byref(t_o[j]), C.byref(c_o[q]), C.byref(cl), seed, chi2, kb, sb, C.byref(o))
            _close_screen(g, o, ("finish", jj, i))
            gpu.ph_screen(C.byref(t_g[j]), C.byref(c_g[q]), C.byref(cl), seed, C.byref(g))
            ora.ph_screen(C.byref(t_o[j]), C.byref(c_o[q]), C.byref(cl), seed, C.byref(o))
            _close_screen(g, o, ("screen", jj, i))
            n += 1
    assert n > 5, n


def test_pair_clone(libs, data):
    """ph_pair_clone of clones drawn by ph_pair_draw: best, tbest, vbest within 1e-6 relative."""
    gpu, ora = libs
    t, cl = data["pulsars"][0], data["clusters"][5]
    ps = np.zeros(12 * 8)
    steps, dt = C.c_int(), C.c_double()
    m = ora.ph_pair_draw(C.byref(t), C.byref(cl), 8, 0.05, ora.ph_seed(t.id, cl.name), pg._ptr(ps), C.byref(steps),
                         C.byref(dt))
    assert m > 0
    for k in range(m):
        p = pg._ptr(np.ascontiguousarray(ps[12 * k:12 * k + 12]))
        out = []
        for L in (gpu, ora):
            b, tb, vb = C.c_double(), C.c_double(), C.c_double()
            L.ph_pair_clone(p, steps.value, dt.value, C.byref(b), C.byref(tb), C.byref(vb))
            out.append((b.value, tb.value, vb.value))
        for a, b in zip(*out):
            assert ot.close_rel(a, b, floor=1e-12), (k, out)


def _pair(L, t, cl, n_clones):
    r = pg.PhResult()
    L.ph_pair(C.byref(t), C.byref(cl), n_clones, 0.05, L.ph_seed(t.id, cl.name), C.byref(r))
    return r


def _close_result(g, o, what):
    assert g.n == o.n, what
    for k in ("f_r50", "f_rtot"):
        assert abs(getattr(g, k) - getattr(o, k)) <= ot.PROB_TOL, (what, k)
    for k in ("d05", "d50", "d95", "t05", "t50", "t95", "v05", "v50", "v95"):
        a, b = getattr(g, k), getattr(o, k)
        assert abs(a - b) <= ot.REL_TOL * abs(b) + 1e-12, (what, k, a, b)


def test_pair(libs, data):
    """ph_pair: 100 clones against three clusters, and 20,000 clones against the cluster with the shortest trace
    (beyond the GPU's shared-memory sort of 16,384: the radix-selection path)."""
    gpu, ora = libs
    t = data["pulsars"][0]
    for i in (5, 17, 40):
        cl = data["clusters"][i]
        _close_result(_pair(gpu, t, cl, 100), _pair(ora, t, cl, 100), ("pair", i))
    i = int(np.argmin([c.tmax_myr for c in data["clusters"]]))
    cl = data["clusters"][i]
    _close_result(_pair(gpu, t, cl, 20000), _pair(ora, t, cl, 20000), ("pair 20000", i))
