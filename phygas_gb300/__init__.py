"""phygas_gb300 -- Python access to libphygas_gb300 (the GB300 implementation of Phygas's screen and pair paths).

The product is the C library and its two CLIs (phygas_screen, phygas_cli) under phygas_gb300/_lib; this module only
binds the C-ABI (include/phygas.h, include/phygas_gb300.h) with ctypes for tests, benchmarks and Python callers.
There is no Python or CPU fallback of the GPU stages: without the built library every call raises.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(HERE, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libphygas_gb300.so")
SCREEN_CLI = os.path.join(LIB_DIR, "phygas_screen")
PAIR_CLI = os.path.join(LIB_DIR, "phygas_cli")
SERVE_CLI = os.path.join(LIB_DIR, "phygas_serve")

PGX_FP64, PGX_MIXED = 0, 1
PGX_E_TIMEOUT = 4
ERRORS = {1: "bad argument", 2: "CUDA error", 3: "out of device memory", 4: "wait timed out",
          5: "size limit", 6: "no usable GPU", 7: "job still running"}


class PhCluster(C.Structure):
    _fields_ = [("name", C.c_char * 40), ("kind", C.c_char), ("ra", C.c_double), ("dec", C.c_double),
                ("dist_pc", C.c_double), ("e_dist_pc", C.c_double), ("pmra", C.c_double), ("e_pmra", C.c_double),
                ("pmdec", C.c_double), ("e_pmdec", C.c_double), ("rv", C.c_double), ("e_rv", C.c_double),
                ("has_rv", C.c_int), ("r50_pc", C.c_double), ("rtot_pc", C.c_double), ("age16", C.c_double),
                ("age50", C.c_double), ("age84", C.c_double), ("tmax_myr", C.c_double)]


class PhTarget(C.Structure):
    _fields_ = [("id", C.c_char * 40), ("kind", C.c_char), ("ra", C.c_double), ("dec", C.c_double),
                ("plx", C.c_double), ("e_plx", C.c_double), ("dist_pc", C.c_double), ("e_lndist", C.c_double),
                ("pmra", C.c_double), ("e_pmra", C.c_double), ("pmdec", C.c_double), ("e_pmdec", C.c_double),
                ("rv", C.c_double), ("e_rv", C.c_double), ("has_rv", C.c_int)]


class PhResult(C.Structure):
    _fields_ = [("n", C.c_int)] + [(k, C.c_double) for k in (
        "d05", "d50", "d95", "t05", "t50", "t95", "v05", "v50", "v95", "f_r50", "f_rtot")]


class PgxScreenRow(C.Structure):
    _fields_ = [("star", C.c_int), ("cluster", C.c_int), ("kb", C.c_int), ("pad", C.c_int)] + [
        (k, C.c_double) for k in ("sb", "chi2", "t_myr", "d_nom_pc", "sig_pc", "p_r50", "p_rtot", "vrel_kms")]


class PgxStats(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("ms_total", "ms_orbit", "ms_cov", "ms_scan", "ms_select", "ms_finish",
                                          "ms_pair")] + [
        (k, C.c_long) for k in ("pairs", "kept", "candidates", "rechecked_points", "rechecked_draws", "clones",
                                "clone_steps", "body_steps", "ambiguous")] + [("kernels", C.c_int),
                                                                               ("orbit_body_steps", C.c_long),
                                                                               ("ms_prefilter", C.c_double),
                                                                               ("prefilter_pairs", C.c_long),
                                                                               ("prefilter_rechecked", C.c_long),
                                                                               ("parts", C.c_int)]


ROW_DTYPE = np.dtype([("star", "i4"), ("cluster", "i4"), ("kb", "i4"), ("pad", "i4"), ("sb", "f8"), ("chi2", "f8"),
                      ("t_myr", "f8"), ("d_nom_pc", "f8"), ("sig_pc", "f8"), ("p_r50", "f8"), ("p_rtot", "f8"),
                      ("vrel_kms", "f8")])
RESULT_DTYPE = np.dtype({"names": ["n", "d05", "d50", "d95", "t05", "t50", "t95", "v05", "v50", "v95", "f_r50",
                                   "f_rtot"],
                         "formats": ["i4"] + ["f8"] * 11, "offsets": [0] + [8 + 8 * i for i in range(11)],
                         "itemsize": 96})

_P = C.POINTER
_D = _P(C.c_double)
_I = _P(C.c_int)
_U64 = _P(C.c_uint64)

class PgxJob(C.Structure):
    _fields_ = [("kind", C.c_int), ("precision", C.c_int), ("targets", C.c_void_p), ("n_targets", C.c_int),
                ("chi2_max", C.c_double), ("p_min", C.c_double), ("n_clones", C.c_int), ("dt_myr", C.c_double)]


class PgxJobResult(C.Structure):
    _fields_ = [("status", C.c_int), ("kind", C.c_int), ("slot", C.c_int), ("t_submit", C.c_double),
                ("t_start", C.c_double), ("t_end", C.c_double), ("n_out", C.c_long), ("work", C.c_double),
                ("digest", C.c_uint64)]


class PgxServerStats(C.Structure):
    _fields_ = [("submitted", C.c_long), ("finished", C.c_long), ("queued", C.c_long), ("running", C.c_int),
                ("max_running", C.c_int), ("slots", C.c_int), ("hbm_budget_gb", C.c_double),
                ("hbm_in_use_gb", C.c_double), ("hbm_peak_gb", C.c_double), ("now_s", C.c_double)]


PGX_JOB_SCREEN, PGX_JOB_CONTROL, PGX_JOB_PAIRS = 0, 1, 2

# (name, restype, argtypes) of every C-ABI entry point bound here
SIGNATURES = [
    ("pgx_open", C.c_int, [C.c_int, _P(C.c_void_p)]),
    ("pgx_close", None, [C.c_void_p]),
    ("pgx_last_error", C.c_char_p, [C.c_void_p]),
    ("pgx_free", None, [C.c_void_p]),
    ("pgx_lin", C.c_int, [C.c_void_p, C.c_int, _D, _D, _I, _D, _D, _D]),
    ("pgx_screen_clusters", C.c_int, [C.c_void_p, C.c_int, _D, _D, _D, _D, _D, C.c_char_p, C.c_double]),
    ("pgx_screen", C.c_int, [C.c_void_p, C.c_int, _D, _D, _U64, C.c_double, C.c_double, C.c_int,
                             _P(_P(PgxScreenRow)), _P(C.c_long)]),
    ("pgx_screen_stage", C.c_int, [C.c_void_p, C.c_int, _D, _D, _U64]),
    ("pgx_screen_exec", C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_int, _P(C.c_long)]),
    ("pgx_screen_fetch", C.c_int, [C.c_void_p, C.c_void_p, C.c_long]),
    ("pgx_screen_into", C.c_int, [C.c_void_p, C.c_int, _D, _D, _U64, C.c_double, C.c_double, C.c_int, C.c_void_p,
                                  C.c_long, _P(C.c_long)]),
    ("pgx_host_alloc", C.c_void_p, [C.c_size_t]),
    ("pgx_screen_split", C.c_int, [C.c_void_p, C.c_int]),
    ("pgx_screen_parts", C.c_int, [C.c_void_p, C.c_int]),
    ("pgx_pair_blocks", C.c_int, [C.c_void_p, C.c_int]),
    ("pgx_pair_blocks_while", C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    ("pgx_pair_targets", C.c_int, [C.c_void_p, C.c_int, _P(PhTarget), _P(C.c_int), _P(PhCluster), _P(C.c_int),
                                   _P(C.c_int), C.c_double, C.c_int, C.c_int, C.c_void_p]),
    ("pgx_screen_chunks", C.c_int, [C.c_void_p, _P(PhTarget), C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                    C.c_double, C.c_int, C.c_void_p, C.c_void_p]),
    ("pgx_host_free", None, [C.c_void_p]),
    ("pgx_screen_chunks_text", C.c_int, [C.c_void_p, _P(PhTarget), C.c_int, _P(PhCluster), C.c_int, C.c_int, C.c_int,
                                         C.c_int, C.c_double, C.c_double, C.c_int, C.c_void_p, C.c_void_p]),
    ("pgx_draw_targets", C.c_int, [_P(PhTarget), C.c_int, C.c_int, C.c_int, _D, _D, _U64]),
    ("pgx_draw_clusters", C.c_int, [_P(PhCluster), C.c_int, C.c_int, C.c_int, _D, _D]),
    ("pgx_draw_targets_gpu", C.c_int, [C.c_void_p, _P(PhTarget), C.c_int, C.c_int, _D, _D, _U64]),
    ("pgx_draw_pair_batch_gpu", C.c_int, [C.c_void_p, C.c_int, _P(PhTarget), _I, _P(PhCluster), _I, _I, C.c_double,
                                          _I, _D, _I, _D, _D, _D]),
    ("pgx_seed_prefix", C.c_uint64, [C.c_char_p]),
    ("pgx_prefilter_pairs", C.c_int, [_P(PhTarget), C.c_int, _P(PhCluster), C.c_int, C.c_int, _I, _I, C.c_long,
                                      _P(C.c_long)]),
    ("pgx_prefilter", C.c_int, [C.c_void_p, _P(PhTarget), C.c_int, _P(PhCluster), C.c_int, C.c_int, _I, _I,
                                C.c_long, _P(C.c_long)]),
    ("pgx_prefilter_margin", C.c_int, [C.c_void_p, C.c_double]),
    ("pgx_pairs_with_lists", C.c_int, [C.c_void_p, _P(PhTarget), C.c_int, _P(C.c_char_p), _P(PhCluster), C.c_int,
                                       C.c_int, _I, _I, C.c_long, _P(C.c_long)]),
    ("pgx_cluster_list", C.c_int, [_P(PhCluster), C.c_int, C.c_char_p, _I, C.c_int]),
    ("pgx_tracks", C.c_int, [C.c_void_p, C.c_int, _D, _I, _D]),
    ("pgx_draw_pair_batch", C.c_int, [C.c_int, _P(PhTarget), _I, _P(PhCluster), _I, _I, C.c_double, C.c_int, _I, _D,
                                      _I, _D, _D, _D]),
    ("pgx_pair", C.c_int, [C.c_void_p, C.c_int, _I, _D, _I, _D, _D, _D, C.c_void_p, _D]),
    ("pgx_tune_pair", C.c_int, [C.c_void_p, C.c_int, _I, _D, _I, _D, _D, _D, _D, _I]),
    ("pgx_pair_shapes", C.c_int, [C.c_int, _I, _I, _I]),
    ("pgx_tune_screen", C.c_int, [C.c_void_p, C.c_double, C.c_double, _D, _I]),
    ("pgx_screen_shapes", C.c_int, [C.c_int, _I]),
    ("pgx_stats", C.c_int, [C.c_void_p, _P(PgxStats)]),
    ("pgx_peaks", C.c_int, [C.c_void_p, _D, _D]),
    ("pgx_check_bounds", C.c_int, [C.c_void_p, C.c_int, _D, _D, _D, C.c_double, _D, _P(C.c_float),
                                   _P(C.c_float), _I]),
    ("pgx_check_draws", C.c_int, [C.c_void_p, C.c_int, _D, _P(C.c_uint64), _D]),
    ("pgx_check_blocks", C.c_int, [C.c_void_p, C.c_double, C.c_double, _P(C.c_long)]),
    ("pgx_control_targets", C.c_int, [_P(PhTarget), C.c_int, _P(PhTarget)]),
    ("pgx_server_open", C.c_int, [C.c_int, C.c_int, C.c_double, _P(PhCluster), C.c_int, C.c_int, C.c_double, C.c_int,
                                  _P(C.c_void_p)]),
    ("pgx_server_submit", C.c_int, [C.c_void_p, _P(PgxJob), _P(C.c_long)]),
    ("pgx_server_wait", C.c_int, [C.c_void_p, C.c_long, _P(PgxJobResult)]),
    ("pgx_server_query", C.c_int, [C.c_void_p, C.c_long, _P(PgxJobResult)]),
    ("pgx_server_wait_for", C.c_int, [C.c_void_p, C.c_long, C.c_double, _P(PgxJobResult)]),
    ("pgx_server_rows", C.c_long, [C.c_void_p, C.c_long, C.c_void_p, C.c_long]),
    ("pgx_server_pairs", C.c_long, [C.c_void_p, C.c_long, C.c_void_p, _I, C.c_long]),
    ("pgx_server_release", None, [C.c_void_p, C.c_long]),
    ("pgx_server_stats", C.c_int, [C.c_void_p, _P(PgxServerStats)]),
    ("pgx_server_close", None, [C.c_void_p]),
    ("ph_init", None, []),
    ("ph_seed", C.c_uint64, [C.c_char_p, C.c_char_p]),
    ("ph_read_clusters", C.c_int, [C.c_char_p, _P(_P(PhCluster))]),
    ("ph_read_targets", C.c_int, [C.c_char_p, _P(_P(PhTarget))]),
    ("ph_pair_draw", C.c_int, [_P(PhTarget), _P(PhCluster), C.c_int, C.c_double, C.c_uint64, _D, _I, _D]),
    ("ph_lin_target_init", None, [_P(PhTarget), C.c_int, C.c_uint64, _D, _D]),
]

_lib = None


def lib():
    """The loaded library; raises if it has not been built (phygas_gb300.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libphygas_gb300.so is not built (%s); run __graft_entry__.build()" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        L.ph_init()
        _lib = L
    return _lib


def _ptr(a, t=C.c_double):
    return a.ctypes.data_as(_P(t))


class GpuError(RuntimeError):
    pass


def read_clusters(path):
    p = _P(PhCluster)()
    n = lib().ph_read_clusters(path.encode(), C.byref(p))
    if n < 0:
        raise OSError("can't read " + path)
    return (PhCluster * n).from_address(C.addressof(p.contents)) if n else (PhCluster * 0)()


def read_targets(path):
    p = _P(PhTarget)()
    n = lib().ph_read_targets(path.encode(), C.byref(p))
    if n < 0:
        raise OSError("can't read " + path)
    return (PhTarget * n).from_address(C.addressof(p.contents)) if n else (PhTarget * 0)()


def as_array(seq, T):
    """A ctypes array of records T from any sequence of T (ctypes slices are lists)."""
    if isinstance(seq, C.Array) and seq._type_ is T:
        return seq
    return (T * len(seq))(*seq)


def draw_targets(targets, n_samp=64, threads=0):
    targets = as_array(targets, PhTarget)
    n = len(targets)
    ps0, sig, pre = np.zeros((n, 6)), np.zeros((n, 36)), np.zeros(n, np.uint64)
    rc = lib().pgx_draw_targets(targets, n, n_samp, threads, _ptr(ps0), _ptr(sig), _ptr(pre, C.c_uint64))
    if rc:
        raise ValueError("pgx_draw_targets: %d" % rc)
    return ps0, sig, pre


def draw_clusters(clusters, n_samp=64, threads=0):
    clusters = as_array(clusters, PhCluster)
    n = len(clusters)
    ps0, sig = np.zeros((n, 6)), np.zeros((n, 36))
    rc = lib().pgx_draw_clusters(clusters, n, n_samp, threads, _ptr(ps0), _ptr(sig))
    if rc:
        raise ValueError("pgx_draw_clusters: %d" % rc)
    return ps0, sig


class Context:
    """One GPU context (pgx_open).  Methods mirror the C-ABI; arrays are numpy."""

    def __init__(self, device=0):
        self.h = C.c_void_p()
        rc = lib().pgx_open(device, C.byref(self.h))
        if rc:
            raise GpuError("pgx_open: %s" % ERRORS.get(rc, rc))

    def close(self):
        if self.h:
            lib().pgx_close(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc, what):
        if rc:
            raise GpuError("%s: %s: %s" % (what, ERRORS.get(rc, rc), lib().pgx_last_error(self.h).decode()))

    def stats(self):
        s = PgxStats()
        self._check(lib().pgx_stats(self.h, C.byref(s)), "pgx_stats")
        return {k: getattr(s, k) for k, _ in PgxStats._fields_}

    def peaks(self):
        """(FP64, FP32) FMA peaks of this GPU in FLOP/s, measured now by the library's probe kernels."""
        a, b = C.c_double(), C.c_double()
        self._check(lib().pgx_peaks(self.h, C.byref(a), C.byref(b)), "pgx_peaks")
        return a.value, b.value

    def check_bounds(self, pos, S, R2, chi2_max=25.0):
        """FP64 point chi2 and the FP32 filter's bounds for n points (see pgx_check_bounds)."""
        pos = np.ascontiguousarray(pos, np.float64)
        S = np.ascontiguousarray(S, np.float64)
        R2 = np.ascontiguousarray(R2, np.float64)
        n = len(R2)
        v, lb, ub, rej = np.zeros(n), np.zeros(n, np.float32), np.zeros(n, np.float32), np.zeros(n, np.int32)
        self._check(lib().pgx_check_bounds(self.h, n, _ptr(pos), _ptr(S), _ptr(R2), chi2_max, _ptr(v),
                                           _ptr(lb, C.c_float), _ptr(ub, C.c_float), _ptr(rej, C.c_int)),
                    "pgx_check_bounds")
        return v, lb, ub, rej

    def draw_targets(self, targets, n_samp=64):
        """pgx_draw_targets_gpu: the targets' nominal states, covariances of their draws and seed prefixes, drawn on
        the GPU (the same draws as pg.draw_targets, within the last bits of the device's math functions)."""
        targets = as_array(targets, PhTarget)
        n = len(targets)
        ps0, sig, pre = np.zeros((n, 6)), np.zeros((n, 36)), np.zeros(n, np.uint64)
        self._check(lib().pgx_draw_targets_gpu(self.h, targets, n, n_samp, _ptr(ps0), _ptr(sig),
                                               _ptr(pre, C.c_uint64)), "pgx_draw_targets_gpu")
        return ps0, sig, pre

    def draw_pair_batch(self, targets, ti, clusters, ci, n_clones, dt_myr=0.05):
        """pgx_draw_pair_batch_gpu: pg.draw_pair_batch's outputs (clone_off, ps, steps, dt, r50, rtot), the clones
        drawn on the GPU."""
        targets, clusters = as_array(targets, PhTarget), as_array(clusters, PhCluster)
        ti, ci = np.ascontiguousarray(ti, np.int32), np.ascontiguousarray(ci, np.int32)
        nc = np.ascontiguousarray(np.broadcast_to(n_clones, ti.shape), np.int32)
        n = len(ti)
        ps = np.zeros(12 * max(int(nc.sum()), 1))
        off = np.zeros(n + 1, np.int32)
        steps, dt, r50, rt = np.zeros(n, np.int32), np.zeros(n), np.zeros(n), np.zeros(n)
        self._check(lib().pgx_draw_pair_batch_gpu(self.h, n, targets, _ptr(ti, C.c_int), clusters, _ptr(ci, C.c_int),
                                                  _ptr(nc, C.c_int), dt_myr, _ptr(off, C.c_int), _ptr(ps),
                                                  _ptr(steps, C.c_int), _ptr(dt), _ptr(r50), _ptr(rt)),
                    "pgx_draw_pair_batch_gpu")
        return off, ps[:12 * int(off[-1])], steps, dt, r50, rt

    def tune_screen(self, tmax, chi2_max=25.0):
        """pgx_tune_screen on the staged chunk: -> (index of the chosen shape, [(min blocks per SM, scan ms), ...])."""
        n = lib().pgx_screen_shapes(0, None)
        mb, ms, best = np.zeros(n, np.int32), np.zeros(n), C.c_int()
        lib().pgx_screen_shapes(n, _ptr(mb, C.c_int))
        self._check(lib().pgx_tune_screen(self.h, tmax, chi2_max, _ptr(ms), C.byref(best)), "pgx_tune_screen")
        return best.value, list(zip(mb.tolist(), ms.tolist()))

    def check_blocks(self, tmax, chi2_max=25.0):
        """The filter's block test on the staged (unsplit) chunk, every point checked in FP64 (pgx_check_blocks):
        {tested, settled, points, violations, settleable, kept_pair_blocks, walked_points, point_settled,
        point_settleable, point_violations}."""
        c = (C.c_long * 12)()
        self._check(lib().pgx_check_blocks(self.h, tmax, chi2_max, c), "pgx_check_blocks")
        return dict(zip(("tested", "settled", "points", "violations", "settleable", "kept_pair_blocks",
                         "walked_points", "point_settled", "point_settleable", "point_violations",
                         "block_point_settled", "block_point_only"), list(c)))

    def check_draws(self, fin11, seeds):
        """Per pair, the FP32 draws' largest error relative to their own bound (see pgx_check_draws)."""
        fin11 = np.ascontiguousarray(fin11, np.float64)
        seeds = np.ascontiguousarray(seeds, np.uint64)
        ratio = np.zeros(len(seeds))
        self._check(lib().pgx_check_draws(self.h, len(seeds), _ptr(fin11), _ptr(seeds, C.c_uint64), _ptr(ratio)),
                    "pgx_check_draws")
        return ratio

    def lin(self, ps0, sig, npts):
        ps0 = np.ascontiguousarray(ps0, np.float64)
        sig = np.ascontiguousarray(sig, np.float64)
        npts = np.ascontiguousarray(npts, np.int32)
        tot = int(npts.sum())
        pos, vel, S = np.zeros((tot, 3)), np.zeros((tot, 3)), np.zeros((tot, 6))
        self._check(lib().pgx_lin(self.h, len(npts), _ptr(ps0), _ptr(sig), _ptr(npts, C.c_int), _ptr(pos),
                                  _ptr(vel), _ptr(S)), "pgx_lin")
        return pos, vel, S

    def set_clusters(self, clusters, n_samp=64, r_kernel=2.0, draws=None):
        clusters = as_array(clusters, PhCluster)
        ps0, sig = draws if draws is not None else draw_clusters(clusters, n_samp)
        n = len(clusters)
        tmax = np.array([c.tmax_myr for c in clusters])
        r50 = np.array([c.r50_pc for c in clusters])
        rt = np.array([c.rtot_pc for c in clusters])
        names = b"".join(bytes(c.name).ljust(40, b"\0")[:40] for c in clusters)
        self._check(lib().pgx_screen_clusters(self.h, n, _ptr(np.ascontiguousarray(ps0)),
                                              _ptr(np.ascontiguousarray(sig)), _ptr(tmax), _ptr(r50), _ptr(rt),
                                              names, r_kernel), "pgx_screen_clusters")

    def screen(self, ps0, sig, prefix, tmax, chi2_max=25.0, precision=PGX_MIXED):
        rows = _P(PgxScreenRow)()
        n = C.c_long()
        ps0 = np.ascontiguousarray(ps0, np.float64)
        sig = np.ascontiguousarray(sig, np.float64)
        prefix = np.ascontiguousarray(prefix, np.uint64)
        self._check(lib().pgx_screen(self.h, len(prefix), _ptr(ps0), _ptr(sig), _ptr(prefix, C.c_uint64), tmax,
                                     chi2_max, precision, C.byref(rows), C.byref(n)), "pgx_screen")
        out = np.zeros(n.value, ROW_DTYPE)
        if n.value:
            C.memmove(out.ctypes.data, rows, n.value * ROW_DTYPE.itemsize)
        lib().pgx_free(rows)
        return out

    def screen_into(self, ps0, sig, prefix, tmax, out, chi2_max=25.0, precision=PGX_MIXED):
        """pgx_screen_into: the rows written into `out` (a HostRows buffer, or any ROW_DTYPE array); returns the
        filled part.  Grows nothing: raises if `out` is too small."""
        n = C.c_long()
        ps0 = np.ascontiguousarray(ps0, np.float64)
        sig = np.ascontiguousarray(sig, np.float64)
        prefix = np.ascontiguousarray(prefix, np.uint64)
        arr = out.rows if isinstance(out, HostRows) else out
        self._check(lib().pgx_screen_into(self.h, len(prefix), _ptr(ps0), _ptr(sig), _ptr(prefix, C.c_uint64), tmax,
                                          chi2_max, precision, arr.ctypes.data, len(arr), C.byref(n)),
                    "pgx_screen_into")
        return arr[:n.value]

    def screen_chunks(self, targets, chunk, tmax, emit, chi2_max=25.0, precision=PGX_MIXED, n_samp=64, threads=0):
        """pgx_screen_chunks: the targets in chunks, host draws of the next chunk overlapping the GPU work on this
        one; emit(first_star, rows) gets each chunk's rows (a view into page-locked memory, valid during the call;
        star indices relative to first_star)."""
        targets = as_array(targets, PhTarget)
        err = []

        def cb(_arg, first, ptr, n):
            try:
                rows = np.ctypeslib.as_array((C.c_char * (n * ROW_DTYPE.itemsize)).from_address(ptr)) if n else b""
                emit(first, np.frombuffer(rows, ROW_DTYPE, n) if n else np.zeros(0, ROW_DTYPE))
                return 0
            except Exception as e:           # stop the run, re-raise after it
                err.append(e)
                return 1
        fn = EMIT_FN(cb)
        rc = lib().pgx_screen_chunks(self.h, targets, len(targets), chunk, n_samp, threads, tmax, chi2_max,
                                     precision, C.cast(fn, C.c_void_p), None)
        if err:
            raise err[0]
        self._check(rc, "pgx_screen_chunks")

    def screen_chunks_text(self, targets, clusters, chunk, tmax, emit, chi2_max=25.0, precision=PGX_MIXED, n_samp=64,
                           threads=0):
        """pgx_screen_chunks_text: as screen_chunks, each chunk's rows as the reference CLI's text lines formatted on
        the GPU; emit(first_star, text, n_rows) gets a memoryview of the chunk's text (valid during the call).
        `clusters` are the resident table's clusters, in its order."""
        targets, clusters = as_array(targets, PhTarget), as_array(clusters, PhCluster)
        err = []

        def cb(_arg, first, ptr, nbytes, n):
            try:
                view = memoryview((C.c_char * nbytes).from_address(ptr)).cast("B") if nbytes else memoryview(b"")
                emit(first, view, n)
                return 0
            except Exception as e:           # stop the run, re-raise after it
                err.append(e)
                return 1
        fn = TEXT_FN(cb)
        rc = lib().pgx_screen_chunks_text(self.h, targets, len(targets), clusters, len(clusters), chunk, n_samp,
                                          threads, tmax, chi2_max, precision, C.cast(fn, C.c_void_p), None)
        if err:
            raise err[0]
        self._check(rc, "pgx_screen_chunks_text")

    def pair_targets(self, targets, ti, clusters, ci, n_clones, dt_myr=0.05, threads=0, batch_pairs=0):
        """pgx_pair_targets: ph_pair over the pairs (targets[ti[q]], clusters[ci[q]]) with n_clones[q] clones, the
        host draws of each batch of pairs overlapping the GPU's tracing of the one before -> PhResult records."""
        targets, clusters = as_array(targets, PhTarget), as_array(clusters, PhCluster)
        ti, ci = np.ascontiguousarray(ti, np.int32), np.ascontiguousarray(ci, np.int32)
        nc = np.ascontiguousarray(np.broadcast_to(n_clones, ti.shape), np.int32)
        res = np.zeros(len(ti), RESULT_DTYPE)
        self._check(lib().pgx_pair_targets(self.h, len(ti), targets, _ptr(ti, C.c_int), clusters, _ptr(ci, C.c_int),
                                           _ptr(nc, C.c_int), dt_myr, threads, batch_pairs, res.ctypes.data),
                    "pgx_pair_targets")
        return res

    def prefilter(self, targets, clusters, threads=0):
        """pgx_prefilter: (target index, cluster index) arrays of the pairs that pass ph_prefilter, tested on the GPU
        (the same pairs as prefilter_pairs)."""
        targets, clusters = as_array(targets, PhTarget), as_array(clusters, PhCluster)
        n = C.c_long()
        cap = len(targets) * len(clusters)
        ti, ci = np.zeros(max(cap, 1), np.int32), np.zeros(max(cap, 1), np.int32)
        self._check(lib().pgx_prefilter(self.h, targets, len(targets), clusters, len(clusters), int(threads),
                                        _ptr(ti, C.c_int), _ptr(ci, C.c_int), cap, C.byref(n)), "pgx_prefilter")
        return ti[:n.value], ci[:n.value]

    def pairs_with_lists(self, targets, lists, clusters, threads=0):
        """pgx_pairs_with_lists: stage-2 pairs -- a target with a "clusters=" list (lists[j], str or None) gets the
        clusters it names, the others the prefilter's; (target index, cluster index) arrays."""
        targets, clusters = as_array(targets, PhTarget), as_array(clusters, PhCluster)
        arr = (C.c_char_p * max(len(targets), 1))(*[(x or "").encode() for x in lists])
        n = C.c_long()
        cap = len(targets) * len(clusters)
        ti, ci = np.zeros(max(cap, 1), np.int32), np.zeros(max(cap, 1), np.int32)
        self._check(lib().pgx_pairs_with_lists(self.h, targets, len(targets), arr, clusters, len(clusters),
                                               int(threads), _ptr(ti, C.c_int), _ptr(ci, C.c_int), cap, C.byref(n)),
                    "pgx_pairs_with_lists")
        return ti[:n.value], ci[:n.value]

    def prefilter_margin(self, margin_kpc):
        """pgx_prefilter_margin: the distance (kpc) the GPU's prefilter decisions keep from the threshold."""
        self._check(lib().pgx_prefilter_margin(self.h, float(margin_kpc)), "pgx_prefilter_margin")

    def tracks(self, ps, npts):
        """pgx_tracks: coarse tracks from nominal starts ps[n, 6]; returns the positions [sum(npts), 3]."""
        ps = np.ascontiguousarray(ps, np.float64).reshape(-1, 6)
        npts = np.ascontiguousarray(npts, np.int32)
        pos = np.zeros((int(npts.sum()), 3))
        self._check(lib().pgx_tracks(self.h, len(npts), _ptr(ps), _ptr(npts, C.c_int), _ptr(pos)), "pgx_tracks")
        return pos

    def pair_blocks(self, blocks_per_sm):
        """pgx_pair_blocks: the persistent clone kernels on at most blocks_per_sm blocks per SM (0 = all that fit)."""
        self._check(lib().pgx_pair_blocks(self.h, int(blocks_per_sm)), "pgx_pair_blocks")

    def pair_blocks_while(self, blocks_per_sm, busy):
        """pgx_pair_blocks_while: the cap only for launches made while the ctypes c_int `busy` is nonzero (the
        caller keeps `busy` alive while the context uses it; None clears it)."""
        self._busy = busy
        ptr = C.cast(C.byref(busy), C.c_void_p) if busy is not None else None
        self._check(lib().pgx_pair_blocks_while(self.h, int(blocks_per_sm), ptr), "pgx_pair_blocks_while")

    def set_split(self, min_stars, parts=None):
        """pgx_screen_split / pgx_screen_parts: stage chunks of at least min_stars stars (0 = never) in `parts`
        parts, each part's orbits traced beside the previous part's screen."""
        self._check(lib().pgx_screen_split(self.h, int(min_stars)), "pgx_screen_split")
        if parts is not None:
            self._check(lib().pgx_screen_parts(self.h, int(parts)), "pgx_screen_parts")

    def stage(self, ps0, sig, prefix):
        self._keep = (np.ascontiguousarray(ps0, np.float64), np.ascontiguousarray(sig, np.float64),
                      np.ascontiguousarray(prefix, np.uint64))
        p, s, q = self._keep
        self._check(lib().pgx_screen_stage(self.h, len(q), _ptr(p), _ptr(s), _ptr(q, C.c_uint64)), "stage")

    def exec(self, tmax, chi2_max=25.0, precision=PGX_MIXED):
        n = C.c_long()
        self._check(lib().pgx_screen_exec(self.h, tmax, chi2_max, precision, C.byref(n)), "exec")
        return n.value

    def fetch(self, n):
        out = np.zeros(n, ROW_DTYPE)
        self._check(lib().pgx_screen_fetch(self.h, out.ctypes.data, n), "fetch")
        return out

    def pair(self, clone_off, ps, steps, dt, r50_pc, rtot_pc, want_clones=False):
        clone_off = np.ascontiguousarray(clone_off, np.int32)
        ps = np.ascontiguousarray(ps, np.float64)
        steps = np.ascontiguousarray(steps, np.int32)
        dt = np.ascontiguousarray(dt, np.float64)
        r50 = np.ascontiguousarray(r50_pc, np.float64)
        rt = np.ascontiguousarray(rtot_pc, np.float64)
        npairs = len(steps)
        res = np.zeros(npairs, RESULT_DTYPE)
        clones = np.zeros((3, int(clone_off[-1]))) if want_clones else None
        self._check(lib().pgx_pair(self.h, npairs, _ptr(clone_off, C.c_int), _ptr(ps), _ptr(steps, C.c_int),
                                   _ptr(dt), _ptr(r50), _ptr(rt), res.ctypes.data,
                                   _ptr(clones) if want_clones else None), "pgx_pair")
        return (res, clones) if want_clones else res

    def tune_pair(self, clone_off, ps, steps, dt, r50_pc, rtot_pc):
        """Time every launch shape of the clone kernel on this batch and keep the fastest (pgx_tune_pair):
        -> (index of the chosen shape, [(warps per block, clones per lane, min blocks per SM, ms), ...])."""
        args = [np.ascontiguousarray(clone_off, np.int32), np.ascontiguousarray(ps, np.float64),
                np.ascontiguousarray(steps, np.int32), np.ascontiguousarray(dt, np.float64),
                np.ascontiguousarray(r50_pc, np.float64), np.ascontiguousarray(rtot_pc, np.float64)]
        shapes = pair_shapes()
        ms, best = np.zeros(len(shapes)), C.c_int()
        self._check(lib().pgx_tune_pair(self.h, len(args[2]), _ptr(args[0], C.c_int), _ptr(args[1]),
                                        _ptr(args[2], C.c_int), _ptr(args[3]), _ptr(args[4]), _ptr(args[5]),
                                        _ptr(ms), C.byref(best)), "pgx_tune_pair")
        return best.value, [(w, c, b, t) for (w, c, b), t in zip(shapes, ms.tolist())]


def pair_shapes():
    """The clone kernel's launch shapes: [(warps per block, clones per lane, min resident blocks per SM), ...]."""
    n = lib().pgx_pair_shapes(0, None, None, None)
    w, c, b = np.zeros(n, np.int32), np.zeros(n, np.int32), np.zeros(n, np.int32)
    lib().pgx_pair_shapes(n, _ptr(w, C.c_int), _ptr(c, C.c_int), _ptr(b, C.c_int))
    return list(zip(w.tolist(), c.tolist(), b.tolist()))


EMIT_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_long)
TEXT_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_size_t, C.c_long)


class HostRows:
    """Page-locked host memory for n screen rows (pgx_host_alloc), reused across calls: the device-to-host copy of
    a chunk's rows runs at the link's rate instead of through pageable staging."""

    def __init__(self, n):
        self.n = int(n)
        self._p = lib().pgx_host_alloc(self.n * ROW_DTYPE.itemsize)
        if not self._p:
            raise MemoryError("pgx_host_alloc(%d rows)" % self.n)
        buf = (C.c_char * (self.n * ROW_DTYPE.itemsize)).from_address(self._p)
        self.rows = np.frombuffer(buf, ROW_DTYPE, self.n)

    def close(self):
        if self._p:
            self.rows = None
            lib().pgx_host_free(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class HostBuffer:
    """Page-locked host memory (pgx_host_alloc) seen as a numpy array of `n` items of `dtype`; keep the object alive
    while the array is in use."""

    def __init__(self, n, dtype=np.float64):
        dtype = np.dtype(dtype)
        self._p = lib().pgx_host_alloc(max(int(n), 1) * dtype.itemsize)
        if not self._p:
            raise MemoryError("pgx_host_alloc(%d x %s)" % (n, dtype))
        self.array = np.frombuffer((C.c_char * (max(int(n), 1) * dtype.itemsize)).from_address(self._p), dtype,
                                   int(n))

    def close(self):
        if self._p:
            self.array = None
            lib().pgx_host_free(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """The request loop (pgx_server_*): slots device contexts with the cluster table resident, jobs admitted in
    arrival order as slots and the device-memory budget allow."""

    def __init__(self, clusters, slots=3, hbm_budget_gb=80.0, device=0, n_samp=64, r_kernel=2.0, host_threads=0):
        self._clusters = as_array(clusters, PhCluster)
        h = C.c_void_p()
        rc = lib().pgx_server_open(device, slots, hbm_budget_gb, self._clusters, len(self._clusters), n_samp,
                                   r_kernel, host_threads, C.byref(h))
        if rc:
            raise GpuError("pgx_server_open: %s" % ERRORS.get(rc, rc))
        self.h = h
        self._keep = {}

    def submit(self, kind, targets, precision=PGX_MIXED, chi2_max=25.0, p_min=0.001, n_clones=1000, dt_myr=0.05):
        t = as_array(targets, PhTarget)
        j = PgxJob(kind, precision, C.cast(t, C.c_void_p), len(t), chi2_max, p_min, n_clones, dt_myr)
        jid = C.c_long()
        rc = lib().pgx_server_submit(self.h, C.byref(j), C.byref(jid))
        if rc:
            raise GpuError("pgx_server_submit: %s" % ERRORS.get(rc, rc))
        return jid.value

    def wait(self, jid, timeout=None):
        """The job's result once it has finished; with a timeout (seconds), TimeoutError if it has not by then."""
        r = PgxJobResult()
        if timeout is None:
            lib().pgx_server_wait(self.h, jid, C.byref(r))
        else:
            rc = lib().pgx_server_wait_for(self.h, jid, float(timeout), C.byref(r))
            if rc == PGX_E_TIMEOUT:
                raise TimeoutError("job %d has not finished after %g s" % (jid, timeout))
            if rc:
                raise GpuError("pgx_server_wait_for: %s" % ERRORS.get(rc, rc))
        return {k: getattr(r, k) for k, _ in PgxJobResult._fields_}

    def rows(self, jid):
        n = lib().pgx_server_rows(self.h, jid, None, 0)
        out = np.zeros(max(n, 0), ROW_DTYPE)
        if n > 0:
            lib().pgx_server_rows(self.h, jid, out.ctypes.data, n)
        return out

    def pairs(self, jid):
        n = lib().pgx_server_pairs(self.h, jid, None, None, 0)
        res, cl = np.zeros(max(n, 0), RESULT_DTYPE), np.zeros(max(n, 0), np.int32)
        if n > 0:
            lib().pgx_server_pairs(self.h, jid, res.ctypes.data, _ptr(cl, C.c_int), n)
        return res, cl

    def release(self, jid):
        lib().pgx_server_release(self.h, jid)

    def stats(self):
        s = PgxServerStats()
        lib().pgx_server_stats(self.h, C.byref(s))
        return {k: getattr(s, k) for k, _ in PgxServerStats._fields_}

    def close(self):
        if self.h:
            lib().pgx_server_close(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def cluster_list(clusters, names):
    """pgx_cluster_list: indices, in cluster order, of the clusters a comma-separated "clusters=" list names."""
    clusters = as_array(clusters, PhCluster)
    ci = np.zeros(max(len(clusters), 1), np.int32)
    k = lib().pgx_cluster_list(clusters, len(clusters), names.encode(), _ptr(ci, C.c_int), len(clusters))
    if k < 0:
        raise ValueError("pgx_cluster_list: %d" % k)
    return ci[:k]


def prefilter_pairs(targets, clusters, threads=0):
    """(target index, cluster index) arrays of the pairs that pass ph_prefilter (see pgx_prefilter_pairs)."""
    targets, clusters = as_array(targets, PhTarget), as_array(clusters, PhCluster)
    n = C.c_long()
    cap = 0
    for _ in range(2):
        ti, ci = np.zeros(max(cap, 1), np.int32), np.zeros(max(cap, 1), np.int32)
        rc = lib().pgx_prefilter_pairs(targets, len(targets), clusters, len(clusters), threads, _ptr(ti, C.c_int),
                                       _ptr(ci, C.c_int), cap, C.byref(n))
        if rc:
            raise ValueError("pgx_prefilter_pairs: %d" % rc)
        if n.value <= cap:
            return ti[:n.value], ci[:n.value]
        cap = n.value
    raise RuntimeError("pgx_prefilter_pairs: pair count changed between calls")


def control_targets(targets):
    """The screen's chance-alignment control (pgx_control_targets): each star with the proper motions (rescaled by
    the parallax ratio) and radial velocity of the star n/2 further on."""
    targets = as_array(targets, PhTarget)
    out = (PhTarget * len(targets))()
    rc = lib().pgx_control_targets(targets, len(targets), out)
    if rc:
        raise ValueError("pgx_control_targets: %d" % rc)
    return out


def draw_pair_batch(targets, ti, clusters, ci, n_clones, dt_myr=0.05, threads=0, out_ps=None):
    """pgx_draw_pair_batch: host clone draws with a clone count per pair -> clone_off, ps, steps, dt, r50, rtot.
    out_ps: a float64 array of at least 12 * sum(n_clones) to draw the clones into (for instance page-locked memory
    from HostBuffer, which the device reads at the link's full rate)."""
    targets, clusters = as_array(targets, PhTarget), as_array(clusters, PhCluster)
    ti, ci = np.ascontiguousarray(ti, np.int32), np.ascontiguousarray(ci, np.int32)
    nc = np.ascontiguousarray(np.broadcast_to(n_clones, ti.shape), np.int32)
    n = len(ti)
    need = 12 * max(int(nc.sum()), 1)
    if out_ps is None:
        ps = np.zeros(need)
    else:
        if out_ps.dtype != np.float64 or not out_ps.flags.c_contiguous or out_ps.size < need:
            raise ValueError("out_ps: a contiguous float64 array of at least %d" % need)
        ps = out_ps
    off = np.zeros(n + 1, np.int32)
    steps, dt, r50, rt = np.zeros(n, np.int32), np.zeros(n), np.zeros(n), np.zeros(n)
    rc = lib().pgx_draw_pair_batch(n, targets, _ptr(ti, C.c_int), clusters, _ptr(ci, C.c_int), _ptr(nc, C.c_int),
                                   dt_myr, threads, _ptr(off, C.c_int), _ptr(ps), _ptr(steps, C.c_int), _ptr(dt),
                                   _ptr(r50), _ptr(rt))
    if rc:
        raise ValueError("pgx_draw_pair_batch: %d" % rc)
    return off, ps[:12 * int(off[-1])], steps, dt, r50, rt


def pair_draws(targets, clusters, pairs, n_clones, dt_myr=0.05):
    """Host draws of ph_pair for a list of (target index, cluster index): clone_off, ps, steps, dt, r50, rtot."""
    L = lib()
    offs, chunks, steps, dts = [0], [], [], []
    buf = np.zeros(12 * max(n_clones, 1))
    st, dtv = C.c_int(), C.c_double()
    for j, i in pairs:
        t, c = targets[j], clusters[i]
        seed = L.ph_seed(t.id, c.name)
        m = L.ph_pair_draw(C.byref(t), C.byref(c), n_clones, dt_myr, seed, _ptr(buf), C.byref(st), C.byref(dtv))
        chunks.append(buf[:12 * m].copy())
        offs.append(offs[-1] + m)
        steps.append(st.value)
        dts.append(dtv.value)
    ps = np.concatenate(chunks) if chunks else np.zeros(0)
    r50 = np.array([clusters[i].r50_pc for _, i in pairs])
    rt = np.array([clusters[i].rtot_pc for _, i in pairs])
    return np.array(offs, np.int32), ps, np.array(steps, np.int32), np.array(dts), r50, rt
