"""pgx_pair_noalloc -- the pair Monte Carlo for callers that cannot allocate GPU memory (they run inside another
framework's device memory pool, or in a loop that must not stall on the allocator, and can only hand over device
buffers they already own).  It must give what the allocating entry point pgx_pair gives, call after call, although
all calls share one fixed scratch array inside the library.

This file is collected last on purpose: if it fails, a run that stops at the first failure has run everything else.
"""
import ctypes as C
import gzip
import os
import tempfile

import numpy as np
import pytest

import phygas_gb300 as pg
from phygas_gb300 import synth
from tests import oracle_tools as ot

pytestmark = pytest.mark.gpu


def _bind():
    L = pg.lib()
    f = L.pgx_pair_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int, C.c_int] + [C.c_void_p] * 7
    return f


def _workloads():
    """Two different batches: the reference's own pulsar draws (4 pairs x 100 clones), and 1 synthetic pulsar x 64
    clusters x 200 clones (400 steps)."""
    with gzip.open(os.path.join(ot.GOLDEN, "ref_dump_pair_pulsar.txt.gz"), "rt") as f:
        pairs = ot.parse_pair_dump(f.read())
    clusters = pg.read_clusters(ot.golden_inputs()["clusters"])
    a = (np.concatenate([[0], np.cumsum([p["m"] for p in pairs])]).astype(np.int32),
         np.concatenate([np.array(p["ps"]).ravel() for p in pairs]),
         np.array([p["steps"] for p in pairs], np.int32), np.array([p["dt"] for p in pairs]),
         np.array([clusters[p["cluster"]].r50_pc for p in pairs]),
         np.array([clusters[p["cluster"]].rtot_pc for p in pairs]))
    with tempfile.TemporaryDirectory() as d:
        cp, tp = synth.write_workload(d, "pair64", 1, 1000)
        targets, cls = pg.read_targets(tp), pg.read_clusters(cp)
        b = pg.pair_draws(targets, cls, [(0, i) for i in range(64)], 200)
    return [a, b]


def test_noalloc_equals_pgx_pair_twice(built):
    torch = pytest.importorskip("torch")
    noalloc = _bind()
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    with pg.Context(0) as ctx:
        for off, ps, steps, dt, r50, rt in _workloads():     # two calls in a row, different inputs
            want = ctx.pair(off, ps, steps, dt, r50, rt)
            n_pairs, n_clones = len(steps), int(off[-1])
            dev = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in
                   dict(off=off, ps=ps, steps=steps, dt=dt, r50=r50, rt=rt).items()}
            res = torch.zeros(n_pairs * pg.RESULT_DTYPE.itemsize // 8, dtype=torch.float64, device="cuda")
            rc = noalloc(stream.cuda_stream, n_pairs, n_clones, dev["off"].data_ptr(), dev["ps"].data_ptr(),
                         dev["steps"].data_ptr(), dev["dt"].data_ptr(), dev["r50"].data_ptr(), dev["rt"].data_ptr(),
                         res.data_ptr())
            assert rc == 0
            stream.synchronize()
            got = res.cpu().numpy().view(pg.RESULT_DTYPE)
            assert np.array_equal(got["n"], want["n"])
            for k in ("f_r50", "f_rtot"):
                assert np.all(np.abs(got[k] - want[k]) <= ot.PROB_TOL), k
            for k in ("d05", "d50", "d95", "t05", "t50", "t95", "v05", "v50", "v95"):
                assert np.all(np.abs(got[k] - want[k]) <= ot.REL_TOL * np.abs(want[k])), k


def test_noalloc_rejects_oversize(built):
    noalloc = _bind()
    assert noalloc(None, 1, (1 << 20) + 1, 1, 1, 1, 1, 1, 1, 1) == 5      # PGX_E_LIMIT, before touching memory
