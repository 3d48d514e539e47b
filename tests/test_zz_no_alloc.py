"""pgx_pair_noalloc -- the pair Monte Carlo for callers that cannot allocate GPU memory (they run inside another
framework's device memory pool, or in a loop that must not stall on the allocator, and can only hand over device
buffers they already own).  It must give what the allocating entry point pgx_pair gives, bit for bit, call after
call, although all calls share one fixed scratch array inside the library, and it must not allocate device memory.

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


class _Dev:
    """The batch in device memory (torch tensors), and a device result buffer: the caller's own buffers."""

    def __init__(self, torch, off, ps, steps, dt, r50, rt):
        self.t = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in
                  dict(off=off, ps=ps, steps=steps, dt=dt, r50=r50, rt=rt).items()}
        self.n_pairs, self.n_clones = len(steps), int(off[-1])
        self.res = torch.zeros(max(self.n_pairs, 1) * pg.RESULT_DTYPE.itemsize // 8, dtype=torch.float64,
                               device="cuda")

    def call(self, f, stream, n_clones):
        t = self.t
        return f(stream.cuda_stream, self.n_pairs, n_clones, t["off"].data_ptr(), t["ps"].data_ptr(),
                 t["steps"].data_ptr(), t["dt"].data_ptr(), t["r50"].data_ptr(), t["rt"].data_ptr(),
                 self.res.data_ptr())

    def result(self, stream):
        stream.synchronize()
        return self.res.cpu().numpy().view(pg.RESULT_DTYPE)[:self.n_pairs]


def _same_bits(got, want):
    """Every field of every row equal bit for bit (fields compared one by one: the record's alignment gap after n is
    not part of the result, and numpy leaves it undefined in copied rows)."""
    assert len(got) == len(want)
    assert np.array_equal(got["n"], want["n"])
    for k in pg.RESULT_DTYPE.names[1:]:
        a, b = np.ascontiguousarray(got[k]).view(np.uint64), np.ascontiguousarray(want[k]).view(np.uint64)
        assert np.array_equal(a, b), (k, got[k][a != b][:3], want[k][a != b][:3])


def test_noalloc_equals_pgx_pair_twice(built):
    """Two calls in a row on different batches: each result row is pgx_pair's, bit for bit."""
    torch = pytest.importorskip("torch")
    noalloc = _bind()
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    with pg.Context(0) as ctx:
        for off, ps, steps, dt, r50, rt in _workloads():
            want = ctx.pair(off, ps, steps, dt, r50, rt)
            d = _Dev(torch, off, ps, steps, dt, r50, rt)
            assert d.call(noalloc, stream, int(off[-1])) == 0
            _same_bits(d.result(stream), want)


def test_noalloc_empty_big_and_bad_pairs(built):
    """A batch with a pair without clones (n = 0, the reference's zeroed result), a pair of 1,025 clones (beyond the
    fixed scratch's per-pair reduction: n = -1) and ordinary pairs (pgx_pair's bits); then offsets that reach past
    n_clones, which the device cannot trust: that pair gets n = -1, the others their own results."""
    torch = pytest.importorskip("torch")
    noalloc = _bind()
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    off, ps, steps, dt, r50, rt = _workloads()[1]
    rng = np.random.default_rng(11)
    # pairs 0..3 of the synthetic batch with 0, 1,025 (clones repeated), 200 and 37 clones
    m = [0, 1025, 200, 37]
    blocks = []
    for q, k in enumerate(m):
        src = ps[12 * off[q]:12 * off[q + 1]].reshape(-1, 12)
        blocks.append(src[rng.integers(0, len(src), k)] if k else np.zeros((0, 12)))
    ps2 = np.concatenate(blocks).ravel()
    off2 = np.concatenate([[0], np.cumsum(m)]).astype(np.int32)
    args = (off2, ps2, steps[:4], dt[:4], r50[:4], rt[:4])
    with pg.Context(0) as ctx:
        want = ctx.pair(*args)
    d = _Dev(torch, *args)
    assert d.call(noalloc, stream, int(off2[-1])) == 0
    got = d.result(stream)
    assert got["n"].tolist() == [0, -1, 200, 37]
    assert want["n"].tolist() == [0, 1025, 200, 37]
    _same_bits(got[[0, 2, 3]], want[[0, 2, 3]])
    # the last pair's offsets claim 37 clones, the call traces only n_clones = off2[3] + 10 of them
    assert d.call(noalloc, stream, int(off2[3]) + 10) == 0
    got = d.result(stream)
    assert got["n"].tolist() == [0, -1, 200, -1]
    _same_bits(got[[0, 2]], want[[0, 2]])


def test_noalloc_leaves_device_memory_alone(built):
    """After the first call on the device (its set-up), further calls allocate nothing: the device's free memory is
    the same before and after them."""
    torch = pytest.importorskip("torch")
    noalloc = _bind()
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    devs = [_Dev(torch, *w) for w in _workloads()]
    for d in devs:                                        # set-up and warm-up
        assert d.call(noalloc, stream, d.n_clones) == 0
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        for d in devs:
            assert d.call(noalloc, stream, d.n_clones) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_oversize(built):
    noalloc = _bind()
    assert noalloc(None, 1, (1 << 20) + 1, 1, 1, 1, 1, 1, 1, 1) == 5      # PGX_E_LIMIT, before touching memory
