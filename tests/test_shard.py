"""The multi-GPU path's host logic (phygas_gb300.shard) on CPU: two gloo ranks each screen their own block of stars
(the oracle stands in for the GPU, as each rank's compute) and rank 0's ordered gather equals the whole list screened
at once; pair results gather in input order; the blocks cover the input exactly."""
import os
import socket

import numpy as np
import pytest

import phygas_gb300 as pg
from phygas_gb300 import shard
from tests import oracle_tools as ot

N_STARS = 4


def test_block_range_partitions():
    for n in (0, 1, 5, 20000, 20001):
        for world in (1, 2, 3, 8):
            blocks = [shard.block_range(n, world, r) for r in range(world)]
            assert blocks[0][0] == 0 and blocks[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(blocks, blocks[1:]))
            sizes = [hi - lo for lo, hi in blocks]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard.block_range(5, 2, 2)


def _rows(oracle, j0):
    """oracle rows {(star, cluster): fields} -> the record array pgx_screen returns (star relative to j0)"""
    out = np.zeros(len(oracle), pg.ROW_DTYPE)
    for h, ((j, i), r) in enumerate(oracle.items()):
        out[h]["star"], out[h]["cluster"], out[h]["kb"] = j - j0, i, r["kb"]
        for k in ("sb", "chi2", "t_myr", "d_nom_pc", "sig_pc", "p_r50", "p_rtot", "vrel_kms"):
            out[h][k] = r[k]
    return out


def _rank(rank, world, port, inputs, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"], os.environ["MASTER_PORT"] = "127.0.0.1", str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        lo, hi = shard.block_range(N_STARS, world, rank)
        rows = _rows(ot.oracle_screen(inputs["clusters"], inputs["screen"], lo, hi), lo)
        allrows = shard.gather_rows(rows, lo)
        res = np.zeros(3 + rank, pg.RESULT_DTYPE)
        res["n"] = np.arange(3 + rank) + 100 * rank
        allres = shard.gather_pairs(res)
        if rank == 0:
            q.put((allrows.tobytes(), allres["n"].tolist()))
    finally:
        dist.destroy_process_group()


def test_two_ranks_gather_in_single_gpu_order(golden):
    mp = pytest.importorskip("torch.multiprocessing")
    pytest.importorskip("torch.distributed")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    paths = {"clusters": golden["clusters"], "screen": golden["screen"]}
    procs = [ctx.Process(target=_rank, args=(r, 2, port, paths, q)) for r in range(2)]
    for p in procs:
        p.start()
    got_rows, got_n = q.get(timeout=600)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    want = _rows(ot.oracle_screen(golden["clusters"], golden["screen"], 0, N_STARS), 0)
    assert len(want) > 0 and got_rows == want.tobytes()
    assert got_n == [0, 1, 2, 100, 101, 102, 103]
