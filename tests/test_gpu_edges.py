"""Edge cases on the GPU: the smallest screen (one star), a screen that keeps no pair, a star whose rows do not depend
on the chunk it is screened in, and pair batches with empty and one-clone pairs between ordinary ones (the reference's
ph_pair_reduce gives a zeroed result with n = 0 for a pair without clones, src/phygas.c:226-233)."""
import numpy as np
import pytest

import phygas_gb300 as pg

pytestmark = pytest.mark.gpu

PRECISIONS = [pg.PGX_FP64, pg.PGX_MIXED]


@pytest.fixture(scope="module")
def ctx(built):
    c = pg.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def data(golden):
    return dict(clusters=pg.read_clusters(golden["clusters"]), stars=pg.read_targets(golden["screen"]),
                pulsars=pg.read_targets(golden["pulsar"]))


@pytest.mark.parametrize("precision", PRECISIONS, ids=["fp64", "mixed"])
def test_one_star_and_no_kept_pair(ctx, data, precision):
    clusters, stars = data["clusters"], data["stars"]
    ctx.set_clusters(clusters)
    tmax = max(c.tmax_myr for c in clusters)
    ps0, sig, pre = pg.draw_targets(stars[:24])
    many = ctx.screen(ps0, sig, pre, tmax, 25.0, precision)
    # star 5 screened alone: its rows, with star index 0, are its rows of the 24-star chunk
    one = ctx.screen(ps0[5:6], sig[5:6], pre[5:6], tmax, 25.0, precision)
    want = many[many["star"] == 5].copy()
    want["star"] = 0
    assert len(want) > 0 and one.tobytes() == want.tobytes()
    # a cut no pair meets: no rows, and the context still screens afterwards
    none = ctx.screen(ps0, sig, pre, tmax, 1e-30, precision)
    assert len(none) == 0
    again = ctx.screen(ps0, sig, pre, tmax, 25.0, precision)
    assert again.tobytes() == many.tobytes()


def test_pair_batch_with_empty_and_single_clone_pairs(ctx, data):
    clusters, pulsars = data["clusters"], data["pulsars"]
    ti, ci = pg.prefilter_pairs(pulsars[:1], clusters)
    ti, ci = ti[:6], ci[:6]
    ncl = np.array([40, 0, 40, 1, 0, 40], np.int32)
    res = ctx.pair(*pg.draw_pair_batch(pulsars[:1], ti, clusters, ci, ncl, 0.05))
    assert len(res) == 6
    for q in (1, 4):                                   # no clones: zeroed, n = 0
        assert res[q]["n"] == 0 and not np.any(res[q:q + 1].view(np.uint8))
    assert res[3]["n"] == 1
    r = res[3]
    assert r["d05"] == r["d50"] == r["d95"] and r["t05"] == r["t50"] == r["t95"]
    # each non-empty pair alone gives the same bits as in the batch
    for q in (0, 2, 3, 5):
        alone = ctx.pair(*pg.draw_pair_batch(pulsars[:1], ti[q:q + 1], clusters, ci[q:q + 1], ncl[q:q + 1], 0.05))
        assert alone.tobytes() == res[q:q + 1].tobytes(), q
