"""The draws from the measurement errors on the GPU (pgx_draw_targets_gpu, pgx_draw_pair_batch_gpu) against the host
draws, which are the reference's bit for bit (tests/test_host_abi.py): the same seeds and streams take the same draws
-- the same successful clones of every pair, the same retries -- and the values agree within the last bits of the
device's math functions.  Results made from them (the screen's rows, the clone Monte Carlo) agree with the
host-draw results within the hot path's tolerances."""
import os
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


@pytest.fixture(scope="module")
def data(golden):
    clusters = pg.read_clusters(golden["clusters"])
    with tempfile.TemporaryDirectory() as d:
        cp, tp = synth.write_workload(d, "screen", 256, 1001)
        stars = pg.read_targets(tp)
        p = os.path.join(d, "pulsars.txt")
        with open(p, "w") as f:
            f.write("\n".join(synth.pulsars(16, 1003)) + "\n")
        pulsars = list(pg.read_targets(golden["pulsar"])) + list(pg.read_targets(p))
    return dict(clusters=clusters, stars=stars, pulsars=pg.as_array(pulsars, pg.PhTarget))


def test_target_draws_match_the_host(ctx, data):
    """Stars with parallaxes and radial velocities, and pulsars with log-normal distances and no radial velocity (the
    circular-velocity prior): nominal states within 1e-13 relative, covariances within 1e-9 of sqrt(S_ii S_jj),
    seed prefixes identical."""
    for objs in (data["stars"], data["pulsars"]):
        hp, hs, hpre = pg.draw_targets(objs)
        gp, gs, gpre = ctx.draw_targets(objs)
        assert np.array_equal(hpre, gpre)
        assert np.all(np.abs(gp - hp) <= 1e-13 * np.maximum(np.abs(hp), 1.0))
        H, G = hs.reshape(-1, 6, 6), gs.reshape(-1, 6, 6)
        d = np.sqrt(np.einsum("nii->ni", H))
        scale = d[:, :, None] * d[:, None, :]
        assert np.all(np.abs(G - H) <= 1e-9 * scale + 1e-300), np.max(np.abs(G - H) / (scale + 1e-300))


def test_pair_draws_match_the_host(ctx, data):
    """ph_pair_draw on the GPU for stars and pulsars against every 97th cluster, clone counts 1 to 600: the same
    successful clones (offsets identical), the same steps, dt and radii, start states within 1e-12 relative."""
    targets = pg.as_array(list(data["stars"][:8]) + list(data["pulsars"][:4]), pg.PhTarget)
    ti, ci = np.meshgrid(np.arange(len(targets)), np.arange(0, len(data["clusters"]), 97), indexing="ij")
    ti, ci = ti.ravel().astype(np.int32), ci.ravel().astype(np.int32)
    ncl = np.random.default_rng(2).integers(1, 600, len(ti)).astype(np.int32)
    h = pg.draw_pair_batch(targets, ti, data["clusters"], ci, ncl)
    g = ctx.draw_pair_batch(targets, ti, data["clusters"], ci, ncl)
    assert np.array_equal(h[0], g[0])
    for a, b in zip(h[2:], g[2:]):
        assert np.array_equal(a, b)
    assert np.all(np.abs(g[1] - h[1]) <= 1e-12 * np.maximum(np.abs(h[1]), 1.0))


def test_screen_and_pairs_from_device_draws(ctx, data):
    """The screen of 64 stars x 4,087 clusters and a pair batch from GPU draws against the same from host draws:
    the same kept pairs (except pairs within 1e-3 of the cut), d and t within 1e-6 relative, probabilities within
    one draw in 512; the pair results' quantiles within 1e-6 relative and the same clone counts."""
    clusters, stars = data["clusters"], data["stars"][:64]
    tmax = max(c.tmax_myr for c in clusters)
    ctx.set_clusters(clusters)
    a = ctx.screen(*pg.draw_targets(stars), tmax)
    b = ctx.screen(*ctx.draw_targets(stars), tmax)
    ka = {(int(r["star"]), int(r["cluster"])): r for r in a}
    kb = {(int(r["star"]), int(r["cluster"])): r for r in b}
    for k in set(ka) ^ set(kb):
        r = ka.get(k, kb.get(k))
        assert abs(r["chi2"] - 25.0) <= 1e-3 * 25.0, (k, r["chi2"])
    both = set(ka) & set(kb)
    assert len(both) > 1000
    for k in both:
        x, y = ka[k], kb[k]
        for f in ("t_myr", "d_nom_pc"):
            assert abs(x[f] - y[f]) <= ot.REL_TOL * abs(x[f]) + 1e-9, (k, f, x[f], y[f])
        for f in ("p_r50", "p_rtot"):
            assert abs(x[f] - y[f]) <= 1.0 / 512 + 1e-12, (k, f, x[f], y[f])
    ti = np.zeros(40, np.int32)
    ci = np.arange(40, dtype=np.int32) * 100
    ha = ctx.pair(*pg.draw_pair_batch(data["pulsars"], ti, clusters, ci, 200))
    ga = ctx.pair(*ctx.draw_pair_batch(data["pulsars"], ti, clusters, ci, 200))
    assert np.array_equal(ha["n"], ga["n"])
    for f in ("d05", "d50", "d95", "t05", "t50", "t95", "v05", "v50", "v95"):
        assert np.all(np.abs(ha[f] - ga[f]) <= ot.REL_TOL * np.abs(ha[f]) + 1e-9), f
