"""The GPU prefilter's margin rule (k_prefilter, phygas_gb300/csrc/cuda/pgx_prefilter.cu) is sound: restated here in
float64, a segment it keeps (or drops) is kept (or dropped) by the reference's rule (ph_prefilter, src/phygas.c:158-168)
for every pair of track points within the margin of the ones it saw -- checked on random segments, including nearly
stationary ones, closest points at either end and distances within a hair of the threshold."""
import numpy as np

STEP = 0.5            # PH_PRE_STEP_MYR


def nearest(x0, x1):
    """The reference's nearest point of the segment x0 -> x1 to the origin: (distance, s)."""
    dx = x1 - x0
    dd = np.einsum("ij,ij->i", dx, dx)
    an = np.einsum("ij,ij->i", x0, dx)
    s = np.where(dd > 0, np.clip(-an / np.where(dd > 0, dd, 1.0), 0.0, 1.0), 0.0)
    m = x0 + dx * s[:, None]
    return np.sqrt(np.einsum("ij,ij->i", m, m)), s


def reference_pass(x0, x1, k, sp, sv, r0):
    d, s = nearest(x0, x1)
    return d < r0 + 3.0 * (sp + sv * ((k + s) * STEP))


def gpu_class(x0, x1, k, sp, sv, r0, margin):
    """k_prefilter's decision for one segment: 1 kept, 0 dropped, 2 within the margin."""
    d, s = nearest(x0, x1)
    dx = x1 - x0
    dd = np.einsum("ij,ij->i", dx, dx)
    a0 = np.sqrt(np.einsum("ij,ij->i", x0, x0))
    a1 = np.sqrt(np.einsum("ij,ij->i", x1, x1))
    M = 2.0 * margin + 1e-12 * (a0 + a1)
    ds = np.where(dd > 0, np.minimum(1.0, 4.0 * M * (np.sqrt(dd) + 6.0 * a0) / np.where(dd > 0, dd, 1.0)), 1.0)
    lo, hi = np.maximum(0.0, s - ds), np.minimum(1.0, s + ds)
    thr_lo = r0 + 3.0 * (sp + sv * ((k + lo) * STEP))
    thr_hi = r0 + 3.0 * (sp + sv * ((k + hi) * STEP))
    T = 1e-12 * np.abs(thr_hi)
    return np.where(d + M < thr_lo - T, 1, np.where(d - M > thr_hi + T, 0, 2))


def unit(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1)[:, None]


def test_margin_rule_is_sound():
    rng = np.random.default_rng(1234)
    margin = 1e-7
    n = 200_000
    scale = 10.0 ** rng.uniform(-3, 1, n)                       # separations from 1 pc to 10 kpc
    x0 = unit(rng, n) * scale[:, None]
    step = 10.0 ** rng.uniform(-9, 0, n)                        # from nearly stationary to fast
    x1 = x0 + unit(rng, n) * (scale * step)[:, None]
    # a third of the segments with the closest point inside, towards the origin
    inner = rng.random(n) < 0.33
    x1[inner] = -x0[inner] * rng.uniform(0.5, 1.5, inner.sum())[:, None]
    k = rng.integers(0, 200, n).astype(float)
    sp = 10.0 ** rng.uniform(-4, -1, n)
    sv = 10.0 ** rng.uniform(-5, -2, n)
    # thresholds placed around the segment's distance: far off, near, and within a hair
    d, s = nearest(x0, x1)
    off = rng.choice([-1e-3, -1e-6, -1e-8, 0.0, 1e-8, 1e-6, 1e-3], n) * rng.uniform(0.5, 2.0, n)
    r0 = d * (1 + off) - 3.0 * (sp + sv * ((k + s) * STEP))    # any real r0: the rule's algebra does not need r0 >= 0
    cls = gpu_class(x0, x1, k, sp, sv, r0, margin)
    assert (cls == 1).sum() > 0.05 * n and (cls == 0).sum() > 0.05 * n
    r0hat = x0 / np.linalg.norm(x0, axis=1)[:, None]
    r1hat = x1 / np.maximum(np.linalg.norm(x1, axis=1), 1e-300)[:, None]
    trials = [(unit(rng, n) * (2 * margin * rng.random(n))[:, None], unit(rng, n) * (2 * margin * rng.random(n))[:, None])
              for _ in range(4)]                                # each object's track point moved by up to the margin
    trials += [(unit(rng, n) * 2 * margin, unit(rng, n) * 2 * margin) for _ in range(4)]      # by all of it
    trials += [(-2 * margin * r0hat, -2 * margin * r1hat), (2 * margin * r0hat, 2 * margin * r1hat)]   # radially
    for e0, e1 in trials:
        ref = reference_pass(x0 + e0, x1 + e1, k, sp, sv, r0)
        assert not np.any((cls == 1) & ~ref), np.flatnonzero((cls == 1) & ~ref)[:5]
        assert not np.any((cls == 0) & ref), np.flatnonzero((cls == 0) & ref)[:5]
    # where the threshold's slope along the segment (1.5 sv) and the margins are small against the distance's offset
    # from it, the GPU decides
    wide = (np.abs(off) >= 1e-6) & (1.5 * sv < 0.1 * d * np.abs(off)) & (d * np.abs(off) > 1e-5)
    assert wide.sum() > 1000 and (cls[wide] == 2).mean() < 0.05
