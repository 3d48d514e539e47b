"""The clone kernel's FP32 segment bound (Clone::step in phygas_gb300/csrc/cuda/pgx_orbit.cu) is sound: restated here
in float32 with the fast reciprocal square root at the far ends of its documented error (rsqrt.approx.f32, within
2^-22.9 relative), a segment it skips never has an FP64 distance (the reference's seg_min, src/phygas.c:147-156)
below the closest approach so far -- so skipping it cannot change the results.  Random segments from nearly
stationary to fast, closest points inside and at the ends, and closest approaches within a hair of the distance."""
import numpy as np

F = np.float32
RSQRT_ERR = 2.0 ** -22.9


def f32_trunc(x):
    """f32_trunc (pgx_bits.cuh): the float nearest x toward zero, 0 below 2^-126, +-FLT_MAX above 2^128."""
    b = np.asarray(x, np.float64).view(np.uint64)
    hi, lo = (b >> np.uint64(32)).astype(np.uint32), (b & np.uint64(0xffffffff)).astype(np.uint32)
    e = (hi >> np.uint32(20)) & np.uint32(0x7ff)
    sign = hi & np.uint32(0x80000000)
    mid = sign | ((e - np.uint32(896)) << np.uint32(23)) | ((hi & np.uint32(0xfffff)) << np.uint32(3)) | \
        (lo >> np.uint32(29))
    out = np.where(e < 897, sign, np.where(e > 1150, sign | np.uint32(0x7f7fffff), mid))
    return out.astype(np.uint32).view(np.float32)


def fmaf(a, b, c):
    # one rounding of a*b + c (the float32 product is exact in float64)
    return (np.float64(a) * np.float64(b) + np.float64(c)).astype(F)


def norm32(x, y, z, sgn, lo):
    q = fmaf(x, x, fmaf(y, y, (x * 0 + z * z).astype(F)))
    r = (1.0 / np.sqrt(np.maximum(q.astype(np.float64), 1e-300)) * (1 + sgn * RSQRT_ERR)).astype(F)
    ok = (q >= F(1e-36)) & (q <= F(1e36))
    v = (q * r).astype(F)
    if lo:
        return np.where(ok, (v * F(1 - 1e-6)).astype(F), F(0))
    return np.where(ok, (v * F(1 + 1e-6)).astype(F), F(np.inf))


def skips(r0, r1, best, sgn):
    f0 = [f32_trunc(r0[:, i]) for i in range(3)]
    f1 = [f32_trunc(r1[:, i]) for i in range(3)]
    n0 = norm32(*f0, sgn, True)
    n1 = norm32(*f1, sgn, True)
    dn = fmaf(F(2.2e-7), (n0 + n1).astype(F), norm32(*[(a - b).astype(F) for a, b in zip(f1, f0)], -sgn, False))
    lb = ((np.minimum(n0, n1) - (F(0.5) * dn).astype(F)).astype(F) * F(1 - 1e-6)).astype(F)
    lb = (lb - (F(1e-12) * (n0 + n1).astype(F)).astype(F)).astype(F)
    best_up = fmaf(f32_trunc(best), F(1 + 2.4e-7), F(1e-37))
    return lb > best_up


def seg_dist(r0, r1):
    """The FP64 segment test's distance, as the kernel computes it."""
    d = r1 - r0
    dd = np.einsum("ij,ij->i", d, d)
    an = np.einsum("ij,ij->i", r0, d)
    s = np.where(dd > 0, np.clip(-an / np.where(dd > 0, dd, 1.0), 0.0, 1.0), 0.0)
    m = r0 + d * s[:, None]
    return np.sqrt(np.einsum("ij,ij->i", m, m))


def test_segment_bound_never_skips_an_improvement():
    rng = np.random.default_rng(77)
    n = 400_000
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    scale = 10.0 ** rng.uniform(-6, 1.5, n)                 # separations from 1 mpc to 30 kpc
    r0 = u * scale[:, None]
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1)[:, None]
    r1 = r0 + v * (scale * 10.0 ** rng.uniform(-9, 0.3, n))[:, None]
    inner = rng.random(n) < 0.3                              # closest point inside the segment
    r1[inner] = -r0[inner] * rng.uniform(0.2, 2.0, inner.sum())[:, None]
    dm = seg_dist(r0, r1)
    off = rng.choice([-1e-2, -1e-5, -1e-7, -1e-9, 0.0, 1e-9, 1e-7, 1e-5, 1e-2], n)
    best = dm * (1 + off)
    for sgn in (-1.0, 1.0):
        with np.errstate(over="ignore", invalid="ignore"):     # q = 0 lanes: masked, as on the GPU
            sk = skips(r0, r1, best, sgn)
        bad = sk & (dm < best)
        assert not bad.any(), (sgn, np.flatnonzero(bad)[:5])
        # and it does skip: a short segment 1 % beyond the closest approach is skipped whatever the rounding -- unless
        # it is shorter than float32 resolves at that separation (|r1 - r0| < 2^-23 |r|: the truncated ends coincide
        # and the bound leaves the segment to the FP64 test; a clone moves 0.5-5 pc a step at kpc separations)
        seg = np.linalg.norm(r1 - r0, axis=1)
        far = (off <= -1e-2) & (seg < 1e-3 * dm) & (seg > 1e-6 * dm) & (dm > 1e-5)
        assert far.sum() > 1000 and sk[far].all(), (sgn, sk[far].mean())


def test_f32_trunc_restatement_matches_the_header():
    """The numpy restatement above against the header's own f32_trunc, on the bound's inputs' range (the header is
    pinned against the C library by tests/test_bits.py)."""
    rng = np.random.default_rng(5)
    x = rng.normal(size=10000) * 10.0 ** rng.uniform(-40, 40, 10000)
    t = f32_trunc(x).astype(np.float64)
    a = np.abs(x)
    normal = (a >= 2.0 ** -126) & (a < 2.0 ** 128)
    assert np.all(np.abs(t[normal]) <= a[normal])
    assert np.all(a[normal] < np.abs(t[normal]) * (1 + 2.0 ** -23))
    assert np.all(t[a < 2.0 ** -126] == 0)
