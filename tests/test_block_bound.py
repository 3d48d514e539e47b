"""The mixed filter's block test (block_skip32 in phygas_gb300/csrc/cuda/pgx_bounds32.cuh) is sound, checked on the CPU
with the header itself compiled as host C++ (the device's FP32 operations, fused multiply-adds written out), the
fast reciprocal and reciprocal square root put at either end of their documented error band (4 eps) and exact:

a block it settles has, at every point the FP64 path evaluates for it, a chi2 >= the cut.  Random blocks, built to
the block tables' contract (pgx_mixed.cu k_block_tables): dominating matrices N = S_t + S_c from isotropic to
needle-thin, lambda lower bounds, velocity and acceleration differences, tube radii; separations scaled so that the
bound lands near the cut, with the relative motion random or along the separation (the closest approach inside the
block).  Each settled block is probed at tube points chosen against it -- over the block's whole time range, at the
closest approach of the tube's linear part, each with the tube's offset along the direction that lowers the N^-1
norm most -- with matrices M(k) <= N."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_SRC = os.path.join(REPO, "phygas_gb300", "csrc", "cuda")
F = np.float32

HARNESS = r"""
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "pgx_bounds32.cuh"
int main(int argc, char **argv) {
    pgx::host_fast_err = (float)atof(argv[1]);
    FILE *f = fopen(argv[2], "rb");
    std::vector<float> v;
    float x;
    while (fread(&x, 4, 1, f) == 1) v.push_back(x);
    fclose(f);
    const size_t rec = 16 + 16 + 3 + 1;
    for (size_t i = 0; i + rec <= v.size(); i += rec) {
        const float *p = &v[i];
        float4 bt[4], bc[4];
        for (int q = 0; q < 4; q++) {
            bt[q] = make_float4(p[4 * q], p[4 * q + 1], p[4 * q + 2], p[4 * q + 3]);
            bc[q] = make_float4(p[16 + 4 * q], p[16 + 4 * q + 1], p[16 + 4 * q + 2], p[16 + 4 * q + 3]);
        }
        const float m[3] = {p[32], p[33], p[34]};
        putchar(pgx::block_skip32(bt, bc, m, p[35]) ? '1' : '0');
    }
    return 0;
}
"""
# host stand-ins for the CUDA vector type the header's block test reads
PRELUDE = r"""
struct float4 { float x, y, z, w; };
inline float4 make_float4(float x, float y, float z, float w) { return float4{x, y, z, w}; }
"""


def _build(tau=None):
    d = tempfile.mkdtemp(prefix="phygas_blk_")
    src, exe = os.path.join(d, "h.cpp"), os.path.join(d, "h")
    with open(src, "w") as f:
        f.write(PRELUDE + HARNESS)
    defs = [] if tau is None else ["-DPGX_BLK_TAU=%sf" % tau]
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off"] + defs + ["-I", CUDA_SRC, src, "-o", exe],
                   check=True)
    return exe, d


@pytest.fixture(scope="module")
def harness():
    return _build()


def _spd(rng, n, lo, hi, needle):
    Q, _ = np.linalg.qr(rng.normal(size=(n, 3, 3)))
    lam = 10.0 ** rng.uniform(lo, hi, size=(n, 3))
    thin = rng.uniform(size=n) < needle
    lam[thin, 1:] *= 10.0 ** rng.uniform(-6, -2, size=(thin.sum(), 2))
    lam = np.maximum(lam, 1e-6 * lam.max(axis=1)[:, None])     # positive definite after rounding to FP32
    return np.einsum("nij,nj,nkj->nik", Q, lam, Q)


def _pack6(S):
    return np.stack([S[:, 0, 0], S[:, 0, 1], S[:, 0, 2], S[:, 1, 1], S[:, 1, 2], S[:, 2, 2]], 1)


def _unpack6(s):
    return np.stack([np.stack([s[:, 0], s[:, 1], s[:, 2]], -1), np.stack([s[:, 1], s[:, 3], s[:, 4]], -1),
                     np.stack([s[:, 2], s[:, 4], s[:, 5]], -1)], -2)


def _blocks(n, seed, toward=False):
    rng = np.random.default_rng(seed)
    S_t = _pack6(_spd(rng, n, -8, -1, 0.2)).astype(F)              # the stored (dominating) matrices
    S_c = _pack6(_spd(rng, n, -8, -2, 0.1)).astype(F)
    N = _unpack6(S_t.astype(np.float64)) + _unpack6(S_c.astype(np.float64))
    lt = np.linalg.eigvalsh(_unpack6(S_t.astype(np.float64)))[:, 0]
    lc = np.linalg.eigvalsh(_unpack6(S_c.astype(np.float64)))[:, 0]
    lam_t = (lt * (1 - 1e-6)).astype(F)
    lam_c = (lc * (1 - 1e-6)).astype(F)
    lo_t = (lam_t * rng.uniform(0.3, 1.0, n)).astype(F)              # the range's smallest lower bound
    lo_c = (lam_c * rng.uniform(0.3, 1.0, n)).astype(F)
    v_t = (rng.normal(size=(n, 3)) * 0.25).astype(F)                 # kpc/Myr
    v_c = (v_t + rng.normal(size=(n, 3)) * (10.0 ** rng.uniform(-4, -1, n))[:, None]).astype(F)
    a_t = (rng.normal(size=(n, 3)) * 0.007).astype(F)                # kpc/Myr^2
    a_c = (a_t + rng.normal(size=(n, 3)) * (10.0 ** rng.uniform(-6, -2.5, n))[:, None]).astype(F)
    e_t = (10.0 ** rng.uniform(-8, -3, n)).astype(F)
    e_c = (10.0 ** rng.uniform(-8, -3, n)).astype(F)
    # star and cluster positions near the Sun, their separation along a random direction at a distance that puts
    # the separation's N^-1 norm near sqrt(cut) plus the tube's reach
    p_t = np.column_stack([-8.122 + rng.uniform(-3, 3, n), rng.uniform(-3, 3, n), rng.uniform(-0.5, 0.5, n)])
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    Ninv = np.linalg.inv(N)
    qd = np.einsum("ni,nij,nj->n", d, Ninv, d)
    cut = np.where(rng.uniform(size=n) < 0.5, 25.0, 10.0 ** rng.uniform(0, 3, n)).astype(F).astype(np.float64)
    dv = v_t.astype(np.float64) - v_c
    da = a_t.astype(np.float64) - a_c
    reach = (2 * np.sqrt(np.einsum("ni,nij,nj->n", dv, Ninv, dv)) + 2 * np.sqrt(np.einsum("ni,nij,nj->n", da, Ninv, da))
             + (e_t.astype(np.float64) + e_c) / np.sqrt(np.linalg.eigvalsh(N)[:, 0]))
    dist = (np.sqrt(cut) + reach) * rng.uniform(0.98, 1.3, n) / np.sqrt(qd)
    if toward:
        # the relative motion along the separation, toward or away, so that the tube's linear part comes closest
        # inside the block or at an end; the distance puts that approach near the cut
        speed = rng.uniform(0.2, 1.5, n) * dist / 2.0 * np.where(rng.uniform(size=n) < 0.5, 1.0, -1.0)
        side = rng.normal(size=(n, 3)) * 0.2 * np.abs(speed)[:, None]
        v_c = (v_t.astype(np.float64) + d * speed[:, None] + side).astype(F)
        dv = v_t.astype(np.float64) - v_c
        dvn = np.sqrt(np.einsum("ni,nij,nj->n", dv, Ninv, dv))
        dist = dist + 2.0 * dvn * rng.uniform(0.0, 1.0, n) / np.sqrt(qd)
    p_c = p_t - d * dist[:, None]
    hi_t, hi_c = p_t.astype(F), p_c.astype(F)
    lo_t_, lo_c_ = (p_t - hi_t).astype(F), (p_c - hi_c).astype(F)
    mref = ((hi_t - hi_c).astype(F) + (lo_t_ - lo_c_).astype(F)).astype(F)   # sep32's sum
    rec = np.zeros((n, 36), F)
    rec[:, 0:3], rec[:, 3] = v_t, e_t
    rec[:, 4:7], rec[:, 7] = a_t, lam_t
    rec[:, 8:14], rec[:, 14] = S_t, lo_t
    rec[:, 16:19], rec[:, 19] = v_c, e_c
    rec[:, 20:23], rec[:, 23] = a_c, lam_c
    rec[:, 24:30], rec[:, 30] = S_c, lo_c
    rec[:, 32:35], rec[:, 35] = mref, cut
    lo_sum = lo_t.astype(np.float64) + lo_c
    return rec, dict(N=N, mref=p_t - p_c, dv=dv, da=da, eps=e_t.astype(np.float64) + e_c, cut=cut, lo=lo_sum)


def _run(harness, rec, err):
    exe, d = harness
    path = os.path.join(d, "in.bin")
    rec.tofile(path)
    out = subprocess.run([exe, repr(err), path], stdout=subprocess.PIPE, check=True).stdout.decode()
    return np.array([c == "1" for c in out])


def _min_chi2(info, idx, rng, lo=-2.0, hi=2.0):
    """The smallest chi2 found in the tube of each block idx, with M(k) <= N: tube points at tau = -2, 0, 2 and the
    block's worst direction (e against N^-1 x, the N^-1-norm's steepest descent), matrices shrunk by random PSD parts
    while keeping lambda_min(M) >= the range's lower bound."""
    N, cut = info["N"][idx], info["cut"][idx]
    out = np.full(len(idx), np.inf)
    m, dv = info["mref"][idx], info["dv"][idx]
    Nm, Nv = np.linalg.solve(N, m[..., None])[..., 0], np.linalg.solve(N, dv[..., None])[..., 0]
    t_star = np.clip(-np.einsum("ni,ni->n", dv, Nm) / np.einsum("ni,ni->n", dv, Nv), lo, hi)
    taus = [np.full(len(idx), t) for t in np.linspace(lo, hi, 17)] + [t_star]
    for tau in taus:
        tau = tau[:, None]
        x = m + dv * tau + 0.5 * info["da"][idx] * tau * tau
        g = np.linalg.solve(N, x[..., None])[..., 0]
        g /= np.linalg.norm(g, axis=1)[:, None]
        x = x - g * info["eps"][idx, None]
        for shrink in (0.0, 1.0):
            lmin = np.linalg.eigvalsh(N)[:, 0]
            room = np.maximum(lmin - info["lo"][idx], 0.0) * shrink
            Q, _ = np.linalg.qr(rng.normal(size=(len(idx), 3, 3)))
            P = np.einsum("nij,nj,nkj->nik", Q, rng.uniform(0, 1, (len(idx), 3)) * room[:, None], Q)
            M = N - P
            q = np.einsum("ni,ni->n", x, np.linalg.solve(M, x[..., None])[..., 0])
            out = np.minimum(out, q / cut)
    return out


@pytest.mark.parametrize("toward", [False, True])
@pytest.mark.parametrize("err", [0.0, 4 * 5.96e-8, -4 * 5.96e-8])
def test_settled_blocks_stay_above_the_cut(harness, err, toward):
    rec, info = _blocks(60_000, 17 + toward, toward)
    settled = _run(harness, rec, err)
    idx = np.flatnonzero(settled)
    assert 0.05 * len(rec) < len(idx) < 0.95 * len(rec), len(idx)          # near the boundary, both outcomes
    worst = _min_chi2(info, idx, np.random.default_rng(3))
    assert worst.min() >= 1.0 - 1e-9, worst.min()


def test_the_test_is_not_vacuous(harness):
    """With a tube radius far below what the block has (the bound wrong on purpose, on the CPU), the same probes
    find settled blocks under the cut: the probes do reach the bound's weak spots."""
    rec, info = _blocks(30_000, 23)
    rec = rec.copy()
    rec[:, 3] *= F(1e-3)
    rec[:, 19] *= F(1e-3)
    settled = _run(harness, rec, 0.0)
    idx = np.flatnonzero(settled)
    worst = _min_chi2(info, idx, np.random.default_rng(4))
    assert worst.min() < 1.0


def test_the_time_range_matters():
    """Built for a block of half the time range (|tau| <= 1 Myr, the bound wrong on purpose, on the CPU), the test
    settles blocks whose tube comes under the cut between 1 and 2 Myr from the middle: the probes reach them."""
    rec, info = _blocks(30_000, 29, True)
    settled = _run(_build("1.0"), rec, 0.0)
    idx = np.flatnonzero(settled)
    worst = _min_chi2(info, idx, np.random.default_rng(5))
    assert worst.min() < 1.0
