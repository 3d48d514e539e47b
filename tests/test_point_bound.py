"""The mixed filter's point test (point_skip32 in phygas_gb300/csrc/cuda/pgx_bounds32.cuh) is sound, checked on the
CPU with the header compiled as host C++ (the device's FP32 operations, fused multiply-adds written out), the fast
reciprocal and reciprocal square root at either end of their documented error band and exact: a point it settles
has the chi2 form at or above the cut at every point of its step's segment.  Random points: matrices from isotropic
to needle-thin, segments of every length and direction, the separation scaled so that the segment's closest approach
in the M^-1 norm lands near the cut; each settled point is probed along its segment (a grid of fractions and the
form's exact minimizer)."""
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
    const size_t rec = 6 + 6 + 2 + 3 + 3 + 1;
    for (size_t i = 0; i + rec <= v.size(); i += rec) {
        const float *p = &v[i];
        const float St[6] = {p[0], p[1], p[2], p[3], p[4], p[5]}, Sc[6] = {p[6], p[7], p[8], p[9], p[10], p[11]};
        const float m0[3] = {p[14], p[15], p[16]}, m1[3] = {p[17], p[18], p[19]};
        putchar(pgx::point_skip32(St, Sc, p[12], p[13], m0, m1, p[20]) ? '1' : '0');
    }
    return 0;
}
"""
PRELUDE = r"""
struct float4 { float x, y, z, w; };
inline float4 make_float4(float x, float y, float z, float w) { return float4{x, y, z, w}; }
"""


@pytest.fixture(scope="module")
def harness():
    d = tempfile.mkdtemp(prefix="phygas_pt_")
    src, exe = os.path.join(d, "h.cpp"), os.path.join(d, "h")
    with open(src, "w") as f:
        f.write(PRELUDE + HARNESS)
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", CUDA_SRC, src, "-o", exe], check=True)
    return exe, d


def _spd(rng, n, lo, hi, needle):
    Q, _ = np.linalg.qr(rng.normal(size=(n, 3, 3)))
    lam = 10.0 ** rng.uniform(lo, hi, size=(n, 3))
    thin = rng.uniform(size=n) < needle
    lam[thin, 1:] *= 10.0 ** rng.uniform(-5, -2, size=(thin.sum(), 2))
    lam = np.maximum(lam, 1e-6 * lam.max(axis=1)[:, None])
    return np.einsum("nij,nj,nkj->nik", Q, lam, Q)


def _pack6(S):
    return np.stack([S[:, 0, 0], S[:, 0, 1], S[:, 0, 2], S[:, 1, 1], S[:, 1, 2], S[:, 2, 2]], 1)


def _unpack6(s):
    return np.stack([np.stack([s[:, 0], s[:, 1], s[:, 2]], -1), np.stack([s[:, 1], s[:, 3], s[:, 4]], -1),
                     np.stack([s[:, 2], s[:, 4], s[:, 5]], -1)], -2)


def _points(n, seed):
    rng = np.random.default_rng(seed)
    St = _pack6(_spd(rng, n, -7, -1, 0.2)).astype(F)
    Sc = _pack6(_spd(rng, n, -7, -2, 0.1)).astype(F)
    M = _unpack6(St.astype(np.float64)) + _unpack6(Sc.astype(np.float64))
    lt = np.linalg.eigvalsh(_unpack6(St.astype(np.float64)))[:, 0] * (1 - 1e-6)
    lc = np.linalg.eigvalsh(_unpack6(Sc.astype(np.float64)))[:, 0] * (1 - 1e-6)
    Minv = np.linalg.inv(M)
    cut = np.where(rng.uniform(size=n) < 0.5, 25.0, 10.0 ** rng.uniform(0, 3, n))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    qd = np.sqrt(np.einsum("ni,nij,nj->n", d, Minv, d))
    # a step along a random direction, of up to a few times the distance scale; the segment's start placed so that
    # the closest approach of the form lands near the cut
    step = rng.normal(size=(n, 3)) * (np.sqrt(cut) / qd * 10.0 ** rng.uniform(-3, 0.5, n))[:, None]
    m0 = d * (np.sqrt(cut) / qd * rng.uniform(0.9, 1.6, n))[:, None] - step * rng.uniform(-0.5, 1.5, n)[:, None]
    m0, m1 = m0.astype(F), (m0 + step).astype(F)
    rec = np.zeros((n, 21), F)
    rec[:, 0:6], rec[:, 6:12], rec[:, 12], rec[:, 13] = St, Sc, lt.astype(F), lc.astype(F)
    rec[:, 14:17], rec[:, 17:20], rec[:, 20] = m0, m1, cut.astype(F)
    return rec, dict(M=M, m0=m0.astype(np.float64), m1=m1.astype(np.float64), cut=rec[:, 20].astype(np.float64))


def _run(harness, rec, err):
    exe, d = harness
    path = os.path.join(d, "in.bin")
    rec.tofile(path)
    out = subprocess.run([exe, repr(err), path], stdout=subprocess.PIPE, check=True).stdout.decode()
    return np.array([c == "1" for c in out])


def _min_over_segment(info, idx):
    M, m0, m1, cut = info["M"][idx], info["m0"][idx], info["m1"][idx], info["cut"][idx]
    dr = m1 - m0
    Mi0, Mid = np.linalg.solve(M, m0[..., None])[..., 0], np.linalg.solve(M, dr[..., None])[..., 0]
    a, b, c = (np.einsum("ni,ni->n", m0, Mi0), np.einsum("ni,ni->n", dr, Mi0), np.einsum("ni,ni->n", dr, Mid))
    s_star = np.clip(-b / np.maximum(c, 1e-300), 0.0, 1.0)
    out = np.full(len(idx), np.inf)
    for s in [np.full(len(idx), t) for t in np.linspace(0.0, 1.0, 11)] + [s_star]:
        out = np.minimum(out, (a + 2 * b * s + c * s * s) / cut)
    return out


@pytest.mark.parametrize("err", [0.0, 4 * 5.96e-8, -4 * 5.96e-8])
def test_settled_points_stay_above_the_cut(harness, err):
    rec, info = _points(200_000, 41)
    settled = _run(harness, rec, err)
    idx = np.flatnonzero(settled)
    assert 0.05 * len(rec) < len(idx) < 0.95 * len(rec), len(idx)
    worst = _min_over_segment(info, idx)
    assert worst.min() >= 1.0 - 1e-6, worst.min()


def test_the_probe_finds_a_wrong_cut(harness):
    """The same points tested against half their cut (the test misused on purpose): the probes find settled points
    under the real cut, so they do reach the segments' closest approaches."""
    rec, info = _points(50_000, 43)
    rec = rec.copy()
    rec[:, 20] *= F(0.5)
    idx = np.flatnonzero(_run(harness, rec, 0.0))
    assert _min_over_segment(info, idx).min() < 1.0
