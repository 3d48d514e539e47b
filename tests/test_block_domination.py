"""The block tables' dominating covariance (pgx_mixed.cu k_block_tables), restated in numpy and checked on the CPU:
for a block's covariances S(k) -- needle-thin ellipsoids that turn, stretch and shrink along the track, as the
benchmark's stars' do -- both dominations the tables choose between hold at every point of the block:

  S(ke) + delta I, delta the Gershgorin bound on the largest eigenvalue of S(k) - S(ke);
  S(ke) + alpha u u^T + beta I, u the top eigenvector of S(k*) - S(ke) (k* the point of the largest delta), beta the
  largest eigenvalue of each S(k) - S(ke) on the plane orthogonal to u, alpha the Schur complement's need;

that is, every eigenvalue of N - S(k) is >= 0.  And the rank-one form is the tighter one on such blocks: its thin
axis grows by beta, where delta I grows it by delta."""
import numpy as np


def _needle(rng, n, t):
    """n blocks of 9 covariances along a track: a needle of length L(t) and width W, turning by a small angle per
    step, its length changing by a few percent per step."""
    out = []
    for _ in range(n):
        L0 = 10.0 ** rng.uniform(-3, -1)
        W = L0 * 10.0 ** rng.uniform(-3, -1)
        theta0, rate = rng.uniform(0, np.pi), rng.normal(0, 0.02)
        grow = rng.normal(0, 0.03)
        axis_z = rng.normal(size=3)
        axis_z /= np.linalg.norm(axis_z)
        Ss = []
        for k in range(9):
            th = theta0 + rate * k
            a = np.array([np.cos(th), np.sin(th), 0.1 * np.sin(2 * th)])
            a /= np.linalg.norm(a)
            L = L0 * (1.0 + grow) ** k
            S = (L * L) * np.outer(a, a) + (W * W) * np.eye(3) + (0.5 * W) ** 2 * np.outer(axis_z, axis_z)
            Ss.append(S)
        out.append(np.array(Ss))
    return out


def _dominations(S):
    ke = len(S) - 1
    Se = S[ke]
    mxe = np.abs(Se).max()
    D = S[:ke] - Se
    g = np.max(np.diagonal(D, axis1=1, axis2=2) + np.abs(D).sum(2) - np.abs(np.diagonal(D, axis1=1, axis2=2)), 1)
    delta = max(0.0, g.max()) * (1 + 1e-12)
    kstar = int(np.argmax(g))
    w, V = np.linalg.eigh(D[kstar])
    u = V[:, -1]
    e = np.array([1.0, 0, 0]) if abs(u[0]) < 0.9 else np.array([0, 1.0, 0])
    w1 = np.cross(u, e)
    w1 /= np.linalg.norm(w1)
    w2 = np.cross(u, w1)
    W = np.stack([w1, w2], 1)
    beta = max(0.0, max(np.linalg.eigvalsh(W.T @ Dk @ W)[-1] for Dk in D))
    beta = beta * (1 + 1e-6) + 1e-9 * mxe
    alpha = 0.0
    for Dk in D:
        B = beta * np.eye(3) - Dk
        a, b, C = u @ B @ u, W.T @ B @ u, W.T @ B @ W
        alpha = max(alpha, b @ np.linalg.solve(C, b) - a)
    alpha = alpha * (1 + 1e-6) + 1e-9 * mxe
    return Se + delta * np.eye(3), Se + alpha * np.outer(u, u) + beta * np.eye(3), delta, beta


def test_both_dominations_hold_and_rank_one_is_tighter():
    rng = np.random.default_rng(11)
    tighter = 0
    blocks = _needle(rng, 2000, 0)
    for S in blocks:
        iso, r1, delta, beta = _dominations(S)
        for Sk in S:
            for N in (iso, r1):
                scale = np.abs(N).max()
                assert np.linalg.eigvalsh(N - Sk)[0] >= -1e-12 * scale
        tighter += np.linalg.eigvalsh(r1)[0] < np.linalg.eigvalsh(iso)[0]
        assert beta <= delta * (1 + 1e-6) + 1e-9 * np.abs(S[-1]).max() + 1e-300
    assert tighter > 0.9 * len(blocks), tighter


def test_a_smaller_alpha_breaks_it():
    """The Schur complement's alpha is needed: a tenth of it leaves S(k) undominated on turning needles (the check
    above does reach the violations)."""
    rng = np.random.default_rng(12)
    broken = 0
    for S in _needle(rng, 300, 0):
        iso, r1, delta, beta = _dominations(S)
        Se = S[-1]
        P = r1 - Se - beta * np.eye(3)                   # alpha u u^T
        weak = Se + 0.1 * P + beta * np.eye(3)
        broken += any(np.linalg.eigvalsh(weak - Sk)[0] < -1e-9 * np.abs(weak).max() for Sk in S)
    assert broken > 0
