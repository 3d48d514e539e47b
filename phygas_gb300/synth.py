"""Seeded synthetic inputs for the Phygas hot-path workloads (the reference's real catalogues are not public data here).

Writes the reference's text formats (clusters: 19 fields, read by ph_read_clusters, reference src/phygas.c:462-484;
targets: 14 fields, ph_read_targets, src/phygas.c:486-506).  Every number is a function of (seed, kind, index) only,
drawn from a splitmix64 stream of its own, so a smaller workload is a prefix of a larger one.

Workloads (sizes and distributions as the benchmark configurations describe them):
  pair64   1 pulsar x 64 clusters, tmax fixed at 20 Myr (400 leapfrog steps at dt 0.05): the plain FP64 ph_pair case
  screen   20,000 stars x 4,087 clusters (878 of them without a radial velocity), tmax = min(1.5 age, 100 Myr)
  pulsars  C0-style pulsars, for the batched Monte Carlo and the serving mix

Stars: heliocentric distance from an exponential disc (scale length 2.6 kpc, scale height 300 pc) cut at 3 kpc,
velocity = circular rotation of the Allen & Santillan potential + isotropic N(0, 30 km/s); fractional parallax error
U(5, 30 %), proper-motion error U(0.02, 0.2) mas/yr, radial-velocity error U(1, 10) km/s.
Clusters: heliocentric distance log-uniform 100 pc - 2 kpc (pair64) or - 5 kpc (screen), l uniform, z ~ N(0, 100 pc),
velocity = rotation + N(0, 10 km/s), distance error 2 %, proper-motion error 0.05 mas/yr, RV error 1 km/s, r50
log-uniform 1-10 pc, rtot = 3 r50, age log-uniform 1-100 Myr.
Pulsars: distance log-normal around 1 kpc (0.3 dex), l uniform, b ~ N(0, 5 deg), velocity = rotation + 3-D N(0, 265
km/s), proper-motion error 1 mas/yr, log-normal distance error 0.25, no radial velocity.
"""
import math
import os

import numpy as np

M64 = (1 << 64) - 1
KMS_PER_KPCMYR = 977.7922216807892
AU_YR_KMS = 1.495978707e8 / 3.15576e7
SUN_R0, SUN_Z0 = 8.122, 0.0208
SUN_V_KMS = np.array([11.1, 229.0 + 12.24, 7.25])
# ICRS -> Galactic rotation (Hipparcos definition, ESA 1997 vol. 1 sec. 1.5.3)
ROT = np.array([[-0.0548755604162154, -0.8734370902348850, -0.4838350155487132],
                [0.4941094278755837, -0.4448296299600112, 0.7469822444972189],
                [-0.8676661490190047, -0.1980763734312015, 0.4559837761750669]])
# Allen & Santillan (1991): GM in kpc^3/Myr^2, scales in kpc
_G = 4.30091e-6 / (KMS_PER_KPCMYR * KMS_PER_KPCMYR)
MW = dict(bulge_GM=_G * 606.0 * 2.325e7, bulge_b=0.3873, disk_GM=_G * 3690.0 * 2.325e7, disk_a=5.3178, disk_b=0.25,
          halo_GM=_G * 4615.0 * 2.325e7, halo_a=12.0, halo_cut=100.0, halo_gamma=2.02)


class Stream:
    """splitmix64 (Vigna), vectorised over items: one independent stream per (seed, kind, item)."""

    def __init__(self, seed, kind, idx):
        idx = np.asarray(idx, dtype=np.uint64)
        with np.errstate(over="ignore"):
            s = (np.uint64(seed) * np.uint64(0xD1342543DE82EF95)) ^ (np.uint64(kind) * np.uint64(0x9E3779B97F4A7C15))
            self.s = s ^ ((idx + np.uint64(1)) * np.uint64(0xBF58476D1CE4E5B9))

    def u64(self):
        with np.errstate(over="ignore"):
            self.s = self.s + np.uint64(0x9E3779B97F4A7C15)
            z = self.s
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            return z ^ (z >> np.uint64(31))

    def u(self):
        return (self.u64() >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)

    def uni(self, a, b):
        return a + (b - a) * self.u()

    def gauss(self):
        u1 = np.maximum(self.u(), 1e-300)
        u2 = self.u()
        return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * math.pi * u2)


def circular_velocity(pos):
    """Velocity (kpc/Myr) of a circular orbit in the Galactic plane at pos's cylindrical radius, rotating so the Sun
    at (-R0, 0) moves along +y; from the in-plane radial force of the Allen & Santillan potential."""
    x, y = pos[:, 0], pos[:, 1]
    R = np.hypot(x, y)
    p = MW
    fb = p["bulge_GM"] * R / (R * R + p["bulge_b"] ** 2) ** 1.5
    az = p["disk_a"] + p["disk_b"]
    fd = p["disk_GM"] * R / (R * R + az * az) ** 1.5
    xh = np.minimum(R, p["halo_cut"]) / p["halo_a"]
    fh = p["halo_GM"] * xh ** p["halo_gamma"] / (1.0 + xh ** (p["halo_gamma"] - 1.0)) / (R * R)
    vc = np.sqrt(R * (fb + fd + fh))
    return np.stack([vc * y / R, -vc * x / R, np.zeros_like(R)], axis=1)


def astrometry(pos, vel):
    """Galactocentric pos (kpc), vel (kpc/Myr) -> ra, dec (deg), distance (pc), pmra*, pmdec (mas/yr), rv (km/s)."""
    hel = pos + np.array([SUN_R0, 0.0, -SUN_Z0])
    p = hel @ ROT                       # ICRS-aligned, kpc (ROT^T applied to row vectors)
    v = (vel * KMS_PER_KPCMYR - SUN_V_KMS) @ ROT
    d = np.linalg.norm(p, axis=1)
    ra = np.arctan2(p[:, 1], p[:, 0])
    ra = np.where(ra < 0, ra + 2 * math.pi, ra)
    dec = np.arcsin(p[:, 2] / d)
    er = p / d[:, None]
    ea = np.stack([-np.sin(ra), np.cos(ra), np.zeros_like(ra)], axis=1)
    ed = np.stack([-np.sin(dec) * np.cos(ra), -np.sin(dec) * np.sin(ra), np.cos(dec)], axis=1)
    k = AU_YR_KMS * 1e-3 * d * 1000.0
    return (np.degrees(ra), np.degrees(dec), d * 1000.0, (v * ea).sum(1) / k, (v * ed).sum(1) / k,
            (v * er).sum(1))


def _helio_to_galcen(d_kpc, l, b):
    h = np.stack([d_kpc * np.cos(b) * np.cos(l), d_kpc * np.cos(b) * np.sin(l), d_kpc * np.sin(b)], axis=1)
    return h + np.array([-SUN_R0, 0.0, SUN_Z0])


def clusters(n, seed, dmax_pc=5000.0, tmax_fixed=None, n_no_rv=None):
    """n clusters -> list of text lines (19 fields)."""
    i = np.arange(n)
    r = Stream(seed, 1, i)
    d = 100.0 * (dmax_pc / 100.0) ** r.u()
    l = r.uni(0.0, 2 * math.pi)
    z = 0.1 * r.gauss()
    dk = d / 1000.0
    b = np.arcsin(np.clip((z - SUN_Z0) / dk, -1, 1))
    pos = _helio_to_galcen(dk, l, b)
    vel = circular_velocity(pos) + np.stack([r.gauss(), r.gauss(), r.gauss()], 1) * (10.0 / KMS_PER_KPCMYR)
    r50 = 10.0 ** r.uni(0.0, 1.0)
    age = 10.0 ** r.uni(0.0, 2.0)
    kind_u = r.u()
    ra, dec, dist, pmra, pmdec, rv = astrometry(pos, vel)
    if n_no_rv is None:
        no_rv = np.zeros(n, bool)
    else:   # a fixed count without RV, spread over the list by a stream of their own
        order = np.argsort(Stream(seed, 5, i).u(), kind="stable")
        no_rv = np.zeros(n, bool)
        no_rv[order[:n_no_rv]] = True
    out = []
    for k in range(n):
        a16, a50, a84 = 0.6 * age[k], age[k], 1.5 * age[k]
        tmax = tmax_fixed if tmax_fixed is not None else min(a84, 100.0)
        rv_s, erv_s = ("nan", "nan") if no_rv[k] else ("%.3f" % rv[k], "1.000")
        out.append("%d SYN%05d %s %.6f %.6f %.2f %.2f %.4f 0.0500 %.4f 0.0500 %s %s %.3f %.3f %.3f %.3f %.3f %.3f" % (
            k, k, "o" if kind_u[k] < 0.85 else "m", ra[k], dec[k], dist[k], 0.02 * dist[k], pmra[k], pmdec[k],
            rv_s, erv_s, r50[k], 3.0 * r50[k], a16, a50, a84, tmax))
    return out


def stars(n, seed):
    """n stars with radial velocities -> list of text lines (14 fields)."""
    i = np.arange(n)
    r = Stream(seed, 2, i)
    # exponential disc (density ~ exp(-R/2.6 kpc) exp(-|z|/0.3 kpc)) within 3 kpc of the Sun: propose uniformly in
    # the plane around the Sun with the vertical exponential, accept with exp(-(R - Rmin)/2.6) (Rmin = R0 - 3 kpc)
    pos = np.zeros((n, 3))
    todo = np.ones(n, bool)
    for _ in range(64):
        rho = 3.0 * np.sqrt(r.u())
        phi = r.uni(0.0, 2 * math.pi)
        zz = -0.3 * np.log(np.maximum(r.u(), 1e-300)) * np.where(r.u() < 0.5, -1.0, 1.0)
        cand = np.stack([-SUN_R0 + rho * np.cos(phi), rho * np.sin(phi), zz], 1)
        hel = np.linalg.norm(cand - np.array([-SUN_R0, 0.0, SUN_Z0]), axis=1)
        R = np.hypot(cand[:, 0], cand[:, 1])
        ok = todo & (hel < 3.0) & (hel > 0.02) & (r.u() < np.exp(-(R - (SUN_R0 - 3.0)) / 2.6))
        pos[ok] = cand[ok]
        todo &= ~ok
    if todo.any():   # the few left over after 64 tries: place them at 1 kpc in the plane
        pos[todo] = np.array([-SUN_R0 + 1.0, 0.0, SUN_Z0])
    vel = circular_velocity(pos) + np.stack([r.gauss(), r.gauss(), r.gauss()], 1) * (30.0 / KMS_PER_KPCMYR)
    f_plx = r.uni(0.05, 0.30)
    e_pm = r.uni(0.02, 0.2)
    e_rv = r.uni(1.0, 10.0)
    ra, dec, dist, pmra, pmdec, rv = astrometry(pos, vel)
    plx = 1000.0 / dist
    return ["%d S %.9f %.9f %.6f %.6f 0 0 %.5f %.5f %.5f %.5f %.4f %.4f" % (
        4100000000000000000 + k, ra[k], dec[k], plx[k], f_plx[k] * plx[k], pmra[k], e_pm[k], pmdec[k], e_pm[k],
        rv[k], e_rv[k]) for k in range(n)]


def pulsars(n, seed):
    """n pulsars (no parallax, no radial velocity) -> list of text lines (14 fields)."""
    i = np.arange(n)
    r = Stream(seed, 3, i)
    d = 10.0 ** (0.3 * r.gauss())                      # kpc, log-normal around 1 kpc
    l = r.uni(0.0, 2 * math.pi)
    b = np.radians(5.0) * r.gauss()
    pos = _helio_to_galcen(d, l, b)
    vel = circular_velocity(pos) + np.stack([r.gauss(), r.gauss(), r.gauss()], 1) * (265.0 / KMS_PER_KPCMYR)
    ra, dec, dist, pmra, pmdec, _ = astrometry(pos, vel)
    return ["JSYN%05d P %.6f %.6f 0.0000 0.0000 %.1f 0.250 %.4f 1.0000 %.4f 1.0000 nan nan" % (
        k, ra[k], dec[k], dist[k], pmra[k], pmdec[k]) for k in range(n)]


WORKLOADS = {
    # name: (cluster args, target generator)
    "pair64": (dict(n=64, dmax_pc=2000.0, tmax_fixed=20.0), lambda n, s: pulsars(n, s)),
    "screen": (dict(n=4087, dmax_pc=5000.0, n_no_rv=878), lambda n, s: stars(n, s)),
}


def write_workload(outdir, name, n_targets, seed, n_clusters=None):
    """Write outdir/clusters.txt and outdir/targets.txt for a named workload; returns the two paths."""
    cargs, tgen = WORKLOADS[name]
    cargs = dict(cargs)
    if n_clusters is not None:
        cargs["n"] = n_clusters
        if "n_no_rv" in cargs:
            cargs["n_no_rv"] = int(round(cargs["n_no_rv"] * n_clusters / 4087))
    os.makedirs(outdir, exist_ok=True)
    cp, tp = os.path.join(outdir, "clusters.txt"), os.path.join(outdir, "targets.txt")
    with open(cp, "w") as f:
        f.write("\n".join(clusters(seed=seed, **cargs)) + "\n")
    with open(tp, "w") as f:
        f.write("\n".join(tgen(n_targets, seed)) + "\n")
    return cp, tp
