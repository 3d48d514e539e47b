"""Test infrastructure: golden fixtures and the CPU oracle (oracle/_build), for the tests and the smoke check only.

The oracle is the checker.  It is pinned bit for bit to the reference (tests/test_oracle.py); the GPU library is
compared against it with the tolerances of the hot-path contract:
  closest distance / time / chi2 / speeds    1e-6 relative
  p_r50, p_rtot, clone fractions              1e-4 absolute (in practice: identical counts out of 512 / m)
  pair sets at the cut                        identical, except pairs within 1e-6 (relative) of the cut
"""
import concurrent.futures as cf
import gzip
import hashlib
import os
import subprocess
import tempfile

TESTS = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(TESTS)
GOLDEN = os.path.join(TESTS, "golden")
ORACLE_BUILD = os.path.join(REPO, "oracle", "_build")
ORACLE_DUMP = os.path.join(ORACLE_BUILD, "oracle_dump")
ORACLE_WU = os.path.join(ORACLE_BUILD, "oracle_wu")
ORACLE_LIB = os.path.join(ORACLE_BUILD, "libphygas_oracle.so")

REL_TOL = 1e-6
PROB_TOL = 1e-4
PUBLISHED = {"screen": ("3e860a4f0e51", 6387), "pulsar": ("73bd8776bd66", 4042)}

_cache = None


def cache_dir():
    global _cache
    if _cache is None:
        _cache = tempfile.mkdtemp(prefix="phygas_golden_")
    return _cache


def unpack(name):
    """Decompressed copy of tests/golden/<name>.gz in a per-process cache directory; returns its path."""
    out = os.path.join(cache_dir(), name)
    if not os.path.exists(out):
        with gzip.open(os.path.join(GOLDEN, name + ".gz"), "rb") as f, open(out, "wb") as g:
            g.write(f.read())
    return out


def golden_inputs():
    clusters = unpack("bench_clusters.txt")

    def first_n(n):
        p = os.path.join(cache_dir(), "clusters_%d.txt" % n)
        if not os.path.exists(p):
            with open(clusters) as f:
                lines = f.readlines()[:n]
            with open(p, "w") as g:
                g.writelines(lines)
        return p

    return {"clusters": clusters, "screen": unpack("screen_in.txt"), "pulsar": unpack("pulsar_in.txt"),
            "clusters_path_n": first_n}


def golden_rows(profile):
    with gzip.open(os.path.join(GOLDEN, profile + "_rows.txt.gz"), "rt") as f:
        return f.readlines()


def rows_hash(lines):
    return hashlib.sha1("".join(lines).encode()).hexdigest()[:12]


def run(cmd, cwd=None):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, cwd=cwd)
    if r.returncode != 0:
        raise RuntimeError("%s failed (%d): %s" % (" ".join(cmd), r.returncode, r.stderr[-2000:]))
    return r.stdout


def hexf(s):
    return float.fromhex(s)


def oracle_screen(clusters, stars, j0, j1, cut=25.0, n_samp=64, r_kernel=2.0, dump=ORACLE_DUMP):
    """{(star, cluster): row} of the oracle's kept pairs (screen mode of oracle/dump_main.c)."""
    out = run([dump, "screen", clusters, stars, str(j0), str(j1), repr(cut), str(n_samp), repr(r_kernel)])
    res = {}
    for ln in out.splitlines():
        f = ln.split()
        res[(int(f[0]), int(f[1]))] = dict(chi2=hexf(f[2]), kb=int(f[3]), sb=hexf(f[4]), t_myr=hexf(f[5]),
                                           d_nom_pc=hexf(f[6]), sig_pc=hexf(f[7]), p_r50=hexf(f[8]),
                                           p_rtot=hexf(f[9]), vrel_kms=hexf(f[10]))
    return res


def oracle_lin(clusters, stars, which, i0, i1, n_samp=64, dump=ORACLE_DUMP):
    """{(object, point): [pos3, vel3, S6]} from the oracle's ph_lin_cluster / ph_lin_target."""
    out = run([dump, "lin", clusters, stars, which, str(i0), str(i1), str(n_samp)])
    res = {}
    for ln in out.splitlines():
        f = ln.split()
        res[(int(f[1]), int(f[2]))] = [hexf(x) for x in f[3:15]]
    return res


def parse_pair_dump(text):
    """oracle/dump_main.c pair mode -> list of dicts (one per pair) with draws, clone results and the reduction."""
    pairs, cur = [], None
    for ln in text.splitlines():
        f = ln.split()
        if f[0] == "draw":
            cur = dict(target=int(f[1]), cluster=int(f[2]), m=int(f[3]), steps=int(f[4]), dt=hexf(f[5]), ps=[],
                       clones=[])
            pairs.append(cur)
        elif f[0] == "ps":
            cur["ps"].append([hexf(x) for x in f[2:14]])
        elif f[0] == "clone":
            cur["clones"].append([hexf(x) for x in f[2:5]])
        elif f[0] == "res":
            cur["res"] = dict(n=int(f[3]), **{k: hexf(v) for k, v in zip(
                ("d05", "d50", "d95", "t05", "t50", "t95", "v05", "v50", "v95", "f_r50", "f_rtot"), f[4:15])})
    return pairs


def wu_rows(clusters, in_file, slices, wu=ORACLE_WU, workers=None):
    """Rows of a work unit from the oracle's work-unit runner, run as parallel slices; slices = [(j0, j1, i0, i1)]."""
    def one(s):
        return run([wu, clusters, in_file] + [str(x) for x in s])
    with cf.ThreadPoolExecutor(max_workers=workers or min(len(slices), os.cpu_count() or 4)) as ex:
        outs = list(ex.map(one, slices))
    lines = []
    for o in outs:
        lines.extend(ln + "\n" for ln in o.splitlines())
    return lines


def rel_err(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def close_rel(a, b, tol=REL_TOL, floor=0.0):
    return abs(a - b) <= tol * abs(b) + floor
