"""One batch of the pair Monte Carlo on the GPU, for profiling and quick checks.

    python -m phygas_gb300.run_pairs [--stars 2000] [--pairs 200] [--pulsars 1] [--seed 1003] [--repeat 1]
                                     [--streamed]

Builds the synthetic star and cluster catalogues (phygas_gb300.synth, the `screen` workload), screens the stars with
the mixed-precision screen, takes `--pairs` of the kept pairs with p_r50 >= 0.001 evenly spaced through the row list,
adds `--pulsars` synthetic pulsars against every cluster the prefilter keeps, draws 200, 500 or 1000 clones per pair
(seeded) at dt 0.05 Myr on the host, and runs the batch through pgx_pair `--repeat` times.  Prints the batch's
shape and the device time and work counts of the last run as one JSON line.  The clone kernel (k_pair_mc_t) is the
only launch of its name, so a profiler filtered on it sees the batch alone.
"""
import argparse
import json
import os
import sys
import tempfile
import time

if __package__ in (None, ""):
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import numpy as np

import phygas_gb300 as pg
from phygas_gb300 import synth


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--stars", type=int, default=2000)
    ap.add_argument("--pairs", type=int, default=200)
    ap.add_argument("--pulsars", type=int, default=1)
    ap.add_argument("--seed", type=int, default=1003)
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--streamed", action="store_true",
                    help="the pulsars' pairs from the GPU prefilter, then pgx_pair_targets over the whole list (host "
                         "draws of each batch of 1,024 pairs beside the tracing of the one before), timed end to end")
    a = ap.parse_args(argv)
    with tempfile.TemporaryDirectory() as d:
        cp, tp = synth.write_workload(d, "screen", a.stars, a.seed)
        clusters, stars = pg.read_clusters(cp), pg.read_targets(tp)
        pp = os.path.join(d, "pulsars.txt")
        with open(pp, "w") as f:
            f.write("\n".join(synth.pulsars(max(a.pulsars, 1), a.seed)) + "\n")
        pulsars = pg.read_targets(pp)[:a.pulsars]
    tmax = max(c.tmax_myr for c in clusters)
    with pg.Context(a.device) as ctx:
        ctx.set_clusters(clusters)
        rows = ctx.screen(*pg.draw_targets(stars), tmax)
        sel = np.flatnonzero(rows["p_r50"] >= 0.001)
        take = sel[np.unique(np.linspace(0, len(sel) - 1, min(a.pairs, len(sel))).astype(np.int64))] \
            if len(sel) and a.pairs > 0 else sel[:0]
        t0 = time.perf_counter()
        if not len(pulsars):
            pti, pci = (np.zeros(0, np.int32),) * 2
        elif a.streamed:
            pti, pci = ctx.prefilter(pulsars, clusters)
        else:
            pti, pci = pg.prefilter_pairs(pulsars, clusters)
        pref_s = time.perf_counter() - t0
        ti = np.concatenate([rows["star"][take], pti + len(stars)]).astype(np.int32)
        ci = np.concatenate([rows["cluster"][take], pci]).astype(np.int32)
        ncl = np.random.default_rng(a.seed).choice([200, 500, 1000], len(ti)).astype(np.int32)
        if a.streamed:
            targets = pg.as_array(list(stars) + list(pulsars), pg.PhTarget)
            t0 = time.perf_counter()
            res = ctx.pair_targets(targets, ti, clusters, ci, ncl, 0.05)
            wall = time.perf_counter() - t0
            st = ctx.stats()
            print(json.dumps({"screen_pairs": int(len(take)), "pulsars": int(len(pulsars)),
                              "pulsar_pairs": int(len(pti)), "pairs": int(len(ti)), "clones": int(st["clones"]),
                              "clone_steps": int(st["clone_steps"]), "prefilter_s": pref_s, "wall_s": wall,
                              "clone_steps_per_s_e2e": st["clone_steps"] / wall,
                              "f_r50_sum": float(res["f_r50"].sum())}))
            return
        batch = pg.draw_pair_batch(list(stars) + list(pulsars), ti, clusters, ci, ncl, 0.05)
        res = None
        for _ in range(a.repeat):
            res = ctx.pair(*batch)
        st = ctx.stats()
        print(json.dumps({"screen_pairs": int(len(take)), "pulsar_pairs": int(len(pti)), "pairs": int(len(ti)),
                          "clones": int(st["clones"]), "clone_steps": int(st["clone_steps"]), "ms_pair": st["ms_pair"],
                          "max_steps": int(batch[2].max()) if len(ti) else 0,
                          "f_r50_sum": float(res["f_r50"].sum()) if res is not None else 0.0}))


if __name__ == "__main__":
    main()
