"""One screen of a synthetic workload on the GPU, for profiling and quick checks.

    python -m phygas_gb300.run_screen --stars 20000 --precision mixed [--clusters 4087] [--seed 1001] [--repeat 1]
                                      [--parts 4]

Builds the synthetic star and cluster catalogues (phygas_gb300.synth, the `screen` workload), uploads the cluster
table, draws and stages the stars, runs the screen `--repeat` times and prints the row count and the device stage
times and work counts of the last run as one JSON line.  Nothing else runs on the GPU, so a profiler attached to
this command sees the cluster-table orbit launch first, then the screen's launches in order.
"""
import argparse
import json
import os
import sys
import tempfile

if __package__ in (None, ""):
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import phygas_gb300 as pg
from phygas_gb300 import synth


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--stars", type=int, default=20000)
    ap.add_argument("--clusters", type=int, default=None, help="default: the workload's 4,087")
    ap.add_argument("--seed", type=int, default=1001)
    ap.add_argument("--precision", choices=("mixed", "fp64"), default="mixed")
    ap.add_argument("--chi2-max", type=float, default=25.0)
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--parts", type=int, default=None,
                    help="parts of a chunk of at least 8,192 stars (pgx_screen_parts; 1 = screened whole; "
                         "default: about 1e7 star-cluster pairs a part)")
    a = ap.parse_args(argv)
    with tempfile.TemporaryDirectory() as d:
        cp, tp = synth.write_workload(d, "screen", a.stars, a.seed, a.clusters)
        clusters, stars = pg.read_clusters(cp), pg.read_targets(tp)
    tmax = max(c.tmax_myr for c in clusters)
    prec = pg.PGX_MIXED if a.precision == "mixed" else pg.PGX_FP64
    with pg.Context(a.device) as ctx:
        ctx.set_clusters(clusters)
        if a.parts is not None:
            ctx.set_split(0 if a.parts <= 1 else 8192, a.parts if a.parts >= 2 else None)
        ps0, sig, pre = pg.draw_targets(stars)
        ctx.stage(ps0, sig, pre)
        rows = 0
        for _ in range(a.repeat):
            rows = ctx.exec(tmax, a.chi2_max, prec)
        print(json.dumps({"stars": len(stars), "clusters": len(clusters), "precision": a.precision, "parts": a.parts,
                          "rows": rows, "stats": ctx.stats()}))


if __name__ == "__main__":
    main()
