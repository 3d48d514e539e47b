#!/usr/bin/env python3
"""Regenerate the golden fixtures in this directory (run in a container that has the reference checkout).

What it writes, all from the reference itself:
  bench_clusters.txt.gz, screen_in.txt.gz, pulsar_in.txt.gz
      the inputs of the reference's own benchmark profiles `screen` (2,000 stars x 4,087 clusters,
      "PHYGAS 1 screen 25 64 2 0.001") and `pulsar` (1 pulsar x 4,087 clusters, "PHYGAS 1 pair 100 0.05"), written by
      the reference's generator scripts/bench/make_bench_data.py --seed 1 (reference scripts/bench/profiles/*.wu)
  screen_rows.txt.gz, pulsar_rows.txt.gz
      the result rows of the reference BOINC app's CPU loop (built against its bench stub by oracle/Makefile) on those
      inputs; their SHA-1 prefixes must equal the published known answers (reference docs/BENCHMARK.md:366)
  ref_dump_*.txt.gz
      raw values (C99 hex floats) from oracle/_ref/ref_dump -- the reference core compiled from its own sources -- for
      small slices: draws, STM tracks, the chi2 scan and finish, pair draws/clones/reduce, tracks and the prefilter
  cli_<case>.txt.gz
      stdout of the reference's own phygas_screen CLI (oracle/_ref/phygas_screen, compiled from its sources) on a
      seeded synthetic workload (phygas_gb300.synth "screen": CLI_STARS stars, CLI_CLUSTERS clusters, seed CLI_SEED):
      default arguments, the chance-alignment control run, and other chi2_max / n_samp / r_kernel
  golden.json
      the published hashes, row counts and the commands above

usage: python3 tests/golden/make_golden.py [--ref /root/reference] [--only-cli]
"""
import argparse
import gzip
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
PUBLISHED = {"screen": ("3e860a4f0e51", 6387), "pulsar": ("73bd8776bd66", 4042)}
PROFILES = {
    "screen": dict(header="PHYGAS 1 screen 25 64 2 0.001", targets=2000, kind="S"),
    "pulsar": dict(header="PHYGAS 1 pair 100 0.05", targets=1, kind="P"),
}
# (name, dump arguments after the mode's input files) -- small slices, a few seconds each
DUMPS = [
    ("draws", ["draws", "C", "S", "0", "64", "64"]),
    ("lin_clusters", ["lin", "C", "S", "c", "0", "24", "64"]),
    ("lin_targets", ["lin", "C", "S", "t", "0", "3", "64"]),
    ("screen", ["screen", "C", "S", "0", "4", "25", "64", "2"]),
    ("chi2", ["chi2", "C", "S", "5", "6", "64", "2"]),
    ("pair_pulsar", ["pair", "C", "P", "0", "0", "4", "100", "0.05"]),
    ("pair_star", ["pair", "C", "S", "3", "0", "2", "40", "0.05"]),
    ("track", ["track", "C", "P", "0", "32"]),
]


# the CLI cases: (name, arguments after clusters.txt stars.txt)
CLI_STARS, CLI_CLUSTERS, CLI_SEED = 64, 1000, 1005
CLI_CASES = [("plain", []), ("control", ["25", "64", "2", "control"]), ("args", ["20", "32", "0"])]


def rows_hash(lines):
    return hashlib.sha1("".join(lines).encode()).hexdigest()[:12]


def write_gz(path, data):
    with gzip.GzipFile(path, "wb", mtime=0) as f:
        f.write(data if isinstance(data, bytes) else data.encode())


def make_cli(info):
    sys.path.insert(0, REPO)
    from phygas_gb300 import synth
    cli = os.path.join(REPO, "oracle", "_ref", "phygas_screen")
    info.setdefault("cli", {})
    with tempfile.TemporaryDirectory() as tmp:
        cp, tp = synth.write_workload(tmp, "screen", CLI_STARS, CLI_SEED, CLI_CLUSTERS)
        for name, args in CLI_CASES:
            out = subprocess.check_output([cli, cp, tp] + args, stderr=subprocess.DEVNULL)
            write_gz(os.path.join(HERE, "cli_%s.txt.gz" % name), out)
            info["cli"][name] = {"args": args, "rows": out.count(b"\n"), "sha1_12": hashlib.sha1(out).hexdigest()[:12],
                                 "workload": "synth screen %d stars %d clusters seed %d" % (CLI_STARS, CLI_CLUSTERS,
                                                                                             CLI_SEED)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("--only-cli", action="store_true", help="only the CLI fixtures (cli_*.txt.gz)")
    a = ap.parse_args()
    subprocess.check_call(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref", "REF=" + a.ref])
    if a.only_cli:
        with open(os.path.join(HERE, "golden.json")) as f:
            info = json.load(f)
        make_cli(info)
        with open(os.path.join(HERE, "golden.json"), "w") as f:
            json.dump(info, f, indent=1, sort_keys=True)
            f.write("\n")
        print("CLI fixtures written to", HERE)
        return
    app = os.path.join(REPO, "oracle", "_ref", "phygas_wu")
    dump = os.path.join(REPO, "oracle", "_ref", "ref_dump")
    info = {"published": {}, "commands": {}}
    with tempfile.TemporaryDirectory() as tmp:
        for prof, p in PROFILES.items():
            d = os.path.join(tmp, prof)
            cmd = [sys.executable, "-B", os.path.join(a.ref, "scripts", "bench", "make_bench_data.py"), d,
                   "--header", p["header"], "--clusters", "4087", "--targets", str(p["targets"]),
                   "--kind", p["kind"], "--seed", "1"]
            subprocess.check_call(cmd)
            info["commands"][prof + "_inputs"] = " ".join(["make_bench_data.py", "<outdir>"] + cmd[4:])
            subprocess.check_call([app], cwd=d, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            with open(os.path.join(d, "out")) as f:
                rows = [ln for ln in f if not ln.startswith("#")]
            h, n = rows_hash(rows), len(rows)
            if (h, n) != PUBLISHED[prof]:
                sys.exit("%s: reference app gives %s / %d rows, published %s / %d" % ((prof, h, n) + PUBLISHED[prof]))
            info["published"][prof] = {"sha1_12": h, "rows": n, "header": p["header"]}
            with open(os.path.join(d, "in"), "rb") as f:
                write_gz(os.path.join(HERE, prof + "_in.txt.gz"), f.read())
            write_gz(os.path.join(HERE, prof + "_rows.txt.gz"), "".join(rows))
            if prof == "screen":
                with open(os.path.join(d, "clusters"), "rb") as f:
                    write_gz(os.path.join(HERE, "bench_clusters.txt.gz"), f.read())
                shutil.copy(os.path.join(d, "clusters"), os.path.join(tmp, "C"))
                shutil.copy(os.path.join(d, "in"), os.path.join(tmp, "S"))
            else:
                shutil.copy(os.path.join(d, "in"), os.path.join(tmp, "P"))
        for name, args in DUMPS:
            argv = [dump] + [os.path.join(tmp, x) if x in ("C", "S", "P") else x for x in args]
            out = subprocess.check_output(argv)
            write_gz(os.path.join(HERE, "ref_dump_%s.txt.gz" % name), out)
            info["commands"]["ref_dump_" + name] = " ".join(args)
    make_cli(info)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(info, f, indent=1, sort_keys=True)
        f.write("\n")
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
