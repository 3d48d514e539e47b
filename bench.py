#!/usr/bin/env python3
"""Benchmark of the stage-1 star x cluster screen on GB300 (one JSON line on stdout).

Workload: one screening chunk of 20,000 synthetic stars x 4,087 synthetic clusters (phygas_gb300.synth "screen",
seed 1001: the reference's stage-1 task size), chi2_max 25, n_samp 64, r_kernel 2.  A step screens the whole chunk:
FP64 orbits + STM covariances of the 20,000 stars, the scan of all 81.7 M pairs, and the 512-draw probabilities of
every kept pair, with the cluster table resident (built once, outside the timed region, as a serving process keeps
it).

  value         pairs/s of the mixed-precision screen, device time per chunk (CUDA events on the library's stream),
                star inputs (nominal state + covariance of the draws) already in HBM; L2 flushed between steps
  e2e           the same metric through the C-ABI call a user makes (pgx_screen_chunks): host star records in, host
                rows out, host draws and host<->device copies inside the timed region
  roofline      the step's largest kernel, the FP32 block filter: the survey's 126 flops per pair-point over
                its CUDA-event launch time, against the FP32 FMA peak measured in this run by the library's probe
  cpu_baseline  the oracle (a pinned C restatement of the reference's CPU code) on all host cores, bounded sample;
                its rows are kept and compared with the GPU's rows of the same stars (parity_vs_oracle)
  plain_fp64    the plain FP64 screen on the same chunk (the comparison the target is stated against)
The line ends with the evidence a reader checks first: the speed-up over the plain FP64 path, the mixed rows against
the FP64 rows, and the GPU rows against the oracle's on the sampled stars.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
Under torchrun (N > 1) every rank screens its own chunk (weak scaling, no data exchange); rank 0 prints.

Profiling modes (one JSON line each; nothing else runs on the GPU, so a profiler sees only their launches):
  python bench.py --mode screen [--stars 20000] [--clusters N] [--precision mixed|fp64] [--parts K] [--repeat R]
      one screen of a synthetic chunk (the cluster-table orbit launch first, then the screen's launches in order)
  python bench.py --mode refgpu [--stars 20000]
      the reference's own GPU kernels (oracle/_ref/ref_kernels.ptx, built from its source for sm_103a) driven as its
      app drives them, timed stage by stage beside this build's kernels on the benchmark chunk and a pulsar pair job,
      with the rows compared
  python bench.py --mode pairs [--stars 2000] [--pairs 200] [--pulsars 1] [--streamed]
      one batch of the pair Monte Carlo: --pairs kept screen pairs (p_r50 >= 0.001, evenly spaced) plus --pulsars
      synthetic pulsars against their prefiltered clusters, clones U{200,500,1000} at dt 0.05 Myr; with --streamed the
      pulsars' pairs come from the GPU prefilter and the whole list runs through pgx_pair_targets, timed end to end
      (--stars 20000 --pairs 10000 --pulsars 702 --streamed is the full batched uneven Monte Carlo configuration)
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

N_STARS, N_CLUSTERS, SEED = 20000, 4087, 1001
CHI2_MAX, N_SAMP, R_KERNEL, P_MIN = 25.0, 64, 2.0, 0.001
# the survey's algorithmic count for one pair-point of the screen (one track point of one star-cluster pair): 9 to
# build M, 6 for m0/m1, 44 per quad_inv x 2, 19 for the segment's nearest point and the interpolation
FLOPS_PER_PAIR_POINT = 126.0
# FP64 flops of one body step (one kick-drift-kick step of one orbit, its force evaluation included), from the
# executed FP64 instructions of k_stm_orbits per body step: 36.0 DFMA + 3.0 DADD + 29.0 DMUL (ncu sass op counters,
# FMA = 2 flops)
FLOPS_PER_BODY_STEP = 104.0
FP64_INSTR_PER_BODY_STEP = 36.0 + 3.0 + 29.0
# the same for one clone-step of the pair Monte Carlo (two body steps, and the FP64 segment test where the FP32 bound
# does not rule it out), from k_pair_mc_t on the 4,052-pair batch of `bench.py --mode pairs` (200 screen pairs of
# 2,000 stars + 1 pulsar x 3,852 prefiltered clusters): 73.3 DFMA + 9.3 DADD + 58.9 DMUL executed
FLOPS_PER_CLONE_STEP = 214.9
FP64_INSTR_PER_CLONE_STEP = 73.3 + 9.3 + 58.9
# DRAM traffic of one k_stm_orbits launch on the whole chunk (dram__bytes_read.sum + dram__bytes_write.sum, one ncu
# capture of `bench.py --mode screen --stars 20000 --parts 1`): 6.7 MB read + 711.9 MB of orbit output written
ORBIT_TRAFFIC_BYTES = 718.6e6
# DRAM traffic of the block filter k_mx_scan32_blocks per pair-point (read + write of one ncu capture of one part's
# launch, `bench.py --mode screen --stars 2500 --parts 1`: 6.30e8 pair-points); a part's launch moves its share
SCAN_TRAFFIC_PER_PAIR_POINT = (103.69e6 + 47.78e6) / 6.303e8
# warp instructions the block filter issues per pair-point (smsp__inst_executed.sum of the same capture: 3.57e9 for
# 6.30e8 pair-points); its issue bound is 4 warp instructions per clock per SM (one per scheduler)
SCAN_WARP_INSTR_PER_PAIR_POINT = 3.5741e9 / 6.303e8
ISSUE_PER_CLK_SM = 4


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def r4(x):
    """x to 4 significant digits (the compact evidence at the end of the line)."""
    if isinstance(x, float) and x != 0 and math.isfinite(x):
        return float("%.4g" % x)
    return x


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    return ws, int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0"))


class Clocks:
    """nvidia-smi samples (200 ms) during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device, self.p, self.lines = device, None, []

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                      stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.p = None
        return self

    def _read(self):
        for ln in self.p.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            self.p.wait()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def make_inputs(tmp, rank):
    from phygas_gb300 import synth
    seed = SEED + 7919 * rank
    cp, tp = synth.write_workload(tmp, "screen", N_STARS, seed)
    return cp, tp


def pair_points(clusters, n_stars, tmax):
    """Pair-points of a chunk: per star-cluster pair, the points both tracks have (the scan's loop count)."""
    npts_star = int(math.ceil(tmax / 0.5)) + 1
    return n_stars * sum(min(npts_star, int(math.ceil(c.tmax_myr / 0.5)) + 1) for c in clusters)


def cpu_baseline(cp, tp, stars_per_proc=192, procs=None, keep_rows=False):
    """Oracle screen on all host cores: P processes, each `stars_per_proc` stars x all clusters; pairs/s from the
    per-target loop time (the per-cluster precompute, done once per task by the reference, is timed apart).
    keep_rows: the processes write their kept pairs as raw records, returned (stars [0, P * stars_per_proc))."""
    import numpy as np
    import phygas_gb300 as pg
    from tests import oracle_tools as ot
    procs = procs or os.cpu_count() or 1
    with open(tp) as f:
        stars = f.readlines()
    tmp = tempfile.mkdtemp(prefix="phygas_cpu_")
    inp = os.path.join(tmp, "in")
    with open(inp, "w") as f:
        f.write("PHYGAS 1 screen %g %d %g 0\n" % (CHI2_MAX, N_SAMP, R_KERNEL))
        f.writelines(stars[:stars_per_proc * procs])
    env = dict(os.environ)
    if keep_rows:
        env["PHYGAS_WU_RAW"] = "1"
    # each process writes its rows to a file of its own (pipes read one after another would hold the others up)
    outf = [open(os.path.join(tmp, "rows%d" % p), "wb") if keep_rows else subprocess.DEVNULL for p in range(procs)]
    t0 = time.time()
    ps = [subprocess.Popen([ot.ORACLE_WU, cp, inp, str(p * stars_per_proc), str((p + 1) * stars_per_proc)],
                           stdout=outf[p], stderr=subprocess.PIPE, env=env) for p in range(procs)]
    runs, preps, outs = [], [], []
    for i, p in enumerate(ps):
        _, err = p.communicate()
        err = err.decode(errors="replace")
        if p.returncode:
            raise RuntimeError("oracle_wu failed: " + err[-500:])
        f = err.split("wu_time")[-1].split()
        preps.append(float(f[1]))
        runs.append(float(f[3]))
        if keep_rows:
            outf[i].close()
            with open(os.path.join(tmp, "rows%d" % i), "rb") as g:
                outs.append(g.read())
    wall = time.time() - t0
    pairs = stars_per_proc * procs * N_CLUSTERS
    res = {"value": pairs / max(runs), "unit": "pairs/s", "cores": procs, "kind": "port",
           "sample": "%d stars x %d clusters on %d processes (%d stars each); per-target loop %.1f s, cluster "
                     "precompute %.1f s per process (excluded), wall %.1f s" % (
                         stars_per_proc * procs, N_CLUSTERS, procs, stars_per_proc, max(runs), max(preps), wall),
           "loop_s": max(runs), "pairs": pairs}
    rows = np.frombuffer(b"".join(outs), pg.ROW_DTYPE) if keep_rows else None
    return res, rows


def compare_to_oracle(gpu, ora, n_stars, cut=CHI2_MAX, p_cut=P_MIN):
    """The GPU's rows of stars [0, n_stars) against the oracle's (the reference's CPU algorithm) on the same stars:
    the kept pair sets (chi2 < cut; pairs within 1e-6 relative of the cut in either are exempt), the emitted sets
    (p_r50 >= p_cut; exempt within 1e-6 of it), and over the pairs both keep: the largest and 99th-percentile
    relative error of chi2, t, d_nom, sig and vrel, the largest p_r50 / p_rtot difference and how many differ."""
    import numpy as np
    gpu = gpu[gpu["star"] < n_stars]
    key = lambda r: r["star"].astype(np.int64) * (1 << 32) + r["cluster"]
    kg, ko = key(gpu), key(ora)
    near = lambda r: np.abs(r["chi2"] - cut) <= 1e-6 * cut
    only_g = np.setdiff1d(kg, ko)
    only_o = np.setdiff1d(ko, kg)
    exempt = set(kg[near(gpu)].tolist()) | set(ko[near(ora)].tolist())
    bad_sets = [k for k in np.concatenate([only_g, only_o]).tolist() if k not in exempt]
    both, ig, io = np.intersect1d(kg, ko, assume_unique=True, return_indices=True)
    a, b = gpu[ig], ora[io]
    em_g = set(kg[gpu["p_r50"] >= p_cut].tolist())
    em_o = set(ko[ora["p_r50"] >= p_cut].tolist())
    near_p = set(kg[np.abs(gpu["p_r50"] - p_cut) <= 1e-6].tolist()) | set(ko[np.abs(ora["p_r50"] - p_cut) <= 1e-6]
                                                                          .tolist())
    em_bad = [k for k in (em_g ^ em_o) if k not in near_p]

    def rel(f, floor=1e-300):
        x = np.abs(a[f] - b[f]) / np.maximum(np.abs(b[f]), floor)
        return {"max": r4(float(x.max())) if len(x) else 0.0,
                "p99": r4(float(np.quantile(x, 0.99))) if len(x) else 0.0}
    dp50, dpt = np.abs(a["p_r50"] - b["p_r50"]), np.abs(a["p_rtot"] - b["p_rtot"])
    gi, oi = {k: i for i, k in enumerate(kg.tolist())}, {k: i for i, k in enumerate(ko.tolist())}
    detail = [{"star": int(k >> 32), "cluster": int(k & 0xffffffff),
               "chi2_gpu": float(gpu["chi2"][gi[k]]) if k in gi else None,
               "chi2_oracle": float(ora["chi2"][oi[k]]) if k in oi else None} for k in bad_sets[:4]]
    return {"stars": int(n_stars), "rows_gpu": int(len(gpu)), "rows_oracle": int(len(ora)),
            "kept_set_mismatches": len(bad_sets), "kept_set_mismatch_pairs": detail,
            "emitted_gpu": len(em_g), "emitted_oracle": len(em_o),
            "emitted_set_mismatches": len(em_bad), "argmin_point_differs": int(np.sum(a["kb"] != b["kb"])),
            "chi2_rel_floor1": rel("chi2", 1.0), "t_rel": rel("t_myr"), "d_nom_rel": rel("d_nom_pc"),
            "sig_rel": rel("sig_pc"),
            "vrel_rel": rel("vrel_kms"),
            "p_r50_abs_max": r4(float(dp50.max())) if len(dp50) else 0.0, "p_r50_differ": int(np.sum(dp50 > 0)),
            "p_rtot_abs_max": r4(float(dpt.max())) if len(dpt) else 0.0, "p_rtot_differ": int(np.sum(dpt > 0)),
            "contract": "sets identical except within 1e-6 of a cut; d, t within 1e-6 rel; p within 1e-4 abs"}


# Batched uneven Monte Carlo (the benchmark spec's C3 shape, scaled to a benchmark step): C3_SCREEN_PAIRS pairs from the
# mixed screen's rows with p_r50 >= 0.001, plus C3_PULSARS synthetic pulsars x their prefiltered clusters; clone
# counts uniform in {200, 500, 1000}; steps = ceil(tmax / 0.05 Myr).  A synthetic pulsar (pm error 1 mas/yr, no
# parallax) reaches ~96 % of the 4,087 clusters, so the 702 pulsars of the full configuration are ~1e12 clone-steps
# (about 5 minutes: `bench.py --mode pairs --stars 20000 --pairs 10000 --pulsars 702 --streamed`); two stand in for
# them here.
C3_SCREEN_PAIRS, C3_PULSARS, C3_SEED = 10000, 2, 1003


def pair_cpu_baseline(cp, pp, n_clones=200, clusters_per_proc=24, procs=None):
    """Oracle pair Monte Carlo on all host cores: process p traces pulsar 0 against clusters
    [p * k, (p + 1) * k) (prefiltered, n_clones clones each); clone-steps/s from the slowest process's loop time."""
    from tests import oracle_tools as ot
    import phygas_gb300 as pg
    procs = procs or os.cpu_count() or 1
    tmp = tempfile.mkdtemp(prefix="phygas_cpu_pair_")
    inp = os.path.join(tmp, "in")
    with open(pp) as f, open(inp, "w") as g:
        g.write("PHYGAS 1 pair %d 0.05\n" % n_clones)
        g.write(f.readline())
    k = clusters_per_proc
    ps = [subprocess.Popen([ot.ORACLE_WU, cp, inp, "0", "1", str(p * k), str((p + 1) * k)], stdout=subprocess.PIPE,
                           stderr=subprocess.PIPE, text=True) for p in range(procs)]
    tmax = {c.name.decode(): c.tmax_myr for c in pg.read_clusters(cp)}
    runs, clone_steps = [], 0
    for p in ps:
        out, err = p.communicate()
        if p.returncode:
            raise RuntimeError("oracle_wu pair failed: " + err[-500:])
        runs.append(float(err.split("wu_time")[-1].split()[3]))
        for ln in out.splitlines():
            f = ln.split()
            clone_steps += int(f[3]) * int(math.ceil(tmax[f[1]] / 0.05 - 1e-9))
    return {"value": clone_steps / max(runs), "unit": "clone-steps/s", "cores": procs, "kind": "port",
            "sample": "1 synthetic pulsar x %d prefiltered clusters (%d per process) x %d clones, %.3g clone-steps; "
                      "slowest process %.1f s" % (procs * k, k, n_clones, clone_steps, max(runs))}


def pair_mc_measure(ctx, stars, clusters, cp, rows, want_cpu, fp64_peak):
    """C3-style batch: draws on the host, the autotuner on a sample of it, then the batch timed on the GPU."""
    import numpy as np
    import phygas_gb300 as pg
    from phygas_gb300 import synth
    sel = np.flatnonzero(rows["p_r50"] >= P_MIN)
    take = sel[np.unique(np.linspace(0, len(sel) - 1, min(C3_SCREEN_PAIRS, len(sel))).astype(np.int64))]
    tmp = tempfile.mkdtemp(prefix="phygas_c3_")
    pp = os.path.join(tmp, "pulsars.txt")
    with open(pp, "w") as f:
        f.write("\n".join(synth.pulsars(C3_PULSARS, C3_SEED)) + "\n")
    pulsars = pg.read_targets(pp)
    # the prefilter on the GPU (first call: the cluster tracks too; second: the targets only, the cluster side kept),
    # and the host code it replaces, which must keep the same pairs
    pref_s = []
    for _ in range(2):
        t0 = time.perf_counter()
        pti, pci = ctx.prefilter(pulsars, clusters)
        pref_s.append(time.perf_counter() - t0)
    pref_st = ctx.stats()
    t0 = time.perf_counter()
    hti, hci = pg.prefilter_pairs(pulsars, clusters)
    t_pref_host = time.perf_counter() - t0
    if not (np.array_equal(hti, pti) and np.array_equal(hci, pci)):
        raise RuntimeError("pgx_prefilter kept other pairs than the host code")
    targets = list(stars) + list(pulsars)
    ti = np.concatenate([rows["star"][take], pti + len(stars)]).astype(np.int32)
    ci = np.concatenate([rows["cluster"][take], pci]).astype(np.int32)
    ncl = np.random.default_rng(C3_SEED).choice([200, 500, 1000], len(ti)).astype(np.int32)
    # the clones drawn into page-locked memory (allocated once, outside the timing), so the batch's H2D runs at the
    # link's rate
    pinned = pg.HostBuffer(12 * int(ncl.sum()))
    t0 = time.perf_counter()
    batch = pg.draw_pair_batch(targets, ti, clusters, ci, ncl, 0.05, out_ps=pinned.array)
    t_draw = time.perf_counter() - t0
    # the same draws on the GPU (pgx_draw_pair_batch_gpu): wall time of the call (records in, clones out) and the
    # draw kernel's device time
    ctx.draw_pair_batch(targets, ti[:64], clusters, ci[:64], ncl[:64], 0.05)        # warm-up
    t0 = time.perf_counter()
    ctx.draw_pair_batch(targets, ti, clusters, ci, ncl, 0.05)
    t_draw_gpu = time.perf_counter() - t0
    draw_gpu_ms = ctx.stats()["ms_total"]
    best, table = ctx.tune_pair(*pg.draw_pair_batch(targets, ti[::25], clusters, ci[::25], ncl[::25], 0.05))
    ctx.pair(*batch)                                         # warm-up
    ms = []
    for _ in range(2):
        ctx.pair(*batch)
        st = ctx.stats()
        ms.append(st["ms_pair"])
    cs = st["clone_steps"]
    # end to end: host records -> clone draws (batches of 1,024 pairs, each drawn while the GPU traces the one
    # before) -> GPU -> results, one pgx_pair_targets call
    e2e_walls = []
    targets_arr = pg.as_array(targets, pg.PhTarget)
    for _ in range(2):
        t0 = time.perf_counter()
        ctx.pair_targets(targets_arr, ti, clusters, ci, ncl, 0.05)
        e2e_walls.append(time.perf_counter() - t0)
    rate = cs / (statistics.mean(ms) * 1e-3)
    out = {"metric": "clone-steps/s", "value": rate, "unit": "clone-steps/s", "ms_per_batch": statistics.mean(ms),
           "workload": "%d screen pairs (p_r50 >= 0.001) + %d pulsars x %d prefiltered clusters; clones U{200,500,1000}, "
                       "dt 0.05 Myr" % (len(take), C3_PULSARS, len(pti)),
           "pairs": int(len(ti)), "clones": int(st["clones"]), "clone_steps": int(cs),
           "launch": "one captured CUDA graph (prep, persistent trace, reduce) per shape, replayed per batch",
           "roofline": {"bound": "fp64", "kernel": "k_pair_mc_t", "achieved": FLOPS_PER_CLONE_STEP * rate / 1e12,
                        "peak": fp64_peak / 1e12, "unit": "TFLOP/s", "frac": FLOPS_PER_CLONE_STEP * rate / fp64_peak,
                        "peak_source": "FP64 FMA probe kernel of this run (pgx_peaks)",
                        "flops_per_clone_step": FLOPS_PER_CLONE_STEP,
                        "fp64_instr_frac": FP64_INSTR_PER_CLONE_STEP * rate / (fp64_peak / 2)},
           "autotune": {"chosen": {"warps_per_block": table[best][0], "clones_per_lane": table[best][1],
                                   "min_blocks_per_sm": table[best][2]},
                        "ms_on_sample": [{"warps_per_block": w, "clones_per_lane": c, "min_blocks_per_sm": b,
                                          "ms": r4(t)} for w, c, b, t in table]},
           "e2e": {"value": cs / min(e2e_walls), "unit": "clone-steps/s", "s_per_step": min(e2e_walls),
                   "how": "pgx_pair_targets: host clone draws of each batch of 1,024 pairs overlap the GPU's tracing "
                          "of the one before (page-locked buffers)",
                   "host_draw_s_unpipelined": t_draw,
                   "device_draws": {"call_s": t_draw_gpu, "kernel_ms": draw_gpu_ms,
                                    "how": "pgx_draw_pair_batch_gpu: the same clones drawn on the GPU"},
                   "prefilter_s": {"gpu_first_call": pref_s[0], "gpu_clusters_kept": pref_s[1],
                                   "gpu_device_ms": pref_st["ms_prefilter"],
                                   "host_decided_pairs": pref_st["prefilter_rechecked"],
                                   "host_code": t_pref_host},
                   "h2d_bytes_per_step": int(12 * 8 * st["clones"] + 28 * len(ti)),
                   "d2h_bytes_per_step": int(96 * len(ti))},
           "cpu_baseline": None}
    if want_cpu:
        try:
            out["cpu_baseline"] = pair_cpu_baseline(cp, pp)
        except Exception as e:
            log("pair cpu baseline failed: %s" % e)
    return out


# Serving (the benchmark spec's C4 shape): a seeded Poisson stream through the request loop with SERVE_SLOTS slots --
# screen and control chunks of 1,000-20,000 of the benchmark stars and single-pulsar Monte Carlo jobs (4,087
# clusters with the prefilter, 1000 clones).  SERVE_JOBS jobs with the mixed screen, so that the 99th percentile is
# one; the first SERVE_JOBS_FP64 of the same stream again with the plain FP64 screen (whose screen jobs are ~35x
# longer) for the comparison.
# The rate keeps the GPU about 60 % busy with the mixed screen (a pulsar job is ~0.7 s of clone tracing): latency, not
# a queue that grows without end.
SERVE_JOBS, SERVE_JOBS_FP64, SERVE_RATE_HZ, SERVE_SLOTS, SERVE_SEED = 200, 40, 2.0, 3, 1004
# the request loop's clone throughput under a backlog: SERVE_BACKLOG single-pulsar jobs submitted at once (the
# stream's rate limits the clone-steps/s of the mixed stream above, not the GPU)
SERVE_BACKLOG = 12
# chunks of the benchmark's stars per end-to-end run (the pipeline's fill is spread over them)
E2E_CHUNKS = 8


def compare_rows(mixed, fp64, cut=P_MIN):
    """The mixed-precision rows against the FP64 path's on the same chunk: pair sets (all kept pairs, and those with
    p_r50 >= cut), and the largest and 99th-percentile differences of d_min (relative), t_min (relative), p_r50 and
    p_rtot (absolute) over the pairs both keep."""
    import numpy as np
    key = lambda r: r["star"].astype(np.int64) * (1 << 32) + r["cluster"]
    km, kf = key(mixed), key(fp64)
    both, im, jf = np.intersect1d(km, kf, assume_unique=True, return_indices=True)
    a, b = mixed[im], fp64[jf]
    em, ef = set(km[mixed["p_r50"] >= cut].tolist()), set(kf[fp64["p_r50"] >= cut].tolist())

    def stat(x):
        x = np.abs(x)
        return {"max": r4(float(x.max())) if len(x) else 0.0, "p99": r4(float(np.quantile(x, 0.99))) if len(x) else 0.0}
    rel = lambda u, v: (u - v) / np.where(v != 0, np.abs(v), 1.0)
    return {"rows_mixed": int(len(mixed)), "rows_fp64": int(len(fp64)), "rows_both": int(len(both)),
            "emitted_mixed": len(em), "emitted_fp64": len(ef), "emitted_differ": len(em ^ ef),
            "rows_bitwise_identical": bool(len(mixed) == len(fp64) and mixed.tobytes() == fp64.tobytes()),
            "d_nom_rel": stat(rel(a["d_nom_pc"], b["d_nom_pc"])), "t_rel": stat(rel(a["t_myr"], b["t_myr"])),
            "p_r50_abs": stat(a["p_r50"] - b["p_r50"]), "p_rtot_abs": stat(a["p_rtot"] - b["p_rtot"])}


def cli_measure(cp, tp, reps=2):
    """The screen CLI end to end (process start, inputs read, cluster table, the pipelined chunks, the lines
    formatted on the GPU and written to /dev/null): wall time, best of `reps`."""
    import phygas_gb300 as pg
    walls, err = [], ""
    for _ in range(reps):
        t0 = time.perf_counter()
        with open(os.devnull, "w") as dn:
            r = subprocess.run([pg.SCREEN_CLI, cp, tp], stdout=dn, stderr=subprocess.PIPE, text=True)
        walls.append(time.perf_counter() - t0)
        err = r.stderr
        if r.returncode:
            raise RuntimeError("phygas_screen: %s" % err.strip()[-200:])
    kept = 0
    for line in err.splitlines():
        if "pairs kept" in line:
            kept = int(line.split(",")[1].split()[0])
    return {"cmd": "phygas_screen clusters.txt stars.txt > /dev/null (%d stars x %d clusters)" % (N_STARS, N_CLUSTERS),
            "wall_s": min(walls), "rows": kept, "pairs_per_s": N_STARS * N_CLUSTERS / min(walls),
            "text": "lines formatted on the GPU (pgx_screen_chunks_text)"}


def serving_measure(cp, tp):
    import phygas_gb300 as pg
    from phygas_gb300 import synth
    pp = os.path.join(tempfile.mkdtemp(prefix="phygas_serve_"), "pulsars.txt")
    with open(pp, "w") as f:
        f.write("\n".join(synth.pulsars(64, SERVE_SEED)) + "\n")
    out = {"workload": "Poisson %.2f/s (seed %d): 40 %% screen, 20 %% control chunks of 1,000-20,000 stars, 40 %% "
                       "single-pulsar jobs (4,087 clusters, prefilter, 1000 clones); %d slots; %d jobs mixed, the "
                       "first %d of the same stream with the FP64 screen"
                       % (SERVE_RATE_HZ, SERVE_SEED, SERVE_SLOTS, SERVE_JOBS, SERVE_JOBS_FP64)}
    for prec, jobs_n in (("mixed", SERVE_JOBS), ("fp64", SERVE_JOBS_FP64)):
        r = subprocess.run([pg.SERVE_CLI, cp, tp, pp, str(jobs_n), str(SERVE_RATE_HZ), str(SERVE_SLOTS), prec,
                            str(SERVE_SEED)], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
        lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
        summ = [x for x in lines if x.get("summary")]
        jobs = [x for x in lines if not x.get("summary")]
        if r.returncode or not summ:
            raise RuntimeError("phygas_serve %s failed: %s" % (prec, r.stderr[-400:]))
        s = dict(summ[0])
        s.pop("summary")
        s["latency_by_kind_p50_s"] = {k: r4(statistics.median([x["latency_s"] for x in jobs if x["kind"] == k] or [0.0]))
                                      for k in ("screen", "control", "pulsar")}
        s["jobs_by_kind"] = {k: sum(1 for x in jobs if x["kind"] == k) for k in ("screen", "control", "pulsar")}
        out[prec] = s
    env = dict(os.environ, PHYGAS_SERVE_MIX="pairs")
    r = subprocess.run([pg.SERVE_CLI, cp, tp, pp, str(SERVE_BACKLOG), "1000", str(SERVE_SLOTS), "mixed",
                        str(SERVE_SEED + 1)], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, env=env)
    summ = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{") and '"summary"' in x]
    if r.returncode or not summ:
        raise RuntimeError("phygas_serve backlog failed: %s" % r.stderr[-400:])
    out["pair_backlog"] = {"jobs": SERVE_BACKLOG, "how": "single-pulsar jobs submitted at once, %d slots" % SERVE_SLOTS,
                           "wall_s": summ[0]["wall_s"], "clone_steps_per_s": summ[0]["clone_steps_per_s"],
                           "latency_p50_s": summ[0]["latency_p50_s"]}
    return out


def reference_arm(args):
    """The reference's CPU screen (the oracle port: the reference's own binaries are not built on the GPU machine) on all
    host cores, each step a bounded sample of the workload: ms_per_step is that sample's measured loop time and
    pairs_per_step its pairs; the rate is pairs/s as for this build's arm."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    import __graft_entry__
    __graft_entry__.build_oracle()
    with tempfile.TemporaryDirectory() as tmp:
        cp, tp = make_inputs(tmp, 0)
        vals = []
        for i in range(args.warmup + args.steps):
            r, _ = cpu_baseline(cp, tp, stars_per_proc=32)
            if i >= args.warmup:
                vals.append(r)
        v = statistics.median(x["value"] for x in vals)
        base = dict(vals[-1])
        base["value"] = v
        ms = statistics.median(x["loop_s"] for x in vals) * 1e3
        print(json.dumps({"impl": "reference", "metric": "pairs/s", "value": v, "unit": "pairs/s",
                          "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                          "ms_per_step": ms, "pairs_per_step": vals[-1]["pairs"],
                          "step": "one bounded sample: %s" % vals[-1]["sample"],
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                          "data": "synthetic", "config": config(args),
                          "cpu_baseline": base,
                          "e2e": {"value": v, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))


def scan_roofline(stats, clocks, pp, fp32_peak, parts):
    """The step's largest kernel, the block filter k_mx_scan32_blocks (one launch per part), against the FP32 FMA
    peak: the survey's 126 flops per pair-point over the launches' CUDA-event time; with it the issue-slot fraction
    (the bound that
    applies to its mix of FP32, integer and compare work) from the warp instructions per pair-point of an ncu
    capture, at the SM clock sampled during the steps."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz")
    ms = statistics.mean(x["ms_scan"] for x in stats)
    if not ms:
        return None
    flops = FLOPS_PER_PAIR_POINT * pp
    out = {"bound": "fp32", "kernel": "k_mx_scan32_blocks", "achieved": flops / (ms * 1e-3) / 1e12,
           "peak": fp32_peak / 1e12, "unit": "TFLOP/s", "frac": flops / (ms * 1e-3) / fp32_peak,
           "peak_source": "FP32 FMA probe kernel of this run (pgx_peaks); not in MEASURED_PEAKS.json",
           "traffic": SCAN_TRAFFIC_PER_PAIR_POINT * pp / parts,
           "flops_per_pair_point": FLOPS_PER_PAIR_POINT, "pair_points_per_launch": pp / parts,
           "launches_per_step": parts, "ms_per_launch": ms / parts,
           "per_launch": "means over the step's launches (its parts ramp up in size); achieved and frac from their sum"}
    if mhz:
        out["issue_frac"] = SCAN_WARP_INSTR_PER_PAIR_POINT * pp / (ms * 1e-3) / (ISSUE_PER_CLK_SM * sms * mhz * 1e6)
    return out


def config(args):
    return {"workload": "screen: %d stars x %d clusters (synthetic, seed %d), chi2_max %g, n_samp %d, r_kernel %g"
                        % (N_STARS, N_CLUSTERS, SEED, CHI2_MAX, N_SAMP, R_KERNEL),
            "stars": N_STARS, "clusters": N_CLUSTERS, "pairs_per_step": N_STARS * N_CLUSTERS,
            "l2": "flushed between steps (256 MiB write)", "cluster_table": "resident, built once outside timing",
            "parallelism": ("%d ranks, a star chunk each (no data exchange)" % args.gpus) if args.gpus > 1
                           else "single GPU"}


def mode_screen(a):
    """One screen of a synthetic chunk, for profiling: the cluster table first, then the screen `--repeat` times;
    prints the row count and the last run's device stage times and work counts."""
    import phygas_gb300 as pg
    from phygas_gb300 import synth
    import __graft_entry__
    __graft_entry__.build()
    with tempfile.TemporaryDirectory() as d:
        cp, tp = synth.write_workload(d, "screen", a.stars, a.seed or SEED, a.clusters)
        clusters, stars = pg.read_clusters(cp), pg.read_targets(tp)
    tmax = max(c.tmax_myr for c in clusters)
    prec = pg.PGX_MIXED if a.precision == "mixed" else pg.PGX_FP64
    with pg.Context(0) as ctx:
        ctx.set_clusters(clusters)
        if a.parts is not None:
            ctx.set_split(0 if a.parts <= 1 else 8192, a.parts if a.parts >= 2 else None)
        ps0, sig, pre = pg.draw_targets(stars)
        ctx.stage(ps0, sig, pre)
        rows = 0
        for _ in range(a.repeat):
            rows = ctx.exec(tmax, CHI2_MAX, prec)
        print(json.dumps({"mode": "screen", "stars": len(stars), "clusters": len(clusters), "precision": a.precision,
                          "parts": a.parts, "rows": rows, "pair_points": pair_points(clusters, len(stars), tmax),
                          "stats": ctx.stats()}))


def mode_pairs(a):
    """One batch of the pair Monte Carlo, for profiling (k_pair_mc_t is the only launch of its name), or with
    --streamed the whole list end to end through pgx_prefilter and pgx_pair_targets."""
    import numpy as np
    import phygas_gb300 as pg
    from phygas_gb300 import synth
    import __graft_entry__
    __graft_entry__.build()
    seed = a.seed or C3_SEED
    with tempfile.TemporaryDirectory() as d:
        cp, tp = synth.write_workload(d, "screen", a.stars, seed)
        clusters, stars = pg.read_clusters(cp), pg.read_targets(tp)
        pp = os.path.join(d, "pulsars.txt")
        with open(pp, "w") as f:
            f.write("\n".join(synth.pulsars(max(a.pulsars, 1), seed)) + "\n")
        pulsars = pg.read_targets(pp)[:a.pulsars]
    tmax = max(c.tmax_myr for c in clusters)
    with pg.Context(0) as ctx:
        ctx.set_clusters(clusters)
        rows = ctx.screen(*pg.draw_targets(stars), tmax)
        sel = np.flatnonzero(rows["p_r50"] >= P_MIN)
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
        ncl = np.random.default_rng(seed).choice([200, 500, 1000], len(ti)).astype(np.int32)
        if a.streamed:
            targets = pg.as_array(list(stars) + list(pulsars), pg.PhTarget)
            t0 = time.perf_counter()
            res = ctx.pair_targets(targets, ti, clusters, ci, ncl, 0.05)
            wall = time.perf_counter() - t0
            st = ctx.stats()
            print(json.dumps({"mode": "pairs", "streamed": True, "screen_pairs": int(len(take)),
                              "pulsars": int(len(pulsars)), "pulsar_pairs": int(len(pti)), "pairs": int(len(ti)),
                              "clones": int(st["clones"]), "clone_steps": int(st["clone_steps"]),
                              "prefilter_s": pref_s, "wall_s": wall, "clone_steps_per_s_e2e": st["clone_steps"] / wall,
                              "f_r50_sum": float(res["f_r50"].sum())}))
            return
        batch = pg.draw_pair_batch(list(stars) + list(pulsars), ti, clusters, ci, ncl, 0.05)
        res = None
        for _ in range(a.repeat):
            res = ctx.pair(*batch)
        st = ctx.stats()
        print(json.dumps({"mode": "pairs", "screen_pairs": int(len(take)), "pulsar_pairs": int(len(pti)),
                          "pairs": int(len(ti)), "clones": int(st["clones"]), "clone_steps": int(st["clone_steps"]),
                          "ms_pair": st["ms_pair"], "max_steps": int(batch[2].max()) if len(ti) else 0,
                          "f_r50_sum": float(res["f_r50"].sum()) if res is not None else 0.0}))


def _ref_gpu_run(cp, wu, j0=None, j1=None):
    """The reference's own GPU kernels driven as its app drives them (oracle/_build/ref_gpu): rows and times."""
    ptx = os.path.join(REPO, "oracle", "_ref", "ref_kernels.ptx")
    exe = os.path.join(REPO, "oracle", "_build", "ref_gpu")
    if not (os.path.exists(ptx) and os.path.exists(exe)):
        raise RuntimeError("reference-GPU comparator not built (%s, %s)" % (ptx, exe))
    cmd = [exe, cp, wu, ptx] + ([str(j0), str(j1)] if j0 is not None else [])
    t0 = time.perf_counter()
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    wall = time.perf_counter() - t0
    if r.returncode:
        raise RuntimeError("ref_gpu failed: %s" % r.stderr[-800:])
    f = r.stderr.split("ref_gpu_time")[-1].split()
    t = {f[i]: float(f[i + 1]) for i in range(0, len(f) - 1, 2) if f[i] in ("prep", "total", "host")}
    for i, k in enumerate(f):
        if k in ("lin", "chi2", "finish", "pair"):
            t[k + "_s"], t[k + "_launches"] = float(f[i + 1]), int(f[i + 2])
        if k in ("pairs", "clones", "clone_steps"):
            t[k] = int(f[i + 1])
    t["process_wall_s"] = wall
    return r.stdout.splitlines(), t, [ln for ln in r.stderr.splitlines() if ln.startswith("GPU ")]


def mode_refgpu(a):
    """The reference's GPU kernels (built from its source for sm_103a, driven as its BOINC app drives them) timed
    on this GPU beside this build's kernels on the same inputs, stage by stage, with the rows compared:
      screen  20,000 stars x 4,087 clusters (the benchmark chunk), work unit "PHYGAS 1 screen 25 64 2 0.001"
      pairs   1 synthetic pulsar x 4,087 clusters (prefilter) x 100 clones, "PHYGAS 1 pair 100 0.05"."""
    import numpy as np
    import phygas_gb300 as pg
    from phygas_gb300 import synth
    import __graft_entry__
    __graft_entry__.build()
    out = {"mode": "refgpu"}
    tmp = tempfile.mkdtemp(prefix="phygas_refgpu_")
    cp, tp = synth.write_workload(tmp, "screen", a.stars or N_STARS, a.seed or SEED)
    clusters, stars = pg.read_clusters(cp), pg.read_targets(tp)
    tmax = max(c.tmax_myr for c in clusters)
    wu = os.path.join(tmp, "wu_screen")
    with open(tp) as f, open(wu, "w") as g:
        g.write("PHYGAS 1 screen %g %d %g %g\n" % (CHI2_MAX, N_SAMP, R_KERNEL, P_MIN))
        g.writelines(f.readlines())
    with Clocks(0) as clk:
        ref_rows, ref_t, ref_msg = _ref_gpu_run(cp, wu)
    out["screen_reference_gpu"] = dict(ref_t, summary=ref_msg, clocks=clk.summary())
    mine = {}
    with pg.Context(0) as ctx:
        ctx.set_clusters(clusters, N_SAMP, R_KERNEL)
        ps0, sig, pre = pg.draw_targets(stars, N_SAMP)
        for prec, name in ((pg.PGX_FP64, "fp64"), (pg.PGX_MIXED, "mixed")):
            ctx.set_split(0 if prec == pg.PGX_FP64 else 8192)
            ctx.stage(ps0, sig, pre)
            ctx.exec(tmax, CHI2_MAX, prec)                    # warm-up
            n = ctx.exec(tmax, CHI2_MAX, prec)
            st = ctx.stats()
            mine[name] = {k: r4(st[k]) for k in ("ms_total", "ms_orbit", "ms_cov", "ms_scan", "ms_select",
                                                 "ms_finish")}
            rows = ctx.fetch(n)
        # the end-to-end call a user makes, for the app's whole-loop time
        t0 = time.perf_counter()
        ctx.screen_chunks(pg.as_array(stars, pg.PhTarget), 20000, tmax, lambda first, r: None, CHI2_MAX,
                          pg.PGX_MIXED)
        mine["e2e_s"] = r4(time.perf_counter() - t0)
    out["screen_this_build_ms"] = mine
    got = []
    for r in rows[rows["p_r50"] >= P_MIN]:
        t, c = stars[r["star"]], clusters[r["cluster"]]
        got.append("%s %s %s %.3f %.3f %.2f %.2f %.4f %.4f %.2f" % (
            t.id.decode(), c.name.decode(), c.kind.decode(), r["chi2"], r["t_myr"], r["d_nom_pc"], r["sig_pc"],
            r["p_r50"], r["p_rtot"], r["vrel_kms"]))
    key = lambda ln: tuple(ln.split()[:2])
    kr, kg = {key(x): x for x in ref_rows}, {key(x): x for x in got}
    out["screen_rows"] = {"reference_gpu": len(ref_rows), "this_build": len(got),
                          "only_reference_gpu": len(set(kr) - set(kg)), "only_this_build": len(set(kg) - set(kr)),
                          "identical_lines": sum(1 for k in set(kr) & set(kg) if kr[k] == kg[k])}
    rt = ref_t
    out["screen_stage_speedup"] = {
        "orbits (pg_lin_k vs k_stm_orbits + k_stm_cov, FP64)": r4(rt["lin_s"] * 1e3 / (mine["fp64"]["ms_orbit"] +
                                                                                      mine["fp64"]["ms_cov"])),
        "chi2 (pg_chi2_k vs k_scan64, FP64)": r4(rt["chi2_s"] * 1e3 / mine["fp64"]["ms_scan"]),
        "chi2 (pg_chi2_k vs k_mx_scan32 + the FP64 selection, mixed)": r4(
            rt["chi2_s"] * 1e3 / (mine["mixed"]["ms_scan"] + mine["mixed"]["ms_select"])),
        "finish (pg_finish_k vs k_finish64, FP64)": r4(rt["finish_s"] * 1e3 / mine["fp64"]["ms_finish"]),
        "finish (pg_finish_k vs k_mx_finish32, mixed)": r4(rt["finish_s"] * 1e3 / mine["mixed"]["ms_finish"]),
        "step (the app's loop vs the mixed device step)": r4(rt["total"] * 1e3 / mine["mixed"]["ms_total"]),
        "end to end (the app's loop vs pgx_screen_chunks)": r4(rt["total"] / mine["e2e_s"])}
    # pair mode: one synthetic pulsar against every cluster (the prefilter's pairs), 100 clones
    pp = os.path.join(tmp, "pulsars.txt")
    with open(pp, "w") as f:
        f.write("\n".join(synth.pulsars(1, C3_SEED)) + "\n")
    wu = os.path.join(tmp, "wu_pair")
    with open(pp) as f, open(wu, "w") as g:
        g.write("PHYGAS 1 pair 100 0.05\n" + f.read())
    with Clocks(0) as clk:
        ref_rows, ref_t, ref_msg = _ref_gpu_run(cp, wu)
    out["pair_reference_gpu"] = dict(ref_t, summary=ref_msg, clocks=clk.summary())
    pulsars = pg.read_targets(pp)
    with pg.Context(0) as ctx:
        ti, ci = ctx.prefilter(pulsars, clusters)
        batch = pg.draw_pair_batch(pulsars, ti, clusters, ci, 100, 0.05)
        ctx.pair(*batch)
        res = ctx.pair(*batch)
        st = ctx.stats()
    got = ["%s %s %s %d %.3f %.3f %.3f %.4f %.4f %.4f %.2f %.2f %.2f %.4f %.4f" % (
        pulsars[0].id.decode(), clusters[c].name.decode(), clusters[c].kind.decode(), r["n"], r["d05"], r["d50"],
        r["d95"], r["t05"], r["t50"], r["t95"], r["v05"], r["v50"], r["v95"], r["f_r50"], r["f_rtot"])
        for c, r in zip(ci.tolist(), res)]
    out["pair_this_build_ms"] = {"ms_pair": r4(st["ms_pair"]), "clone_steps": int(st["clone_steps"])}
    out["pair_rows"] = {"reference_gpu": len(ref_rows), "this_build": len(got),
                        "identical_lines": sum(1 for x, y in zip(ref_rows, got) if x == y)}
    out["pair_stage_speedup"] = {"clones (pg_pair_k vs k_pair_mc_t graph)": r4(ref_t["pair_s"] * 1e3 / st["ms_pair"])}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--mode", default="bench", choices=["bench", "screen", "pairs", "refgpu"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline sample")
    ap.add_argument("--no-pair", action="store_true", help="skip the batched Monte Carlo measurement")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving measurement")
    ap.add_argument("--no-cli", action="store_true", help="skip the end-to-end run of the screen CLI")
    ap.add_argument("--no-control", action="store_true", help="skip the velocity-shuffled control's accuracy check")
    g = ap.add_argument_group("profiling modes")
    g.add_argument("--stars", type=int, default=None, help="screen: 20,000; pairs: 2,000")
    g.add_argument("--clusters", type=int, default=None, help="screen: the workload's 4,087")
    g.add_argument("--seed", type=int, default=None)
    g.add_argument("--precision", choices=("mixed", "fp64"), default="mixed")
    g.add_argument("--parts", type=int, default=None,
                   help="screen: equal parts of a chunk of at least 8,192 stars (1 = screened whole; default parts "
                        "ramping up from about 1e7 star-cluster pairs)")
    g.add_argument("--repeat", type=int, default=1)
    g.add_argument("--pairs", type=int, default=200)
    g.add_argument("--pulsars", type=int, default=1)
    g.add_argument("--streamed", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return reference_arm(args)
    if args.mode == "screen":
        args.stars = args.stars or N_STARS
        return mode_screen(args)
    if args.mode == "pairs":
        args.stars = args.stars or 2000
        return mode_pairs(args)
    if args.mode == "refgpu":
        return mode_refgpu(args)

    import numpy as np
    import torch
    import phygas_gb300 as pg
    import __graft_entry__
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    if rank == 0 or ws > 1:
        __graft_entry__.build()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    tmp = tempfile.mkdtemp(prefix="phygas_bench_")
    cp, tp = make_inputs(tmp, rank)
    clusters, stars = pg.read_clusters(cp), pg.read_targets(tp)
    tmax = max(c.tmax_myr for c in clusters)
    pp = pair_points(clusters, N_STARS, tmax)
    ctx = pg.Context(local)
    fp64_peak, fp32_peak = ctx.peaks()
    t0 = time.time()
    ctx.set_clusters(clusters, N_SAMP, R_KERNEL)
    table_s = time.time() - t0
    t0 = time.perf_counter()
    ps0, sig, pre = pg.draw_targets(stars, N_SAMP)
    draw_s = time.perf_counter() - t0
    ctx.draw_targets(stars[:256], N_SAMP)                                          # warm-up
    t0 = time.perf_counter()
    ctx.draw_targets(stars, N_SAMP)
    draw_gpu_s, draw_gpu_ms = time.perf_counter() - t0, ctx.stats()["ms_total"]
    ctx.stage(ps0, sig, pre)

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()

    def run(precision, k, w):
        for _ in range(w):
            ctx.exec(tmax, CHI2_MAX, precision)
        per, stats, rows = [], [], 0
        barrier()
        for _ in range(k):
            flush.zero_()
            torch.cuda.synchronize()
            rows = ctx.exec(tmax, CHI2_MAX, precision)
            s = ctx.stats()
            per.append(s["ms_total"])
            stats.append(s)
        barrier()
        return per, stats, rows

    scan_tune = None
    try:
        run(pg.PGX_MIXED, 0, 1)
        precision = pg.PGX_MIXED
        # the screen autotuner: the block filter's launch shapes on this chunk, the fastest kept for the steps
        best, table = ctx.tune_screen(tmax, CHI2_MAX)
        scan_tune = {"chosen_min_blocks_per_sm": table[best][0],
                     "scan_ms": [{"min_blocks_per_sm": b, "ms": r4(t)} for b, t in table]}
    except pg.GpuError as e:
        log("mixed-precision screen unavailable (%s); timing the FP64 screen as the value" % e)
        precision = pg.PGX_FP64
    with Clocks(local) as clk:
        per, stats, n_rows = run(precision, args.steps, args.warmup)
    parts = max(1, stats[-1]["parts"])
    rows_mixed = ctx.fetch(n_rows)
    # the plain FP64 comparator: the chunk whole, every stage in turn (no parts, no overlap); its orbit launch is
    # also the orbit roofline's (the whole chunk on the whole GPU)
    ctx.set_split(0)
    ctx.stage(ps0, sig, pre)
    per64, stats64, n_rows64 = run(pg.PGX_FP64, max(2, min(args.steps, 3)), 1)
    rows_fp64 = ctx.fetch(n_rows64)
    ctx.set_split(8192)
    ctx.stage(ps0, sig, pre)
    accuracy = {"screen": compare_rows(rows_mixed, rows_fp64)}
    del rows_fp64
    if rank == 0 and not args.no_control:
        # the chance-alignment control: the same stars with velocities shuffled, mixed against FP64
        ctl = pg.control_targets(stars)
        ctx.stage(*pg.draw_targets(ctl, N_SAMP))
        a = ctx.fetch(ctx.exec(tmax, CHI2_MAX, pg.PGX_MIXED))
        b = ctx.fetch(ctx.exec(tmax, CHI2_MAX, pg.PGX_FP64))
        accuracy["control"] = compare_rows(a, b)
        del a, b
        ctx.stage(ps0, sig, pre)
    ms = statistics.mean(per)
    ms64 = statistics.mean(per64)
    if ws > 1:
        t = torch.tensor([ms, ms64], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms, ms64 = t.tolist()
    pairs = N_STARS * N_CLUSTERS
    value = ws * pairs / (ms * 1e-3)

    # end to end through the C-ABI: host records -> host draws -> H2D -> device -> D2H of the rows into page-locked
    # host memory, E2E_CHUNKS chunks of these stars through pgx_screen_chunks, which draws chunk i + 1 on the host
    # while the GPU screens chunk i (steady state: the time per chunk)
    tk = pg.as_array(list(stars) * E2E_CHUNKS, pg.PhTarget)
    e2e_rows = []
    e2e_times = []
    for i in range(3):                  # the first run allocates the context's page-locked buffers
        e2e_rows.clear()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.screen_chunks(tk, N_STARS, tmax, lambda first, rows: e2e_rows.append(len(rows)), CHI2_MAX, precision)
        e2e_times.append((time.perf_counter() - t0) / E2E_CHUNKS)
    if sum(e2e_rows) != E2E_CHUNKS * n_rows:
        log("e2e chunks kept %d rows, the timed steps %d x %d" % (sum(e2e_rows), E2E_CHUNKS, n_rows))
    e2e_s = min(e2e_times)
    h2d = N_STARS * (6 + 21 + 1) * 8
    d2h = n_rows * pg.ROW_DTYPE.itemsize + 8
    # this chunk's rows on the host, for the Monte Carlo batch below (outside the timing)
    host_rows = pg.HostRows(int(n_rows * 1.25) + 4096)
    a, b, c = pg.draw_targets(stars, N_SAMP)
    r = ctx.screen_into(a, b, c, tmax, host_rows, CHI2_MAX, precision)

    pair_mc = None
    if not args.no_pair:
        try:
            pair_mc = pair_mc_measure(ctx, stars, clusters, cp, r, rank == 0 and not args.no_cpu, fp64_peak)
        except Exception as e:          # reported beside the headline, not part of it
            log("pair Monte Carlo measurement failed: %s" % e)

    cli = None
    if rank == 0 and not args.no_cli:
        try:
            cli = cli_measure(cp, tp)
        except Exception as e:          # reported beside the headline, not part of it
            log("cli measurement failed: %s" % e)

    serving = None
    if rank == 0 and not args.no_serve:
        try:
            serving = serving_measure(cp, tp)
        except Exception as e:          # reported beside the headline, not part of it
            log("serving measurement failed: %s" % e)

    s, s64 = stats[-1], stats64[-1]
    orbit_ms = statistics.mean(x["ms_orbit"] for x in stats64)
    achieved = FLOPS_PER_BODY_STEP * s64["orbit_body_steps"] / (orbit_ms * 1e-3)
    cpu, parity = None, None
    if rank == 0 and not args.no_cpu:
        try:
            cpu, ora_rows = cpu_baseline(cp, tp, keep_rows=True)
            parity = compare_to_oracle(rows_mixed, ora_rows, int(cpu["pairs"] // N_CLUSTERS))
            cpu.pop("loop_s", None)
            cpu.pop("pairs", None)
        except Exception as e:          # the baseline is reported, not required
            log("cpu baseline failed: %s" % e)
    del rows_mixed
    if rank == 0:
        scan = scan_roofline(stats, clk.summary(), pp, fp32_peak, parts)
        out = {
            "metric": "pairs/s", "value": value, "unit": "pairs/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64+f32" if precision == pg.PGX_MIXED else "f64", "data": "synthetic",
            "precision": "mixed" if precision == pg.PGX_MIXED else "fp64",
            "config": config(args),
            "gpu_launches": int(sum(x["kernels"] for x in stats)),
            "clocks": clk.summary(),
            "e2e": {"value": ws * pairs / e2e_s, "unit": "pairs/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "s_per_step": e2e_s,
                    "how": "pgx_screen_chunks over %d copies of the %d stars in chunks of %d (the first ones ramping "
                           "up from 2,447 stars): host draws of chunk i+2, the orbits of chunk i+1 (side stream) and "
                           "the screen of chunk i overlap; rows copied to page-locked host memory; s_per_step = the "
                           "time per %d stars" % (E2E_CHUNKS, N_STARS, N_STARS, N_STARS),
                    "host_draw_s_unpipelined": draw_s,
                    "device_draws": {"call_s": draw_gpu_s, "kernel_ms": draw_gpu_ms,
                                     "how": "pgx_draw_targets_gpu: the chunk's draws on the GPU"}},
            "roofline": scan,
            "roofline_orbits": {"bound": "fp64", "kernel": "k_stm_orbits", "achieved": achieved / 1e12,
                                "peak": fp64_peak / 1e12, "unit": "TFLOP/s", "frac": achieved / fp64_peak,
                                "peak_source": "FP64 FMA probe kernel of this run (pgx_peaks)",
                                "traffic": ORBIT_TRAFFIC_BYTES, "flops_per_body_step": FLOPS_PER_BODY_STEP,
                                "body_steps_per_launch": s64["orbit_body_steps"], "ms_per_launch": orbit_ms,
                                "launch": "the orbits of the whole chunk (the plain FP64 run's launch; the same kernel "
                                          "as the mixed path's)",
                                "fp64_instr_frac": FP64_INSTR_PER_BODY_STEP * s64["orbit_body_steps"]
                                                   / (orbit_ms * 1e-3) / (fp64_peak / 2)},
            "cpu_baseline": cpu,
            "fp32_peak_tflops": fp32_peak / 1e12,
            "cluster_table_s": table_s,
            "scan_autotune": scan_tune,
            "rows_per_step": n_rows, "rows_fp64": n_rows64,
            "work_per_step": {k: int(s[k]) for k in ("candidates", "ambiguous", "rechecked_points",
                                                     "rechecked_draws", "kept")},
            "pair_mc": pair_mc,
            "cli": cli,
            "serving": serving,
            # the evidence a reader checks first, last on the line
            "stages_ms": {k[3:]: r4(statistics.mean(x[k] for x in stats)) for k in
                          ("ms_orbit", "ms_cov", "ms_scan", "ms_select", "ms_finish")},
            "stages_ms_fp64": {k[3:]: r4(statistics.mean(x[k] for x in stats64)) for k in
                               ("ms_orbit", "ms_cov", "ms_scan", "ms_select", "ms_finish")},
            "roofline_scan": {k: r4(scan[k]) for k in ("achieved", "frac", "issue_frac", "ms_per_launch")
                              if scan and k in scan},
            "plain_fp64": {"value": r4(ws * pairs / (ms64 * 1e-3)), "ms_per_step": r4(ms64),
                           "speedup_of_value": r4(ms64 / ms)},
            "mixed_vs_fp64": accuracy,
            "parity_vs_oracle": parity,
        }
        print(json.dumps(out))
    ctx.close()
    if ws > 1:
        torch.distributed.destroy_process_group()



if __name__ == "__main__":
    main()
