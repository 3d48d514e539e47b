"""In-tree build of libphygas_gb300 and its two CLIs (nvcc + gcc, sm_103a only, no cmake).

Outputs go to phygas_gb300/_lib/: libphygas_gb300.so (CUDA kernels + C host code, static cudart), phygas_screen,
phygas_cli, phygas_serve.  (The oracle, the tests' checker, has its own build: oracle/build_oracle.py.)  Objects are rebuilt only when a source or header is newer; compiles run in parallel.

    python -m phygas_gb300.build            (or __graft_entry__.build())
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
LIB = os.path.join(HERE, "_lib")
OBJ = os.path.join(LIB, "obj")
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(REPO, "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# FP contraction off where a result must follow the reference's operation order (the draws too), and for the orbits, whose fused
# multiply-adds are all written out: then every launch shape of a kernel rounds alike
FMAD_OFF = {"pgx_scan.cu", "pgx_mixed.cu", "pgx_orbit.cu", "pgx_draws.cu"}


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _headers():
    return (glob.glob(os.path.join(CSRC, "**", "*.h"), recursive=True)
            + glob.glob(os.path.join(CSRC, "**", "*.cuh"), recursive=True)
            + glob.glob(os.path.join(INCLUDE, "*.h")))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n  %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def build(verbose=False, jobs=None):
    os.makedirs(OBJ, exist_ok=True)
    hdrs = _headers()
    cu = sorted(glob.glob(os.path.join(CSRC, "cuda", "*.cu")))
    host = [os.path.join(CSRC, "host", "ph_host.c")]
    steps = []
    for src in cu:
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        cmd = [nvcc()] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE,
                                 "-I", os.path.join(CSRC, "cuda"), "-c", src, "-o", obj]
        if os.path.basename(src) in FMAD_OFF:
            cmd.insert(-4, "--fmad=false")
        if os.environ.get("PHYGAS_PTXAS_V"):
            cmd.insert(-4, "-Xptxas=-v")
        steps.append((obj, [src] + hdrs, cmd))
    for src in host:
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        cmd = ["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-ffp-contract=off", "-fPIC", "-Wall", "-I", INCLUDE,
               "-c", src, "-o", obj]
        steps.append((obj, [src] + hdrs, cmd))
    todo = [s for s in steps if _stale(s[0], s[1])]
    with cf.ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
        for out in ex.map(lambda s: _run(s[2]), todo):
            if verbose and out.strip():
                print(out)
    objs = [s[0] for s in steps]
    so = os.path.join(LIB, "libphygas_gb300.so")
    if _stale(so, objs):
        _run([nvcc()] + ARCH + ["-shared", "-o", so] + objs + ["-lpthread"])
    for name, src in (("phygas_screen", "phygas_screen_main.c"), ("phygas_cli", "phygas_cli_main.c"),
                      ("phygas_serve", "phygas_serve_main.c")):
        exe = os.path.join(LIB, name)
        s = os.path.join(CSRC, "host", src)
        if _stale(exe, [s, so] + hdrs):
            _run(["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-ffp-contract=off", "-Wall", "-I", INCLUDE,
                  "-I", os.path.join(CSRC, "host"), s, "-o", exe, "-L", LIB, "-lphygas_gb300",
                  "-Wl,-rpath,$ORIGIN", "-lm", "-lpthread"])
    return so


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
