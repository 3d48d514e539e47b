"""Build of the oracle (test infrastructure: the checker, never the product).

    python oracle/build_oracle.py

Compiles oracle/'s C restatement of the reference's CPU algorithm with the reference's own flags (gcc -O2 -std=c99,
no FP contraction) into oracle/_build/: libphygas_oracle.so, oracle_dump and oracle_wu.  When the reference's
sources are present -- PHYGAS_REF, default /root/reference, the read-only checkout of the development container --
it also compiles the reference itself from its own sources through `make -C oracle ref` into oracle/_ref/ (the pin
of the restatement), and the reference's GPU kernels into oracle/_ref/ref_kernels.ptx (`make -C oracle ref-gpu-ptx`).
The GPU machine has no reference checkout; there the restatement is built, and the reference-GPU comparator's host
program (oracle/_build/ref_gpu, `make -C oracle ref-gpu`) when the PTX came with the repository.
"""
import os
import shutil
import subprocess
import sys

ORACLE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(ORACLE)
INCLUDE = os.path.join(REPO, "include")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build step failed:\n  %s\n%s" % (" ".join(cmd), r.stdout))


def build_oracle(reference=None):
    b = os.path.join(ORACLE, "_build")
    os.makedirs(b, exist_ok=True)
    flags = ["-O2", "-std=c99", "-ffp-contract=off", "-fPIC", "-I", INCLUDE]
    src = os.path.join(ORACLE, "phygas_oracle.c")
    obj = os.path.join(b, "phygas_oracle.o")
    if _stale(obj, [src, os.path.join(INCLUDE, "phygas.h")]):
        _run(["gcc"] + flags + ["-c", src, "-o", obj])
    outs = [(os.path.join(b, "libphygas_oracle.so"), ["gcc", "-shared", "-o", None, obj, "-lm"], [obj])]
    for name, main in (("oracle_dump", "dump_main.c"), ("oracle_wu", "wu_main.c")):
        m = os.path.join(ORACLE, main)
        outs.append((os.path.join(b, name), ["gcc"] + flags + [m, obj, "-o", None, "-lm"], [obj, m]))
    for out, cmd, dep in outs:
        if _stale(out, dep):
            _run([out if c is None else c for c in cmd])
    ref = reference if reference is not None else os.environ.get("PHYGAS_REF", "/root/reference")
    if ref and os.path.isdir(os.path.join(ref, "src")) and shutil.which("make"):
        _run(["make", "-s", "-C", ORACLE, "ref", "REF=" + ref])
        _run(["make", "-s", "-C", ORACLE, "ref-gpu-ptx", "REF=" + ref])
    # the reference-GPU comparator's host program, wherever the reference's kernels (PTX) came with the repository
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    if os.path.exists(os.path.join(ORACLE, "_ref", "ref_kernels.ptx")) and os.path.exists(
            os.path.join(cuda, "include", "cuda.h")) and shutil.which("make"):
        _run(["make", "-s", "-C", ORACLE, "ref-gpu", "CUDA=" + cuda])


if __name__ == "__main__":
    build_oracle(sys.argv[1] if len(sys.argv) > 1 else None)
