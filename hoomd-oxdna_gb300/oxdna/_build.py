"""Build recipe of the native library ``liboxdna_gb300.so`` (sm_103a only).

The CUDA sources under ``csrc/`` (kernels are headers included by the engine and
batch units) are compiled unit by unit in parallel and linked by nvcc into a shared
library next to this package, so the library that gets loaded is the in-tree one.
"""

import os
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
LIB = os.path.join(PKG, "liboxdna_gb300.so")
INCLUDE = os.path.join(os.path.dirname(ROOT), "include")

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
# FP32 division and square root to within 2 ulp (the hardware reciprocal / square-root
# approximations) and denormals flushed: the per-pair dependency chains are what bound
# the MD step, and the IEEE-rounded forms add a Newton step and a slow-path branch to
# every division. FP64 arithmetic (FENE, energy sums) is unaffected.
NVCC_FLAGS = [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-shared", "--expt-relaxed-constexpr", "-ftz=true", "-prec-div=false",
              "-prec-sqrt=false"]


def sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))
            if f.endswith((".cu", ".cuh", ".h"))] + [os.path.join(INCLUDE, "oxdna_gb300.h")]


def nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(s) > t for s in sources())


def build(force=False, verbose=False):
    """Compile the library if any source is newer than it. Returns the path.

    Each .cu unit is compiled to an object by its own nvcc process (in parallel), then
    the objects are linked into the shared library."""
    if not force and not stale():
        return LIB
    units = [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith(".cu")]
    tag = ".tmp%d" % os.getpid()
    objdir = os.path.join(PKG, "_obj")
    os.makedirs(objdir, exist_ok=True)
    objs = [os.path.join(objdir, os.path.basename(u)[:-3] + tag + ".o") for u in units]
    compile_flags = [f for f in NVCC_FLAGS if f != "-shared"]
    procs = [(subprocess.Popen([nvcc(), *compile_flags, "-c", "-o", o, u], stdout=subprocess.PIPE,
                               stderr=subprocess.STDOUT, text=True), u) for u, o in zip(units, objs)]
    logs, failed = [], []
    for p, u in procs:
        out, _ = p.communicate()
        logs.append(out)
        if p.returncode != 0:
            failed.append((u, out))
    try:
        if failed:
            raise RuntimeError("nvcc failed:\n" + "\n".join(f"{u}:\n{out}" for u, out in failed))
        tmp = LIB + tag
        cmd = [nvcc(), ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", tmp, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc link failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose:
            print("".join(logs) + r.stdout + r.stderr)
        os.replace(tmp, LIB)
    finally:
        for o in objs:
            if os.path.exists(o):
                os.remove(o)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
