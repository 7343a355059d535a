"""Build recipe for the test oracle (test infrastructure only).

* ``build_oracle()`` compiles the plain-C FP64 restatement ``oxdna_oracle.c`` into
  ``oracle/liboxdna_oracle.so`` (gcc, OpenMP for the multi-core CPU baseline).
* ``build_ref()`` compiles the reference plugin's own evaluator/bonded headers,
  unchanged, from the reference source tree (``OXDNA_REFERENCE_SRC`` or
  ``/root/reference/src``) together with the clean-room HOOMD stand-ins in
  ``oracle/ref_shim`` into ``oracle/_ref/libref64.so`` (ForceReal = double) and
  ``oracle/_ref/libref32.so`` (ForceReal = float, the reference's mixed-precision
  GPU arithmetic emulated on the host) and ``oracle/_ref/librefcount.so`` (ForceReal
  counts its operations: the flop census). Nothing is written outside ``oracle/_ref``;
  the reference sources are only read. Skipped when the reference tree is absent.
"""

import os
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SRC = os.environ.get("OXDNA_REFERENCE_SRC", "/root/reference/src")
ORACLE_SO = os.path.join(HERE, "liboxdna_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force=False):
    src = os.path.join(HERE, "oxdna_oracle.c")
    hdrs = [os.path.join(HERE, "oxdna_oracle.h"),
            os.path.join(HERE, "..", "include", "oxdna_gb300.h")]
    if force or _stale(ORACLE_SO, [src] + hdrs):
        tmp = ORACLE_SO + ".tmp%d" % os.getpid()
        _run(["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-Wall",
              "-o", tmp, src, "-lm"])
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def ref_available():
    return os.path.isfile(os.path.join(REF_SRC, "OxDNABondedKernel.h"))


def build_ref(force=False):
    """Returns the list of built libraries ([] when the reference tree is absent)."""
    if not ref_available():
        return []
    os.makedirs(REF_DIR, exist_ok=True)
    try:
        import pybind11
        pyb = pybind11.get_include()
    except ImportError:
        return []
    pyinc = sysconfig.get_paths()["include"]
    src = os.path.join(HERE, "ref_wrap.cpp")
    shim = os.path.join(HERE, "ref_shim")
    deps = [src, os.path.join(shim, "hoomd", "HOOMDMath.h"),
            os.path.join(shim, "hoomd", "VectorMath.h"), os.path.join(shim, "oxref_count.h"),
            os.path.join(HERE, "oxdna_oracle.h")]
    out = []
    for tag, defs in (("64", []), ("32", ["-DHOOMD_HAS_FORCEREAL"]),
                      ("count", ["-DHOOMD_HAS_FORCEREAL", "-DOXREF_COUNTING"])):
        so = os.path.join(REF_DIR, "libref%s.so" % tag)
        if force or _stale(so, deps):
            tmp = so + ".tmp%d" % os.getpid()
            _run(["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-w", *defs,
                  "-I", shim, "-I", REF_SRC, "-I", pyb, "-I", pyinc, "-o", tmp, src])
            os.replace(tmp, so)
        out.append(so)
    return out


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
