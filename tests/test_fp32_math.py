"""The engine's FP32 device arithmetic (oxg_device.cuh) run on the host through a
test-only harness (tests/native/devmath.cu), against the reference's golden outputs:
catches FP32 conditioning problems before anything runs on a GPU."""

import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from _util import TERMS, TOL_GPU, golden, maxrel, model_forces

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "native", "devmath.cu")
LIB = os.path.join(HERE, "native", "_build", "libdevmath.so")


@pytest.fixture(scope="module")
def devmath():
    from oxdna import _build
    deps = [SRC] + _build.sources()
    if not os.path.exists(LIB) or any(os.path.getmtime(d) > os.path.getmtime(LIB) for d in deps):
        os.makedirs(os.path.dirname(LIB), exist_ok=True)
        tmp = LIB + ".tmp%d" % os.getpid()
        r = subprocess.run([_build.nvcc(), "-x", "cu", _build.ARCH, "-O2", "-std=c++17",
                            "-shared", "-Xcompiler", "-fPIC", "-o", tmp, SRC],
                           capture_output=True, text=True)
        if r.returncode != 0:
            pytest.fail("devmath build failed:\n" + r.stderr)
        os.replace(tmp, LIB)
    L = C.CDLL(LIB)
    dp = C.POINTER(C.c_double)
    L.devmath_pair.argtypes = [C.c_int, C.c_void_p, C.c_double, dp, dp, dp, C.c_double,
                               C.c_double, dp, dp, dp, dp]
    L.devmath_pair.restype = C.c_int
    L.devmath_bonded.argtypes = [C.c_void_p, dp, dp, dp, C.c_int, C.c_int, dp, dp, dp, dp, dp]
    return L


def _p(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(C.POINTER(C.c_double))


@pytest.mark.parametrize("model", ("dna1", "dna2", "rna2"))
@pytest.mark.parametrize("term", range(6))
def test_fp32_pair_math(devmath, model, term):
    from oxdna import _abi, io
    d = golden(f"pairs_{model}.npz")
    name = TERMS[term]
    f = model_forces(model)[0][term]
    n = len(d[name + "/dr"])
    F, E, TI, TJ = np.zeros((n, 3)), np.zeros(n), np.zeros((n, 3)), np.zeros((n, 3))
    for k in range(n):
        a, b = d[name + "/types"][k]
        key = (io.DNA_BASES[a], io.DNA_BASES[b])
        pod = _abi.FROM_DICT[term](f.params[key])
        fo, e, ti, tj = np.zeros(3), np.zeros(1), np.zeros(3), np.zeros(3)
        ci, cj = d[name + "/charges"][k]
        devmath.devmath_pair(term, C.byref(pod), f.rcut_for(*key), _p(d[name + "/dr"][k]),
                             _p(d[name + "/qi"][k]), _p(d[name + "/qj"][k]), ci, cj,
                             fo.ctypes.data_as(C.POINTER(C.c_double)),
                             e.ctypes.data_as(C.POINTER(C.c_double)),
                             ti.ctypes.data_as(C.POINTER(C.c_double)),
                             tj.ctypes.data_as(C.POINTER(C.c_double)))
        F[k], E[k], TI[k], TJ[k] = fo, e[0], ti, tj
    errs = {k: maxrel(v, d[f"{name}/ref64/{k}"]) for k, v in
            (("force", F), ("energy", E), ("torque_i", TI), ("torque_j", TJ))}
    assert max(errs.values()) < TOL_GPU, f"{model} {name}: {errs}"


@pytest.mark.parametrize("model", ("dna1", "dna2", "rna2"))
@pytest.mark.parametrize("avg", ("avg", "seq"))
def test_fp32_bonded_math(devmath, model, avg):
    from oxdna import _abi
    d = golden(f"bonds_{model}.npz")
    _, bonded = model_forces(model, average=(avg == "avg"))
    pod = _abi.bonded_from_dict(bonded.params["backbone"])
    n = len(d[f"{avg}/Rc"])
    out = {k: [] for k in ("FB", "tauA", "tauB", "energy")}
    for k in range(n):
        FB, tA, tB, e, v = (np.zeros(3), np.zeros(3), np.zeros(3), np.zeros(3), np.zeros(6))
        devmath.devmath_bonded(C.byref(pod), _p(d[f"{avg}/Rc"][k]), _p(d[f"{avg}/qA"][k]),
                               _p(d[f"{avg}/qB"][k]), int(d[f"{avg}/types"][k][0]),
                               int(d[f"{avg}/types"][k][1]), *(x.ctypes.data_as(C.POINTER(C.c_double))
                                                               for x in (FB, tA, tB, e, v)))
        for key, val in zip(out, (FB, tA, tB, e)):
            out[key].append(val)
    ok = d[f"{avg}/ref64/energy"][:, 0] < 1e12
    for key in out:
        got = np.array(out[key])[ok]
        ref = d[f"{avg}/ref64/{key}"][ok]
        assert maxrel(got, ref) < TOL_GPU, f"{model} {avg} {key}: {maxrel(got, ref):.2e}"
    e = np.array(out["energy"])
    assert np.array_equal(e[:, 0] >= 1e12, ~ok)
