"""The engine's FP32 device arithmetic (oxg_device.cuh) run on the host through a
test-only harness (tests/native/devmath.cu), against the reference's golden outputs:
catches FP32 conditioning problems before anything runs on a GPU."""

import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from _util import PAIR_CASES, TERMS, TOL_GPU, golden, maxrel, model_forces, pair_golden

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
    L.devmath_bonded.argtypes = [C.c_void_p, dp, dp, dp, C.c_int, C.c_int, dp, dp, dp, dp, dp, C.c_int]
    L.devmath_mlp_map.argtypes = [dp] * 9
    L.devmath_mlp_map.restype = C.c_int
    return L


def _p(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(C.POINTER(C.c_double))


@pytest.mark.parametrize("model,term,avg", PAIR_CASES)
def test_fp32_pair_math(devmath, model, term, avg):
    from oxdna import _abi, io
    d = pair_golden(model, avg)
    name = TERMS[term]
    f = model_forces(model, average=(avg == "avg"))[0][term]
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
@pytest.mark.parametrize("full64", (1, 0))
def test_fp32_bonded_math(devmath, model, avg, full64):
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
                                                               for x in (FB, tA, tB, e, v)), full64)
        for key, val in zip(out, (FB, tA, tB, e)):
            out[key].append(val)
    ok = d[f"{avg}/ref64/energy"][:, 0] < 1e12
    for key in out:
        got = np.array(out[key])[ok]
        ref = d[f"{avg}/ref64/{key}"][ok]
        assert maxrel(got, ref) < TOL_GPU, f"{model} {avg} {key}: {maxrel(got, ref):.2e}"
    e = np.array(out["energy"])
    assert np.array_equal(e[:, 0] >= 1e12, ~ok)


@pytest.mark.parametrize("model", ("dna1", "rna2"))
def test_bond_parts_sum_to_whole_bond(devmath, model):
    """The run kernel may evaluate a bond on two lanes (FENE + bonded excluded volume,
    and stacking): the two parts add up to the whole bond."""
    from oxdna import _abi
    d = golden(f"bonds_{model}.npz")
    _, bonded = model_forces(model, average=False)
    pod = _abi.bonded_from_dict(bonded.params["backbone"])
    n = len(d["seq/Rc"])
    for k in range(n):
        res = []
        for mode in (0, 2, 4):
            FB, tA, tB, e, v = (np.zeros(3), np.zeros(3), np.zeros(3), np.zeros(3), np.zeros(6))
            devmath.devmath_bonded(C.byref(pod), _p(d["seq/Rc"][k]), _p(d["seq/qA"][k]),
                                   _p(d["seq/qB"][k]), int(d["seq/types"][k][0]),
                                   int(d["seq/types"][k][1]),
                                   *(x.ctypes.data_as(C.POINTER(C.c_double)) for x in (FB, tA, tB, e, v)),
                                   mode)
            res.append((FB, tA, tB, e))
        whole, p1, p2 = res
        if whole[3][0] >= 1e12:
            continue
        assert p1[3][2] == 0.0 and p2[3][0] == 0.0 and p2[3][1] == 0.0
        for w, a, b in zip(whole, p1, p2):
            scale = max(np.abs(w).max(), 1.0)
            assert np.abs(a + b - w).max() <= 1e-5 * scale, (k, w, a, b)


def _qmul(a, b):
    w1, x1, y1, z1 = a
    w2, x2, y2, z2 = b
    return np.array([w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2, w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
                     w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2, w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2])


def test_surrogate_force_map_matches_finite_differences(devmath):
    """mlp_grad_to_forces (the surrogate's map from dE/d(features) to forces and lab
    torques, base-site offsets included) against central differences of a smooth test
    energy of the base-base features over positions and small lab-frame rotations."""
    rng = np.random.Generator(np.random.PCG64(3))
    base = np.array([0.4, 0.0, 0.0])
    coef = rng.normal(0.0, 1.0, 14)
    out = [np.zeros(3) for _ in range(4)]

    def run(dr, qi, qj):
        e = np.zeros(1)
        ok = devmath.devmath_mlp_map(_p(base), _p(dr), _p(qi), _p(qj), _p(coef), _p(e), _p(out[1]),
                                     _p(out[2]), _p(out[3]))
        assert ok
        return e[0], out[1].copy(), out[2].copy(), out[3].copy()

    for trial in range(20):
        qi = rng.normal(size=4)
        qi /= np.linalg.norm(qi)
        qj = rng.normal(size=4)
        qj /= np.linalg.norm(qj)
        dr = rng.normal(size=3)
        dr *= rng.uniform(0.6, 1.2) / np.linalg.norm(dr)
        _, F, Ti, Tj = run(dr, qi, qj)

        def central(fn, h):
            # Richardson-extrapolated central difference, O(h^4)
            d1 = (fn(h) - fn(-h)) / (2 * h)
            d2 = (fn(h / 2) - fn(-h / 2)) / h
            return (4 * d2 - d1) / 3

        def rot(k, a):
            return np.concatenate([[np.cos(a / 2)], np.sin(a / 2) * np.eye(3)[k]])

        h = 1e-2
        fd_f = np.zeros(3)
        fd_ti = np.zeros(3)
        fd_tj = np.zeros(3)
        for k in range(3):
            fd_f[k] = -central(lambda a: run(dr + a * np.eye(3)[k], qi, qj)[0], h)
            fd_ti[k] = -central(lambda a: run(dr, _qmul(rot(k, a), qi), qj)[0], h)
            fd_tj[k] = -central(lambda a: run(dr, qi, _qmul(rot(k, a), qj))[0], h)
        scale = max(np.abs(np.concatenate([fd_f, fd_ti, fd_tj])).max(), 1e-3)
        assert np.abs(F - fd_f).max() < 2e-3 * scale, (trial, F, fd_f)
        assert np.abs(Ti - fd_ti).max() < 2e-3 * scale, (trial, Ti, fd_ti)
        assert np.abs(Tj - fd_tj).max() < 2e-3 * scale, (trial, Tj, fd_tj)
