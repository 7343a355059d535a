"""The FP64 C oracle against the reference's own evaluators (golden fixtures made by
tests/golden/make_golden.py from the reference headers compiled unchanged)."""

import numpy as np
import pytest

from _util import PAIR_CASES, TERMS, TOL_ORACLE, golden, maxrel, model_forces, pair_golden

MODELS = ("dna1", "dna2", "rna2")


@pytest.mark.parametrize("model,term,avg", PAIR_CASES)
def test_pair_evaluators_match_reference(oracle, model, term, avg):
    from oxdna import _abi, io
    d = pair_golden(model, avg)
    name = TERMS[term]
    f = model_forces(model, average=(avg == "avg"))[0][term]
    L = oracle.oracle_lib()
    n = len(d[name + "/dr"])
    got = {k: [] for k in ("flag", "force", "energy", "torque_i", "torque_j")}
    for k in range(n):
        ti, tj = d[name + "/types"][k]
        p = _abi.FROM_DICT[term](f.params[(io.DNA_BASES[ti], io.DNA_BASES[tj])])
        ci, cj = d[name + "/charges"][k]
        ok, fi, e, tqi, tqj = oracle.eval_pair(L, "oxo", term, p, d[name + "/dr"][k],
                                               d[name + "/qi"][k], d[name + "/qj"][k],
                                               d[name + "/rcutsq"][k], ci, cj)
        for key, v in zip(got, (ok, fi, e, tqi, tqj)):
            got[key].append(v)
    assert np.array_equal(np.array(got["flag"], np.int8), d[name + "/ref64/flag"])
    for key in ("force", "energy", "torque_i", "torque_j"):
        err = maxrel(np.array(got[key]), d[f"{name}/ref64/{key}"])
        assert err < TOL_ORACLE, f"{model} {name} {key}: {err:.2e}"


@pytest.mark.parametrize("model", MODELS)
@pytest.mark.parametrize("avg", ("avg", "seq"))
def test_bonded_matches_reference(oracle, model, avg):
    from oxdna import _abi
    d = golden(f"bonds_{model}.npz")
    _, bonded = model_forces(model, average=(avg == "avg"))
    p = _abi.bonded_from_dict(bonded.params["backbone"])
    L = oracle.oracle_lib()
    res = [oracle.eval_bonded(L, "oxo", p, d[f"{avg}/Rc"][k], d[f"{avg}/qA"][k], d[f"{avg}/qB"][k],
                              *d[f"{avg}/types"][k]) for k in range(len(d[f"{avg}/Rc"]))]
    for k, fld in enumerate(("FB", "tauA", "tauB", "energy", "virial")):
        got = np.array([r[k] for r in res])
        ref = d[f"{avg}/ref64/{fld}"]
        if fld == "energy":
            # the broken-bond clamp (1e12) must match exactly; compare the rest relatively
            assert np.array_equal(got[:, 0] >= 1e12, ref[:, 0] >= 1e12)
            ok = ref[:, 0] < 1e12
            got, ref = got[ok], ref[ok]
        assert maxrel(got, ref) < TOL_ORACLE, f"{model} {avg} {fld}"


def test_system_driver_matches_reference(oracle):
    """HOOMD driver semantics (half list, third law, torque_j, 0.5 E split, bonds)."""
    from oxdna import io
    g = golden("system_dna2.npz")
    pair, bonded = model_forces("dna2")
    model = oracle.Model(pair + [bonded], io.DNA_BASES)
    sysm = oracle.System(g["pos"], g["quat"], g["typeid"], g["box"], g["bonds"], g["charge"])
    for use_cells in (0, 1):
        for t, name in enumerate(TERMS):
            r = oracle.forces(model, sysm, mask=1 << t, bonded=False, use_cells=use_cells)
            assert abs(r["pair_energy"][t] - g[name + "/energy"]) <= TOL_ORACLE * max(
                1.0, abs(g[name + "/energy"]))
            assert maxrel(r["force"], g[name + "/force"]) < TOL_ORACLE
            assert maxrel(r["torque"], g[name + "/torque"]) < TOL_ORACLE
            assert maxrel(r["energy_pp"], g[name + "/energy_pp"]) < TOL_ORACLE
        r = oracle.forces(model, sysm, mask=0, bonded=True, use_cells=use_cells)
        assert maxrel(r["bonded_energy"], g["bonded/energy"]) < TOL_ORACLE
        assert maxrel(r["force"], g["bonded/force"]) < TOL_ORACLE
        assert maxrel(r["torque"], g["bonded/torque"]) < TOL_ORACLE


def test_reference_system_driver_matches_oracle(oracle):
    """The reference's own evaluators and bonded kernel driven over a whole system with
    HOOMD's CPU semantics (the timed reference-arithmetic CPU baseline) give the
    oracle's forces, torques and energies (every term, fused and not)."""
    if oracle.ref_lib(64) is None:
        pytest.skip("reference source tree not present")
    from oxdna import io
    g = golden("system_dna2.npz")
    for fused in (False, True):
        pair, bonded = model_forces("dna2") if not fused else _fused_dna2()
        model = oracle.Model(pair + [bonded], io.DNA_BASES)
        sysm = oracle.System(g["pos"], g["quat"], g["typeid"], g["box"], g["bonds"], g["charge"])
        rl = max(f.rcut_for(a, b) for f in pair for a in io.DNA_BASES for b in io.DNA_BASES)
        pairs = oracle.half_pairs(sysm, rl * (1 + 1e-9))
        want = oracle.forces(model, sysm)
        got = oracle.ref_system_forces(model, sysm, pairs)
        for k in ("force", "torque", "energy_pp"):
            assert maxrel(got[k], want[k]) < TOL_ORACLE, (fused, k)
        assert np.allclose(got["pair_energy"], want["pair_energy"], rtol=1e-10, atol=1e-10)
        assert np.allclose(got["bonded_energy"], want["bonded_energy"], rtol=1e-10, atol=1e-10)


def _fused_dna2():
    from oxdna.model import dna2
    forces, _ = dna2.forces(fused=True)
    return forces[1:], forces[0]


def test_parameter_structs_match_the_reference_constructors():
    """This build's route from a parameter dict to the evaluators' param_type (dict ->
    POD struct -> field copy in oracle/ref_wrap.cpp) against the reference's own
    pybind11 dict constructors, both serialised by the reference's own toPython() /
    asDict(), for every type pair and bond type of the three models. Needs the
    reference-pin libraries (oracle/_ref, built where the reference tree is present).
    Skipped fields: for DNA bonds the reference constructor leaves the oxRNA-only
    stacking angles (stack_f4_tB1, stack_f4_tB2) uninitialised; they are never read."""
    import ctypes as C
    import os

    from oxdna import _abi
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                        "oracle", "_ref", "libref64.so")
    if not os.path.exists(path):
        pytest.skip("reference-pin libraries not built here")
    fn = C.PyDLL(path).ref_param_dicts
    fn.restype = C.py_object
    fn.argtypes = [C.c_int, C.py_object, C.c_void_p]
    n = 0
    for model in MODELS:
        for avg in (True, False):
            pair, bonded = model_forces(model, average=avg)
            for t, f in enumerate(pair):
                for key, d in f.params.items():
                    p = _abi.FROM_DICT[t](d)
                    ref, ours = fn(t, dict(d), C.addressof(p))
                    assert ref == ours, (model, t, key)
                    n += 1
            for key, d in bonded.params.items():
                p = _abi.bonded_from_dict(d)
                ref, ours = fn(6, dict(d), C.addressof(p))
                skip = set() if d.get("stack_rna") else {"stack_f4_tB1", "stack_f4_tB2"}
                assert set(ref) == set(ours)
                for k in set(ref) - skip:
                    assert ref[k] == ours[k], (model, key, k)
                n += 1
    assert n > 300
