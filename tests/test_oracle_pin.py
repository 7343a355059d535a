"""The FP64 C oracle against the reference's own evaluators (golden fixtures made by
tests/golden/make_golden.py from the reference headers compiled unchanged)."""

import numpy as np
import pytest

from _util import TERMS, TOL_ORACLE, golden, maxrel, model_forces

MODELS = ("dna1", "dna2", "rna2")


@pytest.mark.parametrize("model", MODELS)
@pytest.mark.parametrize("term", range(6))
def test_pair_evaluators_match_reference(oracle, model, term):
    from oxdna import _abi, io
    d = golden(f"pairs_{model}.npz")
    name = TERMS[term]
    f = model_forces(model)[0][term]
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
