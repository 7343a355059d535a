"""The flop census behind the MD step's compute roofline: the committed table
(tests/golden/flop_counts.json) against a fresh census by the reference's own headers
compiled with an operation-counting ForceReal (needs the reference source tree; skipped
elsewhere), and the counting build's arithmetic against the FP64 reference."""

import json
import os
import sys

import numpy as np
import pytest

from _util import TERMS, golden, model_forces

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = os.path.join(HERE, "golden", "flop_counts.json")


def _census_module():
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_flop_counts
    return make_flop_counts


def test_table_is_complete_and_consistent():
    with open(TABLE) as fh:
        t = json.load(fh)
    for name, w in t["workloads"].items():
        assert set(w["terms"]) == {"oxdna_excvol", "oxdna_hbond", "oxdna_crossstacking",
                                   "oxdna_coaxstacking", "oxdna_debye"}, name
        parts = list(w["terms"].values()) + [w["bonded"]]
        assert w["flops_per_step"] == sum(p["add"] + p["mul"] for p in parts)
        for p in parts:
            assert p["flops"] == p["add"] + p["mul"] > 0
        assert w["bonded"]["bonds"] == w["n_bonds"]
    # both workloads are the same duplex at the same density: per-pair costs agree
    a, b = t["workloads"]["8000nt"], t["workloads"]["100k_nt"]
    for k in a["terms"]:
        assert abs(a["terms"][k]["flops_per_pair"] - b["terms"][k]["flops_per_pair"]) < 0.02 * \
            a["terms"][k]["flops_per_pair"]


def test_counting_build_reproduces_fp64_reference(oracle):
    from oxdna import _abi, io
    if not oracle.ref_lib(64):
        pytest.skip("reference source tree not available")
    M = _census_module()
    L, r64 = M.count_lib(), oracle.ref_lib(64)
    d = golden("pairs_dna2.npz")
    pf = model_forces("dna2")[0]
    for t in range(6):
        name, f = TERMS[t], pf[t]
        L.ref_count_reset()
        for k in range(0, len(d[name + "/dr"]), 7):
            a, b = d[name + "/types"][k]
            p = _abi.FROM_DICT[t](f.params[(io.DNA_BASES[a], io.DNA_BASES[b])])
            args = (p, d[name + "/dr"][k], d[name + "/qi"][k], d[name + "/qj"][k],
                    d[name + "/rcutsq"][k], *d[name + "/charges"][k])
            x = oracle.eval_pair(L, "ref", t, *args)
            y = oracle.eval_pair(r64, "ref", t, *args)
            assert x[0] == y[0] and x[2] == y[2]
            for u, v in zip(x[1:], y[1:]):
                assert np.array_equal(u, v)
        c = M.read_counts(L)
        assert c["add"] > 0 and c["mul"] > 0, name


def test_census_of_8000nt_workload_matches_table(oracle):
    if not oracle.ref_lib(64):
        pytest.skip("reference source tree not available")
    M = _census_module()
    with open(TABLE) as fh:
        want = json.load(fh)["workloads"]["8000nt"]
    name, *args = M.WORKLOADS[0]
    got = M.census(M.count_lib(), name, *args)
    assert got["flops_per_step"] == want["flops_per_step"]
    assert got["special_per_step"] == want["special_per_step"]
    for k in want["terms"]:
        assert got["terms"][k]["pairs"] == want["terms"][k]["pairs"]


@pytest.mark.gpu
def test_device_peaks_are_plausible(native):
    """The roofline denominators: FP32 FMA and special-function throughput of a GB300
    (152 SMs; 128 FP32 lanes and 16 special-function lanes per SM at ~1.9-2.1 GHz:
    nominally ~80 TFLOP/s and ~5 Top/s)."""
    from oxdna import runtime
    fp32, sfu = runtime.device_peaks()
    assert 20e3 < fp32 < 200e3, fp32
    assert 500 < sfu < 50e3, sfu
