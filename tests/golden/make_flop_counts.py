"""Flop census of the reference's own evaluator and bonded arithmetic on the
benchmark workloads, written to tests/golden/flop_counts.json.

    python tests/golden/make_flop_counts.py

The reference headers are compiled unchanged with an operation-counting ForceReal
(oracle/ref_shim/oxref_count.h, built by oracle/build.py into oracle/_ref/), so the
counts are those of the reference's FP32 arithmetic: additions/subtractions and
multiplications (one flop each, so an FMA is two), divisions and the calls sqrt, exp,
log, acos, sin, cos, counted separately. Needs the reference source tree (only on the
development machine); the JSON it writes is committed and read by bench.py for the
FP32 roofline of the MD step.

Census rules (the HOOMD driver semantics of the reference):

* every unordered non-bonded pair (i < j, dr = r_i - r_j minimum image, bonded pairs
  excluded as in the reference's neighbour list) within the term's r_cut for its type
  pair is one evaluate() call; pairs beyond r_cut cost nothing;
* every bond is one oxdna_bonded_pair() call (its FP64 FENE part is not counted);
* the snapshot is the initial state of the workload (the count drifts little as the
  duplexes fluctuate).
"""

import ctypes as C
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "hoomd-oxdna_gb300"))

from oracle import build as B  # noqa: E402
from oracle import oracle as O  # noqa: E402
from oxdna import _abi, io  # noqa: E402
from oxdna.model import dna2  # noqa: E402

OPS = ("add", "mul", "div", "sqrt", "exp", "log", "acos", "sin", "cos")
OUT = os.path.join(HERE, "flop_counts.json")

# the benchmark workloads: (name, duplexes, bp per duplex, box, seed)
WORKLOADS = (("8000nt", 200, 20, 100.0, 2), ("100k_nt", 2500, 20, 230.0, 5))


def count_lib():
    libs = B.build_ref()
    path = os.path.join(B.REF_DIR, "librefcount.so")
    if path not in libs:
        raise SystemExit("the reference source tree is needed for the census")
    L = C.CDLL(path)
    O._declare_pairs(L, "ref")
    L.ref_count_get.argtypes = [C.POINTER(C.c_ulonglong)]
    L.ref_count_reset.argtypes = []
    assert L.ref_count_n() == len(OPS)
    return L


def read_counts(L):
    buf = (C.c_ulonglong * len(OPS))()
    L.ref_count_get(buf)
    return {k: int(v) for k, v in zip(OPS, buf)}


def candidate_pairs(pos, L, r):
    from scipy.spatial import cKDTree
    t = cKDTree(np.mod(pos, L), boxsize=L)
    return t.query_pairs(r, output_type="ndarray")


def census(L, name, n_dup, n_bp, box, seed):
    s = io.duplex_system(n_dup, n_bp, box, seed=seed)
    forces, _ = dna2.forces(fused=False)
    bonded = forces[0]
    pair_forces = forces[1:]
    pos, q, ty, ch = s["pos"], s["quat"], s["typeid"], s["charge"]
    bonds = s["bonds"]
    excl = {(int(min(a, b)), int(max(a, b))) for a, b in bonds}
    rmax = max(f.default_r_cut for f in pair_forces)
    cand = candidate_pairs(pos, box, rmax)
    cand = np.array([p for p in map(tuple, np.sort(cand, axis=1)) if p not in excl])
    d = pos[cand[:, 0]] - pos[cand[:, 1]]
    d -= box * np.round(d / box)
    r2 = np.einsum("ij,ij->i", d, d)
    out = {"workload": f"{n_dup} x {n_bp}-bp B-DNA duplexes ({len(pos)} nt), box {box}, "
                       f"oxDNA2 0.5 M, unfused terms, seed {seed}",
           "n_nt": int(len(pos)), "n_bonds": int(len(bonds)), "terms": {}}
    for f in pair_forces:
        t = f._term
        keys = {}
        L.ref_count_reset()
        n_in = n_nonzero = 0
        for k in np.nonzero(r2 < f.default_r_cut ** 2)[0]:
            i, j = int(cand[k, 0]), int(cand[k, 1])
            key = (io.DNA_BASES[ty[i]], io.DNA_BASES[ty[j]])
            if key not in keys:
                keys[key] = (_abi.FROM_DICT[t](f.params[key]), f.rcut_for(*key) ** 2)
            p, rc2 = keys[key]
            if r2[k] >= rc2:
                continue
            n_in += 1
            res = O.eval_pair(L, "ref", t, p, d[k], q[i], q[j], rc2, ch[i], ch[j])
            n_nonzero += res[2] != 0.0
        c = read_counts(L)
        c["pairs"] = n_in
        c["pairs_nonzero_energy"] = int(n_nonzero)
        c["flops"] = c["add"] + c["mul"]
        c["flops_per_pair"] = c["flops"] / max(n_in, 1)
        out["terms"][_abi.TERM_NAMES[t]] = c
    # bonds
    bp = _abi.bonded_from_dict(bonded.params["backbone"])
    L.ref_count_reset()
    for a, b in bonds:
        Rc = pos[b] - pos[a]
        Rc -= box * np.round(Rc / box)
        O.eval_bonded(L, "ref", bp, Rc, q[a], q[b], ty[a], ty[b])
    c = read_counts(L)
    c["bonds"] = int(len(bonds))
    c["flops"] = c["add"] + c["mul"]
    c["flops_per_bond"] = c["flops"] / max(len(bonds), 1)
    out["bonded"] = c
    allc = list(out["terms"].values()) + [c]
    out["flops_per_step"] = int(sum(x["flops"] for x in allc))
    out["special_per_step"] = {k: int(sum(x[k] for x in allc)) for k in OPS[2:]}
    return out


def main():
    L = count_lib()
    res = {"ops": list(OPS),
           "note": "FP32 operations of the reference's evaluate() / oxdna_bonded_pair() "
                   "arithmetic per MD step at the initial snapshot: flops = add + mul "
                   "(an FMA counts two); div, sqrt, exp, log, acos, sin, cos counted apart. "
                   "Driver work (min image, scatter, integrator) is not included.",
           "workloads": {}}
    for name, *args in WORKLOADS:
        t0 = time.time()
        res["workloads"][name] = census(L, name, *args)
        print(f"{name}: {res['workloads'][name]['flops_per_step']:.4g} flops/step "
              f"({time.time() - t0:.0f} s)")
    with open(OUT, "w") as fh:
        json.dump(res, fh, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
