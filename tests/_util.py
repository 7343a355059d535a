"""Shared helpers of the test suite (golden fixtures, tolerances, model builders)."""

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TERMS = ("oxdna_excvol", "oxdna_hbond", "oxdna_crossstacking", "oxdna_hbondcross",
         "oxdna_coaxstacking", "oxdna_debye")

# Parity tolerance of the FP32 GPU path against the FP64 reference (the required
# 1e-4 relative), as a set-level max-norm relative error: max|x - x_ref| / max|x_ref|
# over all samples of one term. Per-pair relative errors are not meaningful where the
# reference force is ~0 (ideal geometries), where even the reference's own FP32 build
# differs from its FP64 build by orders of magnitude relative to the tiny value.
TOL_GPU = 1e-4
# The C oracle restates the reference in FP64: agreement to round-off.
TOL_ORACLE = 1e-10


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


# Pair-term golden cases (model, term id, "avg" | "seq"): every term with the
# sequence-averaged parameters, plus the two terms whose parameters depend on the
# sequence (hydrogen bonding and fused HB + cross-stacking: per-type-pair eps,
# reference oxdna/model/dna1.py:186-194, dna2.py:117-121, rna2.py:147-152) with
# average=False.
SEQ_TERMS = (1, 3)
PAIR_CASES = [(m, t, "avg") for m in ("dna1", "dna2", "rna2") for t in range(6)] + \
             [(m, t, "seq") for m in ("dna1", "dna2", "rna2") for t in SEQ_TERMS]


def pair_golden(model, avg):
    return golden(f"pairs_{model}.npz" if avg == "avg" else f"pairs_{model}_seq.npz")


def maxrel(x, ref):
    x = np.asarray(x, float)
    ref = np.asarray(ref, float)
    scale = np.abs(ref).max()
    if scale == 0.0:
        return float(np.abs(x).max())
    return float(np.abs(x - ref).max() / scale)


def model_forces(name, average=True):
    """Six pair-term forces (index = term id) and the bonded force of a model."""
    from oxdna.model import dna1, dna2, rna2
    mod = {"dna1": dna1, "dna2": dna2, "rna2": rna2}[name]
    nl = mod.make_neighbor_list()
    if name == "rna2":
        pair = [rna2.excluded_volume(nl), rna2.hydrogen_bonding(nl, average=average),
                rna2.cross_stacking(nl), dna2.hbond_cross(nl, average=average),
                rna2.coaxial_stacking(nl), rna2.debye_huckel(nl)]
        bonded = rna2.bonded_force(average=average)
    else:
        pair = [mod.excluded_volume(nl), mod.hydrogen_bonding(nl, average=average),
                mod.cross_stacking(nl) if name == "dna1" else dna1.cross_stacking(nl),
                mod.hbond_cross(nl, average=average), mod.coaxial_stacking(nl),
                dna2.debye_huckel(nl)]
        bonded = mod.bonded_force(average=average)
    return pair, bonded
