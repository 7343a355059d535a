"""Trajectory observables and their statistical comparison.

Used to check that a modified force path (the learned surrogate, the batched engine)
reproduces the plain path's thermodynamics: block-averaged means with standard errors
of per-term energies and of the fraction of formed base pairs, and a test of whether
two such means agree within k combined standard errors (k = 2: the 2-sigma criterion).
"""

import math

import numpy as np

#: A nucleotide counts as base-paired when its share of hydrogen-bonding energy (half
#: of each of its HB pair energies) is below half of this pair-energy threshold
#: (oxDNA analyses count a base pair as formed below -0.1 simulation units).
HB_PAIR_THRESHOLD = -0.1


def block_average(series, n_blocks=10):
    """(mean, standard error) of a correlated time series by block averaging: the
    series is cut into n_blocks equal blocks (a remainder at the start is dropped) and
    the standard error is that of the block means."""
    x = np.asarray(series, dtype=np.float64).ravel()
    if n_blocks < 2 or len(x) < n_blocks:
        raise ValueError("need at least n_blocks >= 2 samples")
    m = len(x) // n_blocks
    blocks = x[len(x) - m * n_blocks:].reshape(n_blocks, m).mean(axis=1)
    return float(blocks.mean()), float(blocks.std(ddof=1) / math.sqrt(n_blocks))


def paired_fraction(hb_energies, threshold=HB_PAIR_THRESHOLD):
    """Fraction of nucleotides whose per-particle hydrogen-bonding energy (the
    ``energies`` of the HB or fused HB + cross-stacking force) is below threshold / 2."""
    e = np.asarray(hb_energies, dtype=np.float64)
    return float(np.mean(e < 0.5 * threshold)) if e.size else 0.0


def agree(a, b, k=2.0):
    """True when two (mean, standard error) estimates differ by at most k combined
    standard errors."""
    (ma, sa), (mb, sb) = a, b
    return abs(ma - mb) <= k * math.hypot(sa, sb)


def sample(sim, forces, steps, every):
    """Run ``steps`` steps, reading after every ``every`` steps the energy per
    nucleotide of each force and the paired fraction from the hydrogen-bonding force
    (the first force whose name mentions HBond / Hydrogen). Returns a dict of series."""
    n = sim.state.N_particles
    hb = next((f for f in forces if "HBond" in type(f).__name__ or "Hydrogen" in type(f).__name__), None)
    out = {type(f).__name__: [] for f in forces}
    out["paired_fraction"] = []
    for _ in range(max(1, steps // every)):
        sim.run(every)
        for f in forces:
            out[type(f).__name__].append(f.energy / n)
        if hb is not None:
            out["paired_fraction"].append(paired_fraction(hb.energies))
    return {k: np.asarray(v) for k, v in out.items()}


def compare(series_a, series_b, n_blocks=10, k=2.0):
    """Per observable: both block-averaged estimates and whether they agree within k
    combined standard errors."""
    res = {}
    for key in series_a:
        if key in series_b and len(series_a[key]) >= n_blocks and len(series_b[key]) >= n_blocks:
            a = block_average(series_a[key], n_blocks)
            b = block_average(series_b[key], n_blocks)
            res[key] = {"a": a, "b": b, "agree": agree(a, b, k)}
    return res
