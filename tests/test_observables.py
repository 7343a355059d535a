"""Observables for comparing force paths: block averages, paired fraction, the 2-sigma
agreement test, and the sampling loop (driven here by a stand-in simulation)."""

import math
import types

import numpy as np
import pytest

from oxdna import observables as obs


def _ar1(n, phi, rng, mu=0.0):
    x = np.empty(n)
    x[0] = rng.normal()
    e = rng.normal(size=n) * math.sqrt(1 - phi * phi)
    for t in range(1, n):
        x[t] = phi * x[t - 1] + e[t]
    return x + mu


def test_block_average_standard_error_of_a_correlated_series():
    rng = np.random.default_rng(0)
    phi, n = 0.9, 200_000
    x = _ar1(n, phi, rng, mu=3.0)
    m, se = obs.block_average(x, n_blocks=100)  # blocks of 2000 >> the correlation time 19
    # AR(1) with unit variance: var(mean) = (1 + phi) / (1 - phi) / n
    se_true = math.sqrt((1 + phi) / (1 - phi) / n)
    assert abs(m - 3.0) < 5 * se_true
    assert 0.7 * se_true < se < 1.35 * se_true  # the estimate's own spread is ~7%
    # the naive standard error of independent samples is far too small
    assert x.std() / math.sqrt(n) < 0.35 * se
    with pytest.raises(ValueError):
        obs.block_average([1.0, 2.0], n_blocks=10)


def test_agreement_and_paired_fraction():
    assert obs.agree((1.0, 0.1), (1.25, 0.1))        # 0.25 <= 2 * 0.141
    assert not obs.agree((1.0, 0.1), (1.35, 0.1))
    assert obs.paired_fraction([-0.3, -0.06, -0.04, 0.0]) == 0.5
    assert obs.paired_fraction([]) == 0.0
    rng = np.random.default_rng(1)
    a = {"E": _ar1(20_000, 0.5, rng, mu=-1.0)}
    b = {"E": _ar1(20_000, 0.5, rng, mu=-1.0)}
    c = {"E": _ar1(20_000, 0.5, rng, mu=-0.9)}
    assert obs.compare(a, b)["E"]["agree"]
    assert not obs.compare(a, c)["E"]["agree"]


def test_sample_loop_reads_each_force_and_the_hb_force():
    class HydrogenBonding:
        def __init__(self):
            self.energy = 0.0
            self.energies = np.zeros(4)

    class ExcludedVolume:
        energy = 2.0

    hb, ev = HydrogenBonding(), ExcludedVolume()
    steps = []

    def run(n):
        steps.append(n)
        k = len(steps)
        hb.energy = -0.1 * k
        hb.energies = np.array([-0.2, -0.2, 0.0, 0.0]) if k % 2 else np.zeros(4)

    sim = types.SimpleNamespace(run=run, state=types.SimpleNamespace(N_particles=4))
    s = obs.sample(sim, [hb, ev], steps=50, every=10)
    assert steps == [10] * 5
    assert np.allclose(s["HydrogenBonding"], [-0.025 * k for k in range(1, 6)])
    assert np.allclose(s["ExcludedVolume"], 0.5)
    assert s["paired_fraction"].tolist() == [0.5, 0.0, 0.5, 0.0, 0.5]
