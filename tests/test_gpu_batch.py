"""Batched replicas (many small independent systems in one persistent launch):
per-replica energies against the FP64 oracle, forces against the single-system engine,
trajectories against single-system runs with the same Philox seed, and invariance of the
results under the tile shape chosen by hand or by the autotuner."""

import numpy as np
import pytest

from _util import TOL_GPU, maxrel

pytestmark = pytest.mark.gpu


def _workload(n=12, seed=4, bp=(12, 64)):
    from oxdna import replicas
    return replicas.replica_workload(n, bp_range=bp, seed=seed)


def _batch(work, seed=11, fused=False):
    from oxdna import replicas
    sims = [replicas.replica_simulation(s, T, seed=seed + r, fused=fused)
            for r, (s, T) in enumerate(work)]
    return replicas.ReplicaBatch(sims, seed=seed), sims


@pytest.mark.parametrize("fused", [False, True])
def test_batch_energies_match_oracle(native, oracle, fused):
    """Each replica's nine energies (six pair terms, FENE, bonded excluded volume,
    stacking) at its own temperature against the FP64 oracle."""
    from oxdna import io
    work = _workload()
    b, sims = _batch(work, fused=fused)
    _, _, e = b.compute()
    for r, (s, _T) in enumerate(work):
        model = oracle.Model(sims[r]._forces, io.DNA_BASES)
        ref = oracle.forces(model, oracle.System(s["pos"], s["quat"], s["typeid"], s["box"],
                                                 s["bonds"]))
        want = np.concatenate([ref["pair_energy"], ref["bonded_energy"]])
        scale = np.abs(want).max()
        assert np.abs(e[r] - want).max() <= TOL_GPU * scale, (r, e[r], want)


def test_batch_forces_match_single_engine(native):
    """Forces and torques of every replica equal the single-system engine's (both FP32;
    only the summation order differs)."""
    work = _workload(10, seed=5)
    b, sims = _batch(work)
    f, t, _ = b.compute()
    for r, sim in enumerate(sims):
        sim.run(0)
        F = sum(sim._force_arrays(x)[0] for x in sim._forces)
        T = sum(sim._force_arrays(x)[1] for x in sim._forces)
        s = slice(int(b.offsets[r]), int(b.offsets[r + 1]))
        assert maxrel(f[s, :3], F) < 1e-5
        assert maxrel(t[s, :3], T) < 1e-5


def test_batch_trajectory_matches_single_runs(native):
    """Replica r with seed + r follows Simulation(seed=seed + r) over 20 steps, in two
    runs of 10 (each run starts with HOOMD's prepRun, as the single engine does)."""
    work = _workload(6, seed=6)
    b, sims = _batch(work, seed=21)
    b.run(10)
    b.run(10)
    for r, sim in enumerate(sims):
        sim.run(10)
        sim.run(10)
        p = sim.state.get_snapshot().particles
        x = b.positions(r)
        L = work[r][0]["box"][0]
        d = x - p.position
        d -= L * np.round(d / L)
        assert np.abs(d).max() < 2e-3, r
        vel = b.get_state()[3][int(b.offsets[r]):int(b.offsets[r + 1]), :3]
        assert np.abs(vel - p.velocity).max() < 2e-2, r


def test_long_run_chunks_continue(native):
    """A run longer than one launch (5000 steps) continues the integrator across
    launches; the replicas stay finite and hybridised."""
    work = _workload(8, seed=7, bp=(20, 30))
    b, sims = _batch(work, seed=3)
    b.run(6000)
    _, _, e = b.compute()
    n = np.diff(b.offsets)
    assert np.isfinite(e).all()
    # oxDNA2 duplexes of 20-30 bp stay hybridised at 290-340 K over 18 time units
    assert (e[:, 1] / n < -0.1).all(), e[:, 1] / n


def test_tile_shapes_agree_and_tuner_keeps_state(native):
    """Forces do not depend on how replicas are packed into tiles; the autotuner picks a
    valid shape and leaves the state as it found it."""
    work = _workload(24, seed=8)
    b, _ = _batch(work)
    ref = b.compute()[0]
    for tile, threads in ((128, 64), (256, 128), (512, 256)):
        b.set_tiling(tile, threads)
        assert maxrel(b.compute()[0][:, :3], ref[:, :3]) < 1e-5, (tile, threads)
    before = b.get_state()
    tile, threads, ms = b.tune(trial_steps=20)
    assert tile >= 128 and threads in (64, 128, 256) and ms > 0.0
    after = b.get_state()
    for x, y in zip(before, after):
        assert np.array_equal(x, y)
    assert maxrel(b.compute()[0][:, :3], ref[:, :3]) < 1e-5


def test_replica_larger_than_tile_is_rejected(native):
    from oxdna import _abi
    work = _workload(2, seed=9, bp=(64, 64))
    b, _ = _batch(work)
    with pytest.raises(_abi.OxgError, match="tile capacity"):
        b.set_tiling(64, 64)


def test_mixed_duplexes_and_hairpins(native, oracle):
    """Replicas of uneven size mixing duplexes and hairpins (half of them single-strand
    hairpins of the same nucleotide count): per-replica energies against the FP64
    oracle, then 20 steps that follow single-system runs with the same seeds."""
    from oxdna import io, replicas
    work = replicas.replica_workload(10, bp_range=(12, 40), seed=12, hairpin_fraction=0.5)
    kinds = [len(s["bonds"]) == len(s["pos"]) - 1 for s, _ in work]  # one strand: a hairpin
    assert any(kinds) and not all(kinds)
    b, sims = _batch(work, seed=31)
    _, _, e = b.compute()
    for r, (s, _T) in enumerate(work):
        model = oracle.Model(sims[r]._forces, io.DNA_BASES)
        ref = oracle.forces(model, oracle.System(s["pos"], s["quat"], s["typeid"], s["box"],
                                                 s["bonds"]))
        want = np.concatenate([ref["pair_energy"], ref["bonded_energy"]])
        assert np.abs(e[r] - want).max() <= TOL_GPU * np.abs(want).max(), (r, kinds[r])
    b.run(20)
    for r, sim in enumerate(sims):
        sim.run(20)
        x = b.positions(r)
        p = sim.state.get_snapshot().particles.position
        L = work[r][0]["box"][0]
        d = x - p
        d -= L * np.round(d / L)
        assert np.abs(d).max() < 2e-3, (r, kinds[r])
