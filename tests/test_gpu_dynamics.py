"""GPU engine at the benchmark sizes: energies against the FP64 oracle on the 8000-nt
system, size-independent properties (Newton's third law, fused == separate), and the
Langevin / NO_SQUISH integrator (oracle trajectory, duplex stability, equipartition)."""

import numpy as np
import pytest

from _util import TOL_GPU, maxrel

pytestmark = pytest.mark.gpu


def _sim(snap, forces, dt=0.0, kT=None, seed=1):
    from oxdna import runtime
    sim = runtime.Simulation(device=runtime.device.GPU(), seed=seed)
    sim.create_state_from_snapshot(snap)
    methods = [] if kT is None else [runtime.md.methods.Langevin(filter=runtime.filter.All(), kT=kT)]
    sim.operations.integrator = runtime.md.Integrator(dt=dt, integrate_rotational_dof=True,
                                                      forces=list(forces), methods=methods)
    sim.run(0)
    return sim


@pytest.mark.parametrize("fused", [False, True])
def test_8000nt_energies_match_oracle(native, oracle, fused):
    """200 x 20-bp duplexes, box 100 (the headline system): every per-term energy."""
    from oxdna import io
    from oxdna.model import dna2
    s = io.duplex_system(200, 20, 100.0, seed=2)
    forces, _ = dna2.forces(fused=fused)
    sim = _sim(io.system_snapshot(s), forces)
    model = oracle.Model(forces, io.DNA_BASES)
    r = oracle.forces(model, oracle.System(s["pos"], s["quat"], s["typeid"], s["box"], s["bonds"]))
    for f in forces[1:]:
        ref = r["pair_energy"][f._term]
        assert abs(f.energy - ref) <= TOL_GPU * max(abs(ref), 1e-6), type(f).__name__
    b = forces[0]
    for k, v in enumerate((b.fene_energy, b.bonded_excvol_energy, b.stacking_energy)):
        ref = r["bonded_energy"][k]
        assert abs(v - ref) <= TOL_GPU * max(abs(ref), 1e-6)
    # Newton's third law on the summed GPU forces
    F = sum(sim._force_arrays(f)[0] for f in forces)
    assert np.linalg.norm(F.sum(axis=0)) < 1e-4 * np.abs(F).max() * np.sqrt(len(F))
    # per-particle forces and torques (measured ~8e-6 / ~6e-6 max-norm relative; pairs
    # across the periodic boundary included: ~2e-4 when the image shift rounded the
    # position difference at the ulp of the box length)
    T = sum(sim._force_arrays(f)[1] for f in forces)
    assert maxrel(F, r["force"]) < 5e-5
    assert maxrel(T, r["torque"]) < 5e-5


def test_rna_hairpins_energies_match_oracle_and_run(native, oracle):
    """oxRNA2 on 64 hairpins x 48 nt (16-bp stem, 16-nt loop, extended-helix start), box
    80, 310.15 K, 1 M salt: every per-term energy against the FP64 oracle, then 500
    Langevin steps (dt 0.002) that stay finite with the strands still stacked (the
    stems start unpaired, as extended helices)."""
    from oxdna import io
    from oxdna.model import dna1, rna2
    s = io.hairpin_system(64, stem=16, loop=16, box_len=80.0, seed=3)
    forces, _ = rna2.forces(temperature=310.15, salt=1.0)
    kT = dna1.kT_from_temperature(310.15)
    sim = _sim(io.system_snapshot(s), forces, dt=0.002, kT=kT, seed=9)
    model = oracle.Model(forces, io.DNA_BASES)
    r = oracle.forces(model, oracle.System(s["pos"], s["quat"], s["typeid"], s["box"], s["bonds"]))
    for f in forces[1:]:
        ref = r["pair_energy"][f._term]
        assert abs(f.energy - ref) <= TOL_GPU * max(abs(ref), 1e-6), type(f).__name__
    b = forces[0]
    for k, v in enumerate((b.fene_energy, b.bonded_excvol_energy, b.stacking_energy)):
        ref = r["bonded_energy"][k]
        assert abs(v - ref) <= TOL_GPU * max(abs(ref), 1e-6)
    sim.run(500)
    assert np.isfinite(sim.state.get_snapshot().particles.position).all()
    assert np.isfinite(b.fene_energy) and b.fene_energy < 1e6  # no broken backbone bond
    assert b.stacking_energy < 0.0


@pytest.mark.parametrize("mode", ["persistent", "graph", "persistent-spill"])
def test_short_trajectory_tracks_oracle(native, oracle, monkeypatch, mode):
    """Same counter-based RNG on both sides: 20 Langevin steps agree closely, on the
    persistent run kernel, on the per-step kernels replayed from a CUDA graph, and on
    the run kernel with its per-block phase-A queues cut to 3 pairs (the pairs that do
    not fit go through the global queues after the force barrier)."""
    from oxdna import io
    from oxdna.model import dna1, dna2
    monkeypatch.setenv("OXG_RUN_MODE", mode.split("-")[0])
    if mode.endswith("spill"):  # per-block phase-A queues of 3 pairs: most pairs spill
        monkeypatch.setenv("OXG_BLOCK_QUEUE", "3")
    s = io.duplex_system(8, 20, 40.0, seed=1)
    kT = dna1.kT_from_temperature(296.15)
    forces, _ = dna2.forces()
    sim = _sim(io.system_snapshot(s), forces, dt=0.003, kT=kT, seed=7)
    sim.run(20)
    snap = sim.state.get_snapshot()
    model = oracle.Model(forces, io.DNA_BASES)
    o = oracle.System(s["pos"], s["quat"], s["typeid"], s["box"], s["bonds"])
    n = len(s["pos"])
    _, vel, am = oracle.langevin(model, o, np.zeros((n, 3)), np.zeros((n, 4)), steps=20, dt=0.003,
                                 kT=kT, seed=7)
    d = snap.particles.position - o.pos
    d -= 40.0 * np.round(d / 40.0)
    assert np.abs(d).max() < 2e-3
    assert np.abs(snap.particles.velocity - vel).max() < 2e-2
    q = snap.particles.orientation
    assert np.abs(np.abs(np.einsum("ij,ij->i", q, o.quat)) - 1.0).max() < 1e-3


def test_large_system_frequent_rebuilds_track_oracle(native, oracle):
    """84,000 nt (more particles than the persistent run kernel has threads) with a
    0.002-sigma list buffer, so the kernel rebuilds its neighbour list every step or two:
    20 steps follow the FP64 oracle's Langevin trajectory (same Philox stream)."""
    import os
    from oxdna import io
    from oxdna.model import dna1, dna2
    s = io.duplex_system(2100, 20, 220.0, seed=3)
    kT = dna1.kT_from_temperature(296.15)
    forces, _ = dna2.forces(nlist=dna2.make_neighbor_list(buffer=0.002))
    sim = _sim(io.system_snapshot(s), forces, dt=0.003, kT=kT, seed=7)
    sim.run(20)
    st = sim.native_stats()
    assert st["nlist_builds"] >= 5
    snap = sim.state.get_snapshot()
    model = oracle.Model(forces, io.DNA_BASES)
    o = oracle.System(s["pos"], s["quat"], s["typeid"], s["box"], s["bonds"])
    n = len(s["pos"])
    _, vel, _ = oracle.langevin(model, o, np.zeros((n, 3)), np.zeros((n, 4)), steps=20,
                                dt=0.003, kT=kT, seed=7, threads=os.cpu_count())
    d = snap.particles.position - o.pos
    d -= 220.0 * np.round(d / 220.0)
    assert np.abs(d).max() < 2e-3
    assert np.abs(snap.particles.velocity - vel).max() < 2e-2


def test_duplexes_stay_bound_and_thermalise(native):
    """pytest/test_oxdna2.py:72-80: HB per nucleotide < -0.15 after 2000 steps; the
    kinetic temperatures approach kT (equipartition, 3 + 3 degrees of freedom)."""
    from oxdna import io
    from oxdna.model import dna1, dna2
    s = io.duplex_system(8, 20, 40.0, seed=1)
    kT = dna1.kT_from_temperature(296.15)
    forces, _ = dna2.forces()
    sim = _sim(io.system_snapshot(s), forces, dt=0.003, kT=kT, seed=5)
    sim.run(2000)
    n = len(s["pos"])
    snap = sim.state.get_snapshot()
    assert np.isfinite(snap.particles.position).all()
    assert forces[2].energy / n < -0.15
    ke_t, ke_r = [], []
    for _ in range(20):
        sim.run(50)
        p = sim.state.get_snapshot().particles
        ke_t.append(0.5 * (p.velocity ** 2).sum() / n)
        q, pm = p.orientation, p.angmom
        # body angular momentum s = (1/2 conj(q) p).v, unit inertia
        sv = 0.5 * (q[:, :1] * pm[:, 1:] - pm[:, :1] * q[:, 1:] - np.cross(q[:, 1:], pm[:, 1:]))
        ke_r.append(0.5 * (sv ** 2).sum() / n)
    assert abs(np.mean(ke_t) / (1.5 * kT) - 1.0) < 0.1
    assert abs(np.mean(ke_r) / (1.5 * kT) - 1.0) < 0.1
    st = sim.native_stats()
    assert st["nlist_builds"] >= 1 and st["steps"] == 3000


def test_state_push_pull_pinned_and_pageable(native):
    """oxg_system_set_state / get_state move the state through one kernel when the host
    arrays are page-locked (mapped) memory and through per-array copies otherwise: both
    routes carry the same bytes, and a pushed state steps the same way from either."""
    import torch
    from oxdna import io
    from oxdna.model import dna1, dna2
    s = io.duplex_system(8, 20, 40.0, seed=3)
    forces, _ = dna2.forces()
    sim = _sim(io.system_snapshot(s), forces, dt=0.003, kT=dna1.kT_from_temperature(296.15), seed=5)
    sim.run(10)
    n = len(s["pos"])
    pageable = [np.zeros((n, 4), np.float32) for _ in range(5)]
    pinned = [torch.zeros((n, 4), dtype=torch.float32).pin_memory().numpy() for _ in range(5)]
    sim.pull_state_arrays(*pageable)
    sim.pull_state_arrays(*pinned)
    for a, b in zip(pageable, pinned):
        assert a.tobytes() == b.tobytes()
    # push a modified state through the pinned route, read it back through the other
    rng = np.random.Generator(np.random.PCG64(1))
    pinned[3][:, :3] = rng.normal(0, 0.1, (n, 3)).astype(np.float32)
    sim.push_state_arrays(*pinned)
    back = [np.zeros((n, 4), np.float32) for _ in range(5)]
    sim.pull_state_arrays(*back)
    for a, b in zip(pinned, back):
        assert a.tobytes() == b.tobytes()
    # the same state pushed either way into twin systems (same seed and timestep) steps
    # identically
    twin = _sim(io.system_snapshot(s), forces, dt=0.003, kT=dna1.kT_from_temperature(296.15), seed=5)
    twin.run(10)
    out = []
    for sm, src in ((sim, pinned), (twin, [a.copy() for a in pinned])):
        sm.push_state_arrays(*src)
        sm.run(1)
        res = [np.zeros((n, 4), np.float32) for _ in range(5)]
        sm.pull_state_arrays(*res)
        out.append(res)
    # (float atomics sum in no fixed order: agreement to rounding, not bitwise)
    for a, b in zip(*out):
        assert np.allclose(a, b, rtol=1e-5, atol=1e-5)
    assert not np.array_equal(out[0][0], pinned[0])


@pytest.mark.parametrize("steps", [1, 4])
@pytest.mark.parametrize("memory", ["pinned", "pageable"])
def test_run_state_arrays_matches_push_run_pull(native, memory, steps):
    """oxg_system_run_host (one call: state in, n steps, state out) against
    push_state_arrays + run + pull_state_arrays on a twin system (same seed and
    timestep): with page-locked arrays the run kernel itself reads the host state at the
    run start (reusing the last step's forces when it equals the device state, as in
    the second and fourth calls here: it then takes the first step one in the same pass
    as the host read) and writes the final state back; with pageable arrays the call
    falls back to the three steps. The first and third calls bring a host-side change of
    the velocities (the step one taken with the host read is undone from the
    checkpoint)."""
    import torch
    from oxdna import io
    from oxdna.model import dna1, dna2
    s = io.duplex_system(8, 20, 40.0, seed=4)
    forces, _ = dna2.forces()
    kT = dna1.kT_from_temperature(296.15)
    a = _sim(io.system_snapshot(s), forces, dt=0.003, kT=kT, seed=9)
    b = _sim(io.system_snapshot(s), forces, dt=0.003, kT=kT, seed=9)
    a.run(5)
    b.run(5)
    n = len(s["pos"])
    if memory == "pinned":
        alloc = lambda: torch.zeros((n, 4), dtype=torch.float32).pin_memory().numpy()  # noqa: E731
    else:
        alloc = lambda: np.zeros((n, 4), np.float32)  # noqa: E731
    st_a = [alloc() for _ in range(5)]
    a.pull_state_arrays(*st_a)
    rng = np.random.Generator(np.random.PCG64(2))
    st_a[3][:, :3] += rng.normal(0, 0.05, (n, 3)).astype(np.float32)  # a host-side change
    st_b = [x.copy() for x in st_a]
    for it in range(4):
        if it == 2:  # another host-side change between calls
            st_a[3][:, :3] *= np.float32(0.9)
            st_b[3][:, :3] *= np.float32(0.9)
        a.run_state_arrays(steps, *st_a)
        b.push_state_arrays(*st_b)
        b.run(steps)
        b.pull_state_arrays(*st_b)
    assert a.timestep == b.timestep
    for x, y in zip(st_a, st_b):
        assert np.allclose(x, y, rtol=1e-5, atol=1e-5)
    # the device state is the returned state: a plain run continues from it
    a.run(2)
    b.run(2)
    pa = [np.zeros((n, 4), np.float32) for _ in range(5)]
    pb = [np.zeros((n, 4), np.float32) for _ in range(5)]
    a.pull_state_arrays(*pa)
    b.pull_state_arrays(*pb)
    for x, y in zip(pa, pb):
        assert np.allclose(x, y, rtol=1e-5, atol=1e-5)
    # a particle type outside the context's types is an error (found by the run kernel
    # on page-locked arrays, before any GPU work on pageable ones)
    from oxdna import _abi
    st_a[0][7, 3] = np.array([99], np.int32).view(np.float32)[0]
    with pytest.raises(_abi.OxgError, match="status 4"):
        a.run_state_arrays(1, *st_a)


def test_host_session_matches_a_launch_per_call(native):
    """A host session (the run kernel resident between run_state_arrays calls, each call
    a request in page-locked memory) against the same calls with a launch each, on twin
    systems driven one after the other (a resident kernel holds every SM, so interleaved
    calls of another system would wait for it to leave): one-step calls with the host
    state unchanged and changed between calls, a four-step call, another call on the
    simulation in between (it ends the session), a pause longer than the idle time (the
    kernel leaves; the next call launches again) and a parameter change (the native system
    is rebuilt, the session set again). Most calls were served by the resident kernel."""
    import time

    import torch
    from oxdna import io
    from oxdna.model import dna1, dna2
    s = io.duplex_system(8, 20, 40.0, seed=4)
    kT = dna1.kT_from_temperature(296.15)
    n = len(s["pos"])

    def drive(session_us):
        forces, _ = dna2.forces()
        sim = _sim(io.system_snapshot(s), forces, dt=0.003, kT=kT, seed=9)
        st = [torch.zeros((n, 4), dtype=torch.float32).pin_memory().numpy() for _ in range(5)]
        sim.pull_state_arrays(*st)
        sim.set_host_session(session_us)
        served = 0
        for it in range(40):
            if it == 10:  # a host-side change of the velocities
                st[3][:, :3] *= np.float32(0.9)
            if it == 20:  # another call on the simulation ends the session
                sim.native_stats()
            if it == 25:  # longer than the idle time: a resident kernel has left
                time.sleep(0.05)
            if it == 30:  # a parameter change (the counter of the system it replaces first)
                served = sim.native_stats()["session_served"]
                for key in list(forces[2].params.keys()):
                    p = dict(forces[2].params[key])
                    p["eps"] = 1.1 * p["eps"]
                    forces[2].params[key] = p
            sim.run_state_arrays(4 if it == 15 else 1, *st)
        served += sim.native_stats()["session_served"]
        assert sim.timestep == 39 + 4
        sim.set_host_session(0)
        return st, served

    st_a, served_a = drive(2000)
    st_b, served_b = drive(0)
    for x, y in zip(st_a, st_b):
        assert np.allclose(x, y, rtol=1e-5, atol=1e-5)
    # launched: the first call and the calls after the stats call, the pause and the
    # rebuild (36 of the 40 served otherwise)
    assert served_a >= 30 and served_b == 0, (served_a, served_b)


@pytest.mark.parametrize("fused", [False, True])
def test_run_kernel_forces_match_oracle(native, oracle, fused):
    """The run kernel's own force evaluation (the run start's and the step's: phase A and
    the block-local phase B) checked through one noiseless Langevin step of the 8000-nt
    system: with kT = 0 the velocity and angular momentum after the step are
    deterministic sums of the forces and torques of the start and end positions, so they
    match the FP64 oracle's step to FP32 rounding."""
    from oxdna import io
    from oxdna.model import dna2
    s = io.duplex_system(200, 20, 100.0, seed=2)
    forces, _ = dna2.forces(fused=fused)
    sim = _sim(io.system_snapshot(s), forces, dt=0.003, kT=0.0, seed=3)
    sim.run(1)
    snap = sim.state.get_snapshot()
    model = oracle.Model(forces, io.DNA_BASES)
    o = oracle.System(s["pos"], s["quat"], s["typeid"], s["box"], s["bonds"])
    n = len(s["pos"])
    import os
    _, vel, am = oracle.langevin(model, o, np.zeros((n, 3)), np.zeros((n, 4)), steps=1, dt=0.003,
                                 kT=0.0, seed=3, threads=os.cpu_count())
    assert maxrel(snap.particles.velocity, vel) < 1e-4
    assert maxrel(snap.particles.angmom, am) < 1e-4
