"""The runtime's paths between run() calls on a real GPU context: a checkpoint written
mid-run and resumed in a fresh simulation continues the same trajectory (the bath
noise of step t depends only on the seed, t and the particle), a changed kT is passed
to the engine without losing the state, and changed force parameters rebuild the
native context and system from the state pulled back to the host. Each case is
compared with a simulation built directly in the end configuration."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KT = 0.1 * 296.15 / 300.0


def _system():
    from oxdna import io
    return io.duplex_system(6, 12, 30.0, seed=9)


def _sim(snap, forces, kT=KT, seed=7):
    from oxdna import runtime
    sim = runtime.Simulation(device=runtime.device.GPU(), seed=seed)
    sim.create_state_from_snapshot(snap)
    lang = runtime.md.methods.Langevin(filter=runtime.filter.All(), kT=kT)
    sim.operations.integrator = runtime.md.Integrator(dt=0.003, integrate_rotational_dof=True,
                                                      forces=forces, methods=[lang])
    return sim, lang


def _pos_diff(a, b, L):
    d = a.particles.position - b.particles.position
    d -= L * np.round(d / L)
    return np.abs(d).max()


def test_checkpoint_resume_continues_the_trajectory(native, tmp_path):
    from oxdna import io, runtime
    from oxdna.model import dna2
    s = _system()
    forces, _ = dna2.forces()
    a, _ = _sim(io.system_snapshot(s), forces)
    a.run(25)
    runtime.write_snapshot(a.state.get_snapshot(), tmp_path / "ck.npz")
    a.run(25)
    end_a = a.state.get_snapshot()
    assert a.timestep == 50 and end_a.configuration.step == 50

    back = runtime.read_snapshot(tmp_path / "ck.npz")
    assert back.configuration.step == 25
    forces_b, _ = dna2.forces()
    b, _ = _sim(back, forces_b)
    assert b.timestep == 25
    b.run(25)
    end_b = b.state.get_snapshot()
    assert b.timestep == 50
    L = s["box"][0]
    # same noise stream and state: only the order of the FP32 force atomics differs
    assert _pos_diff(end_a, end_b, L) < 2e-3
    assert np.abs(end_a.particles.velocity - end_b.particles.velocity).max() < 2e-2
    # a run that replayed the noise from step 0 instead would differ at the noise scale
    c, _ = _sim(back, dna2.forces()[0])
    c.timestep = 0
    c._snap.configuration.step = 0
    c.run(25)
    assert np.abs(end_a.particles.velocity - c.state.get_snapshot().particles.velocity).max() > 5e-2


def test_changed_kT_between_runs(native):
    from oxdna import io
    from oxdna.model import dna2
    s = _system()
    a, lang = _sim(io.system_snapshot(s), dna2.forces()[0])
    a.run(20)
    mid = a.state.get_snapshot()
    lang.kT = 2.0 * KT  # passed to the engine before the next run, state kept
    a.run(20)
    b, _ = _sim(mid, dna2.forces()[0], kT=2.0 * KT)
    b.run(20)
    L = s["box"][0]
    assert a.timestep == b.timestep == 40
    assert _pos_diff(a.state.get_snapshot(), b.state.get_snapshot(), L) < 2e-3


def test_changed_parameters_rebuild_with_state_kept(native):
    """A changed parameter dict rebuilds the native context and system from the state
    pulled back to the host; the next run continues from that state with the new
    parameters, as a simulation built from the same snapshot with them does."""
    from oxdna import io
    from oxdna.model import dna2
    s = _system()
    forces, _ = dna2.forces()
    a, _ = _sim(io.system_snapshot(s), forces)
    a.run(20)
    mid = a.state.get_snapshot()
    e_before = forces[2].energy
    hb = forces[2]  # hydrogen bonding
    for key in list(hb.params.keys()):
        p = dict(hb.params[key])
        p["eps"] = 1.5 * p["eps"]
        hb.params[key] = p
    e_after = hb.energy  # read-out with the new parameters on the carried-over state
    assert e_after == pytest.approx(1.5 * e_before, rel=1e-4)
    a.run(20)

    forces_b, _ = dna2.forces()
    for key in list(forces_b[2].params.keys()):
        p = dict(forces_b[2].params[key])
        p["eps"] = 1.5 * p["eps"]
        forces_b[2].params[key] = p
    b, _ = _sim(mid, forces_b)
    b.run(20)
    L = s["box"][0]
    assert a.timestep == b.timestep == 40
    assert _pos_diff(a.state.get_snapshot(), b.state.get_snapshot(), L) < 2e-3


def test_run_start_reuses_the_last_steps_forces(native):
    """A run that follows another with nothing changed in between starts from the forces
    the previous run left for its final state instead of evaluating them again (HOOMD's
    prepRun recomputes the same forces); the trajectory equals one whose run start does
    evaluate them (the state marked as changed through the C ABI), up to the order of
    the FP32 force sums."""
    import ctypes as C

    from oxdna import _abi, io
    from oxdna.model import dna2
    s = _system()
    ends = []
    for mark_changed in (False, True):
        sim, _ = _sim(io.system_snapshot(s), dna2.forces()[0])
        sim.run(15)
        if mark_changed:
            _abi.check(native.oxg_system_set_state(sim._sys, None, None, None, None, None, None),
                       "oxg_system_set_state")
        sim.run(15)
        ends.append(sim.state.get_snapshot())
    L = s["box"][0]
    assert _pos_diff(ends[0], ends[1], L) < 1e-4
    assert np.abs(ends[0].particles.velocity - ends[1].particles.velocity).max() < 1e-3


@pytest.mark.parametrize("path", ["run", "host", "session"])
@pytest.mark.parametrize("kind", ["nan", "type"])
def test_bad_state_is_reported_and_the_system_recovers(native, path, kind):
    """A NaN coordinate, or a particle type outside the context's types, in the state
    handed to the engine (through push_state_arrays and run(), or page-locked host arrays
    and run_state_arrays, with and without a host session) is reported after the run
    (non-finite state; bad index), the timestep is left where it was, and the system then
    runs on from a valid state as a twin that never saw the bad one does. Both are made
    on the host: a NaN position fails every cutoff test and its cell coordinate is
    clamped, the integrator's check raises the flag; every pair and bond evaluation
    checks both types before it reads a parameter and skips the pair."""
    import torch

    from oxdna import _abi, io
    from oxdna.model import dna2
    s = _system()
    n = len(s["pos"])
    a, _ = _sim(io.system_snapshot(s), dna2.forces()[0])
    b, _ = _sim(io.system_snapshot(s), dna2.forces()[0])
    a.run(5)
    b.run(5)
    good = [torch.zeros((n, 4), dtype=torch.float32).pin_memory().numpy() for _ in range(5)]
    a.pull_state_arrays(*good)
    bad = [torch.zeros((n, 4), dtype=torch.float32).pin_memory().numpy() for _ in range(5)]
    for x, y in zip(bad, good):
        x[:] = y
    if kind == "nan":
        bad[0][3, 0] = np.nan
    else:
        bad[0][3, 3] = np.array([99], dtype=np.int32).view(np.float32)[0]
    if path == "session":
        a.set_host_session(2000)
    with pytest.raises(_abi.OxgError) as err:
        if path == "run":
            a.push_state_arrays(*bad)
            a.run(10)
        else:
            a.run_state_arrays(10, *bad)
    assert err.value.code == (_abi.ERR_NONFINITE if kind == "nan" else _abi.ERR_BAD_INDEX)
    assert a.timestep == 5
    if path == "run":
        a.push_state_arrays(*good)
        a.run(10)
        end_a = a.state.get_snapshot()
        pos_a, vel_a = end_a.particles.position, end_a.particles.velocity
    else:
        a.run_state_arrays(10, *good)
        pos_a = good[0][:, :3].astype(np.float64) + good[1][:, :3]
        vel_a = good[3][:, :3]
    a.set_host_session(0)
    b.run(10)
    end_b = b.state.get_snapshot()
    assert a.timestep == b.timestep == 15
    assert np.isfinite(pos_a).all()
    d = pos_a - end_b.particles.position
    L = s["box"][0]
    d -= L * np.round(d / L)
    assert np.abs(d).max() < 1e-3
    assert np.abs(vel_a - end_b.particles.velocity).max() < 1e-2
