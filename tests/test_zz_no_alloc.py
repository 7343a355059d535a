"""oxg_pair_forces_noalloc: the nonbonded evaluation for callers that cannot
allocate GPU memory (a framework owning the whole device pool, or a host that forbids
cudaMalloc inside its loop). It keeps all scratch in a fixed static device array, so
it must give the same result as the allocating system engine and as the FP64 oracle,
a second call must not be disturbed by what the first left in that shared array, and a
bond table that lists a bond twice must still fit the four exclusion slots a particle
has.

Collected last on purpose (file name), so a failing run that stops at the first
failure has already run every other test."""

import ctypes as C

import numpy as np
import pytest

from _util import TOL_GPU, maxrel

pytestmark = pytest.mark.gpu


def _state(sysarr):
    """float32 positions (so both paths see identical inputs) and packed device arrays."""
    pos = sysarr["pos"].astype(np.float32).astype(np.float64)
    n = len(pos)
    pt = np.zeros((n, 4), np.float32)
    pt[:, :3] = pos
    pt[:, 3] = sysarr["typeid"].astype(np.int32).view(np.float32)
    return pos, pt, sysarr["quat"].astype(np.float32)


def test_noalloc_matches_engine_on_two_calls(native, oracle):
    import torch

    from oxdna import _abi, io, runtime
    from oxdna.model import dna2

    s = io.duplex_system(200, 20, 100.0, seed=2)  # 8000 nt, within the 8192 limit
    pos, pt, q = _state(s)
    snap = io.snapshot_from_arrays(pos, q.astype(np.float64), s["typeid"], s["box"],
                                   bonds=s["bonds"])
    pair_forces = dna2.forces()[0][1:]
    sim = runtime.Simulation(device=runtime.device.GPU())
    sim.create_state_from_snapshot(snap)
    sim.operations.integrator = runtime.md.Integrator(dt=0.0, integrate_rotational_dof=True,
                                                      forces=pair_forces)
    sim.run(0)
    L = native
    n = len(pos)
    mask = sim._mask
    # the existing (allocating) entry point on the same state
    f_ref = np.zeros((n, 4), np.float32)
    t_ref = np.zeros((n, 4), np.float32)
    e_ref = (C.c_double * 6)()
    be = (C.c_double * 3)()
    _abi.check(L.oxg_system_compute(sim._sys, mask, 0, C.c_void_p(f_ref.ctypes.data),
                                    C.c_void_p(t_ref.ctypes.data), e_ref, be), "compute")
    dev = torch.device("cuda")
    pos_d = torch.tensor(pt, device=dev)
    quat_d = torch.tensor(q, device=dev)
    charge_d = torch.ones(n, dtype=torch.float32, device=dev)
    bonds = np.zeros((len(s["bonds"]), 3), np.int32)
    bonds[:, :2] = np.asarray(s["bonds"], np.int32)
    bonds_d = torch.tensor(bonds.astype(np.int64), device=dev).to(torch.int32)
    box = (C.c_float * 3)(*[float(x) for x in s["box"]])
    ptr = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    for call in range(2):
        force = torch.full((n, 4), float("nan"), dtype=torch.float32, device=dev)
        torque = torch.full((n, 4), float("nan"), dtype=torch.float32, device=dev)
        energy = torch.full((6,), float("nan"), dtype=torch.float64, device=dev)
        _abi.check(L.oxg_pair_forces_noalloc(sim._ctx, mask, n, ptr(pos_d), ptr(quat_d),
                                             ptr(charge_d), box, len(bonds), ptr(bonds_d),
                                             ptr(force), ptr(torque), ptr(energy), None),
                   f"oxg_pair_forces_noalloc call {call + 1}")
        F = force.cpu().numpy()
        T = torque.cpu().numpy()
        E = energy.cpu().numpy()
        assert maxrel(F[:, :3], f_ref[:, :3]) < TOL_GPU, f"call {call + 1}: forces"
        assert maxrel(T[:, :3], t_ref[:, :3]) < TOL_GPU, f"call {call + 1}: torques"
        assert maxrel(F[:, 3], f_ref[:, 3]) < TOL_GPU, f"call {call + 1}: per-particle energy"
        for t in range(6):
            if (mask >> t) & 1:
                assert abs(E[t] - e_ref[t]) <= TOL_GPU * max(abs(e_ref[t]), 1e-6), (call, t)
    # directly against the FP64 oracle on the same (float32-rounded) inputs
    model = oracle.Model(pair_forces, io.DNA_BASES)
    r = oracle.forces(model, oracle.System(pos, q.astype(np.float64), s["typeid"], s["box"],
                                           s["bonds"]), bonded=False)
    assert maxrel(F[:, :3], r["force"]) < 5e-5
    assert maxrel(T[:, :3], r["torque"]) < 5e-5
    for t in range(6):
        if (mask >> t) & 1:
            ref = r["pair_energy"][t]
            assert abs(E[t] - ref) <= TOL_GPU * max(abs(ref), 1e-6), t
    # every bond listed twice, once reversed: duplicates take no extra exclusion slot
    dup = np.concatenate([bonds, bonds[:, [1, 0, 2]]])
    dup_d = torch.tensor(dup.astype(np.int64), device=dev).to(torch.int32)
    force.fill_(float("nan"))
    _abi.check(L.oxg_pair_forces_noalloc(sim._ctx, mask, n, ptr(pos_d), ptr(quat_d),
                                         ptr(charge_d), box, len(dup), ptr(dup_d),
                                         ptr(force), ptr(torque), None, None),
               "oxg_pair_forces_noalloc with duplicated bonds")
    assert maxrel(force.cpu().numpy()[:, :3], f_ref[:, :3]) < TOL_GPU
    # sizes beyond the fixed scratch are rejected before any GPU work
    big = L.oxg_pair_forces_noalloc(sim._ctx, mask, 8193, ptr(pos_d), ptr(quat_d), None, box, 0,
                                    None, ptr(force), ptr(torque), None, None)
    assert big == _abi.ERR_CAPACITY
    assert b"exceeds the fixed maximum" in L.oxg_last_error()
