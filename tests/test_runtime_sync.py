"""The runtime's host logic around the native system, driven against a stand-in for the
native library that records every call and keeps the state in host memory: a changed
kT is passed on without rebuilding, changed force parameters rebuild the context and
system from the pulled-back state, the timestep continues, and a checkpoint restores
it. No device is touched."""

import ctypes as C

import numpy as np
import pytest


class _FakeLib:
    """Enough of the C ABI for attach / run / detach / snapshots."""

    def __init__(self):
        self.calls = []
        self.systems = {}
        self.next = 100

    def _handle(self, out):
        self.next += 1
        out._obj.value = self.next
        return self.next

    def oxg_create(self, out, nt, nb):
        self.calls.append(("create",))
        self._handle(out)
        return 0

    def oxg_system_create(self, out, ctx, n, box, nb, bonds):
        h = self._handle(out)
        self.systems[h] = {"n": n, "state": None, "timestep": 0, "integ": None}
        self.calls.append(("system_create", h))
        return 0

    def oxg_system_destroy(self, s):
        self.calls.append(("system_destroy", s.value if hasattr(s, "value") else s))
        return 0

    def oxg_destroy(self, c):
        return 0

    @staticmethod
    def _arr(ptr, n):
        addr = ptr.value if hasattr(ptr, "value") else ptr
        return np.ctypeslib.as_array((C.c_float * (4 * n)).from_address(addr)).reshape(n, 4)

    def oxg_system_set_state(self, s, pos, lo, q, vel, am, ch):
        sy = self.systems[s.value]
        sy["state"] = [self._arr(p, sy["n"]).copy() for p in (pos, lo, q, vel, am)]
        sy["pushed"] = [a.copy() for a in sy["state"]]
        self.calls.append(("set_state", s.value))
        return 0

    def oxg_system_get_state(self, s, pos, lo, q, vel, am):
        sy = self.systems[s.value]
        for p, a in zip((pos, lo, q, vel, am), sy["state"]):
            self._arr(p, sy["n"])[:] = a
        self.calls.append(("get_state", s.value))
        return 0

    def oxg_system_set_integrator(self, s, dt, kT, g, gr, seed, mask, bonded):
        self.systems[s.value]["integ"] = (dt, kT, g, gr, seed)
        self.calls.append(("set_integrator", s.value, kT))
        return 0

    def oxg_system_set_timestep(self, s, step):
        self.systems[s.value]["timestep"] = step
        self.calls.append(("set_timestep", s.value, step))
        return 0

    def oxg_system_run(self, s, n):
        sy = self.systems[s.value]
        sy["state"][1][:, 0] += np.float32(1e-4) * n  # the low parts move
        sy["state"][3][:, 0] += 1.0  # velocities change
        sy["timestep"] += n
        self.calls.append(("run", s.value, n))
        return 0

    def oxg_system_set_surrogate(self, s, mlp, flags, every, mod, tol):
        self.calls.append(("set_surrogate", s.value, mlp, flags))
        return 0

    def __getattr__(self, name):  # parameter setters, buffer, stream
        if not name.startswith("oxg_"):
            raise AttributeError(name)

        def ok(*a):
            return 0
        return ok


@pytest.fixture
def fake(monkeypatch):
    import gc

    from oxdna import _abi
    lib = _FakeLib()
    monkeypatch.setattr(_abi, "_lib", lib)
    yield lib
    # simulations and their forces reference each other: collect them while the
    # stand-in is still installed, so their handles never reach the real library
    gc.collect()


def _sim(seed=7):
    from oxdna import io, runtime
    from oxdna.model import dna1, dna2
    forces, _ = dna2.forces()
    sim = runtime.Simulation(device=runtime.device.GPU(), seed=seed)
    sim.create_state_from_snapshot(io.system_snapshot(io.duplex_system(1, 6, 20.0, seed=2)))
    lang = runtime.md.methods.Langevin(filter=runtime.filter.All(), kT=dna1.kT_from_temperature(300))
    sim.operations.integrator = runtime.md.Integrator(dt=0.003, integrate_rotational_dof=True,
                                                      forces=forces, methods=[lang])
    return sim, forces, lang


def _kinds(fake, start=0):
    return [c[0] for c in fake.calls[start:]]


def test_kT_change_is_passed_on_without_rebuilding(fake):
    sim, forces, lang = _sim()
    sim.run(10)
    assert _kinds(fake).count("system_create") == 1
    n0 = len(fake.calls)
    sim.run(5)  # nothing changed: no sync traffic
    assert _kinds(fake, n0) == ["run"]
    n1 = len(fake.calls)
    lang.kT = 0.05
    sim.run(5)
    assert _kinds(fake, n1) == ["set_integrator", "run"] and fake.calls[n1][2] == 0.05
    assert sim.timestep == 20


def test_parameter_change_rebuilds_from_the_pulled_state(fake):
    sim, forces, lang = _sim()
    sim.run(10)
    h0 = [c for c in fake.calls if c[0] == "system_create"][-1][1]
    moved = [a.copy() for a in fake.systems[h0]["state"]]
    n0 = len(fake.calls)
    hb = forces[2]
    hb.params[("A", "T")] = dict(hb.params[("A", "T")], eps=0.9)
    sim.run(5)
    kinds = _kinds(fake, n0)
    assert kinds[:2] == ["get_state", "system_destroy"]
    assert "create" in kinds and "system_create" in kinds
    h1 = [c for c in fake.calls if c[0] == "system_create"][-1][1]
    assert h1 != h0
    # the new system starts from the moved state: positions (high + low parts) exact
    # through FP64, orientations, velocities and angular momenta bit for bit; and it
    # continues the timestep
    pushed = fake.systems[h1]["pushed"]
    def x(st):
        return st[0][:, :3].astype(np.float64) + st[1][:, :3]
    assert np.array_equal(x(pushed), x(moved))
    for k in (2, 3, 4):
        assert np.array_equal(pushed[k][:, :3], moved[k][:, :3]), k
    assert np.array_equal(pushed[2], moved[2])
    assert ("set_timestep", h1, 10) in fake.calls
    assert kinds.index("set_timestep") < kinds.index("run")
    assert sim.timestep == 15


def test_checkpoint_resume_sets_the_timestep(fake, tmp_path):
    from oxdna import runtime
    sim, forces, lang = _sim()
    sim.run(30)
    snap = sim.state.get_snapshot()
    assert snap.configuration.step == 30
    runtime.write_snapshot(snap, tmp_path / "ck.npz")
    sim2, _, _ = _sim()
    sim2._snap = None
    sim2.create_state_from_snapshot(runtime.read_snapshot(tmp_path / "ck.npz"))
    n0 = len(fake.calls)
    sim2.run(1)
    h = [c for c in fake.calls[n0:] if c[0] == "system_create"][0][1]
    assert ("set_timestep", h, 30) in fake.calls[n0:]
    assert sim2.timestep == 31
    # a fresh simulation (timestep 0) makes no timestep call
    sim3, _, _ = _sim()
    n1 = len(fake.calls)
    sim3.run(1)
    assert "set_timestep" not in _kinds(fake, n1)


def test_integrator_swap_keeps_the_state(fake):
    from oxdna import runtime
    sim, forces, lang = _sim()
    sim.run(10)
    h0 = [c for c in fake.calls if c[0] == "system_create"][-1][1]
    moved = [a.copy() for a in fake.systems[h0]["state"]]
    lang2 = runtime.md.methods.Langevin(filter=runtime.filter.All(), kT=0.11)
    sim.operations.integrator = runtime.md.Integrator(dt=0.002, integrate_rotational_dof=True,
                                                      forces=forces, methods=[lang2])
    sim.run(1)
    h1 = [c for c in fake.calls if c[0] == "system_create"][-1][1]
    assert h1 != h0
    st = fake.systems[h1]["pushed"]
    assert np.array_equal(st[0][:, :3].astype(np.float64) + st[1][:, :3],
                          moved[0][:, :3].astype(np.float64) + moved[1][:, :3])
    assert np.array_equal(st[2], moved[2])
    assert fake.systems[h1]["integ"][0] == 0.002 and fake.systems[h1]["integ"][1] == 0.11


def test_surrogate_is_reapplied_after_a_rebuild(fake):
    import types
    sim, forces, lang = _sim()
    net = types.SimpleNamespace(handle=C.c_void_p(4242))
    sim.set_surrogate(net, run=True, compute=False)
    h0 = [c for c in fake.calls if c[0] == "system_create"][-1][1]
    assert ("set_surrogate", h0) == fake.calls[-1][:2]
    forces[1].params[("A", "A")] = dict(forces[1].params[("A", "A")])  # a parameter write
    sim.run(1)
    h1 = [c for c in fake.calls if c[0] == "system_create"][-1][1]
    assert h1 != h0
    assert [c for c in fake.calls if c[0] == "set_surrogate" and c[1] == h1]
    sim.set_surrogate(None)
    n0 = len(fake.calls)
    forces[1].params[("A", "A")] = dict(forces[1].params[("A", "A")])
    sim.run(1)
    assert "set_surrogate" not in _kinds(fake, n0)  # switched off: not reapplied


def test_state_arrays_are_checked_before_the_engine_sees_them(fake):
    """The host state arrays go to the engine as raw addresses of 16 * N bytes each: an
    array of another dtype, shape or layout is a ValueError, raised before any call."""
    sim, forces, lang = _sim()
    sim.run(1)
    n = sim.state.get_snapshot().particles.N
    good = [np.zeros((n, 4), np.float32) for _ in range(5)]
    sim.pull_state_arrays(*good)
    sim.push_state_arrays(*good)
    sim.run_state_arrays(1, *good)
    bad_cases = [np.zeros((n, 4), np.float64), np.zeros((n, 3), np.float32),
                 np.zeros((n + 1, 4), np.float32), np.zeros((4, n), np.float32).T,
                 list(np.zeros((n, 4), np.float32))]
    for bad in bad_cases:
        n0 = len(fake.calls)
        for call in (sim.push_state_arrays, sim.pull_state_arrays,
                     lambda *a: sim.run_state_arrays(1, *a)):
            with pytest.raises(ValueError):
                call(bad, *good[1:])
        assert len(fake.calls) == n0


def test_repeated_state_arrays_skip_the_checks_but_not_other_arrays(fake):
    """Calls with the same five arrays as the last call take the kept addresses without
    checking the arrays again; any other array is checked (and its address taken), and
    numpy refuses to resize an array whose address is kept."""
    sim, forces, lang = _sim()
    sim.run(1)
    n = sim.state.get_snapshot().particles.N
    good = [np.zeros((n, 4), np.float32) for _ in range(5)]
    first = sim._host_state_ptrs(good)
    again = sim._host_state_ptrs(good)
    assert again == first == [a.ctypes.data for a in good]
    sim.run_state_arrays(1, *good)
    with pytest.raises(ValueError):
        good[0].resize((n + 1, 4))
    other = np.zeros((n, 4), np.float32)
    assert sim._host_state_ptrs([other] + good[1:]) == [other.ctypes.data] + first[1:]
    with pytest.raises(ValueError):
        sim._host_state_ptrs([np.zeros((n, 3), np.float32)] + good[1:])
    assert sim._host_state_ptrs(good) == first
