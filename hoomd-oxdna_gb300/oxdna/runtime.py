"""Minimal simulation runtime with HOOMD-blue's Python surface.

The reference plugin runs inside HOOMD-blue; this package stands that runtime in
with the subset the reference's model files, tests and benchmark use
(``hoomd.Simulation``, ``Snapshot``, ``md.Integrator``, ``md.methods.Langevin``,
``md.nlist.Cell``, ``filter.All``, ``device.GPU``). Everything it runs goes through
the native library: the state lives on the GPU, and a run() call is one launch of
the persistent step kernel (neighbour list, every attached force, Langevin +
NO_SQUISH for each step).
"""

import ctypes as C
import types as _types

import numpy as np

from . import _abi
from . import forces as _forces_mod
from .forces import OxDNABonded, _PairForce

_F32 = np.dtype(np.float32)  # native float32 (a singleton: compared by identity)


# --------------------------------------------------------------------- snapshot
class _Particles:
    def __init__(self):
        self._n = 0
        self.types = []
        self._alloc(0)

    def _alloc(self, n):
        self.position = np.zeros((n, 3))
        self.typeid = np.zeros(n, dtype=np.int64)
        self.mass = np.ones(n)
        self.moment_inertia = np.ones((n, 3))
        self.orientation = np.tile([1.0, 0.0, 0.0, 0.0], (n, 1))
        self.charge = np.zeros(n)
        self.velocity = np.zeros((n, 3))
        self.angmom = np.zeros((n, 4))
        self.image = np.zeros((n, 3), dtype=np.int64)

    @property
    def N(self):
        return self._n

    @N.setter
    def N(self, n):
        self._n = int(n)
        self._alloc(self._n)


class _Bonds:
    def __init__(self):
        self._n = 0
        self.types = []
        self.group = np.zeros((0, 2), dtype=np.int64)
        self.typeid = np.zeros(0, dtype=np.int64)

    @property
    def N(self):
        return self._n

    @N.setter
    def N(self, n):
        self._n = int(n)
        self.group = np.zeros((self._n, 2), dtype=np.int64)
        self.typeid = np.zeros(self._n, dtype=np.int64)


class _Configuration:
    def __init__(self):
        self.box = [1.0, 1.0, 1.0, 0.0, 0.0, 0.0]
        self.step = 0  # the simulation timestep the snapshot was taken at


class _Communicator:
    rank = 0
    num_ranks = 1


class Snapshot:
    """System snapshot (particles, bonds, box) on the host."""

    def __init__(self):
        self.particles = _Particles()
        self.bonds = _Bonds()
        self.configuration = _Configuration()
        self.communicator = _Communicator()


_PARTICLE_FIELDS = ("position", "typeid", "mass", "moment_inertia", "orientation", "charge",
                    "velocity", "angmom", "image")


def write_snapshot(snap, path):
    """Save a snapshot as a .npz file (numpy appends the suffix if missing): every
    particle, bond and box field and the timestep, bit for bit. With
    ``sim.state.get_snapshot()`` this is a checkpoint; :func:`read_snapshot` and
    ``create_state_from_snapshot`` resume from it, the bath noise continuing from the
    saved timestep."""
    p, b, c = snap.particles, snap.bonds, snap.configuration
    arrays = {k: np.asarray(getattr(p, k)) for k in _PARTICLE_FIELDS}
    np.savez(path, N=np.int64(p.N), types=np.array(list(p.types), dtype=str),
             bond_N=np.int64(b.N), bond_types=np.array(list(b.types), dtype=str),
             bond_group=np.asarray(b.group), bond_typeid=np.asarray(b.typeid),
             box=np.asarray(c.box, dtype=np.float64),
             step=np.uint64(int(getattr(c, "step", 0) or 0)), **arrays)


def read_snapshot(path):
    """The snapshot written by :func:`write_snapshot`."""
    with np.load(path) as z:
        snap = Snapshot()
        p = snap.particles
        p.N = int(z["N"])
        p.types = [str(t) for t in z["types"]]
        for k in _PARTICLE_FIELDS:
            getattr(p, k)[:] = z[k]
        snap.bonds.N = int(z["bond_N"])
        snap.bonds.types = [str(t) for t in z["bond_types"]]
        if snap.bonds.N:
            snap.bonds.group[:] = z["bond_group"]
            snap.bonds.typeid[:] = z["bond_typeid"]
        snap.configuration.box = [float(x) for x in z["box"]]
        snap.configuration.step = int(z["step"])
    return snap


# --------------------------------------------------------------------- devices etc.
class _GPU:
    def __init__(self, gpu_ids=None):
        self.gpu_ids = gpu_ids or [0]


class _CPU:
    def __init__(self, *a, **k):
        raise RuntimeError("this framework runs the force path on the GPU only (no CPU fallback)")


device = _types.SimpleNamespace(GPU=_GPU, CPU=_CPU)


class _All:
    pass


filter = _types.SimpleNamespace(All=_All)


class _Tracked:
    """Attribute changes count as changes of the simulation description."""

    def __setattr__(self, name, value):
        object.__setattr__(self, name, value)
        _forces_mod._changed()


class _ChangeList(list):
    """A list whose mutations count as changes (an integrator's forces and methods)."""


def _counting(name):
    def method(self, *a, **k):
        out = getattr(list, name)(self, *a, **k)
        _forces_mod._changed()
        return out
    method.__name__ = name
    return method


for _name in ("append", "extend", "insert", "remove", "pop", "clear", "sort", "reverse",
              "__setitem__", "__delitem__", "__iadd__"):
    setattr(_ChangeList, _name, _counting(_name))


class _Cell(_Tracked):
    """Cell neighbour list: radius max(r_cut) + buffer, bond exclusions."""

    def __init__(self, buffer=0.4, exclusions=("bond",)):
        self.buffer = float(buffer)
        self.exclusions = tuple(exclusions)
        if "bond" not in self.exclusions:
            raise ValueError("oxDNA forces require exclusions=('bond',)")


class _Langevin(_Tracked):
    def __init__(self, filter=None, kT=1.0, default_gamma=1.0, default_gamma_r=(1.0, 1.0, 1.0)):
        self.filter = filter
        self.kT = float(kT)
        self.default_gamma = float(default_gamma)
        self.default_gamma_r = default_gamma_r

    def __setattr__(self, name, value):
        # every assignment, not only the constructor's, is normalised and checked: the
        # engine takes one rotational drag coefficient (isotropic gamma_r)
        if name == "default_gamma_r":
            g = tuple(float(x) for x in value) if hasattr(value, "__len__") else (float(value),) * 3
            if len(g) != 3:
                raise ValueError("default_gamma_r needs 3 components (or one scalar)")
            if len(set(g)) != 1:
                raise ValueError("anisotropic gamma_r is not supported")
            value = g
        elif name in ("kT", "default_gamma"):
            value = float(value)
        super().__setattr__(name, value)


class _Integrator(_Tracked):
    def __init__(self, dt, integrate_rotational_dof=False, forces=(), methods=()):
        self.dt = float(dt)
        self.integrate_rotational_dof = bool(integrate_rotational_dof)
        self.forces = forces
        self.methods = methods

    def __setattr__(self, name, value):
        if name in ("forces", "methods"):
            value = _ChangeList(value)
        super().__setattr__(name, value)


md = _types.SimpleNamespace(
    Integrator=_Integrator,
    methods=_types.SimpleNamespace(Langevin=_Langevin),
    nlist=_types.SimpleNamespace(Cell=_Cell),
)


class _Operations:
    def __init__(self, sim):
        self._sim = sim
        self._integrator = None

    @property
    def integrator(self):
        return self._integrator

    @integrator.setter
    def integrator(self, integ):
        self._integrator = integ
        self._sim._detach()


class _State:
    def __init__(self, sim):
        self._sim = sim

    @property
    def N_particles(self):
        return self._sim._snap.particles.N

    def get_snapshot(self):
        return self._sim._pull_snapshot()


# --------------------------------------------------------------------- simulation
def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _check_unit_inertia(moment_inertia):
    """The engine integrates every particle with the unit moment of inertia the oxDNA
    builders set (reference io.py: moment_inertia = 1); any other value is refused
    rather than ignored."""
    mi = np.asarray(moment_inertia, dtype=np.float64)
    if mi.size and not np.all(mi == 1.0):
        raise ValueError("moment_inertia other than (1, 1, 1) is not supported: the engine "
                         "integrates the rotations with unit moments of inertia")


class Simulation:
    """Owns one native system (state resident on the GPU) and its forces."""

    def __init__(self, device=None, seed=0):
        self.device = device or _GPU()
        self.seed = int(seed)
        self.operations = _Operations(self)
        self.state = None
        self.timestep = 0
        self._snap = None
        self._ctx = None
        self._sys = None
        self._attached = False
        self._cache = {}
        self._stream = None
        self._fkey = self._ikey = None
        self._seen = -1
        self._surrogate_args = None

    def set_stream(self, handle):
        """Run every later engine call on this CUDA stream (a cudaStream_t handle,
        e.g. ``torch.cuda.Stream().cuda_stream``)."""
        self._stream = handle
        if self._sys:
            _abi.check(_abi.lib().oxg_system_set_stream(self._sys, C.c_void_p(handle)),
                       "oxg_system_set_stream")

    # -- state ---------------------------------------------------------------
    def create_state_from_snapshot(self, snap):
        if self._snap is not None:
            raise RuntimeError("state already created")
        self._snap = snap
        self.state = _State(self)
        # HOOMD restores the timestep from the snapshot; the bath noise of step t depends
        # only on (seed, t, particle), so a restored run continues the noise stream
        self.timestep = int(getattr(snap.configuration, "step", 0) or 0)

    def _types(self):
        return list(self._snap.particles.types)

    def _detach(self):
        """Drop the native context and system; the device state comes back into the
        snapshot first, so the next attach continues from it (as HOOMD keeps the state
        when the integrator or the forces change)."""
        if self._attached and self._sys:
            self._snap = self._pull_snapshot()
        self._free()
        self._attached = False
        self._cache = {}

    def _forces_key(self):
        """What the native context was built from: the integrator, its methods, and per
        force its identity, parameter versions, cutoffs and list buffer."""
        integ = self.operations.integrator
        if integ is None:
            return None
        fk = tuple((id(f), getattr(f.params, "_version", 0),
                    getattr(getattr(f, "r_cut", None), "_version", 0),
                    getattr(f, "default_r_cut", None),
                    getattr(getattr(f, "nlist", None), "buffer", None)) for f in integ.forces)
        return (id(integ), fk, tuple(id(m) for m in integ.methods),
                integ.integrate_rotational_dof)

    def _integ_key(self):
        integ = self.operations.integrator
        lang = self._langevin
        if lang is None:
            return (integ.dt,)
        return (integ.dt, lang.kT, lang.default_gamma, tuple(lang.default_gamma_r))

    def _send_integrator(self):
        integ = self.operations.integrator
        if self._langevin is not None:
            _abi.check(_abi.lib().oxg_system_set_integrator(
                self._sys, integ.dt, self._langevin.kT, self._langevin.default_gamma,
                self._langevin.default_gamma_r[0], self.seed, self._mask,
                1 if self._bonded else 0), "oxg_system_set_integrator")
        self._ikey = self._integ_key()

    def _sync(self):
        """Attach, or bring the attached engine up to date with the Python objects: a
        changed force set, force parameters or cutoffs rebuild the native context and
        system with the state carried over; a changed dt, kT or gamma is passed on."""
        if self._attached and _forces_mod._changes[0] != self._seen:
            self._seen = _forces_mod._changes[0]
            if self._forces_key() != self._fkey:
                self._detach()
            elif self._integ_key() != self._ikey:
                self._send_integrator()
                self._cache = {}
        self._attach()

    def _free(self):
        L = _abi.lib()
        if self._sys:
            L.oxg_system_destroy(self._sys)
            self._sys = None
        if self._ctx:
            L.oxg_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self._free()
        except Exception:
            pass

    # -- attach: parameters -> context, snapshot -> device state ----------------
    def _attach(self):
        if self._attached:
            return
        self._make_context()
        self._make_system()

    def _make_context(self):
        """Native parameter context from the attached forces (sets _ctx, _mask,
        _bonded, _nlist, _langevin)."""
        integ = self.operations.integrator
        if integ is None:
            raise RuntimeError("no integrator set")
        L = _abi.lib()
        if self._ctx:
            L.oxg_destroy(self._ctx)
            self._ctx = None
        snap = self._snap
        types = self._types()
        nt = len(types)
        bond_types = list(snap.bonds.types) or ["backbone"]
        ctx = C.c_void_p()
        _abi.check(L.oxg_create(C.byref(ctx), nt, len(bond_types)), "oxg_create")
        self._ctx = ctx
        self._pair_forces = {}
        self._bonded = None
        self._nlist = None
        setters = {
            _abi.EXCVOL: L.oxg_set_excvol_params, _abi.HBOND: L.oxg_set_hbond_params,
            _abi.CROSS: L.oxg_set_cross_params, _abi.HBONDCROSS: L.oxg_set_hbondcross_params,
            _abi.COAX: L.oxg_set_coax_params, _abi.DEBYE: L.oxg_set_debye_params,
        }
        for f in integ.forces:
            f._simulation = self
            if isinstance(f, OxDNABonded):
                if self._bonded is not None:
                    raise RuntimeError("only one OxDNABonded force can be attached")
                self._bonded = f
                for bt, name in enumerate(bond_types):
                    if name not in f.params:
                        raise KeyError(f"OxDNABonded has no parameters for bond type {name!r}")
                    p = _abi.bonded_from_dict(f.params[name])
                    _abi.check(L.oxg_set_bonded_params(ctx, bt, C.byref(p)), "oxg_set_bonded_params")
            elif isinstance(f, _PairForce):
                t = f._term
                if t in self._pair_forces:
                    raise RuntimeError(f"two forces of kind {_abi.TERM_NAMES[t]} attached")
                if self._nlist is None:
                    self._nlist = f.nlist
                self._pair_forces[t] = f
                conv = _abi.FROM_DICT[t]
                for a in range(nt):
                    for b in range(a, nt):
                        key = (types[a], types[b])
                        if key not in f.params:
                            raise KeyError(f"{type(f).__name__} has no parameters for {key}")
                        p = conv(f.params[key])
                        _abi.check(setters[t](ctx, a, b, C.byref(p), f.rcut_for(*key)),
                                   "set params")
            else:
                raise TypeError(f"unsupported force {type(f).__name__}")
        self._mask = 0
        for t in self._pair_forces:
            self._mask |= 1 << t
        lang = [m for m in integ.methods if isinstance(m, _Langevin)]
        if len(integ.methods) != len(lang) or len(lang) > 1:
            raise RuntimeError("only a single Langevin method is supported")
        self._langevin = lang[0] if lang else None
        if self._langevin is not None and not integ.integrate_rotational_dof:
            raise RuntimeError("oxDNA dynamics need integrate_rotational_dof=True")

    def _make_system(self):
        L = _abi.lib()
        snap = self._snap
        integ = self.operations.integrator
        ctx = self._ctx
        n = snap.particles.N
        box = (C.c_float * 3)(*[float(x) for x in snap.configuration.box[:3]])
        bonds = np.zeros((max(1, snap.bonds.N), 3), dtype=np.int32)
        if snap.bonds.N:
            bonds[:snap.bonds.N, 0:2] = np.asarray(snap.bonds.group, dtype=np.int32)
            bonds[:snap.bonds.N, 2] = np.asarray(snap.bonds.typeid, dtype=np.int32)
        sys_ = C.c_void_p()
        _abi.check(L.oxg_system_create(C.byref(sys_), ctx, n, box, int(snap.bonds.N),
                                       bonds.ctypes.data_as(C.POINTER(C.c_int32))),
                   "oxg_system_create")
        self._sys = sys_
        if self._stream is not None:
            _abi.check(L.oxg_system_set_stream(sys_, C.c_void_p(self._stream)), "set stream")
        if self._nlist is not None:
            _abi.check(L.oxg_system_set_nlist_buffer(sys_, self._nlist.buffer), "set buffer")
        self._push_state()
        self._send_integrator()
        if self.timestep:
            _abi.check(L.oxg_system_set_timestep(sys_, int(self.timestep)), "oxg_system_set_timestep")
        self._fkey = self._forces_key()
        self._seen = _forces_mod._changes[0]
        self._attached = True
        if getattr(self, "_surrogate_args", None) is not None:
            self._apply_surrogate(*self._surrogate_args)
        if getattr(self, "_session_idle_us", 0):
            _abi.check(L.oxg_system_set_host_session(sys_, self._session_idle_us), "oxg_system_set_host_session")

    def _host_state_ptrs(self, arrays, allow_none=False):
        """Addresses of the five host state arrays, each checked to be a C-contiguous
        float32 (N, 4) array (the engine reads and writes 16 * N bytes at each). Reading
        an array's address through numpy costs ~2 µs, a sizeable part of a one-step call,
        so the addresses of the last arrays seen are kept (with a reference to each
        array, so that an address is never taken for another array's). A call with the
        same five arrays as the last one, for the same N, takes their addresses without
        checking them again (~0.2 against ~2.4 µs): the references kept make numpy refuse
        to resize them, so each still spans the 16 * N bytes it was checked to span."""
        n = self._snap.particles.N
        last = self.__dict__.get("_last_state")
        if last is not None and last[0] == n:
            p = last[1]
            if (arrays[0] is p[0] and arrays[1] is p[1] and arrays[2] is p[2] and arrays[3] is p[3]
                    and arrays[4] is p[4]):
                return last[2]
        cache = self.__dict__.setdefault("_addr_cache", {})
        out = []
        for a in arrays:
            if a is None and allow_none:
                out.append(None)
                continue
            if (not isinstance(a, np.ndarray) or a.dtype is not _F32 or a.shape != (n, 4)
                    or not a.flags.c_contiguous):
                raise ValueError("state arrays must be C-contiguous float32 arrays of shape "
                                 f"({n}, 4)")
            hit = cache.get(id(a))
            if hit is None or hit[0] is not a:
                if len(cache) >= 32:
                    cache.clear()
                hit = (a, a.__array_interface__["data"][0])
                cache[id(a)] = hit
            out.append(hit[1])
        if len(arrays) == 5 and all(a is not None for a in arrays):
            self.__dict__["_last_state"] = (n, tuple(arrays), out)
        return out

    def push_state_arrays(self, pos_type, pos_lo, quat, vel, angmom):
        """Copy host float32 (N, 4) arrays (pinned or not) into the device state."""
        ptrs = self._host_state_ptrs((pos_type, pos_lo, quat, vel, angmom), allow_none=True)
        _abi.check(_abi.lib().oxg_system_set_state(self._sys, *ptrs, None), "oxg_system_set_state")

    def set_host_session(self, idle_us):
        """Host session for loops of run_state_arrays calls (page-locked arrays, at most
        2000 steps a call): with idle_us > 0 the run kernel stays resident between calls,
        occupying every SM, and serves the next call through page-locked host memory
        instead of a new launch; it leaves after idle_us microseconds without a call, or
        at any other call on this simulation. 0 turns the session off (the default)."""
        self._sync()
        _abi.check(_abi.lib().oxg_system_set_host_session(self._sys, int(idle_us)),
                   "oxg_system_set_host_session")
        self._session_idle_us = int(idle_us)

    def run_state_arrays(self, steps, pos_type, pos_lo, quat, vel, angmom):
        """push_state_arrays + run(steps) + pull_state_arrays in one call: the state is
        read from the host float32 (N, 4) arrays and the final state written back into
        them. With page-locked arrays (torch ``pin_memory()``) the run kernel itself reads
        them at its start and writes them in its last step, over the host link: one
        launch and one synchronisation per call."""
        self._sync()
        self._cache = {}
        steps = int(steps)
        if steps < 1 or self._langevin is None:
            raise ValueError("run_state_arrays needs steps >= 1 and a Langevin method")
        ptrs = self._host_state_ptrs((pos_type, pos_lo, quat, vel, angmom))
        rc = _abi.lib().oxg_system_run_host(self._sys, steps, *ptrs)
        if rc:
            _abi.check(rc, "oxg_system_run_host")
        self.timestep += steps

    def pull_state_arrays(self, pos_type, pos_lo, quat, vel, angmom):
        """Copy the device state into host float32 (N, 4) arrays."""
        ptrs = self._host_state_ptrs((pos_type, pos_lo, quat, vel, angmom), allow_none=True)
        _abi.check(_abi.lib().oxg_system_get_state(self._sys, *ptrs), "oxg_system_get_state")

    def _push_state(self):
        L = _abi.lib()
        pos, lo, q, vel, am, ch = self._state_arrays()
        vp = C.c_void_p
        _abi.check(L.oxg_system_set_state(self._sys, vp(pos.ctypes.data), vp(lo.ctypes.data),
                                          vp(q.ctypes.data), vp(vel.ctypes.data),
                                          vp(am.ctypes.data), vp(ch.ctypes.data)),
                   "oxg_system_set_state")

    def _state_arrays(self):
        """The snapshot as engine arrays: pos_type, pos_lo, quat, vel (mass in w),
        angmom (float32, N x 4) and charge (N)."""
        p = self._snap.particles
        n = p.N
        _check_unit_inertia(p.moment_inertia)
        pos = np.zeros((n, 4), np.float32)
        x = np.asarray(p.position, np.float64)
        pos[:, :3] = x
        pos[:, 3] = np.asarray(p.typeid, np.int32).view(np.float32)
        lo = np.zeros((n, 4), np.float32)
        lo[:, :3] = x - pos[:, :3].astype(np.float64)
        vel = np.zeros((n, 4), np.float32)
        vel[:, :3] = p.velocity
        vel[:, 3] = p.mass
        q = _f32(p.orientation)
        am = _f32(p.angmom)
        ch = _f32(p.charge)
        return pos, lo, q, vel, am, ch

    def _pull_snapshot(self):
        import copy
        snap = copy.deepcopy(self._snap)
        snap.configuration.step = int(self.timestep)
        if not self._attached:
            return snap
        L = _abi.lib()
        n = snap.particles.N
        pos = np.zeros((n, 4), np.float32)
        lo = np.zeros((n, 4), np.float32)
        q = np.zeros((n, 4), np.float32)
        vel = np.zeros((n, 4), np.float32)
        am = np.zeros((n, 4), np.float32)
        vp = C.c_void_p
        _abi.check(L.oxg_system_get_state(self._sys, vp(pos.ctypes.data), vp(lo.ctypes.data),
                                          vp(q.ctypes.data), vp(vel.ctypes.data),
                                          vp(am.ctypes.data)), "get_state")
        snap.particles.position[:] = pos[:, :3].astype(np.float64) + lo[:, :3]
        snap.particles.orientation[:] = q
        snap.particles.velocity[:] = vel[:, :3]
        snap.particles.angmom[:] = am
        return snap

    # -- running -------------------------------------------------------------
    def run(self, steps):
        self._sync()
        self._cache = {}
        L = _abi.lib()
        steps = int(steps)
        if steps > 0 and self._langevin is not None:
            _abi.check(L.oxg_system_run(self._sys, steps), "oxg_system_run")
        self.timestep += steps

    # -- read-outs -----------------------------------------------------------
    def _energies(self):
        self._sync()  # a parameter changed since the last run is in effect for read-outs too
        if "energies" not in self._cache:
            L = _abi.lib()
            pe = (C.c_double * 6)()
            be = (C.c_double * 3)()
            _abi.check(L.oxg_system_compute(self._sys, self._mask, 1 if self._bonded else 0,
                                            None, None, pe, be), "oxg_system_compute")
            self._cache["energies"] = (list(pe), list(be))
        return self._cache["energies"]

    def _force_energy(self, f):
        pe, be = self._energies()
        if f is self._bonded:
            return float(sum(be))
        return float(pe[f._term])

    def _bonded_energy(self, k):
        return float(self._energies()[1][k])

    def _force_arrays(self, f):
        self._sync()
        key = ("arrays", id(f))
        if key not in self._cache:
            L = _abi.lib()
            n = self._snap.particles.N
            force = np.zeros((n, 4), np.float32)
            torque = np.zeros((n, 4), np.float32)
            mask = 0 if f is self._bonded else (1 << f._term)
            _abi.check(L.oxg_system_compute(self._sys, mask, 1 if f is self._bonded else 0,
                                            C.c_void_p(force.ctypes.data),
                                            C.c_void_p(torque.ctypes.data), None, None),
                       "oxg_system_compute")
            self._cache[key] = (force[:, :3].astype(np.float64), torque[:, :3].astype(np.float64),
                                force[:, 3].astype(np.float64))
        return self._cache[key]

    # -- learned surrogate (extension; see oxdna.surrogate) ----------------------
    def set_surrogate(self, network, run=True, compute=False, audit_every=100,
                      audit_fraction=0.01, tol=1e-4):
        """Evaluate the fused HB + cross-stacking term (forces(fused=True)) with a
        trained surrogate network in MD steps (run) and / or in energy and force
        read-outs (compute). Every audit_every steps about audit_fraction of the pairs is
        also evaluated by the plain evaluator; when the audited sample shows the
        relative error of the term's energy above tol (default 1e-4, the per-term
        energy budget) by more than two standard errors, the surrogate is switched off
        for the rest of the simulation. network=None restores the plain evaluator."""
        self._sync()
        self._apply_surrogate(network, run, compute, audit_every, audit_fraction, tol)

    def _apply_surrogate(self, network, run, compute, audit_every, audit_fraction, tol):
        flags = (_abi.SURROGATE_RUN if run else 0) | (_abi.SURROGATE_COMPUTE if compute else 0)
        mod = max(1, int(round(1.0 / audit_fraction))) if audit_fraction > 0 else 1
        every = int(audit_every) if audit_fraction > 0 else 0
        _abi.check(_abi.lib().oxg_system_set_surrogate(
            self._sys, network.handle if network is not None else None,
            flags if network is not None else 0, every, mod, float(tol)), "oxg_system_set_surrogate")
        self._surrogate = network
        # kept so that a rebuilt native system (after a parameter change) gets it again
        self._surrogate_args = ((network, run, compute, audit_every, audit_fraction, tol)
                                if network is not None else None)
        self._cache = {}

    def surrogate_stats(self):
        """Audit statistics: disabled (the kill switch tripped), audited pairs, audits
        that tripped it, rms / max pair energy and force errors against the plain
        evaluator, and the sampled relative error of the term's energy (rel_energy_error)
        with its standard error (rel_energy_error_se)."""
        out = (C.c_double * 11)()
        _abi.check(_abi.lib().oxg_system_surrogate_stats(self._sys, out, 11), "oxg_system_surrogate_stats")
        keys = ("disabled", "n_audited", "n_over", "rms_de", "rms_e", "rms_df", "rms_f",
                "max_abs_de", "max_abs_df", "rel_energy_error", "rel_energy_error_se")
        return dict(zip(keys, list(out)))

    def run_kernel_timing(self, reset=False):
        """(ms, launches, steps) of the persistent run kernel since the last reset, timed
        with CUDA events around each launch."""
        out = (C.c_double * 3)()
        _abi.check(_abi.lib().oxg_system_run_timing(self._sys, out, 3, 1 if reset else 0),
                   "oxg_system_run_timing")
        return out[0], int(out[1]), int(out[2])

    def native_stats(self):
        L = _abi.lib()
        out = (C.c_int64 * 7)()
        _abi.check(L.oxg_system_stats(self._sys, out, 7), "oxg_system_stats")
        return dict(steps=out[0], nlist_builds=out[1], pairs_short=out[2], pairs_long=out[3],
                    session_served=out[5], run_launches=out[6])


def device_peaks(stream=None):
    """(FP32 GFLOP/s, special-function Gop/s) of the current device, measured by the
    library's microbenchmark kernels (oxg_device_peaks)."""
    out = (C.c_double * 2)()
    _abi.check(_abi.lib().oxg_device_peaks(out, 2, C.c_void_p(stream or 0)), "oxg_device_peaks")
    return out[0], out[1]
