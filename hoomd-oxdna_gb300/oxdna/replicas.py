"""Replica bookkeeping shared by the batched engine and multi-GPU runs.

The force hot path does not shard: a single system is evaluated on one GPU. What
scales across GPUs is independent replicas (each GPU runs its own set, no data-path
collective), so multi-GPU runs only need a deterministic split of replica ids and a
max-over-ranks reduction of timings.
"""

import numpy as np


def shard(n_replicas, rank, world_size):
    """Replica ids owned by ``rank`` (contiguous, sizes differ by at most one)."""
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError("bad rank / world size")
    base, extra = divmod(int(n_replicas), int(world_size))
    start = rank * base + min(rank, extra)
    stop = start + base + (1 if rank < extra else 0)
    return np.arange(start, stop)


def max_over_ranks(value, dist=None):
    """Max of a float over the ranks of an initialised torch.distributed group."""
    if dist is None or not dist.is_available() or not dist.is_initialized():
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64)
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ReplicaBatch:
    """Independent small systems stepped together by the batched engine.

    ``simulations`` are configured :class:`oxdna.runtime.Simulation` objects (state
    created, integrator with the forces and one Langevin method set), one per replica.
    Each keeps its own parameters (e.g. ``dna2.forces(temperature=T_r)``), box and bath
    temperature; all must share dt, gamma, gamma_r and the set of force terms. Replica
    r integrates with Philox seed ``seed + r``: it reproduces
    ``Simulation(seed=seed + r)`` run alone. The reference has no batched mode (one
    HOOMD simulation per process); this is the GB300 way to run many small systems.
    """

    def __init__(self, simulations, seed=None):
        import ctypes as C
        from . import _abi
        self._sims = list(simulations)
        if not self._sims:
            raise ValueError("no replicas")
        self.seed = int(self._sims[0].seed if seed is None else seed)
        L = _abi.lib()
        ctxs, nps, boxes, nbs, bonds, kts = [], [], [], [], [], []
        integ0 = None
        for r, sim in enumerate(self._sims):
            sim._make_context()
            integ = sim.operations.integrator
            if sim._langevin is None:
                raise RuntimeError(f"replica {r} has no Langevin method")
            key = (integ.dt, sim._langevin.default_gamma, sim._langevin.default_gamma_r[0],
                   sim._mask, sim._bonded is not None)
            if integ0 is None:
                integ0 = key
            elif key != integ0:
                raise ValueError(f"replica {r} differs in dt, gamma or force terms")
            snap = sim._snap
            ctxs.append(sim._ctx.value)
            nps.append(int(snap.particles.N))
            boxes.extend(float(x) for x in snap.configuration.box[:3])
            nbs.append(int(snap.bonds.N))
            if snap.bonds.N:
                b = np.zeros((snap.bonds.N, 3), np.int32)
                b[:, 0:2] = np.asarray(snap.bonds.group, np.int32)
                b[:, 2] = np.asarray(snap.bonds.typeid, np.int32)
                bonds.append(b)
            kts.append(sim._langevin.kT)
        self.dt, self.gamma, self.gamma_r, self.mask, self.bonded = integ0
        self.n_particles = np.asarray(nps, np.int64)
        self.offsets = np.concatenate([[0], np.cumsum(self.n_particles)])
        self.N = int(self.offsets[-1])
        self.kT = np.asarray(kts, np.float64)
        R = len(self._sims)
        allb = np.concatenate(bonds) if bonds else np.zeros((1, 3), np.int32)
        self._bonds_host = np.ascontiguousarray(allb, np.int32)
        cp = (C.c_void_p * R)(*ctxs)
        h = C.c_void_p()
        _abi.check(L.oxg_batch_create(
            C.byref(h), R, cp, (C.c_int32 * R)(*nps), (C.c_float * (3 * R))(*boxes),
            (C.c_int32 * R)(*nbs), self._bonds_host.ctypes.data_as(C.POINTER(C.c_int32))),
            "oxg_batch_create")
        self._h = h
        arrs = [sim._state_arrays() for sim in self._sims]
        self.set_state(*[np.concatenate([a[k] for a in arrs]) for k in range(6)])
        kt = (C.c_double * R)(*self.kT)
        _abi.check(L.oxg_batch_set_integrator(h, self.dt, kt, self.gamma, self.gamma_r,
                                              self.seed, self.mask, 1 if self.bonded else 0),
                   "oxg_batch_set_integrator")
        self.timestep = 0

    @property
    def n_replicas(self):
        return len(self._sims)

    def _lib(self):
        from . import _abi
        return _abi, _abi.lib()

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                self._lib()[1].oxg_batch_destroy(self._h)
                self._h = None
        except Exception:
            pass

    def set_stream(self, handle):
        import ctypes as C
        abi, L = self._lib()
        abi.check(L.oxg_batch_set_stream(self._h, C.c_void_p(handle)), "oxg_batch_set_stream")

    def set_state(self, pos_type=None, pos_lo=None, quat=None, vel=None, angmom=None,
                  charge=None):
        """Host float32 arrays over all replicas back to back (None = unchanged)."""
        import ctypes as C
        abi, L = self._lib()

        def p(a, w):
            if a is None:
                return None
            a = np.ascontiguousarray(a, np.float32)
            if a.size != self.N * w:
                raise ValueError("state array of the wrong size")
            self._keep.append(a)
            return C.c_void_p(a.ctypes.data)
        self._keep = []
        abi.check(L.oxg_batch_set_state(self._h, p(pos_type, 4), p(pos_lo, 4), p(quat, 4),
                                        p(vel, 4), p(angmom, 4), p(charge, 1)),
                  "oxg_batch_set_state")
        self._keep = []

    def get_state(self):
        """(pos_type, pos_lo, quat, vel, angmom), float32 N x 4 each."""
        import ctypes as C
        abi, L = self._lib()
        out = [np.zeros((self.N, 4), np.float32) for _ in range(5)]
        abi.check(L.oxg_batch_get_state(self._h, *[C.c_void_p(a.ctypes.data) for a in out]),
                  "oxg_batch_get_state")
        return tuple(out)

    def positions(self, r):
        """Positions of replica r (float64, high + low parts)."""
        pos, lo = self.get_state()[:2]
        s = slice(int(self.offsets[r]), int(self.offsets[r + 1]))
        return pos[s, :3].astype(np.float64) + lo[s, :3]

    def set_tiling(self, tile_particles, threads):
        abi, L = self._lib()
        abi.check(L.oxg_batch_set_tiling(self._h, int(tile_particles), int(threads)),
                  "oxg_batch_set_tiling")

    def tune(self, trial_steps=100):
        """Time each admissible (tile particles, threads) shape and keep the fastest;
        returns (tile_particles, threads, ms for trial_steps). The state is unchanged."""
        import ctypes as C
        abi, L = self._lib()
        t, th, ms = C.c_int(), C.c_int(), C.c_double()
        abi.check(L.oxg_batch_tune(self._h, int(trial_steps), C.byref(t), C.byref(th),
                                   C.byref(ms)), "oxg_batch_tune")
        return t.value, th.value, ms.value

    def run(self, steps):
        abi, L = self._lib()
        abi.check(L.oxg_batch_run(self._h, int(steps)), "oxg_batch_run")
        self.timestep += int(steps)

    def compute(self, mask=None, bonded=None):
        """Forces (N x 4, energy/2 in w), torques (N x 4) and per-replica energies
        (R x 9: the six pair terms, then FENE, bonded excluded volume, stacking)."""
        import ctypes as C
        abi, L = self._lib()
        mask = self.mask if mask is None else int(mask)
        bonded = self.bonded if bonded is None else bool(bonded)
        f = np.zeros((self.N, 4), np.float32)
        t = np.zeros((self.N, 4), np.float32)
        e = np.zeros((self.n_replicas, 9), np.float64)
        abi.check(L.oxg_batch_compute(self._h, mask, 1 if bonded else 0,
                                      C.c_void_p(f.ctypes.data), C.c_void_p(t.ctypes.data),
                                      C.c_void_p(e.ctypes.data)), "oxg_batch_compute")
        return f, t, e


def replica_workload(n_replicas=512, bp_range=(12, 64), box_len=30.0, t_range=(290.0, 340.0),
                     seed=4, hairpin_fraction=0.0, hairpin_loop=8):
    """Independent replicas: replica r is one random-sequence B-form duplex of
    uniform-random length n in bp_range (inclusive) in its own periodic cube of side
    box_len, at a temperature uniform in t_range (K). With ``hairpin_fraction`` > 0 that
    fraction of the replicas (chosen at random) are instead single-strand hairpins of
    the same 2n nucleotides: a stem of n - hairpin_loop/2 base pairs closed by a loop
    of hairpin_loop nucleotides, started as an extended helix. The duplex draws do not
    depend on ``hairpin_fraction``, so the default reproduces the all-duplex workload.
    Returns a list of (system arrays as from ``io.duplex_system``, temperature)."""
    from . import io
    rng = np.random.Generator(np.random.PCG64(seed))
    lengths = rng.integers(bp_range[0], bp_range[1] + 1, size=n_replicas)
    temps = rng.uniform(t_range[0], t_range[1], size=n_replicas)
    seeds = rng.integers(1, 2 ** 31 - 1, size=n_replicas)
    hairpin = np.zeros(n_replicas, bool)
    if hairpin_fraction > 0.0:
        if hairpin_loop < 2 or hairpin_loop % 2 or 2 * bp_range[0] - hairpin_loop < 4:
            raise ValueError("hairpin_loop must be even, >= 2, and leave a stem of >= 2 bp")
        pick = np.random.Generator(np.random.PCG64(seed + 1))
        hairpin = pick.random(n_replicas) < hairpin_fraction
    out = []
    for n, t, s, h in zip(lengths, temps, seeds, hairpin):
        if h:
            stem = int(n) - hairpin_loop // 2
            out.append((io.hairpin_system(1, stem=stem, loop=hairpin_loop, box_len=box_len,
                                          seed=int(s)), float(t)))
        else:
            out.append((io.duplex_system(1, int(n), box_len, seed=int(s)), float(t)))
    return out


def replica_simulation(system, temperature, salt=0.5, dt=0.003, seed=1, fused=False):
    """A runtime.Simulation of one replica with oxDNA2 forces at its temperature."""
    from . import io, runtime
    from .model import dna1, dna2
    forces, _ = dna2.forces(temperature=temperature, salt=salt, fused=fused)
    sim = runtime.Simulation(device=runtime.device.GPU(), seed=seed)
    sim.create_state_from_snapshot(io.system_snapshot(system))
    kT = dna1.kT_from_temperature(temperature)
    sim.operations.integrator = runtime.md.Integrator(
        dt=dt, integrate_rotational_dof=True, forces=forces,
        methods=[runtime.md.methods.Langevin(filter=runtime.filter.All(), kT=kT)])
    sim._forces = forces
    return sim
