"""Benchmark: MD steps/s of the oxDNA2 force hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (``config.workload``): oxDNA2, plain FP32 forces (FENE and the energy
reductions FP64), 200 x 20-bp B-form duplexes = 8000 nt, periodic box 100 sigma,
296.15 K, 0.5 M salt, Langevin dt = 0.003 with rotational DOF, forces(fused=False),
seeded synthetic construction. One bench step = one MD timestep (neighbour-list
check/rebuild, every force, Langevin + NO_SQUISH), run by the persistent cooperative
run kernel (one launch per run() call of up to 2000 steps).

Multi-GPU (torchrun, one process per GPU): every rank runs its own independent
replica (the single-system path does not shard; replicas are the scaling axis), no
collective on the data path; ``value`` is the sum of the ranks' steps over the
max-over-ranks time.

``--impl reference`` times the reference algorithm's CPU implementation on the
host cores: the FP64 C restatement of the reference evaluators + HOOMD driver
semantics (the reference's HOOMD build is not available on this machine), OpenMP
over all host threads, on a bounded sample of the same workload.
"""

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "hoomd-oxdna_gb300"))

import numpy as np  # noqa: E402

METRIC = "steps/s at 8k & 100k nt oxDNA2: plain vs batched/surrogate, \u22641e-4 rel energy"
WORKLOAD = ("oxDNA2 plain FP32 (FENE + reductions FP64): 200 x 20-bp duplexes = 8000 nt, "
            "box 100, 296.15 K, 0.5 M, Langevin dt 0.003, fused=False")
KT = 0.1 * 296.15 / 300.0


def _dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(
        os.environ.get("LOCAL_RANK", 0))


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region: one
    `nvidia-smi -lms 200` process, started before the region, writing its samples (each
    with nvidia-smi's own timestamp) to a temporary file that is read after the region.
    The bench runs no reader thread during the region, so a timed call never waits for
    the interpreter lock on its return. __enter__ returns as soon as the second sample is
    in: the process start (which takes the host and the NVIDIA kernel driver for a while,
    longer than a 20-step timed region) and the catch-up query that can follow a slow
    first one stay outside the region, which starts a whole period before the next
    query. The summary covers the samples taken from just before the region to its end,
    with their times relative to its start."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.rows = []  # (time, fields)
        self._proc = None
        self._path = None
        self._t0 = self._t1 = None

    @staticmethod
    def parse(line):
        """(seconds since the epoch, the FIELDS values) of one output line, whose first
        value is nvidia-smi's local timestamp 'YYYY/MM/DD HH:MM:SS.mmm'; None if the line
        is incomplete. A timestamp that does not parse gives time None."""
        f = [x.strip() for x in line.strip().split(",")]
        if len(f) < 6:
            return None
        try:
            day, frac = (f[0].split(".") + ["0"])[:2]
            t = time.mktime(time.strptime(day, "%Y/%m/%d %H:%M:%S")) + float("0." + frac)
        except (ValueError, OverflowError):
            t = None
        return t, f[1:]

    def _lines(self):
        try:
            with open(self._path) as fh:
                return fh.read().split("\n")
        except (OSError, TypeError):
            return []

    def __enter__(self):
        try:
            fd, self._path = tempfile.mkstemp(prefix="clocks_", suffix=".csv")
            with os.fdopen(fd, "w") as out:
                self._proc = subprocess.Popen(
                    ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=timestamp," + self.FIELDS,
                     "--format=csv,noheader,nounits", "-lms", "200"],
                    stdout=out, stderr=subprocess.DEVNULL)
            # a busy wait: a host core that slept through it would run the first timed
            # call at its idle clock (a call right after a 200-ms sleep took ~25 µs longer)
            deadline = time.time() + 15
            polls = 0
            while time.time() < deadline and self._proc.poll() is None:
                polls += 1
                if polls % 1000 == 0 and len(self._lines()) > 2:  # two complete lines
                    break
        except Exception:
            self._proc = None
        self._t0 = time.time()
        return self

    def __exit__(self, *a):
        self._t1 = time.time()
        if self._proc is not None:
            self._proc.terminate()  # (the process started above)
            try:
                self._proc.wait(timeout=5)
            except Exception:
                self._proc.kill()
        for line in self._lines():
            r = self.parse(line)
            if r is not None:
                self.rows.append((self._t0 if r[0] is None else r[0], r[1]))
        if self._path:
            try:
                os.unlink(self._path)
            except OSError:
                pass

    def _window(self):
        if self._t0 is None:
            return [f for _, f in self.rows]
        before = [f for t, f in self.rows if t < self._t0]
        inside = [f for t, f in self.rows if self._t0 <= t <= (self._t1 or self._t0)]
        return (before[-1:] if before else []) + inside

    def summary(self):
        rows = self._window()
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4)
                          if len(r) > 5 + k and r[5 + k].lower().startswith("active")})
        out = {"sm_mhz": float(np.median(sm)) if sm else None,
               "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
               "samples": len(rows)}
        if self._t0 is not None:
            lo = [t for t, _ in self.rows if t < self._t0][-1:]
            inside = [t for t, _ in self.rows if self._t0 <= t <= (self._t1 or self._t0)]
            out["sample_ms_from_start"] = [round((t - self._t0) * 1e3, 1) for t in lo + inside]
            out["region_ms"] = round(((self._t1 or self._t0) - self._t0) * 1e3, 1)
        return out


class nvtx:
    """NVTX range around a timed region (ncu --nvtx --nvtx-include "<name>/" selects the
    kernels launched inside it)."""

    def __init__(self, name):
        self.name = name

    def __enter__(self):
        import torch
        torch.cuda.nvtx.range_push(self.name)

    def __exit__(self, *a):
        import torch
        torch.cuda.nvtx.range_pop()


def build_system(n_dup=200, n_bp=20, box=100.0, seed=2):
    from oxdna import io
    return io.duplex_system(n_dup, n_bp, box, seed=seed)


def make_sim(sysarr, fused=False, seed=1, stream=None):
    from oxdna import io, runtime
    from oxdna.model import dna2
    forces, _ = dna2.forces(fused=fused)
    sim = runtime.Simulation(device=runtime.device.GPU(), seed=seed)
    sim.create_state_from_snapshot(io.system_snapshot(sysarr))
    if stream is not None:
        sim.set_stream(stream)
    lang = runtime.md.methods.Langevin(filter=runtime.filter.All(), kT=KT)
    sim.operations.integrator = runtime.md.Integrator(dt=0.003, integrate_rotational_dof=True,
                                                      forces=forces, methods=[lang])
    return sim, forces


class no_gc:
    """The interpreter's cyclic garbage collector off inside a timed loop (as timeit
    does), so no collection pause lands in a timed call."""

    def __enter__(self):
        import gc
        self._was = gc.isenabled()
        gc.disable()

    def __exit__(self, *a):
        import gc
        if self._was:
            gc.enable()


_FLUSH = []


def l2_flush_buffer(stream):
    """The 256 MB buffer whose write flushes L2 between timed blocks, allocated and
    written once beforehand, so that neither the allocation nor the first load of the
    fill kernel falls into a timed region."""
    import torch
    if not _FLUSH:
        buf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
        with torch.cuda.stream(stream):
            buf.fill_(-1.0)
        torch.cuda.synchronize()
        _FLUSH.append(buf)
    return _FLUSH[0]


def time_resident(sim, steps, warmup, stream, block=1000):
    """K steps in blocks of `block` (one run() call each, as a HOOMD user would call
    sim.run), each timed with CUDA events on the engine stream; L2 is flushed (256 MB
    write) before every block, outside the timed events."""
    import torch
    flush = l2_flush_buffer(stream)
    sim.run(warmup)
    torch.cuda.synchronize()
    total_ms = 0.0
    done = 0
    with no_gc():
        while done < steps:
            n = min(block, steps - done)
            with torch.cuda.stream(stream):
                flush.fill_(float(done))
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            sim.run(n)
            b.record(stream)
            b.synchronize()
            total_ms += a.elapsed_time(b)
            done += n
    return total_ms


def bench_batched(stream, steps=2000, loop_steps=200, n_rep=512, seed=4, hairpin_fraction=0.0):
    """512 independent duplex replicas (12-64 bp, box 30, 290-340 K): aggregate
    nt*steps/s of the batched engine (autotuned tile shape, one persistent launch per
    5000 steps) against looping the single-system engine over the replicas (each
    replica one run(loop_steps) call; skipped when loop_steps is 0). With
    hairpin_fraction > 0 that fraction of the replicas are hairpins of the same size."""
    import torch

    from oxdna import replicas
    work = replicas.replica_workload(n_rep, seed=seed, hairpin_fraction=hairpin_fraction)
    sims = [replicas.replica_simulation(s, T, seed=100 + r) for r, (s, T) in enumerate(work)]
    b = replicas.ReplicaBatch(sims, seed=100)
    b.set_stream(stream.cuda_stream)
    tile, threads, _ = b.tune(trial_steps=50)
    b.run(20)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    with torch.cuda.stream(stream):
        flush.fill_(1.0)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    with nvtx("batched_timed"):
        b.run(steps)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    n_total = b.N
    kind = (f"one duplex of 12-64 bp or ({hairpin_fraction:.0%}) a hairpin of the same size"
            if hairpin_fraction > 0 else "one duplex of 12-64 bp")
    out = {"workload": f"{n_rep} replicas x {kind} ({n_total} nt), box 30, "
                       "290-340 K, 0.5 M, Langevin dt 0.003",
           "n_nt": n_total, "steps": steps, "tile_particles": tile, "threads": threads,
           "replica_steps_per_s": steps / (ms * 1e-3),
           "nt_steps_per_s": n_total * steps / (ms * 1e-3),
           "launches": (steps + 4999) // 5000}
    if loop_steps > 0:
        # the same replicas, one oxg_system each, run one after another
        for sim in sims:
            sim.set_stream(stream.cuda_stream)
            sim.run(20)  # attach (untimed)
        torch.cuda.synchronize()
        e0.record(stream)
        for sim in sims:
            sim.run(loop_steps)
        e1.record(stream)
        e1.synchronize()
        ms_loop = e0.elapsed_time(e1)
        out["looped_single_nt_steps_per_s"] = n_total * loop_steps / (ms_loop * 1e-3)
        out["looped_single_steps_per_call"] = loop_steps
        out["speedup_vs_looped"] = (n_total * steps / ms) / (n_total * loop_steps / ms_loop)
    return out


def bench_rna(stream, steps=2000, warmup=100):
    """oxRNA2, 64 hairpins x 48 nt (16-bp stem, 16-nt loop), box 80, 310.15 K, 1 M salt,
    Langevin dt 0.002: steps/s of the plain FP32 path."""
    from oxdna import io, runtime
    from oxdna.model import dna1, rna2
    s = io.hairpin_system(64, stem=16, loop=16, box_len=80.0, seed=3)
    forces, _ = rna2.forces(temperature=310.15, salt=1.0)
    sim = runtime.Simulation(device=runtime.device.GPU(), seed=1)
    sim.create_state_from_snapshot(io.system_snapshot(s))
    sim.set_stream(stream.cuda_stream)
    lang = runtime.md.methods.Langevin(filter=runtime.filter.All(), kT=dna1.kT_from_temperature(310.15))
    sim.operations.integrator = runtime.md.Integrator(dt=0.002, integrate_rotational_dof=True,
                                                      forces=forces, methods=[lang])
    sim.run(0)
    with nvtx("rna_timed"):
        ms = time_resident(sim, steps, warmup, stream)
    return {"workload": "oxRNA2 64 hairpins x 48 nt (3072 nt), box 80, 310.15 K, 1 M, dt 0.002",
            "steps_per_s": steps / (ms * 1e-3)}


def bench_tiled(stream, steps=10000, warmup=500, copies=8):
    """The layout of the reference's own benchmark (bench/benchmark.py): one 8-bp duplex
    (its 16-nt simple-helix; here an ideal helix with a seeded sequence, the data file
    being absent) tiled on an 8^3 grid of spacing 8 = 8192 nt in a box of 64, oxDNA2 at
    296.15 K, 0.5 M, Langevin dt 0.003; steps/s unfused and fused."""
    import torch

    from oxdna import io
    sysarr = io.tiled_duplex_system(copies)
    out = {"workload": f"oxDNA2 {copies}^3 x 8-bp duplex ({len(sysarr['pos'])} nt), box "
                       f"{copies * 8}, 296.15 K, 0.5 M, dt 0.003 (the reference benchmark's tiling)"}
    for fused in (False, True):
        tag = "fused" if fused else "unfused"
        sim, _ = make_sim(sysarr, fused=fused, stream=stream.cuda_stream)
        sim.run(0)
        sim.run(warmup)
        torch.cuda.synchronize()
        with nvtx("timed"):
            ms = time_resident(sim, steps, 0, stream)
        out[tag + "_steps_per_s"] = steps / (ms * 1e-3)
        # timed as the reference's benchmark times it: run(20), run(0), then the host
        # clock around one run(500) call
        sim.run(20)
        sim.run(0)
        t0 = time.perf_counter()
        sim.run(500)
        out[tag + "_reference_style_steps_per_s"] = 500 / (time.perf_counter() - t0)
        del sim
    return out


def bench_surrogate(stream, big, steps=1000, warmup=100, n_train=4_000_000, epochs=300, md_states=5):
    """The learned HB + cross-stacking surrogate on the 100k-nt system (2500 x 20 bp, box
    230, forces(fused=True)): trained here by the library's kernels on 4M pair geometries
    from 8000-nt trajectories at 280-360 K, its output shift calibrated on the training
    set; steps/s against the plain fused path with 1% of the pairs audited by the plain
    evaluator every 100 steps (speed run: audits recorded, switch disarmed), the fused
    term's energy error against the plain evaluator on the start state and on states of
    the plain trajectory, and a run at the default tolerance (the 1e-4 per-term energy
    budget) showing whether the audit's kill switch trips."""
    import torch

    from oxdna import surrogate
    t0 = time.perf_counter()
    f, e = surrogate.training_set(n_target=n_train)
    t_sample = time.perf_counter() - t0
    g = torch.Generator(device="cuda")
    g.manual_seed(0)
    perm = torch.randperm(f.shape[0], generator=g, device="cuda")
    nh = f.shape[0] // 20
    hold, tr = perm[:nh], perm[nh:]
    net = surrogate.Network(seed=0)
    net.fit_normalization(f[tr], e[tr])
    t0 = time.perf_counter()
    with nvtx("surrogate_train"):
        net.train(f[tr].contiguous(), e[tr].contiguous(), epochs=epochs, batch=4096, lr=3e-3,
                  lr_end=3e-5)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    bias_before = float((net.energies(f[hold]) - e[hold]).mean())
    net.calibrate(f[tr], e[tr])
    d = net.energies(f[hold]) - e[hold]
    out = {"workload": "oxDNA2 2500 x 20 bp (100k nt), box 230, 296.15 K, 0.5 M, forces(fused=True)",
           "train_pairs": int(tr.numel()), "sample_s": t_sample, "train_s": t_train, "epochs": epochs,
           "heldout_rms_pair_energy_error": float(torch.sqrt((d ** 2).mean())),
           "heldout_mean_pair_energy_error": float(d.mean()),
           "heldout_mean_pair_energy_error_before_calibration": bias_before,
           "heldout_pair_energy_sd": float(e[hold].std())}
    for mode in ("plain", "surrogate"):
        sim, forces = make_sim(big, fused=True, stream=stream.cuda_stream)
        sim.run(0)
        if mode == "surrogate":
            e_plain = forces[2].energy
            sim.set_surrogate(net, run=False, compute=True)
            # the built start state: every base pair of the ideal duplexes at one geometry
            out["fused_term_energy_rel_error_vs_plain_built_state"] = abs(forces[2].energy - e_plain) / abs(e_plain)
            sim.set_surrogate(net, run=True, compute=False, audit_every=100, audit_fraction=0.01,
                              tol=1e30)
        with nvtx(mode + "_timed"):
            ms = time_resident(sim, steps, warmup, stream)
        out[mode + "_steps_per_s"] = steps / (ms * 1e-3)
        if mode == "plain":
            # the term's energy on states of the plain trajectory: surrogate read-out
            # against the plain evaluator's on the same state, every 1000 steps
            md = []
            for _ in range(md_states):
                e_plain = forces[2].energy
                sim.set_surrogate(net, run=False, compute=True)
                md.append((forces[2].energy - e_plain) / abs(e_plain))
                sim.set_surrogate(None)
                sim.run(1000)
            out["fused_term_energy_rel_error_vs_plain_md_states"] = md
            out["fused_term_energy_rel_error_vs_plain_md_max"] = max(abs(x) for x in md)
            out["md_states_note"] = (f"states of the plain trajectory after {warmup + steps} steps, "
                                     "then every 1000 steps (signed relative error)")
        if mode == "surrogate":
            st = sim.surrogate_stats()
            out["audit"] = {"pairs": int(st["n_audited"]),
                            "rel_term_energy_error": st["rel_energy_error"],
                            "rel_term_energy_error_se": st["rel_energy_error_se"],
                            "rms_pair_energy_error": st["rms_de"], "rms_pair_energy": st["rms_e"],
                            "rms_pair_force_error": st["rms_df"], "rms_pair_force": st["rms_f"],
                            "rel_force_error": st["rms_df"] / max(st["rms_f"], 1e-30)}
            # the audit at the default tolerance (1e-4): does the kill switch trip?
            sim.set_surrogate(net, run=True, compute=False, audit_every=100, audit_fraction=0.01)
            sim.run(2000)
            st = sim.surrogate_stats()
            out["audit_at_budget"] = {"tol": 1e-4, "steps": 2000, "pairs": int(st["n_audited"]),
                                      "kill_switch": bool(st["disabled"]),
                                      "rel_term_energy_error": st["rel_energy_error"],
                                      "rel_term_energy_error_se": st["rel_energy_error_se"]}
        del sim
    out["speedup_vs_plain"] = out["surrogate_steps_per_s"] / out["plain_steps_per_s"]
    out["observables"] = surrogate_observables(stream, big, net)
    return out


def surrogate_observables(stream, big, net, temps=(296.15, 330.0), steps=10000, every=250):
    """The 2-sigma criterion on MD observables of the 100k-nt system: per-nucleotide
    energy of every force and the fraction of formed base pairs, block-averaged (10
    blocks) over a plain trajectory and over one driven by the surrogate (kill switch
    disarmed), both measured by the plain evaluator, at each temperature."""
    from oxdna import io, observables, runtime
    from oxdna.model import dna1, dna2
    res = {}
    for T in temps:
        runs = {}
        for mode in ("plain", "surrogate"):
            forces, _ = dna2.forces(temperature=T, fused=True)
            sim = runtime.Simulation(device=runtime.device.GPU(), seed=17)
            sim.create_state_from_snapshot(io.system_snapshot(big))
            sim.set_stream(stream.cuda_stream)
            lang = runtime.md.methods.Langevin(filter=runtime.filter.All(),
                                               kT=dna1.kT_from_temperature(T))
            sim.operations.integrator = runtime.md.Integrator(dt=0.003, integrate_rotational_dof=True,
                                                              forces=forces, methods=[lang])
            sim.run(0)
            if mode == "surrogate":
                sim.set_surrogate(net, run=True, compute=False, audit_every=0, tol=1e30)
            sim.run(1000)
            runs[mode] = observables.sample(sim, forces, steps=steps, every=every)
            del sim
        cmp = observables.compare(runs["plain"], runs["surrogate"], n_blocks=10, k=2.0)
        res[f"{T:g}K"] = {k: {"plain": v["a"], "surrogate": v["b"], "agree_2sigma": v["agree"]}
                          for k, v in cmp.items()}
    res["all_agree_2sigma"] = all(v["agree_2sigma"] for t in res.values() for v in t.values())
    res["note"] = (f"{steps} steps after 1000 of equilibration, a sample every {every} steps, "
                   "(mean, standard error) per observable")
    return res


def hoomd_full_nlist(pos, box, r_list, bonds):
    """HOOMD's neighbour-list layout for N particles: a FULL list (each pair from both
    ends, bonded pairs excluded) as n_neigh (uint32), nlist (uint32) and head_list
    (uint64), built on the host with a periodic k-d tree."""
    from scipy.spatial import cKDTree
    L = float(box[0])
    x = np.mod(np.asarray(pos, np.float64) + 0.5 * L, L)
    pairs = cKDTree(x, boxsize=L).query_pairs(r_list, output_type="ndarray")
    n = len(x)
    key = lambda a, b: np.minimum(a, b).astype(np.int64) * n + np.maximum(a, b)  # noqa: E731
    b = np.asarray(bonds, np.int64)
    keep = ~np.isin(key(pairs[:, 0], pairs[:, 1]), key(b[:, 0], b[:, 1]))
    pairs = pairs[keep]
    i = np.concatenate([pairs[:, 0], pairs[:, 1]])
    j = np.concatenate([pairs[:, 1], pairs[:, 0]])
    order = np.lexsort((j, i))
    i, j = i[order], j[order]
    n_neigh = np.bincount(i, minlength=n).astype(np.uint32)
    head = np.concatenate([[0], np.cumsum(n_neigh)[:-1]]).astype(np.uint64)
    return n_neigh, j.astype(np.uint32), head


def bench_dropin(stream, sysarr, calls=200):
    """The evaluator-level entry points a HOOMD build would call in place of the
    reference's kernels, on HOOMD-shaped buffers (Scalar4 double positions and
    orientations, full neighbour list of radius max r_cut + 0.4, device arrays):
    oxg_pair_forces for each of the five oxDNA2 terms of forces(fused=False) alone (the
    reference runs one aniso launch per term) and for all five in one call, and
    oxg_bonded_forces; microseconds per call from CUDA events over `calls` calls."""
    import ctypes as C

    import torch

    from oxdna import _abi, io
    from oxdna.model import dna2
    L = _abi.lib()
    forces, _ = dna2.forces(fused=False)
    bonded, pair = forces[0], forces[1:]
    n = len(sysarr["pos"])
    ctx = C.c_void_p()
    _abi.check(L.oxg_create(C.byref(ctx), 4, 1), "oxg_create")
    setters = {_abi.EXCVOL: L.oxg_set_excvol_params, _abi.HBOND: L.oxg_set_hbond_params,
               _abi.CROSS: L.oxg_set_cross_params, _abi.COAX: L.oxg_set_coax_params,
               _abi.DEBYE: L.oxg_set_debye_params}
    for f in pair:
        for a in range(4):
            for b in range(a, 4):
                key = (io.DNA_BASES[a], io.DNA_BASES[b])
                _abi.check(setters[f._term](ctx, a, b, C.byref(_abi.FROM_DICT[f._term](f.params[key])),
                                            f.rcut_for(*key)), "set params")
    bp = _abi.bonded_from_dict(bonded.params["backbone"])
    _abi.check(L.oxg_set_bonded_params(ctx, 0, C.byref(bp)), "oxg_set_bonded_params")
    dev = torch.device("cuda")
    pt = np.zeros((n, 4))
    pt[:, :3] = sysarr["pos"]
    pt[:, 3] = sysarr["typeid"].astype(np.int64).view(np.float64)
    r_list = max(f.default_r_cut for f in pair) + 0.4
    nn, flat, head = hoomd_full_nlist(sysarr["pos"], sysarr["box"], r_list, sysarr["bonds"])
    pos_d = torch.tensor(pt, dtype=torch.float64, device=dev)
    quat_d = torch.tensor(sysarr["quat"], dtype=torch.float64, device=dev)
    ch_d = torch.ones(n, dtype=torch.float64, device=dev)
    nn_d = torch.tensor(nn.astype(np.int64), device=dev).to(torch.int32)
    fl_d = torch.tensor(flat.astype(np.int64), device=dev).to(torch.int32)
    hd_d = torch.tensor(head.astype(np.int64), device=dev)
    bonds = np.zeros((len(sysarr["bonds"]), 3), np.int64)
    bonds[:, :2] = sysarr["bonds"]
    bonds_d = torch.tensor(bonds, device=dev).to(torch.int32)
    force = torch.zeros((n, 4), dtype=torch.float32, device=dev)
    torque = torch.zeros((n, 4), dtype=torch.float32, device=dev)
    box = (C.c_float * 3)(*[float(x) for x in sysarr["box"]])
    ptr = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    sh = C.c_void_p(stream.cuda_stream)

    def timed(fn):
        for _ in range(5):
            fn()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(calls):
            fn()
        b.record(stream)
        b.synchronize()
        _abi.check(L.oxg_context_status(ctx, 1), "oxg_context_status")
        return a.elapsed_time(b) * 1e3 / calls

    def pair_call(mask):
        return lambda: _abi.check(L.oxg_pair_forces(ctx, mask, n, ptr(pos_d), ptr(quat_d), ptr(ch_d), box,
                                                    ptr(nn_d), ptr(fl_d), ptr(hd_d), ptr(force),
                                                    ptr(torque), None, None, sh), "oxg_pair_forces")

    out = {"workload": f"oxDNA2 {n} nt (the headline system), HOOMD buffers: Scalar4 double "
                       f"positions / orientations, full list r_list {r_list:.2f} "
                       f"({int(nn.sum())} entries, {nn.mean():.1f} per particle)",
           "calls": calls, "us_per_call": {}}
    all_mask = 0
    for f in pair:
        all_mask |= 1 << f._term
    # all five terms first (an ncu capture of this leg meets this call first)
    out["us_per_call"]["all_five_terms_one_call"] = timed(pair_call(all_mask))
    for f in pair:
        out["us_per_call"][_abi.TERM_NAMES[f._term]] = timed(pair_call(1 << f._term))
    out["us_per_call"]["oxdna_bonded"] = timed(lambda: _abi.check(L.oxg_bonded_forces(
        ctx, n, ptr(pos_d), ptr(quat_d), box, len(bonds), ptr(bonds_d), ptr(force), ptr(torque),
        None, None, sh), "oxg_bonded_forces"))
    per = out["us_per_call"]
    out["us_per_step_one_launch_per_term"] = sum(per[_abi.TERM_NAMES[f._term]] for f in pair) + \
        per["oxdna_bonded"]
    out["us_per_step_all_terms_one_call"] = per["all_five_terms_one_call"] + per["oxdna_bonded"]
    L.oxg_destroy(ctx)
    # the same forces through the engine's read-out path (half pair lists, phase A / B
    # kernels, i side summed per run, float4 atomics): host wall time per call, which
    # includes the call's synchronisation and energy copy
    sim, _ = make_sim(sysarr, fused=False, stream=stream.cuda_stream)
    sim.run(0)
    mask = sum(1 << f._term for f in pair)
    comp = lambda: _abi.check(L.oxg_system_compute(sim._sys, mask, 1, None, None, None, None),  # noqa: E731
                              "oxg_system_compute")
    for _ in range(5):
        comp()
    t0 = time.perf_counter()
    for _ in range(calls):
        comp()
    out["engine_readout_us_per_call_host_wall"] = (time.perf_counter() - t0) / calls * 1e6
    return out


FLOP_COUNTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden",
                           "flop_counts.json")


def compute_roofline(ms_per_step, stream, workload="8000nt"):
    """The MD step against the pipes that bound it: the reference's FP32 operation count
    per step (flop census of its own evaluator and bonded arithmetic at the workload's
    initial snapshot) over the run kernel's event-timed step time, against the FP32 FMA
    and special-function throughput measured on this device by the library's
    microbenchmarks (oxg_device_peaks)."""
    from oxdna import runtime
    with open(FLOP_COUNTS) as fh:
        census = json.load(fh)["workloads"][workload]
    fp32_gflops, sfu_gops = runtime.device_peaks(stream.cuda_stream)
    t = ms_per_step * 1e-3
    flops = census["flops_per_step"]
    special = sum(census["special_per_step"].values())
    achieved = flops / t / 1e12
    sfu = special / t / 1e9
    return {"bound": "fp32", "achieved": achieved, "peak": fp32_gflops / 1e3, "unit": "TFLOP/s",
            "frac": achieved / (fp32_gflops / 1e3), "peak_kind": "measured (oxg_device_peaks FMA "
            "microbenchmark on this device)", "flops_per_step": flops,
            "special": {"achieved": sfu, "peak": sfu_gops, "unit": "Gop/s", "frac": sfu / sfu_gops,
                        "ops_per_step": special, "per_step": census["special_per_step"],
                        "note": "each div / sqrt / exp / acos / sin call counted as one "
                                "special-function op (acos and div also cost FMA-pipe work)"},
            "source": "tests/golden/flop_counts.json (reference headers compiled with an "
                      "operation-counting ForceReal; flops = add + mul, FMA = 2)"}


def cpu_baseline(sysarr, seconds=12.0, max_steps=400, threads=None):
    """The oracle port (FP64 C, OpenMP) running Langevin steps on the host cores."""
    from oracle import oracle as O
    from oxdna import io
    from oxdna.model import dna2
    threads = threads or os.cpu_count()
    forces, _ = dna2.forces(fused=False)
    model = O.Model(forces, io.DNA_BASES)
    s = O.System(sysarr["pos"], sysarr["quat"], sysarr["typeid"], sysarr["box"], sysarr["bonds"])
    n = len(sysarr["pos"])
    vel, am = np.zeros((n, 3)), np.zeros((n, 4))
    O.langevin(model, s, vel, am, steps=2, dt=0.003, kT=KT, seed=1, threads=threads)  # warm
    done, t0 = 0, time.perf_counter()
    chunk = 5
    while done < max_steps and time.perf_counter() - t0 < seconds:
        _, vel, am = O.langevin(model, s, vel, am, steps=chunk, dt=0.003, kT=KT, seed=1,
                                step0=done, threads=threads)
        done += chunk
    dt = time.perf_counter() - t0
    return {"value": done / dt, "unit": "steps/s", "cores": threads, "kind": "port",
            "sample": f"{done} Langevin steps of the 8000-nt workload (FP64 C oracle, OpenMP, "
                      f"{threads} threads, run() call per {chunk} steps)"}


def cpu_arithmetic(sysarr, reps=3):
    """Forces of the 8000-nt workload on one host core: the C restatement (its own cell
    list included) beside the reference's own evaluator and bonded headers compiled
    unchanged (oracle/_ref, HOOMD CPU driver semantics over a prebuilt half list) where
    that build exists (the reference source tree is needed to compile it)."""
    from oracle import oracle as O
    from oxdna import io
    from oxdna.model import dna2
    forces, _ = dna2.forces(fused=False)
    model = O.Model(forces, io.DNA_BASES)
    s = O.System(sysarr["pos"], sysarr["quat"], sysarr["typeid"], sysarr["box"], sysarr["bonds"])
    out = {"workload": "forces of the 8000-nt workload (every term, bonds), FP64, one host core"}
    O.forces(model, s)
    t0 = time.perf_counter()
    for _ in range(reps):
        O.forces(model, s)
    out["port_ms"] = (time.perf_counter() - t0) / reps * 1e3
    if O.ref_lib(64) is not None:
        pair = forces[1:]
        rl = max(f.rcut_for(a, b) for f in pair for a in io.DNA_BASES for b in io.DNA_BASES)
        pairs = O.half_pairs(s, rl * (1 + 1e-9))
        O.ref_system_forces(model, s, pairs)
        t0 = time.perf_counter()
        for _ in range(reps):
            O.ref_system_forces(model, s, pairs)
        out["reference_headers_ms"] = (time.perf_counter() - t0) / reps * 1e3
        out["reference_headers_over_port"] = out["reference_headers_ms"] / out["port_ms"]
        out["note"] = ("reference_headers: src/EvaluatorPairOxDNA*.h and src/OxDNABondedKernel.h "
                       "compiled unchanged at -O3 (g++), pair list prebuilt; port: "
                       "oracle/oxdna_oracle.c at -O3 (gcc), its cell list built per call")
    else:
        out["reference_headers_ms"] = None
        out["note"] = "the reference source tree is absent here: only the port is timed"
    return out


def run_reference(args):
    rank, world, _ = _dist_env()
    if rank != 0:
        return
    sysarr = build_system()
    cb = cpu_baseline(sysarr, seconds=max(10.0, min(60.0, 0.02 * args.steps)),
                      max_steps=max(args.steps, 10))
    cb["reference_build"] = ("oracle port: the reference's HOOMD build cannot be installed "
                             "(no HOOMD-blue on this machine)")
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "steps/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 / cb["value"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD},
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


PROFILE_TRAFFIC = os.path.join(ROOT, "profiles", "k_run_8000nt.md")


def profiled_traffic():
    """DRAM bytes per run-kernel launch of the headline workload from the committed ncu
    summary (its ``traffic_bytes_per_launch:`` line; dram__bytes_read.sum +
    dram__bytes_write.sum of one launch). The working set (~5 MB) is read into L2 once
    per launch and stays there, so the figure is per launch whatever its step count."""
    try:
        with open(PROFILE_TRAFFIC) as fh:
            for line in fh:
                if line.strip().startswith("traffic_bytes_per_launch:"):
                    return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


def run_ours(args):
    import torch
    rank, world, local = _dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from oxdna import replicas
    stream = torch.cuda.Stream()
    sysarr = build_system(seed=2 + rank)
    n = len(sysarr["pos"])
    sim, forces = make_sim(sysarr, fused=False, seed=1 + rank, stream=stream.cuda_stream)
    sim.run(0)

    # --- device-resident throughput -------------------------------------------
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    l2_flush_buffer(stream)
    with ClockSampler(local) as clk:
        # the W warm-up steps directly before the timed block, after the sampler's wait
        sim.run(args.warmup)
        sim.run_kernel_timing(reset=True)
        with nvtx("timed"):
            ms = time_resident(sim, args.steps, 0, stream)
    k_ms, k_launches, k_steps = sim.run_kernel_timing(reset=True)
    torch.cuda.synchronize()
    ms = replicas.max_over_ranks(ms, dist)
    steps_per_s = world * args.steps / (ms * 1e-3)
    stats = sim.native_stats()
    if args.quick:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": steps_per_s, "unit": "steps/s",
                              "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                              "quick": True, "kernel_ms": k_ms, "kernel_launches": k_launches,
                              "clocks": clk.summary()}), flush=True)
        if dist is not None:
            dist.destroy_process_group()
        return

    # --- roofline of the dominant kernel: the persistent run kernel k_run ----------
    # Its launches (one per run() block of up to 1000 steps) were timed with CUDA events
    # on the engine stream during the timed region. Algorithmic bytes per step: the
    # pair lists (8 B / pair), the bonds (16 B / bond), per particle the position,
    # low-order position, quaternion and charge reads (52 B), force and torque
    # read-modify-write (64 B) and the integrator's state update (velocity, angular
    # momentum read + write, position and quaternion writes: 96 B).
    st = sim.native_stats()
    pairs = st["pairs_short"] + st["pairs_long"]
    n_bonds = len(sysarr["bonds"])
    alg_bytes_step = 8 * pairs + 16 * n_bonds + (52 + 64 + 96) * n
    kernel_ms = k_ms / max(k_launches, 1)
    steps_per_launch = k_steps / max(k_launches, 1)
    hbm, peak_kind = _peaks()
    achieved = alg_bytes_step * steps_per_launch / (kernel_ms * 1e-3) / 1e9
    compute = compute_roofline(kernel_ms / steps_per_launch, stream)
    # steady state of the same workload: one long run() (the per-call run start and the
    # cold L2 after the flush amortised), beside the K-step figure above
    steady_steps = 20000
    ms_steady = time_resident(sim, steady_steps, 0, stream, block=steady_steps)
    legs = {"steady_state_steps_per_s": steady_steps / (ms_steady * 1e-3),
            "steady_state_note": f"one run({steady_steps}) call of the headline workload"}

    # --- fused=True variant (HBondCross) ---------------------------------------
    sim_f, _ = make_sim(sysarr, fused=True, seed=1 + rank, stream=stream.cuda_stream)
    sim_f.run(0)
    ms_f = time_resident(sim_f, 5000, 100, stream, block=5000)
    legs["fused_true_steps_per_s"] = 5000 / (ms_f * 1e-3)
    del sim_f

    # --- the reference benchmark's own layout (8^3 tiled 8-bp duplex, 8192 nt) ----
    legs["tiled"] = bench_tiled(stream, steps=5000, warmup=200)

    # --- 100k nt (2500 x 20-bp duplexes, box 230): the plain path at the large size --
    big = build_system(n_dup=2500, n_bp=20, box=230.0, seed=5 + rank)
    sim_b, _ = make_sim(big, fused=False, seed=1 + rank, stream=stream.cuda_stream)
    sim_b.run(0)
    ms_b = time_resident(sim_b, 2000, 100, stream, block=2000)
    big_stats = sim_b.native_stats()
    legs["nt100k"] = {"steps_per_s": 2000 / (ms_b * 1e-3),
                      "nt_steps_per_s": 2000 / (ms_b * 1e-3) * len(big["pos"]),
                      "pairs": [big_stats["pairs_short"], big_stats["pairs_long"]]}
    del sim_b

    # --- drop-in entry points, batched replicas, RNA hairpins, learned surrogate ------
    legs["dropin"] = bench_dropin(stream, sysarr)
    legs["batched"] = bench_batched(stream, steps=2000)
    legs["batched_with_hairpins"] = bench_batched(stream, steps=2000, hairpin_fraction=0.5,
                                                  loop_steps=0)
    legs["rna_hairpins"] = bench_rna(stream, steps=2000, warmup=100)
    legs["surrogate_100k"] = bench_surrogate(stream, big, steps=1000, warmup=100)

    # --- end to end through the public API with host buffers ----------------------
    pin = lambda: torch.empty((n, 4), dtype=torch.float32).pin_memory().numpy()  # noqa: E731
    hp, hl, hq, hv, ha = pin(), pin(), pin(), pin(), pin()
    sim.pull_state_arrays(hp, hl, hq, hv, ha)
    e2e_steps = 1000

    def e2e_loop(session_us):
        """Steps/s of run_state_arrays(1, ...) calls, with a host session of the given
        idle time (0: one launch per call). The timed region ends after the session has
        been ended (the resident kernel left) and the device synchronised."""
        sim.set_host_session(session_us)
        for _ in range(3):  # warm-up of the call sequence
            sim.run_state_arrays(1, hp, hl, hq, hv, ha)
        sim.set_host_session(session_us)  # (ends the warm-up's resident kernel)
        torch.cuda.synchronize()
        with no_gc():
            t0 = time.perf_counter()
            for _ in range(e2e_steps):
                # H2D: this step's inputs, one MD step, D2H: this step's result, in one call
                sim.run_state_arrays(1, hp, hl, hq, hv, ha)
            sim.set_host_session(0)
        torch.cuda.synchronize()
        return replicas.max_over_ranks(time.perf_counter() - t0, dist)

    e2e_s = e2e_loop(1000)
    e2e_launch_s = e2e_loop(0)
    # the same through three calls (state push, run, state pull)
    torch.cuda.synchronize()
    with no_gc():
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            sim.push_state_arrays(hp, hl, hq, hv, ha)
            sim.run(1)
            sim.pull_state_arrays(hp, hl, hq, hv, ha)
        torch.cuda.synchronize()
    e2e3_s = replicas.max_over_ranks(time.perf_counter() - t0, dist)
    e2e = {"value": world * e2e_steps / e2e_s, "unit": "steps/s",
           "h2d_bytes_per_step": 5 * 16 * n, "d2h_bytes_per_step": 5 * 16 * n,
           "path": "Simulation.run_state_arrays(1, pinned host arrays) in a host session "
                   "(set_host_session(1000): the run kernel stays resident between calls and takes "
                   "each call as a request in page-locked memory; it reads the host state at the "
                   "run start and writes it back in its last step)",
           "launch_per_call_steps_per_s": world * e2e_steps / e2e_launch_s,
           "launch_per_call_path": "the same calls without a session: one launch of the run kernel "
                                   "per call",
           "three_calls_steps_per_s": world * e2e_steps / e2e3_s,
           "three_calls_path": "push_state_arrays -> run(1) -> pull_state_arrays"}

    # --- CPU baseline (rank 0, N = 1 only) --------------------------------------
    cb = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cb = cpu_baseline(sysarr)
        one = cpu_baseline(sysarr, seconds=8.0, max_steps=100, threads=1)
        cb["single_core"] = {"value": one["value"], "unit": one["unit"], "cores": 1,
                             "sample": one["sample"]}
    if rank != 0:
        dist.destroy_process_group()
        return
    # one persistent run-kernel launch per run() block of up to 1000 steps (its first
    # body is the run start: checkpoint, list check, prepRun forces, the first step one)
    traffic = profiled_traffic()
    line = {
        "metric": METRIC, "value": steps_per_s, "unit": "steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD},
        "workload_detail": {"n_nt": n, "bonds": n_bonds, "pairs_short": st["pairs_short"],
                            "pairs_long": st["pairs_long"],
                            "l2": "flushed (256 MB write) before every timed run() block of up "
                                  "to 1000 steps; within a block the ~5 MB working set stays "
                                  "L2-resident"},
        "legs": legs,
        "reference_published": "~4600 steps/s unfused, ~5000 fused (RTX 4090, 8192-nt tiled "
                               "duplex, box 64; README.md:97-98): compare legs.tiled",
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic,
                     "traffic_note": "DRAM bytes of one run-kernel launch of this workload "
                                     "(ncu, profiles/k_run_8000nt.md); the algorithmic bytes "
                                     "of its steps are served from L2",
                     "peak_kind": peak_kind,
                     "kernel": "k_run (persistent MD step kernel: nlist rebuild when flagged, "
                               "forces, Langevin + NO_SQUISH)",
                     "kernel_ms_per_launch": kernel_ms, "steps_per_launch": steps_per_launch,
                     "alg_bytes_per_step": alg_bytes_step,
                     "note": "latency-bound, not HBM-bound: the 8000-nt working set (~5 MB) "
                             "is L2-resident"},
        "roofline_compute": compute,
        "cpu_baseline": cb, "e2e": e2e,
        "gpu_launches": k_launches,
        "clocks": clk.summary(),
        "nlist_builds": stats["nlist_builds"],
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30000)
    ap.add_argument("--warmup", type=int, default=500)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--quick", action="store_true",
                    help="resident timing only (no fused / e2e / CPU legs); for profiling runs")
    ap.add_argument("--leg", choices=["batched", "rna", "surrogate", "nt100k", "tiled", "dropin",
                                      "cpu"],
                    help="run one extension leg alone and print its numbers (profiling runs)")
    ap.add_argument("--hairpin-fraction", type=float, default=0.0,
                    help="--leg batched: fraction of the replicas that are hairpins")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.leg:
        run_leg(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


def run_leg(args):
    if args.leg == "cpu":
        print(json.dumps({"leg": "cpu", **cpu_arithmetic(build_system())}), flush=True)
        return
    import torch
    stream = torch.cuda.Stream()
    if args.leg == "batched":
        out = bench_batched(stream, steps=args.steps, hairpin_fraction=args.hairpin_fraction)
    elif args.leg == "rna":
        out = bench_rna(stream, steps=args.steps, warmup=args.warmup)
    elif args.leg == "tiled":
        out = bench_tiled(stream, steps=args.steps, warmup=args.warmup)
    elif args.leg == "dropin":
        out = bench_dropin(stream, build_system(), calls=args.steps)
    elif args.leg == "nt100k":
        big = build_system(n_dup=2500, n_bp=20, box=230.0, seed=5)
        sim, _ = make_sim(big, fused=False, stream=stream.cuda_stream)
        sim.run(0)
        sim.run(args.warmup)
        torch.cuda.synchronize()
        with nvtx("timed"):
            ms = time_resident(sim, args.steps, 0, stream, block=args.steps)
        out = {"workload": "oxDNA2 2500 x 20 bp (100k nt), box 230, 296.15 K, 0.5 M, fused=False",
               "steps_per_s": args.steps / (ms * 1e-3)}
    else:
        big = build_system(n_dup=2500, n_bp=20, box=230.0, seed=5)
        out = bench_surrogate(stream, big, steps=args.steps, warmup=args.warmup)
    print(json.dumps({"leg": args.leg, **out}), flush=True)


if __name__ == "__main__":
    main()
