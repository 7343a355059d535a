"""Host-side logic: parameter dicts, ABI structs, models, builders, library exports."""

import ctypes as C
import math
import os
import re

import numpy as np
import pytest

from _util import model_forces

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_hb_complementarity():
    """pytest/test_hbond.py:27-30."""
    from oxdna.model import dna1
    assert dna1.hb_epsilon("A", "T") > 0 and dna1.hb_epsilon("G", "C") > 0
    for a, b in [("A", "A"), ("A", "G"), ("A", "C"), ("G", "G"), ("G", "T"), ("C", "T")]:
        assert dna1.hb_epsilon(a, b) == 0.0


def test_param_dict_validation():
    from oxdna.model import dna2
    nl = dna2.make_neighbor_list()
    f = dna2.debye_huckel(nl)
    assert f.params[("T", "A")] == f.params[("A", "T")]  # unordered pair keys
    with pytest.raises(KeyError):
        f.params[("A", "A")] = dict(back_site=(0, 0, 0))  # missing 'debye'
    with pytest.raises(ValueError):
        f.params[("A", "A")] = dict(back_site=(0, 0), debye=(1, 2, 3, 4, 5))
    with pytest.raises(KeyError):
        f.params[("A", "A")] = dict(back_site=(0, 0, 0), debye=(1, 2, 3, 4, 5), bogus=1)
    c = dna2.coaxial_stacking(nl)
    assert c.params[("A", "C")]["f5_phi4"] == (0.0,) * 4 and c.params[("A", "C")]["rna_coax"] is False
    from oxdna.forces import ExcludedVolume
    with pytest.raises(ValueError):
        ExcludedVolume(nl, 2.0, mode="shift")  # the evaluators implement no energy shift


def test_abi_struct_conversion():
    from oxdna import _abi
    pair, bonded = model_forces("rna2")
    p = _abi.cross_from_dict(pair[2].params[("A", "A")])
    assert p.t4_enabled == 0 and abs(p.f2[0] - 59.9626) < 1e-12
    b = _abi.bonded_from_dict(bonded.params["backbone"])
    assert b.stacking_enabled == 1 and b.rna_stacking == 1
    assert abs(b.delta2 - 0.0625) < 1e-15
    assert abs(b.stack_5_site[0] - 0.124906078525) < 1e-15
    # sizes match the C layout (double-aligned, no hidden padding differences)
    assert C.sizeof(_abi.CoaxParams) == 8 * (3 + 3 + 1 + 9 + 15 + 8) + 4 * 2 + 8 * 2 + 4 * 2
    assert C.sizeof(_abi.CrossParams) % 8 == 0


def test_debye_parameters():
    """dna2.debye_params at 296.15 K, 0.5 M: lambda 0.50815, rc 2.2867 (the 320-nt configuration)."""
    from oxdna.model import dna2
    mk, pref, b, rc, rhigh = dna2.debye_params(296.15, 0.5)
    assert abs(-1.0 / mk - 0.50815) < 1e-4 and abs(rc - 2.2867) < 1e-3
    assert abs(rhigh - 3 * (-1.0 / mk)) < 1e-12


def test_duplex_builder_geometry():
    """Ideal B-form duplexes: every FENE bond within delta, a1/a3 conventions."""
    from oxdna import io
    from oxdna.model import dna2
    s = io.duplex_system(8, 20, 40.0, seed=1)
    R = io.quat_to_matrix(s["quat"])
    back = s["pos"] + np.einsum("nij,j->ni", R, dna2.BACK_SITE)
    for a, b in s["bonds"]:
        d = back[b] - back[a]
        d -= 40.0 * np.round(d / 40.0)
        assert abs(np.linalg.norm(d) - dna2.FENE_R0) < 0.25
    assert len(s["pos"]) == 320 and len(s["bonds"]) == 8 * 38
    # complementary strands: paired bases sum to 3
    t = s["typeid"][:40]
    assert all(t[k] + t[39 - k] == 3 for k in range(20))


def test_quaternion_roundtrip():
    from oxdna import io
    rng = np.random.default_rng(3)
    q = rng.normal(size=(50, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    R = io.quat_to_matrix(q)
    q2 = io.orientations_to_quaternions(R[:, :, 0], R[:, :, 2])
    assert np.allclose(np.abs(np.einsum("ij,ij->i", q, q2)), 1.0, atol=1e-12)


def test_replica_workload_hairpins():
    from oxdna import replicas
    base = replicas.replica_workload(40, seed=9)
    mixed = replicas.replica_workload(40, seed=9, hairpin_fraction=0.5)
    assert replicas.replica_workload(40, seed=9, hairpin_fraction=0.0)[7][0]["pos"].tolist() == \
        base[7][0]["pos"].tolist()
    n_hairpins = 0
    for (d, td), (m, tm) in zip(base, mixed):
        assert td == tm and len(d["pos"]) == len(m["pos"])  # same size and temperature
        strands = len(m["pos"]) - len(m["bonds"])
        assert strands in (1, 2)
        if strands == 1:
            n_hairpins += 1
            n = len(m["pos"])
            t = m["typeid"]
            stem = n // 2 - 4
            # 5'-stem, 8-nt loop, complementary stem-3': paired bases sum to 3
            assert all(t[k] + t[n - 1 - k] == 3 for k in range(stem))
        else:
            assert d["pos"].tolist() == m["pos"].tolist()
    assert 10 <= n_hairpins <= 30
    with pytest.raises(ValueError):
        replicas.replica_workload(4, hairpin_fraction=0.5, hairpin_loop=7)


def test_replica_sharding():
    from oxdna import replicas
    shards = [replicas.shard(103, r, 4) for r in range(4)]
    assert sorted(np.concatenate(shards).tolist()) == list(range(103))
    assert max(len(x) for x in shards) - min(len(x) for x in shards) <= 1


def _header_functions():
    src = open(os.path.join(ROOT, "include", "oxdna_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(oxg_\w+)\(", src, re.M)))


def test_library_exports_every_header_symbol():
    """The C-ABI library builds for sm_103a, loads without a GPU and exports every
    entry point include/oxdna_gb300.h declares (no compute call is made)."""
    from oxdna import _abi, _build
    _build.build()
    L = C.CDLL(_abi.LIB_PATH)
    names = _header_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(_abi.EXPORTS)
    assert b"sm_103a" in _abi.lib().oxg_version()


def test_abi_rejects_null_handles_without_touching_the_device():
    """Every entry point checks its handle and pointers before any device work: called
    with a null handle (and zero / null for the rest) each returns OXG_ERR_INVALID_ARG
    with a message, the destroy calls accept null (OXG_OK), and the status strings
    name every code (the reference's std::runtime_error throws become status codes)."""
    from oxdna import _abi
    L = _abi.lib()
    ints = (C.c_int32, C.c_uint32, C.c_long, C.c_uint64, C.c_int)
    for name in _abi.EXPORTS:
        if name in ("oxg_last_error", "oxg_version", "oxg_status_string"):
            continue
        fn = getattr(L, name)
        args = [0 if t in ints else 0.0 if t in (C.c_double, C.c_float) else None
                for t in fn.argtypes]
        rc = fn(*args)
        if name.endswith("_destroy"):
            assert rc == 0, name
        else:
            assert rc == 1, (name, rc)
            assert L.oxg_last_error(), name
    names = {L.oxg_status_string(k).decode() for k in range(9)}
    assert len(names) == 9 and "unknown status" not in names
    assert L.oxg_status_string(99) == b"unknown status"
    # out-of-range sizes are rejected before the device is looked at
    h = C.c_void_p()
    assert L.oxg_create(C.byref(h), 0, 1) == 1 and not h.value
    assert L.oxg_create(C.byref(h), 5, 1) == 1 and not h.value
    assert L.oxg_create(C.byref(h), 4, -1) == 1 and not h.value
    with pytest.raises(_abi.OxgError, match="status 1"):
        _abi.check(L.oxg_system_run(None, 10), "oxg_system_run")


def test_snapshot_checkpoint_round_trip(tmp_path):
    """write_snapshot / read_snapshot keep every field bit for bit, and a simulation
    created from the snapshot takes its timestep (the noise counter of a resumed run)."""
    from oxdna import io, runtime
    s = io.duplex_system(3, 10, 20.0, seed=5)
    snap = io.system_snapshot(s, half_charged_ends=True)
    rng = np.random.default_rng(1)
    snap.particles.velocity[:] = rng.normal(size=(snap.particles.N, 3))
    snap.particles.angmom[:] = rng.normal(size=(snap.particles.N, 4))
    snap.configuration.step = 123456789012
    runtime.write_snapshot(snap, tmp_path / "ck.npz")
    back = runtime.read_snapshot(tmp_path / "ck.npz")
    for k in ("position", "typeid", "mass", "moment_inertia", "orientation", "charge",
              "velocity", "angmom", "image"):
        a, b = getattr(snap.particles, k), getattr(back.particles, k)
        assert a.dtype == b.dtype and np.array_equal(a, b), k
    assert back.particles.types == snap.particles.types
    assert np.array_equal(back.bonds.group, snap.bonds.group) and back.bonds.types == ["backbone"]
    assert back.configuration.box == snap.configuration.box
    assert back.configuration.step == 123456789012
    sim = runtime.Simulation(device=runtime.device.GPU(), seed=3)
    sim.create_state_from_snapshot(back)
    assert sim.timestep == 123456789012
    assert sim.state.get_snapshot().configuration.step == 123456789012


def test_engine_sync_keys_follow_parameter_changes():
    """The attached engine is rebuilt when a force's parameters, cutoffs or the force
    set change, and only re-sent the integrator when dt / kT / gamma change (the keys
    are plain Python; nothing here touches the device)."""
    from oxdna import io, runtime
    from oxdna.model import dna1, dna2
    forces, _ = dna2.forces()
    sim = runtime.Simulation(device=runtime.device.GPU(), seed=3)
    sim.create_state_from_snapshot(io.system_snapshot(io.duplex_system(1, 8, 20.0)))
    lang = runtime.md.methods.Langevin(filter=runtime.filter.All(), kT=dna1.kT_from_temperature(300))
    sim.operations.integrator = runtime.md.Integrator(dt=0.003, integrate_rotational_dof=True,
                                                      forces=forces, methods=[lang])
    sim._langevin = lang
    k0, i0 = sim._forces_key(), sim._integ_key()
    assert sim._forces_key() == k0
    hb = forces[2]
    hb.params[("A", "T")] = dict(hb.params[("A", "T")], eps=1.0)
    k1 = sim._forces_key()
    assert k1 != k0
    forces[1].r_cut[("A", "A")] = dict(r_cut=1.9)
    assert sim._forces_key() != k1
    assert sim._integ_key() == i0
    k2 = sim._forces_key()
    from oxdna import forces as F
    c0 = F._changes[0]
    lang.kT = 0.2
    assert F._changes[0] > c0  # the cheap test run() makes first
    assert sim._integ_key() != i0 and sim._forces_key() == k2
    c1 = F._changes[0]
    sim.operations.integrator.forces.append(dna2.debye_huckel(forces[1].nlist))
    assert F._changes[0] > c1
    assert sim._forces_key()[1] != k1[1]


def test_header_is_plain_c99_and_cxx(tmp_path):
    """include/oxdna_gb300.h compiles as strict C99 and as C++17 with every entry point
    it declares referenced: what a cgo, N-API or ctypes binding author includes."""
    import shutil
    import subprocess
    names = _header_functions()
    src = tmp_path / "use_header.c"
    src.write_text('#include "oxdna_gb300.h"\n'
                   "typedef void (*fn)(void);\n"
                   "fn table[] = {" + ", ".join(f"(fn){n}" for n in names) + "};\n"
                   "int main(void) { return table[0] == 0; }\n")
    inc = os.path.join(ROOT, "include")
    for cmd in (["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-fsyntax-only"],
                ["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-x", "c++"]):
        if shutil.which(cmd[0]) is None:
            pytest.skip(f"{cmd[0]} not available")
        out = subprocess.run(cmd + ["-I", inc, str(src)], capture_output=True, text=True)
        assert out.returncode == 0, out.stderr


def test_no_cpu_fallback_without_a_gpu():
    """Without a CUDA device the product path fails loudly: the native context cannot
    be created and run() raises the library's CUDA error instead of computing on the
    host (there is no CPU path); a CPU device is refused outright."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from oxdna import _abi, io, runtime
    from oxdna.model import dna1, dna2
    with pytest.raises(RuntimeError, match="GPU only"):
        runtime.device.CPU()
    forces, _ = dna2.forces()
    sim = runtime.Simulation(device=runtime.device.GPU(), seed=1)
    sim.create_state_from_snapshot(io.system_snapshot(io.duplex_system(1, 6, 20.0)))
    lang = runtime.md.methods.Langevin(filter=runtime.filter.All(), kT=dna1.kT_from_temperature(300))
    sim.operations.integrator = runtime.md.Integrator(dt=0.003, integrate_rotational_dof=True,
                                                      forces=forces, methods=[lang])
    with pytest.raises(_abi.OxgError) as err:
        sim.run(10)
    assert err.value.code == 2 and "CUDA" in str(err.value)
    with pytest.raises(RuntimeError, match="not attached"):
        forces[1].energy


def test_langevin_gamma_r_checked_on_every_assignment():
    """default_gamma_r is normalised and checked when assigned after construction too:
    the engine takes one isotropic rotational drag coefficient."""
    from oxdna import runtime
    lang = runtime.md.methods.Langevin(filter=runtime.filter.All(), kT=0.1)
    assert lang.default_gamma_r == (1.0, 1.0, 1.0)
    lang.default_gamma_r = 2
    assert lang.default_gamma_r == (2.0, 2.0, 2.0)
    lang.default_gamma_r = [3, 3, 3]
    assert lang.default_gamma_r == (3.0, 3.0, 3.0)
    with pytest.raises(ValueError, match="anisotropic"):
        lang.default_gamma_r = (1, 2, 3)
    with pytest.raises(ValueError, match="3 components"):
        lang.default_gamma_r = (1, 1)
    assert lang.default_gamma_r == (3.0, 3.0, 3.0)
    with pytest.raises(ValueError, match="anisotropic"):
        runtime.md.methods.Langevin(filter=runtime.filter.All(), kT=0.1, default_gamma_r=(1, 1, 2))


def test_non_unit_moment_of_inertia_is_refused():
    """The engine integrates rotations with unit moments of inertia (the value the oxDNA
    builders set); a snapshot with other values is refused, not silently ignored."""
    from oxdna import io, runtime
    s = io.duplex_system(2, 8, 20.0, seed=1)
    snap = io.system_snapshot(s)
    sim = runtime.Simulation(device=runtime.device.GPU())
    sim.create_state_from_snapshot(snap)
    sim._state_arrays()  # unit inertia: accepted
    snap.particles.moment_inertia[3] = (1.0, 2.0, 1.0)
    with pytest.raises(ValueError, match="moment_inertia"):
        sim._state_arrays()
