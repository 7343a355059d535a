"""GPU parity: the FP32 sm_103a kernels against the reference (golden fixtures made
from the reference's own headers) and against the FP64 oracle.

Tolerance (TOL_GPU = 1e-4): set-level max-norm relative error per term,
max|x - x_ref| / max|x_ref| over all samples, for energies, forces and torques.
"""

import ctypes as C

import numpy as np
import pytest

from _util import PAIR_CASES, TERMS, TOL_GPU, golden, maxrel, model_forces, pair_golden

pytestmark = pytest.mark.gpu
MODELS = ("dna1", "dna2", "rna2")


def _sim(snap, forces):
    from oxdna import runtime
    sim = runtime.Simulation(device=runtime.device.GPU())
    sim.create_state_from_snapshot(snap)
    sim.operations.integrator = runtime.md.Integrator(dt=0.0, integrate_rotational_dof=True,
                                                      forces=list(forces))
    sim.run(0)
    return sim


def _pair_snapshot(dr, qi, qj, types, charges, spacing=12.0):
    """Two particles per sample (i at a grid site, j at site - dr), far apart."""
    from oxdna import io
    n = len(dr)
    side = int(np.ceil(n ** (1 / 3)))
    L = side * spacing
    g = np.array([(a, b, c) for a in range(side) for b in range(side) for c in range(side)])[:n]
    xi = (g + 0.5) * spacing - L / 2
    pos = np.empty((2 * n, 3))
    pos[0::2] = xi
    pos[1::2] = xi - dr
    q = np.empty((2 * n, 4))
    q[0::2] = qi
    q[1::2] = qj
    ty = np.empty(2 * n, int)
    ty[0::2] = types[:, 0]
    ty[1::2] = types[:, 1]
    ch = np.empty(2 * n)
    ch[0::2] = charges[:, 0]
    ch[1::2] = charges[:, 1]
    return io.snapshot_from_arrays(pos, q, ty, [L, L, L], charges=ch)


@pytest.mark.parametrize("model,term,avg", PAIR_CASES)
def test_engine_pair_terms_match_reference(native, model, term, avg):
    d = pair_golden(model, avg)
    name = TERMS[term]
    f = model_forces(model, average=(avg == "avg"))[0][term]
    snap = _pair_snapshot(d[name + "/dr"], d[name + "/qi"], d[name + "/qj"], d[name + "/types"],
                          d[name + "/charges"])
    sim = _sim(snap, [f])
    F, T, Epp = sim._force_arrays(f)
    assert maxrel(F[0::2], d[name + "/ref64/force"]) < TOL_GPU
    assert maxrel(F[1::2], -d[name + "/ref64/force"]) < TOL_GPU
    assert maxrel(T[0::2], d[name + "/ref64/torque_i"]) < TOL_GPU
    assert maxrel(T[1::2], d[name + "/ref64/torque_j"]) < TOL_GPU
    assert maxrel(2.0 * Epp[0::2], d[name + "/ref64/energy"]) < TOL_GPU
    e = d[name + "/ref64/energy"].sum()
    assert abs(f.energy - e) <= TOL_GPU * np.abs(d[name + "/ref64/energy"]).sum()


@pytest.mark.parametrize("model", MODELS)
@pytest.mark.parametrize("avg", ("avg", "seq"))
def test_engine_bonded_matches_reference(native, model, avg):
    from oxdna import io
    d = golden(f"bonds_{model}.npz")
    _, bonded = model_forces(model, average=(avg == "avg"))
    e_ref = d[f"{avg}/ref64/energy"]
    ok = e_ref[:, 0] < 1e12
    Rc, qA, qB, ty = (d[f"{avg}/{k}"] for k in ("Rc", "qA", "qB", "types"))
    n = len(Rc)
    spacing = 10.0
    side = int(np.ceil(n ** (1 / 3)))
    L = side * spacing
    g = np.array([(a, b, c) for a in range(side) for b in range(side) for c in range(side)])[:n]
    xa = (g + 0.5) * spacing - L / 2
    pos = np.empty((2 * n, 3))
    pos[0::2] = xa
    pos[1::2] = xa + Rc
    q = np.empty((2 * n, 4))
    q[0::2] = qA
    q[1::2] = qB
    types = np.empty(2 * n, int)
    types[0::2] = ty[:, 0]
    types[1::2] = ty[:, 1]
    snap = io.snapshot_from_arrays(pos, q, types, [L] * 3, bonds=[(2 * k, 2 * k + 1) for k in range(n)])
    sim = _sim(snap, [bonded])
    F, T, _ = sim._force_arrays(bonded)
    assert maxrel(F[1::2][ok], d[f"{avg}/ref64/FB"][ok]) < TOL_GPU
    assert maxrel(F[0::2][ok], -d[f"{avg}/ref64/FB"][ok]) < TOL_GPU
    assert maxrel(T[0::2][ok], d[f"{avg}/ref64/tauA"][ok]) < TOL_GPU
    assert maxrel(T[1::2][ok], d[f"{avg}/ref64/tauB"][ok]) < TOL_GPU
    # broken bonds: energy clamp 1e12 (FP64 on the GPU), no FENE force
    nb = int((~ok).sum())
    assert abs(bonded.fene_energy - (1e12 * nb + e_ref[ok, 0].sum())) <= 1e-3 * max(1, nb) + \
        TOL_GPU * np.abs(e_ref[ok, 0]).sum()
    assert abs(bonded.bonded_excvol_energy - e_ref[:, 1].sum()) <= TOL_GPU * max(1e-6, np.abs(e_ref[:, 1]).sum())
    assert abs(bonded.stacking_energy - e_ref[:, 2].sum()) <= TOL_GPU * np.abs(e_ref[:, 2]).sum()
    assert np.isfinite(F).all() and np.isfinite(T).all()


def test_engine_system_matches_reference(native):
    """Perturbed 320-nt oxDNA2 system, every term, per-particle arrays and totals."""
    from oxdna import io
    g = golden("system_dna2.npz")
    pair, bonded = model_forces("dna2")
    snap = io.snapshot_from_arrays(g["pos"], g["quat"], g["typeid"], g["box"],
                                   bonds=[tuple(b) for b in g["bonds"]], charges=g["charge"])
    forces = [bonded, pair[0], pair[1], pair[2], pair[4], pair[5]]
    sim = _sim(snap, forces)
    for t in (0, 1, 2, 4, 5):
        name = TERMS[t]
        F, T, Epp = sim._force_arrays(pair[t])
        assert maxrel(F, g[name + "/force"]) < TOL_GPU, name
        assert maxrel(T, g[name + "/torque"]) < TOL_GPU, name
        ref = float(g[name + "/energy"])
        assert abs(pair[t].energy - ref) <= TOL_GPU * max(abs(ref), 1e-6), name
    F, T, _ = sim._force_arrays(bonded)
    assert maxrel(F, g["bonded/force"]) < TOL_GPU
    assert maxrel(T, g["bonded/torque"]) < TOL_GPU
    for k, fld in enumerate(("fene_energy", "bonded_excvol_energy", "stacking_energy")):
        ref = g["bonded/energy"][k]
        assert abs(getattr(bonded, fld) - ref) <= TOL_GPU * max(abs(ref), 1e-6), fld
    # fused HB + cross-stacking equals the separate pair (pytest/test_fused.py:9-40)
    sim2 = _sim(snap, [pair[3]])
    assert abs(pair[3].energy - (pair[1].energy + pair[2].energy)) < 1e-5 * len(g["pos"])


def _full_nlist(pos, box, rc, bonds):
    n = len(pos)
    excl = {(a, b) for a, b in bonds} | {(b, a) for a, b in bonds}
    nbrs = []
    for i in range(n):
        d = pos[i] - pos
        d -= box * np.round(d / box)
        r2 = np.einsum("ij,ij->i", d, d)
        js = [int(j) for j in np.nonzero(r2 < rc * rc)[0] if j != i and (i, int(j)) not in excl]
        nbrs.append(js)
    n_neigh = np.array([len(x) for x in nbrs], np.uint32)
    head = np.concatenate([[0], np.cumsum(n_neigh)[:-1]]).astype(np.uint64)
    flat = np.array([j for x in nbrs for j in x], np.uint32)
    return n_neigh, flat, head


def test_dropin_full_nlist_and_bonds(native, oracle):
    """Evaluator-level entry points with HOOMD Scalar4 (double) device arrays."""
    import torch
    from oxdna import _abi, io
    g = golden("system_dna2.npz")
    pair, bonded = model_forces("dna2")
    n = len(g["pos"])
    L = native
    ctx = C.c_void_p()
    _abi.check(L.oxg_create(C.byref(ctx), 4, 1), "create")
    setters = [L.oxg_set_excvol_params, L.oxg_set_hbond_params, L.oxg_set_cross_params,
               L.oxg_set_hbondcross_params, L.oxg_set_coax_params, L.oxg_set_debye_params]
    for t, f in enumerate(pair):
        for a in range(4):
            for b in range(a, 4):
                key = (io.DNA_BASES[a], io.DNA_BASES[b])
                p = _abi.FROM_DICT[t](f.params[key])
                _abi.check(setters[t](ctx, a, b, C.byref(p), f.rcut_for(*key)), "set")
    bp = _abi.bonded_from_dict(bonded.params["backbone"])
    _abi.check(L.oxg_set_bonded_params(ctx, 0, C.byref(bp)), "set bonded")
    dev = torch.device("cuda")
    pt = np.zeros((n, 4))
    pt[:, :3] = g["pos"]
    pt[:, 3] = g["typeid"].astype(np.int64).view(np.float64)  # low word = type
    pos_d = torch.tensor(pt, dtype=torch.float64, device=dev)
    quat_d = torch.tensor(g["quat"], dtype=torch.float64, device=dev)
    ch_d = torch.tensor(g["charge"], dtype=torch.float64, device=dev)
    rmax = max(f.default_r_cut for f in pair)
    nn, flat, head = _full_nlist(g["pos"], g["box"], rmax + 0.2, [tuple(b) for b in g["bonds"]])
    nn_d = torch.tensor(nn.astype(np.int64), device=dev).to(torch.int32)
    fl_d = torch.tensor(flat.astype(np.int64), device=dev).to(torch.int32)
    hd_d = torch.tensor(head.astype(np.int64), device=dev)
    box = (C.c_float * 3)(*g["box"].astype(float))
    model = oracle.Model(pair, io.DNA_BASES)
    ptr = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    for t in (0, 1, 2, 3, 4, 5):
        force = torch.zeros((n, 4), dtype=torch.float32, device=dev)
        torque = torch.zeros((n, 4), dtype=torch.float32, device=dev)
        virial = torch.zeros((6, n), dtype=torch.float32, device=dev)
        energy = torch.zeros(6, dtype=torch.float64, device=dev)
        _abi.check(L.oxg_pair_forces(ctx, 1 << t, n, ptr(pos_d), ptr(quat_d), ptr(ch_d), box,
                                     ptr(nn_d), ptr(fl_d), ptr(hd_d), ptr(force), ptr(torque),
                                     ptr(virial), ptr(energy), None), "pair_forces")
        _abi.check(L.oxg_context_status(ctx, 1), "status")
        # oracle with the full-list semantics: particle i gets sum_j eval(i, j), and
        # HOOMD's pair virial W_i = sum_j 0.5 * dr_ij (x) F_i (xx, xy, xz, yy, yz, zz)
        Fo = np.zeros((n, 3))
        To = np.zeros((n, 3))
        Vo = np.zeros((6, n))
        Eo = 0.0
        f = pair[t]
        for i in range(n):
            for j in flat[head[i]:head[i] + nn[i]]:
                d = g["pos"][i] - g["pos"][j]
                d -= g["box"] * np.round(d / g["box"])
                key = (io.DNA_BASES[g["typeid"][i]], io.DNA_BASES[g["typeid"][j]])
                p = _abi.FROM_DICT[t](f.params[key])
                ok, fi, e, ti, _ = oracle.eval_pair(oracle.oracle_lib(), "oxo", t, p, d,
                                                    g["quat"][i], g["quat"][j],
                                                    f.rcut_for(*key) ** 2, g["charge"][i],
                                                    g["charge"][j])
                Fo[i] += fi
                To[i] += ti
                Vo[:, i] += 0.5 * np.array([d[0] * fi[0], d[0] * fi[1], d[0] * fi[2],
                                            d[1] * fi[1], d[1] * fi[2], d[2] * fi[2]])
                Eo += 0.5 * e
        Fg = force.cpu().numpy()
        Tg = torque.cpu().numpy()
        if np.abs(Fo).max() > 0:
            assert maxrel(Fg[:, :3], Fo) < TOL_GPU, TERMS[t]
            assert maxrel(Tg[:, :3], To) < TOL_GPU, TERMS[t]
            assert maxrel(virial.cpu().numpy(), Vo) < TOL_GPU, TERMS[t]
        assert abs(energy[t].item() - Eo) <= TOL_GPU * max(abs(Eo), 1e-6), TERMS[t]
    # bonded drop-in
    bonds = torch.tensor(np.c_[g["bonds"], np.zeros(len(g["bonds"]))].astype(np.int64),
                         device=dev).to(torch.int32)
    force = torch.zeros((n, 4), dtype=torch.float32, device=dev)
    torque = torch.zeros((n, 4), dtype=torch.float32, device=dev)
    virial = torch.zeros((6, n), dtype=torch.float32, device=dev)
    split = torch.zeros(3, dtype=torch.float64, device=dev)
    _abi.check(L.oxg_bonded_forces(ctx, n, ptr(pos_d), ptr(quat_d), box, len(g["bonds"]),
                                   ptr(bonds), ptr(force), ptr(torque), ptr(virial), ptr(split),
                                   None), "bonded_forces")
    _abi.check(L.oxg_context_status(ctx, 1), "status")
    assert maxrel(force.cpu().numpy()[:, :3], g["bonded/force"]) < TOL_GPU
    assert maxrel(torque.cpu().numpy()[:, :3], g["bonded/torque"]) < TOL_GPU
    assert maxrel(split.cpu().numpy(), g["bonded/energy"]) < TOL_GPU
    # the bonded half virial (reference OxDNABondedKernel.h:48-58, written to both ends
    # at OxDNABondedGPU.cu:120-121) from the oracle's bonded kernel, pinned to the
    # reference's own by tests/test_oracle_pin.py
    bp_o = _abi.bonded_from_dict(bonded.params["backbone"])
    Vb = np.zeros((6, n))
    for A, B in g["bonds"]:
        Rc = g["pos"][B] - g["pos"][A]
        Rc -= g["box"] * np.round(Rc / g["box"])
        vir = oracle.eval_bonded(oracle.oracle_lib(), "oxo", bp_o, Rc, g["quat"][A], g["quat"][B],
                                 g["typeid"][A], g["typeid"][B])[4]
        Vb[:, A] += vir
        Vb[:, B] += vir
    assert maxrel(virial.cpu().numpy(), Vb) < TOL_GPU
    # an out-of-range neighbour index is skipped and reported, not dereferenced
    bad = fl_d.clone()
    bad[0] = n + 5
    _abi.check(L.oxg_pair_forces(ctx, 1, n, ptr(pos_d), ptr(quat_d), ptr(ch_d), box, ptr(nn_d),
                                 ptr(bad), ptr(hd_d), ptr(force), ptr(torque), None, None, None),
               "pair_forces")
    assert L.oxg_context_status(ctx, 1) == _abi.ERR_BAD_INDEX
    # empty calls (no particles, no terms, no bonds) return at once and leave the
    # outputs as they were
    force.fill_(7.0)
    energy = torch.full((6,), 7.0, dtype=torch.float64, device=dev)
    for N_, mask in ((0, 0x3f), (n, 0)):
        _abi.check(L.oxg_pair_forces(ctx, mask, N_, ptr(pos_d), ptr(quat_d), ptr(ch_d), box,
                                     ptr(nn_d), ptr(fl_d), ptr(hd_d), ptr(force), ptr(torque),
                                     None, ptr(energy), None), "pair_forces (empty)")
    _abi.check(L.oxg_bonded_forces(ctx, n, ptr(pos_d), ptr(quat_d), box, 0, ptr(bonds),
                                   ptr(force), ptr(torque), None, ptr(split), None), "bonded (empty)")
    torch.cuda.synchronize()
    assert (force == 7.0).all() and (energy == 7.0).all()
    # a ragged list: every other particle keeps its neighbours (HOOMD's head offsets
    # unchanged, so the used runs are not contiguous), the rest have none; the
    # particles with neighbours get the oracle's full-list excluded-volume forces, the
    # others nothing
    keep = np.arange(n) % 2 == 0
    nn_r = np.where(keep, nn, 0).astype(np.int64)
    nn_rd = torch.tensor(nn_r, device=dev).to(torch.int32)
    force = torch.zeros((n, 4), dtype=torch.float32, device=dev)
    torque = torch.zeros((n, 4), dtype=torch.float32, device=dev)
    energy = torch.zeros(6, dtype=torch.float64, device=dev)
    _abi.check(L.oxg_pair_forces(ctx, 1, n, ptr(pos_d), ptr(quat_d), ptr(ch_d), box, ptr(nn_rd),
                                 ptr(fl_d), ptr(hd_d), ptr(force), ptr(torque), None, ptr(energy),
                                 None), "pair_forces (ragged)")
    _abi.check(L.oxg_context_status(ctx, 1), "status")
    Fo = np.zeros((n, 3))
    To = np.zeros((n, 3))
    Eo = 0.0
    f = pair[0]
    for i in np.nonzero(keep)[0]:
        for j in flat[head[i]:head[i] + nn[i]]:
            d = g["pos"][i] - g["pos"][j]
            d -= g["box"] * np.round(d / g["box"])
            key = (io.DNA_BASES[g["typeid"][i]], io.DNA_BASES[g["typeid"][j]])
            p = _abi.FROM_DICT[0](f.params[key])
            ok, fi, e, ti, _ = oracle.eval_pair(oracle.oracle_lib(), "oxo", 0, p, d, g["quat"][i],
                                                g["quat"][j], f.rcut_for(*key) ** 2,
                                                g["charge"][i], g["charge"][j])
            Fo[i] += fi
            To[i] += ti
            Eo += 0.5 * e
    assert np.abs(Fo).max() > 0
    Fg = force.cpu().numpy()
    assert maxrel(Fg[:, :3], Fo) < TOL_GPU
    assert maxrel(torque.cpu().numpy()[:, :3], To) < TOL_GPU
    assert not Fg[~keep].any()
    assert abs(energy[0].item() - Eo) <= TOL_GPU * max(abs(Eo), 1e-6)
    L.oxg_destroy(ctx)
