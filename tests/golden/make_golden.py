"""Generate the golden fixtures in tests/golden/ from the REFERENCE's own evaluator
and bonded headers (compiled unchanged into oracle/_ref by oracle/build.py).

    python tests/golden/make_golden.py

Needs the reference source tree (only on the development machine); the fixtures it
writes are committed so that the tests run anywhere. Contents:

* ``pairs_<model>.npz``  per-pair inputs (dr, q_i, q_j, types, charges) and the
  reference's FP64 and FP32 outputs (evaluated flag, force on i, energy, torques)
  for every nonbonded term of oxDNA1 / oxDNA2 / oxRNA2, sampled from the 320-nt
  8 x 20-bp duplex system (ideal and perturbed geometries, bonded neighbours
  included so stacking-like geometries exercise coaxial stacking).
* ``bonds_<model>.npz``  per-bond inputs and FP64/FP32 outputs of
  oxdna_bonded_pair (FENE, bonded excluded volume, DNA/RNA stacking), sequence-
  averaged and sequence-dependent, including stretched and broken bonds.
* ``pairs_<model>_seq.npz``  as ``pairs_<model>.npz`` for the sequence-dependent
  parameters (average=False) of the two terms that have them: hydrogen bonding and
  fused HB + cross-stacking (per-type-pair eps).
* ``system_dna2.npz``  per-term energies, per-particle forces and torques of the
  perturbed 320-nt oxDNA2 system, summed from reference per-pair calls with the
  HOOMD driver semantics (all unordered non-bonded pairs, dr = r_i - r_j minimum
  image, F_j = -F_i, torque_j from the evaluator; bonds scattered to both ends).
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "hoomd-oxdna_gb300"))

from oracle import oracle as O  # noqa: E402
from oxdna import _abi, io  # noqa: E402
from oxdna.model import dna1, dna2, rna2  # noqa: E402

SEED = 20261203
BOX = 40.0


def model_forces(name, average=True):
    """Pair forces (all six terms) and the bonded force for a model variant."""
    mod = {"dna1": dna1, "dna2": dna2, "rna2": rna2}[name]
    nl = mod.make_neighbor_list()
    if name == "rna2":
        pair = [rna2.excluded_volume(nl), rna2.hydrogen_bonding(nl, average=average),
                rna2.cross_stacking(nl), None, rna2.coaxial_stacking(nl),
                rna2.debye_huckel(nl)]
        # the fused term is not part of oxRNA2; take the DNA one for coverage
        pair[3] = dna2.hbond_cross(nl, average=average)
        bonded = rna2.bonded_force(average=average)
    else:
        pair = [mod.excluded_volume(nl), mod.hydrogen_bonding(nl, average=average),
                mod.cross_stacking(nl) if name == "dna1" else dna1.cross_stacking(nl),
                mod.hbond_cross(nl, average=average), mod.coaxial_stacking(nl),
                dna2.debye_huckel(nl)]
        bonded = mod.bonded_force(average=average)
    return pair, bonded


def perturbed(sysarr, rng, sigma_x, sigma_a):
    pos = sysarr["pos"] + rng.normal(0, sigma_x, sysarr["pos"].shape)
    q = sysarr["quat"].copy()
    for k in range(len(q)):
        ax = rng.normal(size=3)
        ax /= np.linalg.norm(ax)
        ang = rng.normal(0, sigma_a)
        dq = np.concatenate([[np.cos(ang / 2)], np.sin(ang / 2) * ax])
        w1, x1, y1, z1 = dq
        w2, x2, y2, z2 = q[k]
        q[k] = [w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2, w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
                w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2, w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2]
        q[k] /= np.linalg.norm(q[k])
    return pos, q


def min_image(d, L=BOX):
    return d - L * np.round(d / L)


def pair_samples(name, rng, average=True, terms=range(6)):
    pair, _ = model_forces(name, average=average)
    base = io.duplex_system(8, 20, BOX, seed=1)
    geoms = [(base["pos"], base["quat"])]
    for sx, sa in ((0.03, 0.05), (0.08, 0.15), (0.15, 0.3)):
        geoms.append(perturbed(base, rng, sx, sa))
    ty = base["typeid"]
    charges = np.where(base["ends"], 0.5, 1.0)
    r64, r32 = O.ref_lib(64), O.ref_lib(32)
    out = {}
    for t in terms:
        f = pair[t]
        rows = []
        for gi, (pos, q) in enumerate(geoms):
            cand = []
            for i in range(len(pos)):
                d = min_image(pos[i] - pos)
                r2 = np.einsum("ij,ij->i", d, d)
                for j in np.nonzero(r2 < (f.default_r_cut * 1.02) ** 2)[0]:
                    if j != i:
                        cand.append((i, int(j)))
            rng.shuffle(cand)
            nz, z = [], []
            for i, j in cand:
                key = (io.DNA_BASES[ty[i]], io.DNA_BASES[ty[j]])
                p = _abi.FROM_DICT[t](f.params[key])
                rc = f.rcut_for(*key)
                d = min_image(pos[i] - pos[j])
                res64 = O.eval_pair(r64, "ref", t, p, d, q[i], q[j], rc * rc, charges[i], charges[j])
                (nz if res64[2] != 0.0 else z).append((i, j, d, res64))
                if len(nz) >= 80 and len(z) >= 15:
                    break
            for i, j, d, res64 in nz[:80] + z[:15]:
                key = (io.DNA_BASES[ty[i]], io.DNA_BASES[ty[j]])
                p = _abi.FROM_DICT[t](f.params[key])
                rc = f.rcut_for(*key)
                res32 = O.eval_pair(r32, "ref", t, p, d, q[i], q[j], rc * rc, charges[i], charges[j])
                rows.append((d, q[i], q[j], ty[i], ty[j], charges[i], charges[j], rc * rc,
                             res64, res32))
        def col(k):
            return np.array([r[k] for r in rows])
        pre = _abi.TERM_NAMES[t]
        out[pre + "/dr"] = col(0)
        out[pre + "/qi"] = col(1)
        out[pre + "/qj"] = col(2)
        out[pre + "/types"] = np.stack([col(3), col(4)], 1).astype(np.int32)
        out[pre + "/charges"] = np.stack([col(5), col(6)], 1)
        out[pre + "/rcutsq"] = col(7)
        for tag, k in (("ref64", 8), ("ref32", 9)):
            out[f"{pre}/{tag}/flag"] = np.array([r[k][0] for r in rows], np.int8)
            out[f"{pre}/{tag}/force"] = np.array([r[k][1] for r in rows])
            out[f"{pre}/{tag}/energy"] = np.array([r[k][2] for r in rows])
            out[f"{pre}/{tag}/torque_i"] = np.array([r[k][3] for r in rows])
            out[f"{pre}/{tag}/torque_j"] = np.array([r[k][4] for r in rows])
    return out


def bond_samples(name, rng):
    out = {}
    base = io.duplex_system(8, 20, BOX, seed=1)
    r64, r32 = O.ref_lib(64), O.ref_lib(32)
    for avg in (True, False):
        _, bonded = model_forces(name, average=avg)
        p = _abi.bonded_from_dict(bonded.params["backbone"])
        rows = []
        geoms = [(base["pos"], base["quat"])]
        for sx, sa in ((0.02, 0.05), (0.05, 0.15), (0.1, 0.3)):
            geoms.append(perturbed(base, rng, sx, sa))
        for pos, q in geoms:
            for A, B in base["bonds"][::5]:
                Rc = min_image(pos[B] - pos[A])
                rows.append((Rc, q[A], q[B], base["typeid"][A], base["typeid"][B]))
        # stretched (near the FENE limit) and broken bonds
        for A, B in base["bonds"][:6]:
            for stretch in (0.2, 0.24, 0.3):
                Rc = min_image(base["pos"][B] - base["pos"][A])
                Rc = Rc * (1.0 + stretch / np.linalg.norm(Rc))
                rows.append((Rc, base["quat"][A], base["quat"][B], base["typeid"][A],
                             base["typeid"][B]))
        tag = "avg" if avg else "seq"
        out[f"{tag}/Rc"] = np.array([r[0] for r in rows])
        out[f"{tag}/qA"] = np.array([r[1] for r in rows])
        out[f"{tag}/qB"] = np.array([r[2] for r in rows])
        out[f"{tag}/types"] = np.array([[r[3], r[4]] for r in rows], np.int32)
        for lab, lib in (("ref64", r64), ("ref32", r32)):
            res = [O.eval_bonded(lib, "ref", p, *r) for r in rows]
            for k, fld in enumerate(("FB", "tauA", "tauB", "energy", "virial")):
                out[f"{tag}/{lab}/{fld}"] = np.array([x[k] for x in res])
    return out


def system_golden(rng):
    """Perturbed 320-nt oxDNA2 system: per-term totals and per-particle arrays."""
    base = io.duplex_system(8, 20, BOX, seed=1)
    pos, q = perturbed(base, rng, 0.03, 0.08)
    ty = base["typeid"]
    charges = np.where(base["ends"], 0.5, 1.0)
    n = len(pos)
    bonded_set = {(min(a, b), max(a, b)) for a, b in base["bonds"]}
    pair, bonded = model_forces("dna2")
    r64 = O.ref_lib(64)
    out = dict(pos=pos, quat=q, typeid=ty, charge=charges, box=np.array([BOX] * 3),
               bonds=np.array(base["bonds"], np.int32))
    for t in range(6):
        f = pair[t]
        F = np.zeros((n, 3))
        T = np.zeros((n, 3))
        Epp = np.zeros(n)
        Etot = 0.0
        for i in range(n):
            d_all = min_image(pos[i] - pos)
            r2 = np.einsum("ij,ij->i", d_all, d_all)
            for j in np.nonzero(r2 < f.default_r_cut ** 2 * 1.0001)[0]:
                j = int(j)
                if j <= i or (i, j) in bonded_set:
                    continue
                key = (io.DNA_BASES[ty[i]], io.DNA_BASES[ty[j]])
                p = _abi.FROM_DICT[t](f.params[key])
                rc = f.rcut_for(*key)
                ok, fi, e, ti, tj = O.eval_pair(r64, "ref", t, p, d_all[j], q[i], q[j], rc * rc,
                                                charges[i], charges[j])
                if not ok:
                    continue
                F[i] += fi
                F[j] -= fi
                T[i] += ti
                T[j] += tj
                Epp[i] += 0.5 * e
                Epp[j] += 0.5 * e
                Etot += e
        pre = _abi.TERM_NAMES[t]
        out[pre + "/force"] = F
        out[pre + "/torque"] = T
        out[pre + "/energy_pp"] = Epp
        out[pre + "/energy"] = np.array(Etot)
    p = _abi.bonded_from_dict(bonded.params["backbone"])
    F = np.zeros((n, 3))
    T = np.zeros((n, 3))
    E = np.zeros(3)
    for A, B in base["bonds"]:
        FB, tA, tB, e, _ = O.eval_bonded(r64, "ref", p, min_image(pos[B] - pos[A]), q[A], q[B],
                                         ty[A], ty[B])
        F[A] -= FB
        F[B] += FB
        T[A] += tA
        T[B] += tB
        E += e
    out["bonded/force"] = F
    out["bonded/torque"] = T
    out["bonded/energy"] = E
    return out


def main():
    if O.ref_lib(64) is None:
        sys.exit("reference tree not available: cannot regenerate golden fixtures")
    rng = np.random.default_rng(SEED)
    for name in ("dna1", "dna2", "rna2"):
        np.savez_compressed(os.path.join(HERE, f"pairs_{name}.npz"), **pair_samples(name, rng))
        np.savez_compressed(os.path.join(HERE, f"bonds_{name}.npz"), **bond_samples(name, rng))
    np.savez_compressed(os.path.join(HERE, "system_dna2.npz"), **system_golden(rng))
    # sequence-dependent hydrogen bonding (per-type-pair eps): the HB and fused HB +
    # cross-stacking terms with average=False, from a stream of their own so the
    # fixtures above do not change
    rng_seq = np.random.default_rng(SEED + 1)
    for name in ("dna1", "dna2", "rna2"):
        np.savez_compressed(os.path.join(HERE, f"pairs_{name}_seq.npz"),
                            **pair_samples(name, rng_seq, average=False, terms=(1, 3)))
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
