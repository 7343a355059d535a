"""Physics properties of the oracle, following the reference's own test logic
(pytest/_helpers.py:137-181 finite differences and Newton's third law,
pytest/test_fused.py fused == separate, pytest/test_oxdna2.py:72-80 stability)."""

import numpy as np
import pytest

from _util import TERMS, golden, model_forces


def _quat_mul(a, b):
    w1, x1, y1, z1 = a
    w2, x2, y2, z2 = b
    return np.array([w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2, w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
                     w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2, w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2])


def _system(oracle):
    g = golden("system_dna2.npz")
    return g, g["pos"].copy(), g["quat"].copy()


def _fd_check(oracle, model, g, pos, quat, mask, use_bonded, label):
    """Forces and torques against central differences of the energy for the three
    most-forced particles (displacements along x, y, z; rotations about x, y, z)."""
    def run(p, q):
        s = oracle.System(p, q, g["typeid"], g["box"], g["bonds"], g["charge"])
        r = oracle.forces(model, s, mask=mask, bonded=use_bonded)
        e = r["bonded_energy"].sum() if use_bonded else r["pair_energy"].sum()
        return e, r

    e0, r0 = run(pos, quat)
    F, T = r0["force"], r0["torque"]
    if np.abs(F).max() == 0.0:
        pytest.skip(f"{label} is zero on this configuration")
    # Newton's third law (_helpers.py:156-157)
    assert np.linalg.norm(F.sum(axis=0)) < 1e-9 * (1 + np.abs(F).max())
    for i in np.argsort(-np.linalg.norm(F, axis=1))[:3]:
        h = 1e-6
        for d in range(3):
            pp = pos.copy()
            pp[i, d] += h
            ep = run(pp, quat)[0]
            pp[i, d] -= 2 * h
            em = run(pp, quat)[0]
            assert abs(-(ep - em) / (2 * h) - F[i, d]) < 1e-5 * max(1.0, abs(F[i, d]))
        for k, axis in enumerate(np.eye(3)):
            qp = quat.copy()
            qp[i] = _quat_mul(np.r_[np.cos(h / 2), np.sin(h / 2) * axis], quat[i])
            ep = run(pos, qp)[0]
            qp[i] = _quat_mul(np.r_[np.cos(-h / 2), np.sin(-h / 2) * axis], quat[i])
            em = run(pos, qp)[0]
            assert abs(-(ep - em) / (2 * h) - T[i, k]) < 1e-5 * max(1.0, abs(T[i, k]))
    return e0


@pytest.mark.parametrize("what", [t for t in TERMS if t != "oxdna_coaxstacking"] + ["bonded"])
def test_finite_difference_force_and_torque(oracle, what):
    from oxdna import io
    g, pos, quat = _system(oracle)
    pair, bonded = model_forces("dna2")
    model = oracle.Model(pair + [bonded], io.DNA_BASES)
    mask = 0 if what == "bonded" else 1 << TERMS.index(what)
    _fd_check(oracle, model, g, pos, quat, mask, what == "bonded", what)


@pytest.mark.parametrize("model_name", ["dna1", "dna2", "rna2"])
def test_finite_difference_coax_on_nicked_duplex(oracle, model_name):
    """Coaxial stacking, which is zero inside an intact duplex: a 20-bp duplex whose
    first strand is nicked between nucleotides 9 and 10 (no backbone bond, so the pair
    is no longer excluded and the two stack coaxially); the reference checks the same
    term on its two-duplex simple-coax case (pytest/test_coaxstacking.py:26-31,
    pytest/test_rna2.py:86-145). Positions and orientations are perturbed: in the ideal
    helix the a3 axes of a strand are exactly parallel, theta4 = 0, a cone point of the
    oxRNA2 theta4 factor (its theta0 is 0.151), where the energy has no derivative."""
    from oxdna import io
    s = io.duplex_system(1, 20, 30.0, seed=7)
    g = dict(typeid=s["typeid"], box=s["box"], charge=s["charge"],
             bonds=[b for b in s["bonds"] if b != (9, 10)])
    rng = np.random.default_rng(2)
    pos = s["pos"] + rng.normal(0, 0.02, s["pos"].shape)
    quat = s["quat"].copy()
    for k in range(len(quat)):
        ax = rng.normal(size=3)
        ang = rng.normal(0, 0.05)
        quat[k] = _quat_mul(np.r_[np.cos(ang / 2), np.sin(ang / 2) * ax / np.linalg.norm(ax)], quat[k])
    pair, bonded = model_forces(model_name)
    model = oracle.Model(pair + [bonded], io.DNA_BASES)
    e = _fd_check(oracle, model, g, pos, quat, 1 << TERMS.index("oxdna_coaxstacking"), False, "coax")
    assert e < -0.1  # the nick's neighbours are stacked


@pytest.mark.parametrize("model_name", ["dna1", "dna2"])
def test_fused_equals_separate(oracle, model_name):
    from oxdna import io
    g, pos, quat = _system(oracle)
    pair, _ = model_forces(model_name)
    model = oracle.Model(pair, io.DNA_BASES)
    s = oracle.System(pos, quat, g["typeid"], g["box"], g["bonds"], g["charge"])
    sep = oracle.forces(model, s, mask=(1 << 1) | (1 << 2), bonded=False)
    fus = oracle.forces(model, s, mask=1 << 3, bonded=False)
    assert abs(sep["pair_energy"][1] + sep["pair_energy"][2] - fus["pair_energy"][3]) < 1e-10
    assert np.abs(sep["force"] - fus["force"]).max() < 1e-10
    assert np.abs(sep["torque"] - fus["torque"]).max() < 1e-10


def test_duplex_stays_bound_under_langevin(oracle):
    """pytest/test_oxdna2.py:72-80 on the oracle: 8 x 20-bp duplexes, 1000 steps."""
    from oxdna import io
    from oxdna.model import dna1, dna2
    sysa = io.duplex_system(8, 20, 40.0, seed=1)
    forces, _ = dna2.forces()
    model = oracle.Model(forces, io.DNA_BASES)
    s = oracle.System(sysa["pos"], sysa["quat"], sysa["typeid"], sysa["box"], sysa["bonds"])
    n = len(sysa["pos"])
    vel = np.zeros((n, 3))
    am = np.zeros((n, 4))
    builds, vel, am = oracle.langevin(model, s, vel, am, steps=1000, dt=0.003,
                                      kT=dna1.kT_from_temperature(296.15), seed=5)
    assert builds >= 1
    assert np.isfinite(s.pos).all()
    r = oracle.forces(model, s)
    assert r["pair_energy"][1] / n < -0.15
    assert r["bonded_energy"][0] < 1e11  # no broken bond


def test_philox_known_answer(oracle):
    """Philox4x32-10 known-answer vectors (Random123 distribution, kat_vectors)."""
    import ctypes as C
    L = oracle.oracle_lib()
    cases = [((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
             ((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
             ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
              (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]
    for ctr, key, want in cases:
        c = (C.c_uint32 * 4)(*ctr)
        k = (C.c_uint32 * 2)(*key)
        o = (C.c_uint32 * 4)()
        L.oxo_philox4x32(c, k, o)
        assert tuple(o) == want
