"""ctypes binding of the FP64 oracle (``liboxdna_oracle.so``) and of the reference-pin
libraries (``_ref/libref64.so``, ``_ref/libref32.so``).

TEST INFRASTRUCTURE ONLY: imported by the test suite, the smoke check and the
bench's CPU-baseline leg, never by the product package. Parameter structs are the
product's ABI structs (``oxdna._abi``), so the oracle is fed exactly the parameters
the GPU engine receives.
"""

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(REPO, "hoomd-oxdna_gb300"))

from oxdna import _abi  # noqa: E402

from . import build as _build  # noqa: E402

dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int32)


class OxoModel(C.Structure):
    _fields_ = [("n_types", C.c_int), ("n_bond_types", C.c_int),
                ("excvol", C.POINTER(_abi.ExcVolParams)), ("hbond", C.POINTER(_abi.HBondParams)),
                ("cross", C.POINTER(_abi.CrossParams)),
                ("hbondcross", C.POINTER(_abi.HBondCrossParams)),
                ("coax", C.POINTER(_abi.CoaxParams)), ("debye", C.POINTER(_abi.DebyeParams)),
                ("r_cut", dp * 6), ("bonded", C.POINTER(_abi.BondedParams))]


class OxoSystem(C.Structure):
    _fields_ = [("N", C.c_int), ("pos", dp), ("quat", dp), ("type", ip), ("charge", dp),
                ("box", C.c_double * 3), ("n_bonds", C.c_int), ("bonds", ip)]


_PAIR_FN = {_abi.EXCVOL: "excvol", _abi.HBOND: "hbond", _abi.CROSS: "cross",
            _abi.HBONDCROSS: "hbondcross", _abi.COAX: "coax", _abi.DEBYE: "debye"}


def _declare_pairs(L, prefix):
    for t, name in _PAIR_FN.items():
        fn = getattr(L, f"{prefix}_{name}")
        args = [C.POINTER(_abi.PARAM_STRUCTS[t]), dp, dp, dp, C.c_double]
        if t == _abi.DEBYE:
            args += [C.c_double, C.c_double]
        fn.argtypes = args + [dp, dp, dp, dp]
        fn.restype = C.c_int
    fn = getattr(L, f"{prefix}_bonded")
    fn.argtypes = [C.POINTER(_abi.BondedParams), dp, dp, dp, C.c_int, C.c_int, dp, dp, dp, dp, dp]
    fn.restype = None


_oracle = None
_refs = {}


def oracle_lib():
    global _oracle
    if _oracle is None:
        path = _build.build_oracle()
        L = C.CDLL(path)
        _declare_pairs(L, "oxo")
        L.oxo_forces.argtypes = [C.POINTER(OxoModel), C.POINTER(OxoSystem), C.c_uint32, C.c_int,
                                 C.c_int, dp, dp, dp, dp, C.POINTER(C.c_int64)]
        L.oxo_forces.restype = C.c_int
        L.oxo_langevin_run.argtypes = [C.POINTER(OxoModel), C.POINTER(OxoSystem), dp, dp, dp, dp,
                                       C.c_uint32, C.c_int, C.c_double, C.c_double, C.c_double,
                                       C.c_double, C.c_uint64, C.c_long, C.c_long, C.c_double,
                                       C.c_int]
        L.oxo_langevin_run.restype = C.c_long
        L.oxo_philox4x32.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                     C.POINTER(C.c_uint32)]
        _oracle = L
    return _oracle


def ref_lib(precision=64):
    """Reference evaluators compiled from the reference tree (None if unavailable)."""
    if precision in _refs:
        return _refs[precision]
    path = os.path.join(_build.REF_DIR, f"libref{precision}.so")
    if not os.path.exists(path):
        _build.build_ref()
    if not os.path.exists(path):
        _refs[precision] = None
        return None
    L = C.CDLL(path)
    _declare_pairs(L, "ref")
    _refs[precision] = L
    return L


def _arr(x, n):
    a = np.ascontiguousarray(x, dtype=np.float64)
    assert a.size == n
    return a


def eval_pair(lib, prefix, term, params, dr, qi, qj, rcutsq, ci=1.0, cj=1.0):
    """One evaluator call -> (evaluated, force_i[3], energy, torque_i[3], torque_j[3])."""
    fn = getattr(lib, f"{prefix}_{_PAIR_FN[term]}")
    dr = _arr(dr, 3)
    qi = _arr(qi, 4)
    qj = _arr(qj, 4)
    f = np.zeros(3)
    ti = np.zeros(3)
    tj = np.zeros(3)
    e = C.c_double(0.0)
    P = lambda a: a.ctypes.data_as(dp)  # noqa: E731
    args = [C.byref(params), P(dr), P(qi), P(qj), C.c_double(rcutsq)]
    if term == _abi.DEBYE:
        args += [C.c_double(ci), C.c_double(cj)]
    r = fn(*args, P(f), C.byref(e), P(ti), P(tj))
    return bool(r), f, e.value, ti, tj


def eval_bonded(lib, prefix, params, Rc, qA, qB, tA, tB):
    fn = getattr(lib, f"{prefix}_bonded")
    Rc = _arr(Rc, 3)
    qA = _arr(qA, 4)
    qB = _arr(qB, 4)
    FB = np.zeros(3)
    tauA = np.zeros(3)
    tauB = np.zeros(3)
    e = np.zeros(3)
    vir = np.zeros(6)
    P = lambda a: a.ctypes.data_as(dp)  # noqa: E731
    fn(C.byref(params), P(Rc), P(qA), P(qB), int(tA), int(tB), P(FB), P(tauA), P(tauB), P(e), P(vir))
    return FB, tauA, tauB, e, vir


class Model:
    """oxo_model built from this package's force objects (model files' output)."""

    def __init__(self, forces, types, bond_types=("backbone",)):
        self.types = list(types)
        nt = len(self.types)
        self.s = OxoModel()
        self.s.n_types = nt
        self.s.n_bond_types = len(bond_types)
        self._keep = []
        self.mask = 0
        self.has_bonded = False
        from oxdna.forces import OxDNABonded
        fields = {_abi.EXCVOL: "excvol", _abi.HBOND: "hbond", _abi.CROSS: "cross",
                  _abi.HBONDCROSS: "hbondcross", _abi.COAX: "coax", _abi.DEBYE: "debye"}
        for f in forces:
            if isinstance(f, OxDNABonded):
                arr = (_abi.BondedParams * len(bond_types))()
                for k, name in enumerate(bond_types):
                    arr[k] = _abi.bonded_from_dict(f.params[name])
                self.s.bonded = arr
                self._keep.append(arr)
                self.has_bonded = True
                continue
            t = f._term
            arr = (_abi.PARAM_STRUCTS[t] * (nt * nt))()
            rc = (C.c_double * (nt * nt))()
            for a in range(nt):
                for b in range(nt):
                    key = (self.types[a], self.types[b])
                    arr[a * nt + b] = _abi.FROM_DICT[t](f.params[key])
                    rc[a * nt + b] = f.rcut_for(*key)
            setattr(self.s, fields[t], arr)
            self.s.r_cut[t] = C.cast(rc, dp)
            self._keep += [arr, rc]
            self.mask |= 1 << t


class System:
    """oxo_system over numpy arrays (kept alive by this object)."""

    def __init__(self, pos, quat, typeid, box, bonds, charge=None, bond_typeid=None):
        self.pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        self.quat = np.ascontiguousarray(quat, dtype=np.float64).reshape(-1, 4)
        self.type = np.ascontiguousarray(typeid, dtype=np.int32)
        n = len(self.pos)
        self.charge = np.ascontiguousarray(np.ones(n) if charge is None else charge, dtype=np.float64)
        b = np.zeros((max(1, len(bonds)), 3), np.int32)
        if len(bonds):
            b[:len(bonds), :2] = np.asarray(bonds, np.int32)
            if bond_typeid is not None:
                b[:len(bonds), 2] = bond_typeid
        self.bonds = b
        self.nb = len(bonds)
        self.box = np.asarray(box, float)[:3]
        self.s = OxoSystem()
        self.s.N = n
        self.s.pos = self.pos.ctypes.data_as(dp)
        self.s.quat = self.quat.ctypes.data_as(dp)
        self.s.type = self.type.ctypes.data_as(ip)
        self.s.charge = self.charge.ctypes.data_as(dp)
        for k in range(3):
            self.s.box[k] = float(self.box[k])
        self.s.n_bonds = self.nb
        self.s.bonds = self.bonds.ctypes.data_as(ip)

    @classmethod
    def from_snapshot(cls, snap):
        p = snap.particles
        return cls(p.position, p.orientation, p.typeid, snap.configuration.box,
                   [tuple(g) for g in snap.bonds.group], p.charge, snap.bonds.typeid)


def forces(model, system, mask=None, bonded=None, use_cells=True):
    """Per-particle force (N,3), per-particle energy (N,), torque (N,3), pair energies
    (6,), bonded energies (3,), pair counts (6,)."""
    L = oracle_lib()
    n = system.s.N
    f = np.zeros((n, 4))
    t = np.zeros((n, 3))
    pe = np.zeros(6)
    be = np.zeros(3)
    pc = np.zeros(6, dtype=np.int64)
    mask = model.mask if mask is None else mask
    bonded = model.has_bonded if bonded is None else bonded
    r = L.oxo_forces(C.byref(model.s), C.byref(system.s), mask, int(bonded), int(use_cells),
                     f.ctypes.data_as(dp), t.ctypes.data_as(dp), pe.ctypes.data_as(dp),
                     be.ctypes.data_as(dp), pc.ctypes.data_as(C.POINTER(C.c_int64)))
    if r != 0:
        raise RuntimeError("oracle rejected the bond table")
    return dict(force=f[:, :3], energy_pp=f[:, 3], torque=t, pair_energy=pe, bonded_energy=be,
                pair_count=pc)


def langevin(model, system, vel, angmom, steps, dt, kT, gamma=1.0, gamma_r=1.0, seed=1,
             step0=0, buffer=0.4, threads=1, mask=None, bonded=None):
    """Advance system.pos / system.quat / vel / angmom in place; returns nlist builds."""
    L = oracle_lib()
    vel = np.ascontiguousarray(vel, dtype=np.float64)
    angmom = np.ascontiguousarray(angmom, dtype=np.float64)
    mask = model.mask if mask is None else mask
    bonded = model.has_bonded if bonded is None else bonded
    builds = L.oxo_langevin_run(C.byref(model.s), C.byref(system.s), system.s.pos, system.s.quat,
                                vel.ctypes.data_as(dp), angmom.ctypes.data_as(dp), mask,
                                int(bonded), dt, kT, gamma, gamma_r, seed, step0, steps, buffer,
                                threads)
    return builds, vel, angmom


def half_pairs(system, r_list):
    """Half neighbour list (i < j) within r_list under the minimum image, bonded pairs
    excluded (HOOMD's bond exclusions): int32 array (n, 2)."""
    from scipy.spatial import cKDTree
    box = np.asarray(system.box, float)
    p = np.mod(system.pos + 0.5 * box, box)
    p = np.where(p >= box, p - box, p)
    pairs = cKDTree(p, boxsize=box).query_pairs(r_list, output_type="ndarray")
    pairs = np.sort(pairs, axis=1)
    if system.nb:
        b = np.sort(system.bonds[:system.nb, :2], axis=1).astype(np.int64)
        n = len(system.pos)
        keep = ~np.isin(pairs[:, 0].astype(np.int64) * n + pairs[:, 1], b[:, 0] * n + b[:, 1])
        pairs = pairs[keep]
    order = np.lexsort((pairs[:, 1], pairs[:, 0]))
    return np.ascontiguousarray(pairs[order], dtype=np.int32)


def ref_system_forces(model, system, pairs, mask=None, bonded=None, precision=64):
    """The system's forces through the reference's own evaluators and bonded kernel with
    HOOMD's CPU driver semantics (``ref_system_forces`` in ref_wrap.cpp), over the given
    half pair list. Same outputs as :func:`forces`; None when the reference build is
    unavailable."""
    L = ref_lib(precision)
    if L is None:
        return None
    fn = L.ref_system_forces
    fn.argtypes = [C.POINTER(OxoModel), C.POINTER(OxoSystem), C.c_uint32, C.c_int, C.c_int, ip,
                   dp, dp, dp, dp]
    fn.restype = C.c_int
    n = system.s.N
    f = np.zeros((n, 4))
    t = np.zeros((n, 3))
    pe = np.zeros(6)
    be = np.zeros(3)
    mask = model.mask if mask is None else mask
    bonded = model.has_bonded if bonded is None else bonded
    pairs = np.ascontiguousarray(pairs, dtype=np.int32)
    fn(C.byref(model.s), C.byref(system.s), mask, int(bonded), len(pairs), pairs.ctypes.data_as(ip),
       f.ctypes.data_as(dp), t.ctypes.data_as(dp), pe.ctypes.data_as(dp), be.ctypes.data_as(dp))
    return dict(force=f[:, :3], energy_pp=f[:, 3], torque=t, pair_energy=pe, bonded_energy=be)
