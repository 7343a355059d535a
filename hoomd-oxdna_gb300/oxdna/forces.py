"""oxDNA force objects backed by the GB300 engine.

The class names, parameter keys, tuple widths, defaults and read-outs are those of
the reference's ``oxdna/forces.py`` (``OxDNABonded`` 15-112, ``ExcludedVolume``
115-145, ``HydrogenBonding`` 148-176, ``CrossStacking`` 179-207, ``HBondCross``
210-247, ``CoaxialStacking`` 250-286, ``DebyeHuckel`` 289-311). Instead of HOOMD
``Force`` subclasses they attach to :class:`oxdna.runtime.Simulation`, which
evaluates every attached force in one fused GPU launch per step.
"""

from . import _abi

# Counts every change of a force's parameters, cutoffs or attributes (and, through
# oxdna.runtime, of integrators, Langevin methods and their force lists): an attached
# simulation compares its full description only when this has moved since it looked.
_changes = [0]


def _changed():
    _changes[0] += 1


class TypeParameterDict:
    """Per-type (len_keys=1) or per-unordered-type-pair (len_keys=2) parameter dict
    with declared keys, tuple widths and defaults (HOOMD TypeParameterDict idiom)."""

    def __init__(self, len_keys, defaults=None, **spec):
        self._len_keys = len_keys
        self._spec = spec
        self._defaults = dict(defaults or {})
        self._data = {}

    def _key(self, key):
        if self._len_keys == 2:
            if not (isinstance(key, tuple) and len(key) == 2):
                raise KeyError(f"pair parameters are keyed by (type_a, type_b), got {key!r}")
            return tuple(sorted(key))
        return key

    def _validate(self, value):
        if not isinstance(value, dict):
            raise TypeError("parameters must be a dict")
        unknown = set(value) - set(self._spec)
        if unknown:
            raise KeyError(f"unknown parameter(s) {sorted(unknown)}")
        out = {}
        for name, kind in self._spec.items():
            if name in value:
                v = value[name]
            elif name in self._defaults:
                v = self._defaults[name]
            else:
                raise KeyError(f"missing parameter {name!r}")
            if isinstance(kind, tuple):
                v = tuple(v)
                if len(v) != len(kind):
                    raise ValueError(f"parameter {name!r} needs {len(kind)} values, got {len(v)}")
                v = tuple(k(x) for k, x in zip(kind, v))
            else:
                v = kind(v)
            out[name] = v
        return out

    def __setitem__(self, key, value):
        self._data[self._key(key)] = self._validate(value)
        self._on_change()

    def __getitem__(self, key):
        return dict(self._data[self._key(key)])

    def __contains__(self, key):
        return self._key(key) in self._data

    def keys(self):
        return self._data.keys()

    def items(self):
        return ((k, dict(v)) for k, v in self._data.items())

    def _on_change(self):
        # a simulation compares this against the value it attached with
        self._version = getattr(self, "_version", 0) + 1
        _changed()


F = float
F3 = (float, float, float)
F4 = (float,) * 4
F5 = (float,) * 5


class _Force:
    """Common read-outs; values come from the simulation the force is attached to."""

    def __init__(self):
        self._simulation = None

    def __setattr__(self, name, value):
        object.__setattr__(self, name, value)
        if not name.startswith("_"):
            _changed()

    def _sim(self):
        if self._simulation is None:
            raise RuntimeError("force is not attached to a simulation (run the simulation first)")
        return self._simulation

    @property
    def energy(self):
        return self._sim()._force_energy(self)

    @property
    def forces(self):
        return self._sim()._force_arrays(self)[0]

    @property
    def torques(self):
        return self._sim()._force_arrays(self)[1]

    @property
    def energies(self):
        """Per-particle energies (HOOMD's Force.energies): half of each pair's or bond's
        energy on each of its two particles, so they sum to ``energy``."""
        return self._sim()._force_arrays(self)[2]


class OxDNABonded(_Force):
    """FENE backbone, bonded excluded volume and (optional) DNA/RNA stacking between
    3'-5' neighbours. Parameters keyed by bond type (reference forces.py:15-112)."""

    def __init__(self):
        super().__init__()
        self.params = TypeParameterDict(
            1,
            defaults={
                "stack_enabled": False, "stack_site": (0.0, 0.0, 0.0),
                "stack_back_ref": (0.0, 0.0, 0.0), "stack_gamma": 0.0,
                "stack_f1": (0.0,) * 9, "stack_eps": (0.0,) * 16, "stack_f4_t4": (0.0,) * 5,
                "stack_f4_t5": (0.0,) * 5, "stack_f5_p1": (0.0,) * 4, "stack_rna": False,
                "stack_3_site": (0.0, 0.0, 0.0), "stack_5_site": (0.0, 0.0, 0.0),
                "stack_bbvector_3": (0.0, 0.0, 0.0), "stack_bbvector_5": (0.0, 0.0, 0.0),
                "stack_f4_tB1": (0.0,) * 5, "stack_f4_tB2": (0.0,) * 5,
            },
            epsilon=F, r0=F, delta=F, pos_back=F3, pos_base=F3, excl_eps=F,
            bexc_base_base=F4, bexc_base_back=F4, bexc_back_base=F4,
            stack_enabled=bool, stack_site=F3, stack_back_ref=F3, stack_gamma=F,
            stack_f1=(float,) * 9, stack_eps=(float,) * 16, stack_f4_t4=F5, stack_f4_t5=F5,
            stack_f5_p1=F4, stack_rna=bool, stack_3_site=F3, stack_5_site=F3,
            stack_bbvector_3=F3, stack_bbvector_5=F3, stack_f4_tB1=F5, stack_f4_tB2=F5,
        )

    @property
    def fene_energy(self):
        """Total FENE energy (recomputed on read)."""
        return self._sim()._bonded_energy(0)

    @property
    def bonded_excvol_energy(self):
        """Total bonded excluded-volume energy (recomputed on read)."""
        return self._sim()._bonded_energy(1)

    @property
    def stacking_energy(self):
        """Total stacking energy (recomputed on read)."""
        return self._sim()._bonded_energy(2)


class _PairForce(_Force):
    _term = None
    _spec = {}
    _defaults = {}

    def __init__(self, nlist, default_r_cut=None, mode="none"):
        super().__init__()
        if mode != "none":
            raise ValueError("oxDNA pair forces support mode='none' only")
        self.nlist = nlist
        self.default_r_cut = default_r_cut
        self.mode = mode
        self.r_cut = TypeParameterDict(2, r_cut=float)
        self.params = TypeParameterDict(2, defaults=self._defaults, **self._spec)

    def rcut_for(self, a, b):
        key = tuple(sorted((a, b)))
        if key in self.r_cut:
            return self.r_cut[key]["r_cut"]
        if self.default_r_cut is None:
            raise KeyError(f"no r_cut for type pair {key}")
        return float(self.default_r_cut)


class ExcludedVolume(_PairForce):
    """Nonbonded excluded volume (BACK/BASE site repulsions; forces.py:115-145)."""
    _term = _abi.EXCVOL
    _spec = dict(eps=F, base_site=F3, back_site=F3, back_back=F4, base_base=F4,
                 base_back=F4, back_base=F4)


class HydrogenBonding(_PairForce):
    """Watson-Crick hydrogen bonding (BASE-BASE; forces.py:148-176)."""
    _term = _abi.HBOND
    _spec = dict(eps=F, shift_factor=F, base_site=F3, f1=(float,) * 8, f4_t1=F5, f4_t23=F5,
                 f4_t4=F5, f4_t78=F5)


class CrossStacking(_PairForce):
    """Cross-stacking (BASE-BASE; forces.py:179-207)."""
    _term = _abi.CROSS
    _spec = dict(base_site=F3, f2=(float,) * 9, f4_t1=F5, f4_t23=F5, f4_t4=F5, f4_t78=F5,
                 t4_enabled=bool)
    _defaults = {"t4_enabled": True}


class HBondCross(_PairForce):
    """Fused hydrogen bonding + cross-stacking (forces.py:210-247)."""
    _term = _abi.HBONDCROSS
    _spec = dict(base_site=F3, eps=F, shift_factor=F, f1=(float,) * 8, hb_f4_t1=F5,
                 hb_f4_t23=F5, hb_f4_t4=F5, hb_f4_t78=F5, f2=(float,) * 9, cs_f4_t1=F5,
                 cs_f4_t23=F5, cs_f4_t4=F5, cs_f4_t78=F5)


class CoaxialStacking(_PairForce):
    """Coaxial stacking (STACK-STACK; forces.py:250-286)."""
    _term = _abi.COAX
    _spec = dict(stack_site=F3, stack_back_ref=F3, gamma=F, f2=(float,) * 9, f4_t1=F5,
                 f4_t4=F5, f4_t56=F5, f5_phi3=F4, f5_phi4=F4, t1_mode=int, t1_sa=F, t1_sb=F,
                 phi3_enabled=bool, rna_coax=bool)
    _defaults = {"f5_phi4": (0.0,) * 4, "rna_coax": False}


class DebyeHuckel(_PairForce):
    """oxDNA2 Debye-Hueckel electrostatics (BACK-BACK; forces.py:289-311)."""
    _term = _abi.DEBYE
    _spec = dict(back_site=F3, debye=F5)
