"""Golden parameter tables: the reference's own model files (oxdna/model/dna1.py,
dna2.py, rna2.py, imported unchanged from the reference tree) evaluated for a set of
temperatures, salts and variants, every force's parameters per type pair (or bond
type) and its default cutoff written to tests/golden/model_params.json.

The reference package imports HOOMD-blue and its compiled ``_engine``, neither of
which exists here; the few HOOMD classes its model code touches (Force,
AnisotropicPair, TypeParameter, TypeParameterDict, nlist.Cell) are replaced by
stand-ins that only record what is assigned. Run from the repository root:

    python tests/golden/make_model_params.py /root/reference
"""

import json
import os
import sys
import types

CASES = [
    ("dna1", dict(temperature=296.15, average=True, fused=False)),
    ("dna1", dict(temperature=330.0, average=False, fused=True)),
    ("dna2", dict(temperature=296.15, salt=0.5, fused=False, average=True)),
    ("dna2", dict(temperature=310.0, salt=0.15, fused=True, average=False)),
    ("dna2", dict(temperature=340.0, salt=1.0, fused=False, average=False)),
    ("rna2", dict(temperature=310.15, salt=1.0, average=True)),
    ("rna2", dict(temperature=300.0, salt=0.3, average=False)),
]


def _install_hoomd_stand_in():
    def module(name):
        m = types.ModuleType(name)
        sys.modules[name] = m
        return m

    class TypeParameterDict:
        def __init__(self, len_keys=1, **spec):
            self.len_keys = len_keys
            self.spec = spec
            self.data = {}

    class TypeParameter:
        def __init__(self, name, type_kind, param_dict):
            self.name = name
            self.param_dict = param_dict

        def __setitem__(self, key, value):
            self.param_dict.data[key] = dict(value)

        def __getitem__(self, key):
            return self.param_dict.data[key]

    class Force:
        def __init__(self):
            self._typeparams = {}

        def _add_typeparam(self, tp):
            self._typeparams[tp.name] = tp

        def __getattr__(self, name):
            tps = self.__dict__.get("_typeparams", {})
            if name in tps:
                return tps[name]
            raise AttributeError(name)

    class AnisotropicPair(Force):
        def __init__(self, nlist, default_r_cut=None, mode="none"):
            super().__init__()
            self.nlist = nlist
            self.default_r_cut = default_r_cut
            self.mode = mode

    class Cell:
        def __init__(self, buffer=0.4, exclusions=("bond",)):
            self.buffer = buffer
            self.exclusions = exclusions

    hoomd = module("hoomd")
    hoomd.md = module("hoomd.md")
    hoomd.md.force = module("hoomd.md.force")
    hoomd.md.force.Force = Force
    hoomd.md.pair = module("hoomd.md.pair")
    hoomd.md.pair.aniso = module("hoomd.md.pair.aniso")
    hoomd.md.pair.aniso.AnisotropicPair = AnisotropicPair
    hoomd.md.nlist = module("hoomd.md.nlist")
    hoomd.md.nlist.Cell = Cell
    hoomd.data = module("hoomd.data")
    hoomd.data.typeparam = module("hoomd.data.typeparam")
    hoomd.data.typeparam.TypeParameter = TypeParameter
    hoomd.data.parameterdicts = module("hoomd.data.parameterdicts")
    hoomd.data.parameterdicts.TypeParameterDict = TypeParameterDict
    hoomd.device = types.SimpleNamespace(GPU=type("GPU", (), {}), CPU=type("CPU", (), {}))
    module("oxdna._engine")


def _is_type_spec(v):
    """A TypeParameterDict entry that only names a type (a required key) rather than
    giving a default value."""
    if isinstance(v, type):
        return True
    return isinstance(v, tuple) and len(v) > 0 and all(isinstance(x, type) for x in v)


def _shape(v):
    """A spec entry as text: 'float', 'bool', or a list of those for a tuple."""
    if isinstance(v, tuple):
        return [_shape(x) for x in v]
    t = v if isinstance(v, type) else type(v)
    return t.__name__


def _plain(v):
    if isinstance(v, (list, tuple)):
        return [_plain(x) for x in v]
    if isinstance(v, bool):
        return v
    if isinstance(v, (int, float)):
        return float(v)
    return v


def main(ref_root):
    sys.path.insert(0, ref_root)
    _install_hoomd_stand_in()
    import importlib
    out = []
    for model, kw in CASES:
        mod = importlib.import_module(f"oxdna.model.{model}")
        forces, nlist = mod.forces(**kw)
        entry = {"model": model, "kwargs": kw, "nlist_buffer": nlist.buffer, "forces": []}
        for f in forces:
            params = {",".join(k) if isinstance(k, tuple) else k: {p: _plain(v) for p, v in d.items()}
                      for k, d in f._typeparams["params"].param_dict.data.items()}
            spec = f._typeparams["params"].param_dict.spec
            # optional keys: the spec's `_defaults` dict (the reference's idiom for
            # keys a model may leave unset) and any entry that gives a value
            defaults = {p: _plain(v) for p, v in spec.get("_defaults", {}).items()}
            defaults.update({p: _plain(v) for p, v in spec.items()
                             if p != "_defaults" and not _is_type_spec(v)})
            shape = {p: _shape(v) for p, v in spec.items() if p != "_defaults"}
            entry["forces"].append({"class": type(f).__name__,
                                    "default_r_cut": getattr(f, "default_r_cut", None),
                                    "params": params, "defaults": defaults, "spec": shape,
                                    "len_keys": f._typeparams["params"].param_dict.len_keys})
        out.append(entry)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "model_params.json")
    with open(path, "w") as fh:
        json.dump(out, fh, indent=0, sort_keys=True)
    print(f"wrote {path}: {len(out)} cases")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
