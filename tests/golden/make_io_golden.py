"""Golden I/O vectors: the reference's own oxdna/io.py (imported unchanged from the
reference tree) run on seeded inputs, written to tests/golden/io_golden.npz:

* orientations_to_quaternions on random frames, including the frames that take each
  branch of the matrix-to-quaternion rule;
* read_topology / iter_conf_frames / build_snapshot (plain and half-charged ends) on
  a small two-strand topology and a two-frame configuration written here as text.

HOOMD-blue is absent; io.py needs only ``hoomd.Snapshot``, replaced by a recording
stand-in. Run from the repository root:

    python tests/golden/make_io_golden.py /root/reference
"""

import os
import sys
import types

import numpy as np

TOP = """12 2
1 A -1 1
1 G 0 2
1 C 1 3
1 T 2 4
1 A 3 5
1 U 4 -1
2 A -1 7
2 G 6 8
2 C 7 9
2 T 8 10
2 T 9 11
2 C 10 -1
"""


def _conf(rng):
    lines = []
    for t in (0, 1000):
        lines += [f"t = {t}", "b = 20.0 21.5 19.0", "E = 0.1 0.2 0.3"]
        for i in range(12):
            com = rng.uniform(0.5, 18.5, 3)
            a1 = rng.normal(size=3)
            a1 /= np.linalg.norm(a1)
            a3 = rng.normal(size=3)
            a3 -= a1 * (a3 @ a1)
            a3 /= np.linalg.norm(a3)
            v, L = rng.normal(size=3), rng.normal(size=3)
            lines.append(" ".join(repr(float(x)) for x in np.concatenate([com, a1, a3, v, L])))
    return "\n".join(lines) + "\n"


def _install_hoomd_stand_in():
    class _P:
        def __init__(self):
            self.N = 0

        def __setattr__(self, name, value):
            object.__setattr__(self, name, value)
            if name == "N":
                n = value
                for k, shape in (("position", (n, 3)), ("typeid", (n,)), ("mass", (n,)),
                                 ("moment_inertia", (n, 3)), ("orientation", (n, 4)),
                                 ("charge", (n,))):
                    object.__setattr__(self, k, np.zeros(shape))
                object.__setattr__(self, "types", [])

    class _B:
        def __init__(self):
            self.N = 0

        def __setattr__(self, name, value):
            object.__setattr__(self, name, value)
            if name == "N":
                object.__setattr__(self, "group", np.zeros((value, 2), dtype=np.int64))
                object.__setattr__(self, "typeid", np.zeros(value, dtype=np.int64))
                object.__setattr__(self, "types", [])

    class Snapshot:
        def __init__(self):
            self.communicator = types.SimpleNamespace(rank=0)
            self.particles = _P()
            self.bonds = _B()
            self.configuration = types.SimpleNamespace(box=None)

    hoomd = types.ModuleType("hoomd")
    hoomd.Snapshot = Snapshot
    sys.modules["hoomd"] = hoomd


def _load_reference_io(ref_root):
    import importlib.util
    spec = importlib.util.spec_from_file_location("reference_io", os.path.join(ref_root, "oxdna", "io.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def main(ref_root):
    _install_hoomd_stand_in()
    rio = _load_reference_io(ref_root)
    rng = np.random.default_rng(20)
    out = {}
    # frames: random, plus rotations by pi / near pi about each axis (every branch)
    q = rng.normal(size=(300, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    extra = [[1.0, 0, 0, 0]]
    for ax in range(3):
        for ang in (np.pi, np.pi - 1e-3, 2.5):
            v = np.zeros(3)
            v[ax] = 1.0
            extra.append([np.cos(ang / 2), *(np.sin(ang / 2) * v)])
    q = np.vstack([q, extra])
    w, x, y, z = q.T
    a1 = np.stack([1 - 2 * (y * y + z * z), 2 * (x * y + z * w), 2 * (x * z - y * w)], axis=1)
    a3 = np.stack([2 * (x * z + y * w), 2 * (y * z - x * w), 1 - 2 * (x * x + y * y)], axis=1)
    out["frames/a1"] = a1
    out["frames/a3"] = a3
    out["frames/quat"] = rio.orientations_to_quaternions(a1, a3)
    # files
    conf = _conf(rng)
    out["files/top"] = np.array(TOP)
    out["files/conf"] = np.array(conf)
    tmp = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_io_tmp")
    os.makedirs(tmp, exist_ok=True)
    tp, cp = os.path.join(tmp, "s.top"), os.path.join(tmp, "s.conf")
    with open(tp, "w") as fh:
        fh.write(TOP)
    with open(cp, "w") as fh:
        fh.write(conf)
    top = rio.read_topology(tp)
    for k in ("strand", "n3", "n5"):
        out[f"top/{k}"] = np.asarray(top[k])
    out["top/base"] = np.array(top["base"])
    frames = list(rio.iter_conf_frames(cp))
    out["conf/t"] = np.array([f[0] for f in frames])
    out["conf/box"] = np.array([f[1] for f in frames])
    out["conf/arr"] = np.array([f[2] for f in frames])
    for tag, half in (("plain", False), ("half", True)):
        for frame in (0, 1):
            s = rio.build_snapshot(tp, cp, frame=frame, half_charged_ends=half)
            p = s.particles
            key = f"snap/{tag}/{frame}"
            out[key + "/position"] = np.asarray(p.position)
            out[key + "/orientation"] = np.asarray(p.orientation)
            out[key + "/typeid"] = np.asarray(p.typeid)
            out[key + "/charge"] = np.asarray(p.charge)
            out[key + "/bonds"] = np.asarray(s.bonds.group)
            out[key + "/box"] = np.asarray(s.configuration.box, dtype=float)
    os.remove(tp)
    os.remove(cp)
    os.rmdir(tmp)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "io_golden.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path}: {len(out)} arrays")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
