"""oxDNA topology / configuration I/O: round trips through the file formats, the
quaternion conversion's branch rule, trajectories and malformed input (CPU only)."""

import math

import numpy as np
import pytest

from oxdna import io


def _shepperd(M):
    """One rotation matrix -> (w, x, y, z): the trace test first, then the largest
    diagonal entry, each branch written out (oxdna/io.py:79-114)."""
    tr = M[0, 0] + M[1, 1] + M[2, 2]
    if tr > 0.0:
        s = 2.0 * math.sqrt(tr + 1.0)
        q = [0.25 * s, (M[2, 1] - M[1, 2]) / s, (M[0, 2] - M[2, 0]) / s, (M[1, 0] - M[0, 1]) / s]
    elif M[0, 0] > M[1, 1] and M[0, 0] > M[2, 2]:
        s = 2.0 * math.sqrt(1.0 + M[0, 0] - M[1, 1] - M[2, 2])
        q = [(M[2, 1] - M[1, 2]) / s, 0.25 * s, (M[0, 1] + M[1, 0]) / s, (M[0, 2] + M[2, 0]) / s]
    elif M[1, 1] > M[2, 2]:
        s = 2.0 * math.sqrt(1.0 + M[1, 1] - M[0, 0] - M[2, 2])
        q = [(M[0, 2] - M[2, 0]) / s, (M[0, 1] + M[1, 0]) / s, 0.25 * s, (M[1, 2] + M[2, 1]) / s]
    else:
        s = 2.0 * math.sqrt(1.0 + M[2, 2] - M[0, 0] - M[1, 1])
        q = [(M[1, 0] - M[0, 1]) / s, (M[0, 2] + M[2, 0]) / s, (M[1, 2] + M[2, 1]) / s, 0.25 * s]
    q = np.array(q)
    return q / np.linalg.norm(q)


def test_matrix_to_quaternion_branch_rule():
    rng = np.random.default_rng(11)
    q = rng.normal(size=(400, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    # rotations by pi and near pi about each axis, and the identity: every branch
    extra = [[1, 0, 0, 0]]
    for ax in range(3):
        for ang in (math.pi, math.pi - 1e-3, 2.5):
            v = np.zeros(3)
            v[ax] = 1.0
            extra.append([math.cos(ang / 2), *(math.sin(ang / 2) * v)])
    q = np.vstack([q, extra])
    R = io.quat_to_matrix(q)
    got = io.matrix_to_quaternion(R)
    want = np.array([_shepperd(M) for M in R])
    assert np.abs(got - want).max() < 1e-14
    # the same rotation: q or -q
    assert np.allclose(np.abs(np.einsum("ij,ij->i", got, q)), 1.0, atol=1e-12)
    # every branch was taken
    tr = np.trace(R, axis1=1, axis2=2)
    d = np.diagonal(R, axis1=1, axis2=2)
    k = np.where(tr > 0, 0, np.argmax(d, axis=1) + 1)
    assert set(k.tolist()) == {0, 1, 2, 3}
    assert io.matrix_to_quaternion(R.reshape(10, 41, 3, 3)).shape == (10, 41, 4)


@pytest.mark.parametrize("half", [False, True])
def test_topology_and_conf_round_trip(tmp_path, half):
    sysarr = io.duplex_system(6, 12, 30.0, seed=4)
    n = len(sysarr["pos"])
    strand, base, n3, n5 = io.topology_from_bonds(n, sysarr["bonds"], sysarr["typeid"])
    top, conf = tmp_path / "sys.top", tmp_path / "sys.conf"
    io.write_topology(top, strand, base, n3, n5)
    io.write_conf(conf, sysarr["pos"], sysarr["quat"], sysarr["box"], t=1500)

    t = io.read_topology(top)
    assert t["n"] == n and t["n_strands"] == 12
    assert np.array_equal(t["n3"], n3) and np.array_equal(t["n5"], n5)
    assert t["base"] == base

    snap = io.build_snapshot(top, conf, half_charged_ends=half)
    p = snap.particles
    assert p.N == n
    assert np.abs(p.position - sysarr["pos"]).max() < 1e-12
    assert np.abs(io.quat_to_matrix(p.orientation) - io.quat_to_matrix(sysarr["quat"])).max() < 1e-12
    assert np.array_equal(p.typeid, sysarr["typeid"])
    assert sorted(map(tuple, snap.bonds.group.tolist())) == sorted(map(tuple, sysarr["bonds"]))
    assert snap.configuration.box[:3] == [30.0, 30.0, 30.0]
    if half:
        # 0.5 at the two ends of each strand
        ends = np.flatnonzero(p.charge == 0.5)
        assert len(ends) == 2 * 12 and np.all(p.charge[p.charge != 0.5] == 1.0)
        assert np.array_equal(np.sort(ends), np.flatnonzero(sysarr["ends"]))
    else:
        assert np.all(p.charge == 1.0)


def test_topology_from_bonds_strands():
    # a 5-nt strand, a 3-nt strand, a 4-nt circle
    bonds = [(0, 1), (1, 2), (2, 3), (3, 4), (5, 6), (6, 7), (8, 9), (9, 10), (10, 11), (11, 8)]
    strand, base, n3, n5 = io.topology_from_bonds(12, bonds, [0, 1, 2, 3] * 3)
    assert strand.tolist() == [1] * 5 + [2] * 3 + [3] * 4
    assert n3.tolist()[:5] == [-1, 0, 1, 2, 3] and n5.tolist()[:5] == [1, 2, 3, 4, -1]
    assert n3[8] == 11 and n5[11] == 8
    assert base[:4] == ["A", "G", "C", "T"]
    with pytest.raises(ValueError):
        io.topology_from_bonds(3, [(0, 1), (0, 2)], [0, 0, 0])


def test_trajectory_frames(tmp_path):
    sysarr = io.duplex_system(2, 8, 20.0, seed=2)
    conf = tmp_path / "traj.dat"
    for k in range(3):
        pos = sysarr["pos"] + 0.01 * k
        io.write_conf(conf, pos, sysarr["quat"], sysarr["box"], t=100 * k, append=k > 0,
                      velocities=np.full((len(pos), 3), float(k)))
    frames = list(io.iter_conf_frames(conf))
    assert [f[0] for f in frames] == [0.0, 100.0, 200.0]
    for k, (_, box, arr) in enumerate(frames):
        assert arr.shape == (32, 15) and np.allclose(box, 20.0)
        assert np.allclose(arr[:, 0:3], sysarr["pos"] + 0.01 * k + 10.0, atol=1e-12)
        assert np.all(arr[:, 9:12] == k)
    top = tmp_path / "traj.top"
    io.write_topology(top, *io.topology_from_bonds(32, sysarr["bonds"], sysarr["typeid"]))
    snap = io.build_snapshot(top, conf, frame=2)
    assert np.abs(snap.particles.position - (sysarr["pos"] + 0.02)).max() < 1e-12
    with pytest.raises(ValueError, match="no frame 3"):
        io.build_snapshot(top, conf, frame=3)


def test_conf_rows_without_velocities(tmp_path):
    conf = tmp_path / "short.conf"
    conf.write_text("t = 7\nb = 10 10 10\nE = 0 0 0\n"
                    "1 2 3 1 0 0 0 0 1\n\n4 5 6 0 1 0 0 0 1 0.5 0.5 0.5\n")
    (t, box, arr), = list(io.iter_conf_frames(conf))
    assert t == 7.0 and arr.shape == (2, 15)
    assert arr[0, 9:].tolist() == [0.0] * 6 and arr[1, 9:12].tolist() == [0.5] * 3


def test_malformed_topology(tmp_path):
    top = tmp_path / "bad.top"
    top.write_text("3 1\n1 A -1 1\n1 G 0 2\n")
    with pytest.raises(ValueError, match="announces 3 nucleotides"):
        io.read_topology(top)
    top.write_text("2 1\n1 A -1 1\n1 G 0 5\n")
    with pytest.raises(ValueError, match=r"bad.top:3: neighbour index"):
        io.read_topology(top)
    top.write_text("2 1\n1 A -1\n1 G 0 -1\n")
    with pytest.raises(ValueError, match=r"bad.top:2: expected"):
        io.read_topology(top)
    top.write_text("2\n1 A -1 1\n1 G 0 -1\n")
    with pytest.raises(ValueError, match=r"bad.top:1: expected the header"):
        io.read_topology(top)
    # blank lines between records are tolerated
    top.write_text("2 1\n\n1 A -1 1\n\n1 U 0 -1\n")
    t = io.read_topology(top)
    assert t["base"] == ["A", "U"] and io.base_typeid(t["base"][1]) == 3


def test_tiled_duplex_system_layout():
    from oxdna.model import dna2
    s = io.tiled_duplex_system(8)
    n = len(s["pos"])
    assert n == 8192 and np.all(s["box"] == 64.0) and len(s["bonds"]) == 512 * 14
    b = np.asarray(s["bonds"])
    r = np.linalg.norm(s["pos"][b[:, 1]] - s["pos"][b[:, 0]], axis=1)
    assert np.all(np.abs(r - dna2.FENE_R0) < 0.25)
    # every copy identical up to its grid shift, inside the box, 8 apart
    p = s["pos"].reshape(512, 16, 3)
    shift = p - p[:1]
    assert np.abs(shift - shift[:, :1]).max() < 1e-12
    assert np.all(np.abs(s["pos"]) < 32.0)
    com = p.mean(axis=1)
    d = np.linalg.norm(com[:, None] - com[None], axis=-1) + 1e9 * np.eye(512)
    assert abs(d.min() - 8.0) < 1e-9
    t = s["typeid"][:16]
    assert all(t[k] + t[15 - k] == 3 for k in range(8))


def test_against_the_reference_io(tmp_path):
    """The reference's own io.py on the same inputs (tests/golden/io_golden.npz, from
    make_io_golden.py): quaternions of every branch (the same sign), the topology and
    both configuration frames, and build_snapshot with and without half-charged ends."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "io_golden.npz"))
    q = io.orientations_to_quaternions(g["frames/a1"], g["frames/a3"])
    assert np.abs(q - g["frames/quat"]).max() < 1e-14
    top, conf = tmp_path / "s.top", tmp_path / "s.conf"
    top.write_text(str(g["files/top"]))
    conf.write_text(str(g["files/conf"]))
    t = io.read_topology(top)
    for k in ("strand", "n3", "n5"):
        assert np.array_equal(t[k], g[f"top/{k}"]), k
    assert t["base"] == list(g["top/base"])
    frames = list(io.iter_conf_frames(conf))
    assert np.array_equal([f[0] for f in frames], g["conf/t"])
    assert np.array_equal([f[1] for f in frames], g["conf/box"])
    assert np.array_equal(np.array([f[2] for f in frames]), g["conf/arr"])
    for tag, half in (("plain", False), ("half", True)):
        for frame in (0, 1):
            s = io.build_snapshot(top, conf, frame=frame, half_charged_ends=half)
            key = f"snap/{tag}/{frame}"
            assert np.array_equal(s.particles.position, g[key + "/position"])
            assert np.abs(s.particles.orientation - g[key + "/orientation"]).max() < 1e-14
            assert np.array_equal(s.particles.typeid, g[key + "/typeid"])
            assert np.array_equal(s.particles.charge, g[key + "/charge"])
            assert np.array_equal(s.bonds.group, g[key + "/bonds"])
            assert np.array_equal(np.asarray(s.configuration.box, float), g[key + "/box"])
