"""oxDNA topology / configuration I/O and seeded synthetic system builders.

Readers and the orientation conversion have the reference's names and conventions
(``oxdna/io.py``): bases map to type ids A=0, G=1, C=2, T=3 (U aliases T);
quaternions are (w, x, y, z) with rotate(q, e_x) = a1 and rotate(q, e_z) = a3;
backbone bonds are (i, n5[i]); charges are 1, or 0.5 at strand ends when asked.

The builders produce the benchmark systems from ideal B-form helices (rise 0.3897,
twist 34.8 deg, centre of mass 0.6 from the axis): duplexes and hairpins placed with
uniform-random centre and orientation without overlap in a periodic cubic box.
"""

import math

import numpy as np

DNA_BASES = ["A", "G", "C", "T"]
BASE_ALIAS = {"U": "T"}

RISE = 0.3897
TWIST = math.radians(34.8)
COM_RADIUS = 0.6


def base_typeid(letter):
    return DNA_BASES.index(BASE_ALIAS.get(letter, letter))


def _fields(fh):
    """(line number, fields) of the non-blank lines of an open text file."""
    for k, line in enumerate(fh, start=1):
        f = line.split()
        if f:
            yield k, f


def read_topology(top_path):
    """Parse an oxDNA .top file (oxdna/io.py:32-52).

    Header ``N n_strands``, then one line per nucleotide ``strand base n3 n5`` (-1 where
    there is no neighbour). Returns a dict with ``n``, ``n_strands``, ``strand``,
    ``base`` (letters), ``n3`` and ``n5``. A short file, a malformed line or a
    neighbour index outside [-1, N) raises ``ValueError`` naming the line.
    """
    with open(top_path) as fh:
        lines = _fields(fh)
        try:
            k, head = next(lines)
        except StopIteration:
            raise ValueError(f"{top_path}: empty topology") from None
        if len(head) < 2:
            raise ValueError(f"{top_path}:{k}: expected the header 'N n_strands'")
        n, n_strands = int(head[0]), int(head[1])
        body = [(k, f) for _, (k, f) in zip(range(n), lines)]
    if len(body) < n:
        raise ValueError(f"{top_path}: the header announces {n} nucleotides, the file lists {len(body)}")
    for k, f in body:
        if len(f) < 4:
            raise ValueError(f"{top_path}:{k}: expected 'strand base n3 n5', got {' '.join(f)!r}")
    strand = np.array([int(f[0]) for _, f in body], dtype=int)
    base = [f[1] for _, f in body]
    links = np.array([(int(f[2]), int(f[3])) for _, f in body], dtype=int).reshape(n, 2)
    bad = np.flatnonzero((links < -1).any(axis=1) | (links >= n).any(axis=1))
    if len(bad):
        k = body[bad[0]][0]
        raise ValueError(f"{top_path}:{k}: neighbour index outside [-1, {n})")
    return dict(n=n, n_strands=n_strands, strand=strand, base=base,
                n3=links[:, 0].copy(), n5=links[:, 1].copy())


def iter_conf_frames(conf_path):
    """Yield (t, box, arr) per frame of an oxDNA configuration or trajectory
    (oxdna/io.py:55-76), reading one frame at a time.

    A frame is ``t = T``, ``b = Lx Ly Lz``, ``E = ...`` and then one line per
    nucleotide; ``arr`` rows are com(3) a1(3) a3(3) v(3) L(3). Lines with fewer than
    nine numbers are skipped; a row without velocities gets zeros there.
    """
    def frame(t, box, rows):
        arr = np.zeros((len(rows), 15))
        for r, f in enumerate(rows):
            m = min(len(f), 15)
            arr[r, :m] = [float(x) for x in f[:m]]
        return t, box, arr

    t = box = None
    rows = []
    skip = 0
    with open(conf_path) as fh:
        for line in fh:
            if line.startswith("t ="):
                if t is not None:
                    yield frame(t, box, rows)
                t, box, rows, skip = float(line.split("=", 1)[1]), None, [], 2
                continue
            if t is None:
                continue
            if skip:
                # the two header lines after 't =': the box, then the energies
                if box is None:
                    box = np.array(line.split("=", 1)[1].split(), dtype=float)
                skip -= 1
                continue
            f = line.split()
            if len(f) >= 9:
                rows.append(f)
    if t is not None:
        yield frame(t, box, rows)


def quat_to_matrix(q):
    """Rotation matrices (..., 3, 3) of (w, x, y, z) quaternions (HOOMD rotate)."""
    q = np.asarray(q, dtype=float)
    w, x, y, z = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    R = np.empty(q.shape[:-1] + (3, 3))
    R[..., 0, 0] = w * w + x * x - y * y - z * z
    R[..., 0, 1] = 2 * (x * y - w * z)
    R[..., 0, 2] = 2 * (x * z + w * y)
    R[..., 1, 0] = 2 * (x * y + w * z)
    R[..., 1, 1] = w * w - x * x + y * y - z * z
    R[..., 1, 2] = 2 * (y * z - w * x)
    R[..., 2, 0] = 2 * (x * z - w * y)
    R[..., 2, 1] = 2 * (y * z + w * x)
    R[..., 2, 2] = w * w - x * x - y * y + z * z
    return R


def matrix_to_quaternion(R):
    """Rotation matrices (..., 3, 3) -> unit (w, x, y, z), vectorised.

    The entries of the symmetric matrix K = 4 q q^T are linear in R: the diagonal is
    1 + tr R with the signs of (w, x, y, z), the off-diagonal the sums and differences
    of R's mirrored entries. q is the row of K through a large diagonal entry, divided
    by 2 sqrt(K_kk). The row is picked with Shepperd's rule (w when tr R > 0, else the
    largest diagonal of R), as the reference does (oxdna/io.py:79-114), so the sign of
    q (the chosen component positive) is the reference's too.
    """
    R = np.asarray(R, dtype=float)
    M = R.reshape(-1, 3, 3)
    m00, m11, m22 = M[:, 0, 0], M[:, 1, 1], M[:, 2, 2]
    K = np.empty((len(M), 4, 4))
    K[:, 0, 0] = 1.0 + m00 + m11 + m22
    K[:, 1, 1] = 1.0 + m00 - m11 - m22
    K[:, 2, 2] = 1.0 - m00 + m11 - m22
    K[:, 3, 3] = 1.0 - m00 - m11 + m22
    for a, b, v in ((0, 1, M[:, 2, 1] - M[:, 1, 2]), (0, 2, M[:, 0, 2] - M[:, 2, 0]),
                    (0, 3, M[:, 1, 0] - M[:, 0, 1]), (1, 2, M[:, 0, 1] + M[:, 1, 0]),
                    (1, 3, M[:, 0, 2] + M[:, 2, 0]), (2, 3, M[:, 1, 2] + M[:, 2, 1])):
        K[:, a, b] = K[:, b, a] = v
    tr = m00 + m11 + m22
    k = np.where(tr > 0.0, 0, np.where((m00 > m11) & (m00 > m22), 1, np.where(m11 > m22, 2, 3)))
    rows = np.arange(len(M))
    s = 2.0 * np.sqrt(K[rows, k, k])
    q = K[rows, k, :] / s[:, None]
    q[rows, k] = 0.25 * s
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    return q.reshape(R.shape[:-2] + (4,))


def orientations_to_quaternions(a1, a3, check=True):
    """Per-nucleotide (a1, a3) -> (w, x, y, z) with rotate(q, e_x) = a1 (io.py:117-136)."""
    a1 = np.asarray(a1, float)
    a3 = np.asarray(a3, float)
    e1 = a1 / np.linalg.norm(a1, axis=1, keepdims=True)
    e3 = a3 / np.linalg.norm(a3, axis=1, keepdims=True)
    e2 = np.cross(e3, e1)
    R = np.stack([e1, e2, e3], axis=-1)
    q = matrix_to_quaternion(R)
    if check:
        err = np.linalg.norm(quat_to_matrix(q)[..., :, 0] - e1, axis=1)
        if len(err) and err.max() > 1e-6:
            i = int(np.argmax(err))
            raise ValueError(f"quaternion convention check failed at nucleotide {i}: {err[i]:.2e}")
    return q


def quaternions_to_orientations(q):
    """(w, x, y, z) -> (a1, a3) = (rotate(q, e_x), rotate(q, e_z)): the inverse map."""
    R = quat_to_matrix(q)
    return R[..., :, 0], R[..., :, 2]


def terminal_charges(top, end_charge=0.5, interior_charge=1.0):
    charges = np.full(top["n"], interior_charge)
    charges[(np.asarray(top["n3"]) < 0) | (np.asarray(top["n5"]) < 0)] = end_charge
    return charges


class SystemArrays(dict):
    """pos (N,3), quat (N,4), typeid (N,), box (3,), bonds [(A,B)], charge (N,),
    plus strand/n3/n5 bookkeeping. Convert with :func:`snapshot_from_arrays`."""


def snapshot_from_arrays(positions, quaternions, typeids, box, bonds=None, types=DNA_BASES,
                         bond_type="backbone", charges=None):
    """Snapshot from arrays (positions box-centred). Unit charge by default."""
    from .runtime import Snapshot
    n = len(positions)
    snap = Snapshot()
    p = snap.particles
    p.N = n
    p.types = list(types)
    p.position[:] = np.asarray(positions, float)
    p.typeid[:] = np.asarray(typeids, int)
    p.mass[:] = 1.0
    p.moment_inertia[:] = 1.0
    p.orientation[:] = np.asarray(quaternions, float)
    p.charge[:] = np.ones(n) if charges is None else np.asarray(charges, float)
    snap.configuration.box = [float(box[0]), float(box[1]), float(box[2]), 0, 0, 0]
    bonds = list(bonds or [])
    snap.bonds.N = len(bonds)
    snap.bonds.types = [bond_type]
    if bonds:
        snap.bonds.group[:] = np.asarray(bonds, int)
        snap.bonds.typeid[:] = 0
    return snap


def build_snapshot(top_path, conf_path, frame=0, bond_type="backbone", half_charged_ends=False):
    """Snapshot from an oxDNA topology + configuration frame (io.py:196-241).

    Positions move from oxDNA's [0, L) box to HOOMD's origin-centred one; backbone
    bonds are (i, n5[i]), one per 5' link.
    """
    top = read_topology(top_path)
    for k, (_, box, arr) in enumerate(iter_conf_frames(conf_path)):
        if k == frame:
            break
    else:
        raise ValueError(f"{conf_path}: no frame {frame}")
    if len(arr) != top["n"]:
        raise ValueError(f"{conf_path}: frame {frame} has {len(arr)} nucleotides, "
                         f"the topology {top['n']}")
    q = orientations_to_quaternions(arr[:, 3:6], arr[:, 6:9])
    typeids = [base_typeid(b) for b in top["base"]]
    n5 = top["n5"]
    bonds = [(int(i), int(n5[i])) for i in np.flatnonzero(n5 >= 0)]
    charges = terminal_charges(top) if half_charged_ends else np.ones(top["n"])
    return snapshot_from_arrays(arr[:, 0:3] - box / 2.0, q, typeids, box, bonds=bonds,
                                bond_type=bond_type, charges=charges)


def topology_from_bonds(n, bonds, typeids):
    """(strand, base, n3, n5) of n nucleotides whose backbone bonds (A, B) link A to its
    5' neighbour B, the convention of :func:`build_snapshot`; strands are numbered from
    1 in order of their 3' ends."""
    n3 = np.full(n, -1, dtype=int)
    n5 = np.full(n, -1, dtype=int)
    for a, b in bonds:
        if n5[a] >= 0 or n3[b] >= 0:
            raise ValueError(f"nucleotide {a} or {b} has two backbone bonds in one direction")
        n5[a], n3[b] = b, a
    strand = np.zeros(n, dtype=int)
    sid = 0
    for start in list(np.flatnonzero(n3 < 0)) + list(range(n)):
        if strand[start]:
            continue
        sid += 1  # a 3' end, then what is left: circular strands
        i = start
        while i >= 0 and not strand[i]:
            strand[i] = sid
            i = n5[i]
    base = [DNA_BASES[int(t)] for t in typeids]
    return strand, base, n3, n5


def write_topology(top_path, strand, base, n3, n5):
    """Write an oxDNA .top file (the format :func:`read_topology` reads)."""
    n = len(base)
    with open(top_path, "w") as fh:
        fh.write(f"{n} {len(set(int(x) for x in strand))}\n")
        for i in range(n):
            fh.write(f"{int(strand[i])} {base[i]} {int(n3[i])} {int(n5[i])}\n")


def write_conf(conf_path, positions, quaternions, box, t=0, velocities=None, angular=None,
               energies=(0.0, 0.0, 0.0), append=False):
    """Write one frame of an oxDNA configuration (the format :func:`iter_conf_frames`
    reads): HOOMD's origin-centred positions move to [0, L), orientations become
    (a1, a3). ``append`` adds the frame to a trajectory file."""
    box = np.asarray(box, float)[:3]
    pos = np.asarray(positions, float) + box / 2.0
    a1, a3 = quaternions_to_orientations(quaternions)
    n = len(pos)
    v = np.zeros((n, 3)) if velocities is None else np.asarray(velocities, float)
    L = np.zeros((n, 3)) if angular is None else np.asarray(angular, float)
    cols = np.hstack([pos, a1, a3, v, L])
    with open(conf_path, "a" if append else "w") as fh:
        fh.write(f"t = {t}\n")
        fh.write("b = " + " ".join(repr(float(x)) for x in box) + "\n")
        fh.write("E = " + " ".join(repr(float(x)) for x in energies) + "\n")
        np.savetxt(fh, cols, fmt="%.17g")


# ------------------------------------------------------------------ synthetic builders
def ideal_strand(n, start=0, direction=+1):
    """Ideal B-form helix positions and frames for n nucleotides of one strand.

    Strand nucleotide k sits at height (start + direction*k)*RISE, azimuth
    phi = (start + direction*k)*TWIST, centre of mass COM_RADIUS from the axis; a1
    points at the axis, a3 along the strand towards its 5' neighbour (the next
    index). Returns pos (n,3), a1 (n,3), a3 (n,3) in the helix frame (axis = z).
    """
    k = start + direction * np.arange(n)
    phi = k * TWIST
    radial = np.stack([np.cos(phi), np.sin(phi), np.zeros(n)], axis=1)
    pos = COM_RADIUS * radial + np.outer(k * RISE, [0.0, 0.0, 1.0])
    a1 = -radial
    a3 = np.tile([0.0, 0.0, float(direction)], (n, 1))
    return pos, a1, a3


def duplex(seq):
    """Ideal duplex: strand 1 (bases seq, 3'->5' along +z) then its complement.

    Strand-2 nucleotide m pairs with strand-1 nucleotide n-1-m and sits on the far
    side of the axis with a1 and a3 reversed. Returns pos, a1, a3, types, bonds
    (local indices, (i, i+1) within each strand) and strand-end flags.
    """
    n = len(seq)
    comp = {"A": "T", "T": "A", "G": "C", "C": "G"}
    p1, a11, a31 = ideal_strand(n)
    # strand 2: nucleotide m pairs with n-1-m (same height, opposite side)
    k = np.arange(n)[::-1]
    phi = k * TWIST
    radial = np.stack([np.cos(phi), np.sin(phi), np.zeros(n)], axis=1)
    p2 = -COM_RADIUS * radial + np.outer(k * RISE, [0.0, 0.0, 1.0])
    a12 = radial
    a32 = np.tile([0.0, 0.0, -1.0], (n, 1))
    seq2 = [comp[seq[n - 1 - m]] for m in range(n)]
    pos = np.vstack([p1, p2])
    a1 = np.vstack([a11, a12])
    a3 = np.vstack([a31, a32])
    types = np.array([base_typeid(b) for b in list(seq) + seq2])
    bonds = [(i, i + 1) for i in range(n - 1)] + [(n + i, n + i + 1) for i in range(n - 1)]
    ends = np.zeros(2 * n, bool)
    ends[[0, n - 1, n, 2 * n - 1]] = True
    return pos, a1, a3, types, bonds, ends


def hairpin_strand(seq):
    """One strand as an extended ideal helix (hairpins start unfolded)."""
    n = len(seq)
    pos, a1, a3 = ideal_strand(n)
    types = np.array([base_typeid(b) for b in seq])
    bonds = [(i, i + 1) for i in range(n - 1)]
    ends = np.zeros(n, bool)
    ends[[0, n - 1]] = True
    return pos, a1, a3, types, bonds, ends


def random_rotation(rng):
    """Uniform random rotation matrix (from a uniform random unit quaternion)."""
    u1, u2, u3 = rng.random(3)
    q = np.array([math.sqrt(1 - u1) * math.sin(2 * math.pi * u2),
                  math.sqrt(1 - u1) * math.cos(2 * math.pi * u2),
                  math.sqrt(u1) * math.sin(2 * math.pi * u3),
                  math.sqrt(u1) * math.cos(2 * math.pi * u3)])
    return quat_to_matrix(q)


def random_sequence(rng, n, alphabet="ACGT"):
    return "".join(alphabet[i] for i in rng.integers(0, len(alphabet), n))


def pack_molecules(molecules, box_len, rng, min_dist=1.5, max_tries=2000):
    """Place molecules (pos, a1, a3, types, bonds, ends) with random centre and
    orientation in a periodic cube without any inter-molecule COM pair closer than
    min_dist. Returns the concatenated system arrays."""
    L = float(box_len)
    ncell = max(1, int(L // max(min_dist, 1e-3)))
    cap = 64
    # occupancy grid: per cell up to `cap` placed positions (NaN = empty)
    grid = np.full((ncell, ncell, ncell, cap, 3), np.nan)
    count = np.zeros((ncell, ncell, ncell), dtype=np.int64)
    offs = np.array([(a, b, c) for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1)])

    def cells(p):
        return (np.floor((p + L / 2) / L * ncell).astype(np.int64)) % ncell

    def overlaps(p):
        ci = cells(p)
        nb = (ci[:, None, :] + offs[None, :, :]) % ncell          # (n, 27, 3)
        cand = grid[nb[..., 0], nb[..., 1], nb[..., 2]]           # (n, 27, cap, 3)
        d = p[:, None, None, :] - cand
        d -= L * np.round(d / L)
        r2 = np.einsum("...k,...k->...", d, d)
        return bool(np.any(r2 < min_dist * min_dist))            # NaN compares False

    out_pos, out_a1, out_a3, out_t, out_b, out_ends, out_mol = [], [], [], [], [], [], []
    offset = 0
    for mid, (pos, a1, a3, types, bonds, ends) in enumerate(molecules):
        centred = pos - pos.mean(axis=0)
        placed = False
        for _ in range(max_tries):
            R = random_rotation(rng)
            c = (rng.random(3) - 0.5) * L
            p = centred @ R.T + c
            p = p - L * np.round(p / L)
            if not overlaps(p):
                placed = True
                break
        if not placed:
            raise RuntimeError(f"could not place molecule {mid} without overlap")
        for x, ci in zip(p, cells(p)):
            k = count[ci[0], ci[1], ci[2]]
            if k >= cap:
                raise RuntimeError("placement grid cell overflow")
            grid[ci[0], ci[1], ci[2], k] = x
            count[ci[0], ci[1], ci[2]] = k + 1
        out_pos.append(p)
        out_a1.append(a1 @ R.T)
        out_a3.append(a3 @ R.T)
        out_t.append(types)
        out_b += [(a + offset, b + offset) for a, b in bonds]
        out_ends.append(ends)
        out_mol.append(np.full(len(p), mid))
        offset += len(p)
    pos = np.vstack(out_pos)
    a1 = np.vstack(out_a1)
    a3 = np.vstack(out_a3)
    return SystemArrays(pos=pos, quat=orientations_to_quaternions(a1, a3),
                        typeid=np.concatenate(out_t), box=np.array([L, L, L]), bonds=out_b,
                        ends=np.concatenate(out_ends), molecule=np.concatenate(out_mol),
                        charge=np.ones(len(pos)))


def duplex_system(n_duplexes, n_bp, box_len, seed=1, min_dist=1.5):
    """n_duplexes random-sequence B-form duplexes of n_bp base pairs (or a list of
    lengths) in a periodic cube of side box_len (seeded PCG64)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lengths = n_bp if hasattr(n_bp, "__len__") else [n_bp] * n_duplexes
    mols = [duplex(random_sequence(rng, int(n))) for n in lengths]
    return pack_molecules(mols, box_len, rng, min_dist=min_dist)


def hairpin_system(n_hairpins, stem=16, loop=16, box_len=80.0, seed=1, min_dist=1.5):
    """Single strands 5'-stem, loop, complementary stem-3' started as extended helices."""
    rng = np.random.Generator(np.random.PCG64(seed))
    comp = {"A": "T", "T": "A", "G": "C", "C": "G"}
    mols = []
    for _ in range(n_hairpins):
        s = random_sequence(rng, stem)
        lp = random_sequence(rng, loop)
        seq = s + lp + "".join(comp[b] for b in reversed(s))
        mols.append(hairpin_strand(seq))
    return pack_molecules(mols, box_len, rng, min_dist=min_dist)


def tiled_duplex_system(copies, n_bp=8, spacing=8.0, seed=1):
    """One ideal duplex of n_bp base pairs (seeded random sequence) repeated, with the
    same orientation, at the centres of a copies^3 grid of cells of side ``spacing``:
    the layout of the reference's benchmark (bench/benchmark.py:22-52, which tiles
    its 16-nt simple-helix duplex, 8 bp, spacing 8; copies = 8 gives 8192 nt in a
    box of 64). Each copy is centred on its COM, so the copies are ``spacing`` apart."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pos0, a10, a30, t0, b0, e0 = duplex(random_sequence(rng, n_bp))
    pos0 = pos0 - pos0.mean(axis=0)
    n0 = len(pos0)
    L = copies * float(spacing)
    g = (np.arange(copies) + 0.5) * spacing - L / 2.0
    shifts = np.stack(np.meshgrid(g, g, g, indexing="ij"), axis=-1).reshape(-1, 3)
    m = len(shifts)
    pos = (pos0[None, :, :] + shifts[:, None, :]).reshape(-1, 3)
    a1 = np.tile(a10, (m, 1))
    a3 = np.tile(a30, (m, 1))
    b0 = np.asarray(b0, dtype=int)
    bonds = (b0[None, :, :] + (n0 * np.arange(m))[:, None, None]).reshape(-1, 2)
    return SystemArrays(pos=pos, quat=orientations_to_quaternions(a1, a3),
                        typeid=np.tile(t0, m), box=np.array([L, L, L]),
                        bonds=[tuple(b) for b in bonds.tolist()], ends=np.tile(e0, m),
                        molecule=np.repeat(np.arange(m), n0), charge=np.ones(m * n0))


def system_snapshot(sysarr, half_charged_ends=False):
    charges = np.where(sysarr["ends"], 0.5, 1.0) if half_charged_ends else sysarr["charge"]
    return snapshot_from_arrays(sysarr["pos"], sysarr["quat"], sysarr["typeid"], sysarr["box"],
                                bonds=sysarr["bonds"], charges=charges)
