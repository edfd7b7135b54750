"""Seeded synthetic molecules of the benchmark configurations.

No public dataset is named for this path; these generators stand in for one:
  * n-octane, all-trans, ideal geometry (C-C 1.54 A, C-H 1.09 A, tetrahedral
    angles, 180 deg C-C-C-C dihedrals)                       -> octane()
  * (H2O)_k clusters: O on a jittered cubic lattice at 2.9 A, ideal water
    (O-H 0.96 A, H-O-H 104.5 deg), random orientations       -> water_cluster()
    and Gaussian-displaced replicas of one cluster           -> water_replicas()
  * random saturated acyclic alkanes CnH2n+2: random tree, ideal bonds and
    angles, uniform random dihedrals, rejecting non-bonded pairs (>= 3 bonds
    apart) closer than 1.8 A                                 -> random_alkane()
  * a Poisson stream of mixed-size requests                  -> serving_stream()
All coordinates are returned in bohr with MolDS's Angstrom conversion.
"""
from __future__ import annotations

import math

import numpy as np

from .inputfile import ANG2AU, Molecule

TET = math.acos(-1.0 / 3.0)          # 109.4712 deg
CC, CH, OH = 1.54, 1.09, 0.96
HOH = math.radians(104.5)


def _unit(v):
    return v / np.linalg.norm(v)


def _place(a, b, c, bond, angle, torsion):
    """Natural-extension reference frame: the atom d with |cd| = bond,
    angle(b, c, d) = angle and dihedral(a, b, c, d) = torsion."""
    bc = _unit(c - b)
    n = _unit(np.cross(b - a, bc))
    m = np.cross(n, bc)
    d2 = np.array([-bond * math.cos(angle), bond * math.sin(angle) * math.cos(torsion),
                   bond * math.sin(angle) * math.sin(torsion)])
    return c + d2[0] * bc + d2[1] * m + d2[2] * n


def _tetrahedron(rng):
    """Four unit vectors of a regular tetrahedron in a random orientation."""
    base = np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], dtype=float) / math.sqrt(3.0)
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    return base @ _quat_to_matrix(q).T


def _quat_to_matrix(q):
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def _alkane_geometry(parent, dihedral, rng):
    """Atoms of an alkane tree.  parent[k] is the carbon carbon k hangs from
    (-1 for the root); dihedral[k] rotates the three substituent slots of
    carbon k about its bond to its parent.  Returns (Z, xyz in Angstrom,
    bond list)."""
    n = len(parent)
    children = [[] for _ in range(n)]
    for k in range(1, n):
        children[parent[k]].append(k)
    pos = np.zeros((n, 3))
    ref = {}                                  # carbon -> reference atom position for its dihedral
    Z, xyz, bonds = [6] * n, [None] * n, []
    tet = _tetrahedron(rng)
    pos[0] = 0.0
    xyz[0] = pos[0]
    hs = []
    # root: children and hydrogens on the four tetrahedral directions
    slots0 = [pos[0] + CC * tet[i] for i in range(4)]
    for i, ch in enumerate(children[0]):
        pos[ch] = slots0[i]
        xyz[ch] = pos[ch]
        bonds.append((0, ch))
        ref[ch] = slots0[(i + 1) % 4]          # another root direction fixes the dihedral frame
    for i in range(len(children[0]), 4):
        hs.append((0, pos[0] + CH * tet[i]))
    order = list(children[0])
    while order:
        c = order.pop(0)
        p = parent[c]
        g = ref[c]
        for s in range(3):
            tor = dihedral[c] + s * 2.0 * math.pi / 3.0
            if s < len(children[c]):
                ch = children[c][s]
                pos[ch] = _place(g, pos[p], pos[c], CC, TET, tor)
                xyz[ch] = pos[ch]
                bonds.append((c, ch))
                ref[ch] = pos[p]
                order.append(ch)
            else:
                hs.append((c, _place(g, pos[p], pos[c], CH, TET, tor)))
    for c, h in hs:
        bonds.append((c, len(Z)))
        Z.append(1)
        xyz.append(h)
    return np.array(Z, dtype=np.int32), np.array(xyz), bonds


def octane() -> Molecule:
    """All-trans n-octane C8H18 (26 atoms, 50 basis functions): a linear chain
    with every C-C-C-C dihedral at 180 degrees."""
    n = 8
    parent = [-1] + list(range(n - 1))
    rng = np.random.default_rng(0)            # orientation only; geometry is ideal
    # with the chain built from carbon 0, the dihedral slot 0 of carbon k sits
    # anti to its grandparent when the reference atom is the grandparent
    dih = [0.0] + [math.pi] * (n - 1)
    Z, xyz, _ = _alkane_geometry(parent, dih, rng)
    # carbon 1's frame uses another root direction; make its slot anti to that
    # direction too (the root has no grandparent: any choice is still all-trans
    # for the C-C-C-C dihedrals, which start at carbon 0)
    return Molecule(Z, xyz * ANG2AU)


def _graph_distance(nat, bonds):
    adj = [[] for _ in range(nat)]
    for a, b in bonds:
        adj[a].append(b)
        adj[b].append(a)
    D = np.full((nat, nat), 99, dtype=np.int32)
    for s in range(nat):
        D[s, s] = 0
        frontier = [s]
        d = 0
        while frontier:
            d += 1
            nxt = []
            for u in frontier:
                for v in adj[u]:
                    if D[s, v] > d:
                        D[s, v] = d
                        nxt.append(v)
            frontier = nxt
    return D


_gen_lib = None


def _generator():
    """The C alkane generator (molds_gb300/_build/libworkloads.so, built with the CUDA library)."""
    global _gen_lib
    if _gen_lib is None:
        import ctypes
        import os
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "libworkloads.so")
        if not os.path.exists(path):
            raise ImportError(f"{path} is missing: build with `python -m molds_gb300.build`")
        L = ctypes.CDLL(path)
        L.alkane_generate.restype = ctypes.c_int
        L.alkane_generate.argtypes = [ctypes.c_ulonglong, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                      ctypes.c_longlong, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                      ctypes.POINTER(ctypes.c_double), ctypes.c_int]
        _gen_lib = L
    return _gen_lib


def alkane_carbons(seed: int, n_range=(3, 60)) -> int:
    """The carbon count random_alkane(seed) draws (uniform in n_range), without
    building the molecule: the basis size N = 6 n + 2 is what a cost-based
    sharder needs."""
    return int(np.random.default_rng(seed).integers(n_range[0], n_range[1] + 1))


def random_alkane(seed: int, n: int | None = None, n_range=(3, 60), min_dist=1.8, min_dist_h=1.0,
                  attempts=48, budget=200000, max_trees=400) -> Molecule:
    """A random saturated acyclic alkane CnH(2n+2).

    Topology: each new carbon attaches to a uniformly chosen carbon with < 4
    carbon neighbours.  Geometry: ideal bonds and tetrahedral angles; the
    molecule is grown carbon by carbon (breadth first) and each carbon's
    dihedral is drawn uniformly in [0, 2 pi).  A draw is rejected and redrawn
    when it puts two carbons >= 3 bonds apart closer than min_dist Angstrom, or
    any other pair >= 3 bonds apart closer than min_dist_h (1-2 and 1-3 pairs
    are exempt: a geminal H-H pair sits at 1.78 A).  Applying 1.8 A to H-H
    pairs as well leaves no acceptable geometry for most trees beyond ~15
    carbons when dihedrals are uniform (hydrogens 5-6 bonds apart meet below
    1.8 A in about half of random hexane conformations), so hydrogens get the
    looser floor.  A carbon that cannot be placed sends the search back to the
    carbon that owns a clashing atom; a tree that cannot be placed within
    `budget` draws is redrawn.  The growth runs in C (csrc/alkane_gen.c); n is
    drawn here from the seed."""
    import ctypes
    if n is None:
        n = alkane_carbons(seed, n_range)
    total = 3 * n + 2
    Z = np.zeros(total, dtype=np.int32)
    xyz = np.zeros((total, 3))
    k = _generator().alkane_generate(int(seed) & 0xFFFFFFFFFFFFFFFF, int(n), float(min_dist), float(min_dist_h),
                                     int(attempts), int(budget), int(max_trees),
                                     Z.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                     xyz.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), total)
    if k != total:
        raise RuntimeError(f"no acceptable geometry for n={n} (generator returned {k})")
    return Molecule(Z, xyz * ANG2AU)


def _grow_alkane(parent, rng, min_dist, min_dist_h, attempts=48, budget=40000, depth_first=False):
    """Places the carbons of a tree breadth first, drawing each carbon's
    dihedral uniformly; `attempts` draws are tested at once and one clash-free
    draw is kept.  When none is clash-free the search jumps back to the most
    recently placed carbon that owns one of the clashing atoms (conflict-
    directed backjumping) and redraws from there.  Returns None when `budget`
    draws did not produce a clash-free molecule."""
    n = len(parent)
    children = [[] for _ in range(n)]
    for k in range(1, n):
        children[parent[k]].append(k)
    order = []
    if depth_first:
        stack = list(reversed(children[0]))
        while stack:
            c = stack.pop()
            order.append(c)
            stack += list(reversed(children[c]))
    else:
        queue = list(children[0])
        while queue:
            c = queue.pop(0)
            order.append(c)
            queue += children[c]
    total = 3 * n + 2
    Z = np.zeros(total, dtype=np.int32)
    pos = np.zeros((total, 3))
    D = np.zeros((total, total), dtype=np.int32)   # bond-graph distances among placed atoms
    owner = np.full(total, -1, dtype=np.int64)     # order index of the carbon that placed an atom
    idx_of_c = [-1] * n
    ref = [None] * n
    count = 0

    def add(zz, p, bonded_to, t):
        nonlocal count
        i = count
        Z[i] = zz
        pos[i] = p
        owner[i] = t
        if bonded_to >= 0:
            D[i, :i] = D[bonded_to, :i] + 1
            D[:i, i] = D[i, :i]
        count += 1
        return i

    tet = _tetrahedron(rng)
    idx_of_c[0] = add(6, np.zeros(3), -1, -1)
    for i in range(4):
        if i < len(children[0]):
            ch = children[0][i]
            idx_of_c[ch] = add(6, CC * tet[i], idx_of_c[0], -1)
            ref[ch] = CC * tet[(i + 1) % 4]
        else:
            add(1, CH * tet[i], idx_of_c[0], -1)
    start_count = [0] * len(order)
    if order:
        start_count[0] = count
    t = 0
    draws = 0
    while t < len(order):
        if draws >= budget:
            return None
        c = order[t]
        count = start_count[t]
        ic, ip = idx_of_c[c], idx_of_c[parent[c]]
        kids = children[c]
        draws += attempts
        phis = rng.uniform(0.0, 2.0 * math.pi, size=attempts)
        bc = _unit(pos[ic] - pos[ip])
        nv = _unit(np.cross(pos[ip] - ref[c], bc))
        mv = np.cross(nv, bc)
        bonds = np.array([CC if s < len(kids) else CH for s in range(3)])
        tors = phis[:, None] + np.arange(3)[None, :] * (2.0 * math.pi / 3.0)
        cands = (pos[ic][None, None, :] - (bonds * math.cos(TET))[None, :, None] * bc
                 + (bonds * math.sin(TET))[None, :, None]
                 * (np.cos(tors)[..., None] * mv + np.sin(tors)[..., None] * nv))
        far = np.nonzero((D[ic, :count] + 1) >= 3)[0]
        if far.size:
            d2 = ((cands[:, :, None, :] - pos[far][None, None, :, :]) ** 2).sum(-1)
            both_c = (np.arange(3) < len(kids))[:, None] & (Z[far] == 6)[None, :]
            lim = np.where(both_c, min_dist * min_dist, min_dist_h * min_dist_h)
            bad = d2 < lim[None, :, :]
            good = np.nonzero(~np.any(bad, axis=(1, 2)))[0]
        else:
            good = np.arange(attempts)
        if good.size == 0:
            culprits = owner[far[np.any(bad, axis=(0, 1))]]
            # jump back to the latest carbon that placed a clashing atom (atoms
            # placed with the root belong to no draw: start over from the first)
            t = max(0, int(culprits.max())) if culprits.size else 0
            continue
        cand = cands[good[0]]
        for s in range(3):
            if s < len(kids):
                ch = kids[s]
                idx_of_c[ch] = add(6, cand[s], ic, t)
                ref[ch] = pos[ip].copy()
            else:
                add(1, cand[s], ic, t)
        t += 1
        if t < len(order):
            start_count[t] = count
    return Molecule(Z[:count].copy(), pos[:count] * ANG2AU)


def _water(rng, center):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    Rm = _quat_to_matrix(q)
    h1 = np.array([OH * math.sin(HOH / 2), 0.0, OH * math.cos(HOH / 2)])
    h2 = np.array([-OH * math.sin(HOH / 2), 0.0, OH * math.cos(HOH / 2)])
    return [center, center + Rm @ h1, center + Rm @ h2]


def water_cluster(shape=(4, 4, 2), spacing=2.9, jitter=0.2, seed=2) -> Molecule:
    """(H2O)_k on a jittered lattice: O at spacing * lattice index + U(-jitter, jitter)
    per coordinate, each water in a uniformly random orientation."""
    rng = np.random.default_rng(seed)
    Z, xyz = [], []
    for i in range(shape[0]):
        for j in range(shape[1]):
            for k in range(shape[2]):
                c = np.array([i, j, k], dtype=float) * spacing + rng.uniform(-jitter, jitter, size=3)
                for zz, p in zip((8, 1, 1), _water(rng, c)):
                    Z.append(zz)
                    xyz.append(p)
    return Molecule(np.array(Z, dtype=np.int32), np.array(xyz) * ANG2AU)


def water_replicas(base: Molecule, count: int, sigma=0.05, seed0=1000):
    """Replica i: every atom displaced by N(0, sigma Angstrom) per coordinate, seed seed0 + i."""
    out = []
    for i in range(count):
        rng = np.random.default_rng(seed0 + i)
        d = rng.normal(0.0, sigma, size=base.xyz.shape) * ANG2AU
        out.append(Molecule(base.Z.copy(), base.xyz + d))
    return out


def water_cluster_k(k: int, seed: int, spacing=2.9, jitter=0.2) -> Molecule:
    """k waters on the first k sites of a cubic lattice large enough to hold them."""
    side = max(1, int(math.ceil(k ** (1.0 / 3.0))))
    rng = np.random.default_rng(seed)
    Z, xyz = [], []
    count = 0
    for i in range(side):
        for j in range(side):
            for l in range(side):
                if count == k:
                    break
                c = np.array([i, j, l], dtype=float) * spacing + rng.uniform(-jitter, jitter, size=3)
                for zz, p in zip((8, 1, 1), _water(rng, c)):
                    Z.append(zz)
                    xyz.append(p)
                count += 1
    return Molecule(np.array(Z, dtype=np.int32), np.array(xyz) * ANG2AU)


def serving_stream(rate_hz: float, count: int, seed=5, min_atoms=5, max_atoms=500, max_alkane_n=60):
    """Poisson arrivals of single-point requests with sizes log-uniform in
    [min_atoms, max_atoms]: even requests are alkanes (n from the size,
    A = 3n + 2), odd ones water clusters (k = round(A / 3)).  The alkanes are
    those of the uneven-batch workload, whose n stops at max_alkane_n (182
    atoms); an alkane request above that size becomes a water cluster of the
    same size.  Returns [(arrival_s, Molecule)]."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(count):
        t += rng.exponential(1.0 / rate_hz)
        a = math.exp(rng.uniform(math.log(min_atoms), math.log(max_atoms)))
        n = max(1, int(round((a - 2) / 3)))
        if i % 2 == 0 and n <= max_alkane_n:
            mol = random_alkane(seed * 1000003 + i, n=n)
        else:
            k = max(1, int(round(a / 3)))
            mol = water_cluster_k(k, seed * 1000003 + i)
        out.append((t, mol))
    return out


def to_input_text(mol: Molecule, theory: str, scf: dict | None = None, limit_heap_mb: float | None = None) -> str:
    """The molecule as a MolDS input file (coordinates back in Angstrom)."""
    from .inputfile import Z_TO_SYMBOL
    lines = ["THEORY", f"   {theory}", "THEORY_END", ""]
    if scf:
        lines.append("SCF")
        for k, v in scf.items():
            lines.append(f"   {k} {v}")
        lines += ["SCF_END", ""]
    if limit_heap_mb:
        lines += ["MEMORY", f"   limit_heap {limit_heap_mb}", "MEMORY_END", ""]
    lines.append("GEOMETRY")
    for z, p in zip(mol.Z, mol.xyz / ANG2AU):
        lines.append(f"   {Z_TO_SYMBOL[int(z)]:<3s} {p[0]:.10f} {p[1]:.10f} {p[2]:.10f}")
    lines.append("GEOMETRY_END")
    return "\n".join(lines) + "\n"
