"""Seeded synthetic molecules for the COSX workloads.

* ``water_cluster(n, box, seed)``: n rigid waters (O-H 0.9572 A, HOH
  104.52 deg), oxygen positions uniform in a cube of edge ``box`` A with
  rejection until every O-O distance is >= 2.7 A, orientations uniform on
  SO(3) from a normalised Gaussian quaternion (the rotation construction of
  ``pyscf_wb97mv_fast/core/testsystems.py:39-45``).
* ``alkane(n)``: all-trans CnH(2n+2), C-C 1.53 A, C-H 1.09 A, tetrahedral
  angles, zig-zag backbone in the xy plane.
* ``drug_like(seed)``: a seeded drug-like test molecule with the elements of
  small-molecule drugs (C, N, O, S, F, Cl, H): a benzene ring carrying the
  halogens and a side chain of C, N, O and S, filled with hydrogens.

* ``read_xyz(path_or_text)``: atoms of an XYZ file (count line, comment
  line, then ``symbol x y z`` in Angstrom), for validation molecules such
  as the reference's drug geometries (benchmarks/systems/drugs/*.xyz).

All coordinates are returned in Angstrom as [(symbol, (x, y, z))].
"""
import math

import numpy as np

OH = 0.9572
HOH = math.radians(104.52)


def _quat_rotation(q):
    a, b, c, d = q
    return np.array([
        [a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
        [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
        [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])


def water_cluster(n, box=7.0, seed=0, min_oo=2.7, max_tries=200000):
    """n seeded waters in a cube of edge box (Angstrom)."""
    rng = np.random.default_rng(seed)
    local = np.array([[0.0, 0.0, 0.0],
                      [OH, 0.0, 0.0],
                      [OH * math.cos(HOH), OH * math.sin(HOH), 0.0]])
    oxy = []
    tries = 0
    while len(oxy) < n:
        tries += 1
        if tries > max_tries:
            raise RuntimeError('could not place %d waters in a %.1f A box'
                               % (n, box))
        p = rng.uniform(0.0, box, 3)
        if all(np.linalg.norm(p - o) >= min_oo for o in oxy):
            oxy.append(p)
    atoms = []
    for o in oxy:
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        xyz = local @ _quat_rotation(q).T + o
        atoms += [('O', tuple(xyz[0])), ('H', tuple(xyz[1])),
                  ('H', tuple(xyz[2]))]
    return atoms


def alkane(n, cc=1.53, ch=1.09):
    """All-trans n-alkane CnH(2n+2) (Angstrom)."""
    tet = math.acos(-1.0 / 3.0)                 # 109.47 deg
    half = tet / 2.0
    # zig-zag backbone in the xy plane along x
    dx = cc * math.sin(half)
    dy = cc * math.cos(half)
    cs = [np.array([i * dx, (dy / 2.0) * (1 if i % 2 else -1), 0.0])
          for i in range(n)]
    atoms = [('C', tuple(c)) for c in cs]
    for i, c in enumerate(cs):
        # the two in-plane backbone bonds point along +-x and away in y; the
        # hydrogens sit out of plane, bisecting the opposite direction
        up = 1.0 if i % 2 == 0 else -1.0       # away from the backbone
        ydir = -up
        # two H: direction = cos(a) * (0, ydir, 0) +- sin(a) * (0, 0, 1),
        # with the H-C-H angle tetrahedral
        a = half
        for sz in (1.0, -1.0):
            d = np.array([0.0, ydir * math.cos(a), sz * math.sin(a)])
            atoms.append(('H', tuple(c + ch * d)))
    # terminal hydrogens continue the zig-zag along the chain axis
    for end, nb in ((0, 1), (n - 1, n - 2)):
        if n == 1:
            v = np.array([1.0, 0.0, 0.0])
        else:
            v = cs[end] - cs[nb]
            v /= np.linalg.norm(v)
        # reflect the bond across the local y axis to keep the zig-zag
        vv = np.array([v[0], -v[1], 0.0])
        vv /= np.linalg.norm(vv)
        atoms.append(('H', tuple(cs[end] + ch * vv)))
    return atoms


def read_xyz(src):
    """[(symbol, (x, y, z))] in Angstrom from an XYZ file path or its text.
    The first line gives the atom count, the second is a comment; element
    symbols are normalised to 'Xx' capitalisation."""
    if '\n' not in src:
        with open(src) as fh:
            src = fh.read()
    lines = src.strip('\n').splitlines()
    try:
        n = int(lines[0].split()[0])
    except (IndexError, ValueError):
        raise ValueError('XYZ: the first line must give the atom count')
    body = lines[2:2 + n]
    if len(body) != n:
        raise ValueError('XYZ: %d atoms announced, %d lines found' % (n, len(body)))
    atoms = []
    for ln in body:
        f = ln.split()
        if len(f) < 4:
            raise ValueError('XYZ: bad atom line %r' % ln)
        sym = f[0][0].upper() + f[0][1:].lower()
        atoms.append((sym, (float(f[1]), float(f[2]), float(f[3]))))
    return atoms


def water_dimer(seed=1):
    """Two waters in a 3.2 A box (the small parity system)."""
    return water_cluster(2, box=3.2, seed=seed)


# single-bond lengths (Angstrom) and valences for drug_like
_BOND = {('C', 'C'): 1.51, ('C', 'N'): 1.47, ('C', 'O'): 1.43, ('C', 'S'): 1.82,
         ('C', 'F'): 1.35, ('C', 'Cl'): 1.75, ('N', 'N'): 1.45, ('N', 'O'): 1.40,
         ('N', 'S'): 1.70, ('O', 'S'): 1.57, ('O', 'O'): 1.48, ('S', 'S'): 2.05}
_XH = {'C': 1.09, 'N': 1.01, 'O': 0.96, 'S': 1.34}
_VALENCE = {'C': 4, 'N': 3, 'O': 2, 'S': 2}


def _bond(a, b):
    return _BOND.get((a, b)) or _BOND[(b, a)]


def _unit(v):
    return v / np.linalg.norm(v)


def drug_like(seed=0, chain=('C', 'N', 'C', 'O', 'C', 'S', 'C'),
              halogens=('F', 'Cl'), max_tries=300):
    """Seeded drug-like molecule (Angstrom).  A planar benzene ring (C-C
    1.39 A) carries the halogens (C-F 1.35, C-Cl 1.75 A, radial) and, at
    ring carbon 0, a side chain with the elements of ``chain`` in seeded
    order, each single-bonded to the previous one (bond angle >= 100 deg,
    non-bonded heavy atoms >= 2.4 A apart).  Hydrogens fill the remaining
    valences (ring C: one; C 4, N 3, O 2, S 2) at X-H bond lengths, at
    >= 100 deg from the atom's other bonds and clear of the other atoms.
    Meant for integral tests, not chemistry."""
    rng = np.random.default_rng(seed)
    sym, pos, nbr = [], [], []

    def add(s, p, parent=None):
        sym.append(s)
        pos.append(np.asarray(p, dtype=np.float64))
        nbr.append([])
        if parent is not None:
            nbr[-1].append(parent)
            nbr[parent].append(len(sym) - 1)
        return len(sym) - 1

    for k in range(6):
        a = k * math.pi / 3.0
        add('C', (1.39 * math.cos(a), 1.39 * math.sin(a), 0.0))
    for k in range(6):
        nbr[k] += [(k + 1) % 6, (k + 5) % 6]
    for k, x in zip((2, 4), halogens):
        add(x, pos[k] * (1.0 + _bond('C', x) / 1.39), k)

    def clear(p, skip, heavy_min, h_min):
        for i, q in enumerate(pos):
            if i in skip:
                continue
            d = np.linalg.norm(p - q)
            if d < (h_min if sym[i] == 'H' else heavy_min):
                return False
        return True

    def direction(i, tries):
        bonds = [_unit(pos[j] - pos[i]) for j in nbr[i]]
        for _ in range(tries):
            v = _unit(rng.normal(size=3))
            if all(np.dot(v, b) <= math.cos(math.radians(100.0)) for b in bonds):
                return v
        return None

    order = list(chain)
    rng.shuffle(order)
    prev = 0
    for x in order:
        placed = False
        for _ in range(200):
            v = direction(prev, 200) if prev != 0 else _unit(pos[0])
            if v is None:
                break
            p = pos[prev] + _bond(sym[prev], x) * v
            if clear(p, {prev}, 2.4, 1.5):
                prev = add(x, p, prev)
                placed = True
                break
            if prev == 0:
                break
        if not placed:
            break
    heavy = len(sym)
    for i in range(heavy):
        s = sym[i]
        if s not in _VALENCE:
            continue
        free = (3 if i < 6 else _VALENCE[s]) - len(nbr[i])
        for _ in range(max(free, 0)):
            for t in range(max_tries):
                v = _unit(pos[i]) if (i < 6 and t == 0) else direction(i, 50)
                if v is None:
                    continue
                p = pos[i] + _XH[s] * v
                if clear(p, {i}, 1.9 if t < max_tries // 2 else 1.5, 1.4):
                    add('H', p, i)
                    break
    return [(s, tuple(float(c) for c in p)) for s, p in zip(sym, pos)]
