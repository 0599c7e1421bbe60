"""Seeded synthetic molecules for the COSX workloads.

* ``water_cluster(n, box, seed)``: n rigid waters (O-H 0.9572 A, HOH
  104.52 deg), oxygen positions uniform in a cube of edge ``box`` A with
  rejection until every O-O distance is >= 2.7 A, orientations uniform on
  SO(3) from a normalised Gaussian quaternion (the rotation construction of
  ``pyscf_wb97mv_fast/core/testsystems.py:39-45``).
* ``alkane(n)``: all-trans CnH(2n+2), C-C 1.53 A, C-H 1.09 A, tetrahedral
  angles, zig-zag backbone in the xy plane.

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


def water_dimer(seed=1):
    """Two waters in a 3.2 A box (the small parity system)."""
    return water_cluster(2, box=3.2, seed=seed)
