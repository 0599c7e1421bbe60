"""Atom-centred integration grids for the COSX exchange (seeded, no PySCF).

Becke's multicentre scheme (A. D. Becke, J. Chem. Phys. 88, 2547 (1988)):
each atom carries a radial x angular product grid, and the fuzzy-cell
weights w_A(r) = P_A(r) / sum_B P_B(r) with three iterations of
p(mu) = 1.5 mu - 0.5 mu^3 partition space.

* radial: Gauss-Chebyshev of the second kind mapped by r = R (1+x)/(1-x)
  (Becke's mapping), R a per-element length scale;
* angular: Gauss-Legendre in cos(theta) times a uniform phi rule (n_theta x
  2 n_theta points), exact for spherical harmonics up to degree
  2 n_theta - 1.

Points are returned in Morton (Z-curve) order of their coordinates, so that
every run of 32 consecutive points -- one COSX sub-block -- is spatially
compact; the screening bound depends on the sub-block radius.

When PySCF is present, its own SGX grids are used instead (the hook reads
``sgx.grids``); these grids stand in for them in the synthetic workloads.
"""
import numpy as np

# level -> (radial points for H/He, radial points for heavier atoms, n_theta)
GRID_LEVELS = {
    0: (20, 30, 6),
    1: (30, 40, 7),
    2: (38, 56, 8),
    3: (50, 70, 11),
    4: (60, 90, 14),
}

# Becke radial length scale per element (bohr)
_RADIAL_SCALE = {'H': 0.9, 'He': 0.9, 'C': 1.3, 'N': 1.2, 'O': 1.1,
                 'F': 1.0, 'S': 1.8, 'Cl': 1.7, 'Br': 1.9}


class Grids:
    """coords (N, 3) bohr, weights (N,), plus the build parameters."""

    def __init__(self, coords, weights, level):
        self.coords = np.ascontiguousarray(coords, dtype=np.float64)
        self.weights = np.ascontiguousarray(weights, dtype=np.float64)
        self.level = level
        self.non0tab = None

    @property
    def size(self):
        return self.weights.size


def radial_grid(n, scale):
    """(r, w) with sum_i w_i f(r_i) ~ int_0^inf f(r) r^2 dr."""
    i = np.arange(1, n + 1)
    x = np.cos(i * np.pi / (n + 1))
    wcheb = np.pi / (n + 1) * np.sin(i * np.pi / (n + 1)) ** 2
    # int_{-1}^{1} g(x) dx = sum wcheb g(x) / sqrt(1 - x^2)
    r = scale * (1.0 + x) / (1.0 - x)
    drdx = 2.0 * scale / (1.0 - x) ** 2
    w = wcheb / np.sqrt(1.0 - x * x) * drdx * r * r
    return r, w


def angular_grid(n_theta):
    """(xyz (M, 3), w (M,)) on the unit sphere, sum w = 4 pi."""
    ct, wt = np.polynomial.legendre.leggauss(n_theta)
    nphi = 2 * n_theta
    phi = (np.arange(nphi) + 0.5) * (2.0 * np.pi / nphi)
    st = np.sqrt(1.0 - ct * ct)
    xyz = np.stack([np.outer(st, np.cos(phi)).ravel(),
                    np.outer(st, np.sin(phi)).ravel(),
                    np.repeat(ct, nphi)], axis=1)
    w = np.repeat(wt, nphi) * (2.0 * np.pi / nphi)
    return xyz, w


def becke_weights_reference(points, atom_coords, owner):
    """Fuzzy-cell weight of each point's owning atom (NumPy; slow, used by
    the tests to check the native routine)."""
    n = points.shape[0]
    nat = atom_coords.shape[0]
    if nat == 1:
        return np.ones(n)
    dist = np.linalg.norm(points[:, None, :] - atom_coords[None, :, :], axis=2)
    rab = np.linalg.norm(atom_coords[:, None, :] - atom_coords[None, :, :],
                         axis=2)
    P = np.ones((n, nat))
    for a in range(nat):
        for b in range(nat):
            if a == b:
                continue
            mu = (dist[:, a] - dist[:, b]) / rab[a, b]
            for _ in range(3):
                mu = 1.5 * mu - 0.5 * mu ** 3
            P[:, a] *= 0.5 * (1.0 - mu)
    tot = P.sum(axis=1)
    return P[np.arange(n), owner] / tot


def _becke_weights(points, atom_coords, owner, partition=None):
    if atom_coords.shape[0] == 1:
        return np.ones(points.shape[0])
    if partition is None:
        from pyscf_wb97mv_fast_gb300.cosx import becke_partition as partition
    return partition(points, owner, atom_coords)


def morton_order(coords, bits=10):
    """Indices sorting points along a Z-curve of their coordinates."""
    lo = coords.min(axis=0)
    span = max(float((coords.max(axis=0) - lo).max()), 1e-12)
    q = np.floor((coords - lo) / span * ((1 << bits) - 1)).astype(np.int64)
    code = np.zeros(len(coords), dtype=np.int64)
    for b in range(bits):
        for ax in range(3):
            code |= ((q[:, ax] >> b) & 1) << (3 * b + ax)
    return np.argsort(code, kind='stable')


def build_grids(mol, level=2, prune=1e-15, order='morton', partition=None):
    """Becke grids for a Molecule (or anything with symbols/atom_coords).
    partition(points, owner, atom_coords) -> weights replaces the native
    Becke routine (the CPU baselines pass the oracle's)."""
    nrad_h, nrad_heavy, n_theta = GRID_LEVELS[level]
    ang_xyz, ang_w = angular_grid(n_theta)
    coords = mol.atom_coords()
    symbols = getattr(mol, 'symbols', None) or [
        mol.atom_symbol(i) for i in range(mol.natm)]
    pts, wts, own = [], [], []
    for ia, sym in enumerate(symbols):
        nr = nrad_h if sym in ('H', 'He') else nrad_heavy
        r, wr = radial_grid(nr, _RADIAL_SCALE.get(sym, 1.5))
        pts.append((r[:, None, None] * ang_xyz[None, :, :]).reshape(-1, 3)
                   + coords[ia])
        wts.append((wr[:, None] * ang_w[None, :]).ravel())
        own.append(np.full(len(pts[-1]), ia))
    pts = np.concatenate(pts)
    wts = np.concatenate(wts) * _becke_weights(pts, coords, np.concatenate(own),
                                               partition)
    keep = wts > prune
    pts, wts = pts[keep], wts[keep]
    if order == 'morton' and len(pts):
        idx = morton_order(pts)
        pts, wts = pts[idx], wts[idx]
    return Grids(pts, wts, level)
