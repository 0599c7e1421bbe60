"""Molecules and spherical Gaussian basis sets in libcint conventions.

The COSX path needs, per shell: its centre, angular momentum l, primitive
exponents and contraction coefficients as libcint stores them (the radial
per-primitive normalisation folded in, each contracted function normalised),
plus the Cartesian -> real-spherical transform.  This module supplies those
without PySCF, and ``Molecule.from_pyscf`` reads them from a PySCF ``Mole``
when PySCF is importable (the attribute names mirror the ones the reference
reads: ``pyscf_wb97mv_fast/gpu/shellpairs.py:187-221``).

Conventions (restated from the mathematics):

* Cartesian order inside a shell: lx descending, then ly descending,
  lz = l - lx - ly (``pyscf_wb97mv_fast/gpu/ao_eval.py:39-43``).
* Spherical order: for l = 1 the components are (x, y, z); for l >= 2 the
  real solid harmonics run m = -l .. l.  ``cart2sph(l)`` (ncart, nsph) holds
  the coefficients of r^l Y_lm normalised on the unit sphere, built from
  the closed-form real solid harmonic expansion (Helgaker, Jorgensen, Olsen,
  "Molecular Electronic-Structure Theory", eq. 6.4.47-6.4.50) times
  sqrt((2l+1)/4pi).
* A primitive r^l exp(-a r^2) carries the radial norm 1/sqrt(int r^(2l+2)
  exp(-2 a r^2) dr); the contracted radial function is normalised to one.
  With the angular normalisation in ``cart2sph`` every spherical AO has unit
  norm.

Without PySCF the basis *data* is synthetic: element shell structures with
the primitive and contraction counts of def2-SVP / def2-TZVP (24 AOs per
water in 'synthetic-svp', 31 per C and 6 per H in 'synthetic-tzvp'),
even-tempered exponents, and contraction coefficients fitted to a Slater
radial function.  The conventions above are the same ones PySCF uses, but
the mapping to PySCF's own tables is not verified in this module.
"""
import math

import numpy as np

LMAX = 3                       # highest supported shell angular momentum (f)
ANGSTROM = 1.0 / 0.52917721092  # bohr per angstrom (CODATA 2010, PySCF's value)

_SYMBOL_Z = {'H': 1, 'He': 2, 'Li': 3, 'Be': 4, 'B': 5, 'C': 6, 'N': 7,
             'O': 8, 'F': 9, 'Ne': 10, 'S': 16, 'Cl': 17, 'Br': 35}


def cart_components(l):
    """[(lx, ly, lz)] in libcint order: lx descending, ly descending."""
    return [(lx, ly, l - lx - ly)
            for lx in range(l, -1, -1)
            for ly in range(l - lx, -1, -1)]


def ncart(l):
    return (l + 1) * (l + 2) // 2


def nsph(l):
    return 2 * l + 1


def _solid_harmonic_terms(l, m):
    """{(i, j, k): coeff} of the unnormalised real solid harmonic S_lm
    (Helgaker et al. 6.4.47-50), S_lm = sqrt(4pi/(2l+1)) r^l Y_lm."""
    am = abs(m)
    vm = 0.0 if m >= 0 else 0.5
    nlm = (1.0 / (2 ** am * math.factorial(l))) * math.sqrt(
        2.0 * math.factorial(l + am) * math.factorial(l - am)
        / (2.0 if m == 0 else 1.0))
    terms = {}
    for t in range((l - am) // 2 + 1):
        for u in range(t + 1):
            # v runs over vm, vm+1, ... <= floor(|m|/2 - vm) + vm
            v = vm
            vmax = math.floor(am / 2.0 - vm) + vm
            while v <= vmax + 1e-12:
                two_v = int(round(2 * v))
                c = ((-1) ** int(round(t + v - vm)) * 0.25 ** t
                     * math.comb(l, t) * math.comb(l - t, am + t)
                     * math.comb(t, u) * math.comb(am, two_v))
                # exponents: x^(2t+|m|-2(u+v)) y^(2(u+v)) z^(l-2t-|m|)
                ex = 2 * t + am - 2 * u - two_v
                ey = 2 * u + two_v
                ez = l - 2 * t - am
                key = (ex, ey, ez)
                terms[key] = terms.get(key, 0.0) + nlm * c
                v += 1.0
    return terms


def cart2sph(l):
    """(ncart(l), nsph(l)) FP64 Cartesian -> spherical coefficients, unit-
    sphere normalised, libcint column order (see module docstring)."""
    comps = cart_components(l)
    index = {c: n for n, c in enumerate(comps)}
    if l == 1:
        ms = [1, -1, 0]                       # x, y, z
    else:
        ms = list(range(-l, l + 1))
    out = np.zeros((len(comps), len(ms)))
    scale = math.sqrt((2 * l + 1) / (4.0 * math.pi))
    for col, m in enumerate(ms):
        for key, c in _solid_harmonic_terms(l, m).items():
            out[index[key], col] += c * scale
    return out


def gto_norm(l, a):
    """1/sqrt(int_0^inf r^(2l+2) exp(-2 a r^2) dr)."""
    a = np.asarray(a, dtype=np.float64)
    integral = math.gamma(l + 1.5) / (2.0 * (2.0 * a) ** (l + 1.5))
    return 1.0 / np.sqrt(integral)


def _radial_overlap(l, a, b):
    """int r^(2l+2) exp(-(a+b) r^2) dr for exponent vectors a, b (outer)."""
    s = np.add.outer(a, b)
    return math.gamma(l + 1.5) / (2.0 * s ** (l + 1.5))


def normalize_contraction(l, exps, raw):
    """libcint-style coefficients: raw (nprim, nctr) -> each primitive times
    gto_norm, then each contracted radial function scaled to unit norm."""
    exps = np.asarray(exps, dtype=np.float64)
    c = np.asarray(raw, dtype=np.float64).reshape(len(exps), -1)
    c = c * gto_norm(l, exps)[:, None]
    s = _radial_overlap(l, exps, exps)
    for k in range(c.shape[1]):
        nrm = float(c[:, k] @ s @ c[:, k])
        c[:, k] /= math.sqrt(nrm)
    return c


class Shell:
    """One shell: atom index, l, exponents (nprim,), libcint coefficients
    (nprim, nctr)."""

    __slots__ = ('atom', 'l', 'exps', 'coeffs')

    def __init__(self, atom, l, exps, coeffs):
        self.atom = int(atom)
        self.l = int(l)
        self.exps = np.asarray(exps, dtype=np.float64).copy()
        self.coeffs = np.asarray(coeffs, dtype=np.float64).reshape(
            len(self.exps), -1).copy()

    @property
    def nprim(self):
        return len(self.exps)

    @property
    def nctr(self):
        return self.coeffs.shape[1]

    @property
    def nao(self):
        return self.nctr * nsph(self.l)


# -- synthetic basis data ------------------------------------------------------
# (l, nprim, largest exponent, ratio) per shell; even-tempered exponents
# a_k = amax / ratio^k.  Primitive and contraction counts follow the def2
# shell structures; the exponent values are synthetic.
_SYNTH = {
    'synthetic-svp': {
        'H': [(0, 3, 13.0, 4.5), (0, 1, 0.12, 1.0), (1, 1, 0.80, 1.0)],
        'C': [(0, 5, 1400.0, 4.6), (0, 1, 0.50, 1.0), (0, 1, 0.15, 1.0),
              (1, 3, 10.0, 4.3), (1, 1, 0.17, 1.0), (2, 1, 0.55, 1.0)],
        'N': [(0, 5, 1700.0, 4.6), (0, 1, 0.62, 1.0), (0, 1, 0.19, 1.0),
              (1, 3, 13.0, 4.3), (1, 1, 0.22, 1.0), (2, 1, 0.85, 1.0)],
        'O': [(0, 5, 2200.0, 4.6), (0, 1, 0.75, 1.0), (0, 1, 0.23, 1.0),
              (1, 3, 16.0, 4.3), (1, 1, 0.27, 1.0), (2, 1, 1.20, 1.0)],
        'F': [(0, 5, 2900.0, 4.6), (0, 1, 0.95, 1.0), (0, 1, 0.29, 1.0),
              (1, 3, 20.0, 4.3), (1, 1, 0.33, 1.0), (2, 1, 1.40, 1.0)],
        'S': [(0, 5, 40000.0, 5.5), (0, 3, 40.0, 3.0), (0, 1, 0.45, 1.0),
              (0, 1, 0.17, 1.0), (1, 5, 300.0, 3.5), (1, 1, 0.35, 1.0),
              (1, 1, 0.12, 1.0), (2, 1, 0.48, 1.0)],
        'Cl': [(0, 5, 48000.0, 5.5), (0, 3, 50.0, 3.0), (0, 1, 0.55, 1.0),
               (0, 1, 0.21, 1.0), (1, 5, 360.0, 3.5), (1, 1, 0.42, 1.0),
               (1, 1, 0.14, 1.0), (2, 1, 0.65, 1.0)],
        # [5s4p2d]
        'Br': [(0, 6, 400000.0, 6.0), (0, 4, 400.0, 3.5), (0, 2, 10.0, 3.0),
               (0, 1, 0.40, 1.0), (0, 1, 0.14, 1.0),
               (1, 5, 2000.0, 4.5), (1, 3, 40.0, 3.0), (1, 1, 0.40, 1.0),
               (1, 1, 0.13, 1.0), (2, 4, 100.0, 3.5), (2, 1, 0.50, 1.0)],
    },
    'synthetic-tzvp': {
        'H': [(0, 3, 34.0, 5.0), (0, 1, 0.32, 1.0), (0, 1, 0.10, 1.0),
              (1, 1, 0.80, 1.0)],
        'C': [(0, 6, 13500.0, 6.0), (0, 2, 18.0, 3.0), (0, 1, 0.55, 1.0),
              (0, 1, 0.22, 1.0), (0, 1, 0.09, 1.0),
              (1, 4, 35.0, 4.0), (1, 1, 0.35, 1.0), (1, 1, 0.11, 1.0),
              (2, 1, 1.10, 1.0), (2, 1, 0.32, 1.0), (3, 1, 0.76, 1.0)],
        'N': [(0, 6, 19700.0, 6.0), (0, 2, 26.0, 3.0), (0, 1, 0.80, 1.0),
              (0, 1, 0.31, 1.0), (0, 1, 0.12, 1.0),
              (1, 4, 50.0, 4.0), (1, 1, 0.50, 1.0), (1, 1, 0.15, 1.0),
              (2, 1, 1.65, 1.0), (2, 1, 0.47, 1.0), (3, 1, 1.10, 1.0)],
        'O': [(0, 6, 27000.0, 6.0), (0, 2, 35.0, 3.0), (0, 1, 1.10, 1.0),
              (0, 1, 0.42, 1.0), (0, 1, 0.16, 1.0),
              (1, 4, 63.0, 4.0), (1, 1, 0.64, 1.0), (1, 1, 0.19, 1.0),
              (2, 1, 2.30, 1.0), (2, 1, 0.65, 1.0), (3, 1, 1.43, 1.0)],
        'F': [(0, 6, 35000.0, 6.0), (0, 2, 45.0, 3.0), (0, 1, 1.40, 1.0),
              (0, 1, 0.53, 1.0), (0, 1, 0.20, 1.0),
              (1, 4, 80.0, 4.0), (1, 1, 0.80, 1.0), (1, 1, 0.24, 1.0),
              (2, 1, 3.00, 1.0), (2, 1, 0.85, 1.0), (3, 1, 1.85, 1.0)],
        'S': [(0, 6, 100000.0, 6.0), (0, 3, 160.0, 3.5), (0, 1, 2.00, 1.0),
              (0, 1, 0.55, 1.0), (0, 1, 0.20, 1.0),
              (1, 5, 600.0, 4.0), (1, 2, 4.00, 3.0), (1, 1, 0.45, 1.0),
              (1, 1, 0.15, 1.0), (2, 1, 1.50, 1.0), (2, 1, 0.40, 1.0),
              (3, 1, 0.56, 1.0)],
        'Cl': [(0, 6, 120000.0, 6.0), (0, 3, 190.0, 3.5), (0, 1, 2.40, 1.0),
               (0, 1, 0.66, 1.0), (0, 1, 0.24, 1.0),
               (1, 5, 700.0, 4.0), (1, 2, 4.80, 3.0), (1, 1, 0.55, 1.0),
               (1, 1, 0.18, 1.0), (2, 1, 1.90, 1.0), (2, 1, 0.52, 1.0),
               (3, 1, 0.70, 1.0)],
        # [6s5p4d1f]
        'Br': [(0, 8, 1200000.0, 5.5), (0, 3, 600.0, 3.5), (0, 2, 20.0, 3.0),
               (0, 1, 1.50, 1.0), (0, 1, 0.45, 1.0), (0, 1, 0.15, 1.0),
               (1, 6, 4000.0, 4.5), (1, 3, 60.0, 3.0), (1, 1, 2.50, 1.0),
               (1, 1, 0.45, 1.0), (1, 1, 0.15, 1.0),
               (2, 4, 150.0, 3.5), (2, 1, 3.00, 1.0), (2, 1, 0.90, 1.0),
               (2, 1, 0.30, 1.0), (3, 1, 0.50, 1.0)],
    },
}


def _slater_fit(l, exps, zeta):
    """Coefficients of sum_k c_k r^l exp(-a_k r^2) fitted (least squares in
    the radial L2 metric) to r^l exp(-zeta r); returned raw (unnormalised,
    the caller normalises)."""
    # radial quadrature: r in (0, 40] bohr on a log grid
    x = np.linspace(-9.0, math.log(40.0), 4000)
    r = np.exp(x)
    w = np.gradient(r) * r ** 2
    g = (r[None, :] ** l) * np.exp(-np.outer(exps, r ** 2))
    g *= gto_norm(l, exps)[:, None]
    target = r ** l * np.exp(-zeta * r)
    m = (g * w) @ g.T
    b = (g * w) @ target
    c = np.linalg.solve(m, b)
    return c * gto_norm(l, exps)


def synthetic_shells(symbol, basis, gen_contract=False):
    """[(l, exps, raw coeffs (nprim, nctr))] of one element."""
    table = _SYNTH[basis]
    if symbol not in table:
        raise ValueError('no %s data for element %s' % (basis, symbol))
    out = []
    for (l, nprim, amax, ratio) in table[symbol]:
        exps = amax / ratio ** np.arange(nprim)
        if nprim == 1:
            raw = np.ones((1, 1))
        else:
            # Slater exponent matched to the geometric middle of the set
            zeta = 1.3 * math.sqrt(float(np.sqrt(exps[0] * exps[-1])))
            raw = _slater_fit(l, exps, zeta)[:, None]
        out.append((l, exps, raw))
    if gen_contract:
        # test variant: the first contracted shell of each l also carries a
        # second contraction over the same primitives (nctr = 2)
        merged = []
        for (l, exps, raw) in out:
            if raw.shape[0] > 1 and not any(m[0] == l and m[2].shape[1] > 1
                                            for m in merged):
                alt = np.cos(np.arange(raw.shape[0]) * 1.3)[:, None] \
                    * np.abs(raw)
                raw = np.hstack([raw, alt])
            merged.append((l, exps, raw))
        out = merged
    return out


class Molecule:
    """Atoms (bohr) plus a list of Shells.  Exposes the PySCF Mole accessors
    the COSX path reads (``nbas``, ``nao``, ``ao_loc_nr``, ``bas_*``,
    ``_libcint_ctr_coeff``, ``atom_coords``), so code written against a Mole
    also runs on it."""

    cart = False

    def __init__(self, symbols, coords_bohr, shells, basis_name='custom'):
        self.symbols = list(symbols)
        self._coords = np.asarray(coords_bohr, dtype=np.float64).reshape(-1, 3)
        self.shells = list(shells)
        self.basis = basis_name
        self.omega = 0.0
        for sh in self.shells:
            if sh.l > LMAX:
                raise ValueError('shell l=%d above LMAX=%d' % (sh.l, LMAX))
        ao = [0]
        for sh in self.shells:
            ao.append(ao[-1] + sh.nao)
        self._ao_loc = np.asarray(ao, dtype=np.int64)
        self._bas = np.asarray([[sh.atom, sh.l, sh.nprim, sh.nctr]
                                for sh in self.shells], dtype=np.int64
                               ).reshape(-1, 4)

    # -- construction -------------------------------------------------------
    @classmethod
    def build(cls, atoms, basis='synthetic-svp', unit='angstrom',
              gen_contract=False):
        """atoms: [(symbol, (x, y, z))]; basis: a synthetic basis name."""
        symbols = [a[0] for a in atoms]
        xyz = np.asarray([a[1] for a in atoms], dtype=np.float64)
        if unit.lower().startswith('ang'):
            xyz = xyz * ANGSTROM
        shells = []
        for ia, sym in enumerate(symbols):
            for (l, exps, raw) in synthetic_shells(sym, basis, gen_contract):
                shells.append(Shell(ia, l, exps,
                                    normalize_contraction(l, exps, raw)))
        return cls(symbols, xyz, shells, basis)

    @classmethod
    def from_pyscf(cls, mol):
        """Read atoms and shells from a PySCF Mole (spherical only)."""
        if mol.cart:
            raise ValueError('only spherical bases are supported')
        shells = []
        for sh in range(mol.nbas):
            if int(mol.bas_kappa(sh)) != 0:
                raise ValueError('spinor shells are not supported')
            coeff = np.asarray(mol._libcint_ctr_coeff(sh), dtype=np.float64)
            shells.append(Shell(int(mol._bas[sh, 0]), int(mol.bas_angular(sh)),
                                np.asarray(mol.bas_exp(sh), dtype=np.float64),
                                coeff))
        symbols = [mol.atom_symbol(i) for i in range(mol.natm)]
        out = cls(symbols, mol.atom_coords(), shells, str(mol.basis))
        return out

    # -- PySCF-style accessors ----------------------------------------------
    @property
    def natm(self):
        return len(self.symbols)

    @property
    def nbas(self):
        return len(self.shells)

    @property
    def nao(self):
        return int(self._ao_loc[-1])

    @property
    def nelectron(self):
        return int(sum(_SYMBOL_Z[s] for s in self.symbols))

    def atom_charges(self):
        """Nuclear charges (all-electron) of the atoms."""
        return np.array([_SYMBOL_Z[s] for s in self.symbols], dtype=np.int64)

    def energy_nuc(self):
        """Nuclear repulsion energy (hartree) of the point charges."""
        z = self.atom_charges().astype(np.float64)
        r = self._coords
        e = 0.0
        for i in range(len(z)):
            d = np.linalg.norm(r[:i] - r[i], axis=1)
            e += float(np.sum(z[i] * z[:i] / d))
        return e

    def ao_loc_nr(self):
        return self._ao_loc.copy()

    def atom_coords(self):
        return self._coords.copy()

    def bas_angular(self, i):
        return self.shells[i].l

    def bas_nctr(self, i):
        return self.shells[i].nctr

    def bas_nprim(self, i):
        return self.shells[i].nprim

    def bas_kappa(self, i):
        return 0

    def bas_atom(self, i):
        return self.shells[i].atom

    def bas_exp(self, i):
        return self.shells[i].exps.copy()

    def _libcint_ctr_coeff(self, i):
        return self.shells[i].coeffs.copy()

    def bas_coord(self, i):
        return self._coords[self.shells[i].atom].copy()

    # -- packed arrays (the C-ABI basis description) --------------------------
    def packed(self):
        """Flat arrays describing the basis for the C-ABI / the oracle:
        shell_atom, shell_l, shell_nprim, shell_nctr (int32, nbas), shell
        exponent/coefficient offsets (int32, nbas), exps (FP64), coeffs
        (FP64, per shell (nprim, nctr) row-major), atom coords (FP64)."""
        nb = self.nbas
        sa = np.zeros(nb, np.int32)
        sl = np.zeros(nb, np.int32)
        sp = np.zeros(nb, np.int32)
        sc = np.zeros(nb, np.int32)
        eo = np.zeros(nb, np.int32)
        co = np.zeros(nb, np.int32)
        exps, coeffs = [], []
        ne = nc = 0
        for i, sh in enumerate(self.shells):
            sa[i], sl[i], sp[i], sc[i] = sh.atom, sh.l, sh.nprim, sh.nctr
            eo[i], co[i] = ne, nc
            exps.append(sh.exps)
            coeffs.append(sh.coeffs.ravel())
            ne += sh.nprim
            nc += sh.nprim * sh.nctr
        return {
            'natm': self.natm, 'nbas': nb, 'nao': self.nao,
            'atom_coords': np.ascontiguousarray(self._coords, np.float64),
            'shell_atom': sa, 'shell_l': sl, 'shell_nprim': sp,
            'shell_nctr': sc, 'shell_exp_off': eo, 'shell_coef_off': co,
            'exps': np.ascontiguousarray(np.concatenate(exps) if exps
                                         else np.zeros(0)),
            'coeffs': np.ascontiguousarray(np.concatenate(coeffs) if coeffs
                                           else np.zeros(0)),
            'ao_loc': self._ao_loc.astype(np.int32),
        }
