"""Molecules and contracted Gaussian basis sets for the AO integral source.

This module stands in for the psi4 set-up calls of apyib/hamiltonian.py:16-26
and apyib/integrals.py:17-28: ``psi4.geometry`` on apyib's geometry strings
(apyib/data/molecules.py), ``psi4.core.BasisSet.build`` for a named basis,
``Molecule.nuclear_repulsion_energy(dipole_field)`` (apyib/hamiltonian.py:61)
and ``BasisSet.nbf() / n_frozen_core()`` (apyib/utils.py:186-188).

Conventions (those of psi4's shell objects, as apyib/integrals.py:35-50 reads them):
  * shells in the order of the atoms, and on each atom in the order of the
    basis-set file; an SP shell is an S shell followed by a P shell with the
    same exponents;
  * Cartesian components of a shell of angular momentum l in the order
    ``for i in 0..l: for j in 0..i: (l-i, i-j, j)``  (x^l first, z^l last);
  * every primitive carries the normalisation of its x^l component,
    N = (2a/pi)^(3/4) (4a)^(l/2) / sqrt((2l-1)!!), and the contraction is scaled
    so that the x^l component of the contracted function has unit norm;
  * pure (spherical) shells are real solid harmonics in the order
    m = 0, +1, -1, +2, -2, ..., each of unit norm, formed from the Cartesian
    functions above; a basis set is pure or Cartesian as a whole.

The built-in data are the published contractions (STO-3G and STO-6G: Hehre,
Stewart and Pople, J. Chem. Phys. 51, 2657 (1969); 6-31G: Hehre, Ditchfield and Pople,
J. Chem. Phys. 56, 2257 (1972), Ditchfield, Hehre and Pople, J. Chem. Phys. 54,
724 (1971); 6-31G(d) polarisation exponent 0.8 on N and O: Hariharan and Pople,
Theor. Chim. Acta 28, 213 (1973); cc-pVDZ: Dunning, J. Chem. Phys. 90, 1007 (1989))
for the elements apyib's tests use (H, N, O).  The last three exponents of the
oxygen STO-6G 2sp shell are from the same least-squares fit of the 2s and 2p
Slater functions (shared exponents, zeta = 2.25) re-done in high precision; it
reproduces the published first three exponents to 3e-8 and all twelve
contraction coefficients.  Further sets are added at run time
with ``register_basis(name, text)`` from Gaussian-94 formatted text, the
format of psi4's basis library files.
"""
from __future__ import annotations

import math
import re
from dataclasses import dataclass, field

import numpy as np

# psi4's conversion factor (CODATA 2014)
BOHR_PER_ANGSTROM = 1.0 / 0.52917721067

_SYMBOLS = ("X H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn "
            "Ga Ge As Se Br Kr").split()
Z_OF = {s.upper(): z for z, s in enumerate(_SYMBOLS) if z > 0}
_AM = {"S": 0, "P": 1, "D": 2, "F": 3, "G": 4}


# ----------------------------------------------------------------------------- molecule
class Molecule(object):
    """The subset of psi4.core.Molecule that apyib's hot path reads."""

    def __init__(self, symbols, Z, xyz, charge=0, multiplicity=1):
        self.symbols = list(symbols)
        self.Z = np.asarray(Z, dtype=np.int64)
        self.xyz = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)     # bohr
        self.charge = charge
        self.multiplicity = multiplicity

    def natom(self):
        return len(self.symbols)

    def Z_of(self, a):
        return float(self.Z[a])

    def true_atomic_number(self, a):
        return int(self.Z[a])

    def geometry(self):
        return self.xyz.copy()

    def nuclear_dipole(self):
        return (self.Z[:, None] * self.xyz).sum(axis=0)

    def set_geometry(self, xyz):
        """New Cartesian coordinates in bohr (psi4's Molecule.set_geometry)."""
        xyz = np.asarray(getattr(xyz, "np", xyz), dtype=np.float64).reshape(-1, 3)
        if xyz.shape[0] != self.natom():
            raise ValueError("set_geometry: wrong number of atoms")
        self.xyz = xyz.copy()

    def create_psi4_string_from_molecule(self):
        """A geometry string that parse_geometry reads back to the same molecule
        (bohr, frame fixed; coordinates in full double precision)."""
        lines = [f"{self.charge} {self.multiplicity}"]
        for sym, r in zip(self.symbols, self.xyz):
            lines.append(f"{sym.capitalize()} {float(r[0])!r} {float(r[1])!r} {float(r[2])!r}")
        lines += ["units bohr", "no_com", "no_reorient", "symmetry c1"]
        return "\n".join(lines) + "\n"

    def nuclear_repulsion_energy(self, dipole_field=(0.0, 0.0, 0.0)):
        """sum_{A<B} Z_A Z_B / R_AB + field . sum_A Z_A R_A (psi4's Molecule method,
        called by apyib/hamiltonian.py:58-61 with the negated electric field)."""
        e = 0.0
        for a in range(self.natom()):
            for b in range(a):
                e += self.Z[a] * self.Z[b] / np.linalg.norm(self.xyz[a] - self.xyz[b])
        f = np.asarray(dipole_field, dtype=np.float64)
        if np.any(f != 0.0):
            e += float(f @ self.nuclear_dipole())
        return float(e)


def parse_geometry(text: str) -> Molecule:
    """A psi4-style Cartesian geometry string: one ``symbol x y z`` line per atom,
    an optional ``charge multiplicity`` line and the keywords apyib's strings use
    (``units bohr|angstrom``, ``symmetry``, ``no_com``/``nocom``,
    ``no_reorient``/``noreorient``).  Coordinates are taken as given: the strings
    of apyib/data/molecules.py all fix the frame with no_com and no_reorient."""
    symbols, Z, xyz = [], [], []
    charge, mult = 0, 1
    scale = BOHR_PER_ANGSTROM
    for raw in text.splitlines():
        line = raw.split("#")[0].strip()
        if not line:
            continue
        tok = line.split()
        key = tok[0].lower()
        if key == "units":
            u = tok[1].lower()
            if u in ("bohr", "au", "a.u."):
                scale = 1.0
            elif u in ("angstrom", "ang", "a"):
                scale = BOHR_PER_ANGSTROM
            else:
                raise ValueError(f"unknown units {tok[1]!r}")
            continue
        if key in ("symmetry", "no_com", "nocom", "no_reorient", "noreorient"):
            continue
        if len(tok) == 2 and all(re.fullmatch(r"[+-]?\d+", t) for t in tok):
            charge, mult = int(tok[0]), int(tok[1])
            continue
        if len(tok) == 4:
            sym = re.sub(r"[^A-Za-z].*$", "", tok[0]).upper()
            if sym not in Z_OF:
                raise ValueError(f"unknown element in {line!r}")
            symbols.append(sym)
            Z.append(Z_OF[sym])
            xyz.append([float(t) for t in tok[1:]])
            continue
        raise ValueError(f"cannot parse geometry line {line!r}")
    mol = Molecule(symbols, Z, np.array(xyz) * 1.0, charge, mult)
    mol.xyz = mol.xyz * scale
    return mol


# ----------------------------------------------------------------------------- basis library
_LIBRARY: dict = {}


def _parse_g94(text: str):
    """Gaussian-94 basis text -> (pure, {element: [(l, exps, coefs), ...]})."""
    pure = None
    lines = [ln.split("!")[0].rstrip() for ln in text.splitlines()]
    lines = [ln for ln in lines if ln.strip()]
    out, i = {}, 0
    while i < len(lines):
        tok = lines[i].split()
        low = tok[0].lower()
        if low in ("spherical", "cartesian"):
            pure = low == "spherical"
            i += 1
            continue
        if tok[0] == "****":
            i += 1
            continue
        el = tok[0].upper()
        if el not in Z_OF:
            raise ValueError(f"basis text: expected an element, got {lines[i]!r}")
        i += 1
        shells = []
        while i < len(lines) and lines[i].split()[0] != "****":
            head = lines[i].split()
            am, nprim = head[0].upper(), int(head[1])
            rows = [[float(x.replace("D", "E").replace("d", "e")) for x in lines[i + 1 + k].split()]
                    for k in range(nprim)]
            rows = np.array(rows)
            if am == "SP":
                shells.append((0, rows[:, 0].copy(), rows[:, 1].copy()))
                shells.append((1, rows[:, 0].copy(), rows[:, 2].copy()))
            else:
                shells.append((_AM[am], rows[:, 0].copy(), rows[:, 1].copy()))
            i += 1 + nprim
        out[el] = shells
    return pure, out


def register_basis(name: str, text: str, pure: bool | None = None):
    """Add (or extend) a named basis set from Gaussian-94 text.  ``pure`` overrides
    a ``spherical``/``cartesian`` header line; without either, Cartesian."""
    p, shells = _parse_g94(text)
    if pure is None:
        pure = bool(p)
    key = name.lower()
    entry = _LIBRARY.setdefault(key, {"pure": pure, "elements": {}})
    entry["pure"] = pure
    entry["elements"].update(shells)


register_basis("sto-3g", """
spherical
****
H     0
S   3   1.00
      3.42525091             0.15432897
      0.62391373             0.53532814
      0.16885540             0.44463454
****
O     0
S   3   1.00
    130.7093200              0.15432897
     23.8088610              0.53532814
      6.4436083              0.44463454
SP   3   1.00
      5.0331513             -0.09996723             0.15591627
      1.1695961              0.39951283             0.60768372
      0.3803890              0.70011547             0.39195739
****
""")



register_basis("sto-6g", """
spherical
****
H     0
S   6   1.00
     35.52322122             0.00916359628
      6.513143725            0.04936149294
      1.822142904            0.16853830490
      0.625955266            0.37056279970
      0.243076747            0.41649152980
      0.100112428            0.13033408410
****
O     0
S   6   1.00
   1355.584234               0.00916359628
    248.5448855              0.04936149294
     69.53390229             0.16853830490
     23.88677211             0.37056279970
      9.275932609            0.41649152980
      3.820341298            0.13033408410
SP   6   1.00
     52.18776196            -0.01325278809           0.003759696623
     10.32932006            -0.04699171014           0.03767936984
      3.210344977           -0.03378537151           0.1738967435
      1.235135423            0.2502417861            0.4180364347
      0.5364201589           0.5951172526            0.4258595477
      0.2458806068           0.2407061763            0.1017082955
****
""")


_631G_D_O = """
D   1   1.00
      0.8000000              1.0000000
"""


def _with_polarisation(text, element, extra):
    """Append shells to one element block of Gaussian-94 text."""
    head = f"{element}     0\n"
    start = text.index(head)
    end = text.index("****", start)
    return text[:end] + extra.lstrip("\n") + text[end:]


_631G_TEXT = """
****
H     0
S   3   1.00
     18.7311370              0.03349460
      2.8253937              0.23472695
      0.6401217              0.81375733
S   1   1.00
      0.1612778              1.0000000
****
O     0
S   6   1.00
   5484.6717000              0.0018311
    825.2349500              0.0139501
    188.0469600              0.0684451
     52.9645000              0.2327143
     16.8975700              0.4701930
      5.7996353              0.3585209
SP   3   1.00
     15.5396160             -0.1107775              0.0708743
      3.5999336             -0.1480263              0.3397528
      1.0137618              1.1307670              0.7271586
SP   1   1.00
      0.2700058              1.0000000              1.0000000
****
N     0
S   6   1.00
   4173.5110000              0.0018348
    627.4579000              0.0139950
    142.9021000              0.0685870
     40.2343300              0.2322410
     12.8202100              0.4690700
      4.3904370              0.3604550
SP   3   1.00
     11.6263580             -0.1149610              0.0675800
      2.7162800             -0.1691180              0.3239070
      0.7722180              1.1458520              0.7408950
SP   1   1.00
      0.2120313              1.0000000              1.0000000
****
"""
register_basis("6-31g", _631G_TEXT, pure=False)
for _name in ("6-31g(d)", "6-31g*"):
    register_basis(_name, _with_polarisation(_with_polarisation(_631G_TEXT, "O", _631G_D_O), "N", _631G_D_O),
                   pure=False)

register_basis("cc-pvdz", """
spherical
****
H     0
S   3   1.00
     13.0100000              0.0196850
      1.9620000              0.1379770
      0.4446000              0.4781480
S   1   1.00
      0.1220000              1.0000000
P   1   1.00
      0.7270000              1.0000000
****
O     0
S   8   1.00
  11720.0000000              0.0007100
   1759.0000000              0.0054700
    400.8000000              0.0278370
    113.7000000              0.1048000
     37.0300000              0.2830620
     13.2700000              0.4487190
      5.0250000              0.2709520
      1.0130000              0.0154580
S   8   1.00
  11720.0000000             -0.0001600
   1759.0000000             -0.0012630
    400.8000000             -0.0062670
    113.7000000             -0.0257160
     37.0300000             -0.0709240
     13.2700000             -0.1654110
      5.0250000             -0.1169550
      1.0130000              0.5573680
S   1   1.00
      0.3023000              1.0000000
P   3   1.00
     17.7000000              0.0430180
      3.8540000              0.2289130
      1.0460000              0.5087280
P   1   1.00
      0.2753000              1.0000000
D   1   1.00
      1.1850000              1.0000000
****
""")


def _library_entry(name):
    key = name.lower()
    if key not in _LIBRARY:
        raise KeyError(f"basis set {name!r} is not in the library; add it with register_basis(name, text)")
    return _LIBRARY[key]


def available_basis_sets():
    return sorted(_LIBRARY)


# ----------------------------------------------------------------------------- shells
def _dfact(n):
    """(n)!! with (-1)!! = 1."""
    r = 1
    while n > 1:
        r *= n
        n -= 2
    return r


def cartesian_components(l):
    return [(l - i, i - j, j) for i in range(l + 1) for j in range(i + 1)]


def normalized_coefficients(l, exps, coefs):
    """Contraction coefficients times the primitive normalisation of the x^l
    component, scaled so that the contracted x^l function has unit norm."""
    exps = np.asarray(exps, dtype=np.float64)
    c = np.asarray(coefs, dtype=np.float64)
    Np = (2.0 * exps / math.pi) ** 0.75 * (4.0 * exps) ** (l / 2.0) / math.sqrt(_dfact(2 * l - 1))
    d = c * Np
    pij = exps[:, None] + exps[None, :]
    S = (math.pi / pij) ** 1.5 * _dfact(2 * l - 1) / (2.0 * pij) ** l
    norm = float(d @ S @ d)
    return d / math.sqrt(norm)


def _solid_harmonic_polys(l):
    """Real solid harmonics of degree l as {m: {(a,b,c): coef}} (unnormalised),
    from the closed form of Helgaker, Jorgensen and Olsen, Molecular
    Electronic-Structure Theory, eq. 6.4.47-6.4.50."""
    out = {}
    for m in range(-l, l + 1):
        am = abs(m)
        vm = 0.0 if m >= 0 else 0.5
        poly = {}
        for t in range((l - am) // 2 + 1):
            for u in range(t + 1):
                v = vm
                while v <= math.floor(am / 2.0 - vm) + vm + 1e-9:
                    c = ((-1.0) ** (t + v - vm) * 0.25 ** t * math.comb(l, t) * math.comb(l - t, am + t)
                         * math.comb(t, u) * math.comb(am, int(round(2 * v))))
                    a = int(round(2 * t + am - 2 * (u + v)))
                    b = int(round(2 * (u + v)))
                    cz = l - 2 * t - am
                    poly[(a, b, cz)] = poly.get((a, b, cz), 0.0) + c
                    v += 1.0
        out[m] = poly
    return out


def _cart_overlap_ratio(p1, p2, l):
    """<x^a1 y^b1 z^c1 | x^a2 y^b2 z^c2> / <x^l | x^l> for one common exponent."""
    s = 1.0
    for k in range(3):
        e = p1[k] + p2[k]
        if e % 2:
            return 0.0
        s *= _dfact(e - 1)
    return s / _dfact(2 * l - 1)


_SPH_CACHE: dict = {}


def pure_transform(l):
    """(2l+1, ncart) matrix taking the Cartesian functions of a shell (each carrying
    the x^l normalisation) to unit-norm real solid harmonics, rows in the order
    m = 0, +1, -1, +2, -2, ..."""
    if l in _SPH_CACHE:
        return _SPH_CACHE[l]
    comps = cartesian_components(l)
    idx = {c: k for k, c in enumerate(comps)}
    polys = _solid_harmonic_polys(l)
    order = [0] + [s * m for m in range(1, l + 1) for s in (1, -1)]
    T = np.zeros((2 * l + 1, len(comps)))
    M = np.array([[_cart_overlap_ratio(a, b, l) for b in comps] for a in comps])
    for r, m in enumerate(order):
        for pw, c in polys[m].items():
            T[r, idx[pw]] += c
        T[r] /= math.sqrt(T[r] @ M @ T[r])
    _SPH_CACHE[l] = T
    return T


@dataclass
class Shell:
    l: int
    atom: int
    center: np.ndarray
    exps: np.ndarray
    coefs: np.ndarray          # normalised (see module docstring)
    bf0: int = 0               # first function in the (pure or Cartesian) AO basis
    cart0: int = 0             # first Cartesian function

    @property
    def ncart(self):
        return (self.l + 1) * (self.l + 2) // 2

    @property
    def nprimitive(self):
        return len(self.exps)


# Frozen core per element: the orbitals of the previous noble-gas shell.
def _core_orbitals(Z):
    for zmax, n in ((2, 0), (10, 1), (18, 5), (36, 9), (54, 18), (86, 27)):
        if Z <= zmax:
            return n
    return 43


@dataclass
class BasisSet:
    """A basis on a molecule: the subset of psi4.core.BasisSet apyib reads, plus
    the flat shell arrays the integral kernels take."""
    name: str
    molecule: Molecule
    shells: list
    pure: bool
    freeze_core: bool = False
    _n: int = field(default=0)
    _ncart: int = field(default=0)

    def nbf(self):
        return self._n

    def nao(self):
        return self._n

    def ncart(self):
        return self._ncart

    def nshell(self):
        return len(self.shells)

    def shell(self, k):
        return self.shells[k]

    def has_puream(self):
        return self.pure

    def n_frozen_core(self):
        if not self.freeze_core:
            return 0
        return int(sum(_core_orbitals(int(z)) for z in self.molecule.Z))

    @classmethod
    def build(cls, molecule: Molecule, name: str, puream: bool | None = None, freeze_core=False):
        entry = _library_entry(name)
        pure = entry["pure"] if puream is None else bool(puream)
        shells = []
        bf = cart = 0
        for a, sym in enumerate(molecule.symbols):
            if sym not in entry["elements"]:
                raise KeyError(f"basis set {name!r} has no functions for element {sym}")
            for (l, exps, coefs) in entry["elements"][sym]:
                sh = Shell(l, a, molecule.xyz[a].copy(), np.asarray(exps, dtype=np.float64),
                           normalized_coefficients(l, exps, coefs), bf0=bf, cart0=cart)
                shells.append(sh)
                bf += (2 * l + 1) if pure else sh.ncart
                cart += sh.ncart
        b = cls(name, molecule, shells, pure, freeze_core)
        b._n, b._ncart = bf, cart
        return b

    def union(self, other):
        """Both bases as one (self's functions first), on the atoms of both
        molecules; the cross block of a union overlap is <self|other>."""
        mol = Molecule(self.molecule.symbols + other.molecule.symbols,
                       np.concatenate([self.molecule.Z, other.molecule.Z]),
                       np.concatenate([self.molecule.xyz, other.molecule.xyz]))
        if self.pure != other.pure:
            raise ValueError("union of a pure and a Cartesian basis")
        na = self.molecule.natom()
        shells = [Shell(sh.l, sh.atom, sh.center, sh.exps, sh.coefs, sh.bf0, sh.cart0) for sh in self.shells]
        shells += [Shell(sh.l, sh.atom + na, sh.center, sh.exps, sh.coefs, sh.bf0 + self._n, sh.cart0 + self._ncart)
                   for sh in other.shells]
        b = BasisSet(self.name, mol, shells, self.pure, self.freeze_core)
        b._n, b._ncart = self._n + other._n, self._ncart + other._ncart
        return b

    def cart_to_ao(self):
        """(nbf, ncart) matrix from the Cartesian functions to the AO basis
        (identity for a Cartesian basis)."""
        T = np.zeros((self._n, self._ncart))
        for sh in self.shells:
            if self.pure and sh.l >= 1:
                T[sh.bf0:sh.bf0 + 2 * sh.l + 1, sh.cart0:sh.cart0 + sh.ncart] = pure_transform(sh.l)
            else:
                T[sh.bf0:sh.bf0 + sh.ncart, sh.cart0:sh.cart0 + sh.ncart] = np.eye(sh.ncart)
        return T

    def flat(self):
        """Flat arrays for the integral kernels (see ``agb_basis`` in the C header)."""
        nprim = np.array([sh.nprimitive for sh in self.shells], dtype=np.int32)
        prim0 = np.concatenate([[0], np.cumsum(nprim)[:-1]]).astype(np.int32)
        bf_shell = np.concatenate([np.full(sh.ncart, k, dtype=np.int32) for k, sh in enumerate(self.shells)])
        return dict(
            atom_xyz=self.molecule.xyz.astype(np.float64).ravel(),
            atom_charge=self.molecule.Z.astype(np.float64),
            shell_l=np.array([sh.l for sh in self.shells], dtype=np.int32),
            shell_atom=np.array([sh.atom for sh in self.shells], dtype=np.int32),
            shell_nprim=nprim, shell_prim0=prim0,
            shell_cart0=np.array([sh.cart0 for sh in self.shells], dtype=np.int32),
            bf_shell=bf_shell,
            exps=np.concatenate([sh.exps for sh in self.shells]),
            coefs=np.concatenate([sh.coefs for sh in self.shells]))
