"""Molecule / basis ingestion (the input side of the Fock build).

Mirrors the reference's ``src/hf/molecule.py``:

* ``Molecule(xyz_filename, bas_filename)`` (molecule.py:51-63): reads an xyz
  file, shifts the geometry to its centre (molecule.py:68-70), converts
  Angstrom -> bohr with 0.52917720859 (molecule.py:72-73), computes the
  nuclear repulsion with the same double loop (molecule.py:75-80).
* ``Atom`` (molecule.py:108-165): finds the ``****``-separated basis block
  that starts with ``<symbol> 0`` and expands every S/P/D/F line into Cartesian
  components in the reference order s; x,y,z; xx,xy,xz,yy,yz,zz; xxx,...,zzz.
* ``ContractedGaussianFunction`` (molecule.py:201-226): primitive
  normalisation factors and the contracted renormalisation.  As in the
  reference, the Cartesian components of one shell share one coefficient list
  that every component renormalises in place; the first component fixes the
  norm and later components rescale by 1 to rounding.

On top of the reference's AO-level objects this module builds the shell-level
table the GPU library consumes (``Molecule.shell_table``): one row per shell
with ``l``, the primitive exponents, the contraction coefficients of the
x^l component (coefs x primitive normalisation of (l,0,0)), the centre and the
first AO index.  The other Cartesian components differ from the x^l one by the
factor sqrt((2l-1)!! / ((2lx-1)!! (2ly-1)!! (2lz-1)!!)), which the library
applies per component, so that every Cartesian AO is normalised individually
exactly as in the reference.

The ase dependency of the reference (``ase.io.read``) is replaced by a plain
xyz reader; ``Molecule.from_geometry`` builds a molecule from arrays.

One deliberate difference: the reference tests ``line[0] in 'SPDF'`` on every
line of a block, which also matches the element header line of sulfur
(``S 0``) and phosphorus (``P 0``) and would create an empty shell; here the
header line is skipped.
"""
from __future__ import annotations

import os
import re
from dataclasses import dataclass, field

import numpy as np

BOHR = 0.52917720859  # molecule.py:73

ELEMENTS = ["X", "H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne",
            "Na", "Mg", "Al", "Si", "P", "S", "Cl", "Ar", "K", "Ca",
            "Sc", "Ti", "V", "Cr", "Mn", "Fe", "Co", "Ni", "Cu", "Zn",
            "Ga", "Ge", "As", "Se", "Br", "Kr"]

# Cartesian component order per l (molecule.py:138-165)
CART = {
    0: [(0, 0, 0)],
    1: [(1, 0, 0), (0, 1, 0), (0, 0, 1)],
    2: [(2, 0, 0), (1, 1, 0), (1, 0, 1), (0, 2, 0), (0, 1, 1), (0, 0, 2)],
    3: [(3, 0, 0), (2, 1, 0), (2, 0, 1), (1, 2, 0), (1, 1, 1), (1, 0, 2),
        (0, 3, 0), (0, 2, 1), (0, 1, 2), (0, 0, 3)],
}
LVAL = {"S": 0, "P": 1, "D": 2, "F": 3}

BASIS_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "basis_data")


class BasisSetNotAvailableError(Exception):
    """molecule.py:14-20: raised when the basis file has no block for an element."""

    def __init__(self, msg: str = "no basis set found for this element", *args):
        super().__init__(*args)
        self.msg = msg

    def __str__(self):
        return self.msg


def factorial2(n: int) -> float:
    """(n)!! with (-1)!! = (0)!! = 1, like utils.safe_factorial2 (utils.py:87-89)."""
    r = 1.0
    while n > 1:
        r *= n
        n -= 2
    return r


def resolve_basis(bas: str) -> str:
    """Accept a path or a basis name shipped in basis_data/ ('6-31g*' etc.)."""
    if os.path.exists(bas):
        return bas
    name = bas.lower().replace("*", "s")
    if not name.endswith(".dat"):
        name += ".dat"
    p = os.path.join(BASIS_DIR, name)
    if os.path.exists(p):
        return p
    raise FileNotFoundError(bas)


def read_basis_block(bas_filename: str, symbol: str):
    """Return [(orbital_type, expns, coefs), ...] for ``symbol`` (molecule.py:115-137)."""
    with open(bas_filename) as f:
        blocks = f.read().split("****")
    target = ""
    for bb in blocks:
        block = bb.strip()
        if re.match(rf"^{symbol}\s+0", block) is not None:
            target = block
            break
    if not target:
        raise BasisSetNotAvailableError()
    lines = target.split("\n")
    out = []
    for idx, line in enumerate(lines):
        if idx == 0:
            continue  # element header line ("O     0")
        if line and line[0] in LVAL:
            n = int(line.split()[1])
            expns, coefs = [], []
            for token in lines[idx + 1: idx + 1 + n]:
                e, c = list(map(float, token.strip().split()))
                expns.append(e)
                coefs.append(c)
            out.append((line[0], expns, coefs))
    return out


class ContractedGaussianFunction:
    """One Cartesian component of a contracted shell (molecule.py:173-226)."""

    def __init__(self, npgf, expns, coefs, orbital_type, shell, center):
        self.npgf = npgf
        self.expns = expns
        self.coefs = coefs          # shared between the components of a shell
        self.orbital_type = orbital_type
        self.shell = shell
        self.center = center
        l = shell[0] + shell[1] + shell[2]
        ex = np.asarray(expns, dtype=np.float64)
        dfac = factorial2(2 * shell[0] - 1) * factorial2(2 * shell[1] - 1) * factorial2(2 * shell[2] - 1)
        self.normalize_factors = np.sqrt(np.power(2, 2 * l + 1.5) * np.power(ex, l + 1.5) / dfac / np.power(np.pi, 1.5))
        prefactor = np.power(np.pi, 1.5) * dfac / np.power(2.0, l)
        N = 0.0
        nf = self.normalize_factors
        for ia in range(len(expns)):
            for ib in range(len(expns)):
                N += nf[ia] * nf[ib] * coefs[ia] * coefs[ib] / np.power(expns[ia] + expns[ib], l + 1.5)
        N *= prefactor
        N = np.power(N, -0.5)
        for ia in range(len(expns)):
            coefs[ia] *= N


@dataclass
class Shell:
    """A contracted Cartesian shell: all components of one basis-file line."""
    l: int
    expns: np.ndarray
    coefs: np.ndarray          # coefficients of the x^l component, normalisation included
    center: np.ndarray         # bohr
    atom: int
    ao_offset: int
    cgfs: list = field(default_factory=list, repr=False)


class Atom:
    """One atom and its contracted functions (molecule.py:84-168)."""

    def __init__(self, bas: str, symbol: str, number: int, xyz):
        self.bas = bas
        self.symbol = symbol
        self.number = number
        self.xyz = xyz
        self.cgfs: list[ContractedGaussianFunction] = []
        self.shell_groups = []   # (l, expns, shared coefs list, [cgf, ...])
        for orbital_type, expns, coefs in read_basis_block(bas, symbol):
            l = LVAL[orbital_type]
            group = []
            for comp in CART[l]:
                cgf = ContractedGaussianFunction(npgf=len(expns), expns=expns, coefs=coefs,
                                                 orbital_type=orbital_type, shell=list(comp), center=self.xyz)
                self.cgfs.append(cgf)
                group.append(cgf)
            self.shell_groups.append((l, expns, coefs, group))

    def __len__(self):
        return len(self.cgfs)


def read_xyz(filename: str):
    """Plain xyz reader (stand-in for ase.io.read(filename, index=0))."""
    with open(filename) as f:
        lines = f.read().split("\n")
    n = int(lines[0].split()[0])
    symbols, pos = [], []
    for l in lines[2:2 + n]:
        t = l.split()
        symbols.append(t[0])
        pos.append([float(v) for v in t[1:4]])
    return symbols, np.array(pos, dtype=np.float64)


class Molecule:
    """Geometry + basis (molecule.py:23-80)."""

    def __init__(self, xyz_filename: str | None, bas_filename: str, *, symbols=None, positions=None):
        if xyz_filename is not None:
            symbols, positions = read_xyz(xyz_filename)
        bas_filename = resolve_basis(bas_filename)
        self.basis_file = bas_filename
        self.symbols = list(symbols)
        self.numbers = np.array([ELEMENTS.index(s) for s in self.symbols])
        self.xyz = np.asarray(positions, dtype=np.float64)        # Angstrom
        self.xyz_ = self.xyz - self.xyz.mean(axis=0)              # centred
        self.xyz__ = self.xyz_ / BOHR                             # bohr
        self.natom = len(self.symbols)
        self.atoms: list[Atom] = []
        self.e_nuc = self.nuclear_repulsion()
        for symbol, number, xyz in zip(self.symbols, self.numbers, self.xyz__):
            self.atoms.append(Atom(bas=bas_filename, symbol=symbol, number=number, xyz=xyz))
        self._build_shells()

    @classmethod
    def from_geometry(cls, symbols, positions_angstrom, basis: str) -> "Molecule":
        return cls(None, basis, symbols=symbols, positions=positions_angstrom)

    def __len__(self):
        return self.natom

    def nuclear_repulsion(self) -> float:
        e = 0.0
        for i in range(self.natom - 1):
            for j in range(i + 1, self.natom):
                e += self.numbers[i] * self.numbers[j] / np.linalg.norm(self.xyz__[i] - self.xyz__[j])
        return float(e)

    @property
    def cgfs(self):
        return [c for a in self.atoms for c in a.cgfs]

    @property
    def nao(self) -> int:
        return sum(len(a) for a in self.atoms)

    @property
    def nelectron(self) -> int:
        return int(np.sum(self.numbers))

    def _build_shells(self):
        self.shells: list[Shell] = []
        off = 0
        for ia, atom in enumerate(self.atoms):
            for l, expns, coefs, group in atom.shell_groups:
                ex = np.asarray(expns, dtype=np.float64)
                # x^l component: coefs (shared, final) x primitive norm of (l,0,0)
                c = np.asarray(coefs, dtype=np.float64) * group[0].normalize_factors
                self.shells.append(Shell(l=l, expns=ex, coefs=c, center=np.asarray(atom.xyz, dtype=np.float64),
                                         atom=ia, ao_offset=off, cgfs=group))
                off += len(group)

    def shell_table(self):
        """Flat arrays for the C-ABI: l, nprim, atom, ao_offset, center[3], prim_offset, exps, coefs."""
        ls = np.array([s.l for s in self.shells], dtype=np.int32)
        nprim = np.array([len(s.expns) for s in self.shells], dtype=np.int32)
        atom = np.array([s.atom for s in self.shells], dtype=np.int32)
        aoff = np.array([s.ao_offset for s in self.shells], dtype=np.int32)
        cen = np.array([s.center for s in self.shells], dtype=np.float64).reshape(-1, 3)
        poff = np.zeros(len(self.shells) + 1, dtype=np.int32)
        poff[1:] = np.cumsum(nprim)
        exps = np.concatenate([s.expns for s in self.shells]).astype(np.float64)
        coefs = np.concatenate([s.coefs for s in self.shells]).astype(np.float64)
        return dict(l=ls, nprim=nprim, atom=atom, ao_offset=aoff, center=np.ascontiguousarray(cen),
                    prim_offset=poff, exps=exps, coefs=coefs)

    def atom_table(self):
        """(natom,3) bohr coordinates and (natom,) nuclear charges."""
        return np.ascontiguousarray(self.xyz__, dtype=np.float64), self.numbers.astype(np.float64)
