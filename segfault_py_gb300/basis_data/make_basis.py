"""Writes the basis files this package ships (Gaussian94 format, as read by
molecule.read_basis_block).

* sto-3g.dat, 6-31g.dat: the H/C/O blocks of the reference's own basis files
  (src/hf/data/basis/sto-3g.dat, 6-31g.dat), unchanged, so that integrals are
  over exactly the reference's functions.
* 6-31gs.dat (6-31G*): 6-31G plus one Cartesian d shell (exponent 0.8,
  coefficient 1) on the heavy atoms C and O -- the polarisation exponent of
  Hariharan & Pople, Theor. Chim. Acta 28, 213 (1973).
* 6-31gss.dat (6-31G**): 6-31G* plus one p shell (exponent 1.1, coefficient 1)
  on H.

The reference ships neither 6-31G* nor 6-31G**; its 6-31g.dat covers H, C and O
only.  Usage: python make_basis.py [reference basis dir]
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout this script reads: $SEGFAULT_PY_REFERENCE, else its usual place here
SRC = os.path.join(os.environ.get("SEGFAULT_PY_REFERENCE", "/root/reference"), "src/hf/data/basis")
D_EXP = {"C": 0.8, "N": 0.8, "O": 0.8}
P_EXP_H = 1.1


def blocks(path):
    with open(path) as f:
        out = {}
        for b in f.read().split("****"):
            b = b.strip()
            if b:
                out[b.split()[0]] = b
        return out


def write(path, bl):
    with open(path, "w") as f:
        f.write("****\n")
        for b in bl:
            f.write(b.rstrip() + "\n****\n")


def main(src=SRC):
    sto = blocks(os.path.join(src, "sto-3g.dat"))
    g631 = blocks(os.path.join(src, "6-31g.dat"))
    order = ["H", "C", "O"]
    write(os.path.join(HERE, "sto-3g.dat"), [sto[e] for e in order])
    write(os.path.join(HERE, "6-31g.dat"), [g631[e] for e in order])
    star = []
    for e in order:
        b = g631[e]
        if e in D_EXP:
            b += "\nD    1   1.00\n      %.10E       %.10E" % (D_EXP[e], 1.0)
        star.append(b)
    write(os.path.join(HERE, "6-31gs.dat"), star)
    sstar = []
    for e, b in zip(order, star):
        if e == "H":
            b += "\nP    1   1.00\n      %.10E       %.10E" % (P_EXP_H, 1.0)
        sstar.append(b)
    write(os.path.join(HERE, "6-31gss.dat"), sstar)


if __name__ == "__main__":
    main(*(sys.argv[1:2]))
