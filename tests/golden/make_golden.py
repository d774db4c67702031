"""Generates the golden fixtures in tests/golden/ from the reference itself.

Run here, where the reference source is available (it is not on the GPU
machines, which only read the committed JSON files):

    python tests/golden/make_golden.py [/path/to/reference]

What it runs:
* the reference's pure-Python McMurchie-Davidson engine (src/hf/mmd.py) and
  molecule/basis code (src/hf/molecule.py), importable once ``ase.io.read`` is
  replaced by a small xyz reader (the only ase call, molecule.py:52-55);
* the reference's Rys root fits (core.f90 root5), transcribed into
  oracle/_ref/ by oracle/gen_ref_root5.py.

Fixtures written:
* h2o_sto3g.json  -- water / STO-3G at O (0,0,0), H (+-0.757, 0.587, 0) A:
  the reference's CGF data, all 406 unique ERIs (mmd.eri), S, T, V
  (mmd.overlap/kinetic/potential), E_nuc and E_RHF from the restated
  scf_diis (hf.py:237-353) with tol 1e-10.
* quartets_mmd.json -- AO-level ERIs of random Cartesian component quartets
  over all 21 canonical shell classes (ss|ss ... dd|dd), built from random
  contracted shells of the reference's ContractedGaussianFunction, evaluated by
  the reference's mmd.eri.
* root5_ref.json  -- root5(x) (5 roots t^2 + 5 weights) on a grid of x that
  visits every branch of core.f90:249-807.
* ccpvdz_recorded.json -- six of the reference's molecules (water, ammonia,
  methane, hydrogen peroxide, methanol, ethane: xyz text), the cc-pVDZ blocks
  of H/C/N/O, and the energies the reference recorded for them with its
  Fortran engine (src/hf/benchmark/molecule_test.json).
"""
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def install_ase_stub():
    class _Atoms:
        def __init__(self, sym, pos):
            self._s = sym
            self.positions = np.array(pos, dtype=float)

        def get_chemical_symbols(self):
            return self._s

        def get_atomic_numbers(self):
            tab = {"H": 1, "C": 6, "N": 7, "O": 8}
            return np.array([tab[x] for x in self._s])

        def __len__(self):
            return len(self._s)

    def read(fn, index=0):
        L = open(fn).read().split("\n")
        n = int(L[0])
        sym, pos = [], []
        for l in L[2:2 + n]:
            t = l.split()
            sym.append(t[0])
            pos.append(list(map(float, t[1:4])))
        return _Atoms(sym, pos)

    ase = types.ModuleType("ase")
    ase.Atoms = _Atoms
    io = types.ModuleType("ase.io")
    io.read = read
    ase.io = io
    sys.modules["ase"] = ase
    sys.modules["ase.io"] = io


def cgf_dict(c):
    return dict(coefs=[float(v) for v in c.coefs], expns=[float(v) for v in c.expns], shell=list(map(int, c.shell)),
                nf=[float(v) for v in c.normalize_factors], center=[float(v) for v in c.center])


def h2o_sto3g(ref, tmpdir):
    import molecule
    import mmd
    sys.path.insert(0, os.path.join(REPO))
    from oracle import oracle as O

    xyz = os.path.join(tmpdir, "h2o.xyz")
    open(xyz, "w").write("3\n\nO 0 0 0\nH 0.757 0.587 0\nH -0.757 0.587 0\n")
    mol = molecule.Molecule(xyz, os.path.join(ref, "src/hf/data/basis/sto-3g.dat"))
    cg = [c for a in mol.atoms for c in a.cgfs]
    n = len(cg)
    S = np.array([[mmd.overlap(a, b) for b in cg] for a in cg])
    T = np.array([[mmd.kinetic(a, b) for b in cg] for a in cg])
    V = np.zeros((n, n))
    for at in mol.atoms:
        V += np.array([[mmd.potential(a, b, at.xyz) for b in cg] for a in cg]) * (-at.number)
    quartets, vals = [], []
    E = np.zeros((n,) * 4)
    for i in range(n):
        for j in range(i + 1):
            for k in range(n):
                for l in range(k + 1):
                    if i * (i + 1) // 2 + j >= k * (k + 1) // 2 + l:
                        v = mmd.eri(cg[i], cg[j], cg[k], cg[l])
                        quartets.append([i, j, k, l])
                        vals.append(float(v))
                        for a, b, c, d in [(i, j, k, l), (j, i, k, l), (i, j, l, k), (j, i, l, k),
                                           (k, l, i, j), (l, k, i, j), (k, l, j, i), (l, k, j, i)]:
                            E[a, b, c, d] = v
    etot, P, F, nit = O.scf_diis(S, T, V, int(np.sum(mol.numbers)), float(mol.e_nuc),
                                 lambda P: O.jk_dense(E, P), tol=1e-10)
    return dict(geometry_angstrom=[["O", 0, 0, 0], ["H", 0.757, 0.587, 0], ["H", -0.757, 0.587, 0]],
                basis="sto-3g", e_nuc=float(mol.e_nuc), cgfs=[cgf_dict(c) for c in cg],
                quartets=quartets, eri=vals, S=S.tolist(), T=T.tolist(), V=V.tolist(),
                e_rhf=float(etot), scf_iterations=int(nit), density=P.tolist(),
                note="ERIs, S, T, V from the reference's src/hf/mmd.py; E_RHF from the restated scf_diis, tol 1e-10")


def random_quartets(seed=2024, per_class=3, comps_per_quartet=6):
    import molecule
    import mmd
    rng = np.random.default_rng(seed)
    ltype = {0: "S", 1: "P", 2: "D"}
    comps = {0: [[0, 0, 0]], 1: [[1, 0, 0], [0, 1, 0], [0, 0, 1]],
             2: [[2, 0, 0], [1, 1, 0], [1, 0, 1], [0, 2, 0], [0, 1, 1], [0, 0, 2]]}
    pair_classes = [(0, 0), (1, 0), (1, 1), (2, 0), (2, 1), (2, 2)]
    classes = [(pair_classes[i], pair_classes[j]) for i in range(6) for j in range(i + 1)]
    shells, out = [], []

    def new_shell(l):
        K = int(rng.integers(1, 4))
        ex = list(np.exp(rng.uniform(np.log(0.1), np.log(50.0), K)))
        co = list(rng.uniform(0.2, 1.0, K))
        cen = rng.uniform(-2.0, 2.0, 3)
        group = [molecule.ContractedGaussianFunction(npgf=K, expns=ex, coefs=co, orbital_type=ltype[l],
                                                     shell=c, center=cen) for c in comps[l]]
        shells.append(dict(l=l, expns=[float(v) for v in ex], coefs_raw=None, center=[float(v) for v in cen],
                           cgfs=[cgf_dict(g) for g in group]))
        return len(shells) - 1, group

    for (la, lb), (lc, ld) in classes:
        for _ in range(per_class):
            ids, groups = zip(*[new_shell(l) for l in (la, lb, lc, ld)])
            for _ in range(comps_per_quartet):
                pick = [int(rng.integers(len(g))) for g in groups]
                v = mmd.eri(*[g[p] for g, p in zip(groups, pick)])
                out.append(dict(shells=list(ids), comps=pick, value=float(v)))
    return dict(shells=shells, quartets=out, seed=seed,
                note="values from the reference's src/hf/mmd.py eri on random contracted shells")


def root5_grid():
    sys.path.insert(0, REPO)
    from oracle import oracle as O
    xs = [0.0, 1e-8, 2.9e-7, 3.1e-7, 0.3, 0.99, 1.0, 2.0, 4.99, 5.0, 7.0, 9.99, 10.0, 12.0, 14.9, 15.0, 18.0,
          20.0, 22.0, 24.9, 25.0, 30.0, 39.9, 40.0, 50.0, 58.9, 59.0, 80.0, 300.0, 1e4, 1e6]
    return dict(x=xs, res=[O.ref_root5(x).tolist() for x in xs],
                note="core.f90 root5 transcribed by oracle/gen_ref_root5.py; res = 5 roots (t^2) + 5 weights")


def ccpvdz_recorded(ref):
    blocks = {}
    for b in open(os.path.join(ref, "src/hf/data/basis/cc-pvdz.dat")).read().split("****"):
        b = b.strip()
        if b and b.split()[0] in ("H", "C", "N", "O"):
            blocks[b.split()[0]] = b
    rec = json.load(open(os.path.join(ref, "src/hf/benchmark/molecule_test.json")))
    flat = {k: v for grp in rec.values() for k, v in grp.items()}
    mols = {}
    for name in ("water", "ammonia", "methane", "hydrogen_peroxide", "methanol", "ethane"):
        mols[name] = dict(xyz=open(os.path.join(ref, "src/hf/data/molecules/%s.xyz" % name)).read(),
                          recorded=flat[name])
    return dict(basis_blocks=blocks, molecules=mols,
                note="recorded = src/hf/benchmark/molecule_test.json (reference energy etot, psi4 energy, wall s)")


def main(ref=None):
    # the reference checkout this script reads: argument, $SEGFAULT_PY_REFERENCE, else its usual place here
    ref = ref or os.environ.get("SEGFAULT_PY_REFERENCE", "/root/reference")
    import tempfile
    sys.path.insert(0, os.path.join(ref, "src/hf"))
    sys.path.insert(0, REPO)
    install_ase_stub()
    subprocess_gen = os.path.join(REPO, "oracle", "gen_ref_root5.py")
    os.system("%s %s %s" % (sys.executable, subprocess_gen, os.path.join(ref, "src/hf/core/core.f90")))
    with tempfile.TemporaryDirectory() as td:
        json.dump(h2o_sto3g(ref, td), open(os.path.join(HERE, "h2o_sto3g.json"), "w"))
    json.dump(root5_grid(), open(os.path.join(HERE, "root5_ref.json"), "w"))
    json.dump(ccpvdz_recorded(ref), open(os.path.join(HERE, "ccpvdz_recorded.json"), "w"), indent=1)
    json.dump(random_quartets(), open(os.path.join(HERE, "quartets_mmd.json"), "w"))


if __name__ == "__main__":
    main(*(sys.argv[1:2]))
