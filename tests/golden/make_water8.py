"""Generates tests/golden/water8_631gs.npz: the oracle's J, K and energies for
the seeded (H2O)8 cluster in 6-31G* (152 AOs), the configuration the Fock-build
numbers are quoted on.

Run here, where the reference source is available (the GPU machines only read
the committed .npz):

    python tests/golden/make_water8.py [/path/to/reference]

What it runs:
* the reference's own Molecule / ContractedGaussianFunction code
  (src/hf/molecule.py, imported with a stub ``ase.io.read``) on the cluster
  geometry, with the repository's 6-31G* file (the reference's 6-31G blocks
  plus the Pople d(0.8) shells, in the reference's format): the CGFs below are
  the reference's own objects;
* the oracle (oracle/rys_oracle.c, a C restatement of core.f90 module rys:
  one call per unique AO quartet, 5 Rys roots, no screening), with the
  reference's own root5 fits (transcribed by oracle/gen_ref_root5.py), for the
  dense ERI tensor of hf.py:33-61; S, T, V from the oracle's restatement of
  mmd.py's one-electron integrals;
* the restated scf_diis of hf.py:237-353 (tol 1e-10) for the converged
  density D and the total energy;
* J, K at that D by the einsums of hf.py:300, and E(D) = 1/2 sum D (2H + J - K/2).

Stored (float64; symmetric matrices as their lower triangles, row-major):
xyz_angstrom, D, J, K, H, e_total (SCF), e_elec_at_D, e_nuc, scf_iterations,
roots ("reference root5" or "oracle table").
"""
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "water8_631gs.npz")


def tril(M):
    return M[np.tril_indices(M.shape[0])]


def main(ref=None):
    ref = ref or os.environ.get("SEGFAULT_PY_REFERENCE", "/root/reference")
    sys.path.insert(0, os.path.join(ref, "src/hf"))
    sys.path.insert(0, REPO)
    sys.path.insert(0, HERE)
    from make_golden import install_ase_stub
    install_ase_stub()
    import molecule as refmol   # the reference's src/hf/molecule.py
    from oracle import oracle as O
    from segfault_py_gb300 import geometry as G
    from segfault_py_gb300.molecule import resolve_basis

    gen = os.path.join(REPO, "oracle", "gen_ref_root5.py")
    os.system("%s %s %s" % (sys.executable, gen, os.path.join(ref, "src/hf/core/core.f90")))
    roots = "reference root5" if O.use_reference_root5(True) else "oracle table"

    sym, xyz = G.water_cluster(8, seed=0)
    with tempfile.TemporaryDirectory() as td:
        fn = os.path.join(td, "w8.xyz")
        with open(fn, "w") as f:
            f.write("%d\n\n" % len(sym))
            for s, p in zip(sym, xyz):
                f.write("%s %.17g %.17g %.17g\n" % (s, p[0], p[1], p[2]))
        mol = refmol.Molecule(fn, resolve_basis("6-31g*"))
    cg = [c for a in mol.atoms for c in a.cgfs]
    n = len(cg)
    print("nao", n, "roots", roots, flush=True)
    atom_xyz = np.array([a.xyz for a in mol.atoms], dtype=np.float64)
    Z = np.array([a.number for a in mol.atoms], dtype=np.float64)
    t = time.time()
    S, T, V = O.one_electron(cg, atom_xyz, Z)
    t1 = time.time()
    E = O.build_eri_dense(cg)
    t2 = time.time()
    print("one-electron %.1f s, ERI %.1f s" % (t1 - t, t2 - t1), flush=True)
    nelec = int(np.sum(Z))
    etot, P, F, nit = O.scf_diis(S, T, V, nelec, float(mol.e_nuc), lambda P: O.jk_dense(E, P), tol=1e-10)
    print("E_total %.12f after %d iterations (%.1f s)" % (etot, nit, time.time() - t2), flush=True)
    P = 0.5 * (P + P.T)
    J, K = O.jk_dense(E, P)
    H = T + V
    e_elec = 0.5 * float(np.sum(P * (2.0 * H + J - 0.5 * K)))
    np.savez_compressed(OUT, xyz_angstrom=np.asarray(xyz, dtype=np.float64), D=tril(P), J=tril(J), K=tril(K),
                        H=tril(H), e_total=etot, e_elec_at_D=e_elec, e_nuc=float(mol.e_nuc),
                        scf_iterations=nit, nao=n, roots=roots)
    print("wrote", OUT, "E(D) %.12f" % (e_elec + mol.e_nuc))


if __name__ == "__main__":
    main(*(sys.argv[1:2]))
