"""The linear-alkane configuration: C20H42 all-trans (C-C 1.54 A, C-H 1.09 A,
tetrahedral angles, +-0.05 A seeded noise), 6-31G** (510 Cartesian AOs): the
mixed-precision SCF captured as a CUDA graph, plus forces, against the
all-FP64 GPU path (energy 1e-6 Eh, forces 1e-6 Eh/bohr)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_alkane_graph_mixed_vs_fp64(cuda):
    from segfault_py_gb300 import geometry as G
    from segfault_py_gb300.fock import FockBuilder
    from segfault_py_gb300.grad import rhf_gradient
    from segfault_py_gb300.molecule import Molecule
    from segfault_py_gb300.scf import scf_diis
    from segfault_py_gb300.scf_graph import GraphSCF
    s, x = G.alkane(20, seed=0)
    mol = Molecule.from_geometry(s, x, "6-31g**")
    assert mol.nao == 510
    fb = FockBuilder(mol, device=cuda, cutoff=1e-12, fp32_cutoff=1e-2)
    ref = scf_diis(mol, tol=1e-9, dtol=1e-7, fb=fb, precision="fp64")
    g64 = rhf_gradient(mol, ref, fb, precision="fp64")
    for prec in ("mixed", "mixed_df"):
        g = GraphSCF(mol, fb=fb, precision=prec, fp32_cutoff=1e-2).capture()
        r = g.run(tol=1e-9)
        assert r.converged
        assert abs(r.energy - ref.energy) < 1e-6
        gmx = rhf_gradient(mol, ref, fb, precision=prec)
        assert float((gmx - g64).abs().max()) < 1e-6
    assert float(g64.sum(dim=0).abs().max()) < 1e-8
