"""SCF iteration captured as a CUDA graph (purification density, device DIIS)
against the eager scf_diis: same energies."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_graph_scf_h2o_sto3g(cuda):
    from segfault_py_gb300.molecule import Molecule
    from segfault_py_gb300.scf_graph import GraphSCF
    mol = Molecule.from_geometry(["O", "H", "H"], [[0, 0, 0], [0.757, 0.587, 0], [-0.757, 0.587, 0]], "sto-3g")
    g = GraphSCF(mol, precision="fp64").capture()
    assert g.graph is not None
    r = g.run(tol=1e-10)
    assert r.converged
    assert abs(r.energy - (-74.96306315472287)) < 1e-9


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", 1e-6), ("mixed_df", 1e-6)])
def test_graph_scf_matches_eager(cuda, precision, tol):
    from segfault_py_gb300 import geometry as G
    from segfault_py_gb300.molecule import Molecule
    from segfault_py_gb300.scf import scf_diis
    from segfault_py_gb300.scf_graph import scf_graph
    s, x = G.water_cluster(4, seed=3)
    mol = Molecule.from_geometry(s, x, "6-31g*")
    ref = scf_diis(mol, tol=1e-10, precision="fp64")
    r = scf_graph(mol, tol=1e-10, precision=precision, fp32_cutoff=1e-2)
    assert r.converged
    assert abs(r.energy - ref.energy) < tol
    assert float((r.D - ref.D).abs().max()) < 1e-4
