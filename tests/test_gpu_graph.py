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


@pytest.mark.parametrize("precision,node_priority", [("fp64", True), ("mixed_df", True), ("mixed_df", False)])
def test_native_fock_graph_matches_eager(cuda, precision, node_priority):
    """One Fock build captured and instantiated by the library
    (sf_fock_jk_graph_create): a replay after D changed gives the eager build
    of the new D; the persistent launch mode captures the same way."""
    import torch
    from segfault_py_gb300 import geometry as G
    from segfault_py_gb300.fock import FockBuilder
    from segfault_py_gb300.molecule import Molecule
    s, x = G.water_cluster(3, seed=4)
    mol = Molecule.from_geometry(s, x, "6-31g*")
    fb = FockBuilder(mol, device=cuda, cutoff=1e-12, fp32_cutoff=1e-2)
    rng = np.random.default_rng(5)
    A = rng.standard_normal((mol.nao, mol.nao)) * 0.1
    D = torch.tensor(A + A.T, device=cuda)
    J = torch.empty_like(D)
    K = torch.empty_like(D)
    for mode in ("streams", "persistent"):
        fb.set_launch_mode(mode)
        g = fb.capture_jk(D, J, K, precision=precision, native=True, node_priority=node_priority)
        B = rng.standard_normal((mol.nao, mol.nao)) * 0.05
        D.add_(torch.tensor(B + B.T, device=cuda))
        g.replay()
        g.replay()
        torch.cuda.synchronize()
        Je, Ke = fb.jk(D, precision=precision)
        scale = max(float(Je.abs().max()), float(Ke.abs().max()))
        assert float((J - Je).abs().max()) <= 1e-12 * scale, mode
        assert float((K - Ke).abs().max()) <= 1e-12 * scale, mode
        g.close()
    fb.set_launch_mode("streams")
    fb.close()
