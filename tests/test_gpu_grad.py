"""Analytic RHF gradients (through the C ABI) against central finite
differences, step 1e-4 bohr: of the oracle's restatement of the reference SCF
(H2O / STO-3G) and of FP64 GPU energies ((H2O)2 / 6-31G*, d shells).
Tolerance 1e-6 Eh/bohr."""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu

H2O = (["O", "H", "H"], np.array([[0, 0, 0], [0.757, 0.587, 0], [-0.757, 0.587, 0]]))
STEP = 1e-4   # bohr


def _oracle_energy(symbols, xyz_bohr, basis):
    from segfault_py_gb300.molecule import BOHR, Molecule
    mol = Molecule.from_geometry(symbols, xyz_bohr * BOHR, basis)
    xyz, Z = mol.atom_table()
    S, T, V = O.one_electron(mol.cgfs, xyz, Z)
    E = O.build_eri_dense(mol.cgfs)
    e, *_ = O.scf_diis(S, T, V, mol.nelectron, mol.e_nuc, lambda P: O.jk_dense(E, P), tol=1e-13, maxiter=200)
    return e


def _gpu_energy(symbols, xyz_bohr, basis, **kw):
    from segfault_py_gb300.molecule import BOHR, Molecule
    from segfault_py_gb300.scf import scf_diis
    mol = Molecule.from_geometry(symbols, xyz_bohr * BOHR, basis)
    return scf_diis(mol, tol=1e-12, dtol=1e-9, maxiter=200, **kw).energy


def _analytic(symbols, xyz_bohr, basis, **opts):
    from segfault_py_gb300.grad import RHFEnergy
    x = torch.tensor(xyz_bohr, dtype=torch.float64, requires_grad=True)
    E = RHFEnergy.apply(x, tuple(symbols), basis, opts)
    E.backward()
    return float(E.detach()), x.grad.numpy().copy()


def test_h2o_sto3g_gradient_vs_reference_fd(cuda):
    from segfault_py_gb300.molecule import BOHR
    sym, xyz = H2O
    x0 = xyz / BOHR
    E, g = _analytic(sym, x0, "sto-3g")
    assert abs(E - (-74.96306315472287)) < 1e-9
    assert np.abs(g.sum(axis=0)).max() < 1e-9          # translational invariance
    for a in range(3):
        for d in range(3):
            xp, xm = x0.copy(), x0.copy()
            xp[a, d] += STEP
            xm[a, d] -= STEP
            fd = (_oracle_energy(sym, xp, "sto-3g") - _oracle_energy(sym, xm, "sto-3g")) / (2 * STEP)
            assert abs(fd - g[a, d]) < 1e-6, (a, d, fd, g[a, d])


def test_water_dimer_631gs_gradient_vs_fd(cuda):
    from segfault_py_gb300 import geometry as G
    from segfault_py_gb300.molecule import BOHR
    sym, xyz = G.water_cluster(2, seed=5)
    x0 = xyz / BOHR
    E, g = _analytic(sym, x0, "6-31g*")
    assert np.abs(g.sum(axis=0)).max() < 1e-8
    rng = np.random.default_rng(1)
    for a, d in [(0, 0), (1, 1), (2, 2), (3, 0), (4, 1), (5, 2)]:
        xp, xm = x0.copy(), x0.copy()
        xp[a, d] += STEP
        xm[a, d] -= STEP
        fd = (_gpu_energy(sym, xp, "6-31g*") - _gpu_energy(sym, xm, "6-31g*")) / (2 * STEP)
        assert abs(fd - g[a, d]) < 1e-6, (a, d, fd, g[a, d])


@pytest.mark.parametrize("precision", ["mixed", "mixed_df"])
def test_mixed_precision_gradient_error(cuda, precision):
    from segfault_py_gb300 import geometry as G
    from segfault_py_gb300.molecule import BOHR
    sym, xyz = G.water_cluster(4, seed=2)
    x0 = xyz / BOHR
    e64, g64 = _analytic(sym, x0, "6-31g*")
    emx, gmx = _analytic(sym, x0, "6-31g*", precision=precision, fp32_cutoff=1e-2)
    assert abs(emx - e64) < 1e-6
    assert np.abs(gmx - g64).max() < 1e-6


def test_double_float_gradient_matches_fp64(cuda):
    """All-double-float derivative kernels against FP64 at the same converged
    density: FP64-class agreement (1e-9 Eh/bohr)."""
    from segfault_py_gb300 import geometry as G
    from segfault_py_gb300.fock import FockBuilder
    from segfault_py_gb300.grad import rhf_gradient
    from segfault_py_gb300.molecule import Molecule
    from segfault_py_gb300.scf import scf_diis
    sym, xyz = G.water_cluster(2, seed=3)
    mol = Molecule.from_geometry(sym, xyz, "6-31g*")
    fb = FockBuilder(mol, device=cuda)
    r = scf_diis(mol, tol=1e-10, fb=fb, precision="fp64")
    g64 = rhf_gradient(mol, r, fb, precision="fp64")
    gdf = rhf_gradient(mol, r, fb, precision="df")
    assert float((gdf - g64).abs().max()) < 1e-9
