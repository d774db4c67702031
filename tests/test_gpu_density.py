"""Density-weighted classification of the quartet lists (sf_set_density_screening):
the Fock build's mixed modes (when switched on) move accurate-tier quartets whose
bound Q_ab Q_cd max|D| is below the FP32 cutoff to FP32, the gradient leaves out
quartets whose Q_ab Q_cd |Gamma| bound is below the Schwarz cutoff.  Checked
against the same builds with the classification off."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cluster():
    from segfault_py_gb300 import geometry as G
    from segfault_py_gb300.fock import FockBuilder
    from segfault_py_gb300.molecule import Molecule
    from segfault_py_gb300.scf import scf_diis
    sym, xyz = G.water_cluster(4, seed=11)
    mol = Molecule.from_geometry(sym, xyz, "6-31g*")
    fb = FockBuilder(mol, device=torch.device("cuda:0"), cutoff=1e-12, fp32_cutoff=1e-2)
    r = scf_diis(mol, tol=1e-10, dtol=1e-8, fb=fb, precision="fp64")
    yield mol, fb, r
    fb.close()


def _energy(fb, r, precision):
    D = r.D.contiguous()
    J, K = fb.jk(D, precision=precision, stats=True)
    return 0.5 * float(torch.sum(D * (2.0 * r.H + J - 0.5 * K))), dict(fb.last_stats)


@pytest.mark.parametrize("precision", ["mixed", "mixed_df"])
def test_fock_demotion_keeps_energy(cuda, cluster, precision):
    mol, fb, r = cluster
    e64, _ = _energy(fb, r, "fp64")
    fb.set_density_screening(fock=False)
    e_off, st_off = _energy(fb, r, precision)
    fb.set_density_screening(fock=True)
    e_on, st_on = _energy(fb, r, precision)
    fb.set_density_screening()
    # quartets move from the accurate tier to FP32, none is lost
    assert st_on["quartets_fp64"] < st_off["quartets_fp64"]
    assert st_on["quartets_fp64"] + st_on["quartets_fp32"] == st_off["quartets_fp64"] + st_off["quartets_fp32"]
    assert (st_on["prim_quartets_fp64"] + st_on["prim_quartets_fp32"]
            == st_off["prim_quartets_fp64"] + st_off["prim_quartets_fp32"])
    assert abs(e_on - e64) < 1e-6 and abs(e_off - e64) < 1e-6


def test_gradient_screening_matches_unscreened(cuda, cluster):
    from segfault_py_gb300.grad import rhf_gradient
    mol, fb, r = cluster
    fb.set_density_screening(grad=False)
    g_off = rhf_gradient(mol, r, fb, precision="fp64")
    fb.set_density_screening(grad=True)
    g_on = rhf_gradient(mol, r, fb, precision="fp64")
    g_mx = rhf_gradient(mol, r, fb, precision="mixed_df")
    assert float((g_on - g_off).abs().max()) < 1e-8
    assert float((g_mx - g_off).abs().max()) < 1e-6


def test_graph_replay_reclassifies_a_new_density(cuda, cluster):
    """The classification is part of the captured build: a replay after D
    changed gives the eager result for the new D."""
    mol, fb, r = cluster
    fb.set_density_screening(fock=True)
    D = r.D.contiguous().clone()
    J = torch.empty_like(D)
    K = torch.empty_like(D)
    g = fb.capture_jk(D, J, K, precision="mixed_df")
    rng = np.random.default_rng(0)
    A = torch.tensor(rng.standard_normal(D.shape) * 0.02, device=D.device)
    D.add_(A + A.T)
    g.replay()
    torch.cuda.synchronize()
    Je, Ke = fb.jk(D, precision="mixed_df")
    fb.set_density_screening()
    scale = max(float(Je.abs().max()), float(Ke.abs().max()))
    assert float((J - Je).abs().max()) <= 1e-12 * scale
    assert float((K - Ke).abs().max()) <= 1e-12 * scale
