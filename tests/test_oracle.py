"""The CPU oracle pinned against the reference's own outputs (golden fixtures)."""
import numpy as np
import pytest

from conftest import CGF, load_golden
from oracle import oracle as O


def test_oracle_rys_matches_reference_mmd_h2o(h2o_golden):
    cg = [CGF(d) for d in h2o_golden["cgfs"]]
    v = O.eri_list(cg, np.array(h2o_golden["quartets"]))
    assert np.abs(v - np.array(h2o_golden["eri"])).max() < 5e-14


def test_oracle_rys_exact_roots_match_reference_mmd(h2o_golden):
    cg = [CGF(d) for d in h2o_golden["cgfs"]]
    O.use_exact_roots(True)
    try:
        v = O.eri_list(cg, np.array(h2o_golden["quartets"]))
    finally:
        O.use_exact_roots(False)
    assert np.abs(v - np.array(h2o_golden["eri"])).max() < 2e-14


def test_oracle_mmd_matches_reference_mmd(h2o_golden):
    cg = [CGF(d) for d in h2o_golden["cgfs"]]
    v = O.eri_list(cg, np.array(h2o_golden["quartets"]), method="mmd")
    assert np.abs(v - np.array(h2o_golden["eri"])).max() < 1e-14


def test_oracle_all_classes_vs_reference_mmd(quartet_golden):
    sh = quartet_golden["shells"]
    worst = 0.0
    for e in quartet_golden["quartets"]:
        cg = [CGF(sh[s]["cgfs"][c]) for s, c in zip(e["shells"], e["comps"])]
        v = O.eri_list(cg, np.array([[0, 1, 2, 3]]))[0]
        worst = max(worst, abs(v - e["value"]) / max(abs(e["value"]), 1e-10))
    assert worst < 1e-11


def test_oracle_roots_vs_reference_root5():
    g = load_golden("root5_ref.json")
    for x, res in zip(g["x"], g["res"]):
        mine = O.root5(x)
        ref = np.array(res)
        np.testing.assert_allclose(mine, ref, rtol=2e-12, atol=1e-300)


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5])
def test_exact_rys_rule_reproduces_boys_moments(n):
    # sum_i w_i u_i^m = F_m(x), m < 2n; F_m from the oracle's Boys function,
    # itself checked against scipy's 1F1 below
    for x in [0.0, 1e-9, 0.37, 2.5, 9.0, 27.0, 63.9, 64.0, 150.0, 4e3]:
        u, w = O.rys_roots_exact(n, x)
        for m in range(2 * n):
            ref = O.boys(m, x)
            assert abs(np.sum(w * u ** m) / ref - 1) < 1e-13, (n, x, m)


def test_boys_vs_scipy_hyp1f1():
    from scipy.special import hyp1f1
    for x in [0.0, 1e-6, 0.3, 4.0, 17.5, 33.0, 44.9, 45.1, 80.0]:
        for m in range(9):
            ref = hyp1f1(m + 0.5, m + 1.5, -x) / (2 * m + 1)
            assert abs(O.boys(m, x) / ref - 1) < 1e-13


def test_oracle_scf_h2o_energy(h2o_golden):
    S, T, V = (np.array(h2o_golden[k]) for k in ("S", "T", "V"))
    n = len(S)
    E = np.zeros((n,) * 4)
    for (i, j, k, l), v in zip(h2o_golden["quartets"], h2o_golden["eri"]):
        for a, b, c, d in [(i, j, k, l), (j, i, k, l), (i, j, l, k), (j, i, l, k),
                           (k, l, i, j), (l, k, i, j), (k, l, j, i), (l, k, j, i)]:
            E[a, b, c, d] = v
    e, *_ = O.scf_diis(S, T, V, 10, h2o_golden["e_nuc"], lambda P: O.jk_dense(E, P), tol=1e-10)
    assert abs(e - (-74.96306315472287)) < 1e-9


def test_oracle_one_electron_vs_reference(h2o_golden):
    cg = [CGF(d) for d in h2o_golden["cgfs"]]
    from segfault_py_gb300.molecule import Molecule
    mol = Molecule.from_geometry(["O", "H", "H"], [[0, 0, 0], [0.757, 0.587, 0], [-0.757, 0.587, 0]], "sto-3g")
    xyz, Z = mol.atom_table()
    S, T, V = O.one_electron(cg, xyz, Z)
    for k, M in zip("STV", (S, T, V)):
        np.testing.assert_allclose(M, np.array(h2o_golden[k]), atol=1e-13)


def test_oracle_jk_direct_equals_dense(h2o_golden):
    cg = [CGF(d) for d in h2o_golden["cgfs"]]
    P = np.array(h2o_golden["density"])
    E = O.build_eri_dense(cg)
    J1, K1 = O.jk_dense(E, P)
    J2, K2 = O.jk_direct(cg, P)
    np.testing.assert_allclose(J2, J1, atol=1e-13)
    np.testing.assert_allclose(K2, K1, atol=1e-13)


@pytest.mark.parametrize("name", ["water", "ammonia", "methane", "hydrogen_peroxide", "methanol", "ethane"])
def test_oracle_scf_ccpvdz_vs_reference_recorded(tmp_path, name):
    """The oracle's integrals and SCF on the reference's own cc-pVDZ inputs
    reproduce the total energies the reference recorded
    (src/hf/benchmark/molecule_test.json), independently of the GPU."""
    from segfault_py_gb300.molecule import Molecule
    g = load_golden("ccpvdz_recorded.json")
    m = g["molecules"][name]
    bas = tmp_path / "cc-pvdz.dat"
    bas.write_text("****\n" + "\n****\n".join(g["basis_blocks"].values()) + "\n****\n")
    xyz = tmp_path / (name + ".xyz")
    xyz.write_text(m["xyz"])
    mol = Molecule(str(xyz), str(bas))
    assert mol.nao == m["recorded"]["ncgf"]
    cg = mol.cgfs
    atom_xyz, Z = mol.atom_table()
    S, T, V = O.one_electron(cg, atom_xyz, Z)
    E = O.build_eri_dense(cg)
    e, *_ = O.scf_diis(S, T, V, mol.nelectron, mol.e_nuc, lambda P: O.jk_dense(E, P), tol=1e-10)
    assert abs(e - m["recorded"]["etot"]) < 1e-8
