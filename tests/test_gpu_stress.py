"""Raw-ERI stress test (the batched configuration): random contracted shell
quartets drawn uniformly over the 21 canonical classes ss|ss ... dd|dd,
contraction depth 1-6, exponents log-uniform in [0.05, 1e4], normalised
coefficients, centres uniform in a 10 A box.  All quartets are evaluated on
the GPU in FP64 and FP32 through sf_eri_batch; a seeded sample is checked
against the oracle (exact Rys roots), FP64 to 1e-10 and FP32 to 1e-4 of the
quartet's largest integral plus 1e-14 / 1e-7 of the largest integral of the
sample (quartets whose integrals underflow)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

def stress_quartets(nq, nshell=600, seed=0):
    from segfault_py_gb300 import geometry as G
    return G.random_quartet_batch(nq, nshell=nshell, seed=seed)


def _oracle_block(table, q):
    from test_gpu_parity import _shell_cgfs
    cg = [_shell_cgfs(table, s) for s in q]
    n0, n1, n2, n3 = (len(c) for c in cg)
    idx = [[i, n0 + j, n0 + n1 + k, n0 + n1 + n2 + l]
           for i in range(n0) for j in range(n1) for k in range(n2) for l in range(n3)]
    return O.eri_list(cg[0] + cg[1] + cg[2] + cg[3], np.array(idx)).reshape(n0, n1, n2, n3)


@pytest.mark.parametrize("precision,rtol,gtol", [("fp64", 1e-10, 1e-14), ("fp32", 1e-4, 1e-7)])
def test_stress_batch_sampled_vs_oracle(cuda, precision, rtol, gtol):
    from segfault_py_gb300.fock import FockBuilder
    table, q = stress_quartets(100_000)
    fb = FockBuilder(table, device=cuda)
    blocks = fb.eri_quartets(q, precision=precision)
    assert len(blocks) == len(q)
    rng = np.random.default_rng(7)
    sample = rng.choice(len(q), 60, replace=False)
    O.use_exact_roots(True)
    try:
        refs = [_oracle_block(table, q[s]) for s in sample]
    finally:
        O.use_exact_roots(False)
    gmax = max(np.abs(r).max() for r in refs)
    for s, ref in zip(sample, refs):
        blk = blocks[s]
        assert np.all(np.isfinite(blk))
        assert np.abs(blk - ref).max() <= rtol * np.abs(ref).max() + gtol * gmax, (q[s].tolist(),)
    fb.close()


def test_eri_plan_matches_batch_with_offsets(cuda):
    """sf_eri_plan (packed outputs) against sf_eri_batch with caller-chosen
    offsets (blocks stored in reverse order); both FP64 and FP32; the packed
    offsets are the running sums of the block sizes."""
    import ctypes as C
    import torch
    from segfault_py_gb300 import _lib
    from segfault_py_gb300.fock import FockBuilder
    table, q = stress_quartets(20_000, seed=3)
    fb = FockBuilder(table, device=cuda)
    nc = (fb.l + 1) * (fb.l + 2) // 2
    sizes = np.prod(nc[q], axis=1).astype(np.int64)
    plan = fb.eri_plan(q)
    assert plan.outputs == int(sizes.sum())
    assert np.array_equal(plan.offsets[1:], np.cumsum(sizes)[:-1]) and plan.offsets[0] == 0
    assert plan.prim_quartets == int(np.sum(table["nprim"][q].prod(axis=1)))
    rev = np.zeros(len(q), dtype=np.int64)
    rev[::-1] = np.concatenate([[0], np.cumsum(sizes[::-1])[:-1]])
    dq = torch.from_numpy(q).to(cuda)
    do = torch.from_numpy(rev).to(cuda)
    for prec in ("fp64", "fp32"):
        packed = plan.run(prec).cpu().numpy()
        again = plan.run(prec).cpu().numpy()
        assert np.array_equal(packed, again)
        out = torch.zeros(plan.outputs, dtype=torch.float64, device=cuda)
        _lib.check(_lib.lib().sf_eri_batch(fb.handle, C.c_void_p(dq.data_ptr()), len(q), _lib.PRECISION[prec],
                                           C.c_void_p(out.data_ptr()), C.c_void_p(do.data_ptr()),
                                           C.c_void_p(torch.cuda.current_stream().cuda_stream)))
        o = out.cpu().numpy()
        for k in range(0, len(q), 97):
            a = packed[plan.offsets[k]:plan.offsets[k] + sizes[k]]
            b = o[rev[k]:rev[k] + sizes[k]]
            assert np.array_equal(a, b), k
    plan.close()


def test_md_engine_matches_rys(cuda):
    """The McMurchie-Davidson engine (Hermite E coefficients, Boys function,
    R_tuv recursion) and the Rys kernels are independent algorithms: on the
    random stress batch (all 21 classes, contraction 1-6, exponents up to 1e4)
    they agree to 1e-10 of each quartet's largest integral plus 1e-14 of the
    batch's largest."""
    from segfault_py_gb300.fock import FockBuilder
    table, q = stress_quartets(20_000, seed=5)
    fb = FockBuilder(table, device=cuda)
    nc = (fb.l + 1) * (fb.l + 2) // 2
    sizes = np.prod(nc[q], axis=1).astype(np.int64)
    plan = fb.eri_plan(q)
    rys = plan.run("fp64").cpu().numpy()
    md = plan.run("fp64", engine="md").cpu().numpy()
    gmax = np.abs(rys).max()
    for k in range(len(q)):
        a = rys[plan.offsets[k]:plan.offsets[k] + sizes[k]]
        b = md[plan.offsets[k]:plan.offsets[k] + sizes[k]]
        assert np.abs(a - b).max() <= 1e-10 * np.abs(a).max() + 1e-14 * gmax, (k, q[k].tolist())
    plan.close()


def test_md_engine_h2o_vs_reference(cuda, h2o_golden):
    """MD engine against the reference's own integrals (all 406 unique H2O/STO-3G ERIs)."""
    from segfault_py_gb300.fock import FockBuilder
    from segfault_py_gb300.molecule import Molecule
    from test_gpu_parity import H2O
    mol = Molecule.from_geometry(*H2O, "sto-3g")
    fb = FockBuilder(mol, device=cuda)
    ns = fb.nshell
    quartets = np.array([(a, b, c, d) for a in range(ns) for b in range(ns) for c in range(ns) for d in range(ns)],
                        dtype=np.int32)
    plan = fb.eri_plan(quartets)
    md = plan.run("fp64", engine="md").cpu().numpy()
    nc = (fb.l + 1) * (fb.l + 2) // 2
    o = fb.ao_offset
    n = mol.nao
    E = np.zeros((n, n, n, n))
    for k, (a, b, c, d) in enumerate(quartets):
        blk = md[plan.offsets[k]:plan.offsets[k] + nc[a] * nc[b] * nc[c] * nc[d]].reshape(nc[a], nc[b], nc[c], nc[d])
        E[o[a]:o[a] + nc[a], o[b]:o[b] + nc[b], o[c]:o[c] + nc[c], o[d]:o[d] + nc[d]] = blk
    qq = np.array(h2o_golden["quartets"])
    got = E[qq[:, 0], qq[:, 1], qq[:, 2], qq[:, 3]]
    assert np.abs(got - np.array(h2o_golden["eri"])).max() < 5e-14
    plan.close()


def test_md_tensor_core_engine_matches_rys(cuda):
    """FP32 McMurchie-Davidson with the bra E contraction as tcgen05 TF32
    GEMMs (three-pass split): against the FP64 Rys integrals on a random batch
    over all 21 classes, to FP32 accuracy (1e-4 of each quartet's largest
    integral plus 1e-7 of the batch's largest, the bound of the FP32 Rys
    kernels)."""
    from segfault_py_gb300.fock import FockBuilder
    table, q = stress_quartets(4_000, seed=9)
    fb = FockBuilder(table, device=cuda)
    nc = (fb.l + 1) * (fb.l + 2) // 2
    sizes = np.prod(nc[q], axis=1).astype(np.int64)
    plan = fb.eri_plan(q)
    ref = plan.run("fp64").cpu().numpy()
    tc = plan.run("fp32", engine="md").cpu().numpy()
    gmax = np.abs(ref).max()
    worst = 0.0
    for k in range(len(q)):
        a = ref[plan.offsets[k]:plan.offsets[k] + sizes[k]]
        b = tc[plan.offsets[k]:plan.offsets[k] + sizes[k]]
        err = np.abs(a - b).max()
        bound = 1e-4 * np.abs(a).max() + 1e-7 * gmax
        worst = max(worst, err / bound)
        assert err <= bound, (k, q[k].tolist(), err, np.abs(a).max())
    plan.close()
