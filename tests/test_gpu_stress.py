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
