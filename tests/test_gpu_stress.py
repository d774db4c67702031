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

PAIR_L = [(0, 0), (1, 0), (1, 1), (2, 0), (2, 1), (2, 2)]
CLASSES = [(PAIR_L[x], PAIR_L[y]) for x in range(6) for y in range(x + 1)]


def stress_quartets(nq, nshell=600, seed=0):
    from segfault_py_gb300 import geometry as G
    table = G.random_quartet_shells(nshell, seed=seed, kmax=6, box=10.0)
    rng = np.random.default_rng(seed + 1)
    ls = table["l"]
    byl = [np.where(ls == l)[0] for l in range(3)]
    cls = rng.integers(0, 21, nq)
    q = np.empty((nq, 4), dtype=np.int32)
    for k, ((la, lb), (lc, ld)) in enumerate(CLASSES):
        sel = np.where(cls == k)[0]
        for col, l in enumerate((la, lb, lc, ld)):
            q[sel, col] = rng.choice(byl[l], len(sel))
    return table, q


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
