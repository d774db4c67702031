"""sf_fock_jk_noalloc: the Fock build for callers that cannot call cudaMalloc
when they build a Fock matrix (their device memory is owned by another
component, or the loop must not enter the allocator).  Its scratch lives in a
static device array of the library instead of in the handle.

The test calls the entry point through the C ABI, twice in a row (the second
call must clear what the first left in the shared array), and compares both
results with sf_fock_jk on the same inputs.  It runs last (file name) so that
a failure here cannot hide the other tests when pytest stops at the first
failure, and it needs nothing from them: it builds its own handle."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def test_noalloc_matches_fock_jk_twice(cuda):
    from segfault_py_gb300 import _lib, geometry as G
    from segfault_py_gb300.fock import FockBuilder
    from segfault_py_gb300.molecule import Molecule
    L = _lib.lib()
    s, x = G.water_cluster(4, seed=7)
    mol = Molecule.from_geometry(s, x, "6-31g*")
    n = mol.nao
    rng = np.random.default_rng(3)
    A = rng.standard_normal((n, n)) * 0.05
    D = torch.tensor(A + A.T, device=cuda)
    for prec, c32 in (("fp64", 1e-5), ("mixed", 1e-6)):
        fb = FockBuilder(mol, device=cuda, cutoff=1e-12, fp32_cutoff=c32)
        Jr, Kr = fb.jk(D, precision=prec)          # reference result; also builds the quartet lists
        torch.cuda.synchronize()
        scale = max(float(Jr.abs().max()), float(Kr.abs().max()))
        st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        for _ in range(2):
            J = torch.full((n, n), float("nan"), dtype=torch.float64, device=cuda)
            K = torch.full((n, n), float("nan"), dtype=torch.float64, device=cuda)
            rc = L.sf_fock_jk_noalloc(fb.handle, _ptr(D), _ptr(J), _ptr(K), _lib.PRECISION[prec],
                                      1e-12, c32, st)
            assert rc == 0, L.sf_last_error()
            torch.cuda.synchronize()
            assert float((J - Jr).abs().max()) <= 1e-12 * scale
            assert float((K - Kr).abs().max()) <= 1e-12 * scale
        fb.close()


def test_noalloc_rejects_unprepared_and_oversized(cuda):
    from segfault_py_gb300 import _lib, geometry as G
    from segfault_py_gb300.fock import FockBuilder
    L = _lib.lib()
    # lists not built for these cutoffs -> SF_ESTATE, nothing launched
    t = G.random_quartet_shells(8, seed=1, kmax=2)
    fb = FockBuilder(t, device=cuda)
    n = fb.nao
    D = torch.zeros((n, n), dtype=torch.float64, device=cuda)
    J = torch.empty_like(D)
    K = torch.empty_like(D)
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert L.sf_fock_jk_noalloc(fb.handle, _ptr(D), _ptr(J), _ptr(K), 0, 1e-12, 1e-5, st) == -4
    assert b"not built" in L.sf_last_error()
    fb.close()
    # more AOs than the static scratch holds -> SF_EINVAL with the limit in the message
    big = G.random_quartet_shells(180, seed=2, kmax=1, box=40.0)
    big["l"][:] = 2
    nc = 6
    big["ao_offset"] = (np.arange(180) * nc).astype(np.int32)
    fb = FockBuilder(big, device=cuda)
    assert fb.nao == 1080 > 1024
    D = torch.zeros((fb.nao, fb.nao), dtype=torch.float64, device=cuda)
    assert L.sf_fock_jk_noalloc(fb.handle, _ptr(D), _ptr(D), _ptr(D), 0, 1e-12, 1e-5, st) == -1
    assert b"SF_NOALLOC_MAX_NAO" in L.sf_last_error()
    fb.close()


def test_noalloc_needs_fresh_lists_after_retuning(cuda):
    """sf_autotune re-cuts the quartet lists: the allocation-free call then
    refuses (SF_ESTATE) until one allocating sf_fock_jk has rebuilt them."""
    from segfault_py_gb300 import _lib, geometry as G
    from segfault_py_gb300.fock import FockBuilder
    from segfault_py_gb300.molecule import Molecule
    L = _lib.lib()
    s, x = G.water_cluster(2, seed=5)
    mol = Molecule.from_geometry(s, x, "6-31g*")
    n = mol.nao
    rng = np.random.default_rng(4)
    A = rng.standard_normal((n, n)) * 0.05
    D = torch.tensor(A + A.T, device=cuda)
    fb = FockBuilder(mol, device=cuda, cutoff=1e-12, fp32_cutoff=1e-5)
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    J = torch.empty_like(D)
    K = torch.empty_like(D)
    fb.autotune(D, precision="fp64", reps=1)
    assert L.sf_fock_jk_noalloc(fb.handle, _ptr(D), _ptr(J), _ptr(K), 0, 1e-12, 1e-5, st) == -4
    Jr, Kr = fb.jk(D, precision="fp64")
    assert L.sf_fock_jk_noalloc(fb.handle, _ptr(D), _ptr(J), _ptr(K), 0, 1e-12, 1e-5, st) == 0, L.sf_last_error()
    torch.cuda.synchronize()
    scale = max(float(Jr.abs().max()), float(Kr.abs().max()))
    assert float((J - Jr).abs().max()) <= 1e-12 * scale
    assert float((K - Kr).abs().max()) <= 1e-12 * scale
    fb.close()
