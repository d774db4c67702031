"""Error paths on the GPU without a fault: a bounded wait that runs out is
reported as an error status and the context stays usable.

The tensor-core McMurchie-Davidson kernels bound every wait for their MMA
commits.  sf_debug_tc_wait_limit(0) makes the first wait count as run out
before its first poll: the kernel flags the timeout, waits (bounded) for the
MMAs still in flight, frees its tensor memory and returns; the run fails with
SF_ECUDA.  With the default restored the same plan runs and matches the FP64
Rys kernels."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tensor_core_wait_timeout_reports_error(cuda):
    from segfault_py_gb300 import _lib
    from segfault_py_gb300.fock import FockBuilder
    from segfault_py_gb300.molecule import Molecule
    mol = Molecule.from_geometry(["O", "H", "H"], [[0, 0, 0], [0.757, 0.587, 0], [-0.757, 0.587, 0]], "6-31g*")
    fb = FockBuilder(mol, device=cuda)
    ns = fb.nshell
    q = np.array([(a, b, c, d) for a in range(ns) for b in range(ns) for c in range(ns) for d in range(ns)],
                 dtype=np.int32)
    plan = fb.eri_plan(q)
    ref = plan.run("fp64").cpu().numpy()
    L = _lib.lib()
    try:
        _lib.check(L.sf_debug_tc_wait_limit(0))
        with pytest.raises(_lib.SegFockError) as ei:
            plan.run("fp32", engine="md")
        assert ei.value.code == -3 and "timed out" in str(ei.value)   # SF_ECUDA
    finally:
        _lib.check(L.sf_debug_tc_wait_limit(-1))
    # the context and the tensor memory are usable again
    tc = plan.run("fp32", engine="md").cpu().numpy()
    assert np.abs(tc - ref).max() < 1e-5
    plan.close()
    fb.close()
