"""Device buffers of a destroyed context serve the next context.

pdds_destroy keeps the context's device buffers (the stream is idle by
then) and the next context of the same device takes buffers of the same
size classes from them instead of calling cudaMalloc.  A context built on
recycled buffers must give the same estimate as the first one (the buffers
hold the old context's values, so every accumulator has to be cleared by
the library itself), and pdds_release_cached_blocks must hand the memory
back to the device."""
import numpy as np
import pytest

import pdds_gb300 as P
from pdds_gb300.config import fac_rule

pytestmark = pytest.mark.gpu


def _run(seed):
    nsub, nnode = 12, 43
    with P.PDDSparseGM((-1.0, -1.0), (1.0, 1.0), nsub, nnode, fac_rule(2.0, nsub, nnode)) as pd:
        est = pd.estimate(P.BVP.poisson_sincos(), 256, 1e-3, mode=P.MODE_MIXED, seed=seed, adaptive_h=True,
                          richardson=True, dup_sum=True)
        u, info = pd.solve_interface()
    return est, u, info


def test_recycled_buffers_give_the_same_estimate():
    torch = pytest.importorskip("torch")
    P.release_cached_blocks()
    a_est, a_u, a_info = _run(7)
    b_est, b_u, b_info = _run(7)  # every buffer of this context comes from the cache
    # the same paths (the step count is exact); the FP32 exit deposits and
    # per-warp score sums are added in arrival order, so G and B differ by
    # FP32 rounding (G ~1e-7, B ~4e-9 measured) from run to run, while a
    # buffer left uncleared would shift them by their own size (~1e-2, ~1)
    assert b_est.info["path_steps"] == a_est.info["path_steps"]
    np.testing.assert_allclose(b_est.val, a_est.val, rtol=0, atol=1e-6)
    np.testing.assert_allclose(b_est.B, a_est.B, rtol=0, atol=1e-6)
    np.testing.assert_allclose(b_u, a_u, rtol=0, atol=1e-5)
    assert abs(b_info["iterations"] - a_info["iterations"]) <= 1
    # a different seed on recycled buffers is a different estimate
    c_est, _, _ = _run(8)
    assert np.abs(c_est.val - a_est.val).max() > 1e-3
    # the kept buffers (G and its square alone are 2 x 32 MB here) go back
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    P.release_cached_blocks(0)
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 - free0 >= 32 << 20, (free0, free1)
    P.release_cached_blocks(-1)  # nothing left: a no-op
