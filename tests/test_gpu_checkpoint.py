"""Knot ranges and checkpoint/resume on the GPU: an estimation split into
parts, interrupted and resumed from the parts on disk, equals one whole run
bit for bit in the replay mode and up to summation order in MIXED."""
import numpy as np
import pytest

import pdds_gb300 as P
from pdds_gb300 import _capi as capi
from pdds_gb300.checkpoint import estimate_resumable
from pdds_gb300.config import fac_rule

pytestmark = pytest.mark.gpu

SW, NE = (-1.0, -1.0), (1.0, 1.0)


def test_replay_resume_is_bit_identical(tmp_path):
    nsub, nnode, N, h = 3, 7, 300, 1e-3
    bvp = P.BVP.poisson_sincos()
    with P.PDDSparseGM(SW, NE, nsub, nnode, fac_rule(2.0, nsub, nnode)) as pd:
        whole = pd.estimate(bvp, N, h, mode=P.MODE_REPLAY_FP64, seed=12, want_var=True, diagnostics=True)
        d = str(tmp_path / "ck")
        opts = dict(mode=P.MODE_REPLAY_FP64, seed=12, want_var=True, diagnostics=True)
        assert estimate_resumable(pd, d, bvp, N, h, parts=5, max_new_parts=2, **opts) is None
    # a new context (a restarted process) picks the run up from disk
    with P.PDDSparseGM(SW, NE, nsub, nnode, fac_rule(2.0, nsub, nnode)) as pd:
        est = estimate_resumable(pd, d, bvp, N, h, parts=5, **opts)
        assert est.info["parts_run"] == 3
        for f in ("val", "var", "B", "BB", "npaths", "diag"):
            assert np.array_equal(getattr(est, f), getattr(whole, f)), f
        u1, _ = pd.solve_interface()
    assert np.all(np.isfinite(u1))


def test_mixed_resume_matches_the_whole_run(tmp_path):
    nsub, nnode, N, h = 4, 11, 2048, 1e-3
    bvp = P.BVP.poisson_sincos()
    opts = dict(mode=P.MODE_MIXED, seed=2, richardson=True, adaptive_h=True)
    with P.PDDSparseGM(SW, NE, nsub, nnode, fac_rule(2.0, nsub, nnode)) as pd:
        whole = pd.estimate(bvp, N, h, **opts)
        d = str(tmp_path / "ck")
        assert estimate_resumable(pd, d, bvp, N, h, parts=4, max_new_parts=3, **opts) is None
        est = estimate_resumable(pd, d, bvp, N, h, parts=4, **opts)
    assert np.array_equal(est.npaths, whole.npaths)
    np.testing.assert_allclose(est.val, whole.val, rtol=0, atol=2e-6)
    np.testing.assert_allclose(est.B, whole.B, rtol=1e-6, atol=1e-9)
    assert est.info["path_steps"] == whole.info["path_steps"]


def test_knot_range_runs_only_its_knots():
    nsub, nnode, N, h = 3, 7, 256, 1e-3
    bvp = P.BVP.poisson_sincos()
    with P.PDDSparseGM(SW, NE, nsub, nnode, fac_rule(2.0, nsub, nnode)) as pd:
        part = pd.estimate(bvp, N, h, mode=P.MODE_FP64, seed=5, knot_first=3, knot_count=10)
        assert int((part.npaths > 0).sum()) == 10
        ran = part.npaths > 0
        rows = np.repeat(np.arange(pd.K), np.diff(pd.row_ptr))
        assert np.all(part.val[~ran[rows]] == 0.0)
        with pytest.raises(P.PDDSError) as e:
            pd.estimate(bvp, N, h, mode=P.MODE_FP64, knot_first=pd.n_mc, knot_count=1)
        assert e.value.status == capi.ERR_INVALID
        with pytest.raises(P.PDDSError) as e:
            pd.estimate(bvp, N, h, mode=P.MODE_MIXED, knot_first=1, adaptive_n=True, npaths_max=512,
                        target_stderr=1e-3)
        assert e.value.status == capi.ERR_INVALID
