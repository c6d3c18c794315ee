"""Variance-adaptive paths per knot (the reference's Compute_h_N rule,
PDDSparseGM.cpp:4338-4395): N_k = 4 V_k / (0.66666 eps)^2 from a pilot,
rounded up to the next multiple of 256 and clamped; the continuation runs
paths N0 .. N_k-1 of the same Philox streams, so a knot's result equals a
uniform run with N = N_k."""
import numpy as np
import pytest

import pdds_gb300 as P
from pdds_gb300.config import fac_rule

pytestmark = pytest.mark.gpu

SW, NE, NSUB, NNODE, H = (-1.0, -1.0), (1.0, 1.0), 4, 11, 1e-3
N0, NMAX, EPS = 512, 16384, 0.01


def expected_n(B, BB):
    var = np.maximum(BB - B * B, 0.0)
    n = (4.0 * var / (EPS * 0.66666) ** 2).astype(np.int64)
    n = (1 + n // 256) * 256
    return np.clip(n, N0, NMAX)


def test_adaptive_paths_follow_the_rule_and_continue_streams():
    fac = fac_rule(2.0, NSUB, NNODE)
    bvp = P.BVP.poisson_sincos()
    with P.PDDSparseGM(SW, NE, NSUB, NNODE, fac) as pd:
        pilot = pd.estimate(bvp, N0, H, mode=P.MODE_MIXED, seed=9, adaptive_h=True)
        ad = pd.estimate(bvp, N0, H, mode=P.MODE_MIXED, seed=9, adaptive_h=True, adaptive_n=True, npaths_max=NMAX,
                         target_stderr=EPS)
        mc = pilot.npaths > 0
        assert np.all(ad.npaths[~mc] == 0)
        nk = ad.npaths[mc]
        assert np.all(nk % 256 == 0) and nk.min() >= N0 and nk.max() <= NMAX
        assert len(np.unique(nk)) > 3, "the workload should spread N_k"
        want = expected_n(pilot.B[mc], pilot.BB[mc])
        # the pilot is recomputed: summation order may move a knot across a rounding edge
        assert np.mean(nk == want) > 0.95 and np.max(np.abs(nk - want)) <= 256
        assert ad.info["paths"] == int(ad.npaths.sum())
        # a knot with N_k = M matches the uniform run with M paths (paths 0 .. M-1)
        M = int(np.bincount(nk // 256).argmax() * 256)
        uni = pd.estimate(bvp, M, H, mode=P.MODE_MIXED, seed=9, adaptive_h=True)
        sel = np.where(mc)[0][nk == M]
        assert len(sel) > 0
        assert np.max(np.abs(ad.B[sel] - uni.B[sel])) < 1e-9
        for k in sel[:20]:
            a, b = pd.row_ptr[k], pd.row_ptr[k + 1]
            assert np.max(np.abs(ad.val[a:b] - uni.val[a:b])) < 1e-5  # FP32 histograms, other chunking
        # standard error of B at or below the target where N_k is not clamped
        free = (nk > N0) & (nk < NMAX)
        var = np.maximum(ad.BB[mc] - ad.B[mc] ** 2, 0.0)
        se = np.sqrt(var[free] / nk[free])
        assert np.quantile(se, 0.95) < 0.5 * EPS
        u, _ = pd.solve_interface()
        assert np.sqrt(np.mean((u - bvp.u(pd.x, pd.y)) ** 2)) < 3e-2


def test_autotuner_keeps_results_and_picks_a_valid_shape():
    """The tuned launch shape changes only the work split: every (knot, path)
    keeps its Philox stream, so the estimate equals the untuned one up to
    summation order."""
    fac = fac_rule(2.0, NSUB, NNODE)
    bvp = P.BVP.poisson_sincos()
    with P.PDDSparseGM(SW, NE, NSUB, NNODE, fac) as pd:
        before = pd.estimate(bvp, 3000, H, mode=P.MODE_MIXED, seed=4, adaptive_h=True, richardson=True)
        t = pd.autotune(bvp, 3000, H, sample_knots=64, adaptive_h=True, richardson=True)
        assert 1 <= t["blocks_per_sm"] <= 8 and 1 <= t["paths_per_item"] <= 3000
        assert t["candidates"] >= 2 and 0 < t["best_ms"] <= t["default_ms"] * 1.2  # timing noise
        assert t["cta_threads"] in (128, 256)
        after = pd.estimate(bvp, 3000, H, mode=P.MODE_MIXED, seed=4, adaptive_h=True, richardson=True)
        assert np.max(np.abs(after.B - before.B)) < 1e-9
        assert np.max(np.abs(after.val - before.val)) < 1e-5
        # a later estimate without a block size of its own runs the tuned one
        assert after.info["cta_threads"] == t["cta_threads"]
        # a block size imposed by the caller is kept and only the rest is searched
        other = 384 - t["cta_threads"]
        t2 = pd.autotune(bvp, 3000, H, sample_knots=64, adaptive_h=True, richardson=True, cta_threads=other)
        assert t2["cta_threads"] == other
        again = pd.estimate(bvp, 3000, H, mode=P.MODE_MIXED, seed=4, adaptive_h=True, richardson=True)
        assert again.info["cta_threads"] == other
        with pytest.raises(P.PDDSError):
            pd.autotune(bvp, 3000, H, sample_knots=64, cta_threads=192)


def test_autotuner_times_the_adaptive_continuation():
    """With adaptive_n the tuner also times the last adaptive estimate's
    continuation (the items of paths N0 .. N_k) at both block sizes and item
    sizes, and the next adaptive estimate continues with the fastest: a different work
    split of the same Philox streams, so the same estimate up to summation
    order where the recomputed pilot gives the same N_k."""
    fac = fac_rule(2.0, NSUB, NNODE)
    bvp = P.BVP.poisson_sincos()
    opts = dict(adaptive_h=True, richardson=True, adaptive_n=True, npaths_max=NMAX, target_stderr=EPS)
    with P.PDDSparseGM(SW, NE, NSUB, NNODE, fac) as pd:
        t0 = pd.autotune(bvp, N0, H, sample_knots=64, adaptive_h=True, richardson=True, adaptive_n=True)
        assert t0["continuation_threads"] == 0  # no adaptive estimate on this layout yet
        before = pd.estimate(bvp, N0, H, mode=P.MODE_MIXED, seed=4, **opts)
        t = pd.autotune(bvp, N0, H, sample_knots=64, adaptive_h=True, richardson=True, adaptive_n=True)
        assert t["continuation_threads"] in (128, 256)
        assert min(t["continuation_ms"]) > 0
        assert t["continuation_ms"][(t["continuation_threads"] // 128) - 1] == min(t["continuation_ms"])
        assert t["continuation_paths_per_item"] in (2048, 4096, 8192, 16384)
        after = pd.estimate(bvp, N0, H, mode=P.MODE_MIXED, seed=4, **opts)
        same = after.npaths == before.npaths
        assert np.mean(same) > 0.95
        assert np.max(np.abs(after.B - before.B)[same]) < 1e-9
