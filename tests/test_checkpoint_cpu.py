"""Checkpoint/resume of an estimation (pdds_gb300.checkpoint) on the host,
against a stand-in for PDDSparseGM whose per-knot results, like the
library's, depend only on the knot and the run's arguments: an interrupted
run resumed from its parts equals one whole run, parts already on disk are
not run again, and parts of another run are refused."""
import os

import numpy as np
import pytest

from pdds_gb300.api import Estimate
from pdds_gb300.checkpoint import estimate_resumable, part_ranges


class FakeBVP:
    kind, params, use_cv, tables = 0, (), True, None


class FakeLayout:
    """K knots, the first nb on the boundary; knot k's row has k % 5 entries."""

    def __init__(self, K=40, nb=7):
        self.K, self.nb = K, nb
        rng = np.random.default_rng(0)
        self.order = np.concatenate([rng.permutation(np.arange(nb, K)), np.arange(nb)]).astype(np.int32)
        lens = np.array([0 if k < nb else k % 5 + 1 for k in range(K)])
        self.row_ptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
        self.nnz = int(self.row_ptr[-1])
        self.col = (np.arange(self.nnz) % K).astype(np.int32)
        self.x = np.linspace(0, 1, K)
        self.y = np.linspace(1, 2, K)
        self.n_mc = K - nb
        self.calls = []

    def estimate(self, bvp, npaths, h, knot_first=0, knot_count=0, seed=1, **kw):
        self.calls.append((knot_first, knot_count))
        mc = self.order[:self.n_mc]
        cnt = knot_count or self.n_mc - knot_first
        run = mc[knot_first:knot_first + cnt]
        val, var = np.zeros(self.nnz), np.zeros(self.nnz)
        B, BB = np.zeros(self.K), np.zeros(self.K)
        B[:self.nb] = np.arange(self.nb) * 0.5  # boundary knots: B = g
        BB[:self.nb] = B[:self.nb] ** 2
        kn = np.zeros(self.K, np.int32)
        for k in run:
            r = np.random.default_rng([seed, int(k)])
            a, b = self.row_ptr[k], self.row_ptr[k + 1]
            val[a:b] = r.normal(size=b - a)
            var[a:b] = r.random(b - a)
            B[k], BB[k] = r.normal(), r.random()
            kn[k] = npaths
        return Estimate(self.row_ptr, self.col, val, var, B, BB, {"path_steps": 10 * len(run), "ms_paths": 1.0}, kn)


def _same(a, b):
    for f in ("val", "var", "B", "BB", "npaths"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f


def test_part_ranges_cover_every_position():
    for n, p in ((33, 8), (5, 5), (100, 7)):
        r = part_ranges(n, p)
        assert r[0][0] == 0 and sum(c for _, c in r) == n
        assert all(r[i][0] + r[i][1] == r[i + 1][0] for i in range(p - 1))


def test_interrupted_run_resumes_to_the_whole_run(tmp_path):
    pd = FakeLayout()
    whole = pd.estimate(FakeBVP(), 100, 1e-3, seed=3)
    d = str(tmp_path / "ck")
    assert estimate_resumable(pd, d, FakeBVP(), 100, 1e-3, parts=6, max_new_parts=2, seed=3) is None
    assert len([f for f in os.listdir(d) if f.startswith("part_")]) == 2
    pd.calls.clear()
    est = estimate_resumable(pd, d, FakeBVP(), 100, 1e-3, parts=6, seed=3)
    assert len(pd.calls) == 4  # only the missing parts ran
    assert est.info["parts_run"] == 4 and est.info["path_steps"] == 10 * pd.n_mc
    _same(est, whole)
    pd.calls.clear()
    again = estimate_resumable(pd, d, FakeBVP(), 100, 1e-3, parts=6, seed=3)
    assert pd.calls == []  # everything from disk
    _same(again, whole)


def test_parts_of_another_run_are_refused(tmp_path):
    pd = FakeLayout()
    d = str(tmp_path / "ck")
    estimate_resumable(pd, d, FakeBVP(), 100, 1e-3, parts=4, max_new_parts=1, seed=3)
    with pytest.raises(ValueError):
        estimate_resumable(pd, d, FakeBVP(), 100, 1e-3, parts=4, seed=4)
    with pytest.raises(ValueError):
        estimate_resumable(pd, d, FakeBVP(), 200, 1e-3, parts=4, seed=3)
    with pytest.raises(ValueError):
        estimate_resumable(pd, d, FakeBVP(), 100, 1e-3, parts=4, seed=3, adaptive_n=True)


def test_an_interrupted_write_leaves_no_part(tmp_path):
    pd = FakeLayout()
    d = str(tmp_path / "ck")
    estimate_resumable(pd, d, FakeBVP(), 100, 1e-3, parts=3, max_new_parts=1, seed=3)
    # a write that died before its rename leaves only the temporary file
    with open(os.path.join(d, "part_0001.npz.tmp.npz"), "wb") as f:
        f.write(b"truncated")
    est = estimate_resumable(pd, d, FakeBVP(), 100, 1e-3, parts=3, seed=3)
    _same(est, pd.estimate(FakeBVP(), 100, 1e-3, seed=3))
