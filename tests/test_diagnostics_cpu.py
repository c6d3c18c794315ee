"""Diagnostic sums of the reduction (Reduce_Analytic's sums[],
Solvers/EMFKACSolver.hpp:14-47, 542-558) in the oracle, and the
knot_metadata.csv writer (Process_Metadata, PDDSparseGM.cpp:3092-3155).

The oracle's sums are checked against identities of the sums themselves and
against the counters its reduction already reports (the normals drawn are
2 per step of both legs, tau sums steps x h, (phi + xi) sums phi and xi),
and the linear-leg sums are recomputed from the oracle's per-path exit
records."""
import os

import numpy as np
import pytest

import oracle as O
from pdds_gb300 import _capi as capi
from pdds_gb300.api import Estimate
from pdds_gb300.config import fac_rule
from pdds_gb300.output_files import KNOT_METADATA_COLUMNS, write_knot_metadata

SW, NE = (0.0, 0.0), (1.0, 1.0)


@pytest.fixture(scope="module")
def run():
    nsub, nnode, N, h = 3, 6, 300, 2e-3
    fac = fac_rule(1.0, nsub, nnode)
    L = O.Layout(SW, NE, nsub, nnode)
    prob = O.make_problem(O.POISSON_SINCOS)
    prm = O.make_params(N, h, seed=5, fac=fac, portable=True, sublinear=True)
    sel = np.arange(0, len(L.work_idx), 3)
    ref = L.run(prob, prm, knots=sel)
    rc, kn, sums = L.run_diag(prob, prm, knots=sel)
    return dict(N=N, h=h, ref=ref, rc=rc, kn=kn, sums=sums, L=L)


def test_diag_layout_matches_library_slots(run):
    assert O.DIAG_N == capi.DIAG_N == len(capi.DIAG_NAMES) == 18
    assert run["rc"] == 0 and run["ref"]["status"] == 0
    assert np.array_equal(run["kn"], run["ref"]["knots"])


def test_diag_counts(run):
    s, N, h, ref = run["sums"], run["N"], run["h"], run["ref"]
    ix = {n: i for i, n in enumerate(capi.DIAG_NAMES)}
    has = s[:, ix["paths"]] > 0
    assert np.all(s[has, ix["paths"]] == N)
    # the boundary-knot shortcut runs no paths: all sums zero
    assert np.all(s[~has] == 0.0)
    # both legs: 2 normals per step; tau = steps x h (no adaptive step)
    assert s[:, ix["rng"]].sum() == 2 * (ref["stats"][0] + ref["stats"][1])
    np.testing.assert_allclose(s[:, ix["tau"]].sum(), ref["stats"][0] * h, rtol=1e-12)
    np.testing.assert_allclose(s[:, ix["sub_tau"]].sum(), (ref["stats"][0] + ref["stats"][1]) * h, rtol=1e-12)
    assert np.all(s[has, ix["sub_tau"]] > s[has, ix["tau"]])  # the sublinear leg takes >= 1 step


def test_diag_identities(run):
    s = run["sums"]
    ix = {n: i for i, n in enumerate(capi.DIAG_NAMES)}
    for p in ("", "sub_"):
        sc, xi = s[:, ix[p + "score"]], s[:, ix[p + "xi"]]
        np.testing.assert_allclose(s[:, ix[p + "score_vr"]], sc + xi, rtol=1e-10, atol=1e-9)
        vr2 = s[:, ix[p + "score2"]] + 2 * s[:, ix[p + "xi_score"]] + s[:, ix[p + "xi2"]]
        np.testing.assert_allclose(s[:, ix[p + "score_vr2"]], vr2, rtol=1e-9, atol=1e-9)
        assert np.all(s[:, ix[p + "score2"]] >= 0) and np.all(s[:, ix[p + "xi2"]] >= 0)


def test_diag_linear_sums_from_the_path_records(run):
    """The linear-leg sums recomputed in numpy from the oracle's per-path
    exit records: phi = Z + Y u(X_tau) at the exit projection."""
    L, s, N, h = run["L"], run["sums"], run["N"], run["h"]
    ix = {n: i for i, n in enumerate(capi.DIAG_NAMES)}
    prob = O.make_problem(O.POISSON_SINCOS)
    prm = O.make_params(N, h, seed=5, fac=fac_rule(1.0, 3, 6), portable=True, sublinear=True)
    sel = np.arange(0, len(L.work_idx), 3)
    k = int(np.flatnonzero(s[:, ix["paths"]] > 0)[0])
    w = sel[k]
    rec = L.knot_paths(prob, prm, int(L.work_idx[w]), float(L.work_x[w]), float(L.work_y[w]))
    assert rec["status"] == 0
    phi = rec["Z"] + rec["Y"] * O.problem_u(prob, rec["x"], rec["y"])
    xi = rec["xi"]
    want = {"score": phi.sum(), "score2": (phi * phi).sum(), "xi": xi.sum(), "xi2": (xi * xi).sum(),
            "score_vr": (phi + xi).sum(), "score_vr2": ((phi + xi) ** 2).sum(), "xi_score": (xi * phi).sum(),
            "tau": rec["steps_l"].sum() * h}
    for name, v in want.items():
        assert s[k, ix[name]] == pytest.approx(v, rel=1e-9, abs=1e-9), name
    assert s[k, ix["rng"]] == 2 * (rec["steps_l"].sum() + rec["steps_s"].sum())


def test_knot_metadata_columns_and_file(tmp_path, run):
    K = len(run["kn"])
    est = Estimate(np.zeros(K + 1, np.int64), np.zeros(0, np.int64), np.zeros(0), np.zeros(0), np.zeros(K),
                   np.zeros(K), {}, np.full(K, run["N"]), run["sums"])
    md = est.knot_metadata()
    assert tuple(md) == KNOT_METADATA_COLUMNS
    ix = {n: i for i, n in enumerate(capi.DIAG_NAMES)}
    s = run["sums"]
    has = s[:, ix["paths"]] > 0
    m = s[has] / s[has, ix["paths"]][:, None]
    np.testing.assert_allclose(md["APL"][has], m[:, ix["tau"]])
    np.testing.assert_allclose(md["Var_Plain"][has], m[:, ix["score2"]] - m[:, ix["score"]] ** 2)
    np.testing.assert_allclose(md["Var_VR"][has], m[:, ix["score_vr2"]] - m[:, ix["score_vr"]] ** 2)
    assert np.all(np.abs(md["PCoeff_old"][has]) <= 1.0 + 1e-9)
    # the control variate removes most of the score's variance
    assert np.median(md["Var_VR"][has]) < np.median(md["Var_Plain"][has])
    write_knot_metadata(str(tmp_path), md)
    lines = open(os.path.join(tmp_path, "Output", "Debug", "knot_metadata.csv")).read().splitlines()
    assert lines[0] == ("index,APL,WCtime,RNGCalls,Estimated_Variance,Estimated_Variance_VR,PCoeff_old,"
                        "PCoeff_new,Var_Plain,Var_VR,bias_num,bias_trap")
    assert len(lines) == K + 1
    first = np.flatnonzero(has)[0]
    f = lines[1 + first].split(",")
    assert int(f[0]) == first and len(f) == 12
    assert float(f[1]) == pytest.approx(md["APL"][first], rel=1e-6)
    assert f[3] == "%e" % md["RNGCalls"][first]


def test_knot_metadata_needs_diagnostics():
    est = Estimate(np.zeros(2, np.int64), np.zeros(0, np.int64), np.zeros(0), np.zeros(0), np.zeros(1),
                   np.zeros(1))
    with pytest.raises(ValueError):
        est.knot_metadata()
