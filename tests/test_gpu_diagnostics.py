"""The reduction's per-knot diagnostic sums on the GPU (Reduce_Analytic's
sums[], Solvers/EMFKACSolver.hpp:14-47, 542-558; pdds_estimate_diagnostics).

The replay mode sums the same paths in the same order as the oracle and must
match it bit for bit, both legs; the FP64 and MIXED forms (linear leg only)
must agree with it within Monte Carlo error and count exactly."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
import pdds_gb300 as P
from pdds_gb300 import _capi as capi
from pdds_gb300.config import fac_rule, varcoef_tables

pytestmark = pytest.mark.gpu

IX = {n: i for i, n in enumerate(capi.DIAG_NAMES)}


def _replay_vs_oracle(SW, NE, nsub, nnode, N, h, bvp, prob, seed):
    fac = fac_rule(NE[0] - SW[0], nsub, nnode)
    L = O.Layout(SW, NE, nsub, nnode)
    ip, _ = O.replay_ipsi(L, fac)
    with P.PDDSparseGM(SW, NE, nsub, nnode, fac) as pd:
        est = pd.estimate(bvp, N, h, mode=P.MODE_REPLAY_FP64, seed=seed, ipsi_override=ip, diagnostics=True)
    rc, kn, sums = L.run_diag(prob, O.make_params(N, h, seed=seed, fac=fac, portable=True, sublinear=True))
    assert rc == 0
    return est, kn, sums


def test_replay_diagnostics_bit_exact_poisson():
    est, kn, sums = _replay_vs_oracle((-1.0, -1.0), (1.0, 1.0), 4, 11, 300, 1e-3, P.BVP.poisson_sincos(),
                                      O.make_problem(O.POISSON_SINCOS), 21)
    assert np.array_equal(est.diag[kn], sums)
    assert np.all(est.diag[kn][:, IX["paths"]][sums[:, IX["paths"]] > 0] == 300)


def test_replay_diagnostics_bit_exact_lut():
    coef, g, b = varcoef_tables(48, (-0.1, -0.1, 1.1, 1.1))
    O.set_lut(coef, g, b)
    est, kn, sums = _replay_vs_oracle((0.0, 0.0), (1.0, 1.0), 3, 6, 150, 5e-4, P.BVP.lut(coef, g, b),
                                      O.make_problem(O.LUT), 17)
    assert np.array_equal(est.diag[kn], sums)


@pytest.mark.parametrize("mode", [P.MODE_FP64, P.MODE_MIXED])
def test_fp64_and_mixed_diagnostics_agree_with_replay(mode):
    SW, NE, nsub, nnode, N, h = (-1.0, -1.0), (1.0, 1.0), 3, 7, 4000, 1e-3
    fac = fac_rule(2.0, nsub, nnode)
    bvp = P.BVP.poisson_sincos()
    with P.PDDSparseGM(SW, NE, nsub, nnode, fac) as pd:
        ref = pd.estimate(bvp, N, h, mode=P.MODE_REPLAY_FP64, seed=8, diagnostics=True)
        est = pd.estimate(bvp, N, h, mode=mode, seed=8, diagnostics=True)
        steps = est.info["path_steps"]
    r, e = ref.diag, est.diag
    has = r[:, IX["paths"]] > 0
    assert np.array_equal(has, e[:, IX["paths"]] > 0)
    assert np.all(e[has, IX["paths"]] == N)
    # normals: 2 per step of the linear leg; its sums fill the sublinear slots
    assert e[:, IX["rng"]].sum() == 2 * steps
    for q in range(8):
        assert np.array_equal(e[:, q], e[:, 8 + q])
    # moments of the two forms within Monte Carlo error of each other
    m_r, m_e = r[has] / N, e[has] / N
    for name, sq in (("score", "score2"), ("score_vr", "score_vr2"), ("xi", "xi2")):
        var = np.maximum(m_r[:, IX[sq]] - m_r[:, IX[name]] ** 2, 1e-12)
        z = (m_e[:, IX[name]] - m_r[:, IX[name]]) / np.sqrt(2 * var / N)
        assert np.sqrt(np.mean(z ** 2)) < 1.6, name
        assert np.max(np.abs(z)) < 5.0, name
    # mean exit time: the Gobet-shifted rule in both forms
    np.testing.assert_allclose(m_e[:, IX["tau"]].mean(), m_r[:, IX["tau"]].mean(), rtol=0.03)


def test_mixed_richardson_diagnostics_and_metadata(tmp_path):
    SW, NE, nsub, nnode, N, h = (-1.0, -1.0), (1.0, 1.0), 3, 7, 2048, 1e-3
    fac = fac_rule(2.0, nsub, nnode)
    with P.PDDSparseGM(SW, NE, nsub, nnode, fac) as pd:
        est = pd.estimate(P.BVP.poisson_sincos(), N, h, mode=P.MODE_MIXED, seed=4, richardson=True,
                          adaptive_h=True, diagnostics=True)
    s = est.diag
    has = s[:, IX["paths"]] > 0
    assert np.all(s[has, IX["paths"]] == N)
    assert np.all(np.isfinite(s))
    md = est.knot_metadata()
    assert np.all(md["APL"][has] > 0)
    assert np.all(md["Var_VR"][has] >= 0)
    assert np.median(md["Var_VR"][has]) < np.median(md["Var_Plain"][has])
    from pdds_gb300.output_files import write_knot_metadata
    write_knot_metadata(str(tmp_path), md)
    assert len(open(tmp_path / "Output" / "Debug" / "knot_metadata.csv").read().splitlines()) == pd.K + 1


def test_per_knot_solver_diagnostics_match_the_layout_run():
    SW, NE, nsub, nnode, N, h = (-1.0, -1.0), (1.0, 1.0), 3, 7, 500, 1e-3
    fac = fac_rule(2.0, nsub, nnode)
    bvp = P.BVP.poisson_sincos()
    with P.PDDSparseGM(SW, NE, nsub, nnode, fac) as pd:
        est = pd.estimate(bvp, N, h, mode=P.MODE_REPLAY_FP64, seed=6, diagnostics=True)
        k = int(np.flatnonzero(est.diag[:, IX["paths"]] > 0)[3])
        st = P.Stencil.of_knot(pd, k)
        with P.EMFKACSolver() as sv:
            sv.Solve_GPU_Analytic((pd.x[k], pd.y[k]), N, h, 0.0, bvp, st, mode=P.MODE_REPLAY_FP64, seed=6,
                                  knot_id=k, diagnostics=True)
            assert np.array_equal(sv.sums, est.diag[k])


def test_diagnostics_errors():
    with P.PDDSparseGM((-1.0, -1.0), (1.0, 1.0), 3, 7, fac_rule(2.0, 3, 7)) as pd:
        pd.estimate(P.BVP.poisson_sincos(), 256, 1e-3, mode=P.MODE_MIXED)
        buf = np.zeros(pd.K * capi.DIAG_N)
        with pytest.raises(P.PDDSError) as e:  # the last estimate ran without diagnostics
            pd._check(pd._lib.pdds_estimate_diagnostics(pd._ctx, buf.ctypes.data_as(C.POINTER(C.c_double))))
        assert e.value.status == capi.ERR_INVALID
        with pytest.raises(P.PDDSError) as e:
            pd.estimate(P.BVP.poisson_sincos(), 256, 1e-3, mode=P.MODE_MIXED, adaptive_n=True, npaths_max=1024,
                        target_stderr=1e-3, diagnostics=True)
        assert e.value.status == capi.ERR_INVALID
    with P.PDDSparseGM.circle_mesh(nrings=3, nsectors=8, nnode=5) as pc:
        with pytest.raises(P.PDDSError) as e:
            pc.estimate(P.BVP.circle_poisson(), 256, 1e-3, mode=P.MODE_MIXED, diagnostics=True)
        assert e.value.status == capi.ERR_INVALID
        est = pc.estimate(P.BVP.circle_poisson(), 256, 1e-3, mode=P.MODE_FP64, diagnostics=True)
        assert np.all(est.diag[est.diag[:, IX["paths"]] > 0, IX["paths"]] == 256)
