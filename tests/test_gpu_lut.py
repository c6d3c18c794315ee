"""LUT-served coefficients (config 3's coefficient source).

The variable-coefficient problem is served from FP32 tables sampled with
bicubic Catmull-Rom interpolation.  Replay is bit-exact against the oracle's
FP64 restatement of the same sampler; MIXED with tables matches MIXED with the
analytic coefficients on the same random stream far inside the Monte Carlo
error (the 1024^2 tables interpolate the smooth coefficients to ~1e-9)."""
import numpy as np
import pytest

import oracle as O
import pdds_gb300 as P
from pdds_gb300.config import fac_rule, varcoef_tables

pytestmark = pytest.mark.gpu

SW, NE = (0.0, 0.0), (1.0, 1.0)


def test_lut_replay_bit_exact():
    nsub, nnode, N, h = 3, 6, 150, 5e-4
    fac = fac_rule(1.0, nsub, nnode)
    coef, g, b = varcoef_tables(48, (-0.1, -0.1, 1.1, 1.1))
    O.set_lut(coef, g, b)
    L = O.Layout(SW, NE, nsub, nnode)
    ip, _ = O.replay_ipsi(L, fac)
    with P.PDDSparseGM(SW, NE, nsub, nnode, fac) as pd:
        est = pd.estimate(P.BVP.lut(coef, g, b), N, h, mode=P.MODE_REPLAY_FP64, seed=17, want_var=True,
                          ipsi_override=ip)
    ref = L.run(O.make_problem(O.LUT), O.make_params(N, h, seed=17, fac=fac, portable=True))
    assert ref["status"] == 0
    for k, kn in enumerate(ref["knots"]):
        kn = int(kn)
        a, c = ref["row_ptr"][k], ref["row_ptr"][k + 1]
        r0, r1 = est.row_ptr[kn], est.row_ptr[kn + 1]
        assert np.array_equal(est.val[r0:r1], ref["g"][a:c]), kn
        assert np.array_equal(est.var[r0:r1], ref["gvar"][a:c]), kn
        assert est.B[kn] == ref["B"][k] and est.BB[kn] == ref["BB"][k], kn


def test_lut_matches_analytic_coefficients():
    nsub, nnode, N, h = 4, 9, 4000, 5e-4
    fac = fac_rule(1.0, nsub, nnode)
    with P.PDDSparseGM(SW, NE, nsub, nnode, fac) as pd:
        lut = pd.estimate(P.BVP.varcoef_lut(1024), N, h, mode=P.MODE_MIXED, seed=3, want_var=True)
        ana = pd.estimate(P.BVP.varcoef(), N, h, mode=P.MODE_MIXED, seed=3, want_var=True)
        u, _ = pd.solve_interface()
        ex = P.BVP.varcoef().u(pd.x, pd.y)
    se = np.sqrt(np.maximum(ana.var, 1e-12) / N)
    assert np.max(np.abs(lut.val - ana.val) / se) < 0.5
    var_b = ana.BB - ana.B ** 2
    mc = var_b > 1e-14  # knots with paths; boundary knots have B = g(x0) exactly
    se_b = np.sqrt(var_b[mc] / N)
    assert np.max(np.abs(lut.B - ana.B)[mc] / se_b) < 0.5
    # boundary values from the FP32 table: interpolation and FP32 rounding only
    assert np.max(np.abs(lut.B - ana.B)[~mc]) < 1e-6
    assert np.sqrt(np.mean((u - ex) ** 2)) < 5e-2
