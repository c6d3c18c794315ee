"""LUT-served coefficients (the table-served variable-coefficient workload's coefficient source).

The variable-coefficient problem is served from FP32 tables.  The FP64 and
replay forms sample them with bicubic Catmull-Rom interpolation: replay is
bit-exact against the oracle's FP64 restatement of the same sampler.  MIXED
samples the interpolating cubic B-spline from textures (or, on request, the
same Catmull-Rom nodes); with either sampler it matches MIXED with the
analytic coefficients on the same random stream far inside the Monte Carlo
error (the 1024^2 tables interpolate the smooth coefficients to ~1e-9; the
texture blend's 8-bit fractions add ~1e-6)."""
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


@pytest.mark.parametrize("sampler", P.BVP.SAMPLERS)
def test_lut_matches_analytic_coefficients(sampler):
    nsub, nnode, N, h = 4, 9, 4000, 5e-4
    fac = fac_rule(1.0, nsub, nnode)
    with P.PDDSparseGM(SW, NE, nsub, nnode, fac) as pd:
        lut = pd.estimate(P.BVP.varcoef_lut(1024, sampler=sampler), N, h, mode=P.MODE_MIXED, seed=3,
                          want_var=True)
        ana = pd.estimate(P.BVP.varcoef(), N, h, mode=P.MODE_MIXED, seed=3, want_var=True)
        u, _ = pd.solve_interface()
        ex = P.BVP.varcoef().u(pd.x, pd.y)
    se = np.sqrt(np.maximum(ana.var, 1e-12) / N)
    z = np.abs(lut.val - ana.val) / se
    var_b = ana.BB - ana.B ** 2
    mc = var_b > 1e-14  # knots with paths; boundary knots have B = g(x0) exactly
    se_b = np.sqrt(var_b[mc] / N)
    zb = np.abs(lut.B - ana.B)[mc] / se_b
    # the same streams: almost every path takes the same steps, and the few
    # that cross an exit threshold differently move one entry by a fraction
    # of its error; the texture samplers' 8-bit blend fractions flip a few
    # more paths than the node sampler's FP32 rounding
    lim = 0.5 if sampler == "catmull_rom" else 1.5
    assert z.max() < lim and zb.max() < lim
    assert np.sqrt(np.mean(z ** 2)) < 0.05 and np.sqrt(np.mean(zb ** 2)) < 0.05
    # boundary values from the FP32 table: interpolation and FP32 rounding only
    assert np.max(np.abs(lut.B - ana.B)[~mc]) < 1e-6
    assert np.sqrt(np.mean((u - ex) ** 2)) < 5e-2


def test_lut_samplers_agree_on_coarse_tables():
    """On 64^2 tables the two interpolants differ by their interpolation
    error (Catmull-Rom O(dx^3), the B-spline O(dx^4)): both MIXED estimates
    stay within the Monte Carlo error of each other and of the FP64 form."""
    nsub, nnode, N, h = 3, 7, 6000, 5e-4
    fac = fac_rule(1.0, nsub, nnode)
    bs = P.BVP.varcoef_lut(64, (-0.1, -0.1, 1.1, 1.1))
    cr = P.BVP(P.BVP.LUT, (1.0,), tables=bs.tables, exact=bs.exact)
    with P.PDDSparseGM(SW, NE, nsub, nnode, fac) as pd:
        a = pd.estimate(bs, N, h, mode=P.MODE_MIXED, seed=11, want_var=True)
        ua, _ = pd.solve_interface()
        b = pd.estimate(cr, N, h, mode=P.MODE_MIXED, seed=11, want_var=True)
        ub, _ = pd.solve_interface()
        ex = bs.u(pd.x, pd.y)
    se = np.sqrt(np.maximum(a.var, 1e-12) / N)
    z = np.abs(a.val - b.val) / se
    mc = (a.BB - a.B ** 2) > 1e-14
    se_b = np.sqrt((a.BB - a.B ** 2)[mc] / N)
    zb = np.abs(a.B - b.B)[mc] / se_b
    assert z.max() < 2.0 and zb.max() < 2.0
    assert np.sqrt(np.mean(z ** 2)) < 0.1 and np.sqrt(np.mean(zb ** 2)) < 0.1
    ra, rb = np.sqrt(np.mean((ua - ex) ** 2)), np.sqrt(np.mean((ub - ex) ** 2))
    assert ra < 5e-2 and rb < 5e-2
    assert abs(ra - rb) < 0.25 * max(ra, rb) + 1e-3


def test_lut_bilinear_texture_on_fine_tables():
    """Bilinear interpolation of 1024^2 tables (error ~1e-6 on these smooth
    coefficients) matches the Catmull-Rom node sampler on the same random
    stream far inside the Monte Carlo error."""
    nsub, nnode, N, h = 4, 9, 4000, 5e-4
    fac = fac_rule(1.0, nsub, nnode)
    bl = P.BVP.varcoef_lut(1024, sampler="bilinear")
    cr = P.BVP(P.BVP.LUT, (1.0,), tables=bl.tables, exact=bl.exact)
    with P.PDDSparseGM(SW, NE, nsub, nnode, fac) as pd:
        a = pd.estimate(bl, N, h, mode=P.MODE_MIXED, seed=5, want_var=True)
        b = pd.estimate(cr, N, h, mode=P.MODE_MIXED, seed=5, want_var=True)
        u, _ = pd.solve_interface()
        ex = bl.u(pd.x, pd.y)
    se = np.sqrt(np.maximum(b.var, 1e-12) / N)
    z = np.abs(a.val - b.val) / se
    mc = (b.BB - b.B ** 2) > 1e-14
    se_b = np.sqrt((b.BB - b.B ** 2)[mc] / N)
    zb = np.abs(a.B - b.B)[mc] / se_b
    assert z.max() < 1.5 and zb.max() < 1.5
    assert np.sqrt(np.mean(z ** 2)) < 0.05 and np.sqrt(np.mean(zb ** 2)) < 0.05
    assert np.sqrt(np.mean((u - ex) ** 2)) < 5e-2
