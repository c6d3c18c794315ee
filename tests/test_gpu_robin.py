"""Robin boundary with reflected paths (the reference's Lepingle step,
FKACIntegrator.hpp:116-165, and the Robin problem BVPs/EDPs/poisson_3.hpp).

On the Robin side paths reflect (Lepingle's step, the bridge maximum of the
normal component) and carry the local-time terms dZ = psi Y dL,
dY = varphi Y dL; knots on that side keep B = g as in the reference's
boundary shortcut.  Checks: the interface solution against the analytic one
with the Robin side (check (c)); the reflection is active (B differs from
the all-Dirichlet problem by many standard errors); MIXED agrees with the
FP64 form on the same random streams; the modes without a reflected form
refuse the problem."""
import numpy as np
import pytest

import pdds_gb300 as P
from pdds_gb300.config import fac_rule

pytestmark = pytest.mark.gpu

SW, NE = (-1.0, -1.0), (1.0, 1.0)
OPTS = dict(adaptive_h=True, richardson=True, dup_sum=True)


def test_robin_side_solution_against_analytic_and_dirichlet():
    N, h = 20000, 1e-3
    with P.PDDSparseGM(SW, NE, 4, 11, fac_rule(2.0, 4, 11)) as pd:
        near = pd.x < -0.5 + 1e-9  # knots of the subdomain column on the Robin side
        out = {}
        for side in ("W", None):
            bvp = P.BVP.robin_poisson(side)
            est = pd.estimate(bvp, N, h, mode=P.MODE_MIXED, seed=3, **OPTS)
            u, si = pd.solve_interface()
            assert si["rel_residual"] < 1e-10
            err = u - bvp.u(pd.x, pd.y)
            out[side] = (est, float(np.sqrt(np.mean(err ** 2))), float(np.sqrt(np.mean(err[near] ** 2))))
    (ew, rw, rw_near), (ed, rd, rd_near) = out["W"], out[None]
    # the Robin side is as accurate as the Dirichlet one (exact local-time terms)
    assert rw < 2e-3 and rw_near < 2e-3, (rw, rw_near)
    assert rd < 2e-3, rd
    # and the reflection is active: B of knots whose stencils touch it changes
    se = np.sqrt(np.maximum(ed.BB - ed.B ** 2, 0.0) / N) + 1e-12
    assert np.max(np.abs(ew.B - ed.B) / se) > 20.0


def test_robin_mixed_matches_fp64_on_the_same_stream():
    N, h = 2000, 1e-3
    bvp = P.BVP.robin_poisson("W")
    with P.PDDSparseGM(SW, NE, 4, 11, fac_rule(2.0, 4, 11)) as pd:
        f = pd.estimate(bvp, N, h, mode=P.MODE_FP64, seed=5, **OPTS)
        m = pd.estimate(bvp, N, h, mode=P.MODE_MIXED, seed=5, want_var=True, **OPTS)
    se = np.sqrt(np.maximum(m.var, 0.0) / N) + 1e-12
    seb = np.sqrt(np.maximum(m.BB - m.B ** 2, 0.0) / N) + 1e-12
    # FP32 and FP64 paths on the same Philox streams: differences are a small
    # fraction of the Monte Carlo standard error (a reflection decision can
    # flip at the FP32 rounding level)
    assert np.max(np.abs(m.val - f.val) / se) < 1.0
    assert np.max(np.abs(m.B - f.B) / seb) < 0.5
    assert abs(m.info["path_steps"] - f.info["path_steps"]) < 1e-3 * f.info["path_steps"]


def test_robin_problem_refuses_forms_without_reflection():
    with P.PDDSparseGM(SW, NE, 4, 11, fac_rule(2.0, 4, 11)) as pd:
        with pytest.raises(P.PDDSError):
            pd.estimate(P.BVP.robin_poisson("W"), 64, 1e-3, mode=P.MODE_REPLAY_FP64)
        with pytest.raises(P.PDDSError):
            pd.estimate(P.BVP(P.BVP.ROBIN_POISSON, (3.0,)), 64, 1e-3, mode=P.MODE_MIXED)
