"""Circle layout on the GPU (MIXED, polar stencils): the interface solution
approaches u = r^2 sin(3 theta) + cos x, the boundary knots hold g, the
Richardson pair removes most of the bias, and the variance-adaptive paths
spread the path counts."""
import numpy as np
import pytest

import pdds_gb300 as P

pytestmark = pytest.mark.gpu


def rmse(a, b):
    return float(np.sqrt(np.mean((a - b) ** 2)))


def test_circle_solution_close_to_analytic():
    bvp = P.BVP.circle_poisson()
    with P.PDDSparseGM.circle_mesh(1.0, 6, 16, 11) as pd:
        ex = bvp.u(pd.x, pd.y)
        plain = pd.estimate(bvp, 4000, 1e-3, mode=P.MODE_MIXED, seed=3, adaptive_h=True)
        bnd = np.abs(np.hypot(pd.x, pd.y) - 1.0) < 1e-12
        assert np.max(np.abs(plain.B[bnd] - ex[bnd])) < 1e-12
        u_plain, info = pd.solve_interface()
        assert info["rel_residual"] <= 1e-10
        rich = pd.estimate(bvp, 4000, 1e-3, mode=P.MODE_MIXED, seed=3, adaptive_h=True, richardson=True)
        u_rich, _ = pd.solve_interface()
        e_plain, e_rich = rmse(u_plain, ex), rmse(u_rich, ex)
        assert e_rich < 5e-3, e_rich
        assert e_rich < e_plain, (e_rich, e_plain)


def test_circle_adaptive_paths():
    bvp = P.BVP.circle_poisson()
    with P.PDDSparseGM.circle_mesh(1.0, 6, 16, 11) as pd:
        est = pd.estimate(bvp, 1000, 1e-3, mode=P.MODE_MIXED, seed=5, adaptive_h=True, adaptive_n=True,
                          npaths_max=100_000, target_stderr=1e-2)
        n = est.npaths[est.npaths > 0]
        assert n.min() >= 1000 and n.max() <= 100_000 and len(np.unique(n)) > 3
        u, _ = pd.solve_interface()
        assert rmse(u, bvp.u(pd.x, pd.y)) < 5e-2


def test_circle_mixed_matches_fp64_on_the_same_stream():
    """The FP32 polar kernel against the all-FP64 polar kernel on the same
    Philox streams: G and B agree far inside the Monte Carlo error."""
    bvp = P.BVP.circle_poisson()
    N = 3000
    with P.PDDSparseGM.circle_mesh(1.0, 6, 16, 11) as pd:
        m = pd.estimate(bvp, N, 1e-3, mode=P.MODE_MIXED, seed=8, adaptive_h=True, want_var=True)
        f = pd.estimate(bvp, N, 1e-3, mode=P.MODE_FP64, seed=8, adaptive_h=True)
    se_g = np.sqrt(np.maximum(m.var, 1e-12) / N)
    assert np.max(np.abs(m.val - f.val) / se_g) < 0.5
    se_b = np.sqrt(np.maximum(m.BB - m.B ** 2, 1e-16) / N)
    assert np.max(np.abs(m.B - f.B) / se_b) < 0.5
    assert abs(m.info["path_steps"] - f.info["path_steps"]) < 1e-3 * f.info["path_steps"]
