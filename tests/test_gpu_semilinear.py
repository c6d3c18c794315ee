"""Table-served subdomain solves and the semilinear Newton loop (the
reference's Solve_SemiLin_numVR + Solve_Subdomains_SemiLin, main_VR.cpp).

* The table-served subdomain solver (variable sigma, drift and reaction,
  BiCGSTAB with a sine-transform preconditioner) against a direct sparse
  solve of the same finite-difference system with the analytic coefficients,
  and against the analytic solution (second-order error).
* The Newton loop on Lap u - u^3 + F = 0 (u = 1.1 + sin(pi x) sin(pi y)):
  the first step around the constant 1.1 is far off, the following steps
  approach the analytic solution at the interface knots and on the subdomain
  grids (check (c)).
* The fixed-point loop of main_LinLoop.cpp (Solve_Iterative_numVR,
  Salou_Iterative.hpp: Lap u + 20 u + F = 0 split with the shift 22, time
  rescale 9): on [0, 0.5]^2 the error's lowest mode shrinks by
  22 / (8 pi^2 + 2) = 0.27 per step, so the loop reaches the Monte Carlo floor
  in a few steps."""
import numpy as np
import pytest

import pdds_gb300 as P
from pdds_gb300.config import fac_rule

pytestmark = pytest.mark.gpu

SW, NE = (0.0, 0.0), (1.0, 1.0)


def varcoef_fd_reference(x0, y0, lx, ly, m, g):
    """Direct solve of the central-difference system of the variable-coefficient
    problem on one subdomain with Dirichlet data g(x, y) (scipy sparse LU)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    hx, hy = lx / (m + 1), ly / (m + 1)
    xs = x0 + hx * np.arange(m + 2)
    ys = y0 + hy * np.arange(m + 2)
    n = m * m
    rows, cols, vals = [], [], []
    rhs = np.zeros(n)
    for j in range(m):
        for i in range(m):
            X, Y = xs[i + 1], ys[j + 1]
            s1, s2 = 1.0 + 0.5 * X * X, 1.0 + 0.5 * Y * Y
            ax, ay, bx, by, c = 0.5 * s1 * s1, 0.5 * s2 * s2, Y, -X, -(1.0 + X * X + Y * Y)
            ux = np.exp(X) * np.cos(2 * Y)
            uy = -2.0 * np.exp(X) * np.sin(2 * Y)
            f = -(0.5 * (s1 * s1 * ux + s2 * s2 * (-4.0 * ux)) + (Y * ux - X * uy) + c * (ux + 1.0))
            e = j * m + i
            rhs[e] = f
            rows.append(e); cols.append(e); vals.append(2 * ax / hx ** 2 + 2 * ay / hy ** 2 - c)
            for di, dj, w in ((1, 0, ax / hx ** 2 + bx / (2 * hx)), (-1, 0, ax / hx ** 2 - bx / (2 * hx)),
                              (0, 1, ay / hy ** 2 + by / (2 * hy)), (0, -1, ay / hy ** 2 - by / (2 * hy))):
                ii, jj = i + di, j + dj
                if 0 <= ii < m and 0 <= jj < m:
                    rows.append(e); cols.append(jj * m + ii); vals.append(-w)
                else:
                    rhs[e] += w * g(xs[ii + 1], ys[jj + 1])
    A = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    return spl.spsolve(A.tocsc(), rhs).reshape(m, m)


def test_table_served_subdomains_match_direct_solve_and_analytic():
    pytest.importorskip("scipy")
    bvp = P.BVP.varcoef_lut(512, (0.0, 0.0, 1.0, 1.0))
    ns, m = 4, 23
    with P.PDDSparseGM(SW, NE, ns, 11, fac_rule(1.0, ns, 11)) as pd:
        pd.estimate(bvp, 64, 1e-3, mode=P.MODE_MIXED)  # uploads the tables, sets the problem
        ex = bvp.u(pd.x, pd.y)
        x, y, v = pd.subdomain_solve(m, ex)
        x2, y2, v2 = pd.subdomain_solve(m, ex)  # scratch reused: the same result
        assert np.array_equal(v, v2)
        lx = 1.0 / ns
        worst_ref = worst_exact = 0.0
        for b in (0, 2, 3):
            for a in (0, 1, 3):
                ref = varcoef_fd_reference(a * lx, b * lx, lx, lx, m, lambda X, Y: bvp.u(X, Y))
                worst_ref = max(worst_ref, float(np.max(np.abs(v[b, a] - ref))))
                X, Y = np.meshgrid(x[a], y[b])
                worst_exact = max(worst_exact, float(np.max(np.abs(v[b, a] - bvp.u(X, Y)))))
        # differences from the direct solve: table interpolation of the
        # coefficients (FP32 tables, 512^2) and the edges' cubic interpolation
        assert worst_ref < 2e-5, worst_ref
        assert worst_exact < 5e-4, worst_exact


def test_semilinear_newton_loop_approaches_the_analytic_solution():
    with P.PDDSparseGM(SW, NE, 4, 11, fac_rule(1.0, 4, 11)) as pd:
        its = pd.solve_semilinear(4, 20000, 5e-4, m=24, seed=7, adaptive_h=True, richardson=True, dup_sum=True)
    knots = [it["rmse_knots"] for it in its]
    grid = [it["rmse_grid"] for it in its]
    # the step around the constant 1.1 misses the sin(pi x) sin(pi y) part
    assert knots[0] > 2e-2, knots
    assert knots[-1] < 4e-3 and grid[-1] < 4e-3, (knots, grid)
    assert knots[-1] < 0.2 * knots[0] and knots[2] < knots[0], knots
    for it in its:
        assert it["solve"]["rel_residual"] < 1e-10


def test_linear_fixed_point_loop_contracts_to_the_analytic_solution():
    sw, ne = (0.0, 0.0), (0.5, 0.5)
    with P.PDDSparseGM(sw, ne, 4, 11, fac_rule(0.5, 4, 11)) as pd:
        its = pd.solve_linear_iteration(4, 20000, 5e-4, m=24, seed=11, adaptive_h=True, richardson=True,
                                        dup_sum=True)
    knots = [it["rmse_knots"] for it in its]
    grid = [it["rmse_grid"] for it in its]
    print("linear loop rmse knots", knots, "grid", grid)
    for it in its:
        assert it["solve"]["rel_residual"] < 1e-10
    # the first step (u_k = 0) misses the alpha u part of the source: the
    # same loop on a 97^2 finite-difference grid without Monte Carlo error
    # gives RMSE 4.5e-2, 5.4e-3, 9.1e-4, 2.8e-4 over the four steps
    assert knots[0] > 2e-2, knots
    # contraction down to the Monte Carlo floor (about 1e-3 here)
    assert knots[1] < 0.25 * knots[0] and knots[2] < 0.7 * knots[1], knots
    assert knots[-1] < 2.5e-3 and grid[-1] < 2.5e-3, (knots, grid)
