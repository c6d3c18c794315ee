"""Subdomain interior solves (the reference's Subdomain::Solve): with the
exact interface values the interior matches the analytic solution to the
second-order finite-difference error, which falls ~4x when the grid is
refined 2x; with the estimated interface solution the interior error is at
the interface error's level (check (c) of the path: the subdomain solution
against the analytic solution)."""
import numpy as np
import pytest

import pdds_gb300 as P
from pdds_gb300.config import fac_rule

pytestmark = pytest.mark.gpu

SW, NE = (-1.0, -1.0), (1.0, 1.0)


def interior_error(pd, bvp, m, u=None):
    x, y, v = pd.subdomain_solve(m, u)
    ns = pd.nsub
    err = 0.0
    for b in range(ns):
        for a in range(ns):
            X, Y = np.meshgrid(x[a], y[b])  # [j][i]
            err = max(err, float(np.max(np.abs(v[b, a] - bvp.u(X, Y)))))
    return err


@pytest.mark.parametrize("bvp", [P.BVP.poisson_sincos(), P.BVP.helmholtz(2.0, 1.5, -2.0)])
def test_exact_interface_data_give_second_order_interior(bvp):
    with P.PDDSparseGM(SW, NE, 4, 11, fac_rule(2.0, 4, 11)) as pd:
        pd.estimate(bvp, 64, 1e-3, mode=P.MODE_MIXED)  # sets the problem
        ex = bvp.u(pd.x, pd.y)
        e16 = interior_error(pd, bvp, 16, ex)
        e32 = interior_error(pd, bvp, 32, ex)
        assert e32 < 2e-4, e32
        assert 2.5 < e16 / e32 < 5.5, (e16, e32)


def test_estimated_interface_gives_interior_at_interface_accuracy():
    bvp = P.BVP.poisson_sincos()
    with P.PDDSparseGM(SW, NE, 4, 11, fac_rule(2.0, 4, 11)) as pd:
        pd.estimate(bvp, 10_000, 1e-3, mode=P.MODE_MIXED, adaptive_h=True, richardson=True)
        u, _ = pd.solve_interface()
        e_if = float(np.max(np.abs(u - bvp.u(pd.x, pd.y))))
        e_in = interior_error(pd, bvp, 32)
        assert e_in < 1e-2 and e_in < 2.0 * e_if + 2e-4, (e_in, e_if)
