"""Interface solve forms on the GPU: the pipelined GMRES (one group barrier
per Arnoldi step, G V kept beside the basis) and the classical two-barrier
step reach the same FP64-refined solution, on a system solved by one thread
block cluster (4 x 4 subdomains, 11 knots) and on one solved over the whole
GPU (12 x 12 subdomains, 43 knots: 10,989 knots, the benchmark's system);
both agree with the FP64 BiCGSTAB of the reference's method."""
import numpy as np
import pytest

import pdds_gb300 as P
from pdds_gb300 import _capi as capi
from pdds_gb300.config import fac_rule

pytestmark = pytest.mark.gpu

SW, NE = (-1.0, -1.0), (1.0, 1.0)


@pytest.mark.parametrize("nsub,nnode,N,h", [(4, 11, 2000, 1e-3), (12, 43, 512, 5e-4)])
def test_pipelined_and_classical_gmres_agree(nsub, nnode, N, h):
    fac = fac_rule(2.0, nsub, nnode)
    with P.PDDSparseGM(SW, NE, nsub, nnode, fac) as pd:
        pd.estimate(P.BVP.poisson_sincos(), N, h, mode=P.MODE_MIXED, seed=17, adaptive_h=True, richardson=True,
                    dup_sum=True)
        up, ip = pd.solve_interface(P.SOLVE_GMRES_FP32_IR, tol=1e-10, gmres_form=capi.GMRES_PIPELINED)
        uc, ic = pd.solve_interface(P.SOLVE_GMRES_FP32_IR, tol=1e-10, gmres_form=capi.GMRES_CLASSICAL)
        ub, ib = pd.solve_interface(P.SOLVE_BICGSTAB_FP64, tol=1e-12)
    assert ip["rel_residual"] <= 1e-10 and ic["rel_residual"] <= 1e-10
    scale = np.max(np.abs(ub))
    np.testing.assert_allclose(up, ub, rtol=0, atol=1e-8 * scale)
    np.testing.assert_allclose(uc, ub, rtol=0, atol=1e-8 * scale)
    # the pipelined recurrence may cost a few more inner steps, not many
    assert ip["iterations"] <= 1.5 * ic["iterations"] + 10, (ip, ic)
