"""The index-checked build (pdds_gb300.build.build(checked=True),
-DPDDS_CHECKED): every checked device index -- exit-histogram deposits, the
warps' exit queues, G row positions, the interface solvers' column gathers
-- is tested against its array before the access, and a failure returns
PDDS_ERR_BOUNDS instead of touching memory.  Every mode and solver runs
through that build here, in a process of its own (a process loads one
library), and must finish with no failed check."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r'''
import sys
sys.path.insert(0, ROOT)
import numpy as np
from pdds_gb300 import _capi as capi, build as B
capi.load(B.LIB_CHECKED)
import pdds_gb300 as P
from pdds_gb300.config import fac_rule, batch_instances, varcoef_tables

sw, ne = (-1.0, -1.0), (1.0, 1.0)
with P.PDDSparseGM(sw, ne, 4, 11, fac_rule(2.0, 4, 11)) as pd:
    bvp = P.BVP.poisson_sincos()
    pd.estimate(bvp, 300, 1e-3, mode=P.MODE_REPLAY_FP64, diagnostics=True)
    pd.estimate(bvp, 2000, 1e-3, mode=P.MODE_FP64, richardson=True, adaptive_h=True, diagnostics=True)
    pd.estimate(bvp, 4000, 1e-3, mode=P.MODE_MIXED, richardson=True, adaptive_h=True, want_var=True,
                dup_sum=True, diagnostics=True)
    pd.solve_interface(P.SOLVE_GMRES_FP32_IR)
    pd.solve_interface(P.SOLVE_BICGSTAB_FP64)
    pd.subdomain_solve(16)
with P.PDDSparseGM(sw, ne, 12, 21, fac_rule(2.0, 12, 21)) as pd:  # whole-GPU GMRES
    pd.estimate(P.BVP.poisson_sincos(), 512, 1e-3, mode=P.MODE_MIXED, richardson=True)
    pd.solve_interface(P.SOLVE_GMRES_FP32_IR)
    pd.solve_interface(P.SOLVE_GMRES_FP32_IR, gmres_form=capi.GMRES_CLASSICAL)
coef, g, b = varcoef_tables(128, (0.0, 0.0, 1.0, 1.0))
with P.PDDSparseGM((0.0, 0.0), (1.0, 1.0), 4, 9, fac_rule(1.0, 4, 9)) as pd:
    for samp in P.BVP.SAMPLERS:
        pd.estimate(P.BVP.lut(coef, g, b, sampler=samp), 2000, 5e-4, mode=P.MODE_MIXED, richardson=True)
    pd.solve_interface()
with P.PDDSparseGM.circle_mesh(1.0, 3, 8, 5) as pc:
    pc.estimate(P.BVP.circle_poisson(), 2000, 1e-3, mode=P.MODE_MIXED, richardson=True, adaptive_h=True)
    pc.estimate(P.BVP.circle_poisson(), 500, 1e-3, mode=P.MODE_FP64)
    pc.solve_interface()
with P.PDDSparseGM((0.0, 0.0), (1.0, 1.0), 4, 9, fac_rule(1.0, 4, 9)) as pd:
    pd.estimate(P.BVP.robin_poisson("W"), 2000, 1e-3, mode=P.MODE_MIXED, richardson=True)
with P.Batch(P.BVP.HELMHOLTZ, batch_instances(8, seed=3, grid=(4, 8), nodes=(11, 17), scaled_h=1e-3)) as bt:
    info = bt.run(1000, 1e-3, richardson=True, use_graph=True)
    assert info["unconverged"] == 0
print("CHECKED-OK")
'''


def test_checked_build_runs_every_path_without_a_failed_check():
    from pdds_gb300 import build as B
    B.build(checked=True)
    r = subprocess.run([sys.executable, "-c", SCRIPT.replace("ROOT", repr(ROOT))], cwd=ROOT,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0 and "CHECKED-OK" in r.stdout, r.stdout[-2000:] + r.stderr[-4000:]
