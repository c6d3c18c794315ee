"""The reference's on-disk outputs from a GPU solve: Solve(trace_dir=...)
writes the phase trace Output/Debug/times.txt and the solution and system
files; an estimate with diagnostics writes Output/Debug/knot_metadata.csv."""
import numpy as np
import pytest

import pdds_gb300 as P
from pdds_gb300.config import fac_rule
from pdds_gb300.output_files import TimeFile, read_triplets, write_knot_metadata

pytestmark = pytest.mark.gpu


def test_solve_writes_the_reference_files(tmp_path):
    nsub, nnode = 3, 7
    with P.PDDSparseGM((-1.0, -1.0), (1.0, 1.0), nsub, nnode, fac_rule(2.0, nsub, nnode)) as pd:
        u, est, _ = pd.Solve(P.BVP.poisson_sincos(), 2000, 1e-3, adaptive_h=True, richardson=True,
                             trace_dir=str(tmp_path), diagnostics=True)
        write_knot_metadata(str(tmp_path), est.knot_metadata())
        K = pd.K
    dbg = tmp_path / "Output" / "Debug"
    times = open(dbg / "times.txt").read().splitlines()
    assert times[0] == TimeFile.HEADER
    assert [ln.split(",")[0] for ln in times[1:]] == ["MC Simulations", "Solving system", "Writing Solution"]
    sol = open(tmp_path / "Output" / "solution.csv").read().splitlines()
    assert len(sol) == K + 1
    got = np.array([float(ln.split(",")[4]) for ln in sol[1:]])
    np.testing.assert_allclose(got, u, rtol=1e-6, atol=1e-6)  # %e keeps 7 digits
    rows, cols, vals = read_triplets(str(dbg / "B.csv"))
    assert len(vals) == K
    meta = open(dbg / "knot_metadata.csv").read().splitlines()
    assert len(meta) == K + 1 and meta[0].startswith("index,APL,")
