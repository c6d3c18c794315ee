"""The reference's output files (Output/solution.csv, Output/Debug/*.csv) are
written in its own format and entry order: writing the reference's recorded
run (tests/golden) through pdds_gb300.output_files on this library's layout
of the same configuration reproduces the recorded files entry for entry."""
import ctypes as C
import os

import numpy as np

from pdds_gb300 import _capi as capi
from pdds_gb300.output_files import read_triplets, write_outputs

from test_capi_cpu import HostLayout, lib  # noqa: F401  (module fixture)

HERE = os.path.dirname(os.path.abspath(__file__))


def test_outputs_match_the_recorded_files(lib, tmp_path):
    ref = np.load(os.path.join(HERE, "golden", "ref_run_4x4_n8_monegros.npz"))
    cfg = ref["config"]
    h = HostLayout(lib, (cfg[0], cfg[1]), (cfg[2], cfg[3]), int(cfg[4]), int(cfg[5]), tuple(cfg[8:12]))
    K = h.info.nknots
    nnz = h.info.nnz
    rp, col = h.rp, h.col[:nnz]
    rows = np.repeat(np.arange(K), np.diff(rp))
    # the recorded G_var and I+G values placed at this layout's CSR positions
    pos = {(int(i), int(j)): e for e, (i, j) in enumerate(zip(rows, col))}
    gv = np.zeros(nnz)
    for i, j, v in ref["G_var"]:
        gv[pos[(int(i), int(j))]] = v
    g = np.zeros(nnz)
    for i, j, v in ref["G"]:
        if (int(i), int(j)) in pos:
            g[pos[(int(i), int(j))]] = v - (1.0 if i == j else 0.0)
    B = ref["B"][:, 2]
    BB = B * B - ref["B_var"][:, 2]
    sol = ref["solution"]
    write_outputs(str(tmp_path), sol[:, 1], sol[:, 2], rp, col, g, gv, B, BB, sol[:, 4], sol[:, 3])
    dbg = os.path.join(str(tmp_path), "Output", "Debug")
    for name, key in (("G_var.csv", "G_var"), ("G.csv", "G"), ("B.csv", "B"), ("B_var.csv", "B_var")):
        i, j, v = read_triplets(os.path.join(dbg, name))
        want = ref[key]
        assert np.array_equal(i, want[:, 0].astype(np.int64)), name   # same entries, same order
        assert np.array_equal(j, want[:, 1].astype(np.int64)), name
        assert np.allclose(v, want[:, 2], rtol=2e-6, atol=1e-300), name
    with open(os.path.join(dbg, "G.csv")) as f:
        assert f.readline().strip() == "G_i,G_j,G_ij"
    s = np.loadtxt(os.path.join(str(tmp_path), "Output", "solution.csv"), delimiter=",", skiprows=1)
    assert np.allclose(s[:, :5], sol, rtol=2e-6)
    assert np.allclose(s[:, 5], sol[:, 4] - sol[:, 3], atol=2e-6 * np.abs(sol[:, 3]).max())


def test_time_file_has_the_reference_format(tmp_path):
    """Output/Debug/times.txt as Update_TimeFile writes it: the recorded run's
    header, then task,total,phase,processes with C's %e."""
    from pdds_gb300.output_files import TimeFile
    rec = open(os.path.join(os.path.dirname(__file__), "golden", "times_header.txt")).read().strip()
    tf = TimeFile(str(tmp_path))
    tf.update("MC Simulations", 4)
    tf.update("Solving system")
    lines = open(tmp_path / "Output" / "Debug" / "times.txt").read().splitlines()
    assert lines[0] == rec == TimeFile.HEADER
    t, total, phase, n = lines[1].split(",")
    assert t == "MC Simulations" and n == "4" and float(total) >= float(phase) >= 0.0
    assert total == "%e" % float(total)
    t2, total2, phase2, n2 = lines[2].split(",")
    assert t2 == "Solving system" and n2 == "1" and float(total2) >= float(total)
