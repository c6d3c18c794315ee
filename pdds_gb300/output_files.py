"""The reference's on-disk outputs of one solve, byte-compatible with its
writers (PDDAlgorithms/PDDSparseGM.cpp:3176-3244, Compute_Solution), so its
MATLAB post-processing reads them unchanged:

  Output/Debug/G_var.csv   Gvar_i,Gvar_j,Gvar_ij   the G_var triplets
  Output/Debug/G.csv       G_i,G_j,G_ij            I + G
  Output/Debug/B_var.csv   B_i,B_j,B_ij            B^2 - BB, column 0
  Output/Debug/B.csv       B_i,B_j,B_ij            B, column 0
  Output/solution.csv      Knot_index,x,y,sol_analytic,sol_PDDS,err,rerr

The matrices are written as the reference's column-major sparse matrices
iterate them: by column, rows ascending within a column; I + G holds the
union of G's entries and the diagonal.  Values use C's %e.  rerr is
|err| / sol_analytic (the reference divides by the signed analytic value).
"""
from __future__ import annotations

import os

import numpy as np


def _colmajor(rows, cols, vals):
    order = np.lexsort((rows, cols))
    return rows[order], cols[order], vals[order]


def _write(path, header, rows, cols, vals):
    with open(path, "w") as f:
        f.write(header + "\n")
        for i, j, v in zip(rows.tolist(), cols.tolist(), vals.tolist()):
            f.write("%d,%d,%e\n" % (i, j, v))


def write_outputs(directory: str, x, y, row_ptr, col, G, G_var, B, BB, u, u_exact):
    """Writes the five files under directory/Output (created if needed)."""
    K = len(B)
    row_ptr = np.asarray(row_ptr, np.int64)
    col = np.asarray(col, np.int64)
    rows = np.repeat(np.arange(K, dtype=np.int64), np.diff(row_ptr))
    G = np.asarray(G, np.float64)
    G_var = np.zeros_like(G) if G_var is None else np.asarray(G_var, np.float64)
    dbg = os.path.join(directory, "Output", "Debug")
    os.makedirs(dbg, exist_ok=True)
    _write(os.path.join(dbg, "G_var.csv"), "Gvar_i,Gvar_j,Gvar_ij", *_colmajor(rows, col, G_var))
    # I + G: diagonal entries added to G's own, or inserted
    diag = np.arange(K, dtype=np.int64)
    on_diag = rows == col
    gval = G.copy()
    gval[on_diag] += 1.0
    missing = np.setdiff1d(diag, rows[on_diag])
    r_all = np.concatenate([rows, missing])
    c_all = np.concatenate([col, missing])
    v_all = np.concatenate([gval, np.ones(len(missing))])
    _write(os.path.join(dbg, "G.csv"), "G_i,G_j,G_ij", *_colmajor(r_all, c_all, v_all))
    B = np.asarray(B, np.float64)
    BB = np.asarray(BB, np.float64)
    zero = np.zeros(K, np.int64)
    _write(os.path.join(dbg, "B_var.csv"), "B_i,B_j,B_ij", diag, zero, B * B - BB)
    _write(os.path.join(dbg, "B.csv"), "B_i,B_j,B_ij", diag, zero, B)
    u = np.asarray(u, np.float64)
    ex = np.asarray(u_exact, np.float64)
    err = u - ex
    with np.errstate(divide="ignore", invalid="ignore"):
        rerr = np.abs(err) / ex
    with open(os.path.join(directory, "Output", "solution.csv"), "w") as f:
        f.write("Knot_index,x,y,sol_analytic,sol_PDDS,err,rerr\n")
        for i in range(K):
            f.write("%d,%e,%e,%e,%e,%e,%e\n" % (i, x[i], y[i], ex[i], u[i], err[i], rerr[i]))


class TimeFile:
    """The reference's phase trace, Output/Debug/times.txt (Update_TimeFile,
    PDDAlgorithms/PDDSparseGM.cpp:4397-4404): one line per phase,
    `task,total since start,phase time,processes` in C's %e, under the
    reference's header.  The clock starts when the object is made."""

    HEADER = "task,total_tike,task_time,N_process"

    def __init__(self, directory: str):
        import time
        self._time = time.perf_counter
        dbg = os.path.join(directory, "Output", "Debug")
        os.makedirs(dbg, exist_ok=True)
        self.path = os.path.join(dbg, "times.txt")
        with open(self.path, "w") as f:
            f.write(self.HEADER + "\n")
        self.start = self.prev = self._time()

    def update(self, task: str, n_processors: int = 1):
        now = self._time()
        with open(self.path, "a") as f:
            f.write("%s,%e,%e,%d\n" % (task, now - self.start, now - self.prev, n_processors))
        self.prev = now


KNOT_METADATA_COLUMNS = ("APL", "WCtime", "RNGCalls", "Estimated_Variance", "Estimated_Variance_VR",
                         "PCoeff_old", "PCoeff_new", "Var_Plain", "Var_VR", "bias_num", "bias_trap")


def write_knot_metadata(directory: str, metadata: dict):
    """directory/Output/Debug/knot_metadata.csv in the reference's format
    (Process_Metadata, PDDAlgorithms/PDDSparseGM.cpp:3128-3154): one line per
    knot, index then the columns of Estimate.knot_metadata() in C's %e."""
    dbg = os.path.join(directory, "Output", "Debug")
    os.makedirs(dbg, exist_ok=True)
    cols = [np.asarray(metadata[c], np.float64) for c in KNOT_METADATA_COLUMNS]
    with open(os.path.join(dbg, "knot_metadata.csv"), "w") as f:
        f.write("index," + ",".join(KNOT_METADATA_COLUMNS) + "\n")
        for i in range(len(cols[0])):
            f.write("%u," % i + ",".join("%e" % c[i] for c in cols) + "\n")


def read_triplets(path):
    """(i, j, value) columns of one of the Debug CSV files."""
    data = np.loadtxt(path, delimiter=",", skiprows=1, ndmin=2)
    return data[:, 0].astype(np.int64), data[:, 1].astype(np.int64), data[:, 2]
