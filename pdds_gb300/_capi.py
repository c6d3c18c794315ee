"""ctypes mirror of include/pdds.h.

Loading fails loudly when the CUDA library has not been built: there is no
CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpdds_gb300.so")

# status codes
OK, ERR_INVALID, ERR_CUDA, ERR_STEP_LIMIT, ERR_TIMEOUT, ERR_ILL_CONDITIONED, ERR_NOT_CONVERGED, \
    ERR_NO_MEMORY, ERR_EXIT_SIDE, ERR_BOUNDS = range(10)
STATUS_NAMES = {0: "PDDS_OK", 1: "PDDS_ERR_INVALID", 2: "PDDS_ERR_CUDA", 3: "PDDS_ERR_STEP_LIMIT",
                4: "PDDS_ERR_TIMEOUT", 5: "PDDS_ERR_ILL_CONDITIONED", 6: "PDDS_ERR_NOT_CONVERGED",
                7: "PDDS_ERR_NO_MEMORY", 8: "PDDS_ERR_EXIT_SIDE", 9: "PDDS_ERR_BOUNDS"}

POISSON_SINCOS, MONEGROS, HELMHOLTZ, VARCOEF, LUT, CIRCLE_POISSON, ROBIN_POISSON = 0, 1, 2, 3, 4, 5, 6
MODE_REPLAY_FP64, MODE_FP64, MODE_MIXED = 0, 1, 2
SOLVE_BICGSTAB_FP64, SOLVE_GMRES_FP32_IR = 0, 1

EXPORTS = [
    "pdds_create", "pdds_destroy", "pdds_release_cached_blocks", "pdds_last_error", "pdds_version",
    "pdds_problem_set", "pdds_problem_set_lut",
    "pdds_layout_build", "pdds_layout_build_circle", "pdds_layout_knots", "pdds_layout_csr", "pdds_layout_stencil",
    "pdds_estimate", "pdds_estimate_knot_paths", "pdds_estimate_knot_steps", "pdds_autotune", "pdds_solve_interface",
    "pdds_subdomain_solve", "pdds_semilinear_tables", "pdds_batch_build", "pdds_batch_run", "pdds_batch_instance",
    "pdds_solve_bicgstab_static", "pdds_check_philox", "pdds_check_portable_math", "pdds_stencils_set",
    "pdds_estimate_knot", "pdds_estimate_step_histogram", "pdds_estimate_diagnostics",
]
# per-knot diagnostic sums (pdds_estimate_diagnostics), in slot order
DIAG_N = 18
DIAG_NAMES = ("score", "score2", "xi", "xi2", "score_vr", "score_vr2", "xi_score", "tau",
              "sub_score", "sub_score2", "sub_xi", "sub_xi2", "sub_score_vr", "sub_score_vr2", "sub_xi_score",
              "sub_tau", "rng", "paths")
STATIC_SOLVE_MAX_K = 131072
PHILOX_PORTABLE, PHILOX_ROUND_KEYS = 0, 1
FN_EXP, FN_LOG, FN_SIN, FN_COS, FN_BOX_MULLER_Z0, FN_BOX_MULLER_Z1 = range(6)


class ProblemDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("use_cv", C.c_int32), ("p", C.c_double * 8)]


class LayoutDesc(C.Structure):
    _fields_ = [("sw", C.c_double * 2), ("ne", C.c_double * 2), ("nsub", C.c_int32),
                ("nnode", C.c_int32), ("fac", C.c_double * 4)]


class CircleDesc(C.Structure):
    _fields_ = [("radius", C.c_double), ("nrings", C.c_int32), ("nsectors", C.c_int32), ("nnode", C.c_int32),
                ("kappa", C.c_double * 4), ("ring_ratio", C.c_double)]


class SemilinearDesc(C.Structure):
    _fields_ = [("m", C.c_int32), ("from_solution", C.c_int32), ("use_cv", C.c_int32), ("equation", C.c_int32),
                ("u0", C.c_double), ("a", C.c_double), ("c2", C.c_double), ("alpha", C.c_double),
                ("k", C.c_double)]


OUTER_NEWTON_U3 = 0
OUTER_LINEAR_SHIFT = 1


class LayoutInfo(C.Structure):
    _fields_ = [("nknots", C.c_int32), ("nboundary", C.c_int32), ("nstencils", C.c_int32),
                ("nsides", C.c_int32), ("nshapes", C.c_int32), ("max_side", C.c_int32),
                ("nnz", C.c_int64), ("h2d_bytes", C.c_int64)]


class StencilDesc(C.Structure):
    _fields_ = [("rect", C.c_double * 4), ("n", C.c_int32 * 4), ("index", C.POINTER(C.c_int32) * 4),
                ("x", C.POINTER(C.c_double) * 4), ("y", C.POINTER(C.c_double) * 4), ("c2", C.c_double * 4)]


class EstimateDesc(C.Structure):
    _fields_ = [("mode", C.c_int32), ("npaths", C.c_int32), ("h", C.c_double), ("seed", C.c_uint64),
                ("instance", C.c_uint32), ("dup_sum", C.c_int32), ("want_var", C.c_int32),
                ("bins_per_gap", C.c_int32), ("max_steps", C.c_int64),
                ("ipsi_override", C.POINTER(C.c_double)), ("ipsi_override_len", C.c_int64),
                ("adaptive_h", C.c_int32), ("richardson", C.c_int32), ("reuse_tables", C.c_int32),
                ("adaptive_n", C.c_int32), ("npaths_max", C.c_int32), ("target_stderr", C.c_double),
                ("cta_threads", C.c_int32), ("plain_launch", C.c_int32), ("step_histogram", C.c_int32),
                ("diagnostics", C.c_int32), ("knot_first", C.c_int32), ("knot_count", C.c_int32)]


class EstimateInfo(C.Structure):
    _fields_ = [("path_steps", C.c_int64), ("paths", C.c_int64), ("exits_global", C.c_int64),
                ("exits_stencil", C.c_int64), ("ms_setup", C.c_double), ("ms_paths", C.c_double),
                ("kernel_launches", C.c_int32), ("cta_threads", C.c_int32), ("h2d_bytes", C.c_int64),
                ("d2h_bytes", C.c_int64)]


class TuneInfo(C.Structure):
    _fields_ = [("blocks_per_sm", C.c_int32), ("paths_per_item", C.c_int32), ("candidates", C.c_int32),
                ("sample_knots", C.c_int32), ("best_ms", C.c_double), ("default_ms", C.c_double),
                ("cta_threads", C.c_int32), ("continuation_threads", C.c_int32),
                ("continuation_ms", C.c_double * 2), ("continuation_paths_per_item", C.c_int32)]


class SolveDesc(C.Structure):
    _fields_ = [("method", C.c_int32), ("restart", C.c_int32), ("max_iter", C.c_int32),
                ("max_refine", C.c_int32), ("tol", C.c_double), ("barrier_poll_limit", C.c_int32),
                ("gmres_form", C.c_int32), ("grid_ctas", C.c_int32)]


GMRES_PIPELINED, GMRES_CLASSICAL = 0, 1


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("refinements", C.c_int32), ("rel_residual", C.c_double),
                ("ms", C.c_double), ("kernel_launches", C.c_int32), ("h2d_bytes", C.c_int64),
                ("d2h_bytes", C.c_int64)]


class InstanceDesc(C.Structure):
    _fields_ = [("layout", LayoutDesc), ("p", C.c_double * 8), ("h", C.c_double)]


class BatchInfo(C.Structure):
    _fields_ = [("ninstances", C.c_int32), ("max_knots", C.c_int32), ("nknots", C.c_int64), ("nnz", C.c_int64)]


class BatchRunDesc(C.Structure):
    _fields_ = [("estimate", EstimateDesc), ("solve", SolveDesc), ("use_graph", C.c_int32), ("waves", C.c_int32)]


class BatchRunInfo(C.Structure):
    _fields_ = [("ms", C.c_double), ("path_steps", C.c_int64), ("paths", C.c_int64),
                ("exits_global", C.c_int64), ("exits_stencil", C.c_int64), ("kernel_launches", C.c_int32),
                ("graph_replayed", C.c_int32), ("max_iterations", C.c_int32), ("unconverged", C.c_int32),
                ("max_rel_residual", C.c_double)]


_lib = None


def load(path: str = LIB_PATH):
    """Loads the CUDA library; raises if it is missing (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"pdds_gb300 CUDA library not found at {path}; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'`")
    L = C.CDLL(path)
    vp = C.c_void_p
    dp = C.POINTER(C.c_double)
    L.pdds_create.argtypes = [C.POINTER(vp), C.c_int, C.c_uint32]
    L.pdds_destroy.argtypes = [vp]
    L.pdds_release_cached_blocks.argtypes = [C.c_int32]
    L.pdds_last_error.restype = C.c_char_p
    L.pdds_last_error.argtypes = [vp]
    L.pdds_version.restype = C.c_char_p
    L.pdds_problem_set.argtypes = [vp, C.POINTER(ProblemDesc)]
    L.pdds_problem_set_lut.argtypes = [vp, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int32, C.c_int32,
                                       C.POINTER(C.c_double)]
    L.pdds_layout_build.argtypes = [vp, C.POINTER(LayoutDesc), C.POINTER(LayoutInfo)]
    L.pdds_layout_build_circle.argtypes = [vp, C.POINTER(CircleDesc), C.POINTER(LayoutInfo)]
    L.pdds_layout_knots.argtypes = [vp, dp, dp, C.POINTER(C.c_int32)]
    L.pdds_layout_csr.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int32)]
    L.pdds_layout_stencil.argtypes = [vp, C.c_int32, dp, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                      C.POINTER(C.c_int32), C.c_int32]
    L.pdds_estimate.argtypes = [vp, C.POINTER(EstimateDesc), dp, dp, dp, dp, C.POINTER(EstimateInfo)]
    i32p = C.POINTER(C.c_int32)
    L.pdds_stencils_set.argtypes = [vp, dp, C.c_int32, dp, dp, i32p, C.POINTER(StencilDesc), C.POINTER(LayoutInfo)]
    L.pdds_estimate_knot.argtypes = [vp, dp, C.c_double, C.c_double, C.c_int32, C.POINTER(StencilDesc),
                                     C.POINTER(EstimateDesc), i32p, dp, dp, C.c_int32, i32p, dp, dp,
                                     C.POINTER(EstimateInfo)]
    L.pdds_autotune.argtypes = [vp, C.POINTER(EstimateDesc), C.c_int32, C.POINTER(TuneInfo)]
    L.pdds_estimate_knot_steps.argtypes = [vp, C.POINTER(C.c_int64)]
    L.pdds_estimate_step_histogram.argtypes = [vp, C.POINTER(C.c_int64)]
    L.pdds_estimate_diagnostics.argtypes = [vp, C.POINTER(C.c_double)]
    L.pdds_estimate_knot_paths.argtypes = [vp, C.POINTER(C.c_int32)]
    L.pdds_subdomain_solve.argtypes = [vp, C.c_int32, dp, dp]
    L.pdds_solve_interface.argtypes = [vp, C.POINTER(SolveDesc), dp, C.POINTER(SolveInfo)]
    L.pdds_batch_build.argtypes = [vp, C.POINTER(InstanceDesc), C.c_int32, C.POINTER(BatchInfo)]
    L.pdds_batch_run.argtypes = [vp, C.POINTER(BatchRunDesc), C.POINTER(BatchRunInfo)]
    L.pdds_batch_instance.argtypes = [vp, C.c_int32, C.POINTER(C.c_int32), dp, dp, dp, dp, C.POINTER(C.c_int32), dp,
                                      dp]
    L.pdds_solve_bicgstab_static.argtypes = [C.c_int, C.c_int32, C.c_int64, vp, vp, vp, vp, vp, C.c_double,
                                             C.c_int32, vp, C.POINTER(C.c_int32), dp, C.c_char_p, C.c_int32]
    u32p = C.POINTER(C.c_uint32)
    L.pdds_check_philox.argtypes = [C.c_int, C.c_int32, u32p, u32p, C.c_int32, u32p, C.c_char_p, C.c_int32]
    L.pdds_check_portable_math.argtypes = [C.c_int, C.c_int32, dp, C.c_int32, dp, C.c_char_p, C.c_int32]
    for name in EXPORTS:
        if not hasattr(L, name):
            raise RuntimeError("missing export " + name)
    _lib = L
    return L


class PDDSError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status
