"""Host-side mirror of the reference's PDDSparse call surface over the C ABI.

  BVP            <- struct bvp (BVPs/BVP.hpp:89-137): problem selected by kind
  read_configuration <- PDDSparseGM::ReadFromFile (PDDAlgorithms/PDDSparseGM.cpp:99-345)
  PDDSparseGM    <- PDDSparseGM (PDDAlgorithms/PDDSparseGM.hpp:103-280):
                    constructor = Fullfill_interfaces, estimate = the worker
                    loop of Solve (:795-848) for every knot at once,
                    solve_interface = Compute_Solution (:3168-3246),
                    Solve = both.
Everything runs through libpdds_gb300.so on one GPU.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _capi as capi
from ._capi import PDDSError


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class BVP:
    """A boundary value problem  1/2 tr(sigma sigma^T D^2 u) + b.grad u + c u + f = 0,
    u = g on the boundary, compiled into the library and selected by kind."""

    POISSON_SINCOS = capi.POISSON_SINCOS
    MONEGROS = capi.MONEGROS
    HELMHOLTZ = capi.HELMHOLTZ
    VARCOEF = capi.VARCOEF
    LUT = capi.LUT
    CIRCLE_POISSON = capi.CIRCLE_POISSON
    ROBIN_POISSON = capi.ROBIN_POISSON
    ROBIN_SIDES = {"N": 1, "S": 2, "E": 4, "W": 8}

    def __init__(self, kind: int, params=(), use_cv: bool = True, tables=None, exact=None):
        self.kind = int(kind)
        self.params = tuple(float(v) for v in params)
        self.use_cv = bool(use_cv)
        self.tables = tables      # (coef [ny][nx][8], g [ny][nx], bounds) for LUT problems
        self.exact = exact        # optional exact solution u(x, y) for LUT problems

    @classmethod
    def poisson_sincos(cls):
        """Lap u = f on the domain with u = sin(pi x)cos(pi y) + x y (sigma = sqrt2 I)."""
        return cls(cls.POISSON_SINCOS)

    @classmethod
    def circle_poisson(cls):
        """Lap u = f on the unit disk with u = r^2 sin(3 theta) + cos x (sigma = sqrt2 I)."""
        return cls(cls.CIRCLE_POISSON)

    @classmethod
    def robin_poisson(cls, side: str = "W"):  # side None: Dirichlet everywhere
        """Lap u + f = 0 with u = sin(pi(0.23x + 0.49y)) + cos(pi(0.331x + 0.667y))
        (BVPs/EDPs/poisson_3.hpp); on the given side of the layout rectangle the
        Robin condition du/dn - varphi u = psi, varphi = -2 + sin(pi y), instead
        of Dirichlet data: paths reflect there (Lepingle's step)."""
        return cls(cls.ROBIN_POISSON, (float(cls.ROBIN_SIDES[side]) if side else 0.0,))

    @classmethod
    def monegros(cls):
        return cls(cls.MONEGROS)

    @classmethod
    def helmholtz(cls, a: float, b: float, c: float):
        """Lap u + c u + f = 0 with u = sin(a x) cos(b y), c <= 0."""
        return cls(cls.HELMHOLTZ, (a, b, c))

    @classmethod
    def varcoef(cls):
        return cls(cls.VARCOEF)

    SAMPLERS = ("bspline", "catmull_rom", "bilinear")  # problem p[0] = position

    @classmethod
    def lut(cls, coef, g, bounds, exact=None, sampler: str = "bspline"):
        """Problem with diagonal sigma, b, c, f, grad u and g served from FP32
        tables; coef [ny][nx][8], g [ny][nx].  The FP64 and replay forms sample
        them with bicubic Catmull-Rom interpolation; the MIXED form with the
        interpolating cubic B-spline from textures (sampler "bspline"), the
        same Catmull-Rom node sampler ("catmull_rom") or hardware-filtered
        bilinear interpolation of the nodes ("bilinear")."""
        import numpy as np
        if sampler not in cls.SAMPLERS:
            raise ValueError(f"sampler must be one of {cls.SAMPLERS}")
        return cls(cls.LUT, (float(cls.SAMPLERS.index(sampler)),),
                   tables=(np.ascontiguousarray(coef, np.float32), np.ascontiguousarray(g, np.float32),
                           tuple(bounds)), exact=exact)

    @classmethod
    def varcoef_lut(cls, n: int = 1024, bounds=(0.0, 0.0, 1.0, 1.0), sampler: str = "bspline"):
        """The variable-coefficient problem served from n x n tables."""
        from .config import varcoef_tables
        coef, g, b = varcoef_tables(n, bounds)
        return cls.lut(coef, g, b, exact=lambda x, y: np.exp(x) * np.cos(2 * y) + 1.0, sampler=sampler)

    def desc(self) -> capi.ProblemDesc:
        d = capi.ProblemDesc()
        d.kind = self.kind
        d.use_cv = int(self.use_cv)
        for i, v in enumerate(self.params):
            d.p[i] = v
        return d

    def u(self, x, y):
        """Exact solution (numpy, FP64)."""
        x = np.asarray(x, np.float64)
        y = np.asarray(y, np.float64)
        if self.kind == self.LUT:
            if self.exact is None:
                raise ValueError("no exact solution attached to this table problem")
            return self.exact(x, y)
        if self.kind == self.POISSON_SINCOS:
            return np.sin(np.pi * x) * np.cos(np.pi * y) + x * y
        if self.kind == self.HELMHOLTZ:
            return np.sin(self.params[0] * x) * np.cos(self.params[1] * y)
        if self.kind == self.VARCOEF:
            return np.exp(x) * np.cos(2 * y) + 1.0
        if self.kind == self.CIRCLE_POISSON:
            r = np.hypot(x, y)
            return r * r * np.sin(3.0 * np.arctan2(y, x)) + np.cos(x)
        if self.kind == self.ROBIN_POISSON:
            return np.sin(np.pi * (0.23 * x + 0.49 * y)) + np.cos(np.pi * (0.331 * x + 0.667 * y))
        q = 1.0 + 0.01 * x * x + 0.02 * y * y
        return 3.0 + 0.333 * (np.sin(np.sqrt(q)) +
                              np.tanh(np.sin(0.12 * x + 0.05 * y) + np.sin(0.05 * x - 0.12 * y)))


def linear_iteration_u(x, y):
    """Exact solution of the linear fixed-point loop's test problem
    (Equation_u, BVPs/EDPs/Salou_Iterative.hpp)."""
    return np.sin(2.0 * np.pi * x + 0.5) * np.cos(np.pi * np.pi * (x + y))


def read_configuration(path: str) -> dict:
    """Key = value configuration file of the reference (ReadFromFile).

    Keys: h0, eps, fac (four values), T, SW (two), NE (two), N, N_job,
    N_subdo, N_node; lines starting with '%' are comments.  As in the
    reference a key is recognised with or without spaces around '=' and only
    the first value of N_subdo / N_node is used for both directions.  A
    single fac value is used for every side kind.
    """
    out = {"T": math.inf}
    with open(path) as f:
        for line in f:
            if not line.strip() or line.lstrip().startswith("%"):
                continue
            if "=" not in line:
                continue
            key, _, rest = line.partition("=")
            key = key.strip()
            vals = rest.split()
            if not vals:
                continue
            if key in ("h0", "eps", "T"):
                out[key] = float(vals[0])
            elif key in ("N", "N_job"):
                out[key] = int(float(vals[0]))
            elif key in ("N_subdo", "N_node"):
                out[key] = int(float(vals[0]))
            elif key in ("SW", "NE"):
                out[key] = (float(vals[0]), float(vals[1]))
            elif key == "fac":
                f4 = [float(v) for v in vals[:4]]
                while len(f4) < 4:
                    f4.append(f4[-1])
                out[key] = tuple(f4)
    return out


@dataclass
class Estimate:
    """G in CSR (row_ptr, col, val, var), B, BB and counters of one estimation."""

    row_ptr: np.ndarray
    col: np.ndarray
    val: np.ndarray
    var: np.ndarray
    B: np.ndarray
    BB: np.ndarray
    info: dict = field(default_factory=dict)
    npaths: np.ndarray = None  # paths per knot (0 for boundary knots)
    diag: np.ndarray = None    # [K, DIAG_N] diagnostic sums (estimate(diagnostics=True))

    @property
    def B_var(self):
        """The reference's signed B_var = B^2 - BB (PDDSparseGM.cpp:833)."""
        return self.B * self.B - self.BB

    def knot_metadata(self) -> dict:
        """Per-knot columns of the reference's knot_metadata.csv
        (Process_Metadata, PDDAlgorithms/PDDSparseGM.cpp:3092-3155) from the
        diagnostic sums, as its iterative loops fill them (:4049-4069) after
        Update (Solvers/EMFKACSolver.hpp:656-685), with the analytic
        reduction's sums: APL = mean tau, RNGCalls = normals drawn, the
        plain and control-variate score variances, the correlation of the
        score with xi at the linear (PCoeff_old) and sublinear (PCoeff_new)
        exit, and the sublinear-minus-linear score (bias_num, bias_trap).
        WCtime is 0: the reference's collection of per-knot times is
        commented out (:3015-3018).  Knots without paths give NaN moments."""
        if self.diag is None:
            raise ValueError("no diagnostics: run estimate(..., diagnostics=True)")
        s = np.asarray(self.diag, np.float64)
        with np.errstate(divide="ignore", invalid="ignore"):
            m = s / s[:, capi.DIAG_N - 1:capi.DIAG_N]
            ix = {n: i for i, n in enumerate(capi.DIAG_NAMES)}
            phi, phiphi = m[:, ix["score"]], m[:, ix["score2"]]
            xi, xixi = m[:, ix["xi"]], m[:, ix["xi2"]]
            vr, vrvr = m[:, ix["score_vr"]], m[:, ix["score_vr2"]]
            xiphi = m[:, ix["xi_score"]]
            phs, phsphs, xiphs = m[:, ix["sub_score"]], m[:, ix["sub_score2"]], m[:, ix["sub_xi_score"]]
            sd_xi = np.sqrt(xixi - xi * xi)
            var_plain = phiphi - phi * phi
            var_vr = vrvr - vr * vr
            return {
                "APL": m[:, ix["tau"]],
                "WCtime": np.zeros(len(s)),
                "RNGCalls": s[:, ix["rng"]],
                "Estimated_Variance": var_plain,
                "Estimated_Variance_VR": var_vr,
                "PCoeff_old": (xiphi - phi * xi) / (np.sqrt(var_plain) * sd_xi),
                "PCoeff_new": (xiphs - phs * xi) / (np.sqrt(phsphs - phs * phs) * sd_xi),
                "Var_Plain": var_plain,
                "Var_VR": var_vr,
                "bias_num": phs - phi,
                "bias_trap": phs - phi,
            }

    def triplets(self):
        rows = np.repeat(np.arange(len(self.row_ptr) - 1), np.diff(self.row_ptr))
        return rows, self.col, self.val


def release_cached_blocks(device: int = -1) -> None:
    """Returns to the device the buffers the library keeps from closed
    PDDSparseGM contexts (pdds_release_cached_blocks; device -1: every
    device), e.g. before handing the GPU's memory to another allocator."""
    st = capi.load().pdds_release_cached_blocks(int(device))
    if st != capi.OK:
        raise PDDSError(st, "pdds_release_cached_blocks failed")


class PDDSparseGM:
    """GPU PDDSparse interface system on a rectangular layout.

    fac[kind] is the Gaussian RBF shape c of a stencil side of that kind
    (the reference's c2[kind], Meshes/stencil.cpp:211-243)."""

    def __init__(self, sw=(-1.0, -1.0), ne=(1.0, 1.0), nsub: int = 4, nnode: int = 11,
                 fac=(1.0, 1.0, 1.0, 1.0), device: int = 0, circle=None, stencils=None):
        self._lib = capi.load()
        self._ctx = C.c_void_p()
        st = self._lib.pdds_create(C.byref(self._ctx), int(device), 0)
        if st != capi.OK:
            raise PDDSError(st, "pdds_create failed (device %d)" % device)
        self.device = device
        info = capi.LayoutInfo()
        if stencils is not None:
            domain, kx, ky, knot_id, sts = stencils
            kx = np.ascontiguousarray(kx, np.float64)
            ky = np.ascontiguousarray(ky, np.float64)
            n = len(kx)
            arr = (capi.StencilDesc * n)()
            for i, st in enumerate(sts):
                arr[i] = st.desc()
            self._keep_stencils = list(sts)
            dom = np.ascontiguousarray(domain, np.float64)
            kid = None if knot_id is None else np.ascontiguousarray(knot_id, np.int32)
            self._check(self._lib.pdds_stencils_set(self._ctx, _p(dom, C.c_double), n, _p(kx, C.c_double),
                                                    _p(ky, C.c_double), None if kid is None else _p(kid, C.c_int32),
                                                    arr, C.byref(info)))
            sw, ne, nsub, fac = (dom[0], dom[1]), (dom[2], dom[3]), 0, (1.0, 1.0, 1.0, 1.0)
        elif circle is not None:
            radius, nrings, nsectors, kappa = circle[:4]
            d = capi.CircleDesc()
            d.radius, d.nrings, d.nsectors, d.nnode = float(radius), int(nrings), int(nsectors), int(nnode)
            d.ring_ratio = float(circle[4]) if len(circle) > 4 else 0.0
            for i in range(4):
                d.kappa[i] = float(kappa[i])
            self._check(self._lib.pdds_layout_build_circle(self._ctx, C.byref(d), C.byref(info)))
            sw, ne, nsub, fac = (-radius, -radius), (radius, radius), nrings, tuple(kappa)
        else:
            d = capi.LayoutDesc()
            d.sw[0], d.sw[1] = float(sw[0]), float(sw[1])
            d.ne[0], d.ne[1] = float(ne[0]), float(ne[1])
            d.nsub = int(nsub)
            d.nnode = int(nnode)
            for i in range(4):
                d.fac[i] = float(fac[i])
            self._check(self._lib.pdds_layout_build(self._ctx, C.byref(d), C.byref(info)))
        self.circle = circle
        self.sw, self.ne, self.nsub, self.nnode, self.fac = tuple(sw), tuple(ne), nsub, nnode, tuple(fac)
        self.layout_info = {f: getattr(info, f) for f, _ in capi.LayoutInfo._fields_}
        K = info.nknots
        self.K = K
        self.x = np.zeros(K)
        self.y = np.zeros(K)
        self.order = np.zeros(K, np.int32)
        self._check(self._lib.pdds_layout_knots(self._ctx, _p(self.x, C.c_double), _p(self.y, C.c_double),
                                                _p(self.order, C.c_int32)))
        self.row_ptr = np.zeros(K + 1, np.int64)
        self.col = np.zeros(max(info.nnz, 1), np.int32)
        self._check(self._lib.pdds_layout_csr(self._ctx, _p(self.row_ptr, C.c_int64),
                                              _p(self.col, C.c_int32)))
        self.col = self.col[:info.nnz]
        self.nnz = int(info.nnz)
        self.n_mc = K - int(info.nboundary)  # knots with paths (hand-out positions of a knot range)

    @classmethod
    def circle_mesh(cls, radius: float = 1.0, nrings: int = 6, nsectors: int = 16, nnode: int = 11,
                    kappa=(3.164, 3.164, 3.164, 3.164), device: int = 0, ring_ratio: float = 0.0):
        """Disk of the given radius split into nrings x nsectors annular
        sectors (MIXED mode, sigma = sqrt2 I problems); kappa[kind] scales
        the RBF shape to each side's knot spacing; ring i is ring_ratio^i as
        wide as the central disk's radius (0: equal rings)."""
        return cls(nnode=nnode, device=device, circle=(radius, nrings, nsectors, kappa, ring_ratio))

    @classmethod
    def from_stencils(cls, domain, x, y, stencils, knot_id=None, device: int = 0):
        """Knots at (x[i], y[i]) with caller-built stencils (Stencil objects)
        in the problem's rectangle domain {x0, y0, x1, y1}; knot i draws the
        Philox knot word knot_id[i] (default i)."""
        return cls(device=device, stencils=(domain, x, y, knot_id, list(stencils)))

    @classmethod
    def from_configuration(cls, path: str, device: int = 0):
        cfg = read_configuration(path)
        return cls(cfg["SW"], cfg["NE"], cfg["N_subdo"], cfg["N_node"], cfg["fac"], device=device)

    # ------------------------------------------------------------------
    def _check(self, st):
        if st != capi.OK:
            msg = self._lib.pdds_last_error(self._ctx).decode() if self._ctx else ""
            raise PDDSError(st, msg)

    def close(self):
        if getattr(self, "_ctx", None) and self._ctx.value:
            self._lib.pdds_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ------------------------------------------------------------------
    def stencil(self, knot: int, maxn: int = 512):
        rect = np.zeros(4)
        kinds = np.zeros(4, np.int32)
        sizes = np.zeros(4, np.int32)
        idx = np.zeros(4 * maxn, np.int32)
        self._check(self._lib.pdds_layout_stencil(self._ctx, int(knot), _p(rect, C.c_double),
                                                  _p(kinds, C.c_int32), _p(sizes, C.c_int32),
                                                  _p(idx, C.c_int32), maxn))
        return rect, kinds, [idx[d * maxn:d * maxn + sizes[d]].copy() for d in range(4)]

    def estimate(self, bvp: BVP, npaths: int, h: float, mode: int = capi.MODE_MIXED, seed: int = 1234,
                 instance: int = 0, dup_sum: bool = False, want_var: bool = False,
                 bins_per_gap: int = 0, max_steps: int = 0, ipsi_override=None,
                 adaptive_h: bool = False, richardson: bool = False, reuse_tables: bool = False,
                 adaptive_n: bool = False, npaths_max: int = 0, target_stderr: float = 0.0,
                 cta_threads: int = 0, plain_launch: bool = False, step_histogram: bool = False,
                 diagnostics: bool = False, knot_first: int = 0, knot_count: int = 0) -> Estimate:
        """Runs the Feynman-Kac estimation of every knot's G row and B entry.

        knot_first, knot_count: only the knots with paths at these hand-out
        positions (count 0: to the last; n_mc = K - nboundary positions);
        the others' rows stay zero and Estimate.npaths is 0 for them (the
        unit of pdds_gb300.checkpoint.estimate_resumable).

        diagnostics: also the reduction's per-knot diagnostic sums
        (Estimate.diag, Estimate.knot_metadata(); pdds_estimate_diagnostics).

        plain_launch: one CTA per work item, knots in layout order (the launch
        the persistent CTAs and the heaviest-first order replace; for
        comparison).

        adaptive_n: npaths is the pilot per knot; each knot then runs
        N_k = 4 Var_k / (0.66666 target_stderr)^2 paths (multiple of 256,
        clamped to [npaths, npaths_max]); Estimate.npaths holds N_k."""
        if bvp.kind == BVP.LUT and bvp.tables is not None and getattr(self, "_lut_owner", None) is not bvp.tables:
            coef, g, bounds = bvp.tables
            ny, nx = g.shape
            b = np.ascontiguousarray(bounds, np.float64)
            self._check(self._lib.pdds_problem_set_lut(self._ctx, _p(coef, C.c_float), _p(g, C.c_float), nx, ny,
                                                       _p(b, C.c_double)))
            self._lut_owner = bvp.tables
        self._check(self._lib.pdds_problem_set(self._ctx, C.byref(bvp.desc())))
        d = capi.EstimateDesc()
        d.mode = int(mode)
        d.npaths = int(npaths)
        d.h = float(h)
        d.seed = int(seed)
        d.instance = int(instance)
        d.dup_sum = int(bool(dup_sum))
        d.want_var = int(bool(want_var))
        d.bins_per_gap = int(bins_per_gap)
        d.max_steps = int(max_steps)
        d.adaptive_h = int(bool(adaptive_h))
        d.richardson = int(bool(richardson))
        d.reuse_tables = int(bool(reuse_tables))
        d.adaptive_n = int(bool(adaptive_n))
        d.npaths_max = int(npaths_max)
        d.target_stderr = float(target_stderr)
        d.cta_threads = int(cta_threads)
        d.plain_launch = int(bool(plain_launch))
        d.step_histogram = int(bool(step_histogram))
        d.diagnostics = int(bool(diagnostics))
        d.knot_first = int(knot_first)
        d.knot_count = int(knot_count)
        keep = None
        if ipsi_override is not None:
            keep = np.ascontiguousarray(ipsi_override, np.float64)
            d.ipsi_override = _p(keep, C.c_double)
            d.ipsi_override_len = keep.size
        # the read-back targets stay uninitialised: pdds_estimate touches
        # their pages while the device runs the paths (a device-to-host copy
        # into never-touched pages faults them in one by one from inside the
        # copy), and the copy then overwrites every element
        read_var = want_var or mode == capi.MODE_REPLAY_FP64
        val = np.empty(max(self.nnz, 1))
        var = np.empty(max(self.nnz, 1)) if read_var else np.zeros(max(self.nnz, 1))
        B = np.zeros(self.K)
        BB = np.zeros(self.K)
        info = capi.EstimateInfo()
        # G_var is only computed by the replay mode and by MIXED with want_var;
        # otherwise var stays the (untouched) zero array and nothing is read
        # back into it
        var_out = _p(var, C.c_double) if read_var else None
        self._check(self._lib.pdds_estimate(self._ctx, C.byref(d), _p(val, C.c_double), var_out,
                                            _p(B, C.c_double), _p(BB, C.c_double), C.byref(info)))
        del keep
        kn = np.zeros(self.K, np.int32)
        self._check(self._lib.pdds_estimate_knot_paths(self._ctx, _p(kn, C.c_int32)))
        dg = None
        if diagnostics:
            dg = np.zeros((self.K, capi.DIAG_N))
            self._check(self._lib.pdds_estimate_diagnostics(self._ctx, _p(dg, C.c_double)))
        return Estimate(self.row_ptr, self.col, val[:self.nnz], var[:self.nnz], B, BB,
                        {f: getattr(info, f) for f, _ in capi.EstimateInfo._fields_}, kn, dg)

    def autotune(self, bvp: BVP, npaths: int, h: float, sample_knots: int = 0, seed: int = 1234,
                 adaptive_h: bool = False, richardson: bool = False, want_var: bool = False,
                 cta_threads: int = 0, adaptive_n: bool = False) -> dict:
        """Times the MIXED path kernel's launch shapes on a sample of knots and
        keeps the fastest for later estimates of this problem kind
        (cta_threads 128 or 256 keeps that block size, 0 searches both).
        adaptive_n: also times the continuation of the last variance-adaptive
        estimate on this layout at both block sizes and keeps the faster for
        later adaptive estimates (continuation_threads; 0 when there was none)."""
        self._check(self._lib.pdds_problem_set(self._ctx, C.byref(bvp.desc())))
        d = capi.EstimateDesc()
        d.mode = capi.MODE_MIXED
        d.npaths = int(npaths)
        d.h = float(h)
        d.seed = int(seed)
        d.adaptive_h = int(bool(adaptive_h))
        d.richardson = int(bool(richardson))
        d.want_var = int(bool(want_var))
        d.cta_threads = int(cta_threads)
        d.adaptive_n = int(bool(adaptive_n))
        info = capi.TuneInfo()
        self._check(self._lib.pdds_autotune(self._ctx, C.byref(d), int(sample_knots), C.byref(info)))
        out = {f: getattr(info, f) for f, _ in capi.TuneInfo._fields_}
        out["continuation_ms"] = list(info.continuation_ms)
        return out

    def knot_steps(self):
        """Path steps per knot of the last MIXED estimate (both Richardson levels)."""
        st = np.zeros(self.K, np.int64)
        self._check(self._lib.pdds_estimate_knot_steps(self._ctx, _p(st, C.c_int64)))
        return st

    def step_histogram(self):
        """Paths of the last MIXED estimate by exit step count: entry b counts
        the paths (each Richardson level) that took 2^b .. 2^(b+1) - 1 steps."""
        hst = np.zeros(32, np.int64)
        self._check(self._lib.pdds_estimate_step_histogram(self._ctx, _p(hst, C.c_int64)))
        return hst

    def subdomain_solve(self, m: int = 32, u=None):
        """Interior solution of every subdomain (the reference's Subdomain::Solve):
        returns (x, y, v) with v[row, col, j, i] at x[col, i], y[row, j] on an
        m x m interior grid per subdomain.  u: interface values (default: the
        last solve_interface)."""
        ns = self.nsub
        out = np.zeros((ns * ns, m, m))
        keep = None if u is None else np.ascontiguousarray(u, np.float64)
        self._check(self._lib.pdds_subdomain_solve(self._ctx, int(m), None if keep is None else _p(keep, C.c_double),
                                                   _p(out, C.c_double)))
        lx = (self.ne[0] - self.sw[0]) / ns
        ly = (self.ne[1] - self.sw[1]) / ns
        t = (np.arange(m) + 1.0) / (m + 1)
        x = self.sw[0] + (np.arange(ns)[:, None] + t[None, :]) * lx
        y = self.sw[1] + (np.arange(ns)[:, None] + t[None, :]) * ly
        return x, y, out.reshape(ns, ns, m, m)

    def semilinear_tables(self, m: int = 32, from_solution: bool = False, u0: float = 1.1, a: float = 1.1,
                          use_cv: bool = True) -> BVP:
        """One Newton linearisation of Lap u - u^3 + F = 0 on the unit square
        (the reference's Solve_SemiLin_numVR with Semilinear_u3_VR.hpp):
        tables of c = -3 u_k^2, f = F + 2 u_k^3 and grad u_k built on the device
        around the last subdomain_solve(m) (from_solution) or the constant u0.
        Returns the table-served BVP (tables stay on the device)."""
        d = capi.SemilinearDesc()
        d.m = int(m)
        d.from_solution = int(bool(from_solution))
        d.use_cv = int(bool(use_cv))
        d.equation = capi.OUTER_NEWTON_U3
        d.u0 = float(u0)
        d.a = float(a)
        self._check(self._lib.pdds_semilinear_tables(self._ctx, C.byref(d)))
        self._lut_owner = None
        return BVP(BVP.LUT, use_cv=use_cv, tables=None,
                   exact=lambda x, y: a + np.sin(np.pi * x) * np.sin(np.pi * y))

    def linear_iteration_tables(self, m: int = 32, from_solution: bool = False, u0: float = 0.0,
                                c2: float = 20.0, alpha: float = 22.0, k: float = 9.0, use_cv: bool = True) -> BVP:
        """One step of the fixed-point loop for Lap u + c2 u + F = 0 with the
        shift alpha and time rescale k (the reference's Solve_Iterative_numVR
        with Salou_Iterative.hpp, u = sin(2 pi x + 1/2) cos(pi^2 (x + y))):
        tables of sigma = sqrt(2/k) I, c = (c2 - alpha)/k, f = (F + alpha u_k)/k
        and grad u_k built on the device around the last subdomain_solve(m)
        (from_solution) or the constant u0 (0 is the reference's first
        iteration).  Returns the table-served BVP."""
        d = capi.SemilinearDesc()
        d.m = int(m)
        d.from_solution = int(bool(from_solution))
        d.use_cv = int(bool(use_cv))
        d.equation = capi.OUTER_LINEAR_SHIFT
        d.u0 = float(u0)
        d.c2 = float(c2)
        d.alpha = float(alpha)
        d.k = float(k)
        self._check(self._lib.pdds_semilinear_tables(self._ctx, C.byref(d)))
        self._lut_owner = None
        return BVP(BVP.LUT, use_cv=use_cv, tables=None, exact=linear_iteration_u)

    def solve_linear_iteration(self, iterations: int, npaths: int, h: float, m: int = 32, u0: float = 0.0,
                               c2: float = 20.0, alpha: float = 22.0, k: float = 9.0, seed: int = 1234, **opts):
        """The fixed-point outer loop of main_LinLoop.cpp: `iterations` steps,
        each an estimate and interface solve of the problem with the source
        built from the previous subdomain solution, then the subdomain solves
        (Solve_Iterative_numVR + Solve_Subdomains_LinIt; the first step, around
        u0, is the reference's Solve + Solve_Subdomains_LinIt_First).  Returns
        a list of per-iteration dicts like solve_semilinear."""
        return self._outer_loop(
            iterations, npaths, h, m, seed, opts,
            lambda it: self.linear_iteration_tables(m, from_solution=it > 0, u0=u0, c2=c2, alpha=alpha, k=k))

    def solve_semilinear(self, iterations: int, npaths: int, h: float, m: int = 32, u0: float = 1.1,
                         a: float = 1.1, seed: int = 1234, **opts):
        """The semilinear outer loop: `iterations` Newton steps, each an
        estimate and interface solve of the problem linearised around the
        previous subdomain solution, then the subdomain solves
        (Solve_SemiLin_numVR + Solve_Subdomains_SemiLin, main_VR.cpp).  Returns
        a list of per-iteration dicts (interface solution u, subdomain grid
        (x, y, v), their RMSE against the exact solution)."""
        return self._outer_loop(iterations, npaths, h, m, seed, opts,
                                lambda it: self.semilinear_tables(m, from_solution=it > 0, u0=u0, a=a))

    def _outer_loop(self, iterations, npaths, h, m, seed, opts, tables):
        out = []
        for k in range(iterations):
            bvp = tables(k)
            est = self.estimate(bvp, npaths, h, mode=capi.MODE_MIXED, seed=seed, instance=k, **opts)
            u, sinfo = self.solve_interface()
            x, y, v = self.subdomain_solve(m)
            ex_knots = bvp.u(self.x, self.y)
            ex_grid = bvp.u(x[None, :, None, :], y[:, None, :, None])  # [row, col, j, i] like v
            out.append({"u": u, "grid": (x, y, v), "estimate": est, "solve": sinfo,
                        "rmse_knots": float(np.sqrt(np.mean((u - ex_knots) ** 2))),
                        "rmse_grid": float(np.sqrt(np.mean((v - ex_grid) ** 2)))})
        return out

    def write_outputs(self, directory: str, est: "Estimate", u, bvp: BVP):
        """Writes Output/solution.csv and Output/Debug/{G,G_var,B,B_var}.csv
        under directory in the reference's format (Compute_Solution,
        PDDSparseGM.cpp:3176-3244)."""
        from .output_files import write_outputs
        write_outputs(directory, self.x, self.y, self.row_ptr, self.col, est.val, est.var, est.B, est.BB, u,
                      bvp.u(self.x, self.y))

    def solve_interface(self, method: int = capi.SOLVE_GMRES_FP32_IR, tol: float = 1e-10,
                        restart: int = 20, max_iter: int = 0, max_refine: int = 0, barrier_poll_limit: int = 0,
                        gmres_form: int = capi.GMRES_PIPELINED, grid_ctas: int = 0):
        """Solves (I + G) u = B for the last estimate; returns (u, info)."""
        d = capi.SolveDesc()
        d.gmres_form = int(gmres_form)
        d.grid_ctas = int(grid_ctas)
        d.method = int(method)
        d.restart = int(restart)
        d.max_iter = int(max_iter)
        d.max_refine = int(max_refine)
        d.tol = float(tol)
        d.barrier_poll_limit = int(barrier_poll_limit)
        u = np.zeros(self.K)
        info = capi.SolveInfo()
        self._check(self._lib.pdds_solve_interface(self._ctx, C.byref(d), _p(u, C.c_double), C.byref(info)))
        return u, {f: getattr(info, f) for f, _ in capi.SolveInfo._fields_}

    def Solve(self, bvp: BVP, npaths: int, h: float, mode: int = capi.MODE_MIXED, seed: int = 1234,
              method: int = capi.SOLVE_GMRES_FP32_IR, tol: float = 1e-10, trace_dir: str = None, **kw):
        """Estimate G and B for all knots, then solve the interface system.
        trace_dir: also write the reference's phase trace
        (trace_dir/Output/Debug/times.txt) and its output files there."""
        tf = None
        if trace_dir is not None:
            from .output_files import TimeFile
            tf = TimeFile(trace_dir)
        est = self.estimate(bvp, npaths, h, mode=mode, seed=seed, **kw)
        if tf:
            tf.update("MC Simulations")
        u, sinfo = self.solve_interface(method=method, tol=tol)
        if tf:
            tf.update("Solving system")
            self.write_outputs(trace_dir, est, u, bvp)
            tf.update("Writing Solution")
        return u, est, sinfo


_DIRS = ("N", "S", "E", "W")


class Stencil:
    """A knot's stencil as the reference's Stencil class holds it
    (Meshes/stencil.hpp:13-98): the rectangle stencil_parameters
    {x0, y0, x1, y1}, the problem's rectangle global_parameters, and per side
    N, S, E, W the knot indices and positions (Init) and the RBF shape c2
    (Compute_ipsi).  The library factorises the RBF matrices itself."""

    def __init__(self, stencil_parameters=None, global_parameters=None):
        self.stencil_parameters = None if stencil_parameters is None else tuple(float(v) for v in stencil_parameters)
        self.global_parameters = None if global_parameters is None else tuple(float(v) for v in global_parameters)
        self.index = {d: np.zeros(0, np.int32) for d in _DIRS}
        self.x = {d: np.zeros(0) for d in _DIRS}
        self.y = {d: np.zeros(0) for d in _DIRS}
        self.c2 = {d: 1.0 for d in _DIRS}

    def Init(self, s_index: dict, s_x: dict, s_y: dict, parameters):
        """Stencil::Init (Meshes/stencil.cpp:11-85): side knot lists by
        direction ('N', 'S', 'E', 'W'), given as the reference lists them (the
        library drops consecutive repeats and keeps an index's last position)."""
        self.stencil_parameters = tuple(float(v) for v in parameters)
        for d in _DIRS:
            self.index[d] = np.ascontiguousarray(s_index.get(d, ()), np.int32)
            self.x[d] = np.ascontiguousarray(s_x.get(d, ()), np.float64)
            self.y[d] = np.ascontiguousarray(s_y.get(d, ()), np.float64)
        return self

    def Compute_ipsi(self, c2):
        """The RBF shape of each side (Stencil::Compute_ipsi with c2[4] in the
        order N, S, E, W, or one value for every side)."""
        vals = [float(c2)] * 4 if np.isscalar(c2) else [float(v) for v in c2]
        self.c2 = dict(zip(_DIRS, vals))
        return self

    @classmethod
    def of_knot(cls, pd: "PDDSparseGM", knot: int, maxn: int = 512):
        """The stencil a built layout gives knot `knot` (positions from the
        layout's knots, shapes from its fac)."""
        rect, kinds, sides = pd.stencil(knot, maxn)
        st = cls(rect, (pd.sw[0], pd.sw[1], pd.ne[0], pd.ne[1]))
        for d, idx in zip(_DIRS, sides):
            st.index[d] = np.ascontiguousarray(idx, np.int32)
            st.x[d] = np.ascontiguousarray(pd.x[idx], np.float64)
            st.y[d] = np.ascontiguousarray(pd.y[idx], np.float64)
        for q, d in enumerate(_DIRS):
            st.c2[d] = float(pd.fac[kinds[q]]) if kinds[q] >= 0 else 1.0
        return st

    def desc(self):
        """The C descriptor (the arrays it points to stay owned by self)."""
        if self.stencil_parameters is None:
            raise ValueError("stencil rectangle not set (Init)")
        d = capi.StencilDesc()
        for q in range(4):
            d.rect[q] = self.stencil_parameters[q]
        for q, dd in enumerate(_DIRS):
            n = len(self.index[dd])
            if len(self.x[dd]) != n or len(self.y[dd]) != n:
                raise ValueError("side %s: index, x and y differ in length" % dd)
            d.n[q] = n
            d.c2[q] = self.c2[dd]
            if n:
                d.index[q] = _p(self.index[dd], C.c_int32)
                d.x[q] = _p(self.x[dd], C.c_double)
                d.y[q] = _p(self.y[dd], C.c_double)
        return d


def _estimate_desc(mode, npaths, h, seed, instance, dup_sum, want_var, max_steps=0, adaptive_h=False,
                   richardson=False, ipsi_override=None):
    d = capi.EstimateDesc()
    d.mode = int(mode)
    d.npaths = int(npaths)
    d.h = float(h)
    d.seed = int(seed)
    d.instance = int(instance)
    d.dup_sum = int(bool(dup_sum))
    d.want_var = int(bool(want_var))
    d.max_steps = int(max_steps)
    d.adaptive_h = int(bool(adaptive_h))
    d.richardson = int(bool(richardson))
    keep = None
    if ipsi_override is not None:
        keep = np.ascontiguousarray(ipsi_override, np.float64)
        d.ipsi_override = _p(keep, C.c_double)
        d.ipsi_override_len = keep.size
    return d, keep


class EMFKACSolver:
    """The reference's per-knot Feynman-Kac solver
    (Solvers/EMFKACSolver.hpp:711-729) on the GPU: one knot from any X0 with a
    caller-built stencil.  Per-knot calls are too fine-grained to fill a GPU;
    PDDSparseGM.estimate runs every knot of a layout at once."""

    def __init__(self, device: int = 0):
        self._lib = capi.load()
        self._ctx = C.c_void_p()
        st = self._lib.pdds_create(C.byref(self._ctx), int(device), 0)
        if st != capi.OK:
            raise PDDSError(st, "pdds_create failed (device %d)" % device)

    def _check(self, st):
        if st != capi.OK:
            raise PDDSError(st, self._lib.pdds_last_error(self._ctx).decode())

    def close(self):
        if getattr(self, "_ctx", None) and self._ctx.value:
            self._lib.pdds_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def Solve_GPU_Analytic(self, X0, N: int, h: float, rho: float, bvp: BVP, stencil: Stencil, c2: float = 0.0,
                           mode: int = capi.MODE_FP64, seed: int = 1234, knot_id: int = 0, instance: int = 0,
                           dup_sum: bool = False, want_var: bool = True, max_steps: int = 0,
                           adaptive_h: bool = False, richardson: bool = False, ipsi_override=None,
                           diagnostics: bool = False):
        """Solve_OMP_Analytic's outputs (G, G_var, G_j, B, BB) for the knot at
        X0: N paths of step h in the stencil, G_j the sorted knot indices of
        its sides.  rho and c2 are accepted for the reference's signature;
        like its G_update, the side shapes come from the stencil.  knot_id is
        the Philox knot word (a layout knot's index reproduces its stream in
        PDDSparseGM.estimate).  diagnostics: self.sums receives the
        reduction's diagnostic sums (the reference's sums[] member)."""
        del rho, c2
        if bvp.kind == BVP.LUT and bvp.tables is not None:
            coef, g, bounds = bvp.tables
            ny, nx = g.shape
            b = np.ascontiguousarray(bounds, np.float64)
            self._check(self._lib.pdds_problem_set_lut(self._ctx, _p(coef, C.c_float), _p(g, C.c_float), nx, ny,
                                                       _p(b, C.c_double)))
        self._check(self._lib.pdds_problem_set(self._ctx, C.byref(bvp.desc())))
        if stencil.global_parameters is None:
            raise ValueError("stencil.global_parameters (the problem's rectangle) not set")
        dom = np.ascontiguousarray(stencil.global_parameters, np.float64)
        sd = stencil.desc()
        ed, keep = _estimate_desc(mode, N, h, seed, instance, dup_sum, want_var, max_steps, adaptive_h, richardson,
                                  ipsi_override)
        ed.diagnostics = int(bool(diagnostics))
        cap = sum(len(stencil.index[d]) for d in _DIRS) + 1
        gj = np.zeros(cap, np.int32)
        G = np.zeros(cap)
        Gv = np.zeros(cap)
        nnz = C.c_int32()
        B = C.c_double()
        BB = C.c_double()
        info = capi.EstimateInfo()
        self._check(self._lib.pdds_estimate_knot(self._ctx, _p(dom, C.c_double), float(X0[0]), float(X0[1]),
                                                 int(knot_id), C.byref(sd), C.byref(ed), _p(gj, C.c_int32),
                                                 _p(G, C.c_double), _p(Gv, C.c_double), cap, C.byref(nnz),
                                                 C.byref(B), C.byref(BB), C.byref(info)))
        del keep
        n = nnz.value
        self.info = {f: getattr(info, f) for f, _ in capi.EstimateInfo._fields_}
        if diagnostics:
            self.sums = np.zeros(capi.DIAG_N)
            self._check(self._lib.pdds_estimate_diagnostics(self._ctx, _p(self.sums, C.c_double)))
        return G[:n].copy(), Gv[:n].copy(), gj[:n].copy(), B.value, BB.value


@dataclass
class Instance:
    """One BVP instance of a batch: its layout and problem parameters."""

    sw: tuple
    ne: tuple
    nsub: int
    nnode: int
    fac: tuple
    params: tuple = ()
    h: float = 0.0  # the instance's step (0: the run's h)


class Batch:
    """Many independent instances of one problem kind solved as one sequence.

    No counterpart in the reference, whose PDDSparseGM solves one problem per
    run.  The instances run in waves (consecutive groups in processing
    order): one path-kernel launch per wave, and one cluster-GMRES launch per
    wave on a higher-priority stream while the next wave's paths run; with
    use_graph=True the sequence is captured once in a CUDA graph and
    replayed.  order="smallest_first" processes the instances by increasing
    knot count, so the small ones finish in the first waves (lower median
    latency, the same batch time); indices in knots() and result() stay the
    caller's.  The instance at processing position j uses Philox instance
    word `instance + j` and its own knot numbering, so its random stream
    equals the one of a PDDSparseGM run of that instance alone with instance
    word `instance + j` (j = i in the given order)."""

    ORDERS = ("given", "smallest_first")

    def __init__(self, kind: int, instances, use_cv: bool = True, device: int = 0, order: str = "given"):
        if order not in self.ORDERS:
            raise ValueError(f"order must be one of {self.ORDERS}")
        self._lib = capi.load()
        self._ctx = C.c_void_p()
        st = self._lib.pdds_create(C.byref(self._ctx), int(device), 0)
        if st != capi.OK:
            raise PDDSError(st, "pdds_create failed (device %d)" % device)
        self.kind = int(kind)
        self.use_cv = bool(use_cv)
        self.instances = list(instances)
        n = len(self.instances)
        # processing position of each instance (pos[i]) and its inverse
        if order == "smallest_first":
            from .config import layout_knot_count
            size = [layout_knot_count(ins.nsub, ins.nnode) for ins in self.instances]
            self._proc = sorted(range(n), key=lambda i: (size[i], i))
        else:
            self._proc = list(range(n))
        self._pos = [0] * n
        for j, i in enumerate(self._proc):
            self._pos[i] = j
        arr = (capi.InstanceDesc * n)()
        for j, i in enumerate(self._proc):
            ins = self.instances[i]
            d = arr[j]
            d.layout.sw[0], d.layout.sw[1] = float(ins.sw[0]), float(ins.sw[1])
            d.layout.ne[0], d.layout.ne[1] = float(ins.ne[0]), float(ins.ne[1])
            d.layout.nsub = int(ins.nsub)
            d.layout.nnode = int(ins.nnode)
            for q in range(4):
                d.layout.fac[q] = float(ins.fac[q])
            for q, v in enumerate(ins.params):
                d.p[q] = float(v)
            d.h = float(ins.h)
        info = capi.BatchInfo()
        self._check(self._lib.pdds_batch_build(self._ctx, arr, n, C.byref(info)))
        self.info = {f: getattr(info, f) for f, _ in capi.BatchInfo._fields_}
        pd = capi.ProblemDesc()
        pd.kind = self.kind
        pd.use_cv = int(self.use_cv)
        self._check(self._lib.pdds_problem_set(self._ctx, C.byref(pd)))

    def _check(self, st):
        if st != capi.OK:
            msg = self._lib.pdds_last_error(self._ctx).decode() if self._ctx else ""
            raise PDDSError(st, msg)

    def close(self):
        if getattr(self, "_ctx", None) and self._ctx.value:
            self._lib.pdds_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def run(self, npaths: int, h: float, seed: int = 1234, instance: int = 0, adaptive_h: bool = True,
            richardson: bool = False, tol: float = 1e-10, restart: int = 30, use_graph: bool = True,
            bins_per_gap: int = 0, reuse_tables: bool = False, dup_sum: bool = False, waves: int = 0,
            gmres_form: int = capi.GMRES_PIPELINED) -> dict:
        """Estimates and solves every instance (in `waves` consecutive groups
        whose solves overlap the next group's paths; 0 = 16); returns the run
        counters."""
        d = capi.BatchRunDesc()
        e = d.estimate
        e.mode = capi.MODE_MIXED
        e.npaths = int(npaths)
        e.h = float(h)
        e.seed = int(seed)
        e.instance = int(instance)
        e.bins_per_gap = int(bins_per_gap)
        e.adaptive_h = int(bool(adaptive_h))
        e.richardson = int(bool(richardson))
        e.reuse_tables = int(bool(reuse_tables))
        e.dup_sum = int(bool(dup_sum))
        d.solve.method = capi.SOLVE_GMRES_FP32_IR
        d.solve.restart = int(restart)
        d.solve.tol = float(tol)
        d.use_graph = int(bool(use_graph))
        d.waves = int(waves)
        d.solve.gmres_form = int(gmres_form)
        info = capi.BatchRunInfo()
        self._check(self._lib.pdds_batch_run(self._ctx, C.byref(d), C.byref(info)))
        return {f: getattr(info, f) for f, _ in capi.BatchRunInfo._fields_}

    def position(self, i: int) -> int:
        """Processing position of instance i (its Philox instance word is the
        run's instance word plus this)."""
        return self._pos[int(i)]

    def knots(self, i: int):
        j = self._pos[int(i)]
        n = C.c_int32()
        self._check(self._lib.pdds_batch_instance(self._ctx, j, C.byref(n), None, None, None, None, None,
                                                  None, None))
        x = np.zeros(n.value)
        y = np.zeros(n.value)
        self._check(self._lib.pdds_batch_instance(self._ctx, j, None, _p(x, C.c_double), _p(y, C.c_double),
                                                  None, None, None, None, None))
        return x, y

    def result(self, i: int) -> dict:
        """u, B, solver iterations, relative residual and latency (ms) of instance i."""
        i = self._pos[int(i)]
        n = C.c_int32()
        self._check(self._lib.pdds_batch_instance(self._ctx, int(i), C.byref(n), None, None, None, None, None,
                                                  None, None))
        u = np.zeros(n.value)
        B = np.zeros(n.value)
        it = C.c_int32()
        rr = C.c_double()
        lat = C.c_double()
        self._check(self._lib.pdds_batch_instance(self._ctx, int(i), None, None, None, _p(u, C.c_double),
                                                  _p(B, C.c_double), C.byref(it), C.byref(rr), C.byref(lat)))
        return {"u": u, "B": B, "iterations": it.value, "rel_residual": rr.value, "latency_ms": lat.value}
