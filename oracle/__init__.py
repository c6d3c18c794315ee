"""CPU ORACLE -- TEST INFRASTRUCTURE ONLY.

ctypes binding of the plain C++ restatement of the reference PDDSparse hot
path (``oracle/*.cpp``).  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import this package; the product library
``pdds_gb300`` never does.

Parity status: pinned against the reference's own recorded run
(``Output/Debug/{cond.txt,G.csv,B.csv,G_var.csv,B_var.csv}``, ``Output/solution.csv``)
through the fixtures in ``tests/golden/``.  The reference itself cannot be
compiled here (Eigen3, GSL, Boost.Random and MPI are absent).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")

POISSON_SINCOS, MONEGROS, HELMHOLTZ, VARCOEF, LUT = 0, 1, 2, 3, 4
DIAG_N = 18  # diagnostic sums per knot (orc_run_diag)


class Problem(C.Structure):
    _fields_ = [("kind", C.c_int), ("p", C.c_double * 8)]


class Params(C.Structure):
    _fields_ = [
        ("N", C.c_int),
        ("h", C.c_double),
        ("seed", C.c_uint64),
        ("instance", C.c_uint32),
        ("portable", C.c_int),
        ("sublinear", C.c_int),
        ("dup_sum", C.c_int),
        ("threads", C.c_int),
        ("fac", C.c_double * 4),
        ("max_steps", C.c_int64),
        ("adaptive_h", C.c_int),
        ("fast_reduce", C.c_int),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++, OpenMP, no FMA contraction)."""
    if force or not os.path.exists(_LIB_PATH):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    else:
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        vp, ip, dp, i64p = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_int64)
        L.orc_layout_new.restype = vp
        L.orc_layout_new.argtypes = [C.c_double] * 4 + [C.c_int, C.c_int]
        L.orc_layout_free.argtypes = [vp]
        L.orc_layout_nknots.argtypes = [vp]
        L.orc_layout_nwork.argtypes = [vp]
        L.orc_layout_work.argtypes = [vp, ip, dp, dp]
        L.orc_layout_ninterfaces.argtypes = [vp]
        L.orc_layout_interface.argtypes = [vp, C.c_int, ip, ip, dp, dp]
        L.orc_stencil.argtypes = [vp, C.c_int, dp, ip, ip, ip, dp, dp, C.c_int]
        L.orc_ipsi.argtypes = [C.c_int, dp, dp, C.c_double, dp, dp]
        L.orc_ipsi_ex.argtypes = [C.c_int, dp, dp, C.c_double, C.c_int, dp, dp]
        L.orc_knot.argtypes = [vp, C.POINTER(Problem), C.POINTER(Params), C.c_int, C.c_double,
                               C.c_double, dp, ip, dp, dp, C.c_int, ip, dp, dp, i64p]
        L.orc_knot_paths.argtypes = [vp, C.POINTER(Problem), C.POINTER(Params), C.c_int, C.c_double,
                                     C.c_double, dp, dp, dp, dp, dp, C.POINTER(C.c_int32),
                                     C.POINTER(C.c_int32)]
        L.orc_run.argtypes = [vp, C.POINTER(Problem), C.POINTER(Params), ip, dp, dp, C.c_int, ip,
                              ip, dp, dp, C.c_int64, dp, dp, i64p]
        L.orc_run_diag.argtypes = [vp, C.POINTER(Problem), C.POINTER(Params), ip, dp, dp, C.c_int, dp]
        L.orc_bicgstab.argtypes = [C.c_int, C.c_int64, ip, ip, dp, dp, dp, C.c_int, C.c_double, ip, dp]
        L.orc_set_lut.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int, C.c_int, dp]
        L.orc_problem_u.restype = C.c_double
        L.orc_problem_u.argtypes = [C.POINTER(Problem), C.c_double, C.c_double]
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def make_problem(kind: int, *params: float) -> Problem:
    p = Problem()
    p.kind = kind
    for i, v in enumerate(params):
        p.p[i] = v
    return p


def make_params(N, h, seed=1234, fac=(1.0, 1.0, 1.0, 1.0), portable=False, sublinear=True,
                dup_sum=False, threads=None, instance=0, max_steps=10**8, adaptive_h=False,
                fast_reduce=False) -> Params:
    prm = Params()
    prm.N = int(N)
    prm.h = float(h)
    prm.seed = int(seed)
    prm.instance = int(instance)
    prm.portable = int(bool(portable))
    prm.sublinear = int(bool(sublinear))
    prm.dup_sum = int(bool(dup_sum))
    prm.threads = int(threads if threads else (os.cpu_count() or 1))
    for i in range(4):
        prm.fac[i] = float(fac[i])
    prm.max_steps = int(max_steps)
    prm.adaptive_h = int(bool(adaptive_h))
    prm.fast_reduce = int(bool(fast_reduce))
    return prm


class Layout:
    """Fullfill_interfaces + Compute_Stencil restatement (PDDSparseGM.cpp:346-689, 1845-2041)."""

    def __init__(self, sw, ne, nsub: int, nnode: int):
        L = lib()
        self._h = L.orc_layout_new(float(sw[0]), float(sw[1]), float(ne[0]), float(ne[1]),
                                   int(nsub), int(nnode))
        if not self._h:
            raise ValueError("invalid layout")
        self.sw, self.ne, self.nsub, self.nnode = tuple(sw), tuple(ne), nsub, nnode
        self.nknots = L.orc_layout_nknots(self._h)
        nw = L.orc_layout_nwork(self._h)
        self.work_idx = np.zeros(nw, np.int32)
        self.work_x = np.zeros(nw)
        self.work_y = np.zeros(nw)
        L.orc_layout_work(self._h, _p(self.work_idx, C.c_int), _p(self.work_x, C.c_double),
                          _p(self.work_y, C.c_double))

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.orc_layout_free(self._h)
            self._h = None

    def interfaces(self):
        L = lib()
        out = []
        for i in range(L.orc_layout_ninterfaces(self._h)):
            lab = np.zeros(2, np.int32)
            n = L.orc_layout_interface(self._h, i, _p(lab, C.c_int), None, None, None)
            idx = np.zeros(n, np.int32)
            x = np.zeros(n)
            y = np.zeros(n)
            L.orc_layout_interface(self._h, i, _p(lab, C.c_int), _p(idx, C.c_int),
                                   _p(x, C.c_double), _p(y, C.c_double))
            out.append((tuple(int(v) for v in lab), idx, x, y))
        return out

    def stencil(self, knot: int, maxn: int = 1024):
        params = np.zeros(4)
        kinds = np.zeros(4, np.int32)
        sizes = np.zeros(4, np.int32)
        idx = np.zeros(4 * maxn, np.int32)
        x = np.zeros(4 * maxn)
        y = np.zeros(4 * maxn)
        rc = lib().orc_stencil(self._h, int(knot), _p(params, C.c_double), _p(kinds, C.c_int),
                               _p(sizes, C.c_int), _p(idx, C.c_int), _p(x, C.c_double),
                               _p(y, C.c_double), maxn)
        if rc != 0:
            raise ValueError("stencil side larger than maxn")
        sides = []
        for d in range(4):
            n = int(sizes[d])
            sides.append((idx[d * maxn:d * maxn + n].copy(), x[d * maxn:d * maxn + n].copy(),
                          y[d * maxn:d * maxn + n].copy()))
        return params, kinds, sides

    def knot(self, problem: Problem, prm: Params, knot: int, x0: float, y0: float, ipsi=None,
             maxnnz: int = 4096):
        gj = np.zeros(maxnnz, np.int32)
        g = np.zeros(maxnnz)
        gv = np.zeros(maxnnz)
        nnz = C.c_int(0)
        B = C.c_double(0)
        BB = C.c_double(0)
        st = np.zeros(4, np.int64)
        ip = None if ipsi is None else _p(np.ascontiguousarray(ipsi, dtype=np.float64), C.c_double)
        rc = lib().orc_knot(self._h, C.byref(problem), C.byref(prm), int(knot), float(x0), float(y0),
                            ip, _p(gj, C.c_int), _p(g, C.c_double), _p(gv, C.c_double), maxnnz,
                            C.byref(nnz), C.byref(B), C.byref(BB), _p(st, C.c_int64))
        n = nnz.value
        return dict(status=rc, gj=gj[:n], g=g[:n], gvar=gv[:n], B=B.value, BB=BB.value, stats=st)

    def knot_paths(self, problem: Problem, prm: Params, knot: int, x0: float, y0: float):
        N = prm.N
        a = {k: np.zeros(N) for k in ("x", "y", "Y", "Z", "xi")}
        sl = np.zeros(N, np.int32)
        ss = np.zeros(N, np.int32)
        rc = lib().orc_knot_paths(self._h, C.byref(problem), C.byref(prm), int(knot), float(x0),
                                  float(y0), *[_p(a[k], C.c_double) for k in ("x", "y", "Y", "Z", "xi")],
                                  _p(sl, C.c_int32), _p(ss, C.c_int32))
        a["steps_l"] = sl
        a["steps_s"] = ss
        a["status"] = rc
        return a

    def run(self, problem: Problem, prm: Params, knots=None, maxnnz_per_row: int = 1024):
        """All knots of the hand-out list (or a subset of its positions), in order."""
        sel = np.arange(len(self.work_idx)) if knots is None else np.asarray(knots)
        kn = np.ascontiguousarray(self.work_idx[sel], np.int32)
        x0 = np.ascontiguousarray(self.work_x[sel])
        y0 = np.ascontiguousarray(self.work_y[sel])
        nk = len(kn)
        cap = nk * maxnnz_per_row
        rp = np.zeros(nk + 1, np.int32)
        gj = np.zeros(cap, np.int32)
        g = np.zeros(cap)
        gv = np.zeros(cap)
        B = np.zeros(nk)
        BB = np.zeros(nk)
        st = np.zeros(4, np.int64)
        rc = lib().orc_run(self._h, C.byref(problem), C.byref(prm), _p(kn, C.c_int), _p(x0, C.c_double),
                           _p(y0, C.c_double), nk, _p(rp, C.c_int), _p(gj, C.c_int), _p(g, C.c_double),
                           _p(gv, C.c_double), cap, _p(B, C.c_double), _p(BB, C.c_double),
                           _p(st, C.c_int64))
        nnz = int(rp[-1])
        return dict(status=rc, knots=kn, x=x0, y=y0, row_ptr=rp, gj=gj[:nnz], g=g[:nnz],
                    gvar=gv[:nnz], B=B, BB=BB, stats=st)

    def run_diag(self, problem: Problem, prm: Params, knots=None):
        """Diagnostic sums of Reduce_Analytic per knot of the hand-out list (or
        a subset of its positions): (status, knots, sums [nk, DIAG_N])."""
        sel = np.arange(len(self.work_idx)) if knots is None else np.asarray(knots)
        kn = np.ascontiguousarray(self.work_idx[sel], np.int32)
        x0 = np.ascontiguousarray(self.work_x[sel])
        y0 = np.ascontiguousarray(self.work_y[sel])
        sums = np.zeros((len(kn), DIAG_N))
        rc = lib().orc_run_diag(self._h, C.byref(problem), C.byref(prm), _p(kn, C.c_int), _p(x0, C.c_double),
                                _p(y0, C.c_double), len(kn), _p(sums, C.c_double))
        return rc, kn, sums


def ipsi(x, y, c, portable=False):
    n = len(x)
    out = np.zeros((n, n))
    cond = C.c_double(0)
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    rank = lib().orc_ipsi_ex(n, _p(x, C.c_double), _p(y, C.c_double), float(c), int(bool(portable)),
                             _p(out, C.c_double), C.byref(cond))
    return out, cond.value, rank


def replay_ipsi(layout: "Layout", fac, portable=True):
    """RBF inverses of every knot that runs paths, packed for the library's
    replay mode: knots in hand-out order, sides N,S,E,W, each n x n row-major
    ipsi(j,i) -- exactly the matrices this oracle uses in portable mode."""
    blocks, mc = [], []
    cache = {}
    for kn, x0, y0 in zip(layout.work_idx, layout.work_x, layout.work_y):
        params, kinds, sides = layout.stencil(int(kn))
        # boundary knots (B = g) run no paths
        cx, cy = 0.5 * (layout.sw[0] + layout.ne[0]), 0.5 * (layout.sw[1] + layout.ne[1])
        hx, hy = layout.ne[0] - cx, layout.ne[1] - cy
        if abs(max(abs(x0 - cx) - hx, abs(y0 - cy) - hy)) <= 1e-8:
            continue
        mc.append(int(kn))
        for d in range(4):
            idx, xs, ys = sides[d]
            if len(idx) == 0:
                continue
            key = (tuple(idx.tolist()), int(kinds[d]))
            if key not in cache:
                cache[key] = ipsi(xs, ys, fac[kinds[d]], portable=portable)[0]
            blocks.append(cache[key].ravel())
    return np.concatenate(blocks) if blocks else np.zeros(0), mc


def bicgstab(K, rows, cols, vals, b, maxit=None, tol=2.220446049250313e-16):
    rows = np.ascontiguousarray(rows, np.int32)
    cols = np.ascontiguousarray(cols, np.int32)
    vals = np.ascontiguousarray(vals, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    x = np.zeros(K)
    it = C.c_int(0)
    err = C.c_double(0)
    lib().orc_bicgstab(int(K), len(vals), _p(rows, C.c_int), _p(cols, C.c_int), _p(vals, C.c_double),
                       _p(b, C.c_double), _p(x, C.c_double), int(maxit if maxit else 2 * K), float(tol),
                       C.byref(it), C.byref(err))
    return x, it.value, err.value


def set_lut(coef, g, bounds):
    """Tables of the LUT problem (coef [ny][nx][8], g [ny][nx] float32)."""
    coef = np.ascontiguousarray(coef, np.float32)
    g = np.ascontiguousarray(g, np.float32)
    b = np.ascontiguousarray(bounds, np.float64)
    ny, nx = g.shape
    lib().orc_set_lut(_p(coef, C.c_float), _p(g, C.c_float), nx, ny, _p(b, C.c_double))


def problem_u(problem: Problem, x, y):
    f = lib().orc_problem_u
    return np.array([f(C.byref(problem), float(a), float(b)) for a, b in zip(np.ravel(x), np.ravel(y))])
