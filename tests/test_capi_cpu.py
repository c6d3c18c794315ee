"""CPU tests of the C-ABI library: it loads, exports every function declared
in include/pdds.h, and its host-side layout (knots, stencils, G sparsity)
equals the oracle's restatement of the reference bit for bit."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import oracle as O
from pdds_gb300 import _capi as capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from pdds_gb300 import build as B
    B.build()
    return capi.load()


def declared_functions():
    txt = open(os.path.join(ROOT, "include", "pdds.h")).read()
    return sorted(set(re.findall(r"\b(pdds_[a-z_0-9]+)\s*\(", txt)))


def test_exports_every_declared_function(lib):
    names = declared_functions()
    assert len(names) >= 11
    for n in names:
        assert hasattr(lib, n), n
    assert set(capi.EXPORTS) == set(names)


class HostLayout:
    def __init__(self, lib, sw, ne, nsub, nnode, fac):
        self.lib = lib
        self.ctx = C.c_void_p()
        assert lib.pdds_create(C.byref(self.ctx), -1, 0) == 0
        d = capi.LayoutDesc()
        d.sw[0], d.sw[1], d.ne[0], d.ne[1] = sw[0], sw[1], ne[0], ne[1]
        d.nsub, d.nnode = nsub, nnode
        for i in range(4):
            d.fac[i] = fac[i]
        self.info = capi.LayoutInfo()
        assert lib.pdds_layout_build(self.ctx, C.byref(d), C.byref(self.info)) == 0
        K = self.info.nknots
        self.x, self.y, self.order = np.zeros(K), np.zeros(K), np.zeros(K, np.int32)
        lib.pdds_layout_knots(self.ctx, self.x.ctypes.data_as(C.POINTER(C.c_double)),
                              self.y.ctypes.data_as(C.POINTER(C.c_double)),
                              self.order.ctypes.data_as(C.POINTER(C.c_int32)))
        self.rp = np.zeros(K + 1, np.int64)
        self.col = np.zeros(max(self.info.nnz, 1), np.int32)
        lib.pdds_layout_csr(self.ctx, self.rp.ctypes.data_as(C.POINTER(C.c_int64)),
                            self.col.ctypes.data_as(C.POINTER(C.c_int32)))

    def stencil(self, k, maxn=512):
        rect, kinds, sizes = np.zeros(4), np.zeros(4, np.int32), np.zeros(4, np.int32)
        idx = np.zeros(4 * maxn, np.int32)
        assert self.lib.pdds_layout_stencil(self.ctx, int(k), rect.ctypes.data_as(C.POINTER(C.c_double)),
                                            kinds.ctypes.data_as(C.POINTER(C.c_int32)),
                                            sizes.ctypes.data_as(C.POINTER(C.c_int32)),
                                            idx.ctypes.data_as(C.POINTER(C.c_int32)), maxn) == 0
        return rect, kinds, [idx[d * maxn:d * maxn + sizes[d]] for d in range(4)]

    def close(self):
        self.lib.pdds_destroy(self.ctx)


CASES = [((-5, -5), (5, 5), 4, 8), ((-1, -1), (1, 1), 4, 11), ((0, 0), (1, 1), 8, 31),
         ((-1, -1), (1, 1), 3, 5), ((0, 0), (1, 1), 5, 17), ((-1, -1), (1, 1), 12, 43)]


@pytest.mark.parametrize("sw,ne,nsub,nnode", CASES)
def test_layout_matches_oracle(lib, sw, ne, nsub, nnode):
    fac = (1.5, 1.27, 1.2, 1.13)
    H = HostLayout(lib, sw, ne, nsub, nnode, fac)
    L = O.Layout(sw, ne, nsub, nnode)
    try:
        assert H.info.nknots == L.nknots
        # hand-out order and the positions sent with the knots, bit for bit
        assert np.array_equal(H.order, L.work_idx)
        assert np.array_equal(H.x[L.work_idx], L.work_x)
        assert np.array_equal(H.y[L.work_idx], L.work_y)
        step = max(1, L.nknots // 150)
        for kn in list(L.work_idx[::step]) + [int(L.work_idx[-1])]:
            params, kinds, sides = L.stencil(int(kn))
            rect, hk, hsides = H.stencil(int(kn))
            assert np.array_equal(rect, params)
            for d in range(4):
                assert np.array_equal(hsides[d], sides[d][0]), (kn, d)
                if len(sides[d][0]):
                    assert hk[d] == kinds[d]
            # G row pattern = sorted union of side indices (empty on the boundary)
            cols = H.col[H.rp[kn]:H.rp[kn + 1]]
            union = np.unique(np.concatenate([s[0] for s in sides]))
            if len(cols):
                assert np.array_equal(cols, union)
    finally:
        H.close()


def test_sparsity_matches_recorded_run(lib):
    """The G pattern of the 4x4/8-knot layout equals the reference's G_var.csv."""
    z = np.load(os.path.join(ROOT, "tests", "golden", "ref_run_4x4_n8_monegros.npz"))
    H = HostLayout(lib, (-5, -5), (5, 5), 4, 8, (1.5, 1.27, 1.2, 1.13))
    try:
        ours = set()
        for k in range(H.info.nknots):
            for j in H.col[H.rp[k]:H.rp[k + 1]]:
                ours.add((k, int(j)))
        rec = {(int(r[0]), int(r[1])) for r in z["G_var"]}
        assert H.info.nnz == len(rec) == 6960
        assert ours == rec
        assert H.info.nboundary == 12
    finally:
        H.close()


def test_invalid_arguments_are_rejected(lib):
    ctx = C.c_void_p()
    assert lib.pdds_create(C.byref(ctx), -1, 0) == 0
    try:
        d = capi.LayoutDesc()
        d.sw[0], d.sw[1], d.ne[0], d.ne[1] = 0, 0, 1, 1
        d.nsub, d.nnode = 1, 5
        for i in range(4):
            d.fac[i] = 1.0
        assert lib.pdds_layout_build(ctx, C.byref(d), None) == capi.ERR_INVALID
        assert b"nsub" in lib.pdds_last_error(ctx)
        # estimation needs a device context
        e = capi.EstimateDesc()
        e.npaths, e.h, e.mode = 10, 1e-3, capi.MODE_MIXED
        assert lib.pdds_estimate(ctx, C.byref(e), None, None, None, None, None) == capi.ERR_INVALID
    finally:
        lib.pdds_destroy(ctx)
