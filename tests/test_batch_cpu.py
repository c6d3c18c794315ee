"""Batches of instances on the host: the block-diagonal union built by
pdds_batch_build holds every instance's own layout (knots, G sparsity) bit
for bit, shifted by the knots of the instances before it."""
import ctypes as C

import numpy as np
import pytest

from pdds_gb300 import _capi as capi
from pdds_gb300.config import batch_instances, fac_rule

from test_capi_cpu import HostLayout, lib  # noqa: F401  (module fixture)

INSTANCES = [((0.0, 0.0), (1.0, 1.0), 4, 11), ((-1.0, -1.0), (1.0, 1.0), 3, 7), ((0.0, 0.0), (1.0, 1.0), 5, 9)]


def build_batch(lib, insts):
    ctx = C.c_void_p()
    assert lib.pdds_create(C.byref(ctx), -1, 0) == 0
    arr = (capi.InstanceDesc * len(insts))()
    for i, (sw, ne, ns, nn) in enumerate(insts):
        d = arr[i]
        d.layout.sw[0], d.layout.sw[1], d.layout.ne[0], d.layout.ne[1] = sw[0], sw[1], ne[0], ne[1]
        d.layout.nsub, d.layout.nnode = ns, nn
        f = fac_rule(ne[0] - sw[0], ns, nn)
        for q in range(4):
            d.layout.fac[q] = f[q]
        d.p[0] = 1.0 + i
    info = capi.BatchInfo()
    assert lib.pdds_batch_build(ctx, arr, len(insts), C.byref(info)) == 0, lib.pdds_last_error(ctx)
    return ctx, info


def test_batch_union_equals_instances(lib):
    ctx, info = build_batch(lib, INSTANCES)
    try:
        singles = [HostLayout(lib, sw, ne, ns, nn, fac_rule(ne[0] - sw[0], ns, nn)) for sw, ne, ns, nn in INSTANCES]
        assert info.ninstances == 3
        assert info.nknots == sum(h.info.nknots for h in singles)
        assert info.nnz == sum(h.info.nnz for h in singles)
        assert info.max_knots == max(h.info.nknots for h in singles)
        K = info.nknots
        rp = np.zeros(K + 1, np.int64)
        col = np.zeros(info.nnz, np.int32)
        assert lib.pdds_layout_csr(ctx, rp.ctypes.data_as(C.POINTER(C.c_int64)),
                                   col.ctypes.data_as(C.POINTER(C.c_int32))) == 0
        k0 = 0
        for i, h in enumerate(singles):
            n = C.c_int32()
            Ki = h.info.nknots
            x, y = np.zeros(Ki), np.zeros(Ki)
            assert lib.pdds_batch_instance(ctx, i, C.byref(n), x.ctypes.data_as(C.POINTER(C.c_double)),
                                           y.ctypes.data_as(C.POINTER(C.c_double)), None, None, None, None,
                                           None) == 0
            assert n.value == Ki
            assert np.array_equal(x, h.x) and np.array_equal(y, h.y)
            # the instance's rows: same lengths, columns shifted by its first knot
            assert np.array_equal(np.diff(rp[k0:k0 + Ki + 1]), np.diff(h.rp))
            e0 = rp[k0]
            assert np.array_equal(col[e0:e0 + h.info.nnz], h.col[:h.info.nnz] + k0)
            assert col[e0:e0 + h.info.nnz].min() >= k0 and col[e0:e0 + h.info.nnz].max() < k0 + Ki
            k0 += Ki
    finally:
        lib.pdds_destroy(ctx)


def test_batch_rejects_bad_input(lib):
    ctx = C.c_void_p()
    assert lib.pdds_create(C.byref(ctx), -1, 0) == 0
    try:
        arr = (capi.InstanceDesc * 1)()
        arr[0].layout.ne[0] = arr[0].layout.ne[1] = 1.0
        arr[0].layout.nsub, arr[0].layout.nnode = 4, 11
        info = capi.BatchInfo()
        assert lib.pdds_batch_build(ctx, arr, 1, C.byref(info)) == capi.ERR_INVALID  # fac = 0
        assert lib.pdds_batch_build(ctx, arr, 0, C.byref(info)) == capi.ERR_INVALID
        run = capi.BatchRunDesc()
        ri = capi.BatchRunInfo()
        assert lib.pdds_batch_run(ctx, C.byref(run), C.byref(ri)) == capi.ERR_INVALID  # no device
    finally:
        lib.pdds_destroy(ctx)


def test_many_instance_workload_is_seeded_and_in_range():
    a = batch_instances(256, seed=5)
    b = batch_instances(256, seed=5)
    assert [i.params for i in a] == [i.params for i in b]
    for ins in a:
        assert 4 <= ins.nsub <= 16 and 11 <= ins.nnode <= 41
        aa, bb, c = ins.params[:3]
        assert 1.0 <= aa <= 4.0 and 1.0 <= bb <= 4.0 and -4.0 <= c <= 0.0
