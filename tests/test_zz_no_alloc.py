"""The allocation-free interface solve, pdds_solve_bicgstab_static.

It serves callers that cannot let the library allocate GPU memory: hosts
whose device memory belongs to another allocator, serving loops where
cudaMalloc/cudaFree would synchronise or stall, foreign-language hosts that
only lend device buffers.  The test hands it caller-owned device buffers (here
allocated by torch, playing such a host) and checks its solution against the
regular entry point pdds_solve_interface and against a dense solve of the
same system, for two calls in a row on different systems (the shared static
work array must not carry state from one call into the next), and checks that
a system larger than the static limit is refused with a message.  This file is
collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

import pdds_gb300 as P
from pdds_gb300 import _capi as capi
from pdds_gb300.config import fac_rule

pytestmark = pytest.mark.gpu

ATOL = 1e-9  # the tolerance of the solver agreement test in test_gpu_parity.py


def _static_solve(lib, torch, est, K, tol):
    dev = torch.device("cuda", 0)
    rp = torch.from_numpy(np.ascontiguousarray(est.row_ptr)).to(dev)
    col = torch.from_numpy(np.ascontiguousarray(est.col)).to(dev)
    val = torch.from_numpy(np.ascontiguousarray(est.val)).to(dev)
    B = torch.from_numpy(np.ascontiguousarray(est.B)).to(dev)
    u = torch.full((K,), float("nan"), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    it = C.c_int32(0)
    rr = C.c_double(0.0)
    err = C.create_string_buffer(256)
    st = lib.pdds_solve_bicgstab_static(0, K, len(est.val), rp.data_ptr(), col.data_ptr(), val.data_ptr(),
                                        B.data_ptr(), u.data_ptr(), tol, 0, None, C.byref(it), C.byref(rr),
                                        err, 256)
    assert st == capi.OK, err.value
    return u.cpu().numpy(), it.value, rr.value


def test_static_solve_matches_regular_entry_twice():
    torch = pytest.importorskip("torch")
    lib = capi.load()
    nsub, nnode = 4, 11
    fac = fac_rule(2.0, nsub, nnode)
    tol = 1e-12
    with P.PDDSparseGM((-1.0, -1.0), (1.0, 1.0), nsub, nnode, fac) as pd:
        for seed in (11, 12):
            est = pd.estimate(P.BVP.poisson_sincos(), 2000, 1e-3, mode=P.MODE_MIXED, seed=seed)
            u_ref, info = pd.solve_interface(P.SOLVE_BICGSTAB_FP64, tol=tol)
            u_st, it, rr = _static_solve(lib, torch, est, pd.K, tol)
            assert np.all(np.isfinite(u_st))
            np.testing.assert_allclose(u_st, u_ref, rtol=0, atol=ATOL)
            assert rr <= tol and it == info["iterations"]
            # and against a dense solve of the same system, independent of
            # the BiCGSTAB kernels both entry points share
            A = np.eye(pd.K)
            r, c, v = est.triplets()
            np.add.at(A, (r, c), v)
            np.testing.assert_allclose(u_st, np.linalg.solve(A, est.B), rtol=0, atol=ATOL)


def test_static_solve_rejects_oversized_systems():
    lib = capi.load()
    err = C.create_string_buffer(256)
    dummy = C.c_void_p(1)
    st = lib.pdds_solve_bicgstab_static(0, capi.STATIC_SOLVE_MAX_K + 1, 0, dummy, None, None, dummy, dummy,
                                        1e-10, 0, None, None, None, err, 256)
    assert st == capi.ERR_INVALID
    assert b"exceeds the static solve limit" in err.value
