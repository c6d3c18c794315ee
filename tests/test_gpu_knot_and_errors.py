"""The per-knot call and the error statuses, on the GPU through the C ABI.

Per-knot call (EMFKACSolver::Solve_OMP_Analytic, Solvers/EMFKACSolver.hpp:711-729):
  * one knot from its caller-built stencil in the replay mode equals the
    oracle's knot bit for bit, through the Python mirror and through the C++
    shim (pdds::EMFKACSolver::Solve_GPU_Analytic), boundary knots included;
  * the same knot in the MIXED mode equals its row of the all-knot estimate
    (same Philox streams) up to FP32 summation order;
  * a layout rebuilt from its knots' stencils gives the estimate and the
    interface solution of the built layout.
Error statuses (the reference prints and continues, or blocks on getchar()):
  * PDDS_ERR_TIMEOUT: a grid-barrier wait of the interface solve given a
    poll limit of one runs out; the kernel winds down and the context keeps
    working;
  * PDDS_ERR_NOT_CONVERGED: an iteration cap of one;
  * PDDS_ERR_ILL_CONDITIONED: a stencil side with two coincident knots makes
    its RBF matrix singular (Meshes/stencil.cpp:159-164 prints "FATAL");
  * PDDS_ERR_EXIT_SIDE: a drift that is not a number sends paths to a
    position on no side (the reference's G_update either matches a side by
    the other coordinate and returns weights that are not numbers, or
    blocks on getchar(), stencil.cpp:302-305).
"""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
import pdds_gb300 as P
from pdds_gb300 import _capi as capi
from pdds_gb300.config import fac_rule

pytestmark = pytest.mark.gpu

SW, NE, NSUB, NNODE = (-1.0, -1.0), (1.0, 1.0), 4, 11
DOMAIN = (SW[0], SW[1], NE[0], NE[1])
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _oracle_knot(L, fac, pos):
    """Stencil, oracle inverses (portable exponentials) of the knot at
    hand-out position pos: (knot, x0, y0, Stencil, ipsi blocks N,S,E,W)."""
    kn, x0, y0 = int(L.work_idx[pos]), float(L.work_x[pos]), float(L.work_y[pos])
    params, kinds, sides = L.stencil(kn)
    st = P.Stencil(params, DOMAIN)
    st.Init({d: s[0] for d, s in zip("NSEW", sides)}, {d: s[1] for d, s in zip("NSEW", sides)},
            {d: s[2] for d, s in zip("NSEW", sides)}, params)
    st.Compute_ipsi([fac[k] if k >= 0 else 1.0 for k in kinds])
    cx, cy = 0.5 * (DOMAIN[0] + DOMAIN[2]), 0.5 * (DOMAIN[1] + DOMAIN[3])
    on_boundary = abs(max(abs(x0 - cx) - (DOMAIN[2] - cx), abs(y0 - cy) - (DOMAIN[3] - cy))) <= 1e-8
    # boundary knots run no paths and take no inverses (B = g)
    blocks = [] if on_boundary else [O.ipsi(s[1], s[2], fac[k], portable=True)[0].ravel()
                                     for s, k in zip(sides, kinds) if len(s[0])]
    return kn, x0, y0, st, np.concatenate(blocks) if blocks else None, sides, kinds


@pytest.fixture(scope="module")
def poisson_4x4():
    fac = fac_rule(2.0, NSUB, NNODE)
    return O.Layout(SW, NE, NSUB, NNODE), fac


def test_single_knot_replay_bit_exact(poisson_4x4):
    L, fac = poisson_4x4
    N, h, seed = 300, 1e-3, 1234
    prob = O.make_problem(O.POISSON_SINCOS)
    prm = O.make_params(N, h, seed=seed, fac=fac, portable=True, sublinear=True)
    with P.EMFKACSolver() as sv:
        for pos in (0, 3, 17, 60, 118, 200, 236):
            kn, x0, y0, st, ip, _, _ = _oracle_knot(L, fac, pos)
            G, Gv, Gj, B, BB = sv.Solve_GPU_Analytic((x0, y0), N, h, 0.0, P.BVP.poisson_sincos(), st,
                                                     mode=P.MODE_REPLAY_FP64, seed=seed, knot_id=kn,
                                                     ipsi_override=ip)
            ref = L.knot(prob, prm, kn, x0, y0)
            assert ref["status"] == 0
            np.testing.assert_array_equal(Gj, ref["gj"])
            assert np.array_equal(G, ref["g"]) and np.array_equal(Gv, ref["gvar"]), kn
            assert B == ref["B"] and BB == ref["BB"], kn


def test_single_knot_replay_bit_exact_through_the_cpp_shim(poisson_4x4, tmp_path):
    from pdds_gb300 import build as Bld
    import shutil
    lib = Bld.build()
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "pdds_cpp_check")
    cuda_lib = "/usr/local/cuda/lib64"
    res = subprocess.run([cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                          os.path.join(ROOT, "tests", "cpp", "pdds_cpp_check.cpp"), "-o", exe, lib,
                          "-Wl,-rpath," + os.path.dirname(lib), "-L" + cuda_lib, "-Wl,-rpath," + cuda_lib,
                          "-lcudart"], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    L, fac = poisson_4x4
    N, h, seed = 256, 1e-3, 77
    prm = O.make_params(N, h, seed=seed, fac=fac, portable=True, sublinear=True)
    for pos in (5, 131):
        kn, x0, y0, st, ip, sides, kinds = _oracle_knot(L, fac, pos)
        lines = [f"{x0!r} {y0!r} {kn}", " ".join(repr(v) for v in DOMAIN),
                 " ".join(repr(float(v)) for v in st.stencil_parameters), f"{N} {h!r} {seed}"]
        for (idx, xs, ys), k in zip(sides, kinds):
            lines.append(f"{len(idx)} {fac[k] if k >= 0 else 1.0!r}")
            lines += [f"{int(i)} {float(a)!r} {float(b)!r}" for i, a, b in zip(idx, xs, ys)]
        lines.append(" ".join(repr(float(v)) for v in ip) if ip is not None else "")
        f = tmp_path / f"knot{pos}.txt"
        f.write_text("\n".join(lines) + "\n")
        out = subprocess.run([exe, "knot", str(f)], capture_output=True, text=True, timeout=300)
        assert out.returncode == 0, out.stderr
        rows = out.stdout.strip().splitlines()
        head = rows[0].split()
        B, BB, nnz = float.fromhex(head[1]), float.fromhex(head[3]), int(head[5])
        gj = np.array([int(r.split()[0]) for r in rows[1:]])
        g = np.array([float.fromhex(r.split()[1]) for r in rows[1:]])
        gv = np.array([float.fromhex(r.split()[2]) for r in rows[1:]])
        ref = L.knot(O.make_problem(O.POISSON_SINCOS), prm, kn, x0, y0)
        assert nnz == len(ref["gj"])
        np.testing.assert_array_equal(gj, ref["gj"])
        assert np.array_equal(g, ref["g"]) and np.array_equal(gv, ref["gvar"])
        assert B == ref["B"] and BB == ref["BB"]


def test_single_knot_mixed_equals_its_row_of_the_layout_estimate():
    fac = fac_rule(2.0, NSUB, NNODE)
    bvp = P.BVP.poisson_sincos()
    N, h = 4096, 1e-3
    with P.PDDSparseGM(SW, NE, NSUB, NNODE, fac) as pd, P.EMFKACSolver() as sv:
        est = pd.estimate(bvp, N, h, mode=P.MODE_MIXED, seed=31, want_var=True)
        for k in (int(pd.order[20]), int(pd.order[150])):
            st = P.Stencil.of_knot(pd, k)
            G, Gv, Gj, B, BB = sv.Solve_GPU_Analytic((pd.x[k], pd.y[k]), N, h, 0.0, bvp, st, mode=P.MODE_MIXED,
                                                     seed=31, knot_id=k)
            r0, r1 = est.row_ptr[k], est.row_ptr[k + 1]
            np.testing.assert_array_equal(Gj, est.col[r0:r1])
            np.testing.assert_allclose(G, est.val[r0:r1], rtol=1e-4, atol=1e-7)
            np.testing.assert_allclose(B, est.B[k], rtol=1e-6, atol=1e-9)
        # a knot on the domain boundary: B = g(X0), no row
        kb = int(np.flatnonzero(np.isclose(np.abs(pd.x), 1.0))[0])
        st = P.Stencil.of_knot(pd, kb)
        G, Gv, Gj, B, BB = sv.Solve_GPU_Analytic((pd.x[kb], pd.y[kb]), N, h, 0.0, bvp, st, mode=P.MODE_MIXED,
                                                 knot_id=kb)
        assert len(G) == 0 and abs(B - bvp.u(pd.x[kb], pd.y[kb])) < 1e-12 and abs(BB - B * B) < 1e-12


def test_layout_rebuilt_from_stencils_estimates_and_solves_the_same():
    fac = fac_rule(2.0, NSUB, NNODE)
    bvp = P.BVP.poisson_sincos()
    N, h = 4096, 1e-3
    with P.PDDSparseGM(SW, NE, NSUB, NNODE, fac) as pd:
        sts = [P.Stencil.of_knot(pd, k) for k in range(pd.K)]
        a = pd.estimate(bvp, N, h, mode=P.MODE_MIXED, seed=8)
        ua, _ = pd.solve_interface(P.SOLVE_BICGSTAB_FP64, tol=1e-12)
        with P.PDDSparseGM.from_stencils(DOMAIN, pd.x, pd.y, sts) as q:
            b = q.estimate(bvp, N, h, mode=P.MODE_MIXED, seed=8)
            ub, _ = q.solve_interface(P.SOLVE_BICGSTAB_FP64, tol=1e-12)
    np.testing.assert_array_equal(a.col, b.col)
    np.testing.assert_allclose(b.val, a.val, rtol=1e-4, atol=1e-7)
    np.testing.assert_allclose(b.B, a.B, rtol=1e-6, atol=1e-9)
    assert a.info["path_steps"] == b.info["path_steps"]
    np.testing.assert_allclose(ub, ua, rtol=0, atol=1e-6)


def test_grid_barrier_timeout_is_reported_and_the_context_survives():
    nsub, nnode = 12, 21  # 5,181 knots: the solve runs over the whole GPU
    fac = fac_rule(2.0, nsub, nnode)
    with P.PDDSparseGM(SW, NE, nsub, nnode, fac) as pd:
        assert pd.K >= 4096
        pd.estimate(P.BVP.poisson_sincos(), 256, 1e-3, mode=P.MODE_MIXED, seed=3)
        with pytest.raises(P.PDDSError) as e:
            pd.solve_interface(P.SOLVE_GMRES_FP32_IR, tol=1e-10, barrier_poll_limit=1)
        assert e.value.status == capi.ERR_TIMEOUT
        u, info = pd.solve_interface(P.SOLVE_GMRES_FP32_IR, tol=1e-10)
        u2, _ = pd.solve_interface(P.SOLVE_BICGSTAB_FP64, tol=1e-12)
        assert info["rel_residual"] <= 1e-10
        np.testing.assert_allclose(u, u2, rtol=0, atol=1e-8)
        with pytest.raises(P.PDDSError):
            pd.solve_interface(P.SOLVE_GMRES_FP32_IR, barrier_poll_limit=-1)


def test_iteration_cap_reports_not_converged():
    fac = fac_rule(2.0, NSUB, NNODE)
    with P.PDDSparseGM(SW, NE, NSUB, NNODE, fac) as pd:
        pd.estimate(P.BVP.poisson_sincos(), 512, 1e-3, mode=P.MODE_MIXED)
        for method in (P.SOLVE_BICGSTAB_FP64, P.SOLVE_GMRES_FP32_IR):
            with pytest.raises(P.PDDSError) as e:
                pd.solve_interface(method, tol=1e-14, max_iter=1, max_refine=1)
            assert e.value.status == capi.ERR_NOT_CONVERGED
        u, info = pd.solve_interface(P.SOLVE_GMRES_FP32_IR, tol=1e-10)
        assert info["rel_residual"] <= 1e-10


def test_coincident_side_knots_report_ill_conditioned():
    fac = fac_rule(2.0, NSUB, NNODE)
    with P.PDDSparseGM(SW, NE, NSUB, NNODE, fac) as pd, P.EMFKACSolver() as sv:
        k = int(pd.order[40])
        good = P.Stencil.of_knot(pd, k)
        bad = P.Stencil.of_knot(pd, k)
        d = next(d for d in "NSEW" if len(bad.index[d]) > 3)
        # the second knot of the side moved onto the first: two equal rows of Psi
        bad.x[d] = bad.x[d].copy()
        bad.y[d] = bad.y[d].copy()
        bad.x[d][1], bad.y[d][1] = bad.x[d][0], bad.y[d][0]
        for mode in (P.MODE_MIXED, P.MODE_FP64):
            with pytest.raises(P.PDDSError) as e:
                sv.Solve_GPU_Analytic((pd.x[k], pd.y[k]), 256, 1e-3, 0.0, P.BVP.poisson_sincos(), bad, mode=mode,
                                      knot_id=k)
            assert e.value.status == capi.ERR_ILL_CONDITIONED
        G, Gv, Gj, B, BB = sv.Solve_GPU_Analytic((pd.x[k], pd.y[k]), 256, 1e-3, 0.0, P.BVP.poisson_sincos(), good,
                                                 mode=P.MODE_MIXED, knot_id=k)
        assert np.all(np.isfinite(G)) and np.isfinite(B)


def test_positions_that_are_not_numbers_report_exit_side():
    from pdds_gb300.config import varcoef_tables
    nsub, nnode = 3, 6
    bounds = (0.0, 0.0, 1.0, 1.0)
    coef, g, b = varcoef_tables(64, bounds)
    bad = coef.copy()
    bad[..., 2] = np.nan  # drift b1: every step lands on a position that is not a number
    fac = fac_rule(1.0, nsub, nnode)
    with P.PDDSparseGM((0.0, 0.0), (1.0, 1.0), nsub, nnode, fac) as pd:
        bvp_bad = P.BVP.lut(bad, g, b)
        for mode in (P.MODE_MIXED, P.MODE_FP64, P.MODE_REPLAY_FP64):
            with pytest.raises(P.PDDSError) as e:
                pd.estimate(bvp_bad, 128, 1e-3, mode=mode)
            assert e.value.status == capi.ERR_EXIT_SIDE, mode
        est = pd.estimate(P.BVP.lut(coef, g, b), 128, 1e-3, mode=P.MODE_MIXED)
        assert np.all(np.isfinite(est.val)) and np.all(np.isfinite(est.B))
