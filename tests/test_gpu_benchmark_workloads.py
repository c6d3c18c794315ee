"""GPU parity on the benchmark configurations themselves, through the C ABI.

(a) Replay of the CPU-runnable configuration exactly as benchmarked: Poisson
    on [-1,1]^2, 4 x 4 subdomains, 11 knots per segment (237 knots), 1e4 paths
    per knot, h = 1e-3, Philox seed 1234, the plain method: G, G_var, B and BB
    of every knot equal the oracle's bit for bit, and so do the step and exit
    counts.
(b) Seeded statistics on the two large configurations, plain method (fixed
    step, no Richardson pair, the reference's overwrite of shared side knots),
    MIXED and FP64 against the oracle on a 16-knot seeded sample:
      Poisson 12 x 12 subdomains, 43 knots per segment, 2e4 paths, h = 5e-4;
      variable coefficients from 1024^2 FP32 tables, 8 x 8, 31 knots,
      5e4 paths (MIXED; 1e4 for the FP64 form), h = 5e-4.
    The oracle runs the reference's reduction in its linearity form (the
    same sums in another order, pinned against the faithful reduction by
    test_oracle_pins.py) on independent random streams.  Compared: B, and
    each knot's G row applied to smooth vectors (1, x, y and the exact u at
    the row's knots); their differences, divided by the Monte Carlo standard
    errors, must look like N(0, 1) samples.
"""
import numpy as np
import pytest

import oracle as O
import pdds_gb300 as P
from pdds_gb300.config import WORKLOADS, fac_rule, varcoef_tables

pytestmark = pytest.mark.gpu


def _sample(L, workload, n, seed=1234):
    """n knots of the hand-out list that run paths (seeded), by list position."""
    cx = 0.5 * (workload["sw"][0] + workload["ne"][0])
    cy = 0.5 * (workload["sw"][1] + workload["ne"][1])
    hx, hy = workload["ne"][0] - cx, workload["ne"][1] - cy
    inner = [i for i in range(len(L.work_idx))
             if abs(max(abs(L.work_x[i] - cx) - hx, abs(L.work_y[i] - cy) - hy)) > 1e-8]
    rng = np.random.default_rng(seed)
    return sorted(rng.choice(inner, size=n, replace=False).tolist())


def _functionals(L, prob, prm, kn, x0, y0, fac, phis):
    """The oracle's G row of knot kn applied to smooth vectors phi (values at
    the row's knots): S_phi = sum_j G_j phi_j, with the per-path variance of
    the sum.  Each path that leaves through interior side d scores
    -Y sum_i H_i(X) phi_i over the side knots the row takes from d (the
    reference's last-side rule); H_i are the side's cardinal functions
    (Meshes/stencil.cpp:244-307).  Individual G entries of the 84- and
    126-knot sides are dominated by a few exits with large oscillating
    weights, so their sample variances are too heavy-tailed for entry-wise
    z-scores; smooth functionals of the row are well behaved."""
    params, kinds, sides = L.stencil(kn)
    P = L.knot_paths(prob, prm, kn, x0, y0)
    assert P["status"] == 0
    N = prm.N
    owner = {}
    for d, (idx, _, _) in enumerate(sides):
        for q, v in enumerate(idx):
            owner[int(v)] = (d, q)
    dom = L.sw + L.ne
    cx, cy = 0.5 * (dom[0] + dom[2]), 0.5 * (dom[1] + dom[3])
    X, Y, W = P["x"], P["y"], P["Y"]
    glob = np.maximum(np.abs(X - cx) - (dom[2] - cx), np.abs(Y - cy) - (dom[3] - cy)) >= -1e-8
    onS = np.abs(Y - params[1]) < 1e-8
    onN = ~onS & (np.abs(Y - params[3]) < 1e-8)
    onW = ~onS & ~onN & (np.abs(X - params[0]) < 1e-8)
    onE = ~onS & ~onN & ~onW & (np.abs(X - params[2]) < 1e-8)
    vals = np.zeros((len(phis), N))
    for d, on in enumerate((onN, onS, onE, onW)):
        idx, xs, ys = sides[d]
        sel = on & ~glob
        if len(idx) == 0 or not sel.any():
            continue
        c = fac[kinds[d]]
        ip = O.ipsi(xs, ys, c)[0]
        R = np.exp(-((xs[None, :] - X[sel, None]) ** 2 + (ys[None, :] - Y[sel, None]) ** 2) / c ** 2)
        H = R @ ip  # H[e, i] = sum_j ipsi(j, i) RBF(p_j, X_e)
        keep = np.array([owner[int(v)] == (d, q) for q, v in enumerate(idx)])
        for f, phi in enumerate(phis):
            vals[f, sel] = -W[sel] * (H[:, keep] @ phi(xs[keep], ys[keep]))
    return vals.mean(axis=1), vals.var(axis=1)


PHIS = (lambda x, y: np.ones_like(x), lambda x, y: x, lambda x, y: y,
        lambda x, y: np.sin(np.pi * x) * np.cos(np.pi * y) + x * y)


def _compare(est, N_gpu, L, ref, prob, prm, fac, gx, gy):
    """z of the row functionals (oracle per-path variances, the same path
    distribution on both sides) and of B (both sides' variances)."""
    zf, zb = [], []
    for k, kn in enumerate(ref["knots"]):
        kn = int(kn)
        r0, r1 = est.row_ptr[kn], est.row_ptr[kn + 1]
        cols = est.col[r0:r1]
        a, b = ref["row_ptr"][k], ref["row_ptr"][k + 1]
        assert np.array_equal(cols, ref["gj"][a:b]), kn
        m, v = _functionals(L, prob, prm, kn, ref["x"][k], ref["y"][k], fac, PHIS)
        for f, phi in enumerate(PHIS):
            s_gpu = float(est.val[r0:r1] @ phi(gx[cols], gy[cols]))
            if v[f] > 1e-20:
                zf.append((s_gpu - m[f]) / np.sqrt(v[f] * (1.0 / N_gpu + 1.0 / prm.N)))
        vb = (est.BB[kn] - est.B[kn] ** 2) / N_gpu + (ref["BB"][k] - ref["B"][k] ** 2) / prm.N
        if vb > 1e-20:
            zb.append((est.B[kn] - ref["B"][k]) / np.sqrt(vb))
    return np.array(zf), np.array(zb)


def _assert_standard_normal(zf, zb):
    # the four functionals of a knot are correlated: about 16 independent
    # samples, so the mean and spread bounds are wide (two oracle runs with
    # independent seeds gave means -0.32..0.09 and spreads 0.75..1.10)
    assert len(zf) >= 48 and len(zb) >= 12
    assert abs(zf.mean()) < 0.6 and 0.55 < zf.std() < 1.45, (zf.mean(), zf.std())
    assert np.abs(zf).max() < 4.5 and np.abs(zb).max() < 4.5, (zf, zb)


def test_poisson_4x4_n11_replay_bit_exact_in_full():
    w = WORKLOADS["poisson_4x4_n11"]
    nsub, nnode, N, h, seed = w["nsub"], w["nnode"], w["npaths"], w["h"], 1234
    assert (nsub, nnode, N, h) == (4, 11, 10_000, 1e-3)
    fac = fac_rule(w["ne"][0] - w["sw"][0], nsub, nnode)
    L = O.Layout(w["sw"], w["ne"], nsub, nnode)
    ip, mc = O.replay_ipsi(L, fac)
    with P.PDDSparseGM(w["sw"], w["ne"], nsub, nnode, fac) as pd:
        est = pd.estimate(P.BVP.poisson_sincos(), N, h, mode=P.MODE_REPLAY_FP64, seed=seed, want_var=True,
                          ipsi_override=ip)
    ref = L.run(O.make_problem(O.POISSON_SINCOS),
                O.make_params(N, h, seed=seed, fac=fac, portable=True, sublinear=True))
    assert ref["status"] == 0 and len(ref["knots"]) == 237 and len(mc) == 225
    for k, kn in enumerate(ref["knots"]):
        kn = int(kn)
        a, b = ref["row_ptr"][k], ref["row_ptr"][k + 1]
        r0, r1 = est.row_ptr[kn], est.row_ptr[kn + 1]
        assert np.array_equal(est.col[r0:r1], ref["gj"][a:b]), kn
        assert np.array_equal(est.val[r0:r1], ref["g"][a:b]), kn
        assert np.array_equal(est.var[r0:r1], ref["gvar"][a:b]), kn
        assert est.B[kn] == ref["B"][k] and est.BB[kn] == ref["BB"][k], kn
    assert est.info["path_steps"] == ref["stats"][0]
    assert est.info["exits_global"] == ref["stats"][2]
    assert est.info["exits_stencil"] == ref["stats"][3]


def test_poisson_12x12_n43_sample_mixed_and_fp64_agree_with_oracle():
    w = WORKLOADS["poisson_12x12_n43"]
    nsub, nnode, N, h = w["nsub"], w["nnode"], w["npaths"], w["h"]
    assert (nsub, nnode, N, h) == (12, 43, 20_000, 5e-4)
    fac = fac_rule(w["ne"][0] - w["sw"][0], nsub, nnode)
    L = O.Layout(w["sw"], w["ne"], nsub, nnode)
    sel = _sample(L, w, 16)
    ref = L.run(O.make_problem(O.POISSON_SINCOS),
                O.make_params(N, h, seed=4321, fac=fac, sublinear=False, fast_reduce=True), knots=sel)
    assert ref["status"] == 0
    bvp = P.BVP.poisson_sincos()
    with P.PDDSparseGM(w["sw"], w["ne"], nsub, nnode, fac) as pd:
        mixed = pd.estimate(bvp, N, h, mode=P.MODE_MIXED, seed=1234, want_var=True)
        fp64 = pd.estimate(bvp, N, h, mode=P.MODE_FP64, seed=1234)
        gx, gy = pd.x.copy(), pd.y.copy()
    prm = O.make_params(N, h, seed=4321, fac=fac, sublinear=False, fast_reduce=True)
    for est in (mixed, fp64):
        zf, zb = _compare(est, N, L, ref, O.make_problem(O.POISSON_SINCOS), prm, fac, gx, gy)
        _assert_standard_normal(zf, zb)


def test_varcoef_lut_8x8_n31_sample_mixed_and_fp64_agree_with_oracle():
    w = WORKLOADS["varcoef_lut_8x8_n31"]
    nsub, nnode, N, h = w["nsub"], w["nnode"], w["npaths"], w["h"]
    assert (nsub, nnode, N, h, w["lut_n"]) == (8, 31, 50_000, 5e-4, 1024)
    bounds = (w["sw"][0], w["sw"][1], w["ne"][0], w["ne"][1])
    fac = fac_rule(w["ne"][0] - w["sw"][0], nsub, nnode)
    L = O.Layout(w["sw"], w["ne"], nsub, nnode)
    sel = _sample(L, w, 16)
    O.set_lut(*varcoef_tables(w["lut_n"], bounds))
    ref = L.run(O.make_problem(O.LUT), O.make_params(N, h, seed=4321, fac=fac, sublinear=False, fast_reduce=True),
                knots=sel)
    assert ref["status"] == 0
    bvp = P.BVP.varcoef_lut(w["lut_n"], bounds)
    N64 = 10_000
    with P.PDDSparseGM(w["sw"], w["ne"], nsub, nnode, fac) as pd:
        mixed = pd.estimate(bvp, N, h, mode=P.MODE_MIXED, seed=1234, want_var=True)
        fp64 = pd.estimate(bvp, N64, h, mode=P.MODE_FP64, seed=1234)
        gx, gy = pd.x.copy(), pd.y.copy()
    prm = O.make_params(N, h, seed=4321, fac=fac, sublinear=False, fast_reduce=True)
    for est, n in ((mixed, N), (fp64, N64)):
        zf, zb = _compare(est, n, L, ref, O.make_problem(O.LUT), prm, fac, gx, gy)
        _assert_standard_normal(zf, zb)


def test_many_instance_helmholtz_agree_with_oracle():
    """Four instances of the many-instance workload (Helmholtz, each on its
    own g x g grid with the step h (4/g)^2), the coarsest and finest grids
    among them: MIXED rows and B of each instance run alone, and B of the
    same instances run as one batch, against the oracle on 4 seeded knots of
    each (plain method, independent streams)."""
    from pdds_gb300.config import batch_instances
    insts = batch_instances(256, seed=1234, scaled_h=1e-3)
    order = sorted(range(len(insts)), key=lambda i: (insts[i].nsub, i))
    pick = [insts[i] for i in (order[0], order[1], order[-2], order[-1])]
    assert pick[0].nsub == 4 and pick[-1].nsub == 16
    N = 10_000
    zf_all, zb_all, zbb_all = [], [], []
    with P.Batch(P.BVP.HELMHOLTZ, pick) as bt:
        bt.run(N, 1e-3, seed=1234, instance=0, adaptive_h=False, richardson=False, use_graph=False)
        batch_B = [bt.result(i)["B"] for i in range(len(pick))]
    for q, ins in enumerate(pick):
        fac = ins.fac
        L = O.Layout(ins.sw, ins.ne, ins.nsub, ins.nnode)
        w = {"sw": ins.sw, "ne": ins.ne}
        sel = _sample(L, w, 4, seed=100 + q)
        prob = O.make_problem(O.HELMHOLTZ, *ins.params)
        prm = O.make_params(N, ins.h, seed=4321 + q, fac=fac, sublinear=False, fast_reduce=True)
        ref = L.run(prob, prm, knots=sel)
        assert ref["status"] == 0
        with P.PDDSparseGM(ins.sw, ins.ne, ins.nsub, ins.nnode, fac) as pd:
            est = pd.estimate(P.BVP.helmholtz(*ins.params), N, ins.h, mode=P.MODE_MIXED, seed=1234,
                              instance=q, want_var=True)
            gx, gy = pd.x.copy(), pd.y.copy()
        zf, zb = _compare(est, N, L, ref, prob, prm, fac, gx, gy)
        zf_all += list(zf)
        zb_all += list(zb)
        # the batch drew the same streams for instance q (word 0 + q): B as alone
        np.testing.assert_allclose(batch_B[q], est.B, rtol=0, atol=1e-5)
        for k, kn in enumerate(ref["knots"]):
            vb = (est.BB[kn] - est.B[kn] ** 2) / N + (ref["BB"][k] - ref["B"][k] ** 2) / N
            if vb > 1e-20:
                zbb_all.append((batch_B[q][kn] - ref["B"][k]) / np.sqrt(vb))
    _assert_standard_normal(np.array(zf_all), np.array(zb_all))
    assert np.abs(np.array(zbb_all)).max() < 4.5
