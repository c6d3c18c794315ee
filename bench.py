"""Benchmark of the GB300 PDDSparse hot path (one JSON line on rank 0).

A step is one pass of the hot path over one batch of synthetic input: the
RBF factorisation of the stencil sides, the Feynman-Kac estimation of every
knot's G row and B entry, and the interface solve (I + G) u = B, on the
12x12-subdomain / 43-knot Poisson workload (10,989 knots, 2e4 paths per knot,
h = 5e-4) in the MIXED form (FP32 paths, FP64 accumulation, FP64 RBF
factorisation, FP32 GMRES under FP64 refinement) with the per-knot adaptive
step and the Richardson pair (h/2, h) that bring the interface RMSE under
2e-3.  The same step without them (the reference's plain method) and the
plain FP64 GPU form are measured beside it.

  value  path-steps/s of the device-timed step (inputs resident in HBM),
         CUDA events on the library's stream, L2 flushed between steps
  e2e    the same metric through the public API call a user makes: a new
         context with the layout built on the host and uploaded, estimation,
         solve, and G/B/u copied back to host, every step (after the same
         warm-up steps as the device-timed step)
  roofline  FP32 issue-slot roof of the path kernel (the path is issue-bound:
         it reads a few MB of stencil tables and no large arrays)
  cpu_baseline  the CPU restatement of the reference (OpenMP paths, serial
         O(n_s^2) reduction), on a bounded sample of knots of the same workload

--impl reference runs the reference's CPU algorithm (the restatement, all host
threads) on the same workload and prints the same metric.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "path-steps/s & interface solves/s at RMSE<=2e-3, mixed+batched vs plain FP64"

# Algorithmic thread-instruction counts (fixed before tuning, counted from the
# algorithm, not from the compiler): one Euler-Maruyama step = half a
# Philox-4x32-10 call (10 rounds of 2 wide multiplies and 2 three-way XORs,
# 40 INT) + Box-Muller (2 converts, log, sqrt, sin, cos, 4 FP32: 10) +
# Poisson coefficients (sin/cos of pi x and pi y, source, gradient: 14) +
# control-variate update and state update (14) + rectangle distance and
# projection (12) + Gobet-shifted exit test (4) = 94.  One exit = side
# classification and projection (10) + cubic weights and 4 shared-memory
# deposits (16) + B accumulation in FP64 (6) + refill (10) = 42.  The G
# contraction adds one FMA per (bin, side knot) pair per knot.
W_STEP = 94
W_EXIT = 42

# DRAM bytes (read + write) of one k_paths_mixed launch, from one ncu capture
# of the same workload (dram__bytes_read.sum + dram__bytes_write.sum); the
# captures and their commands are summarised under profiles/.
PATH_KERNEL_DRAM_BYTES = {
    "poisson_12x12_n43": 35_996_672,
}


def knot_residual_rms(est, exact):
    """RMS over the knots with paths of B_k - u_k - sum_j G_kj u_j at the exact
    solution u: the per-knot error of the estimated system (bias and Monte
    Carlo noise) that the interface solve turns into the solution error."""
    rows = np.repeat(np.arange(len(est.row_ptr) - 1), np.diff(est.row_ptr))
    gu = np.zeros(len(est.row_ptr) - 1)
    np.add.at(gu, rows, est.val * exact[est.col])
    mc = np.diff(est.row_ptr) > 0
    r = est.B - exact - gu
    return float(np.sqrt(np.mean(r[mc] ** 2)))


def poisson_sincos_u(x, y):
    return np.sin(np.pi * x) * np.cos(np.pi * y) + x * y


def _env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [q.strip() for q in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1].split()[0]))
                smax.append(float(p[2].split()[0]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def cpu_baseline(workload: dict, fac, n_knots: int, seed: int = 1234, npaths=None, fast: bool = False):
    """The reference's CPU path restated (oracle): OpenMP over paths with every
    host core, serial O(n_s^2) reduction, libm, per-knot factorisation; on a
    fixed random sample of knots of the workload (seed 1234).  fast: the
    linearity form of the reduction (n_s exponentials per exit, exits reduced
    in parallel) instead of the reference's, a faster CPU form shown beside."""
    import oracle as O
    L = O.Layout(workload["sw"], workload["ne"], workload["nsub"], workload["nnode"])
    rng = np.random.default_rng(seed)
    # sample among knots that run paths
    cx = 0.5 * (workload["sw"][0] + workload["ne"][0])
    cy = 0.5 * (workload["sw"][1] + workload["ne"][1])
    hx, hy = workload["ne"][0] - cx, workload["ne"][1] - cy
    inner = [i for i in range(len(L.work_idx))
             if abs(max(abs(L.work_x[i] - cx) - hx, abs(L.work_y[i] - cy) - hy)) > 1e-8]
    sel = sorted(rng.choice(inner, size=min(n_knots, len(inner)), replace=False).tolist())
    N = npaths or workload["npaths"]
    threads = os.cpu_count() or 1
    prm = O.make_params(N, workload["h"], seed=seed, fac=fac, sublinear=True, threads=threads, fast_reduce=fast)
    if workload.get("problem") == "varcoef_lut":
        from pdds_gb300.config import varcoef_tables
        O.set_lut(*varcoef_tables(workload["lut_n"], (workload["sw"][0], workload["sw"][1],
                                                      workload["ne"][0], workload["ne"][1])))
        prob = O.make_problem(O.LUT)
    else:
        prob = O.make_problem(O.POISSON_SINCOS)
    t0 = time.perf_counter()
    res = L.run(prob, prm, knots=sel)
    dt = time.perf_counter() - t0
    steps = int(res["stats"][0])
    # per-knot residual of the estimated rows at the exact solution
    kx, ky = np.zeros(L.nknots), np.zeros(L.nknots)
    kx[L.work_idx], ky[L.work_idx] = L.work_x, L.work_y
    if workload.get("problem") == "varcoef_lut":
        u = np.exp(kx) * np.cos(2 * ky) + 1.0
    else:
        u = poisson_sincos_u(kx, ky)
    r = []
    for k, kn in enumerate(res["knots"]):
        a, b = res["row_ptr"][k], res["row_ptr"][k + 1]
        r.append(res["B"][k] - u[kn] - float(res["g"][a:b] @ u[res["gj"][a:b]]))
    return {"value": steps / dt, "unit": "path-steps/s", "cores": threads, "kind": "port",
            "sample": f"{len(sel)} random knots (seed {seed}) of {workload['name']}, {N} paths each, "
                      f"{steps} path steps in {dt:.2f} s",
            "seconds": dt, "knots": len(sel), "path_steps": steps, "residuals": r}


def many_instance_batch(local: int, n_inst: int = 256, reps: int = 3, npaths: int = 10_000, h: float = 1e-3):
    """256 independent Helmholtz instances on [0,1]^2 (random g x g grids,
    g in 4..16, 11..41 knots per segment, a, b ~ U[1,4], c ~ U[-4,0]),
    1e4 paths per knot, h = 1e-3 at 4 x 4 and h (4/g)^2 on finer grids, MIXED
    with the adaptive step and the Richardson pair (as the headline step),
    every instance solved by the cluster GMRES; the instances run smallest
    first in 16 groups whose solves overlap the next group's paths (the given
    order is timed too); the sequence is one CUDA graph, replayed with a new
    Philox instance word each run.  The plain method (no Richardson) is timed
    too."""
    import pdds_gb300 as P
    from pdds_gb300.config import batch_instances
    # each instance's step scaled with the square of its subdomain size: h at
    # 4 x 4, h (4/g)^2 at g x g (the same steps per path and step-to-subdomain
    # ratio everywhere; with one h for all, the bias on the finest grids
    # exceeded the 2e-3 target)
    insts = batch_instances(n_inst, seed=1234, scaled_h=h)
    # latency with the instances in the given (random) order
    g0 = P.Batch(P.BVP.HELMHOLTZ, insts, device=local)
    g0.run(npaths, h, seed=1234, instance=0, use_graph=True, richardson=True, dup_sum=True)
    given = [g0.run(npaths, h, seed=1234, instance=1000 * (r + 1), use_graph=True, richardson=True, dup_sum=True)
             for r in range(2)]
    lat0 = [g0.result(i)["latency_ms"] for i in range(n_inst)]
    g0.close()
    # the benchmark: smallest instances first, so they finish in the first waves
    t0 = time.perf_counter()
    bt = P.Batch(P.BVP.HELMHOLTZ, insts, device=local, order="smallest_first")
    t_build = time.perf_counter() - t0
    bt.run(npaths, h, seed=1234, instance=0, use_graph=True, richardson=False)
    plain = bt.run(npaths, h, seed=1234, instance=500, use_graph=True, richardson=False)  # reference's weight rule
    plain_rmse = []
    for i, ins in enumerate(insts):
        x, y = bt.knots(i)
        plain_rmse.append(float(np.sqrt(np.mean((bt.result(i)["u"] - P.BVP.helmholtz(*ins.params).u(x, y)) ** 2))))
    bt.run(npaths, h, seed=1234, instance=0, use_graph=True, richardson=True, dup_sum=True)  # capture + warm-up
    runs = [bt.run(npaths, h, seed=1234, instance=1000 * (r + 1), use_graph=True, richardson=True, dup_sum=True)
            for r in range(reps)]
    lat, rmse, iters = [], [], []
    for i, ins in enumerate(insts):
        r = bt.result(i)
        x, y = bt.knots(i)
        bvp = P.BVP.helmholtz(*ins.params)
        rmse.append(float(np.sqrt(np.mean((r["u"] - bvp.u(x, y)) ** 2))))
        lat.append(r["latency_ms"])
        iters.append(r["iterations"])
    ms = float(np.mean([r["ms"] for r in runs]))
    out = {"instances": n_inst, "knots": int(bt.info["nknots"]), "nnz": int(bt.info["nnz"]),
           "paths_per_knot": npaths, "h": h, "h_rule": "h (4/g)^2 on g x g subdomains (h at g <= 4)",
           "waves": 16, "order": "smallest_first", "ms_per_batch": ms, "solves_per_s": n_inst / (ms / 1000.0),
           "path_steps_per_s": float(np.mean([r["path_steps"] / (r["ms"] / 1000.0) for r in runs])),
           "latency_ms_p50": float(np.percentile(lat, 50)), "latency_ms_p99": float(np.percentile(lat, 99)),
           "rmse_vs_analytic_mean": float(np.mean(rmse)), "rmse_vs_analytic_max": float(np.max(rmse)),
           "solver_iterations_max": int(max(iters)), "unconverged": int(max(r["unconverged"] for r in runs)),
           "kernel_launches_per_batch": int(runs[-1]["kernel_launches"]), "graph_replayed": int(runs[-1]["graph_replayed"]),
           "host_build_s": t_build,
           "given_order": {"ms_per_batch": float(np.mean([r["ms"] for r in given])),
                           "latency_ms_p50": float(np.percentile(lat0, 50)),
                           "latency_ms_p99": float(np.percentile(lat0, 99))},
           "plain_method": {"ms_per_batch": plain["ms"], "solves_per_s": n_inst / (plain["ms"] / 1000.0),
                            "rmse_vs_analytic_mean": float(np.mean(plain_rmse)),
                            "rmse_vs_analytic_max": float(np.max(plain_rmse))}}
    # error against the FP64 form on 4 instances: each instance alone, FP64,
    # Philox instance word base + i (the streams it draws in the batch)
    base = 1000 * reps
    ub, bb_, word = {}, {}, {}
    pick = [int(v) for v in np.random.default_rng(7).choice(n_inst, size=4, replace=False)]
    for i in pick:
        r = bt.result(i)
        ub[i], bb_[i], word[i] = r["u"], r["B"], base + bt.position(i)
    bt.close()
    uerr, berr = 0.0, 0.0
    for i in pick:
        ins = insts[i]
        with P.PDDSparseGM(ins.sw, ins.ne, ins.nsub, ins.nnode, ins.fac, device=local) as q:
            e = q.estimate(P.BVP.helmholtz(*ins.params), npaths, ins.h if ins.h > 0 else h, mode=P.MODE_FP64,
                           seed=1234, instance=word[i], adaptive_h=True, richardson=True, dup_sum=True)
            u64, _ = q.solve_interface(P.SOLVE_BICGSTAB_FP64, tol=1e-12)
        uerr = max(uerr, float(np.max(np.abs(ub[i] - u64))))
        berr = max(berr, float(np.max(np.abs(bb_[i] - e.B))))
    out["mixed_err_vs_fp64"] = {"instances": pick, "u_max_abs": uerr, "B_max_abs": berr}
    return out


def semilinear_newton(local: int, iterations: int = 4, npaths: int = 20_000, h: float = 5e-4, m: int = 32):
    """The semilinear outer loop (Solve_SemiLin_numVR + subdomain solves):
    Lap u - u^3 + F = 0 on [0,1]^2, u = 1.1 + sin(pi x) sin(pi y), 8 x 8
    subdomains, 21 knots per segment, Newton steps from the constant 1.1, each
    one Newton-table build on the device, a MIXED estimate (Richardson pair,
    adaptive step, summed weights), the interface solve and the table-served
    subdomain solves on 32 x 32 grids; wall time per step and the RMSE
    against the analytic solution after each step."""
    import pdds_gb300 as P
    from pdds_gb300.config import fac_rule
    pd = P.PDDSparseGM((0.0, 0.0), (1.0, 1.0), 8, 21, fac_rule(1.0, 8, 21), device=local)
    pd.solve_semilinear(1, 256, h, m=m)  # warm-up (module load, allocations)
    t0 = time.perf_counter()
    its = pd.solve_semilinear(iterations, npaths, h, m=m, seed=7, adaptive_h=True, richardson=True, dup_sum=True)
    dt = time.perf_counter() - t0
    out = {"knots": int(pd.K), "paths_per_knot": npaths, "h": h, "subdomain_grid": m, "newton_steps": iterations,
           "ms_per_newton_step": 1000.0 * dt / iterations,
           "rmse_knots": [round(it["rmse_knots"], 6) for it in its],
           "rmse_grid": [round(it["rmse_grid"], 6) for it in its],
           "path_steps_per_s": float(sum(it["estimate"].info["path_steps"] for it in its) / dt)}
    pd.close()
    return out


def linear_fixed_point(local: int, iterations: int = 6, npaths: int = 20_000, h: float = 5e-4, m: int = 32):
    """The fixed-point loop of main_LinLoop.cpp (Solve_Iterative_numVR +
    subdomain solves): Lap u + 20 u + F = 0 on [0,1]^2 split with the shift
    22 and the time rescale 9 (sigma = sqrt(2/9) I, c = -2/9,
    f = (F + 22 u_k)/9), u = sin(2 pi x + 1/2) cos(pi^2 (x + y)), 8 x 8
    subdomains, 21 knots per segment, from u_0 = 0; wall time per step and the
    RMSE against the analytic solution after each step."""
    import pdds_gb300 as P
    from pdds_gb300.config import fac_rule
    pd = P.PDDSparseGM((0.0, 0.0), (1.0, 1.0), 8, 21, fac_rule(1.0, 8, 21), device=local)
    pd.solve_linear_iteration(1, 256, h, m=m)  # warm-up (module load, allocations)
    t0 = time.perf_counter()
    its = pd.solve_linear_iteration(iterations, npaths, h, m=m, seed=7, adaptive_h=True, richardson=True,
                                    dup_sum=True)
    dt = time.perf_counter() - t0
    out = {"knots": int(pd.K), "paths_per_knot": npaths, "h": h, "subdomain_grid": m, "steps": iterations,
           "ms_per_step": 1000.0 * dt / iterations,
           "rmse_knots": [round(it["rmse_knots"], 6) for it in its],
           "rmse_grid": [round(it["rmse_grid"], 6) for it in its],
           "path_steps_per_s": float(sum(it["estimate"].info["path_steps"] for it in its) / dt)}
    pd.close()
    return out


def plain_poisson_4x4(local: int, reps: int = 3):
    """The CPU-runnable configuration: Poisson on [-1,1]^2, 4 x 4 subdomains,
    11 knots per segment (237 knots), 1e4 paths per knot, h = 1e-3, the plain
    method (fixed step, no Richardson pair, the reference's overwrite of shared
    side knots), seed 1234, in the three modes: the replay mode (FP64, the
    reference's per-exit weights, bit-exact with the CPU restatement), plain
    FP64 and MIXED; device time of the estimate and RMSE of the solved
    interface against the analytic solution."""
    import pdds_gb300 as P
    from pdds_gb300.config import WORKLOADS, fac_rule
    w = WORKLOADS["poisson_4x4_n11"]
    bvp = P.BVP.poisson_sincos()
    pd = P.PDDSparseGM(w["sw"], w["ne"], w["nsub"], w["nnode"], fac_rule(w["ne"][0] - w["sw"][0], w["nsub"],
                                                                         w["nnode"]), device=local)
    ex = bvp.u(pd.x, pd.y)
    out = {"knots": int(pd.K), "paths_per_knot": w["npaths"], "h": w["h"]}
    for name, mode in (("replay_fp64", P.MODE_REPLAY_FP64), ("fp64", P.MODE_FP64), ("mixed", P.MODE_MIXED)):
        pd.estimate(bvp, 64, w["h"], mode=mode)  # warm-up
        ms = []
        for r in range(reps):
            est = pd.estimate(bvp, w["npaths"], w["h"], mode=mode, seed=1234)
            ms.append(est.info["ms_setup"] + est.info["ms_paths"])
        u, si = pd.solve_interface(P.SOLVE_BICGSTAB_FP64, tol=1e-12)
        out[name] = {"ms_estimate": float(np.median(ms)), "path_steps": int(est.info["path_steps"]),
                     "path_steps_per_s": est.info["path_steps"] / (1e-3 * float(np.median(ms))),
                     "rmse_vs_analytic": float(np.sqrt(np.mean((u - ex) ** 2)))}
    pd.close()
    return out


def robin_reflected(local: int, reps: int = 3, npaths: int = 20_000, h: float = 5e-4):
    """The Robin test problem (poisson_3.hpp) on [-1,1]^2, 8 x 8 subdomains,
    21 knots per segment, Robin condition on the west side (paths reflect
    there with Lepingle's step), MIXED with the Richardson pair, adaptive step
    and summed weights; the same layout with Dirichlet data on every side for
    the cost of the reflection.  Device time of the estimate, RMSE of the
    solved interface against the analytic solution (all knots and the knots of
    the subdomain column on the Robin side)."""
    import pdds_gb300 as P
    from pdds_gb300.config import fac_rule
    pd = P.PDDSparseGM((-1.0, -1.0), (1.0, 1.0), 8, 21, fac_rule(2.0, 8, 21), device=local)
    near = pd.x < -0.75 + 1e-9
    opts = dict(adaptive_h=True, richardson=True, dup_sum=True)
    out = {"knots": int(pd.K), "paths_per_knot": npaths, "h": h, "robin_side": "W"}
    for name, side in (("robin_west", "W"), ("dirichlet", None)):
        bvp = P.BVP.robin_poisson(side)
        pd.estimate(bvp, 256, h, mode=P.MODE_MIXED, **opts)  # warm-up
        ms, steps = [], 0
        for r in range(reps):
            est = pd.estimate(bvp, npaths, h, mode=P.MODE_MIXED, seed=1234, instance=r, **opts)
            ms.append(est.info["ms_paths"])
            steps = est.info["path_steps"]
        u, si = pd.solve_interface()
        err = u - bvp.u(pd.x, pd.y)
        out[name] = {"ms_paths": float(np.median(ms)), "path_steps_per_s": steps / (1e-3 * float(np.median(ms))),
                     "rmse_vs_analytic": float(np.sqrt(np.mean(err ** 2))),
                     "rmse_robin_column": float(np.sqrt(np.mean(err[near] ** 2)))}
    pd.close()
    return out


def varcoef_lut(local: int, reps: int = 2):
    """The variable-coefficient problem with coefficients served from 1024^2
    FP32 tables (bicubic), 8 x 8 subdomains, 31 knots per segment, 5e4 paths
    per knot, h = 5e-4, MIXED with the Richardson pair, adaptive step and
    summed weights; device time of the path kernel by the library's events.
    The FP64 form runs the same tables with 2e3 paths per knot for the
    MIXED/FP64 path-step rate comparison."""
    import pdds_gb300 as P
    from pdds_gb300.config import WORKLOADS, fac_rule
    w = WORKLOADS["varcoef_lut_8x8_n31"]
    bvp = P.BVP.varcoef_lut(w["lut_n"], (w["sw"][0], w["sw"][1], w["ne"][0], w["ne"][1]))
    pd = P.PDDSparseGM(w["sw"], w["ne"], w["nsub"], w["nnode"], fac_rule(w["ne"][0] - w["sw"][0], w["nsub"],
                                                                         w["nnode"]), device=local)
    opts = dict(adaptive_h=True, richardson=True, dup_sum=True)
    pd.estimate(bvp, 256, w["h"], mode=P.MODE_MIXED, **opts)  # warm-up, table upload
    ms, steps = [], 0
    for r in range(reps):
        est = pd.estimate(bvp, w["npaths"], w["h"], mode=P.MODE_MIXED, seed=1234, instance=r, **opts)
        u, si = pd.solve_interface()
        ms.append(est.info["ms_paths"])
        steps = est.info["path_steps"]
    rmse = float(np.sqrt(np.mean((u - bvp.u(pd.x, pd.y)) ** 2)))
    # the Catmull-Rom node sampler (the FP64 form's) in the MIXED path kernel
    cr = P.BVP(P.BVP.LUT, (1.0,), tables=bvp.tables, exact=bvp.exact)
    pd.estimate(cr, 256, w["h"], mode=P.MODE_MIXED, **opts)
    ms_cr = []
    for r in range(reps):
        est_cr = pd.estimate(cr, w["npaths"], w["h"], mode=P.MODE_MIXED, seed=1234, instance=r, **opts)
        u_cr, _ = pd.solve_interface()
        ms_cr.append(est_cr.info["ms_paths"])
    rmse_cr = float(np.sqrt(np.mean((u_cr - bvp.u(pd.x, pd.y)) ** 2)))
    # hardware-filtered bilinear interpolation of the nodes
    bl = P.BVP(P.BVP.LUT, (2.0,), tables=bvp.tables, exact=bvp.exact)
    pd.estimate(bl, 256, w["h"], mode=P.MODE_MIXED, **opts)
    ms_bl = []
    for r in range(reps):
        est_bl = pd.estimate(bl, w["npaths"], w["h"], mode=P.MODE_MIXED, seed=1234, instance=r, **opts)
        u_bl, _ = pd.solve_interface()
        ms_bl.append(est_bl.info["ms_paths"])
    rmse_bl = float(np.sqrt(np.mean((u_bl - bvp.u(pd.x, pd.y)) ** 2)))
    e64 = pd.estimate(bvp, 2000, w["h"], mode=P.MODE_FP64, seed=1234, **opts)
    e32 = pd.estimate(bvp, 2000, w["h"], mode=P.MODE_MIXED, seed=1234, **opts)
    # the error against the FP64 form at the benchmark's 5e4 paths, on 16
    # knots (the per-knot call, the same Philox streams as the layout run)
    full = pd.estimate(bvp, w["npaths"], w["h"], mode=P.MODE_MIXED, seed=1234, instance=7, **opts)
    mc = np.flatnonzero(np.diff(pd.row_ptr) > 0)
    pick = np.random.default_rng(1234).choice(mc, size=16, replace=False)
    gerr, berr = 0.0, 0.0
    with P.EMFKACSolver(local) as sv:
        for k in pick:
            st = P.Stencil.of_knot(pd, int(k))
            G, _, Gj, B, _ = sv.Solve_GPU_Analytic((pd.x[k], pd.y[k]), w["npaths"], w["h"], 0.0, bvp, st,
                                                   mode=P.MODE_FP64, seed=1234, instance=7, knot_id=int(k),
                                                   want_var=False, **opts)
            r0, r1 = full.row_ptr[k], full.row_ptr[k + 1]
            gerr = max(gerr, float(np.max(np.abs(full.val[r0:r1] - G))))
            berr = max(berr, abs(float(full.B[k] - B)))
    out = {"knots": int(pd.K), "paths_per_knot": w["npaths"], "h": w["h"],
           "table": "1024^2 x 8 FP32; MIXED: cubic B-spline from textures",
           "ms_paths": float(np.mean(ms)), "path_steps_per_s": steps / (1e-3 * float(np.mean(ms))),
           "rmse_vs_analytic": rmse, "solve_ms": float(si["ms"]),
           "catmull_rom_nodes": {"ms_paths": float(np.mean(ms_cr)),
                                 "path_steps_per_s": est_cr.info["path_steps"] / (1e-3 * float(np.mean(ms_cr))),
                                 "rmse_vs_analytic": rmse_cr},
           "bilinear_texture": {"ms_paths": float(np.mean(ms_bl)),
                                "path_steps_per_s": est_bl.info["path_steps"] / (1e-3 * float(np.mean(ms_bl))),
                                "rmse_vs_analytic": rmse_bl},
           "fp64": {"paths_per_knot": 2000, "ms_paths": e64.info["ms_paths"],
                    "mixed_over_fp64": (e32.info["path_steps"] / e32.info["ms_paths"]) /
                                       (e64.info["path_steps"] / e64.info["ms_paths"]),
                    "mixed_err_vs_fp64": {"knots": 16, "paths_per_knot": w["npaths"], "G_max_abs": gerr,
                                          "B_max_abs": berr}}}
    pd.close()
    return out


def circle_uneven(local: int, reps: int = 2, h: float = 2e-5):
    """Uneven path lengths on the unit disk: 6 rings x 16 sectors (the central
    ring one disk subdomain), 11 knots per segment, Poisson with
    u = r^2 sin(3 theta) + cos x; h = 2e-5 with the per-knot adaptive step, so
    a path takes from 1 to a few 1e4 steps (the paths' step counts fill every
    log2 bin from 1 to 2^14..2^15) and a knot's mean from ~50 to ~1600;
    Richardson pair, variance-adaptive paths per knot N_k in [1e3, 1e5] for a
    score standard error of 1e-3, the launch shape picked by the autotuner
    (after the warm-up estimate, whose continuation it times at both block
    sizes).
    The same estimate with one CTA per work item in layout order shows what
    the persistent CTAs and the heaviest-first order do on it.  The FP64
    form runs the same layout with 1e3 paths per knot for the MIXED/FP64
    comparison."""
    import pdds_gb300 as P
    bvp = P.BVP.circle_poisson()
    pd = P.PDDSparseGM.circle_mesh(1.0, 6, 16, 11, device=local)
    ex = bvp.u(pd.x, pd.y)
    opts = dict(adaptive_h=True, richardson=True, dup_sum=True)
    runs = []
    tune = None
    for r in range(reps + 1):
        est = pd.estimate(bvp, 1000, h, mode=P.MODE_MIXED, seed=1234, instance=r, adaptive_n=True,
                          npaths_max=100_000, target_stderr=1e-3, step_histogram=True, **opts)
        u, si = pd.solve_interface()
        if r > 0:
            runs.append((est, u, si))
        else:  # after the warm-up: the shapes, and the block size of its continuation
            tune = pd.autotune(bvp, 1000, h, adaptive_h=True, richardson=True, adaptive_n=True)
    est, u, si = runs[-1]
    hist = pd.step_histogram()
    steps = pd.knot_steps().astype(np.float64)
    mc = est.npaths > 0
    per_path = steps[mc] / (2.0 * est.npaths[mc])  # both levels of the pair count; per level
    ms = [e.info["ms_setup"] + e.info["ms_paths"] + s_["ms"] for e, _, s_ in runs]
    plain = pd.estimate(bvp, 1000, h, mode=P.MODE_MIXED, seed=1234, instance=reps, adaptive_n=True,
                        npaths_max=100_000, target_stderr=1e-3, plain_launch=True, **opts)
    nz = np.flatnonzero(hist)
    out = {"knots": int(pd.K), "h": h, "adaptive_h": True, "paths_per_knot_min": int(est.npaths[mc].min()),
           "paths_per_knot_max": int(est.npaths[mc].max()), "paths": int(est.info["paths"]),
           "path_steps": int(est.info["path_steps"]), "ms_per_step": float(np.mean(ms)),
           "path_steps_per_s": float(np.mean([e.info["path_steps"] / (m / 1000.0) for (e, _, _), m in zip(runs, ms)])),
           "path_kernel_ms": float(np.mean([e.info["ms_paths"] for e, _, _ in runs])),
           "plain_launch_path_kernel_ms": float(plain.info["ms_paths"]),
           "steps_per_path_histogram_log2": hist[:nz.max() + 1].tolist(),
           "steps_per_path_min": int(2 ** nz.min()), "steps_per_path_max_at_least": int(2 ** nz.max()),
           "mean_steps_per_path_min": float(per_path.min()), "mean_steps_per_path_max": float(per_path.max()),
           "rmse_vs_analytic": float(np.sqrt(np.mean((u - ex) ** 2))), "solver_iterations": int(si["iterations"]),
           "autotune": tune}
    m = pd.estimate(bvp, 1000, h, mode=P.MODE_MIXED, seed=77, **opts)
    f = pd.estimate(bvp, 1000, h, mode=P.MODE_FP64, seed=77, **opts)
    tm = m.info["ms_setup"] + m.info["ms_paths"]
    tf = f.info["ms_setup"] + f.info["ms_paths"]
    out["fp64"] = {"ms_estimate": tf, "mixed_ms_estimate": tm, "mixed_over_fp64": tf / tm,
                   "G_max_abs": float(np.max(np.abs(m.val - f.val))), "B_max_abs": float(np.max(np.abs(m.B - f.B)))}
    pd.close()
    return out


def run_reference(args, workload, fac):
    rank, world, _ = _env_rank()
    if rank != 0:
        return
    per_step = []
    steps_total = 0
    knots_total = 0
    residuals = []
    base = None
    for s in range(args.warmup + args.steps):
        r = cpu_baseline(workload, fac, args.ref_knots, seed=1234 + s)
        if s >= args.warmup:
            per_step.append(r["seconds"])
            steps_total += r["path_steps"]
            knots_total += r["knots"]
            residuals += r["residuals"]
            base = r
    value = steps_total / sum(per_step)
    # The reference's algorithm: every knot's row from N paths of the fixed
    # step, no Richardson pair, the overwrite of shared side knots; the
    # accuracy of its rows is their residual at the exact solution (an
    # interface RMSE would need every knot: about 5 hours on these cores).
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "path-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * float(np.mean(per_step)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": workload["name"], "knots": base["knots"], "knots_per_step": base["knots"],
                       "paths_per_knot": workload["npaths"], "h": workload["h"], "mode": "FP64 (CPU, OpenMP paths, "
                       "serial reduction)", "adaptive_h": False, "richardson": False,
                       "shared_side_knots": "overwrite (reference)"},
            "knots_per_s": knots_total / sum(per_step),
            "knot_residual_rms": float(np.sqrt(np.mean(np.square(residuals)))),
            "rmse_vs_analytic": None,
            "cpu_baseline": {"value": value, "unit": "path-steps/s", "cores": base["cores"], "kind": "port",
                             "sample": base["sample"]},
            "e2e": {"value": value, "unit": "path-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def aggregate_ranks(t_dev: float, units: float, dist, device: str):
    """Whole-job figures over the replicas: the slowest rank's timed region
    and the units (path steps) all ranks processed.  dist: torch.distributed
    or None for one process; device: where the collective's tensors live
    ("cuda" under NCCL, "cpu" under gloo)."""
    if not dist:
        return float(t_dev), float(units)
    import torch
    tt = torch.tensor([float(t_dev)], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    st = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.all_reduce(st)
    return float(tt.item()), float(st.item())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="poisson_12x12_n43")
    ap.add_argument("--npaths", type=int, default=0)
    ap.add_argument("--ref-knots", type=int, default=4, help="knots per step of the reference arm")
    ap.add_argument("--cpu-knots", type=int, default=16, help="knots of the cpu_baseline sample (about 10 s)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-circle", action="store_true")
    ap.add_argument("--no-semilinear", action="store_true")
    ap.add_argument("--no-linloop", action="store_true")
    ap.add_argument("--no-lut", action="store_true")
    ap.add_argument("--no-poisson-4x4", action="store_true")
    ap.add_argument("--no-robin", action="store_true")
    ap.add_argument("--lut-sampler", default="bspline", choices=["bspline", "catmull_rom", "bilinear"],
                    help="MIXED table sampler of the table-served workload")
    args = ap.parse_args()

    from pdds_gb300.config import WORKLOADS, fac_rule
    workload = dict(WORKLOADS[args.workload])
    workload["name"] = args.workload
    if args.npaths:
        workload["npaths"] = args.npaths
    side = workload["ne"][0] - workload["sw"][0]
    fac = fac_rule(side, workload["nsub"], workload["nnode"])

    if args.impl == "reference":
        run_reference(args, workload, fac)
        return

    rank, world, local = _env_rank()
    dist = None
    if world > 1:
        import torch
        import torch.distributed as td
        td.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        dist = td
    import torch
    torch.cuda.set_device(local)
    import pdds_gb300 as P

    if workload.get("problem") == "varcoef_lut":
        bvp = P.BVP.varcoef_lut(workload["lut_n"], (workload["sw"][0], workload["sw"][1],
                                                     workload["ne"][0], workload["ne"][1]), sampler=args.lut_sampler)
    else:
        bvp = P.BVP.poisson_sincos()
    N, h = workload["npaths"], workload["h"]
    pd = P.PDDSparseGM(workload["sw"], workload["ne"], workload["nsub"], workload["nnode"], fac, device=local)
    exact = bvp.u(pd.x, pd.y)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    # the consistent weight rule for knots shared by two stencil sides (the
    # reference's overwrite is the API default, checked by the parity tests)
    OPTS = dict(adaptive_h=True, richardson=True, dup_sum=True)

    def step(instance, mode=P.MODE_MIXED, method=P.SOLVE_GMRES_FP32_IR, **opts):
        o = dict(OPTS)
        o.update(opts)
        est = pd.estimate(bvp, N, h, mode=mode, seed=1234, instance=instance, **o)
        u, sinfo = pd.solve_interface(method, tol=1e-10)
        return est, u, sinfo

    for w in range(args.warmup):
        step(1000 + w)
        flush.fill_(float(w))
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    ms_dev, steps_done, exits, launches, ms_paths, rmses, solve_ms = [], 0, 0, 0, [], [], []
    t_wall0 = time.perf_counter()
    for s in range(args.steps):
        est, u, sinfo = step(rank * 100000 + s)
        ms_dev.append(est.info["ms_setup"] + est.info["ms_paths"] + sinfo["ms"])
        ms_paths.append(est.info["ms_paths"])
        solve_ms.append(sinfo["ms"])
        steps_done += est.info["path_steps"]
        exits += est.info["exits_global"] + est.info["exits_stencil"]
        launches += est.info["kernel_launches"] + sinfo["kernel_launches"]
        rmses.append(float(np.sqrt(np.mean((u - exact) ** 2))))
        flush.fill_(float(s))
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall0
    clk = clocks.stop()
    t_dev, steps_all = aggregate_ranks(sum(ms_dev) / 1000.0, steps_done, dist, "cuda")
    value = steps_all / t_dev

    extra = {}
    # the reference's plain method (no adaptive step, no extrapolation), MIXED
    if rank == 0:
        estp, up, sp = step(999, adaptive_h=False, richardson=False, dup_sum=False)
        tp = (estp.info["ms_setup"] + estp.info["ms_paths"] + sp["ms"]) / 1000.0
        extra["plain_method"] = {"path_steps_per_s": estp.info["path_steps"] / tp, "ms_per_step": 1000 * tp,
                                 "knots_per_s": pd.K / tp, "path_steps": estp.info["path_steps"],
                                 "rmse_vs_analytic": float(np.sqrt(np.mean((up - exact) ** 2))),
                                 "knot_residual_rms": knot_residual_rms(estp, exact),
                                 "form": "the reference's algorithm: fixed step, no Richardson pair, overwrite "
                                         "of shared side knots"}
    # the same estimate with one CTA per work item, knots in layout order
    # (what the persistent CTAs and the heaviest-first order replace)
    if rank == 0:
        estl = pd.estimate(bvp, N, h, mode=P.MODE_MIXED, seed=1234, instance=998, plain_launch=True, **OPTS)
        extra["launch_policy"] = {"path_kernel_ms": float(np.mean(ms_paths)),
                                  "plain_launch_path_kernel_ms": float(estl.info["ms_paths"]),
                                  "plain_launch": "one CTA per work item, knots in layout order"}
    # plain FP64 GPU form on the same workload (the >= 3x comparison)
    if not args.no_fp64 and rank == 0:
        est64, u64, s64 = step(7, mode=P.MODE_FP64, method=P.SOLVE_BICGSTAB_FP64)
        t64 = (est64.info["ms_setup"] + est64.info["ms_paths"] + s64["ms"]) / 1000.0
        estm, um, sm = step(7)
        extra["fp64"] = {
            "path_steps_per_s": est64.info["path_steps"] / t64,
            "ms_per_step": 1000 * t64,
            "rmse_vs_analytic": float(np.sqrt(np.mean((u64 - exact) ** 2))),
            "mixed_over_fp64": value / (est64.info["path_steps"] / t64),
            "mixed_err_vs_fp64": {
                "G_max_abs": float(np.max(np.abs(estm.val - est64.val))),
                "B_max_abs": float(np.max(np.abs(estm.B - est64.B))),
                "u_max_abs": float(np.max(np.abs(um - u64))),
            },
        }

    # end to end through the public API: layout upload, estimation, solve,
    # and G, B, u back on the host, every step
    e2e = None
    if not args.no_e2e:
        # every step: a new context (layout built on the host and uploaded),
        # the estimate, the solve, G, B and u read back to host memory; the
        # bytes are the library's own counts of what it copied
        for s in range(args.warmup):  # untimed, like the device-timed steps
            q = P.PDDSparseGM(workload["sw"], workload["ne"], workload["nsub"], workload["nnode"], fac,
                              device=local)
            q.estimate(bvp, N, h, mode=P.MODE_MIXED, seed=1234, instance=40 + s, **OPTS)
            q.solve_interface()
            q.close()
        h2d = d2h = 0
        ph = {"layout": 0.0, "estimate": 0.0, "solve": 0.0, "close": 0.0}
        t0 = time.perf_counter()
        e2e_steps = 0
        for s in range(args.steps):
            ta = time.perf_counter()
            q = P.PDDSparseGM(workload["sw"], workload["ne"], workload["nsub"], workload["nnode"], fac,
                              device=local)
            tb = time.perf_counter()
            est2 = q.estimate(bvp, N, h, mode=P.MODE_MIXED, seed=1234, instance=50 + s, **OPTS)
            tc = time.perf_counter()
            u2, si2 = q.solve_interface()
            td = time.perf_counter()
            e2e_steps += est2.info["path_steps"]
            h2d += q.layout_info["h2d_bytes"] + est2.info["h2d_bytes"] + si2["h2d_bytes"]
            d2h += est2.info["d2h_bytes"] + si2["d2h_bytes"]
            q.close()
            te = time.perf_counter()
            for k, v in zip(ph, (tb - ta, tc - tb, td - tc, te - td)):
                ph[k] += v
        dt = time.perf_counter() - t0
        ns = args.steps
        e2e = {"value": e2e_steps / dt, "unit": "path-steps/s", "h2d_bytes_per_step": int(h2d // ns),
               "d2h_bytes_per_step": int(d2h // ns), "ms_per_step": 1000 * dt / ns, "steps": ns,
               "knots_per_s": pd.K * ns / dt,
               "phases_ms": {k: round(1000 * v / ns, 2) for k, v in ph.items()}}

    if not args.no_batch and rank == 0:
        extra["many_instance_batch"] = many_instance_batch(local)
    if not args.no_circle and rank == 0:
        extra["circle_uneven_lengths"] = circle_uneven(local)
    if not args.no_poisson_4x4 and rank == 0:
        extra["poisson_4x4_n11_plain"] = plain_poisson_4x4(local)
    if not args.no_lut and rank == 0:
        extra["varcoef_lut"] = varcoef_lut(local)
    if not args.no_robin and rank == 0:
        extra["robin_reflected"] = robin_reflected(local)
    if not args.no_semilinear and rank == 0:
        extra["semilinear_newton"] = semilinear_newton(local)
    if not args.no_linloop and rank == 0:
        extra["linear_fixed_point"] = linear_fixed_point(local)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            cpu = cpu_baseline(workload, fac, args.cpu_knots)
            cpu["knot_residual_rms"] = float(np.sqrt(np.mean(np.square(cpu.pop("residuals")))))
            fast = cpu_baseline(workload, fac, args.cpu_knots, fast=True)
            extra["cpu_linearity_form"] = {
                "value": fast["value"], "unit": "path-steps/s", "cores": fast["cores"],
                "sample": fast["sample"],
                "form": "the reference's reduction in its linearity form (n_s exponentials per exit, "
                        "G = -ipsi^T S / N) with the exits reduced in parallel; same paths"}
        except Exception as exc:  # report, do not fail the bench
            cpu = {"value": None, "unit": "path-steps/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"failed: {exc}"}

    # issue-slot roofline of the path kernel
    sm_count = torch.cuda.get_device_properties(local).multi_processor_count
    f_mhz = clk.get("sm_mhz") or 1920.0
    peak = sm_count * 4 * 32 * f_mhz * 1e6  # thread-instructions per second
    t_paths = sum(ms_paths) / 1000.0
    work = steps_done * W_STEP + exits * W_EXIT
    achieved = work / t_paths if t_paths > 0 else 0.0
    roof = {"bound": "issue", "achieved": achieved / 1e9, "peak": peak / 1e9, "unit": "Ginst/s",
            "frac": achieved / peak, "traffic": PATH_KERNEL_DRAM_BYTES.get(workload["name"]),
            "peak_source": f"{sm_count} SMs x 128 issue lanes x median SM clock {f_mhz:.0f} MHz under load",
            "kernel": "k_paths_mixed", "kernel_ms_per_launch": 1000 * t_paths / args.steps}

    line = {
        "metric": METRIC, "value": value, "unit": "path-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * t_dev / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
        "config": {"workload": workload["name"], "knots": pd.K, "paths_per_knot": N, "h": h,
                   "mode": "MIXED", "adaptive_h": True, "richardson": "h/2,h",
                   "solver": "GMRES(20) FP32 + FP64 refinement", "l2": "flushed (256 MB write)",
                   "shared_side_knots": "weights summed (dup_sum)"},
        "interface_solves_per_s": world * args.steps / t_dev,
        "knots_per_s": world * pd.K * args.steps / t_dev,
        "rmse_vs_analytic": float(np.mean(rmses)),
        "knot_residual_rms": knot_residual_rms(est, exact),
        "solve_ms": float(np.mean(solve_ms)),
        "wall_s": wall,
        "gpu_launches": int(launches),
        "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
    }
    if workload.get("problem") == "varcoef_lut":
        line["config"]["lut_sampler"] = args.lut_sampler
    line.update(extra)
    if rank == 0:
        print(json.dumps(line), flush=True)
    pd.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
