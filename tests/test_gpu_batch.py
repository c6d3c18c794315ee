"""Many-instance batches on the GPU: every instance of a batch gets the
answer a run of that instance alone gets (same random stream, agreement far
inside the Monte Carlo error), each converges to its own tolerance and
approaches its analytic solution, and the CUDA-graph replay of the sequence
equals the directly launched sequence."""
import numpy as np
import pytest

import pdds_gb300 as P
from pdds_gb300.config import batch_instances, fac_rule

pytestmark = pytest.mark.gpu

N, H = 2000, 1e-3


def small_instances():
    return [P.Instance((0.0, 0.0), (1.0, 1.0), g, k, fac_rule(1.0, g, k), (a, b, c))
            for g, k, a, b, c in [(4, 11, 1.5, 2.0, -1.0), (6, 9, 3.0, 1.2, 0.0), (5, 13, 2.2, 3.7, -3.5)]]


def test_batch_instance_equals_single_run():
    insts = small_instances()
    with P.Batch(P.BVP.HELMHOLTZ, insts) as bt:
        info = bt.run(N, H, seed=11, instance=100, adaptive_h=True, use_graph=False)
        assert info["unconverged"] == 0
        res = [bt.result(i) for i in range(len(insts))]
    for i, ins in enumerate(insts):
        with P.PDDSparseGM(ins.sw, ins.ne, ins.nsub, ins.nnode, ins.fac) as pd:
            bvp = P.BVP.helmholtz(*ins.params)
            est = pd.estimate(bvp, N, H, mode=P.MODE_MIXED, seed=11, instance=100 + i, adaptive_h=True)
            u, _ = pd.solve_interface(P.SOLVE_GMRES_FP32_IR, tol=1e-10)
            # same Philox streams: only the order of the FP32/FP64 sums differs
            assert np.max(np.abs(res[i]["B"] - est.B)) < 1e-5
            assert np.max(np.abs(res[i]["u"] - u)) < 1e-4
            rmse = np.sqrt(np.mean((res[i]["u"] - bvp.u(pd.x, pd.y)) ** 2))
            assert rmse < 5e-2, rmse


def test_smallest_first_order_keeps_the_callers_indices():
    """order="smallest_first" runs the instances by increasing knot count;
    every result still belongs to the caller's index i, and instance i draws
    the stream of its processing position."""
    insts = small_instances()[::-1]  # 472 (5x5/13), 465 (6x6/9), 237 (4x4/11) knots
    with P.Batch(P.BVP.HELMHOLTZ, insts, order="smallest_first") as bt:
        assert [bt.position(i) for i in range(3)] == [2, 1, 0]
        info = bt.run(N, H, seed=11, instance=100, adaptive_h=True, use_graph=True)
        assert info["unconverged"] == 0
        res = [(bt.result(i), bt.knots(i), bt.position(i)) for i in range(len(insts))]
    for i, ins in enumerate(insts):
        r, (x, y), j = res[i]
        with P.PDDSparseGM(ins.sw, ins.ne, ins.nsub, ins.nnode, ins.fac) as pd:
            assert len(x) == pd.K
            np.testing.assert_array_equal(x, pd.x)
            est = pd.estimate(P.BVP.helmholtz(*ins.params), N, H, mode=P.MODE_MIXED, seed=11, instance=100 + j,
                              adaptive_h=True)
            assert np.max(np.abs(r["B"] - est.B)) < 1e-5


def test_batch_graph_replay_matches_direct_launch():
    insts = small_instances()
    with P.Batch(P.BVP.HELMHOLTZ, insts) as bt:
        bt.run(N, H, seed=5, use_graph=False)
        direct = [bt.result(i)["u"] for i in range(len(insts))]
        first = bt.run(N, H, seed=5, use_graph=True)
        second = bt.run(N, H, seed=5, use_graph=True)
        assert first["graph_replayed"] == 0 and second["graph_replayed"] == 1
        assert second["kernel_launches"] == first["kernel_launches"] > 0
        replay = [bt.result(i) for i in range(len(insts))]
        # a new seed and instance replay the same graph, its path-kernel
        # nodes re-keyed: the results equal a direct launch with them
        third = bt.run(N, H, seed=6, instance=3, use_graph=True)
        assert third["graph_replayed"] == 1
        other = [bt.result(i)["u"] for i in range(len(insts))]
        bt.run(N, H, seed=6, instance=3, use_graph=False)
        direct6 = [bt.result(i)["u"] for i in range(len(insts))]
    for d, r in zip(direct, replay):
        assert np.max(np.abs(d - r["u"])) < 1e-6
        assert r["latency_ms"] > 0.0 and r["iterations"] > 0
    assert max(np.max(np.abs(d - o)) for d, o in zip(direct, other)) > 1e-6
    for d, o in zip(direct6, other):
        assert np.max(np.abs(d - o)) < 1e-6


def test_batch_scaled_steps_reach_the_accuracy_target_in_waves():
    """The many-instance workload's policy: each instance's step scaled with
    the square of its subdomain size (h at 4 x 4, h (4/g)^2 on g x g), the
    Richardson pair and the adaptive step, 1e4 paths: every instance's
    interface RMSE is below 2e-3, grids up to 16 x 16 and 11..41 knots per
    segment.  Run in groups whose solves overlap the next group's paths, the
    first instances complete well before the batch; the grouping changes no
    result beyond summation order."""
    insts = batch_instances(20, seed=11, scaled_h=1e-3)
    assert max(i.nsub for i in insts) >= 14 and min(i.h for i in insts) < 1e-4
    opts = dict(seed=5, instance=40, use_graph=True, richardson=True, dup_sum=True)
    with P.Batch(P.BVP.HELMHOLTZ, insts) as bt:
        one = bt.run(10_000, 1e-3, waves=1, **opts)
        u1 = [bt.result(i)["u"] for i in range(len(insts))]
        info = bt.run(10_000, 1e-3, waves=5, **opts)
        assert info["unconverged"] == 0
        lat, rmse = [], []
        for i, ins in enumerate(insts):
            r = bt.result(i)
            x, y = bt.knots(i)
            rmse.append(float(np.sqrt(np.mean((r["u"] - P.BVP.helmholtz(*ins.params).u(x, y)) ** 2))))
            lat.append(r["latency_ms"])
            np.testing.assert_allclose(r["u"], u1[i], rtol=0, atol=2e-5)
    assert max(rmse) < 2e-3, rmse
    assert min(lat) < 0.5 * info["ms"] and max(lat) <= info["ms"] * 1.05
    assert one["path_steps"] == info["path_steps"]


def test_batch_many_instances_converge():
    insts = batch_instances(24, seed=3, grid=(4, 10), nodes=(11, 25))
    with P.Batch(P.BVP.HELMHOLTZ, insts) as bt:
        info = bt.run(1000, H, seed=2, use_graph=True)
        assert info["unconverged"] == 0
        assert info["max_rel_residual"] <= 1e-10 * 1.0000001
        lat = []
        for i, ins in enumerate(insts):
            r = bt.result(i)
            x, y = bt.knots(i)
            bvp = P.BVP.helmholtz(*ins.params)
            assert np.sqrt(np.mean((r["u"] - bvp.u(x, y)) ** 2)) < 0.1  # N = 1e3, plain step
            lat.append(r["latency_ms"])
        assert 0.0 < min(lat) <= max(lat) <= info["ms"] * 1.5
