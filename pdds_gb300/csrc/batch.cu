// Batches of independent instances (include/pdds.h, "batch"): layout union,
// the one-sequence run (estimation of every instance in one path-kernel
// launch, every instance's interface solve in one cluster-GMRES launch),
// CUDA-graph capture and replay of that sequence, per-instance results.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/pdds.h"
#include "ctx.h"
#include "kernels.h"
#include "pdds_internal.h"
#include "solve.h"

using namespace pdds;

namespace {

// Number of instance groups of a run.
int batch_waves(const pdds_ctx* ctx, const pdds_batch_run_desc* d) {
  return std::max(1, std::min(ctx->n_inst, d->waves > 0 ? d->waves : 16));
}

// The whole batch step, without host synchronisation.  The stream runs the
// factorisation, zeroing and boundary knots, then the instances in W
// consecutive groups (a path-kernel launch and the finalisation per group);
// the solve stream, once a group's finalisation is done, copies its G rows
// to FP32 and runs the cluster GMRES of its systems while the next group's
// paths run.  The last solve joins the stream again.
pdds_status enqueue_batch(pdds_ctx* ctx, const pdds_batch_run_desc* d, int cluster, int* launches) {
  cudaStream_t s = ctx->stream, s2 = ctx->solve_stream;
  const int n = ctx->n_inst;
  const int W = batch_waves(ctx, d);
  CK(launch_stamp(ctx->b_tend.p + n, s));
  ++*launches;
  pdds_status st = enqueue_mixed(ctx, &d->estimate, launches, 0, 0, true);  // prefix only
  if (st != PDDS_OK) return st;
  ClusterGmresArgs a{};
  a.err_flags = ctx->errf.p;
  a.K = ctx->L.K;
  a.row_ptr = ctx->row_ptr.p;
  a.col = ctx->col.p;
  a.val64 = ctx->G.p;
  a.val32 = ctx->sval32.p;
  a.b = ctx->B.p;
  a.x = ctx->su.p;
  a.r64 = ctx->sv64.p;
  a.V = ctx->sV32.p;
  a.Z = d->solve.gmres_form == PDDS_GMRES_PIPELINED ? ctx->sZ32.p : nullptr;
  a.m = std::max(2, std::min(d->solve.restart > 0 ? d->solve.restart : 30, GMRES_CLUSTER_MAX_M));
  a.max_iter = d->solve.max_iter > 0 ? d->solve.max_iter : 1000;
  a.max_refine = d->solve.max_refine > 0 ? d->solve.max_refine : 30;
  a.tol = d->solve.tol > 0 ? d->solve.tol : 1e-10;
  a.inner_tol = 1e-6;
  for (int w = 0; w < W; w++) {
    const int i0 = (int)((int64_t)n * w / W), i1 = (int)((int64_t)n * (w + 1) / W);
    const int m0 = ctx->inst_mc0[i0], m1 = ctx->inst_mc0[i1];
    st = enqueue_mixed(ctx, &d->estimate, launches, m0, m1 - m0, false);
    if (st != PDDS_OK) return st;
    CK(cudaEventRecord(ctx->wave_ev[w], s));
    CK(cudaStreamWaitEvent(s2, ctx->wave_ev[w], 0));
    const int64_t e0 = ctx->inst_nnz0[i0], e1 = ctx->inst_nnz0[i1];
    CK(launch_to_f32(ctx->G.p + e0, ctx->sval32.p + e0, e1 - e0, s2));
    ++*launches;
    a.n_sys = i1 - i0;
    a.sys_row0 = ctx->inst_knot0.p + i0;
    a.out_iters = ctx->b_iters.p + i0;
    a.out_refines = ctx->b_refines.p + i0;
    a.out_relres = ctx->b_relres.p + i0;
    a.out_t_end = ctx->b_tend.p + i0;
    CK(launch_gmres_cluster(a, cluster, ctx->max_inst_knots, s2));
    ++*launches;
  }
  CK(cudaEventRecord(ctx->wave_ev[W], s2));
  CK(cudaStreamWaitEvent(s, ctx->wave_ev[W], 0));
  return PDDS_OK;
}

}  // namespace

extern "C" {

pdds_status pdds_batch_build(pdds_ctx* ctx, const pdds_instance_desc* inst, int32_t n, pdds_batch_info* info) {
  if (!ctx || !inst || n < 1) return fail(ctx, PDDS_ERR_INVALID, "a batch needs n >= 1 instances");
  std::vector<HostLayout> parts(n);
  for (int i = 0; i < n; i++)
    for (int q = 0; q < 4; q++)
      if (!(inst[i].layout.fac[q] > 0.0))
        return fail(ctx, PDDS_ERR_INVALID, "instance " + std::to_string(i) + ": fac must be positive");
  {  // the instances' layouts are independent: host threads over instances
    std::vector<std::string> errs(n);
    const int nth = std::max(1, std::min<int>({(int)std::thread::hardware_concurrency(), 16, n}));
    auto worker = [&](int t) {
      for (int i = t; i < n; i += nth) {
        const pdds_layout_desc& ld = inst[i].layout;
        try {
          errs[i] = build_rect_layout(parts[i], ld.sw, ld.ne, ld.nsub, ld.nnode, ld.fac, ctx->bins, 1);
        } catch (const std::exception& ex) {
          errs[i] = ex.what();
        }
      }
    };
    std::vector<std::thread> pool;
    int t = 1;
    try {
      for (; t < nth; t++) pool.emplace_back(worker, t);
    } catch (const std::exception&) {  // no thread: the workers left run here
    }
    for (int r = t; r < nth; r++) worker(r);
    worker(0);
    for (auto& th : pool) th.join();
    for (int i = 0; i < n; i++)
      if (!errs[i].empty()) return fail(ctx, PDDS_ERR_INVALID, "instance " + std::to_string(i) + ": " + errs[i]);
  }
  if (ctx->device >= 0) {
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  drop_graph(ctx);
  clear_tune(ctx);
  const std::string e = merge_layouts(ctx->L, parts, ctx->bins);
  if (!e.empty()) return fail(ctx, PDDS_ERR_INVALID, e);
  ctx->n_inst = n;
  ctx->inst_k0.assign(n + 1, 0);
  ctx->inst_nnz0.assign(n + 1, 0);
  ctx->inst_p.assign((size_t)8 * n, 0.0);
  ctx->inst_hv.assign((size_t)n, 0.0);
  ctx->max_inst_knots = 0;
  for (int i = 0; i < n; i++) {
    if (!(inst[i].h >= 0.0)) return fail(ctx, PDDS_ERR_INVALID, "instance " + std::to_string(i) + ": h must be >= 0");
    ctx->inst_hv[i] = inst[i].h;
    ctx->inst_k0[i + 1] = ctx->inst_k0[i] + parts[i].K;
    ctx->inst_nnz0[i + 1] = ctx->inst_nnz0[i] + parts[i].row_ptr[parts[i].K];
    for (int q = 0; q < 8; q++) ctx->inst_p[8 * i + q] = inst[i].p[q];
    ctx->max_inst_knots = std::max(ctx->max_inst_knots, parts[i].K);
  }
  ctx->is_batch = true;
  ctx->has_layout = true;
  ctx->has_estimate = false;
  ctx->has_batch_run = false;
  if (ctx->device >= 0) {
    std::vector<int> knot_inst(ctx->L.K);
    for (int i = 0; i < n; i++)
      for (int k = ctx->inst_k0[i]; k < ctx->inst_k0[i + 1]; k++) knot_inst[k] = i;
    cudaStream_t s = ctx->stream;
    CK(ctx->knot_inst.upload(knot_inst, s));
    CK(ctx->inst_knot0.upload(ctx->inst_k0, s));
    CK(ctx->inst_pd.upload(ctx->inst_p, s));
    CK(ctx->inst_hd.upload(ctx->inst_hv, s));
    CK(ctx->b_iters.resize(n));
    CK(ctx->b_refines.resize(n));
    CK(ctx->b_relres.resize(n));
    CK(ctx->b_tend.resize(n + 1));
    pdds_status st = upload_layout(ctx);
    if (st != PDDS_OK) return st;
    CK(cudaStreamSynchronize(s));
    // first entry of each instance in the list of knots with paths (the
    // merged hand-out order runs instance by instance)
    const std::vector<int>& mc = ctx->mc_host;
    ctx->inst_mc0.assign(n + 1, (int)mc.size());
    int m = 0;
    for (int i = 0; i < n; i++) {
      while (m < (int)mc.size() && knot_inst[mc[m]] < i) m++;
      ctx->inst_mc0[i] = m;
    }
  }
  if (info) {
    info->ninstances = n;
    info->max_knots = ctx->max_inst_knots;
    info->nknots = ctx->L.K;
    info->nnz = ctx->L.row_ptr[ctx->L.K];
  }
  return PDDS_OK;
}

pdds_status pdds_batch_run(pdds_ctx* ctx, const pdds_batch_run_desc* desc, pdds_batch_run_info* info) {
  if (!ctx || !desc) return PDDS_ERR_INVALID;
  if (ctx->device < 0) return fail(ctx, PDDS_ERR_INVALID, "context has no device");
  if (!ctx->is_batch) return fail(ctx, PDDS_ERR_INVALID, "no batch built");
  if (!ctx->has_problem) return fail(ctx, PDDS_ERR_INVALID, "no problem set");
  const pdds_estimate_desc& ed = desc->estimate;
  if (ed.mode != PDDS_MODE_MIXED) return fail(ctx, PDDS_ERR_INVALID, "batches run in PDDS_MODE_MIXED");
  if (ed.npaths < 1 || !(ed.h > 0.0)) return fail(ctx, PDDS_ERR_INVALID, "npaths >= 1 and h > 0 required");
  if (ed.ipsi_override) return fail(ctx, PDDS_ERR_INVALID, "ipsi_override is a replay option");
  if (ed.adaptive_n) return fail(ctx, PDDS_ERR_INVALID, "batches use a fixed number of paths per knot");
  if (ed.diagnostics || ed.knot_first || ed.knot_count)
    return fail(ctx, PDDS_ERR_INVALID, "diagnostics and knot ranges are pdds_estimate options");
  if (desc->solve.method != PDDS_SOLVE_GMRES_FP32_IR)
    return fail(ctx, PDDS_ERR_INVALID, "batches solve with PDDS_SOLVE_GMRES_FP32_IR");
  if (desc->solve.restart > GMRES_CLUSTER_MAX_M) return fail(ctx, PDDS_ERR_INVALID, "restart must be <= 40");
  CK(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  HostLayout& L = ctx->L;
  const int bins = ed.bins_per_gap > 0 ? ed.bins_per_gap : 16;
  if (bins != ctx->bins) {
    drop_graph(ctx);
    ctx->bins = bins;
    set_shape_bins(L, bins);
    pdds_status st = upload_layout(ctx);
    if (st != PDDS_OK) return st;
  }
  if (desc->waves < 0) return fail(ctx, PDDS_ERR_INVALID, "waves must be >= 0");
  if (!ctx->solve_stream) {
    int least = 0, greatest = 0;
    CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    CK(cudaStreamCreateWithPriority(&ctx->solve_stream, cudaStreamNonBlocking, greatest));
  }
  while ((int)ctx->wave_ev.size() < batch_waves(ctx, desc) + 1) {
    cudaEvent_t ev = nullptr;
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    ctx->wave_ev.push_back(ev);
  }
  const int cluster = gmres_cluster_pick(ctx->max_inst_knots);
  if (cluster <= 0)
    return fail(ctx, PDDS_ERR_INVALID, "largest instance (" + std::to_string(ctx->max_inst_knots) +
                                           " knots) exceeds the batched solve's shared-memory staging");
  const int64_t K = L.K;
  const int64_t nnz = L.row_ptr[L.K];
  const int m = std::max(2, std::min(desc->solve.restart > 0 ? desc->solve.restart : 30, GMRES_CLUSTER_MAX_M));
  // buffers first: a captured graph holds their addresses
  const void* before[5] = {ctx->sV32.p, ctx->sval32.p, ctx->sv64.p, ctx->su.p, ctx->sZ32.p};
  CK(ctx->sV32.resize((size_t)(m + 1) * K));
  if (desc->solve.gmres_form == PDDS_GMRES_PIPELINED) CK(ctx->sZ32.resize((size_t)(m + 1) * K));
  CK(ctx->sval32.resize(std::max<int64_t>(nnz, 1)));
  CK(ctx->sv64.resize(std::max<int64_t>(K, 1) * 6));
  CK(ctx->su.resize(std::max<int64_t>(K, 1)));
  const void* after[5] = {ctx->sV32.p, ctx->sval32.p, ctx->sv64.p, ctx->su.p, ctx->sZ32.p};
  if (std::memcmp(before, after, sizeof(before)) != 0) drop_graph(ctx);
  // the graph is reused while the descriptor, the cluster size and the solve
  // scratch (which pdds_solve_interface may also reallocate) are unchanged;
  // layout, problem and table changes drop it where they happen
  // seed and instance are not part of the key: a replay re-keys the
  // path-kernel nodes' parameters
  pdds_batch_run_desc kd = *desc;
  kd.estimate.seed = 0;
  kd.estimate.instance = 0;
  std::vector<unsigned char> key(sizeof(pdds_batch_run_desc) + sizeof(int) + sizeof(after));
  std::memcpy(key.data(), &kd, sizeof(pdds_batch_run_desc));
  std::memcpy(key.data() + sizeof(pdds_batch_run_desc), &cluster, sizeof(int));
  std::memcpy(key.data() + sizeof(pdds_batch_run_desc) + sizeof(int), after, sizeof(after));
  int launches = 0;
  bool replayed = false;
  if (desc->use_graph) {
    if (!ctx->graph_exec || ctx->graph_key != key) {
      drop_graph(ctx);
      CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
      int nl = 0;
      pdds_status st = enqueue_batch(ctx, desc, cluster, &nl);
      cudaGraph_t g = nullptr;
      cudaError_t ce = cudaStreamEndCapture(s, &g);
      if (st != PDDS_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
      }
      if (ce != cudaSuccess) return fail(ctx, PDDS_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
      ctx->graph = g;
      CK(cudaGraphInstantiate(&ctx->graph_exec, ctx->graph, 0));
      ctx->graph_key = key;
      ctx->graph_launches = nl;
      size_t nn = 0;
      CK(cudaGraphGetNodes(g, nullptr, &nn));
      std::vector<cudaGraphNode_t> nodes(nn);
      if (nn) CK(cudaGraphGetNodes(g, nodes.data(), &nn));
      for (cudaGraphNode_t nd : nodes) {
        cudaGraphNodeType ty;
        CK(cudaGraphNodeGetType(nd, &ty));
        if (ty != cudaGraphNodeTypeKernel) continue;
        cudaKernelNodeParams p;
        CK(cudaGraphKernelNodeGetParams(nd, &p));
        if (is_mixed_path_kernel(p.func)) ctx->graph_path_nodes.push_back(nd);
      }
    } else {
      replayed = true;
      // the path kernels of this run draw the streams of its seed and instance
      for (cudaGraphNode_t nd : ctx->graph_path_nodes) {
        cudaKernelNodeParams p;
        CK(cudaGraphKernelNodeGetParams(nd, &p));
        MixedArgs ma = *static_cast<const MixedArgs*>(p.kernelParams[0]);
        mixed_set_rng(ma, ed.seed, (uint32_t)ed.instance);
        void* args[1] = {&ma};
        p.kernelParams = args;
        p.extra = nullptr;
        CK(cudaGraphExecKernelNodeSetParams(ctx->graph_exec, nd, &p));
      }
    }
    launches = ctx->graph_launches;
    CK(cudaEventRecord(ctx->ev0, s));
    CK(cudaGraphLaunch(ctx->graph_exec, s));
    CK(cudaEventRecord(ctx->ev1, s));
  } else {
    CK(cudaEventRecord(ctx->ev0, s));
    pdds_status st = enqueue_batch(ctx, desc, cluster, &launches);
    if (st != PDDS_OK) return st;
    CK(cudaEventRecord(ctx->ev1, s));
  }
  unsigned long long stats[8] = {0};
  CK(copy_async(stats, ctx->stats.p, sizeof(stats), cudaMemcpyDeviceToHost, s));
  std::vector<int> it(ctx->n_inst);
  std::vector<double> rr(ctx->n_inst);
  CK(copy_async(it.data(), ctx->b_iters.p, ctx->n_inst * sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(copy_async(rr.data(), ctx->b_relres.p, ctx->n_inst * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  ctx->has_estimate = true;
  ctx->has_batch_run = true;
  const double tol = desc->solve.tol > 0 ? desc->solve.tol : 1e-10;
  if (info) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    info->ms = ms;
    info->path_steps = (int64_t)stats[0];
    info->paths = (int64_t)ctx->n_mc * ed.npaths;
    info->exits_global = (int64_t)stats[2];
    info->exits_stencil = (int64_t)stats[3];
    info->kernel_launches = launches;
    info->graph_replayed = replayed ? 1 : 0;
    info->max_iterations = 0;
    info->unconverged = 0;
    info->max_rel_residual = 0.0;
    for (int i = 0; i < ctx->n_inst; i++) {
      info->max_iterations = std::max(info->max_iterations, it[i]);
      info->max_rel_residual = std::max(info->max_rel_residual, rr[i]);
      if (!(rr[i] <= tol * 1.0000001) && rr[i] != 0.0) info->unconverged++;
    }
  }
  return check_err_flags(ctx);
}

pdds_status pdds_batch_instance(pdds_ctx* ctx, int32_t i, int32_t* nknots, double* x, double* y, double* u,
                                double* B, int32_t* iterations, double* rel_residual, double* latency_ms) {
  if (!ctx || !ctx->is_batch) return fail(ctx, PDDS_ERR_INVALID, "no batch built");
  if (i < 0 || i >= ctx->n_inst) return fail(ctx, PDDS_ERR_INVALID, "instance out of range");
  const int k0 = ctx->inst_k0[i], nk = ctx->inst_k0[i + 1] - k0;
  if (nknots) *nknots = nk;
  if (x) std::copy(ctx->L.kx.begin() + k0, ctx->L.kx.begin() + k0 + nk, x);
  if (y) std::copy(ctx->L.ky.begin() + k0, ctx->L.ky.begin() + k0 + nk, y);
  if (!(u || B || iterations || rel_residual || latency_ms)) return PDDS_OK;
  if (!ctx->has_batch_run) return fail(ctx, PDDS_ERR_INVALID, "no batch run yet");
  CK(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  int it = 0;
  double rr = 0.0;
  unsigned long long t[2] = {0, 0};
  if (u) CK(copy_async(u, ctx->su.p + k0, nk * sizeof(double), cudaMemcpyDeviceToHost, s));
  if (B) CK(copy_async(B, ctx->B.p + k0, nk * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(copy_async(&it, ctx->b_iters.p + i, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(copy_async(&rr, ctx->b_relres.p + i, sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(copy_async(&t[0], ctx->b_tend.p + i, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
  CK(copy_async(&t[1], ctx->b_tend.p + ctx->n_inst, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (iterations) *iterations = it;
  if (rel_residual) *rel_residual = rr;
  if (latency_ms) *latency_ms = t[0] >= t[1] ? (double)(t[0] - t[1]) * 1e-6 : 0.0;
  return PDDS_OK;
}

}  // extern "C"
