// C ABI of pdds_gb300 (declared in include/pdds.h): context, problem, layout,
// estimation and interface solve.  Host orchestration in C++; the work runs in
// the kernels of k_*.cu on the context's stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/pdds.h"
#include "ctx.h"
#include "kernels.h"
#include "pdds_internal.h"
#include "solve.h"

using namespace pdds;

namespace pdds {

XferCount& xfer() {
  thread_local XferCount t;
  return t;
}

namespace {

struct BlockCache {
  std::mutex mu;
  std::map<int, std::multimap<size_t, void*>> free_blocks;  // per device: bytes -> block
  std::map<int, size_t> held;                                // per device: bytes cached
};

BlockCache& block_cache() {
  static BlockCache* c = new BlockCache();  // never destroyed: no CUDA calls at exit
  return *c;
}

constexpr size_t CACHE_MAX_BLOCK = size_t(2) << 30;  // larger blocks are freed at once
constexpr size_t CACHE_MAX_HELD = size_t(8) << 30;   // per device

}  // namespace

// 512 B, then four classes per octave up to 64 MB, then multiples of 2 MB;
// a class size maps to itself.
size_t block_class(size_t bytes) {
  if (bytes <= 512) return 512;
  if (bytes > (size_t(64) << 20)) {
    const size_t m = size_t(2) << 20;
    return (bytes + m - 1) / m * m;
  }
  int e = 0;
  while ((size_t(1) << (e + 1)) < bytes) e++;  // 2^e < bytes <= 2^(e+1)
  const size_t step = size_t(1) << (e - 2);
  return (bytes + step - 1) / step * step;
}

cudaError_t block_alloc(void** p, size_t bytes) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  {
    BlockCache& c = block_cache();
    std::lock_guard<std::mutex> lk(c.mu);
    auto& fb = c.free_blocks[dev];
    auto it = fb.find(bytes);
    if (it != fb.end()) {
      *p = it->second;
      fb.erase(it);
      c.held[dev] -= bytes;
      return cudaSuccess;
    }
  }
  e = cudaMalloc(p, bytes);
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    block_cache_clear(dev);
    e = cudaMalloc(p, bytes);
  }
  return e;
}

void block_recycle(void* p, size_t bytes) {
  if (!p) return;
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && bytes <= CACHE_MAX_BLOCK) {
    BlockCache& c = block_cache();
    std::lock_guard<std::mutex> lk(c.mu);
    if (c.held[dev] + bytes <= CACHE_MAX_HELD) {
      c.free_blocks[dev].emplace(bytes, p);
      c.held[dev] += bytes;
      return;
    }
  }
  cudaFree(p);
}

void block_cache_clear(int device) {
  std::vector<std::pair<int, void*>> drop;
  {
    BlockCache& c = block_cache();
    std::lock_guard<std::mutex> lk(c.mu);
    for (auto& kv : c.free_blocks) {
      if (device >= 0 && kv.first != device) continue;
      for (auto& b : kv.second) drop.push_back({kv.first, b.second});
      kv.second.clear();
      c.held[kv.first] = 0;
    }
  }
  if (drop.empty()) return;
  int cur = 0;
  const bool have = cudaGetDevice(&cur) == cudaSuccess;
  for (auto& d : drop) {
    cudaSetDevice(d.first);
    cudaFree(d.second);
  }
  if (have) cudaSetDevice(cur);
}

pdds_status fail(pdds_ctx* c, pdds_status s, const std::string& msg) {
  if (c) c->err = msg;
  return s;
}

void drop_graph(pdds_ctx* ctx) {
  if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
  if (ctx->graph) cudaGraphDestroy(ctx->graph);
  ctx->graph_exec = nullptr;
  ctx->graph = nullptr;
  ctx->graph_key.clear();
  ctx->graph_launches = 0;
  ctx->graph_path_nodes.clear();
}

void clear_tune(pdds_ctx* ctx) {
  ctx->tune_bps = 0;
  ctx->tune_ppc = 0;
  ctx->tune_threads = 0;
  ctx->tune_cont_threads = 0;
  ctx->tune_cont_ppc = 0;
  ctx->tune_kind = -1;
  ctx->tune_rich = -1;
  ctx->cont_knots.clear();
  ctx->cont_N0 = 0;
  ctx->cont_kind = -1;
}

// Work items of an adaptive continuation: each knot's paths N0 .. N_k-1 in
// chunks of ppc, knots in the given order.
void continuation_items(const std::vector<int>& knots, const std::vector<int>& nk, int N0, int ppc,
                        std::vector<int>& ik, std::vector<int>& ip0, std::vector<int>& ip1) {
  ik.clear();
  ip0.clear();
  ip1.clear();
  for (int v : knots)
    for (long long p = N0; p < nk[v]; p += ppc) {
      ik.push_back(v);
      ip0.push_back((int)p);
      ip1.push_back((int)std::min<long long>(nk[v], p + ppc));
    }
}

// paths per work item of an adaptive continuation when the autotuner timed
// none: long items amortise the end of an item, where a CTA waits for its
// longest path (circle at h = 2e-5: 389, 339, 317, 315 ms at 1024 .. 8192)
constexpr int CONT_PPC_DEFAULT = 4096;

void release_lut_tex(pdds_ctx* ctx) {
  for (int t = 0; t < 4; t++) {
    if (ctx->lut_tex[t]) cudaDestroyTextureObject(ctx->lut_tex[t]);
    if (ctx->lut_arr[t]) cudaFreeArray(ctx->lut_arr[t]);
    ctx->lut_tex[t] = 0;
    ctx->lut_arr[t] = nullptr;
  }
}

namespace {

// Writes one zero byte per 4 KB of a host output buffer.  A device-to-host
// copy into pages that were never touched faults them in from inside the
// copy; touching them from the host thread while the device still runs the
// kernels takes that cost off the critical path (the copy then overwrites
// every byte).
void prefault(void* p, size_t bytes) {
  if (!p) return;
  volatile unsigned char* c = static_cast<volatile unsigned char*>(p);
  for (size_t i = 0; i < bytes; i += 4096) c[i] = 0;
  if (bytes) c[bytes - 1] = 0;
}

// Cubic B-spline coefficients c of the samples f along one line of n nodes
// with stride `stride`, in place: (c_{i-1} + 4 c_i + c_{i+1}) / 6 = f_i, with
// c_{-1} = c_0 and c_n = c_{n-1} (the texture's clamp addressing), so the
// spline the FP32 sampler evaluates passes through every node.  Thomas
// elimination of the tridiagonal system (diagonally dominant).
void bspline_line(double* v, int n, size_t stride, std::vector<double>& cp) {
  cp.resize(n);
  const double off = 1.0 / 6.0;
  double d = 5.0 / 6.0;
  cp[0] = off / d;
  v[0] /= d;
  for (int i = 1; i < n; i++) {
    d = (i == n - 1 ? 5.0 / 6.0 : 4.0 / 6.0) - off * cp[i - 1];
    cp[i] = off / d;
    v[i * stride] = (v[i * stride] - off * v[(i - 1) * stride]) / d;
  }
  for (int i = n - 2; i >= 0; i--) v[i * stride] -= cp[i] * v[(i + 1) * stride];
}

// The float4 textures of the tables coef [ny][nx][8] (fields 0-3 and 4-7),
// linear filtering, clamped, unnormalised coordinates (node k's texel centre
// at k + 0.5): lut_tex[0..1] their cubic B-spline coefficients, lut_tex[2..3]
// the node values.
pdds_status build_lut_tex(pdds_ctx* ctx, const float* coef, int nx, int ny) {
  release_lut_tex(ctx);
  const size_t n = (size_t)nx * ny;
  std::vector<double> c(coef, coef + 8 * n);
  std::vector<double> cp;
  for (int f = 0; f < 8; f++) {
    for (int j = 0; j < ny; j++) bspline_line(c.data() + (size_t)j * nx * 8 + f, nx, 8, cp);
    for (int i = 0; i < nx; i++) bspline_line(c.data() + (size_t)i * 8 + f, ny, (size_t)nx * 8, cp);
  }
  std::vector<float4> tx(n);
  const cudaChannelFormatDesc ch = cudaCreateChannelDesc<float4>();
  for (int t = 0; t < 4; t++) {
    const int h = t & 1;  // fields 4h .. 4h+3
    for (size_t q = 0; q < n; q++) {
      if (t < 2)
        tx[q] = make_float4((float)c[8 * q + 4 * h], (float)c[8 * q + 4 * h + 1], (float)c[8 * q + 4 * h + 2],
                            (float)c[8 * q + 4 * h + 3]);
      else
        tx[q] = make_float4(coef[8 * q + 4 * h], coef[8 * q + 4 * h + 1], coef[8 * q + 4 * h + 2],
                            coef[8 * q + 4 * h + 3]);
    }
    CK(cudaMallocArray(&ctx->lut_arr[t], &ch, nx, ny));
    const size_t pitch = (size_t)nx * sizeof(float4);
    xfer().h2d += (int64_t)(pitch * ny);
    CK(cudaMemcpy2DToArrayAsync(ctx->lut_arr[t], 0, 0, tx.data(), pitch, pitch, ny, cudaMemcpyHostToDevice,
                                ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));  // tx is reused for the second texture
    cudaResourceDesc rd;
    std::memset(&rd, 0, sizeof(rd));
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = ctx->lut_arr[t];
    cudaTextureDesc td;
    std::memset(&td, 0, sizeof(td));
    td.addressMode[0] = cudaAddressModeClamp;
    td.addressMode[1] = cudaAddressModeClamp;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 0;
    CK(cudaCreateTextureObject(&ctx->lut_tex[t], &rd, &td, nullptr));
  }
  return PDDS_OK;
}

}  // namespace

pdds_status upload_layout(pdds_ctx* ctx) {
  drop_graph(ctx);  // the buffers below may move
  ctx->edges_ready = false;
  ctx->has_solution = false;
  ctx->ugrid_m = 0;
  ctx->lpt_ready = false;
  HostLayout& L = ctx->L;
  cudaStream_t s = ctx->stream;
  std::vector<double> st_rect;
  std::vector<int> st_side, st_glob;
  std::vector<int64_t> st_map_off;
  for (auto& st : L.stencils) {
    for (int q = 0; q < 4; q++) {
      st_rect.push_back(st.rect[q]);
      st_side.push_back(st.side[q]);
      st_glob.push_back(st.glob[q]);
    }
    st_map_off.push_back(st.map_off);
  }
  std::vector<int> sd_n, sd_orient, sd_shape;
  std::vector<double> sd_c, sd_origin;
  std::vector<int64_t> sd_knot_off;
  for (auto& sd : L.sides) {
    sd_n.push_back(sd.n);
    sd_orient.push_back(sd.orient);
    sd_shape.push_back(sd.shape);
    sd_c.push_back(sd.c);
    sd_origin.push_back(sd.origin);
    sd_knot_off.push_back(sd.knot_off);
  }
  std::vector<int> sh_n, sh_nbins;
  std::vector<double> sh_c, sh_lo, sh_delta, sh_t, sh_R;
  std::vector<int64_t> sh_tab_off, sh_ipsi_off, sh_t_off;
  int64_t ipsi_len = 0, tab_len = 0;
  int max_n = 0;
  ctx->max_nbins = 0;
  for (auto& sh : L.shapes) {
    sh_n.push_back(sh.n);
    sh_nbins.push_back(sh.nbins);
    sh_c.push_back(sh.c);
    sh_R.push_back(sh.R);
    sh_lo.push_back(sh.lo);
    sh_delta.push_back(sh.delta);
    sh_tab_off.push_back(sh.tab_off);
    sh_ipsi_off.push_back(sh.ipsi_off);
    sh_t_off.push_back((int64_t)sh_t.size());
    for (double v : sh.t) sh_t.push_back(v);
    ipsi_len = std::max<int64_t>(ipsi_len, sh.ipsi_off + (int64_t)sh.n * sh.n);
    tab_len = std::max<int64_t>(tab_len, sh.tab_off + (int64_t)sh.nbins * sh.n);
    max_n = std::max(max_n, sh.n);
    ctx->max_nbins = std::max(ctx->max_nbins, sh.nbins);
  }
  if (max_n > 160) return fail(ctx, PDDS_ERR_INVALID, "stencil side larger than 160 knots");
  std::vector<int> mc, bnd;
  for (int v : L.order) (L.knot_boundary[v] ? bnd : mc).push_back(v);
  ctx->n_mc = (int)mc.size();
  ctx->mc_host = mc;
  ctx->n_bnd = (int)bnd.size();
  // shared-memory needs of the path kernels
  size_t msm = 0, fsm = 0;
  for (auto& st : L.stencils) {
    size_t nb = 0, nn = 0;
    for (int q = 0; q < 4; q++)
      if (st.side[q] >= 0) {
        nb += L.shapes[L.sides[st.side[q]].shape].nbins;
        nn += L.sides[st.side[q]].n;
      }
    msm = std::max(msm, nb);
    fsm = std::max(fsm, nn);
  }
  ctx->mixed_smem = msm * sizeof(float);
  ctx->fp64_smem = (FP64_THREADS / 32 + 1) * fsm * sizeof(double);  // per-warp sums, knot coordinates
  // the layout's arrays in one device block: one allocation and one copy
  // (a small pageable copy or an allocation costs about as much as the
  // whole 3 MB block of the 12x12/43 layout)
  std::vector<int64_t> st_col_off;
  std::vector<int32_t> st_cols;
  layout_stencil_cols(L, st_col_off, st_cols);  // G's columns, expanded on the device
  std::vector<int> kr(L.knot_rng.begin(), L.knot_rng.end());
  PackedUpload pk;
  pk.add(ctx->kx, L.kx);
  pk.add(ctx->ky, L.ky);
  pk.add(ctx->knot_stencil, L.knot_stencil);
  pk.add(ctx->row_ptr, L.row_ptr);
  pk.add(ctx->st_col_off, st_col_off);
  pk.add(ctx->st_cols, st_cols);
  pk.add(ctx->st_rect, st_rect);
  pk.add(ctx->st_side, st_side);
  pk.add(ctx->st_glob, st_glob);
  pk.add(ctx->st_map_off, st_map_off);
  pk.add(ctx->map_pos, L.map_pos);
  pk.add(ctx->map_owner, L.map_owner);
  pk.add(ctx->sd_n, sd_n);
  pk.add(ctx->sd_orient, sd_orient);
  pk.add(ctx->sd_shape, sd_shape);
  pk.add(ctx->sd_c, sd_c);
  pk.add(ctx->sd_origin, sd_origin);
  pk.add(ctx->sd_knot_off, sd_knot_off);
  pk.add(ctx->side_knot, L.side_knot);
  pk.add(ctx->side_px, L.side_px);
  pk.add(ctx->side_py, L.side_py);
  pk.add(ctx->sh_n, sh_n);
  pk.add(ctx->sh_nbins, sh_nbins);
  pk.add(ctx->sh_c, sh_c);
  pk.add(ctx->sh_R, sh_R);
  pk.add(ctx->sh_lo, sh_lo);
  pk.add(ctx->sh_delta, sh_delta);
  pk.add(ctx->sh_tab_off, sh_tab_off);
  pk.add(ctx->sh_ipsi_off, sh_ipsi_off);
  pk.add(ctx->sh_t_off, sh_t_off);
  pk.add(ctx->sh_t, sh_t);
  pk.add(ctx->mc_knots, mc);
  pk.add(ctx->bnd_knots, bnd);
  if (!kr.empty()) pk.add(ctx->knot_rng, kr);
  else ctx->knot_rng.release();
  pk.pack();
  CK(ctx->lay_block.resize(pk.host.size()));
  CK(copy_async(ctx->lay_block.p, pk.host.data(), pk.host.size(), cudaMemcpyHostToDevice, s));
  pk.bind(ctx->lay_block.p);
  CK(ctx->col.resize(std::max<int64_t>(L.row_ptr[L.K], 1)));
  CK(launch_expand_cols(L.K, ctx->row_ptr.p, ctx->knot_stencil.p, ctx->st_col_off.p, ctx->st_cols.p, ctx->col.p, s));
  CK(ctx->ipsi.resize(std::max<int64_t>(ipsi_len, 1)));
  CK(ctx->rbf_lu.resize(std::max<int64_t>(ipsi_len, 1)));
  CK(ctx->rbf_uinv.resize(std::max<size_t>(sh_t.size(), 1)));
  CK(ctx->rbf_piv.resize(std::max<size_t>(sh_t.size(), 1)));
  CK(ctx->tab.resize(std::max<int64_t>(tab_len, 1)));
  const int64_t nnz = L.row_ptr[L.K];
  CK(ctx->G.resize(std::max<int64_t>(nnz, 1)));
  CK(ctx->GG.resize(std::max<int64_t>(nnz, 1)));
  CK(ctx->B.resize(std::max(L.K, 1)));
  CK(ctx->BB.resize(std::max(L.K, 1)));
  CK(ctx->Bsum.resize(std::max(L.K, 1)));
  CK(ctx->BBsum.resize(std::max(L.K, 1)));
  CK(ctx->knot_steps.resize(std::max(L.K, 1)));
  DevLayout& d = ctx->dl;
  d.K = L.K;
  d.S = (int)L.stencils.size();
  d.D = (int)L.sides.size();
  d.P = (int)L.shapes.size();
  d.dom[0] = L.sw[0]; d.dom[1] = L.sw[1]; d.dom[2] = L.ne[0]; d.dom[3] = L.ne[1];
  d.geom = L.geom;
  d.radius = L.radius;
  d.sh_R = ctx->sh_R.p;
  d.kx = ctx->kx.p; d.ky = ctx->ky.p; d.knot_stencil = ctx->knot_stencil.p; d.row_ptr = ctx->row_ptr.p;
  d.st_rect = ctx->st_rect.p; d.st_side = ctx->st_side.p; d.st_glob = ctx->st_glob.p;
  d.st_map_off = ctx->st_map_off.p; d.map_pos = ctx->map_pos.p; d.map_owner = ctx->map_owner.p;
  d.sd_n = ctx->sd_n.p; d.sd_orient = ctx->sd_orient.p; d.sd_shape = ctx->sd_shape.p;
  d.sd_c = ctx->sd_c.p; d.sd_origin = ctx->sd_origin.p; d.sd_knot_off = ctx->sd_knot_off.p;
  d.side_knot = ctx->side_knot.p; d.side_px = ctx->side_px.p; d.side_py = ctx->side_py.p;
  d.sh_n = ctx->sh_n.p; d.sh_c = ctx->sh_c.p; d.sh_lo = ctx->sh_lo.p; d.sh_delta = ctx->sh_delta.p;
  d.sh_nbins = ctx->sh_nbins.p; d.sh_tab_off = ctx->sh_tab_off.p; d.sh_ipsi_off = ctx->sh_ipsi_off.p;
  d.sh_t_off = ctx->sh_t_off.p; d.sh_t = ctx->sh_t.p;
  d.tab = ctx->tab.p;
  d.ipsi = ctx->ipsi.p;
  d.knot_inst = ctx->is_batch ? ctx->knot_inst.p : nullptr;
  d.inst_knot0 = ctx->is_batch ? ctx->inst_knot0.p : nullptr;
  d.inst_p = ctx->is_batch ? ctx->inst_pd.p : nullptr;
  d.inst_h = ctx->is_batch ? ctx->inst_hd.p : nullptr;
  d.knot_rng = kr.empty() ? nullptr : ctx->knot_rng.p;
  ctx->tables_ready = false;
  return PDDS_OK;
}

ProblemDev problem_dev(const pdds_ctx* ctx) {
  const pdds_problem_desc& p = ctx->prob;
  ProblemDev d;
  d.kind = p.kind;
  d.use_cv = p.use_cv;
  for (int i = 0; i < 8; i++) d.p[i] = p.p[i];
  d.lut.coef = reinterpret_cast<const float4*>(ctx->lut_coef.p);
  d.lut.g = ctx->lut_g.p;
  d.lut.nx = ctx->lut_nx;
  d.lut.ny = ctx->lut_ny;
  d.lut.x0 = ctx->lut_bounds[0];
  d.lut.y0 = ctx->lut_bounds[1];
  d.lut.inv_dx = ctx->lut_nx > 1 ? 1.0 / ((ctx->lut_bounds[2] - ctx->lut_bounds[0]) / (ctx->lut_nx - 1)) : 0.0;
  d.lut.inv_dy = ctx->lut_ny > 1 ? 1.0 / ((ctx->lut_bounds[3] - ctx->lut_bounds[1]) / (ctx->lut_ny - 1)) : 0.0;
  // the FP32 sampler by p[0]: 0 cubic B-spline (textures), 1 Catmull-Rom
  // (node loads), 2 bilinear (textures)
  const int sm = p.kind == PK_LUT && ctx->lut_tex[0] ? (p.p[0] == 1.0 ? 0 : (p.p[0] == 2.0 ? 2 : 1)) : 0;
  d.lut.tex_mode = sm;
  d.lut.tex[0] = sm ? (unsigned long long)ctx->lut_tex[sm == 2 ? 2 : 0] : 0ull;
  d.lut.tex[1] = sm ? (unsigned long long)ctx->lut_tex[sm == 2 ? 3 : 1] : 0ull;
  return d;
}

pdds_status check_err_flags(pdds_ctx* ctx) {
  unsigned f = 0;
  CK(copy_async(&f, ctx->errf.p, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (f & ERR_FLAG_SINGULAR) return fail(ctx, PDDS_ERR_ILL_CONDITIONED, "RBF matrix numerically singular");
  if (f & ERR_FLAG_STEP_LIMIT) return fail(ctx, PDDS_ERR_STEP_LIMIT, "a path exceeded max_steps");
  if (f & ERR_FLAG_EXIT_SIDE) return fail(ctx, PDDS_ERR_EXIT_SIDE, "an exit matched no stencil side");
  if (f & ERR_FLAG_SUB_NOCONV)
    return fail(ctx, PDDS_ERR_NOT_CONVERGED, "a subdomain solve missed its tolerance in 200 iterations");
  if (f & ERR_FLAG_TIMEOUT) return fail(ctx, PDDS_ERR_TIMEOUT, "a grid barrier of the interface solve timed out");
  if (f & ERR_FLAG_BOUNDS)
    return fail(ctx, PDDS_ERR_BOUNDS, "a device index check failed (checked build): an access was skipped");
  return PDDS_OK;
}

pdds_status enqueue_prefix(pdds_ctx* ctx, const pdds_estimate_desc* desc, const ProblemDev& P, bool events,
                           int* launches) {
  cudaStream_t s = ctx->stream;
  HostLayout& L = ctx->L;
  const int mode = desc->mode;
  const int64_t nnz = L.row_ptr[L.K];
  if (events) CK(cudaEventRecord(ctx->ev0, s));
  CK(cudaMemsetAsync(ctx->errf.p, 0, sizeof(unsigned), s));
  CK(cudaMemsetAsync(ctx->stats.p, 0, 8 * sizeof(unsigned long long), s));
  const bool need_ipsi = !(mode == PDDS_MODE_REPLAY_FP64 && desc->ipsi_override);
  if (need_ipsi && (!ctx->tables_ready || !desc->reuse_tables)) {
    int max_n = 0;
    for (auto& sh : L.shapes) max_n = std::max(max_n, sh.n);
    CK(launch_rbf_setup(ctx->dl, max_n, ctx->max_nbins, ctx->ipsi.p, ctx->tab.p, ctx->rbf_lu.p, ctx->rbf_piv.p,
                        ctx->rbf_uinv.p, ctx->errf.p, s));
    *launches += 4;
    ctx->tables_ready = true;
  }
  if (events) CK(cudaEventRecord(ctx->ev1, s));
  CK(cudaMemsetAsync(ctx->G.p, 0, std::max<int64_t>(nnz, 1) * sizeof(double), s));
  CK(cudaMemsetAsync(ctx->GG.p, 0, std::max<int64_t>(nnz, 1) * sizeof(double), s));
  CK(cudaMemsetAsync(ctx->Bsum.p, 0, L.K * sizeof(double), s));
  CK(cudaMemsetAsync(ctx->BBsum.p, 0, L.K * sizeof(double), s));
  CK(cudaMemsetAsync(ctx->knot_steps.p, 0, L.K * sizeof(unsigned long long), s));
  CK(ctx->step_hist.resize(32));
  CK(cudaMemsetAsync(ctx->step_hist.p, 0, 32 * sizeof(unsigned long long), s));
  ctx->has_knot_steps = (mode == PDDS_MODE_MIXED);
  CK(launch_boundary_b(ctx->dl, P, mode, ctx->bnd_knots.p, ctx->n_bnd, ctx->B.p, ctx->BB.p, s));
  *launches += ctx->n_bnd > 0;
  return PDDS_OK;
}

// Items are (knot, chunk of paths): enough chunks per knot to give every SM
// several items, but at least 256 paths per chunk.
bool tuned_for(const pdds_ctx* ctx, const pdds_estimate_desc* desc) {
  return ctx->tune_ppc > 0 && ctx->tune_kind == ctx->prob.kind && ctx->tune_rich == (desc->richardson ? 1 : 0);
}

// threads per CTA of the MIXED path kernel for this estimate: the caller's,
// else the autotuned one for this problem kind, else by layout size
int cta_threads_for(const pdds_ctx* ctx, const pdds_estimate_desc* d) {
  if (d && d->cta_threads > 0) return d->cta_threads;
  if (d && tuned_for(ctx, d) && ctx->tune_threads > 0) return ctx->tune_threads;
  return mixed_threads(ctx->n_mc);
}

void item_split(const pdds_ctx* ctx, int N, int* chunks_out, int* ppc_out, int tuned_ppc = 0, int threads = 0,
                int n_knots = -1) {
  if (tuned_ppc > 0) {
    const int ppc = std::max(1, std::min(N, tuned_ppc));
    *chunks_out = (N + ppc - 1) / ppc;
    *ppc_out = ppc;
    return;
  }
  // about four items per persistent CTA (1024 / threads CTAs per SM)
  const int n_mc = n_knots >= 0 ? n_knots : ctx->n_mc;
  const int target = 4 * std::max(ctx->num_sms, 1) * (1024 / (threads > 0 ? threads : mixed_threads(ctx->n_mc)));
  int chunks = std::max(1, (target + std::max(n_mc, 1) - 1) / std::max(n_mc, 1));
  chunks = std::min(chunks, std::max(1, N / 256));
  const int ppc = (N + chunks - 1) / chunks;
  *chunks_out = (N + ppc - 1) / ppc;
  *ppc_out = ppc;
}

// explicit work items of a continuation pass (variance-adaptive paths)
struct ItemList {
  const int* knot;
  const int* p0;
  const int* p1;
  int n;
  const double* knot_invN;
};

pdds_status enqueue_mixed_paths(pdds_ctx* ctx, const pdds_estimate_desc* desc, const ProblemDev& P, int chunks,
                                int ppc, int* launches, const ItemList* items = nullptr, int mc0 = 0,
                                int mc_n = -1) {
  cudaStream_t s = ctx->stream;
  if (mc_n < 0) mc_n = ctx->n_mc;
  if (!items && P.kind == PK_ROBIN && (int)P.p[0] != 0 && !ctx->is_batch && mc0 == 0 && mc_n == ctx->n_mc) {
    // Knots whose stencil has a reflecting side take several times the
    // steps per path of the others (their paths leave only through the
    // absorbing sides): they go first, in chunks of an eighth of the paths,
    // so that no single long item sets the end of the launch.
    const HostLayout& L = ctx->L;
    const int rm = (int)P.p[0], N = desc->npaths;
    const int small = std::max(256, ppc / 8);
    std::vector<int> ik, ip0, ip1, other;
    for (int v : L.order) {
      if (L.knot_boundary[v]) continue;
      const StencilRec& st = L.stencils[L.knot_stencil[v]];
      bool refl = false;
      for (int d = 0; d < 4; d++) refl = refl || (st.glob[d] && (rm & (1 << d)));
      if (!refl) {
        other.push_back(v);
        continue;
      }
      for (int p = 0; p < N; p += small) {
        ik.push_back(v);
        ip0.push_back(p);
        ip1.push_back(std::min(N, p + small));
      }
    }
    for (int v : other)
      for (int p = 0; p < N; p += ppc) {
        ik.push_back(v);
        ip0.push_back(p);
        ip1.push_back(std::min(N, p + ppc));
      }
    CK(ctx->item_knot.upload(ik, s));
    CK(ctx->item_p0.upload(ip0, s));
    CK(ctx->item_p1.upload(ip1, s));
    const ItemList il{ctx->item_knot.p, ctx->item_p0.p, ctx->item_p1.p, (int)ik.size(), nullptr};
    return enqueue_mixed_paths(ctx, desc, P, 1, ppc, launches, &il);
  }
  const int N = desc->npaths;
  const int n_items = items ? items->n : mc_n * chunks;
  const long long max_steps = desc->max_steps > 0 ? desc->max_steps : 1000000LL;
  CK(cudaMemsetAsync(ctx->counter.p, 0, sizeof(int), s));
  MixedArgs a{};
  a.L = ctx->dl;
  a.P = P;
  a.N = N;
  a.h = (float)desc->h;
  a.sqrth = (float)std::sqrt(desc->h);
  a.inv_N = 1.0 / N;
  mixed_set_rng(a, desc->seed, desc->instance);
  a.chunks = chunks;
  a.paths_per_chunk = ppc;
  a.n_items = n_items;
  a.want_var = desc->want_var ? 1 : 0;
  a.dup_sum = ctx->L.geom == 1 ? 1 : desc->dup_sum;  // circle layouts sum shared side knots
  a.adaptive_h = desc->adaptive_h ? 1 : 0;
  a.richardson = desc->richardson ? 1 : 0;
  a.h64 = desc->h;
  a.max_steps = max_steps;
  // work items of the default split are handed out heaviest knot first: by
  // the steps per knot that the last estimate on this layout counted, or
  // before the first one by a geometric estimate of the steps per path
  const bool lpt = !items && !ctx->is_batch && !desc->plain_launch && mc0 == 0 && mc_n == ctx->n_mc;
  if (lpt && !ctx->lpt_ready && ctx->L.geom == 0) {
    // E[steps] ~ tau / h_k: tau = tx ty / (tx + ty) combines the expected
    // exit times a (w - a) / 2 across the stencil in x and in y, h_k is the
    // knot's step (the adaptive one shrinks with the distance d to the
    // nearest side).  It ranks the heavy knots (the cross knots of large
    // stencils and knots close to a side) near the top.
    const HostLayout& L = ctx->L;
    std::vector<std::pair<double, int>> cost;
    for (int v : L.order) {
      if (L.knot_boundary[v]) continue;
      const double* r = L.stencils[L.knot_stencil[v]].rect;
      const double ax = L.kx[v] - r[0], bx = r[2] - L.kx[v], ay = L.ky[v] - r[1], by = r[3] - L.ky[v];
      const double tx = 0.5 * std::max(ax * bx, 0.0), ty = 0.5 * std::max(ay * by, 0.0);
      const double tau = tx + ty > 0.0 ? tx * ty / (tx + ty) : 0.0;
      const double d = std::min(std::min(ax, bx), std::min(ay, by));
      double hk = desc->h;
      if (desc->adaptive_h && d > 1e-4) hk = std::min(hk, std::pow(d / (2.0 * 0.5826 * 1.4142135623730951), 2.0));
      cost.push_back({-tau / hk, v});
    }
    std::stable_sort(cost.begin(), cost.end());
    std::vector<int> ord;
    ord.reserve(cost.size());
    for (auto& c : cost) ord.push_back(c.second);
    CK(ctx->mc_lpt.upload(ord, s));
    ctx->lpt_ready = true;
  }
  a.mc_knots = (lpt && ctx->lpt_ready) ? ctx->mc_lpt.p : ctx->mc_knots.p + mc0;
  a.item_counter = ctx->counter.p;
  a.G = ctx->G.p;
  a.GG = ctx->GG.p;
  a.Bsum = ctx->Bsum.p;
  a.BBsum = ctx->BBsum.p;
  a.stats = ctx->stats.p;
  a.err_flags = ctx->errf.p;
  a.item_knot = items ? items->knot : nullptr;
  a.item_p0 = items ? items->p0 : nullptr;
  a.item_p1 = items ? items->p1 : nullptr;
  a.knot_invN = items ? items->knot_invN : nullptr;
  a.knot_steps = ctx->knot_steps.p;
  a.step_hist = desc->step_histogram ? ctx->step_hist.p : nullptr;
  a.diag = (desc->diagnostics && ctx->diag.n >= (size_t)ctx->L.K * PDDS_DIAG_N) ? ctx->diag.p : nullptr;
  const int threads = cta_threads_for(ctx, desc);
  const size_t smem = ctx->mixed_smem * (a.want_var ? 2 : 1) + mixed_queue_smem(threads, a.richardson);
  if (smem > 200 * 1024) return fail(ctx, PDDS_ERR_INVALID, "exit histograms exceed shared memory; lower bins_per_gap");
  const int mk = mixed_kind(P);
  int bps = mixed_blocks_per_sm(mk, smem, a.richardson, threads, a.diag != nullptr);
  if (bps < 1) bps = 1;
  if (ctx->force_bps > 0) bps = std::min(bps, ctx->force_bps);
  else if (tuned_for(ctx, desc) && !items) bps = std::min(bps, ctx->tune_bps);  // the shape it was timed on
  int grid = std::max(1, std::min(n_items, bps * ctx->num_sms));
  if (desc->plain_launch) grid = std::max(1, n_items);  // one CTA per work item
  if (ctx->force_grid_frac > 0.0 && ctx->force_grid_frac < 1.0)
    grid = std::max(1, std::min(grid, (int)std::lround(ctx->force_grid_frac * bps * ctx->num_sms)));
  if (n_items > 0) {
    CK(launch_paths_mixed(a, mk, grid, threads, smem, s));
    ++*launches;
    if (lpt) {
      CK(ctx->mc_lpt.resize(std::max(ctx->n_mc, 1)));
      CK(launch_lpt_order(ctx->mc_knots.p, ctx->n_mc, ctx->knot_steps.p, ctx->mc_lpt.p, s));
      ++*launches;
      ctx->lpt_ready = true;
    }
  }
  return PDDS_OK;
}

// Variance-adaptive paths per knot after a pilot of desc->npaths paths
// (Compute_h_N, PDDSparseGM.cpp:4338-4395): N_k = 4 V_k / (0.66666 eps)^2,
// rounded up to the next multiple of 256 as the reference rounds to N_job,
// clamped to [N0, npaths_max]; paths N0 .. N_k-1 continue the knot's Philox
// streams.  Synchronises once to read the pilot's sums.
pdds_status adaptive_continue(pdds_ctx* ctx, const pdds_estimate_desc* desc, const ProblemDev& P, int* launches) {
  cudaStream_t s = ctx->stream;
  const HostLayout& L = ctx->L;
  const int K = L.K;
  const int N0 = desc->npaths;
  const int nmax = std::max(N0, desc->npaths_max > 0 ? desc->npaths_max : 100000);
  const double eps = desc->target_stderr > 0 ? desc->target_stderr : 1e-3;
  std::vector<double> bs(K), bbs(K);
  std::vector<unsigned long long> pst(K);
  CK(copy_async(bs.data(), ctx->Bsum.p, K * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(copy_async(bbs.data(), ctx->BBsum.p, K * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(copy_async(pst.data(), ctx->knot_steps.p, K * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  std::vector<int> kn(K, 0), ik, ip0, ip1;
  std::vector<double> scale(K, 1.0), inv(K, 0.0);
  std::vector<std::pair<double, int>> cost;  // the continuation's steps per knot, from the pilot
  const int granule = 256;
  const int ppc = tuned_for(ctx, desc) && ctx->tune_cont_ppc > 0 ? ctx->tune_cont_ppc : CONT_PPC_DEFAULT;
  for (int v : L.order) {
    if (L.knot_boundary[v]) continue;
    const double mean = bs[v] / N0;
    const double var = std::max(0.0, bbs[v] / N0 - mean * mean);
    const double want = 4.0 * var / ((eps * 0.66666) * (eps * 0.66666));
    long long nk = want < 2e9 ? (long long)want : 2000000000LL;
    nk = (1 + nk / granule) * granule;
    nk = std::max<long long>(N0, std::min<long long>(nmax, nk));
    kn[v] = (int)nk;
    scale[v] = (double)N0 / (double)nk;
    inv[v] = 1.0 / (double)nk;
    if (nk > N0) cost.push_back({-(double)pst[v] * (double)(nk - N0) / (double)N0, v});
  }
  // work items heaviest knot first, so that no long item starts near the end
  std::stable_sort(cost.begin(), cost.end());
  std::vector<int> order;
  order.reserve(cost.size());
  for (auto& c : cost) order.push_back(c.second);
  continuation_items(order, kn, N0, ppc, ik, ip0, ip1);
  ctx->last_knot_N = kn;
  CK(ctx->knot_N.upload(kn, s));
  CK(ctx->knot_scale.upload(scale, s));
  CK(ctx->knot_invN.upload(inv, s));
  CK(launch_scale_rows(ctx->mc_knots.p, ctx->n_mc, ctx->row_ptr.p, ctx->knot_scale.p, ctx->G.p,
                       desc->want_var ? ctx->GG.p : nullptr, s));
  ++*launches;
  // kept for the autotuner, which times this continuation's shapes
  ctx->cont_knots = order;
  ctx->cont_N0 = N0;
  ctx->cont_kind = ctx->prob.kind;
  if (!ik.empty()) {
    CK(ctx->item_knot.upload(ik, s));
    CK(ctx->item_p0.upload(ip0, s));
    CK(ctx->item_p1.upload(ip1, s));
    ItemList items{ctx->item_knot.p, ctx->item_p0.p, ctx->item_p1.p, (int)ik.size(), ctx->knot_invN.p};
    pdds_estimate_desc dc = *desc;  // the continuation's block size, when the autotuner timed one
    if (dc.cta_threads == 0 && tuned_for(ctx, desc) && ctx->tune_cont_threads > 0)
      dc.cta_threads = ctx->tune_cont_threads;
    pdds_status st = enqueue_mixed_paths(ctx, &dc, P, 1, ppc, launches, &items);
    if (st != PDDS_OK) return st;
  }
  return PDDS_OK;
}

pdds_status enqueue_mixed(pdds_ctx* ctx, const pdds_estimate_desc* desc, int* launches, int mc0, int mc_n,
                          bool prefix) {
  const ProblemDev P = problem_dev(ctx);
  if (prefix) {
    pdds_status st = enqueue_prefix(ctx, desc, P, false, launches);
    if (st != PDDS_OK) return st;
  }
  if (mc_n < 0) mc_n = ctx->n_mc - mc0;
  if (mc_n == 0) return PDDS_OK;
  int chunks = 1, ppc = 1;
  item_split(ctx, desc->npaths, &chunks, &ppc, tuned_for(ctx, desc) ? ctx->tune_ppc : 0, cta_threads_for(ctx, desc),
             mc_n);
  pdds_status st = enqueue_mixed_paths(ctx, desc, P, chunks, ppc, launches, nullptr, mc0, mc_n);
  if (st != PDDS_OK) return st;
  // finalisation of the range's knots: B and BB, and G_var over the range's rows
  const HostLayout& L = ctx->L;
  int64_t e0 = 0, e1 = L.row_ptr[L.K];
  if (!(mc0 == 0 && mc_n == ctx->n_mc)) {  // the rows of the range's knots
    e0 = e1;
    e1 = 0;
    for (int m = mc0; m < mc0 + mc_n; m++) {
      const int k = ctx->mc_host[m];
      e0 = std::min(e0, L.row_ptr[k]);
      e1 = std::max(e1, L.row_ptr[k + 1]);
    }
  }
  CK(launch_finalize(ctx->mc_knots.p + mc0, mc_n, desc->npaths, ctx->Bsum.p, ctx->BBsum.p, ctx->B.p, ctx->BB.p,
                     ctx->row_ptr.p, e1 - e0, ctx->G.p + e0, ctx->GG.p + e0, desc->want_var ? 1 : 0, ctx->stream));
  *launches += 1 + (desc->want_var ? 1 : 0);
  return PDDS_OK;
}

}  // namespace pdds

extern "C" {

const char* pdds_version(void) { return "pdds_gb300 0.1 (sm_103a)"; }

pdds_status pdds_create(pdds_ctx** out, int device, uint32_t flags) {
  (void)flags;
  if (!out) return PDDS_ERR_INVALID;
  pdds_ctx* ctx = new pdds_ctx();
  ctx->device = device;
  if (device >= 0) {
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev2);
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->host_rr, sizeof(double));
    if (e == cudaSuccess) e = ctx->stats.resize(8);
    if (e == cudaSuccess) e = ctx->errf.resize(1);
    if (e == cudaSuccess) e = ctx->counter.resize(1);
    if (e != cudaSuccess) {
      delete ctx;
      return PDDS_ERR_CUDA;
    }
  }
  *out = ctx;
  return PDDS_OK;
}

pdds_status pdds_release_cached_blocks(int32_t device) {
  block_cache_clear(device);
  return PDDS_OK;
}

pdds_status pdds_destroy(pdds_ctx* ctx) {
  if (!ctx) return PDDS_ERR_INVALID;
  if (ctx->device >= 0) {
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->solve_stream) cudaStreamSynchronize(ctx->solve_stream);
    // both streams are idle: the buffers go to the block cache for the next
    // context
    DBuf<double>* d64[] = {&ctx->kx, &ctx->ky, &ctx->st_rect, &ctx->sd_c, &ctx->sd_origin, &ctx->side_px,
                           &ctx->side_py, &ctx->sh_c, &ctx->sh_R, &ctx->sh_lo, &ctx->sh_delta, &ctx->sh_t, &ctx->ipsi,
                           &ctx->G, &ctx->GG, &ctx->B, &ctx->BB, &ctx->Bsum, &ctx->BBsum, &ctx->rx,
                           &ctx->ry, &ctx->rY, &ctx->rZ, &ctx->rxi, &ctx->Gside, &ctx->GGside,
                           &ctx->ipsi_knot, &ctx->sv64, &ctx->sscal, &ctx->spart, &ctx->shess, &ctx->su,
                           &ctx->rbf_lu, &ctx->rbf_uinv};
    for (auto* b : d64) b->recycle();
    DBuf<int>* di[] = {&ctx->knot_stencil, &ctx->st_side, &ctx->st_glob, &ctx->map_pos, &ctx->sd_n,
                       &ctx->sd_orient, &ctx->sd_shape, &ctx->side_knot, &ctx->sh_n, &ctx->sh_nbins,
                       &ctx->col, &ctx->mc_knots, &ctx->bnd_knots, &ctx->counter, &ctx->rside,
                       &ctx->rsl, &ctx->rss, &ctx->task_m, &ctx->task_d, &ctx->task_i, &ctx->rbf_piv};
    for (auto* b : di) b->recycle();
    DBuf<int64_t>* dl[] = {&ctx->row_ptr, &ctx->st_map_off, &ctx->sd_knot_off, &ctx->sh_tab_off,
                           &ctx->sh_ipsi_off, &ctx->sh_t_off, &ctx->task_out, &ctx->knot_task_off,
                           &ctx->knot_ipsi_off};
    for (auto* b : dl) b->recycle();
    ctx->st_col_off.recycle();
    ctx->st_cols.recycle();
    ctx->map_owner.recycle();
    ctx->lay_block.recycle();
    ctx->knot_rng.recycle();
    ctx->tab.recycle();
    ctx->lut_coef.recycle();
    ctx->lut_g.recycle();
    release_lut_tex(ctx);
    ctx->stats.recycle();
    ctx->errf.recycle();
    ctx->sV32.recycle();
    ctx->sZ32.recycle();
    ctx->sw32.recycle();
    ctx->sval32.recycle();
    ctx->sctl.recycle();
    ctx->sgpart.recycle();
    ctx->sbar.recycle();
    drop_graph(ctx);
    ctx->knot_inst.recycle();
    ctx->inst_knot0.recycle();
    ctx->b_iters.recycle();
    ctx->b_refines.recycle();
    ctx->inst_pd.recycle();
    ctx->inst_hd.recycle();
    ctx->b_relres.recycle();
    ctx->b_tend.recycle();
    ctx->knot_N.recycle();
    ctx->knot_steps.recycle();
    ctx->mc_lpt.recycle();
    ctx->edge_knots.recycle();
    ctx->sub_u.recycle();
    ctx->sub_out.recycle();
    ctx->sub_work.recycle();
    ctx->sub_iters.recycle();
    ctx->ugrid.recycle();
    ctx->item_knot.recycle();
    ctx->item_p0.recycle();
    ctx->item_p1.recycle();
    ctx->knot_scale.recycle();
    ctx->knot_invN.recycle();
    ctx->step_hist.recycle();
    for (auto* b : {&ctx->diag, &ctx->rsx, &ctx->rsy, &ctx->rsY, &ctx->rsZ, &ctx->rsxi, &ctx->rknot_h}) b->recycle();
    if (ctx->host_rr) cudaFreeHost(ctx->host_rr);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->ev2) cudaEventDestroy(ctx->ev2);
    for (cudaEvent_t ev : ctx->wave_ev) cudaEventDestroy(ev);
    if (ctx->solve_stream) cudaStreamDestroy(ctx->solve_stream);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
  }
  delete ctx;
  return PDDS_OK;
}

const char* pdds_last_error(const pdds_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

pdds_status pdds_problem_set(pdds_ctx* ctx, const pdds_problem_desc* desc) {
  if (!ctx || !desc) return PDDS_ERR_INVALID;
  if (desc->kind < 0 || desc->kind > 6) return fail(ctx, PDDS_ERR_INVALID, "unknown problem kind");
  if (desc->kind == PDDS_ROBIN_POISSON) {
    const double mk = desc->p[0];
    if (!(mk == 0.0 || mk == 1.0 || mk == 2.0 || mk == 4.0 || mk == 8.0))
      return fail(ctx, PDDS_ERR_INVALID,
                  "PDDS_ROBIN_POISSON: p[0] names at most one Robin side (N 1, S 2, E 4, W 8; 0 none)");
  }
  if (desc->kind == PDDS_LUT && ctx->lut_nx < 4)
    return fail(ctx, PDDS_ERR_INVALID, "PDDS_LUT needs pdds_problem_set_lut first");
  if (desc->kind == PDDS_HELMHOLTZ && desc->p[2] > 0.0)
    return fail(ctx, PDDS_ERR_INVALID, "Helmholtz reaction c must be <= 0");
  drop_graph(ctx);  // a captured batch sequence holds the problem by value
  ctx->prob = *desc;
  ctx->has_problem = true;
  return PDDS_OK;
}

pdds_status pdds_problem_set_lut(pdds_ctx* ctx, const float* coef, const float* g, int32_t nx, int32_t ny,
                                 const double bounds[4]) {
  if (!ctx || !coef || !g || !bounds) return PDDS_ERR_INVALID;
  if (nx < 4 || ny < 4) return fail(ctx, PDDS_ERR_INVALID, "tables need at least 4 x 4 nodes");
  if (!(bounds[2] > bounds[0] && bounds[3] > bounds[1])) return fail(ctx, PDDS_ERR_INVALID, "bad table bounds");
  if (ctx->device < 0) return fail(ctx, PDDS_ERR_INVALID, "context has no device");
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  drop_graph(ctx);
  const size_t n = (size_t)nx * ny;
  CK(ctx->lut_coef.resize(8 * n));
  CK(ctx->lut_g.resize(n));
  CK(copy_async(ctx->lut_coef.p, coef, 8 * n * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  CK(copy_async(ctx->lut_g.p, g, n * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  const pdds_status st = build_lut_tex(ctx, coef, nx, ny);
  if (st != PDDS_OK) return st;
  ctx->lut_nx = nx;
  ctx->lut_ny = ny;
  for (int q = 0; q < 4; q++) ctx->lut_bounds[q] = bounds[q];
  return PDDS_OK;
}

pdds_status pdds_layout_build(pdds_ctx* ctx, const pdds_layout_desc* desc, pdds_layout_info* info) {
  if (!ctx || !desc) return PDDS_ERR_INVALID;
  for (int q = 0; q < 4; q++)
    if (!(desc->fac[q] > 0.0)) return fail(ctx, PDDS_ERR_INVALID, "fac must be positive");
  if (ctx->device >= 0) {
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  drop_graph(ctx);
  clear_tune(ctx);
  ctx->is_batch = false;
  ctx->n_inst = 0;
  ctx->has_batch_run = false;
  const std::string e = build_rect_layout(ctx->L, desc->sw, desc->ne, desc->nsub, desc->nnode, desc->fac,
                                          ctx->bins);
  if (!e.empty()) return fail(ctx, PDDS_ERR_INVALID, e);
  ctx->has_layout = true;
  ctx->has_estimate = false;
  const int64_t h2d0 = xfer().h2d;
  if (ctx->device >= 0) {
    pdds_status st = upload_layout(ctx);
    if (st != PDDS_OK) return st;
  }
  if (info) {
    info->h2d_bytes = xfer().h2d - h2d0;
    info->nknots = ctx->L.K;
    info->nboundary = ctx->L.nboundary;
    info->nstencils = (int)ctx->L.stencils.size();
    info->nsides = (int)ctx->L.sides.size();
    info->nshapes = (int)ctx->L.shapes.size();
    info->max_side = ctx->L.max_side;
    info->nnz = ctx->L.row_ptr[ctx->L.K];
  }
  return PDDS_OK;
}

pdds_status pdds_layout_build_circle(pdds_ctx* ctx, const pdds_circle_desc* desc, pdds_layout_info* info) {
  if (!ctx || !desc) return PDDS_ERR_INVALID;
  for (int q = 0; q < 4; q++)
    if (!(desc->kappa[q] > 0.0)) return fail(ctx, PDDS_ERR_INVALID, "kappa must be positive");
  if (ctx->device >= 0) {
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  drop_graph(ctx);
  clear_tune(ctx);
  ctx->is_batch = false;
  ctx->n_inst = 0;
  ctx->has_batch_run = false;
  if (!(desc->ring_ratio >= 0.0)) return fail(ctx, PDDS_ERR_INVALID, "ring_ratio must be >= 0");
  const std::string e = build_circle_layout(ctx->L, desc->radius, desc->nrings, desc->nsectors, desc->nnode,
                                            desc->kappa, ctx->bins, desc->ring_ratio > 0.0 ? desc->ring_ratio : 1.0);
  if (!e.empty()) return fail(ctx, PDDS_ERR_INVALID, e);
  ctx->has_layout = true;
  ctx->has_estimate = false;
  const int64_t h2d0 = xfer().h2d;
  if (ctx->device >= 0) {
    pdds_status st = upload_layout(ctx);
    if (st != PDDS_OK) return st;
  }
  if (info) {
    info->h2d_bytes = xfer().h2d - h2d0;
    info->nknots = ctx->L.K;
    info->nboundary = ctx->L.nboundary;
    info->nstencils = (int)ctx->L.stencils.size();
    info->nsides = (int)ctx->L.sides.size();
    info->nshapes = (int)ctx->L.shapes.size();
    info->max_side = ctx->L.max_side;
    info->nnz = ctx->L.row_ptr[ctx->L.K];
  }
  return PDDS_OK;
}

pdds_status pdds_stencils_set(pdds_ctx* ctx, const double domain[4], int32_t nknots, const double* x,
                              const double* y, const int32_t* knot_id, const pdds_stencil_desc* st,
                              pdds_layout_info* info) {
  if (!ctx || !domain || !x || !y || !st || nknots < 1) return fail(ctx, PDDS_ERR_INVALID, "invalid arguments");
  if (ctx->device >= 0) {
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  drop_graph(ctx);
  clear_tune(ctx);
  ctx->is_batch = false;
  ctx->n_inst = 0;
  ctx->has_batch_run = false;
  std::vector<CustomStencil> cs((size_t)nknots);
  for (int k = 0; k < nknots; k++) {
    for (int q = 0; q < 4; q++) {
      cs[k].rect[q] = st[k].rect[q];
      cs[k].n[q] = st[k].n[q];
      cs[k].index[q] = st[k].index[q];
      cs[k].x[q] = st[k].x[q];
      cs[k].y[q] = st[k].y[q];
      cs[k].c2[q] = st[k].c2[q];
    }
  }
  const std::string e = build_custom_layout(ctx->L, domain, nknots, x, y, knot_id, cs.data(), ctx->bins);
  if (!e.empty()) {
    ctx->has_layout = false;
    ctx->has_estimate = false;
    return fail(ctx, PDDS_ERR_INVALID, e);
  }
  ctx->has_layout = true;
  ctx->has_estimate = false;
  const int64_t h2d0 = xfer().h2d;
  if (ctx->device >= 0) {
    pdds_status s = upload_layout(ctx);
    if (s != PDDS_OK) return s;
  }
  if (info) {
    info->h2d_bytes = xfer().h2d - h2d0;
    info->nknots = ctx->L.K;
    info->nboundary = ctx->L.nboundary;
    info->nstencils = (int)ctx->L.stencils.size();
    info->nsides = (int)ctx->L.sides.size();
    info->nshapes = (int)ctx->L.shapes.size();
    info->max_side = ctx->L.max_side;
    info->nnz = ctx->L.row_ptr[ctx->L.K];
  }
  return PDDS_OK;
}

pdds_status pdds_estimate_knot(pdds_ctx* ctx, const double domain[4], double x0, double y0, int32_t knot_id,
                               const pdds_stencil_desc* st, const pdds_estimate_desc* desc, int32_t* G_j,
                               double* G, double* G_var, int32_t max_nnz, int32_t* nnz, double* B, double* BB,
                               pdds_estimate_info* info) {
  if (!ctx || !desc || !st || !nnz || max_nnz < 0 || knot_id < 0)
    return fail(ctx, PDDS_ERR_INVALID, "invalid arguments");
  pdds_status s = pdds_stencils_set(ctx, domain, 1, &x0, &y0, &knot_id, st, nullptr);
  if (s != PDDS_OK) return s;
  const int64_t len = ctx->L.row_ptr[1];
  *nnz = (int32_t)len;
  if (len > max_nnz) return fail(ctx, PDDS_ERR_INVALID, "G row longer than max_nnz (see *nnz)");
  std::vector<double> val(std::max<int64_t>(len, 1)), var(std::max<int64_t>(len, 1));
  double b = 0.0, bb = 0.0;
  s = pdds_estimate(ctx, desc, val.data(), G_var ? var.data() : nullptr, &b, &bb, info);
  if (s != PDDS_OK) return s;
  if (G_j && len > 0) layout_csr_cols(ctx->L, G_j);
  for (int64_t e = 0; e < len; e++) {
    if (G) G[e] = val[e];
    if (G_var) G_var[e] = var[e];
  }
  if (B) *B = b;
  if (BB) *BB = bb;
  return PDDS_OK;
}

pdds_status pdds_layout_knots(pdds_ctx* ctx, double* x, double* y, int32_t* order) {
  if (!ctx || !ctx->has_layout) return fail(ctx, PDDS_ERR_INVALID, "no layout");
  const HostLayout& L = ctx->L;
  if (x) std::copy(L.kx.begin(), L.kx.end(), x);
  if (y) std::copy(L.ky.begin(), L.ky.end(), y);
  if (order) std::copy(L.order.begin(), L.order.end(), order);
  return PDDS_OK;
}

pdds_status pdds_layout_csr(pdds_ctx* ctx, int64_t* row_ptr, int32_t* col) {
  if (!ctx || !ctx->has_layout) return fail(ctx, PDDS_ERR_INVALID, "no layout");
  if (row_ptr) std::copy(ctx->L.row_ptr.begin(), ctx->L.row_ptr.end(), row_ptr);
  if (col) layout_csr_cols(ctx->L, col);
  return PDDS_OK;
}

pdds_status pdds_layout_stencil(pdds_ctx* ctx, int32_t knot, double* rect, int32_t* kinds,
                                int32_t* sizes, int32_t* idx, int32_t maxn) {
  if (!ctx || !ctx->has_layout) return fail(ctx, PDDS_ERR_INVALID, "no layout");
  const HostLayout& L = ctx->L;
  if (knot < 0 || knot >= L.K) return fail(ctx, PDDS_ERR_INVALID, "knot out of range");
  const StencilRec& st = L.stencils[L.knot_stencil[knot]];
  for (int q = 0; q < 4; q++) {
    if (rect) rect[q] = st.rect[q];
    if (kinds) kinds[q] = st.kind[q];
    const int sd = st.side[q];
    const int n = sd >= 0 ? L.sides[sd].n : 0;
    if (sizes) sizes[q] = n;
    if (n > maxn) return fail(ctx, PDDS_ERR_INVALID, "maxn too small");
    if (idx)
      for (int i = 0; i < n; i++) idx[q * maxn + i] = L.side_knot[L.sides[sd].knot_off + i];
  }
  return PDDS_OK;
}

pdds_status pdds_estimate(pdds_ctx* ctx, const pdds_estimate_desc* desc, double* val, double* var,
                          double* Bout, double* BBout, pdds_estimate_info* info) {
  if (!ctx || !desc) return PDDS_ERR_INVALID;
  if (ctx->device < 0) return fail(ctx, PDDS_ERR_INVALID, "context has no device");
  if (!ctx->has_problem) return fail(ctx, PDDS_ERR_INVALID, "no problem set");
  if (!ctx->has_layout) return fail(ctx, PDDS_ERR_INVALID, "no layout built");
  if (desc->npaths < 1 || !(desc->h > 0.0)) return fail(ctx, PDDS_ERR_INVALID, "npaths >= 1 and h > 0 required");
  const int mode = desc->mode;
  if (mode < 0 || mode > 2) return fail(ctx, PDDS_ERR_INVALID, "unknown mode");
  if (mode == PDDS_MODE_REPLAY_FP64 && desc->richardson)
    return fail(ctx, PDDS_ERR_INVALID, "the replay mode follows the reference and has no Richardson form");
  if (mode == PDDS_MODE_REPLAY_FP64 && ctx->prob.kind == PDDS_MONEGROS)
    return fail(ctx, PDDS_ERR_INVALID, "the Monegros problem has no replay form");
  if (ctx->L.geom == 1 && mode == PDDS_MODE_REPLAY_FP64)
    return fail(ctx, PDDS_ERR_INVALID, "circle layouts have no replay form (MIXED and FP64 modes)");
  if (ctx->L.geom == 1 && ctx->prob.kind != PDDS_POISSON_SINCOS && ctx->prob.kind != PDDS_CIRCLE_POISSON)
    return fail(ctx, PDDS_ERR_INVALID, "circle layouts take the sigma = sqrt2 I problems");
  if (mode == PDDS_MODE_REPLAY_FP64 && ctx->prob.kind == PDDS_CIRCLE_POISSON)
    return fail(ctx, PDDS_ERR_INVALID, "the circle problem has no replay form");
  if (mode == PDDS_MODE_REPLAY_FP64 && ctx->prob.kind == PDDS_ROBIN_POISSON)
    return fail(ctx, PDDS_ERR_INVALID, "the Robin problem has no replay form (MIXED and FP64 modes)");
  if (desc->adaptive_n && mode != PDDS_MODE_MIXED)
    return fail(ctx, PDDS_ERR_INVALID, "variance-adaptive paths (adaptive_n) run in PDDS_MODE_MIXED");
  if (desc->adaptive_n && desc->target_stderr < 0.0) return fail(ctx, PDDS_ERR_INVALID, "target_stderr < 0");
  if (desc->cta_threads != 0 && desc->cta_threads != 128 && desc->cta_threads != 256)
    return fail(ctx, PDDS_ERR_INVALID, "cta_threads must be 0, 128 or 256");
  if (desc->knot_first < 0 || desc->knot_count < 0)
    return fail(ctx, PDDS_ERR_INVALID, "knot_first and knot_count must be >= 0");
  if ((desc->knot_first > 0 || desc->knot_count > 0) && desc->adaptive_n)
    return fail(ctx, PDDS_ERR_INVALID, "a knot range runs a fixed number of paths per knot (adaptive_n = 0)");
  const bool diag = desc->diagnostics != 0;
  if (diag && mode == PDDS_MODE_MIXED && ctx->L.geom == 1)
    return fail(ctx, PDDS_ERR_INVALID, "MIXED diagnostics need rectangular stencils (FP64 mode on circle layouts)");
  if (diag && desc->adaptive_n)
    return fail(ctx, PDDS_ERR_INVALID, "diagnostics need a fixed number of paths per knot (adaptive_n = 0)");
  CK(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  HostLayout& L = ctx->L;
  const XferCount x0 = xfer();
  ctx->has_diag = false;
  if (diag) {
    CK(ctx->diag.resize((size_t)L.K * PDDS_DIAG_N));
    CK(cudaMemsetAsync(ctx->diag.p, 0, (size_t)L.K * PDDS_DIAG_N * sizeof(double), s));
  }
  const int bins = desc->bins_per_gap > 0 ? desc->bins_per_gap : 16;
  if (bins != ctx->bins) {
    ctx->bins = bins;
    set_shape_bins(L, bins);
    pdds_status st = upload_layout(ctx);
    if (st != PDDS_OK) return st;
  }
  const int64_t nnz = L.row_ptr[L.K];
  const long long max_steps = desc->max_steps > 0 ? desc->max_steps : 1000000LL;
  const ProblemDev P = problem_dev(ctx);
  const int N = desc->npaths;
  int launches = 0;
  {
    pdds_status st = enqueue_prefix(ctx, desc, P, true, &launches);
    if (st != PDDS_OK) return st;
  }
  const int n_mc = ctx->n_mc;
  // the hand-out positions this call runs
  const int r0 = desc->knot_first;
  const int rn = desc->knot_count > 0 ? desc->knot_count : n_mc - r0;
  if (r0 > n_mc || (int64_t)r0 + rn > n_mc)
    return fail(ctx, PDDS_ERR_INVALID, "knot range beyond the layout's " + std::to_string(n_mc) + " knots with paths");
  if (mode == PDDS_MODE_REPLAY_FP64) {
    const int64_t total = (int64_t)rn * N;
    CK(ctx->rx.resize(std::max<int64_t>(total, 1)));
    CK(ctx->ry.resize(std::max<int64_t>(total, 1)));
    CK(ctx->rY.resize(std::max<int64_t>(total, 1)));
    CK(ctx->rZ.resize(std::max<int64_t>(total, 1)));
    CK(ctx->rxi.resize(std::max<int64_t>(total, 1)));
    CK(ctx->rside.resize(std::max<int64_t>(total, 1)));
    CK(ctx->rsl.resize(std::max<int64_t>(total, 1)));
    CK(ctx->rss.resize(std::max<int64_t>(total, 1)));
    if (diag) {
      DBuf<double>* db[] = {&ctx->rsx, &ctx->rsy, &ctx->rsY, &ctx->rsZ, &ctx->rsxi};
      for (auto* b : db) CK(b->resize(std::max<int64_t>(total, 1)));
      CK(ctx->rknot_h.resize(std::max(rn, 1)));
    }
    // (knot, side, side knot) tasks of the range's knots in hand-out order;
    // knot m of the range is hand-out position r0 + m (ipsi_override packs
    // every knot, so its offsets count them all)
    std::vector<int> tm, td, ti;
    std::vector<int64_t> tout, ktoff(std::max(rn, 1), 0), kipoff(4 * std::max(rn, 1), -1);
    std::vector<int> mc;
    for (int v : L.order) if (!L.knot_boundary[v]) mc.push_back(v);
    int64_t ipo = 0;
    for (int mg = 0; mg < n_mc; mg++) {
      const StencilRec& st = L.stencils[L.knot_stencil[mc[mg]]];
      const bool in = mg >= r0 && mg < r0 + rn;
      const int m = mg - r0;
      if (in) ktoff[m] = (int64_t)tm.size();
      for (int d = 0; d < 4; d++) {
        if (st.side[d] < 0) continue;
        const int n = L.sides[st.side[d]].n;
        if (in) kipoff[4 * m + d] = ipo;
        ipo += (int64_t)n * n;
        if (!in) continue;
        for (int i = 0; i < n; i++) {
          tm.push_back(m); td.push_back(d); ti.push_back(i);
          tout.push_back((int64_t)tout.size());
        }
      }
    }
    if (desc->ipsi_override && desc->ipsi_override_len != ipo)
      return fail(ctx, PDDS_ERR_INVALID, "ipsi_override_len does not match the layout (expected " +
                                             std::to_string(ipo) + ")");
    CK(ctx->task_m.upload(tm, s));
    CK(ctx->task_d.upload(td, s));
    CK(ctx->task_i.upload(ti, s));
    CK(ctx->task_out.upload(tout, s));
    CK(ctx->knot_task_off.upload(ktoff, s));
    CK(ctx->Gside.resize(std::max<size_t>(tm.size(), 1)));
    CK(ctx->GGside.resize(std::max<size_t>(tm.size(), 1)));
    if (desc->ipsi_override) {
      CK(ctx->knot_ipsi_off.upload(kipoff, s));
      CK(ctx->ipsi_knot.resize(std::max<int64_t>(ipo, 1)));
      CK(copy_async(ctx->ipsi_knot.p, desc->ipsi_override, ipo * sizeof(double),
                         cudaMemcpyHostToDevice, s));
    }
    ReplayArgs a{};
    a.L = ctx->dl;
    a.P = P;
    a.N = N;
    a.h = desc->h;
    a.sqrth = std::sqrt(desc->h);
    a.seed = desc->seed;
    a.instance = desc->instance;
    a.sublinear = 1;
    a.adaptive_h = desc->adaptive_h ? 1 : 0;
    a.max_steps = max_steps;
    a.mc_knots = ctx->mc_knots.p + r0;
    a.n_mc = rn;
    a.knot_ipsi_off = desc->ipsi_override ? ctx->knot_ipsi_off.p : nullptr;
    a.ipsi_knot = desc->ipsi_override ? ctx->ipsi_knot.p : nullptr;
    a.ex = ctx->rx.p; a.ey = ctx->ry.p; a.eY = ctx->rY.p; a.eZ = ctx->rZ.p; a.exi = ctx->rxi.p;
    a.eside = ctx->rside.p; a.esteps_l = ctx->rsl.p; a.esteps_s = ctx->rss.p;
    a.diag = diag ? ctx->diag.p : nullptr;
    a.sx = diag ? ctx->rsx.p : nullptr; a.sy = diag ? ctx->rsy.p : nullptr;
    a.sY = diag ? ctx->rsY.p : nullptr; a.sZ = diag ? ctx->rsZ.p : nullptr;
    a.sxi = diag ? ctx->rsxi.p : nullptr; a.knot_h = diag ? ctx->rknot_h.p : nullptr;
    a.G = ctx->G.p;
    a.GG = ctx->GG.p;
    a.B = ctx->B.p;
    a.BB = ctx->BB.p;
    a.dup_sum = ctx->L.geom == 1 ? 1 : desc->dup_sum;  // circle layouts sum shared side knots
    a.err_flags = ctx->errf.p;
    CK(launch_replay_paths(a, P.kind, s));
    CK(launch_replay_reduce(a, P.kind, ctx->task_m.p, ctx->task_d.p, ctx->task_i.p, (int)tm.size(),
                            ctx->task_out.p, ctx->knot_task_off.p, ctx->Gside.p, ctx->GGside.p, s));
    launches += 4;
    if (info) {
      // step counts from the exit records
      std::vector<int> sl(total), ss(total), sd(total);
      CK(copy_async(sl.data(), ctx->rsl.p, total * sizeof(int), cudaMemcpyDeviceToHost, s));
      CK(copy_async(sd.data(), ctx->rside.p, total * sizeof(int), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      int64_t steps = 0, ng = 0, nsn = 0;
      for (int64_t q = 0; q < total; q++) {
        steps += sl[q];
        if (sd[q] == -1) ng++;
        else if (sd[q] >= 0) nsn++;
      }
      info->path_steps = steps;
      info->exits_global = ng;
      info->exits_stencil = nsn;
    }
  } else {
    int chunks = 1, ppc = 1;
    item_split(ctx, N, &chunks, &ppc, (mode == PDDS_MODE_MIXED && tuned_for(ctx, desc)) ? ctx->tune_ppc : 0,
               cta_threads_for(ctx, desc), rn);
    const int n_items = rn * chunks;
    CK(cudaMemsetAsync(ctx->counter.p, 0, sizeof(int), s));
    if (mode == PDDS_MODE_MIXED) {
      pdds_status st = enqueue_mixed_paths(ctx, desc, P, chunks, ppc, &launches, nullptr, r0, rn);
      if (st != PDDS_OK) return st;
      if (desc->adaptive_n) {
        st = adaptive_continue(ctx, desc, P, &launches);
        if (st != PDDS_OK) return st;
      }
    } else {
      Fp64Args a{};
      a.L = ctx->dl;
      a.P = P;
      a.N = N;
      a.h = desc->h;
      a.sqrth = std::sqrt(desc->h);
      a.inv_N = 1.0 / N;
      a.seed = desc->seed;
      a.instance = desc->instance;
      a.chunks = chunks;
      a.paths_per_chunk = ppc;
      a.n_items = n_items;
      a.dup_sum = ctx->L.geom == 1 ? 1 : desc->dup_sum;  // circle layouts sum shared side knots
      a.adaptive_h = desc->adaptive_h ? 1 : 0;
      a.richardson = desc->richardson ? 1 : 0;
      a.max_steps = max_steps;
      a.mc_knots = ctx->mc_knots.p + r0;
      a.item_counter = ctx->counter.p;
      a.G = ctx->G.p;
      a.Bsum = ctx->Bsum.p;
      a.BBsum = ctx->BBsum.p;
      a.stats = ctx->stats.p;
      a.err_flags = ctx->errf.p;
      a.diag = diag ? ctx->diag.p : nullptr;
      const size_t smem = ctx->fp64_smem;
      cudaFuncAttributes fa;
      (void)fa;
      int bps = fp64_blocks_per_sm(P.kind, smem, a.richardson);
      if (bps < 1) bps = 1;
      const int grid = std::max(1, std::min(n_items, bps * ctx->num_sms));
      if (n_items > 0) {
        CK(launch_paths_fp64(a, P.kind, grid, smem, s));
        launches++;
      }
    }
    if (mode == PDDS_MODE_MIXED && desc->adaptive_n)
      CK(launch_finalize_n(ctx->mc_knots.p, n_mc, ctx->knot_N.p, ctx->Bsum.p, ctx->BBsum.p, ctx->B.p, ctx->BB.p,
                           nnz, ctx->G.p, ctx->GG.p, desc->want_var ? 1 : 0, s));
    else
      CK(launch_finalize(ctx->mc_knots.p, n_mc, N, ctx->Bsum.p, ctx->BBsum.p, ctx->B.p, ctx->BB.p,
                         ctx->row_ptr.p, nnz, ctx->G.p, ctx->GG.p,
                         (mode == PDDS_MODE_MIXED && desc->want_var) ? 1 : 0, s));
    launches += 1 + ((mode == PDDS_MODE_MIXED && desc->want_var) ? 1 : 0);
  }
  CK(cudaEventRecord(ctx->ev2, s));
  if (!(mode == PDDS_MODE_MIXED && desc->adaptive_n)) {
    ctx->last_knot_N.assign(L.K, 0);
    for (int m = r0; m < r0 + rn; m++) ctx->last_knot_N[ctx->mc_host[m]] = N;
  }
  prefault(val, nnz * sizeof(double));
  if (mode != PDDS_MODE_FP64) prefault(var, nnz * sizeof(double));
  if (val && nnz) CK(copy_async(val, ctx->G.p, nnz * sizeof(double), cudaMemcpyDeviceToHost, s));
  if (var && nnz) {
    if (mode == PDDS_MODE_FP64) std::fill(var, var + nnz, 0.0);
    else CK(copy_async(var, ctx->GG.p, nnz * sizeof(double), cudaMemcpyDeviceToHost, s));
  }
  if (Bout) CK(copy_async(Bout, ctx->B.p, L.K * sizeof(double), cudaMemcpyDeviceToHost, s));
  if (BBout) CK(copy_async(BBout, ctx->BB.p, L.K * sizeof(double), cudaMemcpyDeviceToHost, s));
  unsigned long long st[8] = {0};
  CK(copy_async(st, ctx->stats.p, sizeof(st), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  ctx->has_estimate = true;
  ctx->has_diag = diag;
  if (info) {
    float ms_setup = 0.f, ms_paths = 0.f;
    cudaEventElapsedTime(&ms_setup, ctx->ev0, ctx->ev1);
    cudaEventElapsedTime(&ms_paths, ctx->ev1, ctx->ev2);
    info->ms_setup = ms_setup;
    info->ms_paths = ms_paths;
    info->kernel_launches = launches;
    if (mode == PDDS_MODE_MIXED && desc->adaptive_n) {
      int64_t tot = 0;
      for (int v : ctx->last_knot_N) tot += v;
      info->paths = tot;
    } else {
      info->paths = (int64_t)n_mc * N;
    }
    if (mode != PDDS_MODE_REPLAY_FP64) {
      info->path_steps = (int64_t)st[0];
      info->exits_global = (int64_t)st[2];
      info->exits_stencil = (int64_t)st[3];
    }
    info->cta_threads = mode == PDDS_MODE_MIXED ? cta_threads_for(ctx, desc) : 0;
  }
  const pdds_status fst = check_err_flags(ctx);
  if (info) {
    info->h2d_bytes = xfer().h2d - x0.h2d;
    info->d2h_bytes = xfer().d2h - x0.d2h;
  }
  return fst;
}

pdds_status pdds_autotune(pdds_ctx* ctx, const pdds_estimate_desc* desc, int32_t sample_knots,
                          pdds_tune_info* info) {
  if (!ctx || !desc) return PDDS_ERR_INVALID;
  if (ctx->device < 0) return fail(ctx, PDDS_ERR_INVALID, "context has no device");
  if (!ctx->has_problem || !ctx->has_layout) return fail(ctx, PDDS_ERR_INVALID, "problem and layout needed");
  if (desc->mode != PDDS_MODE_MIXED) return fail(ctx, PDDS_ERR_INVALID, "the autotuner tunes PDDS_MODE_MIXED");
  if (desc->knot_first || desc->knot_count || desc->diagnostics)
    return fail(ctx, PDDS_ERR_INVALID, "the autotuner times whole runs (no knot range, no diagnostics)");
  if (desc->npaths < 1 || !(desc->h > 0.0)) return fail(ctx, PDDS_ERR_INVALID, "npaths >= 1 and h > 0 required");
  if (desc->cta_threads != 0 && desc->cta_threads != 128 && desc->cta_threads != 256)
    return fail(ctx, PDDS_ERR_INVALID, "cta_threads must be 0, 128 or 256");
  CK(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  const HostLayout& L = ctx->L;
  const ProblemDev P = problem_dev(ctx);
  const int N = desc->npaths;
  // sample: knots spread evenly through the hand-out order
  std::vector<int> mc;
  for (int v : L.order)
    if (!L.knot_boundary[v]) mc.push_back(v);
  if (mc.empty()) return fail(ctx, PDDS_ERR_INVALID, "layout has no knots with paths");
  // the whole layout by default; a sample runs on a proportionally smaller
  // grid so every CTA sees as many work items as in the full run
  const int ns = std::max(1, std::min<int>(sample_knots > 0 ? sample_knots : (int)mc.size(), (int)mc.size()));
  const double frac = (double)ns / (double)mc.size();
  std::vector<int> sample(ns);
  for (int i = 0; i < ns; i++) sample[i] = mc[(size_t)i * mc.size() / ns];
  pdds_estimate_desc d = *desc;
  d.adaptive_n = 0;
  int launches = 0;
  pdds_status st = enqueue_prefix(ctx, &d, P, false, &launches);
  if (st != PDDS_OK) return st;
  // a block size imposed by the caller is kept: only the other shape
  // parameters are searched; 0 searches both block sizes
  const int fixed_threads = desc->cta_threads;
  d.cta_threads = fixed_threads > 0 ? fixed_threads : mixed_threads(ctx->n_mc);  // the default shape first
  auto occupancy = [&](int threads) {
    const size_t smem = ctx->mixed_smem * (d.want_var ? 2 : 1) + mixed_queue_smem(threads, d.richardson);
    return std::max(1, mixed_blocks_per_sm(mixed_kind(P), smem, d.richardson, threads));
  };
  const int occ = occupancy(d.cta_threads);
  std::vector<int> ppc_c;
  for (int p = 256; p < N; p *= 4) ppc_c.push_back(p);
  ppc_c.push_back(N);
  int def_chunks = 1, def_ppc = 1;
  item_split(ctx, N, &def_chunks, &def_ppc);
  ppc_c.push_back(def_ppc);
  std::sort(ppc_c.begin(), ppc_c.end());
  ppc_c.erase(std::unique(ppc_c.begin(), ppc_c.end()), ppc_c.end());
  auto time_shape = [&](int bps, int ppc, float* ms_out) -> pdds_status {
    std::vector<int> ik, ip0, ip1;
    for (int k : sample)
      for (int p = 0; p < N; p += ppc) {
        ik.push_back(k);
        ip0.push_back(p);
        ip1.push_back(std::min(N, p + ppc));
      }
    CK(ctx->item_knot.upload(ik, s));
    CK(ctx->item_p0.upload(ip0, s));
    CK(ctx->item_p1.upload(ip1, s));
    ItemList items{ctx->item_knot.p, ctx->item_p0.p, ctx->item_p1.p, (int)ik.size(), nullptr};
    float best = 1e30f;
    for (int rep = 0; rep < 2; rep++) {
      ctx->force_bps = bps;
      ctx->force_grid_frac = frac;
      CK(cudaEventRecord(ctx->ev0, s));
      int nl = 0;
      pdds_status e = enqueue_mixed_paths(ctx, &d, P, 1, ppc, &nl, &items);
      ctx->force_bps = 0;
      ctx->force_grid_frac = 0.0;
      if (e != PDDS_OK) return e;
      CK(cudaEventRecord(ctx->ev1, s));
      CK(cudaEventSynchronize(ctx->ev1));
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
      best = std::min(best, ms);
    }
    *ms_out = best;
    return PDDS_OK;
  };
  float best_ms = 1e30f, def_ms = 0.f;
  int best_bps = occ, best_ppc = def_ppc, best_threads = d.cta_threads, ncand = 0;
  st = time_shape(occ, def_ppc, &def_ms);
  if (st != PDDS_OK) return st;
  for (int th : {128, 256}) {
    if (fixed_threads > 0 && th != fixed_threads) continue;
    d.cta_threads = th;
    const int occ_t = occupancy(th);
    for (int b = 1; b <= occ_t; b++)
      for (int p : ppc_c) {
        float ms = 0.f;
        st = time_shape(b, p, &ms);
        if (st != PDDS_OK) return st;
        ++ncand;
        if (ms < best_ms) {
          best_ms = ms;
          best_bps = b;
          best_ppc = p;
          best_threads = th;
        }
      }
  }
  // the last adaptive estimate's continuation (knot paths N0 .. N_k), whole:
  // both block sizes at the default item size, then item sizes at the
  // faster block size; its items carry the long paths whose tail a uniform
  // sample does not show
  int cont_threads = 0, cont_ppc = 0;
  float cont_ms[2] = {0.f, 0.f};
  if (desc->adaptive_n && fixed_threads == 0 && !ctx->cont_knots.empty() && ctx->cont_kind == ctx->prob.kind &&
      (int)ctx->last_knot_N.size() == L.K) {
    std::vector<int> ik, ip0, ip1;
    auto time_cont = [&](int threads, int ppc, float* ms_out) -> pdds_status {
      continuation_items(ctx->cont_knots, ctx->last_knot_N, ctx->cont_N0, ppc, ik, ip0, ip1);
      if (ik.empty()) {
        *ms_out = 0.f;
        return PDDS_OK;
      }
      CK(ctx->item_knot.upload(ik, s));
      CK(ctx->item_p0.upload(ip0, s));
      CK(ctx->item_p1.upload(ip1, s));
      ItemList items{ctx->item_knot.p, ctx->item_p0.p, ctx->item_p1.p, (int)ik.size(), ctx->knot_invN.p};
      pdds_estimate_desc dc = d;
      dc.cta_threads = threads;
      CK(cudaEventRecord(ctx->ev0, s));
      int nl = 0;
      pdds_status e = enqueue_mixed_paths(ctx, &dc, P, 1, ppc, &nl, &items);
      if (e != PDDS_OK) return e;
      CK(cudaEventRecord(ctx->ev1, s));
      CK(cudaEventSynchronize(ctx->ev1));
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
      *ms_out = ms;
      return PDDS_OK;
    };
    float best_c = 1e30f;
    for (int ti = 0; ti < 2; ti++) {
      const int th = ti == 0 ? 128 : 256;
      st = time_cont(th, CONT_PPC_DEFAULT, &cont_ms[ti]);
      if (st != PDDS_OK) return st;
      ++ncand;
      if (cont_ms[ti] < best_c) {
        best_c = cont_ms[ti];
        cont_threads = th;
        cont_ppc = CONT_PPC_DEFAULT;
      }
    }
    for (int ppc : {2048, 8192, 16384}) {
      float ms = 0.f;
      st = time_cont(cont_threads, ppc, &ms);
      if (st != PDDS_OK) return st;
      ++ncand;
      if (ms < best_c) {
        best_c = ms;
        cont_ppc = ppc;
      }
    }
  }
  st = check_err_flags(ctx);
  if (st != PDDS_OK) return st;
  ctx->tune_bps = best_bps;
  ctx->tune_ppc = best_ppc;
  ctx->tune_threads = best_threads;
  ctx->tune_cont_threads = cont_threads;
  ctx->tune_cont_ppc = cont_ppc;
  ctx->tune_kind = ctx->prob.kind;
  ctx->tune_rich = d.richardson ? 1 : 0;
  ctx->has_estimate = false;
  drop_graph(ctx);  // a captured batch sequence holds the old launch shape
  if (info) {
    info->blocks_per_sm = best_bps;
    info->paths_per_item = best_ppc;
    info->cta_threads = best_threads;
    info->continuation_threads = cont_threads;
    info->continuation_paths_per_item = cont_ppc;
    info->continuation_ms[0] = cont_ms[0];
    info->continuation_ms[1] = cont_ms[1];
    info->candidates = ncand;
    info->sample_knots = ns;
    info->best_ms = best_ms;
    info->default_ms = def_ms;
  }
  return PDDS_OK;
}

pdds_status pdds_subdomain_solve(pdds_ctx* ctx, int32_t m, const double* u, double* out) {
  if (!ctx || !out) return PDDS_ERR_INVALID;
  if (ctx->device < 0) return fail(ctx, PDDS_ERR_INVALID, "context has no device");
  if (!ctx->has_layout || ctx->L.geom != 0 || ctx->is_batch || ctx->L.custom)
    return fail(ctx, PDDS_ERR_INVALID, "subdomain solves need a rectangular layout");
  if (!ctx->has_problem) return fail(ctx, PDDS_ERR_INVALID, "no problem set");
  const int kind = ctx->prob.kind;
  if (kind != PDDS_POISSON_SINCOS && kind != PDDS_MONEGROS && kind != PDDS_HELMHOLTZ && kind != PDDS_LUT)
    return fail(ctx, PDDS_ERR_INVALID,
                "subdomain solves take operators Lap + c (Poisson, Monegros, Helmholtz) or table-served problems");
  if (m < 2 || m > 64) return fail(ctx, PDDS_ERR_INVALID, "2 <= m <= 64");
  if (!u && !ctx->has_solution) return fail(ctx, PDDS_ERR_INVALID, "no interface solution");
  CK(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  const HostLayout& L = ctx->L;
  const int ns = L.nsub, n = L.nnode, S = ns * ns;
  if (!ctx->edges_ready) {
    // knots of every subdomain edge, ordered along it, from the knot positions
    const double lx = (L.ne[0] - L.sw[0]) / ns, ly = (L.ne[1] - L.sw[1]) / ns;
    const double tol = 1e-9 * std::max(lx, ly);
    std::vector<int> ek((size_t)S * 4 * n, -1);
    for (int b = 0; b < ns; b++)
      for (int a = 0; a < ns; a++) {
        const int sub = a + ns * b;
        const double x0 = L.sw[0] + a * lx, y0 = L.sw[1] + b * ly;
        for (int d = 0; d < 4; d++) {
          const bool on_bnd = (d == 0 && b == 0) || (d == 1 && b == ns - 1) || (d == 2 && a == 0) || (d == 3 && a == ns - 1);
          if (on_bnd) continue;
          std::vector<std::pair<double, int>> hit;
          for (int v = 0; v < L.K; v++) {
            const double x = L.kx[v], y = L.ky[v];
            if (d <= 1) {
              const double yl = d == 0 ? y0 : y0 + ly;
              if (std::fabs(y - yl) < tol && x > x0 - tol && x < x0 + lx + tol) hit.push_back({x, v});
            } else {
              const double xl = d == 2 ? x0 : x0 + lx;
              if (std::fabs(x - xl) < tol && y > y0 - tol && y < y0 + ly + tol) hit.push_back({y, v});
            }
          }
          if ((int)hit.size() != n) return fail(ctx, PDDS_ERR_INVALID, "internal: subdomain edge knot count");
          std::sort(hit.begin(), hit.end());
          for (int q = 0; q < n; q++) ek[((size_t)sub * 4 + d) * n + q] = hit[q].second;
        }
      }
    CK(ctx->edge_knots.upload(ek, s));
    ctx->edges_ready = true;
  }
  const double* ud = ctx->su.p;
  if (u) {
    CK(ctx->sub_u.resize(std::max(L.K, 1)));
    CK(copy_async(ctx->sub_u.p, u, L.K * sizeof(double), cudaMemcpyHostToDevice, s));
    ud = ctx->sub_u.p;
  }
  CK(ctx->sub_out.resize((size_t)S * m * m));
  const int G = ns * (m + 1) + 1;
  CK(ctx->ugrid.resize((size_t)G * G));
  if (kind == PDDS_LUT) {
    CK(ctx->sub_work.resize((size_t)S * 13 * m * m));
    CK(ctx->sub_iters.resize(S));
    CK(cudaMemsetAsync(ctx->errf.p, 0, sizeof(unsigned), s));
    CK(launch_subdomain_lut(ctx->dl, problem_dev(ctx), ns, m, n, ctx->edge_knots.p, ud, ctx->sub_out.p,
                            ctx->sub_work.p, ctx->ugrid.p, 200, 1e-12, ctx->sub_iters.p, ctx->errf.p, s));
  } else {
    CK(launch_subdomain(ctx->dl, problem_dev(ctx), ns, m, n, ctx->edge_knots.p, ud, ctx->sub_out.p, ctx->ugrid.p, s));
  }
  CK(copy_async(out, ctx->sub_out.p, (size_t)S * m * m * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  ctx->ugrid_m = m;
  if (kind == PDDS_LUT) return check_err_flags(ctx);
  return PDDS_OK;
}

pdds_status pdds_semilinear_tables(pdds_ctx* ctx, const pdds_semilinear_desc* desc) {
  if (!ctx || !desc) return PDDS_ERR_INVALID;
  if (ctx->device < 0) return fail(ctx, PDDS_ERR_INVALID, "context has no device");
  if (!ctx->has_layout || ctx->L.geom != 0 || ctx->is_batch || ctx->L.custom)
    return fail(ctx, PDDS_ERR_INVALID, "the semilinear step needs a rectangular layout");
  const HostLayout& L = ctx->L;
  if (desc->equation != PDDS_OUTER_NEWTON_U3 && desc->equation != PDDS_OUTER_LINEAR_SHIFT)
    return fail(ctx, PDDS_ERR_INVALID, "unknown outer-loop equation");
  if (desc->equation == PDDS_OUTER_NEWTON_U3 &&
      (std::fabs(L.sw[0]) > 1e-12 || std::fabs(L.sw[1]) > 1e-12 || std::fabs(L.ne[0] - 1.0) > 1e-12 ||
       std::fabs(L.ne[1] - 1.0) > 1e-12))
    return fail(ctx, PDDS_ERR_INVALID, "the semilinear test equation lives on the unit square [0,1]^2");
  if (desc->equation == PDDS_OUTER_LINEAR_SHIFT &&
      !(desc->k > 0.0 && std::isfinite(desc->k) && std::isfinite(desc->c2) && std::isfinite(desc->alpha) &&
        std::isfinite(desc->u0)))
    return fail(ctx, PDDS_ERR_INVALID, "the linear iteration needs k > 0 and finite c2, alpha, u0");
  const int m = desc->m;
  if (m < 2 || m > 64) return fail(ctx, PDDS_ERR_INVALID, "2 <= m <= 64");
  if (desc->from_solution && ctx->ugrid_m != m)
    return fail(ctx, PDDS_ERR_INVALID, "from_solution needs a pdds_subdomain_solve with the same m on this layout");
  CK(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  drop_graph(ctx);
  const int ns = L.nsub;
  const int G = ns * (m + 1) + 1;
  const size_t nn = (size_t)G * G;
  release_lut_tex(ctx);  // tables computed on the device: the FP32 sampler reads the nodes
  CK(ctx->lut_coef.resize(8 * nn));
  CK(ctx->lut_g.resize(nn));
  const double hx = (L.ne[0] - L.sw[0]) / ns / (m + 1), hy = (L.ne[1] - L.sw[1]) / ns / (m + 1);
  OuterStep eq;
  eq.equation = desc->equation == PDDS_OUTER_LINEAR_SHIFT ? OUTER_LINEAR_SHIFT : OUTER_NEWTON_U3;
  eq.u0 = desc->u0;
  eq.a = desc->a;
  eq.c2 = desc->c2;
  eq.alpha = desc->alpha;
  eq.k = desc->k;
  CK(launch_newton_tables(desc->from_solution ? ctx->ugrid.p : nullptr, G, L.sw[0], L.sw[1], hx, hy, eq,
                          ctx->lut_coef.p, ctx->lut_g.p, s));
  CK(cudaStreamSynchronize(s));
  ctx->lut_nx = G;
  ctx->lut_ny = G;
  ctx->lut_bounds[0] = L.sw[0];
  ctx->lut_bounds[1] = L.sw[1];
  ctx->lut_bounds[2] = L.ne[0];
  ctx->lut_bounds[3] = L.ne[1];
  pdds_problem_desc pd;
  std::memset(&pd, 0, sizeof(pd));
  pd.kind = PDDS_LUT;
  pd.use_cv = desc->use_cv ? 1 : 0;
  ctx->prob = pd;
  ctx->has_problem = true;
  return PDDS_OK;
}

pdds_status pdds_estimate_knot_steps(pdds_ctx* ctx, int64_t* steps) {
  if (!ctx || !steps) return PDDS_ERR_INVALID;
  if (!ctx->has_estimate || !ctx->has_knot_steps) return fail(ctx, PDDS_ERR_INVALID, "no MIXED estimate on this layout");
  CK(cudaSetDevice(ctx->device));
  CK(copy_async(steps, ctx->knot_steps.p, ctx->L.K * sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return PDDS_OK;
}

pdds_status pdds_estimate_diagnostics(pdds_ctx* ctx, double* sums) {
  if (!ctx || !sums) return PDDS_ERR_INVALID;
  if (!ctx->has_estimate || !ctx->has_diag)
    return fail(ctx, PDDS_ERR_INVALID, "no estimate with diagnostics on this layout");
  CK(cudaSetDevice(ctx->device));
  CK(copy_async(sums, ctx->diag.p, (size_t)ctx->L.K * PDDS_DIAG_N * sizeof(double), cudaMemcpyDeviceToHost,
                ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return PDDS_OK;
}

pdds_status pdds_estimate_step_histogram(pdds_ctx* ctx, int64_t* hist) {
  if (!ctx || !hist) return PDDS_ERR_INVALID;
  if (!ctx->has_estimate || !ctx->has_knot_steps) return fail(ctx, PDDS_ERR_INVALID, "no MIXED estimate on this layout");
  CK(cudaSetDevice(ctx->device));
  CK(copy_async(hist, ctx->step_hist.p, 32 * sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return PDDS_OK;
}

pdds_status pdds_estimate_knot_paths(pdds_ctx* ctx, int32_t* npaths) {
  if (!ctx || !npaths) return PDDS_ERR_INVALID;
  if (!ctx->has_estimate || ctx->last_knot_N.size() != (size_t)ctx->L.K)
    return fail(ctx, PDDS_ERR_INVALID, "no estimate on this layout");
  std::copy(ctx->last_knot_N.begin(), ctx->last_knot_N.end(), npaths);
  return PDDS_OK;
}

pdds_status pdds_solve_interface(pdds_ctx* ctx, const pdds_solve_desc* desc, double* u,
                                 pdds_solve_info* info) {
  if (!ctx || !desc) return PDDS_ERR_INVALID;
  if (!ctx->has_estimate) return fail(ctx, PDDS_ERR_INVALID, "no estimate to solve");
  if (ctx->L.custom && ctx->L.max_col >= ctx->L.K)
    return fail(ctx, PDDS_ERR_INVALID, "G has columns outside the layout's knots (column " +
                                           std::to_string(ctx->L.max_col) + "): the system is not square");
  CK(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  const HostLayout& L = ctx->L;
  const int K = L.K;
  const int64_t nnz = L.row_ptr[K];
  const XferCount x0 = xfer();
  // GMRES(20): on the 12x12 / 43-knot layout every restart length from 20 to 40 needs the same
  // 120 Arnoldi steps, and the shorter basis makes each step cheaper
  const int m = std::max(2, std::min(desc->restart > 0 ? desc->restart : 20, 40));
  CK(ctx->sv64.resize((size_t)6 * K));
  CK(ctx->sscal.resize(64));
  CK(ctx->spart.resize(std::max<size_t>(64 * 256 + 1024, (size_t)((K + 127) / 128) * 48 + 64)));
  CK(ctx->shess.resize((size_t)(m + 1) * m + 2 * m + 4 * (m + 1) + 16));
  CK(ctx->sctl.resize(8));
  CK(ctx->sgpart.resize((size_t)2 * std::max(ctx->num_sms, 1) * (GMRES_CLUSTER_MAX_M + 3)));
  CK(ctx->sbar.resize(2));
  CK(ctx->su.resize(std::max(K, 1)));
  SolveCsr A{K, nnz, ctx->row_ptr.p, ctx->col.p, ctx->G.p};
  if (desc->barrier_poll_limit < 0) return fail(ctx, PDDS_ERR_INVALID, "barrier_poll_limit must be >= 0");
  SolveWork w{};
  w.err = ctx->errf.p;
  w.spin_limit = (unsigned)desc->barrier_poll_limit;
  if (desc->grid_ctas < 0) return fail(ctx, PDDS_ERR_INVALID, "grid_ctas must be >= 0");
  w.grid_ctas = desc->grid_ctas;
  CK(cudaMemsetAsync(ctx->errf.p, 0, sizeof(unsigned), s));
  for (int q = 0; q < 6; q++) w.v64[q] = ctx->sv64.p + (size_t)q * K;
  w.scal = ctx->sscal.p;
  w.part = ctx->spart.p;
  w.hess = ctx->shess.p;
  w.host_rr = ctx->host_rr;
  w.ctl = ctx->sctl.p;
  w.gpart = ctx->sgpart.p;
  w.bar = ctx->sbar.p;
  int iters = 0, refines = 0;
  double relres = 0.0;
  const double tol = desc->tol > 0 ? desc->tol : 1e-10;
  CK(cudaEventRecord(ctx->ev0, s));
  if (desc->method == PDDS_SOLVE_BICGSTAB_FP64) {
    const int maxit = desc->max_iter > 0 ? desc->max_iter : 2 * K;
    CK(solve_bicgstab(A, ctx->B.p, ctx->su.p, w, maxit, tol, &iters, &relres, s));
  } else if (desc->method == PDDS_SOLVE_GMRES_FP32_IR) {
    CK(ctx->sV32.resize((size_t)(m + 1) * K));
    CK(ctx->sw32.resize(std::max(K, 1)));
    CK(ctx->sval32.resize(std::max<int64_t>(nnz, 1)));
    if (desc->gmres_form == PDDS_GMRES_PIPELINED) CK(ctx->sZ32.resize((size_t)(m + 1) * K));
    w.Z32 = desc->gmres_form == PDDS_GMRES_PIPELINED ? ctx->sZ32.p : nullptr;
    w.V32 = ctx->sV32.p;
    w.w32 = ctx->sw32.p;
    w.val32 = ctx->sval32.p;
    const int maxit = desc->max_iter > 0 ? desc->max_iter : 1000;
    const int maxref = desc->max_refine > 0 ? desc->max_refine : 30;
    bool used = false;
    CK(solve_gmres_ir_cluster(A, ctx->B.p, ctx->su.p, w, m, maxit, maxref, tol, &iters, &refines, &relres, s,
                              &used));
    if (!used)
      CK(solve_gmres_ir(A, ctx->B.p, ctx->su.p, w, m, maxit, maxref, tol, &iters, &refines, &relres, s));
  } else {
    return fail(ctx, PDDS_ERR_INVALID, "unknown solve method");
  }
  CK(cudaEventRecord(ctx->ev1, s));
  if (u) CK(copy_async(u, ctx->su.p, K * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  ctx->has_solution = true;
  if (info) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    info->iterations = iters;
    info->refinements = refines;
    info->rel_residual = relres;
    info->ms = ms;
    info->kernel_launches = w.launches;
  }
  {
    pdds_status st = check_err_flags(ctx);
    if (info) {
      info->h2d_bytes = xfer().h2d - x0.h2d;
      info->d2h_bytes = xfer().d2h - x0.d2h;
    }
    if (st != PDDS_OK) return st;
  }
  if (!(relres <= tol * 1.0000001) && !(relres == 0.0))
    return fail(ctx, PDDS_ERR_NOT_CONVERGED, "interface solve reached " + std::to_string(relres));
  return PDDS_OK;
}

}  // extern "C"
