// Context of the C ABI (internal to the library): device buffers of the
// layout, the problem, results and scratch, shared by capi.cu and batch.cu.
#pragma once
#include <cuda_runtime.h>

#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "../../include/pdds.h"
#include "kernels.h"
#include "pdds_internal.h"
#include "xfer.h"

namespace pdds {

// Device blocks of destroyed contexts, kept per device for the next context
// (a context allocates some 60 buffers; each cudaMalloc and cudaFree costs
// about 10 us).  Only pdds_destroy hands blocks back, after synchronizing
// its stream, so a cached block has no work in flight.  block_alloc rounds
// the size up to the block classes and takes a cached block of that class,
// else calls cudaMalloc (after emptying the cache if that fails).
size_t block_class(size_t bytes);
cudaError_t block_alloc(void** p, size_t bytes);
void block_recycle(void* p, size_t bytes);  // into the cache (or cudaFree)
void block_cache_clear(int device);         // -1: every device

// A device array: owned (cudaMalloc) or a view into another buffer's block
// (set_view; not freed here, and replaced by an owned block if it must grow).
template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  bool view = false;
  cudaError_t resize(size_t count) {
    if (count <= n && p) return cudaSuccess;
    release();
    if (count == 0) return cudaSuccess;
    const size_t bytes = block_class(count * sizeof(T));
    cudaError_t e = block_alloc(reinterpret_cast<void**>(&p), bytes);
    if (e == cudaSuccess) n = bytes / sizeof(T);
    else p = nullptr;
    return e;
  }
  cudaError_t upload(const std::vector<T>& v, cudaStream_t s) {
    cudaError_t e = resize(std::max<size_t>(v.size(), 1));
    if (e != cudaSuccess || v.empty()) return e;
    return copy_async(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s);
  }
  void set_view(void* base, size_t count) {
    release();
    p = static_cast<T*>(base);
    n = count;
    view = true;
  }
  void release() {
    if (p && !view) cudaFree(p);
    p = nullptr;
    n = 0;
    view = false;
  }
  // release into the block cache (pdds_destroy, after its stream is idle)
  void recycle() {
    if (p && !view) block_recycle(p, block_class(n * sizeof(T)));
    p = nullptr;
    n = 0;
    view = false;
  }
};

// Host arrays packed into one block (each at a 256-byte offset) that is
// copied to the device at once: add() records the parts, pack() sizes the
// host block once and copies them in, bind() points each DBuf at its part.
// The sources must stay alive until pack().
struct PackedUpload {
  struct Part {
    const void* src;
    size_t bytes, off;
  };
  std::vector<Part> parts;
  std::vector<unsigned char> host;
  std::vector<std::function<void(unsigned char*)>> binds;
  size_t size = 0;
  template <typename T>
  void add(DBuf<T>& b, const T* src, size_t count) {
    const size_t off = (size + 255) & ~size_t(255);
    const size_t cnt = std::max<size_t>(count, 1);
    size = off + cnt * sizeof(T);
    parts.push_back({src, count * sizeof(T), off});
    binds.push_back([&b, off, cnt](unsigned char* base) { b.set_view(base + off, cnt); });
  }
  template <typename T>
  void add(DBuf<T>& b, const std::vector<T>& v) {
    add(b, v.data(), v.size());
  }
  void pack() {
    host.assign(size, 0);
    for (const Part& q : parts)
      if (q.bytes) std::memcpy(host.data() + q.off, q.src, q.bytes);
  }
  void bind(unsigned char* base) {
    for (auto& f : binds) f(base);
  }
};

}  // namespace pdds

using pdds::DBuf;
using pdds::DevLayout;
using pdds::HostLayout;

struct pdds_ctx {
  int device = -1;
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  std::string err;
  bool has_problem = false;
  pdds_problem_desc prob{};
  DBuf<float> lut_coef, lut_g;
  // textures of the 8 table fields for the FP32 sampler, two float4 each
  // (linear filtering), built by pdds_problem_set_lut: [0..1] cubic B-spline
  // coefficients, [2..3] the node values (bilinear)
  cudaArray_t lut_arr[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaTextureObject_t lut_tex[4] = {0, 0, 0, 0};
  int lut_nx = 0, lut_ny = 0;
  double lut_bounds[4] = {0, 0, 0, 0};
  bool has_layout = false;
  HostLayout L;
  int bins = 16;
  bool tables_ready = false;
  // device layout
  DBuf<double> kx, ky, st_rect, sd_c, sd_origin, side_px, side_py, sh_c, sh_R, sh_lo, sh_delta, sh_t, ipsi;
  DBuf<int> knot_stencil, st_side, st_glob, map_pos, sd_n, sd_orient, sd_shape, side_knot, sh_n,
      sh_nbins, col, mc_knots, bnd_knots;
  DBuf<double> rbf_lu, rbf_uinv;  // factorisation scratch (ipsi and sh_t layouts)
  DBuf<int64_t> st_col_off;       // stencils' column lists, expanded into col on the device
  DBuf<int> st_cols;
  DBuf<int> rbf_piv;
  DBuf<int64_t> row_ptr, st_map_off, sd_knot_off, sh_tab_off, sh_ipsi_off, sh_t_off;
  DBuf<unsigned char> map_owner;
  DBuf<unsigned char> lay_block;  // one device block holding the layout arrays above (views)
  DBuf<int> knot_rng;             // Philox knot word per knot (caller-built stencils)
  DBuf<float> tab;
  DevLayout dl{};
  int n_mc = 0, n_bnd = 0;
  std::vector<int> mc_host;  // knots with paths, in hand-out order (the device mc_knots)
  size_t mixed_smem = 0, fp64_smem = 0;
  int max_nbins = 0;
  // results and scratch
  DBuf<double> G, GG, B, BB, Bsum, BBsum;
  DBuf<unsigned long long> stats;
  DBuf<unsigned> errf;
  DBuf<int> counter;
  bool has_estimate = false;
  // replay scratch
  DBuf<double> rx, ry, rY, rZ, rxi, Gside, GGside, ipsi_knot;
  DBuf<int> rside, rsl, rss, task_m, task_d, task_i;
  DBuf<int64_t> task_out, knot_task_off, knot_ipsi_off;
  // solve scratch
  DBuf<double> sv64, sscal, spart, shess, su;
  DBuf<float> sV32, sw32, sval32, sZ32;
  DBuf<unsigned> sctl, sbar;
  DBuf<double> sgpart;
  double* host_rr = nullptr;
  int solve_m = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr;
  // batch of independent instances (pdds_batch_build): the layout above is
  // the block-diagonal union of the instances' layouts
  bool is_batch = false;
  int n_inst = 0;
  std::vector<int> inst_k0;         // first knot of each instance, n_inst + 1
  std::vector<int64_t> inst_nnz0;   // first G entry of each instance, n_inst + 1
  std::vector<double> inst_p;       // 8 problem parameters per instance
  std::vector<double> inst_hv;      // step per instance (0: the run's)
  std::vector<int> inst_mc0;        // first entry of each instance in mc_host, n_inst + 1
  DBuf<int> knot_inst, inst_knot0, b_iters, b_refines;
  DBuf<double> inst_pd, inst_hd, b_relres;
  DBuf<unsigned long long> b_tend;  // per instance, then the start stamp
  int max_inst_knots = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  std::vector<unsigned char> graph_key;
  int graph_launches = 0;
  std::vector<cudaGraphNode_t> graph_path_nodes;  // path-kernel nodes, re-keyed per run
  bool has_batch_run = false;
  // batch waves: the solves of a wave run on solve_stream (higher priority)
  // while the next wave's paths run on stream; wave_ev orders them
  cudaStream_t solve_stream = nullptr;
  std::vector<cudaEvent_t> wave_ev;
  // subdomain solves: knots of each subdomain edge (S, N, W, E; -1 = domain boundary)
  DBuf<int> edge_knots;
  DBuf<double> sub_u, sub_out;
  DBuf<double> sub_work;          // Krylov vectors of the table-served subdomain solver
  DBuf<int> sub_iters;            // its iterations per subdomain
  DBuf<double> ugrid;             // last subdomain solution on the global grid
  int ugrid_m = 0;                // its interior points per subdomain side (0 = none)
  bool edges_ready = false;
  bool has_solution = false;
  // autotuned launch shape of the MIXED path kernel (0 = defaults)
  int tune_bps = 0, tune_ppc = 0, tune_kind = -1, tune_rich = -1, tune_threads = 0;
  int tune_cont_threads = 0, tune_cont_ppc = 0;  // adaptive continuation's shape (0: untuned)
  std::vector<int> cont_knots;                   // last adaptive continuation: knots, heaviest first
  int cont_N0 = 0;                               // and its pilot's paths (N_k in last_knot_N)
  int cont_kind = -1;                            // and its problem kind
  int force_bps = 0;             // CTAs per SM imposed while the autotuner times a shape
  double force_grid_frac = 0.0;  // grid scaled to a knot sample while it times
  // variance-adaptive paths (pdds_estimate with adaptive_n)
  DBuf<int> knot_N, item_knot, item_p0, item_p1;
  DBuf<double> knot_scale, knot_invN;
  std::vector<int> last_knot_N;  // paths per knot of the last estimate
  DBuf<unsigned long long> knot_steps;  // path steps per knot of the last MIXED estimate
  DBuf<unsigned long long> step_hist;   // [32] paths by steps (log2 bins) of the last MIXED estimate
  DBuf<double> diag;              // [K][PDDS_DIAG_N] diagnostic sums of the last estimate
  bool has_diag = false;
  DBuf<double> rsx, rsy, rsY, rsZ, rsxi, rknot_h;  // replay diagnostics: sublinear ends, knot steps
  DBuf<int> mc_lpt;               // MIXED hand-out order, heaviest knots first (from knot_steps)
  bool lpt_ready = false;
  bool has_knot_steps = false;
};

namespace pdds {

pdds_status fail(pdds_ctx* c, pdds_status s, const std::string& msg);
// Uploads ctx->L into the device layout buffers and fills ctx->dl.
pdds_status upload_layout(pdds_ctx* ctx);
ProblemDev problem_dev(const pdds_ctx* ctx);
// Reads the device error flags (synchronises the stream).
pdds_status check_err_flags(pdds_ctx* ctx);
// Enqueues the MIXED estimation on ctx->stream: RBF factorisation and tables
// (unless reused), zeroing, boundary knots, the path kernel and the
// finalisation.  No host synchronisation, so it can be graph-captured.
// mc0, mc_n: only the knots mc_knots[mc0 .. mc0 + mc_n) (mc_n < 0: to the
// end); prefix: also the factorisation, zeroing and boundary knots.
pdds_status enqueue_mixed(pdds_ctx* ctx, const pdds_estimate_desc* desc, int* launches, int mc0 = 0,
                          int mc_n = -1, bool prefix = true);
// Destroys the captured batch graph (its kernels hold buffer addresses).
void drop_graph(pdds_ctx* ctx);
// Forgets the autotuned launch shape (it was timed on the previous layout).
void clear_tune(pdds_ctx* ctx);
// Destroys the textures of the tables (the FP32 sampler then reads the nodes).
void release_lut_tex(pdds_ctx* ctx);

}  // namespace pdds

#define CK(call)                                                                         \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail(ctx, PDDS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)
