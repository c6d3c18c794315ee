// Launch arguments and entry points of the device kernels (host-visible).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pdds.h"
#include "dev_common.cuh"

namespace pdds {

constexpr int MIXED_MAX_THREADS = 256;
// Block size of the MIXED path kernel: 128-thread CTAs (8 per SM) for large
// layouts, where they were faster (12x12/n43: 27.7 against 28.2 ms), 256
// (4 per SM) below 8192 Monte Carlo knots, where 128 measured 6-17 % slower.
inline int mixed_threads(int n_mc) { return n_mc >= 8192 ? 128 : 256; }
constexpr int FP64_THREADS = 256;
constexpr int FP64_QCAP = 96;  // exits queued per warp in the FP64 kernel
constexpr unsigned ERR_FLAG_STEP_LIMIT = 1u;
constexpr unsigned ERR_FLAG_EXIT_SIDE = 2u;
constexpr unsigned ERR_FLAG_SINGULAR = 4u;
constexpr unsigned ERR_FLAG_TIMEOUT = 8u;  // a bounded device wait ran out
constexpr unsigned ERR_FLAG_SUB_NOCONV = 16u;  // a subdomain solve missed its tolerance
constexpr unsigned ERR_FLAG_BOUNDS = 32u;      // an index check of the checked build failed

// Index check of the checked build (compiled with -DPDDS_CHECKED,
// pdds_gb300.build.build(checked=True)): i must lie in [0, n); a failed
// check sets ERR_FLAG_BOUNDS and the caller skips the access.  The default
// build compiles every check to true.
__device__ __forceinline__ bool idx_ok(long long i, long long n, unsigned* flags) {
#ifdef PDDS_CHECKED
  if (i >= 0 && i < n) return true;
  if (flags) atomicOr(flags, ERR_FLAG_BOUNDS);
  return false;
#else
  (void)i;
  (void)n;
  (void)flags;
  return true;
#endif
}

// Diagnostic sums of one finished path (or Richardson pair) into a CTA's
// shared sums: phi, phi^2, xi, xi^2, phi + xi, (phi + xi)^2, xi phi, tau, normals.
__device__ __forceinline__ void diag_add(double* sd, double phi, double xi, double tau, double rng) {
  atomicAdd(sd + PDDS_DIAG_SCORE, phi);
  atomicAdd(sd + PDDS_DIAG_SCORE2, phi * phi);
  atomicAdd(sd + PDDS_DIAG_XI, xi);
  atomicAdd(sd + PDDS_DIAG_XI2, xi * xi);
  atomicAdd(sd + PDDS_DIAG_SCORE_VR, phi + xi);
  atomicAdd(sd + PDDS_DIAG_SCORE_VR2, (phi + xi) * (phi + xi));
  atomicAdd(sd + PDDS_DIAG_XI_SCORE, xi * phi);
  atomicAdd(sd + PDDS_DIAG_TAU, tau);
  atomicAdd(sd + PDDS_DIAG_RNG, rng);
  atomicAdd(sd + PDDS_DIAG_PATHS, 1.0);
}
// A CTA's sums into the knot's (the linear sums also fill the sublinear
// slots: the FP64 and MIXED forms run no sublinear leg).
__device__ __forceinline__ void diag_flush(const double* sd, double* out, int tid) {
  if (tid < PDDS_DIAG_SUB) {
    atomicAdd(out + tid, sd[tid]);
    atomicAdd(out + PDDS_DIAG_SUB + tid, sd[tid]);
  } else if (tid == PDDS_DIAG_SUB || tid == PDDS_DIAG_SUB + 1) {
    const int q = tid == PDDS_DIAG_SUB ? PDDS_DIAG_RNG : PDDS_DIAG_PATHS;
    atomicAdd(out + q, sd[q]);
  }
}

struct MixedArgs {
  DevLayout L;
  ProblemDev P;
  int N;                 // paths per knot
  float h, sqrth;
  double inv_N;
  // Philox-4x32-10 round keys of the seed (k0 + r W0, k1 + r W1 for rounds
  // r = 0..9, set by mixed_set_rng): kernel parameters, so every round's key
  // is an operand of its XOR instead of a key-schedule addition per call
  uint32_t rk[20];
  uint32_t instance;
  int chunks, paths_per_chunk, n_items;
  int want_var, dup_sum;
  int adaptive_h;
  int richardson;        // 1: common-random-number Richardson pair (h/2, h)
  double h64;            // h in FP64 (for the adaptive step)
  long long max_steps;
  const int* mc_knots;   // knots that need paths, in hand-out order
  int* item_counter;
  double* G;             // [nnz] accumulates -sum Y H / N
  double* GG;            // [nnz] accumulates sum (Y H)^2 / N
  double* Bsum;          // [K]
  double* BBsum;         // [K]
  unsigned long long* stats;  // [0] steps [1] unused [2] global exits [3] stencil exits
  unsigned* err_flags;
  // optional explicit items (knot, paths [p0, p1)) instead of n_mc x chunks,
  // and per-knot 1/N_k instead of inv_N (variance-adaptive paths)
  const int* item_knot;
  const int* item_p0;
  const int* item_p1;
  const double* knot_invN;
  unsigned long long* knot_steps;  // optional: path steps per knot (both levels)
  // optional [32]: paths (each level of a Richardson pair counts) by their
  // steps, bin b = steps in [2^b, 2^(b+1))
  unsigned long long* step_hist;
  // optional [K][PDDS_DIAG_N]: the reduction's diagnostic sums per knot
  double* diag;
};

struct Fp64Args {
  DevLayout L;
  ProblemDev P;
  int N;
  double h, sqrth, inv_N;
  uint64_t seed;
  uint32_t instance;
  int chunks, paths_per_chunk, n_items;
  int dup_sum;
  int adaptive_h;
  int richardson;
  long long max_steps;
  const int* mc_knots;
  int* item_counter;
  double* G;
  double* Bsum;
  double* BBsum;
  unsigned long long* stats;
  unsigned* err_flags;
  double* diag;          // optional [K][PDDS_DIAG_N]: diagnostic sums per knot
};

struct ReplayArgs {
  DevLayout L;
  ProblemDev P;
  int N;
  double h, sqrth;
  uint64_t seed;
  uint32_t instance;
  int sublinear;
  int adaptive_h;
  long long max_steps;
  const int* mc_knots;   // knots with paths
  int n_mc;
  // per-knot side data for the reduction (actual positions, ipsi per knot)
  const int64_t* knot_ipsi_off;  // [n_mc][4] offset into ipsi_knot, -1 if none
  const double* ipsi_knot;
  // exit records [n_mc * N]
  double* ex;
  double* ey;
  double* eY;
  double* eZ;
  double* exi;
  int* eside;            // -1 global, 0..3 stencil side, -2 no side
  int* esteps_l;
  int* esteps_s;
  // diagnostics (all null when off): sums [K][PDDS_DIAG_N], the sublinear
  // leg's end states [n_mc * N] and each knot's step [n_mc]
  double* diag;
  double* sx;
  double* sy;
  double* sY;
  double* sZ;
  double* sxi;
  double* knot_h;
  // outputs
  double* G;             // [nnz] final values
  double* GG;            // [nnz] final GG/N values (before - G^2)
  double* B;             // [K]
  double* BB;            // [K]
  int dup_sum;
  unsigned* err_flags;
};

// The FP32 path-kernel instantiation of a problem: table-served problems
// with textures run PK_LUT_TEX, every other problem its own kind.
inline int mixed_kind(const ProblemDev& P) { return P.kind == PK_LUT && P.lut.tex_mode ? PK_LUT_TEX : P.kind; }

// smem: mixed_queue_smem(threads, richardson) + the exit histograms
cudaError_t launch_paths_mixed(const MixedArgs& a, int kind, int grid, int threads, size_t smem, cudaStream_t s);
size_t mixed_queue_smem(int threads, int richardson);
// knots mc[n] reordered heaviest first by steps[knot] (quarter-octave groups)
cudaError_t launch_lpt_order(const int* mc, int n, const unsigned long long* steps, int* out, cudaStream_t s);
// Sets the Philox key schedule (rk) of `seed` and the instance word.
void mixed_set_rng(MixedArgs& a, uint64_t seed, uint32_t instance);
// out[4i..4i+3] = the MIXED kernel's Philox block for counter ctr[4i..4i+3]
// and the 64-bit key (low word first), device arrays.
cudaError_t launch_philox_rk_check(uint64_t key, const uint32_t* ctr, int n, uint32_t* out, cudaStream_t s);
// The portable Philox (form 0) and FP64 functions (selfcheck.cu).
cudaError_t launch_philox_check(const uint32_t* ctr, const uint32_t* key, int n, uint32_t* out, cudaStream_t s);
cudaError_t launch_portable_math_check(int fn, const double* x, int n, double* out, cudaStream_t s);
void philox_check_host(const uint32_t* ctr, const uint32_t* key, int n, uint32_t* out);
void portable_math_check_host(int fn, const double* x, int n, double* out);
// True when `func` is one of the MIXED path kernels (a captured graph's
// nodes are re-keyed with a new seed through their parameters).
bool is_mixed_path_kernel(const void* func);
int mixed_blocks_per_sm(int kind, size_t smem, int richardson, int threads, bool diag = false);
cudaError_t launch_paths_fp64(const Fp64Args& a, int kind, int grid, size_t smem, cudaStream_t s);
int fp64_blocks_per_sm(int kind, size_t smem, int richardson);
cudaError_t launch_replay_paths(const ReplayArgs& a, int kind, cudaStream_t s);
cudaError_t launch_replay_reduce(const ReplayArgs& a, int kind, const int* task_m, const int* task_d,
                                 const int* task_i, int ntask, const int64_t* task_out,
                                 const int64_t* knot_task_off, double* Gside, double* GGside,
                                 cudaStream_t s);
// FP64 factorisation of every shape's Psi and the cardinal-function tables.
// lu: scratch of the ipsi layout; piv, uinv: scratch of the sh_t layout
cudaError_t launch_rbf_setup(const DevLayout& L, int max_n, int max_nbins, double* ipsi, float* tab,
                             double* lu, int* piv, double* uinv,
                             unsigned* err_flags, cudaStream_t s);
// CSR column indices of G from the stencils' column lists
cudaError_t launch_expand_cols(int K, const int64_t* row_ptr, const int* knot_stencil, const int64_t* st_off,
                               const int* st_cols, int* col, cudaStream_t s);
// B = g(x0) for boundary knots; finalisation of B, BB, G_var.
cudaError_t launch_boundary_b(const DevLayout& L, const ProblemDev& P, int mode, const int* knots,
                              int n, double* B, double* BB, cudaStream_t s);
// Variance-adaptive paths: rescale the pilot's G/GG rows, finalise with per-knot N.
cudaError_t launch_scale_rows(const int* mc, int n, const int64_t* row_ptr, const double* scale, double* G,
                              double* GG, cudaStream_t s);
cudaError_t launch_finalize_n(const int* mc_knots, int n_mc, const int* knot_N, const double* Bsum,
                              const double* BBsum, double* B, double* BB, int64_t nnz, const double* G,
                              double* GG_to_var, int want_var, cudaStream_t s);
// Subdomain interior solves (k_subdomain.cu).
size_t subdomain_smem(int m);
// grid: optional nsub (m + 1) + 1 nodes per side, the solution with its edges
cudaError_t launch_subdomain(const DevLayout& L, const ProblemDev& P, int nsub, int m, int n, const int* edge_knots,
                             const double* u, double* out, double* grid, cudaStream_t s);
// table-served problems (PK_LUT): BiCGSTAB with a sine-transform preconditioner;
// work = 13 m^2 doubles per subdomain
cudaError_t launch_subdomain_lut(const DevLayout& L, const ProblemDev& P, int nsub, int m, int n, const int* edge_knots,
                                 const double* u, double* out, double* work, double* grid, int max_iter, double tol,
                                 int* iters, unsigned* err, cudaStream_t s);
// tables of one outer-loop step around the grid (or the constant u0)
enum { OUTER_NEWTON_U3 = 0, OUTER_LINEAR_SHIFT = 1 };
struct OuterStep {
  int equation;                  // OUTER_*
  double u0;                     // constant iterate when there is no grid
  double a;                      // NEWTON_U3: u = a + sin(pi x) sin(pi y)
  double c2, alpha, k;           // LINEAR_SHIFT: Lap u + c2 u + F = 0, shift alpha, rescale k
};
cudaError_t launch_newton_tables(const double* grid, int G, double x0, double y0, double hx, double hy,
                                 const OuterStep& eq, float* coef, float* gtab, cudaStream_t s);
cudaError_t launch_finalize(const int* mc_knots, int n_mc, int N, const double* Bsum,
                            const double* BBsum, double* B, double* BB, const int64_t* row_ptr,
                            int64_t nnz, const double* G, double* GG_to_var, int want_var,
                            cudaStream_t s);

}  // namespace pdds
