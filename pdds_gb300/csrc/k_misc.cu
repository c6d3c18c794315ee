// Boundary knots and the per-knot finalisation of B, BB and G_var.
//   Solve_OMP_Analytic boundary shortcut  Solvers/EMFKACSolver.hpp:720-727 (B = g, BB = B^2)
//   B = b/N, BB = bb/N                     Solvers/EMFKACSolver.hpp:570-571
//   var_G = GG/N - (G/N)^2                 Meshes/stencil.cpp:403
#include "kernels.h"

namespace pdds {

namespace {

template <int KIND>
__device__ double g_port(const ProblemDev& P, double x, double y) {
  if (KIND == PK_POISSON_SINCOS) {
    double sx, cx, sy, cy;
    pm::sincos(pm::PI * x, &sx, &cx);
    pm::sincos(pm::PI * y, &sy, &cy);
    return sx * cy + x * y;
  } else if (KIND == PK_HELMHOLTZ) {
    double sa, ca, sb, cb;
    pm::sincos(P.p[0] * x, &sa, &ca);
    pm::sincos(P.p[1] * y, &sb, &cb);
    return sa * cb;
  } else if (KIND == PK_VARCOEF) {
    double s2, c2;
    pm::sincos(2.0 * y, &s2, &c2);
    return pm::exp(x) * c2 + 1.0;
  } else if (KIND == PK_LUT) {
    return lut_sample_g<double>(P.lut, x, y);
  }
  return u_f64<PK_MONEGROS>(P, x, y);
}

template <int KIND>
__global__ void k_boundary(const DevLayout L, const ProblemDev P, int portable, const int* knots,
                           int n, double* B, double* BB) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int k = knots[t];
  const double x = L.kx[k], y = L.ky[k];
  ProblemDev Pk = P;
  uint32_t ri = 0, rk = 0;
  instance_params(L, k, Pk, ri, rk);
  const double g = portable ? g_port<KIND>(Pk, x, y) : u_f64<KIND>(Pk, x, y);
  B[k] = g;
  BB[k] = g * g;
}

__global__ void k_finalize_b(const int* mc, int n, int N, const double* Bsum, const double* BBsum,
                             double* B, double* BB) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int k = mc[t];
  B[k] = Bsum[k] / N;
  BB[k] = BBsum[k] / N;
}

// Per-knot path counts (variance-adaptive N): B = b / N_k, BB = bb / N_k.
__global__ void k_finalize_b_n(const int* mc, int n, const int* knot_N, const double* Bsum, const double* BBsum,
                               double* B, double* BB) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int k = mc[t];
  const double inv = 1.0 / (double)knot_N[k];
  B[k] = Bsum[k] * inv;
  BB[k] = BBsum[k] * inv;
}

// G and GG rows of the given knots scaled by scale[k] (one warp per knot):
// the pilot's entries, normalised by its N, renormalised to the final N_k.
__global__ void k_scale_rows(const int* mc, int n, const int64_t* row_ptr, const double* scale, double* G,
                             double* GG) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= n) return;
  const int k = mc[w];
  const double f = scale[k];
  for (int64_t e = row_ptr[k] + lane; e < row_ptr[k + 1]; e += 32) {
    G[e] *= f;
    if (GG) GG[e] *= f;
  }
}

__global__ void k_finalize_var(int64_t nnz, const double* G, double* GG) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nnz) return;
  GG[e] = GG[e] - G[e] * G[e];
}

}  // namespace

cudaError_t launch_boundary_b(const DevLayout& L, const ProblemDev& P, int mode, const int* knots,
                              int n, double* B, double* BB, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const int portable = (mode == 0 && P.kind != PK_MONEGROS) ? 1 : 0;
  const int g = (n + 127) / 128;
  switch (P.kind) {
    case PK_POISSON_SINCOS: k_boundary<PK_POISSON_SINCOS><<<g, 128, 0, s>>>(L, P, portable, knots, n, B, BB); break;
    case PK_MONEGROS: k_boundary<PK_MONEGROS><<<g, 128, 0, s>>>(L, P, 0, knots, n, B, BB); break;
    case PK_HELMHOLTZ: k_boundary<PK_HELMHOLTZ><<<g, 128, 0, s>>>(L, P, portable, knots, n, B, BB); break;
    case PK_LUT: k_boundary<PK_LUT><<<g, 128, 0, s>>>(L, P, portable, knots, n, B, BB); break;
    case PK_CIRCLE: k_boundary<PK_CIRCLE><<<g, 128, 0, s>>>(L, P, 0, knots, n, B, BB); break;
    case PK_ROBIN: k_boundary<PK_ROBIN><<<g, 128, 0, s>>>(L, P, 0, knots, n, B, BB); break;
    default: k_boundary<PK_VARCOEF><<<g, 128, 0, s>>>(L, P, portable, knots, n, B, BB); break;
  }
  return cudaGetLastError();
}

cudaError_t launch_finalize(const int* mc_knots, int n_mc, int N, const double* Bsum,
                            const double* BBsum, double* B, double* BB, const int64_t* row_ptr,
                            int64_t nnz, const double* G, double* GG_to_var, int want_var,
                            cudaStream_t s) {
  (void)row_ptr;
  if (n_mc > 0) k_finalize_b<<<(n_mc + 127) / 128, 128, 0, s>>>(mc_knots, n_mc, N, Bsum, BBsum, B, BB);
  if (want_var && nnz > 0)
    k_finalize_var<<<(unsigned)((nnz + 255) / 256), 256, 0, s>>>(nnz, G, GG_to_var);
  return cudaGetLastError();
}

cudaError_t launch_scale_rows(const int* mc, int n, const int64_t* row_ptr, const double* scale, double* G,
                              double* GG, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_scale_rows<<<(n + 7) / 8, 256, 0, s>>>(mc, n, row_ptr, scale, G, GG);
  return cudaGetLastError();
}

cudaError_t launch_finalize_n(const int* mc_knots, int n_mc, const int* knot_N, const double* Bsum,
                              const double* BBsum, double* B, double* BB, int64_t nnz, const double* G,
                              double* GG_to_var, int want_var, cudaStream_t s) {
  if (n_mc > 0) k_finalize_b_n<<<(n_mc + 127) / 128, 128, 0, s>>>(mc_knots, n_mc, knot_N, Bsum, BBsum, B, BB);
  if (want_var && nnz > 0)
    k_finalize_var<<<(unsigned)((nnz + 255) / 256), 256, 0, s>>>(nnz, G, GG_to_var);
  return cudaGetLastError();
}

// Hand-out order of the MIXED work items, heaviest knots first: the knots
// sorted by the path steps of the last estimate in decreasing groups of a
// quarter octave (a counting sort in one CTA, key = 4 log2(steps) + the next
// two bits; order inside a group is arbitrary).  Longest-first hand-out keeps
// a long item from starting near the end of the launch.
namespace {
__device__ __forceinline__ int lpt_key(unsigned long long s) {
  if (s < 4ull) return (int)s;
  const int e = 63 - __clzll((long long)s);
  return 4 * e + (int)((s >> (e - 2)) & 3ull);  // <= 255
}
__global__ void k_lpt_order(const int* mc, int n, const unsigned long long* steps, int* out) {
  __shared__ int cnt[256], off[256];
  for (int b = threadIdx.x; b < 256; b += blockDim.x) cnt[b] = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) atomicAdd(&cnt[255 - lpt_key(steps[mc[i]])], 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int b = 0; b < 256; b++) {
      off[b] = acc;
      acc += cnt[b];
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) out[atomicAdd(&off[255 - lpt_key(steps[mc[i]])], 1)] = mc[i];
}
}  // namespace

// CSR column indices of G: row k is its stencil's column list (one warp per knot).
namespace {
__global__ void k_expand_cols(int K, const int64_t* row_ptr, const int* knot_stencil, const int64_t* st_off,
                              const int* st_cols, int* col) {
  const int k = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (k >= K) return;
  const int64_t e0 = row_ptr[k], len = row_ptr[k + 1] - e0;
  if (len == 0) return;
  const int* src = st_cols + st_off[knot_stencil[k]];
  for (int64_t q = lane; q < len; q += 32) col[e0 + q] = src[q];
}
}  // namespace

cudaError_t launch_expand_cols(int K, const int64_t* row_ptr, const int* knot_stencil, const int64_t* st_off,
                               const int* st_cols, int* col, cudaStream_t s) {
  if (K <= 0) return cudaSuccess;
  k_expand_cols<<<(unsigned)(((int64_t)K * 32 + 255) / 256), 256, 0, s>>>(K, row_ptr, knot_stencil, st_off, st_cols,
                                                                          col);
  return cudaGetLastError();
}

cudaError_t launch_lpt_order(const int* mc, int n, const unsigned long long* steps, int* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_lpt_order<<<1, 1024, 0, s>>>(mc, n, steps, out);
  return cudaGetLastError();
}

}  // namespace pdds
