// FP64 factorisation of the Gaussian RBF interpolation matrices and the
// cardinal-function tables used by the MIXED kernel.
//
// The reference inverts Psi_ij = exp(-|p_i - p_j|^2 / c^2) for every side of
// every knot with Eigen's FullPivLU (Meshes/stencil.cpp:115-184, 211-243).
// Here each side shape (sides that are translates of each other share Psi)
// is inverted by LU factorisation with partial pivoting (one CTA per shape,
// in shared memory) followed by one forward/back substitution per column
// (one warp per column, over the whole GPU), in FP64: cond(Psi)
// reaches 1e10..3e11, so the inverse needs double precision, and it needs a
// backward-stable method -- Gauss-Jordan elimination, tried first, gave
// cardinal weights wrong by 1e-3 (and by O(1) for 126-knot sides) against an
// extended-precision solve, where LU stays within 1e-7..2e-5.  The tables H[b][i] = sum_j Psi^-1(j,i) exp(-(t_j - s_b)^2/c^2)
// on the exit-bin grid s_b are accumulated in FP64 and stored in FP32: the
// cardinal functions are bounded by ~1, so storing them in FP32 costs 6e-8
// relative and no amplification.
#include "kernels.h"

namespace pdds {

namespace {

constexpr int RBF_THREADS = 256;

// Psi of every shape, row-major, one element per thread over many CTAs
// (FP64 exponentials issue slowly: spread over the GPU, not one CTA per shape).
__global__ void __launch_bounds__(RBF_THREADS) k_psi(const DevLayout L, double* psi) {
  const int sh = blockIdx.y;
  const int n = L.sh_n[sh];
  const int e = blockIdx.x * RBF_THREADS + threadIdx.x;
  if (e >= n * n) return;
  const double c = L.sh_c[sh];
  const double* t = L.sh_t + L.sh_t_off[sh];
  const double ic2 = 1.0 / (c * c);
  const double Rarc = L.sh_R ? L.sh_R[sh] : 0.0;  // arcs: chord 2 R sin(dphi / 2)
  const int i = e / n, j = e % n;
  const double d = Rarc > 0.0 ? 2.0 * Rarc * sin(0.5 * (t[i] - t[j])) : t[i] - t[j];
  psi[L.sh_ipsi_off[sh] + e] = exp(-(d * d) * ic2);
}

// |x| of a double as an integer whose order is the order of |x| (IEEE
// encoding of non-negative values): the pivot search compares integers.
__device__ __forceinline__ unsigned long long abs_key(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}

// LU factorisation with partial (row) pivoting of one shape's Psi, right-
// looking, in shared memory (one CTA per shape).  Pivot: the largest |a_ik|,
// the smallest row index among equal ones.  Output, for the inverse kernel:
// the factors column-major (lu[j n + i] = (L\U)_ij), the row permutation and
// 1 / u_ii.
__global__ void __launch_bounds__(RBF_THREADS) k_lu(const DevLayout L, double* lu, int* piv, double* uinv,
                                                    unsigned* err_flags) {
  extern __shared__ double A[];  // n x n, row-major; becomes L\U
  __shared__ unsigned long long s_key[RBF_THREADS / 32];
  __shared__ int s_row[RBF_THREADS / 32];
  __shared__ int s_piv;
  __shared__ double s_ipiv;
  __shared__ int prow[512];
  const int sh = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n = L.sh_n[sh];
  double* g = lu + L.sh_ipsi_off[sh];
  for (int e = tid; e < n * n; e += RBF_THREADS) A[e] = g[e];  // Psi from k_psi
  for (int i = tid; i < n; i += RBF_THREADS) prow[i] = i;
  __syncthreads();
  for (int k = 0; k < n; k++) {
    unsigned long long best = 0;
    int bi = n;
    for (int i = k + tid; i < n; i += RBF_THREADS) {
      const unsigned long long v = abs_key(A[i * n + k]);
      if (v > best || bi == n) { best = v; bi = i; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long v2 = __shfl_xor_sync(0xffffffffu, best, o);
      const int i2 = __shfl_xor_sync(0xffffffffu, bi, o);
      if (v2 > best || (v2 == best && i2 < bi)) { best = v2; bi = i2; }
    }
    if (lane == 0) { s_key[warp] = best; s_row[warp] = bi; }
    __syncthreads();
    if (tid == 0) {
      best = s_key[0];
      bi = s_row[0];
      for (int w = 1; w < RBF_THREADS / 32; w++)
        if (s_key[w] > best || (s_key[w] == best && s_row[w] < bi)) { best = s_key[w]; bi = s_row[w]; }
      const double pv = A[bi * n + k];
      if (!(fabs(pv) > 1e-300)) atomicOr(err_flags, ERR_FLAG_SINGULAR);
      s_piv = bi;
      s_ipiv = 1.0 / pv;
      if (bi != k) {
        const int tmp = prow[k];
        prow[k] = prow[bi];
        prow[bi] = tmp;
      }
    }
    __syncthreads();
    const int p = s_piv;
    if (p != k) {
      for (int j = tid; j < n; j += RBF_THREADS) {
        const double tmp = A[k * n + j];
        A[k * n + j] = A[p * n + j];
        A[p * n + j] = tmp;
      }
      __syncthreads();
    }
    const double ipiv = s_ipiv;
    for (int i = k + 1 + tid; i < n; i += RBF_THREADS) A[i * n + k] *= ipiv;
    __syncthreads();
    // trailing update: warps over rows, lanes over columns
    for (int i = k + 1 + warp; i < n; i += RBF_THREADS / 32) {
      const double lik = A[i * n + k];
      for (int j = k + 1 + lane; j < n; j += 32) A[i * n + j] -= lik * A[k * n + j];
    }
    __syncthreads();
  }
  for (int e = tid; e < n * n; e += RBF_THREADS) {
    const int j = e / n, i = e % n;
    g[e] = A[i * n + j];
  }
  const int64_t vo = L.sh_t_off[sh];
  for (int i = tid; i < n; i += RBF_THREADS) {
    piv[vo + i] = prow[i];
    uinv[vo + i] = 1.0 / A[i * n + i];
  }
}

// Columns of Psi^-1 from the factors: L U x = P e_c, one warp per column c,
// rows k = 32 s + lane held in registers v[s].  Column-oriented substitution:
// once x_i is final it is broadcast and every later (forward) or earlier
// (backward) row subtracts l_ki x_i, reading column i of the factors
// (contiguous): one shuffle and at most RBF_SLOTS FMAs per row instead of a
// dependent chain of n FMAs per column.  The CTA first stages the factors in
// shared memory (16 loads in flight per thread), so the per-row reads on the
// dependent chain are shared-memory reads.
constexpr int RBF_SLOTS = 5;  // n <= 160
constexpr int INV_WARPS = 4;
__global__ void __launch_bounds__(INV_WARPS * 32) k_lu_inverse(const DevLayout L, const double* lu, const int* piv,
                                                               const double* uinv, double* ipsi_out) {
  extern __shared__ double F[];  // n x n factors, column-major
  const int sh = blockIdx.y, lane = threadIdx.x & 31;
  const int n = L.sh_n[sh];
  if (blockIdx.x * INV_WARPS >= n) return;  // CTA-uniform
  {
    const double* g = lu + L.sh_ipsi_off[sh];
    const int nn = n * n;
    constexpr int T = INV_WARPS * 32, U = 16;
    for (int e0 = threadIdx.x; e0 < nn; e0 += T * U) {
      double t[U];
#pragma unroll
      for (int u = 0; u < U; u++) t[u] = e0 + T * u < nn ? __ldg(g + e0 + T * u) : 0.0;
#pragma unroll
      for (int u = 0; u < U; u++)
        if (e0 + T * u < nn) F[e0 + T * u] = t[u];
    }
  }
  __syncthreads();
  const int col = blockIdx.x * INV_WARPS + (threadIdx.x >> 5);
  if (col >= n) return;
  const int64_t vo = L.sh_t_off[sh];
  double v[RBF_SLOTS];
#pragma unroll
  for (int s = 0; s < RBF_SLOTS; s++) {
    const int k = 32 * s + lane;
    v[s] = (k < n && piv[vo + k] == col) ? 1.0 : 0.0;
  }
  // forward: unit lower triangle
  for (int i = 0; i < n - 1; i++) {
    const int si = i >> 5;
    double own = v[0];
#pragma unroll
    for (int s = 1; s < RBF_SLOTS; s++)
      if (s == si) own = v[s];
    const double xi = __shfl_sync(0xffffffffu, own, i & 31);
    const double* Fi = F + (int64_t)i * n;
#pragma unroll
    for (int s = 0; s < RBF_SLOTS; s++) {
      const int k = 32 * s + lane;
      if (s >= si && k > i && k < n) v[s] = fma(-Fi[k], xi, v[s]);
    }
  }
  // backward: upper triangle, x_i = v_i / u_ii
  for (int i = n - 1; i >= 0; i--) {
    const int si = i >> 5;
    double own = v[0];
#pragma unroll
    for (int s = 1; s < RBF_SLOTS; s++)
      if (s == si) own = v[s];
    const double xi = __shfl_sync(0xffffffffu, own, i & 31) * __ldg(uinv + vo + i);
    const double* Fi = F + (int64_t)i * n;
#pragma unroll
    for (int s = 0; s < RBF_SLOTS; s++) {
      const int k = 32 * s + lane;
      if (s <= si) {
        if (k < i) v[s] = fma(-Fi[k], xi, v[s]);
        else if (k == i) v[s] = xi;
      }
    }
  }
  double* out = ipsi_out + L.sh_ipsi_off[sh];
#pragma unroll
  for (int s = 0; s < RBF_SLOTS; s++) {
    const int k = 32 * s + lane;
    if (k < n) out[(int64_t)k * n + col] = v[s];
  }
}

// H[b][i] for one shape and a tile of bins.
constexpr int TAB_TILE = 16;
__global__ void __launch_bounds__(RBF_THREADS) k_tables(const DevLayout L, const double* ipsi,
                                                        float* tab) {
  extern __shared__ double r[];  // [TAB_TILE][n]
  const int sh = blockIdx.y, tid = threadIdx.x;
  const int n = L.sh_n[sh], nb = L.sh_nbins[sh];
  const int b0 = blockIdx.x * TAB_TILE;
  if (b0 >= nb) return;
  const int nt = min(TAB_TILE, nb - b0);
  const double c = L.sh_c[sh], ic2 = 1.0 / (c * c);
  const double* t = L.sh_t + L.sh_t_off[sh];
  const double delta = L.sh_delta[sh];
  const double s0 = L.sh_lo[sh] - delta;
  const double Rarc = L.sh_R ? L.sh_R[sh] : 0.0;
  for (int e = tid; e < nt * n; e += RBF_THREADS) {
    const int q = e / n, j = e % n;
    const double s = s0 + (double)(b0 + q) * delta;
    const double d = Rarc > 0.0 ? 2.0 * Rarc * sin(0.5 * (t[j] - s)) : t[j] - s;
    r[e] = exp(-(d * d) * ic2);
  }
  __syncthreads();
  const double* ip = ipsi + L.sh_ipsi_off[sh];
  float* out = tab + L.sh_tab_off[sh];
  for (int e = tid; e < nt * n; e += RBF_THREADS) {
    const int q = e / n, i = e % n;
    double acc = 0.0;
    for (int j = 0; j < n; j++) acc += ip[(int64_t)j * n + i] * r[q * n + j];
    out[(int64_t)(b0 + q) * n + i] = (float)acc;
  }
}

}  // namespace

cudaError_t launch_rbf_setup(const DevLayout& L, int max_n, int max_nbins, double* ipsi, float* tab,
                             double* lu, int* piv, double* uinv, unsigned* err_flags, cudaStream_t s) {
  if (L.P == 0) return cudaSuccess;
  if (max_n > 32 * RBF_SLOTS) return cudaErrorInvalidValue;
  k_psi<<<dim3((max_n * max_n + RBF_THREADS - 1) / RBF_THREADS, L.P), RBF_THREADS, 0, s>>>(L, lu);
  const size_t smem = (size_t)(max_n * max_n) * sizeof(double);
  cudaFuncSetAttribute(k_lu, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_lu<<<L.P, RBF_THREADS, smem, s>>>(L, lu, piv, uinv, err_flags);
  cudaFuncSetAttribute(k_lu_inverse, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_lu_inverse<<<dim3((max_n + INV_WARPS - 1) / INV_WARPS, L.P), INV_WARPS * 32, smem, s>>>(L, lu, piv, uinv,
                                                                                           ipsi);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (tab) {
    const size_t smem2 = (size_t)TAB_TILE * max_n * sizeof(double);
    dim3 grid((max_nbins + TAB_TILE - 1) / TAB_TILE, L.P);
    k_tables<<<grid, RBF_THREADS, smem2, s>>>(L, ipsi, tab);
    e = cudaGetLastError();
  }
  return e;
}

}  // namespace pdds
