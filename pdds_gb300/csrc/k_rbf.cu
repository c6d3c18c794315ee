// FP64 factorisation of the Gaussian RBF interpolation matrices and the
// cardinal-function tables used by the MIXED kernel.
//
// The reference inverts Psi_ij = exp(-|p_i - p_j|^2 / c^2) for every side of
// every knot with Eigen's FullPivLU (Meshes/stencil.cpp:115-184, 211-243).
// Here one CTA inverts one side shape (sides that are translates of each
// other share Psi) by LU factorisation with partial pivoting in shared memory
// followed by one forward/back substitution per column, in FP64: cond(Psi)
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

__global__ void __launch_bounds__(RBF_THREADS) k_invert(const DevLayout L, double* ipsi_out,
                                                        unsigned* err_flags) {
  extern __shared__ double A[];  // n x n, row-major; becomes L\U
  __shared__ int s_piv;
  __shared__ double s_val[RBF_THREADS];
  __shared__ int s_idx[RBF_THREADS];
  __shared__ int prow[512];
  const int sh = blockIdx.x, tid = threadIdx.x;
  const int n = L.sh_n[sh];
  const double c = L.sh_c[sh];
  const double* t = L.sh_t + L.sh_t_off[sh];
  const double ic2 = 1.0 / (c * c);
  const double Rarc = L.sh_R ? L.sh_R[sh] : 0.0;  // arcs: chord 2 R sin(dphi / 2)
  for (int e = tid; e < n * n; e += RBF_THREADS) {
    const int i = e / n, j = e % n;
    const double d = Rarc > 0.0 ? 2.0 * Rarc * sin(0.5 * (t[i] - t[j])) : t[i] - t[j];
    A[e] = exp(-(d * d) * ic2);
  }
  for (int i = tid; i < n; i += RBF_THREADS) prow[i] = i;
  __syncthreads();
  // LU factorisation with partial (row) pivoting, right-looking
  for (int k = 0; k < n; k++) {
    double best = -1.0;
    int bi = k;
    for (int i = k + tid; i < n; i += RBF_THREADS) {
      const double v = fabs(A[i * n + k]);
      if (v > best) { best = v; bi = i; }
    }
    s_val[tid] = best;
    s_idx[tid] = bi;
    __syncthreads();
    for (int o = RBF_THREADS / 2; o > 0; o >>= 1) {
      if (tid < o) {
        const double v2 = s_val[tid + o];
        const int i2 = s_idx[tid + o];
        if (v2 > s_val[tid] || (v2 == s_val[tid] && i2 < s_idx[tid])) { s_val[tid] = v2; s_idx[tid] = i2; }
      }
      __syncthreads();
    }
    if (tid == 0) {
      s_piv = s_idx[0];
      if (!(s_val[0] > 1e-300)) atomicOr(err_flags, ERR_FLAG_SINGULAR);
      if (s_idx[0] != k) {
        const int tmp = prow[k];
        prow[k] = prow[s_idx[0]];
        prow[s_idx[0]] = tmp;
      }
    }
    __syncthreads();
    const int p = s_piv;
    if (p != k)
      for (int j = tid; j < n; j += RBF_THREADS) {
        const double tmp = A[k * n + j];
        A[k * n + j] = A[p * n + j];
        A[p * n + j] = tmp;
      }
    __syncthreads();
    const double ipiv = 1.0 / A[k * n + k];
    for (int i = k + 1 + tid; i < n; i += RBF_THREADS) A[i * n + k] *= ipiv;
    __syncthreads();
    const int m = n - k - 1;
    for (int e = tid; e < m * m; e += RBF_THREADS) {
      const int i = k + 1 + e / m, j = k + 1 + e % m;
      A[i * n + j] -= A[i * n + k] * A[k * n + j];
    }
    __syncthreads();
  }
  // inverse column by column: L U x = P e_c, one thread per column, the
  // output column itself is the work vector (coalesced across threads)
  double* out = ipsi_out + L.sh_ipsi_off[sh];
  for (int col = tid; col < n; col += RBF_THREADS) {
    for (int i = 0; i < n; i++) {
      double v = (prow[i] == col) ? 1.0 : 0.0;
      for (int j = 0; j < i; j++) v -= A[i * n + j] * out[(int64_t)j * n + col];
      out[(int64_t)i * n + col] = v;
    }
    for (int i = n - 1; i >= 0; i--) {
      double v = out[(int64_t)i * n + col];
      for (int j = i + 1; j < n; j++) v -= A[i * n + j] * out[(int64_t)j * n + col];
      out[(int64_t)i * n + col] = v / A[i * n + i];
    }
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
                             unsigned* err_flags, cudaStream_t s) {
  if (L.P == 0) return cudaSuccess;
  if (max_n > 160) return cudaErrorInvalidValue;
  const size_t smem = (size_t)(max_n * max_n) * sizeof(double);
  cudaFuncSetAttribute(k_invert, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_invert<<<L.P, RBF_THREADS, smem, s>>>(L, ipsi, err_flags);
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
