// Interface solve (I + G) u = B on the device.
//
// The reference assembles the COO triplets into an Eigen SparseMatrix, adds
// the identity and runs Jacobi-preconditioned BiCGSTAB in FP64 from a zero
// guess (PDDAlgorithms/PDDSparseGM.cpp:3168-3246).  G is produced here
// directly in CSR (rows sorted by column), and the diagonal of I + G is 1
// (a knot never belongs to its own stencil sides), so the Jacobi
// preconditioner is the identity.  Two methods:
//   BiCGSTAB in FP64 (van der Vorst 1992), the reference's method;
//   GMRES(m) in FP32 (Saad & Schultz 1986, classical Gram-Schmidt with one
//   re-orthogonalisation pass) as the inner solver of FP64 iterative
//   refinement: residuals are formed in FP64 and each refinement step restarts
//   GMRES on the normalised residual.
// Reductions are deterministic (fixed-shape two-stage sums).
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <vector>

#include "solve.h"
#include "xfer.h"

namespace pdds {

namespace {

constexpr int SPMV_THREADS = 256;
constexpr int RED_THREADS = 256;
constexpr int RED_BLOCKS = 256;

template <typename T>
__global__ void k_spmv(int K, const int64_t* __restrict__ rp, const int* __restrict__ col,
                       const T* __restrict__ val, const T* __restrict__ x, T* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < K; row += warps) {
    const int64_t e0 = rp[row], e1 = rp[row + 1];
    T acc = T(0);
    for (int64_t e = e0 + lane; e < e1; e += 32) acc += val[e] * x[col[e]];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) y[row] = x[row] + acc;
  }
}

// Stage 1 of up to two dot products: per-block partial sums (FP64).
template <typename T>
__global__ void k_dot2_part(int n, const T* a, const T* b, const T* c, const T* d, double* part) {
  __shared__ double s1[RED_THREADS], s2[RED_THREADS];
  double p1 = 0.0, p2 = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    p1 += (double)a[i] * (double)b[i];
    if (c) p2 += (double)c[i] * (double)d[i];
  }
  s1[threadIdx.x] = p1;
  s2[threadIdx.x] = p2;
  __syncthreads();
  for (int o = RED_THREADS / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      s1[threadIdx.x] += s1[threadIdx.x + o];
      s2[threadIdx.x] += s2[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s1[0];
    part[2 * blockIdx.x + 1] = s2[0];
  }
}

__global__ void k_dot2_final(int nb, const double* part, double* out1, double* out2) {
  __shared__ double s1[RED_THREADS], s2[RED_THREADS];
  double p1 = 0.0, p2 = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    p1 += part[2 * i];
    p2 += part[2 * i + 1];
  }
  s1[threadIdx.x] = p1;
  s2[threadIdx.x] = p2;
  __syncthreads();
  for (int o = RED_THREADS / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      s1[threadIdx.x] += s1[threadIdx.x + o];
      s2[threadIdx.x] += s2[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *out1 = s1[0];
    if (out2) *out2 = s2[0];
  }
}

// BiCGSTAB scalars, in one device array.
enum { S_RR = 0, S_RHO_NEW, S_RHO, S_ALPHA, S_W, S_BETA, S_R0V, S_TS, S_TT, S_COUNT };

__global__ void k_bicg_scal1(double* sc) {  // after <r,r>, <r0,r>
  const double rho_old = sc[S_RHO];
  sc[S_RHO] = sc[S_RHO_NEW];
  sc[S_BETA] = (sc[S_RHO] / rho_old) * (sc[S_ALPHA] / sc[S_W]);
}
__global__ void k_bicg_scal2(double* sc) { sc[S_ALPHA] = sc[S_RHO] / sc[S_R0V]; }
__global__ void k_bicg_scal3(double* sc) { sc[S_W] = (sc[S_TT] > 0.0) ? sc[S_TS] / sc[S_TT] : 0.0; }

__global__ void k_bicg_p(int n, const double* r, double* p, const double* v, const double* sc) {
  const double beta = sc[S_BETA], w = sc[S_W];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    p[i] = r[i] + beta * (p[i] - w * v[i]);
}
__global__ void k_bicg_s(int n, const double* r, const double* v, double* s, const double* sc) {
  const double alpha = sc[S_ALPHA];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    s[i] = r[i] - alpha * v[i];
}
__global__ void k_bicg_x(int n, double* x, const double* p, const double* s, double* r,
                         const double* t, const double* sc) {
  const double alpha = sc[S_ALPHA], w = sc[S_W];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i] += alpha * p[i] + w * s[i];
    r[i] = s[i] - w * t[i];
  }
}

__global__ void k_fill(int n, double* a, double v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = v;
}
__global__ void k_copy(int n, const double* a, double* b) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] = a[i];
}
__global__ void k_init_scal(double* sc) {
  sc[S_RHO] = 1.0; sc[S_ALPHA] = 1.0; sc[S_W] = 1.0;
}

// ---------------------------------------------------------------- GMRES
__global__ void k_to_f32(int64_t n, const double* a, float* b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}
// r = b - A x in FP64 from y = A x
__global__ void k_resid(int n, const double* b, const double* Ax, double* r) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) r[i] = b[i] - Ax[i];
}
__global__ void k_scale_to_f32(int n, const double* r, const double* nrm, float* v) {
  const double inv = 1.0 / sqrt(*nrm);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = (float)(r[i] * inv);
}

inline int vgrid(int n) { return std::max(1, std::min(1024, (n + 255) / 256)); }

}  // namespace

// ---------------------------------------------------------------- drivers
static void dot2(cudaStream_t s, int n, const double* a, const double* b, const double* c,
                 const double* d, double* part, double* o1, double* o2, int* cnt) {
  *cnt += 2;
  const int nb = std::min(RED_BLOCKS, std::max(1, (n + RED_THREADS - 1) / RED_THREADS));
  k_dot2_part<double><<<nb, RED_THREADS, 0, s>>>(n, a, b, c, d, part);
  k_dot2_final<<<1, RED_THREADS, 0, s>>>(nb, part, o1, o2);
}

cudaError_t solve_bicgstab(const SolveCsr& A, const double* b, double* x, SolveWork& w,
                           int max_iter, double tol, int* iters, double* relres, cudaStream_t s) {
  w.launches = 0;
  const int n = A.K;
  const int sg = std::max(1, std::min(4096, (n * 32 + SPMV_THREADS - 1) / SPMV_THREADS));
  const int vg = vgrid(n);
  double* r = w.v64[0];
  double* r0 = w.v64[1];
  double* p = w.v64[2];
  double* v = w.v64[3];
  double* sv = w.v64[4];
  double* t = w.v64[5];
  double* sc = w.scal;
  ++w.launches;
  k_fill<<<vg, 256, 0, s>>>(n, x, 0.0);
  ++w.launches;
  k_copy<<<vg, 256, 0, s>>>(n, b, r);
  ++w.launches;
  k_copy<<<vg, 256, 0, s>>>(n, b, r0);
  ++w.launches;
  k_fill<<<vg, 256, 0, s>>>(n, p, 0.0);
  ++w.launches;
  k_fill<<<vg, 256, 0, s>>>(n, v, 0.0);
  ++w.launches;
  k_init_scal<<<1, 1, 0, s>>>(sc);
  dot2(s, n, b, b, nullptr, nullptr, w.part, sc + S_COUNT, nullptr, &w.launches);
  double rhs_sq = 0.0;
  *iters = 0;
  *relres = 0.0;
  // launch errors of this solve, then the copy and the wait: the first
  // failure ends the solve (no further launches against a stale residual)
  cudaError_t e = cudaPeekAtLastError();
  if (e == cudaSuccess) e = copy_async(&rhs_sq, sc + S_COUNT, sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return e;
  if (rhs_sq == 0.0) return cudaSuccess;
  const double tol2 = tol * tol * rhs_sq;
  int it = 0;
  double rr = rhs_sq;
  while (it < max_iter) {
    dot2(s, n, r, r, r0, r, w.part, sc + S_RR, sc + S_RHO_NEW, &w.launches);
    e = cudaPeekAtLastError();
    if (e == cudaSuccess) e = copy_async(w.host_rr, sc + S_RR, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      *iters = it;
      return e;
    }
    rr = *w.host_rr;
    if (!(rr > tol2)) break;
    ++w.launches;
    k_bicg_scal1<<<1, 1, 0, s>>>(sc);
    ++w.launches;
    k_bicg_p<<<vg, 256, 0, s>>>(n, r, p, v, sc);
    ++w.launches;
    k_spmv<double><<<sg, SPMV_THREADS, 0, s>>>(n, A.row_ptr, A.col, A.val64, p, v);
    dot2(s, n, r0, v, nullptr, nullptr, w.part, sc + S_R0V, nullptr, &w.launches);
    ++w.launches;
    k_bicg_scal2<<<1, 1, 0, s>>>(sc);
    ++w.launches;
    k_bicg_s<<<vg, 256, 0, s>>>(n, r, v, sv, sc);
    ++w.launches;
    k_spmv<double><<<sg, SPMV_THREADS, 0, s>>>(n, A.row_ptr, A.col, A.val64, sv, t);
    dot2(s, n, t, sv, t, t, w.part, sc + S_TS, sc + S_TT, &w.launches);
    ++w.launches;
    k_bicg_scal3<<<1, 1, 0, s>>>(sc);
    ++w.launches;
    k_bicg_x<<<vg, 256, 0, s>>>(n, x, p, sv, r, t, sc);
    ++it;
  }
  *iters = it;
  if (it == max_iter) {
    dot2(s, n, r, r, nullptr, nullptr, w.part, sc + S_RR, nullptr, &w.launches);
    e = cudaPeekAtLastError();
    if (e == cudaSuccess) e = copy_async(w.host_rr, sc + S_RR, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    rr = *w.host_rr;
  }
  *relres = std::sqrt(rr / rhs_sq);
  return cudaSuccess;
}

// ---------------------------------------------------------------- fused GMRES
// One Arnoldi step is five launches and no host synchronisation: SpMV,
// dots with the basis, subtract + re-orthogonalising dots, subtract + norm
// (whose last block also applies the Givens rotations and tests
// convergence), normalise.  Reductions finish in the last block to arrive
// (a ticket counter, no waiting), and every kernel returns at once after
// the device-side convergence flag is set.
namespace {

constexpr int GM_THREADS = 256;
constexpr int GM_CHUNK = 128;    // elements per block
constexpr int GM_MAXV = 48;      // basis vectors (m + 1 <= 41)

struct GmCtl {
  unsigned ticket;
  unsigned converged;
  unsigned jdim;
  unsigned pad;
};

// last-block ticket: returns true in the block that finishes last
__device__ __forceinline__ bool gm_last_block(GmCtl* ctl) {
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned t = atomicAdd(&ctl->ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (last) __threadfence();
  return last;
}

__global__ void k_gm_spmv(int K, const int64_t* __restrict__ rp, const int* __restrict__ col,
                          const float* __restrict__ val, const float* __restrict__ x, float* __restrict__ y,
                          const GmCtl* ctl) {
  if (ctl->converged) return;
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < K; row += warps) {
    const int64_t e0 = rp[row], e1 = rp[row + 1];
    float acc = 0.f;
    for (int64_t e = e0 + lane; e < e1; e += 32) acc += val[e] * x[col[e]];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) y[row] = x[row] + acc;
  }
}

// partial dots of the chunk of wc (shared) with V[0..nv): one warp per vector
__device__ __forceinline__ void gm_chunk_dots(int n, int nv, const float* V, const float* wc, int k0, int cn,
                                              double* part) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = warp; i < nv; i += GM_THREADS / 32) {
    const float* vi = V + (int64_t)i * n + k0;
    float acc = 0.f;
    for (int k = lane; k < cn; k += 32) acc += vi[k] * wc[k];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) part[(int64_t)blockIdx.x * GM_MAXV + i] = (double)acc;
  }
}

__device__ __forceinline__ void gm_finish_dots(int nv, const double* part, double* out, bool accumulate) {
  for (int i = threadIdx.x; i < nv; i += blockDim.x) {
    double s = 0.0;
    for (int b = 0; b < (int)gridDim.x; b++) s += part[(int64_t)b * GM_MAXV + i];
    out[i] = accumulate ? out[i] + s : s;
  }
}

// h = V^T w
__global__ void k_gm_dots(int n, int nv, const float* V, const float* w, double* part, double* h, GmCtl* ctl) {
  if (ctl->converged) return;
  __shared__ float wc[GM_CHUNK];
  const int k0 = blockIdx.x * GM_CHUNK, cn = min(GM_CHUNK, n - k0);
  for (int k = threadIdx.x; k < cn; k += GM_THREADS) wc[k] = w[k0 + k];
  __syncthreads();
  gm_chunk_dots(n, nv, V, wc, k0, cn, part);
  if (gm_last_block(ctl)) {
    gm_finish_dots(nv, part, h, false);
    if (threadIdx.x == 0) ctl->ticket = 0;
  }
}

// w -= V h1; h2 = V^T w; h1 += h2
__global__ void k_gm_sub_dots(int n, int nv, const float* V, double* h1, double* h2, float* w, double* part,
                              GmCtl* ctl) {
  if (ctl->converged) return;
  __shared__ float wc[GM_CHUNK];
  __shared__ float hs[GM_MAXV];
  for (int i = threadIdx.x; i < nv; i += GM_THREADS) hs[i] = (float)h1[i];
  __syncthreads();
  const int k0 = blockIdx.x * GM_CHUNK, cn = min(GM_CHUNK, n - k0);
  for (int k = threadIdx.x; k < cn; k += GM_THREADS) {
    float acc = w[k0 + k];
    for (int i = 0; i < nv; i++) acc -= hs[i] * V[(int64_t)i * n + k0 + k];
    wc[k] = acc;
    w[k0 + k] = acc;
  }
  __syncthreads();
  gm_chunk_dots(n, nv, V, wc, k0, cn, part);
  if (gm_last_block(ctl)) {
    gm_finish_dots(nv, part, h2, false);
    __syncthreads();
    for (int i = threadIdx.x; i < nv; i += blockDim.x) h1[i] += h2[i];
    if (threadIdx.x == 0) ctl->ticket = 0;
  }
}

// w -= V h2; |w|; last block: Givens rotation of column j, convergence test
__global__ void k_gm_sub_norm(int n, int nv, const float* V, const double* h2, float* w, double* part,
                              GmCtl* ctl, int m, int j, const double* hcol, double* H, double* cs,
                              double* sn, double* g, double* inv_norm, double inner_tol) {
  if (ctl->converged) return;
  __shared__ float hs[GM_MAXV];
  __shared__ double red[GM_THREADS];
  for (int i = threadIdx.x; i < nv; i += GM_THREADS) hs[i] = (float)h2[i];
  __syncthreads();
  const int k0 = blockIdx.x * GM_CHUNK, cn = min(GM_CHUNK, n - k0);
  double ss = 0.0;
  for (int k = threadIdx.x; k < cn; k += GM_THREADS) {
    float acc = w[k0 + k];
    for (int i = 0; i < nv; i++) acc -= hs[i] * V[(int64_t)i * n + k0 + k];
    w[k0 + k] = acc;
    ss += (double)acc * (double)acc;
  }
  red[threadIdx.x] = ss;
  __syncthreads();
  for (int o = GM_THREADS / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[(int64_t)blockIdx.x * GM_MAXV] = red[0];
  if (gm_last_block(ctl) && threadIdx.x == 0) {
    double nrm2 = 0.0;
    for (int b = 0; b < (int)gridDim.x; b++) nrm2 += part[(int64_t)b * GM_MAXV];
    const double nrm = sqrt(nrm2);
    double* colj = H + (int64_t)j * (m + 1);
    for (int i = 0; i <= j; i++) colj[i] = hcol[i];
    colj[j + 1] = nrm;
    for (int i = 0; i < j; i++) {
      const double x0 = colj[i], x1 = colj[i + 1];
      colj[i] = cs[i] * x0 + sn[i] * x1;
      colj[i + 1] = -sn[i] * x0 + cs[i] * x1;
    }
    const double x0 = colj[j], x1 = colj[j + 1];
    const double r = sqrt(x0 * x0 + x1 * x1);
    cs[j] = (r > 0.0) ? x0 / r : 1.0;
    sn[j] = (r > 0.0) ? x1 / r : 0.0;
    colj[j] = r;
    colj[j + 1] = 0.0;
    g[j + 1] = -sn[j] * g[j];
    g[j] = cs[j] * g[j];
    *inv_norm = (nrm > 0.0) ? 1.0 / nrm : 0.0;
    ctl->jdim = (unsigned)(j + 1);
    if (fabs(g[j + 1]) < inner_tol || !(nrm > 0.0)) ctl->converged = 1u;
    ctl->ticket = 0;
  }
}

__global__ void k_gm_normalize(int n, const float* w, const double* inv_norm, float* vnext, const GmCtl* ctl) {
  if (ctl->converged) return;
  const float s = (float)*inv_norm;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) vnext[k] = w[k] * s;
}

__global__ void k_gm_init(double* g, int m, GmCtl* ctl) {
  for (int i = 0; i <= m; i++) g[i] = 0.0;
  g[0] = 1.0;
  ctl->ticket = 0;
  ctl->converged = 0;
  ctl->jdim = 0;
}

__global__ void k_gm_backsolve(int m, const double* H, const double* g, double* y, const GmCtl* ctl,
                               double* jdim_out) {
  const int jd = (int)ctl->jdim;
  for (int i = jd - 1; i >= 0; i--) {
    double s = g[i];
    for (int k = i + 1; k < jd; k++) s -= H[(int64_t)k * (m + 1) + i] * y[k];
    y[i] = s / H[(int64_t)i * (m + 1) + i];
  }
  *jdim_out = (double)jd;
}

__global__ void k_gm_update_x(int n, int m, const float* V, const double* y, const double* nrm2r, double* x,
                              const GmCtl* ctl) {
  const int jd = (int)ctl->jdim;
  const double scale = sqrt(*nrm2r);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int i = 0; i < jd; i++) acc += y[i] * (double)V[(int64_t)i * n + k];
    x[k] += scale * acc;
  }
}

}  // namespace

cudaError_t solve_gmres_ir(const SolveCsr& A, const double* b, double* x, SolveWork& w, int m,
                           int max_iter, int max_refine, double tol, int* iters, int* refines,
                           double* relres, cudaStream_t s) {
  w.launches = 0;
  const int n = A.K;
  if (m + 1 > GM_MAXV) m = GM_MAXV - 1;
  const int sg = std::max(1, std::min(4096, (n * 32 + SPMV_THREADS - 1) / SPMV_THREADS));
  const int vg = vgrid(n);
  const int gb = (n + GM_CHUNK - 1) / GM_CHUNK;
  double* r = w.v64[0];
  double* Ax = w.v64[1];
  double* sc = w.scal;
  double* bb = sc + 0;       // <b,b>
  double* rr = sc + 1;       // <r,r>, then jdim of the last cycle at sc[2]
  double* inv_norm = sc + 3;
  double* H = w.hess;
  double* cs = H + (m + 1) * m;
  double* sn = cs + m;
  double* g = sn + m;
  double* hcol = g + (m + 1);
  double* y = hcol + (m + 1);
  double* h2 = y + (m + 1);
  float* V = w.V32;
  float* wv = w.w32;
  GmCtl* ctl = reinterpret_cast<GmCtl*>(w.ctl);
  const int nb = std::min(RED_BLOCKS, std::max(1, (n + RED_THREADS - 1) / RED_THREADS));
  ++w.launches;
  k_to_f32<<<vgrid((int)std::min<int64_t>(A.nnz, 1 << 28)), 256, 0, s>>>(A.nnz, A.val64, w.val32);
  ++w.launches;
  k_fill<<<vg, 256, 0, s>>>(n, x, 0.0);
  dot2(s, n, b, b, nullptr, nullptr, w.part, bb, nullptr, &w.launches);
  double hb = 0.0;
  copy_async(&hb, bb, sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  *iters = 0;
  *refines = 0;
  *relres = 0.0;
  if (hb == 0.0) return cudaGetLastError();
  const double tol2 = tol * tol * hb;
  int total = 0, ref = 0;
  double hr = hb;
  for (; ref <= max_refine; ref++) {
    // FP64 residual; also reads back the size of the previous cycle
    ++w.launches;
    k_spmv<double><<<sg, SPMV_THREADS, 0, s>>>(n, A.row_ptr, A.col, A.val64, x, Ax);
    ++w.launches;
    k_resid<<<vg, 256, 0, s>>>(n, b, Ax, r);
    dot2(s, n, r, r, nullptr, nullptr, w.part, rr, nullptr, &w.launches);
    double hv[2] = {0.0, 0.0};
    copy_async(hv, rr, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    hr = hv[0];
    if (ref > 0) total += (int)hv[1];
    if (!(hr > tol2) || ref == max_refine || total >= max_iter) break;
    // FP32 GMRES(m) on A d = r / |r|
    ++w.launches;
    k_scale_to_f32<<<vg, 256, 0, s>>>(n, r, rr, V);
    ++w.launches;
    k_gm_init<<<1, 1, 0, s>>>(g, m, ctl);
    const double inner_tol = 1e-6;
    for (int j = 0; j < m; j++) {
      const int nv = j + 1;
      k_gm_spmv<<<sg, SPMV_THREADS, 0, s>>>(n, A.row_ptr, A.col, w.val32, V + (int64_t)j * n, wv, ctl);
      k_gm_dots<<<gb, GM_THREADS, 0, s>>>(n, nv, V, wv, w.part, hcol, ctl);
      k_gm_sub_dots<<<gb, GM_THREADS, 0, s>>>(n, nv, V, hcol, h2, wv, w.part, ctl);
      k_gm_sub_norm<<<gb, GM_THREADS, 0, s>>>(n, nv, V, h2, wv, w.part, ctl, m, j, hcol, H, cs, sn, g, inv_norm,
                                              inner_tol);
      k_gm_normalize<<<vg, 256, 0, s>>>(n, wv, inv_norm, V + (int64_t)(j + 1) * n, ctl);
      w.launches += 5;
    }
    k_gm_backsolve<<<1, 1, 0, s>>>(m, H, g, y, ctl, sc + 2);
    k_gm_update_x<<<vg, 256, 0, s>>>(n, m, V, y, rr, x, ctl);
    w.launches += 2;
  }
  *iters = total;
  *refines = ref;
  *relres = std::sqrt(hr / hb);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- cluster GMRES
__global__ void k_cl_single_rows(int* sys_row0, int K) {
  sys_row0[0] = 0;
  sys_row0[1] = K;
}

cudaError_t solve_gmres_ir_cluster(const SolveCsr& A, const double* b, double* x, SolveWork& w, int m,
                                   int max_iter, int max_refine, double tol, int* iters, int* refines,
                                   double* relres, cudaStream_t s, bool* used) {
  *used = false;
  w.launches = 0;
  const int n = A.K;
  if (m < 2 || m > GMRES_CLUSTER_MAX_M) return cudaSuccess;
  // large systems: the whole GPU with grid barriers; small ones: one cluster
  int gb = (n >= 4096 && w.bar && w.gpart && w.err) ? gmres_grid_blocks(n) : 0;
  if (gb > 0 && w.grid_ctas > 0) gb = std::min(gb, w.grid_ctas);
  const int cl = gb > 0 ? 0 : gmres_cluster_pick(n);
  if (gb <= 0 && cl <= 0) return cudaSuccess;
  *used = true;
  int* ctl = reinterpret_cast<int*>(w.ctl);  // [0..1] rows, [2] iterations, [3] refinements
  ++w.launches;
  k_to_f32<<<vgrid((int)std::min<int64_t>(A.nnz, 1 << 28)), 256, 0, s>>>(A.nnz, A.val64, w.val32);
  ++w.launches;
  k_cl_single_rows<<<1, 1, 0, s>>>(ctl, n);
  ClusterGmresArgs a{};
  a.err_flags = w.err;
  a.n_sys = 1;
  a.sys_row0 = ctl;
  a.K = n;
  a.row_ptr = A.row_ptr;
  a.col = A.col;
  a.val64 = A.val64;
  a.val32 = w.val32;
  a.b = b;
  a.x = x;
  a.r64 = w.v64[0];
  a.V = w.V32;
  a.Z = w.Z32;
  a.m = m;
  a.max_iter = max_iter;
  a.max_refine = max_refine;
  a.tol = tol;
  a.inner_tol = 1e-6;
  a.out_iters = ctl + 2;
  a.out_refines = ctl + 3;
  a.out_relres = w.scal;
  a.out_t_end = nullptr;
  a.spin_limit = w.spin_limit;
  ++w.launches;
  cudaError_t e = gb > 0 ? launch_gmres_grid(a, gb, n, w.bar, w.err, w.gpart, s) : launch_gmres_cluster(a, cl, n, s);
  if (e != cudaSuccess) return e;
  int hi[2] = {0, 0};
  double hr = 0.0;
  copy_async(hi, ctl + 2, 2 * sizeof(int), cudaMemcpyDeviceToHost, s);
  copy_async(&hr, w.scal, sizeof(double), cudaMemcpyDeviceToHost, s);
  e = cudaStreamSynchronize(s);
  *iters = hi[0];
  *refines = hi[1];
  *relres = hr;
  return e == cudaSuccess ? cudaGetLastError() : e;
}

cudaError_t launch_to_f32(const double* a, float* b, int64_t n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_to_f32<<<vgrid((int)std::min<int64_t>(n, 1 << 28)), 256, 0, s>>>(n, a, b);
  return cudaGetLastError();
}

}  // namespace pdds
