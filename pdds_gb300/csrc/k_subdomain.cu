// Interior solution of every subdomain from the interface solution.
//
// The reference hands each subdomain's four interfaces (knot positions and
// interface solution) to an Octave spectral solver (Subdomain::Solve,
// Meshes/subdomain.cpp:80-122, Solvers/SemLin_first_VR.m).  Here one CTA
// solves one subdomain of a rectangular layout, for problems whose operator
// is Lap + c with constant c (sigma = sqrt2 I, b = 0): -Lap_h v - c v = f on
// an m x m interior grid with the 5-point Laplacian, Dirichlet data on the
// grid's boundary points = the interface solution interpolated along each
// edge (cubic Lagrange through the 4 nearest of the edge's uniform knots) or
// g on the domain boundary.  The operator is diagonalised by the orthonormal
// sine transform S (S_kl = sqrt(2/(m+1)) sin(pi k l/(m+1)), S = S^-1):
// V = S [ (S R S)_kl / (lx_k + ly_l - c) ] S, four m x m products in FP64 in
// shared memory.
#include "kernels.h"

namespace pdds {

namespace {

constexpr int SUB_THREADS = 256;

// C = A * B for m x m row-major matrices in shared memory
__device__ void mat_mul(const double* A, const double* B, double* C, int m) {
  for (int e = threadIdx.x; e < m * m; e += SUB_THREADS) {
    const int i = e / m, j = e % m;
    double acc = 0.0;
    for (int k = 0; k < m; k++) acc += A[i * m + k] * B[k * m + j];
    C[e] = acc;
  }
  __syncthreads();
}

// value at parameter s in [0, 1] along an edge with n uniform knots values[]
__device__ double edge_interp(const double* u, const int* knots, int n, double s) {
  const double g = s * (n - 1);
  int i0 = (int)floor(g) - 1;
  i0 = max(0, min(i0, n - 4));
  const double t = g - i0;  // nodes at t = 0, 1, 2, 3
  double v = 0.0;
#pragma unroll
  for (int a = 0; a < 4; a++) {
    double w = 1.0;
#pragma unroll
    for (int b = 0; b < 4; b++)
      if (b != a) w *= (t - b) / (double)(a - b);
    v += w * u[knots[i0 + a]];
  }
  return v;
}

template <int KIND>
__global__ void __launch_bounds__(SUB_THREADS) k_subdomain(const DevLayout L, const ProblemDev P, int nsub, int m,
                                                           int n, const int* edge_knots, const double* u,
                                                           double* out) {
  extern __shared__ double sm[];
  double* S = sm;              // m x m sine transform
  double* R = S + m * m;       // right-hand side, then the solution
  double* T = R + m * m;       // work
  __shared__ double s_edge[4][66];  // boundary values on the grid lines (m + 2 points), S, N, W, E
  const int sub = blockIdx.x;
  const int a = sub % nsub, b = sub / nsub;
  const double lx = (L.dom[2] - L.dom[0]) / nsub, ly = (L.dom[3] - L.dom[1]) / nsub;
  const double x0 = L.dom[0] + a * lx, y0 = L.dom[1] + b * ly;
  const double hx = lx / (m + 1), hy = ly / (m + 1);
  const double PI = 3.141592653589793;
  const double norm = sqrt(2.0 / (m + 1));
  for (int e = threadIdx.x; e < m * m; e += SUB_THREADS) {
    const int k = e / m, l = e % m;
    S[e] = norm * sin(PI * (k + 1) * (l + 1) / (m + 1));
  }
  // edges: 0 = south (y = y0), 1 = north (y = y0 + ly), 2 = west (x = x0), 3 = east (x = x0 + lx)
  for (int e = threadIdx.x; e < 4 * (m + 2); e += SUB_THREADS) {
    const int d = e / (m + 2), q = e % (m + 2);
    const int* kn = edge_knots + ((size_t)sub * 4 + d) * n;
    const double s = (double)q / (m + 1);
    double x, y;
    if (d <= 1) { x = x0 + s * lx; y = d == 0 ? y0 : y0 + ly; }
    else { x = d == 2 ? x0 : x0 + lx; y = y0 + s * ly; }
    s_edge[d][q] = kn[0] >= 0 ? edge_interp(u, kn, n, s) : u_f64<KIND>(P, x, y);
  }
  __syncthreads();
  Coef<double> kc;
  coef_f64<KIND>(P, x0 + 0.5 * lx, y0 + 0.5 * ly, kc);
  const double c = kc.c;
  // R = f + boundary neighbours of the 5-point Laplacian
  for (int e = threadIdx.x; e < m * m; e += SUB_THREADS) {
    const int j = e / m, i = e % m;  // row j (y), column i (x)
    Coef<double> k;
    coef_f64<KIND>(P, x0 + (i + 1) * hx, y0 + (j + 1) * hy, k);
    double r = k.f;
    if (i == 0) r += s_edge[2][j + 1] / (hx * hx);
    if (i == m - 1) r += s_edge[3][j + 1] / (hx * hx);
    if (j == 0) r += s_edge[0][i + 1] / (hy * hy);
    if (j == m - 1) r += s_edge[1][i + 1] / (hy * hy);
    R[e] = r;
  }
  __syncthreads();
  mat_mul(S, R, T, m);  // T = S R  (rows: y modes)
  mat_mul(T, S, R, m);  // R = S R S
  for (int e = threadIdx.x; e < m * m; e += SUB_THREADS) {
    const int l = e / m, k = e % m;  // y mode l, x mode k
    const double lxk = (2.0 - 2.0 * cos(PI * (k + 1) / (m + 1))) / (hx * hx);
    const double lyl = (2.0 - 2.0 * cos(PI * (l + 1) / (m + 1))) / (hy * hy);
    R[e] /= (lxk + lyl - c);
  }
  __syncthreads();
  mat_mul(S, R, T, m);
  mat_mul(T, S, R, m);
  double* o = out + (size_t)sub * m * m;
  for (int e = threadIdx.x; e < m * m; e += SUB_THREADS) o[e] = R[e];
}

}  // namespace

size_t subdomain_smem(int m) { return (size_t)3 * m * m * sizeof(double); }

cudaError_t launch_subdomain(const DevLayout& L, const ProblemDev& P, int nsub, int m, int n, const int* edge_knots,
                             const double* u, double* out, cudaStream_t s) {
  if (m < 2 || m > 64) return cudaErrorInvalidValue;
  const size_t smem = subdomain_smem(m);
  const int grid = nsub * nsub;
#define PDDS_SUB_CASE(KK)                                                                             \
  case KK:                                                                                            \
    cudaFuncSetAttribute(k_subdomain<KK>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);   \
    k_subdomain<KK><<<grid, SUB_THREADS, smem, s>>>(L, P, nsub, m, n, edge_knots, u, out);            \
    break;
  switch (P.kind) {
    PDDS_SUB_CASE(PK_POISSON_SINCOS)
    PDDS_SUB_CASE(PK_MONEGROS)
    PDDS_SUB_CASE(PK_HELMHOLTZ)
    default: return cudaErrorInvalidValue;
  }
#undef PDDS_SUB_CASE
  return cudaGetLastError();
}

}  // namespace pdds
