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
//
// Table-served problems (PK_LUT: diagonal sigma, drift, reaction and source
// from the tables) have variable coefficients; their finite-difference
// problem is solved by BiCGSTAB, right-preconditioned with the sine-transform
// solve of the constant-coefficient operator (subdomain means), one CTA per
// subdomain.  Both solvers can also write the solution with its edge values
// into one global grid of nsub (m + 1) + 1 nodes per side, from which
// k_newton_tables builds the tables of the semilinear Newton step.
#include <algorithm>

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

// Dirichlet data on the grid lines of the subdomain's edges (m + 2 points
// each; S, N, W, E): the interface solution interpolated along the edge, or g
// on the domain boundary.
template <int KIND>
__device__ void load_edges(const ProblemDev& P, int sub, int m, int n, const int* edge_knots, const double* u,
                           double x0, double y0, double lx, double ly, double (*s_edge)[66]) {
  for (int e = threadIdx.x; e < 4 * (m + 2); e += SUB_THREADS) {
    const int d = e / (m + 2), q = e % (m + 2);
    const int* kn = edge_knots + ((size_t)sub * 4 + d) * n;
    const double s = (double)q / (m + 1);
    double x, y;
    if (d <= 1) { x = x0 + s * lx; y = d == 0 ? y0 : y0 + ly; }
    else { x = d == 2 ? x0 : x0 + lx; y = y0 + s * ly; }
    s_edge[d][q] = kn[0] >= 0 ? edge_interp(u, kn, n, s) : u_f64<KIND>(P, x, y);
  }
}

// The subdomain's (m + 2)^2 grid nodes (edges and interior V[j][i]) into the
// global grid: node (a (m+1) + i', b (m+1) + j') of G per side.  Edge nodes
// shared with a neighbour receive the same interpolated value from both.
__device__ void write_grid(double* grid, int G, int a, int b, int m, const double* V, const double (*s_edge)[66]) {
  for (int e = threadIdx.x; e < (m + 2) * (m + 2); e += SUB_THREADS) {
    const int jj = e / (m + 2), ii = e % (m + 2);
    double v;
    if (jj == 0) v = s_edge[0][ii];
    else if (jj == m + 1) v = s_edge[1][ii];
    else if (ii == 0) v = s_edge[2][jj];
    else if (ii == m + 1) v = s_edge[3][jj];
    else v = V[(jj - 1) * m + (ii - 1)];
    grid[(size_t)(b * (m + 1) + jj) * G + (size_t)a * (m + 1) + ii] = v;
  }
}

// Sum over the CTA (fixed order: warp shuffles, then the warps' partials),
// returned to every thread.
__device__ double block_sum(double v, double* s_red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < SUB_THREADS / 32; w++) t += s_red[w];
  __syncthreads();
  return t;
}

template <int KIND>
__global__ void __launch_bounds__(SUB_THREADS) k_subdomain(const DevLayout L, const ProblemDev P, int nsub, int m,
                                                           int n, const int* edge_knots, const double* u,
                                                           double* out, double* grid, int G) {
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
  load_edges<KIND>(P, sub, m, n, edge_knots, u, x0, y0, lx, ly, s_edge);
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
  if (grid) write_grid(grid, G, a, b, m, R, s_edge);
}

// Table-served operator ax v_xx + ay v_yy + bx v_x + by v_y + c v + f = 0
// (ax = sigma11^2 / 2, ay = sigma22^2 / 2, coefficients sampled from the
// tables at the grid nodes), central differences:
//   (A v)_ij = -(ax (v_i+1 - 2 v_ij + v_i-1) / hx^2 + ay (v_j+1 - 2 v_ij + v_j-1) / hy^2
//               + bx (v_i+1 - v_i-1) / (2 hx) + by (v_j+1 - v_j-1) / (2 hy) + c v_ij),
// A v = f + the known edge neighbours.  BiCGSTAB (van der Vorst) with the
// right preconditioner M = -(mean ax D_xx + mean ay D_yy + min(mean c, 0)),
// inverted by the sine transform; vectors in `work` (13 m^2 doubles per
// subdomain), the transform in shared memory.  Stops at ||r|| <= tol ||b|| or
// after max_iter iterations (then ERR_FLAG_SUB_NOCONV).
__global__ void __launch_bounds__(SUB_THREADS) k_subdomain_lut(const DevLayout L, const ProblemDev P, int nsub, int m,
                                                               int n, const int* edge_knots, const double* u,
                                                               double* out, double* work, double* grid, int G,
                                                               int max_iter, double tol, int* iters, unsigned* err) {
  extern __shared__ double sm[];
  double* S = sm;
  double* R = S + m * m;
  double* T = R + m * m;
  __shared__ double s_edge[4][66];
  __shared__ double s_red[SUB_THREADS / 32];
  const int sub = blockIdx.x;
  const int a = sub % nsub, b = sub / nsub;
  const double lx = (L.dom[2] - L.dom[0]) / nsub, ly = (L.dom[3] - L.dom[1]) / nsub;
  const double x0 = L.dom[0] + a * lx, y0 = L.dom[1] + b * ly;
  const double hx = lx / (m + 1), hy = ly / (m + 1);
  const double ihx2 = 1.0 / (hx * hx), ihy2 = 1.0 / (hy * hy), i2hx = 0.5 / hx, i2hy = 0.5 / hy;
  const double PI = 3.141592653589793;
  const double norm = sqrt(2.0 / (m + 1));
  const int mm = m * m;
  double* W = work + (size_t)sub * 13 * mm;
  double* cax = W;
  double* cay = W + mm;
  double* cbx = W + 2 * mm;
  double* cby = W + 3 * mm;
  double* cc = W + 4 * mm;
  double* x = W + 5 * mm;
  double* r = W + 6 * mm;
  double* r0 = W + 7 * mm;
  double* p = W + 8 * mm;
  double* v = W + 9 * mm;
  double* ph = W + 10 * mm;
  double* sh = W + 11 * mm;
  double* t = W + 12 * mm;
  for (int e = threadIdx.x; e < mm; e += SUB_THREADS) {
    const int k = e / m, l = e % m;
    S[e] = norm * sin(PI * (k + 1) * (l + 1) / (m + 1));
  }
  load_edges<PK_LUT>(P, sub, m, n, edge_knots, u, x0, y0, lx, ly, s_edge);
  __syncthreads();
  double pa = 0.0, pb = 0.0, pc = 0.0;
  for (int e = threadIdx.x; e < mm; e += SUB_THREADS) {
    const int j = e / m, i = e % m;
    double fv[8];
    lut_sample<double, 8>(P.lut, x0 + (i + 1) * hx, y0 + (j + 1) * hy, fv);
    const double ax = 0.5 * fv[0] * fv[0], ay = 0.5 * fv[1] * fv[1], bx = fv[2], by = fv[3], c = fv[4];
    double rhs = fv[5];
    if (i == 0) rhs += (ax * ihx2 - bx * i2hx) * s_edge[2][j + 1];
    if (i == m - 1) rhs += (ax * ihx2 + bx * i2hx) * s_edge[3][j + 1];
    if (j == 0) rhs += (ay * ihy2 - by * i2hy) * s_edge[0][i + 1];
    if (j == m - 1) rhs += (ay * ihy2 + by * i2hy) * s_edge[1][i + 1];
    cax[e] = ax; cay[e] = ay; cbx[e] = bx; cby[e] = by; cc[e] = c;
    x[e] = 0.0; r[e] = rhs; r0[e] = rhs; p[e] = 0.0; v[e] = 0.0;
    pa += ax; pb += ay; pc += c;
  }
  const double ma = block_sum(pa, s_red) / mm, mb = block_sum(pb, s_red) / mm;
  const double mc = fmin(block_sum(pc, s_red) / mm, 0.0);
  auto dot = [&](const double* A, const double* B) {
    double q = 0.0;
    for (int e = threadIdx.x; e < mm; e += SUB_THREADS) q += A[e] * B[e];
    return block_sum(q, s_red);  // synchronises: the vectors' writes are visible after it
  };
  auto apply = [&](const double* in, double* o) {
    for (int e = threadIdx.x; e < mm; e += SUB_THREADS) {
      const int j = e / m, i = e % m;
      const double c0 = in[e];
      const double w = i > 0 ? in[e - 1] : 0.0, ea = i < m - 1 ? in[e + 1] : 0.0;
      const double so = j > 0 ? in[e - m] : 0.0, no = j < m - 1 ? in[e + m] : 0.0;
      o[e] = -(cax[e] * (ea - 2.0 * c0 + w) * ihx2 + cay[e] * (no - 2.0 * c0 + so) * ihy2 +
               cbx[e] * (ea - w) * i2hx + cby[e] * (no - so) * i2hy + cc[e] * c0);
    }
    __syncthreads();
  };
  auto precond = [&](const double* in, double* o) {
    for (int e = threadIdx.x; e < mm; e += SUB_THREADS) R[e] = in[e];
    __syncthreads();
    mat_mul(S, R, T, m);
    mat_mul(T, S, R, m);
    for (int e = threadIdx.x; e < mm; e += SUB_THREADS) {
      const int l = e / m, k = e % m;
      const double lxk = (2.0 - 2.0 * cos(PI * (k + 1) / (m + 1))) * ihx2;
      const double lyl = (2.0 - 2.0 * cos(PI * (l + 1) / (m + 1))) * ihy2;
      R[e] /= (ma * lxk + mb * lyl - mc);
    }
    __syncthreads();
    mat_mul(S, R, T, m);
    mat_mul(T, S, R, m);
    for (int e = threadIdx.x; e < mm; e += SUB_THREADS) o[e] = R[e];
    __syncthreads();
  };
  const double bnorm = sqrt(dot(r, r));
  double rho = 1.0, alpha = 1.0, omega = 1.0;
  int it = 0;
  bool conv = !(bnorm > 0.0);
  while (!conv && it < max_iter) {
    ++it;
    const double rho1 = dot(r0, r);
    if (rho1 == 0.0) break;
    const double beta = (rho1 / rho) * (alpha / omega);
    rho = rho1;
    for (int e = threadIdx.x; e < mm; e += SUB_THREADS) p[e] = r[e] + beta * (p[e] - omega * v[e]);
    __syncthreads();
    precond(p, ph);
    apply(ph, v);
    const double r0v = dot(r0, v);
    if (r0v == 0.0) break;
    alpha = rho / r0v;
    for (int e = threadIdx.x; e < mm; e += SUB_THREADS) r[e] -= alpha * v[e];  // r holds s
    __syncthreads();
    if (sqrt(dot(r, r)) <= tol * bnorm) {
      for (int e = threadIdx.x; e < mm; e += SUB_THREADS) x[e] += alpha * ph[e];
      __syncthreads();
      conv = true;
      break;
    }
    precond(r, sh);
    apply(sh, t);
    const double tt = dot(t, t);
    omega = tt > 0.0 ? dot(t, r) / tt : 0.0;
    for (int e = threadIdx.x; e < mm; e += SUB_THREADS) {
      x[e] += alpha * ph[e] + omega * sh[e];
      r[e] -= omega * t[e];
    }
    __syncthreads();
    if (sqrt(dot(r, r)) <= tol * bnorm) conv = true;
    if (omega == 0.0) break;
  }
  if (threadIdx.x == 0) {
    iters[sub] = it;
    if (!conv) atomicOr(err, ERR_FLAG_SUB_NOCONV);
  }
  double* o = out + (size_t)sub * mm;
  for (int e = threadIdx.x; e < mm; e += SUB_THREADS) o[e] = x[e];
  if (grid) write_grid(grid, G, a, b, m, x, s_edge);
}

// Tables of one step of an outer loop around the iterate u_k, on the G x G
// grid of spacings (hx, hy) from (x0, y0); u_k = the grid values, or the
// constant u0 (grad 0) when grid is null; grad u_k (second-order differences)
// feeds the control variate.  Two equations:
//
// NEWTON_U3: the Newton linearisation of Lap u - u^3 + F = 0
//   (BVPs/EDPs/Semilinear_u3_VR.hpp: u = A + sin(pi x) sin(pi y),
//   F = 2 pi^2 sin(pi x) sin(pi y) + u^3; EquationSM_c_LUT, EquationSM_f_LUT,
//   EquationSM_grad_LUT): sigma = sqrt2 I, b = 0, c = -3 u_k^2,
//   f = F + 2 u_k^3; g table = A + sin(pi x) sin(pi y), the Dirichlet data on
//   the boundary of the unit square.
// LINEAR_SHIFT: the fixed-point splitting of Lap u + C2 u + F = 0 with the
//   shift alpha and time rescale k (BVPs/EDPs/Salou_Iterative.hpp:
//   u = sin(2 pi x + 1/2) cos(pi^2 (x + y)), F = -Lap u - C2 u;
//   EquationLI_sigma, EquationLI_c_LUT, EquationLI_f_LUT):
//   sigma = sqrt(2/k) I, b = 0, c = (C2 - alpha)/k, f = (F + alpha u_k)/k;
//   g table = u.
__global__ void k_newton_tables(const double* grid, int G, double x0, double y0, double hx, double hy,
                                const OuterStep eq, float4* coef, float* gtab) {
  const int64_t N = (int64_t)G * G;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < N; q += (int64_t)gridDim.x * blockDim.x) {
    const int I = (int)(q % G), J = (int)(q / G);
    const double X = x0 + I * hx, Y = y0 + J * hy;
    double uk = eq.u0, gx = 0.0, gy = 0.0;
    if (grid) {
      const double* row = grid + (size_t)J * G;
      uk = row[I];
      const double i2hx = 0.5 / hx, i2hy = 0.5 / hy;
      if (I == 0) gx = (-3.0 * row[0] + 4.0 * row[1] - row[2]) * i2hx;
      else if (I == G - 1) gx = (3.0 * row[G - 1] - 4.0 * row[G - 2] + row[G - 3]) * i2hx;
      else gx = (row[I + 1] - row[I - 1]) * i2hx;
      const double* col = grid + I;
      if (J == 0) gy = (-3.0 * col[0] + 4.0 * col[G] - col[2 * (size_t)G]) * i2hy;
      else if (J == G - 1)
        gy = (3.0 * col[(size_t)(G - 1) * G] - 4.0 * col[(size_t)(G - 2) * G] + col[(size_t)(G - 3) * G]) * i2hy;
      else gy = (col[(size_t)(J + 1) * G] - col[(size_t)(J - 1) * G]) * i2hy;
    }
    constexpr double PI = 3.141592653589793, PI2 = 9.869604401089358;
    if (eq.equation == OUTER_LINEAR_SHIFT) {
      // u = S C with S = sin(2 pi x + 1/2), C = cos(pi^2 (x + y)):
      // u_xx = -(4 pi^2 + pi^4) u - 4 pi^3 cos(2 pi x + 1/2) sin(pi^2 (x + y)),
      // u_yy = -pi^4 u
      double S, Sc, Cs, C;
      sincos(2.0 * PI * X + 0.5, &S, &Sc);
      sincos(PI2 * (X + Y), &Cs, &C);
      const double ue = S * C;
      const double lap = -(4.0 * PI2 + 2.0 * PI2 * PI2) * ue - 4.0 * PI2 * PI * Sc * Cs;
      const double F = -lap - eq.c2 * ue;
      const double ik = 1.0 / eq.k;
      const float sg = (float)sqrt(2.0 * ik);
      coef[2 * q] = make_float4(sg, sg, 0.f, 0.f);
      coef[2 * q + 1] =
          make_float4((float)((eq.c2 - eq.alpha) * ik), (float)((F + eq.alpha * uk) * ik), (float)gx, (float)gy);
      gtab[q] = (float)ue;
    } else {
      double sx, cx, sy, cy;
      sincospi(X, &sx, &cx);
      sincospi(Y, &sy, &cy);
      const double sp = sx * sy, ue = eq.a + sp;
      const double F = 2.0 * PI2 * sp + ue * ue * ue;
      coef[2 * q] = make_float4(1.41421356f, 1.41421356f, 0.f, 0.f);
      coef[2 * q + 1] = make_float4((float)(-3.0 * uk * uk), (float)(F + 2.0 * uk * uk * uk), (float)gx, (float)gy);
      gtab[q] = (float)ue;
    }
  }
}

}  // namespace

size_t subdomain_smem(int m) { return (size_t)3 * m * m * sizeof(double); }

cudaError_t launch_subdomain(const DevLayout& L, const ProblemDev& P, int nsub, int m, int n, const int* edge_knots,
                             const double* u, double* out, double* grid, cudaStream_t s) {
  if (m < 2 || m > 64) return cudaErrorInvalidValue;
  const size_t smem = subdomain_smem(m);
  const int nblk = nsub * nsub;
  const int G = nsub * (m + 1) + 1;
#define PDDS_SUB_CASE(KK)                                                                             \
  case KK:                                                                                            \
    cudaFuncSetAttribute(k_subdomain<KK>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);   \
    k_subdomain<KK><<<nblk, SUB_THREADS, smem, s>>>(L, P, nsub, m, n, edge_knots, u, out, grid, G);   \
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

cudaError_t launch_subdomain_lut(const DevLayout& L, const ProblemDev& P, int nsub, int m, int n, const int* edge_knots,
                                 const double* u, double* out, double* work, double* grid, int max_iter, double tol,
                                 int* iters, unsigned* err, cudaStream_t s) {
  if (m < 2 || m > 64) return cudaErrorInvalidValue;
  const size_t smem = subdomain_smem(m);
  cudaFuncSetAttribute(k_subdomain_lut, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_subdomain_lut<<<nsub * nsub, SUB_THREADS, smem, s>>>(L, P, nsub, m, n, edge_knots, u, out, work, grid,
                                                         nsub * (m + 1) + 1, max_iter, tol, iters, err);
  return cudaGetLastError();
}

cudaError_t launch_newton_tables(const double* grid, int G, double x0, double y0, double hx, double hy,
                                 const OuterStep& eq, float* coef, float* gtab, cudaStream_t s) {
  const int64_t N = (int64_t)G * G;
  const int blocks = (int)std::min<int64_t>((N + 255) / 256, 4096);
  k_newton_tables<<<blocks, 256, 0, s>>>(grid, G, x0, y0, hx, hy, eq, reinterpret_cast<float4*>(coef), gtab);
  return cudaGetLastError();
}

}  // namespace pdds
