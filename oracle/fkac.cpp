// CPU ORACLE -- TEST INFRASTRUCTURE ONLY (see oracle_internal.h).
// Feynman-Kac path loop, exit reduction, RBF stencil weights and the
// interface solve, restated from
//   BVPs/Domains/rectangle.hpp:7-229      Rectangle2D (signed distance, projection)
//   BVPs/BVP.hpp:84-87                    Default_RBF (Gaussian)
//   Integrators/FKACIntegrator.hpp:46-57  Step, control-variate variant
//   Integrators/FKACIntegrator.hpp:167-222 Inside (Gobet-Menozzi shifted exit)
//   Solvers/EMFKACSolver.hpp:108-216      Simulate_OMP (linear + sublinear legs)
//   Solvers/EMFKACSolver.hpp:514-575      Reduce_Analytic (G, B)
//   Solvers/EMFKACSolver.hpp:711-729      Solve_OMP_Analytic (boundary shortcut)
//   Meshes/stencil.cpp:115-184            Compute_ipsi (FullPivLU inverse, cond)
//   Meshes/stencil.cpp:244-307            G_update (side order S, N, W, E)
//   Meshes/stencil.cpp:343-406            G_return_withrep ("=+" overwrite)
//   PDDAlgorithms/PDDSparseGM.cpp:795-848 worker loop (B_var = B^2 - BB)
//   PDDAlgorithms/PDDSparseGM.cpp:3168-3246 Compute_Solution (I+G, BiCGSTAB)
// The Boost mt19937 + normal_distribution increments of the reference are
// replaced by Philox-4x32-10 + Box-Muller (pdds_portable.h), keyed by
// (seed, instance, knot, path, step pair), so runs are reproducible.
#include <cmath>
#include <algorithm>
#include <cstring>
#include <limits>
#include <map>
#include <vector>

#include "../pdds_gb300/csrc/pdds_portable.h"
#include "oracle.h"
#include "oracle_internal.h"

#if defined(_OPENMP)
#include <omp.h>
#endif

namespace orc {
namespace {

struct LibmMath {
  static double exp(double x) { return std::exp(x); }
  static double log(double x) { return std::log(x); }
  static void sincos(double x, double* s, double* c) { *s = std::sin(x); *c = std::cos(x); }
  static void normals(uint32_t a, uint32_t b, double* z0, double* z1) {
    const double u0 = pdds::u01_fp64(a), u1 = pdds::u01_fp64(b);
    const double rho = std::sqrt(-2.0 * std::log(u0));
    const double t = pdds::pm::TWO_PI * u1;
    *z0 = rho * std::cos(t);
    *z1 = rho * std::sin(t);
  }
};
struct PortMath {
  static double exp(double x) { return pdds::pm::exp(x); }
  static double log(double x) { return pdds::pm::log(x); }
  static void sincos(double x, double* s, double* c) { pdds::pm::sincos(x, s, c); }
  static void normals(uint32_t a, uint32_t b, double* z0, double* z1) {
    pdds::box_muller_portable(a, b, z0, z1);
  }
};

const double SQRT2 = 1.4142135623730951;
const double PI = pdds::pm::PI;
const double TWO_PI_SQ = 19.739208802178716;  // 2 pi^2

// Tables of the LUT problem (orc_set_lut): bicubic Catmull-Rom in FP64 from
// FP32 nodes, clamped at the edges, in the operation order of the device
// sampler so the replay mode stays bit-exact.
struct LutTables {
  std::vector<float> coef, g;  // [ny][nx][8], [ny][nx]
  int nx = 0, ny = 0;
  double x0 = 0, y0 = 0, inv_dx = 0, inv_dy = 0;
};
LutTables g_lut;

void cr_w(double t, double* w) {
  const double t2 = t * t, t3 = t2 * t;
  w[0] = 0.5 * ((2.0 * t2 - t3) - t);
  w[1] = 0.5 * ((3.0 * t3 - 5.0 * t2) + 2.0);
  w[2] = 0.5 * ((4.0 * t2 - 3.0 * t3) + t);
  w[3] = 0.5 * (t3 - t2);
}
void lut_c(double x, double x0, double inv, int n, int& i, double& t) {
  double g = (x - x0) * inv;
  g = g < 0.0 ? 0.0 : g;
  g = g > (double)(n - 1) ? (double)(n - 1) : g;
  i = (int)std::floor(g);
  if (i > n - 2) i = n - 2;
  t = g - (double)i;
}
int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
void lut_sample8(double x, double y, double* out) {
  const LutTables& L = g_lut;
  int ix, iy;
  double tx, ty, wx[4], wy[4];
  lut_c(x, L.x0, L.inv_dx, L.nx, ix, tx);
  lut_c(y, L.y0, L.inv_dy, L.ny, iy, ty);
  cr_w(tx, wx);
  cr_w(ty, wy);
  for (int f = 0; f < 8; f++) out[f] = 0.0;
  for (int r = 0; r < 4; r++) {
    const float* row = &L.coef[(size_t)8 * clampi(iy - 1 + r, 0, L.ny - 1) * L.nx];
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int c = 0; c < 4; c++) {
      const float* v = row + 8 * clampi(ix - 1 + c, 0, L.nx - 1);
      for (int f = 0; f < 8; f++) acc[f] += wx[c] * (double)v[f];
    }
    for (int f = 0; f < 8; f++) out[f] += wy[r] * acc[f];
  }
}
double lut_sample_g(double x, double y) {
  const LutTables& L = g_lut;
  int ix, iy;
  double tx, ty, wx[4], wy[4];
  lut_c(x, L.x0, L.inv_dx, L.nx, ix, tx);
  lut_c(y, L.y0, L.inv_dy, L.ny, iy, ty);
  cr_w(tx, wx);
  cr_w(ty, wy);
  double out = 0.0;
  for (int r = 0; r < 4; r++) {
    const float* row = &L.g[(size_t)clampi(iy - 1 + r, 0, L.ny - 1) * L.nx];
    double acc = 0.0;
    for (int c = 0; c < 4; c++) acc += wx[c] * (double)row[clampi(ix - 1 + c, 0, L.nx - 1)];
    out += wy[r] * acc;
  }
  return out;
}

// Coefficients at one point: sigma (row-major 2x2), drift b, reaction c,
// source f, gradient of u (control variate).
struct Coef {
  double s[4], b[2], c, f, gr[2];
};

// Monegros problem, BVPs/EDPs/Monegros_Poisson_CPP.hpp:4-81, libm only.
namespace mon {
const double k1 = 1.0, k2 = 0.01, k3 = 0.02, k4 = 0.12, k5 = 0.05, k6 = 0.05, k7 = -0.12,
             sf = 0.333;
double u(double x, double y) {
  return 3.0 + sf * (std::sin(std::sqrt(k1 + k2 * x * x + k3 * y * y)) +
                     std::tanh(std::sin(k4 * x + k5 * y) + std::sin(k6 * x + k7 * y)));
}
double dudx(double x, double y) {
  return sf * ((std::cos(std::sqrt(k1 + k2 * x * x + k3 * y * y)) * k2 * x /
                std::sqrt(k1 + k2 * x * x + k3 * y * y)) -
               (k4 * std::cos(k4 * x + k5 * y) + k6 * std::cos(k6 * x + k7 * y)) *
                   (std::pow(std::tanh(std::sin(k4 * x + k5 * y) + std::sin(k6 * x + k7 * y)), 2) - 1));
}
double dudy(double x, double y) {
  return sf * (std::cos(std::sqrt(k1 + k2 * x * x + k3 * y * y)) * k1 * k3 * y /
                   std::sqrt(k1 + k2 * x * x + k3 * y * y) -
               (k5 * std::cos(k4 * x + k5 * y) + k7 * std::cos(k6 * x + k7 * y)) *
                   (std::pow(std::tanh(std::sin(k4 * x + k5 * y) + std::sin(k6 * x + k7 * y)), 2) - 1));
}
double d2x(double x, double y) {
  double a1 = std::sqrt(k1 + k2 * x * x + k3 * y * y),
         a2 = std::tanh(std::sin(k4 * x + k5 * y) + std::sin(k6 * x + k7 * y));
  return sf * (((k2 / a1) - (k2 * k2 * x * x / std::pow(a1, 3))) * std::cos(a1) -
               (x * x * k2 * k2 / (a1 * a1)) * std::sin(a1) +
               2.0 * std::pow(k4 * std::cos(k4 * x + k5 * y) + k6 * std::cos(k6 * x + k7 * y), 2) *
                   (std::pow(a2, 2) - 1) * a2 +
               (k4 * k4 * std::sin(k4 * x + k5 * y) + k6 * k6 * std::sin(k6 * x + k7 * y)) *
                   (std::pow(a2, 2) - 1));
}
double d2y(double x, double y) {
  double a1 = std::sqrt(k1 + k2 * x * x + k3 * y * y),
         a2 = std::tanh(std::sin(k4 * x + k5 * y) + std::sin(k6 * x + k7 * y));
  return sf * (((k3 / a1) - (k3 * k3 * y * y / std::pow(a1, 3))) * std::cos(a1) -
               (y * y * k3 * k3 / (a1 * a1)) * std::sin(a1) +
               2.0 * std::pow(k5 * std::cos(k4 * x + k5 * y) + k7 * std::cos(k6 * x + k7 * y), 2) *
                   (std::pow(a2, 2) - 1) * a2 +
               (k5 * k5 * std::sin(k4 * x + k5 * y) + k7 * k7 * std::sin(k6 * x + k7 * y)) *
                   (std::pow(a2, 2) - 1));
}
}  // namespace mon

template <class M>
struct Problem {
  const orc_problem* P;
  double u(double x, double y) const {
    switch (P->kind) {
      case ORC_POISSON_SINCOS: {
        double sx, cx, sy, cy;
        M::sincos(PI * x, &sx, &cx);
        M::sincos(PI * y, &sy, &cy);
        return sx * cy + x * y;
      }
      case ORC_MONEGROS: return mon::u(x, y);
      case ORC_HELMHOLTZ: {
        double sa, ca, sb, cb;
        M::sincos(P->p[0] * x, &sa, &ca);
        M::sincos(P->p[1] * y, &sb, &cb);
        return sa * cb;
      }
      case ORC_VARCOEF: {
        double s2, c2;
        M::sincos(2.0 * y, &s2, &c2);
        return M::exp(x) * c2 + 1.0;
      }
      case ORC_LUT: return lut_sample_g(x, y);
    }
    return 0.0;
  }
  double g(double x, double y) const { return u(x, y); }
  void coef(double x, double y, Coef& k) const {
    switch (P->kind) {
      case ORC_LUT: {
        double v[8];
        lut_sample8(x, y, v);
        k.s[0] = v[0]; k.s[1] = 0.0; k.s[2] = 0.0; k.s[3] = v[1];
        k.b[0] = v[2]; k.b[1] = v[3]; k.c = v[4]; k.f = v[5]; k.gr[0] = v[6]; k.gr[1] = v[7];
        return;
      }
      case ORC_POISSON_SINCOS: {
        double sx, cx, sy, cy;
        M::sincos(PI * x, &sx, &cx);
        M::sincos(PI * y, &sy, &cy);
        k.s[0] = SQRT2; k.s[1] = 0.0; k.s[2] = 0.0; k.s[3] = SQRT2;
        k.b[0] = 0.0; k.b[1] = 0.0; k.c = 0.0;
        k.f = TWO_PI_SQ * (sx * cy);
        k.gr[0] = PI * (cx * cy) + y;
        k.gr[1] = x - PI * (sx * sy);
        return;
      }
      case ORC_MONEGROS: {
        const double s = 1.41421356237;  // Equation_sigma
        k.s[0] = s; k.s[1] = 0.0; k.s[2] = 0.0; k.s[3] = s;
        k.b[0] = 0.0; k.b[1] = 0.0; k.c = -0.0;
        k.f = -mon::d2x(x, y) - mon::d2y(x, y);
        k.gr[0] = mon::dudx(x, y);
        k.gr[1] = mon::dudy(x, y);
        return;
      }
      case ORC_HELMHOLTZ: {
        const double a = P->p[0], b = P->p[1], c = P->p[2];
        double sa, ca, sb, cb;
        M::sincos(a * x, &sa, &ca);
        M::sincos(b * y, &sb, &cb);
        k.s[0] = SQRT2; k.s[1] = 0.0; k.s[2] = 0.0; k.s[3] = SQRT2;
        k.b[0] = 0.0; k.b[1] = 0.0; k.c = c;
        k.f = ((a * a + b * b) - c) * (sa * cb);
        k.gr[0] = a * (ca * cb);
        k.gr[1] = -(b * (sa * sb));
        return;
      }
      case ORC_VARCOEF: {
        const double s1 = 1.0 + 0.5 * (x * x), s2 = 1.0 + 0.5 * (y * y);
        double sn, cs;
        M::sincos(2.0 * y, &sn, &cs);
        const double ex = M::exp(x);
        const double ux = ex * cs, uy = -2.0 * (ex * sn), uxx = ux, uyy = -4.0 * ux;
        const double c = -(1.0 + x * x + y * y);
        const double u = ux + 1.0;
        k.s[0] = s1; k.s[1] = 0.0; k.s[2] = 0.0; k.s[3] = s2;
        k.b[0] = y; k.b[1] = -x; k.c = c;
        k.f = -(0.5 * (s1 * s1 * uxx + s2 * s2 * uyy) + (y * ux - x * uy) + c * u);
        k.gr[0] = ux;
        k.gr[1] = uy;
        return;
      }
    }
  }
};

// Rectangle2D (rectangle.hpp:7-229): signed distance (negative inside), the
// projection E onto the nearest side, and the outward normal N.
double rect2d(const double* p, double x, double y, double* E, double* N) {
  const double c0 = 0.5 * (p[0] + p[2]), c1 = 0.5 * (p[1] + p[3]);
  const double h0 = p[2] - c0, h1 = p[3] - c1;
  const double d0 = std::fabs(x - c0), d1 = std::fabs(y - c1);
  const bool right = x > c0, top = y > c1;
  const double ex = right ? (h0 + c0) : (-h0 + c0);
  const double ey = top ? (h1 + c1) : (-h1 + c1);
  const double nx = right ? 1.0 : -1.0, ny = top ? 1.0 : -1.0;
  const double diag = (double)0.70710678118f;
  E[0] = x; E[1] = y;
  if (d0 <= h0 && d1 <= h1) {
    if (d0 - h0 > d1 - h1) {
      E[0] = ex; N[0] = nx; N[1] = 0.0;
      return d0 - h0;
    }
    E[1] = ey; N[0] = 0.0; N[1] = ny;
    return d1 - h1;
  }
  if (d0 > h0) {
    if (d1 > h1) {
      const double r = std::sqrt((d0 - h0) * (d0 - h0) + (d1 - h1) * (d1 - h1));
      E[0] = ex; E[1] = ey; N[0] = right ? diag : -diag; N[1] = top ? diag : -diag;
      return r;
    }
    E[0] = ex; N[0] = nx; N[1] = 0.0;
    return d0 - h0;
  }
  E[1] = ey; N[0] = 0.0; N[1] = ny;
  return d1 - h1;
}

// Gaussian RBF exp(-|X - Xj|^2 / c^2) with the norm squared as in BVP.hpp:86.
template <class M>
double rbf(double ax, double ay, double bx, double by, double c) {
  const double d0 = ax - bx, d1 = ay - by;
  const double nrm = std::sqrt(d0 * d0 + d1 * d1);
  return M::exp(-(nrm * nrm) / (c * c));
}

struct PathOut {
  double x, y, Y, Z, xi;       // end of the linear leg (projection, weights)
  double sx, sy, sY, sZ, sxi;  // end of the sublinear leg (the linear one's when it does not run)
  int32_t steps_l, steps_s;
  int status;
};

// One path of Simulate_OMP (EMFKACSolver.hpp:138-213).
template <class M>
PathOut run_path(const Problem<M>& pb, const double* sp, double x0, double y0, double h,
                 double sqrth, uint64_t seed, uint32_t inst, uint32_t knot, uint32_t path,
                 bool sublinear, int64_t max_steps) {
  double X[2] = {x0, y0}, Y = 1.0, Z = 0.0, xi = 0.0;
  double E[2], Nn[2];
  Coef k;
  uint32_t step = 0;
  pdds::u32x4 blk;
  auto one_step = [&]() {
    // Step, control-variate variant (FKACIntegrator.hpp:46-57)
    pb.coef(X[0], X[1], k);
    if ((step & 1u) == 0) blk = pdds::path_block(seed, inst, knot, path, step >> 1);
    double z0, z1;
    if ((step & 1u) == 0) M::normals(blk.v[0], blk.v[1], &z0, &z1);
    else M::normals(blk.v[2], blk.v[3], &z0, &z1);
    step++;
    const double i0 = sqrth * z0, i1 = sqrth * z1;
    const double v0 = (-k.s[0]) * k.gr[0] + (-k.s[2]) * k.gr[1];
    const double v1 = (-k.s[1]) * k.gr[0] + (-k.s[3]) * k.gr[1];
    xi += Y * (v0 * i0 + v1 * i1);
    Z += k.f * Y * h;
    Y += k.c * Y * h;
    const double t0 = k.b[0] * h + (k.s[0] * i0 + k.s[1] * i1);
    const double t1 = k.b[1] * h + (k.s[2] * i0 + k.s[3] * i1);
    X[0] += t0;
    X[1] += t1;
  };
  // Inside (FKACIntegrator.hpp:168-222) for an absorbing boundary: true = keep going.
  auto inside = [&](double gobet) {
    const double d = rect2d(sp, X[0], X[1], E, Nn);
    Coef ks;
    pb.coef(X[0], X[1], ks);
    const double w0 = Nn[0] * ks.s[0] + Nn[1] * ks.s[2];
    const double w1 = Nn[0] * ks.s[1] + Nn[1] * ks.s[3];
    return d < gobet * std::sqrt(w0 * w0 + w1 * w1) * sqrth;
  };
  PathOut o;
  o.status = 0;
  int64_t n = 0;
  do {
    one_step();
    if (++n > max_steps) { o.status = 3; break; }
  } while (inside(-0.5826));
  o.x = E[0]; o.y = E[1]; o.Y = Y; o.Z = Z; o.xi = xi;
  o.steps_l = (int32_t)n;
  int64_t ns = 0;
  if (sublinear && o.status == 0) {
    do {
      one_step();
      if (++ns > max_steps) { o.status = 3; break; }
    } while (inside(0.0));
  }
  o.steps_s = (int32_t)ns;
  // X_tau_sublin etc. of Simulate_OMP (EMFKACSolver.hpp:205-209)
  o.sx = ns ? E[0] : o.x; o.sy = ns ? E[1] : o.y; o.sY = Y; o.sZ = Z; o.sxi = xi;
  return o;
}

// Full-pivot LU inverse (the algorithm of Eigen::FullPivLU::compute/inverse,
// restated): returns the rank.
int fullpiv_inverse(int n, std::vector<double> A, std::vector<double>& inv) {
  std::vector<int> rt(n), ct(n);
  double maxpivot = 0.0;
  int nz = n;
  for (int k = 0; k < n; k++) {
    double big = -1.0;
    int bi = k, bj = k;
    for (int j = k; j < n; j++)  // column-major scan, first maximum wins
      for (int i = k; i < n; i++) {
        const double a = std::fabs(A[i * n + j]);
        if (a > big) { big = a; bi = i; bj = j; }
      }
    if (big == 0.0) {
      nz = k;
      for (int q = k; q < n; q++) { rt[q] = q; ct[q] = q; }
      break;
    }
    if (big > maxpivot) maxpivot = big;
    rt[k] = bi;
    ct[k] = bj;
    if (bi != k)
      for (int j = 0; j < n; j++) std::swap(A[k * n + j], A[bi * n + j]);
    if (bj != k)
      for (int i = 0; i < n; i++) std::swap(A[i * n + k], A[i * n + bj]);
    const double piv = A[k * n + k];
    for (int i = k + 1; i < n; i++) A[i * n + k] /= piv;
    for (int i = k + 1; i < n; i++) {
      const double l = A[i * n + k];
      for (int j = k + 1; j < n; j++) A[i * n + j] -= l * A[k * n + j];
    }
  }
  const double thr = std::fabs(maxpivot) * (std::numeric_limits<double>::epsilon() * n);
  int rank = 0;
  for (int i = 0; i < nz; i++)
    if (std::fabs(A[i * n + i]) > thr) rank++;
  // inverse = Q U^-1 L^-1 P, column by column of the identity
  std::vector<int> prow(n), pcol(n);
  for (int i = 0; i < n; i++) { prow[i] = i; pcol[i] = i; }
  for (int k = 0; k < n; k++) std::swap(prow[k], prow[rt[k]]);
  for (int k = n - 1; k >= 0; k--) std::swap(pcol[k], pcol[ct[k]]);
  inv.assign((size_t)n * n, 0.0);
  std::vector<double> c(n);
  for (int col = 0; col < n; col++) {
    for (int i = 0; i < n; i++) c[i] = (prow[i] == col) ? 1.0 : 0.0;
    for (int i = 0; i < n; i++)
      for (int j = 0; j < i; j++) c[i] -= A[i * n + j] * c[j];
    for (int i = rank - 1; i >= 0; i--) {
      for (int j = i + 1; j < rank; j++) c[i] -= A[i * n + j] * c[j];
      c[i] /= A[i * n + i];
    }
    for (int i = rank; i < n; i++) c[i] = 0.0;
    for (int i = 0; i < n; i++) inv[(size_t)i * n + col] = c[pcol[i]];
  }
  return rank;
}

template <class M>
void build_psi(int n, const double* x, const double* y, double c, std::vector<double>& psi) {
  psi.resize((size_t)n * n);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) psi[(size_t)i * n + j] = rbf<M>(x[i], y[i], x[j], y[j], c);
}

struct SideData {
  int n = 0;
  double c = 0.0;
  std::vector<double> ipsi;  // ipsi(j,i) at [j*n + i]
  std::vector<double> G, GG;
};

template <class M>
int knot_impl(const Layout& L, const orc_problem* P, const orc_params* prm, int knot, double x0,
              double y0, const double* ipsi_in, std::vector<int>& gj, std::vector<double>& g,
              std::vector<double>& gvar, double* B, double* BB, int64_t* stats,
              std::vector<PathOut>* paths_out, double* diag) {
  Problem<M> pb{P};
  Stencil st = compute_stencil(L, knot);
  SideData sd[4];
  int status = 0;
  size_t off = 0;
  for (int d = 0; d < 4; d++) {  // Compute_ipsi per side, c = fac[kind] (stencil.cpp:211-243)
    const int n = (int)st.index[d].size();
    sd[d].n = n;
    if (n == 0) continue;
    const int kind = st.kind[d];
    sd[d].c = (kind >= 0 && kind < 4) ? prm->fac[kind] : prm->fac[0];
    if (ipsi_in) {
      sd[d].ipsi.assign(ipsi_in + off, ipsi_in + off + (size_t)n * n);
      off += (size_t)n * n;
    } else {
      std::vector<double> xs(n), ys(n), psi;
      for (int i = 0; i < n; i++) { xs[i] = st.pos[d][i][0]; ys[i] = st.pos[d][i][1]; }
      build_psi<M>(n, xs.data(), ys.data(), sd[d].c, psi);
      if (fullpiv_inverse(n, psi, sd[d].ipsi) < n) status = 5;
    }
    sd[d].G.assign(n, 0.0);
    sd[d].GG.assign(n, 0.0);
  }
  gj.clear(); g.clear(); gvar.clear();
  for (int q = 0; q < 4; q++) stats[q] = 0;
  double E[2], Nn[2];
  // Solve_OMP_Analytic boundary shortcut (EMFKACSolver.hpp:720-727)
  if (!(std::fabs(rect2d(st.global, x0, y0, E, Nn)) > 1e-08)) {
    *B = pb.g(x0, y0);
    *BB = (*B) * (*B);
    return status;
  }
  const int N = prm->N;
  double h = prm->h;
  if (prm->adaptive_h) {
    // adaptive step of the reference's iterative solvers (PDDSparseGM.cpp:4026-4028)
    const double d = rect2d(st.params, x0, y0, E, Nn);
    if (d <= -1E-04) {
      Coef k0;
      pb.coef(x0, y0, k0);
      const double w0 = Nn[0] * k0.s[0] + Nn[1] * k0.s[2];
      const double w1 = Nn[0] * k0.s[1] + Nn[1] * k0.s[3];
      const double q = d / (std::sqrt(w0 * w0 + w1 * w1) * 2 * 0.5826);
      const double ha = q * q;
      h = std::min(h, ha);
    }
  }
  const double sqrth = std::sqrt(h);
  std::vector<PathOut> paths(N);
#if defined(_OPENMP)
#pragma omp parallel for schedule(static) num_threads(prm->threads > 0 ? prm->threads : 1)
#endif
  for (int n = 0; n < N; n++)
    paths[n] = run_path<M>(pb, st.params, x0, y0, h, sqrth, prm->seed, prm->instance,
                           (uint32_t)knot, (uint32_t)n, prm->sublinear != 0, prm->max_steps);
  double b = 0.0, bb = 0.0;
  if (prm->fast_reduce) {
    // linearity form of Reduce_Analytic + G_update: S_j = sum over the exits
    // on a side of Y r_j(X), per thread, then G_i = -sum_j ipsi(j,i) S_j
    int off[5] = {0, 0, 0, 0, 0};
    for (int d = 0; d < 4; d++) off[d + 1] = off[d] + sd[d].n;
    const int nthr = prm->threads > 0 ? prm->threads : 1;
    std::vector<double> Sth((size_t)nthr * off[4], 0.0);
    int64_t s0 = 0, s1 = 0, s2 = 0, s3 = 0;
    int err = 0;
#if defined(_OPENMP)
#pragma omp parallel for schedule(static) num_threads(nthr) reduction(+ : b, bb, s0, s1, s2, s3) reduction(max : err)
#endif
    for (int n = 0; n < N; n++) {
#if defined(_OPENMP)
      double* S = Sth.data() + (size_t)omp_get_thread_num() * off[4];
#else
      double* S = Sth.data();
#endif
      const PathOut& o = paths[n];
      double Ea[2], Na[2];
      if (o.status) err = std::max(err, o.status);
      s0 += o.steps_l;
      s1 += o.steps_s;
      const double score_vr = o.Z + o.Y * pb.g(o.x, o.y) + o.xi;
      if (rect2d(st.global, o.x, o.y, Ea, Na) >= -1e-08) {
        s2++;
        b += score_vr;
        bb += score_vr * score_vr;
        continue;
      }
      s3++;
      int d = -1;
      if (std::fabs(o.y - st.params[1]) < 1e-8) d = South;
      else if (std::fabs(o.y - st.params[3]) < 1e-8) d = North;
      else if (std::fabs(o.x - st.params[0]) < 1e-8) d = West;
      else if (std::fabs(o.x - st.params[2]) < 1e-8) d = East;
      if (d < 0) { err = std::max(err, 1); continue; }
      for (int j = 0; j < sd[d].n; j++)
        S[off[d] + j] += o.Y * rbf<M>(st.pos[d][j][0], st.pos[d][j][1], o.x, o.y, sd[d].c);
      b += o.Z + o.xi;
      bb += (o.Z + o.xi) * (o.Z + o.xi);
    }
    if (err) status = err;
    stats[0] = s0; stats[1] = s1; stats[2] = s2; stats[3] = s3;
    for (int d = 0; d < 4; d++)
      for (int i = 0; i < sd[d].n; i++) {
        double H = 0.0;
        for (int j = 0; j < sd[d].n; j++) {
          double Sj = 0.0;
          for (int t = 0; t < nthr; t++) Sj += Sth[(size_t)t * off[4] + off[d] + j];
          H += sd[d].ipsi[(size_t)j * sd[d].n + i] * Sj;
        }
        sd[d].G[i] = -H;
        sd[d].GG[i] = 0.0;
      }
  }
  // Reduce_Analytic (EMFKACSolver.hpp:514-575), serial
  for (int n = 0; n < N && !prm->fast_reduce; n++) {
    const PathOut& o = paths[n];
    if (o.status) status = o.status;
    stats[0] += o.steps_l;
    stats[1] += o.steps_s;
    const double score = o.Z + o.Y * pb.g(o.x, o.y);
    const double score_vr = score + o.xi;
    if (rect2d(st.global, o.x, o.y, E, Nn) >= -1e-08) {
      stats[2]++;
      b += score_vr;
      bb += score_vr * score_vr;
    } else {
      stats[3]++;
      // G_update (stencil.cpp:244-307): side order S, N, W, E
      int d = -1;
      if (std::fabs(o.y - st.params[1]) < 1e-8) d = South;
      else if (std::fabs(o.y - st.params[3]) < 1e-8) d = North;
      else if (std::fabs(o.x - st.params[0]) < 1e-8) d = West;
      else if (std::fabs(o.x - st.params[2]) < 1e-8) d = East;
      if (d < 0) { status = 1; continue; }  // the reference blocks on getchar() here
      SideData& s = sd[d];
      for (int i = 0; i < s.n; i++) {
        double H = 0.0;
        for (int j = 0; j < s.n; j++)
          H += s.ipsi[(size_t)j * s.n + i] *
               rbf<M>(st.pos[d][j][0], st.pos[d][j][1], o.x, o.y, s.c);
        s.G[i] += -H * o.Y;
        s.GG[i] += (H * o.Y) * (H * o.Y);
      }
      b += o.Z + o.xi;
      bb += (o.Z + o.xi) * (o.Z + o.xi);
    }
  }
  // G_return_withrep (stencil.cpp:343-406): sorted union; sides written in
  // N, S, E, W order, a later side overwriting (reference) or adding.
  const double norm = 1.0 / (N * 1.0);
  std::map<int, double> Gm, GGm;
  for (int d = 0; d < 4; d++)
    for (int v : st.index[d]) { Gm[v] = 0.0; GGm[v] = 0.0; }
  for (int d = 0; d < 4; d++)
    for (int i = 0; i < sd[d].n; i++) {
      const int v = st.index[d][i];
      if (prm->dup_sum) {
        Gm[v] += sd[d].G[i] * norm;
        GGm[v] += sd[d].GG[i] * norm;
      } else {
        Gm[v] = sd[d].G[i] * norm;
        GGm[v] = sd[d].GG[i] * norm;
      }
    }
  for (const auto& kv : Gm) {
    gj.push_back(kv.first);
    g.push_back(kv.second);
    gvar.push_back(GGm[kv.first] - kv.second * kv.second);
  }
  *B = b / N;
  *BB = bb / N;
  if (diag) {
    // the diagnostic sums of Reduce_Analytic (EMFKACSolver.hpp:542-558), paths
    // in order, xi and xi^2 in their own slots (the reference's enum gives
    // them one, :22-25) and tau = steps x h (the reference's clock starts at
    // +infinity, :145, and counts down, FKACIntegrator.hpp:56)
    for (int q = 0; q < ORC_DIAG_N; q++) diag[q] = 0.0;
    for (int n = 0; n < N; n++) {
      const PathOut& o = paths[n];
      const double phl = o.Z + o.Y * pb.g(o.x, o.y);
      const double phs = o.sZ + o.sY * pb.g(o.sx, o.sy);
      const double xl = o.xi, xs = o.sxi;
      const double sl = (double)o.steps_l, ss = sl + (double)o.steps_s;
      diag[0] += phl;
      diag[8] += phs;
      diag[1] += phl * phl;
      diag[9] += phs * phs;
      diag[2] += xl;
      diag[10] += xs;
      diag[3] += xl * xl;
      diag[11] += xs * xs;
      diag[4] += phl + xl;
      diag[12] += phs + xs;
      diag[5] += (phl + xl) * (phl + xl);
      diag[13] += (phs + xs) * (phs + xs);
      diag[6] += xl * phl;
      diag[14] += xs * phs;
      diag[16] += 2.0 * ss;  // RNGCalls: 2 normals per step, both legs
      diag[7] += sl * h;
      diag[15] += ss * h;
      diag[17] += 1.0;
    }
  }
  if (paths_out) paths_out->swap(paths);
  return status;
}

}  // namespace
}  // namespace orc

using namespace orc;

extern "C" {

void* orc_layout_new(double swx, double swy, double nex, double ney, int nsub, int nnode) {
  if (nsub < 2 || nnode < 3) return nullptr;
  Layout* L = new Layout();
  build_layout(*L, swx, swy, nex, ney, nsub, nnode);
  return L;
}
void orc_layout_free(void* L) { delete (Layout*)L; }
int orc_layout_nknots(const void* L) { return ((const Layout*)L)->nNodes; }
int orc_layout_nwork(const void* L) { return (int)((const Layout*)L)->work_index.size(); }
void orc_layout_work(const void* Lv, int* idx, double* x, double* y) {
  const Layout* L = (const Layout*)Lv;
  for (size_t i = 0; i < L->work_index.size(); i++) {
    idx[i] = L->work_index[i];
    x[i] = L->work_pos[i][0];
    y[i] = L->work_pos[i][1];
  }
}
int orc_layout_ninterfaces(const void* L) { return (int)((const Layout*)L)->interfaces.size(); }
int orc_layout_interface(const void* Lv, int i, int* label, int* idx, double* x, double* y) {
  const Interface& it = ((const Layout*)Lv)->interfaces[i];
  label[0] = it.label[0];
  label[1] = it.label[1];
  for (size_t k = 0; k < it.index.size(); k++) {
    if (idx) idx[k] = it.index[k];
    if (x) x[k] = it.position[k][0];
    if (y) y[k] = it.position[k][1];
  }
  return (int)it.index.size();
}
int orc_stencil(const void* Lv, int knot, double* params, int* kinds, int* sizes, int* idx,
                double* x, double* y, int maxn) {
  Stencil st = compute_stencil(*(const Layout*)Lv, knot);
  for (int i = 0; i < 4; i++) params[i] = st.params[i];
  for (int d = 0; d < 4; d++) {
    kinds[d] = st.kind[d];
    sizes[d] = (int)st.index[d].size();
    if (sizes[d] > maxn) return -1;
    for (int i = 0; i < sizes[d]; i++) {
      idx[d * maxn + i] = st.index[d][i];
      x[d * maxn + i] = st.pos[d][i][0];
      y[d * maxn + i] = st.pos[d][i][1];
    }
  }
  return 0;
}
int orc_ipsi(int n, const double* x, const double* y, double c, double* ipsi, double* cond) {
  return orc_ipsi_ex(n, x, y, c, 0, ipsi, cond);
}
int orc_ipsi_ex(int n, const double* x, const double* y, double c, int portable, double* ipsi,
                double* cond) {
  std::vector<double> psi, inv;
  if (portable) build_psi<PortMath>(n, x, y, c, psi);
  else build_psi<LibmMath>(n, x, y, c, psi);
  const int rank = fullpiv_inverse(n, psi, inv);
  double a = 0.0, b = 0.0;
  for (size_t i = 0; i < psi.size(); i++) { a += psi[i] * psi[i]; b += inv[i] * inv[i]; }
  if (cond) *cond = std::sqrt(a) * std::sqrt(b);
  if (ipsi) std::memcpy(ipsi, inv.data(), sizeof(double) * inv.size());
  return rank;
}

static int knot_dispatch(const void* Lv, const orc_problem* P, const orc_params* prm, int knot,
                         double x0, double y0, const double* ipsi_in, std::vector<int>& gj,
                         std::vector<double>& g, std::vector<double>& gv, double* B, double* BB,
                         int64_t* stats, std::vector<PathOut>* po, double* diag = nullptr) {
  const Layout& L = *(const Layout*)Lv;
  if (prm->portable) {
    if (P->kind == ORC_MONEGROS) return 2;  // libm-only problem
    return knot_impl<PortMath>(L, P, prm, knot, x0, y0, ipsi_in, gj, g, gv, B, BB, stats, po, diag);
  }
  return knot_impl<LibmMath>(L, P, prm, knot, x0, y0, ipsi_in, gj, g, gv, B, BB, stats, po, diag);
}

int orc_knot(const void* Lv, const orc_problem* P, const orc_params* prm, int knot, double x0,
             double y0, const double* ipsi_in, int* gj, double* g, double* gvar, int maxnnz,
             int* nnz, double* B, double* BB, int64_t* stats) {
  std::vector<int> vj;
  std::vector<double> vg, vv;
  int64_t st[4];
  const int s = knot_dispatch(Lv, P, prm, knot, x0, y0, ipsi_in, vj, vg, vv, B, BB, st, nullptr);
  if ((int)vj.size() > maxnnz) return -1;
  for (size_t i = 0; i < vj.size(); i++) { gj[i] = vj[i]; g[i] = vg[i]; gvar[i] = vv[i]; }
  *nnz = (int)vj.size();
  if (stats) for (int q = 0; q < 4; q++) stats[q] = st[q];
  return s;
}

int orc_knot_paths(const void* Lv, const orc_problem* P, const orc_params* prm, int knot,
                   double x0, double y0, double* xl, double* yl, double* Yl, double* Zl,
                   double* xil, int32_t* steps_l, int32_t* steps_s) {
  std::vector<int> vj;
  std::vector<double> vg, vv;
  int64_t st[4];
  double B, BB;
  std::vector<PathOut> po;
  const int s = knot_dispatch(Lv, P, prm, knot, x0, y0, nullptr, vj, vg, vv, &B, &BB, st, &po);
  for (size_t n = 0; n < po.size(); n++) {
    xl[n] = po[n].x; yl[n] = po[n].y; Yl[n] = po[n].Y; Zl[n] = po[n].Z; xil[n] = po[n].xi;
    steps_l[n] = po[n].steps_l; steps_s[n] = po[n].steps_s;
  }
  return s;
}

int orc_run(const void* Lv, const orc_problem* P, const orc_params* prm, const int* knots,
            const double* x0, const double* y0, int nk, int* row_ptr, int* gj, double* g,
            double* gvar, int64_t maxnnz, double* B, double* BB, int64_t* stats) {
  int status = 0;
  int64_t pos = 0;
  for (int q = 0; q < 4; q++) stats[q] = 0;
  row_ptr[0] = 0;
  std::vector<int> vj;
  std::vector<double> vg, vv;
  for (int k = 0; k < nk; k++) {
    int64_t st[4];
    const int s = knot_dispatch(Lv, P, prm, knots[k], x0[k], y0[k], nullptr, vj, vg, vv, &B[k],
                                &BB[k], st, nullptr);
    if (s) status = s;
    if (pos + (int64_t)vj.size() > maxnnz) return -1;
    for (size_t i = 0; i < vj.size(); i++, pos++) { gj[pos] = vj[i]; g[pos] = vg[i]; gvar[pos] = vv[i]; }
    row_ptr[k + 1] = (int)pos;
    for (int q = 0; q < 4; q++) stats[q] += st[q];
  }
  return status;
}

int orc_run_diag(const void* Lv, const orc_problem* P, const orc_params* prm, const int* knots,
                 const double* x0, const double* y0, int nk, double* sums) {
  int status = 0;
  std::vector<int> vj;
  std::vector<double> vg, vv;
  for (int k = 0; k < nk; k++) {
    int64_t st[4];
    double B, BB;
    double* d = sums + (size_t)k * ORC_DIAG_N;
    for (int q = 0; q < ORC_DIAG_N; q++) d[q] = 0.0;
    const int s = knot_dispatch(Lv, P, prm, knots[k], x0[k], y0[k], nullptr, vj, vg, vv, &B, &BB, st, nullptr, d);
    if (s) status = s;
  }
  return status;
}

int orc_bicgstab(int K, int64_t nnz, const int* ri, const int* ci, const double* v,
                 const double* bvec, double* x, int maxit, double tol, int* iters, double* err) {
  // setFromTriplets (duplicates summed) + identity, as CSR
  std::vector<std::map<int, double>> rows(K);
  for (int i = 0; i < K; i++) rows[i][i] = 1.0;
  for (int64_t e = 0; e < nnz; e++) rows[ri[e]][ci[e]] += v[e];
  std::vector<int> rp(K + 1, 0), cj;
  std::vector<double> av;
  for (int i = 0; i < K; i++) {
    for (const auto& kv : rows[i]) { cj.push_back(kv.first); av.push_back(kv.second); }
    rp[i + 1] = (int)cj.size();
  }
  auto spmv = [&](const std::vector<double>& in, std::vector<double>& out) {
    for (int i = 0; i < K; i++) {
      double s = 0.0;
      for (int e = rp[i]; e < rp[i + 1]; e++) s += av[e] * in[cj[e]];
      out[i] = s;
    }
  };
  auto dot = [&](const std::vector<double>& a, const std::vector<double>& b) {
    double s = 0.0;
    for (int i = 0; i < K; i++) s += a[i] * b[i];
    return s;
  };
  std::vector<double> inv(K, 1.0);
  for (int i = 0; i < K; i++)
    for (int e = rp[i]; e < rp[i + 1]; e++)
      if (cj[e] == i && av[e] != 0.0) inv[i] = 1.0 / av[e];
  std::vector<double> b(bvec, bvec + K), xv(K, 0.0), r(K), r0, p(K, 0.0), v_(K, 0.0), y(K),
      s(K), z(K), t(K), tmp(K);
  // Eigen-style BiCGSTAB (van der Vorst), Jacobi preconditioner
  spmv(xv, tmp);
  for (int i = 0; i < K; i++) r[i] = b[i] - tmp[i];
  r0 = r;
  double r0_sq = dot(r0, r0), rhs_sq = dot(b, b);
  if (rhs_sq == 0.0) {
    for (int i = 0; i < K; i++) x[i] = 0.0;
    *iters = 0; *err = 0.0;
    return 0;
  }
  double rho = 1.0, alpha = 1.0, w = 1.0;
  const double tol2 = tol * tol * rhs_sq;
  const double eps2 = std::numeric_limits<double>::epsilon() * std::numeric_limits<double>::epsilon();
  int i = 0, restarts = 0;
  while (dot(r, r) > tol2 && i < maxit) {
    const double rho_old = rho;
    rho = dot(r0, r);
    if (std::fabs(rho) < eps2 * r0_sq) {
      spmv(xv, tmp);
      for (int q = 0; q < K; q++) r[q] = b[q] - tmp[q];
      r0 = r;
      rho = r0_sq = dot(r, r);
      if (restarts++ == 0) i = 0;
    }
    const double beta = (rho / rho_old) * (alpha / w);
    for (int q = 0; q < K; q++) p[q] = r[q] + beta * (p[q] - w * v_[q]);
    for (int q = 0; q < K; q++) y[q] = inv[q] * p[q];
    spmv(y, v_);
    alpha = rho / dot(r0, v_);
    for (int q = 0; q < K; q++) s[q] = r[q] - alpha * v_[q];
    for (int q = 0; q < K; q++) z[q] = inv[q] * s[q];
    spmv(z, t);
    const double tt = dot(t, t);
    w = (tt > 0.0) ? dot(t, s) / tt : 0.0;
    for (int q = 0; q < K; q++) xv[q] += alpha * y[q] + w * z[q];
    for (int q = 0; q < K; q++) r[q] = s[q] - w * t[q];
    ++i;
  }
  for (int q = 0; q < K; q++) x[q] = xv[q];
  *iters = i;
  *err = std::sqrt(dot(r, r) / rhs_sq);
  return 0;
}

void orc_set_lut(const float* coef, const float* g, int nx, int ny, const double* bounds) {
  g_lut.coef.assign(coef, coef + (size_t)8 * nx * ny);
  g_lut.g.assign(g, g + (size_t)nx * ny);
  g_lut.nx = nx;
  g_lut.ny = ny;
  g_lut.x0 = bounds[0];
  g_lut.y0 = bounds[1];
  g_lut.inv_dx = 1.0 / ((bounds[2] - bounds[0]) / (nx - 1));
  g_lut.inv_dy = 1.0 / ((bounds[3] - bounds[1]) / (ny - 1));
}

double orc_problem_u(const orc_problem* P, double x, double y) {
  return Problem<LibmMath>{P}.u(x, y);
}

}  // extern "C"
