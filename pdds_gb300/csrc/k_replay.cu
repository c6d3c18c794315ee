// REPLAY_FP64 mode: bit-exact replay of the CPU restatement of the reference.
//
// Compiled with -fmad=false so no multiply-add is contracted, and every
// elementary function comes from pdds_portable.h, so each operation below
// rounds exactly as the host restatement does.  The path phase follows
//   Step (control variate)   Integrators/FKACIntegrator.hpp:46-57
//   Inside (Gobet shift)     Integrators/FKACIntegrator.hpp:168-222
//   Simulate_OMP             Solvers/EMFKACSolver.hpp:138-213 (linear + sublinear legs)
// one thread per path.  The reduction keeps the reference's serial order:
//   Reduce_Analytic          Solvers/EMFKACSolver.hpp:514-575 (paths in order)
//   G_update                 Meshes/stencil.cpp:244-307 (H_i over j in order)
//   G_return_withrep         Meshes/stencil.cpp:343-406 (sides N,S,E,W)
// with one thread per (knot, side, side knot) walking the paths in order.
#include "dev_common.cuh"
#include "kernels.h"

namespace pdds {

namespace {

constexpr int DIR_N_ = 0, DIR_S_ = 1, DIR_E_ = 2, DIR_W_ = 3;

template <int KIND>
__device__ void coef_port(const ProblemDev& P, double x, double y, Coef<double>& k) {
  const double PI = pm::PI;
  if (KIND == PK_LUT) {
    double v[8];
    lut_sample<double, 8>(P.lut, x, y, v);
    k.s00 = v[0]; k.s01 = 0.0; k.s10 = 0.0; k.s11 = v[1];
    k.b0 = v[2]; k.b1 = v[3]; k.c = v[4]; k.f = v[5]; k.g0 = v[6]; k.g1 = v[7];
  } else if (KIND == PK_POISSON_SINCOS) {
    double sx, cx, sy, cy;
    pm::sincos(PI * x, &sx, &cx);
    pm::sincos(PI * y, &sy, &cy);
    k.s00 = 1.4142135623730951; k.s01 = 0.0; k.s10 = 0.0; k.s11 = 1.4142135623730951;
    k.b0 = 0.0; k.b1 = 0.0; k.c = 0.0;
    k.f = 19.739208802178716 * (sx * cy);
    k.g0 = PI * (cx * cy) + y;
    k.g1 = x - PI * (sx * sy);
  } else if (KIND == PK_HELMHOLTZ) {
    const double a = P.p[0], b = P.p[1], c = P.p[2];
    double sa, ca, sb, cb;
    pm::sincos(a * x, &sa, &ca);
    pm::sincos(b * y, &sb, &cb);
    k.s00 = 1.4142135623730951; k.s01 = 0.0; k.s10 = 0.0; k.s11 = 1.4142135623730951;
    k.b0 = 0.0; k.b1 = 0.0; k.c = c;
    k.f = ((a * a + b * b) - c) * (sa * cb);
    k.g0 = a * (ca * cb);
    k.g1 = -(b * (sa * sb));
  } else {  // PK_VARCOEF (the Monegros problem has no portable form)
    const double s1 = 1.0 + 0.5 * (x * x), s2 = 1.0 + 0.5 * (y * y);
    double sn, cs;
    pm::sincos(2.0 * y, &sn, &cs);
    const double ex = pm::exp(x);
    const double ux = ex * cs, uy = -2.0 * (ex * sn), uxx = ux, uyy = -4.0 * ux;
    const double c = -(1.0 + x * x + y * y);
    const double u = ux + 1.0;
    k.s00 = s1; k.s01 = 0.0; k.s10 = 0.0; k.s11 = s2;
    k.b0 = y; k.b1 = -x; k.c = c;
    k.f = -(0.5 * (s1 * s1 * uxx + s2 * s2 * uyy) + (y * ux - x * uy) + c * u);
    k.g0 = ux;
    k.g1 = uy;
  }
  if (!P.use_cv) { k.g0 = 0.0; k.g1 = 0.0; }
}

template <int KIND>
__device__ double u_port(const ProblemDev& P, double x, double y) {
  if (KIND == PK_LUT) {
    return lut_sample_g<double>(P.lut, x, y);
  } else if (KIND == PK_POISSON_SINCOS) {
    double sx, cx, sy, cy;
    pm::sincos(pm::PI * x, &sx, &cx);
    pm::sincos(pm::PI * y, &sy, &cy);
    return sx * cy + x * y;
  } else if (KIND == PK_HELMHOLTZ) {
    double sa, ca, sb, cb;
    pm::sincos(P.p[0] * x, &sa, &ca);
    pm::sincos(P.p[1] * y, &sb, &cb);
    return sa * cb;
  } else {
    double s2, c2;
    pm::sincos(2.0 * y, &s2, &c2);
    return pm::exp(x) * c2 + 1.0;
  }
}

__device__ double rbf_port(double ax, double ay, double bx, double by, double c) {
  const double d0 = ax - bx, d1 = ay - by;
  const double nrm = ::sqrt(d0 * d0 + d1 * d1);
  return pm::exp(-(nrm * nrm) / (c * c));
}

template <int KIND>
struct PathState {
  const ProblemDev* P;
  const double* sp;
  double X0, X1, Y, Z, xi, E0, E1;
  double h, sqrth;
  uint64_t seed;
  uint32_t inst, knot, path, step;
  u32x4 blk;

  __device__ void one_step() {
    Coef<double> k;
    coef_port<KIND>(*P, X0, X1, k);
    if ((step & 1u) == 0) blk = path_block(seed, inst, knot, path, step >> 1);
    double z0, z1;
    if ((step & 1u) == 0) box_muller_portable(blk.v[0], blk.v[1], &z0, &z1);
    else box_muller_portable(blk.v[2], blk.v[3], &z0, &z1);
    step++;
    const double i0 = sqrth * z0, i1 = sqrth * z1;
    const double v0 = (-k.s00) * k.g0 + (-k.s10) * k.g1;
    const double v1 = (-k.s01) * k.g0 + (-k.s11) * k.g1;
    xi += Y * (v0 * i0 + v1 * i1);
    Z += k.f * Y * h;
    Y += k.c * Y * h;
    const double t0 = k.b0 * h + (k.s00 * i0 + k.s01 * i1);
    const double t1 = k.b1 * h + (k.s10 * i0 + k.s11 * i1);
    X0 += t0;
    X1 += t1;
  }
  __device__ bool inside(double gobet) {
    double Nx, Ny;
    int onmask;
    const double d = rect2d<double>(sp, X0, X1, E0, E1, Nx, Ny, onmask);
    Coef<double> ks;
    coef_port<KIND>(*P, X0, X1, ks);
    const double w0 = Nx * ks.s00 + Ny * ks.s10;
    const double w1 = Nx * ks.s01 + Ny * ks.s11;
    return d < gobet * ::sqrt(w0 * w0 + w1 * w1) * sqrth;
  }
};

template <int KIND>
__global__ void k_replay_paths(const ReplayArgs a) {
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= (int64_t)a.n_mc * a.N) return;
  const int m = (int)(gid / a.N), n = (int)(gid % a.N);
  const DevLayout& L = a.L;
  const int knot = a.mc_knots[m];
  const int st = L.knot_stencil[knot];
  const double* sp = L.st_rect + 4 * st;
  PathState<KIND> ps;
  ps.P = &a.P;
  ps.sp = sp;
  ps.X0 = L.kx[knot];
  ps.X1 = L.ky[knot];
  ps.Y = 1.0; ps.Z = 0.0; ps.xi = 0.0; ps.E0 = ps.X0; ps.E1 = ps.X1;
  ps.h = a.h;
  ps.sqrth = a.sqrth;
  if (a.adaptive_h) {
    Coef<double> k0;
    coef_port<KIND>(a.P, ps.X0, ps.X1, k0);
    ps.h = adaptive_step<double>(sp, ps.X0, ps.X1, a.h, k0);
    ps.sqrth = ::sqrt(ps.h);
  }
  ps.seed = a.seed;
  ps.inst = a.instance;
  ps.knot = knot_word(a.L, knot);
  ps.path = (uint32_t)n;
  ps.step = 0;
  ps.blk.v[0] = ps.blk.v[1] = ps.blk.v[2] = ps.blk.v[3] = 0;
  long long nl = 0, ns = 0;
  bool capped = false;
  do {
    ps.one_step();
    if (++nl > a.max_steps) { capped = true; break; }
  } while (ps.inside(-0.5826));
  const double ex = ps.E0, ey = ps.E1, eY = ps.Y, eZ = ps.Z, exi = ps.xi;
  if (a.sublinear && !capped) {
    do {
      ps.one_step();
      if (++ns > a.max_steps) { capped = true; break; }
    } while (ps.inside(0.0));
  }
  // exit classification of Reduce_Analytic (:559) and G_update (stencil.cpp:246-301)
  int side;
  {
    double E0, E1, Nx, Ny;
    int onm;
    const double gd = rect2d<double>(L.dom, ex, ey, E0, E1, Nx, Ny, onm);
    if (isnan(ps.X0) || isnan(ps.X1)) side = -2;  // a position that is not a number lies on no side
    else if (gd >= -1e-08) side = -1;
    else if (fabs(ey - sp[1]) < 1e-8) side = DIR_S_;
    else if (fabs(ey - sp[3]) < 1e-8) side = DIR_N_;
    else if (fabs(ex - sp[0]) < 1e-8) side = DIR_W_;
    else if (fabs(ex - sp[2]) < 1e-8) side = DIR_E_;
    else side = -2;
  }
  const int64_t o = gid;
  a.ex[o] = ex; a.ey[o] = ey; a.eY[o] = eY; a.eZ[o] = eZ; a.exi[o] = exi;
  if (a.diag) {  // the sublinear leg's end (the linear one's when it did not run)
    a.sx[o] = ps.E0; a.sy[o] = ps.E1; a.sY[o] = ps.Y; a.sZ[o] = ps.Z; a.sxi[o] = ps.xi;
    if (n == 0) a.knot_h[m] = ps.h;
  }
  a.esteps_l[o] = (int)nl;
  a.esteps_s[o] = (int)ns;
  a.eside[o] = capped ? -4 : side;
  if (capped) atomicOr(a.err_flags, ERR_FLAG_STEP_LIMIT);
  if (side == -2) atomicOr(a.err_flags, ERR_FLAG_EXIT_SIDE);
}

// B and BB of one knot: Reduce_Analytic's serial loop over the paths.
template <int KIND>
__global__ void k_replay_b(const ReplayArgs a) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= a.n_mc) return;
  const int knot = a.mc_knots[m];
  double b = 0.0, bb = 0.0;
  for (int n = 0; n < a.N; n++) {
    const int64_t o = (int64_t)m * a.N + n;
    const int side = a.eside[o];
    const double Z = a.eZ[o], Y = a.eY[o], xi = a.exi[o];
    if (side == -1) {
      const double score = Z + Y * u_port<KIND>(a.P, a.ex[o], a.ey[o]);
      const double score_vr = score + xi;
      b += score_vr;
      bb += score_vr * score_vr;
    } else if (side >= 0) {
      b += Z + xi;
      bb += (Z + xi) * (Z + xi);
    }
  }
  a.B[knot] = b / a.N;
  a.BB[knot] = bb / a.N;
  if (a.diag) {
    // the diagnostic sums of Reduce_Analytic (Solvers/EMFKACSolver.hpp:542-558),
    // paths in order; tau = steps x h (elapsed time)
    double sm[PDDS_DIAG_N];
    for (int q = 0; q < PDDS_DIAG_N; q++) sm[q] = 0.0;
    const double hk = a.knot_h[m];
    for (int n = 0; n < a.N; n++) {
      const int64_t o = (int64_t)m * a.N + n;
      const double phl = a.eZ[o] + a.eY[o] * u_port<KIND>(a.P, a.ex[o], a.ey[o]);
      const double phs = a.sZ[o] + a.sY[o] * u_port<KIND>(a.P, a.sx[o], a.sy[o]);
      const double xl = a.exi[o], xs = a.sxi[o];
      const double sl = (double)a.esteps_l[o], ss = sl + (double)a.esteps_s[o];
      sm[PDDS_DIAG_SCORE] += phl;
      sm[PDDS_DIAG_SUB + PDDS_DIAG_SCORE] += phs;
      sm[PDDS_DIAG_SCORE2] += phl * phl;
      sm[PDDS_DIAG_SUB + PDDS_DIAG_SCORE2] += phs * phs;
      sm[PDDS_DIAG_XI] += xl;
      sm[PDDS_DIAG_SUB + PDDS_DIAG_XI] += xs;
      sm[PDDS_DIAG_XI2] += xl * xl;
      sm[PDDS_DIAG_SUB + PDDS_DIAG_XI2] += xs * xs;
      sm[PDDS_DIAG_SCORE_VR] += phl + xl;
      sm[PDDS_DIAG_SUB + PDDS_DIAG_SCORE_VR] += phs + xs;
      sm[PDDS_DIAG_SCORE_VR2] += (phl + xl) * (phl + xl);
      sm[PDDS_DIAG_SUB + PDDS_DIAG_SCORE_VR2] += (phs + xs) * (phs + xs);
      sm[PDDS_DIAG_XI_SCORE] += xl * phl;
      sm[PDDS_DIAG_SUB + PDDS_DIAG_XI_SCORE] += xs * phs;
      sm[PDDS_DIAG_RNG] += 2.0 * ss;
      sm[PDDS_DIAG_TAU] += sl * hk;
      sm[PDDS_DIAG_SUB + PDDS_DIAG_TAU] += ss * hk;
      sm[PDDS_DIAG_PATHS] += 1.0;
    }
    for (int q = 0; q < PDDS_DIAG_N; q++) a.diag[(int64_t)knot * PDDS_DIAG_N + q] = sm[q];
  }
}

// G_update accumulation for one (knot, side, side knot i), paths in order.
__global__ void k_replay_g(const ReplayArgs a, const int* task_m, const int* task_d,
                           const int* task_i, int ntask, double* Gside, double* GGside,
                           const int64_t* task_out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntask) return;
  const int m = task_m[t], d = task_d[t], i = task_i[t];
  const DevLayout& L = a.L;
  const int knot = a.mc_knots[m];
  const int st = L.knot_stencil[knot];
  const int sd = L.st_side[4 * st + d];
  const int n = L.sd_n[sd];
  const double c = L.sd_c[sd];
  const double* px = L.side_px + L.sd_knot_off[sd];
  const double* py = L.side_py + L.sd_knot_off[sd];
  const double* ip;
  if (a.knot_ipsi_off) ip = a.ipsi_knot + a.knot_ipsi_off[4 * m + d];
  else ip = L.ipsi + L.sh_ipsi_off[L.sd_shape[sd]];
  double G = 0.0, GG = 0.0;
  for (int p = 0; p < a.N; p++) {
    const int64_t o = (int64_t)m * a.N + p;
    if (a.eside[o] != d) continue;
    const double X0 = a.ex[o], X1 = a.ey[o], Y = a.eY[o];
    double H = 0.0;
    for (int j = 0; j < n; j++) H += ip[(int64_t)j * n + i] * rbf_port(px[j], py[j], X0, X1, c);
    G += -H * Y;
    GG += (H * Y) * (H * Y);
  }
  Gside[task_out[t]] = G;
  GGside[task_out[t]] = GG;
}

// G_return_withrep for one knot: sides N, S, E, W in order, G = G_side * (1/N).
__global__ void k_replay_row(const ReplayArgs a, const int64_t* knot_task_off, const double* Gside,
                             const double* GGside) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= a.n_mc) return;
  const DevLayout& L = a.L;
  const int knot = a.mc_knots[m];
  const int st = L.knot_stencil[knot];
  const int64_t r0 = L.row_ptr[knot], r1 = L.row_ptr[knot + 1];
  for (int64_t e = r0; e < r1; e++) { a.G[e] = 0.0; a.GG[e] = 0.0; }
  const double norm = 1.0 / (a.N * 1.0);
  int64_t mo = L.st_map_off[st];
  int64_t to = knot_task_off[m];
  for (int d = 0; d < 4; d++) {
    const int sd = L.st_side[4 * st + d];
    if (sd < 0) continue;
    const int n = L.sd_n[sd];
    for (int i = 0; i < n; i++, mo++, to++) {
      const int64_t e = r0 + L.map_pos[mo];
      if (!idx_ok(e - r0, r1 - r0, a.err_flags)) continue;
      if (a.dup_sum) {
        a.G[e] += Gside[to] * norm;
        a.GG[e] += GGside[to] * norm;
      } else {
        a.G[e] = Gside[to] * norm;
        a.GG[e] = GGside[to] * norm;
      }
    }
  }
  for (int64_t e = r0; e < r1; e++) a.GG[e] = a.GG[e] - a.G[e] * a.G[e];
}

}  // namespace

cudaError_t launch_replay_paths(const ReplayArgs& a, int kind, cudaStream_t s) {
  const int64_t total = (int64_t)a.n_mc * a.N;
  const int th = 128;
  const unsigned grid = (unsigned)((total + th - 1) / th);
  if (total == 0) return cudaSuccess;
  switch (kind) {
    case PK_POISSON_SINCOS: k_replay_paths<PK_POISSON_SINCOS><<<grid, th, 0, s>>>(a); break;
    case PK_HELMHOLTZ: k_replay_paths<PK_HELMHOLTZ><<<grid, th, 0, s>>>(a); break;
    case PK_VARCOEF: k_replay_paths<PK_VARCOEF><<<grid, th, 0, s>>>(a); break;
    case PK_LUT: k_replay_paths<PK_LUT><<<grid, th, 0, s>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_replay_reduce(const ReplayArgs& a, int kind, const int* task_m, const int* task_d,
                                 const int* task_i, int ntask, const int64_t* task_out,
                                 const int64_t* knot_task_off, double* Gside, double* GGside,
                                 cudaStream_t s) {
  if (a.n_mc == 0) return cudaSuccess;
  const int gb = (a.n_mc + 127) / 128;
  switch (kind) {
    case PK_POISSON_SINCOS: k_replay_b<PK_POISSON_SINCOS><<<gb, 128, 0, s>>>(a); break;
    case PK_HELMHOLTZ: k_replay_b<PK_HELMHOLTZ><<<gb, 128, 0, s>>>(a); break;
    case PK_VARCOEF: k_replay_b<PK_VARCOEF><<<gb, 128, 0, s>>>(a); break;
    case PK_LUT: k_replay_b<PK_LUT><<<gb, 128, 0, s>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  if (ntask > 0)
    k_replay_g<<<(ntask + 63) / 64, 64, 0, s>>>(a, task_m, task_d, task_i, ntask, Gside, GGside, task_out);
  k_replay_row<<<gb, 128, 0, s>>>(a, knot_task_off, Gside, GGside);
  return cudaGetLastError();
}

}  // namespace pdds
