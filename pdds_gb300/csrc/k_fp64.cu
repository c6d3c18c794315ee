// FP64 mode: the plain double-precision GPU form of the estimator.
//
// Same persistent work-item structure as the MIXED kernel, but every path
// quantity is FP64 and each stencil exit adds its exact RBF vector
// Y * r_j(X), r_j = exp(-|p_j - X|^2 / c^2), into per-side FP64 sums S_j in
// shared memory.  At the end of the item G_i = -(1/N) sum_j ipsi(j,i) S_j.
// Exits are queued per warp (side, coordinate, weight) and the warp adds
// their RBF vectors one exit at a time with the side knots spread over the
// lanes, into its own copy of the sums (no atomics; the copies are added at
// the end of the item), so the n_s exponentials of an exit run at full width.
// By linearity this equals the reference's per-exit
// H_i = sum_j ipsi(j,i) RBF(p_j, X) accumulation (Meshes/stencil.cpp:244-307)
// with n_s instead of n_s^2 exponentials per exit.  It is the all-FP64 GPU
// oracle that MIXED results are compared with.
#include "dev_common.cuh"
#include "kernels.h"

namespace pdds {

namespace {

struct ItemSide64 {
  int n;
  int orient;
  int glob;
  int s_off;         // offset into the shared S arrays
  double origin;
  double inv_c2;
  int64_t t_off;     // shape's local knot coordinates
  int64_t ipsi_off;
  int64_t map_off;
  double R;          // arc radius (polar stencils): RBF distance = chord 2 R sin(dt / 2)
};

constexpr unsigned FULL = 0xffffffffu;

struct Lvl64 {
  double x, y, Y, Z, xi;
  double phi;  // Z + Y g(X_tau) at the exit (diagnostics)
  Coef<double> k;
  unsigned steps;
};

// Box-Muller in FP64: z0 = rho cos(2 pi u1), z1 = rho sin(2 pi u1).
__device__ __forceinline__ void normals_f64(uint32_t ua, uint32_t ub, double& z0, double& z1) {
  const double u0 = u01_fp64(ua), u1 = u01_fp64(ub);
  const double rho = ::sqrt(-2.0 * ::log(u0));
  double sn, cs;
  sincospi(2.0 * u1, &sn, &cs);
  z0 = rho * cs;
  z1 = rho * sn;
}

template <int KIND, bool RICH, int GEOM>
__global__ void __launch_bounds__(FP64_THREADS)
k_paths_fp64(const Fp64Args a) {
  // [warps][sum n] per-warp per-side RBF sums, then [sum n] local t
  extern __shared__ double Ssum[];
  __shared__ double s_qs[FP64_THREADS / 32][FP64_QCAP], s_qy[FP64_THREADS / 32][FP64_QCAP];
  __shared__ int s_qd[FP64_THREADS / 32][FP64_QCAP];
  __shared__ int s_qn[FP64_THREADS / 32];
  __shared__ ItemSide64 s_side[4];
  __shared__ double s_rect[4];
  __shared__ int s_item, s_knot, s_path_end, s_nall;
  __shared__ double s_h;
  __shared__ unsigned s_next_path;
  __shared__ double s_red[FP64_THREADS / 32][2];
  __shared__ double s_diag[PDDS_DIAG_N];
  __shared__ unsigned long long s_redi[FP64_THREADS / 32][3];
  const DevLayout& L = a.L;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  for (;;) {
    if (tid == 0) s_item = atomicAdd(a.item_counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= a.n_items) break;
    if (tid == 0) {
      const int k = a.mc_knots[item / a.chunks];
      const int chunk = item % a.chunks;
      s_knot = k;
      for (int q = 0; q < PDDS_DIAG_N; q++) s_diag[q] = 0.0;
      const int p0 = chunk * a.paths_per_chunk;
      s_path_end = min(a.N, p0 + a.paths_per_chunk);
      s_next_path = (unsigned)(p0 + FP64_THREADS);
      const int st = L.knot_stencil[k];
      for (int q = 0; q < 4; q++) s_rect[q] = L.st_rect[4 * st + q];
      s_h = a.h;
      if (a.adaptive_h) {
        Coef<double> kd;
        coef_f64<KIND>(a.P, L.kx[k], L.ky[k], kd);
        s_h = GEOM == 1 ? adaptive_step_polar(L.st_rect + 4 * st, L.kx[k], L.ky[k], a.h, kd)
                        : adaptive_step<double>(L.st_rect + 4 * st, L.kx[k], L.ky[k], a.h, kd);
      }
      int off = 0;
      int64_t moff = L.st_map_off[st];
      for (int d = 0; d < 4; d++) {
        const int sd = L.st_side[4 * st + d];
        ItemSide64 is;
        is.glob = L.st_glob[4 * st + d];
        is.map_off = moff;
        if (sd < 0) {
          is.n = 0; is.orient = 0; is.s_off = off; is.origin = 0.0; is.inv_c2 = 0.0;
          is.t_off = 0; is.ipsi_off = 0; is.R = 0.0;
        } else {
          const int sh = L.sd_shape[sd];
          is.n = L.sd_n[sd];
          is.orient = L.sd_orient[sd];
          is.s_off = off;
          is.origin = L.sd_origin[sd];
          is.R = L.sh_R ? L.sh_R[sh] : 0.0;
          if (GEOM == 1 && is.orient == 0) {  // arc: the side's angles in this stencil's turn
            const double tw = 6.283185307179586;
            is.origin += tw * nearbyint((L.st_rect[4 * st + 1] - is.origin) / tw);
          }
          const double c = L.sh_c[sh];
          is.inv_c2 = 1.0 / (c * c);
          is.t_off = L.sh_t_off[sh];
          is.ipsi_off = L.sh_ipsi_off[sh];
          off += is.n;
          moff += is.n;
        }
        s_side[d] = is;
      }
      s_nall = off;
    }
    __syncthreads();
    const int knot = s_knot, path_end = s_path_end, nall = s_nall;
    const double h = s_h, sqrth = ::sqrt(s_h);
    constexpr int NW = FP64_THREADS / 32;
    double* tloc = Ssum + NW * nall;
    double* Sw = Ssum + warp * nall;  // this warp's sums
    for (int i = tid; i < NW * nall; i += FP64_THREADS) Ssum[i] = 0.0;
    if (lane == 0) s_qn[warp] = 0;
    for (int d = 0; d < 4; d++)
      for (int i = tid; i < s_side[d].n; i += FP64_THREADS)
        tloc[s_side[d].s_off + i] = L.sh_t[s_side[d].t_off + i];
    __syncthreads();

    const double x0 = L.kx[knot], y0 = L.ky[knot];
    const double rect[4] = {s_rect[0], s_rect[1], s_rect[2], s_rect[3]};
    const double pa0 = GEOM == 1 ? ::cos(rect[1]) : 0.0, pa1 = GEOM == 1 ? ::sin(rect[1]) : 0.0;
    const double pb0 = GEOM == 1 ? ::cos(rect[3]) : 0.0, pb1 = GEOM == 1 ? ::sin(rect[3]) : 0.0;
    // PK_ROBIN: the reflecting stencil side (a global side in the Robin set
    // P.p[0], bits N 1, S 2, E 4, W 8), its line n . (x, y) = rc
    const int globmask = (s_side[0].glob ? 1 : 0) | (s_side[1].glob ? 2 : 0) | (s_side[2].glob ? 4 : 0) |
                         (s_side[3].glob ? 8 : 0);
    const int rmask = KIND == PK_ROBIN ? (globmask & (int)a.P.p[0]) : 0;
    double rn0 = 0.0, rn1 = 0.0, rc = 0.0;
    if (rmask & 1) { rn1 = 1.0; rc = rect[3]; }
    else if (rmask & 2) { rn1 = -1.0; rc = -rect[1]; }
    else if (rmask & 4) { rn0 = 1.0; rc = rect[2]; }
    else if (rmask & 8) { rn0 = -1.0; rc = -rect[0]; }
    Coef<double> k0;
    coef_f64<KIND>(a.P, x0, y0, k0);
    const int chunk = item % a.chunks;
    unsigned path = (unsigned)(chunk * a.paths_per_chunk + tid);
    bool active = (int)path < path_end;
    double b = 0.0, bb = 0.0;
    unsigned long long nsteps = 0, nglob = 0, nsten = 0;
    // exit on side d at side coordinate `along` (x or y on rectangles, angle
    // or radius on polar stencils), projection (Ex, Ey)
    auto exit_level = [&](Lvl64& s, double wgt, double Ex, double Ey, int d, bool glob,
                          double along) -> double {
      if (isnan(s.x) || isnan(s.y)) {
        // a position that is not a number lies on no side: reported, scores nothing
        atomicOr(a.err_flags, ERR_FLAG_EXIT_SIDE);
        return 0.0;
      }
      if (glob) {
        ++nglob;
        s.phi = s.Z + s.Y * u_f64<KIND>(a.P, Ex, Ey);
        return s.phi + s.xi;
      }
      if (a.diag) s.phi = s.Z + s.Y * u_f64<KIND>(a.P, Ex, Ey);
      ++nsten;
      if (d < 0) {
        atomicOr(a.err_flags, ERR_FLAG_EXIT_SIDE);
      } else {
        // queue the exit: < 32 left over + at most 2 exits per lane and
        // iteration fit in FP64_QCAP
        const int e = atomicAdd(&s_qn[warp], 1);
        if (idx_ok(e, FP64_QCAP, a.err_flags)) {
          s_qd[warp][e] = d;
          s_qs[warp][e] = along - s_side[d].origin;
          s_qy[warp][e] = wgt * s.Y;
        }
      }
      return s.Z + s.xi;
    };
    // Add the queued exits' RBF vectors to this warp's sums (warp-uniform
    // call; only when at least minq exits are queued).
    auto flush = [&](int minq) {
      __syncwarp();
      const int n = s_qn[warp];
      if (n < minq) return;
      for (int e = 0; e < min(n, FP64_QCAP); e++) {
        const ItemSide64& is = s_side[s_qd[warp][e]];
        const double sc = s_qs[warp][e], yw = s_qy[warp][e];
        for (int j = lane; j < is.n; j += 32) {
          const double dt0 = tloc[is.s_off + j] - sc;
          const double dt = is.R > 0.0 ? 2.0 * is.R * ::sin(0.5 * dt0) : dt0;
          Sw[is.s_off + j] += yw * ::exp(-(dt * dt) * is.inv_c2);
        }
      }
      __syncwarp();
      if (lane == 0) s_qn[warp] = 0;
      __syncwarp();
    };
    // ex: Exp(1) sample of the reflected step (PK_ROBIN), see k_mixed.cu
    auto step_level = [&](Lvl64& s, double i0, double i1, double hh, double sq, double wgt, double& val,
                          double ex) -> bool {
      const double v0 = -(s.k.s00 * s.k.g0 + s.k.s10 * s.k.g1);
      const double v1 = -(s.k.s01 * s.k.g0 + s.k.s11 * s.k.g1);
      s.xi += s.Y * (v0 * i0 + v1 * i1);
      s.Z += s.k.f * s.Y * hh;
      s.Y += s.k.c * s.Y * hh;
      if constexpr (KIND == PK_ROBIN) {
        const double d0 = s.k.s00 * i0, d1 = s.k.s11 * i1;
        double dL = 0.0;
        if (rmask) {
          const double dR = rn0 * s.x + rn1 * s.y - rc;
          const double U = rn0 * d0 + rn1 * d1;
          const double M = 0.5 * (U + ::sqrt(U * U + 4.0 * hh * ex));  // |sigma^T n|^2 = 2
          dL = ::fmax(0.0, M + dR);
          if (dL > 0.0) {  // exact in dL, as in k_mixed.cu
            double vphi, psi;
            robin_data<double>(s.x - dR * rn0, s.y - dR * rn1, rn0, rn1, vphi, psi);
            const double t = vphi * dL;
            const double em1 = ::expm1(t);
            s.Z += psi * s.Y * (t != 0.0 ? em1 / vphi : dL);
            s.Y += s.Y * em1;
          }
        }
        s.x += d0 - dL * rn0;
        s.y += d1 - dL * rn1;
      } else {
        s.x += s.k.b0 * hh + (s.k.s00 * i0 + s.k.s01 * i1);
        s.y += s.k.b1 * hh + (s.k.s10 * i0 + s.k.s11 * i1);
      }
      ++s.steps;
      coef_f64<KIND>(a.P, s.x, s.y, s.k);
      if constexpr (GEOM == 1) {
        // polar stencil, isotropic sigma: outside distances beyond the inner
        // arc (none at the centre), the outer arc and the two rays
        const double rho = ::sqrt(s.x * s.x + s.y * s.y);
        const double d_in = rect[0] > 0.0 ? rect[0] - rho : -1e300;
        const double d_out = rho - rect[2];
        const bool has_rays = rect[3] - rect[1] < 6.2;  // a full disk has one side, its arc
        const double d_a = has_rays ? pa1 * s.x - pa0 * s.y : -1e300;
        const double d_b = has_rays ? pb0 * s.y - pb1 * s.x : -1e300;
        int d = 1;
        double mx = d_in;
        if (d_out > mx) { mx = d_out; d = 0; }
        if (d_a > mx) { mx = d_a; d = 3; }
        if (d_b > mx) { mx = d_b; d = 2; }
        if (mx < -0.5826 * ::fabs(s.k.s00) * sq) {
          if (s.steps < (unsigned)a.max_steps) return false;
          atomicOr(a.err_flags, ERR_FLAG_STEP_LIMIT);
          val = 0.0;
          return true;
        }
        double along, Ex = 0.0, Ey = 0.0;
        if (d <= 1) {
          const double rel = ::atan2(pa0 * s.y - pa1 * s.x, pa0 * s.x + pa1 * s.y);
          along = rect[1] + (has_rays ? ::fmin(::fmax(rel, 0.0), rect[3] - rect[1])
                                      : (rel < 0.0 ? rel + 6.283185307179586 : rel));
          ::sincos(along, &Ey, &Ex);
          Ex *= rect[d == 0 ? 2 : 0];
          Ey *= rect[d == 0 ? 2 : 0];
        } else {
          const double t = d == 3 ? pa0 * s.x + pa1 * s.y : pb0 * s.x + pb1 * s.y;
          along = ::fmin(::fmax(t, rect[0]), rect[2]);
        }
        val = exit_level(s, wgt, Ex, Ey, d, d == 0 && s_side[0].glob, along);
        return true;
      } else if constexpr (KIND == PK_ROBIN) {
        // absorbing sides only; the exit side is the one with the largest
        // outside distance (ties S, N, W, E), the other coordinate clamped
        const double o0 = (rmask & 1) ? -1e300 : s.y - rect[3], o1 = (rmask & 2) ? -1e300 : rect[1] - s.y;
        const double o2 = (rmask & 4) ? -1e300 : s.x - rect[2], o3 = (rmask & 8) ? -1e300 : rect[0] - s.x;
        int d = 1;
        double mx = o1;
        if (o0 > mx) { mx = o0; d = 0; }
        if (o3 > mx) { mx = o3; d = 3; }
        if (o2 > mx) { mx = o2; d = 2; }
        if (mx < -0.5826 * 1.4142135623730951 * sq) {
          if (s.steps < (unsigned)a.max_steps) return false;
          atomicOr(a.err_flags, ERR_FLAG_STEP_LIMIT);
          val = 0.0;
          return true;
        }
        const double Ex = d == 3 ? rect[0] : (d == 2 ? rect[2] : ::fmin(::fmax(s.x, rect[0]), rect[2]));
        const double Ey = d == 1 ? rect[1] : (d == 0 ? rect[3] : ::fmin(::fmax(s.y, rect[1]), rect[3]));
        val = exit_level(s, wgt, Ex, Ey, d, s_side[d].glob != 0, s_side[d].orient == 0 ? Ex : Ey);
        return true;
      } else {
        double Ex, Ey, Nx, Ny;
        int onmask;
        const double dist = rect2d<double>(rect, s.x, s.y, Ex, Ey, Nx, Ny, onmask);
        const double w0 = Nx * s.k.s00 + Ny * s.k.s10, w1 = Nx * s.k.s01 + Ny * s.k.s11;
        const double thr = -0.5826 * ::sqrt(w0 * w0 + w1 * w1) * sq;
        if (dist < thr) {
          if (s.steps < (unsigned)a.max_steps) return false;
          atomicOr(a.err_flags, ERR_FLAG_STEP_LIMIT);
          val = 0.0;
          return true;
        }
        const int d = exit_side(onmask);
        const bool glob = ((onmask & 1) && s_side[0].glob) || ((onmask & 2) && s_side[1].glob) ||
                          ((onmask & 4) && s_side[2].glob) || ((onmask & 8) && s_side[3].glob);
        val = exit_level(s, wgt, Ex, Ey, d, glob, d >= 0 && s_side[d].orient == 0 ? Ex : Ey);
        return true;
      }
    };
    Lvl64 fine, coarse;
    auto reset = [&]() {
      fine.x = x0; fine.y = y0; fine.Y = 1.0; fine.Z = 0.0; fine.xi = 0.0; fine.phi = 0.0; fine.k = k0;
      fine.steps = 0;
      coarse = fine;
    };
    reset();
    bool fine_alive = active, coarse_alive = RICH && active;
    double val_f = 0.0, val_c = 0.0;
    unsigned m = 0;
    u32x4 blk;
    blk.v[0] = blk.v[1] = blk.v[2] = blk.v[3] = 0;
    while (__any_sync(FULL, active)) {
      if (active) {
        bool fin = false;  // the lane's path (pair) finished in this iteration
        if (RICH) {
          const unsigned mi = m++;
          blk = path_block(a.seed, a.instance, knot_word(a.L, knot), path, mi);
          double za0, za1, zb0, zb1;
          normals_f64(blk.v[0], blk.v[1], za0, za1);
          normals_f64(blk.v[2], blk.v[3], zb0, zb1);
          double x0e = 0.0, x1e = 0.0, x2e = 0.0;  // Exp(1) samples of reflected steps
          if (KIND == PK_ROBIN && rmask) {
            const u32x4 bx = path_block(a.seed, a.instance, knot_word(a.L, knot) | 0x80000000u, path, mi);
            x0e = -::log(u01_fp64(bx.v[0]));
            x1e = -::log(u01_fp64(bx.v[1]));
            x2e = -::log(u01_fp64(bx.v[2]));
          }
          const double hf = 0.5 * h, sqf = ::sqrt(hf);
          if (fine_alive) fine_alive = !step_level(fine, sqf * za0, sqf * za1, hf, sqf, 2.0, val_f, x0e);
          if (fine_alive) fine_alive = !step_level(fine, sqf * zb0, sqf * zb1, hf, sqf, 2.0, val_f, x1e);
          if (coarse_alive)
            coarse_alive =
                !step_level(coarse, sqf * (za0 + zb0), sqf * (za1 + zb1), h, sqrth, -1.0, val_c, x2e);
          if (!fine_alive && !coarse_alive) {
            const double v = 2.0 * val_f - val_c;
            b += v;
            bb += v * v;
            nsteps += fine.steps + coarse.steps;
            fin = true;
            if (a.diag)
              diag_add(s_diag, 2.0 * fine.phi - coarse.phi, 2.0 * fine.xi - coarse.xi, fine.steps * hf,
                       2.0 * fine.steps);
          }
        } else {
          if ((m & 1u) == 0) blk = path_block(a.seed, a.instance, knot_word(a.L, knot), path, m >> 1);
          double z0, z1;
          if (m & 1u) normals_f64(blk.v[2], blk.v[3], z0, z1);
          else normals_f64(blk.v[0], blk.v[1], z0, z1);
          double xe = 0.0;
          if (KIND == PK_ROBIN && rmask) {
            const u32x4 bx = path_block(a.seed, a.instance, knot_word(a.L, knot) | 0x80000000u, path, m >> 1);
            xe = -::log(u01_fp64(bx.v[m & 1u]));
          }
          ++m;
          if (step_level(fine, sqrth * z0, sqrth * z1, h, sqrth, 1.0, val_f, xe)) {
            b += val_f;
            bb += val_f * val_f;
            nsteps += fine.steps;
            fin = true;
            if (a.diag) diag_add(s_diag, fine.phi, fine.xi, fine.steps * h, 2.0 * fine.steps);
          }
        }
        if (fin) {
          path = atomicAdd(&s_next_path, 1u);
          if ((int)path >= path_end) {
            active = false;
          } else {
            reset();
            fine_alive = true;
            coarse_alive = RICH;
            m = 0;
          }
        }
      }
      flush(32);
    }
    flush(1);
    __syncthreads();
    // S_j: the warps' sums added in a fixed order, into warp 0's copy
    for (int i = tid; i < nall; i += FP64_THREADS) {
      double t = Ssum[i];
      for (int w = 1; w < NW; w++) t += Ssum[w * nall + i];
      Ssum[i] = t;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      b += __shfl_xor_sync(FULL, b, o);
      bb += __shfl_xor_sync(FULL, bb, o);
      nsteps += __shfl_xor_sync(FULL, nsteps, o);
      nglob += __shfl_xor_sync(FULL, nglob, o);
      nsten += __shfl_xor_sync(FULL, nsten, o);
    }
    if (lane == 0) {
      s_red[warp][0] = b;
      s_red[warp][1] = bb;
      s_redi[warp][0] = nsteps;
      s_redi[warp][1] = nglob;
      s_redi[warp][2] = nsten;
    }
    __syncthreads();
    if (tid == 0) {
      double tb = 0.0, tbb = 0.0;
      unsigned long long ts = 0, tg = 0, tt = 0;
      for (int w = 0; w < FP64_THREADS / 32; w++) {
        tb += s_red[w][0]; tbb += s_red[w][1];
        ts += s_redi[w][0]; tg += s_redi[w][1]; tt += s_redi[w][2];
      }
      atomicAdd(a.Bsum + knot, tb);
      atomicAdd(a.BBsum + knot, tbb);
      atomicAdd(a.stats + 0, ts);
      atomicAdd(a.stats + 2, tg);
      atomicAdd(a.stats + 3, tt);
    }
    if (a.diag) diag_flush(s_diag, a.diag + (int64_t)knot * PDDS_DIAG_N, tid);
    // G_i = -(1/N) sum_j ipsi(j,i) S_j
    const int64_t row0 = L.row_ptr[knot];
    for (int pr = tid; pr < nall; pr += FP64_THREADS) {
      int d = 0, i = pr;
      while (i >= s_side[d].n) { i -= s_side[d].n; ++d; }
      const ItemSide64& is = s_side[d];
      const int64_t m = is.map_off + i;
      if (!a.dup_sum && !L.map_owner[m]) continue;
      const double* ip = L.ipsi + is.ipsi_off + i;
      double acc = 0.0;
      for (int j = 0; j < is.n; j++) acc += ip[(int64_t)j * is.n] * Ssum[is.s_off + j];
      if (idx_ok(L.map_pos[m], L.row_ptr[knot + 1] - row0, a.err_flags))
        atomicAdd(a.G + row0 + L.map_pos[m], -acc * a.inv_N);
    }
    __syncthreads();
  }
}

}  // namespace

template <bool RICH>
static cudaError_t launch_fp64_t(const Fp64Args& a, int kind, int grid, size_t smem, cudaStream_t s) {
#define PDDS_FP64_CASE(KK, GG)                                                                           \
  case KK:                                                                                               \
    cudaFuncSetAttribute(k_paths_fp64<KK, RICH, GG>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
    k_paths_fp64<KK, RICH, GG><<<grid, FP64_THREADS, smem, s>>>(a);                                      \
    break;
  if (a.L.geom == 1) {
    switch (kind) {
      PDDS_FP64_CASE(0, 1)
      PDDS_FP64_CASE(5, 1)
      default: return cudaErrorInvalidValue;
    }
  } else {
    switch (kind) {
      PDDS_FP64_CASE(0, 0)
      PDDS_FP64_CASE(1, 0)
      PDDS_FP64_CASE(2, 0)
      PDDS_FP64_CASE(3, 0)
      PDDS_FP64_CASE(4, 0)
      PDDS_FP64_CASE(5, 0)
      PDDS_FP64_CASE(6, 0)
      default: return cudaErrorInvalidValue;
    }
  }
#undef PDDS_FP64_CASE
  return cudaGetLastError();
}

cudaError_t launch_paths_fp64(const Fp64Args& a, int kind, int grid, size_t smem, cudaStream_t s) {
  return a.richardson ? launch_fp64_t<true>(a, kind, grid, smem, s) : launch_fp64_t<false>(a, kind, grid, smem, s);
}

template <bool RICH>
static int blocks64_t(int kind, size_t smem) {
  int nb = 0;
  switch (kind) {
    case 0: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_paths_fp64<0, RICH, 0>, FP64_THREADS, smem); break;
    case 1: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_paths_fp64<1, RICH, 0>, FP64_THREADS, smem); break;
    case 2: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_paths_fp64<2, RICH, 0>, FP64_THREADS, smem); break;
    case 4: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_paths_fp64<4, RICH, 0>, FP64_THREADS, smem); break;
    case 5: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_paths_fp64<5, RICH, 0>, FP64_THREADS, smem); break;
    default: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_paths_fp64<3, RICH, 0>, FP64_THREADS, smem); break;
  }
  return nb;
}

int fp64_blocks_per_sm(int kind, size_t smem, int richardson) {
  return richardson ? blocks64_t<true>(kind, smem) : blocks64_t<false>(kind, smem);
}

}  // namespace pdds
