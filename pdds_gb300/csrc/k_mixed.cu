// MIXED mode: FP32 Euler-Maruyama paths, compensated per-lane sums, FP64 per-knot accumulation.
//
// One persistent CTA per slot processes work items (knot, chunk of paths).
// Lanes step paths in FP32 with Philox-4x32-10 normals held in registers and
// refill from the item's path counter the moment their path exits, so a warp
// keeps stepping while path lengths vary.  A level that exits keeps its exit
// state; when both levels of a lane's Richardson pair have exited, the lane
// pushes the pair to a per-warp queue in shared memory, and the warp
// processes the queue 32 pairs at a time, one per lane, so exit handling runs
// at full width and needs no bookkeeping across lanes.  An exit
// on an interior stencil side deposits Y with cubic Lagrange weights into a
// per-side histogram of the exit coordinate in shared memory (4 FP32 atomics,
// O(1) per exit).  At the end of
// the item the histograms are contracted with the FP32 table of cardinal
// functions H_i(s) = sum_j Psi^-1(j,i) exp(-(t_j - s)^2 / c^2), computed in
// FP64 from the factorised RBF matrix, and added into the G row in FP64.
// This is the same estimator as the reference's per-exit G_update
// (Meshes/stencil.cpp:244-307) up to the cubic interpolation of H between grid
// points; it avoids evaluating RBF weights in FP32, where the condition number
// of Psi (1e9..1e11) would amplify rounding by that factor.
#include "dev_common.cuh"
#include "kernels.h"

namespace pdds {

namespace {

struct ItemSide {
  int n;
  int nbins;
  int hist_off;
  int orient;
  int glob;
  float base;
  float inv_delta;
  int64_t tab_off;
  int64_t map_off;
};

constexpr unsigned FULL = 0xffffffffu;

// State of one level of a path.  With table-served coefficients the level
// also carries the 8 table fields at its position: the end-of-step sample
// gives sigma for the exit test and the coefficients of the next step.
template <int KIND>
struct Lvl {
  float x, y, Y, Z, xi;
  unsigned steps;
};
template <>
struct Lvl<PK_LUT> {
  float x, y, Y, Z, xi;
  unsigned steps;
  float cf[8];
};
template <>
struct Lvl<PK_LUT_TEX> : Lvl<PK_LUT> {};

// Exit queue of a warp: a lane whose path pair has finished pushes both
// levels' exit states (x, y, Y, Z + xi of the fine level, then of the coarse
// level, then the step-limit flags) and the warp processes 32 pairs at a
// time, one per lane.  <= 31 left over + one push of 32; slot XQCAP is the
// spare slot written by lanes that push nothing.
constexpr int XQCAP = 64;

// Kahan step: s + c tracks the exact sum to O(eps^2); c holds the negated
// rounding error of the running sum.
__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
  const float y = __fsub_rn(x, c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
}

// Box-Muller in FP32 from two Philox words: z0 = rho cos(2 pi u1),
// z1 = rho sin(2 pi u1) with rho = sqrt(-2 ln u0), u = (word + 1/2) 2^-32,
// evaluated as -rho cos/sin(a) at a = 2 pi u1 - pi in [-pi, pi], which the
// fast intrinsics take directly (a is formed from the word in one FMA).
__device__ __forceinline__ float2 normals_f32(uint32_t ua, uint32_t ub) {
  const float u0 = fmaf((float)ua, 2.3283064e-10f, 1.1641532e-10f);
  const float rho = sqrt_approx(-1.38629436f * lg2_approx(u0));  // -2 ln u0 = -2 ln2 log2 u0
  const float ang = fmaf((float)ub, 1.46291808e-9f, -3.14159265f);
  float sn, cs;
  __sincosf(ang, &sn, &cs);
  // (z0, z1) = -rho (cos, sin) in one paired multiply (the same two roundings)
  return __fmul2_rn(make_float2(-rho, -rho), make_float2(cs, sn));
}

// path_block (counter = (step pair, path, knot, instance)) with the key
// schedule read from the kernel parameters: the same stream.
__device__ __forceinline__ u32x4 path_block_rk(const uint32_t (&rk)[20], uint32_t instance, uint32_t knot,
                                               uint32_t path, uint32_t step_pair) {
  u32x4 c;
  c.v[0] = step_pair;
  c.v[1] = path;
  c.v[2] = knot;
  c.v[3] = instance;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = __umulhi(0xD2511F53u, c.v[0]), lo0 = 0xD2511F53u * c.v[0];
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.v[2]), lo1 = 0xCD9E8D57u * c.v[2];
    u32x4 n;
    n.v[0] = hi1 ^ c.v[1] ^ rk[2 * r];
    n.v[1] = lo1;
    n.v[2] = hi0 ^ c.v[3] ^ rk[2 * r + 1];
    n.v[3] = lo0;
    c = n;
  }
  return c;
}

// Table-served coefficients sampled from the nodes (PK_LUT) need more live
// registers for the bicubic accumulation: 128 registers there; the texture
// samplers (PK_LUT_TEX) leave the interpolation to the texture units and
// run with LUT_TEX_MIN_BLOCKS blocks' worth; 64 otherwise.  The block size
// is chosen at launch (mixed_threads: 128 or 256 threads).
constexpr int LUT_TEX_MIN_BLOCKS = 2;
// DIAG: the instantiation that also accumulates the reduction's diagnostic
// sums (pdds_estimate_diagnostics); a separate one, so that the estimate
// without them carries none of that code.
template <int KIND, bool RICH, int GEOM, bool DIAG>
__global__ void __launch_bounds__(MIXED_MAX_THREADS, KIND == PK_LUT ? 2 : (KIND == PK_LUT_TEX ? LUT_TEX_MIN_BLOCKS : 4))
k_paths_mixed(const MixedArgs a) {
  // dynamic shared memory: the warps' exit queues, then the exit histograms
  // [sum nbins] (and the Y^2 histogram after them)
  extern __shared__ float dyn[];
  __shared__ ItemSide s_side[4];
  __shared__ float s_rect[4];
  __shared__ float s_dir[4];  // polar stencils: (cos, sin) of phi0 and phi1
  __shared__ int s_item, s_knot, s_p0, s_path_end, s_hist_len;
  __shared__ float s_h, s_sqrth;
  __shared__ unsigned s_next_path;
  __shared__ double s_red[MIXED_MAX_THREADS / 32][4];
  __shared__ unsigned long long s_redi[MIXED_MAX_THREADS / 32][3];
  __shared__ unsigned s_sth[32];  // this item's paths by steps (log2 bins), when step_hist is set
  __shared__ double s_dg[DIAG ? PDDS_DIAG_N : 1];  // this item's diagnostic sums (DIAG)
  // exit queue of each warp: word w of slot i at q[w][i]
  constexpr int QW = RICH ? 9 : 5;
  const int nthr = blockDim.x, nwarps = nthr >> 5;
  float* hist = dyn + nwarps * QW * (XQCAP + 1);
  const DevLayout& L = a.L;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  for (;;) {
    if (tid == 0) s_item = atomicAdd(a.item_counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= a.n_items) break;
    if (tid == 0) {
      int k, p0, p1;
      if (a.item_knot) {
        k = a.item_knot[item];
        p0 = a.item_p0[item];
        p1 = a.item_p1[item];
      } else {
        k = a.mc_knots[item / a.chunks];
        p0 = (item % a.chunks) * a.paths_per_chunk;
        p1 = min(a.N, p0 + a.paths_per_chunk);
      }
      s_knot = k;
      s_p0 = p0;
      s_path_end = p1;
      s_next_path = (unsigned)(p0 + nthr);
      const int st = L.knot_stencil[k];
      for (int q = 0; q < 4; q++) s_rect[q] = (float)L.st_rect[4 * st + q];
      if (GEOM == 1) {
        s_dir[0] = (float)cos(L.st_rect[4 * st + 1]);
        s_dir[1] = (float)sin(L.st_rect[4 * st + 1]);
        s_dir[2] = (float)cos(L.st_rect[4 * st + 3]);
        s_dir[3] = (float)sin(L.st_rect[4 * st + 3]);
      }
      // the step of the knot's instance (batches), else the run's
      double h0 = a.h64;
      if (L.inst_h && L.knot_inst) {
        const double hi = L.inst_h[L.knot_inst[k]];
        if (hi > 0.0) h0 = hi;
      }
      s_h = (float)h0;
      s_sqrth = (float)sqrt(h0);
      if (a.adaptive_h) {
        ProblemDev Pk = a.P;
        uint32_t ri = 0, rk = 0;
        instance_params(L, k, Pk, ri, rk);
        Coef<double> kd;
        coef_f64<KIND>(Pk, L.kx[k], L.ky[k], kd);
        const double hk = GEOM == 1 ? adaptive_step_polar(L.st_rect + 4 * st, L.kx[k], L.ky[k], h0, kd)
                                    : adaptive_step<double>(L.st_rect + 4 * st, L.kx[k], L.ky[k], h0, kd);
        s_h = (float)hk;
        s_sqrth = (float)sqrt(hk);
      }
      int off = 0;
      for (int d = 0; d < 4; d++) {
        const int sd = L.st_side[4 * st + d];
        ItemSide is;
        is.glob = L.st_glob[4 * st + d];
        if (sd < 0) {
          is.n = 0; is.nbins = 0; is.hist_off = 0; is.orient = 0; is.base = 0.f; is.inv_delta = 0.f;
          is.tab_off = 0; is.map_off = 0;
        } else {
          const int sh = L.sd_shape[sd];
          is.n = L.sd_n[sd];
          is.nbins = L.sh_nbins[sh];
          is.hist_off = off;
          is.orient = L.sd_orient[sd];
          const double delta = L.sh_delta[sh];
          double origin = L.sd_origin[sd];
          if (GEOM == 1 && is.orient == 0) {  // arc: the side's angles in this stencil's turn
            const double tw = 6.283185307179586;
            origin += tw * nearbyint((L.st_rect[4 * st + 1] - origin) / tw);
          }
          is.base = (float)(origin + L.sh_lo[sh] - delta);
          is.inv_delta = (float)(1.0 / delta);
          is.tab_off = L.sh_tab_off[sh];
          off += is.nbins;
        }
        s_side[d] = is;
      }
      // side-knot -> row position maps, in side order
      int64_t moff = L.st_map_off[st];
      for (int d = 0; d < 4; d++) {
        s_side[d].map_off = moff;
        moff += s_side[d].n;
      }
      s_hist_len = off;
    }
    __syncthreads();
    const int knot = s_knot, path_end = s_path_end, hist_len = s_hist_len;
    // the problem of this knot's instance, and its Philox instance and knot words
    ProblemDev P = a.P;
    uint32_t rng_inst = a.instance, rng_knot = 0;
    instance_params(L, knot, P, rng_inst, rng_knot);
    const float h = s_h, sqrth = s_sqrth;
    const int nh = a.want_var ? 2 * hist_len : hist_len;
    for (int i = tid; i < nh; i += nthr) hist[i] = 0.f;
    if (tid < 32) s_sth[tid] = 0u;
    if (DIAG && tid < PDDS_DIAG_N) s_dg[tid] = 0.0;
    float* hist2 = hist + hist_len;
    __syncthreads();

    // ------------------------------------------------------------ paths
    // Every iteration of a lane: one Philox block, two Box-Muller pairs, and
    // a fixed sequence of steps -- (fine A, fine B, coarse) for the
    // Richardson pair, (A, B) otherwise -- so the warp's control flow stays
    // uniform while path lengths differ.  Exit deposits go through a
    // per-warp queue in shared memory and are applied 32 at a time by the
    // whole warp; finished lanes refill with a warp-aggregated atomic.
    const float x0 = (float)L.kx[knot], y0 = (float)L.ky[knot];
    const float rect[4] = {s_rect[0], s_rect[1], s_rect[2], s_rect[3]};
    const float cx = 0.5f * (rect[0] + rect[2]), cy = 0.5f * (rect[1] + rect[3]);
    const float hx = rect[2] - cx, hy = rect[3] - cy;
    // polar stencils: outside distances beyond the inner arc (none at the
    // centre), the outer arc, the ray at phi0 and the ray at phi1 (straight
    // lines through the centre: the wedge is narrower than pi)
    const float ua0 = s_dir[0], ua1 = s_dir[1], ub0 = s_dir[2], ub1 = s_dir[3];
    const bool has_inner = rect[0] > 0.f;
    const bool has_rays = rect[3] - rect[1] < 6.2f;  // a full disk has one side, its arc
    auto polar_out = [&](float x, float y, float& d_in, float& d_out, float& d_a, float& d_b) {
      const float rho = sqrt_approx(x * x + y * y);
      d_in = has_inner ? rect[0] - rho : -3.0e38f;
      d_out = rho - rect[2];
      d_a = has_rays ? ua1 * x - ua0 * y : -3.0e38f;
      d_b = has_rays ? ub0 * y - ub1 * x : -3.0e38f;
    };
    // bit d set when stencil side d lies on the global boundary
    const int globmask = (s_side[0].glob ? 1 : 0) | (s_side[1].glob ? 2 : 0) | (s_side[2].glob ? 4 : 0) |
                         (s_side[3].glob ? 8 : 0);
    // PK_ROBIN: the stencil side on the Robin part of the boundary (P.p[0],
    // bits N 1, S 2, E 4, W 8) reflects instead of absorbing; its line is
    // n . (x, y) = rc with the outward unit normal n
    const int rmask = KIND == PK_ROBIN ? (globmask & (int)P.p[0]) : 0;
    float rn0 = 0.f, rn1 = 0.f, rc = 0.f;
    if (rmask & 1) { rn1 = 1.f; rc = rect[3]; }
    else if (rmask & 2) { rn1 = -1.f; rc = -rect[1]; }
    else if (rmask & 4) { rn0 = 1.f; rc = rect[2]; }
    else if (rmask & 8) { rn0 = -1.f; rc = -rect[0]; }
    // outside distances to the absorbing sides (N, S, E, W order of the side
    // index), the reflecting side excluded
    auto absorb_out = [&](float x, float y, float* o) {
      o[0] = (rmask & 1) ? -3.0e38f : y - rect[3];
      o[1] = (rmask & 2) ? -3.0e38f : rect[1] - y;
      o[2] = (rmask & 4) ? -3.0e38f : x - rect[2];
      o[3] = (rmask & 8) ? -3.0e38f : rect[0] - x;
    };
    unsigned path = (unsigned)(s_p0 + tid);
    bool active = (int)path < path_end;
    // per-lane B sums in compensated FP32 (Kahan), folded into FP64 per item:
    // the error is at most 2 eps_32 sum |v| over the lane's paths of the item
    float bs = 0.f, bc = 0.f, bbs = 0.f, bbc = 0.f;
    unsigned long long nsteps = 0;
    unsigned nglob = 0, nsten = 0;  // exits of the lane in this item (<= 2 N)
    int qcount = 0;  // warp-uniform
    const unsigned lt = (1u << lane) - 1u;
    float (*q)[XQCAP + 1] = reinterpret_cast<float (*)[XQCAP + 1]>(dyn + warp * QW * (XQCAP + 1));
    const bool use_cv = P.use_cv != 0;
    // increment scales (sqrt2 sqrt(h) for iso kinds, sqrt(h) otherwise) and
    // Gobet thresholds of the fine (h/2) and coarse (h) levels
    const float hf = 0.5f * h;
    const float scc = KindTraits<KIND>::iso ? 1.41421356f * sqrth : sqrth;
    const float scf = scc * 0.70710678f;
    const float thrc = -0.5826f * scc, thrf = -0.5826f * scf;
    const unsigned maxs = (unsigned)a.max_steps;

    // One step of a level (Step, control-variate variant,
    // FKACIntegrator.hpp:46-57) and the Gobet-shifted exit test (Inside,
    // :168-222), branch-free: with dx = |x - cx| - hx, dy = |y - cy| - hy the
    // reference's signed distance is max(dx, dy) except in the outer corner
    // region (where both are positive and the path exits anyway), and its
    // normal is the x normal exactly when dx > dy.
    // Every kind has a diagonal sigma.  For iso kinds (sigma = sqrt2 I) e is
    // the diffusion increment sqrt2 dW and thr the shift -0.5826 sqrt2 sqrt(h);
    // otherwise e = dW and thr = -0.5826 sqrt(h), scaled by |N^T sigma| here.
    // The control-variate sum xi = -sum Y grad u . sigma dW is always
    // accumulated; the exit drops it when the control variate is off.
    // PK_ROBIN with a reflecting side: Lepingle's reflected Euler step
    // (FKACIntegrator.hpp:116-165 restated from the published scheme): with
    // U = n . sigma dW and an Exp(1) sample ex, the largest outward excursion
    // of the step is M = (U + sqrt(U^2 + 2 |sigma^T n|^2 h ex)) / 2 (the
    // maximum of the Brownian bridge); the local time dL = max(0, M + d),
    // d the signed distance to the side (negative inside), pushes the path
    // back along -n and enters dZ = psi Y dL, dY = varphi Y dL.
    // The (x, y) arithmetic of a step runs as paired FP32 instructions
    // (FADD2 / FMUL2 / FFMA2: two lanes' worth of work per issue slot, the
    // same roundings as the scalar pair).
    auto advance = [&](Lvl<KIND>& s, float2 e, float hh, float thr, float ex) -> bool {
      Coef<float> k;
      if constexpr (is_lut_kind(KIND)) {
        k.s00 = s.cf[0]; k.s11 = s.cf[1];
        k.b0 = s.cf[2]; k.b1 = s.cf[3]; k.c = s.cf[4]; k.f = s.cf[5];
        k.g0 = s.cf[6]; k.g1 = s.cf[7];
      } else {
        coef_f32<KIND>(P, s.x, s.y, k);
      }
      float2 d = e;
      if constexpr (!KindTraits<KIND>::iso) d = __fmul2_rn(make_float2(k.s00, k.s11), e);
      const float d0 = d.x, d1 = d.y;
      s.xi -= s.Y * (k.g0 * d0 + k.g1 * d1);
      s.Z += k.f * s.Y * hh;
      if constexpr (KindTraits<KIND>::react) s.Y += k.c * s.Y * hh;
      if constexpr (KIND == PK_ROBIN) {
        float dL = 0.f;
        if (rmask) {
          const float dR = rn0 * s.x + rn1 * s.y - rc;
          const float U = rn0 * d0 + rn1 * d1;
          const float M = 0.5f * (U + sqrt_approx(U * U + 4.f * hh * ex));  // |sigma^T n|^2 = 2
          dL = fmaxf(0.f, M + dR);
          if (dL > 0.f) {
            // dY = varphi Y dL and dZ = psi Y dL integrated exactly over dL:
            // an Euler update would leave an O(sqrt h) bias (sum of dL^2)
            float vphi, psi;
            robin_data<float>(s.x - dR * rn0, s.y - dR * rn1, rn0, rn1, vphi, psi);
            const float t = vphi * dL;
            const float em1 = expm1f(t);
            s.Z += psi * s.Y * (t != 0.f ? em1 / vphi : dL);
            s.Y += s.Y * em1;
          }
        }
        s.x += d0 - dL * rn0;
        s.y += d1 - dL * rn1;
        ++s.steps;
        float o[4];
        absorb_out(s.x, s.y, o);
        return !(fmaxf(fmaxf(o[0], o[1]), fmaxf(o[2], o[3])) < thr) || s.steps >= (unsigned)a.max_steps;
      } else if constexpr (KindTraits<KIND>::iso) {
        const float2 np = __fadd2_rn(make_float2(s.x, s.y), d);
        s.x = np.x;
        s.y = np.y;
      } else {
        const float2 np =
            __fadd2_rn(make_float2(s.x, s.y), __ffma2_rn(make_float2(k.b0, k.b1), make_float2(hh, hh), d));
        s.x = np.x;
        s.y = np.y;
      }
      ++s.steps;
      if constexpr (GEOM == 1) {  // iso kinds only: |N^T sigma| = sqrt2 for every normal
        float d_in, d_out, d_a, d_b;
        polar_out(s.x, s.y, d_in, d_out, d_a, d_b);
        const float dist = fmaxf(fmaxf(d_in, d_out), fmaxf(d_a, d_b));
        return !(dist < thr) || s.steps >= (unsigned)a.max_steps;
      } else {
        const float dx = fabsf(s.x - cx) - hx, dy = fabsf(s.y - cy) - hy;
        float t = thr;
        if constexpr (is_lut_kind(KIND)) {
          lut_sample_f32<KIND, 8>(P.lut, s.x, s.y, s.cf);
          t *= dx > dy ? fabsf(s.cf[0]) : fabsf(s.cf[1]);
        } else if constexpr (!KindTraits<KIND>::iso) {
          float nx, ny;  // |N^T sigma| for the x and y normals
          sigma_normals_f32<KIND>(P, s.x, s.y, nx, ny);
          t *= dx > dy ? nx : ny;
        }
        return !(fmaxf(dx, dy) < t) || s.steps >= (unsigned)a.max_steps;
      }
    };
    // Value of one exit of a level, weighted: projection onto the stencil
    // (Rectangle2D, rectangle.hpp:7-229) as selects -- the x side is taken
    // exactly when dx > dy, the other coordinate is clamped to the rectangle
    // (the identity inside, the corner outside both slabs), and the sides the
    // projection lies on are read off by equality, first match in the order
    // S, N, W, E as in G_update (stencil.cpp:246-301) -- then g at a global
    // side or a deposit of wgt Y on an interior side.  Returns wgt (Z + xi +
    // Y g) for the pair's B contribution.  `limit`: the level stopped at the
    // step limit, an error unless it had exited anyway.
    auto score = [&](float x, float y, float Y, float val, float wgt, bool limit, float sql) -> float {
      bool ok = true;
      if (limit) {  // step limit reached: an error unless the path had exited anyway
        float dist, wn;
        if constexpr (GEOM == 1) {
          float d_in, d_out, d_a, d_b;
          polar_out(x, y, d_in, d_out, d_a, d_b);
          dist = fmaxf(fmaxf(d_in, d_out), fmaxf(d_a, d_b));
          wn = 1.41421356f;
        } else if constexpr (KIND == PK_ROBIN) {
          float o[4];
          absorb_out(x, y, o);
          dist = fmaxf(fmaxf(o[0], o[1]), fmaxf(o[2], o[3]));
          wn = 1.41421356f;
        } else {
          float Ex, Ey, Nx, Ny;
          int om;
          dist = rect2d<float>(rect, x, y, Ex, Ey, Nx, Ny, om);
          float g00, g01, g10, g11;
          sigma_f32<KIND>(P, x, y, g00, g01, g10, g11);
          const float w0 = Nx * g00 + Ny * g10, w1 = Nx * g01 + Ny * g11;
          wn = sqrtf(w0 * w0 + w1 * w1);
        }
        if (dist < -0.5826f * wn * sql) {
          atomicOr(a.err_flags, ERR_FLAG_STEP_LIMIT);
          ok = false;
          val = 0.f;
        }
      }
      if (ok && (isnan(x) || isnan(y))) {
        // a position that is not a number lies on no side (the reference's
        // G_update stops there): reported, and the pair scores nothing
        atomicOr(a.err_flags, ERR_FLAG_EXIT_SIDE);
        ok = false;
        val = 0.f;
      }
      if (ok && GEOM == 1) {
        // polar stencil: the side with the largest outside distance (ties
        // S, N, W, E); arcs are parameterised by the angle (measured from
        // phi0, clamped to the stencil), rays by the radius (clamped)
        float d_in, d_out, d_a, d_b;
        polar_out(x, y, d_in, d_out, d_a, d_b);
        int d = 1;
        float mx = d_in;
        if (d_out > mx) { mx = d_out; d = 0; }
        if (d_a > mx) { mx = d_a; d = 3; }
        if (d_b > mx) { mx = d_b; d = 2; }
        float sc;
        bool glob = false;
        if (d <= 1) {
          const float rel = atan2f(ua0 * y - ua1 * x, ua0 * x + ua1 * y);
          const float ang = rect[1] + (has_rays ? fminf(fmaxf(rel, 0.f), rect[3] - rect[1])
                                                : (rel < 0.f ? rel + 6.28318531f : rel));
          sc = ang;
          if (d == 0 && (globmask & 1)) {
            glob = true;
            float sa, ca;
            sincosf(ang, &sa, &ca);
            val += Y * u_f32<KIND>(P, rect[2] * ca, rect[2] * sa);
          }
        } else {
          const float t = d == 3 ? ua0 * x + ua1 * y : ub0 * x + ub1 * y;
          sc = fminf(fmaxf(t, rect[0]), rect[2]);
        }
        if (glob) {
          ++nglob;
        } else {
          ++nsten;
          const ItemSide& is = s_side[d];
          if (is.n > 0) {
            const float uu = (sc - is.base) * is.inv_delta;
            int b0 = (int)floorf(uu);
            b0 = max(1, min(b0, is.nbins - 3));
            float w[4];
            cubic_weights(uu - (float)b0, w[0], w[1], w[2], w[3]);
            const float yw = wgt * Y;
            float* hp = hist + is.hist_off + b0 - 1;
            // the 4 bins lie in the side's histogram, inside the CTA's
            const bool in = idx_ok(b0 - 1, is.nbins - 3, a.err_flags) &&
                            idx_ok(is.hist_off + b0 + 2, hist_len, a.err_flags);
#pragma unroll
            for (int r = 0; r < 4; r++)
              if (in) atomicAdd(hp + r, yw * w[r]);
            if (a.want_var && in) {
              float* hq = hist2 + is.hist_off + b0 - 1;
              const float y2 = yw * yw;
#pragma unroll
              for (int r = 0; r < 4; r++) atomicAdd(hq + r, y2 * w[r]);
            }
          }
        }
      } else if (ok) {
        float Ex, Ey;
        int onmask, d;
        if constexpr (KIND == PK_ROBIN) {
          // the absorbing side with the largest outside distance (ties S, N,
          // W, E), the other coordinate clamped to it
          float o[4];
          absorb_out(x, y, o);
          d = 1;
          float mx = o[1];
          if (o[0] > mx) { mx = o[0]; d = 0; }
          if (o[3] > mx) { mx = o[3]; d = 3; }
          if (o[2] > mx) { mx = o[2]; d = 2; }
          Ex = d == 3 ? rect[0] : (d == 2 ? rect[2] : fminf(fmaxf(x, rect[0]), rect[2]));
          Ey = d == 1 ? rect[1] : (d == 0 ? rect[3] : fminf(fmaxf(y, rect[1]), rect[3]));
          onmask = 1 << d;
        } else {
          const float dx = fabsf(x - cx) - hx, dy = fabsf(y - cy) - hy;
          const bool xs = dx > dy;
          Ex = xs ? (x > cx ? rect[2] : rect[0]) : fminf(fmaxf(x, rect[0]), rect[2]);
          Ey = xs ? fminf(fmaxf(y, rect[1]), rect[3]) : (y > cy ? rect[3] : rect[1]);
          const bool onS = Ey == rect[1], onN = Ey == rect[3], onW = Ex == rect[0], onE = Ex == rect[2];
          onmask = (onN ? 1 : 0) | (onS ? 2 : 0) | (onE ? 4 : 0) | (onW ? 8 : 0);
          d = onS ? 1 : (onN ? 0 : (onW ? 3 : 2));
        }
        if (onmask & globmask) {
          ++nglob;
          val += Y * u_f32<KIND>(P, Ex, Ey);
        } else {
          ++nsten;
          const ItemSide& is = s_side[d];
          if (is.n > 0) {
            const float sc = is.orient == 0 ? Ex : Ey;
            const float uu = (sc - is.base) * is.inv_delta;
            int b0 = (int)floorf(uu);
            b0 = max(1, min(b0, is.nbins - 3));
            float w[4];
            cubic_weights(uu - (float)b0, w[0], w[1], w[2], w[3]);
            const float yw = wgt * Y;
            float* hp = hist + is.hist_off + b0 - 1;
            // the 4 bins lie in the side's histogram, inside the CTA's
            const bool in = idx_ok(b0 - 1, is.nbins - 3, a.err_flags) &&
                            idx_ok(is.hist_off + b0 + 2, hist_len, a.err_flags);
#pragma unroll
            for (int r = 0; r < 4; r++)
              if (in) atomicAdd(hp + r, yw * w[r]);
            if (a.want_var && in) {
              float* hq = hist2 + is.hist_off + b0 - 1;
              const float y2 = yw * yw;
#pragma unroll
              for (int r = 0; r < 4; r++) atomicAdd(hq + r, y2 * w[r]);
            }
          }
        }
      }
      return wgt * val;
    };
    Lvl<KIND> F, Cs;  // fine (or only) and coarse level of the lane's pair
    // Push the finished pairs of the warp (both levels' exit states; the
    // warp-synchronous ballot gives each its slot) and return their mask.
    // Lanes without a finished pair write the spare slot XQCAP instead of
    // branching around the stores.
    auto push = [&](bool ex) -> unsigned {
      const unsigned mk = __ballot_sync(FULL, ex);
      int i = ex ? qcount + __popc(mk & lt) : XQCAP;
      if (!idx_ok(i, XQCAP + 1, a.err_flags)) i = XQCAP;
      q[0][i] = F.x;
      q[1][i] = F.y;
      q[2][i] = F.Y;
      q[3][i] = use_cv ? F.Z + F.xi : F.Z;
      unsigned meta = F.steps >= maxs ? 1u : 0u;
      if (RICH) {
        q[4][i] = Cs.x;
        q[5][i] = Cs.y;
        q[6][i] = Cs.Y;
        q[7][i] = use_cv ? Cs.Z + Cs.xi : Cs.Z;
        meta |= Cs.steps >= maxs ? 2u : 0u;
      }
      q[QW - 1][i] = __uint_as_float(meta);
      qcount += __popc(mk);
      return mk;
    };
    // Process the pair at queue index i (lane-parallel): both exits scored,
    // B += 2 v_fine - v_coarse (v otherwise) in the lane's compensated sums.
    auto process = [&](int i, bool valid) {
      if (valid) {
        const unsigned meta = __float_as_uint(q[QW - 1][i]);
        float v = 0.f;
#pragma unroll 1
        for (int lv = 0; lv < (RICH ? 2 : 1); lv++) {
          const int o = 4 * lv;
          const float wgt = RICH ? (lv ? -1.f : 2.f) : 1.f;
          const float sql = (RICH && lv == 0) ? sqrth * 0.70710678f : sqrth;
          v += score(q[o][i], q[o + 1][i], q[o + 2][i], q[o + 3][i], wgt, ((meta >> lv) & 1u) != 0, sql);
        }
        kahan_add(bs, bc, v);
        kahan_add(bbs, bbc, v * v);
      }
    };
    auto drain_full = [&]() {
      __syncwarp();
      while (qcount >= 32) {
        process(qcount - 32 + lane, true);
        __syncwarp();
        qcount -= 32;
      }
    };
    auto drain_all = [&]() {
      drain_full();
      if (qcount > 0) {
        process(lane, lane < qcount);
        __syncwarp();
        qcount = 0;
      }
    };

    float cf0[8];  // table fields at the knot (table-served kinds)
    if constexpr (is_lut_kind(KIND)) lut_sample_f32<KIND, 8>(P.lut, x0, y0, cf0);
    auto reset = [&]() {
      F.x = x0; F.y = y0; F.Y = 1.f; F.Z = 0.f; F.xi = 0.f; F.steps = 0;
      if constexpr (is_lut_kind(KIND)) {
#pragma unroll
        for (int f = 0; f < 8; f++) F.cf[f] = cf0[f];
      }
      Cs = F;
    };
    reset();
    bool f_alive = active, c_alive = RICH && active;
    unsigned m = 0;
    while (__any_sync(FULL, active)) {
      if (active) {
        const unsigned mi = m++;
        const u32x4 blk = path_block_rk(a.rk, rng_inst, rng_knot, path, mi);
        const float2 za = normals_f32(blk.v[0], blk.v[1]), zb = normals_f32(blk.v[2], blk.v[3]);
        // Exp(1) samples of the reflected steps: a second Philox block with
        // the knot word's top bit set (fine A, fine B, coarse)
        float x0e = 0.f, x1e = 0.f, x2e = 0.f;
        if (KIND == PK_ROBIN && rmask) {
          const u32x4 bx = path_block_rk(a.rk, rng_inst, rng_knot | 0x80000000u, path, mi);
          x0e = -0.69314718f * lg2_approx(fmaf((float)bx.v[0], 2.3283064e-10f, 1.1641532e-10f));
          x1e = -0.69314718f * lg2_approx(fmaf((float)bx.v[1], 2.3283064e-10f, 1.1641532e-10f));
          x2e = -0.69314718f * lg2_approx(fmaf((float)bx.v[2], 2.3283064e-10f, 1.1641532e-10f));
        }
        if (RICH) {
          // Richardson pair: two fine steps of h/2 and one coarse step of h
          // on the same Brownian increments (dW_coarse = dW_fine1 + dW_fine2);
          // 2 E[fine] - E[coarse] cancels the O(h) bias.  A level that has
          // exited keeps its exit state until the pair is pushed.
          const float2 sf = make_float2(scf, scf);
          const float2 ea = __fmul2_rn(sf, za), eb = __fmul2_rn(sf, zb);
          if (f_alive) {
            bool fx = advance(F, ea, hf, thrf, x0e);
            if (!fx) fx = advance(F, eb, hf, thrf, x1e);
            f_alive = !fx;
          }
          if (c_alive) c_alive = !advance(Cs, __fadd2_rn(ea, eb), h, thrc, x2e);
        } else {
          const float2 sc = make_float2(scc, scc);
          bool fx = advance(F, __fmul2_rn(sc, za), h, thrc, x0e);
          if (!fx) fx = advance(F, __fmul2_rn(sc, zb), h, thrc, x1e);
          f_alive = !fx;
        }
      }
      // finished pairs: queue both exits, then refill from the item's
      // path counter with one warp-aggregated atomic
      const bool done = active && !f_alive && !c_alive;
      const unsigned dm = push(done);
      drain_full();
      if (dm) {
        const int leader = __ffs(dm) - 1;
        unsigned base = 0;
        if (lane == leader) base = atomicAdd(&s_next_path, (unsigned)__popc(dm));
        base = __shfl_sync(FULL, base, leader);
        if (done) {
          if (a.step_hist) {  // finished pairs only: a few lanes per iteration
            atomicAdd(&s_sth[31 - __clz(max(F.steps, 1u))], 1u);
            if (RICH) atomicAdd(&s_sth[31 - __clz(max(Cs.steps, 1u))], 1u);
          }
          if constexpr (DIAG && GEOM == 0) {
            // phi = Z + Y g at the nearest point of the stencil rectangle
            // (the exit projection), per level; a pair adds 2 fine - coarse
            auto phi_of = [&](const Lvl<KIND>& v) -> float {
              float Ex, Ey, Nx, Ny;
              int om;
              rect2d<float>(rect, v.x, v.y, Ex, Ey, Nx, Ny, om);
              return v.Z + v.Y * u_f32<KIND>(P, Ex, Ey);
            };
            float ph = phi_of(F), xv = F.xi;
            if (RICH) {
              ph = 2.f * ph - phi_of(Cs);
              xv = 2.f * xv - Cs.xi;
            }
            diag_add(s_dg, ph, xv, (double)F.steps * (RICH ? 0.5 * (double)h : (double)h), 2.0 * F.steps);
          }
          nsteps += F.steps + (RICH ? Cs.steps : 0u);
          path = base + __popc(dm & lt);
          active = (int)path < path_end;
          reset();
          f_alive = active;
          c_alive = RICH && active;
          m = 0;
        }
      }
    }
    drain_all();
    // ------------------------------------------------------------ reduce B
    double b = (double)bs - (double)bc, bb = (double)bbs - (double)bbc;
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
      for (int w = 0; w < nwarps; w++) {
        tb += s_red[w][0]; tbb += s_red[w][1];
        ts += s_redi[w][0]; tg += s_redi[w][1]; tt += s_redi[w][2];
      }
      atomicAdd(a.Bsum + knot, tb);
      atomicAdd(a.BBsum + knot, tbb);
      atomicAdd(a.stats + 0, ts);
      if (a.knot_steps) atomicAdd(a.knot_steps + knot, ts);
      atomicAdd(a.stats + 2, tg);
      atomicAdd(a.stats + 3, tt);
    }
    if (a.step_hist && tid < 32 && s_sth[tid]) atomicAdd(a.step_hist + tid, (unsigned long long)s_sth[tid]);
    if constexpr (DIAG) diag_flush(s_dg, a.diag + (int64_t)knot * PDDS_DIAG_N, tid);
    // ------------------------------------------------------------ contract G
    const int64_t row0 = L.row_ptr[knot];
    const double invN = a.knot_invN ? a.knot_invN[knot] : a.inv_N;
    const int n_all = s_side[0].n + s_side[1].n + s_side[2].n + s_side[3].n;
    for (int pr = tid; pr < n_all; pr += nthr) {
      int d = 0, i = pr;
      while (i >= s_side[d].n) { i -= s_side[d].n; ++d; }
      const ItemSide& is = s_side[d];
      const int64_t m = is.map_off + i;
      if (!a.dup_sum && !L.map_owner[m]) continue;
      const float* tab = L.tab + is.tab_off + i;
      const float* hs = hist + is.hist_off;
      const float* hs2 = hist2 + is.hist_off;
      double acc = 0.0, acc2 = 0.0;
      for (int b0 = 0; b0 < is.nbins; b0 += 64) {
        const int b1 = min(is.nbins, b0 + 64);
        float part = 0.f, part2 = 0.f;
        for (int q = b0; q < b1; q++) {
          const float hv = __ldg(tab + (int64_t)q * is.n);
          part = fmaf(hs[q], hv, part);
          if (a.want_var) part2 = fmaf(hs2[q], hv * hv, part2);
        }
        acc += (double)part;
        acc2 += (double)part2;
      }
      const int64_t e = row0 + L.map_pos[m];
      if (!idx_ok(e - row0, L.row_ptr[knot + 1] - row0, a.err_flags)) continue;
      atomicAdd(a.G + e, -acc * invN);
      if (a.want_var) atomicAdd(a.GG + e, acc2 * invN);
    }
    __syncthreads();
  }
}

}  // namespace

// Polar stencils are instantiated for the isotropic problems only.
template <bool RICH>
static cudaError_t launch_mixed_t(const MixedArgs& a, int kind, int grid, int threads, size_t smem, cudaStream_t s) {
#define PDDS_MIXED_LAUNCH(KK, GG, DD)                                                                         \
  cudaFuncSetAttribute(k_paths_mixed<KK, RICH, GG, DD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
  k_paths_mixed<KK, RICH, GG, DD><<<grid, threads, smem, s>>>(a);
#define PDDS_MIXED_CASE(KK, GG)            \
  case KK:                                 \
    if (GG == 0 && a.diag) {               \
      PDDS_MIXED_LAUNCH(KK, GG * 0, true)  \
    } else {                               \
      PDDS_MIXED_LAUNCH(KK, GG, false)     \
    }                                      \
    break;
  if (a.L.geom == 1) {
    switch (kind) {
      PDDS_MIXED_CASE(0, 1)
      PDDS_MIXED_CASE(5, 1)
      default: return cudaErrorInvalidValue;
    }
  } else {
    switch (kind) {
      PDDS_MIXED_CASE(0, 0)
      PDDS_MIXED_CASE(1, 0)
      PDDS_MIXED_CASE(2, 0)
      PDDS_MIXED_CASE(3, 0)
      PDDS_MIXED_CASE(4, 0)
      PDDS_MIXED_CASE(5, 0)
      PDDS_MIXED_CASE(6, 0)
      PDDS_MIXED_CASE(7, 0)
      default: return cudaErrorInvalidValue;
    }
  }
#undef PDDS_MIXED_CASE
#undef PDDS_MIXED_LAUNCH
  return cudaGetLastError();
}

// Known-answer check of path_block_rk, the generator form of the MIXED path
// kernel: block i of out is the Philox-4x32-10 output for the counter
// ctr[4i..4i+3] = (step pair, path, knot, instance) under the key schedule
// rk of one key, exactly as the path kernel calls it.
__global__ void k_philox_rk_check(const MixedArgs a, const uint32_t* __restrict__ ctr, int n,
                                  uint32_t* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const u32x4 b = path_block_rk(a.rk, ctr[4 * i + 3], ctr[4 * i + 2], ctr[4 * i + 1], ctr[4 * i]);
  for (int q = 0; q < 4; q++) out[4 * i + q] = b.v[q];
}

cudaError_t launch_philox_rk_check(uint64_t key, const uint32_t* ctr, int n, uint32_t* out, cudaStream_t s) {
  MixedArgs a{};
  mixed_set_rng(a, key, 0);
  if (n > 0) k_philox_rk_check<<<(n + 127) / 128, 128, 0, s>>>(a, ctr, n, out);
  return cudaGetLastError();
}

void mixed_set_rng(MixedArgs& a, uint64_t seed, uint32_t instance) {
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  for (int r = 0; r < 10; r++) {
    a.rk[2 * r] = k0;
    a.rk[2 * r + 1] = k1;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  a.instance = instance;
}

template <bool RICH>
static bool is_mixed_t(const void* f) {
  return f == (const void*)k_paths_mixed<0, RICH, 0, false> || f == (const void*)k_paths_mixed<1, RICH, 0, false> ||
         f == (const void*)k_paths_mixed<2, RICH, 0, false> || f == (const void*)k_paths_mixed<3, RICH, 0, false> ||
         f == (const void*)k_paths_mixed<4, RICH, 0, false> || f == (const void*)k_paths_mixed<5, RICH, 0, false> ||
         f == (const void*)k_paths_mixed<6, RICH, 0, false> || f == (const void*)k_paths_mixed<7, RICH, 0, false> ||
         f == (const void*)k_paths_mixed<0, RICH, 1, false> || f == (const void*)k_paths_mixed<5, RICH, 1, false>;
}

bool is_mixed_path_kernel(const void* func) { return is_mixed_t<true>(func) || is_mixed_t<false>(func); }

size_t mixed_queue_smem(int threads, int richardson) {
  return (size_t)(threads / 32) * (richardson ? 9 : 5) * (XQCAP + 1) * sizeof(float);
}

cudaError_t launch_paths_mixed(const MixedArgs& a, int kind, int grid, int threads, size_t smem, cudaStream_t s) {
  if (threads != 128 && threads != 256) return cudaErrorInvalidValue;
  return a.richardson ? launch_mixed_t<true>(a, kind, grid, threads, smem, s)
                      : launch_mixed_t<false>(a, kind, grid, threads, smem, s);
}

template <bool RICH, bool DIAG>
static int blocks_t(int kind, size_t smem, int threads) {
  int nb = 0;
#define PDDS_OCC(KK)                                                                                          \
  case KK:                                                                                                    \
    cudaFuncSetAttribute(k_paths_mixed<KK, RICH, 0, DIAG>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_paths_mixed<KK, RICH, 0, DIAG>, threads, smem);       \
    break;
  switch (kind) {
    PDDS_OCC(0)
    PDDS_OCC(1)
    PDDS_OCC(2)
    PDDS_OCC(4)
    PDDS_OCC(5)
    PDDS_OCC(6)
    PDDS_OCC(7)
    default:
    PDDS_OCC(3)
  }
#undef PDDS_OCC
  return nb;
}

int mixed_blocks_per_sm(int kind, size_t smem, int richardson, int threads, bool diag) {
  if (diag) return richardson ? blocks_t<true, true>(kind, smem, threads) : blocks_t<false, true>(kind, smem, threads);
  return richardson ? blocks_t<true, false>(kind, smem, threads) : blocks_t<false, false>(kind, smem, threads);
}

}  // namespace pdds
