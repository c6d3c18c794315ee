// MIXED mode: FP32 Euler-Maruyama paths, FP64 per-knot accumulation.
//
// One persistent CTA per slot processes work items (knot, chunk of paths).
// Lanes step paths in FP32 with Philox-4x32-10 normals held in registers and
// refill from the item's path counter the moment their path exits, so a warp
// keeps stepping while path lengths vary.  An exit on an interior stencil side
// deposits Y with cubic Lagrange weights into a per-side histogram of the exit
// coordinate in shared memory (4 FP32 atomics, O(1) per exit).  At the end of
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

template <int KIND>
__global__ void __launch_bounds__(MIXED_THREADS)
k_paths_mixed(const MixedArgs a) {
  extern __shared__ float hist[];  // [sum nbins] (and the Y^2 histogram after it)
  __shared__ ItemSide s_side[4];
  __shared__ float s_rect[4];
  __shared__ int s_item, s_knot, s_path_end, s_hist_len;
  __shared__ unsigned s_next_path;
  __shared__ double s_red[MIXED_THREADS / 32][4];
  __shared__ unsigned long long s_redi[MIXED_THREADS / 32][3];
  const DevLayout& L = a.L;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const float h = a.h, sqrth = a.sqrth;

  for (;;) {
    if (tid == 0) s_item = atomicAdd(a.item_counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= a.n_items) break;
    if (tid == 0) {
      const int k = a.mc_knots[item / a.chunks];
      const int chunk = item % a.chunks;
      s_knot = k;
      const int p0 = chunk * a.paths_per_chunk;
      s_path_end = min(a.N, p0 + a.paths_per_chunk);
      s_next_path = (unsigned)(p0 + MIXED_THREADS);
      const int st = L.knot_stencil[k];
      for (int q = 0; q < 4; q++) s_rect[q] = (float)L.st_rect[4 * st + q];
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
          is.base = (float)(L.sd_origin[sd] + L.sh_lo[sh] - delta);
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
    const int nh = a.want_var ? 2 * hist_len : hist_len;
    for (int i = tid; i < nh; i += MIXED_THREADS) hist[i] = 0.f;
    float* hist2 = hist + hist_len;
    __syncthreads();

    // ------------------------------------------------------------ paths
    const float x0 = (float)L.kx[knot], y0 = (float)L.ky[knot];
    const float rect[4] = {s_rect[0], s_rect[1], s_rect[2], s_rect[3]};
    Coef<float> k0;
    coef_f32<KIND>(a.P, x0, y0, k0);
    const int chunk = item % a.chunks;
    unsigned path = (unsigned)(chunk * a.paths_per_chunk + tid);
    bool active = (int)path < path_end;
    float x = x0, y = y0, Y = 1.f, Z = 0.f, xi = 0.f;
    Coef<float> k = k0;
    unsigned step = 0;
    u32x4 blk;
    blk.v[0] = blk.v[1] = blk.v[2] = blk.v[3] = 0;
    double b = 0.0, bb = 0.0;
    unsigned long long nsteps = 0, nglob = 0, nsten = 0;
    while (__any_sync(FULL, active)) {
      if (!active) continue;
      // Step, control-variate variant (FKACIntegrator.hpp:46-57)
      if ((step & 1u) == 0) blk = path_block(a.seed, a.instance, (uint32_t)knot, path, step >> 1);
      const uint32_t ua = (step & 1u) ? blk.v[2] : blk.v[0];
      const uint32_t ub = (step & 1u) ? blk.v[3] : blk.v[1];
      const float u0 = fmaf((float)ua, 2.3283064e-10f, 1.1641532e-10f);
      const float u1 = fmaf((float)ub, 2.3283064e-10f, 1.1641532e-10f);
      const float rho = sqrtf(-2.f * __logf(u0));
      float sn, cs;
      __sincosf(6.28318531f * (u1 - 0.5f), &sn, &cs);  // angle 2 pi u1 - pi
      const float i0 = -rho * cs * sqrth, i1 = -rho * sn * sqrth;
      const float v0 = -(k.s00 * k.g0 + k.s10 * k.g1);
      const float v1 = -(k.s01 * k.g0 + k.s11 * k.g1);
      xi += Y * (v0 * i0 + v1 * i1);
      Z += k.f * Y * h;
      Y += k.c * Y * h;
      x += k.b0 * h + (k.s00 * i0 + k.s01 * i1);
      y += k.b1 * h + (k.s10 * i0 + k.s11 * i1);
      ++step;
      // Inside with the Gobet-Menozzi shift (FKACIntegrator.hpp:168-222)
      coef_f32<KIND>(a.P, x, y, k);
      float Ex, Ey, Nx, Ny;
      int onmask;
      const float dist = rect2d<float>(rect, x, y, Ex, Ey, Nx, Ny, onmask);
      const float w0 = Nx * k.s00 + Ny * k.s10, w1 = Nx * k.s01 + Ny * k.s11;
      const float thr = -0.5826f * sqrtf(w0 * w0 + w1 * w1) * sqrth;
      const bool capped = step >= (unsigned)a.max_steps;
      if (dist < thr && !capped) continue;
      // ---------------------------------------------------------- exit
      nsteps += step;
      if (capped && dist < thr) {
        atomicOr(a.err_flags, ERR_FLAG_STEP_LIMIT);
      } else {
        const int d = exit_side(onmask);
        const bool glob = ((onmask & 1) && s_side[0].glob) || ((onmask & 2) && s_side[1].glob) ||
                          ((onmask & 4) && s_side[2].glob) || ((onmask & 8) && s_side[3].glob);
        float val;
        if (glob) {
          val = Z + Y * u_f32<KIND>(a.P, Ex, Ey) + xi;
          ++nglob;
        } else {
          val = Z + xi;
          ++nsten;
          if (d < 0) {
            atomicOr(a.err_flags, ERR_FLAG_EXIT_SIDE);
          } else {
            const ItemSide& is = s_side[d];
            if (is.n > 0) {
              const float s = is.orient == 0 ? Ex : Ey;
              const float u = (s - is.base) * is.inv_delta;
              int b0 = (int)floorf(u);
              b0 = max(1, min(b0, is.nbins - 3));
              const float fu = u - (float)b0;
              float w[4];
              cubic_weights(fu, w[0], w[1], w[2], w[3]);
              float* hp = hist + is.hist_off + b0 - 1;
#pragma unroll
              for (int q = 0; q < 4; q++) atomicAdd(hp + q, Y * w[q]);
              if (a.want_var) {
                float* hq = hist2 + is.hist_off + b0 - 1;
                const float y2 = Y * Y;
#pragma unroll
                for (int q = 0; q < 4; q++) atomicAdd(hq + q, y2 * w[q]);
              }
            }
          }
        }
        b += (double)val;
        bb += (double)val * (double)val;
      }
      // refill from the item's path counter
      path = atomicAdd(&s_next_path, 1u);
      if ((int)path >= path_end) {
        active = false;
      } else {
        x = x0; y = y0; Y = 1.f; Z = 0.f; xi = 0.f; step = 0; k = k0;
      }
    }
    // ------------------------------------------------------------ reduce B
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
      for (int w = 0; w < MIXED_THREADS / 32; w++) {
        tb += s_red[w][0]; tbb += s_red[w][1];
        ts += s_redi[w][0]; tg += s_redi[w][1]; tt += s_redi[w][2];
      }
      atomicAdd(a.Bsum + knot, tb);
      atomicAdd(a.BBsum + knot, tbb);
      atomicAdd(a.stats + 0, ts);
      atomicAdd(a.stats + 2, tg);
      atomicAdd(a.stats + 3, tt);
    }
    // ------------------------------------------------------------ contract G
    const int64_t row0 = L.row_ptr[knot];
    const int n_all = s_side[0].n + s_side[1].n + s_side[2].n + s_side[3].n;
    for (int pr = tid; pr < n_all; pr += MIXED_THREADS) {
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
      atomicAdd(a.G + e, -acc * a.inv_N);
      if (a.want_var) atomicAdd(a.GG + e, acc2 * a.inv_N);
    }
    __syncthreads();
  }
}

}  // namespace

cudaError_t launch_paths_mixed(const MixedArgs& a, int kind, int grid, size_t smem, cudaStream_t s) {
  switch (kind) {
    case 0: {
      cudaFuncSetAttribute(k_paths_mixed<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      k_paths_mixed<0><<<grid, MIXED_THREADS, smem, s>>>(a);
      break;
    }
    case 1: {
      cudaFuncSetAttribute(k_paths_mixed<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      k_paths_mixed<1><<<grid, MIXED_THREADS, smem, s>>>(a);
      break;
    }
    case 2: {
      cudaFuncSetAttribute(k_paths_mixed<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      k_paths_mixed<2><<<grid, MIXED_THREADS, smem, s>>>(a);
      break;
    }
    default: {
      cudaFuncSetAttribute(k_paths_mixed<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      k_paths_mixed<3><<<grid, MIXED_THREADS, smem, s>>>(a);
      break;
    }
  }
  return cudaGetLastError();
}

int mixed_blocks_per_sm(int kind, size_t smem) {
  int nb = 0;
  switch (kind) {
    case 0: cudaFuncSetAttribute(k_paths_mixed<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_paths_mixed<0>, MIXED_THREADS, smem); break;
    case 1: cudaFuncSetAttribute(k_paths_mixed<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_paths_mixed<1>, MIXED_THREADS, smem); break;
    case 2: cudaFuncSetAttribute(k_paths_mixed<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_paths_mixed<2>, MIXED_THREADS, smem); break;
    default: cudaFuncSetAttribute(k_paths_mixed<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
             cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_paths_mixed<3>, MIXED_THREADS, smem); break;
  }
  return nb;
}

}  // namespace pdds
