// FP64 mode: the plain double-precision GPU form of the estimator.
//
// Same persistent work-item structure as the MIXED kernel, but every path
// quantity is FP64 and each stencil exit adds its exact RBF vector
// Y * r_j(X), r_j = exp(-|p_j - X|^2 / c^2), into per-side FP64 sums S_j in
// shared memory.  At the end of the item G_i = -(1/N) sum_j ipsi(j,i) S_j.
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
};

constexpr unsigned FULL = 0xffffffffu;

template <int KIND>
__global__ void __launch_bounds__(FP64_THREADS)
k_paths_fp64(const Fp64Args a) {
  extern __shared__ double Ssum[];  // [sum n] per-side RBF sums, then [sum n] local t
  __shared__ ItemSide64 s_side[4];
  __shared__ double s_rect[4];
  __shared__ int s_item, s_knot, s_path_end, s_nall;
  __shared__ unsigned s_next_path;
  __shared__ double s_red[FP64_THREADS / 32][2];
  __shared__ unsigned long long s_redi[FP64_THREADS / 32][3];
  const DevLayout& L = a.L;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const double h = a.h, sqrth = a.sqrth;

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
      s_next_path = (unsigned)(p0 + FP64_THREADS);
      const int st = L.knot_stencil[k];
      for (int q = 0; q < 4; q++) s_rect[q] = L.st_rect[4 * st + q];
      int off = 0;
      int64_t moff = L.st_map_off[st];
      for (int d = 0; d < 4; d++) {
        const int sd = L.st_side[4 * st + d];
        ItemSide64 is;
        is.glob = L.st_glob[4 * st + d];
        is.map_off = moff;
        if (sd < 0) {
          is.n = 0; is.orient = 0; is.s_off = off; is.origin = 0.0; is.inv_c2 = 0.0;
          is.t_off = 0; is.ipsi_off = 0;
        } else {
          const int sh = L.sd_shape[sd];
          is.n = L.sd_n[sd];
          is.orient = L.sd_orient[sd];
          is.s_off = off;
          is.origin = L.sd_origin[sd];
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
    double* tloc = Ssum + nall;
    for (int i = tid; i < nall; i += FP64_THREADS) Ssum[i] = 0.0;
    for (int d = 0; d < 4; d++)
      for (int i = tid; i < s_side[d].n; i += FP64_THREADS)
        tloc[s_side[d].s_off + i] = L.sh_t[s_side[d].t_off + i];
    __syncthreads();

    const double x0 = L.kx[knot], y0 = L.ky[knot];
    const double rect[4] = {s_rect[0], s_rect[1], s_rect[2], s_rect[3]};
    Coef<double> k0;
    coef_f64<KIND>(a.P, x0, y0, k0);
    const int chunk = item % a.chunks;
    unsigned path = (unsigned)(chunk * a.paths_per_chunk + tid);
    bool active = (int)path < path_end;
    double x = x0, y = y0, Y = 1.0, Z = 0.0, xi = 0.0;
    Coef<double> k = k0;
    unsigned step = 0;
    u32x4 blk;
    blk.v[0] = blk.v[1] = blk.v[2] = blk.v[3] = 0;
    double b = 0.0, bb = 0.0;
    unsigned long long nsteps = 0, nglob = 0, nsten = 0;
    while (__any_sync(FULL, active)) {
      if (!active) continue;
      if ((step & 1u) == 0) blk = path_block(a.seed, a.instance, (uint32_t)knot, path, step >> 1);
      const uint32_t ua = (step & 1u) ? blk.v[2] : blk.v[0];
      const uint32_t ub = (step & 1u) ? blk.v[3] : blk.v[1];
      const double u0 = u01_fp64(ua), u1 = u01_fp64(ub);
      const double rho = ::sqrt(-2.0 * ::log(u0));
      double sn, cs;
      sincospi(2.0 * u1, &sn, &cs);
      const double i0 = sqrth * (rho * cs), i1 = sqrth * (rho * sn);
      const double v0 = -(k.s00 * k.g0 + k.s10 * k.g1);
      const double v1 = -(k.s01 * k.g0 + k.s11 * k.g1);
      xi += Y * (v0 * i0 + v1 * i1);
      Z += k.f * Y * h;
      Y += k.c * Y * h;
      x += k.b0 * h + (k.s00 * i0 + k.s01 * i1);
      y += k.b1 * h + (k.s10 * i0 + k.s11 * i1);
      ++step;
      coef_f64<KIND>(a.P, x, y, k);
      double Ex, Ey, Nx, Ny;
      int onmask;
      const double dist = rect2d<double>(rect, x, y, Ex, Ey, Nx, Ny, onmask);
      const double w0 = Nx * k.s00 + Ny * k.s10, w1 = Nx * k.s01 + Ny * k.s11;
      const double thr = -0.5826 * ::sqrt(w0 * w0 + w1 * w1) * sqrth;
      const bool capped = step >= (unsigned)a.max_steps;
      if (dist < thr && !capped) continue;
      nsteps += step;
      if (capped && dist < thr) {
        atomicOr(a.err_flags, ERR_FLAG_STEP_LIMIT);
      } else {
        const int d = exit_side(onmask);
        const bool glob = ((onmask & 1) && s_side[0].glob) || ((onmask & 2) && s_side[1].glob) ||
                          ((onmask & 4) && s_side[2].glob) || ((onmask & 8) && s_side[3].glob);
        double val;
        if (glob) {
          val = Z + Y * u_f64<KIND>(a.P, Ex, Ey) + xi;
          ++nglob;
        } else {
          val = Z + xi;
          ++nsten;
          if (d < 0) {
            atomicOr(a.err_flags, ERR_FLAG_EXIT_SIDE);
          } else {
            const ItemSide64& is = s_side[d];
            const double s = (is.orient == 0 ? Ex : Ey) - is.origin;
            for (int j = 0; j < is.n; j++) {
              const double dt = tloc[is.s_off + j] - s;
              atomicAdd(Ssum + is.s_off + j, Y * ::exp(-(dt * dt) * is.inv_c2));
            }
          }
        }
        b += val;
        bb += val * val;
      }
      path = atomicAdd(&s_next_path, 1u);
      if ((int)path >= path_end) {
        active = false;
      } else {
        x = x0; y = y0; Y = 1.0; Z = 0.0; xi = 0.0; step = 0; k = k0;
      }
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
      atomicAdd(a.G + row0 + L.map_pos[m], -acc * a.inv_N);
    }
    __syncthreads();
  }
}

}  // namespace

#define PDDS_FP64_CASE(KK)                                                                        \
  case KK:                                                                                        \
    cudaFuncSetAttribute(k_paths_fp64<KK>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
    k_paths_fp64<KK><<<grid, FP64_THREADS, smem, s>>>(a);                                         \
    break;

cudaError_t launch_paths_fp64(const Fp64Args& a, int kind, int grid, size_t smem, cudaStream_t s) {
  switch (kind) {
    PDDS_FP64_CASE(0)
    PDDS_FP64_CASE(1)
    PDDS_FP64_CASE(2)
    PDDS_FP64_CASE(3)
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

int fp64_blocks_per_sm(int kind, size_t smem) {
  int nb = 0;
  switch (kind) {
    case 0: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_paths_fp64<0>, FP64_THREADS, smem); break;
    case 1: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_paths_fp64<1>, FP64_THREADS, smem); break;
    case 2: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_paths_fp64<2>, FP64_THREADS, smem); break;
    default: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_paths_fp64<3>, FP64_THREADS, smem); break;
  }
  return nb;
}

}  // namespace pdds
