// Interface solve (I + G) u = B in one launch: FP32 GMRES(m) under FP64
// iterative refinement, one thread-block cluster per system.
//
// The reference assembles the system with duplicate triplets summed and
// solves it with Eigen's BiCGSTAB (PDDAlgorithms/PDDSparseGM.cpp:3168-3246).
// Here each system (one interface system, or one instance of a batch) is
// owned by one cluster of up to 16 CTAs; the CTAs split its rows, keep their
// rows of the Arnoldi vector w in shared memory, and read the basis V and
// the iterate from global memory (L2).  Dot products are reduced inside each
// CTA, then across the cluster through distributed shared memory after a
// hardware cluster barrier; every CTA adds the per-CTA partials in the same
// order, so all CTAs hold bit-identical scalars and take the same branches.
// Nothing waits on a flag: the only synchronisation is __syncthreads and the
// cluster barrier, and every loop is bounded by max_iter / max_refine.
//
// The system's current Krylov vector (FP32) or iterate (FP64) is staged whole
// in each CTA's shared memory before a product, so the SpMV gathers come from
// shared memory and only the CSR rows stream from L2/HBM.
//
// Per Arnoldi step: FP32 SpMV of the CTA's rows, one classical Gram-Schmidt
// pass whose reduction also carries |w|^2 (the new norm follows from
// |w - V h|^2 = |w|^2 - |h|^2), and the Givens update of the Hessenberg
// column (FP32, replicated per CTA): two group barriers per step.  Lane
// partial sums are FP32; warp, CTA and cluster sums are two-float (hi + lo)
// sums in FP32 instructions (FP64 issues far slower on this GPU and, in the
// serial parts of a step, set its length).  The outer FP64
// residual b - (I + G) x uses the FP64 G, so the refined solution reaches the
// FP64 tolerance whatever the FP32 inner accuracy; the loss of orthogonality
// of a single pass only costs inner accuracy, which the refinement absorbs
// (on the 12x12/n43 system a re-orthogonalising second pass needed the same
// 120 Arnoldi steps and three barriers per step).
#include <cooperative_groups.h>

#include <algorithm>

#include "kernels.h"
#include "solve.h"

namespace cg = cooperative_groups;

namespace pdds {

namespace {

constexpr int CG_THREADS = 1024;
constexpr int CG_WARPS = CG_THREADS / 32;
constexpr int CG_MAXM = 40;
constexpr int CG_MAXV = CG_MAXM + 1;
constexpr int SPMV_U = 8;  // CSR entries per lane in flight in the FP32 product
static_assert(CG_MAXM == GMRES_CLUSTER_MAX_M, "restart bound");

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Two-float sums.  FP64 instructions issue at a small fraction of the FP32
// rate on this GPU (a warp-wide FP64 add holds its scheduler for tens of
// cycles), so the per-step reductions carry each value as an unevaluated
// sum hi + lo of two floats (Knuth's TwoSum, Dekker's product by FMA):
// about 48 significant bits with FP32 instructions only.
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
  const float s = a.x + b.x;
  const float bb = s - a.x;
  const float e = (a.x - (s - bb)) + (b.x - bb) + (a.y + b.y);
  const float hi = s + e;
  return make_float2(hi, e - (hi - s));
}
__device__ __forceinline__ float2 df_sq(float a) {  // a^2 exactly as hi + lo
  const float p = a * a;
  return make_float2(p, fmaf(a, a, -p));
}
__device__ __forceinline__ float2 df_from(double v) {
  const float hi = (float)v;
  return make_float2(hi, (float)(v - (double)hi));
}
__device__ __forceinline__ double df_val(float2 v) { return (double)v.x + (double)v.y; }
__device__ __forceinline__ float2 warp_sum_df(float2 v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float2 w = make_float2(__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o));
    v = df_add(v, w);
  }
  return v;
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// The CTAs that own one system: a thread-block cluster (hardware barrier,
// partials read through distributed shared memory), or the whole grid of a
// cooperative launch (a counting barrier in global memory whose wait is
// bounded, partials published in global memory).  reduce() sums the CTAs'
// partials slot[0 .. nv) in rank order into out in every CTA; sync() and
// reduce() return false only when a grid barrier timed out.
struct ClusterGroup {
  cg::cluster_group cl;
  __device__ ClusterGroup() : cl(cg::this_cluster()) {}
  __device__ unsigned rank() const { return cl.block_rank(); }
  __device__ unsigned size() const { return cl.num_blocks(); }
  __device__ int system() const { return (int)(blockIdx.x / cl.num_blocks()); }
  __device__ bool sync() {
    cl.sync();
    return true;
  }
  // one warp per value, lanes over ranks, a fixed shuffle tree: the same
  // order in every CTA
  __device__ bool reduce(float2* slot, int nv, float2* out, int) {
    cl.sync();
    const unsigned lane = threadIdx.x & 31, n = cl.num_blocks();
    for (int i = threadIdx.x >> 5; i < nv; i += CG_WARPS) {
      float2 s = make_float2(0.f, 0.f);
      for (unsigned rk = lane; rk < n; rk += 32) s = df_add(s, cl.map_shared_rank(slot, rk)[i]);
      s = warp_sum_df(s);
      if (lane == 0) out[i] = s;
    }
    __syncthreads();
    return true;
  }
};

constexpr unsigned GRID_SPIN_LIMIT = 1u << 24;  // ~1 s of polling

// The barrier is one arrival counter that only grows (zeroed before the
// launch): barrier b of the launch is complete when the counter reaches
// (b + 1) * gridDim.x, so the last CTA to arrive releases the others with its
// own arrival and nothing is reset.  The wait polls with acquire loads and
// gives up after GRID_SPIN_LIMIT polls.
struct GridGroup {
  unsigned* count;  // arrivals since the launch
  unsigned* err;    // ERR_FLAG_TIMEOUT on a wait that ran out
  double* gpart;    // [2][gridDim.x][CG_MAXV + 2] published partials
  unsigned limit;   // polls before a wait gives up
  __device__ unsigned rank() const { return blockIdx.x; }
  __device__ unsigned size() const { return gridDim.x; }
  __device__ int system() const { return 0; }
  __device__ bool sync() {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();  // the CTA's writes (ordered before this by the barrier) before the arrival
      const unsigned arrived = atomicAdd(count, 1u);
      const unsigned target = (arrived / gridDim.x + 1u) * gridDim.x;
      int ok = 1;
      unsigned spins = 0, cur;
      for (;;) {
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(cur) : "l"(count) : "memory");
        if ((int)(cur - target) >= 0) break;
        if (++spins > limit) {
          atomicOr(err, ERR_FLAG_TIMEOUT);
          ok = 0;
          break;
        }
        if (spins > 64) __nanosleep(16);
      }
      __threadfence();
      s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
  }
  // partials of all CTAs, 8 loads in flight per lane
  __device__ bool reduce(float2* slot, int nv, float2* out, int parity) {
    float2* part = reinterpret_cast<float2*>(gpart);
    float2* mine = part + ((size_t)parity * gridDim.x + blockIdx.x) * (CG_MAXV + 2);
    for (int i = threadIdx.x; i < nv; i += CG_THREADS) mine[i] = slot[i];
    const bool ok = sync();
    const unsigned lane = threadIdx.x & 31, n = gridDim.x;
    const float2* base = part + (size_t)parity * n * (CG_MAXV + 2);
    for (int i = threadIdx.x >> 5; i < nv; i += CG_WARPS) {
      float2 s = make_float2(0.f, 0.f);
      for (unsigned rk0 = lane; rk0 < n; rk0 += 32 * 8) {
        float2 t[8];
#pragma unroll
        for (int u = 0; u < 8; u++) {
          const unsigned rk = rk0 + 32u * u;
          t[u] = rk < n ? __ldcg(base + (size_t)rk * (CG_MAXV + 2) + i) : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < 8; u++) s = df_add(s, t[u]);
      }
      s = warp_sum_df(s);
      if (lane == 0) out[i] = s;
    }
    __syncthreads();
    return ok;
  }
};

template <class Group>
__device__ __forceinline__ void gmres_body(const ClusterGmresArgs& a, Group& grp) {
  const unsigned crank = grp.rank(), csize = grp.size();
  const int sys = grp.system();  // uniform within the group
  if (sys >= a.n_sys) return;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int R0 = a.sys_row0[sys], R1 = a.sys_row0[sys + 1];
  const int nr = R1 - R0;
  const int per = (nr + (int)csize - 1) / (int)csize;
  const int r0 = min(R1, R0 + (int)crank * per), r1 = min(R1, r0 + per);
  const int nown = r1 - r0;
  const int m = a.m;
  const int64_t K = a.K;

  extern __shared__ __align__(16) unsigned char s_dyn[];
  float* s_w = reinterpret_cast<float*>(s_dyn);  // own rows of the Arnoldi vector
  const size_t wbytes = ((size_t)per * sizeof(float) + 15) & ~(size_t)15;
  float* s_vf = reinterpret_cast<float*>(s_dyn + wbytes);    // system vector, FP32
  double* s_vd = reinterpret_cast<double*>(s_dyn + wbytes);  // system iterate, FP64
  __shared__ float2 s_slot[2][CG_MAXV + 2];
  __shared__ float2 s_red[CG_MAXV + 2];
  __shared__ float s_H[CG_MAXV * CG_MAXM];  // column j at s_H[j * (m + 1)]
  __shared__ float s_cs[CG_MAXM], s_sn[CG_MAXM], s_g[CG_MAXV], s_y[CG_MAXM];
  __shared__ float2 s_bsum[CG_WARPS];
  __shared__ int s_flag[2];
  __shared__ float s_hn, s_inv;
  __shared__ double s_beta[2];
  int parity = 0;
  static_assert(CG_WARPS == 32, "one warp sums the warps' partials");

  bool alive = true;  // false once a grid barrier timed out: the CTA winds down
  // group all-reduce of s_slot[parity][0 .. nv) into s_red
  auto allreduce = [&](int nv) {
    alive = grp.reduce(&s_slot[parity][0], nv, s_red, parity) && alive;
    parity ^= 1;
  };
  // CTA sum of one per-thread value into s_slot[parity][0]
  auto block_sum = [&](float2 v) {
    v = warp_sum_df(v);
    if (lane == 0) s_bsum[warp] = v;
    __syncthreads();
    if (warp == 0) {
      const float2 t = warp_sum_df(s_bsum[lane]);
      if (lane == 0) s_slot[parity][0] = t;
    }
    __syncthreads();
  };
  // dots of the own rows of w with V[0 .. nv): one warp per basis vector
  auto basis_dots = [&](int nv) {
    for (int i = warp; i < nv; i += CG_WARPS) {
      const float* Vi = a.V + (int64_t)i * K + r0;
      float acc = 0.f;
      for (int q = lane; q < nown; q += 32 * 4) {
        float t[4];
#pragma unroll
        for (int u = 0; u < 4; u++) t[u] = q + 32 * u < nown ? __ldcg(Vi + q + 32 * u) : 0.f;
#pragma unroll
        for (int u = 0; u < 4; u++)
          if (q + 32 * u < nown) acc = fmaf(t[u], s_w[q + 32 * u], acc);
      }
      const float2 t = warp_sum_df(make_float2(acc, 0.f));
      if (lane == 0) s_slot[parity][i] = t;
    }
    __syncthreads();
  };

  // ||b||^2 and x = 0
  {
    double bb = 0.0;
    for (int r = r0 + tid; r < r1; r += CG_THREADS) {
      const double v = a.b[r];
      bb += v * v;
      a.x[r] = 0.0;
    }
    block_sum(df_from(bb));
    allreduce(1);
  }
  const double bnorm2 = df_val(s_red[0]);
  int total = 0, ref = 0;
  double rr = bnorm2;
  if (bnorm2 > 0.0 && alive) {
    const double tol2 = a.tol * a.tol * bnorm2;
    for (ref = 0;; ref++) {
      // FP64 residual r = b - x - G x of the own rows (x complete after the barrier above / below)
      for (int i0 = tid; i0 < nr; i0 += CG_THREADS * 4) {
        double t[4];
#pragma unroll
        for (int u = 0; u < 4; u++) t[u] = i0 + CG_THREADS * u < nr ? __ldcg(a.x + R0 + i0 + CG_THREADS * u) : 0.0;
#pragma unroll
        for (int u = 0; u < 4; u++)
          if (i0 + CG_THREADS * u < nr) s_vd[i0 + CG_THREADS * u] = t[u];
      }
      __syncthreads();
      double prr = 0.0;
      for (int r = r0 + warp; r < r1; r += CG_WARPS) {
        double acc0 = 0.0, acc1 = 0.0;
        const int64_t e1 = a.row_ptr[r + 1];
        for (int64_t e = a.row_ptr[r] + lane; e < e1; e += 32 * 4) {
          double v[4];
          int c[4];
#pragma unroll
          for (int u = 0; u < 4; u++) {
            const bool in = e + 32 * u < e1;
            v[u] = in ? __ldg(a.val64 + e + 32 * u) : 0.0;
            c[u] = in ? __ldg(a.col + e + 32 * u) - R0 : 0;
            if (!idx_ok(c[u], nr, a.err_flags)) c[u] = 0;
          }
          acc0 += v[0] * s_vd[c[0]];
          acc1 += v[1] * s_vd[c[1]];
          acc0 += v[2] * s_vd[c[2]];
          acc1 += v[3] * s_vd[c[3]];
        }
        const double acc = warp_sum(acc0 + acc1);
        if (lane == 0) {
          const double rv = a.b[r] - s_vd[r - R0] - acc;
          a.r64[r] = rv;
          prr += rv * rv;
        }
      }
      block_sum(df_from(prr));
      allreduce(1);
      rr = df_val(s_red[0]);
      if (!(rr > tol2) || ref >= a.max_refine || total >= a.max_iter || !alive) break;
      // v0 = r / |r|
      if (tid == 0) {
        s_beta[0] = sqrt(rr);
        s_beta[1] = 1.0 / s_beta[0];
        for (int i = 0; i <= m; i++) s_g[i] = 0.f;
        s_g[0] = 1.f;
      }
      __syncthreads();
      const double beta = s_beta[0], ibeta = s_beta[1];
      for (int r = r0 + tid; r < r1; r += CG_THREADS) a.V[r] = (float)(a.r64[r] * ibeta);
      int jdim = 0;
      for (int j = 0; j < m; j++) {
        alive = grp.sync() && alive;  // V[j] complete in every CTA
        if (!alive) break;
        // w = (I + G32) V[j], own rows
        const float* vj = a.V + (int64_t)j * K + R0;
        for (int i0 = tid; i0 < nr; i0 += CG_THREADS * 8) {
          float t[8];
#pragma unroll
          for (int u = 0; u < 8; u++) t[u] = i0 + CG_THREADS * u < nr ? __ldcg(vj + i0 + CG_THREADS * u) : 0.f;
#pragma unroll
          for (int u = 0; u < 8; u++)
            if (i0 + CG_THREADS * u < nr) s_vf[i0 + CG_THREADS * u] = t[u];
        }
        __syncthreads();
        // one warp per row, SPMV_U entries per lane loaded before any is used
        for (int r = r0 + warp; r < r1; r += CG_WARPS) {
          float acc0 = 0.f, acc1 = 0.f;
          const int64_t e1 = a.row_ptr[r + 1];
          for (int64_t e = a.row_ptr[r] + lane; e < e1; e += 32 * SPMV_U) {
            float v[SPMV_U];
            int c[SPMV_U];
#pragma unroll
            for (int u = 0; u < SPMV_U; u++) {
              const bool in = e + 32 * u < e1;
              v[u] = in ? __ldg(a.val32 + e + 32 * u) : 0.f;
              c[u] = in ? __ldg(a.col + e + 32 * u) - R0 : 0;
              if (!idx_ok(c[u], nr, a.err_flags)) c[u] = 0;
            }
#pragma unroll
            for (int u = 0; u < SPMV_U; u += 2) {
              acc0 = fmaf(v[u], s_vf[c[u]], acc0);
              acc1 = fmaf(v[u + 1], s_vf[c[u + 1]], acc1);
            }
          }
          float acc = acc0 + acc1;
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
          if (lane == 0) s_w[r - r0] = s_vf[r - R0] + acc;
        }
        __syncthreads();
        const int nv = j + 1;
        // h = V^T w and |w|^2 in one reduction; then w -= V h and
        // |w - V h|^2 = |w|^2 - |h|^2 (V orthonormal)
        {
          float2 pn = make_float2(0.f, 0.f);
          for (int r = tid; r < nown; r += CG_THREADS) pn = df_add(pn, df_sq(s_w[r]));
          pn = warp_sum_df(pn);
          if (lane == 0) s_bsum[warp] = pn;
        }
        basis_dots(nv);  // ends with __syncthreads: s_bsum complete
        if (warp == 0) {
          const float2 t = warp_sum_df(s_bsum[lane]);
          if (lane == 0) s_slot[parity][nv] = t;
        }
        __syncthreads();
        allreduce(nv + 1);
        // w -= V h over the own rows; the last warp then forms h_{j+1,j}
        // and, in one lane, the Givens update of the Hessenberg column (FP32)
        for (int r = tid; r < nown; r += CG_THREADS) {
          float acc = s_w[r];
#pragma unroll 4
          for (int i = 0; i < nv; i++) acc = fmaf(-s_red[i].x, __ldcg(a.V + (int64_t)i * K + r0 + r), acc);
          s_w[r] = acc;
        }
        if (warp == CG_WARPS - 1) {
          float2 hh = make_float2(0.f, 0.f);
          for (int i = lane; i < nv; i += 32) {
            float2 t = df_sq(s_red[i].x);
            t.y = fmaf(2.f * s_red[i].x, s_red[i].y, t.y);
            hh = df_add(hh, t);
          }
          hh = warp_sum_df(hh);
          if (lane == 0) {
            const float2 d = df_add(s_red[nv], make_float2(-hh.x, -hh.y));
            const float hn = sqrtf(fmaxf(d.x + d.y, 0.f));
            float* col = s_H + j * (m + 1);
            for (int i = 0; i <= j; i++) col[i] = s_red[i].x;
            col[j + 1] = hn;
            for (int i = 0; i < j; i++) {
              const float p = col[i], q = col[i + 1];
              col[i] = s_cs[i] * p + s_sn[i] * q;
              col[i + 1] = -s_sn[i] * p + s_cs[i] * q;
            }
            const float p = col[j], q = col[j + 1];
            const float rho = sqrtf(p * p + q * q);
            s_cs[j] = rho > 0.f ? p / rho : 1.f;
            s_sn[j] = rho > 0.f ? q / rho : 0.f;
            col[j] = rho;
            col[j + 1] = 0.f;
            s_g[j + 1] = -s_sn[j] * s_g[j];
            s_g[j] = s_cs[j] * s_g[j];
            s_flag[0] = (fabsf(s_g[j + 1]) <= (float)a.inner_tol || !(hn > 0.f)) ? 1 : 0;
            s_hn = hn;
            s_inv = hn > 0.f ? 1.f / hn : 0.f;
          }
        }
        __syncthreads();
        ++total;
        jdim = j + 1;
        if (s_hn > 0.f && j + 1 < m) {
          const float inv = s_inv;
          float* vn = a.V + (int64_t)(j + 1) * K;
          for (int r = tid; r < nown; r += CG_THREADS) vn[r0 + r] = s_w[r] * inv;
        }
        if (s_flag[0] || total >= a.max_iter || !alive) break;
      }
      // y = H^-1 g (upper triangular, FP32), x += beta V y (FP64 iterate)
      if (tid == 0) {
        for (int i = jdim - 1; i >= 0; i--) {
          float sacc = s_g[i];
          for (int k = i + 1; k < jdim; k++) sacc -= s_H[k * (m + 1) + i] * s_y[k];
          const float d = s_H[i * (m + 1) + i];
          s_y[i] = d != 0.f ? sacc / d : 0.f;
        }
      }
      __syncthreads();
      for (int r = r0 + tid; r < r1; r += CG_THREADS) {
        float acc = 0.f;
#pragma unroll 4
        for (int i = 0; i < jdim; i++) acc = fmaf(s_y[i], __ldcg(a.V + (int64_t)i * K + r), acc);
        a.x[r] += beta * (double)acc;
      }
      alive = grp.sync() && alive;  // x complete before the next residual
    }
  }
  if (alive) grp.sync();  // no CTA leaves while another may still read its shared memory
  if (crank == 0 && tid == 0) {
    a.out_iters[sys] = total;
    a.out_refines[sys] = ref;
    a.out_relres[sys] = !alive ? -1.0 : (bnorm2 > 0.0 ? sqrt(rr / bnorm2) : 0.0);
    if (a.out_t_end) a.out_t_end[sys] = global_ns();
  }
}

// Pipelined GMRES(m): one group barrier per Arnoldi step.
//
// The Krylov space of I + G is the one of G, so the Arnoldi process runs on
// G, and the Hessenberg matrix of I + G is the one of G plus the identity.
// Besides the basis V it keeps Z = G V.  Step j (after the barrier that ends
// step j - 1, at which t_j = G v_{j-1} = Z[j-1] is complete in every CTA and
// its dots with v_0 .. v_{j-1} and |t_j|^2 are reduced) forms column j - 1
// of the Hessenberg matrix, h_i = v_i . t_j and beta = |t_j - V h|, and then,
// for its own rows:
//   the product a = G t_j (t_j staged whole in shared memory),
//   v_j = (t_j - sum_i h_i v_i) / beta  and  z_j = (a - sum_i h_i z_i) / beta,
// since G v_j = (G t_j - sum_i h_i G v_i) / beta; z_j is the next t.  Its
// dots with v_0 .. v_j and |z_j|^2 go into the step's one reduction, whose
// barrier also publishes V[j] and Z[j].  The classical two-barrier step
// needs the reduced h before it can form v_j and a second barrier before the
// product of v_j; here the product is applied to t_j, which is complete one
// barrier earlier.  The recurrence for z_j carries the rounding of earlier
// steps (the Arnoldi relation holds only to that accuracy): the FP64
// residual of every refinement step is formed from the FP64 G, so that
// error costs inner iterations, not accuracy.
template <class Group>
__device__ __forceinline__ void gmres_body_p1(const ClusterGmresArgs& a, Group& grp) {
  const unsigned crank = grp.rank(), csize = grp.size();
  const int sys = grp.system();
  if (sys >= a.n_sys) return;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int R0 = a.sys_row0[sys], R1 = a.sys_row0[sys + 1];
  const int nr = R1 - R0;
  const int per = (nr + (int)csize - 1) / (int)csize;
  const int r0 = min(R1, R0 + (int)crank * per), r1 = min(R1, r0 + per);
  const int nown = r1 - r0;
  const int m = a.m;
  const int64_t K = a.K;

  extern __shared__ __align__(16) unsigned char s_dyn[];
  float* s_w = reinterpret_cast<float*>(s_dyn);  // own rows of the product G t
  const size_t wbytes = ((size_t)per * sizeof(float) + 15) & ~(size_t)15;
  float* s_vf = reinterpret_cast<float*>(s_dyn + wbytes);    // system vector, FP32
  double* s_vd = reinterpret_cast<double*>(s_dyn + wbytes);  // system iterate, FP64
  __shared__ float2 s_slot[2][CG_MAXV + 2];
  __shared__ float2 s_red[CG_MAXV + 2];
  __shared__ float s_H[CG_MAXV * CG_MAXM];  // column j at s_H[j * (m + 1)]
  __shared__ float s_cs[CG_MAXM], s_sn[CG_MAXM], s_g[CG_MAXV], s_y[CG_MAXM];
  __shared__ float s_h[CG_MAXV];            // h_i of the current column (G part)
  __shared__ float2 s_bsum[CG_WARPS];
  __shared__ int s_flag[2];
  __shared__ float s_inv;
  __shared__ double s_beta[2];
  int parity = 0;

  bool alive = true;
  auto allreduce = [&](int nv) {
    alive = grp.reduce(&s_slot[parity][0], nv, s_red, parity) && alive;
    parity ^= 1;
  };
  auto block_sum = [&](float2 v) {
    v = warp_sum_df(v);
    if (lane == 0) s_bsum[warp] = v;
    __syncthreads();
    if (warp == 0) {
      const float2 t = warp_sum_df(s_bsum[lane]);
      if (lane == 0) s_slot[parity][0] = t;
    }
    __syncthreads();
  };
  // own-row dots of y (global, own rows at y + r0) with V[0 .. nv) into
  // s_slot[parity][0 .. nv) and |y|^2 into s_slot[parity][nv]
  auto dots_and_norm = [&](const float* y, int nv) {
    {
      float2 pn = make_float2(0.f, 0.f);
      for (int r = tid; r < nown; r += CG_THREADS) pn = df_add(pn, df_sq(__ldcg(y + r0 + r)));
      pn = warp_sum_df(pn);
      if (lane == 0) s_bsum[warp] = pn;
    }
    for (int i = warp; i < nv; i += CG_WARPS) {
      const float* Vi = a.V + (int64_t)i * K + r0;
      float acc = 0.f;
      for (int q = lane; q < nown; q += 32) acc = fmaf(__ldcg(Vi + q), __ldcg(y + r0 + q), acc);
      const float2 t = warp_sum_df(make_float2(acc, 0.f));
      if (lane == 0) s_slot[parity][i] = t;
    }
    __syncthreads();
    if (warp == 0) {
      const float2 t = warp_sum_df(s_bsum[lane]);
      if (lane == 0) s_slot[parity][nv] = t;
    }
    __syncthreads();
  };
  // s_w = G x over the own rows, x (FP32, the whole system vector) staged first
  auto spmv_g = [&](const float* x) {
    const float* xs = x + R0;
    for (int i0 = tid; i0 < nr; i0 += CG_THREADS * 8) {
      float t[8];
#pragma unroll
      for (int u = 0; u < 8; u++) t[u] = i0 + CG_THREADS * u < nr ? __ldcg(xs + i0 + CG_THREADS * u) : 0.f;
#pragma unroll
      for (int u = 0; u < 8; u++)
        if (i0 + CG_THREADS * u < nr) s_vf[i0 + CG_THREADS * u] = t[u];
    }
    __syncthreads();
    for (int r = r0 + warp; r < r1; r += CG_WARPS) {
      float acc0 = 0.f, acc1 = 0.f;
      const int64_t e1 = a.row_ptr[r + 1];
      for (int64_t e = a.row_ptr[r] + lane; e < e1; e += 32 * SPMV_U) {
        float v[SPMV_U];
        int c[SPMV_U];
#pragma unroll
        for (int u = 0; u < SPMV_U; u++) {
          const bool in = e + 32 * u < e1;
          v[u] = in ? __ldg(a.val32 + e + 32 * u) : 0.f;
          c[u] = in ? __ldg(a.col + e + 32 * u) - R0 : 0;
          if (!idx_ok(c[u], nr, a.err_flags)) c[u] = 0;
        }
#pragma unroll
        for (int u = 0; u < SPMV_U; u += 2) {
          acc0 = fmaf(v[u], s_vf[c[u]], acc0);
          acc1 = fmaf(v[u + 1], s_vf[c[u + 1]], acc1);
        }
      }
      float acc = acc0 + acc1;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) s_w[r - r0] = acc;
    }
    __syncthreads();
  };

  // ||b||^2 and x = 0
  {
    double bb = 0.0;
    for (int r = r0 + tid; r < r1; r += CG_THREADS) {
      const double v = a.b[r];
      bb += v * v;
      a.x[r] = 0.0;
    }
    block_sum(df_from(bb));
    allreduce(1);
  }
  const double bnorm2 = df_val(s_red[0]);
  int total = 0, ref = 0;
  double rr = bnorm2;
  if (bnorm2 > 0.0 && alive) {
    const double tol2 = a.tol * a.tol * bnorm2;
    for (ref = 0;; ref++) {
      // FP64 residual r = b - x - G x of the own rows
      for (int i0 = tid; i0 < nr; i0 += CG_THREADS * 4) {
        double t[4];
#pragma unroll
        for (int u = 0; u < 4; u++) t[u] = i0 + CG_THREADS * u < nr ? __ldcg(a.x + R0 + i0 + CG_THREADS * u) : 0.0;
#pragma unroll
        for (int u = 0; u < 4; u++)
          if (i0 + CG_THREADS * u < nr) s_vd[i0 + CG_THREADS * u] = t[u];
      }
      __syncthreads();
      double prr = 0.0;
      for (int r = r0 + warp; r < r1; r += CG_WARPS) {
        double acc0 = 0.0, acc1 = 0.0;
        const int64_t e1 = a.row_ptr[r + 1];
        for (int64_t e = a.row_ptr[r] + lane; e < e1; e += 32 * 4) {
          double v[4];
          int c[4];
#pragma unroll
          for (int u = 0; u < 4; u++) {
            const bool in = e + 32 * u < e1;
            v[u] = in ? __ldg(a.val64 + e + 32 * u) : 0.0;
            c[u] = in ? __ldg(a.col + e + 32 * u) - R0 : 0;
            if (!idx_ok(c[u], nr, a.err_flags)) c[u] = 0;
          }
          acc0 += v[0] * s_vd[c[0]];
          acc1 += v[1] * s_vd[c[1]];
          acc0 += v[2] * s_vd[c[2]];
          acc1 += v[3] * s_vd[c[3]];
        }
        const double acc = warp_sum(acc0 + acc1);
        if (lane == 0) {
          const double rv = a.b[r] - s_vd[r - R0] - acc;
          a.r64[r] = rv;
          prr += rv * rv;
        }
      }
      block_sum(df_from(prr));
      allreduce(1);
      rr = df_val(s_red[0]);
      if (!(rr > tol2) || ref >= a.max_refine || total >= a.max_iter || !alive) break;
      if (tid == 0) {
        s_beta[0] = sqrt(rr);
        s_beta[1] = 1.0 / s_beta[0];
        for (int i = 0; i <= m; i++) s_g[i] = 0.f;
        s_g[0] = 1.f;
      }
      __syncthreads();
      const double beta = s_beta[0], ibeta = s_beta[1];
      // v0 = r / |r| over the own rows; the next group barrier publishes it
      for (int r = r0 + tid; r < r1; r += CG_THREADS) a.V[r] = (float)(a.r64[r] * ibeta);
      alive = grp.sync() && alive;
      int jdim = 0;
      for (int j = 0;; j++) {
        if (j >= 1) {
          // column j - 1 from the reduced dots of t_j (s_red[0 .. j), |t_j|^2
          // at s_red[j]): h_i, beta = |t_j - V h|, Givens update (one lane)
          if (warp == CG_WARPS - 1) {
            float2 hh = make_float2(0.f, 0.f);
            for (int i = lane; i < j; i += 32) {
              float2 t = df_sq(s_red[i].x);
              t.y = fmaf(2.f * s_red[i].x, s_red[i].y, t.y);
              hh = df_add(hh, t);
              s_h[i] = s_red[i].x;
            }
            hh = warp_sum_df(hh);
            if (lane == 0) {
              const float2 d = df_add(s_red[j], make_float2(-hh.x, -hh.y));
              const float hn = sqrtf(fmaxf(d.x + d.y, 0.f));
              float* col = s_H + (j - 1) * (m + 1);
              for (int i = 0; i < j; i++) col[i] = s_red[i].x;
              col[j - 1] += 1.f;  // the identity of I + G
              col[j] = hn;
              for (int i = 0; i < j - 1; i++) {
                const float p = col[i], q = col[i + 1];
                col[i] = s_cs[i] * p + s_sn[i] * q;
                col[i + 1] = -s_sn[i] * p + s_cs[i] * q;
              }
              const float p = col[j - 1], q = col[j];
              const float rho = sqrtf(p * p + q * q);
              s_cs[j - 1] = rho > 0.f ? p / rho : 1.f;
              s_sn[j - 1] = rho > 0.f ? q / rho : 0.f;
              col[j - 1] = rho;
              col[j] = 0.f;
              s_g[j] = -s_sn[j - 1] * s_g[j - 1];
              s_g[j - 1] = s_cs[j - 1] * s_g[j - 1];
              s_flag[0] = (fabsf(s_g[j]) <= (float)a.inner_tol || !(hn > 0.f)) ? 1 : 0;
              s_inv = hn > 0.f ? 1.f / hn : 0.f;
            }
          }
          __syncthreads();
          jdim = j;
          if (s_flag[0] || j >= m || total >= a.max_iter || !alive) break;
        }
        // a = G t_j (t_0 = v_0)
        const float* tj = j == 0 ? a.V : a.Z + (int64_t)(j - 1) * K;
        spmv_g(tj);
        float* vj = a.V + (int64_t)j * K;
        float* zj = a.Z + (int64_t)j * K;
        if (j == 0) {
          for (int r = tid; r < nown; r += CG_THREADS) zj[r0 + r] = s_w[r];
        } else {
          // v_j and z_j of the own rows: the j basis terms of a row are split
          // over pp lanes of one warp (a CTA has a few dozen rows and 1024
          // threads: one thread per row would wait on j dependent loads)
          const float inv = s_inv;
          int pp = 1;
          while (pp < 32 && pp < j && 2 * pp * nown <= CG_THREADS) pp *= 2;
          const int rows_w = 32 / pp, part = lane & (pp - 1);
          for (int base = warp * rows_w; base < nown; base += CG_WARPS * rows_w) {
            const int r = base + lane / pp;
            float v = 0.f, z = 0.f;
            if (r < nown) {
              for (int i = part; i < j; i += pp) {
                const float hi = s_h[i];
                v = fmaf(-hi, __ldcg(a.V + (int64_t)i * K + r0 + r), v);
                z = fmaf(-hi, __ldcg(a.Z + (int64_t)i * K + r0 + r), z);
              }
            }
            for (int o = pp >> 1; o > 0; o >>= 1) {
              v += __shfl_xor_sync(0xffffffffu, v, o);
              z += __shfl_xor_sync(0xffffffffu, z, o);
            }
            if (r < nown && part == 0) {
              vj[r0 + r] = (__ldcg(tj + r0 + r) + v) * inv;
              zj[r0 + r] = (s_w[r] + z) * inv;
            }
          }
          __syncthreads();
        }
        // dots of t_{j+1} = z_j with v_0 .. v_j and |z_j|^2, one reduction
        // (its barrier also publishes V[j] and Z[j])
        __syncthreads();
        dots_and_norm(zj, j + 1);
        allreduce(j + 2);
        ++total;
      }
      // y = H^-1 g (upper triangular, FP32), x += beta V y (FP64 iterate)
      if (tid == 0) {
        for (int i = jdim - 1; i >= 0; i--) {
          float sacc = s_g[i];
          for (int k = i + 1; k < jdim; k++) sacc -= s_H[k * (m + 1) + i] * s_y[k];
          const float d = s_H[i * (m + 1) + i];
          s_y[i] = d != 0.f ? sacc / d : 0.f;
        }
      }
      __syncthreads();
      for (int r = r0 + tid; r < r1; r += CG_THREADS) {
        float acc = 0.f;
#pragma unroll 4
        for (int i = 0; i < jdim; i++) acc = fmaf(s_y[i], __ldcg(a.V + (int64_t)i * K + r), acc);
        a.x[r] += beta * (double)acc;
      }
      alive = grp.sync() && alive;  // x complete before the next residual
    }
  }
  if (alive) grp.sync();  // no CTA leaves while another may still read its shared memory
  if (crank == 0 && tid == 0) {
    a.out_iters[sys] = total;
    a.out_refines[sys] = ref;
    a.out_relres[sys] = !alive ? -1.0 : (bnorm2 > 0.0 ? sqrt(rr / bnorm2) : 0.0);
    if (a.out_t_end) a.out_t_end[sys] = global_ns();
  }
}

__global__ void __launch_bounds__(CG_THREADS, 1) k_gmres_cluster(const ClusterGmresArgs a) {
  ClusterGroup grp;
  if (a.Z) gmres_body_p1(a, grp);
  else gmres_body(a, grp);
}

// One system over the whole grid (cooperative launch, one CTA per SM).
__global__ void __launch_bounds__(CG_THREADS, 1) k_gmres_grid(const ClusterGmresArgs a, unsigned* bar,
                                                              unsigned* err, double* gpart) {
  GridGroup grp{bar, err, gpart, a.spin_limit ? a.spin_limit : GRID_SPIN_LIMIT};
  if (a.Z) gmres_body_p1(a, grp);
  else gmres_body(a, grp);
}

__global__ void k_stamp(unsigned long long* t) { *t = global_ns(); }

}  // namespace

cudaError_t launch_stamp(unsigned long long* t, cudaStream_t s) {
  k_stamp<<<1, 1, 0, s>>>(t);
  return cudaGetLastError();
}

size_t gmres_cluster_smem(int max_rows, int cluster) {
  const int per = (max_rows + cluster - 1) / cluster;
  return (((size_t)per * sizeof(float) + 15) & ~(size_t)15) + (size_t)max_rows * sizeof(double);
}

int gmres_cluster_pick(int max_rows) {
  static bool init = false;
  if (!init) {
    cudaFuncSetAttribute(k_gmres_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaFuncSetAttribute(k_gmres_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CG_SMEM_CAP);
    init = true;
  }
  // about 512 rows per CTA, at most 16 CTAs, and a cluster the device can place
  int want = std::max(1, std::min(16, (max_rows + 511) / 512));
  for (int cs = want; cs >= 1; cs--) {
    const size_t smem = gmres_cluster_smem(max_rows, cs);
    if (smem > CG_SMEM_CAP) return 0;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(cs, 1, 1);
    cfg.blockDim = dim3(CG_THREADS, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int ncl = 0;
    if (cudaOccupancyMaxActiveClusters(&ncl, k_gmres_cluster, &cfg) == cudaSuccess && ncl > 0) return cs;
    cudaGetLastError();
  }
  return 0;
}

int gmres_grid_blocks(int max_rows) {
  static int sms = -1;
  if (sms < 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (!coop) sms = 0;
    cudaFuncSetAttribute(k_gmres_grid, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CG_SMEM_CAP);
  }
  if (sms <= 0) return 0;
  const size_t smem = gmres_cluster_smem(max_rows, sms);
  if (smem > CG_SMEM_CAP) return 0;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gmres_grid, CG_THREADS, smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return per_sm >= 1 ? sms : 0;
}

cudaError_t launch_gmres_grid(const ClusterGmresArgs& a, int blocks, int max_rows, unsigned* bar, unsigned* err,
                              double* gpart, cudaStream_t s) {
  if (a.n_sys != 1 || a.m < 2 || a.m > CG_MAXM || blocks < 1) return cudaErrorInvalidValue;
  const size_t smem = gmres_cluster_smem(max_rows, blocks);
  if (smem > CG_SMEM_CAP) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  ClusterGmresArgs aa = a;
  void* args[] = {&aa, &bar, &err, &gpart};
  return cudaLaunchCooperativeKernel((const void*)k_gmres_grid, dim3(blocks), dim3(CG_THREADS), args, smem, s);
}

cudaError_t launch_gmres_cluster(const ClusterGmresArgs& a, int cluster, int max_rows, cudaStream_t s) {
  if (a.m < 2 || a.m > CG_MAXM || cluster < 1 || cluster > 16) return cudaErrorInvalidValue;
  const size_t smem = gmres_cluster_smem(max_rows, cluster);
  if (smem > CG_SMEM_CAP) return cudaErrorInvalidValue;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = cluster;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3((unsigned)(a.n_sys * cluster), 1, 1);
  cfg.blockDim = dim3(CG_THREADS, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_gmres_cluster, a);
}

}  // namespace pdds
