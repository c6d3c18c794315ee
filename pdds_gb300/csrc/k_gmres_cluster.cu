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
// column (FP64, replicated per CTA): two group barriers per step.  Lane
// partial sums are FP32; warp, CTA and cluster sums are FP64.  The outer FP64
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
static_assert(CG_MAXM == GMRES_CLUSTER_MAX_M, "restart bound");

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
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
  __device__ bool reduce(double* slot, int nv, double* out, int) {
    cl.sync();
    const unsigned lane = threadIdx.x & 31, n = cl.num_blocks();
    for (int i = threadIdx.x >> 5; i < nv; i += CG_WARPS) {
      double s = 0.0;
      for (unsigned rk = lane; rk < n; rk += 32) s += cl.map_shared_rank(slot, rk)[i];
      s = warp_sum(s);
      if (lane == 0) out[i] = s;
    }
    __syncthreads();
    return true;
  }
};

constexpr unsigned GRID_SPIN_LIMIT = 1u << 24;  // ~1 s of polling

struct GridGroup {
  unsigned* count;  // arrivals at the current barrier (zeroed before the launch)
  unsigned* gen;    // barrier generation
  unsigned* err;    // ERR_FLAG_TIMEOUT on a wait that ran out
  double* gpart;    // [2][gridDim.x][CG_MAXV + 2] published partials
  __device__ unsigned rank() const { return blockIdx.x; }
  __device__ unsigned size() const { return gridDim.x; }
  __device__ int system() const { return 0; }
  __device__ bool sync() {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
      volatile unsigned* vg = gen;
      const unsigned g = *vg;
      __threadfence();
      int ok = 1;
      if (atomicAdd(count, 1u) == gridDim.x - 1) {
        atomicExch(count, 0u);
        __threadfence();
        atomicAdd(gen, 1u);
      } else {
        unsigned spins = 0;
        while (*vg == g) {
          if (++spins > GRID_SPIN_LIMIT) {
            atomicOr(err, ERR_FLAG_TIMEOUT);
            ok = 0;
            break;
          }
          __nanosleep(32);
        }
      }
      __threadfence();
      s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
  }
  __device__ bool reduce(double* slot, int nv, double* out, int parity) {
    double* mine = gpart + ((size_t)parity * gridDim.x + blockIdx.x) * (CG_MAXV + 2);
    for (int i = threadIdx.x; i < nv; i += CG_THREADS) mine[i] = slot[i];
    const bool ok = sync();
    const unsigned lane = threadIdx.x & 31;
    for (int i = threadIdx.x >> 5; i < nv; i += CG_WARPS) {
      double s = 0.0;
      for (unsigned rk = lane; rk < gridDim.x; rk += 32)
        s += __ldcg(gpart + ((size_t)parity * gridDim.x + rk) * (CG_MAXV + 2) + i);
      s = warp_sum(s);
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
  __shared__ double s_slot[2][CG_MAXV + 2];
  __shared__ double s_red[CG_MAXV + 2];
  __shared__ double s_h[CG_MAXV];
  __shared__ double s_H[CG_MAXV * CG_MAXM];  // column j at s_H[j * (m + 1)]
  __shared__ double s_cs[CG_MAXM], s_sn[CG_MAXM], s_g[CG_MAXV], s_y[CG_MAXM];
  __shared__ double s_bsum[CG_WARPS][2];
  __shared__ int s_flag[2];
  __shared__ double s_hn;
  int parity = 0;

  bool alive = true;  // false once a grid barrier timed out: the CTA winds down
  // group all-reduce of s_slot[parity][0 .. nv) into s_red
  auto allreduce = [&](int nv) {
    alive = grp.reduce(&s_slot[parity][0], nv, s_red, parity) && alive;
    parity ^= 1;
  };
  // CTA sum of up to two per-thread values into s_slot[parity][0..1]
  auto block_sum2 = [&](double v0, double v1) {
    v0 = warp_sum(v0);
    v1 = warp_sum(v1);
    if (lane == 0) { s_bsum[warp][0] = v0; s_bsum[warp][1] = v1; }
    __syncthreads();
    if (tid == 0) {
      double t0 = 0.0, t1 = 0.0;
      for (int q = 0; q < CG_WARPS; q++) { t0 += s_bsum[q][0]; t1 += s_bsum[q][1]; }
      s_slot[parity][0] = t0;
      s_slot[parity][1] = t1;
    }
    __syncthreads();
  };
  // dots of the own rows of w with V[0 .. nv): one warp per basis vector
  auto basis_dots = [&](int nv) {
    for (int i = warp; i < nv; i += CG_WARPS) {
      const float* Vi = a.V + (int64_t)i * K;
      float acc = 0.f;
      for (int r = lane; r < nown; r += 32) acc = fmaf(__ldcg(Vi + r0 + r), s_w[r], acc);
      const double t = warp_sum((double)acc);
      if (lane == 0) s_slot[parity][i] = t;
    }
    __syncthreads();
  };
  // w -= sum_i h_i V_i over the own rows
  auto subtract = [&](int nv, const double* h) {
    for (int r = tid; r < nown; r += CG_THREADS) {
      float acc = s_w[r];
      for (int i = 0; i < nv; i++) acc = fmaf(-(float)h[i], __ldcg(a.V + (int64_t)i * K + r0 + r), acc);
      s_w[r] = acc;
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
    block_sum2(bb, 0.0);
    allreduce(1);
  }
  const double bnorm2 = s_red[0];
  int total = 0, ref = 0;
  double rr = bnorm2;
  if (bnorm2 > 0.0 && alive) {
    const double tol2 = a.tol * a.tol * bnorm2;
    for (ref = 0;; ref++) {
      // FP64 residual r = b - x - G x of the own rows (x complete after the barrier above / below)
      for (int i = tid; i < nr; i += CG_THREADS) s_vd[i] = __ldcg(a.x + R0 + i);
      __syncthreads();
      double prr = 0.0;
      for (int r = r0 + warp; r < r1; r += CG_WARPS) {
        double acc0 = 0.0, acc1 = 0.0;
        const int64_t e1 = a.row_ptr[r + 1];
        int64_t e = a.row_ptr[r] + lane;
        for (; e + 32 < e1; e += 64) {
          acc0 += a.val64[e] * s_vd[a.col[e] - R0];
          acc1 += a.val64[e + 32] * s_vd[a.col[e + 32] - R0];
        }
        if (e < e1) acc0 += a.val64[e] * s_vd[a.col[e] - R0];
        const double acc = warp_sum(acc0 + acc1);
        if (lane == 0) {
          const double rv = a.b[r] - s_vd[r - R0] - acc;
          a.r64[r] = rv;
          prr += rv * rv;
        }
      }
      block_sum2(prr, 0.0);
      allreduce(1);
      rr = s_red[0];
      if (!(rr > tol2) || ref >= a.max_refine || total >= a.max_iter || !alive) break;
      // v0 = r / |r|
      const double beta = sqrt(rr);
      for (int r = r0 + tid; r < r1; r += CG_THREADS) a.V[r] = (float)(a.r64[r] / beta);
      if (tid == 0) {
        for (int i = 0; i <= m; i++) s_g[i] = 0.0;
        s_g[0] = 1.0;
      }
      int jdim = 0;
      for (int j = 0; j < m; j++) {
        alive = grp.sync() && alive;  // V[j] complete in every CTA
        if (!alive) break;
        // w = (I + G32) V[j], own rows
        const float* vj = a.V + (int64_t)j * K + R0;
        for (int i = tid; i < nr; i += CG_THREADS) s_vf[i] = __ldcg(vj + i);
        __syncthreads();
        for (int r = r0 + warp; r < r1; r += CG_WARPS) {
          float acc0 = 0.f, acc1 = 0.f, acc2 = 0.f, acc3 = 0.f;
          const int64_t e1 = a.row_ptr[r + 1];
          int64_t e = a.row_ptr[r] + lane;
          for (; e + 96 < e1; e += 128) {
            acc0 = fmaf(a.val32[e], s_vf[a.col[e] - R0], acc0);
            acc1 = fmaf(a.val32[e + 32], s_vf[a.col[e + 32] - R0], acc1);
            acc2 = fmaf(a.val32[e + 64], s_vf[a.col[e + 64] - R0], acc2);
            acc3 = fmaf(a.val32[e + 96], s_vf[a.col[e + 96] - R0], acc3);
          }
          for (; e < e1; e += 32) acc0 = fmaf(a.val32[e], s_vf[a.col[e] - R0], acc0);
          float acc = (acc0 + acc1) + (acc2 + acc3);
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
          if (lane == 0) s_w[r - r0] = s_vf[r - R0] + acc;
        }
        __syncthreads();
        const int nv = j + 1;
        for (int i = tid; i < nv; i += CG_THREADS) s_h[i] = 0.0;
        __syncthreads();
        // h = V^T w and |w|^2 in one reduction; then w -= V h and
        // |w - V h|^2 = |w|^2 - |h|^2 (V orthonormal)
        {
          double pn = 0.0;
          for (int r = tid; r < nown; r += CG_THREADS) pn += (double)s_w[r] * (double)s_w[r];
          pn = warp_sum(pn);
          if (lane == 0) s_bsum[warp][0] = pn;
        }
        basis_dots(nv);  // ends with __syncthreads: s_bsum complete
        if (tid == 0) {
          double t0 = 0.0;
          for (int q = 0; q < CG_WARPS; q++) t0 += s_bsum[q][0];
          s_slot[parity][nv] = t0;
        }
        __syncthreads();
        allreduce(nv + 1);
        subtract(nv, s_red);  // ends with __syncthreads
        if (tid == 0) {  // one thread: FP64 throughput is scarce on this GPU
          double h2sq = 0.0;
          for (int i = 0; i < nv; i++) h2sq += s_red[i] * s_red[i];
          s_hn = sqrt(fmax(s_red[nv] - h2sq, 0.0));
        }
        for (int i = tid; i < nv; i += CG_THREADS) s_h[i] += s_red[i];
        __syncthreads();
        const double hn = s_hn;
        if (tid == 0) {
          double* col = s_H + j * (m + 1);
          for (int i = 0; i <= j; i++) col[i] = s_h[i];
          col[j + 1] = hn;
          for (int i = 0; i < j; i++) {
            const double p = col[i], q = col[i + 1];
            col[i] = s_cs[i] * p + s_sn[i] * q;
            col[i + 1] = -s_sn[i] * p + s_cs[i] * q;
          }
          const double p = col[j], q = col[j + 1];
          const double rho = sqrt(p * p + q * q);
          s_cs[j] = rho > 0.0 ? p / rho : 1.0;
          s_sn[j] = rho > 0.0 ? q / rho : 0.0;
          col[j] = rho;
          col[j + 1] = 0.0;
          s_g[j + 1] = -s_sn[j] * s_g[j];
          s_g[j] = s_cs[j] * s_g[j];
          s_flag[0] = (fabs(s_g[j + 1]) <= a.inner_tol || !(hn > 0.0)) ? 1 : 0;
        }
        __syncthreads();
        ++total;
        jdim = j + 1;
        if (hn > 0.0 && j + 1 < m) {
          const float inv = (float)(1.0 / hn);
          float* vn = a.V + (int64_t)(j + 1) * K;
          for (int r = tid; r < nown; r += CG_THREADS) vn[r0 + r] = s_w[r] * inv;
        }
        if (s_flag[0] || total >= a.max_iter || !alive) break;
      }
      // y = H^-1 g (upper triangular), x += beta V y in FP64
      if (tid == 0) {
        for (int i = jdim - 1; i >= 0; i--) {
          double sacc = s_g[i];
          for (int k = i + 1; k < jdim; k++) sacc -= s_H[k * (m + 1) + i] * s_y[k];
          const double d = s_H[i * (m + 1) + i];
          s_y[i] = d != 0.0 ? sacc / d : 0.0;
        }
      }
      __syncthreads();
      for (int r = r0 + tid; r < r1; r += CG_THREADS) {
        double acc = 0.0;
        for (int i = 0; i < jdim; i++) acc += s_y[i] * (double)__ldcg(a.V + (int64_t)i * K + r);
        a.x[r] += beta * acc;
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
  gmres_body(a, grp);
}

// One system over the whole grid (cooperative launch, one CTA per SM).
__global__ void __launch_bounds__(CG_THREADS, 1) k_gmres_grid(const ClusterGmresArgs a, unsigned* bar,
                                                              unsigned* err, double* gpart) {
  GridGroup grp{bar, bar + 1, err, gpart};
  gmres_body(a, grp);
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
