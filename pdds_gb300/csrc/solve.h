// Interface-solve drivers (device CSR of I + G without the unit diagonal).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace pdds {

struct SolveCsr {
  int K;
  int64_t nnz;
  const int64_t* row_ptr;
  const int* col;
  const double* val64;
};

struct SolveWork {
  unsigned* err;    // device error flags (grid barrier timeouts)
  double* v64[6];   // K doubles each
  double* scal;     // 32 doubles
  double* part;     // reduction partials, >= 2*256 and 48*64 doubles
  double* hess;     // (m+1)m + 2m + 4(m+1) doubles
  float* V32;       // (m+1) K floats
  float* Z32;       // (m+1) K floats (pipelined GMRES; null: the two-barrier step)
  float* w32;       // K floats
  float* val32;     // nnz floats
  double* host_rr;  // pinned host scalar
  unsigned* ctl;    // 4 unsigned: GMRES ticket, convergence flag, basis size
  unsigned* bar;    // 2 unsigned: grid barrier count and generation
  double* gpart;    // grid-reduction partials, 2 * SMs * (GMRES_CLUSTER_MAX_M + 3)
  unsigned spin_limit;  // grid-barrier polls before a wait gives up (0: the default)
  int grid_ctas;        // CTAs of the whole-GPU solve (0: one per SM)
  int launches;     // kernels launched by the last solve
};

// One-launch GMRES(m)-IR, one thread-block cluster per system (k_gmres_cluster.cu).
// Systems are row ranges [sys_row0[s], sys_row0[s+1]) of one CSR whose
// columns stay inside the system's range (a block-diagonal batch).
constexpr int GMRES_CLUSTER_MAX_M = 40;
constexpr size_t CG_SMEM_CAP = 200 * 1024;  // dynamic shared memory per CTA

struct ClusterGmresArgs {
  int n_sys;
  const int* sys_row0;   // n_sys + 1
  int64_t K;             // rows of the whole CSR (stride of the basis)
  const int64_t* row_ptr;
  const int* col;
  const double* val64;
  const float* val32;
  const double* b;
  double* x;
  double* r64;           // K
  float* V;              // (m + 1) K
  float* Z;              // (m + 1) K: G V, the pipelined one-barrier step (null: two barriers per step)
  int m;
  int max_iter;
  int max_refine;
  double tol;
  double inner_tol;
  int* out_iters;        // per system
  int* out_refines;
  double* out_relres;
  unsigned long long* out_t_end;  // optional: %globaltimer when the system finished
  unsigned spin_limit;   // grid barrier: polls before a wait gives up (0: 2^24, about 1 s)
  unsigned* err_flags;   // optional: index checks of the checked build
};

// Cluster size for systems of at most max_rows rows (about 512 rows per CTA,
// <= 16 CTAs, placeable on the device), 0 when a system of that size does not
// fit the kernel's shared-memory staging (8 max_rows + 4 max_rows / cluster bytes).
int gmres_cluster_pick(int max_rows);
cudaError_t launch_gmres_cluster(const ClusterGmresArgs& a, int cluster, int max_rows, cudaStream_t s);
// One system over the whole GPU: a cooperative launch of one CTA per SM that
// runs the same GMRES with grid barriers (bounded waits; a wait that runs out
// sets ERR_FLAG_TIMEOUT in *err and the kernel returns).  gmres_grid_blocks
// gives the grid (0 when the device or the system size does not allow it);
// bar holds 2 words, gpart 2 * blocks * (GMRES_CLUSTER_MAX_M + 3) doubles.
int gmres_grid_blocks(int max_rows);
cudaError_t launch_gmres_grid(const ClusterGmresArgs& a, int blocks, int max_rows, unsigned* bar, unsigned* err,
                              double* gpart, cudaStream_t s);
// Writes %globaltimer (ns) to *t when the stream reaches it.
cudaError_t launch_stamp(unsigned long long* t, cudaStream_t s);
// b[i] = (float)a[i]
cudaError_t launch_to_f32(const double* a, float* b, int64_t n, cudaStream_t s);

// The same solve through k_gmres_cluster for one system; *used is false (and
// nothing ran) when the system does not fit the cluster kernel.
cudaError_t solve_gmres_ir_cluster(const SolveCsr& A, const double* b, double* x, SolveWork& w, int m,
                                   int max_iter, int max_refine, double tol, int* iters, int* refines,
                                   double* relres, cudaStream_t s, bool* used);

cudaError_t solve_bicgstab(const SolveCsr& A, const double* b, double* x, SolveWork& w,
                           int max_iter, double tol, int* iters, double* relres, cudaStream_t s);
cudaError_t solve_gmres_ir(const SolveCsr& A, const double* b, double* x, SolveWork& w, int m,
                           int max_iter, int max_refine, double tol, int* iters, int* refines,
                           double* relres, cudaStream_t s);

}  // namespace pdds
