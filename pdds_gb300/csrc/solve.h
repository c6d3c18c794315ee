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
  double* v64[6];   // K doubles each
  double* scal;     // 32 doubles
  double* part;     // reduction partials, >= 2*256 and 48*64 doubles
  double* hess;     // (m+1)m + 2m + 4(m+1) doubles
  float* V32;       // (m+1) K floats
  float* w32;       // K floats
  float* val32;     // nnz floats
  double* host_rr;  // pinned host scalar
  unsigned* ctl;    // 4 unsigned: GMRES ticket, convergence flag, basis size
  int launches;     // kernels launched by the last solve
};

cudaError_t solve_bicgstab(const SolveCsr& A, const double* b, double* x, SolveWork& w,
                           int max_iter, double tol, int* iters, double* relres, cudaStream_t s);
cudaError_t solve_gmres_ir(const SolveCsr& A, const double* b, double* x, SolveWork& w, int m,
                           int max_iter, int max_refine, double tol, int* iters, int* refines,
                           double* relres, cudaStream_t s);

}  // namespace pdds
