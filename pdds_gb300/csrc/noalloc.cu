// Allocation-free interface solve: pdds_solve_bicgstab_static.
//
// Some callers cannot let a library call cudaMalloc or cudaFree: hosts whose
// GPU memory is owned by another allocator (a framework's caching allocator
// that has already reserved most of the device, so a raw cudaMalloc fails or
// fragments its pool), serving loops that must not block, because cudaFree
// synchronises the whole device and cudaMalloc can stall behind other work,
// and foreign-language hosts that hand over device buffers but have no way to
// release memory the library would keep.  For them this entry point solves
// (I + G) u = B with the same FP64 BiCGSTAB kernels as pdds_solve_interface,
// on caller-owned device buffers, and takes its Krylov vectors and reduction
// partials from the file-scope device array below instead of allocating.
//
// Limits and sharing:
//   * K <= PDDS_STATIC_SOLVE_MAX_K (131072 knots); larger systems are rejected.
//   * The array (6.3 MB) exists on every GPU on which the library's module is
//     loaded and stays reserved until the process exits.
//   * All calls share the one array and leave their contents in it; each call
//     clears its scalars and partials and initialises its vectors first.
//     Calls that overlap on the GPU (other streams or threads) race on it.
//   * The first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (once per device); make that first call before any
//     stream capture on that device.
//   * The looked-up address belongs to the device's current primary context.
//     cudaDeviceReset destroys that context (and the array with it); the
//     library, this entry point included, must not be used on a device after
//     it has been reset (the address kept here would then be stale).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/pdds.h"
#include "solve.h"

namespace {

constexpr int MAX_K = PDDS_STATIC_SOLVE_MAX_K;
constexpr int SCAL = 64;     // solver scalars
constexpr int PART = 1024;   // reduction partials (2 x 256 used)
constexpr size_t SCRATCH_DOUBLES = (size_t)6 * MAX_K + SCAL + PART;

static __device__ __align__(256) double g_solve_scratch[SCRATCH_DOUBLES];

constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mutex;
double* g_scratch_addr[MAX_DEVICES] = {nullptr};

void set_err(char* err, int32_t len, const char* msg) {
  if (err && len > 0) {
    std::strncpy(err, msg, (size_t)len - 1);
    err[len - 1] = '\0';
  }
}

}  // namespace

extern "C" pdds_status pdds_solve_bicgstab_static(int device, int32_t K, int64_t nnz,
                                                  const int64_t* row_ptr, const int32_t* col,
                                                  const double* val, const double* B, double* u,
                                                  double tol, int32_t max_iter, void* stream,
                                                  int32_t* iterations, double* rel_residual,
                                                  char* err, int32_t err_len) {
  if (K < 1 || nnz < 0 || !row_ptr || !B || !u || (nnz > 0 && (!col || !val))) {
    set_err(err, err_len, "invalid arguments");
    return PDDS_ERR_INVALID;
  }
  if (K > MAX_K) {
    char msg[160];
    std::snprintf(msg, sizeof msg, "K = %d exceeds the static solve limit of %d knots", (int)K, MAX_K);
    set_err(err, err_len, msg);
    return PDDS_ERR_INVALID;
  }
  if (device < 0 || device >= MAX_DEVICES) {
    set_err(err, err_len, "device id out of range");
    return PDDS_ERR_INVALID;
  }
  int prev = -1;
  cudaGetDevice(&prev);
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    set_err(err, err_len, cudaGetErrorString(e));
    return PDDS_ERR_CUDA;
  }
  double* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[device]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_solve_scratch);
      if (e != cudaSuccess) {
        set_err(err, err_len, cudaGetErrorString(e));
        if (prev >= 0) cudaSetDevice(prev);
        return PDDS_ERR_CUDA;
      }
      g_scratch_addr[device] = static_cast<double*>(p);
    }
    base = g_scratch_addr[device];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // an error left behind by an earlier, unrelated runtime call of the caller
  // is not this solve's failure: clear it before the first enqueue
  (void)cudaGetLastError();
  pdds::SolveWork w;
  std::memset(&w, 0, sizeof w);
  for (int q = 0; q < 6; q++) w.v64[q] = base + (size_t)q * K;
  w.scal = base + (size_t)6 * MAX_K;
  w.part = w.scal + SCAL;
  double host_rr = 0.0;  // residual read back through pageable host memory
  w.host_rr = &host_rr;
  e = cudaMemsetAsync(w.scal, 0, (SCAL + PART) * sizeof(double), s);
  int it = 0;
  double rr = 0.0;
  if (e == cudaSuccess) {
    pdds::SolveCsr A{K, nnz, row_ptr, col, val};
    e = pdds::solve_bicgstab(A, B, u, w, max_iter > 0 ? max_iter : 2 * K, tol > 0 ? tol : 1e-10, &it, &rr, s);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (prev >= 0) cudaSetDevice(prev);
  if (e != cudaSuccess) {
    set_err(err, err_len, cudaGetErrorString(e));
    return PDDS_ERR_CUDA;
  }
  if (iterations) *iterations = it;
  if (rel_residual) *rel_residual = rr;
  const double t = tol > 0 ? tol : 1e-10;
  if (!(rr <= t * 1.0000001) && rr != 0.0) {
    set_err(err, err_len, "BiCGSTAB did not reach the tolerance");
    return PDDS_ERR_NOT_CONVERGED;
  }
  set_err(err, err_len, "");
  return PDDS_OK;
}
