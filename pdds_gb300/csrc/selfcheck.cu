// Self-checks of the generator and of the portable FP64 functions that the
// replay kernels share with the CPU restatement (pdds_portable.h).  Replay
// parity cannot catch an error in them, because both sides compile the same
// code; these entry points evaluate them on given inputs, on the device and
// on the host, so that tests can hold them against published known answers
// (Philox-4x32-10) and against libm (exp, log, sin, cos).  Compiled without
// FMA contraction, like the replay kernels, so the device results round
// exactly as the replay kernels' do.
#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <vector>

#include "../../include/pdds.h"
#include "kernels.h"
#include "pdds_portable.h"
#include "xfer.h"

namespace pdds {

namespace {

__host__ __device__ inline void philox_one(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
  u32x4 c;
  for (int q = 0; q < 4; q++) c.v[q] = ctr[q];
  const u32x4 r = philox4x32_10(c, key[0], key[1]);
  for (int q = 0; q < 4; q++) out[q] = r.v[q];
}

__host__ __device__ inline double math_one(int fn, double x) {
  switch (fn) {
    case PDDS_FN_EXP: return pm::exp(x);
    case PDDS_FN_LOG: return pm::log(x);
    case PDDS_FN_SIN: return pm::sin(x);
    case PDDS_FN_COS: return pm::cos(x);
    default: {
      // Box-Muller of the replay kernels: x holds two Philox words
      const uint64_t b = pm::double_to_bits(x);
      double z0, z1;
      box_muller_portable((uint32_t)b, (uint32_t)(b >> 32), &z0, &z1);
      return fn == PDDS_FN_BOX_MULLER_Z0 ? z0 : z1;
    }
  }
}

__global__ void k_philox_check(const uint32_t* __restrict__ ctr, const uint32_t* __restrict__ key, int n,
                               uint32_t* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) philox_one(ctr + 4 * i, key + 2 * i, out + 4 * i);
}

__global__ void k_portable_math_check(int fn, const double* __restrict__ x, int n, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = math_one(fn, x[i]);
}

}  // namespace

cudaError_t launch_philox_check(const uint32_t* ctr, const uint32_t* key, int n, uint32_t* out, cudaStream_t s) {
  if (n > 0) k_philox_check<<<(n + 127) / 128, 128, 0, s>>>(ctr, key, n, out);
  return cudaGetLastError();
}

cudaError_t launch_portable_math_check(int fn, const double* x, int n, double* out, cudaStream_t s) {
  if (n > 0) k_portable_math_check<<<(n + 127) / 128, 128, 0, s>>>(fn, x, n, out);
  return cudaGetLastError();
}

void philox_check_host(const uint32_t* ctr, const uint32_t* key, int n, uint32_t* out) {
  for (int i = 0; i < n; i++) philox_one(ctr + 4 * i, key + 2 * i, out + 4 * i);
}

void portable_math_check_host(int fn, const double* x, int n, double* out) {
  for (int i = 0; i < n; i++) out[i] = math_one(fn, x[i]);
}

}  // namespace pdds

namespace {

void set_err(char* err, int32_t len, const std::string& msg) {
  if (err && len > 0) {
    std::strncpy(err, msg.c_str(), (size_t)len - 1);
    err[len - 1] = '\0';
  }
}

// Runs `launch` on the device with the inputs copied in and the outputs
// copied back (one stream of its own, synchronous).
template <typename TI, typename TO, typename F>
pdds_status run_on_device(int device, const TI* in, size_t n_in, TO* out, size_t n_out, F launch, char* err,
                          int32_t err_len) {
  int prev = -1;
  cudaGetDevice(&prev);
  cudaError_t e = cudaSetDevice(device);
  TI* din = nullptr;
  TO* dout = nullptr;
  cudaStream_t s = nullptr;
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&din, n_in * sizeof(TI));
  if (e == cudaSuccess) e = cudaMalloc(&dout, n_out * sizeof(TO));
  if (e == cudaSuccess) e = pdds::copy_async(din, in, n_in * sizeof(TI), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = launch(din, dout, s);
  if (e == cudaSuccess) e = pdds::copy_async(out, dout, n_out * sizeof(TO), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (din) cudaFree(din);
  if (dout) cudaFree(dout);
  if (s) cudaStreamDestroy(s);
  if (prev >= 0) cudaSetDevice(prev);
  if (e != cudaSuccess) {
    set_err(err, err_len, cudaGetErrorString(e));
    return PDDS_ERR_CUDA;
  }
  return PDDS_OK;
}

}  // namespace

extern "C" {

pdds_status pdds_check_philox(int device, int32_t form, const uint32_t* ctr, const uint32_t* key, int32_t n,
                              uint32_t* out, char* err, int32_t err_len) {
  if (n < 1 || !ctr || !key || !out || (form != PDDS_PHILOX_PORTABLE && form != PDDS_PHILOX_ROUND_KEYS)) {
    set_err(err, err_len, "invalid arguments");
    return PDDS_ERR_INVALID;
  }
  if (form == PDDS_PHILOX_ROUND_KEYS && device < 0) {
    set_err(err, err_len, "the round-key form is the MIXED kernel's: device only");
    return PDDS_ERR_INVALID;
  }
  if (device < 0) {
    pdds::philox_check_host(ctr, key, n, out);
    set_err(err, err_len, "");
    return PDDS_OK;
  }
  if (form == PDDS_PHILOX_PORTABLE) {
    // counters and keys travel in one array: 4 counter words then 2 key words
    std::vector<uint32_t> in((size_t)6 * n);
    std::memcpy(in.data(), ctr, (size_t)4 * n * sizeof(uint32_t));
    std::memcpy(in.data() + (size_t)4 * n, key, (size_t)2 * n * sizeof(uint32_t));
    const pdds_status st = run_on_device(
        device, in.data(), in.size(), out, (size_t)4 * n,
        [n](const uint32_t* d, uint32_t* o, cudaStream_t s) {
          return pdds::launch_philox_check(d, d + (size_t)4 * n, n, o, s);
        },
        err, err_len);
    if (st == PDDS_OK) set_err(err, err_len, "");
    return st;
  }
  // round-key form: the key schedule is a kernel parameter, one launch per key
  for (int i = 0; i < n; i++) {
    const uint64_t k = (uint64_t)key[2 * i] | ((uint64_t)key[2 * i + 1] << 32);
    const pdds_status st = run_on_device(
        device, ctr + (size_t)4 * i, 4, out + (size_t)4 * i, 4,
        [k](const uint32_t* d, uint32_t* o, cudaStream_t s) { return pdds::launch_philox_rk_check(k, d, 1, o, s); },
        err, err_len);
    if (st != PDDS_OK) return st;
  }
  set_err(err, err_len, "");
  return PDDS_OK;
}

pdds_status pdds_check_portable_math(int device, int32_t fn, const double* x, int32_t n, double* out, char* err,
                                     int32_t err_len) {
  if (n < 1 || !x || !out || fn < PDDS_FN_EXP || fn > PDDS_FN_BOX_MULLER_Z1) {
    set_err(err, err_len, "invalid arguments");
    return PDDS_ERR_INVALID;
  }
  if (device < 0) {
    pdds::portable_math_check_host(fn, x, n, out);
    set_err(err, err_len, "");
    return PDDS_OK;
  }
  const pdds_status st = run_on_device(
      device, x, (size_t)n, out, (size_t)n,
      [fn, n](const double* d, double* o, cudaStream_t s) { return pdds::launch_portable_math_check(fn, d, n, o, s); },
      err, err_len);
  if (st == PDDS_OK) set_err(err, err_len, "");
  return st;
}

}  // extern "C"
