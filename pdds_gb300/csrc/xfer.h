// Host<->device copy accounting.  Every copy between host memory and the
// device that the library makes goes through copy_async, which adds its
// bytes to counters of the calling host thread (one context per host
// thread), so an entry point can report exactly the bytes it moved.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace pdds {

struct XferCount {
  int64_t h2d = 0;
  int64_t d2h = 0;
};

// counters of the calling host thread (capi.cu)
XferCount& xfer();

inline cudaError_t copy_async(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s) {
  if (kind == cudaMemcpyHostToDevice)
    xfer().h2d += (int64_t)bytes;
  else if (kind == cudaMemcpyDeviceToHost)
    xfer().d2h += (int64_t)bytes;
  return cudaMemcpyAsync(dst, src, bytes, kind, s);
}

}  // namespace pdds
