// device_sms.h -- the streaming-multiprocessor count of the current device,
// read once per device from cudaDevAttrMultiProcessorCount.  Launch caps
// are multiples of it; no kernel's result depends on it (every capped kernel
// walks its range with a grid-stride loop).
#pragma once
#include <cuda_runtime.h>

namespace sphgpu {

inline int sm_count() {
  static int cache[64];  // 0 = not read yet
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return 1;
  }
  int v = __atomic_load_n(&cache[dev], __ATOMIC_RELAXED);
  if (v == 0) {
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v < 1) {
      cudaGetLastError();
      v = 1;
    }
    __atomic_store_n(&cache[dev], v, __ATOMIC_RELAXED);
  }
  return v;
}

}  // namespace sphgpu
