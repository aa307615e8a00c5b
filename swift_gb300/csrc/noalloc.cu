// noalloc.cu -- a density first pass that allocates no device memory.
//
// Some callers cannot allocate device memory at the moment they need a
// density pass: code running inside CUDA stream capture (a cudaMalloc there
// invalidates the capture), hosts that hand all device memory to their own
// pool and account for every byte (as the reference's memuse layer does for
// its host allocations), and latency-critical serving loops that must not
// stall on the allocator.  For them this file offers the density gather in a
// form whose only scratch -- the work-queue counter and the list of active
// particles -- lives in a file-scope static device array of fixed size,
// loaded with the library's code and held by every GPU that loads the
// library until the process exits.  The caller passes the resident space
// (inputs) and device buffers for the results (outputs).
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "gather_impl.cuh"

namespace sphgpu {

// Largest particle count the scratch below can serve.
#define NOALLOC_MAX_PARTICLES (1 << 20)
// [0] number of listed particles, [1] work-queue counter, [2..63] unused,
// [64..] the list of active particles.
#define NOALLOC_LIST_OFFSET 64

static __device__ __align__(256) int g_noalloc_scratch[NOALLOC_LIST_OFFSET +
                                                        NOALLOC_MAX_PARTICLES];

// Compact the active particles (flag bit 0) into the scratch list; within a
// warp the store order is kept (ballot + popc), so neighbouring particles
// stay close in the list.
__global__ void noalloc_list(const uint8_t* __restrict__ flags, int n) {
  int* cnt = &g_noalloc_scratch[0];
  int* list = &g_noalloc_scratch[NOALLOC_LIST_OFFSET];
  const int lane = threadIdx.x & 31;
  for (int base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31; base < n;
       base += gridDim.x * blockDim.x) {
    const int i = base + lane;
    const bool act = i < n && (flags[i] & 1);
    const unsigned m = __ballot_sync(0xffffffffu, act);
    int first = 0;
    if (lane == 0 && m) first = atomicAdd(cnt, __popc(m));
    first = __shfl_sync(0xffffffffu, first, 0);
    if (act) list[first + __popc(m & ((1u << lane) - 1u))] = i;
  }
}

// Address of the scratch array for the current device, looked up once per
// device (cudaGetSymbolAddress) and cached.
static cudaError_t scratch_for_current_device(int** out) {
  static std::mutex mu;
  static int* cached[256] = {nullptr};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 256) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(mu);
  if (!cached[dev]) {
    int* p = nullptr;
    e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    cached[dev] = p;
  }
  *out = cached[dev];
  return cudaSuccess;
}

int noalloc_max_particles() { return NOALLOC_MAX_PARTICLES; }

cudaError_t launch_density_noalloc(const G2Args& base, const uint8_t* flags,
                                   float* fields, int32_t* ngb,
                                   const int32_t* perm, int num_sms,
                                   cudaStream_t s) {
  const int n = base.p.n;
  if (n > NOALLOC_MAX_PARTICLES) return cudaErrorInvalidValue;
  int* scratch = nullptr;
  cudaError_t e = scratch_for_current_device(&scratch);
  if (e != cudaSuccess) return e;
  // the counters must start at zero on every call
  e = cudaMemsetAsync(scratch, 0, NOALLOC_LIST_OFFSET * sizeof(int), s);
  if (e != cudaSuccess) return e;
  const int lgrid = std::max(1, std::min((n + 255) / 256, num_sms * 8));
  noalloc_list<<<lgrid, 256, 0, s>>>(flags, n);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  G2Args a = base;
  a.list = scratch + NOALLOC_LIST_OFFSET;
  a.count = 0;
  a.count_ptr = scratch;
  a.items = nullptr;
  a.queue = scratch + 1;
  a.hits = nullptr;
  a.mode = MODE_FIRST;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, gather_warp<false, OUT_CALLER>, WARPS_PER_BLOCK * 32, 0);
  int grid = std::max(1, per_sm) * num_sms;
  grid = std::max(1, std::min(grid, (n + WARPS_PER_BLOCK - 1) / WARPS_PER_BLOCK));
  gather_warp<false, OUT_CALLER><<<grid, WARPS_PER_BLOCK * 32, 0, s>>>(
      a, CallerOut{fields, ngb, perm});
  return cudaGetLastError();
}

}  // namespace sphgpu
