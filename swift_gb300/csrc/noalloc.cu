// noalloc.cu -- a density first pass that allocates no device memory.
//
// Some callers cannot allocate device memory at the moment they need a
// density pass: hosts that hand all device memory to their own pool and
// account for every byte (as the reference's memuse layer does for its host
// allocations), and latency-critical serving loops that must not stall on
// the allocator.  For them this file offers the density gather in a
// form whose only scratch -- the work-queue counter and the list of work
// groups (32-particle windows of active particles) -- lives in a file-scope
// static device array of fixed size,
// loaded with the library's code and held by every GPU that loads the
// library until the process exits.  The caller passes the resident space
// (inputs) and device buffers for the results (outputs).
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "gather_impl.cuh"

namespace sphgpu {

// Largest particle count, and largest number of 32-particle leaf windows,
// the scratch below can serve.
#define NOALLOC_MAX_PARTICLES (1 << 20)
#define NOALLOC_MAX_UNITS (1 << 16)
// ints [0] unused, [1] work-queue counter, [2..63] unused; then the work
// groups (int4 each, one per 32-particle leaf window).
#define NOALLOC_UNITS_OFFSET 64

static __device__ __align__(256) int g_noalloc_scratch[NOALLOC_UNITS_OFFSET +
                                                        4 * NOALLOC_MAX_UNITS];

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
int noalloc_max_units() { return NOALLOC_MAX_UNITS; }

cudaError_t launch_density_noalloc(const G2Args& base, const LeafInfo* leaves,
                                   int nleaves, const int* leaf_window_begin,
                                   int nwindows, const int* leaf_pair_begin,
                                   float* fields, int32_t* ngb,
                                   const int32_t* perm, int num_sms,
                                   cudaStream_t s) {
  const int n = base.p.n;
  if (n > NOALLOC_MAX_PARTICLES || nwindows > NOALLOC_MAX_UNITS)
    return cudaErrorInvalidValue;
  int* scratch = nullptr;
  cudaError_t e = scratch_for_current_device(&scratch);
  if (e != cudaSuccess) return e;
  // the counters must start at zero on every call
  e = cudaMemsetAsync(scratch, 0, NOALLOC_UNITS_OFFSET * sizeof(int), s);
  if (e != cudaSuccess) return e;
  int4* units = reinterpret_cast<int4*>(scratch + NOALLOC_UNITS_OFFSET);
  const int g = std::max(1, std::min((nleaves * 32 + 255) / 256, num_sms * 16));
  build_units<<<g, 256, 0, s>>>(leaves, nleaves, leaf_window_begin, base.p.flags,
                                1, 0, leaf_pair_begin, units, nullptr);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  G2Args a = base;
  a.units = units;
  a.count = nwindows;
  a.count_ptr = nullptr;
  a.queue = scratch + 1;
  a.hits = nullptr;
  a.gate = nullptr;
  a.mode = MODE_FIRST;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, gather_lanes<false, OUT_CALLER>, WARPS_PER_BLOCK * 32, 0);
  int grid = std::max(1, per_sm) * num_sms;
  grid = std::max(1, std::min(grid, (nwindows + WARPS_PER_BLOCK - 1) /
                                        WARPS_PER_BLOCK));
  gather_lanes<false, OUT_CALLER><<<grid, WARPS_PER_BLOCK * 32, 0, s>>>(
      a, CallerOut{fields, ngb, perm});
  return cudaGetLastError();
}

}  // namespace sphgpu
