// gather.cu -- warp-per-particle neighbour gathers for the density and force
// loops (sm_103a).
//
// One warp owns one updated particle i at a time (particles are pulled from
// a device work queue: the active list, or the ghost's re-run list).  For
// each partner cell of i's leaf the warp
//   1. tests 32 candidate j-blocks at once (one per lane; the leaf's
//      candidate list flattens all its partner cells) against i's search
//      sphere (bounding box of <= 32 spatially sorted particles; FP32,
//      conservative), compacting the survivors into shared memory;
//   2. for each surviving block, evaluates the neighbour predicate with one
//      partner particle per lane: FP32 r^2 from top-cell-relative offsets,
//      and -- only inside a 2^-12 relative band around H^2 -- the exact FP64
//      evaluation in the reference's frame for that cell pair;
//   3. appends hits to a per-warp buffer in shared memory (ballot + popc);
//      whenever 32 hits are buffered, every lane computes one interaction.
// Partial sums are reduced over the warp with shuffles at the end.  There
// are no atomics on particle data and no block-wide barriers.
//
// Physics per hit: runner_iact_nonsym_density (hydro/Minimal/hydro_iact.h:
// 137-189) and runner_iact_nonsym_force (:378-490), Wendland C2 kernel
// (kernel_hydro.h:121-147, :257-284).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "gather_impl.cuh"

namespace sphgpu {

// Per-block h_max (force culling radius, kernel_gamma^2 h^2 of the block's
// largest h), refreshed once the ghost has moved h.
__global__ void block_hmax(const int2* __restrict__ fc, float4* __restrict__ lo,
                           const float4* __restrict__ posh, int nblocks) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nblocks;
       b += gridDim.x * blockDim.x) {
    const int2 r = fc[b];
    float hm = 0.f;
    for (int k = r.x; k < r.x + r.y; k++) hm = fmaxf(hm, posh[k].w);
    lo[b].w = h2_exact(hm);
  }
}

cudaError_t launch_gather(const G2Args& a, bool force, int num_sms, int max_items,
                          cudaStream_t s) {
  int per_sm = 0;
  if (force)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gather_warp<true>,
                                                  WARPS_PER_BLOCK * 32, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gather_warp<false>,
                                                  WARPS_PER_BLOCK * 32, 0);
  int grid = std::max(1, per_sm) * num_sms;
  const int need = (max_items + WARPS_PER_BLOCK - 1) / WARPS_PER_BLOCK;
  grid = std::max(1, std::min(grid, need));
  if (force)
    gather_warp<true><<<grid, WARPS_PER_BLOCK * 32, 0, s>>>(a);
  else
    gather_warp<false><<<grid, WARPS_PER_BLOCK * 32, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_block_hmax(const int2* fc, float4* lo, const float4* posh,
                              int nblocks, cudaStream_t s) {
  int g = (nblocks + 255) / 256;
  g = std::max(1, std::min(g, 152 * 8));
  block_hmax<<<g, 256, 0, s>>>(fc, lo, posh, nblocks);
  return cudaGetLastError();
}

}  // namespace sphgpu
