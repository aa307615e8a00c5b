// gather.cu -- launchers of the neighbour gathers (kernels in
// gather_impl.cuh) for the density and force loops (sm_103a).
//
// One warp owns a group of up to 32 particles of one leaf, one per lane
// (groups come from a device-built list of 32-particle windows with a lane
// mask: all active particles, or those the ghost sends to another round).
// The group's box culls the leaf's candidate j-blocks; each surviving block
// is staged in shared memory (frame offset applied) and every lane tests its
// own particle against it with broadcast reads -- FP32 r^2 from
// top-cell-relative offsets and, only inside a 2^-12 relative band around
// H^2, the exact FP64 evaluation in the reference's frame for that cell
// pair.  Hits queue per lane in shared memory and are computed in batches;
// every lane keeps its own particle's sums in registers.  No atomics on
// particle data, no block-wide barriers.
//
// Physics per hit: runner_iact_nonsym_density (hydro/Minimal/hydro_iact.h:
// 137-189) and runner_iact_nonsym_force (:378-490), Wendland C2 kernel
// (kernel_hydro.h:121-147, :257-284).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "device_sms.h"
#include "gather_impl.cuh"
#include "gather_tc.cuh"

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

template <bool FORCE, int WPB, int MINB, bool LISTS = false, int TPP = 1, bool BULK = false>
static cudaError_t launch_variant(const G2Args& a, int num_sms, int max_units,
                                  cudaStream_t s) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, gather_lanes<FORCE, OUT_STORE, WPB, MINB, LISTS, TPP, BULK>, WPB * 32, 0);
  int grid = std::max(1, per_sm) * num_sms;
  grid = std::max(1, std::min(grid, (max_units + WPB - 1) / WPB));
  gather_lanes<FORCE, OUT_STORE, WPB, MINB, LISTS, TPP, BULK><<<grid, WPB * 32, 0, s>>>(a);
  return cudaGetLastError();
}

template <int WPB, int MINB, bool LISTS, int TPP>
static cudaError_t launch_tc(const G2Args& a, int num_sms, int max_units, cudaStream_t s) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, gather_density_tc<OUT_STORE, WPB, MINB, LISTS, TPP>, WPB * 32, 0);
  int grid = std::max(1, per_sm) * num_sms;
  grid = std::max(1, std::min(grid, (max_units + WPB - 1) / WPB));
  gather_density_tc<OUT_STORE, WPB, MINB, LISTS, TPP><<<grid, WPB * 32, 0, s>>>(a);
  return cudaGetLastError();
}

template <bool LISTS, int TPP>
static cudaError_t launch_tc_shape(const G2Args& a, int num_sms, int max_units, cudaStream_t s,
                                   int block_warps) {
  return block_warps == 4 ? launch_tc<4, 6, LISTS, TPP>(a, num_sms, max_units, s)
                          : launch_tc<8, 3, LISTS, TPP>(a, num_sms, max_units, s);
}

// The bulk-copy staging (G2Args::bulk) exists for the 8-warp tile shape with
// one or two lanes per particle; other shapes stage with loads.
template <int TPP>
static cudaError_t launch_bulk(const G2Args& a, bool force, bool lists, int num_sms,
                               int max_units, cudaStream_t s) {
  if (force) return launch_variant<true, 8, 3, false, TPP, true>(a, num_sms, max_units, s);
  if (lists) return launch_variant<false, 8, 3, true, TPP, true>(a, num_sms, max_units, s);
  return launch_variant<false, 8, 3, false, TPP, true>(a, num_sms, max_units, s);
}

template <int TPP>
static cudaError_t launch_shape(const G2Args& a, bool force, int num_sms, int max_units,
                                cudaStream_t s, int block_warps) {
  if (block_warps == 4)
    return force ? launch_variant<true, 4, 6, false, TPP>(a, num_sms, max_units, s)
                 : launch_variant<false, 4, 6, false, TPP>(a, num_sms, max_units, s);
  return force ? launch_variant<true, 8, 3, false, TPP>(a, num_sms, max_units, s)
               : launch_variant<false, 8, 3, false, TPP>(a, num_sms, max_units, s);
}

// Tile shapes the autotuner chooses from: 8 warps x 3 blocks per SM (up to
// 85 registers) or 4 warps x 6 blocks per SM (up to 85 registers, finer
// blocks for the tail of the work queue); one, two or four lanes per particle
// (work groups of 32-, 16- or 8-particle windows).  Recording gathers use one
// or two lanes.
cudaError_t launch_gather(const G2Args& a, bool force, int num_sms, int max_units,
                          cudaStream_t s, int block_warps, bool lists, int tpp) {
  if (a.tc && !force && !a.bulk && (tpp == 1 || tpp == 2)) {
    if (lists)
      return tpp == 2 ? launch_tc_shape<true, 2>(a, num_sms, max_units, s, block_warps)
                      : launch_tc_shape<true, 1>(a, num_sms, max_units, s, block_warps);
    return tpp == 2 ? launch_tc_shape<false, 2>(a, num_sms, max_units, s, block_warps)
                    : launch_tc_shape<false, 1>(a, num_sms, max_units, s, block_warps);
  }
  if (a.bulk && block_warps == 8 && (tpp == 1 || tpp == 2))
    return tpp == 2 ? launch_bulk<2>(a, force, lists, num_sms, max_units, s)
                    : launch_bulk<1>(a, force, lists, num_sms, max_units, s);
  if (lists && !force) {
    if (tpp == 2)
      return block_warps == 4 ? launch_variant<false, 4, 6, true, 2>(a, num_sms, max_units, s)
                              : launch_variant<false, 8, 3, true, 2>(a, num_sms, max_units, s);
    return block_warps == 4 ? launch_variant<false, 4, 6, true>(a, num_sms, max_units, s)
                            : launch_variant<false, 8, 3, true>(a, num_sms, max_units, s);
  }
  if (tpp == 4) return launch_shape<4>(a, force, num_sms, max_units, s, block_warps);
  return tpp == 2 ? launch_shape<2>(a, force, num_sms, max_units, s, block_warps)
                  : launch_shape<1>(a, force, num_sms, max_units, s, block_warps);
}

cudaError_t launch_build_units(const LeafInfo* leaves, int nleaves,
                               const int* leaf_window_begin, const uint8_t* flags,
                               int need, int veto, const int* leaf_pair_begin,
                               int4* units, const int* gate, cudaStream_t s, int win,
                               int* compact) {
  int g = (nleaves * 32 + 255) / 256;
  g = std::max(1, std::min(g, sm_count() * 16));
  build_units<<<g, 256, 0, s>>>(leaves, nleaves, leaf_window_begin, flags, need, veto,
                                leaf_pair_begin, units, gate, win, compact);
  return cudaGetLastError();
}


cudaError_t launch_solve_from_lists(const ListArgs& a, const GhostArgs& g, int max_iter,
                                    cudaStream_t s) {
  long long grid = ((long long)a.p.n * 4 + 255) / 256;  // four lanes per particle
  const long long cap = 16LL * sm_count();
  grid = grid < 1 ? 1 : (grid > cap ? cap : grid);
  if (a.leaf_tw)
    solve_from_lists<true><<<(int)grid, 256, 0, s>>>(a, g, max_iter);
  else
    solve_from_lists<false><<<(int)grid, 256, 0, s>>>(a, g, max_iter);
  return cudaGetLastError();
}

cudaError_t launch_block_hmax(const int2* fc, float4* lo, const float4* posh,
                              int nblocks, cudaStream_t s) {
  int g = (nblocks + 255) / 256;
  g = std::max(1, std::min(g, sm_count() * 8));
  block_hmax<<<g, 256, 0, s>>>(fc, lo, posh, nblocks);
  return cudaGetLastError();
}

}  // namespace sphgpu
