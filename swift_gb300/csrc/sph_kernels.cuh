// sph_kernels.cuh -- device-side particle store and kernel launchers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "sph_types.h"

namespace sphgpu {

// Particle store in HBM, cell-sorted order, structure of arrays.
struct DevParticles {
  int n;
  const double* xd;     // [3n] FP64 positions (exact neighbour predicate)
  float4* posh;         // [n] offset from top-cell corner (xyz), h (w)
  float4* velm;         // [n] velocity (xyz), mass (w)
  float* u;             // [n] internal energy
  float* h0;            // [n] smoothing length at the start of the step
  uint8_t* flags;       // [n] bit0 active, bit1 needs another ghost round
  int8_t* depth_h;      // [n]
  const int8_t* depth_h0;  // [n] depth_h of the input h (a step's start)
  int32_t* leaf_of;     // [n]
  // density sums: rho, rho_dh, wcount, wcount_dh | div_v, rot_v[3]
  float4* dens0;
  float4* dens1;
  // ghost state
  float* left;
  float* right;
  int32_t* ghost_iters;
  // force inputs: rho, f, P/rho^2 (without f_ij), soundspeed | balsara, pressure
  float4* fin0;
  float2* fin1;
  // force outputs: a[3], u_dt | h_dt, v_sig
  float4* acc;
  float2* hdt_vsig;
  // neighbour counters: density (last pass), density (first pass), force
  int32_t* ngb_d;
  int32_t* ngb_d_first;
  int32_t* ngb_f;
  // optional (null: not kept): time bins, and the smallest time bin > 0
  // among each particle's force neighbours (limiter_data.min_ngb_time_bin,
  // num_time_bins + 1 when none), which limits its next time step
  const int8_t* tbin = nullptr;
  int8_t* ngb_bin = nullptr;
};

enum GatherMode { MODE_FIRST = 0, MODE_REDO = 1, MODE_ACCUM = 2 };

// Lane-per-particle gather (gather_impl.cuh).
struct G2Args {
  DevParticles p;
  const int4* units;            // (window base, lane mask, pair begin, end)
  int count;                    // number of units, or
  const int* count_ptr;         //   read from device memory when non-null
  const int* pair_block;        // candidate j-block ...
  const int* pair_entry;        // ... and the gather-list entry it belongs to
  const Entry* entries;
  const float4* bb_lo;          // j-block boxes: lo.xyz, (K h_max)^2
  const float4* bb_hi;
  const int2* bb_fc;            // j-block particle range
  float3 top_width;             // top-level cell width (frame offsets)
  const float4* leaf_tw;        // or per leaf (boxes of different sizes)
  int* queue;                   // work counter, zero before the launch
  unsigned long long* hits;     // optional: total neighbour hits of the launch
  const int* gate;              // optional: do nothing when *gate == 0
  float band;                   // relative band of the exact predicate
  int mode;                     // GatherMode
  // Neighbour lists of the ghost's re-runs, recorded by the first re-run
  // (gathers launched with lists), for every candidate with FP32 r^2 below
  // (gamma h)^2 (1 + band): items (partner index | frame-offset index << 27)
  // of particle i in nl[i * nl_cap ...], one segment of nl_cap / TPP items
  // per lane of the particle; segment sizes are multiples of 8 (items are
  // written 8 at a time).
  int* nl;
  int* nl_cnt;                  // items per particle (two lanes: segment 0's
                                // count | segment 1's << 16), -1 when a
                                // segment overflowed
  float* nl_T;                  // the r^2 bound the items were recorded under
  int nl_cap;
  // lists recorded by the first density pass cover a wider radius than the
  // pass's own: r^2 below min(nl_widen (gamma h)^2 (1 + band), the square of
  // the smallest width of the particle's depth_h cell) -- every particle
  // closer than that width lies in a cell the recursion pairs at that depth
  float nl_widen = 1.f;
  const LeafInfo* leaves = nullptr;  // for that width (lists only)
  // force gathers: take each group's partners from the first pass's rows
  // where they cover them (rows recorded this step, nl_seg segments each)
  int force_rows = 0;
  int nl_seg = 1;
  const int* blk_of = nullptr;  // j-block of every particle (frame lookups)
  // j-blocks staged by bulk copies (cp.async.bulk into shared memory, one
  // per block, completing on an mbarrier) instead of a load per lane; a
  // wait that runs out sets *err (the host reports it) and ends the warp
  int bulk = 0;
  int* err = nullptr;
  // density gathers: the boxes of each j-block's runs of 8 particles (4 per
  // block); a run no particle of the group can reach is not tested
  const float4* sb_lo = nullptr;
  const float4* sb_hi = nullptr;
  // density gathers: candidates pre-filtered on the tensor cores
  // (gather_density_tc: one or two lanes per particle, loads)
  int tc = 0;
};

// Later re-runs from the lists: particles whose list covers their new
// search radius are computed from it (and flagged 8); the others are left
// to the gather.  Candidates inside the band around H^2 are decided exactly
// in the frame of the re-run list entry that pairs them.
struct ListArgs {
  DevParticles p;
  const int* nl;
  const int* nl_cnt;
  const float* nl_T;
  int nl_cap;
  int nl_seg;                   // segments per row (lanes per particle of the
                                // recording gather: 1 or 2)
  const int* leaf_pair_begin;   // the re-run (subset) lists, per leaf
  const int* pair_block;
  const int* pair_entry;
  const Entry* entries;
  const int* blk_of;            // j-block of every particle
  float3 top_width;
  float band;
  const int* gate;              // do nothing when *gate == 0
  unsigned long long* hits;     // optional: total neighbour hits
  int* handover;                // solver: particles left to the catch-up rounds
  const float4* leaf_tw = nullptr;  // per leaf top-cell width (boxes of different
                                    // sizes in one store), else top_width
};

struct GhostArgs {
  DevParticles p;
  const LeafInfo* leaves;
  float eta_dim, h_tol, h_max, h_min, alpha;
  int iter;                     // 0-based round
  int lo, hi;                   // particle range handled (store order)
  int* redo_count;              // [max_iter] particles sent to another round
};

// lists: record the re-run neighbour lists (density re-run mode, a.nl set);
// tpp: lanes per particle, 1 (32-particle work groups) or 2 (16-particle
// groups; not with lists)
cudaError_t launch_gather(const G2Args& a, bool force, int num_sms, int max_units,
                          cudaStream_t s, int block_warps = 8, bool lists = false,
                          int tpp = 1);
// Work groups (windows of `win` particles, 32 or 16) of the particles whose
// flags hold every bit of `need` and no bit of `veto`; with `compact` (zero
// before the launch) only the non-empty ones, *compact of them.
cudaError_t launch_build_units(const LeafInfo* leaves, int nleaves,
                               const int* leaf_window_begin, const uint8_t* flags,
                               int need, int veto, const int* leaf_pair_begin,
                               int4* units, const int* gate, cudaStream_t s, int win = 32,
                               int* compact = nullptr);
// The ghost's rounds 1.. max_iter - 1 for every particle still iterating
// after round 0, each particle on its own: density from its list (or, where
// its h outgrew the list, from its leaf's re-run candidate blocks), then the
// Newton update, until it converges.
cudaError_t launch_solve_from_lists(const ListArgs& a, const GhostArgs& g, int max_iter,
                                    cudaStream_t s);
int noalloc_max_particles();
int noalloc_max_units();
cudaError_t launch_density_noalloc(const G2Args& base, const LeafInfo* leaves,
                                   int nleaves, const int* leaf_window_begin,
                                   int nwindows, const int* leaf_pair_begin,
                                   float* fields, int32_t* ngb,
                                   const int32_t* perm, int num_sms,
                                   cudaStream_t s);
cudaError_t launch_block_hmax(const int2* fc, float4* lo, const float4* posh,
                              int nblocks, cudaStream_t s);
cudaError_t launch_ghost(const GhostArgs& g, cudaStream_t s);
// A catch-up round after the list solver: every particle still iterating
// takes its own next round (its iteration count, ghost_iters) from the sums
// a re-run gather just computed; *sent counts those it sends on.  Does
// nothing when *gate == 0.
cudaError_t launch_ghost_catchup(const GhostArgs& g, int max_iter, const int* gate, int* sent,
                                 cudaStream_t s);
cudaError_t launch_begin_step(const DevParticles& p, int max_iter,
                              int* redo_count, float h_max, cudaStream_t s);
cudaError_t launch_set_flags(uint8_t* flags, const int* idx, int n, uint8_t v,
                             cudaStream_t s);
cudaError_t launch_gather_h(const float4* posh, const int* idx, int n, float* out,
                            cudaStream_t s);
cudaError_t launch_sum_active_ngb(const DevParticles& p, unsigned long long* out,
                                  cudaStream_t s);
cudaError_t launch_end_force(const DevParticles& p, cudaStream_t s);
cudaError_t launch_prepare_posh(DevParticles p, const int32_t* top_of,
                                const double* top_loc, cudaStream_t s);
// Host-order v, m, u -> store; sets *differ when x or h differ from the
// space's own (x_ref: the space's input positions, input order).
cudaError_t launch_verify_force_plan(DevParticles p, const int4* chk, int nchk,
                                    const uint8_t* planned, int* flag, cudaStream_t s);
cudaError_t launch_permute_vmu_in(DevParticles p, const int32_t* perm, const float* v,
                                  const float* m, const float* u, cudaStream_t s);
cudaError_t launch_permute_in(DevParticles p, const int32_t* perm,
                              const double* x_in, const double* x_ref,
                              const float* v_in, const float* m_in,
                              const float* h_in, const float* u_in, int* differ,
                              cudaStream_t s);
cudaError_t launch_set_state(DevParticles p, const int32_t* perm, const float* v,
                             const float* m, const float* u, const float* rho,
                             const float* f, const float* pressure, const float* soundspeed,
                             const float* balsara, const int8_t* time_bin, int8_t* tbin,
                             cudaStream_t s);
cudaError_t launch_collect_out(DevParticles p, const int32_t* perm,
                               float* fields, int32_t* ints, cudaStream_t s);

}  // namespace sphgpu
