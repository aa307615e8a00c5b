// devplan.cuh -- the gather lists of a step planned on the device.
//
// The host planner (space.cpp) expands each top-level task through the
// reference's DOSUB recursions (runner_doiact_functions_hydro.h:2933-3100)
// and the ghost's subset recursion (runner_doiact_functions_hydro.h:3290-3400)
// into per-leaf entries.  Here one warp plans one leaf: each lane takes one
// task linked to the leaf's top cell (at most 27), replays the recursion
// restricted to the branches that contain the leaf, and emits the leaf's
// entries in the host's order (tasks in order, depth first within a task).
// Two passes (count, emit) around an exclusive scan over the leaves give the
// same arrays the host's flatten() gives, per leaf.
//
// The cells' h_max, h_max_active and activity come from the particles on the
// device (a zero-displacement drift of every cell, cell_drift.c:330-371),
// and the force lists from the post-ghost h_max (runner_ghost.c:1617-1632:
// the larger of each cell's pre-ghost h_max and its particles' new h).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "sph_types.h"

namespace sphgpu {

// One cell of the tree, static between rebuilds.
struct DPCell {
  double loc[3];
  float dmin;
  int32_t first, count;
  int32_t parent, top;
  int32_t jb_begin, jb_end;  // j-block range of the cell's particles
  int16_t depth;
  int8_t split;
  int8_t pad0;
  int32_t pad1;
};
static_assert(sizeof(DPCell) == 64, "DPCell layout");

struct DPTree {
  const DPCell* cell = nullptr;
  const int32_t* progeny = nullptr;    // [8 * ncells], -1 where absent
  const int32_t* leaf_cell = nullptr;  // [nleaves]
  const int2* task = nullptr;          // [ntasks] (ci, cj); cj < 0: self task
  const int32_t* link_begin = nullptr; // [ntop + 1]
  const int32_t* link = nullptr;       // tasks of each top cell, in task order
  int ncells = 0, nleaves = 0, ntop = 0, ntasks = 0;
  double dim[3] = {0, 0, 0};
  int periodic = 1;
};

// Per-step cell state (float bits of non-negative h: ordered as integers).
struct DPCellState {
  unsigned* hmax = nullptr;    // h_max at activation (the recursions' h_max_old)
  unsigned* hact = nullptr;    // h_max_active at activation
  unsigned* hforce = nullptr;  // h_max after the ghost
  int* active = nullptr;
  // dx_max_part: the largest motion of the cell's particles since the
  // rebuild (cell_drift.c:330-382), all zero until the space drifts
  const unsigned* dx = nullptr;
};

enum DPKind { DP_DENSITY = 0, DP_SUBSET = 1, DP_FORCE = 2 };

// Output of one plan: entries grouped by leaf, the per-leaf (j-block, entry)
// candidate pairs and their leaf offsets (leaf_pair_begin).
struct DPOut {
  Entry* entries = nullptr;
  int32_t* lpb = nullptr;  // [nleaves + 1]
  int32_t* pb = nullptr;
  int32_t* pe = nullptr;
  long long cap_e = 0, cap_p = 0;
  // scratch shared by the plans of a step
  int2* lane_off = nullptr;  // [32 * nleaves] per-lane (entries, pairs) prefix
  int2* leaf_off = nullptr;  // [nleaves + 1] scanned (entries, pairs)
  int2* tiles = nullptr;     // [dp_scan_tiles(nleaves + 1)]
  // status[0]: error bits (1 = a plan outgrew its buffers, 2 = recursion
  // deeper than the stack, 4 = more than 32 tasks on a top cell);
  // status[1 + 2 k], [2 + 2 k]: entries and pairs plan k needed
  int* status = nullptr;
};

constexpr int kDPStack = 28;  // recursion frames: tree depth + 2 at most

int dp_scan_tiles(long long n);

// flags[i] = time_bin[i] <= *max_active_bin (bit 0 = active)
cudaError_t launch_dp_flags(uint8_t* flags, const int8_t* tbin, int n, const int* max_bin,
                            cudaStream_t st);
// Cell state from the particles: activation values (force = false) from the
// current h and flags, or the post-ghost h_max (force = true) from the
// current h and the step's starting h of the active particles.
cudaError_t launch_dp_cells(const DPTree& t, const DPCellState& cs, const float4* posh,
                            const float* h0, const uint8_t* flags, bool force,
                            cudaStream_t st);
// One plan (count, scan, emit); writes lpb as zeros when the plan does not
// fit (status[0] bit 1 set, status[1 + 2 kind ...] the sizes it needs).
cudaError_t launch_dp_plan(const DPTree& t, const DPCellState& cs, int kind, const DPOut& o,
                           cudaStream_t st);

// Drift without a rebuild (drift.cu).  The proposed positions x_new and
// smoothing lengths h_new are in input order; perm maps store index to input
// index.  drift_cells: every cell's largest motion since the rebuild (dxn,
// from x_rebuild) and its largest new h (hmx), as float bits.
cudaError_t launch_drift_cells(const DPTree& t, const int32_t* perm, const double* x_new,
                               const double* x_rebuild, const float* h_new, unsigned* dxn,
                               unsigned* hmx, cudaStream_t st);
// cell_need_rebuild_for_hydro_pair (cell.h:1237) over every pair of
// neighbouring top-level cells: *flag = 1 when one needs a rebuild.
cudaError_t launch_drift_check(const DPTree& t, const unsigned* dxn, const unsigned* hmx,
                               int* flag, cudaStream_t st);
// The particles take the new positions and h: FP64 positions (xd), FP32
// offsets from their top cells with h (P.posh), the step's starting h
// (P.h0), depth_h and the starting depth_h0 (cell_set_part_h_depth on the
// leaf chain).
struct DevParticles;
cudaError_t launch_drift_commit(const DevParticles& P, double* xd, int8_t* depth_h0,
                                const int32_t* perm, const double* x_new, const float* h_new,
                                const int32_t* top_of, const double* top_loc,
                                const LeafInfo* leaves, cudaStream_t st);
// j-block bounding boxes (and the boxes of their runs of 8) from the
// particles' FP32 offsets, as the host build computes them.
cudaError_t launch_block_boxes(const int2* fc, const float4* posh, float4* lo, float4* hi,
                               float4* sub_lo, float4* sub_hi, int nblocks, cudaStream_t st);

}  // namespace sphgpu
