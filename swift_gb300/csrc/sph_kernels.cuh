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
};

struct GatherArgs {
  DevParticles p;
  const Unit* units;
  int nunits;
  const Entry* entries;
  int* queue;            // persistent work counter (reset before launch)
  const int* gate;       // optional: skip everything when *gate == 0
  float band;            // relative band of the exact predicate check
};

struct GhostArgs {
  DevParticles p;
  const LeafInfo* leaves;
  float eta_dim, h_tol, h_max, h_min, alpha;
  int iter;              // 0-based round
  int lo, hi;            // particle range handled (cell-sorted order)
  int max_iter;
  int* redo_count;       // [max_iter] particles sent to another round
  int* status;           // non-convergence flag
};

enum GatherMode { MODE_FIRST = 0, MODE_REDO = 1, MODE_ACCUM = 2 };

struct LaunchCfg {
  int tpi;        // threads per i-particle (1, 2, 4, 8)
  int jtile;      // j-tile depth staged in shared memory (64, 128, 256)
  int persistent; // 1: grid of resident blocks pulling units from a queue
  int block;      // threads per block (fixed at 128)
};

cudaError_t launch_density(const GatherArgs& a, int mode, const LaunchCfg& c,
                           int num_sms, cudaStream_t s);
cudaError_t launch_force(const GatherArgs& a, int mode, const LaunchCfg& c,
                         int num_sms, cudaStream_t s);
cudaError_t launch_ghost(const GhostArgs& g, cudaStream_t s);
cudaError_t launch_begin_step(const DevParticles& p, int max_iter,
                              int* redo_count, int* status, cudaStream_t s);
cudaError_t launch_end_force(const DevParticles& p, cudaStream_t s);
cudaError_t launch_prepare_posh(DevParticles p, const int32_t* top_of,
                                const double* top_loc, cudaStream_t s);
cudaError_t launch_permute_in(DevParticles p, const int32_t* perm,
                              const double* x_in, const float* v_in,
                              const float* m_in, const float* h_in,
                              const float* u_in, cudaStream_t s);
cudaError_t launch_collect_out(DevParticles p, const int32_t* perm,
                               float* fields, int32_t* ints, cudaStream_t s);

}  // namespace sphgpu
