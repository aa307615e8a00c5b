// sph_kernels.cu -- per-particle kernels of the SPH path (sm_103a): the
// ghost's Newton-Raphson round on h, step set-up, end of force, and the
// permutations between the caller's order and the cell-sorted store.  The
// neighbour gathers live in gather.cu.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "device_sms.h"
#include "ghost_impl.cuh"
#include "sph_kernels.cuh"

namespace sphgpu {

// ---------------------------------------------------------------------------
// Ghost: one Newton-Raphson round on h for every particle still iterating
// (runner_ghost.c:1113-1500; hydro.h:543-574, :626, :669-761).

__global__ void ghost_round(GhostArgs g) {
  if (g.iter > 0 && g.redo_count[g.iter - 1] == 0) return;
  const DevParticles& P = g.p;
  for (int i = g.lo + blockIdx.x * blockDim.x + threadIdx.x; i < g.hi;
       i += gridDim.x * blockDim.x) {
    const uint8_t fl = P.flags[i];
    if ((fl & 3) != 3) continue;  // active and still iterating
    ghost_update(g, i, g.iter, P.dens0[i], P.dens1[i]);
  }
}

// Start of a step: active particles restart from the input h with cleared
// sums; inactive ones keep the state of their last step, which the loops of
// their active neighbours read.
__global__ void begin_step(DevParticles P, int max_iter, int* redo_count, float h_max) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid < max_iter) redo_count[tid] = 0;
  for (int i = tid; i < P.n; i += gridDim.x * blockDim.x) {
    if (!(P.flags[i] & 1)) {
      P.flags[i] = 0;
      continue;
    }
    float4 ph = P.posh[i];
    ph.w = P.h0[i];
    P.posh[i] = ph;
    P.flags[i] = 3;
    P.depth_h[i] = P.depth_h0[i];
    // the ghost's bisection bracket starts at [0, h_max] (runner_ghost.c:1181-1182)
    P.left[i] = 0.f;
    P.right[i] = h_max;
    P.ghost_iters[i] = 0;
    P.dens0[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    P.dens1[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    P.ngb_d[i] = 0;
    P.ngb_d_first[i] = 0;
    P.ngb_f[i] = 0;
  }
}

// Activity flags of a list of particles (bit 0 = active).
__global__ void set_flags_k(uint8_t* flags, const int* __restrict__ idx, int n,
                            uint8_t v) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += gridDim.x * blockDim.x)
    flags[idx[k]] = v;
}

// Smoothing lengths of a list of particles.
__global__ void gather_h_k(const float4* __restrict__ posh, const int* __restrict__ idx,
                           int n, float* out) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += gridDim.x * blockDim.x)
    out[k] = posh[idx[k]].w;
}

// Density neighbours at the converged h, summed over the active particles.
__global__ void sum_active_ngb(DevParticles P, unsigned long long* out) {
  unsigned long long acc = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n;
       i += gridDim.x * blockDim.x)
    if (P.flags[i] & 1) acc += (unsigned long long)P.ngb_d[i];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0 && acc) atomicAdd(out, acc);
}

__global__ void end_force_k(DevParticles P) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n;
       i += gridDim.x * blockDim.x) {
    if (!(P.flags[i] & 1)) continue;
    float2 hv = P.hdt_vsig[i];
    hv.x *= P.posh[i].w * SPH_HDIM_INV;
    P.hdt_vsig[i] = hv;
  }
}

__global__ void prepare_posh(DevParticles P, const int32_t* __restrict__ top_of,
                             const double* __restrict__ top_loc) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n;
       i += gridDim.x * blockDim.x) {
    const int t = top_of[i];
    float4 q;
    q.x = __double2float_rn(P.xd[3 * (size_t)i + 0] - top_loc[3 * t + 0]);
    q.y = __double2float_rn(P.xd[3 * (size_t)i + 1] - top_loc[3 * t + 1]);
    q.z = __double2float_rn(P.xd[3 * (size_t)i + 2] - top_loc[3 * t + 2]);
    q.w = P.h0[i];
    P.posh[i] = q;
  }
}

// Host-order inputs -> cell-sorted store (perm: sorted index -> input index).
__global__ void permute_in(DevParticles P, const int32_t* __restrict__ perm,
                           const double* __restrict__ x, const double* __restrict__ x_ref,
                           const float* __restrict__ v, const float* __restrict__ m,
                           const float* __restrict__ h, const float* __restrict__ u,
                           int* differ) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n;
       i += gridDim.x * blockDim.x) {
    const size_t k = (size_t)perm[i];
    // the cell tree and the gather lists were built from the space's own
    // positions and smoothing lengths: only v, m and u may change
    if (x[3 * k] != x_ref[3 * k] || x[3 * k + 1] != x_ref[3 * k + 1] ||
        x[3 * k + 2] != x_ref[3 * k + 2] || h[k] != P.h0[i])
      atomicExch(differ, 1);
    P.velm[i] = make_float4(v[3 * k], v[3 * k + 1], v[3 * k + 2], m[k]);
    P.u[i] = u[k];
  }
}

// The force recursion's decisions at the step's post-ghost h_max (per
// checked cell: the larger of the step's starting h and the ghost's result
// over its particles, runner_ghost.c:1617-1632; gamma h_max < dmin / 2,
// cell.h:966-1010) against the ones the force lists were planned with; any
// difference sets *flag.  One warp per cell.
__global__ void verify_force_plan(DevParticles P, const int4* __restrict__ chk, int nchk,
                                  const uint8_t* __restrict__ planned, int* flag) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int q = warp; q < nchk; q += nwarps) {
    const int4 c = chk[q];
    float m = 0.f;
    for (int k = c.x + lane; k < c.x + c.y; k += 32) {
      float h = P.posh[k].w;
      if (P.flags[k] & 1) h = fmaxf(h, P.h0[k]);
      m = fmaxf(m, h);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
    if (lane == 0) {
      const bool d = __fmul_rn(SPH_KG, m) < __fmul_rn(0.5f, __int_as_float(c.z));
      if ((uint8_t)(d ? 1 : 0) != planned[q]) atomicOr(flag, 1);
    }
  }
}

// New velocities, masses and internal energies (input order) into the
// store; positions and h stay the space's.
__global__ void permute_vmu_in(DevParticles P, const int32_t* __restrict__ perm,
                               const float* __restrict__ v, const float* __restrict__ m,
                               const float* __restrict__ u) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n;
       i += gridDim.x * blockDim.x) {
    const size_t k = (size_t)perm[i];
    P.velm[i] = make_float4(v[3 * k], v[3 * k + 1], v[3 * k + 2], m[k]);
    P.u[i] = u[k];
  }
}

// Cell-sorted results -> input order, float [n][24] and int32 [n][4].
__global__ void collect_out(DevParticles P, const int32_t* __restrict__ perm,
                            float* __restrict__ fields, int32_t* __restrict__ ints) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n;
       i += gridDim.x * blockDim.x) {
    const size_t k = (size_t)perm[i];
    if (fields) {
      float* o = fields + 24 * k;
      const float4 d0 = P.dens0[i], d1 = P.dens1[i];
      o[0] = d0.x; o[1] = d0.y; o[2] = d0.z; o[3] = d0.w;
      o[4] = d1.x; o[5] = d1.y; o[6] = d1.z; o[7] = d1.w;
      const float4 f0 = P.fin0[i];
      const float2 f1 = P.fin1[i];
      o[8] = P.posh[i].w;
      o[9] = f0.x; o[10] = f0.y; o[11] = f1.y; o[12] = f0.w; o[13] = f1.x;
      o[14] = 2.f * f0.w;
      const float4 ac = P.acc[i];
      const float2 hv = P.hdt_vsig[i];
      o[15] = ac.x; o[16] = ac.y; o[17] = ac.z; o[18] = ac.w;
      o[19] = hv.x; o[20] = hv.y;
      o[21] = P.ngb_bin ? (float)P.ngb_bin[i] : (float)(SPH_NUM_TIME_BINS + 1);
      o[22] = 0.f; o[23] = 0.f;
    }
    if (ints) {
      int32_t* o = ints + 4 * k;
      o[0] = P.ngb_d_first[i];
      o[1] = P.ngb_d[i];
      o[2] = P.ngb_f[i];
      o[3] = P.ghost_iters[i];
    }
  }
}

// ---------------------------------------------------------------------------
// Launchers

static int grid_for(int n) {
  int g = (n + 255) / 256;
  const int cap = 16 * sm_count();
  return g < 1 ? 1 : (g > cap ? cap : g);
}

__global__ void ghost_catchup(GhostArgs g, int max_iter, const int* gate, int* sent) {
  if (*gate == 0) return;
  const DevParticles& P = g.p;
  for (int i = g.lo + blockIdx.x * blockDim.x + threadIdx.x; i < g.hi;
       i += gridDim.x * blockDim.x) {
    if ((P.flags[i] & 3) != 3) continue;  // active and still iterating
    const int it = P.ghost_iters[i];        // rounds taken so far
    if (it >= max_iter) continue;           // gave up: counted as unconverged
    if (ghost_update(g, i, it, P.dens0[i], P.dens1[i])) atomicAdd(sent, 1);
  }
}

cudaError_t launch_ghost_catchup(const GhostArgs& g, int max_iter, const int* gate, int* sent,
                                 cudaStream_t s) {
  ghost_catchup<<<grid_for(g.hi - g.lo), 256, 0, s>>>(g, max_iter, gate, sent);
  return cudaGetLastError();
}

cudaError_t launch_ghost(const GhostArgs& g, cudaStream_t s) {
  ghost_round<<<grid_for(g.hi - g.lo), 256, 0, s>>>(g);
  return cudaGetLastError();
}

cudaError_t launch_begin_step(const DevParticles& p, int max_iter,
                              int* redo_count, float h_max, cudaStream_t s) {
  begin_step<<<grid_for(std::max(p.n, max_iter)), 256, 0, s>>>(p, max_iter, redo_count,
                                                                h_max);
  return cudaGetLastError();
}

cudaError_t launch_set_flags(uint8_t* flags, const int* idx, int n, uint8_t v,
                             cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  set_flags_k<<<grid_for(n), 256, 0, s>>>(flags, idx, n, v);
  return cudaGetLastError();
}

cudaError_t launch_gather_h(const float4* posh, const int* idx, int n, float* out,
                            cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  gather_h_k<<<grid_for(n), 256, 0, s>>>(posh, idx, n, out);
  return cudaGetLastError();
}

cudaError_t launch_sum_active_ngb(const DevParticles& p, unsigned long long* out,
                                  cudaStream_t s) {
  sum_active_ngb<<<grid_for(p.n), 256, 0, s>>>(p, out);
  return cudaGetLastError();
}

cudaError_t launch_end_force(const DevParticles& p, cudaStream_t s) {
  end_force_k<<<grid_for(p.n), 256, 0, s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_permute_in(DevParticles p, const int32_t* perm,
                              const double* x_in, const double* x_ref,
                              const float* v_in, const float* m_in,
                              const float* h_in, const float* u_in, int* differ,
                              cudaStream_t s) {
  permute_in<<<grid_for(p.n), 256, 0, s>>>(p, perm, x_in, x_ref, v_in, m_in, h_in, u_in,
                                           differ);
  return cudaGetLastError();
}

cudaError_t launch_verify_force_plan(DevParticles p, const int4* chk, int nchk,
                                    const uint8_t* planned, int* flag, cudaStream_t s) {
  if (nchk <= 0) return cudaSuccess;
  int g = (nchk + 7) / 8;  // 8 warps per block, one warp per cell
  const int cap = 16 * sm_count();
  g = g > cap ? cap : g;
  verify_force_plan<<<g, 256, 0, s>>>(p, chk, nchk, planned, flag);
  return cudaGetLastError();
}

cudaError_t launch_permute_vmu_in(DevParticles p, const int32_t* perm, const float* v,
                                  const float* m, const float* u, cudaStream_t s) {
  permute_vmu_in<<<grid_for(p.n), 256, 0, s>>>(p, perm, v, m, u);
  return cudaGetLastError();
}

// A caller's state (input order; null arrays keep the store's): velocities,
// masses, internal energies, the force inputs (rho, pressure, sound speed
// together; the grad-h term, the Balsara switch), time bins.
__global__ void set_state_k(DevParticles P, const int32_t* __restrict__ perm,
                            const float* __restrict__ v, const float* __restrict__ m,
                            const float* __restrict__ u, const float* __restrict__ rho,
                            const float* __restrict__ gf, const float* __restrict__ pr,
                            const float* __restrict__ cs, const float* __restrict__ bal,
                            const int8_t* __restrict__ tb, int8_t* __restrict__ tbin) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n;
       i += gridDim.x * blockDim.x) {
    const size_t k = (size_t)perm[i];
    if (v || m) {
      float4 vm = P.velm[i];
      if (v) {
        vm.x = v[3 * k];
        vm.y = v[3 * k + 1];
        vm.z = v[3 * k + 2];
      }
      if (m) vm.w = m[k];
      P.velm[i] = vm;
    }
    if (u) P.u[i] = u[k];
    if (rho || gf || bal) {
      // hydro_prepare_force's force inputs (as sphgpu_force_from_state)
      float4 f0 = P.fin0[i];
      float2 f1 = P.fin1[i];
      if (rho) {
        f0.x = rho[k];
        f0.z = pr[k] / (rho[k] * rho[k]);
        f0.w = cs[k];
        f1.y = pr[k];
      }
      if (gf) f0.y = gf[k];
      if (bal) f1.x = bal[k];
      P.fin0[i] = f0;
      P.fin1[i] = f1;
    }
    if (tb) tbin[i] = tb[k];
  }
}

cudaError_t launch_set_state(DevParticles p, const int32_t* perm, const float* v,
                             const float* m, const float* u, const float* rho,
                             const float* f, const float* pressure, const float* soundspeed,
                             const float* balsara, const int8_t* time_bin, int8_t* tbin,
                             cudaStream_t s) {
  set_state_k<<<grid_for(p.n), 256, 0, s>>>(p, perm, v, m, u, rho, f, pressure, soundspeed,
                                            balsara, time_bin, tbin);
  return cudaGetLastError();
}

cudaError_t launch_collect_out(DevParticles p, const int32_t* perm,
                               float* fields, int32_t* ints, cudaStream_t s) {
  collect_out<<<grid_for(p.n), 256, 0, s>>>(p, perm, fields, ints);
  return cudaGetLastError();
}

cudaError_t launch_prepare_posh(DevParticles p, const int32_t* top_of,
                                const double* top_loc, cudaStream_t s) {
  prepare_posh<<<grid_for(p.n), 256, 0, s>>>(p, top_of, top_loc);
  return cudaGetLastError();
}

}  // namespace sphgpu
