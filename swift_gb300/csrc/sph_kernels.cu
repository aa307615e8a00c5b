// sph_kernels.cu -- per-particle kernels of the SPH path (sm_103a): the
// ghost's Newton-Raphson round on h, step set-up, end of force, and the
// permutations between the caller's order and the cell-sorted store.  The
// neighbour gathers live in gather.cu.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "sph_kernels.cuh"

namespace sphgpu {

// ---------------------------------------------------------------------------
// Ghost: one Newton-Raphson round on h for every particle still iterating
// (runner_ghost.c:1113-1500; hydro.h:543-574, :626, :669-761).

__device__ void prepare_force(const DevParticles& P, int i, float h, float rho,
                              float wcount, float wcount_dh, float rho_dh,
                              float divv, float rx, float ry, float rz,
                              float u, float alpha, float hmax) {
  const float h_inv = 1.f / h;
  const float curl_v = sqrtf(rx * rx + ry * ry + rz * rz);
  const float abs_div = fabsf(divv);
  const float pressure = SPH_GAMMA_M1 * u * rho;
  const float c = sqrtf(SPH_GAMMA * pressure / rho);
  const float common = h * SPH_HDIM_INV / wcount;
  float grad_h;
  if (h > 0.9999f * hmax) {
    grad_h = 0.f;
  } else {
    const float gw = common * wcount_dh;
    grad_h = (gw < -0.9999f) ? 0.f : common * rho_dh / (1.f + gw);
  }
  const float balsara = alpha * abs_div / (abs_div + curl_v + 0.0001f * c * h_inv);
  P.fin0[i] = make_float4(rho, grad_h, pressure / (rho * rho), c);
  P.fin1[i] = make_float2(balsara, pressure);
  P.acc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  P.hdt_vsig[i] = make_float2(0.f, 2.f * c);
  if (P.ngb_bin) P.ngb_bin[i] = SPH_NUM_TIME_BINS + 1;  // timestep_limiter_prepare_force
}

__global__ void ghost_round(GhostArgs g) {
  if (g.iter > 0 && g.redo_count[g.iter - 1] == 0) return;
  const DevParticles& P = g.p;
  for (int i = g.lo + blockIdx.x * blockDim.x + threadIdx.x; i < g.hi;
       i += gridDim.x * blockDim.x) {
    const uint8_t fl = P.flags[i];
    if ((fl & 3) != 3) continue;  // active and still iterating
    P.ghost_iters[i] = g.iter + 1;
    float4 ph = P.posh[i];
    const float h_old = ph.w;
    const float h_old_dim = h_old * h_old * h_old;
    const float h_old_dim_m1 = h_old * h_old;
    float4 d0 = P.dens0[i], d1 = P.dens1[i];
    float rho = d0.x, rho_dh = d0.y, wc = d0.z, wc_dh = d0.w;
    float divv = d1.x, rx = d1.y, ry = d1.z, rz = d1.w;
    float left = P.left[i], right = P.right[i];
    const float mass = P.velm[i].w;
    float h_new;
    bool no_ngb = false;
    if ((double)wc < 1.e-5 * (double)SPH_KROOT) {
      no_ngb = true;
      h_new = 2.f * h_old;
    } else {
      // hydro_end_density
      const float h_inv = 1.f / h_old;
      const float hid = h_inv * h_inv * h_inv;
      const float hid1 = hid * h_inv;
      rho += mass * SPH_KROOT;
      rho_dh -= SPH_HDIM * mass * SPH_KROOT;
      wc += SPH_KROOT;
      wc_dh -= SPH_HDIM * SPH_KROOT;
      rho *= hid;
      rho_dh *= hid1;
      wc *= hid;
      wc_dh *= hid1;
      const float rho_inv = 1.f / rho;
      rx *= hid1 * rho_inv;
      ry *= hid1 * rho_inv;
      rz *= hid1 * rho_inv;
      divv *= hid1 * rho_inv;
      const float n_sum = wc * h_old_dim;
      const float f = n_sum - g.eta_dim;
      const float fp = wc_dh * h_old_dim + SPH_HDIM * wc * h_old_dim_m1;
      if (n_sum < g.eta_dim)
        left = fmaxf(left, h_old);
      else if (n_sum > g.eta_dim)
        right = fminf(right, h_old);
      if ((h_old >= g.h_max && f < 0.f) || (h_old <= g.h_min && f > 0.f)) {
        prepare_force(P, i, h_old, rho, wc, wc_dh, rho_dh, divv, rx, ry, rz,
                      P.u[i], g.alpha, g.h_max);
        P.flags[i] = fl & ~2;
        P.left[i] = left;
        P.right[i] = right;
        continue;
      }
      h_new = h_old - f / (fp + 1.17549435e-38f);
      h_new = fminf(h_new, 2.f * h_old);
      h_new = fmaxf(h_new, 0.5f * h_old);
      h_new = fmaxf(h_new, left);
      h_new = fminf(h_new, right);
    }
    float h = h_old;
    if (fabsf(h_new - h_old) > g.h_tol * h_old) {
      if ((h_new == left && h_old == right) || (h_old == left && h_new == right)) {
        h = cbrtf(0.5f * (left * left * left + right * right * right));
      } else {
        h = h_new;
      }
      if (h < g.h_max && h > g.h_min) {
        ph.w = h;
        P.posh[i] = ph;
        P.left[i] = left;
        P.right[i] = right;
        atomicAdd(&g.redo_count[g.iter], 1);
        continue;  // flags keep bit 1: another round
      } else if (h <= g.h_min) {
        h = g.h_min;
      } else {
        h = g.h_max;
        if (no_ngb) {
          const float hinv = 1.f / h;
          const float hid = hinv * hinv * hinv;
          rho = mass * SPH_KROOT * hid;
          wc = SPH_KROOT * hid;
          rho_dh = 0.f;
          wc_dh = 0.f;
          divv = rx = ry = rz = 0.f;
        }
      }
    }
    // cell_set_part_h_depth (cell.h:1787) on the particle's leaf chain
    const LeafInfo* L = &g.leaves[P.leaf_of[i]];
    if (h < L->hmin[0]) {
      P.depth_h[i] = L->depth[0];
    } else {
      for (int lev = 0; lev < L->nlevels; lev++)
        if (h >= L->hmin[lev] && h < L->hmax[lev]) {
          P.depth_h[i] = L->depth[lev];
          break;
        }
    }
    ph.w = h;
    P.posh[i] = ph;
    P.left[i] = left;
    P.right[i] = right;
    prepare_force(P, i, h, rho, wc, wc_dh, rho_dh, divv, rx, ry, rz, P.u[i],
                  g.alpha, g.h_max);
    P.flags[i] = fl & ~2;
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
      o[19] = hv.x; o[20] = hv.y; o[21] = 0.f; o[22] = 0.f; o[23] = 0.f;
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
  return g < 1 ? 1 : (g > 152 * 16 ? 152 * 16 : g);
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
