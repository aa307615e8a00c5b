// sph_kernels.cu -- sm_103a kernels of the SPH neighbour-interaction path:
// density gather (first pass and the ghost's re-runs), the ghost's
// Newton-Raphson update of h, and the force gather.
//
// Gather formulation: every updated particle i accumulates over its own
// neighbours in registers (no atomics, no cross-block reduction); a block
// owns a chunk of one leaf cell's particles and walks that leaf's gather
// list (partner cells with their reference evaluation frames).  Partner
// particles are staged in shared memory in j-tiles; TPI threads cooperate on
// one i-particle and reduce their partial sums with warp shuffles.
//
// The neighbour predicate r^2 < H^2 is first evaluated in FP32 from
// top-cell-relative offsets; pairs whose r^2 lies within a relative band of
// H^2 are re-evaluated exactly as the reference evaluates them (FP64
// positions, the reference's frame for that cell pair, no FMA contraction),
// so that neighbour sets match the reference bit for bit.  The physics of a
// hit follows hydro/Minimal/hydro_iact.h:137-189 (density) and :378-490
// (force), with the Wendland C2 kernel of kernel_hydro.h:121-147, :257-284.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "sph_kernels.cuh"

namespace sphgpu {

#define BLOCK 128

__device__ __forceinline__ void wendland_c2(float u, float& W, float& dW) {
  const float x = u * SPH_KG_INV;
  if (x >= 1.f) {  // second branch of the reference table: all zero
    W = 0.f;
    dW = 0.f;
    return;
  }
  float w = 4.f * x - 15.f;
  float dw = 4.f;
  dw = dw * x + w;
  w = x * w + 20.f;
  dw = dw * x + w;
  w = x * w - 10.f;
  dw = dw * x + w;
  w = x * w;
  dw = dw * x + w;
  w = x * w + 1.f;
  w = fmaxf(w, 0.f);
  dw = fminf(dw, 0.f);
  W = w * (SPH_KCONST * SPH_KG_INV_DIM);
  dW = dw * (SPH_KCONST * SPH_KG_INV_DIM1);
}

// Squared distance exactly as the reference loop owning this pair forms it.
__device__ __noinline__ float exact_r2(const double* __restrict__ xd, int u,
                                       int p, const Entry* __restrict__ E) {
  const int kind = E->kind;
  float d[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const double xu = xd[3 * (size_t)u + k];
    const double xp = xd[3 * (size_t)p + k];
    if (kind == FRAME_SELF_DBL) {
      d[k] = __double2float_rn(__dsub_rn(xu, xp));
    } else if (kind == FRAME_PAIR_ABS) {
      d[k] = __double2float_rn(__dsub_rn(__dsub_rn(xu, E->ou[k]), xp));
    } else {
      const float a = __double2float_rn(__dsub_rn(xu, E->ou[k]));
      const float b = __double2float_rn(__dsub_rn(xp, E->op[k]));
      d[k] = __fsub_rn(a, b);
    }
  }
  return __fadd_rn(__fadd_rn(__fmul_rn(d[0], d[0]), __fmul_rn(d[1], d[1])),
                   __fmul_rn(d[2], d[2]));
}

__device__ __forceinline__ float exact_h2(float h) {
  return __fmul_rn(__fmul_rn(h, h), SPH_KG2);
}

// ---------------------------------------------------------------------------
// Density gather

template <int TPI, int JT>
__global__ void __launch_bounds__(BLOCK)
density_gather(GatherArgs a, int mode, int persistent) {
  __shared__ float4 s_pos[JT];
  __shared__ float4 s_vm[JT];
  __shared__ int s_unit;
  const DevParticles& P = a.p;
  if (a.gate && *a.gate == 0) return;
  const int tid = threadIdx.x;
  const int slot = tid / TPI, sub = tid % TPI;
  int iter = 0;
  for (;;) {
    __syncthreads();
    if (tid == 0)
      s_unit = persistent ? atomicAdd(a.queue, 1) : (iter == 0 ? (int)blockIdx.x : a.nunits);
    __syncthreads();
    const int ui = s_unit;
    iter++;
    if (ui >= a.nunits) break;
    const Unit U = a.units[ui];
    const int i = U.i_first + slot;
    const bool valid = slot < U.i_count;
    float4 pi = make_float4(0.f, 0.f, 0.f, 1.f), vi = make_float4(0.f, 0.f, 0.f, 0.f);
    int dh = 0;
    bool upd = false;
    if (valid) {
      const uint8_t fl = P.flags[i];
      upd = (fl & 1) && (mode != MODE_REDO || (fl & 2));
      pi = P.posh[i];
      vi = P.velm[i];
      dh = P.depth_h[i];
    }
    if (!__syncthreads_or(upd)) continue;
    const float hi = pi.w;
    const float hig2 = exact_h2(hi);
    const float lo = hig2 * (1.f - a.band), hi2b = hig2 * (1.f + a.band);
    const float hi_inv = 1.f / hi;
    float rho = 0.f, rho_dh = 0.f, wc = 0.f, wc_dh = 0.f, divv = 0.f;
    float rx = 0.f, ry = 0.f, rz = 0.f;
    int ngb = 0;
    for (int e = U.e_begin; e < U.e_end; e++) {
      const Entry* E = &a.entries[e];
      const int first = __ldg(&E->first), cnt = __ldg(&E->count);
      const int mind = __ldg(&E->min_depth), maxd = __ldg(&E->max_depth);
      const bool ue = upd && dh >= mind && dh <= maxd;
      if (!__syncthreads_or(ue)) continue;
      const float fx = __ldg(&E->fdx), fy = __ldg(&E->fdy), fz = __ldg(&E->fdz);
      for (int base = 0; base < cnt; base += JT) {
        const int nt = min(JT, cnt - base);
        __syncthreads();
        for (int t = tid; t < nt; t += BLOCK) {
          const int j = first + base + t;
          float4 q = P.posh[j];
          q.x += fx;
          q.y += fy;
          q.z += fz;
          s_pos[t] = q;
          s_vm[t] = P.velm[j];
        }
        __syncthreads();
        if (ue) {
          for (int t = sub; t < nt; t += TPI) {
            const float4 q = s_pos[t];
            const float dx = pi.x - q.x, dy = pi.y - q.y, dz = pi.z - q.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (r2 < hi2b) {
              const int j = first + base + t;
              if (j == i) continue;
              if (r2 >= lo && !(exact_r2(P.xd, i, j, E) < hig2)) continue;
              const float4 vm = s_vm[t];
              const float mj = vm.w;
              const float r = sqrtf(r2);
              const float r_inv = r > 0.f ? 1.f / r : 0.f;
              const float ui_ = r * hi_inv;
              float W, dW;
              wendland_c2(ui_, W, dW);
              rho += mj * W;
              const float t3 = SPH_HDIM * W + ui_ * dW;
              rho_dh -= mj * t3;
              wc += W;
              wc_dh -= t3;
              const float fac = mj * dW * r_inv;
              const float dvx = vi.x - vm.x, dvy = vi.y - vm.y, dvz = vi.z - vm.z;
              const float dvdr = dvx * dx + dvy * dy + dvz * dz;
              divv -= fac * dvdr;
              rx += fac * (dvy * dz - dvz * dy);
              ry += fac * (dvz * dx - dvx * dz);
              rz += fac * (dvx * dy - dvy * dx);
              ngb++;
            }
          }
        }
      }
    }
#pragma unroll
    for (int off = TPI / 2; off > 0; off >>= 1) {
      rho += __shfl_xor_sync(0xffffffffu, rho, off);
      rho_dh += __shfl_xor_sync(0xffffffffu, rho_dh, off);
      wc += __shfl_xor_sync(0xffffffffu, wc, off);
      wc_dh += __shfl_xor_sync(0xffffffffu, wc_dh, off);
      divv += __shfl_xor_sync(0xffffffffu, divv, off);
      rx += __shfl_xor_sync(0xffffffffu, rx, off);
      ry += __shfl_xor_sync(0xffffffffu, ry, off);
      rz += __shfl_xor_sync(0xffffffffu, rz, off);
      ngb += __shfl_xor_sync(0xffffffffu, ngb, off);
    }
    if (upd && sub == 0) {
      if (mode == MODE_ACCUM) {
        float4 d0 = P.dens0[i], d1 = P.dens1[i];
        d0.x += rho;
        d0.y += rho_dh;
        d0.z += wc;
        d0.w += wc_dh;
        d1.x += divv;
        d1.y += rx;
        d1.z += ry;
        d1.w += rz;
        P.dens0[i] = d0;
        P.dens1[i] = d1;
        P.ngb_d[i] += ngb;
        P.ngb_d_first[i] += ngb;
      } else {
        P.dens0[i] = make_float4(rho, rho_dh, wc, wc_dh);
        P.dens1[i] = make_float4(divv, rx, ry, rz);
        P.ngb_d[i] = ngb;
        if (mode == MODE_FIRST) P.ngb_d_first[i] = ngb;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Force gather

template <int TPI, int JT>
__global__ void __launch_bounds__(BLOCK)
force_gather(GatherArgs a, int mode, int persistent) {
  __shared__ float4 s_pos[JT];   // offset xyz, h
  __shared__ float4 s_vm[JT];    // v, m
  __shared__ float4 s_f0[JT];    // rho, f, P/rho^2, c
  __shared__ float s_bal[JT];
  __shared__ float s_h2[JT];
  __shared__ int s_unit;
  const DevParticles& P = a.p;
  if (a.gate && *a.gate == 0) return;
  const int tid = threadIdx.x;
  const int slot = tid / TPI, sub = tid % TPI;
  int iter = 0;
  for (;;) {
    __syncthreads();
    if (tid == 0)
      s_unit = persistent ? atomicAdd(a.queue, 1) : (iter == 0 ? (int)blockIdx.x : a.nunits);
    __syncthreads();
    const int ui = s_unit;
    iter++;
    if (ui >= a.nunits) break;
    const Unit U = a.units[ui];
    const int i = U.i_first + slot;
    const bool valid = slot < U.i_count;
    float4 pi = make_float4(0.f, 0.f, 0.f, 1.f), vi = make_float4(0.f, 0.f, 0.f, 1.f);
    float4 fi = make_float4(1.f, 0.f, 0.f, 0.f);
    float bi = 0.f;
    int dh = 0;
    bool upd = false;
    if (valid) {
      upd = (P.flags[i] & 1) != 0;
      pi = P.posh[i];
      vi = P.velm[i];
      fi = P.fin0[i];
      bi = P.fin1[i].x;
      dh = P.depth_h[i];
    }
    if (!__syncthreads_or(upd)) continue;
    const float hi = pi.w;
    const float hig2 = exact_h2(hi);
    const float hi_inv = 1.f / hi;
    const float hi2 = hi_inv * hi_inv;
    const float hid_inv = hi2 * hi2;
    const float mi = vi.w;
    float ax = 0.f, ay = 0.f, az = 0.f, udt = 0.f, hdt = 0.f;
    float vsig = 2.f * fi.w;
    int ngb = 0;
    for (int e = U.e_begin; e < U.e_end; e++) {
      const Entry* E = &a.entries[e];
      const int first = __ldg(&E->first), cnt = __ldg(&E->count);
      const int mind = __ldg(&E->min_depth), maxd = __ldg(&E->max_depth);
      const bool ue = upd && dh >= mind && dh <= maxd;
      if (!__syncthreads_or(ue)) continue;
      const float fx = __ldg(&E->fdx), fy = __ldg(&E->fdy), fz = __ldg(&E->fdz);
      for (int base = 0; base < cnt; base += JT) {
        const int nt = min(JT, cnt - base);
        __syncthreads();
        for (int t = tid; t < nt; t += BLOCK) {
          const int j = first + base + t;
          float4 q = P.posh[j];
          q.x += fx;
          q.y += fy;
          q.z += fz;
          s_pos[t] = q;
          s_h2[t] = exact_h2(q.w);
          s_vm[t] = P.velm[j];
          s_f0[t] = P.fin0[j];
          s_bal[t] = P.fin1[j].x;
        }
        __syncthreads();
        if (ue) {
          for (int t = sub; t < nt; t += TPI) {
            const float4 q = s_pos[t];
            const float dx = pi.x - q.x, dy = pi.y - q.y, dz = pi.z - q.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            const float H2 = fmaxf(hig2, s_h2[t]);
            if (r2 < H2 * (1.f + a.band)) {
              const int j = first + base + t;
              if (j == i) continue;
              if (r2 >= H2 * (1.f - a.band) && !(exact_r2(P.xd, i, j, E) < H2)) continue;
              const float4 vm = s_vm[t];
              const float4 fj = s_f0[t];
              const float mj = vm.w;
              const float r = sqrtf(r2);
              const float r_inv = r > 0.f ? 1.f / r : 0.f;
              float Wi, dWi, Wj, dWj;
              wendland_c2(r * hi_inv, Wi, dWi);
              const float wi_dr = hid_inv * dWi;
              const float hj_inv = 1.f / q.w;
              const float hj2 = hj_inv * hj_inv;
              wendland_c2(r * hj_inv, Wj, dWj);
              const float wj_dr = hj2 * hj2 * dWj;
              const float f_ij = 1.f - fi.y / mj;
              const float f_ji = 1.f - fj.y / mi;
              const float Pi = fi.z * f_ij;
              const float Pj = fj.z * f_ji;
              const float dvx = vi.x - vm.x, dvy = vi.y - vm.y, dvz = vi.z - vm.z;
              const float dvdr = dvx * dx + dvy * dy + dvz * dz;
              const float omega = fminf(dvdr, 0.f);
              const float mu = r_inv * omega;
              const float vs = fi.w + fj.w - SPH_VISC_BETA * mu;
              const float rho_ij = 0.5f * (fi.x + fj.x);
              const float visc = -0.25f * vs * (bi + s_bal[t]) * mu / rho_ij;
              const float visc_acc = 0.5f * visc * (wi_dr * f_ij + wj_dr * f_ji) * r_inv;
              const float sph_acc = (Pi * wi_dr + Pj * wj_dr) * r_inv;
              const float accv = sph_acc + visc_acc;
              ax -= mj * accv * dx;
              ay -= mj * accv * dy;
              az -= mj * accv * dz;
              udt += (Pi * dvdr * r_inv * wi_dr + 0.5f * visc_acc * dvdr) * mj;
              hdt -= mj * dvdr * r_inv / fj.x * wi_dr * f_ij;
              vsig = fmaxf(vsig, vs);
              ngb++;
            }
          }
        }
      }
    }
#pragma unroll
    for (int off = TPI / 2; off > 0; off >>= 1) {
      ax += __shfl_xor_sync(0xffffffffu, ax, off);
      ay += __shfl_xor_sync(0xffffffffu, ay, off);
      az += __shfl_xor_sync(0xffffffffu, az, off);
      udt += __shfl_xor_sync(0xffffffffu, udt, off);
      hdt += __shfl_xor_sync(0xffffffffu, hdt, off);
      vsig = fmaxf(vsig, __shfl_xor_sync(0xffffffffu, vsig, off));
      ngb += __shfl_xor_sync(0xffffffffu, ngb, off);
    }
    if (upd && sub == 0) {
      if (mode == MODE_ACCUM) {
        float4 ac = P.acc[i];
        float2 hv = P.hdt_vsig[i];
        ac.x += ax;
        ac.y += ay;
        ac.z += az;
        ac.w += udt;
        hv.x += hdt;
        hv.y = fmaxf(hv.y, vsig);
        P.acc[i] = ac;
        P.hdt_vsig[i] = hv;
        P.ngb_f[i] += ngb;
      } else {
        // runner_do_end_hydro_force -> hydro_end_force (hydro.h:878) folded
        // in: every contribution to h_dt of an active particle is here.
        P.acc[i] = make_float4(ax, ay, az, udt);
        P.hdt_vsig[i] = make_float2(hdt * (hi * SPH_HDIM_INV), vsig);
        P.ngb_f[i] = ngb;
      }
    }
  }
}

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
}

__global__ void ghost_round(GhostArgs g) {
  if (g.iter > 0 && g.redo_count[g.iter - 1] == 0) return;
  const DevParticles& P = g.p;
  for (int i = g.lo + blockIdx.x * blockDim.x + threadIdx.x; i < g.hi;
       i += gridDim.x * blockDim.x) {
    const uint8_t fl = P.flags[i];
    if ((fl & 3) != 3) continue;
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
    bool done = false;
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
        continue;  // flags keep bit1: another round
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
    done = true;
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
    (void)done;
  }
}

__global__ void begin_step(DevParticles P, int max_iter, int* redo_count,
                           int* status) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid < max_iter) redo_count[tid] = 0;
  if (tid == 0) *status = 0;
  for (int i = tid; i < P.n; i += gridDim.x * blockDim.x) {
    float4 ph = P.posh[i];
    ph.w = P.h0[i];
    P.posh[i] = ph;
    const uint8_t fl = P.flags[i] & 1;
    P.flags[i] = fl ? 3 : 0;
    P.left[i] = 0.f;
    P.right[i] = 3.40282347e+38f;
    P.ghost_iters[i] = 0;
    P.dens0[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    P.dens1[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    P.ngb_d[i] = 0;
    P.ngb_d_first[i] = 0;
    P.ngb_f[i] = 0;
  }
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
                           const double* __restrict__ x, const float* __restrict__ v,
                           const float* __restrict__ m, const float* __restrict__ h,
                           const float* __restrict__ u, double* xd) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n;
       i += gridDim.x * blockDim.x) {
    const size_t k = (size_t)perm[i];
    xd[3 * (size_t)i + 0] = x[3 * k + 0];
    xd[3 * (size_t)i + 1] = x[3 * k + 1];
    xd[3 * (size_t)i + 2] = x[3 * k + 2];
    P.velm[i] = make_float4(v[3 * k], v[3 * k + 1], v[3 * k + 2], m[k]);
    P.h0[i] = h[k];
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

template <int TPI, int JT>
static cudaError_t launch_d(const GatherArgs& a, int mode, int persistent,
                            int num_sms, cudaStream_t s) {
  int grid = a.nunits;
  if (persistent) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, density_gather<TPI, JT>, BLOCK, 0);
    grid = std::min(a.nunits, std::max(1, per_sm) * num_sms);
  }
  if (grid <= 0) return cudaSuccess;
  density_gather<TPI, JT><<<grid, BLOCK, 0, s>>>(a, mode, persistent);
  return cudaGetLastError();
}

template <int TPI, int JT>
static cudaError_t launch_f(const GatherArgs& a, int mode, int persistent,
                            int num_sms, cudaStream_t s) {
  int grid = a.nunits;
  if (persistent) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, force_gather<TPI, JT>, BLOCK, 0);
    grid = std::min(a.nunits, std::max(1, per_sm) * num_sms);
  }
  if (grid <= 0) return cudaSuccess;
  force_gather<TPI, JT><<<grid, BLOCK, 0, s>>>(a, mode, persistent);
  return cudaGetLastError();
}

#define DISPATCH(FN)                                                         \
  switch (c.tpi * 1000 + c.jtile) {                                          \
    case 1064: return FN<1, 64>(a, mode, c.persistent, num_sms, s);          \
    case 1128: return FN<1, 128>(a, mode, c.persistent, num_sms, s);         \
    case 2064: return FN<2, 64>(a, mode, c.persistent, num_sms, s);          \
    case 2128: return FN<2, 128>(a, mode, c.persistent, num_sms, s);         \
    case 4064: return FN<4, 64>(a, mode, c.persistent, num_sms, s);          \
    case 4128: return FN<4, 128>(a, mode, c.persistent, num_sms, s);         \
    case 8064: return FN<8, 64>(a, mode, c.persistent, num_sms, s);          \
    case 8128: return FN<8, 128>(a, mode, c.persistent, num_sms, s);         \
    default: return cudaErrorInvalidValue;                                   \
  }

cudaError_t launch_density(const GatherArgs& a, int mode, const LaunchCfg& c,
                           int num_sms, cudaStream_t s) {
  DISPATCH(launch_d)
}

cudaError_t launch_force(const GatherArgs& a, int mode, const LaunchCfg& c,
                         int num_sms, cudaStream_t s) {
  DISPATCH(launch_f)
}

static int grid_for(int n) {
  int g = (n + 255) / 256;
  return g < 1 ? 1 : (g > 152 * 16 ? 152 * 16 : g);
}

cudaError_t launch_ghost(const GhostArgs& g, cudaStream_t s) {
  ghost_round<<<grid_for(g.hi - g.lo), 256, 0, s>>>(g);
  return cudaGetLastError();
}

cudaError_t launch_begin_step(const DevParticles& p, int max_iter,
                              int* redo_count, int* status, cudaStream_t s) {
  begin_step<<<grid_for(std::max(p.n, max_iter)), 256, 0, s>>>(p, max_iter, redo_count, status);
  return cudaGetLastError();
}

cudaError_t launch_end_force(const DevParticles& p, cudaStream_t s) {
  end_force_k<<<grid_for(p.n), 256, 0, s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_permute_in(DevParticles p, const int32_t* perm,
                              const double* x_in, const float* v_in,
                              const float* m_in, const float* h_in,
                              const float* u_in, cudaStream_t s) {
  permute_in<<<grid_for(p.n), 256, 0, s>>>(p, perm, x_in, v_in, m_in, h_in, u_in,
                                           const_cast<double*>(p.xd));
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
