// ghost_impl.cuh -- the ghost's per-particle Newton-Raphson update on h
// (runner_ghost.c:1113-1500; hydro_end_density hydro.h:543-574,
// hydro_part_has_no_neighbours :626, hydro_prepare_force :669-739,
// hydro_reset_acceleration :749-761), shared by the round kernel
// (sph_kernels.cu) and the list solver (gather_impl.cuh).
#pragma once
#include "sph_kernels.cuh"

namespace sphgpu {
namespace {

__device__ __forceinline__ void prepare_force(const DevParticles& P, int i, float h, float rho,
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

// One update of particle i at round `iter` from its density sums at its
// current h (d0 = rho, rho_dh, wcount, wcount_dh; d1 = div_v, rot_v[3]).
// Returns 1 when i needs another round (its new h is in posh.w), 0 when it
// is done (h final, force inputs prepared).
__device__ __forceinline__ int ghost_update(const GhostArgs& g, int i, int iter, float4 d0,
                                            float4 d1) {
  const DevParticles& P = g.p;
  const uint8_t fl = P.flags[i];
  P.ghost_iters[i] = iter + 1;
  float4 ph = P.posh[i];
  const float h_old = ph.w;
  const float h_old_dim = h_old * h_old * h_old;
  const float h_old_dim_m1 = h_old * h_old;
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
      return 0;
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
      atomicAdd(&g.redo_count[iter], 1);
      return 1;  // flags keep bit 1: another round
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
  return 0;
}

}  // namespace
}  // namespace sphgpu
