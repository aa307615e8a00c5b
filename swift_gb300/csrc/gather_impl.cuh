// gather_impl.cuh -- the warp-per-particle gather kernel template (see
// gather.cu for the algorithm).  Included by gather.cu (the library's
// launches) and noalloc.cu (the variant that takes its scratch from a
// static device array).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "sph_kernels.cuh"

namespace sphgpu {

#ifndef WARPS_PER_BLOCK
#define WARPS_PER_BLOCK 8
#endif
#define FULL 0xffffffffu

// Where a gather writes its sums: OUT_STORE into the particle store (the
// library's own path); OUT_CALLER into caller-provided arrays in the
// caller's particle order (density only: float [n][8] sums, int32 [n]
// neighbour counts).
enum GatherOut { OUT_STORE = 0, OUT_CALLER = 1 };

struct CallerOut {
  float* fields;       // [n][8]
  int32_t* ngb;        // [n]
  const int32_t* perm; // store index -> caller index
};

static __device__ __forceinline__ void wendland(float u, float& W, float& dW) {
  const float x = u * SPH_KG_INV;
  if (x >= 1.f) {
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
  W = fmaxf(w, 0.f) * (SPH_KCONST * SPH_KG_INV_DIM);
  dW = fminf(dw, 0.f) * (SPH_KCONST * SPH_KG_INV_DIM1);
}

static __device__ __noinline__ float exact_r2_2(const double* __restrict__ xd, int u,
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

static __device__ __forceinline__ float h2_exact(float h) {
  return __fmul_rn(__fmul_rn(h, h), SPH_KG2);
}

struct WarpSmem {
  int j[64];
  float4 d[64];   // dx, dy, dz (i - j, in i's frame), r2
  int sb[32];     // surviving candidate blocks of the current chunk
  int se[32];     // their gather-list entries
  float4 sf[32];  // their frame offsets
};

template <bool FORCE, int OUT = OUT_STORE>
__global__ void __launch_bounds__(WARPS_PER_BLOCK * 32, 3)
gather_warp(G2Args a, CallerOut co = CallerOut{nullptr, nullptr, nullptr}) {
  __shared__ WarpSmem smem[WARPS_PER_BLOCK];
  const int lane = threadIdx.x & 31;
  WarpSmem& ws = smem[threadIdx.x >> 5];
  const DevParticles& P = a.p;
  const int count = a.count_ptr ? *a.count_ptr : a.count;
  const unsigned lt_mask = (1u << lane) - 1u;
  const float band = a.band;
  int base = 0, left = 0;
  for (;;) {
    if (left == 0) {
      int w = 0;
      if (lane == 0) w = atomicAdd(a.queue, 4);
      base = __shfl_sync(FULL, w, 0);
      left = 4;
    }
    const int w = base++;
    left--;
    if (w >= count) break;
    int i, p0, p1;
    if (a.items) {
      const int4 it = a.items[w];
      i = it.x;
      p0 = it.y;
      p1 = it.z;
    } else {
      i = a.list[w];
      const int leaf = P.leaf_of[i];
      p0 = a.leaf_pair_begin[leaf];
      p1 = a.leaf_pair_begin[leaf + 1];
    }
    const float4 pi = P.posh[i];
    const float4 vi = P.velm[i];
    const int dh = P.depth_h[i];
    const float hi = pi.w;
    const float hig2 = h2_exact(hi);
    const float hi_inv = 1.f / hi;
    float4 fi = make_float4(0.f, 0.f, 0.f, 0.f);
    float bi = 0.f, hid_inv = 0.f;
    if (FORCE) {
      fi = P.fin0[i];
      bi = P.fin1[i].x;
      const float t = hi_inv * hi_inv;
      hid_inv = t * t;
    }
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f, s4 = 0.f, s5 = 0.f, s6 = 0.f,
          s7 = 0.f;
    if (FORCE) s5 = 2.f * fi.w;
    int ngb = 0;
    int nbuf = 0;

    auto interact = [&](int j, float4 d) {
      const float r2 = d.w;
      const float4 vm = P.velm[j];
      const float mj = vm.w;
      const float r = sqrtf(r2);
      const float r_inv = r > 0.f ? 1.f / r : 0.f;
      const float dvx = vi.x - vm.x, dvy = vi.y - vm.y, dvz = vi.z - vm.z;
      const float dvdr = dvx * d.x + dvy * d.y + dvz * d.z;
      if (!FORCE) {
        const float ui = r * hi_inv;
        float W, dW;
        wendland(ui, W, dW);
        const float t3 = SPH_HDIM * W + ui * dW;
        s0 += mj * W;
        s1 -= mj * t3;
        s2 += W;
        s3 -= t3;
        const float fac = mj * dW * r_inv;
        s4 -= fac * dvdr;
        s5 += fac * (dvy * d.z - dvz * d.y);
        s6 += fac * (dvz * d.x - dvx * d.z);
        s7 += fac * (dvx * d.y - dvy * d.x);
      } else {
        const float hj = P.posh[j].w;
        const float4 fj = P.fin0[j];
        const float bj = P.fin1[j].x;
        float Wi, dWi, Wj, dWj;
        wendland(r * hi_inv, Wi, dWi);
        const float wi_dr = hid_inv * dWi;
        const float hj_inv = 1.f / hj;
        const float hj2 = hj_inv * hj_inv;
        wendland(r * hj_inv, Wj, dWj);
        const float wj_dr = hj2 * hj2 * dWj;
        const float f_ij = 1.f - fi.y / mj;
        const float f_ji = 1.f - fj.y / vi.w;
        const float Pi = fi.z * f_ij;
        const float Pj = fj.z * f_ji;
        const float mu = r_inv * fminf(dvdr, 0.f);
        const float vs = fi.w + fj.w - SPH_VISC_BETA * mu;
        const float visc = -0.25f * vs * (bi + bj) * mu / (0.5f * (fi.x + fj.x));
        const float visc_acc = 0.5f * visc * (wi_dr * f_ij + wj_dr * f_ji) * r_inv;
        const float acc = (Pi * wi_dr + Pj * wj_dr) * r_inv + visc_acc;
        s0 -= mj * acc * d.x;
        s1 -= mj * acc * d.y;
        s2 -= mj * acc * d.z;
        s3 += (Pi * dvdr * r_inv * wi_dr + 0.5f * visc_acc * dvdr) * mj;
        s4 -= mj * dvdr * r_inv / fj.x * wi_dr * f_ij;
        s5 = fmaxf(s5, vs);
      }
      ngb++;
    };

    // Test one surviving block: one partner particle per lane.
    auto test_block = [&](int k) {
      const int b = ws.sb[k];
      const int2 fc = a.bb_fc[b];
      const float4 fd = ws.sf[k];
      bool hit = false;
      float4 d = make_float4(0.f, 0.f, 0.f, 0.f);
      int j = -1;
      if (lane < fc.y) {
        j = fc.x + lane;
        const float4 q = P.posh[j];
        d.x = pi.x - (q.x + fd.x);
        d.y = pi.y - (q.y + fd.y);
        d.z = pi.z - (q.z + fd.z);
        d.w = d.x * d.x + d.y * d.y + d.z * d.z;
        const float H2 = FORCE ? fmaxf(hig2, h2_exact(q.w)) : hig2;
        if (d.w < H2 * (1.f + band) && j != i)
          hit = (d.w < H2 * (1.f - band)) ||
                (exact_r2_2(P.xd, i, j, &a.entries[ws.se[k]]) < H2);
      }
      const unsigned hm = __ballot_sync(FULL, hit);
      if (hit) {
        const int slot = nbuf + __popc(hm & lt_mask);
        ws.j[slot] = j;
        ws.d[slot] = d;
      }
      nbuf += __popc(hm);
      if (nbuf >= 32) {
        __syncwarp();
        interact(ws.j[lane], ws.d[lane]);
        __syncwarp();
        if (lane + 32 < nbuf) {
          ws.j[lane] = ws.j[lane + 32];
          ws.d[lane] = ws.d[lane + 32];
        }
        nbuf -= 32;
        __syncwarp();
      }
    };

    for (int c0 = p0; c0 < p1; c0 += 32) {
      const int p = c0 + lane;
      bool ov = false;
      int b = 0, e = 0;
      float4 fd = make_float4(0.f, 0.f, 0.f, 0.f);
      if (p < p1) {
        b = a.pair_block[p];
        e = a.pair_entry[p];
        const Entry* E = &a.entries[e];
        const int mind = E->min_depth, maxd = E->max_depth;
        fd = make_float4(E->fdx, E->fdy, E->fdz, 0.f);
        if (dh >= mind && dh <= maxd) {
          const float4 lo = a.bb_lo[b];
          const float4 hb = a.bb_hi[b];
          const float px = pi.x - fd.x, py = pi.y - fd.y, pz = pi.z - fd.z;
          const float dx = fmaxf(fmaxf(lo.x - px, px - hb.x), 0.f);
          const float dy = fmaxf(fmaxf(lo.y - py, py - hb.y), 0.f);
          const float dz = fmaxf(fmaxf(lo.z - pz, pz - hb.z), 0.f);
          const float R2 = FORCE ? fmaxf(hig2, lo.w) : hig2;
          ov = dx * dx + dy * dy + dz * dz < R2 * (1.f + 4.f * band) + 1e-30f;
        }
      }
      const unsigned mask = __ballot_sync(FULL, ov);
      if (ov) {
        const int slot = __popc(mask & lt_mask);
        ws.sb[slot] = b;
        ws.se[slot] = e;
        ws.sf[slot] = fd;
      }
      __syncwarp();
      const int nsurv = __popc(mask);
      for (int k = 0; k < nsurv; k++) test_block(k);
      __syncwarp();
    }
    __syncwarp();
    if (lane < nbuf) interact(ws.j[lane], ws.d[lane]);
    __syncwarp();
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      s0 += __shfl_xor_sync(FULL, s0, off);
      s1 += __shfl_xor_sync(FULL, s1, off);
      s2 += __shfl_xor_sync(FULL, s2, off);
      s3 += __shfl_xor_sync(FULL, s3, off);
      s4 += __shfl_xor_sync(FULL, s4, off);
      if (!FORCE) {
        s5 += __shfl_xor_sync(FULL, s5, off);
        s6 += __shfl_xor_sync(FULL, s6, off);
        s7 += __shfl_xor_sync(FULL, s7, off);
      } else {
        s5 = fmaxf(s5, __shfl_xor_sync(FULL, s5, off));
      }
      ngb += __shfl_xor_sync(FULL, ngb, off);
    }
    if (OUT == OUT_CALLER && lane == 0) {
      const size_t k = (size_t)co.perm[i];
      float* o = co.fields + 8 * k;
      o[0] = s0; o[1] = s1; o[2] = s2; o[3] = s3;
      o[4] = s4; o[5] = s5; o[6] = s6; o[7] = s7;
      co.ngb[k] = ngb;
    }
    if (OUT == OUT_STORE && lane == 0) {
      if (a.hits) atomicAdd(a.hits, (unsigned long long)ngb);
      if (!FORCE) {
        if (a.mode == MODE_ACCUM) {
          float4 d0 = P.dens0[i], d1 = P.dens1[i];
          d0.x += s0; d0.y += s1; d0.z += s2; d0.w += s3;
          d1.x += s4; d1.y += s5; d1.z += s6; d1.w += s7;
          P.dens0[i] = d0;
          P.dens1[i] = d1;
          P.ngb_d[i] += ngb;
          P.ngb_d_first[i] += ngb;
        } else {
          P.dens0[i] = make_float4(s0, s1, s2, s3);
          P.dens1[i] = make_float4(s4, s5, s6, s7);
          P.ngb_d[i] = ngb;
          if (a.mode == MODE_FIRST) P.ngb_d_first[i] = ngb;
        }
      } else {
        if (a.mode == MODE_ACCUM) {
          float4 ac = P.acc[i];
          float2 hv = P.hdt_vsig[i];
          ac.x += s0; ac.y += s1; ac.z += s2; ac.w += s3;
          hv.x += s4;
          hv.y = fmaxf(hv.y, s5);
          P.acc[i] = ac;
          P.hdt_vsig[i] = hv;
          P.ngb_f[i] += ngb;
        } else {
          // hydro_end_force (hydro.h:878) folded in
          P.acc[i] = make_float4(s0, s1, s2, s3);
          P.hdt_vsig[i] = make_float2(s4 * (hi * SPH_HDIM_INV), s5);
          P.ngb_f[i] = ngb;
        }
      }
    }
  }
}

}  // namespace sphgpu
