// gather_impl.cuh -- the warp-per-particle gather kernel template (see
// gather.cu for the algorithm).  Included by gather.cu (the library's
// launches) and noalloc.cu (the variant that takes its scratch from a
// static device array).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "ghost_impl.cuh"
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

// Density sums of one hit (runner_iact_nonsym_density, hydro_iact.h:137-189);
// dx = x_i - x_j in the group's frame.
static __device__ __forceinline__ void density_hit(float dx, float dy, float dz, float r2,
                                                   const float4& vi, const float4& vm,
                                                   float hi_inv, float& s0, float& s1,
                                                   float& s2, float& s3, float& s4,
                                                   float& s5, float& s6, float& s7) {
  const float mj = vm.w;
  // hardware reciprocal square root (MUFU.RSQ, ~2 ulp): the sums are held
  // to 1e-4 relative, and the neighbour decision was made exactly
  const float r_inv = r2 > 0.f ? rsqrtf(r2) : 0.f;
  const float r = r2 * r_inv;
  const float dvx = vi.x - vm.x, dvy = vi.y - vm.y, dvz = vi.z - vm.z;
  const float dvdr = dvx * dx + dvy * dy + dvz * dz;
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
  s5 += fac * (dvy * dz - dvz * dy);
  s6 += fac * (dvz * dx - dvx * dz);
  s7 += fac * (dvx * dy - dvy * dx);
}

// Per-warp shared memory: the staged partner block and each lane's ring of
// pending hits (partner index and frame-offset index packed in 32 bits).
#define QCAP 32  // power of two: ring positions wrap with & (QCAP - 1)
struct LaneSmem {
  float4 jp[32];       // staged block, candidates in pairs (2p, 2p+1):
                       // jp[2p] = -(x, x', y, y'), jp[2p+1] = (-z, -z', (K h)^2,
                       // (K h')^2), positions offset into the group's frame
  int sfirst[32];      // surviving candidate blocks of the current chunk
  int scount[32];
  int se[32];
  int sdep[32];        // their entries' depth window: min | max << 8, and the
                       // runs of 8 the group can reach << 16
  float4 sf[32];       // their frame offsets (w: frame-offset index)
  float4 slo[32];      // their boxes
  float4 shi[32];
  int q[QCAP][32];     // per-lane hit ring
  int lb[8][32];       // per-lane staging of neighbour-list items (LISTS)
  float4 ftab[27];     // frame offsets of the 27 partner top cells (offset_of)
};

// Per-warp staging of the bulk-copy variant (BULK): the next block's records
// as they lie in the store, and the mbarrier its copy completes on.
struct BulkSmem {
  float4 raw[32];
  unsigned long long bar;  // transaction bytes of one copy
  unsigned parity;         // phase of bar the next copy completes
};

// --- bulk copies (the TMA engine's untiled cp.async.bulk) ------------------
// A j-block is a contiguous run of the store, so its records (16 bytes
// each, 16-byte aligned) can be fetched by one bulk copy issued by one lane
// into the warp's shared memory, completing on an mbarrier.
__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void bulk_bar_init(unsigned long long* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
  // the barrier's initialisation is seen by the async proxy before any copy
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void bulk_fetch(float4* dst, const float4* src, int count,
                                           unsigned long long* bar) {
  const unsigned bytes = 16u * (unsigned)count;
  // earlier generic-proxy reads of dst are ordered before the async write
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
               ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}
// Wait for the barrier's phase `parity` to complete, at most `tries` polls
// (each poll may suspend the thread for a while); false when it did not.
__device__ __forceinline__ bool bulk_wait(unsigned long long* bar, unsigned parity, int tries) {
  for (int t = 0; t < tries; t++) {
    unsigned done;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; "
        "selp.u32 %0, 1, 0, p; }"
        : "=r"(done) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    if (done) return true;
  }
  return false;
}
#define BULK_WAIT_TRIES (1 << 20)

// Frame offset of a partner top cell from its index in the 3x3x3
// neighbourhood of the group's top cell (ix + 3 iy + 9 iz, each in 0..2).
__device__ __forceinline__ float3 offset_of(int idx, float3 tw) {
  return make_float3((float)(idx % 3 - 1) * tw.x, (float)((idx / 3) % 3 - 1) * tw.y,
                     (float)(idx / 9 - 1) * tw.z);
}

// One warp = one group of <= 32 particles of a leaf (one lane each).
//   1. the group's box, grown by the largest search radius, culls the
//      leaf's candidate blocks 32 at a time (one per lane), survivors are
//      compacted into shared memory;
//   2. each survivor is tested against every lane's own search sphere
//      (skipped when no lane reaches it), then staged in shared memory with
//      the frame offset applied;
//   3. every lane tests its own particle against each staged partner
//      (broadcast reads), eight at a time into bit masks: FP32 r^2 below a
//      2^-12 band around H^2 is a hit, pushed to the lane's ring from the
//      mask; candidates inside the band are decided by the exact FP64
//      predicate in the reference frame;
//   4. when a ring is nearly full, all lanes compute interactions from
//      their rings for about as many passes as the rings hold on average;
//      the last drain empties them.  Sums stay in the lane's registers.
// LISTS (density re-runs): also record every candidate below the band's top
// into the particle's neighbour list (G2Args::nl).
// TPP (threads per particle, 1 or 2): a warp serves 32 / TPP particles of a
// window; the TPP lanes of a particle split each staged block's candidates
// and add their partial sums at the end.
// BULK: each surviving j-block is fetched into shared memory by one bulk
// copy (cp.async.bulk, one lane) while the previous one is tested, instead
// of a register load per lane.
template <bool FORCE, int OUT = OUT_STORE, int WPB = WARPS_PER_BLOCK, int MINB = 3,
          bool LISTS = false, int TPP = 1, bool BULK = false>
__global__ void __launch_bounds__(WPB * 32, MINB)
gather_lanes(G2Args a, CallerOut co = CallerOut{nullptr, nullptr, nullptr}) {
  static_assert(TPP == 1 || TPP == 2 || TPP == 4, "one, two or four lanes per particle");
  static_assert(TPP == 1 || (OUT == OUT_STORE && (!LISTS || TPP == 2)),
                "several lanes: stored sums; lists with one or two lanes");
  __shared__ LaneSmem smem[WPB];
  __shared__ BulkSmem bsm[BULK ? WPB : 1];
  const int lane = threadIdx.x & 31;
  const int sub = lane % TPP, pl = lane / TPP;  // lane within the particle, particle
  LaneSmem& ws = smem[threadIdx.x >> 5];
  const DevParticles& P = a.p;
  if (a.gate && *a.gate == 0) return;
  const int nunits = a.count_ptr ? *a.count_ptr : a.count;
  const unsigned lt_mask = (1u << lane) - 1u;
  const float band = a.band;
  float3 tw = a.top_width;
  // frame offsets by index, looked up for every hit (the warp's own table:
  // with per-leaf top widths it changes between groups)
  auto fill_ftab = [&]() {
    if (lane < 27) {
      const float3 o = offset_of(lane, tw);
      ws.ftab[lane] = make_float4(o.x, o.y, o.z, 0.f);
    }
    __syncwarp();
  };
  fill_ftab();
  BulkSmem& wb = bsm[BULK ? (threadIdx.x >> 5) : 0];
  if (BULK) {
    if (lane == 0) {
      bulk_bar_init(&wb.bar);
      wb.parity = 0u;
    }
    __syncwarp();
  }
  for (;;) {
    int u = 0;
    if (lane == 0) u = atomicAdd(a.queue, 1);
    u = __shfl_sync(FULL, u, 0);
    if (u >= nunits) break;
    const int4 U = a.units[u];  // base, mask, pair begin, pair end
    if (U.y == 0) continue;     // no particle of this window takes part
    if (a.leaf_tw) {
      const float4 t = a.leaf_tw[P.leaf_of[U.x]];
      if (t.x != tw.x || t.y != tw.y || t.z != tw.z) {
        tw = make_float3(t.x, t.y, t.z);
        __syncwarp();
        fill_ftab();
      }
    }
    const bool valid = (U.y >> pl) & 1;
    const int i = U.x + pl;
    float4 pi = make_float4(0.f, 0.f, 0.f, 0.f), vi = make_float4(0.f, 0.f, 0.f, 1.f);
    float4 fi = make_float4(1.f, 0.f, 0.f, 0.f);
    float bi = 0.f;
    int dh = 0;
    if (valid) {
      pi = P.posh[i];
      vi = P.velm[i];
      dh = P.depth_h[i];
      if (FORCE) {
        fi = P.fin0[i];
        bi = P.fin1[i].x;
      }
    }
    const float hi = valid ? pi.w : 1.f;
    const float hig2 = valid ? h2_exact(hi) : 0.f;
    const float hi_inv = 1.f / hi;
    const float hid_inv = (hi_inv * hi_inv) * (hi_inv * hi_inv);
    const float mi_inv = 1.f / vi.w;
    const float lo2 = hig2 * (1.f - band), hi2 = hig2 * (1.f + band);
    // recording bound of the lists (r^2, FP32) and the radius the culls use
    float lw2 = hi2;
    if (LISTS && valid && a.nl_widen > 1.f) {
      const LeafInfo& L = a.leaves[P.leaf_of[i]];
      float cover = 0.f;
      for (int lev = 0; lev < L.nlevels; lev++)
        if (L.depth[lev] == dh) cover = SPH_KG * L.hmax[lev] * (1.f - 1.f / 1024.f);
      lw2 = fmaxf(hi2, fminf(hi2 * a.nl_widen, cover * cover));
    }
    const float cr2 = LISTS ? lw2 : hig2;
    const float2 pix2 = make_float2(pi.x, pi.x), piy2 = make_float2(pi.y, pi.y),
                 piz2 = make_float2(pi.z, pi.z);
    const float2 lo22 = make_float2(lo2, lo2), hi22 = make_float2(hi2, hi2);
    const float2 omb2 = make_float2(1.f - band, 1.f - band), opb2 = make_float2(1.f + band, 1.f + band);
    // Recording re-run: the list keeps every candidate below the band's top,
    // which covers any later re-run whose h is not larger (Newton's iterates
    // on the increasing, convex n(h) - eta^3 fall towards the root after the
    // first step, so almost all of them are)
    int lcnt = 0;
    // group box grown by the group's largest radius
    float gx0 = valid ? pi.x : 3.4e38f, gy0 = valid ? pi.y : 3.4e38f,
          gz0 = valid ? pi.z : 3.4e38f;
    float gx1 = valid ? pi.x : -3.4e38f, gy1 = valid ? pi.y : -3.4e38f,
          gz1 = valid ? pi.z : -3.4e38f;
    float gh2 = cr2;
    int gd0 = valid ? dh : 1 << 20, gd1 = valid ? dh : -(1 << 20);  // depth range
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      gd0 = min(gd0, __shfl_xor_sync(FULL, gd0, off));
      gd1 = max(gd1, __shfl_xor_sync(FULL, gd1, off));
      gx0 = fminf(gx0, __shfl_xor_sync(FULL, gx0, off));
      gy0 = fminf(gy0, __shfl_xor_sync(FULL, gy0, off));
      gz0 = fminf(gz0, __shfl_xor_sync(FULL, gz0, off));
      gx1 = fmaxf(gx1, __shfl_xor_sync(FULL, gx1, off));
      gy1 = fmaxf(gy1, __shfl_xor_sync(FULL, gy1, off));
      gz1 = fmaxf(gz1, __shfl_xor_sync(FULL, gz1, off));
      gh2 = fmaxf(gh2, __shfl_xor_sync(FULL, gh2, off));
    }
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f, s4 = 0.f, s5 = 0.f, s6 = 0.f,
          s7 = 0.f;
    if (FORCE) s5 = 2.f * fi.w;
    int ngb = 0;
    int nbin = SPH_NUM_TIME_BINS + 1;  // smallest time bin > 0 of the force neighbours
    int qh = 0, qt = 0;  // ring head / tail (pending hits: qt - qh)

    auto interact = [&](int packed) {
      const int j = packed & 0x07ffffff;
      const float4 fd = ws.ftab[(unsigned)packed >> 27];
      const float4 q = P.posh[j];
      const float dx = pi.x - (q.x + fd.x), dy = pi.y - (q.y + fd.y),
                  dz = pi.z - (q.z + fd.z);
      const float r2 = dx * dx + dy * dy + dz * dz;
      const float4 vm = P.velm[j];
      if (!FORCE) {
        density_hit(dx, dy, dz, r2, vi, vm, hi_inv, s0, s1, s2, s3, s4, s5, s6, s7);
      } else {
        const float mj = vm.w;
        // hardware reciprocal square root (MUFU.RSQ, ~2 ulp): the sums are
        // held to 1e-4 relative, and the neighbour decision was made exactly
        const float r_inv = r2 > 0.f ? rsqrtf(r2) : 0.f;
        const float r = r2 * r_inv;
        const float dvx = vi.x - vm.x, dvy = vi.y - vm.y, dvz = vi.z - vm.z;
        const float dvdr = dvx * dx + dvy * dy + dvz * dz;
        const float hj = q.w;
        const float4 fj = P.fin0[j];
        const float bj = P.fin1[j].x;
        float Wi, dWi, Wj, dWj;
        wendland(r * hi_inv, Wi, dWi);
        const float wi_dr = hid_inv * dWi;
        const float hj_inv = __fdividef(1.f, hj);
        const float hj2 = hj_inv * hj_inv;
        wendland(r * hj_inv, Wj, dWj);
        const float wj_dr = hj2 * hj2 * dWj;
        const float f_ij = 1.f - __fdividef(fi.y, mj);
        const float f_ji = 1.f - fj.y * mi_inv;
        const float Pi = fi.z * f_ij;
        const float Pj = fj.z * f_ji;
        const float mu = r_inv * fminf(dvdr, 0.f);
        const float vs = fi.w + fj.w - SPH_VISC_BETA * mu;
        const float visc =
            __fdividef(-0.25f * vs * (bi + bj) * mu, 0.5f * (fi.x + fj.x));
        const float visc_acc = 0.5f * visc * (wi_dr * f_ij + wj_dr * f_ji) * r_inv;
        const float acc = (Pi * wi_dr + Pj * wj_dr) * r_inv + visc_acc;
        s0 -= mj * acc * dx;
        s1 -= mj * acc * dy;
        s2 -= mj * acc * dz;
        s3 += (Pi * dvdr * r_inv * wi_dr + 0.5f * visc_acc * dvdr) * mj;
        s4 -= __fdividef(mj * dvdr * r_inv, fj.x) * wi_dr * f_ij;
        s5 = fmaxf(s5, vs);
        if (P.tbin) {  // runner_iact_nonsym_timebin (timestep_limiter_iact.h:64)
          const int tb = P.tbin[j];
          if (tb > 0) nbin = min(nbin, tb);
        }
      }
      ngb++;
    };

    // Hits are computed in passes over the rings: a pass takes the same
    // ring position from every lane.  A partial drain (when a ring is
    // nearly full) runs about as many positions as the lanes hold on
    // average, so that most lanes have work in every pass; the rest stays
    // queued.  The final drain empties every ring.
    auto drain = [&](bool all) {
      const int cnt = qt - qh;
      const int mx = (int)__reduce_max_sync(FULL, (unsigned)cnt);
      int m = mx;
      if (!all) {
        const int sum = (int)__reduce_add_sync(FULL, (unsigned)cnt);
        m = min(mx, max(8, (sum + 31) / 32 + 4));
      }
      __syncwarp();
      for (int k = 0; k < m; k++)
        if (k < cnt) interact(ws.q[(qh + k) & (QCAP - 1)][lane]);
      qh += min(m, cnt);
      __syncwarp();
    };
    auto push = [&](int v) {
      ws.q[qt & (QCAP - 1)][lane] = v;
      qt++;
    };
    // at most 8 pushes per lane between two of these checks
    auto room = [&]() {
      if (__any_sync(FULL, qt - qh > QCAP - 8)) drain(false);
    };

    // Force from the first pass's rows: when every lane's row covers its own
    // radius and the largest radius among the blocks the group reaches (the
    // cull below), each row holds every force partner of its particle
    // (r < max(H_i, H_j) < the row's bound), and the candidate search is
    // skipped: the rows' items are tested instead, with the same criterion.
    bool use_rows = false;
    int rcnt = 0, rc0 = 0;
    if (FORCE && a.force_rows) {
      bool ok = true;
      float rT = 3.4e38f;
      if (valid) {
        const int c = a.nl_cnt[i];
        rT = a.nl_T[i];
        if (c < 0 || !(hi2 <= rT)) {
          ok = false;
        } else {
          rc0 = a.nl_seg == 2 ? (c & 0xffff) : c;
          rcnt = rc0 + (a.nl_seg == 2 ? c >> 16 : 0);
        }
      }
      if (__all_sync(FULL, ok)) {
        float maxW = 0.f;
        for (int c0 = U.z; c0 < U.w; c0 += 32) {
          const int p = c0 + lane;
          if (p < U.w) {
            const int b = a.pair_block[p];
            const Entry* E = &a.entries[a.pair_entry[p]];
            const float4 lo = a.bb_lo[b], hb = a.bb_hi[b];
            const float dx = fmaxf(fmaxf(lo.x + E->fdx - gx1, gx0 - hb.x - E->fdx), 0.f);
            const float dy = fmaxf(fmaxf(lo.y + E->fdy - gy1, gy0 - hb.y - E->fdy), 0.f);
            const float dz = fmaxf(fmaxf(lo.z + E->fdz - gz1, gz0 - hb.z - E->fdz), 0.f);
            if (dx * dx + dy * dy + dz * dz < fmaxf(gh2, lo.w) * (1.f + 4.f * band) + 1e-30f &&
                gd1 >= E->min_depth && gd0 <= E->max_depth)
              maxW = fmaxf(maxW, lo.w);
          }
        }
        float minT = rT;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          maxW = fmaxf(maxW, __shfl_xor_sync(FULL, maxW, off));
          minT = fminf(minT, __shfl_xor_sync(FULL, minT, off));
        }
        use_rows = maxW * (1.f + band) <= minT;
      }
    }
    if (FORCE && use_rows) {
      // each lane reads the row segment it recorded in the first pass (the
      // first pass ran with the same lanes per particle), four items per
      // 16-byte load, the partners' positions all in flight together
      const int* row = a.nl + (size_t)(valid ? i : 0) * a.nl_cap;
      const bool own_seg = a.nl_seg == TPP;
      const int nmine = !valid ? 0
                        : own_seg ? (TPP == 1 ? rcnt : (sub == 0 ? rc0 : rcnt - rc0))
                                  : (rcnt - sub + TPP - 1) / TPP;
      const int* seg = row + (own_seg ? sub * (a.nl_cap / TPP) : 0);
      const int kmax = (int)__reduce_max_sync(FULL, (unsigned)max(nmine, 0));
      auto test_item = [&](int pk, const float4& q) {
        const int j = pk & 0x07ffffff;
        const float4 fd = ws.ftab[(unsigned)pk >> 27];
        const float dx = pi.x - (q.x + fd.x), dy = pi.y - (q.y + fd.y), dz = pi.z - (q.z + fd.z);
        const float r2 = dx * dx + dy * dy + dz * dz;
        const float H2 = fmaxf(hig2, h2_exact(q.w));
        if (r2 < H2 * (1.f - band)) {
          push(pk);
        } else if (r2 < H2 * (1.f + band)) {
          // exact, in the frame of the force-list entry pairing the leaf
          // with the partner's block at this particle's depth
          const int blk = a.blk_of[j];
          const Entry* E = nullptr;
          for (int p = U.z; p < U.w && !E; p++)
            if (a.pair_block[p] == blk) {
              const Entry* X = &a.entries[a.pair_entry[p]];
              if (dh >= X->min_depth && dh <= X->max_depth) E = X;
            }
          if (E && exact_r2_2(P.xd, i, j, E) < H2) push(pk);
        }
      };
      for (int k0 = 0; k0 < kmax; k0 += 8) {
#pragma unroll
        for (int h4 = 0; h4 < 8; h4 += 4) {
          int pk[4];
          if (own_seg) {
            // k0 + h4 + 4 stays inside the segment's capacity (a multiple of 8)
            const int4 v4 = k0 + h4 < nmine ? *reinterpret_cast<const int4*>(seg + k0 + h4)
                                            : make_int4(i, i, i, i);
            pk[0] = v4.x; pk[1] = v4.y; pk[2] = v4.z; pk[3] = v4.w;
          } else {
#pragma unroll
            for (int u = 0; u < 4; u++) {
              const int t = sub + (k0 + h4 + u) * TPP;
              pk[u] = k0 + h4 + u < nmine ? row[t < rc0 ? t : t - rc0 + a.nl_cap / 2] : i;
            }
          }
          float4 q[4];
          unsigned okm = 0u;  // items to test (the packed items use the sign bit)
#pragma unroll
          for (int u = 0; u < 4; u++) {
            // an item always names a store particle; anything else is skipped
            const bool ok = k0 + h4 + u < nmine && (pk[u] & 0x07ffffff) < P.n &&
                            ((unsigned)pk[u] >> 27) <= 26;
            okm |= ok ? 1u << u : 0u;
            q[u] = P.posh[ok ? (pk[u] & 0x07ffffff) : (valid ? i : 0)];
          }
#pragma unroll
          for (int u = 0; u < 4; u++)
            if (okm & (1u << u)) test_item(pk[u], q[u]);
        }
        room();  // at most 8 pushes per lane since the last check
      }
    }
    for (int c0 = U.z; c0 < (FORCE && use_rows ? U.z : U.w); c0 += 32) {
      const int p = c0 + lane;
      bool ov = false;
      int e = 0;
      float4 fd = make_float4(0.f, 0.f, 0.f, 0.f), lo = fd, hb = fd;
      int2 fc = make_int2(0, 0);
      int dep = 0;
      if (p < U.w) {
        const int b = a.pair_block[p];
        e = a.pair_entry[p];
        const Entry* E = &a.entries[e];
        fd = make_float4(E->fdx, E->fdy, E->fdz, 0.f);
        dep = (int)(uint8_t)E->min_depth | (int)(uint8_t)E->max_depth << 8;
        lo = a.bb_lo[b];
        hb = a.bb_hi[b];
        const float dx = fmaxf(fmaxf(lo.x + fd.x - gx1, gx0 - hb.x - fd.x), 0.f);
        const float dy = fmaxf(fmaxf(lo.y + fd.y - gy1, gy0 - hb.y - fd.y), 0.f);
        const float dz = fmaxf(fmaxf(lo.z + fd.z - gz1, gz0 - hb.z - fd.z), 0.f);
        const float R2 = FORCE ? fmaxf(gh2, lo.w) : gh2;
        // the box reaches the group and some lane's depth may use the entry
        ov = dx * dx + dy * dy + dz * dz < R2 * (1.f + 4.f * band) + 1e-30f &&
             gd1 >= E->min_depth && gd0 <= E->max_depth;
        if (ov) {
          fc = a.bb_fc[b];
          // frame-offset index of the partner top cell (for the queues)
          const int ix = (int)rintf(fd.x / tw.x) + 1, iy = (int)rintf(fd.y / tw.y) + 1,
                    iz = (int)rintf(fd.z / tw.z) + 1;
          fd.w = __int_as_float(ix + 3 * iy + 9 * iz);
          // the block's runs of 8 particles the group's box can reach (bits
          // 16-19 of the depth word); the force's radius depends on each
          // partner's h, so it tests every run
          unsigned runs = 0xfu;
          if (!FORCE && a.sb_lo) {
            runs = 0u;
#pragma unroll
            for (int q = 0; q < 4; q++) {
              const float4 sl = a.sb_lo[4 * b + q], sh = a.sb_hi[4 * b + q];
              const float ex = fmaxf(fmaxf(sl.x + fd.x - gx1, gx0 - sh.x - fd.x), 0.f);
              const float ey = fmaxf(fmaxf(sl.y + fd.y - gy1, gy0 - sh.y - fd.y), 0.f);
              const float ez = fmaxf(fmaxf(sl.z + fd.z - gz1, gz0 - sh.z - fd.z), 0.f);
              if (ex * ex + ey * ey + ez * ez < R2 * (1.f + 4.f * band) + 1e-30f) runs |= 1u << q;
            }
          }
          dep |= (int)(runs << 16);
        }
      }
      const unsigned mask = __ballot_sync(FULL, ov);
      if (ov) {
        const int slot = __popc(mask & lt_mask);
        ws.sfirst[slot] = fc.x;
        ws.scount[slot] = fc.y;
        ws.se[slot] = e;
        ws.sdep[slot] = dep;
        ws.sf[slot] = fd;
        ws.slo[slot] = lo;
        ws.shi[slot] = hb;
      }
      __syncwarp();
      const int nsurv = __popc(mask);
      // positions of the next surviving block, loaded one block ahead: by
      // every lane into registers, or (bulk) by one bulk copy into the
      // warp's shared memory
      float4 qn = make_float4(0.f, 0.f, 0.f, 0.f);
      if (BULK) {
        if (nsurv > 0 && lane == 0) bulk_fetch(wb.raw, P.posh + ws.sfirst[0], ws.scount[0], &wb.bar);
      } else if (nsurv > 0 && lane < ws.scount[0]) {
        qn = P.posh[ws.sfirst[0] + lane];
      }
      for (int k = 0; k < nsurv; k++) {
        float4 q = qn;
        if (BULK) {
          // the copy of block k has landed: take this lane's record, then
          // start the copy of block k + 1 into the same buffer
          int ok = 1;
          if (lane == 0) ok = bulk_wait(&wb.bar, wb.parity, BULK_WAIT_TRIES);
          ok = __shfl_sync(FULL, ok, 0);
          if (!ok) {
            // give up on the launch: report, let the copy in flight finish
            // (bounded), leave
            if (lane == 0) {
              if (a.err) atomicExch(a.err, 1);
              bulk_wait(&wb.bar, wb.parity, BULK_WAIT_TRIES);
            }
            return;
          }
          if (lane == 0) wb.parity ^= 1u;
          if (lane < ws.scount[k]) q = wb.raw[lane];
          __syncwarp();
          if (k + 1 < nsurv && lane == 0)
            bulk_fetch(wb.raw, P.posh + ws.sfirst[k + 1], ws.scount[k + 1], &wb.bar);
        } else if (k + 1 < nsurv && lane < ws.scount[k + 1]) {
          qn = P.posh[ws.sfirst[k + 1] + lane];
        }
        const float4 sfd = ws.sf[k];
        const float4 slo = ws.slo[k], shi = ws.shi[k];
        const int eidx = ws.se[k];
        const Entry* E = &a.entries[eidx];
        const int sdep = ws.sdep[k];
        // does this lane's own sphere reach the block, and may it use the
        // entry (depth filter)?
        bool mine = false;
        if (valid && dh >= (sdep & 0xff) && dh <= ((sdep >> 8) & 0xff)) {
          const float px = pi.x - sfd.x, py = pi.y - sfd.y, pz = pi.z - sfd.z;
          const float dx = fmaxf(fmaxf(slo.x - px, px - shi.x), 0.f);
          const float dy = fmaxf(fmaxf(slo.y - py, py - shi.y), 0.f);
          const float dz = fmaxf(fmaxf(slo.z - pz, pz - shi.z), 0.f);
          const float R2 = FORCE ? fmaxf(hig2, slo.w) : cr2;
          mine = dx * dx + dy * dy + dz * dz < R2 * (1.f + 4.f * band) + 1e-30f;
        }
        if (!__any_sync(FULL, mine)) continue;
        const int bfirst = ws.sfirst[k], bcount = ws.scount[k];
        const int fidx = __float_as_int(sfd.w);
        __syncwarp();
        if (lane < bcount) {
          float* f = reinterpret_cast<float*>(ws.jp) + (lane >> 1) * 8 + (lane & 1);
          f[0] = -(q.x + sfd.x);
          f[2] = -(q.y + sfd.y);
          f[4] = -(q.z + sfd.z);
          f[6] = FORCE ? h2_exact(q.w) : 0.f;
        }
        __syncwarp();
        // the lane's own particle never pairs with itself
        const int tself = (i >= bfirst && i < bfirst + bcount) ? i - bfirst : -1;
        const int pk = bfirst | (fidx << 27);
        // Eight candidates per lane at a time, as four pairs: bit u is
        // candidate t0 + 2 TPP (u / 2) + 2 sub + u % 2, and a pair's distances
        // are evaluated with packed FP32 operations (the same IEEE roundings
        // as scalar ones).  FP32 r^2 below the band around H^2 sets a hit bit,
        // inside the band a band bit; hits are pushed from the mask, band
        // candidates are decided by the exact FP64 predicate in the reference
        // frame (rare: the warp votes once per chunk).
        auto cidx = [&](int t0, int u) { return t0 + 2 * TPP * (u >> 1) + 2 * sub + (u & 1); };
        const unsigned runs = (unsigned)sdep >> 16;
        for (int t0 = 0; t0 < bcount; t0 += 8 * TPP) {
          // candidates t0 .. t0 + 8 TPP - 1 are the block's runs t0 / 8 ..;
          // none of them within any lane's reach: nothing to test
          if (!((runs >> (t0 >> 3)) & ((1u << TPP) - 1u))) continue;
          unsigned hm = 0u, cm = 0u, wm = 0u;
#pragma unroll
          for (int v = 0; v < 4; v++) {
            const int pp = (t0 >> 1) + v * TPP + sub;
            const float4 qa = ws.jp[2 * pp], qb = ws.jp[2 * pp + 1];
            const float2 dx = __fadd2_rn(pix2, make_float2(qa.x, qa.y));
            const float2 dy = __fadd2_rn(piy2, make_float2(qa.z, qa.w));
            const float2 dz = __fadd2_rn(piz2, make_float2(qb.x, qb.y));
            float2 r2 = __fmul2_rn(dx, dx);
            r2 = __ffma2_rn(dy, dy, r2);
            r2 = __ffma2_rn(dz, dz, r2);
            float2 L2 = lo22, U2 = hi22;
            if (FORCE) {
              const float2 H2 = make_float2(fmaxf(hig2, qb.z), fmaxf(hig2, qb.w));
              L2 = __fmul2_rn(H2, omb2);
              U2 = __fmul2_rn(H2, opb2);
            }
            if (r2.x < L2.x) hm |= 1u << (2 * v);
            if (r2.y < L2.y) hm |= 2u << (2 * v);
            if (r2.x < U2.x) cm |= 1u << (2 * v);
            if (r2.y < U2.y) cm |= 2u << (2 * v);
            if (LISTS) {
              if (r2.x < lw2) wm |= 1u << (2 * v);
              if (r2.y < lw2) wm |= 2u << (2 * v);
            }
          }
          unsigned bm = cm & ~hm;
          // this lane's candidates in the block come first in bit order
          const int L = bcount - t0 - 2 * sub;
          const int nl = L <= 0 ? 0 : min(8, 2 * (L / (2 * TPP)) + min(L % (2 * TPP), 2));
          unsigned live = (1u << nl) - 1u;
          const int ds = tself - t0 - 2 * sub;
          if (tself >= 0 && ds >= 0 && ds % (2 * TPP) < 2 && ds / (2 * TPP) < 4)
            live &= ~(1u << (2 * (ds / (2 * TPP)) + ds % (2 * TPP)));
          if (!mine) live = 0u;
          hm &= live;
          bm &= live;
          if (LISTS) {
            // items go to the lane's row of the list 8 at a time (32 bytes)
            unsigned lm = wm & live;
            while (lm) {
              const int u = __ffs(lm) - 1;
              lm &= lm - 1u;
              ws.lb[lcnt & 7][lane] = pk + cidx(t0, u);
              lcnt++;
              if ((lcnt & 7) == 0 && lcnt <= a.nl_cap / TPP) {
                int4* row = reinterpret_cast<int4*>(a.nl + (size_t)i * a.nl_cap +
                                                    sub * (a.nl_cap / TPP) + (lcnt - 8));
                row[0] = make_int4(ws.lb[0][lane], ws.lb[1][lane], ws.lb[2][lane], ws.lb[3][lane]);
                row[1] = make_int4(ws.lb[4][lane], ws.lb[5][lane], ws.lb[6][lane], ws.lb[7][lane]);
              }
            }
          }
          while (hm) {
            const int u = __ffs(hm) - 1;
            hm &= hm - 1u;
            push(pk + cidx(t0, u));
          }
          if (__any_sync(FULL, bm != 0u)) {
            while (bm) {
              const int u = __ffs(bm) - 1;
              bm &= bm - 1u;
              const int t = cidx(t0, u);
              const float H2 =
                  FORCE ? fmaxf(hig2, reinterpret_cast<const float*>(ws.jp)[(t >> 1) * 8 + 6 + (t & 1)])
                        : hig2;
              if (exact_r2_2(P.xd, i, bfirst + t, E) < H2) push(pk + t);
            }
          }
          room();  // at most 8 pushes per lane since the last check
        }
      }
      __syncwarp();
    }
    drain(true);
    // the particle's lanes add their partial sums
#pragma unroll
    for (int o = 1; o < TPP; o <<= 1) {
      s0 += __shfl_xor_sync(FULL, s0, o);
      s1 += __shfl_xor_sync(FULL, s1, o);
      s2 += __shfl_xor_sync(FULL, s2, o);
      s3 += __shfl_xor_sync(FULL, s3, o);
      s4 += __shfl_xor_sync(FULL, s4, o);
      s5 = FORCE ? fmaxf(s5, __shfl_xor_sync(FULL, s5, o)) : s5 + __shfl_xor_sync(FULL, s5, o);
      s6 += __shfl_xor_sync(FULL, s6, o);
      s7 += __shfl_xor_sync(FULL, s7, o);
      ngb += __shfl_xor_sync(FULL, ngb, o);
      if (FORCE) nbin = min(nbin, __shfl_xor_sync(FULL, nbin, o));
    }
    // lists: each lane of a particle fills its own segment of the row
    // (nl_cap / TPP items); the count word holds both segments' counts
    const int segcap = LISTS ? a.nl_cap / TPP : 0;
    if (LISTS && valid && lcnt <= segcap)
      for (int k = lcnt & ~7; k < lcnt; k++)
        a.nl[(size_t)i * a.nl_cap + sub * segcap + k] = ws.lb[k & 7][lane];
    const int lc1 = TPP == 2 ? __shfl_xor_sync(FULL, lcnt, 1) : 0;
    if (!valid || sub != 0) continue;
    if (LISTS) {
      a.nl_cnt[i] = lcnt <= segcap && lc1 <= segcap ? (lcnt | lc1 << 16) : -1;
      a.nl_T[i] = lw2;
    }
    if (OUT == OUT_CALLER) {
      const size_t k = (size_t)co.perm[i];
      float* o = co.fields + 8 * k;
      o[0] = s0; o[1] = s1; o[2] = s2; o[3] = s3;
      o[4] = s4; o[5] = s5; o[6] = s6; o[7] = s7;
      co.ngb[k] = ngb;
      continue;
    }
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
        if (P.ngb_bin) P.ngb_bin[i] = (int8_t)min((int)P.ngb_bin[i], nbin);
      } else {
        // hydro_end_force (hydro.h:878) folded in
        P.acc[i] = make_float4(s0, s1, s2, s3);
        P.hdt_vsig[i] = make_float2(s4 * (hi * SPH_HDIM_INV), s5);
        P.ngb_f[i] = ngb;
        if (P.ngb_bin) P.ngb_bin[i] = (int8_t)nbin;
      }
    }
  }
}

// Work groups for the gathers: one slot per 32-particle window of every
// leaf, in leaf order (so consecutive groups are spatial neighbours and
// share cache lines), holding (window base, mask of the particles whose
// flags contain `need`, candidate-list begin, end).  Windows with an empty
// mask are skipped by the gathers.  With `compact` (sparse launches: the
// ghost's re-runs, steps with few active particles) only the windows with a
// non-empty mask are written, one after another (in no fixed order; each
// window's sums do not depend on it), and *compact counts them: the gather
// then takes no unit off its work queue for an empty window.
static __global__ void build_units(const LeafInfo* __restrict__ leaves, int nleaves,
                                   const int* __restrict__ leaf_window_begin,
                                   const uint8_t* __restrict__ flags, int need, int veto,
                                   const int* __restrict__ leaf_pair_begin,
                                   int4* __restrict__ units, const int* gate, int win = 32,
                                   int* compact = nullptr) {
  if (gate && *gate == 0) return;
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int l = warp; l < nleaves; l += nwarps) {
    const int first = leaves[l].first, count = leaves[l].count;
    const int p0 = leaf_pair_begin[l], p1 = leaf_pair_begin[l + 1];
    int slot = leaf_window_begin[l];
    for (int w0 = 0; w0 < count; w0 += win, slot++) {
      const bool in = lane < win && w0 + lane < count;
      const int f = in ? flags[first + w0 + lane] : 0;
      const bool ok = in && (f & need) == need && !(f & veto);
      const unsigned m = __ballot_sync(FULL, ok);
      if (compact) {
        if (lane == 0 && m != 0u && p0 != p1)
          units[atomicAdd(compact, 1)] = make_int4(first + w0, (int)m, p0, p1);
      } else if (lane == 0) {
        units[slot] = make_int4(first + w0, p0 == p1 ? 0 : (int)m, p0, p1);
      }
    }
  }
}

// The re-run list entry that pairs particle i (depth_h dh, in `leaf`) with
// j-block b, or null (runner_ghost.c:1548-1579 pairs each (i, j) once).
static __device__ const Entry* rerun_entry(const ListArgs& a, int leaf, int b, int dh) {
  for (int p = a.leaf_pair_begin[leaf]; p < a.leaf_pair_begin[leaf + 1]; p++) {
    if (a.pair_block[p] != b) continue;
    const Entry* E = &a.entries[a.pair_entry[p]];
    if (dh >= E->min_depth && dh <= E->max_depth) return E;
  }
  return nullptr;
}


// The ghost's rounds after the first: each particle iterates on its own
// (its density at h_k depends on nothing that changes during the ghost):
// the density from its list (the first pass recorded it; four lanes, three
// partners in flight each, misses evaluated beyond the kernel's support),
// then the Newton update of round k (ghost_update, the round kernel's own
// code), until it converges or round max_iter - 1 sends it on
// (non-convergence is counted in redo_count[max_iter - 1]).  A particle
// whose h_k is beyond its list stops there and is handed to the catch-up
// rounds (gathers; *a.handover counts them).  Same sums, same updates, in
// the same order as the rounds one at a time.
// ARENA: boxes of different sizes share the store (ListArgs::leaf_tw).
template <bool ARENA = false>
static __global__ void __launch_bounds__(256, 4)
    solve_from_lists(ListArgs a, GhostArgs g, int max_iter) {
  constexpr int LPP = 4;
  const DevParticles& P = a.p;
  __shared__ float4 ftab[27];
  if (threadIdx.x < 27) {
    const float3 o = offset_of(threadIdx.x, a.top_width);
    ftab[threadIdx.x] = make_float4(o.x, o.y, o.z, 0.f);
  }
  __syncthreads();
  const int sub = threadIdx.x % LPP;
  const int gl = (threadIdx.x & 31) & ~(LPP - 1);  // the group's first lane
  const int stride = gridDim.x * blockDim.x / LPP;
  for (int base = (blockIdx.x * blockDim.x + (threadIdx.x & ~31)) / LPP; base < P.n;
       base += stride) {
    const int i = base + (threadIdx.x & 31) / LPP;
    bool going = i < P.n && (P.flags[i] & 3) == 3;  // sent on by round 0
    int cnt = 0, c0 = 0;
    float T = 0.f;
    if (going) {
      cnt = a.nl_cnt[i];
      T = a.nl_T[i];
      if (cnt >= 0) {
        c0 = a.nl_seg == 2 ? (cnt & 0xffff) : cnt;
        cnt = c0 + (a.nl_seg == 2 ? cnt >> 16 : 0);
      }
    }
    const int* row = a.nl + (size_t)(i < P.n ? i : 0) * a.nl_cap;
    // boxes of different sizes in one store (the serving arena): the frame
    // offsets come from the particle's own top-cell width
    float3 twi = a.top_width;
    if (ARENA && i < P.n) {
      const float4 t = a.leaf_tw[P.leaf_of[i]];
      twi = make_float3(t.x, t.y, t.z);
    }
    for (int it = 1; it < max_iter && __any_sync(FULL, going); it++) {
      float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f, s4 = 0.f, s5 = 0.f, s6 = 0.f, s7 = 0.f;
      int ngb = 0;
      if (going) {
        const float4 pi = P.posh[i];
        const float4 vi = P.velm[i];
        const float hig2 = h2_exact(pi.w);
        const float L2 = hig2 * (1.f - a.band), U2 = hig2 * (1.f + a.band);
        const float hi_inv = 1.f / pi.w;
        if (!(cnt >= 0 && U2 <= T)) {
          // beyond the list: the catch-up rounds take it from here (it keeps
          // its iteration count in ghost_iters and its flags)
          going = false;
          if (sub == 0) atomicAdd(a.handover, 1);
        } else {
          for (int t0 = sub; t0 < cnt; t0 += 3 * LPP) {
            int pk[3];
            float4 q[3], vm[3];
#pragma unroll
            for (int u = 0; u < 3; u++) {
              const int t = t0 + u * LPP;
              pk[u] = t < cnt ? row[t < c0 ? t : t - c0 + a.nl_cap / 2] : i;
              if ((pk[u] & 0x07ffffff) >= P.n || ((unsigned)pk[u] >> 27) > 26) pk[u] = i;
            }
            // the partners' positions and velocities in flight together (a
            // row recorded at another h holds many items beyond this
            // particle's radius: a miss is evaluated beyond the kernel's
            // support, its terms exactly zero)
#pragma unroll
            for (int u = 0; u < 3; u++) {
              q[u] = P.posh[pk[u] & 0x07ffffff];
              vm[u] = P.velm[pk[u] & 0x07ffffff];
            }
            float dxs[3], dys[3], dzs[3], r2s[3];
#pragma unroll
            for (int u = 0; u < 3; u++) {
              float4 fd;
              if (ARENA) {
                const float3 o = offset_of((unsigned)pk[u] >> 27, twi);
                fd = make_float4(o.x, o.y, o.z, 0.f);
              } else {
                fd = ftab[(unsigned)pk[u] >> 27];
              }
              dxs[u] = pi.x - (q[u].x + fd.x);
              dys[u] = pi.y - (q[u].y + fd.y);
              dzs[u] = pi.z - (q[u].z + fd.z);
              r2s[u] = dxs[u] * dxs[u] + dys[u] * dys[u] + dzs[u] * dzs[u];
            }
#pragma unroll
            for (int u = 0; u < 3; u++) {
              const int j = pk[u] & 0x07ffffff;
              const float r2 = r2s[u];
              const bool item = t0 + u * LPP < cnt;
              bool hit = item && r2 < L2;
              if (item && !hit && r2 < U2) {
                const Entry* E = rerun_entry(a, P.leaf_of[i], a.blk_of[j], P.depth_h[i]);
                hit = E != nullptr && exact_r2_2(P.xd, i, j, E) < hig2;
              }
              density_hit(dxs[u], dys[u], dzs[u], hit ? r2 : 4.f * U2, vi, vm[u], hi_inv, s0, s1,
                          s2, s3, s4, s5, s6, s7);
              ngb += hit;
            }
          }
        }
      }
#pragma unroll
      for (int o = 1; o < LPP; o <<= 1) {
        s0 += __shfl_xor_sync(FULL, s0, o);
        s1 += __shfl_xor_sync(FULL, s1, o);
        s2 += __shfl_xor_sync(FULL, s2, o);
        s3 += __shfl_xor_sync(FULL, s3, o);
        s4 += __shfl_xor_sync(FULL, s4, o);
        s5 += __shfl_xor_sync(FULL, s5, o);
        s6 += __shfl_xor_sync(FULL, s6, o);
        s7 += __shfl_xor_sync(FULL, s7, o);
        ngb += __shfl_xor_sync(FULL, ngb, o);
      }
      int more = 0;
      if (going && sub == 0) {
        const float4 d0 = make_float4(s0, s1, s2, s3), d1 = make_float4(s4, s5, s6, s7);
        P.dens0[i] = d0;
        P.dens1[i] = d1;
        P.ngb_d[i] = ngb;
        if (a.hits) atomicAdd(a.hits, (unsigned long long)ngb);
        more = ghost_update(g, i, it, d0, d1);
      }
      more = __shfl_sync(FULL, more, gl);
      going = going && more;
      __syncwarp();  // the new h (posh.w) is read by the group's lanes next round
    }
  }
}


}  // namespace sphgpu
