// gather_tc.cuh -- the density gathers with a tensor-core candidate filter
// (included by gather.cu).
//
// Same work groups, culls, frames, rings and sums as gather_lanes<density>
// (gather_impl.cuh); what changes is how a surviving j-block's candidates
// are tested.  In the group's frame (origin at the centre c of the group's
// box) the squared distance is
//   r^2 = |x_i - c|^2 + |x_j - c|^2 - 2 (x_i - c).(x_j - c),
// a rank-5 product of per-particle rows [x', y', z', 1, |x'|^2] and
// per-candidate columns [-2x', -2y', -2z', |x'|^2, 1].  One warp-level
// mma.sync.m16n8k8 (TF32 inputs, FP32 accumulation) gives it for 16 group
// particles x 8 candidates at once, minus each particle's threshold
// (the accumulator's initial value), so the sign of each of the 128 results
// says "may be within the threshold".  A ballot per accumulator register
// turns the signs into masks; each lane takes its own particle's 8 bits.
//
// The filter only prunes: its threshold is the particle's widest bound
// (the re-run row's bound when rows are recorded, the band's top otherwise)
// plus a margin that covers the TF32 rounding of every term for the group's
// geometry, so no candidate that the FP32 test would keep is dropped.  Each
// lane then takes the candidates that passed for its particle one by one:
// the FP32 r^2 of gather_lanes' test (same operands, same roundings), the
// row item, the band and the exact FP64 predicate in the block's entry
// frame, and the hit pushed to the lane's ring.  Drains and sums are
// gather_lanes' own.  Counts and rows are identical; the sums differ only
// where a band hit shares an 8-candidate batch with a plain hit after it
// (gather_lanes queues band hits after the batch's plain ones).
#pragma once
#include "gather_impl.cuh"

namespace sphgpu {

__device__ __forceinline__ uint32_t f2tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// D = A B + C for one 16 x 8 tile, K = 8 (PTX mma.m16n8k8, .tf32).
// Fragments (g = lane / 4, t = lane % 4): a0 = A[g][t], a1 = A[g + 8][t],
// a2 = A[g][t + 4], a3 = A[g + 8][t + 4]; b0 = B[t][g], b1 = B[t + 4][g];
// c0 = C[g][2t], c1 = C[g][2t + 1], c2 = C[g + 8][2t], c3 = C[g + 8][2t + 1].
// Here C's rows are constant: c0 = c1 = ca, c2 = c3 = cb.
__device__ __forceinline__ void mma_tf32_16x8x8(float (&d)[4], const uint32_t (&a)[4],
                                                uint32_t b0, uint32_t b1, float ca,
                                                float cb) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 "
      "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%10, %10, %11, %11};\n"
      : "=f"(d[0]), "=f"(d[1]), "=f"(d[2]), "=f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1), "f"(ca), "f"(cb));
}

// Per-warp shared memory of the filtered gather.
#define TC_BSTRIDE 40  // candidate features: 4 rows of 32 (+8: no bank conflicts)
struct TcSmem {
  float bf[4][TC_BSTRIDE];  // staged block's columns, TF32 bit patterns:
                            // -2x', -2y', -2z', |x'|^2 of candidate j at [k][j]
  float4 jq[32];            // staged block: -(x, y, z) in the group's frame
  int sfirst[32];           // surviving blocks of the current chunk
  int scount[32];
  int se[32];
  int sdep[32];             // depth window min | max << 8, runs << 16
  float4 sf[32];            // frame offsets (w: frame-offset index)
  float4 slo[32];           // boxes
  float4 shi[32];
  int q[QCAP][32];          // per-lane ring of hits (partner | frame index << 27)
  int lb[8][32];            // row items staged 8 at a time (LISTS)
  float4 ftab[27];
};

template <int OUT = OUT_STORE, int WPB = WARPS_PER_BLOCK, int MINB = 3, bool LISTS = false,
          int TPP = 1>
__global__ void __launch_bounds__(WPB * 32, MINB)
gather_density_tc(G2Args a, CallerOut co = CallerOut{nullptr, nullptr, nullptr}) {
  static_assert(TPP == 1 || TPP == 2, "one or two lanes per particle");
  static_assert(TPP == 1 || OUT == OUT_STORE, "several lanes: stored sums");
  constexpr int NT = 2 / TPP;  // 16-particle tiles per warp
  __shared__ TcSmem smem[WPB];
  const int lane = threadIdx.x & 31;
  const int sub = lane % TPP, pl = lane / TPP;
  const int g8 = lane >> 2, t4 = lane & 3;  // fragment coordinates
  TcSmem& ws = smem[threadIdx.x >> 5];
  const DevParticles& P = a.p;
  if (a.gate && *a.gate == 0) return;
  const int nunits = a.count_ptr ? *a.count_ptr : a.count;
  const unsigned lt_mask = (1u << lane) - 1u;
  const float band = a.band;
  float3 tw = a.top_width;
  auto fill_ftab = [&]() {
    if (lane < 27) {
      const float3 o = offset_of(lane, tw);
      ws.ftab[lane] = make_float4(o.x, o.y, o.z, 0.f);
    }
    __syncwarp();
  };
  fill_ftab();
  // b1 = B[t + 4][g]: feature rows 4..7 of every column are [1, 0, 0, 0]
  const uint32_t b1 = t4 == 0 ? f2tf32(1.f) : 0u;
  // column g of a run's tile holds candidate g / 2 (g even) or g / 2 + 4
  const int ccol = (g8 & 1) ? (g8 >> 1) + 4 : (g8 >> 1);
  // this lane's particle: tile, row within the tile
  const int my_tile = pl >> 4, my_row = pl & 15;
  const int my_sh = 4 * (my_row & 7);
  const unsigned sub_keep = TPP == 1 ? 0xffu : (sub ? 0xaau : 0x55u);
  for (;;) {
    int u = 0;
    if (lane == 0) u = atomicAdd(a.queue, 1);
    u = __shfl_sync(FULL, u, 0);
    if (u >= nunits) break;
    const int4 U = a.units[u];  // base, mask, pair begin, pair end
    if (U.y == 0) continue;
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
    int dh = 0;
    if (valid) {
      pi = P.posh[i];
      vi = P.velm[i];
      dh = P.depth_h[i];
    }
    const float hi = valid ? pi.w : 1.f;
    const float hig2 = valid ? h2_exact(hi) : 0.f;
    const float hi_inv = 1.f / hi;
    const float lo2 = hig2 * (1.f - band), hi2 = hig2 * (1.f + band);
    float lw2 = hi2;
    if (LISTS && valid && a.nl_widen > 1.f) {
      const LeafInfo& L = a.leaves[P.leaf_of[i]];
      float cover = 0.f;
      for (int lev = 0; lev < L.nlevels; lev++)
        if (L.depth[lev] == dh) cover = SPH_KG * L.hmax[lev] * (1.f - 1.f / 1024.f);
      lw2 = fmaxf(hi2, fminf(hi2 * a.nl_widen, cover * cover));
    }
    // the widest r^2 bound this particle classifies against (the culls'
    // radius too)
    const float cr2 = LISTS ? lw2 : hi2;
    int lcnt = 0;
    float gx0 = valid ? pi.x : 3.4e38f, gy0 = valid ? pi.y : 3.4e38f,
          gz0 = valid ? pi.z : 3.4e38f;
    float gx1 = valid ? pi.x : -3.4e38f, gy1 = valid ? pi.y : -3.4e38f,
          gz1 = valid ? pi.z : -3.4e38f;
    float gh2 = valid ? cr2 : 0.f;
    int gd0 = valid ? dh : 1 << 20, gd1 = valid ? dh : -(1 << 20);
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
    // the group's frame and the filter's margin: with every particle within
    // rg of c and a kept candidate within sqrt(threshold) of its particle,
    // each of the product's terms is below (2 rg + sqrt(gh2))^2 + gh2 in
    // magnitude, and the TF32 roundings (2^-11 per input, so 2^-10 per
    // product) and the FP32 sums move the result by less than 2^-8 of that
    const float cx = 0.5f * (gx0 + gx1), cy = 0.5f * (gy0 + gy1), cz = 0.5f * (gz0 + gz1);
    const float ex = gx1 - gx0, ey = gy1 - gy0, ez = gz1 - gz0;
    const float rg = 0.5f * sqrtf(ex * ex + ey * ey + ez * ez);
    const float reach = 2.f * rg + sqrtf(gh2);
    const float margin = (reach * reach + gh2) * (1.f / 256.f);
    const float thr = valid ? cr2 + margin : -1.f;
    const float xq = valid ? pi.x - cx : 0.f, yq = valid ? pi.y - cy : 0.f,
                zq = valid ? pi.z - cz : 0.f;
    const float sq = xq * xq + yq * yq + zq * zq;
    // A = rows [x', y', z', 1, |x'|^2, 0, 0, 0] of the tile's 16 particles,
    // C = minus their thresholds
    uint32_t afr[NT][4];
    float cfa[NT], cfb[NT];
#pragma unroll
    for (int T = 0; T < NT; T++) {
      const int la = (16 * T + g8) * TPP, lb = (16 * T + g8 + 8) * TPP;
      const float xa = __shfl_sync(FULL, xq, la), ya = __shfl_sync(FULL, yq, la),
                  za = __shfl_sync(FULL, zq, la), sa = __shfl_sync(FULL, sq, la),
                  ta = __shfl_sync(FULL, thr, la);
      const float xb = __shfl_sync(FULL, xq, lb), yb = __shfl_sync(FULL, yq, lb),
                  zb = __shfl_sync(FULL, zq, lb), sb = __shfl_sync(FULL, sq, lb),
                  tb = __shfl_sync(FULL, thr, lb);
      const float fa = t4 == 0 ? xa : t4 == 1 ? ya : t4 == 2 ? za : 1.f;
      const float fb = t4 == 0 ? xb : t4 == 1 ? yb : t4 == 2 ? zb : 1.f;
      afr[T][0] = f2tf32(fa);
      afr[T][1] = f2tf32(fb);
      afr[T][2] = t4 == 0 ? f2tf32(sa) : 0u;
      afr[T][3] = t4 == 0 ? f2tf32(sb) : 0u;
      cfa[T] = -ta;
      cfb[T] = -tb;
    }
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f, s4 = 0.f, s5 = 0.f, s6 = 0.f, s7 = 0.f;
    int ngb = 0;
    int qh = 0, qt = 0;

    // a hit's sums (gather_lanes' interaction: the frame offset from the
    // table by index)
    auto interact = [&](int packed) {
      const int j = packed & 0x07ffffff;
      const float4 fd = ws.ftab[(unsigned)packed >> 27];
      const float4 q = P.posh[j];
      const float dx = pi.x - (q.x + fd.x), dy = pi.y - (q.y + fd.y),
                  dz = pi.z - (q.z + fd.z);
      const float r2 = dx * dx + dy * dy + dz * dz;
      const float4 vm = P.velm[j];
      density_hit(dx, dy, dz, r2, vi, vm, hi_inv, s0, s1, s2, s3, s4, s5, s6, s7);
      ngb++;
    };
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
    auto room = [&]() {
      if (__any_sync(FULL, qt - qh > QCAP - 8)) drain(false);
    };

    for (int c0 = U.z; c0 < U.w; c0 += 32) {
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
        ov = dx * dx + dy * dy + dz * dz < gh2 * (1.f + 4.f * band) + 1e-30f &&
             gd1 >= E->min_depth && gd0 <= E->max_depth;
        if (ov) {
          fc = a.bb_fc[b];
          const int ix = (int)rintf(fd.x / tw.x) + 1, iy = (int)rintf(fd.y / tw.y) + 1,
                    iz = (int)rintf(fd.z / tw.z) + 1;
          fd.w = __int_as_float(ix + 3 * iy + 9 * iz);
          unsigned runs = 0xfu;
          if (a.sb_lo) {
            runs = 0u;
#pragma unroll
            for (int q = 0; q < 4; q++) {
              const float4 sl = a.sb_lo[4 * b + q], sh = a.sb_hi[4 * b + q];
              const float rx = fmaxf(fmaxf(sl.x + fd.x - gx1, gx0 - sh.x - fd.x), 0.f);
              const float ry = fmaxf(fmaxf(sl.y + fd.y - gy1, gy0 - sh.y - fd.y), 0.f);
              const float rz = fmaxf(fmaxf(sl.z + fd.z - gz1, gz0 - sh.z - fd.z), 0.f);
              if (rx * rx + ry * ry + rz * rz < gh2 * (1.f + 4.f * band) + 1e-30f)
                runs |= 1u << q;
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
      float4 qn = make_float4(0.f, 0.f, 0.f, 0.f);
      if (nsurv > 0 && lane < ws.scount[0]) qn = P.posh[ws.sfirst[0] + lane];
      for (int k = 0; k < nsurv; k++) {
        const float4 q = qn;
        if (k + 1 < nsurv && lane < ws.scount[k + 1]) qn = P.posh[ws.sfirst[k + 1] + lane];
        const float4 sfd = ws.sf[k];
        const float4 slo = ws.slo[k], shi = ws.shi[k];
        const int sdep = ws.sdep[k];
        bool mine = false;
        if (valid && dh >= (sdep & 0xff) && dh <= ((sdep >> 8) & 0xff)) {
          const float px = pi.x - sfd.x, py = pi.y - sfd.y, pz = pi.z - sfd.z;
          const float dx = fmaxf(fmaxf(slo.x - px, px - shi.x), 0.f);
          const float dy = fmaxf(fmaxf(slo.y - py, py - shi.y), 0.f);
          const float dz = fmaxf(fmaxf(slo.z - pz, pz - shi.z), 0.f);
          mine = dx * dx + dy * dy + dz * dz < cr2 * (1.f + 4.f * band) + 1e-30f;
        }
        if (!__any_sync(FULL, mine)) continue;
        const int bfirst = ws.sfirst[k], bcount = ws.scount[k];
        const int pk = bfirst | (__float_as_int(sfd.w) << 27);
        __syncwarp();
        {
          // the block's columns in the group's frame; past the block's end a
          // column that passes no threshold
          float bx = 0.f, by = 0.f, bz = 0.f, bs = 3.0e30f;
          if (lane < bcount) {
            const float qx = __fadd_rn(q.x, sfd.x), qy = __fadd_rn(q.y, sfd.y),
                        qz = __fadd_rn(q.z, sfd.z);
            ws.jq[lane] = make_float4(-qx, -qy, -qz, 0.f);
            const float xj = qx - cx, yj = qy - cy, zj = qz - cz;
            bx = -2.f * xj;
            by = -2.f * yj;
            bz = -2.f * zj;
            bs = xj * xj + yj * yj + zj * zj;
          }
          ws.bf[0][lane] = __uint_as_float(f2tf32(bx));
          ws.bf[1][lane] = __uint_as_float(f2tf32(by));
          ws.bf[2][lane] = __uint_as_float(f2tf32(bz));
          ws.bf[3][lane] = __uint_as_float(f2tf32(bs));
        }
        __syncwarp();
        // candidates this lane may take: its own sphere reaches the block and
        // its depth may use the entry, never itself
        unsigned live = mine ? 0xffffffffu : 0u;
        if (bcount < 32) live &= (1u << bcount) - 1u;
        if (i >= bfirst && i < bfirst + bcount) live &= ~(1u << (i - bfirst));
        const unsigned runs = (unsigned)sdep >> 16;
        for (int r = 0; 8 * r < bcount; r++) {
          if (!((runs >> r) & 1u)) continue;  // no lane of the group reaches the run
          const uint32_t b0 = __float_as_uint(ws.bf[t4][8 * r + ccol]);
          unsigned m8 = 0u;
#pragma unroll
          for (int T = 0; T < NT; T++) {
            float d[4];
            mma_tf32_16x8x8(d, afr[T], b0, b1, cfa[T], cfb[T]);
            const unsigned B0 = __ballot_sync(FULL, d[0] < 0.f);
            const unsigned B1 = __ballot_sync(FULL, d[1] < 0.f);
            const unsigned B2 = __ballot_sync(FULL, d[2] < 0.f);
            const unsigned B3 = __ballot_sync(FULL, d[3] < 0.f);
            if (my_tile == T) {
              const unsigned ev = ((my_row < 8 ? B0 : B2) >> my_sh) & 0xfu;
              const unsigned od = ((my_row < 8 ? B1 : B3) >> my_sh) & 0xfu;
              m8 = ev | (od << 4);
            }
          }
          m8 &= (live >> (8 * r)) & sub_keep;
          while (m8) {
            const int t = 8 * r + __ffs(m8) - 1;
            m8 &= m8 - 1u;
            // gather_lanes' FP32 test of candidate t: pi + (-(q + fd)), then
            // one multiply and two fused multiply-adds
            const float4 nq = ws.jq[t];
            const float ddx = __fadd_rn(pi.x, nq.x), ddy = __fadd_rn(pi.y, nq.y),
                        ddz = __fadd_rn(pi.z, nq.z);
            const float r2 = __fmaf_rn(ddz, ddz, __fmaf_rn(ddy, ddy, __fmul_rn(ddx, ddx)));
            if (LISTS && r2 < lw2) {
              ws.lb[lcnt & 7][lane] = pk + t;
              lcnt++;
              if ((lcnt & 7) == 0 && lcnt <= a.nl_cap / TPP) {
                int4* row = reinterpret_cast<int4*>(a.nl + (size_t)i * a.nl_cap +
                                                    sub * (a.nl_cap / TPP) + (lcnt - 8));
                row[0] = make_int4(ws.lb[0][lane], ws.lb[1][lane], ws.lb[2][lane], ws.lb[3][lane]);
                row[1] = make_int4(ws.lb[4][lane], ws.lb[5][lane], ws.lb[6][lane], ws.lb[7][lane]);
              }
            }
            if (r2 < lo2) {
              push(pk + t);
            } else if (r2 < hi2) {
              // inside the band: the exact predicate in the entry's frame
              if (exact_r2_2(P.xd, i, bfirst + t, &a.entries[ws.se[k]]) < hig2) push(pk + t);
            }
          }
          room();  // at most 8 pushes per lane since the last check
        }
      }
      __syncwarp();
    }
    drain(true);
#pragma unroll
    for (int o = 1; o < TPP; o <<= 1) {
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
      const size_t kk = (size_t)co.perm[i];
      float* o = co.fields + 8 * kk;
      o[0] = s0; o[1] = s1; o[2] = s2; o[3] = s3;
      o[4] = s4; o[5] = s5; o[6] = s6; o[7] = s7;
      co.ngb[kk] = ngb;
      continue;
    }
    if (a.hits) atomicAdd(a.hits, (unsigned long long)ngb);
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
  }
}

}  // namespace sphgpu
