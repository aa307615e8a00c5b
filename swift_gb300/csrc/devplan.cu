// devplan.cu -- the gather lists of a step planned on the device (see
// devplan.cuh).  The recursions follow space.cpp's host planner step for
// step, restricted to the branches that contain one leaf:
//   DOSUB_SELF1/2, DOSUB_PAIR1/2 (runner_doiact_functions_hydro.h:2933-3100;
//     cell.h:934-1010 for the recursion predicates, dx_max terms zero),
//   DOSUB_SUBSET (runner_doiact_functions_hydro.h:3290-3400) for the ghost's
//     re-runs of one leaf (runner_ghost.c:1548-1579),
//   space_getsid_and_swap_cells (space_getsid.h:47-80) for the pair frames.
#include <algorithm>

#include "devplan.cuh"
#include "device_sms.h"

namespace sphgpu {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kRecurse = 100;  // space.h:64-65 (Space::kRecurseSize)

// Direction of each of the 13 sort axes (sort_part.h:42-57), the same table
// the host planner's child_pairs() uses.
__constant__ int8_t c_dir[13][3] = {{1, 1, 1},  {1, 1, 0},  {1, 1, -1}, {1, 0, 1},
                                    {1, 0, 0},  {1, 0, -1}, {1, -1, 1}, {1, -1, 0},
                                    {1, -1, -1}, {0, 1, 1}, {0, 1, 0},  {0, 1, -1},
                                    {0, 0, 1}};

// Child p of ci and child q of cj touch across axis sid.
__device__ __forceinline__ bool touch(int sid, int p, int q) {
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const int pb = (p >> (2 - k)) & 1, qb = (q >> (2 - k)) & 1;
    const int d = 2 * c_dir[sid][k] + qb - pb;
    if (d > 1 || d < -1) return false;
  }
  return true;
}

__device__ int getsid_swap(const DPTree& t, int& ci, int& cj, double shift[3]) {
  double dx[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    dx[k] = t.cell[cj].loc[k] - t.cell[ci].loc[k];
    if (t.periodic && dx[k] < -t.dim[k] / 2)
      shift[k] = t.dim[k];
    else if (t.periodic && dx[k] > t.dim[k] / 2)
      shift[k] = -t.dim[k];
    else
      shift[k] = 0.0;
    dx[k] += shift[k];
  }
  int idx = 0;
#pragma unroll
  for (int k = 0; k < 3; k++) idx = 3 * idx + ((dx[k] < 0.0) ? 0 : ((dx[k] > 0.0) ? 2 : 1));
  if (idx < 13) {
    const int tmp = ci;
    ci = cj;
    cj = tmp;
#pragma unroll
    for (int k = 0; k < 3; k++) shift[k] = -shift[k];
    return idx;
  }
  return 26 - idx;
}

// One entry of leaf L (space.cpp make_entry).
__device__ void make_entry(const DPTree& t, int L, int partner, int kind, bool u_is_ci,
                           const double shift[3], int frame_cell, int min_depth,
                           int max_depth, Entry& e) {
  const DPCell& pc = t.cell[partner];
  e.first = pc.first;
  e.count = pc.count;
  e.bfirst = pc.jb_begin;
  e.bcount = pc.jb_end - pc.jb_begin;
  e.kind = (int8_t)kind;
  e.min_depth = (int8_t)min_depth;
  e.max_depth = (int8_t)max_depth;
  e.pad0 = 0;
  double seff[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int k = 0; k < 3; k++) e.ou[k] = e.op[k] = 0.0;
  if (kind == FRAME_PAIR_CELLREL) {
    const DPCell& fc = t.cell[frame_cell];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const double oi = fc.loc[k] + shift[k];
      const double oj = fc.loc[k];
      e.ou[k] = u_is_ci ? oi : oj;
      e.op[k] = u_is_ci ? oj : oi;
      seff[k] = u_is_ci ? shift[k] : -shift[k];
    }
  } else if (kind == FRAME_PAIR_ABS) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      e.ou[k] = shift[k];
      seff[k] = shift[k];
    }
  } else if (kind == FRAME_SELF_CELLREL) {
    const DPCell& fc = t.cell[frame_cell];
#pragma unroll
    for (int k = 0; k < 3; k++) e.ou[k] = e.op[k] = fc.loc[k];
  }
  const DPCell& tl = t.cell[t.cell[L].top];
  const DPCell& tp = t.cell[pc.top];
  e.fdx = (float)(tp.loc[0] + seff[0] - tl.loc[0]);
  e.fdy = (float)(tp.loc[1] + seff[1] - tl.loc[1]);
  e.fdz = (float)(tp.loc[2] + seff[2] - tl.loc[2]);
}

struct CountSink {
  const DPTree* t;
  int ne = 0, np = 0;
  __device__ void operator()(int, int partner, int, bool, const double*, int, int, int) {
    ne++;
    np += t->cell[partner].jb_end - t->cell[partner].jb_begin;
  }
};

struct EmitSink {
  const DPTree* t;
  Entry* entries;
  int32_t* pb;
  int32_t* pe;
  int e, p;
  __device__ void operator()(int L, int partner, int kind, bool u_is_ci, const double* shift,
                             int frame, int mind, int maxd) {
    Entry en;
    make_entry(*t, L, partner, kind, u_is_ci, shift, frame, mind, maxd, en);
    entries[e] = en;
    for (int b = en.bfirst; b < en.bfirst + en.bcount; b++, p++) {
      pb[p] = b;
      pe[p] = e;
    }
    e++;
  }
};

struct LeafCtx {
  const DPTree* t;
  const DPCellState* cs;
  int L, Lfirst;
  __device__ bool under(int c) const {
    const int f = t->cell[c].first, n = t->cell[c].count;
    return n > 0 && Lfirst >= f && Lfirst < f + n;
  }
  __device__ bool active(int c) const { return cs->active[c] != 0; }
  __device__ int count(int c) const { return t->cell[c].count; }
  // kernel_gamma h + dx_max_part < dmin / 2, each operation rounded on its
  // own (the host planner's Space::reach)
  __device__ bool reach_ok(int c, float h) const {
    const float dx = cs->dx ? __uint_as_float(cs->dx[c]) : 0.f;
    return __fadd_rn(__fmul_rn(SPH_KG, h), dx) < 0.5f * t->cell[c].dmin;
  }
};

// DOSUB_SELF / DOSUB_PAIR of one task, restricted to leaf L.  SECOND selects
// the force loop's predicates (h_max after the ghost) over the density
// loop's (h_max_active).  Returns 0, or 2 when the recursion is deeper than
// the frame stack.
template <bool SECOND, class Sink>
__device__ int dosub_leaf(const LeafCtx& x, int ci, int cj, Sink& sink) {
  const DPTree& t = *x.t;
  struct F {
    int a, b, below, it, sid;
  };
  F st[kDPStack];
  int sp = 0;
  const double zero[3] = {0.0, 0.0, 0.0};
  auto h_of = [&](int c) {
    return __uint_as_float(SECOND ? x.cs->hforce[c] : x.cs->hact[c]);
  };
  auto self_branch = [&](int c, int lmin, int lmax) {
    if (x.count(c) == 0 || !x.active(c)) return;
    const int d = t.cell[c].depth;
    sink(x.L, c, FRAME_SELF_DBL, true, zero, c, lmax ? d : 0, lmin ? d : 127);
  };
  auto pair_branch = [&](int A, int B, int lmin, int lmax) {
    if (x.count(A) == 0 || x.count(B) == 0) return;
    if (!x.active(A) && !x.active(B)) return;
    double sh[3];
    int a = A, b = B;
    getsid_swap(t, a, b, sh);
    const int d = t.cell[a].depth;
    const int mind = lmax ? d : 0, maxd = lmin ? d : 127;
    if (x.under(a)) sink(x.L, b, FRAME_PAIR_CELLREL, true, sh, b, mind, maxd);
    if (x.under(b)) sink(x.L, a, FRAME_PAIR_CELLREL, false, sh, b, mind, maxd);
  };
  st[sp++] = F{ci, cj, 0, -1, 0};
  while (sp > 0) {
    F& f = st[sp - 1];
    int na = -1, nb = -1;
    bool push = false;
    if (f.b < 0) {
      const int c = f.a;
      if (f.it < 0) {
        const int cnt = x.count(c);
        if (cnt == 0 || !x.active(c)) {
          sp--;
          continue;
        }
        if (!t.cell[c].split || cnt < kRecurse) {
          self_branch(c, 0, f.below);
          sp--;
          continue;
        }
        if (!f.below) {
          const float hm = h_of(c);
          const bool ok = SECOND ? (t.cell[c].split && SPH_KG * hm < 0.5f * t.cell[c].dmin)
                                 : (SPH_KG * hm < 0.5f * t.cell[c].dmin);
          if (!ok) f.below = 1;
        }
        if (f.below) self_branch(c, 1, 1);
        f.it = 0;
      }
      // slots (k, j), j >= k: progeny k's self recursion (j == k), then its
      // pairs with the later progeny j
      while (f.it < 64) {
        const int k = f.it >> 3, j = f.it & 7;
        f.it = (j + 1 < 8) ? f.it + 1 : ((k + 1 < 8) ? (k + 1) * 9 : 64);
        const int p = t.progeny[8 * c + k];
        if (p < 0) continue;
        if (j == k) {
          if (x.under(p)) {
            na = p;
            push = true;
            break;
          }
        } else {
          const int q = t.progeny[8 * c + j];
          if (q >= 0 && (x.under(p) || x.under(q))) {
            na = p;
            nb = q;
            push = true;
            break;
          }
        }
      }
    } else {
      if (f.it < 0) {
        int A = f.a, B = f.b;
        if (!x.active(A) && !x.active(B)) {
          sp--;
          continue;
        }
        if (x.count(A) == 0 || x.count(B) == 0) {
          sp--;
          continue;
        }
        double sh[3];
        f.sid = getsid_swap(t, A, B, sh);
        f.a = A;
        f.b = B;
        if (!t.cell[A].split || x.count(A) < kRecurse || !t.cell[B].split ||
            x.count(B) < kRecurse) {
          pair_branch(A, B, 0, f.below);
          sp--;
          continue;
        }
        if (!f.below) {
          const bool ok = x.reach_ok(A, h_of(A)) && x.reach_ok(B, h_of(B));
          if (!ok) f.below = 1;
        }
        if (f.below) pair_branch(A, B, 1, 1);
        f.it = 0;
      }
      while (f.it < 64) {
        const int idx = f.it++;
        const int p = idx >> 3, q = idx & 7;
        if (!touch(f.sid, p, q)) continue;
        const int P = t.progeny[8 * f.a + p], Q = t.progeny[8 * f.b + q];
        if (P >= 0 && Q >= 0 && (x.under(P) || x.under(Q))) {
          na = P;
          nb = Q;
          push = true;
          break;
        }
      }
    }
    if (!push) {
      sp--;
      continue;
    }
    if (sp == kDPStack) return 2;
    const int below = f.below;
    st[sp++] = F{na, nb, below, -1, 0};
  }
  return 0;
}

// The child of c that holds leaf L, or -1.
__device__ int find_sub(const LeafCtx& x, int c) {
  for (int k = 0; k < 8; k++) {
    const int p = x.t->progeny[8 * c + k];
    if (p >= 0 && x.under(p)) return p;
  }
  return -1;
}

// The subset recursion of the ghost's re-runs for leaf L through one task
// of its top cell (other < 0: the self task).  Returns 0, 2 (stack) or 8
// (a split cell without the child that holds L: an inconsistent tree).
template <class Sink>
__device__ int subset_leaf(const LeafCtx& x, int top, int other, Sink& sink) {
  const DPTree& t = *x.t;
  struct F {
    int ci, cj, it, a, b, sid, sub;
  };
  F st[kDPStack];
  int sp = 0;
  const double zero[3] = {0.0, 0.0, 0.0};
  auto can_old = [&](int c) {
    return t.cell[c].split && x.reach_ok(c, __uint_as_float(x.cs->hmax[c]));
  };
  st[sp++] = F{top, other, -1, 0, 0, 0, -1};
  while (sp > 0) {
    F& f = st[sp - 1];
    int nci = -1, ncj = -1;
    bool push = false;
    if (f.cj < 0) {
      if (f.it < 0) {
        const int c = f.ci;
        if (x.count(c) == 0 || !x.active(c)) {
          sp--;
          continue;
        }
        if (t.cell[c].split &&
            SPH_KG * __uint_as_float(x.cs->hmax[c]) < 0.5f * t.cell[c].dmin) {
          f.sub = find_sub(x, c);
          if (f.sub < 0) return 8;
          f.it = 0;
        } else {
          sink(x.L, c, FRAME_SELF_CELLREL, true, zero, c, 0, 127);
          sp--;
          continue;
        }
      }
      while (f.it < 9) {
        const int s = f.it++;
        if (s == 0) {
          nci = f.sub;
          push = true;
          break;
        }
        const int q = t.progeny[8 * f.ci + s - 1];
        if (q != f.sub && q >= 0) {
          nci = f.sub;
          ncj = q;
          push = true;
          break;
        }
      }
    } else {
      if (f.it < 0) {
        const int ci = f.ci, cj = f.cj;
        if (x.count(ci) == 0 || x.count(cj) == 0 || !x.active(ci)) {
          sp--;
          continue;
        }
        if (can_old(ci) && can_old(cj)) {
          f.sub = find_sub(x, ci);
          if (f.sub < 0) return 8;
          int a = ci, b = cj;
          double sh[3];
          f.sid = getsid_swap(t, a, b, sh);
          f.a = a;
          f.b = b;
          f.it = 0;
        } else {
          double sh[3];
#pragma unroll
          for (int k = 0; k < 3; k++) {
            const double d = t.cell[cj].loc[k] - t.cell[ci].loc[k];
            sh[k] = d < -t.dim[k] / 2 ? t.dim[k] : (d > t.dim[k] / 2 ? -t.dim[k] : 0.0);
          }
          sink(x.L, cj, FRAME_PAIR_ABS, true, sh, cj, 0, 127);
          sp--;
          continue;
        }
      }
      while (f.it < 64) {
        const int idx = f.it++;
        const int p = idx >> 3, q = idx & 7;
        if (!touch(f.sid, p, q)) continue;
        const int P = t.progeny[8 * f.a + p], Q = t.progeny[8 * f.b + q];
        if (P == f.sub && Q >= 0) {
          nci = P;
          ncj = Q;
          push = true;
          break;
        }
        if (P >= 0 && Q == f.sub) {
          nci = Q;
          ncj = P;
          push = true;
          break;
        }
      }
    }
    if (!push) {
      sp--;
      continue;
    }
    if (sp == kDPStack) return 2;
    st[sp++] = F{nci, ncj, -1, 0, 0, 0, -1};
  }
  return 0;
}

template <int KIND, class Sink>
__device__ int run_task(const LeafCtx& x, int top, int2 tk, Sink& sink) {
  if (KIND == DP_SUBSET) return subset_leaf(x, top, tk.y < 0 ? -1 : (tk.x == top ? tk.y : tk.x), sink);
  return dosub_leaf<KIND == DP_FORCE>(x, tk.x, tk.y, sink);
}

template <int KIND>
__global__ void __launch_bounds__(256) dp_count_k(DPTree t, DPCellState cs, DPOut o) {
  const int lane = threadIdx.x & 31;
  const int warp = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int nwarps = (int)((gridDim.x * (size_t)blockDim.x) >> 5);
  if (warp == 0 && lane == 0) o.leaf_off[t.nleaves] = make_int2(0, 0);
  for (int l = warp; l < t.nleaves; l += nwarps) {
    const int L = t.leaf_cell[l];
    int ne = 0, np = 0, err = 0;
    if (cs.active[L]) {
      const int top = t.cell[L].top;
      const int lb = t.link_begin[top], nlk = t.link_begin[top + 1] - lb;
      if (nlk > 32) {
        err = 4;
      } else if (lane < nlk) {
        const LeafCtx x{&t, &cs, L, t.cell[L].first};
        CountSink sink{&t};
        err = run_task<KIND>(x, top, t.task[t.link[lb + lane]], sink);
        ne = sink.ne;
        np = sink.np;
      }
    }
    int ie = ne, ip = np;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int ue = __shfl_up_sync(kFull, ie, d), up = __shfl_up_sync(kFull, ip, d);
      if (lane >= d) {
        ie += ue;
        ip += up;
      }
    }
    o.lane_off[32 * (size_t)l + lane] = make_int2(ie - ne, ip - np);
    if (lane == 31) o.leaf_off[l] = make_int2(ie, ip);
    err = (int)__reduce_or_sync(kFull, (unsigned)err);
    if (err && lane == 0) atomicOr(o.status, err);
  }
}

template <int KIND>
__global__ void __launch_bounds__(256) dp_emit_k(DPTree t, DPCellState cs, DPOut o) {
  const int lane = threadIdx.x & 31;
  const int warp = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int nwarps = (int)((gridDim.x * (size_t)blockDim.x) >> 5);
  const int2 tot = o.leaf_off[t.nleaves];
  const bool over = tot.x < 0 || tot.y < 0 || tot.x > o.cap_e || tot.y > o.cap_p;
  if (warp == 0 && lane == 0) {
    o.status[1 + 2 * KIND] = tot.x;
    o.status[2 + 2 * KIND] = tot.y;
    if (over) atomicOr(o.status, 1);
    o.lpb[t.nleaves] = over ? 0 : tot.y;
  }
  for (int l = warp; l < t.nleaves; l += nwarps) {
    const int2 base = o.leaf_off[l];
    if (lane == 0) o.lpb[l] = over ? 0 : base.y;
    const int L = t.leaf_cell[l];
    if (over || !cs.active[L]) continue;
    const int top = t.cell[L].top;
    const int lb = t.link_begin[top], nlk = t.link_begin[top + 1] - lb;
    if (nlk > 32 || lane >= nlk) continue;
    const int2 lo = o.lane_off[32 * (size_t)l + lane];
    const LeafCtx x{&t, &cs, L, t.cell[L].first};
    EmitSink sink{&t, o.entries, o.pb, o.pe, base.x + lo.x, base.y + lo.y};
    run_task<KIND>(x, top, t.task[t.link[lb + lane]], sink);
  }
}

// ---------------------------------------------------------------------------
// Exclusive scan of (entries, pairs) over the leaves: tile sums, one block
// over the tile sums, tiles again with their offsets.

constexpr int kScanTile = 1024;  // 256 threads x 4 items

__device__ __forceinline__ int2 add2(int2 a, int2 b) { return make_int2(a.x + b.x, a.y + b.y); }

// Exclusive scan of v over the block (blockDim.x a multiple of 32, at most
// 1024); *total gets the block's sum.
__device__ int2 block_exclusive(int2 v, int2* total) {
  __shared__ int2 wsum[32];
  __shared__ int2 wtot;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int2 inc = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int ux = __shfl_up_sync(kFull, inc.x, d), uy = __shfl_up_sync(kFull, inc.y, d);
    if (lane >= d) inc = add2(inc, make_int2(ux, uy));
  }
  if (lane == 31) wsum[w] = inc;
  __syncthreads();
  if (w == 0) {
    int2 s = lane < nw ? wsum[lane] : make_int2(0, 0);
    int2 si = s;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int ux = __shfl_up_sync(kFull, si.x, d), uy = __shfl_up_sync(kFull, si.y, d);
      if (lane >= d) si = add2(si, make_int2(ux, uy));
    }
    if (lane < nw) wsum[lane] = make_int2(si.x - s.x, si.y - s.y);
    if (lane == nw - 1) wtot = si;
  }
  __syncthreads();
  const int2 off = wsum[w];
  const int2 tot = wtot;
  __syncthreads();
  if (total) *total = tot;
  return make_int2(off.x + inc.x - v.x, off.y + inc.y - v.y);
}

__global__ void __launch_bounds__(256) scan_tile_sums(const int2* __restrict__ a, long long n,
                                                      int2* __restrict__ tiles) {
  const long long base = (long long)blockIdx.x * kScanTile + 4 * threadIdx.x;
  int2 s = make_int2(0, 0);
#pragma unroll
  for (int k = 0; k < 4; k++)
    if (base + k < n) s = add2(s, a[base + k]);
  int2 tot;
  block_exclusive(s, &tot);
  if (threadIdx.x == 0) tiles[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(1024) scan_tile_prefix(int2* tiles, int ntiles) {
  const int per = (ntiles + blockDim.x - 1) / blockDim.x;
  const int b = threadIdx.x * per;
  int2 s = make_int2(0, 0);
  for (int k = 0; k < per; k++)
    if (b + k < ntiles) s = add2(s, tiles[b + k]);
  int2 run = block_exclusive(s, nullptr);
  for (int k = 0; k < per; k++)
    if (b + k < ntiles) {
      const int2 v = tiles[b + k];
      tiles[b + k] = run;
      run = add2(run, v);
    }
}

__global__ void __launch_bounds__(256) scan_apply(int2* __restrict__ a, long long n,
                                                  const int2* __restrict__ tiles) {
  const long long base = (long long)blockIdx.x * kScanTile + 4 * threadIdx.x;
  int2 v[4];
  int2 s = make_int2(0, 0);
#pragma unroll
  for (int k = 0; k < 4; k++) {
    v[k] = base + k < n ? a[base + k] : make_int2(0, 0);
    s = add2(s, v[k]);
  }
  int2 run = add2(block_exclusive(s, nullptr), tiles[blockIdx.x]);
#pragma unroll
  for (int k = 0; k < 4; k++)
    if (base + k < n) {
      a[base + k] = run;
      run = add2(run, v[k]);
    }
}

// ---------------------------------------------------------------------------

__global__ void dp_flags_k(uint8_t* __restrict__ flags, const int8_t* __restrict__ tbin, int n,
                           const int* __restrict__ max_bin) {
  const int b = *max_bin;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    flags[i] = (int)tbin[i] <= b ? 1 : 0;
}

__global__ void dp_cells_reset(DPCellState cs, int ncells, int force) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += gridDim.x * blockDim.x) {
    if (force) {
      cs.hforce[c] = 0u;
    } else {
      cs.hmax[c] = 0u;
      cs.hact[c] = 0u;
      cs.active[c] = 0;
    }
  }
}

// One warp per leaf: the leaf's values from its particles, then an atomic
// maximum into every ancestor.
__global__ void __launch_bounds__(256) dp_cells_leaf(DPTree t, DPCellState cs,
                                                     const float4* __restrict__ posh,
                                                     const float* __restrict__ h0,
                                                     const uint8_t* __restrict__ flags,
                                                     int force) {
  const int lane = threadIdx.x & 31;
  const int warp = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int nwarps = (int)((gridDim.x * (size_t)blockDim.x) >> 5);
  for (int l = warp; l < t.nleaves; l += nwarps) {
    const int L = t.leaf_cell[l];
    const int first = t.cell[L].first, count = t.cell[L].count;
    unsigned m = 0u, ma = 0u, any = 0u;
    for (int i = first + lane; i < first + count; i += 32) {
      const float h = posh[i].w;
      const bool a = flags[i] & 1;
      if (force) {
        m = max(m, __float_as_uint(a ? fmaxf(h0[i], h) : h));
      } else {
        m = max(m, __float_as_uint(h));
        if (a) {
          ma = max(ma, __float_as_uint(h));
          any = 1u;
        }
      }
    }
    m = __reduce_max_sync(kFull, m);
    ma = __reduce_max_sync(kFull, ma);
    any = __reduce_or_sync(kFull, any);
    if (lane == 0) {
      for (int c = L; c >= 0; c = t.cell[c].parent) {
        if (force) {
          atomicMax(&cs.hforce[c], m);
        } else {
          atomicMax(&cs.hmax[c], m);
          atomicMax(&cs.hact[c], ma);
          if (any) atomicOr(&cs.active[c], 1);
        }
      }
    }
  }
}

int leaf_blocks(int nleaves) {
  // 8 warps (leaves) per block, at most 16 blocks per SM resident at once
  return std::max(1, std::min((nleaves + 7) / 8, 16 * sm_count()));
}

int grid_for(long long n) {
  return (int)std::max(1LL, std::min((n + 255) / 256, 8LL * sm_count()));
}

}  // namespace

int dp_scan_tiles(long long n) { return (int)((n + kScanTile - 1) / kScanTile); }

cudaError_t launch_dp_flags(uint8_t* flags, const int8_t* tbin, int n, const int* max_bin,
                            cudaStream_t st) {
  dp_flags_k<<<grid_for(n), 256, 0, st>>>(flags, tbin, n, max_bin);
  return cudaGetLastError();
}

cudaError_t launch_dp_cells(const DPTree& t, const DPCellState& cs, const float4* posh,
                            const float* h0, const uint8_t* flags, bool force,
                            cudaStream_t st) {
  dp_cells_reset<<<grid_for(t.ncells), 256, 0, st>>>(cs, t.ncells, force ? 1 : 0);
  dp_cells_leaf<<<leaf_blocks(t.nleaves), 256, 0, st>>>(t, cs, posh, h0, flags, force ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t launch_dp_plan(const DPTree& t, const DPCellState& cs, int kind, const DPOut& o,
                           cudaStream_t st) {
  const int nb = leaf_blocks(t.nleaves);
  switch (kind) {
    case DP_DENSITY:
      dp_count_k<DP_DENSITY><<<nb, 256, 0, st>>>(t, cs, o);
      break;
    case DP_SUBSET:
      dp_count_k<DP_SUBSET><<<nb, 256, 0, st>>>(t, cs, o);
      break;
    default:
      dp_count_k<DP_FORCE><<<nb, 256, 0, st>>>(t, cs, o);
      break;
  }
  const long long n = (long long)t.nleaves + 1;
  const int nt = dp_scan_tiles(n);
  scan_tile_sums<<<nt, 256, 0, st>>>(o.leaf_off, n, o.tiles);
  scan_tile_prefix<<<1, 1024, 0, st>>>(o.tiles, nt);
  scan_apply<<<nt, 256, 0, st>>>(o.leaf_off, n, o.tiles);
  switch (kind) {
    case DP_DENSITY:
      dp_emit_k<DP_DENSITY><<<nb, 256, 0, st>>>(t, cs, o);
      break;
    case DP_SUBSET:
      dp_emit_k<DP_SUBSET><<<nb, 256, 0, st>>>(t, cs, o);
      break;
    default:
      dp_emit_k<DP_FORCE><<<nb, 256, 0, st>>>(t, cs, o);
      break;
  }
  return cudaGetLastError();
}

}  // namespace sphgpu
