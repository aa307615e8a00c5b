// cellassign.cu -- the rebuild's cell assignment on the device, from
// positions and smoothing lengths already in device memory:
//   top-level grid      space_regrid (space_regrid.c:46-121), cell_min from
//                       space.c:1263-1272 (Space::top_grid, shared with the
//                       host build)
//   top cell per part   space_parts_get_cell_index (space_cell_index.c:64-150)
//   octree split        space_split_recursive (space_split.c:196-300) /
//                       cell_split (cell_split.c:55-175): a cell of more than
//                       400 particles splits at its centre into octants
//   depth_h             cell_set_part_h_depth (cell.h:1787)
//
// Every particle gets one 64-bit key: its top cell in the high bits, then
// the octant it falls in at every level below the top cell, three bits per
// level, found with the split's own comparisons (x >= loc + width / 2, the
// child's corner loc + width / 2, all in FP64).  A stable radix sort of the
// keys puts every cell of every level in one contiguous range, in the
// reference's cell order (top cells by cell_getid, octants 0..7 below).
// Cell boundaries are then found level by level by binary searches in the
// sorted keys; the host keeps only the tree (O(cells)).
//
// The result is the reference's tree: the same cells, the same particle
// ranges and the same depth_h.  Inside a leaf the particles follow their
// octant path below the leaf and then the caller's order, where the
// reference's in-place bucket walk (space_sort.c:42-93) leaves another
// order; nothing in the loops depends on the order inside a leaf except the
// summation order.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <stdexcept>
#include <vector>

#include "../../include/swift_gb300.h"
#include "capi_util.h"
#include "device_sms.h"
#include "space.h"
#include "sph_types.h"

namespace sphgpu {
namespace {

using capi::DBuf;
using capi::fail;
using capi::guard;

constexpr int kThreads = 256;              // 8 warps
constexpr int kWarpItems = 256;            // items per warp in the radix passes
constexpr int kTile = 8 * kWarpItems;      // items per block
constexpr int kScanItems = 8;              // items per thread in the scan
constexpr int kScanTile = kThreads * kScanItems;

thread_local int g_launches;  // kernels launched by the calling thread's last call

enum CheckFlags : int {
  kNonFinite = 1,     // a non-finite position
  kOutside = 2,       // more than one box length outside the periodic box
  kOutsideOpen = 4,   // outside the non-periodic box
  kBadH = 8,          // h not positive and finite
};

// The largest h (and whether every h is positive and finite).
__global__ void ca_check_h(const float* __restrict__ h, int n, unsigned* hmax_bits, int* flags) {
  int bad = 0;
  unsigned hb = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float hh = h[i];
    if (!(hh > 0.f) || !isfinite(hh))
      bad |= kBadH;
    else
      hb = max(hb, __float_as_uint(hh));  // positive floats order as their bits
  }
  hb = __reduce_max_sync(0xffffffffu, hb);
  bad = __reduce_or_sync(0xffffffffu, (unsigned)bad);
  if ((threadIdx.x & 31) == 0) {
    if (hb) atomicMax(hmax_bits, hb);
    if (bad) atomicOr(flags, bad);
  }
}

struct Grid {
  double dim[3], width[3], iw[3];
  long long dim_bits[3];  // the bits of dim: non-negative doubles order as their bits
  double scale[3];        // 2^(levels + frac_bits) / width: x in fixed-point octant units
  long long eps;          // fixed-point units within which x may fall on either side
  int frac_bits;
  int cdim[3];
  int periodic, levels, path_bits;
};

// Key of every particle: top cell << path_bits | octant path (levels x 3
// bits, the first level highest); the value is the particle's index.  Bad
// positions are flagged (the keys are then not used).
//
// The split compares x with the pivots loc + width / 2 that the FP64 chain
// of child corners produces.  Those pivots lie within a few ulps of the
// dyadic points i width + k width / 2^l, which are whole numbers in units
// of the finest octant, T = x 2^levels / width.  T is taken in fixed point
// (frac_bits fractional bits, one FP64 multiply); where it is farther than
// eps from every whole number, its integer bits are the top cell and the
// octants of all levels at once.  Otherwise (a position on or next to a
// cell boundary) the rebuild's own FP64 chain decides.
__global__ void ca_keys(const double* __restrict__ x, int n, Grid g,
                        unsigned long long* __restrict__ key, int* __restrict__ val,
                        int* __restrict__ flags) {
  int bad = 0;
  const long long one = 1LL << g.frac_bits, fmask = one - 1;
  const long long qmask = (1LL << g.levels) - 1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double pos[3];
    bool chain = false;
    long long c[3], q[3];
    for (int d = 0; d < 3; d++) {
      double xx = x[3 * (size_t)i + d];
      long long b = __double_as_longlong(xx);
      if (((b >> 52) & 0x7ff) == 0x7ff) {
        bad |= kNonFinite;
        xx = 0.0;
        b = 0;
      }
      // outside [0, dim) (-0.0 counts as 0): the rebuild's wrap
      if ((b < 0 && b != (long long)0x8000000000000000ULL) || b >= g.dim_bits[d]) {
        if (g.periodic) {
          xx = wrap_periodic(xx, g.dim[d]);
          if (xx < 0.0 || xx > g.dim[d]) bad |= kOutside;
        } else {
          bad |= kOutsideOpen;
        }
        if (xx == g.dim[d]) xx = 0.0;
      }
      pos[d] = xx;
      const long long t = (long long)(xx * g.scale[d]);
      const long long fr = t & fmask;
      c[d] = t >> (g.levels + g.frac_bits);
      q[d] = (t >> g.frac_bits) & qmask;
      if (t < 0 || fr < g.eps || fr > one - g.eps || c[d] >= g.cdim[d]) chain = true;
    }
    int top;
    unsigned long long path = 0;
    if (!chain) {
      top = (int)(c[2] + g.cdim[2] * (c[1] + g.cdim[1] * c[0]));
      for (int l = g.levels - 1; l >= 0; l--)
        path = (path << 3) | (unsigned long long)((((q[0] >> l) & 1) << 2) |
                                                  (((q[1] >> l) & 1) << 1) | ((q[2] >> l) & 1));
    } else {
      top = top_cell_index(pos, g.iw, g.cdim);
      const int c2 = top % g.cdim[2], c1 = (top / g.cdim[2]) % g.cdim[1],
                c0 = top / (g.cdim[2] * g.cdim[1]);
      double loc[3] = {c0 * g.width[0], c1 * g.width[1], c2 * g.width[2]};
      double w[3] = {g.width[0], g.width[1], g.width[2]};
      for (int l = 0; l < g.levels; l++) {
        int digit = 0;
        for (int d = 0; d < 3; d++) {
          const double half = w[d] / 2;
          const double pivot = loc[d] + half;
          const int bb = pos[d] >= pivot;
          digit = 2 * digit + bb;
          if (bb) loc[d] = pivot;
          w[d] = half;
        }
        path = (path << 3) | (unsigned long long)digit;
      }
    }
    key[i] = ((unsigned long long)top << g.path_bits) | path;
    val[i] = i;
  }
  bad = __reduce_or_sync(0xffffffffu, (unsigned)bad);
  if ((threadIdx.x & 31) == 0 && bad) atomicOr(flags, bad);
}

// --- stable LSD radix sort, 8 bits per pass ---------------------------------

__device__ __forceinline__ int digit_of(unsigned long long k, int shift) {
  return (int)((k >> shift) & 0xffu);
}

// Per-block digit counts, digit-major: hist[d * nblocks + block].
__global__ void rs_hist(const unsigned long long* __restrict__ key, int n, int shift,
                        unsigned* __restrict__ hist) {
  __shared__ unsigned cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const long long base = (long long)blockIdx.x * kTile;
  for (int t = threadIdx.x; t < kTile; t += kThreads) {
    const long long e = base + t;
    if (e < n) atomicAdd(&cnt[digit_of(key[e], shift)], 1u);
  }
  __syncthreads();
  hist[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = cnt[threadIdx.x];
}

// Exclusive scan of a[0, n) in tiles of kScanTile; tile totals to sums.
__global__ void scan_tiles(unsigned* __restrict__ a, long long n, unsigned* __restrict__ sums) {
  __shared__ unsigned wsum[kThreads / 32];
  const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
  unsigned v[kScanItems], run = 0;
  for (int k = 0; k < kScanItems; k++) {
    v[k] = base + k < n ? a[base + k] : 0u;
    run += v[k];
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned inc = run;
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) wsum[w] = inc;
  __syncthreads();
  unsigned wpre = 0, tot = 0;
  for (int k = 0; k < kThreads / 32; k++) {
    if (k < w) wpre += wsum[k];
    tot += wsum[k];
  }
  unsigned ex = wpre + inc - run;
  for (int k = 0; k < kScanItems; k++) {
    if (base + k < n) a[base + k] = ex;
    ex += v[k];
  }
  if (threadIdx.x == 0 && sums) sums[blockIdx.x] = tot;
}

__global__ void add_tile_offsets(unsigned* __restrict__ a, long long n,
                                 const unsigned* __restrict__ offs) {
  const long long base = (long long)blockIdx.x * kScanTile;
  const unsigned o = offs[blockIdx.x];
  for (int t = threadIdx.x; t < kScanTile; t += kThreads)
    if (base + t < n) a[base + t] += o;
}

// Stable scatter: warp w of a block owns items [w * 256, (w + 1) * 256) of
// the block's tile and ranks them in index order, 32 at a time (lanes with
// the same digit in one round are ranked by lane); the tile is first
// ordered by digit in shared memory, then written out in runs of equal
// digits, so that consecutive threads store to consecutive addresses.
__global__ void rs_scatter(const unsigned long long* __restrict__ kin, const int* __restrict__ vin,
                           unsigned long long* __restrict__ kout, int* __restrict__ vout, int n,
                           int shift, const unsigned* __restrict__ offs) {
  __shared__ unsigned wcnt[8][256];
  __shared__ unsigned dstart[256], goff[256], wtot[8];
  __shared__ unsigned long long sk[kTile];
  __shared__ int sv[kTile];
  for (int t = threadIdx.x; t < 8 * 256; t += kThreads) (&wcnt[0][0])[t] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long long tbase = (long long)blockIdx.x * kTile;
  const long long wbase = tbase + (long long)w * kWarpItems;
  for (int r = 0; r < kWarpItems; r += 32) {
    const long long e = wbase + r + lane;
    if (e < n) atomicAdd(&wcnt[w][digit_of(kin[e], shift)], 1u);
  }
  __syncthreads();
  {
    // digit d = thread: its count in the tile, the tile's exclusive prefix
    // over digits (block scan), then per-warp starts inside the digit's run
    const int d = threadIdx.x;
    unsigned tot = 0;
    for (int k = 0; k < 8; k++) tot += wcnt[k][d];
    unsigned inc = tot;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    if (lane == 31) wtot[w] = inc;
    __syncthreads();
    unsigned pre = 0;
    for (int k = 0; k < w; k++) pre += wtot[k];
    unsigned run = pre + inc - tot;
    dstart[d] = run;
    goff[d] = offs[(size_t)d * gridDim.x + blockIdx.x];
    for (int k = 0; k < 8; k++) {
      const unsigned c = wcnt[k][d];
      wcnt[k][d] = run;
      run += c;
    }
  }
  __syncthreads();
  const unsigned lt = (1u << lane) - 1u;
  for (int r = 0; r < kWarpItems; r += 32) {
    const long long e = wbase + r + lane;
    const bool ok = e < n;
    unsigned long long k = 0;
    int v = 0, d = 256 + lane;  // a lane past the end is alone in its group
    if (ok) {
      k = kin[e];
      v = vin[e];
      d = digit_of(k, shift);
    }
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int leader = __ffs(peers) - 1;
    unsigned b = 0;
    if (ok && lane == leader) b = wcnt[w][d];
    b = __shfl_sync(0xffffffffu, b, leader);
    if (ok) {
      const unsigned pos = b + __popc(peers & lt);
      sk[pos] = k;
      sv[pos] = v;
      if (lane == leader) wcnt[w][d] = b + __popc(peers);
    }
    __syncwarp();
  }
  __syncthreads();
  const int tcount = (int)min((long long)kTile, (long long)n - tbase);
  for (int t = threadIdx.x; t < tcount; t += kThreads) {
    const unsigned long long k = sk[t];
    const int d = digit_of(k, shift);
    const unsigned dst = goff[d] + (unsigned)t - dstart[d];
    kout[dst] = k;
    vout[dst] = sv[t];
  }
}

// --- tree ------------------------------------------------------------------

__device__ __forceinline__ int lower_bound(const unsigned long long* __restrict__ key, int lo,
                                           int hi, unsigned long long v) {
  while (lo < hi) {
    const int mid = lo + ((hi - lo) >> 1);
    if (key[mid] < v)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

// Particle range of every top cell: int2 (first, count).
__global__ void ca_top_ranges(const unsigned long long* __restrict__ key, int n, int ntop,
                              int path_bits, int2* __restrict__ range) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntop) return;
  const int a = lower_bound(key, 0, n, (unsigned long long)t << path_bits);
  // (t + 1) << path_bits would leave the 64 bits for the last top cell
  const int b = t + 1 < ntop ? lower_bound(key, a, n, (unsigned long long)(t + 1) << path_bits) : n;
  range[t] = make_int2(a, b - a);
}

// Octant counts of every cell that splits: cell f = (first, count, depth);
// its particles share the key bits above level depth; child k's range
// starts at the first key with octant >= k at level depth.
__global__ void ca_children(const unsigned long long* __restrict__ key, const int4* __restrict__ split,
                            int nsplit, int levels, int* __restrict__ child_count) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nsplit) return;
  const int4 c = split[f];
  const int shift = 3 * (levels - c.z - 1);  // the child level's octant
  const unsigned long long pre = key[c.x] >> (shift + 3) << (shift + 3);
  int b[9];
  b[0] = c.x;
  b[8] = c.x + c.y;
  for (int k = 1; k < 8; k++)
    b[k] = lower_bound(key, b[k - 1], b[8], pre | ((unsigned long long)k << shift));
  for (int k = 0; k < 8; k++) child_count[8 * f + k] = b[k + 1] - b[k];
}

// depth_h of every particle, one warp per leaf (first, count, depth).
__global__ void ca_depth_h(const int2* __restrict__ leaf, int nleaf, const int* __restrict__ order,
                           const float* __restrict__ h, const float* __restrict__ hmin_d,
                           const float* __restrict__ hmax_d, int8_t* __restrict__ depth_h) {
  const int lw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (lw >= nleaf) return;
  const int2 l2 = leaf[lw];  // first, count | depth << 16
  const int4 L = make_int4(l2.x, l2.y & 0xffff, l2.y >> 16, 0);
  for (int k = L.x + (threadIdx.x & 31); k < L.x + L.y; k += 32) {
    const float hh = h[order[k]];
    int dh = 0;  // above the top cell: the reference leaves depth_h as it was
    if (hh < hmin_d[L.z]) {
      dh = L.z;
    } else {
      for (int d = L.z; d >= 0; d--)
        if (hh >= hmin_d[d] && hh < hmax_d[d]) {
          dh = d;
          break;
        }
    }
    depth_h[k] = (int8_t)dh;
  }
}

int blocks_for(long long n, int per_block, int cap = 0) {
  if (cap <= 0) cap = 32 * sm_count();
  const long long b = (n + per_block - 1) / per_block;
  return (int)std::max(1LL, std::min<long long>(b, cap));
}

// Exclusive scan of a device array of n unsigned (n < 2^31).
// tmp is a deque: its elements never move, so the buffers stay owned once.
void exclusive_scan(unsigned* a, long long n, cudaStream_t st, std::deque<DBuf<unsigned>>& tmp) {
  const long long tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles <= 1) {
    scan_tiles<<<1, kThreads, 0, st>>>(a, n, nullptr);
    CK(cudaGetLastError());
    ++g_launches;
    return;
  }
  tmp.emplace_back();
  DBuf<unsigned>& sums = tmp.back();
  sums.alloc((size_t)tiles);
  unsigned* sp = sums.p;
  scan_tiles<<<(unsigned)tiles, kThreads, 0, st>>>(a, n, sp);
  CK(cudaGetLastError());
  ++g_launches;
  exclusive_scan(sp, tiles, st, tmp);
  add_tile_offsets<<<(unsigned)tiles, kThreads, 0, st>>>(a, n, sp);
  CK(cudaGetLastError());
  ++g_launches;
}

// The tree on the host, one entry per cell in creation order (top cells,
// then every level's children, a parent's children consecutive).
struct Tree {
  std::vector<int> first, count, depth, parent, top, kid0, nkid;
  void clear() {
    for (auto* v : {&first, &count, &depth, &parent, &top, &kid0, &nkid}) v->clear();
  }
  void reserve(size_t m) {
    for (auto* v : {&first, &count, &depth, &parent, &top, &kid0, &nkid}) v->reserve(m);
  }
  int add(int f, int c, int d, int p, int t) {
    first.push_back(f);
    count.push_back(c);
    depth.push_back(d);
    parent.push_back(p);
    top.push_back(t);
    kid0.push_back(-1);
    nkid.push_back(0);
    return (int)first.size() - 1;
  }
  int size() const { return (int)first.size(); }
};

// Page-locked host staging that grows as needed.
template <class T>
struct Pinned {
  T* p = nullptr;
  size_t n = 0;
  T* get(size_t count) {
    if (count > n) {
      if (p) cudaFreeHost(p);
      p = nullptr;
      n = 0;
      CK(cudaMallocHost(&p, std::max<size_t>(count, 1) * sizeof(T)));
      n = count;
    }
    return p;
  }
  ~Pinned() {
    if (p) cudaFreeHost(p);
  }
};

// Device scratch kept between the calls of a host thread (a rebuild runs
// every step); it grows to the largest box seen and moves with the device.
struct Scratch {
  int device = -1;
  DBuf<unsigned long long> k0, k1;
  DBuf<int> v1, cbuf, flags;
  DBuf<unsigned> hist, scal;
  DBuf<int2> rng;
  DBuf<int4> fbuf;
  DBuf<int2> lbuf;
  DBuf<float> tab;
  Pinned<int> ch;
  Pinned<int2> leaves;
  template <class T>
  static void ensure(DBuf<T>& b, size_t count) {
    if (b.n < count || !b.p) b.alloc(count);
  }
  void on_device(int dev) {
    if (dev == device) return;
    k0.release(); k1.release(); v1.release(); cbuf.release(); flags.release();
    hist.release(); scal.release(); rng.release(); fbuf.release(); lbuf.release();
    tab.release();
    device = dev;
  }
};
thread_local Scratch g_scratch;

// Host-clock phases of the calling thread's last call (ms): [0] h scan and
// grid, [1] keys and sort, [2] tree levels, [3] numbering and records, [4]
// depth_h (each up to its own synchronisation).
thread_local double g_phase_ms[5];
using Clock = std::chrono::steady_clock;
double ms_since(Clock::time_point& t) {
  const auto now = Clock::now();
  const double ms = std::chrono::duration<double, std::milli>(now - t).count();
  t = now;
  return ms;
}

}  // namespace
}  // namespace sphgpu

using namespace sphgpu;

int sphgpu_cell_assign(const sphgpu_params* prm, const double* x, const float* h, int64_t n,
                       int32_t* order, int8_t* depth_h, int32_t cdim_out[3], int32_t* ncells,
                       int32_t* cells, int32_t max_cells, void* stream) {
  if (!prm || !x || !h || !order || !depth_h || !cdim_out || !ncells || n <= 0)
    return fail(SPHGPU_EINVAL, "sphgpu_cell_assign: null argument or n <= 0");
  if (n > SPHGPU_MAX_PARTICLES)
    return fail(SPHGPU_EINVAL, "sphgpu_cell_assign: more than SPHGPU_MAX_PARTICLES particles");
  if (prm->max_top_level_cells < 3 || !(prm->dim[0] > 0) || !(prm->dim[1] > 0) ||
      !(prm->dim[2] > 0))
    return fail(SPHGPU_EINVAL, "sphgpu_cell_assign: invalid parameters");
  return guard([&]() {
    cudaStream_t st = (cudaStream_t)stream;
    const int N = (int)n;
    Params P;
    for (int d = 0; d < 3; d++) P.dim[d] = prm->dim[d];
    P.periodic = prm->periodic;
    P.max_top_level_cells = prm->max_top_level_cells;

    auto tmark = Clock::now();
    for (double& v : g_phase_ms) v = 0.0;
    g_launches = 0;
    int dev = 0;
    CK(cudaGetDevice(&dev));
    Scratch& S = g_scratch;
    S.on_device(dev);

    // 1. the largest h (positions are checked with the keys)
    Scratch::ensure(S.scal, 2);
    CK(cudaMemsetAsync(S.scal.p, 0, 2 * sizeof(unsigned), st));
    ca_check_h<<<blocks_for(N, kThreads), kThreads, 0, st>>>(h, N, S.scal.p,
                                                              (int*)(S.scal.p + 1));
    CK(cudaGetLastError());
    ++g_launches;
    unsigned hs[2];
    CK(cudaMemcpyAsync(hs, S.scal.p, sizeof(hs), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (hs[1] & kBadH) throw std::runtime_error("smoothing lengths must be positive and finite");
    float max_h;
    std::memcpy(&max_h, &hs[0], sizeof(float));
    g_phase_ms[0] += ms_since(tmark);

    // 2. grid and key layout
    Grid g{};
    Space::top_grid(P, max_h, g.cdim, g.width);
    for (int d = 0; d < 3; d++) {
      g.dim[d] = P.dim[d];
      g.iw[d] = 1.0 / g.width[d];
      cdim_out[d] = g.cdim[d];
    }
    g.periodic = P.periodic;
    const long long ntop_l = (long long)g.cdim[0] * g.cdim[1] * g.cdim[2];
    if (ntop_l > (1LL << 30)) throw std::runtime_error("too many top-level cells");
    const int ntop = (int)ntop_l;
    int top_bits = 1;
    while ((1LL << top_bits) < ntop_l) top_bits++;
    // Keys of at most 32 bits first (four radix passes); where the tree
    // reaches below their levels, once more with as many levels as 64 bits
    // hold.
    const int levels_full = std::min(SPH_MAX_DEPTH - 1, (64 - top_bits) / 3);
    const int levels_short = std::max(1, std::min(levels_full, (32 - top_bits) / 3));

    Scratch::ensure(S.k0, N);
    Scratch::ensure(S.k1, N);
    Scratch::ensure(S.v1, N);
    const int nblk = (int)((n + kTile - 1) / kTile);
    Scratch::ensure(S.hist, (size_t)256 * nblk);
    Scratch::ensure(S.rng, ntop);
    Scratch::ensure(S.flags, 1);
    DBuf<unsigned long long>&k0 = S.k0, &k1 = S.k1;
    DBuf<int>&v1 = S.v1, &cbuf = S.cbuf;
    DBuf<unsigned>& hist = S.hist;
    DBuf<int2>& rng = S.rng;
    DBuf<int4>& fbuf = S.fbuf;
    Tree T;
    T.reserve((size_t)ntop + 16 * ((size_t)n / (Space::kSplitSize + 1)) + 64);
    const unsigned long long* key = nullptr;
    double wmin = g.width[0], dmax = g.dim[0];
    for (int d = 1; d < 3; d++) {
      wmin = std::min(wmin, g.width[d]);
      dmax = std::max(dmax, g.dim[d]);
    }
    for (int attempt = 0; attempt < 2; attempt++) {
      g.levels = attempt == 0 ? levels_short : levels_full;
      g.path_bits = 3 * g.levels;
      const int key_bits = top_bits + g.path_bits;
      // Fixed point: T = x 2^levels / width < cdim 2^levels, held with
      // frac_bits more bits while T 2^frac_bits stays exact in FP64 to 2^-1.
      int axis_bits = 1;
      for (int d = 0; d < 3; d++)
        while ((1LL << axis_bits) < g.cdim[d]) axis_bits++;
      g.frac_bits = std::max(0, std::min(20, 51 - g.levels - axis_bits));
      for (int d = 0; d < 3; d++) {
        g.scale[d] = std::ldexp(std::ldexp(1.0, g.levels) * g.iw[d], g.frac_bits);
        std::memcpy(&g.dim_bits[d], &g.dim[d], sizeof(double));
      }
      // Distance (octant units) between a chain pivot and its dyadic point
      // (a rounding per level of the corner chain and of loc_top), plus the
      // rounding of T itself and the fixed-point truncation, generously.
      const double tmax = std::ldexp(1.0, g.levels);
      const double eps_t = 1024.0 * DBL_EPSILON * dmax * tmax / wmin +
                           8.0 * std::ldexp(1.0, g.levels + axis_bits - 52);
      g.eps = (long long)std::ceil(eps_t * std::ldexp(1.0, g.frac_bits)) + 2;

      // 3. keys, sorted
      int* v0 = order;  // the sort ends in the caller's buffer after an even pass count
      CK(cudaMemsetAsync(S.flags.p, 0, sizeof(int), st));
      ca_keys<<<blocks_for(N, kThreads), kThreads, 0, st>>>(x, N, g, k0.p, v0, S.flags.p);
      CK(cudaGetLastError());
      ++g_launches;
      const int npass = (key_bits + 7) / 8;
      unsigned long long *ka = k0.p, *kb = k1.p;
      int *va = v0, *vb = v1.p;
      std::deque<DBuf<unsigned>> scan_tmp;
      for (int p = 0; p < npass; p++) {
        const int shift = 8 * p;
        rs_hist<<<nblk, kThreads, 0, st>>>(ka, N, shift, hist.p);
        CK(cudaGetLastError());
        ++g_launches;
        exclusive_scan(hist.p, (long long)256 * nblk, st, scan_tmp);
        rs_scatter<<<nblk, kThreads, 0, st>>>(ka, va, kb, vb, N, shift, hist.p);
        CK(cudaGetLastError());
        ++g_launches;
        std::swap(ka, kb);
        std::swap(va, vb);
      }
      if (va != order)
        CK(cudaMemcpyAsync(order, va, sizeof(int) * (size_t)N, cudaMemcpyDeviceToDevice, st));
      key = ka;

      // 4. the tree, level by level
      ca_top_ranges<<<(ntop + kThreads - 1) / kThreads, kThreads, 0, st>>>(key, N, ntop,
                                                                            g.path_bits, rng.p);
      CK(cudaGetLastError());
      ++g_launches;
      std::vector<int2> top(ntop);
      CK(cudaMemcpyAsync(top.data(), rng.p, sizeof(int2) * ntop, cudaMemcpyDeviceToHost, st));
      int bad = 0;
      CK(cudaMemcpyAsync(&bad, S.flags.p, sizeof(int), cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      if (bad & kNonFinite) throw std::runtime_error("non-finite position");
      if (bad & kOutside)
        throw std::runtime_error("particle more than one box length outside the periodic box");
      if (bad & kOutsideOpen) throw std::runtime_error("particle outside the non-periodic box");
      g_phase_ms[1] += ms_since(tmark);
      T.clear();
      long long total = 0;
      for (int t = 0; t < ntop; t++) {
        T.add(top[t].x, top[t].y, 0, -1, t);
        total += top[t].y;
      }
      if (total != n) throw std::runtime_error("cell assignment lost particles");
      std::vector<int> frontier;
      for (int t = 0; t < ntop; t++)
        if (T.count[t] > Space::kSplitSize) frontier.push_back(t);
      std::vector<int4> fh;
      bool deeper = false;
      while (!frontier.empty() && !deeper) {
        fh.resize(frontier.size());
        for (size_t f = 0; f < frontier.size(); f++) {
          const int c = frontier[f];
          if (T.depth[c] >= SPH_MAX_DEPTH - 1)
            throw std::runtime_error(
                "cell tree deeper than supported (particles at identical positions?)");
          if (T.depth[c] >= g.levels) {
            if (g.levels == levels_full)
              throw std::runtime_error("cell tree deeper than the device keys resolve");
            deeper = true;
          }
          fh[f] = make_int4(T.first[c], T.count[c], T.depth[c], 0);
        }
        if (deeper) break;
        const int nf = (int)fh.size();
        fbuf.upload(fh.data(), nf, st);
        if (cbuf.n < (size_t)8 * nf) cbuf.alloc((size_t)8 * nf);
        ca_children<<<(nf + kThreads - 1) / kThreads, kThreads, 0, st>>>(key, fbuf.p, nf,
                                                                          g.levels, cbuf.p);
        CK(cudaGetLastError());
        ++g_launches;
        int* ch = S.ch.get((size_t)8 * nf);
        CK(cudaMemcpyAsync(ch, cbuf.p, sizeof(int) * 8 * nf, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        std::vector<int> next;
        for (int f = 0; f < nf; f++) {
          const int pc = frontier[f];
          int off = T.first[pc];
          const int dep = T.depth[pc] + 1, tp = T.top[pc];
          T.kid0[pc] = T.size();
          for (int k = 0; k < 8; k++) {
            const int cnt = ch[8 * f + k];
            if (cnt == 0) continue;
            const int c = T.add(off, cnt, dep, pc, tp);
            T.nkid[pc]++;
            off += cnt;
            if (cnt > Space::kSplitSize) next.push_back(c);
          }
          if (off != T.first[pc] + T.count[pc])
            throw std::runtime_error("cell assignment lost particles in a split");
        }
        frontier.swap(next);
      }
      g_phase_ms[2] += ms_since(tmark);
      if (!deeper) break;
    }

    // 5. the host build's numbering: top cells in cell_getid order, then
    // every top cell's subtree in preorder (a cell before its children, a
    // child's whole subtree before the next child), from subtree sizes;
    // creation order has parents before children
    const int nc = T.size();
    *ncells = nc;
    std::vector<int> size(nc, 1), id(nc, -1);
    for (int c = nc - 1; c >= ntop; c--) size[T.parent[c]] += size[c];
    int base = ntop;
    for (int c = 0; c < nc; c++) {
      int pos;
      if (c < ntop) {
        id[c] = c;
        pos = base;
        base += size[c] - 1;
      } else {
        pos = id[c] + 1;
      }
      for (int k = 0; k < T.nkid[c]; k++) {
        const int kid = T.kid0[c] + k;
        id[kid] = pos;
        pos += size[kid];
      }
    }
    if (cells && max_cells >= nc) {
      for (int c = 0; c < nc; c++) {
        int32_t* r = cells + 5 * (size_t)id[c];
        r[0] = T.first[c];
        r[1] = T.count[c];
        r[2] = T.depth[c];
        r[3] = T.parent[c] >= 0 ? id[T.parent[c]] : -1;
        r[4] = T.top[c];
      }
    }
    g_phase_ms[3] += ms_since(tmark);

    // 6. depth_h
    float hmin_d[SPH_MAX_DEPTH], hmax_d[SPH_MAX_DEPTH];
    {
      float dmin = std::min(std::min((float)g.width[0], (float)g.width[1]), (float)g.width[2]);
      for (int d = 0; d < SPH_MAX_DEPTH; d++) {
        Cell c;
        c.dmin = dmin;
        c.h_min_allowed = c.dmin * 0.5 * (1. / SPH_KG);
        c.h_max_allowed = c.dmin * (1. / SPH_KG);
        hmin_d[d] = c.h_min_allowed;
        hmax_d[d] = c.h_max_allowed;
        dmin = c.dmin / 2;
      }
    }
    int nl = 0;
    for (int c = 0; c < nc; c++)
      if (T.count[c] > 0 && T.nkid[c] == 0) nl++;
    int2* leaves = S.leaves.get(nl);
    nl = 0;
    for (int c = 0; c < nc; c++)
      if (T.count[c] > 0 && T.nkid[c] == 0)
        leaves[nl++] = make_int2(T.first[c], T.count[c] | T.depth[c] << 16);
    DBuf<int2>& lbuf = S.lbuf;
    lbuf.upload(leaves, nl, st);
    DBuf<float>& tab = S.tab;
    std::vector<float> tabh(hmin_d, hmin_d + SPH_MAX_DEPTH);
    tabh.insert(tabh.end(), hmax_d, hmax_d + SPH_MAX_DEPTH);
    tab.upload(tabh.data(), tabh.size(), st);
    ca_depth_h<<<(nl * 32 + kThreads - 1) / kThreads, kThreads, 0, st>>>(
        lbuf.p, nl, order, h, tab.p, tab.p + SPH_MAX_DEPTH, depth_h);
    CK(cudaGetLastError());
    ++g_launches;
    CK(cudaStreamSynchronize(st));
    g_phase_ms[4] += ms_since(tmark);
    if (cells && max_cells < nc)
      return fail(SPHGPU_EINVAL, "sphgpu_cell_assign: cells buffer too small (see *ncells)");
    return SPHGPU_OK;
  });
}

int sphgpu_cell_assign_times(double ms[6]) {
  if (!ms) return fail(SPHGPU_EINVAL, "sphgpu_cell_assign_times: null argument");
  for (int k = 0; k < 5; k++) ms[k] = g_phase_ms[k];
  ms[5] = g_launches;
  return SPHGPU_OK;
}
