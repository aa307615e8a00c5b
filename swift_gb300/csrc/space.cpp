// space.cpp -- host-side planner: the reference's space build (top-level
// grid, particle -> cell index, octree split, h-depth) and the reference's
// task recursion, turned into gather lists for the sm_103a kernels.
//
// The tree must be the reference's tree, bit for bit, because the reference
// evaluates every neighbour pair in the frame of the cell pair that its
// recursion reaches; the kernels reproduce that frame for borderline pairs.
// References (paths relative to the reference's src/):
//   grid size        space.c:1263-1272, space_regrid.c:46-121
//   cell index       space_cell_index.c:64-150 (cell_getid, cell.h:532)
//   particle order   space_sort.c:42-93 (bucket permutation)
//   split            space_split.c:196-300, cell_split.c:55-175
//   h-depth          cell.h:1787 (cell_set_part_h_depth)
//   pair direction   space_getsid.h:47-80
//   recursion        runner_doiact_functions_hydro.h:2933 (DOSUB_PAIR1),
//                    :3037 (DOSUB_SELF1), :3102 (DOSUB_PAIR2),
//                    :3203 (DOSUB_SELF2), :3290-3360 (subset recursion)
//   predicates       cell.h:934-1010
#include "space.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <exception>
#include <mutex>
#include <thread>
#include <cstring>
#include <stdexcept>

namespace sphgpu {

// Planning runs on the host cores: work items are handed out in blocks by an
// atomic counter; each block keeps its own output, merged in block order so
// that the plan is the same for any number of threads.
namespace {
int planner_threads() {
  const unsigned t = std::thread::hardware_concurrency();
  return (int)std::max(1u, std::min(t, 16u));
}

template <class F>
void parallel_blocks(int nthreads, int nblocks, F&& body) {
  const int nt = std::min(nthreads, nblocks);
  if (nt <= 1) {
    for (int b = 0; b < nblocks; b++) body(b);
    return;
  }
  std::atomic<int> next{0};
  std::exception_ptr err;
  std::mutex mu;
  auto run = [&]() {
    try {
      for (int b = next++; b < nblocks; b = next++) body(b);
    } catch (...) {
      std::lock_guard<std::mutex> lock(mu);
      if (!err) err = std::current_exception();
      next = nblocks;
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; t++) pool.emplace_back(run);
  run();
  for (auto& th : pool) th.join();
  if (err) std::rethrow_exception(err);
}
}  // namespace


static inline float fmaxr(float a, float b) { return a > b ? a : b; }
static inline float fminr(float a, float b) { return a < b ? a : b; }

// Children of ci (after the canonical swap) that touch children of cj, for
// each of the 13 axes: child p of ci at octant (px,py,pz), child q of cj at
// octant (qx,qy,qz), cj displaced by the axis direction d; they touch when
// |2 d_k + q_k - p_k| <= 1 on every axis.
static void child_pairs(int sid, std::vector<std::pair<int, int>>& out) {
  static const int dir[13][3] = {{1, 1, 1},  {1, 1, 0},  {1, 1, -1}, {1, 0, 1},
                                 {1, 0, 0},  {1, 0, -1}, {1, -1, 1}, {1, -1, 0},
                                 {1, -1, -1}, {0, 1, 1}, {0, 1, 0},  {0, 1, -1},
                                 {0, 0, 1}};
  out.clear();
  for (int p = 0; p < 8; p++)
    for (int q = 0; q < 8; q++) {
      const int pb[3] = {(p >> 2) & 1, (p >> 1) & 1, p & 1};
      const int qb[3] = {(q >> 2) & 1, (q >> 1) & 1, q & 1};
      bool touch = true;
      for (int k = 0; k < 3; k++)
        if (std::abs(2 * dir[sid][k] + qb[k] - pb[k]) > 1) touch = false;
      if (touch) out.emplace_back(p, q);
    }
}

Space::Space(const Params& prm) : prm_(prm) {
  for (int s = 0; s < 13; s++) child_pairs(s, cpairs_[s]);
}

int Space::getsid_and_swap(int& ci, int& cj, double shift[3]) const {
  double dx[3];
  for (int k = 0; k < 3; k++) {
    dx[k] = cells_[cj].loc[k] - cells_[ci].loc[k];
    if (prm_.periodic && dx[k] < -prm_.dim[k] / 2)
      shift[k] = prm_.dim[k];
    else if (prm_.periodic && dx[k] > prm_.dim[k] / 2)
      shift[k] = -prm_.dim[k];
    else
      shift[k] = 0.0;
    dx[k] += shift[k];
  }
  int idx = 0;
  for (int k = 0; k < 3; k++)
    idx = 3 * idx + ((dx[k] < 0.0) ? 0 : ((dx[k] > 0.0) ? 2 : 1));
  if (idx < 13) {
    std::swap(ci, cj);
    for (int k = 0; k < 3; k++) shift[k] = -shift[k];
    return idx;
  }
  return 26 - idx;
}

// ---------------------------------------------------------------------------
// Space build

void Space::bucket_permute(std::vector<int>& bin, int nbins, int first,
                           int n, std::vector<int>& counts_out) {
  // In-place cycle walk of space_sort.c:42-93 / cell_split.c:120-150; the
  // order inside each bin is the reference's.
  std::vector<int> count(nbins, 0), off(nbins + 1, 0);
  for (int k = 0; k < n; k++) count[bin[k]]++;
  for (int k = 1; k <= nbins; k++) {
    off[k] = off[k - 1] + count[k - 1];
    count[k - 1] = 0;
  }
  int* perm = perm_.data() + first;
  for (int b = 0; b < nbins; b++) {
    for (int k = off[b] + count[b]; k < off[b + 1]; k++) {
      count[b]++;
      int target = bin[k];
      if (target == b) continue;
      int tmp = perm[k];
      while (target != b) {
        int j = off[target] + count[target]++;
        while (bin[j] == target) j = off[target] + count[target]++;
        std::swap(perm[j], tmp);
        std::swap(bin[j], target);
      }
      perm[k] = tmp;
      bin[k] = target;
    }
  }
  counts_out.assign(nbins, 0);
  for (int b = 0; b < nbins; b++) counts_out[b] = off[b + 1] - off[b];
}

void Space::octant_permute(int first, int n, const double pivot[3],
                           int counts[8]) {
  std::vector<int> bin(n);
  int bcount[8] = {0, 0, 0, 0, 0, 0, 0, 0}, boff[9];
  int* perm = perm_.data() + first;
  for (int k = 0; k < n; k++) {
    const double* x = &x_[3 * (size_t)perm[k]];
    bin[k] = (x[0] >= pivot[0]) * 4 + (x[1] >= pivot[1]) * 2 + (x[2] >= pivot[2]);
    bcount[bin[k]]++;
  }
  boff[0] = 0;
  for (int k = 1; k <= 8; k++) {
    boff[k] = boff[k - 1] + bcount[k - 1];
    bcount[k - 1] = 0;
  }
  for (int b = 0; b < 8; b++) {
    for (int k = boff[b] + bcount[b]; k < boff[b + 1]; k++) {
      int bid = bin[k];
      if (bid != b) {
        int part = perm[k];
        int tbin = bin[k];
        while (bid != b) {
          int j = boff[bid] + bcount[bid]++;
          while (bin[j] == bid) {
            j++;
            bcount[bid]++;
          }
          std::swap(perm[j], part);
          std::swap(bin[j], tbin);
          bid = tbin;
        }
        perm[k] = part;
        bin[k] = tbin;
      }
      bcount[bid]++;
    }
  }
  for (int b = 0; b < 8; b++) counts[b] = bcount[b];
}

int8_t Space::h_depth_of(float h, int leaf) const {
  int c = leaf;
  if (h < cells_[c].h_min_allowed) return (int8_t)cells_[c].depth;
  while (c >= 0) {
    if (h >= cells_[c].h_min_allowed && h < cells_[c].h_max_allowed)
      return (int8_t)cells_[c].depth;
    c = cells_[c].parent;
  }
  return 0;  // above the top cell: the reference leaves depth_h unchanged
}

void Space::set_h_depth(int sorted_idx, int leaf) {
  const float h = h_[sorted_idx];
  int c = leaf;
  if (h < cells_[c].h_min_allowed) {
    depth_h_[sorted_idx] = (int8_t)cells_[c].depth;
    return;
  }
  while (c >= 0) {
    if (h >= cells_[c].h_min_allowed && h < cells_[c].h_max_allowed) {
      depth_h_[sorted_idx] = (int8_t)cells_[c].depth;
      return;
    }
    c = cells_[c].parent;
  }
}

void Space::top_grid(const Params& prm, float max_h, int cdim[3], double width[3]) {
  // space_regrid (space_regrid.c:46-121) with cell_min from space_init
  // (space.c:1263-1272): cells at least 1.10 * gamma * h_max wide, at most
  // max_top_level_cells per side of the largest dimension.
  const int maxt = prm.max_top_level_cells;
  const double dmax = std::max(std::max(prm.dim[0], prm.dim[1]), prm.dim[2]);
  const float tol = fmaxr((float)(1.0 - 1.0 / (maxt * maxt)), (float)0.99);
  const double cell_min = tol * dmax / maxt;
  float hmax = cell_min / SPH_KG / 1.10f;
  if (max_h > hmax) hmax = max_h;
  for (int d = 0; d < 3; d++) {
    cdim[d] = (int)std::floor(prm.dim[d] / std::fmax(hmax * SPH_KG * 1.10f, cell_min));
    if (cdim[d] < 1) throw std::runtime_error("top-level cell dimension of 0");
    if (prm.periodic && cdim[d] < 3)
      throw std::runtime_error("periodic box needs at least 3 top cells per axis");
    width[d] = prm.dim[d] / cdim[d];
  }
}

void Space::build(int64_t n, const double* x, const float* h,
                  const int8_t* time_bin, const int32_t* order, const int32_t* tree,
                  int ncells) {
  if (n <= 0 || n > (int64_t)0x7fffffff - 16)
    throw std::runtime_error("particle count out of range");
  n_ = (int)n;
  x_.assign(x, x + 3 * (size_t)n);
  for (int k = 0; k < n_; k++)
    for (int d = 0; d < 3; d++) {
      double& xx = x_[3 * (size_t)k + d];
      if (!std::isfinite(xx)) throw std::runtime_error("non-finite position");
      if (prm_.periodic) {
        xx = wrap_periodic(xx, prm_.dim[d]);
        if (xx < 0 || xx > prm_.dim[d])
          throw std::runtime_error("particle more than one box length outside the periodic box");
      } else if (xx < 0 || xx >= prm_.dim[d]) {
        throw std::runtime_error("particle outside the non-periodic box");
      }
    }
  // Top-level grid.
  float max_h = 0.f;
  for (int k = 0; k < n_; k++) {
    if (!(h[k] > 0.f) || !std::isfinite(h[k]))
      throw std::runtime_error("smoothing lengths must be positive and finite");
    if (h[k] > max_h) max_h = h[k];
  }
  top_grid(prm_, max_h, cdim_, width_);
  const double iw[3] = {1.0 / width_[0], 1.0 / width_[1], 1.0 / width_[2]};
  const float dmin = fminr(fminr((float)width_[0], (float)width_[1]), (float)width_[2]);
  const int ntop = cdim_[0] * cdim_[1] * cdim_[2];
  std::vector<int> bin(n_);
  for (int k = 0; k < n_; k++) {
    double pos[3];
    for (int d = 0; d < 3; d++) {
      double xx = x_[3 * (size_t)k + d];
      if (xx == prm_.dim[d]) xx = 0.0;
      pos[d] = xx;
      x_[3 * (size_t)k + d] = xx;
    }
    bin[k] = top_cell_index(pos, iw, cdim_);
  }
  perm_.resize(n_);
  std::vector<int> counts;
  adopted_ = order != nullptr;
  if (order) {
    // the tree came from the device assignment: its order and top counts
    if (ncells < ntop) throw std::runtime_error("assigned tree has fewer cells than the grid");
    std::vector<uint8_t> seen(n_, 0);
    for (int k = 0; k < n_; k++) {
      const int i = order[k];
      if (i < 0 || i >= n_ || seen[i]) throw std::runtime_error("assigned order is not a permutation");
      seen[i] = 1;
      perm_[k] = i;
    }
    // top-cell counts: non-negative, adding up to n, and every particle in
    // the range of the top cell its position falls in
    counts.resize(ntop);
    long long total = 0;
    for (int c = 0; c < ntop; c++) {
      counts[c] = tree[5 * (size_t)c + 1];
      if (counts[c] < 0) throw std::runtime_error("assigned tree: negative top-cell count");
      total += counts[c];
    }
    if (total != n_) throw std::runtime_error("assigned tree: top-cell counts do not add up to n");
    for (int c = 0, k = 0; c < ntop; c++)
      for (int e = k + counts[c]; k < e; k++)
        if (bin[perm_[k]] != c)
          throw std::runtime_error("assigned tree: a particle is not in its top cell's range");
  } else {
    for (int k = 0; k < n_; k++) perm_[k] = k;
    bucket_permute(bin, ntop, 0, n_, counts);
  }
  cells_.clear();
  cells_.resize(ntop);
  for (int i = 0; i < cdim_[0]; i++)
    for (int j = 0; j < cdim_[1]; j++)
      for (int k = 0; k < cdim_[2]; k++) {
        const int cid = k + cdim_[2] * (j + cdim_[1] * i);
        Cell& c = cells_[cid];
        c.loc[0] = i * width_[0];
        c.loc[1] = j * width_[1];
        c.loc[2] = k * width_[2];
        for (int d = 0; d < 3; d++) c.width[d] = width_[d];
        c.dmin = dmin;
        c.h_min_allowed = c.dmin * 0.5 * (1. / SPH_KG);
        c.h_max_allowed = c.dmin * (1. / SPH_KG);
        c.top = cid;
      }
  // Octree split needs sorted-order h and activity; fill them in the
  // permuted order first (octant permutations below keep them in step).
  h_in_.assign(h, h + n_);
  tb_in_.assign(time_bin, time_bin + n_);
  int off = 0;
  for (int cid = 0; cid < ntop; cid++) {
    cells_[cid].first = off;
    cells_[cid].count = counts[cid];
    off += counts[cid];
  }
  h_.assign(n_, 0.f);
  active_.assign(n_, 0);
  depth_h_.assign(n_, 0);
  leaf_of_.assign(n_, -1);
  leaves_.clear();
  // The split permutes perm_ inside each top cell; h_/active_ are refreshed
  // from perm_ before each leaf is finalised, so refresh them per top cell
  // after the split of that cell has reordered it.
  if (order) {
    adopt_tree(tree, ncells);
    for (int cid = 0; cid < ntop; cid++)
      if (cells_[cid].count > 0) finalize_h(cid);
  } else {
    for (int cid = 0; cid < ntop; cid++) {
      if (cells_[cid].count == 0) continue;
      // Octant permutations only reorder within [first, first+count); h and
      // activity are gathered for the final order once the subtree is built.
      split_tree_then_gather(cid);
    }
  }
  // Inverse permutation.
  inv_perm_.resize(n_);
  for (int k = 0; k < n_; k++) inv_perm_[perm_[k]] = k;
  build_top_pairs();
  build_gpu_order();
  bin_members_.assign(256, {});
  active_list_.clear();
  for (int k = 0; k < n_; k++) {
    bin_members_[tb_in_[perm_[k]] + 128].push_back(k);
    if (active_[k]) active_list_.push_back(k);
  }
  cell_mark_.assign(cells_.size(), 0);
  force_checks_.clear();
  for (size_t c = 0; c < cells_.size(); c++)
    if (cells_[c].split && cells_[c].count >= kRecurseSize)
      force_checks_.push_back({cells_[c].first, cells_[c].count, cells_[c].dmin, (int)c});
  h_conv_.clear();
}

static inline uint32_t spread10(uint32_t v) {
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000ffu;
  v = (v | (v << 8)) & 0x0300f00fu;
  v = (v | (v << 4)) & 0x030c30c3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

void Space::build_gpu_order() {
  gperm_ = perm_;
  g_of_s_.assign(n_, 0);
  jb_ = JBlocks();
  jb_.cell_begin.assign(cells_.size(), 0);
  jb_.cell_end.assign(cells_.size(), 0);
  std::vector<std::pair<uint32_t, int>> key;
  std::vector<int> leaf_block_begin(leaves_.size() + 1, 0);
  // An adopted order follows each particle's octant path down to the levels
  // the device cell assignment's keys hold: as many as 32-bit keys hold
  // (top cell in the high bits, 3 bits a level) when every split cell lies
  // above them, else as many as 64-bit keys hold.  A leaf at that depth has
  // no path bits left below it (its particles keep their input order).
  int adopt_levels = 1 << 30;
  if (adopted_) {
    const long long ntop = (long long)cdim_[0] * cdim_[1] * cdim_[2];
    int top_bits = 1;
    while ((1LL << top_bits) < ntop) top_bits++;
    const int lfull = std::min(SPH_MAX_DEPTH - 1, (64 - top_bits) / 3);
    const int lshort = std::max(1, std::min(lfull, (32 - top_bits) / 3));
    int max_split = -1;
    for (const Cell& c : cells_)
      if (c.split) max_split = std::max(max_split, c.depth);
    adopt_levels = max_split < lshort ? lshort : lfull;
  }
  for (size_t l = 0; l < leaves_.size(); l++) {
    const Cell& c = cells_[leaves_[l]];
    if (adopted_ && c.depth < adopt_levels) {
      // an adopted order already follows each particle's octant path inside
      // its leaf (a Morton order at the split's own pivots): keep it
      for (int k = c.first; k < c.first + c.count; k++) {
        gperm_[k] = perm_[k];
        g_of_s_[k] = k;
      }
    } else {
    key.clear();
    for (int k = c.first; k < c.first + c.count; k++) {
      const double* x = &x_[3 * (size_t)perm_[k]];
      uint32_t q[3];
      for (int d = 0; d < 3; d++) {
        double t = (x[d] - c.loc[d]) / c.width[d];
        t = t < 0 ? 0 : (t > 0.999999 ? 0.999999 : t);
        q[d] = (uint32_t)(t * 1024.0);
      }
      key.emplace_back((spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]), k);
    }
    std::stable_sort(key.begin(), key.end());
    for (size_t r = 0; r < key.size(); r++) {
      gperm_[c.first + (int)r] = perm_[key[r].second];
      g_of_s_[key[r].second] = c.first + (int)r;
    }
    }
    leaf_block_begin[l] = (int)jb_.first.size();
    const Cell& top = cells_[c.top];
    for (int b0 = c.first; b0 < c.first + c.count; b0 += jblock_) {
      const int bc = std::min(jblock_, c.first + c.count - b0);
      float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
      for (int k = b0; k < b0 + bc; k++) {
        const double* x = &x_[3 * (size_t)gperm_[k]];
        for (int d = 0; d < 3; d++) {
          const float o = (float)(x[d] - top.loc[d]);
          lo[d] = std::min(lo[d], o);
          hi[d] = std::max(hi[d], o);
        }
      }
      jb_.first.push_back(b0);
      jb_.count.push_back(bc);
      for (int d = 0; d < 3; d++) {
        jb_.lo.push_back(lo[d]);
        jb_.hi.push_back(hi[d]);
      }
      for (int q = 0; q < 4; q++) {
        float sl[3] = {3.4e38f, 3.4e38f, 3.4e38f}, sh[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
        const int k0 = b0 + q * kSubBlock, k1 = std::min(b0 + bc, k0 + kSubBlock);
        for (int k = k0; k < k1; k++) {
          const double* x = &x_[3 * (size_t)gperm_[k]];
          for (int d = 0; d < 3; d++) {
            const float o = (float)(x[d] - top.loc[d]);
            sl[d] = std::min(sl[d], o);
            sh[d] = std::max(sh[d], o);
          }
        }
        for (int d = 0; d < 3; d++) {
          jb_.sub_lo.push_back(sl[d]);
          jb_.sub_hi.push_back(sh[d]);
        }
      }
    }
  }
  leaf_block_begin[leaves_.size()] = (int)jb_.first.size();
  // Cell block ranges: the leaves under a cell are consecutive.
  for (size_t c = cells_.size(); c-- > 0;) {
    const Cell& cc = cells_[c];
    if (cc.count == 0) continue;
    if (!cc.split) {
      jb_.cell_begin[c] = leaf_block_begin[cc.leaf];
      jb_.cell_end[c] = leaf_block_begin[cc.leaf + 1];
    } else {
      int b = 0x7fffffff, e = -1;
      for (int k = 0; k < 8; k++) {
        const int p = cc.progeny[k];
        if (p < 0) continue;
        b = std::min(b, jb_.cell_begin[p]);
        e = std::max(e, jb_.cell_end[p]);
      }
      jb_.cell_begin[c] = b;
      jb_.cell_end[c] = e;
    }
  }
}

// Splitting reorders particles; leaves need the final-order h to compute
// their h_max and depth_h.  Split first (positions only), then walk the
// finished subtree to fill per-particle and per-cell h data bottom-up.
void Space::split_tree_then_gather(int top) {
  // Pass 1: geometry and order only.
  split_geometry(top);
  // Pass 2: bottom-up h data.
  finalize_h(top);
}

void Space::split_geometry(int c) {
  const int count = cells_[c].count;
  for (int k = 0; k < 8; k++) cells_[c].progeny[k] = -1;
  if (count > kSplitSize) {
    if (cells_[c].depth >= SPH_MAX_DEPTH - 1)
      throw std::runtime_error("cell tree deeper than supported (particles at identical positions?)");
    cells_[c].split = 1;
    const double pivot[3] = {cells_[c].loc[0] + cells_[c].width[0] / 2,
                             cells_[c].loc[1] + cells_[c].width[1] / 2,
                             cells_[c].loc[2] + cells_[c].width[2] / 2};
    int counts[8];
    octant_permute(cells_[c].first, count, pivot, counts);
    int off = cells_[c].first;
    for (int k = 0; k < 8; k++) {
      if (counts[k] == 0) continue;
      Cell p;
      const Cell pc = cells_[c];
      for (int d = 0; d < 3; d++) {
        p.loc[d] = pc.loc[d];
        p.width[d] = pc.width[d] / 2;
      }
      p.dmin = pc.dmin / 2;
      p.h_min_allowed = p.dmin * 0.5 * (1. / SPH_KG);
      p.h_max_allowed = p.dmin * (1. / SPH_KG);
      if (k & 4) p.loc[0] += p.width[0];
      if (k & 2) p.loc[1] += p.width[1];
      if (k & 1) p.loc[2] += p.width[2];
      p.depth = pc.depth + 1;
      p.parent = c;
      p.top = pc.top;
      p.count = counts[k];
      p.first = off;
      off += counts[k];
      const int pid = (int)cells_.size();
      cells_.push_back(p);
      cells_[c].progeny[k] = pid;
      split_geometry(pid);
    }
  } else {
    cells_[c].split = 0;
  }
}

// The cells below the top level from tree records (first, count, depth,
// parent, top) numbered as split_geometry numbers them (parents first, each
// top cell's subtree in preorder): every child's octant is that of its
// first particle about the parent's centre, and its geometry follows from
// the parent's exactly as split_geometry derives it.
void Space::adopt_tree(const int32_t* tree, int ncells) {
  const int ntop = (int)cells_.size();
  for (int c = ntop; c < ncells; c++) {
    const int32_t* r = tree + 5 * (size_t)c;
    const int pc = r[3];
    if (pc < 0 || pc >= c) throw std::runtime_error("assigned tree: parent after child");
    const Cell& par = cells_[pc];
    if (r[1] <= 0 || r[0] < par.first || r[0] + r[1] > par.first + par.count ||
        r[2] != par.depth + 1 || par.count <= kSplitSize)
      throw std::runtime_error("assigned tree: child outside its parent");
    const double pivot[3] = {par.loc[0] + par.width[0] / 2, par.loc[1] + par.width[1] / 2,
                             par.loc[2] + par.width[2] / 2};
    auto octant = [&](int q) {
      const double* x = &x_[3 * (size_t)perm_[q]];
      return (x[0] >= pivot[0]) * 4 + (x[1] >= pivot[1]) * 2 + (x[2] >= pivot[2]);
    };
    const int k = octant(r[0]);
    // every particle of the child lies in the child's octant of the parent
    for (int q = r[0] + 1; q < r[0] + r[1]; q++)
      if (octant(q) != k) throw std::runtime_error("assigned tree: a particle outside its octant");
    Cell p;
    for (int d = 0; d < 3; d++) {
      p.loc[d] = par.loc[d];
      p.width[d] = par.width[d] / 2;
    }
    p.dmin = par.dmin / 2;
    p.h_min_allowed = p.dmin * 0.5 * (1. / SPH_KG);
    p.h_max_allowed = p.dmin * (1. / SPH_KG);
    if (k & 4) p.loc[0] += p.width[0];
    if (k & 2) p.loc[1] += p.width[1];
    if (k & 1) p.loc[2] += p.width[2];
    p.depth = par.depth + 1;
    p.parent = pc;
    p.top = par.top;
    p.count = r[1];
    p.first = r[0];
    if (cells_[pc].progeny[k] >= 0) throw std::runtime_error("assigned tree: octant taken twice");
    cells_.push_back(p);
    cells_[pc].progeny[k] = c;
    cells_[pc].split = 1;
  }
  for (const Cell& c : cells_) {
    if (c.count > kSplitSize && !c.split)
      throw std::runtime_error("assigned tree: a cell of more than 400 particles is not split");
    if (!c.split) continue;
    // the children tile the parent: in octant order their ranges follow one
    // another from the parent's first particle to its last (the split's
    // bucket order), with no gap and no overlap
    int next = c.first;
    for (int k = 0; k < 8; k++) {
      const int p = c.progeny[k];
      if (p < 0) continue;
      if (cells_[p].first != next)
        throw std::runtime_error("assigned tree: children do not tile their parent");
      next += cells_[p].count;
    }
    if (next != c.first + c.count)
      throw std::runtime_error("assigned tree: children do not tile their parent");
  }
}

void Space::finalize_h(int c) {
  Cell& cc = cells_[c];
  if (cc.split) {
    float h_max = 0.f, h_max_active = 0.f;
    int any_active = 0;
    for (int k = 0; k < 8; k++) {
      const int p = cells_[c].progeny[k];
      if (p < 0) continue;
      finalize_h(p);
      h_max = fmaxr(h_max, cells_[p].h_max);
      h_max_active = fmaxr(h_max_active, cells_[p].h_max_active);
      any_active |= cells_[p].active;
    }
    cells_[c].h_max = h_max;
    cells_[c].h_max_active = h_max_active;
    cells_[c].active = any_active;
  } else {
    float h_max = 0.f, h_max_active = 0.f;
    int any_active = 0;
    const int first = cc.first, count = cc.count;
    const int leaf_id = (int)leaves_.size();
    for (int k = first; k < first + count; k++) {
      h_[k] = h_in_[perm_[k]];
      active_[k] = tb_in_[perm_[k]] <= prm_.max_active_bin;
      h_max = fmaxr(h_max, h_[k]);
      if (active_[k]) {
        h_max_active = fmaxr(h_max_active, h_[k]);
        any_active = 1;
      }
      set_h_depth(k, c);
      leaf_of_[k] = leaf_id;
    }
    cells_[c].h_max = h_max;
    cells_[c].h_max_active = h_max_active;
    cells_[c].active = any_active;
    cells_[c].leaf = leaf_id;
    leaves_.push_back(c);
  }
  cells_[c].h_max_old = cells_[c].h_max;
}

void Space::build_top_pairs() {
  tasks_.clear();
  const int* cdim = cdim_;
  for (int i = 0; i < cdim[0]; i++)
    for (int j = 0; j < cdim[1]; j++)
      for (int k = 0; k < cdim[2]; k++) {
        const int cid = k + cdim[2] * (j + cdim[1] * i);
        if (cells_[cid].count == 0) continue;
        tasks_.push_back({cid, -1});
        for (int di = -1; di <= 1; di++)
          for (int dj = -1; dj <= 1; dj++)
            for (int dk = -1; dk <= 1; dk++) {
              int ii = i + di, jj = j + dj, kk = k + dk;
              if (prm_.periodic) {
                ii = (ii + cdim[0]) % cdim[0];
                jj = (jj + cdim[1]) % cdim[1];
                kk = (kk + cdim[2]) % cdim[2];
              } else if (ii < 0 || ii >= cdim[0] || jj < 0 || jj >= cdim[1] ||
                         kk < 0 || kk >= cdim[2]) {
                continue;
              }
              const int cjd = kk + cdim[2] * (jj + cdim[1] * ii);
              if (cjd <= cid || cells_[cjd].count == 0) continue;
              tasks_.push_back({cid, cjd});
            }
      }
  top_links_.assign((size_t)cdim[0] * cdim[1] * cdim[2], {});
  for (int t = 0; t < (int)tasks_.size(); t++) {
    top_links_[tasks_[t].ci].push_back(t);
    if (tasks_[t].cj >= 0) top_links_[tasks_[t].cj].push_back(t);
  }
}

// Only particles whose h or activity can have changed since the last call
// -- the previous step's active particles and this step's -- are visited;
// their leaves are recomputed from their particles and every ancestor from
// its progeny, which gives the same cells as recomputing the whole tree.
void Space::set_activity(int max_active_bin) {
  prm_.max_active_bin = max_active_bin;
  std::vector<int> dirty;
  auto mark_leaf = [&](int k) {
    const int c = leaves_[leaf_of_[k]];
    if (!cell_mark_[c]) {
      cell_mark_[c] = 1;
      dirty.push_back(c);
    }
  };
  for (int k : active_list_) {
    active_[k] = 0;
    mark_leaf(k);
  }
  active_list_.clear();
  for (int b = 0; b < 256; b++) {
    if (b - 128 > max_active_bin) break;
    for (int k : bin_members_[b]) {
      active_[k] = 1;
      h_[k] = h_in_[perm_[k]];
      active_list_.push_back(k);
      mark_leaf(k);
    }
  }
  constexpr int kLeafBlock = 64;  // dirty leaves per work block
  parallel_blocks(threads(), (int)((dirty.size() + kLeafBlock - 1) / kLeafBlock), [&](int blk) {
    const size_t e = std::min(dirty.size(), (size_t)(blk + 1) * kLeafBlock);
    for (size_t q = (size_t)blk * kLeafBlock; q < e; q++) redrift_leaf(dirty[q]);
  });
  // ancestors, deepest first, each once
  std::vector<std::vector<int>> by_depth;
  std::vector<int> anc;
  for (int c : dirty)
    for (int p = cells_[c].parent; p >= 0 && !cell_mark_[p]; p = cells_[p].parent) {
      cell_mark_[p] = 1;
      const int d = cells_[p].depth;
      if ((int)by_depth.size() <= d) by_depth.resize(d + 1);
      by_depth[d].push_back(p);
    }
  for (int d = (int)by_depth.size() - 1; d >= 0; d--) {
    const std::vector<int>& lev = by_depth[d];
    parallel_blocks(threads(), (int)((lev.size() + kLeafBlock - 1) / kLeafBlock), [&](int blk) {
      const size_t e = std::min(lev.size(), (size_t)(blk + 1) * kLeafBlock);
      for (size_t q = (size_t)blk * kLeafBlock; q < e; q++) {
        const int c = lev[q];
        float h_max = 0.f, h_max_active = 0.f;
        int any = 0;
        for (int k = 0; k < 8; k++) {
          const int p = cells_[c].progeny[k];
          if (p < 0) continue;
          h_max = fmaxr(h_max, cells_[p].h_max);
          h_max_active = fmaxr(h_max_active, cells_[p].h_max_active);
          any |= cells_[p].active;
        }
        cells_[c].h_max = h_max;
        cells_[c].h_max_active = h_max_active;
        cells_[c].active = any;
        cells_[c].h_max_old = h_max;
      }
    });
    anc.insert(anc.end(), lev.begin(), lev.end());
  }
  for (int c : dirty) cell_mark_[c] = 0;
  for (int c : anc) cell_mark_[c] = 0;
}

void Space::redrift_leaf(int c) {
  float h_max = 0.f, h_max_active = 0.f;
  int any = 0;
  const Cell& cc = cells_[c];
  for (int k = cc.first; k < cc.first + cc.count; k++) {
    set_h_depth(k, c);
    h_max = fmaxr(h_max, h_[k]);
    if (active_[k]) {
      h_max_active = fmaxr(h_max_active, h_[k]);
      any = 1;
    }
  }
  cells_[c].h_max = h_max;
  cells_[c].h_max_active = h_max_active;
  cells_[c].active = any;
  cells_[c].h_max_old = h_max;
}

void Space::update_h_active(const float* h_active) {
  // runner_ghost.c:1617-1632: a cell's h_max only grows (atomic max with the
  // pre-ghost value); only the active particles' h changed.
  if (h_conv_.size() != (size_t)n_) h_conv_ = h_;
  for (size_t a = 0; a < active_list_.size(); a++) {
    const int k = active_list_[a];
    const float h = h_active[a];
    h_[k] = h;
    h_conv_[k] = h;
    for (int c = leaves_[leaf_of_[k]]; c >= 0; c = cells_[c].parent) {
      if (cells_[c].h_max >= h && cells_[c].h_max_active >= h) break;
      cells_[c].h_max = fmaxr(cells_[c].h_max, h);
      cells_[c].h_max_active = fmaxr(cells_[c].h_max_active, h);
    }
  }
}

void Space::assign_h(const float* h_sorted) {
  for (int k = 0; k < n_; k++) h_[k] = h_sorted[k];
}

void Space::set_dx_max(const float* per_cell) {
  for (size_t c = 0; c < cells_.size(); c++) cells_[c].dx_max = per_cell ? per_cell[c] : 0.f;
}

void Space::set_input_h(const float* h_input_order) {
  for (int k = 0; k < n_; k++) h_in_[k] = h_input_order[k];
}

void Space::set_bins(const int8_t* time_bin_input_order) {
  tb_in_.assign(time_bin_input_order, time_bin_input_order + n_);
  bin_members_.assign(256, {});
  for (int k = 0; k < n_; k++) bin_members_[tb_in_[perm_[k]] + 128].push_back(k);
}

void Space::refresh_all() {
  const int ntop = cdim_[0] * cdim_[1] * cdim_[2];
  constexpr int kTopBlock = 8;  // top cells per work block
  parallel_blocks(threads(), (ntop + kTopBlock - 1) / kTopBlock, [&](int blk) {
    for (int c = blk * kTopBlock; c < std::min(ntop, (blk + 1) * kTopBlock); c++) redrift(c);
  });
}

void Space::redrift(int c) {
  Cell& cc = cells_[c];
  float h_max = 0.f, h_max_active = 0.f;
  int any = 0;
  if (cc.split) {
    for (int k = 0; k < 8; k++) {
      const int p = cells_[c].progeny[k];
      if (p < 0) continue;
      redrift(p);
      h_max = fmaxr(h_max, cells_[p].h_max);
      h_max_active = fmaxr(h_max_active, cells_[p].h_max_active);
      any |= cells_[p].active;
    }
  } else {
    for (int k = cc.first; k < cc.first + cc.count; k++) {
      set_h_depth(k, c);
      h_max = fmaxr(h_max, h_[k]);
      if (active_[k]) {
        h_max_active = fmaxr(h_max_active, h_[k]);
        any = 1;
      }
    }
  }
  cells_[c].h_max = h_max;
  cells_[c].h_max_active = h_max_active;
  cells_[c].active = any;
  cells_[c].h_max_old = h_max;
}

// ---------------------------------------------------------------------------
// Recursions -> evaluation items

void Space::emit_pair(std::vector<Item>& out, int ci, int cj,
                      const double shift[3], int lmin, int lmax) const {
  Item it;
  it.kind = FRAME_PAIR_CELLREL;
  it.a = ci;
  it.b = cj;
  for (int k = 0; k < 3; k++) it.shift[k] = shift[k];
  it.min_depth = lmax ? cells_[ci].depth : 0;
  it.max_depth = lmin ? cells_[ci].depth : 127;
  out.push_back(it);
}

void Space::emit_self(std::vector<Item>& out, int c, int lmin, int lmax) const {
  Item it;
  it.kind = FRAME_SELF_DBL;
  it.a = c;
  it.b = -1;
  it.shift[0] = it.shift[1] = it.shift[2] = 0.0;
  it.min_depth = lmax ? cells_[c].depth : 0;
  it.max_depth = lmin ? cells_[c].depth : 127;
  out.push_back(it);
}

void Space::pair_branch(std::vector<Item>& out, int ci, int cj, int lmin,
                        int lmax) const {
  if (cells_[ci].count == 0 || cells_[cj].count == 0) return;
  if (!cells_[ci].active && !cells_[cj].active) return;
  double shift[3] = {0.0, 0.0, 0.0};
  getsid_and_swap(ci, cj, shift);
  emit_pair(out, ci, cj, shift, lmin, lmax);
}

void Space::self_branch(std::vector<Item>& out, int c, int lmin,
                        int lmax) const {
  if (cells_[c].count == 0 || !cells_[c].active) return;
  emit_self(out, c, lmin, lmax);
}

// DOSUB_PAIR1 / DOSUB_PAIR2: `second` selects the force-loop predicates.
void Space::dosub_pair(std::vector<Item>& out, int ci, int cj, int below,
                       bool second) const {
  if (!cells_[ci].active && !cells_[cj].active) return;
  if (cells_[ci].count == 0 || cells_[cj].count == 0) return;
  double shift[3];
  const int sid = getsid_and_swap(ci, cj, shift);
  const Cell &a = cells_[ci], &b = cells_[cj];
  if (!a.split || a.count < kRecurseSize || !b.split || b.count < kRecurseSize) {
    pair_branch(out, ci, cj, 0, below);
  } else {
    if (!below) {
      const bool ok = second ? (can_recurse_pair2(a) && can_recurse_pair2(b))
                             : (can_recurse_pair1(a) && can_recurse_pair1(b));
      if (!ok) below = 1;
    }
    if (below) pair_branch(out, ci, cj, 1, 1);
    for (const auto& pq : cpairs_[sid]) {
      const int p = cells_[ci].progeny[pq.first], q = cells_[cj].progeny[pq.second];
      if (p >= 0 && q >= 0) dosub_pair(out, p, q, below, second);
    }
  }
}

void Space::dosub_self(std::vector<Item>& out, int c, int below,
                       bool second) const {
  if (cells_[c].count == 0 || !cells_[c].active) return;
  const Cell& cc = cells_[c];
  if (!cc.split || cc.count < kRecurseSize) {
    self_branch(out, c, 0, below);
  } else {
    if (!below) {
      const bool ok = second ? can_recurse_self2(cc) : can_recurse_self1(cc);
      if (!ok) below = 1;
    }
    if (below) self_branch(out, c, 1, 1);
    for (int k = 0; k < 8; k++) {
      const int p = cells_[c].progeny[k];
      if (p < 0) continue;
      dosub_self(out, p, below, second);
      for (int j = k + 1; j < 8; j++) {
        const int q = cells_[c].progeny[j];
        if (q >= 0) dosub_pair(out, p, q, below, second);
      }
    }
  }
}

// Subset recursion of the ghost's re-runs for the particles of one leaf.
void Space::subset_pair(std::vector<Item>& out, int ci, int leaf_cell,
                        int cj) const {
  if (cells_[ci].count == 0 || cells_[cj].count == 0) return;
  if (!cells_[ci].active) return;
  if (can_recurse_pair_old(cells_[ci]) && can_recurse_pair_old(cells_[cj])) {
    const int sub = find_sub(ci, leaf_cell);
    double shift[3];
    int a = ci, b = cj;
    const int sid = getsid_and_swap(a, b, shift);
    for (const auto& pq : cpairs_[sid]) {
      const int p = cells_[a].progeny[pq.first], q = cells_[b].progeny[pq.second];
      if (p == sub && q >= 0) subset_pair(out, p, leaf_cell, q);
      if (p >= 0 && q == sub) subset_pair(out, q, leaf_cell, p);
    }
  } else if (cells_[ci].active) {
    if (cells_[cj].count == 0) return;
    double shift[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < 3; k++) {
      if (cells_[cj].loc[k] - cells_[ci].loc[k] < -prm_.dim[k] / 2)
        shift[k] = prm_.dim[k];
      else if (cells_[cj].loc[k] - cells_[ci].loc[k] > prm_.dim[k] / 2)
        shift[k] = -prm_.dim[k];
    }
    Item it;
    it.kind = FRAME_PAIR_ABS;
    it.a = ci;
    it.b = cj;
    for (int k = 0; k < 3; k++) it.shift[k] = shift[k];
    it.min_depth = 0;
    it.max_depth = 127;
    out.push_back(it);
  }
}

void Space::subset_self(std::vector<Item>& out, int ci, int leaf_cell) const {
  if (cells_[ci].count == 0 || !cells_[ci].active) return;
  if (cells_[ci].split && can_recurse_self_old(cells_[ci])) {
    const int sub = find_sub(ci, leaf_cell);
    subset_self(out, sub, leaf_cell);
    for (int j = 0; j < 8; j++) {
      const int q = cells_[ci].progeny[j];
      if (q != sub && q >= 0) subset_pair(out, sub, leaf_cell, q);
    }
  } else {
    Item it;
    it.kind = FRAME_SELF_CELLREL;
    it.a = ci;
    it.b = -1;
    it.shift[0] = it.shift[1] = it.shift[2] = 0.0;
    it.min_depth = 0;
    it.max_depth = 127;
    out.push_back(it);
  }
}

int Space::find_sub(int c, int leaf_cell) const {
  const int first = cells_[leaf_cell].first;
  for (int k = 0; k < 8; k++) {
    const int p = cells_[c].progeny[k];
    if (p >= 0 && first >= cells_[p].first && first < cells_[p].first + cells_[p].count)
      return p;
  }
  throw std::runtime_error("subset recursion: sub-cell not found");
}

// ---------------------------------------------------------------------------
// Items -> per-leaf gather entries

static inline bool is_ancestor_or_self(const std::vector<Cell>& cells, int anc,
                                       int c) {
  const Cell& a = cells[anc];
  const Cell& x = cells[c];
  return x.first >= a.first && x.first + x.count <= a.first + a.count &&
         x.depth >= a.depth;
}

Entry Space::make_entry(int leaf_cell, int partner, int kind, bool u_is_ci,
                        const double shift[3], int frame_cell, int min_depth,
                        int max_depth) const {
  Entry e;
  std::memset(&e, 0, sizeof(e));
  e.first = cells_[partner].first;
  e.count = cells_[partner].count;
  e.bfirst = jb_.cell_begin[partner];
  e.bcount = jb_.cell_end[partner] - jb_.cell_begin[partner];
  e.kind = (int8_t)kind;
  e.min_depth = (int8_t)min_depth;
  e.max_depth = (int8_t)max_depth;
  // Effective periodic shift of the partner seen from the updated particle.
  double seff[3] = {0.0, 0.0, 0.0};
  if (kind == FRAME_PAIR_CELLREL) {
    // frame_cell is cj (after the swap); ci particles use cj.loc + shift.
    const Cell& fc = cells_[frame_cell];
    for (int k = 0; k < 3; k++) {
      const double oi = fc.loc[k] + shift[k];
      const double oj = fc.loc[k];
      e.ou[k] = u_is_ci ? oi : oj;
      e.op[k] = u_is_ci ? oj : oi;
      seff[k] = u_is_ci ? shift[k] : -shift[k];
    }
  } else if (kind == FRAME_PAIR_ABS) {
    for (int k = 0; k < 3; k++) {
      e.ou[k] = shift[k];
      e.op[k] = 0.0;
      seff[k] = shift[k];
    }
  } else if (kind == FRAME_SELF_CELLREL) {
    for (int k = 0; k < 3; k++) e.ou[k] = e.op[k] = cells_[frame_cell].loc[k];
  }
  const Cell& tl = cells_[cells_[leaf_cell].top];
  const Cell& tp = cells_[cells_[partner].top];
  e.fdx = (float)(tp.loc[0] + seff[0] - tl.loc[0]);
  e.fdy = (float)(tp.loc[1] + seff[1] - tl.loc[1]);
  e.fdz = (float)(tp.loc[2] + seff[2] - tl.loc[2]);
  return e;
}

void Space::leaves_under(int c, std::vector<int>& out) const {
  if (!cells_[c].split) {
    out.push_back(c);
    return;
  }
  for (int k = 0; k < 8; k++)
    if (cells_[c].progeny[k] >= 0) leaves_under(cells_[c].progeny[k], out);
}

void Space::items_to_entries(const std::vector<Item>& items,
                             std::vector<std::vector<Entry>>& per_leaf) const {
  std::vector<std::pair<int, Entry>> out;
  items_to_entry_list(items, out);
  for (auto& le : out) per_leaf[le.first].push_back(le.second);
}

// Entries of a list of items, as (leaf id, entry) in emission order; leaves
// without an active particle get none (nothing of theirs is updated).
void Space::items_to_entry_list(const std::vector<Item>& items,
                                std::vector<std::pair<int, Entry>>& out) const {
  std::vector<int> lv;
  for (const Item& it : items) {
    const int side = it.b < 0 ? it.a : it.b;
    lv.clear();
    leaves_under(it.a, lv);
    for (int L : lv)
      if (cells_[L].active)
        out.emplace_back(cells_[L].leaf, make_entry(L, side, it.kind, true, it.shift,
                                                    side, it.min_depth, it.max_depth));
    if (it.b >= 0 && it.kind == FRAME_PAIR_CELLREL) {
      lv.clear();
      leaves_under(it.b, lv);
      for (int L : lv)
        if (cells_[L].active)
          out.emplace_back(cells_[L].leaf, make_entry(L, it.a, it.kind, false, it.shift,
                                                      it.b, it.min_depth, it.max_depth));
    }
  }
}

int Space::threads() const { return threads_ > 0 ? threads_ : planner_threads(); }

void Space::plan_density(Plan& plan, bool second) const {
  constexpr int kBlock = 32;  // top-level tasks per work block
  const int nt = (int)tasks_.size();
  const int nb = (nt + kBlock - 1) / kBlock;
  std::vector<std::vector<std::pair<int, Entry>>> outs(nb);
  parallel_blocks(threads(), nb, [&](int blk) {
    std::vector<Item> items;
    for (int t = blk * kBlock; t < std::min(nt, (blk + 1) * kBlock); t++) {
      const TopTask& tk = tasks_[t];
      if (!cells_[tk.ci].active && (tk.cj < 0 || !cells_[tk.cj].active)) continue;
      items.clear();
      if (tk.cj < 0)
        dosub_self(items, tk.ci, 0, second);
      else
        dosub_pair(items, tk.ci, tk.cj, 0, second);
      items_to_entry_list(items, outs[blk]);
    }
  });
  flatten(outs, plan);
}

void Space::plan_subset(Plan& plan) const {
  // The ghost re-runs density for the unconverged particles of one leaf
  // through the density tasks linked to the leaf's ancestors
  // (runner_ghost.c:1548-1579); here all tasks hang on top cells.
  std::vector<int> act;
  for (size_t l = 0; l < leaves_.size(); l++)
    if (cells_[leaves_[l]].active) act.push_back((int)l);
  constexpr int kBlock = 16;  // leaves per work block
  const int na = (int)act.size();
  const int nb = (na + kBlock - 1) / kBlock;
  std::vector<std::vector<std::pair<int, Entry>>> outs(nb);
  parallel_blocks(threads(), nb, [&](int blk) {
    std::vector<Item> items;
    for (int a = blk * kBlock; a < std::min(na, (blk + 1) * kBlock); a++) {
      const int l = act[a];
      const int L = leaves_[l];
      items.clear();
      for (int finger = L; finger >= 0; finger = cells_[finger].parent) {
        if (cells_[finger].parent >= 0) continue;  // tasks hang on top cells
        for (int ti : top_links_[finger]) {
          const TopTask& t = tasks_[ti];
          if (t.cj < 0)
            subset_self(items, finger, L);
          else
            subset_pair(items, finger, L, t.ci == finger ? t.cj : t.ci);
        }
      }
      for (const Item& it : items) {
        // Subset items are always oriented with the leaf's side first.
        const int side = it.kind == FRAME_SELF_CELLREL ? it.a : it.b;
        outs[blk].emplace_back(l, make_entry(L, side, it.kind, true, it.shift, side, 0, 127));
      }
    }
  });
  flatten(outs, plan);
}

// Plan arrays from (leaf, entry) lists in emission order: the entries stay
// in that order; every leaf's (j-block, entry) candidate pairs are grouped by
// leaf, in the order its entries were emitted.
void Space::flatten(const std::vector<std::vector<std::pair<int, Entry>>>& outs,
                    Plan& plan) const {
  const size_t nl = leaves_.size();
  size_t ne = 0;
  for (const auto& o : outs) ne += o.size();
  plan.entries.resize(ne);
  std::vector<int> leaf(ne);
  auto& lpb = plan.leaf_pair_begin;
  lpb.assign(nl + 1, 0);
  size_t e = 0;
  for (const auto& o : outs)
    for (const auto& le : o) {
      plan.entries[e] = le.second;
      leaf[e] = le.first;
      lpb[le.first + 1] += le.second.bcount;
      e++;
    }
  for (size_t l = 0; l < nl; l++) lpb[l + 1] += lpb[l];
  plan.pair_block.resize(lpb[nl]);
  plan.pair_entry.resize(lpb[nl]);
  std::vector<int> pos(lpb.begin(), lpb.end() - 1);
  for (size_t k = 0; k < ne; k++) {
    const Entry& E = plan.entries[k];
    int w = pos[leaf[k]];
    for (int b = E.bfirst; b < E.bfirst + E.bcount; b++, w++) {
      plan.pair_block[w] = b;
      plan.pair_entry[w] = (int)k;
    }
    pos[leaf[k]] = w;
  }
}

void Space::leaf_infos(std::vector<LeafInfo>& out) const {
  out.resize(leaves_.size());
  for (size_t l = 0; l < leaves_.size(); l++) {
    LeafInfo& li = out[l];
    std::memset(&li, 0, sizeof(li));
    const int L = leaves_[l];
    li.first = cells_[L].first;
    li.count = cells_[L].count;
    li.top = cells_[L].top;
    int n = 0;
    for (int c = L; c >= 0 && n < SPH_MAX_DEPTH; c = cells_[c].parent, n++) {
      li.hmin[n] = cells_[c].h_min_allowed;
      li.hmax[n] = cells_[c].h_max_allowed;
      li.depth[n] = (int8_t)cells_[c].depth;
    }
    li.nlevels = n;
  }
}

void Space::force_decisions(std::vector<uint8_t>& pred) const {
  pred.resize(force_checks_.size());
  for (size_t q = 0; q < force_checks_.size(); q++) {
    const Cell& c = cells_[force_checks_[q].cell];
    pred[q] = can_recurse_pair2(c) ? 1 : 0;
  }
}

void Space::plan_force_predicted(Plan& plan, std::vector<uint8_t>& pred) {
  if (h_conv_.size() != (size_t)n_) h_conv_ = h_;
  // the cells' h_max as update_h_active would leave it, with each active
  // particle at its last converged h
  std::vector<float> saved(cells_.size());
  for (size_t c = 0; c < cells_.size(); c++) saved[c] = cells_[c].h_max;
  for (int k : active_list_) {
    const float h = h_conv_[k];
    for (int c = leaves_[leaf_of_[k]]; c >= 0; c = cells_[c].parent) {
      if (cells_[c].h_max >= h) break;
      cells_[c].h_max = h;
    }
  }
  force_decisions(pred);
  try {
    plan_density(plan, true);
  } catch (...) {
    for (size_t c = 0; c < cells_.size(); c++) cells_[c].h_max = saved[c];
    throw;
  }
  for (size_t c = 0; c < cells_.size(); c++) cells_[c].h_max = saved[c];
}

void Space::update_h_after_ghost(const float* h_sorted) {
  // runner_ghost.c:1617-1632: cell h_max only grows (atomic max with the
  // pre-ghost value), bottom-up over the tree.
  for (int k = 0; k < n_; k++) h_[k] = h_sorted[k];
  const int ntop = cdim_[0] * cdim_[1] * cdim_[2];
  for (int c = 0; c < ntop; c++)
    if (cells_[c].count > 0) refresh_hmax(c);
}

void Space::refresh_hmax(int c) {
  float hm = cells_[c].h_max, hma = cells_[c].h_max_active;
  if (cells_[c].split) {
    for (int k = 0; k < 8; k++) {
      const int p = cells_[c].progeny[k];
      if (p < 0) continue;
      refresh_hmax(p);
      hm = fmaxr(hm, cells_[p].h_max);
      hma = fmaxr(hma, cells_[p].h_max_active);
    }
  } else {
    for (int k = cells_[c].first; k < cells_[c].first + cells_[c].count; k++) {
      hm = fmaxr(hm, h_[k]);
      if (active_[k]) hma = fmaxr(hma, h_[k]);
    }
  }
  cells_[c].h_max = hm;
  cells_[c].h_max_active = hma;
}

}  // namespace sphgpu
