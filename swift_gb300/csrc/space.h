// space.h -- host planner: reference space build and recursion -> gather
// lists (see space.cpp for the reference citations).
#pragma once
#include <stdint.h>

#include <utility>
#include <vector>

#include "sph_types.h"

namespace sphgpu {

struct Params {
  double dim[3] = {1.0, 1.0, 1.0};
  int periodic = 1;
  float eta = 1.2348f;
  float h_tolerance = 1e-4f;
  float h_max = 3.40282347e+38f;
  float h_min = 0.f;
  float alpha = 0.8f;
  int max_iter = 30;
  int max_active_bin = 56;
  int max_top_level_cells = 12;
};

struct Cell {
  double loc[3] = {0, 0, 0}, width[3] = {0, 0, 0};
  float dmin = 0, h_min_allowed = 0, h_max_allowed = 0;
  float h_max = 0, h_max_active = 0, h_max_old = 0;
  // largest motion of the cell's particles since the rebuild
  // (hydro.dx_max_part, cell_drift.c:330-382); 0 until the space drifts
  float dx_max = 0;
  int count = 0, first = 0, depth = 0, split = 0, active = 0;
  int parent = -1, top = -1, leaf = -1;
  int progeny[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
};

struct TopTask {
  int ci, cj;  // cj < 0: self task
};

struct Item {
  int kind;
  int a, b;  // a = ci after the swap (or the self cell), b = cj or -1
  double shift[3];
  int min_depth, max_depth;
};

struct Plan {
  std::vector<Entry> entries;  // in the order the recursions emit them
  // Flattened candidate list: every (j-block, entry) a leaf's particles may
  // interact with, grouped by leaf.
  std::vector<int32_t> pair_block, pair_entry;
  std::vector<int> leaf_pair_begin;
};

// A cell whose decision the force recursion can read (16 bytes: uploaded as
// one int4 per cell, dmin's bits in the third word).
struct ForceCheck {
  int32_t first, count;
  float dmin;
  int32_t cell;
};

constexpr int kSubBlock = 8;  // particles per sub-box of a j-block (4 per block of 32)

struct JBlocks {
  std::vector<int32_t> first, count;   // particle range (GPU order)
  std::vector<float> lo, hi;           // [3 * nblocks] bounding box, top frame
  // [4 * 3 * nblocks] boxes of the block's runs of 8 particles (kSubBlock);
  // a run past the block's end is empty (lo > hi)
  std::vector<float> sub_lo, sub_hi;
  std::vector<int32_t> cell_begin, cell_end;  // per cell: block range
};

class Space {
 public:
  static constexpr int kSplitSize = 400;     // space.h:49
  static constexpr int kRecurseSize = 100;   // space.h:64-65

  explicit Space(const Params& prm);
  // Top-level grid for particles whose largest h is max_h: cells per side
  // and cell widths (throws where the reference would refuse the box).
  static void top_grid(const Params& prm, float max_h, int cdim[3], double width[3]);
  // order / tree / ncells (optional): the cell assignment made elsewhere
  // (the device's sphgpu_cell_assign: particle order and tree records), used
  // instead of the host's bucket and octant permutations.
  void build(int64_t n, const double* x, const float* h, const int8_t* time_bin,
             const int32_t* order = nullptr, const int32_t* tree = nullptr, int ncells = 0);
  // Start of a step at max_active_bin, with the reference's drift at zero
  // displacement (cell_drift.c:330-371): active particles restart from the
  // caller's h (the input h), every particle takes the depth_h of its h,
  // every cell its h_max / h_max_active from its particles, h_max_old =
  // h_max.  Inactive particles keep the h of their last step (assign_h).
  void set_activity(int max_active_bin);
  // Current smoothing lengths of all particles (reference sorted order).
  void assign_h(const float* h_sorted);
  // Every cell's h_max, h_max_active, activity, h_max_old and its
  // particles' depth_h recomputed from the current h and activity (after
  // assign_h changed the h of particles outside the last activations).
  void refresh_all();
  // After the particles moved without a rebuild: every cell's dx_max (per
  // cell, 0 where null) and the particles' new input h (input order), from
  // which active particles restart.
  void set_dx_max(const float* per_cell);
  void set_input_h(const float* h_input_order);
  // New time bins (input order): the activity of later activations.
  void set_bins(const int8_t* time_bin_input_order);
  // New h of the active particles after a ghost (same order as
  // active_list()); cells grow their h_max as runner_ghost.c:1617-1632 does.
  void update_h_active(const float* h_active);
  // Sorted indices of the active particles, grouped by time bin.
  const std::vector<int>& active_list() const { return active_list_; }
  // depth_h that cell_set_part_h_depth (cell.h:1787) gives h in this leaf.
  int8_t h_depth_of(float h, int leaf_cell) const;
  // j-block depth (partner particles per culled block, <= 32)
  void set_jblock(int jb) {
    jblock_ = jb;
    build_gpu_order();
  }
  int jblock() const { return jblock_; }
  // Host threads the planner uses (0: one per core, at most 16).
  void set_threads(int t) { threads_ = t; }
  int threads() const;

  // Gather lists: first density pass (second=false) or force pass
  // (second=true, call update_h_after_ghost first); ghost re-runs.
  void plan_density(Plan& plan, bool second) const;
  void plan_subset(Plan& plan) const;
  // The force pass's lists planned before the step's ghost, with every
  // active particle at the h it converged to the last time a ghost ran on
  // it (the cells' post-ghost h_max predicted); the force recursion's
  // decision of every checked cell (force_checks) goes to pred[] -- the
  // step verifies them against the real post-ghost h_max on the device.
  void plan_force_predicted(Plan& plan, std::vector<uint8_t>& pred);
  // Decisions of the force recursion (cell.h:966-1010: gamma h_max <
  // dmin / 2) for the checked cells at the cells' current h_max.
  void force_decisions(std::vector<uint8_t>& pred) const;
  // The cells whose decision the force recursion can read: split, with at
  // least kRecurseSize particles (first, count, dmin, cell id).
  const std::vector<ForceCheck>& force_checks() const { return force_checks_; }
  void leaf_infos(std::vector<LeafInfo>& out) const;
  void update_h_after_ghost(const float* h_sorted);

  int n() const { return n_; }
  const int* cdim() const { return cdim_; }
  const double* width() const { return width_; }
  const std::vector<Cell>& cells() const { return cells_; }
  const std::vector<int>& leaves() const { return leaves_; }
  const std::vector<int>& perm() const { return perm_; }          // sorted -> input
  // GPU store order: the reference's cell order with each leaf re-sorted
  // along a Morton curve (cell ranges are unchanged).
  const std::vector<int>& gperm() const { return gperm_; }        // gpu -> input
  const std::vector<int>& gpu_of_sorted() const { return g_of_s_; }
  const JBlocks& jblocks() const { return jb_; }
  const std::vector<int>& inv_perm() const { return inv_perm_; }  // input -> sorted
  const std::vector<int8_t>& depth_h() const { return depth_h_; }
  const std::vector<int>& leaf_of() const { return leaf_of_; }
  const std::vector<uint8_t>& active() const { return active_; }
  const std::vector<double>& x() const { return x_; }  // wrapped, input order
  const std::vector<TopTask>& tasks() const { return tasks_; }
  // per top cell: its tasks, in task order
  const std::vector<std::vector<int>>& top_links() const { return top_links_; }
  const Params& params() const { return prm_; }

  // Recursion entry points (also used for per-task plans of the plain form).
  void dosub_self(std::vector<Item>& out, int c, int below, bool second) const;
  void dosub_pair(std::vector<Item>& out, int ci, int cj, int below, bool second) const;
  void items_to_entries(const std::vector<Item>& items,
                        std::vector<std::vector<Entry>>& per_leaf) const;
  void items_to_entry_list(const std::vector<Item>& items,
                           std::vector<std::pair<int, Entry>>& out) const;
  void flatten(const std::vector<std::vector<std::pair<int, Entry>>>& outs,
               Plan& plan) const;

 private:
  int getsid_and_swap(int& ci, int& cj, double shift[3]) const;
  void bucket_permute(std::vector<int>& bin, int nbins, int first, int n,
                      std::vector<int>& counts_out);
  void octant_permute(int first, int n, const double pivot[3], int counts[8]);
  void set_h_depth(int sorted_idx, int leaf);
  void split_tree_then_gather(int top);
  void split_geometry(int c);
  void finalize_h(int c);
  void adopt_tree(const int32_t* tree, int ncells);
  void build_top_pairs();
  void redrift(int c);
  void redrift_leaf(int c);
  void refresh_hmax(int c);
  void emit_pair(std::vector<Item>& out, int ci, int cj, const double shift[3],
                 int lmin, int lmax) const;
  void emit_self(std::vector<Item>& out, int c, int lmin, int lmax) const;
  void pair_branch(std::vector<Item>& out, int ci, int cj, int lmin, int lmax) const;
  void self_branch(std::vector<Item>& out, int c, int lmin, int lmax) const;
  void subset_pair(std::vector<Item>& out, int ci, int leaf_cell, int cj) const;
  void subset_self(std::vector<Item>& out, int ci, int leaf_cell) const;
  int find_sub(int c, int leaf_cell) const;
  Entry make_entry(int leaf_cell, int partner, int kind, bool u_is_ci,
                   const double shift[3], int frame_cell, int min_depth,
                   int max_depth) const;
  void leaves_under(int c, std::vector<int>& out) const;

  // kernel_gamma * h + dx_max rounded as two operations (no fused
  // multiply-add, whatever the host compiler contracts): the device planner
  // evaluates the same expression with __fmul_rn / __fadd_rn
  static float reach(float h, float dx) {
    volatile float g = SPH_KG * h;
    return g + dx;
  }
  // cell.h:934-1010 (the dx_max terms are the cells' motion since the rebuild)
  static bool can_recurse_pair1(const Cell& c) {
    return reach(c.h_max_active, c.dx_max) < 0.5f * c.dmin;
  }
  static bool can_recurse_self1(const Cell& c) {
    return SPH_KG * c.h_max_active < 0.5f * c.dmin;
  }
  static bool can_recurse_pair2(const Cell& c) {
    return reach(c.h_max, c.dx_max) < 0.5f * c.dmin;
  }
  static bool can_recurse_self2(const Cell& c) {
    return c.split && (SPH_KG * c.h_max < 0.5f * c.dmin);
  }
  static bool can_recurse_pair_old(const Cell& c) {
    return c.split && (reach(c.h_max_old, c.dx_max) < 0.5f * c.dmin);
  }
  static bool can_recurse_self_old(const Cell& c) {
    return c.split && (SPH_KG * c.h_max_old < 0.5f * c.dmin);
  }

  Params prm_;
  int n_ = 0;
  int cdim_[3] = {0, 0, 0};
  double width_[3] = {0, 0, 0};
  int jblock_ = SPH_JBLOCK;
  bool adopted_ = false;  // the cell assignment (and leaf order) came from outside
  int threads_ = 0;
  std::vector<double> x_;
  std::vector<float> h_in_, h_;
  std::vector<float> h_conv_;        // each particle's h after its last ghost
  std::vector<ForceCheck> force_checks_;
  std::vector<int8_t> tb_in_;
  std::vector<uint8_t> active_;
  std::vector<int> active_list_;
  std::vector<std::vector<int>> bin_members_;  // sorted indices per bin + 128
  std::vector<uint8_t> cell_mark_;
  std::vector<int8_t> depth_h_;
  std::vector<int> perm_, inv_perm_, leaf_of_, leaves_;
  std::vector<int> gperm_, g_of_s_;
  JBlocks jb_;
  void build_gpu_order();
  std::vector<Cell> cells_;
  std::vector<TopTask> tasks_;
  std::vector<std::vector<int>> top_links_;  // per top cell: its tasks, in order
  std::vector<std::pair<int, int>> cpairs_[13];
};

}  // namespace sphgpu
