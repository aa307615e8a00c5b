// capi.cu -- the C ABI (include/swift_gb300.h): space lifecycle, the batched
// step (one CUDA graph per step), the plain per-task entry points, host I/O.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <exception>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../../include/swift_gb300.h"
#include "space.h"
#include "capi_util.h"
#include "devplan.cuh"
#include "sort.cuh"
#include "sph_kernels.cuh"

using namespace sphgpu;
using namespace sphgpu::capi;

thread_local std::string sphgpu::capi::g_err;

namespace {

struct DevPlan {
  DBuf<Entry> entries;
  DBuf<int> lpb, pb, pe;  // leaf_pair_begin, pair_block, pair_entry
  // true when a buffer had to grow (its address changed: a captured step
  // graph that reads it is stale)
  bool upload(const Plan& pl, cudaStream_t s) {
    const void* before[4] = {entries.p, lpb.p, pb.p, pe.p};
    entries.upload(pl.entries.data(), pl.entries.size(), s);
    lpb.upload(pl.leaf_pair_begin.data(), pl.leaf_pair_begin.size(), s);
    pb.upload(pl.pair_block.data(), pl.pair_block.size(), s);
    pe.upload(pl.pair_entry.data(), pl.pair_entry.size(), s);
    return before[0] != entries.p || before[1] != lpb.p || before[2] != pb.p ||
           before[3] != pe.p;
  }
};

}  // namespace

struct sphgpu_space {
  Params prm;
  std::unique_ptr<Space> space;
  std::vector<double> x_in;
  std::vector<float> v_in, m_in, h_in, u_in;
  std::vector<int8_t> tb_in;
  DBuf<int8_t> tbin, ngb_bin;  // store order: time bins, neighbours' smallest bin
  // list solver: [0] particles handed to the catch-up rounds, [r + 1] those
  // catch-up round r sends on
  DBuf<int> catchup;
  sphgpu_tuning tune{1, SPH_JBLOCK, 1, 8, 0, 0.f, 0, 0};

  // host plans
  Plan plan_d, plan_s, plan_f;
  bool force_planned = false;
  // the planner's copy of h lags the device's (a ghost ran since it was
  // last read back)
  bool h_stale = false;
  // plain-form per-task plans
  std::vector<Plan> task_d, task_f;  // non-empty once the per-task lists exist
  std::vector<std::pair<int, int>> sub_units_of_top;  // subset units per top cell

  // device
  bool dev = false;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  DevParticles P{};
  DBuf<double> xd;
  DBuf<float4> posh, velm, dens0, dens1, fin0, acc;
  DBuf<float2> fin1, hdt_vsig;
  DBuf<float> u, h0, left, right;
  DBuf<uint8_t> flags;
  DBuf<int8_t> depth_h, depth_h0;
  DBuf<int32_t> leaf_of, ghost_iters, ngb_d, ngb_d_first, ngb_f, perm, top_of;
  DBuf<double> top_loc;
  DBuf<LeafInfo> leaves;
  DevPlan dplan_d, dplan_s, dplan_f;
  DBuf<int> queue, redo;
  DBuf<int> act_g;     // store indices of the active particles (active_list order)
  DBuf<float> act_h;   // their h, gathered for the planner
  int n_act_dev = 0;
  DBuf<float4> bb_lo, bb_hi;
  DBuf<int2> bb_fc;
  int bb_n = 0;
  DBuf<int4> units;              // gather work groups (device-built)
  // neighbour lists of the ghost's re-runs (when they fit in HBM)
  bool lists = false;
  int rows_cap = 0;  // items per row the rows were allocated with
  DBuf<int> nl, nl_cnt, blk_of;
  DBuf<float4> sb_lo, sb_hi;  // sub-boxes of the j-blocks (4 per block)
  DBuf<float> nl_T;
  int max_units = 0;             // 32-particle windows of all leaves
  DBuf<int> leaf_window_begin;   // per leaf: its first window
  std::vector<int> lwb_host;
  // the same for 16- and 8-particle windows (two and four lanes per
  // particle), index tpp / 2 - 0 or 1
  int max_units_n[2] = {0, 0};
  DBuf<int> leaf_window_begin_n[2];
  std::vector<int> lwb_host_n[2];
  std::vector<int> top_leaf;     // per top cell: first leaf (+1 sentinel)
  DBuf<int4> task_units_d, task_units_f;
  DBuf<Entry> task_entries_d, task_entries_f;
  DBuf<int> task_pb_d, task_pe_d, task_pb_f, task_pe_f;
  std::vector<int> task_units_begin_d, task_units_begin_f;
  int n_active = 0;
  std::vector<int> s_of_g;             // store index -> reference sorted index
  // host staging for step_host
  DBuf<double> x_stage, x_ref;  // x_ref: the space's input positions
  DBuf<int> differ;
  DBuf<float> v_stage, m_stage, h_stage, u_stage, out_stage;
  // The batched step is one CUDA graph (density first pass, ghost rounds,
  // the force plan's check, force) in graph[0]; event-record nodes inside it
  // time each loop of every step (graph[1] is unused)
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  double plan_ms = 0;  // host planning inside steps (force re-plans)
  double act_plan_ms = 0, act_upload_ms = 0;  // sphgpu_set_active
  double phase_ms[3] = {0, 0, 0};
  long long phase_steps = 0;
  DBuf<unsigned long long> hit_ctr;
  DBuf<int> err;  // set by a kernel that gave up (a bounded wait ran out)
  // the force recursion's decisions the force lists were planned with, per
  // checked cell, and the flag the step's verification sets
  DBuf<int4> chk;
  DBuf<uint8_t> chk_pred;
  DBuf<int> vflag;
  int nchk = 0;
  // [0] steps run as one graph, [1] of them whose force plan the real h
  // changed (re-planned on the host), [2] that needed ghost rounds beyond the
  // graph's, [3] graph captures
  int64_t step_stats[4] = {0, 0, 0, 0};
  bool count_hits = false;
  // Device planner (devplan.cu).  After a sparse activation of a resident
  // space every step plans its own gather lists inside its graph (density
  // and re-run lists from the activation state, force lists from the
  // post-ghost h_max); the host planner's h, activity and plans then lag the
  // device's until leave_device_mode() brings them level.
  bool dmode = false;
  bool dp_ready = false;      // the tree is on the device for the current j-blocks
  bool dp_usable = true;      // false: the tree is too deep, or the planner failed once
  bool dp_off_by_caller = false;  // sphgpu_set_device_planning(s, 0)
  bool host_refresh = false;  // the next host activation recomputes every cell
  int dp_bin = 0;             // max_active_bin of the device-planned steps
  int max_bin = 0;            // largest time bin of the particles
  DPTree dpt;
  DBuf<DPCell> dp_cell;
  DBuf<int32_t> dp_prog, dp_leaf, dp_lbeg, dp_link;
  DBuf<int2> dp_task;
  DBuf<unsigned> dp_hmax, dp_hact, dp_hforce;
  DBuf<int> dp_active;
  DBuf<int2> dp_lane, dp_off, dp_tiles;
  DBuf<int> dp_status, dp_bin_dev;
  long long dp_cap_e[3] = {0, 0, 0}, dp_cap_p[3] = {0, 0, 0};
  // events around the planning inside a step: [0, 1] the activation plans,
  // [2, 3] the force plan
  cudaEvent_t pev[4] = {nullptr, nullptr, nullptr, nullptr};
  double dp_ms = 0;
  long long dp_steps = 0;
  // Drift without a rebuild (sphgpu_space_drift): the rebuild's positions
  // (input order), per cell the dx_max_part in use and the one proposed, the
  // proposed h_max, the rebuild flag; the host planner's dx_max and input h
  // lag the device's while drift_host_stale
  bool drifted = false;
  bool drift_host_stale = false;
  bool bins_host_stale = false;  // sphgpu_space_set_state gave new time bins
  DBuf<int8_t> tb_stage;
  DBuf<double> x_rb;
  DBuf<unsigned> dp_dx, dp_dxn, dp_hdrift;
  DBuf<int> drift_flag;
  // per-cell sort arrays (sphgpu_hydro_sort)
  DBuf<SortCell> sort_cells;
  DBuf<int> sort_leaf_ids, sort_split_ids, g_of_s_dev;
  DBuf<float> sort_d;
  DBuf<int> sort_i;
  std::vector<int> sc_of_cell;            // cell -> SortCell index (-1: empty)
  std::vector<SortCell> sc_host;
  std::vector<int> split_begin, split_n;  // per depth, into sort_split_ids
  int sort_nleaves = 0, sort_max_depth = 0, sorted_mask = 0;

  // Pipelined host steps (sphgpu_step_host_async): two slots of staging
  // buffers; a slot's inputs go up on `cin`, its results come down on `cout`
  // while the next step computes.
  struct AsyncSlot {
    DBuf<double> x;
    DBuf<float> v, m, h, u, out;
    DBuf<int> dflags;                 // [0] inputs differ, [1] unconverged
    int* hflags = nullptr;            // pinned copy of dflags
    float* fields = nullptr;          // the caller's result buffer
    cudaEvent_t in_done = nullptr, comp_done = nullptr, out_done = nullptr;
    bool busy = false;
  } slot[2];
  cudaStream_t cin = nullptr, cout = nullptr;
  int64_t async_k = 0;
  // A batched step whose graph is launched and whose status words (particles
  // still iterating, the force check's flag, the device plans' status) are on
  // their way to pinned host memory: 0 none, 1 host-planned, 2 device-planned
  // (finish_step reads them and runs what the step still needs).
  int pending = 0;
  int pending_slot = -1;  // the pipelined step's slot, or -1
  int* hw = nullptr;      // [0] left, [1] changed, [2..9] device plan status
  cudaEvent_t hw_ev = nullptr;

  ~sphgpu_space() {
    if (hw_ev) {
      cudaEventSynchronize(hw_ev);
      cudaEventDestroy(hw_ev);
    }
    if (hw) cudaFreeHost(hw);
    for (auto& sl : slot) {
      if (sl.out_done) cudaEventSynchronize(sl.out_done);
      for (cudaEvent_t e : {sl.in_done, sl.comp_done, sl.out_done})
        if (e) cudaEventDestroy(e);
      if (sl.hflags) cudaFreeHost(sl.hflags);
    }
    for (auto& g : graph)
      if (g) cudaGraphExecDestroy(g);
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
    for (auto& e : pev)
      if (e) cudaEventDestroy(e);
    if (cin) cudaStreamDestroy(cin);
    if (cout) cudaStreamDestroy(cout);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

// The first-pass and re-run lists depend only on the tree and the activity:
// they are built side by side (each also spreads over the host cores, but at
// low activity few of their work blocks hold active cells).
void build_plans(sphgpu_space* s) {
  std::exception_ptr err;
  std::thread t([&]() {
    try {
      s->space->plan_subset(s->plan_s);
    } catch (...) {
      err = std::current_exception();
    }
  });
  try {
    s->space->plan_density(s->plan_d, false);
  } catch (...) {
    t.join();
    throw;
  }
  t.join();
  if (err) std::rethrow_exception(err);
}

void upload_activity(sphgpu_space* s, cudaStream_t st);

// Re-run neighbour lists: at most kListCap items per particle (the
// default of sphgpu_tuning::row_cap).
constexpr int kListCap = 160;
int row_cap(const sphgpu_space* s);

// The particle rows of the first density pass (row_cap items each), kept
// only while they fit in a quarter of the free HBM.
void alloc_rows(sphgpu_space* s, cudaStream_t st) {
  const int n = s->space->n();  // (s->P is not filled in yet on the first call)
  s->nl.release();
  s->nl_cnt.release();
  s->nl_T.release();
  s->lists = false;
  size_t fr = 0, tot = 0;
  CK(cudaMemGetInfo(&fr, &tot));
  const size_t bytes = (size_t)n * row_cap(s) * sizeof(int);
  if (bytes <= fr / 4) {
    s->nl.alloc((size_t)n * row_cap(s));
    s->nl_cnt.alloc(n);
    s->nl_T.alloc(n);
    CK(cudaMemsetAsync(s->nl_cnt.p, 0xff, sizeof(int) * n, st));  // -1: no list
    s->lists = true;
  }
  s->rows_cap = row_cap(s);
}
// The first density pass records each particle's candidates within
// sqrt(kListWiden) its search radius (capped by its depth_h cell's width), so
// that the ghost's re-runs -- Newton's first step moves h by less than 10 %
// for almost every particle -- run from the lists.
constexpr float kListWiden = 1.21f;

// j-block boxes and particle ranges of the current j-block depth.
void upload_blocks(sphgpu_space* s, cudaStream_t st) {
  const JBlocks& jb = s->space->jblocks();
  const size_t nb = jb.first.size();
  std::vector<float4> blo(nb), bhi(nb);
  std::vector<int2> bfc(nb);
  for (size_t b = 0; b < nb; b++) {
    blo[b] = make_float4(jb.lo[3 * b], jb.lo[3 * b + 1], jb.lo[3 * b + 2], 0.f);
    bhi[b] = make_float4(jb.hi[3 * b], jb.hi[3 * b + 1], jb.hi[3 * b + 2], 0.f);
    bfc[b] = make_int2(jb.first[b], jb.count[b]);
  }
  s->bb_lo.upload(blo.data(), nb, st);
  s->bb_hi.upload(bhi.data(), nb, st);
  s->bb_fc.upload(bfc.data(), nb, st);
  std::vector<float4> slo(4 * nb), shi(4 * nb);
  for (size_t q = 0; q < 4 * nb; q++) {
    slo[q] = make_float4(jb.sub_lo[3 * q], jb.sub_lo[3 * q + 1], jb.sub_lo[3 * q + 2], 0.f);
    shi[q] = make_float4(jb.sub_hi[3 * q], jb.sub_hi[3 * q + 1], jb.sub_hi[3 * q + 2], 0.f);
  }
  s->sb_lo.upload(slo.data(), 4 * nb, st);
  s->sb_hi.upload(shi.data(), 4 * nb, st);
  s->bb_n = (int)nb;
  std::vector<int> bo(s->space->n());
  for (size_t b = 0; b < nb; b++)
    for (int k = jb.first[b]; k < jb.first[b] + jb.count[b]; k++) bo[k] = (int)b;
  s->blk_of.upload(bo.data(), bo.size(), st);
  CK(cudaStreamSynchronize(st));  // the host vectors above die here
}

void ensure_device(sphgpu_space* s) {
  if (s->dev) return;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    throw std::runtime_error("no CUDA device available");
  int devid = 0;
  CK(cudaGetDevice(&devid));
  CK(cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, devid));
  CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
  cudaStream_t st = s->stream;
  const Space& sp = *s->space;
  const int n = sp.n();
  // Store order: the reference's cell order, Morton-sorted inside leaves.
  const auto& gperm = sp.gperm();
  const auto& g_of_s = sp.gpu_of_sorted();
  s->s_of_g.assign(n, 0);
  for (int k = 0; k < n; k++) s->s_of_g[g_of_s[k]] = k;
  std::vector<double> xs(3 * (size_t)n);
  std::vector<float4> vm(n);
  std::vector<float> hs(n), us(n);
  std::vector<uint8_t> fl(n);
  std::vector<int8_t> dh(n), dh0(n), tb(n);
  std::vector<int32_t> top(n), lf(n);
  const auto& xw = sp.x();
  const auto& act = sp.active();
  const auto& cells = sp.cells();
  const auto& leaf_of = sp.leaf_of();
  const auto& lvs = sp.leaves();
  const int ntop = sp.cdim()[0] * sp.cdim()[1] * sp.cdim()[2];
  for (int g = 0; g < n; g++) {
    const int k = gperm[g];
    const int srt = s->s_of_g[g];
    for (int d = 0; d < 3; d++) xs[3 * (size_t)g + d] = xw[3 * (size_t)k + d];
    vm[g] = make_float4(s->v_in[3 * (size_t)k], s->v_in[3 * (size_t)k + 1],
                        s->v_in[3 * (size_t)k + 2], s->m_in[k]);
    hs[g] = s->h_in[k];
    us[g] = s->u_in[k];
    fl[g] = act[srt] ? 1 : 0;
    tb[g] = s->tb_in[k];
    dh[g] = sp.depth_h()[srt];
    dh0[g] = sp.h_depth_of(s->h_in[k], lvs[leaf_of[srt]]);
    lf[g] = leaf_of[srt];
    top[g] = cells[lvs[leaf_of[srt]]].top;
  }
  s->n_active = 0;
  for (int g = 0; g < n; g++) s->n_active += fl[g];
  // one work group per 32-particle window of every leaf at most
  s->max_units = s->max_units_n[0] = s->max_units_n[1] = 0;
  std::vector<int> lwb(lvs.size() + 1, 0), lwbn[2];
  lwbn[0].assign(lvs.size() + 1, 0);
  lwbn[1].assign(lvs.size() + 1, 0);
  for (size_t l = 0; l < lvs.size(); l++) {
    lwb[l] = s->max_units;
    s->max_units += (cells[lvs[l]].count + 31) / 32;
    for (int w = 0; w < 2; w++) {
      lwbn[w][l] = s->max_units_n[w];
      s->max_units_n[w] += (cells[lvs[l]].count + (15 >> w)) / (16 >> w);
    }
  }
  lwb[lvs.size()] = s->max_units;
  s->lwb_host = lwb;
  for (int w = 0; w < 2; w++) {
    lwbn[w][lvs.size()] = s->max_units_n[w];
    s->lwb_host_n[w] = lwbn[w];
  }
  s->top_leaf.assign(ntop + 1, (int)lvs.size());
  for (int l = (int)lvs.size() - 1; l >= 0; l--) s->top_leaf[cells[lvs[l]].top] = l;
  for (int t = ntop - 1; t >= 0; t--)
    if (s->top_leaf[t] > s->top_leaf[t + 1]) s->top_leaf[t] = s->top_leaf[t + 1];
  std::vector<double> tl(3 * (size_t)ntop);
  for (int t = 0; t < ntop; t++)
    for (int d = 0; d < 3; d++) tl[3 * (size_t)t + d] = cells[t].loc[d];
  std::vector<LeafInfo> li;
  sp.leaf_infos(li);

  s->xd.upload(xs.data(), xs.size(), st);
  s->velm.upload(vm.data(), n, st);
  s->h0.upload(hs.data(), n, st);
  s->u.upload(us.data(), n, st);
  s->flags.upload(fl.data(), n, st);
  s->n_act_dev = 0;
  upload_activity(s, st);
  s->depth_h.upload(dh.data(), n, st);
  s->depth_h0.upload(dh0.data(), n, st);
  s->tbin.upload(tb.data(), n, st);
  s->ngb_bin.alloc(n);
  CK(cudaMemsetAsync(s->ngb_bin.p, SPH_NUM_TIME_BINS + 1, n, st));
  s->leaf_of.upload(lf.data(), n, st);
  s->top_of.upload(top.data(), n, st);
  s->perm.upload(gperm.data(), n, st);
  s->top_loc.upload(tl.data(), tl.size(), st);
  s->leaves.upload(li.data(), li.size(), st);
  upload_blocks(s, st);
  s->units.alloc(std::max(1, std::max(s->max_units, s->max_units_n[1])));
  s->leaf_window_begin.upload(lwb.data(), lwb.size(), st);
  for (int w = 0; w < 2; w++)
    s->leaf_window_begin_n[w].upload(lwbn[w].data(), lwbn[w].size(), st);
  s->posh.alloc(n);
  s->dens0.alloc(n);
  s->dens1.alloc(n);
  s->fin0.alloc(n);
  s->fin1.alloc(n);
  s->acc.alloc(n);
  s->hdt_vsig.alloc(n);
  s->left.alloc(n);
  s->right.alloc(n);
  s->ghost_iters.alloc(n);
  s->ngb_d.alloc(n);
  s->ngb_d_first.alloc(n);
  s->ngb_f.alloc(n);
  s->queue.alloc(16);  // [0..7] work counters, [8..15] unit counts
  s->redo.alloc(std::max(1, s->prm.max_iter));
  s->catchup.alloc(s->prm.max_iter + 1);
  s->hit_ctr.alloc(4);
  s->err.alloc(1);
  CK(cudaMemsetAsync(s->err.p, 0, sizeof(int), st));
  {
    const auto& fc = s->space->force_checks();
    static_assert(sizeof(ForceCheck) == sizeof(int4), "one int4 per checked cell");
    s->nchk = (int)fc.size();
    s->chk.upload(reinterpret_cast<const int4*>(fc.data()), fc.size(), st);
    if (!s->chk.p) s->chk.alloc(1);
    s->chk_pred.alloc(std::max<size_t>(1, fc.size()));
    CK(cudaMemsetAsync(s->chk_pred.p, 0, std::max<size_t>(1, fc.size()), st));
    s->vflag.alloc(1);
  }
  alloc_rows(s, st);
  for (auto& e : s->ev) CK(cudaEventCreate(&e));
  for (auto& e : s->pev) CK(cudaEventCreate(&e));
  CK(cudaMemsetAsync(s->fin0.p, 0, sizeof(float4) * n, st));
  CK(cudaMemsetAsync(s->fin1.p, 0, sizeof(float2) * n, st));
  CK(cudaMemsetAsync(s->acc.p, 0, sizeof(float4) * n, st));
  CK(cudaMemsetAsync(s->hdt_vsig.p, 0, sizeof(float2) * n, st));

  DevParticles& P = s->P;
  P.n = n;
  P.xd = s->xd.p;
  P.posh = s->posh.p;
  P.velm = s->velm.p;
  P.u = s->u.p;
  P.h0 = s->h0.p;
  P.flags = s->flags.p;
  P.depth_h = s->depth_h.p;
  P.depth_h0 = s->depth_h0.p;
  P.leaf_of = s->leaf_of.p;
  P.dens0 = s->dens0.p;
  P.dens1 = s->dens1.p;
  P.left = s->left.p;
  P.right = s->right.p;
  P.ghost_iters = s->ghost_iters.p;
  P.fin0 = s->fin0.p;
  P.fin1 = s->fin1.p;
  P.acc = s->acc.p;
  P.hdt_vsig = s->hdt_vsig.p;
  P.ngb_d = s->ngb_d.p;
  P.ngb_d_first = s->ngb_d_first.p;
  P.ngb_f = s->ngb_f.p;
  // The neighbours' smallest time bin can only limit a time step when the
  // bins differ (a step grows at most 2x, i.e. one bin, per step): with one
  // bin everywhere the force loops skip the extra load and leave it at
  // num_time_bins + 1.
  const bool mixed_bins = std::any_of(s->tb_in.begin(), s->tb_in.end(),
                                      [&](int8_t b) { return b != s->tb_in[0]; });
  P.tbin = mixed_bins ? s->tbin.p : nullptr;
  P.ngb_bin = s->ngb_bin.p;
  CK(launch_prepare_posh(P, s->top_of.p, s->top_loc.p, st));
  s->dplan_d.upload(s->plan_d, st);
  s->dplan_s.upload(s->plan_s, st);
  CK(cudaStreamSynchronize(st));
  s->dev = true;
}

// Relative band of the FP32 pre-test around H^2.  The FP32 offsets carry
// about 1e-8 absolute error; for the smallest H of the supported boxes
// (~0.005 box units) that is < 1e-5 relative on r^2, far inside this band.
constexpr float kBand = 2.44140625e-4f;  // 2^-12

// qslot selects the work counter (queue[qslot]) and the unit count
// (queue[8 + qslot]) of a launch.
G2Args gargs(sphgpu_space* s, DevPlan& dp, int qslot, int mode) {
  G2Args a;
  a.p = s->P;
  a.units = s->units.p;
  a.count = 0;
  a.count_ptr = s->queue.p + 8 + qslot;
  a.pair_block = dp.pb.p;
  a.pair_entry = dp.pe.p;
  a.entries = dp.entries.p;
  a.bb_lo = s->bb_lo.p;
  a.bb_hi = s->bb_hi.p;
  a.bb_fc = s->bb_fc.p;
  const double* w = s->space->width();
  a.top_width = make_float3((float)w[0], (float)w[1], (float)w[2]);
  a.leaf_tw = nullptr;
  a.queue = s->queue.p + qslot;
  a.hits = nullptr;
  a.gate = nullptr;
  if (s->count_hits) a.hits = s->hit_ctr.p + (qslot == 0 ? 0 : (qslot == 2 ? 2 : 1));
  a.band = kBand;
  a.mode = mode;
  a.nl = nullptr;
  a.nl_cnt = nullptr;
  a.nl_T = nullptr;
  a.nl_cap = 0;
  a.nl_widen = 1.f;
  a.leaves = s->leaves.p;
  a.force_rows = 0;
  a.nl_seg = 1;
  a.blk_of = s->blk_of.p;
  a.bulk = s->tune.bulk_stage;
  a.tc = s->tune.tc_filter;
  a.err = s->err.p;
  a.sb_lo = s->sb_lo.p;
  a.sb_hi = s->sb_hi.p;
  return a;
}

// Lanes per particle of the gather that records the re-run lists (one row
// segment per lane).
int rec_tpp(const sphgpu_space* s) { return std::min(2, s->tune.threads_per_particle); }

// Build the work groups of a loop (windows whose particles carry `need`
// in their flags) and run the gather over them.
// veto: skip particles with any of these flag bits; lists: record the re-run
// neighbour lists (density re-run mode)
void enqueue_gather(sphgpu_space* s, cudaStream_t st, DevPlan& dp, int qslot,
                    int mode, bool force, int need, const int* gate,
                    int leaf_begin = 0, int leaf_end = -1, int veto = 0,
                    bool lists = false, bool force_rows = false) {
  const int nl = (int)s->space->leaves().size();
  if (leaf_end < 0) leaf_end = nl;
  // two or four lanes per particle: 16- or 8-particle windows
  const int tpp = lists ? rec_tpp(s) : s->tune.threads_per_particle;
  const DBuf<int>& lwb = tpp == 1 ? s->leaf_window_begin : s->leaf_window_begin_n[tpp / 4];
  const std::vector<int>& lwbh = tpp == 1 ? s->lwb_host : s->lwb_host_n[tpp / 4];
  CK(cudaMemsetAsync(s->queue.p + qslot, 0, sizeof(int), st));
  // sparse launches (the ghost's re-runs over the particles still
  // iterating, steps planned on the device for few active particles) over
  // every leaf take only the non-empty windows: the gather then spends no
  // work-queue atomic on an empty one
  const bool compact = leaf_begin == 0 && leaf_end == nl && (mode == MODE_REDO || s->dmode);
  int* ncompact = s->queue.p + 8 + qslot;
  if (compact) CK(cudaMemsetAsync(ncompact, 0, sizeof(int), st));
  CK(launch_build_units(s->leaves.p + leaf_begin, leaf_end - leaf_begin, lwb.p + leaf_begin,
                        s->flags.p, need, veto, dp.lpb.p + leaf_begin, s->units.p, gate, st,
                        32 / tpp, compact ? ncompact : nullptr));
  // the groups of this leaf range occupy [w0, w1) of the window slots (or,
  // compacted, the first *ncompact)
  G2Args a = gargs(s, dp, qslot, mode);
  const int w0 = lwbh[leaf_begin], w1 = lwbh[leaf_end];
  a.units = s->units.p + (compact ? 0 : w0);
  a.count = w1 - w0;
  a.count_ptr = compact ? ncompact : nullptr;
  a.gate = gate;  // gated loops (ghost re-runs) do nothing when it reads 0
  if (lists) {
    a.nl = s->nl.p;
    a.nl_cnt = s->nl_cnt.p;
    a.nl_T = s->nl_T.p;
    a.nl_cap = row_cap(s);
    if (mode == MODE_FIRST)
      a.nl_widen = s->tune.row_widen > 0.f ? s->tune.row_widen : kListWiden;
  }
  if (force && force_rows) {
    // the force reads the rows the first pass recorded this step
    a.nl = s->nl.p;
    a.nl_cnt = s->nl_cnt.p;
    a.nl_T = s->nl_T.p;
    a.nl_cap = row_cap(s);
    a.nl_seg = rec_tpp(s);
    a.force_rows = 1;
  }
  CK(launch_gather(a, force, s->num_sms, w1 - w0, st, s->tune.block_warps, lists, tpp));
}

ListArgs largs(sphgpu_space* s, const int* gate) {
  ListArgs l;
  l.p = s->P;
  l.nl = s->nl.p;
  l.nl_cnt = s->nl_cnt.p;
  l.nl_T = s->nl_T.p;
  l.nl_cap = row_cap(s);
  l.nl_seg = rec_tpp(s);
  l.leaf_pair_begin = s->dplan_s.lpb.p;
  l.pair_block = s->dplan_s.pb.p;
  l.pair_entry = s->dplan_s.pe.p;
  l.entries = s->dplan_s.entries.p;
  l.blk_of = s->blk_of.p;
  const double* w = s->space->width();
  l.top_width = make_float3((float)w[0], (float)w[1], (float)w[2]);
  l.band = kBand;
  l.gate = gate;
  l.hits = s->count_hits ? s->hit_ctr.p + 1 : nullptr;
  l.handover = s->catchup.p;
  return l;
}

GhostArgs ghargs(sphgpu_space* s, int iter, int lo, int hi) {
  GhostArgs g;
  g.p = s->P;
  g.leaves = s->leaves.p;
  g.eta_dim = s->prm.eta * s->prm.eta * s->prm.eta;
  g.h_tol = s->prm.h_tolerance;
  g.h_max = s->prm.h_max;
  g.h_min = s->prm.h_min;
  g.alpha = s->prm.alpha;
  g.iter = iter;
  g.lo = lo;
  g.hi = hi;
  g.redo_count = s->redo.p;
  return g;
}

// Ghost rounds over all particles: round k iterates the particles still
// flagged, and re-runs the density of those it sends to another round
// (subset gather lists); both kernels return at once when the previous
// round sent none (gates on the redo counts).
bool lists_on(const sphgpu_space* s) { return s->lists && s->tune.rerun_lists; }
int row_cap(const sphgpu_space* s) { return s->tune.row_cap > 0 ? s->tune.row_cap : kListCap; }

// The step graph holds the first kGraphRounds ghost rounds (h converges in
// 2-4 for almost every particle); the rare later ones run outside it, only
// when particles are left.
constexpr int kGraphRounds = 8;

void enqueue_ghost_rounds(sphgpu_space* s, cudaStream_t st, int k0 = 0, int k1 = -1) {
  if (k1 < 0) k1 = s->prm.max_iter;
  if (lists_on(s)) {
    // round 0, then the later rounds particle by particle from the lists;
    // the particles whose h outgrew their list catch up by gathers, each at
    // its own round count (catch-up rounds k0 .. k1 - 1)
    if (k0 == 0) {
      CK(launch_ghost(ghargs(s, 0, 0, s->P.n), st));
      CK(cudaMemsetAsync(s->catchup.p, 0, sizeof(int) * (s->prm.max_iter + 1), st));
      CK(launch_solve_from_lists(largs(s, s->redo.p), ghargs(s, 1, 0, s->P.n),
                                 s->prm.max_iter, st));
    }
    for (int r = k0; r < k1 && r < s->prm.max_iter; r++) {
      enqueue_gather(s, st, s->dplan_s, 1, MODE_REDO, false, 3, s->catchup.p + r);
      CK(launch_ghost_catchup(ghargs(s, 0, 0, s->P.n), s->prm.max_iter, s->catchup.p + r,
                              s->catchup.p + r + 1, st));
    }
    return;
  }
  for (int k = k0; k < k1; k++) {
    CK(launch_ghost(ghargs(s, k, 0, s->P.n), st));
    enqueue_gather(s, st, s->dplan_s, 1, MODE_REDO, false, 3, s->redo.p + k);
  }
}

void enqueue_density(sphgpu_space* s, cudaStream_t st, bool density) {
  CK(launch_begin_step(s->P, s->prm.max_iter, s->redo.p, s->prm.h_max, st));
  // the first pass records the re-runs' lists
  if (density)
    enqueue_gather(s, st, s->dplan_d, 0, MODE_FIRST, false, 1, nullptr, 0, -1, 0, lists_on(s));
}

void enqueue_density_ghost(sphgpu_space* s, cudaStream_t st, int stages) {
  enqueue_density(s, st, (stages & SPHGPU_STAGE_DENSITY) != 0);
  if (stages & SPHGPU_STAGE_GHOST) enqueue_ghost_rounds(s, st);
}

void enqueue_force(sphgpu_space* s, cudaStream_t st) {
  CK(launch_block_hmax(s->bb_fc.p, s->bb_lo.p, s->posh.p, s->bb_n, st));
  enqueue_gather(s, st, s->dplan_f, 2, MODE_FIRST, true, 1, nullptr, 0, -1, 0, false,
                 lists_on(s));
}

int check_conv(sphgpu_space* s, cudaStream_t st) {
  int last = 0, err = 0;
  CK(cudaMemcpyAsync(&last, s->redo.p + s->prm.max_iter - 1, sizeof(int),
                     cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&err, s->err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (err) {
    CK(cudaMemsetAsync(s->err.p, 0, sizeof(int), st));
    return fail(SPHGPU_ECUDA, "a gather gave up waiting for a bulk copy of a j-block; "
                              "the step's results are incomplete");
  }
  if (last > 0)
    return fail(SPHGPU_ENOCONV, "smoothing length failed to converge on " +
                                    std::to_string(last) + " particles");
  return SPHGPU_OK;
}

// Activity of the store: clears the flags of the previously active
// particles, sets those of the current active list.
void upload_activity(sphgpu_space* s, cudaStream_t st) {
  const auto& al = s->space->active_list();
  const auto& gos = s->space->gpu_of_sorted();
  std::vector<int> g(al.size());
  for (size_t a = 0; a < al.size(); a++) g[a] = gos[al[a]];
  CK(launch_set_flags(s->flags.p, s->act_g.p, s->n_act_dev, 0, st));
  s->act_g.upload(g.data(), g.size(), st);
  s->n_act_dev = (int)g.size();
  s->n_active = s->n_act_dev;
  CK(launch_set_flags(s->flags.p, s->act_g.p, s->n_act_dev, 1, st));
}

// Bring the planner's h up to date: only the active particles' h changes
// on the device between two activations, so only theirs is read back.
void fetch_active_h(sphgpu_space* s, cudaStream_t st) {
  const int m = s->n_act_dev;
  std::vector<float> h(m);
  if (m) {
    if (s->act_h.n < (size_t)m) s->act_h.alloc(m);
    CK(launch_gather_h(s->posh.p, s->act_g.p, m, s->act_h.p, st));
    CK(cudaMemcpyAsync(h.data(), s->act_h.p, sizeof(float) * m, cudaMemcpyDeviceToHost, st));
  }
  CK(cudaStreamSynchronize(st));
  s->space->update_h_active(h.data());
  s->h_stale = false;
}

// The force loop's recursion depends on the post-ghost h_max of every cell
// (cell.h:966-1010 use hydro.h_max); plan it once the ghost has run.
void drop_graph(sphgpu_space* s);

// The force lists and the decisions they were planned with (one per checked
// cell) to the device; false when the buffers kept their addresses.
bool upload_force_plan(sphgpu_space* s, const std::vector<uint8_t>& pred, cudaStream_t st) {
  const bool moved = s->dplan_f.upload(s->plan_f, st);
  if (!pred.empty())
    CK(cudaMemcpyAsync(s->chk_pred.p, pred.data(), pred.size(), cudaMemcpyHostToDevice, st));
  CK(cudaStreamSynchronize(st));  // the host vectors may change after this
  return moved;
}

void plan_force(sphgpu_space* s, cudaStream_t st) {
  fetch_active_h(s, st);
  s->space->plan_density(s->plan_f, true);
  std::vector<uint8_t> pred;
  s->space->force_decisions(pred);
  if (upload_force_plan(s, pred, st)) drop_graph(s);
  s->force_planned = true;
  s->h_stale = false;
}

cudaStream_t pick(sphgpu_space* s, void* stream) {
  return stream ? (cudaStream_t)stream : s->stream;
}


void drop_graph(sphgpu_space* s) {
  for (auto& g : s->graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

template <class F>
cudaGraphExec_t capture(cudaStream_t st, F&& body) {
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  try {
    body();
  } catch (...) {
    cudaGraph_t dead = nullptr;
    cudaStreamEndCapture(st, &dead);
    if (dead) cudaGraphDestroy(dead);
    throw;
  }
  CK(cudaStreamEndCapture(st, &g));
  cudaGraphExec_t ex = nullptr;
  const cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
  cudaGraphDestroy(g);
  CK(e);
  return ex;
}

// ---------------------------------------------------------------------------
// Device planning

// The tree, the tasks and the j-block ranges for the device planner (again
// after a change of the j-block depth).
void dp_upload_tree(sphgpu_space* s, cudaStream_t st) {
  const Space& sp = *s->space;
  const auto& cells = sp.cells();
  const auto& jb = sp.jblocks();
  const size_t nc = cells.size();
  std::vector<DPCell> dc(nc);
  std::vector<int32_t> prog(8 * nc);
  int maxd = 0;
  for (size_t c = 0; c < nc; c++) {
    const Cell& x = cells[c];
    DPCell& d = dc[c];
    std::memset(&d, 0, sizeof(d));
    for (int k = 0; k < 3; k++) d.loc[k] = x.loc[k];
    d.dmin = x.dmin;
    d.first = x.first;
    d.count = x.count;
    d.parent = x.parent;
    d.top = x.top;
    d.jb_begin = jb.cell_begin[c];
    d.jb_end = jb.cell_end[c];
    d.depth = (int16_t)x.depth;
    d.split = (int8_t)(x.split ? 1 : 0);
    for (int k = 0; k < 8; k++) prog[8 * c + k] = x.progeny[k];
    maxd = std::max(maxd, x.depth);
  }
  const auto& tasks = sp.tasks();
  std::vector<int2> tk(tasks.size());
  for (size_t t = 0; t < tasks.size(); t++) tk[t] = make_int2(tasks[t].ci, tasks[t].cj);
  const auto& links = sp.top_links();
  std::vector<int32_t> lb(links.size() + 1, 0), lk;
  for (size_t c = 0; c < links.size(); c++) {
    lb[c] = (int32_t)lk.size();
    lk.insert(lk.end(), links[c].begin(), links[c].end());
  }
  lb[links.size()] = (int32_t)lk.size();
  const std::vector<int>& lv = sp.leaves();
  s->dp_cell.upload(dc.data(), nc, st);
  s->dp_prog.upload(prog.data(), prog.size(), st);
  s->dp_leaf.upload(lv.data(), lv.size(), st);
  s->dp_task.upload(tk.data(), std::max<size_t>(1, tk.size()), st);
  s->dp_lbeg.upload(lb.data(), lb.size(), st);
  s->dp_link.upload(lk.data(), std::max<size_t>(1, lk.size()), st);
  if (s->dp_hmax.n < nc) {
    s->dp_hmax.alloc(nc);
    s->dp_hact.alloc(nc);
    s->dp_hforce.alloc(nc);
    s->dp_active.alloc(nc);
  }
  const size_t nl = lv.size();
  if (s->dp_off.n < nl + 1) {
    s->dp_lane.alloc(32 * nl);
    s->dp_off.alloc(nl + 1);
    s->dp_tiles.alloc(dp_scan_tiles((long long)nl + 1));
  }
  if (!s->dp_status.p) {
    s->dp_status.alloc(8);
    s->dp_bin_dev.alloc(1);
  }
  DPTree& t = s->dpt;
  t.cell = s->dp_cell.p;
  t.progeny = s->dp_prog.p;
  t.leaf_cell = s->dp_leaf.p;
  t.task = s->dp_task.p;
  t.link_begin = s->dp_lbeg.p;
  t.link = s->dp_link.p;
  t.ncells = (int)nc;
  t.nleaves = (int)nl;
  t.ntop = (int)links.size();
  t.ntasks = (int)tasks.size();
  for (int k = 0; k < 3; k++) t.dim[k] = s->prm.dim[k];
  t.periodic = s->prm.periodic;
  CK(cudaStreamSynchronize(st));  // the host vectors above die here
  // frames: one per level below the top cell, the root task and a margin
  if (maxd + 3 > kDPStack) s->dp_usable = false;
  s->dp_ready = true;
}

DPCellState dp_state(sphgpu_space* s) {
  DPCellState cs;
  cs.hmax = s->dp_hmax.p;
  cs.hact = s->dp_hact.p;
  cs.hforce = s->dp_hforce.p;
  cs.active = s->dp_active.p;
  cs.dx = s->drifted ? s->dp_dx.p : nullptr;
  return cs;
}

DevPlan& dp_plan_of(sphgpu_space* s, int kind) {
  return kind == DP_DENSITY ? s->dplan_d : (kind == DP_SUBSET ? s->dplan_s : s->dplan_f);
}

DPOut dp_out(sphgpu_space* s, int kind) {
  DevPlan& dp = dp_plan_of(s, kind);
  DPOut o;
  o.entries = dp.entries.p;
  o.lpb = dp.lpb.p;
  o.pb = dp.pb.p;
  o.pe = dp.pe.p;
  o.cap_e = s->dp_cap_e[kind];
  o.cap_p = s->dp_cap_p[kind];
  o.lane_off = s->dp_lane.p;
  o.leaf_off = s->dp_off.p;
  o.tiles = s->dp_tiles.p;
  o.status = s->dp_status.p;
  return o;
}

// Plan buffers of at least the capacities asked for; true when one moved.
bool dp_reserve(sphgpu_space* s) {
  const size_t nl = s->space->leaves().size();
  bool moved = false;
  for (int k = 0; k < 3; k++) {
    DevPlan& dp = dp_plan_of(s, k);
    auto grow = [&](auto& buf, size_t want) {
      if (buf.n >= want) return;
      buf.alloc(want);
      moved = true;
    };
    grow(dp.entries, (size_t)s->dp_cap_e[k]);
    grow(dp.lpb, nl + 1);
    grow(dp.pb, (size_t)s->dp_cap_p[k]);
    grow(dp.pe, (size_t)s->dp_cap_p[k]);
    // the capacity is what the buffers hold (they may have been larger)
    s->dp_cap_e[k] = (long long)dp.entries.n;
    s->dp_cap_p[k] = (long long)std::min(dp.pb.n, dp.pe.n);
  }
  return moved;
}

// Flags from the time bins, the step's start (begin_step), the cells'
// activation state and the density and re-run lists.
void enqueue_dev_plans(sphgpu_space* s, cudaStream_t st, bool timed) {
  CK(launch_dp_flags(s->flags.p, s->tbin.p, s->P.n, s->dp_bin_dev.p, st));
  CK(launch_begin_step(s->P, s->prm.max_iter, s->redo.p, s->prm.h_max, st));
  if (timed) CK(cudaEventRecordWithFlags(s->pev[0], st, cudaEventRecordExternal));
  const DPCellState cs = dp_state(s);
  CK(launch_dp_cells(s->dpt, cs, s->posh.p, s->h0.p, s->flags.p, false, st));
  CK(launch_dp_plan(s->dpt, cs, DP_DENSITY, dp_out(s, DP_DENSITY), st));
  CK(launch_dp_plan(s->dpt, cs, DP_SUBSET, dp_out(s, DP_SUBSET), st));
  if (timed) CK(cudaEventRecordWithFlags(s->pev[1], st, cudaEventRecordExternal));
}

void enqueue_dev_force(sphgpu_space* s, cudaStream_t st, bool timed) {
  if (timed) CK(cudaEventRecordWithFlags(s->pev[2], st, cudaEventRecordExternal));
  const DPCellState cs = dp_state(s);
  CK(launch_dp_cells(s->dpt, cs, s->posh.p, s->h0.p, s->flags.p, true, st));
  CK(launch_dp_plan(s->dpt, cs, DP_FORCE, dp_out(s, DP_FORCE), st));
  if (timed) CK(cudaEventRecordWithFlags(s->pev[3], st, cudaEventRecordExternal));
  enqueue_force(s, st);
}

// The whole step with device planning: flags, plans, density, ghost rounds
// (the first `rounds` of them), force plan, force.  `captured`: enqueued
// into a graph capture (the phase events become external event-record
// nodes, and the planning is timed).
void enqueue_dev_step(sphgpu_space* s, cudaStream_t st, int rounds, bool captured) {
  auto mark = [&](cudaEvent_t e) {
    if (captured)
      CK(cudaEventRecordWithFlags(e, st, cudaEventRecordExternal));
    else
      CK(cudaEventRecord(e, st));
  };
  CK(cudaMemsetAsync(s->dp_status.p, 0, 8 * sizeof(int), st));
  enqueue_dev_plans(s, st, captured);
  enqueue_gather(s, st, s->dplan_d, 0, MODE_FIRST, false, 1, nullptr, 0, -1, 0, lists_on(s));
  mark(s->ev[1]);
  enqueue_ghost_rounds(s, st, 0, rounds);
  mark(s->ev[2]);
  enqueue_dev_force(s, st, captured);
}

// The time bins a caller set on the device (store order) into the planner.
void sync_host_bins(sphgpu_space* s) {
  if (!s->bins_host_stale) return;
  const int n = s->P.n;
  std::vector<int8_t> tb(n);
  CK(cudaStreamSynchronize(s->stream));
  CK(cudaMemcpy(tb.data(), s->tbin.p, n, cudaMemcpyDeviceToHost));
  const auto& gperm = s->space->gperm();
  for (int g = 0; g < n; g++) s->tb_in[gperm[g]] = tb[g];
  s->space->set_bins(s->tb_in.data());
  s->bins_host_stale = false;
}

// The host planner's dx_max per cell and input h after drifts.
void sync_host_drift(sphgpu_space* s) {
  if (!s->drifted || !s->drift_host_stale) return;
  cudaStream_t st = s->stream;
  const int n = s->P.n;
  const size_t nc = s->space->cells().size();
  std::vector<float> dx(nc), h0(n);
  CK(cudaMemcpyAsync(dx.data(), s->dp_dx.p, sizeof(float) * nc, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(h0.data(), s->h0.p, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  s->space->set_dx_max(dx.data());
  const auto& gperm = s->space->gperm();
  for (int g = 0; g < n; g++) s->h_in[gperm[g]] = h0[g];
  s->space->set_input_h(s->h_in.data());
  s->drift_host_stale = false;
}

// Bring the host planner level with the device: every particle's current h
// into the planner, the device flags cleared (the next host activation sets
// them by index lists again), every cell recomputed at that activation.
void leave_device_mode(sphgpu_space* s) {
  if (!s->dmode) return;
  cudaStream_t st = s->stream;
  const int n = s->P.n;
  std::vector<float> hw(n), hs(n);
  CK(cudaStreamSynchronize(st));
  // posh.w of every particle: a 4-byte column of 16-byte rows
  CK(cudaMemcpy2DAsync(hw.data(), sizeof(float), reinterpret_cast<const char*>(s->posh.p) + 12,
                       sizeof(float4), sizeof(float), n, cudaMemcpyDeviceToHost, st));
  CK(cudaMemsetAsync(s->flags.p, 0, n, st));
  CK(cudaStreamSynchronize(st));
  for (int g = 0; g < n; g++) hs[s->s_of_g[g]] = hw[g];
  s->space->assign_h(hs.data());
  sync_host_drift(s);
  s->n_act_dev = 0;
  s->dmode = false;
  s->h_stale = false;
  s->force_planned = false;
  s->host_refresh = true;
  drop_graph(s);
}

// The host planner's activation (the body of sphgpu_set_active without the
// device planner).
void host_activate(sphgpu_space* s, int32_t max_active_bin) {
  if (s->dev) CK(cudaStreamSynchronize(s->stream));
  if (s->dev && s->h_stale) fetch_active_h(s, s->stream);
  sync_host_bins(s);
  const auto t0 = std::chrono::steady_clock::now();
  s->prm.max_active_bin = max_active_bin;
  s->space->set_activity(max_active_bin);
  if (s->host_refresh) {
    s->space->refresh_all();
    s->host_refresh = false;
  }
  build_plans(s);
  const auto t1 = std::chrono::steady_clock::now();
  s->act_plan_ms += std::chrono::duration<double, std::milli>(t1 - t0).count();
  s->force_planned = false;
  s->task_d.clear();
  s->task_f.clear();
  if (s->dev) {
    upload_activity(s, s->stream);
    bool moved = s->dplan_d.upload(s->plan_d, s->stream);
    moved |= s->dplan_s.upload(s->plan_s, s->stream);
    CK(cudaStreamSynchronize(s->stream));
    s->act_upload_ms += std::chrono::duration<double, std::milli>(
                            std::chrono::steady_clock::now() - t1).count();
    // the force lists ahead of the step, from each active particle's last
    // converged h; the step checks the plan's decisions on the device
    // after its ghost and re-plans on the host if any differs
    // (a drifted space's recursion decisions also depend on dx_max, which
    // the device check does not see: its force lists are planned after the
    // ghost)
    if (!s->drifted) {
      const auto t2 = std::chrono::steady_clock::now();
      std::vector<uint8_t> pred;
      s->space->plan_force_predicted(s->plan_f, pred);
      moved |= upload_force_plan(s, pred, s->stream);
      s->force_planned = true;
      s->plan_ms += std::chrono::duration<double, std::milli>(
                        std::chrono::steady_clock::now() - t2).count();
    }
    // the step graph reads the plans in place: it stays valid unless a
    // buffer moved
    if (moved) drop_graph(s);
  } else {
    drop_graph(s);
  }
}

// Entry points that use the host planner's state call this first.
void ensure_host_state(sphgpu_space* s) {
  if (!s->dmode) return;
  leave_device_mode(s);
  host_activate(s, s->prm.max_active_bin);
}

// Device planning for activations that leave some particles inactive on a
// space that is resident already (all-active steps keep the host's plans,
// which they reuse from step to step).
bool want_device_plans(const sphgpu_space* s, int32_t max_active_bin) {
  return s->dev && s->dp_usable && !s->dp_off_by_caller &&
         (max_active_bin < s->max_bin || s->drifted);
}

void enter_device_mode(sphgpu_space* s, int32_t max_active_bin) {
  cudaStream_t st = s->stream;
  if (!s->dp_ready) dp_upload_tree(s, st);
  if (!s->dp_usable) return;
  if (!s->dmode) {
    // first capacities: the host's current plans (usually the all-active
    // step's) with a margin; a step that needs more grows them
    const Plan* hp[3] = {&s->plan_d, &s->plan_s, &s->plan_f};
    for (int k = 0; k < 3; k++) {
      s->dp_cap_e[k] = std::max<long long>(
          s->dp_cap_e[k], std::max<long long>(1024, 3 * (long long)hp[k]->entries.size() / 2));
      s->dp_cap_p[k] = std::max<long long>(
          s->dp_cap_p[k], std::max<long long>(4096, 3 * (long long)hp[k]->pair_block.size() / 2));
    }
    s->dmode = true;
    drop_graph(s);  // the host-planned step graph has another shape
  }
  if (dp_reserve(s)) drop_graph(s);
  s->dp_bin = max_active_bin;
  s->prm.max_active_bin = max_active_bin;
  // the plan buffers hold another activation's lists until a step runs
  s->force_planned = false;
}

// One step with device planning.  After the graph the host reads the
// planner's status and the particles still iterating: a plan that outgrew
// its buffers makes them grow and the step run again uncaptured (the step
// only writes the active particles' fields, which begin_step resets); a
// planner error hands the space back to the host planner for good; late
// ghost rounds run here, then the force plan and the force again.
// Returns false when the step must be run by the host-planned path.
// Pinned status words and their event (launch_step_*).
void ensure_status_words(sphgpu_space* s) {
  if (s->hw) return;
  CK(cudaMallocHost(&s->hw, 10 * sizeof(int)));
  CK(cudaEventCreateWithFlags(&s->hw_ev, cudaEventDisableTiming));
}

// A device-planned step: its graph and the copies of its status words
// (particles still iterating after the graph's rounds, the plans' status).
void launch_step_device(sphgpu_space* s, cudaStream_t st) {
  ensure_status_words(s);
  s->h_stale = true;
  const int rounds = std::min(kGraphRounds, s->prm.max_iter);
  CK(cudaMemcpyAsync(s->dp_bin_dev.p, &s->dp_bin, sizeof(int), cudaMemcpyHostToDevice, st));
  if (!s->graph[0]) {
    s->graph[0] = capture(st, [&]() { enqueue_dev_step(s, st, rounds, true); });
    s->step_stats[3]++;
  }
  CK(cudaEventRecord(s->ev[0], st));
  CK(cudaGraphLaunch(s->graph[0], st));
  CK(cudaEventRecord(s->ev[3], st));
  s->step_stats[0]++;
  s->hw[0] = 0;
  if (rounds < s->prm.max_iter) {
    const int* cnt = lists_on(s) ? s->catchup.p + rounds : s->redo.p + rounds - 1;
    CK(cudaMemcpyAsync(s->hw, cnt, sizeof(int), cudaMemcpyDeviceToHost, st));
  }
  CK(cudaMemcpyAsync(s->hw + 2, s->dp_status.p, 8 * sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaEventRecord(s->hw_ev, st));
  s->pending = 2;
}

// The rest of a device-planned step once its status words are in: 0 done,
// 1 more work enqueued (late rounds, a re-run with larger plan buffers),
// -1 the host planner took the space over (the step is still to be run).
int finish_step_device(sphgpu_space* s, cudaStream_t st) {
  CK(cudaEventSynchronize(s->hw_ev));
  s->pending = 0;
  const int rounds = std::min(kGraphRounds, s->prm.max_iter);
  int status[8];
  for (int k = 0; k < 8; k++) status[k] = s->hw[2 + k];
  int left = s->hw[0];
  int more = 0;
  auto read_back = [&]() {
    if (rounds < s->prm.max_iter) {
      const int* cnt = lists_on(s) ? s->catchup.p + rounds : s->redo.p + rounds - 1;
      CK(cudaMemcpyAsync(&left, cnt, sizeof(int), cudaMemcpyDeviceToHost, st));
    }
    CK(cudaMemcpyAsync(status, s->dp_status.p, sizeof(status), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
  };
  for (int attempt = 0; attempt < 2 && status[0] == 1; attempt++) {
    // a plan outgrew its buffers: grow them to what it needed, run again
    for (int k = 0; k < 3; k++) {
      s->dp_cap_e[k] = std::max(s->dp_cap_e[k], 5LL * status[1 + 2 * k] / 4 + 1024);
      s->dp_cap_p[k] = std::max(s->dp_cap_p[k], 5LL * status[2 + 2 * k] / 4 + 4096);
    }
    dp_reserve(s);
    drop_graph(s);
    s->step_stats[1]++;
    CK(cudaEventRecord(s->ev[0], st));
    enqueue_dev_step(s, st, rounds, false);
    CK(cudaEventRecord(s->pev[0], st));  // (no planning times for this step)
    CK(cudaEventRecord(s->pev[1], st));
    CK(cudaEventRecord(s->pev[2], st));
    CK(cudaEventRecord(s->pev[3], st));
    CK(cudaEventRecord(s->ev[3], st));
    read_back();
    more = 1;
  }
  if (status[0] != 0) {
    // too deep a recursion, too many tasks on a top cell or an
    // inconsistent tree (or buffers that would not do): the host plans
    s->dp_usable = false;
    leave_device_mode(s);
    host_activate(s, s->dp_bin);
    return -1;
  }
  if (left > 0) {
    enqueue_ghost_rounds(s, st, rounds, s->prm.max_iter);
    enqueue_dev_force(s, st, false);
    CK(cudaEventRecord(s->ev[3], st));
    s->step_stats[2]++;
    more = 1;
  }
  s->force_planned = true;
  return more;
}

bool run_step_device(sphgpu_space* s, cudaStream_t st) {
  launch_step_device(s, st);
  return finish_step_device(s, st) >= 0;
}

// Staging buffers of host-side inputs (sphgpu_step_host, sphgpu_space_drift).
void ensure_stage(sphgpu_space* s, cudaStream_t st) {
  const int n = s->P.n;
  if (!s->x_stage.p) {
    s->x_stage.alloc(3 * (size_t)n);
    s->v_stage.alloc(3 * (size_t)n);
    s->m_stage.alloc(n);
    s->h_stage.alloc(n);
    s->u_stage.alloc(n);
    s->out_stage.alloc(24 * (size_t)n);
  }
  if (!s->x_ref.p) {
    s->x_ref.upload(s->x_in.data(), s->x_in.size(), st);
    s->differ.alloc(1);
  }
}

// The drift of x_stage / h_stage (input order): measure, check the rebuild
// criterion, then commit (sphgpu_space_drift).
int drift_space(sphgpu_space* s, cudaStream_t st) {
  if (!s->dp_ready) dp_upload_tree(s, st);
  if (!s->dp_usable)
    return fail(SPHGPU_EINVAL, "sphgpu_space_drift: the cell tree is deeper than the device "
                               "planner's recursion stack; create a new space instead");
  const int n = s->P.n;
  const size_t nc = s->space->cells().size();
  if (!s->x_rb.p) {
    s->x_rb.upload(s->x_in.data(), s->x_in.size(), st);
    s->dp_dx.alloc(nc);
    CK(cudaMemsetAsync(s->dp_dx.p, 0, sizeof(unsigned) * nc, st));
    s->dp_dxn.alloc(nc);
    s->dp_hdrift.alloc(nc);
    s->drift_flag.alloc(1);
  }
  CK(cudaMemsetAsync(s->drift_flag.p, 0, sizeof(int), st));
  CK(launch_drift_cells(s->dpt, s->perm.p, s->x_stage.p, s->x_rb.p, s->h_stage.p, s->dp_dxn.p,
                        s->dp_hdrift.p, st));
  CK(launch_drift_check(s->dpt, s->dp_dxn.p, s->dp_hdrift.p, s->drift_flag.p, st));
  int flag = 0;
  CK(cudaMemcpyAsync(&flag, s->drift_flag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (flag)
    return fail(SPHGPU_EREBUILD,
                "the particles moved too far for the cell tree (cell_need_rebuild_for_hydro_pair "
                "holds for a pair of neighbouring top-level cells): create a new space");
  CK(launch_drift_commit(s->P, s->xd.p, s->depth_h0.p, s->perm.p, s->x_stage.p, s->h_stage.p,
                         s->top_of.p, s->top_loc.p, s->leaves.p, st));
  CK(cudaMemcpyAsync(s->dp_dx.p, s->dp_dxn.p, sizeof(unsigned) * nc, cudaMemcpyDeviceToDevice, st));
  CK(launch_block_boxes(s->bb_fc.p, s->posh.p, s->bb_lo.p, s->bb_hi.p, s->sb_lo.p, s->sb_hi.p,
                        s->bb_n, st));
  CK(cudaMemcpyAsync(s->x_ref.p, s->x_stage.p, sizeof(double) * 3 * (size_t)n,
                     cudaMemcpyDeviceToDevice, st));
  if (!s->drifted) drop_graph(s);  // the captured plans read no dx_max yet
  s->drifted = true;
  s->drift_host_stale = true;
  s->h_stale = true;
  s->sorted_mask = 0;
  s->task_d.clear();
  s->task_f.clear();
  // the next steps plan with the new dx_max and h
  const int b = s->prm.max_active_bin;
  if (want_device_plans(s, b)) {
    enter_device_mode(s, b);
  } else if (!s->dmode) {
    s->h_stale = false;
    CK(cudaStreamSynchronize(st));
    // every particle's h changed: the host planner takes them all
    std::vector<float> hw(n), hs(n);
    CK(cudaMemcpy2DAsync(hw.data(), sizeof(float), reinterpret_cast<const char*>(s->posh.p) + 12,
                         sizeof(float4), sizeof(float), n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    for (int g = 0; g < n; g++) hs[s->s_of_g[g]] = hw[g];
    s->space->assign_h(hs.data());
    sync_host_drift(s);
    s->host_refresh = true;
    host_activate(s, b);
  }
  return SPHGPU_OK;
}

}  // namespace

extern "C" {

namespace {
// Finishes a pipelined step still in flight (defined with the pipelined form).
void settle(sphgpu_space* s);
}  // namespace

int sphgpu_abi_version(void) { return SPHGPU_ABI_VERSION; }

const char* sphgpu_last_error(void) { return g_err.c_str(); }

void sphgpu_default_params(sphgpu_params* p) {
  if (!p) return;
  Params d;
  p->dim[0] = d.dim[0];
  p->dim[1] = d.dim[1];
  p->dim[2] = d.dim[2];
  p->periodic = d.periodic;
  p->eta = d.eta;
  p->h_tolerance = d.h_tolerance;
  p->h_max = d.h_max;
  p->h_min = d.h_min;
  p->alpha = d.alpha;
  p->max_iter = d.max_iter;
  p->max_active_bin = d.max_active_bin;
  p->max_top_level_cells = d.max_top_level_cells;
}

static int space_create(const sphgpu_params* prm, int64_t n, const double* x,
                        const float* v, const float* m, const float* h,
                        const float* u, const int8_t* time_bin, const int32_t* order,
                        const int32_t* tree, int32_t ncells, sphgpu_space** out);

int sphgpu_space_create(const sphgpu_params* prm, int64_t n, const double* x,
                        const float* v, const float* m, const float* h,
                        const float* u, const int8_t* time_bin,
                        sphgpu_space** out) {
  return space_create(prm, n, x, v, m, h, u, time_bin, nullptr, nullptr, 0, out);
}

int sphgpu_space_create_assigned(const sphgpu_params* prm, int64_t n, const double* x,
                                 const float* v, const float* m, const float* h,
                                 const float* u, const int8_t* time_bin,
                                 const int32_t* order, const int32_t* cells, int32_t ncells,
                                 sphgpu_space** out) {
  if (!order || !cells || ncells <= 0)
    return fail(SPHGPU_EINVAL, "sphgpu_space_create_assigned: no order or tree");
  return space_create(prm, n, x, v, m, h, u, time_bin, order, cells, ncells, out);
}

static int space_create(const sphgpu_params* prm, int64_t n, const double* x,
                        const float* v, const float* m, const float* h,
                        const float* u, const int8_t* time_bin, const int32_t* order,
                        const int32_t* tree, int32_t ncells, sphgpu_space** out) {
  if (!prm || !x || !v || !m || !h || !u || !time_bin || !out || n <= 0)
    return fail(SPHGPU_EINVAL, "sphgpu_space_create: null argument or n <= 0");
  if (n > SPHGPU_MAX_PARTICLES)
    return fail(SPHGPU_EINVAL, "sphgpu_space_create: more than SPHGPU_MAX_PARTICLES "
                               "particles (partner indices are packed in 27 bits)");
  if (prm->max_iter < 1 || prm->max_iter > 1000 || prm->max_top_level_cells < 3 ||
      !(prm->eta > 0.f) || !(prm->dim[0] > 0) || !(prm->dim[1] > 0) || !(prm->dim[2] > 0))
    return fail(SPHGPU_EINVAL, "sphgpu_space_create: invalid parameters");
  *out = nullptr;
  return guard([&]() {
    auto s = std::make_unique<sphgpu_space>();
    Params& P = s->prm;
    for (int d = 0; d < 3; d++) P.dim[d] = prm->dim[d];
    P.periodic = prm->periodic;
    P.eta = prm->eta;
    P.h_tolerance = prm->h_tolerance;
    P.h_max = prm->h_max;
    P.h_min = prm->h_min;
    P.alpha = prm->alpha;
    P.max_iter = prm->max_iter;
    P.max_active_bin = prm->max_active_bin;
    P.max_top_level_cells = prm->max_top_level_cells;
    s->x_in.assign(x, x + 3 * (size_t)n);
    s->v_in.assign(v, v + 3 * (size_t)n);
    s->m_in.assign(m, m + n);
    s->h_in.assign(h, h + n);
    s->u_in.assign(u, u + n);
    s->tb_in.assign(time_bin, time_bin + n);
    s->max_bin = *std::max_element(time_bin, time_bin + n);
    s->space = std::make_unique<Space>(P);
    s->space->build(n, x, h, time_bin, order, tree, ncells);
    build_plans(s.get());
    *out = s.release();
    return SPHGPU_OK;
  });
}

int sphgpu_space_destroy(sphgpu_space* s) {
  delete s;
  return SPHGPU_OK;
}

int sphgpu_space_info(const sphgpu_space* s, int64_t info[8]) {
  if (!s || !info) return fail(SPHGPU_EINVAL, "null argument");
  info[0] = s->space->n();
  info[1] = s->space->cdim()[0];
  info[2] = s->space->cdim()[1];
  info[3] = s->space->cdim()[2];
  info[4] = (int64_t)s->space->cells().size();
  info[5] = (int64_t)s->space->leaves().size();
  info[6] = (int64_t)s->space->tasks().size();
  info[7] = (int64_t)s->plan_d.entries.size();
  return SPHGPU_OK;
}

int sphgpu_space_cells(const sphgpu_space* s, int32_t* out) {
  if (!s || !out) return fail(SPHGPU_EINVAL, "null argument");
  const Space& sp = *s->space;
  const auto& cells = sp.cells();
  const auto& lvs = sp.leaves();
  for (int i = 0; i < sp.n(); i++) {
    const Cell& L = cells[lvs[sp.leaf_of()[i]]];
    int32_t* o = out + 6 * (size_t)sp.perm()[i];
    o[0] = L.first;
    o[1] = L.count;
    o[2] = L.depth;
    o[3] = sp.depth_h()[i];
    o[4] = i;
    o[5] = L.top;
  }
  return SPHGPU_OK;
}

int sphgpu_space_leaves(const sphgpu_space* s, double* geom, int32_t* ints) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  const auto& cells = s->space->cells();
  const auto& lvs = s->space->leaves();
  for (size_t l = 0; l < lvs.size(); l++) {
    const Cell& c = cells[lvs[l]];
    if (geom)
      for (int d = 0; d < 3; d++) {
        geom[6 * l + d] = c.loc[d];
        geom[6 * l + 3 + d] = c.width[d];
      }
    if (ints) {
      ints[3 * l] = c.first;
      ints[3 * l + 1] = c.count;
      ints[3 * l + 2] = c.depth;
    }
  }
  return SPHGPU_OK;
}

int sphgpu_set_tuning(sphgpu_space* s, const sphgpu_tuning* t) {
  if (!s || !t) return fail(SPHGPU_EINVAL, "null argument");
  if (!(t->threads_per_particle == 1 || t->threads_per_particle == 2 ||
        t->threads_per_particle == 4) ||
      !(t->jtile == 8 || t->jtile == 16 || t->jtile == 32) ||
      !(t->block_warps == 4 || t->block_warps == 8) ||
      !(t->bulk_stage == 0 || t->bulk_stage == 1) ||
      !(t->row_widen == 0.f || (t->row_widen >= 1.f && t->row_widen <= 4.f)) ||
      !(t->row_cap == 0 || (t->row_cap >= 64 && t->row_cap <= 512 && t->row_cap % 16 == 0)) ||
      !(t->tc_filter == 0 || t->tc_filter == 1))
    return fail(SPHGPU_EINVAL,
                "tuning: threads_per_particle 1, 2 or 4, jtile 8, 16 or 32, block_warps 4 or 8, "
                "bulk_stage 0 or 1, row_widen 0 or in [1, 4], row_cap 0 or a multiple of 16 "
                "in [64, 512], tc_filter 0 or 1");
  return guard([&]() {
    settle(s);
    if (s->dev) CK(cudaStreamSynchronize(s->stream));
    const bool reblock = t->jtile != s->tune.jtile;
    s->tune = *t;
    s->tune.rerun_lists = t->rerun_lists ? 1 : 0;
    drop_graph(s);
    if (s->dev && row_cap(s) != s->rows_cap) alloc_rows(s, s->stream);
    if (reblock) {
      // blocks, candidate lists and every plan referring to them change
      s->space->set_jblock(t->jtile);
      s->task_d.clear();
      s->task_f.clear();
      s->dp_ready = false;
      if (s->dmode) {
        // the steps plan on the device: only the tree's block ranges change
        // (the host's plans are rebuilt when the host planner takes over)
        upload_blocks(s, s->stream);
        dp_upload_tree(s, s->stream);
        s->force_planned = false;
      } else {
        build_plans(s);
        s->force_planned = false;
        if (s->dev) {
          upload_blocks(s, s->stream);
          s->dplan_d.upload(s->plan_d, s->stream);
          s->dplan_s.upload(s->plan_s, s->stream);
          CK(cudaStreamSynchronize(s->stream));
        }
      }
    }
    return SPHGPU_OK;
  });
}

int sphgpu_get_tuning(const sphgpu_space* s, sphgpu_tuning* t) {
  if (!s || !t) return fail(SPHGPU_EINVAL, "null argument");
  *t = s->tune;
  return SPHGPU_OK;
}

int sphgpu_set_active(sphgpu_space* s, int32_t max_active_bin) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  return guard([&]() {
    settle(s);
    if (want_device_plans(s, max_active_bin)) {
      // the steps plan their own lists on the device: nothing to do here
      const auto t0 = std::chrono::steady_clock::now();
      enter_device_mode(s, max_active_bin);
      s->act_plan_ms += std::chrono::duration<double, std::milli>(
                            std::chrono::steady_clock::now() - t0).count();
      if (s->dmode) return SPHGPU_OK;
    }
    leave_device_mode(s);
    host_activate(s, max_active_bin);
    return SPHGPU_OK;
  });
}

namespace {
void launch_step_graphs(sphgpu_space* s, cudaStream_t st) {
  ensure_status_words(s);
  s->h_stale = true;
  const int rounds = std::min(kGraphRounds, s->prm.max_iter);
  if (!s->graph[0]) {
    s->graph[0] = capture(st, [&]() {
      // external event-record nodes: the events can be timed from the host
      enqueue_density(s, st, true);
      CK(cudaEventRecordWithFlags(s->ev[1], st, cudaEventRecordExternal));
      enqueue_ghost_rounds(s, st, 0, rounds);
      CK(cudaEventRecordWithFlags(s->ev[2], st, cudaEventRecordExternal));
      CK(cudaMemsetAsync(s->vflag.p, 0, sizeof(int), st));
      CK(launch_verify_force_plan(s->P, s->chk.p, s->nchk, s->chk_pred.p, s->vflag.p, st));
      enqueue_force(s, st);
    });
    s->step_stats[3]++;
  }
  CK(cudaEventRecord(s->ev[0], st));
  CK(cudaGraphLaunch(s->graph[0], st));
  CK(cudaEventRecord(s->ev[3], st));
  s->step_stats[0]++;
  s->hw[0] = 0;
  if (rounds < s->prm.max_iter) {
    const int* cnt = lists_on(s) ? s->catchup.p + rounds : s->redo.p + rounds - 1;
    CK(cudaMemcpyAsync(s->hw, cnt, sizeof(int), cudaMemcpyDeviceToHost, st));
  }
  CK(cudaMemcpyAsync(s->hw + 1, s->vflag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaEventRecord(s->hw_ev, st));
  s->pending = 1;
}

// After the graph the host reads two words: particles still iterating after
// the graph's rounds (rare: the remaining rounds run here) and the check's
// flag (a decision of the force recursion that the real h changed: the
// lists are re-planned on the host); either way the force runs again on the
// host's plan.  Returns 1 when it enqueued more work.
int finish_step_graphs(sphgpu_space* s, cudaStream_t st) {
  CK(cudaEventSynchronize(s->hw_ev));
  s->pending = 0;
  const int rounds = std::min(kGraphRounds, s->prm.max_iter);
  const int left = s->hw[0], changed = s->hw[1];
  if (left <= 0 && !changed) return 0;
  if (left > 0) {
    enqueue_ghost_rounds(s, st, rounds, s->prm.max_iter);
    s->step_stats[2]++;
  }
  if (changed) s->step_stats[1]++;
  const auto t0 = std::chrono::steady_clock::now();
  plan_force(s, st);  // the real post-ghost h
  s->plan_ms += std::chrono::duration<double, std::milli>(
                    std::chrono::steady_clock::now() - t0).count();
  enqueue_force(s, st);
  CK(cudaEventRecord(s->ev[3], st));
  return 1;
}

// A planned step is one CUDA graph: density, the first kGraphRounds ghost
// rounds, the check of the force plan's decisions against the post-ghost
// h_max, force.  Events ev[0..3] bracket the phases (ev[1], ev[2] are
// event-record nodes inside the graph).
void run_step_graphs(sphgpu_space* s, cudaStream_t st) {
  launch_step_graphs(s, st);
  finish_step_graphs(s, st);
}
}  // namespace

int sphgpu_step(sphgpu_space* s, int32_t stages, void* stream) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  if (stages <= 0 || stages > SPHGPU_STAGE_ALL)
    return fail(SPHGPU_EINVAL, "stages must be a non-empty subset of SPHGPU_STAGE_ALL");
  if ((stages & SPHGPU_STAGE_FORCE) && !(stages & SPHGPU_STAGE_GHOST))
    return fail(SPHGPU_EINVAL, "the force stage needs the ghost stage");
  return guard([&]() {
    settle(s);
    ensure_device(s);
    cudaStream_t st = pick(s, stream);
    if (s->dmode && stages == SPHGPU_STAGE_ALL) {
      if (run_step_device(s, st)) {
        const int rc = check_conv(s, st);  // synchronises the stream
        float ms[3] = {0.f, 0.f, 0.f}, pm[2] = {0.f, 0.f};
        for (int k = 0; k < 3; k++) CK(cudaEventElapsedTime(&ms[k], s->ev[k], s->ev[k + 1]));
        CK(cudaEventElapsedTime(&pm[0], s->pev[0], s->pev[1]));
        CK(cudaEventElapsedTime(&pm[1], s->pev[2], s->pev[3]));
        for (int k = 0; k < 3; k++) s->phase_ms[k] += ms[k];
        s->phase_steps++;
        s->dp_ms += pm[0] + pm[1];
        s->dp_steps++;
        return rc;
      }
    }
    ensure_host_state(s);
    if (stages != SPHGPU_STAGE_ALL) {
      if (stages & SPHGPU_STAGE_GHOST) s->h_stale = true;
      enqueue_density_ghost(s, st, stages);
      if (stages & SPHGPU_STAGE_GHOST) return check_conv(s, st);
      CK(cudaStreamSynchronize(st));
      return SPHGPU_OK;
    }
    if (!s->force_planned) {
      // First step on these plans: the force recursion needs the post-ghost
      // h_max, so density and ghost run, the force loop is planned on the
      // host, then runs; the graphs are captured at the next step.
      s->h_stale = true;
      CK(cudaEventRecord(s->ev[0], st));
      enqueue_density(s, st, true);
      CK(cudaEventRecord(s->ev[1], st));
      enqueue_ghost_rounds(s, st);
      CK(cudaEventRecord(s->ev[2], st));
      int rc = check_conv(s, st);
      if (rc != SPHGPU_OK) return rc;
      const auto t0 = std::chrono::steady_clock::now();
      plan_force(s, st);
      s->plan_ms += std::chrono::duration<double, std::milli>(
                        std::chrono::steady_clock::now() - t0).count();
      CK(cudaEventRecord(s->ev[4], st));
      enqueue_force(s, st);
      CK(cudaEventRecord(s->ev[5], st));
      CK(cudaStreamSynchronize(st));
      float ms[3] = {0.f, 0.f, 0.f};
      CK(cudaEventElapsedTime(&ms[0], s->ev[0], s->ev[1]));
      CK(cudaEventElapsedTime(&ms[1], s->ev[1], s->ev[2]));
      CK(cudaEventElapsedTime(&ms[2], s->ev[4], s->ev[5]));
      for (int k = 0; k < 3; k++) s->phase_ms[k] += ms[k];
      s->phase_steps++;
      return SPHGPU_OK;
    }
    run_step_graphs(s, st);
    const int rc = check_conv(s, st);  // synchronises the stream
    for (int k = 0; k < 3; k++) {
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, s->ev[k], s->ev[k + 1]));
      s->phase_ms[k] += ms;
    }
    s->phase_steps++;
    return rc;
  });
}

int sphgpu_download(sphgpu_space* s, float* fields, int32_t* ints) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  if (!s->dev) return fail(SPHGPU_ESTATE, "no step has run on this space");
  return guard([&]() {
    settle(s);
    const int n = s->P.n;
    cudaStream_t st = s->stream;
    // device destinations are written in place; host ones through a
    // device buffer (unified addressing for the copies)
    auto on_device = [](const void* p) {
      cudaPointerAttributes at{};
      if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
      }
      return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
    };
    const bool fdev = fields && on_device(fields), idev = ints && on_device(ints);
    DBuf<float> df;
    DBuf<int32_t> di;
    if (fields && !fdev) df.alloc(24 * (size_t)n);
    if (ints && !idev) di.alloc(4 * (size_t)n);
    CK(cudaStreamSynchronize(st));
    CK(launch_collect_out(s->P, s->perm.p, fields ? (fdev ? fields : df.p) : nullptr,
                          ints ? (idev ? ints : di.p) : nullptr, st));
    if (fields && !fdev)
      CK(cudaMemcpyAsync(fields, df.p, sizeof(float) * 24 * (size_t)n, cudaMemcpyDefault, st));
    if (ints && !idev)
      CK(cudaMemcpyAsync(ints, di.p, sizeof(int32_t) * 4 * (size_t)n, cudaMemcpyDefault, st));
    CK(cudaStreamSynchronize(st));
    return SPHGPU_OK;
  });
}

int sphgpu_download_min_ngb_bin(sphgpu_space* s, int8_t* out) {
  if (!s || !out) return fail(SPHGPU_EINVAL, "null argument");
  if (!s->dev) return fail(SPHGPU_ESTATE, "no step has run on this space");
  return guard([&]() {
    settle(s);
    const int n = s->P.n;
    std::vector<int8_t> st_order(n);
    CK(cudaStreamSynchronize(s->stream));
    CK(cudaMemcpy(st_order.data(), s->ngb_bin.p, n, cudaMemcpyDeviceToHost));
    const auto& gperm = s->space->gperm();
    for (int g = 0; g < n; g++) out[gperm[g]] = st_order[g];
    return SPHGPU_OK;
  });
}

int sphgpu_step_host(sphgpu_space* s, const double* x, const float* v,
                     const float* m, const float* h, const float* u,
                     float* fields, void* stream) {
  if (!s || !x || !v || !m || !h || !u) return fail(SPHGPU_EINVAL, "null argument");
  return guard([&]() {
    settle(s);
    ensure_device(s);
    cudaStream_t st = pick(s, stream);
    const int n = s->P.n;
    ensure_stage(s, st);
    CK(cudaMemcpyAsync(s->x_stage.p, x, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(s->v_stage.p, v, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(s->m_stage.p, m, sizeof(float) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(s->h_stage.p, h, sizeof(float) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(s->u_stage.p, u, sizeof(float) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(s->differ.p, 0, sizeof(int), st));
    CK(launch_permute_in(s->P, s->perm.p, s->x_stage.p, s->x_ref.p, s->v_stage.p,
                         s->m_stage.p, s->h_stage.p, s->u_stage.p, s->differ.p, st));
    int differ = 0;
    CK(cudaMemcpyAsync(&differ, s->differ.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (differ) {
      // moved particles: a drift without a rebuild, if the tree allows it
      const int rc = drift_space(s, st);
      if (rc != SPHGPU_OK) return rc;
    }
    const int rc = sphgpu_step(s, SPHGPU_STAGE_ALL, (void*)st);
    if (rc != SPHGPU_OK && rc != SPHGPU_ENOCONV) return rc;
    if (fields) {
      CK(launch_collect_out(s->P, s->perm.p, s->out_stage.p, nullptr, st));
      CK(cudaMemcpyAsync(fields, s->out_stage.p, sizeof(float) * 24 * (size_t)n,
                         cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
    }
    if (rc == SPHGPU_ENOCONV) return fail(rc, g_err);
    return SPHGPU_OK;
  });
}

int sphgpu_space_update(sphgpu_space* s, const float* v, const float* m, const float* u,
                        void* stream) {
  if (!s || !v || !m || !u) return fail(SPHGPU_EINVAL, "null argument");
  const int n = s->space->n();
  for (int k = 0; k < n; k++)
    if (!(m[k] > 0.f) || !std::isfinite(m[k]) || !std::isfinite(u[k]) ||
        !std::isfinite(v[3 * (size_t)k]) || !std::isfinite(v[3 * (size_t)k + 1]) ||
        !std::isfinite(v[3 * (size_t)k + 2]))
      return fail(SPHGPU_EINVAL, "sphgpu_space_update: non-finite v or u, or mass <= 0 "
                                 "(particle " + std::to_string(k) + ")");
  return guard([&]() {
    settle(s);
    // the host copies feed the next upload (first GPU call, re-plans)
    s->v_in.assign(v, v + 3 * (size_t)n);
    s->m_in.assign(m, m + n);
    s->u_in.assign(u, u + n);
    ensure_device(s);
    cudaStream_t st = pick(s, stream);
    if (!s->v_stage.p) {
      s->v_stage.alloc(3 * (size_t)n);
      s->m_stage.alloc(n);
      s->u_stage.alloc(n);
    }
    CK(cudaMemcpyAsync(s->v_stage.p, v, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(s->m_stage.p, m, sizeof(float) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(s->u_stage.p, u, sizeof(float) * n, cudaMemcpyHostToDevice, st));
    CK(launch_permute_vmu_in(s->P, s->perm.p, s->v_stage.p, s->m_stage.p, s->u_stage.p, st));
    CK(cudaStreamSynchronize(st));
    return SPHGPU_OK;
  });
}

namespace {
// Wait for a slot's step to come back: its results are in the caller's
// buffer, and its status is read.
int finish_slot(sphgpu_space* s, int b) {
  auto& S = s->slot[b];
  if (!S.busy) return SPHGPU_OK;
  CK(cudaEventSynchronize(S.out_done));
  S.busy = false;
  if (S.hflags[0])
    return fail(SPHGPU_EINVAL,
                "sphgpu_step_host_async: positions or smoothing lengths differ from the "
                "space's; move them with sphgpu_space_drift (or sphgpu_step_host) first");
  if (S.hflags[1] > 0)
    return fail(SPHGPU_ENOCONV, "smoothing length failed to converge on " +
                                    std::to_string(S.hflags[1]) + " particles");
  return SPHGPU_OK;
}
}  // namespace

namespace {
// The results of a slot's step: collected into the caller's order and
// copied down behind it.
void enqueue_slot_out(sphgpu_space* s, int b, cudaStream_t st) {
  auto& S = s->slot[b];
  CK(cudaMemcpyAsync(S.dflags.p + 1, s->redo.p + s->prm.max_iter - 1, sizeof(int),
                     cudaMemcpyDeviceToDevice, st));
  CK(launch_collect_out(s->P, s->perm.p, S.out.p, nullptr, st));
  CK(cudaEventRecord(S.comp_done, st));
  CK(cudaStreamWaitEvent(s->cout, S.comp_done, 0));
  CK(cudaMemcpyAsync(S.fields, S.out.p, sizeof(float) * 24 * (size_t)s->P.n,
                     cudaMemcpyDeviceToHost, s->cout));
  CK(cudaMemcpyAsync(S.hflags, S.dflags.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, s->cout));
  CK(cudaEventRecord(S.out_done, s->cout));
}

// The pipelined step still in flight: read its status words and run what
// it still needs (late ghost rounds, a force re-planned on the host, larger
// device-plan buffers, or the whole step on the host's plans), then copy its
// results again.  Its slot stays the caller's until a later call or the wait
// finishes it, so the corrected results land before anyone reads them.
void settle(sphgpu_space* s) {
  if (!s->pending) return;
  cudaStream_t st = s->stream;
  int more = s->pending == 1 ? finish_step_graphs(s, st) : finish_step_device(s, st);
  if (more < 0) {
    run_step_graphs(s, st);
    more = 1;
  }
  const int b = s->pending_slot;
  s->pending_slot = -1;
  if (more && b >= 0) enqueue_slot_out(s, b, st);
}
}  // namespace

int sphgpu_step_host_async(sphgpu_space* s, const double* x, const float* v, const float* m,
                           const float* h, const float* u, float* fields) {
  if (!s || !x || !v || !m || !h || !u || !fields) return fail(SPHGPU_EINVAL, "null argument");
  return guard([&]() {
    ensure_device(s);
    if (!s->force_planned) {
      // the first step plans the force lists on the host: run it whole
      int rc = sphgpu_step_host_wait(s);
      if (rc != SPHGPU_OK) return rc;
      return sphgpu_step_host(s, x, v, m, h, u, fields, nullptr);
    }
    const int n = s->P.n;
    if (!s->cin) {
      CK(cudaStreamCreateWithFlags(&s->cin, cudaStreamNonBlocking));
      CK(cudaStreamCreateWithFlags(&s->cout, cudaStreamNonBlocking));
      for (auto& S : s->slot) {
        S.x.alloc(3 * (size_t)n);
        S.v.alloc(3 * (size_t)n);
        S.m.alloc(n);
        S.h.alloc(n);
        S.u.alloc(n);
        S.out.alloc(24 * (size_t)n);
        S.dflags.alloc(2);
        CK(cudaMallocHost(&S.hflags, 2 * sizeof(int)));
        for (cudaEvent_t* e : {&S.in_done, &S.comp_done, &S.out_done})
          CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
      }
      if (!s->x_ref.p) s->x_ref.upload(s->x_in.data(), s->x_in.size(), s->stream);
    }
    const int b = (int)(s->async_k & 1);
    auto& S = s->slot[b];
    // the step that used this slot two calls ago must be back first
    int rc = finish_slot(s, b);
    if (rc != SPHGPU_OK) return rc;
    // inputs up, while the previous step still computes
    CK(cudaMemcpyAsync(S.x.p, x, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s->cin));
    CK(cudaMemcpyAsync(S.v.p, v, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, s->cin));
    CK(cudaMemcpyAsync(S.m.p, m, sizeof(float) * n, cudaMemcpyHostToDevice, s->cin));
    CK(cudaMemcpyAsync(S.h.p, h, sizeof(float) * n, cudaMemcpyHostToDevice, s->cin));
    CK(cudaMemcpyAsync(S.u.p, u, sizeof(float) * n, cudaMemcpyHostToDevice, s->cin));
    CK(cudaEventRecord(S.in_done, s->cin));
    // the previous step's status (the host waits for it here, with these
    // inputs already on their way), then this step
    settle(s);
    cudaStream_t st = s->stream;
    CK(cudaStreamWaitEvent(st, S.in_done, 0));
    CK(cudaMemsetAsync(S.dflags.p, 0, 2 * sizeof(int), st));
    CK(launch_permute_in(s->P, s->perm.p, S.x.p, s->x_ref.p, S.v.p, S.m.p, S.h.p, S.u.p,
                         S.dflags.p, st));
    if (s->dmode)
      launch_step_device(s, st);
    else
      launch_step_graphs(s, st);
    s->pending_slot = b;
    // results down (overlaps the next step)
    S.fields = fields;
    enqueue_slot_out(s, b, st);
    S.busy = true;
    s->async_k++;
    return SPHGPU_OK;
  });
}

int sphgpu_step_host_wait(sphgpu_space* s) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  return guard([&]() {
    settle(s);
    // oldest first
    const int b0 = (int)(s->async_k & 1);
    int rc = finish_slot(s, b0);
    const int rc1 = finish_slot(s, 1 - b0);
    return rc != SPHGPU_OK ? rc : rc1;
  });
}

int sphgpu_force_from_state(sphgpu_space* s, const float* h, const float* rho,
                            const float* f, const float* pressure,
                            const float* soundspeed, const float* balsara,
                            void* stream) {
  if (!s || !h || !rho || !f || !pressure || !soundspeed || !balsara)
    return fail(SPHGPU_EINVAL, "null argument");
  return guard([&]() {
    settle(s);
    ensure_device(s);
    ensure_host_state(s);
    cudaStream_t st = pick(s, stream);
    const int n = s->P.n;
    const auto& gperm = s->space->gperm();
    std::vector<float4> ph(n), f0(n), acc(n, make_float4(0, 0, 0, 0));
    std::vector<float2> f1(n), hv(n);
    std::vector<float> hs(n);  // reference sorted order
    CK(cudaStreamSynchronize(st));
    CK(cudaMemcpyAsync(ph.data(), s->posh.p, sizeof(float4) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    for (int g = 0; g < n; g++) {
      const int k = gperm[g];
      ph[g].w = h[k];
      hs[s->s_of_g[g]] = h[k];
      f0[g] = make_float4(rho[k], f[k], pressure[k] / (rho[k] * rho[k]), soundspeed[k]);
      f1[g] = make_float2(balsara[k], pressure[k]);
      hv[g] = make_float2(0.f, 2.f * soundspeed[k]);
    }
    s->posh.upload(ph.data(), n, st);
    s->fin0.upload(f0.data(), n, st);
    s->fin1.upload(f1.data(), n, st);
    s->acc.upload(acc.data(), n, st);
    s->hdt_vsig.upload(hv.data(), n, st);
    // depth_h from the given h (cell_set_part_h_depth on the leaf chain)
    s->space->update_h_after_ghost(hs.data());
    std::vector<LeafInfo> li;
    s->space->leaf_infos(li);
    std::vector<int8_t> dh(n);
    for (int g = 0; g < n; g++) {
      const int srt = s->s_of_g[g];
      const LeafInfo& L = li[s->space->leaf_of()[srt]];
      const float hh = hs[srt];
      dh[g] = s->space->depth_h()[srt];
      if (hh < L.hmin[0]) {
        dh[g] = L.depth[0];
      } else {
        for (int lev = 0; lev < L.nlevels; lev++)
          if (hh >= L.hmin[lev] && hh < L.hmax[lev]) {
            dh[g] = L.depth[lev];
            break;
          }
      }
    }
    s->depth_h.upload(dh.data(), n, st);
    Plan pf;
    s->space->plan_density(pf, true);
    DevPlan dp;
    dp.upload(pf, st);
    CK(launch_block_hmax(s->bb_fc.p, s->bb_lo.p, s->posh.p, s->bb_n, st));
    enqueue_gather(s, st, dp, 3, MODE_FIRST, true, 1, nullptr);
    CK(cudaStreamSynchronize(st));
    // the step's plans assume its own ghost: re-plan on the next step
    s->force_planned = false;
    drop_graph(s);
    return SPHGPU_OK;
  });
}

static void build_sort_tree(sphgpu_space* s, cudaStream_t st) {
  const Space& sp = *s->space;
  const auto& cells = sp.cells();
  const int nc = (int)cells.size();
  s->sc_of_cell.assign(nc, -1);
  s->sc_host.clear();
  long long off = 0;
  int maxd = 0;
  for (int c = 0; c < nc; c++) {
    if (cells[c].count == 0) continue;
    s->sc_of_cell[c] = (int)s->sc_host.size();
    SortCell sc;
    sc.off = off;
    sc.first = cells[c].first;
    sc.count = cells[c].count;
    for (int k = 0; k < 8; k++) sc.progeny[k] = -1;
    s->sc_host.push_back(sc);
    off += 13LL * (cells[c].count + 1);
    maxd = std::max(maxd, cells[c].depth);
  }
  std::vector<int> leaves;
  std::vector<std::vector<int>> split(maxd + 1);
  for (int c = 0; c < nc; c++) {
    const int k = s->sc_of_cell[c];
    if (k < 0) continue;
    if (cells[c].split) {
      for (int q = 0; q < 8; q++) {
        const int p = cells[c].progeny[q];
        if (p >= 0) s->sc_host[k].progeny[q] = s->sc_of_cell[p];
      }
      split[cells[c].depth].push_back(k);
    } else {
      leaves.push_back(k);
    }
  }
  std::vector<int> sids;
  s->split_begin.assign(maxd + 1, 0);
  s->split_n.assign(maxd + 1, 0);
  for (int d = 0; d <= maxd; d++) {
    s->split_begin[d] = (int)sids.size();
    s->split_n[d] = (int)split[d].size();
    sids.insert(sids.end(), split[d].begin(), split[d].end());
  }
  s->sort_cells.upload(s->sc_host.data(), s->sc_host.size(), st);
  s->sort_leaf_ids.upload(leaves.data(), leaves.size(), st);
  s->sort_split_ids.upload(sids.data(), sids.size(), st);
  const auto& gos = sp.gpu_of_sorted();
  s->g_of_s_dev.upload(gos.data(), gos.size(), st);
  s->sort_d.alloc(std::max<long long>(off, 1));
  s->sort_i.alloc(std::max<long long>(off, 1));
  s->sort_nleaves = (int)leaves.size();
  s->sort_max_depth = maxd;
  CK(cudaStreamSynchronize(st));
}

int sphgpu_hydro_sort(sphgpu_space* s, int32_t flags, void* stream) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  if (flags <= 0 || flags > 0x1FFF) return fail(SPHGPU_EINVAL, "flags: a non-empty set of the 13 axes");
  return guard([&]() {
    settle(s);
    ensure_device(s);
    cudaStream_t st = pick(s, stream);
    if (!s->sort_cells.p) build_sort_tree(s, st);
    SortTree t;
    t.cells = s->sort_cells.p;
    t.leaves = s->sort_leaf_ids.p;
    t.nleaves = s->sort_nleaves;
    t.g_of_s = s->g_of_s_dev.p;
    t.xd = s->xd.p;
    t.d = s->sort_d.p;
    t.i = s->sort_i.p;
    std::vector<const int*> by_depth(s->sort_max_depth + 1);
    for (int d = 0; d <= s->sort_max_depth; d++)
      by_depth[d] = s->sort_split_ids.p + s->split_begin[d];
    CK(launch_hydro_sort(t, by_depth.data(), s->split_n.data(), s->sort_max_depth, flags, st));
    s->sorted_mask |= flags;
    return SPHGPU_OK;
  });
}

int sphgpu_space_tree(const sphgpu_space* s, int32_t* ncells, int32_t* records) {
  if (!s || !ncells) return fail(SPHGPU_EINVAL, "null argument");
  const auto& cells = s->space->cells();
  *ncells = (int32_t)cells.size();
  if (records)
    for (size_t c = 0; c < cells.size(); c++) {
      int32_t* r = records + 5 * c;
      r[0] = cells[c].first;
      r[1] = cells[c].count;
      r[2] = cells[c].depth;
      r[3] = cells[c].parent;
      r[4] = cells[c].top;
    }
  return SPHGPU_OK;
}

int sphgpu_cell_sort(sphgpu_space* s, int32_t cell, int32_t axis, float* d, int32_t* idx) {
  if (!s || !d || !idx) return fail(SPHGPU_EINVAL, "null argument");
  if (axis < 0 || axis >= 13) return fail(SPHGPU_EINVAL, "axis out of range");
  if (!(s->sorted_mask & (1 << axis))) return fail(SPHGPU_ESTATE, "axis not sorted");
  if (cell < 0 || cell >= (int32_t)s->sc_of_cell.size() || s->sc_of_cell[cell] < 0)
    return fail(SPHGPU_EINVAL, "not a non-empty cell");
  return guard([&]() {
    const SortCell& c = s->sc_host[s->sc_of_cell[cell]];
    const long long o = c.off + (long long)axis * (c.count + 1);
    CK(cudaStreamSynchronize(s->stream));
    CK(cudaDeviceSynchronize());
    CK(cudaMemcpy(d, s->sort_d.p + o, sizeof(float) * (c.count + 1), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(idx, s->sort_i.p + o, sizeof(int32_t) * (c.count + 1), cudaMemcpyDeviceToHost));
    return SPHGPU_OK;
  });
}

int sphgpu_autotune(sphgpu_space* s, int32_t reps, sphgpu_tuning* best, float ms[24],
                    int32_t* ncand) {
  if (!s || !best || !ms || !ncand || reps < 1)
    return fail(SPHGPU_EINVAL, "sphgpu_autotune: null argument or reps < 1");
  const int jt[3] = {32, 16, 8}, bw[2] = {8, 4};
  float best_ms = 3.4e38f;
  sphgpu_tuning bt = s->tune;
  // the fastest shape with one and with two lanes per particle
  float lane_ms[2] = {3.4e38f, 3.4e38f};
  sphgpu_tuning lane_bt[2] = {s->tune, s->tune};
  int k = 0;
  auto time_it = [&](const sphgpu_tuning& t, float* out) {
    int rc = sphgpu_set_tuning(s, &t);
    if (rc) return rc;
    rc = sphgpu_step(s, SPHGPU_STAGE_ALL, nullptr);  // plan + capture + warm
    if (rc) return rc;
    double sum[3];
    int64_t n = 0;
    sphgpu_phase_times(s, sum, &n, 1);
    for (int r = 0; r < reps; r++) {
      rc = sphgpu_step(s, SPHGPU_STAGE_ALL, nullptr);
      if (rc) return rc;
    }
    sphgpu_phase_times(s, sum, &n, 1);
    *out = (float)((sum[0] + sum[1] + sum[2]) / std::max<int64_t>(1, n));
    return (int)SPHGPU_OK;
  };
  // j-tile outermost: only a new j-tile re-plans the blocks
  for (int a = 0; a < 3; a++)
    for (int c = 0; c < 4; c++, k++) {
      sphgpu_tuning t{1 + (c >> 1), jt[a], s->tune.rerun_lists, bw[c & 1],
                      s->tune.bulk_stage, s->tune.row_widen, s->tune.row_cap,
                      s->tune.tc_filter};
      const int rc = time_it(t, &ms[k]);
      if (rc) return rc;
      if (ms[k] < best_ms) {
        best_ms = ms[k];
        bt = t;
      }
      if (ms[k] < lane_ms[c >> 1]) {
        lane_ms[c >> 1] = ms[k];
        lane_bt[c >> 1] = t;
      }
    }
  // then the rows' radius for the fastest shape of each lane count: wider
  // rows cover more of the ghost's iterates and of the force's partners on
  // boxes where h moves far from its input, at the price of recording and
  // reading more items (and with them the cheaper lane count can change)
  if (s->lists && s->tune.rerun_lists) {
    const float widen[4] = {1.32f, 1.44f, 1.56f, 1.69f};
    for (int l = 0; l < 2; l++)
      for (int w = 0; w < 4 && k < 24; w++, k++) {
        sphgpu_tuning t = lane_bt[l];
        t.row_widen = widen[w];
        const int rc = time_it(t, &ms[k]);
        if (rc) return rc;
        if (ms[k] < best_ms) {
          best_ms = ms[k];
          bt = t;
        }
      }
  }
  *ncand = k;
  const int rc = sphgpu_set_tuning(s, &bt);
  if (rc) return rc;
  *best = bt;
  return SPHGPU_OK;
}

int sphgpu_step_stats(sphgpu_space* s, int64_t out[4], int32_t reset) {
  if (!s || !out) return fail(SPHGPU_EINVAL, "null argument");
  for (int k = 0; k < 4; k++) out[k] = s->step_stats[k];
  if (reset)
    for (int k = 0; k < 4; k++) s->step_stats[k] = 0;
  return SPHGPU_OK;
}

int sphgpu_space_drift(sphgpu_space* s, const double* x, const float* h, void* stream) {
  if (!s || !x || !h) return fail(SPHGPU_EINVAL, "null argument");
  return guard([&]() {
    settle(s);
    ensure_device(s);
    cudaStream_t st = pick(s, stream);
    const int n = s->P.n;
    ensure_stage(s, st);
    // host or device memory (unified addressing)
    CK(cudaMemcpyAsync(s->x_stage.p, x, sizeof(double) * 3 * (size_t)n, cudaMemcpyDefault, st));
    CK(cudaMemcpyAsync(s->h_stage.p, h, sizeof(float) * n, cudaMemcpyDefault, st));
    return drift_space(s, st);
  });
}

int sphgpu_space_set_state(sphgpu_space* s, const float* v, const float* m, const float* u,
                           const float* rho, const float* f, const float* pressure,
                           const float* soundspeed, const float* balsara,
                           const int8_t* time_bin, void* stream) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  if ((rho != nullptr) != (pressure != nullptr) || (rho != nullptr) != (soundspeed != nullptr))
    return fail(SPHGPU_EINVAL, "sphgpu_space_set_state: rho, pressure and soundspeed go together");
  return guard([&]() {
    settle(s);
    ensure_device(s);
    cudaStream_t st = pick(s, stream);
    const int n = s->P.n;
    ensure_stage(s, st);
    // staged (host or device sources); the density state in out_stage
    auto stage = [&](auto* dst, const auto* src, size_t count) -> decltype(dst) {
      if (!src) return nullptr;
      CK(cudaMemcpyAsync(dst, src, sizeof(*src) * count, cudaMemcpyDefault, st));
      return dst;
    };
    const float* dv = stage(s->v_stage.p, v, 3 * (size_t)n);
    const float* dm = stage(s->m_stage.p, m, n);
    const float* du = stage(s->u_stage.p, u, n);
    float* o = s->out_stage.p;
    const float* dr = stage(o, rho, n);
    const float* dp = stage(o + n, pressure, n);
    const float* dc = stage(o + 2 * (size_t)n, soundspeed, n);
    const float* df = stage(o + 3 * (size_t)n, f, n);
    const float* dbs = stage(o + 4 * (size_t)n, balsara, n);
    const int8_t* db = nullptr;
    if (time_bin) {
      if (s->tb_stage.n < (size_t)n) s->tb_stage.alloc(n);
      db = stage(s->tb_stage.p, time_bin, n);
    }
    CK(launch_set_state(s->P, s->perm.p, dv, dm, du, dr, df, dp, dc, dbs, db, s->tbin.p, st));
    if (time_bin) {
      // the bins are the caller's from now on: any activation may be sparse,
      // and the force loops keep the limiter's neighbour bin
      s->max_bin = SPH_NUM_TIME_BINS + 1;
      s->bins_host_stale = true;
      if (s->P.tbin != s->tbin.p) {
        s->P.tbin = s->tbin.p;
        drop_graph(s);  // the captured kernels hold the particle view
      }
    }
    CK(cudaStreamSynchronize(st));
    return SPHGPU_OK;
  });
}

int sphgpu_set_device_planning(sphgpu_space* s, int32_t on) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  return guard([&]() {
    if (on) {
      s->dp_off_by_caller = false;
    } else {
      s->dp_off_by_caller = true;
      ensure_host_state(s);
    }
    return SPHGPU_OK;
  });
}

int sphgpu_plan_times(sphgpu_space* s, double* ms, int64_t* steps, int32_t reset) {
  if (!s || !ms || !steps) return fail(SPHGPU_EINVAL, "null argument");
  *ms = s->dp_ms;
  *steps = s->dp_steps;
  if (reset) {
    s->dp_ms = 0;
    s->dp_steps = 0;
  }
  return SPHGPU_OK;
}

int sphgpu_check_device_plans(sphgpu_space* s, int64_t out[6]) {
  if (!s || !out) return fail(SPHGPU_EINVAL, "null argument");
  if (!s->dmode || !s->force_planned)
    return fail(SPHGPU_ESTATE, "sphgpu_check_device_plans: no device-planned step has run "
                               "since the last activation");
  return guard([&]() {
    cudaStream_t st = s->stream;
    const int n = s->P.n;
    Space& sp = *s->space;
    const size_t nl = sp.leaves().size();
    std::vector<float> hw(n), h0(n), hpre(n);
    std::vector<uint8_t> fl(n);
    int status[8];
    CK(cudaStreamSynchronize(st));
    CK(cudaMemcpy2DAsync(hw.data(), sizeof(float), reinterpret_cast<const char*>(s->posh.p) + 12,
                         sizeof(float4), sizeof(float), n, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(h0.data(), s->h0.p, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(fl.data(), s->flags.p, n, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(status, s->dp_status.p, sizeof(status), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    // the step's starting h: the active particles restarted from h0
    for (int g = 0; g < n; g++) hpre[s->s_of_g[g]] = (fl[g] & 1) ? h0[g] : hw[g];
    sync_host_drift(s);  // the cells' dx_max and the active particles' starting h
    sync_host_bins(s);
    sp.assign_h(hpre.data());
    sp.set_activity(s->dp_bin);
    sp.refresh_all();
    Plan host[3];
    sp.plan_density(host[0], false);
    sp.plan_subset(host[1]);
    // the ghost's growth of the cells' h_max with the active particles' new h
    const auto& al = sp.active_list();
    const auto& gos = sp.gpu_of_sorted();
    std::vector<float> hact(al.size());
    for (size_t a = 0; a < al.size(); a++) hact[a] = hw[gos[al[a]]];
    sp.update_h_active(hact.data());
    sp.plan_density(host[2], true);
    s->host_refresh = true;  // the planner's cells hold this check's state now
    for (int k = 0; k < 3; k++) {
      const DevPlan& dp = dp_plan_of(s, k);
      const long long ne = std::min<long long>(status[1 + 2 * k], dp.entries.n);
      const long long np =
          std::min<long long>(status[2 + 2 * k], std::min(dp.pb.n, dp.pe.n));
      std::vector<int32_t> lpb(nl + 1), pb(np), pe(np);
      std::vector<Entry> en(ne);
      CK(cudaMemcpy(lpb.data(), dp.lpb.p, sizeof(int32_t) * (nl + 1), cudaMemcpyDeviceToHost));
      if (np) {
        CK(cudaMemcpy(pb.data(), dp.pb.p, sizeof(int32_t) * np, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(pe.data(), dp.pe.p, sizeof(int32_t) * np, cudaMemcpyDeviceToHost));
      }
      if (ne) CK(cudaMemcpy(en.data(), dp.entries.p, sizeof(Entry) * ne, cudaMemcpyDeviceToHost));
      const Plan& h = host[k];
      long long bad = 0;
      for (size_t l = 0; l < nl; l++) {
        const int hb = h.leaf_pair_begin[l], he = h.leaf_pair_begin[l + 1];
        const int db = lpb[l], de = lpb[l + 1];
        if (he - hb != de - db) {
          bad += std::max(he - hb, de - db);
          continue;
        }
        for (int w = 0; w < he - hb; w++) {
          const int dw = db + w;
          if (dw < 0 || dw >= np || pe[dw] < 0 || pe[dw] >= ne || pb[dw] != h.pair_block[hb + w] ||
              std::memcmp(&en[pe[dw]], &h.entries[h.pair_entry[hb + w]], sizeof(Entry)) != 0)
            bad++;
        }
      }
      out[k] = bad;
      out[3 + k] = np;
    }
    return SPHGPU_OK;
  });
}

int sphgpu_host_times(sphgpu_space* s, double ms[3], int32_t reset) {
  if (!s || !ms) return fail(SPHGPU_EINVAL, "null argument");
  ms[0] = s->act_plan_ms;
  ms[1] = s->act_upload_ms;
  ms[2] = s->plan_ms;
  if (reset) s->act_plan_ms = s->act_upload_ms = s->plan_ms = 0;
  return SPHGPU_OK;
}

int sphgpu_phase_times(sphgpu_space* s, double ms_sum[3], int64_t* steps,
                       int32_t reset) {
  if (!s || !ms_sum || !steps) return fail(SPHGPU_EINVAL, "null argument");
  for (int k = 0; k < 3; k++) ms_sum[k] = s->phase_ms[k];
  *steps = s->phase_steps;
  if (reset) {
    for (int k = 0; k < 3; k++) s->phase_ms[k] = 0;
    s->phase_steps = 0;
  }
  return SPHGPU_OK;
}

int sphgpu_count_hits(sphgpu_space* s, int64_t hits[4]) {
  if (!s || !hits) return fail(SPHGPU_EINVAL, "null argument");
  return guard([&]() {
    settle(s);
    ensure_device(s);
    cudaStream_t st = s->stream;
    int rc = SPHGPU_OK;
    if (!s->force_planned) rc = sphgpu_step(s, SPHGPU_STAGE_ALL, st);
    if (rc != SPHGPU_OK) return rc;
    CK(cudaMemsetAsync(s->hit_ctr.p, 0, 4 * sizeof(unsigned long long), st));
    s->count_hits = true;
    try {
      enqueue_density_ghost(s, st, SPHGPU_STAGE_DENSITY | SPHGPU_STAGE_GHOST);
      enqueue_force(s, st);
    } catch (...) {
      s->count_hits = false;
      throw;
    }
    s->count_hits = false;
    CK(launch_sum_active_ngb(s->P, s->hit_ctr.p + 3, st));
    rc = check_conv(s, st);
    unsigned long long h[4];
    CK(cudaMemcpy(h, s->hit_ctr.p, sizeof(h), cudaMemcpyDeviceToHost));
    for (int k = 0; k < 4; k++) hits[k] = (int64_t)h[k];
    return rc;
  });
}

int sphgpu_density_noalloc(sphgpu_space* s, float* d_fields, int32_t* d_ngb,
                           void* stream) {
  if (!s || !d_fields || !d_ngb)
    return fail(SPHGPU_EINVAL, "sphgpu_density_noalloc: null argument");
  if (!s->dev)
    return fail(SPHGPU_ESTATE,
                "sphgpu_density_noalloc: the space is not resident on the device "
                "yet; run one GPU call on it first (that call allocates)");
  if (s->P.n > noalloc_max_particles())
    return fail(SPHGPU_EINVAL,
                "sphgpu_density_noalloc: " + std::to_string(s->P.n) +
                    " particles exceed the static scratch limit of " +
                    std::to_string(noalloc_max_particles()));
  if (s->max_units > noalloc_max_units())
    return fail(SPHGPU_EINVAL,
                "sphgpu_density_noalloc: " + std::to_string(s->max_units) +
                    " particle windows exceed the static scratch limit of " +
                    std::to_string(noalloc_max_units()));
  const cudaError_t e = launch_density_noalloc(
      gargs(s, s->dplan_d, 0, MODE_FIRST), s->leaves.p,
      (int)s->space->leaves().size(), s->leaf_window_begin.p, s->max_units,
      s->dplan_d.lpb.p, d_fields, d_ngb, s->perm.p, s->num_sms, pick(s, stream));
  if (e != cudaSuccess)
    return fail(SPHGPU_ECUDA, std::string("sphgpu_density_noalloc: ") +
                                  cudaGetErrorString(e));
  return SPHGPU_OK;
}

// ---------------------------------------------------------------------------
// Plain per-task form: one launch per reference task, as runner_main.c would
// issue them (self/pair density, per-top-cell ghost, self/pair force).

static void ensure_task_plans(sphgpu_space* s, bool force) {
  auto& plans = force ? s->task_f : s->task_d;
  if (!plans.empty()) return;
  // One concatenated entry array for all tasks; each task's work is a list
  // of (particle, entry range) items over the leaves the task touches.
  const Space& sp = *s->space;
  const auto& tasks = sp.tasks();
  plans.resize(tasks.size());
  std::vector<Item> items;
  std::vector<Entry> all_entries;
  std::vector<int4> all_units;
  std::vector<int> all_pb, all_pe;
  std::vector<int> ib(tasks.size() + 1, 0);
  const auto& cells = sp.cells();
  const auto& lvs = sp.leaves();
  const auto& active = sp.active();
  std::vector<std::vector<Entry>> per_leaf(lvs.size());
  std::vector<int> touched;
  // leaves are numbered top cell by top cell
  const int ntop = sp.cdim()[0] * sp.cdim()[1] * sp.cdim()[2];
  std::vector<int> top_leaf(ntop + 1, (int)lvs.size());
  for (int l = (int)lvs.size() - 1; l >= 0; l--) top_leaf[cells[lvs[l]].top] = l;
  for (int t = ntop - 1; t >= 0; t--)
    if (top_leaf[t] > top_leaf[t + 1]) top_leaf[t] = top_leaf[t + 1];
  for (size_t t = 0; t < tasks.size(); t++) {
    items.clear();
    if (tasks[t].cj < 0)
      sp.dosub_self(items, tasks[t].ci, 0, force);
    else
      sp.dosub_pair(items, tasks[t].ci, tasks[t].cj, 0, force);
    sp.items_to_entries(items, per_leaf);
    ib[t] = (int)all_units.size();
    touched.clear();
    // leaves touched by this task: those of its cells whose list is non-empty
    const int ci = tasks[t].ci, cj = tasks[t].cj;
    for (int c : {ci, cj}) {
      if (c < 0) continue;
      for (int l = top_leaf[c]; l < top_leaf[c + 1]; l++)
        if (!per_leaf[l].empty()) touched.push_back(l);
    }
    for (int l : touched) {
      const int pb0 = (int)all_pb.size();
      for (const Entry& E : per_leaf[l]) {
        const int e = (int)all_entries.size();
        all_entries.push_back(E);
        for (int b = E.bfirst; b < E.bfirst + E.bcount; b++) {
          all_pb.push_back(b);
          all_pe.push_back(e);
        }
      }
      const int pb1 = (int)all_pb.size();
      per_leaf[l].clear();
      const Cell& c = cells[lvs[l]];
      for (int w0 = c.first; w0 < c.first + c.count; w0 += 32) {
        unsigned m = 0;
        for (int q = 0; q < 32 && w0 + q < c.first + c.count; q++)
          if (active[s->s_of_g[w0 + q]]) m |= 1u << q;
        if (m) all_units.push_back(make_int4(w0, (int)m, pb0, pb1));
      }
    }
  }
  ib[tasks.size()] = (int)all_units.size();
  auto& di = force ? s->task_units_f : s->task_units_d;
  auto& de = force ? s->task_entries_f : s->task_entries_d;
  di.upload(all_units.data(), all_units.size(), s->stream);
  de.upload(all_entries.data(), all_entries.size(), s->stream);
  (force ? s->task_pb_f : s->task_pb_d).upload(all_pb.data(), all_pb.size(), s->stream);
  (force ? s->task_pe_f : s->task_pe_d).upload(all_pe.data(), all_pe.size(), s->stream);
  (force ? s->task_units_begin_f : s->task_units_begin_d) = ib;
  CK(cudaStreamSynchronize(s->stream));
}

static int find_task(const sphgpu_space* s, int ci, int cj) {
  const auto& tasks = s->space->tasks();
  for (size_t t = 0; t < tasks.size(); t++)
    if ((tasks[t].ci == ci && tasks[t].cj == cj) || (tasks[t].ci == cj && tasks[t].cj == ci))
      return (int)t;
  return -1;
}

static int run_task(sphgpu_space* s, int t, bool force, cudaStream_t st) {
  const auto& ib = force ? s->task_units_begin_f : s->task_units_begin_d;
  const int b = ib[t], e = ib[t + 1];
  if (e == b) return SPHGPU_OK;
  G2Args a = gargs(s, s->dplan_d, 4, MODE_ACCUM);
  a.units = (force ? s->task_units_f.p : s->task_units_d.p) + b;
  a.count = e - b;
  a.count_ptr = nullptr;
  a.entries = force ? s->task_entries_f.p : s->task_entries_d.p;
  a.pair_block = force ? s->task_pb_f.p : s->task_pb_d.p;
  a.pair_entry = force ? s->task_pe_f.p : s->task_pe_d.p;
  CK(cudaMemsetAsync(s->queue.p + 4, 0, sizeof(int), st));
  CK(launch_gather(a, force, s->num_sms, e - b, st, s->tune.block_warps));
  return SPHGPU_OK;
}

int sphgpu_begin_loops(sphgpu_space* s, void* stream) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  return guard([&]() {
    ensure_device(s);
    ensure_host_state(s);
    ensure_task_plans(s, false);
    CK(launch_begin_step(s->P, s->prm.max_iter, s->redo.p, s->prm.h_max, pick(s, stream)));
    return SPHGPU_OK;
  });
}

int sphgpu_dosub_self1_density(sphgpu_space* s, int32_t cell, void* stream) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  return guard([&]() {
    ensure_device(s);
    ensure_host_state(s);
    ensure_task_plans(s, false);
    const int t = find_task(s, cell, -1);
    if (t < 0) return SPHGPU_OK;  // empty cell: nothing to do
    return run_task(s, t, false, pick(s, stream));
  });
}

int sphgpu_dosub_pair1_density(sphgpu_space* s, int32_t ci, int32_t cj, void* stream) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  return guard([&]() {
    ensure_device(s);
    ensure_host_state(s);
    ensure_task_plans(s, false);
    const int t = find_task(s, ci, cj);
    if (t < 0) return fail(SPHGPU_EINVAL, "cells are not neighbours");
    return run_task(s, t, false, pick(s, stream));
  });
}

int sphgpu_do_ghost(sphgpu_space* s, int32_t cell, void* stream) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  const int ntop = s->space->cdim()[0] * s->space->cdim()[1] * s->space->cdim()[2];
  if (cell < 0 || cell >= ntop) return fail(SPHGPU_EINVAL, "cell id out of range");
  return guard([&]() {
    ensure_device(s);
    ensure_host_state(s);
    cudaStream_t st = pick(s, stream);
    const Cell& c = s->space->cells()[cell];
    if (c.count == 0 || !c.active) return SPHGPU_OK;
    s->h_stale = true;
    CK(cudaMemsetAsync(s->redo.p, 0, sizeof(int) * s->prm.max_iter, st));
    for (int k = 0; k < s->prm.max_iter; k++) {
      CK(launch_ghost(ghargs(s, k, c.first, c.first + c.count), st));
      int cnt = 0;
      CK(cudaMemcpyAsync(&cnt, s->redo.p + k, sizeof(int), cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      if (cnt == 0) return SPHGPU_OK;
      enqueue_gather(s, st, s->dplan_s, 5, MODE_REDO, false, 3, nullptr,
                     s->top_leaf[cell], s->top_leaf[cell + 1]);
      if (k == s->prm.max_iter - 1)
        return fail(SPHGPU_ENOCONV, "smoothing length failed to converge on " +
                                        std::to_string(cnt) + " particles");
    }
    return SPHGPU_OK;
  });
}

static void ensure_force_plans(sphgpu_space* s, cudaStream_t st) {
  if (!s->task_f.empty()) return;
  // the force recursion needs the post-ghost h_max of every cell
  plan_force(s, st);
  ensure_task_plans(s, true);
  CK(launch_block_hmax(s->bb_fc.p, s->bb_lo.p, s->posh.p, s->bb_n, st));
}

int sphgpu_dosub_self2_force(sphgpu_space* s, int32_t cell, void* stream) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  return guard([&]() {
    ensure_device(s);
    ensure_host_state(s);
    ensure_force_plans(s, pick(s, stream));
    const int t = find_task(s, cell, -1);
    if (t < 0) return SPHGPU_OK;
    return run_task(s, t, true, pick(s, stream));
  });
}

int sphgpu_dosub_pair2_force(sphgpu_space* s, int32_t ci, int32_t cj, void* stream) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  return guard([&]() {
    ensure_device(s);
    ensure_host_state(s);
    ensure_force_plans(s, pick(s, stream));
    const int t = find_task(s, ci, cj);
    if (t < 0) return fail(SPHGPU_EINVAL, "cells are not neighbours");
    return run_task(s, t, true, pick(s, stream));
  });
}

int sphgpu_do_end_hydro_force(sphgpu_space* s, void* stream) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  return guard([&]() {
    ensure_device(s);
    ensure_host_state(s);
    CK(launch_end_force(s->P, pick(s, stream)));
    return SPHGPU_OK;
  });
}

int sphgpu_step_plain(sphgpu_space* s, void* stream) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  return guard([&]() {
    settle(s);
    ensure_device(s);
    cudaStream_t st = pick(s, stream);
    int rc = sphgpu_begin_loops(s, st);
    if (rc) return rc;
    const size_t ntasks = s->space->tasks().size();
    for (size_t t = 0; t < ntasks; t++) {
      rc = run_task(s, (int)t, false, st);
      if (rc) return rc;
    }
    const int ntop = s->space->cdim()[0] * s->space->cdim()[1] * s->space->cdim()[2];
    for (int c = 0; c < ntop; c++) {
      rc = sphgpu_do_ghost(s, c, st);
      if (rc) return rc;
    }
    ensure_force_plans(s, st);
    CK(launch_block_hmax(s->bb_fc.p, s->bb_lo.p, s->posh.p, s->bb_n, st));
    for (size_t t = 0; t < ntasks; t++) {
      rc = run_task(s, (int)t, true, st);
      if (rc) return rc;
    }
    CK(launch_end_force(s->P, st));
    CK(cudaStreamSynchronize(st));
    return SPHGPU_OK;
  });
}

}  // extern "C"
