// serve.cu -- the serving loop: many independent SPH boxes resident in one
// device arena and stepped together by the same persistent launches
// (continuous batching).
//
// A request is a box (positions, velocities, masses, h, u) and a number of
// density -> ghost -> force steps.  Submitted boxes are planned on host
// worker threads (tree build, sort order, gather lists: the same planner as a
// single space), then admitted into the arena as soon as every range they
// need is free: particles, leaves (plus one sentinel), 32-particle windows,
// j-blocks, top cells, and the entries / candidate pairs of their density
// and ghost-re-run lists.  The arena is sized from the device's free memory
// when the server starts, so admission is admission by free HBM.
//
// One pump advances every resident box by one step: one begin-step kernel,
// one density gather over the windows of all boxes that also records every
// particle's row of candidates, ghost round 0, the per-particle ghost solver
// over the rows with gated catch-up rounds (a re-run gather and a round
// update) for the particles whose h outgrew their row, one force gather that
// takes a group's partners from the rows where they cover them -- the
// single-space path's kernels and configuration (when the rows do not fit
// beside the arena, the ghost rounds re-run by gathers instead).  Every
// index a box's lists hold is rebased to its arena ranges when it is
// uploaded, and the gathers and the solver take the top-cell width per leaf,
// so boxes of different sizes share a launch and never see each other's
// particles.  A box joining in the middle of the stream has its force
// lists planned after its first ghost (the recursion reads the post-ghost
// h_max), inside the pump that runs its first step.  Finished boxes are read
// back and their ranges freed for the next admissions.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <exception>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "capi_util.h"
#include "space.h"
#include "sph_kernels.cuh"

using namespace sphgpu;
using namespace sphgpu::capi;

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

// First-fit allocator of index ranges in [0, cap), coalescing on release.
class Ranges {
 public:
  void init(int64_t cap) {
    free_.clear();
    if (cap > 0) free_[0] = cap;
    cap_ = cap;
    used_ = 0;
  }
  int64_t alloc(int64_t n) {
    if (n <= 0) return 0;
    for (auto it = free_.begin(); it != free_.end(); ++it)
      if (it->second >= n) {
        const int64_t base = it->first, len = it->second;
        free_.erase(it);
        if (len > n) free_[base + n] = len - n;
        used_ += n;
        return base;
      }
    return -1;
  }
  void release(int64_t base, int64_t n) {
    if (n <= 0 || base < 0) return;
    used_ -= n;
    auto it = free_.emplace(base, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  int64_t cap() const { return cap_; }
  int64_t used() const { return used_; }

 private:
  std::map<int64_t, int64_t> free_;
  int64_t cap_ = 0, used_ = 0;
};

// A submitted box and what a planner worker makes of it (store-order host
// arrays with box-local indices, ready to be rebased and uploaded).
struct Job {
  int64_t id = 0;
  int n = 0, nsteps = 0;
  Params prm;
  std::vector<double> x;
  std::vector<float> v, m, h, u;
  double t_submit = 0, t_ready = 0;
  std::unique_ptr<Space> sp;
  Plan pd, ps, pf;
  std::vector<double> xs, tl;
  std::vector<float4> vm, blo, bhi;
  std::vector<float> hs, us;
  std::vector<int8_t> dh, dh0;
  std::vector<int32_t> lf, top, gperm, s_of_g;
  std::vector<int> lwb;
  std::vector<LeafInfo> li;
  std::vector<int2> bfc;
  std::vector<int32_t> bo;  // j-block of every store particle
  int nleaves = 0, nwin = 0, nblk = 0, ntop = 0;
  float4 tw{0.f, 0.f, 0.f, 0.f};
  std::string err;
  // force lists, planned by a worker from the post-ghost h of a warm-up pass
  const float4* ph = nullptr;       // pinned copy of the box's posh
  std::atomic<int> pf_state{0};     // 0 pending, 1 planned, -1 failed
  std::string pf_err;
};

struct Resident {
  std::unique_ptr<Job> job;
  // 0: warming up (its first density + ghost pass gives the h the force
  // recursion needs), 1: force lists being planned, 2: stepping
  int phase = 0;
  int64_t pin0 = -1;  // its slice of the pinned h buffer while planning
  int64_t p0 = -1, l0 = -1, w0 = -1, b0 = -1, t0 = -1;
  int64_t e0[3] = {-1, -1, -1}, ne[3] = {0, 0, 0};  // entries of the d, s, f lists
  int64_t q0[3] = {-1, -1, -1}, nq[3] = {0, 0, 0};  // candidate pairs
  int steps = 0;
  bool force_planned = false;
  double t_admit = 0;
};

struct Done {
  int64_t id = 0;
  int n = 0, steps = 0;
  std::vector<float> fields;
  std::vector<int32_t> ints;
  double t_submit = 0, t_admit = 0, t_done = 0;
};

void plan_job(Job& j) {
  j.sp = std::make_unique<Space>(j.prm);
  j.sp->set_threads(1);  // the workers plan boxes side by side
  std::vector<int8_t> tb(j.n, 0);  // every particle active at every step
  j.sp->build(j.n, j.x.data(), j.h.data(), tb.data());
  j.sp->plan_density(j.pd, false);
  j.sp->plan_subset(j.ps);
  const Space& sp = *j.sp;
  const int n = j.n;
  const auto& gperm = sp.gperm();
  const auto& g_of_s = sp.gpu_of_sorted();
  j.s_of_g.assign(n, 0);
  for (int k = 0; k < n; k++) j.s_of_g[g_of_s[k]] = k;
  j.xs.resize(3 * (size_t)n);
  j.vm.resize(n);
  j.hs.resize(n);
  j.us.resize(n);
  j.dh.resize(n);
  j.dh0.resize(n);
  j.lf.resize(n);
  j.top.resize(n);
  j.gperm.assign(gperm.begin(), gperm.end());
  const auto& xw = sp.x();
  const auto& cells = sp.cells();
  const auto& leaf_of = sp.leaf_of();
  const auto& lvs = sp.leaves();
  for (int g = 0; g < n; g++) {
    const int k = gperm[g];
    const int srt = j.s_of_g[g];
    for (int d = 0; d < 3; d++) j.xs[3 * (size_t)g + d] = xw[3 * (size_t)k + d];
    j.vm[g] = make_float4(j.v[3 * (size_t)k], j.v[3 * (size_t)k + 1], j.v[3 * (size_t)k + 2],
                          j.m[k]);
    j.hs[g] = j.h[k];
    j.us[g] = j.u[k];
    j.dh[g] = sp.depth_h()[srt];
    j.dh0[g] = sp.h_depth_of(j.h[k], lvs[leaf_of[srt]]);
    j.lf[g] = leaf_of[srt];
    j.top[g] = cells[lvs[leaf_of[srt]]].top;
  }
  j.nleaves = (int)lvs.size();
  j.lwb.assign(j.nleaves + 1, 0);
  int w = 0;
  for (int l = 0; l < j.nleaves; l++) {
    j.lwb[l] = w;
    w += (cells[lvs[l]].count + 31) / 32;
  }
  j.lwb[j.nleaves] = w;
  j.nwin = w;
  j.ntop = sp.cdim()[0] * sp.cdim()[1] * sp.cdim()[2];
  j.tl.resize(3 * (size_t)j.ntop);
  for (int t = 0; t < j.ntop; t++)
    for (int d = 0; d < 3; d++) j.tl[3 * (size_t)t + d] = cells[t].loc[d];
  sp.leaf_infos(j.li);
  const JBlocks& jb = sp.jblocks();
  j.nblk = (int)jb.first.size();
  j.blo.resize(j.nblk);
  j.bhi.resize(j.nblk);
  j.bfc.resize(j.nblk);
  for (int b = 0; b < j.nblk; b++) {
    j.blo[b] = make_float4(jb.lo[3 * b], jb.lo[3 * b + 1], jb.lo[3 * b + 2], 0.f);
    j.bhi[b] = make_float4(jb.hi[3 * b], jb.hi[3 * b + 1], jb.hi[3 * b + 2], 0.f);
    j.bfc[b] = make_int2(jb.first[b], jb.count[b]);
  }
  j.bo.assign(n, 0);
  for (int b = 0; b < j.nblk; b++)
    for (int k = jb.first[b]; k < jb.first[b] + jb.count[b]; k++) j.bo[k] = b;
  const double* wd = sp.width();
  j.tw = make_float4((float)wd[0], (float)wd[1], (float)wd[2], 0.f);
  // Host copies of the inputs are no longer needed.
  std::vector<double>().swap(j.x);
  std::vector<float>().swap(j.v);
  std::vector<float>().swap(j.m);
  std::vector<float>().swap(j.u);
}

constexpr float kServeBand = 2.44140625e-4f;  // 2^-12, as the single-space path
// Rows of the first density pass, as the single-space path's defaults: at
// most kRowCap candidates per particle, within sqrt(kRowWiden) x its radius.
constexpr int kRowCap = 160;
constexpr float kRowWiden = 1.21f;

}  // namespace

struct sphgpu_server {
  Params phys;
  int num_sms = 0;
  cudaStream_t st = nullptr;
  int64_t free_hbm_at_start = 0, arena_bytes = 0;
  Ranges rP, rL, rW, rB, rT, rE[3], rQ[3];
  // device arena
  DBuf<double> xd, top_loc;
  DBuf<float4> posh, velm, dens0, dens1, fin0, acc, bb_lo, bb_hi, leaf_tw;
  DBuf<float2> fin1, hdt_vsig;
  DBuf<float> u, h0, left, right;
  DBuf<uint8_t> flags;
  DBuf<int8_t> depth_h, depth_h0;
  DBuf<int32_t> leaf_of, ghost_iters, ngb_d, ngb_d_first, ngb_f, top_of, perm;
  DBuf<LeafInfo> leaves;
  DBuf<int> lwb;
  DBuf<int4> units;
  DBuf<int2> bb_fc;
  DBuf<Entry> ent[3];
  DBuf<int> pblk[3], pent[3], lpb[3];
  DBuf<int> queue, redo;
  // rows of the first density pass (the ghost's per-particle solver and the
  // force read them), on when they fit with the arena
  bool rows = false;
  DBuf<int> nl, nl_cnt, blk_of, catchup;
  DBuf<float> nl_T;
  DBuf<float> stage_f;
  DBuf<int32_t> stage_i;
  DevParticles P{};
  // host state
  std::map<int64_t, Resident> res;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<std::unique_ptr<Job>> todo, ready;
  std::vector<std::thread> workers;
  bool stop = false;
  int planning = 0;
  std::map<int64_t, Done> done;
  std::vector<int64_t> done_order;
  int64_t hwP = 0, hwL = 0, hwW = 0, hwB = 0;
  int64_t pumps = 0, retired = 0;
  int host_threads = 1;
  float4* pin = nullptr;  // pinned host buffer for warm-up h read-backs
  Ranges rPin;
  std::deque<Job*> ftodo;  // force lists to plan
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  double gpu_ms = 0, force_plan_s = 0, admit_s = 0, retire_s = 0;

  ~sphgpu_server() {
    {
      std::lock_guard<std::mutex> lock(mu);
      stop = true;
    }
    cv.notify_all();
    for (auto& t : workers) t.join();
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
    if (st) cudaStreamDestroy(st);
    if (pin) cudaFreeHost(pin);
  }

  void worker() {
    for (;;) {
      std::unique_ptr<Job> j;
      Job* fj = nullptr;
      {
        std::unique_lock<std::mutex> lock(mu);
        cv.wait(lock, [&] { return stop || !todo.empty() || !ftodo.empty(); });
        if (stop) return;
        if (!ftodo.empty()) {  // force lists first: a box waits on them
          fj = ftodo.front();
          ftodo.pop_front();
        } else {
          j = std::move(todo.front());
          todo.pop_front();
          planning++;
        }
      }
      if (fj) {
        try {
          plan_force_lists(*fj);
          fj->pf_state = 1;
        } catch (const std::exception& e) {
          fj->pf_err = e.what();
          fj->pf_state = -1;
        }
        continue;
      }
      try {
        plan_job(*j);
      } catch (const std::exception& e) {
        j->err = e.what();
      }
      j->t_ready = now_s();
      {
        std::lock_guard<std::mutex> lock(mu);
        planning--;
        ready.push_back(std::move(j));
      }
      cv.notify_all();
    }
  }

  // The box's post-ghost h (pinned copy, store order) -> its planner, whose
  // force recursion reads the new h_max.
  static void plan_force_lists(Job& j) {
    std::vector<float> hs(j.n);
    for (int g = 0; g < j.n; g++) hs[j.s_of_g[g]] = j.ph[g].w;
    j.sp->update_h_after_ghost(hs.data());
    j.sp->plan_density(j.pf, true);
  }

  void recompute_high_water() {
    hwP = hwL = hwW = hwB = 0;
    for (auto& kv : res) {
      const Resident& r = kv.second;
      const Job& j = *r.job;
      hwP = std::max(hwP, r.p0 + j.n);
      hwL = std::max(hwL, r.l0 + j.nleaves + 1);
      hwW = std::max(hwW, r.w0 + j.nwin);
      hwB = std::max(hwB, r.b0 + j.nblk);
    }
  }

  // Rebased copy of a plan into the arena lists of kind k (0 density,
  // 1 ghost re-runs, 2 force); returns false when the lists do not fit.
  bool place_plan(Resident& r, const Plan& pl, int k) {
    const Job& j = *r.job;
    const int64_t ne = (int64_t)pl.entries.size(), nq = (int64_t)pl.pair_block.size();
    const int64_t e0 = rE[k].alloc(ne);
    if (e0 < 0) return false;
    const int64_t q0 = rQ[k].alloc(nq);
    if (q0 < 0) {
      rE[k].release(e0, ne);
      return false;
    }
    r.e0[k] = e0;
    r.ne[k] = ne;
    r.q0[k] = q0;
    r.nq[k] = nq;
    std::vector<Entry> es(pl.entries);
    for (Entry& e : es) {
      e.first += (int32_t)r.p0;
      e.bfirst += (int32_t)r.b0;
    }
    std::vector<int> pb(pl.pair_block), pe(pl.pair_entry);
    for (int& b : pb) b += (int)r.b0;
    for (int& e : pe) e += (int)e0;
    std::vector<int> lp(j.nleaves + 1);
    for (int l = 0; l <= j.nleaves; l++) lp[l] = pl.leaf_pair_begin[l] + (int)q0;
    if (ne) CK(cudaMemcpyAsync(ent[k].p + e0, es.data(), sizeof(Entry) * ne,
                               cudaMemcpyHostToDevice, st));
    if (nq) {
      CK(cudaMemcpyAsync(pblk[k].p + q0, pb.data(), sizeof(int) * nq, cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(pent[k].p + q0, pe.data(), sizeof(int) * nq, cudaMemcpyHostToDevice, st));
    }
    CK(cudaMemcpyAsync(lpb[k].p + r.l0, lp.data(), sizeof(int) * (j.nleaves + 1),
                       cudaMemcpyHostToDevice, st));
    // the uploads read host vectors that die here
    CK(cudaStreamSynchronize(st));
    return true;
  }

  void release_plan(Resident& r, int k) {
    rE[k].release(r.e0[k], r.ne[k]);
    rQ[k].release(r.q0[k], r.nq[k]);
    r.e0[k] = r.q0[k] = -1;
    r.ne[k] = r.nq[k] = 0;
  }

  void release_ranges(Resident& r) {
    const Job& j = *r.job;
    rP.release(r.p0, j.n);
    rL.release(r.l0, j.nleaves + 1);
    rW.release(r.w0, j.nwin);
    rB.release(r.b0, j.nblk);
    rT.release(r.t0, j.ntop);
    for (int k = 0; k < 3; k++) release_plan(r, k);
  }

  // Clears what the kernels read for a range that no box owns any more.
  void clear_ranges(const Resident& r) {
    const Job& j = *r.job;
    CK(cudaMemsetAsync(flags.p + r.p0, 0, j.n, st));
    CK(cudaMemsetAsync(leaves.p + r.l0, 0, sizeof(LeafInfo) * (j.nleaves + 1), st));
    if (j.nwin) CK(cudaMemsetAsync(units.p + r.w0, 0, sizeof(int4) * j.nwin, st));
    if (j.nblk) CK(cudaMemsetAsync(bb_fc.p + r.b0, 0, sizeof(int2) * j.nblk, st));
  }

  // Claims every range of a planned box and uploads it; false when a range
  // does not fit (nothing is kept then).
  bool admit(std::unique_ptr<Job>& jp) {
    Job& j = *jp;
    Resident r;
    r.p0 = rP.alloc(j.n);
    r.l0 = rL.alloc(j.nleaves + 1);
    r.w0 = rW.alloc(j.nwin);
    r.b0 = rB.alloc(j.nblk);
    r.t0 = rT.alloc(j.ntop);
    auto undo = [&]() {
      rP.release(r.p0, j.n);
      rL.release(r.l0, j.nleaves + 1);
      rW.release(r.w0, j.nwin);
      rB.release(r.b0, j.nblk);
      rT.release(r.t0, j.ntop);
    };
    if (r.p0 < 0 || r.l0 < 0 || r.w0 < 0 || r.b0 < 0 || r.t0 < 0) {
      if (r.p0 >= 0) rP.release(r.p0, j.n);
      if (r.l0 >= 0) rL.release(r.l0, j.nleaves + 1);
      if (r.w0 >= 0) rW.release(r.w0, j.nwin);
      if (r.b0 >= 0) rB.release(r.b0, j.nblk);
      if (r.t0 >= 0) rT.release(r.t0, j.ntop);
      return false;
    }
    r.job = std::move(jp);
    if (!place_plan(r, j.pd, 0)) {
      undo();
      jp = std::move(r.job);
      return false;
    }
    if (!place_plan(r, j.ps, 1)) {
      release_plan(r, 0);
      undo();
      jp = std::move(r.job);
      return false;
    }
    const int n = j.n;
    const int64_t p0 = r.p0;
    // particles
    std::vector<int32_t> lf(n), top(n);
    for (int g = 0; g < n; g++) {
      lf[g] = j.lf[g] + (int32_t)r.l0;
      top[g] = j.top[g] + (int32_t)r.t0;
    }
    std::vector<uint8_t> fl(n, 1);
    CK(cudaMemcpyAsync(xd.p + 3 * p0, j.xs.data(), sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(velm.p + p0, j.vm.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(h0.p + p0, j.hs.data(), sizeof(float) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(u.p + p0, j.us.data(), sizeof(float) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(flags.p + p0, fl.data(), n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(depth_h.p + p0, j.dh.data(), n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(depth_h0.p + p0, j.dh0.data(), n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(leaf_of.p + p0, lf.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(top_of.p + p0, top.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(perm.p + p0, j.gperm.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(fin0.p + p0, 0, sizeof(float4) * n, st));
    CK(cudaMemsetAsync(fin1.p + p0, 0, sizeof(float2) * n, st));
    CK(cudaMemsetAsync(acc.p + p0, 0, sizeof(float4) * n, st));
    CK(cudaMemsetAsync(hdt_vsig.p + p0, 0, sizeof(float2) * n, st));
    // top cells, leaves (+ sentinel), windows, j-blocks
    CK(cudaMemcpyAsync(top_loc.p + 3 * r.t0, j.tl.data(), sizeof(double) * 3 * j.ntop,
                       cudaMemcpyHostToDevice, st));
    std::vector<LeafInfo> li(j.li);
    li.resize(j.nleaves + 1);
    std::memset(&li[j.nleaves], 0, sizeof(LeafInfo));
    for (int l = 0; l < j.nleaves; l++) {
      li[l].first += (int32_t)p0;
      li[l].top += (int32_t)r.t0;
    }
    CK(cudaMemcpyAsync(leaves.p + r.l0, li.data(), sizeof(LeafInfo) * (j.nleaves + 1),
                       cudaMemcpyHostToDevice, st));
    std::vector<int> lw(j.nleaves + 1);
    for (int l = 0; l <= j.nleaves; l++) lw[l] = j.lwb[l] + (int)r.w0;
    CK(cudaMemcpyAsync(lwb.p + r.l0, lw.data(), sizeof(int) * (j.nleaves + 1),
                       cudaMemcpyHostToDevice, st));
    std::vector<float4> tw(j.nleaves + 1, j.tw);
    CK(cudaMemcpyAsync(leaf_tw.p + r.l0, tw.data(), sizeof(float4) * (j.nleaves + 1),
                       cudaMemcpyHostToDevice, st));
    std::vector<int> zero(j.nleaves + 1, 0);
    CK(cudaMemcpyAsync(lpb[2].p + r.l0, zero.data(), sizeof(int) * (j.nleaves + 1),
                       cudaMemcpyHostToDevice, st));
    if (j.nwin) CK(cudaMemsetAsync(units.p + r.w0, 0, sizeof(int4) * j.nwin, st));
    std::vector<int2> bfc(j.bfc);
    for (auto& b : bfc) b.x += (int)p0;
    if (rows) {
      std::vector<int32_t> bo(j.bo);
      for (auto& b : bo) b += (int32_t)r.b0;
      CK(cudaMemcpyAsync(blk_of.p + p0, bo.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, st));
      CK(cudaMemsetAsync(nl_cnt.p + p0, 0xff, sizeof(int) * n, st));  // -1: no row yet
    }
    if (j.nblk) {
      CK(cudaMemcpyAsync(bb_lo.p + r.b0, j.blo.data(), sizeof(float4) * j.nblk, cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(bb_hi.p + r.b0, j.bhi.data(), sizeof(float4) * j.nblk, cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(bb_fc.p + r.b0, bfc.data(), sizeof(int2) * j.nblk, cudaMemcpyHostToDevice, st));
    }
    DevParticles V = view(p0, n);
    CK(launch_prepare_posh(V, top_of.p + p0, top_loc.p, st));
    CK(cudaStreamSynchronize(st));  // the host vectors above die here
    // the store copies are on the device now
    std::vector<double>().swap(r.job->xs);
    std::vector<float4>().swap(r.job->vm);
    r.t_admit = now_s();
    const int64_t id = r.job->id;
    res.emplace(id, std::move(r));
    recompute_high_water();
    return true;
  }

  DevParticles view(int64_t p0, int n) const {
    DevParticles V = P;
    V.n = n;
    V.xd = P.xd + 3 * p0;
    V.posh = P.posh + p0;
    V.velm = P.velm + p0;
    V.u = P.u + p0;
    V.h0 = P.h0 + p0;
    V.flags = P.flags + p0;
    V.depth_h = P.depth_h + p0;
    V.depth_h0 = P.depth_h0 + p0;
    V.leaf_of = P.leaf_of + p0;
    V.dens0 = P.dens0 + p0;
    V.dens1 = P.dens1 + p0;
    V.left = P.left + p0;
    V.right = P.right + p0;
    V.ghost_iters = P.ghost_iters + p0;
    V.fin0 = P.fin0 + p0;
    V.fin1 = P.fin1 + p0;
    V.acc = P.acc + p0;
    V.hdt_vsig = P.hdt_vsig + p0;
    V.ngb_d = P.ngb_d + p0;
    V.ngb_d_first = P.ngb_d_first + p0;
    V.ngb_f = P.ngb_f + p0;
    return V;
  }

  G2Args gargs(int k, int qslot, int mode, const int* gate) {
    G2Args a;
    a.p = P;
    a.p.n = (int)hwP;
    a.units = units.p;
    a.count = (int)hwW;
    a.count_ptr = nullptr;
    a.pair_block = pblk[k].p;
    a.pair_entry = pent[k].p;
    a.entries = ent[k].p;
    a.bb_lo = bb_lo.p;
    a.bb_hi = bb_hi.p;
    a.bb_fc = bb_fc.p;
    a.top_width = make_float3(1.f, 1.f, 1.f);
    a.leaf_tw = leaf_tw.p;
    a.queue = queue.p + qslot;
    a.hits = nullptr;
    a.gate = gate;
    a.band = kServeBand;
    a.mode = mode;
    a.nl = nullptr;
    a.nl_cnt = nullptr;
    a.nl_T = nullptr;
    a.nl_cap = 0;
    a.leaves = leaves.p;
    a.blk_of = blk_of.p;
    return a;
  }

  // lists: the first pass records the rows; force_rows: the force reads
  // them where they cover a group's partners
  void gather(int k, int qslot, int mode, bool force, int need, const int* gate,
              bool lists = false, bool force_rows = false) {
    CK(cudaMemsetAsync(queue.p + qslot, 0, sizeof(int), st));
    CK(launch_build_units(leaves.p, (int)hwL, lwb.p, flags.p, need, 0, lpb[k].p, units.p, gate,
                          st));
    G2Args a = gargs(k, qslot, mode, gate);
    if (lists || force_rows) {
      a.nl = nl.p;
      a.nl_cnt = nl_cnt.p;
      a.nl_T = nl_T.p;
      a.nl_cap = kRowCap;
      a.nl_seg = 1;
    }
    if (lists) a.nl_widen = kRowWiden;
    if (force_rows) a.force_rows = 1;
    CK(launch_gather(a, force, num_sms, (int)hwW, st, 8, lists, 1));
  }

  ListArgs largs() {
    ListArgs l;
    l.p = P;
    l.p.n = (int)hwP;
    l.nl = nl.p;
    l.nl_cnt = nl_cnt.p;
    l.nl_T = nl_T.p;
    l.nl_cap = kRowCap;
    l.nl_seg = 1;
    l.leaf_pair_begin = lpb[1].p;
    l.pair_block = pblk[1].p;
    l.pair_entry = pent[1].p;
    l.entries = ent[1].p;
    l.blk_of = blk_of.p;
    l.top_width = make_float3(1.f, 1.f, 1.f);
    l.leaf_tw = leaf_tw.p;
    l.band = kServeBand;
    l.gate = redo.p;
    l.hits = nullptr;
    l.handover = catchup.p;
    return l;
  }

  GhostArgs ghargs(int iter) {
    GhostArgs g;
    g.p = P;
    g.p.n = (int)hwP;
    g.leaves = leaves.p;
    g.eta_dim = phys.eta * phys.eta * phys.eta;
    g.h_tol = phys.h_tolerance;
    g.h_max = phys.h_max;
    g.h_min = phys.h_min;
    g.alpha = phys.alpha;
    g.iter = iter;
    g.lo = 0;
    g.hi = (int)hwP;
    g.redo_count = redo.p;
    return g;
  }

  // Force lists of the boxes that just ran their first ghost: their
  // post-ghost h goes to their planners, whose recursion then reads the new
  // h_max; the boxes are planned side by side on host threads.
  void plan_forces(std::vector<Resident*>& rs) {
    std::vector<std::vector<float4>> ph(rs.size());
    for (size_t k = 0; k < rs.size(); k++) {
      ph[k].resize(rs[k]->job->n);
      CK(cudaMemcpyAsync(ph[k].data(), posh.p + rs[k]->p0, sizeof(float4) * rs[k]->job->n,
                         cudaMemcpyDeviceToHost, st));
    }
    CK(cudaStreamSynchronize(st));
    const auto t0 = now_s();
    std::atomic<int> next{0};
    std::exception_ptr err;
    std::mutex emu;
    auto work = [&]() {
      for (int k = next++; k < (int)rs.size(); k = next++) {
        try {
          Job& j = *rs[k]->job;
          std::vector<float> hs(j.n);
          for (int g = 0; g < j.n; g++) hs[j.s_of_g[g]] = ph[k][g].w;
          j.sp->update_h_after_ghost(hs.data());
          j.sp->plan_density(j.pf, true);
        } catch (...) {
          std::lock_guard<std::mutex> lock(emu);
          if (!err) err = std::current_exception();
        }
      }
    };
    const int nt = std::min<int>((int)rs.size(), std::max(1, host_threads));
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; t++) pool.emplace_back(work);
    work();
    for (auto& t : pool) t.join();
    if (err) std::rethrow_exception(err);
    for (Resident* r : rs) {
      if (!place_plan(*r, r->job->pf, 2))
        throw std::runtime_error("serving arena: no room for a box's force lists");
      r->force_planned = true;
    }
    force_plan_s += now_s() - t0;
  }

  void retire(Resident& r) {
    Job& j = *r.job;
    const int n = j.n;
    if (stage_f.n < 24 * (size_t)n) stage_f.alloc(24 * (size_t)n);
    if (stage_i.n < 4 * (size_t)n) stage_i.alloc(4 * (size_t)n);
    CK(launch_collect_out(view(r.p0, n), perm.p + r.p0, stage_f.p, stage_i.p, st));
    Done d;
    d.id = j.id;
    d.n = n;
    d.steps = r.steps;
    d.fields.resize(24 * (size_t)n);
    d.ints.resize(4 * (size_t)n);
    CK(cudaMemcpyAsync(d.fields.data(), stage_f.p, sizeof(float) * 24 * n, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(d.ints.data(), stage_i.p, sizeof(int32_t) * 4 * n, cudaMemcpyDeviceToHost, st));
    clear_ranges(r);
    CK(cudaStreamSynchronize(st));
    d.t_submit = j.t_submit;
    d.t_admit = r.t_admit;
    d.t_done = now_s();
    release_ranges(r);
    done_order.push_back(d.id);
    done.emplace(d.id, std::move(d));
    retired++;
  }

  // One step of every resident box.
  void step_all() {
    // boxes whose force lists a worker finished: upload them; they step
    // in full from this pump on
    for (auto& kv : res) {
      Resident& r = kv.second;
      if (r.phase != 1) continue;
      const int state = r.job->pf_state;
      if (state == 0) continue;
      if (state < 0) throw std::runtime_error("force lists: " + r.job->pf_err);
      rPin.release(r.pin0, r.job->n);
      r.pin0 = -1;
      if (!place_plan(r, r.job->pf, 2))
        throw std::runtime_error("serving arena: no room for a box's force lists");
      r.force_planned = true;
      r.phase = 2;
    }
    CK(cudaEventRecord(ev[0], st));
    CK(launch_begin_step(view(0, (int)hwP), phys.max_iter, redo.p, phys.h_max, st));
    gather(0, 0, MODE_FIRST, false, 1, nullptr, rows);
    if (rows) {
      // as the single-space path with rows: round 0, then every particle
      // iterates on its own from its row; those whose h outgrew it catch up
      // by gathers, each at its own round count
      CK(launch_ghost(ghargs(0), st));
      CK(cudaMemsetAsync(catchup.p, 0, sizeof(int) * (phys.max_iter + 1), st));
      CK(launch_solve_from_lists(largs(), ghargs(1), phys.max_iter, st));
      for (int r = 0; r < phys.max_iter; r++) {
        gather(1, 1, MODE_REDO, false, 3, catchup.p + r);
        CK(launch_ghost_catchup(ghargs(0), phys.max_iter, catchup.p + r, catchup.p + r + 1,
                                st));
      }
    } else {
      for (int k = 0; k < phys.max_iter; k++) {
        CK(launch_ghost(ghargs(k), st));
        gather(1, 1, MODE_REDO, false, 3, redo.p + k);
      }
    }
    int last = 0;
    CK(cudaMemcpyAsync(&last, redo.p + phys.max_iter - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaEventRecord(ev[1], st));
    // warming boxes: their h goes to pinned memory (in stream order, before
    // the next pump resets it) and their force lists to the workers; when
    // the pinned buffer is full, they are planned here instead
    std::vector<Resident*> inline_plan, to_workers;
    for (auto& kv : res) {
      Resident& r = kv.second;
      if (r.phase != 0) continue;
      const int64_t off = rPin.alloc(r.job->n);
      if (off < 0) {
        inline_plan.push_back(&r);
        continue;
      }
      r.pin0 = off;
      r.job->ph = pin + off;
      r.job->pf_state = 0;
      CK(cudaMemcpyAsync(pin + off, posh.p + r.p0, sizeof(float4) * r.job->n,
                         cudaMemcpyDeviceToHost, st));
      r.phase = 1;
      to_workers.push_back(&r);
    }
    if (!inline_plan.empty()) {
      plan_forces(inline_plan);
      for (Resident* r : inline_plan) r->phase = 2;
    }
    CK(cudaEventRecord(ev[2], st));
    CK(launch_block_hmax(bb_fc.p, bb_lo.p, posh.p, (int)hwB, st));
    gather(2, 2, MODE_FIRST, true, 1, nullptr, false, rows);  // writes the finished sums
    CK(cudaEventRecord(ev[3], st));
    CK(cudaStreamSynchronize(st));
    if (!to_workers.empty()) {
      {
        std::lock_guard<std::mutex> lock(mu);
        for (Resident* r : to_workers) ftodo.push_back(r->job.get());
      }
      cv.notify_all();
    }
    float a = 0.f, b = 0.f;
    CK(cudaEventElapsedTime(&a, ev[0], ev[1]));
    CK(cudaEventElapsedTime(&b, ev[2], ev[3]));
    gpu_ms += a + b;
    if (last > 0)
      throw std::runtime_error("smoothing length failed to converge on " +
                               std::to_string(last) + " particles");
    std::vector<int64_t> fin;
    for (auto& kv : res) {
      if (kv.second.phase != 2) continue;  // a warm-up pass is not a step
      kv.second.steps++;
      if (kv.second.steps >= kv.second.job->nsteps) fin.push_back(kv.first);
    }
    const double tr = now_s();
    for (int64_t id : fin) {
      retire(res.at(id));
      res.erase(id);
    }
    retire_s += now_s() - tr;
    recompute_high_water();
  }
};

extern "C" {

int sphgpu_server_create(const sphgpu_params* prm, int64_t max_particles,
                         int32_t planner_threads, sphgpu_server** out) {
  if (!prm || !out || planner_threads < 0 || max_particles < 0)
    return fail(SPHGPU_EINVAL, "sphgpu_server_create: bad argument");
  if (prm->max_iter < 1 || prm->max_iter > 1000 || !(prm->eta > 0.f))
    return fail(SPHGPU_EINVAL, "sphgpu_server_create: invalid parameters");
  *out = nullptr;
  return guard([&]() {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
      throw std::runtime_error("no CUDA device available");
    auto s = std::make_unique<sphgpu_server>();
    Params& P = s->phys;
    for (int d = 0; d < 3; d++) P.dim[d] = prm->dim[d];
    P.periodic = prm->periodic;
    P.eta = prm->eta;
    P.h_tolerance = prm->h_tolerance;
    P.h_max = prm->h_max;
    P.h_min = prm->h_min;
    P.alpha = prm->alpha;
    P.max_iter = prm->max_iter;
    P.max_active_bin = 127;
    P.max_top_level_cells = prm->max_top_level_cells;
    int dev = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, dev));
    CK(cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking));
    size_t fr = 0, tot = 0;
    CK(cudaMemGetInfo(&fr, &tot));
    s->free_hbm_at_start = (int64_t)fr;
    // Bytes the arena holds per particle slot (particle state, leaves,
    // windows, j-blocks, top cells, three sets of lists), see below.
    const double per_particle = 8 * 3 + 16 * 7 + 8 * 2 + 4 * 4 + 3 + 4 * 7 +
                                (sizeof(LeafInfo) + 16 + 4 * 4) / 4.0 + 16 / 8.0 +
                                36 / 8.0 + 24 / 2.0 + 3 * (sizeof(Entry) / 2.0 + 8 * 4.0);
    // the rows of the first density pass and the j-block of every slot
    const double per_particle_rows = 4.0 * kRowCap + 4 + 4 + 4;
    int64_t cap = max_particles;
    const int64_t afford = (int64_t)(0.5 * (double)fr / per_particle);
    // rows while the arena with them still fits in half the free HBM
    const int64_t afford_rows =
        (int64_t)(0.5 * (double)fr / (per_particle + per_particle_rows));
    if (cap == 0) cap = std::min<int64_t>(afford, (int64_t)1 << 24);
    if (cap > afford)
      return fail(SPHGPU_ENOMEM, "sphgpu_server_create: arena larger than half the free HBM");
    if (cap > ((int64_t)1 << 26))  // partner indices are packed in 27 bits
      return fail(SPHGPU_EINVAL, "sphgpu_server_create: at most 2^26 particles");
    if (cap < 4096) cap = 4096;
    s->rows = cap <= afford_rows;
    const int64_t capL = cap / 4 + 1024, capW = cap / 32 + capL, capB = cap / 8 + capL,
                  capT = cap / 2 + 1728, capE = cap / 2 + 64 * 1024, capQ = 4 * cap;
    s->rP.init(cap);
    s->rL.init(capL);
    s->rW.init(capW);
    s->rB.init(capB);
    s->rT.init(capT);
    for (int k = 0; k < 3; k++) {
      s->rE[k].init(capE);
      s->rQ[k].init(capQ);
    }
    s->xd.alloc(3 * cap);
    s->posh.alloc(cap);
    s->velm.alloc(cap);
    s->dens0.alloc(cap);
    s->dens1.alloc(cap);
    s->fin0.alloc(cap);
    s->acc.alloc(cap);
    s->fin1.alloc(cap);
    s->hdt_vsig.alloc(cap);
    s->u.alloc(cap);
    s->h0.alloc(cap);
    s->left.alloc(cap);
    s->right.alloc(cap);
    s->flags.alloc(cap);
    s->depth_h.alloc(cap);
    s->depth_h0.alloc(cap);
    s->leaf_of.alloc(cap);
    s->ghost_iters.alloc(cap);
    s->ngb_d.alloc(cap);
    s->ngb_d_first.alloc(cap);
    s->ngb_f.alloc(cap);
    s->top_of.alloc(cap);
    s->perm.alloc(cap);
    s->leaves.alloc(capL);
    s->leaf_tw.alloc(capL);
    s->lwb.alloc(capL + 1);
    s->units.alloc(capW);
    s->bb_lo.alloc(capB);
    s->bb_hi.alloc(capB);
    s->bb_fc.alloc(capB);
    s->top_loc.alloc(3 * capT);
    for (int k = 0; k < 3; k++) {
      s->ent[k].alloc(capE);
      s->pblk[k].alloc(capQ);
      s->pent[k].alloc(capQ);
      s->lpb[k].alloc(capL + 1);
    }
    s->queue.alloc(16);
    s->redo.alloc(std::max(1, P.max_iter));
    s->catchup.alloc(P.max_iter + 1);
    if (s->rows) {
      s->nl.alloc((size_t)cap * kRowCap);
      s->nl_cnt.alloc(cap);
      s->nl_T.alloc(cap);
      s->blk_of.alloc(cap);
    } else {
      s->blk_of.alloc(1);
    }
    cudaStream_t st = s->st;
    CK(cudaMemsetAsync(s->flags.p, 0, cap, st));
    CK(cudaMemsetAsync(s->leaves.p, 0, sizeof(LeafInfo) * capL, st));
    CK(cudaMemsetAsync(s->units.p, 0, sizeof(int4) * capW, st));
    CK(cudaMemsetAsync(s->bb_fc.p, 0, sizeof(int2) * capB, st));
    for (int k = 0; k < 3; k++) CK(cudaMemsetAsync(s->lpb[k].p, 0, sizeof(int) * (capL + 1), st));
    CK(cudaStreamSynchronize(st));
    size_t fr2 = 0;
    CK(cudaMemGetInfo(&fr2, &tot));
    s->arena_bytes = (int64_t)fr - (int64_t)fr2;
    DevParticles& D = s->P;
    D.n = 0;
    D.xd = s->xd.p;
    D.posh = s->posh.p;
    D.velm = s->velm.p;
    D.u = s->u.p;
    D.h0 = s->h0.p;
    D.flags = s->flags.p;
    D.depth_h = s->depth_h.p;
    D.depth_h0 = s->depth_h0.p;
    D.leaf_of = s->leaf_of.p;
    D.dens0 = s->dens0.p;
    D.dens1 = s->dens1.p;
    D.left = s->left.p;
    D.right = s->right.p;
    D.ghost_iters = s->ghost_iters.p;
    D.fin0 = s->fin0.p;
    D.fin1 = s->fin1.p;
    D.acc = s->acc.p;
    D.hdt_vsig = s->hdt_vsig.p;
    D.ngb_d = s->ngb_d.p;
    D.ngb_d_first = s->ngb_d_first.p;
    D.ngb_f = s->ngb_f.p;
    int nt = planner_threads;
    if (nt == 0) nt = (int)std::max(1u, std::min(std::thread::hardware_concurrency(), 16u));
    s->host_threads = (int)std::max(1u, std::min(std::thread::hardware_concurrency(), 16u));
    // pinned room for the warm-up h of up to 2^22 particles at a time
    const int64_t npin = std::min<int64_t>(cap, (int64_t)1 << 22);
    CK(cudaHostAlloc((void**)&s->pin, sizeof(float4) * npin, cudaHostAllocDefault));
    s->rPin.init(npin);
    for (auto& e : s->ev) CK(cudaEventCreate(&e));
    for (int t = 0; t < nt; t++) s->workers.emplace_back([p = s.get()] { p->worker(); });
    *out = s.release();
    return SPHGPU_OK;
  });
}

int sphgpu_server_destroy(sphgpu_server* s) {
  delete s;
  return SPHGPU_OK;
}

int sphgpu_server_submit(sphgpu_server* s, int64_t id, const sphgpu_params* box, int64_t n,
                         const double* x, const float* v, const float* m, const float* h,
                         const float* u, int32_t nsteps) {
  if (!s || !box || !x || !v || !m || !h || !u || n <= 0 || nsteps < 1)
    return fail(SPHGPU_EINVAL, "sphgpu_server_submit: bad argument");
  if (n > s->rP.cap())
    return fail(SPHGPU_EINVAL, "sphgpu_server_submit: box larger than the arena");
  if (!(box->dim[0] > 0) || !(box->dim[1] > 0) || !(box->dim[2] > 0) ||
      box->max_top_level_cells < 3)
    return fail(SPHGPU_EINVAL, "sphgpu_server_submit: invalid box parameters");
  return guard([&]() {
    {
      std::lock_guard<std::mutex> lock(s->mu);
      if (s->res.count(id) || s->done.count(id))
        return fail(SPHGPU_EINVAL, "sphgpu_server_submit: request id in use");
    }
    auto j = std::make_unique<Job>();
    j->id = id;
    j->n = (int)n;
    j->nsteps = nsteps;
    j->prm = s->phys;
    for (int d = 0; d < 3; d++) j->prm.dim[d] = box->dim[d];
    j->prm.periodic = box->periodic;
    j->prm.max_top_level_cells = box->max_top_level_cells;
    j->x.assign(x, x + 3 * n);
    j->v.assign(v, v + 3 * n);
    j->m.assign(m, m + n);
    j->h.assign(h, h + n);
    j->u.assign(u, u + n);
    j->t_submit = now_s();
    {
      std::lock_guard<std::mutex> lock(s->mu);
      s->todo.push_back(std::move(j));
    }
    s->cv.notify_one();
    return SPHGPU_OK;
  });
}

int sphgpu_server_pump(sphgpu_server* s, double wait_s, int32_t* resident) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  return guard([&]() {
    // admissions, in submission order of what the planners finished
    std::deque<std::unique_ptr<Job>> got;
    {
      std::unique_lock<std::mutex> lock(s->mu);
      if (s->res.empty() && s->ready.empty() && wait_s > 0 &&
          (s->planning > 0 || !s->todo.empty()))
        s->cv.wait_for(lock, std::chrono::duration<double>(wait_s),
                       [&] { return !s->ready.empty(); });
      got.swap(s->ready);
    }
    std::sort(got.begin(), got.end(),
              [](const std::unique_ptr<Job>& a, const std::unique_ptr<Job>& b) {
                return a->t_submit < b->t_submit;
              });
    std::string first_err;
    const double ta = now_s();
    while (!got.empty()) {
      std::unique_ptr<Job>& j = got.front();
      if (!j->err.empty()) {
        if (first_err.empty()) first_err = "request " + std::to_string(j->id) + ": " + j->err;
        got.pop_front();
        continue;
      }
      if (!s->admit(j)) {
        if (!s->res.empty()) break;  // wait for room; keep the order
        // nothing resident and still no room: it can never fit
        if (first_err.empty())
          first_err = "request " + std::to_string(j->id) + ": box does not fit the arena";
      }
      got.pop_front();
    }
    s->admit_s += now_s() - ta;
    if (!got.empty()) {
      std::lock_guard<std::mutex> lock(s->mu);
      for (auto it = got.rbegin(); it != got.rend(); ++it) s->ready.push_front(std::move(*it));
    }
    if (!s->res.empty()) {
      s->step_all();
      s->pumps++;
    }
    if (resident) *resident = (int32_t)s->res.size();
    if (!first_err.empty()) return fail(SPHGPU_EINVAL, first_err);
    return SPHGPU_OK;
  });
}

int sphgpu_server_poll(sphgpu_server* s, int64_t* ids, int32_t max_ids, int32_t* count) {
  if (!s || !count || (max_ids > 0 && !ids)) return fail(SPHGPU_EINVAL, "null argument");
  int k = 0;
  for (int64_t id : s->done_order) {
    if (k >= max_ids) break;
    ids[k++] = id;
  }
  s->done_order.erase(s->done_order.begin(), s->done_order.begin() + k);
  *count = k;
  return SPHGPU_OK;
}

int sphgpu_server_fetch(sphgpu_server* s, int64_t id, float* fields, int32_t* ints,
                        double times[3]) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  auto it = s->done.find(id);
  if (it == s->done.end()) return fail(SPHGPU_ESTATE, "request not finished (or fetched)");
  const Done& d = it->second;
  if (fields) std::memcpy(fields, d.fields.data(), sizeof(float) * d.fields.size());
  if (ints) std::memcpy(ints, d.ints.data(), sizeof(int32_t) * d.ints.size());
  if (times) {
    times[0] = d.t_submit;
    times[1] = d.t_admit;
    times[2] = d.t_done;
  }
  s->done.erase(it);
  return SPHGPU_OK;
}

int sphgpu_server_times(sphgpu_server* s, double times[4]) {
  if (!s || !times) return fail(SPHGPU_EINVAL, "null argument");
  times[0] = s->gpu_ms / 1e3;
  times[1] = s->force_plan_s;
  times[2] = s->admit_s;
  times[3] = s->retire_s;
  return SPHGPU_OK;
}

int sphgpu_server_stats(sphgpu_server* s, int64_t stats[8]) {
  if (!s || !stats) return fail(SPHGPU_EINVAL, "null argument");
  std::lock_guard<std::mutex> lock(s->mu);
  stats[0] = (int64_t)s->res.size();
  stats[1] = s->rP.used();
  stats[2] = s->rP.cap();
  stats[3] = (int64_t)(s->todo.size() + s->ready.size()) + s->planning;
  stats[4] = s->pumps;
  stats[5] = s->retired;
  stats[6] = s->arena_bytes;
  stats[7] = s->free_hbm_at_start;
  return SPHGPU_OK;
}

}  // extern "C"
