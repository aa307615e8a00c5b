// capi.cu -- the C ABI (include/swift_gb300.h): space lifecycle, the batched
// step (one CUDA graph per step), the plain per-task entry points, host I/O.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/swift_gb300.h"
#include "space.h"
#include "sph_kernels.cuh"

using namespace sphgpu;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

struct CudaError : std::runtime_error {
  explicit CudaError(const std::string& m) : std::runtime_error(m) {}
};

#define CK(call)                                                              \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess)                                                    \
      throw CudaError(std::string(#call) + ": " + cudaGetErrorString(e_));    \
  } while (0)

template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  void alloc(size_t count) {
    release();
    n = count;
    if (count == 0) count = 1;
    CK(cudaMalloc(&p, count * sizeof(T)));
  }
  void upload(const T* h, size_t count, cudaStream_t s) {
    if (count > n) alloc(count);
    if (count) CK(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  ~DBuf() { release(); }
};

struct DevPlan {
  DBuf<Entry> entries;
  DBuf<Unit> units;
  int nunits = 0;
  void upload(const Plan& pl, cudaStream_t s) {
    entries.upload(pl.entries.data(), pl.entries.size(), s);
    units.upload(pl.units.data(), pl.units.size(), s);
    nunits = (int)pl.units.size();
  }
};

// Sort units so that the most expensive go first (longest-processing-time
// order for the persistent queue); cost = i_count x sum of partner counts,
// the reference's pair cost model (scheduler.c:516-629) at particle level.
void order_units(Plan& pl) {
  std::vector<std::pair<double, Unit>> tmp;
  tmp.reserve(pl.units.size());
  for (const Unit& u : pl.units) {
    double c = 0;
    for (int e = u.e_begin; e < u.e_end; e++) c += pl.entries[e].count;
    tmp.emplace_back(c * u.i_count, u);
  }
  std::stable_sort(tmp.begin(), tmp.end(),
                   [](const auto& a, const auto& b) { return a.first > b.first; });
  for (size_t k = 0; k < tmp.size(); k++) pl.units[k] = tmp[k].second;
}

}  // namespace

struct sphgpu_space {
  Params prm;
  std::unique_ptr<Space> space;
  std::vector<double> x_in;
  std::vector<float> v_in, m_in, h_in, u_in;
  std::vector<int8_t> tb_in;
  sphgpu_tuning tune{1, 64, 1};

  // host plans
  Plan plan_d, plan_s, plan_f;
  bool force_planned = false;
  // plain-form per-task plans
  std::vector<Plan> task_d, task_f;
  std::vector<int> task_of_pair;  // unused placeholder for lookups
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
  DBuf<int8_t> depth_h;
  DBuf<int32_t> leaf_of, ghost_iters, ngb_d, ngb_d_first, ngb_f, perm, top_of;
  DBuf<double> top_loc;
  DBuf<LeafInfo> leaves;
  DevPlan dplan_d, dplan_s, dplan_f;
  std::vector<DevPlan> dtask_d, dtask_f;
  DBuf<int> queue, redo, status;
  // host staging for step_host
  DBuf<double> x_stage;
  DBuf<float> v_stage, m_stage, h_stage, u_stage, out_stage;
  cudaGraphExec_t graph = nullptr;
  int graph_stages = 0;

  ~sphgpu_space() {
    if (graph) cudaGraphExecDestroy(graph);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

int unit_chunk(const sphgpu_tuning& t) { return 128 / t.threads_per_particle; }

void build_plans(sphgpu_space* s) {
  s->space->set_unit_chunk(unit_chunk(s->tune));
  s->space->plan_density(s->plan_d, false);
  s->space->plan_subset(s->plan_s);
  order_units(s->plan_d);
  // subset units stay in leaf order: the plain-form ghost addresses them by
  // top cell.
  s->sub_units_of_top.clear();
  const auto& cells = s->space->cells();
  const int ntop = s->space->cdim()[0] * s->space->cdim()[1] * s->space->cdim()[2];
  s->sub_units_of_top.assign(ntop, {0, 0});
  const auto& lv = s->space->leaves();
  int k = 0;
  const int nu = (int)s->plan_s.units.size();
  for (int t = 0; t < ntop; t++) {
    const int b = k;
    while (k < nu && cells[lv[s->plan_s.units[k].leaf]].top == t) k++;
    s->sub_units_of_top[t] = {b, k};
  }
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
  // Cell-sorted copies of the inputs.
  const auto& perm = sp.perm();
  std::vector<double> xs(3 * (size_t)n);
  std::vector<float4> vm(n);
  std::vector<float> hs(n), us(n);
  std::vector<uint8_t> fl(n);
  std::vector<int32_t> top(n);
  const auto& xw = sp.x();
  const auto& act = sp.active();
  const auto& cells = sp.cells();
  const auto& leaf_of = sp.leaf_of();
  const auto& lvs = sp.leaves();
  for (int i = 0; i < n; i++) {
    const int k = perm[i];
    for (int d = 0; d < 3; d++) xs[3 * (size_t)i + d] = xw[3 * (size_t)k + d];
    vm[i] = make_float4(s->v_in[3 * (size_t)k], s->v_in[3 * (size_t)k + 1],
                        s->v_in[3 * (size_t)k + 2], s->m_in[k]);
    hs[i] = s->h_in[k];
    us[i] = s->u_in[k];
    fl[i] = act[i] ? 1 : 0;
    top[i] = cells[lvs[leaf_of[i]]].top;
  }
  const int ntop = sp.cdim()[0] * sp.cdim()[1] * sp.cdim()[2];
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
  s->depth_h.upload(sp.depth_h().data(), n, st);
  s->leaf_of.upload(leaf_of.data(), n, st);
  s->top_of.upload(top.data(), n, st);
  s->perm.upload(perm.data(), n, st);
  s->top_loc.upload(tl.data(), tl.size(), st);
  s->leaves.upload(li.data(), li.size(), st);
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
  s->queue.alloc(8);
  s->redo.alloc(std::max(1, s->prm.max_iter));
  s->status.alloc(1);
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
  CK(launch_prepare_posh(P, s->top_of.p, s->top_loc.p, st));
  s->dplan_d.upload(s->plan_d, st);
  s->dplan_s.upload(s->plan_s, st);
  CK(cudaStreamSynchronize(st));
  s->dev = true;
}

LaunchCfg cfg_of(const sphgpu_space* s) {
  LaunchCfg c;
  c.tpi = s->tune.threads_per_particle;
  c.jtile = s->tune.jtile;
  c.persistent = s->tune.persistent;
  c.block = 128;
  return c;
}

// Relative band of the FP32 pre-test around H^2.  The FP32 offsets carry
// about 1e-8 absolute error; for the smallest H of the supported boxes
// (~0.005 box units) that is < 1e-5 relative on r^2, far inside this band.
constexpr float kBand = 2.44140625e-4f;  // 2^-12

GatherArgs gargs(sphgpu_space* s, DevPlan& dp, int qslot, const int* gate) {
  GatherArgs a;
  a.p = s->P;
  a.units = dp.units.p;
  a.nunits = dp.nunits;
  a.entries = dp.entries.p;
  a.queue = s->queue.p + qslot;
  a.gate = gate;
  a.band = kBand;
  return a;
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
  g.max_iter = s->prm.max_iter;
  g.redo_count = s->redo.p;
  g.status = s->status.p;
  return g;
}

// Enqueue density (first pass) and the ghost's rounds.
void enqueue_density_ghost(sphgpu_space* s, cudaStream_t st, int stages) {
  const LaunchCfg c = cfg_of(s);
  CK(launch_begin_step(s->P, s->prm.max_iter, s->redo.p, s->status.p, st));
  CK(cudaMemsetAsync(s->queue.p, 0, 8 * sizeof(int), st));
  if (stages & SPHGPU_STAGE_DENSITY)
    CK(launch_density(gargs(s, s->dplan_d, 0, nullptr), MODE_FIRST, c, s->num_sms, st));
  if (stages & SPHGPU_STAGE_GHOST) {
    for (int k = 0; k < s->prm.max_iter; k++) {
      CK(launch_ghost(ghargs(s, k, 0, s->P.n), st));
      // re-run density for the particles sent to another round; the kernel
      // returns at once when the round sent none (gate = its redo count)
      CK(cudaMemsetAsync(s->queue.p + 1, 0, sizeof(int), st));
      CK(launch_density(gargs(s, s->dplan_s, 1, s->redo.p + k), MODE_REDO, c,
                        s->num_sms, st));
    }
  }
}

void enqueue_force(sphgpu_space* s, cudaStream_t st) {
  CK(cudaMemsetAsync(s->queue.p + 2, 0, sizeof(int), st));
  CK(launch_force(gargs(s, s->dplan_f, 2, nullptr), MODE_FIRST, cfg_of(s),
                  s->num_sms, st));
}

int check_conv(sphgpu_space* s, cudaStream_t st) {
  int last = 0;
  CK(cudaMemcpyAsync(&last, s->redo.p + s->prm.max_iter - 1, sizeof(int),
                     cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (last > 0)
    return fail(SPHGPU_ENOCONV, "smoothing length failed to converge on " +
                                    std::to_string(last) + " particles");
  return SPHGPU_OK;
}

// The force loop's recursion depends on the post-ghost h_max of every cell
// (cell.h:966-1010 use hydro.h_max); plan it once the ghost has run.
void plan_force(sphgpu_space* s, cudaStream_t st) {
  const int n = s->P.n;
  std::vector<float4> ph(n);
  CK(cudaMemcpyAsync(ph.data(), s->posh.p, sizeof(float4) * n, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  std::vector<float> h(n);
  for (int i = 0; i < n; i++) h[i] = ph[i].w;
  s->space->update_h_after_ghost(h.data());
  s->space->plan_density(s->plan_f, true);
  order_units(s->plan_f);
  s->dplan_f.upload(s->plan_f, st);
  s->force_planned = true;
}

cudaStream_t pick(sphgpu_space* s, void* stream) {
  return stream ? (cudaStream_t)stream : s->stream;
}

int guard(const std::function<int()>& f) {
  try {
    return f();
  } catch (const CudaError& e) {
    return fail(SPHGPU_ECUDA, e.what());
  } catch (const std::bad_alloc&) {
    return fail(SPHGPU_ENOMEM, "host allocation failed");
  } catch (const std::exception& e) {
    const std::string m = e.what();
    if (m.find("no CUDA device") != std::string::npos) return fail(SPHGPU_ENODEV, m);
    return fail(SPHGPU_EINVAL, m);
  }
}

}  // namespace

extern "C" {

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

int sphgpu_space_create(const sphgpu_params* prm, int64_t n, const double* x,
                        const float* v, const float* m, const float* h,
                        const float* u, const int8_t* time_bin,
                        sphgpu_space** out) {
  if (!prm || !x || !v || !m || !h || !u || !time_bin || !out || n <= 0)
    return fail(SPHGPU_EINVAL, "sphgpu_space_create: null argument or n <= 0");
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
    s->space = std::make_unique<Space>(P);
    s->space->build(n, x, h, time_bin);
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
  const int tpi = t->threads_per_particle;
  if (!(tpi == 1 || tpi == 2 || tpi == 4 || tpi == 8) ||
      !(t->jtile == 64 || t->jtile == 128))
    return fail(SPHGPU_EINVAL, "tuning: tpi in {1,2,4,8}, jtile in {64,128}");
  return guard([&]() {
    const bool replan = tpi != s->tune.threads_per_particle;
    s->tune = *t;
    if (replan) {
      build_plans(s);
      if (s->dev) {
        s->dplan_d.upload(s->plan_d, s->stream);
        s->dplan_s.upload(s->plan_s, s->stream);
      }
      s->force_planned = false;
      s->task_d.clear();
      s->task_f.clear();
      s->dtask_d.clear();
      s->dtask_f.clear();
    }
    if (s->graph) {
      cudaGraphExecDestroy(s->graph);
      s->graph = nullptr;
    }
    if (s->dev) CK(cudaStreamSynchronize(s->stream));
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
    s->prm.max_active_bin = max_active_bin;
    s->space->set_activity(max_active_bin);
    build_plans(s);
    s->force_planned = false;
    s->task_d.clear();
    s->task_f.clear();
    s->dtask_d.clear();
    s->dtask_f.clear();
    if (s->graph) {
      cudaGraphExecDestroy(s->graph);
      s->graph = nullptr;
    }
    if (s->dev) {
      const int n = s->P.n;
      std::vector<uint8_t> fl(n);
      for (int i = 0; i < n; i++) fl[i] = s->space->active()[i] ? 1 : 0;
      s->flags.upload(fl.data(), n, s->stream);
      s->dplan_d.upload(s->plan_d, s->stream);
      s->dplan_s.upload(s->plan_s, s->stream);
      CK(cudaStreamSynchronize(s->stream));
    }
    return SPHGPU_OK;
  });
}

int sphgpu_step(sphgpu_space* s, int32_t stages, void* stream) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  if (stages <= 0 || stages > SPHGPU_STAGE_ALL)
    return fail(SPHGPU_EINVAL, "stages must be a non-empty subset of SPHGPU_STAGE_ALL");
  if ((stages & SPHGPU_STAGE_FORCE) && !(stages & SPHGPU_STAGE_GHOST))
    return fail(SPHGPU_EINVAL, "the force stage needs the ghost stage");
  return guard([&]() {
    ensure_device(s);
    cudaStream_t st = pick(s, stream);
    if (stages != SPHGPU_STAGE_ALL) {
      enqueue_density_ghost(s, st, stages);
      if (stages & SPHGPU_STAGE_GHOST) return check_conv(s, st);
      CK(cudaStreamSynchronize(st));
      return SPHGPU_OK;
    }
    if (!s->force_planned) {
      enqueue_density_ghost(s, st, SPHGPU_STAGE_DENSITY | SPHGPU_STAGE_GHOST);
      const int rc = check_conv(s, st);
      if (rc != SPHGPU_OK) return rc;
      plan_force(s, st);
    }
    if (!s->graph) {
      cudaGraph_t g;
      CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      try {
        enqueue_density_ghost(s, st, SPHGPU_STAGE_DENSITY | SPHGPU_STAGE_GHOST);
        enqueue_force(s, st);
      } catch (...) {
        cudaGraph_t dead;
        cudaStreamEndCapture(st, &dead);
        if (dead) cudaGraphDestroy(dead);
        throw;
      }
      CK(cudaStreamEndCapture(st, &g));
      const cudaError_t e = cudaGraphInstantiate(&s->graph, g, 0);
      cudaGraphDestroy(g);
      CK(e);
    }
    CK(cudaGraphLaunch(s->graph, st));
    return check_conv(s, st);
  });
}

int sphgpu_download(sphgpu_space* s, float* fields, int32_t* ints) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  if (!s->dev) return fail(SPHGPU_ESTATE, "no step has run on this space");
  return guard([&]() {
    const int n = s->P.n;
    cudaStream_t st = s->stream;
    DBuf<float> df;
    DBuf<int32_t> di;
    if (fields) df.alloc(24 * (size_t)n);
    if (ints) di.alloc(4 * (size_t)n);
    CK(cudaStreamSynchronize(st));
    CK(launch_collect_out(s->P, s->perm.p, fields ? df.p : nullptr,
                          ints ? di.p : nullptr, st));
    if (fields)
      CK(cudaMemcpyAsync(fields, df.p, sizeof(float) * 24 * (size_t)n,
                         cudaMemcpyDeviceToHost, st));
    if (ints)
      CK(cudaMemcpyAsync(ints, di.p, sizeof(int32_t) * 4 * (size_t)n,
                         cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return SPHGPU_OK;
  });
}

int sphgpu_step_host(sphgpu_space* s, const double* x, const float* v,
                     const float* m, const float* h, const float* u,
                     float* fields, void* stream) {
  if (!s || !x || !v || !m || !h || !u) return fail(SPHGPU_EINVAL, "null argument");
  return guard([&]() {
    ensure_device(s);
    cudaStream_t st = pick(s, stream);
    const int n = s->P.n;
    if (!s->x_stage.p) {
      s->x_stage.alloc(3 * (size_t)n);
      s->v_stage.alloc(3 * (size_t)n);
      s->m_stage.alloc(n);
      s->h_stage.alloc(n);
      s->u_stage.alloc(n);
      s->out_stage.alloc(24 * (size_t)n);
    }
    CK(cudaMemcpyAsync(s->x_stage.p, x, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(s->v_stage.p, v, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(s->m_stage.p, m, sizeof(float) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(s->h_stage.p, h, sizeof(float) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(s->u_stage.p, u, sizeof(float) * n, cudaMemcpyHostToDevice, st));
    CK(launch_permute_in(s->P, s->perm.p, s->x_stage.p, s->v_stage.p, s->m_stage.p,
                         s->h_stage.p, s->u_stage.p, st));
    CK(launch_prepare_posh(s->P, s->top_of.p, s->top_loc.p, st));
    int rc;
    {
      // run the batched step on the same stream
      rc = sphgpu_step(s, SPHGPU_STAGE_ALL, (void*)st);
      if (rc != SPHGPU_OK && rc != SPHGPU_ENOCONV) return rc;
    }
    if (fields) {
      CK(launch_collect_out(s->P, s->perm.p, s->out_stage.p, nullptr, st));
      CK(cudaMemcpyAsync(fields, s->out_stage.p, sizeof(float) * 24 * (size_t)n,
                         cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
    }
    return rc;
  });
}

int sphgpu_force_from_state(sphgpu_space* s, const float* h, const float* rho,
                            const float* f, const float* pressure,
                            const float* soundspeed, const float* balsara,
                            void* stream) {
  if (!s || !h || !rho || !f || !pressure || !soundspeed || !balsara)
    return fail(SPHGPU_EINVAL, "null argument");
  return guard([&]() {
    ensure_device(s);
    cudaStream_t st = pick(s, stream);
    const int n = s->P.n;
    const auto& perm = s->space->perm();
    std::vector<float4> ph(n), f0(n), acc(n, make_float4(0, 0, 0, 0));
    std::vector<float2> f1(n), hv(n);
    std::vector<float> hs(n);
    CK(cudaMemcpyAsync(ph.data(), s->posh.p, sizeof(float4) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    for (int i = 0; i < n; i++) {
      const int k = perm[i];
      ph[i].w = h[k];
      hs[i] = h[k];
      f0[i] = make_float4(rho[k], f[k], pressure[k] / (rho[k] * rho[k]), soundspeed[k]);
      f1[i] = make_float2(balsara[k], pressure[k]);
      hv[i] = make_float2(0.f, 2.f * soundspeed[k]);
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
    for (int i = 0; i < n; i++) {
      const LeafInfo& L = li[s->space->leaf_of()[i]];
      dh[i] = s->space->depth_h()[i];
      if (hs[i] < L.hmin[0]) {
        dh[i] = L.depth[0];
      } else {
        for (int lev = 0; lev < L.nlevels; lev++)
          if (hs[i] >= L.hmin[lev] && hs[i] < L.hmax[lev]) {
            dh[i] = L.depth[lev];
            break;
          }
      }
    }
    s->depth_h.upload(dh.data(), n, st);
    Plan pf;
    s->space->plan_density(pf, true);
    order_units(pf);
    DevPlan dp;
    dp.upload(pf, st);
    CK(cudaMemsetAsync(s->queue.p + 3, 0, sizeof(int), st));
    CK(launch_force(gargs(s, dp, 3, nullptr), MODE_FIRST, cfg_of(s), s->num_sms, st));
    CK(cudaStreamSynchronize(st));
    // the space's step plans assume its own ghost: re-plan on the next step
    s->force_planned = false;
    if (s->graph) {
      cudaGraphExecDestroy(s->graph);
      s->graph = nullptr;
    }
    return SPHGPU_OK;
  });
}

// ---------------------------------------------------------------------------
// Plain per-task form

static void ensure_task_plans(sphgpu_space* s, bool force) {
  auto& plans = force ? s->task_f : s->task_d;
  auto& dplans = force ? s->dtask_f : s->dtask_d;
  if (!plans.empty()) return;
  const Space& sp = *s->space;
  const auto& tasks = sp.tasks();
  plans.resize(tasks.size());
  dplans.resize(tasks.size());
  std::vector<Item> items;
  for (size_t t = 0; t < tasks.size(); t++) {
    items.clear();
    if (tasks[t].cj < 0)
      sp.dosub_self(items, tasks[t].ci, 0, force);
    else
      sp.dosub_pair(items, tasks[t].ci, tasks[t].cj, 0, force);
    std::vector<std::vector<Entry>> per_leaf(sp.leaves().size());
    sp.items_to_entries(items, per_leaf);
    sp.flatten(per_leaf, plans[t]);
    dplans[t].upload(plans[t], s->stream);
  }
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
  DevPlan& dp = force ? s->dtask_f[t] : s->dtask_d[t];
  if (dp.nunits == 0) return SPHGPU_OK;
  LaunchCfg c = cfg_of(s);
  c.persistent = 0;
  if (force)
    CK(launch_force(gargs(s, dp, 4, nullptr), MODE_ACCUM, c, s->num_sms, st));
  else
    CK(launch_density(gargs(s, dp, 4, nullptr), MODE_ACCUM, c, s->num_sms, st));
  return SPHGPU_OK;
}

int sphgpu_begin_loops(sphgpu_space* s, void* stream) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  return guard([&]() {
    ensure_device(s);
    ensure_task_plans(s, false);
    CK(launch_begin_step(s->P, s->prm.max_iter, s->redo.p, s->status.p, pick(s, stream)));
    return SPHGPU_OK;
  });
}

int sphgpu_dosub_self1_density(sphgpu_space* s, int32_t cell, void* stream) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  return guard([&]() {
    ensure_device(s);
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
    cudaStream_t st = pick(s, stream);
    const Cell& c = s->space->cells()[cell];
    if (c.count == 0 || !c.active) return SPHGPU_OK;
    CK(cudaMemsetAsync(s->redo.p, 0, sizeof(int) * s->prm.max_iter, st));
    const auto ur = s->sub_units_of_top[cell];
    DevPlan sub;  // view of the subset units of this top cell
    const int nu = ur.second - ur.first;
    LaunchCfg cfg = cfg_of(s);
    cfg.persistent = 0;
    for (int k = 0; k < s->prm.max_iter; k++) {
      CK(launch_ghost(ghargs(s, k, c.first, c.first + c.count), st));
      int cnt = 0;
      CK(cudaMemcpyAsync(&cnt, s->redo.p + k, sizeof(int), cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      if (cnt == 0) return SPHGPU_OK;
      if (nu > 0) {
        GatherArgs a = gargs(s, s->dplan_s, 4, nullptr);
        a.units = s->dplan_s.units.p + ur.first;
        a.nunits = nu;
        CK(launch_density(a, MODE_REDO, cfg, s->num_sms, st));
      }
      if (k == s->prm.max_iter - 1)
        return fail(SPHGPU_ENOCONV, "smoothing length failed to converge on " +
                                        std::to_string(cnt) + " particles");
    }
    (void)sub;
    return SPHGPU_OK;
  });
}

int sphgpu_dosub_self2_force(sphgpu_space* s, int32_t cell, void* stream) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  return guard([&]() {
    ensure_device(s);
    if (s->task_f.empty()) {
      // the force recursion needs the post-ghost h_max of every cell
      plan_force(s, pick(s, stream));
      ensure_task_plans(s, true);
    }
    const int t = find_task(s, cell, -1);
    if (t < 0) return SPHGPU_OK;
    return run_task(s, t, true, pick(s, stream));
  });
}

int sphgpu_dosub_pair2_force(sphgpu_space* s, int32_t ci, int32_t cj, void* stream) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  return guard([&]() {
    ensure_device(s);
    if (s->task_f.empty()) {
      plan_force(s, pick(s, stream));
      ensure_task_plans(s, true);
    }
    const int t = find_task(s, ci, cj);
    if (t < 0) return fail(SPHGPU_EINVAL, "cells are not neighbours");
    return run_task(s, t, true, pick(s, stream));
  });
}

int sphgpu_do_end_hydro_force(sphgpu_space* s, void* stream) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  return guard([&]() {
    ensure_device(s);
    CK(launch_end_force(s->P, pick(s, stream)));
    return SPHGPU_OK;
  });
}

int sphgpu_step_plain(sphgpu_space* s, void* stream) {
  if (!s) return fail(SPHGPU_EINVAL, "null argument");
  return guard([&]() {
    ensure_device(s);
    cudaStream_t st = pick(s, stream);
    int rc = sphgpu_begin_loops(s, st);
    if (rc) return rc;
    const auto tasks = s->space->tasks();
    for (size_t t = 0; t < tasks.size(); t++) {
      rc = run_task(s, (int)t, false, st);
      if (rc) return rc;
    }
    const int ntop = s->space->cdim()[0] * s->space->cdim()[1] * s->space->cdim()[2];
    for (int c = 0; c < ntop; c++) {
      rc = sphgpu_do_ghost(s, c, st);
      if (rc) return rc;
    }
    if (s->task_f.empty()) {
      plan_force(s, st);
      ensure_task_plans(s, true);
    }
    for (size_t t = 0; t < tasks.size(); t++) {
      rc = run_task(s, (int)t, true, st);
      if (rc) return rc;
    }
    CK(launch_end_force(s->P, st));
    CK(cudaStreamSynchronize(st));
    return SPHGPU_OK;
  });
}

}  // extern "C"
