// integrate.cu -- time integration of the gas particles on the device: the
// half kicks, the drift with its predicted quantities (and the periodic wrap
// of a rebuild), and the time-step / time-bin assignment, for a state held
// in the caller's order (sphgpu_integ_state of include/swift_gb300.h).
//
// Each operation is the reference's, expression for expression, with the
// same float / double promotions; every rounding is explicit (the _rn
// intrinsics) so that no multiply-add is fused and the results are the
// reference's bits -- except expf(w) for |w| >= 0.2 in the drift (a large
// change of h in one step), where the device's expf is used:
//   runner_do_kick1 / runner_do_kick2 (runner_time_integration.c:141-184,
//     :421-457) -> kick_part (kick.h) + hydro_kick_extra
//     (hydro/Minimal/hydro.h:901-927) and hydro_reset_predicted_values (:771)
//   cell_drift_part (cell_drift.c:253-332) -> drift_part (drift.h:138-200) +
//     hydro_predict_extra (hydro.h:815-865) and the h clamp
//   runner_do_timestep (runner_time_integration.c:699-749) ->
//     get_part_timestep (timestep.h:142-214), hydro_compute_timestep
//     (hydro.h:440-452), make_integer_timestep (timestep.h:46-86)
//   the integer time line (timeline.h:36-154); box_wrap of the rebuild
//     (space_cell_index.c:113-123).
// Element-wise kernels over the particles (HBM-bound, grid-stride).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cfloat>

#include "../../include/swift_gb300.h"
#include "capi_util.h"
#include "device_sms.h"
#include "sph_types.h"

namespace sphgpu {
namespace {

using capi::DBuf;
using capi::fail;
using capi::guard;

constexpr long long kMaxNrTimesteps = 1LL << (SPH_NUM_TIME_BINS + 1);
constexpr int kNgbMaxDeltaBin = 2;   // time_bin_neighbour_max_delta_bin
#define IG_KG ((float)(1.936492))    // kernel_gamma
#define IG_GAMMA 1.66666666666666667f
#define IG_GAMMA_M1 0.66666666666666667f

__device__ __forceinline__ float maxf_ref(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float minf_ref(float a, float b) { return a < b ? a : b; }

__device__ __forceinline__ long long integer_timestep(int bin) {
  return bin <= 0 ? 0LL : (1LL << (bin + 1));
}
__device__ __forceinline__ int time_bin_of(long long dti) {
  return 62 - __clzll(dti);
}
// The steps are powers of two, so the divisions of the time line are shifts
// and masks (non-negative operands; (ti - 1) / dti truncates to 0 at ti = 0).
__device__ __forceinline__ long long time_begin(long long ti, int bin) {
  const long long dti = integer_timestep(bin);
  if (dti == 0 || ti <= 0) return 0;
  return ((ti - 1) >> (bin + 1)) << (bin + 1);
}
__device__ __forceinline__ long long time_end(long long ti, int bin) {
  const long long dti = integer_timestep(bin);
  if (dti == 0) return 0;
  const long long mod = ti & (dti - 1);
  return mod == 0 ? ti : ti - mod + dti;
}

// gas_pressure_from_internal_energy / gas_soundspeed_from_pressure
// (equation_of_state/ideal_gas/equation_of_state.h:121, :164)
__device__ __forceinline__ float pressure_from_u(float rho, float u) {
  return __fmul_rn(__fmul_rn(IG_GAMMA_M1, u), rho);
}
__device__ __forceinline__ float soundspeed_from_pressure(float rho, float P) {
  return __fsqrt_rn(__fdiv_rn(__fmul_rn(IG_GAMMA, P), rho));
}
// approx_expf (approx_math.h:35), the reference's own 4th-order expansion
__device__ __forceinline__ float approx_expf(float x) {
  float t = __fadd_rn(1.f / 6.f, __fmul_rn(1.f / 24.f, x));
  t = __fadd_rn(0.5f, __fmul_rn(x, t));
  t = __fadd_rn(1.f, __fmul_rn(x, t));
  return __fadd_rn(1.f, __fmul_rn(x, t));
}
// float += float * double, evaluated in double as C does
__device__ __forceinline__ float add_prod_d(float v, float a, double dt) {
  return __double2float_rn(__dadd_rn((double)v, __dmul_rn((double)a, dt)));
}

__global__ void kick_k(sphgpu_integ_params ip, sphgpu_integ_state st, long long n, int which,
                       long long ti_current, int max_active_bin) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    const int bin = st.time_bin[k];
    if (bin > max_active_bin) continue;
    const long long ti_step = integer_timestep(bin);
    const long long ti_begin = which == 1 ? time_begin(ti_current + 1, bin)
                                          : time_begin(ti_current, bin) + ti_step / 2;
    const long long ti_end = ti_begin + ti_step / 2;
    const double dt = __dmul_rn((double)(ti_end - ti_begin), ip.time_base);
    for (int d = 0; d < 3; d++)
      st.v_full[3 * k + d] = add_prod_d(st.v_full[3 * k + d], st.a[3 * k + d], dt);
    // hydro_kick_extra (dt_therm passed as float)
    const float dtt = __double2float_rn(dt);
    const float delta_u = __fmul_rn(st.u_dt[k], dtt);
    const float uf = st.u_full[k];
    float ufn = maxf_ref(__fadd_rn(uf, delta_u), __fmul_rn(0.5f, uf));
    const float energy_min = maxf_ref(ip.minimal_u, 0.f);  // no entropy floor
    if (ufn < energy_min) {
      ufn = energy_min;
      st.u_dt[k] = 0.f;
    }
    st.u_full[k] = ufn;
    if (which == 2) {  // hydro_reset_predicted_values
      for (int d = 0; d < 3; d++) st.v[3 * k + d] = st.v_full[3 * k + d];
      st.u[k] = ufn;
      const float P = pressure_from_u(st.rho[k], ufn);
      const float c = soundspeed_from_pressure(st.rho[k], P);
      st.P[k] = P;
      st.c[k] = c;
      st.v_sig[k] = maxf_ref(st.v_sig[k], __fmul_rn(2.f, c));
    }
  }
}

__global__ void drift_k(sphgpu_integ_params ip, sphgpu_integ_state st, long long n,
                        long long ti_old, long long ti_current, int wrap) {
  const double dt = __dmul_rn((double)(ti_current - ti_old), ip.time_base);
  const float dtf = __double2float_rn(dt);
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    for (int d = 0; d < 3; d++) {
      double x = __dadd_rn(st.x[3 * k + d], __dmul_rn((double)st.v_full[3 * k + d], dt));
      if (wrap) {  // box_wrap at the rebuild that follows
        const double D = ip.dim[d];
        x = x < 0.0 ? __dadd_rn(x, D) : (x >= D ? __dsub_rn(x, D) : x);
        if (x == D) x = 0.0;  // wrapped exactly onto the far edge
      }
      st.x[3 * k + d] = x;
    }
    for (int d = 0; d < 3; d++)
      st.v[3 * k + d] = add_prod_d(st.v[3 * k + d], st.a[3 * k + d], dt);
    // hydro_predict_extra
    float u = __fadd_rn(st.u[k], __fmul_rn(st.u_dt[k], dtf));
    float h = st.h[k];
    const float h_inv = __fdiv_rn(1.f, h);
    const float w1 = __fmul_rn(__fmul_rn(st.h_dt[k], h_inv), dtf);
    h = __fmul_rn(h, fabsf(w1) < 0.2f ? approx_expf(w1) : expf(w1));
    const float w2 = __fmul_rn(-3.f, w1);
    const float rho = __fmul_rn(st.rho[k], fabsf(w2) < 0.2f ? approx_expf(w2) : expf(w2));
    u = maxf_ref(u, 0.f);  // no entropy floor
    u = maxf_ref(u, ip.minimal_u);
    const float P = pressure_from_u(rho, u);
    const float c = soundspeed_from_pressure(rho, P);
    st.u[k] = u;
    st.rho[k] = rho;
    st.P[k] = P;
    st.c[k] = c;
    st.v_sig[k] = maxf_ref(st.v_sig[k], __fmul_rn(2.f, c));
    h = minf_ref(h, ip.h_max);
    h = maxf_ref(h, ip.h_min);
    st.h[k] = h;
  }
}

// out[0]: particles whose step fell below dt_min; out[1]: ti_end_min over
// every particle after the update (atomicMin).
__global__ void timestep_k(sphgpu_integ_params ip, sphgpu_integ_state st, long long n,
                           long long ti_current, int max_active_bin, double time_base_inv,
                           unsigned long long* out) {
  unsigned long long bad = 0, tmin = (unsigned long long)kMaxNrTimesteps;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    int bin = st.time_bin[k];
    if (bin <= max_active_bin) {
      // hydro_compute_timestep, a = a_factor_sound_speed = 1 (double)
      const float f1 = __fmul_rn(__fmul_rn(2.f, IG_KG), ip.CFL);
      const double num = __dmul_rn(__dmul_rn((double)f1, 1.0), (double)st.h[k]);
      const double den = __dmul_rn(1.0, (double)st.v_sig[k]);
      float new_dt = __double2float_rn(__ddiv_rn(num, den));
      const float hdt = st.h_dt[k];
      const float dt_h_change =
          hdt != 0.0f ? fabsf(__fdiv_rn(__fmul_rn(ip.log_max_h_change, st.h[k]), hdt)) : FLT_MAX;
      new_dt = minf_ref(new_dt, dt_h_change);
      new_dt = (double)new_dt < (double)FLT_MAX ? new_dt : __double2float_rn((double)FLT_MAX);
      new_dt = __double2float_rn(__dmul_rn((double)new_dt, 1.0));  // time_step_factor
      new_dt = (double)new_dt < ip.dt_max ? new_dt : __double2float_rn(ip.dt_max);
      if ((double)new_dt < ip.dt_min) bad++;
      // make_integer_timestep
      long long new_dti = __double2ll_rz(__dmul_rn((double)new_dt, time_base_inv));
      int new_bin = time_bin_of(new_dti);
      new_bin = min(new_bin, (int)st.min_ngb_bin[k] + kNgbMaxDeltaBin);
      new_dti = integer_timestep(new_bin);
      const long long current_dti = integer_timestep(bin);
      const long long ti_end = time_end(ti_current, bin);
      if (bin > 0) new_dti = min(new_dti, 2 * current_dti);
      // the largest power of two on the time line not above new_dti (the
      // reference halves max_nr_timesteps until it is not above new_dti)
      new_dti = new_dti >= kMaxNrTimesteps ? kMaxNrTimesteps
              : (new_dti <= 0 ? 0 : (1LL << (63 - __clzll(new_dti))));
      if (new_dti > current_dti && ((kMaxNrTimesteps - ti_end) & (new_dti - 1)) != 0)
        new_dti = current_dti;
      bin = time_bin_of(new_dti);
      st.time_bin[k] = (int8_t)bin;
    }
    tmin = min(tmin, (unsigned long long)time_end(ti_current + 1, bin));
  }
  for (int o = 16; o > 0; o >>= 1) {
    bad += __shfl_xor_sync(0xffffffffu, bad, o);
    tmin = min(tmin, __shfl_xor_sync(0xffffffffu, tmin, o));
  }
  if ((threadIdx.x & 31) == 0) {
    if (bad) atomicAdd(&out[0], bad);
    atomicMin(&out[1], tmin);
  }
}

int grid_for(long long n) { return (int)std::max(1LL, std::min((n + 255) / 256, 8LL * sm_count())); }

int check_args(const sphgpu_integ_params* ip, const sphgpu_integ_state* st, long long n) {
  if (!ip || !st || n < 0) return fail(SPHGPU_EINVAL, "integrator: null argument or n < 0");
  if (!(ip->time_base > 0.0)) return fail(SPHGPU_EINVAL, "integrator: time_base must be > 0");
  return SPHGPU_OK;
}

}  // namespace
}  // namespace sphgpu

using namespace sphgpu;
using sphgpu::capi::fail;
using sphgpu::capi::guard;
using sphgpu::capi::DBuf;

extern "C" {

int sphgpu_integ_kick(const sphgpu_integ_params* ip, const sphgpu_integ_state* st, int64_t n,
                      int32_t which, int64_t ti_current, int32_t max_active_bin, void* stream) {
  if (int rc = check_args(ip, st, n)) return rc;
  if (which != 1 && which != 2) return fail(SPHGPU_EINVAL, "sphgpu_integ_kick: which is 1 or 2");
  return guard([&]() {
    if (n == 0) return SPHGPU_OK;
    kick_k<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(*ip, *st, n, which, ti_current,
                                                          max_active_bin);
    CK(cudaGetLastError());
    return SPHGPU_OK;
  });
}

int sphgpu_integ_drift(const sphgpu_integ_params* ip, const sphgpu_integ_state* st, int64_t n,
                       int64_t ti_old, int64_t ti_current, int32_t wrap, void* stream) {
  if (int rc = check_args(ip, st, n)) return rc;
  if (ti_current < ti_old) return fail(SPHGPU_EINVAL, "sphgpu_integ_drift: drift to the past");
  return guard([&]() {
    if (n == 0) return SPHGPU_OK;
    drift_k<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(*ip, *st, n, ti_old, ti_current,
                                                           wrap && ip->periodic);
    CK(cudaGetLastError());
    return SPHGPU_OK;
  });
}

int sphgpu_integ_timestep(const sphgpu_integ_params* ip, const sphgpu_integ_state* st,
                          int64_t n, int64_t ti_current, int32_t max_active_bin,
                          int64_t* ti_end_min, int64_t* n_too_small, void* stream) {
  if (int rc = check_args(ip, st, n)) return rc;
  if (!ti_end_min || !n_too_small || !st->min_ngb_bin)
    return fail(SPHGPU_EINVAL, "sphgpu_integ_timestep: null argument");
  return guard([&]() {
    cudaStream_t s = (cudaStream_t)stream;
    DBuf<unsigned long long> out;
    out.alloc(2);
    const unsigned long long init[2] = {0ULL, (unsigned long long)kMaxNrTimesteps};
    CK(cudaMemcpyAsync(out.p, init, sizeof(init), cudaMemcpyHostToDevice, s));
    if (n > 0)
      timestep_k<<<grid_for(n), 256, 0, s>>>(*ip, *st, n, ti_current, max_active_bin,
                                             1.0 / ip->time_base, out.p);
    CK(cudaGetLastError());
    unsigned long long res[2];
    CK(cudaMemcpyAsync(res, out.p, sizeof(res), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    *n_too_small = (int64_t)res[0];
    *ti_end_min = (int64_t)res[1];
    return SPHGPU_OK;
  });
}

int sphgpu_integ_max_active_bin(int64_t ti) {
  if (ti == 0) return SPH_NUM_TIME_BINS;
  int bin = 1;
  while (!((1LL << (bin + 1)) & ti)) ++bin;
  return bin;
}

}  // extern "C"
