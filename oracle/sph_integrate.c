/*
 * sph_integrate.c -- the oracle's C restatement of the reference's time
 * integration of gas particles (Minimal SPH, no cosmology, no gravity, no
 * cooling, no entropy floor): the half kicks, the drift with its predicted
 * quantities, and the time-step / time-bin assignment.  TEST INFRASTRUCTURE:
 * only the tests, the smoke check and the CPU baseline of the benchmark use
 * it, as the checker of the GPU integrator; nothing in the product calls it.
 *
 * Every operation follows the reference's C expression for expression, with
 * the same float / double promotions, so that a build with
 * -ffp-contract=off gives the reference's bits:
 *   kick_part (kick.h) + hydro_kick_extra (hydro/Minimal/hydro.h:901-927),
 *   hydro_reset_predicted_values (hydro.h:771-795),
 *   drift_part (drift.h:138-200) + hydro_predict_extra (hydro.h:815-865),
 *     the h clamp of cell_drift_part (cell_drift.c:330-332),
 *   get_part_timestep (timestep.h:142-214) + hydro_compute_timestep
 *     (hydro.h:440-452) + make_integer_timestep (timestep.h:46-86),
 *   the integer time line (timeline.h:36-154),
 *   the per-particle loops of runner_do_kick1 / runner_do_kick2 /
 *     runner_do_timestep (runner_time_integration.c:87-190, :360-470,
 *     :639-760).
 * Arrays are SoA in the caller's order (see sph_oracle.h, integ_state).
 */
#include <float.h>
#include <math.h>
#include <stdint.h>

#include "sph_oracle.h"

#define NUM_TIME_BINS 56
#define MAX_NR_TIMESTEPS (1LL << (NUM_TIME_BINS + 1))
#define NGB_MAX_DELTA_BIN 2
#define KG ((float)(1.936492))
#define HDIM 3.f
#define GAMMA 1.66666666666666667f
#define GAMMA_M1 0.66666666666666667f
/* the reference's min / max macros (minmax.h): a > b ? a : b */
#define MAXF(a, b) ((a) > (b) ? (a) : (b))
#define MINF(a, b) ((a) < (b) ? (a) : (b))

/* ---- integer time line (timeline.h) ------------------------------------ */

static int64_t integer_timestep(int bin) { /* get_integer_timestep :59 */
  if (bin <= 0) return 0;
  return 1LL << (bin + 1);
}

static int time_bin_of(int64_t dti) { /* get_time_bin :78 */
  return (int)((8 * (int)sizeof(int64_t) - 2) - __builtin_clzll((unsigned long long)dti));
}

static int64_t time_begin(int64_t ti, int bin) { /* get_integer_time_begin :107 */
  const int64_t dti = integer_timestep(bin);
  return dti == 0 ? 0 : dti * ((ti - 1) / dti);
}

static int64_t time_end(int64_t ti, int bin) { /* get_integer_time_end :126 */
  const int64_t dti = integer_timestep(bin);
  if (dti == 0) return 0;
  const int64_t mod = ti % dti;
  return mod == 0 ? ti : ti - mod + dti;
}

int sph_integ_max_active_bin(int64_t ti) { /* get_max_active_bin :146 */
  if (ti == 0) return NUM_TIME_BINS;
  int bin = 1;
  while (!((1LL << (bin + 1)) & ti)) ++bin;
  return bin;
}

int64_t sph_integ_time_end(int64_t ti, int bin) { return time_end(ti, bin); }

/* ---- equation of state (adiabatic_index.h / equation_of_state.h) -------- */

static float pressure_from_u(float rho, float u) { return GAMMA_M1 * u * rho; }
static float soundspeed_from_pressure(float rho, float P) {
  return sqrtf(GAMMA * P / rho);
}

/* approx_expf (approx_math.h:35) */
static float approx_expf(float x) {
  return 1.f + x * (1.f + x * (0.5f + x * (1.f / 6.f + 1.f / 24.f * x)));
}

/* ---- kicks ---------------------------------------------------------------- */

/* kick_part + hydro_kick_extra for one particle over [ti_begin, ti_end):
 * dt_kick_hydro = dt_kick_therm = (ti_end - ti_begin) * time_base (the
 * non-cosmological kick factors, kick.h / timeline). */
static void kick_one(const integ_params *ip, integ_state *st, int64_t k, int64_t ti_begin,
                     int64_t ti_end) {
  const double dt_hydro = (ti_end - ti_begin) * ip->time_base;
  const double dt_therm = (ti_end - ti_begin) * ip->time_base;
  for (int d = 0; d < 3; d++) st->v_full[3 * k + d] += st->a[3 * k + d] * dt_hydro;
  /* hydro_kick_extra: dt_therm is passed as float */
  const float dtt = (float)dt_therm;
  const float delta_u = st->u_dt[k] * dtt;
  const float uf = st->u_full[k];
  st->u_full[k] = MAXF(uf + delta_u, 0.5f * uf);
  const float floor_u = 0.f; /* no entropy floor */
  const float energy_min = MAXF(ip->minimal_u, floor_u);
  if (st->u_full[k] < energy_min) {
    st->u_full[k] = energy_min;
    st->u_dt[k] = 0.f;
  }
}

/* hydro_reset_predicted_values (hydro.h:771-795) */
static void reset_predicted(integ_state *st, int64_t k) {
  for (int d = 0; d < 3; d++) st->v[3 * k + d] = st->v_full[3 * k + d];
  st->u[k] = st->u_full[k];
  const float P = pressure_from_u(st->rho[k], st->u[k]);
  const float c = soundspeed_from_pressure(st->rho[k], P);
  st->P[k] = P;
  st->c[k] = c;
  st->v_sig[k] = MAXF(st->v_sig[k], 2.f * c);
}

/* which = 1: runner_do_kick1, the first half kick of particles starting a
 * step at ti_current (part_is_starting, active.h:702); which = 2:
 * runner_do_kick2, the second half kick of active particles ending their
 * step at ti_current, then hydro_reset_predicted_values. */
void sph_integ_kick(const integ_params *ip, integ_state *st, int64_t n, int which,
                    int64_t ti_current, int max_active_bin) {
  for (int64_t k = 0; k < n; k++) {
    const int bin = st->time_bin[k];
    if (bin > max_active_bin) continue;
    const int64_t ti_step = integer_timestep(bin);
    if (which == 1) {
      const int64_t ti_begin = time_begin(ti_current + 1, bin);
      kick_one(ip, st, k, ti_begin, ti_begin + ti_step / 2);
    } else {
      const int64_t ti_begin = time_begin(ti_current, bin) + ti_step / 2;
      kick_one(ip, st, k, ti_begin, ti_begin + ti_step / 2);
      reset_predicted(st, k);
    }
  }
}

/* ---- drift ------------------------------------------------------------------ */

/* drift_part + hydro_predict_extra + the h clamp of cell_drift_part for
 * every particle, from ti_old to ti_current (non-cosmological drift and
 * kick factors: (ti_current - ti_old) * time_base). */
void sph_integ_drift(const integ_params *ip, integ_state *st, int64_t n, int64_t ti_old,
                     int64_t ti_current) {
  const double dt_drift = (ti_current - ti_old) * ip->time_base;
  const double dt_kick_hydro = (ti_current - ti_old) * ip->time_base;
  const double dt_therm = (ti_current - ti_old) * ip->time_base;
  const float dtd = (float)dt_drift, dtt = (float)dt_therm; /* float parameters */
  for (int64_t k = 0; k < n; k++) {
    for (int d = 0; d < 3; d++) st->x[3 * k + d] += st->v_full[3 * k + d] * dt_drift;
    for (int d = 0; d < 3; d++) st->v[3 * k + d] += st->a[3 * k + d] * dt_kick_hydro;
    /* hydro_predict_extra */
    st->u[k] += st->u_dt[k] * dtt;
    const float h_inv = 1.f / st->h[k];
    const float w1 = st->h_dt[k] * h_inv * dtd;
    if (fabsf(w1) < 0.2f)
      st->h[k] *= approx_expf(w1);
    else
      st->h[k] *= expf(w1);
    const float w2 = -HDIM * w1;
    if (fabsf(w2) < 0.2f)
      st->rho[k] *= approx_expf(w2);
    else
      st->rho[k] *= expf(w2);
    const float floor_u = 0.f; /* no entropy floor */
    const float min_u = ip->minimal_u;
    st->u[k] = MAXF(st->u[k], floor_u);
    st->u[k] = MAXF(st->u[k], min_u);
    const float P = pressure_from_u(st->rho[k], st->u[k]);
    const float c = soundspeed_from_pressure(st->rho[k], P);
    st->P[k] = P;
    st->c[k] = c;
    st->v_sig[k] = MAXF(st->v_sig[k], 2.f * c);
    /* cell_drift.c:330-332 */
    st->h[k] = MINF(st->h[k], ip->h_max);
    st->h[k] = MAXF(st->h[k], ip->h_min);
  }
}

/* ---- time step -------------------------------------------------------------- */

static int64_t make_integer_timestep(float new_dt, int old_bin, int min_ngb_bin,
                                     int64_t ti_current, double time_base_inv) {
  int64_t new_dti = (int64_t)(new_dt * time_base_inv);
  int new_bin = time_bin_of(new_dti);
  if (new_bin > min_ngb_bin + NGB_MAX_DELTA_BIN) new_bin = min_ngb_bin + NGB_MAX_DELTA_BIN;
  new_dti = integer_timestep(new_bin);
  const int64_t current_dti = integer_timestep(old_bin);
  const int64_t ti_end = time_end(ti_current, old_bin);
  if (old_bin > 0 && new_dti > 2 * current_dti) new_dti = 2 * current_dti;
  int64_t dti_timeline = MAX_NR_TIMESTEPS;
  while (new_dti < dti_timeline) dti_timeline /= 2;
  new_dti = dti_timeline;
  if (new_dti > current_dti) {
    if ((MAX_NR_TIMESTEPS - ti_end) % new_dti > 0) new_dti = current_dti;
  }
  return new_dti;
}

/* runner_do_timestep for the active particles: the new time bin from the
 * CFL condition and the limit on the change of h, limited by the
 * neighbours' smallest bin (min_ngb_bin, from the force loop).  Returns the
 * number of particles whose time step fell below dt_min (the reference
 * aborts there), 0 when none did. */
int64_t sph_integ_timestep(const integ_params *ip, integ_state *st, int64_t n,
                           const signed char *min_ngb_bin, int64_t ti_current,
                           int max_active_bin) {
  int64_t bad = 0;
  const double time_base_inv = 1.0 / ip->time_base;
  for (int64_t k = 0; k < n; k++) {
    const int bin = st->time_bin[k];
    if (bin > max_active_bin) continue;
    /* hydro_compute_timestep with a = a_factor_sound_speed = 1 (double) */
    const double a = 1.0, a_factor_sound_speed = 1.0;
    const float dt_cfl =
        2.f * KG * ip->CFL * a * st->h[k] / (a_factor_sound_speed * st->v_sig[k]);
    float new_dt = dt_cfl; /* min3 / min4 with FLT_MAX terms */
    const float dt_h_change =
        (st->h_dt[k] != 0.0f) ? fabsf(ip->log_max_h_change * st->h[k] / st->h_dt[k]) : FLT_MAX;
    new_dt = MINF(new_dt, dt_h_change);
    new_dt = (float)MINF((double)new_dt, (double)FLT_MAX); /* dt_max_RMS_displacement */
    const double time_step_factor = 1.0;
    new_dt *= time_step_factor;
    new_dt = (float)(new_dt < ip->dt_max ? (double)new_dt : ip->dt_max);
    if (new_dt < ip->dt_min) bad++;
    const int64_t dti =
        make_integer_timestep(new_dt, bin, min_ngb_bin[k], ti_current, time_base_inv);
    st->time_bin[k] = (signed char)time_bin_of(dti);
  }
  return bad;
}

/* The next synchronisation point: the smallest end of step over all
 * particles (engine's ti_end_min, collected by runner_do_timestep). */
int64_t sph_integ_ti_end_min(const integ_state *st, int64_t n, int64_t ti_current) {
  int64_t t = MAX_NR_TIMESTEPS;
  for (int64_t k = 0; k < n; k++) {
    const int64_t e = time_end(ti_current + 1, st->time_bin[k]);
    if (e < t) t = e;
  }
  return t;
}
