/* sph_oracle.c -- CPU restatement of SWIFT's Minimal-SPH / Wendland-C2
 * neighbour-loop hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: tests/, the smoke check
 * and bench.py's CPU-baseline leg call it to check or to time against; the
 * GPU library never links it.
 *
 * It restates, in plain serial C, the reference algorithm for one
 * density -> ghost -> force pass over a periodic box:
 *   - top-level grid and particle -> cell index (space_regrid.c:39-140,
 *     space_cell_index.c:64-190), the in-place bucket permutation
 *     (space_sort.c:42-93), the octree split (space_split.c:53-300,
 *     cell_split.c:55-175) and h-depth (cell.h:1787);
 *   - the per-cell sorts along 13 axes (runner_sort.c:70-180, :203-463);
 *   - the density loops DOSELF1 / DOPAIR1 and their recursion
 *     (runner_doiact_functions_hydro.h:2299, :1234, :3037, :2933);
 *   - the ghost's Newton-Raphson iteration on h with subset re-runs
 *     (runner_ghost.c:1113-1635; DOSELF_SUBSET :1108, DOPAIR_SUBSET :855,
 *     DOSUB_*_SUBSET :3290-3360);
 *   - the force loops DOSELF2 / DOPAIR2 and their recursion (:2624, :1601,
 *     :3203, :3102) and the end of force (runner_others.c:815);
 *   - the particle physics of hydro/Minimal/hydro_iact.h and hydro.h with the
 *     Wendland C2 kernel of kernel_hydro.h:121-147, :257-284.
 * Loop orders and floating-point expression orders follow the reference so
 * that, built with -O2 -ffp-contract=off, its sums are bit-identical to the
 * reference's own loops run in the same task order (oracle/ref_harness.c).
 * On top it counts, per particle, the neighbours each loop interacted with
 * (the reference has no such counter for Minimal SPH), and it offers an
 * FP64 O(N^2)-free brute force (cell-list based) for error statements.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "sph_oracle.h"

/* ------------------------------------------------------------------------ */
/* Constants of the scheme (values and float/double evaluation as in
 * kernel_hydro.h, dimension.h, adiabatic_index.h, hydro_parameters.h).    */

#define KG ((float)(1.936492))                       /* kernel_gamma        */
#define KCONST ((float)(21. * M_1_PI / 2.))          /* kernel_constant     */
#define KG_INV ((float)(1. / KG))
#define KG2 ((float)(KG * KG))
#define KG_INV_DIM ((float)(1. / (KG * KG * KG)))
#define KG_INV_DIM1 ((float)(1. / (KG * KG * KG * KG)))
#define KROOT ((float)(1.f) * KCONST * KG_INV_DIM)  /* W(0) / h^-3        */
#define HDIM 3.f
#define HDIM_INV 0.3333333333f
#define GAMMA 1.66666666666666667f
#define GAMMA_M1 0.66666666666666667f
#define VISC_BETA 3.0f
#define STRETCH 1.10f
#define MAXRELDX 0.1f
#define SPLIT_SIZE 400
#define RECURSE_SIZE 100
#define NUM_TIME_BINS 56 /* timeline.h:36 */

static const float wendland_c2[12] = {4.f, -15.f, 20.f, -10.f, 0.f, 1.f,
                                      0.f, 0.f,   0.f,  0.f,   0.f, 0.f};

/* Unit vectors of the 13 sort axes; the decimal literals are those of the
 * reference's table (sort_part.h:42-57) so that the double products, and
 * hence the float sort keys, are bit-identical. */
#define S3 5.773502691896258e-01
#define S2 7.071067811865475e-01
static const double axis[13][3] = {
    {S3, S3, S3},  {S2, S2, 0.0},  {S3, S3, -S3}, {S2, 0.0, S2},  {1.0, 0.0, 0.0},
    {S2, 0.0, -S2}, {S3, -S3, S3}, {S2, -S2, 0.0}, {S3, -S3, -S3}, {0.0, S2, S2},
    {0.0, 1.0, 0.0}, {0.0, S2, -S2}, {0.0, 0.0, 1.0}};

/* Child-pair lists for the pair recursion, per axis, in the reference's
 * order (cell.c:63-...).  The set is "children that touch"; the order fixes
 * the summation order and therefore the bits of the sums. */
static const int split_pairs_n[13] = {1, 4, 1, 4, 16, 4, 1, 4, 1, 4, 16, 4, 16};
static const unsigned char split_pairs[13][16][2] = {
    {{7, 0}},
    {{6, 0}, {7, 1}, {6, 1}, {7, 0}},
    {{6, 1}},
    {{5, 0}, {7, 2}, {5, 2}, {7, 0}},
    {{4, 0}, {5, 0}, {6, 0}, {7, 0}, {4, 1}, {5, 1}, {6, 1}, {7, 1},
     {4, 2}, {5, 2}, {6, 2}, {7, 2}, {4, 3}, {5, 3}, {6, 3}, {7, 3}},
    {{4, 1}, {6, 3}, {4, 3}, {6, 1}},
    {{5, 2}},
    {{4, 3}, {5, 2}, {4, 2}, {5, 3}},
    {{4, 3}},
    {{3, 0}, {7, 4}, {3, 4}, {7, 0}},
    {{2, 0}, {3, 0}, {6, 0}, {7, 0}, {2, 1}, {3, 1}, {6, 1}, {7, 1},
     {2, 4}, {3, 4}, {6, 4}, {7, 4}, {2, 5}, {3, 5}, {6, 5}, {7, 5}},
    {{2, 1}, {6, 5}, {2, 5}, {6, 1}},
    {{1, 0}, {3, 0}, {5, 0}, {7, 0}, {1, 2}, {3, 2}, {5, 2}, {7, 2},
     {1, 4}, {3, 4}, {5, 4}, {7, 4}, {1, 6}, {3, 6}, {5, 6}, {7, 6}}};

static inline float fmaxf_ref(float a, float b) { return a > b ? a : b; }
static inline float fminf_ref(float a, float b) { return a < b ? a : b; }

/* ------------------------------------------------------------------------ */
/* Data structures                                                          */

typedef struct {
  float d;
  int i;
} sentry;

typedef struct {
  long long id;
  double x[3];
  float v[3], a[3];
  float mass, h, u, u_dt, rho;
  float wcount, wcount_dh, rho_dh, div_v, rot_v[3];
  float f, pressure, soundspeed, v_sig, h_dt, balsara;
  signed char time_bin, depth_h;
  signed char min_ngb_bin; /* limiter_data.min_ngb_time_bin */
  int ngb_d, ngb_d_first, ngb_f, ghost_iters;
} opart;

struct olink;
typedef struct ocell {
  double loc[3], width[3];
  float dmin, h_min_allowed, h_max_allowed;
  float h_max, h_max_active, h_max_old;
  int count, depth, split, active;
  opart *parts;
  struct ocell *progeny[8], *parent;
  sentry *sort[13];
  struct olink *density;
} ocell;

typedef struct otask {
  int is_pair;
  ocell *ci, *cj;
} otask;

typedef struct olink {
  otask *t;
  struct olink *next;
} olink;

typedef struct {
  const oracle_params *prm;
  double dim[3];
  int periodic;
  int max_active_bin;
} octx;

static void *ocalloc(size_t n, size_t sz) {
  void *p = calloc(n ? n : 1, sz ? sz : 1);
  if (!p) {
    fprintf(stderr, "sph_oracle: out of memory\n");
    abort();
  }
  return p;
}

static inline int part_active(const octx *e, const opart *p) {
  return p->time_bin <= e->max_active_bin;
}

/* ------------------------------------------------------------------------ */
/* Kernel and particle physics                                              */

static inline void kernel_deval(float u, float *W, float *dW_dx) {
  const float x = u * KG_INV;
  const int t = (int)(x * (float)1);
  const int ind = t > 1 ? 1 : t;
  const float *c = &wendland_c2[ind * 6];
  float w = c[0] * x + c[1];
  float dw = c[0];
  for (int k = 2; k <= 5; k++) {
    dw = dw * x + w;
    w = x * w + c[k];
  }
  w = fmaxf_ref(w, 0.f);
  dw = fminf_ref(dw, 0.f);
  *W = w * KCONST * KG_INV_DIM;
  *dW_dx = dw * KCONST * KG_INV_DIM1;
}

/* runner_iact_density (hydro_iact.h:53-121) */
static void iact_density(float r2, const float dx[3], float hi, float hj,
                         opart *pi, opart *pj) {
  float wi, wj, wi_dx, wj_dx;
  const float r = sqrtf(r2);
  const float r_inv = r ? 1.0f / r : 0.0f;
  const float mi = pi->mass, mj = pj->mass;
  const float hi_inv = 1.f / hi;
  const float ui = r * hi_inv;
  kernel_deval(ui, &wi, &wi_dx);
  pi->rho += mj * wi;
  pi->rho_dh -= mj * (HDIM * wi + ui * wi_dx);
  pi->wcount += wi;
  pi->wcount_dh -= (HDIM * wi + ui * wi_dx);
  const float hj_inv = 1.f / hj;
  const float uj = r * hj_inv;
  kernel_deval(uj, &wj, &wj_dx);
  pj->rho += mi * wj;
  pj->rho_dh -= mi * (HDIM * wj + uj * wj_dx);
  pj->wcount += wj;
  pj->wcount_dh -= (HDIM * wj + uj * wj_dx);
  const float faci = mj * wi_dx * r_inv;
  const float facj = mi * wj_dx * r_inv;
  float dv[3], cv[3];
  dv[0] = pi->v[0] - pj->v[0];
  dv[1] = pi->v[1] - pj->v[1];
  dv[2] = pi->v[2] - pj->v[2];
  const float dvdr = dv[0] * dx[0] + dv[1] * dx[1] + dv[2] * dx[2];
  pi->div_v -= faci * dvdr;
  pj->div_v -= facj * dvdr;
  cv[0] = dv[1] * dx[2] - dv[2] * dx[1];
  cv[1] = dv[2] * dx[0] - dv[0] * dx[2];
  cv[2] = dv[0] * dx[1] - dv[1] * dx[0];
  pi->rot_v[0] += faci * cv[0];
  pi->rot_v[1] += faci * cv[1];
  pi->rot_v[2] += faci * cv[2];
  pj->rot_v[0] += facj * cv[0];
  pj->rot_v[1] += facj * cv[1];
  pj->rot_v[2] += facj * cv[2];
  pi->ngb_d++;
  pj->ngb_d++;
}

/* runner_iact_nonsym_density (hydro_iact.h:137-189) */
static void iact_nonsym_density(float r2, const float dx[3], float hi,
                                float hj, opart *pi, const opart *pj) {
  float wi, wi_dx;
  (void)hj;
  const float mj = pj->mass;
  const float r = sqrtf(r2);
  const float r_inv = r ? 1.0f / r : 0.0f;
  const float h_inv = 1.f / hi;
  const float ui = r * h_inv;
  kernel_deval(ui, &wi, &wi_dx);
  pi->rho += mj * wi;
  pi->rho_dh -= mj * (HDIM * wi + ui * wi_dx);
  pi->wcount += wi;
  pi->wcount_dh -= (HDIM * wi + ui * wi_dx);
  const float faci = mj * wi_dx * r_inv;
  float dv[3], cv[3];
  dv[0] = pi->v[0] - pj->v[0];
  dv[1] = pi->v[1] - pj->v[1];
  dv[2] = pi->v[2] - pj->v[2];
  const float dvdr = dv[0] * dx[0] + dv[1] * dx[1] + dv[2] * dx[2];
  pi->div_v -= faci * dvdr;
  cv[0] = dv[1] * dx[2] - dv[2] * dx[1];
  cv[1] = dv[2] * dx[0] - dv[0] * dx[2];
  cv[2] = dv[0] * dx[1] - dv[1] * dx[0];
  pi->rot_v[0] += faci * cv[0];
  pi->rot_v[1] += faci * cv[1];
  pi->rot_v[2] += faci * cv[2];
  pi->ngb_d++;
}

/* Shared part of runner_iact_force / runner_iact_nonsym_force
 * (hydro_iact.h:243-366, :378-490) with a = 1, H = 0. */
static void iact_force_impl(float r2, const float dx[3], float hi, float hj,
                            opart *pi, opart *pj, int sym) {
  const float fac_mu = 1.f;
  const float a2_Hubble = 1.f * 1.f * 0.f;
  const float r = sqrtf(r2);
  const float r_inv = r ? 1.0f / r : 0.0f;
  const float mi = pi->mass, mj = pj->mass;
  const float rhoi = pi->rho, rhoj = pj->rho;
  const float pressurei = pi->pressure, pressurej = pj->pressure;
  const float hi_inv = 1.0f / hi;
  const float hi2 = hi_inv * hi_inv;
  const float hid_inv = hi2 * hi2;
  const float xi = r * hi_inv;
  float wi, wi_dx;
  kernel_deval(xi, &wi, &wi_dx);
  const float wi_dr = hid_inv * wi_dx;
  const float hj_inv = 1.0f / hj;
  const float hj2 = hj_inv * hj_inv;
  const float hjd_inv = hj2 * hj2;
  const float xj = r * hj_inv;
  float wj, wj_dx;
  kernel_deval(xj, &wj, &wj_dx);
  const float wj_dr = hjd_inv * wj_dx;
  const float f_ij = 1.f - pi->f / mj;
  const float f_ji = 1.f - pj->f / mi;
  const float P_over_rho2_i = pressurei / (rhoi * rhoi) * f_ij;
  const float P_over_rho2_j = pressurej / (rhoj * rhoj) * f_ji;
  const float dvdr = (pi->v[0] - pj->v[0]) * dx[0] +
                     (pi->v[1] - pj->v[1]) * dx[1] +
                     (pi->v[2] - pj->v[2]) * dx[2];
  const float dvdr_Hubble = dvdr + a2_Hubble * r2;
  const float omega_ij = fminf_ref(dvdr_Hubble, 0.f);
  const float mu_ij = fac_mu * r_inv * omega_ij;
  const float v_sig = pi->soundspeed + pj->soundspeed - VISC_BETA * mu_ij;
  const float balsara_i = pi->balsara, balsara_j = pj->balsara;
  const float rho_ij = 0.5f * (rhoi + rhoj);
  const float visc = -0.25f * v_sig * (balsara_i + balsara_j) * mu_ij / rho_ij;
  const float visc_acc_term = 0.5f * visc * (wi_dr * f_ij + wj_dr * f_ji) * r_inv;
  const float sph_acc_term = (P_over_rho2_i * wi_dr + P_over_rho2_j * wj_dr) * r_inv;
  const float acc = sph_acc_term + visc_acc_term + 0.f;
  pi->a[0] -= mj * acc * dx[0];
  pi->a[1] -= mj * acc * dx[1];
  pi->a[2] -= mj * acc * dx[2];
  if (sym) {
    pj->a[0] += mi * acc * dx[0];
    pj->a[1] += mi * acc * dx[1];
    pj->a[2] += mi * acc * dx[2];
  }
  const float sph_du_term_i = P_over_rho2_i * dvdr * r_inv * wi_dr;
  const float sph_du_term_j = P_over_rho2_j * dvdr * r_inv * wj_dr;
  const float visc_du_term = 0.5f * visc_acc_term * dvdr_Hubble;
  const float du_dt_i = sph_du_term_i + visc_du_term;
  const float du_dt_j = sph_du_term_j + visc_du_term;
  pi->u_dt += du_dt_i * mj;
  if (sym) pj->u_dt += du_dt_j * mi;
  pi->h_dt -= mj * dvdr * r_inv / rhoj * wi_dr * f_ij;
  if (sym) pj->h_dt -= mi * dvdr * r_inv / rhoi * wj_dr * f_ji;
  pi->v_sig = fmaxf_ref(pi->v_sig, v_sig);
  if (sym) pj->v_sig = fmaxf_ref(pj->v_sig, v_sig);
  pi->ngb_f++;
  if (sym) pj->ngb_f++;
  /* runner_iact_timebin / runner_iact_nonsym_timebin
   * (timestep_limiter_iact.h:34-72), called after every force interaction
   * (runner_doiact_functions_hydro.h:161, :489, ...) */
  if (pj->time_bin > 0 && pj->time_bin < pi->min_ngb_bin) pi->min_ngb_bin = pj->time_bin;
  if (sym && pi->time_bin > 0 && pi->time_bin < pj->min_ngb_bin)
    pj->min_ngb_bin = pi->time_bin;
}

static inline void iact_force(float r2, const float dx[3], float hi, float hj,
                              opart *pi, opart *pj) {
  iact_force_impl(r2, dx, hi, hj, pi, pj, 1);
}
static inline void iact_nonsym_force(float r2, const float dx[3], float hi,
                                     float hj, opart *pi, opart *pj) {
  iact_force_impl(r2, dx, hi, hj, pi, pj, 0);
}

/* hydro_init_part (hydro.h:517) */
static void init_part(opart *p) {
  p->wcount = 0.f;
  p->wcount_dh = 0.f;
  p->rho = 0.f;
  p->rho_dh = 0.f;
  p->div_v = 0.f;
  p->rot_v[0] = p->rot_v[1] = p->rot_v[2] = 0.f;
  p->ngb_d = 0;
}

/* hydro_end_density (hydro.h:543-574), a = 1 */
static void end_density(opart *p) {
  const float h = p->h;
  const float h_inv = 1.0f / h;
  const float h_inv_dim = h_inv * h_inv * h_inv;
  const float h_inv_dim_plus_one = h_inv_dim * h_inv;
  p->rho += p->mass * KROOT;
  p->rho_dh -= HDIM * p->mass * KROOT;
  p->wcount += KROOT;
  p->wcount_dh -= HDIM * KROOT;
  p->rho *= h_inv_dim;
  p->rho_dh *= h_inv_dim_plus_one;
  p->wcount *= h_inv_dim;
  p->wcount_dh *= h_inv_dim_plus_one;
  const float rho_inv = 1.f / p->rho;
  const float a_inv2 = 1.f;
  p->rot_v[0] *= h_inv_dim_plus_one * a_inv2 * rho_inv;
  p->rot_v[1] *= h_inv_dim_plus_one * a_inv2 * rho_inv;
  p->rot_v[2] *= h_inv_dim_plus_one * a_inv2 * rho_inv;
  p->div_v *= h_inv_dim_plus_one * a_inv2 * rho_inv;
}

/* hydro_part_has_no_neighbours (hydro.h:626) */
static void no_neighbours(opart *p) {
  const float h = p->h;
  const float h_inv = 1.0f / h;
  const float h_inv_dim = h_inv * h_inv * h_inv;
  p->rho = p->mass * KROOT * h_inv_dim;
  p->wcount = KROOT * h_inv_dim;
  p->rho_dh = 0.f;
  p->wcount_dh = 0.f;
  p->div_v = 0.f;
  p->rot_v[0] = p->rot_v[1] = p->rot_v[2] = 0.f;
}

/* hydro_prepare_force (hydro.h:669-739) + hydro_reset_acceleration (:749) */
static void prepare_force(const octx *e, opart *p) {
  const float fac_Balsara_eps = 1.f;
  const float h_inv = 1.f / p->h;
  const float curl_v = sqrtf(p->rot_v[0] * p->rot_v[0] +
                             p->rot_v[1] * p->rot_v[1] +
                             p->rot_v[2] * p->rot_v[2]);
  const float div_physical_v = p->div_v + HDIM * 0.f;
  const float abs_div_physical_v = fabsf(div_physical_v);
  const float pressure = GAMMA_M1 * p->u * p->rho;
  const float soundspeed = sqrtf(GAMMA * pressure / p->rho);
  const float common_factor = p->h * HDIM_INV / p->wcount;
  float grad_h_term;
  if (p->h > 0.9999f * e->prm->h_max) {
    grad_h_term = 0.f;
  } else {
    const float grad_W_term = common_factor * p->wcount_dh;
    if (grad_W_term < -0.9999f)
      grad_h_term = 0.f;
    else
      grad_h_term = common_factor * p->rho_dh / (1.f + grad_W_term);
  }
  const float balsara = e->prm->alpha * abs_div_physical_v /
                        (abs_div_physical_v + curl_v +
                         0.0001f * fac_Balsara_eps * soundspeed * h_inv);
  p->f = grad_h_term;
  p->pressure = pressure;
  p->soundspeed = soundspeed;
  p->balsara = balsara;
  /* reset acceleration */
  p->a[0] = p->a[1] = p->a[2] = 0.f;
  p->u_dt = 0.f;
  p->h_dt = 0.f;
  p->v_sig = 2.f * p->soundspeed;
  p->ngb_f = 0;
  /* timestep_limiter_prepare_force (timestep_limiter.h:35) */
  p->min_ngb_bin = NUM_TIME_BINS + 1;
}

/* ------------------------------------------------------------------------ */
/* Geometry helpers                                                         */

/* space_getsid_and_swap_cells (space_getsid.h:47-80): the direction index
 * of cj relative to ci, with a swap into one of the 13 canonical axes. */
static int getsid_and_swap(const octx *e, ocell **ci, ocell **cj,
                           double shift[3]) {
  double dx[3];
  for (int k = 0; k < 3; k++) {
    dx[k] = (*cj)->loc[k] - (*ci)->loc[k];
    if (e->periodic && dx[k] < -e->dim[k] / 2)
      shift[k] = e->dim[k];
    else if (e->periodic && dx[k] > e->dim[k] / 2)
      shift[k] = -e->dim[k];
    else
      shift[k] = 0.0;
    dx[k] += shift[k];
  }
  int idx = 0;
  for (int k = 0; k < 3; k++)
    idx = 3 * idx + ((dx[k] < 0.0) ? 0 : ((dx[k] > 0.0) ? 2 : 1));
  if (idx < 13) { /* the axis runs from cj to ci: swap */
    ocell *t = *ci;
    *ci = *cj;
    *cj = t;
    for (int k = 0; k < 3; k++) shift[k] = -shift[k];
    return idx;
  }
  return 26 - idx;
}

static inline int can_recurse_subself(const ocell *c) {
  return KG * c->h_max_active < 0.5f * c->dmin;
}
static inline int can_recurse_subpair(const ocell *c) {
  return (KG * c->h_max_active + 0.f) < 0.5f * c->dmin;
}
static inline int can_recurse_subself2(const ocell *c) {
  return c->split && (KG * c->h_max < 0.5f * c->dmin);
}
static inline int can_recurse_subpair2(const ocell *c) {
  return (KG * c->h_max + 0.f) < 0.5f * c->dmin;
}
static inline int can_recurse_pair_old(const ocell *c) {
  return c->split && ((KG * c->h_max_old + 0.f) < 0.5f * c->dmin);
}
static inline int can_recurse_self_old(const ocell *c) {
  return c->split && (KG * c->h_max_old < 0.5f * c->dmin);
}

/* ------------------------------------------------------------------------ */
/* Density loops                                                            */

static void dopair1(const octx *e, ocell *ci, ocell *cj, int lmin, int lmax,
                    int sid, const double shift[3]) {
  double rshift = 0.0;
  for (int k = 0; k < 3; k++) rshift += shift[k] * axis[sid][k];
  const sentry *sort_i = ci->sort[sid];
  const sentry *sort_j = cj->sort[sid];
  const int min_depth = lmax ? ci->depth : 0;
  const int max_depth = lmin ? ci->depth : 127;
  const float h_max = lmax ? ci->h_max_allowed : FLT_MAX;
  const double hi_max = fminf_ref(h_max, ci->h_max_active) * KG - rshift;
  const double hj_max = fminf_ref(h_max, cj->h_max_active) * KG;
  const int count_i = ci->count, count_j = cj->count;
  opart *parts_i = ci->parts, *parts_j = cj->parts;
  const double di_max = sort_i[count_i - 1].d - rshift;
  const double dj_min = sort_j[0].d;
  const float dx_max = 0.f + 0.f;

  if (ci->active) {
    for (int pid = count_i - 1;
         pid >= 0 && sort_i[pid].d + hi_max + dx_max > dj_min; pid--) {
      opart *pi = &parts_i[sort_i[pid].i];
      const int depth_i = pi->depth_h;
      const float hi = pi->h;
      if (!part_active(e, pi)) continue;
      if (depth_i < min_depth) continue;
      if (depth_i > max_depth) continue;
      const double di = sort_i[pid].d + hi * KG + dx_max - rshift;
      if (di < dj_min) continue;
      const float hig2 = hi * hi * KG2;
      const float pix = pi->x[0] - (cj->loc[0] + shift[0]);
      const float piy = pi->x[1] - (cj->loc[1] + shift[1]);
      const float piz = pi->x[2] - (cj->loc[2] + shift[2]);
      for (int pjd = 0; pjd < count_j && sort_j[pjd].d < di; pjd++) {
        opart *pj = &parts_j[sort_j[pjd].i];
        const float hj = pj->h;
        const float pjx = pj->x[0] - cj->loc[0];
        const float pjy = pj->x[1] - cj->loc[1];
        const float pjz = pj->x[2] - cj->loc[2];
        const float dx[3] = {pix - pjx, piy - pjy, piz - pjz};
        const float r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
        if (r2 < hig2) iact_nonsym_density(r2, dx, hi, hj, pi, pj);
      }
    }
  }
  if (cj->active) {
    for (int pjd = 0;
         pjd < count_j && sort_j[pjd].d - hj_max - dx_max < di_max; pjd++) {
      opart *pj = &parts_j[sort_j[pjd].i];
      const int depth_j = pj->depth_h;
      const float hj = pj->h;
      if (!part_active(e, pj)) continue;
      if (depth_j < min_depth) continue;
      if (depth_j > max_depth) continue;
      const double dj = sort_j[pjd].d - hj * KG - dx_max + rshift;
      if (dj - rshift > di_max) continue;
      const float hjg2 = hj * hj * KG2;
      const float pjx = pj->x[0] - cj->loc[0];
      const float pjy = pj->x[1] - cj->loc[1];
      const float pjz = pj->x[2] - cj->loc[2];
      for (int pid = count_i - 1; pid >= 0 && sort_i[pid].d > dj; pid--) {
        opart *pi = &parts_i[sort_i[pid].i];
        const float hi = pi->h;
        const float pix = pi->x[0] - (cj->loc[0] + shift[0]);
        const float piy = pi->x[1] - (cj->loc[1] + shift[1]);
        const float piz = pi->x[2] - (cj->loc[2] + shift[2]);
        const float dx[3] = {pjx - pix, pjy - piy, pjz - piz};
        const float r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
        if (r2 < hjg2) iact_nonsym_density(r2, dx, hj, hi, pj, pi);
      }
    }
  }
}

static void dopair1_branch(const octx *e, ocell *ci, ocell *cj, int lmin,
                           int lmax) {
  if (ci->count == 0 || cj->count == 0) return;
  if (!ci->active && !cj->active) return;
  double shift[3] = {0.0, 0.0, 0.0};
  const int sid = getsid_and_swap(e, &ci, &cj, shift);
  dopair1(e, ci, cj, lmin, lmax, sid, shift);
}

static void doself1(const octx *e, ocell *c, int lmin, int lmax) {
  opart *parts = c->parts;
  const int count = c->count;
  const int min_depth = lmax ? c->depth : 0;
  const int max_depth = lmin ? c->depth : 127;
  int *indt = ocalloc((size_t)count, sizeof(int));
  int countdt = 0, firstdt = 0;
  for (int k = 0; k < count; k++) {
    const opart *p = &parts[k];
    const int depth = p->depth_h;
    if (part_active(e, p) && depth >= min_depth && depth <= max_depth)
      indt[countdt++] = k;
  }
  for (int pid = 0; pid < count && firstdt < countdt; pid++) {
    opart *pi = &parts[pid];
    const int depth_i = pi->depth_h;
    const double pix[3] = {pi->x[0], pi->x[1], pi->x[2]};
    const float hi = pi->h;
    const float hig2 = hi * hi * KG2;
    const int update_i =
        part_active(e, pi) && depth_i >= min_depth && depth_i <= max_depth;
    if (!update_i) {
      for (int pjd = firstdt; pjd < countdt; pjd++) {
        opart *pj = &parts[indt[pjd]];
        const float hj = pj->h;
        const float hjg2 = hj * hj * KG2;
        const float dx[3] = {(float)(pj->x[0] - pix[0]),
                             (float)(pj->x[1] - pix[1]),
                             (float)(pj->x[2] - pix[2])};
        const float r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
        if (r2 < hjg2) iact_nonsym_density(r2, dx, hj, hi, pj, pi);
      }
    } else {
      firstdt += 1;
      for (int pjd = pid + 1; pjd < count; pjd++) {
        opart *pj = &parts[pjd];
        const int depth_j = pj->depth_h;
        const float hj = pj->h;
        const float hjg2 = hj * hj * KG2;
        float dx[3] = {(float)(pix[0] - pj->x[0]), (float)(pix[1] - pj->x[1]),
                       (float)(pix[2] - pj->x[2])};
        const float r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
        const int doi = (r2 < hig2);
        const int doj = part_active(e, pj) && depth_j >= min_depth &&
                        depth_j <= max_depth && (r2 < hjg2);
        if (doi && doj) {
          iact_density(r2, dx, hi, hj, pi, pj);
        } else if (doi) {
          iact_nonsym_density(r2, dx, hi, hj, pi, pj);
        } else if (doj) {
          dx[0] = -dx[0];
          dx[1] = -dx[1];
          dx[2] = -dx[2];
          iact_nonsym_density(r2, dx, hj, hi, pj, pi);
        }
      }
    }
  }
  free(indt);
}

static void doself1_branch(const octx *e, ocell *c, int lmin, int lmax) {
  if (c->count == 0 || !c->active) return;
  doself1(e, c, lmin, lmax);
}

static void dosub_pair1(const octx *e, ocell *ci, ocell *cj, int below) {
  if (!ci->active && !cj->active) return;
  if (ci->count == 0 || cj->count == 0) return;
  double shift[3];
  const int sid = getsid_and_swap(e, &ci, &cj, shift);
  if (!ci->split || ci->count < RECURSE_SIZE || !cj->split ||
      cj->count < RECURSE_SIZE) {
    dopair1_branch(e, ci, cj, 0, below);
  } else {
    if (!below && (!can_recurse_subpair(ci) || !can_recurse_subpair(cj)))
      below = 1;
    if (below) dopair1_branch(e, ci, cj, 1, 1);
    for (int k = 0; k < split_pairs_n[sid]; k++) {
      const int pid = split_pairs[sid][k][0], pjd = split_pairs[sid][k][1];
      if (ci->progeny[pid] && cj->progeny[pjd])
        dosub_pair1(e, ci->progeny[pid], cj->progeny[pjd], below);
    }
  }
}

static void dosub_self1(const octx *e, ocell *c, int below) {
  if (c->count == 0 || !c->active) return;
  if (!c->split || c->count < RECURSE_SIZE) {
    doself1_branch(e, c, 0, below);
  } else {
    if (!below && !can_recurse_subself(c)) below = 1;
    if (below) doself1_branch(e, c, 1, 1);
    for (int k = 0; k < 8; k++) {
      if (c->progeny[k]) {
        dosub_self1(e, c->progeny[k], below);
        for (int j = k + 1; j < 8; j++)
          if (c->progeny[j]) dosub_pair1(e, c->progeny[k], c->progeny[j], below);
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Subset density loops (the ghost's re-runs)                               */

static void dopair_subset(const octx *e, const ocell *ci, opart *parts_i,
                          const int *ind, int count, const ocell *cj, int sid,
                          int flipped, const double shift[3]) {
  (void)ci;
  const int count_j = cj->count;
  opart *parts_j = cj->parts;
  const sentry *sort_j = cj->sort[sid];
  const float dxj = 0.f;
  if (!flipped) {
    for (int pid = 0; pid < count; pid++) {
      opart *pi = &parts_i[ind[pid]];
      const double pix = pi->x[0] - (shift[0]);
      const double piy = pi->x[1] - (shift[1]);
      const double piz = pi->x[2] - (shift[2]);
      const float hi = pi->h;
      const float hig2 = hi * hi * KG2;
      const double di = hi * KG + dxj + pix * axis[sid][0] +
                        piy * axis[sid][1] + piz * axis[sid][2];
      for (int pjd = 0; pjd < count_j && sort_j[pjd].d < di; pjd++) {
        opart *pj = &parts_j[sort_j[pjd].i];
        const float hj = pj->h;
        float dx[3] = {(float)(pix - pj->x[0]), (float)(piy - pj->x[1]),
                       (float)(piz - pj->x[2])};
        const float r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
        if (r2 < hig2) iact_nonsym_density(r2, dx, hi, hj, pi, pj);
      }
    }
  } else {
    for (int pid = 0; pid < count; pid++) {
      opart *pi = &parts_i[ind[pid]];
      const double pix = pi->x[0] - (shift[0]);
      const double piy = pi->x[1] - (shift[1]);
      const double piz = pi->x[2] - (shift[2]);
      const float hi = pi->h;
      const float hig2 = hi * hi * KG2;
      const double di = -hi * KG - dxj + pix * axis[sid][0] +
                        piy * axis[sid][1] + piz * axis[sid][2];
      for (int pjd = count_j - 1; pjd >= 0 && di < sort_j[pjd].d; pjd--) {
        opart *pj = &parts_j[sort_j[pjd].i];
        const float hj = pj->h;
        float dx[3] = {(float)(pix - pj->x[0]), (float)(piy - pj->x[1]),
                       (float)(piz - pj->x[2])};
        const float r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
        if (r2 < hig2) iact_nonsym_density(r2, dx, hi, hj, pi, pj);
      }
    }
  }
}

static void dopair_subset_branch(const octx *e, const ocell *ci,
                                 opart *parts_i, const int *ind, int count,
                                 const ocell *cj) {
  if (cj->count == 0) return;
  double shift[3] = {0.0, 0.0, 0.0};
  for (int k = 0; k < 3; k++) {
    if (cj->loc[k] - ci->loc[k] < -e->dim[k] / 2)
      shift[k] = e->dim[k];
    else if (cj->loc[k] - ci->loc[k] > e->dim[k] / 2)
      shift[k] = -e->dim[k];
  }
  int idx = 0;
  for (int k = 0; k < 3; k++)
    idx = 3 * idx + ((cj->loc[k] - ci->loc[k] + shift[k] < 0)   ? 0
                     : (cj->loc[k] - ci->loc[k] + shift[k] > 0) ? 2
                                                                : 1);
  const int flipped = idx < 13;
  const int sid = idx < 13 ? idx : 26 - idx;
  dopair_subset(e, ci, parts_i, ind, count, cj, sid, flipped, shift);
}

static void doself_subset(const octx *e, const ocell *c, opart *parts,
                          const int *ind, int count) {
  (void)e;
  const int count_cell = c->count;
  opart *parts_j = c->parts;
  for (int pid = 0; pid < count; pid++) {
    opart *pi = &parts[ind[pid]];
    const float pix[3] = {(float)(pi->x[0] - c->loc[0]),
                          (float)(pi->x[1] - c->loc[1]),
                          (float)(pi->x[2] - c->loc[2])};
    const float hi = pi->h;
    const float hig2 = hi * hi * KG2;
    for (int pjd = 0; pjd < count_cell; pjd++) {
      opart *pj = &parts_j[pjd];
      if (pi == pj) continue;
      const float hj = pj->h;
      const float pjx[3] = {(float)(pj->x[0] - c->loc[0]),
                            (float)(pj->x[1] - c->loc[1]),
                            (float)(pj->x[2] - c->loc[2])};
      float dx[3] = {pix[0] - pjx[0], pix[1] - pjx[1], pix[2] - pjx[2]};
      const float r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
      if (r2 < hig2) iact_nonsym_density(r2, dx, hi, hj, pi, pj);
    }
  }
}

static ocell *find_sub(const ocell *c, const opart *parts, const int *ind) {
  for (int k = 0; k < 8; k++) {
    const ocell *p = c->progeny[k];
    if (p && &parts[ind[0]] >= &p->parts[0] && &parts[ind[0]] < &p->parts[p->count])
      return c->progeny[k];
  }
  fprintf(stderr, "sph_oracle: invalid sub\n");
  abort();
}

static void dosub_pair_subset(const octx *e, ocell *ci, opart *parts,
                              const int *ind, int count, ocell *cj) {
  if (ci->count == 0 || cj->count == 0) return;
  if (!ci->active) return;
  if (can_recurse_pair_old(ci) && can_recurse_pair_old(cj)) {
    ocell *const sub = find_sub(ci, parts, ind);
    double shift[3];
    const int sid = getsid_and_swap(e, &ci, &cj, shift);
    for (int k = 0; k < split_pairs_n[sid]; k++) {
      const int pid = split_pairs[sid][k][0], pjd = split_pairs[sid][k][1];
      if (ci->progeny[pid] == sub && cj->progeny[pjd] != NULL)
        dosub_pair_subset(e, ci->progeny[pid], parts, ind, count,
                          cj->progeny[pjd]);
      if (ci->progeny[pid] != NULL && cj->progeny[pjd] == sub)
        dosub_pair_subset(e, cj->progeny[pjd], parts, ind, count,
                          ci->progeny[pid]);
    }
  } else if (ci->active) {
    dopair_subset_branch(e, ci, parts, ind, count, cj);
  }
}

static void dosub_self_subset(const octx *e, ocell *ci, opart *parts,
                              const int *ind, int count) {
  if (ci->count == 0) return;
  if (!ci->active) return;
  if (ci->split && can_recurse_self_old(ci)) {
    ocell *const sub = find_sub(ci, parts, ind);
    dosub_self_subset(e, sub, parts, ind, count);
    for (int j = 0; j < 8; j++)
      if (ci->progeny[j] != sub && ci->progeny[j] != NULL)
        dosub_pair_subset(e, sub, parts, ind, count, ci->progeny[j]);
  } else {
    doself_subset(e, ci, parts, ind, count);
  }
}

/* ------------------------------------------------------------------------ */
/* Ghost                                                                    */

static void set_h_depth(opart *p, const ocell *leaf) {
  const float h = p->h;
  const ocell *c = leaf;
  if (h < c->h_min_allowed) {
    p->depth_h = (signed char)c->depth;
    return;
  }
  while (c != NULL) {
    if (h >= c->h_min_allowed && h < c->h_max_allowed) {
      p->depth_h = (signed char)c->depth;
      return;
    }
    c = c->parent;
  }
}

static int do_ghost(const octx *e, ocell *c) {
  opart *parts = c->parts;
  const float hydro_h_max = e->prm->h_max;
  const float hydro_h_min = e->prm->h_min;
  const float eps = e->prm->h_tolerance;
  const float eta = e->prm->eta;
  const float hydro_eta_dim = eta * eta * eta;
  const int max_iter = e->prm->max_iter;
  float h_max = c->h_max;
  float h_max_active = 0.f;
  int status = 0;
  if (c->count == 0) return 0;
  if (!c->active) return 0;
  if (c->split) {
    for (int k = 0; k < 8; k++) {
      if (c->progeny[k] != NULL) {
        status |= do_ghost(e, c->progeny[k]);
        h_max = fmaxf_ref(h_max, c->progeny[k]->h_max);
        h_max_active = fmaxf_ref(h_max_active, c->progeny[k]->h_max_active);
      }
    }
  } else {
    int *pid = ocalloc((size_t)c->count, sizeof(int));
    float *left = ocalloc((size_t)c->count, sizeof(float));
    float *right = ocalloc((size_t)c->count, sizeof(float));
    int count = 0;
    for (int k = 0; k < c->count; k++)
      if (part_active(e, &parts[k])) {
        pid[count] = k;
        left[count] = 0.f;
        right[count] = hydro_h_max;
        ++count;
      }
    for (int num_reruns = 0; count > 0 && num_reruns < max_iter;
         num_reruns++) {
      int redo = 0;
      for (int i = 0; i < count; i++) {
        opart *p = &parts[pid[i]];
        p->ghost_iters = num_reruns + 1;
        const float h_old = p->h;
        const float h_old_dim = h_old * h_old * h_old;
        const float h_old_dim_minus_one = h_old * h_old;
        float h_new;
        int has_no_neighbours = 0;
        if (p->wcount < 1.e-5 * KROOT) {
          has_no_neighbours = 1;
          h_new = 2.f * h_old;
        } else {
          end_density(p);
          const float n_sum = p->wcount * h_old_dim;
          const float n_target = hydro_eta_dim;
          const float f = n_sum - n_target;
          const float f_prime = p->wcount_dh * h_old_dim +
                                HDIM * p->wcount * h_old_dim_minus_one;
          if (n_sum < n_target)
            left[i] = fmaxf_ref(left[i], h_old);
          else if (n_sum > n_target)
            right[i] = fminf_ref(right[i], h_old);
          if (((p->h >= hydro_h_max) && (f < 0.f)) ||
              ((p->h <= hydro_h_min) && (f > 0.f))) {
            prepare_force(e, p);
            h_max = fmaxf_ref(h_max, p->h);
            h_max_active = fmaxf_ref(h_max_active, p->h);
            continue;
          }
          h_new = h_old - f / (f_prime + FLT_MIN);
          h_new = fminf_ref(h_new, 2.f * h_old);
          h_new = fmaxf_ref(h_new, 0.5f * h_old);
          h_new = fmaxf_ref(h_new, left[i]);
          h_new = fminf_ref(h_new, right[i]);
        }
        if (fabsf(h_new - h_old) > eps * h_old) {
          if ((h_new == left[i] && h_old == right[i]) ||
              (h_old == left[i] && h_new == right[i])) {
            const float l3 = left[i] * left[i] * left[i];
            const float r3 = right[i] * right[i] * right[i];
            p->h = cbrtf(0.5f * (l3 + r3));
          } else {
            p->h = h_new;
          }
          if (p->h < hydro_h_max && p->h > hydro_h_min) {
            pid[redo] = pid[i];
            left[redo] = left[i];
            right[redo] = right[i];
            redo += 1;
            init_part(p);
            continue;
          } else if (p->h <= hydro_h_min) {
            p->h = hydro_h_min;
          } else if (p->h >= hydro_h_max) {
            p->h = hydro_h_max;
            if (has_no_neighbours) no_neighbours(p);
          }
        }
        set_h_depth(p, c);
        h_max = fmaxf_ref(h_max, p->h);
        h_max_active = fmaxf_ref(h_max_active, p->h);
        prepare_force(e, p);
      }
      count = redo;
      if (count > 0) {
        for (ocell *finger = c; finger != NULL; finger = finger->parent) {
          for (olink *l = finger->density; l != NULL; l = l->next) {
            if (!l->t->is_pair)
              dosub_self_subset(e, finger, parts, pid, count);
            else if (l->t->ci == finger)
              dosub_pair_subset(e, finger, parts, pid, count, l->t->cj);
            else
              dosub_pair_subset(e, finger, parts, pid, count, l->t->ci);
          }
        }
      }
    }
    if (count) status = 1; /* failed to converge within max_iter */
    free(pid);
    free(left);
    free(right);
  }
  c->h_max = fmaxf_ref(c->h_max, h_max);
  c->h_max_active = fmaxf_ref(c->h_max_active, h_max_active);
  return status;
}

/* ------------------------------------------------------------------------ */
/* Force loops                                                              */

static void dopair2(const octx *e, ocell *ci, ocell *cj, int lmin, int lmax,
                    int sid, const double shift[3]) {
  double rshift = 0.0;
  for (int k = 0; k < 3; k++) rshift += shift[k] * axis[sid][k];
  const sentry *sort_i = ci->sort[sid];
  const sentry *sort_j = cj->sort[sid];
  const int min_depth = lmax ? ci->depth : 0;
  const int max_depth = lmin ? ci->depth : 127;
  const double hi_max = ci->h_max;
  const double hj_max = cj->h_max;
  const int count_i = ci->count, count_j = cj->count;
  opart *parts_i = ci->parts, *parts_j = cj->parts;
  const double dx_max = (0.f + 0.f);
  const double di_max = sort_i[count_i - 1].d;
  const double dj_min = sort_j[0].d;
  const double shift_i[3] = {cj->loc[0] + shift[0], cj->loc[1] + shift[1],
                             cj->loc[2] + shift[2]};
  const double shift_j[3] = {cj->loc[0], cj->loc[1], cj->loc[2]};
  int count_active_i = 0, count_active_j = 0;
  sentry *sort_active_i = NULL, *sort_active_j = NULL;
  if (ci->active) {
    sort_active_i = ocalloc((size_t)count_i, sizeof(sentry));
    for (int k = 0; k < count_i; k++) {
      const opart *p = &parts_i[sort_i[k].i];
      const int depth = p->depth_h;
      if (part_active(e, p) && depth >= min_depth && depth <= max_depth)
        sort_active_i[count_active_i++] = sort_i[k];
    }
  }
  if (cj->active) {
    sort_active_j = ocalloc((size_t)count_j, sizeof(sentry));
    for (int k = 0; k < count_j; k++) {
      const opart *p = &parts_j[sort_j[k].i];
      const int depth = p->depth_h;
      if (part_active(e, p) && depth >= min_depth && depth <= max_depth)
        sort_active_j[count_active_j++] = sort_j[k];
    }
  }
  for (int pid = count_i - 1;
       pid >= 0 && sort_i[pid].d + hi_max * KG + dx_max - rshift > dj_min;
       pid--) {
    opart *pi = &parts_i[sort_i[pid].i];
    const int depth_i = pi->depth_h;
    const float hi = pi->h;
    const double di = sort_i[pid].d + hi * KG + dx_max - rshift;
    if (di < dj_min) continue;
    const float hig2 = hi * hi * KG2;
    const float pix = pi->x[0] - shift_i[0];
    const float piy = pi->x[1] - shift_i[1];
    const float piz = pi->x[2] - shift_i[2];
    const int update_i =
        part_active(e, pi) && depth_i >= min_depth && depth_i <= max_depth;
    if (!update_i) {
      for (int pjd = 0; pjd < count_active_j && sort_active_j[pjd].d < di;
           pjd++) {
        opart *pj = &parts_j[sort_active_j[pjd].i];
        const float hj = pj->h;
        const float pjx = pj->x[0] - shift_j[0];
        const float pjy = pj->x[1] - shift_j[1];
        const float pjz = pj->x[2] - shift_j[2];
        const float dx[3] = {pjx - pix, pjy - piy, pjz - piz};
        const float r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
        if (r2 < hig2) iact_nonsym_force(r2, dx, hj, hi, pj, pi);
      }
    } else {
      for (int pjd = 0; pjd < count_j && sort_j[pjd].d < di; pjd++) {
        opart *pj = &parts_j[sort_j[pjd].i];
        const int depth_j = pj->depth_h;
        const float hj = pj->h;
        const float pjx = pj->x[0] - shift_j[0];
        const float pjy = pj->x[1] - shift_j[1];
        const float pjz = pj->x[2] - shift_j[2];
        const float dx[3] = {pix - pjx, piy - pjy, piz - pjz};
        const float r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
        if (r2 < hig2) {
          const int doj = part_active(e, pj) && depth_j >= min_depth &&
                          depth_j <= max_depth;
          if (doj)
            iact_force(r2, dx, hi, hj, pi, pj);
          else
            iact_nonsym_force(r2, dx, hi, hj, pi, pj);
        }
      }
    }
  }
  for (int pjd = 0;
       pjd < count_j && sort_j[pjd].d - hj_max * KG - dx_max < di_max - rshift;
       pjd++) {
    opart *pj = &parts_j[sort_j[pjd].i];
    const int depth_j = pj->depth_h;
    const float hj = pj->h;
    const double dj = sort_j[pjd].d - hj * KG - dx_max;
    if (dj > di_max - rshift) continue;
    const float hjg2 = hj * hj * KG2;
    const float pjx = pj->x[0] - shift_j[0];
    const float pjy = pj->x[1] - shift_j[1];
    const float pjz = pj->x[2] - shift_j[2];
    const int update_j =
        part_active(e, pj) && depth_j >= min_depth && depth_j <= max_depth;
    if (!update_j) {
      for (int pid = count_active_i - 1;
           pid >= 0 && sort_active_i[pid].d - rshift > dj; pid--) {
        opart *pi = &parts_i[sort_active_i[pid].i];
        const float hi = pi->h;
        const float hig2 = hi * hi * KG2;
        const float pix = pi->x[0] - shift_i[0];
        const float piy = pi->x[1] - shift_i[1];
        const float piz = pi->x[2] - shift_i[2];
        const float dx[3] = {pix - pjx, piy - pjy, piz - pjz};
        const float r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
        if (r2 < hjg2 && r2 >= hig2) iact_nonsym_force(r2, dx, hi, hj, pi, pj);
      }
    } else {
      for (int pid = count_i - 1; pid >= 0 && sort_i[pid].d - rshift > dj;
           pid--) {
        opart *pi = &parts_i[sort_i[pid].i];
        const int depth_i = pi->depth_h;
        const float hi = pi->h;
        const float hig2 = hi * hi * KG2;
        const float pix = pi->x[0] - shift_i[0];
        const float piy = pi->x[1] - shift_i[1];
        const float piz = pi->x[2] - shift_i[2];
        const float dx[3] = {pjx - pix, pjy - piy, pjz - piz};
        const float r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
        if (r2 < hjg2 && r2 >= hig2) {
          const int doi = part_active(e, pi) && depth_i >= min_depth &&
                          depth_i <= max_depth;
          if (doi)
            iact_force(r2, dx, hj, hi, pj, pi);
          else
            iact_nonsym_force(r2, dx, hj, hi, pj, pi);
        }
      }
    }
  }
  free(sort_active_i);
  free(sort_active_j);
}

static void dopair2_branch(const octx *e, ocell *ci, ocell *cj, int lmin,
                           int lmax) {
  if (ci->count == 0 || cj->count == 0) return;
  if (!ci->active && !cj->active) return;
  double shift[3] = {0.0, 0.0, 0.0};
  const int sid = getsid_and_swap(e, &ci, &cj, shift);
  dopair2(e, ci, cj, lmin, lmax, sid, shift);
}

static void doself2(const octx *e, ocell *c, int lmin, int lmax) {
  opart *parts = c->parts;
  const int count = c->count;
  const int min_depth = lmax ? c->depth : 0;
  const int max_depth = lmin ? c->depth : 127;
  int *indt = ocalloc((size_t)count, sizeof(int));
  int countdt = 0, firstdt = 0;
  for (int k = 0; k < count; k++) {
    const opart *p = &parts[k];
    const int depth = p->depth_h;
    if (part_active(e, p) && depth >= min_depth && depth <= max_depth)
      indt[countdt++] = k;
  }
  for (int pid = 0; pid < count && firstdt < countdt; pid++) {
    opart *pi = &parts[pid];
    const int depth_i = pi->depth_h;
    const double pix[3] = {pi->x[0], pi->x[1], pi->x[2]};
    const float hi = pi->h;
    const float hig2 = hi * hi * KG2;
    const int update_i =
        part_active(e, pi) && depth_i >= min_depth && depth_i <= max_depth;
    if (!update_i) {
      for (int pjd = firstdt; pjd < countdt; pjd++) {
        opart *pj = &parts[indt[pjd]];
        const float hj = pj->h;
        const float hjg2 = hj * hj * KG2;
        const float dx[3] = {(float)(pj->x[0] - pix[0]),
                             (float)(pj->x[1] - pix[1]),
                             (float)(pj->x[2] - pix[2])};
        const float r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
        if (r2 < hig2 || r2 < hjg2) iact_nonsym_force(r2, dx, hj, hi, pj, pi);
      }
    } else {
      firstdt += 1;
      for (int pjd = pid + 1; pjd < count; pjd++) {
        opart *pj = &parts[pjd];
        const int depth_j = pj->depth_h;
        const float hj = pj->h;
        const float hjg2 = hj * hj * KG2;
        float dx[3] = {(float)(pix[0] - pj->x[0]), (float)(pix[1] - pj->x[1]),
                       (float)(pix[2] - pj->x[2])};
        const float r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
        const int doi = (r2 < hig2) || (r2 < hjg2);
        const int doj = part_active(e, pj) && depth_j >= min_depth &&
                        depth_j <= max_depth && ((r2 < hjg2) || (r2 < hig2));
        if (doi && doj) {
          iact_force(r2, dx, hi, hj, pi, pj);
        } else if (doi) {
          iact_nonsym_force(r2, dx, hi, hj, pi, pj);
        } else if (doj) {
          dx[0] = -dx[0];
          dx[1] = -dx[1];
          dx[2] = -dx[2];
          iact_nonsym_force(r2, dx, hj, hi, pj, pi);
        }
      }
    }
  }
  free(indt);
}

static void doself2_branch(const octx *e, ocell *c, int lmin, int lmax) {
  if (c->count == 0 || !c->active) return;
  doself2(e, c, lmin, lmax);
}

static void dosub_pair2(const octx *e, ocell *ci, ocell *cj, int below) {
  if (!ci->active && !cj->active) return;
  if (ci->count == 0 || cj->count == 0) return;
  double shift[3];
  const int sid = getsid_and_swap(e, &ci, &cj, shift);
  if (!ci->split || ci->count < RECURSE_SIZE || !cj->split ||
      cj->count < RECURSE_SIZE) {
    dopair2_branch(e, ci, cj, 0, below);
  } else {
    if (!below && (!can_recurse_subpair2(ci) || !can_recurse_subpair2(cj)))
      below = 1;
    if (below) dopair2_branch(e, ci, cj, 1, 1);
    for (int k = 0; k < split_pairs_n[sid]; k++) {
      const int pid = split_pairs[sid][k][0], pjd = split_pairs[sid][k][1];
      if (ci->progeny[pid] && cj->progeny[pjd])
        dosub_pair2(e, ci->progeny[pid], cj->progeny[pjd], below);
    }
  }
}

static void dosub_self2(const octx *e, ocell *c, int below) {
  if (c->count == 0 || !c->active) return;
  if (!c->split || c->count < RECURSE_SIZE) {
    doself2_branch(e, c, 0, below);
  } else {
    if (!below && !can_recurse_subself2(c)) below = 1;
    if (below) doself2_branch(e, c, 1, 1);
    for (int k = 0; k < 8; k++) {
      if (c->progeny[k]) {
        dosub_self2(e, c->progeny[k], below);
        for (int j = k + 1; j < 8; j++)
          if (c->progeny[j]) dosub_pair2(e, c->progeny[k], c->progeny[j], below);
      }
    }
  }
}

/* runner_do_end_hydro_force -> hydro_end_force (hydro.h:878) */
static void end_force(const octx *e, ocell *c) {
  if (!c->active) return;
  if (c->split) {
    for (int k = 0; k < 8; k++)
      if (c->progeny[k]) end_force(e, c->progeny[k]);
  } else {
    for (int k = 0; k < c->count; k++) {
      opart *p = &c->parts[k];
      if (part_active(e, p)) p->h_dt *= p->h * HDIM_INV;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Space build                                                              */

static void sort_ascending(sentry *s, int N) {
  struct {
    int lo, hi;
  } stack[64];
  int qpos = 0;
  stack[0].lo = 0;
  stack[0].hi = N - 1;
  while (qpos >= 0) {
    const int lo = stack[qpos].lo, hi = stack[qpos].hi;
    qpos -= 1;
    if (hi - lo < 15) {
      /* selection sort of the short range */
      for (int i = lo; i < hi; i++) {
        int imin = i;
        for (int j = i + 1; j <= hi; j++)
          if (s[j].d < s[imin].d) imin = j;
        if (imin != i) {
          const sentry t = s[imin];
          s[imin] = s[i];
          s[i] = t;
        }
      }
    } else {
      const float pivot = s[(lo + hi) / 2].d;
      int i = lo, j = hi;
      while (i <= j) {
        while (s[i].d < pivot) i++;
        while (s[j].d > pivot) j--;
        if (i <= j) {
          if (i < j) {
            const sentry t = s[i];
            s[i] = s[j];
            s[j] = t;
          }
          i += 1;
          j -= 1;
        }
      }
      if (j > (lo + hi) / 2) {
        if (lo < j) {
          qpos++;
          stack[qpos].lo = lo;
          stack[qpos].hi = j;
        }
        if (i < hi) {
          qpos++;
          stack[qpos].lo = i;
          stack[qpos].hi = hi;
        }
      } else {
        if (i < hi) {
          qpos++;
          stack[qpos].lo = i;
          stack[qpos].hi = hi;
        }
        if (lo < j) {
          qpos++;
          stack[qpos].lo = lo;
          stack[qpos].hi = j;
        }
      }
    }
  }
}

static void do_sort(ocell *c) {
  const int count = c->count;
  for (int j = 0; j < 13; j++)
    c->sort[j] = ocalloc((size_t)count + 1, sizeof(sentry));
  if (c->split) {
    for (int k = 0; k < 8; k++)
      if (c->progeny[k] && c->progeny[k]->count > 0) do_sort(c->progeny[k]);
    for (int j = 0; j < 13; j++) {
      int off[8];
      off[0] = 0;
      for (int k = 1; k < 8; k++)
        off[k] = off[k - 1] + (c->progeny[k - 1] ? c->progeny[k - 1]->count : 0);
      const sentry *fingers[8];
      float buff[8];
      int inds[8];
      for (int k = 0; k < 8; k++) {
        inds[k] = k;
        if (c->progeny[k] && c->progeny[k]->count > 0) {
          fingers[k] = c->progeny[k]->sort[j];
          buff[k] = fingers[k]->d;
        } else {
          fingers[k] = NULL;
          buff[k] = FLT_MAX;
        }
      }
      for (int i = 0; i < 7; i++)
        for (int k = i + 1; k < 8; k++)
          if (buff[inds[k]] < buff[inds[i]]) {
            const int t = inds[i];
            inds[i] = inds[k];
            inds[k] = t;
          }
      sentry *out = c->sort[j];
      for (int ind = 0; ind < count; ind++) {
        out[ind].d = buff[inds[0]];
        out[ind].i = fingers[inds[0]]->i + off[inds[0]];
        fingers[inds[0]] += 1;
        buff[inds[0]] = fingers[inds[0]]->d;
        for (int k = 1; k < 8 && buff[inds[k]] < buff[inds[k - 1]]; k++) {
          const int t = inds[k - 1];
          inds[k - 1] = inds[k];
          inds[k] = t;
        }
      }
      out[count].d = FLT_MAX;
      out[count].i = 0;
    }
  } else {
    for (int k = 0; k < count; k++) {
      const double *px = c->parts[k].x;
      for (int j = 0; j < 13; j++) {
        c->sort[j][k].i = k;
        c->sort[j][k].d =
            px[0] * axis[j][0] + px[1] * axis[j][1] + px[2] * axis[j][2];
      }
    }
    for (int j = 0; j < 13; j++) {
      c->sort[j][count].d = FLT_MAX;
      c->sort[j][count].i = 0;
      sort_ascending(c->sort[j], count);
    }
  }
}

/* In-place bucket permutation by a per-particle bin (space_sort.c:42-93 and
 * the identical scheme of cell_split.c:120-150): the resulting order within
 * a bin is that of the cycle walk, which the reference's loops then see. */
static void bucket_permute(opart *parts, int *bin, int n, int nbins,
                           int *counts_out) {
  int *count = ocalloc((size_t)nbins, sizeof(int));
  int *off = ocalloc((size_t)nbins + 1, sizeof(int));
  for (int k = 0; k < n; k++) count[bin[k]]++;
  off[0] = 0;
  for (int k = 1; k <= nbins; k++) {
    off[k] = off[k - 1] + count[k - 1];
    count[k - 1] = 0;
  }
  for (int b = 0; b < nbins; b++) {
    for (int k = off[b] + count[b]; k < off[b + 1]; k++) {
      count[b]++;
      int target = bin[k];
      if (target == b) continue;
      opart tmp = parts[k];
      while (target != b) {
        int j = off[target] + count[target]++;
        while (bin[j] == target) j = off[target] + count[target]++;
        const opart sw = parts[j];
        parts[j] = tmp;
        tmp = sw;
        const int tb = bin[j];
        bin[j] = target;
        target = tb;
      }
      parts[k] = tmp;
      bin[k] = target;
    }
  }
  if (counts_out)
    for (int b = 0; b < nbins; b++) counts_out[b] = off[b + 1] - off[b];
  free(count);
  free(off);
}

/* The octant partition of cell_split.c:108-150. */
static void octant_permute(opart *parts, int n, const double pivot[3],
                           int counts[8]) {
  int *bin = ocalloc((size_t)n, sizeof(int));
  int bcount[8] = {0}, boff[9];
  for (int k = 0; k < n; k++) {
    bin[k] = (parts[k].x[0] >= pivot[0]) * 4 + (parts[k].x[1] >= pivot[1]) * 2 +
             (parts[k].x[2] >= pivot[2]);
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
        opart part = parts[k];
        int tbin = bin[k];
        while (bid != b) {
          int j = boff[bid] + bcount[bid]++;
          while (bin[j] == bid) {
            j++;
            bcount[bid]++;
          }
          const opart sw = parts[j];
          parts[j] = part;
          part = sw;
          const int sb = bin[j];
          bin[j] = tbin;
          tbin = sb;
          bid = tbin;
        }
        parts[k] = part;
        bin[k] = tbin;
      }
      bcount[bid]++;
    }
  }
  for (int b = 0; b < 8; b++) counts[b] = bcount[b];
  free(bin);
}

typedef struct {
  ocell *cells;
  int ncells, cap;
} cellpool;

static ocell *new_cell(cellpool *cp) {
  if (cp->ncells == cp->cap) {
    fprintf(stderr, "sph_oracle: cell pool exhausted\n");
    abort();
  }
  ocell *c = &cp->cells[cp->ncells++];
  memset(c, 0, sizeof(*c));
  return c;
}

/* space_split_recursive (space_split.c:53-560), hydro part only. */
static void split_recursive(const octx *e, cellpool *cp, ocell *c) {
  const int count = c->count;
  if (count > SPLIT_SIZE) {
    c->split = 1;
    const double pivot[3] = {c->loc[0] + c->width[0] / 2,
                             c->loc[1] + c->width[1] / 2,
                             c->loc[2] + c->width[2] / 2};
    int counts[8];
    octant_permute(c->parts, count, pivot, counts);
    int off = 0;
    float h_max = 0.f, h_max_active = 0.f;
    int any_active = 0;
    for (int k = 0; k < 8; k++) {
      if (counts[k] == 0) {
        c->progeny[k] = NULL;
        continue;
      }
      ocell *p = new_cell(cp);
      for (int d = 0; d < 3; d++) {
        p->loc[d] = c->loc[d];
        p->width[d] = c->width[d] / 2;
      }
      p->dmin = c->dmin / 2;
      p->h_min_allowed = p->dmin * 0.5 * (1. / KG);
      p->h_max_allowed = p->dmin * (1. / KG);
      if (k & 4) p->loc[0] += p->width[0];
      if (k & 2) p->loc[1] += p->width[1];
      if (k & 1) p->loc[2] += p->width[2];
      p->depth = c->depth + 1;
      p->parent = c;
      p->count = counts[k];
      p->parts = c->parts + off;
      off += counts[k];
      c->progeny[k] = p;
      split_recursive(e, cp, p);
      h_max = fmaxf_ref(h_max, p->h_max);
      h_max_active = fmaxf_ref(h_max_active, p->h_max_active);
      any_active |= p->active;
    }
    c->h_max = h_max;
    c->h_max_active = h_max_active;
    c->active = any_active;
  } else {
    c->split = 0;
    float h_max = 0.f, h_max_active = 0.f;
    int any_active = 0;
    for (int k = 0; k < count; k++) {
      opart *p = &c->parts[k];
      h_max = fmaxf_ref(h_max, p->h);
      if (part_active(e, p)) {
        h_max_active = fmaxf_ref(h_max_active, p->h);
        any_active = 1;
      }
      set_h_depth(p, c);
    }
    c->h_max = h_max;
    c->h_max_active = h_max_active;
    c->active = any_active;
  }
  c->h_max_old = c->h_max;
}

/* ------------------------------------------------------------------------ */
/* Driver                                                                   */

typedef struct {
  octx e;
  opart *parts;
  int n;
  cellpool pool;
  ocell *top;
  int cdim[3];
  double width[3];
  otask *tasks;
  int ntasks, tcap;
  olink *links;
  int nlinks;
} ospace;

static void link_add(ospace *s, ocell *c, otask *t) {
  olink *l = &s->links[s->nlinks++];
  l->t = t;
  l->next = c->density;
  c->density = l;
}

static int task_add(ospace *s, int is_pair, ocell *ci, ocell *cj) {
  if (s->ntasks == s->tcap) {
    s->tcap *= 2;
    s->tasks = realloc(s->tasks, sizeof(otask) * (size_t)s->tcap);
    if (!s->tasks) {
      fprintf(stderr, "sph_oracle: out of memory\n");
      abort();
    }
  }
  otask *t = &s->tasks[s->ntasks];
  t->is_pair = is_pair;
  t->ci = ci;
  t->cj = cj;
  return s->ntasks++;
}

/* cell_can_split_pair_hydro_task / cell_can_split_self_hydro_task
 * (cell.h:1152-1186): the cut-off with the space_stretch leeway (1.10f,
 * space.h:74) fits in half the progeny width.  Tasks are split right after a
 * rebuild, so h_max is the rebuild's. */
static inline int can_split_task(const ocell *c) {
  return c->split && (1.10f * KG * c->h_max < 0.5f * c->dmin);
}

/* sid_scale (sort_part.h:93-95): relative cost of a pair along each axis. */
static const float sid_scale[13] = {0.1897f, 0.4025f, 0.1897f, 0.4025f, 0.5788f,
                                    0.4025f, 0.1897f, 0.4025f, 0.1897f, 0.4025f,
                                    0.5788f, 0.4025f, 0.5788f};

/* The reference scheduler's hydro task split (scheduler_splittask_hydro,
 * scheduler_splittasks.c:45-265, with scheduler_dosub = 1 and
 * scheduler_doforcesplit = 0, scheduler.h:45-51), gas only.  Task ti is
 * recycled into its first piece and redone; every other piece is appended
 * and split at once, as scheduler_addtask + the recursive call do, so the
 * final order is the reference's.  An emptied task keeps ci = NULL.
 *   self on a cell that can split and holds >= subsize_self particles:
 *     the self tasks of the non-empty progeny, then a pair task for every
 *     two non-empty progeny (j < k);
 *   pair whose cells (after the sid swap) can both split, when the sid is
 *     a corner (sort_is_corner, sort_part.h:111) or
 *     count_i * sid_scale[sid] >= subsize_pair / count_j:
 *     the progeny pairs of the sid's split list, in list order. */
static void split_task(ospace *s, int ti) {
  const int sub_self = s->e.prm->subsize_self, sub_pair = s->e.prm->subsize_pair;
  for (;;) {
    otask t = s->tasks[ti];
    const int live = t.ci != NULL && t.ci->count > 0 &&
                     (!t.is_pair || (t.cj != NULL && t.cj->count > 0));
    if (!live) {
      s->tasks[ti].ci = s->tasks[ti].cj = NULL;
      return;
    }
    if (!t.is_pair) {
      ocell *ci = t.ci;
      if (!can_split_task(ci) || ci->count < sub_self) return;
      int first = 0;
      while (ci->progeny[first] == NULL) first++;
      s->tasks[ti].ci = ci->progeny[first];
      for (int k = first + 1; k < 8; k++)
        if (ci->progeny[k] != NULL && ci->progeny[k]->count)
          split_task(s, task_add(s, 0, ci->progeny[k], NULL));
      for (int j = 0; j < 8; j++)
        if (ci->progeny[j] != NULL && ci->progeny[j]->count)
          for (int k = j + 1; k < 8; k++)
            if (ci->progeny[k] != NULL && ci->progeny[k]->count)
              split_task(s, task_add(s, 1, ci->progeny[j], ci->progeny[k]));
    } else {
      ocell *ci = t.ci, *cj = t.cj;
      double shift[3];
      const int sid = getsid_and_swap(&s->e, &ci, &cj, shift);
      if (!(can_split_task(ci) && can_split_task(cj))) return;
      const int do_sub = (float)ci->count * sid_scale[sid] < (float)(sub_pair / cj->count);
      const int corner = sid == 0 || sid == 2 || sid == 6 || sid == 8;
      if (do_sub && !corner) return;
      s->tasks[ti].ci = ci->progeny[split_pairs[sid][0][0]];
      s->tasks[ti].cj = cj->progeny[split_pairs[sid][0][1]];
      for (int k = 1; k < split_pairs_n[sid]; k++)
        split_task(s, task_add(s, 1, ci->progeny[split_pairs[sid][k][0]],
                               cj->progeny[split_pairs[sid][k][1]]));
    }
  }
}

/* sort_all = 0 leaves every cell unsorted: the caller sorts the cells its
 * tasks need. */
static void build_space_sorted(ospace *s, const oracle_params *prm, int n,
                               const double *x, const float *v, const float *m,
                               const float *h, const float *u,
                               const signed char *time_bin, int sort_all) {
  memset(s, 0, sizeof(*s));
  s->e.prm = prm;
  for (int k = 0; k < 3; k++) s->e.dim[k] = prm->dim[k];
  s->e.periodic = prm->periodic;
  s->e.max_active_bin = prm->max_active_bin;
  s->n = n;
  s->parts = ocalloc((size_t)n, sizeof(opart));
  for (int k = 0; k < n; k++) {
    opart *p = &s->parts[k];
    p->id = k;
    for (int d = 0; d < 3; d++) {
      double xx = x[3 * k + d];
      if (prm->periodic) {
        while (xx < 0) xx += prm->dim[d];
        while (xx >= prm->dim[d]) xx -= prm->dim[d];
      }
      p->x[d] = xx;
      p->v[d] = v[3 * k + d];
    }
    p->mass = m[k];
    p->h = h[k];
    p->u = u[k];
    p->time_bin = time_bin[k];
  }
  /* Top-level grid (space.c:1263-1272, space_regrid.c:46-121). */
  const int maxtcells = prm->max_top_level_cells;
  const double dmax = fmax(fmax(prm->dim[0], prm->dim[1]), prm->dim[2]);
  const float tol = fmaxf_ref(1.0 - 1.0 / (maxtcells * maxtcells), 0.99);
  const double cell_min = tol * dmax / maxtcells;
  float h_max = cell_min / KG / STRETCH;
  for (int k = 0; k < n; k++)
    if (s->parts[k].h > h_max) h_max = s->parts[k].h;
  for (int d = 0; d < 3; d++) {
    s->cdim[d] = (int)floor(prm->dim[d] / fmax(h_max * KG * STRETCH, cell_min));
    s->width[d] = prm->dim[d] / s->cdim[d];
  }
  const double iw[3] = {1.0 / s->width[0], 1.0 / s->width[1],
                        1.0 / s->width[2]};
  const float dmin = fminf_ref(fminf_ref(s->width[0], s->width[1]), s->width[2]);
  const int ntop = s->cdim[0] * s->cdim[1] * s->cdim[2];
  /* Particle -> top cell (space_cell_index.c:64-150). */
  int *bin = ocalloc((size_t)n, sizeof(int));
  for (int k = 0; k < n; k++) {
    double pos[3];
    for (int d = 0; d < 3; d++) {
      double xx = s->parts[k].x[d];
      xx = xx < 0.0 ? xx + prm->dim[d] : (xx >= prm->dim[d] ? xx - prm->dim[d] : xx);
      if (xx == prm->dim[d]) xx = 0.0;
      pos[d] = xx;
      s->parts[k].x[d] = xx;
    }
    bin[k] = (int)(pos[2] * iw[2]) +
             s->cdim[2] * ((int)(pos[1] * iw[1]) + s->cdim[1] * (int)(pos[0] * iw[0]));
  }
  int *counts = ocalloc((size_t)ntop, sizeof(int));
  bucket_permute(s->parts, bin, n, ntop, counts);
  free(bin);
  /* Tree. */
  s->pool.cap = ntop + 2 * n + 64;
  s->pool.cells = ocalloc((size_t)s->pool.cap, sizeof(ocell));
  s->top = s->pool.cells;
  s->pool.ncells = ntop;
  int off = 0;
  for (int i = 0; i < s->cdim[0]; i++)
    for (int j = 0; j < s->cdim[1]; j++)
      for (int k = 0; k < s->cdim[2]; k++) {
        const int cid = k + s->cdim[2] * (j + s->cdim[1] * i);
        ocell *c = &s->top[cid];
        memset(c, 0, sizeof(*c));
        c->loc[0] = i * s->width[0];
        c->loc[1] = j * s->width[1];
        c->loc[2] = k * s->width[2];
        for (int d = 0; d < 3; d++) c->width[d] = s->width[d];
        c->dmin = dmin;
        c->h_min_allowed = c->dmin * 0.5 * (1. / KG);
        c->h_max_allowed = c->dmin * (1. / KG);
      }
  for (int cid = 0; cid < ntop; cid++) {
    ocell *c = &s->top[cid];
    c->count = counts[cid];
    c->parts = s->parts + off;
    off += counts[cid];
    if (c->count > 0) split_recursive(&s->e, &s->pool, c);
  }
  free(counts);
  for (int cid = 0; cid < ntop; cid++)
    if (s->top[cid].count > 0 && sort_all) do_sort(&s->top[cid]);
  /* Tasks, in the order oracle/ref_harness.c creates them: per non-empty
   * top cell its self task, then its pair tasks with the non-empty
   * neighbours of higher index (26-neighbourhood, periodic). */
  s->tcap = ntop * 14 + 16;
  s->tasks = ocalloc((size_t)s->tcap, sizeof(otask));
  const int *cdim = s->cdim;
  for (int i = 0; i < cdim[0]; i++)
    for (int j = 0; j < cdim[1]; j++)
      for (int k = 0; k < cdim[2]; k++) {
        const int cid = k + cdim[2] * (j + cdim[1] * i);
        ocell *ci = &s->top[cid];
        if (ci->count == 0) continue;
        task_add(s, 0, ci, NULL);
        for (int di = -1; di <= 1; di++)
          for (int dj = -1; dj <= 1; dj++)
            for (int dk = -1; dk <= 1; dk++) {
              int ii = i + di, jj = j + dj, kk = k + dk;
              if (prm->periodic) {
                ii = (ii + cdim[0]) % cdim[0];
                jj = (jj + cdim[1]) % cdim[1];
                kk = (kk + cdim[2]) % cdim[2];
              } else if (ii < 0 || ii >= cdim[0] || jj < 0 || jj >= cdim[1] ||
                         kk < 0 || kk >= cdim[2])
                continue;
              const int cjd = kk + cdim[2] * (jj + cdim[1] * ii);
              if (cjd <= cid) continue;
              ocell *cj = &s->top[cjd];
              if (cj->count == 0) continue;
              task_add(s, 1, ci, cj);
            }
      }
  if (prm->subsize_self > 0 || prm->subsize_pair > 0) {
    const int ntop_tasks = s->ntasks;
    for (int t = 0; t < ntop_tasks; t++) split_task(s, t);
    int kept = 0; /* drop the tasks the split left empty, keeping the order */
    for (int t = 0; t < s->ntasks; t++)
      if (s->tasks[t].ci != NULL) s->tasks[kept++] = s->tasks[t];
    s->ntasks = kept;
  }
  if (prm->reverse_tasks)
    for (int a = 0, z = s->ntasks - 1; a < z; a++, z--) {
      const otask t = s->tasks[a];
      s->tasks[a] = s->tasks[z];
      s->tasks[z] = t;
    }
  /* Density links on the cells each task holds (engine_maketasks.c:
   * 2311-2333), in task order. */
  s->links = ocalloc((size_t)2 * s->ntasks + 1, sizeof(olink));
  for (int t = 0; t < s->ntasks; t++) {
    otask *tk = &s->tasks[t];
    link_add(s, tk->ci, tk);
    if (tk->is_pair) link_add(s, tk->cj, tk);
  }
}

static void build_space(ospace *s, const oracle_params *prm, int n,
                        const double *x, const float *v, const float *m,
                        const float *h, const float *u,
                        const signed char *time_bin) {
  build_space_sorted(s, prm, n, x, v, m, h, u, time_bin, 1);
}

static void free_space(ospace *s) {
  for (int c = 0; c < s->pool.ncells; c++)
    for (int j = 0; j < 13; j++) free(s->pool.cells[c].sort[j]);
  free(s->pool.cells);
  free(s->parts);
  free(s->tasks);
  free(s->links);
}

/* The state change between the priming step and the measured step: the
 * reference's drift with a zero drift (cell_drift.c:330-371).  Active
 * particles restart from the caller's h, every particle takes the depth_h of
 * its h (cell.h:1787), every cell its h_max / h_max_active from its
 * particles, and h_max_old = h_max as the unskip sets it
 * (cell_unskip.c:875-880).  Inactive particles keep their state. */
static void redrift(const octx *e, ocell *c, const float *h_in) {
  float h_max = 0.f, h_max_active = 0.f;
  int any_active = 0;
  if (c->split) {
    for (int k = 0; k < 8; k++) {
      ocell *p = c->progeny[k];
      if (!p) continue;
      redrift(e, p, h_in);
      h_max = fmaxf_ref(h_max, p->h_max);
      h_max_active = fmaxf_ref(h_max_active, p->h_max_active);
      any_active |= p->active;
    }
  } else {
    for (int k = 0; k < c->count; k++) {
      opart *p = &c->parts[k];
      if (part_active(e, p)) p->h = h_in[p->id];
      set_h_depth(p, c);
      h_max = fmaxf_ref(h_max, p->h);
      if (part_active(e, p)) {
        h_max_active = fmaxf_ref(h_max_active, p->h);
        any_active = 1;
      }
    }
  }
  c->h_max = h_max;
  c->h_max_active = h_max_active;
  c->active = any_active;
  c->h_max_old = h_max;
}

int sph_oracle_run(const oracle_params *prm, int n, const double *x,
                   const float *v, const float *m, const float *h,
                   const float *u, const signed char *time_bin, int stages_in,
                   oracle_result *res) {
  ospace s;
  const int prime = (stages_in & ORACLE_STAGE_PRIME) != 0;
  oracle_params prm0 = *prm;
  prm0.max_active_bin = 127;
  build_space(&s, prime ? &prm0 : prm, n, x, v, m, h, u, time_bin);
  const int ntop = s.cdim[0] * s.cdim[1] * s.cdim[2];
  int status = 0;
  for (int k = 0; k < n; k++) init_part(&s.parts[k]);
  for (int pass = prime ? 0 : 1; pass <= 1; pass++) {
  int stages = stages_in & (ORACLE_STAGE_DENSITY | ORACLE_STAGE_GHOST |
                            ORACLE_STAGE_FORCE);
  if (pass == 0) {
    stages = ORACLE_STAGE_DENSITY | ORACLE_STAGE_GHOST | ORACLE_STAGE_FORCE;
  } else if (prime) {
    s.e.prm = prm;
    s.e.max_active_bin = prm->max_active_bin;
    for (int c = 0; c < ntop; c++)
      if (s.top[c].count > 0) redrift(&s.e, &s.top[c], h);
    for (int k = 0; k < n; k++)
      if (part_active(&s.e, &s.parts[k])) init_part(&s.parts[k]);
  }
  if (stages & ORACLE_STAGE_DENSITY) {
    for (int t = 0; t < s.ntasks; t++) {
      if (!s.tasks[t].is_pair)
        dosub_self1(&s.e, s.tasks[t].ci, 0);
      else
        dosub_pair1(&s.e, s.tasks[t].ci, s.tasks[t].cj, 0);
    }
    for (int k = 0; k < n; k++) {
      opart *p = &s.parts[k];
      float *o = &res->fields[ORACLE_NFIELDS * p->id];
      o[0] = p->rho;
      o[1] = p->rho_dh;
      o[2] = p->wcount;
      o[3] = p->wcount_dh;
      o[4] = p->div_v;
      o[5] = p->rot_v[0];
      o[6] = p->rot_v[1];
      o[7] = p->rot_v[2];
      p->ngb_d_first = p->ngb_d;
    }
  }
  if (stages & ORACLE_STAGE_GHOST) {
    for (int c = 0; c < ntop; c++) status |= do_ghost(&s.e, &s.top[c]);
    for (int k = 0; k < n; k++) {
      opart *p = &s.parts[k];
      float *o = &res->fields[ORACLE_NFIELDS * p->id];
      o[8] = p->h;
      o[9] = p->rho;
      o[10] = p->f;
      o[11] = p->pressure;
      o[12] = p->soundspeed;
      o[13] = p->balsara;
      o[14] = p->v_sig;
    }
  }
  if (stages & ORACLE_STAGE_FORCE) {
    for (int t = 0; t < s.ntasks; t++) {
      if (!s.tasks[t].is_pair)
        dosub_self2(&s.e, s.tasks[t].ci, 0);
      else
        dosub_pair2(&s.e, s.tasks[t].ci, s.tasks[t].cj, 0);
    }
    for (int c = 0; c < ntop; c++) end_force(&s.e, &s.top[c]);
    for (int k = 0; k < n; k++) {
      opart *p = &s.parts[k];
      float *o = &res->fields[ORACLE_NFIELDS * p->id];
      o[15] = p->a[0];
      o[16] = p->a[1];
      o[17] = p->a[2];
      o[18] = p->u_dt;
      o[19] = p->h_dt;
      o[20] = p->v_sig;
    }
  }
  }
  /* Per-particle tree placement and counters. */
  for (int c = 0; c < s.pool.ncells; c++) {
    const ocell *cc = &s.pool.cells[c];
    if (cc->split || cc->count == 0) continue;
    const ocell *top = cc;
    while (top->parent) top = top->parent;
    for (int k = 0; k < cc->count; k++) {
      const opart *p = &cc->parts[k];
      int32_t *ip = &res->ints[ORACLE_NINTS * p->id];
      ip[0] = (int32_t)(cc->parts - s.parts);
      ip[1] = cc->count;
      ip[2] = cc->depth;
      ip[3] = p->depth_h;
      ip[4] = (int32_t)(p - s.parts);
      ip[5] = (int32_t)(top - s.top);
      ip[6] = p->ngb_d_first;
      ip[7] = p->ngb_d;
      ip[8] = p->ngb_f;
      ip[9] = p->ghost_iters;
      ip[10] = p->min_ngb_bin;
    }
  }
  res->cdim[0] = s.cdim[0];
  res->cdim[1] = s.cdim[1];
  res->cdim[2] = s.cdim[2];
  res->ncells = s.pool.ncells;
  res->status = status;
  res->ntasks = s.ntasks;
  free_space(&s);
  return status;
}

/* The first density pass restricted to the tasks that touch the top cells
 * tops[0..ntops): those cells and their neighbours are sorted, the tasks
 * run in sph_oracle_run's order, and every particle of a listed top cell
 * gets its complete first-pass sums and neighbour count -- the same bits
 * as the whole pass, since it receives the same contributions from the
 * same tasks in the same order.  Other particles' values are partial.
 * Fields 0-7 and all ints are written.  For boxes whose whole pass would
 * take minutes. */
int sph_oracle_first_pass_tops(const oracle_params *prm, int n, const double *x,
                               const float *v, const float *m, const float *h,
                               const float *u, const signed char *time_bin,
                               int ntops, const int32_t *tops, oracle_result *res) {
  /* the tree without sorts; the listed cells and their neighbours are
   * sorted below */
  ospace s;
  build_space_sorted(&s, prm, n, x, v, m, h, u, time_bin, 0);
  const int *cdim = s.cdim;
  const int ntop = cdim[0] * cdim[1] * cdim[2];
  unsigned char *sel = (unsigned char *)ocalloc((size_t)ntop, 1);
  unsigned char *near = (unsigned char *)ocalloc((size_t)ntop, 1);
  for (int t = 0; t < ntops; t++) {
    const int cid = tops[t];
    if (cid < 0 || cid >= ntop) continue;
    sel[cid] = 1;
    const int i = cid / (cdim[1] * cdim[2]), j = (cid / cdim[2]) % cdim[1], k = cid % cdim[2];
    for (int di = -1; di <= 1; di++)
      for (int dj = -1; dj <= 1; dj++)
        for (int dk = -1; dk <= 1; dk++) {
          int ii = i + di, jj = j + dj, kk = k + dk;
          if (prm->periodic) {
            ii = (ii + cdim[0]) % cdim[0];
            jj = (jj + cdim[1]) % cdim[1];
            kk = (kk + cdim[2]) % cdim[2];
          } else if (ii < 0 || ii >= cdim[0] || jj < 0 || jj >= cdim[1] || kk < 0 ||
                     kk >= cdim[2])
            continue;
          near[kk + cdim[2] * (jj + cdim[1] * ii)] = 1;
        }
  }
  for (int cid = 0; cid < ntop; cid++)
    if (near[cid] && s.top[cid].count > 0) do_sort(&s.top[cid]);
  for (int k = 0; k < n; k++) init_part(&s.parts[k]);
  for (int t = 0; t < s.ntasks; t++) {
    const otask *tk = &s.tasks[t];
    const int ci = (int)(tk->ci - s.top);
    const int cj = tk->is_pair ? (int)(tk->cj - s.top) : ci;
    if (!sel[ci] && !sel[cj]) continue;
    if (!tk->is_pair)
      dosub_self1(&s.e, tk->ci, 0);
    else
      dosub_pair1(&s.e, tk->ci, tk->cj, 0);
  }
  for (int k = 0; k < n; k++) {
    const opart *p = &s.parts[k];
    float *o = &res->fields[ORACLE_NFIELDS * p->id];
    o[0] = p->rho;
    o[1] = p->rho_dh;
    o[2] = p->wcount;
    o[3] = p->wcount_dh;
    o[4] = p->div_v;
    o[5] = p->rot_v[0];
    o[6] = p->rot_v[1];
    o[7] = p->rot_v[2];
  }
  for (int c = 0; c < s.pool.ncells; c++) {
    const ocell *cc = &s.pool.cells[c];
    if (cc->split || cc->count == 0) continue;
    const ocell *top = cc;
    while (top->parent) top = top->parent;
    for (int k = 0; k < cc->count; k++) {
      const opart *p = &cc->parts[k];
      int32_t *ip = &res->ints[ORACLE_NINTS * p->id];
      ip[0] = (int32_t)(cc->parts - s.parts);
      ip[1] = cc->count;
      ip[2] = cc->depth;
      ip[3] = p->depth_h;
      ip[4] = (int32_t)(p - s.parts);
      ip[5] = (int32_t)(top - s.top);
      ip[6] = p->ngb_d;
      ip[7] = p->ngb_d;
      ip[8] = 0;
      ip[9] = 0;
      ip[10] = 0;
    }
  }
  res->cdim[0] = cdim[0];
  res->cdim[1] = cdim[1];
  res->cdim[2] = cdim[2];
  res->ncells = s.pool.ncells;
  res->status = 0;
  res->ntasks = s.ntasks;
  free(sel);
  free(near);
  free_space(&s);
  return 0;
}

/* The force loops alone on a given state: every particle takes h, rho,
 * grad-h f, P, c and Balsara from state[6 n] (input order); the active
 * ones (time_bin <= max_active_bin) restart their accelerations the way the
 * ghost leaves them (hydro_reset_acceleration, hydro.h:749;
 * timestep_limiter_prepare_force) and run the force loops and end_force.
 * This is the force task of a step in which inactive particles keep the
 * predicted state of their last step.  Fields 15-20 and ints 8, 10 are
 * written. */
int sph_oracle_run_state(const oracle_params *prm, int n, const double *x,
                         const float *v, const float *m, const float *u,
                         const signed char *time_bin, const float *state,
                         oracle_result *res) {
  float *h = (float *)ocalloc((size_t)n, sizeof(float));
  for (int k = 0; k < n; k++) h[k] = state[6 * (size_t)k];
  ospace s;
  build_space(&s, prm, n, x, v, m, h, u, time_bin);
  const int ntop = s.cdim[0] * s.cdim[1] * s.cdim[2];
  for (int k = 0; k < n; k++) {
    opart *p = &s.parts[k];
    const float *st = &state[6 * (size_t)p->id];
    p->rho = st[1];
    p->f = st[2];
    p->pressure = st[3];
    p->soundspeed = st[4];
    p->balsara = st[5];
    if (part_active(&s.e, p)) {
      p->a[0] = p->a[1] = p->a[2] = 0.f;
      p->u_dt = 0.f;
      p->h_dt = 0.f;
      p->v_sig = 2.f * p->soundspeed;
      p->min_ngb_bin = NUM_TIME_BINS + 1;
    }
    p->ngb_f = 0;
  }
  for (int t = 0; t < s.ntasks; t++) {
    if (!s.tasks[t].is_pair)
      dosub_self2(&s.e, s.tasks[t].ci, 0);
    else
      dosub_pair2(&s.e, s.tasks[t].ci, s.tasks[t].cj, 0);
  }
  for (int c = 0; c < ntop; c++) end_force(&s.e, &s.top[c]);
  for (int k = 0; k < n; k++) {
    const opart *p = &s.parts[k];
    float *o = &res->fields[ORACLE_NFIELDS * p->id];
    o[15] = p->a[0];
    o[16] = p->a[1];
    o[17] = p->a[2];
    o[18] = p->u_dt;
    o[19] = p->h_dt;
    o[20] = p->v_sig;
    int32_t *ip = &res->ints[ORACLE_NINTS * p->id];
    ip[8] = p->ngb_f;
    ip[10] = p->min_ngb_bin;
  }
  res->cdim[0] = s.cdim[0];
  res->cdim[1] = s.cdim[1];
  res->cdim[2] = s.cdim[2];
  res->ncells = s.pool.ncells;
  res->status = 0;
  res->ntasks = s.ntasks;
  free_space(&s);
  free(h);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Sort arrays of the whole tree (runner_sort.c:203-463), depth first over
 * the non-empty cells: records [first, count, depth] and 13 arrays of
 * count + 1 entries per cell.  With rec == NULL only the sizes are
 * returned. */

static void walk_sorts(const ospace *s, const ocell *c, int32_t *ncells,
                       int64_t *nent, int32_t *rec, float *d, int32_t *idx) {
  if (c->count == 0) return;
  if (rec) {
    int32_t *r = rec + 3 * (size_t)*ncells;
    r[0] = (int32_t)(c->parts - s->parts);
    r[1] = c->count;
    r[2] = c->depth;
    for (int j = 0; j < 13; j++)
      for (int k = 0; k <= c->count; k++) {
        d[*nent + (int64_t)j * (c->count + 1) + k] = c->sort[j][k].d;
        idx[*nent + (int64_t)j * (c->count + 1) + k] = c->sort[j][k].i;
      }
  }
  *ncells += 1;
  *nent += 13 * (int64_t)(c->count + 1);
  if (c->split)
    for (int k = 0; k < 8; k++)
      if (c->progeny[k]) walk_sorts(s, c->progeny[k], ncells, nent, rec, d, idx);
}

int sph_oracle_tree_sorts(const oracle_params *prm, int n, const double *x,
                          const float *v, const float *m, const float *h,
                          const float *u, const signed char *time_bin,
                          int32_t *ncells, int64_t *nentries, int32_t *rec,
                          float *d, int32_t *idx) {
  ospace s;
  build_space(&s, prm, n, x, v, m, h, u, time_bin);
  const int ntop = s.cdim[0] * s.cdim[1] * s.cdim[2];
  *ncells = 0;
  *nentries = 0;
  for (int c = 0; c < ntop; c++) walk_sorts(&s, &s.top[c], ncells, nentries, rec, d, idx);
  free_space(&s);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* FP64 brute-force density/force over a cell list, for error statements.
 * Computes, for every particle with the given h, the double-precision
 * density sums and the force sums over all j != i with r < gamma*h (density)
 * or r < gamma*max(hi,hj) (force), using the minimum-image convention.
 * Inputs are the post-ghost fields (h, rho, f, P, c, balsara).            */

static inline void kernel_deval_d(double u, double *W, double *dW) {
  const double kg = (double)KG;
  const double x = u / kg;
  if (x >= 1.0) {
    *W = 0.0;
    *dW = 0.0;
    return;
  }
  const double om = 1.0 - x;
  const double C = 21.0 / (2.0 * M_PI);
  *W = C / (kg * kg * kg) * om * om * om * om * (1.0 + 4.0 * x);
  *dW = C / (kg * kg * kg * kg) * (-20.0) * x * om * om * om;
}

static void exact64_impl(const oracle_params *prm, int n, const double *x,
                         const float *v, const float *m, const float *h,
                         const float *rho, const float *f, const float *P,
                         const float *cs, const float *bal, const unsigned char *which,
                         double *out) {
  /* out per particle: rho, wcount, div_v, a[3], u_dt (7 doubles) */
  double hmax = 0;
  for (int k = 0; k < n; k++) hmax = fmax(hmax, h[k]);
  const double H = hmax * (double)KG;
  int cd[3];
  for (int d = 0; d < 3; d++) {
    cd[d] = (int)floor(prm->dim[d] / H);
    if (cd[d] < 1) cd[d] = 1;
    if (cd[d] > 256) cd[d] = 256;
  }
  const int nc = cd[0] * cd[1] * cd[2];
  int *head = ocalloc((size_t)nc, sizeof(int));
  int *next = ocalloc((size_t)n, sizeof(int));
  for (int c = 0; c < nc; c++) head[c] = -1;
  for (int k = 0; k < n; k++) {
    int ix[3];
    for (int d = 0; d < 3; d++) {
      ix[d] = (int)(x[3 * k + d] / prm->dim[d] * cd[d]);
      if (ix[d] >= cd[d]) ix[d] = cd[d] - 1;
      if (ix[d] < 0) ix[d] = 0;
    }
    const int c = (ix[0] * cd[1] + ix[1]) * cd[2] + ix[2];
    next[k] = head[c];
    head[c] = k;
  }
  const int reach[3] = {cd[0] < 3 ? 0 : 1, cd[1] < 3 ? 0 : 1, cd[2] < 3 ? 0 : 1};
  for (int i = 0; i < n; i++) {
    if (which && !which[i]) continue;
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};
    const double hi = h[i], hi_inv = 1.0 / hi;
    int ix[3];
    for (int d = 0; d < 3; d++) {
      ix[d] = (int)(x[3 * i + d] / prm->dim[d] * cd[d]);
      if (ix[d] >= cd[d]) ix[d] = cd[d] - 1;
    }
    const double fi = f ? f[i] : 0.0;
    for (int a = -reach[0]; a <= (cd[0] < 3 ? cd[0] - 1 : 1); a++)
      for (int b = -reach[1]; b <= (cd[1] < 3 ? cd[1] - 1 : 1); b++)
        for (int c3 = -reach[2]; c3 <= (cd[2] < 3 ? cd[2] - 1 : 1); c3++) {
          const int jx = (reach[0] ? (ix[0] + a + cd[0]) % cd[0] : a);
          const int jy = (reach[1] ? (ix[1] + b + cd[1]) % cd[1] : b);
          const int jz = (reach[2] ? (ix[2] + c3 + cd[2]) % cd[2] : c3);
          for (int j = head[(jx * cd[1] + jy) * cd[2] + jz]; j >= 0; j = next[j]) {
            if (j == i) continue;
            double dx[3];
            for (int d = 0; d < 3; d++) {
              double t = x[3 * i + d] - x[3 * j + d];
              if (prm->periodic) {
                if (t > 0.5 * prm->dim[d]) t -= prm->dim[d];
                if (t < -0.5 * prm->dim[d]) t += prm->dim[d];
              }
              dx[d] = t;
            }
            const double r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
            const double r = sqrt(r2);
            const double hj = h[j];
            const double Hi = hi * (double)KG, Hj = hj * (double)KG;
            double dv[3] = {(double)v[3 * i] - v[3 * j],
                            (double)v[3 * i + 1] - v[3 * j + 1],
                            (double)v[3 * i + 2] - v[3 * j + 2]};
            const double dvdr = dv[0] * dx[0] + dv[1] * dx[1] + dv[2] * dx[2];
            if (r < Hi) {
              double W, dW;
              kernel_deval_d(r * hi_inv, &W, &dW);
              acc[0] += m[j] * W * hi_inv * hi_inv * hi_inv;
              acc[1] += W * hi_inv * hi_inv * hi_inv;
              if (r > 0)
                acc[2] -= m[j] * dW * hi_inv * hi_inv * hi_inv * hi_inv * dvdr / r;
            }
            if (f && (r < Hi || r < Hj) && r > 0) {
              double Wi, dWi, Wj, dWj;
              kernel_deval_d(r * hi_inv, &Wi, &dWi);
              kernel_deval_d(r / hj, &Wj, &dWj);
              const double wi_dr = dWi * pow(hi_inv, 4);
              const double wj_dr = dWj * pow(1.0 / hj, 4);
              const double fj = f[j];
              const double f_ij = 1.0 - fi / m[j];
              const double f_ji = 1.0 - fj / m[i];
              const double Pi = (double)P[i] / ((double)rho[i] * rho[i]) * f_ij;
              const double Pj = (double)P[j] / ((double)rho[j] * rho[j]) * f_ji;
              const double mu = fmin(dvdr, 0.0) / r;
              const double vsig = (double)cs[i] + cs[j] - 3.0 * mu;
              const double visc = -0.25 * vsig * ((double)bal[i] + bal[j]) * mu /
                                   (0.5 * ((double)rho[i] + rho[j]));
              const double visc_acc = 0.5 * visc * (wi_dr * f_ij + wj_dr * f_ji) / r;
              const double sph_acc = (Pi * wi_dr + Pj * wj_dr) / r;
              const double a = sph_acc + visc_acc;
              for (int d = 0; d < 3; d++) acc[3 + d] -= m[j] * a * dx[d];
              acc[6] += m[j] * (Pi * dvdr / r * wi_dr + 0.5 * visc_acc * dvdr);
            }
          }
        }
    /* self contribution */
    acc[0] += m[i] * (double)KROOT * hi_inv * hi_inv * hi_inv;
    acc[1] += (double)KROOT * hi_inv * hi_inv * hi_inv;
    if (rho) acc[2] /= rho[i];
    for (int q = 0; q < 7; q++) out[7 * (size_t)i + q] = acc[q];
  }
  free(head);
  free(next);
}

void sph_oracle_exact64(const oracle_params *prm, int n, const double *x,
                        const float *v, const float *m, const float *h,
                        const float *rho, const float *f, const float *P,
                        const float *cs, const float *bal, double *out) {
  exact64_impl(prm, n, x, v, m, h, rho, f, P, cs, bal, NULL, out);
}

/* The same sums for the particles with which[i] != 0 only (the others'
 * rows of out are left as they are). */
void sph_oracle_exact64_some(const oracle_params *prm, int n, const double *x,
                             const float *v, const float *m, const float *h,
                             const float *rho, const float *f, const float *P,
                             const float *cs, const float *bal,
                             const unsigned char *which, double *out) {
  exact64_impl(prm, n, x, v, m, h, rho, f, P, cs, bal, which, out);
}
