/* sph_oracle.h -- interface of the oracle's C restatement (test
 * infrastructure; see sph_oracle.c).  Plain C, called through ctypes. */
#ifndef SPH_ORACLE_H
#define SPH_ORACLE_H
#include <stdint.h>

#define ORACLE_STAGE_DENSITY 1
#define ORACLE_STAGE_GHOST 2
#define ORACLE_STAGE_FORCE 4
/* One full step with every particle active runs first; the requested stages
 * then run at max_active_bin on the state it leaves: active particles
 * restart from the input h, inactive ones keep their state. */
#define ORACLE_STAGE_PRIME 8

/* Per-particle float results, in input order (same columns as the
 * reference driver's output block): 0-7 first density pass (rho, rho_dh,
 * wcount, wcount_dh, div_v, rot_v[3]); 8-14 after the ghost (h, rho, f,
 * pressure, soundspeed, balsara, v_sig); 15-20 after the force (a[3], u_dt,
 * h_dt, v_sig). */
#define ORACLE_NFIELDS 24
/* Per-particle integers: 0 leaf first index, 1 leaf count, 2 leaf depth,
 * 3 depth_h, 4 position in the cell-sorted order, 5 top cell id,
 * 6 density neighbours (first pass), 7 density neighbours (last pass),
 * 8 force neighbours, 9 ghost iterations, 10 smallest time bin among the
 * force neighbours (limiter_data.min_ngb_time_bin; num_time_bins + 1 when
 * there is none). */
#define ORACLE_NINTS 11

typedef struct {
  double dim[3];
  int32_t periodic;
  float eta, h_tolerance, h_max, h_min, alpha;
  int32_t max_iter, max_active_bin, max_top_level_cells;
  /* Task splitting (Scheduler:cell_sub_size_self_hydro / _pair_hydro):
   * both 0 keeps one task per top cell and top-cell pair; otherwise the
   * tasks are split as the reference's scheduler splits them. */
  int32_t subsize_self, subsize_pair;
  /* 0: the tasks in the reference driver's creation order; 1: the same
   * tasks in reverse order (another order the reference's scheduler may
   * run them in: density and force tasks are independent of each other). */
  int32_t reverse_tasks;
} oracle_params;

typedef struct {
  float *fields;  /* n * ORACLE_NFIELDS */
  int32_t *ints;  /* n * ORACLE_NINTS */
  int32_t cdim[3];
  int32_t ncells;
  int32_t status; /* 0 ok, 1 ghost did not converge */
  int32_t ntasks; /* density tasks after splitting */
} oracle_result;

int sph_oracle_run(const oracle_params *prm, int n, const double *x,
                   const float *v, const float *m, const float *h,
                   const float *u, const signed char *time_bin, int stages,
                   oracle_result *res);

/* The force loops alone on a given state (h, rho, f, P, c, Balsara per
 * particle, state[6 n]); see sph_oracle.c. */
int sph_oracle_run_state(const oracle_params *prm, int n, const double *x,
                         const float *v, const float *m, const float *u,
                         const signed char *time_bin, const float *state,
                         oracle_result *res);

/* The first density pass of the tasks touching the top cells tops[0..ntops)
 * only: complete (bit-identical to sph_oracle_run) for the particles of
 * those cells, partial elsewhere; fields 0-7 and the ints are written. */
int sph_oracle_first_pass_tops(const oracle_params *prm, int n, const double *x,
                               const float *v, const float *m, const float *h,
                               const float *u, const signed char *time_bin,
                               int ntops, const int32_t *tops, oracle_result *res);

/* Sort arrays of every non-empty cell, depth first: rec [ncells][3] =
 * first (cell-sorted order), count, depth; d / idx: per cell 13 arrays of
 * count + 1 entries (keys ascending, FLT_MAX sentinel).  Call with
 * rec == NULL for the sizes. */
int sph_oracle_tree_sorts(const oracle_params *prm, int n, const double *x,
                          const float *v, const float *m, const float *h,
                          const float *u, const signed char *time_bin,
                          int32_t *ncells, int64_t *nentries, int32_t *rec,
                          float *d, int32_t *idx);

void sph_oracle_exact64(const oracle_params *prm, int n, const double *x,
                        const float *v, const float *m, const float *h,
                        const float *rho, const float *f, const float *P,
                        const float *cs, const float *bal, double *out);
void sph_oracle_exact64_some(const oracle_params *prm, int n, const double *x,
                             const float *v, const float *m, const float *h,
                             const float *rho, const float *f, const float *P,
                             const float *cs, const float *bal,
                             const unsigned char *which, double *out);
/* Time integration (sph_integrate.c).  State arrays are SoA in the
 * caller's order: x[3 n] (double), v_full, v (predicted), a (a_hydro) [3 n];
 * u_full, u (predicted), u_dt, h, h_dt, rho, P, c, v_sig [n]; time_bin [n]. */
typedef struct {
  double time_base;     /* physical time of one integer tick */
  double dt_min, dt_max;
  float CFL;            /* hydro_props->CFL_condition */
  float log_max_h_change;
  float h_min, h_max;
  float minimal_u;      /* hydro_props->minimal_internal_energy */
} integ_params;

typedef struct {
  double *x;
  float *v_full, *v, *a;
  float *u_full, *u, *u_dt, *h, *h_dt, *rho, *P, *c, *v_sig;
  signed char *time_bin;
} integ_state;

void sph_integ_kick(const integ_params *ip, integ_state *st, int64_t n, int which,
                    int64_t ti_current, int max_active_bin);
void sph_integ_drift(const integ_params *ip, integ_state *st, int64_t n, int64_t ti_old,
                     int64_t ti_current);
int64_t sph_integ_timestep(const integ_params *ip, integ_state *st, int64_t n,
                           const signed char *min_ngb_bin, int64_t ti_current,
                           int max_active_bin);
int64_t sph_integ_ti_end_min(const integ_state *st, int64_t n, int64_t ti_current);
int sph_integ_max_active_bin(int64_t ti);
int64_t sph_integ_time_end(int64_t ti, int bin);
#endif
