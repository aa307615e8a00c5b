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
 * 8 force neighbours, 9 ghost iterations. */
#define ORACLE_NINTS 10

typedef struct {
  double dim[3];
  int32_t periodic;
  float eta, h_tolerance, h_max, h_min, alpha;
  int32_t max_iter, max_active_bin, max_top_level_cells;
} oracle_params;

typedef struct {
  float *fields;  /* n * ORACLE_NFIELDS */
  int32_t *ints;  /* n * ORACLE_NINTS */
  int32_t cdim[3];
  int32_t ncells;
  int32_t status; /* 0 ok, 1 ghost did not converge */
} oracle_result;

int sph_oracle_run(const oracle_params *prm, int n, const double *x,
                   const float *v, const float *m, const float *h,
                   const float *u, const signed char *time_bin, int stages,
                   oracle_result *res);

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
#endif
