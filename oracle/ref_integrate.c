/* Reference driver for the time integration of gas particles.
 *
 * Test infrastructure only: linked against the reference sources compiled by
 * oracle/build_ref.sh, it applies the reference's own per-particle
 * integration functions to an input state, so that the oracle's C
 * restatement (oracle/sph_integrate.c) can be pinned against them bit for
 * bit.  The per-particle loops follow the reference's runner functions:
 *   kick1:    runner_do_kick1 (runner_time_integration.c:141-184) -> kick_part
 *   kick2:    runner_do_kick2 (:421-457) -> kick_part,
 *             hydro_reset_predicted_values (hydro/Minimal/hydro.h:771)
 *   drift:    cell_drift_part (cell_drift.c:253-332) -> drift_part (drift.h:138)
 *             and the h clamp
 *   timestep: runner_do_timestep (:699-749) -> get_part_timestep (timestep.h:142)
 *
 * Input (argv[1]):  "SPHINT01", int64 n, op (1 kick1, 2 kick2, 3 drift,
 *   4 timestep), int64 ti_old, ti_current, int32 max_active_bin, double
 *   time_base, dt_min, dt_max, float CFL, log_max_h_change, h_min, h_max,
 *   minimal_u, then the state arrays (x 3n f64; v_full, v, a 3n f32; u_full,
 *   u, u_dt, h, h_dt, rho, P, c, v_sig n f32; time_bin, min_ngb_bin n i8).
 * Output (argv[2]): "SPHINT02" + the same arrays after the operation.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* config.h and swift.h come in through -include on the command line. */
#include "drift.h"
#include "kick.h"
#include "timestep.h"

struct integ_header {
  char magic[8];
  int64_t n, op, ti_old, ti_current;
  int32_t max_active_bin, pad;
  double time_base, dt_min, dt_max;
  float CFL, log_max_h_change, h_min, h_max, minimal_u, pad2;
};

static void *xmalloc(size_t n) {
  void *p = calloc(1, n ? n : 1);
  if (!p) {
    fprintf(stderr, "ref_integrate: out of memory\n");
    exit(3);
  }
  return p;
}

static void xio(void *p, size_t sz, size_t n, FILE *f, int wr) {
  const size_t got = wr ? fwrite(p, sz, n, f) : fread(p, sz, n, f);
  if (got != n) {
    fprintf(stderr, "ref_integrate: short %s\n", wr ? "write" : "read");
    exit(2);
  }
}

/* The state arrays in file order; wr = 0 reads them into the parts. */
static void io_state(FILE *f, struct part *P, struct xpart *X, size_t n, int wr) {
  double *d = xmalloc(3 * n * sizeof(double));
  float *a = xmalloc(3 * n * sizeof(float));
  float *s = xmalloc(n * sizeof(float));
  int8_t *b = xmalloc(n);
  /* x */
  if (wr) for (size_t k = 0; k < n; k++) for (int j = 0; j < 3; j++) d[3 * k + j] = P[k].x[j];
  xio(d, sizeof(double), 3 * n, f, wr);
  if (!wr) for (size_t k = 0; k < n; k++) for (int j = 0; j < 3; j++) P[k].x[j] = d[3 * k + j];
#define VEC(FIELD)                                                                \
  if (wr) for (size_t k = 0; k < n; k++) for (int j = 0; j < 3; j++) a[3 * k + j] = FIELD[j]; \
  xio(a, sizeof(float), 3 * n, f, wr);                                            \
  if (!wr) for (size_t k = 0; k < n; k++) for (int j = 0; j < 3; j++) FIELD[j] = a[3 * k + j];
  VEC(X[k].v_full)
  VEC(P[k].v)
  VEC(P[k].a_hydro)
#undef VEC
#define SCA(FIELD)                                                   \
  if (wr) for (size_t k = 0; k < n; k++) s[k] = FIELD;               \
  xio(s, sizeof(float), n, f, wr);                                   \
  if (!wr) for (size_t k = 0; k < n; k++) FIELD = s[k];
  SCA(X[k].u_full)
  SCA(P[k].u)
  SCA(P[k].u_dt)
  SCA(P[k].h)
  SCA(P[k].force.h_dt)
  SCA(P[k].rho)
  SCA(P[k].force.pressure)
  SCA(P[k].force.soundspeed)
  SCA(P[k].force.v_sig)
#undef SCA
  if (wr) for (size_t k = 0; k < n; k++) b[k] = P[k].time_bin;
  xio(b, 1, n, f, wr);
  if (!wr) for (size_t k = 0; k < n; k++) P[k].time_bin = b[k];
  if (wr) for (size_t k = 0; k < n; k++) b[k] = P[k].limiter_data.min_ngb_time_bin;
  xio(b, 1, n, f, wr);
  if (!wr) for (size_t k = 0; k < n; k++) P[k].limiter_data.min_ngb_time_bin = b[k];
  free(d);
  free(a);
  free(s);
  free(b);
}

int main(int argc, char **argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: ref_integrate in.bin out.bin\n");
    return 1;
  }
  FILE *fin = fopen(argv[1], "rb");
  if (!fin) return 2;
  struct integ_header hdr;
  xio(&hdr, sizeof(hdr), 1, fin, 0);
  if (memcmp(hdr.magic, "SPHINT01", 8) != 0) {
    fprintf(stderr, "ref_integrate: bad magic\n");
    return 2;
  }
  const size_t n = (size_t)hdr.n;
  struct part *P = xmalloc(n * sizeof(struct part));
  struct xpart *X = xmalloc(n * sizeof(struct xpart));
  io_state(fin, P, X, n, 0);
  fclose(fin);

  struct hydro_props hp;
  hydro_props_init_no_hydro(&hp);
  hp.CFL_condition = hdr.CFL;
  hp.log_max_h_change = hdr.log_max_h_change;
  hp.h_max = hdr.h_max;
  hp.h_min = hdr.h_min;
  hp.minimal_internal_energy = hdr.minimal_u;
  struct cosmology cosmo;
  cosmology_init_no_cosmo(&cosmo);
  struct phys_const pc;
  memset(&pc, 0, sizeof(pc));
  struct pressure_floor_props pfloor;
  memset(&pfloor, 0, sizeof(pfloor));
  struct entropy_floor_properties efloor;
  memset(&efloor, 0, sizeof(efloor));
  static struct space s;
  static struct engine e;
  memset(&e, 0, sizeof(e));
  e.hydro_properties = &hp;
  e.cosmology = &cosmo;
  e.physical_constants = &pc;
  e.pressure_floor_props = &pfloor;
  e.entropy_floor = &efloor;
  e.s = &s;
  e.policy = engine_policy_hydro;
  e.ti_current = hdr.ti_current;
  e.max_active_bin = (timebin_t)hdr.max_active_bin;
  e.time_base = hdr.time_base;
  e.time_base_inv = 1.0 / hdr.time_base;
  e.dt_min = hdr.dt_min;
  e.dt_max = hdr.dt_max;
  e.dt_max_RMS_displacement = FLT_MAX;

  const integertime_t ti_current = hdr.ti_current;
  const double time_base = hdr.time_base;
  for (size_t k = 0; k < n; k++) {
    struct part *p = &P[k];
    struct xpart *xp = &X[k];
    p->gpart = NULL;
    if (hdr.op == 1 || hdr.op == 2) {
      if (!part_is_active(p, &e)) continue; /* part_is_starting is the same test */
      const integertime_t ti_step = get_integer_timestep(p->time_bin);
      integertime_t ti_begin, ti_end;
      if (hdr.op == 1) {
        ti_begin = get_integer_time_begin(ti_current + 1, p->time_bin);
        ti_end = ti_begin + ti_step / 2;
      } else {
        ti_begin = get_integer_time_begin(ti_current, p->time_bin) + ti_step / 2;
        ti_end = ti_begin + ti_step / 2;
      }
      const double dt_kick_grav = kick_get_grav_kick_dt(ti_begin, ti_end, time_base, 0, &cosmo);
      const double dt_kick_hydro = kick_get_hydro_kick_dt(ti_begin, ti_end, time_base, 0, &cosmo);
      const double dt_kick_therm = kick_get_therm_kick_dt(ti_begin, ti_end, time_base, 0, &cosmo);
      const double dt_kick_corr = kick_get_corr_kick_dt(ti_begin, ti_end, time_base, 0, &cosmo);
      kick_part(p, xp, dt_kick_hydro, dt_kick_grav, 0., dt_kick_therm, dt_kick_corr, &cosmo,
                &hp, &efloor, NULL, ti_begin, ti_end, -1, 0);
      if (hdr.op == 2) hydro_reset_predicted_values(p, xp, &cosmo, &pfloor);
    } else if (hdr.op == 3) {
      const integertime_t ti_old = hdr.ti_old;
      const double dt = (ti_current - ti_old) * time_base;
      const double cell_loc[3] = {0., 0., 0.};
      drift_part(p, xp, dt, dt, dt, dt, ti_old, ti_current, &e, NULL, cell_loc);
      p->h = min(p->h, hp.h_max);
      p->h = max(p->h, hp.h_min);
    } else if (hdr.op == 4) {
      if (!part_is_active(p, &e)) continue;
      const integertime_t ti_rt = get_part_rt_timestep(p, xp, &e);
      const integertime_t ti_new_step = get_part_timestep(p, xp, &e, ti_rt);
      p->time_bin = get_time_bin(ti_new_step);
    }
  }

  FILE *fo = fopen(argv[2], "wb");
  if (!fo) return 2;
  xio("SPHINT02", 1, 8, fo, 1);
  io_state(fo, P, X, n, 1);
  fclose(fo);
  return 0;
}
