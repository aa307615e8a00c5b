/* runner_gb300.c -- the reference-side binding of the GB300 library.
 *
 * A SWIFT maintainer adds this file to SWIFT's src/ and links
 * libswiftgb300.so in place of the reference's hydro loops: it defines the
 * reference's own runner symbols for the Minimal-SPH hot path with the
 * reference's signatures, and forwards each to the library's C ABI
 * (include/swift_gb300.h):
 *
 *   runner_dosub_self1_density, runner_dosub_pair1_density,
 *   runner_dosub_self2_force, runner_dosub_pair2_force
 *                                       (runner_doiact_hydro.h:187-195)
 *   runner_do_ghost                     (runner.h:94, runner_ghost.c:1113)
 *   runner_do_end_hydro_force           (runner.h:121, runner_others.c:815)
 *   runner_do_hydro_sort                (runner.h:105, runner_sort.c:203)
 *
 * plus three engine hooks: gb300_rebuild after space_rebuild
 * (engine_rebuild, engine.c:1351), gb300_start_step before the hydro tasks
 * of a step (the drifted positions and h, the struct part fields a kick
 * changed, the active set), gb300_fetch after the force tasks (results back
 * into struct part).
 *
 * Error convention: the reference's loops are void and call error()
 * (error.h:60) on fatal conditions; the library returns codes, which this
 * file turns back into error() with the library's message (on a machine
 * without a GPU the first GPU call reports SPHGPU_ENODEV).
 *
 * Threading: runner_main calls these symbols from every runner thread; the
 * library serialises on the space's CUDA stream, and one mutex here keeps
 * calls on the space from overlapping.
 *
 * Task granularity: the library plans the loops per top-level cell and
 * top-cell pair (the recursion below them is its own), so the scheduler's
 * hydro tasks must stay at the top level (Scheduler:cell_sub_size_*_hydro
 * large); a task on a deeper cell is reported through error().
 */
#include "../../include/swift_gb300.h"

#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>

#include "cell.h"
#include "engine.h"
#include "error.h"
#include "runner.h"
#include "space.h"

static sphgpu_space *g_space = NULL;
static pthread_mutex_t g_lock = PTHREAD_MUTEX_INITIALIZER;
/* The library's cell records (first, count, depth, parent, top), refreshed
 * at every rebuild: they map SWIFT cells to library cell ids for the sorts. */
static int32_t *g_tree = NULL;
static int32_t g_ncells = 0;
static integertime_t g_sorted_ti = -1;

#define GB300_CHECK(call)                                              \
  do {                                                                 \
    const int rc_ = (call);                                            \
    if (rc_ != SPHGPU_OK) {                                            \
      pthread_mutex_unlock(&g_lock);                                   \
      error("gb300: %s (code %d)", sphgpu_last_error(), rc_);          \
    }                                                                  \
  } while (0)

static void *gb300_malloc(size_t bytes) {
  void *p = malloc(bytes ? bytes : 1);
  if (!p) error("gb300: host allocation of %zu bytes failed", bytes);
  return p;
}

/* Called after space_rebuild: one library space per rebuild, built from
 * the particles as the rebuild left them. */
void gb300_rebuild(struct engine *e) {
  const struct space *s = e->s;
  const size_t n = s->nr_parts;
  double *x = gb300_malloc(3 * n * sizeof(double));
  float *v = gb300_malloc(3 * n * sizeof(float));
  float *m = gb300_malloc(n * sizeof(float));
  float *h = gb300_malloc(n * sizeof(float));
  float *u = gb300_malloc(n * sizeof(float));
  int8_t *tb = gb300_malloc(n);
  for (size_t k = 0; k < n; k++) {
    const struct part *p = &s->parts[k];
    for (int d = 0; d < 3; d++) {
      x[3 * k + d] = p->x[d];
      v[3 * k + d] = p->v[d];
    }
    m[k] = p->mass;
    h[k] = p->h;
    u[k] = p->u;
    tb[k] = p->time_bin;
  }
  sphgpu_params prm;
  sphgpu_default_params(&prm);
  for (int d = 0; d < 3; d++) prm.dim[d] = s->dim[d];
  prm.periodic = s->periodic;
  prm.eta = e->hydro_properties->eta_neighbours;
  prm.h_tolerance = e->hydro_properties->h_tolerance;
  prm.h_max = e->hydro_properties->h_max;
  prm.h_min = e->hydro_properties->h_min;
  prm.alpha = e->hydro_properties->viscosity.alpha;
  prm.max_iter = e->hydro_properties->max_smoothing_iterations;
  prm.max_active_bin = e->max_active_bin;
  pthread_mutex_lock(&g_lock);
  if (g_space) sphgpu_space_destroy(g_space);
  g_space = NULL;
  GB300_CHECK(sphgpu_space_create(&prm, (int64_t)n, x, v, m, h, u, tb, &g_space));
  GB300_CHECK(sphgpu_space_tree(g_space, &g_ncells, NULL));
  free(g_tree);
  g_tree = gb300_malloc(5 * (size_t)g_ncells * sizeof(int32_t));
  GB300_CHECK(sphgpu_space_tree(g_space, &g_ncells, g_tree));
  g_sorted_ti = -1;
  pthread_mutex_unlock(&g_lock);
  free(x);
  free(v);
  free(m);
  free(h);
  free(u);
  free(tb);
}

/* Before the hydro tasks of a step: the positions and h the drift gave
 * since the rebuild (the particles keep their cells: the library measures
 * dx_max_part and checks cell_need_rebuild_for_hydro_pair, cell.h:1237, the
 * test the engine's own rebuild decision makes), the struct part fields the
 * loops read that a kick changed (v, mass, u), then the active set
 * (active.h:349 part_is_active). */
void gb300_start_step(struct engine *e) {
  const struct space *s = e->s;
  const size_t n = s->nr_parts;
  double *x = gb300_malloc(3 * n * sizeof(double));
  float *h = gb300_malloc(n * sizeof(float));
  float *v = gb300_malloc(3 * n * sizeof(float));
  float *m = gb300_malloc(n * sizeof(float));
  float *u = gb300_malloc(n * sizeof(float));
  for (size_t k = 0; k < n; k++) {
    const struct part *p = &s->parts[k];
    for (int d = 0; d < 3; d++) {
      x[3 * k + d] = p->x[d];
      v[3 * k + d] = p->v[d];
    }
    h[k] = p->h;
    m[k] = p->mass;
    u[k] = p->u;
  }
  pthread_mutex_lock(&g_lock);
  if (!g_space) {
    pthread_mutex_unlock(&g_lock);
    error("gb300: no space; call gb300_rebuild after space_rebuild");
  }
  GB300_CHECK(sphgpu_space_drift(g_space, x, h, NULL));
  GB300_CHECK(sphgpu_space_update(g_space, v, m, u, NULL));
  GB300_CHECK(sphgpu_set_active(g_space, e->max_active_bin));
  pthread_mutex_unlock(&g_lock);
  free(x);
  free(h);
  free(v);
  free(m);
  free(u);
}

/* After the force tasks: the results into struct part (column layout of
 * sphgpu_download, include/swift_gb300.h). */
void gb300_fetch(struct engine *e) {
  const size_t n = e->s->nr_parts;
  float *f = gb300_malloc(24 * n * sizeof(float));
  pthread_mutex_lock(&g_lock);
  GB300_CHECK(sphgpu_download(g_space, f, NULL));
  pthread_mutex_unlock(&g_lock);
  for (size_t k = 0; k < n; k++) {
    struct part *p = &e->s->parts[k];
    const float *o = f + 24 * k;
    p->h = o[8];
    p->rho = o[9];
    p->force.f = o[10];
    p->force.pressure = o[11];
    p->force.soundspeed = o[12];
    p->force.balsara = o[13];
    p->a_hydro[0] = o[15];
    p->a_hydro[1] = o[16];
    p->a_hydro[2] = o[17];
    p->u_dt = o[18];
    p->force.h_dt = o[19];
    p->force.v_sig = o[20];
  }
  free(f);
}

/* The library's id of a top-level cell: SWIFT's cells_top are numbered by
 * cell_getid (cell.h:532), as the library numbers its top cells. */
static int32_t top_id(const struct runner *r, const struct cell *c) {
  if (c->top != c)
    error("gb300: hydro task on a cell below the top level; set "
          "Scheduler:cell_sub_size_self_hydro / cell_sub_size_pair_hydro large");
  return (int32_t)(c - r->e->s->cells_top);
}

void runner_dosub_self1_density(struct runner *r, struct cell *c,
                                int recurse_below_h_max, const int gettimer) {
  const int32_t id = top_id(r, c);
  pthread_mutex_lock(&g_lock);
  GB300_CHECK(sphgpu_dosub_self1_density(g_space, id, NULL));
  pthread_mutex_unlock(&g_lock);
}

void runner_dosub_pair1_density(struct runner *r, struct cell *ci, struct cell *cj,
                                int recurse_below_h_max, const int gettimer) {
  const int32_t a = top_id(r, ci), b = top_id(r, cj);
  pthread_mutex_lock(&g_lock);
  GB300_CHECK(sphgpu_dosub_pair1_density(g_space, a, b, NULL));
  pthread_mutex_unlock(&g_lock);
}

void runner_do_ghost(struct runner *r, struct cell *c, const int offset,
                     const int ntasks, const int timer) {
  const int32_t id = top_id(r, c);
  pthread_mutex_lock(&g_lock);
  GB300_CHECK(sphgpu_do_ghost(g_space, id, NULL));
  pthread_mutex_unlock(&g_lock);
}

void runner_dosub_self2_force(struct runner *r, struct cell *c,
                              int recurse_below_h_max, const int gettimer) {
  const int32_t id = top_id(r, c);
  pthread_mutex_lock(&g_lock);
  GB300_CHECK(sphgpu_dosub_self2_force(g_space, id, NULL));
  pthread_mutex_unlock(&g_lock);
}

void runner_dosub_pair2_force(struct runner *r, struct cell *ci, struct cell *cj,
                              int recurse_below_h_max, const int gettimer) {
  const int32_t a = top_id(r, ci), b = top_id(r, cj);
  pthread_mutex_lock(&g_lock);
  GB300_CHECK(sphgpu_dosub_pair2_force(g_space, a, b, NULL));
  pthread_mutex_unlock(&g_lock);
}

void runner_do_end_hydro_force(struct runner *r, struct cell *c, int timer) {
  pthread_mutex_lock(&g_lock);
  GB300_CHECK(sphgpu_do_end_hydro_force(g_space, NULL));
  pthread_mutex_unlock(&g_lock);
}

/* The library cell with the same first particle and depth (the library
 * keeps the rebuild's particle order, so every SWIFT cell has one). */
static int32_t lib_cell(const struct space *s, const struct cell *c) {
  const int32_t first = (int32_t)(c->hydro.parts - s->parts);
  for (int32_t k = 0; k < g_ncells; k++)
    if (g_tree[5 * k] == first && g_tree[5 * k + 2] == c->depth && g_tree[5 * k + 1] > 0)
      return k;
  return -1;
}

/* The library sorts the whole tree on the device once per step
 * (sphgpu_hydro_sort: the reference's arrays, ties included); each call then
 * copies one cell's requested arrays into the cell's own sort memory. */
void runner_do_hydro_sort(struct runner *r, struct cell *c, int flags,
                          const int cleanup, const int lock,
                          const int rt_requests_sort, const int clock) {
  pthread_mutex_lock(&g_lock);
  if (g_sorted_ti != r->e->ti_current) {
    GB300_CHECK(sphgpu_hydro_sort(g_space, 0x1FFF, NULL));
    g_sorted_ti = r->e->ti_current;
  }
  const int32_t id = lib_cell(r->e->s, c);
  if (id < 0) {
    pthread_mutex_unlock(&g_lock);
    error("gb300: cell (depth %d, %d particles) not in the library's tree", c->depth,
          c->hydro.count);
  }
  cell_malloc_hydro_sorts(c, flags);
  float *d = gb300_malloc((c->hydro.count + 1) * sizeof(float));
  int32_t *i = gb300_malloc((c->hydro.count + 1) * sizeof(int32_t));
  for (int j = 0; j < 13; j++) {
    if (!(flags & (1 << j))) continue;
    GB300_CHECK(sphgpu_cell_sort(g_space, id, j, d, i));
    struct sort_entry *se = cell_get_hydro_sorts(c, j);
    for (int k = 0; k <= c->hydro.count; k++) {
      se[k].d = d[k];
      se[k].i = i[k];
    }
    c->hydro.sorted |= (1 << j);
  }
  pthread_mutex_unlock(&g_lock);
  free(d);
  free(i);
}
