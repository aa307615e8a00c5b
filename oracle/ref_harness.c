/* Oracle driver for the reference SWIFT hydro hot path.
 *
 * Test infrastructure only: this program is linked against the reference
 * sources compiled by oracle/build_ref.sh and runs the reference's own
 * functions on an input box, one stage at a time, in a fixed single-threaded
 * order, dumping every per-particle result so the oracle's C restatement
 * (oracle/sph_oracle.c) and the GPU path can be pinned against it.
 *
 * Reference calls used (paths relative to the reference's src/):
 *   space_init (space.c:1136), space_rebuild (space_rebuild.c:49)
 *   runner_do_hydro_sort (runner_sort.c:203)
 *   runner_dosub_self1_density / runner_dosub_pair1_density
 *       (runner_doiact_functions_hydro.h:3037 / :2933)
 *   runner_do_ghost (runner_ghost.c:1113)
 *   runner_dosub_self2_force / runner_dosub_pair2_force (:3203 / :3102)
 *   runner_do_end_hydro_force (runner_others.c:815)
 *   scheduler_addtask (scheduler.c:164), scheduler_splittasks_mapper
 *       (scheduler_splittasks.c:538) when the header asks for task splitting
 *
 * Input  (argv[1]): "SPHIN002" header + SoA arrays (see oracle/io.py).
 * Output (argv[2]): "SPHOUT01" header + per-particle results in input order,
 *                   followed by the cell tree in depth-first order.
 * Optional (argv[3]): "SPHSRT01" + the 13 sort arrays of every non-empty
 *                   cell, depth first: per cell int32 first (cell-sorted
 *                   order), count, depth, then 13 x (count + 1) entries
 *                   {float d; int i} as runner_do_hydro_sort left them.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* config.h and swift.h come in through -include on the command line. */
#include "runner.h"
#include "runner_doiact_hydro.h"
#include "scheduler.h"
#include "space_getsid.h"

/* Defined (not static) in scheduler_splittasks.c:538; no header declares it. */
void scheduler_splittasks_mapper(void *map_data, int num_elements, void *extra_data);

#define STAGE_DENSITY 1
#define STAGE_GHOST 2
#define STAGE_FORCE 4
/* Run one full step with every particle active first, then the requested
 * stages at max_active_bin on the state it leaves (see redrift below). */
#define STAGE_PRIME 8

struct in_header {
  char magic[8];
  int64_t n;
  double dim[3];
  float eta, h_tolerance, h_max, h_min, alpha;
  int32_t max_iter, max_active_bin, periodic, stages, max_top_level_cells;
  int32_t subsize_self, subsize_pair; /* both 0: no task splitting */
};

static void *xmalloc(size_t n) {
  void *p = NULL;
  if (posix_memalign(&p, 64, n ? n : 64) != 0) {
    fprintf(stderr, "ref_harness: out of memory\n");
    exit(2);
  }
  memset(p, 0, n ? n : 64);
  return p;
}

static void xread(void *dst, size_t sz, size_t n, FILE *f) {
  if (fread(dst, sz, n, f) != n) {
    fprintf(stderr, "ref_harness: short read\n");
    exit(2);
  }
}

/* Density links of the cells the tasks hold, so that the ghost's redo path
 * (runner_ghost.c:1548-1579) walks real links as in the engine. */
static struct link *link_pool;
static int link_used;
static void add_link(struct link **head, struct task *t) {
  struct link *l = &link_pool[link_used++];
  l->t = t;
  l->next = *head;
  *head = l;
}

/* Depth-first enumeration of the tree, writing one record per cell. */
struct cell_rec {
  double loc[3], width[3];
  float h_max, h_max_active, dmin;
  int32_t depth, split, count, first, parent, top;
};
static struct cell_rec *recs;
static int nrecs;
static void collect(const struct cell *c, const struct part *base, int parent,
                    int top, int32_t *leaf_of) {
  const int me = nrecs++;
  struct cell_rec *r = &recs[me];
  for (int k = 0; k < 3; k++) {
    r->loc[k] = c->loc[k];
    r->width[k] = c->width[k];
  }
  r->h_max = c->hydro.h_max;
  r->h_max_active = c->hydro.h_max_active;
  r->dmin = c->dmin;
  r->depth = c->depth;
  r->split = c->split;
  r->count = c->hydro.count;
  r->first = (int32_t)(c->hydro.parts - base);
  r->parent = parent;
  r->top = top;
  if (c->split) {
    for (int k = 0; k < 8; k++)
      if (c->progeny[k] != NULL) collect(c->progeny[k], base, me, top, leaf_of);
  } else {
    for (int k = 0; k < c->hydro.count; k++)
      leaf_of[c->hydro.parts[k].id] = me;
  }
}

/* State change between the priming step and the measured step, as the
 * reference's drift does it with a zero drift (cell_drift.c:330-371): active
 * particles restart from the caller's predicted h (h_in, already inside
 * [h_min, h_max]), every particle takes the depth_h of its h
 * (cell_set_part_h_depth, cell.h:1787), every cell its h_max / h_max_active
 * from its particles, and the unskip sets h_max_old = h_max
 * (cell_unskip.c:875-880).  Inactive particles keep everything. */
static void redrift(struct cell *c, const struct engine *e, const float *h_in) {
  float h_max = 0.f, h_max_active = 0.f;
  if (c->split) {
    for (int k = 0; k < 8; k++) {
      struct cell *cp = c->progeny[k];
      if (cp == NULL) continue;
      redrift(cp, e, h_in);
      h_max = max(h_max, cp->hydro.h_max);
      h_max_active = max(h_max_active, cp->hydro.h_max_active);
    }
  } else {
    for (int k = 0; k < c->hydro.count; k++) {
      struct part *p = &c->hydro.parts[k];
      if (part_is_active(p, e)) p->h = h_in[p->id];
      cell_set_part_h_depth(p, c);
      h_max = max(h_max, p->h);
      if (part_is_active(p, e)) h_max_active = max(h_max_active, p->h);
    }
  }
  c->hydro.h_max = h_max;
  c->hydro.h_max_active = h_max_active;
  c->hydro.h_max_old = h_max;
  c->hydro.dx_max_part_old = 0.f;
}

static void dump_sorts(FILE *f, const struct cell *c, const struct part *base) {
  if (c->hydro.count == 0) return;
  const int32_t rec[3] = {(int32_t)(c->hydro.parts - base), c->hydro.count, c->depth};
  fwrite(rec, sizeof(int32_t), 3, f);
  for (int j = 0; j < 13; j++)
    fwrite(cell_get_hydro_sorts(c, j), sizeof(struct sort_entry),
           (size_t)c->hydro.count + 1, f);
  if (c->split)
    for (int k = 0; k < 8; k++)
      if (c->progeny[k] != NULL) dump_sorts(f, c->progeny[k], base);
}

int main(int argc, char **argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: ref_harness in.bin out.bin\n");
    return 1;
  }
  FILE *fin = fopen(argv[1], "rb");
  if (!fin) return 2;
  struct in_header hdr;
  xread(&hdr, sizeof(hdr), 1, fin);
  if (memcmp(hdr.magic, "SPHIN002", 8) != 0) {
    fprintf(stderr, "ref_harness: bad magic\n");
    return 2;
  }
  const size_t n = (size_t)hdr.n;
  double *x = xmalloc(n * 3 * sizeof(double));
  float *v = xmalloc(n * 3 * sizeof(float));
  float *m = xmalloc(n * sizeof(float));
  float *h = xmalloc(n * sizeof(float));
  float *u = xmalloc(n * sizeof(float));
  int8_t *tb = xmalloc(n);
  xread(x, sizeof(double), 3 * n, fin);
  xread(v, sizeof(float), 3 * n, fin);
  xread(m, sizeof(float), n, fin);
  xread(h, sizeof(float), n, fin);
  xread(u, sizeof(float), n, fin);
  xread(tb, 1, n, fin);
  fclose(fin);

  struct part *parts = xmalloc(n * sizeof(struct part));
  for (size_t k = 0; k < n; k++) {
    struct part *p = &parts[k];
    p->id = (long long)k;
    for (int d = 0; d < 3; d++) {
      p->x[d] = x[3 * k + d];
      p->v[d] = v[3 * k + d];
    }
    p->mass = m[k];
    p->h = h[k];
    p->u = u[k];
    p->time_bin = tb[k];
  }

  /* Physics and engine context, filled the way the reference's own hydro
   * tests do it (tests/test125cells.c:586-626). */
  struct hydro_props hp;
  hydro_props_init_no_hydro(&hp);
  hp.eta_neighbours = hdr.eta;
  hp.h_tolerance = hdr.h_tolerance;
  hp.h_max = hdr.h_max;
  hp.h_min = hdr.h_min;
  hp.h_min_ratio = 0.f;
  hp.max_smoothing_iterations = hdr.max_iter;
  hp.CFL_condition = 0.1f;
  hp.viscosity.alpha = hdr.alpha;

  struct cosmology cosmo;
  cosmology_init_no_cosmo(&cosmo);
  struct phys_const pc;
  memset(&pc, 0, sizeof(pc));
  pc.const_newton_G = 1.f;
  struct pressure_floor_props pfloor;
  memset(&pfloor, 0, sizeof(pfloor));
  struct sink_props sink_props;
  memset(&sink_props, 0, sizeof(sink_props));
  struct lightcone_array_props lc;
  memset(&lc, 0, sizeof(lc));

  struct swift_params *params = xmalloc(sizeof(struct swift_params));
  if (hdr.max_top_level_cells > 0) {
    char kv[128];
    snprintf(kv, sizeof(kv), "Scheduler:max_top_level_cells:%d",
             (int)hdr.max_top_level_cells);
    parser_set_param(params, kv);
  }

  static struct space s;
  static struct engine e;
  memset(&e, 0, sizeof(e));
  e.hydro_properties = &hp;
  e.physical_constants = &pc;
  e.cosmology = &cosmo;
  e.pressure_floor_props = &pfloor;
  e.sink_properties = &sink_props;
  e.lightcone_array_properties = &lc;
  e.policy = engine_policy_hydro;
  e.ti_current = 0;
  /* the tree's h_max_active is built for the first step that runs */
  e.max_active_bin =
      (hdr.stages & STAGE_PRIME) ? 127 : (timebin_t)hdr.max_active_bin;
  e.nodeID = 0;
  e.nr_nodes = 1;
  e.nr_threads = 1;
  e.time_base = 1e-10;
  threadpool_init(&e.threadpool, 1);

  double dim[3] = {hdr.dim[0], hdr.dim[1], hdr.dim[2]};
  space_init(&s, params, &cosmo, dim, &hp, parts, NULL, NULL, NULL, NULL, n, 0,
             0, 0, 0, 0, hdr.periodic, 1, 0, 0, /*hydro=*/1, 0, 0, 0, 0, 0, 0,
             /*verbose=*/0, /*dry_run=*/0, 1);
  s.e = &e;
  e.s = &s;
  /* Per-thread sub-cell pools, as engine_config.c:894-897 sets them up. */
  s.cells_sub = (struct cell **)calloc(2, sizeof(struct cell *));
  s.multipoles_sub =
      (struct gravity_tensors **)calloc(2, sizeof(struct gravity_tensors *));
  space_rebuild(&s, 0, 0);

  struct part *P = s.parts; /* the space may have reordered particles */
  struct runner r;
  memset(&r, 0, sizeof(r));
  r.e = &e;

  /* h_max_old / dx_max_part_old are refreshed by the unskip pass in the
   * engine (cell_unskip.c:875-880); set them the same way here. */
  const int ncells = s.nr_cells;
  for (int c = 0; c < ncells; c++) {
    struct cell *top = &s.cells_top[c];
    struct cell *stack[256];
    int sp = 0;
    stack[sp++] = top;
    while (sp) {
      struct cell *cc = stack[--sp];
      cc->hydro.h_max_old = cc->hydro.h_max;
      cc->hydro.dx_max_part_old = 0.f;
      cc->hydro.dx_max_sort_old = 0.f;
      if (cc->split)
        for (int k = 0; k < 8; k++)
          if (cc->progeny[k]) stack[sp++] = cc->progeny[k];
    }
  }

  /* Sort every top cell along all 13 axes (and its progeny, recursively). */
  for (int c = 0; c < ncells; c++)
    if (s.cells_top[c].hydro.count > 0)
      runner_do_hydro_sort(&r, &s.cells_top[c], 0x1FFF, 0, 0, 0, 0);

  if (argc > 3) {
    FILE *fs = fopen(argv[3], "wb");
    if (!fs) return 2;
    fwrite("SPHSRT01", 1, 8, fs);
    for (int c = 0; c < ncells; c++) dump_sorts(fs, &s.cells_top[c], s.parts);
    fclose(fs);
  }

  /* Task list: one self task per non-empty top cell, one pair task per
   * neighbouring non-empty top-cell pair (26-neighbourhood, periodic),
   * created through the reference's scheduler_addtask.  With split sizes in
   * the header the reference's own splitter then splits them
   * (Scheduler:cell_sub_size_self_hydro / cell_sub_size_pair_hydro), one
   * task at a time in array order as a single-threaded mapper call does. */
  const int *cdim = s.cdim;
  static struct scheduler sched;
  memset(&sched, 0, sizeof(sched));
  sched.space = &s;
  sched.nodeID = 0;
  /* a cell holds at most one self task and 26 pair tasks */
  sched.size = 27 * (s.tot_cells + ncells) + 64;
  sched.tasks = xmalloc(sizeof(struct task) * (size_t)sched.size);
  sched.tasks_ind = xmalloc(sizeof(int) * (size_t)sched.size);
  for (int i = 0; i < cdim[0]; i++)
    for (int j = 0; j < cdim[1]; j++)
      for (int k = 0; k < cdim[2]; k++) {
        const int cid = cell_getid(cdim, i, j, k);
        struct cell *ci = &s.cells_top[cid];
        if (ci->hydro.count == 0) continue;
        scheduler_addtask(&sched, task_type_self, task_subtype_density, 0, 0, ci, NULL);
        for (int di = -1; di <= 1; di++)
          for (int dj = -1; dj <= 1; dj++)
            for (int dk = -1; dk <= 1; dk++) {
              int ii = i + di, jj = j + dj, kk = k + dk;
              if (hdr.periodic) {
                ii = (ii + cdim[0]) % cdim[0];
                jj = (jj + cdim[1]) % cdim[1];
                kk = (kk + cdim[2]) % cdim[2];
              } else if (ii < 0 || ii >= cdim[0] || jj < 0 || jj >= cdim[1] ||
                         kk < 0 || kk >= cdim[2])
                continue;
              const int cjd = cell_getid(cdim, ii, jj, kk);
              if (cjd <= cid) continue;
              struct cell *cj = &s.cells_top[cjd];
              if (cj->hydro.count == 0) continue;
              struct cell *a = ci, *b = cj;
              double shift[3];
              const int sid = space_getsid_and_swap_cells(&s, &a, &b, shift);
              scheduler_addtask(&sched, task_type_pair, task_subtype_density, sid, 0, ci, cj);
            }
      }
  if (hdr.subsize_self > 0 || hdr.subsize_pair > 0) {
    space_subsize_self_hydro = hdr.subsize_self;
    space_subsize_pair_hydro = hdr.subsize_pair;
    scheduler_splittasks_mapper(sched.tasks, sched.tasks_next, &sched);
  }
  /* The tasks the split left (type none dropped, order kept), linked to the
   * cells they hold in task order (engine_maketasks.c:2311-2333). */
  struct task *tasks = sched.tasks;
  int ntasks = 0;
  for (int t = 0; t < sched.tasks_next; t++)
    if (tasks[t].type == task_type_self || tasks[t].type == task_type_pair)
      tasks[ntasks++] = tasks[t];
  link_pool = xmalloc(sizeof(struct link) * ((size_t)ntasks * 2 + 1));
  for (int t = 0; t < ntasks; t++) {
    add_link(&tasks[t].ci->hydro.density, &tasks[t]);
    if (tasks[t].type == task_type_pair) add_link(&tasks[t].cj->hydro.density, &tasks[t]);
  }

  const size_t nf = 24;
  float *res = xmalloc(n * nf * sizeof(float));
/* the oracle's integer columns 0-5 and 10; 6-9 (neighbour counters the
 * reference does not keep) are written as -1 */
#define NI 11
  int32_t *ipart = xmalloc(n * NI * sizeof(int32_t));

  const int prime = (hdr.stages & STAGE_PRIME) != 0;
  for (int pass = prime ? 0 : 1; pass <= 1; pass++) {
    int stages = hdr.stages & (STAGE_DENSITY | STAGE_GHOST | STAGE_FORCE);
    if (pass == 0) {
      stages = STAGE_DENSITY | STAGE_GHOST | STAGE_FORCE;
      e.max_active_bin = 127; /* every particle active */
    } else {
      e.max_active_bin = (timebin_t)hdr.max_active_bin;
      if (prime)
        for (int c = 0; c < ncells; c++)
          if (s.cells_top[c].hydro.count > 0) redrift(&s.cells_top[c], &e, h);
    }
    if (stages & STAGE_DENSITY) {
      for (size_t k = 0; k < s.nr_parts; k++)
        if (pass == 0 || !prime || part_is_active(&P[k], &e))
          hydro_init_part(&P[k], &s.hs);
      for (int t = 0; t < ntasks; t++) {
        if (tasks[t].type == task_type_self)
          runner_dosub_self1_density(&r, tasks[t].ci, 0, 0);
        else
          runner_dosub_pair1_density(&r, tasks[t].ci, tasks[t].cj, 0, 0);
      }
      for (size_t k = 0; k < s.nr_parts; k++) {
        const struct part *p = &P[k];
        float *o = &res[nf * (size_t)p->id];
        o[0] = p->rho;
        o[1] = p->density.rho_dh;
        o[2] = p->density.wcount;
        o[3] = p->density.wcount_dh;
        o[4] = p->density.div_v;
        o[5] = p->density.rot_v[0];
        o[6] = p->density.rot_v[1];
        o[7] = p->density.rot_v[2];
      }
    }
    if (stages & STAGE_GHOST) {
      for (int c = 0; c < ncells; c++)
        runner_do_ghost(&r, &s.cells_top[c], 0, 1, 0);
      for (size_t k = 0; k < s.nr_parts; k++) {
        const struct part *p = &P[k];
        float *o = &res[nf * (size_t)p->id];
        o[8] = p->h;
        o[9] = p->rho;
        o[10] = p->force.f;
        o[11] = p->force.pressure;
        o[12] = p->force.soundspeed;
        o[13] = p->force.balsara;
        o[14] = p->force.v_sig;
      }
    }
    if (stages & STAGE_FORCE) {
      for (int t = 0; t < ntasks; t++) {
        if (tasks[t].type == task_type_self)
          runner_dosub_self2_force(&r, tasks[t].ci, 0, 0);
        else
          runner_dosub_pair2_force(&r, tasks[t].ci, tasks[t].cj, 0, 0);
      }
      for (int c = 0; c < ncells; c++)
        runner_do_end_hydro_force(&r, &s.cells_top[c], 0);
      for (size_t k = 0; k < s.nr_parts; k++) {
        const struct part *p = &P[k];
        float *o = &res[nf * (size_t)p->id];
        o[15] = p->a_hydro[0];
        o[16] = p->a_hydro[1];
        o[17] = p->a_hydro[2];
        o[18] = p->u_dt;
        o[19] = p->force.h_dt;
        o[20] = p->force.v_sig;
      }
    }
  }

  /* Tree placement per particle (same layout as the oracle's integer
   * block): leaf first index, leaf count, leaf depth, depth_h, position in
   * the cell-sorted order, top cell id. */
  recs = xmalloc(sizeof(struct cell_rec) * (size_t)(s.tot_cells + ncells + 8));
  int32_t *leaf_of = xmalloc(n * sizeof(int32_t));
  for (int c = 0; c < ncells; c++) collect(&s.cells_top[c], P, -1, c, leaf_of);
  for (size_t k = 0; k < n; k++) {
    const struct cell_rec *lr = &recs[leaf_of[P[k].id]];
    int32_t *ip = &ipart[NI * (size_t)P[k].id];
    ip[0] = lr->first;
    ip[1] = lr->count;
    ip[2] = lr->depth;
    ip[3] = P[k].depth_h;
    ip[4] = (int32_t)k;
    ip[5] = lr->top;
    ip[6] = ip[7] = ip[8] = ip[9] = -1;
    ip[10] = (hdr.stages & STAGE_FORCE) ? P[k].limiter_data.min_ngb_time_bin : -1;
  }

  FILE *fo = fopen(argv[2], "wb");
  if (!fo) return 2;
  fwrite("SPHOUT01", 1, 8, fo);
  int64_t hdr_out[7] = {(int64_t)n, (int64_t)nf, nrecs, cdim[0], cdim[1],
                        cdim[2], NI};
  fwrite(hdr_out, sizeof(int64_t), 7, fo);
  fwrite(s.width, sizeof(double), 3, fo);
  fwrite(res, sizeof(float), n * nf, fo);
  fwrite(ipart, sizeof(int32_t), NI * n, fo);
  fwrite(recs, sizeof(struct cell_rec), (size_t)nrecs, fo);
  fclose(fo);
  return 0;
}
