/* shim_driver.c -- a test program for the reference-side shim
 * (swift_gb300/shim/runner_gb300.c), built against the reference's own
 * headers and objects the way tests/test125cells.c builds its cells: a
 * periodic unit box of 8^3 jittered-lattice particles in struct part, a
 * hand-filled engine, space and runner, 2^3 top-level cells.  argv[1] names
 * the reference symbol to call after gb300_rebuild; the program prints
 * "rebuild ok" and, if the call returns, "returned".  A failing library call
 * ends the program through the reference's error() (exit status 1). */
#include <float.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

void gb300_rebuild(struct engine *e);
void gb300_start_step(struct engine *e);
void gb300_fetch(struct engine *e);

int main(int argc, char **argv) {
  if (argc < 2) return 2;
  const int side = 8, ncell = 2;
  const size_t n = (size_t)side * side * side;
  static struct engine e;
  static struct space s;
  static struct hydro_props hp;
  static struct runner r;
  struct part *parts = NULL;
  if (posix_memalign((void **)&parts, 128, n * sizeof(struct part)) != 0) return 3;
  memset(parts, 0, n * sizeof(struct part));
  srand(7);
  for (int i = 0; i < side; i++)
    for (int j = 0; j < side; j++)
      for (int k = 0; k < side; k++) {
        struct part *p = &parts[(i * side + j) * side + k];
        const int ijk[3] = {i, j, k};
        for (int d = 0; d < 3; d++) {
          const double jit = 0.2 * ((double)rand() / RAND_MAX - 0.5);
          p->x[d] = (ijk[d] + 0.5 + jit) / side;
          p->v[d] = 0.05f * ((float)rand() / RAND_MAX - 0.5f);
        }
        p->mass = 1.f / n;
        p->h = 1.2348f / side;
        p->u = 1.f;
        p->time_bin = 1;
      }
  hp.eta_neighbours = 1.2348f;
  hp.h_tolerance = 1e-4f;
  hp.h_max = FLT_MAX;
  hp.h_min = 0.f;
  hp.max_smoothing_iterations = 30;
  hp.viscosity.alpha = 0.8f;
  s.dim[0] = s.dim[1] = s.dim[2] = 1.0;
  s.periodic = 1;
  s.nr_parts = n;
  s.parts = parts;
  s.cdim[0] = s.cdim[1] = s.cdim[2] = ncell;
  s.cells_top = calloc(ncell * ncell * ncell, sizeof(struct cell));
  for (int c = 0; c < ncell * ncell * ncell; c++) {
    s.cells_top[c].top = &s.cells_top[c];
    s.cells_top[c].hydro.parts = parts;
    s.cells_top[c].hydro.count = 0;
  }
  s.cells_top[0].hydro.count = (int)n;
  e.s = &s;
  e.hydro_properties = &hp;
  e.max_active_bin = num_time_bins;
  e.ti_current = 0;
  r.e = &e;
  gb300_rebuild(&e);
  printf("rebuild ok\n");
  fflush(stdout);
  struct cell *c0 = &s.cells_top[0], *c1 = &s.cells_top[1];
  const char *call = argv[1];
  if (!strcmp(call, "rebuild")) {
  } else if (!strcmp(call, "runner_dosub_self1_density")) {
    runner_dosub_self1_density(&r, c0, 0, 0);
  } else if (!strcmp(call, "runner_dosub_pair1_density")) {
    runner_dosub_pair1_density(&r, c0, c1, 0, 0);
  } else if (!strcmp(call, "runner_do_ghost")) {
    runner_do_ghost(&r, c0, 0, 1, 0);
  } else if (!strcmp(call, "runner_dosub_self2_force")) {
    runner_dosub_self2_force(&r, c0, 0, 0);
  } else if (!strcmp(call, "runner_dosub_pair2_force")) {
    runner_dosub_pair2_force(&r, c0, c1, 0, 0);
  } else if (!strcmp(call, "runner_do_end_hydro_force")) {
    runner_do_end_hydro_force(&r, c0, 0);
  } else if (!strcmp(call, "runner_do_hydro_sort")) {
    runner_do_hydro_sort(&r, c0, 0x1FFF, 0, 0, 0, 0);
  } else if (!strcmp(call, "gb300_start_step")) {
    gb300_start_step(&e);
  } else if (!strcmp(call, "gb300_fetch")) {
    gb300_fetch(&e);
  } else if (!strcmp(call, "deep_cell")) {
    struct cell child;
    memset(&child, 0, sizeof(child));
    child.top = c0;
    runner_dosub_self1_density(&r, &child, 0, 0);
  } else {
    return 2;
  }
  printf("returned\n");
  return 0;
}
