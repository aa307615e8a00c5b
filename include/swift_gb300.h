/* swift_gb300.h -- C ABI of the GB300 SPH neighbour-interaction library.
 *
 * Plain C types only (pointers, sizes, integers).  Every function returns 0
 * on success or a negative SPHGPU_E* code; sphgpu_last_error() gives the
 * message of the last failure on the calling thread.  Nothing here aborts
 * the process: where the reference's runner functions call error() (e.g.
 * runner_ghost.c:1592 when h does not converge) this library returns
 * SPHGPU_ENOCONV and leaves the decision to the caller.
 *
 * Particle arrays are passed in the caller's order ("input order"); the
 * library keeps its own cell-sorted copy in HBM and maps results back.
 * Positions are FP64 [n][3]; velocities FP32 [n][3]; mass, h, u FP32 [n];
 * time bins int8 [n].
 *
 * Reference interfaces replaced (paths relative to SWIFT's src/):
 *   sphgpu_space_create        space_init + space_rebuild (space.c:1136,
 *                              space_rebuild.c:49): grid, cell index, split
 *   sphgpu_dosub_self1_density runner_dosub_self1_density
 *                              (runner_doiact_functions_hydro.h:3037,
 *                               declared runner_doiact_hydro.h:187-195)
 *   sphgpu_dosub_pair1_density runner_dosub_pair1_density (:2933)
 *   sphgpu_do_ghost            runner_do_ghost (runner_ghost.c:1113)
 *   sphgpu_dosub_self2_force   runner_dosub_self2_force (:3203)
 *   sphgpu_dosub_pair2_force   runner_dosub_pair2_force (:3102)
 *   sphgpu_do_end_hydro_force  runner_do_end_hydro_force (runner_others.c:815)
 *   sphgpu_step                one engine_init_particles-style pass
 *                              (engine.c:2245): all density tasks, the
 *                              ghosts and all force tasks, batched into one
 *                              persistent launch per loop and one CUDA graph.
 */
#ifndef SWIFT_GB300_H
#define SWIFT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPHGPU_ABI_VERSION 2

#define SPHGPU_OK 0
#define SPHGPU_EINVAL -1   /* bad argument */
#define SPHGPU_ECUDA -2    /* CUDA runtime error (message has details) */
#define SPHGPU_ENOMEM -3   /* device or host allocation failed */
#define SPHGPU_ENOCONV -4  /* smoothing lengths did not converge */
#define SPHGPU_ESTATE -5   /* call out of order (e.g. no step run yet) */
#define SPHGPU_ENODEV -6   /* no CUDA device */
#define SPHGPU_EREBUILD -7 /* particles moved too far for the cell tree: rebuild */

/* Stages of a step (bit mask). */
#define SPHGPU_STAGE_DENSITY 1
#define SPHGPU_STAGE_GHOST 2
#define SPHGPU_STAGE_FORCE 4
#define SPHGPU_STAGE_ALL 7

typedef struct sphgpu_space sphgpu_space;

/* Run-time parameters; names follow the reference's parameter file
 * (SPH:resolution_eta, SPH:h_tolerance, SPH:h_max, SPH:h_min_ratio,
 * SPH:max_ghost_iterations, SPH:viscosity_alpha,
 * Scheduler:max_top_level_cells; hydro_properties.c:58-110). */
typedef struct {
  double dim[3];
  int32_t periodic;
  float eta;
  float h_tolerance;
  float h_max;
  float h_min;
  float alpha;
  int32_t max_iter;
  int32_t max_active_bin;
  int32_t max_top_level_cells;
} sphgpu_params;

/* Launch configuration of the gather kernels (what the autotuner picks). */
typedef struct {
  int32_t threads_per_particle; /* lanes per updated particle: 1 (one warp
                                   serves a group of up to 32 particles)
                                   or 2 (a group of up to 16, the two
                                   lanes split each j-block's candidates;
                                   the list-recording re-run keeps 1) */
  int32_t jtile;                /* partner particles per culled j-block:
                                   8, 16 or 32 */
  int32_t rerun_lists;          /* 1: the ghost's first density re-run
                                   records each particle's neighbour list
                                   and the later re-runs compute from it
                                   (when the lists fit in a quarter of the
                                   free HBM); 0: every re-run gathers */
  int32_t block_warps;          /* tile shape: 8 warps x 3 blocks per SM,
                                   or 4 warps x 6 blocks per SM */
  int32_t bulk_stage;           /* 1: each culled j-block (a contiguous run
                                   of the store) is fetched into shared
                                   memory by one bulk copy (the TMA
                                   engine's cp.async.bulk) instead of one
                                   load per lane; 0: loads (8-warp tile
                                   shape, one or two lanes per particle;
                                   other shapes always load) */
  float row_widen;              /* the first density pass records each
                                   particle's candidates within
                                   sqrt(row_widen) x its search radius
                                   (capped by its depth_h cell's width)
                                   for the ghost's re-runs and the force;
                                   0: the default 1.21; else 1 to 4 */
  int32_t row_cap;              /* items per particle row (a particle with
                                   more candidates is gathered instead);
                                   0: the default 160; else a multiple of
                                   16 in [64, 512]; the rows are kept only
                                   while they fit in a quarter of the free
                                   HBM */
  int32_t tc_filter;            /* 1: the density gathers (one or two lanes
                                   per particle, loads) test each surviving
                                   j-block's candidates on the tensor cores
                                   first (TF32 mma.sync of r^2 with a
                                   margin that drops no candidate the FP32
                                   test keeps); the candidates that pass are
                                   classified exactly as without it (same
                                   counts); 0: every candidate gets the
                                   FP32 test */
} sphgpu_tuning;

int sphgpu_abi_version(void);
const char *sphgpu_last_error(void);
void sphgpu_default_params(sphgpu_params *p);

/* Largest space: the gathers pack a partner's store index in 27 bits. */
#define SPHGPU_MAX_PARTICLES ((1 << 27) - 1)

/* Build the cell tree of a box (host) and keep its particles for the GPU.
 * Replaces space_init + space_rebuild.  No device is touched until the
 * first GPU call, so tree queries work without a GPU. */
int sphgpu_space_create(const sphgpu_params *prm, int64_t n, const double *x,
                        const float *v, const float *m, const float *h,
                        const float *u, const int8_t *time_bin,
                        sphgpu_space **out);
int sphgpu_space_destroy(sphgpu_space *s);

/* info[0..7] = n, cdim[0..2], cells, leaves, top-level tasks, gather entries */
int sphgpu_space_info(const sphgpu_space *s, int64_t info[8]);

/* Cell assignment per particle (input order), int32 [n][6]: first index of
 * the particle's leaf, leaf count, leaf depth, depth_h, position in the
 * cell-sorted order, top-level cell id (cell_getid order). */
int sphgpu_space_cells(const sphgpu_space *s, int32_t *out);

/* Leaf geometry, double [leaves][6] = loc[3], width[3], plus int32
 * [leaves][3] = first, count, depth (may be NULL). */
int sphgpu_space_leaves(const sphgpu_space *s, double *geom, int32_t *ints);

/* The cell tree: int32 [ncells][5] = first particle (cell-sorted order),
 * count, depth, parent cell (-1 at the top), top-level cell; records may be
 * NULL to read *ncells only.  Cell ids index sphgpu_cell_sort. */
int sphgpu_space_tree(const sphgpu_space *s, int32_t *ncells, int32_t *records);

/* Replaces runner_do_hydro_sort (runner_sort.c:203) for the whole tree at
 * once: for every non-empty cell and every axis j set in flags (13 axes,
 * sort_part.h:42-57) the keys d = (float)(x . axis_j) of the cell's
 * particles, ascending with their indices in the cell, plus a sentinel
 * {FLT_MAX, 0} -- bit-identical to the reference's arrays (its leaf
 * quicksort and 8-way merge, ties included).  Built on the device. */
int sphgpu_hydro_sort(sphgpu_space *s, int32_t flags, void *stream);
/* Copies sort array `axis` of one cell (count + 1 entries) to the host, the
 * array cell_get_hydro_sorts (cell.h:1471) returns in the reference. */
int sphgpu_cell_sort(sphgpu_space *s, int32_t cell, int32_t axis, float *d,
                     int32_t *idx);

/* Change the active set (particles with time_bin <= max_active_bin). */
int sphgpu_set_active(sphgpu_space *s, int32_t max_active_bin);

int sphgpu_set_tuning(sphgpu_space *s, const sphgpu_tuning *t);
int sphgpu_get_tuning(const sphgpu_space *s, sphgpu_tuning *t);

/* Autotuner: times the batched step of this space (CUDA events, `reps`
 * steps per candidate after one warm-up) for every candidate configuration
 * (j-block depth x lanes per particle x tile shape), keeps the fastest and
 * returns it in *best; ms[k] receives the mean step time of candidate k (up
 * to 24 candidates, order: jtile 32/16/8 x threads_per_particle 1/2 x
 * block_warps 8/4, then -- when the rows are on -- the fastest of those with
 * one lane per particle and the fastest with two, each with row_widen 1.32,
 * 1.44, 1.56, 1.69), *ncand their number. */
int sphgpu_autotune(sphgpu_space *s, int32_t reps, sphgpu_tuning *best,
                    float ms[24], int32_t *ncand);

/* Batched form: density -> ghost -> force over the whole box, one
 * persistent launch per loop, captured as one CUDA graph on the first call
 * (stages == SPHGPU_STAGE_ALL).  Inputs and outputs stay in HBM.  `stream`
 * is a cudaStream_t (NULL: the library's own stream).  Returns
 * SPHGPU_ENOCONV if some h did not converge in max_iter rounds. */
int sphgpu_step(sphgpu_space *s, int32_t stages, void *stream);

/* Steps of the batched form since the last reset: out[0] steps run as one
 * CUDA graph, out[1] of them that ran a second time outside it (host
 * planning: the force lists planned before the step from each active
 * particle's last converged h, whose recursion decisions the post-ghost h
 * changed, were re-planned; device planning: a plan outgrew its buffers,
 * which grew), out[2] that needed ghost rounds beyond the graph's, out[3]
 * graph captures. */
int sphgpu_step_stats(sphgpu_space *s, int64_t out[4], int32_t reset);

/* Host time (ms, summed since the last reset) of the planning that steps
 * need: [0] sphgpu_set_active's cell refresh and list building, [1] its
 * uploads, [2] the force lists planned inside steps after a ghost.  With
 * device planning [0] is the time sphgpu_set_active takes and [1], [2]
 * stay 0. */
int sphgpu_host_times(sphgpu_space *s, double ms[3], int32_t reset);

/* Device planning.  After sphgpu_set_active with a max_active_bin that
 * leaves some particles inactive, on a space resident on the device (one
 * GPU call has run on it), every batched step plans its own gather lists
 * inside its CUDA graph: the flags from the time bins, each cell's h_max,
 * h_max_active and activity from its particles, the density and re-run
 * lists of the reference's recursions for every active leaf, and after the
 * ghost the force lists from the post-ghost h_max -- the lists the host
 * planner gives for the same state.  Activations with every particle
 * active keep the host's plans (they stay valid from step to step).  The
 * host planner takes over again, with the device's h, for the plain form,
 * the per-task entry points and sphgpu_force_from_state.  on = 0 turns
 * device planning off for the space (the default is on). */
int sphgpu_set_device_planning(sphgpu_space *s, int32_t on);

/* Moves the space's particles to new positions x (3 per particle) with new
 * smoothing lengths h, input order, host or device memory, without a
 * rebuild: every particle stays in the cell the rebuild gave it, as the
 * reference's drift does between rebuilds (cell_drift.c:330-382).  Each
 * cell's dx_max_part (the largest motion of its particles since the
 * rebuild) and h_max are measured; if cell_need_rebuild_for_hydro_pair
 * (cell.h:1237: kernel_gamma max(h_max_i, h_max_j) + dx_max_part_i +
 * dx_max_part_j > dmin) holds for any pair of neighbouring top-level cells
 * the call returns SPHGPU_EREBUILD and changes nothing (create a new space
 * from the new positions).  Otherwise the positions, the particles' h (the
 * h the next step's active particles start from, and the h of the inactive
 * ones), their depth_h and the j-blocks' boxes are replaced, and the
 * recursions of later steps add dx_max_part to their cut-offs (cell.h:
 * 934-1010); later steps plan on the device (whatever their activity).
 * sphgpu_step_host calls this when its x or h differ from the space's. */
int sphgpu_space_drift(sphgpu_space *s, const double *x, const float *h, void *stream);

/* Device time (ms, summed since the last reset) of the planning inside
 * device-planned steps (cell state and lists, before the density loop and
 * after the ghost), and the number of those steps. */
int sphgpu_plan_times(sphgpu_space *s, double *ms, int64_t *steps, int32_t reset);

/* Self-check of device planning: after a device-planned step, rebuilds the
 * host planner's density, re-run and force lists from the device's state
 * (the step's starting h, its activity and its post-ghost h) and compares
 * them with the lists the step planned on the device, leaf by leaf.
 * out[0..2]: (j-block, entry) pairs that differ in the density, re-run and
 * force lists (a leaf whose pair count differs counts all its pairs);
 * out[3..5]: the pairs of each device plan.  SPHGPU_ESTATE when the space
 * is not device-planned or no step has run since the activation. */
int sphgpu_check_device_plans(sphgpu_space *s, int64_t out[6]);

/* Per-loop device time of the batched steps run so far (CUDA events on the
 * step's stream): ms_sum[0] density first pass, [1] ghost rounds (Newton
 * updates + density re-runs), [2] force loop; *steps = steps timed. */
int sphgpu_phase_times(sphgpu_space *s, double ms_sum[3], int64_t *steps,
                       int32_t reset);

/* One instrumented (uncaptured) step that counts neighbour interactions:
 * hits[0] density first pass, [1] density re-runs of the ghost, [2] force,
 * [3] density neighbours at the converged h (the last pass of every active
 * particle). */
int sphgpu_count_hits(sphgpu_space *s, int64_t hits[4]);

/* The first density pass of a resident space with no device allocation:
 * for callers that cannot call cudaMalloc when they run it -- a host that
 * hands all device memory to its own pool and accounts for every byte, or a
 * latency-bound serving loop that must not stall on the allocator.  No
 * counterpart in the reference.
 * The space must already be resident on the device (any earlier GPU call on
 * it allocates and uploads); the first call on a device also looks up the
 * library's static scratch array, so make it before any stream capture.
 * Scratch (work-queue counter and active-particle list) lives in one static
 * device array sized for SPHGPU_NOALLOC_MAX_PARTICLES particles, held by
 * every GPU that loads the library until the process exits; larger spaces
 * get SPHGPU_EINVAL.  Every call reuses that array and resets its counters,
 * so calls that overlap on the GPU (other streams, other threads) race.
 * Outputs, in the caller's particle order, go to device buffers the caller
 * provides: d_fields float [n][8] = rho, rho_dh, wcount, wcount_dh, div_v,
 * rot_v[3] (the raw sums of sphgpu_download columns 0-7) and d_ngb int32 [n]
 * neighbour counts.  Asynchronous on `stream` (NULL: the space's stream).
 * The pass reads the space's device state: a caller that passes a stream
 * other than the space's own must order it after the work it queued on the
 * space's stream (for example sphgpu_step_host_async uploads), e.g. with an
 * event recorded there and cudaStreamWaitEvent on `stream`. */
#define SPHGPU_NOALLOC_MAX_PARTICLES (1 << 20)
int sphgpu_density_noalloc(sphgpu_space *s, float *d_fields, int32_t *d_ngb,
                           void *stream);

/* New velocities, masses and internal energies of every particle (input
 * order: v float [n][3], m, u float [n]), e.g. after the kicks of a step, for
 * the loops that follow.  Positions and h stay the space's (sphgpu_space_drift
 * moves them).  Replaces the copy of these
 * struct part fields that the reference's loops read in place
 * (hydro/Minimal/hydro_part.h:103-240).  Synchronous; on a machine without
 * a GPU the host copies are updated and SPHGPU_ENODEV is returned. */
int sphgpu_space_update(sphgpu_space *s, const float *v, const float *m, const float *u,
                        void *stream);

/* Same pass through host buffers: copies x, v, m, h, u (input order) from
 * host memory, runs the step, copies the results back.  `fields` receives
 * float [n][24] in the column layout of sphgpu_download; NULL skips it.
 * v, m and u may change from step to step; x and h are compared with the
 * space's on the device and, where they differ, the particles are moved
 * without a rebuild first (sphgpu_space_drift): SPHGPU_EREBUILD, with no step
 * run, when they moved too far for the cell tree. */
int sphgpu_step_host(sphgpu_space *s, const double *x, const float *v,
                     const float *m, const float *h, const float *u,
                     float *fields, void *stream);

/* Pipelined form of sphgpu_step_host for a stream of steps: enqueues the
 * copies in (on an upload stream), the step and the copies out (on a
 * download stream) and returns; a step's inputs go up while the previous
 * step computes, and its results come down while the next one does.  At
 * most two steps are in flight: a call first waits for the step issued two
 * calls earlier.  A step's `fields` (required) and input buffers must stay
 * valid, and its results are complete, once a later call has waited for it
 * or sphgpu_step_host_wait returns.  x and h must be the space's (move
 * particles with sphgpu_space_drift or sphgpu_step_host first): a step whose
 * x or h differ runs on the space's own and SPHGPU_EINVAL, like
 * non-convergence, is reported by the call that waits for that step.  Pinned host buffers make
 * the copies asynchronous. */
int sphgpu_step_host_async(sphgpu_space *s, const double *x, const float *v,
                           const float *m, const float *h, const float *u,
                           float *fields);
/* Wait for every step issued by sphgpu_step_host_async. */
int sphgpu_step_host_wait(sphgpu_space *s);

/* Plain form: the same pass issued task by task as the reference's runner
 * would (one launch per self/pair task and loop, one ghost per top cell). */
int sphgpu_step_plain(sphgpu_space *s, void *stream);

/* Results in input order, into host or device memory (device destinations
 * are written in place by a kernel, with no allocation).  fields float
 * [n][24]: 0-7 raw density sums of the last density pass (rho, rho_dh,
 * wcount, wcount_dh, div_v, rot_v[3]), 8-14 after the ghost (h, rho, f,
 * pressure, soundspeed, balsara, v_sig seed), 15-20 after the force
 * (a_hydro[3], u_dt, h_dt, v_sig), 21 the smallest time bin among the force
 * neighbours (limiter_data.min_ngb_time_bin, num_time_bins + 1 when none),
 * 22-23 zero.  ints int32 [n][4]: density neighbours (first pass), density
 * neighbours (last pass), force neighbours, ghost rounds.  Either may be
 * NULL. */
int sphgpu_download(sphgpu_space *s, float *fields, int32_t *ints);

/* A caller's particle state for the next steps (input order, host or device
 * memory; a NULL array keeps the space's): velocities v[3], masses,
 * internal energies u, the force inputs the inactive particles lend their
 * active neighbours (rho, pressure, soundspeed as the reference's drift
 * predicts them, hydro_predict_extra -- the three go together -- and the
 * grad-h term f and the Balsara switch of their last ghost), and time bins
 * (the activity of later sphgpu_set_active calls).  Unlike
 * sphgpu_space_update it does not check the values on the host. */
int sphgpu_space_set_state(sphgpu_space *s, const float *v, const float *m, const float *u,
                           const float *rho, const float *f, const float *pressure,
                           const float *soundspeed, const float *balsara,
                           const int8_t *time_bin, void *stream);

/* Force loop only, from caller-provided post-ghost state (input order):
 * h, rho, f, pressure, soundspeed, balsara.  For parity checks of the force
 * loop against the reference's own post-ghost values. */
int sphgpu_force_from_state(sphgpu_space *s, const float *h, const float *rho,
                            const float *f, const float *pressure,
                            const float *soundspeed, const float *balsara,
                            void *stream);

/* After a force pass: each particle's smallest time bin > 0 among its force
 * neighbours (limiter_data.min_ngb_time_bin, set by runner_iact_timebin,
 * timestep_limiter_iact.h:34-72; num_time_bins + 1 = 57 when it has none),
 * input order.  Valid for the active particles of the last force pass. */
int sphgpu_download_min_ngb_bin(sphgpu_space *s, int8_t *out);

/* Drop-in per-task entry points (plain form).  `cell` / `ci`, `cj` are
 * top-level cell ids (cell_getid order).  Density and force accumulate into
 * the particle sums like the reference's loops; call sphgpu_begin_loops()
 * first to zero them. */
int sphgpu_begin_loops(sphgpu_space *s, void *stream);
int sphgpu_dosub_self1_density(sphgpu_space *s, int32_t cell, void *stream);
int sphgpu_dosub_pair1_density(sphgpu_space *s, int32_t ci, int32_t cj,
                               void *stream);
int sphgpu_do_ghost(sphgpu_space *s, int32_t cell, void *stream);
int sphgpu_dosub_self2_force(sphgpu_space *s, int32_t cell, void *stream);
int sphgpu_dosub_pair2_force(sphgpu_space *s, int32_t ci, int32_t cj,
                             void *stream);
int sphgpu_do_end_hydro_force(sphgpu_space *s, void *stream);

/* ------------------------------------------------------------------------
 * Serving: many independent boxes resident on the device, stepped together
 * by the same persistent launches (continuous batching).  No counterpart in
 * the reference, whose engine runs one simulation per process.
 *
 * sphgpu_server_create sizes one device arena for max_particles particles
 * (0: a share of the free HBM) and starts planner_threads host workers
 * (0: one per core, at most 16).  prm gives the physics (eta, tolerances,
 * alpha, max_iter) every box shares.
 * sphgpu_server_submit copies a box (its own dim / periodic /
 * max_top_level_cells from *box, every particle active) and queues it for
 * planning; it runs nsteps density -> ghost -> force steps once admitted.
 * sphgpu_server_pump admits the planned boxes that fit (first come, first
 * served; admission by free arena ranges), then advances every resident box
 * by one step and retires the finished ones; when nothing is resident it
 * first waits up to wait_s for a planner.  *resident: boxes on the device.
 * sphgpu_server_poll lists finished request ids (each once);
 * sphgpu_server_fetch copies one finished box out -- fields as
 * sphgpu_download (24 per particle, input order), ints 4 per particle
 * (density neighbours first / last pass, force neighbours, ghost
 * iterations), times = submit, admission, completion (seconds, steady
 * clock) -- and forgets it.
 * stats: [0] resident boxes, [1] arena particles in use, [2] arena particle
 * capacity, [3] boxes waiting or being planned, [4] pumps, [5] boxes
 * retired, [6] arena bytes, [7] free HBM when the server started. */
typedef struct sphgpu_server sphgpu_server;
int sphgpu_server_create(const sphgpu_params *prm, int64_t max_particles,
                         int32_t planner_threads, sphgpu_server **out);
int sphgpu_server_destroy(sphgpu_server *s);
int sphgpu_server_submit(sphgpu_server *s, int64_t id, const sphgpu_params *box,
                         int64_t n, const double *x, const float *v,
                         const float *m, const float *h, const float *u,
                         int32_t nsteps);
int sphgpu_server_pump(sphgpu_server *s, double wait_s, int32_t *resident);
int sphgpu_server_poll(sphgpu_server *s, int64_t *ids, int32_t max_ids,
                       int32_t *count);
int sphgpu_server_fetch(sphgpu_server *s, int64_t id, float *fields,
                        int32_t *ints, double times[3]);
int sphgpu_server_stats(sphgpu_server *s, int64_t stats[8]);
/* Where the pumps spent their time (seconds): [0] GPU (density, ghost
 * rounds, force launches), [1] host planning of new boxes' force lists,
 * [2] admissions (uploads), [3] retirements (read-back). */
int sphgpu_server_times(sphgpu_server *s, double times[4]);

/* ---- Time integration (replaces runner_do_kick1 / runner_do_kick2 /
 * runner_do_timestep, runner_time_integration.c:87 / :360 / :639, and the
 * particle drift of cell_drift_part, cell_drift.c:159, for gas particles
 * without cosmology, gravity, cooling or entropy floor).  The state lives
 * in DEVICE memory, in the caller's order; every pointer of
 * sphgpu_integ_state is a device pointer.  Kernels are enqueued on `stream`
 * (a cudaStream_t; NULL: the legacy default stream). */
typedef struct {
  double time_base;        /* physical time of one integer tick */
  double dt_min, dt_max;   /* engine dt_min / dt_max */
  float CFL;               /* hydro_props->CFL_condition */
  float log_max_h_change;  /* hydro_props->log_max_h_change */
  float h_min, h_max;
  float minimal_u;         /* hydro_props->minimal_internal_energy */
  double dim[3];           /* box, for the periodic wrap of a rebuild */
  int32_t periodic;
} sphgpu_integ_params;

typedef struct {
  double *x;               /* [3n] positions */
  float *v_full;           /* [3n] xpart.v_full */
  float *v;                /* [3n] predicted velocities (part.v) */
  float *a;                /* [3n] a_hydro */
  float *u_full;           /* [n] xpart.u_full */
  float *u, *u_dt;         /* [n] predicted internal energy, du/dt */
  float *h, *h_dt;         /* [n] */
  float *rho, *P, *c;      /* [n] density, pressure, sound speed */
  float *v_sig;            /* [n] */
  int8_t *time_bin;        /* [n] */
  const int8_t *min_ngb_bin; /* [n] from the force pass (timestep only) */
} sphgpu_integ_state;

/* which = 1: the first half kick of the particles starting their step at
 * ti_current (time_bin <= max_active_bin); which = 2: the second half kick
 * of the particles ending it there, then hydro_reset_predicted_values. */
int sphgpu_integ_kick(const sphgpu_integ_params *ip, const sphgpu_integ_state *st,
                      int64_t n, int32_t which, int64_t ti_current,
                      int32_t max_active_bin, void *stream);
/* Drift every particle from ti_old to ti_current (drift_part +
 * hydro_predict_extra + the h clamp); wrap != 0 also applies the periodic
 * box_wrap of the rebuild that follows (space_cell_index.c:113-123). */
int sphgpu_integ_drift(const sphgpu_integ_params *ip, const sphgpu_integ_state *st,
                       int64_t n, int64_t ti_old, int64_t ti_current, int32_t wrap,
                       void *stream);
/* New time bins of the active particles; *ti_end_min = the next
 * synchronisation point over all particles, *n_too_small = particles whose
 * step fell below dt_min (the reference aborts there).  Synchronises the
 * stream. */
int sphgpu_integ_timestep(const sphgpu_integ_params *ip, const sphgpu_integ_state *st,
                          int64_t n, int64_t ti_current, int32_t max_active_bin,
                          int64_t *ti_end_min, int64_t *n_too_small, void *stream);
/* get_max_active_bin (timeline.h:146) */
int sphgpu_integ_max_active_bin(int64_t ti);

/* ---- Device-resident cell assignment ------------------------------------
 * Replaces the cell assignment of space_rebuild (space_rebuild.c:49):
 * space_regrid's top-level grid (space_regrid.c:46-121), the top cell of
 * every particle (space_parts_get_cell_index, space_cell_index.c:64-150),
 * the octree split of cells of more than 400 particles (space_split.c:
 * 196-300, cell_split.c:55-175) and depth_h (cell_set_part_h_depth,
 * cell.h:1787), computed on the device from positions x [3n] (FP64) and
 * smoothing lengths h [n] already in device memory (the caller's order;
 * periodic boxes are wrapped by one period as the rebuild does, x itself is
 * not changed).  Outputs:
 *   order [n]   device: the caller's index of each particle in cell order
 *               (every cell of every level one contiguous range, ranges as
 *               the reference's; inside a leaf, particles follow their
 *               octant path, then the caller's order)
 *   depth_h [n] device, cell order
 *   cdim [3], *ncells, and cells [ncells][5] (host, may be NULL) in the
 *               format and numbering of sphgpu_space_tree: first, count,
 *               depth, parent, top.  With max_cells < *ncells the records
 *               are not written and SPHGPU_EINVAL is returned.
 * The call synchronises the stream (it reads back the grid and the tree).
 * Its device scratch (about 21 bytes per particle) and page-locked staging
 * stay allocated for the calling host thread's next call, until the thread
 * ends. */
int sphgpu_cell_assign(const sphgpu_params *prm, const double *x, const float *h,
                       int64_t n, int32_t *order, int8_t *depth_h, int32_t cdim[3],
                       int32_t *ncells, int32_t *cells, int32_t max_cells, void *stream);
/* Host-clock phases (ms) of the calling thread's last sphgpu_cell_assign:
 * [0] h scan and grid, [1] keys and radix sort, [2] tree levels, [3] cell
 * numbering and records, [4] depth_h; [5] the number of kernels it
 * launched. */
int sphgpu_cell_assign_times(double ms[6]);

/* sphgpu_space_create with the cell assignment already made by
 * sphgpu_cell_assign (its order, copied to the host, and its cell records):
 * the space adopts that tree instead of building one with the host's bucket
 * and octant permutations (space_rebuild without its cell assignment).  The
 * tree is checked for consistency (a permutation, children inside their
 * parents, every cell of more than 400 particles split). */
int sphgpu_space_create_assigned(const sphgpu_params *prm, int64_t n, const double *x,
                                 const float *v, const float *m, const float *h,
                                 const float *u, const int8_t *time_bin,
                                 const int32_t *order, const int32_t *cells, int32_t ncells,
                                 sphgpu_space **out);

#ifdef __cplusplus
}
#endif
#endif /* SWIFT_GB300_H */
