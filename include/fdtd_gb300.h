/*
 * fdtd_gb300.h -- C ABI of the GB300 (sm_103a) FDTD step loop.
 *
 * Drop-in replacement for the operations behind the reference's MEX entry
 * point simFDTD (enricoballini/maxwell_solver, src/simFDTD.cu:19-187).  Each
 * function below replaces one op string of that dispatcher; the comment on
 * each cites the dispatcher branch and the `simulation` method it calls
 * (src/simulation.h).  Argument meaning, units, array layouts (x fastest,
 * i + j*Imax + k*Imax*Jmax) and the order in which the ops may be called are
 * the reference's.  A MATLAB binding is maxwell_solver_gb300/csrc/mex/
 * simFDTD_mex.c; a Python binding is maxwell_solver_gb300.simfdtd.
 *
 * Conventions
 *  - Every function returns an fdtd_status; FDTD_OK is 0.  On failure,
 *    fdtd_last_error() gives a message (thread-local).
 *  - Handles are opaque 64-bit ids checked against a registry: a deleted or
 *    forged handle yields FDTD_ERR_INVALID_HANDLE instead of a crash.
 *  - All pointers are host pointers; lengths are element counts.  Work is
 *    queued on the handle's own CUDA stream; only the output functions wait.
 *  - Fields, coefficients and CPML state stay in device memory (HBM) for
 *    the lifetime of the handle.
 */
#ifndef FDTD_GB300_H
#define FDTD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef uint64_t fdtd_handle;

typedef enum {
  FDTD_OK = 0,
  FDTD_ERR_INVALID_HANDLE = 1,   /* unknown / deleted handle */
  FDTD_ERR_INVALID_ARG = 2,      /* bad size, flag, index, null pointer */
  FDTD_ERR_STATE = 3,            /* op called before its prerequisite */
  FDTD_ERR_ALREADY_INITIALIZED = 4, /* SetConst twice (simFDTD:AlreadyInitialized) */
  FDTD_ERR_CUDA = 5,             /* CUDA runtime / launch error */
  FDTD_ERR_OOM = 6,              /* device or pinned allocation failed */
  FDTD_ERR_UNSUPPORTED = 7,      /* outside the supported envelope */
  FDTD_ERR_CANCELLED = 8         /* a served request cancelled before it finished */
} fdtd_status;

/* Extension (no reference counterpart): runtime CPML and TF/SF settings.
 * fdtd_default_params() returns the reference's compile-time constants
 * (src/simulation.h:17, :86-90, :102): pml 10, poly_m 3, alpha_m 1,
 * alpha_max 0.08, kappa_max 1, sigma_max = 0.8 (m+1) / (eta dx), inset 15.
 * When r0 > 0, sigma_max = -(m+1) ln(r0) / (2 eta pml dx) instead. */
typedef struct {
  int32_t pml;          /* CPML thickness in cells, 2..32 */
  int32_t tfsf_width;   /* TF/SF box inset from the outer boundary */
  double poly_m, alpha_m, alpha_max, kappa_max, sig_factor, r0;
} fdtd_params;

fdtd_params fdtd_default_params(void);
/* Must precede fdtd_set_const. */
int fdtd_set_params(fdtd_handle h, const fdtd_params *p);

/* 'CreateSimulation' -- src/simFDTD.cu:30-38, simulation::simulation()
 * src/simulation.h:71-77.  Creates a handle with its own CUDA stream. */
int fdtd_create(fdtd_handle *out);

/* 'DeleteSimulation' -- src/simFDTD.cu:49-52, ~simulation()
 * src/simulation.h:1153-1269. */
int fdtd_destroy(fdtd_handle h);

/* 'SetConst' -- src/simFDTD.cu:103-110, setConst src/simulation.h:79-131.
 * freqRes = [fctr, delX, delT]; timeDim = [T, Imax, Jmax, Kmax, numAnt].
 * A second call fails with FDTD_ERR_ALREADY_INITIALIZED. */
int fdtd_set_const(fdtd_handle h, const float freqRes[3], const int32_t timeDim[5]);

/* 'SetSource' with 3 arguments -- src/simFDTD.cu:111-125, setSource
 * src/simulation.h:1068-1082.  n must be >= T; the first T values are used.
 * A second call is ignored (the reference prints and returns). */
int fdtd_set_source(fdtd_handle h, const float *src, size_t n);

/* 'SetSource' with a 4th argument -- updateSource src/simulation.h:1084-1095. */
int fdtd_update_source(fdtd_handle h, const float *src, size_t n);

/* Oblique plane-wave incidence, TF/SF mode 5 (no reference counterpart:
 * the reference has the axis-aligned modes 1-4 of src/simulation.h:330-369).
 * Propagation along (sin t cos p, sin t sin p, cos t), E along
 * cos(psi) theta_hat + sin(psi) phi_hat (radians).  Call after SetConst and
 * before Init1D; Init1D then also runs the 1D line along that direction
 * (speed matched to the 3D grid's numerical phase velocity there at the
 * centre frequency fctr), and the PlaneWave ops / fdtd_step_n accept mode 5.
 * Needs the TF/SF box at least one cell inside the CPML (tfsf_width >=
 * pml + 1) and no current source on its faces. */
int fdtd_set_incidence(fdtd_handle h, double theta, double phi, double psi);

/* 'UpdateMaterial' -- src/simFDTD.cu:150-157, updateMaterial
 * src/simulation.h:288-328.  flag 1,2,3 = sigma_x,y,z; 4,5,6 = eps_x,y,z;
 * other flags are ignored.  Takes effect at ReadySimulation / UpdateCuda. */
int fdtd_update_material(fdtd_handle h, int32_t flag, const float *values, size_t n);

/* Media given as shapes, rasterised on the device at ReadySimulation (and
 * UpdateCuda) into the same six per-cell arrays UpdateMaterial takes (no
 * reference counterpart: the reference's scripts build those arrays in
 * MATLAB, GICsimulation.m:59-94).  Every cell starts at (bg_eps_r,
 * bg_sigma); shapes apply in order, later ones overwriting, with the same
 * eps_r and sigma on all three components.  Indices cover the whole grid
 * (CPML included), cell (i,j,k) centred at (i+0.5, j+0.5, k+0.5). */
#define FDTD_MAX_SHAPES 4096
enum { FDTD_SHAPE_SPHERE = 1, FDTD_SHAPE_LAYER_Z = 2, FDTD_SHAPE_BOX = 3 };
typedef struct {
  int32_t kind;
  float eps_r, sigma; /* inside the shape: relative permittivity, S/m */
  int32_t reserved;
  /* sphere: centre x, y, z and radius r (cells); inside when
   *   ((i+0.5-x)^2 + (j+0.5-y)^2) + (k+0.5-z)^2 <= r*r in double arithmetic
   * layer: g[0] <= k < g[1]
   * box: g[0] <= i < g[1], g[2] <= j < g[3], g[4] <= k < g[5] */
  double g[6];
} fdtd_shape;
int fdtd_set_shapes(fdtd_handle h, float bg_eps_r, float bg_sigma, const fdtd_shape *shapes,
                    int32_t n);

/* 'CreateMu' -- src/simFDTD.cu:133-141, createMu src/simulation.h:28-68.
 * As in the reference, a call after ReadySimulation computes the
 * coefficients but leaves the H update unchanged; a call before it is
 * rejected with FDTD_ERR_STATE (the reference reads unset state there). */
int fdtd_create_mu(fdtd_handle h, const float *mu_x, const float *mu_y,
                   const float *mu_z, size_t n);

/* 'SetMagnetic' -- per-cell magnetic media, what createMu
 * (src/simulation.h:28-68) sets out to do: relative permeability mu_r and
 * magnetic conductivity sigma_m (ohm/m) of each H component at its Yee
 * position, Imax*Jmax*Kmax values each (x fastest); sm_* may
 * all be NULL (lossless).  After ReadySimulation; applies from the next H
 * update to the curl, the CPML corrections and the TF/SF corrections:
 * q = sigma_m delT / (2 mu0 mu_r), Chh = (1 - q) / (1 + q),
 * Che = delT / (mu0 mu_r) / (1 + q) / delX, in double, rounded once
 * (mu_r = 1, sigma_m = 0 give the scalar coefficients exactly).  Handles
 * with per-cell H coefficients cannot join a batch. */
int fdtd_set_magnetic(fdtd_handle h, const float *mu_x, const float *mu_y,
                      const float *mu_z, const float *sm_x, const float *sm_y,
                      const float *sm_z, size_t n);

/* 'SetAntennaLocations' -- src/simFDTD.cu:126-132, setAntennaLocations
 * src/simulation.h:1047-1067.  loc is numAnt x 3 int32, column-major
 * (x column, then y, then z), offsets inside the CPML (pml is added).
 * Must precede ReadySimulation (src/simulation.h:954). */
int fdtd_set_antenna_locations(fdtd_handle h, const int32_t *loc, size_t n);

/* 'ReadySimulation' -- src/simFDTD.cu:81-84, readySimulation
 * src/simulation.h:640-979: CPML tables, coefficients, field allocation. */
int fdtd_ready_simulation(fdtd_handle h);

/* 'Init1D' -- src/simFDTD.cu:142-149, init1D src/simulation.h:134-254.
 * Precomputes the forward and inverse 1D incident runs for all T steps
 * (one launch).  Requires ReadySimulation. */
int fdtd_init_1d(fdtd_handle h, float rate, const float *pw_source, size_t n);

/* 'UpdateCuda' -- src/simFDTD.cu:69-72, updateCuda src/simulation.h:1097-1127. */
int fdtd_update_cuda(fdtd_handle h);

/* 'ResetFieldAll' -- src/simFDTD.cu:85-88, src/simulation.h:1128-1151.
 * Also rewinds the probe recorder to row 0. */
int fdtd_reset_field_all(fdtd_handle h);

/* 'UpdateH_All' -- src/simFDTD.cu:57-60, src/simulation.h:371-385. */
int fdtd_update_h_all(fdtd_handle h);
/* 'UpdateE_All' -- src/simFDTD.cu:53-56, src/simulation.h:386-391. */
int fdtd_update_e_all(fdtd_handle h);
/* 'UpdateH_PML' -- src/simFDTD.cu:65-68, src/simulation.h:392-403. */
int fdtd_update_h_pml(fdtd_handle h);
/* 'UpdateE_PML' -- src/simFDTD.cu:61-64, src/simulation.h:404-418. */
int fdtd_update_e_pml(fdtd_handle h);
/* 'UpdateH_PlaneWave' [step, mode] -- src/simFDTD.cu:96-102,
 * src/simulation.h:330-349.  mode 1..4; other modes do nothing. */
int fdtd_update_h_planewave(fdtd_handle h, int32_t step, int32_t mode);
/* 'UpdateE_PlaneWave' [step, mode] -- src/simFDTD.cu:89-95,
 * src/simulation.h:350-369. */
int fdtd_update_e_planewave(fdtd_handle h, int32_t step, int32_t mode);

/* 'AddCurrents' [step, mode], [i0 i1 j0 j1 k0 k1] -- src/simFDTD.cu:73-80,
 * addCurrents src/simulation.h:256-286.  mode 1,2,3 = Ex,Ey,Ez. */
int fdtd_add_currents(fdtd_handle h, int32_t step, int32_t mode, const int32_t box[6]);

/* 'OutputAnt' N -- src/simFDTD.cu:159-168, outputAnt src/simulation.h:621-638.
 * Writes min(n, numAnt*T) values: the Ez probe record, probe fastest
 * (value of probe a at step row r at a + r*numAnt).  Row r holds the fields
 * at the start of step r (before its H update), r counting UpdateH_All
 * calls since ResetFieldAll.  (The reference allocates this record but
 * never fills it.) */
int fdtd_output_ant(fdtd_handle h, float *out, size_t n);

/* 'OutputVis' N, flag -- src/simFDTD.cu:169-179, outputVis
 * src/simulation.h:572-619.  flag 1,2,3 = Ex,Ey,Ez; 0,-1,-2 = sigma_x,y,z.
 * Extension: 4,5,6 = Hx,Hy,Hz; -3,-4,-5 = eps_x,y,z.  Writes
 * min(n, Imax*Jmax*Kmax) values; other flags write nothing. */
int fdtd_output_vis(fdtd_handle h, float *out, size_t n, int32_t flag);

/* ---------------------------------------------------------------------
 * Extensions (no reference counterpart)
 * --------------------------------------------------------------------- */

/* Current-source description for fdtd_step_n (mode 0 = none). */
typedef struct {
  int32_t mode;     /* 1,2,3 = Ex,Ey,Ez */
  int32_t box[6];   /* i0 i1 j0 j1 k0 k1 */
} fdtd_current;

/* Runs steps first..first+count-1 of the reference step order
 * (highfrequency.m:85-91, plus AddCurrents as in GICsimulation.m:119-124
 * when cur != NULL and cur->mode != 0), each step as two fused half-step
 * kernels, with the loop captured in a CUDA graph.  tfsf_mode 0 skips the
 * plane-wave corrections.  Bitwise identical to issuing the per-op calls. */
int fdtd_step_n(fdtd_handle h, int32_t first, int32_t count, int32_t tfsf_mode,
                const fdtd_current *cur);

/* All six probe components: out[(r*numAnt + a)*6 + c], c = Ex,Ey,Ez,Hx,Hy,Hz. */
int fdtd_output_probes(fdtd_handle h, float *out, size_t n);

/* Waits for the handle's stream. */
int fdtd_synchronize(fdtd_handle h);

typedef struct {
  int32_t I, J, K, T, num_ant, pml, size_1d;
  int32_t i0, i1, j0, j1, k0, k1;
  int32_t coef_mode;       /* 0 per-cell arrays, 1 material-indexed */
  int32_t num_materials;   /* distinct coefficient tuples (coef_mode 1) */
  uint64_t device_bytes;   /* device memory held by the handle */
  float Chh, Che;
  int32_t zchunk_h, zchunk_e; /* z-planes per work item of the TMA half-steps
                                 (autotuned; 0 = built-in heuristic) */
  int32_t hcoef_mode;      /* H coefficients: 0 uniform, per cell
                              (fdtd_set_magnetic): 1 arrays, 2 indexed */
  int32_t fused;           /* 1: fdtd_step_n runs pairs of steps as the fused
                              H+E pass (a second field buffer is held; chosen
                              by the autotuner) */
  int32_t zchunk_f;        /* z-planes per work item of the fused pass (0:
                              default) */
  int32_t tile_h, tile_e;  /* tile geometry of the H / E curl kernels
                              (autotuned): 0 64x8, 1 32x16, 2 128x4 */
} fdtd_info;
int fdtd_get_info(fdtd_handle h, fdtd_info *out);

/* Copies one of the CPML tables (0 b_E, 1 c_E, 2 b_H, 3 c_H: 2*pml floats),
 * the x-only stretch denominators (4 den_ex, 5 den_hx: Imax floats), or
 * the material-indexed coefficient table (6: num_materials x 6 floats,
 * Cexe Ceye Ceze Cexh Ceyh Cezh per id; coef_mode 1 only). */
int fdtd_get_table(fdtd_handle h, int32_t which, float *out, size_t n);

/* Checkpoint / resume (no reference counterpart): the evolving state of a
 * ready handle -- the six fields, the CPML psi arrays, the step and probe
 * counters and the probe record -- as an opaque byte image in host memory.
 * Load it into a handle set up the same way (SetParams, SetConst, media,
 * probes, ReadySimulation, Init1D) and stepping continues exactly as the
 * saved handle would have (steps are numbered by the caller, as always).
 * A different set-up is rejected with FDTD_ERR_INVALID_ARG. */
int fdtd_checkpoint_size(fdtd_handle h, size_t *bytes);
int fdtd_checkpoint_save(fdtd_handle h, void *buf, size_t n);
int fdtd_checkpoint_load(fdtd_handle h, const void *buf, size_t n);

/* Timing on the handle's stream (CUDA events).  slot 0..15. */
int fdtd_event_record(fdtd_handle h, int32_t slot);
int fdtd_event_elapsed_ms(fdtd_handle h, int32_t slot_a, int32_t slot_b, float *ms);

/* Runs steps like fdtd_step_n but with direct launches and CUDA events
 * around every kernel; adds summed device times (ms) to ms_out:
 * [0] H half-steps (curl kernel and its face pass), [1] E half-steps (curl
 * kernel, x-slab and face passes), [2] the remaining kernels (probe
 * gather), [3] the H curl kernel alone, [4] the E curl kernel alone,
 * [5] steps whose H and E half-steps ran as one fused kernel (that kernel
 * alone; its passes are in [0] and [1]).  For measurement only. */
int fdtd_profile_steps(fdtd_handle h, int32_t first, int32_t count, int32_t tfsf_mode,
                       const fdtd_current *cur, float ms_out[6]);

/* Selects the CUDA device used by handles created afterwards on the calling
 * thread (one process per GPU: pass the local rank). */
int fdtd_set_device(int32_t device);

/* ---------------------------------------------------------------------
 * Batched execution (extension, no reference counterpart): many ready
 * simulation handles of different sizes, materials and sources advance
 * together, one H and one E launch per step for all of them (persistent
 * TMA kernels over the work items of every member).  The arithmetic per
 * cell is unchanged: each member ends bit-identical to running it alone.
 * --------------------------------------------------------------------- */
typedef uint64_t fdtd_batch;
int fdtd_batch_create(fdtd_batch *out);
int fdtd_batch_destroy(fdtd_batch b);
/* Adds handle h to run steps first..first+count-1 (TF/SF mode 0..4, current
 * source cur or NULL).  h must be ready and keeps its own state; calls on h
 * issued after the batch finishes it see the batch's results. */
int fdtd_batch_add(fdtd_batch b, fdtd_handle h, int32_t first, int32_t count,
                   int32_t tfsf_mode, const fdtd_current *cur);
/* Advances every active member by the same number of steps: the fewest
 * remaining of any active member, at most max_steps.  *active_left (may be
 * NULL) receives the number of members still running. */
int fdtd_batch_step(fdtd_batch b, int32_t max_steps, int32_t *active_left);
/* Runs every member to its last step and waits. */
int fdtd_batch_run(fdtd_batch b);
/* Drops all members. */
int fdtd_batch_clear(fdtd_batch b);
/* Steps member h has completed (-1 when h is not a member). */
int fdtd_batch_progress(fdtd_batch b, fdtd_handle h, int32_t *done);
/* Drops member h (finished or not); calls on h issued afterwards follow the
 * batch's queued work. */
int fdtd_batch_remove(fdtd_batch b, fdtd_handle h);
/* The z-planes per batched work item: measured once per batch (the first
 * step call of more than 12 steps with at least 8 active members runs 4 of
 * the members' real steps with each of 8, 16 and 32 and keeps the fastest;
 * FDTD_BATCH_ZRUN fixes it, FDTD_AUTOTUNE=0 keeps 16); 0 before that.  No
 * reference counterpart. */
int fdtd_batch_get_zrun(fdtd_batch b, int32_t *zrun);
/* Waits for the batch's queued work and reports whether every pipelined
 * half-step completed (FDTD_ERR_CUDA if a bounded wait timed out; the
 * members' fields are then not valid). */
int fdtd_batch_status(fdtd_batch b);

/* ---------------------------------------------------------------------
 * Serving (extension, no reference counterpart): a request loop in a
 * server thread.  Solve requests of different sizes are admitted in
 * arrival order while the device memory their handles will hold fits a
 * budget; each is set up on the device (its fields, psi arrays and
 * coefficients stay resident until it finishes), joins one batch that
 * advances every active solve together, and is retired when it finishes,
 * its outputs copied to the host and its memory returned -- continuous
 * batching: requests arriving while others run start at the next round.
 * A one-at-a-time mode runs the same requests as a plain FIFO queue
 * through fdtd_step_n, one solve on the device at a time.
 * --------------------------------------------------------------------- */
typedef uint64_t fdtd_server;

typedef struct {
  int32_t I, J, K;        /* grid, CPML included (SetConst TimeDim[1..3]) */
  int32_t steps;          /* time steps (TimeDim[0]) */
  float fctr, delX, delT; /* SetConst freqRes */
  fdtd_params params;     /* CPML and TF/SF settings (fdtd_default_params) */
  int32_t tfsf_mode;      /* plane-wave mode 1..4 (0: none) */
  float rate;             /* Init1D rate */
  const float *waveform;  /* [steps] plane-wave source (Init1D PW_source) */
  float bg_eps_r, bg_sigma;
  const fdtd_shape *shapes; /* media (fdtd_set_shapes) */
  int32_t n_shapes;
  int32_t n_probes;       /* probes (SetAntennaLocations, n_probes x 3) */
  const int32_t *probes;
  int32_t out_field;      /* OutputVis flag 1..6 of a field returned at the end,
                             0: none */
  double theta, phi, psi; /* tfsf_mode 5: incidence (fdtd_set_incidence) */
} fdtd_request;           /* everything is copied at submission */

typedef struct {
  uint64_t hbm_budget;    /* device bytes the admitted solves may hold at their
                             peak (fdtd_estimate_device_bytes); 0: 90 % of the
                             device memory free when the server is created */
  int32_t max_active;     /* solves on the device at once (0: no limit) */
  int32_t round_steps;    /* most steps per batch round between admissions
                             (0: 32) */
  int32_t one_at_a_time;  /* 1: plain FIFO queue through fdtd_step_n */
  int64_t fill_cells;     /* cells stepped per round: the resident requests
                             with the least remaining work are taken until
                             their cells reach this (0: 2^25) */
  int64_t solo_cells;     /* a request of at least this many cells fills the
                             device alone: it runs by itself (fdtd_step_n)
                             when its turn comes, and the batched rounds take
                             only the smaller ones (0: 2^22; -1: never) */
  int32_t policy;         /* order of the resident requests:
                             FDTD_SERVE_SRPT (0): least remaining work first;
                             FDTD_SERVE_HRRN (1): highest response ratio
                             (waited + remaining) / remaining first, which
                             bounds how long a large request waits;
                             FDTD_SERVE_BOUNDED (2): least remaining work
                             first, except that requests whose response
                             ratio reached 3 go ahead of the others, highest
                             ratio first;
                             FDTD_SERVE_DEADLINE (3): least remaining work
                             first, except that a request that would finish
                             later than it would have in a one-at-a-time
                             queue (its deadline: the queue's finish time,
                             from the arrival order and an estimate of each
                             request's time alone) goes ahead, earliest
                             deadline first -- running alone for a round if
                             it fills the device */
} fdtd_server_config;
#define FDTD_SERVE_SRPT 0
#define FDTD_SERVE_HRRN 1
#define FDTD_SERVE_BOUNDED 2
#define FDTD_SERVE_DEADLINE 3

typedef struct {
  double submit_s, admit_s, finish_s; /* server clock, seconds */
  uint64_t device_bytes;  /* held while running */
  int32_t status;         /* FDTD_OK, or the failing call's status */
  int32_t steps;
  char message[128];      /* why it failed */
} fdtd_request_info;

typedef struct {
  uint64_t submitted, completed, failed;
  uint64_t cell_steps;          /* of completed solves */
  uint64_t peak_reserved_bytes; /* highest sum of admitted peaks */
  int32_t peak_active;          /* most solves on the device at once */
  int32_t queued;               /* waiting now */
  int32_t active;               /* on the device now */
  double elapsed_s;             /* first submission to last completion */
  double latency_p50_s, latency_p90_s, latency_p99_s, latency_mean_s;
  double solves_per_s;          /* completed / elapsed_s */
  uint64_t hbm_budget;          /* the budget in use */
  uint64_t cancelled;           /* finished by fdtd_server_cancel (not in failed) */
} fdtd_server_stats;

int fdtd_server_create(fdtd_server *out, const fdtd_server_config *cfg);
/* Waits for every submitted request to finish, then stops the loop. */
int fdtd_server_destroy(fdtd_server srv);
int fdtd_server_submit(fdtd_server srv, const fdtd_request *req, uint64_t *ticket);
/* Blocks until the request finished (timeout_s < 0: no limit);
 * FDTD_ERR_STATE on timeout. */
int fdtd_server_wait(fdtd_server srv, uint64_t ticket, double timeout_s);
/* Copies a finished request's outputs (probes: steps x n_probes x 6 floats
 * as OutputProbes; field: I*J*K floats as OutputVis) and info, and releases
 * the ticket.  Either buffer may be NULL. */
int fdtd_server_result(fdtd_server srv, uint64_t ticket, float *probes, size_t n_probes,
                       float *field, size_t n_field, fdtd_request_info *info);
/* Blocks until nothing is queued or running. */
int fdtd_server_drain(fdtd_server srv);
int fdtd_server_get_stats(fdtd_server srv, fdtd_server_stats *out);
/* Cancels a request.  A queued request finishes at once with status
 * FDTD_ERR_CANCELLED; a request on the device leaves at the end of the
 * current round (its handle deleted, its memory returned to the budget) and
 * finishes with FDTD_ERR_CANCELLED -- the others keep stepping and their
 * results do not change.  In one_at_a_time mode a running request runs to
 * its end.  Returns FDTD_ERR_STATE when the request had already finished,
 * FDTD_ERR_INVALID_ARG for an unknown or released ticket.  The ticket is
 * released by fdtd_server_result as usual. */
int fdtd_server_cancel(fdtd_server srv, uint64_t ticket);

/* ---------------------------------------------------------------------
 * Host-side fault injection, for tests of the error paths (no reference
 * counterpart: the reference checks no CUDA call).  Nothing here faults,
 * traps or stalls the GPU: the failures are made on the host.
 * --------------------------------------------------------------------- */
#define FDTD_FAULT_NONE 0
#define FDTD_FAULT_DEVICE_ALLOC 1
/* FDTD_FAULT_DEVICE_ALLOC: the countdown-th device allocation a handle makes
 * from now on (any handle, any thread; countdown >= 1) fails as if the
 * device were out of memory (FDTD_ERR_OOM), once.  FDTD_FAULT_NONE disarms
 * a pending one. */
int fdtd_inject_fault(int32_t kind, int32_t countdown);
/* Writes value into the handle's device error word, as a kernel whose
 * bounded pipeline wait gave up would: the handle's next synchronising call
 * (fdtd_synchronize, a readout) reports FDTD_ERR_CUDA and clears the word.
 * Other handles are unaffected. */
int fdtd_inject_device_error(fdtd_handle h, int32_t value);

/* Allocation-free coefficient indexing.  No counterpart in the reference:
 * it serves callers that cannot allocate device memory -- hosts whose
 * device memory all comes from their own pool or a fixed budget, and loops
 * that must not stall other streams with the device-wide synchronisation
 * cudaMalloc / cudaFree imply.
 *
 * Replaces six per-cell E-coefficient arrays (ce[0..5] = Cexe Ceye Ceze
 * Cexh Ceyh Cezh, device pointers, cell (i,j,k) at i + j*pitch +
 * k*pitch*J) by a 2-byte id per cell (ids, device, pitch*J*K entries) and
 * a table of the distinct tuples (table, device, max_ids*6 floats, row id =
 * the six coefficients); *n_ids (host) receives the number of ids.  The
 * result is the one ReadySimulation builds internally (fdtd_get_table 6).
 *
 * Allocates nothing: the hash-table scratch is a file-scope device array of
 * 1.25 MiB that every GPU loading the library holds until the process
 * exits.  Limit: max_ids <= 32768; larger values are rejected with
 * FDTD_ERR_INVALID_ARG, and inputs with more distinct tuples than max_ids
 * fail with FDTD_ERR_UNSUPPORTED.  FDTD_ERR_UNSUPPORTED is also returned when
 * two distinct tuples share a 64-bit hash (fdtd_last_error says which of the
 * two happened); ReadySimulation keeps the six arrays in either case.  The
 * first call on a device looks up the array's device address and keeps it
 * for the process; make that first call before any stream capture, and do
 * not call it again on a device after cudaDeviceReset (the kept address
 * would be stale).
 * All calls share the one array, so calls that overlap on the GPU (on
 * different streams or host threads) race; serialise them.  stream is a
 * cudaStream_t (NULL: the legacy default stream); the call waits for it. */
int fdtd_index_coefficients_static(const float *const ce[6], int32_t I, int32_t J, int32_t K,
                                   int32_t pitch, uint16_t *ids, float *table, int32_t max_ids,
                                   int32_t *n_ids, void *stream);

/* Upper bound of the device memory one handle of these dimensions takes
 * at its peak (during ReadySimulation and Init1D), in bytes (no reference
 * counterpart; used for admission by memory budget). */
int fdtd_estimate_device_bytes(int32_t I, int32_t J, int32_t K, int32_t pml, int32_t T,
                               int32_t num_ant, uint64_t *bytes);

/* The plan the kernels use for the CPML recurrences' division by the cell
 * size (no reference counterpart; the reference divides): out[0] =
 * RN(1/dx); for numerators a with out[1] <= |a| < out[2] the quotient is
 * RN(a*out[0]) corrected by one fused multiply-add step, which the library
 * has checked to equal the IEEE quotient a/dx for every such a; for
 * out[3] <= |a| < out[1] the same is done on a*2^64 and scaled back; zero
 * and other numerators are exact or divided.  Host only. */
int fdtd_division_plan(float dx, float out[4]);

/* Evaluates that plan on the current GPU for every float bit pattern as a
 * numerator (2^32 inputs, about a second) and stores in *mismatches the
 * number whose quotient differs bitwise from the GPU's IEEE division a/dx
 * (no reference counterpart: a self-check). */
int fdtd_check_division(float dx, uint64_t *mismatches);

/* Bounded-wait self-check on the current GPU: every pipeline wait of the
 * kernels gives up after a fixed time of the GPU's global timer (2 s),
 * raises the device error word and returns (the host then reports
 * FDTD_ERR_CUDA) instead of hanging.  This runs that wait with a 1 ms limit
 * on a barrier nothing completes -- *timed_out must be 1, *poll_ns receives
 * the ns it waited -- and then on one the waiting thread completes --
 * *completed must be 1, so the context is still usable; *limit_ms is the
 * production limit.  No reference counterpart. */
int fdtd_check_bounded_wait(int32_t *timed_out, int32_t *completed, double *poll_ns,
                            double *limit_ms);

/* Number of kernels this library has launched (all handles). */
uint64_t fdtd_launch_count(void);

/* Message for the last failing call on this thread. */
const char *fdtd_last_error(void);

/* Source waveform of FunLib('CreateSignal', ...) --
 * src/cpucode/FunLib.cpp:6-45 (double precision, 1-based n). */
int fdtd_create_signal(double fctr, double delT, double percentage_bw,
                       double num_side_lobes, size_t time_steps, double *out,
                       double *fmaxx);

#ifdef __cplusplus
}
#endif
#endif
