/* cflbm.h -- C ABI of the GB300 lattice-Boltzmann cylinder-flow solver.
 *
 * One handle = one channel (or one reference-profile box) resident on one GPU,
 * with its own CUDA stream.  Every call returns 0 on success or a CFLBM_E_* code;
 * cflbm_last_error() gives the message of the last failure on the calling thread.
 * Calls on one handle are not thread-safe; separate handles are independent.
 *
 * The entry points replace the per-step methods of the reference's solver class
 * (Maccchiatooo/Cylinder-flow, "3D MPI+KOKKOS+MPIIO/lbm.hpp:106-233" and
 * "MPI Kokkos/lbm.hpp:64-128"); each declaration names the reference code it
 * stands in for.  Array arguments are plain host pointers unless a name says
 * otherwise; field arrays cover the interior only, x fastest ("Fortran order"),
 * the order the reference writes its Tecplot blocks in
 * ("3D MPI+KOKKOS+MPIIO/lbm.cpp:444-460").
 */
#ifndef CFLBM_H
#define CFLBM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CFLBM_ABI_VERSION 1

/* ---- error codes ---------------------------------------------------------- */
#define CFLBM_OK 0
#define CFLBM_E_INVALID 1     /* bad argument or configuration */
#define CFLBM_E_CUDA 2        /* a CUDA runtime call failed */
#define CFLBM_E_NOMEM 3       /* device or host allocation failed */
#define CFLBM_E_NUMERIC 4     /* NaN/Inf detected in a checked quantity */
#define CFLBM_E_IO 5          /* file I/O failed */
#define CFLBM_E_UNSUPPORTED 6 /* combination not built */

/* ---- enumerations ----------------------------------------------------------- */
enum cflbm_lattice { CFLBM_D2Q9 = 9, CFLBM_D3Q27 = 27 };
/* Population storage.  FP16DEV stores f_i / t_i (f_i is already the deviation
 * from t_i*rho0, as in the reference) as IEEE binary16. */
enum cflbm_storage { CFLBM_STORE_FP64 = 0, CFLBM_STORE_FP32 = 1, CFLBM_STORE_FP16DEV = 2 };
/* Arithmetic of the collision.  DF64: double-float (pairs of binary32, about 48
 * significant bits) on the FP32 units, with FP64 storage only; for the channel
 * and reference profiles (not the adjoint or the batch). */
enum cflbm_compute { CFLBM_COMPUTE_FP64 = 0, CFLBM_COMPUTE_FP32 = 1, CFLBM_COMPUTE_DF64 = 2 };
/* Boundary/initial-condition profile.
 *  CHANNEL: the benchmark channel (equilibrium inlet, zero-gradient outlet,
 *           free-slip/no-slip/periodic walls, halfway bounce-back on solids).
 *  REF2D:   the reference's 2-D solver at one rank, "MPI Kokkos/lbm.cpp"
 *           (Poiseuille inlet override, p = 0 outlet, its wall and solid rules,
 *           disk of diameter 0.03125*(nx-1) at the box centre).
 *  REF3D:   the reference's 3-D solver at one rank, "3D MPI+KOKKOS+MPIIO/lbm.cpp"
 *           (sphere at ((nx-1)/8)^3, radius (nx-1)/64).
 *  REF2DS:  the reference's serial 2-D solver, "Kokkos/lbm.cpp" (its LBM(sx, sy)
 *           is nx = sx + 1 by ny = sy + 1 interior nodes; disk at
 *           (0.25 (nx - 1), 0.5 (ny + 3)) of its ghosted box with radius
 *           0.1 (ny - 1); Poiseuille u times (1 + 0.001 ran); wall ghost rows
 *           without their corner nodes; no force in the reference). */
enum cflbm_profile {
  CFLBM_PROFILE_CHANNEL = 0,
  CFLBM_PROFILE_REF2D = 1,
  CFLBM_PROFILE_REF3D = 2,
  CFLBM_PROFILE_REF2DS = 3
};
enum cflbm_wall { CFLBM_WALL_FREESLIP = 0, CFLBM_WALL_NOSLIP = 1, CFLBM_WALL_PERIODIC = 2 };
enum cflbm_geom { CFLBM_GEOM_NONE = 0, CFLBM_GEOM_CYLINDER = 1, CFLBM_GEOM_SPHERE = 2 };
/* Population layout in device memory (x fastest in both):
 *  SOA:  f[i][z][y][x] -- one array per population;
 *  ROWS: f[z][y][i][x] -- the Q rows of a (y, z) line are adjacent. */
enum cflbm_layout { CFLBM_LAYOUT_SOA = 0, CFLBM_LAYOUT_ROWS = 1 };
/* Rounding of FP16-deviation stores: to nearest, or stochastic (hardware
 * cvt.rs fed with a hash of value and element: deterministic and identical
 * across kernels and layouts). */
enum cflbm_rounding { CFLBM_ROUND_NEAREST = 0, CFLBM_ROUND_STOCHASTIC = 1 };

typedef struct cflbm_handle cflbm_handle;

/* Construction parameters.  Fill with cflbm_config_default() first. */
typedef struct cflbm_config {
  int lattice;          /* CFLBM_D2Q9 or CFLBM_D3Q27 */
  int nx, ny, nz;       /* interior cells (reference glx, gly, glz); nz = 1 in 2-D */
  int storage;          /* enum cflbm_storage */
  int compute;          /* enum cflbm_compute */
  int profile;          /* enum cflbm_profile */
  int wall_y, wall_z;   /* CHANNEL only: enum cflbm_wall for the y and z face pairs */
  double tau0;          /* reference System::tau = u0*R/Re/cs2; omega = 1/(tau0+0.5) */
  double u0;            /* CHANNEL: inlet speed; REF*: Poiseuille peak speed */
  int geom;             /* CHANNEL: enum cflbm_geom */
  double cx, cy, cz;    /* CHANNEL: body centre in cell coordinates */
  double diam;          /* CHANNEL: body diameter in cells (Cd reference length) */
  double perturb_amp;   /* CHANNEL: amplitude of the seeded uniform u_y perturbation */
  uint64_t seed;        /* CHANNEL: perturbation seed */
  const uint8_t *solid; /* CHANNEL: optional nx*ny*nz mask (1 = solid), overrides geom */
  const double *alpha;  /* CHANNEL: optional nx*ny*nz Brinkman porosity in [0,1] */
  const int32_t *ref_ran; /* REF*: the reference's per-node draw over the ghosted box
                             (its layout, (i*ly+j)*lz+k), or NULL for a seeded draw */
  int force_history;    /* capacity (steps) of the on-device force history; 0 = 65536 */
  int device;           /* CUDA device ordinal */
  int layout;           /* enum cflbm_layout */
  int rounding;         /* enum cflbm_rounding (FP16 storage only; default stochastic) */
} cflbm_config;

/* Geometry/step counters and device layout of a handle. */
typedef struct cflbm_info {
  int lattice, nx, ny, nz, storage, compute, profile;
  int ghost;            /* ghost layers around the interior */
  int pitch_x;          /* elements per padded x row */
  int64_t pop_stride;   /* elements between populations */
  int64_t steps_done;   /* time steps advanced since creation (or last set_f) */
  int64_t n_links;      /* fluid->solid links (bounce-back, force) */
  int64_t n_solid;      /* solid interior cells */
  double omega;         /* 1/(tau0+0.5) */
  double bytes_per_cell_step; /* algorithmic HBM bytes per cell update of the sweep */
  size_t device_bytes;  /* device memory held by the handle */
  int layout;           /* enum cflbm_layout */
} cflbm_info;

/* Defaults: D2Q9 64x32, FP64 storage and arithmetic, CHANNEL, free-slip y,
 * periodic z, tau0 = 0.03, u0 = 0.05, no body, no perturbation, ROWS layout,
 * stochastic rounding of FP16 stores. */
int cflbm_config_default(cflbm_config *cfg);

/* Allocate device state and initialise it (f = equilibrium of the initial
 * macroscopic fields).  Replaces LBM::LBM + LBM::Initialize
 * ("3D MPI+KOKKOS+MPIIO/lbm.hpp:146-219", "lbm.cpp:36-256";
 * "MPI Kokkos/lbm.hpp:114", "lbm.cpp:47-126"). */
int cflbm_create(const cflbm_config *cfg, cflbm_handle **out);

/* Free everything the handle owns.  NULL is accepted. */
int cflbm_destroy(cflbm_handle *h);

/* Advance nsteps time steps.  One step = the reference's
 * Collision(); [pack(); exchange(); unpack();] Streaming(); Update();
 * ("3D MPI+KOKKOS+MPIIO/main.cpp:29-45", lbm.cpp:257-417;
 * "MPI Kokkos/main.cpp:26-37", lbm.cpp:127-457), fused into one pull sweep plus
 * a boundary kernel.  The halo exchange collapses to nothing at one rank.
 * Asynchronous with respect to the host; errors of earlier launches surface here
 * or at the next synchronising call. */
int cflbm_step(cflbm_handle *h, int nsteps);

/* Block until all work queued on the handle's stream has finished. */
int cflbm_synchronize(cflbm_handle *h);

/* Self-test of the bounded-wait error path (no reference counterpart): queues
 * on h's stream a kernel whose one waiting thread gives up on an mbarrier that
 * nothing arrives on after `polls` polls (1 .. 2^22) and records the timeout
 * in h's device error word, as the line-staged sweep's waits do.  The next
 * synchronising call (cflbm_synchronize, cflbm_mass) then returns
 * CFLBM_E_CUDA naming the timeout, and every later one does too: the handle is
 * marked failed; destroy it.  The CUDA context stays usable. */
int cflbm_selftest_wait_timeout(cflbm_handle *h, int64_t polls);

/* Macroscopic fields after the last step: u, v, w, p over the interior, x
 * fastest, as LBM::Update leaves them ("3D.../lbm.cpp:374-417": p = sum f/3,
 * u = sum f e, zero in solids, reference-profile inlet/outlet overrides).
 * Any pointer may be NULL.  Host pointers; synchronises.  CHANNEL profile: the
 * steps do not write these fields; the first call after a step forms them from
 * the state that step read (one read of the populations, bit-identical to
 * forming them inside the step). */
int cflbm_macros(cflbm_handle *h, double *u, double *v, double *w, double *p);

/* Same, into device pointers (no synchronisation; ordered on the handle's
 * stream). */
int cflbm_macros_device(cflbm_handle *h, double *d_u, double *d_v, double *d_w, double *d_p);

/* Momentum-exchange force of the last step and its coefficients.  Replaces the
 * force block of "MPI Kokkos/lbm.cpp:356-407": fxyz = (Fx, Fy, Fz) in lattice
 * units, cd_cl = (2 Fx / (u0^2 A), 2 Fy / (u0^2 A)) with A the reference area
 * (2-D: D; spanwise cylinder: D*nz; sphere: pi D^2/4; REF2D: D = 0.03125*(nx-1)).
 * Either pointer may be NULL.  Synchronises. */
int cflbm_forces(cflbm_handle *h, double fxyz[3], double cd_cl[2]);

/* The same (Fx, Fy, Fz) of the last step queued on the handle's stream as an
 * asynchronous device-to-host copy into fxyz (page-locked memory makes it
 * asynchronous); valid after cflbm_synchronize.  Lets a caller that reads every
 * step's force (the reference writes test.dat every step) queue the next step
 * before that force has arrived. */
int cflbm_forces_async(cflbm_handle *h, double fxyz[3]);

/* Per-step force history (Fx, Fy, Fz per step, oldest first) of the last
 * min(steps_done, capacity) steps.  Writes up to max_steps rows into out
 * (3*max_steps doubles) and the row count into *n_out.  Synchronises. */
int cflbm_force_history(cflbm_handle *h, double *out, int64_t max_steps, int64_t *n_out);

/* Domain sums in FP64: mass = sum over fluid cells of (1 + sum_i f_i)
 * (i.e. rho), and momentum (3 doubles).  Either pointer may be NULL. */
int cflbm_mass(cflbm_handle *h, double *mass, double momentum[3]);

/* Dump / restore the post-collision populations of the interior in FP64,
 * layout [i][z][y][x] (x fastest), q*nx*ny*nz doubles.  The reference has no
 * restart; this is the checkpoint path.  set_f also sets steps_done. */
int cflbm_get_f(cflbm_handle *h, double *out);
int cflbm_set_f(cflbm_handle *h, const double *in, int64_t steps_done);

/* The post-stream (pre-collision) populations of the last step in FP64, layout
 * [i][z][y][x] (x fastest), q*nx*ny*nz doubles: what the reference's f holds
 * after Streaming() and Update() ("3D MPI+KOKKOS+MPIIO/lbm.cpp:359-371",
 * "MPI Kokkos/lbm.cpp:409-418", "Kokkos/lbm.cpp:178-186"), i.e. the state its Output() writes population 1 of
 * ("3D MPI+KOKKOS+MPIIO/lbm.cpp:741-771").  Before the first step: the initial
 * state, f = feq of the initial fields (as after LBM::Initialize).  The handle
 * keeps the post-collision state; this forms the pull of the last step from the
 * state that step read.  Synchronises. */
int cflbm_get_f_stream(cflbm_handle *h, double *out);

/* The interior solid mask, nx*ny*nz bytes (x fastest), 1 = solid: the
 * complement of the reference's usr ("3D MPI+KOKKOS+MPIIO/lbm.cpp:238",
 * usr = 1 in fluid).  Synchronises. */
int cflbm_get_solid(cflbm_handle *h, uint8_t *out);

/* Handle geometry, counters and memory. */
int cflbm_get_info(cflbm_handle *h, cflbm_info *info);

/* Write the Tecplot binary file of LBM::MPIoutput(n)
 * ("3D MPI+KOKKOS+MPIIO/lbm.cpp:419-739"; 2-D: "MPI Kokkos/lbm.cpp:459-737"):
 * "#!TDV112" header with variables x,y,(z,)u,v,(w,)p, zone "ZONE 001", solution
 * time n, min/max of every variable, then the variables as x-fastest FP64
 * blocks.  Byte-identical to the reference's file for the same fields. */
int cflbm_write_tecplot(cflbm_handle *h, const char *path, int n);

/* The same writer for caller-supplied host fields (dim 2: u, v, p used, w
 * ignored; nz ignored).  Needs no GPU. */
int cflbm_write_tecplot_fields(const char *path, int dim, int nx, int ny, int nz,
                               const double *u, const double *v, const double *w,
                               const double *p, int n);

/* ---- batched channels ------------------------------------------------------
 * Many independent CHANNEL-profile instances (uneven sizes, Reynolds numbers)
 * advanced together: per step one persistent work-list launch over every
 * instance's interior tiles and one over every instance's solid-adjacent tiles,
 * replayed from a captured CUDA graph of graph_steps steps; the tile height and
 * persistent grid size are picked at creation by timing every candidate on the
 * real state (which is left unchanged).  The reference runs one channel per
 * process; this has no counterpart there beyond the per-instance physics of
 * LBM::Collision/Streaming/Update.  All instances share lattice, storage and
 * device, and use FP32 arithmetic. */
typedef struct cflbm_batch cflbm_batch;

typedef struct cflbm_batch_options {
  int graph_steps;    /* steps per captured graph (even, default 100) */
  int autotune;       /* 1 (default): time candidates at creation */
  int tile_height;    /* rows per block when not autotuning: 1, 2, 4 or 8 */
  int blocks_per_sm;  /* persistent grid = SMs * this when not autotuning; 0 = one
                         interior work item per block */
} cflbm_batch_options;

typedef struct cflbm_batch_info {
  int instances;
  int64_t cells;               /* interior cells over all instances */
  int64_t steps_done;
  int tile_height;             /* chosen launch shape */
  int grid_blocks;             /* persistent grid, 0 = one interior item per block */
  int graph_steps;
  int tuned_candidates;        /* launch shapes timed by the autotuner */
  double tuned_step_ms;        /* best candidate's step time */
  double bytes_per_cell_step;  /* algorithmic HBM bytes per cell update */
} cflbm_batch_info;

int cflbm_batch_options_default(cflbm_batch_options *opt);
/* Create n instances from cfgs[0..n-1] (each as cflbm_create would). */
int cflbm_batch_create(const cflbm_config *cfgs, int n, const cflbm_batch_options *opt,
                       cflbm_batch **out);
int cflbm_batch_destroy(cflbm_batch *b);
/* Advance every instance nsteps steps (asynchronous). */
int cflbm_batch_step(cflbm_batch *b, int nsteps);
int cflbm_batch_synchronize(cflbm_batch *b);
/* Instance k as a handle for the result calls (macros, forces, force history,
 * mass, get_f, write_tecplot); stepping it alone is rejected.  Owned by the
 * batch.  NULL if k is out of range. */
cflbm_handle *cflbm_batch_handle(cflbm_batch *b, int k);
int cflbm_batch_get_info(cflbm_batch *b, cflbm_batch_info *info);

/* The CUDA stream (cudaStream_t) the handle launches on, for callers that
 * order their own work or events against the solver. */
int cflbm_get_stream(cflbm_handle *h, void **stream);

/* Kernel timing: when enabled, CUDA events are recorded on the handle's stream
 * around every sweep launch and around every boundary phase (ghost fill +
 * bounce-back/force).  cflbm_get_timing synchronises and returns
 * ms[0] = total sweep time, ms[1] = total boundary time, counts[0] = sweeps,
 * counts[1] = boundary phases since the last reset, then resets. */
int cflbm_set_timing(cflbm_handle *h, int enable);
int cflbm_get_timing(cflbm_handle *h, double ms[2], int64_t counts[2]);

/* Domain sums that allocate nothing -- no counterpart in the reference.
 *
 * For callers that cannot call cudaMalloc (a memory pool or framework that owns
 * every device byte, a fixed memory budget, code running where allocation is
 * forbidden) but hold populations in device memory.  cflbm_mass() needs a
 * handle, and creating one allocates; this call needs none.
 *
 * d_f:     device array, dense [i][z][y][x] (x fastest), q*nx*ny*nz elements of
 *          the storage type (FP16DEV: f_i times the lattice's per-direction
 *          power-of-two scale, as cflbm stores it).
 * d_solid: optional device uint8 mask, nx*ny*nz (1 = solid, skipped), or NULL.
 * d_out:   device, 4 doubles: sum over fluid cells of (1 + sum_i f_i), then the
 *          momentum sum_i f_i e_i (x, y, z); all accumulated in FP64.
 * stream:  cudaStream_t to launch on (NULL = legacy default stream).
 *
 * Scratch (per-block partials and a completion counter) is a file-scope device
 * array of 512 KiB held by every GPU that loads the library until exit; grids of
 * more than 134,217,728 cells are rejected with CFLBM_E_INVALID.  The first call
 * on a device looks up the array's device address; make it before any stream
 * capture.  The address is kept for the process, so the call serves the
 * device's primary context only: not after cudaDeviceReset, not from another
 * driver context.  Calls share the array, so calls that overlap on the GPU race.
 * Asynchronous: read d_out after synchronising the stream. */
int cflbm_domain_sums_noalloc(int lattice, int storage, int nx, int ny, int nz,
                              const void *d_f, const uint8_t *d_solid, double *d_out,
                              void *stream);

/* Discrete adjoint of the D2Q9 channel step -- no counterpart in the reference,
 * which has no gradients.  It differentiates the step the reference performs in
 * LBM::Collision and LBM::Streaming ("Kokkos/lbm.cpp:134-186": BGK collision,
 * pull streaming, halfway bounce-back; momentum-exchange force of
 * "MPI Kokkos/lbm.cpp:356-377") for the channel profile, with the Brinkman
 * porosity field of cflbm_config.alpha, free-slip / no-slip / periodic y walls.
 *
 * Objective J = mean over steps [window_begin, window_end] (1-based) of F_x
 * (objective 0, drag) or F_y (1, lift), the force history the solver records.
 * The call runs `steps` forward steps from a fresh handle (steps_done == 0,
 * force_history >= steps), keeping a checkpoint every `checkpoint_every` steps,
 * then runs the reverse sweep segment by segment (recomputing each segment's
 * states from its checkpoint while the previous one is reversed), so device
 * memory is ceil(steps/K) + 2K states on top of the handle.  FP32/FP32 or
 * FP64/FP64 storage/arithmetic.
 * dJ_dalpha: host, nx*ny doubles (x fastest) or NULL; the gradient with respect
 * to the per-cell porosity (at alpha = 0 where the handle has no field). */
typedef struct cflbm_adjoint_spec {
  int32_t steps;            /* forward steps T */
  int32_t checkpoint_every; /* K */
  int32_t window_begin;     /* first step of the averaging window */
  int32_t window_end;       /* last step of the window (<= T) */
  int32_t objective;        /* 0: F_x, 1: F_y */
} cflbm_adjoint_spec;

typedef struct cflbm_adjoint_result {
  double J;                 /* objective of the forward run */
  double dJ_du_in;          /* inlet speed (inlet equilibrium and initial u_x) */
  double dJ_dtau;           /* relaxation time tau = tau0 + 0.5 */
  double seconds_forward;   /* wall time of the forward run with checkpoints */
  double seconds_reverse;   /* wall time of recomputation + reverse sweep */
  int64_t device_bytes;     /* scratch the call allocated */
} cflbm_adjoint_result;

int cflbm_adjoint(cflbm_handle *h, const cflbm_adjoint_spec *spec, double *dJ_dalpha,
                  cflbm_adjoint_result *result);

/* Message of the last failing call on this thread ("" if none). */
const char *cflbm_last_error(void);

/* Number of kernel launches issued by this library since load (all handles). */
int64_t cflbm_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif /* CFLBM_H */
