/*
 * lbdem.h - C ABI of the GB300 coupled free-surface lattice-Boltzmann / DEM
 * impact solver (liblbdem.so).
 *
 * This boundary replaces the reference's in-process C++ classes:
 *   LB  (src/LB.h:32-230)   latticeDefinition, latticeBoltzmannGet,
 *        latticeBolzmannInit, latticeBolzmannStep,
 *        latticeBoltzmannCouplingStep, latticeBoltzmannFreeSurfaceStep
 *   DEM (src/DEM.h:21-190)  discreteElementGet, discreteElementInit,
 *        discreteElementStep
 * and the per-step driver goCycle (src/main.cpp:38-67).
 * All quantities are in the reference's units: configuration values and
 * particle/object/wall state in physical units, lattice fields in lattice
 * units. The vertical axis is y, as in the reference.
 *
 * Conventions
 *  - Every call returns an int status (LBDEM_OK == 0). lbdem_last_error()
 *    gives a message for the most recent failure on a context.
 *  - Plain pointers and sizes only; caller-owned host buffers; the context
 *    owns all device memory. One context is one impact run on one GPU.
 *  - Calls on one context are not thread-safe; distinct contexts are.
 *  - Every call on a context makes the context's device current for its
 *    own duration and restores the calling thread's device on return.
 *  - Download calls synchronise the context's stream; step calls only
 *    enqueue work (no host synchronisation inside a step).
 */
#ifndef LBDEM_H
#define LBDEM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LBDEM_ABI_VERSION 1

/* status codes */
#define LBDEM_OK 0
#define LBDEM_ERR_INVALID 1      /* bad argument or unsupported option   */
#define LBDEM_ERR_CUDA 2         /* CUDA runtime error                   */
#define LBDEM_ERR_OOM 3          /* device allocation failed             */
#define LBDEM_ERR_IO 4           /* configuration / input file error     */
#define LBDEM_ERR_NONFINITE 5    /* NaN or Inf detected in the state     */
#define LBDEM_ERR_OVERFLOW 6     /* neighbour list or cell list overflow */
#define LBDEM_ERR_DEVICE_STATE 7 /* kernel reported an internal error    */
#define LBDEM_ERR_NO_DEVICE 8    /* no CUDA device present               */

/* node types, src/node.h:130-143 */
#define LBDEM_FLUID 0
#define LBDEM_GAS 2
#define LBDEM_INTERFACE 3
#define LBDEM_PERIODIC 4
#define LBDEM_SLIP_STAT_WALL 5
#define LBDEM_SLIP_DYN_WALL 6
#define LBDEM_STAT_WALL 7
#define LBDEM_DYN_WALL 8
#define LBDEM_CYLINDER 9
#define LBDEM_TOPOGRAPHY 11
#define LBDEM_OBJECT 12

/* rheology models (enum Rheology, src/node.h:17) */
#define LBDEM_NEWTONIAN 0
#define LBDEM_BINGHAM 1
#define LBDEM_FRICTIONAL 2
#define LBDEM_VOELLMY 3

/* precision forms */
#define LBDEM_PLAIN_FP64 0 /* FP64 throughout, reproduces the reference    */
#define LBDEM_MIXED 1      /* FP32 deviation storage, FP64 islands         */

/* One suspended sphere as read from particles.dat (src/DEM.cpp:88-134):
 * radius, position (after the reader's -0.05 shift and scale), velocity,
 * angular velocity. */
typedef struct lbdem_particle_in {
  double r;
  double x[3];
  double v[3];
  double w[3];
  int32_t size;  /* constituent count, multiplies mass and inertia        */
  int32_t index; /* index column of particles.dat (informational)         */
} lbdem_particle_in;

/* One impactor as read from objects.dat (src/DEM.cpp:142-166). */
typedef struct lbdem_object_in {
  int32_t index;
  double r;
  double x[3];
  double v[3];
} lbdem_object_in;

/* One body as read from body.dat (src/DEM.cpp:168-196): a sphere joined to
 * every impactor by a spring of stiffness k and rest length L0 along y
 * (DEM::bodyObjectInteraction, src/DEM.cpp:798-869). */
typedef struct lbdem_body_in {
  int32_t index;
  double r;
  double x[3]; /* position, times scale */
  double v[3];
  double k, L0;
} lbdem_body_in;

/* Every configuration key of parameters.cfg the step depends on, with the
 * reference's names (src/main.cpp:128-185, src/LB.cpp:128-338,
 * src/DEM.cpp:17-78). Unsupported keys (topography, rotation,
 * non-Newtonian rheology, bodies) are accepted only at their inert values. */
typedef struct lbdem_config {
  /* switches and time integration */
  int32_t demSolve, lbSolve, freeSurfaceSolve, forceFieldSolve;
  double demInitialRepeat;
  int32_t lbmInitialRepeat;
  double maxTime;
  int32_t maximumTimeSteps;
  /* output cadences (host-side IO only) */
  double screenExpTime, fluidExpTime, fluidLagrangianExpTime, partExpTime,
      partRecycleExpTime, fluidRecycleExpTime;
  /* LB */
  double unitLength, unitTime, unitDensity;
  double lbSizeX, lbSizeY, lbSizeZ;
  int32_t lbRestart, lbTopography;
  double initVelocity[3];
  double lbF[3];
  double lbRot[3];
  double lbRotCenter[3];
  int32_t boundary[6];
  double slipCoefficient;
  double fluidHeight;
  int32_t rheologyNewtonian; /* 1 when rheologyModel = NEWTONIAN          */
  double initVisc;
  int32_t turbulenceSolve;
  double turbConst;
  /* DEM */
  double density, objectDensity, bodyDensity;
  double linearStiff, frictionCoefPart;
  double lubNormal, lubTangential, lubRotation, lubCutoff, kinVisc;
  double debyeLength, electroForce;
  int32_t objWaitTime, intervalTime;
  double springDamp, epsilon;
  int32_t nonLinType;
  double k13, scale;
  /* inputs (./input/*.dat) */
  int32_t n_particles;
  const lbdem_particle_in* particles;
  int32_t n_objects;
  const lbdem_object_in* objects;
  int32_t n_bodies;
  /* lbRestartFile (src/LB.cpp:139): the fluid recycle file read under
   * lbRestart, as given (relative to the working directory) */
  const char* lbRestartFile;
  /* rheology (src/LB.cpp:196-242): the model (LBDEM_NEWTONIAN ...) and its
   * parameters in physical units; a key the model does not read keeps its
   * default, as in the reference (BINGHAM reads no initVisc: initVisc is
   * then the default 1/6 of the reference's FluidMaterial). Apparent
   * viscosity and the Smagorinsky term (turbulenceSolve, turbConst) follow
   * node::computeApparentViscosity (src/node.cpp:113-168). */
  int32_t rheologyModel;
  double plasticVisc, yieldStress, frictionCoefFluid, voellmyConstant;
  /* body.dat records (n_bodies of them) */
  const lbdem_body_in* bodies;
} lbdem_config;

/* Run options that are not part of the reference's configuration. */
typedef struct lbdem_options {
  int32_t precision;   /* LBDEM_PLAIN_FP64 or LBDEM_MIXED                 */
  int32_t device;      /* CUDA device ordinal                             */
  int32_t check_every; /* NaN/Inf guard cadence in steps (0 = off)        */
  int32_t chunks_per_block; /* mixed lattice step: 256-node chunks per block
                               at least (0: 8); fewer blocks for a small
                               lattice leave SMs to other runs            */
  int32_t async_init;  /* 1: lbdem_create returns once the device
                          initialisation is enqueued; its device errors
                          surface at the next lbdem_sync                  */
  int32_t debug_flags; /* tests of the failure paths only; 0 otherwise    */
  int32_t reserved[2];
} lbdem_options;

/* debug_flags: the mixed form's lattice step issues none of its bulk copies
 * into shared memory, so its bounded waits for them run out (after a short
 * limit; nothing is in flight) and the step reports
 * LBDEM_ERR_DEVICE_STATE at the next lbdem_sync. For tests of that path. */
#define LBDEM_DEBUG_NO_LATTICE_COPIES 1

typedef struct lbdem_ctx lbdem_ctx;

/* ---- configuration (host only; no GPU needed) ----------------------- */

/* Fill *cfg with the reference's defaults for every key
 * (the third argument of each PARSE_CLASS_MEMBER). */
int lbdem_config_defaults(lbdem_config* cfg);

/* Parse a GetPot parameters file plus input_dir/{particles,objects,body}.dat
 * into *cfg, with "-key value" overrides from argv (src/macros.h:14-19).
 * Replaces LB::latticeBoltzmannGet (src/LB.cpp:128) and
 * DEM::discreteElementGet (src/DEM.cpp:17). Arrays are owned by the library
 * until lbdem_config_release(). */
int lbdem_config_load(const char* cfg_path, const char* input_dir, int argc,
                      const char* const* argv, lbdem_config* cfg, char* err,
                      size_t err_len);
void lbdem_config_release(lbdem_config* cfg);

/* ---- lifecycle ------------------------------------------------------- */

/* Build the lattice, walls, impactor and particle state on the device.
 * Replaces LB::latticeDefinition (src/LB.cpp:85), DEM::discreteElementInit
 * (src/DEM.cpp:199) and LB::latticeBolzmannInit (src/LB.cpp:340), in the
 * order of src/main.cpp:264-283. */
int lbdem_create(const lbdem_config* cfg, const lbdem_options* opt,
                 lbdem_ctx** out);
void lbdem_destroy(lbdem_ctx* ctx);
const char* lbdem_last_error(const lbdem_ctx* ctx);
/* Use a caller-provided cudaStream_t (NULL restores the context's own). */
int lbdem_set_stream(lbdem_ctx* ctx, void* cuda_stream);

/* ---- step entry points (enqueue only) -------------------------------- */

/* DEM::discreteElementStep, src/DEM.cpp:359-401 */
int lbdem_dem_step(lbdem_ctx* ctx);
/* LB::latticeBoltzmannCouplingStep, src/LB.cpp:432-467. One departure: a
 * wall-layer node that an impactor covered and then uncovered becomes gas
 * (the reference makes it fluid or interface when it has fluid
 * neighbours, and then streams it beyond the lattice). */
int lbdem_coupling_step(lbdem_ctx* ctx);
/* LB::latticeBolzmannStep, src/LB.cpp:400-418 */
int lbdem_lb_step(lbdem_ctx* ctx);
/* LB::latticeBoltzmannFreeSurfaceStep, src/LB.cpp:422-430 */
int lbdem_free_surface_step(lbdem_ctx* ctx);
/* n repetitions of goCycle (src/main.cpp:38-67) without IO */
int lbdem_cycle(lbdem_ctx* ctx, int32_t n);
/* wait for all enqueued work; returns the first device-side error */
int lbdem_sync(lbdem_ctx* ctx);

/* ---- state access (synchronising) ------------------------------------ */

typedef struct lbdem_info {
  int32_t lb_size[3];
  int64_t nodes;
  int32_t n_particles, n_objects, n_walls;
  int32_t precision;
  int64_t time_step;   /* goCycle count (LB::time)          */
  int64_t dem_step;    /* DEM::demTimeStep                  */
  double dem_time;     /* DEM::demTime                      */
  double unit_length, unit_time, unit_density;
  int64_t device_bytes;
  int32_t neighbour_rebuilds;
  int32_t reserved[7];
} lbdem_info;
int lbdem_get_info(lbdem_ctx* ctx, lbdem_info* info);

/* Lattice fields, dense over all nodes (index = x + y*X + z*X*Y):
 * type[N], pflag[N] (inside-particle flag), solid[N] (solid index),
 * n[N], u[3N] (x-block, y-block, z-block), mass[N], f[19N] (direction
 * blocks). Values of non-active nodes are 0. Any pointer may be NULL. */
int lbdem_download_lattice(lbdem_ctx* ctx, uint8_t* type, uint8_t* pflag,
                           int32_t* solid, double* n, double* u, double* mass,
                           double* f);

/* Body state [B][3] (physical units): position, velocity, spring force
 * and total force of the last DEM step, and the spring length L of
 * DEM::bodyObjectInteraction [B]. Any pointer may be NULL. */
int lbdem_download_bodies(lbdem_ctx* ctx, double* x0, double* x1, double* FSpring,
                          double* FTotal, double* L);

/* Viscosity of every node in lattice units, visc[N]: node::visc
 * (src/node.h:54-114), which LB::collision updates per node for
 * non-Newtonian rheology and the Smagorinsky term (src/LB.cpp:1322-1325,
 * src/node.cpp:113-168); initVisc at every active node of a Newtonian run;
 * 0 at non-active nodes. */
int lbdem_download_viscosity(lbdem_ctx* ctx, double* visc);

/* Particle state, row-major [P][3]; any pointer may be NULL. */
typedef struct lbdem_particle_view {
  double* x0;
  double* x1;
  double* w1;
  double* FHydro;
  double* MHydro;
  double* FContact;
  double* MContact;
  double* FLub;
  double* MLub;
  double* FRep;
  double* FTotal;
  double* MTotal;
  double* fluidVolume; /* [P]     */
  double* SHydro;      /* [P][9]  */
  int32_t* list;       /* [P][50] neighbour list, slot 0 = count */
  double* xi;          /* [P][3][50] tangential springs           */
  double* xiw;         /* [P][3] wall spring                      */
  double* xio;         /* [P][3] object spring                    */
} lbdem_particle_view;
int lbdem_download_particles(lbdem_ctx* ctx, const lbdem_particle_view* v);

/* Object (impactor) state [O][3] and wall forces [W][3]. */
typedef struct lbdem_object_view {
  double* x0;
  double* x1;
  double* w1;
  double* FHydro;
  double* MHydro;
  double* FContact;
  double* MContact;
  double* FLub;
  double* MLub;
  double* FTotal;
} lbdem_object_view;
int lbdem_download_objects(lbdem_ctx* ctx, const lbdem_object_view* v);
int lbdem_download_walls(lbdem_ctx* ctx, double* FHydro, double* FContact,
                         double* FLub, double* FTotal);

/* Diagnostics: total mass of active nodes, interface-node count, active
 * count (device reductions). */
int lbdem_mass_summary(lbdem_ctx* ctx, double* total_mass,
                       int64_t* interface_nodes, int64_t* active_nodes);
/* Total mass of every active node, those inside particles included (the
 * conserved quantity of the free-surface mass budget). */
int lbdem_mass_total(lbdem_ctx* ctx, double* total_mass);

/* ---- checkpoint / restore -------------------------------------------- */

/* Write a snapshot of the whole run to `path`: every device buffer at full
 * precision (lattice, interface masses, particle and impactor state,
 * neighbour lists, tangential springs, the free-surface budget) and the
 * step counters. Synchronises the context's stream first, so everything
 * enqueued before the call is part of the snapshot.
 * Replaces the reference's resume files IO::exportRecycleFluid
 * (src/IO.cpp:973-997) and IO::exportRecycleParticles (src/IO.cpp:999),
 * which keep six significant digits and neither the neighbour lists, the
 * springs nor the counters. Returns LBDEM_ERR_IO if the file cannot be
 * written. */
int lbdem_checkpoint(lbdem_ctx* ctx, const char* path);

/* Load a snapshot written by lbdem_checkpoint into `ctx`, which must have
 * been created from the same configuration in the same form: the snapshot
 * replaces its whole state and its step counters, and the next step
 * continues the snapshotted run. Replaces the reference's restart read
 * (LB::restartInterface / LB::restartVariables, src/LB.cpp:994-1138, under
 * lbRestart). A snapshot of another lattice size, particle, impactor or
 * wall count, form, library build, or a truncated file is refused with
 * LBDEM_ERR_INVALID or LBDEM_ERR_IO before any state is changed. */
int lbdem_restore(lbdem_ctx* ctx, const char* path);

/* ---- the reference's fluid recycle file ------------------------------- */

/* Write the reference's fluid recycle file (IO::exportRecycleFluid,
 * src/IO.cpp:973-997) of the run's current state: the lattice size, the
 * type of every node, and per fluid or interface node in index order its
 * density and mass less the initial density, velocity, viscosity and 19
 * populations, with the reference's six significant digits. The density
 * and velocity are those of the current populations (the reference writes
 * the values of the last collision, with the force shift); restarts read
 * neither. Synchronises
 * the context's stream. A run created with lbRestart = 1 and
 * lbRestartFile = this file starts from it as the reference's restart does
 * (LB::restartInterface / restartVariables, src/LB.cpp:994-1138). */
int lbdem_export_recycle_fluid(lbdem_ctx* ctx, const char* path);

/* ---- the reference's screen-phase output files ------------------------ */

/* Open the reference's screen-phase files in directory `dir` (which must
 * exist; its particleData and fluidData folders are created) and append
 * their header lines as IO::initialize does
 * (src/IO.cpp:43-94): export.dat and, with the DEM on, objPosition.dat,
 * objForce.dat, wallForce.dat, bodyPosition.dat and the three stress files.
 * From then on lbdem_cycle appends the lines IO::outputStep writes
 * (src/IO.cpp:113-158) at every cycle where the reference's screen counter
 * (unsigned)(realTime / screen_exp_time) + 1 advances, realTime being the
 * sum of unitTime over the cycles; a run opened before its first cycle
 * also gets the line the reference writes before the first goCycle
 * (src/main.cpp:286). Same numbers and layout as the reference: "%g",
 * vectors as "x y z ", tab-separated groups. Lines are formatted from
 * copies taken on the context's stream into pinned memory, without
 * synchronising it; lbdem_sync and lbdem_output_close write all pending
 * lines. The stress files carry DEM::evaluateForces' stress sums of the
 * cycle, formed on the output cycles only. screen_exp_time 0 writes headers
 * only.
 * Only lbdem_cycle advances the output clock; the four single-step entry
 * points do not. */
int lbdem_output_open(lbdem_ctx* ctx, const char* dir, double screen_exp_time);
/* With output open, also write the reference's recycle files
 * (IO::createFiles, src/IO.cpp:201-210, 268-274): dir/fluidData/
 * fluidRecycle%010u.dat named by the cycle, at every cycle where
 * (unsigned)(realTime / fluid_recycle_exp_time) + 1 advances (each is
 * lbdem_export_recycle_fluid), and dir/particleData/partRecycle%04u.dat
 * named by its counter, at every cycle where the part_recycle_exp_time
 * counter advances (IO::exportRecycleParticles: radius, position,
 * velocity, negated total stresslet and vertical displacement); both also
 * now for a run that has not cycled yet. Each file synchronises the
 * stream. 0 turns either off. */
int lbdem_output_recycle(lbdem_ctx* ctx, double fluid_recycle_exp_time,
                         double part_recycle_exp_time);
/* Write every pending line and close the files (also done by
 * lbdem_destroy). */
int lbdem_output_close(lbdem_ctx* ctx);

/* ---- measurement (no counterpart in the reference) --------------------- */

typedef struct lbdem_profile {
  double lb_kernel_ms;          /* summed CUDA-event time of the main lattice
                                   kernel over the profiled launches        */
  int64_t lb_kernel_launches;   /* profiled launches of that kernel         */
  int64_t kernel_launches;      /* all kernels this context launched        */
  int64_t active_node_updates;  /* active nodes collided and streamed       */
  double phase_ms[4];           /* CUDA-event time of the profiled cycles'
                                   DEM, coupling, lattice and free-surface
                                   steps (lbdem_cycle only)                 */
} lbdem_profile;
/* Record CUDA events around every main lattice kernel launch (on the
 * context's stream) while enabled. */
int lbdem_profile_enable(lbdem_ctx* ctx, int enable);
/* Synchronise, report the counters since the last reset, optionally reset. */
int lbdem_profile_read(lbdem_ctx* ctx, lbdem_profile* out, int reset);

/* ---- many runs on one GPU (no counterpart in the reference: a serving
 * layer of this library) ------------------------------------------------- */

/* Device bytes lbdem_create would allocate for cfg in the given form. */
int lbdem_estimate_device_bytes(const lbdem_config* cfg, int32_t precision,
                                int64_t* bytes);

typedef struct lbdem_server lbdem_server;
typedef struct lbdem_server_options {
  int32_t device;
  int32_t precision;      /* LBDEM_PLAIN_FP64 or LBDEM_MIXED for every run */
  int32_t max_active;     /* runs resident at once                         */
  int32_t slice_cycles;   /* goCycles enqueued per run per turn            */
  int64_t device_budget_bytes; /* 0: 90 % of the free memory at creation   */
  int32_t batch_runs;     /* 0: every run on its own stream; N > 0: runs in
                             their steady cycle share launches in groups of
                             up to N, each group on its own stream          */
  int32_t chunks_per_block; /* passed to every run (lbdem_options)         */
  int32_t reserved[4];
} lbdem_server_options;

typedef struct lbdem_job_result {
  int64_t job_id;
  int32_t status;         /* LBDEM_OK or the failing call's status         */
  int32_t cycles;         /* goCycles run (for a failed run: up to the end of
                             the slice whose error bits showed the failure) */
  double submit_time, start_time, end_time; /* s since lbdem_server_create */
  double impactor_x0[3], impactor_x1[3];    /* object 0 at the end         */
  double fluid_mass;      /* as lbdem_mass_summary                         */
  int64_t active_node_updates;
  int64_t device_bytes;   /* the run's footprint estimate                  */
  int32_t batched_cycles; /* cycles run in launches shared with other runs */
  int32_t reserved;
} lbdem_job_result;

/* Jobs queue in submission order. A job is admitted when its footprint fits
 * the budget next to the runs in progress and fewer than max_active runs
 * are resident. Each admitted job is a context with its own stream, and
 * lbdem_server_poll advances every resident run by slice_cycles goCycles
 * per turn, each run's steady cycles replayed from its own CUDA graphs on its
 * own stream. With batch_runs > 0, runs in their steady cycle with the same
 * switches (free surface, impactor, walls) are advanced in batch groups of
 * up to batch_runs runs instead: one launch per kernel for all runs of a
 * group (grid z = run), the pair of cycles captured in a CUDA graph that is
 * rebuilt when the group's runs change, each group on its own stream. Set
 * CUDA_DEVICE_MAX_CONNECTIONS (for example 32) before the first CUDA call
 * when more than 8 streams are to run concurrently. A finished run frees its memory for the
 * next job. Each run's device error bits are read back after every slice: a
 * run that diverged (LBDEM_ERR_NONFINITE, a sphere out of the domain:
 * LBDEM_ERR_DEVICE_STATE) or overflowed a list ends at that slice with its
 * status, and lbdem_server_last_error describes it. The server's calls must
 * come from one host thread. */
int lbdem_server_create(const lbdem_server_options* opt, lbdem_server** out);
/* Queue a run of `cycles` goCycles; the configuration and its tables are
 * copied. A run larger than the whole budget is refused (LBDEM_ERR_OOM). */
int lbdem_server_submit(lbdem_server* s, const lbdem_config* cfg, int32_t cycles,
                        int64_t* job_id);
/* Admit and advance runs for up to wait_seconds, or until a run finishes
 * or nothing is left; hand back up to max_out finished runs. */
int lbdem_server_poll(lbdem_server* s, double wait_seconds, lbdem_job_result* out,
                      int32_t max_out, int32_t* n_out);
int lbdem_server_status(const lbdem_server* s, int32_t* queued, int32_t* running,
                        int32_t* unread, int64_t* device_bytes_in_use);
/* The server's last error message; with s = NULL, the message of this
 * thread's last failed lbdem_server_tune (the schedule and the failing run). */
const char* lbdem_server_last_error(const lbdem_server* s);
/* Ends the runs still resident (without results) and frees everything. */
void lbdem_server_destroy(lbdem_server* s);
/* Autotuner: runs the n sample configurations for `cycles` goCycles under
 * each candidate schedule (batch_runs 0, 2, 4, 8 x chunks_per_block 8, 32)
 * with the other fields of *opt, and writes the fastest schedule into
 * opt->batch_runs and opt->chunks_per_block; *best_seconds (optional) gets
 * its time. Runs on the device of opt. */
int lbdem_server_tune(lbdem_server_options* opt, const lbdem_config* const* cfgs, int32_t n,
                      int32_t cycles, double* best_seconds);

/* ---- readback without device allocation (no counterpart in the
 * reference; a diagnostic of this library) ------------------------------ */

/* Largest node range one lbdem_download_nodes_noalloc call accepts. */
#define LBDEM_NOALLOC_MAX_NODES 16384

/* Populations and mass of the `count` consecutive nodes starting at node
 * index `first` (index = x + y*X + z*X*Y): f[19*count] (direction blocks of
 * `count`), mass[count]; the same values lbdem_download_lattice returns for
 * those nodes. Either pointer may be NULL.
 *
 * Allocates no device memory (no cudaMalloc/cudaFree): it stages through a
 * fixed buffer of LBDEM_NOALLOC_MAX_NODES nodes (2.5 MiB) compiled into the
 * library. For callers that cannot allocate device memory at the time of the
 * call, e.g. a monitor sampling lattice rows every step while the run holds
 * nearly all of HBM: lbdem_download_lattice takes a temporary of 160 bytes
 * per lattice node with cudaMalloc, which also synchronises the device.
 * count > LBDEM_NOALLOC_MAX_NODES or a range outside the lattice returns
 * LBDEM_ERR_INVALID with a message in lbdem_last_error.
 *
 * The buffer is shared by every context on a device: calls that overlap in
 * time on one device race on it; serialise them. The first call on each
 * device looks up the buffer's address (cudaGetSymbolAddress); make that
 * first call before any stream capture. Synchronises the context's stream
 * and makes the context's device current for the call. Unlike
 * lbdem_download_lattice it does not return the run's device error: after a
 * step reported a fault (LBDEM_ERR_NONFINITE, LBDEM_ERR_OVERFLOW, ...) the
 * nodes can still be read, to inspect the state at the fault. */
int lbdem_download_nodes_noalloc(lbdem_ctx* ctx, int64_t first, int64_t count,
                                 double* f, double* mass);

/* Number of device allocations (cudaMalloc, cudaMallocAsync) this library
 * has made in the process so far, over all contexts and servers. A
 * diagnostic: a caller checks with it that a stretch of calls allocated
 * nothing on the device. */
int64_t lbdem_device_allocations(void);

#ifdef __cplusplus
}
#endif
#endif /* LBDEM_H */
