/*
 * sph_gb300 -- C ABI of the GB300 (sm_103a) SPH substep library.
 *
 * Drop-in for the per-substep SPH pipeline of Allkams/Fluid-Simulation-3D
 * (engine/physics/physicsWorld.cc): spatial-hash build, density and near
 * density, pressure + near pressure + viscosity, integrate with box
 * collision. The library owns all device memory; host pointers passed in are
 * caller-owned and only read/written during the call -- except page-locked
 * (pinned) input arrays, which the upload calls read asynchronously on the
 * stream, as cudaMemcpyAsync does (see sph_upload). Every call returns an
 * int status (SPH_OK = 0); sph_last_error() gives the message of the last
 * failure on a handle. A handle is used from one host thread and enqueues its
 * work on the caller's CUDA stream (passed as a plain pointer, NULL = the
 * legacy default stream). There is no CPU fallback: without a usable CUDA
 * device every compute call returns SPH_ERR_CUDA.
 *
 * Particle arrays on the host side are AoS float[3*n] in the caller's
 * particle order (the reference's `positions` / `velocity` index order,
 * physicsWorld.h:79,119).
 */
#ifndef SPH_GB300_H
#define SPH_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPH_OK 0
#define SPH_ERR_INVALID -1   /* bad argument or size                      */
#define SPH_ERR_CUDA -2      /* CUDA runtime error / no device            */
#define SPH_ERR_NOMEM -3     /* device allocation or budget exhausted     */
#define SPH_ERR_STATE -4     /* call not valid in the handle's state      */
#define SPH_ERR_DEVICE -5    /* reserved: no call returns it; kernel
                                status flags are read with sph_status and
                                sph_batch_status                          */

/* Device status flags (sph_status). */
#define SPH_STATUS_NONFINITE 0x1u  /* a position/velocity became NaN/inf   */
#define SPH_STATUS_RANGE 0x2u      /* an index fell outside its buffer     */

/* Settings surface of Physics::Fluid::FluidSimulation
 * (engine/physics/physicsWorld.h:96-106,145) plus the two constants the
 * reference hard-codes: collision damping 0.95 (physicsWorld.cc:87) and the
 * 1/120 s prediction look-ahead (physicsWorld.cc:47). */
typedef struct sph_params {
  float radius;             /* interactionRadius,  default 0.35          */
  float cutoff_sq;          /* sqrRadius, default 0.35f*0.35f (the
                               reference never updates it, :234-237)     */
  float target_density;     /* TargetDensity,      default 99.7          */
  float pressure_mult;      /* pressureMultiplier, default 300           */
  float near_pressure_mult; /* nearPressureMultiplier, default 20        */
  float viscosity;          /* viscosityStrength,  default 0.5           */
  float gravity_scale;      /* gravityScale,       default 10            */
  int32_t gravity_on;       /* gravity,            default 0 (off)       */
  float bound[3];           /* BoundScale,         default 20,20,20      */
  float damping;            /* collision damping,  default 0.95          */
  float predict_dt;         /* prediction look-ahead, default 1/120      */
} sph_params;

typedef struct sph_sim sph_sim;

/* Launch configuration of the neighbour kernels, chosen by the autotuner
 * (sph_autotune / sph_batch_autotune) by timing real steps. */
typedef struct sph_tuning {
  int32_t block;      /* threads per block of the neighbour kernels
                         (multiple of 32, 32..1024), default 128          */
  int32_t cell_tile;  /* density kernel: 1 = one lane per particle walking
                         its cell's runs (default); 64, 128, 192 or 256 =
                         warp-cooperative form holding that many candidates
                         of a cell in registers per pass                  */
  int32_t particles_per_warp; /* pressure and viscosity kernels: 32 (one
                         lane per particle, default) or 16 (two lanes per
                         particle, each summing every other neighbour of
                         its list; agrees with 32 to rounding)            */
  int32_t gather;     /* neighbour-list entries whose gathers the force
                         kernels issue together: 2, 3, 4 or 8 (default 2) */
  int32_t force_block; /* threads per block of the pressure and viscosity
                          kernels (multiple of 32, 32..1024); 0 = block   */
  int32_t table;      /* key table of the sort: 0 = one entry per cell of
                         the scene's grid where the grid has at most four
                         cells per particle, else n entries (cell index
                         mod n); 1 = n entries for every scene; 2 = as 0,
                         and grid tables for larger grids too while an
                         allowance of 65,536 extra entries lasts (scenes
                         in layout order). Results agree to rounding; they
                         are bit-identical unless a predicted position lies
                         more than one cell beyond the box (or the box
                         spans more than 32,764 cells along an axis)      */
} sph_tuning;

/* Reference defaults of physicsWorld.h:96-106,145 and physicsWorld.cc:47,87. */
void sph_default_params(sph_params *out);

/* Create a single-scene simulation of n particles (replaces
 * FluidSimulation::getInstance + InitializeData, physicsWorld.cc:32-37,
 * 112-147; the lattice layout is left to the caller: state is zero until
 * sph_upload). n must be in [1, 2^24) -- the reference stores particle
 * indices as floats (physicsWorld.h:128). */
int sph_create(const sph_params *params, uint32_t n, sph_sim **out);
int sph_destroy(sph_sim *sim);

/* Settings setters/getters (physicsWorld.cc:214-302). Take effect at the
 * next sph_step. */
int sph_set_params(sph_sim *sim, const sph_params *params);
int sph_get_params(const sph_sim *sim, sph_params *out);
uint32_t sph_num_particles(const sph_sim *sim);

/* Load positions / velocities (host, float[3n]; vel may be NULL = zero).
 * Replaces writing the public `positions` buffer (physicsWorld.h:79).
 * Pageable arrays are copied before the call returns. Page-locked arrays
 * (cudaHostAlloc, or registered) are read when `stream` reaches the call --
 * 16-byte aligned ones by the import kernel itself, over the host link --
 * so keep them unchanged until then (a later sph_download on the same
 * stream has passed it). */
int sph_upload(sph_sim *sim, const float *pos3, const float *vel3,
               void *stream);

/* Advance by dt split into `substeps` equal substeps: each substep is one
 * reference FluidSimulation::Update(dt / substeps) (physicsWorld.cc:39-111)
 * with Jacobi viscosity (every particle reads the post-pressure velocity
 * snapshot). Asynchronous on `stream`. */
int sph_step(sph_sim *sim, float dt, int substeps, void *stream);

/* Read back state in the caller's particle order (host pointers; any may be
 * NULL): pos3/vel3 float[3n], dens2 float[2n] (density, near density of the
 * last substep, getDensity/getNearDensity physicsWorld.cc:161-170).
 * Page-locked outputs that are all 16-byte aligned are written by the device
 * directly over the host link; other memory goes through device staging and
 * copies. Synchronises `stream`. */
int sph_download(sph_sim *sim, float *pos3, float *vel3, float *dens2,
                 void *stream);

/* Snapshots: the state (positions, velocities, densities, in the caller's
 * order) and settings (sph_params and the step dt) of a scene in a binary
 * file, for checkpoint / resume (the reference has no state I/O). The file
 * is little-endian, 80 header bytes + 32 bytes per particle, with a
 * checksum; a loaded scene continues bit for bit as if it had never been
 * saved. sph_load needs a file of the handle's particle count and replaces
 * its settings and state. Both synchronise `stream`. */
int sph_save(sph_sim *sim, const char *path, void *stream);
int sph_load(sph_sim *sim, const char *path, void *stream);

/* Headless render (replaces FluidSimCPU::render and updateColors,
 * projects/Simulation/code/simulations/fluidSimCPU.cc:53-124, with the
 * billboard shaders bin/shaders/particleRender.vs/.fs): every particle is a
 * screen-aligned splat of size `scale` coloured by its speed, depth-tested
 * with GL_LESS, into an RGBA8 image and its window depth. */
typedef struct sph_view {
  float view_proj[16]; /* cam.GetViewProjection() = P * V, column-major (glm) */
  float proj[16];      /* cam.GetProjection(): columns 0 and 1 must be
                          (a, 0, 0, 0) and (0, b, 0, 0) with a, b > 0, as
                          glm::perspective / glm::ortho give              */
  uint32_t width;      /* viewport in pixels, width * height <= 2^28      */
  uint32_t height;
  float scale;         /* billboard size: OutPositions.w = 0.34           */
  float clear[4];      /* glClearColor, the app uses (0, 0, 0, 1)         */
} sph_view;

/* Render the current state. rgba: uint8[4 * width * height], depth:
 * float[width * height] in [0, 1] (1 where no particle), rows bottom to
 * top as glReadPixels returns them; host pointers, either may be NULL.
 * Synchronises `stream`. */
int sph_render(sph_sim *sim, const sph_view *view, uint8_t *rgba, float *depth,
               void *stream);

/* Device pointer to the headless OutPositions buffer (physicsWorld.h:80):
 * float4[n] = (position, 0.34) in the caller's order, refreshed by every
 * sph_step. Valid until sph_destroy. */
int sph_out_positions(sph_sim *sim, void **dev_float4);

/* Same as sph_step/sph_upload/sph_download but with device pointers
 * (float[3n] on the handle's device) -- no host copies. */
int sph_upload_device(sph_sim *sim, const float *dpos3, const float *dvel3,
                      void *stream);
int sph_download_device(sph_sim *sim, float *dpos3, float *dvel3,
                        float *ddens2, void *stream);

/* Parity capture: when enabled, the FIRST substep of the next sph_step
 * records the intermediates of the reference's phases. sph_debug_export then
 * returns them (host pointers, any may be NULL):
 *   hash[n], key[n]    -- HashCell / GetKeyFromHash of each particle
 *                         (physicsWorld.cc:505-516), caller order;
 *   sorted_ids[n]      -- spatialLookup order, canonical (key, index);
 *   start[n]           -- startIndices (0x7fffffff = empty key);
 *   dens2[2n]          -- density, near density;
 *   acc_p3[3n]         -- pressureForce / density (physicsWorld.cc:421);
 *   vel_p3[3n]         -- velocity after the pressure pass;
 *   vel_v3[3n]         -- velocity after the viscosity pass (pre-collision).
 * Synchronises `stream`. */
int sph_debug_enable(sph_sim *sim, int enable);
int sph_debug_export(sph_sim *sim, uint32_t *hash, uint32_t *key,
                     uint32_t *sorted_ids, uint32_t *start, float *dens2,
                     float *acc_p3, float *vel_p3, float *vel_v3,
                     void *stream);

/* The timed path's own spatial sort of the same captured substep (the
 * layout every kernel of a substep reads; it replaces UpdateSpatialLookup,
 * physicsWorld.cc:466-498, whose reference order sph_debug_export gives).
 * Particles are sorted by an internal cell index: with the cell coordinates
 * c = floor(pred / radius) and a grid of (gnx, gny, gnz) cells around the
 * box, cell = cx' + cy' * gnx + cz' * gnx * gny (mod 2^32), where c' is c
 * clamped to the grid (grid key table, one entry per cell: key = cell) or
 * c minus the grid origin (bucket table, n entries: key = cell mod n). The
 * order is stable by (key, cell, caller index), and start[k] is the slot of
 * the first particle with key >= k (exclusive prefix of the key counts),
 * start[table_len] = n. Outputs (host pointers, any may be NULL):
 *   cell[n], key[n]   -- per particle, caller order;
 *   slot_ids[n]       -- the caller index of the particle at each slot;
 *   start[table_len+1] -- copied only when start_cap >= table_len + 1;
 *   table_len, direct -- table entries, 1 for a grid table (0: buckets).
 * Synchronises `stream`. */
int sph_debug_export_layout(sph_sim *sim, uint32_t *cell, uint32_t *key,
                            uint32_t *slot_ids, uint32_t *start,
                            uint64_t start_cap, uint32_t *table_len,
                            int *direct, void *stream);

/* Device status flags OR-ed by kernels since the last call (cleared by the
 * read). Synchronises `stream`. */
int sph_status(sph_sim *sim, uint32_t *flags, void *stream);

/* Per-phase device timing (replaces getElapsedTime{Gravity,Spatial,Density,
 * Pressure,Viscosity,PosNColl}, physicsWorld.h:45-50, whose values are
 * host-clock ms of the last Update). When enabled, every sph_step records
 * CUDA events on its stream between the phases; sph_phase_times returns the
 * last step's ms per phase summed over its substeps, in that order
 * (integration runs inside the viscosity kernel, so PosNColl is 0).
 * Synchronises on the last event. */
int sph_profile_enable(sph_sim *sim, int enable);
int sph_phase_times(sph_sim *sim, double out_ms[6]);

/* Kernel launch configuration of a single-scene handle, and its autotuner:
 * times real steps of dt/substeps (steps_per_trial per candidate, after one
 * untimed step) over the neighbour block size x cell tile, then the force
 * kernels' block size, then their particles per warp x gather batch; keeps
 * the fastest and reports
 * it (best may be NULL) with its ms per step. The state (positions,
 * velocities, densities, OutPositions) is saved before the sweep and
 * restored after it. */
int sph_set_tuning(sph_sim *sim, const sph_tuning *t);
int sph_get_tuning(const sph_sim *sim, sph_tuning *t);
int sph_autotune(sph_sim *sim, float dt, int substeps, int steps_per_trial,
                 sph_tuning *best, float *best_ms, void *stream);

/* Number of this library's kernels the handle has launched so far
 * (including those replayed from captured graphs). */
uint64_t sph_kernel_launches(const sph_sim *sim);

/* Message of the last failed call on this handle ("" if none). */
const char *sph_last_error(const sph_sim *sim);

/* Message of the last failed sph_create / batch create (no handle yet). */
const char *sph_global_error(void);

/* ------------------------------------------------------------------------
 * Spatial lookup without device allocation. No counterpart in the
 * reference: this is an extra entry point for callers that cannot allocate
 * device memory -- a render loop that must not stall a frame on cudaMalloc's
 * device-wide synchronisation, an engine that owns a fixed memory pool and
 * forbids plug-ins to allocate.
 *
 * Builds, for n predicted positions (device float[3n], the caller's
 * buffers), the same lookup as the main path: hash[n] and key[n] = hash % n
 * per particle, sorted_ids[n] in (key, index) order and start[n]
 * (0x7fffffff for an empty key) -- all device buffers of the caller. The
 * working memory is one array inside the library of 8 B per particle for
 * at most SPH_STATIC_LOOKUP_MAX particles (512 KiB, held on every GPU that
 * loads the library until the process exits); larger n is rejected with
 * SPH_ERR_INVALID. The work is linear in n whatever the keys (particles
 * that all share one key included). Nothing is allocated: no cudaMalloc/cudaFree or
 * allocating library call. The first call on a device resolves that array's
 * address (cudaGetSymbolAddress) with the device current, so make the first
 * call on each device before any stream capture. Each device has its own
 * copy of the array and every call on that device shares it, keeping the
 * last call's contents (each call clears what must start at zero): two calls
 * whose work overlaps on the same GPU, e.g. on different streams, race, so
 * serialise them (one stream does). Asynchronous on `stream`; the message of
 * the last failure is sph_static_error(). */
#define SPH_STATIC_LOOKUP_MAX 65536u
int sph_spatial_lookup_static(const float *dpred3, uint32_t n, float radius,
                              uint32_t *dhash, uint32_t *dkey,
                              uint32_t *dsorted_ids, uint32_t *dstart,
                              void *stream);
const char *sph_static_error(void);

/* ------------------------------------------------------------------------
 * Batched form: many independent scenes of uneven sizes advanced together.
 * Each kernel of a substep is one segmented, persistent launch over all
 * scenes; a whole step is captured once in a CUDA graph and replayed.
 * Scenes keep their own settings, table (key = hash % n_scene) and dt.
 * ---------------------------------------------------------------------- */
typedef struct sph_batch sph_batch;

/* capacity: total particles resident at once (device memory is sized for
 * it); max_scenes: scene slots. */
int sph_batch_create(uint64_t capacity, uint32_t max_scenes, sph_batch **out);
int sph_batch_destroy(sph_batch *b);

/* Add a scene (host arrays float[3n]; vel may be NULL). Becomes part of the
 * next sph_batch_step. Returns its id in *scene_id. Fails with SPH_ERR_NOMEM
 * when it does not fit the capacity. */
int sph_batch_add(sph_batch *b, const sph_params *params, uint32_t n,
                  const float *pos3, const float *vel3, float dt,
                  uint32_t *scene_id, void *stream);

/* Remove a scene (its slot and particles are released at the next step). */
int sph_batch_remove(sph_batch *b, uint32_t scene_id);

/* Wait until the work queued on `stream` (and the batch's own stream) has
 * finished. */
int sph_batch_sync(sph_batch *b, void *stream);

/* Advance every resident scene by one step of `substeps` substeps of its own
 * dt / substeps. */
int sph_batch_step(sph_batch *b, int substeps, void *stream);

/* Device status flags (SPH_STATUS_*) OR-ed by the batch's kernels since the
 * last call, over every scene (cleared by the read). Synchronises `stream`. */
int sph_batch_status(sph_batch *b, uint32_t *flags, void *stream);

/* Read one scene back (host pointers, caller order, any may be NULL).
 * Synchronises `stream`. */
int sph_batch_download(sph_batch *b, uint32_t scene_id, float *pos3,
                       float *vel3, float *dens2, void *stream);

/* Snapshot one scene of the batch to a file, or add a saved scene to the
 * batch (SPH_ERR_NOMEM when it does not fit). */
int sph_batch_save(sph_batch *b, uint32_t scene_id, const char *path, void *stream);
int sph_batch_add_snapshot(sph_batch *b, const char *path, uint32_t *scene_id,
                           void *stream);

/* sph_render for one scene of the batch. */
int sph_batch_render(sph_batch *b, uint32_t scene_id, const sph_view *view,
                     uint8_t *rgba, float *depth, void *stream);

/* Launch configuration of the batch's neighbour kernels and its autotuner
 * (see sph_tuning above). */
int sph_batch_set_tuning(sph_batch *b, const sph_tuning *t);
int sph_batch_get_tuning(const sph_batch *b, sph_tuning *t);
/* Sweep the tuning space on the resident scenes as sph_autotune does (real
 * steps; every scene's state is saved before and restored after), keep the
 * fastest and report it in *best (may be NULL) and its ms per step in
 * *best_ms. */
int sph_batch_autotune(sph_batch *b, int substeps, int steps_per_trial,
                       sph_tuning *best, float *best_ms, void *stream);

/* Native serving loop (the served form): continuous batching of scene jobs
 * on a worker thread over one batch engine whose capacity is
 * budget_bytes / sph_bytes_per_particle(). Jobs are admitted in submission
 * order while the budget has room (smaller later jobs may backfill); every
 * resident job advances one step of dt (in `substeps` substeps, one count
 * per server) per batched launch; a job leaves after its `steps` steps with
 * its state read back. Results equal the job run alone, bit for bit.
 * submit / cancel / wait / stats may be called from any thread; call
 * destroy only when no other thread is inside a server call. */
typedef struct sph_server sph_server;
typedef struct sph_server_stats {
  uint64_t submitted, completed, cancelled, failed;
  uint32_t queued, resident;     /* jobs waiting / on the device now        */
  uint64_t steps;                /* batched steps run                       */
  uint64_t particle_steps;       /* sum over steps of resident particles    */
  uint64_t capacity_particles;
  double wall_s;                 /* first admission to the end of the last step */
  double particle_steps_per_s;
  double p50_step_ms, p99_step_ms; /* per-step wall clock as the jobs see it:
                                    every step weighted by the jobs it
                                    advanced; from a fixed log histogram of
                                    0.5%-wide bins (within 0.25%)            */
  double step_s;   /* worker seconds from each step's launch to its end
                      (the admission uploads of the round overlap it)     */
  double admit_s;  /* of which: staging and queueing admitted jobs' inputs */
  double retire_s; /* worker seconds reading finished jobs back           */
  uint32_t status_flags; /* device status flags (SPH_STATUS_*) raised by any
                            step so far, read after every step            */
} sph_server_stats;

int sph_server_create(uint64_t budget_bytes, uint32_t max_scenes, int substeps,
                      sph_server **out);
int sph_server_destroy(sph_server *s);
/* Copies the job's inputs (pos3, vel3 float[3n]; vel3 may be NULL); a job
 * larger than the whole capacity is refused with SPH_ERR_NOMEM. */
int sph_server_submit(sph_server *s, const sph_params *params, uint32_t n,
                      const float *pos3, const float *vel3, float dt,
                      uint32_t steps, uint64_t *job_id);
/* A queued job is dropped at once, a resident one at the next step
 * boundary; its wait returns SPH_ERR_STATE. */
int sph_server_cancel(sph_server *s, uint64_t job_id);
/* Blocks up to timeout_s for the job, then copies its result (host
 * pointers, any may be NULL) and forgets it. SPH_ERR_STATE: still running
 * after the timeout (wait again), or cancelled; other codes: the job
 * failed (sph_server_last_error says why). */
int sph_server_wait(sph_server *s, uint64_t job_id, float *pos3, float *vel3,
                    float *dens2, double timeout_s);
int sph_server_get_stats(sph_server *s, sph_server_stats *out);
const char *sph_server_last_error(sph_server *s);

/* Device bytes an engine allocates per particle of capacity (state, sort,
 * cell tables, neighbour lists): admission by an HBM budget divides by it. */
uint64_t sph_bytes_per_particle(void);

uint32_t sph_batch_num_scenes(const sph_batch *b);
uint64_t sph_batch_num_particles(const sph_batch *b);
uint64_t sph_batch_kernel_launches(const sph_batch *b);
int sph_batch_profile_enable(sph_batch *b, int enable);
int sph_batch_phase_times(sph_batch *b, double out_ms[6]);
const char *sph_batch_last_error(const sph_batch *b);

#ifdef __cplusplus
}
#endif
#endif
