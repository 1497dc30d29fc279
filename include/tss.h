/*
 * tss.h -- C ABI of the GB300-native two-scale WCSPH solver.
 *
 * The surface mirrors the reference's WCSPHConfig / ParticleSystem / WCSPHSolver
 * classes (TwoScale2D/WCSPHSolver.h:14-131, TwoScale2D/ParticleSystem.h:17-86):
 * build a configuration, construct a solver from particle arrays, advance steps,
 * and read device buffers for an (optional) renderer.  Every entry point returns a
 * tss_status; no C++ exception crosses this boundary.  Host arrays passed in are
 * copied; the solver owns all device memory it allocates.
 *
 * Threading: one solver handle per host thread; handles share no state.
 */
#ifndef TSS_H
#define TSS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The reference threw std::runtime_error (stdutil.h:22-33,
 * CUDA/cuda.h:37-51) and printed + paused in CheckLastError (cuda.h:24-35). */
typedef enum tss_status {
    TSS_OK = 0,
    TSS_INVALID_ARG = 1,   /* bad argument or configuration                      */
    TSS_OOM = 2,           /* device or host allocation failed                    */
    TSS_CUDA_ERROR = 3,    /* a CUDA runtime call failed                          */
    TSS_CAPACITY = 4,      /* a particle pool would overflow its capacity         */
    TSS_NUMERIC = 5,       /* NaN/Inf in a density, pressure or acceleration      */
    TSS_GRID_INDEX = 6,    /* a grid index check failed: inconsistent cell offsets */
                           /* (the affected entries were skipped, nothing written  */
                           /* outside a buffer)                                    */
    TSS_NO_DEVICE = 7      /* no CUDA device                                      */
} tss_status;

/* Configuration flags. */
#define TSS_FLAG_Q1_COMPAT 0x1u
/* TSS_FLAG_Q1_COMPAT: compute the high-res density's low-res term the way the
 * reference does (TwoScale2D/WCSPHSolver.cu:1483-1510): it iterates the HIGH-res
 * sorted list over LOW-grid cell ranges (including the never-written identity
 * tail of that list) and accumulates into the high-res sum, while the low-res
 * term stays zero.  Without the flag the term uses the low-res particles, as the
 * kernel's parameter list intends. */
#define TSS_FLAG_TETHER_GUARD 0x4u
/* TSS_FLAG_TETHER_GUARD: the tether (adjustPosition, WCSPHSolver.cu:1007-1022)
 * scales the child-parent offset by lim / dist; a child that lands exactly on its
 * parent (dist == 0) gets 0/0 = NaN there.  With the flag such a child keeps its
 * position (the formula's limit: for dist below the tether radius it leaves the
 * child where it is).  Off by default: the reference's arithmetic. */
#define TSS_FLAG_OLDER_PLACEMENT 0x8u
/* TSS_FLAG_OLDER_PLACEMENT: place a split parent's four children as the reference's
 * older snapshot does (TwoScale2D-master/TwoScale2D/WCSPHSolver.cu:840-850): at the
 * predicted position +-DIR_LEN * r on both diagonals, DIR_LEN = 0.35355339 (so each
 * child sits r/2 from its parent), instead of the current tree's
 * +-0.5*sqrt(m/(2 rho pi)) (WCSPHSolver.cu:956-1005).  The older snapshot relaxes
 * the children so placed before they couple (relax_iters = 4); the current tree's
 * placement puts them so close to their parent that the relaxation's first
 * sub-step finds them at 2-3 rest densities.  The tether, the parent's place in the
 * low-res list and the coupling stay the current tree's. */
#define TSS_FLAG_MERGE 0x2u
/* TSS_FLAG_MERGE: a split parent (low-res state 1) whose predicted position is
 * outside the region of interest returns to state 0, and its four children are
 * removed: they are marked state 2 ("deleted", WCSPHSolver.h:105) in that step's
 * output and dropped by the next grid build.  The reference has no live removal
 * (its stub, WCSPHSolver.cu:1053-1095, is under `if (false)`); this rule is this
 * library's.  Mass m*#(low state 0) + m_high*#(high) is conserved exactly. */

/* Solver parameters.  Mirrors WCSPHConfig (TwoScale2D/WCSPHSolver.h:14-35) plus the
 * constants the reference hard-codes (gravity 9.81: WCSPHSolver.cu:1805,2012; split
 * half-plane x > 0.5: WCSPHSolver.cu:1835; relax 4 x dt/10:
 * TwoScale2D-master/TwoScale2D/WCSPHSolver.cu:2380-2446). */
typedef struct tss_config {
    float domain_origin[2];
    float domain_end[2];
    int   dims_low[2];        /* ceil((end - origin) / r_low)   (WCSPHSolver.cu:2323-2326) */
    int   dims_high[2];       /* ceil((end - origin) / r_high)  (WCSPHSolver.cu:2328-2331) */
    float r_low;              /* EffectiveRadius: support radius of the low-res scale      */
    float r_high;             /* EffectiveRadiusHigh                                        */
                              /* both in [2^-40, 2^40], else TSS_INVALID_ARG at creation    */
    float rest_density;
    float tait_b;             /* Tait coefficient B in p = B((rho/rho0)^7 - 1)              */
    float speed_sound;
    float alpha;              /* artificial viscosity                                       */
    float tension;            /* "tension" coefficient sigma                                */
    float dt;
    float gravity;            /* subtracted from a_y; the reference hard-codes 9.81f        */
    float roi[4];             /* split region x0,y0,x1,y1: open rectangle on the predicted  */
                              /* position; {0.5,-inf,inf,inf} is the reference's x > 0.5    */
    int   relax_iters;        /* relaxation sub-steps for newly created high-res particles  */
                              /* (0 = the current reference tree, 4 = its older snapshot)   */
    float relax_dt_div;       /* relaxation sub-step = dt / relax_dt_div (10 in reference)  */
    unsigned flags;           /* TSS_FLAG_*                                                 */
    float roi_velocity[2];    /* the ROI translates: at a scene's step k (from 0) it is     */
                              /* roi + k * (roi_velocity * dt), in FP32; {0,0} = fixed      */
} tss_config;

/* Fill *cfg like WCSPHConfig::WCSPHConfig (TwoScale2D/WCSPHSolver.cu:2287-2332):
 * rejects xs >= xe or ys >= ye, derives both grids' dimensions by ceil, and sets
 * the reference's hard-coded constants (gravity 9.81, ROI x > 0.5, no relaxation,
 * relax_dt_div 10, TSS_FLAG_Q1_COMPAT). */
tss_status tss_config_init(tss_config* cfg, float xs, float ys, float xe, float ye,
                           float effective_radius, float effective_radius_high,
                           float rest_density, float tait_coeff, float speed_sound,
                           float alpha, float tension_coefficient, float time_step);

/* ------------------------------------------------------------------------- */
/* Solver                                                                     */
/* ------------------------------------------------------------------------- */
typedef struct tss_solver tss_solver;

/* Construct a solver.  Replaces `new ParticleSystem` x3 + CreateParticleBox(Canvas) +
 * WCSPHSolver ctor + Bind() (ParticleSystem.cpp:13-179, WCSPHSolver.cu:2391-2639).
 *   low_pos, low_vel : host, 2*n_low floats (x,y interleaved); low_vel may be NULL (= 0)
 *   cap_high         : high-res pool capacity (the reference uses 4 * n_low)
 *   wall_pos         : host, 2*n_wall floats, the fixed boundary particles
 * Low-res particle i gets slot id i; its children get high-res slot ids 4*i+0..3. */
tss_status tss_solver_create(const tss_config* cfg,
                             int n_low, const float* low_pos, const float* low_vel,
                             float mass_low, int cap_high, float mass_high,
                             int n_wall, const float* wall_pos, float mass_wall,
                             tss_solver** out);
void tss_solver_destroy(tss_solver* s);

/* ------------------------------------------------------------------------- */
/* Batches: many independent scenes advanced by the same kernel launches        */
/* ------------------------------------------------------------------------- */
/* One scene of a batch: its own configuration (domain, radii, constants, ROI,
 * dt; relax_iters must be equal across a batch), particles and walls. */
typedef struct tss_scene_desc {
    const tss_config* config;
    int n_low;
    const float* low_pos;      /* host, 2*n_low floats  */
    const float* low_vel;      /* may be NULL           */
    float mass_low;
    float mass_high;
    int n_wall;
    const float* wall_pos;     /* host, 2*n_wall floats */
    float mass_wall;
} tss_scene_desc;

/* Create a batch of n_scenes scenes sharing one high-res pool of cap_high
 * particles.  The scenes' grids are laid side by side in one global cell space,
 * so one grid build and one launch of each kernel advance all of them; a scene's
 * results are the same as when it runs alone (the reference's solver held one
 * scene per process, WCSPHSolver.cu:2728).  The returned handle works with every
 * tss_solver_* call; slot ids are global (scene k's low-res particle i has slot
 * base_k + i, base_k a multiple of TSS_POOL_SLOT_PAGE); tss_solver_download_scene
 * returns one scene with its own ids.  A batch is a pool (below) sized for exactly
 * these scenes, with scene k admitted as scene k. */
tss_status tss_batch_create(int n_scenes, const tss_scene_desc* scenes, int cap_high, tss_solver** out);
tss_status tss_solver_num_scenes(tss_solver* s, int* n_scenes);
/* Per-scene particle counts (arrays of n_scenes ints, either may be NULL). */
tss_status tss_solver_scene_counts(tss_solver* s, int* n_low, int* n_high);
/* One scene's state, scene-local ids (low: 0..n_low-1, high: 4*low id + child). */
struct tss_scale_state;
tss_status tss_solver_download_scene(tss_solver* s, int scene, int scale, struct tss_scale_state* out);

/* ------------------------------------------------------------------------- */
/* Pools: scenes admitted and retired between steps (continuous batching)       */
/* ------------------------------------------------------------------------- */
/* No counterpart in the reference (one scene per process).  A pool is a batch
 * whose device arrays are sized once, for capacities, and whose scenes come and
 * go between steps: tss_pool_admit places a scene in free pages of each resource,
 * tss_pool_retire frees them, and tss_solver_step advances every admitted scene
 * together (the step is one CUDA graph for the pool's capacities; the work of each
 * kernel follows the particles and cells in use).  A scene's results do not
 * depend on what else is in the pool or where it was placed.  All calls that take
 * a stream are ordered on it; use the same stream for tss_solver_step. */
#define TSS_POOL_SLOT_PAGE 256   /* low-res slots per page (high-res slots: 4x) */
#define TSS_POOL_CELL_PAGE 64    /* grid cells per page, both scales */
#define TSS_POOL_WALL_PAGE 64    /* wall particles per page */
#define TSS_POOL_MAX_SCENES 65535

typedef struct tss_pool_config {
    int64_t low_slots;       /* low-res particles over all admitted scenes */
    int64_t high_particles;  /* high-res list capacity; each admission reserves 4 per low-res particle */
    int64_t low_cells;       /* low-res grid cells (a scene takes its grid's cells + 1) */
    int64_t high_cells;      /* high-res grid cells */
    int64_t wall_particles;
    int32_t max_scenes;      /* <= TSS_POOL_MAX_SCENES */
    int32_t relax_iters;     /* every admitted scene's config must have this relax_iters */
} tss_pool_config;

/* What a scene takes from a pool (host only; rounded to pages). */
typedef struct tss_footprint {
    int64_t low_slots, high_particles, low_cells, high_cells, wall_particles;
} tss_footprint;

/* Device bytes of a pool (host only, no device needed). */
tss_status tss_pool_bytes(const tss_pool_config* cfg, size_t* bytes);
/* The largest pool of `bytes` device bytes whose resources are in the given
 * proportions per low-res slot (high-res list 4 per slot; low_cells_per_slot
 * low-res cells, 4x that high-res; walls_per_slot walls).  Host only. */
tss_status tss_pool_config_for_budget(size_t bytes, double low_cells_per_slot, double walls_per_slot,
                                      int max_scenes, int relax_iters, tss_pool_config* out);
tss_status tss_scene_footprint(const tss_scene_desc* scene, tss_footprint* out);

tss_status tss_pool_create(const tss_pool_config* cfg, tss_solver** out);
/* Place a scene and enqueue its upload, grid keys and wall grid on `stream`.
 * TSS_CAPACITY: some resource has no free run large enough now (retry after a
 * retirement); TSS_INVALID_ARG: the scene can never fit this pool, or its
 * relax_iters differs.  Pageable host arrays are copied before the call returns;
 * page-locked ones are read by the stream and must stay unchanged until it has
 * passed the admission. */
tss_status tss_pool_admit(tss_solver* s, const tss_scene_desc* scene, void* stream, int* scene_id);
/* Would tss_pool_admit succeed now?  TSS_OK, TSS_CAPACITY or TSS_INVALID_ARG as
 * it would return, without admitting anything. */
tss_status tss_pool_can_admit(tss_solver* s, const tss_scene_desc* scene);
/* Drop a scene's particles from the next grid build and free its pages at once
 * (the pages may be admitted to again before the next step). */
tss_status tss_pool_retire(tss_solver* s, int scene_id, void* stream);
/* Resources free now (host-side accounting). */
tss_status tss_pool_free(tss_solver* s, tss_footprint* free_now);

/* A scene's state in caller memory: arrays of each scale (0 low, 1 high) with
 * capacities cap[k]; NULL arrays are skipped; ids are scene-local.  n[] is what a
 * host-side call wrote. */
typedef struct tss_scene_result {
    int32_t cap[2];
    int32_t n[2];
    int32_t* id[2];
    float* pos[2];     /* 2 floats per particle */
    float* vel[2];
    uint8_t* state[2];
    float* dens[2];    /* density of the last step (0 for children created in it) */
    float* pres[2];
} tss_scene_result;

/* Enqueue a copy of an admitted scene's state after its last step into `dst`,
 * whose arrays must be device-accessible (device memory or mapped page-locked
 * host memory) and 8-byte aligned; d_counts (3 device-accessible ints) receives
 * the particles of each scale and the number of them with a non-finite position,
 * velocity or density (a scene that went unstable; the other scenes of the pool
 * are not affected by it).  Valid between a step and the next one, before
 * the scene's retirement; cap[0] >= n_low and cap[1] >= 4 n_low always suffice.
 * Order within each scale: the list order (the last step's (cell, id) order,
 * then that step's new children); with TSS_FLAG_MERGE, children removed in the
 * last step are included with state 2. */
tss_status tss_pool_extract(tss_solver* s, int scene_id, const tss_scene_result* dst, int32_t* d_counts,
                            void* stream);

/* ------------------------------------------------------------------------- */
/* Serving: a request loop over a pool                                           */
/* ------------------------------------------------------------------------- */
/* Replays a trace of scene requests in real time: a request is visible from its
 * arrival time on, is admitted (first come, first served) as soon as the pool
 * has room for it, advances with every other admitted scene, and after `horizon`
 * steps its final state is extracted, copied to `result` and its pages freed.
 * Steps are issued in chunks that end when some scene reaches its horizon (at
 * most max_steps_per_launch), so admission and retirement happen between steps
 * while the GPU works on the chunks queued before. */
typedef struct tss_server tss_server;
typedef struct tss_server_config {
    tss_pool_config pool;
    int32_t max_steps_per_launch;   /* e.g. 8 */
    int32_t max_in_flight;          /* chunks queued ahead of the GPU, e.g. 2 */
    int64_t staging_bytes;          /* page-locked staging for uploads and results */
} tss_server_config;

typedef struct tss_request {
    tss_scene_desc scene;
    int32_t horizon;            /* steps, >= 1 */
    double arrival_s;           /* seconds after the start of tss_server_run */
    tss_scene_result* result;   /* host arrays for the final state, or NULL */
} tss_request;

typedef struct tss_request_stats {
    double arrival_s;
    double admit_s;             /* host time of the admission call */
    double done_s;              /* the final state is in host memory (GPU event time) */
    int64_t first_step;         /* pool step index of the scene's first step */
    int32_t status;             /* TSS_OK; TSS_NUMERIC: the final state has non-finite
                                   particles; TSS_INVALID_ARG: it can never fit */
    int32_t n_low, n_high;      /* final counts */
} tss_request_stats;

typedef struct tss_serve_summary {
    double makespan_s;          /* trace start to the last result */
    int64_t steps;              /* pool steps launched */
    int64_t scene_steps;        /* sum of the served requests' horizons */
    double low_particle_steps;  /* sum of n_low * horizon */
    double mean_active;         /* scenes per step, averaged over steps */
    int32_t max_active;
    int32_t served;
} tss_serve_summary;

tss_status tss_server_create(const tss_server_config* cfg, tss_server** out);
/* The arithmetic of the server pool's gathers (tss_solver_set_arith on its pool;
 * TSS_ARITH_EXACT by default).  Call between runs. */
tss_status tss_server_set_arith(tss_server* sv, int mode);
tss_status tss_server_run(tss_server* sv, int n, const tss_request* reqs, tss_request_stats* stats,
                          tss_serve_summary* summary);
void tss_server_destroy(tss_server* sv);
/* Text of the last failure of a server call (or of its pool's last call). */
tss_status tss_server_last_error(tss_server* sv, char* buf, int len);

/* Advance n_steps steps (WCSPHSolver::AdvanceTS, WCSPHSolver.cu:2726-2810), enqueued
 * on `stream` (a cudaStream_t; NULL = the default stream, as the reference used).
 * Nothing is copied back to the host; the particle counts stay on the device.  The
 * steps are replayed from CUDA graphs of 8, 4, 2 and 1 steps (n_steps taken as a
 * sum of those buckets; each graph is captured on a private stream at its first
 * use and does not depend on the particle counts).  With profiling on, every step
 * is its own graph. */
tss_status tss_solver_step(tss_solver* s, int n_steps, void* stream);

/* Block until all enqueued work is done; returns the device error word mapped to a
 * status (TSS_CAPACITY, TSS_NUMERIC, TSS_GRID_INDEX) or TSS_OK. */
tss_status tss_solver_sync(tss_solver* s);

typedef struct tss_counts {
    int n_low;                /* low-res particles (constant)                         */
    int n_high;               /* high-res particles                                   */
    int n_transient_low;      /* low-res particles in state 1 (split parents)         */
    int n_split_last;         /* parents split in the last step                       */
    long long steps;          /* steps taken                                          */
    unsigned error_bits;      /* device error word (TSS_ERR_*)                        */
    int n_removed_last;       /* high-res particles removed by merges in the last step */
    long long total_split;    /* splits since creation                                 */
    long long total_removed;  /* high-res particles removed by merges since creation   */
} tss_counts;

#define TSS_ERR_CAPACITY 0x1u /* a split would overflow the high-res pool            */
#define TSS_ERR_NUMERIC  0x2u /* NaN/Inf density, pressure or acceleration            */
#define TSS_ERR_GRID_INDEX 0x4u /* a grid index check failed (inconsistent offsets)  */

tss_status tss_solver_counts(tss_solver* s, tss_counts* out);

/* Particle state of one scale, in list order (the order the next step starts from:
 * this step's sorted order, with newly created children appended to the high list).
 * Caller-owned host buffers with room for n entries (pos/vel: 2n floats). */
typedef struct tss_scale_state {
    int       n;
    int32_t*  id;             /* slot ids                                              */
    float*    pos;            /* 2n                                                    */
    float*    vel;            /* 2n                                                    */
    uint8_t*  state;          /* 0 default, 1 transient, 2 deleted                     */
    float*    dens;           /* last densities (may be NULL)                          */
    float*    pres;           /* last pressures (may be NULL)                          */
} tss_scale_state;

#define TSS_SCALE_LOW  0
#define TSS_SCALE_HIGH 1

/* Download / replace the state of one scale (checkpoint and per-step resync).
 * Upload checks ids are unique and in range and sets the count. */
tss_status tss_solver_download(tss_solver* s, int scale, tss_scale_state* out);
tss_status tss_solver_upload(tss_solver* s, int scale, const tss_scale_state* in);

/* The low-res parents split in the last step; their children are relaxed at the
 * start of the next step when relax_iters > 0. */
tss_status tss_solver_get_fresh(tss_solver* s, int* n, int32_t* parents /* may be NULL */);
tss_status tss_solver_set_fresh(tss_solver* s, int n, const int32_t* parents);

/* Per-step intermediate buffers, for parity checks (host copies). */
typedef enum tss_buffer {
    TSS_BUF_SORTED_ID = 0,    /* int32[n]   ids in (cell, id) order, the sorted list    */
    TSS_BUF_CELL_OFFSET = 1,  /* int32[C+1] dense cell offsets (start = off[c],         */
                              /*            end = off[c+1])                             */
    TSS_BUF_DENSITY = 2,      /* float[n]   densities, sorted order                     */
    TSS_BUF_PRESSURE = 3,     /* float[n]   pressures, sorted order                     */
    TSS_BUF_ACCEL = 4,        /* float[2n]  accelerations, sorted order                 */
    TSS_BUF_SPLIT = 5,        /* int32[k]   low-res slot ids split this step (low only) */
    TSS_BUF_WALL_CELL_OFFSET = 6 /* int32[C_low+1] boundary cell offsets (low only)     */
} tss_buffer;
/* Copies buffer `which` of `scale` into `dst` (capacity `count` elements); *written
 * receives the element count (may be NULL).  Values refer to the last step. */
tss_status tss_solver_copy(tss_solver* s, int scale, int which, void* dst, size_t count,
                           size_t* written);

/* Device pointers for a renderer (replaces the GL VBO interop of
 * ParticleSystem.cpp:20-46,78-98).  Valid until the next tss_solver_step. */
typedef struct tss_buffers {
    const float*   pos[2];    /* float2[n], list order                                 */
    const float*   vel[2];
    const float*   dens[2];   /* float[n], sorted order of the last step               */
    const int32_t* id[2];     /* int32[n], list order                                  */
    const uint8_t* state[2];
    const int*     counts;    /* device int[2] = {n_low, n_high}                       */
} tss_buffers;
tss_status tss_solver_device_buffers(tss_solver* s, tss_buffers* out);

/* Asynchronous position read-back: enqueues on `stream` one kernel that writes the
 * positions of both lists after the last enqueued step (list order, as
 * tss_buffers.pos; high-res entries removed in that step are still in the list,
 * with state 2) into page-locked host memory, and the two list lengths into
 * counts[2] (page-locked host ints).  Entries beyond cap_low / cap_high are not
 * written (counts still gives the full lengths).  Nothing is synchronised: the
 * caller waits on the stream (or an event recorded after this call) before reading,
 * and may meanwhile enqueue the next steps.  The host buffers must be page-locked
 * (cudaHostAlloc / cudaMallocHost or registered), which the GPU writes through
 * unified addressing; other memory is TSS_INVALID_ARG.  Replaces mapping the VBOs
 * each frame (ParticleSystem.cpp:78-98) for a renderer that reads on the host. */
tss_status tss_solver_read_positions(tss_solver* s, float* host_low, int cap_low, float* host_high, int cap_high,
                                     int* counts, void* stream);

/* The same read-back overlapped with the steps that follow.  On `stream` one
 * kernel copies the positions and lengths into one of two device staging buffers
 * of the solver (device-to-device, a few microseconds for a million particles);
 * a stream of the solver's own then writes them from there into the page-locked
 * host memory while `stream` goes on with the next steps (for a single scene by
 * copy engine: the whole low-res list and host_high's first cap_high entries, of
 * which those past counts[1] are undefined).  *ticket names the read-back for
 * tss_solver_read_wait, which blocks the calling thread until its host memory is
 * written.  The staging buffers are used in turn: a read-back waits on `stream`
 * until the one two calls earlier has left its buffer.  The host buffers must stay
 * untouched until the ticket has been waited for. */
tss_status tss_solver_read_positions_async(tss_solver* s, float* host_low, int cap_low, float* host_high,
                                           int cap_high, int* counts, void* stream, int64_t* ticket);
tss_status tss_solver_read_wait(tss_solver* s, int64_t ticket);

/* Stage timing.  With profiling on, the captured step graph also records a CUDA
 * event at each stage boundary; tss_solver_stage_times then returns the device time
 * (ms) of each stage of the LAST step (it synchronises).  Stages, in order:
 *   0 high-res grid, 1 low-res grid, 2 relaxation, 3 high-res density,
 *   4 low-res density, 5 low-res force + advance + split marks,
 *   6 split compaction + children, 7 high-res force + integrate + tether.
 * The reference's CUDA::Timer (CUDA/cuda.h:88-108) was the counterpart; all its
 * uses are commented out (WCSPHSolver.cu:2653-2676). */
#define TSS_NUM_STAGES 8
tss_status tss_solver_profile(tss_solver* s, int enable);
tss_status tss_solver_stage_times(tss_solver* s, float* ms, int n);

/* Launch shape of the four gather kernels, indexed high-res density, low-res
 * density, low-res force, high-res force (stages 3, 4, 5, 7).  Every kernel walks
 * its list with a grid-stride loop over a device-side count, so results do not
 * depend on the shape.  The reference launched 256-thread blocks covering the
 * list (WCSPHSolver.cu:2421,2437); that shape is the default here. */
#define TSS_NUM_GATHERS 4
typedef struct tss_launch {
    int threads[TSS_NUM_GATHERS];     /* threads per block: 64, 128 or 256                          */
    int persistent[TSS_NUM_GATHERS];  /* 0: blocks cover the list's capacity (at most 4096 threads
                                         per SM, grid-striding beyond); 1: one wave of resident
                                         blocks (SMs x blocks per SM), each striding over the list */
    int per_warp[TSS_NUM_GATHERS];    /* 0: one particle per thread (32 per warp); 1: one particle
                                         per warp, its candidates spread over the lanes (for
                                         scenes too small to fill the GPU)                         */
} tss_launch;
tss_status tss_solver_get_launch(tss_solver* s, tss_launch* out);
/* Replaces the launch shape (the step graphs are captured again at the next step). */
tss_status tss_solver_set_launch(tss_solver* s, const tss_launch* in);
/* Launch-shape autotuner: times every candidate shape (threads 64/128/256, covering
 * or persistent grids, one particle per thread; and one particle per warp) on this
 * handle's own steps, stage by stage, and keeps the fastest shape of each gather (a
 * gather keeps the default shape unless a candidate is more than 5% faster).  Then
 * it times whole unprofiled steps with that choice, with the default shape and with
 * one particle per warp throughout, and installs the fastest of the three (the
 * choice unless another is more than 5% faster).  The trial steps are real steps of
 * the handle's state (the shape does not change results); *steps_taken (may be
 * NULL) receives how many were taken: 10 x (steps_per_trial + 1).  Synchronises. */
tss_status tss_solver_autotune(tss_solver* s, int steps_per_trial, tss_launch* best, int* steps_taken);

/* Arithmetic of the gathers' pair terms.  TSS_ARITH_EXACT (the default) is the
 * reference's FP32 arithmetic: IEEE square root and division, no fused
 * multiply-adds, the reference's association, so results equal the reference's
 * bit for bit for the same list order.  TSS_ARITH_FAST spends the step's tolerance
 * (densities, forces and positions within 1e-5 relative in FP32) instead: one
 * approximate reciprocal square root and one approximate reciprocal per pair,
 * fused multiply-adds, the cubic spline and its gradient in expanded form.  The
 * neighbour sets, summation order, cutoffs, grid and split logic are the same in
 * both; only the per-pair values differ, by a few units in the last place, so a
 * split decision can differ only for a particle within rounding of the region's
 * edge.  The reference has no counterpart (its Release build used IEEE arithmetic,
 * WCSPHSolver.cu.cache's FastMath=false).  Applies to every scene of a handle; the
 * step graphs are captured again at the next step. */
#define TSS_ARITH_EXACT 0
#define TSS_ARITH_FAST 1
tss_status tss_solver_set_arith(tss_solver* s, int mode);
tss_status tss_solver_get_arith(tss_solver* s, int* mode);

/* Last error message of this handle (NUL-terminated, truncated to len). */
tss_status tss_solver_last_error(tss_solver* s, char* buf, int len);
const char* tss_status_string(tss_status st);

/* ------------------------------------------------------------------------- */
/* Grid build on caller-owned device memory                                   */
/* ------------------------------------------------------------------------- */
/* Uniform-grid neighbour structure of n particles, replacing computeParticleHash +
 * thrust::sort_by_key + computeCellStartEndIndices (WCSPHSolver.cu:1246-1340,
 * 2814-2854).  cell(p) = clamp(int((p - origin)/cell_size), 0, dim-1) per axis,
 * hash = cy*dimx + cx (WCSPHSolver.cu:241-296).  Outputs, all device memory:
 *   d_order[n]       : source index of each sorted position; the order is by
 *                      (cell, d_id) ascending, i.e. a stable sort by cell of an
 *                      id-ascending list
 *   d_cell_off[C+1]  : dense offsets: particles of cell c are order[off[c]..off[c+1])
 *                      (the reference's cellStart/cellEnd, with empty cells as
 *                      empty ranges instead of -1)
 * d_id holds distinct ids (any non-negative int32); with repeated ids d_order is
 * undefined (entries are skipped or written twice; nothing outside the buffers is
 * touched).  d_workspace is scratch of tss_grid_workspace_size bytes.  Enqueued on
 * `stream`; nothing is synchronised.  Cells of any fullness cost O(k log k): cells
 * of more than 32 entries are sorted by id in one block each. */
tss_status tss_grid_workspace_size(int n, int dimx, int dimy, size_t* bytes);
tss_status tss_grid_build(const float* d_pos, const int32_t* d_id, int n,
                          float origin_x, float origin_y, float cell_size,
                          int dimx, int dimy, int32_t* d_order, int32_t* d_cell_off,
                          void* d_workspace, size_t workspace_bytes, void* stream);

/* ------------------------------------------------------------------------- */
/* Headless rendering                                                            */
/* ------------------------------------------------------------------------- */
/* Particle splats into a device RGBA image (4 floats per pixel, row 0 at the
 * bottom), the reference's display() without OpenGL (TwoScale2D/main.cpp:65-102;
 * QuantityRenderer/PointRenderer and their shaders): each particle is a disc of
 * radius point_size in normalised device coordinates around
 * ((p - xs) / (xe - xs) * 2 - 1, (p - ys) / (ye - ys) * 2 - 1), coloured by the jet
 * map of min(|rho - rho0|, 400) / 400 or by a constant colour, alpha 0.5, blended
 * as dst = 0.5 src + 0.5 dst in particle order.  A pixel is covered when its
 * centre lies in the disc. */
typedef struct tss_view {
    float xs, ys, xe, ye;   /* display rectangle (scene units) */
    int width, height;      /* image size in pixels (the reference's window: 1100 x 1100) */
} tss_view;
tss_status tss_render_workspace_size(int n, const tss_view* view, float point_size, size_t* bytes);
/* Fill with the clear colour (1, 1, 1, 0) (main.cpp:73-74). */
tss_status tss_render_clear(float* d_rgba, int width, int height, void* stream);
/* Splat n particles (d_pos: 2 floats each).  d_dens non-NULL: jet colour of the
 * visual quantity; NULL: the colour rgb[3]. */
tss_status tss_render_splats(const tss_view* view, int n, const float* d_pos, const float* d_dens,
                             float rest_density, const float* rgb, float point_size, float* d_rgba,
                             void* d_workspace, size_t workspace_bytes, void* stream);
/* One frame of a single-scene solver: clear, low-res (jet, point_sizes[0]), high-res
 * (jet, point_sizes[1]), walls (black, point_sizes[2]); the reference drew with
 * 0.005, 0.003 and 0.005 (main.cpp:176-190).  Densities are the last step's (the
 * children created in it count as 0).  The first call allocates the solver's
 * render scratch. */
tss_status tss_solver_render(tss_solver* s, const tss_view* view, const float* point_sizes, float* d_rgba,
                             void* stream);

/* Grid build that allocates nothing.  No counterpart in the reference: it is
 * tss_grid_build with its scratch in a fixed array inside this library, for callers
 * that may not call cudaMalloc/cudaFree (a host application's per-frame callback,
 * where those calls can stall the whole device, or a plug-in whose device memory is
 * owned by its host's memory manager).  The caller still passes d_pos, d_id,
 * d_order and d_cell_off as for tss_grid_build.
 *   - Limit: tss_grid_workspace_size(n, dimx, dimy) must not exceed
 *     TSS_GRID_NOALLOC_MAX_BYTES (32 MiB: up to 1,277,759 particles on a
 *     1400x1400 grid); larger problems get TSS_CAPACITY and should use
 *     tss_grid_build.
 *   - The array occupies TSS_GRID_NOALLOC_MAX_BYTES on every GPU that loads the
 *     library, until the process exits.
 *   - The first call on a device looks up the array's device address on that
 *     device; make that first call before any stream capture.  The address is
 *     kept for the life of the process: after cudaDeviceReset the library's
 *     module is loaded again and the kept address is stale, so do not call this
 *     entry point after resetting a device.
 *   - All calls share the array: calls whose work overlaps on the GPU (other
 *     streams, other host threads) race and give undefined results.  Each call
 *     clears the parts that must start at zero. */
#define TSS_GRID_NOALLOC_MAX_BYTES (32u << 20)
tss_status tss_grid_build_noalloc(const float* d_pos, const int32_t* d_id, int n,
                                  float origin_x, float origin_y, float cell_size,
                                  int dimx, int dimy, int32_t* d_order, int32_t* d_cell_off,
                                  void* stream);

#ifdef __cplusplus
}
#endif
#endif /* TSS_H */
