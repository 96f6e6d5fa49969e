/*
 * rfmm.h -- C ABI of the GB300 FMM solver (the dispatch-sequence drop-in).
 *
 * The reference host encodes one solver frame as WGSL compute passes
 * clear_cells -> deposit -> upward x depth -> m2l_all -> downward x depth ->
 * near_all -> integrate, sized by the planner and fed by a 16-slot Params
 * table (iskamag/fmm-rainbow app.js:141-213, 525-648; native/main.rs:36-128,
 * 353-421).  This ABI replaces that whole sequence: the host creates a solver
 * for N bodies, uploads or seeds particles, and calls rfmm_step /
 * rfmm_solve_fields; the library owns device memory and runs sm_103a
 * kernels on one GPU.  Buffers keep the reference layouts (Particle 32 B,
 * Moment 16 B, Field 48 B; src/rainbow_fmm.wgsl:52-73) so content digests
 * stay comparable with the reference harness (native/main.rs:152-163).
 *
 * Conventions: every function returns an int status (0 = RFMM_OK, negative
 * = RFMM_ERR_*); no exception or abort crosses the ABI.  The library owns
 * device memory, the caller owns host memory.  A handle is bound to one CUDA
 * device and one stream and is not thread-safe; separate handles may be used
 * from separate threads.  Calls are asynchronous on the handle's stream
 * unless they return host data (download, digest, phase times, sync).
 */
#ifndef RFMM_H
#define RFMM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RFMM_ABI_VERSION 1u

enum rfmm_status {
  RFMM_OK = 0,
  RFMM_ERR_INVALID = -1,   /* bad argument (null pointer, size mismatch, range) */
  RFMM_ERR_CUDA = -2,      /* a CUDA runtime call failed */
  RFMM_ERR_OOM = -3,       /* device memory allocation failed */
  RFMM_ERR_STATE = -4,     /* call out of order (e.g. step before particles exist) */
  RFMM_ERR_TIMEOUT = -5,   /* a kernel's bounded wait gave up; see rfmm_device_error */
  RFMM_ERR_NO_DEVICE = -6, /* no CUDA device, or the device is not sm_103 */
  RFMM_ERR_DEVICE = -7,    /* a kernel reported an internal error word */
  RFMM_ERR_BUDGET = -8     /* request does not fit the memory budget (server) */
};

/* Which buffer rfmm_download / rfmm_digest read. */
enum rfmm_buffer {
  RFMM_BUF_PARTICLES = 0, /* N x 32 B, in the caller's body order */
  RFMM_BUF_MOMENTS = 1,   /* C x 16 B, the moment tree of the last solve */
  RFMM_BUF_FIELDS = 2     /* C x 48 B, the fields of the last solve */
};

/* Physics parameters: the compute-relevant fields of `struct Params`
 * (src/rainbow_fmm.wgsl:18-50).  depth/fixed_point_scale 0 = use the
 * planner's unclamped plan (src/lib.rs:45-69), as the native harness does
 * (native/main.rs:89-92). */
typedef struct rfmm_params {
  float dt;                   /* Params.dt */
  float gravity;              /* Params.gravity */
  float softening;            /* Params.softening */
  float speed;                /* Params.speed; the step uses dt * speed */
  float control_point[4];     /* xyz brush centre; w > 0.5 = control active */
  float control_axis_mode[4]; /* xyz vortex axis; w 1 = pull, 2 = push, 3 = vortex */
  float control_strength;     /* control_settings.x */
  float control_radius;       /* control_settings.y */
  float fixed_point_scale;    /* control_settings.z; 0 = planner scale */
  uint32_t depth;             /* 0 = planner depth; else 4..6 */
} rfmm_params;

/* The plan a handle runs with. */
typedef struct rfmm_plan {
  uint32_t particles;
  uint32_t depth;
  uint32_t cells; /* total_cells(depth) */
  float fixed_point_scale;
} rfmm_plan;

typedef struct rfmm_handle rfmm_handle;

/* Fill `p` with the native harness's defaults (native/main.rs:57-81):
 * dt 0.0009, gravity 0.34, softening 0.012, speed 1, control off,
 * strength 0.7, radius 0.22. */
void rfmm_default_params(rfmm_params *p);

/* Human-readable name of a status code (static string). */
const char *rfmm_status_string(int status);

/* Create a solver for `n` bodies (1 <= n <= 2^23) on the current CUDA
 * device.  Allocates the particle, moment and field buffers
 * (app.js:543-559, native/main.rs:307-309).  `params` may be NULL for the
 * harness defaults. */
int rfmm_create(uint32_t n, const rfmm_params *params, rfmm_handle **out);
int rfmm_destroy(rfmm_handle *h);

/* Run the handle's work on `stream` (a cudaStream_t; NULL = the handle's
 * own stream). */
int rfmm_set_stream(rfmm_handle *h, void *stream);
int rfmm_get_plan(const rfmm_handle *h, rfmm_plan *out);

/* Replace the physics parameters (app.js updateComputeParams, 189-205).
 * depth and fixed_point_scale must match the plan the handle was made with
 * (0 = keep). */
int rfmm_set_params(rfmm_handle *h, const rfmm_params *params);

/* Upload N bodies (N x 32 B, reference Particle layout) from host memory
 * (pinned or pageable) or from device memory.  The copy and the leaf sort
 * are enqueued on the handle's stream; from pinned memory the call returns
 * before the copy has run, so the source must stay valid until the handle's
 * next synchronising call (rfmm_download, rfmm_sync). */
int rfmm_upload_particles(rfmm_handle *h, const void *host_aos, size_t bytes);
int rfmm_upload_particles_device(rfmm_handle *h, const void *device_aos, size_t bytes);

/* Seed the reference galaxy (`initialize`, src/rainbow_fmm.wgsl:232-374). */
int rfmm_seed_galaxy(rfmm_handle *h);

/* One field solve without integrate: clear, deposit, upward, m2l, downward,
 * near (native/main.rs:437-449).  Moments and fields then hold the tree and
 * the field of the current positions. */
int rfmm_solve_fields(rfmm_handle *h);

/* `steps` full solver frames (native/main.rs:411-421), enqueued on the
 * handle's stream. */
int rfmm_step(rfmm_handle *h, uint32_t steps);

/* Wait for the handle's queued work; reports kernel error words. */
int rfmm_sync(rfmm_handle *h);

/* Copy a buffer to host memory (bytes must equal the buffer size:
 * N*32, C*16 or C*48) or to device memory.  Particles come back in the
 * caller's body order.  Returns once the bytes are in place (it waits for
 * the handle's stream), reporting kernel error words like rfmm_sync. */
int rfmm_download(rfmm_handle *h, int which, void *host_dst, size_t bytes);
int rfmm_download_device(rfmm_handle *h, int which, void *device_dst, size_t bytes);

/* FNV-1a digest of a buffer's little-endian bytes (native/main.rs:152-163). */
int rfmm_digest(rfmm_handle *h, int which, uint32_t *out);

/* Per-phase device time in ms of one instrumented frame, in the reference
 * harness's phase order (native/main.rs:468): clear, deposit, upward, m2l,
 * downward, near, integrate.  Fused phases report their time in the first
 * phase of the fusion and 0 in the others: clear is folded into upward,
 * downward carries L2L+near, integrate carries the next step's deposit;
 * in RFMM_NEAR_P2P mode near carries the exact pair sums.
 * deposit is a standalone P2M of the current positions into a scratch tree
 * (in a step the deposit rides on integrate).  The frame advances the
 * simulation by one step. */
int rfmm_phase_times(rfmm_handle *h, float ms[7]);

/* Non-finite count and max |value| over the first min(N, probe) bodies'
 * 8 floats (native/main.rs:536-549). */
int rfmm_check_finite(rfmm_handle *h, uint32_t probe, uint32_t *non_finite, float *max_abs);

/* Steps between refreshes of the resident leaf order (0 = never; default
 * 16; the autotuner also tunes it).  Results do not depend on it. */
int rfmm_set_resort_interval(rfmm_handle *h, uint32_t steps);

/* Near-field mode.  RFMM_NEAR_REFERENCE (default) is the reference's: 26
 * neighbour-cell monopoles at each adaptive leaf's centre plus the self-cell
 * monopole (wgsl:521-572, 646-657).  RFMM_NEAR_P2P has no reference
 * counterpart: the fields carry M2L + L2L only, and each body adds the exact
 * softened pair forces (softening = params.softening, masses 1/N) of every
 * body in the 3x3x3 cells around its sample cell.  Every P2P step ends with a
 * leaf sort from the caller's order, so the pair sums run in a fixed order
 * (cells z-, y-, x-major; bodies by leaf, then caller index) and results are
 * reproducible.  Switching re-sorts the uploaded bodies; positions and
 * velocities are kept. */
#define RFMM_NEAR_REFERENCE 0u
#define RFMM_NEAR_P2P 1u
int rfmm_set_near_mode(rfmm_handle *h, uint32_t mode);

/* Floating-point variant of the step kernels (no counterpart in the
 * reference, whose WGSL leaves these details to the implementation).
 * RFMM_FLOAT_EXACT (default): binary32 round-to-nearest without contraction,
 * IEEE division and square root, inverseSqrt as 1/sqrt -- the CPU oracle's
 * contract, so results are reproducible bit for bit.  RFMM_FLOAT_FAST: the
 * latitude WGSL gives (multiply-add contraction, approximate division and
 * square root within a few ulp, inverseSqrt as the hardware reciprocal
 * square root).  Leaf assignment, moments and every integer result of a
 * field solve are identical in both; floating-point results agree within
 * the tolerances stated by the fast-mode tests (accelerations ~1e-6
 * relative rms), and trajectories drift apart at that level per step.
 * Switching drops the captured graphs. */
#define RFMM_FLOAT_EXACT 0u
#define RFMM_FLOAT_FAST 1u
int rfmm_set_float_mode(rfmm_handle *h, uint32_t mode);

/* Last kernel error word (0 = none) and its detail. */
int rfmm_device_error(rfmm_handle *h, uint32_t *code, uint32_t *info);
/* Self-check of the kernels' bounded waits: one CTA waits on an mbarrier
 * phase nothing completes, giving up after `polls` polls (1 .. 2^22).
 * Returns RFMM_ERR_TIMEOUT when the wait gave up as it must (the handle stays
 * usable and its error word is untouched), RFMM_OK never in practice. */
int rfmm_check_wait_timeout(rfmm_handle *h, uint32_t polls);

/* Kernel kinds of rfmm_profile_steps. */
enum rfmm_kernel_kind {
  RFMM_KERNEL_UPWARD = 0,    /* M2M + source records + work list */
  RFMM_KERNEL_M2L = 1,       /* 189-cell M2L */
  RFMM_KERNEL_L2L_NEAR = 2,  /* L2L chain + adaptive-leaf near field */
  RFMM_KERNEL_INTEGRATE = 3, /* L2P + self leaf + kick/drift + next deposit */
  RFMM_KERNEL_RESORT = 4,    /* refresh of the resident leaf order */
  RFMM_KERNEL_NEAR_P2P = 5,  /* RFMM_NEAR_P2P: exact near-field pair sums */
  RFMM_KERNEL_KINDS = 6
};

/* Profiling counterpart of rfmm_step: runs `steps` frames with direct
 * launches and a CUDA event pair around every kernel on the handle's
 * stream, and ADDS each kind's device time (ms) and launch count into the
 * caller's arrays (RFMM_KERNEL_KINDS entries each). Same results as
 * rfmm_step; only the launch mechanism differs (no graph). */
int rfmm_profile_steps(rfmm_handle *h, uint32_t steps, float *kernel_ms, uint32_t *launches);

/* Number of solver kernels this handle has launched so far (kernels inside
 * CUDA graphs included). */
int rfmm_launch_count(rfmm_handle *h, uint64_t *out);

/* Device timeline of the step kernels as they run inside the captured
 * graphs (no counterpart in the reference; its harness reads per-pass GPU
 * timestamps, native/main.rs:462-520).  With the timeline on, every graph
 * captured afterwards stamps, for each step kernel, the %globaltimer time at
 * which its first CTA passed its dependency wait and the time its last CTA
 * finished; each graph keeps the records of its most recent run.  Turning
 * it on or off drops the captured graphs (they are captured again on the
 * next step).  The stamps cost one atomic per CTA and launch. */
typedef struct rfmm_timeline {
  uint32_t steps;                        /* steps the records cover */
  uint32_t launches[RFMM_KERNEL_KINDS];  /* recorded launches per kernel kind */
  double busy_ms[RFMM_KERNEL_KINDS];     /* sum of (last CTA end - first CTA begin) */
  double gap_ms[RFMM_KERNEL_KINDS];      /* sum of (first CTA begin - previous kernel's end):
                                          * launch and dependency latency in front of it */
  double span_ms;                        /* sum over the recorded graph runs of
                                          * (last end - first begin) */
} rfmm_timeline;
int rfmm_set_timeline(rfmm_handle *h, uint32_t enable);
int rfmm_get_timeline(rfmm_handle *h, rfmm_timeline *out);

/* ---------------------------------------------------------------- accuracy
 *
 * Each runs a field solve of the current positions first (like
 * rfmm_solve_fields) and does not advance the simulation.  FP64 is used only
 * here: the direct-sum reference and the compensated reductions. */
typedef struct rfmm_diagnostics {
  double kinetic;             /* sum 1/2 m v^2, m = 1/N */
  double potential;           /* sum 1/2 m phi, phi from the FMM expansion */
  double total;
  double momentum[3];         /* sum m v */
  double angular_momentum[3]; /* sum m x cross v */
} rfmm_diagnostics;

/* FMM acceleration and potential per body (N x 4 floats: ax ay az phi) in
 * the caller's order, as integrate applies them (wgsl:619-657). */
int rfmm_accelerations(rfmm_handle *h, float *host_out, size_t bytes);
/* Relative force error of the FMM against an FP64 softened direct sum
 * (softening = params.softening, masses 1/N) on `targets` bodies sampled
 * uniformly without replacement (seeded): rms = sqrt(sum|da|^2 / sum|a|^2). */
int rfmm_force_error(rfmm_handle *h, uint32_t targets, uint64_t seed, double *rms_rel,
                     double *max_rel);
/* Energy and momentum with FP64 compensated (Neumaier) reductions. */
int rfmm_get_diagnostics(rfmm_handle *h, rfmm_diagnostics *out);

/* ---------------------------------------------------------------- render
 *
 * Headless restatement of the reference's display passes (wgsl:780-1009,
 * app.js:650-710): every drawn point (instance i shows body (i * 747796405 +
 * 2891336453) mod N in the caller's order) is splatted additively into an
 * accumulation image of half the canvas size, blurred by the 5-tap separable
 * filter and tone-mapped into an RGBA8 image of width x height (row 0 at the
 * top).  No window or graphics API is involved.  The accumulation is a
 * fixed-point sum (exact, order-independent) instead of an rgba16float blend.
 * The control field highlight uses the handle's params. */
typedef struct rfmm_render_params {
  uint32_t width, height; /* canvas size in pixels */
  uint32_t instances;     /* points drawn; 0 = N */
  float yaw, pitch;       /* camera angles (radians) */
  float zoom;             /* camera distance in world half-extents */
  float point_size;       /* blur radius in canvas pixels (the "gradient radius") */
  float exposure;
} rfmm_render_params;

/* Defaults of the reference app: yaw -0.18, pitch -0.14, zoom 1.78, point
 * size 5, exposure 1, instances = N, 1280 x 720. */
void rfmm_default_render_params(rfmm_render_params *out);
int rfmm_render(rfmm_handle *h, const rfmm_render_params *params, void *host_rgba, size_t bytes);
int rfmm_render_device(rfmm_handle *h, const rfmm_render_params *params, void *device_rgba,
                       size_t bytes);

/* ------------------------------------------------------------------- tuning
 *
 * Launch shapes and scheduling of the step kernels.  Results never depend on
 * them (every choice computes the same bits); only speed does.
 * rfmm_autotune picks them by timing candidate settings on the resident
 * scene (coordinate descent), which advances the simulation by the trial
 * steps. */
typedef struct rfmm_tuning {
  uint32_t upward_ctas_per_sm;    /* persistent upward grid, 1..16 */
  uint32_t m2l_ctas_per_sm;       /* persistent M2L grid, 1..6 */
  uint32_t l2l_ctas_per_sm;       /* persistent L2L + near grid, 1..8 */
  uint32_t integrate_ctas_per_sm; /* persistent integrate grid, 1..resident limit */
  uint32_t integrate_dynamic;     /* 0: interleaved tiles per CTA, 1: tiles from a counter */
  uint32_t resort_interval;       /* steps between resident-order refreshes, 0 = never */
  uint32_t graph_steps;           /* steps per captured CUDA graph, 1..64 */
  uint32_t pdl;                   /* programmatic dependent launch between step kernels */
  uint32_t m2l_compact;           /* 1 (default): M2L lists each child's contributing slots
                                   * first; 0: every stencil slot, in chunks */
  uint32_t m2l_lanes;             /* M2L with one lane per target, four parents per warp:
                                   * 0 never, 1 always, 2 when the parent list is long */
  uint32_t l2l_lanes;             /* L2L + near with one lane per target (else one warp):
                                   * 0 never, 1 always, 2 when the parent list is long */
  uint32_t upward_warps;          /* upward pass with one warp (else one CTA) per subtree:
                                   * 0 never, 1 always, 2 when there are many subtrees */
} rfmm_tuning;

int rfmm_get_tuning(rfmm_handle *h, rfmm_tuning *out);
int rfmm_set_tuning(rfmm_handle *h, const rfmm_tuning *tuning);
/* `steps_per_trial` steps are timed per candidate; the best setting is
 * applied and returned in `best` (may be NULL). */
int rfmm_autotune(rfmm_handle *h, uint32_t steps_per_trial, rfmm_tuning *best);

/* ------------------------------------------------------------------ batches
 *
 * Many independent scenes of uneven size in one set of launches: every
 * kernel of a step covers all scenes (concatenated body tiles, concatenated
 * per-scene trees, one parent work list), and each scene keeps its own plan,
 * parameters and buffers in the reference layouts.  Results per scene are
 * identical to a plain handle's.  A batch replaces running the reference's
 * dispatch sequence once per scene. */
typedef struct rfmm_batch rfmm_batch;

/* `params` points to `scenes` parameter blocks, or is NULL for the harness
 * defaults for every scene. */
int rfmm_batch_create(uint32_t scenes, const uint32_t *bodies_per_scene, const rfmm_params *params,
                      rfmm_batch **out);
int rfmm_batch_destroy(rfmm_batch *b);
int rfmm_batch_set_stream(rfmm_batch *b, void *stream);
int rfmm_batch_get_plan(const rfmm_batch *b, uint32_t scene, rfmm_plan *out);
int rfmm_batch_set_params(rfmm_batch *b, uint32_t scene, const rfmm_params *params);
/* Stage a scene's bodies (host or device memory); rfmm_batch_commit makes
 * every staged scene resident (sort + deposit) in one pass. */
int rfmm_batch_upload(rfmm_batch *b, uint32_t scene, const void *host_aos, size_t bytes);
int rfmm_batch_upload_device(rfmm_batch *b, uint32_t scene, const void *device_aos, size_t bytes);
/* Stage every scene at once: device_aos[s] holds scene s's bodies (32 B each,
 * caller order) in device memory; one copy launch for all scenes instead of
 * one call per scene. */
int rfmm_batch_upload_device_all(rfmm_batch *b, const void *const *device_aos);
int rfmm_batch_seed_galaxy(rfmm_batch *b, uint32_t scene);
int rfmm_batch_commit(rfmm_batch *b);
int rfmm_batch_solve_fields(rfmm_batch *b);
int rfmm_batch_step(rfmm_batch *b, uint32_t steps);
int rfmm_batch_sync(rfmm_batch *b);
int rfmm_batch_download(rfmm_batch *b, uint32_t scene, int which, void *host_dst, size_t bytes);
/* Every scene's buffer `which` at once: host_dst[s] receives scene s's
 * buffer (sized as for rfmm_batch_download); one synchronisation in total
 * instead of one per scene. */
int rfmm_batch_download_all(rfmm_batch *b, int which, void *const *host_dst);
int rfmm_batch_download_device(rfmm_batch *b, uint32_t scene, int which, void *device_dst,
                               size_t bytes);
int rfmm_batch_digest(rfmm_batch *b, uint32_t scene, int which, uint32_t *out);
int rfmm_batch_launch_count(rfmm_batch *b, uint64_t *out);
int rfmm_batch_profile_steps(rfmm_batch *b, uint32_t steps, float *kernel_ms, uint32_t *launches);
int rfmm_batch_set_timeline(rfmm_batch *b, uint32_t enable);
int rfmm_batch_get_timeline(rfmm_batch *b, rfmm_timeline *out);
int rfmm_batch_set_resort_interval(rfmm_batch *b, uint32_t steps);
int rfmm_batch_set_near_mode(rfmm_batch *b, uint32_t mode);
int rfmm_batch_set_float_mode(rfmm_batch *b, uint32_t mode);
int rfmm_batch_get_tuning(rfmm_batch *b, rfmm_tuning *out);
int rfmm_batch_set_tuning(rfmm_batch *b, const rfmm_tuning *tuning);
int rfmm_batch_autotune(rfmm_batch *b, uint32_t steps_per_trial, rfmm_tuning *best);
int rfmm_batch_force_error(rfmm_batch *b, uint32_t scene, uint32_t targets, uint64_t seed,
                           double *rms_rel, double *max_rel);

/* ------------------------------------------------------------------ serving
 *
 * Continuous batching of solve requests (scene + parameters + step count).
 * The server preallocates slots of `max_bodies` capacity within the device
 * memory budget; a request waits until a slot is free, is admitted at the
 * next step boundary while other requests keep running, and every step
 * advances all occupied slots in the same launches.  Results are
 * bit-identical to a plain solve of the same scene.  Submit, status, wait and
 * result may be called from any thread. */
typedef struct rfmm_server rfmm_server;

typedef struct rfmm_server_config {
  uint64_t memory_budget_bytes; /* device memory the slots may use */
  uint32_t max_bodies;          /* slot capacity = largest admissible request */
  uint32_t max_slots;           /* 0 = as many as the budget allows (<= 4096) */
  uint32_t max_chunk_steps;     /* steps between admission points (0 = 4) */
  uint64_t staging_bytes;       /* pinned host memory for request inputs (3/4) and
                                 * results (1/4); 0 = 4 GiB */
  uint32_t float_mode;          /* RFMM_FLOAT_EXACT (0) or RFMM_FLOAT_FAST for every request */
  uint32_t timeline;            /* 1: record the step kernels' in-graph timeline
                                 * (rfmm_server_get_timeline) */
} rfmm_server_config;

typedef struct rfmm_server_stats {
  uint64_t submitted, completed, queued, in_flight;
  uint32_t slots, slot_capacity;
  uint64_t device_bytes;
  double p50_ms, p99_ms, mean_ms, max_ms; /* arrival -> result in host memory */
  double body_steps_per_s;                /* completed work / (last done - first arrival) */
  double body_steps;
  uint64_t chunks;                        /* batched step chunks run */
  double mean_active_slots;               /* occupied slots per chunk, on average */
  uint64_t pageable_inputs;               /* requests whose input missed the pinned ring */
  /* Where the worker thread's time went: waiting for the GPU (the run-ahead
   * bound and list-buffer reuse), admitting slots (sort + deposit enqueue),
   * rebuilding the active lists, enqueuing steps, retiring finished slots. */
  double worker_gpu_wait_ms, worker_admit_ms, worker_lists_ms, worker_step_ms, worker_retire_ms;
  /* Device time of the batched step chunks, and from the end of one chunk to
   * the start of the next (admissions, list copies, retirements, and any
   * time the GPU waited for the worker), from events around every chunk
   * (all but the last few chunks). */
  double gpu_step_ms, gpu_between_ms;
} rfmm_server_stats;

enum rfmm_request_state { RFMM_REQ_QUEUED = 0, RFMM_REQ_RUNNING = 1, RFMM_REQ_DONE = 2, RFMM_REQ_FAILED = 3 };

int rfmm_server_create(const rfmm_server_config *config, rfmm_server **out);
/* The step kernels' timeline (the most recent run of each captured graph)
 * when the server was created with timeline = 1; waits for the worker's
 * current iteration. */
int rfmm_server_get_timeline(rfmm_server *server, rfmm_timeline *out);
int rfmm_server_destroy(rfmm_server *server);
/* Copies the n bodies (n x 32 B) before it returns (into a pinned staging
 * buffer when one is free); returns RFMM_ERR_BUDGET if n exceeds the slot
 * capacity.  The request's latency runs from the entry into this call. */
int rfmm_server_submit(rfmm_server *server, const void *host_aos, uint32_t n,
                       const rfmm_params *params, uint32_t steps, uint64_t *request_id);
/* The same, with the request's arrival time given on rfmm_server_clock's
 * clock (seconds): latency runs from `arrival_s` instead of the call, so a
 * load generator replaying an arrival schedule measures from the scheduled
 * arrival even when its call starts late (no coordinated omission). */
int rfmm_server_submit_at(rfmm_server *server, const void *host_aos, uint32_t n,
                          const rfmm_params *params, uint32_t steps, double arrival_s,
                          uint64_t *request_id);
/* The server's clock (monotonic seconds). */
int rfmm_server_clock(double *now_s);
int rfmm_server_status(rfmm_server *server, uint64_t request_id, int *state);
/* RFMM_ERR_TIMEOUT if the request is not done within timeout_ms. */
int rfmm_server_wait(rfmm_server *server, uint64_t request_id, uint32_t timeout_ms);
/* Copies the final bodies (caller's order, n x 32 B) and forgets the request. */
int rfmm_server_result(rfmm_server *server, uint64_t request_id, void *host_dst, size_t bytes);
int rfmm_server_get_stats(rfmm_server *server, rfmm_server_stats *out);

/* Allocation-free field solve (this entry point has no counterpart in the
 * reference).  For callers that cannot allocate device memory -- a plugin
 * whose device memory is owned by the host framework, or code running where
 * a cudaMalloc would synchronise the device -- it computes exactly what
 * rfmm_solve_fields followed by rfmm_download_device(MOMENTS / FIELDS)
 * computes, on caller-owned device buffers: `device_particles` (n x 32 B,
 * reference Particle layout), `device_moments` (C x 16 B) and
 * `device_fields` (C x 48 B), C = total_cells(depth) of the unclamped plan
 * (rainbow_plan_depth_unclamped).  All pointers 16-byte aligned; `params`
 * may be NULL for the harness defaults; `stream` is a cudaStream_t (NULL =
 * default stream).  Work is enqueued asynchronously on `stream`.
 *
 * It calls no cudaMalloc/cudaFree: its intermediate data lives in one fixed
 * __device__ array of about 7.9 MB that every GPU loading this library holds
 * until exit, so n is limited to 1..131072 (tree depth 4 or 5); larger n
 * returns RFMM_ERR_INVALID.  Every call reuses that one array: calls that
 * overlap on the GPU race on it.  The first call on a device does a one-time
 * set-up (resolving the array's device address, encoding TMA descriptors);
 * make that first call before any stream capture.
 *
 * The call returns once its work is enqueued, so a kernel-side error (a
 * bounded TMA wait that gave up, a work list over its capacity) cannot be
 * its return value: it is left in the array's status word, which the next
 * call clears.  Read it with rfmm_noalloc_device_error after the call's work
 * and before the next call. */
int rfmm_solve_fields_noalloc(const void *device_particles, uint32_t n, const rfmm_params *params,
                              void *device_moments, void *device_fields, void *stream);

/* Status word of the last rfmm_solve_fields_noalloc call on the current
 * device (no counterpart in the reference; companion of the entry point
 * above).  Waits for the work queued on `stream` (a cudaStream_t, NULL = the
 * default stream), then copies the word: *code 0 = no error, 1 = a bounded
 * TMA wait gave up, 2 = a work list overflowed; *info is its detail.
 * Returns RFMM_OK, RFMM_ERR_TIMEOUT (code 1) or RFMM_ERR_DEVICE (other
 * codes).  Allocates nothing. */
int rfmm_noalloc_device_error(uint32_t *code, uint32_t *info, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* RFMM_H */
