/*
 * hairsim.h -- C-ABI of the GB300 hair-strand simulation step.
 *
 * This library replaces the compute pass that tcoppex/barbu runs every frame
 * for its hair (src/fx/hair.cc:89-125 dispatching
 * src/shaders/hair/01_simulation/cs_simulation.glsl). The entry points follow
 * the reference's `class Hair` (src/fx/hair.h:24-121) one for one:
 *
 *   Hair::init()                  src/fx/hair.h:61    -> hs_create
 *   Hair::deinit()                src/fx/hair.h:64    -> hs_groom_destroy / hs_destroy
 *   Hair::setup(scalp)            src/fx/hair.h:67    -> hs_groom_init
 *   Hair::set_bounding_sphere(v4) src/fx/hair.h:72-74 -> hs_set_bounding_sphere
 *   Hair::update(dt)              src/fx/hair.h:69    -> hs_update
 *   Hair::initialized()           src/fx/hair.h:76-78 -> hs_groom_info (nstrands != 0)
 *   pbuffer_.read_ssbo_id()       src/memory/pingpong_buffer.h:49
 *                                                     -> hs_device_positions / hs_readback
 *
 * Everything is plain C: pointers, sizes and POD structs, no CUDA or torch
 * types. Host arrays passed in are copied during the call; the caller keeps
 * ownership. Device memory is owned by the library.
 *
 * Errors: every call returns an hs_status and never aborts. The text of the
 * last error on the calling thread is returned by hs_last_error_string().
 * The reference logs and returns early instead (src/fx/hair.cc:45-48, :90-93).
 *
 * Threading: one hs_ctx per host thread, or external synchronisation. All
 * device work of a context is ordered on the context's CUDA stream;
 * hs_update() is asynchronous, readbacks and hs_sync() synchronise. A call
 * runs on its context's device (the one current at hs_create) whichever
 * device the calling thread has selected, and leaves that selection as it
 * found it.
 */
#ifndef HAIRSIM_H_
#define HAIRSIM_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define HS_API __attribute__((visibility("default")))
#else
#define HS_API
#endif

/* Limits. The reference fixes 4 points per strand at compile time
 * (src/shaders/hair/interop.h:8) and one collision sphere
 * (cs_simulation.glsl:43); here both are per-groom runtime values. */
#define HS_MIN_POINTS_PER_STRAND 2
#define HS_MAX_POINTS_PER_STRAND 64
#define HS_MAX_SPHERES 32
#define HS_MAX_BONES 8
#define HS_MAX_SUBSTEPS 64
#define HS_MAX_ITERATIONS 64

typedef enum hs_status {
  HS_OK = 0,
  HS_ERR_INVALID_ARG = 1,
  HS_ERR_OUT_OF_MEMORY = 2,
  HS_ERR_ADMISSION_DENIED = 3,
  HS_ERR_CUDA = 4,
  HS_ERR_TIMEOUT = 5,
  HS_ERR_NOT_INITIALIZED = 6,
  HS_ERR_UNSUPPORTED = 7
} hs_status;

/* Simulation semantics.
 * HS_MODE_REFERENCE reproduces cs_simulation.glsl:170-207: one prediction
 * per frame (S = 1), `iterations` (8) rounds of follow-the-leader length
 * projection then sphere push-out, velocity := the tip-ward shifted, damped
 * FTL correction (:119-121), reflected on contact (:137).
 * HS_MODE_DFTL is Mueller et al. 2012 with S substeps: predict with gravity
 * and wind, FTL projection root to tip, sphere push-out, then the velocity
 * of Eq. 9, v_i = (p_i - x_i)/h - damping * d_{i+1}/h. */
typedef enum hs_mode { HS_MODE_REFERENCE = 0, HS_MODE_DFTL = 1 } hs_mode;

/* Where the root control point goes each substep.
 * PINNED   : stays where it is (the reference: identity model, :188-192).
 * RIGID    : target = M * rest_root, M from hs_set_root_transform.
 * EXPLICIT : target given per strand by hs_set_roots.
 * SKINNED  : target = dual-quaternion blend of the rest root over up to
 *            four bones (hs_set_skin, hs_set_bone_matrices).
 * Within a frame the root moves linearly from its position at the start of
 * the frame to the target, reaching it at the last substep. */
typedef enum hs_root_mode {
  HS_ROOT_PINNED = 0,
  HS_ROOT_RIGID = 1,
  HS_ROOT_EXPLICIT = 2,
  HS_ROOT_SKINNED = 3
} hs_root_mode;

/* How hs_groom_init lays the control points out along the root normal.
 * REFERENCE : offset_i = i * (max_length / N) * rv, restlength_i =
 *             offset_i - offset_{i-1} (src/fx/hair.cc:262-288), with
 *             rv = 1 + length_jitter * (1 - 2u), u a seeded hash in [0,1)
 *             in place of the reference's time-seeded rand().
 * TOTAL     : the strand's total length L (lengths[s] if given, else
 *             max_length * rv) is split in N-1 equal segments. */
typedef enum hs_length_rule { HS_LENGTH_REFERENCE = 0, HS_LENGTH_TOTAL = 1 } hs_length_rule;

typedef struct hs_strand_params {
  uint32_t points_per_strand; /* N, HS_MIN..HS_MAX_POINTS_PER_STRAND (reference: 4) */
  uint32_t length_rule;       /* hs_length_rule */
  float max_length;           /* reference Parameters_t::sim.maxlength = 0.5 */
  float length_jitter;        /* reference 0.1 */
  uint64_t seed;              /* seeds length and wind jitter hashes */
  const float* lengths;       /* optional, nstrands total lengths (TOTAL rule) */
  uint32_t strand_base;       /* index of the first strand in the whole groom, when a
                                 groom is split across processes: the per-strand hashes
                                 use base + local index, so shards match the whole */
  uint32_t keep_order;        /* 0: the groom stores its strands in a spatial (Z-order)
                                 order of their roots, whatever order the caller gives
                                 them in; every input and output of the API stays in the
                                 caller's order (hs_groom_strand_order gives the map).
                                 Nonzero: stored in the caller's order. Results are the
                                 same either way: strands do not interact. */
} hs_strand_params;

typedef struct hs_sim_params {
  uint32_t mode;          /* hs_mode */
  uint32_t substeps;      /* S >= 1; reference 1 */
  uint32_t iterations;    /* FTL+collision rounds per substep; reference 8 */
  uint32_t root_mode;     /* hs_root_mode */
  float gravity[3];       /* (0,-9.81,0) (cs_simulation.glsl:71) */
  float gravity_scale;    /* reference kForceCoeff = 20 (:72) */
  float damping;          /* reference mix(0.80,0.94,0) = 0.80 (:100-102) */
  float length_scale;     /* reference uScaleFactor (:41), set to lengthScale */
  float wind_jitter;      /* per-strand wind factor 1 +- wind_jitter */
  uint32_t contract;      /* hs_contract: the chain link's arithmetic (DFTL); 0 = EXACT */
} hs_sim_params;

/* Arithmetic of the DFTL step's reciprocal square roots: the chain link's
 * (most of a point-substep's work) and the sphere push-out's normal.
 * EXACT: a fixed sequence of rounded float operations (magic-constant
 *        estimate, two Newton steps, a residual correction), which the
 *        FP32 oracle repeats bit for bit on the CPU. The default.
 * FAST : the GPU's reciprocal square root instruction (PTX rsqrt.approx),
 *        two instructions instead of thirteen. Frames are held to
 *        the DFTL tolerances against FP64 and to a bound against the EXACT
 *        contract, not bit for bit; the same inputs give the same frames
 *        on one GPU model. DFTL mode only. */
typedef enum hs_contract { HS_CONTRACT_EXACT = 0, HS_CONTRACT_FAST = 1 } hs_contract;

/* Device layout of a groom's state, returned by hs_device_positions.
 * Structure of arrays [point][strand]: point i of STORED strand j is the
 * float4 at index i * strand_stride + j, for both positions
 * (x,y,z,restlength) and velocities (x,y,z,0). strand_stride >= nstrands,
 * a multiple of 32. Stored strand j is the caller's strand order[j]
 * (hs_groom_strand_order; the identity with keep_order). */
typedef struct hs_layout {
  uint32_t nstrands;
  uint32_t points_per_strand;
  uint32_t strand_stride;
  uint32_t reserved;
} hs_layout;

typedef struct hs_ctx hs_ctx;
typedef struct hs_groom hs_groom;

/* ---- context ----------------------------------------------------------- */

/* Creates a context on the current CUDA device with its own stream
 * (Hair::init, src/fx/hair.cc:26-40). */
HS_API hs_status hs_create(hs_ctx** out_ctx);
/* Destroys the context and every groom still attached to it. */
HS_API hs_status hs_destroy(hs_ctx* ctx);
/* Text of the last error raised on the calling thread ("" if none). */
HS_API const char* hs_last_error_string(void);
/* The context's CUDA stream (a cudaStream_t), for callers that order their
 * own work after the simulation. */
HS_API hs_status hs_ctx_stream(hs_ctx* ctx, void** out_stream);
/* Blocks until all work queued on the context has finished. */
HS_API hs_status hs_sync(hs_ctx* ctx);
/* Number of kernels the context has launched so far. */
HS_API hs_status hs_ctx_launch_count(hs_ctx* ctx, uint64_t* out_count);

/* Parameter presets: the constants cs_simulation.glsl hard-codes, and the
 * DFTL defaults (S = 4, damping 0.9, gravity x1). */
HS_API void hs_sim_params_reference(hs_sim_params* p);
HS_API void hs_sim_params_dftl(hs_sim_params* p);
HS_API void hs_strand_params_reference(hs_strand_params* p);

/* ---- grooms ------------------------------------------------------------- */

/* Hair::setup + Hair::init_simulation (src/fx/hair.cc:42-64, :236-361):
 * one strand per root, N control points laid along the root normal.
 * root_pos, root_nrm: nstrands * 3 floats (host). */
HS_API hs_status hs_groom_init(hs_ctx* ctx, const float* root_pos, const float* root_nrm,
                               uint32_t nstrands, const hs_strand_params* strand,
                               const hs_sim_params* sim, hs_groom** out_groom);
/* Creates a groom from a full state in the renderer's strand-major layout:
 * pos_xyzw, vel_xyzw are nstrands * npoints * 4 floats, point i of strand s
 * at (s * npoints + i) * 4. Rest roots (for RIGID) are the given roots. */
HS_API hs_status hs_groom_init_from_state(hs_ctx* ctx, const float* pos_xyzw, const float* vel_xyzw,
                                          uint32_t nstrands, uint32_t npoints, uint64_t seed,
                                          const hs_sim_params* sim, hs_groom** out_groom);
HS_API hs_status hs_groom_destroy(hs_groom* groom);
HS_API hs_status hs_groom_set_params(hs_groom* groom, const hs_sim_params* sim);
HS_API hs_status hs_groom_info(const hs_groom* groom, uint32_t* out_nstrands, uint32_t* out_npoints);

/* ---- per-frame inputs (take effect at the next update) ----------------- */

/* Hair::set_bounding_sphere (src/fx/hair.h:72-74): one sphere (x,y,z,r). */
HS_API hs_status hs_set_bounding_sphere(hs_groom* groom, const float xyzr[4]);
/* Replaces the collision sphere list: n <= HS_MAX_SPHERES spheres (x,y,z,r),
 * tested in order. */
HS_API hs_status hs_set_spheres(hs_groom* groom, const float* xyzr, uint32_t n);
/* Wind force per unit mass for the next frame (DFTL mode). */
HS_API hs_status hs_set_wind(hs_groom* groom, const float wind[3]);
/* Root transform for HS_ROOT_RIGID: 4x4 column-major (glm layout). */
HS_API hs_status hs_set_root_transform(hs_groom* groom, const float m[16]);
/* hs_set_root_transform for n grooms at once: m holds n column-major 4x4
 * matrices (16 * n floats), one per groom in list order. */
HS_API hs_status hs_set_root_transforms(hs_groom* const* grooms, uint32_t n, const float* m);
/* Root targets for HS_ROOT_EXPLICIT: nstrands * 3 floats (host). */
HS_API hs_status hs_set_roots(hs_groom* groom, const float* xyz, uint32_t nstrands);

/* Skinned roots (HS_ROOT_SKINNED): each frame's root target is the rest
 * root skinned by dual-quaternion blending, as the reference skins mesh
 * vertices (apply_skinning + skinning_DQBS, src/shaders/shared/inc_skinning.glsl:22-82;
 * Kavan et al. 2008). The reference never skins hair roots (its root
 * transform is the identity, cs_simulation.glsl:188-192); this is the
 * skinning stage a rigged scalp needs, computed inside the step kernel.
 * Influences per strand: 4 bone indices (< HS_MAX_BONES) and the first 3
 * weights; the 4th weight is 1 - (w0 + w1 + w2). A strand whose first
 * weight is <= 1e-6 keeps its rest root. Copied to the device (set-up). */
HS_API hs_status hs_set_skin(hs_groom* groom, const uint8_t* bones, const float* weights, uint32_t nstrands);
/* This frame's bone palette as unit dual quaternions, 8 floats per bone:
 * real (x, y, z, w) then dual (x, y, z, w), the layout the reference's
 * shader reads (inc_skinning.glsl:37-52). nbones <= HS_MAX_BONES. */
HS_API hs_status hs_set_bone_dual_quats(hs_groom* groom, const float* dq, uint32_t nbones);
/* Same from skinning matrices (global pose x inverse bind, rigid, 4x4
 * column-major), converted on the host as the reference does before
 * skinning (src/fx/animation/skeleton_controller.cc:248-265). */
HS_API hs_status hs_set_bone_matrices(hs_groom* groom, const float* m, uint32_t nbones);

/* ---- step --------------------------------------------------------------- */

/* Hair::update (src/fx/hair.cc:89-125): advances one frame of dt seconds.
 * Asynchronous on the context stream. */
HS_API hs_status hs_update(hs_groom* groom, float dt);

/* How hs_update maps a strand onto the GPU (results are bit-identical
 * either way).
 * THREAD: one thread per strand, its substeps one after the other.
 * LANES : a group of K lanes per strand, K the smallest power of two >= S,
 *         lane k running substep k as a wavefront (the reference spreads a
 *         strand over a work group, cs_simulation.glsl:89): S x N dependent
 *         steps become N + 3 (S - 1) + 1. DFTL mode with one iteration and
 *         2 <= S <= 16 only; hs_update fails with HS_ERR_UNSUPPORTED
 *         otherwise.
 * AUTO  : LANES for grooms too small to fill the GPU a thread per strand
 *         (and that LANES supports), THREAD otherwise. The default. */
typedef enum hs_mapping { HS_MAPPING_AUTO = 0, HS_MAPPING_THREAD = 1, HS_MAPPING_LANES = 2 } hs_mapping;
HS_API hs_status hs_groom_set_mapping(hs_groom* groom, uint32_t mapping);
/* The mapping the groom's next hs_update takes (THREAD or LANES). */
HS_API hs_status hs_groom_mapping(hs_groom* groom, uint32_t* out_mapping);

/* Batched update: advances every groom of the list by one frame of dt,
 * exactly as hs_update on each would (bit-identical results), in one CUDA
 * graph launch. Grooms are cut into 32-strand tiles, bucketed by point
 * count and mode, and each bucket runs as one persistent kernel. The graph
 * is captured on the first call for a given list and replayed after.
 * Replaces the per-groom glDispatchCompute of Hair::update
 * (src/fx/hair.cc:112) when many grooms are resident. */
HS_API hs_status hs_update_many(hs_ctx* ctx, hs_groom* const* grooms, uint32_t n, float dt);
/* Autotuner: times candidate launch shapes (warps per block, persistent
 * grid size) for every bucket of the list and keeps the fastest per
 * (point capacity, mode, size class) in the context; later hs_update_many
 * calls use them. The grooms' state is restored after the trials. */
HS_API hs_status hs_autotune(hs_ctx* ctx, hs_groom* const* grooms, uint32_t n, float dt, uint32_t* out_trials);

/* Kernel variants of a batched bucket (the autotuner's mapping choice).
 * Values 3-5 are not built and are rejected. */
typedef enum hs_variant {
  HS_VARIANT_REGISTERS = 0,        /* positions and velocities in registers (<= 8 points) */
  HS_VARIANT_REGISTERS_SHARED = 1, /* positions in registers, velocities in shared memory (<= 8) */
  HS_VARIANT_STREAM = 2,           /* state in shared memory, runtime point loop (<= 64) */
  HS_VARIANT_STREAM_TMEM = 6,      /* streaming, velocities in tensor memory (4 or 8 warps per block) */
  HS_VARIANT_LANES = 7             /* a lane group per strand, its substeps as a wavefront (hs_mapping
                                      LANES): warps per block = lanes per strand (2, 4, 8 or 16); DFTL
                                      buckets whose grooms all have one iteration and at most that
                                      many substeps, else the bucket takes the default shape */
} hs_variant;
/* Pins the launch shape hs_update_many uses for the point class of
 * `points` (the grooms with the same capacity: up to 4, 8, 16, 24, 32 or
 * 64 points per strand) in `mode`, all size classes, overriding the
 * autotuner and the defaults: variant, warps per block (1, 2, 4 or 8; 16 for LANES) and
 * persistent grid in waves of resident blocks (1, 2 or 4). Unpinned DFTL
 * grooms of up to 32 points share one flat bucket per contract (each
 * contract runs kernels of its own); a pinned class runs in a bucket of
 * its own with the pinned shape, under either contract. HS_ERR_UNSUPPORTED
 * where the variant is not built for that class or the shape does not fit
 * an SM. */
HS_API hs_status hs_tune_override(hs_ctx* ctx, uint32_t points, uint32_t mode, uint32_t variant,
                                  uint32_t warps_per_block, uint32_t waves);

/* Largest groom list hs_update_many_noalloc takes in one call. */
#define HS_NOALLOC_MAX_GROOMS 256

/* Batched update that allocates nothing. No counterpart in the reference.
 *
 * For callers that cannot allocate device memory once their grooms exist:
 * engines and renderers that reserve their GPU budget at load time and
 * forbid allocation in the frame loop (cudaMalloc/cudaFree can synchronise
 * the device and stall a frame, and hs_update_many grows its buffers when
 * the groom list grows). Same results as hs_update_many (bit-identical),
 * same arguments; the per-call scratch (tile counters, bucket directory,
 * groom table, about 310 KiB) lives in one fixed device array that every GPU
 * loading this library holds until exit. Lists longer than
 * HS_NOALLOC_MAX_GROOMS are rejected with HS_ERR_INVALID_ARG. The launch
 * shape is fixed: one bucket per (point capacity, mode), the streaming
 * variant at one warp per block, whatever hs_tune_override or hs_autotune
 * chose for hs_update_many.
 *
 * Each call looks up the array's device address on the context's device
 * (cudaGetSymbolAddress, no allocation), so it stays right after a
 * cudaDeviceReset; the first call on a device also reads the device's
 * launch limits: make it before any stream capture. Every call shares the
 * array; calls on one context stream are ordered, calls that overlap on the
 * GPU (other streams or contexts of the same device) race on it. */
HS_API hs_status hs_update_many_noalloc(hs_ctx* ctx, hs_groom* const* grooms, uint32_t n, float dt);

/* One autotuned launch shape (hs_tune_entries). */
typedef struct hs_tune_entry {
  uint32_t capacity;        /* point capacity of the bucket (4, 8, 16, 24, 32, 64) */
  uint32_t mode;            /* hs_mode */
  uint32_t tiles_log2;      /* size class: floor(log2(32-strand tiles)) */
  uint32_t variant;         /* hs_variant */
  uint32_t warps_per_block;
  uint32_t waves;
  float ms;                 /* best trial time of the bucket */
  uint32_t contract;        /* hs_contract of the bucket's grooms (DFTL; each contract has its own kernels) */
} hs_tune_entry;
/* Copies up to `capacity` entries of the context's autotuner cache;
 * *out_count is the number of entries in the cache. */
HS_API hs_status hs_tune_entries(hs_ctx* ctx, hs_tune_entry* out, uint32_t capacity, uint32_t* out_count);

/* ---- serving ------------------------------------------------------------ */

/* A served stream: grooms arrive (hs_server_submit), are admitted into a
 * device slab pool as bytes free up, are advanced together every tick
 * (hs_server_tick: one batched graph launch for all resident grooms), and
 * leave after their requested number of frames. No counterpart in the
 * reference, whose single Hair instance is set up once (src/fx/hair.cc:42). */
typedef struct hs_server hs_server;

typedef struct hs_server_config {
  uint64_t budget_bytes; /* device bytes of strand state resident at most */
  uint32_t max_grooms;   /* resident grooms at most (0: limited by the budget only) */
  uint32_t reserved;
} hs_server_config;

typedef struct hs_request {
  const float* root_pos; /* nstrands * 3 (host, copied by submit) */
  const float* root_nrm; /* nstrands * 3 */
  const float* lengths;  /* optional, nstrands total lengths (HS_LENGTH_TOTAL) */
  uint32_t nstrands;
  uint32_t frames;       /* frames to simulate; then the groom leaves */
  hs_strand_params strand; /* strand.lengths is ignored: use `lengths` */
  hs_sim_params sim;     /* root_mode PINNED, RIGID (hs_server_set_root_transform, identity
                            until set) or SKINNED (skin_* below, hs_server_set_bone_matrices) */
  const float* spheres;  /* nspheres * 4: the initial spheres (hs_server_set_spheres moves them) */
  uint32_t nspheres;
  uint32_t keep_result;  /* nonzero: hold the final state until hs_server_collect */
  float wind[3];         /* wind(t) = wind + (swing_amp sin(swing_omega t), 0, 0), */
  float swing_amp;       /* t = the groom's own elapsed time, so a groom's frames */
  float swing_omega;     /* do not depend on when it arrived or who shares the GPU */
  uint32_t reserved;
  const uint8_t* skin_bones;  /* SKINNED: nstrands * 4 bone indices (< HS_MAX_BONES), as hs_set_skin */
  const float* skin_weights;  /* SKINNED: nstrands * 3 weights (the 4th derived) */
} hs_request;

typedef enum hs_request_state {
  HS_REQ_QUEUED = 0,   /* waiting for room */
  HS_REQ_RESIDENT = 1, /* on the device, being advanced */
  HS_REQ_DONE = 2,     /* all frames done, result held for hs_server_collect */
  HS_REQ_GONE = 3      /* finished and released (or never existed) */
} hs_request_state;

typedef struct hs_tick_stats {
  uint32_t advanced;        /* grooms advanced this tick */
  uint32_t queued;          /* requests still waiting after the tick */
  uint32_t admitted;        /* admitted this tick (advanced from the next tick) */
  uint32_t retired;         /* left this tick */
  uint64_t resident_bytes;  /* slab bytes held after the tick */
  uint64_t point_substeps;  /* strands x points x substeps advanced this tick */
  double tick_ms;           /* host wall time of hs_server_tick, device work included */
} hs_tick_stats;

/* Creates a server on a context; reserves budget_bytes of device memory. */
HS_API hs_status hs_server_create(hs_ctx* ctx, const hs_server_config* cfg, hs_server** out_server);
HS_API hs_status hs_server_destroy(hs_server* srv);
/* Queues a request (arrays are copied). HS_ERR_ADMISSION_DENIED if the
 * groom alone exceeds the budget. */
HS_API hs_status hs_server_submit(hs_server* srv, const hs_request* req, uint64_t* out_ticket);
/* One tick of dt seconds: retire finished grooms, admit queued requests in
 * arrival order while the budget allows (their set-up overlaps this tick),
 * advance every active groom one frame; returns when the tick is done. */
HS_API hs_status hs_server_tick(hs_server* srv, float dt, hs_tick_stats* out_stats);
/* Per-tick inputs of a served groom, by ticket: its collision spheres, its
 * root transform (RIGID requests) or its bone palette as skinning matrices
 * (SKINNED requests, converted like hs_set_bone_matrices). They reach the
 * groom's next frame; on a request still queued they are kept and applied
 * when it is admitted. A skinned groom does not advance until it has a
 * palette. The reference feeds its groom a new bounding sphere every frame
 * (src/core/renderer.cc:69-81, Hair::set_bounding_sphere). HS_ERR_INVALID_ARG
 * for a request that is neither queued nor running, HS_ERR_UNSUPPORTED for
 * an input its root mode does not take. */
HS_API hs_status hs_server_set_spheres(hs_server* srv, uint64_t ticket, const float* xyzr, uint32_t n);
HS_API hs_status hs_server_set_root_transform(hs_server* srv, uint64_t ticket, const float m[16]);
HS_API hs_status hs_server_set_bone_matrices(hs_server* srv, uint64_t ticket, const float* m, uint32_t nbones);
HS_API hs_status hs_server_poll(hs_server* srv, uint64_t ticket, uint32_t* out_state, uint32_t* out_frames_done);
/* Copies a DONE request's final positions and velocities (strand-major,
 * nstrands * npoints * 4 floats each; either may be null) and releases it. */
HS_API hs_status hs_server_collect(hs_server* srv, uint64_t ticket, float* pos_xyzw, float* vel_xyzw,
                                   size_t capacity_floats);

/* ---- tessellation stream ----------------------------------------------- */

/* The reference's second pass (src/fx/hair.cc:145-170 with
 * src/shaders/hair/02_tess_stream/{vs,tcs,tes,gs}_stream_hair.glsl): every
 * scalp triangle and control segment j is an isoline patch of 6 control
 * points (points j, j+1 of the triangle's 3 strands, hair.cc:396-407);
 * each of `ninstances` instances tessellates it into `nlines` interpolated
 * strands of `nsubsegments` line segments: Hermite interpolation along the
 * segment (tes :37-39, inc_maths.glsl:210-228), a random point of the
 * triangle (sample_triangle2, inc_maths.glsl:107-115, coordinates from the
 * random buffer at (40 v + instance) mod 4096, tes :52-54), and the
 * relative position along the strand through smoothstep2 (tes :65-66,
 * inc_maths.glsl:263-266). The
 * geometry shader's line list (gs :20-28), captured by transform feedback
 * into a GL buffer in the reference, is written here into a device buffer
 * of float4 (x, y, z, relative position), 2 vertices per line segment, in
 * the order [instance][triangle][segment j][line][subsegment]. */
#define HS_TESS_RANDOM_SIZE 4096 /* HAIR_TF_RANDOMBUFFER_SIZE (interop.h:36) */

typedef struct hs_tess_params {
  uint32_t ninstances;   /* Parameters_t::tess.ninstances = 3 (1..16, HairView.h:38) */
  uint32_t nlines;       /* tess.nlines = 2 (1..16): tessellation level outer[0] (tcs :34) */
  uint32_t nsubsegments; /* tess.nsubsegments = 16 (1..16): level outer[1] (tcs :35) */
  float length_scale;    /* uScaleFactor = render.lengthScale = 1.45: scales tangents (tcs :41) */
} hs_tess_params;

HS_API void hs_tess_params_reference(hs_tess_params* p);
/* Static inputs of the pass: triangles (3 strand indices each), one
 * tangent per control point (x, y, z, w; strand-major, nstrands * N * 4
 * floats, the reference's tangent stream, hair.cc:290-326) and the random
 * buffer (HS_TESS_RANDOM_SIZE floats in [0, 1), random_buffer.cc:22-35). */
HS_API hs_status hs_tess_setup(hs_groom* groom, const uint32_t* faces, uint32_t nfaces, const float* tangents_xyzw,
                               const float* random, uint32_t nrandom);
/* Vertices one pass writes: 2 * ninstances * nfaces * (N - 1) * nlines * nsubsegments. */
HS_API hs_status hs_tess_count(const hs_groom* groom, const hs_tess_params* p, uint64_t* out_vertices);
/* Runs the pass on the groom's current positions into its tessellation
 * buffer (grown on demand). Asynchronous on the context stream. */
HS_API hs_status hs_tess_stream(hs_groom* groom, const hs_tess_params* p, uint64_t* out_vertices);
/* Zero-copy access to the last pass's vertices (valid until the next pass
 * or destroy). */
HS_API hs_status hs_tess_device(hs_groom* groom, const void** out_dptr, uint64_t* out_vertices);
/* Copies the last pass's vertices to host (4 floats each). Synchronises. */
HS_API hs_status hs_tess_readback(hs_groom* groom, float* host_xyzw, size_t capacity_floats);

/* ---- Marschner lookup tables -------------------------------------------- */

/* The reference's shading tables (src/fx/marschner.cc:33-67, Marschner et
 * al. 2003): M (cs_marschner_m.glsl: the R, TT, TRT longitudinal lobes and
 * cos(theta_d) over sin(theta_i) x sin(theta_r)) and N
 * (cs_marschner_n.glsl: the azimuthal N_R, N_TT, N_TRT over cos(phi_d) x
 * cos(theta_d)), resolution x resolution RGBA texels each, row y at
 * y * resolution. Written into the caller's device buffers, as half
 * (the reference's RGBA16F) or float, asynchronously on the context stream.
 * Either buffer may be null. */
typedef struct hs_marschner_params {
  float eta;             /* 1.55  (Marschner::ShadingParameters_t, src/fx/marschner.h:33) */
  float absorption;      /* 0.20 */
  float eccentricity;    /* 0.85 (not used by the tables) */
  float ar;              /* longitudinal shift, degrees: -5 */
  float br;              /* longitudinal width, degrees: +5 */
  float glint_scale;     /* 0.5  (not used by the tables) */
  float azimuthal_width; /* 10   (not used by the tables) */
  float delta_caustic;   /* 0.2  (not used by the tables) */
  float delta_hm;        /* 0.5  (not used by the tables) */
  uint32_t resolution;   /* 128 (kTextureResolution, :24) */
} hs_marschner_params;
typedef enum hs_lut_format { HS_LUT_HALF4 = 0, HS_LUT_FLOAT4 = 1 } hs_lut_format;
HS_API void hs_marschner_params_reference(hs_marschner_params* p);
HS_API hs_status hs_marschner_luts(hs_ctx* ctx, const hs_marschner_params* p, uint32_t format, void* d_m, void* d_n);

/* ---- output ------------------------------------------------------------- */

/* Per-groom reductions of the last frame, computed inside the step kernel
 * as it writes the state back (warp shuffles per 32-strand tile, tiles
 * combined here): bounds of the control points, kinetic energy and the
 * largest speed. For culling, stability monitoring and bounding volumes.
 * Synchronises the context stream. `valid` is 0 before the first update. */
typedef struct hs_frame_stats {
  float bounds_min[3];
  float bounds_max[3];
  float max_speed;        /* largest |v| of a control point */
  uint32_t valid;
  double kinetic_energy;  /* sum over control points of 0.5 |v|^2 (unit mass) */
} hs_frame_stats;
HS_API hs_status hs_groom_stats(hs_groom* groom, hs_frame_stats* out);


/* Copies positions (x,y,z,restlength) to host in the renderer's
 * strand-major layout (src/fx/hair.cc:369-392): capacity_floats >=
 * nstrands * N * 4. Synchronises the context stream. */
HS_API hs_status hs_readback(hs_groom* groom, float* host_xyzw, size_t capacity_floats);
/* Same for velocities (x,y,z,0). */
HS_API hs_status hs_readback_velocities(hs_groom* groom, float* host_xyzw, size_t capacity_floats);
/* Asynchronous hs_readback, for a frame loop that overlaps the copy of
 * frame f with the update of frame f + 1 (the reference renders from
 * device memory and reads nothing back; this is the host-side consumer's
 * path). Enqueues, after the updates queued before it, a device snapshot
 * of the positions in the same strand-major layout and its copy to
 * host_xyzw on a second stream of the context, and returns at once. The
 * host buffer holds the frame when hs_readback_wait returns; it must stay
 * valid and unread until then, and be page-locked (pinned) memory for the
 * copy to run asynchronously. The groom stages its snapshots in two buffers
 * taken in turn: a third readback in flight waits on the device for the
 * first one's copy. */
HS_API hs_status hs_readback_async(hs_groom* groom, float* host_xyzw, size_t capacity_floats);
/* Positions without the rest length: (x, y, z) per control point in the
 * same strand-major order, 12 bytes a point (capacity_floats >=
 * nstrands * N * 3). The rest lengths do not change from frame to frame;
 * a host consumer that took them once (hs_readback) moves a quarter fewer
 * bytes per frame. Blocking, and queued like hs_readback_async. */
HS_API hs_status hs_readback_xyz(hs_groom* groom, float* host_xyz, size_t capacity_floats);
HS_API hs_status hs_readback_xyz_async(hs_groom* groom, float* host_xyz, size_t capacity_floats);
/* Several grooms of the context in one call: each groom's positions,
 * strand-major like hs_readback_async ((x, y, z) per point with comps = 3,
 * (x, y, z, rest length) with comps = 4), one after the other in list
 * order in one host buffer (capacity_floats >= comps * the sum of nstrands
 * * N). The snapshots go to a staging buffer of the context and reach the
 * host in one copy on the copy stream; asynchronous like
 * hs_readback_async, with the same rules for the host buffer. */
HS_API hs_status hs_readback_many_async(hs_ctx* ctx, hs_groom* const* grooms, uint32_t n, uint32_t comps,
                                        float* host, size_t capacity_floats);
/* Waits for every asynchronous readback of the context. */
HS_API hs_status hs_readback_wait(hs_ctx* ctx);
/* Waits until at most `keep` of the context's asynchronous readbacks
 * (hs_readback_async, _xyz_async, _many_async) are still in flight, the
 * oldest first: a consumer that queues the readback of frame f + 1 and then
 * drains to 1 holds frame f while frame f + 1's snapshot and copy run. Each
 * groom, and the context's batched readback, stage in two buffers taken
 * in turn, so two readbacks in flight never wait for each other on the
 * device; a third waits for the first. */
HS_API hs_status hs_readback_drain(hs_ctx* ctx, uint32_t keep);
/* Zero-copy access: device pointer to the [point][strand] position array.
 * Valid until the groom is destroyed; contents change with each update. */
HS_API hs_status hs_device_positions(hs_groom* groom, const void** out_dptr, hs_layout* out_layout);
/* The groom's stored strand order: out[j] = the caller's index of stored
 * strand j (the column j of hs_device_positions), for j < min(capacity,
 * nstrands); *out_count = nstrands. The identity when the groom was made
 * with keep_order. */
HS_API hs_status hs_groom_strand_order(hs_groom* groom, uint32_t* out, uint32_t capacity, uint32_t* out_count);

/* Device-to-device export of the state into a caller's buffer (for
 * example a graphics buffer mapped for CUDA), asynchronous on the context
 * stream, ordered after the updates queued before it. The reference's
 * renderer reads positions strand-major from the read half of its
 * ping-pong buffer (src/fx/hair.cc:369-392), which PingPongBuffer::swap
 * refreshes by a device copy every frame (src/memory/pingpong_buffer.cc:73-84);
 * here the state is updated in place and exported on demand.
 * layout STRAND_MAJOR: point i of strand s at s * N + i (the reference's);
 * POINT_MAJOR: at i * nstrands + s (point-major, unpadded), s the
 * caller's strand index in both layouts.
 * d_dst must be 16-byte aligned and hold nstrands * N * 4 floats. */
typedef enum hs_export_layout { HS_EXPORT_STRAND_MAJOR = 0, HS_EXPORT_POINT_MAJOR = 1 } hs_export_layout;
typedef enum hs_export_field { HS_FIELD_POSITIONS = 0, HS_FIELD_VELOCITIES = 1 } hs_export_field;
HS_API hs_status hs_export(hs_groom* groom, uint32_t field, uint32_t layout, void* d_dst, size_t capacity_floats);

#ifdef __cplusplus
}
#endif

#endif /* HAIRSIM_H_ */
