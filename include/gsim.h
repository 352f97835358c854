/*
 * gsim.h -- C ABI of the GB300 force-and-integrate path for Gravity-Sim.
 *
 * One gs_sim replaces one reference simulation object plus the particle buffers it
 * drives (paths relative to the reference project):
 *   gs_create      ParticleSystem(...) ctor (src/Particles/ParticleSystem.hpp:58,72) followed by
 *                  DirectSimulation(device, system) (src/Simulation/Direct/DirectSimulation.hpp:11-81)
 *                  or BarnesHutSimulation(device, system) (src/Simulation/BarnesHut/BarnesHutSimulation.hpp:11-110)
 *   gs_run         RunSimulations(uint32_t) (src/Simulation/Direct/DirectSimulation.cpp:271,
 *                  src/Simulation/BarnesHut/BarnesHutSimulation.cpp:849)
 *   gs_sync        the simulation fence wait of the destructor and vkDeviceWaitIdle (src/Main.cpp:286)
 *   gs_get_particles  ParticleSystem::GetParticles (src/Particles/ParticleSystem.hpp:178)
 *   gs_destroy     ~DirectSimulation / ~BarnesHutSimulation + ~ParticleSystem
 *   gs_required_alignment  GetRequiredParticleAlignment() (src/Simulation/Direct/DirectSimulation.cpp:26-28,
 *                  src/Simulation/BarnesHut/BarnesHutSimulation.cpp:834-836)
 *   gs_read_particles / gs_write_particles  ParticleSystem file ctor and SaveParticles
 *                  (src/Particles/ParticleSystem.cpp:438-501, 727-750)
 *   gs_generate    the four generators (src/Particles/ParticleSystem.cpp:15-149), seeded
 *
 * Conventions: every call returns a gs_status; nothing throws across the ABI.  Host
 * arrays are caller-owned, interleaved x,y for vectors, and hold the first N particles
 * (the library pads to the required alignment with zero particles, like the reference,
 * src/Particles/ParticleSystem.cpp:487-491).  Device state is library-owned and stays
 * resident between calls.  Every gs_sim owns one CUDA stream; gs_run is asynchronous.
 */
#ifndef GSIM_H
#define GSIM_H

#include <stdint.h>

#if defined(__GNUC__)
#define GS_API __attribute__((visibility("default")))
#else
#define GS_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gs_status {
    GS_OK = 0,
    GS_ERR_INVALID_ARGUMENT = 1,
    GS_ERR_CUDA = 2,
    GS_ERR_OUT_OF_MEMORY = 3,
    GS_ERR_TIMEOUT = 4,
    GS_ERR_DEVICE = 5,   /* a kernel reported an error (e.g. a bounded wait ran out) */
    GS_ERR_IO = 6,
    GS_ERR_CAPACITY = 7, /* a size limit of the library was exceeded */
    GS_ERR_NO_DEVICE = 8
} gs_status;

/* ParticleSystem::SimulationAlgorithm (src/Particles/ParticleSystem.hpp:27-34). */
typedef enum gs_algorithm { GS_DIRECT_SUM = 0, GS_BARNES_HUT = 1 } gs_algorithm;

/* Barnes-Hut box: the reference's fixed +-500 box with a 1024x1024 finest grid and
 * removal of particles that leave it, or a per-step square bounding box with
 * 2^k x 2^k finest cells (gs_params.key_bits = k: 12 by default, 24-bit Morton keys; 15
 * gives 30-bit keys) and no removal. */
typedef enum gs_box_mode { GS_BOX_FIXED_500 = 0, GS_BOX_BOUNDING = 1 } gs_box_mode;

/* FAST: hardware rsqrt; direct sum in shared-memory tiles with Kahan-compensated
 * tile partials.  REFERENCE: correctly rounded 1/sqrt and the shaders' summation
 * order, bit-identical to the CPU restatement. */
typedef enum gs_math_mode { GS_MATH_FAST = 0, GS_MATH_REFERENCE = 1 } gs_math_mode;

/* gs_params.flags */
#define GS_FLAG_RECORD_ACCEL 0x1u  /* keep the last step's accelerations (gs_get_accel) */
#define GS_FLAG_PROFILE 0x2u       /* time each stage with CUDA events (gs_get_stats) */
#define GS_FLAG_NO_GRAPH 0x4u      /* launch kernels one by one instead of a CUDA graph */
#define GS_FLAG_COUNT_INTERACTIONS 0x8u /* count accepted Barnes-Hut interactions */
/* Accurate Barnes-Hut mode (no counterpart in the reference, whose opening rule
 * s^2/2 <= d^2 theta^2 with monopoles is tens of percent off at theta = 1).  The tree
 * (keys, order, topology) is unchanged; these flags add:
 *   QUADRUPOLE   second central moments per node, quadrupole term for accepted nodes;
 *                every node's mass, centre of mass and second moments come from exact
 *                integer sums over its particles (masses on a grid of 2^-31 of the
 *                largest, positions of 2^-30 of the box half-size; masses <= 0 count
 *                as 0), rounded to FP32 once, so they do not depend on the order in
 *                which particles are added (the reference's FP32 child sums do)
 *   SAFE_RADIUS  opening radius = squared distance from the centre of mass to the
 *                farthest cell corner (equals s^2/2 for a centred mass)
 *   GROUP_WALK   each warp's 64 particles (two per lane) share one walk that tests
 *                records against up to four sub-boxes of the group, 32 records at a
 *                time, and sums interaction items densely
 * GS_FLAGS_ACCURATE sets all three (theta = 0.3 gives <= 1e-3 RMS force error on the
 * 500k spiral at most steps; GS_FLAG_RELATIVE_MAC below does so at every step). */
#define GS_FLAG_QUADRUPOLE 0x10u
#define GS_FLAG_SAFE_RADIUS 0x20u
#define GS_FLAG_GROUP_WALK 0x40u
#define GS_FLAGS_ACCURATE 0x70u
/* Direct sum, FAST math: add the 64-wide tile partials and the j-chunks plainly instead
 * of with Kahan compensation (the precision study's uncompensated variant). */
#define GS_FLAG_PLAIN_SUM 0x80u
/* Barnes-Hut with GS_FLAG_GROUP_WALK and GS_FLAG_QUADRUPOLE: open nodes by the relative
 * criterion instead of theta.  A node of mass m and opening radius r (the stored squared
 * radius R = r^2) is accepted for a group at softened squared distance D = d^2 + eps^2
 * from the group's nearest sub-box when
 *     R <= D   and   m^2 R^3 <= (alpha a_min)^2 D^5
 * i.e. m r^3 / d^5 (the size of the first term a quadrupole expansion leaves out) is at
 * most alpha times the smallest |a| the group's particles had in the previous step
 * (without G) -- or when R <= D theta_f^2: the floor theta_f bounds the walk of a group
 * whose smallest |a| is tiny (near the centre of a disk, or where neighbours cancel the
 * field).  alpha is gs_params.relative_accuracy, theta_f gs_params.relative_theta_floor
 * (0: theta).  A group with no previous |a| for some particle (every group in the first
 * step after gs_create or gs_set_particles) first estimates its particles' |a| by a walk
 * with the theta test (accuracy_parameter; the reference's theta = 1 is enough), then
 * opens nodes by the relative criterion with those estimates.  alpha = 0.006 with floor
 * 0.2 gives <= 8e-4 RMS force error at every step on the 500k spiral and on uniform disks
 * at rest, measured on 4096-17000-particle samples against the FP64 direct sum.
 * In a system of at least 2^18 (padded) particles, a group whose previous |a| are all
 * known and whose smallest is below a tenth of its largest is walked by two warps:
 * 64-record pops, and item i of its node (leaf) list summed by warp (i / 32) mod 2 from
 * zero, the two partial sums added -- the same interactions, in another summation order
 * (alone and in a batch alike). */
#define GS_FLAG_RELATIVE_MAC 0x100u

typedef struct gs_params {
    float gravitational_const; /* ParticleSystem::GetGravitationalConst, default 1 (src/Main.cpp:59) */
    float simulation_time;     /* GetSimulationTime, default 1e-3 */
    float simulation_speed;    /* GetSimulationSpeed, default 1 (Barnes-Hut only, as in the reference) */
    float softening_len;       /* GetSofteningLen, default 0.2 */
    float accuracy_parameter;  /* GetAccuracyParameter (theta), default 1 */
    int32_t algorithm;         /* gs_algorithm */
    int32_t box_mode;          /* gs_box_mode, Barnes-Hut only */
    int32_t math_mode;         /* gs_math_mode */
    int32_t device;            /* CUDA device ordinal */
    uint32_t flags;            /* GS_FLAG_* */
    float relative_accuracy;   /* alpha of GS_FLAG_RELATIVE_MAC, default 0.006 */
    float relative_theta_floor; /* theta floor of GS_FLAG_RELATIVE_MAC, default 0: accuracy_parameter */
    int32_t key_bits;          /* GS_BOX_BOUNDING: Morton bits per axis, 1..15 (default 12: 24-bit keys
                                  in 3 radix passes; 15: 30-bit keys in 4); 0 means 12.  The reference's
                                  fixed box uses 10 (InitShader.comp:80-98) */
} gs_params;

typedef struct gs_sim gs_sim;

/* Launch shapes of a system's kernels.  The reference fixes its workgroup sizes
 * (src/Simulation/BarnesHut/BarnesHutSimulation.cpp:9-10,
 * src/Simulation/Direct/DirectSimulation.cpp:9); here each system gets a shape from the
 * tuned table (gs_tune_shape) or the defaults, and gs_set_shape can change it between
 * steps.  No field changes a result bit, except direct_blocks_per_sm in FAST math, which
 * sets how the direct sum splits its j-range over blocks (and so its summation grouping). */
typedef struct gs_shape {
    uint32_t sort_keys_per_thread; /* radix-sort tile = 256 threads x this: 8 or 16 (default) */
    uint32_t sort_lookback;        /* earlier tiles a radix pass reads per look-back round trip: 8, 16, 32 */
    uint32_t scan_lookback;        /* the same for the node scan: 32, 64, 128 */
    uint32_t force_warps;          /* group walks per block of the accurate traversal: 1, 2 (default), 4;
                                      1 runs as 2 where costly groups are walked by warp pairs */
    uint32_t force_short_lists;    /* 0: evaluate after 160 nodes / 96 leaf runs; 1: after 96 / 64 */
    uint32_t direct_targets;       /* direct-sum particles per thread (FAST math): 2 (default) or 4 */
    uint32_t direct_blocks_per_sm; /* direct-sum j-split target, blocks per SM: 1..32 (default 12) */
    uint32_t moment_blocks_per_sm; /* blocks per SM of the cooperative moments launch of the monopole
                                      mode: 1 or 2 (default); the quadrupole mode has no such launch */
} gs_shape;

/* Statistics: stage times accumulate over steps since gs_reset_stats (GS_FLAG_PROFILE);
 * tree counts are those of the most recent step. */
#define GS_STAGE_COUNT 8
typedef struct gs_stats {
    uint64_t steps_done;
    uint64_t tree_records;     /* Barnes-Hut preorder records (internal nodes + leaves) */
    uint64_t internal_nodes;
    uint64_t placed_particles; /* particles inside the box */
    uint64_t interactions;     /* accepted (particle, record) pairs, GS_FLAG_COUNT_INTERACTIONS */
    uint64_t warp_visits;      /* records visited summed over warps, GS_FLAG_COUNT_INTERACTIONS */
    uint64_t kernel_launches;  /* CUDA kernels this simulation launched since creation */
    float stage_ms[GS_STAGE_COUNT]; /* bbox, keys, sort, scan, records, sums, force, direct */
    uint32_t stage_launches[GS_STAGE_COUNT];
    uint64_t node_interactions; /* of `interactions`, those with internal nodes (accurate mode:
                                   quadrupoles), GS_FLAG_COUNT_INTERACTIONS with GS_FLAG_GROUP_WALK */
} gs_stats;

GS_API void gs_params_init(gs_params* p);
GS_API const char* gs_status_string(gs_status s);
/* Message of the last failure on the calling thread ("" if none). */
GS_API const char* gs_last_error(void);

GS_API uint64_t gs_required_alignment(int32_t algorithm);

GS_API gs_status gs_create(const gs_params* params, uint64_t particle_count, const float* pos_xy,
                    const float* vel_xy, const float* mass, gs_sim** out);
/* Enqueue `count` steps.  Like RunSimulations it first waits for the previous gs_run
 * batch to finish (bounded: GS_ERR_TIMEOUT after the system's timeout), then submits and
 * returns. */
GS_API gs_status gs_run(gs_sim* sim, uint32_t count);
/* Wait for all submitted steps; timeout_ns = 0 uses the system's timeout. */
GS_API gs_status gs_sync(gs_sim* sim, uint64_t timeout_ns);
/* The system's launch shapes; changing them drops its captured step graphs.  A
 * direct_blocks_per_sm that needs more j-chunk scratch than gs_create laid out is refused
 * (GS_ERR_CAPACITY). */
GS_API gs_status gs_get_shape(gs_sim* sim, gs_shape* out);
GS_API gs_status gs_set_shape(gs_sim* sim, const gs_shape* shape);
GS_API void gs_shape_defaults(gs_shape* out);
/* Bound of every host wait this system makes (gs_run, gs_sync with 0, the particle
 * transfers, readbacks): GS_ERR_TIMEOUT after timeout_ns nanoseconds; 0 (the default)
 * means 600 s.  No counterpart in the reference, whose fence waits do not time out. */
GS_API gs_status gs_set_timeout(gs_sim* sim, uint64_t timeout_ns);
/* Copy the current state (first N particles) to host arrays; any may be NULL.  Pinned
 * (page-locked or registered) arrays are written in place by a kernel queued behind the
 * submitted steps.  If the wait for it times out (GS_ERR_TIMEOUT), that kernel may still
 * write them later: keep the arrays alive and untouched until gs_sync returns GS_OK. */
GS_API gs_status gs_get_particles(gs_sim* sim, float* pos_xy, float* vel_xy, float* mass);
/* Replace the whole state (first N particles; padding reset to zero particles).  Pinned
 * arrays are read in place by a kernel queued behind the submitted steps; the call
 * returns once they have been read, except after GS_ERR_TIMEOUT, when they stay in use
 * until gs_sync returns GS_OK.  A device error raised by steps submitted before this call
 * is returned by it (GS_ERR_DEVICE) after the upload has replaced the state. */
GS_API gs_status gs_set_particles(gs_sim* sim, const float* pos_xy, const float* vel_xy,
                           const float* mass);
/* Accelerations (without G) of the last step, in particle order; needs GS_FLAG_RECORD_ACCEL. */
GS_API gs_status gs_get_accel(gs_sim* sim, float* acc_xy);
/* Accumulated per-stage times (GS_FLAG_PROFILE) and tree counts of the last step. */
GS_API gs_status gs_get_stats(gs_sim* sim, gs_stats* stats);
GS_API gs_status gs_reset_stats(gs_sim* sim);
GS_API uint64_t gs_particle_count(const gs_sim* sim);
GS_API uint64_t gs_aligned_particle_count(const gs_sim* sim);
/* CUDA stream the simulation runs on (a cudaStream_t), for event timing by callers. */
GS_API void* gs_stream(gs_sim* sim);
GS_API void gs_destroy(gs_sim* sim);

/* FP64 direct-sum accelerations (without G) of the current state on the GPU, for the
 * listed particle indices over all particles; the error reference for every result. */
GS_API gs_status gs_accel_f64(gs_sim* sim, uint32_t n_targets, const uint32_t* targets, double* acc_xy);
/* Energy of the current state in FP64 (diagnostic, O(N^2)): kinetic = sum 1/2 m |v|^2,
 * potential = -G sum_{i<j} m_i m_j / sqrt(|p_i - p_j|^2 + softening^2), the potential of
 * the softened force law.  No counterpart in the reference. */
GS_API gs_status gs_energy_f64(gs_sim* sim, double* kinetic, double* potential);

/* Barnes-Hut tree of the most recent step, in the reference's layout
 * (BarnesHutSimulation.cpp:52-142: counts, radiuses, nodePos, nodeMass, sortedSrc).
 * keys: per particle cell key (0xFFFFFFFF for removed); sorted_src: original index per
 * sorted slot (N_al for empty slots); node_quad: 3 second moments per record (zeros
 * without GS_FLAG_QUADRUPOLE).  Any pointer may be NULL. */
GS_API gs_status gs_debug_bh_tree(gs_sim* sim, uint32_t* keys, uint32_t* sorted_src,
                           uint32_t* node_skip, float* node_radius, float* node_pos,
                           float* node_mass, float* node_quad, uint64_t capacity,
                           uint64_t* tree_records);
/* The whole current state, padding included: N_al = gs_aligned_particle_count particles
 * (zero-mass padding particles move under the field like the reference's), and the |a|
 * per particle that the relative opening criterion of the next step reads (NaN where
 * unknown or without GS_FLAG_RELATIVE_MAC).  Any pointer may be NULL.  Diagnostic: it lets
 * a checker restart a CPU restatement from the device's exact state at any step. */
GS_API gs_status gs_debug_state(gs_sim* sim, float* pos_xy, float* vel_xy, float* mass, float* amag);
/* Records the tree of aligned_count particles can hold: the leaves plus, for every level
 * d of the box mode (0..10 fixed box, 0..15 bounding box: any key_bits), min(4^d,
 * aligned_count/2 + 1) internal nodes, plus 64. */
GS_API uint64_t gs_bh_node_capacity(int32_t box_mode, uint64_t aligned_count);

/* One direct-sum step (FAST math) on caller-owned device buffers, allocating nothing.
 * No counterpart in the reference: it is for callers that cannot let a library allocate
 * device memory -- a host application that owns every allocation and hands its plugins
 * fixed buffers, or a loop with a fixed memory budget that must not pay for, or be
 * synchronised by, cudaMalloc / cudaFree mid-run.
 *   - Inputs pos/vel/mass and outputs pos/vel are device arrays of n particles (x,y
 *     interleaved for pos and vel); n must be a multiple of 64 (pad with zero-mass
 *     particles at the origin, as ParticleSystem does) and at most
 *     GS_NOALLOC_MAX_PARTICLES, else GS_ERR_INVALID_ARGUMENT / GS_ERR_CAPACITY.
 *     Outputs must not alias inputs.  d_pos_in must be 16-byte aligned, the other arrays
 *     8-byte aligned (cudaMalloc gives 256), else GS_ERR_INVALID_ARGUMENT.
 *   - Runs on the calling thread's current device, on `stream` (a cudaStream_t, NULL for
 *     the legacy default stream), asynchronously.
 *   - Scratch lives in fixed device arrays inside this library (about 4 MiB per GPU that
 *     loads it, held until the process exits).  Every call looks up their device
 *     addresses in the current context (no allocation); the first call on a device also
 *     loads the library's module there, so make it before any stream capture.
 *   - Every call shares those arrays: calls that overlap on the GPU (other streams,
 *     other threads) race and give wrong results.  Serialise them on one stream. */
#define GS_NOALLOC_MAX_PARTICLES 65536
GS_API gs_status gs_direct_step_noalloc(const float* d_pos_in, const float* d_vel_in,
                                        const float* d_mass, float* d_pos_out, float* d_vel_out,
                                        uint64_t n, float gravitational_const,
                                        float simulation_time, float softening_len,
                                        void* stream);

/* ---- many systems at once (no counterpart in the reference, which runs one system) ----
 *
 * A batch advances a set of independent gs_sim systems together: every stage of the step
 * is ONE kernel launch over all member systems (Barnes-Hut: clear, bounding box, keys,
 * radix passes, scan, records, nodes, moments, force; direct sum: one launch, run beside
 * the Barnes-Hut stages), and the step is captured once per ping-pong parity as a CUDA
 * graph.  Each system keeps its own device buffers and parameters and computes the same
 * bits in a batch as with gs_run.
 *   - Members live on one device, appear once, and the Barnes-Hut members share
 *     box_mode, math_mode and the GS_FLAG_QUADRUPOLE / SAFE_RADIUS / GROUP_WALK /
 *     COUNT_INTERACTIONS flags; the direct-sum members share math_mode.
 *   - gs_batch_run is asynchronous.  It orders itself after work already submitted to
 *     each member (gs_run), and later calls on a member wait for the batch.
 *   - The batch does not own its members: destroy it before them. */
typedef struct gs_batch gs_batch;
#define GS_BATCH_NO_GRAPH 0x1u  /* launch the stage kernels one by one every step */
GS_API gs_status gs_batch_create(gs_sim* const* sims, uint32_t count, uint32_t flags,
                                 gs_batch** out);
GS_API gs_status gs_batch_run(gs_batch* batch, uint32_t steps);
/* Waits for the batch, then checks every member's device-side error flags. */
GS_API gs_status gs_batch_sync(gs_batch* batch, uint64_t timeout_ns);
/* Kernel launches per batched step (the same for any number of members). */
GS_API uint32_t gs_batch_kernels_per_step(const gs_batch* batch);
GS_API void* gs_batch_stream(gs_batch* batch);
GS_API void gs_batch_destroy(gs_batch* batch);

/* Direct-sum / Barnes-Hut crossover by measurement.  For N = min_n, 2*min_n, ... up to
 * max_n, runs a batch of max(1, particles_per_probe / N) uniform-disk systems with each
 * algorithm (direct_params, bh_params; seeded), times warm batched steps with CUDA events
 * and records the time per system-step.  crossover = the smallest measured N at which
 * Barnes-Hut was faster, from a log-log interpolation between the two sizes around it
 * (max_n when direct sum wins throughout).  Probing stops one size after Barnes-Hut wins. */
#define GS_TUNE_MAX_SIZES 16
typedef struct gs_tuning {
    uint64_t crossover;
    uint32_t sizes;
    uint64_t n[GS_TUNE_MAX_SIZES];
    double direct_ms[GS_TUNE_MAX_SIZES];  /* per system-step, batched */
    double bh_ms[GS_TUNE_MAX_SIZES];
} gs_tuning;
GS_API gs_status gs_tune_crossover(const gs_params* direct_params, const gs_params* bh_params,
                                   uint64_t min_n, uint64_t max_n, uint64_t particles_per_probe,
                                   uint64_t seed, gs_tuning* out);

/* ---- launch-shape autotuner (no counterpart in the reference) ----
 *
 * gs_tune_shape times candidate gs_shape values on a system of n particles made by
 * gs_generate(generator, seed) with these parameters, and keeps the fastest: coordinate
 * descent over the knobs that apply (Barnes-Hut: sort tile, sort and scan look-back
 * widths, group-walk warps per block and list caps, moments grid; direct sum: targets per
 * thread and the j-split), each candidate timed with CUDA events as the median of `steps`
 * warm steps with the L2 flushed before each.  The winner goes into the process's tuned
 * table under (device name and SM count, algorithm, box mode, key bits, math mode, the
 * accurate / relative / plain-sum flags, floor(log2 N)); gs_create gives a new system the
 * entry of its key, else the defaults (gs_shape_defaults).  With `cache_path` (or, when it
 * is NULL, the environment variable GSIM_SHAPE_CACHE) the table is also written there as
 * JSON, and gs_load_shape_cache reads such a file back (later processes, other callers).
 * gs_tune_batch_shape does the same for the batched kernels of an existing batch, keyed by
 * the batch's total particles; gs_batch_create consults those entries. */
typedef struct gs_tune_result {
    gs_shape best;
    double best_ms;          /* per step with the best shape */
    double default_ms;       /* per step with gs_shape_defaults */
    uint32_t candidates;     /* shapes timed */
} gs_tune_result;
GS_API gs_status gs_tune_shape(const gs_params* params, uint64_t n, int32_t generator, uint64_t seed,
                               uint32_t steps, const char* cache_path, gs_tune_result* out);
GS_API gs_status gs_tune_batch_shape(gs_batch* batch, uint32_t steps, const char* cache_path, gs_tune_result* out);
/* Reads a cache file written by the tuner into the tuned table (path NULL:
 * GSIM_SHAPE_CACHE; no such file: GS_ERR_IO).  *entries (may be NULL) gets the count. */
GS_API gs_status gs_load_shape_cache(const char* path, uint32_t* entries);
/* Empties the tuned table (new systems get the defaults again). */
GS_API void gs_clear_shape_table(void);
/* Launch shape of a batch's kernels, and changing it (re-plans; drops the step graphs). */
GS_API gs_status gs_batch_get_shape(gs_batch* batch, gs_shape* out);
GS_API gs_status gs_batch_set_shape(gs_batch* batch, const gs_shape* shape);

/* Device bytes gs_create allocates for a system with these parameters (the admission
 * measure of gs_server).  The default memory pool may round each allocation up. */
GS_API uint64_t gs_footprint(const gs_params* params, uint64_t particle_count);

/* ---- serving: continuous batching of simulation requests (no counterpart in the
 * reference) ----
 *
 * A server keeps every admitted system resident on the device and advances all of them
 * together, one batched step (gs_batch machinery) per gs_server_poll.  Requests that
 * arrive while others run are admitted between two steps as soon as their footprint
 * (gs_footprint) fits the memory budget, and leave the batch as soon as their last step
 * is enqueued; their final state is read back once that step has finished.  Systems with
 * N below `crossover` use direct_params (direct sum), the others bh_params (Barnes-Hut).
 * Generator inputs are made on worker threads.  One host thread drives a server. */
typedef struct gs_server gs_server;
#define GS_SERVE_FIFO 0           /* admit in arrival order (later requests may pass a
                                     blocked one when they fit) */
#define GS_SERVE_SHORTEST_FIRST 1 /* admit the queued request with the least N x steps first */
typedef struct gs_server_config {
    uint64_t memory_budget;       /* bytes the resident systems may hold (sum of footprints) */
    uint64_t max_resident_particles; /* sum of N of resident systems (0: no limit) */
    uint64_t crossover;           /* direct sum below this N, Barnes-Hut at or above */
    gs_params direct_params;
    gs_params bh_params;
    uint32_t steps_in_flight;     /* batched steps the host may run ahead of the GPU (0: 2) */
    uint32_t policy;              /* GS_SERVE_FIFO or GS_SERVE_SHORTEST_FIRST */
    uint32_t keep_results;        /* nonzero: keep final particles for gs_server_result */
    uint32_t worker_threads;      /* input generators (0: 4) */
} gs_server_config;

typedef struct gs_request {
    uint64_t particle_count;
    uint32_t steps;
    int32_t generator;            /* gs_generate type, used when pos_xy is NULL */
    uint64_t seed;
    float generate_size, min_mass, max_mass;
    const float* pos_xy;          /* or the caller's particles, copied at submit (vel_xy may be NULL) */
    const float* vel_xy;
    const float* mass;
} gs_request;

#define GS_REQUEST_QUEUED 0
#define GS_REQUEST_RESIDENT 1
#define GS_REQUEST_DONE 2
#define GS_REQUEST_FAILED 3
typedef struct gs_request_status {
    int32_t state;
    int32_t algorithm;
    uint32_t steps_enqueued;
    uint32_t steps;
    uint64_t particle_count;
    uint64_t footprint;
    double arrival_s, admit_s, finish_s;  /* server clock, seconds since gs_server_create */
} gs_request_status;

typedef struct gs_server_stats {
    uint64_t submitted, finished, failed, queued, resident;
    uint64_t memory_in_use, peak_memory_in_use;
    uint64_t resident_particles, peak_resident_particles;
    uint64_t batched_steps;       /* gs_server_poll steps enqueued */
    uint64_t plan_changes;        /* member-set changes */
    uint64_t particle_steps;      /* sum of N x steps of finished requests */
    double gpu_busy_seconds;      /* device time of the finished batched steps (CUDA events) */
} gs_server_stats;

GS_API gs_status gs_server_create(const gs_server_config* config, gs_server** out);
/* Queues a request; its latency is counted from `arrival_s` on the server clock (pass a
 * negative value for "now"). */
GS_API gs_status gs_server_submit(gs_server* server, const gs_request* request, double arrival_s,
                                  uint64_t* id);
/* One scheduling turn: retire finished requests, admit queued ones that fit, enqueue one
 * batched step.  *finished (may be NULL) gets the number of requests retired. */
GS_API gs_status gs_server_poll(gs_server* server, uint32_t* finished);
GS_API gs_status gs_server_request(gs_server* server, uint64_t id, gs_request_status* out);
/* Final particles of a finished request (keep_results); the first N particles. */
GS_API gs_status gs_server_result(gs_server* server, uint64_t id, float* pos_xy, float* vel_xy,
                                  float* mass);
GS_API gs_status gs_server_get_stats(gs_server* server, gs_server_stats* out);
GS_API double gs_server_clock(gs_server* server);
/* Replays a trace in real time: request i is submitted when the server clock reaches
 * start + arrival_s[i] (start = the clock at the call), and the server is polled until
 * every request of the trace has finished or failed, or timeout_s passed
 * (GS_ERR_TIMEOUT).  ids (may be NULL) receives the request ids. */
GS_API gs_status gs_server_run_trace(gs_server* server, const gs_request* requests,
                                     const double* arrival_s, uint32_t count, double timeout_s,
                                     uint64_t* ids);
GS_API void gs_server_destroy(gs_server* server);

/* ---- headless point splat and snapshot ring ----
 *
 * The reference draws each particle as a one-pixel white point on black through Vulkan
 * (src/Graphics/Shaders/VertShader.vert:13-18, FragShader.frag, GraphicsPipeline.cpp:287-391).
 * Here a CUDA kernel writes the same picture into a device framebuffer: camera =
 * {x, y, width, height} in world units, screen = (pos - camera.xy) / camera.wh with y
 * flipped, pixel = floor((screen + 1) * size / 2); image = width x height bytes, row 0
 * at the top, 255 where a particle lands and 0 elsewhere.  No graphics API is used. */
/* The reference's start camera (ParticleSystem::GetCameraInfo, src/Particles/ParticleSystem.cpp:408-435):
 * centre of the particles' extent and its larger side, as {x, y, size, size}; the
 * reference's window then uses {x, y, size * aspect / zoom, size / zoom}. */
GS_API gs_status gs_camera_start(gs_sim* sim, float* camera4);
/* Render the current state (waits for submitted steps). */
GS_API gs_status gs_render_points(gs_sim* sim, uint32_t width, uint32_t height, const float* camera4,
                                  uint8_t* image);
/* Snapshot ring, the counterpart of the reference's third particle buffer set that the
 * graphics path reads while compute uses the other two (src/Particles/ParticleSystem.hpp:146-174).
 * gs_snapshot_take copies the current positions into slot (ticket mod slots) in stream
 * order -- after every step submitted so far, before any submitted later -- without
 * waiting.  Reading or rendering a ticket waits only for that copy and runs beside the
 * simulation's stream.  A ticket is valid until `slots` later snapshots reuse its slot
 * (then GS_ERR_CAPACITY).  The slot count is fixed by the first call on a system. */
GS_API gs_status gs_snapshot_take(gs_sim* sim, uint32_t slots, uint64_t* ticket);
GS_API gs_status gs_snapshot_positions(gs_sim* sim, uint64_t ticket, float* pos_xy);
GS_API gs_status gs_snapshot_render(gs_sim* sim, uint64_t ticket, uint32_t width, uint32_t height,
                                    const float* camera4, uint8_t* image);
/* Binary PPM (P6) of an image from the calls above, white points on black. */
GS_API gs_status gs_write_ppm(const char* path, uint32_t width, uint32_t height, const uint8_t* image);

/* ---- host-only helpers (no GPU) ---- */

/* Generator types: the reference's four presets (ParticleSystem::GenerateType) and the
 * seeded workloads the measurements are quoted on. */
typedef enum gs_generate_type {
    GS_GEN_RANDOM = 0,
    GS_GEN_GALAXY = 1,
    GS_GEN_GALAXY_COLLISION = 2,
    GS_GEN_SYMMETRICAL_GALAXY_COLLISION = 3,
    GS_GEN_UNIFORM_DISK = 16,       /* r = R*sqrt(u), v = 0 */
    GS_GEN_SPIRAL = 17,             /* exponential disk, two-arm log spiral, circular v */
    GS_GEN_EXP_DISK_COLLISION = 18  /* two exponential disks at (+-50, 0), v = (0, +-3) */
} gs_generate_type;

GS_API gs_status gs_generate(int32_t type, uint64_t count, float generate_size, float min_mass,
                      float max_mass, float gravitational_const, uint64_t seed, float* pos_xy,
                      float* vel_xy, float* mass);
/* Reads "x y vx vy m" records (fscanf %f, stops at the first incomplete record).
 * Call with NULL arrays to get the count; then again with arrays of that size. */
GS_API gs_status gs_read_particles(const char* path, uint64_t capacity, uint64_t* count,
                            float* pos_xy, float* vel_xy, float* mass);
/* Writes "%.7f %.7f %.7f %.7f %.7f\n" per particle, byte-identical to SaveParticles. */
GS_API gs_status gs_write_particles(const char* path, uint64_t count, const float* pos_xy,
                             const float* vel_xy, const float* mass);

#ifdef __cplusplus
}
#endif
#endif
