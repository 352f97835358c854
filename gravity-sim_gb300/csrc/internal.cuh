// internal.cuh -- shared definitions of the GB300 Gravity-Sim library.
//
// Device data layout (one gs_sim, N_al = N rounded up to 64):
//   state      2 sets x { pos float2[N_al], vel float2[N_al], mass float[N_al] }  (ping-pong,
//              the reference's compute-input / compute-output buffer pair)
//   Barnes-Hut scratch (N_al-sized, never a fixed 1024^2 grid):
//              keys/idx u32[N_al] x 2 (radix-sort ping-pong), E u32[N_al+1] (exclusive
//              scan of internal nodes per sorted slot), rec float4[cap] = {x, y, m, radius}
//              and skip u32[cap] (preorder records, cap = N_al + 64 + sum over levels of min(4^d, N_al/2 + 1)),
//              nend u32[cap] and msum float2[cap] (cell end slot and mass moments)
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/gsim.h"

namespace gsim {

constexpr int kWarp = 32;
constexpr uint32_t kAlignment = 64;         // GetRequiredParticleAlignment()
constexpr float kSimSize = 500.0f;          // BarnesHutSimulation.cpp:580
constexpr uint32_t kGrid = 1024;            // BarnesHutSimulation.cpp:582
constexpr int kFixedDepth = 10;             // finest level of the fixed box
constexpr int kBBoxBits = 12;               // default per-axis bits in bounding-box mode (24-bit keys)
constexpr int kBBoxMaxBits = 15;            // largest per-axis bits (30-bit keys, 4 radix passes)
constexpr uint32_t kKeyRemovedSort = 1u << 20;  // sort key of removed particles (fixed box)
// Relative criterion: costly groups are walked by warp pairs in systems of at least this
// many (padded) particles -- more groups than the traversal keeps resident at once, where
// the longest walks trail the launch; smaller systems walk every group on one warp.
constexpr uint32_t kHeavyMinParticles = 1u << 18;
constexpr uint32_t kKeyRemoved = 0xFFFFFFFFu;   // reported key of removed particles

// pinned host words of a system (gs_sim::h_err): the device error word at 0, counter
// readbacks from kHostCounters on
constexpr int kHostWords = 64;
constexpr int kHostCounters = 16;

// stage indices of gs_stats.stage_ms
enum Stage { kStageBBox = 0, kStageKeys, kStageSort, kStageScan, kStageRecords, kStageSums, kStageForce, kStageDirect };

// device error bits (sim->d_err)
constexpr int kErrSortWait = 1;
constexpr int kErrScanWait = 2;
constexpr int kErrTree = 4;
constexpr int kErrBarrierWait = 8;

// radix sort: 256 threads x 8 or 16 keys per tile (gs_shape.sort_keys_per_thread)
constexpr int kSortThreads = 256;
// single-pass scan shape
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;
// moments: levels at or above kLevelTop (<= 341 nodes) are summed by one block, every
// deeper level by a launch of its own
constexpr int kLevelTop = 4;
// bounded spin for decoupled look-back: after this many polls the kernel flags an error
constexpr uint32_t kSpinLimit = 1u << 24;

// Order-preserving code of a float: unsigned comparison of the words orders the values
// (-inf < ... < -0 < +0 < ... < +inf), so atomicMin on words takes a minimum and atomicMin
// on complemented words a maximum.  All-ones words (the cleared state) decode to NaN and
// lose to every value.  NaN inputs are left out by the callers, as fminf/fmaxf do.
__host__ __device__ __forceinline__ uint32_t ord_word(uint32_t bits) {
    return (bits & 0x80000000u) ? ~bits : (bits | 0x80000000u);
}
__host__ __device__ __forceinline__ uint32_t ord_bits(uint32_t w) {
    return (w & 0x80000000u) ? (w & 0x7FFFFFFFu) : ~w;
}

// Packed two-lane FP32 (Blackwell f32x2): each lane of the pair rounds exactly like the
// scalar instruction, so a packed evaluation gives the same bits as two scalar ones.
__device__ __forceinline__ float2 add2(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "add.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "sub.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "mul.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "mov.b64 rc, {%6, %7};\n\tfma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}

struct BHParams {
    float cx, cy, scale, radius0;  // bounding box (fixed box: 0, 0, 1.024, 500000)
    float inv_scale;               // float(1 / scale), taken once in FP64
    int bits;                      // cells per axis 2^bits (bounding box; 10 for the fixed box)
};

struct MomSums;  // moments.cuh

struct BHWork {
    int depth = 0;        // finest level D (10 fixed box, key_bits in bounding-box mode)
    int passes = 0;       // radix passes of 8 bits
    uint64_t cap = 0;     // record capacity
    uint32_t* keys[2] = {nullptr, nullptr};
    uint32_t* idx[2] = {nullptr, nullptr};
    uint32_t* hist = nullptr;          // [4][256] digit counts
    uint32_t* sort_status = nullptr;   // [passes][tiles][256]
    uint32_t* counters = nullptr;      // [0..3] sort tile tickets, [4] scan ticket, [5] bbox ticket,
                                       // [6] valid count, [7] internal count, [8..13] interaction,
                                       // test and node counts (3 x u64), [16..31] nodes per level
    uint32_t* scan_status = nullptr;   // [scan tiles]
    uint32_t* E = nullptr;             // [N_al + 1]
    float4* rec = nullptr;             // [cap + 32]
    uint32_t* skip = nullptr;          // [cap + 32]
    float2* msum = nullptr;            // [cap]
    float4* quad = nullptr;            // [cap] {sxx, sxy, syy, -} (GS_FLAG_QUADRUPOLE)
    float* amag = nullptr;             // [n_al] |a| of the last step, NaN: unknown (GS_FLAG_RELATIVE_MAC)
    uint8_t* heavy_flag = nullptr;     // [n_al / 64] costly group (walked by a warp pair), relative criterion
    uint2* heavy_list = nullptr;       // [n_al / 64] {0, group} of the costly groups of the step
    uint32_t* ext = nullptr;           // [2][4] extent of each state set's positions (bounding-box mode):
                                       // {min x, ~max x, min y, ~max y} as ordered words (ord_word)
    int sums_per_sm = 0, sms = 0;      // co-resident blocks per SM of the cooperative moments launch, SMs
    uint4* kids = nullptr;             // [cap] child descriptors of internal records
    // quadrupole mode: exact moment sums (moments.cuh)
    int4* mom_q = nullptr;             // [N_al] integer mass and position per sorted slot
    __int128* mom_prefix = nullptr;    // [6][N_al + 1] exclusive prefix of the six sums per slot
    MomSums* mom_agg = nullptr;        // [mom_blocks] sums of each tile of the moment scan
    uint32_t* mom_nend = nullptr;      // [cap] one past the last slot of each internal node
    uint32_t mom_blocks = 0;           // tiles of the moment scan
    uint32_t* levels = nullptr;        // internal records by level (level_off / level_cap in bh.cu)
    uint2* nodeinfo = nullptr;         // [cap] {a key of the cell, level} of an internal record
    uint32_t* node_slot = nullptr;     // [cap] start slot of internal node j (ordinal)
    float* bbox_part = nullptr;        // [blocks][4]
    BHParams* params = nullptr;        // device
    uint32_t sort_tiles = 0, scan_tiles = 0;
    int final_keys = 0;                // which keys/idx buffer holds the sorted result
    size_t zero_bytes = 0;             // bytes of the contiguous block cleared each step
    void* zero_base = nullptr;
};

struct DirectWork {
    int ipt = 2;           // particles per thread of the creation shape
    int block = 128;       // threads per block
    float4* partials = nullptr;  // [direct_max_chunks][N_al] {sx, sy, cx, cy}
    uint32_t* tickets = nullptr; // [i-tiles]
};

// One system of a batch as the batched stage kernels see it: its buffers (both ping-pong
// sets; the compute-input set of batch step t is (parity + t) & 1) and its scalars.
struct SysDesc {
    float2* pos[2];
    float2* vel[2];
    float* mass[2];
    float2* acc;
    int* err;
    uint32_t n_al;
    uint32_t parity;
    float eps2, theta2, k, hdt;
    // Barnes-Hut scratch (BHWork)
    uint32_t* keys[2];
    uint32_t* idx[2];
    uint32_t* hist;
    uint32_t* sort_status;
    uint32_t* counters;
    uint32_t* scan_status;
    uint32_t* E;
    float4* rec;
    uint32_t* skip;
    float2* msum;
    float4* quad;
    float* amag;      // relative criterion: |a| per particle, or null for the theta test
    uint8_t* heavy;   // relative criterion: costly-group flag per group of 64 slots
    uint32_t* ext;    // extents of the two state sets (bounding-box mode), or null
    float alpha, floor2;
    uint4* kids;
    int4* mom_q;
    __int128* mom_prefix;
    MomSums* mom_agg;
    uint32_t* mom_nend;
    uint32_t* levels;
    uint2* nodeinfo;
    uint32_t* node_slot;
    float* bbox_part;
    BHParams* params;
    uint32_t* zero_base;
    uint32_t zero_words;
    uint32_t cap;
    uint32_t sort_tiles, scan_tiles;
    int depth, passes, bbox, safe;
    // direct sum (DirectWork)
    float4* partials;
    uint32_t* tickets;
    uint32_t itiles, chunks, jchunk;
};

// Per-stage block tables of a batch: table t holds the exclusive prefix of the blocks each
// system gets in stage t; a block finds its system by binary search.
enum BatchTable {
    kTabClear = 0, kTabBBox, kTabKeys, kTabGrid, kTabSort, kTabScan, kTabOne, kTabForce, kTabDirect, kTabMom, kTabCount
};

// What the batched launchers need: descriptors (Barnes-Hut systems first, largest first),
// block tables, and the batch-wide work counters cleared by the first stage.
struct BatchPlan {
    uint32_t n_bh = 0, n_direct = 0;
    SysDesc* d_descs = nullptr;
    uint32_t* d_tab[kTabCount] = {};
    uint32_t total[kTabCount] = {};
    uint32_t* d_work = nullptr;  // [0] next force block, [1] next estimate-pass block,
                                 // [2] entries of d_heavy, [3] next entry for a warp pair
    uint2* d_heavy = nullptr;    // {member, group} of the costly groups of a step (relative criterion)
    int passes = 0;
    int depth = 0;               // finest level of the Barnes-Hut members (all share the box mode)
    bool bbox = false, quad = false, group = false, exact = false, count = false, direct_exact = false;
    bool direct_plain = false;   // direct-sum members add their partials plainly (GS_FLAG_PLAIN_SUM)
    gs_shape shape{};            // launch shapes of the batched kernels (the batch's, see gs_batch_create)
    int force_grid = 0;          // persistent force grid (resident blocks)
};

}  // namespace gsim

struct gs_sim {
    gs_params p{};
    uint64_t n = 0, n_al = 0;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;     // second stream of a step's fork (quadrupole moment prefix)
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    float2* pos[2] = {nullptr, nullptr};
    float2* vel[2] = {nullptr, nullptr};
    float* mass[2] = {nullptr, nullptr};
    int in = 0;  // compute-input set
    float dt_eff = 0, G = 0, eps2 = 0, theta2 = 0;
    float floor2 = 0;       // squared theta floor of the relative criterion
    float2* acc = nullptr;  // GS_FLAG_RECORD_ACCEL
    int* d_err = nullptr;
    int* h_err = nullptr;   // pinned host words: [0] copy of d_err (check_device_error),
                            // [kHostCounters ..) counter readbacks (gsim::kHostWords in all)
    gsim::BHWork bh;
    gsim::DirectWork dw;
    cudaEvent_t batch_done = nullptr;
    bool batch_pending = false;
    cudaEvent_t ev[2 * GS_STAGE_COUNT] = {};
    gs_stats stats{};
    // CUDA graphs: one per ping-pong parity [in], and [2 + in] with the |a| estimate pass
    cudaGraphExec_t graph[4] = {nullptr, nullptr, nullptr, nullptr};
    uint64_t steps_done = 0;
    bool capturing = false;          // stage events become external event-record graph nodes
    uint32_t stage_ran = 0;          // stages recorded in the current step (GS_FLAG_PROFILE)
    bool profile_pending = false;    // stage events of the last step not yet accumulated
    uint32_t graph_stages[4] = {0, 0, 0, 0};  // stages recorded by each captured graph
    uint32_t launches_in_step = 0;   // kernels enqueued by the step being built
    uint32_t launches_per_step[4] = {0, 0, 0, 0};  // per graph (replay count)
    bool amag_known = false;         // relative criterion: every particle has its previous |a|
    gs_shape shape{};                // launch shapes (gs_set_shape; graphs are captured with them)
    uint32_t direct_max_chunks = 1;  // j-chunks the direct-sum scratch was laid out for
    uint64_t kernel_launches = 0;    // kernels launched since creation
    void* slab = nullptr;            // every device buffer of the system
    size_t carved = 0;               // bytes laid out so far (sim_carve)
    cudaEvent_t follow = nullptr;    // a batch step this system's next work must follow
    bool own_work = false;           // work submitted on its own stream since the last batch run
    uint64_t timeout_ns = 0;         // bound of every host wait on this system (0: 600 s)
};

namespace gsim {

// error reporting: thread-local message
void set_error(const std::string& msg);
gs_status cuda_fail(cudaError_t e, const char* what);

#define GS_CUDA(call)                                          \
    do {                                                       \
        cudaError_t _e = (call);                               \
        if (_e != cudaSuccess) return gsim::cuda_fail(_e, #call); \
    } while (0)

// Launch shapes: checks a shape's values (message on failure); the shape a new system of
// these parameters gets (the tuned table of tune.cu, else the defaults).
bool shape_valid(const gs_shape& sh, std::string* why);
void shape_for(const gs_params* p, uint64_t n, gs_shape* out);
void batch_shape_for(const gs_params* p, uint64_t total, gs_shape* out);
// The parameters and total particles a batch's tuned-table entry is keyed by.
gs_status batch_key(gs_batch* b, gs_params* params, uint64_t* total);

// Bounded host waits (GS_ERR_TIMEOUT after timeout_ns; 0: 600 s): an event, a stream
// (through a private event), or everything enqueued on a system's stream so far (its
// timeout, gs_set_timeout).
gs_status wait_event(cudaEvent_t ev, uint64_t timeout_ns);
gs_status wait_stream(cudaStream_t st, uint64_t timeout_ns);
gs_status sim_wait(gs_sim* s);

// Device memory of a system: one slab from the device's default pool (stream-ordered on
// the system's stream, kept cached), carved into 256-byte aligned buffers.  Carving with
// no slab yet only counts bytes, which sizes the slab and gives gs_footprint.
void sim_carve(gs_sim* s, void** p, size_t bytes);
cudaError_t keep_pool_memory(int device);

// layout, initial contents and step launchers (return cudaError_t of the launch)
void bh_carve(gs_sim* s);
cudaError_t bh_init(gs_sim* s);
cudaError_t bh_step(gs_sim* s, int in, int out, bool profile, bool estimate);
void direct_carve(gs_sim* s);
cudaError_t direct_init(gs_sim* s);
cudaError_t direct_step(gs_sim* s, int in, int out, bool profile);
cudaError_t accel_f64(gs_sim* s, uint32_t n_targets, const uint32_t* d_targets, double2* d_out);
gs_status energy_f64(gs_sim* s, double* kinetic, double* potential);
void free_snapshot_ring(const gs_sim* s);
uint64_t bh_capacity(int depth, uint64_t n_al);
int bh_key_bits(const gs_params* p);

// One launch of a system's traversal kernel (force_fast.cu / force_exact.cu).  The group
// walk takes its warps per block and list caps from `shape`; the interaction-counting
// variants exist for the default shape only (2 warps, long lists) and use it.
struct ForceLaunch {
    cudaStream_t st = nullptr;
    bool pdl = false;
    bool group = false, quad = false, count = false, estimate = false;
    gs_shape shape{};
    const uint32_t* sidx = nullptr;
    const uint32_t* skey = nullptr;
    const uint32_t* counts = nullptr;
    const float4* rec = nullptr;
    const uint32_t* skip = nullptr;
    const float4* quad_m = nullptr;
    const uint4* kids = nullptr;
    const float2* pos_in = nullptr;
    const float2* vel_in = nullptr;
    float2* pos_out = nullptr;
    float2* vel_out = nullptr;
    float2* acc = nullptr;
    uint32_t n_al = 0, cap = 0;
    float eps2 = 0, theta2 = 0, k = 0, hdt = 0, alpha = 0, floor2 = 0;
    unsigned long long* stat = nullptr;
    int* err = nullptr;
    float* amag = nullptr;
    uint32_t* ext = nullptr;
    // costly groups walked by warp pairs (relative criterion, main pass): flag per group,
    // the step's list, and [0] its length, [1] the next entry to take
    const uint8_t* heavy = nullptr;
    const uint2* heavy_list = nullptr;
    uint32_t* heavy_work = nullptr;
};
cudaError_t force_launch_fast(const ForceLaunch& f);
cudaError_t force_launch_exact(const ForceLaunch& f);

// One launch of the batched (persistent) traversal kernel over the Barnes-Hut systems of
// a plan; `grid` 0 asks only for the resident-block count (returned in *grid_out).
struct BatchForceLaunch {
    cudaStream_t st = nullptr;
    const SysDesc* descs = nullptr;
    const uint32_t* first = nullptr;
    uint32_t nsys = 0, step = 0;
    uint32_t* work = nullptr;
    int grid = 0;
    bool group = false, quad = false, count = false, estimate = false;
    gs_shape shape{};
    const uint2* heavy_list = nullptr;  // the batch's costly groups, or null
    uint32_t* heavy_work = nullptr;     // [0] entries, [1] next entry
};
cudaError_t batch_force_launch_fast(const BatchForceLaunch& b, int* grid_out);
cudaError_t batch_force_launch_exact(const BatchForceLaunch& b, int* grid_out);
// Group-walk (warps, short lists) combinations that exist as kernels.
bool force_shape_supported(uint32_t warps, uint32_t short_lists);

// batched stages (one launch per stage over every system of a plan)
// force_warps: group walks per block of the batch's traversal launch (its block table)
void bh_batch_desc(gs_sim* s, SysDesc& d, uint32_t blocks[kTabCount], const gs_shape& shape, uint32_t force_warps);
void direct_batch_desc(gs_sim* s, SysDesc& d, uint32_t blocks[kTabCount], const gs_shape& batch_shape);
// j-chunks the direct sum of `s` splits into under a shape (its scratch holds direct_max_chunks)
uint32_t direct_chunks_needed(const gs_sim* s, const gs_shape& sh);
int bh_batch_force_grid(const BatchPlan& p);
// A second stream and two events: the moment prefix of the quadrupole mode runs there,
// beside the node layout (no fork when `side` is null).
struct StepFork {
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};
cudaError_t bh_batch_step(const BatchPlan& p, uint32_t step, cudaStream_t st, bool estimate, const StepFork& f);
cudaError_t direct_batch_step(const BatchPlan& p, uint32_t step, cudaStream_t st);
void bh_set_final_keys(gs_sim* s);

// profiling helpers
void stage_begin(gs_sim* s, int stage, bool profile);
void stage_end(gs_sim* s, int stage, bool profile);
inline void count_launch(gs_sim* s, uint32_t k = 1) { s->launches_in_step += k; }

}  // namespace gsim
