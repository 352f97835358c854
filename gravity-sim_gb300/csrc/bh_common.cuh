// bh_common.cuh -- device helpers and launch wrappers shared by the Barnes-Hut tree
// kernels (bh.cu) and the traversal kernels (force_kernels.cuh, one translation unit per
// math mode so that they compile in parallel).
#pragma once
#include "internal.cuh"

namespace gsim {

// counters layout inside the zeroed block
// [kCtrStat..+5]: accepted interactions, records tested, node interactions (u64 each);
// [kCtrLevel..+15]: internal nodes per level; [kCtrMaxMass]: float bits of the largest
// mass (quadrupole mode); [kCtrHeavy]: entries of the costly-group list, [+1] the next one
enum {
    kCtrSort = 0, kCtrScan = 4, kCtrBBox = 5, kCtrValid = 6, kCtrInternal = 7, kCtrStat = 8, kCtrLevel = 16,
    kCtrBarrier = 32, kCtrMaxMass = 33, kCtrHeavy = 34, kCtrCount = 40
};
static_assert(kHostCounters + kCtrCount <= kHostWords, "counter readback fits the pinned word block");

namespace {

constexpr int kForceWarps = 4;  // warps per block of the reference's warp-vote walk
constexpr int kGroupSize = 64;  // particles per group walk (two per lane)

// Every stage is written as a __device__ body that takes its block's index and the
// number of blocks working on its system.  A plain launch passes blockIdx.x / gridDim.x;
// a batched launch (one grid over many systems) passes the block's index within its
// system.  No body's result depends on how many blocks it gets, so a system computes the
// same bits alone and in a batch.
struct Blk {
    uint32_t id, count;
};
__device__ __forceinline__ Blk grid_blk() { return Blk{blockIdx.x, gridDim.x}; }

// Programmatic dependent launch: every step kernel lets the next launch in its stream
// start as soon as all of its blocks have begun, then waits until the kernel before it
// has finished and its writes are visible.  Each kernel therefore still runs strictly
// after its predecessor (and transitively after all earlier ones); only the launch
// latency between them is hidden.  Without the launch attribute both are no-ops.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t* p) {
    return *((volatile const uint32_t*)p);
}

// Acquire load of a barrier counter.
__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// The extent {min x, max x, min y, max y} of a state set from its ordered words.
__device__ __forceinline__ float4 ext_decode(const uint32_t* __restrict__ ext) {
    return make_float4(__uint_as_float(ord_bits(__ldcg(ext + 0))), __uint_as_float(ord_bits(~__ldcg(ext + 1))),
                       __uint_as_float(ord_bits(__ldcg(ext + 2))), __uint_as_float(ord_bits(~__ldcg(ext + 3))));
}

// Adds min/max of positions to a state set's extent words: a warp reduction (fminf/fmaxf
// skip NaN), then one atomic per word from lane 0.  Every lane of the warp must call it.
__device__ __forceinline__ void ext_add(uint32_t* __restrict__ ext, float mnx, float mxx, float mny, float mxy) {
    for (int o = 16; o; o >>= 1) {
        mnx = fminf(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
        mxx = fmaxf(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
        mny = fminf(mny, __shfl_xor_sync(0xffffffffu, mny, o));
        mxy = fmaxf(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(ext + 0, ord_word(__float_as_uint(mnx)));
        atomicMin(ext + 1, ~ord_word(__float_as_uint(mxx)));
        atomicMin(ext + 2, ord_word(__float_as_uint(mny)));
        atomicMin(ext + 3, ~ord_word(__float_as_uint(mxy)));
    }
}

// Child descriptors of an internal record: up to four children in Morton order, each a
// record index with kKidLeaf set for a particle leaf, kKidNone when absent; a
// finest-level cell stores {kKidFinest, first leaf, leaf count, -}.
constexpr uint32_t kKidNone = 0xFFFFFFFFu;
constexpr uint32_t kKidFinest = 0xFFFFFFFEu;
constexpr uint32_t kKidLeaf = 0x80000000u;

// system s with first[s] <= b < first[s + 1] (systems with no blocks are skipped)
__device__ __forceinline__ uint32_t batch_sys(const uint32_t* __restrict__ first, uint32_t nsys, uint32_t b) {
    uint32_t lo = 0, hi = nsys;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&first[mid]) <= b) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Costly groups of the relative criterion's main pass (their walks run on warp pairs,
// force_kernels.cuh): every previous |a| of the group known and the smallest below
// kHeavyRatio times the largest.
constexpr float kHeavyRatio = 0.1f;

// One warp per group: the group's flag for the main traversal and, for a costly group, an
// entry {tag, group} of the list the warp pairs take (relative criterion, main pass).
__device__ __forceinline__ void heavy_list_body(Blk blk, const uint32_t* __restrict__ sidx,
                                                const uint32_t* __restrict__ counts, const float* __restrict__ amag,
                                                uint32_t n_al, uint8_t* __restrict__ flag, uint2* __restrict__ list,
                                                uint32_t* __restrict__ list_count, uint32_t tag) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t nv = counts[0];
    const uint32_t G = (nv + kGroupSize - 1) / kGroupSize;
    const uint32_t wpb = blockDim.x >> 5;
    for (uint32_t grp = blk.id * wpb + warp; grp < G; grp += blk.count * wpb) {
        const uint32_t s0 = grp * kGroupSize + lane, s1 = s0 + 32;
        const uint32_t i0 = s0 < nv ? sidx[s0] : 0u, i1 = s1 < nv ? sidx[s1] : 0u;
        const bool v0 = s0 < nv && i0 < n_al, v1 = s1 < nv && i1 < n_al;
        const float a0 = v0 ? amag[i0] : INFINITY, a1 = v1 ? amag[i1] : INFINITY;
        const bool unknown = __any_sync(0xffffffffu, isnan(a0) || isnan(a1));
        float amin = fminf(a0, a1), amax = fmaxf(v0 ? a0 : 0.0f, v1 ? a1 : 0.0f);
        for (int o = 16; o; o >>= 1) {
            amin = fminf(amin, __shfl_xor_sync(0xffffffffu, amin, o));
            amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
        }
        const bool heavy = !unknown && amin < kHeavyRatio * amax;
        if (lane == 0) {
            flag[grp] = heavy ? 1u : 0u;
            if (heavy) list[atomicAdd(list_count, 1u)] = make_uint2(tag, grp);
        }
    }
}

struct BatchArgs {
    const SysDesc* descs;
    const uint32_t* first;
    uint32_t nsys;
    uint32_t step;
};

struct BatchBlock {
    const SysDesc* d;
    Blk blk;
    int in, out;
};

__device__ __forceinline__ BatchBlock batch_block(const BatchArgs& a, uint32_t b) {
    const uint32_t s = batch_sys(a.first, a.nsys, b);
    const uint32_t f0 = __ldg(&a.first[s]), f1 = __ldg(&a.first[s + 1]);
    BatchBlock r;
    r.d = a.descs + s;
    r.blk = Blk{b - f0, f1 - f0};
    r.in = (int)((r.d->parity + a.step) & 1u);
    r.out = r.in ^ 1;
    return r;
}

inline int grid_for(uint64_t n, int threads) {
    uint64_t b = (n + threads - 1) / threads;
    if (b > 152ull * 16) b = 152ull * 16;
    if (b < 1) b = 1;
    return (int)b;
}

// Launch `kernel` on `st`.  With `pdl` the launch may begin while the previous kernel in
// the stream is still running; the kernel waits for it on entry (pdl_enter).
template <typename... KArgs, typename... Args>
cudaError_t launch(bool pdl, void (*kernel)(KArgs...), int grid, int block, cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// The same as a cooperative launch: every block of the grid is resident at once.
template <typename... KArgs, typename... Args>
cudaError_t launch_coop(bool pdl, void (*kernel)(KArgs...), int grid, int block, cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 2 : 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}
#define GS_TRY_LAUNCH(call)                    \
    do {                                       \
        cudaError_t _e = (call);               \
        if (_e != cudaSuccess) return _e;      \
    } while (0)

}  // namespace
}  // namespace gsim
