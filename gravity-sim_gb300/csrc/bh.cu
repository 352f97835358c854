// bh.cu -- Barnes-Hut step: cell keys, onesweep radix sort, quadtree build from sorted
// keys, mass/centre-of-mass reduction and the warp-coherent traversal with the
// integrator fused into its epilogue.
//
// Replaces the seven shaders of src/Simulation/BarnesHut/Shaders/ and the 35 dispatches
// per step of src/Simulation/BarnesHut/BarnesHutSimulation.cpp:885-918.  The reference
// clears and fills a fixed 1024x1024 grid and walks 11 levels of it every step; here
// every stage is sized by N:
//
//   k_ext_keys    (bounding-box mode) box parameters in FP64 from the extent of the input
//                 positions, which the traversal kernel that wrote them (or the upload)
//                 gathered with atomics, then the keys (a batch runs kb_bbox and kb_keygen)
//   k_keygen      cell key per particle (InitShader.comp:80-98 arithmetic), removal of
//                 particles outside the fixed box (InitShader.comp:110-117), digit
//                 histograms for every radix pass
//   k_sort_pass   onesweep LSD pass: 8-bit digits, decoupled look-back, stable
//   k_meta_scan   per sorted slot s the internal nodes that start at s: levels
//                 dmin(s)..dmax(s) from the common prefix with the neighbouring keys,
//                 exclusive scan E(s) with decoupled look-back
//   k_records     preorder records: node (d, s) at s + E(s) + d - dmin(s), particle leaf
//                 at s + E(s) + e(s); skip = end + E(end) - index (the reference's count.y),
//                 radius = radius0 / 4^d (TreeMoveShader.comp:70-71)
//   monopole mode (the reference's rule):
//   k_coop_sums   mass and mass-moment sums level by level, finest first (one cooperative
//                 launch, a grid barrier between deep levels, one block for the top
//                 levels; a batch launches kb_level_sums per level), children in the order
//                 of TreeInitShader.comp:78-80; centre of mass as TreeMoveShader.comp:66-67
//   quadrupole mode (accurate mode, moments.cuh): exact integer sums instead --
//   k_mom_tiles   the sums of every tile of 1024 sorted slots
//   k_mom_scan    their exclusive prefix at every slot
//   k_mom_nodes   each internal node's centre, mass, opening radius and second moments
//                 from the prefix at its first slot and one past its last (k_nodes keeps
//                 the end)
//   k_force       ForceShader.comp:78-152 semantics: one warp walks the preorder records
//                 for 32 consecutive sorted slots; a record is accepted only if every
//                 lane satisfies radius <= d2 * theta^2; 32-record window staged in shared
//                 memory; the integrator and the scatter to original order are fused.
#include <algorithm>
#include <cstdio>
#include <cstring>

#include "bh_common.cuh"
#include "moments.cuh"

namespace gsim {
namespace {

// ------------------------------------------------------------------------------------
// keys
// ------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t spread_bits(uint32_t v) {  // InitShader.comp:88-96
    v = (v | (v << 8)) & 0x00ff00ffu;
    v = (v | (v << 4)) & 0x0f0f0f0fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

// InitShader.comp:80-85: rel = ((p / S) + 1) * 0.5 * 1024, inside iff 0 <= rel < 1024
__device__ __forceinline__ bool fixed_key(float px, float py, uint32_t& key) {
    float rx = __fmul_rn(__fmul_rn(__fadd_rn(__fdiv_rn(px, kSimSize), 1.0f), 0.5f), (float)kGrid);
    float ry = __fmul_rn(__fmul_rn(__fadd_rn(__fdiv_rn(py, kSimSize), 1.0f), 0.5f), (float)kGrid);
    if (rx >= 0.0f && rx < (float)kGrid && ry >= 0.0f && ry < (float)kGrid) {
        key = spread_bits((uint32_t)rx) | (spread_bits((uint32_t)ry) << 1);
        return true;
    }
    return false;
}

// cell index along one axis, 2^bits cells (bits <= 15: exact in FP32)
__device__ __forceinline__ uint32_t bbox_cell(float p, float c, float scale, int bits) {
    float t = __fadd_rn(__fmul_rn(__fsub_rn(p, c), scale), (float)(1u << (bits - 1)));
    if (!(t >= 0.0f)) return 0u;
    if (t >= (float)((1u << bits) - 1)) return (1u << bits) - 1;
    return (uint32_t)t;
}

__device__ __forceinline__ int common_bits(uint32_t a, uint32_t b, int key_bits) {
    return a == b ? key_bits : __clz(a ^ b) - (32 - key_bits);
}
// first level at which slot s starts a cell (0 for s == 0); D+1 if none
__device__ __forceinline__ int slot_dmin(const uint32_t* k, uint32_t s, int D) {
    return s == 0 ? 0 : common_bits(k[s - 1], k[s], 2 * D) / 2 + 1;
}
// finest level at which the cell starting at s holds >= 2 particles; -1 if none
__device__ __forceinline__ int slot_dmax(const uint32_t* k, uint32_t s, uint32_t nv, int D) {
    return s + 1 < nv ? common_bits(k[s], k[s + 1], 2 * D) / 2 : -1;
}

// ------------------------------------------------------------------------------------
// bounding box: grid-stride min/max; the last block derives the box in FP64
// ------------------------------------------------------------------------------------
constexpr int kBBoxThreads = 256;
constexpr int kBBoxBlocks = 608;  // 4 per SM: enough loads in flight to reach HBM rate

// bbox_blocks(n): blocks of a plain launch, every thread reading at least 4 particle pairs
inline int bbox_blocks(uint64_t n) {
    const uint64_t b = (n / 2 + kBBoxThreads * 4 - 1) / (kBBoxThreads * 4);
    return (int)(b < 1 ? 1 : b > (uint64_t)kBBoxBlocks ? kBBoxBlocks : b);
}

// Min/max of this block's particles, reduced over the block (every thread returns it).
// n is a multiple of 64: two particles per 16-byte load.  Min/max ignore NaN and are
// exact in any order.
__device__ __forceinline__ float4 bbox_block_minmax(Blk blk, const float2* __restrict__ pos, uint32_t n) {
    __shared__ float s[4][kBBoxThreads / 32];
    float mnx = INFINITY, mxx = -INFINITY, mny = INFINITY, mxy = -INFINITY;
    const float4* __restrict__ pos2 = reinterpret_cast<const float4*>(pos);
    for (uint32_t i = blk.id * kBBoxThreads + threadIdx.x; i < n / 2; i += blk.count * kBBoxThreads) {
        const float4 p = pos2[i];
        mnx = fminf(mnx, fminf(p.x, p.z));
        mxx = fmaxf(mxx, fmaxf(p.x, p.z));
        mny = fminf(mny, fminf(p.y, p.w));
        mxy = fmaxf(mxy, fmaxf(p.y, p.w));
    }
    for (int o = 16; o; o >>= 1) {
        mnx = fminf(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
        mxx = fmaxf(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
        mny = fminf(mny, __shfl_xor_sync(0xffffffffu, mny, o));
        mxy = fmaxf(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();  // s may still be read from a previous call
    if (lane == 0) {
        s[0][warp] = mnx;
        s[1][warp] = mxx;
        s[2][warp] = mny;
        s[3][warp] = mxy;
    }
    __syncthreads();
    for (int w = 0; w < kBBoxThreads / 32; ++w) {
        mnx = fminf(mnx, s[0][w]);
        mxx = fmaxf(mxx, s[1][w]);
        mny = fminf(mny, s[2][w]);
        mxy = fmaxf(mxy, s[3][w]);
    }
    return make_float4(mnx, mxx, mny, mxy);
}

// The box parameters from the extent: a square around it, 1/1024 margin, 2^bits cells
// per axis, in FP64.
__device__ __forceinline__ BHParams bbox_params(float4 ext4, int bits) {
    const double a = ext4.x, b = ext4.y, c = ext4.z, d = ext4.w;
    double cx = 0.5 * (a + b), cy = 0.5 * (c + d);
    double ext = b - a > d - c ? b - a : d - c;
    if (!(ext > 0.0) || !isfinite(ext)) ext = 1.0;
    if (!isfinite(cx)) cx = 0.0;
    if (!isfinite(cy)) cy = 0.0;
    double half = ext * 0.5 * (1.0 + 1.0 / 1024.0);
    double scale = (double)(1u << (bits - 1)) / half;
    BHParams p;
    p.bits = bits;
    p.cx = (float)cx;
    p.cy = (float)cy;
    p.scale = (float)scale;
    double side0 = (double)(1u << bits) / (double)p.scale;
    p.radius0 = (float)(side0 * side0 * 0.5);
    p.inv_scale = (float)(1.0 / (double)p.scale);
    return p;
}

// The extent of `count` block partials, reduced by the whole block (every thread).
__device__ __forceinline__ float4 bbox_reduce_partials(const float* __restrict__ part, uint32_t count) {
    float mnx = INFINITY, mxx = -INFINITY, mny = INFINITY, mxy = -INFINITY;
    for (uint32_t bl = threadIdx.x; bl < count; bl += kBBoxThreads) {
        mnx = fminf(mnx, __ldcg(&part[4 * bl + 0]));
        mxx = fmaxf(mxx, __ldcg(&part[4 * bl + 1]));
        mny = fminf(mny, __ldcg(&part[4 * bl + 2]));
        mxy = fmaxf(mxy, __ldcg(&part[4 * bl + 3]));
    }
    __shared__ float s[4][kBBoxThreads / 32];
    for (int o = 16; o; o >>= 1) {
        mnx = fminf(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
        mxx = fmaxf(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
        mny = fminf(mny, __shfl_xor_sync(0xffffffffu, mny, o));
        mxy = fmaxf(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) {
        s[0][warp] = mnx;
        s[1][warp] = mxx;
        s[2][warp] = mny;
        s[3][warp] = mxy;
    }
    __syncthreads();
    for (int w = 0; w < kBBoxThreads / 32; ++w) {
        mnx = fminf(mnx, s[0][w]);
        mxx = fmaxf(mxx, s[1][w]);
        mny = fminf(mny, s[2][w]);
        mxy = fmaxf(mxy, s[3][w]);
    }
    return make_float4(mnx, mxx, mny, mxy);
}

// One launch: block partials, then the last block to finish (ticket) reduces them all
// and writes the box parameters.
__device__ __forceinline__ void bbox_body(Blk blk, const float2* __restrict__ pos, uint32_t n,
                                          float* __restrict__ part, uint32_t* __restrict__ ticket,
                                          BHParams* __restrict__ out, int bits) {
    __shared__ bool last;
    const float4 m = bbox_block_minmax(blk, pos, n);
    if (threadIdx.x == 0) {
        part[4 * blk.id + 0] = m.x;
        part[4 * blk.id + 1] = m.y;
        part[4 * blk.id + 2] = m.z;
        part[4 * blk.id + 3] = m.w;
        __threadfence();
        last = atomicAdd(ticket, 1u) == blk.count - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    const float4 e = bbox_reduce_partials(part, blk.count);
    if (threadIdx.x == 0) *out = bbox_params(e, bits);
}

// ------------------------------------------------------------------------------------
// keygen + digit histograms
// ------------------------------------------------------------------------------------
constexpr int kKeyThreads = 256;
// Keygen blocks: each block adds its digit histograms to the global ones with up to
// 4 x 256 atomics, so a few blocks per SM (grid-stride) keep those atomics few; one
// block per 256 particles spent 25 us of a 500k step on them, 608 blocks 10 us.
constexpr int kKeyBlocks = 608;
inline int keygen_blocks(uint64_t n) {
    const uint64_t b = (n + kKeyThreads - 1) / kKeyThreads;
    return (int)(b < 1 ? 1 : b > (uint64_t)kKeyBlocks ? kKeyBlocks : b);
}

// mmax (quadrupole mode, else null): the largest mass after the removal, as float bits
// (masses >= 0 order like their bits), for the grid of the exact moment sums.
__device__ __forceinline__ void keygen_body(Blk blk, int bbox_mode, const BHParams* __restrict__ bp,
                                            float2* __restrict__ pos_in, float* mass_in, float2* __restrict__ pos_out,
                                            float* mass_out,  // mass sets may alias
                                            uint32_t n, uint32_t* __restrict__ keys, uint32_t* __restrict__ hist,
                                            int passes, uint32_t* __restrict__ valid_count,
                                            uint32_t* __restrict__ mmax = nullptr) {
    __shared__ uint32_t sh[4][256];
    for (int i = threadIdx.x; i < 4 * 256; i += kKeyThreads) (&sh[0][0])[i] = 0u;
    __syncthreads();
    BHParams p;
    if (bbox_mode) p = *bp;
    uint32_t valid = 0, mbits = 0;
    for (uint32_t i = blk.id * kKeyThreads + threadIdx.x; i < n; i += blk.count * kKeyThreads) {
        float2 q = pos_in[i];
        uint32_t key;
        if (bbox_mode) {
            key = spread_bits(bbox_cell(q.x, p.cx, p.scale, p.bits)) |
                  (spread_bits(bbox_cell(q.y, p.cy, p.scale, p.bits)) << 1);
            ++valid;
            if (mmax) {
                const float m = mass_in[i];
                if (m > 0.0f) mbits = max(mbits, __float_as_uint(m));
            }
        } else if (fixed_key(q.x, q.y, key)) {
            ++valid;
            if (mmax) {
                const float m = mass_in[i];
                if (m > 0.0f) mbits = max(mbits, __float_as_uint(m));
            }
        } else {  // InitShader.comp:110-117
            key = kKeyRemovedSort;
            const float2 gone = make_float2(-kSimSize * 2.0f, -kSimSize * 2.0f);
            pos_in[i] = gone;
            pos_out[i] = gone;
            mass_in[i] = 0.0f;
            mass_out[i] = 0.0f;
        }
        keys[i] = key;
        for (int ps = 0; ps < passes; ++ps) atomicAdd(&sh[ps][(key >> (8 * ps)) & 255u], 1u);
    }
    for (int o = 16; o; o >>= 1) valid += __shfl_xor_sync(0xffffffffu, valid, o);
    if ((threadIdx.x & 31) == 0 && valid) atomicAdd(valid_count, valid);
    if (mmax) {
        mbits = __reduce_max_sync(0xffffffffu, mbits);
        if ((threadIdx.x & 31) == 0 && mbits) atomicMax(mmax, mbits);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * 256; i += kKeyThreads) {
        uint32_t c = (&sh[0][0])[i];
        if (c) atomicAdd(&hist[i], c);
    }
}

__global__ void __launch_bounds__(kKeyThreads)
k_keygen(int bbox_mode, const BHParams* __restrict__ bp, float2* __restrict__ pos_in, float* mass_in,
         float2* __restrict__ pos_out, float* mass_out, uint32_t n, uint32_t* __restrict__ keys,
         uint32_t* __restrict__ hist, int passes, uint32_t* __restrict__ valid_count, uint32_t* __restrict__ mmax) {
    pdl_enter();
    keygen_body(grid_blk(), bbox_mode, bp, pos_in, mass_in, pos_out, mass_out, n, keys, hist, passes, valid_count,
                mmax);
}

// ------------------------------------------------------------------------------------
// block-wide exclusive scan of one value per thread (256 threads)
// ------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t block_exclusive_scan_256(uint32_t v, uint32_t* s_warp, uint32_t& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < 8 ? s_warp[lane] : 0u;
        for (int o = 1; o < 8; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < 8) s_warp[lane] = w;  // inclusive per warp
    }
    __syncthreads();
    total = s_warp[7];
    uint32_t warp_off = warp ? s_warp[warp - 1] : 0u;
    uint32_t r = warp_off + x - v;
    __syncthreads();
    return r;
}

// Barrier over every block of a cooperative launch (all blocks are co-resident, so
// every block reaches it).  Block leaders count arrivals on `bar` and wait for `target`;
// the wait is bounded, and a block that gives up sets the error flag, which makes the
// others stop waiting too.  Returns false after a failed wait.
__device__ __forceinline__ bool grid_sync(uint32_t* bar, uint32_t target, int* err) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();  // this block's moments are visible before it is counted
        atomicAdd(bar, 1u);
        int ok = 1;
        uint32_t spins = 0;
        while (ld_acquire_u32(bar) < target) {
            if (++spins > kSpinLimit) {
                atomicOr(err, kErrBarrierWait);
                ok = 0;
                break;
            }
            if ((spins & 255u) == 0u && ld_volatile((const uint32_t*)err) & kErrBarrierWait) {
                ok = 0;
                break;
            }
            __nanosleep(32);
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Keys in bounding-box mode.  The extent of the input positions was gathered while they
// were written (by the previous step's traversal kernel, or by the upload), so every
// block derives the box from those four words and goes on to the keys: no pass over
// the positions and no grid barrier before them.  Block 0 stores the box for the later
// stages and clears the output set's extent for this step's traversal kernel.
__global__ void __launch_bounds__(kKeyThreads)
k_ext_keys(float2* __restrict__ pos_in, float* mass_in, float2* __restrict__ pos_out, float* mass_out, uint32_t n,
           uint32_t* __restrict__ keys, uint32_t* __restrict__ hist, int passes, uint32_t* __restrict__ valid_count,
           BHParams* __restrict__ params, const uint32_t* __restrict__ ext_in, uint32_t* __restrict__ ext_out,
           int bits, uint32_t* __restrict__ mmax) {
    pdl_enter();
    __shared__ BHParams sp;
    if (threadIdx.x == 0) {
        sp = bbox_params(ext_decode(ext_in), bits);
        if (blockIdx.x == 0) {
            *params = sp;
            for (int j = 0; j < 4; ++j) ext_out[j] = 0xFFFFFFFFu;
        }
    }
    __syncthreads();
    keygen_body(grid_blk(), 1, &sp, pos_in, mass_in, pos_out, mass_out, n, keys, hist, passes, valid_count, mmax);
}


// ------------------------------------------------------------------------------------
// onesweep radix pass (stable, 8-bit digit at `shift`)
// ------------------------------------------------------------------------------------
// Tiles are taken from a per-system ticket, so a tile only waits on tiles that earlier
// running blocks took: no deadlock, whichever grid the blocks belong to.
// KPT keys per thread: tiles of 256 * KPT keys; LB: look-back width.
template <bool IDENTITY, int KPT, int LB>
__device__ __forceinline__ void sort_pass_body(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                                               uint32_t* __restrict__ kout, uint32_t* __restrict__ vout, uint32_t n,
                                               int shift, const uint32_t* __restrict__ hist,
                                               uint32_t* __restrict__ status, uint32_t* __restrict__ ticket,
                                               int* __restrict__ err) {
    constexpr int kSortTile = kSortThreads * KPT;
    constexpr int W = kSortThreads / 32;
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_whist[W][256];
    __shared__ uint32_t s_start[256];
    __shared__ uint32_t s_gbase[256];
    __shared__ uint32_t s_warp[8];
    __shared__ uint32_t s_keys[kSortTile];
    __shared__ uint32_t s_vals[kSortTile];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    for (int i = t; i < W * 256; i += kSortThreads) (&s_whist[0][0])[i] = 0u;
    if (t == 0) s_tile = atomicAdd(ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t base = tile * kSortTile;
    const uint32_t wbase = base + warp * 32 * KPT;

    uint32_t key[KPT], val[KPT], rank[KPT];
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
        uint32_t i = wbase + j * 32 + lane;
        bool ok = i < n;
        key[j] = ok ? kin[i] : 0u;
        val[j] = ok ? (IDENTITY ? i : vin[i]) : 0u;
    }
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int j = 0; j < KPT; ++j) {  // warp-local stable ranks, order (j, lane)
        uint32_t i = wbase + j * 32 + lane;
        bool ok = i < n;
        uint32_t d = (key[j] >> shift) & 255u;
        uint32_t peers = __match_any_sync(0xffffffffu, ok ? d : 0xffffffffu);
        uint32_t prev = ok ? s_whist[warp][d] : 0u;
        rank[j] = prev + __popc(peers & lt);
        __syncwarp();
        if (ok && (__ffs(peers) - 1) == lane) s_whist[warp][d] = prev + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // per digit (thread t = digit t): exclusive offsets over warps, tile count
    uint32_t tot = 0;
#pragma unroll
    for (int w = 0; w < W; ++w) {
        uint32_t c = s_whist[w][t];
        s_whist[w][t] = tot;
        tot += c;
    }
    // decoupled look-back over earlier tiles for digit t, LB tiles per round trip: the
    // aggregates are added nearest first up to the first inclusive prefix; a tile not yet
    // published ends the window, and the next window starts there.  Tile t resolves about
    // t / LB round trips after tile 0, so the window width sets the pass's latency.
    uint32_t excl = 0;
    uint32_t* st = status + (size_t)tile * 256 + t;
    if (tile == 0) {
        atomicExch(st, (2u << 30) | tot);
    } else {
        atomicExch(st, (1u << 30) | tot);
        int64_t p = (int64_t)tile - 1;
        uint32_t spins = 0;
        while (p >= 0) {
            uint32_t w[LB];
#pragma unroll
            for (int k = 0; k < LB; ++k)
                w[k] = p - k >= 0 ? ld_volatile(status + (size_t)(p - k) * 256 + t) : (2u << 30);
            bool stop = false, done = false;
            int used = 0;
#pragma unroll
            for (int k = 0; k < LB; ++k) {
                if (stop) continue;
                const uint32_t f = w[k] >> 30;
                if (f == 0u) {
                    stop = true;
                } else {
                    excl += w[k] & 0x3fffffffu;
                    ++used;
                    if (f == 2u) stop = done = true;
                }
            }
            if (done) break;
            if (used < LB && ++spins > kSpinLimit) {
                atomicOr(err, kErrSortWait);
                break;
            }
            p -= used;
        }
        atomicExch(st, (2u << 30) | (excl + tot));
    }
    uint32_t total;
    const uint32_t gofs = block_exclusive_scan_256(hist[t], s_warp, total);
    const uint32_t lstart = block_exclusive_scan_256(tot, s_warp, total);
    s_start[t] = lstart;
    s_gbase[t] = gofs + excl - lstart;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
        uint32_t i = wbase + j * 32 + lane;
        if (i < n) {
            uint32_t d = (key[j] >> shift) & 255u;
            uint32_t lp = s_start[d] + s_whist[warp][d] + rank[j];
            s_keys[lp] = key[j];
            s_vals[lp] = val[j];
        }
    }
    __syncthreads();
    const uint32_t tile_n = min((uint32_t)kSortTile, n - base);
    for (uint32_t i = t; i < tile_n; i += kSortThreads) {
        uint32_t k = s_keys[i];
        uint32_t g = s_gbase[(k >> shift) & 255u] + i;
        if (g < n) {  // always true unless a look-back wait gave up (error flag set)
            kout[g] = k;
            vout[g] = s_vals[i];
        }
    }
}

template <bool IDENTITY, int KPT, int LB>
__global__ void __launch_bounds__(kSortThreads)
k_sort_pass(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin, uint32_t* __restrict__ kout,
            uint32_t* __restrict__ vout, uint32_t n, int shift, const uint32_t* __restrict__ hist,
            uint32_t* __restrict__ status, uint32_t* __restrict__ ticket, int* __restrict__ err) {
    pdl_enter();
    sort_pass_body<IDENTITY, KPT, LB>(kin, vin, kout, vout, n, shift, hist, status, ticket, err);
}

// radix pass kernel of a tile size and look-back width (first pass: values are the identity)
using SortPassFn = void (*)(const uint32_t*, const uint32_t*, uint32_t*, uint32_t*, uint32_t, int, const uint32_t*,
                            uint32_t*, uint32_t*, int*);
template <int KPT>
SortPassFn sort_pass_kernel_kpt(bool identity, uint32_t lb) {
    switch (lb) {
        case 8: return identity ? k_sort_pass<true, KPT, 8> : k_sort_pass<false, KPT, 8>;
        case 16: return identity ? k_sort_pass<true, KPT, 16> : k_sort_pass<false, KPT, 16>;
        default: return identity ? k_sort_pass<true, KPT, 32> : k_sort_pass<false, KPT, 32>;
    }
}
SortPassFn sort_pass_kernel(bool identity, const gs_shape& sh) {
    return sh.sort_keys_per_thread == 8 ? sort_pass_kernel_kpt<8>(identity, sh.sort_lookback)
                                        : sort_pass_kernel_kpt<16>(identity, sh.sort_lookback);
}
// radix-sort tiles of n keys under a shape
inline uint32_t sort_tiles_of(uint64_t n, const gs_shape& sh) {
    const uint64_t tile = (uint64_t)kSortThreads * (sh.sort_keys_per_thread == 8 ? 8 : 16);
    return (uint32_t)((n + tile - 1) / tile);
}

// ------------------------------------------------------------------------------------
// internal nodes per slot + exclusive scan (decoupled look-back)
// ------------------------------------------------------------------------------------
// R: earlier tiles each lane of the look-back warp reads per round trip (32 R per warp).
template <int R>
__device__ __forceinline__ void meta_scan_body(const uint32_t* __restrict__ skey, uint32_t n_items,
                                               const uint32_t* __restrict__ valid_count, int D,
                                               uint32_t* __restrict__ E, uint32_t* __restrict__ status,
                                               uint32_t* __restrict__ ticket, uint32_t* __restrict__ internal_count,
                                               int* __restrict__ err) {
    __shared__ uint32_t s_tile, s_prefix;
    __shared__ uint32_t s_warp[8];
    const int t = threadIdx.x;
    if (t == 0) s_tile = atomicAdd(ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t nv = *valid_count;
    const uint32_t first = tile * kScanTile + t * kScanItems;
    uint32_t e[kScanItems];
    uint32_t sum = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        uint32_t s = first + j;
        int c = 0;
        if (s < nv) c = slot_dmax(skey, s, nv, D) - slot_dmin(skey, s, D) + 1;
        e[j] = c > 0 ? (uint32_t)c : 0u;
        sum += e[j];
    }
    uint32_t total;
    uint32_t texcl = block_exclusive_scan_256(sum, s_warp, total);
    if (t < 32) {  // warp 0: publish, then look back over 32 R earlier tiles per round trip
        uint32_t excl = 0;
        uint32_t* st = status + tile;
        if (tile == 0) {
            if (t == 0) atomicExch(st, (2u << 30) | total);
        } else {
            if (t == 0) atomicExch(st, (1u << 30) | total);
            int64_t p = (int64_t)tile - 1;
            uint32_t spins = 0;
            while (p >= 0) {  // every value below is uniform over the warp
                uint32_t w[R];
#pragma unroll
                for (int r = 0; r < R; ++r) {  // lane t reads the (32 r + t)-th tile back
                    const int64_t q = p - 32 * r - t;
                    w[r] = q >= 0 ? ld_volatile(status + q) : (2u << 30);
                }
                bool done = false, wait = false;
                int64_t used = 0;
#pragma unroll
                for (int r = 0; r < R; ++r) {  // nearest 32 first
                    if (done || wait) continue;
                    const uint32_t f = w[r] >> 30;
                    const uint32_t stopm = __ballot_sync(0xffffffffu, f != 1u);  // unpublished or inclusive
                    const int k = stopm ? __ffs(stopm) - 1 : 32;
                    const uint32_t kf = __shfl_sync(0xffffffffu, f, k & 31);
                    const bool inclusive = k < 32 && kf == 2u;
                    // the aggregates nearer than lane k, and lane k's value if it is inclusive
                    excl += __reduce_add_sync(0xffffffffu,
                                              (t < k || (t == k && inclusive)) ? (w[r] & 0x3fffffffu) : 0u);
                    if (inclusive) done = true;
                    else if (k < 32) wait = true;  // tile p - used - k has not published yet
                    used += inclusive ? 0 : k;
                }
                if (done) break;
                if (wait && ++spins > kSpinLimit) {
                    if (t == 0) atomicOr(err, kErrScanWait);
                    break;
                }
                p -= used;
            }
            if (t == 0) atomicExch(st, (2u << 30) | (excl + total));
        }
        if (t == 0) s_prefix = excl;
    }
    __syncthreads();
    uint32_t run = s_prefix + texcl;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        uint32_t s = first + j;
        if (s < n_items) E[s] = run;
        if (s == nv) *internal_count = run;
        run += e[j];
    }
}

// Quadrupole mode: the exact moment sums of the sorted slots (moments.cuh).
struct MomIn {
    const BHParams* bp;          // box of the step
    const uint32_t* mmax;        // float bits of the largest mass
    int bbox;                    // box mode
    int4* qv;                    // [N_al] integer mass and position per slot (k_records)
    i128* prefix;                // six columns [stride] of exclusive prefixes (null: monopole mode)
    size_t stride;               // N_al + 1
    MomSums* agg;                // [tiles] each tile's sums
    uint32_t* nend;              // [cap] one past the last slot of internal node j (k_nodes)
};

constexpr int kMomThreads = 256, kMomItems = 4;  // k_mom_scan: threads and slots per thread
constexpr int kMomTile = kMomThreads * kMomItems;

// one column of a slot's sums from its integer mass and position
__device__ __forceinline__ i128 mom_column(int4 q, int ch) {
    switch (ch) {
        case 0: return (i128)q.x;
        case 1: return (i128)((long long)q.x * q.y);
        case 2: return (i128)((long long)q.x * q.z);
        case 3: return mul_i64_i32((long long)q.x * q.y, q.y);
        case 4: return mul_i64_i32((long long)q.x * q.y, q.z);
        default: return mul_i64_i32((long long)q.x * q.z, q.z);
    }
}
__device__ __forceinline__ i128 mom_get(const MomSums& a, int ch) {
    return ch == 0 ? a.m : ch == 1 ? a.x : ch == 2 ? a.y : ch == 3 ? a.xx : ch == 4 ? a.xy : a.yy;
}

// Exact sums of every slot of one tile, in every thread of the block (s_w: scratch).
__device__ __forceinline__ MomSums mom_block_total(MomSums a, MomSums* s_w) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    mom_warp_sum(a);
    __syncthreads();  // s_w may still be read by an earlier use
    if (lane == 0) s_w[warp] = a;
    __syncthreads();
    MomSums tsum;
    mom_clear(tsum);
    for (int w = 0; w < kMomThreads / 32; ++w) mom_add(tsum, s_w[w]);
    return tsum;
}

// k_mom_tiles: the exact sums of each tile of kMomTile slots.
__device__ __forceinline__ void mom_tiles_body(uint32_t tile, uint32_t nv, const MomIn& mi) {
    __shared__ MomSums s_w[kMomThreads / 32];
    const uint64_t first = (uint64_t)tile * kMomTile;
    MomSums c;
    mom_clear(c);
#pragma unroll
    for (int j = 0; j < kMomItems; ++j) {
        const uint64_t sl = first + (uint64_t)j * kMomThreads + threadIdx.x;  // coalesced
        if (sl < nv) mom_add_q(c, mi.qv[sl]);
    }
    const MomSums tsum = mom_block_total(c, s_w);
    if (threadIdx.x == 0) mi.agg[tile] = tsum;
}

// k_mom_scan: the exclusive prefix of the exact sums at the slots of one tile: the sums
// of the tiles before it (every block adds them up itself: integer sums, any order),
// then, with the tile staged in shared memory, each thread's kMomItems consecutive slots
// and a block scan.  The prefix is written one column at a time through shared memory,
// so that the stores are contiguous.
// 16-byte elements padded by one every eight: a thread's kMomItems consecutive elements
// and a warp's consecutive elements both fall in distinct banks
__device__ __forceinline__ int mom_pad(int i) { return i + (i >> 3); }

__device__ __forceinline__ void mom_scan_body(uint32_t tile, uint32_t n_items, uint32_t nv, const MomIn& mi) {
    __shared__ int4 s_q[kMomTile + kMomTile / 8];
    __shared__ ulonglong2 s_out[kMomTile + kMomTile / 8];
    __shared__ MomSums s_w[kMomThreads / 32];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint64_t first = (uint64_t)tile * kMomTile;
    MomSums a;
    mom_clear(a);
    for (uint32_t j = t; j < tile; j += kMomThreads) mom_add(a, mom_ldcg(mi.agg + j));
    const MomSums base = mom_block_total(a, s_w);
    for (int k = t; k < kMomTile; k += kMomThreads) {
        const uint64_t sl = first + k;
        s_q[mom_pad(k)] = sl < nv ? mi.qv[sl] : make_int4(0, 0, 0, 0);
    }
    __syncthreads();
    MomSums c;
    mom_clear(c);
#pragma unroll
    for (int j = 0; j < kMomItems; ++j) mom_add_q(c, s_q[mom_pad(t * kMomItems + j)]);
    MomSums incl = c;
    mom_warp_scan(incl, lane);
    if (lane == 31) s_w[warp] = incl;  // the last read of s_w was before the staging sync
    __syncthreads();
    MomSums b = base;  // this thread's first slot
    for (int w = 0; w < warp; ++w) mom_add(b, s_w[w]);
    b.m += incl.m - c.m;
    b.x += incl.x - c.x;
    b.y += incl.y - c.y;
    b.xx += incl.xx - c.xx;
    b.xy += incl.xy - c.xy;
    b.yy += incl.yy - c.yy;
    ulonglong2* out = reinterpret_cast<ulonglong2*>(mi.prefix);
#pragma unroll
    for (int ch = 0; ch < 6; ++ch) {
        i128 run = mom_get(b, ch);
#pragma unroll
        for (int j = 0; j < kMomItems; ++j) {
            s_out[mom_pad(t * kMomItems + j)] = make_ulonglong2((unsigned long long)run,
                                                                (unsigned long long)((u128)run >> 64));
            run += mom_column(s_q[mom_pad(t * kMomItems + j)], ch);
        }
        __syncthreads();
        for (int k = t; k < kMomTile; k += kMomThreads) {
            const uint64_t sl = first + k;
            if (sl < n_items) out[ch * mi.stride + sl] = s_out[mom_pad(k)];
        }
        __syncthreads();
    }
}

template <int R>
__global__ void __launch_bounds__(kScanThreads)
k_meta_scan(const uint32_t* __restrict__ skey, uint32_t n_items, const uint32_t* __restrict__ valid_count,
            int D, uint32_t* __restrict__ E, uint32_t* __restrict__ status, uint32_t* __restrict__ ticket,
            uint32_t* __restrict__ internal_count, int* __restrict__ err) {
    pdl_enter();
    meta_scan_body<R>(skey, n_items, valid_count, D, E, status, ticket, internal_count, err);
}
// Quadrupole mode: the exact moment sums of every tile, then their exclusive prefix at
// every slot.
__global__ void __launch_bounds__(kMomThreads)
k_mom_tiles(const uint32_t* __restrict__ valid_count, MomIn mi) {
    pdl_enter();
    mom_tiles_body(blockIdx.x, *valid_count, mi);
}
__global__ void __launch_bounds__(kMomThreads, 2)
k_mom_scan(uint32_t n_items, const uint32_t* __restrict__ valid_count, MomIn mi) {
    pdl_enter();
    mom_scan_body(blockIdx.x, n_items, *valid_count, mi);
}

inline auto meta_scan_kernel(uint32_t lookback) {
    return lookback >= 128 ? k_meta_scan<4> : lookback >= 64 ? k_meta_scan<2> : k_meta_scan<1>;
}

// ------------------------------------------------------------------------------------
// preorder records (topology, radius, particle leaves)
// ------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t cell_end(const uint32_t* k, uint32_t a, uint32_t nv, int shift, uint32_t pre) {
    // smallest t >= a with (k[t] >> shift) != pre, or nv; all t < a match
    uint32_t step = 1, hi = a;
    while (hi < nv && (k[hi] >> shift) == pre) {
        a = hi + 1;
        hi = a + step;
        step <<= 1;
    }
    if (hi > nv) hi = nv;
    while (a < hi) {
        uint32_t mid = a + ((hi - a) >> 1);
        if ((k[mid] >> shift) == pre) a = mid + 1;
        else hi = mid;
    }
    return a;
}

// record index of the particle leaf of sorted slot t
__device__ __forceinline__ uint32_t leaf_of(const uint32_t* skey, const uint32_t* E, uint32_t t, uint32_t nv, int D) {
    const int cmin = slot_dmin(skey, t, D), cmax = slot_dmax(skey, t, nv, D);
    return t + E[t] + (uint32_t)(cmax >= cmin ? cmax - cmin + 1 : 0);
}

// One thread per sorted slot s: the particle leaf of s, and the slot of every internal
// node that starts at s in the node -> slot map (internal ordinal j = E(s) + d - dmin(s),
// record index s + j).
__device__ __forceinline__ void records_body(Blk blk, const uint32_t* __restrict__ skey,
                                             const uint32_t* __restrict__ sidx, const uint32_t* __restrict__ E,
                                             const uint32_t* __restrict__ valid_count, int D,
                                             const float2* __restrict__ pos, const float* __restrict__ mass,
                                             float4* __restrict__ rec, uint32_t* __restrict__ skip,
                                             uint32_t* __restrict__ node_slot, uint64_t cap, uint32_t n_al,
                                             int* __restrict__ err, const MomIn& mi) {
    const uint32_t nv = *valid_count;
    MomScale sc;
    if (mi.prefix) sc = mom_scale(mi.bbox, *mi.bp, *mi.mmax);
    for (uint32_t s = blk.id * 256 + threadIdx.x; s < nv; s += blk.count * 256) {
        const int dmin = slot_dmin(skey, s, D), dmax = slot_dmax(skey, s, nv, D);
        const uint32_t Es = E[s];
        const int e = dmax >= dmin ? dmax - dmin + 1 : 0;
        const uint64_t leaf = (uint64_t)s + Es + e;
        if (leaf >= cap) {
            atomicOr(err, kErrTree);
            continue;
        }
        const uint32_t i = sidx[s];
        if (i >= n_al) {  // only after a failed sort (error flag already set)
            atomicOr(err, kErrTree);
            continue;
        }
        const float2 p = pos[i];
        const float m = mass[i];
        rec[leaf] = make_float4(p.x, p.y, m, 0.0f);
        skip[leaf] = 1u;
        if (mi.prefix) mi.qv[s] = mom_quantize(p, m, sc);
        for (int k = 0; k < e; ++k) node_slot[Es + k] = s;
    }
}

// The costly groups of the step (relative criterion, quadrupole mode): a flag per group
// and the list the traversal's warp pairs take (heavy_list_body).  Written by the records
// kernel, which every later stage of the step follows by a full dependency (the moment
// prefix starts after it completes).
struct HeavyOut {
    const float* amag;  // null: no costly groups
    uint8_t* flag;
    uint2* list;
    uint32_t* count;
    uint32_t tag;
};

__global__ void __launch_bounds__(256)
k_records(const uint32_t* __restrict__ skey, const uint32_t* __restrict__ sidx, const uint32_t* __restrict__ E,
          const uint32_t* __restrict__ valid_count, int D, const float2* __restrict__ pos,
          const float* __restrict__ mass, float4* __restrict__ rec, uint32_t* __restrict__ skip,
          uint32_t* __restrict__ node_slot, uint64_t cap, uint32_t n_al, int* __restrict__ err, MomIn mi,
          HeavyOut ho) {
    pdl_enter();
    records_body(grid_blk(), skey, sidx, E, valid_count, D, pos, mass, rec, skip, node_slot, cap, n_al, err, mi);
    if (ho.amag) heavy_list_body(grid_blk(), sidx, valid_count, ho.amag, n_al, ho.flag, ho.list, ho.count, ho.tag);
}

__device__ __forceinline__ uint32_t compact_bits(uint32_t v) {  // inverse of spread_bits
    v &= 0x55555555u;
    v = (v | (v >> 1)) & 0x33333333u;
    v = (v | (v >> 2)) & 0x0f0f0f0fu;
    v = (v | (v >> 4)) & 0x00ff00ffu;
    v = (v | (v >> 8)) & 0x0000ffffu;
    return v;
}

// Squared distance from the centre of mass to the farthest corner of the level-d cell
// holding `key` (the accurate mode's opening radius), in FP32 with the same operation
// sequence as the CPU restatement:
//   fixed box:    side = 1000 / 2^d, x0 = -500 + ix * side          (both exact)
//   bounding box: side = 2^(D-d) * inv, x0 = cx + (ix * 2^(D-d) - 2^(D-1)) * inv
//   m = max(|c - x0|, |x0 + side - c|) per axis, bmax^2 = fma(mx, mx, my * my)
__device__ __forceinline__ float cell_bmax2(int bbox_mode, const BHParams& bp, int D, int d, uint32_t key, float cx,
                                            float cy) {
    const uint32_t pre = key >> (2 * (D - d));
    const float ix = (float)compact_bits(pre), iy = (float)compact_bits(pre >> 1);
    float x0, y0, side;
    if (bbox_mode) {
        const float w = (float)(1u << (D - d));
        side = __fmul_rn(w, bp.inv_scale);
        x0 = __fadd_rn(bp.cx, __fmul_rn(__fsub_rn(__fmul_rn(ix, w), (float)(1u << (D - 1))), bp.inv_scale));
        y0 = __fadd_rn(bp.cy, __fmul_rn(__fsub_rn(__fmul_rn(iy, w), (float)(1u << (D - 1))), bp.inv_scale));
    } else {
        side = __fdiv_rn(2.0f * kSimSize, (float)(1u << d));
        x0 = __fadd_rn(-kSimSize, __fmul_rn(ix, side));
        y0 = __fadd_rn(-kSimSize, __fmul_rn(iy, side));
    }
    const float mx = fmaxf(fabsf(__fsub_rn(cx, x0)), fabsf(__fsub_rn(__fadd_rn(x0, side), cx)));
    const float my = fmaxf(fabsf(__fsub_rn(cy, y0)), fabsf(__fsub_rn(__fadd_rn(y0, side), cy)));
    return __fmaf_rn(mx, mx, __fmul_rn(my, my));
}

// Internal nodes by level: the nodes of level d are listed in levels[level_off(d) ..),
// at most level_cap(d) of them (disjoint cells of >= 2 particles: <= 4^d and <= N/2).
__host__ __device__ __forceinline__ uint32_t level_cap(int d, uint32_t n_al) {
    const uint64_t c = 1ull << (2 * d), h = n_al / 2 + 1;
    return (uint32_t)(c < h ? c : h);
}
__host__ __device__ __forceinline__ uint32_t level_off(int d, uint32_t n_al) {
    uint32_t o = 0;
    for (int e = 0; e < d; ++e) o += level_cap(e, n_al);
    return o;
}

// One thread per internal node (d, s): skip (the reference's count.y), the level radius
// of TreeMoveShader.comp:70-71, the child descriptors, and the node's entry in the list
// of its level (slots reserved per block: a shared histogram, one atomic per level).
// Quadrupole mode (mi.prefix set): the record itself is left to k_mom_nodes, which reads
// the node's end slot from mi.nend.
__device__ __forceinline__ void nodes_body(Blk blk, const uint32_t* __restrict__ skey, const uint32_t* __restrict__ E,
                                           const uint32_t* __restrict__ counts, int D,
                                           const BHParams* __restrict__ bp, const uint32_t* __restrict__ node_slot,
                                           float4* __restrict__ rec, uint32_t* __restrict__ skip,
                                           uint4* __restrict__ kids, uint2* __restrict__ nodeinfo,
                                           uint32_t* __restrict__ level_count, uint32_t* __restrict__ levels,
                                           uint32_t n_al, uint64_t cap, int* __restrict__ err, const MomIn& mi,
                                           float4* __restrict__ quad, int safe) {
    __shared__ uint32_t s_cnt[16], s_base[16];
    const uint32_t nv = counts[0], M = counts[1];
    const float radius0 = bp->radius0;
    const bool lists = mi.prefix == nullptr;  // the level lists serve only the level-by-level moments
    for (uint32_t j0 = blk.id * 256; j0 < M; j0 += blk.count * 256) {  // uniform over the block
        if (lists) {
            if (threadIdx.x < 16) s_cnt[threadIdx.x] = 0u;
            __syncthreads();
        }
        const uint32_t j = j0 + threadIdx.x;
        int d = -1;
        uint32_t at = 0, rank = 0;
        if (j < M) {
            const uint32_t s = node_slot[j];
            at = s + j;
            if (s >= nv || at >= cap) {  // only after a failed sort or scan (error flag already set)
                atomicOr(err, kErrTree);
            } else {
                d = slot_dmin(skey, s, D) + (int)(j - E[s]);
                const int shift = 2 * (D - d);
                const uint32_t ks = skey[s];
                uint32_t end;
                if (d == D) {
                    end = cell_end(skey, s + 1, nv, shift, ks >> shift);
                    kids[at] = make_uint4(kKidFinest, at + 1, end - s, 0u);  // all children are leaves
                } else {
                    // The cell ends where its level-d prefix changes (galloping search); its
                    // level-(d+1) cells, in Morton order, are the runs of prefix 4p + c,
                    // c = 0..3, inside it.  The ends of the first three are found by three
                    // binary searches run in lockstep (their loads overlap), so a large cell
                    // costs about three times log2(size) dependent loads, not four gallops.
                    end = cell_end(skey, s + 1, nv, shift, ks >> shift);
                    const int cshift = 2 * (D - d - 1);
                    const uint32_t p4 = (ks >> shift) << 2;
                    uint32_t lo[3] = {s, s, s}, hi[3] = {end, end, end};
                    while (lo[0] < hi[0] || lo[1] < hi[1] || lo[2] < hi[2]) {
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            if (lo[c] < hi[c]) {
                                const uint32_t mid = lo[c] + ((hi[c] - lo[c]) >> 1);
                                if ((skey[mid] >> cshift) <= p4 + (uint32_t)c) lo[c] = mid + 1;
                                else hi[c] = mid;
                            }
                        }
                    }
                    const uint32_t cend[4] = {lo[0], lo[1], lo[2], end};
                    uint32_t kid[4] = {kKidNone, kKidNone, kKidNone, kKidNone};
                    uint32_t nk = 0, t = s;
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        const uint32_t tend = cend[c];
                        if (tend == t) continue;  // no particle in this child cell
                        if (tend - t >= 2) kid[nk] = t + E[t] + (uint32_t)(d + 1 - slot_dmin(skey, t, D));  // node (d+1, t)
                        else kid[nk] = leaf_of(skey, E, t, nv, D) | kKidLeaf;
                        ++nk;
                        t = tend;
                    }
                    kids[at] = make_uint4(kid[0], kid[1], kid[2], kid[3]);
                }
                if (mi.prefix) mi.nend[j] = end;
                else rec[at] = make_float4(0.0f, 0.0f, 0.0f, __fdiv_rn(radius0, (float)(1u << (2 * d))));
                skip[at] = end + E[end] - at;
                nodeinfo[at] = make_uint2(ks, (uint32_t)d);  // a key of the cell, its level
                if (lists) rank = atomicAdd(&s_cnt[d], 1u);
            }
        }
        if (!lists) continue;
        __syncthreads();
        if (threadIdx.x < 16 && s_cnt[threadIdx.x]) s_base[threadIdx.x] = atomicAdd(&level_count[threadIdx.x], s_cnt[threadIdx.x]);
        __syncthreads();
        if (d >= 0) {
            const uint32_t slot = s_base[d] + rank;
            if (slot < level_cap(d, n_al)) levels[level_off(d, n_al) + slot] = at;
            else atomicOr(err, kErrTree);
        }
        __syncthreads();  // s_cnt / s_base are reused
    }
}

// Quadrupole mode: one thread per internal node: its centre, mass, opening radius and
// second moments from the exact prefix sums at its first slot and one past its last.
__device__ __forceinline__ void mom_nodes_body(Blk blk, const uint32_t* __restrict__ counts, int D,
                                               const BHParams* __restrict__ bp,
                                               const uint32_t* __restrict__ node_slot,
                                               const uint2* __restrict__ nodeinfo, float4* __restrict__ rec,
                                               float4* __restrict__ quad, int safe, uint64_t cap, const MomIn& mi) {
    const uint32_t nv = counts[0], M = counts[1];
    const BHParams bpv = *bp;
    const MomScale sc = mom_scale(mi.bbox, bpv, *mi.mmax);
    for (uint32_t j = blk.id * 256 + threadIdx.x; j < M; j += blk.count * 256) {
        const uint32_t s = node_slot[j];
        const uint64_t at = (uint64_t)s + j;
        if (s >= nv || at >= cap) continue;  // only after a failed sort or scan (k_nodes set the error flag)
        const uint32_t end = mi.nend[j];
        if (end > nv) continue;
        const uint2 info = nodeinfo[at];
        const int d = (int)info.y;
        float cx, cy, m;
        float4 q;
        mom_node(mom_load(mi.prefix, mi.stride, end), mom_load(mi.prefix, mi.stride, s), sc, cx, cy, m, q);
        const float r0 = __fdiv_rn(bpv.radius0, (float)(1u << (2 * d)));
        rec[at] = make_float4(cx, cy, m, safe ? cell_bmax2(mi.bbox, bpv, D, d, info.x, cx, cy) : r0);
        quad[at] = q;
    }
}

__global__ void __launch_bounds__(256, 4)  // 64 registers: 20.2 -> 19.1 us at 500k against 74
k_mom_nodes(const uint32_t* __restrict__ counts, int D, const BHParams* __restrict__ bp,
            const uint32_t* __restrict__ node_slot, const uint2* __restrict__ nodeinfo, float4* __restrict__ rec,
            float4* __restrict__ quad, int safe, uint64_t cap, MomIn mi) {
    pdl_enter();
    mom_nodes_body(grid_blk(), counts, D, bp, node_slot, nodeinfo, rec, quad, safe, cap, mi);
}

__global__ void __launch_bounds__(256)
k_nodes(const uint32_t* __restrict__ skey, const uint32_t* __restrict__ E, const uint32_t* __restrict__ counts,
        int D, const BHParams* __restrict__ bp, const uint32_t* __restrict__ node_slot, float4* __restrict__ rec,
        uint32_t* __restrict__ skip, uint4* __restrict__ kids, uint2* __restrict__ nodeinfo,
        uint32_t* __restrict__ level_count, uint32_t* __restrict__ levels, uint32_t n_al, uint64_t cap,
        int* __restrict__ err, MomIn mi, float4* __restrict__ quad, int safe) {
    pdl_enter();
    nodes_body(grid_blk(), skey, E, counts, D, bp, node_slot, rec, skip, kids, nodeinfo, level_count, levels, n_al,
               cap, err, mi, quad, safe);
}

// One child's contribution: mass, centre of mass and mass moments.  Loads go through L2
// (ld.cg): internal children were written by other threads of the same launch.
struct KidData {
    float m, x, y;   // mass and centre of mass (particle position for a leaf)
    float mx, my;    // mass moments (x*m, y*m for a leaf)
};

__device__ __forceinline__ KidData kid_data(uint32_t c, const float4* rec, const float2* msum) {
    KidData k;
    if (c & kKidLeaf) {
        const float4 r = __ldcg(&rec[c & ~kKidLeaf]);
        k.m = r.z;
        k.x = r.x;
        k.y = r.y;
        k.mx = __fmul_rn(r.x, r.z);
        k.my = __fmul_rn(r.y, r.z);
    } else {
        const float4 r = __ldcg(&rec[c]);
        const float2 m2 = __ldcg(&msum[c]);
        k.m = r.z;
        k.x = r.x;
        k.y = r.y;
        k.mx = m2.x;
        k.my = m2.y;
    }
    return k;
}

// Monopole mode: mass, mass moments (children in Morton order, TreeInitShader.comp:78-80),
// centre of mass (TreeMoveShader.comp:66-67) and the opening radius (the safe radius
// with GS_FLAG_SAFE_RADIUS) of node `at`.
__device__ void compute_node(uint32_t at, int D, int safe, int bbox_mode, const BHParams& bp,
                             const uint32_t* __restrict__ skey, float4* rec, const uint4* __restrict__ kids,
                             const uint2* __restrict__ nodeinfo, float2* msum) {
    const uint4 kd = kids[at];
    const uint2 info = nodeinfo[at];                    // {a key of the cell, level}
    const float r0 = safe ? 0.0f : __ldcg(&rec[at]).w;  // the level radius k_nodes wrote
    float sx = 0.0f, sy = 0.0f, sm = 0.0f;
    if (kd.x == kKidFinest) {  // particle leaves at kd.y .. kd.y + kd.z - 1
        for (uint32_t t = 0; t < kd.z; ++t) {
            const float4 r = __ldcg(&rec[kd.y + t]);
            sx = __fadd_rn(sx, __fmul_rn(r.x, r.z));
            sy = __fadd_rn(sy, __fmul_rn(r.y, r.z));
            sm = __fadd_rn(sm, r.z);
        }
    } else {
        // children fill the descriptor from the front; kKidNone marks the unused tail
        const uint32_t kk[4] = {kd.x, kd.y, kd.z, kd.w};
        KidData c[4];
#pragma unroll
        for (int t = 0; t < 4; ++t)
            if (kk[t] != kKidNone) c[t] = kid_data(kk[t], rec, msum);
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            if (kk[t] == kKidNone) continue;
            sx = __fadd_rn(sx, c[t].mx);
            sy = __fadd_rn(sy, c[t].my);
            sm = __fadd_rn(sm, c[t].m);
        }
    }
    float cx = sx, cy = sy;
    if (sm != 0.0f) {
        cx = __fdiv_rn(sx, sm);
        cy = __fdiv_rn(sy, sm);
    }
    msum[at] = make_float2(sx, sy);
    const float r = safe ? cell_bmax2(bbox_mode, bp, D, (int)info.y, info.x, cx, cy) : r0;
    rec[at] = make_float4(cx, cy, sm, r);
}

// Moments level by level, finest first: every node of level d is computed by one thread
// once the launch for level d + 1 has finished, so no node waits on another.  Every node
// sums its children in the fixed Morton order.
__device__ __forceinline__ void level_sums_body(Blk blk, int d, const uint32_t* __restrict__ level_count,
                                                const uint32_t* __restrict__ levels, uint32_t n_al,
                                                const uint32_t* __restrict__ skey, int D, float4* rec,
                                                const uint4* __restrict__ kids, const uint2* __restrict__ nodeinfo,
                                                float2* msum, int safe, int bbox_mode,
                                                const BHParams* __restrict__ bpp) {
    const uint32_t cnt = min(level_count[d], level_cap(d, n_al));
    const uint32_t* list = levels + level_off(d, n_al);
    const BHParams bp = *bpp;
    for (uint32_t t = blk.id * 256 + threadIdx.x; t < cnt; t += blk.count * 256)
        compute_node(list[t], D, safe, bbox_mode, bp, skey, rec, kids, nodeinfo, msum);
}

// Levels kLevelTop .. 0 in one block, a barrier between levels.
__device__ __forceinline__ void top_sums_body(const uint32_t* __restrict__ level_count,
                                              const uint32_t* __restrict__ levels, uint32_t n_al,
                                              const uint32_t* __restrict__ skey, int D, float4* rec,
                                              const uint4* __restrict__ kids, const uint2* __restrict__ nodeinfo,
                                              float2* msum, int safe, int bbox_mode,
                                              const BHParams* __restrict__ bpp) {
    const BHParams bp = *bpp;
    for (int d = min(kLevelTop, D); d >= 0; --d) {
        const uint32_t cnt = min(level_count[d], level_cap(d, n_al));
        const uint32_t* list = levels + level_off(d, n_al);
        for (uint32_t t = threadIdx.x; t < cnt; t += blockDim.x)
            compute_node(list[t], D, safe, bbox_mode, bp, skey, rec, kids, nodeinfo, msum);
        __syncthreads();  // level d is complete (and visible to the block) before level d - 1
    }
}

// Monopole moments of every level in one cooperative launch: levels D .. kLevelTop + 1
// spread over the whole grid, a grid barrier after each, then levels kLevelTop .. 0 in
// block 0 with block barriers.  Each level's nodes are computed exactly as by the
// per-level launches.
constexpr int kCoopSumsThreads = 256;

__global__ void __launch_bounds__(kCoopSumsThreads, 2)
k_coop_sums(const uint32_t* __restrict__ level_count, const uint32_t* __restrict__ levels, uint32_t n_al,
            const uint32_t* __restrict__ skey, int D, float4* rec, const uint4* __restrict__ kids,
            const uint2* __restrict__ nodeinfo, float2* msum, int safe, int bbox_mode,
            const BHParams* __restrict__ bpp, uint32_t* __restrict__ bar, int* __restrict__ err) {
    pdl_enter();
    const BHParams bp = *bpp;
    uint32_t target = 0;
    for (int d = D; d > kLevelTop; --d) {
        const uint32_t cnt = min(level_count[d], level_cap(d, n_al));
        const uint32_t* list = levels + level_off(d, n_al);
        for (uint32_t t = blockIdx.x * kCoopSumsThreads + threadIdx.x; t < cnt; t += gridDim.x * kCoopSumsThreads)
            compute_node(list[t], D, safe, bbox_mode, bp, skey, rec, kids, nodeinfo, msum);
        target += gridDim.x;
        if (!grid_sync(bar, target, err)) return;
    }
    if (blockIdx.x == 0) top_sums_body(level_count, levels, n_al, skey, D, rec, kids, nodeinfo, msum, safe, bbox_mode, bpp);
}

__global__ void k_set_params(BHParams* __restrict__ out, BHParams v) { *out = v; }

}  // namespace

// Bits per axis of the bounding-box keys (gs_params.key_bits, 0: the default 12).
int bh_key_bits(const gs_params* p) { return p->key_bits ? p->key_bits : kBBoxBits; }

// Records: the particle leaves plus at most level_cap(d) internal nodes per level d
// (disjoint cells of >= 2 particles).
uint64_t bh_capacity(int D, uint64_t n_al) {
    uint64_t c = n_al + 64;
    for (int d = 0; d <= D; ++d) c += level_cap(d, (uint32_t)n_al);
    return c;
}

// Lays the Barnes-Hut scratch out in the system's slab (sim_carve); while the system is
// being sized (no slab yet) this only counts bytes.
void bh_carve(gs_sim* s) {
    BHWork& w = s->bh;
    const uint64_t n = s->n_al;
    const bool bbox = s->p.box_mode == GS_BOX_BOUNDING;
    w.depth = bbox ? bh_key_bits(&s->p) : kFixedDepth;
    // 8-bit digits: 2 * depth key bits in the bounding box (3 passes for 24-bit keys, 4 for
    // 30-bit keys), 20-bit keys + removal bit in the fixed box (3 passes)
    w.passes = bbox ? (2 * w.depth + 7) / 8 : 3;
    w.cap = bh_capacity(w.depth, n);
    w.sort_tiles = (uint32_t)((n + kSortThreads * 8 - 1) / (kSortThreads * 8));  // status for the smallest tiles
    w.scan_tiles = (uint32_t)((n + 1 + kScanTile - 1) / kScanTile);
    for (int b = 0; b < 2; ++b) {
        sim_carve(s, (void**)&w.keys[b], n * sizeof(uint32_t));
        sim_carve(s, (void**)&w.idx[b], n * sizeof(uint32_t));
    }
    sim_carve(s, (void**)&w.E, (n + 1) * sizeof(uint32_t));
    sim_carve(s, (void**)&w.rec, (w.cap + 32) * sizeof(float4));
    sim_carve(s, (void**)&w.skip, (w.cap + 32) * sizeof(uint32_t));
    sim_carve(s, (void**)&w.msum, w.cap * sizeof(float2));
    sim_carve(s, (void**)&w.kids, w.cap * sizeof(uint4));
    w.levels = nullptr;  // internal records by level: only the level-by-level moments read them
    if (!(s->p.flags & GS_FLAG_QUADRUPOLE))
        sim_carve(s, (void**)&w.levels, (size_t)level_off(w.depth + 1, (uint32_t)n) * sizeof(uint32_t));
    sim_carve(s, (void**)&w.nodeinfo, w.cap * sizeof(uint2));
    sim_carve(s, (void**)&w.node_slot, w.cap * sizeof(uint32_t));
    w.quad = nullptr;
    w.mom_q = nullptr;
    w.mom_prefix = nullptr;
    w.mom_agg = nullptr;
    w.mom_nend = nullptr;
    w.mom_blocks = 0;
    if (s->p.flags & GS_FLAG_QUADRUPOLE) {
        w.mom_blocks = (uint32_t)((n + 1 + kMomTile - 1) / kMomTile);
        sim_carve(s, (void**)&w.quad, w.cap * sizeof(float4));
        sim_carve(s, (void**)&w.mom_q, n * sizeof(int4));
        sim_carve(s, (void**)&w.mom_prefix, 6 * (n + 1) * sizeof(__int128));
        sim_carve(s, (void**)&w.mom_agg, (size_t)w.mom_blocks * sizeof(MomSums));
        sim_carve(s, (void**)&w.mom_nend, w.cap * sizeof(uint32_t));
    }
    w.amag = nullptr;
    w.heavy_flag = nullptr;
    w.heavy_list = nullptr;
    if (s->p.flags & GS_FLAG_RELATIVE_MAC) {
        sim_carve(s, (void**)&w.amag, n * sizeof(float));
        sim_carve(s, (void**)&w.heavy_flag, (n / kGroupSize + 1) * sizeof(uint8_t));
        sim_carve(s, (void**)&w.heavy_list, (n / kGroupSize + 1) * sizeof(uint2));
    }
    w.ext = nullptr;
    if (bbox) sim_carve(s, (void**)&w.ext, 8 * sizeof(uint32_t));
    sim_carve(s, (void**)&w.bbox_part, kBBoxBlocks * 4 * sizeof(float));
    sim_carve(s, (void**)&w.params, sizeof(BHParams));
    // one block cleared per step: hist | counters | sort status | scan status
    const size_t hist_b = 4 * 256 * sizeof(uint32_t);
    const size_t ctr_b = kCtrCount * sizeof(uint32_t);
    const size_t sort_b = (size_t)w.passes * w.sort_tiles * 256 * sizeof(uint32_t);
    const size_t scan_b = (size_t)w.scan_tiles * sizeof(uint32_t);
    w.zero_bytes = hist_b + ctr_b + sort_b + scan_b;
    sim_carve(s, &w.zero_base, w.zero_bytes);
    char* zb = (char*)w.zero_base;
    w.hist = zb ? (uint32_t*)zb : nullptr;
    w.counters = zb ? (uint32_t*)(zb + hist_b) : nullptr;
    w.sort_status = zb ? (uint32_t*)(zb + hist_b + ctr_b) : nullptr;
    w.scan_status = zb ? (uint32_t*)(zb + hist_b + ctr_b + sort_b) : nullptr;
}

// Initial contents: everything a debug read of a never-built tree could see is zero, the
// fixed-box parameters are in place.
cudaError_t bh_init(gs_sim* s) {
    BHWork& w = s->bh;
    cudaError_t e = cudaSuccess;
    if (w.quad) e = cudaMemsetAsync(w.quad, 0, w.cap * sizeof(float4), s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(w.zero_base, 0, w.zero_bytes, s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(w.rec, 0, (w.cap + 32) * sizeof(float4), s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(w.skip, 0, (w.cap + 32) * sizeof(uint32_t), s->stream);
    const BHParams fixed{0.0f, 0.0f, (float)kGrid / (2.0f * kSimSize), kSimSize * kSimSize * 2.0f,
                         2.0f * kSimSize / (float)kGrid, kFixedDepth};
    if (e == cudaSuccess) {  // by value through a kernel argument: nothing on the host to wait for
        k_set_params<<<1, 1, 0, s->stream>>>(w.params, fixed);
        e = cudaGetLastError();
    }
    // the cooperative moments launch: as many blocks as fit on the device at once
    int per_sm = 0, sms = 0;
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, k_coop_sums, kCoopSumsThreads, 0);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device);
    if (e == cudaSuccess && per_sm < 1) e = cudaErrorCooperativeLaunchTooLarge;
    w.sums_per_sm = per_sm;
    w.sms = sms;
    return e;
}

cudaError_t bh_step(gs_sim* s, int in, int out, bool profile, bool estimate) {
    BHWork& w = s->bh;
    cudaStream_t st = s->stream;
    const uint32_t n = (uint32_t)s->n_al;
    const bool bbox = s->p.box_mode == GS_BOX_BOUNDING;
    cudaError_t e = cudaMemsetAsync(w.zero_base, 0, w.zero_bytes, st);
    if (e != cudaSuccess) return e;
    uint32_t* ctr = w.counters;
    // programmatic launches everywhere except right after the memset, and not while
    // stage events sit between the launches
    const bool pdl = !profile;
    bool first = true;
    auto next_pdl = [&]() {
        const bool r = pdl && !first;
        first = false;
        return r;
    };
    stage_begin(s, kStageKeys, profile);
    if (bbox) {  // the box from the extent carried with the input set
        GS_TRY_LAUNCH(launch(next_pdl(), k_ext_keys, keygen_blocks(n), kKeyThreads, st, s->pos[in], s->mass[in],
                             s->pos[out], s->mass[out], n, w.keys[0], w.hist, w.passes, ctr + kCtrValid, w.params,
                             (const uint32_t*)(w.ext + 4 * in), w.ext + 4 * out, w.depth,
                             w.quad ? ctr + kCtrMaxMass : nullptr));
    } else {
        GS_TRY_LAUNCH(launch(next_pdl(), k_keygen, keygen_blocks(n), kKeyThreads, st, 0,
                             (const BHParams*)w.params, s->pos[in], s->mass[in], s->pos[out], s->mass[out], n,
                             w.keys[0], w.hist, w.passes, ctr + kCtrValid, w.quad ? ctr + kCtrMaxMass : nullptr));
    }
    count_launch(s);
    stage_end(s, kStageKeys, profile);
    stage_begin(s, kStageSort, profile);
    for (int ps = 0; ps < w.passes; ++ps) {
        const int a = ps & 1, b = a ^ 1;
        uint32_t* status = w.sort_status + (size_t)ps * w.sort_tiles * 256;
        GS_TRY_LAUNCH(launch(next_pdl(), sort_pass_kernel(ps == 0, s->shape), (int)sort_tiles_of(n, s->shape),
                             kSortThreads, st, (const uint32_t*)w.keys[a], (const uint32_t*)(ps == 0 ? nullptr : w.idx[a]),
                             w.keys[b], w.idx[b], n, 8 * ps, (const uint32_t*)(w.hist + 256 * ps), status,
                             ctr + kCtrSort + ps, s->d_err));
    }
    count_launch(s, w.passes);
    w.final_keys = w.passes & 1;
    stage_end(s, kStageSort, profile);
    const uint32_t* skey = w.keys[w.final_keys];
    const uint32_t* sidx = w.idx[w.final_keys];
    stage_begin(s, kStageScan, profile);
    GS_TRY_LAUNCH(launch(next_pdl(), meta_scan_kernel(s->shape.scan_lookback), (int)w.scan_tiles, kScanThreads, st,
                         skey, n + 1,
                         (const uint32_t*)(ctr + kCtrValid), w.depth, w.E, w.scan_status, ctr + kCtrScan,
                         ctr + kCtrInternal, s->d_err));
    count_launch(s);
    stage_end(s, kStageScan, profile);
    MomIn mi{};
    if (w.quad) {  // exact moment sums: integer values in k_records, prefix in k_mom_scan, moments in k_nodes
        mi.bp = w.params;
        mi.mmax = ctr + kCtrMaxMass;
        mi.bbox = bbox ? 1 : 0;
        mi.qv = w.mom_q;
        mi.prefix = w.mom_prefix;
        mi.stride = n + 1;
        mi.agg = w.mom_agg;
        mi.nend = w.mom_nend;
    }
    // costly groups of the relative criterion's main pass, walked by warp pairs
    const bool heavy = w.heavy_flag && w.quad && (s->p.flags & GS_FLAG_GROUP_WALK) && n >= kHeavyMinParticles;
    HeavyOut ho{};
    if (heavy) ho = HeavyOut{w.amag, w.heavy_flag, w.heavy_list, ctr + kCtrHeavy, 0u};
    stage_begin(s, kStageRecords, profile);
    GS_TRY_LAUNCH(launch(next_pdl(), k_records, grid_for(n, 256), 256, st, skey, sidx, (const uint32_t*)w.E,
                         (const uint32_t*)(ctr + kCtrValid), w.depth, (const float2*)s->pos[in],
                         (const float*)s->mass[in], w.rec, w.skip, w.node_slot, w.cap, n, s->d_err, mi, ho));
    // Quadrupole mode without stage events: the moment prefix (k_mom_tiles, k_mom_scan)
    // and the node layout (k_nodes) read only what k_records and the scan wrote and write
    // disjoint buffers, so the prefix runs on the second stream beside k_nodes and
    // k_mom_nodes waits for both.
    const bool fork = w.quad && pdl;
    cudaStream_t mst = fork ? s->side : st;
    if (fork) {
        GS_TRY_LAUNCH(cudaEventRecord(s->fork_ev, st));
        GS_TRY_LAUNCH(cudaStreamWaitEvent(mst, s->fork_ev, 0));
    }
    if (w.quad) {
        GS_TRY_LAUNCH(launch(fork ? false : next_pdl(), k_mom_tiles, (int)w.mom_blocks, kMomThreads, mst,
                             (const uint32_t*)(ctr + kCtrValid), mi));
        GS_TRY_LAUNCH(launch(fork ? true : next_pdl(), k_mom_scan, (int)w.mom_blocks, kMomThreads, mst, n + 1,
                             (const uint32_t*)(ctr + kCtrValid), mi));
        count_launch(s, 2);
    }
    GS_TRY_LAUNCH(launch(next_pdl(), k_nodes, grid_for(n, 256), 256, st, skey, (const uint32_t*)w.E,
                         (const uint32_t*)(ctr + kCtrValid), w.depth, (const BHParams*)w.params,
                         (const uint32_t*)w.node_slot, w.rec, w.skip, w.kids, w.nodeinfo, ctr + kCtrLevel, w.levels,
                         n, w.cap, s->d_err, mi, w.quad, (s->p.flags & GS_FLAG_SAFE_RADIUS) ? 1 : 0));
    count_launch(s, 2);
    if (fork) {  // the join: k_mom_nodes follows both streams with a plain launch
        GS_TRY_LAUNCH(cudaEventRecord(s->join_ev, mst));
        GS_TRY_LAUNCH(cudaStreamWaitEvent(st, s->join_ev, 0));
        first = true;
    }
    if (w.quad) {
        GS_TRY_LAUNCH(launch(next_pdl(), k_mom_nodes, grid_for(n, 256), 256, st, (const uint32_t*)(ctr + kCtrValid),
                             w.depth, (const BHParams*)w.params, (const uint32_t*)w.node_slot,
                             (const uint2*)w.nodeinfo, w.rec, w.quad, (s->p.flags & GS_FLAG_SAFE_RADIUS) ? 1 : 0,
                             (uint64_t)w.cap, mi));
        count_launch(s);
    }
    stage_end(s, kStageRecords, profile);
    stage_begin(s, kStageSums, profile);
    if (!w.quad) {  // monopole moments, level by level (the quadrupole mode has them from k_nodes)
        const int safe = (s->p.flags & GS_FLAG_SAFE_RADIUS) ? 1 : 0;
        const int bb = bbox ? 1 : 0;
        const int per_sm = (int)s->shape.moment_blocks_per_sm < w.sums_per_sm ? (int)s->shape.moment_blocks_per_sm
                                                                                : w.sums_per_sm;
        GS_TRY_LAUNCH(launch_coop(next_pdl(), k_coop_sums, w.sms * per_sm, kCoopSumsThreads, st,
                                  (const uint32_t*)(ctr + kCtrLevel), (const uint32_t*)w.levels, n, skey, w.depth,
                                  w.rec, (const uint4*)w.kids, (const uint2*)w.nodeinfo, w.msum, safe, bb,
                                  (const BHParams*)w.params, ctr + kCtrBarrier, s->d_err));
        count_launch(s);
    }
    stage_end(s, kStageSums, profile);
    stage_begin(s, kStageForce, profile);
    const float k = s->G * s->dt_eff;  // ForceShader.comp:145 (GRAVITATIONAL_CONST * SIMULATION_TIME)
    const float hdt = 0.5f * s->dt_eff;
    const bool exact = s->p.math_mode == GS_MATH_REFERENCE;
    const bool count = (s->p.flags & GS_FLAG_COUNT_INTERACTIONS) != 0;
    unsigned long long* stat = (unsigned long long*)(ctr + kCtrStat);
    const bool fpdl = next_pdl();
    ForceLaunch f;
    f.st = st;
    f.pdl = fpdl;
    f.group = (s->p.flags & GS_FLAG_GROUP_WALK) != 0;
    f.quad = w.quad != nullptr;
    f.count = count;
    f.shape = s->shape;
    f.sidx = sidx;
    f.skey = skey;
    f.counts = ctr + kCtrValid;
    f.rec = w.rec;
    f.skip = w.skip;
    f.quad_m = w.quad;
    f.kids = w.kids;
    f.pos_in = s->pos[in];
    f.vel_in = s->vel[in];
    f.pos_out = s->pos[out];
    f.vel_out = s->vel[out];
    f.n_al = n;
    f.cap = (uint32_t)w.cap;
    f.eps2 = s->eps2;
    f.theta2 = s->theta2;
    f.k = k;
    f.hdt = hdt;
    f.alpha = s->p.relative_accuracy;
    f.floor2 = s->floor2;
    f.stat = stat;
    f.err = s->d_err;
    f.amag = w.amag;
    if (heavy) {
        f.heavy = w.heavy_flag;
        f.heavy_list = w.heavy_list;
        f.heavy_work = ctr + kCtrHeavy;
    }
    auto run = exact ? force_launch_exact : force_launch_fast;
    if (f.group && estimate && w.amag && f.quad) {  // |a| of groups that have none, by the theta test
        ForceLaunch e = f;
        e.estimate = true;  // writes |a| only: no integration, no extent
        GS_TRY_LAUNCH(run(e));
        count_launch(s);
        f.pdl = pdl;
    }
    f.acc = s->acc;
    f.ext = w.ext ? w.ext + 4 * out : nullptr;
    GS_TRY_LAUNCH(run(f));
    count_launch(s);
    stage_end(s, kStageForce, profile);
    return cudaGetLastError();
}

// Host readback of the most recent tree (not on the hot path).
// Device-to-host copy on the system's stream, waited for with the system's bound.
static gs_status read_back(gs_sim* s, void* dst, const void* src, size_t bytes) {
    GS_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s->stream));
    return sim_wait(s);
}

// Host readback of the most recent tree (not on the hot path).  A wait that times out
// leaves its host buffer allocated: the copy into it may still be pending.
gs_status bh_debug_tree(gs_sim* s, uint32_t* keys, uint32_t* sorted_src, uint32_t* node_skip, float* node_radius,
                        float* node_pos, float* node_mass, float* node_quad, uint64_t capacity,
                        uint64_t* tree_records) {
    BHWork& w = s->bh;
    const uint64_t n = s->n_al;
    uint32_t* ctr = (uint32_t*)s->h_err + kHostCounters;  // pinned, owned by the system
    gs_status st = read_back(s, ctr, w.counters, kCtrCount * sizeof(uint32_t));
    if (st != GS_OK) return st;
    const uint64_t nv = ctr[kCtrValid];
    const uint64_t T = nv + ctr[kCtrInternal];
    if (tree_records) *tree_records = T;
    if (keys || sorted_src) {
        uint32_t* hk = new uint32_t[2 * n];
        uint32_t* hi = hk + n;
        GS_CUDA(cudaMemcpyAsync(hk, w.keys[w.final_keys], n * 4, cudaMemcpyDeviceToHost, s->stream));
        st = read_back(s, hi, w.idx[w.final_keys], n * 4);
        if (st == GS_ERR_TIMEOUT) return st;
        if (st == GS_OK) {
            for (uint64_t q = 0; q < n; ++q) {
                if (keys && hi[q] < n) keys[hi[q]] = q < nv ? hk[q] : kKeyRemoved;
                if (sorted_src) sorted_src[q] = q < nv ? hi[q] : (uint32_t)n;
            }
        }
        delete[] hk;
        if (st != GS_OK) return st;
    }
    const uint64_t m = T < capacity ? T : capacity;
    if (m && (node_radius || node_pos || node_mass)) {
        float4* hr = new float4[m];
        st = read_back(s, hr, w.rec, m * sizeof(float4));
        if (st == GS_ERR_TIMEOUT) return st;
        if (st == GS_OK) {
            for (uint64_t q = 0; q < m; ++q) {
                if (node_pos) {
                    node_pos[2 * q] = hr[q].x;
                    node_pos[2 * q + 1] = hr[q].y;
                }
                if (node_mass) node_mass[q] = hr[q].z;
                if (node_radius) node_radius[q] = hr[q].w;
            }
        }
        delete[] hr;
        if (st != GS_OK) return st;
    }
    if (m && node_skip) {
        st = read_back(s, node_skip, w.skip, m * sizeof(uint32_t));
        if (st != GS_OK) return st;
    }
    if (m && node_quad) {
        if (!w.quad) {
            std::memset(node_quad, 0, 3 * m * sizeof(float));
        } else {
            float4* hq = new float4[m];
            uint32_t* hs = new uint32_t[m];
            GS_CUDA(cudaMemcpyAsync(hq, w.quad, m * sizeof(float4), cudaMemcpyDeviceToHost, s->stream));
            st = read_back(s, hs, w.skip, m * sizeof(uint32_t));
            if (st == GS_ERR_TIMEOUT) return st;
            if (st == GS_OK)
                for (uint64_t q = 0; q < m; ++q) {  // a particle leaf has no spread: zero moments
                    const bool leaf = hs[q] == 1u;
                    node_quad[3 * q] = leaf ? 0.0f : hq[q].x;
                    node_quad[3 * q + 1] = leaf ? 0.0f : hq[q].y;
                    node_quad[3 * q + 2] = leaf ? 0.0f : hq[q].z;
                }
            delete[] hq;
            delete[] hs;
            if (st != GS_OK) return st;
        }
    }
    return GS_OK;
}

gs_status bh_read_counts(gs_sim* s, uint64_t* nv, uint64_t* internal, uint64_t* inter, uint64_t* visits,
                         uint64_t* nodes) {
    uint32_t* ctr = (uint32_t*)s->h_err + kHostCounters;
    gs_status st = read_back(s, ctr, s->bh.counters, kCtrCount * sizeof(uint32_t));
    if (st != GS_OK) return st;
    *nv = ctr[kCtrValid];
    *internal = ctr[kCtrInternal];
    unsigned long long c[3];
    memcpy(c, ctr + kCtrStat, sizeof c);
    *inter = c[0];
    *visits = c[1];
    *nodes = c[2];
    return GS_OK;
}

void bh_set_final_keys(gs_sim* s) { s->bh.final_keys = s->bh.passes & 1; }

// ------------------------------------------------------------------------------------
// Batched stages: one launch per stage covers every Barnes-Hut system of a plan.  Block
// b of a launch belongs to the system whose range of the stage's block table holds b,
// and runs the same body as a plain launch with its index inside that system.  The
// force stage is persistent: resident blocks take the next block index from a counter,
// largest systems first.
// ------------------------------------------------------------------------------------
namespace {

__global__ void __launch_bounds__(256) kb_clear(BatchArgs a, uint32_t* __restrict__ work) {
    const BatchBlock bb = batch_block(a, blockIdx.x);
    if (blockIdx.x == 0 && threadIdx.x < 4) work[threadIdx.x] = 0u;
    uint32_t* z = bb.d->zero_base;
    const uint32_t nw = bb.d->zero_words;
    for (uint32_t i = bb.blk.id * 256 + threadIdx.x; i < nw; i += bb.blk.count * 256) z[i] = 0u;
}

__global__ void __launch_bounds__(kBBoxThreads) kb_bbox(BatchArgs a) {
    pdl_enter();
    const BatchBlock bb = batch_block(a, blockIdx.x);
    const SysDesc& d = *bb.d;
    bbox_body(bb.blk, d.pos[bb.in], d.n_al, d.bbox_part, d.counters + kCtrBBox, d.params, d.depth);
}

__global__ void __launch_bounds__(kKeyThreads) kb_keygen(BatchArgs a) {
    pdl_enter();
    const BatchBlock bb = batch_block(a, blockIdx.x);
    const SysDesc& d = *bb.d;
    // the output set's extent, gathered by this step's traversal kernel (kb_bbox derived the
    // box from the positions themselves)
    if (d.ext && bb.blk.id == 0 && threadIdx.x < 4) d.ext[4 * bb.out + threadIdx.x] = 0xFFFFFFFFu;
    keygen_body(bb.blk, d.bbox, d.params, d.pos[bb.in], d.mass[bb.in], d.pos[bb.out], d.mass[bb.out], d.n_al,
                d.keys[0], d.hist, d.passes, d.counters + kCtrValid, d.quad ? d.counters + kCtrMaxMass : nullptr);
}

// the exact moment sums of a quadrupole-mode member (all fields null otherwise)
__device__ __forceinline__ MomIn batch_mom_in(const SysDesc& d) {
    MomIn mi{};
    if (d.quad) {
        mi.bp = d.params;
        mi.mmax = d.counters + kCtrMaxMass;
        mi.bbox = d.bbox;
        mi.qv = d.mom_q;
        mi.prefix = d.mom_prefix;
        mi.stride = (size_t)d.n_al + 1;
        mi.agg = d.mom_agg;
        mi.nend = d.mom_nend;
    }
    return mi;
}

template <bool IDENTITY, int KPT, int LB>
__global__ void __launch_bounds__(kSortThreads) kb_sort_pass(BatchArgs a, int ps) {
    pdl_enter();
    const BatchBlock bb = batch_block(a, blockIdx.x);
    const SysDesc& d = *bb.d;
    const int x = ps & 1, y = x ^ 1;
    sort_pass_body<IDENTITY, KPT, LB>(d.keys[x], IDENTITY ? nullptr : d.idx[x], d.keys[y], d.idx[y], d.n_al, 8 * ps,
                             d.hist + 256 * ps, d.sort_status + (size_t)ps * d.sort_tiles * 256,
                             d.counters + kCtrSort + ps, d.err);
}

template <int R>
__global__ void __launch_bounds__(kScanThreads) kb_meta_scan(BatchArgs a) {
    pdl_enter();
    const BatchBlock bb = batch_block(a, blockIdx.x);
    const SysDesc& d = *bb.d;
    meta_scan_body<R>(d.keys[d.passes & 1], d.n_al + 1, d.counters + kCtrValid, d.depth, d.E, d.scan_status,
                   d.counters + kCtrScan, d.counters + kCtrInternal, d.err);
}

__global__ void __launch_bounds__(kMomThreads) kb_mom_tiles(BatchArgs a) {
    pdl_enter();
    const BatchBlock bb = batch_block(a, blockIdx.x);
    const SysDesc& d = *bb.d;
    const MomIn mi = batch_mom_in(d);
    if (mi.prefix) mom_tiles_body(bb.blk.id, d.counters[kCtrValid], mi);
}
__global__ void __launch_bounds__(kMomThreads, 2) kb_mom_scan(BatchArgs a) {
    pdl_enter();
    const BatchBlock bb = batch_block(a, blockIdx.x);
    const SysDesc& d = *bb.d;
    const MomIn mi = batch_mom_in(d);
    if (mi.prefix) mom_scan_body(bb.blk.id, d.n_al + 1, d.counters[kCtrValid], mi);
}

__global__ void __launch_bounds__(256) kb_records(BatchArgs a, uint2* __restrict__ heavy_list,
                                                  uint32_t* __restrict__ heavy_count) {
    pdl_enter();
    const BatchBlock bb = batch_block(a, blockIdx.x);
    const SysDesc& d = *bb.d;
    const int f = d.passes & 1;
    records_body(bb.blk, d.keys[f], d.idx[f], d.E, d.counters + kCtrValid, d.depth, d.pos[bb.in], d.mass[bb.in],
                 d.rec, d.skip, d.node_slot, d.cap, d.n_al, d.err, batch_mom_in(d));
    if (heavy_list && d.heavy)  // the costly groups of every large member with the relative criterion
        heavy_list_body(bb.blk, d.idx[f], d.counters + kCtrValid, d.amag, d.n_al, d.heavy, heavy_list, heavy_count,
                        (uint32_t)(bb.d - a.descs));
}

__global__ void __launch_bounds__(256) kb_nodes(BatchArgs a) {
    pdl_enter();
    const BatchBlock bb = batch_block(a, blockIdx.x);
    const SysDesc& d = *bb.d;
    nodes_body(bb.blk, d.keys[d.passes & 1], d.E, d.counters + kCtrValid, d.depth, d.params, d.node_slot, d.rec,
               d.skip, d.kids, d.nodeinfo, d.counters + kCtrLevel, d.levels, d.n_al, d.cap, d.err,
               batch_mom_in(d), d.quad, d.safe);
}

__global__ void __launch_bounds__(256) kb_mom_nodes(BatchArgs a) {
    pdl_enter();
    const BatchBlock bb = batch_block(a, blockIdx.x);
    const SysDesc& d = *bb.d;
    const MomIn mi = batch_mom_in(d);
    if (mi.prefix)
        mom_nodes_body(bb.blk, d.counters + kCtrValid, d.depth, d.params, d.node_slot, d.nodeinfo, d.rec, d.quad,
                       d.safe, d.cap, mi);
}

// level lv of every system (systems shallower than lv have nothing to do)
__global__ void __launch_bounds__(256) kb_level_sums(BatchArgs a, int lv) {
    pdl_enter();
    const BatchBlock bb = batch_block(a, blockIdx.x);
    const SysDesc& d = *bb.d;
    if (lv > d.depth) return;
    level_sums_body(bb.blk, lv, d.counters + kCtrLevel, d.levels, d.n_al, d.keys[d.passes & 1], d.depth, d.rec,
                    d.kids, d.nodeinfo, d.msum, d.safe, d.bbox, d.params);
}

__global__ void __launch_bounds__(512) kb_top_sums(BatchArgs a) {
    pdl_enter();
    const BatchBlock bb = batch_block(a, blockIdx.x);
    const SysDesc& d = *bb.d;
    top_sums_body(d.counters + kCtrLevel, d.levels, d.n_al, d.keys[d.passes & 1], d.depth, d.rec, d.kids, d.nodeinfo,
                  d.msum, d.safe, d.bbox, d.params);
}

}  // namespace

// Descriptor and per-stage block counts of one Barnes-Hut system; the counts are the
// plain path's, except that the bounding box uses no more blocks than its particles fill.
void bh_batch_desc(gs_sim* s, SysDesc& d, uint32_t blocks[kTabCount], const gs_shape& shape,
                   uint32_t force_warps) {
    const BHWork& w = s->bh;
    d.keys[0] = w.keys[0];
    d.keys[1] = w.keys[1];
    d.idx[0] = w.idx[0];
    d.idx[1] = w.idx[1];
    d.hist = w.hist;
    d.sort_status = w.sort_status;
    d.counters = w.counters;
    d.scan_status = w.scan_status;
    d.E = w.E;
    d.rec = w.rec;
    d.skip = w.skip;

    d.msum = w.msum;
    d.quad = w.quad;
    d.mom_q = w.mom_q;
    d.mom_prefix = w.mom_prefix;
    d.mom_agg = w.mom_agg;
    d.mom_nend = w.mom_nend;
    d.amag = w.amag;
    d.heavy = s->n_al >= kHeavyMinParticles ? w.heavy_flag : nullptr;  // costly groups paired
    d.ext = w.ext;
    d.alpha = s->p.relative_accuracy;
    d.floor2 = s->floor2;
    d.kids = w.kids;
    d.levels = w.levels;
    d.nodeinfo = w.nodeinfo;
    d.node_slot = w.node_slot;
    d.bbox_part = w.bbox_part;
    d.params = w.params;
    d.zero_base = (uint32_t*)w.zero_base;
    d.zero_words = (uint32_t)(w.zero_bytes / sizeof(uint32_t));
    d.cap = (uint32_t)w.cap;
    d.sort_tiles = w.sort_tiles;
    d.scan_tiles = w.scan_tiles;
    d.depth = w.depth;
    d.passes = w.passes;
    d.bbox = s->p.box_mode == GS_BOX_BOUNDING ? 1 : 0;
    d.safe = (s->p.flags & GS_FLAG_SAFE_RADIUS) ? 1 : 0;
    const uint64_t n = s->n_al;
    for (int t = 0; t < kTabCount; ++t) blocks[t] = 0;
    uint64_t cb = (d.zero_words + 1023) / 1024;
    blocks[kTabClear] = (uint32_t)(cb < 1 ? 1 : cb > 64 ? 64 : cb);
    if (d.bbox) {
        blocks[kTabBBox] = (uint32_t)bbox_blocks(n);
    }
    blocks[kTabGrid] = (uint32_t)grid_for(n, 256);
    blocks[kTabKeys] = (uint32_t)keygen_blocks(n);
    blocks[kTabSort] = sort_tiles_of(n, shape);
    blocks[kTabScan] = w.scan_tiles;
    blocks[kTabMom] = w.mom_blocks;
    blocks[kTabOne] = 1;
    const uint64_t per_block = (s->p.flags & GS_FLAG_GROUP_WALK) ? (uint64_t)force_warps * kGroupSize
                                                                   : (uint64_t)kForceWarps * 32;
    blocks[kTabForce] = (uint32_t)((n + per_block - 1) / per_block);
}

namespace {
template <int KPT>
auto batch_sort_pass_kernel_kpt(bool identity, uint32_t lb) {
    switch (lb) {
        case 8: return identity ? kb_sort_pass<true, KPT, 8> : kb_sort_pass<false, KPT, 8>;
        case 16: return identity ? kb_sort_pass<true, KPT, 16> : kb_sort_pass<false, KPT, 16>;
        default: return identity ? kb_sort_pass<true, KPT, 32> : kb_sort_pass<false, KPT, 32>;
    }
}
auto batch_sort_pass_kernel(bool identity, const gs_shape& sh) {
    return sh.sort_keys_per_thread == 8 ? batch_sort_pass_kernel_kpt<8>(identity, sh.sort_lookback)
                                        : batch_sort_pass_kernel_kpt<16>(identity, sh.sort_lookback);
}
}  // namespace

static BatchForceLaunch batch_force(const BatchPlan& p, uint32_t step, cudaStream_t st) {
    BatchForceLaunch b;
    b.st = st;
    b.descs = p.d_descs;
    b.first = p.d_tab[kTabForce];
    b.nsys = p.n_bh;
    b.step = step;
    b.group = p.group;
    b.quad = p.quad;
    b.count = p.count;
    b.shape = p.shape;
    if (p.d_heavy) {
        b.heavy_list = p.d_heavy;
        b.heavy_work = p.d_work + 2;
    }
    return b;
}

int bh_batch_force_grid(const BatchPlan& p) {
    BatchForceLaunch b = batch_force(p, 0, nullptr);
    int grid = 0;
    const cudaError_t e = (p.exact ? batch_force_launch_exact : batch_force_launch_fast)(b, &grid);
    return e == cudaSuccess && grid > 0 ? grid : 152;
}

cudaError_t bh_batch_step(const BatchPlan& p, uint32_t step, cudaStream_t st, bool estimate, const StepFork& f) {
    if (!p.n_bh) return cudaSuccess;
    auto args = [&](int tab) { return BatchArgs{p.d_descs, p.d_tab[tab], p.n_bh, step}; };
    // the clear follows whatever the stream did before; every later stage overlaps its
    // launch with the stage before it (programmatic dependent launch)
    GS_TRY_LAUNCH(launch(false, kb_clear, (int)p.total[kTabClear], 256, st, args(kTabClear), p.d_work));
    if (p.bbox) GS_TRY_LAUNCH(launch(true, kb_bbox, (int)p.total[kTabBBox], kBBoxThreads, st, args(kTabBBox)));
    GS_TRY_LAUNCH(launch(true, kb_keygen, (int)p.total[kTabKeys], kKeyThreads, st, args(kTabKeys)));
    for (int ps = 0; ps < p.passes; ++ps)
        GS_TRY_LAUNCH(launch(true, batch_sort_pass_kernel(ps == 0, p.shape), (int)p.total[kTabSort], kSortThreads, st,
                             args(kTabSort), ps));
    {
        const uint32_t lb = p.shape.scan_lookback;
        GS_TRY_LAUNCH(launch(true, lb >= 128 ? kb_meta_scan<4> : lb >= 64 ? kb_meta_scan<2> : kb_meta_scan<1>,
                             (int)p.total[kTabScan], kScanThreads, st, args(kTabScan)));
    }
    GS_TRY_LAUNCH(launch(true, kb_records, (int)p.total[kTabGrid], 256, st, args(kTabGrid), p.d_heavy,
                         p.d_heavy ? p.d_work + 2 : nullptr));
    // the moment prefix beside the node layout, as in bh_step
    const bool fork = p.quad && f.side;
    cudaStream_t mst = fork ? f.side : st;
    if (fork) {
        GS_TRY_LAUNCH(cudaEventRecord(f.fork, st));
        GS_TRY_LAUNCH(cudaStreamWaitEvent(mst, f.fork, 0));
    }
    if (p.quad) {
        GS_TRY_LAUNCH(launch(!fork, kb_mom_tiles, (int)p.total[kTabMom], kMomThreads, mst, args(kTabMom)));
        GS_TRY_LAUNCH(launch(true, kb_mom_scan, (int)p.total[kTabMom], kMomThreads, mst, args(kTabMom)));
    }
    GS_TRY_LAUNCH(launch(true, kb_nodes, (int)p.total[kTabGrid], 256, st, args(kTabGrid)));
    if (fork) {
        GS_TRY_LAUNCH(cudaEventRecord(f.join, mst));
        GS_TRY_LAUNCH(cudaStreamWaitEvent(st, f.join, 0));
    }
    if (p.quad) GS_TRY_LAUNCH(launch(!fork, kb_mom_nodes, (int)p.total[kTabGrid], 256, st, args(kTabGrid)));
    if (!p.quad) {  // monopole moments level by level; the quadrupole mode has them from kb_nodes
        for (int lv = p.depth; lv > kLevelTop; --lv)
            GS_TRY_LAUNCH(launch(true, kb_level_sums, (int)p.total[kTabGrid], 256, st, args(kTabGrid), lv));
        GS_TRY_LAUNCH(launch(true, kb_top_sums, (int)p.total[kTabOne], 512, st, args(kTabOne)));
    }
    const int fg = p.force_grid < (int)p.total[kTabForce] ? p.force_grid : (int)p.total[kTabForce];
    BatchForceLaunch b = batch_force(p, step, st);
    b.grid = fg;
    auto run = p.exact ? batch_force_launch_exact : batch_force_launch_fast;
    if (estimate && p.group && p.quad) {  // |a| of the groups that have none (members that just joined or were reset)
        BatchForceLaunch e = b;
        e.estimate = true;
        e.work = p.d_work + 1;
        GS_TRY_LAUNCH(run(e, nullptr));
    }
    b.work = p.d_work;
    GS_TRY_LAUNCH(run(b, nullptr));
    return cudaGetLastError();
}

}  // namespace gsim
