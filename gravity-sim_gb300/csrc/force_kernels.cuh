// force_kernels.cuh -- the Barnes-Hut traversal kernels with the integrator fused into
// their epilogue (ForceShader.comp:78-152 and the accurate group walk), plain and batched,
// templated on the math mode and on the launch shape (gs_shape: warps per block, list
// caps).  force_fast.cu and force_exact.cu instantiate them for FAST and REFERENCE math.
#pragma once
#include "bh_common.cuh"

namespace gsim {
namespace {

// ------------------------------------------------------------------------------------
// traversal + integrator (ForceShader.comp:78-152)
// ------------------------------------------------------------------------------------

template <bool EXACT, bool COUNT>
__device__ __forceinline__ void force_body(Blk blk, const uint32_t* __restrict__ sidx,
                                           const uint32_t* __restrict__ counts, const float4* __restrict__ rec,
                                           const uint32_t* __restrict__ skip, const float2* __restrict__ pos_in,
                                           const float2* __restrict__ vel_in, float2* __restrict__ pos_out,
                                           float2* __restrict__ vel_out, float2* __restrict__ acc_rec, uint32_t n_al,
                                           float eps2, float theta2, float k, float hdt, uint32_t cap,
                                           unsigned long long* __restrict__ stat, uint32_t* __restrict__ ext) {
    __shared__ float4 wrec[kForceWarps][32];
    __shared__ uint32_t wskip[kForceWarps][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t group = blk.id * kForceWarps + warp;
    const uint32_t nv = counts[0];
    const uint32_t T = min(nv + counts[1], cap);  // preorder records
    if (group * 32 >= nv) return;       // no particle in this warp: nothing to write
    const uint32_t s = group * 32 + lane;
    const uint32_t i = s < nv ? sidx[s] : 0u;
    const bool valid = s < nv && i < n_al;  // i < n_al unless the sort failed (error flag set)
    const float2 p = valid ? pos_in[i] : make_float2(0.0f, 0.0f);
    float ax = 0.0f, ay = 0.0f;
    unsigned long long n_acc = 0, n_vis = 0;
    uint32_t base = 0, ind = 0;
    wrec[warp][lane] = rec[lane];
    wskip[warp][lane] = skip[lane];
    __syncwarp();
    while (ind < T) {
        if (ind - base >= 32u) {  // warp-uniform: reload the 32-record window
            base = ind & ~31u;
            __syncwarp();
            wrec[warp][lane] = rec[base + lane];
            wskip[warp][lane] = skip[base + lane];
            __syncwarp();
        }
        const float4 q = wrec[warp][ind - base];
        const float dx = q.x - p.x, dy = q.y - p.y;
        const float d2 = fmaf(dx, dx, fmaf(dy, dy, eps2));
        const bool ok = !valid || q.w <= d2 * theta2;
        if (COUNT) ++n_vis;
        if (__all_sync(0xffffffffu, ok)) {
            const float r = EXACT ? __fdiv_rn(1.0f, __fsqrt_rn(d2)) : rsqrtf(d2);
            const float sc = ((q.z * r) * r) * r;
            ax = fmaf(dx, sc, ax);
            ay = fmaf(dy, sc, ay);
            if (COUNT) n_acc += valid;
            ind += max(wskip[warp][ind - base], 1u);  // >= 1: the walk always advances
        } else {
            ++ind;
        }
    }
    if (COUNT) {
        for (int o = 16; o; o >>= 1) n_acc += __shfl_xor_sync(0xffffffffu, n_acc, o);
        if (lane == 0) {
            atomicAdd(&stat[0], n_acc);
            atomicAdd(&stat[1], n_vis);
        }
    }
    float2 np = make_float2(0.0f, 0.0f);
    if (valid) {
        if (acc_rec) acc_rec[i] = make_float2(ax, ay);
        const float2 v = vel_in[i];
        const float nvx = fmaf(ax, k, v.x), nvy = fmaf(ay, k, v.y);  // ForceShader.comp:145-146
        np = make_float2(fmaf(v.x + nvx, hdt, p.x), fmaf(v.y + nvy, hdt, p.y));
        pos_out[i] = np;
        vel_out[i] = make_float2(nvx, nvy);
    }
    if (ext)  // bounding-box mode: the next step's box
        ext_add(ext, valid ? np.x : INFINITY, valid ? np.x : -INFINITY, valid ? np.y : INFINITY,
                valid ? np.y : -INFINITY);
}

template <bool EXACT, bool COUNT>
__global__ void __launch_bounds__(kForceWarps * 32)
k_force(const uint32_t* __restrict__ sidx, const uint32_t* __restrict__ counts, const float4* __restrict__ rec,
        const uint32_t* __restrict__ skip, const float2* __restrict__ pos_in, const float2* __restrict__ vel_in,
        float2* __restrict__ pos_out, float2* __restrict__ vel_out, float2* __restrict__ acc_rec, uint32_t n_al,
        float eps2, float theta2, float k, float hdt, uint32_t cap, unsigned long long* __restrict__ stat,
        uint32_t* __restrict__ ext) {
    pdl_enter();
    force_body<EXACT, COUNT>(grid_blk(), sidx, counts, rec, skip, pos_in, vel_in, pos_out, vel_out, acc_rec, n_al,
                             eps2, theta2, k, hdt, cap, stat, ext);
}

// ------------------------------------------------------------------------------------
// accurate-mode traversal (no counterpart in the reference): the 64 particles of 64
// consecutive sorted slots share one walk, run by one warp (two particles per lane); 32
// records are tested at once (one per lane) against the bounding boxes of the group;
// accepted nodes and runs of particle leaves are collected and every lane then sums them
// for its two particles with packed f32x2 instructions (quadrupole term for nodes).
// ------------------------------------------------------------------------------------
// Records still to test.  Pops take the top 32 and push at most four internal children
// each, one level deeper, so the stack holds at most one block of <= 128 entries per level
// and blocks of strictly increasing level: <= 96 * D + 128 = 1568 for D = 15.  Overflow
// is still checked and reported.
constexpr int kStackCap = 1568;
static_assert(kStackCap >= 96 * (kBBoxMaxBits > kFixedDepth ? kBBoxMaxBits : kFixedDepth) + 128, "walk stack bound");
// Accepted nodes and runs of particle leaves collected between evaluations: 160 / 128
// (long lists) or 96 / 64 (short lists, gs_shape.force_short_lists); a pop adds at most
// 32 nodes and 64 runs.

// 1/sqrt: correctly rounded (REFERENCE math) or the hardware approximation (FAST math;
// d2 >= eps^2 > 0 is never subnormal, so the flush-to-zero form loses nothing)
__device__ __forceinline__ float rsqrt_fast(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

template <bool EXACT>
__device__ __forceinline__ float inv_sqrt(float d2) {
    return EXACT ? __fdiv_rn(1.0f, __fsqrt_rn(d2)) : rsqrt_fast(d2);
}

// Evaluation order.  Each particle sums the accepted nodes and the particle leaves of its
// walk separately, each in walk order, into a node and a leaf accumulator; its
// acceleration is node + leaf.  How the warp batches its evaluations therefore does not
// change a bit of the result.
template <int NODE, int ITEM>
struct GroupSmem {
    static constexpr int kNode = NODE, kItem = ITEM;
    static_assert(NODE >= 64 && ITEM >= 64 && ITEM % 32 == 0, "a pop adds <= 32 nodes and <= 64 leaf runs");
    uint32_t stack[kStackCap];
    uint32_t node[NODE];          // accepted node records
    uint32_t it_start[ITEM];      // runs of particle leaves: first record
    uint32_t it_count[ITEM];      // record count
    uint32_t off[ITEM];           // exclusive record offsets of the runs
    float cx[32], cy[32], cm[32];     // one chunk of gathered records: centre of mass (or particle), mass
    float qxx[32], qxy[32], qyy[32], mt[32];  // node terms 7.5 S and -1.5 tr(S) of node records
};

// One record (x, y, m) on the lane's two particles (P = their x, Q = their y):
// d = (x, y) - p, d2 = dx^2 + dy^2 + eps^2, a += d * (((m r) r) r) with r = 1/sqrt(d2),
// the CPU restatement's pair_scale sequence, two particles at once.
template <bool EXACT>
__device__ __forceinline__ void monopole_x2(float x, float y, float m, float2 P, float2 Q, float2 E2, float2& acx,
                                            float2& acy) {
    const float2 dx = sub2(make_float2(x, x), P), dy = sub2(make_float2(y, y), Q);
    const float2 d2 = fma2(dx, dx, fma2(dy, dy, E2));
    const float2 r = make_float2(inv_sqrt<EXACT>(d2.x), inv_sqrt<EXACT>(d2.y));
    const float2 sc = mul2(mul2(mul2(make_float2(m, m), r), r), r);
    acx = fma2(dx, sc, acx);
    acy = fma2(dy, sc, acy);
}

// One node with second moments on the lane's two particles.  The monopole and
// quadrupole terms of the softened potential,
//   a = d (m r^3 - 1.5 tr(S) r^5 + 7.5 (d.S.d) r^7) - 3 r^5 S d,   r = 1/sqrt(d2),
// are evaluated as r^3 (d (m + r^2 (mt + r^2 u)) - 0.4 r^2 S'' d) with the node terms
// S'' = 7.5 S and mt = -1.5 tr(S) formed once per node (eval_nodes): 21 operations per
// particle instead of 23, the CPU restatement's sequence (quad_accumulate).
template <bool EXACT>
__device__ __forceinline__ void quadrupole_x2(float x, float y, float m, float qxx, float qxy, float qyy, float mt,
                                              float2 P, float2 Q, float2 E2, float2& acx, float2& acy) {
    const float2 dx = sub2(make_float2(x, x), P), dy = sub2(make_float2(y, y), Q);
    const float2 d2 = fma2(dx, dx, fma2(dy, dy, E2));
    const float2 r = make_float2(inv_sqrt<EXACT>(d2.x), inv_sqrt<EXACT>(d2.y));
    const float2 r2 = mul2(r, r);
    const float2 r3 = mul2(r2, r);
    const float2 Sxx = make_float2(qxx, qxx), Sxy = make_float2(qxy, qxy), Syy = make_float2(qyy, qyy);
    const float2 srx = fma2(Sxx, dx, mul2(Sxy, dy));
    const float2 sry = fma2(Sxy, dx, mul2(Syy, dy));
    const float2 u = fma2(dx, srx, mul2(dy, sry));
    const float2 t = fma2(fma2(u, r2, make_float2(mt, mt)), r2, make_float2(m, m));
    const float2 k = mul2(make_float2(-0.4f, -0.4f), r2);
    const float2 ix = fma2(srx, k, mul2(dx, t));
    const float2 iy = fma2(sry, k, mul2(dy, t));
    acx = fma2(r3, ix, acx);
    acy = fma2(r3, iy, acy);
}

// Sum the count accepted nodes (quadrupole term with QUAD) for the lane's two particles,
// 32 at a time: lane l loads node l of the next chunk while the current one is summed.
template <bool EXACT, bool QUAD, class SM>
__device__ __forceinline__ void eval_nodes(SM& g, uint32_t count, const float4* __restrict__ rec,
                                           const float4* __restrict__ quad, float2 P, float2 Q, float2 E2,
                                           float2& acx, float2& acy, int lane) {
    if (!count) return;
    float4 q = make_float4(0.0f, 0.0f, 0.0f, 0.0f), qq = q;
    if ((uint32_t)lane < count) {
        const uint32_t r = g.node[lane];
        q = __ldg(&rec[r]);
        if (QUAD) qq = __ldg(&quad[r]);
    }
    for (uint32_t f0 = 0; f0 < count; f0 += 32) {
        const uint32_t m = min(count - f0, 32u);
        g.cx[lane] = q.x;
        g.cy[lane] = q.y;
        g.cm[lane] = q.z;
        if (QUAD) {
            g.qxx[lane] = 7.5f * qq.x;
            g.qxy[lane] = 7.5f * qq.y;
            g.qyy[lane] = 7.5f * qq.z;
            g.mt[lane] = -1.5f * (qq.x + qq.z);
        }
        __syncwarp();
        const uint32_t fn = f0 + 32 + lane;
        if (fn < count) {
            const uint32_t r = g.node[fn];
            q = __ldg(&rec[r]);
            if (QUAD) qq = __ldg(&quad[r]);
        }
#pragma unroll 4
        for (uint32_t j = 0; j < m; ++j) {
            if (QUAD)
                quadrupole_x2<EXACT>(g.cx[j], g.cy[j], g.cm[j], g.qxx[j], g.qxy[j], g.qyy[j], g.mt[j], P, Q, E2, acx,
                                     acy);
            else
                monopole_x2<EXACT>(g.cx[j], g.cy[j], g.cm[j], P, Q, E2, acx, acy);
        }
        __syncwarp();
    }
}

// Record f of the leaf runs (last run with off <= f).
template <class SM>
__device__ __forceinline__ float4 gather_leaf(const SM& g, uint32_t n_items, uint32_t f,
                                              const float4* __restrict__ rec) {
    uint32_t lo = 0, hi = n_items - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (g.off[mid] <= f) lo = mid;
        else hi = mid - 1;
    }
    return __ldg(&rec[g.it_start[lo] + (f - g.off[lo])]);
}

// Sum the particle leaves of the n_items runs as monopoles, 32 records at a time.
template <bool EXACT, class SM>
__device__ __forceinline__ void eval_leaves(SM& g, uint32_t n_items, const float4* __restrict__ rec,
                                            float2 P, float2 Q, float2 E2, float2& acx, float2& acy, int lane) {
    if (!n_items) return;
    // exclusive record offsets of all runs: lane l owns runs [4l, 4l + 4)
    uint32_t c4[SM::kItem / 32], sum = 0;
#pragma unroll
    for (int t = 0; t < SM::kItem / 32; ++t) {
        const uint32_t it = lane * (SM::kItem / 32) + t;
        c4[t] = it < n_items ? g.it_count[it] : 0u;
        sum += c4[t];
    }
    uint32_t x = sum;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, x, 31);
    uint32_t run = x - sum;
#pragma unroll
    for (int t = 0; t < SM::kItem / 32; ++t) {
        g.off[lane * (SM::kItem / 32) + t] = run;
        run += c4[t];
    }
    __syncwarp();
    float4 q = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if ((uint32_t)lane < total) q = gather_leaf(g, n_items, lane, rec);
    for (uint32_t f0 = 0; f0 < total; f0 += 32) {
        const uint32_t m = min(total - f0, 32u);
        g.cx[lane] = q.x;
        g.cy[lane] = q.y;
        g.cm[lane] = q.z;
        __syncwarp();
        const uint32_t fn = f0 + 32 + lane;
        if (fn < total) q = gather_leaf(g, n_items, fn, rec);
#pragma unroll 4
        for (uint32_t j = 0; j < m; ++j) monopole_x2<EXACT>(g.cx[j], g.cy[j], g.cm[j], P, Q, E2, acx, acy);
        __syncwarp();
    }
}

// The end of a group's walk: |a| for the relative criterion, then (main pass) the
// integrator and the new positions' extent.  ax, ay: node + leaf per particle (.x particle
// 0, .y particle 1).  Every lane of the warp must call it.
template <bool ESTIMATE>
__device__ __forceinline__ void group_finish(float2 ax, float2 ay, bool v0, bool v1, uint32_t i0, uint32_t i1,
                                             float2 p0, float2 p1, const float2* __restrict__ vel_in,
                                             float2* __restrict__ pos_out, float2* __restrict__ vel_out,
                                             float2* __restrict__ acc_rec, float k, float hdt,
                                             float* __restrict__ amag, uint32_t* __restrict__ ext) {
    if (amag) {
        if (v0) amag[i0] = __fsqrt_rn(fmaf(ax.x, ax.x, ay.x * ay.x));
        if (v1) amag[i1] = __fsqrt_rn(fmaf(ax.y, ax.y, ay.y * ay.y));
    }
    if (ESTIMATE) return;
    float mnx = INFINITY, mxx = -INFINITY, mny = INFINITY, mxy = -INFINITY;  // of the new positions
    if (v0) {
        if (acc_rec) acc_rec[i0] = make_float2(ax.x, ay.x);
        const float2 v = vel_in[i0];
        const float nvx = fmaf(ax.x, k, v.x), nvy = fmaf(ay.x, k, v.y);
        const float2 np = make_float2(fmaf(v.x + nvx, hdt, p0.x), fmaf(v.y + nvy, hdt, p0.y));
        pos_out[i0] = np;
        vel_out[i0] = make_float2(nvx, nvy);
        mnx = fminf(mnx, np.x);
        mxx = fmaxf(mxx, np.x);
        mny = fminf(mny, np.y);
        mxy = fmaxf(mxy, np.y);
    }
    if (v1) {
        if (acc_rec) acc_rec[i1] = make_float2(ax.y, ay.y);
        const float2 v = vel_in[i1];
        const float nvx = fmaf(ax.y, k, v.x), nvy = fmaf(ay.y, k, v.y);
        const float2 np = make_float2(fmaf(v.x + nvx, hdt, p1.x), fmaf(v.y + nvy, hdt, p1.y));
        pos_out[i1] = np;
        vel_out[i1] = make_float2(nvx, nvy);
        mnx = fminf(mnx, np.x);
        mxx = fmaxf(mxx, np.x);
        mny = fminf(mny, np.y);
        mxy = fmaxf(mxy, np.y);
    }
    if (ext) ext_add(ext, mnx, mxx, mny, mxy);  // bounding-box mode: the next step's box
}

// The outcome of testing one stacked record (an internal node) against a group's boxes:
// accepted (nn = 1), or opened into at most two runs of particle leaves {a, c} and at most
// four internal children to push, in Morton order.
struct RecTest {
    uint32_t nn, nl, a0, c0, a1, c1, npu;
    uint32_t pu[4];
};

__device__ __forceinline__ void test_record(uint32_t n, const float4* __restrict__ rec, const uint4* __restrict__ kids,
                                            const float* bx0, const float* bx1, const float* by0, const float* by1,
                                            float eps2, bool relative, float tol2, float floor2, float theta2,
                                            RecTest& r) {
    const float4 q = rec[n];
    const uint4 kd = kids[n];
    float d2 = INFINITY;  // nearest sub-box; an empty one gives +inf
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        const float ex = fmaxf(fmaxf(bx0[b] - q.x, q.x - bx1[b]), 0.0f);
        const float ey = fmaxf(fmaxf(by0[b] - q.y, q.y - by1[b]), 0.0f);
        d2 = fminf(d2, fmaf(ex, ex, fmaf(ey, ey, eps2)));
    }
    bool accept;
    if (relative) {  // m^2 R^3 <= tol^2 D^5 with R <= D (R: squared opening radius), or theta
        const float lhs = (q.z * q.z) * ((q.w * q.w) * q.w);
        const float d4 = d2 * d2;
        accept = (q.w <= d2 && lhs <= tol2 * ((d4 * d4) * d2)) || q.w <= d2 * floor2;
    } else {
        accept = q.w <= d2 * theta2;
    }
    if (accept) {
        r.nn = 1;
    } else if (kd.x == kKidFinest) {
        r.a0 = kd.y;
        r.c0 = kd.z;
        r.nl = 1;
    } else {
        const uint32_t kk[4] = {kd.x, kd.y, kd.z, kd.w};
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const uint32_t c = kk[t];
            if (c == kKidNone) continue;
            if (c & kKidLeaf) {
                const uint32_t l = c & ~kKidLeaf;
                if (r.nl == 1 && r.a0 + r.c0 == l) ++r.c0;        // extend the open run
                else if (r.nl == 2 && r.a1 + r.c1 == l) ++r.c1;
                else if (r.nl == 0) { r.a0 = l; r.c0 = 1; r.nl = 1; }
                else { r.a1 = l; r.c1 = 1; r.nl = 2; }
            } else {
                if (r.npu == 0) r.pu[0] = c;
                else if (r.npu == 1) r.pu[1] = c;
                else if (r.npu == 2) r.pu[2] = c;
                else r.pu[3] = c;
                ++r.npu;
            }
        }
    }
}

// Sub-boxes of a group: the particles are split by their cell at the coarsest level where
// the first and last keys of the group differ, so a group that crosses a coarse Morton
// boundary is not given one box spanning the empty space between its ends.  Each box is
// the bounding box of its particles (+inf..-inf when empty).  Every lane must call it.
__device__ __forceinline__ void group_boxes(const uint32_t* __restrict__ skey, uint32_t g0, uint32_t nv, uint32_t s0,
                                            uint32_t s1, bool v0, bool v1, float2 p0, float2 p1, float* bx0,
                                            float* bx1, float* by0, float* by1) {
    const uint32_t kf = skey[g0], kl = skey[min(g0 + kGroupSize - 1, nv - 1)];
    const int shift = kf == kl ? -1 : ((31 - __clz(kf ^ kl)) & ~1);
    const int box0 = !v0 ? -1 : (shift < 0 ? 0 : (int)((skey[s0] >> shift) & 3u));
    const int box1 = !v1 ? -1 : (shift < 0 ? 0 : (int)((skey[s1] >> shift) & 3u));
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        const bool in0 = box0 == b, in1 = box1 == b;
        float x0 = fminf(in0 ? p0.x : INFINITY, in1 ? p1.x : INFINITY);
        float x1 = fmaxf(in0 ? p0.x : -INFINITY, in1 ? p1.x : -INFINITY);
        float y0 = fminf(in0 ? p0.y : INFINITY, in1 ? p1.y : INFINITY);
        float y1 = fmaxf(in0 ? p0.y : -INFINITY, in1 ? p1.y : -INFINITY);
        for (int o = 16; o; o >>= 1) {
            x0 = fminf(x0, __shfl_xor_sync(0xffffffffu, x0, o));
            x1 = fmaxf(x1, __shfl_xor_sync(0xffffffffu, x1, o));
            y0 = fminf(y0, __shfl_xor_sync(0xffffffffu, y0, o));
            y1 = fmaxf(y1, __shfl_xor_sync(0xffffffffu, y1, o));
        }
        bx0[b] = x0;
        bx1[b] = x1;
        by0[b] = y0;
        by1[b] = y1;
    }
}

// ESTIMATE: the |a| estimate pass of the relative criterion.  A group whose particles all
// have a previous |a| returns at once; any other group walks with the theta test and
// writes only the |a| of its particles (no integration), which the following normal pass
// then opens nodes by.
template <bool EXACT, bool QUAD, bool COUNT, bool ESTIMATE, int WARPS, class SM>
__device__ __forceinline__ void force_group_body(
    Blk blk, SM& g, const uint32_t* __restrict__ sidx, const uint32_t* __restrict__ skey,
    const uint32_t* __restrict__ counts, const float4* __restrict__ rec, const uint32_t* __restrict__ skip,
    const float4* __restrict__ quad, const uint4* __restrict__ kids, const float2* __restrict__ pos_in,
    const float2* __restrict__ vel_in, float2* __restrict__ pos_out, float2* __restrict__ vel_out,
    float2* __restrict__ acc_rec, uint32_t n_al, float eps2, float theta2, float k, float hdt, uint32_t cap,
    unsigned long long* __restrict__ stat, int* __restrict__ err, float* __restrict__ amag, float alpha,
    float floor2, uint32_t* __restrict__ ext, const uint8_t* __restrict__ heavy) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t group = blk.id * WARPS + warp;
    const uint32_t nv = counts[0];
    const uint32_t T = min(nv + counts[1], cap);
    const uint32_t g0 = group * kGroupSize;
    if (g0 >= nv || T == 0) return;
    if (ESTIMATE && !amag) return;  // a batch member without the relative criterion
    if (heavy && heavy[group]) return;  // a costly group: walked by a warp pair (force_pair_body)
    // particles: slot g0 + lane (.x of every pair) and g0 + 32 + lane (.y)
    const uint32_t s0 = g0 + lane, s1 = s0 + 32;
    const uint32_t i0 = s0 < nv ? sidx[s0] : 0u, i1 = s1 < nv ? sidx[s1] : 0u;
    const bool v0 = s0 < nv && i0 < n_al, v1 = s1 < nv && i1 < n_al;  // i < n_al unless the sort failed
    const float2 p0 = v0 ? pos_in[i0] : make_float2(0.0f, 0.0f);
    const float2 p1 = v1 ? pos_in[i1] : make_float2(0.0f, 0.0f);
    float bx0[4], bx1[4], by0[4], by1[4];
    group_boxes(skey, g0, nv, s0, s1, v0, v1, p0, p1, bx0, bx1, by0, by1);
    // Relative criterion: the smallest previous |a| of the group, NaN when any is unknown
    // (then the group takes the theta test).  Each group reads and rewrites only its own
    // particles' |a|, so one buffer serves as input and output.
    bool relative = false;
    float tol2 = 0.0f;
    if (amag) {
        const float a0 = v0 ? amag[i0] : INFINITY, a1 = v1 ? amag[i1] : INFINITY;
        const bool unknown = __any_sync(0xffffffffu, isnan(a0) || isnan(a1));
        if (ESTIMATE && !unknown) return;  // warp-uniform: nothing to estimate
        float amin = fminf(a0, a1);
        for (int o = 16; o; o >>= 1) amin = fminf(amin, __shfl_xor_sync(0xffffffffu, amin, o));
        relative = !ESTIMATE && !unknown;
        const float tol = alpha * amin;
        tol2 = tol * tol;
    }
    const float2 P = make_float2(p0.x, p1.x), Q = make_float2(p0.y, p1.y), E2 = make_float2(eps2, eps2);
    // node and leaf accumulators of the two particles (.x particle 0, .y particle 1)
    float2 anx = make_float2(0.0f, 0.0f), any = anx, alx = anx, aly = anx;
    unsigned long long n_int = 0, n_test = 0, n_node = 0;
    uint32_t size = 0, n_nodes = 0, n_items = 0;
    if (skip[0] == 1u) {  // a single particle: the root is its leaf
        if (lane == 0) {
            g.it_start[0] = 0u;
            g.it_count[0] = 1u;
        }
        n_items = 1;
    } else {
        if (lane == 0) g.stack[0] = 0u;
        size = 1;
    }
    __syncwarp();

    while (size > 0) {
        if (n_nodes > (uint32_t)(SM::kNode - 32)) {
            eval_nodes<EXACT, QUAD, SM>(g, n_nodes, rec, quad, P, Q, E2, anx, any, lane);
            n_nodes = 0;
        }
        if (n_items > (uint32_t)(SM::kItem - 64)) {
            eval_leaves<EXACT, SM>(g, n_items, rec, P, Q, E2, alx, aly, lane);
            n_items = 0;
        }
        const uint32_t np = min(size, 32u);
        const uint32_t base = size - np;
        const bool act = lane < (int)np;
        const uint32_t n = act ? g.stack[base + lane] : 0u;
        __syncwarp();
        size = base;
        if (COUNT) n_test += np;
        RecTest r{};
        if (act) test_record(n, rec, kids, bx0, bx1, by0, by1, eps2, relative, tol2, floor2, theta2, r);
        const uint32_t a0 = r.a0, c0 = r.c0, a1 = r.a1, c1 = r.c1, nl = r.nl, nn = r.nn;
        const uint32_t pu0 = r.pu[0], pu1 = r.pu[1], pu2 = r.pu[2], pu3 = r.pu[3];
        uint32_t npu = r.npu;
        // offsets in lane order, three counts in one scan: nodes <= 32, runs <= 64 and
        // pushes <= 128 in warp total, so the 8/8/16-bit fields never carry
        const uint32_t mine = nn | (nl << 8) | (npu << 16);
        uint32_t x = mine;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        const uint32_t ex = x - mine, tot = __shfl_sync(0xffffffffu, x, 31);
        const uint32_t noff = ex & 0xffu, loff = (ex >> 8) & 0xffu, poff = ex >> 16;
        const uint32_t ntot = tot & 0xffu, ltot = (tot >> 8) & 0xffu;
        uint32_t ptot = tot >> 16;
        if (size + ptot > (uint32_t)kStackCap) {  // beyond the depth bound: report, do not overrun
            if (lane == 0) atomicOr(err, kErrTree);
            ptot = 0;
            npu = 0;
        }
        if (nn) g.node[n_nodes + noff] = n;
        if (nl > 0) {
            g.it_start[n_items + loff] = a0;
            g.it_count[n_items + loff] = c0;
        }
        if (nl > 1) {
            g.it_start[n_items + loff + 1] = a1;
            g.it_count[n_items + loff + 1] = c1;
        }
        if (COUNT) {
            n_int += nn + (nl > 0 ? c0 : 0u) + (nl > 1 ? c1 : 0u);
            n_node += nn;
        }
        uint32_t* dst = g.stack + size + poff;
        if (npu > 0) dst[0] = pu0;
        if (npu > 1) dst[1] = pu1;
        if (npu > 2) dst[2] = pu2;
        if (npu > 3) dst[3] = pu3;

        n_nodes += ntot;
        n_items += ltot;
        size += ptot;
        __syncwarp();
    }
    eval_nodes<EXACT, QUAD, SM>(g, n_nodes, rec, quad, P, Q, E2, anx, any, lane);
    eval_leaves<EXACT, SM>(g, n_items, rec, P, Q, E2, alx, aly, lane);
    if (COUNT) {
        if (skip[0] == 1u && lane == 0) n_int += 1;
        for (int o = 16; o; o >>= 1) {
            n_int += __shfl_xor_sync(0xffffffffu, n_int, o);
            n_node += __shfl_xor_sync(0xffffffffu, n_node, o);
        }
        const unsigned long long nval = __popc(__ballot_sync(0xffffffffu, v0)) + __popc(__ballot_sync(0xffffffffu, v1));
        if (lane == 0) {
            atomicAdd(&stat[0], n_int * nval);
            atomicAdd(&stat[1], n_test);
            atomicAdd(&stat[2], n_node * nval);
        }
    }
    group_finish<ESTIMATE>(add2(anx, alx), add2(any, aly), v0, v1, i0, i1, p0, p1, vel_in, pos_out, vel_out, acc_rec,
                           k, hdt, amag, ext);
}

// ------------------------------------------------------------------------------------
// Costly groups: a warp pair per walk.  With the relative criterion a group whose smallest
// previous |a| is far below its largest (every |a| known and a_min < kHeavyRatio a_max)
// opens many more records than the others: on the 500k spiral such groups sum 2.4x the
// mean interactions and their single-warp walks trailed the traversal launch.  In systems
// of at least kHeavyMinParticles particles (more groups than the launch keeps resident)
// their walks run first, each on two warps of one block: pops take the top min(64, size)
// records (warp w tests entries [32w, 32w + 32) of the popped range), the block's pair
// scans the counts of both warps, and item i of the node list (record i of the flattened
// leaf runs) is summed by warp (i / 32) mod 2, each warp from zero in walk order; the node
// (leaf) accumulator is warp 0's + warp 1's.  The tested and accepted records are the
// same as with 32-record pops (a record is tested iff all its ancestors were opened);
// only the summation order differs, and the CPU restatement follows it.
// ------------------------------------------------------------------------------------
// 64-record pops push at most 256 children, one level deeper than the shallowest popped
// record: <= 192 D + 256 entries.
constexpr int kPairStackCap = 192 * (kBBoxMaxBits > kFixedDepth ? kBBoxMaxBits : kFixedDepth) + 256;
constexpr int kPairNode = 192, kPairItem = 256;  // a round adds <= 64 nodes and <= 128 runs

// No larger than the two single-warp walks it shares a block's shared memory with (the
// traversal is sensitive to the L1 that shared memory leaves).
struct PairSmem {
    uint32_t stack[kPairStackCap];
    uint32_t node[kPairNode];
    uint32_t it_start[kPairItem], it_count[kPairItem], off[kPairItem];
    union {
        struct {
            float cx[2][32], cy[2][32], cm[2][32];  // one staged chunk per warp
            float qxx[2][32], qxy[2][32], qyy[2][32], mt[2][32];
        };
        float2 part[4][32];  // after the sums: warp 1's accumulators, added by warp 0
    };
    uint32_t tot[2];  // packed round counts of each warp
};
static_assert(sizeof(PairSmem) <= 2 * sizeof(GroupSmem<160, 128>), "a pair walk fits in two warp walks");

// Barrier of the two warps of pair `pair` (named barrier 1 + pair; __syncthreads uses 0).
__device__ __forceinline__ void pair_sync(int pair) { asm volatile("bar.sync %0, 64;" ::"r"(1 + pair) : "memory"); }

// Warp wp's share of the count accepted nodes in g.node, whose global list indices are
// gbase .. gbase + count - 1: the 32-item chunks c with c mod 2 == wp, in order (each
// chunk's records loaded while the one before is summed).
template <bool EXACT, bool QUAD>
__device__ __forceinline__ void pair_eval_nodes(PairSmem& g, int wp, uint32_t count, uint32_t gbase,
                                                const float4* __restrict__ rec, const float4* __restrict__ quad,
                                                float2 P, float2 Q, float2 E2, float2& acx, float2& acy, int lane) {
    const uint32_t end = gbase + count;
    uint32_t c = gbase >> 5;
    if ((c & 1u) != (uint32_t)wp) ++c;
    if (!count || c * 32 >= end) return;
    float4 q = make_float4(0.0f, 0.0f, 0.0f, 0.0f), qq = q;
    {
        const uint32_t f = c * 32 + (uint32_t)lane;  // global index of the lane's item
        if (f >= gbase && f < end) {
            const uint32_t r = g.node[f - gbase];
            q = __ldg(&rec[r]);
            if (QUAD) qq = __ldg(&quad[r]);
        }
    }
    for (; c * 32 < end; c += 2) {
        g.cx[wp][lane] = q.x;
        g.cy[wp][lane] = q.y;
        g.cm[wp][lane] = q.z;
        if (QUAD) {
            g.qxx[wp][lane] = 7.5f * qq.x;
            g.qxy[wp][lane] = 7.5f * qq.y;
            g.qyy[wp][lane] = 7.5f * qq.z;
            g.mt[wp][lane] = -1.5f * (qq.x + qq.z);
        }
        __syncwarp();
        const uint32_t fn = (c + 2) * 32 + (uint32_t)lane;  // the warp's next chunk (all past gbase)
        if (fn < end) {
            const uint32_t r = g.node[fn - gbase];
            q = __ldg(&rec[r]);
            if (QUAD) qq = __ldg(&quad[r]);
        }
        const uint32_t klo = gbase > c * 32 ? gbase - c * 32 : 0u;
        const uint32_t khi = min(end - c * 32, 32u);
#pragma unroll 4
        for (uint32_t j = klo; j < khi; ++j) {
            if (QUAD)
                quadrupole_x2<EXACT>(g.cx[wp][j], g.cy[wp][j], g.cm[wp][j], g.qxx[wp][j], g.qxy[wp][j], g.qyy[wp][j],
                                     g.mt[wp][j], P, Q, E2, acx, acy);
            else
                monopole_x2<EXACT>(g.cx[wp][j], g.cy[wp][j], g.cm[wp][j], P, Q, E2, acx, acy);
        }
        __syncwarp();
    }
}

// Record fl of the flattened leaf runs of a pair (last run with off <= fl).
__device__ __forceinline__ float4 pair_gather_leaf(const PairSmem& g, uint32_t n_items, uint32_t fl,
                                                   const float4* __restrict__ rec) {
    uint32_t lo = 0, hi = n_items - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (g.off[mid] <= fl) lo = mid;
        else hi = mid - 1;
    }
    return __ldg(&rec[g.it_start[lo] + (fl - g.off[lo])]);
}

// Warp wp's share of the particle leaves of the n_items runs, whose flattened records have
// global indices lbase ..; returns the number of records.  Both warps of the pair must call
// it (warp 0 writes the run offsets, then the pair synchronises).
template <bool EXACT>
__device__ __forceinline__ uint32_t pair_eval_leaves(PairSmem& g, int pair, int wp, uint32_t n_items, uint32_t lbase,
                                                     const float4* __restrict__ rec, float2 P, float2 Q, float2 E2,
                                                     float2& acx, float2& acy, int lane) {
    if (!n_items) return 0u;
    constexpr int kPer = kPairItem / 32;
    uint32_t cnt[kPer], sum = 0;
#pragma unroll
    for (int t = 0; t < kPer; ++t) {
        const uint32_t it = (uint32_t)lane * kPer + t;
        cnt[t] = it < n_items ? g.it_count[it] : 0u;
        sum += cnt[t];
    }
    uint32_t x = sum;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, x, 31);
    if (wp == 0) {
        uint32_t run = x - sum;
#pragma unroll
        for (int t = 0; t < kPer; ++t) {
            g.off[lane * kPer + t] = run;
            run += cnt[t];
        }
    }
    pair_sync(pair);
    const uint32_t end = lbase + total;
    uint32_t c = lbase >> 5;
    if ((c & 1u) != (uint32_t)wp) ++c;
    if (c * 32 >= end) return total;
    float4 q = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    {
        const uint32_t f = c * 32 + (uint32_t)lane;
        if (f >= lbase && f < end) q = pair_gather_leaf(g, n_items, f - lbase, rec);
    }
    for (; c * 32 < end; c += 2) {
        g.cx[wp][lane] = q.x;
        g.cy[wp][lane] = q.y;
        g.cm[wp][lane] = q.z;
        __syncwarp();
        const uint32_t fn = (c + 2) * 32 + (uint32_t)lane;
        if (fn < end) q = pair_gather_leaf(g, n_items, fn - lbase, rec);
        const uint32_t klo = lbase > c * 32 ? lbase - c * 32 : 0u;
        const uint32_t khi = min(end - c * 32, 32u);
#pragma unroll 4
        for (uint32_t j = klo; j < khi; ++j) monopole_x2<EXACT>(g.cx[wp][j], g.cy[wp][j], g.cm[wp][j], P, Q, E2, acx, acy);
        __syncwarp();
    }
    return total;
}

// The walk of costly group `group` by warp wp (0, 1) of pair `pair`; both warps call it
// with the same arguments.  Warp 0 integrates.
template <bool EXACT, bool COUNT>
__device__ __forceinline__ void force_pair_body(
    uint32_t group, int pair, int wp, PairSmem& g, const uint32_t* __restrict__ sidx,
    const uint32_t* __restrict__ skey, const uint32_t* __restrict__ counts, const float4* __restrict__ rec,
    const uint32_t* __restrict__ skip, const float4* __restrict__ quad, const uint4* __restrict__ kids,
    const float2* __restrict__ pos_in, const float2* __restrict__ vel_in, float2* __restrict__ pos_out,
    float2* __restrict__ vel_out, float2* __restrict__ acc_rec, uint32_t n_al, float eps2, float k, float hdt,
    uint32_t cap, unsigned long long* __restrict__ stat, int* __restrict__ err, float* __restrict__ amag,
    float alpha, float floor2, uint32_t* __restrict__ ext) {
    const int lane = threadIdx.x & 31;
    const uint32_t nv = counts[0];
    const uint32_t T = min(nv + counts[1], cap);
    const uint32_t g0 = group * kGroupSize;
    if (g0 >= nv || T == 0) return;  // never for a listed group; the same for both warps
    const uint32_t s0 = g0 + lane, s1 = s0 + 32;
    const uint32_t i0 = s0 < nv ? sidx[s0] : 0u, i1 = s1 < nv ? sidx[s1] : 0u;
    const bool v0 = s0 < nv && i0 < n_al, v1 = s1 < nv && i1 < n_al;
    const float2 p0 = v0 ? pos_in[i0] : make_float2(0.0f, 0.0f);
    const float2 p1 = v1 ? pos_in[i1] : make_float2(0.0f, 0.0f);
    float bx0[4], bx1[4], by0[4], by1[4];
    group_boxes(skey, g0, nv, s0, s1, v0, v1, p0, p1, bx0, bx1, by0, by1);
    float amin = fminf(v0 ? amag[i0] : INFINITY, v1 ? amag[i1] : INFINITY);  // every |a| is known
    for (int o = 16; o; o >>= 1) amin = fminf(amin, __shfl_xor_sync(0xffffffffu, amin, o));
    const float tol = alpha * amin, tol2 = tol * tol;
    const float2 P = make_float2(p0.x, p1.x), Q = make_float2(p0.y, p1.y), E2 = make_float2(eps2, eps2);
    float2 anx = make_float2(0.0f, 0.0f), any = anx, alx = anx, aly = anx;
    unsigned long long n_int = 0, n_test = 0, n_node = 0;
    uint32_t size = 0, n_nodes = 0, n_items = 0, gnode = 0, gleaf = 0;
    if (skip[0] == 1u) {  // a single particle: the root is its leaf
        if (wp == 0 && lane == 0) {
            g.it_start[0] = 0u;
            g.it_count[0] = 1u;
        }
        n_items = 1;
    } else {
        if (wp == 0 && lane == 0) g.stack[0] = 0u;
        size = 1;
    }
    for (;;) {
        pair_sync(pair);  // the last round's lists, pushes and counts are visible
        if (size == 0) break;
        if (n_nodes > (uint32_t)(kPairNode - 64)) {
            pair_eval_nodes<EXACT, true>(g, wp, n_nodes, gnode, rec, quad, P, Q, E2, anx, any, lane);
            gnode += n_nodes;
            n_nodes = 0;
            pair_sync(pair);
        }
        if (n_items > (uint32_t)(kPairItem - 128)) {
            gleaf += pair_eval_leaves<EXACT>(g, pair, wp, n_items, gleaf, rec, P, Q, E2, alx, aly, lane);
            n_items = 0;
            pair_sync(pair);
        }
        const uint32_t np = min(size, 64u);
        const uint32_t base = size - np;
        const uint32_t L = (uint32_t)(wp * 32 + lane);
        const bool act = L < np;
        const uint32_t n = act ? g.stack[base + L] : 0u;
        pair_sync(pair);  // both warps hold their records before pushes overwrite the stack top
        size = base;
        if (COUNT) n_test += __popc(__ballot_sync(0xffffffffu, act));
        RecTest r{};
        if (act) test_record(n, rec, kids, bx0, bx1, by0, by1, eps2, true, tol2, floor2, 0.0f, r);
        // offsets in pair order: this warp's scan plus warp 0's total for warp 1; nodes
        // <= 64, runs <= 128 and pushes <= 256 in pair total, so the 8/8/16-bit fields
        // never carry
        const uint32_t mine = r.nn | (r.nl << 8) | (r.npu << 16);
        uint32_t x = mine;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) g.tot[wp] = x;
        pair_sync(pair);
        const uint32_t t0 = g.tot[0], t1 = g.tot[1];
        const uint32_t ex = x - mine + (wp ? t0 : 0u), tot = t0 + t1;
        const uint32_t noff = ex & 0xffu, loff = (ex >> 8) & 0xffu, poff = ex >> 16;
        const uint32_t ntot = tot & 0xffu, ltot = (tot >> 8) & 0xffu;
        uint32_t ptot = tot >> 16, npu = r.npu;
        if (size + ptot > (uint32_t)kPairStackCap) {  // beyond the depth bound: report, do not overrun
            if (wp == 0 && lane == 0) atomicOr(err, kErrTree);
            ptot = 0;
            npu = 0;
        }
        if (r.nn) g.node[n_nodes + noff] = n;
        if (r.nl > 0) {
            g.it_start[n_items + loff] = r.a0;
            g.it_count[n_items + loff] = r.c0;
        }
        if (r.nl > 1) {
            g.it_start[n_items + loff + 1] = r.a1;
            g.it_count[n_items + loff + 1] = r.c1;
        }
        if (COUNT) {
            n_int += r.nn + (r.nl > 0 ? r.c0 : 0u) + (r.nl > 1 ? r.c1 : 0u);
            n_node += r.nn;
        }
        uint32_t* dst = g.stack + size + poff;
        if (npu > 0) dst[0] = r.pu[0];
        if (npu > 1) dst[1] = r.pu[1];
        if (npu > 2) dst[2] = r.pu[2];
        if (npu > 3) dst[3] = r.pu[3];
        n_nodes += ntot;
        n_items += ltot;
        size += ptot;
    }
    pair_eval_nodes<EXACT, true>(g, wp, n_nodes, gnode, rec, quad, P, Q, E2, anx, any, lane);
    pair_eval_leaves<EXACT>(g, pair, wp, n_items, gleaf, rec, P, Q, E2, alx, aly, lane);
    if (COUNT) {
        if (skip[0] == 1u && wp == 0 && lane == 0) n_int += 1;
        for (int o = 16; o; o >>= 1) {
            n_int += __shfl_xor_sync(0xffffffffu, n_int, o);
            n_node += __shfl_xor_sync(0xffffffffu, n_node, o);
        }
        const unsigned long long nval = __popc(__ballot_sync(0xffffffffu, v0)) + __popc(__ballot_sync(0xffffffffu, v1));
        if (lane == 0) {
            atomicAdd(&stat[0], n_int * nval);
            atomicAdd(&stat[1], n_test);
            atomicAdd(&stat[2], n_node * nval);
        }
    }
    pair_sync(pair);  // both warps are done with their staged chunks
    if (wp == 1) {
        g.part[0][lane] = anx;
        g.part[1][lane] = any;
        g.part[2][lane] = alx;
        g.part[3][lane] = aly;
    }
    pair_sync(pair);
    if (wp == 0) {
        anx = add2(anx, g.part[0][lane]);
        any = add2(any, g.part[1][lane]);
        alx = add2(alx, g.part[2][lane]);
        aly = add2(aly, g.part[3][lane]);
        group_finish<false>(add2(anx, alx), add2(any, aly), v0, v1, i0, i1, p0, p1, vel_in, pos_out, vel_out,
                            acc_rec, k, hdt, amag, ext);
    }
    pair_sync(pair);  // the pair's shared memory is free for its next group
}

// list caps of a shape
template <bool SHORT>
using GroupSmemOf = GroupSmem<SHORT ? 96 : 160, SHORT ? 64 : 128>;

// Shared memory of a traversal block: a walk per warp, and with HEAVY (the main pass of
// the relative criterion) the bytes of warps 2p and 2p + 1 also hold the walk of warp pair
// p, so that a pair done with costly groups starts its own warps' walks at once.
template <bool SHORT, int WARPS, bool HEAVY>
struct ForceSmem {
    GroupSmemOf<SHORT> warp[WARPS];
    __device__ __forceinline__ GroupSmemOf<SHORT>& walk(int w) { return warp[w]; }
};
template <bool SHORT>
union PairSlot {
    GroupSmemOf<SHORT> warp[2];
    PairSmem pair;
};
template <bool SHORT, int WARPS>
struct ForceSmem<SHORT, WARPS, true> {
    PairSlot<SHORT> slot[WARPS / 2];
    __device__ __forceinline__ GroupSmemOf<SHORT>& walk(int w) { return slot[w >> 1].warp[w & 1]; }
};

// The next listed costly group for warp pair `pair` (hwork[0] entries, hwork[1] the next
// to take), or a value >= hwork[0] when none is left.  Both warps of the pair call it.
__device__ __forceinline__ uint32_t pair_ticket(uint32_t* __restrict__ hwork, uint32_t cnt, uint32_t* s_u, int pair) {
    if ((threadIdx.x & 63u) == 0) s_u[pair] = __ldcg(&hwork[1]) < cnt ? atomicAdd(&hwork[1], 1u) : cnt;
    pair_sync(pair);
    const uint32_t u = s_u[pair];
    pair_sync(pair);  // read by both warps before the pair's next ticket
    return u;
}

// With HEAVY every warp pair first walks listed costly groups (heavy_list[u].y, taken in
// order from hwork) and then each warp its own group: the costly walks start first.
template <bool EXACT, bool QUAD, bool COUNT, bool ESTIMATE, int WARPS, bool SHORT, bool HEAVY>
__global__ void __launch_bounds__(WARPS * 32)
k_force_group(const uint32_t* __restrict__ sidx, const uint32_t* __restrict__ skey, const uint32_t* __restrict__ counts,
              const float4* __restrict__ rec, const uint32_t* __restrict__ skip, const float4* __restrict__ quad,
              const uint4* __restrict__ kids, const float2* __restrict__ pos_in, const float2* __restrict__ vel_in,
              float2* __restrict__ pos_out, float2* __restrict__ vel_out, float2* __restrict__ acc_rec,
              uint32_t n_al, float eps2, float theta2, float k, float hdt, uint32_t cap,
              unsigned long long* __restrict__ stat, int* __restrict__ err, float* __restrict__ amag, float alpha,
              float floor2, uint32_t* __restrict__ ext, const uint8_t* __restrict__ heavy,
              const uint2* __restrict__ heavy_list, uint32_t* __restrict__ hwork) {
    pdl_enter();
    __shared__ ForceSmem<SHORT, WARPS, HEAVY> sm;
    if constexpr (HEAVY) {
        static_assert(QUAD && !ESTIMATE && WARPS % 2 == 0, "warp pairs walk costly groups of the relative main pass");
        __shared__ uint32_t s_u[WARPS / 2];
        const int pair = (int)(threadIdx.x >> 6), wp = (int)((threadIdx.x >> 5) & 1u);
        const uint32_t cnt = hwork[0];
        for (uint32_t u; (u = pair_ticket(hwork, cnt, s_u, pair)) < cnt;)
            force_pair_body<EXACT, COUNT>(heavy_list[u].y, pair, wp, sm.slot[pair].pair, sidx, skey, counts, rec, skip,
                                          quad, kids, pos_in, vel_in, pos_out, vel_out, acc_rec, n_al, eps2, k, hdt,
                                          cap, stat, err, amag, alpha, floor2, ext);
    }
    force_group_body<EXACT, QUAD, COUNT, ESTIMATE, WARPS>(grid_blk(), sm.walk((int)(threadIdx.x >> 5)), sidx, skey,
                                                   counts, rec, skip, quad, kids, pos_in, vel_in, pos_out, vel_out,
                                                   acc_rec, n_al, eps2, theta2, k, hdt, cap, stat, err, amag, alpha,
                                                   floor2, ext, HEAVY ? heavy : nullptr);
}

// Batched: a persistent grid; with HEAVY each warp pair first takes costly groups
// {member, group} from the batch's list, then every block takes block units of the
// members from `work`.
template <bool EXACT, bool QUAD, bool COUNT, bool ESTIMATE, int WARPS, bool SHORT, bool HEAVY>
__global__ void __launch_bounds__(WARPS * 32)
kb_force_group(BatchArgs a, uint32_t* __restrict__ work, const uint2* __restrict__ heavy_list,
               uint32_t* __restrict__ hwork) {
    pdl_enter();
    __shared__ ForceSmem<SHORT, WARPS, HEAVY> sm;
    __shared__ uint32_t s_b;
    if constexpr (HEAVY) {
        static_assert(QUAD && !ESTIMATE && WARPS % 2 == 0, "warp pairs walk costly groups of the relative main pass");
        __shared__ uint32_t s_u[WARPS / 2];
        const int pair = (int)(threadIdx.x >> 6), wp = (int)((threadIdx.x >> 5) & 1u);
        const uint32_t cnt = hwork[0];
        for (uint32_t u; (u = pair_ticket(hwork, cnt, s_u, pair)) < cnt;) {
            const uint2 e = heavy_list[u];
            const SysDesc& d = a.descs[e.x];
            const int in = (int)((d.parity + a.step) & 1u), out = in ^ 1;
            const int f = d.passes & 1;
            force_pair_body<EXACT, COUNT>(e.y, pair, wp, sm.slot[pair].pair, d.idx[f], d.keys[f],
                                          d.counters + kCtrValid, d.rec, d.skip, d.quad, d.kids, d.pos[in],
                                          d.vel[in], d.pos[out], d.vel[out], d.acc, d.n_al, d.eps2, d.k, d.hdt,
                                          d.cap, (unsigned long long*)(d.counters + kCtrStat), d.err, d.amag,
                                          d.alpha, d.floor2, d.ext ? d.ext + 4 * out : nullptr);
        }
    }
    const uint32_t total = __ldg(&a.first[a.nsys]);
    for (;;) {
        __syncthreads();  // every thread has read the previous s_b
        if (threadIdx.x == 0) s_b = atomicAdd(work, 1u);
        __syncthreads();
        const uint32_t b = s_b;
        if (b >= total) break;
        const BatchBlock bb = batch_block(a, b);
        const SysDesc& d = *bb.d;
        const int f = d.passes & 1;
        force_group_body<EXACT, QUAD, COUNT, ESTIMATE, WARPS>(bb.blk, sm.walk((int)(threadIdx.x >> 5)), d.idx[f],
                                             d.keys[f], d.counters + kCtrValid, d.rec, d.skip, d.quad, d.kids,
                                             d.pos[bb.in], d.vel[bb.in], d.pos[bb.out], d.vel[bb.out], d.acc, d.n_al,
                                             d.eps2, d.theta2, d.k, d.hdt, d.cap,
                                             (unsigned long long*)(d.counters + kCtrStat), d.err, d.amag, d.alpha,
                                             d.floor2, d.ext ? d.ext + 4 * bb.out : nullptr,
                                             HEAVY ? d.heavy : nullptr);
    }
}

template <bool EXACT, bool COUNT>
__global__ void __launch_bounds__(kForceWarps * 32) kb_force(BatchArgs a, uint32_t* __restrict__ work) {
    pdl_enter();
    __shared__ uint32_t s_b;
    const uint32_t total = __ldg(&a.first[a.nsys]);
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_b = atomicAdd(work, 1u);
        __syncthreads();
        const uint32_t b = s_b;
        if (b >= total) break;
        const BatchBlock bb = batch_block(a, b);
        const SysDesc& d = *bb.d;
        const int f = d.passes & 1;
        force_body<EXACT, COUNT>(bb.blk, d.idx[f], d.counters + kCtrValid, d.rec, d.skip, d.pos[bb.in],
                                 d.vel[bb.in], d.pos[bb.out], d.vel[bb.out], d.acc, d.n_al, d.eps2, d.theta2, d.k,
                                 d.hdt, d.cap, (unsigned long long*)(d.counters + kCtrStat),
                                 d.ext ? d.ext + 4 * bb.out : nullptr);
    }
}

}  // namespace
}  // namespace gsim

namespace gsim {
namespace {

using GroupFn = void (*)(const uint32_t*, const uint32_t*, const uint32_t*, const float4*, const uint32_t*,
                         const float4*, const uint4*, const float2*, const float2*, float2*, float2*, float2*,
                         uint32_t, float, float, float, float, uint32_t, unsigned long long*, int*, float*, float,
                         float, uint32_t*, const uint8_t*, const uint2*, uint32_t*);
using BatchGroupFn = void (*)(BatchArgs, uint32_t*, const uint2*, uint32_t*);

// The group-walk kernel of one shape (counting variants: the default shape only); heavy:
// the main pass with warp pairs for costly groups (quadrupoles, relative criterion).
template <bool EXACT, int W, bool S>
GroupFn group_fn(bool quad, bool est, bool heavy) {
    if (est) return k_force_group<EXACT, true, false, true, W, S, false>;
    if constexpr (W % 2 == 0)
        if (heavy) return k_force_group<EXACT, true, false, false, W, S, true>;
    return quad ? k_force_group<EXACT, true, false, false, W, S, false>
                : k_force_group<EXACT, false, false, false, W, S, false>;
}
template <bool EXACT>
GroupFn group_fn_count(bool quad, bool est, bool heavy) {
    if (est) return k_force_group<EXACT, true, true, true, 2, false, false>;
    if (heavy) return k_force_group<EXACT, true, true, false, 2, false, true>;
    return quad ? k_force_group<EXACT, true, true, false, 2, false, false>
                : k_force_group<EXACT, false, true, false, 2, false, false>;
}
template <bool EXACT, int W, bool S>
BatchGroupFn batch_group_fn(bool quad, bool est, bool heavy) {
    if (est) return kb_force_group<EXACT, true, false, true, W, S, false>;
    if constexpr (W % 2 == 0)
        if (heavy) return kb_force_group<EXACT, true, false, false, W, S, true>;
    return quad ? kb_force_group<EXACT, true, false, false, W, S, false>
                : kb_force_group<EXACT, false, false, false, W, S, false>;
}
template <bool EXACT>
BatchGroupFn batch_group_fn_count(bool quad, bool est, bool heavy) {
    if (est) return kb_force_group<EXACT, true, true, true, 2, false, false>;
    if (heavy) return kb_force_group<EXACT, true, true, false, 2, false, true>;
    return quad ? kb_force_group<EXACT, true, true, false, 2, false, false>
                : kb_force_group<EXACT, false, true, false, 2, false, false>;
}

// warps per block and list caps actually launched for a request (warp pairs need an even
// number of warps: a one-warp shape runs with two when costly groups are paired)
inline void group_shape(bool count, const gs_shape& sh, bool heavy, int* warps, bool* shrt) {
    *warps = count ? 2 : (int)sh.force_warps;
    if (heavy && *warps == 1) *warps = 2;
    *shrt = count ? false : sh.force_short_lists != 0;
}

template <bool EXACT>
GroupFn pick_group(bool count, const gs_shape& sh, bool quad, bool est, bool heavy, int* warps) {
    bool shrt;
    group_shape(count, sh, heavy, warps, &shrt);
    if (count) return group_fn_count<EXACT>(quad, est, heavy);
    switch (*warps * 2 + (shrt ? 1 : 0)) {
        case 2: return group_fn<EXACT, 1, false>(quad, est, false);
        case 5: return group_fn<EXACT, 2, true>(quad, est, heavy);
        case 8: return group_fn<EXACT, 4, false>(quad, est, heavy);
        default: *warps = 2; return group_fn<EXACT, 2, false>(quad, est, heavy);
    }
}

template <bool EXACT>
BatchGroupFn pick_batch_group(bool count, const gs_shape& sh, bool quad, bool est, bool heavy, int* warps) {
    bool shrt;
    group_shape(count, sh, heavy, warps, &shrt);
    if (count) return batch_group_fn_count<EXACT>(quad, est, heavy);
    switch (*warps * 2 + (shrt ? 1 : 0)) {
        case 2: return batch_group_fn<EXACT, 1, false>(quad, est, false);
        case 5: return batch_group_fn<EXACT, 2, true>(quad, est, heavy);
        case 8: return batch_group_fn<EXACT, 4, false>(quad, est, heavy);
        default: *warps = 2; return batch_group_fn<EXACT, 2, false>(quad, est, heavy);
    }
}

template <bool EXACT>
cudaError_t force_launch_impl(const ForceLaunch& f) {
    if (!f.group) {  // the reference's warp-vote walk
        auto fn = f.count ? k_force<EXACT, true> : k_force<EXACT, false>;
        const int blocks = (int)((f.n_al / 32 + kForceWarps - 1) / kForceWarps);
        return launch(f.pdl, fn, blocks, kForceWarps * 32, f.st, f.sidx, f.counts, f.rec, f.skip, f.pos_in, f.vel_in,
                      f.pos_out, f.vel_out, f.acc, f.n_al, f.eps2, f.theta2, f.k, f.hdt, f.cap, f.stat, f.ext);
    }
    int warps = 2;
    const bool heavy = f.heavy && f.quad && !f.estimate;
    GroupFn fn = pick_group<EXACT>(f.count, f.shape, f.quad, f.estimate, heavy, &warps);
    const int blocks = (int)((f.n_al / kGroupSize + warps - 1) / warps);
    return launch(f.pdl, fn, blocks, warps * 32, f.st, f.sidx, f.skey, f.counts, f.rec, f.skip, f.quad_m, f.kids,
                  f.pos_in, f.vel_in, f.pos_out, f.vel_out, f.acc, f.n_al, f.eps2, f.theta2, f.k, f.hdt, f.cap,
                  f.stat, f.err, f.amag, f.alpha, f.floor2, f.ext, heavy ? f.heavy : nullptr,
                  heavy ? f.heavy_list : nullptr, heavy ? f.heavy_work : nullptr);
}

template <bool EXACT>
cudaError_t batch_force_launch_impl(const BatchForceLaunch& b, int* grid_out) {
    int dev = 0, sms = 0, per_sm = 0, threads = kForceWarps * 32;
    const bool heavy = b.heavy_list && b.quad && !b.estimate;
    auto resident = [&](auto fn) -> cudaError_t {  // resident blocks of the persistent launch
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0);
        if (e != cudaSuccess) return e;
        *grid_out = (sms > 0 ? sms : 152) * (per_sm > 0 ? per_sm : 1);
        return cudaSuccess;
    };
    if (!b.group) {
        auto fn = b.count ? kb_force<EXACT, true> : kb_force<EXACT, false>;
        if (grid_out) return resident(fn);
        return launch(true, fn, b.grid, threads, b.st, BatchArgs{b.descs, b.first, b.nsys, b.step}, b.work);
    }
    int warps = 2;
    BatchGroupFn fn = pick_batch_group<EXACT>(b.count, b.shape, b.quad, b.estimate, heavy, &warps);
    threads = warps * 32;
    if (grid_out) return resident(fn);
    return launch(true, fn, b.grid, threads, b.st, BatchArgs{b.descs, b.first, b.nsys, b.step}, b.work,
                  heavy ? b.heavy_list : nullptr, heavy ? b.heavy_work : nullptr);
}

}  // namespace
}  // namespace gsim
