// moments.cuh -- node moments of the accurate mode (GS_FLAG_QUADRUPOLE) from exact integer
// sums.  No counterpart in the reference, whose moments are FP32 sums of the children
// level by level (TreeInitShader.comp:78-80, TreeMoveShader.comp:66-67); the reference
// rule keeps those (k_coop_sums in bh.cu).
//
// Every particle is put on an integer grid: its mass as m_q = rint(m 2^(31-em)), the
// largest mass of the system being f 2^em (f in [0.5, 1)), and its position as
// x_q = rint(x 2^(30-e)) - rint(bx 2^(30-e)), clamped to +-2^30, with the box centre bx and
// half-size h = f 2^e.  A node's sums M = sum m_q, X = sum m_q x_q, Y, XX = sum m_q x_q^2, XY, YY
// are exact 128-bit integers: the same whatever order they are added in.  They are the
// differences of exclusive prefix sums over the sorted slots at the node's first slot and
// one past its last:
//   k_records    each slot's integer mass and position (m_q, x_q, y_q),
//   k_mom_scan   the exclusive prefix of the six sums at every slot: one pass, 256 slots
//                per block, a decoupled look-back over the blocks' exact sums,
//   k_nodes      each node's sums and its rounded moments (mom_node):
//     centre  cx = bx + (f(X) / f(M)) 2^(e-30),  mass  m = f(M) 2^(em-31),
//     second central moments about an integer origin x0 = rint(f(X) / f(M)) (exact:
//     Dx = X - x0 M, Sxx = XX - x0 (X + Dx), Sxy = XY - x0 Y - y0 Dx), then
//     Qxx = f(Sxx) - f(Dx) (f(Dx) / f(M)) and so on, scaled by 2^(2(e-30)) and 2^(em-31);
// f() rounds a 128-bit integer to the nearest float.  The levels of the tree need no
// grid barrier between them, and the result does not depend on how the sums are split
// over blocks.  A node of zero mass gets centre (0, 0) and zero moments.
#pragma once
#include "bh_common.cuh"

namespace gsim {

// exact sums of one node, tile or prefix (96 bytes)
struct __align__(16) MomSums {
    __int128 m, x, y, xx, xy, yy;
};

namespace {

typedef __int128 i128;
typedef unsigned __int128 u128;

struct MomScale {
    float bx, by, iqs, ims;  // box centre, 2^(e-30), 2^(em-31)
    float qs, ms;            // 2^(30-e), 2^(31-em)
};

__device__ __forceinline__ int exponent_of(float v, int lo, int hi) {
    int e = 0;
    if (v > 0.0f) frexpf(v, &e);
    return e < lo ? lo : e > hi ? hi : e;
}

// The grid of a step: the box of its keys (fixed box: centre 0, half-size 500) and the
// largest mass (the float bits that k_keygen / k_ext_keys took the maximum of).
__device__ __forceinline__ MomScale mom_scale(int bbox_mode, const BHParams& bp, uint32_t mmax_bits) {
    const float half = bbox_mode ? ldexpf(bp.inv_scale, bp.bits - 1) : kSimSize;
    const int e = exponent_of(half, -96, 127), em = exponent_of(__uint_as_float(mmax_bits), -94, 127);
    MomScale s;
    s.bx = bbox_mode ? bp.cx : 0.0f;
    s.by = bbox_mode ? bp.cy : 0.0f;
    s.qs = ldexpf(1.0f, 30 - e);
    s.iqs = ldexpf(1.0f, e - 30);
    s.ms = ldexpf(1.0f, 31 - em);
    s.ims = ldexpf(1.0f, em - 31);
    return s;
}

// p 2^(30-e), b 2^(30-e) and m 2^(31-em) are exact scalings by powers of two; each is
// rounded to the nearest integer (a float subtraction p - b would round to the spacing of
// the larger operand, coarser than the grid where |b| > |p - b|)
__device__ __forceinline__ int quantize_pos(float p, float b, float qs) {
    const float pq = rintf(__fmul_rn(p, qs)), bq = rintf(__fmul_rn(b, qs));
    if (!(fabsf(pq) < 9.0e18f) || !(fabsf(bq) < 9.0e18f)) return 0;  // beyond 64 bits, or NaN
    long long q = (long long)pq - (long long)bq;
    if (q < -1073741824ll) q = -1073741824ll;
    if (q > 1073741824ll) q = 1073741824ll;
    return (int)q;
}

__device__ __forceinline__ int quantize_mass(float m, float ms) {
    return m > 0.0f ? (int)rintf(__fmul_rn(m, ms)) : 0;
}

__device__ __forceinline__ void mom_clear(MomSums& a) { a.m = a.x = a.y = a.xx = a.xy = a.yy = 0; }

__device__ __forceinline__ void mom_add(MomSums& a, const MomSums& b) {
    a.m += b.m;
    a.x += b.x;
    a.y += b.y;
    a.xx += b.xx;
    a.xy += b.xy;
    a.yy += b.yy;
}

// Exact products from 32 x 32 -> 64-bit multiplies (a generic 128-bit product takes about
// four times the instructions): a * b for |a| < 2^63, and the low 128 bits of a * b.
__device__ __forceinline__ i128 mul_i64_i32(long long a, int b) {
    const long long lo = (long long)(unsigned long long)(unsigned)a * b;  // |.| < 2^63
    const long long hi = (a >> 32) * (long long)b;                         // |.| < 2^62
    return ((i128)hi << 32) + lo;
}
__device__ __forceinline__ i128 mul_i128_i32(i128 a, int b) {
    const unsigned long long lo = (unsigned long long)a;
    const long long p0 = (long long)(unsigned long long)(unsigned)lo * b;
    const long long p1 = (long long)(lo >> 32) * b;
    const unsigned long long p2 = (unsigned long long)(long long)(a >> 64) * (unsigned long long)(long long)b;
    return (i128)(((u128)p2 << 64) + (u128)((i128)p1 << 32) + (u128)(i128)p0);  // modulo 2^128
}

// a particle's integer mass and position {m_q, x_q, y_q, 0}
__device__ __forceinline__ int4 mom_quantize(float2 p, float m, const MomScale& sc) {
    return make_int4(quantize_mass(m, sc.ms), quantize_pos(p.x, sc.bx, sc.qs), quantize_pos(p.y, sc.by, sc.qs), 0);
}

__device__ __forceinline__ void mom_add_q(MomSums& a, int4 q) {
    const int mq = q.x, xq = q.y, yq = q.z;
    const long long mx = (long long)mq * xq, my = (long long)mq * yq;  // |m_q x_q| <= 2^61
    a.m += mq;
    a.x += mx;
    a.y += my;
    a.xx += mul_i64_i32(mx, xq);
    a.xy += mul_i64_i32(mx, yq);
    a.yy += mul_i64_i32(my, yq);
}

__device__ __forceinline__ i128 shfl_xor_i128(i128 v, int o) {
    const unsigned long long lo = (unsigned long long)v, hi = (unsigned long long)((u128)v >> 64);
    const unsigned long long l2 = __shfl_xor_sync(0xffffffffu, lo, o), h2 = __shfl_xor_sync(0xffffffffu, hi, o);
    return (i128)(((u128)h2 << 64) | l2);
}
__device__ __forceinline__ i128 shfl_up_i128(i128 v, int o) {
    const unsigned long long lo = (unsigned long long)v, hi = (unsigned long long)((u128)v >> 64);
    const unsigned long long l2 = __shfl_up_sync(0xffffffffu, lo, o), h2 = __shfl_up_sync(0xffffffffu, hi, o);
    return (i128)(((u128)h2 << 64) | l2);
}

__device__ __forceinline__ void mom_warp_sum(MomSums& a) {
    for (int o = 16; o; o >>= 1) {
        a.m += shfl_xor_i128(a.m, o);
        a.x += shfl_xor_i128(a.x, o);
        a.y += shfl_xor_i128(a.y, o);
        a.xx += shfl_xor_i128(a.xx, o);
        a.xy += shfl_xor_i128(a.xy, o);
        a.yy += shfl_xor_i128(a.yy, o);
    }
}

// inclusive scan over the lanes of a warp
__device__ __forceinline__ void mom_warp_scan(MomSums& a, int lane) {
    for (int o = 1; o < 32; o <<= 1) {
        MomSums b;
        b.m = shfl_up_i128(a.m, o);
        b.x = shfl_up_i128(a.x, o);
        b.y = shfl_up_i128(a.y, o);
        b.xx = shfl_up_i128(a.xx, o);
        b.xy = shfl_up_i128(a.xy, o);
        b.yy = shfl_up_i128(a.yy, o);
        if (lane >= o) mom_add(a, b);
    }
}

// a 128-bit integer rounded to the nearest float (ties to even): the top 64 bits with a
// sticky bit for the rest round like the whole value
__device__ __forceinline__ float i128_to_float(i128 v) {
    const bool neg = v < 0;
    const u128 u = neg ? (u128)0 - (u128)v : (u128)v;
    const unsigned long long hi = (unsigned long long)(u >> 64);
    float f;
    if (!hi) {
        f = __ull2float_rn((unsigned long long)u);
    } else {
        const int sh = 64 - __clzll((long long)hi);
        const unsigned long long t =
            (unsigned long long)(u >> sh) | (unsigned long long)((u & (((u128)1 << sh) - 1)) != 0);
        f = __fmul_rn(__ull2float_rn(t), ldexpf(1.0f, sh));
    }
    return neg ? -f : f;
}

// the exclusive prefix at slot s: six columns of `stride` 128-bit values
__device__ __forceinline__ i128 ld_i128(const i128* p) {
    const ulonglong2 v = __ldcg(reinterpret_cast<const ulonglong2*>(p));
    return (i128)(((u128)v.y << 64) | v.x);
}
__device__ __forceinline__ MomSums mom_load(const i128* prefix, size_t stride, uint32_t s) {
    MomSums a;
    a.m = ld_i128(prefix + s);
    a.x = ld_i128(prefix + stride + s);
    a.y = ld_i128(prefix + 2 * stride + s);
    a.xx = ld_i128(prefix + 3 * stride + s);
    a.xy = ld_i128(prefix + 4 * stride + s);
    a.yy = ld_i128(prefix + 5 * stride + s);
    return a;
}
__device__ __forceinline__ void mom_store(i128* prefix, size_t stride, uint32_t s, const MomSums& a) {
    prefix[s] = a.m;
    prefix[stride + s] = a.x;
    prefix[2 * stride + s] = a.y;
    prefix[3 * stride + s] = a.xx;
    prefix[4 * stride + s] = a.xy;
    prefix[5 * stride + s] = a.yy;
}
__device__ __forceinline__ MomSums mom_ldcg(const MomSums* p) {
    MomSums a;
    const i128* q = &p->m;
    a.m = ld_i128(q);
    a.x = ld_i128(q + 1);
    a.y = ld_i128(q + 2);
    a.xx = ld_i128(q + 3);
    a.xy = ld_i128(q + 4);
    a.yy = ld_i128(q + 5);
    return a;
}

// centre, mass and second central moments of the node whose sums are hi - lo
__device__ __forceinline__ void mom_node(const MomSums& hi, const MomSums& lo, const MomScale& sc, float& cx,
                                         float& cy, float& m, float4& q) {
    const i128 am = hi.m - lo.m, ax = hi.x - lo.x, ay = hi.y - lo.y;
    if (am == 0) {
        cx = cy = m = 0.0f;
        q = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return;
    }
    const float mf = i128_to_float(am);
    const float cxq = __fdiv_rn(i128_to_float(ax), mf), cyq = __fdiv_rn(i128_to_float(ay), mf);
    cx = __fadd_rn(sc.bx, __fmul_rn(cxq, sc.iqs));
    cy = __fadd_rn(sc.by, __fmul_rn(cyq, sc.iqs));
    m = __fmul_rn(mf, sc.ims);
    const int x0 = (int)rintf(cxq), y0 = (int)rintf(cyq);  // |.| <= 2^30: a mean of clamped values
    const i128 dx = ax - mul_i128_i32(am, x0), dy = ay - mul_i128_i32(am, y0);
    const i128 sxx = (hi.xx - lo.xx) - mul_i128_i32(ax + dx, x0);
    const i128 sxy = (hi.xy - lo.xy) - mul_i128_i32(ay, x0) - mul_i128_i32(dx, y0);
    const i128 syy = (hi.yy - lo.yy) - mul_i128_i32(ay + dy, y0);
    const float dxf = i128_to_float(dx), dyf = i128_to_float(dy);
    const float ux = __fdiv_rn(dxf, mf), uy = __fdiv_rn(dyf, mf);
    const float qxx = __fsub_rn(i128_to_float(sxx), __fmul_rn(dxf, ux));
    const float qxy = __fsub_rn(i128_to_float(sxy), __fmul_rn(dxf, uy));
    const float qyy = __fsub_rn(i128_to_float(syy), __fmul_rn(dyf, uy));
    const float s2 = __fmul_rn(sc.iqs, sc.iqs);
    q = make_float4(__fmul_rn(__fmul_rn(qxx, s2), sc.ims), __fmul_rn(__fmul_rn(qxy, s2), sc.ims),
                    __fmul_rn(__fmul_rn(qyy, s2), sc.ims), 0.0f);
}

}  // namespace
}  // namespace gsim
