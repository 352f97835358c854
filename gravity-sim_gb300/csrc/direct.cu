// direct.cu -- O(N^2) direct-sum force with the integrator fused into the epilogue.
//
// Replaces src/Simulation/Direct/Shaders/SimShader.comp:37-74 (one dispatch per step,
// src/Simulation/Direct/DirectSimulation.cpp:306-319).
//
// FAST mode (k_direct_fast): each block owns an i-tile of 128*IPT particles and one
// j-chunk; j is staged 64 at a time in shared memory as float4 {x, y, m, 0} (loaded as
// float4 pairs of positions and float2 pairs of masses: j-tiles start at multiples of 64)
// and broadcast to all threads; every thread keeps IPT targets in registers.  Each 64-wide
// tile is summed plainly in FP32, and the tile partials are added with Kahan
// compensation.  When the j-range is split over several blocks (small N, to fill 152
// SMs), every block stores its compensated partial and the last block to finish an
// i-tile (ticket counter, no waiting) combines the chunks in chunk order, again with
// Kahan, and applies the integrator.  Results do not depend on block scheduling.
//
// REFERENCE mode (k_direct_ref): one thread per particle, j ascending over all N_al
// particles, plain FP32 accumulation and correctly rounded 1/sqrt -- the shader's order,
// bit-identical to the CPU restatement.
//
// Roofline: 14 algorithmic FLOP per pair (2 sub, 2 FMA for r^2, rsqrt, 3 mul, 2 FMA),
// 9 FP32 operations + 1 MUFU per pair, issued as packed f32x2 instructions for a thread's
// two targets (4.5 issues + 1 MUFU per pair); FP32-bound.
#include "internal.cuh"

namespace gsim {
namespace {

constexpr int kDirectBlock = 128;
constexpr int kDirectTileJ = 64;
constexpr int kDirectIpt = 2;  // default targets per thread (gs_shape.direct_targets: 2 or 4), in packed f32x2 pairs

// Block (bx, by) of a system: i-tile bx, j-chunk by.  A plain launch passes blockIdx.x /
// blockIdx.y, a batched launch the block's position inside its system's grid.  KAHAN
// false (GS_FLAG_PLAIN_SUM) adds the tile partials and the chunks plainly, for the
// precision study against the compensated sums.
template <int IPT, bool KAHAN>
__device__ __forceinline__ void direct_fast_body(uint32_t bx, uint32_t by, const float2* __restrict__ pos,
                                                 const float2* __restrict__ vel, const float* __restrict__ mass,
                                                 float2* __restrict__ pos_out, float2* __restrict__ vel_out,
                                                 float2* __restrict__ acc_rec, uint32_t n_al, int chunks,
                                                 uint32_t jchunk, float eps2, float k, float hdt,
                                                 float4* __restrict__ partials, uint32_t* __restrict__ tickets) {
    __shared__ float4 sj[kDirectTileJ];
    __shared__ uint32_t s_ticket;
    const int t = threadIdx.x;
    const uint32_t tile_base = bx * (kDirectBlock * IPT);
    const uint32_t j0 = by * jchunk;
    const uint32_t j1 = min(j0 + jchunk, n_al);

    static_assert(IPT % 2 == 0, "targets per thread come in packed f32x2 pairs");
    float px[IPT], py[IPT], sx[IPT], sy[IPT], cx[IPT], cy[IPT];
#pragma unroll
    for (int r = 0; r < IPT; ++r) {
        uint32_t i = tile_base + t + r * kDirectBlock;
        float2 p = i < n_al ? pos[i] : make_float2(0.f, 0.f);
        px[r] = p.x;
        py[r] = p.y;
        sx[r] = sy[r] = cx[r] = cy[r] = 0.f;
    }
    constexpr int NP = IPT / 2;
    float2 P2[NP], Q2[NP];
#pragma unroll
    for (int h = 0; h < NP; ++h) {
        P2[h] = make_float2(px[2 * h], px[2 * h + 1]);
        Q2[h] = make_float2(py[2 * h], py[2 * h + 1]);
    }
    const float2 E2 = make_float2(eps2, eps2);

    for (uint32_t jt = j0; jt < j1; jt += kDirectTileJ) {
        __syncthreads();
        if (t < kDirectTileJ / 2) {  // one float4 of two positions and one float2 of their masses per thread
            const float4 q = reinterpret_cast<const float4*>(pos)[(jt >> 1) + t];
            const float2 m = reinterpret_cast<const float2*>(mass)[(jt >> 1) + t];
            sj[2 * t] = make_float4(q.x, q.y, m.x, 0.f);
            sj[2 * t + 1] = make_float4(q.z, q.w, m.y, 0.f);
        }
        __syncthreads();
        // Pairs of the thread's targets share packed f32x2 instructions (each lane rounds
        // like the scalar one, in the same order: dx, dy, d2 = fma(dx, dx, fma(dy, dy,
        // eps2)), s = ((m r) r) r, t += d s), so the bits are those of scalar evaluations.
        float2 tx2[NP], ty2[NP];
#pragma unroll
        for (int h = 0; h < NP; ++h) tx2[h] = ty2[h] = make_float2(0.f, 0.f);
#pragma unroll 16
        for (int jj = 0; jj < kDirectTileJ; ++jj) {
            const float4 q = sj[jj];
#pragma unroll
            for (int h = 0; h < NP; ++h) {
                const float2 dx = sub2(make_float2(q.x, q.x), P2[h]), dy = sub2(make_float2(q.y, q.y), Q2[h]);
                const float2 d2 = fma2(dx, dx, fma2(dy, dy, E2));
                const float2 rr = make_float2(rsqrtf(d2.x), rsqrtf(d2.y));
                const float2 s = mul2(mul2(mul2(make_float2(q.z, q.z), rr), rr), rr);
                tx2[h] = fma2(dx, s, tx2[h]);
                ty2[h] = fma2(dy, s, ty2[h]);
            }
        }
        float tx[IPT], ty[IPT];
#pragma unroll
        for (int h = 0; h < NP; ++h) {
            tx[2 * h] = tx2[h].x;
            tx[2 * h + 1] = tx2[h].y;
            ty[2 * h] = ty2[h].x;
            ty[2 * h + 1] = ty2[h].y;
        }
#pragma unroll
        for (int r = 0; r < IPT; ++r) {  // Kahan-compensated add of the tile partial
            if (!KAHAN) {
                sx[r] += tx[r];
                sy[r] += ty[r];
                continue;
            }
            float y = tx[r] - cx[r];
            float u = sx[r] + y;
            cx[r] = (u - sx[r]) - y;
            sx[r] = u;
            y = ty[r] - cy[r];
            u = sy[r] + y;
            cy[r] = (u - sy[r]) - y;
            sy[r] = u;
        }
    }

    if (chunks > 1) {
#pragma unroll
        for (int r = 0; r < IPT; ++r) {
            uint32_t i = tile_base + t + r * kDirectBlock;
            if (i < n_al) partials[(size_t)by * n_al + i] = make_float4(sx[r], sy[r], cx[r], cy[r]);
        }
        __threadfence();
        __syncthreads();
        if (t == 0) s_ticket = atomicAdd(&tickets[bx], 1u);
        __syncthreads();
        if (s_ticket != (uint32_t)chunks - 1) return;
        __threadfence();
#pragma unroll
        for (int r = 0; r < IPT; ++r) {
            uint32_t i = tile_base + t + r * kDirectBlock;
            float ax = 0.f, ay = 0.f, kx = 0.f, ky = 0.f;
            if (i < n_al) {
                for (int c = 0; c < chunks; ++c) {
                    float4 q = __ldcg(&partials[(size_t)c * n_al + i]);
                    if (!KAHAN) {
                        ax += q.x;
                        ay += q.y;
                        continue;
                    }
                    float y = (q.x - q.z) - kx;
                    float u = ax + y;
                    kx = (u - ax) - y;
                    ax = u;
                    y = (q.y - q.w) - ky;
                    u = ay + y;
                    ky = (u - ay) - y;
                    ay = u;
                }
            }
            sx[r] = ax;
            cx[r] = kx;
            sy[r] = ay;
            cy[r] = ky;
        }
        if (t == 0) tickets[bx] = 0u;  // ready for the next step
    }

#pragma unroll
    for (int r = 0; r < IPT; ++r) {
        uint32_t i = tile_base + t + r * kDirectBlock;
        if (i >= n_al) continue;
        float ax = sx[r] - cx[r], ay = sy[r] - cy[r];
        if (acc_rec) acc_rec[i] = make_float2(ax, ay);
        float2 v = vel[i];
        float nvx = fmaf(ax, k, v.x), nvy = fmaf(ay, k, v.y);  // SimShader.comp:68
        pos_out[i] = make_float2(fmaf(v.x + nvx, hdt, px[r]), fmaf(v.y + nvy, hdt, py[r]));  // :69
        vel_out[i] = make_float2(nvx, nvy);
    }
}

__device__ __forceinline__ void direct_ref_body(uint32_t bx, const float2* __restrict__ pos,
                                                const float2* __restrict__ vel, const float* __restrict__ mass,
                                                float2* __restrict__ pos_out, float2* __restrict__ vel_out,
                                                float2* __restrict__ acc_rec, uint32_t n_al, float eps2, float k,
                                                float hdt) {
    __shared__ float2 sp[64];
    __shared__ float sm[64];
    const uint32_t i = bx * 64 + threadIdx.x;
    const float2 p = pos[i];
    float ax = 0.f, ay = 0.f;
    for (uint32_t jt = 0; jt < n_al; jt += 64) {  // SimShader.comp:43-65
        sp[threadIdx.x] = pos[jt + threadIdx.x];
        sm[threadIdx.x] = mass[jt + threadIdx.x];
        __syncthreads();
        for (int jj = 0; jj < 64; ++jj) {
            float dx = sp[jj].x - p.x;
            float dy = sp[jj].y - p.y;
            float d2 = fmaf(dx, dx, fmaf(dy, dy, eps2));
            float r = __fdiv_rn(1.0f, __fsqrt_rn(d2));
            float s = ((sm[jj] * r) * r) * r;
            ax = fmaf(dx, s, ax);
            ay = fmaf(dy, s, ay);
        }
        __syncthreads();
    }
    if (acc_rec) acc_rec[i] = make_float2(ax, ay);
    float2 v = vel[i];
    float nvx = fmaf(ax, k, v.x), nvy = fmaf(ay, k, v.y);
    pos_out[i] = make_float2(fmaf(v.x + nvx, hdt, p.x), fmaf(v.y + nvy, hdt, p.y));
    vel_out[i] = make_float2(nvx, nvy);
}

template <int IPT, bool KAHAN>
__global__ void __launch_bounds__(kDirectBlock)
k_direct_fast(const float2* __restrict__ pos, const float2* __restrict__ vel, const float* __restrict__ mass,
              float2* __restrict__ pos_out, float2* __restrict__ vel_out, float2* __restrict__ acc_rec,
              uint32_t n_al, int chunks, uint32_t jchunk, float eps2, float k, float hdt,
              float4* __restrict__ partials, uint32_t* __restrict__ tickets) {
    direct_fast_body<IPT, KAHAN>(blockIdx.x, blockIdx.y, pos, vel, mass, pos_out, vel_out, acc_rec, n_al, chunks, jchunk,
                          eps2, k, hdt, partials, tickets);
}

__global__ void __launch_bounds__(64)
k_direct_ref(const float2* __restrict__ pos, const float2* __restrict__ vel, const float* __restrict__ mass,
             float2* __restrict__ pos_out, float2* __restrict__ vel_out, float2* __restrict__ acc_rec,
             uint32_t n_al, float eps2, float k, float hdt) {
    direct_ref_body(blockIdx.x, pos, vel, mass, pos_out, vel_out, acc_rec, n_al, eps2, k, hdt);
}

// Batched direct sum: one launch over every direct-sum system of a plan.  Block b belongs
// to the system whose table range holds it; inside the system it is block (b mod i-tiles,
// b div i-tiles) of the plain grid, so each system sums in the plain order.
__device__ __forceinline__ uint32_t direct_batch_sys(const uint32_t* __restrict__ first, uint32_t nsys,
                                                     uint32_t b) {
    uint32_t lo = 0, hi = nsys;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&first[mid]) <= b) lo = mid;
        else hi = mid;
    }
    return lo;
}

template <bool EXACT, bool KAHAN, int IPT>
__global__ void __launch_bounds__(EXACT ? 64 : kDirectBlock)
kb_direct(const SysDesc* __restrict__ descs, const uint32_t* __restrict__ first, uint32_t nsys, uint32_t step) {
    const uint32_t s = direct_batch_sys(first, nsys, blockIdx.x);
    const SysDesc& d = descs[s];
    const uint32_t b = blockIdx.x - __ldg(&first[s]);
    const int in = (int)((d.parity + step) & 1u), out = in ^ 1;
    if (EXACT)
        direct_ref_body(b, d.pos[in], d.vel[in], d.mass[in], d.pos[out], d.vel[out], d.acc, d.n_al, d.eps2, d.k,
                        d.hdt);
    else
        direct_fast_body<IPT, KAHAN>(b % d.itiles, b / d.itiles, d.pos[in], d.vel[in], d.mass[in], d.pos[out], d.vel[out],
                            d.acc, d.n_al, (int)d.chunks, d.jchunk, d.eps2, d.k, d.hdt, d.partials, d.tickets);
}

__global__ void __launch_bounds__(256)
k_accel_f64(const uint32_t* __restrict__ targets, const float2* __restrict__ pos,
            const float* __restrict__ mass, uint32_t n, double eps2, double2* __restrict__ out) {
    __shared__ double sx[256], sy[256];
    const uint32_t i = targets[blockIdx.x];
    const double px = pos[i].x, py = pos[i].y;
    double ax = 0.0, ay = 0.0;
    for (uint32_t j = threadIdx.x; j < n; j += 256) {
        double dx = (double)pos[j].x - px, dy = (double)pos[j].y - py;
        double d2 = dx * dx + dy * dy + eps2;
        double s = (double)mass[j] / (d2 * sqrt(d2));
        ax += dx * s;
        ay += dy * s;
    }
    sx[threadIdx.x] = ax;
    sy[threadIdx.x] = ay;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            sx[threadIdx.x] += sx[threadIdx.x + w];
            sy[threadIdx.x] += sy[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = make_double2(sx[0], sy[0]);
}

// Energy in FP64 (diagnostic, not on the step path): per block of 256 particles i, the
// kinetic energy 1/2 m |v|^2 and m_i * sum_{j != i} m_j / sqrt(|p_j - p_i|^2 + eps^2), the
// latter over j tiles staged in shared memory; block sums in a fixed tree order.
__global__ void __launch_bounds__(256)
k_energy_f64(const float2* __restrict__ pos, const float2* __restrict__ vel, const float* __restrict__ mass,
             uint32_t n, double eps2, double2* __restrict__ part) {
    __shared__ double sx[256], sy[256], sm[256];
    const uint32_t t = threadIdx.x, i = blockIdx.x * 256 + t;
    const bool own = i < n;
    const double px = own ? (double)pos[i].x : 0.0, py = own ? (double)pos[i].y : 0.0;
    const double mi = own ? (double)mass[i] : 0.0;
    double pot = 0.0;
    for (uint32_t jt = 0; jt < n; jt += 256) {
        const uint32_t j = jt + t;
        sx[t] = j < n ? (double)pos[j].x : 0.0;
        sy[t] = j < n ? (double)pos[j].y : 0.0;
        sm[t] = j < n ? (double)mass[j] : 0.0;
        __syncthreads();
        for (uint32_t jj = 0; jj < 256; ++jj) {
            if (jt + jj == i) continue;
            const double dx = sx[jj] - px, dy = sy[jj] - py;
            pot += sm[jj] / sqrt(dx * dx + dy * dy + eps2);
        }
        __syncthreads();
    }
    const double vx = own ? (double)vel[i].x : 0.0, vy = own ? (double)vel[i].y : 0.0;
    sx[t] = 0.5 * mi * (vx * vx + vy * vy);
    sy[t] = mi * pot;
    __syncthreads();
    for (uint32_t w = 128; w > 0; w >>= 1) {
        if (t < w) {
            sx[t] += sx[t + w];
            sy[t] += sy[t + w];
        }
        __syncthreads();
    }
    if (t == 0) part[blockIdx.x] = make_double2(sx[0], sy[0]);
}

}  // namespace

gs_status energy_f64(gs_sim* s, double* kinetic, double* potential) {
    const uint32_t n = (uint32_t)s->n_al;
    const uint32_t blocks = (n + 255) / 256;
    double2* part = nullptr;
    GS_CUDA(cudaMallocAsync(&part, blocks * sizeof(double2), s->stream));
    k_energy_f64<<<blocks, 256, 0, s->stream>>>(s->pos[s->in], s->vel[s->in], s->mass[s->in], n, (double)s->eps2,
                                                 part);
    double2* host = new double2[blocks];
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(host, part, blocks * sizeof(double2), cudaMemcpyDeviceToHost, s->stream);
    cudaFreeAsync(part, s->stream);
    gs_status w = e == cudaSuccess ? sim_wait(s) : cuda_fail(e, "energy_f64");
    if (w != GS_OK) {  // the readback may still be pending: keep its destination alive
        if (w != GS_ERR_TIMEOUT) delete[] host;
        return w;
    }
    double ke = 0.0, pp = 0.0;
    for (uint32_t b = 0; b < blocks; ++b) {
        ke += host[b].x;
        pp += host[b].y;
    }
    delete[] host;
    *kinetic = ke;
    *potential = -0.5 * (double)s->G * pp;  // every pair was counted from both ends
    return GS_OK;
}

// j-chunks of a plain launch: enough blocks for blocks_per_sm on every SM, at least 256
// sources per chunk, at most 64 chunks
static int pick_chunks(uint64_t n_al, int ipt, uint32_t blocks_per_sm) {
    const uint64_t itiles = (n_al + kDirectBlock * ipt - 1) / (kDirectBlock * ipt);
    const uint64_t want_blocks = 152ull * blocks_per_sm;
    uint64_t c = (want_blocks + itiles - 1) / itiles;
    uint64_t max_c = n_al / 256;  // keep at least 256 sources per chunk
    if (c > max_c) c = max_c;
    if (c < 1) c = 1;
    if (c > 64) c = 64;
    return (int)c;
}

static int shape_ipt(const gs_shape& sh) { return sh.direct_targets == 4 ? 4 : 2; }

// Lays the j-chunk partials and tickets out in the system's slab (sizing pass: counts):
// for the chunks of the creation shape with either targets-per-thread value, tickets for
// the most i-tiles (2 targets per thread).
void direct_carve(gs_sim* s) {
    DirectWork& w = s->dw;
    w.ipt = shape_ipt(s->shape);
    w.block = kDirectBlock;
    const int c2 = pick_chunks(s->n_al, 2, s->shape.direct_blocks_per_sm);
    const int c4 = pick_chunks(s->n_al, 4, s->shape.direct_blocks_per_sm);
    s->direct_max_chunks = (uint32_t)(c2 > c4 ? c2 : c4);
    w.partials = nullptr;
    w.tickets = nullptr;
    if (s->direct_max_chunks > 1) {
        const uint64_t itiles = (s->n_al + kDirectBlock * 2 - 1) / (kDirectBlock * 2);
        sim_carve(s, (void**)&w.partials, sizeof(float4) * s->n_al * (size_t)s->direct_max_chunks);
        sim_carve(s, (void**)&w.tickets, sizeof(uint32_t) * itiles);
    }
}

uint32_t direct_chunks_needed(const gs_sim* s, const gs_shape& sh) {
    return (uint32_t)pick_chunks(s->n_al, shape_ipt(sh), sh.direct_blocks_per_sm);
}

cudaError_t direct_init(gs_sim* s) {
    const DirectWork& w = s->dw;
    if (!w.tickets) return cudaSuccess;
    const uint64_t itiles = (s->n_al + kDirectBlock * 2 - 1) / (kDirectBlock * 2);
    return cudaMemsetAsync(w.tickets, 0, sizeof(uint32_t) * itiles, s->stream);
}

// Grid of k_direct_fast for `ipt` targets per thread: i-tiles x j-chunks, each chunk a
// multiple of 64 sources.  The chunks come from the system's own shape, so a system sums
// in the same order whichever targets per thread run it (alone or in a batch).
static void direct_grid(const gs_sim* s, int ipt, uint32_t& itiles, uint32_t& jchunk, uint32_t& chunks) {
    const uint32_t n_al = (uint32_t)s->n_al;
    const uint32_t c = direct_chunks_needed(s, s->shape);
    itiles = (n_al + kDirectBlock * ipt - 1) / (kDirectBlock * ipt);
    jchunk = (n_al + c - 1) / c;
    jchunk = (jchunk + kDirectTileJ - 1) / kDirectTileJ * kDirectTileJ;
    chunks = (n_al + jchunk - 1) / jchunk;
}

cudaError_t direct_step(gs_sim* s, int in, int out, bool profile) {
    const float k = s->dt_eff * s->G;  // SimShader.comp:68 (SIMULATION_TIME * GRAVITATIONAL_CONST)
    const float hdt = 0.5f * s->dt_eff;
    const uint32_t n_al = (uint32_t)s->n_al;
    stage_begin(s, kStageDirect, profile);
    if (s->p.math_mode == GS_MATH_REFERENCE) {
        k_direct_ref<<<n_al / 64, 64, 0, s->stream>>>(s->pos[in], s->vel[in], s->mass[in], s->pos[out],
                                                       s->vel[out], s->acc, n_al, s->eps2, k, hdt);
    } else {
        DirectWork& w = s->dw;
        const int ipt = shape_ipt(s->shape);
        uint32_t itiles, jchunk, chunks;
        direct_grid(s, ipt, itiles, jchunk, chunks);
        dim3 grid(itiles, chunks);
        const bool plain = (s->p.flags & GS_FLAG_PLAIN_SUM) != 0;
        auto fn = ipt == 4 ? (plain ? k_direct_fast<4, false> : k_direct_fast<4, true>)
                           : (plain ? k_direct_fast<2, false> : k_direct_fast<2, true>);
        fn<<<grid, kDirectBlock, 0, s->stream>>>(s->pos[in], s->vel[in], s->mass[in], s->pos[out], s->vel[out],
                                                  s->acc, n_al, (int)chunks, jchunk, s->eps2, k, hdt, w.partials,
                                                  w.tickets);
    }
    count_launch(s);
    stage_end(s, kStageDirect, profile);
    return cudaGetLastError();
}

void direct_batch_desc(gs_sim* s, SysDesc& d, uint32_t blocks[kTabCount], const gs_shape& batch_shape) {
    for (int t = 0; t < kTabCount; ++t) blocks[t] = 0;
    uint32_t itiles, jchunk, chunks;
    direct_grid(s, shape_ipt(batch_shape), itiles, jchunk, chunks);
    d.itiles = itiles;
    d.jchunk = jchunk;
    d.chunks = chunks;
    d.partials = s->dw.partials;
    d.tickets = s->dw.tickets;
    blocks[kTabDirect] = s->p.math_mode == GS_MATH_REFERENCE ? (uint32_t)(s->n_al / 64) : itiles * chunks;
}

cudaError_t direct_batch_step(const BatchPlan& p, uint32_t step, cudaStream_t st) {
    if (!p.n_direct) return cudaSuccess;
    const SysDesc* descs = p.d_descs + p.n_bh;
    const bool four = shape_ipt(p.shape) == 4;
    if (p.direct_exact)
        kb_direct<true, false, 2><<<p.total[kTabDirect], 64, 0, st>>>(descs, p.d_tab[kTabDirect], p.n_direct, step);
    else
        (p.direct_plain ? (four ? kb_direct<false, false, 4> : kb_direct<false, false, 2>)
                        : (four ? kb_direct<false, true, 4> : kb_direct<false, true, 2>))
            <<<p.total[kTabDirect], kDirectBlock, 0, st>>>(descs, p.d_tab[kTabDirect], p.n_direct, step);
    return cudaGetLastError();
}

cudaError_t accel_f64(gs_sim* s, uint32_t n_targets, const uint32_t* d_targets, double2* d_out) {
    const double eps2 = (double)s->eps2;  // the softening the FP32 path uses, exactly
    k_accel_f64<<<n_targets, 256, 0, s->stream>>>(d_targets, s->pos[s->in], s->mass[s->in],
                                                  (uint32_t)s->n_al, eps2, d_out);
    return cudaGetLastError();
}

}  // namespace gsim

// ------------------------------------------------------------------------------------
// Direct-sum step that allocates nothing (gs_direct_step_noalloc).
//
// Some callers cannot let a library allocate device memory: a host application that owns
// every device allocation and hands its plugins fixed buffers, or a loop with a fixed
// memory budget that must not pay for (or be synchronised by) cudaMalloc / cudaFree in
// the middle of a run.  For them this entry point takes the particle buffers from the
// caller and keeps its own scratch -- the j-chunk partial sums and the per-tile tickets
// of k_direct_fast -- in the file-scope device arrays below.  Those arrays exist on every
// GPU that loads this library and stay allocated until the process exits.
// ------------------------------------------------------------------------------------
namespace gsim {
namespace {

constexpr size_t kNoAllocPartialBytes = 4u << 20;  // j-chunk partials, 4 MiB
constexpr uint32_t kNoAllocMaxTiles = GS_NOALLOC_MAX_PARTICLES / (kDirectBlock * 2);

static __device__ __align__(256) float4 g_noalloc_partials[kNoAllocPartialBytes / sizeof(float4)];
static __device__ __align__(256) uint32_t g_noalloc_tickets[kNoAllocMaxTiles];

// Device addresses of the two arrays in the current context, looked up on every call:
// the lookup allocates nothing and is cheap, and a cached address could outlive the
// module it points into (cudaDeviceReset, or another context on the same ordinal).  The
// host-side names are stand-ins, not device addresses, so they are never passed to a
// kernel directly.
gs_status noalloc_scratch(float4** partials, uint32_t** tickets) {
    void* p = nullptr;
    void* t = nullptr;
    GS_CUDA(cudaGetSymbolAddress(&p, g_noalloc_partials));
    GS_CUDA(cudaGetSymbolAddress(&t, g_noalloc_tickets));
    *partials = (float4*)p;
    *tickets = (uint32_t*)t;
    return GS_OK;
}

}  // namespace
}  // namespace gsim

extern "C" gs_status gs_direct_step_noalloc(const float* d_pos_in, const float* d_vel_in, const float* d_mass,
                                            float* d_pos_out, float* d_vel_out, uint64_t n,
                                            float gravitational_const, float simulation_time, float softening_len,
                                            void* stream) {
    using namespace gsim;
    if (!d_pos_in || !d_vel_in || !d_mass || !d_pos_out || !d_vel_out) {
        set_error("gs_direct_step_noalloc: NULL buffer");
        return GS_ERR_INVALID_ARGUMENT;
    }
    if (n == 0 || n % kAlignment != 0) {
        set_error("gs_direct_step_noalloc: the particle count must be a positive multiple of 64 "
                  "(pad with zero-mass particles, as ParticleSystem does)");
        return GS_ERR_INVALID_ARGUMENT;
    }
    if (((uintptr_t)d_pos_in & 15u) || ((uintptr_t)d_mass & 7u) || ((uintptr_t)d_vel_in & 7u) ||
        ((uintptr_t)d_pos_out & 7u) || ((uintptr_t)d_vel_out & 7u)) {
        set_error("gs_direct_step_noalloc: pos_in must be 16-byte aligned and the other arrays 8-byte aligned "
                  "(the kernel reads positions as float4 pairs)");
        return GS_ERR_INVALID_ARGUMENT;
    }
    if (n > GS_NOALLOC_MAX_PARTICLES) {
        set_error("gs_direct_step_noalloc: particle count above GS_NOALLOC_MAX_PARTICLES (65536), the size "
                  "of its built-in scratch; use gs_create / gs_run for larger systems");
        return GS_ERR_CAPACITY;
    }
    float4* partials = nullptr;
    uint32_t* tickets = nullptr;
    gs_status st = noalloc_scratch(&partials, &tickets);
    if (st != GS_OK) return st;

    const uint32_t n_al = (uint32_t)n;
    const uint32_t itiles = (n_al + kDirectBlock * kDirectIpt - 1) / (kDirectBlock * kDirectIpt);
    int chunks = pick_chunks(n_al, kDirectIpt, 12);
    const int fit = (int)(kNoAllocPartialBytes / (sizeof(float4) * n_al));  // >= 4 for n <= 65536
    if (chunks > fit) chunks = fit;
    uint32_t jchunk = (n_al + chunks - 1) / chunks;
    jchunk = (jchunk + kDirectTileJ - 1) / kDirectTileJ * kDirectTileJ;
    chunks = (int)((n_al + jchunk - 1) / jchunk);
    cudaStream_t s = (cudaStream_t)stream;
    // the tickets must start at zero; the array keeps whatever the previous call left
    if (chunks > 1) GS_CUDA(cudaMemsetAsync(tickets, 0, itiles * sizeof(uint32_t), s));
    const float eps2 = softening_len * softening_len;
    const float k = simulation_time * gravitational_const;
    const float hdt = 0.5f * simulation_time;
    k_direct_fast<kDirectIpt, true><<<dim3(itiles, chunks), kDirectBlock, 0, s>>>(
        (const float2*)d_pos_in, (const float2*)d_vel_in, d_mass, (float2*)d_pos_out, (float2*)d_vel_out, nullptr,
        n_al, chunks, jchunk, eps2, k, hdt, partials, tickets);
    GS_CUDA(cudaGetLastError());
    return GS_OK;
}
