// batch.cu -- many independent systems advanced together (gs_batch_*), and the
// direct-sum / Barnes-Hut crossover tuner (gs_tune_crossover).
//
// The reference runs one system per process (src/Main.cpp:250-321).  A batch runs every
// stage of the step as one launch over all of its systems: the Barnes-Hut stages of
// bh.cu (bh_batch_step) on the batch's stream, and the direct-sum kernel of direct.cu
// (direct_batch_step) beside them on a second stream.  Each block finds its system in a
// per-stage table of block prefixes (BatchPlan); the per-system work is the plain path's,
// so results are bit-identical to gs_run.  The step is captured once per ping-pong
// parity into a CUDA graph, so a step costs one graph launch whatever the member count.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "internal.cuh"

using namespace gsim;

struct gs_batch {
    std::vector<gs_sim*> sims;   // caller order
    std::vector<gs_sim*> order;  // plan order: Barnes-Hut largest first, then direct sum
    int device = 0;
    uint32_t flags = 0;
    cudaStream_t root = nullptr, side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr, done = nullptr;
    std::vector<cudaEvent_t> member_ev;  // orders the batch after each member's own work
    BatchPlan plan;
    void* d_block = nullptr;  // descriptors | tables | work counters
    size_t d_block_bytes = 0;
    std::vector<int> parity0;  // each member's compute-input set when the plan was built
    uint64_t step = 0;         // batched steps since then
    bool planned = false;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    bool pending = false;
};

namespace {

gs_status fail(const char* msg) {
    set_error(msg);
    return GS_ERR_INVALID_ARGUMENT;
}

void drop_graphs(gs_batch* b) {
    for (auto& g : b->graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
}

void free_batch(gs_batch* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->root) cudaStreamSynchronize(b->root);
    if (b->side) cudaStreamSynchronize(b->side);
    drop_graphs(b);
    for (auto e : b->member_ev)
        if (e) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->join) cudaEventDestroy(b->join);
    if (b->done) cudaEventDestroy(b->done);
    if (b->root) cudaStreamDestroy(b->root);
    if (b->side) cudaStreamDestroy(b->side);
    cudaFree(b->d_block);
    delete b;
}

constexpr uint32_t kBHFlagMask = GS_FLAG_QUADRUPOLE | GS_FLAG_SAFE_RADIUS | GS_FLAG_GROUP_WALK |
                                 GS_FLAG_COUNT_INTERACTIONS;

gs_status check_members(gs_sim* const* sims, uint32_t count) {
    const gs_sim* bh0 = nullptr;
    const gs_sim* dir0 = nullptr;
    for (uint32_t i = 0; i < count; ++i) {
        const gs_sim* s = sims[i];
        if (!s) return fail("gs_batch_create: NULL system");
        if (s->device != sims[0]->device) return fail("gs_batch_create: all systems must live on one device");
        for (uint32_t j = 0; j < i; ++j)
            if (sims[j] == s) return fail("gs_batch_create: a system appears twice");
        if (s->p.algorithm == GS_BARNES_HUT) {
            if (!bh0) bh0 = s;
            else if (s->p.box_mode != bh0->p.box_mode || s->p.math_mode != bh0->p.math_mode ||
                     (s->p.flags & kBHFlagMask) != (bh0->p.flags & kBHFlagMask))
                return fail("gs_batch_create: Barnes-Hut systems must share box_mode, math_mode and the "
                            "QUADRUPOLE / SAFE_RADIUS / GROUP_WALK / COUNT_INTERACTIONS flags");
        } else {
            if (!dir0) dir0 = s;
            else if (s->p.math_mode != dir0->p.math_mode)
                return fail("gs_batch_create: direct-sum systems must share math_mode");
        }
    }
    return GS_OK;
}

// Descriptors, block tables and launch shapes for the current member states.
gs_status build_plan(gs_batch* b) {
    BatchPlan& p = b->plan;
    const size_t n = b->order.size();
    std::vector<SysDesc> descs(n);
    std::vector<std::vector<uint32_t>> blocks(n, std::vector<uint32_t>(kTabCount, 0));
    p.n_bh = p.n_direct = 0;
    b->parity0.assign(n, 0);
    for (size_t i = 0; i < n; ++i) {
        gs_sim* s = b->order[i];
        SysDesc& d = descs[i];
        std::memset(&d, 0, sizeof d);
        for (int t = 0; t < 2; ++t) {
            d.pos[t] = s->pos[t];
            d.vel[t] = s->vel[t];
            d.mass[t] = s->mass[t];
        }
        d.acc = s->acc;
        d.err = s->d_err;
        d.n_al = (uint32_t)s->n_al;
        d.parity = (uint32_t)s->in;
        d.eps2 = s->eps2;
        d.theta2 = s->theta2;
        d.k = s->G * s->dt_eff;  // the factor of both integrators (ForceShader.comp:145, SimShader.comp:68)
        d.hdt = 0.5f * s->dt_eff;
        b->parity0[i] = s->in;
        if (s->p.algorithm == GS_BARNES_HUT) {
            bh_batch_desc(s, d, blocks[i].data());
            bh_set_final_keys(s);
            ++p.n_bh;
        } else {
            direct_batch_desc(s, d, blocks[i].data());
            ++p.n_direct;
        }
    }
    // tables: Barnes-Hut stages over members [0, n_bh), the direct table over [n_bh, n)
    std::vector<uint32_t> tabs;
    size_t off[kTabCount];
    for (int t = 0; t < kTabCount; ++t) {
        const size_t lo = t == kTabDirect ? p.n_bh : 0, hi = t == kTabDirect ? n : p.n_bh;
        off[t] = tabs.size();
        uint64_t acc = 0;
        tabs.push_back(0u);
        for (size_t i = lo; i < hi; ++i) {
            acc += blocks[i][t];
            if (acc > 0x7fffffffull) return fail("gs_batch_create: too many blocks in one stage");
            tabs.push_back((uint32_t)acc);
        }
        p.total[t] = (uint32_t)acc;
    }
    const size_t desc_b = n * sizeof(SysDesc);
    const size_t tab_off = (desc_b + 255) / 256 * 256;
    const size_t work_off = (tab_off + tabs.size() * sizeof(uint32_t) + 255) / 256 * 256;
    const size_t bytes = work_off + 256;
    if (bytes > b->d_block_bytes) {
        cudaFree(b->d_block);
        b->d_block = nullptr;
        b->d_block_bytes = 0;
        GS_CUDA(cudaMalloc(&b->d_block, bytes));
        b->d_block_bytes = bytes;
    }
    char* base = (char*)b->d_block;
    GS_CUDA(cudaMemcpyAsync(base, descs.data(), desc_b, cudaMemcpyHostToDevice, b->root));
    GS_CUDA(cudaMemcpyAsync(base + tab_off, tabs.data(), tabs.size() * sizeof(uint32_t), cudaMemcpyHostToDevice,
                            b->root));
    GS_CUDA(cudaMemsetAsync(base + work_off, 0, 256, b->root));
    GS_CUDA(cudaStreamSynchronize(b->root));  // the host vectors go out of scope
    p.d_descs = (SysDesc*)base;
    for (int t = 0; t < kTabCount; ++t) p.d_tab[t] = (uint32_t*)(base + tab_off) + off[t];
    p.d_work = (uint32_t*)(base + work_off);
    const gs_sim* bh0 = p.n_bh ? b->order[0] : nullptr;
    const gs_sim* dir0 = p.n_direct ? b->order[p.n_bh] : nullptr;
    p.passes = bh0 ? bh0->bh.passes : 0;
    p.bbox = bh0 && bh0->p.box_mode == GS_BOX_BOUNDING;
    p.quad = bh0 && bh0->bh.quad != nullptr;
    p.group = bh0 && (bh0->p.flags & GS_FLAG_GROUP_WALK);
    p.exact = bh0 && bh0->p.math_mode == GS_MATH_REFERENCE;
    p.count = bh0 && (bh0->p.flags & GS_FLAG_COUNT_INTERACTIONS);
    p.direct_exact = dir0 && dir0->p.math_mode == GS_MATH_REFERENCE;
    p.force_grid = bh0 ? bh_batch_force_grid(p) : 0;
    b->step = 0;
    b->planned = true;
    drop_graphs(b);
    return GS_OK;
}

// One batched step: the Barnes-Hut stages on root, the direct-sum launch on side.
cudaError_t enqueue(gs_batch* b, uint32_t step) {
    const BatchPlan& p = b->plan;
    cudaError_t e = cudaSuccess;
    const bool both = p.n_bh && p.n_direct;
    if (both) {
        e = cudaEventRecord(b->fork, b->root);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(b->side, b->fork, 0);
    }
    if (e == cudaSuccess) e = bh_batch_step(p, step, b->root);
    if (e == cudaSuccess) e = direct_batch_step(p, step, both ? b->side : b->root);
    if (both) {
        if (e == cudaSuccess) e = cudaEventRecord(b->join, b->side);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(b->root, b->join, 0);
    }
    return e;
}

uint32_t launches_per_step(const BatchPlan& p) {
    uint32_t k = 0;
    if (p.n_bh) k += 7u + (uint32_t)p.passes + (p.bbox ? 1u : 0u);  // clear keys scan records nodes sums force
    if (p.n_direct) k += 1u;
    return k;
}

}  // namespace

extern "C" {

gs_status gs_batch_create(gs_sim* const* sims, uint32_t count, uint32_t flags, gs_batch** out) {
    if (!out) return fail("gs_batch_create: out is NULL");
    *out = nullptr;
    if (!sims || !count) return fail("gs_batch_create: empty system list");
    if (flags & ~GS_BATCH_NO_GRAPH) return fail("gs_batch_create: unknown flags");
    gs_status st = check_members(sims, count);
    if (st != GS_OK) return st;
    gs_batch* b = new (std::nothrow) gs_batch();
    if (!b) {
        set_error("gs_batch_create: host allocation failed");
        return GS_ERR_OUT_OF_MEMORY;
    }
    b->sims.assign(sims, sims + count);
    b->order = b->sims;
    std::stable_sort(b->order.begin(), b->order.end(), [](const gs_sim* x, const gs_sim* y) {
        const bool bx = x->p.algorithm == GS_BARNES_HUT, by = y->p.algorithm == GS_BARNES_HUT;
        if (bx != by) return bx;
        return x->n_al > y->n_al;
    });
    b->device = sims[0]->device;
    b->flags = flags;
    b->member_ev.assign(count, nullptr);
    cudaError_t e = cudaSetDevice(b->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->root, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
    for (uint32_t i = 0; i < count && e == cudaSuccess; ++i)
        e = cudaEventCreateWithFlags(&b->member_ev[i], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        st = cuda_fail(e, "gs_batch_create");
        free_batch(b);
        return st;
    }
    st = build_plan(b);
    if (st != GS_OK) {
        free_batch(b);
        return st;
    }
    *out = b;
    return GS_OK;
}

gs_status gs_batch_run(gs_batch* b, uint32_t steps) {
    if (!b) return fail("gs_batch_run: batch is NULL");
    GS_CUDA(cudaSetDevice(b->device));
    if (!steps) return GS_OK;
    // members moved on alone since the plan was built: re-plan (parities changed)
    bool stale = !b->planned;
    for (size_t i = 0; i < b->order.size() && !stale; ++i)
        if (b->order[i]->in != ((b->parity0[i] + (int)(b->step & 1)) & 1)) stale = true;
    if (stale) {
        gs_status st = build_plan(b);
        if (st != GS_OK) return st;
    }
    for (size_t i = 0; i < b->sims.size(); ++i) {  // after each member's own submitted work
        gs_sim* s = b->sims[i];
        GS_CUDA(cudaEventRecord(b->member_ev[i], s->stream));
        GS_CUDA(cudaStreamWaitEvent(b->root, b->member_ev[i], 0));
    }
    const bool graphs = !(b->flags & GS_BATCH_NO_GRAPH);
    for (uint32_t c = 0; c < steps; ++c) {
        const uint32_t par = (uint32_t)(b->step & 1);
        if (graphs) {
            if (!b->graph[par]) {
                cudaGraph_t g = nullptr;
                GS_CUDA(cudaStreamBeginCapture(b->root, cudaStreamCaptureModeThreadLocal));
                cudaError_t e = enqueue(b, par);
                cudaError_t e2 = cudaStreamEndCapture(b->root, &g);
                if (e != cudaSuccess) {
                    if (g) cudaGraphDestroy(g);
                    return cuda_fail(e, "gs_batch_run capture");
                }
                GS_CUDA(e2);
                e = cudaGraphInstantiate(&b->graph[par], g, 0);
                cudaGraphDestroy(g);
                GS_CUDA(e);
            }
            GS_CUDA(cudaGraphLaunch(b->graph[par], b->root));
        } else {
            GS_CUDA(enqueue(b, par));
        }
        ++b->step;
        for (gs_sim* s : b->sims) {
            s->in ^= 1;  // NextComputeIndices
            ++s->steps_done;
        }
    }
    GS_CUDA(cudaEventRecord(b->done, b->root));
    for (gs_sim* s : b->sims) GS_CUDA(cudaStreamWaitEvent(s->stream, b->done, 0));
    b->pending = true;
    return GS_OK;
}

gs_status gs_batch_sync(gs_batch* b, uint64_t timeout_ns) {
    if (!b) return fail("gs_batch_sync: batch is NULL");
    GS_CUDA(cudaSetDevice(b->device));
    if (b->pending) {
        if (!timeout_ns) timeout_ns = 600ull * 1000000000ull;
        const auto t0 = std::chrono::steady_clock::now();
        for (;;) {
            const cudaError_t e = cudaEventQuery(b->done);
            if (e == cudaSuccess) break;
            if (e != cudaErrorNotReady) return cuda_fail(e, "gs_batch_sync");
            const auto ns = std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0);
            if ((uint64_t)ns.count() > timeout_ns) {
                set_error("gs_batch_sync: timed out waiting for the batch");
                return GS_ERR_TIMEOUT;
            }
        }
        b->pending = false;
    }
    for (gs_sim* s : b->sims) {  // device-side error flags of every member
        const gs_status st = gs_sync(s, 0);
        if (st != GS_OK) return st;
    }
    return GS_OK;
}

uint32_t gs_batch_kernels_per_step(const gs_batch* b) { return b ? launches_per_step(b->plan) : 0u; }

void* gs_batch_stream(gs_batch* b) { return b ? (void*)b->root : nullptr; }

void gs_batch_destroy(gs_batch* b) { free_batch(b); }

}  // extern "C"

// ------------------------------------------------------------------------------------
// crossover tuner
// ------------------------------------------------------------------------------------
namespace {

struct Probe {
    std::vector<gs_sim*> sims;
    gs_batch* batch = nullptr;
    ~Probe() {
        gs_batch_destroy(batch);
        for (gs_sim* s : sims) gs_destroy(s);
    }
};

// milliseconds per system-step of a batch of `count` uniform disks of n particles
gs_status time_probe(const gs_params* params, uint64_t n, uint32_t count, uint64_t seed, double* ms) {
    std::vector<float> pos(2 * n), vel(2 * n), mass(n);
    Probe pr;
    for (uint32_t i = 0; i < count; ++i) {
        gs_status st = gs_generate(GS_GEN_UNIFORM_DISK, n, 100.0f, 1.0f, 10.0f, params->gravitational_const,
                                   seed + i, pos.data(), vel.data(), mass.data());
        if (st != GS_OK) return st;
        gs_sim* s = nullptr;
        st = gs_create(params, n, pos.data(), vel.data(), mass.data(), &s);
        if (st != GS_OK) return st;
        pr.sims.push_back(s);
    }
    gs_status st = gs_batch_create(pr.sims.data(), count, 0, &pr.batch);
    if (st != GS_OK) return st;
    st = gs_batch_run(pr.batch, 2);  // warm-up, graph capture
    if (st == GS_OK) st = gs_batch_sync(pr.batch, 0);
    if (st != GS_OK) return st;
    cudaStream_t root = (cudaStream_t)gs_batch_stream(pr.batch);
    cudaEvent_t a = nullptr, z = nullptr;
    GS_CUDA(cudaEventCreate(&a));
    GS_CUDA(cudaEventCreate(&z));
    const uint32_t steps = 4;
    cudaEventRecord(a, root);
    st = gs_batch_run(pr.batch, steps);
    cudaEventRecord(z, root);
    if (st == GS_OK) st = gs_batch_sync(pr.batch, 0);
    float t = 0.0f;
    if (st == GS_OK && cudaEventElapsedTime(&t, a, z) != cudaSuccess) st = GS_ERR_CUDA;
    cudaEventDestroy(a);
    cudaEventDestroy(z);
    *ms = (double)t / ((double)steps * (double)count);
    return st;
}

}  // namespace

extern "C" gs_status gs_tune_crossover(const gs_params* direct_params, const gs_params* bh_params, uint64_t min_n,
                                       uint64_t max_n, uint64_t particles_per_probe, uint64_t seed, gs_tuning* out) {
    if (!direct_params || !bh_params || !out) return fail("gs_tune_crossover: NULL argument");
    if (direct_params->algorithm != GS_DIRECT_SUM || bh_params->algorithm != GS_BARNES_HUT)
        return fail("gs_tune_crossover: direct_params must select direct sum and bh_params Barnes-Hut");
    if (min_n < 64 || max_n < min_n) return fail("gs_tune_crossover: need 64 <= min_n <= max_n");
    std::memset(out, 0, sizeof *out);
    out->crossover = max_n;
    bool bh_won = false;
    for (uint64_t n = min_n; n <= max_n && out->sizes < GS_TUNE_MAX_SIZES; n *= 2) {
        uint64_t c = particles_per_probe / n;
        const uint32_t count = (uint32_t)(c < 1 ? 1 : c > 4096 ? 4096 : c);
        double td = 0.0, tb = 0.0;
        gs_status st = time_probe(direct_params, n, count, seed, &td);
        if (st == GS_OK) st = time_probe(bh_params, n, count, seed, &tb);
        if (st != GS_OK) return st;
        const uint32_t k = out->sizes++;
        out->n[k] = n;
        out->direct_ms[k] = td;
        out->bh_ms[k] = tb;
        if (tb < td && !bh_won) {
            bh_won = true;
            if (k == 0) {
                out->crossover = n;
            } else {  // log(ratio) is close to linear in log(N): interpolate its zero
                const double r0 = std::log(out->direct_ms[k - 1] / out->bh_ms[k - 1]);
                const double r1 = std::log(td / tb);
                const double f = r0 < 0.0 && r1 > r0 ? -r0 / (r1 - r0) : 1.0;
                const double ln = std::log((double)out->n[k - 1]) + f * (std::log((double)n) - std::log((double)out->n[k - 1]));
                out->crossover = (uint64_t)std::llround(std::exp(ln));
            }
        } else if (bh_won) {
            break;  // one size past the crossover
        }
    }
    return GS_OK;
}
