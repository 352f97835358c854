// batch.cu -- many independent systems advanced together (gs_batch_*), and the
// direct-sum / Barnes-Hut crossover tuner (gs_tune_crossover).
//
// The reference runs one system per process (src/Main.cpp:250-321).  A batch runs every
// stage of the step as one launch over all of its systems: the Barnes-Hut stages of
// bh.cu (bh_batch_step) on the root stream, and the direct-sum kernel of direct.cu
// (direct_batch_step) beside them on a second stream.  Each block finds its system in a
// per-stage table of block prefixes (BatchPlan); the per-system work is the plain path's,
// so results are bit-identical to gs_run.  gs_batch captures the step once per ping-pong
// parity into a CUDA graph, so a step costs one graph launch whatever the member count.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "batch.cuh"

namespace gsim {

namespace {
constexpr uint32_t kBHFlagMask = GS_FLAG_QUADRUPOLE | GS_FLAG_SAFE_RADIUS | GS_FLAG_GROUP_WALK |
                                 GS_FLAG_COUNT_INTERACTIONS;

gs_status fail(const std::string& msg) {
    set_error(msg);
    return GS_ERR_INVALID_ARGUMENT;
}
}  // namespace

gs_status check_batch_members(gs_sim* const* sims, size_t count, const char* who) {
    const std::string w(who);
    const gs_sim* bh0 = nullptr;
    const gs_sim* dir0 = nullptr;
    for (size_t i = 0; i < count; ++i) {
        const gs_sim* s = sims[i];
        if (!s) return fail(w + ": NULL system");
        if (s->device != sims[0]->device) return fail(w + ": all systems must live on one device");
        if (s->p.algorithm == GS_BARNES_HUT) {
            if (!bh0) bh0 = s;
            else if (s->p.box_mode != bh0->p.box_mode || s->p.math_mode != bh0->p.math_mode ||
                     (s->p.flags & kBHFlagMask) != (bh0->p.flags & kBHFlagMask) || s->bh.depth != bh0->bh.depth)
                return fail(w + ": Barnes-Hut systems must share box_mode, key_bits, math_mode and the "
                                "QUADRUPOLE / SAFE_RADIUS / GROUP_WALK / COUNT_INTERACTIONS flags");
        } else {
            if (!dir0) dir0 = s;
            else if (s->p.math_mode != dir0->p.math_mode ||
                     (s->p.flags & GS_FLAG_PLAIN_SUM) != (dir0->p.flags & GS_FLAG_PLAIN_SUM))
                return fail(w + ": direct-sum systems must share math_mode and GS_FLAG_PLAIN_SUM");
        }
    }
    return GS_OK;
}

cudaError_t BatchEngine::init(int dev) {
    device = dev;
    gs_shape_defaults(&shape);
    cudaError_t e = cudaSetDevice(dev);
    if (e == cudaSuccess) e = keep_pool_memory(dev);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&root, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&moments.side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&moments.fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&moments.join, cudaEventDisableTiming);
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) e = cudaEventCreateWithFlags(&staged[k], cudaEventDisableTiming);
    return e;
}

void BatchEngine::destroy() {
    cudaSetDevice(device);
    if (root) (void)wait_stream(root, 0);
    if (side) (void)wait_stream(side, 0);
    if (moments.side) (void)wait_stream(moments.side, 0);
    for (int k = 0; k < 2; ++k) {
        if (d_block[k]) cudaFreeAsync(d_block[k], root);
        if (h_stage[k]) cudaFreeHost(h_stage[k]);
        if (staged[k]) cudaEventDestroy(staged[k]);
        d_block[k] = h_stage[k] = nullptr;
        staged[k] = nullptr;
    }
    if (d_heavy) cudaFreeAsync(d_heavy, root);
    d_heavy = nullptr;
    heavy_cap = 0;
    if (root) (void)wait_stream(root, 0);
    if (fork) cudaEventDestroy(fork);
    if (join) cudaEventDestroy(join);
    if (root) cudaStreamDestroy(root);
    if (side) cudaStreamDestroy(side);
    if (moments.fork) cudaEventDestroy(moments.fork);
    if (moments.join) cudaEventDestroy(moments.join);
    if (moments.side) cudaStreamDestroy(moments.side);
    moments = StepFork{};
    fork = join = nullptr;
    root = side = nullptr;
}

gs_status BatchEngine::set_members(const std::vector<gs_sim*>& members) {
    order = members;
    std::stable_sort(order.begin(), order.end(), [](const gs_sim* x, const gs_sim* y) {
        const bool bx = x->p.algorithm == GS_BARNES_HUT, by = y->p.algorithm == GS_BARNES_HUT;
        if (bx != by) return bx;
        return x->n_al > y->n_al;
    });
    const size_t n = order.size();
    BatchPlan p;
    p.shape = shape;
    // the counting kernels exist for the default shape only (2 group walks per block), and
    // warp pairs for costly groups need an even number of warps per block (one runs as two)
    bool counting = false, pairs = false;
    for (const gs_sim* s : order) {
        if (s->p.algorithm != GS_BARNES_HUT) continue;
        if (s->p.flags & GS_FLAG_COUNT_INTERACTIONS) counting = true;
        if (s->bh.heavy_flag && s->bh.quad && (s->p.flags & GS_FLAG_GROUP_WALK) && s->n_al >= kHeavyMinParticles)
            pairs = true;
    }
    const uint32_t force_warps = counting ? 2u : (pairs && shape.force_warps == 1) ? 2u : shape.force_warps;
    std::vector<SysDesc> descs(n);
    std::vector<uint32_t> blocks(n * kTabCount, 0u);
    parity0.assign(n, 0);
    for (size_t i = 0; i < n; ++i) {
        gs_sim* s = order[i];
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
        parity0[i] = s->in;
        if (s->p.algorithm == GS_BARNES_HUT) {
            bh_batch_desc(s, d, &blocks[i * kTabCount], shape, force_warps);
            bh_set_final_keys(s);
            ++p.n_bh;
        } else {
            direct_batch_desc(s, d, &blocks[i * kTabCount], shape);
            ++p.n_direct;
        }
    }
    // tables: Barnes-Hut stages over members [0, n_bh), the direct table over [n_bh, n)
    size_t off[kTabCount];
    size_t words = 0;
    for (int t = 0; t < kTabCount; ++t) {
        off[t] = words;
        words += (t == kTabDirect ? p.n_direct : p.n_bh) + 1;
    }
    const size_t desc_b = n * sizeof(SysDesc);
    const size_t tab_off = (desc_b + 255) / 256 * 256;
    const size_t work_off = (tab_off + words * sizeof(uint32_t) + 255) / 256 * 256;
    const size_t bytes = work_off + 256;

    const int k = cur ^ 1;  // the block the steps in flight are not reading
    {  // staging k is free again (long done in practice)
        gs_status w = wait_event(staged[k], 0);
        if (w != GS_OK) return w;
    }
    if (h_bytes[k] < bytes) {
        if (h_stage[k]) GS_CUDA(cudaFreeHost(h_stage[k]));
        h_stage[k] = nullptr;
        h_bytes[k] = 0;
        const size_t want = std::max(bytes, 2 * h_bytes[k ^ 1]);
        GS_CUDA(cudaHostAlloc(&h_stage[k], want, cudaHostAllocDefault));
        h_bytes[k] = want;
    }
    char* h = (char*)h_stage[k];
    std::memcpy(h, descs.data(), desc_b);
    uint32_t* tabs = (uint32_t*)(h + tab_off);
    for (int t = 0; t < kTabCount; ++t) {
        const size_t lo = t == kTabDirect ? p.n_bh : 0, hi = t == kTabDirect ? n : p.n_bh;
        uint64_t acc = 0;
        uint32_t* out = tabs + off[t];
        out[0] = 0u;
        for (size_t i = lo; i < hi; ++i) {
            acc += blocks[i * kTabCount + t];
            if (acc > 0x7fffffffull) return fail("batch plan: too many blocks in one stage");
            out[i - lo + 1] = (uint32_t)acc;
        }
        p.total[t] = (uint32_t)acc;
    }
    std::memset(h + work_off, 0, 256);
    if (d_bytes[k] < bytes) {  // stream-ordered: after every step that read the old block
        if (d_block[k]) GS_CUDA(cudaFreeAsync(d_block[k], root));
        d_block[k] = nullptr;
        d_bytes[k] = 0;
        const size_t want = std::max(bytes, d_bytes[k ^ 1]);
        GS_CUDA(cudaMallocAsync(&d_block[k], want, root));
        d_bytes[k] = want;
    }
    char* d = (char*)d_block[k];
    GS_CUDA(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, root));
    GS_CUDA(cudaEventRecord(staged[k], root));
    p.d_descs = (SysDesc*)d;
    for (int t = 0; t < kTabCount; ++t) p.d_tab[t] = (uint32_t*)(d + tab_off) + off[t];
    p.d_work = (uint32_t*)(d + work_off);
    const gs_sim* bh0 = p.n_bh ? order[0] : nullptr;
    const gs_sim* dir0 = p.n_direct ? order[p.n_bh] : nullptr;
    p.passes = bh0 ? bh0->bh.passes : 0;
    p.depth = bh0 ? bh0->bh.depth : 0;
    p.bbox = bh0 && bh0->p.box_mode == GS_BOX_BOUNDING;
    p.quad = bh0 && bh0->bh.quad != nullptr;
    p.group = bh0 && (bh0->p.flags & GS_FLAG_GROUP_WALK);
    p.exact = bh0 && bh0->p.math_mode == GS_MATH_REFERENCE;
    p.count = bh0 && (bh0->p.flags & GS_FLAG_COUNT_INTERACTIONS);
    p.direct_exact = dir0 && dir0->p.math_mode == GS_MATH_REFERENCE;
    p.direct_plain = dir0 && (dir0->p.flags & GS_FLAG_PLAIN_SUM);
    // the costly-group list of the relative criterion: one entry per group of 64 slots of
    // every member that has the criterion (stream-ordered growth, like the plan blocks)
    size_t groups = 0;
    for (size_t i = 0; i < p.n_bh; ++i)
        if (order[i]->bh.heavy_flag && order[i]->n_al >= kHeavyMinParticles) groups += order[i]->n_al / 64 + 1;
    if (groups && p.quad && p.group) {
        if (heavy_cap < groups) {
            if (d_heavy) GS_CUDA(cudaFreeAsync(d_heavy, root));
            d_heavy = nullptr;
            heavy_cap = 0;
            GS_CUDA(cudaMallocAsync((void**)&d_heavy, groups * sizeof(uint2), root));
            heavy_cap = groups;
        }
        p.d_heavy = d_heavy;
    }
    if (bh0) p.force_grid = bh_batch_force_grid(p);  // resident blocks of the persistent force launch
    plan = p;
    cur = k;
    step = 0;
    return GS_OK;
}

bool BatchEngine::needs_estimate() const {
    for (const gs_sim* s : order)
        if (s->p.algorithm == GS_BARNES_HUT && (s->p.flags & GS_FLAG_RELATIVE_MAC) && !s->amag_known) return true;
    return false;
}

cudaError_t BatchEngine::enqueue(uint32_t par, bool estimate) {
    const bool both = plan.n_bh && plan.n_direct;
    cudaError_t e = cudaSuccess;
    if (both) {
        e = cudaEventRecord(fork, root);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(side, fork, 0);
    }
    if (e == cudaSuccess) e = bh_batch_step(plan, par, root, estimate, moments);
    if (e == cudaSuccess) e = direct_batch_step(plan, par, both ? side : root);
    if (both) {
        if (e == cudaSuccess) e = cudaEventRecord(join, side);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(root, join, 0);
    }
    return e;
}

void BatchEngine::advance() {
    ++step;
    for (gs_sim* s : order) {
        s->in ^= 1;  // NextComputeIndices
        ++s->steps_done;
        s->amag_known = true;
    }
}

bool BatchEngine::in_step() const {
    for (size_t i = 0; i < order.size(); ++i)
        if (order[i]->in != ((parity0[i] + (int)(step & 1)) & 1)) return false;
    return true;
}

uint32_t BatchEngine::launches_per_step() const {
    uint32_t k = 0;
    if (plan.n_bh)  // clear keys scan records nodes force, radix passes, box, then the moment
                    // prefix (quadrupole mode) or the moment levels (the |a| estimate pass of a
                    // step after a member joined or was reset not included)
        k += 6u + (uint32_t)plan.passes + (plan.bbox ? 1u : 0u) +
             (plan.quad ? 3u : (uint32_t)(plan.depth - kLevelTop + 1));
    if (plan.n_direct) k += 1u;
    return k;
}

}  // namespace gsim

using namespace gsim;

struct gs_batch {
    std::vector<gs_sim*> sims;  // caller order
    uint32_t flags = 0;
    BatchEngine eng;
    std::vector<cudaEvent_t> member_ev;  // orders the batch after each member's own work
    cudaEvent_t done = nullptr;
    cudaGraphExec_t graph[4] = {nullptr, nullptr, nullptr, nullptr};  // [parity], [2 + parity] with the estimate
    bool pending = false;
};

namespace {

void drop_graphs(gs_batch* b) {
    for (auto& g : b->graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
}

void free_batch(gs_batch* b) {
    if (!b) return;
    cudaSetDevice(b->eng.device);
    for (gs_sim* s : b->sims)  // the event goes away: members follow it now
        if (s->follow == b->done) {
            cudaStreamWaitEvent(s->stream, b->done, 0);
            s->follow = nullptr;
        }
    drop_graphs(b);
    b->eng.destroy();
    for (auto e : b->member_ev)
        if (e) cudaEventDestroy(e);
    if (b->done) cudaEventDestroy(b->done);
    delete b;
}

}  // namespace

namespace gsim {
gs_status batch_key(gs_batch* b, gs_params* params, uint64_t* total) {
    const gs_sim* first_bh = nullptr;
    uint64_t sum = 0;
    for (const gs_sim* s : b->sims) {
        sum += s->n;
        if (!first_bh && s->p.algorithm == GS_BARNES_HUT) first_bh = s;
    }
    *params = first_bh ? first_bh->p : b->sims[0]->p;
    *total = sum;
    return GS_OK;
}
}  // namespace gsim

extern "C" {

gs_status gs_batch_create(gs_sim* const* sims, uint32_t count, uint32_t flags, gs_batch** out) {
    if (!out) return fail("gs_batch_create: out is NULL");
    *out = nullptr;
    if (!sims || !count) return fail("gs_batch_create: empty system list");
    if (flags & ~GS_BATCH_NO_GRAPH) return fail("gs_batch_create: unknown flags");
    gs_status st = check_batch_members(sims, count, "gs_batch_create");
    if (st != GS_OK) return st;
    for (uint32_t i = 0; i < count; ++i)
        for (uint32_t j = 0; j < i; ++j)
            if (sims[j] == sims[i]) return fail("gs_batch_create: a system appears twice");
    gs_batch* b = new (std::nothrow) gs_batch();
    if (!b) {
        set_error("gs_batch_create: host allocation failed");
        return GS_ERR_OUT_OF_MEMORY;
    }
    b->sims.assign(sims, sims + count);
    b->flags = flags;
    b->member_ev.assign(count, nullptr);
    cudaError_t e = b->eng.init(sims[0]->device);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
    for (uint32_t i = 0; i < count && e == cudaSuccess; ++i)
        e = cudaEventCreateWithFlags(&b->member_ev[i], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        st = cuda_fail(e, "gs_batch_create");
        free_batch(b);
        return st;
    }
    {  // the batch's launch shape: the tuned entry of its total particles, else the defaults
        gs_params kp;
        uint64_t total = 0;
        st = batch_key(b, &kp, &total);
        if (st == GS_OK) batch_shape_for(&kp, total, &b->eng.shape);
    }
    st = b->eng.set_members(b->sims);
    if (st != GS_OK) {
        free_batch(b);
        return st;
    }
    *out = b;
    return GS_OK;
}

gs_status gs_batch_get_shape(gs_batch* b, gs_shape* out) {
    if (!b || !out) return fail("gs_batch_get_shape: NULL argument");
    *out = b->eng.shape;
    return GS_OK;
}

gs_status gs_batch_set_shape(gs_batch* b, const gs_shape* sh) {
    if (!b || !sh) return fail("gs_batch_set_shape: NULL argument");
    std::string why;
    if (!shape_valid(*sh, &why)) return fail("gs_batch_set_shape: " + why);
    GS_CUDA(cudaSetDevice(b->eng.device));
    if (b->pending) {  // the step graphs may still run: wait before dropping them
        gs_status w = wait_event(b->done, 0);
        if (w != GS_OK) return w;
    }
    drop_graphs(b);
    b->eng.shape = *sh;
    for (gs_sim* s : b->sims)  // a direct-sum member keeps its own j-split: it must fit its scratch
        if (s->p.algorithm == GS_DIRECT_SUM && direct_chunks_needed(s, s->shape) > s->direct_max_chunks) {
            set_error("gs_batch_set_shape: a member's j-split does not fit its scratch");
            return GS_ERR_CAPACITY;
        }
    return b->eng.set_members(b->sims);
}

gs_status gs_batch_run(gs_batch* b, uint32_t steps) {
    if (!b) return fail("gs_batch_run: batch is NULL");
    GS_CUDA(cudaSetDevice(b->eng.device));
    if (!steps) return GS_OK;
    if (!b->eng.in_step()) {  // members moved on alone since the plan was built
        drop_graphs(b);
        gs_status st = b->eng.set_members(b->sims);
        if (st != GS_OK) return st;
    }
    for (size_t i = 0; i < b->sims.size(); ++i) {  // after work submitted on a member's own stream
        gs_sim* s = b->sims[i];
        if (s->follow == b->done) s->follow = nullptr;  // nothing ran alone since: already ordered
        if (!s->own_work && !s->follow) continue;
        if (s->follow) GS_CUDA(cudaStreamWaitEvent(s->stream, s->follow, 0));
        s->follow = nullptr;
        GS_CUDA(cudaEventRecord(b->member_ev[i], s->stream));
        GS_CUDA(cudaStreamWaitEvent(b->eng.root, b->member_ev[i], 0));
        s->own_work = false;
    }
    const bool graphs = !(b->flags & GS_BATCH_NO_GRAPH);
    for (uint32_t c = 0; c < steps; ++c) {
        const uint32_t par = (uint32_t)(b->eng.step & 1);
        const bool est = b->eng.needs_estimate();
        const uint32_t gi = par + (est ? 2u : 0u);
        if (graphs) {
            if (!b->graph[gi]) {
                cudaGraph_t g = nullptr;
                GS_CUDA(cudaStreamBeginCapture(b->eng.root, cudaStreamCaptureModeThreadLocal));
                cudaError_t e = b->eng.enqueue(par, est);
                cudaError_t e2 = cudaStreamEndCapture(b->eng.root, &g);
                if (e != cudaSuccess) {
                    if (g) cudaGraphDestroy(g);
                    return cuda_fail(e, "gs_batch_run capture");
                }
                GS_CUDA(e2);
                e = cudaGraphInstantiate(&b->graph[gi], g, 0);
                cudaGraphDestroy(g);
                GS_CUDA(e);
            }
            GS_CUDA(cudaGraphLaunch(b->graph[gi], b->eng.root));
        } else {
            GS_CUDA(b->eng.enqueue(par, est));
        }
        b->eng.advance();
    }
    GS_CUDA(cudaEventRecord(b->done, b->eng.root));
    for (gs_sim* s : b->sims) s->follow = b->done;  // a member's next own work waits for this
    b->pending = true;
    return GS_OK;
}

gs_status gs_batch_sync(gs_batch* b, uint64_t timeout_ns) {
    if (!b) return fail("gs_batch_sync: batch is NULL");
    GS_CUDA(cudaSetDevice(b->eng.device));
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

uint32_t gs_batch_kernels_per_step(const gs_batch* b) { return b ? b->eng.launches_per_step() : 0u; }

void* gs_batch_stream(gs_batch* b) { return b ? (void*)b->eng.root : nullptr; }

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
    const uint32_t steps = 8;
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
            } else {  // log(direct / bh) is close to linear in log N: interpolate its zero
                const double r0 = std::log(out->direct_ms[k - 1] / out->bh_ms[k - 1]);
                const double r1 = std::log(td / tb);
                const double f = r0 < 0.0 && r1 > r0 ? -r0 / (r1 - r0) : 1.0;
                const double l0 = std::log((double)out->n[k - 1]);
                out->crossover = (uint64_t)std::llround(std::exp(l0 + f * (std::log((double)n) - l0)));
            }
        } else if (bh_won) {
            break;  // one size past the crossover
        }
    }
    return GS_OK;
}
