// sim.cu -- gs_sim lifecycle and the C ABI entry points of include/gsim.h.
//
// The step loop mirrors DirectSimulation::RunSimulations / BarnesHutSimulation::RunSimulations
// (src/Simulation/Direct/DirectSimulation.cpp:271-353,
// src/Simulation/BarnesHut/BarnesHutSimulation.cpp:849-952): wait for the previous batch,
// enqueue `count` steps that read set `in` and write set `out`, flip the indices on the
// host after every step (ParticleSystem::NextComputeIndices, src/Particles/ParticleSystem.hpp:169-174).
// Instead of re-recording command buffers, each parity of the ping-pong is captured
// once into a CUDA graph and replayed.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <thread>

#include "internal.cuh"

namespace gsim {

static thread_local std::string g_last_error;
constexpr uint64_t kDefaultTimeoutNs = 600ull * 1000000000ull;

void set_error(const std::string& msg) { g_last_error = msg; }

gs_status cuda_fail(cudaError_t e, const char* what) {
    set_error(std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
    if (e == cudaErrorMemoryAllocation) return GS_ERR_OUT_OF_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return GS_ERR_NO_DEVICE;
    return GS_ERR_CUDA;
}

static void record(gs_sim* s, cudaEvent_t e) {
    if (s->capturing) cudaEventRecordWithFlags(e, s->stream, cudaEventRecordExternal);
    else cudaEventRecord(e, s->stream);
}
void stage_begin(gs_sim* s, int stage, bool profile) {
    if (profile) record(s, s->ev[2 * stage]);
}
void stage_end(gs_sim* s, int stage, bool profile) {
    if (profile) {
        record(s, s->ev[2 * stage + 1]);
        s->stage_ran |= 1u << stage;
    }
}

// A system's device memory is one slab from the device's default pool, allocated and
// freed in order on the system's stream: creating or destroying a system never waits for
// work elsewhere on the device (cudaFree would), and freed slabs stay in the pool for the
// next system.  One allocation per system keeps the pool's bookkeeping small however
// many systems are alive.
void sim_carve(gs_sim* s, void** p, size_t bytes) {
    const size_t off = (s->carved + 255) & ~(size_t)255;
    s->carved = off + bytes;
    *p = s->slab ? (void*)((char*)s->slab + off) : nullptr;
}

// every buffer of the system, in one fixed order
void carve_all(gs_sim* s) {
    s->carved = 0;
    for (int b = 0; b < 2; ++b) {
        sim_carve(s, (void**)&s->pos[b], s->n_al * sizeof(float2));
        sim_carve(s, (void**)&s->vel[b], s->n_al * sizeof(float2));
    }
    sim_carve(s, (void**)&s->mass[0], s->n_al * sizeof(float));
    s->mass[1] = s->mass[0];  // no step writes mass except removal, which writes both sets alike
    sim_carve(s, (void**)&s->d_err, sizeof(int));
    s->acc = nullptr;
    if (s->p.flags & GS_FLAG_RECORD_ACCEL) sim_carve(s, (void**)&s->acc, s->n_al * sizeof(float2));
    if (s->p.algorithm == GS_BARNES_HUT) bh_carve(s);
    else direct_carve(s);
}

// A batch left this system an event to follow (gs_batch_run): its next work on its own
// stream waits for that batch step.
void follow_batch(gs_sim* s) {
    if (s->follow) {
        cudaStreamWaitEvent(s->stream, s->follow, 0);
        s->follow = nullptr;
    }
}

cudaError_t keep_pool_memory(int device) {
    static std::mutex mu;
    static bool done[64] = {};
    std::lock_guard<std::mutex> lock(mu);
    if (device < 0 || device >= 64 || done[device]) return cudaSuccess;
    cudaMemPool_t pool;
    cudaError_t e = cudaDeviceGetDefaultMemPool(&pool, device);
    uint64_t keep = ~0ull;  // never trim freed blocks back to the driver
    if (e == cudaSuccess) e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    if (e == cudaSuccess) done[device] = true;
    return e;
}

// Host waits on the GPU are bounded: they poll with a deadline and give up with
// GS_ERR_TIMEOUT after it (timeout_ns 0: 600 s), so a hung device never hangs the caller.
gs_status wait_event(cudaEvent_t ev, uint64_t timeout_ns) {
    if (!timeout_ns) timeout_ns = kDefaultTimeoutNs;
    auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        cudaError_t e = cudaEventQuery(ev);
        if (e == cudaSuccess) return GS_OK;
        if (e != cudaErrorNotReady) return cuda_fail(e, "cudaEventQuery");
        auto el = std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0).count();
        if ((uint64_t)el > timeout_ns) {
            set_error("timed out waiting for the GPU");
            return GS_ERR_TIMEOUT;
        }
        // spin for the first 2 ms: a sleep lasts the thread's timer slack (50 us on Linux)
        // on top of the 20 asked for, which is a tenth of a 500k-particle step
        if (el < 2000000) std::this_thread::yield();
        else std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}

gs_status wait_stream(cudaStream_t st, uint64_t timeout_ns) {
    cudaEvent_t ev = nullptr;
    GS_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaError_t e = cudaEventRecord(ev, st);
    gs_status r = e == cudaSuccess ? wait_event(ev, timeout_ns) : cuda_fail(e, "cudaEventRecord");
    cudaEventDestroy(ev);  // released once it completes, if the wait gave up
    return r;
}

gs_status sim_wait(gs_sim* s) {
    GS_CUDA(cudaEventRecord(s->batch_done, s->stream));
    s->batch_pending = true;
    gs_status w = wait_event(s->batch_done, s->timeout_ns);
    if (w == GS_OK) s->batch_pending = false;
    return w;
}

gs_status bh_debug_tree(gs_sim* s, uint32_t* keys, uint32_t* sorted_src, uint32_t* node_skip, float* node_radius,
                        float* node_pos, float* node_mass, float* node_quad, uint64_t capacity,
                        uint64_t* tree_records);
gs_status bh_read_counts(gs_sim* s, uint64_t* nv, uint64_t* internal, uint64_t* inter, uint64_t* visits,
                         uint64_t* nodes);

}  // namespace gsim

using namespace gsim;

namespace {

constexpr uint64_t kMaxParticles = 1ull << 28;
constexpr uint64_t kMaxBarnesHutParticles = 1ull << 26;  // keeps record indices below 2^31

gs_status invalid(const char* msg) {
    set_error(msg);
    return GS_ERR_INVALID_ARGUMENT;
}

// Status of a device error word.
gs_status device_error(int err) {
    if (err) {
        set_error(std::string("device-side error flags ") + std::to_string(err) +
                  " (1: radix-sort look-back wait ran out, 2: scan look-back wait ran out, 4: tree capacity, "
                  "8: moments grid barrier wait ran out)");
        return GS_ERR_DEVICE;
    }
    return GS_OK;
}

// Reads the device error word after everything enqueued so far (one round trip: the copy
// into the system's pinned word, then the stream synchronisation).
gs_status check_device_error(gs_sim* s) {
    GS_CUDA(cudaMemcpyAsync(s->h_err, s->d_err, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    gs_status w = sim_wait(s);
    if (w != GS_OK) return w;
    return device_error(*s->h_err);
}

void free_sim(gs_sim* s) {
    if (!s) return;
    cudaSetDevice(s->device);
    if (s->stream) (void)wait_stream(s->stream, s->timeout_ns);
    if (s->side) (void)wait_stream(s->side, s->timeout_ns);
    free_snapshot_ring(s);
    for (auto& g : s->graph)
        if (g) cudaGraphExecDestroy(g);
    if (s->slab) cudaFreeAsync(s->slab, s->stream);
    s->slab = nullptr;
    for (auto& e : s->ev)
        if (e) cudaEventDestroy(e);
    if (s->batch_done) cudaEventDestroy(s->batch_done);
    if (s->fork_ev) cudaEventDestroy(s->fork_ev);
    if (s->join_ev) cudaEventDestroy(s->join_ev);
    if (s->side) cudaStreamDestroy(s->side);
    if (s->stream) cudaStreamDestroy(s->stream);
    if (s->h_err) cudaFreeHost(s->h_err);
    delete s;
}

// Device address of a host array that the GPU can read and write in place (pinned or
// registered host memory of this device, mapped under unified addressing), or null for
// pageable memory, a device pointer, or an address not aligned to `align` bytes.
const void* host_mapped(const gs_sim* s, const void* p, uintptr_t align) {
    if (!p || ((uintptr_t)p & (align - 1))) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost && a.device == s->device ? a.devicePointer : nullptr;
}

// Fills both sets from the N source particles (mapped host arrays read in place, or set a
// after the copy engine filled it), zeroes the padding slots (and every velocity when none
// was given) and marks every |a| unknown (all-ones words are NaN, so the next step opens
// nodes by theta).  With `ext` (bounding-box mode, words cleared before the launch) it
// gathers the extent of set a's positions, padding included, for the next step's box.
// The sources may alias set a, so no pointer is restrict-qualified.
__global__ void k_upload(const float2* src_pos, const float2* src_vel, const float* src_mass, float2* pos_a,
                         float2* vel_a, float* mass, float2* pos_b, float2* vel_b, float* amag, uint32_t n,
                         uint32_t n_al, uint32_t* ext, const int* d_err, int* h_err) {
    // the error word of the work before the upload (stream order), for the caller's check
    if (blockIdx.x == 0 && threadIdx.x == 0) *h_err = *d_err;
    float mnx = INFINITY, mxx = -INFINITY, mny = INFINITY, mxy = -INFINITY;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_al; i += gridDim.x * blockDim.x) {
        float2 p = make_float2(0.0f, 0.0f), v = p;
        float m = 0.0f;
        if (i < n) {
            p = src_pos[i];
            if (src_vel) v = src_vel[i];
            m = src_mass[i];
        }
        pos_a[i] = p;
        pos_b[i] = p;
        vel_a[i] = v;
        vel_b[i] = v;
        mass[i] = m;
        if (amag) amag[i] = __uint_as_float(0xFFFFFFFFu);
        mnx = fminf(mnx, p.x);
        mxx = fmaxf(mxx, p.x);
        mny = fminf(mny, p.y);
        mxy = fmaxf(mxy, p.y);
    }
    if (!ext) return;  // uniform over the grid
    for (int o = 16; o; o >>= 1) {
        mnx = fminf(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
        mxx = fmaxf(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
        mny = fminf(mny, __shfl_xor_sync(0xffffffffu, mny, o));
        mxy = fmaxf(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(ext + 0, gsim::ord_word(__float_as_uint(mnx)));
        atomicMin(ext + 1, ~gsim::ord_word(__float_as_uint(mxx)));
        atomicMin(ext + 2, gsim::ord_word(__float_as_uint(mny)));
        atomicMin(ext + 3, ~gsim::ord_word(__float_as_uint(mxy)));
    }
}

// Writes the N particles of one set into mapped host arrays (any of them may be null) and
// the device error word into the system's pinned word.
__global__ void k_download(const float2* __restrict__ pos, const float2* __restrict__ vel,
                           const float* __restrict__ mass, float2* __restrict__ host_pos, float2* __restrict__ host_vel,
                           float* __restrict__ host_mass, uint32_t n, const int* __restrict__ d_err,
                           int* __restrict__ h_err) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (host_pos) host_pos[i] = pos[i];
        if (host_vel) host_vel[i] = vel[i];
        if (host_mass) host_mass[i] = mass[i];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *h_err = *d_err;
}

uint32_t copy_blocks(uint64_t n) { return (uint32_t)std::min<uint64_t>((n + 255) / 256, 152ull * 8); }

// Uploads N host particles into both sets (ParticleSystem.cpp:206-217: the reference's
// staging upload fills every buffer set) and pads with zero particles.  Pinned host arrays
// are read in place by one kernel; any other memory goes through the copy engine into set
// a first.  Returns after the host arrays have been read.
gs_status upload(gs_sim* s, const float* pos, const float* vel, const float* mass) {
    const size_t n = s->n;
    const int a = s->in, b = a ^ 1;
    const float2* sp = (const float2*)host_mapped(s, pos, 8);
    const float2* sv = vel ? (const float2*)host_mapped(s, vel, 8) : nullptr;
    const float* sm = (const float*)host_mapped(s, mass, 4);
    if (!sp || (vel && !sv) || !sm) {
        GS_CUDA(cudaMemcpyAsync(s->pos[a], pos, n * sizeof(float2), cudaMemcpyHostToDevice, s->stream));
        sp = s->pos[a];
        if (vel) {
            GS_CUDA(cudaMemcpyAsync(s->vel[a], vel, n * sizeof(float2), cudaMemcpyHostToDevice, s->stream));
            sv = s->vel[a];
        }
        GS_CUDA(cudaMemcpyAsync(s->mass[0], mass, n * sizeof(float), cudaMemcpyHostToDevice, s->stream));
        sm = s->mass[0];
    }
    uint32_t* ext = s->bh.ext ? s->bh.ext + 4 * a : nullptr;
    if (ext) GS_CUDA(cudaMemsetAsync(ext, 0xFF, 4 * sizeof(uint32_t), s->stream));
    s->amag_known = false;  // k_upload marks every |a| unknown
    k_upload<<<copy_blocks(s->n_al), 256, 0, s->stream>>>(sp, sv, sm, s->pos[a], s->vel[a], s->mass[0], s->pos[b],
                                                          s->vel[b], s->bh.amag, (uint32_t)n, (uint32_t)s->n_al, ext,
                                                          s->d_err, s->h_err);
    GS_CUDA(cudaGetLastError());
    ++s->kernel_launches;
    // the host arrays must have been read before this returns; a bounded wait (it also
    // covers whatever was submitted before the upload).  After a timeout the kernel may
    // still read them: the caller keeps them until a gs_sync succeeds.
    return sim_wait(s);
}

cudaError_t enqueue_step(gs_sim* s, int in, bool profile, bool estimate) {
    const int out = in ^ 1;
    if (s->p.algorithm == GS_BARNES_HUT) return bh_step(s, in, out, profile, estimate);
    return direct_step(s, in, out, profile);
}

// The next step has to estimate |a| first: the relative criterion with no previous |a|
// (after gs_create or gs_set_particles).
bool needs_estimate(const gs_sim* s) {
    return s->p.algorithm == GS_BARNES_HUT && (s->p.flags & GS_FLAG_RELATIVE_MAC) && !s->amag_known;
}

gs_status account_profile(gs_sim* s) {
    s->profile_pending = false;
    for (int st = 0; st < GS_STAGE_COUNT; ++st) {
        if (!(s->stage_ran & (1u << st))) continue;
        gs_status w = wait_event(s->ev[2 * st + 1], s->timeout_ns);
        if (w != GS_OK) return w;
        float ms = 0.f;
        GS_CUDA(cudaEventElapsedTime(&ms, s->ev[2 * st], s->ev[2 * st + 1]));
        s->stats.stage_ms[st] += ms;
        s->stats.stage_launches[st] += 1;
    }
    return GS_OK;
}

}  // namespace

extern "C" {

void gs_params_init(gs_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof *p);
    p->gravitational_const = 1.0f;  // src/Main.cpp:59-63
    p->simulation_time = 0.001f;
    p->simulation_speed = 1.0f;
    p->softening_len = 0.2f;
    p->accuracy_parameter = 1.0f;
    p->algorithm = GS_DIRECT_SUM;
    p->box_mode = GS_BOX_FIXED_500;
    p->math_mode = GS_MATH_FAST;
    p->device = 0;
    p->flags = 0;
    p->relative_accuracy = 0.006f;
    p->relative_theta_floor = 0.0f;
    p->key_bits = kBBoxBits;
}

const char* gs_status_string(gs_status s) {
    switch (s) {
        case GS_OK: return "ok";
        case GS_ERR_INVALID_ARGUMENT: return "invalid argument";
        case GS_ERR_CUDA: return "CUDA error";
        case GS_ERR_OUT_OF_MEMORY: return "out of device memory";
        case GS_ERR_TIMEOUT: return "timeout";
        case GS_ERR_DEVICE: return "device-side error";
        case GS_ERR_IO: return "I/O error";
        case GS_ERR_CAPACITY: return "capacity exceeded";
        case GS_ERR_NO_DEVICE: return "no CUDA device";
    }
    return "unknown status";
}

const char* gs_last_error(void) { return g_last_error.c_str(); }

uint64_t gs_required_alignment(int32_t algorithm) {
    (void)algorithm;  // both simulations align to 64 (DirectSimulation.cpp:26-28, BarnesHutSimulation.cpp:834-836)
    return kAlignment;
}

uint64_t gs_bh_node_capacity(int32_t box_mode, uint64_t aligned_count) {
    return bh_capacity(box_mode == GS_BOX_BOUNDING ? kBBoxMaxBits : kFixedDepth, aligned_count);
}

uint64_t gs_footprint(const gs_params* p, uint64_t n) {
    if (!p || !n) return 0;
    gs_sim t;  // a sizing pass of gs_create's layout: host only, no slab
    t.p = *p;
    t.n = n;
    t.n_al = (n + kAlignment - 1) / kAlignment * kAlignment;
    carve_all(&t);
    return t.carved;
}

gs_status gs_create(const gs_params* params, uint64_t n, const float* pos, const float* vel, const float* mass,
                    gs_sim** out) {
    if (!out) return invalid("gs_create: out is NULL");
    *out = nullptr;
    if (!params) return invalid("gs_create: params is NULL");
    if (!n) return invalid("The simulation must contain at least one particle!");
    if (!pos || !mass) return invalid("gs_create: pos_xy and mass are required");
    if (params->algorithm != GS_DIRECT_SUM && params->algorithm != GS_BARNES_HUT)
        return invalid("Invalid simulation algorithm requested!");
    if (params->box_mode != GS_BOX_FIXED_500 && params->box_mode != GS_BOX_BOUNDING)
        return invalid("gs_create: invalid box_mode");
    if (params->math_mode != GS_MATH_FAST && params->math_mode != GS_MATH_REFERENCE)
        return invalid("gs_create: invalid math_mode");
    if ((params->flags & GS_FLAG_QUADRUPOLE) && !(params->flags & GS_FLAG_GROUP_WALK))
        return invalid("gs_create: GS_FLAG_QUADRUPOLE needs GS_FLAG_GROUP_WALK");
    if ((params->flags & GS_FLAG_RELATIVE_MAC) &&
        (~params->flags & (GS_FLAG_GROUP_WALK | GS_FLAG_QUADRUPOLE)))
        return invalid("gs_create: GS_FLAG_RELATIVE_MAC needs GS_FLAG_GROUP_WALK and GS_FLAG_QUADRUPOLE");
    if ((params->flags & GS_FLAG_RELATIVE_MAC) &&
        !(params->relative_accuracy >= 0.0f && params->relative_accuracy < INFINITY))
        return invalid("gs_create: relative_accuracy must be finite and >= 0");
    if ((params->flags & GS_FLAG_RELATIVE_MAC) &&
        !(params->relative_theta_floor >= 0.0f && params->relative_theta_floor < INFINITY))
        return invalid("gs_create: relative_theta_floor must be finite and >= 0");
    if (params->key_bits < 0 || params->key_bits > kBBoxMaxBits)
        return invalid("gs_create: key_bits must be 1..15 (0: 12)");
    if ((params->flags & GS_FLAG_PLAIN_SUM) && params->algorithm != GS_DIRECT_SUM)
        return invalid("gs_create: GS_FLAG_PLAIN_SUM applies to direct sum only");
    if ((params->flags & (GS_FLAG_QUADRUPOLE | GS_FLAG_SAFE_RADIUS | GS_FLAG_GROUP_WALK)) &&
        params->algorithm != GS_BARNES_HUT)
        return invalid("gs_create: the accurate-mode flags apply to Barnes-Hut only");
    if (n > kMaxParticles || (params->algorithm == GS_BARNES_HUT && n > kMaxBarnesHutParticles)) {
        set_error("gs_create: particle count above the library's limit (2^28 direct sum, 2^26 Barnes-Hut)");
        return GS_ERR_CAPACITY;
    }
    int ndev = 0;
    cudaError_t ce = cudaGetDeviceCount(&ndev);
    if (ce != cudaSuccess || ndev == 0) {
        set_error("no CUDA device available");
        return GS_ERR_NO_DEVICE;
    }
    if (params->device < 0 || params->device >= ndev) return invalid("gs_create: device ordinal out of range");

    gs_sim* s = new (std::nothrow) gs_sim();
    if (!s) return invalid("gs_create: host allocation failed");
    s->p = *params;
    s->device = params->device;
    s->n = n;
    s->n_al = (n + kAlignment - 1) / kAlignment * kAlignment;  // ParticleSystem.cpp:487
    // Specialization constants of the reference (DirectSimulation.cpp:175-181, BarnesHutSimulation.cpp:571-582)
    s->G = params->gravitational_const;
    s->eps2 = params->softening_len * params->softening_len;
    s->theta2 = params->accuracy_parameter * params->accuracy_parameter;
    {
        const float f = params->relative_theta_floor > 0.0f ? params->relative_theta_floor : params->accuracy_parameter;
        s->floor2 = f * f;
    }
    s->dt_eff = params->algorithm == GS_BARNES_HUT ? params->simulation_time * params->simulation_speed
                                                   : params->simulation_time;  // direct sum ignores speed

    gs_status st = GS_OK;
#define GS_TRY(call)                                   \
    do {                                               \
        cudaError_t _e = (call);                       \
        if (_e != cudaSuccess) {                       \
            st = cuda_fail(_e, #call);                 \
            free_sim(s);                               \
            return st;                                 \
        }                                              \
    } while (0)
    GS_TRY(cudaSetDevice(s->device));
    GS_TRY(keep_pool_memory(s->device));
    GS_TRY(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    GS_TRY(cudaEventCreateWithFlags(&s->batch_done, cudaEventDisableTiming));
    GS_TRY(cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking));
    GS_TRY(cudaEventCreateWithFlags(&s->fork_ev, cudaEventDisableTiming));
    GS_TRY(cudaEventCreateWithFlags(&s->join_ev, cudaEventDisableTiming));
    GS_TRY(cudaMallocHost((void**)&s->h_err, kHostWords * sizeof(int)));
    shape_for(params, n, &s->shape);
    for (auto& e : s->ev) GS_TRY(cudaEventCreate(&e));
    carve_all(s);  // sizing pass
    GS_TRY(cudaMallocAsync(&s->slab, s->carved, s->stream));
    carve_all(s);  // the same layout inside the slab
    GS_TRY(cudaMemsetAsync(s->d_err, 0, sizeof(int), s->stream));
    if (s->acc) GS_TRY(cudaMemsetAsync(s->acc, 0, s->n_al * sizeof(float2), s->stream));
    if (params->algorithm == GS_BARNES_HUT) GS_TRY(bh_init(s));
    else GS_TRY(direct_init(s));
#undef GS_TRY
    st = upload(s, pos, vel, mass);
    if (st != GS_OK) {
        free_sim(s);
        return st;
    }
    *out = s;
    return GS_OK;
}

gs_status gs_run(gs_sim* s, uint32_t count) {
    if (!s) return invalid("gs_run: sim is NULL");
    GS_CUDA(cudaSetDevice(s->device));
    follow_batch(s);
    s->own_work = true;
    if (s->batch_pending) {  // wait for the previous submit, like the reference's fence wait
        gs_status w = wait_event(s->batch_done, s->timeout_ns);
        if (w != GS_OK) return w;
        s->batch_pending = false;
    }
    if (!count) return GS_OK;
    const bool profile = (s->p.flags & GS_FLAG_PROFILE) != 0;
    const bool graphs = !(s->p.flags & GS_FLAG_NO_GRAPH);
    for (uint32_t c = 0; c < count; ++c) {
        const int in = s->in;
        if (s->profile_pending) {  // the previous step's stage events are about to be re-recorded
            gs_status a = account_profile(s);
            if (a != GS_OK) return a;
        }
        s->stage_ran = 0;
        const bool est = needs_estimate(s);
        const int gi = in + (est ? 2 : 0);
        if (graphs) {
            if (!s->graph[gi]) {
                cudaGraph_t g = nullptr;
                s->launches_in_step = 0;
                s->capturing = true;
                GS_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
                cudaError_t e = enqueue_step(s, in, profile, est);
                cudaError_t e2 = cudaStreamEndCapture(s->stream, &g);
                s->capturing = false;
                if (e != cudaSuccess) {
                    if (g) cudaGraphDestroy(g);
                    return cuda_fail(e, "step capture");
                }
                GS_CUDA(e2);
                e = cudaGraphInstantiate(&s->graph[gi], g, 0);
                cudaGraphDestroy(g);
                GS_CUDA(e);
                s->launches_per_step[gi] = s->launches_in_step;
                s->graph_stages[gi] = s->stage_ran;
            }
            s->stage_ran = s->graph_stages[gi];
            GS_CUDA(cudaGraphLaunch(s->graph[gi], s->stream));
            s->kernel_launches += s->launches_per_step[gi];
        } else {
            s->launches_in_step = 0;
            GS_CUDA(enqueue_step(s, in, profile, est));
            s->kernel_launches += s->launches_in_step;
        }
        s->amag_known = true;  // this step leaves every particle's |a|
        if (profile) s->profile_pending = true;  // read back before the next step records again
        s->in ^= 1;  // NextComputeIndices
        ++s->steps_done;
    }
    GS_CUDA(cudaEventRecord(s->batch_done, s->stream));
    s->batch_pending = true;
    return GS_OK;
}

gs_status gs_sync(gs_sim* s, uint64_t timeout_ns) {
    if (!s) return invalid("gs_sync: sim is NULL");
    GS_CUDA(cudaSetDevice(s->device));
    follow_batch(s);
    if (s->batch_pending) {
        gs_status w = wait_event(s->batch_done, timeout_ns ? timeout_ns : s->timeout_ns);
        if (w != GS_OK) return w;
        s->batch_pending = false;
    }
    if (s->profile_pending) {
        gs_status a = account_profile(s);
        if (a != GS_OK) return a;
    }
    return check_device_error(s);  // synchronises the stream
}

gs_status gs_get_particles(gs_sim* s, float* pos, float* vel, float* mass) {
    if (!s) return invalid("gs_get_particles: sim is NULL");
    GS_CUDA(cudaSetDevice(s->device));
    follow_batch(s);
    const int in = s->in;  // ParticleSystem::GetParticles reads buffers[computeInputIndex]
    float2* hp = (float2*)host_mapped(s, pos, 8);
    float2* hv = (float2*)host_mapped(s, vel, 8);
    float* hm = (float*)host_mapped(s, mass, 4);
    if ((!pos || hp) && (!vel || hv) && (!mass || hm)) {
        // pinned arrays: one kernel writes them and the error word, enqueued right behind
        // the submitted steps (stream order), then one bounded wait for all of it
        k_download<<<copy_blocks(s->n), 256, 0, s->stream>>>(s->pos[in], s->vel[in], s->mass[in], hp, hv, hm,
                                                             (uint32_t)s->n, s->d_err, s->h_err);
        GS_CUDA(cudaGetLastError());
        ++s->kernel_launches;
        GS_CUDA(cudaEventRecord(s->batch_done, s->stream));
        s->batch_pending = true;
        gs_status w = wait_event(s->batch_done, s->timeout_ns);
        if (w != GS_OK) return w;
        s->batch_pending = false;
        if (s->profile_pending) {
            gs_status a = account_profile(s);
            if (a != GS_OK) return a;
        }
        return device_error(*s->h_err);
    }
    if (s->batch_pending) {
        gs_status w = wait_event(s->batch_done, s->timeout_ns);
        if (w != GS_OK) return w;
        s->batch_pending = false;
    }
    if (s->profile_pending) {
        gs_status a = account_profile(s);
        if (a != GS_OK) return a;
    }
    gs_status st = check_device_error(s);
    if (st != GS_OK) return st;
    // copies in order on the stream, one synchronisation for all three
    if (pos) GS_CUDA(cudaMemcpyAsync(pos, s->pos[in], s->n * sizeof(float2), cudaMemcpyDeviceToHost, s->stream));
    if (vel) GS_CUDA(cudaMemcpyAsync(vel, s->vel[in], s->n * sizeof(float2), cudaMemcpyDeviceToHost, s->stream));
    if (mass) GS_CUDA(cudaMemcpyAsync(mass, s->mass[in], s->n * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    return sim_wait(s);
}

gs_status gs_set_particles(gs_sim* s, const float* pos, const float* vel, const float* mass) {
    if (!s) return invalid("gs_set_particles: sim is NULL");
    if (!pos || !mass) return invalid("gs_set_particles: pos_xy and mass are required");
    GS_CUDA(cudaSetDevice(s->device));
    follow_batch(s);
    s->own_work = true;
    // enqueued behind the submitted steps (stream order); the upload's synchronisation
    // covers them, and its kernel reports their error word
    gs_status st = upload(s, pos, vel, mass);
    if (st != GS_OK) return st;
    s->batch_pending = false;
    if (s->profile_pending) {
        st = account_profile(s);
        if (st != GS_OK) return st;
    }
    return device_error(*s->h_err);
}

gs_status gs_get_accel(gs_sim* s, float* acc) {
    if (!s || !acc) return invalid("gs_get_accel: NULL argument");
    if (!s->acc) return invalid("gs_get_accel: create the simulation with GS_FLAG_RECORD_ACCEL");
    gs_status st = gs_sync(s, 0);
    if (st != GS_OK) return st;
    GS_CUDA(cudaMemcpyAsync(acc, s->acc, s->n * sizeof(float2), cudaMemcpyDeviceToHost, s->stream));
    return sim_wait(s);
}

gs_status gs_get_stats(gs_sim* s, gs_stats* out) {
    if (!s || !out) return invalid("gs_get_stats: NULL argument");
    gs_status st = gs_sync(s, 0);
    if (st != GS_OK) return st;
    *out = s->stats;
    out->steps_done = s->steps_done;
    out->kernel_launches = s->kernel_launches;
    if (s->p.algorithm == GS_BARNES_HUT && s->steps_done) {
        uint64_t nv, internal, inter, vis, nodes;
        st = bh_read_counts(s, &nv, &internal, &inter, &vis, &nodes);
        if (st != GS_OK) return st;
        out->placed_particles = nv;
        out->internal_nodes = internal;
        out->tree_records = nv + internal;
        out->interactions = inter;
        out->warp_visits = vis;
        out->node_interactions = nodes;
    }
    return GS_OK;
}

gs_status gs_reset_stats(gs_sim* s) {
    if (!s) return invalid("gs_reset_stats: sim is NULL");
    std::memset(&s->stats, 0, sizeof s->stats);
    return GS_OK;
}

void gs_shape_defaults(gs_shape* out) {
    if (!out) return;
    out->sort_keys_per_thread = 16;
    out->sort_lookback = 32;
    out->scan_lookback = 32;
    out->force_warps = 2;
    out->force_short_lists = 0;
    out->direct_targets = 2;
    out->direct_blocks_per_sm = 12;
    out->moment_blocks_per_sm = 2;
}

gs_status gs_get_shape(gs_sim* s, gs_shape* out) {
    if (!s || !out) return invalid("gs_get_shape: NULL argument");
    *out = s->shape;
    return GS_OK;
}

gs_status gs_set_shape(gs_sim* s, const gs_shape* sh) {
    if (!s || !sh) return invalid("gs_set_shape: NULL argument");
    std::string why;
    if (!shape_valid(*sh, &why)) return invalid(("gs_set_shape: " + why).c_str());
    if (s->p.algorithm == GS_DIRECT_SUM && direct_chunks_needed(s, *sh) > s->direct_max_chunks) {
        set_error("gs_set_shape: direct_blocks_per_sm needs more j-chunk scratch than the system was created with");
        return GS_ERR_CAPACITY;
    }
    GS_CUDA(cudaSetDevice(s->device));
    if (s->batch_pending) {  // captured graphs may be running: wait before dropping them
        gs_status w = wait_event(s->batch_done, s->timeout_ns);
        if (w != GS_OK) return w;
        s->batch_pending = false;
    }
    for (auto& g : s->graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    s->shape = *sh;
    return GS_OK;
}

gs_status gs_set_timeout(gs_sim* s, uint64_t timeout_ns) {
    if (!s) return invalid("gs_set_timeout: sim is NULL");
    s->timeout_ns = timeout_ns;
    return GS_OK;
}

uint64_t gs_particle_count(const gs_sim* s) { return s ? s->n : 0; }
uint64_t gs_aligned_particle_count(const gs_sim* s) { return s ? s->n_al : 0; }
void* gs_stream(gs_sim* s) { return s ? (void*)s->stream : nullptr; }

void gs_destroy(gs_sim* s) { free_sim(s); }

gs_status gs_accel_f64(gs_sim* s, uint32_t n_targets, const uint32_t* targets, double* acc) {
    if (!s || !targets || !acc) return invalid("gs_accel_f64: NULL argument");
    if (!n_targets) return GS_OK;
    for (uint32_t t = 0; t < n_targets; ++t)
        if (targets[t] >= s->n) return invalid("gs_accel_f64: target index out of range");
    gs_status st = gs_sync(s, 0);
    if (st != GS_OK) return st;
    s->own_work = true;
    uint32_t* dt = nullptr;
    double2* dout = nullptr;
    GS_CUDA(cudaMallocAsync(&dt, n_targets * sizeof(uint32_t), s->stream));
    cudaError_t e = cudaMallocAsync(&dout, n_targets * sizeof(double2), s->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dt, targets, n_targets * sizeof(uint32_t), cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = accel_f64(s, n_targets, dt, dout);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(acc, dout, n_targets * sizeof(double2), cudaMemcpyDeviceToHost, s->stream);
    if (dt) cudaFreeAsync(dt, s->stream);
    if (dout) cudaFreeAsync(dout, s->stream);
    GS_CUDA(e);
    return sim_wait(s);
}

gs_status gs_energy_f64(gs_sim* s, double* kinetic, double* potential) {
    if (!s || !kinetic || !potential) return invalid("gs_energy_f64: NULL argument");
    gs_status st = gs_sync(s, 0);
    if (st != GS_OK) return st;
    s->own_work = true;
    return energy_f64(s, kinetic, potential);
}

gs_status gs_debug_state(gs_sim* s, float* pos, float* vel, float* mass, float* amag) {
    if (!s) return invalid("gs_debug_state: sim is NULL");
    gs_status st = gs_sync(s, 0);
    if (st != GS_OK) return st;
    const int in = s->in;
    const size_t n = s->n_al;
    if (pos) GS_CUDA(cudaMemcpyAsync(pos, s->pos[in], n * sizeof(float2), cudaMemcpyDeviceToHost, s->stream));
    if (vel) GS_CUDA(cudaMemcpyAsync(vel, s->vel[in], n * sizeof(float2), cudaMemcpyDeviceToHost, s->stream));
    if (mass) GS_CUDA(cudaMemcpyAsync(mass, s->mass[in], n * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    const float* d_amag = s->p.algorithm == GS_BARNES_HUT ? s->bh.amag : nullptr;
    if (amag && d_amag) GS_CUDA(cudaMemcpyAsync(amag, d_amag, n * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    st = sim_wait(s);
    if (st != GS_OK) return st;
    if (amag && !d_amag)
        for (size_t i = 0; i < n; ++i) amag[i] = std::nanf("");
    return GS_OK;
}

gs_status gs_debug_bh_tree(gs_sim* s, uint32_t* keys, uint32_t* sorted_src, uint32_t* node_skip, float* node_radius,
                           float* node_pos, float* node_mass, float* node_quad, uint64_t capacity,
                           uint64_t* tree_records) {
    if (!s) return invalid("gs_debug_bh_tree: sim is NULL");
    if (s->p.algorithm != GS_BARNES_HUT) return invalid("gs_debug_bh_tree: not a Barnes-Hut simulation");
    gs_status st = gs_sync(s, 0);
    if (st != GS_OK) return st;
    return bh_debug_tree(s, keys, sorted_src, node_skip, node_radius, node_pos, node_mass, node_quad, capacity,
                         tree_records);
}

}  // extern "C"
