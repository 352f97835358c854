// serve.cu -- continuous batching of simulation requests (gs_server_*).  No counterpart
// in the reference, which runs one system per process (src/Main.cpp:250-321).
//
// One host thread drives the server.  Every gs_server_poll:
//   1. retires requests whose last batched step has finished on the GPU: reads their
//      final state back (keep_results), destroys the system (stream-ordered frees) and
//      returns its footprint to the budget;
//   2. admits queued requests whose inputs are ready (generated on worker threads) while
//      the sum of footprints (gs_footprint) stays within the memory budget and the sum of
//      N within max_resident_particles, in FIFO or shortest-first order;
//   3. enqueues ONE batched step over every member (BatchEngine: one launch per stage
//      over all members, the member set re-planned whenever it changed), at most
//      steps_in_flight steps ahead of the GPU.  A request leaves the member set right
//      after its last step is enqueued; an event recorded after that step tells step 1
//      when its state is final.
// A member computes exactly the bits it would compute alone with gs_run.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "batch.cuh"

using namespace gsim;

namespace {

struct Request {
    uint64_t id = 0;
    gs_request spec{};
    gs_params params{};
    uint64_t footprint = 0;
    std::vector<float> pos, vel, mass;  // inputs until admission, then the results
    std::atomic<int> ready{0};          // inputs made (1) or failed (-1)
    int state = GS_REQUEST_QUEUED;
    double arrival_s = 0, admit_s = -1, finish_s = -1;
    gs_sim* sim = nullptr;
    uint32_t steps_enqueued = 0;
    bool joined = false;         // the batch's root stream already follows the system's upload
    cudaEvent_t last = nullptr;  // recorded after the request's last step
    std::string error;
};

}  // namespace

struct gs_server {
    gs_server_config cfg{};
    BatchEngine eng;
    std::chrono::steady_clock::time_point t0;
    uint64_t next_id = 1;
    std::unordered_map<uint64_t, Request*> all;
    std::vector<Request*> queue;     // submitted, not admitted (arrival order)
    std::vector<Request*> members;   // resident, still stepping
    std::vector<Request*> draining;  // resident, every step enqueued
    bool dirty = false;
    std::deque<cudaEvent_t> inflight;  // one event per enqueued step, oldest first
    std::vector<cudaEvent_t> spare;
    // device time of the batched steps: a timing-event pair around each, summed once done
    std::deque<std::pair<cudaEvent_t, cudaEvent_t>> timed;
    std::vector<cudaEvent_t> spare_timing;
    gs_server_stats st{};
    // input generators
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Request*> jobs;
    std::vector<std::thread> workers;
    bool stopping = false;
};

namespace {

gs_status bad(const char* msg) {
    set_error(msg);
    return GS_ERR_INVALID_ARGUMENT;
}

double clock_of(const gs_server* s) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - s->t0).count();
}

void worker_main(gs_server* s) {
    for (;;) {
        Request* r = nullptr;
        {
            std::unique_lock<std::mutex> lock(s->mu);
            s->cv.wait(lock, [&] { return s->stopping || !s->jobs.empty(); });
            if (s->stopping && s->jobs.empty()) return;
            r = s->jobs.front();
            s->jobs.pop_front();
        }
        const uint64_t n = r->spec.particle_count;
        gs_status g = gs_generate(r->spec.generator, n, r->spec.generate_size, r->spec.min_mass, r->spec.max_mass,
                                  r->params.gravitational_const, r->spec.seed, r->pos.data(), r->vel.data(),
                                  r->mass.data());
        if (g != GS_OK) r->error = std::string("generator: ") + gs_status_string(g);
        r->ready.store(g == GS_OK ? 1 : -1, std::memory_order_release);
    }
}

cudaEvent_t take_event(gs_server* s) {
    if (!s->spare.empty()) {
        cudaEvent_t e = s->spare.back();
        s->spare.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    return e;
}

cudaEvent_t take_timing_event(gs_server* s) {
    if (!s->spare_timing.empty()) {
        cudaEvent_t e = s->spare_timing.back();
        s->spare_timing.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Adds the device time of finished batched steps to the statistics (no waiting).
void account_gpu_time(gs_server* s) {
    while (!s->timed.empty()) {
        auto [a, b] = s->timed.front();
        if (cudaEventQuery(b) != cudaSuccess) {
            (void)cudaGetLastError();
            break;
        }
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, a, b) == cudaSuccess) s->st.gpu_busy_seconds += 1e-3 * ms;
        s->spare_timing.push_back(a);
        s->spare_timing.push_back(b);
        s->timed.pop_front();
    }
}

void fail_request(gs_server* s, Request* r, const std::string& why) {
    r->state = GS_REQUEST_FAILED;
    r->error = why;
    r->finish_s = clock_of(s);
    ++s->st.failed;
}

void release(gs_server* s, Request* r) {
    if (r->sim) {
        s->st.memory_in_use -= r->footprint;
        s->st.resident_particles -= r->spec.particle_count;
        gs_destroy(r->sim);  // its stream waits on r->last: frees follow the last use
        r->sim = nullptr;
    }
    if (r->last) {
        s->spare.push_back(r->last);
        r->last = nullptr;
    }
}

// 1. requests whose last step has finished
gs_status retire(gs_server* s, uint32_t* finished) {
    for (size_t i = 0; i < s->draining.size();) {
        Request* r = s->draining[i];
        const cudaError_t q = cudaEventQuery(r->last);
        if (q == cudaErrorNotReady) {
            ++i;
            continue;
        }
        if (q != cudaSuccess) return cuda_fail(q, "gs_server_poll");
        const uint64_t n = r->spec.particle_count;
        gs_status g = GS_OK;
        if (s->cfg.keep_results) {
            r->pos.resize(2 * n);
            r->vel.resize(2 * n);
            r->mass.resize(n);
            g = gs_get_particles(r->sim, r->pos.data(), r->vel.data(), r->mass.data());
        } else {
            g = gs_sync(r->sim, 0);  // device-side error flags
        }
        if (g == GS_OK) {
            r->state = GS_REQUEST_DONE;
            r->finish_s = clock_of(s);
            ++s->st.finished;
            s->st.particle_steps += n * (uint64_t)r->spec.steps;
        } else {
            fail_request(s, r, gs_last_error());
        }
        release(s, r);
        s->draining.erase(s->draining.begin() + (long)i);
        --s->st.resident;
        if (finished) ++*finished;
    }
    return GS_OK;
}

// 2. admission
gs_status admit(gs_server* s) {
    if (s->cfg.policy == GS_SERVE_SHORTEST_FIRST)
        std::stable_sort(s->queue.begin(), s->queue.end(), [](const Request* a, const Request* b) {
            return a->spec.particle_count * (uint64_t)a->spec.steps < b->spec.particle_count * (uint64_t)b->spec.steps;
        });
    // A request that does not fit keeps its place: later ones are admitted only if they fit
    // beside everything queued ahead of them (conservative backfill, no starvation).
    uint64_t held_mem = 0, held_n = 0;
    for (size_t i = 0; i < s->queue.size();) {
        Request* r = s->queue[i];
        const int ready = r->ready.load(std::memory_order_acquire);
        if (ready < 0) {
            fail_request(s, r, r->error);
            --s->st.queued;
            s->queue.erase(s->queue.begin() + (long)i);
            continue;
        }
        if (!ready) {  // inputs still being made
            ++i;
            continue;
        }
        const uint64_t n = r->spec.particle_count;
        const uint64_t maxp = s->cfg.max_resident_particles;
        const bool fits = s->st.memory_in_use + held_mem + r->footprint <= s->cfg.memory_budget &&
                          (!maxp || s->st.resident_particles + held_n + n <= maxp ||
                           (s->st.resident == 0 && held_n == 0));
        if (!fits) {
            held_mem += r->footprint;
            held_n += n;
            ++i;
            continue;
        }
        gs_sim* sim = nullptr;
        gs_status g = gs_create(&r->params, n, r->pos.data(), r->vel.data(), r->mass.data(), &sim);
        if (g != GS_OK) {
            if (g == GS_ERR_OUT_OF_MEMORY && s->st.resident > 0) {  // wait for a slot to free up
                held_mem += r->footprint;
                held_n += n;
                ++i;
                continue;
            }
            fail_request(s, r, gs_last_error());
            --s->st.queued;
            s->queue.erase(s->queue.begin() + (long)i);
            continue;
        }
        std::vector<float>().swap(r->pos);  // inputs are on the device now
        std::vector<float>().swap(r->vel);
        std::vector<float>().swap(r->mass);
        r->sim = sim;
        r->state = GS_REQUEST_RESIDENT;
        r->admit_s = clock_of(s);
        s->st.memory_in_use += r->footprint;
        s->st.peak_memory_in_use = std::max(s->st.peak_memory_in_use, s->st.memory_in_use);
        s->st.resident_particles += n;
        s->st.peak_resident_particles = std::max(s->st.peak_resident_particles, s->st.resident_particles);
        --s->st.queued;
        ++s->st.resident;
        s->queue.erase(s->queue.begin() + (long)i);
        if (r->spec.steps == 0) {  // nothing to run: final at once
            r->last = take_event(s);
            GS_CUDA(cudaEventRecord(r->last, sim->stream));
            s->draining.push_back(r);
        } else {
            s->members.push_back(r);
            s->dirty = true;
        }
    }
    return GS_OK;
}

// 3. one batched step over the members
gs_status step(gs_server* s) {
    if (s->members.empty()) return GS_OK;
    const uint32_t depth = s->cfg.steps_in_flight ? s->cfg.steps_in_flight : 2;
    while (s->inflight.size() >= depth) {
        gs_status w = wait_event(s->inflight.front(), 0);
        if (w != GS_OK) return w;
        s->spare.push_back(s->inflight.front());
        s->inflight.pop_front();
    }
    if (s->dirty || !s->eng.in_step()) {
        std::vector<gs_sim*> sims;
        sims.reserve(s->members.size());
        for (Request* r : s->members) {
            if (!r->joined) {  // the system's work on its own stream precedes the batch
                cudaEvent_t e = take_event(s);
                GS_CUDA(cudaEventRecord(e, r->sim->stream));
                GS_CUDA(cudaStreamWaitEvent(s->eng.root, e, 0));
                s->spare.push_back(e);
                r->joined = true;
            }
            sims.push_back(r->sim);
        }
        gs_status g = s->eng.set_members(sims);
        if (g != GS_OK) return g;
        s->dirty = false;
        ++s->st.plan_changes;
    }
    cudaEvent_t t_begin = take_timing_event(s), t_end = take_timing_event(s);
    GS_CUDA(cudaEventRecord(t_begin, s->eng.root));
    GS_CUDA(s->eng.enqueue((uint32_t)(s->eng.step & 1), s->eng.needs_estimate()));
    GS_CUDA(cudaEventRecord(t_end, s->eng.root));
    s->timed.emplace_back(t_begin, t_end);
    s->eng.advance();
    ++s->st.batched_steps;
    cudaEvent_t done = take_event(s);
    GS_CUDA(cudaEventRecord(done, s->eng.root));
    s->inflight.push_back(done);
    for (size_t i = 0; i < s->members.size();) {
        Request* r = s->members[i];
        if (++r->steps_enqueued < r->spec.steps) {
            ++i;
            continue;
        }
        r->last = take_event(s);
        GS_CUDA(cudaEventRecord(r->last, s->eng.root));
        GS_CUDA(cudaStreamWaitEvent(r->sim->stream, r->last, 0));  // later calls on the system follow the batch
        s->draining.push_back(r);
        s->members.erase(s->members.begin() + (long)i);
        s->dirty = true;
    }
    return GS_OK;
}

void destroy_server(gs_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stopping = true;
        s->jobs.clear();  // inputs not yet made are not needed any more
    }
    s->cv.notify_all();
    for (auto& t : s->workers) t.join();
    cudaSetDevice(s->eng.device);
    if (s->eng.root) (void)wait_stream(s->eng.root, 0);
    for (auto& kv : s->all) {
        release(s, kv.second);
        delete kv.second;
    }
    for (auto e : s->inflight) cudaEventDestroy(e);
    for (auto e : s->spare) cudaEventDestroy(e);
    for (auto& ab : s->timed) {
        cudaEventDestroy(ab.first);
        cudaEventDestroy(ab.second);
    }
    for (auto e : s->spare_timing) cudaEventDestroy(e);
    s->eng.destroy();
    delete s;
}

}  // namespace

extern "C" {

gs_status gs_server_create(const gs_server_config* cfg, gs_server** out) {
    if (!out) return bad("gs_server_create: out is NULL");
    *out = nullptr;
    if (!cfg) return bad("gs_server_create: config is NULL");
    if (cfg->direct_params.algorithm != GS_DIRECT_SUM || cfg->bh_params.algorithm != GS_BARNES_HUT)
        return bad("gs_server_create: direct_params must select direct sum and bh_params Barnes-Hut");
    if (cfg->direct_params.device != cfg->bh_params.device)
        return bad("gs_server_create: direct_params and bh_params must name the same device");
    if (!cfg->memory_budget) return bad("gs_server_create: memory_budget is zero");
    if (cfg->policy != GS_SERVE_FIFO && cfg->policy != GS_SERVE_SHORTEST_FIRST)
        return bad("gs_server_create: unknown policy");
    gs_server* s = new (std::nothrow) gs_server();
    if (!s) return bad("gs_server_create: host allocation failed");
    s->cfg = *cfg;
    s->t0 = std::chrono::steady_clock::now();
    cudaError_t e = s->eng.init(cfg->bh_params.device);
    if (e != cudaSuccess) {
        gs_status st = cuda_fail(e, "gs_server_create");
        destroy_server(s);
        return st;
    }
    const uint32_t nw = cfg->worker_threads ? cfg->worker_threads : 4;
    for (uint32_t i = 0; i < nw; ++i) s->workers.emplace_back(worker_main, s);
    *out = s;
    return GS_OK;
}

gs_status gs_server_submit(gs_server* s, const gs_request* req, double arrival_s, uint64_t* id) {
    if (!s || !req) return bad("gs_server_submit: NULL argument");
    if (!req->particle_count) return bad("The simulation must contain at least one particle!");
    if (!req->pos_xy && (req->generator < 0 || (req->generator > 3 && (req->generator < 16 || req->generator > 18))))
        return bad("gs_server_submit: no particles and no valid generator");
    if (req->pos_xy && !req->mass) return bad("gs_server_submit: pos_xy given without mass");
    Request* r = new (std::nothrow) Request();
    if (!r) return bad("gs_server_submit: host allocation failed");
    const uint64_t n = req->particle_count;
    r->id = s->next_id++;
    r->spec = *req;
    r->spec.pos_xy = r->spec.vel_xy = r->spec.mass = nullptr;
    r->params = n < s->cfg.crossover ? s->cfg.direct_params : s->cfg.bh_params;
    r->footprint = gs_footprint(&r->params, n);
    r->arrival_s = arrival_s >= 0 ? arrival_s : clock_of(s);
    if (r->footprint > s->cfg.memory_budget) {
        delete r;
        set_error("gs_server_submit: the request's footprint exceeds the whole memory budget");
        return GS_ERR_CAPACITY;
    }
    try {
        r->pos.resize(2 * n);
        r->vel.resize(2 * n);
        r->mass.resize(n);
    } catch (...) {
        delete r;
        set_error("gs_server_submit: host allocation failed");
        return GS_ERR_OUT_OF_MEMORY;
    }
    s->all[r->id] = r;
    s->queue.push_back(r);
    ++s->st.submitted;
    ++s->st.queued;
    if (req->pos_xy) {
        std::memcpy(r->pos.data(), req->pos_xy, 2 * n * sizeof(float));
        if (req->vel_xy) std::memcpy(r->vel.data(), req->vel_xy, 2 * n * sizeof(float));
        std::memcpy(r->mass.data(), req->mass, n * sizeof(float));
        r->ready.store(1, std::memory_order_release);
    } else {
        {
            std::lock_guard<std::mutex> lock(s->mu);
            s->jobs.push_back(r);
        }
        s->cv.notify_one();
    }
    if (id) *id = r->id;
    return GS_OK;
}

gs_status gs_server_poll(gs_server* s, uint32_t* finished) {
    if (!s) return bad("gs_server_poll: server is NULL");
    if (finished) *finished = 0;
    GS_CUDA(cudaSetDevice(s->eng.device));
    account_gpu_time(s);
    gs_status g = retire(s, finished);
    if (g == GS_OK) g = admit(s);
    if (g == GS_OK) g = step(s);
    return g;
}

gs_status gs_server_request(gs_server* s, uint64_t id, gs_request_status* out) {
    if (!s || !out) return bad("gs_server_request: NULL argument");
    auto it = s->all.find(id);
    if (it == s->all.end()) return bad("gs_server_request: unknown request id");
    const Request* r = it->second;
    out->state = r->state;
    out->algorithm = r->params.algorithm;
    out->steps_enqueued = r->steps_enqueued;
    out->steps = r->spec.steps;
    out->particle_count = r->spec.particle_count;
    out->footprint = r->footprint;
    out->arrival_s = r->arrival_s;
    out->admit_s = r->admit_s;
    out->finish_s = r->finish_s;
    return GS_OK;
}

gs_status gs_server_result(gs_server* s, uint64_t id, float* pos, float* vel, float* mass) {
    if (!s) return bad("gs_server_result: server is NULL");
    auto it = s->all.find(id);
    if (it == s->all.end()) return bad("gs_server_result: unknown request id");
    const Request* r = it->second;
    if (r->state == GS_REQUEST_FAILED) {
        set_error("gs_server_result: the request failed: " + r->error);
        return GS_ERR_DEVICE;
    }
    if (r->state != GS_REQUEST_DONE) return bad("gs_server_result: the request has not finished");
    if (!s->cfg.keep_results) return bad("gs_server_result: the server keeps no results (keep_results = 0)");
    const uint64_t n = r->spec.particle_count;
    if (pos) std::memcpy(pos, r->pos.data(), 2 * n * sizeof(float));
    if (vel) std::memcpy(vel, r->vel.data(), 2 * n * sizeof(float));
    if (mass) std::memcpy(mass, r->mass.data(), n * sizeof(float));
    return GS_OK;
}

gs_status gs_server_get_stats(gs_server* s, gs_server_stats* out) {
    if (!s || !out) return bad("gs_server_get_stats: NULL argument");
    GS_CUDA(cudaSetDevice(s->eng.device));
    account_gpu_time(s);
    *out = s->st;
    return GS_OK;
}

double gs_server_clock(gs_server* s) { return s ? clock_of(s) : 0.0; }

gs_status gs_server_run_trace(gs_server* s, const gs_request* reqs, const double* arrival_s, uint32_t count,
                              double timeout_s, uint64_t* ids) {
    if (!s || (count && (!reqs || !arrival_s))) return bad("gs_server_run_trace: NULL argument");
    const double start = clock_of(s);
    std::vector<uint64_t> mine(count, 0);
    uint32_t next = 0;
    for (;;) {
        const double now = clock_of(s);
        while (next < count && start + arrival_s[next] <= now) {
            gs_status g = gs_server_submit(s, &reqs[next], start + arrival_s[next], &mine[next]);
            if (g != GS_OK) return g;
            if (ids) ids[next] = mine[next];
            ++next;
        }
        bool open = next < count;
        for (uint32_t i = 0; i < next && !open; ++i) {
            const int state = s->all[mine[i]]->state;
            open = state == GS_REQUEST_QUEUED || state == GS_REQUEST_RESIDENT;
        }
        if (!open) return GS_OK;
        if (timeout_s > 0 && now - start > timeout_s) {
            set_error("gs_server_run_trace: timed out");
            return GS_ERR_TIMEOUT;
        }
        const bool idle = s->members.empty() && s->draining.empty();
        gs_status g = gs_server_poll(s, nullptr);
        if (g != GS_OK) return g;
        if (idle && s->members.empty() && s->draining.empty()) {  // nothing on the GPU: wait a little
            double wait = next < count ? start + arrival_s[next] - clock_of(s) : 1e-4;
            wait = std::min(std::max(wait, 0.0), 1e-3);
            std::this_thread::sleep_for(std::chrono::duration<double>(wait));
        } else if (s->members.empty()) {
            std::this_thread::sleep_for(std::chrono::microseconds(50));  // only draining: let the GPU finish
        }
    }
}

void gs_server_destroy(gs_server* s) { destroy_server(s); }

}  // extern "C"
