// tune.cu -- launch-shape autotuner and the tuned table (gs_tune_shape, gs_tune_batch_shape,
// gs_load_shape_cache).
//
// The reference fixes its workgroup sizes at compile time
// (src/Simulation/BarnesHut/BarnesHutSimulation.cpp:9-10, src/Simulation/Direct/DirectSimulation.cpp:9).
// Here every kernel shape that can vary without changing a result bit is a gs_shape field,
// and the tuner measures which values are fastest for a workload on this device:
//   - coordinate descent from the defaults: each knob in turn takes each of its values with
//     the others at their best so far, and keeps the fastest;
//   - a candidate's time is the median of `steps` device-timed steps (CUDA events on the
//     system's stream), each after a 256 MiB write that flushes L2, after 3 warm steps;
//   - winners are kept in a process-wide table keyed by device, algorithm, box mode, key
//     bits, math mode, the accurate / relative / plain-sum flags and floor(log2 N), which
//     gs_create and gs_batch_create consult, and written to a JSON cache file on request.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "internal.cuh"

namespace gsim {
namespace {

constexpr int kAlgoBatch = 2;  // table entries of a batch's kernels
constexpr uint32_t kKeyFlags = GS_FLAGS_ACCURATE | GS_FLAG_RELATIVE_MAC | GS_FLAG_PLAIN_SUM;

struct Key {
    std::string device;
    int sms = 0, algorithm = 0, box_mode = 0, key_bits = 0, math = 0;
    uint32_t flags = 0;
    int bucket = 0;
    bool operator==(const Key& o) const {
        return device == o.device && sms == o.sms && algorithm == o.algorithm && box_mode == o.box_mode &&
               key_bits == o.key_bits && math == o.math && flags == o.flags && bucket == o.bucket;
    }
};

struct Entry {
    Key key;
    gs_shape shape;
    double best_ms = 0, default_ms = 0;
};

std::mutex g_mu;
std::vector<Entry> g_table;

int log2_bucket(uint64_t n) {
    int b = 0;
    while (n > 1) {
        n >>= 1;
        ++b;
    }
    return b;
}

bool device_ident(int dev, std::string* name, int* sms) {
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    *name = prop.name;
    *sms = prop.multiProcessorCount;
    return true;
}

bool key_of(const gs_params* p, int algorithm, uint64_t n, Key* k) {
    if (!device_ident(p->device, &k->device, &k->sms)) return false;
    k->algorithm = algorithm;
    const bool bh = p->algorithm == GS_BARNES_HUT;
    k->box_mode = bh ? p->box_mode : 0;
    k->key_bits = bh && p->box_mode == GS_BOX_BOUNDING ? (p->key_bits ? p->key_bits : kBBoxBits) : 0;
    k->math = p->math_mode;
    k->flags = p->flags & kKeyFlags;
    k->bucket = log2_bucket(n);
    return true;
}

void table_put(const Entry& e) {
    std::lock_guard<std::mutex> lock(g_mu);
    for (auto& x : g_table)
        if (x.key == e.key) {
            x = e;
            return;
        }
    g_table.push_back(e);
}

bool table_get(const Key& k, gs_shape* out) {
    std::lock_guard<std::mutex> lock(g_mu);
    for (const auto& x : g_table)
        if (x.key == k) {
            *out = x.shape;
            return true;
        }
    return false;
}

// ---- the JSON cache: {"format": "gsim-shapes-1", "entries": [ one object per line ]} ----
const char* kShapeFields[] = {"sort_keys_per_thread", "sort_lookback", "scan_lookback", "force_warps",
                              "force_short_lists", "direct_targets", "direct_blocks_per_sm", "moment_blocks_per_sm"};
uint32_t* shape_field(gs_shape& s, int i) {
    uint32_t* f[] = {&s.sort_keys_per_thread, &s.sort_lookback, &s.scan_lookback, &s.force_warps,
                     &s.force_short_lists, &s.direct_targets, &s.direct_blocks_per_sm, &s.moment_blocks_per_sm};
    return f[i];
}

std::string json_escape(const std::string& v) {
    std::string o;
    for (char c : v) {
        if (c == '"' || c == '\\') o += '\\';
        if ((unsigned char)c >= 0x20) o += c;
    }
    return o;
}

gs_status write_cache(const char* path) {
    std::vector<Entry> t;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        t = g_table;
    }
    const std::string tmp = std::string(path) + ".tmp";
    FILE* f = std::fopen(tmp.c_str(), "w");
    if (!f) {
        set_error(std::string("cannot write the shape cache ") + path);
        return GS_ERR_IO;
    }
    std::fprintf(f, "{\"format\": \"gsim-shapes-1\", \"entries\": [\n");
    for (size_t i = 0; i < t.size(); ++i) {
        const Entry& e = t[i];
        std::fprintf(f,
                     "{\"device\": \"%s\", \"sms\": %d, \"algorithm\": %d, \"box_mode\": %d, \"key_bits\": %d, "
                     "\"math\": %d, \"flags\": %u, \"n_bucket\": %d",
                     json_escape(e.key.device).c_str(), e.key.sms, e.key.algorithm, e.key.box_mode, e.key.key_bits,
                     e.key.math, e.key.flags, e.key.bucket);
        gs_shape s = e.shape;
        for (int k = 0; k < 8; ++k) std::fprintf(f, ", \"%s\": %u", kShapeFields[k], *shape_field(s, k));
        std::fprintf(f, ", \"best_ms\": %.6f, \"default_ms\": %.6f}%s\n", e.best_ms, e.default_ms,
                     i + 1 < t.size() ? "," : "");
    }
    std::fprintf(f, "]}\n");
    const bool ok = std::fclose(f) == 0;
    if (!ok || std::rename(tmp.c_str(), path) != 0) {
        set_error(std::string("cannot write the shape cache ") + path);
        return GS_ERR_IO;
    }
    return GS_OK;
}

// value of "name": in one entry line (numbers), false when absent
bool json_number(const char* line, const char* name, double* v) {
    const std::string pat = std::string("\"") + name + "\":";
    const char* at = std::strstr(line, pat.c_str());
    if (!at) return false;
    char* end = nullptr;
    *v = std::strtod(at + pat.size(), &end);
    return end != at + pat.size();
}

bool json_string(const char* line, const char* name, std::string* v) {
    const std::string pat = std::string("\"") + name + "\": \"";
    const char* at = std::strstr(line, pat.c_str());
    if (!at) return false;
    v->clear();
    for (const char* c = at + pat.size(); *c && *c != '"'; ++c) {
        if (*c == '\\' && c[1]) ++c;
        *v += *c;
    }
    return true;
}

const char* cache_path_of(const char* path) {
    if (path && *path) return path;
    const char* env = std::getenv("GSIM_SHAPE_CACHE");
    return env && *env ? env : nullptr;
}

// ---- timing ----
struct Flush {  // 256 MiB written before every timed step: larger than L2
    void* buf = nullptr;
    size_t bytes = 256u << 20;
    ~Flush() {
        if (buf) cudaFree(buf);
    }
};

// median milliseconds of `steps` device-timed steps of `run` on `st` (after 3 warm ones)
template <typename Run>
gs_status time_steps(cudaStream_t st, Flush& fl, uint32_t steps, Run run, double* ms) {
    for (int w = 0; w < 3; ++w) {
        gs_status r = run();
        if (r != GS_OK) return r;
    }
    cudaEvent_t a = nullptr, b = nullptr;
    GS_CUDA(cudaEventCreate(&a));
    cudaError_t e = cudaEventCreate(&b);
    std::vector<float> t;
    gs_status r = GS_OK;
    for (uint32_t k = 0; k < steps && r == GS_OK && e == cudaSuccess; ++k) {
        e = cudaMemsetAsync(fl.buf, (int)(k & 0xff), fl.bytes, st);
        if (e == cudaSuccess) e = cudaEventRecord(a, st);
        if (e == cudaSuccess) r = run();
        if (r == GS_OK && e == cudaSuccess) e = cudaEventRecord(b, st);
        if (r == GS_OK && e == cudaSuccess) r = wait_event(b, 0);
        float x = 0;
        if (r == GS_OK && e == cudaSuccess) e = cudaEventElapsedTime(&x, a, b);
        t.push_back(x);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (r != GS_OK) return r;
    GS_CUDA(e);
    std::sort(t.begin(), t.end());
    *ms = t.empty() ? 0.0 : (double)t[t.size() / 2];
    return GS_OK;
}

// One knob: its field and the values the search tries.
struct Knob {
    int field;                    // index into shape_field, or -1: the (warps, short lists) pair
    std::vector<uint32_t> values;
};

// quadrupole mode: the moments come from exact sums (no cooperative moments launch), so
// the moments grid is not a knob
std::vector<Knob> knobs_for(int algorithm, bool group_walk, bool quadrupole) {
    std::vector<Knob> k;
    if (algorithm == GS_DIRECT_SUM) {
        k.push_back({5, {2, 4}});
        k.push_back({6, {4, 8, 12, 16, 24}});
        return k;
    }
    k.push_back({0, {8, 16}});
    k.push_back({1, {8, 16, 32}});
    k.push_back({2, {32, 64, 128}});
    if (group_walk) k.push_back({-1, {10, 20, 21, 40}});  // warps * 10 + short lists
    if (!quadrupole) k.push_back({7, {1, 2}});
    if (algorithm == kAlgoBatch) k.push_back({5, {2, 4}});  // the batch's direct-sum members
    return k;
}

void set_knob(gs_shape& s, const Knob& k, uint32_t v) {
    if (k.field < 0) {
        s.force_warps = v / 10;
        s.force_short_lists = v % 10;
    } else {
        *shape_field(s, k.field) = v;
    }
}

// Coordinate descent: `measure(shape, &ms)` times one candidate.
template <typename Measure>
gs_status descend(const std::vector<Knob>& knobs, Measure measure, gs_tune_result* out) {
    gs_shape best;
    gs_shape_defaults(&best);
    double best_ms = 0;
    gs_status r = measure(best, &best_ms);
    if (r != GS_OK) return r;
    out->default_ms = best_ms;
    out->candidates = 1;
    for (const Knob& k : knobs) {
        gs_shape base = best;
        for (uint32_t v : k.values) {
            gs_shape c = base;
            set_knob(c, k, v);
            if (std::memcmp(&c, &base, sizeof c) == 0) continue;  // the current best, measured already
            std::string why;
            if (!shape_valid(c, &why)) continue;
            double ms = 0;
            r = measure(c, &ms);
            if (r == GS_ERR_CAPACITY) continue;
            if (r != GS_OK) return r;
            ++out->candidates;
            if (ms < best_ms) {
                best_ms = ms;
                best = c;
            }
        }
    }
    out->best = best;
    out->best_ms = best_ms;
    return GS_OK;
}

thread_local const gs_shape* t_shape_override = nullptr;  // the tuner's creation shape

}  // namespace

bool shape_valid(const gs_shape& s, std::string* why) {
    auto bad = [&](const char* m) {
        if (why) *why = m;
        return false;
    };
    if (s.sort_keys_per_thread != 8 && s.sort_keys_per_thread != 16) return bad("sort_keys_per_thread must be 8 or 16");
    if (s.sort_lookback != 8 && s.sort_lookback != 16 && s.sort_lookback != 32)
        return bad("sort_lookback must be 8, 16 or 32");
    if (s.scan_lookback != 32 && s.scan_lookback != 64 && s.scan_lookback != 128)
        return bad("scan_lookback must be 32, 64 or 128");
    if (!force_shape_supported(s.force_warps, s.force_short_lists))
        return bad("force_warps must be 1, 2 or 4, and short lists need 2 warps");
    if (s.direct_targets != 2 && s.direct_targets != 4) return bad("direct_targets must be 2 or 4");
    if (s.direct_blocks_per_sm < 1 || s.direct_blocks_per_sm > 32) return bad("direct_blocks_per_sm must be 1..32");
    if (s.moment_blocks_per_sm != 1 && s.moment_blocks_per_sm != 2) return bad("moment_blocks_per_sm must be 1 or 2");
    return true;
}

void shape_for(const gs_params* p, uint64_t n, gs_shape* out) {
    if (t_shape_override) {
        *out = *t_shape_override;
        return;
    }
    gs_shape_defaults(out);
    Key k;
    if (key_of(p, p->algorithm, n, &k)) table_get(k, out);
}

// The batch's shape: the tuned entry of its total particles (keyed by its Barnes-Hut
// members' parameters, else the direct-sum ones), else the defaults.
void batch_shape_for(const gs_params* p, uint64_t total, gs_shape* out) {
    gs_shape_defaults(out);
    Key k;
    if (key_of(p, kAlgoBatch, total, &k)) table_get(k, out);
}

}  // namespace gsim

using namespace gsim;

extern "C" {

gs_status gs_tune_shape(const gs_params* params, uint64_t n, int32_t generator, uint64_t seed, uint32_t steps,
                        const char* cache_path, gs_tune_result* out) {
    if (!params || !out || !n) {
        set_error("gs_tune_shape: NULL argument or no particles");
        return GS_ERR_INVALID_ARGUMENT;
    }
    if (!steps) steps = 10;
    std::vector<float> pos(2 * n), vel(2 * n), mass(n);
    gs_status st = gs_generate(generator, n, 100.0f, 1.0f, 10.0f, params->gravitational_const, seed, pos.data(),
                               vel.data(), mass.data());
    if (st != GS_OK) return st;
    GS_CUDA(cudaSetDevice(params->device));
    Flush fl;
    GS_CUDA(cudaMalloc(&fl.buf, fl.bytes));
    gs_params p = *params;
    p.flags &= ~(uint32_t)(GS_FLAG_PROFILE | GS_FLAG_COUNT_INTERACTIONS | GS_FLAG_NO_GRAPH);
    const bool bh = p.algorithm == GS_BARNES_HUT;
    gs_sim* sim = nullptr;  // Barnes-Hut: one system, shapes switched by gs_set_shape
    auto measure = [&](const gs_shape& sh, double* ms) -> gs_status {
        if (!bh) {  // the direct sum's scratch depends on its creation shape: a system per candidate
            t_shape_override = &sh;
            gs_sim* d = nullptr;
            gs_status r = gs_create(&p, n, pos.data(), vel.data(), mass.data(), &d);
            t_shape_override = nullptr;
            if (r != GS_OK) return r;
            r = time_steps(d->stream, fl, steps, [&]() { return gs_run(d, 1); }, ms);
            gs_destroy(d);
            return r;
        }
        gs_status r = gs_set_shape(sim, &sh);
        if (r != GS_OK) return r;
        return time_steps(sim->stream, fl, steps, [&]() { return gs_run(sim, 1); }, ms);
    };
    if (bh) {
        st = gs_create(&p, n, pos.data(), vel.data(), mass.data(), &sim);
        if (st != GS_OK) return st;
    }
    std::memset(out, 0, sizeof *out);
    st = descend(knobs_for(p.algorithm, (p.flags & GS_FLAG_GROUP_WALK) != 0, (p.flags & GS_FLAG_QUADRUPOLE) != 0),
                 measure, out);
    if (sim) gs_destroy(sim);
    if (st != GS_OK) return st;
    Entry e;
    if (!key_of(&p, p.algorithm, n, &e.key)) {
        set_error("gs_tune_shape: cannot read the device properties");
        return GS_ERR_CUDA;
    }
    e.shape = out->best;
    e.best_ms = out->best_ms;
    e.default_ms = out->default_ms;
    table_put(e);
    const char* path = cache_path_of(cache_path);
    return path ? write_cache(path) : GS_OK;
}

gs_status gs_tune_batch_shape(gs_batch* b, uint32_t steps, const char* cache_path, gs_tune_result* out) {
    if (!b || !out) {
        set_error("gs_tune_batch_shape: NULL argument");
        return GS_ERR_INVALID_ARGUMENT;
    }
    if (!steps) steps = 5;
    gs_params key_params;
    uint64_t total = 0;
    gs_status st = batch_key(b, &key_params, &total);
    if (st != GS_OK) return st;
    gs_shape keep;
    st = gs_batch_get_shape(b, &keep);
    if (st != GS_OK) return st;
    GS_CUDA(cudaSetDevice(key_params.device));
    Flush fl;
    GS_CUDA(cudaMalloc(&fl.buf, fl.bytes));
    cudaStream_t bs = (cudaStream_t)gs_batch_stream(b);
    auto measure = [&](const gs_shape& sh, double* ms) -> gs_status {
        gs_status r = gs_batch_set_shape(b, &sh);
        if (r != GS_OK) return r;
        return time_steps(bs, fl, steps, [&]() { return gs_batch_run(b, 1); }, ms);
    };
    std::memset(out, 0, sizeof *out);
    st = descend(knobs_for(kAlgoBatch, (key_params.flags & GS_FLAG_GROUP_WALK) != 0,
                           (key_params.flags & GS_FLAG_QUADRUPOLE) != 0),
                 measure, out);
    if (st != GS_OK) {
        gs_batch_set_shape(b, &keep);
        return st;
    }
    st = gs_batch_set_shape(b, &out->best);
    if (st != GS_OK) return st;
    Entry e;
    if (!key_of(&key_params, kAlgoBatch, total, &e.key)) {
        set_error("gs_tune_batch_shape: cannot read the device properties");
        return GS_ERR_CUDA;
    }
    e.shape = out->best;
    e.best_ms = out->best_ms;
    e.default_ms = out->default_ms;
    table_put(e);
    const char* path = cache_path_of(cache_path);
    return path ? write_cache(path) : GS_OK;
}

gs_status gs_load_shape_cache(const char* path, uint32_t* entries) {
    const char* p = cache_path_of(path);
    if (!p) {
        set_error("gs_load_shape_cache: no path and GSIM_SHAPE_CACHE is not set");
        return GS_ERR_INVALID_ARGUMENT;
    }
    FILE* f = std::fopen(p, "r");
    if (!f) {
        set_error(std::string("gs_load_shape_cache: cannot open ") + p);
        return GS_ERR_IO;
    }
    uint32_t count = 0;
    char line[2048];
    while (std::fgets(line, sizeof line, f)) {
        if (!std::strstr(line, "\"device\":")) continue;
        Entry e;
        double v[8];
        const char* names[] = {"sms", "algorithm", "box_mode", "key_bits", "math", "flags", "n_bucket"};
        bool ok = json_string(line, "device", &e.key.device);
        for (int i = 0; i < 7 && ok; ++i) ok = json_number(line, names[i], &v[i]);
        if (!ok) continue;
        e.key.sms = (int)v[0];
        e.key.algorithm = (int)v[1];
        e.key.box_mode = (int)v[2];
        e.key.key_bits = (int)v[3];
        e.key.math = (int)v[4];
        e.key.flags = (uint32_t)v[5];
        e.key.bucket = (int)v[6];
        gs_shape_defaults(&e.shape);
        for (int k = 0; k < 8 && ok; ++k) {
            double x;
            if (json_number(line, kShapeFields[k], &x)) *shape_field(e.shape, k) = (uint32_t)x;
        }
        json_number(line, "best_ms", &e.best_ms);
        json_number(line, "default_ms", &e.default_ms);
        if (!shape_valid(e.shape, nullptr)) continue;
        table_put(e);
        ++count;
    }
    std::fclose(f);
    if (entries) *entries = count;
    return GS_OK;
}

void gs_clear_shape_table(void) {
    std::lock_guard<std::mutex> lock(g_mu);
    g_table.clear();
}

}  // extern "C"
