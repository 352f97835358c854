// render.cu -- headless point splat and snapshot ring.
//
// The reference draws every particle as a one-pixel white point over a black clear
// (src/Graphics/Shaders/VertShader.vert:13-18, FragShader.frag:1-7, draw setup in
// src/Graphics/GraphicsPipeline.cpp:287-391) into a swapchain image.  Here the same
// arithmetic writes a device framebuffer of width x height bytes (0 or 255), which the
// caller reads back or saves as a binary PPM.  No graphics API is involved.
//
//   screen = (pos - camera_pos) / camera_size;  screen.y = -screen.y      (VertShader.vert:14-15)
//   framebuffer x = (screen.x + 1) * width / 2, y = (screen.y + 1) * height / 2
//                                                      (the viewport transform of the draw)
//   the point covers pixel (floor(x), floor(y)) when 0 <= x < width and 0 <= y < height
//
// Every covering write stores the same value, so the image does not depend on the order
// of the writes.  The reference's graphics path reads one of three particle buffer sets
// while compute uses the other two (src/Particles/ParticleSystem.hpp:146-174); the
// snapshot ring below plays that part: a snapshot is a stream-ordered copy of the current
// positions, and it is read or rendered on a side stream while the simulation goes on.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "internal.cuh"

namespace gsim {
namespace {

__global__ void __launch_bounds__(256)
k_splat(const float2* __restrict__ pos, uint32_t n, float cx, float cy, float cw, float ch, uint32_t width,
        uint32_t height, uint8_t* __restrict__ fb) {
    const float hw = __fmul_rn(0.5f, (float)width), hh = __fmul_rn(0.5f, (float)height);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float2 p = pos[i];
        const float sx = __fdiv_rn(__fsub_rn(p.x, cx), cw);
        const float sy = -__fdiv_rn(__fsub_rn(p.y, cy), ch);
        const float fx = __fmul_rn(__fadd_rn(sx, 1.0f), hw);
        const float fy = __fmul_rn(__fadd_rn(sy, 1.0f), hh);
        if (!(fx >= 0.0f && fx < (float)width && fy >= 0.0f && fy < (float)height)) continue;  // also NaN
        const uint32_t x = (uint32_t)fx, y = (uint32_t)fy;  // floor of a non-negative value
        if (x < width && y < height) fb[(size_t)y * width + x] = 255u;
    }
}

int splat_blocks(uint64_t n) {
    const uint64_t b = (n + 255) / 256;
    return (int)(b < 1 ? 1 : b > 152ull * 8 ? 152ull * 8 : b);
}

}  // namespace

// Render n particle positions (device) into the device framebuffer fb on stream st.
cudaError_t splat(const float2* pos, uint32_t n, const float* cam, uint32_t width, uint32_t height, uint8_t* fb,
                  cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(fb, 0, (size_t)width * height, st);
    if (e != cudaSuccess || !n) return e;
    k_splat<<<splat_blocks(n), 256, 0, st>>>(pos, n, cam[0], cam[1], cam[2], cam[3], width, height, fb);
    return cudaGetLastError();
}

}  // namespace gsim

using namespace gsim;

// one snapshot ring per system, created on first use
struct SnapshotRing {
    int device = 0;
    uint32_t slots = 0;
    uint64_t n = 0;
    float2* pos = nullptr;  // [slots][n]
    std::vector<cudaEvent_t> ready;
    std::vector<uint64_t> ticket_of;  // ticket held by each slot (0: none)
    uint64_t next_ticket = 1;
    cudaStream_t reader = nullptr;  // reads and renders, beside the simulation stream
    uint8_t* fb = nullptr;          // device framebuffer
    size_t fb_bytes = 0;
};

namespace {

std::mutex g_rings_mu;
std::vector<std::pair<const gs_sim*, SnapshotRing*>> g_rings;

SnapshotRing* find_ring(const gs_sim* s) {
    std::lock_guard<std::mutex> lock(g_rings_mu);
    for (auto& kv : g_rings)
        if (kv.first == s) return kv.second;
    return nullptr;
}

gs_status bad(const char* msg) {
    set_error(msg);
    return GS_ERR_INVALID_ARGUMENT;
}

gs_status check_view(uint32_t width, uint32_t height, const float* cam) {
    if (!width || !height || width > 32768 || height > 32768) return bad("render: width and height must be 1..32768");
    if (!cam) return bad("render: camera is NULL");
    if (!(cam[2] != 0.0f) || !(cam[3] != 0.0f)) return bad("render: camera size must be non-zero");
    return GS_OK;
}

gs_status ensure_fb(SnapshotRing* r, uint32_t width, uint32_t height) {
    const size_t bytes = (size_t)width * height;
    if (r->fb_bytes >= bytes) return GS_OK;
    if (r->fb) cudaFreeAsync(r->fb, r->reader);
    r->fb = nullptr;
    r->fb_bytes = 0;
    GS_CUDA(cudaMallocAsync((void**)&r->fb, bytes, r->reader));
    r->fb_bytes = bytes;
    return GS_OK;
}

}  // namespace

namespace gsim {
// called by gs_destroy
void free_snapshot_ring(const gs_sim* s) {
    SnapshotRing* r = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_rings_mu);
        for (size_t i = 0; i < g_rings.size(); ++i)
            if (g_rings[i].first == s) {
                r = g_rings[i].second;
                g_rings.erase(g_rings.begin() + (long)i);
                break;
            }
    }
    if (!r) return;
    cudaSetDevice(r->device);
    if (r->pos) cudaFreeAsync(r->pos, r->reader);  // stream-ordered after every read
    if (r->fb) cudaFreeAsync(r->fb, r->reader);
    (void)wait_stream(r->reader, s->timeout_ns);
    for (auto e : r->ready)
        if (e) cudaEventDestroy(e);
    cudaStreamDestroy(r->reader);
    delete r;
}
}  // namespace gsim

extern "C" {

gs_status gs_camera_start(gs_sim* s, float* camera) {
    if (!s || !camera) return bad("gs_camera_start: NULL argument");
    std::vector<float> pos(2 * s->n);
    gs_status st = gs_get_particles(s, pos.data(), nullptr, nullptr);
    if (st != GS_OK) return st;
    // ParticleSystem::GetCameraInfo (src/Particles/ParticleSystem.cpp:408-435)
    float mnx = INFINITY, mny = INFINITY, mxx = -INFINITY, mxy = -INFINITY;
    for (uint64_t i = 0; i < s->n; ++i) {
        const float x = pos[2 * i], y = pos[2 * i + 1];
        if (x < mnx) mnx = x;
        if (x > mxx) mxx = x;
        if (y < mny) mny = y;
        if (y > mxy) mxy = y;
    }
    const float width = mxx - mnx, height = mxy - mny;
    camera[0] = (mnx + mxx) * 0.5f;
    camera[1] = (mny + mxy) * 0.5f;
    camera[2] = width > height ? width : height;
    camera[3] = camera[2];
    return GS_OK;
}

gs_status gs_render_points(gs_sim* s, uint32_t width, uint32_t height, const float* camera, uint8_t* image) {
    if (!s || !image) return bad("gs_render_points: NULL argument");
    gs_status st = check_view(width, height, camera);
    if (st != GS_OK) return st;
    st = gs_sync(s, 0);
    if (st != GS_OK) return st;
    uint8_t* fb = nullptr;
    const size_t bytes = (size_t)width * height;
    GS_CUDA(cudaMallocAsync((void**)&fb, bytes, s->stream));
    cudaError_t e = splat(s->pos[s->in], (uint32_t)s->n, camera, width, height, fb, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(image, fb, bytes, cudaMemcpyDeviceToHost, s->stream);
    cudaFreeAsync(fb, s->stream);
    GS_CUDA(e);
    return sim_wait(s);
}

gs_status gs_snapshot_take(gs_sim* s, uint32_t slots, uint64_t* ticket) {
    if (!s || !ticket) return bad("gs_snapshot_take: NULL argument");
    if (!slots || slots > 64) return bad("gs_snapshot_take: slots must be 1..64");
    GS_CUDA(cudaSetDevice(s->device));
    SnapshotRing* r = find_ring(s);
    if (r && r->slots != slots) return bad("gs_snapshot_take: the ring of this system has another slot count");
    if (!r) {
        r = new (std::nothrow) SnapshotRing();
        if (!r) return bad("gs_snapshot_take: host allocation failed");
        r->device = s->device;
        r->slots = slots;
        r->n = s->n;
        r->ready.assign(slots, nullptr);
        r->ticket_of.assign(slots, 0);
        cudaError_t e = cudaStreamCreateWithFlags(&r->reader, cudaStreamNonBlocking);
        for (uint32_t k = 0; k < slots && e == cudaSuccess; ++k)
            e = cudaEventCreateWithFlags(&r->ready[k], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaMallocAsync((void**)&r->pos, (size_t)slots * s->n * sizeof(float2), s->stream);
        if (e != cudaSuccess) {
            for (auto ev : r->ready)
                if (ev) cudaEventDestroy(ev);
            if (r->reader) cudaStreamDestroy(r->reader);
            delete r;
            return cuda_fail(e, "gs_snapshot_take");
        }
        std::lock_guard<std::mutex> lock(g_rings_mu);
        g_rings.emplace_back(s, r);
    }
    const uint64_t t = r->next_ticket++;
    const uint32_t k = (uint32_t)(t % slots);
    // the slot's previous readers (on the reader stream) finish before it is overwritten
    GS_CUDA(cudaEventRecord(r->ready[k], r->reader));
    GS_CUDA(cudaStreamWaitEvent(s->stream, r->ready[k], 0));
    // after every step submitted so far, before any submitted later (stream order)
    GS_CUDA(cudaMemcpyAsync(r->pos + (size_t)k * r->n, s->pos[s->in], r->n * sizeof(float2),
                            cudaMemcpyDeviceToDevice, s->stream));
    GS_CUDA(cudaEventRecord(r->ready[k], s->stream));
    s->own_work = true;
    r->ticket_of[k] = t;
    *ticket = t;
    return GS_OK;
}

namespace {
gs_status ring_slot(gs_sim* s, uint64_t ticket, SnapshotRing** out, uint32_t* slot) {
    SnapshotRing* r = find_ring(s);
    if (!r) return bad("gs_snapshot: no snapshot has been taken on this system");
    const uint32_t k = (uint32_t)(ticket % r->slots);
    if (!ticket || r->ticket_of[k] != ticket) {
        set_error("gs_snapshot: the snapshot was overwritten by a later one (or never taken)");
        return GS_ERR_CAPACITY;
    }
    *out = r;
    *slot = k;
    return GS_OK;
}
}  // namespace

gs_status gs_snapshot_positions(gs_sim* s, uint64_t ticket, float* pos_xy) {
    if (!s || !pos_xy) return bad("gs_snapshot_positions: NULL argument");
    SnapshotRing* r;
    uint32_t k;
    gs_status st = ring_slot(s, ticket, &r, &k);
    if (st != GS_OK) return st;
    GS_CUDA(cudaSetDevice(s->device));
    GS_CUDA(cudaStreamWaitEvent(r->reader, r->ready[k], 0));
    GS_CUDA(cudaMemcpyAsync(pos_xy, r->pos + (size_t)k * r->n, r->n * sizeof(float2), cudaMemcpyDeviceToHost,
                            r->reader));
    return wait_stream(r->reader, s->timeout_ns);
}

gs_status gs_snapshot_render(gs_sim* s, uint64_t ticket, uint32_t width, uint32_t height, const float* camera,
                             uint8_t* image) {
    if (!s || !image) return bad("gs_snapshot_render: NULL argument");
    gs_status st = check_view(width, height, camera);
    if (st != GS_OK) return st;
    SnapshotRing* r;
    uint32_t k;
    st = ring_slot(s, ticket, &r, &k);
    if (st != GS_OK) return st;
    GS_CUDA(cudaSetDevice(s->device));
    st = ensure_fb(r, width, height);
    if (st != GS_OK) return st;
    GS_CUDA(cudaStreamWaitEvent(r->reader, r->ready[k], 0));
    GS_CUDA(splat(r->pos + (size_t)k * r->n, (uint32_t)r->n, camera, width, height, r->fb, r->reader));
    GS_CUDA(cudaMemcpyAsync(image, r->fb, (size_t)width * height, cudaMemcpyDeviceToHost, r->reader));
    return wait_stream(r->reader, s->timeout_ns);
}

gs_status gs_write_ppm(const char* path, uint32_t width, uint32_t height, const uint8_t* image) {
    if (!path || !image || !width || !height) return bad("gs_write_ppm: invalid argument");
    FILE* f = std::fopen(path, "wb");
    if (!f) {
        set_error(std::string("gs_write_ppm: cannot open ") + path);
        return GS_ERR_IO;
    }
    std::fprintf(f, "P6\n%u %u\n255\n", width, height);
    std::vector<uint8_t> row(3 * (size_t)width);
    bool ok = true;
    for (uint32_t y = 0; y < height && ok; ++y) {
        for (uint32_t x = 0; x < width; ++x) {
            const uint8_t v = image[(size_t)y * width + x];  // white points, black clear
            row[3 * x] = row[3 * x + 1] = row[3 * x + 2] = v;
        }
        ok = std::fwrite(row.data(), 1, row.size(), f) == row.size();
    }
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) {
        set_error(std::string("gs_write_ppm: write failed for ") + path);
        return GS_ERR_IO;
    }
    return GS_OK;
}

}  // extern "C"
