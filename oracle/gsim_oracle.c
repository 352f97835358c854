/*
 * gsim_oracle.c -- CPU restatement of Gravity-Sim's per-step force-and-integrate path.
 *
 * TEST INFRASTRUCTURE ONLY (the tests' reference, never the product).  Compile with
 * -ffp-contract=off: every fused multiply-add below is written out with fmaf().
 *
 * What each function restates (paths relative to the reference project):
 *   orc_direct_step       src/Simulation/Direct/Shaders/SimShader.comp:37-74
 *   orc_bh_grid_step      src/Simulation/BarnesHut/Shaders/ClearShader.comp:71-83,
 *                         InitShader.comp:73-119, TreeInitShader.comp:58-90,
 *                         TreeSortShader.comp:57-94, TreeMoveShader.comp:53-84,
 *                         ParticleSortShader.comp:71-110, ForceShader.comp:78-152, in the
 *                         dispatch order of src/Simulation/BarnesHut/BarnesHutSimulation.cpp:782-825,885-918
 *   orc_bh_sorted_step    the same tree, built from stably sorted cell keys (the
 *                         construction the CUDA path uses), plus the bounding-box mode.
 *
 * Where the reference is nondeterministic this restatement fixes one meaning:
 *   - particles inside one finest cell are ordered by ascending original index (the
 *     reference orders them by atomic arrival, ParticleSortShader.comp:99-103);
 *   - a finest cell with k >= 2 particles has k + 1 records (InitShader.comp:104-106
 *     intends this, but its two separate atomics can race);
 *   - finest-cell mass and mass-moment sums add particles in ascending index order
 *     (the reference uses float atomics, InitShader.comp:107-109);
 *   - the root's preorder start is 0 (TreeSortShader.comp:72 reads a never-written slot).
 */
#include "gsim_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define WARP 32
#define SIM_SIZE 500.0f  /* BarnesHutSimulation.cpp:580 simulationSize */
#define GRID 1024u       /* BarnesHutSimulation.cpp:582 treeSize */
#define GRID_LEVELS 11   /* depths 0..10 */
#define BBOX_BITS 12     /* bounding-box mode default: 12 bits per axis, 24-bit keys */
#define BBOX_MAX_BITS 15 /* bounding-box mode maximum: 15 bits per axis, 30-bit keys */

/* ------------------------------------------------------------------------------ */
/* tiny parallel-for: dynamic chunks over [0, n), deterministic results because   */
/* every item writes only its own outputs                                          */
/* ------------------------------------------------------------------------------ */
typedef void (*item_fn)(void* ctx, uint64_t item, int worker);
typedef struct {
    item_fn fn;
    void* ctx;
    uint64_t n;
    uint64_t chunk;
    atomic_uint_fast64_t next;
    int worker;
} pf_job;
typedef struct {
    pf_job* job;
    int worker;
} pf_arg;

static void* pf_thread(void* p) {
    pf_arg* a = (pf_arg*)p;
    pf_job* j = a->job;
    for (;;) {
        uint64_t b = atomic_fetch_add(&j->next, j->chunk);
        if (b >= j->n) break;
        uint64_t e = b + j->chunk < j->n ? b + j->chunk : j->n;
        for (uint64_t i = b; i < e; ++i) j->fn(j->ctx, i, a->worker);
    }
    return NULL;
}

static void parallel_for(int nthreads, uint64_t n, uint64_t chunk, item_fn fn, void* ctx) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pf_job job;
    job.fn = fn;
    job.ctx = ctx;
    job.n = n;
    job.chunk = chunk ? chunk : 1;
    atomic_init(&job.next, 0);
    if (nthreads == 1) {
        pf_arg a = {&job, 0};
        pf_thread(&a);
        return;
    }
    pthread_t th[256];
    pf_arg args[256];
    int started = 0;
    for (int t = 1; t < nthreads; ++t) {
        args[t].job = &job;
        args[t].worker = t;
        if (pthread_create(&th[t], NULL, pf_thread, &args[t]) != 0) break;
        started = t;
    }
    args[0].job = &job;
    args[0].worker = 0;
    pf_thread(&args[0]);
    for (int t = 1; t <= started; ++t) pthread_join(th[t], NULL);
}

static double now_seconds(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* ------------------------------------------------------------------------------ */
/* canonical pair arithmetic                                                       */
/* ------------------------------------------------------------------------------ */
static inline float pair_d2(float dx, float dy, float eps2) { return fmaf(dx, dx, fmaf(dy, dy, eps2)); }
static inline float pair_scale(float m, float d2) {
    float r = 1.0f / sqrtf(d2);
    return ((m * r) * r) * r;
}

/* Quadrupole-corrected acceleration from a node with mass m, centre of mass at offset
 * (dx, dy) from the particle and second central moments S = {sxx, sxy, syy}:
 *   a = d (m r^3 + 7.5 u r^7 - 1.5 T r^5) - 3 r^5 S d,   u = d^T S d,  T = sxx + syy,
 * with r = 1 / sqrt(|d|^2 + eps^2) (Plummer-softened expansion of sum m_k / |x_k - p|). */
/* Node terms of the quadrupole formula, once per node: S'' = 7.5 S, mt = -1.5 tr S. */
typedef struct { float qxx, qxy, qyy, mt; } quad_terms;
static inline quad_terms quad_node(float sxx, float sxy, float syy) {
    quad_terms q = {7.5f * sxx, 7.5f * sxy, 7.5f * syy, -1.5f * (sxx + syy)};
    return q;
}

/* Monopole + quadrupole term of the softened potential, r = 1/sqrt(d2):
 *   a = d (m r^3 - 1.5 tr(S) r^5 + 7.5 (d.S.d) r^7) - 3 r^5 S d
 * evaluated as r^3 (d (m + r^2 (mt + r^2 u'')) - 0.4 r^2 S'' d), u'' = d.S''.d. */
static inline void quad_accumulate(float dx, float dy, float d2, float m, quad_terms q, float* ax, float* ay) {
    float r = 1.0f / sqrtf(d2);
    float r2 = r * r;
    float r3 = r2 * r;
    float srx = fmaf(q.qxx, dx, q.qxy * dy);
    float sry = fmaf(q.qxy, dx, q.qyy * dy);
    float u = fmaf(dx, srx, dy * sry);
    float t = fmaf(fmaf(u, r2, q.mt), r2, m);
    float k = -0.4f * r2;
    float ix = fmaf(srx, k, dx * t);
    float iy = fmaf(sry, k, dy * t);
    *ax = fmaf(r3, ix, *ax);
    *ay = fmaf(r3, iy, *ay);
}

/* ------------------------------------------------------------------------------ */
/* direct sum -- SimShader.comp:37-74                                              */
/* ------------------------------------------------------------------------------ */
typedef struct {
    uint32_t n;
    const float *pos, *vel, *mass;
    float *pos_out, *vel_out, *acc;
    float dt, G, eps2;
} direct_ctx;

static void direct_accel_one(const direct_ctx* c, uint32_t i, float* axo, float* ayo) {
    const float px = c->pos[2 * i], py = c->pos[2 * i + 1];
    float ax = 0.0f, ay = 0.0f;
    for (uint32_t j = 0; j < c->n; ++j) { /* SimShader.comp:43-65: j ascending */
        float dx = c->pos[2 * j] - px;
        float dy = c->pos[2 * j + 1] - py;
        float s = pair_scale(c->mass[j], pair_d2(dx, dy, c->eps2));
        ax = fmaf(dx, s, ax);
        ay = fmaf(dy, s, ay);
    }
    *axo = ax;
    *ayo = ay;
}

static void direct_step_item(void* p, uint64_t i, int w) {
    (void)w;
    const direct_ctx* c = (const direct_ctx*)p;
    float ax, ay;
    direct_accel_one(c, (uint32_t)i, &ax, &ay);
    /* SimShader.comp:68-73 */
    const float k = c->dt * c->G;
    const float hdt = 0.5f * c->dt;
    float vx = c->vel[2 * i], vy = c->vel[2 * i + 1];
    float nvx = fmaf(ax, k, vx), nvy = fmaf(ay, k, vy);
    c->pos_out[2 * i] = fmaf(vx + nvx, hdt, c->pos[2 * i]);
    c->pos_out[2 * i + 1] = fmaf(vy + nvy, hdt, c->pos[2 * i + 1]);
    c->vel_out[2 * i] = nvx;
    c->vel_out[2 * i + 1] = nvy;
}

void orc_direct_step(uint32_t n, const float* pos_in, const float* vel_in, const float* mass_in,
                     float* pos_out, float* vel_out, float dt, float G, float eps2, int nthreads) {
    direct_ctx c = {n, pos_in, vel_in, mass_in, pos_out, vel_out, NULL, dt, G, eps2};
    parallel_for(nthreads, n, 16, direct_step_item, &c);
}

static void direct_accel_item(void* p, uint64_t i, int w) {
    (void)w;
    const direct_ctx* c = (const direct_ctx*)p;
    direct_accel_one(c, (uint32_t)i, &c->acc[2 * i], &c->acc[2 * i + 1]);
}

void orc_direct_accel(uint32_t n, const float* pos, const float* mass, float eps2, float* acc,
                      int nthreads) {
    direct_ctx c = {n, pos, NULL, mass, NULL, NULL, acc, 0, 0, eps2};
    parallel_for(nthreads, n, 16, direct_accel_item, &c);
}

typedef struct {
    uint32_t n;
    const float *pos, *mass;
    double eps2;
    const uint32_t* targets;
    double* acc;
} f64_ctx;

static void f64_item(void* p, uint64_t t, int w) {
    (void)w;
    const f64_ctx* c = (const f64_ctx*)p;
    uint32_t i = c->targets ? c->targets[t] : (uint32_t)t;
    double px = c->pos[2 * i], py = c->pos[2 * i + 1];
    double ax = 0.0, ay = 0.0;
    for (uint32_t j = 0; j < c->n; ++j) {
        double dx = (double)c->pos[2 * j] - px, dy = (double)c->pos[2 * j + 1] - py;
        double d2 = dx * dx + dy * dy + c->eps2;
        double s = (double)c->mass[j] / (d2 * sqrt(d2));
        ax += dx * s;
        ay += dy * s;
    }
    c->acc[2 * t] = ax;
    c->acc[2 * t + 1] = ay;
}

void orc_direct_accel_f64(uint32_t n, const float* pos, const float* mass, double eps2,
                          uint32_t n_targets, const uint32_t* targets, double* acc, int nthreads) {
    f64_ctx c = {n, pos, mass, eps2, targets, acc};
    parallel_for(nthreads, n_targets, 4, f64_item, &c);
}

typedef struct {
    uint32_t n;
    const float *pos, *mass;
    double eps2;
    double* partial; /* per i */
} energy_ctx;

static void energy_item(void* p, uint64_t i, int w) {
    (void)w;
    const energy_ctx* c = (const energy_ctx*)p;
    double px = c->pos[2 * i], py = c->pos[2 * i + 1], mi = c->mass[i], e = 0.0;
    for (uint32_t j = (uint32_t)i + 1; j < c->n; ++j) {
        double dx = (double)c->pos[2 * j] - px, dy = (double)c->pos[2 * j + 1] - py;
        e -= mi * (double)c->mass[j] / sqrt(dx * dx + dy * dy + c->eps2);
    }
    c->partial[i] = e;
}

/* src/Graphics/Shaders/VertShader.vert:13-18 (screenPos = (pos - cameraPos) / cameraSize,
 * y negated, point size 1), FragShader.frag:5-7 (white), the viewport transform of
 * GraphicsPipeline.cpp:349-358 written as (ndc + 1) * size / 2, over a black clear
 * (GraphicsPipeline.cpp:327). */
void orc_render_points(uint32_t n, const float* pos, const float* camera, uint32_t width, uint32_t height,
                       uint8_t* image) {
    memset(image, 0, (size_t)width * height);
    const float hw = 0.5f * (float)width, hh = 0.5f * (float)height;
    for (uint32_t i = 0; i < n; ++i) {
        const float sx = (pos[2 * i] - camera[0]) / camera[2];
        const float sy = -((pos[2 * i + 1] - camera[1]) / camera[3]);
        const float fx = (sx + 1.0f) * hw, fy = (sy + 1.0f) * hh;
        if (!(fx >= 0.0f && fx < (float)width && fy >= 0.0f && fy < (float)height)) continue;
        const uint32_t x = (uint32_t)fx, y = (uint32_t)fy;
        if (x < width && y < height) image[(size_t)y * width + x] = 255;
    }
}

double orc_energy_f64(uint32_t n, const float* pos, const float* vel, const float* mass,
                      double G, double eps2) {
    double* part = (double*)calloc(n ? n : 1, sizeof(double));
    energy_ctx c = {n, pos, mass, eps2, part};
    parallel_for(8, n, 64, energy_item, &c);
    double pot = 0.0, kin = 0.0;
    for (uint32_t i = 0; i < n; ++i) {
        pot += part[i];
        double vx = vel[2 * i], vy = vel[2 * i + 1];
        kin += 0.5 * (double)mass[i] * (vx * vx + vy * vy);
    }
    free(part);
    return kin + G * pot;
}

/* ------------------------------------------------------------------------------ */
/* cell keys                                                                       */
/* ------------------------------------------------------------------------------ */
static inline uint32_t spread_bits(uint32_t v) { /* InitShader.comp:88-96 (and 15-bit use) */
    v = (v | (v << 8)) & 0x00ff00ffu;
    v = (v | (v << 4)) & 0x0f0f0f0fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

/* InitShader.comp:80-98: returns 1 and the 20-bit key when the particle is inside. */
static inline int fixed_box_key(float px, float py, uint32_t* key) {
    float rx = ((px / SIM_SIZE) + 1.0f) * 0.5f;
    float ry = ((py / SIM_SIZE) + 1.0f) * 0.5f;
    rx = rx * (float)GRID;
    ry = ry * (float)GRID;
    if (rx >= 0.0f && rx < (float)GRID && ry >= 0.0f && ry < (float)GRID) {
        *key = spread_bits((uint32_t)rx) | (spread_bits((uint32_t)ry) << 1);
        return 1;
    }
    return 0;
}

typedef struct {
    float cx, cy, scale, radius0, inv_scale;
    int bits; /* cells per axis: 2^bits */
} bbox_params;

/* Bounding-box mode: square box around min/max of all positions (1/1024 margin),
 * 2^bits cells per axis (bits 12: 24-bit keys, 15: 30-bit keys). */
static bbox_params bbox_from_minmax(double minx, double maxx, double miny, double maxy, int bits) {
    bbox_params b;
    b.bits = bits;
    double cx = 0.5 * (minx + maxx), cy = 0.5 * (miny + maxy);
    double ext = maxx - minx > maxy - miny ? maxx - minx : maxy - miny;
    if (!(ext > 0.0) || !isfinite(ext)) ext = 1.0;
    if (!isfinite(cx)) cx = 0.0;
    if (!isfinite(cy)) cy = 0.0;
    double half = ext * 0.5 * (1.0 + 1.0 / 1024.0);
    double scale = (double)(1u << (bits - 1)) / half;
    b.cx = (float)cx;
    b.cy = (float)cy;
    b.scale = (float)scale;
    double side0 = (double)(1u << bits) / (double)b.scale;
    b.radius0 = (float)(side0 * side0 * 0.5);
    b.inv_scale = (float)(1.0 / (double)b.scale);
    return b;
}

static inline uint32_t bbox_cell(float p, float c, float scale, int bits) {
    float t = (p - c) * scale + (float)(1u << (bits - 1));
    if (!(t >= 0.0f)) return 0;
    if (t >= (float)((1u << bits) - 1)) return (1u << bits) - 1;
    return (uint32_t)t;
}

static inline uint32_t bbox_key(float px, float py, const bbox_params* b) {
    return spread_bits(bbox_cell(px, b->cx, b->scale, b->bits)) |
           (spread_bits(bbox_cell(py, b->cy, b->scale, b->bits)) << 1);
}

uint64_t orc_bh_node_capacity(int box_mode, uint32_t n_al) {
    uint64_t levels = box_mode == ORC_BOX_BOUNDING ? BBOX_MAX_BITS + 1 : GRID_LEVELS;
    return (uint64_t)n_al + levels * (uint64_t)(n_al / 2) + 64;
}

/* ------------------------------------------------------------------------------ */
/* force walk -- ForceShader.comp:78-152                                           */
/* ------------------------------------------------------------------------------ */
typedef struct {
    const uint32_t* skip;
    const float *radius, *npos, *nmass;
    const float* quad; /* second central moments {sxx, sxy, syy} per record, NULL: monopoles */
    uint64_t tree_size;
    const uint32_t* src; /* original index per sorted slot, n_al for empty slots */
    const uint32_t* skey; /* cell key per sorted slot (group walk) */
    uint32_t n_al;
    const float *pos_in, *vel_in, *mass_in;
    float *pos_out, *vel_out;
    float eps2, theta2, k, hdt;
    uint64_t* interactions; /* per worker */
    uint64_t* visits;       /* per worker */
    uint32_t stride;        /* walk warps stride*item */
    int group_walk;         /* ORC_BH_GROUP_WALK semantics */
    uint32_t* max_stack;    /* per worker */
    uint32_t* group_visits; /* optional per-group outputs (orc_bh_out) */
    uint64_t* group_inter;
    uint64_t* max_inter;    /* per worker: largest per-warp interaction count */
    uint32_t group_size;    /* particles per group walk (64) */
    float rel_alpha, rel_floor2; /* ORC_BH_RELATIVE_MAC: alpha, floor^2, previous and new |a| */
    const float* amag_in;
    float* amag_out;
} walk_ctx;

static void walk_warp(void* p, uint64_t item, int worker) {
    const walk_ctx* c = (const walk_ctx*)p;
    const uint64_t w = item * c->stride;
    float px[WARP], py[WARP], ax[WARP], ay[WARP], dx[WARP], dy[WARP], d2[WARP];
    int valid[WARP];
    int nvalid = 0;
    for (int l = 0; l < WARP; ++l) {
        uint32_t s = (uint32_t)w * WARP + (uint32_t)l;
        uint32_t i = c->src[s];
        valid[l] = i != c->n_al; /* ForceShader.comp:84-92 */
        px[l] = valid[l] ? c->pos_in[2 * i] : 0.0f;
        py[l] = valid[l] ? c->pos_in[2 * i + 1] : 0.0f;
        ax[l] = ay[l] = 0.0f;
        nvalid += valid[l];
    }
    if (!nvalid) return;
    uint64_t ind = 0, inter = 0, visits = 0;
    while (ind < c->tree_size) { /* ForceShader.comp:111 */
        const float nx = c->npos[2 * ind], ny = c->npos[2 * ind + 1];
        const float nr = c->radius[ind], nm = c->nmass[ind];
        int all = 1;
        for (int l = 0; l < WARP; ++l) {
            if (!valid[l]) continue; /* empty lanes vote yes */
            dx[l] = nx - px[l];
            dy[l] = ny - py[l];
            d2[l] = pair_d2(dx[l], dy[l], c->eps2);
            if (!(nr <= d2[l] * c->theta2)) all = 0; /* ForceShader.comp:131 */
        }
        ++visits;
        if (all) {
            if (c->quad && c->skip[ind] > 1) { /* internal node: quadrupole term */
                const quad_terms qt = quad_node(c->quad[3 * ind], c->quad[3 * ind + 1], c->quad[3 * ind + 2]);
                for (int l = 0; l < WARP; ++l) {
                    if (!valid[l]) continue;
                    quad_accumulate(dx[l], dy[l], d2[l], nm, qt, &ax[l], &ay[l]);
                }
            } else {
                for (int l = 0; l < WARP; ++l) {
                    if (!valid[l]) continue;
                    float s = pair_scale(nm, d2[l]);
                    ax[l] = fmaf(dx[l], s, ax[l]);
                    ay[l] = fmaf(dy[l], s, ay[l]);
                }
            }
            inter += (uint64_t)nvalid;
            ind += c->skip[ind];
        } else {
            ++ind;
        }
    }
    for (int l = 0; l < WARP; ++l) { /* ForceShader.comp:143-151 */
        if (!valid[l]) continue;
        uint32_t i = c->src[(uint32_t)w * WARP + (uint32_t)l];
        float vx = c->vel_in[2 * i], vy = c->vel_in[2 * i + 1];
        float nvx = fmaf(ax[l], c->k, vx), nvy = fmaf(ay[l], c->k, vy);
        c->pos_out[2 * i] = fmaf(vx + nvx, c->hdt, px[l]);
        c->pos_out[2 * i + 1] = fmaf(vy + nvy, c->hdt, py[l]);
        c->vel_out[2 * i] = nvx;
        c->vel_out[2 * i + 1] = nvy;
    }
    c->interactions[worker] += inter;
    c->visits[worker] += visits;
}

/* Accurate-mode walk (ORC_BH_GROUP_WALK), for the 64 consecutive sorted slots of one group:
 *   - the group is cut into at most four sub-boxes: the particles are split by their
 *     cell at the coarsest level where the first and last cell keys of the group differ
 *     (so a group that crosses a coarse Morton boundary does not get one box spanning
 *     the empty space between its two ends); each sub-box is the bounding box of its
 *     particles;
 *   - a LIFO stack starts with the root; each step pops the top min(32, size) records
 *     (lane j gets stack[size - k + j]) and tests each against the box:
 *       d2 = ex^2 + ey^2 + eps^2 with (ex, ey) the distance from the box to the centre of
 *       mass, accepted iff radius <= d2 * theta^2;
 *   - an accepted record becomes one interaction item; an opened record pushes its
 *     internal children (in preorder) and turns each run of consecutive particle-leaf
 *     children into one range item;
 *   - lanes are handled in order, so items and pushes are in lane order;
 *   - every particle of the group sums the accepted nodes (quadrupole term) and the
 *     particle leaves (monopoles) separately, each in walk order, into a node and a leaf
 *     accumulator; its acceleration is node + leaf; then it is integrated.
 *   - a costly group (relative criterion, a system of at least HEAVY_MIN_PARTICLES
 *     padded particles, every previous |a| of the group known, the smallest below
 *     HEAVY_RATIO times the largest) is walked by two warps at once: pops take the top
 *     min(64, size) records, and item i of the node list (record i of the leaf runs) goes
 *     to part (i / 32) mod 2; each part sums its items in walk order from zero, and the
 *     node (leaf) accumulator is part 0 + part 1.  The set of tested and accepted records
 *     is the same as with 32-record pops; only the order of the sums differs.
 * The CUDA kernel (force_kernels.cuh, force_group_body / force_pair_body) batches its
 * evaluations differently; with this accumulation rule the batching changes no bit. */
#define HEAVY_RATIO 0.1f
#define HEAVY_MIN_PARTICLES (1u << 18) /* systems with fewer (padded) particles walk every group alone */
/* 0: every group walks alone whatever its size (a check that pairing changes only the
 * order of the sums; not a mode of the library) */
static int g_heavy_pairs = 1;
void orc_set_heavy_pairs(int on) { g_heavy_pairs = on; }
#define GROUP_SIZE 64
#define GROUP_STACK_CAP 4096
#define GMAX 64
/* One walk of a group: every valid lane's node and leaf accelerations (ax/ay[l][0] node,
 * [1] leaf) for the opening test `relative` (tol2 = (alpha a_min)^2, with the floor) or
 * theta (theta2).  Adds the interactions and visits, and raises *max_size. */
static void group_walk_once(const walk_ctx* c, uint64_t w, uint32_t G, int nvalid, const int* valid,
                            const float* px, const float* py, const float* gx0, const float* gx1,
                            const float* gy0, const float* gy1, int relative, float tol2, float theta2,
                            int pair, float (*ax)[2], float (*ay)[2], uint64_t* inter_out, uint64_t* visits_out,
                            uint32_t* max_size_out) {
    (void)w;
    /* accumulators per particle, part and kind (node 0, leaf 1) */
    static _Thread_local float acx[GMAX][2][2], acy[GMAX][2][2];
    for (uint32_t l = 0; l < G; ++l)
        for (int q = 0; q < 2; ++q) acx[l][q][0] = acy[l][q][0] = acx[l][q][1] = acy[l][q][1] = 0.0f;
    const uint32_t width = pair ? 2 * WARP : WARP;
    uint64_t n_node_items = 0, n_leaf_items = 0; /* item indices in walk order */
    static _Thread_local uint32_t stack[GROUP_STACK_CAP + 4 * 2 * WARP];
    uint32_t size = 1, max_size = *max_size_out;
    stack[0] = 0;
    uint64_t inter = 0, visits = 0;
    while (size) {
        uint32_t np = size < width ? size : width;
        uint32_t base = size - np;
        uint32_t popped[2 * WARP];
        for (uint32_t j = 0; j < np; ++j) popped[j] = stack[base + j];
        size = base;
        for (uint32_t j = 0; j < np; ++j) {
            const uint32_t n = popped[j];
            ++visits;
            const uint32_t sk = c->skip[n];
            int accept = 1;
            if (sk > 1) {
                const float cx = c->npos[2 * n], cy = c->npos[2 * n + 1];
                float d2 = INFINITY; /* nearest sub-box (empty sub-boxes give +inf) */
                for (int b = 0; b < 4; ++b) {
                    float ex = fmaxf(fmaxf(gx0[b] - cx, cx - gx1[b]), 0.0f);
                    float ey = fmaxf(fmaxf(gy0[b] - cy, cy - gy1[b]), 0.0f);
                    d2 = fminf(d2, pair_d2(ex, ey, c->eps2));
                }
                if (relative) {
                    const float r = c->radius[n], m = c->nmass[n];
                    const float lhs = (m * m) * ((r * r) * r);
                    const float d4 = d2 * d2;
                    const float rhs = tol2 * ((d4 * d4) * d2);
                    accept = (r <= d2 && lhs <= rhs) || r <= d2 * c->rel_floor2;
                } else {
                    accept = c->radius[n] <= d2 * theta2;
                }
            }
            if (accept) { /* one item: the record itself (a leaf only when the root is one) */
                const float nx = c->npos[2 * n], ny = c->npos[2 * n + 1], nm = c->nmass[n];
                const int a = sk > 1 ? 0 : 1;
                const int q = pair ? (int)((n_node_items++ >> 5) & 1u) : 0;
                const quad_terms qt = c->quad ? quad_node(c->quad[3 * n], c->quad[3 * n + 1], c->quad[3 * n + 2])
                                              : quad_node(0.0f, 0.0f, 0.0f);
                for (uint32_t l = 0; l < G; ++l) {
                    if (!valid[l]) continue;
                    float dx = nx - px[l], dy = ny - py[l];
                    float d2 = pair_d2(dx, dy, c->eps2);
                    if (c->quad && sk > 1) {
                        quad_accumulate(dx, dy, d2, nm, qt, &acx[l][q][a], &acy[l][q][a]);
                    } else {
                        float sc = pair_scale(nm, d2);
                        acx[l][q][a] = fmaf(dx, sc, acx[l][q][a]);
                        acy[l][q][a] = fmaf(dy, sc, acy[l][q][a]);
                    }
                }
                inter += (uint64_t)nvalid;
                continue;
            }
            const uint32_t end = n + sk;
            uint32_t ch = n + 1;
            while (ch < end) {
                if (c->skip[ch] == 1) { /* a run of particle leaves: one range item */
                    uint32_t r = ch;
                    while (r < end && c->skip[r] == 1) ++r;
                    for (uint32_t q = ch; q < r; ++q) {
                        const float nx = c->npos[2 * q], ny = c->npos[2 * q + 1], nm = c->nmass[q];
                        const int a = 1;
                        const int pq = pair ? (int)((n_leaf_items++ >> 5) & 1u) : 0;
                        for (uint32_t l = 0; l < G; ++l) {
                            if (!valid[l]) continue;
                            float dx = nx - px[l], dy = ny - py[l];
                            float sc = pair_scale(nm, pair_d2(dx, dy, c->eps2));
                            acx[l][pq][a] = fmaf(dx, sc, acx[l][pq][a]);
                            acy[l][pq][a] = fmaf(dy, sc, acy[l][pq][a]);
                        }
                    }
                    inter += (uint64_t)nvalid * (r - ch);
                    ch = r;
                } else {
                    if (size < GROUP_STACK_CAP + 4 * 2 * WARP) stack[size] = ch;
                    ++size;
                    ch += c->skip[ch];
                }
            }
        }
        if (size > max_size) max_size = size;
        if (size > GROUP_STACK_CAP) size = GROUP_STACK_CAP; /* reported through max_stack */
    }
    for (uint32_t l = 0; l < G; ++l)
        for (int a = 0; a < 2; ++a) {
            ax[l][a] = pair ? acx[l][0][a] + acx[l][1][a] : acx[l][0][a];
            ay[l][a] = pair ? acy[l][0][a] + acy[l][1][a] : acy[l][0][a];
        }
    *inter_out += inter;
    *visits_out += visits;
    *max_size_out = max_size;
}

/* |a| of an acceleration, the value the relative criterion compares against */
static inline float accel_magnitude(float ax, float ay) { return sqrtf(fmaf(ax, ax, ay * ay)); }

static void group_walk_warp(void* p, uint64_t item, int worker) {
    const walk_ctx* c = (const walk_ctx*)p;
    const uint64_t w = item * c->stride;
    float px[GMAX], py[GMAX], ax[GMAX][2], ay[GMAX][2]; /* node, leaf */
    int valid[GMAX];
    const uint32_t G = c->group_size;
    int nvalid = 0;
    float gx0[4], gx1[4], gy0[4], gy1[4];
    for (int b = 0; b < 4; ++b) {
        gx0[b] = gy0[b] = INFINITY;
        gx1[b] = gy1[b] = -INFINITY;
    }
    for (uint32_t l = 0; l < G; ++l) {
        uint32_t s = (uint32_t)w * G + l;
        uint32_t i = c->src[s];
        valid[l] = i != c->n_al;
        px[l] = valid[l] ? c->pos_in[2 * i] : 0.0f;
        py[l] = valid[l] ? c->pos_in[2 * i + 1] : 0.0f;
        nvalid += valid[l];
    }
    if (!nvalid || !c->tree_size) return;
    {
        const uint32_t kf = c->skey[(uint32_t)w * G], kl = c->skey[(uint32_t)w * G + (uint32_t)nvalid - 1];
        const int shift = kf == kl ? -1 : ((31 - __builtin_clz(kf ^ kl)) & ~1);
        for (int l = 0; l < nvalid; ++l) { /* valid lanes are a prefix of the warp */
            const int b = shift < 0 ? 0 : (int)((c->skey[(uint32_t)w * G + (uint32_t)l] >> shift) & 3u);
            gx0[b] = fminf(gx0[b], px[l]);
            gx1[b] = fmaxf(gx1[b], px[l]);
            gy0[b] = fminf(gy0[b], py[l]);
            gy1[b] = fmaxf(gy1[b], py[l]);
        }
    }
    uint64_t inter = 0, visits = 0;
    uint32_t max_size = 1;
    /* relative criterion: the group's smallest previous |a|; NaN if any is unknown */
    float amin = INFINITY;
    if (c->amag_in)
        for (uint32_t l = 0; l < G; ++l) {
            if (!valid[l]) continue;
            const float a = c->amag_in[c->src[(uint32_t)w * G + l]];
            if (isnan(a) || isnan(amin)) amin = NAN;
            else if (a < amin) amin = a;
        }
    const int amag_known = c->amag_in && !isnan(amin);
    if (c->amag_in && isnan(amin)) {
        /* no previous |a| for some particle (first step after a reset): estimate every
         * particle's |a| of the group by a walk with the theta test, then open nodes by the
         * relative criterion with those estimates */
        group_walk_once(c, w, G, nvalid, valid, px, py, gx0, gx1, gy0, gy1, 0, 0.0f, c->theta2, 0, ax, ay, &inter,
                        &visits, &max_size);
        amin = INFINITY;
        for (uint32_t l = 0; l < G; ++l) {
            if (!valid[l]) continue;
            const float a = accel_magnitude(ax[l][0] + ax[l][1], ay[l][0] + ay[l][1]);
            if (isnan(a) || isnan(amin)) amin = NAN;
            else if (a < amin) amin = a;
        }
    }
    const int relative = c->amag_in && amin >= 0.0f;
    const float tol = c->rel_alpha * amin, tol2 = tol * tol;
    /* a costly group: every previous |a| known and the smallest below HEAVY_RATIO times
     * the largest; walked by a warp pair (64-record pops, two-part sums) */
    int pair = 0;
    if (g_heavy_pairs && relative && amag_known && c->n_al >= HEAVY_MIN_PARTICLES) {
        float amax = 0.0f;
        for (uint32_t l = 0; l < G; ++l)
            if (valid[l]) amax = fmaxf(amax, c->amag_in[c->src[(uint32_t)w * G + l]]);
        pair = amin < HEAVY_RATIO * amax;
    }
    group_walk_once(c, w, G, nvalid, valid, px, py, gx0, gx1, gy0, gy1, relative, tol2, c->theta2, pair, ax, ay,
                    &inter, &visits, &max_size);
    for (uint32_t l = 0; l < G; ++l) {
        if (!valid[l]) continue;
        uint32_t i = c->src[(uint32_t)w * G + l];
        float vx = c->vel_in[2 * i], vy = c->vel_in[2 * i + 1];
        const float axl = ax[l][0] + ax[l][1], ayl = ay[l][0] + ay[l][1];
        if (c->amag_out) c->amag_out[i] = accel_magnitude(axl, ayl);
        float nvx = fmaf(axl, c->k, vx), nvy = fmaf(ayl, c->k, vy);
        c->pos_out[2 * i] = fmaf(vx + nvx, c->hdt, px[l]);
        c->pos_out[2 * i + 1] = fmaf(vy + nvy, c->hdt, py[l]);
        c->vel_out[2 * i] = nvx;
        c->vel_out[2 * i + 1] = nvy;
    }
    c->interactions[worker] += inter;
    c->visits[worker] += visits;
    if (c->group_visits) c->group_visits[w] = (uint32_t)visits;
    if (c->group_inter) c->group_inter[w] = inter;
    if (max_size > c->max_stack[worker]) c->max_stack[worker] = max_size;
    if (inter > c->max_inter[worker]) c->max_inter[worker] = inter;
}

static void run_walk(walk_ctx* c, int nthreads, orc_bh_out* out) {
    uint64_t inter[256] = {0}, vis[256] = {0};
    uint32_t mstack[256] = {0};
    uint64_t minter[256] = {0};
    c->interactions = inter;
    c->visits = vis;
    c->max_stack = mstack;
    c->max_inter = minter;
    c->stride = out && out->walk_stride > 1 ? out->walk_stride : 1;
    uint64_t warps = c->n_al / (c->group_walk ? c->group_size : WARP);
    double t0 = now_seconds();
    parallel_for(nthreads, (warps + c->stride - 1) / c->stride, 4, c->group_walk ? group_walk_warp : walk_warp, c);
    if (out) {
        out->max_stack = 0;
        out->max_warp_interactions = 0;
        for (int t = 0; t < 256; ++t) {
            if (mstack[t] > out->max_stack) out->max_stack = mstack[t];
            if (minter[t] > out->max_warp_interactions) out->max_warp_interactions = minter[t];
        }
    }
    if (out) out->walk_seconds = now_seconds() - t0;
    if (out) {
        out->interactions = 0;
        out->warp_visits = 0;
        for (int t = 0; t < 256; ++t) {
            out->interactions += inter[t];
            out->warp_visits += vis[t];
        }
    }
}

static void copy_tree_out(orc_bh_out* out, const uint32_t* skip, const float* radius,
                          const float* npos, const float* nmass, uint64_t tree_size) {
    if (!out) return;
    uint64_t n = tree_size < out->node_capacity ? tree_size : out->node_capacity;
    if (out->node_skip) memcpy(out->node_skip, skip, n * sizeof(uint32_t));
    if (out->node_radius) memcpy(out->node_radius, radius, n * sizeof(float));
    if (out->node_pos) memcpy(out->node_pos, npos, 2 * n * sizeof(float));
    if (out->node_mass) memcpy(out->node_mass, nmass, n * sizeof(float));
}

/* ------------------------------------------------------------------------------ */
/* literal grid restatement (fixed box)                                            */
/* ------------------------------------------------------------------------------ */
int orc_bh_grid_step(uint32_t n_al, float* pos_in, float* vel_in, float* mass_in,
                     float* pos_out, float* vel_out, float* mass_out, float dt, float G,
                     float eps2, float theta2, orc_bh_out* out, int nthreads) {
    uint32_t* cnt[GRID_LEVELS][2];
    uint32_t* st[GRID_LEVELS][2];
    float* lp[GRID_LEVELS][2];
    float* lm[GRID_LEVELS];
    for (int d = 0; d < GRID_LEVELS; ++d) {
        size_t nc = (size_t)1 << (2 * d);
        for (int k = 0; k < 2; ++k) {
            cnt[d][k] = (uint32_t*)calloc(nc, sizeof(uint32_t));
            st[d][k] = (uint32_t*)calloc(nc, sizeof(uint32_t));
            lp[d][k] = (float*)calloc(nc, sizeof(float));
        }
        lm[d] = (float*)calloc(nc, sizeof(float));
    }
    uint64_t cap = orc_bh_node_capacity(ORC_BOX_FIXED_500, n_al);
    uint32_t* skip = (uint32_t*)calloc(cap, sizeof(uint32_t));
    float* radius = (float*)calloc(cap, sizeof(float));
    float* npos = (float*)calloc(2 * cap, sizeof(float));
    float* nmass = (float*)calloc(cap, sizeof(float));
    uint32_t* src = (uint32_t*)malloc((size_t)n_al * sizeof(uint32_t));
    const double t_build = now_seconds();

    /* ClearShader.comp:71-83 (level 10 arrays are calloc'ed above) */
    for (uint32_t i = 0; i < n_al; ++i) src[i] = n_al;

    /* InitShader.comp:73-119, particles in ascending index order */
    const int L = GRID_LEVELS - 1;
    uint64_t valid = 0;
    for (uint32_t i = 0; i < n_al; ++i) {
        float px = pos_in[2 * i], py = pos_in[2 * i + 1], m = mass_in[i];
        uint32_t key;
        if (fixed_box_key(px, py, &key)) {
            if (out && out->keys) out->keys[i] = key;
            cnt[L][0][key] += 1;
            if (cnt[L][1][key] == 1) cnt[L][1][key] = 2; /* :105 */
            cnt[L][1][key] += 1;
            lp[L][0][key] = lp[L][0][key] + px * m;
            lp[L][1][key] = lp[L][1][key] + py * m;
            lm[L][key] = lm[L][key] + m;
            ++valid;
        } else { /* :110-117 removal */
            if (out && out->keys) out->keys[i] = ORC_KEY_REMOVED;
            pos_in[2 * i] = pos_in[2 * i + 1] = -SIM_SIZE * 2.0f;
            pos_out[2 * i] = pos_out[2 * i + 1] = -SIM_SIZE * 2.0f;
            mass_in[i] = 0.0f;
            mass_out[i] = 0.0f;
        }
    }

    /* TreeInitShader.comp:58-90, depths 9 .. 0 */
    for (int d = L - 1; d >= 0; --d) {
        size_t nc = (size_t)1 << (2 * d);
        for (size_t c = 0; c < nc; ++c) {
            uint32_t cx = 0, cy = 0;
            float sx = 0.0f, sy = 0.0f, sm = 0.0f;
            for (int q = 0; q < 4; ++q) {
                size_t ch = 4 * c + (size_t)q;
                cx += cnt[d + 1][0][ch];
                cy += cnt[d + 1][1][ch];
                if (q == 0) {
                    sx = lp[d + 1][0][ch];
                    sy = lp[d + 1][1][ch];
                    sm = lm[d + 1][ch];
                } else {
                    sx = sx + lp[d + 1][0][ch];
                    sy = sy + lp[d + 1][1][ch];
                    sm = sm + lm[d + 1][ch];
                }
            }
            cy += (uint32_t)(cy > 1); /* :83 */
            cnt[d][0][c] = cx;
            cnt[d][1][c] = cy;
            lp[d][0][c] = sx;
            lp[d][1][c] = sy;
            lm[d][c] = sm;
        }
    }

    /* TreeSortShader.comp:57-94, depths 0 .. 9; root start is 0 */
    for (int d = 0; d < L; ++d) {
        size_t nc = (size_t)1 << (2 * d);
        for (size_t c = 0; c < nc; ++c) {
            uint32_t ox = st[d][0][c], oy = st[d][1][c];
            if (cnt[d][1][c] > 1) oy += 1;
            for (int q = 0; q < 4; ++q) {
                size_t ch = 4 * c + (size_t)q;
                st[d + 1][0][ch] = ox;
                st[d + 1][1][ch] = oy;
                ox += cnt[d + 1][0][ch];
                oy += cnt[d + 1][1][ch];
            }
        }
    }

    /* TreeMoveShader.comp:53-84, depths 0 .. 10 */
    for (int d = 0; d <= L; ++d) {
        size_t nc = (size_t)1 << (2 * d);
        for (size_t c = 0; c < nc; ++c) {
            if (cnt[d][1][c] > 1) {
                float px = lp[d][0][c], py = lp[d][1][c], m = lm[d][c];
                if (m != 0.0f) {
                    px = px / m;
                    py = py / m;
                }
                float r = SIM_SIZE * SIM_SIZE * 2.0f;
                r = r / (float)(1u << (2 * d));
                uint32_t at = st[d][1][c];
                skip[at] = cnt[d][1][c];
                radius[at] = r;
                npos[2 * at] = px;
                npos[2 * at + 1] = py;
                nmass[at] = m;
                if (d == L) st[d][1][c] += 1;
            }
        }
    }

    /* ParticleSortShader.comp:71-110, ascending index order */
    for (uint32_t i = 0; i < n_al; ++i) {
        float px = pos_in[2 * i], py = pos_in[2 * i + 1];
        uint32_t key;
        if (!fixed_box_key(px, py, &key)) continue;
        uint32_t a = st[L][0][key]++;
        src[a] = i;
        uint32_t b = st[L][1][key]++;
        skip[b] = 1;
        radius[b] = 0.0f;
        npos[2 * b] = px;
        npos[2 * b + 1] = py;
        nmass[b] = mass_in[i];
    }

    uint64_t tree_size = valid ? skip[0] : 0;
    if (out) out->build_seconds = now_seconds() - t_build;
    walk_ctx wc;
    memset(&wc, 0, sizeof wc);
    wc.skip = skip;
    wc.radius = radius;
    wc.npos = npos;
    wc.nmass = nmass;
    wc.tree_size = tree_size;
    wc.src = src;
    wc.n_al = n_al;
    wc.pos_in = pos_in;
    wc.vel_in = vel_in;
    wc.mass_in = mass_in;
    wc.pos_out = pos_out;
    wc.vel_out = vel_out;
    wc.eps2 = eps2;
    wc.theta2 = theta2;
    wc.k = G * dt;
    wc.hdt = 0.5f * dt;
    run_walk(&wc, nthreads, out);

    if (out) {
        out->tree_size = tree_size;
        out->valid_count = valid;
        out->internal_count = tree_size >= valid ? tree_size - valid : 0;
        if (out->sorted_src) memcpy(out->sorted_src, src, (size_t)n_al * sizeof(uint32_t));
        copy_tree_out(out, skip, radius, npos, nmass, tree_size);
        out->box_center_x = out->box_center_y = 0.0f;
        out->box_scale = (float)GRID / (2.0f * SIM_SIZE);
        out->box_radius0 = SIM_SIZE * SIM_SIZE * 2.0f;
    }

    for (int d = 0; d < GRID_LEVELS; ++d) {
        for (int k = 0; k < 2; ++k) {
            free(cnt[d][k]);
            free(st[d][k]);
            free(lp[d][k]);
        }
        free(lm[d]);
    }
    free(skip);
    free(radius);
    free(npos);
    free(nmass);
    free(src);
    return 0;
}

/* ------------------------------------------------------------------------------ */
/* sorted-key construction (fixed box and bounding box)                            */
/* ------------------------------------------------------------------------------ */
static void stable_sort_keys(uint32_t n, const uint32_t* key, uint32_t* skey, uint32_t* sidx) {
    uint32_t* k2 = (uint32_t*)malloc((size_t)n * sizeof(uint32_t));
    uint32_t* i2 = (uint32_t*)malloc((size_t)n * sizeof(uint32_t));
    for (uint32_t i = 0; i < n; ++i) {
        skey[i] = key[i];
        sidx[i] = i;
    }
    for (int pass = 0; pass < 4; ++pass) { /* LSD, 8-bit digits, stable */
        int shift = 8 * pass;
        uint32_t count[257];
        memset(count, 0, sizeof count);
        for (uint32_t i = 0; i < n; ++i) count[((skey[i] >> shift) & 255u) + 1]++;
        for (int b = 0; b < 256; ++b) count[b + 1] += count[b];
        for (uint32_t i = 0; i < n; ++i) {
            uint32_t b = (skey[i] >> shift) & 255u;
            uint32_t at = count[b]++;
            k2[at] = skey[i];
            i2[at] = sidx[i];
        }
        memcpy(skey, k2, (size_t)n * sizeof(uint32_t));
        memcpy(sidx, i2, (size_t)n * sizeof(uint32_t));
    }
    free(k2);
    free(i2);
}

static inline int common_bits(uint32_t a, uint32_t b, int key_bits) {
    if (a == b) return key_bits;
    return __builtin_clz(a ^ b) - (32 - key_bits);
}

static inline uint32_t compact_bits(uint32_t v) { /* inverse of spread_bits */
    v &= 0x55555555u;
    v = (v | (v >> 1)) & 0x33333333u;
    v = (v | (v >> 2)) & 0x0f0f0f0fu;
    v = (v | (v >> 4)) & 0x00ff00ffu;
    v = (v | (v >> 8)) & 0x0000ffffu;
    return v;
}

/* Squared distance from the centre of mass (cx, cy) to the farthest corner of the cell
 * at level d that holds key `key` (the opening radius of ORC_BH_SAFE_RADIUS), in FP32:
 *   fixed box:    side = 1000 / 2^d, x0 = -500 + ix * side          (both exact)
 *   bounding box: side = 2^(D-d) * inv, x0 = cx + (ix * 2^(D-d) - 2^(D-1)) * inv
 *                 with inv = float(1 / scale) taken once in FP64
 *   m = max(|c - x0|, |x0 + side - c|) per axis, bmax^2 = fma(mx, mx, my * my) */
static float cell_bmax2(int box_mode, const bbox_params* bp, int D, int d, uint32_t key, float cx, float cy) {
    uint32_t pre = key >> (2 * (D - d));
    float ix = (float)compact_bits(pre), iy = (float)compact_bits(pre >> 1);
    float x0, y0, side;
    if (box_mode == ORC_BOX_BOUNDING) {
        float w = (float)(1u << (D - d));
        side = w * bp->inv_scale;
        x0 = bp->cx + (ix * w - (float)(1u << (D - 1))) * bp->inv_scale;
        y0 = bp->cy + (iy * w - (float)(1u << (D - 1))) * bp->inv_scale;
    } else {
        side = 2.0f * SIM_SIZE / (float)(1u << d);
        x0 = -SIM_SIZE + ix * side;
        y0 = -SIM_SIZE + iy * side;
    }
    float mx = fmaxf(fabsf(cx - x0), fabsf((x0 + side) - cx));
    float my = fmaxf(fabsf(cy - y0), fabsf((y0 + side) - cy));
    return fmaf(mx, mx, my * my);
}

/* ------------------------------------------------------------------------------ */
/* accurate-mode moments (ORC_BH_QUADRUPOLE): exact integer sums                   */
/* ------------------------------------------------------------------------------ */
/* Every particle is put on an integer grid: masses as m_q = rint(m 2^(31-em)) with
 * max mass = f 2^em (f in [0.5, 1)), positions as x_q = rint(x 2^(30-e)) - rint(bx 2^(30-e))
 * with the box centre bx and half-size h = f 2^e, clamped to +-2^30.  A node's sums M = sum m_q,
 * X = sum m_q x_q, Y, XX = sum m_q x_q^2, XY, YY are exact 128-bit integers (no order
 * of summation changes them), taken as differences of prefix sums over the sorted
 * slots.  They are rounded to FP32 once:
 *   centre  cx = bx + (f(X) / f(M)) 2^(e-30),  mass  m = f(M) 2^(em-31)
 *   second central moments about an integer origin x0 = rint(f(X) / f(M)) near the
 *   centre (exact: Dx = X - x0 M, Sxx = XX - x0 (X + Dx), Sxy = XY - x0 Y - y0 Dx),
 *   Qxx = f(Sxx) - f(Dx) (f(Dx) / f(M)), Qxy = f(Sxy) - f(Dx) (f(Dy) / f(M)),
 *   Qyy = f(Syy) - f(Dy) (f(Dy) / f(M)), scaled by 2^(2(e-30)) then 2^(em-31);
 * f() rounds a 128-bit integer to the nearest float (ties to even).  A node of zero mass
 * gets centre (0, 0) and zero moments.  Positions: 2^-30 of the half-size; masses:
 * 2^-31 of the largest. */
typedef __int128 i128;
typedef unsigned __int128 u128;
typedef struct {
    i128 m, x, y, xx, xy, yy;
} mom_sums;
typedef struct {
    float bx, by, iqs, ims, qs, ms;
} mom_scale;

static float i128_to_float(i128 v) {
    const int neg = v < 0;
    const u128 u = neg ? (u128)0 - (u128)v : (u128)v;
    const uint64_t hi = (uint64_t)(u >> 64);
    float f;
    if (!hi) {
        f = (float)(uint64_t)u;
    } else { /* the top 64 bits with a sticky bit round like the whole value */
        const int sh = 64 - __builtin_clzll(hi);
        const uint64_t t = (uint64_t)(u >> sh) | (uint64_t)((u & (((u128)1 << sh) - 1)) != 0);
        f = (float)t * ldexpf(1.0f, sh);
    }
    return neg ? -f : f;
}

static int exponent_of(float v, int lo, int hi) { /* v = f 2^e, f in [0.5, 1); 0 for v <= 0 */
    int e = 0;
    if (v > 0.0f) frexpf(v, &e);
    return e < lo ? lo : e > hi ? hi : e;
}

static mom_scale moment_scale(float bx, float by, float half, float mmax) {
    mom_scale s;
    const int e = exponent_of(half, -96, 127), em = exponent_of(mmax, -94, 127);
    s.bx = bx;
    s.by = by;
    s.qs = ldexpf(1.0f, 30 - e);
    s.iqs = ldexpf(1.0f, e - 30);
    s.ms = ldexpf(1.0f, 31 - em);
    s.ims = ldexpf(1.0f, em - 31);
    return s;
}

/* p 2^(30-e), b 2^(30-e) and m 2^(31-em) are exact scalings by powers of two, each
 * rounded to the nearest integer (not p - b, which rounds to the spacing of the larger
 * operand) */
static inline int64_t quantize_pos(float p, float b, float qs) {
    const float pq = rintf(p * qs), bq = rintf(b * qs);
    if (!(fabsf(pq) < 9.0e18f) || !(fabsf(bq) < 9.0e18f)) return 0; /* beyond 64 bits, or NaN */
    int64_t q = (int64_t)pq - (int64_t)bq;
    if (q < -1073741824ll) q = -1073741824ll;
    if (q > 1073741824ll) q = 1073741824ll;
    return q;
}

static inline int64_t quantize_mass(float m, float ms) {
    return m > 0.0f ? (int64_t)rintf(m * ms) : 0;
}

static inline void mom_add_particle(mom_sums* a, float px, float py, float m, const mom_scale* sc) {
    const int64_t mq = quantize_mass(m, sc->ms);
    const int64_t xq = quantize_pos(px, sc->bx, sc->qs), yq = quantize_pos(py, sc->by, sc->qs);
    const int64_t mx = mq * xq, my = mq * yq;
    a->m += mq;
    a->x += mx;
    a->y += my;
    a->xx += (i128)mx * xq;
    a->xy += (i128)mx * yq;
    a->yy += (i128)my * yq;
}

static void mom_node(const mom_sums* hi, const mom_sums* lo, const mom_scale* sc, float* cx, float* cy, float* m,
                     float* q3) {
    mom_sums a;
    a.m = hi->m - lo->m;
    a.x = hi->x - lo->x;
    a.y = hi->y - lo->y;
    a.xx = hi->xx - lo->xx;
    a.xy = hi->xy - lo->xy;
    a.yy = hi->yy - lo->yy;
    if (a.m == 0) {
        *cx = *cy = *m = 0.0f;
        q3[0] = q3[1] = q3[2] = 0.0f;
        return;
    }
    const float mf = i128_to_float(a.m);
    const float cxq = i128_to_float(a.x) / mf, cyq = i128_to_float(a.y) / mf;
    *cx = sc->bx + cxq * sc->iqs;
    *cy = sc->by + cyq * sc->iqs;
    *m = mf * sc->ims;
    const int64_t x0 = (int64_t)rintf(cxq), y0 = (int64_t)rintf(cyq);
    const i128 dx = a.x - (i128)x0 * a.m, dy = a.y - (i128)y0 * a.m;
    const i128 sxx = a.xx - (i128)x0 * (a.x + dx);
    const i128 sxy = a.xy - (i128)x0 * a.y - (i128)y0 * dx;
    const i128 syy = a.yy - (i128)y0 * (a.y + dy);
    const float dxf = i128_to_float(dx), dyf = i128_to_float(dy);
    const float ux = dxf / mf, uy = dyf / mf;
    const float qxx = i128_to_float(sxx) - dxf * ux;
    const float qxy = i128_to_float(sxy) - dxf * uy;
    const float qyy = i128_to_float(syy) - dyf * uy;
    const float s2 = sc->iqs * sc->iqs;
    q3[0] = (qxx * s2) * sc->ims;
    q3[1] = (qxy * s2) * sc->ims;
    q3[2] = (qyy * s2) * sc->ims;
}

int orc_bh_sorted_step(int box_mode, uint32_t n_al, float* pos_in, float* vel_in,
                       float* mass_in, float* pos_out, float* vel_out, float* mass_out,
                       float dt, float G, float eps2, float theta2, orc_bh_out* out,
                       int nthreads) {
    return orc_bh_sorted_step_ex(box_mode, 0, n_al, pos_in, vel_in, mass_in, pos_out, vel_out, mass_out, dt, G,
                                 eps2, theta2, out, nthreads);
}

int orc_bh_sorted_step_ex(int box_mode, int flags, uint32_t n_al, float* pos_in, float* vel_in,
                          float* mass_in, float* pos_out, float* vel_out, float* mass_out,
                          float dt, float G, float eps2, float theta2, orc_bh_out* out,
                          int nthreads) {
    int bits = out && out->key_bits ? (int)out->key_bits : BBOX_BITS;
    if (bits < 1 || bits > BBOX_MAX_BITS) return -1;
    const int D = box_mode == ORC_BOX_BOUNDING ? bits : GRID_LEVELS - 1;
    const int key_bits = 2 * D;
    const double t_build = now_seconds();
    uint32_t* key = (uint32_t*)malloc((size_t)n_al * sizeof(uint32_t));
    uint32_t* skey = (uint32_t*)malloc((size_t)n_al * sizeof(uint32_t));
    uint32_t* sidx = (uint32_t*)malloc((size_t)n_al * sizeof(uint32_t));
    float radius0;
    bbox_params bp = {0.0f, 0.0f, (float)GRID / (2.0f * SIM_SIZE), SIM_SIZE * SIM_SIZE * 2.0f,
                      2.0f * SIM_SIZE / (float)GRID, 10};

    if (box_mode == ORC_BOX_BOUNDING) {
        double mnx = INFINITY, mxx = -INFINITY, mny = INFINITY, mxy = -INFINITY;
        for (uint32_t i = 0; i < n_al; ++i) {
            double x = pos_in[2 * i], y = pos_in[2 * i + 1];
            if (x < mnx) mnx = x;
            if (x > mxx) mxx = x;
            if (y < mny) mny = y;
            if (y > mxy) mxy = y;
        }
        bp = bbox_from_minmax(mnx, mxx, mny, mxy, bits);
        for (uint32_t i = 0; i < n_al; ++i) key[i] = bbox_key(pos_in[2 * i], pos_in[2 * i + 1], &bp);
        radius0 = bp.radius0;
    } else {
        for (uint32_t i = 0; i < n_al; ++i) {
            uint32_t k;
            if (fixed_box_key(pos_in[2 * i], pos_in[2 * i + 1], &k)) {
                key[i] = k;
            } else { /* InitShader.comp:110-117 */
                key[i] = ORC_KEY_REMOVED;
                pos_in[2 * i] = pos_in[2 * i + 1] = -SIM_SIZE * 2.0f;
                pos_out[2 * i] = pos_out[2 * i + 1] = -SIM_SIZE * 2.0f;
                mass_in[i] = 0.0f;
                mass_out[i] = 0.0f;
            }
        }
        radius0 = SIM_SIZE * SIM_SIZE * 2.0f;
    }
    if (out && out->keys) memcpy(out->keys, key, (size_t)n_al * sizeof(uint32_t));

    stable_sort_keys(n_al, key, skey, sidx);
    uint32_t nv = 0;
    while (nv < n_al && skey[nv] != ORC_KEY_REMOVED) ++nv;

    /* per-slot levels: nodes (d, s) for d in [dmin(s), dmax(s)] start at slot s */
    int* dmin = (int*)malloc(((size_t)nv + 1) * sizeof(int));
    int* dmax = (int*)malloc(((size_t)nv + 1) * sizeof(int));
    uint64_t* E = (uint64_t*)malloc(((size_t)nv + 1) * sizeof(uint64_t));
    uint64_t total = 0;
    for (uint32_t s = 0; s < nv; ++s) {
        dmin[s] = s == 0 ? 0 : common_bits(skey[s - 1], skey[s], key_bits) / 2 + 1;
        dmax[s] = s + 1 < nv ? common_bits(skey[s], skey[s + 1], key_bits) / 2 : -1;
        E[s] = total;
        int e = dmax[s] - dmin[s] + 1;
        total += (uint64_t)(e > 0 ? e : 0);
    }
    E[nv] = total;
    const uint64_t tree_size = (uint64_t)nv + total;

    uint64_t cap = orc_bh_node_capacity(box_mode, n_al);
    uint32_t* skip = (uint32_t*)calloc(cap, sizeof(uint32_t));
    float* radius = (float*)calloc(cap, sizeof(float));
    float* npos = (float*)calloc(2 * cap, sizeof(float));
    float* nmass = (float*)calloc(cap, sizeof(float));
    uint32_t* nend = (uint32_t*)calloc(cap, sizeof(uint32_t));
    float* msx = (float*)calloc(cap, sizeof(float));
    float* msy = (float*)calloc(cap, sizeof(float));
    float* quad = (flags & ORC_BH_QUADRUPOLE) ? (float*)calloc(3 * cap, sizeof(float)) : NULL;

    /* records: topology, radius and particle leaves */
    for (uint32_t s = 0; s < nv; ++s) {
        for (int d = dmin[s]; d <= dmax[s]; ++d) {
            uint64_t at = s + E[s] + (uint64_t)(d - dmin[s]);
            uint32_t shift = (uint32_t)(key_bits - 2 * d);
            uint32_t pre = shift >= 32 ? 0 : skey[s] >> shift;
            uint32_t end = s + 1;
            while (end < nv && (shift >= 32 ? 0 : skey[end] >> shift) == pre) ++end;
            nend[at] = end;
            skip[at] = (uint32_t)((uint64_t)end + E[end] - at);
            radius[at] = radius0 / (float)(1u << (2 * d));
        }
        uint64_t leaf = s + E[s] + (uint64_t)(dmax[s] >= dmin[s] ? dmax[s] - dmin[s] + 1 : 0);
        uint32_t i = sidx[s];
        skip[leaf] = 1;
        radius[leaf] = 0.0f;
        npos[2 * leaf] = pos_in[2 * i];
        npos[2 * leaf + 1] = pos_in[2 * i + 1];
        nmass[leaf] = mass_in[i];
    }

    if (quad) { /* accurate mode: exact integer sums over each node's particles */
        float mmax = 0.0f;
        for (uint32_t i = 0; i < n_al; ++i)
            if (mass_in[i] > mmax) mmax = mass_in[i];
        const float half = box_mode == ORC_BOX_BOUNDING ? ldexpf(bp.inv_scale, bp.bits - 1) : SIM_SIZE;
        const float bx = box_mode == ORC_BOX_BOUNDING ? bp.cx : 0.0f;
        const float by = box_mode == ORC_BOX_BOUNDING ? bp.cy : 0.0f;
        const mom_scale sc = moment_scale(bx, by, half, mmax);
        mom_sums* P = (mom_sums*)calloc((size_t)nv + 1, sizeof(mom_sums));
        for (uint32_t t = 0; t < nv; ++t) { /* exclusive prefix over the sorted slots */
            P[t + 1] = P[t];
            const uint32_t i = sidx[t];
            mom_add_particle(&P[t + 1], pos_in[2 * i], pos_in[2 * i + 1], mass_in[i], &sc);
        }
        for (uint32_t s = 0; s < nv; ++s) {
            for (int d = dmin[s]; d <= dmax[s]; ++d) {
                uint64_t at = s + E[s] + (uint64_t)(d - dmin[s]);
                float cx, cy, m;
                mom_node(&P[nend[at]], &P[s], &sc, &cx, &cy, &m, &quad[3 * at]);
                npos[2 * at] = cx;
                npos[2 * at + 1] = cy;
                nmass[at] = m;
                if (flags & ORC_BH_SAFE_RADIUS) radius[at] = cell_bmax2(box_mode, &bp, D, d, skey[s], cx, cy);
            }
        }
        free(P);
    } else {
        /* mass and mass-moment sums, finest level first, children in Morton order
         * (TreeInitShader.comp:78-80), centre of mass TreeMoveShader.comp:66-67 */
        for (int d = D; d >= 0; --d) {
            for (uint32_t s = 0; s < nv; ++s) {
                if (d < dmin[s] || d > dmax[s]) continue;
                uint64_t at = s + E[s] + (uint64_t)(d - dmin[s]);
                uint32_t end = nend[at];
                float sx = 0.0f, sy = 0.0f, sm = 0.0f;
                uint32_t t = s;
                while (t < end) {
                    if (d < D && dmin[t] <= d + 1 && d + 1 <= dmax[t]) {
                        uint64_t ch = t + E[t] + (uint64_t)(d + 1 - dmin[t]);
                        sx = sx + msx[ch];
                        sy = sy + msy[ch];
                        sm = sm + nmass[ch];
                        t = nend[ch];
                    } else {
                        uint32_t i = sidx[t];
                        float m = mass_in[i];
                        sx = sx + pos_in[2 * i] * m;
                        sy = sy + pos_in[2 * i + 1] * m;
                        sm = sm + m;
                        t += 1;
                    }
                }
                msx[at] = sx;
                msy[at] = sy;
                nmass[at] = sm;
                if (sm != 0.0f) {
                    sx = sx / sm;
                    sy = sy / sm;
                }
                npos[2 * at] = sx;
                npos[2 * at + 1] = sy;
                if (flags & ORC_BH_SAFE_RADIUS) radius[at] = cell_bmax2(box_mode, &bp, D, d, skey[s], sx, sy);
            }
        }
    }

    uint32_t* src = (uint32_t*)malloc((size_t)n_al * sizeof(uint32_t));
    for (uint32_t s = 0; s < n_al; ++s) src[s] = s < nv ? sidx[s] : n_al;
    if (out) out->build_seconds = now_seconds() - t_build;

    walk_ctx wc;
    memset(&wc, 0, sizeof wc);
    wc.skip = skip;
    wc.radius = radius;
    wc.npos = npos;
    wc.nmass = nmass;
    wc.quad = quad;
    wc.group_walk = (flags & ORC_BH_GROUP_WALK) != 0;
    wc.skey = skey;
    wc.group_size = GROUP_SIZE;
    wc.tree_size = tree_size;
    wc.src = src;
    wc.n_al = n_al;
    wc.pos_in = pos_in;
    wc.vel_in = vel_in;
    wc.mass_in = mass_in;
    wc.pos_out = pos_out;
    wc.vel_out = vel_out;
    wc.eps2 = eps2;
    wc.theta2 = theta2;
    wc.k = G * dt;
    wc.hdt = 0.5f * dt;
    if ((flags & ORC_BH_RELATIVE_MAC) && out) {
        wc.rel_alpha = out->rel_alpha;
        wc.rel_floor2 = out->rel_floor2;
        wc.amag_in = out->amag_in;
        wc.amag_out = out->amag_out;
    }
    if (out) {
        wc.group_visits = out->group_visits;
        wc.group_inter = out->group_interactions;
    }
    run_walk(&wc, nthreads, out);

    if (out) {
        out->tree_size = tree_size;
        out->valid_count = nv;
        out->internal_count = total;
        if (out->node_quad && quad) {
            uint64_t nq = tree_size < out->node_capacity ? tree_size : out->node_capacity;
            memcpy(out->node_quad, quad, 3 * nq * sizeof(float));
        }
        if (out->sorted_src) memcpy(out->sorted_src, src, (size_t)n_al * sizeof(uint32_t));
        copy_tree_out(out, skip, radius, npos, nmass, tree_size);
        out->box_center_x = bp.cx;
        out->box_center_y = bp.cy;
        out->box_scale = bp.scale;
        out->box_radius0 = radius0;
    }
    free(key);
    free(skey);
    free(sidx);
    free(dmin);
    free(dmax);
    free(E);
    free(skip);
    free(radius);
    free(npos);
    free(nmass);
    free(nend);
    free(msx);
    free(msy);
    free(quad);
    free(src);
    return 0;
}

/* ------------------------------------------------------------------------------ */
/* seeded generators -- the library's gs_generate restated, so that the CPU       */
/* baseline and the reference arm make their inputs without the library.  The     */
/* presets follow ParticleSystem.cpp:15-149 (draw order per particle: angle,       */
/* radius, mass) with an explicit seed: splitmix64, 24-bit float conversion.      */
/* ------------------------------------------------------------------------------ */
static const double ORC_PI = 3.14159265358979323846;

typedef struct { uint64_t s; } orc_rng;
static uint64_t rng_next(orc_rng* r) { /* splitmix64 */
    uint64_t z = (r->s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static float rng_uniform(orc_rng* r) { return (float)(rng_next(r) >> 40) * (1.0f / 16777216.0f); }
static double rng_uniform_open(orc_rng* r) {
    return ((double)(rng_next(r) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}
static double rng_normal(orc_rng* r) { /* Box-Muller */
    double u1 = rng_uniform_open(r), u2 = rng_uniform_open(r);
    return sqrt(-2.0 * log(u1)) * cos(2.0 * ORC_PI * u2);
}

static void og_random(orc_rng* r, size_t n, float size, float mn, float mx, float* p, float* v, float* m) {
    for (size_t i = 0; i < n; ++i) {
        float theta = (float)((double)(rng_uniform(r) * 2.0f) * ORC_PI);
        float rad = sqrtf(1.0f - rng_uniform(r)) * size;
        p[2 * i] = rad * cosf(theta);
        p[2 * i + 1] = rad * sinf(theta);
        v[2 * i] = v[2 * i + 1] = 0.0f;
        m[i] = rng_uniform(r) * (mx - mn) + mn;
    }
}

static void og_galaxy(orc_rng* r, size_t n, float size, float mn, float mx, float G, float* p, float* v, float* m) {
    float avg = (mn + mx) * 0.5f;
    float vel = sqrtf(G * (float)n * avg / (size * size * size));
    for (size_t i = 0; i < n; ++i) {
        float theta = (float)((double)(rng_uniform(r) * 2.0f) * ORC_PI);
        float rad = (1.0f - rng_uniform(r)) * size;
        float sn = sinf(theta), cs = cosf(theta);
        p[2 * i] = rad * cs;
        p[2 * i + 1] = rad * sn;
        v[2 * i] = -sn * rad * vel;
        v[2 * i + 1] = cs * rad * vel;
        m[i] = rng_uniform(r) * (mx - mn) + mn;
    }
}

static void og_collision(orc_rng* r, size_t n, float size, float mn, float mx, float G, float* p, float* v,
                         float* m) {
    float gs = size / 3.0f;
    float avg = (mn + mx) * 0.25f;
    float vel = sqrtf(G * (float)n * avg / (gs * gs * gs));
    for (size_t i = 0; i < n; ++i) {
        float side = i < (n >> 1) ? -1.0f : 1.0f;
        float theta = (float)((double)(rng_uniform(r) * 2.0f) * ORC_PI);
        float rad = (1.0f - rng_uniform(r)) * gs;
        float sn = sinf(theta), cs = cosf(theta);
        p[2 * i] = rad * cs + side * gs * 2.0f;
        p[2 * i + 1] = rad * sn;
        v[2 * i] = -sn * rad * vel - side * gs * 0.1f;
        v[2 * i + 1] = cs * rad * vel;
        m[i] = rng_uniform(r) * (mx - mn) + mn;
    }
}

static void og_symmetric(orc_rng* r, size_t n, float size, float mn, float mx, float G, float* p, float* v,
                         float* m) {
    float gs = size / 3.0f;
    float avg = (mn + mx) * 0.25f;
    float vel = sqrtf(G * (float)n * avg / (gs * gs * gs));
    for (size_t i = 0; i + 1 < n; i += 2) {
        float theta = (float)((double)(rng_uniform(r) * 2.0f) * ORC_PI);
        float rad = (1.0f - rng_uniform(r)) * gs;
        float sn = sinf(theta), cs = cosf(theta);
        p[2 * i] = rad * cs - gs * 2.0f;
        p[2 * i + 1] = rad * sn;
        v[2 * i] = -sn * rad * vel + gs * 0.1f;
        v[2 * i + 1] = cs * rad * vel;
        m[i] = rng_uniform(r) * (mx - mn) + mn;
        p[2 * i + 2] = -p[2 * i];
        p[2 * i + 3] = p[2 * i + 1];
        v[2 * i + 2] = -sn * rad * vel - gs * 0.1f;
        v[2 * i + 3] = -cs * rad * vel;
        m[i + 1] = m[i];
    }
}

static void og_uniform_disk(orc_rng* r, size_t n, float radius, float mn, float mx, float* p, float* v, float* m) {
    for (size_t i = 0; i < n; ++i) {
        double rad = radius * sqrt((double)rng_uniform(r));
        double phi = 2.0 * ORC_PI * (double)rng_uniform(r);
        p[2 * i] = (float)(rad * cos(phi));
        p[2 * i + 1] = (float)(rad * sin(phi));
        v[2 * i] = v[2 * i + 1] = 0.0f;
        m[i] = mn + (mx - mn) * rng_uniform(r);
    }
}

static const double* og_sort_key;
static int og_by_radius(const void* a, const void* b) { /* radius, then index: a total order */
    const size_t i = *(const size_t*)a, j = *(const size_t*)b;
    if (og_sort_key[i] < og_sort_key[j]) return -1;
    if (og_sort_key[i] > og_sort_key[j]) return 1;
    return i < j ? -1 : (i > j ? 1 : 0);
}

/* exponential disk (scale h, truncated at rmax) around (cx, cy), optional two-arm
 * logarithmic spiral, circular velocity from the enclosed sample mass plus Gaussian
 * dispersion disp * v_c per component, plus a bulk velocity */
static void og_exp_disk(orc_rng* r, size_t n, double h, double rmax, double pitch_deg, double amp, double disp,
                        double cx, double cy, double bvx, double bvy, float mn, float mx, float G, float* p, float* v,
                        float* m) {
    double* rad = (double*)malloc(n * sizeof(double));
    double* phi = (double*)malloc(n * sizeof(double));
    size_t* order = (size_t*)malloc(n * sizeof(size_t));
    const double cot = 1.0 / tan(pitch_deg * ORC_PI / 180.0);
    for (size_t i = 0; i < n; ++i) {
        double rr;
        do {
            rr = -h * log(rng_uniform_open(r) * rng_uniform_open(r)); /* Gamma(2, h) */
        } while (rr > rmax);
        double ph;
        if (amp > 0.0) {
            for (;;) {
                ph = 2.0 * ORC_PI * rng_uniform_open(r);
                double f = 1.0 + amp * cos(2.0 * (ph - log(rr) * cot));
                if (rng_uniform_open(r) * (1.0 + amp) <= f) break;
            }
        } else {
            ph = 2.0 * ORC_PI * rng_uniform_open(r);
        }
        rad[i] = rr;
        phi[i] = ph;
        m[i] = mn + (mx - mn) * rng_uniform(r);
        order[i] = i;
    }
    og_sort_key = rad;
    qsort(order, n, sizeof(size_t), og_by_radius);
    double enclosed = 0.0;
    for (size_t q = 0; q < n; ++q) {
        size_t i = order[q];
        double rr = rad[i];
        double vc = rr > 0.0 ? sqrt((double)G * enclosed / rr) : 0.0;
        enclosed += m[i];
        double c = cos(phi[i]), s = sin(phi[i]);
        p[2 * i] = (float)(cx + rr * c);
        p[2 * i + 1] = (float)(cy + rr * s);
        double vx = -s * vc + disp * vc * rng_normal(r) + bvx;
        double vy = c * vc + disp * vc * rng_normal(r) + bvy;
        v[2 * i] = (float)vx;
        v[2 * i + 1] = (float)vy;
    }
    free(rad);
    free(phi);
    free(order);
}

int orc_generate(int type, uint64_t count, float size, float mn, float mx, float G, uint64_t seed, float* pos,
                 float* vel, float* mass) {
    if (!count || !pos || !vel || !mass) return -1;
    orc_rng r = {seed};
    switch (type) {
        case 0: og_random(&r, count, size, mn, mx, pos, vel, mass); break;
        case 1: og_galaxy(&r, count, size, mn, mx, G, pos, vel, mass); break;
        case 2: og_collision(&r, count, size, mn, mx, G, pos, vel, mass); break;
        case 3:
            if (count & 1) return -1;
            og_symmetric(&r, count, size, mn, mx, G, pos, vel, mass);
            break;
        case 16: og_uniform_disk(&r, count, size, mn, mx, pos, vel, mass); break;
        case 17: /* scale 30, radius 100 confines, pitch 15 deg, amplitude 0.3, 5% dispersion */
            og_exp_disk(&r, count, 30.0 * size / 100.0, size, 15.0, 0.3, 0.05, 0.0, 0.0, 0.0, 0.0, mn, mx, G, pos, vel,
                        mass);
            break;
        case 18: { /* two disks, scale 20, truncated at r <= 50, at (+-50, 0), v = (0, +-3) */
            size_t h = count / 2;
            og_exp_disk(&r, h, 20.0, 50.0, 15.0, 0.0, 0.0, -50.0, 0.0, 0.0, -3.0, mn, mx, G, pos, vel, mass);
            og_exp_disk(&r, count - h, 20.0, 50.0, 15.0, 0.0, 0.0, 50.0, 0.0, 0.0, 3.0, mn, mx, G, pos + 2 * h,
                        vel + 2 * h, mass + h);
            break;
        }
        default: return -1;
    }
    return 0;
}
