/*
 * gsim_oracle.h -- CPU restatement of Gravity-Sim's force-and-integrate path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product links this library: it is the
 * checker that the CUDA path is compared against (tests/, the smoke check and the
 * CPU-baseline leg of bench.py).
 *
 * Parity status: the reference computes forces only in Vulkan compute shaders and
 * ships no tests, fixtures or golden vectors, so this restatement cannot be pinned
 * against reference outputs.  It is pinned against (a) the FP64 direct sum, (b)
 * invariants the reference's design implies (momentum conservation, mirror symmetry,
 * two-body orbit, permutation invariance) and (c) two independent restatements of the
 * Barnes-Hut tree that must agree bit for bit: the literal 1024x1024 grid of the
 * shaders (orc_bh_grid_step) and the sorted-key construction (orc_bh_sorted_step).
 *
 * Canonical arithmetic.  GLSL leaves FMA contraction and the precision of division
 * to the driver; the library and this restatement fix one sequence and use it alike:
 *   d2  = fma(dx, dx, fma(dy, dy, eps2))
 *   r   = 1 / sqrt(d2)           (correctly rounded sqrt, then correctly rounded divide)
 *   s   = ((m * r) * r) * r
 *   a   = fma(d, s, a)           (per component)
 *   v'  = fma(a, G*dt, v)
 *   x'  = fma(v + v', 0.5*dt, x)
 * Barnes-Hut cell keys use IEEE division and addition exactly as written in the
 * shaders: rel = ((p / S) + 1) * 0.5 * 1024.
 */
#ifndef GSIM_ORACLE_H
#define GSIM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Key value given to particles that the fixed-box mode removes (outside +-500). */
#define ORC_KEY_REMOVED 0xFFFFFFFFu

/* Box modes for the sorted-key construction. */
#define ORC_BOX_FIXED_500 0
#define ORC_BOX_BOUNDING 1

/* Everything one Barnes-Hut step exposes for bit-exact comparison.  Arrays are
 * caller-allocated; any pointer may be NULL to skip that output.
 *   keys       [n_al]        per-particle cell key in original order
 *   sorted_src [n_al]        original index per sorted slot, n_al for empty slots
 *   node_skip  [capacity]    preorder node records (the reference's counts[] buffer)
 *   node_radius[capacity]
 *   node_pos   [2*capacity]
 *   node_mass  [capacity]
 *   interactions             accepted (lane, node) pairs over valid lanes   */
typedef struct orc_bh_out {
    uint32_t* keys;
    uint32_t* sorted_src;
    uint32_t* node_skip;
    float* node_radius;
    float* node_pos;
    float* node_mass;
    float* node_quad;        /* [3*capacity] second central moments (ORC_BH_QUADRUPOLE) */
    uint64_t node_capacity;
    uint32_t walk_stride;    /* input: walk only warps w with w % stride == 0 (0 or 1: all) */
    /* filled by the step */
    uint64_t tree_size;      /* number of preorder records (internal nodes + leaves) */
    uint64_t valid_count;    /* particles that were placed in the tree */
    uint64_t internal_count; /* internal nodes */
    uint64_t interactions;   /* accepted (valid lane, node) pairs */
    uint64_t warp_visits;    /* visited nodes summed over warps */
    /* bounding-box mode parameters actually used */
    float box_center_x, box_center_y, box_scale, box_radius0;
    double build_seconds;    /* keys, sort and tree (single thread) */
    double walk_seconds;     /* force walk + integration (nthreads) */
    uint32_t max_stack;      /* deepest group-walk stack seen (ORC_BH_GROUP_WALK) */
    uint64_t max_warp_interactions; /* largest interaction count of one warp (valid lanes) */
    /* inputs of ORC_BH_RELATIVE_MAC */
    float rel_alpha;         /* alpha of the relative opening criterion */
    float rel_floor2;        /* squared theta floor of the relative criterion */
    const float* amag_in;    /* [n_al] |a| of the previous step per particle (NaN: unknown) */
    float* amag_out;         /* [n_al] |a| of this step (written when not NULL) */
    /* input of the bounding-box mode */
    uint32_t key_bits;       /* bits per axis, 1..15 (0: 12, 24-bit keys; 15: 30-bit keys) */
    /* optional outputs of the group walk: records tested and interactions of each group
     * of 64 sorted slots (n_al / 64 entries, estimate walk included) */
    uint32_t* group_visits;
    uint64_t* group_interactions;
} orc_bh_out;

/* Direct sum, SimShader.comp order: for every i, sum j = 0 .. n-1 in order. */
void orc_direct_step(uint32_t n, const float* pos_in, const float* vel_in, const float* mass_in,
                     float* pos_out, float* vel_out, float dt, float G, float eps2, int nthreads);

/* FP32 accelerations (no G), same arithmetic and order as orc_direct_step. */
void orc_direct_accel(uint32_t n, const float* pos, const float* mass, float eps2, float* acc,
                      int nthreads);

/* FP64 accelerations (no G) for the listed targets over all n sources. */
void orc_direct_accel_f64(uint32_t n, const float* pos, const float* mass, double eps2,
                          uint32_t n_targets, const uint32_t* targets, double* acc, int nthreads);

/* Barnes-Hut step on the literal 1024x1024 grid of the seven shaders (fixed box). */
int orc_bh_grid_step(uint32_t n_al, float* pos_in, float* vel_in, float* mass_in,
                     float* pos_out, float* vel_out, float* mass_out, float dt, float G,
                     float eps2, float theta2, orc_bh_out* out, int nthreads);

/* Barnes-Hut step built from sorted cell keys (fixed box or bounding box). */
int orc_bh_sorted_step(int box_mode, uint32_t n_al, float* pos_in, float* vel_in,
                       float* mass_in, float* pos_out, float* vel_out, float* mass_out,
                       float dt, float G, float eps2, float theta2, orc_bh_out* out,
                       int nthreads);

/* Flags of the accurate Barnes-Hut mode (not in the reference):
 *   ORC_BH_QUADRUPOLE   nodes carry second central moments; accepted nodes add the
 *                       quadrupole term (particle leaves stay monopoles)
 *   ORC_BH_SAFE_RADIUS  the opening radius is the squared distance from the centre of
 *                       mass to the farthest corner of the cell (the reference's s^2/2
 *                       is that value for a centred centre of mass), so a cell that holds
 *                       the particle is never accepted for theta <= 1 */
#define ORC_BH_QUADRUPOLE 1
#define ORC_BH_SAFE_RADIUS 2
#define ORC_BH_GROUP_WALK 4  /* box-tested stack walk shared by 64 particles, see group_walk_warp */
/* With ORC_BH_GROUP_WALK: relative opening criterion (not in the reference).  A node of
 * mass m and stored squared opening radius R is accepted for a group at softened squared
 * distance D (nearest sub-box) when R <= D and m^2 R^3 <= (alpha a_min)^2 D^5, in that
 * FP32 operation order: lhs = (m*m)*((R*R)*R), rhs = tol^2*((D^2*D^2)*D) with
 * tol = alpha*a_min, a_min the smallest previous |a| (without G) of the group's particles
 * (out->amag_in) -- or when R <= D floor^2 (out->rel_floor2; the floor bounds the walk
 * of a group whose a_min is tiny).  A group with an unknown |a| (NaN) uses the
 * geometric test R <= D theta^2 alone. */
#define ORC_BH_RELATIVE_MAC 8
int orc_bh_sorted_step_ex(int box_mode, int flags, uint32_t n_al, float* pos_in, float* vel_in,
                          float* mass_in, float* pos_out, float* vel_out, float* mass_out,
                          float dt, float G, float eps2, float theta2, orc_bh_out* out,
                          int nthreads);

/* The library's seeded generators (gs_generate types 0-3, 16-18), restated: the same
 * particles for the same arguments.  Returns 0, or -1 for an unknown type or bad count. */
int orc_generate(int type, uint64_t count, float size, float mn, float mx, float G, uint64_t seed, float* pos,
                 float* vel, float* mass);

/* 0: costly groups walk alone as well (a test switch: pairing changes only the order of
 * the sums); 1 (default): they walk as warp pairs, as the library does. */
void orc_set_heavy_pairs(int on);

/* Upper bound on preorder records for n_al particles in either mode. */
uint64_t orc_bh_node_capacity(int box_mode, uint32_t n_al);

/* Energy of a state (kinetic + softened pairwise potential, FP64, includes G). */
/* Point splat of VertShader.vert:13-18 / FragShader.frag (one white pixel per particle on
 * black): camera = {x, y, width, height}; screen = (p - cam.xy) / cam.wh, y flipped;
 * pixel = floor((screen + 1) * size / 2) when inside; image = width x height bytes. */
void orc_render_points(uint32_t n, const float* pos, const float* camera, uint32_t width, uint32_t height,
                       uint8_t* image);
double orc_energy_f64(uint32_t n, const float* pos, const float* vel, const float* mass,
                      double G, double eps2);

#ifdef __cplusplus
}
#endif
#endif
