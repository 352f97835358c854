// host.cpp -- host-only helpers of the C ABI: seeded particle generators and the
// particle text format.  No GPU is touched here.
//
// Generators.  The reference seeds std::default_random_engine from time(nullptr)
// (src/Particles/ParticleSystem.cpp:18,40,69,118), so its presets are not reproducible;
// here every generator takes an explicit 64-bit seed and draws from splitmix64 with a
// 24-bit float conversion, so that the same seed gives the same particles on every
// host.  The four presets follow the shapes of ParticleSystem.cpp:15-149 (same draw
// order per particle: angle, radius, mass); the three measurement workloads are the
// seeded uniform disk, spiral galaxy and exponential-disk collision.
//
// File format.  Records "x y vx vy m" read with fscanf("%f%f%f%f%f") until the first
// incomplete record (ParticleSystem.cpp:462), written with "%.7f %.7f %.7f %.7f %.7f\n"
// (ParticleSystem.cpp:743), so files are byte-identical to the reference's output.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/gsim.h"

namespace gsim {
void set_error(const std::string& msg);
}

namespace {

constexpr double kPi = 3.14159265358979323846;

struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next() {  // splitmix64
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    float uniform() { return (float)(next() >> 40) * (1.0f / 16777216.0f); }  // [0, 1), 24 bits
    double uniform_open() { return ((double)(next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }  // (0, 1)
    double normal() {  // Box-Muller
        double u1 = uniform_open(), u2 = uniform_open();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * kPi * u2);
    }
};

gs_status bad(const char* msg) {
    gsim::set_error(msg);
    return GS_ERR_INVALID_ARGUMENT;
}

// ---- the reference's presets, ParticleSystem.cpp:15-149 ----
void gen_random(Rng& r, size_t n, float size, float mn, float mx, float* p, float* v, float* m) {
    for (size_t i = 0; i < n; ++i) {
        float theta = (float)((double)(r.uniform() * 2.0f) * kPi);
        float rad = std::sqrt(1.0f - r.uniform()) * size;
        p[2 * i] = rad * std::cos(theta);
        p[2 * i + 1] = rad * std::sin(theta);
        v[2 * i] = v[2 * i + 1] = 0.0f;
        m[i] = r.uniform() * (mx - mn) + mn;
    }
}

void gen_galaxy(Rng& r, size_t n, float size, float mn, float mx, float G, float* p, float* v, float* m) {
    float avg = (mn + mx) * 0.5f;
    float vel = std::sqrt(G * (float)n * avg / (size * size * size));
    for (size_t i = 0; i < n; ++i) {
        float theta = (float)((double)(r.uniform() * 2.0f) * kPi);
        float rad = (1.0f - r.uniform()) * size;
        float sn = std::sin(theta), cs = std::cos(theta);
        p[2 * i] = rad * cs;
        p[2 * i + 1] = rad * sn;
        v[2 * i] = -sn * rad * vel;
        v[2 * i + 1] = cs * rad * vel;
        m[i] = r.uniform() * (mx - mn) + mn;
    }
}

void gen_collision(Rng& r, size_t n, float size, float mn, float mx, float G, float* p, float* v, float* m) {
    float gs = size / 3.0f;
    float avg = (mn + mx) * 0.25f;
    float vel = std::sqrt(G * (float)n * avg / (gs * gs * gs));
    for (size_t i = 0; i < n; ++i) {
        float side = i < (n >> 1) ? -1.0f : 1.0f;
        float theta = (float)((double)(r.uniform() * 2.0f) * kPi);
        float rad = (1.0f - r.uniform()) * gs;
        float sn = std::sin(theta), cs = std::cos(theta);
        p[2 * i] = rad * cs + side * gs * 2.0f;
        p[2 * i + 1] = rad * sn;
        v[2 * i] = -sn * rad * vel - side * gs * 0.1f;
        v[2 * i + 1] = cs * rad * vel;
        m[i] = r.uniform() * (mx - mn) + mn;
    }
}

void gen_symmetric(Rng& r, size_t n, float size, float mn, float mx, float G, float* p, float* v, float* m) {
    float gs = size / 3.0f;
    float avg = (mn + mx) * 0.25f;
    float vel = std::sqrt(G * (float)n * avg / (gs * gs * gs));
    for (size_t i = 0; i + 1 < n; i += 2) {
        float theta = (float)((double)(r.uniform() * 2.0f) * kPi);
        float rad = (1.0f - r.uniform()) * gs;
        float sn = std::sin(theta), cs = std::cos(theta);
        p[2 * i] = rad * cs - gs * 2.0f;
        p[2 * i + 1] = rad * sn;
        v[2 * i] = -sn * rad * vel + gs * 0.1f;
        v[2 * i + 1] = cs * rad * vel;
        m[i] = r.uniform() * (mx - mn) + mn;
        p[2 * i + 2] = -p[2 * i];  // mirror image in x
        p[2 * i + 3] = p[2 * i + 1];
        v[2 * i + 2] = -sn * rad * vel - gs * 0.1f;
        v[2 * i + 3] = -cs * rad * vel;
        m[i + 1] = m[i];
    }
}

// ---- measurement workloads ----
void gen_uniform_disk(Rng& r, size_t n, float radius, float mn, float mx, float* p, float* v, float* m) {
    for (size_t i = 0; i < n; ++i) {
        double rad = radius * std::sqrt((double)r.uniform());
        double phi = 2.0 * kPi * (double)r.uniform();
        p[2 * i] = (float)(rad * std::cos(phi));
        p[2 * i + 1] = (float)(rad * std::sin(phi));
        v[2 * i] = v[2 * i + 1] = 0.0f;
        m[i] = mn + (mx - mn) * r.uniform();
    }
}

// Exponential disk (scale h, truncated at rmax) around (cx, cy), optional two-arm
// logarithmic spiral (pitch, amplitude), circular velocity from the enclosed sample mass
// sqrt(G M(<r) / r) plus Gaussian dispersion `disp` * v_c per component, bulk velocity.
void gen_exp_disk(Rng& r, size_t n, double h, double rmax, double pitch_deg, double amp, double disp, double cx,
                  double cy, double bvx, double bvy, float mn, float mx, float G, float* p, float* v, float* m) {
    std::vector<double> rad(n), phi(n);
    const double cot = 1.0 / std::tan(pitch_deg * kPi / 180.0);
    for (size_t i = 0; i < n; ++i) {
        double rr;
        do {
            rr = -h * std::log(r.uniform_open() * r.uniform_open());  // Gamma(2, h): density ~ r exp(-r/h)
        } while (rr > rmax);
        double ph;
        if (amp > 0.0) {
            for (;;) {
                ph = 2.0 * kPi * r.uniform_open();
                double f = 1.0 + amp * std::cos(2.0 * (ph - std::log(rr) * cot));
                if (r.uniform_open() * (1.0 + amp) <= f) break;
            }
        } else {
            ph = 2.0 * kPi * r.uniform_open();
        }
        rad[i] = rr;
        phi[i] = ph;
        m[i] = mn + (mx - mn) * r.uniform();
    }
    std::vector<size_t> order(n);
    std::iota(order.begin(), order.end(), size_t(0));
    std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return rad[a] < rad[b] || (rad[a] == rad[b] && a < b); });
    double enclosed = 0.0;
    for (size_t q = 0; q < n; ++q) {
        size_t i = order[q];
        double rr = rad[i];
        double vc = rr > 0.0 ? std::sqrt((double)G * enclosed / rr) : 0.0;
        enclosed += m[i];
        double c = std::cos(phi[i]), s = std::sin(phi[i]);
        p[2 * i] = (float)(cx + rr * c);
        p[2 * i + 1] = (float)(cy + rr * s);
        double vx = -s * vc + disp * vc * r.normal() + bvx;
        double vy = c * vc + disp * vc * r.normal() + bvy;
        v[2 * i] = (float)vx;
        v[2 * i + 1] = (float)vy;
    }
}

}  // namespace

extern "C" {

gs_status gs_generate(int32_t type, uint64_t count, float size, float mn, float mx, float G, uint64_t seed, float* pos,
                      float* vel, float* mass) {
    if (!count) return bad("The simulation must contain at least one particle!");
    if (!pos || !vel || !mass) return bad("gs_generate: output arrays are required");
    Rng r(seed);
    switch (type) {
        case GS_GEN_RANDOM: gen_random(r, count, size, mn, mx, pos, vel, mass); break;
        case GS_GEN_GALAXY: gen_galaxy(r, count, size, mn, mx, G, pos, vel, mass); break;
        case GS_GEN_GALAXY_COLLISION: gen_collision(r, count, size, mn, mx, G, pos, vel, mass); break;
        case GS_GEN_SYMMETRICAL_GALAXY_COLLISION:
            if (count & 1) return bad("gs_generate: the symmetrical preset needs an even count");
            gen_symmetric(r, count, size, mn, mx, G, pos, vel, mass);
            break;
        case GS_GEN_UNIFORM_DISK: gen_uniform_disk(r, count, size, mn, mx, pos, vel, mass); break;
        case GS_GEN_SPIRAL:  // scale 30, radius 100 confines, pitch 15 deg, amplitude 0.3, 5% dispersion
            gen_exp_disk(r, count, 30.0 * size / 100.0, size, 15.0, 0.3, 0.05, 0.0, 0.0, 0.0, 0.0, mn, mx, G, pos, vel,
                         mass);
            break;
        case GS_GEN_EXP_DISK_COLLISION: {  // two disks, scale 20, truncated at r <= 50, at (+-50, 0), v = (0, +-3)
            size_t h = count / 2;
            gen_exp_disk(r, h, 20.0, 50.0, 15.0, 0.0, 0.0, -50.0, 0.0, 0.0, -3.0, mn, mx, G, pos, vel, mass);
            gen_exp_disk(r, count - h, 20.0, 50.0, 15.0, 0.0, 0.0, 50.0, 0.0, 0.0, 3.0, mn, mx, G, pos + 2 * h,
                         vel + 2 * h, mass + h);
            break;
        }
        default: return bad("gs_generate: unknown generator type");
    }
    return GS_OK;
}

gs_status gs_read_particles(const char* path, uint64_t capacity, uint64_t* count, float* pos, float* vel, float* mass) {
    if (!path || !count) return bad("gs_read_particles: NULL argument");
    FILE* f = std::fopen(path, "r");
    if (!f) {
        gsim::set_error("Failed to open particle input file!");
        return GS_ERR_IO;
    }
    uint64_t n = 0;
    float x, y, vx, vy, m;
    while (std::fscanf(f, "%f%f%f%f%f", &x, &y, &vx, &vy, &m) == 5) {
        if (pos && vel && mass && n < capacity) {
            pos[2 * n] = x;
            pos[2 * n + 1] = y;
            vel[2 * n] = vx;
            vel[2 * n + 1] = vy;
            mass[n] = m;
        }
        ++n;
    }
    std::fclose(f);
    *count = n;
    if (!n) {
        gsim::set_error("The particle input file must contain at least one valid particle!");
        return GS_ERR_IO;
    }
    return GS_OK;
}

gs_status gs_write_particles(const char* path, uint64_t count, const float* pos, const float* vel, const float* mass) {
    if (!path || (count && (!pos || !vel || !mass))) return bad("gs_write_particles: NULL argument");
    FILE* f = std::fopen(path, "w");
    if (!f) {
        gsim::set_error("Failed to open particle output file!");
        return GS_ERR_IO;
    }
    for (uint64_t i = 0; i < count; ++i)
        std::fprintf(f, "%.7f %.7f %.7f %.7f %.7f\n", pos[2 * i], pos[2 * i + 1], vel[2 * i], vel[2 * i + 1], mass[i]);
    if (std::fclose(f) != 0) {
        gsim::set_error("Failed to write particle output file!");
        return GS_ERR_IO;
    }
    return GS_OK;
}

}  // extern "C"
