// gsim-cli -- headless command line of the GB300 path, with the flags of the reference's
// src/Main.cpp:20-48 (parsing at :167-217, headless loop at :242-321).
//
// Differences from the reference, each a fix or a consequence of having no graphics:
//   - --help prints and exits (the reference prints and carries on, src/Main.cpp:159-162);
//   - without --simulation-count the run is refused (the reference checks the wrong
//     variable, src/Main.cpp:233);
//   - the windowed mode does not exist: every run is headless (--no-graphics is accepted);
//   - --benchmark reports wall-clock time around the synchronised run, not clock() CPU time;
//   - generators take --seed (the reference seeds from time(nullptr));
//   - extra switches select the library's modes: --box=fixed|bbox, --accurate, --relative-accuracy,
//     --math=fast|reference;
//   - the window's picture can be saved instead: --image-out=file.ppm writes the final state as
//     the reference would draw it (one white pixel per particle, the start camera of the initial
//     state, src/Main.cpp:351-352, corrected for the image's aspect ratio as at :133).
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <vector>

#include "../../include/gsim.hpp"

namespace {

const char* kHelp =
    "gsim-cli (GB300 force-and-integrate path for Gravity-Sim)\n"
    "Available parameters:\n"
    "\t--log-file: The file to output all logs to.\n"
    "\t--particles-in: The input file containing the starting variables of the particles.\n"
    "\t--particles-out: The optional output file in which the variables of the particles will be written.\n"
    "\t--particle-count: The number of particles to generate.\n"
    "\t--generate-type: random | galaxy | galaxy-collision | symmetrical-galaxy-collision\n"
    "\t--generate-size: The radius of the resulting generation's size.\n"
    "\t--min-mass, --max-mass: The mass range of the generated particles.\n"
    "\t--seed: Seed of the generator (default 1).\n"
    "\t--gravitational-const: Defaulted to 1.\n"
    "\t--simulation-time: Defaulted to 1e-3.\n"
    "\t--simulation-speed: Defaulted to 1 (Barnes-Hut only).\n"
    "\t--softening-len: Defaulted to 0.2.\n"
    "\t--accuracy-parameter: Defaulted to 1 (Barnes-Hut only).\n"
    "\t--simulation-algorithm: direct-sum | barnes-hut\n"
    "\t--simulation-count: The number of simulations to run (required).\n"
    "\t--box: fixed (the reference's +-500 box, default) | bbox (per-step bounding box)\n"
    "\t--key-bits: With --box=bbox, Morton bits per axis, 1..15 (default 12: 24-bit keys; 15: 30-bit).\n"
    "\t--math: fast (default) | reference (bit-identical to the CPU restatement)\n"
    "\t--image-out: Optional PPM file with the final state drawn as the reference's window would.\n"
    "\t--image-size: WIDTHxHEIGHT of that image, defaulted to 1280x720.\n"
    "Available options:\n"
    "\t--help: Displays the current message and exits the program.\n"
    "\t--log-detailed: Outputs non-crucial logs.\n"
    "\t--no-graphics: Accepted for compatibility; every run is headless.\n"
    "\t--benchmark: Reports the wall-clock runtime of all simulations.\n"
    "\t--accurate: Barnes-Hut accurate mode (quadrupoles, safe opening radius, group walk).\n"
    "\t--relative-accuracy: With --accurate, open nodes by the relative criterion with this alpha\n"
    "\t\t(0.006 with floor 0.2: below 1e-3 RMS force error; the accuracy parameter then sets\n"
    "\t\tthe walk that estimates |a| for a step without a previous one, 1 is enough).\n"
    "\t--relative-floor: The theta floor of that criterion, defaulted to the accuracy parameter.\n";

struct Logger {
    FILE* file = nullptr;
    bool detailed = false;
    void log(const char* level, bool essential, const char* fmt, ...) {
        if (!essential && !detailed) return;
        char buf[1024];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        std::fprintf(stdout, "[%s] %s\n", level, buf);
        if (file) std::fprintf(file, "[%s] %s\n", level, buf);
    }
};

bool starts(const char* a, const char* p, const char** v) {
    size_t n = std::strlen(p);
    if (std::strncmp(a, p, n)) return false;
    *v = a + n;
    return true;
}

}  // namespace

int main(int argc, char** argv) {
    using namespace gsim_gb300;
    const char *log_file = nullptr, *in_file = nullptr, *out_file = nullptr, *image_file = nullptr;
    unsigned image_w = 1280, image_h = 720;
    uint64_t count = 0, seed = 1, max_steps = 0;
    int gen = -1, algo = -1;
    float gen_size = 0, min_mass = 0, max_mass = 0, G = 1.0f, dt = 0.001f, speed = 1.0f, eps = 0.2f, theta = 1.0f;
    bool detailed = false, benchmark = false, accurate = false, have_steps = false;
    float rel_alpha = -1.0f;  // < 0: theta criterion
    float rel_floor = 0.0f;   // 0: the accuracy parameter
    int box = GS_BOX_FIXED_500, math = GS_MATH_FAST, key_bits = 0;
    for (int i = 1; i < argc; ++i) {
        const char* a = argv[i];
        const char* v;
        if (!std::strcmp(a, "--help")) {
            std::printf("%s", kHelp);
            return 0;
        } else if (starts(a, "--log-file=", &v)) log_file = v;
        else if (starts(a, "--particles-in=", &v)) in_file = v;
        else if (starts(a, "--particles-out=", &v)) out_file = v;
        else if (starts(a, "--image-out=", &v)) image_file = v;
        else if (starts(a, "--image-size=", &v)) {
            if (std::sscanf(v, "%ux%u", &image_w, &image_h) != 2 || !image_w || !image_h) {
                std::printf("[FATAL] --image-size must be WIDTHxHEIGHT\n");
                return 1;
            }
        }
        else if (starts(a, "--particle-count=", &v)) count = std::strtoull(v, nullptr, 10);
        else if (starts(a, "--generate-type=", &v)) {
            if (!std::strcmp(v, "random")) gen = GS_GEN_RANDOM;
            else if (!std::strcmp(v, "galaxy")) gen = GS_GEN_GALAXY;
            else if (!std::strcmp(v, "galaxy-collision")) gen = GS_GEN_GALAXY_COLLISION;
            else if (!std::strcmp(v, "symmetrical-galaxy-collision")) gen = GS_GEN_SYMMETRICAL_GALAXY_COLLISION;
        } else if (starts(a, "--generate-size=", &v)) gen_size = std::strtof(v, nullptr);
        else if (starts(a, "--min-mass=", &v)) min_mass = std::strtof(v, nullptr);
        else if (starts(a, "--max-mass=", &v)) max_mass = std::strtof(v, nullptr);
        else if (starts(a, "--seed=", &v)) seed = std::strtoull(v, nullptr, 10);
        else if (starts(a, "--gravitational-const=", &v)) G = std::strtof(v, nullptr);
        else if (starts(a, "--simulation-time=", &v)) dt = std::strtof(v, nullptr);
        else if (starts(a, "--simulation-speed=", &v)) speed = std::strtof(v, nullptr);
        else if (starts(a, "--softening-len=", &v)) eps = std::strtof(v, nullptr);
        else if (starts(a, "--accuracy-parameter=", &v)) theta = std::strtof(v, nullptr);
        else if (starts(a, "--relative-accuracy=", &v)) rel_alpha = std::strtof(v, nullptr);
        else if (starts(a, "--relative-floor=", &v)) rel_floor = std::strtof(v, nullptr);
        else if (starts(a, "--simulation-algorithm=", &v)) {
            if (!std::strcmp(v, "direct-sum")) algo = GS_DIRECT_SUM;
            else if (!std::strcmp(v, "barnes-hut")) algo = GS_BARNES_HUT;
        } else if (starts(a, "--simulation-count=", &v)) {
            max_steps = std::strtoull(v, nullptr, 10);
            have_steps = true;
        } else if (starts(a, "--box=", &v)) box = !std::strcmp(v, "bbox") ? GS_BOX_BOUNDING : GS_BOX_FIXED_500;
        else if (starts(a, "--key-bits=", &v)) key_bits = (int)std::strtol(v, nullptr, 10);
        else if (starts(a, "--math=", &v)) math = !std::strcmp(v, "reference") ? GS_MATH_REFERENCE : GS_MATH_FAST;
        else if (!std::strcmp(a, "--log-detailed")) detailed = true;
        else if (!std::strcmp(a, "--no-graphics")) {
        } else if (!std::strcmp(a, "--benchmark")) benchmark = true;
        else if (!std::strcmp(a, "--accurate")) accurate = true;
    }
    Logger log;
    log.detailed = detailed;
    if (log_file) log.file = std::fopen(log_file, "w");
    if (!in_file && !(count && gen >= 0 && gen_size && min_mass && max_mass)) {
        log.log("FATAL", true, "If a particle input file is not provided, valid generation args must be provided!");
        return 1;
    }
    if (in_file && (count || gen >= 0 || gen_size || min_mass || max_mass))
        log.log("WARNING", true, "A particle input file was provided, therefore the given generation args will be ignored.");
    if (algo < 0) {
        log.log("FATAL", true, "A valid simulation algorithm must be given!");
        return 1;
    }
    if (!have_steps) {
        log.log("FATAL", true, "A valid simulation count must be given (every run is headless)!");
        return 1;
    }
    if (rel_alpha >= 0.0f && !accurate) {
        log.log("FATAL", true, "--relative-accuracy needs --accurate!");
        return 1;
    }
    uint32_t flags = accurate ? GS_FLAGS_ACCURATE : 0u;
    if (rel_alpha >= 0.0f) flags |= GS_FLAG_RELATIVE_MAC;
    try {
        const auto sa = (ParticleSystem::SimulationAlgorithm)algo;
        std::unique_ptr<ParticleSystem> system;
        if (in_file)
            system.reset(new ParticleSystem(in_file, G, dt, speed, eps, theta, sa, 0, flags));
        else
            system.reset(new ParticleSystem(count, (ParticleSystem::GenerateType)gen, gen_size, min_mass, max_mass, G,
                                            dt, speed, eps, theta, sa, seed, 0, flags));
        system->GetParams().box_mode = box;
        system->GetParams().math_mode = math;
        if (key_bits) system->GetParams().key_bits = key_bits;
        if (rel_alpha >= 0.0f) {
            system->GetParams().relative_accuracy = rel_alpha;
            system->GetParams().relative_theta_floor = rel_floor;
        }
        log.log("INFO", false, "%zu particles (%zu aligned), algorithm %s", system->GetParticleCount(),
                system->GetAlignedParticleCount(), algo == GS_BARNES_HUT ? "barnes-hut" : "direct-sum");
        std::unique_ptr<detail::SimulationBase> sim;
        if (algo == GS_DIRECT_SUM) sim.reset(new DirectSimulation(system.get()));
        else sim.reset(new BarnesHutSimulation(system.get()));
        float camera[4] = {0.0f, 0.0f, 1.0f, 1.0f};  // the start camera of the initial state
        if (image_file) {
            Check(gs_camera_start(sim->Handle(), camera));
            camera[2] = camera[3] * ((float)image_w / (float)image_h);  // size * aspect / zoom, zoom 1
        }
        auto t0 = std::chrono::steady_clock::now();
        for (uint64_t done = 0; done < max_steps;) {  // batches of at most 100 steps (src/Main.cpp:280)
            uint64_t k = max_steps - done < 100 ? max_steps - done : 100;
            sim->RunSimulations((uint32_t)k);
            done += k;
        }
        Check(gs_sync(sim->Handle(), 0));
        double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (benchmark) {  // the reference's report format (src/Main.cpp:295-310), wall clock
            double avg_ms = max_steps ? sec * 1000.0 / (double)max_steps : 0.0;
            if (sec >= 1) log.log("INFO", true, "Total simulation runtime: %.3fs", sec);
            else log.log("INFO", true, "Total simulation runtime: %.1fms", sec * 1000);
            if (avg_ms >= 5000) log.log("INFO", true, "Average runtime/simulation: %.3fs", avg_ms * 0.001);
            else if (avg_ms >= 1) log.log("INFO", true, "Average runtime/simulation: %.3fms", avg_ms);
            else log.log("INFO", true, "Average runtime/simulation: %.1fus", avg_ms * 1000);
        }
        if (out_file) system->SaveParticles(out_file);
        if (image_file) {
            std::vector<uint8_t> image((size_t)image_w * image_h);
            Check(gs_render_points(sim->Handle(), image_w, image_h, camera, image.data()));
            Check(gs_write_ppm(image_file, image_w, image_h, image.data()));
            log.log("INFO", false, "Wrote %ux%u image to %s", image_w, image_h, image_file);
        }
        sim.reset();
    } catch (const Exception& e) {
        log.log("FATAL", true, "%s (status %d)", e.what(), (int)e.GetStatus());
        return 2;
    }
    if (log.file) std::fclose(log.file);
    return 0;
}
