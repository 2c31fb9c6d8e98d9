// Headless ports of the reference applications' simulation loops on
// GB_Lattice (the GB300 engine).  The Qt/VTK/OpenGL viewers of the reference
// cannot run here (no graphics stack); their per-frame loop is kept and the
// rendering is replaced by optional .vti / PNG files.
//
//   lgca_headless --case pipe       apps/pipe:      FHP-III, Re 80, Ma 0.3, r 10, 5 steps/frame,
//                                   forcing controller (apps/pipe/pipe_viewer.cpp:100-184)
//   lgca_headless --case karman     apps/karman:    FHP-III, Re 80, Ma 0.3, r 20, 5 steps/frame
//   lgca_headless --case diffusion  apps/diffusion: FHP-III, Re 200, r 1, reflecting walls
//   lgca_headless --case single     apps/single:    FHP-III, "collision" lattice, two particles
//   lgca_headless --case box|periodic  apps/box and apps/periodic (CLI loop: step, then force,
//                                   apps/box/main.cpp:230-312)
//
// Common options: --frames N (viewer cases) or --steps N (box/periodic),
// --model HPP|FHP_I|FHP_II|FHP_III, --Re, --Ma, --r, --seed, --out DIR,
// --format none|vti|png, --every N, --dump FILE (the final state, one byte
// per cell, bit d = channel d).  Prints the reference's messages and a final
// JSON line with the run's summary; for the pipe and karman cases it carries
// the forcing controller's trace, one entry per frame: the bits of the mean
// x velocity (float), the forcing applied (-1: none) and the particles
// reverted.
#include "lgca/gb_lattice.h"
#include "lgca/io.h"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

using namespace lgca_gb300;

struct Options {
    std::string test_case = "pipe";
    std::string model = "FHP_III";
    std::string out = "./";
    std::string format = "none";
    std::string dump;
    float Re = -1, Ma = -1;
    int r = -1;
    int frames = 20;
    int steps = 100;
    int every = 1;
    int write_steps = 10, bf_steps = 1;
    float bf_intensity = 0.0f;
    unsigned long long seed = 0;
};

static void usage()
{
    std::fprintf(stderr,
                 "usage: lgca_headless --case pipe|karman|diffusion|single|box|periodic "
                 "[--frames N] [--steps N] [--model M] [--Re x] [--Ma x] [--r n] [--seed s] "
                 "[--out dir] [--format none|vti|png] [--every N] [--write-steps N] "
                 "[--bf-steps N] [--bf-intensity x] [--dump file]\n");
    std::exit(2);
}

static Options parse(int argc, char **argv)
{
    Options o;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        auto val = [&]() -> std::string {
            if (i + 1 >= argc) usage();
            return argv[++i];
        };
        if (a == "--case") o.test_case = val();
        else if (a == "--model") o.model = val();
        else if (a == "--out") o.out = val();
        else if (a == "--format") o.format = val();
        else if (a == "--Re") o.Re = std::stof(val());
        else if (a == "--Ma") o.Ma = std::stof(val());
        else if (a == "--r") o.r = std::stoi(val());
        else if (a == "--frames") o.frames = std::stoi(val());
        else if (a == "--steps") o.steps = std::stoi(val());
        else if (a == "--every") o.every = std::stoi(val());
        else if (a == "--write-steps") o.write_steps = std::stoi(val());
        else if (a == "--bf-steps") o.bf_steps = std::stoi(val());
        else if (a == "--bf-intensity") o.bf_intensity = std::stof(val());
        else if (a == "--seed") o.seed = std::stoull(val());
        else if (a == "--dump") o.dump = val();
        else usage();
    }
    if (!o.out.empty() && o.out.back() != '/') o.out += '/';
    return o;
}

// defaults of the reference viewers (apps/*/..._viewer.h)
static void viewer_defaults(Options &o, int &pp_interval)
{
    float Re = 80, Ma = 0.3f;
    int r = 10;
    pp_interval = 5;
    if (o.test_case == "karman") { r = 20; }
    else if (o.test_case == "diffusion") { Re = 200; Ma = 0.2f; r = 1; pp_interval = 1; }
    else if (o.test_case == "single") { Re = 80; Ma = 0.2f; r = 1; pp_interval = 1; }
    if (o.Re < 0) o.Re = Re;
    if (o.Ma < 0) o.Ma = Ma;
    if (o.r < 0) o.r = r;
}

template <class L> static void output(L &lat, const Options &o, size_t step)
{
    if (o.format == "vti") {
        VtiWriter<L> io(&lat, "Cell density");
        io.write(step, o.out);
    } else if (o.format == "png") {
        const std::string path = o.out + "res_" + std::to_string(step) + ".png";
        write_png_field(path, (int)lat.coarse_dim_x(), (int)lat.coarse_dim_y(), lat.mean_density(),
                        0.0f, (float)L::NUM_DIR * 0.5f);
    }
}

template <class L> static void dump_state(L &lat, const Options &o)
{
    if (o.dump.empty()) return;
    FILE *f = std::fopen(o.dump.c_str(), "wb");
    if (!f || std::fwrite(lat.node_state(), 1, lat.num_cells(), f) != lat.num_cells()) {
        std::fprintf(stderr, "cannot write %s\n", o.dump.c_str());
        std::exit(1);
    }
    std::fclose(f);
}

template <Model M> static int run_viewer(Options o)
{
    int pp = 5;
    viewer_defaults(o, pp);
    const std::string tc = o.test_case == "single" ? "collision" : o.test_case;
    GB_Lattice<M> lat(tc, o.Re, o.Ma, o.r, o.seed);
    if (o.test_case == "pipe") lat.apply_bc_pipe();
    else if (o.test_case == "karman") lat.apply_bc_karman_vortex_street();
    else if (o.test_case == "diffusion") lat.apply_bc_reflecting("back");
    else lat.apply_bc_pipe();
    if (o.test_case == "diffusion") lat.init_diffusion();
    else if (o.test_case == "single") lat.init_single_collision();
    else lat.init_random();
    const size_t n0 = lat.get_n_particles();
    lat.copy_data_to_output_buffer();
    lat.post_process();
    int forcing = (int)lat.get_initial_forcing();
    lat.setup_parallel();
    const bool controller = o.test_case == "pipe" || o.test_case == "karman";
    size_t steps = 0;
    double sim_time = 0;
    std::vector<Real> u{0, 0};
    std::string trace;
    for (int frame = 0; frame < o.frames; ++frame) {
        if (controller) {  // apps/pipe/pipe_viewer.cpp:107-125
            u = lat.get_mean_velocity();
            int applied = -1;
            if (u[0] < lat.u()) {
                if (u[0] > 0.9 * lat.u()) forcing = (int)lat.get_equilibrium_forcing();
                lat.apply_body_force(forcing);
                applied = forcing;
            }
            uint32_t bits;
            std::memcpy(&bits, &u[0], sizeof(bits));
            char e[96];
            std::snprintf(e, sizeof(e), "%s[%u, %d, %llu]", trace.empty() ? "" : ", ", bits, applied,
                          applied >= 0 ? (unsigned long long)lat.last_reverted() : 0ull);
            trace += e;
        }
        const auto t0 = std::chrono::steady_clock::now();
        for (int s = 0; s < pp; ++s) {
            lat.collide_and_propagate(o.test_case == "karman" ? (steps % 2) : false);
            ++steps;
        }
        lat.copy_data_to_output_buffer();  // synchronises with the GPU
        sim_time += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        lat.post_process();
        if (o.format != "none" && frame % o.every == 0) output(lat, o, steps);
    }
    const size_t n1 = lat.get_n_particles();
    if (n1 == n0)
        std::fprintf(stderr, "Error check PASSED: There is no difference in the number of particles.\n");
    else
        std::fprintf(stderr, "Error check FAILED: There is a difference in the number of particles of %lld.\n",
                     (long long)n1 - (long long)n0);
    u = lat.get_mean_velocity();
    dump_state(lat, o);
    const double mnups = sim_time > 0 ? lat.num_cells() * (double)steps / (sim_time * 1e6) : 0.0;
    std::printf("{\"case\": \"%s\", \"dims\": [%u, %u], \"steps\": %zu, \"particles_start\": %zu, "
                "\"particles_end\": %zu, \"mean_velocity\": [%.6g, %.6g], \"mnups\": %.1f, "
                "\"forcing\": %d, \"trace\": [%s]}\n",
                o.test_case.c_str(), lat.dim_x(), lat.dim_y(), steps, n0, n1, u[0], u[1], mnups,
                forcing, trace.c_str());
    return n1 == n0 ? 0 : 1;
}

// apps/box/main.cpp:97-347 (same file as apps/periodic/main.cpp)
template <Model M> static int run_cli(Options o)
{
    if (o.Re < 0) o.Re = 128;
    if (o.Ma < 0) o.Ma = 0.3f;
    if (o.r < 0) o.r = 4;
    GB_Lattice<M> lat(o.test_case, o.Re, o.Ma, o.r, o.seed);
    if (o.test_case == "box") lat.apply_bc_reflecting("back");
    else lat.apply_bc_periodic();
    lat.init_random();
    const size_t n0 = lat.get_n_particles();
    int forcing = (int)(o.bf_intensity * lat.get_initial_forcing());
    std::vector<Real> u{0, 0};
    auto t_start = std::chrono::steady_clock::now();
    const auto t_all = t_start;
    for (int step = 0; step <= o.steps; ++step) {
        if (step % o.bf_steps == 0 || step % o.write_steps == 0) {
            lat.copy_data_to_output_buffer();
            lat.post_process();
            u = lat.get_mean_velocity();
        }
        if (step % o.write_steps == 0) {
            std::printf("\nExecuting step %d...\n", step);
            std::printf("Current mean velocity: (%6.4f, %6.4f)\n", u[0], u[1]);
            if (step > 0) {
                const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
                std::printf("Current MNUPS: %d\n", (int)((lat.dim_x() * lat.dim_y() * (double)o.write_steps) / (dt * 1.0e06)));
            }
            if (o.format != "none") output(lat, o, step);
            t_start = std::chrono::steady_clock::now();
        }
        lat.collide_and_propagate(step);
        if (o.bf_intensity > 1.0e-06 && u[0] < lat.u() && lat.bf_dir() == 'x') {
            if (u[0] > 0.9 * lat.u()) forcing = (int)lat.get_equilibrium_forcing();
            lat.apply_body_force(forcing);
        }
    }
    const size_t n1 = lat.get_n_particles();
    dump_state(lat, o);
    const double total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_all).count();
    if (n1 == n0) std::printf("Error check PASSED: There is no difference in the number of particles.\n");
    else std::printf("Error check FAILED: There is a difference in the number of particles of %lld.\n",
                     (long long)n1 - (long long)n0);
    std::printf("Total elapsed time: %e s for %d simulation steps.\n", total, o.steps);
    std::printf("Average MNUPS: %d\n", (int)((lat.dim_x() * lat.dim_y() * (double)o.steps) / (total * 1.0e06)));
    std::printf("{\"case\": \"%s\", \"dims\": [%u, %u], \"steps\": %d, \"particles_start\": %zu, "
                "\"particles_end\": %zu, \"mean_velocity\": [%.6g, %.6g]}\n",
                o.test_case.c_str(), lat.dim_x(), lat.dim_y(), o.steps + 1, n0, n1, u[0], u[1]);
    return n1 == n0 ? 0 : 1;
}

template <Model M> static int run(const Options &o)
{
    if (o.test_case == "box" || o.test_case == "periodic") return run_cli<M>(o);
    if (o.test_case == "pipe" || o.test_case == "karman" || o.test_case == "diffusion" ||
        o.test_case == "single")
        return run_viewer<M>(o);
    usage();
    return 2;
}

int main(int argc, char **argv)
{
    const Options o = parse(argc, argv);
    if (o.model == "HPP") return run<Model::HPP>(o);
    if (o.model == "FHP_I") return run<Model::FHP_I>(o);
    if (o.model == "FHP_II") return run<Model::FHP_II>(o);
    if (o.model == "FHP_III") return run<Model::FHP_III>(o);
    usage();
    return 2;
}
