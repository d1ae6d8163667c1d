// headless.cpp -- gvs_headless, the GPU counterpart of gravis's headless runner
// (crates/headless/src/main.rs): the same flags, defaults, step loop, dt growth
// cap, diagnostics cadence and diagnostics CSV, with the particle state kept on
// the GPU between diagnostics (the runner reads it back only for diagnostics,
// which are themselves computed on the GPU).
//
// Extra flags (no reference counterpart): --precision fp64-exact|fp64|fp32|mixed
// for the force paths, --device N, and --restart SNAPSHOT (continue from an
// NBODY snapshot: its time, step, softening and dt; accelerations recomputed,
// as Snapshot::initialize does).  Scenarios: plummer, two-body (kepler),
// cold-collapse, cold-collapse-gas, evrard-collapse; the others are outside the
// engine's scope.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <memory>
#include <string>

#include "gravis.hpp"

using namespace gravis;

namespace {

struct Cli {
    std::string scenario = "plummer";
    long long particles = -1;
    unsigned long long steps = 1000;
    double dt = -1.0, softening = -1.0;
    unsigned long long diag_interval = 100;
    std::string diag_csv;
    unsigned long long seed = 42;
    double eccentricity = 0.5;
    std::string algorithm = "brute-force";
    double theta = 0.5;
    std::string precision = "fp64-exact";
    int device = 0;
    unsigned long long snapshot_interval = 0;
    std::string snapshot_dir = "artifacts/snapshots";
    std::string restart;
};

[[noreturn]] void die(const std::string &msg) {
    std::fprintf(stderr, "Error: %s\n", msg.c_str());
    std::exit(1);
}

void usage() {
    std::printf(
        "gvs_headless: headless N-body runner on one GB300 (the counterpart of nbody-headless)\n"
        "  -s, --scenario NAME        plummer | two-body | kepler | cold-collapse | cold-collapse-gas |\n"
        "                             evrard-collapse (default plummer)\n"
        "  -n, --particles N          particle count (scenario default otherwise)\n"
        "      --steps N              timesteps (default 1000)\n"
        "      --dt DT                timestep (scenario suggestion otherwise)\n"
        "      --softening EPS        softening (scenario suggestion otherwise)\n"
        "      --diag-interval N      diagnostics every N steps, 0 = off (default 100)\n"
        "      --diag-csv PATH        write the diagnostics CSV\n"
        "      --seed N               RNG seed (default 42)\n"
        "      --eccentricity E       two-body eccentricity in [0, 1) (default 0.5)\n"
        "      --algorithm NAME       brute-force | barnes-hut (default brute-force)\n"
        "      --theta T              Barnes-Hut opening angle (default 0.5)\n"
        "      --precision P          fp64-exact | fp64 | fp32 | mixed (default fp64-exact)\n"
        "      --device N             CUDA device (default 0)\n"
        "      --snapshot-interval N  write an NBODY003 snapshot every N steps, 0 = off (default 0)\n"
        "      --snapshot-dir DIR     snapshot directory (default artifacts/snapshots)\n"
        "      --restart PATH         continue from a snapshot (its time, step, softening, dt)\n");
}

Cli parse(int argc, char **argv) {
    Cli c;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto val = [&]() -> std::string {
            if (i + 1 >= argc) die("missing value for " + a);
            return argv[++i];
        };
        if (a == "-h" || a == "--help") { usage(); std::exit(0); }
        else if (a == "-s" || a == "--scenario") c.scenario = val();
        else if (a == "-n" || a == "--particles") c.particles = std::atoll(val().c_str());
        else if (a == "--steps") c.steps = std::strtoull(val().c_str(), nullptr, 10);
        else if (a == "--dt") c.dt = std::atof(val().c_str());
        else if (a == "--softening") c.softening = std::atof(val().c_str());
        else if (a == "--diag-interval") c.diag_interval = std::strtoull(val().c_str(), nullptr, 10);
        else if (a == "--diag-csv") c.diag_csv = val();
        else if (a == "--seed") c.seed = std::strtoull(val().c_str(), nullptr, 10);
        else if (a == "--eccentricity") c.eccentricity = std::atof(val().c_str());
        else if (a == "--algorithm") c.algorithm = val();
        else if (a == "--theta") c.theta = std::atof(val().c_str());
        else if (a == "--precision") c.precision = val();
        else if (a == "--device") c.device = std::atoi(val().c_str());
        else if (a == "--snapshot-interval") c.snapshot_interval = std::strtoull(val().c_str(), nullptr, 10);
        else if (a == "--snapshot-dir") c.snapshot_dir = val();
        else if (a == "--restart") c.restart = val();
        else die("unknown argument " + a);
    }
    // the reference's input checks (main.rs:66-95)
    if (c.particles == 0) die("--particles must be > 0");
    if (c.eccentricity < 0.0 || c.eccentricity >= 1.0)
        die("--eccentricity must be in [0, 1), got " + std::to_string(c.eccentricity));
    if (c.dt != -1.0 && !(c.dt > 0.0)) die("--dt must be positive, got " + std::to_string(c.dt));
    if (c.softening != -1.0 && c.softening < 0.0)
        die("--softening must be non-negative, got " + std::to_string(c.softening));
    if (c.algorithm != "brute-force" && c.algorithm != "barnes-hut")
        die("--algorithm must be brute-force or barnes-hut");
    return c;
}

int precision_of(const std::string &p) {
    if (p == "fp64-exact") return GVS_PREC_FP64_EXACT;
    if (p == "fp64") return GVS_PREC_FP64;
    if (p == "fp32") return GVS_PREC_FP32;
    if (p == "mixed") return GVS_PREC_MIXED;
    die("--precision must be fp64-exact, fp64, fp32 or mixed");
}

struct Built {
    Particles particles;
    double dt, softening;
    std::string name;
};

// scenario_builder::build (crates/sim-core/src/scenario_builder.rs:37-96)
Built build(const Cli &c) {
    Built b;
    if (c.scenario == "plummer") {
        PlummerSphere s;
        s.n = c.particles > 0 ? (size_t)c.particles : 1000;
        s.seed = c.seed;
        b = {s.generate(), s.suggested_dt(), s.suggested_softening(), s.name()};
    } else if (c.scenario == "two-body" || c.scenario == "kepler") {
        TwoBody s;
        s.eccentricity = c.eccentricity;
        b = {s.generate(), s.suggested_dt(), s.suggested_softening(), s.name()};
    } else if (c.scenario == "cold-collapse" || c.scenario == "cold-collapse-gas") {
        ColdCollapse s;
        s.n = c.particles > 0 ? (size_t)c.particles : 5000;
        s.sph = c.scenario == "cold-collapse-gas";
        s.seed = c.seed;
        b = {s.generate(), s.suggested_dt(), s.suggested_softening(), s.name()};
    } else if (c.scenario == "evrard-collapse") {
        EvrardCollapse s;
        s.n_particles = c.particles > 0 ? (size_t)c.particles : 5000;
        s.seed = c.seed;
        b = {s.generate(), s.suggested_dt(), s.suggested_softening(), s.name()};
    } else {
        die("Unknown scenario: " + c.scenario +
            ". Available here: plummer, two-body, cold-collapse, cold-collapse-gas, evrard-collapse");
    }
    if (c.dt > 0.0) b.dt = c.dt;
    if (c.softening >= 0.0) b.softening = c.softening;
    return b;
}

void write_snapshot(const Context &ctx, Particles &p, const std::string &dir, double time, unsigned long long step,
                    double softening, double dt) {
    download(ctx, p);
    char name[64];
    std::snprintf(name, sizeof name, "/snap_%08llu.bin", step);
    std::ofstream f(dir + name, std::ios::binary);
    if (!f) die("Failed to create snapshot " + dir + name);
    Snapshot::capture(p, time, step, softening, dt).write_to(f);
}

}  // namespace

int main(int argc, char **argv) {
    const Cli cli = parse(argc, argv);
    try {
        Built built;
        double t_start = 0.0;
        unsigned long long step0 = 0;
        if (!cli.restart.empty()) {
            std::ifstream f(cli.restart, std::ios::binary);
            if (!f) die("Failed to open snapshot " + cli.restart);
            Snapshot snap = Snapshot::read_from(f);
            built = {snap.particles, snap.dt, snap.softening, "restart of " + cli.restart};
            t_start = snap.time;
            step0 = snap.step;
            if (cli.dt > 0.0) built.dt = cli.dt;
            if (cli.softening >= 0.0) built.softening = cli.softening;
        } else {
            built = build(cli);
        }
        Particles &p = built.particles;
        const double softening = built.softening;
        const int prec = precision_of(cli.precision);
        const bool use_sph = p.has_gas();
        const int algo = cli.algorithm == "barnes-hut" ? GVS_ALGO_BH : GVS_ALGO_DIRECT;

        Context ctx(cli.device);
        SphSolver sph(ctx);
        std::fprintf(stderr, "Scenario:   %s\nParticles:  %zu\nAlgorithm:  %s\n", built.name.c_str(), p.count,
                     cli.algorithm.c_str());
        if (algo == GVS_ALGO_BH) std::fprintf(stderr, "Theta:      %g\n", cli.theta);
        std::fprintf(stderr, "Precision:  %s\nSteps:      %llu\ndt:         %.6e\nSoftening:  %.6e\n\n",
                     cli.precision.c_str(), cli.steps, built.dt, softening);

        std::unique_ptr<std::ofstream> csv;
        if (!cli.diag_csv.empty()) {
            csv.reset(new std::ofstream(cli.diag_csv));
            if (!*csv) die("Failed to create diagnostics CSV " + cli.diag_csv);
            *csv << Diagnostics::csv_header() << "\n";
        }

        if (cli.snapshot_interval > 0) std::filesystem::create_directories(cli.snapshot_dir);
        // initial accelerations (main.rs:150-155): clear, gravity, SPH
        upload(ctx, p, false);
        ctx.check(gvs_compute_forces(ctx.get(), algo, prec, softening, cli.theta));
        if (use_sph) ctx.check(gvs_sph_compute(ctx.get(), &sph.params, nullptr, nullptr, nullptr, nullptr));

        const bool full = cli.diag_interval > 0 || csv;
        const Diagnostics d0 = compute_diagnostics(ctx, softening, t_start, step0, full);
        std::fprintf(stderr, "Initial:    E=%.10e  2K/|U|=%.4f\n", d0.total_energy, d0.virial_ratio);
        if (csv) *csv << d0.to_csv_row() << "\n";

        const auto t0 = std::chrono::steady_clock::now();
        double sim_time = t_start, current_dt = built.dt;
        unsigned long long step = step0;
        const unsigned long long last = step0 + cli.steps;
        while (step < last) {
            if (use_sph) {
                // step_with_sph, dt_next capped at 1.5x (main.rs:181-187)
                double dt_next = 0.0;
                ctx.check(gvs_sph_step(ctx.get(), &sph.params, algo, prec, softening, cli.theta, current_dt,
                                       &dt_next));
                sim_time += current_dt;
                current_dt = std::fmin(dt_next, current_dt * 1.5);
                ++step;
            } else {
                // a fixed dt: run up to the next diagnostics step in one device-resident call
                unsigned long long k = last - step;
                if (cli.diag_interval > 0) k = std::min(k, cli.diag_interval - step % cli.diag_interval);
                if (cli.snapshot_interval > 0)
                    k = std::min(k, cli.snapshot_interval - step % cli.snapshot_interval);
                ctx.check(gvs_kdk_steps(ctx.get(), algo, prec, softening, cli.theta, current_dt, (long long)k));
                for (unsigned long long s = 0; s < k; ++s) sim_time += current_dt;  // same sum as step by step
                step += k;
            }
            if (cli.diag_interval > 0 && step % cli.diag_interval == 0) {
                const Diagnostics d = compute_diagnostics(ctx, softening, sim_time, step);
                const double de = (d.total_energy - d0.total_energy) / std::fabs(d0.total_energy);
                std::fprintf(stderr, "Step %8llu  t=%.4e  E=%.10e  dE/E=%+.4e  2K/|U|=%.4f\n", step, sim_time,
                             d.total_energy, de, d.virial_ratio);
                if (csv) *csv << d.to_csv_row() << "\n";
            }
            if (cli.snapshot_interval > 0 && step % cli.snapshot_interval == 0)
                write_snapshot(ctx, p, cli.snapshot_dir, sim_time, step, softening, current_dt);
        }
        ctx.check(gvs_sync(ctx.get()));
        const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();

        const Diagnostics fd = compute_diagnostics(ctx, softening, sim_time, last, full);
        const double de = (fd.total_energy - d0.total_energy) / std::fabs(d0.total_energy);
        std::fprintf(stderr, "\n=== Final ===\nSim time:   %.6e\nWall time:  %.3fs\nSteps/sec:  %.0f\n", sim_time, wall,
                     (double)cli.steps / wall);
        std::fprintf(stderr, "Energy:     %.10e  (dE/E = %+.6e)\nMomentum:   %.6e\nAng. Mom:   %.6e\n",
                     fd.total_energy, de, fd.momentum_magnitude(), fd.angular_momentum_magnitude());
        std::fprintf(stderr, "COM drift:  %.6e\nVirial:     %.4f\n", fd.com_drift(), fd.virial_ratio);
        const bool already = cli.diag_interval > 0 && last % cli.diag_interval == 0;
        if (csv && !already) *csv << fd.to_csv_row() << "\n";
        std::printf("{\"steps\": %llu, \"wall_s\": %.6f, \"particle_steps_per_s\": %.6e, \"dE_over_E\": %.6e}\n",
                    cli.steps, wall, (double)p.count * (double)cli.steps / wall, de);
    } catch (const Error &e) {
        die(e.what());
    }
    return 0;
}
