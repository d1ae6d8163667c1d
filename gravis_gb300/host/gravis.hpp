// gravis.hpp -- C++ host layer over libgvs.so (include/gvs.h), mirroring the
// interfaces of gravis sim-core that the GPU engine replaces:
//
//   Particles                         crates/sim-core/src/particle.rs:22-227
//   GravitySolver, NoGravity          crates/sim-core/src/gravity.rs:6-19
//   BruteForce                        crates/sim-core/src/gravity.rs:47-80
//   BarnesHut                         crates/sim-core/src/barnes_hut.rs:21-192
//   Integrator, LeapfrogKDK           crates/sim-core/src/integrator.rs:5-76
//   SphSolver, ForceIntermediates,    crates/sim-core/src/sph/solver.rs:20-212,
//   step_with_sph                     crates/sim-core/src/sph/forces.rs:12-60
//   Diagnostics, compute_diagnostics  crates/sim-core/src/diagnostics.rs:8-190
//   PlummerSphere, TwoBody,           crates/sim-core/src/scenarios/{plummer_sphere,
//   EvrardCollapse, ColdCollapse        two_body,evrard_collapse,cold_collapse}.rs
//
// Names, argument meanings and the accumulate contract are sim-core's.  Every
// numeric operation runs on the GPU through the C ABI; a failing call throws
// gravis::Error with the engine's message (the reference panics there).
#pragma once

#include <array>
#include <cstdint>
#include <iosfwd>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/gvs.h"

namespace gravis {

struct Error : std::runtime_error {
    gvs_status status;
    Error(gvs_status s, const std::string &msg) : std::runtime_error(msg), status(s) {}
};

constexpr uint8_t GAS = 4;  // particle.rs: ParticleType::Gas

// One engine context (a CUDA stream and the device-resident state) on one GPU.
class Context {
public:
    explicit Context(int device = 0);
    ~Context();
    Context(const Context &) = delete;
    Context &operator=(const Context &) = delete;
    gvs_ctx *get() const { return h_; }
    void check(gvs_status s) const;  // throws on anything but GVS_OK

private:
    gvs_ctx *h_ = nullptr;
};

// Structure-of-arrays particle store (particle.rs:22-64).
struct Particles {
    size_t count = 0;
    std::vector<double> x, y, z, vx, vy, vz, ax, ay, az, mass;
    std::vector<uint8_t> particle_type;
    std::vector<double> density, pressure, internal_energy, du_dt, smoothing_length, sound_speed, alpha_visc;

    Particles() = default;
    explicit Particles(size_t n) { resize(n); }
    void resize(size_t n);
    size_t add(double px, double py, double pz, double pvx, double pvy, double pvz, double m,
               uint8_t type = 0);                                                     // particle.rs:94-132
    size_t add_gas(double px, double py, double pz, double pvx, double pvy, double pvz, double m, double u,
                   double h);                                                         // particle.rs:136-154
    bool is_gas(size_t i) const { return particle_type[i] == GAS; }
    bool has_gas() const;
    double total_mass() const;
    void clear_accelerations();                                                       // particle.rs:173-180
    void clear_sph_rates();                                                           // particle.rs:183-187
    void shift_to_com_frame();                                                        // particle.rs:189-226
};

// Uploads p to the context's resident state (positions, velocities, masses and,
// for systems with gas, the gas fields and accelerations).
void upload(const Context &c, const Particles &p, bool with_accelerations = true);
// Downloads the resident state into p (positions, velocities, accelerations, gas fields).
void download(const Context &c, Particles &p);

// Accumulating force interface (gravity.rs:6-10): the caller zeroes a first.
class GravitySolver {
public:
    virtual ~GravitySolver() = default;
    virtual void compute_accelerations(Particles &p) const = 0;
    virtual int algo() const = 0;
    virtual int precision() const { return GVS_PREC_FP64_EXACT; }
    virtual double softening() const { return 0.0; }
    virtual double theta() const { return 0.5; }
};

class NoGravity : public GravitySolver {  // gravity.rs:13-19
public:
    void compute_accelerations(Particles &) const override {}
    int algo() const override { return GVS_ALGO_NONE; }
};

class BruteForce : public GravitySolver {  // gravity.rs:47-80 (FP64_EXACT: bit-identical)
public:
    BruteForce(Context &c, double softening, int precision = GVS_PREC_FP64_EXACT)
        : c_(c), eps_(softening), prec_(precision) {}
    void compute_accelerations(Particles &p) const override;
    int algo() const override { return GVS_ALGO_DIRECT; }
    int precision() const override { return prec_; }
    double softening() const override { return eps_; }

private:
    Context &c_;
    double eps_;
    int prec_;
};

class BarnesHut : public GravitySolver {  // barnes_hut.rs:139-192
public:
    BarnesHut(Context &c, double softening, double theta, int precision = GVS_PREC_FP64)
        : c_(c), eps_(softening), theta_(theta), prec_(precision) {}
    void compute_accelerations(Particles &p) const override;
    int algo() const override { return GVS_ALGO_BH; }
    int precision() const override { return prec_; }
    double softening() const override { return eps_; }
    double theta() const override { return theta_; }

private:
    Context &c_;
    double eps_, theta_;
    int prec_;
};

class Integrator {  // integrator.rs:5-8
public:
    virtual ~Integrator() = default;
    virtual void step(Particles &p, const GravitySolver &gravity, double dt) const = 0;
};

// integrator.rs:42-76: kick, drift, clear, forces, kick -- one GPU call per step.
class LeapfrogKDK : public Integrator {
public:
    explicit LeapfrogKDK(Context &c) : c_(c) {}
    void step(Particles &p, const GravitySolver &gravity, double dt) const override;

private:
    Context &c_;
};

struct ForceIntermediates {  // forces.rs:44-60
    std::vector<double> div_v, max_mu, dalpha_dt, omega;
};

class SphSolver {  // solver.rs:20-131
public:
    explicit SphSolver(Context &c);
    gvs_sph_params params;  // SphSolver::new + ForceParams::default; precision FP64_EXACT
    // a and du/dt accumulate into p (call after gravity, as the reference does)
    ForceIntermediates compute(Particles &p);
    double compute_timestep(const Particles &p) const;  // for the state of the last compute
    Context &context() const { return c_; }

private:
    Context &c_;
};

// step_with_sph (solver.rs:145-212); returns the next timestep.
double step_with_sph(Particles &p, const GravitySolver &gravity, SphSolver &sph, double dt);

// diagnostics.rs:8-190
struct Diagnostics {
    double kinetic_energy = 0, potential_energy = 0, thermal_energy = 0, total_energy = 0;
    std::array<double, 3> momentum{}, angular_momentum{}, center_of_mass{}, center_of_mass_velocity{};
    double virial_ratio = 0, time = 0;
    uint64_t step = 0;
    double momentum_magnitude() const;
    double angular_momentum_magnitude() const;
    double com_drift() const;
    static const char *csv_header();
    std::string to_csv_row() const;  // Rust's {:.6e} / {:.10e} / {:.6} formats
};
Diagnostics from_c(const gvs_diag &d, double time, uint64_t step);
// diagnostics::compute (with_potential) / compute_fast on the resident state
Diagnostics compute_diagnostics(const Context &c, double softening, double time, uint64_t step,
                                bool with_potential = true);

// Scenarios (scenario.rs:8-20): generate() plus the suggested dt and softening.
struct PlummerSphere {  // plummer_sphere.rs:79-153
    size_t n = 1000;
    double scale_radius = 1.0, total_mass = 1.0;
    uint64_t seed = 42;
    const char *name() const { return "Plummer Sphere"; }
    Particles generate() const;
    double suggested_dt() const;
    double suggested_softening() const;
};

struct TwoBody {  // two_body.rs:17-106
    double mass_ratio = 0.5, eccentricity = 0.5, semi_major_axis = 1.0;
    const char *name() const { return "Two-Body Kepler Orbit"; }
    double period() const;
    Particles generate() const;
    double suggested_dt() const { return period() / 10000.0; }
    double suggested_softening() const { return semi_major_axis * (1.0 - eccentricity) * 0.001; }
};

struct EvrardCollapse {  // evrard_collapse.rs:15-71
    size_t n_particles = 5000;
    double total_mass = 1.0, radius = 1.0, u_0 = 0.05;
    uint64_t seed = 42;
    const char *name() const { return "Evrard Collapse"; }
    Particles generate() const;
    double suggested_dt() const;
    double suggested_softening() const;
};

struct ColdCollapse {  // cold_collapse.rs:26-123
    size_t n = 5000;
    double radius = 1.0, total_mass = 1.0;
    uint64_t seed = 42;
    bool sph = false;
    const char *name() const { return sph ? "Cold Collapse (Gas)" : "Cold Collapse"; }
    Particles generate() const;
    double suggested_dt() const;
    double suggested_softening() const;
};

// Snapshot (crates/sim-core/src/snapshot.rs:1-170): the NBODY003 binary format --
// magic, time, step, softening, dt, count, then x y z vx vy vz mass (f64 each),
// particle_type (u8), internal_energy, smoothing_length, density (f64), all
// little-endian.  read_from also accepts NBODY001/002.  Accelerations are not
// stored: initialize() recomputes them before stepping, as the reference requires.
struct Snapshot {
    double time = 0.0;
    uint64_t step = 0;
    double softening = 0.0, dt = 0.0;
    Particles particles;
    static Snapshot capture(const Particles &p, double time, uint64_t step, double softening, double dt);
    void write_to(std::ostream &w) const;
    static Snapshot read_from(std::istream &r);
    void initialize(const GravitySolver &gravity);
};

// Rust's `{:.Ne}` formatting of an f64 (exponent without sign padding or '+').
std::string rust_exp(double v, int prec);

}  // namespace gravis
