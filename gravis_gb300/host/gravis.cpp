// gravis.cpp -- the C++ host layer over libgvs.so (see gravis.hpp).
#include "gravis.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <istream>
#include <ostream>

namespace gravis {

namespace {
std::string last_error(gvs_ctx *h) {
    char buf[512] = {0};
    gvs_last_error(h, buf, sizeof buf);
    return buf;
}
void ck(gvs_status s, gvs_ctx *h) {
    if (s != GVS_OK) throw Error(s, last_error(h));
}
}  // namespace

Context::Context(int device) {
    const gvs_status s = gvs_create(&h_, device);
    if (s != GVS_OK) throw Error(s, last_error(nullptr));
}

Context::~Context() {
    if (h_) gvs_destroy(h_);
}

void Context::check(gvs_status s) const { ck(s, h_); }

// ---- Particles -----------------------------------------------------------------------
void Particles::resize(size_t n) {
    count = n;
    for (auto *v : {&x, &y, &z, &vx, &vy, &vz, &ax, &ay, &az, &mass, &density, &pressure, &internal_energy, &du_dt,
                    &smoothing_length, &sound_speed, &alpha_visc})
        v->assign(n, 0.0);
    particle_type.assign(n, 0);
}

size_t Particles::add(double px, double py, double pz, double pvx, double pvy, double pvz, double m, uint8_t type) {
    const size_t i = count;
    for (auto *v : {&x, &y, &z, &vx, &vy, &vz, &ax, &ay, &az, &mass, &density, &pressure, &internal_energy, &du_dt,
                    &smoothing_length, &sound_speed, &alpha_visc})
        v->push_back(0.0);
    particle_type.push_back(type);
    x[i] = px; y[i] = py; z[i] = pz;
    vx[i] = pvx; vy[i] = pvy; vz[i] = pvz;
    mass[i] = m;
    ++count;
    return i;
}

size_t Particles::add_gas(double px, double py, double pz, double pvx, double pvy, double pvz, double m, double u,
                          double h) {
    const size_t i = add(px, py, pz, pvx, pvy, pvz, m, GAS);
    internal_energy[i] = u;
    smoothing_length[i] = h;
    alpha_visc[i] = 1.0;
    return i;
}

bool Particles::has_gas() const {
    for (uint8_t t : particle_type)
        if (t == GAS) return true;
    return false;
}

double Particles::total_mass() const {
    double s = 0.0;
    for (double m : mass) s += m;
    return s;
}

void Particles::clear_accelerations() {
    std::fill(ax.begin(), ax.end(), 0.0);
    std::fill(ay.begin(), ay.end(), 0.0);
    std::fill(az.begin(), az.end(), 0.0);
}

void Particles::clear_sph_rates() { std::fill(du_dt.begin(), du_dt.end(), 0.0); }

void Particles::shift_to_com_frame() {
    const double mt = total_mass();
    if (mt == 0.0) return;
    double c[6] = {0, 0, 0, 0, 0, 0};
    for (size_t i = 0; i < count; ++i) {
        c[0] += mass[i] * x[i]; c[1] += mass[i] * y[i]; c[2] += mass[i] * z[i];
        c[3] += mass[i] * vx[i]; c[4] += mass[i] * vy[i]; c[5] += mass[i] * vz[i];
    }
    for (double &v : c) v /= mt;
    for (size_t i = 0; i < count; ++i) {
        x[i] -= c[0]; y[i] -= c[1]; z[i] -= c[2];
        vx[i] -= c[3]; vy[i] -= c[4]; vz[i] -= c[5];
    }
}

void upload(const Context &c, const Particles &p, bool with_accelerations) {
    const bool gas = p.has_gas();
    c.check(gvs_set_state(c.get(), p.count, p.x.data(), p.y.data(), p.z.data(), p.vx.data(), p.vy.data(),
                          p.vz.data(), p.mass.data(), gas ? p.particle_type.data() : nullptr,
                          gas ? p.internal_energy.data() : nullptr, gas ? p.smoothing_length.data() : nullptr,
                          gas ? p.alpha_visc.data() : nullptr));
    if (with_accelerations) c.check(gvs_set_accelerations(c.get(), p.ax.data(), p.ay.data(), p.az.data()));
    if (gas)
        c.check(gvs_set_gas(c.get(), p.density.data(), p.pressure.data(), p.internal_energy.data(), p.du_dt.data(),
                            p.smoothing_length.data(), p.sound_speed.data(), p.alpha_visc.data()));
}

void download(const Context &c, Particles &p) {
    c.check(gvs_get_state(c.get(), p.x.data(), p.y.data(), p.z.data(), p.vx.data(), p.vy.data(), p.vz.data(),
                          p.ax.data(), p.ay.data(), p.az.data()));
    if (p.has_gas())
        c.check(gvs_get_gas(c.get(), p.density.data(), p.pressure.data(), p.internal_energy.data(), p.du_dt.data(),
                            p.smoothing_length.data(), p.sound_speed.data(), p.alpha_visc.data()));
}

// ---- gravity -------------------------------------------------------------------------
void BruteForce::compute_accelerations(Particles &p) const {
    c_.check(gvs_gravity_direct(c_.get(), p.count, p.x.data(), p.y.data(), p.z.data(), p.mass.data(), eps_, prec_,
                                p.ax.data(), p.ay.data(), p.az.data()));
}

void BarnesHut::compute_accelerations(Particles &p) const {
    c_.check(gvs_gravity_bh(c_.get(), p.count, p.x.data(), p.y.data(), p.z.data(), p.mass.data(), eps_, theta_,
                            prec_, p.ax.data(), p.ay.data(), p.az.data()));
}

void LeapfrogKDK::step(Particles &p, const GravitySolver &g, double dt) const {
    c_.check(gvs_kdk_step_host(c_.get(), p.count, p.x.data(), p.y.data(), p.z.data(), p.vx.data(), p.vy.data(),
                               p.vz.data(), p.ax.data(), p.ay.data(), p.az.data(), p.mass.data(), g.algo(),
                               g.precision(), g.softening(), g.theta(), dt));
}

// ---- SPH -----------------------------------------------------------------------------
SphSolver::SphSolver(Context &c) : c_(c) { c_.check(gvs_sph_params_default(&params)); }

ForceIntermediates SphSolver::compute(Particles &p) {
    upload(c_, p);
    ForceIntermediates f;
    f.omega.assign(p.count, 0.0);
    f.div_v.assign(p.count, 0.0);
    f.max_mu.assign(p.count, 0.0);
    f.dalpha_dt.assign(p.count, 0.0);
    c_.check(gvs_sph_compute(c_.get(), &params, f.omega.data(), f.div_v.data(), f.max_mu.data(),
                             f.dalpha_dt.data()));
    download(c_, p);
    return f;
}

double SphSolver::compute_timestep(const Particles &) const {
    double dt = 0.0;
    c_.check(gvs_sph_timestep(c_.get(), &params, &dt));
    return dt;
}

double step_with_sph(Particles &p, const GravitySolver &g, SphSolver &sph, double dt) {
    Context &c = sph.context();
    upload(c, p);
    double dt_next = 0.0;
    c.check(gvs_sph_step(c.get(), &sph.params, g.algo(), g.precision(), g.softening(), g.theta(), dt, &dt_next));
    download(c, p);
    return dt_next;
}

// ---- diagnostics ---------------------------------------------------------------------
double Diagnostics::momentum_magnitude() const {
    return std::sqrt(momentum[0] * momentum[0] + momentum[1] * momentum[1] + momentum[2] * momentum[2]);
}
double Diagnostics::angular_momentum_magnitude() const {
    const auto &l = angular_momentum;
    return std::sqrt(l[0] * l[0] + l[1] * l[1] + l[2] * l[2]);
}
double Diagnostics::com_drift() const {
    const auto &c = center_of_mass;
    return std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
}
const char *Diagnostics::csv_header() {
    return "step,time,kinetic_energy,potential_energy,thermal_energy,total_energy,momentum_mag,"
           "angular_momentum_mag,com_drift,virial_ratio";
}

std::string rust_exp(double v, int prec) {
    // printf gives "1.5000000000e-01"; Rust prints "1.5000000000e-1" (no zero padding, no '+')
    char buf[64];
    std::snprintf(buf, sizeof buf, "%.*e", prec, v);
    std::string s(buf);
    const size_t e = s.find('e');
    if (e == std::string::npos) return s;  // inf / nan
    const int ex = std::atoi(s.c_str() + e + 1);
    return s.substr(0, e) + "e" + std::to_string(ex);
}

std::string Diagnostics::to_csv_row() const {
    char vr[64];
    std::snprintf(vr, sizeof vr, "%.6f", virial_ratio);
    return std::to_string(step) + "," + rust_exp(time, 6) + "," + rust_exp(kinetic_energy, 10) + "," +
           rust_exp(potential_energy, 10) + "," + rust_exp(thermal_energy, 10) + "," + rust_exp(total_energy, 10) +
           "," + rust_exp(momentum_magnitude(), 10) + "," + rust_exp(angular_momentum_magnitude(), 10) + "," +
           rust_exp(com_drift(), 10) + "," + vr;
}

Diagnostics from_c(const gvs_diag &d, double time, uint64_t step) {
    Diagnostics o;
    o.kinetic_energy = d.kinetic_energy;
    o.potential_energy = d.potential_energy;
    o.thermal_energy = d.thermal_energy;
    o.total_energy = d.total_energy;
    for (int k = 0; k < 3; ++k) {
        o.momentum[k] = d.momentum[k];
        o.angular_momentum[k] = d.angular_momentum[k];
        o.center_of_mass[k] = d.center_of_mass[k];
        o.center_of_mass_velocity[k] = d.center_of_mass_velocity[k];
    }
    o.virial_ratio = d.virial_ratio;
    o.time = time;
    o.step = step;
    return o;
}

Diagnostics compute_diagnostics(const Context &c, double softening, double time, uint64_t step,
                                bool with_potential) {
    gvs_diag d;
    c.check(gvs_diagnostics(c.get(), softening, with_potential ? 1 : 0, &d));
    return from_c(d, time, step);
}

// ---- snapshots (NBODY001..003) -------------------------------------------------------
namespace {
static_assert(sizeof(double) == 8 && sizeof(uint64_t) == 8, "64-bit fields");
bool little_endian() {
    const uint16_t one = 1;
    uint8_t b;
    std::memcpy(&b, &one, 1);
    return b == 1;
}
template <class T> void put(std::ostream &w, T v) { w.write(reinterpret_cast<const char *>(&v), sizeof v); }
template <class T> T get(std::istream &r) {
    T v;
    if (!r.read(reinterpret_cast<char *>(&v), sizeof v)) throw Error(GVS_ERR_INVALID_ARG, "snapshot: truncated");
    return v;
}
void put_vec(std::ostream &w, const std::vector<double> &v) {
    w.write(reinterpret_cast<const char *>(v.data()), (std::streamsize)(v.size() * 8));
}
void get_vec(std::istream &r, std::vector<double> &v, size_t n) {
    v.assign(n, 0.0);
    if (n && !r.read(reinterpret_cast<char *>(v.data()), (std::streamsize)(n * 8)))
        throw Error(GVS_ERR_INVALID_ARG, "snapshot: truncated");
}
}  // namespace

Snapshot Snapshot::capture(const Particles &p, double time, uint64_t step, double softening, double dt) {
    Snapshot s;
    s.time = time;
    s.step = step;
    s.softening = softening;
    s.dt = dt;
    s.particles = p;
    return s;
}

void Snapshot::write_to(std::ostream &w) const {
    if (!little_endian()) throw Error(GVS_ERR_INVALID_ARG, "snapshot: big-endian hosts are not supported");
    const Particles &p = particles;
    w.write("NBODY003", 8);
    put(w, time);
    put(w, step);
    put(w, softening);
    put(w, dt);
    put(w, (uint64_t)p.count);
    for (const auto *v : {&p.x, &p.y, &p.z, &p.vx, &p.vy, &p.vz, &p.mass}) put_vec(w, *v);
    w.write(reinterpret_cast<const char *>(p.particle_type.data()), (std::streamsize)p.count);
    for (const auto *v : {&p.internal_energy, &p.smoothing_length, &p.density}) put_vec(w, *v);
    if (!w) throw Error(GVS_ERR_INVALID_ARG, "snapshot: write failed");
}

Snapshot Snapshot::read_from(std::istream &r) {
    if (!little_endian()) throw Error(GVS_ERR_INVALID_ARG, "snapshot: big-endian hosts are not supported");
    char magic[8];
    if (!r.read(magic, 8)) throw Error(GVS_ERR_INVALID_ARG, "snapshot: truncated");
    int version = 0;
    if (std::memcmp(magic, "NBODY003", 8) == 0) version = 3;
    else if (std::memcmp(magic, "NBODY002", 8) == 0) version = 2;
    else if (std::memcmp(magic, "NBODY001", 8) == 0) version = 1;
    else throw Error(GVS_ERR_INVALID_ARG, "Invalid snapshot magic bytes");
    Snapshot s;
    s.time = get<double>(r);
    s.step = get<uint64_t>(r);
    s.softening = get<double>(r);
    s.dt = get<double>(r);
    const size_t n = (size_t)get<uint64_t>(r);
    Particles &p = s.particles;
    p.resize(n);  // accelerations and the computed gas fields stay zero
    for (auto *v : {&p.x, &p.y, &p.z, &p.vx, &p.vy, &p.vz, &p.mass}) get_vec(r, *v, n);
    if (version >= 2 && n && !r.read(reinterpret_cast<char *>(p.particle_type.data()), (std::streamsize)n))
        throw Error(GVS_ERR_INVALID_ARG, "snapshot: truncated");
    if (version >= 3)
        for (auto *v : {&p.internal_energy, &p.smoothing_length, &p.density}) get_vec(r, *v, n);
    return s;
}

void Snapshot::initialize(const GravitySolver &gravity) {
    particles.clear_accelerations();
    gravity.compute_accelerations(particles);
}

// ---- scenarios -----------------------------------------------------------------------
Particles PlummerSphere::generate() const {
    Particles p(n);
    ck(gvs_ic_plummer(n, seed, scale_radius, total_mass, p.x.data(), p.y.data(), p.z.data(), p.vx.data(),
                      p.vy.data(), p.vz.data(), p.mass.data()),
       nullptr);
    return p;
}
// plummer_sphere.rs:135-152 (powi(3) is a product, powf(1/3) is pow)
double PlummerSphere::suggested_dt() const {
    return std::sqrt(scale_radius * scale_radius * scale_radius / (1.0 * total_mass)) / 100.0;
}
double PlummerSphere::suggested_softening() const {
    const double r_h = 1.305 * scale_radius;  // half-mass radius of the Plummer profile
    return std::pow(4.0 / 3.0 * M_PI * (r_h * r_h * r_h) / (double)n, 1.0 / 3.0) * 0.5;
}

double TwoBody::period() const { return 2.0 * M_PI * std::sqrt(semi_major_axis * semi_major_axis * semi_major_axis); }
Particles TwoBody::generate() const {
    Particles p(2);
    ck(gvs_ic_two_body(mass_ratio, eccentricity, semi_major_axis, p.x.data(), p.y.data(), p.z.data(), p.vx.data(),
                       p.vy.data(), p.vz.data(), p.mass.data()),
       nullptr);
    return p;
}

Particles EvrardCollapse::generate() const {
    Particles p(n_particles);
    ck(gvs_ic_evrard(n_particles, seed, total_mass, radius, u_0, p.x.data(), p.y.data(), p.z.data(), p.mass.data(),
                     p.internal_energy.data(), p.smoothing_length.data()),
       nullptr);
    std::fill(p.particle_type.begin(), p.particle_type.end(), GAS);
    std::fill(p.alpha_visc.begin(), p.alpha_visc.end(), 1.0);
    return p;
}
double EvrardCollapse::suggested_dt() const {
    return M_PI / 2.0 * std::sqrt(radius * radius * radius / (2.0 * total_mass)) / 500.0;
}
// evrard_collapse.rs:68-71 with scenarios/mod.rs:17-22 (sphere_spacing uses cbrt)
double EvrardCollapse::suggested_softening() const {
    return 0.3 * std::cbrt(4.0 / 3.0 * M_PI * (radius * radius * radius) / (double)n_particles);
}

Particles ColdCollapse::generate() const {
    Particles p(n);
    ck(gvs_ic_cold_collapse(n, seed, radius, total_mass, sph ? 1 : 0, p.x.data(), p.y.data(), p.z.data(),
                            p.vx.data(), p.vy.data(), p.vz.data(), p.mass.data(), p.internal_energy.data(),
                            p.smoothing_length.data()),
       nullptr);
    if (sph) {
        std::fill(p.particle_type.begin(), p.particle_type.end(), GAS);
        std::fill(p.alpha_visc.begin(), p.alpha_visc.end(), 1.0);
    }
    return p;
}
// cold_collapse.rs:104-122: free-fall time over 200 (gas 500); 0.3 x (4/3 pi R^3 / n)^(1/3) by powf
double ColdCollapse::suggested_dt() const {
    const double t_ff = M_PI / 2.0 * std::sqrt(radius * radius * radius / (2.0 * 1.0 * total_mass));
    return sph ? t_ff / 500.0 : t_ff / 200.0;
}
double ColdCollapse::suggested_softening() const {
    return std::pow(4.0 / 3.0 * M_PI * (radius * radius * radius) / (double)n, 1.0 / 3.0) * 0.3;
}

}  // namespace gravis
