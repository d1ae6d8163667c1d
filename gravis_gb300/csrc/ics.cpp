// ics.cpp -- initial conditions on the host (the engine's own generators).
//
// The sim-core scenarios draw from ChaCha20Rng::seed_from_u64 (rand_chacha
// 0.9.0 / rand_core 0.9.5) through rand 0.9.2's f64 samplers.  This file
// implements those published algorithms so the engine can produce the same
// particle arrays as the reference scenarios:
//   seed_from_u64 : 32-byte key filled with PCG32 (XSH-RR) words;
//   ChaCha20      : DJB layout, 20 rounds, 64-bit block counter from 0,
//                   zero 64-bit stream id, keystream read as LE u32 words,
//                   a u64 draw = two consecutive words, low word first;
//   random::<f64> : (u64 >> 11) * 2^-53;
//   random_range  : mantissa (u64 >> 12) in [1,2), minus 1, times (hi-lo), plus lo.
// Transcendentals use the C library, as Rust's f64 methods do.
//
// Scenarios:
//   Plummer        PlummerSphere::generate (scenarios/plummer_sphere.rs:106-133)
//   two-body       TwoBody::generate (scenarios/two_body.rs:49-94)
//   Evrard         EvrardCollapse::generate (scenarios/evrard_collapse.rs:45-57)
//   cold collapse  ColdCollapse::generate (scenarios/cold_collapse.rs:60-101)
//   collision      two Plummer spheres on a parabolic head-on orbit (composed from
//                  sample_plummer_particle like galaxy_collision.rs:94-155)
//   gas sphere 1/r a seedless stretched, perturbed lattice with rho ~ 1/r
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "../../include/gvs.h"

namespace gvs {
// The ChaCha20 key of ChaCha20Rng::seed_from_u64(seed): eight PCG32 (XSH-RR) outputs of
// the seed (used by the host generators below and by the device Plummer generator).
void chacha_key_from_seed(uint64_t seed, uint32_t key[8]) {
    uint64_t st = seed;
    for (int i = 0; i < 8; ++i) {
        st = st * 6364136223846793005ull + 11634580027462260723ull;
        const uint32_t xs = (uint32_t)(((st >> 18) ^ st) >> 27);
        const unsigned rot = (unsigned)(st >> 59) & 31u;
        key[i] = rot ? (xs >> rot) | (xs << (32 - rot)) : xs;
    }
}
}  // namespace gvs

namespace {

const double PI = 3.14159265358979323846;

class ChaCha20Rng {
  public:
    explicit ChaCha20Rng(uint64_t seed) { gvs::chacha_key_from_seed(seed, key_); }
    uint32_t next_u32() {
        if (idx_ >= 16) {
            block(ctr_++, buf_);
            idx_ = 0;
        }
        return buf_[idx_++];
    }
    uint64_t next_u64() {
        uint64_t lo = next_u32();
        uint64_t hi = next_u32();
        return (hi << 32) | lo;
    }
    double uniform() { return (double)(next_u64() >> 11) * (1.0 / 9007199254740992.0); }
    double range(double lo, double hi) {
        uint64_t bits = (next_u64() >> 12) | (1023ull << 52);
        double v;
        memcpy(&v, &bits, 8);
        return (v - 1.0) * (hi - lo) + lo;
    }

  private:
    static uint32_t rl(uint32_t v, int c) { return (v << c) | (v >> (32 - c)); }
    void block(uint64_t counter, uint32_t out[16]) const {
        uint32_t s[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u};
        for (int i = 0; i < 8; ++i) s[4 + i] = key_[i];
        s[12] = (uint32_t)counter;
        s[13] = (uint32_t)(counter >> 32);
        s[14] = s[15] = 0;
        uint32_t x[16];
        memcpy(x, s, sizeof x);
        auto qr = [&](int a, int b, int c, int d) {
            x[a] += x[b]; x[d] ^= x[a]; x[d] = rl(x[d], 16);
            x[c] += x[d]; x[b] ^= x[c]; x[b] = rl(x[b], 12);
            x[a] += x[b]; x[d] ^= x[a]; x[d] = rl(x[d], 8);
            x[c] += x[d]; x[b] ^= x[c]; x[b] = rl(x[b], 7);
        };
        for (int r = 0; r < 10; ++r) {
            qr(0, 4, 8, 12); qr(1, 5, 9, 13); qr(2, 6, 10, 14); qr(3, 7, 11, 15);
            qr(0, 5, 10, 15); qr(1, 6, 11, 12); qr(2, 7, 8, 13); qr(3, 4, 9, 14);
        }
        for (int i = 0; i < 16; ++i) out[i] = x[i] + s[i];
    }
    uint32_t key_[8];
    uint64_t ctr_ = 0;
    uint32_t buf_[16];
    int idx_ = 16;
};

// sample_plummer_particle (scenarios/plummer_sphere.rs:13-58).
void plummer_particle(ChaCha20Rng &rng, double total_mass, double a, double pos[3], double vel[3]) {
    const double x_mass = rng.range(0.001, 1.0);
    const double r = a / sqrt(pow(x_mass, -2.0 / 3.0) - 1.0);
    const double ct = rng.range(-1.0, 1.0);
    const double st = sqrt(1.0 - ct * ct);
    const double phi = rng.range(0.0, 2.0 * PI);
    pos[0] = r * st * cos(phi);
    pos[1] = r * st * sin(phi);
    pos[2] = r * ct;
    const double v_esc = sqrt(2.0 * 1.0 * total_mass / sqrt(r * r + a * a));
    double q;
    for (;;) {
        const double qq = rng.range(0.0, 1.0);
        const double g = qq * qq * pow(1.0 - qq * qq, 3.5);
        const double u = rng.uniform();
        if (u < g / 0.1) { q = qq; break; }
    }
    const double v = q * v_esc;
    const double cv = rng.range(-1.0, 1.0);
    const double sv = sqrt(1.0 - cv * cv);
    const double pv = rng.range(0.0, 2.0 * PI);
    vel[0] = v * sv * cos(pv);
    vel[1] = v * sv * sin(pv);
    vel[2] = v * cv;
}

// Particles::shift_to_com_frame (particle.rs:189-226).
void com_frame(size_t n, double *x, double *y, double *z, double *vx, double *vy, double *vz, const double *m) {
    double mt = 0.0;
    for (size_t i = 0; i < n; ++i) mt += m[i];
    if (mt == 0.0) return;
    double c[6] = {0, 0, 0, 0, 0, 0};
    for (size_t i = 0; i < n; ++i) {
        c[0] += m[i] * x[i]; c[1] += m[i] * y[i]; c[2] += m[i] * z[i];
        c[3] += m[i] * vx[i]; c[4] += m[i] * vy[i]; c[5] += m[i] * vz[i];
    }
    for (int k = 0; k < 6; ++k) c[k] /= mt;
    for (size_t i = 0; i < n; ++i) {
        x[i] -= c[0]; y[i] -= c[1]; z[i] -= c[2];
        vx[i] -= c[3]; vy[i] -= c[4]; vz[i] -= c[5];
    }
}

uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

}  // namespace

extern "C" {

gvs_status gvs_ic_plummer(size_t n, uint64_t seed, double scale_radius, double total_mass, double *x, double *y,
                          double *z, double *vx, double *vy, double *vz, double *mass) {
    if (n == 0 || !x || !y || !z || !vx || !vy || !vz || !mass || !(scale_radius > 0.0) || !(total_mass > 0.0))
        return GVS_ERR_INVALID_ARG;
    ChaCha20Rng rng(seed);
    const double m = total_mass / (double)n;
    for (size_t i = 0; i < n; ++i) {
        double p[3], v[3];
        plummer_particle(rng, total_mass, scale_radius, p, v);
        x[i] = p[0]; y[i] = p[1]; z[i] = p[2];
        vx[i] = v[0]; vy[i] = v[1]; vz[i] = v[2];
        mass[i] = m;
    }
    com_frame(n, x, y, z, vx, vy, vz, mass);
    return GVS_OK;
}

gvs_status gvs_ic_two_body(double mass_ratio, double e, double a, double *x, double *y, double *z, double *vx,
                           double *vy, double *vz, double *mass) {
    if (!(e >= 0.0 && e < 1.0) || !(a > 0.0) || !(mass_ratio > 0.0 && mass_ratio < 1.0) || !x || !y || !z ||
        !vx || !vy || !vz || !mass)
        return GVS_ERR_INVALID_ARG;
    const double mt = 1.0, m1 = mt * mass_ratio, m2 = mt * (1.0 - mass_ratio);
    const double rp = a * (1.0 - e);
    const double vp = sqrt(1.0 * mt * (2.0 / rp - 1.0 / a));
    x[0] = -m2 / mt * rp; x[1] = m1 / mt * rp;
    y[0] = y[1] = z[0] = z[1] = 0.0;
    vx[0] = vx[1] = vz[0] = vz[1] = 0.0;
    vy[0] = -m2 / mt * vp; vy[1] = m1 / mt * vp;
    mass[0] = m1; mass[1] = m2;
    return GVS_OK;
}

gvs_status gvs_ic_evrard(size_t n, uint64_t seed, double total_mass, double radius, double u0, double *x, double *y,
                         double *z, double *mass, double *u, double *h) {
    if (n == 0 || !x || !y || !z || !mass || !u || !h || !(radius > 0.0)) return GVS_ERR_INVALID_ARG;
    ChaCha20Rng rng(seed);
    const double m = total_mass / (double)n;
    const double vol = 4.0 / 3.0 * PI * (radius * radius * radius);
    const double hh = 1.5 * cbrt(vol / (double)n);
    size_t count = 0;
    while (count < n) {
        const double px = rng.uniform() * 2.0 * radius - radius;
        const double py = rng.uniform() * 2.0 * radius - radius;
        const double pz = rng.uniform() * 2.0 * radius - radius;
        if (px * px + py * py + pz * pz <= radius * radius) {
            x[count] = px; y[count] = py; z[count] = pz;
            mass[count] = m; u[count] = u0; h[count] = hh;
            ++count;
        }
    }
    return GVS_OK;
}

// ColdCollapse::generate (scenarios/cold_collapse.rs:60-101): at rest, uniform in a
// sphere of radius R.  Gravity-only: per particle, x, y, z ~ U[-1, 1) until inside
// the unit sphere, scaled by R.  Gas: fill_uniform_gas_sphere (mod.rs:33-52) with
// u = 0.05 and h = 1.5 x the mean spacing.  Then the COM frame.
gvs_status gvs_ic_cold_collapse(size_t n, uint64_t seed, double radius, double total_mass, int sph, double *x,
                                double *y, double *z, double *vx, double *vy, double *vz, double *mass, double *u,
                                double *h) {
    if (n == 0 || !x || !y || !z || !vx || !vy || !vz || !mass || !(radius > 0.0) || !(total_mass > 0.0) ||
        (sph && (!u || !h)))
        return GVS_ERR_INVALID_ARG;
    ChaCha20Rng rng(seed);
    const double m = total_mass / (double)n;
    if (sph) {
        const double vol = 4.0 / 3.0 * PI * (radius * radius * radius);
        const double hh = 1.5 * cbrt(vol / (double)n);
        size_t count = 0;
        while (count < n) {
            const double px = rng.uniform() * 2.0 * radius - radius;
            const double py = rng.uniform() * 2.0 * radius - radius;
            const double pz = rng.uniform() * 2.0 * radius - radius;
            if (px * px + py * py + pz * pz <= radius * radius) {
                x[count] = px; y[count] = py; z[count] = pz;
                u[count] = 0.05; h[count] = hh;
                ++count;
            }
        }
    } else {
        for (size_t i = 0; i < n; ++i) {
            double px, py, pz;
            for (;;) {
                px = rng.range(-1.0, 1.0);
                py = rng.range(-1.0, 1.0);
                pz = rng.range(-1.0, 1.0);
                if (px * px + py * py + pz * pz <= 1.0) break;
            }
            x[i] = px * radius; y[i] = py * radius; z[i] = pz * radius;
        }
    }
    for (size_t i = 0; i < n; ++i) {
        vx[i] = vy[i] = vz[i] = 0.0;
        mass[i] = m;
    }
    com_frame(n, x, y, z, vx, vy, vz, mass);
    return GVS_OK;
}

// Two Plummer spheres of n/2 particles each (total mass 1, scale radius 1),
// drawn from ONE ChaCha20 stream (sphere A first, then sphere B), centred at
// x = -d/2 and +d/2 and given the parabolic relative speed sqrt(2GM/d),
// split equally and directed toward each other; then the COM frame.
gvs_status gvs_ic_collision(size_t n, uint64_t seed, double separation, double *x, double *y, double *z,
                            double *vx, double *vy, double *vz, double *mass) {
    if (n < 2 || !x || !y || !z || !vx || !vy || !vz || !mass || !(separation > 0.0)) return GVS_ERR_INVALID_ARG;
    ChaCha20Rng rng(seed);
    const size_t na = n / 2;
    const double m = 1.0 / (double)n;
    const double vrel = sqrt(2.0 * 1.0 * 1.0 / separation);
    for (size_t i = 0; i < n; ++i) {
        const bool a = i < na;
        const double msph = a ? (double)na * m : (double)(n - na) * m;
        double p[3], v[3];
        plummer_particle(rng, msph, 1.0, p, v);
        x[i] = p[0] + (a ? -0.5 : 0.5) * separation;
        y[i] = p[1];
        z[i] = p[2];
        vx[i] = v[0] + (a ? 0.5 : -0.5) * vrel;
        vy[i] = v[1];
        vz[i] = v[2];
        mass[i] = m;
    }
    com_frame(n, x, y, z, vx, vy, vz, mass);
    return GVS_OK;
}

// Gas sphere with rho ~ 1/r (M(<r) = M r^2/R^2): a cubic lattice inside the
// unit ball, each point jittered by up to 0.15 spacing (splitmix64 of its
// lattice index, no RNG state), the n points of smallest radius kept, scaled
// to radius 1, then stretched radially r -> r^{3/2} so that the uniform
// enclosed mass r0^3 becomes r^2.  h starts at eta (m / rho(r))^{1/3} with
// rho = M/(2 pi R^2 r), clamped below at r = 0.02 R.
gvs_status gvs_ic_gas_sphere_1r(size_t n, double total_mass, double radius, double u0, double eta, double *x,
                                double *y, double *z, double *mass, double *u, double *h) {
    if (n == 0 || !x || !y || !z || !mass || !u || !h || !(radius > 0.0)) return GVS_ERR_INVALID_ARG;
    const double s = cbrt(4.0 / 3.0 * PI / (double)n) * 0.97;
    const long long side = (long long)ceil(1.0 / s) + 1;
    struct P { double r, x, y, z; uint64_t id; };
    std::vector<P> pts;
    pts.reserve((size_t)(n * 1.2) + 16);
    for (long long ix = -side; ix <= side; ++ix)
        for (long long iy = -side; iy <= side; ++iy)
            for (long long iz = -side; iz <= side; ++iz) {
                const uint64_t id = ((uint64_t)(ix + side) * (2 * side + 1) + (uint64_t)(iy + side)) *
                                        (2 * side + 1) + (uint64_t)(iz + side);
                double q[3] = {(double)ix * s, (double)iy * s, (double)iz * s};
                for (int d = 0; d < 3; ++d) {
                    const uint64_t hsh = splitmix64(id * 3 + d);
                    q[d] += 0.15 * s * (((double)(hsh >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0);
                }
                const double r = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
                if (r <= 1.0) pts.push_back({r, q[0], q[1], q[2], id});
            }
    if (pts.size() < n) return GVS_ERR_INVALID_ARG;
    std::sort(pts.begin(), pts.end(), [](const P &a, const P &b) { return a.r < b.r || (a.r == b.r && a.id < b.id); });
    const double rmax = pts[n - 1].r;
    const double m = total_mass / (double)n;
    for (size_t i = 0; i < n; ++i) {
        const double r0 = pts[i].r / rmax;
        const double scale = r0 > 0.0 ? sqrt(r0) / rmax : 0.0;  // r = r0^{3/2}: factor r0^{1/2} on r0-unit vector
        const double rr = r0 * sqrt(r0) * radius;
        x[i] = pts[i].x * scale * radius;
        y[i] = pts[i].y * scale * radius;
        z[i] = pts[i].z * scale * radius;
        mass[i] = m;
        u[i] = u0;
        const double rho = total_mass / (2.0 * PI * radius * radius * std::max(rr, 0.02 * radius));
        h[i] = eta * cbrt(m / rho);
    }
    return GVS_OK;
}

// N_i = round(exp(U[ln lo, ln hi])) for the batched ensemble, from the
// engine's own ChaCha20 stream (seed recorded by the caller).
gvs_status gvs_ic_ensemble_sizes(size_t count, uint64_t seed, double lo, double hi, int64_t *sizes) {
    if (!sizes || !(lo > 0.0) || !(hi >= lo)) return GVS_ERR_INVALID_ARG;
    ChaCha20Rng rng(seed);
    for (size_t i = 0; i < count; ++i) sizes[i] = (int64_t)llround(exp(rng.range(log(lo), log(hi))));
    return GVS_OK;
}

}  // extern "C"
