/*
 * gvs_oracle.c -- CPU restatement of gravis sim-core (TEST INFRASTRUCTURE).
 *
 * This is the parity oracle for the GPU engine.  It is not shipped and is
 * never called by the engine: only the tests, the smoke check and the bench's
 * CPU-baseline leg load it.  Each function restates the reference algorithm
 * statement by statement, keeping its loop orders and operation order, and
 * cites the reference file:line it follows (paths relative to the gravis
 * repository).  It must be compiled with -ffp-contract=off: Rust never fuses
 * a*b+c into an FMA, so neither may this file.
 *
 * The reference's random numbers come from two third-party crates that are
 * not vendored in the reference tree: rand_core 0.9.5 / rand 0.9.2 and
 * rand_chacha 0.9.0 (Cargo.lock).  Their published algorithms are restated
 * here from the public specifications:
 *   - SeedableRng::seed_from_u64: the 32-byte seed is filled with PCG32
 *     (XSH-RR output, LCG multiplier 6364136223846793005, increment
 *     11634580027462260723), state advanced before each 4-byte output;
 *   - ChaCha20Rng: the original (DJB) ChaCha20 block function with 20 rounds,
 *     a 64-bit block counter starting at 0 and a zero 64-bit stream id; the
 *     keystream is consumed as little-endian u32 words, and next_u64 pairs
 *     two consecutive words (low word first);
 *   - StandardUniform for f64: (u64 >> 11) * 2^-53;
 *   - random_range(lo..hi) for f64: take u64 >> 12 as the mantissa of a
 *     float in [1, 2), subtract 1, multiply by (hi - lo), add lo.
 * The restatement is pinned by reproducing the reference's own Plummer
 * diagnostics file (see tests/test_oracle_pins.py).
 */
#include "gvs_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PI 3.14159265358979323846
#define ORC_NONE 0xFFFFFFFFu

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static int nthreads_or_max(int nt) { return nt > 0 ? nt : orc_max_threads(); }

/* ======================================================================== */
/* RNG                                                                       */
/* ======================================================================== */

static uint32_t rotl32(uint32_t v, int c) { return (v << c) | (v >> (32 - c)); }
static uint32_t rotr32(uint32_t v, unsigned c) { c &= 31u; return c ? (v >> c) | (v << (32 - c)) : v; }

/* PCG32 step used by rand_core's default seed_from_u64. */
static uint32_t pcg32_step(uint64_t *state) {
    const uint64_t MUL = 6364136223846793005ull;
    const uint64_t INC = 11634580027462260723ull;
    *state = *state * MUL + INC;
    uint64_t s = *state;
    uint32_t xorshifted = (uint32_t)(((s >> 18) ^ s) >> 27);
    unsigned rot = (unsigned)(s >> 59);
    return rotr32(xorshifted, rot);
}

void orc_rng_seed_u64(orc_rng *r, uint64_t seed) {
    uint64_t st = seed;
    for (int i = 0; i < 8; ++i) r->key[i] = pcg32_step(&st); /* LE bytes -> LE word */
    r->counter = 0;
    r->idx = 16;
}

#define QR(a, b, c, d)                 \
    a += b; d ^= a; d = rotl32(d, 16); \
    c += d; b ^= c; b = rotl32(b, 12); \
    a += b; d ^= a; d = rotl32(d, 8);  \
    c += d; b ^= c; b = rotl32(b, 7);

static void chacha20_block(const uint32_t key[8], uint64_t counter, uint32_t out[16]) {
    uint32_t s[16];
    s[0] = 0x61707865u; s[1] = 0x3320646eu; s[2] = 0x79622d32u; s[3] = 0x6b206574u;
    for (int i = 0; i < 8; ++i) s[4 + i] = key[i];
    s[12] = (uint32_t)counter;
    s[13] = (uint32_t)(counter >> 32);
    s[14] = 0; s[15] = 0; /* stream id 0 */
    uint32_t x[16];
    memcpy(x, s, sizeof x);
    for (int i = 0; i < 10; ++i) {
        QR(x[0], x[4], x[8], x[12]);
        QR(x[1], x[5], x[9], x[13]);
        QR(x[2], x[6], x[10], x[14]);
        QR(x[3], x[7], x[11], x[15]);
        QR(x[0], x[5], x[10], x[15]);
        QR(x[1], x[6], x[11], x[12]);
        QR(x[2], x[7], x[8], x[13]);
        QR(x[3], x[4], x[9], x[14]);
    }
    for (int i = 0; i < 16; ++i) out[i] = x[i] + s[i];
}

static uint32_t rng_next_u32(orc_rng *r) {
    if (r->idx >= 16) {
        chacha20_block(r->key, r->counter, r->buf);
        r->counter++;
        r->idx = 0;
    }
    return r->buf[r->idx++];
}

uint64_t orc_rng_next_u64(orc_rng *r) {
    uint64_t lo = rng_next_u32(r);
    uint64_t hi = rng_next_u32(r);
    return (hi << 32) | lo;
}

double orc_rng_f64(orc_rng *r) {
    uint64_t v = orc_rng_next_u64(r) >> 11;
    return (double)v * (1.0 / 9007199254740992.0);
}

double orc_rng_range(orc_rng *r, double lo, double hi) {
    uint64_t bits = (orc_rng_next_u64(r) >> 12) | (1023ull << 52);
    double v12;
    memcpy(&v12, &bits, sizeof v12);
    double v01 = v12 - 1.0;
    double scale = hi - lo;
    return v01 * scale + lo;
}

/* ======================================================================== */
/* Particles helpers                                                          */
/* ======================================================================== */

static void zero_particle(orc_particles *p, int64_t i) {
    p->ax[i] = p->ay[i] = p->az[i] = 0.0;
    p->ptype[i] = 0;
    p->density[i] = p->pressure[i] = p->u[i] = p->du_dt[i] = 0.0;
    p->h[i] = p->cs[i] = p->alpha[i] = 0.0;
}

/* Particles::add (particle.rs:94-132) at a given slot. */
static void set_particle(orc_particles *p, int64_t i, double x, double y, double z, double vx, double vy,
                         double vz, double m) {
    p->x[i] = x; p->y[i] = y; p->z[i] = z;
    p->vx[i] = vx; p->vy[i] = vy; p->vz[i] = vz;
    p->mass[i] = m;
    zero_particle(p, i);
}

/* Particles::add_gas (particle.rs:136-154). */
static void set_gas(orc_particles *p, int64_t i, double x, double y, double z, double m, double u, double h) {
    set_particle(p, i, x, y, z, 0.0, 0.0, 0.0, m);
    p->ptype[i] = ORC_GAS;
    p->u[i] = u;
    p->h[i] = h;
    p->alpha[i] = 1.0;
}

/* Particles::shift_to_com_frame (particle.rs:189-226). */
void orc_shift_to_com_frame(orc_particles *p) {
    double m_total = 0.0;
    for (int64_t i = 0; i < p->n; ++i) m_total += p->mass[i];
    if (m_total == 0.0) return;
    double cx = 0, cy = 0, cz = 0, cvx = 0, cvy = 0, cvz = 0;
    for (int64_t i = 0; i < p->n; ++i) {
        cx += p->mass[i] * p->x[i];
        cy += p->mass[i] * p->y[i];
        cz += p->mass[i] * p->z[i];
        cvx += p->mass[i] * p->vx[i];
        cvy += p->mass[i] * p->vy[i];
        cvz += p->mass[i] * p->vz[i];
    }
    cx /= m_total; cy /= m_total; cz /= m_total;
    cvx /= m_total; cvy /= m_total; cvz /= m_total;
    for (int64_t i = 0; i < p->n; ++i) {
        p->x[i] -= cx; p->y[i] -= cy; p->z[i] -= cz;
        p->vx[i] -= cvx; p->vy[i] -= cvy; p->vz[i] -= cvz;
    }
}

/* ======================================================================== */
/* Scenarios                                                                  */
/* ======================================================================== */

/* sample_plummer_particle (scenarios/plummer_sphere.rs:13-58). */
void orc_plummer_sample(orc_rng *r, double total_mass, double a, double pos[3], double vel[3]) {
    double x_mass = orc_rng_range(r, 0.001, 1.0);
    double rad = a / sqrt(pow(x_mass, -2.0 / 3.0) - 1.0);
    double cos_theta = orc_rng_range(r, -1.0, 1.0);
    double sin_theta = sqrt(1.0 - cos_theta * cos_theta);
    double phi = orc_rng_range(r, 0.0, 2.0 * ORC_PI);
    pos[0] = rad * sin_theta * cos(phi);
    pos[1] = rad * sin_theta * sin(phi);
    pos[2] = rad * cos_theta;

    double v_esc = sqrt(2.0 * 1.0 * total_mass / sqrt(rad * rad + a * a));
    double q;
    for (;;) {
        double qq = orc_rng_range(r, 0.0, 1.0);
        double g = qq * qq * pow(1.0 - qq * qq, 3.5);
        double g_max = 0.1;
        double u = orc_rng_f64(r);
        if (u < g / g_max) { q = qq; break; }
    }
    double v = q * v_esc;
    double cos_theta_v = orc_rng_range(r, -1.0, 1.0);
    double sin_theta_v = sqrt(1.0 - cos_theta_v * cos_theta_v);
    double phi_v = orc_rng_range(r, 0.0, 2.0 * ORC_PI);
    vel[0] = v * sin_theta_v * cos(phi_v);
    vel[1] = v * sin_theta_v * sin(phi_v);
    vel[2] = v * cos_theta_v;
}

/* PlummerSphere::generate (plummer_sphere.rs:106-133). p must hold n slots. */
void orc_plummer_generate(orc_particles *p, int64_t n, double scale_radius, double total_mass, uint64_t seed) {
    orc_rng r;
    orc_rng_seed_u64(&r, seed);
    p->n = n;
    double m = total_mass / (double)n;
    for (int64_t i = 0; i < n; ++i) {
        double pos[3], vel[3];
        orc_plummer_sample(&r, total_mass, scale_radius, pos, vel);
        set_particle(p, i, pos[0], pos[1], pos[2], vel[0], vel[1], vel[2], m);
    }
    orc_shift_to_com_frame(p);
}

/* plummer_sphere.rs:135-142 */
double orc_plummer_suggested_dt(double scale_radius, double total_mass) {
    double t_dyn = sqrt(scale_radius * scale_radius * scale_radius / (1.0 * total_mass));
    return t_dyn / 100.0;
}

/* plummer_sphere.rs:144-152 */
double orc_plummer_suggested_softening(int64_t n, double scale_radius) {
    double r_h = 1.305 * scale_radius;
    double mean_spacing = pow(4.0 / 3.0 * ORC_PI * (r_h * r_h * r_h) / (double)n, 1.0 / 3.0);
    return mean_spacing * 0.5;
}

/* TwoBody::generate (scenarios/two_body.rs:49-94). */
void orc_two_body_generate(orc_particles *p, double mass_ratio, double e, double a) {
    double m_total = 1.0;
    double m1 = m_total * mass_ratio;
    double m2 = m_total * (1.0 - mass_ratio);
    double r_peri = a * (1.0 - e);
    double v_peri = sqrt(1.0 * m_total * (2.0 / r_peri - 1.0 / a));
    double x1 = -m2 / m_total * r_peri;
    double x2 = m1 / m_total * r_peri;
    double vy1 = -m2 / m_total * v_peri;
    double vy2 = m1 / m_total * v_peri;
    p->n = 2;
    set_particle(p, 0, x1, 0.0, 0.0, 0.0, vy1, 0.0, m1);
    set_particle(p, 1, x2, 0.0, 0.0, 0.0, vy2, 0.0, m2);
}

/* two_body.rs:40-45 */
double orc_two_body_period(double a) { return 2.0 * ORC_PI * sqrt(a * a * a / (1.0 * 1.0)); }
/* two_body.rs:101-106 */
double orc_two_body_suggested_softening(double e, double a) { return a * (1.0 - e) * 0.001; }

/* sphere_spacing (scenarios/mod.rs:17-22) */
static void sphere_spacing(double radius, int64_t n, double *vol, double *spacing, double *h) {
    double v = 4.0 / 3.0 * ORC_PI * (radius * radius * radius);
    double s = cbrt(v / (double)n);
    *vol = v; *spacing = s; *h = 1.5 * s;
}

/* EvrardCollapse::generate (evrard_collapse.rs:45-57) + fill_uniform_gas_sphere (mod.rs:33-52). */
void orc_evrard_generate(orc_particles *p, int64_t n, double total_mass, double radius, double u0, uint64_t seed) {
    orc_rng r;
    orc_rng_seed_u64(&r, seed);
    double mass = total_mass / (double)n;
    double vol, sp, h;
    sphere_spacing(radius, n, &vol, &sp, &h);
    p->n = n;
    int64_t count = 0;
    while (count < n) {
        double x = orc_rng_f64(&r) * 2.0 * radius - radius;
        double y = orc_rng_f64(&r) * 2.0 * radius - radius;
        double z = orc_rng_f64(&r) * 2.0 * radius - radius;
        if (x * x + y * y + z * z <= radius * radius) {
            set_gas(p, count, x, y, z, mass, u0, h);
            count++;
        }
    }
}

/* ColdCollapse::generate (cold_collapse.rs:60-101): at rest, uniform in a sphere.
 * Gravity-only: per particle, draw x, y, z ~ U[-1, 1) until inside the unit sphere,
 * scale by R.  Gas (sph): fill_uniform_gas_sphere (mod.rs:33-52) with u = 0.05 and
 * h from sphere_spacing.  Then shift_to_com_frame. */
void orc_cold_collapse_generate(orc_particles *p, int64_t n, double radius, double total_mass, uint64_t seed,
                                int sph) {
    orc_rng r;
    orc_rng_seed_u64(&r, seed);
    p->n = n;
    double m = total_mass / (double)n;
    if (sph) {
        double vol, sp, h;
        sphere_spacing(radius, n, &vol, &sp, &h);
        int64_t count = 0;
        while (count < n) {
            double x = orc_rng_f64(&r) * 2.0 * radius - radius;
            double y = orc_rng_f64(&r) * 2.0 * radius - radius;
            double z = orc_rng_f64(&r) * 2.0 * radius - radius;
            if (x * x + y * y + z * z <= radius * radius) {
                set_gas(p, count, x, y, z, m, 0.05, h);
                count++;
            }
        }
    } else {
        for (int64_t i = 0; i < n; ++i) {
            double x, y, z;
            for (;;) {
                x = orc_rng_range(&r, -1.0, 1.0);
                y = orc_rng_range(&r, -1.0, 1.0);
                z = orc_rng_range(&r, -1.0, 1.0);
                if (x * x + y * y + z * z <= 1.0) break;
            }
            set_particle(p, i, x * radius, y * radius, z * radius, 0.0, 0.0, 0.0, m);
        }
    }
    orc_shift_to_com_frame(p);
}

/* cold_collapse.rs:104-114: free-fall time / 200 (gravity) or / 500 (gas) */
double orc_cold_collapse_suggested_dt(double radius, double total_mass, int sph) {
    double t_ff = (ORC_PI / 2.0) * sqrt((radius * radius * radius) / (2.0 * 1.0 * total_mass));
    return sph ? t_ff / 500.0 : t_ff / 200.0;
}

/* cold_collapse.rs:117-122: 0.3 x mean spacing, (4/3 pi R^3 / n)^(1/3) by powf */
double orc_cold_collapse_suggested_softening(int64_t n, double radius) {
    double s = pow(4.0 / 3.0 * ORC_PI * (radius * radius * radius) / (double)n, 1.0 / 3.0);
    return s * 0.3;
}

/* evrard_collapse.rs:68-71 */
double orc_evrard_suggested_softening(int64_t n, double radius) {
    double vol, sp, h;
    sphere_spacing(radius, n, &vol, &sp, &h);
    return 0.3 * sp;
}

/* ======================================================================== */
/* Direct-sum gravity                                                         */
/* ======================================================================== */

/* BruteForce::compute_accelerations (gravity.rs:47-80), serial symmetric form. */
void orc_bf_serial(orc_particles *p, double softening) {
    double eps2 = softening * softening;
    int64_t n = p->n;
    for (int64_t i = 0; i < n; ++i) {
        for (int64_t j = i + 1; j < n; ++j) {
            double dx = p->x[j] - p->x[i];
            double dy = p->y[j] - p->y[i];
            double dz = p->z[j] - p->z[i];
            double r2 = dx * dx + dy * dy + dz * dz + eps2;
            double inv_r3 = 1.0 / (r2 * sqrt(r2));
            double ai = 1.0 * p->mass[j] * inv_r3;
            double aj = 1.0 * p->mass[i] * inv_r3;
            p->ax[i] += ai * dx; p->ay[i] += ai * dy; p->az[i] += ai * dz;
            p->ax[j] -= aj * dx; p->ay[j] -= aj * dy; p->az[j] -= aj * dz;
        }
    }
}

/* Gather restatement of gravity.rs:55-78.  For target i the reference adds
 * the j>i terms and subtracts the j<i terms, in ascending j, onto a zeroed
 * a_i.  Computing dx = x_j - x_i for every j and always adding gives the same
 * IEEE result (negation is exact), so this equals orc_bf_serial bit for bit
 * when ax..az start at zero. */
static inline void bf_target(const orc_particles *p, double eps2, int64_t i, double *rax, double *ray,
                             double *raz) {
    double xi = p->x[i], yi = p->y[i], zi = p->z[i];
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int64_t j = 0; j < p->n; ++j) {
        if (j == i) continue;
        double dx = p->x[j] - xi;
        double dy = p->y[j] - yi;
        double dz = p->z[j] - zi;
        double r2 = dx * dx + dy * dy + dz * dz + eps2;
        double inv_r3 = 1.0 / (r2 * sqrt(r2));
        double f = 1.0 * p->mass[j] * inv_r3;
        sx += f * dx; sy += f * dy; sz += f * dz;
    }
    *rax = sx; *ray = sy; *raz = sz;
}

void orc_bf_gather(orc_particles *p, double softening, int nthreads) {
    double eps2 = softening * softening;
    int64_t n = p->n;
    (void)nthreads;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads_or_max(nthreads))
    for (int64_t i = 0; i < n; ++i) {
        double sx, sy, sz;
        bf_target(p, eps2, i, &sx, &sy, &sz);
        p->ax[i] += sx; p->ay[i] += sy; p->az[i] += sz;
    }
}

void orc_bf_gather_subset(const orc_particles *p, double softening, const int64_t *idx, int64_t nidx,
                          double *oax, double *oay, double *oaz, int nthreads) {
    double eps2 = softening * softening;
    (void)nthreads;
#pragma omp parallel for schedule(dynamic, 8) num_threads(nthreads_or_max(nthreads))
    for (int64_t k = 0; k < nidx; ++k) bf_target(p, eps2, idx[k], &oax[k], &oay[k], &oaz[k]);
}

/* ======================================================================== */
/* Octree (octree.rs)                                                         */
/* ======================================================================== */

/* BoundingBox::containing (octree.rs:14-44). */
void orc_bbox_containing(const orc_particles *p, double center[3], double *half_width) {
    double mn[3] = {INFINITY, INFINITY, INFINITY};
    double mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = 0; i < p->n; ++i) {
        double pos[3] = {p->x[i], p->y[i], p->z[i]};
        for (int d = 0; d < 3; ++d) {
            mn[d] = fmin(mn[d], pos[d]);
            mx[d] = fmax(mx[d], pos[d]);
        }
    }
    for (int d = 0; d < 3; ++d) center[d] = 0.5 * (mn[d] + mx[d]);
    double extent = fmax(fmax(mx[0] - mn[0], mx[1] - mn[1]), mx[2] - mn[2]);
    *half_width = 0.5 * extent * 1.001 + 1e-10;
}

/* BoundingBox::octant (octree.rs:67-79). */
int orc_octant(const double c[3], double x, double y, double z) {
    int oct = 0;
    if (x >= c[0]) oct |= 1;
    if (y >= c[1]) oct |= 2;
    if (z >= c[2]) oct |= 4;
    return oct;
}

static uint32_t tree_alloc(orc_octree *t, const double c[3], double hw) {
    if (t->count == t->cap) {
        t->cap = t->cap ? t->cap * 2 : 1024;
        t->nodes = (orc_node *)realloc(t->nodes, (size_t)t->cap * sizeof(orc_node));
    }
    orc_node *nd = &t->nodes[t->count];
    nd->center[0] = c[0]; nd->center[1] = c[1]; nd->center[2] = c[2];
    nd->half_width = hw;
    nd->total_mass = 0.0;
    nd->com[0] = nd->com[1] = nd->com[2] = 0.0;
    for (int k = 0; k < 8; ++k) nd->children[k] = ORC_NONE;
    nd->particle_index = ORC_NONE;
    return (uint32_t)t->count++;
}

/* BoundingBox::child_bounds (octree.rs:52-64). */
static void child_bounds(const orc_node *nd, int oct, double c[3], double *hw) {
    double q = nd->half_width * 0.5;
    c[0] = nd->center[0] + ((oct & 1) ? q : -q);
    c[1] = nd->center[1] + ((oct & 2) ? q : -q);
    c[2] = nd->center[2] + ((oct & 4) ? q : -q);
    *hw = q;
}

/* Octree::update_com (octree.rs:312-324). */
static void update_com(orc_node *nd, double px, double py, double pz, double mass) {
    double new_mass = nd->total_mass + mass;
    if (new_mass > 0.0) {
        double inv_new = 1.0 / new_mass;
        nd->com[0] = (nd->total_mass * nd->com[0] + mass * px) * inv_new;
        nd->com[1] = (nd->total_mass * nd->com[1] + mass * py) * inv_new;
        nd->com[2] = (nd->total_mass * nd->com[2] + mass * pz) * inv_new;
    }
    nd->total_mass = new_mass;
}

static uint32_t child_or_alloc(orc_octree *t, uint32_t node, int oct) {
    if (t->nodes[node].children[oct] == ORC_NONE) {
        double c[3], hw;
        child_bounds(&t->nodes[node], oct, c, &hw);
        uint32_t ci = tree_alloc(t, c, hw);
        t->nodes[node].children[oct] = ci;
    }
    return t->nodes[node].children[oct];
}

/* Octree::insert (octree.rs:188-239); the reference recursion is a chain of
 * tail calls, restated as a loop. */
static void tree_insert(orc_octree *t, uint32_t node, uint32_t pidx, double px, double py, double pz,
                        double mass, int depth) {
    for (;;) {
        orc_node *nd = &t->nodes[node];
        if (nd->total_mass == 0.0) { /* is_empty */
            nd->particle_index = pidx;
            nd->total_mass = mass;
            nd->com[0] = px; nd->com[1] = py; nd->com[2] = pz;
            return;
        }
        if (depth >= 64) { /* MAX_DEPTH, octree.rs:89,197-200 */
            update_com(nd, px, py, pz, mass);
            return;
        }
        uint32_t existing = nd->particle_index;
        if (existing != ORC_NONE) {
            double oc[3] = {nd->com[0], nd->com[1], nd->com[2]};
            double om = nd->total_mass;
            nd->particle_index = ORC_NONE;
            int old_oct = orc_octant(nd->center, oc[0], oc[1], oc[2]);
            double c[3], hw;
            child_bounds(nd, old_oct, c, &hw);
            uint32_t ci = tree_alloc(t, c, hw);
            t->nodes[node].children[old_oct] = ci;
            tree_insert(t, ci, existing, oc[0], oc[1], oc[2], om, depth + 1); /* child empty: leaf */
            int new_oct = orc_octant(t->nodes[node].center, px, py, pz);
            uint32_t nc = child_or_alloc(t, node, new_oct);
            update_com(&t->nodes[node], px, py, pz, mass);
            node = nc;
            depth += 1;
        } else {
            update_com(nd, px, py, pz, mass);
            int oct = orc_octant(nd->center, px, py, pz);
            node = child_or_alloc(t, node, oct);
            depth += 1;
        }
    }
}

/* Octree::rebuild (octree.rs:156-164). */
void orc_octree_rebuild(orc_octree *t, const orc_particles *p) {
    t->count = 0;
    double c[3], hw;
    orc_bbox_containing(p, c, &hw);
    tree_alloc(t, c, hw);
    for (int64_t i = 0; i < p->n; ++i)
        tree_insert(t, 0, (uint32_t)i, p->x[i], p->y[i], p->z[i], p->mass[i], 0);
}

/* Depth-first pre-order walk of the tree (children 0..7, the order of
 * query_ball_walk, octree.rs:285-289): for each leaf, its particle index,
 * depth and octant path (3 bits per level, levels 1..21 in path_hi, 22..42
 * in path_lo, left-aligned as in a 126-bit key truncated at the leaf).
 * Returns the number of leaves (fills at most cap). */
int64_t orc_octree_leaves(const orc_octree *t, uint32_t *pidx, int32_t *depth, uint64_t *path_hi,
                          uint64_t *path_lo, int64_t cap) {
    if (t->count == 0) return 0;
    typedef struct { uint32_t node; int32_t d; uint64_t hi, lo; } item;
    item *stack = (item *)malloc(sizeof(item) * (size_t)(t->count + 8));
    int64_t sp = 0, nl = 0;
    stack[sp++] = (item){0, 0, 0, 0};
    while (sp > 0) {
        item it = stack[--sp];
        const orc_node *nd = &t->nodes[it.node];
        if (nd->particle_index != ORC_NONE) {
            if (nl < cap) {
                pidx[nl] = nd->particle_index;
                depth[nl] = it.d;
                path_hi[nl] = it.hi;
                path_lo[nl] = it.lo;
            }
            nl++;
            continue;
        }
        for (int k = 7; k >= 0; --k) {
            if (nd->children[k] == ORC_NONE) continue;
            item ch = {nd->children[k], it.d + 1, it.hi, it.lo};
            int L = it.d + 1;
            if (L <= 21) ch.hi |= (uint64_t)k << (63 - 3 * L);
            else if (L <= 42) ch.lo |= (uint64_t)k << (63 - 3 * (L - 21));
            stack[sp++] = ch;
        }
    }
    free(stack);
    return nl;
}

int64_t orc_octree_count(const orc_octree *t) { return t->count; }

/* Builds the reference octree of p and returns its node count and leaves. */
int64_t orc_octree_build_leaves(const orc_particles *p, int64_t *nnodes, uint32_t *pidx, int32_t *depth,
                                uint64_t *path_hi, uint64_t *path_lo, int64_t cap) {
    orc_octree t = {0};
    orc_octree_rebuild(&t, p);
    *nnodes = t.count;
    int64_t nl = orc_octree_leaves(&t, pidx, depth, path_hi, path_lo, cap);
    orc_octree_free(&t);
    return nl;
}

void orc_octree_free(orc_octree *t) {
    free(t->nodes);
    t->nodes = NULL;
    t->count = t->cap = 0;
}

/* sphere_intersects_aabb (octree.rs:294-308). */
static int sphere_intersects_aabb(const double pos[3], double radius, const orc_node *nd) {
    double dist_sq = 0.0;
    for (int d = 0; d < 3; ++d) {
        double lo = nd->center[d] - nd->half_width;
        double hi = nd->center[d] + nd->half_width;
        double pv = pos[d];
        if (pv < lo) {
            double delta = lo - pv;
            dist_sq += delta * delta;
        } else if (pv > hi) {
            double delta = pv - hi;
            dist_sq += delta * delta;
        }
    }
    return dist_sq <= radius * radius;
}

typedef struct { uint32_t *v; int64_t len, cap; } u32vec;
static void u32vec_push(u32vec *a, uint32_t x) {
    if (a->len == a->cap) {
        a->cap = a->cap ? a->cap * 2 : 128;
        a->v = (uint32_t *)realloc(a->v, (size_t)a->cap * sizeof(uint32_t));
    }
    a->v[a->len++] = x;
}

/* Octree::query_ball / query_ball_walk (octree.rs:245-290): recursive DFS
 * over children 0..7.  An explicit stack with children pushed 7..0 pops them
 * 0..7, which is the same pre-order. */
static void query_ball_vec(const orc_octree *t, const orc_particles *p, const double pos[3], double radius,
                           u32vec *out) {
    if (t->count == 0) return;
    double radius_sq = radius * radius;
    uint32_t stack[64 * 8 + 8];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const orc_node *nd = &t->nodes[stack[--sp]];
        if (nd->total_mass == 0.0) continue;
        if (!sphere_intersects_aabb(pos, radius, nd)) continue;
        if (nd->particle_index != ORC_NONE) {
            uint32_t pi = nd->particle_index;
            double dx = p->x[pi] - pos[0];
            double dy = p->y[pi] - pos[1];
            double dz = p->z[pi] - pos[2];
            double dist_sq = dx * dx + dy * dy + dz * dz;
            if (dist_sq <= radius_sq) u32vec_push(out, pi);
            continue;
        }
        for (int k = 7; k >= 0; --k)
            if (nd->children[k] != ORC_NONE) stack[sp++] = nd->children[k];
    }
}

int64_t orc_octree_query_ball(const orc_octree *t, const orc_particles *p, const double pos[3], double radius,
                              uint32_t *out, int64_t cap) {
    u32vec v = {0};
    query_ball_vec(t, p, pos, radius, &v);
    int64_t n = v.len < cap ? v.len : cap;
    if (n > 0) memcpy(out, v.v, (size_t)n * sizeof(uint32_t));
    int64_t total = v.len;
    free(v.v);
    return total;
}

/* ======================================================================== */
/* Barnes-Hut (barnes_hut.rs)                                                 */
/* ======================================================================== */

/* BarnesHut::add_force (barnes_hut.rs:114-135). */
static inline void bh_add_force(double px, double py, double pz, double sx, double sy, double sz, double mass,
                                double eps2, double acc[3]) {
    double dx = sx - px, dy = sy - py, dz = sz - pz;
    double r2 = dx * dx + dy * dy + dz * dz + eps2;
    double inv_r3 = 1.0 / (r2 * sqrt(r2));
    double f = 1.0 * mass * inv_r3;
    acc[0] += f * dx; acc[1] += f * dy; acc[2] += f * dz;
}

/* BarnesHut::tree_walk_accel (barnes_hut.rs:44-108). */
static void bh_walk(const orc_octree *t, double px, double py, double pz, uint32_t pidx, double eps2,
                    double theta2, double acc[3]) {
    acc[0] = acc[1] = acc[2] = 0.0;
    uint32_t stack[512];
    int sp = 1;
    stack[0] = 0;
    while (sp > 0) {
        const orc_node *nd = &t->nodes[stack[--sp]];
        if (nd->total_mass == 0.0) continue;
        if (nd->particle_index != ORC_NONE) {
            if (nd->particle_index == pidx) continue;
            bh_add_force(px, py, pz, nd->com[0], nd->com[1], nd->com[2], nd->total_mass, eps2, acc);
            continue;
        }
        double dx = nd->com[0] - px, dy = nd->com[1] - py, dz = nd->com[2] - pz;
        double d2 = dx * dx + dy * dy + dz * dz;
        double s = nd->half_width * 2.0;
        if (s * s < theta2 * d2) {
            bh_add_force(px, py, pz, nd->com[0], nd->com[1], nd->com[2], nd->total_mass, eps2, acc);
            continue;
        }
        for (int k = 0; k < 8; ++k) {
            if (nd->children[k] != ORC_NONE) {
                if (sp >= 512) return; /* the reference would panic on overflow */
                stack[sp++] = nd->children[k];
            }
        }
    }
}

/* BarnesHut::compute_accelerations (barnes_hut.rs:139-192). */
void orc_bh(orc_particles *p, double softening, double theta, int nthreads) {
    int64_t n = p->n;
    if (n == 0) return;
    orc_octree t = {0};
    orc_octree_rebuild(&t, p);
    double eps2 = softening * softening;
    double theta2 = theta * theta;
    double *acc = (double *)malloc((size_t)n * 3 * sizeof(double));
    (void)nthreads;
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads_or_max(nthreads))
    for (int64_t i = 0; i < n; ++i) bh_walk(&t, p->x[i], p->y[i], p->z[i], (uint32_t)i, eps2, theta2, &acc[3 * i]);
    for (int64_t i = 0; i < n; ++i) {
        p->ax[i] += acc[3 * i];
        p->ay[i] += acc[3 * i + 1];
        p->az[i] += acc[3 * i + 2];
    }
    free(acc);
    orc_octree_free(&t);
}

/* BarnesHut::compute_accelerations restricted to the targets idx[0..nidx)
 * (barnes_hut.rs:139-192): the reference's tree of ALL particles
 * (Octree::rebuild, octree.rs:156-164), walked by tree_walk_accel
 * (barnes_hut.rs:44-108) for the listed targets only.  Writes (does not
 * accumulate) out_ax..out_az[k] for target idx[k]. */
void orc_bh_subset(const orc_particles *p, double softening, double theta, const int64_t *idx, int64_t nidx,
                   double *oax, double *oay, double *oaz, int nthreads) {
    if (p->n == 0 || nidx == 0) return;
    orc_octree t = {0};
    orc_octree_rebuild(&t, p);
    double eps2 = softening * softening;
    double theta2 = theta * theta;
    (void)nthreads;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads_or_max(nthreads))
    for (int64_t k = 0; k < nidx; ++k) {
        const int64_t i = idx[k];
        double acc[3];
        bh_walk(&t, p->x[i], p->y[i], p->z[i], (uint32_t)i, eps2, theta2, acc);
        oax[k] = acc[0];
        oay[k] = acc[1];
        oaz[k] = acc[2];
    }
    orc_octree_free(&t);
}

void orc_gravity_apply(const orc_gravity *g, orc_particles *p) {
    switch (g->kind) {
    case ORC_GRAV_BF: orc_bf_serial(p, g->softening); break;
    case ORC_GRAV_BF_GATHER: orc_bf_gather(p, g->softening, g->nthreads); break;
    case ORC_GRAV_BH: orc_bh(p, g->softening, g->theta, g->nthreads); break;
    default: break; /* NoGravity (gravity.rs:13-19) */
    }
}

/* Particles::clear_accelerations (particle.rs:173-179). */
static void clear_acc(orc_particles *p) {
    for (int64_t i = 0; i < p->n; ++i) p->ax[i] = p->ay[i] = p->az[i] = 0.0;
}

/* LeapfrogKDK::step (integrator.rs:42-76). */
void orc_kdk_step(orc_particles *p, const orc_gravity *g, double dt) {
    double half_dt = 0.5 * dt;
    int64_t n = p->n;
    for (int64_t i = 0; i < n; ++i) {
        p->vx[i] += p->ax[i] * half_dt;
        p->vy[i] += p->ay[i] * half_dt;
        p->vz[i] += p->az[i] * half_dt;
    }
    for (int64_t i = 0; i < n; ++i) {
        p->x[i] += p->vx[i] * dt;
        p->y[i] += p->vy[i] * dt;
        p->z[i] += p->vz[i] * dt;
    }
    clear_acc(p);
    orc_gravity_apply(g, p);
    for (int64_t i = 0; i < n; ++i) {
        p->vx[i] += p->ax[i] * half_dt;
        p->vy[i] += p->ay[i] * half_dt;
        p->vz[i] += p->az[i] * half_dt;
    }
}

void orc_kdk_steps(orc_particles *p, const orc_gravity *g, double dt, int64_t nsteps) {
    for (int64_t s = 0; s < nsteps; ++s) orc_kdk_step(p, g, dt);
}

/* ======================================================================== */
/* Diagnostics (diagnostics.rs:50-148)                                        */
/* ======================================================================== */

void orc_diagnostics(const orc_particles *p, double softening, int compute_potential, orc_diag *o) {
    int64_t n = p->n;
    double eps2 = softening * softening;
    double ke = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        double v2 = p->vx[i] * p->vx[i] + p->vy[i] * p->vy[i] + p->vz[i] * p->vz[i];
        ke += 0.5 * p->mass[i] * v2;
    }
    double pe = 0.0;
    if (compute_potential) {
        for (int64_t i = 0; i < n; ++i) {
            for (int64_t j = i + 1; j < n; ++j) {
                double dx = p->x[j] - p->x[i];
                double dy = p->y[j] - p->y[i];
                double dz = p->z[j] - p->z[i];
                double r2 = dx * dx + dy * dy + dz * dz + eps2;
                pe -= 1.0 * p->mass[i] * p->mass[j] / sqrt(r2);
            }
        }
    }
    double th = 0.0;
    for (int64_t i = 0; i < n; ++i)
        if (p->ptype[i] == ORC_GAS) th += p->mass[i] * p->u[i];
    double mom[3] = {0, 0, 0};
    for (int64_t i = 0; i < n; ++i) {
        mom[0] += p->mass[i] * p->vx[i];
        mom[1] += p->mass[i] * p->vy[i];
        mom[2] += p->mass[i] * p->vz[i];
    }
    double am[3] = {0, 0, 0};
    for (int64_t i = 0; i < n; ++i) {
        am[0] += p->mass[i] * (p->y[i] * p->vz[i] - p->z[i] * p->vy[i]);
        am[1] += p->mass[i] * (p->z[i] * p->vx[i] - p->x[i] * p->vz[i]);
        am[2] += p->mass[i] * (p->x[i] * p->vy[i] - p->y[i] * p->vx[i]);
    }
    double m_total = 0.0;
    for (int64_t i = 0; i < n; ++i) m_total += p->mass[i];
    double com[3] = {0, 0, 0}, cv[3] = {0, 0, 0};
    if (m_total > 0.0) {
        for (int64_t i = 0; i < n; ++i) {
            com[0] += p->mass[i] * p->x[i];
            com[1] += p->mass[i] * p->y[i];
            com[2] += p->mass[i] * p->z[i];
            cv[0] += p->mass[i] * p->vx[i];
            cv[1] += p->mass[i] * p->vy[i];
            cv[2] += p->mass[i] * p->vz[i];
        }
        for (int d = 0; d < 3; ++d) { com[d] /= m_total; cv[d] /= m_total; }
    }
    o->kinetic = ke;
    o->potential = pe;
    o->thermal = th;
    o->total = ke + pe + th;
    for (int d = 0; d < 3; ++d) {
        o->momentum[d] = mom[d];
        o->angular_momentum[d] = am[d];
        o->com[d] = com[d];
        o->com_vel[d] = cv[d];
    }
    o->virial = fabs(pe) > 0.0 ? 2.0 * ke / fabs(pe) : 0.0;
}

/* ======================================================================== */
/* SPH kernel (sph/kernel.rs:17-108), Wendland C2 with support 2h             */
/* ======================================================================== */

#define NORM_3D (21.0 / (16.0 * ORC_PI))

double orc_sph_w(double r, double h) {
    double q = r / h;
    if (q >= 2.0) return 0.0;
    double h3 = h * h * h;
    double s = 1.0 - 0.5 * q;
    double s4 = s * s * s * s;
    return NORM_3D / h3 * s4 * (1.0 + 2.0 * q);
}

void orc_sph_grad_w(double dx, double dy, double dz, double r, double h, double out[3]) {
    out[0] = out[1] = out[2] = 0.0;
    if (r < 1e-30) return;
    double q = r / h;
    if (q >= 2.0) return;
    double h3 = h * h * h;
    double s = 1.0 - 0.5 * q;
    double s3 = s * s * s;
    double dwdq = NORM_3D / h3 * (-5.0 * q) * s3;
    double factor = dwdq / (h * r);
    out[0] = factor * dx; out[1] = factor * dy; out[2] = factor * dz;
}

double orc_sph_dw_dh(double r, double h) {
    double q = r / h;
    if (q >= 2.0) return 0.0;
    double h3 = h * h * h;
    double s = 1.0 - 0.5 * q;
    double s3 = s * s * s;
    double s4 = s3 * s;
    double w_val = NORM_3D / h3 * s4 * (1.0 + 2.0 * q);
    double dwdq = NORM_3D / h3 * (-5.0 * q) * s3;
    return -3.0 / h * w_val - q / h * dwdq;
}

double orc_sph_abs_grad_w(double r, double h) {
    if (r < 1e-30) return 0.0;
    double q = r / h;
    if (q >= 2.0) return 0.0;
    double h3 = h * h * h;
    double s = 1.0 - 0.5 * q;
    double s3 = s * s * s;
    double dwdq = NORM_3D / h3 * (-5.0 * q) * s3;
    return -dwdq / h;
}

/* ======================================================================== */
/* SPH solver                                                                 */
/* ======================================================================== */

orc_sph *orc_sph_new(int nthreads) {
    orc_sph *s = (orc_sph *)calloc(1, sizeof(orc_sph));
    s->gamma = 5.0 / 3.0;    /* solver.rs:43 */
    s->eta = 1.2;            /* solver.rs:44 */
    s->cfl_factor = 0.3;     /* solver.rs:46 */
    s->force_factor = 0.25;  /* solver.rs:47 */
    s->h_max = INFINITY;     /* solver.rs:48 */
    s->beta_visc = 2.0;      /* forces.rs:34 */
    s->alpha_min = 0.1;      /* forces.rs:35 */
    s->alpha_max = 2.0;      /* forces.rs:36 */
    s->alpha_cond = 1.0;     /* forces.rs:37 */
    s->sigma_visc = 0.1;     /* forces.rs:38 */
    s->nthreads = nthreads;
    return s;
}

static void sph_resize(orc_sph *s, int64_t n) {
    if (s->n == n && s->omega) return;
    free(s->nl_start); free(s->nl_end); free(s->omega); free(s->div_v); free(s->max_mu); free(s->dalpha_dt);
    s->n = n;
    s->nl_start = (uint32_t *)calloc((size_t)n + 1, sizeof(uint32_t));
    s->nl_end = (uint32_t *)calloc((size_t)n + 1, sizeof(uint32_t));
    s->omega = (double *)calloc((size_t)n + 1, sizeof(double));
    s->div_v = (double *)calloc((size_t)n + 1, sizeof(double));
    s->max_mu = (double *)calloc((size_t)n + 1, sizeof(double));
    s->dalpha_dt = (double *)calloc((size_t)n + 1, sizeof(double));
}

void orc_sph_free(orc_sph *s) {
    if (!s) return;
    orc_octree_free(&s->tree);
    free(s->nl_idx); free(s->nl_start); free(s->nl_end);
    free(s->omega); free(s->div_v); free(s->max_mu); free(s->dalpha_dt);
    free(s);
}

static void nl_append(orc_sph *s, int64_t i, const uint32_t *v, int64_t cnt) {
    if (s->nl_len + cnt > s->nl_cap) {
        int64_t nc = s->nl_cap ? s->nl_cap : 1024;
        while (nc < s->nl_len + cnt) nc *= 2;
        s->nl_idx = (uint32_t *)realloc(s->nl_idx, (size_t)nc * sizeof(uint32_t));
        s->nl_cap = nc;
    }
    s->nl_start[i] = (uint32_t)s->nl_len;
    if (cnt) memcpy(s->nl_idx + s->nl_len, v, (size_t)cnt * sizeof(uint32_t));
    s->nl_len += cnt;
    s->nl_end[i] = (uint32_t)s->nl_len;
}

/* build_neighbor_lists (sph/neighbors.rs:56-119): queries in parallel, then
 * flattened in ascending i (neighbors.rs:86-91). */
static void build_neighbor_lists(orc_sph *s, const orc_particles *p, double factor) {
    int64_t n = p->n;
    s->nl_len = 0;
    u32vec *res = (u32vec *)calloc((size_t)n, sizeof(u32vec));
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads_or_max(s->nthreads))
    for (int64_t i = 0; i < n; ++i) {
        if (p->ptype[i] != ORC_GAS) continue;
        double hh = p->h[i];
        double radius = 2.0 * hh * factor;
        double pos[3] = {p->x[i], p->y[i], p->z[i]};
        query_ball_vec(&s->tree, p, pos, radius, &res[i]);
    }
    for (int64_t i = 0; i < n; ++i) {
        s->nl_start[i] = s->nl_end[i] = 0;
        if (p->ptype[i] != ORC_GAS) continue;
        nl_append(s, i, res[i].v, res[i].len);
        free(res[i].v);
    }
    free(res);
}

void orc_sph_neighbors_only(orc_sph *s, orc_particles *p, double factor) {
    sph_resize(s, p->n);
    orc_octree_rebuild(&s->tree, p);
    build_neighbor_lists(s, p, factor);
}

/* density_and_dw_dh (sph/density.rs:129-157). */
static void density_and_dw_dh(const orc_particles *p, const uint32_t *nb, int64_t cnt, int64_t i, double h,
                              double *rho_out, double *dwdh_out) {
    double xi = p->x[i], yi = p->y[i], zi = p->z[i];
    double rho = 0.0, dws = 0.0;
    for (int64_t k = 0; k < cnt; ++k) {
        uint32_t j = nb[k];
        double dx = xi - p->x[j];
        double dy = yi - p->y[j];
        double dz = zi - p->z[j];
        double r = sqrt(dx * dx + dy * dy + dz * dz);
        if (r < 2.0 * h) {
            double mj = p->mass[j];
            rho += mj * orc_sph_w(r, h);
            dws += mj * orc_sph_dw_dh(r, h);
        }
    }
    *rho_out = rho;
    *dwdh_out = dws;
}

/* compute_density (sph/density.rs:42-125).  The per-particle loop only reads
 * positions and masses of other particles, so it is run over particles in
 * parallel; re-queried lists are appended afterwards in ascending i, the
 * order the serial reference appends them in. */
void orc_sph_density(orc_sph *s, orc_particles *p) {
    int64_t n = p->n;
    const double search_padding = 1.1; /* density.rs:52 */
    build_neighbor_lists(s, p, search_padding);
    for (int64_t i = 0; i < n; ++i) s->omega[i] = 1.0;
    u32vec *requery = (u32vec *)calloc((size_t)n, sizeof(u32vec));
    char *has_rq = (char *)calloc((size_t)n, 1);
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads_or_max(s->nthreads))
    for (int64_t i = 0; i < n; ++i) {
        if (p->ptype[i] != ORC_GAS) continue;
        double h = p->h[i];
        double m_i = p->mass[i];
        const uint32_t *nb = s->nl_idx + s->nl_start[i];
        int64_t cnt = (int64_t)s->nl_end[i] - (int64_t)s->nl_start[i];
        for (int it = 0; it < 5; ++it) { /* MAX_H_ITERATIONS, density.rs:13 */
            double rho, dws;
            density_and_dw_dh(p, nb, cnt, i, h, &rho, &dws);
            double h_new = rho > 0.0 ? fmin(s->eta * cbrt(m_i / rho), s->h_max) : fmin(h, s->h_max);
            if (rho > 0.0) {
                double dh_drho = -h_new / (3.0 * rho);
                double om = 1.0 - dh_drho * dws;
                if (om < 0.1) om = 0.1;
                s->omega[i] = om;
            }
            p->density[i] = rho;
            p->h[i] = h_new;
            if (fabs(h_new - h) / fmax(h, 1e-30) < 1e-3) break; /* H_TOLERANCE, density.rs:16 */
            double search_radius = 2.0 * h * search_padding;
            if (2.0 * h_new > search_radius) {
                double new_radius = 2.0 * h_new * search_padding;
                double pos[3] = {p->x[i], p->y[i], p->z[i]};
                requery[i].len = 0;
                query_ball_vec(&s->tree, p, pos, new_radius, &requery[i]);
                has_rq[i] = 1;
                nb = requery[i].v;
                cnt = requery[i].len;
            }
            h = h_new;
        }
    }
    for (int64_t i = 0; i < n; ++i) {
        if (has_rq[i]) nl_append(s, i, requery[i].v, requery[i].len);
        free(requery[i].v);
    }
    free(requery);
    free(has_rq);
    /* EOS (density.rs:111-119) */
    for (int64_t i = 0; i < n; ++i) {
        if (p->ptype[i] != ORC_GAS) continue;
        double rho = p->density[i];
        double u = p->u[i];
        p->pressure[i] = (s->gamma - 1.0) * rho * u;
        p->cs[i] = sqrt(s->gamma * (s->gamma - 1.0) * fmax(u, 0.0));
    }
}

/* compute_forces (sph/forces.rs:69-232); every target is independent. */
void orc_sph_forces(orc_sph *s, orc_particles *p) {
    int64_t n = p->n;
    const double DENSITY_FLOOR = 1e-10; /* forces.rs:12 */
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads_or_max(s->nthreads))
    for (int64_t i = 0; i < n; ++i) {
        s->div_v[i] = 0.0;
        s->max_mu[i] = 0.0;
        s->dalpha_dt[i] = 0.0;
        if (p->ptype[i] != ORC_GAS) continue;
        double xi = p->x[i], yi = p->y[i], zi = p->z[i];
        double vxi = p->vx[i], vyi = p->vy[i], vzi = p->vz[i];
        double hi = p->h[i];
        double rho_i = fmax(p->density[i], DENSITY_FLOOR);
        double p_i = p->pressure[i];
        double u_i = p->u[i];
        double c_i = p->cs[i];
        double alpha_i = p->alpha[i];
        double omega_i = s->omega[i];
        double por2_i = rho_i > 0.0 ? p_i / (omega_i * rho_i * rho_i) : 0.0;
        double axa = 0.0, aya = 0.0, aza = 0.0, dua = 0.0, dva = 0.0, mmu = 0.0;
        for (uint32_t k = s->nl_start[i]; k < s->nl_end[i]; ++k) {
            int64_t j = s->nl_idx[k];
            if (j == i) continue;
            double dx = xi - p->x[j], dy = yi - p->y[j], dz = zi - p->z[j];
            double r = sqrt(dx * dx + dy * dy + dz * dz);
            double hj = p->h[j];
            double h_avg = 0.5 * (hi + hj);
            if (r >= 2.0 * hi && r >= 2.0 * hj) continue;
            double mj = p->mass[j];
            double rho_j = fmax(p->density[j], DENSITY_FLOOR);
            double p_j = p->pressure[j];
            double c_j = p->cs[j];
            double alpha_j = p->alpha[j];
            double omega_j = s->omega[j];
            double dvx = vxi - p->vx[j], dvy = vyi - p->vy[j], dvz = vzi - p->vz[j];
            double vr = dvx * dx + dvy * dy + dvz * dz;
            double gwi[3], gwj[3], gwa[3];
            orc_sph_grad_w(dx, dy, dz, r, hi, gwi);
            orc_sph_grad_w(dx, dy, dz, r, hj, gwj);
            orc_sph_grad_w(dx, dy, dz, r, h_avg, gwa);
            double por2_j = rho_j > 0.0 ? p_j / (omega_j * rho_j * rho_j) : 0.0;
            double pi_ij = 0.0;
            if (vr < 0.0) {
                double alpha_avg = 0.5 * (alpha_i + alpha_j);
                double c_avg = 0.5 * (c_i + c_j);
                double rho_avg = 0.5 * (rho_i + rho_j);
                double eta2 = 0.01 * h_avg * h_avg;
                double mu = h_avg * vr / (r * r + eta2);
                mmu = fmax(mmu, fabs(mu));
                pi_ij = rho_avg > 0.0 ? (-alpha_avg * c_avg * mu + s->beta_visc * mu * mu) / rho_avg : 0.0;
            }
            axa -= mj * (por2_i * gwi[0] + por2_j * gwj[0] + pi_ij * gwa[0]);
            aya -= mj * (por2_i * gwi[1] + por2_j * gwj[1] + pi_ij * gwa[1]);
            aza -= mj * (por2_i * gwi[2] + por2_j * gwj[2] + pi_ij * gwa[2]);
            double vdgi = dvx * gwi[0] + dvy * gwi[1] + dvz * gwi[2];
            double vdga = dvx * gwa[0] + dvy * gwa[1] + dvz * gwa[2];
            dua += mj * (por2_i * vdgi + 0.5 * pi_ij * vdga);
            dva -= mj * vdgi;
            if (s->alpha_cond > 0.0) {
                double u_j = p->u[j];
                double rho_sum = rho_i + rho_j;
                if (rho_sum > 0.0) {
                    double rho_avg = 0.5 * rho_sum;
                    double dp = fabs(p_i - p_j);
                    double v_sig_u = sqrt(dp / rho_avg);
                    double abs_gw = orc_sph_abs_grad_w(r, h_avg);
                    dua += mj * s->alpha_cond * v_sig_u * (u_i - u_j) / rho_sum * abs_gw;
                }
            }
        }
        p->ax[i] += axa;
        p->ay[i] += aya;
        p->az[i] += aza;
        p->du_dt[i] += dua;
        if (rho_i > 0.0) s->div_v[i] = dva / rho_i;
        s->max_mu[i] = mmu;
        double tau = c_i > 0.0 ? hi / (2.0 * s->sigma_visc * c_i) : 1e10;
        double source = fmax(-s->div_v[i], 0.0) * (s->alpha_max - alpha_i);
        s->dalpha_dt[i] = -(alpha_i - s->alpha_min) / tau + source;
    }
}

/* SphSolver::compute (sph/solver.rs:61-80). */
void orc_sph_compute(orc_sph *s, orc_particles *p) {
    sph_resize(s, p->n);
    orc_octree_rebuild(&s->tree, p);
    orc_sph_density(s, p);
    orc_sph_forces(s, p);
}

/* SphSolver::compute_timestep (sph/solver.rs:90-131). */
double orc_sph_timestep(const orc_sph *s, const orc_particles *p) {
    double dt_min = INFINITY;
    for (int64_t i = 0; i < p->n; ++i) {
        if (p->ptype[i] != ORC_GAS) continue;
        double h = p->h[i];
        double a_mag = sqrt(p->ax[i] * p->ax[i] + p->ay[i] * p->ay[i] + p->az[i] * p->az[i]);
        if (a_mag > 0.0) {
            double dt_force = s->force_factor * sqrt(h / a_mag);
            dt_min = fmin(dt_min, dt_force);
        }
        double c = p->cs[i];
        double alpha = p->alpha[i];
        double dva = fabs(s->div_v[i]);
        double mu_max = s->max_mu[i];
        double v_sig = c + h * dva + 1.2 * (alpha * c + s->beta_visc * mu_max);
        if (v_sig > 0.0) {
            double dt_cfl = s->cfl_factor * h / v_sig;
            dt_min = fmin(dt_min, dt_cfl);
        }
    }
    return dt_min < 1e-6 ? 1e-6 : dt_min; /* DT_FLOOR, solver.rs:17,130 */
}

/* step_with_sph (sph/solver.rs:145-212). */
double orc_sph_step(orc_particles *p, const orc_gravity *g, orc_sph *s, double dt) {
    const double ENERGY_FLOOR = 1e-10; /* solver.rs:13 */
    double half_dt = 0.5 * dt;
    int64_t n = p->n;
    for (int64_t i = 0; i < n; ++i) {
        p->vx[i] += p->ax[i] * half_dt;
        p->vy[i] += p->ay[i] * half_dt;
        p->vz[i] += p->az[i] * half_dt;
    }
    for (int64_t i = 0; i < n; ++i) {
        if (p->ptype[i] == ORC_GAS) {
            p->u[i] += p->du_dt[i] * half_dt;
            if (p->u[i] < ENERGY_FLOOR) p->u[i] = ENERGY_FLOOR;
        }
    }
    for (int64_t i = 0; i < n; ++i) {
        p->x[i] += p->vx[i] * dt;
        p->y[i] += p->vy[i] * dt;
        p->z[i] += p->vz[i] * dt;
    }
    clear_acc(p);
    for (int64_t i = 0; i < n; ++i) p->du_dt[i] = 0.0;
    orc_gravity_apply(g, p);
    orc_sph_compute(s, p);
    for (int64_t i = 0; i < n; ++i) {
        p->vx[i] += p->ax[i] * half_dt;
        p->vy[i] += p->ay[i] * half_dt;
        p->vz[i] += p->az[i] * half_dt;
    }
    for (int64_t i = 0; i < n; ++i) {
        if (p->ptype[i] == ORC_GAS) {
            p->u[i] += p->du_dt[i] * half_dt;
            if (p->u[i] < ENERGY_FLOOR) p->u[i] = ENERGY_FLOOR;
            p->alpha[i] += s->dalpha_dt[i] * dt;
            p->alpha[i] = fmin(fmax(p->alpha[i], s->alpha_min), s->alpha_max);
        }
    }
    return orc_sph_timestep(s, p);
}
