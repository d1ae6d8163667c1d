/*
 * gvs_oracle.h -- CPU restatement of gravis sim-core, used ONLY as a checker.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load liboracle.so.  The GPU engine in
 * gravis_gb300/ never calls into it.
 *
 * Parity status: pinned.  The RNG + Plummer sampler + direct sum + KDK +
 * diagnostics chain reproduces the reference's committed diagnostics files
 * (artifacts/benchmarks/m1_kepler_diag.csv, m1_plummer_1k_diag.csv) and its
 * Barnes-Hut accuracy table (artifacts/benchmarks/m3_accuracy.csv); see
 * tests/test_oracle_pins.py.
 *
 * All arrays are structure-of-arrays f64, one entry per particle, exactly as
 * crates/sim-core/src/particle.rs:22-64 lays them out.
 */
#ifndef GVS_ORACLE_H
#define GVS_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Particle state: crates/sim-core/src/particle.rs:22-64 (18 arrays). */
typedef struct orc_particles {
    int64_t n;
    double *x, *y, *z;
    double *vx, *vy, *vz;
    double *ax, *ay, *az;
    double *mass;
    uint8_t *ptype;
    double *density, *pressure, *u, *du_dt, *h, *cs, *alpha;
} orc_particles;

#define ORC_GAS 4 /* ParticleType::Gas, particle.rs:9 */

/* ---- RNG: rand_chacha 0.9.0 ChaCha20Rng + rand 0.9.2 sampling ---------- */
typedef struct orc_rng {
    uint32_t key[8];
    uint64_t counter;   /* next 64-byte block number */
    uint32_t buf[16];
    int idx;            /* next unread word in buf (16 = empty) */
} orc_rng;

void     orc_rng_seed_u64(orc_rng *r, uint64_t seed);
uint64_t orc_rng_next_u64(orc_rng *r);
double   orc_rng_f64(orc_rng *r);                       /* rng.random::<f64>() */
double   orc_rng_range(orc_rng *r, double lo, double hi); /* rng.random_range(lo..hi) */

/* ---- scenarios ---------------------------------------------------------- */
void   orc_plummer_sample(orc_rng *r, double total_mass, double a, double pos[3], double vel[3]);
void   orc_plummer_generate(orc_particles *p, int64_t n, double scale_radius, double total_mass, uint64_t seed);
double orc_plummer_suggested_dt(double scale_radius, double total_mass);
double orc_plummer_suggested_softening(int64_t n, double scale_radius);
void   orc_two_body_generate(orc_particles *p, double mass_ratio, double e, double a);
double orc_two_body_period(double a);
double orc_two_body_suggested_softening(double e, double a);
void   orc_evrard_generate(orc_particles *p, int64_t n, double total_mass, double radius, double u0, uint64_t seed);
double orc_evrard_suggested_softening(int64_t n, double radius);
void   orc_cold_collapse_generate(orc_particles *p, int64_t n, double radius, double total_mass, uint64_t seed,
                                  int sph);
double orc_cold_collapse_suggested_dt(double radius, double total_mass, int sph);
double orc_cold_collapse_suggested_softening(int64_t n, double radius);
void   orc_shift_to_com_frame(orc_particles *p);

/* ---- gravity ------------------------------------------------------------ */
/* BruteForce::compute_accelerations, serial symmetric j>i form (gravity.rs:55-78). */
void orc_bf_serial(orc_particles *p, double softening);
/* Gather form, OpenMP over i; bit-identical to orc_bf_serial (j ascending). */
void orc_bf_gather(orc_particles *p, double softening, int nthreads);
/* Gather form for a subset of targets: out[k] = a(idx[k]) (not accumulated). */
void orc_bf_gather_subset(const orc_particles *p, double softening, const int64_t *idx, int64_t nidx,
                          double *oax, double *oay, double *oaz, int nthreads);

/* BarnesHut::compute_accelerations (barnes_hut.rs:139-192), octree rebuilt per call. */
void orc_bh(orc_particles *p, double softening, double theta, int nthreads);
/* The reference tree of all particles, walked for the targets idx[0..nidx) only. */
void orc_bh_subset(const orc_particles *p, double softening, double theta, const int64_t *idx, int64_t nidx,
                   double *out_ax, double *out_ay, double *out_az, int nthreads);

enum { ORC_GRAV_NONE = 0, ORC_GRAV_BF = 1, ORC_GRAV_BF_GATHER = 2, ORC_GRAV_BH = 3 };
typedef struct orc_gravity {
    int kind;
    double softening;
    double theta;
    int nthreads;
} orc_gravity;
void orc_gravity_apply(const orc_gravity *g, orc_particles *p);

/* LeapfrogKDK::step (integrator.rs:42-76). */
void orc_kdk_step(orc_particles *p, const orc_gravity *g, double dt);
void orc_kdk_steps(orc_particles *p, const orc_gravity *g, double dt, int64_t nsteps);

/* ---- diagnostics (diagnostics.rs:50-148) -------------------------------- */
typedef struct orc_diag {
    double kinetic, potential, thermal, total;
    double momentum[3], angular_momentum[3], com[3], com_vel[3];
    double virial;
} orc_diag;
void orc_diagnostics(const orc_particles *p, double softening, int compute_potential, orc_diag *out);

/* ---- octree (octree.rs) ------------------------------------------------- */
typedef struct orc_node {
    double center[3];
    double half_width;
    double total_mass;
    double com[3];
    uint32_t children[8];
    uint32_t particle_index;
} orc_node;

typedef struct orc_octree {
    orc_node *nodes;
    int64_t count, cap;
} orc_octree;

void orc_octree_rebuild(orc_octree *t, const orc_particles *p);
void orc_octree_free(orc_octree *t);
/* query_ball: appends indices in DFS order; returns count written (<= cap) and total in *total. */
int64_t orc_octree_query_ball(const orc_octree *t, const orc_particles *p, const double pos[3], double radius,
                              uint32_t *out, int64_t cap);
void orc_bbox_containing(const orc_particles *p, double center[3], double *half_width);
int64_t orc_octree_leaves(const orc_octree *t, uint32_t *pidx, int32_t *depth, uint64_t *path_hi,
                          uint64_t *path_lo, int64_t cap);
int64_t orc_octree_count(const orc_octree *t);
int64_t orc_octree_build_leaves(const orc_particles *p, int64_t *nnodes, uint32_t *pidx, int32_t *depth,
                                uint64_t *path_hi, uint64_t *path_lo, int64_t cap);
int  orc_octant(const double center[3], double x, double y, double z);

/* ---- SPH ---------------------------------------------------------------- */
double orc_sph_w(double r, double h);
void   orc_sph_grad_w(double dx, double dy, double dz, double r, double h, double out[3]);
double orc_sph_dw_dh(double r, double h);
double orc_sph_abs_grad_w(double r, double h);

typedef struct orc_sph {
    /* SphSolver::new (solver.rs:40-49) + ForceParams::default (forces.rs:30-41) */
    double gamma, eta, cfl_factor, force_factor, h_max;
    double beta_visc, alpha_min, alpha_max, alpha_cond, sigma_visc;
    int nthreads;
    /* state produced by compute() */
    orc_octree tree;
    int64_t n;
    uint32_t *nl_idx; int64_t nl_len, nl_cap; /* NeighborList.indices */
    uint32_t *nl_start, *nl_end;              /* NeighborList.offsets */
    double *omega, *div_v, *max_mu, *dalpha_dt;
} orc_sph;

orc_sph *orc_sph_new(int nthreads);
void     orc_sph_free(orc_sph *s);
/* build_neighbor_lists(particles, tree, factor) on a freshly built tree. */
void     orc_sph_neighbors_only(orc_sph *s, orc_particles *p, double search_radius_factor);
void     orc_sph_density(orc_sph *s, orc_particles *p);   /* density::compute_density */
void     orc_sph_forces(orc_sph *s, orc_particles *p);    /* forces::compute_forces */
void     orc_sph_compute(orc_sph *s, orc_particles *p);   /* SphSolver::compute */
double   orc_sph_timestep(const orc_sph *s, const orc_particles *p);
double   orc_sph_step(orc_particles *p, const orc_gravity *g, orc_sph *s, double dt); /* step_with_sph */

/* ---- misc --------------------------------------------------------------- */
int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
