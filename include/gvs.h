/*
 * gvs.h -- C ABI of the gravis GB300 engine (libgvs.so, CUDA sm_103a).
 *
 * The engine replaces the hot path of gravis sim-core: force calculation and
 * time integration.  Each entry point names the sim-core interface it stands
 * in for (paths inside the gravis repository, file:line).  Plain pointers and
 * sizes only; no C++ or torch types cross this boundary.
 *
 * Conventions
 *   - Every function returns a gvs_status; nothing throws or aborts across
 *     the ABI.  gvs_last_error() gives the message of the last failure.
 *   - Host arrays are f64 structure-of-arrays of length n, in the caller's
 *     particle order, exactly the Vec<f64> fields of sim-core's Particles
 *     (crates/sim-core/src/particle.rs:22-64).  They are borrowed for the
 *     duration of one call only.
 *   - A context owns one CUDA stream, the device-resident copy of the state
 *     and all scratch.  One context is used by one host thread at a time.
 *   - "accumulate" means: results are ADDED to the caller's arrays, which the
 *     caller zeroed before, as GravitySolver::compute_accelerations requires
 *     (crates/sim-core/src/gravity.rs:6-10).
 */
#ifndef GVS_H
#define GVS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gvs_status {
    GVS_OK = 0,
    GVS_ERR_INVALID_ARG = 1,  /* bad pointer / size / parameter */
    GVS_ERR_OOM = 2,          /* device or pinned allocation failed */
    GVS_ERR_LAUNCH = 3,       /* kernel launch or CUDA runtime error */
    GVS_ERR_DEVICE = 4,       /* a kernel raised a flag in the device error word */
    GVS_ERR_TIMEOUT = 5,      /* a bounded device-side wait gave up */
    GVS_ERR_INJECTED = 6,     /* fault injected on the host (GVS_FAULT / gvs_set_fault) */
    GVS_ERR_NO_DEVICE = 7,    /* no CUDA device / wrong architecture */
    GVS_ERR_STATE = 8         /* call made in the wrong state (e.g. no particles) */
} gvs_status;

/* Force precision of the direct-sum (and tree-walk) paths. */
enum {
    GVS_PREC_FP64_EXACT = 0, /* f64, j ascending, no FMA: bit-identical to BruteForce (gravity.rs:55-78) */
    GVS_PREC_FP64 = 1,       /* f64 tiled kernel with FMA and rsqrt: the FP64 form of the mixed kernel */
    GVS_PREC_FP32 = 2,       /* f32 absolute positions, plain f32 accumulation */
    GVS_PREC_MIXED = 3       /* f32 pairs on f64 tile centre + f32 offsets, two-sum compensated sums */
};

/* Gravity algorithm selector (headless --algorithm, crates/headless/src/main.rs:114-121). */
enum {
    GVS_ALGO_NONE = 0,   /* NoGravity (gravity.rs:13-19) */
    GVS_ALGO_DIRECT = 1, /* BruteForce (gravity.rs:47-80) */
    GVS_ALGO_BH = 2      /* BarnesHut (barnes_hut.rs:21-192) */
};

typedef struct gvs_ctx gvs_ctx;

/* Diagnostics::compute / compute_fast (crates/sim-core/src/diagnostics.rs:37-148). */
typedef struct gvs_diag {
    double kinetic_energy, potential_energy, thermal_energy, total_energy;
    double momentum[3], angular_momentum[3], center_of_mass[3], center_of_mass_velocity[3];
    double virial_ratio;
} gvs_diag;

/* SphSolver::new + ForceParams::default (crates/sim-core/src/sph/solver.rs:40-49,
 * crates/sim-core/src/sph/forces.rs:30-41). */
typedef struct gvs_sph_params {
    double gamma, eta, cfl_factor, force_factor, h_max;
    double beta_visc, alpha_min, alpha_max, alpha_cond, sigma_visc;
    /* GVS_PREC_FP64_EXACT (default): the reference's f64 arithmetic, statement by
     * statement.  GVS_PREC_MIXED (no reference counterpart): density and force pair
     * terms in f32 on float-float separations with compensated sums; neighbour lists,
     * the h iteration's decisions, Omega, EOS and the epilogues stay the f64 ones. */
    int precision;
} gvs_sph_params;

/* Kernel-time counters of one context (CUDA events on the context stream). */
typedef struct gvs_profile {
    double force_ms;          /* device time of the force kernels since reset */
    long long force_launches; /* force-kernel launches since reset */
    long long launches;       /* all kernel launches since reset */
    double force_flops;       /* algorithmic flops of those launches (20 per pair) */
    double force_bytes;       /* algorithmic bytes of those launches */
    double tile_visits;       /* (warp of 32 targets, source tile, 32-source chunk, target pair)
                                 blocks of the f32 pair kernel */
    double near_tile_visits;  /* of which took the float-float near-field path */
    double vjp_ms;            /* device time of the fused force + VJP kernels (adjoint) */
    long long vjp_launches;
    long long sph_f64_redo;   /* mixed SPH: particles whose h iteration was rerun on the f64 path
                                 (a stopping or re-query decision within 1e-5 of its threshold) */
    long long bh_groups;           /* FP32 Barnes-Hut group walk: groups walked */
    long long bh_group_fallbacks;  /* of which were walked per particle (over the iteration budget) */
    long long bh_group_iterations; /* group-walk iterations (32 nodes each) */
    long long bh_group_interactions; /* particle-node (or particle-particle) terms the group walk
                                        evaluated for real particles (fallback groups excluded) */
    long long bh_walk_terms;         /* node and particle terms summed by the per-particle walks
                                        (f64, mixed and per-particle f32 Barnes-Hut) */
} gvs_profile;

/* ---- library / context ---------------------------------------------------- */
const char *gvs_version(void);
/* Creates a context on `device` (one stream, no particles yet). */
gvs_status gvs_create(gvs_ctx **out, int device);
gvs_status gvs_destroy(gvs_ctx *ctx);
/* Copies the last error message of ctx (or of the library if ctx is NULL). */
gvs_status gvs_last_error(const gvs_ctx *ctx, char *buf, size_t len);
/* Host-side fault injection: "none", "alloc", "launch", "nan@K" (K = step). */
gvs_status gvs_set_fault(gvs_ctx *ctx, const char *spec);
/* Waits for the context stream; returns GVS_ERR_DEVICE if a kernel flagged an error. */
gvs_status gvs_sync(gvs_ctx *ctx);
/* Reads and clears the device error word.  Bits: 1 an mbarrier wait hit its cap,
 * 2 tree-walk stack overflow, 4 SPH neighbour row overflow, 8 non-finite value,
 * 16 tree invariant violated and 32 index out of range (both raised only by the checked
 * build, libgvs_checked.so, whose kernels test the indices they compute and skip bad
 * accesses instead of trapping; gvs_version() then ends in "checked)"), 64 a radix-sort
 * look-back wait hit its cap. */
gvs_status gvs_device_errors(gvs_ctx *ctx, unsigned *flags);

/* ---- state transfer (Particles <-> device) ------------------------------------ */
/* Uploads the particle state (Particles fields, particle.rs:22-64).  ptype, u,
 * h and alpha may be NULL (non-gas system).  Accelerations are zeroed. */
gvs_status gvs_set_state(gvs_ctx *ctx, size_t n, const double *x, const double *y, const double *z,
                         const double *vx, const double *vy, const double *vz, const double *mass,
                         const uint8_t *ptype, const double *u, const double *h, const double *alpha);
/* Downloads any subset of the state; NULL pointers are skipped. */
gvs_status gvs_get_state(gvs_ctx *ctx, double *x, double *y, double *z, double *vx, double *vy, double *vz,
                         double *ax, double *ay, double *az);
/* Sets / reads the resident accelerations (e.g. after a snapshot restore). */
gvs_status gvs_set_accelerations(gvs_ctx *ctx, const double *ax, const double *ay, const double *az);
gvs_status gvs_get_gas(gvs_ctx *ctx, double *density, double *pressure, double *u, double *du_dt, double *h,
                       double *sound_speed, double *alpha);
/* Overwrites any subset of the resident gas fields (NULL pointers are skipped). */
gvs_status gvs_set_gas(gvs_ctx *ctx, const double *density, const double *pressure, const double *u,
                       const double *du_dt, const double *h, const double *sound_speed, const double *alpha);
size_t gvs_count(const gvs_ctx *ctx);

/* ---- GravitySolver drop-ins (host arrays in, accelerations accumulated) -------- */
/* BruteForce::compute_accelerations (crates/sim-core/src/gravity.rs:47-80).
 * Uploads x,y,z,mass (replacing the resident positions), adds a_i to ax..az. */
gvs_status gvs_gravity_direct(gvs_ctx *ctx, size_t n, const double *x, const double *y, const double *z,
                              const double *mass, double softening, int precision, double *ax, double *ay,
                              double *az);

/* BarnesHut::compute_accelerations (crates/sim-core/src/barnes_hut.rs:139-192): octree
 * of the given positions, opening test s^2 < theta^2 d^2, monopoles.  precision
 * GVS_PREC_FP64 / FP64_EXACT walks in f64 (the reference's arithmetic per term);
 * GVS_PREC_MIXED takes the reference's opening decisions (an f32 test with a
 * certified margin, the f64 test near the boundary) and sums f32 terms on
 * float-float separations with compensated sums (within 1e-6 of f64);
 * GVS_PREC_FP32 walks on plain f32 positions and moments (fastest).  Accumulates. */
gvs_status gvs_gravity_bh(gvs_ctx *ctx, size_t n, const double *x, const double *y, const double *z,
                          const double *mass, double softening, double theta, int precision, double *ax, double *ay,
                          double *az);
/* Octree of the resident positions (Octree::rebuild, crates/sim-core/src/octree.rs:156-239),
 * in depth-first pre-order (children 0..7).  Always sets *nnodes; fills the arrays only
 * if cap >= *nnodes (any may be NULL): depth, first sorted slot, leaf particle count (0
 * for internal nodes), skip (index after the subtree), mass, com (x[nn], y[nn], z[nn]),
 * order (sorted slot -> caller index, length n) and keys (126-bit octant paths of the
 * sorted particles: high words [n] then low words [n]). */
gvs_status gvs_tree_export(gvs_ctx *ctx, size_t cap, size_t *nnodes, uint8_t *level, uint32_t *first,
                           uint32_t *count, uint32_t *skip, double *mass, double *com, uint32_t *order,
                           uint64_t *keys);

/* ---- device-resident force / integration --------------------------------------- */
/* clear_accelerations + compute_accelerations on the resident state
 * (integrator.rs:67-68): a = forces (overwrites the resident a). */
gvs_status gvs_compute_forces(gvs_ctx *ctx, int algo, int precision, double softening, double theta);
/* LeapfrogKDK::step x nsteps on the resident state (crates/sim-core/src/integrator.rs:42-76).
 * Requires valid resident accelerations (as after gvs_compute_forces). */
gvs_status gvs_kdk_steps(gvs_ctx *ctx, int algo, int precision, double softening, double theta, double dt,
                         long long nsteps);
/* Integrator::step drop-in with host arrays (integrator.rs:5-8,42-76): uploads
 * x,v,a,m, runs one KDK step on the GPU and writes x,v,a back. */
gvs_status gvs_kdk_step_host(gvs_ctx *ctx, size_t n, double *x, double *y, double *z, double *vx, double *vy,
                             double *vz, double *ax, double *ay, double *az, const double *mass, int algo,
                             int precision, double softening, double theta, double dt);

/* ---- diagnostics (crates/sim-core/src/diagnostics.rs:37-148) ------------------- */
gvs_status gvs_diagnostics(gvs_ctx *ctx, double softening, int with_potential, gvs_diag *out);

/* ---- adjoint (no reference counterpart; differentiates LeapfrogKDK::step,
 * crates/sim-core/src/integrator.rs:42-76, with BruteForce forces) ---------------- */
/* Runs nsteps KDK steps from the resident state (direct-sum forces at `precision`),
 * keeping the f64 state every checkpoint_every steps (and the last) on the device.
 * The resident state ends at the final time T. */
gvs_status gvs_adjoint_forward(gvs_ctx *ctx, int precision, double softening, double dt, long long nsteps,
                               long long checkpoint_every);
/* Reverse-mode sweep of the last gvs_adjoint_forward: given dL/dx(T), dL/dv(T) (host
 * arrays, NULL = zero), returns dL/dx(0), dL/dv(0) and the mass gradient through the
 * dynamics (host arrays, NULL = skip).  One fused force + VJP all-pairs launch per step;
 * states are recomputed backward by time reversibility and reset at every checkpoint.
 * A loss that depends on the masses directly adds its own dL/dm.  The resident state
 * is the initial state again on return. */
gvs_status gvs_adjoint_backward(gvs_ctx *ctx, const double *dl_dx, const double *dl_dy, const double *dl_dz,
                                const double *dl_dvx, const double *dl_dvy, const double *dl_dvz, double *g_x,
                                double *g_y, double *g_z, double *g_vx, double *g_vy, double *g_vz, double *g_m);
/* Checkpoints of the last forward run, for writing as NBODY003 snapshots
 * (crates/sim-core/src/snapshot.rs:40-65) and reading back in another process.
 * gvs_adjoint_checkpoints: their number, and (if cap >= *count) the step of each:
 * 0, every, 2 every, ..., nsteps.  gvs_adjoint_checkpoint_read: checkpoint k's f64
 * positions and velocities (host arrays of n, caller order).
 * gvs_adjoint_prepare: the plan of a forward run (the arguments of gvs_adjoint_forward)
 * on the resident state, without running it; gvs_adjoint_checkpoint_write then fills
 * checkpoint k, and once every checkpoint is written gvs_adjoint_backward runs as after
 * the forward run itself, with the same gradients bit for bit (the resident masses are
 * the ones the forward run used). */
gvs_status gvs_adjoint_checkpoints(gvs_ctx *ctx, long long cap, long long *count, long long *steps);
gvs_status gvs_adjoint_checkpoint_read(gvs_ctx *ctx, long long k, double *x, double *y, double *z, double *vx,
                                       double *vy, double *vz);
gvs_status gvs_adjoint_prepare(gvs_ctx *ctx, int precision, double softening, double dt, long long nsteps,
                               long long checkpoint_every);
gvs_status gvs_adjoint_checkpoint_write(gvs_ctx *ctx, long long k, const double *x, const double *y,
                                        const double *z, const double *vx, const double *vy, const double *vz);

/* ---- batched ensembles (no reference counterpart; each system is the reference's
 * BruteForce + LeapfrogKDK problem, gravity.rs:47-80, integrator.rs:42-76) ----------- */
/* The resident state (gvs_set_state) holds nsys independent systems back to back:
 * system s owns particles [sizes[0] + .. + sizes[s-1], .. + sizes[s]).  Forces act only
 * within a system, mixed precision (f32 pairs on f64 tile centres), softening shared.
 * Builds the static tile layout and work list; call again after a new upload. */
gvs_status gvs_ensemble_setup(gvs_ctx *ctx, int nsys, const int64_t *sizes, double softening);
/* a = forces of every system (one persistent launch of the pair kernel for all systems). */
gvs_status gvs_ensemble_forces(gvs_ctx *ctx);
/* nsteps KDK steps of every system; use_graph != 0 captures one step into a CUDA graph
 * (on the first call for this dt) and replays it.  Needs valid accelerations first. */
gvs_status gvs_ensemble_kdk_steps(gvs_ctx *ctx, double dt, long long nsteps, int use_graph);

/* ---- SPH (crates/sim-core/src/sph/) ---------------------------------------------- */
/* SphSolver::new defaults (solver.rs:40-49) and ForceParams::default (forces.rs:30-41). */
gvs_status gvs_sph_params_default(gvs_sph_params *out);
/* SphSolver::compute (solver.rs:61-80) on the resident state: octree, neighbour lists
 * (radius 2 h 1.1), fixed-point h / density / Omega, EOS, then forces.  Accelerations and
 * du/dt ACCUMULATE into the resident arrays (call after gravity, as the reference does).
 * The ForceIntermediates (Omega, div v, max mu, d alpha/dt) are copied to the host arrays
 * that are non-NULL. */
gvs_status gvs_sph_compute(gvs_ctx *ctx, const gvs_sph_params *params, double *omega, double *div_v,
                           double *max_mu, double *dalpha_dt);
/* SphSolver::compute_timestep (solver.rs:90-131) from the last gvs_sph_compute. */
gvs_status gvs_sph_timestep(gvs_ctx *ctx, const gvs_sph_params *params, double *dt);
/* step_with_sph (solver.rs:145-212) on the resident state with gravity `algo`;
 * *dt_next = the CFL / force timestep for the next step. */
gvs_status gvs_sph_step(gvs_ctx *ctx, const gvs_sph_params *params, int algo, int precision, double softening,
                        double theta, double dt, double *dt_next);
/* NeighborList of the last gvs_sph_compute (neighbors.rs:13-45) in caller indices:
 * *total = number of entries; if cap >= *total, particle i's neighbours are
 * idx[start[i] .. start[i] + count[i]) in the reference's depth-first order. */
gvs_status gvs_sph_neighbors(gvs_ctx *ctx, size_t cap, size_t *total, uint32_t *start, uint32_t *count,
                             uint32_t *idx);

/* Diagnostics of caller-owned device arrays WITHOUT ANY ALLOCATION.  No counterpart in
 * the reference.  For callers that cannot allocate device memory: a host whose own
 * allocator owns every device byte (an engine or framework with its own memory pool),
 * or a real-time loop that cannot afford the device synchronisation an allocation
 * implies.  x..mass (and ptype/u, which may both be NULL for a gas-free system) are
 * DEVICE pointers of length n on `device`; work is queued on `stream` (a cudaStream_t,
 * NULL for the legacy default stream) and the call waits for it.  The calling thread's
 * current device is restored on return.  Results agree with gvs_diagnostics on the same
 * state within f64 rounding (1e-12 relative; small systems sum the potential over a
 * different block layout there).
 * Scratch is a fixed ~270 KB array inside the library image that every GPU loading the
 * library keeps until the process exits; n above 4,194,304 is rejected with
 * GVS_ERR_INVALID_ARG.  The first call on a device looks the array's address up
 * (cudaGetSymbolAddress) and keeps it for the later calls.  All calls
 * share the array and each overwrites what it reads: calls on one device that overlap on
 * the GPU (other streams or other host threads) race and must be serialised by the
 * caller. */
gvs_status gvs_diagnostics_noalloc(int device, void *stream, size_t n, const double *x, const double *y,
                                   const double *z, const double *vx, const double *vy, const double *vz,
                                   const double *mass, const uint8_t *ptype, const double *u, double softening,
                                   int with_potential, gvs_diag *out);

/* ---- direct-sum accuracy probe ---------------------------------------------------- */
/* Accelerations of the targets idx[0..nidx) against all resident particles,
 * written (not accumulated) to out_ax..out_az (host arrays of length nidx). */
gvs_status gvs_direct_subset(gvs_ctx *ctx, int precision, double softening, const int64_t *idx, size_t nidx,
                             double *out_ax, double *out_ay, double *out_az);

/* Autotuner (no reference counterpart): times the compiled (block size, targets per
 * thread) variants of the f32 pair kernel on the resident state, keeps the fastest
 * for this N (power-of-two bucket) and reports it. */
gvs_status gvs_autotune_direct(gvs_ctx *ctx, int precision, double softening, int *nthreads, int *ipt, double *ms);
/* Fixes the shape of the f32 pair kernel (block size = source tile size, targets per
 * thread, minimum resident blocks per SM, source-loop unroll) instead of the autotuned or
 * default one; GVS_ERR_INVALID_ARG unless the shape is one gvs_autotune_report lists.
 * The tile size changes the f32 rounding, so a fixed shape gives run-to-run identical
 * forces across processes; the unroll does not change results.  A shape whose tile
 * holds more than n/64 particles runs with 128-particle tiles (mixed-precision accuracy
 * needs tiles that are small against the system); the autotuner skips such shapes. */
gvs_status gvs_set_direct_shape(gvs_ctx *ctx, int nthreads, int ipt, int min_blocks, int unroll);
/* Barnes-Hut walk forms (gvs_gravity_bh / ALGO_BH).
 * FP32: group_size 32, 64 or 128: one warp walks the tree for a group of up to that
 * many particles sharing a tree cell, opening a node unless s^2 < theta^2 d^2 with d
 * the distance from its COM to the group's bounding box.  Every particle then sums a
 * refinement of its own Barnes-Hut node set (the reference's test accepts every node
 * the group accepts, up to the f32 rounding of the test at the opening boundary).
 * -1 (default): 128 from 2^21 particles, else 64.  0: the per-particle walk with the
 * reference's test on f32 positions.  A group whose walk takes more than `budget`
 * iterations (32 nodes each; 0 = the default 1024) is walked per particle instead: its
 * box lies close to much denser matter, which the group test would open down to
 * single particles.
 * FP64 and MIXED walks are always per-particle. */
gvs_status gvs_set_bh_walk(gvs_ctx *ctx, int group_size, int budget);
/* Every candidate of the last gvs_autotune_direct with its kernel time (ms per force
 * evaluation).  Always sets *count; fills the arrays (any may be NULL) if cap >= *count.
 * min_blocks is the kernel's minimum resident blocks per SM (its register budget),
 * unroll the unroll depth of its source loop. */
gvs_status gvs_autotune_report(gvs_ctx *ctx, int cap, int *count, int *nthreads, int *ipt, int *min_blocks,
                               int *unroll, double *ms);

/* ---- initial conditions (crates/sim-core/src/scenarios/) --------------------------- */
/* PlummerSphere::generate (plummer_sphere.rs:106-133): ChaCha20Rng::seed_from_u64(seed),
 * sample_plummer_particle x n, shift_to_com_frame.  Outputs have length n. */
gvs_status gvs_ic_plummer(size_t n, uint64_t seed, double scale_radius, double total_mass, double *x, double *y,
                          double *z, double *vx, double *vy, double *vz, double *mass);

/* PlummerSphere::generate on the GPU, straight into ctx's resident state (n particles,
 * masses total_mass / n, gas-free, accelerations zero): the same ChaCha20 stream and draw
 * sequence as gvs_ic_plummer (every particle starts at the same stream word), values
 * within a few ulps of it (CUDA's pow/sin/cos against the C library's, parallel COM
 * sums).  n <= 2^27; scratch of about 48 n log2(n) + 100 n bytes during the call
 * (19 GB at n = 2^24).
 * GVS_ERR_STATE if a rejection decision lies within 2^-40 of its threshold, where the
 * two libraries could decide differently (use gvs_ic_plummer then); after any error the
 * resident state is allocated for n particles but its contents are unspecified. */
gvs_status gvs_ic_plummer_device(gvs_ctx *ctx, size_t n, uint64_t seed, double scale_radius, double total_mass);
/* gvs_ic_collision (two Plummer spheres from one stream, the Barnes-Hut workload's ICs) on
 * the GPU into ctx's resident state, on the same terms as gvs_ic_plummer_device. */
gvs_status gvs_ic_collision_device(gvs_ctx *ctx, size_t n, uint64_t seed, double separation);

/* TwoBody::generate (scenarios/two_body.rs:49-94): 2 particles at periapsis, COM frame. */
gvs_status gvs_ic_two_body(double mass_ratio, double e, double a, double *x, double *y, double *z, double *vx,
                           double *vy, double *vz, double *mass);
/* EvrardCollapse::generate (scenarios/evrard_collapse.rs:45-57, mod.rs:33-52): uniform gas
 * sphere by cube rejection; outputs positions, mass, u and h (velocities are zero). */
gvs_status gvs_ic_evrard(size_t n, uint64_t seed, double total_mass, double radius, double u0, double *x, double *y,
                         double *z, double *mass, double *u, double *h);
/* ColdCollapse::generate (scenarios/cold_collapse.rs:60-101): n particles at rest, uniform
 * in a sphere of `radius`, COM frame.  sph != 0: gas particles (fill_uniform_gas_sphere,
 * mod.rs:33-52; u = 0.05, h = 1.5 x mean spacing, written to u and h); else u and h may be
 * NULL.  Outputs have length n. */
gvs_status gvs_ic_cold_collapse(size_t n, uint64_t seed, double radius, double total_mass, int sph, double *x,
                                double *y, double *z, double *vx, double *vy, double *vz, double *mass, double *u,
                                double *h);
/* Two Plummer spheres (n/2 each, total mass 1, scale radius 1) from one ChaCha20 stream,
 * `separation` apart on x, parabolic head-on approach, COM frame (composed from
 * sample_plummer_particle, plummer_sphere.rs:13-58, as galaxy_collision.rs:94-155 does). */
gvs_status gvs_ic_collision(size_t n, uint64_t seed, double separation, double *x, double *y, double *z,
                            double *vx, double *vy, double *vz, double *mass);
/* Seedless gas sphere with rho ~ 1/r (stretched, jittered cubic lattice); no reference
 * counterpart (the reference's Evrard sphere is uniform). */
gvs_status gvs_ic_gas_sphere_1r(size_t n, double total_mass, double radius, double u0, double eta, double *x,
                                double *y, double *z, double *mass, double *u, double *h);
/* N_i = round(exp(U[ln lo, ln hi])) for batched ensembles, engine RNG (no reference counterpart). */
gvs_status gvs_ic_ensemble_sizes(size_t count, uint64_t seed, double lo, double hi, int64_t *sizes);

/* ---- timing / profiling ------------------------------------------------------------- */
gvs_status gvs_profile_enable(gvs_ctx *ctx, int on);  /* resets counters */
gvs_status gvs_profile_read(gvs_ctx *ctx, gvs_profile *out);
/* Records event `slot` (0..15) on the context stream; elapsed ms between two slots. */
gvs_status gvs_event_record(gvs_ctx *ctx, int slot);
gvs_status gvs_event_elapsed(gvs_ctx *ctx, int slot_a, int slot_b, float *ms);
/* The context's CUDA stream (a cudaStream_t), so that a caller can order its own CUDA
 * work against the context's (events, stream waits).  No reference counterpart. */
gvs_status gvs_stream(gvs_ctx *ctx, void **stream);
/* Writes a buffer larger than L2 on the context stream (cold-cache timing). */
gvs_status gvs_l2_flush(gvs_ctx *ctx);
/* Self-test of failure detection (no reference counterpart): a kernel waits on an
 * mbarrier that nothing completes, gives up after `polls` polls (1 .. 2^20), sets the
 * timeout bit of the device error word and exits.  Returns GVS_ERR_TIMEOUT when the
 * bounded-wait path works; the error word is cleared and the context stays usable. */
gvs_status gvs_check_bounded_wait(gvs_ctx *ctx, unsigned polls);
/* Measured FP32 FMA throughput of this GPU (TFLOP/s, 2 flop per FMA). */
gvs_status gvs_measure_fp32_peak(gvs_ctx *ctx, double *tflops);
/* The three probe forms of the last gvs_measure_fp32_peak: scalar FMA, packed f32x2 FMA,
 * and both interleaved (TFLOP/s; NULL pointers are skipped). */
gvs_status gvs_fp32_peak_variants(gvs_ctx *ctx, double *scalar, double *packed, double *mixed);

#ifdef __cplusplus
}
#endif
#endif
