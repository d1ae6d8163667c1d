// sph.cu -- grad-h SPH on the GPU (crates/sim-core/src/sph/).
//
// Everything follows the reference in f64, in the same operation order; this
// translation unit is compiled with --fmad=false so that every a*b+c rounds
// twice, as Rust does.  Particles are processed in the octree's sorted order
// (spatially coherent); results are scattered back to the caller's order.
//
//  neighbours   build_neighbor_lists + Octree::query_ball (neighbors.rs:56-119,
//               octree.rs:245-308): for each gas particle, every particle with
//               d^2 <= (2 h 1.1)^2, found by a depth-first walk of the same octree
//               with the same sphere/AABB prune, so each list is the reference's
//               set in the reference's order.  Lists live in fixed-width rows of
//               kmax slots; an overflow is flagged and the search rerun wider.
//  density      compute_density + density_and_dw_dh (density.rs:42-157): the
//               fixed-point h iteration (<= 5 iterations, tolerance 1e-3, re-query
//               when 2 h_new > 2 h 1.1), Omega, then the ideal-gas EOS.
//  forces       compute_forces (forces.rs:69-232): pressure with grad-h terms,
//               Monaghan viscosity with the per-particle alpha, Price conductivity,
//               div v, max mu, d alpha / dt.
//  timestep     SphSolver::compute_timestep (solver.rs:90-131), a min-reduction.
//  step         step_with_sph (solver.rs:145-212).
//
// The neighbour search settles its box and distance tests with an f32
// prefilter and runs the f64 test only near the boundary (lists unchanged).
// GVS_PREC_MIXED (opt-in) moves the density and force pair terms to f32 on
// float-float separations with compensated sums; the f64 pipe is a small
// fraction of the f32 one on this part, and those kernels were bound by it.
#include "gvs_internal.cuh"

namespace gvs {

namespace {

constexpr double PI_D = 3.14159265358979323846;
constexpr int MAXL_S = 42;

struct SphState {
    int kmax = 160;
    size_t n = 0;
    DevBuf list, cnt;                                  // neighbour rows [n][kmax] (sorted slots), counts
    DevBuf gas;                                        // sorted: 1 if gas
    DevBuf sx, sy, sz, svx, svy, svz, sm, sh, su, salpha;  // sorted inputs
    DevBuf srho, spres, scs, somega, sdivv, smaxmu, sdalpha, sax, say, saz, sdu;  // sorted outputs
    DevBuf dtpart;
    DevBuf pos4, nrec;  // neighbour search: f32 positions, interleaved node records (see k_sph_f32copies)
    DevBuf a4, b4, c4, d4, e4, f4;  // mixed precision: packed sources (see k_sph_src_*)
    DevBuf redo_idx, redo_count;    // mixed precision: particles whose h iteration runs again in f64
    bool have_intermediates = false;
};

SphState *sph_of(Ctx *c) {
    if (!c->sph) c->sph = new SphState();
    return static_cast<SphState *>(c->sph);
}

__device__ __forceinline__ double norm3d() { return 21.0 / (16.0 * PI_D); }

// sph/kernel.rs:26-35
__device__ __forceinline__ double kw(double r, double h) {
    const double q = r / h;
    if (q >= 2.0) return 0.0;
    const double h3 = h * h * h;
    const double s = 1.0 - 0.5 * q;
    const double s4 = s * s * s * s;
    return norm3d() / h3 * s4 * (1.0 + 2.0 * q);
}

// sph/kernel.rs:75-87
__device__ __forceinline__ double kdwdh(double r, double h) {
    const double q = r / h;
    if (q >= 2.0) return 0.0;
    const double h3 = h * h * h;
    const double s = 1.0 - 0.5 * q;
    const double s3 = s * s * s;
    const double s4 = s3 * s;
    const double w_val = norm3d() / h3 * s4 * (1.0 + 2.0 * q);
    const double dwdq = norm3d() / h3 * (-5.0 * q) * s3;
    return -3.0 / h * w_val - q / h * dwdq;
}

// sph/kernel.rs:48-64
__device__ __forceinline__ void kgrad(double dx, double dy, double dz, double r, double h, double &gx, double &gy,
                                      double &gz) {
    gx = gy = gz = 0.0;
    if (r < 1e-30) return;
    const double q = r / h;
    if (q >= 2.0) return;
    const double h3 = h * h * h;
    const double s = 1.0 - 0.5 * q;
    const double s3 = s * s * s;
    const double dwdq = norm3d() / h3 * (-5.0 * q) * s3;
    const double factor = dwdq / (h * r);
    gx = factor * dx;
    gy = factor * dy;
    gz = factor * dz;
}

// sph/kernel.rs:94-108
__device__ __forceinline__ double kabsgrad(double r, double h) {
    if (r < 1e-30) return 0.0;
    const double q = r / h;
    if (q >= 2.0) return 0.0;
    const double h3 = h * h * h;
    const double s = 1.0 - 0.5 * q;
    const double s3 = s * s * s;
    const double dwdq = norm3d() / h3 * (-5.0 * q) * s3;
    return -dwdq / h;
}

// Octree::sphere_intersects_aabb (octree.rs:294-308) on the node's cell box.
__device__ __forceinline__ bool sphere_hits_box(double px, double py, double pz, double radius, double cx, double cy,
                                                double cz, double hw) {
    double d2 = 0.0;
    const double p[3] = {px, py, pz}, c[3] = {cx, cy, cz};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double lo = c[d] - hw, hi = c[d] + hw;
        if (p[d] < lo) {
            const double e = lo - p[d];
            d2 += e * e;
        } else if (p[d] > hi) {
            const double e = p[d] - hi;
            d2 += e * e;
        }
    }
    return d2 <= radius * radius;
}

// ---- f32 prefilter of the neighbour search ------------------------------------------
// The ball query decides membership and pruning with the reference's f64 tests.
// Most decisions are far from the boundary: an f32 test with a certified margin
// settles them, and only the rare borderline case runs the f64 test, so lists
// (set and order) are exactly the f64 ones.  With X bounding every coordinate,
// node centre and half width (the root cell: max |c_root| + root half width),
// f32 rounding moves a point-point or point-box distance by at most ~1.8 E with
// E = 2^-21 X; the margin is 3 E, plus a relative 2^-19 on the squared bounds.
struct Prefilter {
    float px, py, pz, rin2, rout2;
};

__device__ __forceinline__ float prefilter_scale(const TreeView &tv) {
    const double x = fmax(fabs(tv.bx[0]), fmax(fabs(tv.by[0]), fabs(tv.bz[0]))) + tv.root_hw;
    return (float)(x * 0x1p-21);
}

__device__ __forceinline__ Prefilter prefilter(double px, double py, double pz, double radius, float E) {
    Prefilter f;
    f.px = (float)px; f.py = (float)py; f.pz = (float)pz;
    const float rf = (float)radius, m = 3.0f * E;
    const float rin = rf - m, rout = rf + m;
    f.rin2 = rin > 0.f ? rin * rin * (1.0f - 0x1p-19f) : -1.0f;
    f.rout2 = rout * rout * (1.0f + 0x1p-19f);
    return f;
}

// 1 inside, 0 outside, -1 undecided (run the f64 test)
__device__ __forceinline__ int pref_point(const Prefilter &f, float4 q) {
    const float ex = q.x - f.px, ey = q.y - f.py, ez = q.z - f.pz;
    const float d2 = ex * ex + ey * ey + ez * ez;
    return d2 < f.rin2 ? 1 : (d2 > f.rout2 ? 0 : -1);
}

__device__ __forceinline__ int pref_box(const Prefilter &f, float4 b) {
    float d2 = 0.f;
    const float p[3] = {f.px, f.py, f.pz}, c[3] = {b.x, b.y, b.z};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const float lo = c[d] - b.w, hi = c[d] + b.w;
        if (p[d] < lo) {
            const float e = lo - p[d];
            d2 += e * e;
        } else if (p[d] > hi) {
            const float e = p[d] - hi;
            d2 += e * e;
        }
    }
    return d2 < f.rin2 ? 1 : (d2 > f.rout2 ? 0 : -1);
}

// Node records of the walk: meta4 = (skip, first, count, depth); node4 = the cell
// box (centre, half width) in f32, except for a one-particle leaf, where it is
// that particle's f32 position: the particle test then decides (a particle
// certainly inside the sphere lies in a box that certainly meets it, and one
// certainly outside adds nothing either way), and only an undecided one runs
// both of the reference's f64 tests, box then particle.
//
// meta4 = (skip, first particle, count, depth): count > 0 for a leaf, minus the
// subtree's particle count for an internal node.
// Node k's records sit side by side (meta4[2k], node4[2k + 1] of one buffer): the
// walk reads both at every step, so they share a cache line.
__global__ void k_sph_f32copies(const TreeView tv, float4 *__restrict__ pos4, float4 *__restrict__ node4,
                                int4 *__restrict__ meta4) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < tv.n) pos4[i] = make_float4((float)tv.sx[i], (float)tv.sy[i], (float)tv.sz[i], 0.f);
    if (i < tv.nnodes) {
        const uint32_t c = tv.cnt[i], f = tv.first[i], sk = tv.skip[i];
        const uint32_t sub = (uint32_t)((sk < tv.nnodes ? (size_t)tv.first[sk] : tv.n) - f);
        meta4[2 * i] = make_int4((int)sk, (int)f, c > 0 ? (int)c : -(int)sub, (int)tv.level[i]);
        node4[2 * i + 1] = c == 1 ? make_float4((float)tv.sx[f], (float)tv.sy[f], (float)tv.sz[f], 0.f)
                          : make_float4((float)tv.bx[i], (float)tv.by[i], (float)tv.bz[i],
                                        (float)ldexp(tv.root_hw, -(int)tv.level[i]));
    }
}

// The reference's query (octree.rs:245-308) for one sphere and particle j: every
// cell on the path from the root to j's leaf passes sphere_intersects_aabb, then
// the distance test.  For the prefilter's undecided cases.
__device__ bool member_exact(const TreeView &tv, uint32_t leaf, uint32_t j, double px, double py, double pz,
                             double radius) {
    for (uint32_t a = leaf; a != 0xFFFFFFFFu; a = tv.parent[a]) {
        const double hw = ldexp(tv.root_hw, -(int)tv.level[a]);
        if (!sphere_hits_box(px, py, pz, radius, tv.bx[a], tv.by[a], tv.bz[a], hw)) return false;
    }
    const double dx = tv.sx[j] - px, dy = tv.sy[j] - py, dz = tv.sz[j] - pz;
    return dx * dx + dy * dy + dz * dz <= radius * radius;
}

// Cells of at most RANGE_MAX particles are not descended: their particles (a
// contiguous, depth-first-ordered range) are tested directly.  A particle
// certainly inside the sphere lies in cells that all certainly meet it; one
// certainly outside is dropped either way; an undecided one runs the reference's
// tests on its whole path (member_exact), so the lists are the reference's.
constexpr int RANGE_MAX = 32;

// One node of the ball query: appends its hits to row in depth-first order and
// returns the next node.  See k_sph_f32copies for the record layout.
__device__ __forceinline__ uint32_t ball_visit(const TreeView &tv, const float4 *__restrict__ pos4, int4 mt,
                                               float4 nd, uint32_t k, const Prefilter &pf, double px, double py,
                                               double pz, double radius, uint32_t *row, int kmax, int &count) {
    const double r2 = radius * radius;
    if (mt.z == 1) {  // one-particle leaf
        const uint32_t j = (uint32_t)mt.y;
        int in = pref_point(pf, nd);
        if (in < 0) {
            const double hw = ldexp(tv.root_hw, -mt.w);
            in = sphere_hits_box(px, py, pz, radius, tv.bx[k], tv.by[k], tv.bz[k], hw);
            if (in) {
                const double dx = tv.sx[j] - px, dy = tv.sy[j] - py, dz = tv.sz[j] - pz;
                in = dx * dx + dy * dy + dz * dz <= r2;
            }
        }
        if (in) {
            if (count < kmax) row[count] = j;
            ++count;
        }
        return (uint32_t)mt.x;
    }
    int hit = pref_box(pf, nd);
    if (hit < 0) {
        const double hw = ldexp(tv.root_hw, -mt.w);
        hit = sphere_hits_box(px, py, pz, radius, tv.bx[k], tv.by[k], tv.bz[k], hw);
    }
    if (!hit) return (uint32_t)mt.x;
    if (mt.z < -RANGE_MAX) return k + 1;  // internal: descend
    const bool bucket = mt.z > 1;         // else a small internal cell, tested as a range
    const uint32_t c = (uint32_t)(bucket ? mt.z : -mt.z);
    for (uint32_t j = (uint32_t)mt.y; j < (uint32_t)mt.y + c; ++j) {
        int in = pref_point(pf, pos4[j]);
        if (in < 0) {
            if (bucket) {  // this leaf's box passed: the particle test decides
                const double dx = tv.sx[j] - px, dy = tv.sy[j] - py, dz = tv.sz[j] - pz;
                in = dx * dx + dy * dy + dz * dz <= r2;
            } else {
                in = member_exact(tv, tv.leaf_of[j], j, px, py, pz, radius) ? 1 : 0;
            }
        }
        if (in) {
            if (count < kmax) row[count] = j;
            ++count;
        }
    }
    return (uint32_t)mt.x;
}

__global__ void k_gather_sph(size_t n, const uint32_t *__restrict__ perm, const uint8_t *__restrict__ ptype,
                             const double *__restrict__ vx, const double *__restrict__ vy,
                             const double *__restrict__ vz, const double *__restrict__ m,
                             const double *__restrict__ h, const double *__restrict__ u,
                             const double *__restrict__ alpha, const double *__restrict__ rho,
                             const double *__restrict__ pres, const double *__restrict__ cs,
                             uint8_t *__restrict__ gas, double *__restrict__ svx,
                             double *__restrict__ svy, double *__restrict__ svz, double *__restrict__ sm,
                             double *__restrict__ sh, double *__restrict__ su, double *__restrict__ salpha,
                             double *__restrict__ srho, double *__restrict__ spres, double *__restrict__ scs) {
    const size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const uint32_t o = perm[s];
    if (!CHK_IDX(o, n)) return;
    gas[s] = ptype[o] == 4 ? 1 : 0;
    svx[s] = vx[o]; svy[s] = vy[o]; svz[s] = vz[o];
    sm[s] = m[o]; sh[s] = h[o]; su[s] = u[o]; salpha[s] = alpha[o];
    // non-gas neighbours keep their stored rho, P, c (zero unless set), as in the reference
    srho[s] = rho[o]; spres[s] = pres[o]; scs[s] = cs[o];
}

// Ball query of one target (per-thread walk), used for the re-queries of the
// density iteration.  Returns the number found (writes at most kmax).
__device__ int ball_query_thread(const TreeView &tv, const float4 *__restrict__ pos4,
                                 const float4 *__restrict__ node4, const int4 *__restrict__ meta4, float E, double px,
                                 double py, double pz, double radius, uint32_t *row, int kmax) {
    const Prefilter pf = prefilter(px, py, pz, radius, E);
    int count = 0;
    uint32_t k = 0;
    while ((size_t)k < tv.nnodes)
        k = ball_visit(tv, pos4, meta4[2 * (size_t)k], node4[2 * (size_t)k + 1], k, pf, px, py, pz, radius, row, kmax,
                       count);
    return count;
}

// Neighbour lists of all gas particles (build_neighbor_lists with factor):
// warp-synchronous walk, each lane with its own next-node pointer.
// One particle per lane; warps take chunks of 32 sorted particles from a counter
// (work[0]), so uneven walks balance across the GPU and no partial wave is left.
__global__ void __launch_bounds__(128) k_neighbors(const TreeView tv, const float4 *__restrict__ pos4,
                                                   const float4 *__restrict__ node4, const int4 *__restrict__ meta4,
                                                   const uint8_t *__restrict__ gas, const double *__restrict__ sh,
                                                   double factor, int kmax, uint32_t *__restrict__ list,
                                                   uint32_t *__restrict__ cnt, unsigned *__restrict__ err,
                                                   unsigned *__restrict__ work) {
    const int lane = threadIdx.x & 31;
    const float E = prefilter_scale(tv);
    for (;;) {
        unsigned base = 0;
        if (lane == 0) base = atomicAdd(work, 32u);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if ((size_t)base >= tv.n) break;
        const size_t t = (size_t)base + lane;
        const bool active = t < tv.n && gas[t];
        double px = 0, py = 0, pz = 0, radius = 0;
        if (active) {
            px = tv.sx[t]; py = tv.sy[t]; pz = tv.sz[t];
            radius = 2.0 * sh[t] * factor;
        }
        const Prefilter pf = prefilter(px, py, pz, radius, E);
        uint32_t *row = list + t * (size_t)kmax;
        int count = 0;
        uint32_t next = active ? 0u : 0xFFFFFFFFu;
        for (;;) {
            const uint32_t k = __reduce_min_sync(0xFFFFFFFFu, next);
            if ((size_t)k >= tv.nnodes) break;
            if (next != k) continue;
            next = ball_visit(tv, pos4, meta4[2 * (size_t)k], node4[2 * (size_t)k + 1], k, pf, px, py, pz, radius, row,
                              kmax, count);
        }
        if (t < tv.n) {
            cnt[t] = active ? (uint32_t)count : 0u;
            if (count > kmax) atomicOr(err, (unsigned)DERR_NEIGH_OVERFLOW);
        }
    }
}

// The two sums of one density iteration (density.rs:60-75), f64, in list order.
__device__ __forceinline__ void density_sums_f64(const TreeView &tv, const double *__restrict__ sm,
                                                 const uint32_t *row, int count, double xi, double yi, double zi,
                                                 double h, double &rho, double &dws) {
    rho = 0.0;
    dws = 0.0;
    for (int k = 0; k < count; ++k) {
        const uint32_t j = row[k];
        if (!CHK_IDX(j, tv.n)) continue;
        const double dx = xi - tv.sx[j], dy = yi - tv.sy[j], dz = zi - tv.sz[j];
        const double r = sqrt(dx * dx + dy * dy + dz * dz);
        if (r < 2.0 * h) {
            const double mj = sm[j];
            rho += mj * kw(r, h);
            dws += mj * kdwdh(r, h);
        }
    }
}

// compute_density (density.rs:42-125) for one target per thread, then the EOS.
__device__ void density_particle_f64(const TreeView &tv, const float4 *__restrict__ pos4,
                                     const float4 *__restrict__ node4, const int4 *__restrict__ meta4,
                                     const double *__restrict__ sm,
                                     const double *__restrict__ su, double *__restrict__ sh,
                                     uint32_t *__restrict__ list, uint32_t *__restrict__ cnt, int kmax, double gamma,
                                     double eta, double h_max, double *__restrict__ rho_out,
                                     double *__restrict__ omega_out, double *__restrict__ pres,
                                     double *__restrict__ cs, unsigned *__restrict__ err, size_t i) {
    const double search_padding = 1.1;
    const double xi = tv.sx[i], yi = tv.sy[i], zi = tv.sz[i];
    const double m_i = sm[i];
    double h = sh[i];
    uint32_t *row = list + i * (size_t)kmax;
    int count = (int)cnt[i];
    double rho_last = rho_out[i];
    for (int it = 0; it < 5; ++it) {
        double rho, dws;
        density_sums_f64(tv, sm, row, count, xi, yi, zi, h, rho, dws);
        const double h_new = rho > 0.0 ? fmin(eta * cbrt(m_i / rho), h_max) : fmin(h, h_max);
        if (rho > 0.0) {
            const double dh_drho = -h_new / (3.0 * rho);
            double om = 1.0 - dh_drho * dws;
            if (om < 0.1) om = 0.1;
            omega_out[i] = om;
        }
        rho_last = rho;
        sh[i] = h_new;
        if (fabs(h_new - h) / fmax(h, 1e-30) < 1e-3) break;
        const double search_radius = 2.0 * h * search_padding;
        if (2.0 * h_new > search_radius) {
            const double new_radius = 2.0 * h_new * search_padding;
            count = ball_query_thread(tv, pos4, node4, meta4, prefilter_scale(tv), xi, yi, zi, new_radius, row, kmax);
            if (count > kmax) {
                atomicOr(err, (unsigned)DERR_NEIGH_OVERFLOW);
                count = kmax;
            }
            cnt[i] = (uint32_t)count;
        }
        h = h_new;
    }
    rho_out[i] = rho_last;
    // EOS (density.rs:111-119)
    const double u = su[i];
    pres[i] = (gamma - 1.0) * rho_last * u;
    cs[i] = sqrt(gamma * (gamma - 1.0) * fmax(u, 0.0));
}

__global__ void k_density(const TreeView tv, const float4 *__restrict__ pos4, const float4 *__restrict__ node4,
                          const int4 *__restrict__ meta4, const uint8_t *__restrict__ gas, const double *__restrict__ sm,
                          const double *__restrict__ su, double *__restrict__ sh, uint32_t *__restrict__ list,
                          uint32_t *__restrict__ cnt, int kmax, double gamma, double eta, double h_max,
                          double *__restrict__ rho_out, double *__restrict__ omega_out, double *__restrict__ pres,
                          double *__restrict__ cs, unsigned *__restrict__ err) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= tv.n) return;
    omega_out[i] = 1.0;
    if (!gas[i]) return;
    density_particle_f64(tv, pos4, node4, meta4, sm, su, sh, list, cnt, kmax, gamma, eta, h_max, rho_out, omega_out,
                         pres, cs, err, i);
}

// compute_forces (forces.rs:69-232), one target per thread.
__global__ void k_forces(const TreeView tv, const uint8_t *__restrict__ gas, const uint32_t *__restrict__ list,
                         const uint32_t *__restrict__ cnt, int kmax, const double *__restrict__ svx,
                         const double *__restrict__ svy, const double *__restrict__ svz,
                         const double *__restrict__ sm, const double *__restrict__ sh, const double *__restrict__ srho,
                         const double *__restrict__ spres, const double *__restrict__ su,
                         const double *__restrict__ scs, const double *__restrict__ salpha,
                         const double *__restrict__ somega, gvs_sph_params prm, double *__restrict__ sax,
                         double *__restrict__ say, double *__restrict__ saz, double *__restrict__ sdu,
                         double *__restrict__ sdivv, double *__restrict__ smaxmu, double *__restrict__ sdalpha) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= tv.n) return;
    sdivv[i] = 0.0;
    smaxmu[i] = 0.0;
    sdalpha[i] = 0.0;
    sax[i] = say[i] = saz[i] = sdu[i] = 0.0;
    if (!gas[i]) return;
    const double DENSITY_FLOOR = 1e-10;
    const double xi = tv.sx[i], yi = tv.sy[i], zi = tv.sz[i];
    const double vxi = svx[i], vyi = svy[i], vzi = svz[i];
    const double hi = sh[i];
    const double rho_i = fmax(srho[i], DENSITY_FLOOR);
    const double p_i = spres[i], u_i = su[i], c_i = scs[i], alpha_i = salpha[i], omega_i = somega[i];
    const double por2_i = rho_i > 0.0 ? p_i / (omega_i * rho_i * rho_i) : 0.0;
    double axa = 0.0, aya = 0.0, aza = 0.0, dua = 0.0, dva = 0.0, mmu = 0.0;
    const uint32_t *row = list + i * (size_t)kmax;
    const int count = CHK(cnt[i] <= (uint32_t)kmax, DERR_BOUNDS) ? (int)cnt[i] : 0;
    for (int k = 0; k < count; ++k) {
        const uint32_t j = row[k];
        if ((size_t)j == i || !CHK_IDX(j, tv.n)) continue;
        const double dx = xi - tv.sx[j], dy = yi - tv.sy[j], dz = zi - tv.sz[j];
        const double r = sqrt(dx * dx + dy * dy + dz * dz);
        const double hj = sh[j];
        const double h_avg = 0.5 * (hi + hj);
        if (r >= 2.0 * hi && r >= 2.0 * hj) continue;
        const double mj = sm[j];
        const double rho_j = fmax(srho[j], DENSITY_FLOOR);
        const double p_j = spres[j], c_j = scs[j], alpha_j = salpha[j], omega_j = somega[j];
        const double dvx = vxi - svx[j], dvy = vyi - svy[j], dvz = vzi - svz[j];
        const double vr = dvx * dx + dvy * dy + dvz * dz;
        double gix, giy, giz, gjx, gjy, gjz, gax, gay, gaz;
        kgrad(dx, dy, dz, r, hi, gix, giy, giz);
        kgrad(dx, dy, dz, r, hj, gjx, gjy, gjz);
        kgrad(dx, dy, dz, r, h_avg, gax, gay, gaz);
        const double por2_j = rho_j > 0.0 ? p_j / (omega_j * rho_j * rho_j) : 0.0;
        double pi_ij = 0.0;
        if (vr < 0.0) {
            const double alpha_avg = 0.5 * (alpha_i + alpha_j);
            const double c_avg = 0.5 * (c_i + c_j);
            const double rho_avg = 0.5 * (rho_i + rho_j);
            const double eta2 = 0.01 * h_avg * h_avg;
            const double mu = h_avg * vr / (r * r + eta2);
            mmu = fmax(mmu, fabs(mu));
            pi_ij = rho_avg > 0.0 ? (-alpha_avg * c_avg * mu + prm.beta_visc * mu * mu) / rho_avg : 0.0;
        }
        axa -= mj * (por2_i * gix + por2_j * gjx + pi_ij * gax);
        aya -= mj * (por2_i * giy + por2_j * gjy + pi_ij * gay);
        aza -= mj * (por2_i * giz + por2_j * gjz + pi_ij * gaz);
        const double vdgi = dvx * gix + dvy * giy + dvz * giz;
        const double vdga = dvx * gax + dvy * gay + dvz * gaz;
        dua += mj * (por2_i * vdgi + 0.5 * pi_ij * vdga);
        dva -= mj * vdgi;
        if (prm.alpha_cond > 0.0) {
            const double u_j = su[j];
            const double rho_sum = rho_i + rho_j;
            if (rho_sum > 0.0) {
                const double rho_avg = 0.5 * rho_sum;
                const double dp = fabs(p_i - p_j);
                const double v_sig_u = sqrt(dp / rho_avg);
                const double abs_gw = kabsgrad(r, h_avg);
                dua += mj * prm.alpha_cond * v_sig_u * (u_i - u_j) / rho_sum * abs_gw;
            }
        }
    }
    sax[i] = axa;
    say[i] = aya;
    saz[i] = aza;
    sdu[i] = dua;
    double dv = 0.0;
    if (rho_i > 0.0) dv = dva / rho_i;
    sdivv[i] = dv;
    smaxmu[i] = mmu;
    const double tau = c_i > 0.0 ? hi / (2.0 * prm.sigma_visc * c_i) : 1e10;
    const double source = fmax(-dv, 0.0) * (prm.alpha_max - alpha_i);
    sdalpha[i] = -(alpha_i - prm.alpha_min) / tau + source;
}


// ---- mixed precision (GVS_PREC_MIXED): f32 pair arithmetic ------------------------------
// Positions and velocities as f32 hi + lo (their f64 value to ~2^-48), so a
// neighbour separation (x_i hi - x_j hi) + (x_i lo - x_j lo) is good to an f32
// ulp of the separation itself.  Pair terms in f32 (explicit FMA), sums in f32
// (hi, lo) with two-sum, kernel constants factored out and applied in f64 per
// target.  The h iteration, Omega, EOS and the per-target epilogues stay f64.
// This translation unit is built without FMA contraction; the f32 code below
// asks for its FMAs explicitly.

__device__ __forceinline__ void tsum(float &hi, float &lo, float v) {
    const float s = __fadd_rn(hi, v);
    const float bp = __fsub_rn(s, hi);
    lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(v, bp)));
    hi = s;
}

__device__ __forceinline__ void split_ff(double v, float &hi, float &lo) {
    hi = __double2float_rn(v);
    lo = __double2float_rn(v - (double)hi);
}

// sources for the mixed density: (x hi, y hi, z hi, m), (x lo, y lo, z lo, 0)
__global__ void k_sph_src_pos(const TreeView tv, const double *__restrict__ sm, float4 *__restrict__ a,
                              float4 *__restrict__ b) {
    const size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= tv.n) return;
    float xh, xl, yh, yl, zh, zl;
    split_ff(tv.sx[j], xh, xl);
    split_ff(tv.sy[j], yh, yl);
    split_ff(tv.sz[j], zh, zl);
    a[j] = make_float4(xh, yh, zh, (float)sm[j]);
    b[j] = make_float4(xl, yl, zl, 0.f);
}

// sources for the mixed forces (after the density pass):
//   c = (vx hi, vy hi, vz hi, 1/h)  d = (vx lo, vy lo, vz lo, -5 norm / h^5)
//   e = (h, max(rho, floor), P / (Omega rho^2), c)  f = (alpha, P, u, m P / (Omega rho^2) K(h))
__global__ void k_sph_src_hydro(size_t n, const double *__restrict__ svx, const double *__restrict__ svy,
                                const double *__restrict__ svz, const double *__restrict__ sh,
                                const double *__restrict__ srho, const double *__restrict__ spres,
                                const double *__restrict__ scs, const double *__restrict__ salpha,
                                const double *__restrict__ somega, const double *__restrict__ su,
                                const double *__restrict__ sm, float4 *__restrict__ c4, float4 *__restrict__ d4,
                                float4 *__restrict__ e4, float4 *__restrict__ f4) {
    const size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    float vxh, vxl, vyh, vyl, vzh, vzl;
    split_ff(svx[j], vxh, vxl);
    split_ff(svy[j], vyh, vyl);
    split_ff(svz[j], vzh, vzl);
    const double h = sh[j];
    const double rho = fmax(srho[j], 1e-10);
    const double p = spres[j];
    const double por2 = rho > 0.0 ? p / (somega[j] * rho * rho) : 0.0;
    const double h2 = h * h;
    const double K = -5.0 * norm3d() / (h2 * h2 * h);
    c4[j] = make_float4(vxh, vyh, vzh, (float)(1.0 / h));
    d4[j] = make_float4(vxl, vyl, vzl, (float)K);
    e4[j] = make_float4((float)h, (float)rho, (float)por2, (float)scs[j]);
    f4[j] = make_float4((float)salpha[j], (float)p, (float)su[j], (float)(sm[j] * por2 * K));
}

// Mixed sums of one density iteration: S1 = sum m f(q), S2 = sum m (5 q^2 s^3 - 3 f(q))
// with f(q) = s^4 (1 + 2q), s = 1 - q/2; rho = norm/h^3 S1, dW/dh sum = norm/h^4 S2.
__device__ __forceinline__ void density_sums_mixed(const float4 *__restrict__ a4, const float4 *__restrict__ b4,
                                                   const uint32_t *row, int count, float4 pa, float4 pb, float ih,
                                                   double &s1, double &s2, size_t n) {
    float h1 = 0.f, l1 = 0.f, h2 = 0.f, l2 = 0.f;
    for (int k = 0; k < count; ++k) {
        const uint32_t j = row[k];
        if (!CHK_IDX(j, n)) continue;
        const float4 a = a4[j], b = b4[j];
        const float dx = __fadd_rn(__fsub_rn(pa.x, a.x), __fsub_rn(pb.x, b.x));
        const float dy = __fadd_rn(__fsub_rn(pa.y, a.y), __fsub_rn(pb.y, b.y));
        const float dz = __fadd_rn(__fsub_rn(pa.z, a.z), __fsub_rn(pb.z, b.z));
        const float d2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
        const float r = __fsqrt_rn(d2);  // correctly rounded: the net SPH force is a small remainder of the pair terms
        const float q = __fmul_rn(r, ih);
        if (q < 2.0f) {
            const float sq = __fmaf_rn(-0.5f, q, 1.0f);
            const float s2q = __fmul_rn(sq, sq), s3 = __fmul_rn(s2q, sq);
            const float f = __fmul_rn(__fmul_rn(s2q, s2q), __fmaf_rn(2.0f, q, 1.0f));
            const float g = __fmaf_rn(5.0f * q * q, s3, -3.0f * f);
            tsum(h1, l1, __fmul_rn(a.w, f));
            tsum(h2, l2, __fmul_rn(a.w, g));
        }
    }
    s1 = (double)h1 + (double)l1;
    s2 = (double)h2 + (double)l2;
}

// compute_density with mixed sums.  The mixed h sequence drifts from the f64
// one by ~3e-8 relative, so a stopping or re-query decision that comes within
// 1e-5 of its threshold (convergence at 1e-3, re-query at a ratio of 1.1) could
// go the other way.  Such a particle is listed for k_density_redo, which runs
// its whole iteration again on the f64 path from the initial h: every
// particle's iteration path is then the f64 one.
__global__ void k_density_mixed(const TreeView tv, const float4 *__restrict__ pos4, const float4 *__restrict__ node4,
                                const int4 *__restrict__ meta4,
                                const float4 *__restrict__ a4, const float4 *__restrict__ b4,
                                const uint8_t *__restrict__ gas, const double *__restrict__ sm,
                                const double *__restrict__ su, double *__restrict__ sh, uint32_t *__restrict__ list,
                                uint32_t *__restrict__ cnt, int kmax, double gamma, double eta, double h_max,
                                double *__restrict__ rho_out, double *__restrict__ omega_out,
                                double *__restrict__ pres, double *__restrict__ cs, unsigned *__restrict__ err,
                                uint32_t *__restrict__ redo_idx, unsigned *__restrict__ redo_count) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= tv.n) return;
    omega_out[i] = 1.0;
    if (!gas[i]) return;
    const double search_padding = 1.1;
    const double xi = tv.sx[i], yi = tv.sy[i], zi = tv.sz[i];
    const float4 pa = a4[i], pb = b4[i];
    const double m_i = sm[i];
    double h = sh[i];
    uint32_t *row = list + i * (size_t)kmax;
    int count = (int)cnt[i];
    double rho_last = rho_out[i];
    bool close = false, requeried = false;
    for (int it = 0; it < 5; ++it) {
        double s1, s2;
        density_sums_mixed(a4, b4, row, count, pa, pb, (float)(1.0 / h), s1, s2, tv.n);
        const double nh3 = norm3d() / (h * h * h);
        const double rho = nh3 * s1, dws = nh3 / h * s2;
        const double h_new = rho > 0.0 ? fmin(eta * cbrt(m_i / rho), h_max) : fmin(h, h_max);
        const double ratio = fabs(h_new - h) / fmax(h, 1e-30);
        close = close || fabs(ratio - 1e-3) < 1e-5 || fabs(h_new / h - search_padding) < 1e-5;
        if (rho > 0.0) {
            const double dh_drho = -h_new / (3.0 * rho);
            double om = 1.0 - dh_drho * dws;
            if (om < 0.1) om = 0.1;
            omega_out[i] = om;
        }
        rho_last = rho;
        sh[i] = h_new;
        if (fabs(h_new - h) / fmax(h, 1e-30) < 1e-3) break;
        const double search_radius = 2.0 * h * search_padding;
        if (2.0 * h_new > search_radius) {
            const double new_radius = 2.0 * h_new * search_padding;
            count = ball_query_thread(tv, pos4, node4, meta4, prefilter_scale(tv), xi, yi, zi, new_radius, row, kmax);
            requeried = true;
            if (count > kmax) {
                atomicOr(err, (unsigned)DERR_NEIGH_OVERFLOW);
                count = kmax;
            }
            cnt[i] = (uint32_t)count;
        }
        h = h_new;
    }
    // the top bit marks a row that no longer holds the original list
    if (close) redo_idx[atomicAdd(redo_count, 1u)] = (uint32_t)i | (requeried ? 0x80000000u : 0u);
    rho_out[i] = rho_last;
    const double u = su[i];
    pres[i] = (gamma - 1.0) * rho_last * u;
    cs[i] = sqrt(gamma * (gamma - 1.0) * fmax(u, 0.0));
}

// The listed particles' h iteration again, from the initial h h0 and the
// original neighbour list (re-queried at radius 2 h0 1.1 when the mixed pass
// had replaced it), with f64 sums.  One warp per particle: the lanes stride the
// list and the partial sums meet in a fixed shuffle tree, so the sums differ
// from the sequential f64 ones only in rounding (~1e-16), far below the 1e-5
// band that sent the particle here; the decisions are the f64 path's.
__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}

__global__ void __launch_bounds__(128) k_density_redo(
    const TreeView tv, const float4 *__restrict__ pos4, const float4 *__restrict__ node4,
    const int4 *__restrict__ meta4, const double *__restrict__ sm, const double *__restrict__ su,
    const double *__restrict__ h0, double *__restrict__ sh, uint32_t *__restrict__ list,
    uint32_t *__restrict__ cnt, int kmax, double gamma, double eta, double h_max, double *__restrict__ rho_out,
    double *__restrict__ omega_out, double *__restrict__ pres, double *__restrict__ cs, unsigned *__restrict__ err,
    const uint32_t *__restrict__ redo_idx, const unsigned *__restrict__ redo_count, unsigned *__restrict__ redo_total) {
    const unsigned m = *redo_count;
    if (blockIdx.x == 0 && threadIdx.x == 0 && m) atomicAdd(redo_total, m);
    const int lane = threadIdx.x & 31;
    const unsigned wpb = blockDim.x >> 5;
    for (unsigned k = blockIdx.x * wpb + (threadIdx.x >> 5); k < m; k += gridDim.x * wpb) {
        const uint32_t code = redo_idx[k];
        const size_t i = code & 0x7FFFFFFFu;
        if (!CHK_IDX(i, tv.n)) continue;  // warp-uniform: the warp reads one entry
        const double xi = tv.sx[i], yi = tv.sy[i], zi = tv.sz[i], m_i = sm[i];
        uint32_t *row = list + i * (size_t)kmax;
        double h = h0[i];
        int count = (int)cnt[i];
        if (code & 0x80000000u) {  // restore the original list
            if (lane == 0) {
                count = ball_query_thread(tv, pos4, node4, meta4, prefilter_scale(tv), xi, yi, zi, 2.0 * h * 1.1,
                                          row, kmax);
                if (count > kmax) {
                    atomicOr(err, (unsigned)DERR_NEIGH_OVERFLOW);
                    count = kmax;
                }
                cnt[i] = (uint32_t)count;
            }
            count = __shfl_sync(0xFFFFFFFFu, count, 0);
            __syncwarp();
        }
        double rho_last = rho_out[i], om_last = 1.0;
        for (int it = 0; it < 5; ++it) {
            double rho = 0.0, dws = 0.0;
            for (int q = lane; q < count; q += 32) {
                const uint32_t j = row[q];
                if (!CHK_IDX(j, tv.n)) continue;
                const double dx = xi - tv.sx[j], dy = yi - tv.sy[j], dz = zi - tv.sz[j];
                const double r = sqrt(dx * dx + dy * dy + dz * dz);
                if (r < 2.0 * h) {
                    rho += sm[j] * kw(r, h);
                    dws += sm[j] * kdwdh(r, h);
                }
            }
            rho = warp_sum(rho);
            dws = warp_sum(dws);
            const double h_new = rho > 0.0 ? fmin(eta * cbrt(m_i / rho), h_max) : fmin(h, h_max);
            if (rho > 0.0) {
                const double dh_drho = -h_new / (3.0 * rho);
                om_last = fmax(1.0 - dh_drho * dws, 0.1);
            }
            rho_last = rho;
            const bool done = fabs(h_new - h) / fmax(h, 1e-30) < 1e-3;
            if (!done && 2.0 * h_new > 2.0 * h * 1.1) {  // re-query at the new radius
                if (lane == 0) {
                    count = ball_query_thread(tv, pos4, node4, meta4, prefilter_scale(tv), xi, yi, zi,
                                              2.0 * h_new * 1.1, row, kmax);
                    if (count > kmax) {
                        atomicOr(err, (unsigned)DERR_NEIGH_OVERFLOW);
                        count = kmax;
                    }
                    cnt[i] = (uint32_t)count;
                }
                count = __shfl_sync(0xFFFFFFFFu, count, 0);
                __syncwarp();
            }
            h = h_new;
            if (done) break;
        }
        if (lane == 0) {
            sh[i] = h;
            omega_out[i] = om_last;
            rho_out[i] = rho_last;
            const double u = su[i];
            pres[i] = (gamma - 1.0) * rho_last * u;
            cs[i] = sqrt(gamma * (gamma - 1.0) * fmax(u, 0.0));
        }
    }
}

// compute_forces (forces.rs:69-232) with f32 pair terms.  With q/r = 1/h the
// kernel gradient is dx * K(h) s^3, K(h) = -5 norm / h^5, and |grad W| =
// -K(h) s^3 r.  The net pressure force is a small remainder of its pair terms,
// so the per-target factors are kept out of the sums and applied in f64:
//   a   = -(P_i/(Omega_i rho_i^2) K_i) sum m_j s_i^3 dx - sum (m P/(Omega rho^2) K)_j s_j^3 dx
//         - sum m_j Pi_ij K_avg s_avg^3 dx
//   du  =  (P_i/(Omega_i rho_i^2) K_i) sum m_j s_i^3 (v.dx) + 1/2 sum m_j Pi_ij K_avg s_avg^3 (v.dx) + cond.
//   div v = -(K_i / rho_i) sum m_j s_i^3 (v.dx)
__global__ void __launch_bounds__(128) k_forces_mixed(
    size_t n, const uint8_t *__restrict__ gas, const uint32_t *__restrict__ list, const uint32_t *__restrict__ cnt,
    int kmax, const float4 *__restrict__ a4, const float4 *__restrict__ b4, const float4 *__restrict__ c4,
    const float4 *__restrict__ d4, const float4 *__restrict__ e4, const float4 *__restrict__ f4,
    const double *__restrict__ sh, const double *__restrict__ srho, const double *__restrict__ scs,
    const double *__restrict__ salpha, const double *__restrict__ spres, const double *__restrict__ somega,
    gvs_sph_params prm, double *__restrict__ sax, double *__restrict__ say,
    double *__restrict__ saz, double *__restrict__ sdu, double *__restrict__ sdivv, double *__restrict__ smaxmu,
    double *__restrict__ sdalpha) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    sdivv[i] = 0.0;
    smaxmu[i] = 0.0;
    sdalpha[i] = 0.0;
    sax[i] = say[i] = saz[i] = sdu[i] = 0.0;
    if (!gas[i]) return;
    const float4 pa = a4[i], pb = b4[i], pc = c4[i], pd = d4[i], pe = e4[i], pf = f4[i];
    const float hi_f = pe.x, ih_i = pc.w, rho_i = pe.y, c_i = pe.w;
    const float alpha_i = pf.x, p_i = pf.y, u_i = pf.z;
    const float beta = (float)prm.beta_visc, acond = (float)prm.alpha_cond;
    const float cnorm5 = (float)(-5.0 * norm3d() * 32.0);  // K(h_avg) = cnorm5 / (hi + hj)^5
    // (hi, lo) sums: A = m s_i^3 dx, B = c_j s_j^3 dx, C = m Pi K_avg s_avg^3 dx (3 components each),
    // D1 = m s_i^3 v.dx, D2 = m Pi K_avg s_avg^3 v.dx, E = conduction
    float sum[12][2];
#pragma unroll
    for (int k = 0; k < 12; ++k) sum[k][0] = sum[k][1] = 0.f;
    float mmu = 0.f;
    const uint32_t *row = list + i * (size_t)kmax;
    const int count = CHK(cnt[i] <= (uint32_t)kmax, DERR_BOUNDS) ? (int)cnt[i] : 0;
    uint32_t jn = count > 0 ? row[0] : 0u;  // the next row entry, read one neighbour ahead
    for (int k = 0; k < count; ++k) {
        const uint32_t j = jn;
        if (k + 1 < count) jn = row[k + 1];
        if ((size_t)j == i || !CHK_IDX(j, n)) continue;
        // all six records at once: one memory round trip per neighbour (the quarter of
        // the rows beyond both radii read theirs for nothing, from cache)
        const float4 a = a4[j], b = b4[j], e = e4[j], c = c4[j], d = d4[j], f = f4[j];
        const float dx = __fadd_rn(__fsub_rn(pa.x, a.x), __fsub_rn(pb.x, b.x));
        const float dy = __fadd_rn(__fsub_rn(pa.y, a.y), __fsub_rn(pb.y, b.y));
        const float dz = __fadd_rn(__fsub_rn(pa.z, a.z), __fsub_rn(pb.z, b.z));
        const float d2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
        const float r = __fsqrt_rn(d2);  // correctly rounded: the net SPH force is a small remainder of the pair terms
        const float hj = e.x;
        if (r >= 2.0f * hi_f && r >= 2.0f * hj) continue;
        const float mj = a.w;
        const float dvx = __fadd_rn(__fsub_rn(pc.x, c.x), __fsub_rn(pd.x, d.x));
        const float dvy = __fadd_rn(__fsub_rn(pc.y, c.y), __fsub_rn(pd.y, d.y));
        const float dvz = __fadd_rn(__fsub_rn(pc.z, c.z), __fsub_rn(pd.z, d.z));
        const float vr = __fmaf_rn(dvz, dz, __fmaf_rn(dvy, dy, __fmul_rn(dvx, dx)));
        // kernel-gradient scalars (gradient = scalar * (dx, dy, dz)); zero at r = 0 or q >= 2
        float si3 = 0.f, sj3 = 0.f, fa = 0.f, sa3 = 0.f, Ka = 0.f;
        const float hsum = __fadd_rn(hi_f, hj);
        const float h_avg = 0.5f * hsum;
        if (r >= 1e-30f) {
            const float qi = __fmul_rn(r, ih_i), qj = __fmul_rn(r, c.w);
            if (qi < 2.0f) { const float s = __fmaf_rn(-0.5f, qi, 1.0f); si3 = __fmul_rn(__fmul_rn(s, s), s); }
            if (qj < 2.0f) { const float s = __fmaf_rn(-0.5f, qj, 1.0f); sj3 = __fmul_rn(__fmul_rn(s, s), s); }
            const float iha = __frcp_rn(h_avg);
            const float qa = __fmul_rn(r, iha);
            if (qa < 2.0f) {
                const float s = __fmaf_rn(-0.5f, qa, 1.0f);
                const float ih = __frcp_rn(hsum), ih2 = __fmul_rn(ih, ih);
                Ka = __fmul_rn(cnorm5, __fmul_rn(__fmul_rn(ih2, ih2), ih));
                sa3 = __fmul_rn(__fmul_rn(s, s), s);
                fa = __fmul_rn(Ka, sa3);
            }
        }
        const float rho_j = e.y, c_j = e.w, alpha_j = f.x, p_j = f.y, u_j = f.z, cw_j = f.w;
        float pi_ij = 0.f;
        if (vr < 0.f) {
            const float alpha_avg = 0.5f * __fadd_rn(alpha_i, alpha_j);
            const float c_avg = 0.5f * __fadd_rn(c_i, c_j);
            const float rho_avg = 0.5f * __fadd_rn(rho_i, rho_j);
            const float eta2 = 0.01f * __fmul_rn(h_avg, h_avg);
            const float mu = __fdiv_rn(__fmul_rn(h_avg, vr), __fadd_rn(d2, eta2));
            mmu = fmaxf(mmu, fabsf(mu));
            if (rho_avg > 0.f)
                pi_ij = __fdiv_rn(__fmaf_rn(beta * mu, mu, -__fmul_rn(__fmul_rn(alpha_avg, c_avg), mu)), rho_avg);
        }
        const float ma = __fmul_rn(mj, si3), mb = __fmul_rn(cw_j, sj3);
        tsum(sum[0][0], sum[0][1], __fmul_rn(ma, dx));
        tsum(sum[1][0], sum[1][1], __fmul_rn(ma, dy));
        tsum(sum[2][0], sum[2][1], __fmul_rn(ma, dz));
        tsum(sum[3][0], sum[3][1], __fmul_rn(mb, dx));
        tsum(sum[4][0], sum[4][1], __fmul_rn(mb, dy));
        tsum(sum[5][0], sum[5][1], __fmul_rn(mb, dz));
        tsum(sum[9][0], sum[9][1], __fmul_rn(ma, vr));
        if (pi_ij != 0.f) {
            const float mc = __fmul_rn(__fmul_rn(mj, pi_ij), fa);
            tsum(sum[6][0], sum[6][1], __fmul_rn(mc, dx));
            tsum(sum[7][0], sum[7][1], __fmul_rn(mc, dy));
            tsum(sum[8][0], sum[8][1], __fmul_rn(mc, dz));
            tsum(sum[10][0], sum[10][1], __fmul_rn(mc, vr));
        }
        if (acond > 0.f) {
            const float rho_sum = __fadd_rn(rho_i, rho_j);
            if (rho_sum > 0.f) {
                const float v_sig = sqrtf(__fdiv_rn(fabsf(__fsub_rn(p_i, p_j)), 0.5f * rho_sum));
                const float abs_gw = -__fmul_rn(__fmul_rn(Ka, sa3), r);
                tsum(sum[11][0], sum[11][1],
                     __fmul_rn(__fmul_rn(mj, acond),
                               __fmul_rn(__fdiv_rn(__fmul_rn(v_sig, __fsub_rn(u_i, u_j)), rho_sum), abs_gw)));
            }
        }
    }
    double S[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) S[k] = (double)sum[k][0] + (double)sum[k][1];
    const double rho_i64 = fmax(srho[i], 1e-10);
    const double hh = sh[i], hh2 = hh * hh;
    const double K_i64 = -5.0 * norm3d() / (hh2 * hh2 * hh);
    const double por2_i64 = rho_i64 > 0.0 ? spres[i] / (somega[i] * rho_i64 * rho_i64) : 0.0;
    const double pk = por2_i64 * K_i64;
    sax[i] = -(pk * S[0] + S[3] + S[6]);
    say[i] = -(pk * S[1] + S[4] + S[7]);
    saz[i] = -(pk * S[2] + S[5] + S[8]);
    sdu[i] = pk * S[9] + 0.5 * S[10] + S[11];
    const double dva = -K_i64 * S[9];
    double dv = 0.0;
    if (rho_i64 > 0.0) dv = dva / rho_i64;
    sdivv[i] = dv;
    smaxmu[i] = (double)mmu;
    const double hi = sh[i], ci = scs[i], al = salpha[i];
    const double tau = ci > 0.0 ? hi / (2.0 * prm.sigma_visc * ci) : 1e10;
    const double source = fmax(-dv, 0.0) * (prm.alpha_max - al);
    sdalpha[i] = -(al - prm.alpha_min) / tau + source;
}

// Sorted results back to caller order; a and du/dt are accumulated.
__global__ void k_scatter_sph(size_t n, const uint32_t *__restrict__ perm, const uint8_t *__restrict__ gas,
                              const double *__restrict__ srho, const double *__restrict__ sh,
                              const double *__restrict__ spres, const double *__restrict__ scs,
                              const double *__restrict__ somega, const double *__restrict__ sax,
                              const double *__restrict__ say, const double *__restrict__ saz,
                              const double *__restrict__ sdu, const double *__restrict__ sdivv,
                              const double *__restrict__ smaxmu, const double *__restrict__ sdalpha,
                              double *__restrict__ rho, double *__restrict__ h, double *__restrict__ pres,
                              double *__restrict__ cs, double *__restrict__ omega, double *__restrict__ ax,
                              double *__restrict__ ay, double *__restrict__ az, double *__restrict__ du,
                              double *__restrict__ divv, double *__restrict__ maxmu, double *__restrict__ dalpha) {
    const size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const uint32_t o = perm[s];
    if (!CHK_IDX(o, n)) return;
    omega[o] = somega[s];
    divv[o] = sdivv[s];
    maxmu[o] = smaxmu[s];
    dalpha[o] = sdalpha[s];
    if (!gas[s]) return;
    rho[o] = srho[s];
    h[o] = sh[s];
    pres[o] = spres[s];
    cs[o] = scs[s];
    ax[o] += sax[s];
    ay[o] += say[s];
    az[o] += saz[s];
    du[o] += sdu[s];
}

// compute_timestep (solver.rs:90-131): per-block minima.
__global__ void k_dt_part(size_t n, const uint8_t *__restrict__ ptype, const double *__restrict__ h,
                          const double *__restrict__ ax, const double *__restrict__ ay, const double *__restrict__ az,
                          const double *__restrict__ cs, const double *__restrict__ alpha,
                          const double *__restrict__ divv, const double *__restrict__ maxmu, gvs_sph_params prm,
                          double *__restrict__ part) {
    double dt_min = INFINITY;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        if (ptype[i] != 4) continue;
        const double hh = h[i];
        const double a_mag = sqrt(ax[i] * ax[i] + ay[i] * ay[i] + az[i] * az[i]);
        if (a_mag > 0.0) dt_min = fmin(dt_min, prm.force_factor * sqrt(hh / a_mag));
        const double c = cs[i];
        const double v_sig = c + hh * fabs(divv[i]) + 1.2 * (alpha[i] * c + prm.beta_visc * maxmu[i]);
        if (v_sig > 0.0) dt_min = fmin(dt_min, prm.cfl_factor * hh / v_sig);
    }
    for (int o = 16; o > 0; o >>= 1) dt_min = fmin(dt_min, __shfl_xor_sync(0xFFFFFFFFu, dt_min, o));
    __shared__ double w[32];
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = dt_min;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = w[0];
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) m = fmin(m, w[k]);
        part[blockIdx.x] = m;
    }
}

// First half of step_with_sph (solver.rs:155-180): v and u half-kicks, drift,
// clear a and du/dt.
__global__ void k_sph_kick1(size_t n, double half_dt, double dt, const uint8_t *__restrict__ ptype,
                            double *__restrict__ x, double *__restrict__ y, double *__restrict__ z,
                            double *__restrict__ vx, double *__restrict__ vy, double *__restrict__ vz,
                            double *__restrict__ ax, double *__restrict__ ay, double *__restrict__ az,
                            double *__restrict__ u, double *__restrict__ du) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v0 = vx[i] + ax[i] * half_dt, v1 = vy[i] + ay[i] * half_dt, v2 = vz[i] + az[i] * half_dt;
    vx[i] = v0; vy[i] = v1; vz[i] = v2;
    if (ptype[i] == 4) {
        double uu = u[i] + du[i] * half_dt;
        if (uu < 1e-10) uu = 1e-10;
        u[i] = uu;
    }
    x[i] = x[i] + v0 * dt;
    y[i] = y[i] + v1 * dt;
    z[i] = z[i] + v2 * dt;
    ax[i] = 0.0; ay[i] = 0.0; az[i] = 0.0;
    du[i] = 0.0;
}

// Second half (solver.rs:188-208): v and u half-kicks, alpha update and clamp.
__global__ void k_sph_kick2(size_t n, double half_dt, double dt, const uint8_t *__restrict__ ptype,
                            double *__restrict__ vx, double *__restrict__ vy, double *__restrict__ vz,
                            const double *__restrict__ ax, const double *__restrict__ ay,
                            const double *__restrict__ az, double *__restrict__ u, const double *__restrict__ du,
                            double *__restrict__ alpha, const double *__restrict__ dalpha, double amin, double amax) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    vx[i] = vx[i] + ax[i] * half_dt;
    vy[i] = vy[i] + ay[i] * half_dt;
    vz[i] = vz[i] + az[i] * half_dt;
    if (ptype[i] == 4) {
        double uu = u[i] + du[i] * half_dt;
        if (uu < 1e-10) uu = 1e-10;
        u[i] = uu;
        double a = alpha[i] + dalpha[i] * dt;
        a = fmin(fmax(a, amin), amax);
        alpha[i] = a;
    }
}

inline int nb(size_t n, int t = 256) { return (int)std::max<size_t>(1, (n + t - 1) / t); }

}  // namespace

void sph_free(Ctx *c) {
    SphState *s = static_cast<SphState *>(c->sph);
    if (!s) return;
    DevBuf *all[] = {&s->list, &s->cnt, &s->gas, &s->sx, &s->sy, &s->sz, &s->svx, &s->svy, &s->svz, &s->sm,
                     &s->sh, &s->su, &s->salpha, &s->srho, &s->spres, &s->scs, &s->somega, &s->sdivv, &s->smaxmu,
                     &s->sdalpha, &s->sax, &s->say, &s->saz, &s->sdu, &s->dtpart, &s->pos4, &s->nrec,
                     &s->a4, &s->b4, &s->c4, &s->d4, &s->e4, &s->f4, &s->redo_idx, &s->redo_count};
    for (DevBuf *b : all)
        if (b->ptr) cudaFree(b->ptr);
    delete s;
    c->sph = nullptr;
}

// Clears one bit of the error word, atomically (other streams may be setting others).
__global__ void k_clear_flag(unsigned *err, unsigned bit) { atomicAnd(err, ~bit); }

// SphSolver::compute (solver.rs:61-80) on the resident state: a and du/dt accumulate.
gvs_status sph_compute(Ctx *c, const gvs_sph_params *prm) {
    const size_t n = c->n;
    if (n == 0) return GVS_OK;
    if (!c->has_gas) return GVS_OK;  // no gas: SPH adds nothing
    SphState *S = sph_of(c);
    TreeView tv;
    GVS_TRY(tree_view(c, &tv));
    cudaStream_t st = c->stream;
    const size_t b8 = n * 8;
    DevBuf *f64s[] = {&S->svx, &S->svy, &S->svz, &S->sm, &S->sh, &S->su, &S->salpha, &S->srho, &S->spres,
                      &S->scs, &S->somega, &S->sdivv, &S->smaxmu, &S->sdalpha, &S->sax, &S->say, &S->saz, &S->sdu};
    for (DevBuf *d : f64s) GVS_CUDA(c, ensure(c, *d, b8));
    GVS_CUDA(c, ensure(c, S->gas, n));
    GVS_CUDA(c, ensure(c, S->cnt, n * 4));
    GVS_CUDA(c, ensure(c, S->pos4, n * 16));
    GVS_CUDA(c, ensure(c, S->nrec, tv.nnodes * 32));
    k_sph_f32copies<<<nb(std::max(n, tv.nnodes)), 256, 0, st>>>(tv, as<float4>(S->pos4), as<float4>(S->nrec),
                                                                as<int4>(S->nrec));
    const bool mixed = prm->precision == GVS_PREC_MIXED;
    if (mixed) {
        DevBuf *f4s[] = {&S->a4, &S->b4, &S->c4, &S->d4, &S->e4, &S->f4};
        for (DevBuf *d : f4s) GVS_CUDA(c, ensure(c, *d, n * 16));
        GVS_CUDA(c, ensure(c, S->redo_idx, n * 4));
        GVS_CUDA(c, ensure(c, S->redo_count, 4));
    }
    k_gather_sph<<<nb(n), 256, 0, st>>>(n, tv.perm, as<uint8_t>(c->ptype), as<double>(c->vx), as<double>(c->vy),
                                        as<double>(c->vz), as<double>(c->m), as<double>(c->h), as<double>(c->u),
                                        as<double>(c->alpha), as<double>(c->rho), as<double>(c->pres),
                                        as<double>(c->cs), as<uint8_t>(S->gas), as<double>(S->svx),
                                        as<double>(S->svy), as<double>(S->svz), as<double>(S->sm),
                                        as<double>(S->sh), as<double>(S->su), as<double>(S->salpha),
                                        as<double>(S->srho), as<double>(S->spres), as<double>(S->scs));
    c->prof.launches += 1;
    GVS_TRY(check_launch(c, "sph gather"));
    // keep a copy of the initial h: the density pass overwrites sh, and an
    // overflow rerun must start again from the same h
    GVS_CUDA(c, ensure(c, c->scratch_b, b8));
    GVS_CUDA(c, cudaMemcpyAsync(c->scratch_b.ptr, S->sh.ptr, b8, cudaMemcpyDeviceToDevice, st));
    if (mixed) {
        k_sph_src_pos<<<nb(n), 256, 0, st>>>(tv, as<double>(S->sm), as<float4>(S->a4), as<float4>(S->b4));
        c->prof.launches += 1;
    }
    for (int attempt = 0; attempt < 4; ++attempt) {
        GVS_CUDA(c, ensure(c, S->list, n * (size_t)S->kmax * 4));
        GVS_CUDA(c, cudaMemcpyAsync(S->sh.ptr, c->scratch_b.ptr, b8, cudaMemcpyDeviceToDevice, st));
        {
            int per_sm = 0;
            GVS_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_neighbors, 128, 0));
            const int blocks = (int)std::min<size_t>(nb(n, 128), (size_t)std::max(1, per_sm) * c->num_sms);
            GVS_CUDA(c, cudaMemsetAsync(err_ptr(c) + EW_NEIGH_WORK, 0, 4, st));
            k_neighbors<<<blocks, 128, 0, st>>>(tv, as<float4>(S->pos4), as<float4>(S->nrec), as<int4>(S->nrec),
                                                as<uint8_t>(S->gas), as<double>(S->sh), 1.1, S->kmax,
                                                as<uint32_t>(S->list), as<uint32_t>(S->cnt), err_ptr(c),
                                                err_ptr(c) + EW_NEIGH_WORK);
        }
        if (mixed) {
            GVS_CUDA(c, cudaMemsetAsync(S->redo_count.ptr, 0, 4, st));
            k_density_mixed<<<nb(n, 128), 128, 0, st>>>(
                tv, as<float4>(S->pos4), as<float4>(S->nrec), as<int4>(S->nrec), as<float4>(S->a4), as<float4>(S->b4),
                as<uint8_t>(S->gas), as<double>(S->sm), as<double>(S->su), as<double>(S->sh), as<uint32_t>(S->list),
                as<uint32_t>(S->cnt), S->kmax, prm->gamma, prm->eta, prm->h_max, as<double>(S->srho),
                as<double>(S->somega), as<double>(S->spres), as<double>(S->scs), err_ptr(c),
                as<uint32_t>(S->redo_idx), as<unsigned>(S->redo_count));
            k_density_redo<<<std::max(1, c->num_sms * 2), 128, 0, st>>>(
                tv, as<float4>(S->pos4), as<float4>(S->nrec), as<int4>(S->nrec), as<double>(S->sm), as<double>(S->su),
                as<double>(c->scratch_b), as<double>(S->sh), as<uint32_t>(S->list), as<uint32_t>(S->cnt), S->kmax,
                prm->gamma, prm->eta, prm->h_max, as<double>(S->srho), as<double>(S->somega), as<double>(S->spres),
                as<double>(S->scs), err_ptr(c), as<uint32_t>(S->redo_idx), as<unsigned>(S->redo_count),
                err_ptr(c) + EW_SPH_REDO);
            c->prof.launches += 1;
        } else
            k_density<<<nb(n, 128), 128, 0, st>>>(tv, as<float4>(S->pos4), as<float4>(S->nrec), as<int4>(S->nrec), as<uint8_t>(S->gas),
                                                  as<double>(S->sm), as<double>(S->su),
                                                  as<double>(S->sh), as<uint32_t>(S->list), as<uint32_t>(S->cnt),
                                                  S->kmax, prm->gamma, prm->eta, prm->h_max, as<double>(S->srho),
                                                  as<double>(S->somega), as<double>(S->spres), as<double>(S->scs),
                                                  err_ptr(c));
        c->prof.launches += 2;
        GVS_TRY(check_launch(c, "sph neighbours/density"));
        unsigned flags = 0;
        GVS_CUDA(c, cudaMemcpyAsync(&flags, c->err_word.ptr, 4, cudaMemcpyDeviceToHost, st));
        GVS_CUDA(c, cudaStreamSynchronize(st));
        if (!(flags & DERR_NEIGH_OVERFLOW)) break;
        // rows too narrow: clear the flag (atomically: gravity may be setting others on
        // the side stream) and rerun with twice the width
        k_clear_flag<<<1, 1, 0, st>>>(err_ptr(c), (unsigned)DERR_NEIGH_OVERFLOW);
        GVS_TRY(check_launch(c, "sph flag clear"));
        if (attempt == 3) return fail(c, GVS_ERR_DEVICE, "SPH neighbour rows overflow at kmax=%d", S->kmax);
        S->kmax *= 2;
    }
    if (mixed) {
        k_sph_src_hydro<<<nb(n), 256, 0, st>>>(n, as<double>(S->svx), as<double>(S->svy), as<double>(S->svz),
                                               as<double>(S->sh), as<double>(S->srho), as<double>(S->spres),
                                               as<double>(S->scs), as<double>(S->salpha), as<double>(S->somega),
                                               as<double>(S->su), as<double>(S->sm), as<float4>(S->c4), as<float4>(S->d4),
                                               as<float4>(S->e4), as<float4>(S->f4));
        k_forces_mixed<<<nb(n, 128), 128, 0, st>>>(
            n, as<uint8_t>(S->gas), as<uint32_t>(S->list), as<uint32_t>(S->cnt), S->kmax, as<float4>(S->a4),
            as<float4>(S->b4), as<float4>(S->c4), as<float4>(S->d4), as<float4>(S->e4), as<float4>(S->f4),
            as<double>(S->sh), as<double>(S->srho), as<double>(S->scs), as<double>(S->salpha), as<double>(S->spres),
            as<double>(S->somega), *prm,
            as<double>(S->sax), as<double>(S->say), as<double>(S->saz), as<double>(S->sdu), as<double>(S->sdivv),
            as<double>(S->smaxmu), as<double>(S->sdalpha));
        c->prof.launches += 1;
    } else {
        k_forces<<<nb(n, 128), 128, 0, st>>>(tv, as<uint8_t>(S->gas), as<uint32_t>(S->list), as<uint32_t>(S->cnt),
                                         S->kmax, as<double>(S->svx), as<double>(S->svy), as<double>(S->svz),
                                         as<double>(S->sm), as<double>(S->sh), as<double>(S->srho),
                                         as<double>(S->spres), as<double>(S->su), as<double>(S->scs),
                                         as<double>(S->salpha), as<double>(S->somega), *prm, as<double>(S->sax),
                                         as<double>(S->say), as<double>(S->saz), as<double>(S->sdu),
                                         as<double>(S->sdivv), as<double>(S->smaxmu), as<double>(S->sdalpha));
    }
    // the SPH accelerations add to gravity's, after them (as the reference's step does)
    if (c->sph_join) GVS_CUDA(c, cudaStreamWaitEvent(st, c->sph_join, 0));
    k_scatter_sph<<<nb(n), 256, 0, st>>>(n, tv.perm, as<uint8_t>(S->gas), as<double>(S->srho), as<double>(S->sh),
                                         as<double>(S->spres), as<double>(S->scs), as<double>(S->somega),
                                         as<double>(S->sax), as<double>(S->say), as<double>(S->saz),
                                         as<double>(S->sdu), as<double>(S->sdivv), as<double>(S->smaxmu),
                                         as<double>(S->sdalpha), as<double>(c->rho), as<double>(c->h),
                                         as<double>(c->pres), as<double>(c->cs), as<double>(c->omega),
                                         as<double>(c->ax), as<double>(c->ay), as<double>(c->az),
                                         as<double>(c->du_dt), as<double>(c->div_v), as<double>(c->max_mu),
                                         as<double>(c->dalpha_dt));
    c->prof.launches += 2;
    S->n = n;
    S->have_intermediates = true;
    return check_launch(c, "sph forces");
}

gvs_status sph_timestep(Ctx *c, const gvs_sph_params *prm, double *dt_out) {
    const size_t n = c->n;
    SphState *S = sph_of(c);
    if (!S->have_intermediates) return fail(c, GVS_ERR_STATE, "compute_timestep needs a prior SPH compute");
    const int nbk = std::max(1, std::min(c->num_sms * 8, nb(n)));  // enough warps to cover the f64 and load latency
    GVS_CUDA(c, ensure(c, S->dtpart, (size_t)nbk * 8));
    k_dt_part<<<nbk, 256, 0, c->stream>>>(n, as<uint8_t>(c->ptype), as<double>(c->h), as<double>(c->ax),
                                          as<double>(c->ay), as<double>(c->az), as<double>(c->cs),
                                          as<double>(c->alpha), as<double>(c->div_v), as<double>(c->max_mu), *prm,
                                          as<double>(S->dtpart));
    c->prof.launches += 1;
    GVS_TRY(check_launch(c, "sph timestep"));
    std::vector<double> part(nbk);
    GVS_CUDA(c, cudaMemcpyAsync(part.data(), S->dtpart.ptr, nbk * 8, cudaMemcpyDeviceToHost, c->stream));
    GVS_CUDA(c, cudaStreamSynchronize(c->stream));
    double m = INFINITY;
    for (double v : part) m = fmin(m, v);
    *dt_out = m < 1e-6 ? 1e-6 : m;  // DT_FLOOR (solver.rs:17,130)
    return GVS_OK;
}

// step_with_sph (solver.rs:145-212) on the resident state; returns dt_next.
gvs_status sph_step(Ctx *c, const gvs_sph_params *prm, int algo, int precision, double eps, double theta, double dt,
                    double *dt_next) {
    const size_t n = c->n;
    if (n == 0) return GVS_OK;
    const double half = 0.5 * dt;
    k_sph_kick1<<<nb(n), 256, 0, c->stream>>>(n, half, dt, as<uint8_t>(c->ptype), as<double>(c->x),
                                              as<double>(c->y), as<double>(c->z), as<double>(c->vx),
                                              as<double>(c->vy), as<double>(c->vz), as<double>(c->ax),
                                              as<double>(c->ay), as<double>(c->az), as<double>(c->u),
                                              as<double>(c->du_dt));
    c->prof.launches += 1;
    c->pos_version++;
    GVS_TRY(check_launch(c, "sph kick/drift"));
    if (c->has_gas && algo != GVS_ALGO_NONE) {
        // Gravity and the SPH pass read the same new positions and tree and write
        // disjoint buffers: gravity runs on the side stream while the neighbour search,
        // density and forces run on the main one, and the SPH scatter waits for gravity
        // before adding its accelerations to gravity's.
        TreeView tv;
        GVS_TRY(tree_view(c, &tv));  // the tree both passes read, built once, on the main stream
        GVS_CUDA(c, cudaEventRecord(c->fork_ev, c->stream));
        GVS_CUDA(c, cudaStreamWaitEvent(c->side, c->fork_ev, 0));
        cudaStream_t main_stream = c->stream;
        c->stream = c->side;
        const gvs_status g = gravity(c, algo, precision, eps, theta, true);
        c->stream = main_stream;
        GVS_CUDA(c, cudaEventRecord(c->join_ev, c->side));
        if (g != GVS_OK) {
            GVS_CUDA(c, cudaStreamWaitEvent(c->stream, c->join_ev, 0));
            return g;
        }
        c->sph_join = c->join_ev;
        const gvs_status s = sph_compute(c, prm);
        c->sph_join = nullptr;
        GVS_CUDA(c, cudaStreamWaitEvent(c->stream, c->join_ev, 0));
        GVS_TRY(s);
    } else {
        GVS_TRY(gravity(c, algo, precision, eps, theta, true));
        GVS_TRY(sph_compute(c, prm));
    }
    k_sph_kick2<<<nb(n), 256, 0, c->stream>>>(n, half, dt, as<uint8_t>(c->ptype), as<double>(c->vx),
                                              as<double>(c->vy), as<double>(c->vz), as<double>(c->ax),
                                              as<double>(c->ay), as<double>(c->az), as<double>(c->u),
                                              as<double>(c->du_dt), as<double>(c->alpha), as<double>(c->dalpha_dt),
                                              prm->alpha_min, prm->alpha_max);
    c->prof.launches += 1;
    GVS_TRY(check_launch(c, "sph kick"));
    c->step_counter++;
    return sph_timestep(c, prm, dt_next);
}

// Neighbour lists in caller indices (for parity tests and callers that want
// the reference's NeighborList): start/count per caller index, indices packed.
gvs_status sph_neighbors_export(Ctx *c, size_t cap, uint32_t *start, uint32_t *count, uint32_t *idx, size_t *total) {
    SphState *S = sph_of(c);
    if (!S->have_intermediates || S->n != c->n) return fail(c, GVS_ERR_STATE, "no SPH neighbour lists yet");
    const size_t n = c->n;
    TreeView tv;
    GVS_TRY(tree_view(c, &tv));
    std::vector<uint32_t> cnt(n), perm(n), rows;
    GVS_CUDA(c, cudaMemcpyAsync(cnt.data(), S->cnt.ptr, n * 4, cudaMemcpyDeviceToHost, c->stream));
    GVS_CUDA(c, cudaMemcpyAsync(perm.data(), tv.perm, n * 4, cudaMemcpyDeviceToHost, c->stream));
    rows.resize(n * (size_t)S->kmax);
    GVS_CUDA(c, cudaMemcpyAsync(rows.data(), S->list.ptr, rows.size() * 4, cudaMemcpyDeviceToHost, c->stream));
    GVS_CUDA(c, cudaStreamSynchronize(c->stream));
    size_t tot = 0;
    for (size_t s = 0; s < n; ++s) tot += cnt[s];
    *total = tot;
    if (cap < tot || !start || !count || !idx) return GVS_OK;
    // caller order: particle o's list follows the caller-index order of particles
    std::vector<uint32_t> slot_of(n);
    for (size_t s = 0; s < n; ++s) slot_of[perm[s]] = (uint32_t)s;
    size_t pos = 0;
    for (size_t o = 0; o < n; ++o) {
        const size_t s = slot_of[o];
        start[o] = (uint32_t)pos;
        count[o] = cnt[s];
        for (uint32_t k = 0; k < cnt[s]; ++k) idx[pos++] = perm[rows[s * (size_t)S->kmax + k]];
    }
    return GVS_OK;
}

GVS_CHECKED_UNIT(sph)

}  // namespace gvs
