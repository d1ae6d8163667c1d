// kdk.cu -- leapfrog kick / drift on the resident f64 state
// (LeapfrogKDK::step, crates/sim-core/src/integrator.rs:42-76).
//
// All updates are f64 with no FMA contraction, so that v += a*dt/2 and
// x += v*dt round exactly as the reference's separate multiply and add do.
// kick_drift fuses the first half-kick with the drift (one pass over
// x, v, a instead of two), which is bit-identical to running them one after
// the other because each element is touched independently.
#include "gvs_internal.cuh"

#include <algorithm>

namespace gvs {
namespace {

__global__ void k_kick(size_t n, double h, const double *__restrict__ ax, const double *__restrict__ ay,
                       const double *__restrict__ az, double *__restrict__ vx, double *__restrict__ vy,
                       double *__restrict__ vz) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        vx[i] = __dadd_rn(vx[i], __dmul_rn(ax[i], h));
        vy[i] = __dadd_rn(vy[i], __dmul_rn(ay[i], h));
        vz[i] = __dadd_rn(vz[i], __dmul_rn(az[i], h));
    }
}

// v += a*h; x += v*dt; a = 0 (the clear_accelerations that precedes the force call).
__global__ void k_kick_drift(size_t n, double h, double dt, double *__restrict__ ax, double *__restrict__ ay,
                             double *__restrict__ az, double *__restrict__ vx, double *__restrict__ vy,
                             double *__restrict__ vz, double *__restrict__ x, double *__restrict__ y,
                             double *__restrict__ z) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        double v0 = __dadd_rn(vx[i], __dmul_rn(ax[i], h));
        double v1 = __dadd_rn(vy[i], __dmul_rn(ay[i], h));
        double v2 = __dadd_rn(vz[i], __dmul_rn(az[i], h));
        vx[i] = v0; vy[i] = v1; vz[i] = v2;
        x[i] = __dadd_rn(x[i], __dmul_rn(v0, dt));
        y[i] = __dadd_rn(y[i], __dmul_rn(v1, dt));
        z[i] = __dadd_rn(z[i], __dmul_rn(v2, dt));
        ax[i] = 0.0; ay[i] = 0.0; az[i] = 0.0;
    }
}

// Whole KDK trajectories of systems of at most 32 particles in one launch
// (one warp, lane i = particle i), with BruteForce's f64 arithmetic and order:
// half-kick, drift, a = sum over j ascending (j != i) of m_j r_ij / (r2 sqrt(r2)),
// half-kick.  Bit-identical to the per-step kernels (and so to the reference),
// without three launches per step: a two-body orbit needs 10^4 steps a period.
constexpr int TINY_MAX = 32;

__global__ void __launch_bounds__(32) k_kdk_tiny_exact(int n, long long nsteps, double h, double dt, double eps2,
                                                        double *__restrict__ X, double *__restrict__ Y,
                                                        double *__restrict__ Z, double *__restrict__ VX,
                                                        double *__restrict__ VY, double *__restrict__ VZ,
                                                        double *__restrict__ AX, double *__restrict__ AY,
                                                        double *__restrict__ AZ, const double *__restrict__ M) {
    __shared__ double sx[TINY_MAX], sy[TINY_MAX], sz[TINY_MAX], sm[TINY_MAX];
    const int i = threadIdx.x;
    const bool on = i < n;
    double x = 0, y = 0, z = 0, vx = 0, vy = 0, vz = 0, ax = 0, ay = 0, az = 0;
    if (on) {
        x = X[i]; y = Y[i]; z = Z[i]; vx = VX[i]; vy = VY[i]; vz = VZ[i]; ax = AX[i]; ay = AY[i]; az = AZ[i];
        sm[i] = M[i];
    }
    for (long long s = 0; s < nsteps; ++s) {
        vx = __dadd_rn(vx, __dmul_rn(ax, h));
        vy = __dadd_rn(vy, __dmul_rn(ay, h));
        vz = __dadd_rn(vz, __dmul_rn(az, h));
        x = __dadd_rn(x, __dmul_rn(vx, dt));
        y = __dadd_rn(y, __dmul_rn(vy, dt));
        z = __dadd_rn(z, __dmul_rn(vz, dt));
        __syncwarp();  // every lane is done reading the previous step's positions
        if (on) { sx[i] = x; sy[i] = y; sz[i] = z; }
        __syncwarp();
        double fx = 0.0, fy = 0.0, fz = 0.0;
        for (int j = 0; j < n; ++j) {
            if (j == i) continue;
            const double dx = __dsub_rn(sx[j], x), dy = __dsub_rn(sy[j], y), dz = __dsub_rn(sz[j], z);
            const double r2 = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)),
                                        eps2);
            const double f = __dmul_rn(sm[j], __ddiv_rn(1.0, __dmul_rn(r2, __dsqrt_rn(r2))));
            fx = __dadd_rn(fx, __dmul_rn(f, dx));
            fy = __dadd_rn(fy, __dmul_rn(f, dy));
            fz = __dadd_rn(fz, __dmul_rn(f, dz));
        }
        ax = fx; ay = fy; az = fz;
        vx = __dadd_rn(vx, __dmul_rn(ax, h));
        vy = __dadd_rn(vy, __dmul_rn(ay, h));
        vz = __dadd_rn(vz, __dmul_rn(az, h));
    }
    if (on) {
        X[i] = x; Y[i] = y; Z[i] = z; VX[i] = vx; VY[i] = vy; VZ[i] = vz; AX[i] = ax; AY[i] = ay; AZ[i] = az;
    }
}

int grid_for(Ctx *c, size_t n) {
    long long b = ((long long)n + 255) / 256;
    long long cap = (long long)c->num_sms * 8;
    return (int)std::max(1LL, std::min(b, cap));
}

}  // namespace

gvs_status kick(Ctx *c, double half_dt) {
    if (c->n == 0) return GVS_OK;
    k_kick<<<grid_for(c, c->n), 256, 0, c->stream>>>(c->n, half_dt, as<double>(c->ax), as<double>(c->ay),
                                                     as<double>(c->az), as<double>(c->vx), as<double>(c->vy),
                                                     as<double>(c->vz));
    c->prof.launches += 1;
    return check_launch(c, "kick");
}

gvs_status kick_drift(Ctx *c, double half_dt, double dt) {
    if (c->n == 0) return GVS_OK;
    c->pos_version++;
    k_kick_drift<<<grid_for(c, c->n), 256, 0, c->stream>>>(
        c->n, half_dt, dt, as<double>(c->ax), as<double>(c->ay), as<double>(c->az), as<double>(c->vx),
        as<double>(c->vy), as<double>(c->vz), as<double>(c->x), as<double>(c->y), as<double>(c->z));
    c->prof.launches += 1;
    return check_launch(c, "kick_drift");
}

bool kdk_tiny_eligible(const Ctx *c) { return c->n >= 1 && c->n <= (size_t)TINY_MAX; }

gvs_status kdk_tiny_exact(Ctx *c, double eps, double dt, long long nsteps) {
    if (!kdk_tiny_eligible(c)) return fail(c, GVS_ERR_STATE, "kdk_tiny_exact: n = %zu", c->n);
    constexpr long long CHUNK = 1LL << 20;  // steps per launch (well under a second each)
    for (long long s = 0; s < nsteps; s += CHUNK) {
        const long long k = std::min(CHUNK, nsteps - s);
        c->pos_version++;
        k_kdk_tiny_exact<<<1, 32, 0, c->stream>>>((int)c->n, k, 0.5 * dt, dt, eps * eps, as<double>(c->x),
                                                  as<double>(c->y), as<double>(c->z), as<double>(c->vx),
                                                  as<double>(c->vy), as<double>(c->vz), as<double>(c->ax),
                                                  as<double>(c->ay), as<double>(c->az), as<double>(c->m));
        c->prof.launches += 1;
        GVS_TRY(check_launch(c, "kdk_tiny_exact"));
    }
    c->step_counter += nsteps;
    return GVS_OK;
}

gvs_status clear_acc(Ctx *c) {
    if (c->n == 0) return GVS_OK;
    GVS_CUDA(c, cudaMemsetAsync(c->ax.ptr, 0, c->n * sizeof(double), c->stream));
    GVS_CUDA(c, cudaMemsetAsync(c->ay.ptr, 0, c->n * sizeof(double), c->stream));
    GVS_CUDA(c, cudaMemsetAsync(c->az.ptr, 0, c->n * sizeof(double), c->stream));
    return GVS_OK;
}

}  // namespace gvs
