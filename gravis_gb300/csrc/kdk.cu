// kdk.cu -- leapfrog kick / drift on the resident f64 state
// (LeapfrogKDK::step, crates/sim-core/src/integrator.rs:42-76).
//
// All updates are f64 with no FMA contraction, so that v += a*dt/2 and
// x += v*dt round exactly as the reference's separate multiply and add do.
// kick_drift fuses the first half-kick with the drift (one pass over
// x, v, a instead of two), which is bit-identical to running them one after
// the other because each element is touched independently.
#include "gvs_internal.cuh"

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

gvs_status clear_acc(Ctx *c) {
    if (c->n == 0) return GVS_OK;
    GVS_CUDA(c, cudaMemsetAsync(c->ax.ptr, 0, c->n * sizeof(double), c->stream));
    GVS_CUDA(c, cudaMemsetAsync(c->ay.ptr, 0, c->n * sizeof(double), c->stream));
    GVS_CUDA(c, cudaMemsetAsync(c->az.ptr, 0, c->n * sizeof(double), c->stream));
    return GVS_OK;
}

}  // namespace gvs
