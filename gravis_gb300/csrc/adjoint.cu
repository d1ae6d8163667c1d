// adjoint.cu -- gradients of final-state losses through the leapfrog KDK
// (no counterpart in the reference; the forward map is LeapfrogKDK::step,
// crates/sim-core/src/integrator.rs:42-76, with BruteForce forces).
//
// Forward: nsteps KDK steps from the resident state, storing the f64 state
// (x, v) every `every` steps (and the last one) in HBM.
//
// Backward (reverse mode).  One forward step n is
//   K1: v' = v_n + h/2 a(x_n);  D: x_{n+1} = x_n + h v';  K2: v_{n+1} = v' + h/2 a(x_{n+1}).
// Its adjoint with lx = dL/dx, lv = dL/dv is
//   K2^T: lx += J(x_{n+1})^T (h/2 lv);   D^T: lv += h lx;   K1^T: lx += J(x_n)^T (h/2 lv)
// (J = da/dx; the mass gradient collects the same VJPs through da/dm).  The
// VJPs of K1 of step n and K2 of step n-1 act at the same x_n with the same
// lv, so the sweep does ONE fused force+VJP launch per step, at x_n with
// h lv (h/2 at the two ends).  The states x_n, v_n are recomputed backward by
// leapfrog's time reversibility (v' = v_{n+1} - h/2 a_{n+1}, x_n = x_{n+1} - h v',
// v_n = v' - h/2 a_n) and reset to the stored f64 state at every checkpoint,
// so round-off never accumulates over more than `every` steps.
#include "gvs_internal.cuh"

#include <algorithm>

namespace gvs {

namespace {

struct AdjState {
    size_t n = 0;
    long long nsteps = 0, every = 0, nck = 0;
    int precision = GVS_PREC_MIXED;
    double eps = 0.0, dt = 0.0;
    bool have_forward = false;
    std::vector<char> written;                  // checkpoints present (all after a forward run)
    DevBuf ck;                                  // [nck][6][n] f64 checkpoints (x, y, z, vx, vy, vz)
    DevBuf lx, ly, lz, lvx, lvy, lvz, gm;       // adjoints
    DevBuf vhx, vhy, vhz;                       // v' of the current step
    double fwd_ms = 0.0, bwd_ms = 0.0;          // wall times of the last forward / backward
};

AdjState *adj_of(Ctx *c) {
    if (!c->adj) c->adj = new AdjState();
    return static_cast<AdjState *>(c->adj);
}

__global__ void k_store(size_t n, const double *__restrict__ x, const double *__restrict__ y,
                        const double *__restrict__ z, const double *__restrict__ vx, const double *__restrict__ vy,
                        const double *__restrict__ vz, double *__restrict__ dst) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dst[i] = x[i]; dst[n + i] = y[i]; dst[2 * n + i] = z[i];
    dst[3 * n + i] = vx[i]; dst[4 * n + i] = vy[i]; dst[5 * n + i] = vz[i];
}

__global__ void k_load(size_t n, const double *__restrict__ src, double *__restrict__ x, double *__restrict__ y,
                       double *__restrict__ z, double *__restrict__ vx, double *__restrict__ vy,
                       double *__restrict__ vz, int with_v) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    x[i] = src[i]; y[i] = src[n + i]; z[i] = src[2 * n + i];
    if (with_v) { vx[i] = src[3 * n + i]; vy[i] = src[4 * n + i]; vz[i] = src[5 * n + i]; }
}

// v' = v - h/2 a;  lv += h lx;  x -= h v'
__global__ void k_rev1(size_t n, double half, double dt, double *__restrict__ x, double *__restrict__ y,
                       double *__restrict__ z, const double *__restrict__ vx, const double *__restrict__ vy,
                       const double *__restrict__ vz, const double *__restrict__ ax, const double *__restrict__ ay,
                       const double *__restrict__ az, double *__restrict__ vhx, double *__restrict__ vhy,
                       double *__restrict__ vhz, const double *__restrict__ lx, const double *__restrict__ ly,
                       const double *__restrict__ lz, double *__restrict__ lvx, double *__restrict__ lvy,
                       double *__restrict__ lvz) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double a = vx[i] - half * ax[i], b = vy[i] - half * ay[i], c = vz[i] - half * az[i];
    vhx[i] = a; vhy[i] = b; vhz[i] = c;
    lvx[i] += dt * lx[i]; lvy[i] += dt * ly[i]; lvz[i] += dt * lz[i];
    x[i] -= dt * a; y[i] -= dt * b; z[i] -= dt * c;
}

// v = v' - h/2 a
__global__ void k_rev2(size_t n, double half, const double *__restrict__ vhx, const double *__restrict__ vhy,
                       const double *__restrict__ vhz, const double *__restrict__ ax, const double *__restrict__ ay,
                       const double *__restrict__ az, double *__restrict__ vx, double *__restrict__ vy,
                       double *__restrict__ vz) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    vx[i] = vhx[i] - half * ax[i];
    vy[i] = vhy[i] - half * ay[i];
    vz[i] = vhz[i] - half * az[i];
}

inline int nb(size_t n) { return (int)std::max<size_t>(1, (n + 255) / 256); }

gvs_status store_ck(Ctx *c, AdjState *A, long long slot) {
    const size_t n = c->n;
    k_store<<<nb(n), 256, 0, c->stream>>>(n, as<double>(c->x), as<double>(c->y), as<double>(c->z),
                                          as<double>(c->vx), as<double>(c->vy), as<double>(c->vz),
                                          as<double>(A->ck) + (size_t)slot * 6 * n);
    c->prof.launches += 1;
    return check_launch(c, "checkpoint store");
}

}  // namespace

void adj_free(Ctx *c) {
    AdjState *A = static_cast<AdjState *>(c->adj);
    if (!A) return;
    DevBuf *all[] = {&A->ck, &A->lx, &A->ly, &A->lz, &A->lvx, &A->lvy, &A->lvz, &A->gm, &A->vhx, &A->vhy, &A->vhz};
    for (DevBuf *b : all)
        if (b->ptr) cudaFree(b->ptr);
    delete A;
    c->adj = nullptr;
}

// Checkpoint index of step s: checkpoints hold steps 0, every, 2 every, ..., and nsteps.
static long long ck_slot(const AdjState *A, long long s) {
    if (s == A->nsteps) return A->nck - 1;
    return (s % A->every == 0) ? s / A->every : -1;
}

// The plan of a forward run (sizes, step, forces) and its checkpoint storage, with no
// checkpoint present yet.
static gvs_status adjoint_plan(Ctx *c, AdjState *A, int precision, double eps, double dt, long long nsteps,
                               long long every) {
    const size_t n = c->n;
    A->have_forward = false;
    A->n = n;
    A->nsteps = nsteps;
    A->every = every;
    A->nck = (nsteps + every - 1) / every + 1;
    A->precision = precision;
    A->eps = eps;
    A->dt = dt;
    A->written.assign((size_t)A->nck, 0);
    GVS_CUDA(c, ensure(c, A->ck, (size_t)A->nck * 6 * n * sizeof(double)));
    return GVS_OK;
}

// Step index of checkpoint k (the inverse of ck_slot).
static long long ck_step(const AdjState *A, long long k) { return k == A->nck - 1 ? A->nsteps : k * A->every; }

gvs_status adjoint_forward(Ctx *c, int precision, double eps, double dt, long long nsteps, long long every) {
    AdjState *A = adj_of(c);
    GVS_TRY(adjoint_plan(c, A, precision, eps, dt, nsteps, every));
    GVS_TRY(gravity(c, GVS_ALGO_DIRECT, precision, eps, 0.0, false));  // a(x_0)
    GVS_TRY(store_ck(c, A, 0));
    const double half = 0.5 * dt;
    for (long long s = 1; s <= nsteps; ++s) {
        GVS_TRY(kick_drift(c, half, dt));
        GVS_TRY(gravity(c, GVS_ALGO_DIRECT, precision, eps, 0.0, false));
        GVS_TRY(kick(c, half));
        const long long slot = ck_slot(A, s);
        if (slot >= 0) GVS_TRY(store_ck(c, A, slot));
    }
    std::fill(A->written.begin(), A->written.end(), 1);
    A->have_forward = true;
    return GVS_OK;
}

// dL/d(final x, v) in, dL/d(x0, v0, m) out (device arrays, caller order).  On
// return the resident state is the initial state again.
gvs_status adjoint_backward(Ctx *c, const double *const dl[6], double *const grad[7]) {
    AdjState *A = adj_of(c);
    if (!A->have_forward || A->n != c->n) return fail(c, GVS_ERR_STATE, "adjoint backward needs a forward run");
    const size_t n = c->n, b = n * sizeof(double);
    cudaStream_t st = c->stream;
    DevBuf *bufs[] = {&A->lx, &A->ly, &A->lz, &A->lvx, &A->lvy, &A->lvz, &A->gm, &A->vhx, &A->vhy, &A->vhz};
    for (DevBuf *d : bufs) GVS_CUDA(c, ensure(c, *d, b));
    double *lx = as<double>(A->lx), *ly = as<double>(A->ly), *lz = as<double>(A->lz);
    double *lvx = as<double>(A->lvx), *lvy = as<double>(A->lvy), *lvz = as<double>(A->lvz);
    double *gm = as<double>(A->gm);
    GVS_CUDA(c, cudaMemcpyAsync(lx, dl[0], b, cudaMemcpyDeviceToDevice, st));
    GVS_CUDA(c, cudaMemcpyAsync(ly, dl[1], b, cudaMemcpyDeviceToDevice, st));
    GVS_CUDA(c, cudaMemcpyAsync(lz, dl[2], b, cudaMemcpyDeviceToDevice, st));
    GVS_CUDA(c, cudaMemcpyAsync(lvx, dl[3], b, cudaMemcpyDeviceToDevice, st));
    GVS_CUDA(c, cudaMemcpyAsync(lvy, dl[4], b, cudaMemcpyDeviceToDevice, st));
    GVS_CUDA(c, cudaMemcpyAsync(lvz, dl[5], b, cudaMemcpyDeviceToDevice, st));
    GVS_CUDA(c, cudaMemsetAsync(gm, 0, b, st));
    const double h = A->dt, half = 0.5 * h;
    const int prec = A->precision;
    const double eps = A->eps;
    // the final state (exactly as the forward left it) and K2^T of the last step
    k_load<<<nb(n), 256, 0, st>>>(n, as<double>(A->ck) + (size_t)(A->nck - 1) * 6 * n, as<double>(c->x),
                                  as<double>(c->y), as<double>(c->z), as<double>(c->vx), as<double>(c->vy),
                                  as<double>(c->vz), 1);
    c->pos_version++;
    GVS_TRY(direct_force_vjp(c, prec, eps, lvx, lvy, lvz, half, lx, ly, lz, gm));
    for (long long s = A->nsteps - 1; s >= 0; --s) {
        k_rev1<<<nb(n), 256, 0, st>>>(n, half, h, as<double>(c->x), as<double>(c->y), as<double>(c->z),
                                      as<double>(c->vx), as<double>(c->vy), as<double>(c->vz), as<double>(c->ax),
                                      as<double>(c->ay), as<double>(c->az), as<double>(A->vhx), as<double>(A->vhy),
                                      as<double>(A->vhz), lx, ly, lz, lvx, lvy, lvz);
        c->prof.launches += 1;
        c->pos_version++;
        const long long slot = ck_slot(A, s);
        if (slot >= 0) {  // back on a stored step: exact positions before the VJP
            k_load<<<nb(n), 256, 0, st>>>(n, as<double>(A->ck) + (size_t)slot * 6 * n, as<double>(c->x),
                                          as<double>(c->y), as<double>(c->z), as<double>(c->vx), as<double>(c->vy),
                                          as<double>(c->vz), 0);
            c->prof.launches += 1;
        }
        GVS_TRY(direct_force_vjp(c, prec, eps, lvx, lvy, lvz, s > 0 ? h : half, lx, ly, lz, gm));
        k_rev2<<<nb(n), 256, 0, st>>>(n, half, as<double>(A->vhx), as<double>(A->vhy), as<double>(A->vhz),
                                      as<double>(c->ax), as<double>(c->ay), as<double>(c->az), as<double>(c->vx),
                                      as<double>(c->vy), as<double>(c->vz));
        c->prof.launches += 1;
        if (slot >= 0) {
            k_load<<<nb(n), 256, 0, st>>>(n, as<double>(A->ck) + (size_t)slot * 6 * n, as<double>(c->x),
                                          as<double>(c->y), as<double>(c->z), as<double>(c->vx), as<double>(c->vy),
                                          as<double>(c->vz), 1);
            c->prof.launches += 1;
        }
        GVS_TRY(check_launch(c, "adjoint step"));
    }
    double *dst[7] = {lx, ly, lz, lvx, lvy, lvz, gm};
    for (int k = 0; k < 7; ++k)
        if (grad[k]) GVS_CUDA(c, cudaMemcpyAsync(grad[k], dst[k], b, cudaMemcpyDeviceToDevice, st));
    return GVS_OK;
}

}  // namespace gvs

// ---- C ABI ---------------------------------------------------------------------
using namespace gvs;

extern "C" gvs_status gvs_adjoint_forward(gvs_ctx *ctx, int precision, double softening, double dt,
                                          long long nsteps, long long checkpoint_every) {
    Ctx *c = reinterpret_cast<Ctx *>(ctx);
    if (!c) return fail(nullptr, GVS_ERR_INVALID_ARG, "null context");
    if (precision < GVS_PREC_FP64_EXACT || precision > GVS_PREC_MIXED)
        return fail(c, GVS_ERR_INVALID_ARG, "bad precision %d", precision);
    if (!(softening >= 0.0) || !(dt > 0.0) || nsteps < 1 || checkpoint_every < 1)
        return fail(c, GVS_ERR_INVALID_ARG, "need softening >= 0, dt > 0, nsteps >= 1, checkpoint_every >= 1");
    if (c->n == 0) return fail(c, GVS_ERR_STATE, "no particles");
    cudaSetDevice(c->device);
    GVS_TRY(adjoint_forward(c, precision, softening, dt, nsteps, checkpoint_every));
    GVS_CUDA(c, cudaStreamSynchronize(c->stream));
    return read_device_errors(c);
}

extern "C" gvs_status gvs_adjoint_backward(gvs_ctx *ctx, const double *dl_dx, const double *dl_dy,
                                           const double *dl_dz, const double *dl_dvx, const double *dl_dvy,
                                           const double *dl_dvz, double *g_x, double *g_y, double *g_z,
                                           double *g_vx, double *g_vy, double *g_vz, double *g_m) {
    Ctx *c = reinterpret_cast<Ctx *>(ctx);
    if (!c) return fail(nullptr, GVS_ERR_INVALID_ARG, "null context");
    const size_t n = c->n, b = n * sizeof(double);
    if (n == 0) return fail(c, GVS_ERR_STATE, "no particles");
    cudaSetDevice(c->device);
    AdjState *A = adj_of(c);
    if (!A->have_forward || A->n != n)
        return fail(c, GVS_ERR_STATE,
                    "gvs_adjoint_backward needs gvs_adjoint_forward, or gvs_adjoint_prepare and every checkpoint");
    GVS_CUDA(c, ensure(c, c->scratch_b, 13 * b));
    double *io = as<double>(c->scratch_b);
    const double *in[6] = {dl_dx, dl_dy, dl_dz, dl_dvx, dl_dvy, dl_dvz};
    const double *dl[6];
    for (int k = 0; k < 6; ++k) {
        double *d = io + (size_t)k * n;
        if (in[k]) GVS_CUDA(c, cudaMemcpyAsync(d, in[k], b, cudaMemcpyHostToDevice, c->stream));
        else GVS_CUDA(c, cudaMemsetAsync(d, 0, b, c->stream));
        dl[k] = d;
    }
    double *grad[7];
    for (int k = 0; k < 7; ++k) grad[k] = io + (size_t)(6 + k) * n;
    GVS_TRY(adjoint_backward(c, dl, grad));
    double *out[7] = {g_x, g_y, g_z, g_vx, g_vy, g_vz, g_m};
    for (int k = 0; k < 7; ++k)
        if (out[k]) GVS_CUDA(c, cudaMemcpyAsync(out[k], grad[k], b, cudaMemcpyDeviceToHost, c->stream));
    GVS_CUDA(c, cudaStreamSynchronize(c->stream));
    return read_device_errors(c);
}

// ---- checkpoints in and out --------------------------------------------------------
// The f64 checkpoints of a forward run leave the device (to be written as NBODY003
// snapshots, crates/sim-core/src/snapshot.rs:40-65, by the host) and come back into a
// fresh context, so that the backward sweep can run in another process or after a
// restart and give the same gradients bit for bit.

static gvs_status adj_args(Ctx *c, const char *what) {
    if (!c) return fail(nullptr, GVS_ERR_INVALID_ARG, "null context");
    AdjState *A = static_cast<AdjState *>(c->adj);
    if (!A || A->nck == 0) return fail(c, GVS_ERR_STATE, "%s needs gvs_adjoint_forward or gvs_adjoint_prepare", what);
    if (A->n != c->n)
        return fail(c, GVS_ERR_STATE, "%s: the resident state has %zu particles, the checkpoints %zu", what, c->n, A->n);
    return GVS_OK;
}

extern "C" gvs_status gvs_adjoint_checkpoints(gvs_ctx *ctx, long long cap, long long *count, long long *steps) {
    Ctx *c = reinterpret_cast<Ctx *>(ctx);
    GVS_TRY(adj_args(c, "gvs_adjoint_checkpoints"));
    if (!count) return fail(c, GVS_ERR_INVALID_ARG, "count is NULL");
    const AdjState *A = static_cast<AdjState *>(c->adj);
    *count = A->nck;
    if (steps && cap >= A->nck)
        for (long long k = 0; k < A->nck; ++k) steps[k] = ck_step(A, k);
    return GVS_OK;
}

extern "C" gvs_status gvs_adjoint_prepare(gvs_ctx *ctx, int precision, double softening, double dt, long long nsteps,
                                          long long checkpoint_every) {
    Ctx *c = reinterpret_cast<Ctx *>(ctx);
    if (!c) return fail(nullptr, GVS_ERR_INVALID_ARG, "null context");
    if (precision < GVS_PREC_FP64_EXACT || precision > GVS_PREC_MIXED)
        return fail(c, GVS_ERR_INVALID_ARG, "bad precision %d", precision);
    if (!(softening >= 0.0) || !(dt > 0.0) || nsteps < 1 || checkpoint_every < 1)
        return fail(c, GVS_ERR_INVALID_ARG, "need softening >= 0, dt > 0, nsteps >= 1, checkpoint_every >= 1");
    if (c->n == 0) return fail(c, GVS_ERR_STATE, "no particles");
    cudaSetDevice(c->device);
    return adjoint_plan(c, adj_of(c), precision, softening, dt, nsteps, checkpoint_every);
}

extern "C" gvs_status gvs_adjoint_checkpoint_read(gvs_ctx *ctx, long long k, double *x, double *y, double *z,
                                                  double *vx, double *vy, double *vz) {
    Ctx *c = reinterpret_cast<Ctx *>(ctx);
    GVS_TRY(adj_args(c, "gvs_adjoint_checkpoint_read"));
    AdjState *A = static_cast<AdjState *>(c->adj);
    if (k < 0 || k >= A->nck) return fail(c, GVS_ERR_INVALID_ARG, "checkpoint %lld of %lld", k, A->nck);
    if (!A->written[(size_t)k]) return fail(c, GVS_ERR_STATE, "checkpoint %lld has not been written", k);
    if (!x || !y || !z || !vx || !vy || !vz) return fail(c, GVS_ERR_INVALID_ARG, "null output array");
    cudaSetDevice(c->device);
    const size_t n = A->n, b = n * sizeof(double);
    const double *src = as<double>(A->ck) + (size_t)k * 6 * n;
    double *out[6] = {x, y, z, vx, vy, vz};
    for (int f = 0; f < 6; ++f)
        GVS_CUDA(c, cudaMemcpyAsync(out[f], src + (size_t)f * n, b, cudaMemcpyDeviceToHost, c->stream));
    GVS_CUDA(c, cudaStreamSynchronize(c->stream));
    return GVS_OK;
}

extern "C" gvs_status gvs_adjoint_checkpoint_write(gvs_ctx *ctx, long long k, const double *x, const double *y,
                                                   const double *z, const double *vx, const double *vy,
                                                   const double *vz) {
    Ctx *c = reinterpret_cast<Ctx *>(ctx);
    GVS_TRY(adj_args(c, "gvs_adjoint_checkpoint_write"));
    AdjState *A = static_cast<AdjState *>(c->adj);
    if (k < 0 || k >= A->nck) return fail(c, GVS_ERR_INVALID_ARG, "checkpoint %lld of %lld", k, A->nck);
    if (!x || !y || !z || !vx || !vy || !vz) return fail(c, GVS_ERR_INVALID_ARG, "null input array");
    cudaSetDevice(c->device);
    const size_t n = A->n, b = n * sizeof(double);
    double *dst = as<double>(A->ck) + (size_t)k * 6 * n;
    const double *in[6] = {x, y, z, vx, vy, vz};
    for (int f = 0; f < 6; ++f)
        GVS_CUDA(c, cudaMemcpyAsync(dst + (size_t)f * n, in[f], b, cudaMemcpyHostToDevice, c->stream));
    GVS_CUDA(c, cudaStreamSynchronize(c->stream));
    A->written[(size_t)k] = 1;
    A->have_forward = std::all_of(A->written.begin(), A->written.end(), [](char w) { return w != 0; });
    return GVS_OK;
}
