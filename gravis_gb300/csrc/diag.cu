// diag.cu -- energy / momentum diagnostics on the resident state
// (Diagnostics::compute and compute_fast, crates/sim-core/src/diagnostics.rs:37-148).
//
// O(N) sums (kinetic, thermal, momentum, angular momentum, centre of mass) are
// f64 block reductions with a fixed block assignment and a fixed final order,
// so repeated calls agree bit for bit.  The O(N^2) softened potential
// U = -sum_{i<j} m_i m_j / sqrt(r_ij^2 + eps^2) is an all-pairs f64 kernel:
// each target i sums j > i in ascending j (the reference's inner loop), and
// the per-target partial sums are added in a fixed tree order.  Up to 16384
// particles the pairs run on a 2D grid of target blocks and source tiles.
#include "gvs_internal.cuh"

#include <atomic>
#include <mutex>

namespace gvs {
namespace {

constexpr int NQ = 17;  // K, th, p[3], L[3], mx[3], mv[3], M, (pad)
constexpr int RNT = 256;

__global__ void __launch_bounds__(RNT) k_sums(size_t n, const double *__restrict__ x, const double *__restrict__ y,
                                              const double *__restrict__ z, const double *__restrict__ vx,
                                              const double *__restrict__ vy, const double *__restrict__ vz,
                                              const double *__restrict__ m, const uint8_t *__restrict__ pt,
                                              const double *__restrict__ u, double *__restrict__ part) {
    double q[NQ];
#pragma unroll
    for (int k = 0; k < NQ; ++k) q[k] = 0.0;
    for (size_t i = (size_t)blockIdx.x * RNT + threadIdx.x; i < n; i += (size_t)gridDim.x * RNT) {
        const double mi = m[i], X = x[i], Y = y[i], Z = z[i], VX = vx[i], VY = vy[i], VZ = vz[i];
        const double v2 = VX * VX + VY * VY + VZ * VZ;
        q[0] += 0.5 * mi * v2;
        if (pt && pt[i] == 4) q[1] += mi * u[i];
        q[2] += mi * VX; q[3] += mi * VY; q[4] += mi * VZ;
        q[5] += mi * (Y * VZ - Z * VY);
        q[6] += mi * (Z * VX - X * VZ);
        q[7] += mi * (X * VY - Y * VX);
        q[8] += mi * X; q[9] += mi * Y; q[10] += mi * Z;
        q[11] += mi * VX; q[12] += mi * VY; q[13] += mi * VZ;
        q[14] += mi;
    }
    __shared__ double s[RNT];
    for (int k = 0; k < NQ; ++k) {
        s[threadIdx.x] = q[k];
        __syncthreads();
        for (int w = RNT / 2; w > 0; w >>= 1) {
            if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) part[blockIdx.x * NQ + k] = s[0];
        __syncthreads();
    }
}

// U partial per target block: target i sums j>i ascending.
__global__ void __launch_bounds__(RNT) k_potential(size_t n, const double *__restrict__ x,
                                                   const double *__restrict__ y, const double *__restrict__ z,
                                                   const double *__restrict__ m, double eps2,
                                                   double *__restrict__ part) {
    __shared__ double4 tile[RNT];
    const size_t i = (size_t)blockIdx.x * RNT + threadIdx.x;
    const bool active = i < n;
    const double xi = active ? x[i] : 0.0, yi = active ? y[i] : 0.0, zi = active ? z[i] : 0.0;
    const double mi = active ? m[i] : 0.0;
    double acc = 0.0;
    const size_t jstart = (size_t)blockIdx.x * RNT;
    for (size_t j0 = jstart; j0 < n; j0 += RNT) {
        __syncthreads();
        const size_t jl = j0 + threadIdx.x;
        if (jl < n) tile[threadIdx.x] = make_double4(x[jl], y[jl], z[jl], m[jl]);
        __syncthreads();
        const int jn = (int)min((size_t)RNT, n - j0);
        for (int jj = 0; jj < jn; ++jj) {
            const size_t j = j0 + jj;
            if (j <= i) continue;
            const double4 q = tile[jj];
            const double dx = q.x - xi, dy = q.y - yi, dz = q.z - zi;
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            acc -= mi * q.w / sqrt(r2);
        }
    }
    __shared__ double s[RNT];
    s[threadIdx.x] = active ? acc : 0.0;
    __syncthreads();
    for (int w = RNT / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

// Small systems: the same pair terms over a 2D grid of (64-target block, 64-source
// tile) so that a thousand particles occupy a hundred SMs instead of four.  Tiles
// wholly below the diagonal (every j <= i) add nothing; each block writes one
// partial, summed on the host in a fixed order.
constexpr int PNT = 64;
constexpr size_t POT2D_MAX = 16384;

__global__ void __launch_bounds__(PNT) k_potential2d(size_t n, const double *__restrict__ x,
                                                     const double *__restrict__ y, const double *__restrict__ z,
                                                     const double *__restrict__ m, double eps2,
                                                     double *__restrict__ part) {
    __shared__ double4 tile[PNT];
    __shared__ double s[PNT];
    const size_t bi = blockIdx.x, bj = blockIdx.y;
    double acc = 0.0;
    if (bj >= bi) {  // whole block takes the same branch
        const size_t i = bi * PNT + threadIdx.x;
        const bool active = i < n;
        const double xi = active ? x[i] : 0.0, yi = active ? y[i] : 0.0, zi = active ? z[i] : 0.0;
        const double mi = active ? m[i] : 0.0;
        const size_t j0 = bj * PNT, jl = j0 + threadIdx.x;
        tile[threadIdx.x] = jl < n ? make_double4(x[jl], y[jl], z[jl], m[jl]) : make_double4(0.0, 0.0, 0.0, 0.0);
        __syncthreads();
        const int jn = (int)min((size_t)PNT, n - j0);
        for (int jj = 0; jj < jn; ++jj) {
            const size_t j = j0 + jj;
            if (j <= i) continue;
            const double4 q = tile[jj];
            const double dx = q.x - xi, dy = q.y - yi, dz = q.z - zi;
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            acc -= mi * q.w / sqrt(r2);
        }
        if (!active) acc = 0.0;
    }
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int w = PNT / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[bi * gridDim.y + bj] = s[0];
}

}  // namespace

gvs_status diagnostics(Ctx *c, double eps, int with_potential, gvs_diag *out) {
    const size_t n = c->n;
    memset(out, 0, sizeof(*out));
    if (n == 0) return GVS_OK;
    const int nb = std::max(1, std::min(c->num_sms * 2, ceil_div((long long)n, RNT)));
    const bool pot2d = n <= POT2D_MAX;
    const int nt2 = ceil_div((long long)n, PNT);
    const int npb = pot2d ? nt2 * nt2 : ceil_div((long long)n, RNT);
    const size_t need = ((size_t)nb * NQ + (with_potential ? (size_t)npb : 0)) * sizeof(double);
    GVS_CUDA(c, ensure(c, c->red_part, need));
    double *part = as<double>(c->red_part);
    k_sums<<<nb, RNT, 0, c->stream>>>(n, as<double>(c->x), as<double>(c->y), as<double>(c->z), as<double>(c->vx),
                                      as<double>(c->vy), as<double>(c->vz), as<double>(c->m),
                                      c->has_gas ? as<uint8_t>(c->ptype) : nullptr, as<double>(c->u), part);
    c->prof.launches += 1;
    GVS_TRY(check_launch(c, "diagnostic sums"));
    if (with_potential) {
        if (pot2d)
            k_potential2d<<<dim3(nt2, nt2), PNT, 0, c->stream>>>(n, as<double>(c->x), as<double>(c->y),
                                                                 as<double>(c->z), as<double>(c->m), eps * eps,
                                                                 part + (size_t)nb * NQ);
        else
            k_potential<<<npb, RNT, 0, c->stream>>>(n, as<double>(c->x), as<double>(c->y), as<double>(c->z),
                                                    as<double>(c->m), eps * eps, part + (size_t)nb * NQ);
        c->prof.launches += 1;
        GVS_TRY(check_launch(c, "potential"));
    }
    std::vector<double> h((size_t)nb * NQ + (with_potential ? (size_t)npb : 0));
    GVS_CUDA(c, cudaMemcpyAsync(h.data(), part, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    GVS_CUDA(c, cudaStreamSynchronize(c->stream));
    double q[NQ] = {0};
    for (int b = 0; b < nb; ++b)
        for (int k = 0; k < NQ; ++k) q[k] += h[(size_t)b * NQ + k];
    double pe = 0.0;
    if (with_potential)
        for (int b = 0; b < npb; ++b) pe += h[(size_t)nb * NQ + b];
    out->kinetic_energy = q[0];
    out->thermal_energy = q[1];
    out->potential_energy = pe;
    out->total_energy = q[0] + pe + q[1];
    for (int d = 0; d < 3; ++d) {
        out->momentum[d] = q[2 + d];
        out->angular_momentum[d] = q[5 + d];
    }
    const double mt = q[14];
    if (mt > 0.0)
        for (int d = 0; d < 3; ++d) {
            out->center_of_mass[d] = q[8 + d] / mt;
            out->center_of_mass_velocity[d] = q[11 + d] / mt;
        }
    out->virial_ratio = fabs(pe) > 0.0 ? 2.0 * q[0] / fabs(pe) : 0.0;
    return GVS_OK;
}

}  // namespace gvs

// ---------------------------------------------------------------------------
// Diagnostics without any allocation (gvs_diagnostics_noalloc).
//
// Some callers cannot allocate device memory: a host that owns every device
// byte through its own allocator (a game or visualisation engine, an ML
// framework's caching allocator, a Rust host with an arena), or a real-time
// loop where an allocation's implicit device synchronisation is not
// acceptable.  For them the reductions below use a
// fixed scratch array that lives in the library image: a file-scope
// __device__ array that every GPU which loads the library holds until the
// process exits.  The caller passes device pointers for the inputs; nothing
// is allocated, freed or resized, on the device or in the library.
// ---------------------------------------------------------------------------
namespace gvs {
namespace {

constexpr size_t NOALLOC_MAX_N = (size_t)1 << 22;    // largest particle count accepted
constexpr int NOALLOC_MAX_SUM_BLOCKS = 1024;          // O(N) reduction blocks
constexpr size_t NOALLOC_SCRATCH_DOUBLES =
    (size_t)NOALLOC_MAX_SUM_BLOCKS * NQ + NOALLOC_MAX_N / RNT + NQ + 1;  // about 270 KB

// Shared by every call on a device; holds the last call's partial sums.
static __device__ __align__(256) double g_diag_scratch[NOALLOC_SCRATCH_DOUBLES];

// Device address of g_diag_scratch and SM count, per device, looked up once per
// device.  The pointer is published (release) after the SM count is written, and
// the look-up runs under a mutex, so host threads making their first call on the
// same device at the same time see a complete set-up.
constexpr int NOALLOC_MAX_DEVICES = 64;
static std::atomic<double *> g_diag_scratch_ptr[NOALLOC_MAX_DEVICES];
static int g_diag_sms[NOALLOC_MAX_DEVICES] = {0};
static std::mutex g_diag_setup_mu;

// Restores the calling thread's current device on every return path.
struct DeviceGuard {
    int saved = -1;
    DeviceGuard() {
        if (cudaGetDevice(&saved) != cudaSuccess) saved = -1;
    }
    ~DeviceGuard() {
        if (saved >= 0) cudaSetDevice(saved);
    }
};

// Adds the partial sums in a fixed order (blocks in order, then potential
// blocks in order), so repeated calls agree bit for bit.  gvs_diagnostics sums
// the potential of small systems over a different block layout, so the two
// entry points agree within f64 rounding (1e-12 relative), not bit for bit.
__global__ void k_sums_final(const double *__restrict__ part, int nb, int npb, double *__restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int k = 0; k < NQ; ++k) {
        double q = 0.0;
        for (int b = 0; b < nb; ++b) q += part[(size_t)b * NQ + k];
        out[k] = q;
    }
    double pe = 0.0;
    for (int b = 0; b < npb; ++b) pe += part[(size_t)nb * NQ + b];
    out[NQ] = pe;
}

}  // namespace
}  // namespace gvs

extern "C" gvs_status gvs_diagnostics_noalloc(int device, void *stream, size_t n, const double *x, const double *y,
                                              const double *z, const double *vx, const double *vy, const double *vz,
                                              const double *mass, const uint8_t *ptype, const double *u,
                                              double softening, int with_potential, gvs_diag *out) {
    using namespace gvs;
    if (!out || !x || !y || !z || !vx || !vy || !vz || !mass || (ptype && !u))
        return fail(nullptr, GVS_ERR_INVALID_ARG, "gvs_diagnostics_noalloc: null pointer");
    if (!(softening >= 0.0)) return fail(nullptr, GVS_ERR_INVALID_ARG, "softening must be >= 0");
    if (n > NOALLOC_MAX_N)
        return fail(nullptr, GVS_ERR_INVALID_ARG,
                    "gvs_diagnostics_noalloc: n = %zu exceeds the fixed scratch limit of %zu particles", n,
                    NOALLOC_MAX_N);
    if (device < 0 || device >= NOALLOC_MAX_DEVICES)
        return fail(nullptr, GVS_ERR_INVALID_ARG, "gvs_diagnostics_noalloc: device %d out of range", device);
    memset(out, 0, sizeof(*out));
    if (n == 0) return GVS_OK;
    DeviceGuard guard;  // the caller's current device is restored on return
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaSetDevice");
    double *part = g_diag_scratch_ptr[device].load(std::memory_order_acquire);
    if (!part) {  // one-time set-up on this device
        std::lock_guard<std::mutex> lock(g_diag_setup_mu);
        part = g_diag_scratch_ptr[device].load(std::memory_order_relaxed);
        if (!part) {
            double *p = nullptr;
            e = cudaGetSymbolAddress((void **)&p, g_diag_scratch);
            if (e != cudaSuccess || !p) return cuda_fail(nullptr, e, "cudaGetSymbolAddress(g_diag_scratch)");
            int sms = 0;
            e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
            if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaDeviceGetAttribute");
            g_diag_sms[device] = sms;
            g_diag_scratch_ptr[device].store(p, std::memory_order_release);
            part = p;
        }
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int nb = std::max(1, std::min(std::min(g_diag_sms[device] * 2, NOALLOC_MAX_SUM_BLOCKS),
                                        ceil_div((long long)n, RNT)));
    const int npb = with_potential ? ceil_div((long long)n, RNT) : 0;
    double *result = part + (size_t)NOALLOC_MAX_SUM_BLOCKS * NQ + NOALLOC_MAX_N / RNT;  // NQ + 1 slots
    // every slot read below is written by this call first, so nothing needs clearing
    k_sums<<<nb, RNT, 0, st>>>(n, x, y, z, vx, vy, vz, mass, ptype, u, part);
    if (with_potential) k_potential<<<npb, RNT, 0, st>>>(n, x, y, z, mass, softening * softening, part + (size_t)nb * NQ);
    k_sums_final<<<1, 32, 0, st>>>(part, nb, npb, result);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "gvs_diagnostics_noalloc launch");
    double q[NQ + 1];
    e = cudaMemcpyAsync(q, result, sizeof q, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "gvs_diagnostics_noalloc result copy");
    const double pe = q[NQ];
    out->kinetic_energy = q[0];
    out->thermal_energy = q[1];
    out->potential_energy = pe;
    out->total_energy = q[0] + pe + q[1];
    for (int d = 0; d < 3; ++d) {
        out->momentum[d] = q[2 + d];
        out->angular_momentum[d] = q[5 + d];
    }
    const double mt = q[14];
    if (mt > 0.0)
        for (int d = 0; d < 3; ++d) {
            out->center_of_mass[d] = q[8 + d] / mt;
            out->center_of_mass_velocity[d] = q[11 + d] / mt;
        }
    out->virial_ratio = fabs(pe) > 0.0 ? 2.0 * q[0] / fabs(pe) : 0.0;
    return GVS_OK;
}
