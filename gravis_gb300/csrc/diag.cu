// diag.cu -- energy / momentum diagnostics on the resident state
// (Diagnostics::compute and compute_fast, crates/sim-core/src/diagnostics.rs:37-148).
//
// O(N) sums (kinetic, thermal, momentum, angular momentum, centre of mass) are
// f64 block reductions with a fixed block assignment and a fixed final order,
// so repeated calls agree bit for bit.  The O(N^2) softened potential
// U = -sum_{i<j} m_i m_j / sqrt(r_ij^2 + eps^2) is an all-pairs f64 kernel:
// each target i sums j > i in ascending j (the reference's inner loop), and
// the per-target partial sums are added in a fixed tree order.
#include "gvs_internal.cuh"

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

}  // namespace

gvs_status diagnostics(Ctx *c, double eps, int with_potential, gvs_diag *out) {
    const size_t n = c->n;
    memset(out, 0, sizeof(*out));
    if (n == 0) return GVS_OK;
    const int nb = std::max(1, std::min(c->num_sms * 2, ceil_div((long long)n, RNT)));
    const int npb = ceil_div((long long)n, RNT);
    const size_t need = ((size_t)nb * NQ + (with_potential ? (size_t)npb : 0)) * sizeof(double);
    GVS_CUDA(c, ensure(c, c->red_part, need));
    double *part = as<double>(c->red_part);
    k_sums<<<nb, RNT, 0, c->stream>>>(n, as<double>(c->x), as<double>(c->y), as<double>(c->z), as<double>(c->vx),
                                      as<double>(c->vy), as<double>(c->vz), as<double>(c->m),
                                      c->has_gas ? as<uint8_t>(c->ptype) : nullptr, as<double>(c->u), part);
    c->prof.launches += 1;
    GVS_TRY(check_launch(c, "diagnostic sums"));
    if (with_potential) {
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
