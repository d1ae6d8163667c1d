// ics_dev.cu -- Plummer initial conditions generated on the device
// (PlummerSphere::generate, crates/sim-core/src/scenarios/plummer_sphere.rs:106-133, with
// sample_plummer_particle, :13-58), from the same ChaCha20 stream as the reference and the
// host generator (ics.cpp), straight into a context's resident state.
//
// The sampler reads a variable number of stream words per particle: 6 (mass fraction,
// cos theta, phi), 4 per attempt of its velocity rejection loop, then 4 (velocity
// direction).  Particle i's first word therefore depends on every earlier particle.  The
// GPU resolves that dependence in parallel:
//  1. the keystream, one 64-byte ChaCha20 block per thread (a budget of 24 words per
//     particle; the mean is 10 + 4 / 0.43 ~ 19.3);
//  2. for every even word offset p, succ(p): where a particle that started at p would
//     end, its rejection loop replayed (most offsets are never a start; that is the
//     price of not knowing which are);
//  3. succ^(2^k) for k < log2(n) by repeated squaring; particle i starts at succ^i(0),
//     composed from the bits of i;
//  4. every particle sampled from its start with the reference's arithmetic (this file
//     compiles without FMA contraction; pow, sin, cos are CUDA's, sqrt is correctly
//     rounded on both sides);
//  5. Particles::shift_to_com_frame (particle.rs:189-226) with fixed-order f64 sums.
// The rejection decision u < g / 0.1 is taken in f32 when u lies more than 1e-5 from
// the f32 ratio (its error is below 1e-6) and in f64 otherwise.  A particle whose f64
// ratio lies within 2^-40 of u -- where CUDA's pow and the C library's could decide
// differently -- fails the call (GVS_ERR_STATE) instead of silently leaving the
// reference's stream; on random inputs that has probability ~1e-12 per attempt.
#include <algorithm>

#include "gvs_internal.cuh"

namespace gvs {

void chacha_key_from_seed(uint64_t seed, uint32_t key[8]);  // ics.cpp

namespace {

constexpr double PI_D = 3.14159265358979323846;
constexpr int MAX_ATTEMPTS = 4096;  // rejection attempts replayed per offset (0.57^4096 ~ 0)
constexpr unsigned F_TIE = 1u, F_BUDGET = 2u;

struct Key {
    uint32_t k[8];
};

__device__ __forceinline__ uint32_t rotl(uint32_t v, int c) { return (v << c) | (v >> (32 - c)); }

// ChaCha20 block b (DJB layout: constants, key, 64-bit block counter, zero stream id;
// 20 rounds; output = state + input), 16 little-endian words per block.
__global__ void k_chacha(Key key, size_t nblocks, uint4 *__restrict__ out) {
    const size_t b = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nblocks) return;
    uint32_t s[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u,
                      key.k[0],    key.k[1],    key.k[2],    key.k[3],
                      key.k[4],    key.k[5],    key.k[6],    key.k[7],
                      (uint32_t)b, (uint32_t)(b >> 32), 0u, 0u};
    uint32_t x[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) x[i] = s[i];
    auto qr = [&](int a, int bb, int c, int d) {
        x[a] += x[bb]; x[d] ^= x[a]; x[d] = rotl(x[d], 16);
        x[c] += x[d]; x[bb] ^= x[c]; x[bb] = rotl(x[bb], 12);
        x[a] += x[bb]; x[d] ^= x[a]; x[d] = rotl(x[d], 8);
        x[c] += x[d]; x[bb] ^= x[c]; x[bb] = rotl(x[bb], 7);
    };
#pragma unroll 1
    for (int r = 0; r < 10; ++r) {
        qr(0, 4, 8, 12); qr(1, 5, 9, 13); qr(2, 6, 10, 14); qr(3, 7, 11, 15);
        qr(0, 5, 10, 15); qr(1, 6, 11, 12); qr(2, 7, 8, 13); qr(3, 4, 9, 14);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
        out[4 * b + q] = make_uint4(x[4 * q] + s[4 * q], x[4 * q + 1] + s[4 * q + 1], x[4 * q + 2] + s[4 * q + 2],
                                    x[4 * q + 3] + s[4 * q + 3]);
}

// rand's draws from two consecutive words (low word first): random::<f64>() and
// random_range(lo..hi) for f64 (the same conversions as ics.cpp).
__device__ __forceinline__ uint64_t word64(const uint32_t *w, uint32_t p) {
    return (uint64_t)w[p] | ((uint64_t)w[p + 1] << 32);
}
__device__ __forceinline__ double draw_uniform(const uint32_t *w, uint32_t p) {
    return (double)(word64(w, p) >> 11) * (1.0 / 9007199254740992.0);
}
__device__ __forceinline__ double draw_range(const uint32_t *w, uint32_t p, double lo, double hi) {
    const double v = __longlong_as_double((long long)((word64(w, p) >> 12) | (1023ull << 52)));
    return (v - 1.0) * (hi - lo) + lo;
}

// The velocity rejection test u < q^2 (1 - q^2)^3.5 / 0.1; *tie is set when the f64
// ratio lies within 2^-40 of u.
__device__ __forceinline__ bool plummer_accept(double qq, double u, bool *tie) {
    const float qf = (float)qq, uf = (float)u;
    const float q2f = qf * qf;
    const float rf = q2f * powf(1.0f - q2f, 3.5f) / 0.1f;
    if (uf < rf - 1e-5f) return true;
    if (uf > rf + 1e-5f) return false;
    const double g = qq * qq * pow(1.0 - qq * qq, 3.5);
    const double r = g / 0.1;
    if (tie && fabs(u - r) <= 0x1p-40 * r) *tie = true;
    return u < r;
}

// succ[h]: the even offset / 2 where a particle starting at word 2h ends; H (= W / 2) when
// it would run past the W words.  succ[H] = H.
__global__ void k_succ(const uint32_t *__restrict__ w, uint32_t W, uint32_t H, uint32_t *__restrict__ succ) {
    const size_t hs = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (hs > H) return;
    const uint32_t h = (uint32_t)hs;
    uint32_t out = H;
    if (h < H) {
        uint32_t p = 2u * h + 6u;  // after the mass fraction, cos theta and phi
        for (int att = 0; att < MAX_ATTEMPTS; ++att) {
            if ((size_t)p + 8 > W) break;  // this attempt and the final direction must fit
            const double qq = draw_range(w, p, 0.0, 1.0), u = draw_uniform(w, p + 2);
            p += 4;
            if (plummer_accept(qq, u, nullptr)) {
                out = (p + 4u) / 2u;
                break;
            }
        }
    }
    succ[h] = out;
}

// next[h] = cur[cur[h]]: jumps of twice as many particles.
__global__ void k_square(const uint32_t *__restrict__ cur, uint32_t H, uint32_t *__restrict__ next) {
    const size_t h = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (h > H) return;
    next[h] = cur[cur[h]];
}

// start[i] = 2 succ^i(0), composed from the bits of i.
__global__ void k_starts(const uint32_t *__restrict__ J, int levels, uint32_t H, size_t n,
                         uint32_t *__restrict__ start, unsigned *__restrict__ flags) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t h = 0;
    for (int k = 0; k < levels; ++k)
        if ((i >> k) & 1) h = J[(size_t)k * (H + 1) + h];
    if (h >= H) {  // the chain left the keystream budget
        atomicOr(flags, F_BUDGET);
        h = 0;
    }
    start[i] = 2u * h;
}

// What is drawn: one Plummer sphere (PlummerSphere::generate), or two spheres of n/2 and
// n - n/2 particles from one stream, offset by -+separation/2 on x and approaching at
// +-vrel/2 (ics.cpp's gvs_ic_collision).
struct Spheres {
    double a;               // scale radius
    double mass_a, mass_b;  // sampler's total mass for particles i < na and i >= na
    double particle_mass;
    size_t na;              // n for one sphere
    double separation, vrel;
    int two;
};

// sample_plummer_particle (plummer_sphere.rs:13-58) from word start[i], as ics.cpp's
// plummer_particle, then the sphere's offset.
__global__ void k_plummer(const uint32_t *__restrict__ w, const uint32_t *__restrict__ start, size_t n, uint32_t W,
                          const Spheres sp, double *__restrict__ x, double *__restrict__ y,
                          double *__restrict__ z, double *__restrict__ vx, double *__restrict__ vy,
                          double *__restrict__ vz, double *__restrict__ m, unsigned *__restrict__ flags) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool first = i < sp.na;
    const double a = sp.a, total_mass = first ? sp.mass_a : sp.mass_b;
    uint32_t p = start[i];
    if ((size_t)p + 14 > W) {  // not even the shortest particle fits: the budget ran out
        atomicOr(flags, F_BUDGET);
        return;
    }
    const double x_mass = draw_range(w, p, 0.001, 1.0);
    const double r = a / sqrt(pow(x_mass, -2.0 / 3.0) - 1.0);
    const double ct = draw_range(w, p + 2, -1.0, 1.0);
    const double st = sqrt(1.0 - ct * ct);
    const double phi = draw_range(w, p + 4, 0.0, 2.0 * PI_D);
    double px = r * st * cos(phi);
    y[i] = r * st * sin(phi);
    z[i] = r * ct;
    const double v_esc = sqrt(2.0 * 1.0 * total_mass / sqrt(r * r + a * a));
    p += 6;
    bool tie = false, done = false;
    double q = 0.0;
    for (int att = 0; att < MAX_ATTEMPTS; ++att) {
        if ((size_t)p + 8 > W) break;  // this attempt and the final direction must fit
        const double qq = draw_range(w, p, 0.0, 1.0), u = draw_uniform(w, p + 2);
        p += 4;
        if (plummer_accept(qq, u, &tie)) {
            q = qq;
            done = true;
            break;
        }
    }
    if (tie) atomicOr(flags, F_TIE);
    if (!done) {  // the budget ran out inside this particle's loop
        atomicOr(flags, F_BUDGET);
        return;
    }
    const double v = q * v_esc;
    const double cv = draw_range(w, p, -1.0, 1.0);
    const double sv = sqrt(1.0 - cv * cv);
    const double pv = draw_range(w, p + 2, 0.0, 2.0 * PI_D);
    double pvx = v * sv * cos(pv);
    vy[i] = v * sv * sin(pv);
    vz[i] = v * cv;
    if (sp.two) {
        px = px + (first ? -0.5 : 0.5) * sp.separation;
        pvx = pvx + (first ? 0.5 : -0.5) * sp.vrel;
    }
    x[i] = px;
    vx[i] = pvx;
    m[i] = sp.particle_mass;
}

// Sums of m, m x, m y, m z, m vx, m vy, m vz: per block in a fixed tree, then the blocks
// in order by one thread.
constexpr int COM_NT = 256;
__global__ void __launch_bounds__(COM_NT) k_com_part(size_t n, const double *__restrict__ x,
                                                     const double *__restrict__ y, const double *__restrict__ z,
                                                     const double *__restrict__ vx, const double *__restrict__ vy,
                                                     const double *__restrict__ vz, const double *__restrict__ m,
                                                     double *__restrict__ part) {
    __shared__ double sh[7][COM_NT];
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};
    for (size_t i = (size_t)blockIdx.x * COM_NT + threadIdx.x; i < n; i += (size_t)gridDim.x * COM_NT) {
        const double mi = m[i];
        acc[0] += mi;
        acc[1] += mi * x[i]; acc[2] += mi * y[i]; acc[3] += mi * z[i];
        acc[4] += mi * vx[i]; acc[5] += mi * vy[i]; acc[6] += mi * vz[i];
    }
#pragma unroll
    for (int k = 0; k < 7; ++k) sh[k][threadIdx.x] = acc[k];
    __syncthreads();
    for (int s = COM_NT / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s)
#pragma unroll
            for (int k = 0; k < 7; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x < 7) part[(size_t)blockIdx.x * 7 + threadIdx.x] = sh[threadIdx.x][0];
}

// The blocks' partial sums in a fixed tree (one block of COM_FINAL threads, nparts <=
// COM_FINAL), then the total mass and the COM position and velocity.
constexpr int COM_FINAL = 1024;
__global__ void __launch_bounds__(COM_FINAL) k_com_final(const double *__restrict__ part, int nparts,
                                                          double *__restrict__ com) {
    __shared__ double sh[COM_FINAL];
    double tot[7];
    for (int k = 0; k < 7; ++k) {
        sh[threadIdx.x] = (int)threadIdx.x < nparts ? part[(size_t)threadIdx.x * 7 + k] : 0.0;
        __syncthreads();
        for (int s = COM_FINAL / 2; s > 0; s >>= 1) {
            if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
            __syncthreads();
        }
        tot[k] = sh[0];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        com[0] = tot[0];
        for (int k = 1; k < 7; ++k) com[k] = tot[0] != 0.0 ? tot[k] / tot[0] : 0.0;
    }
}

__global__ void k_com_shift(size_t n, const double *__restrict__ com, double *__restrict__ x,
                            double *__restrict__ y, double *__restrict__ z, double *__restrict__ vx,
                            double *__restrict__ vy, double *__restrict__ vz) {
    __shared__ double c[7];
    if (threadIdx.x < 7) c[threadIdx.x] = com[threadIdx.x];
    __syncthreads();
    if (c[0] == 0.0) return;  // shift_to_com_frame leaves a massless system alone
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        x[i] -= c[1]; y[i] -= c[2]; z[i] -= c[3];
        vx[i] -= c[4]; vy[i] -= c[5]; vz[i] -= c[6];
    }
}

inline unsigned grid_of(size_t n, int t = 256) { return (unsigned)std::max<size_t>(1, (n + t - 1) / t); }

struct Scratch {
    void *p = nullptr;
    ~Scratch() {
        if (p) cudaFree(p);
    }
};

}  // namespace

// The spheres into the resident state arrays x..m (length n).
static gvs_status ic_spheres_device(Ctx *c, size_t n, uint64_t seed, const Spheres &sph) {
    cudaStream_t st = c->stream;
    Key key;
    chacha_key_from_seed(seed, key.k);
    // keystream budget: 24 words per particle plus slack, whole blocks
    const size_t words = ((24 * n + 4096) + 15) / 16 * 16;
    if (words >= (size_t(1) << 32)) return fail(c, GVS_ERR_INVALID_ARG, "device Plummer ICs: n = %zu too large", n);
    const uint32_t W = (uint32_t)words, H = W / 2;
    int levels = 1;
    while (levels < 63 && (size_t(1) << levels) < n) ++levels;
    const size_t jn = (size_t)levels * (H + 1);
    Scratch sw, sj, ss, sp, sf;
    const int nparts = (int)std::min<size_t>(COM_FINAL, grid_of(n, COM_NT));
    GVS_CUDA(c, cudaMalloc(&sw.p, (size_t)W * 4));
    GVS_CUDA(c, cudaMalloc(&sj.p, jn * 4));
    GVS_CUDA(c, cudaMalloc(&ss.p, n * 4));
    GVS_CUDA(c, cudaMalloc(&sp.p, ((size_t)nparts + 1) * 7 * sizeof(double)));  // partials, then the COM
    GVS_CUDA(c, cudaMalloc(&sf.p, 16));
    GVS_CUDA(c, cudaMemsetAsync(sf.p, 0, 16, st));
    uint32_t *w = static_cast<uint32_t *>(sw.p), *J = static_cast<uint32_t *>(sj.p);
    uint32_t *start = static_cast<uint32_t *>(ss.p);
    unsigned *flags = static_cast<unsigned *>(sf.p);
    k_chacha<<<grid_of(W / 16), 256, 0, st>>>(key, W / 16, reinterpret_cast<uint4 *>(w));
    k_succ<<<grid_of((size_t)H + 1), 256, 0, st>>>(w, W, H, J);
    for (int k = 1; k < levels; ++k)
        k_square<<<grid_of((size_t)H + 1), 256, 0, st>>>(J + (size_t)(k - 1) * (H + 1), H, J + (size_t)k * (H + 1));
    k_starts<<<grid_of(n), 256, 0, st>>>(J, levels, H, n, start, flags);
    double *x = as<double>(c->x), *y = as<double>(c->y), *z = as<double>(c->z);
    double *vx = as<double>(c->vx), *vy = as<double>(c->vy), *vz = as<double>(c->vz), *m = as<double>(c->m);
    k_plummer<<<grid_of(n, 128), 128, 0, st>>>(w, start, n, W, sph, x, y, z, vx, vy, vz, m, flags);
    double *part = static_cast<double *>(sp.p);
    double *com = part + (size_t)nparts * 7;
    k_com_part<<<nparts, COM_NT, 0, st>>>(n, x, y, z, vx, vy, vz, m, part);
    k_com_final<<<1, COM_FINAL, 0, st>>>(part, nparts, com);
    k_com_shift<<<(unsigned)std::min<size_t>(grid_of(n), (size_t)c->num_sms * 8), 256, 0, st>>>(n, com, x, y, z, vx,
                                                                                              vy, vz);
    c->prof.launches += 6 + (levels - 1);
    GVS_TRY(check_launch(c, "device Plummer ICs"));
    unsigned hf = 0;
    GVS_CUDA(c, cudaMemcpyAsync(&hf, flags, 4, cudaMemcpyDeviceToHost, st));
    GVS_CUDA(c, cudaStreamSynchronize(st));
    if (hf & F_BUDGET) return fail(c, GVS_ERR_STATE, "device Plummer ICs: the stream ran past its word budget");
    if (hf & F_TIE)
        return fail(c, GVS_ERR_STATE,
                    "device Plummer ICs: a rejection decision lies within 2^-40 of its threshold; "
                    "generate these ICs on the host (gvs_ic_plummer / gvs_ic_collision)");
    return GVS_OK;
}

gvs_status ic_plummer_device(Ctx *c, size_t n, uint64_t seed, double a, double total_mass) {
    Spheres sp{};
    sp.a = a;
    sp.mass_a = sp.mass_b = total_mass;
    sp.particle_mass = total_mass / (double)n;
    sp.na = n;
    return ic_spheres_device(c, n, seed, sp);
}

// gvs_ic_collision (ics.cpp): the host's constants, computed here the same way.
gvs_status ic_collision_device(Ctx *c, size_t n, uint64_t seed, double separation) {
    Spheres sp{};
    const size_t na = n / 2;
    const double m = 1.0 / (double)n;
    sp.a = 1.0;
    sp.mass_a = (double)na * m;
    sp.mass_b = (double)(n - na) * m;
    sp.particle_mass = m;
    sp.na = na;
    sp.separation = separation;
    sp.vrel = sqrt(2.0 * 1.0 * 1.0 / separation);
    sp.two = 1;
    return ic_spheres_device(c, n, seed, sp);
}

}  // namespace gvs
