// ensemble.cu -- many independent N-body systems of uneven size in one launch
// (no counterpart in the reference; each system is the reference's direct-sum
// KDK problem: BruteForce, crates/sim-core/src/gravity.rs:47-80, and
// LeapfrogKDK, crates/sim-core/src/integrator.rs:42-76).
//
// The systems are concatenated in the resident state (system s owns caller
// indices [off_s, off_s + N_s)).  Every step:
//   kick+drift over all particles; per-system bounding boxes; 63-bit Hilbert
//   keys in each system's own box; a stable sort by key and then by system
//   (so each system's order is exactly its single-system order); packing into
//   128-particle tiles, each system padded to whole target blocks; ONE
//   persistent launch of the mixed-precision pair kernel over a static list
//   of work items (target block x chunk of source tiles, never crossing
//   systems); a reduce of the chunk partials; the closing half-kick.
// The whole step is captured once into a CUDA graph and replayed.
#include <algorithm>

#include "gvs_internal.cuh"

namespace gvs {

// direct.cu
gvs_status ens_pack(Ctx *c, int ntiles, const uint32_t *map, float4 *pack);
gvs_status ens_pairs(Ctx *c, const float4 *pack, const int4 *items, int nitems, unsigned *counter, float eps2,
                     double *partial, size_t npad, int ntiles, int nsplit);
int ens_tile_float4s();
int ens_tile();
int ens_targets_per_block();

namespace {

constexpr uint32_t PAD = 0x80000000u;
constexpr int CHUNK_TILES = 32;  // source tiles per work item

struct EnsState {
    int nsys = 0;
    size_t n = 0;
    std::vector<long long> off;      // caller-order offsets (nsys + 1)
    std::vector<int> tile_off;       // padded tile offsets (nsys + 1)
    std::vector<int> nsplit;         // source chunks per system
    int ntiles = 0, nitems = 0, max_split = 1;
    size_t npad = 0;
    double eps = 0.0;
    double pairs = 0.0;              // sum over systems of N_i^2 (pair terms of one evaluation)
    DevBuf sys_of, off_dev, nsplit_dev, bb, keys, keys2, perm, perm2, sk, sk2, slot_orig, pslot, items, counter,
        pack, partial;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    double graph_dt = 0.0;
};

EnsState *ens_of(Ctx *c) {
    if (!c->ens) c->ens = new EnsState();
    return static_cast<EnsState *>(c->ens);
}

__global__ void k_sys_bbox(const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z,
                           const long long *__restrict__ off, double *__restrict__ bb) {
    const int s = blockIdx.x;
    const long long a = off[s], b = off[s + 1];
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (long long i = a + threadIdx.x; i < b; i += blockDim.x) {
        const double v[3] = {x[i], y[i], z[i]};
#pragma unroll
        for (int d = 0; d < 3; ++d) { mn[d] = fmin(mn[d], v[d]); mx[d] = fmax(mx[d], v[d]); }
    }
    __shared__ double sh[256][6];
#pragma unroll
    for (int d = 0; d < 3; ++d) { sh[threadIdx.x][d] = mn[d]; sh[threadIdx.x][3 + d] = mx[d]; }
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int d = 0; d < 3; ++d) {
                sh[threadIdx.x][d] = fmin(sh[threadIdx.x][d], sh[threadIdx.x + w][d]);
                sh[threadIdx.x][3 + d] = fmax(sh[threadIdx.x][3 + d], sh[threadIdx.x + w][3 + d]);
            }
        __syncthreads();
    }
    if (threadIdx.x < 6) bb[s * 6 + threadIdx.x] = sh[0][threadIdx.x];
}

__global__ void k_sys_keys(const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z,
                           size_t n, const uint32_t *__restrict__ sys_of, const double *__restrict__ bb,
                           uint64_t *__restrict__ keys, uint32_t *__restrict__ perm) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *b = bb + 6 * sys_of[i];
    const double ext = fmax(fmax(b[3] - b[0], b[4] - b[1]), b[5] - b[2]);
    const double inv = ext > 0.0 ? 2097151.99 / ext : 0.0;
    const double v[3] = {x[i], y[i], z[i]};
    uint32_t q[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) q[d] = (uint32_t)fmin(fmax((v[d] - b[d]) * inv, 0.0), 2097151.0);
    keys[i] = hilbert_key(q[0], q[1], q[2]);
    perm[i] = (uint32_t)i;
}

__global__ void k_iota_u32(uint32_t *a, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = (uint32_t)i;
}

__global__ void k_sys_gather(const uint32_t *__restrict__ perm, const uint32_t *__restrict__ sys_of, size_t n,
                             uint64_t *__restrict__ sk) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const uint32_t j = perm[i];
        sk[i] = CHK_IDX(j, n) ? sys_of[j] : 0;
    }
}

__global__ void k_compose(const uint32_t *__restrict__ p1, const uint32_t *__restrict__ p2, size_t n,
                          uint32_t *__restrict__ out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const uint32_t j = p2[i];
        out[i] = CHK_IDX(j, n) ? p1[j] : 0;
    }
}

__global__ void k_slot_map(const uint32_t *__restrict__ perm, const uint32_t *__restrict__ pslot, size_t n,
                           uint32_t *__restrict__ slot_orig, size_t npad) {
    const size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) {
        const uint32_t d = pslot[s];
        if (CHK_IDX(d, npad)) slot_orig[d] = perm[s];
    }
}

// a = sum over the system's chunks (fixed order), sorted slot -> caller index.
__global__ void k_ens_reduce(const double *__restrict__ partial, size_t npad, size_t n,
                             const uint32_t *__restrict__ perm, const uint32_t *__restrict__ pslot,
                             const uint32_t *__restrict__ sys_sorted_nsplit, double *__restrict__ AX,
                             double *__restrict__ AY, double *__restrict__ AZ) {
    const size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const size_t ps = pslot[s];
    const int ns = (int)sys_sorted_nsplit[s];
    const uint32_t o = perm[s];
    if (!CHK_IDX(ps, npad) || !CHK_IDX(o, n)) return;
    double r[3] = {0, 0, 0};
    for (int k = 0; k < ns; ++k)
#pragma unroll
        for (int c = 0; c < 3; ++c) r[c] += partial[((size_t)k * 3 + c) * npad + ps];
    AX[o] = r[0]; AY[o] = r[1]; AZ[o] = r[2];
}

inline int nb(size_t n) { return (int)std::max<size_t>(1, (n + 255) / 256); }

}  // namespace

void ens_free(Ctx *c) {
    EnsState *E = static_cast<EnsState *>(c->ens);
    if (!E) return;
    if (E->exec) cudaGraphExecDestroy(E->exec);
    if (E->graph) cudaGraphDestroy(E->graph);
    DevBuf *all[] = {&E->sys_of, &E->off_dev, &E->nsplit_dev, &E->bb, &E->keys, &E->keys2, &E->perm, &E->perm2,
                     &E->sk, &E->sk2, &E->slot_orig, &E->pslot, &E->items, &E->counter, &E->pack, &E->partial};
    for (DevBuf *b : all)
        if (b->ptr) cudaFree(b->ptr);
    delete E;
    c->ens = nullptr;
}

// Static layout of the ensemble: tiles, padding, work items.
gvs_status ens_setup(Ctx *c, int nsys, const int64_t *sizes, double eps) {
    ens_free(c);
    EnsState *E = ens_of(c);
    const int TJ = ens_tile(), TPB = ens_targets_per_block(), IPT = TPB / TJ;
    E->nsys = nsys;
    E->n = c->n;
    E->eps = eps;
    E->pairs = 0.0;
    for (int k = 0; k < nsys; ++k) E->pairs += (double)sizes[k] * (double)sizes[k];
    E->off.assign(nsys + 1, 0);
    E->tile_off.assign(nsys + 1, 0);
    E->nsplit.assign(nsys, 1);
    for (int s = 0; s < nsys; ++s) {
        E->off[s + 1] = E->off[s] + sizes[s];
        const int real = (int)((sizes[s] + TJ - 1) / TJ);
        const int padded = (real + IPT - 1) / IPT * IPT;
        E->tile_off[s + 1] = E->tile_off[s] + padded;
        E->nsplit[s] = (real + CHUNK_TILES - 1) / CHUNK_TILES;
        E->max_split = std::max(E->max_split, E->nsplit[s]);
    }
    if ((size_t)E->off[nsys] != c->n)
        return fail(c, GVS_ERR_INVALID_ARG, "ensemble sizes sum to %lld, resident state has %zu particles",
                    E->off[nsys], c->n);
    E->ntiles = E->tile_off[nsys];
    E->npad = (size_t)E->ntiles * TJ;
    // static maps
    std::vector<uint32_t> sys_of(c->n), pslot(c->n), ns_sorted(c->n), slot_orig(E->npad);
    struct Item { int tgt, src, nsrc, split; };
    std::vector<Item> items;
    for (int s = 0; s < nsys; ++s) {
        const long long a = E->off[s], b = E->off[s + 1];
        for (long long i = a; i < b; ++i) {
            sys_of[i] = (uint32_t)s;
            pslot[i] = (uint32_t)((size_t)E->tile_off[s] * TJ + (size_t)(i - a));
            ns_sorted[i] = (uint32_t)E->nsplit[s];
        }
        const size_t p0 = (size_t)E->tile_off[s] * TJ, p1 = (size_t)E->tile_off[s + 1] * TJ;
        for (size_t ps = p0 + (size_t)(b - a); ps < p1; ++ps) slot_orig[ps] = PAD | (uint32_t)a;
        const int real = (int)((b - a + TJ - 1) / TJ);
        for (int blk = E->tile_off[s]; blk < E->tile_off[s + 1]; blk += IPT)
            for (int k = 0; k < E->nsplit[s]; ++k) {
                const int src = E->tile_off[s] + k * CHUNK_TILES;
                items.push_back({blk, src, std::min(CHUNK_TILES, real - k * CHUNK_TILES), k});
            }
    }
    // biggest items first: the persistent CTAs then finish together
    std::stable_sort(items.begin(), items.end(), [](const Item &x, const Item &y) { return x.nsrc > y.nsrc; });
    E->nitems = (int)items.size();
    std::vector<int4> it4(items.size());
    for (size_t k = 0; k < items.size(); ++k) it4[k] = make_int4(items[k].tgt, items[k].src, items[k].nsrc, items[k].split);
    const size_t n = c->n;
    GVS_CUDA(c, ensure(c, E->sys_of, n * 4));
    GVS_CUDA(c, ensure(c, E->off_dev, (nsys + 1) * 8));
    GVS_CUDA(c, ensure(c, E->nsplit_dev, n * 4));
    GVS_CUDA(c, ensure(c, E->bb, (size_t)nsys * 6 * 8));
    GVS_CUDA(c, ensure(c, E->keys, n * 8)); GVS_CUDA(c, ensure(c, E->keys2, n * 8));
    GVS_CUDA(c, ensure(c, E->perm, n * 4)); GVS_CUDA(c, ensure(c, E->perm2, n * 4));
    GVS_CUDA(c, ensure(c, E->sk, n * 8)); GVS_CUDA(c, ensure(c, E->sk2, n * 8));
    GVS_CUDA(c, ensure(c, E->slot_orig, E->npad * 4));
    GVS_CUDA(c, ensure(c, E->pslot, n * 4));
    GVS_CUDA(c, ensure(c, E->items, it4.size() * sizeof(int4)));
    GVS_CUDA(c, ensure(c, E->counter, 16));
    GVS_CUDA(c, ensure(c, E->pack, (size_t)E->ntiles * ens_tile_float4s() * sizeof(float4)));
    GVS_CUDA(c, ensure(c, E->partial, (size_t)E->max_split * 3 * E->npad * sizeof(double)));
    cudaStream_t st = c->stream;
    GVS_CUDA(c, cudaMemcpyAsync(E->sys_of.ptr, sys_of.data(), n * 4, cudaMemcpyHostToDevice, st));
    GVS_CUDA(c, cudaMemcpyAsync(E->off_dev.ptr, E->off.data(), (nsys + 1) * 8, cudaMemcpyHostToDevice, st));
    GVS_CUDA(c, cudaMemcpyAsync(E->nsplit_dev.ptr, ns_sorted.data(), n * 4, cudaMemcpyHostToDevice, st));
    GVS_CUDA(c, cudaMemcpyAsync(E->slot_orig.ptr, slot_orig.data(), E->npad * 4, cudaMemcpyHostToDevice, st));
    GVS_CUDA(c, cudaMemcpyAsync(E->pslot.ptr, pslot.data(), n * 4, cudaMemcpyHostToDevice, st));
    GVS_CUDA(c, cudaMemcpyAsync(E->items.ptr, it4.data(), it4.size() * sizeof(int4), cudaMemcpyHostToDevice, st));
    GVS_CUDA(c, cudaStreamSynchronize(st));
    return GVS_OK;
}

// a = forces within each system (overwrites the resident accelerations).
gvs_status ens_forces(Ctx *c) {
    EnsState *E = ens_of(c);
    const size_t n = c->n;
    cudaStream_t st = c->stream;
    k_sys_bbox<<<E->nsys, 256, 0, st>>>(as<double>(c->x), as<double>(c->y), as<double>(c->z),
                                        as<long long>(E->off_dev), as<double>(E->bb));
    k_sys_keys<<<nb(n), 256, 0, st>>>(as<double>(c->x), as<double>(c->y), as<double>(c->z), n,
                                      as<uint32_t>(E->sys_of), as<double>(E->bb), as<uint64_t>(E->keys),
                                      as<uint32_t>(E->perm));
    c->prof.launches += 2;
    GVS_TRY(check_launch(c, "ensemble keys"));
    uint64_t *ko;
    uint32_t *p1;
    GVS_TRY(radix_sort_u64(c, as<uint64_t>(E->keys), as<uint32_t>(E->perm), as<uint64_t>(E->keys2),
                           as<uint32_t>(E->perm2), n, 0, 64, &ko, &p1));
    // stable sort by system: keys = system of each key-sorted particle, values = key-order slot
    k_sys_gather<<<nb(n), 256, 0, st>>>(p1, as<uint32_t>(E->sys_of), n, as<uint64_t>(E->sk));
    uint32_t *slot = (p1 == as<uint32_t>(E->perm)) ? as<uint32_t>(E->perm2) : as<uint32_t>(E->perm);
    k_iota_u32<<<nb(n), 256, 0, st>>>(slot, n);
    c->prof.launches += 2;
    uint32_t *other = (slot == as<uint32_t>(E->perm)) ? as<uint32_t>(E->perm2) : as<uint32_t>(E->perm);
    // sort the system ids carrying key-order slots; p1 must survive, so it goes through sk2/keys2 scratch
    uint64_t *sko;
    uint32_t *slot_sorted;
    GVS_CUDA(c, ensure(c, c->scratch_a, n * 4));
    GVS_TRY(radix_sort_u64(c, as<uint64_t>(E->sk), slot, as<uint64_t>(E->sk2), as<uint32_t>(c->scratch_a), n, 0,
                           16, &sko, &slot_sorted));
    (void)other;
    uint32_t *final_perm = as<uint32_t>(E->keys2);  // reuse as u32 storage (n * 8 bytes available)
    k_compose<<<nb(n), 256, 0, st>>>(p1, slot_sorted, n, final_perm);
    k_slot_map<<<nb(n), 256, 0, st>>>(final_perm, as<uint32_t>(E->pslot), n, as<uint32_t>(E->slot_orig), E->npad);
    c->prof.launches += 2;
    GVS_TRY(ens_pack(c, E->ntiles, as<uint32_t>(E->slot_orig), as<float4>(E->pack)));
    const float e2 = (float)(E->eps * E->eps);
    int span = -1;  // profile timing span
    GVS_TRY(prof_begin(c, st, &span));
    GVS_TRY(ens_pairs(c, as<float4>(E->pack), as<int4>(E->items), E->nitems, as<unsigned>(E->counter), e2,
                      as<double>(E->partial), E->npad, E->ntiles, E->max_split));
    if (c->prof.on) {  // kernel time of the batched pair kernel
        GVS_TRY(prof_end(c, span, st, &c->prof.force_ms));
        c->prof.force_launches += 1;
        c->prof.force_flops += 20.0 * E->pairs;
    }
    k_ens_reduce<<<nb(n), 256, 0, st>>>(as<double>(E->partial), E->npad, n, final_perm, as<uint32_t>(E->pslot),
                                        as<uint32_t>(E->nsplit_dev), as<double>(c->ax), as<double>(c->ay),
                                        as<double>(c->az));
    c->prof.launches += 1;
    return check_launch(c, "ensemble reduce");
}

gvs_status ens_step(Ctx *c, double dt) {
    const double half = 0.5 * dt;
    GVS_TRY(kick_drift(c, half, dt));
    GVS_TRY(ens_forces(c));
    return kick(c, half);
}

// nsteps KDK steps; with use_graph the step is captured once and replayed.
gvs_status ens_steps(Ctx *c, double dt, long long nsteps, bool use_graph) {
    EnsState *E = ens_of(c);
    if (!use_graph) {
        for (long long s = 0; s < nsteps; ++s) GVS_TRY(ens_step(c, dt));
        return GVS_OK;
    }
    if (!E->exec || E->graph_dt != dt) {
        if (E->exec) { cudaGraphExecDestroy(E->exec); E->exec = nullptr; }
        if (E->graph) { cudaGraphDestroy(E->graph); E->graph = nullptr; }
        // one uncaptured step first: every buffer the step needs is then allocated
        GVS_TRY(ens_step(c, dt));
        --nsteps;
        const bool prof = c->prof.on;
        c->prof.on = false;
        GVS_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        gvs_status stt = ens_step(c, dt);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        c->prof.on = prof;
        if (stt != GVS_OK) { if (g) cudaGraphDestroy(g); return stt; }
        if (e != cudaSuccess) return cuda_fail(c, e, "ensemble graph capture");
        E->graph = g;
        GVS_CUDA(c, cudaGraphInstantiate(&E->exec, E->graph, 0));
        E->graph_dt = dt;
    }
    for (long long s = 0; s < nsteps; ++s) {
        GVS_CUDA(c, cudaGraphLaunch(E->exec, c->stream));
        c->pos_version++;
        c->step_counter++;
    }
    return GVS_OK;
}

GVS_CHECKED_UNIT(ensemble)

}  // namespace gvs

using namespace gvs;

extern "C" gvs_status gvs_ensemble_setup(gvs_ctx *ctx, int nsys, const int64_t *sizes, double softening) {
    Ctx *c = reinterpret_cast<Ctx *>(ctx);
    if (!c) return fail(nullptr, GVS_ERR_INVALID_ARG, "null context");
    if (nsys < 1 || !sizes || !(softening >= 0.0)) return fail(c, GVS_ERR_INVALID_ARG, "bad ensemble arguments");
    for (int s = 0; s < nsys; ++s)
        if (sizes[s] < 1) return fail(c, GVS_ERR_INVALID_ARG, "system %d has no particles", s);
    cudaSetDevice(c->device);
    GVS_TRY(ens_setup(c, nsys, sizes, softening));
    return read_device_errors(c);
}

extern "C" gvs_status gvs_ensemble_forces(gvs_ctx *ctx) {
    Ctx *c = reinterpret_cast<Ctx *>(ctx);
    if (!c) return fail(nullptr, GVS_ERR_INVALID_ARG, "null context");
    if (!c->ens || static_cast<EnsState *>(c->ens)->n != c->n)
        return fail(c, GVS_ERR_STATE, "gvs_ensemble_setup must follow the state upload");
    cudaSetDevice(c->device);
    return ens_forces(c);
}

extern "C" gvs_status gvs_ensemble_kdk_steps(gvs_ctx *ctx, double dt, long long nsteps, int use_graph) {
    Ctx *c = reinterpret_cast<Ctx *>(ctx);
    if (!c) return fail(nullptr, GVS_ERR_INVALID_ARG, "null context");
    if (!(dt > 0.0) || nsteps < 0) return fail(c, GVS_ERR_INVALID_ARG, "dt must be > 0, nsteps >= 0");
    if (!c->ens || static_cast<EnsState *>(c->ens)->n != c->n)
        return fail(c, GVS_ERR_STATE, "gvs_ensemble_setup must follow the state upload");
    cudaSetDevice(c->device);
    if (nsteps == 0) return GVS_OK;
    return ens_steps(c, dt, nsteps, use_graph != 0);
}
