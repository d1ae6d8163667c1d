// sort.cu -- stable LSD radix sort of (key, u32 value) pairs on the device.
//
// Used to put particles in space-filling-curve order: the direct sum sorts
// 63-bit Hilbert keys so that consecutive particles form compact tiles (the
// tile-centre split of the mixed-precision kernel needs that), and the
// Barnes-Hut build sorts 126-bit octant-path keys (two u64 words, sorted as
// low word then high word) so that the sorted order is the depth-first order
// of the reference octree (crates/sim-core/src/octree.rs:156-239).
//
// Onesweep form (one kernel per 8-bit digit pass, after Adinets and Merrill,
// "Onesweep: a faster least significant digit radix sort for GPUs", 2022):
//  1. one read of the keys counts the digits of every pass (global histograms);
//  2. one tiny launch turns each pass's 256 counts into exclusive offsets;
//  3. per pass, each block takes the next tile index from a counter, counts its
//     tile's digits, publishes the counts, and adds up its predecessors' counts
//     by decoupled look-back (a predecessor publishes its local count first and
//     its inclusive prefix as soon as it knows it); then it scatters its keys
//     stably: in index order within the tile (warp match and per-warp counts).
// A block only waits on tiles that took their index before it did, and so are
// already running; every wait is still bounded: after the cap the block sets
// DERR_SPIN_TIMEOUT, counts the missing tile as empty and carries on.
// 3 + passes launches per sort instead of five per pass.
#include "gvs_internal.cuh"

namespace gvs {

namespace {
constexpr int NT = 256;              // threads per block
constexpr int IPT = 8;               // keys per thread per pass
constexpr int TILE = NT * IPT;       // keys per tile
constexpr int RADIX = 256;
constexpr int NWARP = NT / 32;
constexpr int MAXPASS = 8;
constexpr uint32_t ST_INCL = 1u << 31;   // the tile's inclusive prefix (this digit, tiles 0..t)
constexpr uint32_t ST_LOCAL = 1u << 30;  // only the tile's own count so far
constexpr uint32_t ST_VALUE = ST_LOCAL - 1u;
constexpr unsigned SPIN_CAP = 1u << 22;  // polls of one predecessor's status before giving up

__device__ __forceinline__ uint32_t ld_status(const uint32_t *p) {
    return *reinterpret_cast<const volatile uint32_t *>(p);
}
__device__ __forceinline__ void st_status(uint32_t *p, uint32_t v) { *reinterpret_cast<volatile uint32_t *>(p) = v; }

// Digit counts of every pass in one read of the keys.
template <class K>
__global__ void __launch_bounds__(NT) k_os_hist(const K *__restrict__ keys, size_t n, int begin_bit, int npass,
                                                uint32_t *__restrict__ ghist) {
    __shared__ uint32_t h[MAXPASS][RADIX];
    for (int i = threadIdx.x; i < MAXPASS * RADIX; i += NT) (&h[0][0])[i] = 0u;
    __syncthreads();
    for (size_t i = (size_t)blockIdx.x * NT + threadIdx.x; i < n; i += (size_t)gridDim.x * NT) {
        const K k = keys[i];
        for (int p = 0; p < npass; ++p) atomicAdd(&h[p][(unsigned)(k >> (begin_bit + 8 * p)) & 0xFFu], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < npass * RADIX; i += NT) {
        const uint32_t v = (&h[0][0])[i];
        if (v) atomicAdd(ghist + i, v);
    }
}

// ghist[p][*] -> exclusive offsets, one block of RADIX threads per pass.
__global__ void __launch_bounds__(RADIX) k_os_scan(uint32_t *__restrict__ ghist) {
    __shared__ uint32_t ws[RADIX / 32];
    uint32_t *h = ghist + (size_t)blockIdx.x * RADIX;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const uint32_t v = h[t];
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    uint32_t before = 0;
    for (int k = 0; k < w; ++k) before += ws[k];
    h[t] = before + x - v;
}

template <class K>
__global__ void __launch_bounds__(NT) k_os_pass(const K *__restrict__ keys, const uint32_t *__restrict__ vals,
                                                K *__restrict__ kout, uint32_t *__restrict__ vout, size_t n,
                                                int shift, const uint32_t *__restrict__ gbase,
                                                uint32_t *__restrict__ status, uint32_t *__restrict__ counter,
                                                unsigned *__restrict__ err) {
    __shared__ uint32_t tile_s;
    __shared__ uint32_t base[RADIX];
    __shared__ uint32_t wcnt[NWARP][RADIX];  // per warp: digit counts so far, then the warps' exclusive prefix
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) tile_s = atomicAdd(counter, 1u);
    for (int i = tid; i < NWARP * RADIX; i += NT) (&wcnt[0][0])[i] = 0u;
    __syncthreads();
    const uint32_t tile = tile_s;
    // warp w holds keys [w * 32 IPT, (w + 1) * 32 IPT) of the tile, slice k at lane offsets
    // k * 32: index order is (warp, slice, lane) order, so ranking slice by slice within
    // each warp and then warp by warp keeps the sort stable with no block barrier per slice
    const size_t wbase = (size_t)tile * TILE + (size_t)warp * (32 * IPT);
    K key[IPT];
    unsigned dig[IPT], rank[IPT];
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const size_t idx = wbase + (size_t)k * 32 + lane;
        dig[k] = RADIX;  // out-of-range slots: no digit, never stored
        key[k] = 0;
        if (idx < n) {
            key[k] = keys[idx];
            dig[k] = (unsigned)(key[k] >> shift) & 0xFFu;
        }
    }
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const unsigned d = dig[k];
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
        const unsigned before = d < RADIX ? wcnt[warp][d] : 0u;
        rank[k] = before + __popc(peers & ((1u << lane) - 1u));
        __syncwarp();
        if (d < RADIX && lane == __ffs(peers) - 1) wcnt[warp][d] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // per digit: the tile's count, published, then the prefix of the tiles before it by
    // decoupled look-back; and the warps' exclusive prefix within the tile
    for (int d = tid; d < RADIX; d += NT) {
        uint32_t own = 0;
#pragma unroll
        for (int w = 0; w < NWARP; ++w) {
            const uint32_t c = wcnt[w][d];
            wcnt[w][d] = own;
            own += c;
        }
        uint32_t *mine = status + (size_t)tile * RADIX + d;
        if (tile == 0) {
            st_status(mine, ST_INCL | own);
            base[d] = gbase[d];
            continue;
        }
        st_status(mine, ST_LOCAL | own);
        uint32_t sum = 0;
        for (long t = (long)tile - 1; t >= 0; --t) {
            const uint32_t *p = status + (size_t)t * RADIX + d;
            uint32_t v = 0;
            for (unsigned it = 0; it < SPIN_CAP; ++it) {
                v = ld_status(p);
                if (v & (ST_INCL | ST_LOCAL)) break;
            }
            if (!(v & (ST_INCL | ST_LOCAL))) {
                atomicOr(err, (unsigned)DERR_SPIN_TIMEOUT);
                continue;
            }
            sum += v & ST_VALUE;
            if (v & ST_INCL) break;
        }
        st_status(mine, ST_INCL | (sum + own));
        base[d] = gbase[d] + sum;
    }
    __syncthreads();
    // stable scatter: tile base + earlier warps' count + rank within the warp
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const unsigned d = dig[k];
        if (d < RADIX) {
            const size_t idx = wbase + (size_t)k * 32 + lane;
            const size_t dst = (size_t)base[d] + wcnt[warp][d] + rank[k];
            if (CHK_IDX(dst, n)) {
                kout[dst] = key[k];
                vout[dst] = vals[idx];
            }
        }
    }
}

template <class K>
gvs_status radix_sort_impl(Ctx *c, K *keys, uint32_t *vals, K *keys_alt, uint32_t *vals_alt, size_t n,
                           int begin_bit, int end_bit, K **keys_out, uint32_t **vals_out) {
    K *kin = keys, *kout = keys_alt;
    uint32_t *vin = vals, *vout = vals_alt;
    if (n > 1) {
        if (n >= (size_t)ST_LOCAL) return fail(c, GVS_ERR_INVALID_ARG, "radix sort: n = %zu exceeds 2^30", n);
        const int npass = (end_bit - begin_bit + 7) / 8;
        if (npass > MAXPASS) return fail(c, GVS_ERR_INVALID_ARG, "radix sort: %d passes", npass);
        const size_t ntiles = (n + TILE - 1) / TILE;
        // scratch: histograms [npass][256], tile counters [npass] (padded), status [npass][ntiles][256]
        const size_t words = (size_t)npass * RADIX + 64 + (size_t)npass * ntiles * RADIX;
        GVS_CUDA(c, ensure(c, c->sort_state, words * sizeof(uint32_t)));
        uint32_t *ghist = as<uint32_t>(c->sort_state);
        uint32_t *counters = ghist + (size_t)npass * RADIX;
        uint32_t *status = counters + 64;
        GVS_CUDA(c, cudaMemsetAsync(ghist, 0, words * sizeof(uint32_t), c->stream));
        const int hblocks = (int)std::min<size_t>((n + NT - 1) / NT, (size_t)c->num_sms * 4);
        k_os_hist<K><<<hblocks, NT, 0, c->stream>>>(kin, n, begin_bit, npass, ghist);
        k_os_scan<<<npass, RADIX, 0, c->stream>>>(ghist);
        c->prof.launches += 2;
        for (int p = 0; p < npass; ++p) {
            k_os_pass<K><<<(int)ntiles, NT, 0, c->stream>>>(kin, vin, kout, vout, n, begin_bit + 8 * p,
                                                          ghist + (size_t)p * RADIX, status + (size_t)p * ntiles * RADIX,
                                                          counters + p, err_ptr(c));
            c->prof.launches += 1;
            GVS_TRY(check_launch(c, "radix sort pass"));
            K *tk = kin; kin = kout; kout = tk;
            uint32_t *tv = vin; vin = vout; vout = tv;
        }
    }
    *keys_out = kin;
    *vals_out = vin;
    return GVS_OK;
}

// Exclusive scan of m entries by one block of 1024 threads.
__global__ void __launch_bounds__(1024) k_scan1(uint32_t *a, int m) {
    __shared__ uint32_t part[1024];
    int t = threadIdx.x;
    int per = (m + 1023) / 1024;
    int s = t * per, e = min(m, s + per);
    uint32_t sum = 0;
    for (int i = s; i < e; ++i) sum += a[i];
    part[t] = sum;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        uint32_t v = (t >= off) ? part[t - off] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    uint32_t run = (t == 0) ? 0u : part[t - 1];
    for (int i = s; i < e; ++i) {
        uint32_t v = a[i];
        a[i] = run;
        run += v;
    }
}

__global__ void k_add_u32(uint32_t *a, const uint32_t *b) { a[0] += b[0]; }
}  // namespace

gvs_status radix_sort_u64(Ctx *c, uint64_t *keys, uint32_t *vals, uint64_t *keys_alt, uint32_t *vals_alt, size_t n,
                          int begin_bit, int end_bit, uint64_t **keys_out, uint32_t **vals_out) {
    return radix_sort_impl<uint64_t>(c, keys, vals, keys_alt, vals_alt, n, begin_bit, end_bit, keys_out, vals_out);
}

GVS_CHECKED_UNIT(sort)

}  // namespace gvs

// ---------------------------------------------------------------------------
// exclusive prefix sum of u32 counts (three phases: block sums, one-block scan
// of the block sums, block-local scan plus offset).  out may alias in.
// ---------------------------------------------------------------------------
namespace gvs {
namespace {
constexpr int SCAN_NT = 512;
constexpr int SCAN_IPT = 8;
constexpr int SCAN_TILE = SCAN_NT * SCAN_IPT;

__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *total) {
    __shared__ uint32_t ws[SCAN_NT / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t s = lane < SCAN_NT / 32 ? ws[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xFFFFFFFFu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < SCAN_NT / 32) ws[lane] = s;
    }
    __syncthreads();
    const uint32_t before = (w > 0 ? ws[w - 1] : 0u) + x - v;
    if (total) *total = ws[SCAN_NT / 32 - 1];
    __syncthreads();
    return before;
}

__global__ void __launch_bounds__(SCAN_NT) k_scan_blocksum(const uint32_t *__restrict__ in, size_t n,
                                                           uint32_t *__restrict__ bsum) {
    const size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_IPT;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_IPT; ++k)
        if (base + k < n) s += in[base + k];
    uint32_t tot;
    block_excl_scan(s, &tot);
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(SCAN_NT) k_scan_apply(const uint32_t *in, size_t n, const uint32_t *__restrict__ boff,
                                                        uint32_t *out) {
    const size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_IPT;
    uint32_t v[SCAN_IPT];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_IPT; ++k) {
        v[k] = base + k < n ? in[base + k] : 0u;
        s += v[k];
    }
    uint32_t run = block_excl_scan(s, nullptr) + boff[blockIdx.x];
#pragma unroll
    for (int k = 0; k < SCAN_IPT; ++k)
        if (base + k < n) {
            out[base + k] = run;
            run += v[k];
        }
}
}  // namespace

// out[i] = sum_{k<i} in[i], for i in [0, n); also returns the total in *total_dev[0] (device).
gvs_status exclusive_scan_u32(Ctx *c, const uint32_t *in, uint32_t *out, size_t n, uint32_t *total_dev) {
    if (n == 0) return GVS_OK;
    const int nb = ceil_div((long long)n, SCAN_TILE);
    GVS_CUDA(c, ensure(c, c->sort_hist, ((size_t)nb + 1) * sizeof(uint32_t) * 2));
    uint32_t *bsum = as<uint32_t>(c->sort_hist);
    uint32_t *boff = bsum + nb + 1;
    k_scan_blocksum<<<nb, SCAN_NT, 0, c->stream>>>(in, n, bsum);
    GVS_CUDA(c, cudaMemcpyAsync(boff, bsum, nb * sizeof(uint32_t), cudaMemcpyDeviceToDevice, c->stream));
    k_scan1<<<1, 1024, 0, c->stream>>>(boff, nb);
    k_scan_apply<<<nb, SCAN_NT, 0, c->stream>>>(in, n, boff, out);
    c->prof.launches += 3;
    GVS_TRY(check_launch(c, "exclusive scan"));
    if (total_dev) {
        // total = offset of the last block + its sum
        GVS_CUDA(c, cudaMemcpyAsync(total_dev, boff + nb - 1, sizeof(uint32_t), cudaMemcpyDeviceToDevice, c->stream));
        k_add_u32<<<1, 1, 0, c->stream>>>(total_dev, bsum + nb - 1);
        c->prof.launches += 1;
    }
    return GVS_OK;
}
}  // namespace gvs
