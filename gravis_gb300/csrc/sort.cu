// sort.cu -- stable LSD radix sort of (key, u32 value) pairs on the device.
//
// Used to put particles in space-filling-curve order: the direct sum sorts
// 63-bit Hilbert keys so that consecutive particles form compact tiles (the
// tile-centre split of the mixed-precision kernel needs that), and the
// Barnes-Hut build sorts 126-bit octant-path keys (two u64 words, sorted as
// low word then high word) so that the sorted order is the depth-first order
// of the reference octree (crates/sim-core/src/octree.rs:156-239).
//
// One pass per 8-bit digit: (1) per-block digit histograms, (2) one exclusive
// scan over the [digit][block] table, (3) a stable scatter in which each block
// ranks its keys in index order with warp match/ballot and per-warp counters.
#include "gvs_internal.cuh"

namespace gvs {

namespace {
constexpr int NT = 256;              // threads per block
constexpr int IPT = 16;              // keys per thread per pass
constexpr int TILE = NT * IPT;       // keys per block
constexpr int RADIX = 256;
constexpr int NWARP = NT / 32;

template <class K>
__global__ void __launch_bounds__(NT) k_hist(const K *__restrict__ keys, size_t n, int shift,
                                             uint32_t *__restrict__ hist, int nblocks) {
    __shared__ uint32_t h[RADIX];
    for (int i = threadIdx.x; i < RADIX; i += NT) h[i] = 0;
    __syncthreads();
    size_t base = (size_t)blockIdx.x * TILE;
#pragma unroll 4
    for (int k = 0; k < IPT; ++k) {
        size_t idx = base + (size_t)k * NT + threadIdx.x;
        if (idx < n) atomicAdd(&h[(unsigned)(keys[idx] >> shift) & 0xFFu], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < RADIX; i += NT) hist[(size_t)i * nblocks + blockIdx.x] = h[i];
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

template <class K>
__global__ void __launch_bounds__(NT) k_scatter(const K *__restrict__ keys, const uint32_t *__restrict__ vals,
                                                K *__restrict__ kout, uint32_t *__restrict__ vout, size_t n,
                                                int shift, const uint32_t *__restrict__ hist, int nblocks) {
    __shared__ uint32_t base[RADIX];
    __shared__ uint32_t wcnt[NWARP][RADIX];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i < RADIX; i += NT) base[i] = hist[(size_t)i * nblocks + blockIdx.x];
    const size_t tbase = (size_t)blockIdx.x * TILE;
    for (int k = 0; k < IPT; ++k) {
        for (int i = tid; i < NWARP * RADIX; i += NT) (&wcnt[0][0])[i] = 0u;
        __syncthreads();
        const size_t idx = tbase + (size_t)k * NT + tid;
        const bool valid = idx < n;
        K key = 0;
        unsigned d = 256u;  // out-of-range lanes form their own group
        if (valid) {
            key = keys[idx];
            d = (unsigned)(key >> shift) & 0xFFu;
        }
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
        const unsigned rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && lane == __ffs(peers) - 1) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t off = base[d];
            for (int w = 0; w < warp; ++w) off += wcnt[w][d];
            const size_t dst = (size_t)off + rank;
            kout[dst] = key;
            vout[dst] = vals[idx];
        }
        __syncthreads();
        for (int dd = tid; dd < RADIX; dd += NT) {
            uint32_t s = 0;
#pragma unroll
            for (int w = 0; w < NWARP; ++w) s += wcnt[w][dd];
            base[dd] += s;
        }
        __syncthreads();
    }
}

}  // namespace

// In-place exclusive scan of m counts; bsum holds ceil(m / 4096) + 1 words of scratch.
void scan_counts_inplace(Ctx *c, uint32_t *a, size_t m, uint32_t *bsum);

namespace {
template <class K>
gvs_status radix_sort_impl(Ctx *c, K *keys, uint32_t *vals, K *keys_alt, uint32_t *vals_alt, size_t n,
                           int begin_bit, int end_bit, K **keys_out, uint32_t **vals_out) {
    K *kin = keys, *kout = keys_alt;
    uint32_t *vin = vals, *vout = vals_alt;
    if (n > 1) {
        const int nblocks = ceil_div((long long)n, TILE);
        const size_t m = (size_t)RADIX * nblocks;
        GVS_CUDA(c, ensure(c, c->sort_hist, (m + m / 1024 + 64) * sizeof(uint32_t)));
        uint32_t *hist = as<uint32_t>(c->sort_hist);
        uint32_t *bsum = hist + m;
        for (int bit = begin_bit; bit < end_bit; bit += 8) {
            k_hist<K><<<nblocks, NT, 0, c->stream>>>(kin, n, bit, hist, nblocks);
            scan_counts_inplace(c, hist, m, bsum);
            k_scatter<K><<<nblocks, NT, 0, c->stream>>>(kin, vin, kout, vout, n, bit, hist, nblocks);
            c->prof.launches += 2;
            GVS_TRY(check_launch(c, "radix sort pass"));
            K *tk = kin; kin = kout; kout = tk;
            uint32_t *tv = vin; vin = vout; vout = tv;
        }
    }
    *keys_out = kin;
    *vals_out = vin;
    return GVS_OK;
}
}  // namespace

gvs_status radix_sort_u64(Ctx *c, uint64_t *keys, uint32_t *vals, uint64_t *keys_alt, uint32_t *vals_alt, size_t n,
                          int begin_bit, int end_bit, uint64_t **keys_out, uint32_t **vals_out) {
    return radix_sort_impl<uint64_t>(c, keys, vals, keys_alt, vals_alt, n, begin_bit, end_bit, keys_out, vals_out);
}

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

// Three launches, each wide: block sums, one-block scan of the (few) block sums,
// then the block-local scans plus their offsets.  In place is safe: every thread
// reads its own elements before writing them.
void scan_counts_inplace(Ctx *c, uint32_t *a, size_t m, uint32_t *bsum) {
    if (m <= 4 * 1024) {  // small tables: one launch of one block beats three launches
        k_scan1<<<1, 1024, 0, c->stream>>>(a, (int)m);
        c->prof.launches += 1;
        return;
    }
    const int nb = ceil_div((long long)m, SCAN_TILE);
    k_scan_blocksum<<<nb, SCAN_NT, 0, c->stream>>>(a, m, bsum);
    k_scan1<<<1, 1024, 0, c->stream>>>(bsum, nb);
    k_scan_apply<<<nb, SCAN_NT, 0, c->stream>>>(a, m, bsum, a);
    c->prof.launches += 3;
}

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
