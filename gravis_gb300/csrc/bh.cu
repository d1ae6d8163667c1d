// bh.cu -- octree build and Barnes-Hut walk on the GPU
// (Octree: crates/sim-core/src/octree.rs:14-324; BarnesHut: crates/sim-core/src/barnes_hut.rs:21-192).
//
// The reference builds its octree by inserting particles one at a time into a
// cubic root box (BoundingBox::containing, octree.rs:14-44) that is halved
// level by level (child_bounds, octree.rs:52-64), each particle descending by
// the octant test x >= centre (octree.rs:67-79), leaves holding one particle.
// That tree does not depend on insertion order: a cell at depth L is a node
// iff its parent holds >= 2 particles, and it is a leaf iff it holds exactly
// one.  So the GPU builds the same tree from sorted keys:
//
//  1. Key: each particle replays the reference's f64 halving arithmetic for
//     42 levels (centre +- hw/2, same rounding), recording 3 octant bits per
//     level: a 126-bit octant-path key (two u64 words, 21 levels each).
//  2. Sort: by (high word, low word), ties in index order.  Sorted order = the
//     depth-first order of the reference tree with children 0..7.  The low
//     word is computed only for particles whose high word a neighbour shares:
//     everyone else's cell ends above depth 22.
//  3. Nodes: with d_i = common prefix depth of sorted keys i-1 and i, particle
//     i starts exactly the nodes at depths d_i+1 .. max(d_i, d_{i+1})+1 (the
//     last is its leaf).  A prefix sum of those counts gives every node an
//     index in pre-order; the node (i, L) covers particles [i, e) and its
//     subtree covers node indices [idx, off[e]) -- the skip pointer.
//     Particles that share all 42 levels (closer than 2^-42 of the box) form
//     one bucket leaf; the reference would keep splitting down to depth 64.
//  4. Moments: mass and centre of mass in f64, bottom-up in one pass (the
//     last child to finish sums its parent's children in child order, so
//     results are deterministic); the centre is the mass-weighted sum times
//     the f64 reciprocal of the mass.  Built when the f64 or mixed walk (or
//     the export) first needs them; the FP32 walk sums f32 moments instead,
//     as offsets from each node's first particle.
//     The reference updates the COM incrementally in insertion order; the
//     two agree to a few ulps.
//  5. Walk: the reference's per-particle stack walk (barnes_hut.rs:44-108):
//     skip empty, leaf != self -> direct term, internal -> accept if
//     s^2 < theta^2 d^2 with s = 2*half_width and d = |com - p|, else open.
//     Here each lane of a warp keeps its own "next node" pointer and the warp
//     processes the smallest pointer among its lanes each step, so every lane
//     visits exactly the nodes its own walk would (same accept decisions)
//     while node loads are broadcast.  Children are visited 0..7 (pre-order)
//     rather than the reference's LIFO 7..0: the same terms summed in another
//     order (differences at the 1e-16 relative level).
#include <algorithm>
#include <cmath>

#include "gvs_internal.cuh"

namespace gvs {

constexpr int MAXL = 42;

struct Tree {
    unsigned long long version = ~0ull;  // c->pos_version the tree was built for
    size_t n = 0, nnodes = 0;
    int precision = -1;
    double root[4] = {0, 0, 0, 0};  // centre x, y, z, half width (host copy)
    DevBuf bb, bbpart;              // device: min/max (6) then centre + hw (4)
    DevBuf khi, klo, khi2, klo2, perm, perm2, iota, iota2;
    DevBuf delta, nown, off, total;
    DevBuf level, first, cnt, skip;  // per node
    DevBuf mass, comx, comy, comz;   // per node (f64)
    DevBuf boxx, boxy, boxz;         // per node cell centre (f64)
    DevBuf sx, sy, sz, sm;           // sorted particle positions / masses (f64)
    DevBuf pos32, cm32, cm64, meta;
    DevBuf pos32lo;          // mixed walk: f32 lo words of the sorted positions
    DevBuf mrec;             // mixed walk: per node (meta, f32 COM + mass, f32 COM lo word), 48 B
    // group walk (f32): child-slot records, groups of <= 32*NPL particles, work counter
    DevBuf nk, koff, krec, groups, gcount;
    unsigned long long koff_version = ~0ull;
    DevBuf parent, arrive;  // per node: parent index, children that finished their moments
    DevBuf leaf_of;         // per sorted particle: the leaf that holds it
    unsigned long long grp_version = ~0ull;
    unsigned long long centres_version = ~0ull;  // tree version the cell centres were built for
    unsigned long long m64_version = ~0ull;      // ... the f64 moments were built for
    DevBuf mo32;                                  // FP32 walk: per node (offset from first particle, mass)
    int grp_size = 0;
    int walk_blocks = 0;  // resident blocks of the group walk (per GPU)
};

namespace {

__device__ __forceinline__ int common_levels(uint64_t ah, uint64_t al, uint64_t bh, uint64_t bl) {
    uint64_t x = ah ^ bh;
    if (x) return (__clzll(x) - 1) / 3;
    x = al ^ bl;
    if (x) return 21 + (__clzll(x) - 1) / 3;
    return MAXL;
}

// same cell at depth L (L in 0..42)?
__device__ __forceinline__ bool same_prefix(uint64_t ah, uint64_t al, uint64_t bh, uint64_t bl, int L) {
    if (L <= 21) return L == 0 || ((ah ^ bh) >> (63 - 3 * L)) == 0;
    if (ah != bh) return false;
    return ((al ^ bl) >> (63 - 3 * (L - 21))) == 0;
}

__device__ __forceinline__ int octant_at(uint64_t hi, uint64_t lo, int L) {  // L in 1..42
    return L <= 21 ? (int)((hi >> (63 - 3 * L)) & 7u) : (int)((lo >> (63 - 3 * (L - 21))) & 7u);
}

// Root cube: BoundingBox::containing (octree.rs:29-43), f64 without contraction.
// bb[10], bb[11]: the fixed-point frame of the keys' fast path (see k_keys).
__global__ void k_root(double *bb) {
    if (threadIdx.x || blockIdx.x) return;
    double c[3];
    for (int d = 0; d < 3; ++d) c[d] = __dmul_rn(0.5, __dadd_rn(bb[d], bb[3 + d]));
    double e = fmax(fmax(__dsub_rn(bb[3], bb[0]), __dsub_rn(bb[4], bb[1])), __dsub_rn(bb[5], bb[2]));
    double hw = __dadd_rn(__dmul_rn(__dmul_rn(0.5, e), 1.001), 1e-10);
    bb[6] = c[0]; bb[7] = c[1]; bb[8] = c[2]; bb[9] = hw;
    // V = (x - c)/(2 hw) + 1/2 in [0, 1): its binary digits are the octant tests
    // against the exact cell planes.  margin (units of 2^-62 of V) bounds the
    // f64 error of V (~2^-51) plus the drift of the reference's rounded centres
    // from the exact planes (<= 21 half-ulps of X = max|c| + hw), doubled; 0
    // disables the fast path.
    const double X = fmax(fabs(c[0]), fmax(fabs(c[1]), fabs(c[2]))) + hw;
    const double ratio = X / hw;
    const bool ok = isfinite(hw) && hw > 0.0 && isfinite(X) && ratio < 1e6;
    bb[10] = ok ? 1.0 / (2.0 * hw) : 0.0;
    bb[11] = ok ? 8192.0 + 65536.0 * ceil(ratio) : 0.0;
}

// hw * 0.5 for the cell half widths: exact for normal hw (a root half width is
// >= 1e-10, so 42 halvings stay far above the subnormal range); an exponent
// decrement instead of an f64 multiply (GB300 runs f64 at 1/64 of the f32 rate).
__device__ __forceinline__ double half_of(double hw, bool finite) {
    return finite ? __longlong_as_double(__double_as_longlong(hw) - (1ll << 52)) : __dmul_rn(hw, 0.5);
}

// Order-preserving map of f64 to u64: a >= b <=> ord64(a) >= ord64(b) for non-NaN
// a, b, with -0 mapped like +0 -- so the octant tests x >= centre run on the
// integer pipe with the f64 compare's result.
__device__ __forceinline__ unsigned long long ord64(double v) {
    unsigned long long b = (unsigned long long)__double_as_longlong(v);
    if (b == 0x8000000000000000ull) b = 0ull;
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ bool nan64(double v) {
    return ((unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull) > 0x7FF0000000000000ull;
}

// Octant path of one point (octant, child_bounds: octree.rs:52-79): the
// reference's f64 centre updates (round to nearest, no contraction) and its
// x >= centre tests (false when either side is NaN), levels 1..LMAX; levels
// 1..21 go to hi, 22..42 to lo.
template <int LMAX>
__device__ __forceinline__ void octant_path(double x, double y, double z, const double *__restrict__ bb, uint64_t &hi,
                                            uint64_t &lo) {
    const unsigned long long ox = ord64(x), oy = ord64(y), oz = ord64(z);
    const bool nx = nan64(x), ny = nan64(y), nz = nan64(z);
    double cx = bb[6], cy = bb[7], cz = bb[8], hw = bb[9];
    const bool fin = isfinite(hw);
    hi = 0;
    lo = 0;
    for (int L = 1; L <= LMAX; ++L) {
        const bool gx = !nx && !nan64(cx) && ox >= ord64(cx);
        const bool gy = !ny && !nan64(cy) && oy >= ord64(cy);
        const bool gz = !nz && !nan64(cz) && oz >= ord64(cz);
        const int oct = (gx ? 1 : 0) | (gy ? 2 : 0) | (gz ? 4 : 0);
        if (L <= 21) hi = (hi << 3) | (uint64_t)oct;
        else lo = (lo << 3) | (uint64_t)oct;
        if (L == LMAX) break;
        const double q = half_of(hw, fin);
        cx = __dadd_rn(cx, gx ? q : -q);
        cy = __dadd_rn(cy, gy ? q : -q);
        cz = __dadd_rn(cz, gz ? q : -q);
        hw = q;
    }
}

// The high key word on the integer pipe.  The reference's centres c~_L are f64
// sums that drift from the exact planes c_L = c + hw * sum(+-2^-k) by at most 21
// half-ulps of X; a coordinate farther than that from every plane it is tested
// against gets the same octant from the exact plane, which is one bit of its
// fixed-point position V.  Returns false (the caller replays the f64 path) if
// any tested plane lies within the certified margin, or for NaN / out-of-box
// input.
__device__ __forceinline__ bool fast_hi(double x, double y, double z, const double *__restrict__ bb,
                                        uint64_t &hi) {
    const double inv = bb[10];
    if (inv == 0.0) return false;
    const unsigned long long margin = (unsigned long long)bb[11];
    const double p[3] = {x, y, z}, c[3] = {bb[6], bb[7], bb[8]};
    unsigned long long W[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double v = __dadd_rn(__dmul_rn(__dsub_rn(p[d], c[d]), inv), 0.5);
        // v in (0, 1) and W = floor(v 2^62), from the bit pattern (NaN and v <= 0 fail)
        const long long b = __double_as_longlong(v);
        if (!(b > 0 && b < 0x3FF0000000000000ll)) return false;
        const int sh = (int)((b >> 52) & 0x7FF) - 1023 + 10;  // exponent e in [-1022, -1]: v 2^62 = m 2^(e + 10)
        const unsigned long long m = ((unsigned long long)b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
        W[d] = sh >= 0 ? m << sh : (sh > -64 ? m >> -sh : 0ull);
    }
    uint64_t h = 0;
    bool ok = true;
#pragma unroll
    for (int L = 1; L <= 21; ++L) {
        const unsigned long long half = 1ull << (62 - L), mask = (half << 1) - 1ull;
        int oct = 0;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const unsigned long long r = W[d] & mask;
            const unsigned long long dist = r >= half ? r - half : half - r;
            ok = ok && dist > margin;
            oct |= (int)((W[d] >> (62 - L)) & 1ull) << d;
        }
        h = (h << 3) | (uint64_t)oct;
    }
    hi = h;
    return ok;
}

// Keys, levels 1..LMAX (42: both words; 21: the high word, lo = 0).
template <int LMAX>
__global__ void k_keys(const double *__restrict__ X, const double *__restrict__ Y, const double *__restrict__ Z,
                       size_t n, const double *__restrict__ bb, uint64_t *__restrict__ khi,
                       uint64_t *__restrict__ klo, uint32_t *__restrict__ perm) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t hi, lo = 0;
    if (LMAX != 21 || !fast_hi(X[i], Y[i], Z[i], bb, hi)) octant_path<LMAX>(X[i], Y[i], Z[i], bb, hi, lo);
    khi[i] = hi;
    if (klo) klo[i] = lo;
    perm[i] = (uint32_t)i;
}

// After the sort by the high word: particles whose high word equals a
// neighbour's (runs of points closer than 2^-21 of the root box) get their low
// word; everyone else's stays 0 (their cells end above depth 22, where the low
// word is never consulted).  stat[0] counts them; stat[1] is set if a run is
// longer than RUN_MAX.
constexpr int RUN_MAX = 64;
__global__ void k_keys_lo(const uint64_t *__restrict__ khi, const uint32_t *__restrict__ perm,
                          const double *__restrict__ X, const double *__restrict__ Y, const double *__restrict__ Z,
                          size_t n, const double *__restrict__ bb, uint64_t *__restrict__ klo,
                          uint32_t *__restrict__ stat) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t h = khi[i];
    const bool prev = i > 0 && khi[i - 1] == h, next = i + 1 < n && khi[i + 1] == h;
    uint64_t lo = 0;
    if (prev || next) {
        const uint32_t o = perm[i];
        if (!CHK_IDX(o, n)) {
            klo[i] = 0;
            return;
        }
        uint64_t hh;
        octant_path<MAXL>(X[o], Y[o], Z[o], bb, hh, lo);
        atomicAdd(stat, 1u);
        if (!prev && i + RUN_MAX < n && khi[i + RUN_MAX] == h) atomicOr(stat + 1, 1u);
    }
    klo[i] = lo;
}

// Sorts each run of equal high words by (low word, original index) -- the
// order a stable sort by (high, low) gives -- one thread per run start,
// insertion sort (runs hold at most RUN_MAX particles).
__global__ void k_sort_runs(const uint64_t *__restrict__ khi, size_t n, uint64_t *__restrict__ klo,
                            uint32_t *__restrict__ perm) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i + 1 >= n) return;
    const uint64_t h = khi[i];
    if ((i > 0 && khi[i - 1] == h) || khi[i + 1] != h) return;
    size_t e = i + 1;
    while (e < n && khi[e] == h) ++e;
    for (size_t a = i + 1; a < e; ++a) {
        const uint64_t kl = klo[a];
        const uint32_t kp = perm[a];
        size_t b = a;
        while (b > i && (klo[b - 1] > kl || (klo[b - 1] == kl && perm[b - 1] > kp))) {
            klo[b] = klo[b - 1];
            perm[b] = perm[b - 1];
            --b;
        }
        klo[b] = kl;
        perm[b] = kp;
    }
}

__global__ void k_iota(uint32_t *a, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = (uint32_t)i;
}

template <class T>
__global__ void k_gather(const T *__restrict__ src, const uint32_t *__restrict__ idx, T *__restrict__ dst, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const uint32_t j = idx[i];
        if (CHK_IDX(j, n)) dst[i] = src[j];
    }
}

// delta[i] = common depth of sorted keys i-1 and i (delta[0] = delta[n] = -1);
// nown[i] = number of nodes particle i starts; nown[n] = 0.
__global__ void k_delta(const uint64_t *__restrict__ khi, const uint64_t *__restrict__ klo, size_t n,
                        int *__restrict__ delta) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n) return;
    delta[i] = (i == 0 || i == n) ? -1 : common_levels(khi[i - 1], klo[i - 1], khi[i], klo[i]);
}

__global__ void k_nown(const int *__restrict__ delta, size_t n, uint32_t *__restrict__ nown) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n) return;
    if (i == n) { nown[i] = 0; return; }
    const int a = delta[i] + 1;
    const int b = min(max(delta[i], delta[i + 1]) + 1, MAXL);
    nown[i] = b >= a ? (uint32_t)(b - a + 1) : 0u;
}

// One thread per particle: writes the nodes it starts (integer work only).
__global__ void k_nodes(const uint64_t *__restrict__ khi, const uint64_t *__restrict__ klo,
                        const int *__restrict__ delta, const uint32_t *__restrict__ off, size_t n,
                        uint8_t *__restrict__ level, uint32_t *__restrict__ first, uint32_t *__restrict__ cnt,
                        uint32_t *__restrict__ skip, size_t nnodes) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int a = delta[i] + 1;
    const int b = min(max(delta[i], delta[i + 1]) + 1, MAXL);
    if (b < a) return;
    const uint64_t hi = khi[i], lo = klo[i];
    const uint32_t base = off[i];
    for (int L = a; L <= b; ++L) {
        // end of the depth-L cell of particle i
        size_t e;
        if (delta[i + 1] < L) {
            e = i + 1;
        } else {
            size_t lo_j = i + 1, hi_j = n;
            while (lo_j < hi_j) {
                const size_t mid = (lo_j + hi_j) >> 1;
                if (same_prefix(khi[mid], klo[mid], hi, lo, L)) lo_j = mid + 1;
                else hi_j = mid;
            }
            e = lo_j;
        }
        const uint32_t idx = base + (uint32_t)(L - a);
        if (!CHK_IDX(idx, nnodes)) return;
        const bool leaf = (e - i == 1) || L == MAXL;
        level[idx] = (uint8_t)L;
        first[idx] = (uint32_t)i;
        cnt[idx] = leaf ? (uint32_t)(e - i) : 0u;
        skip[idx] = off[e];
    }
}

// Cell centres of the nodes particle i starts (child_bounds, octree.rs:52-64):
// the reference's f64 halving replayed down the particle's key.  Only the SPH
// neighbour search reads them, so they are built on its first request.
__global__ void k_centres(const uint64_t *__restrict__ khi, const uint64_t *__restrict__ klo,
                          const int *__restrict__ delta, const uint32_t *__restrict__ off, size_t n,
                          const double *__restrict__ bb, double *__restrict__ bx, double *__restrict__ by,
                          double *__restrict__ bz) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int a = delta[i] + 1;
    const int b = min(max(delta[i], delta[i + 1]) + 1, MAXL);
    if (b < a) return;
    const uint64_t hi = khi[i], lo = klo[i];
    double cx = bb[6], cy = bb[7], cz = bb[8], hw = bb[9];
    const bool fin = isfinite(hw);
    const uint32_t base = off[i];
    for (int L = 1; L <= b; ++L) {
        const int oct = octant_at(hi, lo, L);
        const double q = half_of(hw, fin);
        cx = __dadd_rn(cx, (oct & 1) ? q : -q);
        cy = __dadd_rn(cy, (oct & 2) ? q : -q);
        cz = __dadd_rn(cz, (oct & 4) ? q : -q);
        hw = q;
        if (L >= a) {
            const uint32_t idx = base + (uint32_t)(L - a);
            bx[idx] = cx; by[idx] = cy; bz[idx] = cz;
        }
    }
    if (a == 0) {  // the root
        bx[base] = bb[6]; by[base] = bb[7]; bz[base] = bb[8];
    }
}

// Parent links and child counts: each internal node walks its children (the
// skip chain k+1, skip[k+1], ... up to skip[k]); each leaf records itself as
// the leaf of its particles.
__global__ void k_links(size_t nnodes, const uint32_t *__restrict__ first, const uint32_t *__restrict__ cnt,
                        const uint32_t *__restrict__ skip, uint32_t *__restrict__ parent, uint32_t *__restrict__ nk,
                        uint32_t *__restrict__ leaf_of, size_t n) {
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nnodes) return;
    if (k == 0) parent[0] = 0xFFFFFFFFu;
    uint32_t c = 0;
    const uint32_t lc = cnt[k];
    for (uint32_t j = first[k]; j < first[k] + lc; ++j)
        if (CHK_IDX(j, n)) leaf_of[j] = (uint32_t)k;
    if (lc == 0) {
        const uint32_t end = skip[k];
        for (uint32_t ch = (uint32_t)k + 1; ch < end && CHK_IDX(ch, nnodes); ch = skip[ch], ++c) parent[ch] = (uint32_t)k;
    }
    nk[k] = c;
}

// Mass and centre of mass in f64, bottom-up in one pass.  Each leaf sums its
// members in order; then the thread whose child finishes a parent last (an
// arrival counter per node) sums that parent's children in child order 0..7 and
// moves up.  Every node's sum has a fixed order, so the result does not depend
// on which thread computes it.  Writes are fenced before the arrival count;
// the last arriver fences after it and reads the children through L2.
__global__ void k_moments_up(size_t nnodes, const uint32_t *__restrict__ first, const uint32_t *__restrict__ cnt,
                             const uint32_t *__restrict__ skip, const uint32_t *__restrict__ parent,
                             const uint32_t *__restrict__ nk, uint32_t *__restrict__ arrive,
                             const double *__restrict__ sx, const double *__restrict__ sy,
                             const double *__restrict__ sz, const double *__restrict__ sm, double *mass, double *cx,
                             double *cy, double *cz) {
    const size_t k0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k0 >= nnodes) return;
    const uint32_t c0 = cnt[k0];
    if (c0 == 0) return;
    uint32_t k = (uint32_t)k0;
    if (c0 == 1) {
        const uint32_t p = first[k];
        mass[k] = sm[p]; cx[k] = sx[p]; cy[k] = sy[p]; cz[k] = sz[p];
    } else {  // bucket leaf: members in order
        double M = 0.0, X = 0.0, Yv = 0.0, Zv = 0.0;
        for (uint32_t p = first[k]; p < first[k] + c0; ++p) {
            const double m = sm[p];
            M += m; X += m * sx[p]; Yv += m * sy[p]; Zv += m * sz[p];
        }
        mass[k] = M;
        if (M > 0.0) {
            const double r = 1.0 / M;  // one f64 division per node, not three
            cx[k] = X * r; cy[k] = Yv * r; cz[k] = Zv * r;
        } else {
            cx[k] = cy[k] = cz[k] = 0.0;
        }
    }
    for (;;) {
        const uint32_t up = parent[k];
        if (up == 0xFFFFFFFFu) return;
        __threadfence();
        if (atomicAdd(arrive + up, 1u) != nk[up] - 1u) return;
        __threadfence();
        k = up;
        double M = 0.0, X = 0.0, Yv = 0.0, Zv = 0.0;
        const uint32_t end = skip[k];
        for (uint32_t ch = k + 1; ch < end; ch = skip[ch]) {
            const double m = __ldcg(mass + ch);
            M += m; X += m * __ldcg(cx + ch); Yv += m * __ldcg(cy + ch); Zv += m * __ldcg(cz + ch);
        }
        mass[k] = M;
        if (M > 0.0) {
            const double r = 1.0 / M;  // one f64 division per node, not three
            cx[k] = X * r; cy[k] = Yv * r; cz[k] = Zv * r;
        } else {
            cx[k] = cy[k] = cz[k] = 0.0;
        }
    }
}

// FP32-walk moments: mass and centre of mass in f32 on the FMA pipe, bottom-up
// like k_moments_up.  Each node's centre is kept as an offset from its first
// particle (f32), so the sums see differences of the size of the cell, not of the
// coordinates: mo[k] = (offset, mass), cm32[k] = (first particle + offset, mass).
// A one-particle leaf's record is that particle's f32 position and mass exactly.
__global__ void k_moments32_up(size_t nnodes, const uint32_t *__restrict__ first, const uint32_t *__restrict__ cnt,
                               const uint32_t *__restrict__ skip, const uint32_t *__restrict__ parent,
                               const uint32_t *__restrict__ nk, uint32_t *__restrict__ arrive,
                               const float4 *__restrict__ p32, float4 *mo, float4 *__restrict__ cm32) {
    const size_t k0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k0 >= nnodes) return;
    const uint32_t c0 = cnt[k0];
    if (c0 == 0) return;
    uint32_t k = (uint32_t)k0;
    float4 r = p32[first[k]];
    float M = 0.f, X = 0.f, Yv = 0.f, Zv = 0.f;
    if (c0 == 1) {
        M = r.w;
    } else {  // bucket leaf: members in order
        for (uint32_t p = first[k]; p < first[k] + c0; ++p) {
            const float4 q = p32[p];
            M += q.w;
            X = fmaf(q.w, q.x - r.x, X); Yv = fmaf(q.w, q.y - r.y, Yv); Zv = fmaf(q.w, q.z - r.z, Zv);
        }
    }
    for (;;) {
        const float inv = M > 0.f ? 1.0f / M : 0.f;
        const float ox = X * inv, oy = Yv * inv, oz = Zv * inv;
        mo[k] = make_float4(ox, oy, oz, M);
        cm32[k] = make_float4(r.x + ox, r.y + oy, r.z + oz, M);
        const uint32_t up = parent[k];
        if (up == 0xFFFFFFFFu) return;
        __threadfence();
        if (atomicAdd(arrive + up, 1u) != nk[up] - 1u) return;
        __threadfence();
        k = up;
        r = p32[first[k]];
        M = 0.f; X = 0.f; Yv = 0.f; Zv = 0.f;
        const uint32_t end = skip[k];
        for (uint32_t ch = k + 1; ch < end; ch = skip[ch]) {
            const float4 q = __ldcg(mo + ch);
            const float4 rc = p32[first[ch]];
            M += q.w;
            X = fmaf(q.w, (rc.x - r.x) + q.x, X);
            Yv = fmaf(q.w, (rc.y - r.y) + q.y, Yv);
            Zv = fmaf(q.w, (rc.z - r.z) + q.z, Zv);
        }
    }
}

// Per-node records of the walks: meta (skip, first, count, level) for every walk,
// the f64 moments for the f64 walk and the mixed walk's band tests, and for the
// mixed walk one 48-byte record (meta, f32 COM + mass, f32 lo word of the COM),
// so that each step of that walk reads one block of memory.
__global__ void k_pack_nodes(size_t nnodes, const uint8_t *__restrict__ level, const uint32_t *__restrict__ first,
                             const uint32_t *__restrict__ cnt, const uint32_t *__restrict__ skip,
                             const double *__restrict__ mass, const double *__restrict__ cx,
                             const double *__restrict__ cy, const double *__restrict__ cz,
                             double4 *__restrict__ cm64, int4 *__restrict__ meta, float4 *__restrict__ mrec) {
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nnodes) return;
    const int4 mt = make_int4((int)skip[k], (int)first[k], (int)cnt[k], (int)level[k]);
    meta[k] = mt;
    if (cm64) cm64[k] = make_double4(cx[k], cy[k], cz[k], mass[k]);
    if (mrec) {
        const float hx = (float)cx[k], hy = (float)cy[k], hz = (float)cz[k];
        mrec[3 * k] = make_float4(__int_as_float(mt.x), __int_as_float(mt.y), __int_as_float(mt.z),
                                  __int_as_float(mt.w));
        mrec[3 * k + 1] = make_float4(hx, hy, hz, (float)mass[k]);
        // .w: the largest |hi word| of the COM, for the walk's decision band
        mrec[3 * k + 2] = make_float4((float)(cx[k] - (double)hx), (float)(cy[k] - (double)hy),
                                      (float)(cz[k] - (double)hz), fmaxf(fabsf(hx), fmaxf(fabsf(hy), fabsf(hz))));
    }
}

__global__ void k_pack_particles(size_t n, const double *__restrict__ sx, const double *__restrict__ sy,
                                 const double *__restrict__ sz, const double *__restrict__ sm, float4 *__restrict__ p32,
                                 float4 *__restrict__ p32lo) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float hx = (float)sx[i], hy = (float)sy[i], hz = (float)sz[i];
    p32[i] = make_float4(hx, hy, hz, (float)sm[i]);
    if (p32lo)  // .w: the largest |hi word| of the position, for the mixed walk's decision band
        p32lo[i] = make_float4((float)(sx[i] - (double)hx), (float)(sy[i] - (double)hy), (float)(sz[i] - (double)hz),
                               fmaxf(fabsf(hx), fmaxf(fabsf(hy), fabsf(hz))));
}

// ---- walk -------------------------------------------------------------------
struct S2Table {
    double s2[MAXL + 1];   // (2 * half_width_L)^2, half_width_L = hw0 * 2^-L
    float s2f[MAXL + 1];
    // mixed walk: the opening radius s / theta in f32 (clamped to 3e38); the walk decides
    // with the f32 distance of the hi words outside a certified band around it and with the
    // reference's f64 test inside (see mixed_band)
    float rcf[MAXL + 1];
};

// The mixed walk's band around the opening radius rc = s / theta, in which the f32
// distance of the hi words cannot decide.  Hi words round f64 coordinates to nearest,
// so each component of the f32 difference of a node COM c and a particle p is within
// 2^-24 (|c| + |p| + |c - p|) <= 2^-23 (Mc + Mp)(1 + 2^-25) of the true one (M: the
// largest |coordinate| of the hi words), and the distance within sqrt(3) of that,
// < 0.87 * 2^-22 (Mc + Mp).  The band half-width is three times that bound plus
// 2^-20 rc, which covers the f32 rounding of rc and keeps the decision far (relative
// 2^-20) from the rounding of the reference's f64 test.  The squared limits carry a
// factor 1 +- 2^-19 for the f32 rounding of d^2 and of the limits themselves (at most
// ~6 * 2^-24 relative).  Outside the band: d^2 > hi2 means d > rc for sure (accept),
// d^2 < lo2 means d < rc for sure (open).
__device__ __forceinline__ void mixed_band(float rc, float mc, float mp, float &lo2, float &hi2) {
    const float dl = fmaf(0x1.8p-22f, mc + mp, 0x1p-20f * rc);
    const float hi = rc + dl, lo = rc - dl;
    hi2 = hi * hi * (1.0f + 0x1p-19f);
    lo2 = lo > 0.f ? lo * lo * (1.0f - 0x1p-19f) : -1.0f;
}

// Where a walk leaves its sums: caller-order acceleration arrays, written (or
// added to) at perm[i] for sorted particle i.
struct AccOut {
    const uint32_t *perm;
    double *ax, *ay, *az;
    int accumulate;
    size_t n;  // length of perm's targets (the checked build tests every perm[i] against it)
};

__device__ __forceinline__ void store_acc(const AccOut &o, size_t i, double fx, double fy, double fz) {
    const uint32_t k = o.perm[i];
    if (!CHK_IDX(k, o.n)) return;
    if (o.accumulate) {
        o.ax[k] += fx; o.ay[k] += fy; o.az[k] += fz;
    } else {
        o.ax[k] = fx; o.ay[k] = fy; o.az[k] = fz;
    }
}

// BarnesHut::add_force (barnes_hut.rs:114-135), IEEE f64 with no contraction.
__device__ __forceinline__ void add_force64(double px, double py, double pz, double sx, double sy, double sz,
                                            double m, double eps2, double &ax, double &ay, double &az) {
    const double dx = __dsub_rn(sx, px), dy = __dsub_rn(sy, py), dz = __dsub_rn(sz, pz);
    const double r2 = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)), eps2);
    const double inv_r3 = __ddiv_rn(1.0, __dmul_rn(r2, __dsqrt_rn(r2)));
    const double f = __dmul_rn(m, inv_r3);
    ax = __dadd_rn(ax, __dmul_rn(f, dx));
    ay = __dadd_rn(ay, __dmul_rn(f, dy));
    az = __dadd_rn(az, __dmul_rn(f, dz));
}

// Compensated accumulators of the mixed walk: x and y as one f32x2 pair, z alone.
struct FFAcc {
    f2 hxy = 0ull, lxy = 0ull;
    float hz = 0.f, lz = 0.f;
};

// f32 monopole term on a float-float separation (hi - hi) + (lo - lo), added to
// (hi, lo) accumulators by Knuth's two-sum (error-free: the product is rounded
// once, then added).  x and y run as packed f32x2 operations, z as scalars: the
// same operations per component, one instruction for two.
__device__ __forceinline__ void add_force_ff(float4 q, float4 ql, float sx, float sy, float sz, float sxl, float syl,
                                             float szl, float m, float eps2, FFAcc &acc) {
    const f2 dxy = add2(sub2(pk(sx, sy), pk(q.x, q.y)), sub2(pk(sxl, syl), pk(ql.x, ql.y)));
    const float dz = __fadd_rn(__fsub_rn(sz, q.z), __fsub_rn(szl, ql.z));
    float dx, dy;
    upk(dxy, dx, dy);
    const float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
    const float ri = rsqrt_approx(r2);
    const float f = __fmul_rn(__fmul_rn(__fmul_rn(m, ri), ri), ri);
    two_sum2(acc.hxy, acc.lxy, mul2(pk(f, f), dxy));
    const float v = __fmul_rn(f, dz);
    const float sum = __fadd_rn(acc.hz, v);
    const float bp = __fsub_rn(sum, acc.hz);
    acc.lz = __fadd_rn(acc.lz, __fadd_rn(__fsub_rn(acc.hz, __fsub_rn(sum, bp)), __fsub_rn(v, bp)));
    acc.hz = sum;
}

__device__ __forceinline__ void add_force32(float px, float py, float pz, float sx, float sy, float sz, float m,
                                            float eps2, float &ax, float &ay, float &az) {
    const float dx = sx - px, dy = sy - py, dz = sz - pz;
    const float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
    const float ri = rsqrt_approx(r2);
    const float f = m * ri * ri * ri;
    ax = fmaf(f, dx, ax);
    ay = fmaf(f, dy, ay);
    az = fmaf(f, dz, az);
}

// MODE 0: f64, the reference's arithmetic per term.  MODE 1: f32 positions and
// moments, f32 opening test.  MODE 2 (mixed): f32 terms on float-float
// separations with compensated sums, and the reference's opening decisions --
// an f32 test of the hi words with a certified margin, the f64 test in between.
template <int MODE>
__global__ void __launch_bounds__(128) k_walk(size_t n, size_t nnodes, const int4 *__restrict__ meta,
                                              const float4 *__restrict__ cm32, const double4 *__restrict__ cm64,
                                              const float4 *__restrict__ p32, const double *__restrict__ sx,
                                              const double *__restrict__ sy, const double *__restrict__ sz,
                                              const double *__restrict__ sm, const S2Table tab, double theta2,
                                              double eps2, const AccOut out, const float4 *__restrict__ p32lo,
                                              const float4 *__restrict__ mrec, unsigned *__restrict__ err) {
    constexpr bool F64 = MODE == 0;
    unsigned nterm = 0;  // node and particle terms this particle summed (profile counter)
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = t < n;
    double px = 0, py = 0, pz = 0;
    float qx = 0, qy = 0, qz = 0;
    float4 qh = make_float4(0.f, 0.f, 0.f, 0.f), ql = qh;
    if (active) {
        if (MODE != 1) { px = sx[t]; py = sy[t]; pz = sz[t]; }
        if (MODE != 0) { qh = p32[t]; qx = qh.x; qy = qh.y; qz = qh.z; }
        if (MODE == 2) ql = p32lo[t];
    }
    const float theta2f = (float)theta2, eps2f = (float)eps2;
    double ax = 0, ay = 0, az = 0;
    float fx = 0, fy = 0, fz = 0;
    FFAcc fa;  // mixed: compensated sums
    uint32_t next = active ? 0u : 0xFFFFFFFFu;
    for (;;) {
        const uint32_t m = __reduce_min_sync(0xFFFFFFFFu, next);
        if ((size_t)m >= nnodes) break;
        if (next != m) continue;
        // the node's records, loaded together: one memory latency per step of the walk
        // instead of a chain of dependent loads
        int4 mt;
        double4 c64v = make_double4(0.0, 0.0, 0.0, 0.0);
        float4 c32v = make_float4(0.f, 0.f, 0.f, 0.f), c32l = c32v;
        if (MODE == 2) {  // one 48-byte record: meta, COM hi + mass, COM lo
            const float4 r0 = mrec[3 * (size_t)m];
            c32v = mrec[3 * (size_t)m + 1];
            c32l = mrec[3 * (size_t)m + 2];
            mt = make_int4(__float_as_int(r0.x), __float_as_int(r0.y), __float_as_int(r0.z), __float_as_int(r0.w));
        } else {
            mt = meta[m];
            if (F64) c64v = cm64[m];
            else c32v = cm32[m];
        }
        if (!CHK((size_t)mt.x > m && (size_t)mt.x <= nnodes, DERR_TREE)) {  // a skip pointer must move forward
            next = (uint32_t)nnodes;
            continue;
        }
        if (mt.z > 0) {  // leaf
            if (!CHK(mt.y >= 0 && (size_t)mt.y + (size_t)mt.z <= n, DERR_BOUNDS)) {
                next = (uint32_t)mt.x;
            } else if (mt.z == 1) {
                if ((size_t)mt.y != t) {
                    ++nterm;
                    if (F64) {
                        const double4 c = c64v;
                        if (c.w != 0.0) add_force64(px, py, pz, c.x, c.y, c.z, c.w, eps2, ax, ay, az);
                    } else if (MODE == 1) {
                        const float4 c = c32v;
                        if (c.w != 0.f) add_force32(qx, qy, qz, c.x, c.y, c.z, c.w, eps2f, fx, fy, fz);
                    } else {
                        const float4 c = c32v;
                        if (c.w != 0.f) {
                            const float4 cl = c32l;
                            add_force_ff(qh, ql, c.x, c.y, c.z, cl.x, cl.y, cl.z, c.w, eps2f, fa);
                        }
                    }
                }
            } else {  // bucket of coincident-key particles: direct terms
                for (int j = mt.y; j < mt.y + mt.z; ++j) {
                    if ((size_t)j == t) continue;
                    ++nterm;
                    if (F64) {
                        if (sm[j] != 0.0) add_force64(px, py, pz, sx[j], sy[j], sz[j], sm[j], eps2, ax, ay, az);
                    } else if (MODE == 1) {
                        const float4 q = p32[j];
                        if (q.w != 0.f) add_force32(qx, qy, qz, q.x, q.y, q.z, q.w, eps2f, fx, fy, fz);
                    } else {
                        const float4 q = p32[j];
                        if (q.w != 0.f) {
                            const float4 l = p32lo[j];
                            add_force_ff(qh, ql, q.x, q.y, q.z, l.x, l.y, l.z, q.w, eps2f, fa);
                        }
                    }
                }
            }
            next = (uint32_t)mt.x;
        } else if (F64) {
            const double4 c = c64v;
            if (c.w == 0.0) {
                next = (uint32_t)mt.x;
            } else {
                const double dx = __dsub_rn(c.x, px), dy = __dsub_rn(c.y, py), dz = __dsub_rn(c.z, pz);
                const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
                if (tab.s2[mt.w] < __dmul_rn(theta2, d2)) {
                    add_force64(px, py, pz, c.x, c.y, c.z, c.w, eps2, ax, ay, az);
                    ++nterm;
                    next = (uint32_t)mt.x;
                } else {
                    next = m + 1;
                }
            }
        } else {
            const float4 c = c32v;
            if (c.w == 0.f) {
                next = (uint32_t)mt.x;
            } else {
                const float dx = c.x - qx, dy = c.y - qy, dz = c.z - qz;
                const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                bool accept;
                float lo2 = 0.f, hi2 = 0.f;
                if (MODE == 2) mixed_band(tab.rcf[mt.w], c32l.w, ql.w, lo2, hi2);
                if (MODE == 1) {
                    accept = tab.s2f[mt.w] < theta2f * d2;
                } else if (d2 > hi2) {
                    accept = true;
                } else if (d2 < lo2) {
                    accept = false;
                } else {  // near the boundary: the reference's f64 test
                    const double4 c64 = cm64[m];
                    const double ex = __dsub_rn(c64.x, px), ey = __dsub_rn(c64.y, py), ez = __dsub_rn(c64.z, pz);
                    const double e2 = __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez));
                    accept = tab.s2[mt.w] < __dmul_rn(theta2, e2);
                }
                if (accept) {
                    ++nterm;
                    if (MODE == 1) {
                        add_force32(qx, qy, qz, c.x, c.y, c.z, c.w, eps2f, fx, fy, fz);
                    } else {
                        const float4 cl = c32l;
                        add_force_ff(qh, ql, c.x, c.y, c.z, cl.x, cl.y, cl.z, c.w, eps2f, fa);
                    }
                    next = (uint32_t)mt.x;
                } else {
                    next = m + 1;
                }
            }
        }
    }
    const unsigned wterms = __reduce_add_sync(0xFFFFFFFFu, active ? nterm : 0u);
    if ((threadIdx.x & 31) == 0 && wterms)
        atomicAdd(reinterpret_cast<unsigned long long *>(err + EW_WALK_TERMS), (unsigned long long)wterms);
    if (!active) return;
    if (MODE == 1) { ax = fx; ay = fy; az = fz; }
    if (MODE == 2) {
        float hx, hy, lx, ly;
        upk(fa.hxy, hx, hy);
        upk(fa.lxy, lx, ly);
        ax = (double)hx + (double)lx;
        ay = (double)hy + (double)ly;
        az = (double)fa.hz + (double)fa.lz;
    }
    store_acc(out, t, ax, ay, az);
}

// ---- group walk (FP32) ---------------------------------------------------------
// A faster f32 form of the walk for GVS_PREC_FP32.  One warp serves a group of
// up to 32*NPL particles that share a tree cell: the cells with at most that
// many particles whose parent has more (siblings merged while they fit).  The
// warp opens nodes 32 at a time with a group test -- accept if
// s^2 < theta^2 d^2 with d the distance from the node's COM to the box of the
// group's particles -- and collects accepted nodes and leaves in a shared
// interaction list that every lane then evaluates for its own particles.
// d <= |com - p| for every particle p of the group, so each particle accepts
// only nodes its own walk (the reference's test) would accept -- up to the f32
// rounding of the test at the opening boundary: its force is a refinement of the
// per-particle Barnes-Hut sum (more nodes opened, never fewer).  Node records are stored by child slot (the children of a node are
// contiguous) so that opening a node pushes one (slot, count) range.
//
// Stack bound: an iteration pops whole ranges (at most 32 nodes) from the top
// and pushes at most 32 ranges, the children of the nodes it popped.  Grouping
// the stack into the batches that iterations pushed, the least node depth of
// each batch increases strictly from bottom to top (a batch's nodes are one
// level below the shallowest node popped to make it, and that node's batch is
// the one it lands on or lies above it).  Depths run 0..42, so the stack never
// holds more than 43 batches of 32 ranges.
constexpr int GW_WARPS = 4;
constexpr int GW_SCAP = (MAXL + 1) * 32;
constexpr int GW_ICAP = 128;

struct GroupSmem {
    uint32_t stack[GW_SCAP];  // (first child slot << 3) | (children - 1)
    float4 il[2 * GW_ICAP];   // interaction list: (x, x, y, y), (z, z, m, m)
};

__device__ __forceinline__ uint32_t sub_count(uint32_t k, size_t nnodes, size_t n, const uint32_t *__restrict__ first,
                                              const uint32_t *__restrict__ skip) {
    const uint32_t e = skip[k];
    return (uint32_t)((e < nnodes ? (size_t)first[e] : n) - first[k]);
}

struct S2f {
    float s2[MAXL + 1];
};

// Record of node x: (com, mass) and (first child slot, children, 0, s^2) for an
// internal node, (-1, particle, 1, 0) for a one-particle leaf, (-2, first, count, 0)
// for a bucket leaf.
__device__ __forceinline__ void write_rec(float4 *__restrict__ krec, uint32_t slot, uint32_t x,
                                          const uint8_t *__restrict__ level, const uint32_t *__restrict__ first,
                                          const uint32_t *__restrict__ cnt, const uint32_t *__restrict__ nk,
                                          const uint32_t *__restrict__ koff, const float4 *__restrict__ cm32,
                                          const S2f &tab) {
    krec[2 * (size_t)slot] = cm32[x];
    const uint32_t c = cnt[x];
    int4 b;
    if (c == 0) b = make_int4((int)(1u + koff[x]), (int)nk[x], 0, __float_as_int(tab.s2[level[x]]));
    else if (c == 1) b = make_int4(-1, (int)first[x], 1, 0);
    else b = make_int4(-2, (int)first[x], (int)c, 0);
    reinterpret_cast<int4 *>(krec)[2 * (size_t)slot + 1] = b;
}

// Each internal node writes its children's records at slots 1 + koff[k] + c;
// node 0 also writes the root's record at slot 0.
__global__ void k_krec(size_t nnodes, const uint8_t *__restrict__ level, const uint32_t *__restrict__ first,
                       const uint32_t *__restrict__ cnt, const uint32_t *__restrict__ skip,
                       const uint32_t *__restrict__ nk, const uint32_t *__restrict__ koff,
                       const float4 *__restrict__ cm32, const S2f tab, float4 *__restrict__ krec) {
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nnodes) return;
    if (k == 0) write_rec(krec, 0, 0, level, first, cnt, nk, koff, cm32, tab);
    if (cnt[k] != 0) return;
    const uint32_t end = skip[k];
    uint32_t slot = 1u + koff[k];
    for (uint32_t ch = (uint32_t)k + 1; ch < end; ch = skip[ch], ++slot)
        if (CHK_IDX(slot, nnodes)) write_rec(krec, slot, ch, level, first, cnt, nk, koff, cm32, tab);
}

// Groups: a node with more than G particles emits its children's particle
// ranges, merging children of an aligned block of octants (an x pair, an xy quad)
// while all of them and their sum stay within G: the union of such octants is a
// box that holds no other child's particles, so a merged group never spans a
// denser sibling.  A bucket leaf with more than G particles is cut into runs of
// G; a root with at most G particles is one group.  Runs are contiguous in
// sorted particle order.
// Appends a group (the list holds at most n groups: every group has a particle).
__device__ __forceinline__ void push_group(int2 *__restrict__ groups, uint32_t *__restrict__ ngroups, size_t n,
                                           int2 g) {
    const uint32_t slot = atomicAdd(ngroups, 1u);
    if (CHK_IDX(slot, n) && CHK(g.x >= 0 && g.y > 0 && (size_t)g.x + (size_t)g.y <= n, DERR_TREE)) groups[slot] = g;
}

__global__ void k_groups(size_t nnodes, size_t n, uint32_t G, const uint8_t *__restrict__ level,
                         const uint32_t *__restrict__ first, const uint32_t *__restrict__ cnt,
                         const uint32_t *__restrict__ skip, const uint64_t *__restrict__ khi,
                         const uint64_t *__restrict__ klo, int2 *__restrict__ groups,
                         uint32_t *__restrict__ ngroups) {
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nnodes) return;
    const uint32_t ck = sub_count((uint32_t)k, nnodes, n, first, skip);
    if (ck <= G) {
        if (k == 0) push_group(groups, ngroups, n, make_int2((int)first[0], (int)ck));
        return;
    }
    if (cnt[k] != 0) {
        for (uint32_t j = 0; j < ck; j += G)
            push_group(groups, ngroups, n, make_int2((int)(first[k] + j), (int)min(G, ck - j)));
        return;
    }
    uint32_t c8[8], f8[8];
    for (int o = 0; o < 8; ++o) c8[o] = 0u, f8[o] = 0u;
    const int L = level[k] + 1;
    const uint32_t end = skip[k];
    for (uint32_t ch = (uint32_t)k + 1; ch < end; ch = skip[ch]) {
        const uint32_t f = first[ch];
        const int o = octant_at(khi[f], klo[f], L);
        c8[o] = sub_count(ch, nnodes, n, first, skip);
        f8[o] = f;
    }
    for (int a = 0; a < 8;) {
        int size = 4;
        for (;; size >>= 1) {
            if (a % size) continue;
            uint32_t tot = 0;
            bool ok = true;
            for (int o = a; o < a + size; ++o) {
                ok = ok && c8[o] <= G;
                tot += c8[o];
            }
            if ((ok && tot <= G) || size == 1) break;
        }
        uint32_t tot = 0, f0 = 0;
        bool ok = true;
        for (int o = a + size - 1; o >= a; --o) {
            ok = ok && c8[o] <= G;
            tot += c8[o];
            if (c8[o]) f0 = f8[o];
        }
        if (ok && tot > 0u) push_group(groups, ngroups, n, make_int2((int)f0, (int)tot));
        a += size;
    }
}

__device__ __forceinline__ float warp_min(float v) {
    for (int o = 16; o; o >>= 1) v = fminf(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
    return v;
}
__device__ __forceinline__ float warp_max(float v) {
    for (int o = 16; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
    return v;
}

// Every lane adds the list's monopole terms to its NPL particles: packed f32x2
// over a particle pair (NPL 2), scalar f32 for one particle.  GUARD (unsoftened
// runs) keeps r^2 > 0, so a particle's own leaf adds exactly zero.
template <int NPL, bool GUARD, int NP = (NPL >= 2 ? NPL / 2 : 1)>
__device__ __forceinline__ void group_eval(const float4 *__restrict__ il, int cnt, const f2 *nx, const f2 *ny,
                                           const f2 *nz, float eps2, f2 *ax, f2 *ay, f2 *az) {
    if constexpr (NPL >= 2) {  // NP particle pairs per lane (fewer than NPL/2 when the group leaves slots empty)
        const f2 e2 = pk(eps2, eps2);
#pragma unroll (NP == 1 ? 4 : 2)
        for (int k = 0; k < cnt; ++k) {
            const float4 a = il[2 * k], b = il[2 * k + 1];
            const f2 sx = pk(a.x, a.y), sy = pk(a.z, a.w), sz = pk(b.x, b.y), sm = pk(b.z, b.w);
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                const f2 dx = add2(sx, nx[p]), dy = add2(sy, ny[p]), dz = add2(sz, nz[p]);
                f2 r2 = fma2(dx, dx, e2);
                r2 = fma2(dy, dy, r2);
                r2 = fma2(dz, dz, r2);
                float ra, rb;
                upk(r2, ra, rb);
                if (GUARD) { ra = fmaxf(ra, 1e-24f); rb = fmaxf(rb, 1e-24f); }
                const f2 ri = pk(rsqrt_approx(ra), rsqrt_approx(rb));
                const f2 f = mul2(mul2(sm, ri), mul2(ri, ri));
                ax[p] = fma2(f, dx, ax[p]);
                ay[p] = fma2(f, dy, ay[p]);
                az[p] = fma2(f, dz, az[p]);
            }
        }
    } else {
        float x0, x1, y0, y1, z0, z1, fx, fy, fz, u;
        upk(nx[0], x0, x1); upk(ny[0], y0, y1); upk(nz[0], z0, z1);
        upk(ax[0], fx, u); upk(ay[0], fy, u); upk(az[0], fz, u);
#pragma unroll 4
        for (int k = 0; k < cnt; ++k) {
            const float4 a = il[2 * k], b = il[2 * k + 1];
            const float dx = a.x + x0, dy = a.z + y0, dz = b.x + z0;
            float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
            if (GUARD) r2 = fmaxf(r2, 1e-24f);
            const float ri = rsqrt_approx(r2);
            const float sm = b.z * ri * (ri * ri);
            fx = fmaf(sm, dx, fx);
            fy = fmaf(sm, dy, fy);
            fz = fmaf(sm, dz, fz);
        }
        ax[0] = pk(fx, 0.f); ay[0] = pk(fy, 0.f); az[0] = pk(fz, 0.f);
    }
}

// The per-particle f32 walk (k_walk<1>'s loop) of one particle per lane: the
// group walk's fallback for groups whose box lies close to much denser matter.
__device__ __forceinline__ void walk_lanes_f32(size_t t, bool active, size_t nnodes, const int4 *__restrict__ meta,
                                               const float4 *__restrict__ cm32, const float4 *__restrict__ p32,
                                               const float *s2f, float theta2f, float eps2f, float &fx, float &fy,
                                               float &fz) {
    float qx = 0.f, qy = 0.f, qz = 0.f;
    if (active) {
        const float4 q = p32[t];
        qx = q.x; qy = q.y; qz = q.z;
    }
    uint32_t next = active ? 0u : 0xFFFFFFFFu;
    for (;;) {
        const uint32_t m = __reduce_min_sync(0xFFFFFFFFu, next);
        if ((size_t)m >= nnodes) break;
        if (next != m) continue;
        const int4 mt = meta[m];
        if (mt.z > 0) {
            for (int j = mt.y; j < mt.y + mt.z; ++j) {
                if ((size_t)j == t) continue;
                const float4 q = p32[j];
                if (q.w != 0.f) add_force32(qx, qy, qz, q.x, q.y, q.z, q.w, eps2f, fx, fy, fz);
            }
            next = (uint32_t)mt.x;
        } else {
            const float4 c = cm32[m];
            if (c.w == 0.f) {
                next = (uint32_t)mt.x;
            } else {
                const float dx = c.x - qx, dy = c.y - qy, dz = c.z - qz;
                const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                if (s2f[mt.w] < theta2f * d2) {
                    add_force32(qx, qy, qz, c.x, c.y, c.z, c.w, eps2f, fx, fy, fz);
                    next = (uint32_t)mt.x;
                } else {
                    next = m + 1;
                }
            }
        }
    }
}

template <int NPL, bool GUARD>
__global__ void __launch_bounds__(GW_WARPS * 32) k_walk_group(const int2 *__restrict__ groups,
                                                             uint32_t *__restrict__ gcount,
                                                             const float4 *__restrict__ krec,
                                                             const float4 *__restrict__ p32, float theta2f,
                                                             float eps2f, size_t n, size_t nnodes,
                                                             const int4 *__restrict__ meta,
                                                             const float4 *__restrict__ cm32, const S2Table tab,
                                                             int budget, const AccOut out,
                                                             unsigned *__restrict__ err) {
    constexpr unsigned FULL = 0xFFFFFFFFu;
    __shared__ GroupSmem smem[GW_WARPS];
    const int lane = threadIdx.x & 31;
    uint32_t *stack = smem[threadIdx.x >> 5].stack;
    float4 *il = smem[threadIdx.x >> 5].il;
    const unsigned lt = (1u << lane) - 1u;
    const uint32_t ngroups = gcount[0];
    for (;;) {
        uint32_t g = 0;
        if (lane == 0) g = atomicAdd(gcount + 1, 1u);
        g = __shfl_sync(FULL, g, 0);
        if (g >= ngroups) break;
        const int2 gr = groups[g];
        if (!CHK(gr.x >= 0 && gr.y > 0 && gr.y <= 32 * NPL && (size_t)gr.x + (size_t)gr.y <= n, DERR_BOUNDS))
            continue;  // warp-uniform: every lane read the same group
        constexpr int NQ = NPL < 2 ? 2 : NPL;  // particle slots per lane (the scalar form pads to a pair)
        constexpr int NP = NQ / 2;
        float px[NQ], py[NQ], pz[NQ];
        float lox = INFINITY, loy = INFINITY, loz = INFINITY, hix = -INFINITY, hiy = -INFINITY, hiz = -INFINITY;
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            const int k = q * 32 + lane;
            const float4 p = p32[gr.x + (q < NPL && k < gr.y ? k : 0)];
            px[q] = p.x; py[q] = p.y; pz[q] = p.z;
            lox = fminf(lox, p.x); loy = fminf(loy, p.y); loz = fminf(loz, p.z);
            hix = fmaxf(hix, p.x); hiy = fmaxf(hiy, p.y); hiz = fmaxf(hiz, p.z);
        }
        lox = warp_min(lox); loy = warp_min(loy); loz = warp_min(loz);
        hix = warp_max(hix); hiy = warp_max(hiy); hiz = warp_max(hiz);
        f2 nx[NP], ny[NP], nz[NP], ax[NP], ay[NP], az[NP];
        // a 128-slot group with at most 64 particles uses only the first slot pair of each lane
        const bool half = NPL == 4 && gr.y <= 64;
        auto eval = [&](const float4 *list, int count) {
            if (half) group_eval<NPL, GUARD, 1>(list, count, nx, ny, nz, eps2f, ax, ay, az);
            else group_eval<NPL, GUARD>(list, count, nx, ny, nz, eps2f, ax, ay, az);
        };
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            nx[p] = pk(-px[2 * p], -px[2 * p + 1]);
            ny[p] = pk(-py[2 * p], -py[2 * p + 1]);
            nz[p] = pk(-pz[2 * p], -pz[2 * p + 1]);
            ax[p] = ay[p] = az[p] = 0ull;
        }
        int top = 1, nil = 0;
        if (lane == 0) stack[0] = 0u;  // the root: slot 0, one node
        __syncwarp();
        // a group that needs more than `budget` iterations (its box lies close to much
        // denser matter, which it would open down to the particles) is walked per particle
        int iters = 0;
        long long terms = 0;  // list entries evaluated (each against every particle of the group)
        bool fallback = false;
        while (top > 0) {
            if (++iters > budget) {
                fallback = true;
                break;
            }
            // pop whole ranges from the top, at most 32 nodes
            const uint32_t e = lane < top ? stack[top - 1 - lane] : 0u;
            const int nkl = lane < top ? (int)(e & 7u) + 1 : 0;
            int cum = nkl;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(FULL, cum, o);
                if (lane >= o) cum += v;
            }
            const bool take = lane < top && cum <= 32;
            const int kr = __popc(__ballot_sync(FULL, take));
            const int total = __shfl_sync(FULL, cum, kr - 1);
            const unsigned starts = __reduce_or_sync(FULL, take ? (1u << (cum - nkl)) : 0u);
            top -= kr;
            __syncwarp();
            const bool has = lane < total;
            const unsigned upto = lane == 31 ? FULL : ((2u << lane) - 1u);
            const int r = max(__popc(starts & upto) - 1, 0);
            const uint32_t er = __shfl_sync(FULL, e, r);
            const int sr = __shfl_sync(FULL, cum - nkl, r);
            float4 A = make_float4(0.f, 0.f, 0.f, 0.f);
            int4 B = make_int4(0, 0, 0, 0);
            if (has) {
                const size_t slot = (size_t)(er >> 3) + (size_t)(lane - sr);
                if (CHK_IDX(slot, nnodes)) {  // a bad slot reads as an empty node (A.w == 0)
                    A = krec[2 * slot];
                    B = reinterpret_cast<const int4 *>(krec)[2 * slot + 1];
                }
            }
            bool accept = false, open = false, bucket = false;
            if (has && A.w != 0.f) {
                if (B.x == -1) {
                    accept = true;
                } else if (B.x == -2) {
                    bucket = true;
                } else {
                    const float dx = fmaxf(fmaxf(lox - A.x, A.x - hix), 0.f);
                    const float dy = fmaxf(fmaxf(loy - A.y, A.y - hiy), 0.f);
                    const float dz = fmaxf(fmaxf(loz - A.z, A.z - hiz), 0.f);
                    const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                    if (__int_as_float(B.w) < theta2f * d2) accept = true;
                    else open = true;
                }
            }
            const unsigned om = __ballot_sync(FULL, open);
            if (top + __popc(om) > GW_SCAP) {  // unreachable by the bound above; flagged, never written
                if (lane == 0) atomicOr(err, DERR_STACK_OVERFLOW);
            } else {
                if (open) stack[top + __popc(om & lt)] = ((uint32_t)B.x << 3) | (uint32_t)(B.y - 1);
                top += __popc(om);
            }
            const unsigned am = __ballot_sync(FULL, accept);
            if (accept) {
                float4 *s = il + 2 * (nil + __popc(am & lt));
                s[0] = make_float4(A.x, A.x, A.y, A.y);
                s[1] = make_float4(A.z, A.z, A.w, A.w);
            }
            nil += __popc(am);
            unsigned bm = __ballot_sync(FULL, bucket);
            while (bm) {  // leaves of coincident-key particles (rare): members one by one
                const int b = __ffs(bm) - 1;
                bm &= bm - 1;
                const int bf = __shfl_sync(FULL, B.y, b);
                const int bc = CHK(bf >= 0 && (size_t)bf + (size_t)__shfl_sync(FULL, B.z, b) <= n, DERR_BOUNDS)
                                   ? __shfl_sync(FULL, B.z, b) : 0;
                for (int j0 = 0; j0 < bc; j0 += 32) {
                    if (nil > GW_ICAP - 32) {
                        __syncwarp();
                        terms += nil;
                        eval(il, nil);
                        nil = 0;
                        __syncwarp();
                    }
                    const int j = j0 + lane;
                    const float4 q = j < bc ? p32[bf + j] : make_float4(0.f, 0.f, 0.f, 0.f);
                    const bool ok = j < bc && q.w != 0.f;
                    const unsigned qm = __ballot_sync(FULL, ok);
                    if (ok) {
                        float4 *s = il + 2 * (nil + __popc(qm & lt));
                        s[0] = make_float4(q.x, q.x, q.y, q.y);
                        s[1] = make_float4(q.z, q.z, q.w, q.w);
                    }
                    nil += __popc(qm);
                }
            }
            __syncwarp();
            if (nil > GW_ICAP - 32) {
                terms += nil;
                eval(il, nil);
                nil = 0;
                __syncwarp();
            }
        }
        float fx[NQ], fy[NQ], fz[NQ];
        if (lane == 0) {
            atomicAdd(reinterpret_cast<unsigned long long *>(err + EW_BH_ITERS), (unsigned long long)iters);
            atomicAdd(err + EW_BH_GROUPS, 1u);
            if (fallback) atomicAdd(err + EW_BH_FALLBACKS, 1u);
            else atomicAdd(reinterpret_cast<unsigned long long *>(err + EW_BH_TERMS),
                           (unsigned long long)(terms + nil) * (unsigned long long)gr.y);
        }
        if (fallback) {
#pragma unroll
            for (int q = 0; q < NPL; ++q) {
                const int k = q * 32 + lane;
                fx[q] = fy[q] = fz[q] = 0.f;
                walk_lanes_f32((size_t)gr.x + k, k < gr.y, nnodes, meta, cm32, p32, tab.s2f, theta2f, eps2f, fx[q],
                               fy[q], fz[q]);
            }
        } else {
            if (nil) eval(il, nil);
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                upk(ax[p], fx[2 * p], fx[2 * p + 1]);
                upk(ay[p], fy[2 * p], fy[2 * p + 1]);
                upk(az[p], fz[2 * p], fz[2 * p + 1]);
            }
        }
        __syncwarp();
#pragma unroll
        for (int q = 0; q < NPL; ++q) {
            const int k = q * 32 + lane;
            if (k < gr.y) store_acc(out, (size_t)gr.x + k, fx[q], fy[q], fz[q]);
        }
    }
}

inline int nblk(size_t n, int t = 256) { return (int)std::max<size_t>(1, (n + t - 1) / t); }

}  // namespace

Tree *tree_of(Ctx *c) {
    if (!c->tree) c->tree = new Tree();
    return static_cast<Tree *>(c->tree);
}

void tree_free(Ctx *c) {
    Tree *t = static_cast<Tree *>(c->tree);
    if (!t) return;
    DevBuf *all[] = {&t->bb, &t->bbpart, &t->khi, &t->klo, &t->khi2, &t->klo2, &t->perm, &t->perm2, &t->iota,
                     &t->iota2, &t->delta, &t->nown, &t->off, &t->total, &t->level, &t->first, &t->cnt, &t->skip,
                     &t->mass, &t->comx, &t->comy, &t->comz, &t->boxx, &t->boxy, &t->boxz, &t->sx, &t->sy,
                     &t->sz, &t->sm, &t->pos32, &t->cm32, &t->cm64, &t->meta, &t->pos32lo, &t->mrec, &t->nk, &t->koff, &t->krec,
                     &t->groups, &t->gcount, &t->parent, &t->arrive, &t->mo32, &t->leaf_of};
    for (DevBuf *b : all)
        if (b->ptr) cudaFree(b->ptr);
    delete t;
    c->tree = nullptr;
}

namespace {
// Structural invariants of the node arrays (checked build): pre-order with skip
// pointers that move forward, a root at depth 0 over every particle, contiguous
// particle ranges, children one level below their parent (1 to 8 of them,
// tiling its range in order), leaves of one particle or buckets at depth 42.
__global__ void k_tree_check(size_t nnodes, size_t n, const uint8_t *__restrict__ level,
                             const uint32_t *__restrict__ first, const uint32_t *__restrict__ cnt,
                             const uint32_t *__restrict__ skip) {
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nnodes) return;
    const uint32_t s = skip[k], f = first[k], c = cnt[k];
    const int L = level[k];
    bool ok = s > k && s <= nnodes && f < n && L <= MAXL;
    if (k == 0) ok = ok && L == 0 && f == 0 && s == nnodes;
    if (ok) {
        const size_t pe = s < nnodes ? (size_t)first[s] : n;
        ok = pe > f && pe <= n;
        if (ok && c > 0) {
            ok = s == k + 1 && c == pe - f && (c == 1 || L == MAXL);
        } else if (ok) {
            ok = pe - f >= 2 && k + 1 < s;
            uint32_t ch = (uint32_t)k + 1;
            int nch = 0;
            size_t pf = f;
            while (ok && ch < s) {
                const uint32_t sk = skip[ch];
                ok = level[ch] == L + 1 && first[ch] == pf && sk > ch && sk <= s && ++nch <= 8;
                pf = sk < nnodes ? (size_t)first[sk] : n;
                ch = sk;
            }
            ok = ok && ch == s && pf == pe;
        }
    }
    if (!CHK(ok, DERR_TREE)) return;
}
}  // namespace

// Checked build: verifies the node arrays before any kernel follows their links,
// and fails the call if they are broken.
static gvs_status tree_check(Ctx *c, Tree *t, size_t nnodes) {
#ifdef GVS_CHECKED
    k_tree_check<<<nblk(nnodes), 256, 0, c->stream>>>(nnodes, c->n, as<uint8_t>(t->level), as<uint32_t>(t->first),
                                                      as<uint32_t>(t->cnt), as<uint32_t>(t->skip));
    c->prof.launches += 1;
    GVS_TRY(check_launch(c, "tree check"));
    const unsigned f = checked_take_bh(c->stream);
    if (f) return fail(c, GVS_ERR_DEVICE, "tree build: invariants violated (device flags 0x%x)", f);
#else
    (void)c; (void)t; (void)nnodes;
#endif
    return GVS_OK;
}

// Builds (or reuses) the tree of the resident positions.
gvs_status tree_build(Ctx *c) {
    Tree *t = tree_of(c);
    const size_t n = c->n;
    if (n == 0) return fail(c, GVS_ERR_STATE, "tree build with no particles");
    if (t->version == c->pos_version && t->n == n) return GVS_OK;
    cudaStream_t st = c->stream;
    GVS_CUDA(c, ensure(c, t->bb, 16 * sizeof(double)));
    GVS_TRY(bbox_minmax(c, as<double>(t->bb), t->bbpart));
    k_root<<<1, 1, 0, st>>>(as<double>(t->bb));
    const size_t b8 = n * 8, b4 = n * 4;
    GVS_CUDA(c, ensure(c, t->khi, b8)); GVS_CUDA(c, ensure(c, t->klo, b8));
    GVS_CUDA(c, ensure(c, t->khi2, b8)); GVS_CUDA(c, ensure(c, t->klo2, b8));
    GVS_CUDA(c, ensure(c, t->perm, b4)); GVS_CUDA(c, ensure(c, t->perm2, b4));
    GVS_CUDA(c, ensure(c, t->iota, b4)); GVS_CUDA(c, ensure(c, t->iota2, b4));
    // keys: the high word (levels 1..21) for everyone, sorted; the low word only
    // for runs of equal high words, which are then sorted by it.  A run longer
    // than RUN_MAX (hundreds of near-coincident points) takes the full path: both
    // words for everyone, sorted by low then (stably) by high.
    GVS_CUDA(c, ensure(c, t->total, 16));
    k_keys<21><<<nblk(n), 256, 0, st>>>(as<double>(c->x), as<double>(c->y), as<double>(c->z), n, as<double>(t->bb),
                                        as<uint64_t>(t->khi), nullptr, as<uint32_t>(t->perm));
    c->prof.launches += 2;
    GVS_TRY(check_launch(c, "tree keys"));
    uint64_t *khi_s;
    uint32_t *perm_s;
    GVS_TRY(radix_sort_u64(c, as<uint64_t>(t->khi), as<uint32_t>(t->perm), as<uint64_t>(t->khi2),
                           as<uint32_t>(t->perm2), n, 0, 64, &khi_s, &perm_s));
    if (khi_s != as<uint64_t>(t->khi)) std::swap(t->khi, t->khi2);
    if (perm_s != as<uint32_t>(t->perm)) std::swap(t->perm, t->perm2);
    uint32_t stat[2] = {0, 0};
    GVS_CUDA(c, cudaMemsetAsync(t->total.ptr, 0, 16, st));
    k_keys_lo<<<nblk(n), 256, 0, st>>>(as<uint64_t>(t->khi), as<uint32_t>(t->perm), as<double>(c->x),
                                       as<double>(c->y), as<double>(c->z), n, as<double>(t->bb),
                                       as<uint64_t>(t->klo), as<uint32_t>(t->total) + 2);
    GVS_CUDA(c, cudaMemcpyAsync(stat, as<uint32_t>(t->total) + 2, 8, cudaMemcpyDeviceToHost, st));
    GVS_CUDA(c, cudaStreamSynchronize(st));
    c->prof.launches += 1;
    if (stat[1]) {
        k_keys<MAXL><<<nblk(n), 256, 0, st>>>(as<double>(c->x), as<double>(c->y), as<double>(c->z), n,
                                              as<double>(t->bb), as<uint64_t>(t->khi), as<uint64_t>(t->klo),
                                              as<uint32_t>(t->perm));
        c->prof.launches += 1;
        uint64_t *klo_s;
        uint32_t *perm1;
        GVS_TRY(radix_sort_u64(c, as<uint64_t>(t->klo), as<uint32_t>(t->perm), as<uint64_t>(t->klo2),
                               as<uint32_t>(t->perm2), n, 0, 64, &klo_s, &perm1));
        // khi in lo-sorted order, then the stable sort by hi carrying lo-order slots
        uint64_t *khi_g = as<uint64_t>(t->khi2);
        k_gather<uint64_t><<<nblk(n), 256, 0, st>>>(as<uint64_t>(t->khi), perm1, khi_g, n);
        k_iota<<<nblk(n), 256, 0, st>>>(as<uint32_t>(t->iota), n);
        c->prof.launches += 2;
        uint32_t *slot;
        GVS_TRY(radix_sort_u64(c, khi_g, as<uint32_t>(t->iota), as<uint64_t>(t->khi), as<uint32_t>(t->iota2), n, 0,
                               64, &khi_s, &slot));
        uint32_t *perm_final = (perm1 == as<uint32_t>(t->perm)) ? as<uint32_t>(t->perm2) : as<uint32_t>(t->perm);
        uint64_t *klo_final = (klo_s == as<uint64_t>(t->klo)) ? as<uint64_t>(t->klo2) : as<uint64_t>(t->klo);
        k_gather<uint32_t><<<nblk(n), 256, 0, st>>>(perm1, slot, perm_final, n);
        k_gather<uint64_t><<<nblk(n), 256, 0, st>>>(klo_s, slot, klo_final, n);
        c->prof.launches += 2;
        if (perm_final != as<uint32_t>(t->perm)) std::swap(t->perm, t->perm2);
        if (klo_final != as<uint64_t>(t->klo)) std::swap(t->klo, t->klo2);
        if (khi_s != as<uint64_t>(t->khi)) std::swap(t->khi, t->khi2);
    } else if (stat[0]) {
        k_sort_runs<<<nblk(n), 256, 0, st>>>(as<uint64_t>(t->khi), n, as<uint64_t>(t->klo), as<uint32_t>(t->perm));
        c->prof.launches += 1;
    }
    GVS_TRY(check_launch(c, "tree key runs"));
    uint64_t *KH = as<uint64_t>(t->khi), *KL = as<uint64_t>(t->klo);
    uint32_t *P = as<uint32_t>(t->perm);
    // node enumeration
    GVS_CUDA(c, ensure(c, t->delta, (n + 1) * 4));
    GVS_CUDA(c, ensure(c, t->nown, (n + 1) * 4));
    GVS_CUDA(c, ensure(c, t->off, (n + 1) * 4));
    k_delta<<<nblk(n + 1), 256, 0, st>>>(KH, KL, n, as<int>(t->delta));
    k_nown<<<nblk(n + 1), 256, 0, st>>>(as<int>(t->delta), n, as<uint32_t>(t->nown));
    c->prof.launches += 2;
    GVS_TRY(exclusive_scan_u32(c, as<uint32_t>(t->nown), as<uint32_t>(t->off), n + 1, as<uint32_t>(t->total)));
    uint32_t nn = 0;
    GVS_CUDA(c, cudaMemcpyAsync(&nn, t->total.ptr, 4, cudaMemcpyDeviceToHost, st));
    GVS_CUDA(c, cudaMemcpyAsync(t->root, as<double>(t->bb) + 6, 4 * sizeof(double), cudaMemcpyDeviceToHost, st));
    GVS_CUDA(c, cudaStreamSynchronize(st));
    const size_t nnodes = nn;
    t->nnodes = nnodes;
    GVS_CUDA(c, ensure(c, t->level, nnodes));
    GVS_CUDA(c, ensure(c, t->first, nnodes * 4)); GVS_CUDA(c, ensure(c, t->cnt, nnodes * 4));
    GVS_CUDA(c, ensure(c, t->skip, nnodes * 4));
    k_nodes<<<nblk(n), 256, 0, st>>>(KH, KL, as<int>(t->delta), as<uint32_t>(t->off), n, as<uint8_t>(t->level),
                                     as<uint32_t>(t->first), as<uint32_t>(t->cnt), as<uint32_t>(t->skip), nnodes);
    if (kChecked) GVS_TRY(tree_check(c, t, nnodes));
    // sorted particle data
    GVS_CUDA(c, ensure(c, t->sx, b8)); GVS_CUDA(c, ensure(c, t->sy, b8));
    GVS_CUDA(c, ensure(c, t->sz, b8)); GVS_CUDA(c, ensure(c, t->sm, b8));
    k_gather<double><<<nblk(n), 256, 0, st>>>(as<double>(c->x), P, as<double>(t->sx), n);
    k_gather<double><<<nblk(n), 256, 0, st>>>(as<double>(c->y), P, as<double>(t->sy), n);
    k_gather<double><<<nblk(n), 256, 0, st>>>(as<double>(c->z), P, as<double>(t->sz), n);
    k_gather<double><<<nblk(n), 256, 0, st>>>(as<double>(c->m), P, as<double>(t->sm), n);
    c->prof.launches += 5;
    GVS_TRY(check_launch(c, "tree nodes"));
    GVS_CUDA(c, ensure(c, t->parent, nnodes * 4));
    GVS_CUDA(c, ensure(c, t->nk, nnodes * 4));
    GVS_CUDA(c, ensure(c, t->arrive, nnodes * 4));
    GVS_CUDA(c, ensure(c, t->leaf_of, n * 4));
    k_links<<<nblk(nnodes), 256, 0, st>>>(nnodes, as<uint32_t>(t->first), as<uint32_t>(t->cnt), as<uint32_t>(t->skip),
                                          as<uint32_t>(t->parent), as<uint32_t>(t->nk), as<uint32_t>(t->leaf_of), n);
    c->prof.launches += 1;
    GVS_TRY(check_launch(c, "tree links"));
    t->n = n;
    t->version = c->pos_version;
    t->precision = -1;
    return GVS_OK;
}

// The f64 moments (mass, centre of mass) of the current tree, on first request:
// the f64 and mixed walks and the tree export read them; the FP32 walk has its own.
static gvs_status tree_moments64(Ctx *c, Tree *t) {
    if (t->m64_version == t->version) return GVS_OK;
    const size_t nnodes = t->nnodes;
    cudaStream_t st = c->stream;
    GVS_CUDA(c, ensure(c, t->mass, nnodes * 8)); GVS_CUDA(c, ensure(c, t->comx, nnodes * 8));
    GVS_CUDA(c, ensure(c, t->comy, nnodes * 8)); GVS_CUDA(c, ensure(c, t->comz, nnodes * 8));
    GVS_CUDA(c, cudaMemsetAsync(t->arrive.ptr, 0, nnodes * 4, st));
    k_moments_up<<<nblk(nnodes), 256, 0, st>>>(nnodes, as<uint32_t>(t->first), as<uint32_t>(t->cnt),
                                               as<uint32_t>(t->skip), as<uint32_t>(t->parent), as<uint32_t>(t->nk),
                                               as<uint32_t>(t->arrive), as<double>(t->sx), as<double>(t->sy),
                                               as<double>(t->sz), as<double>(t->sm), as<double>(t->mass),
                                               as<double>(t->comx), as<double>(t->comy), as<double>(t->comz));
    c->prof.launches += 1;
    GVS_TRY(check_launch(c, "tree moments"));
    t->m64_version = t->version;
    return GVS_OK;
}

// First child slot of every node (exclusive scan of the child counts).
static gvs_status koff_prepare(Ctx *c, Tree *t) {
    if (t->koff_version == t->version) return GVS_OK;
    GVS_CUDA(c, ensure(c, t->koff, t->nnodes * 4));
    GVS_TRY(exclusive_scan_u32(c, as<uint32_t>(t->nk), as<uint32_t>(t->koff), t->nnodes, nullptr));
    t->koff_version = t->version;
    return GVS_OK;
}

// Child-slot records and particle groups of the current tree for the group walk.
static gvs_status group_prepare(Ctx *c, Tree *t, int gsize) {
    if (t->grp_version == t->version && t->grp_size == gsize) return GVS_OK;
    const size_t nn = t->nnodes, n = t->n;
    cudaStream_t st = c->stream;
    GVS_CUDA(c, ensure(c, t->krec, nn * 2 * sizeof(float4)));
    GVS_CUDA(c, ensure(c, t->groups, n * sizeof(int2)));
    GVS_CUDA(c, ensure(c, t->gcount, 16));
    GVS_TRY(koff_prepare(c, t));
    S2f tab;
    for (int L = 0; L <= MAXL; ++L) {
        const double s = 2.0 * std::ldexp(t->root[3], -L);
        tab.s2[L] = (float)(s * s);
    }
    k_krec<<<nblk(nn), 256, 0, st>>>(nn, as<uint8_t>(t->level), as<uint32_t>(t->first), as<uint32_t>(t->cnt),
                                     as<uint32_t>(t->skip), as<uint32_t>(t->nk), as<uint32_t>(t->koff),
                                     as<float4>(t->cm32), tab, as<float4>(t->krec));
    GVS_CUDA(c, cudaMemsetAsync(t->gcount.ptr, 0, 8, st));
    k_groups<<<nblk(nn), 256, 0, st>>>(nn, n, (uint32_t)gsize, as<uint8_t>(t->level), as<uint32_t>(t->first),
                                       as<uint32_t>(t->cnt), as<uint32_t>(t->skip), as<uint64_t>(t->khi),
                                       as<uint64_t>(t->klo), as<int2>(t->groups), as<uint32_t>(t->gcount));
    c->prof.launches += 2;
    GVS_TRY(check_launch(c, "group walk setup"));
    t->grp_version = t->version;
    t->grp_size = gsize;
    return GVS_OK;
}

gvs_status bh_forces(Ctx *c, double eps, double theta, int precision, bool accumulate) {
    const size_t n = c->n;
    if (n == 0) return GVS_OK;
    GVS_TRY(tree_build(c));
    Tree *t = tree_of(c);
    cudaStream_t st = c->stream;
    const size_t nnodes = t->nnodes;
    // walk mode: 0 f64 (FP64, FP64_EXACT), 1 f32 (FP32), 2 mixed (MIXED)
    const int mode = (precision == GVS_PREC_FP64_EXACT || precision == GVS_PREC_FP64) ? 0
                     : precision == GVS_PREC_FP32 ? 1 : 2;
    GVS_CUDA(c, ensure(c, t->meta, nnodes * sizeof(int4)));
    if (mode != 1) GVS_CUDA(c, ensure(c, t->cm64, nnodes * sizeof(double4)));
    if (mode != 0) GVS_CUDA(c, ensure(c, t->pos32, n * sizeof(float4)));
    if (mode == 1) GVS_CUDA(c, ensure(c, t->cm32, nnodes * sizeof(float4)));
    if (mode == 2) {
        GVS_CUDA(c, ensure(c, t->mrec, nnodes * 3 * sizeof(float4)));
        GVS_CUDA(c, ensure(c, t->pos32lo, n * sizeof(float4)));
    }
    if (t->precision != mode + 1) {
        if (mode != 1) GVS_TRY(tree_moments64(c, t));
        k_pack_nodes<<<nblk(nnodes), 256, 0, st>>>(nnodes, as<uint8_t>(t->level), as<uint32_t>(t->first),
                                                    as<uint32_t>(t->cnt), as<uint32_t>(t->skip), as<double>(t->mass),
                                                    as<double>(t->comx), as<double>(t->comy), as<double>(t->comz),
                                                    mode != 1 ? as<double4>(t->cm64) : nullptr,
                                                    as<int4>(t->meta), mode == 2 ? as<float4>(t->mrec) : nullptr);
        if (mode != 0)
            k_pack_particles<<<nblk(n), 256, 0, st>>>(n, as<double>(t->sx), as<double>(t->sy), as<double>(t->sz),
                                                      as<double>(t->sm), as<float4>(t->pos32),
                                                      mode == 2 ? as<float4>(t->pos32lo) : nullptr);
        c->prof.launches += mode != 0 ? 2 : 1;
        if (mode == 1) {  // f32 moments from the f32 particles
            GVS_CUDA(c, ensure(c, t->mo32, nnodes * sizeof(float4)));
            GVS_CUDA(c, cudaMemsetAsync(t->arrive.ptr, 0, nnodes * 4, st));
            k_moments32_up<<<nblk(nnodes), 256, 0, st>>>(nnodes, as<uint32_t>(t->first), as<uint32_t>(t->cnt),
                                                         as<uint32_t>(t->skip), as<uint32_t>(t->parent),
                                                         as<uint32_t>(t->nk), as<uint32_t>(t->arrive),
                                                         as<float4>(t->pos32), as<float4>(t->mo32),
                                                         as<float4>(t->cm32));
            c->prof.launches += 1;
        }
        GVS_TRY(check_launch(c, "walk packing"));
        t->precision = mode + 1;
    }
    S2Table tab;
    for (int L = 0; L <= MAXL; ++L) {
        const double hw = ldexp(t->root[3], -L);  // exact: child half width = parent * 0.5
        const double s = hw * 2.0;
        tab.s2[L] = s * s;
        tab.s2f[L] = (float)(s * s);
        const double rc = theta > 0.0 ? s / theta : INFINITY;  // accept iff d > s / theta
        tab.rcf[L] = (float)std::min(rc, 3.0e38);  // finite: the band's limits stay ordered (no inf - inf)
    }
    const AccOut out{as<uint32_t>(t->perm), as<double>(c->ax), as<double>(c->ay), as<double>(c->az),
                     accumulate ? 1 : 0, n};
    // FP32 with a group size set: the group walk (slot records fit 29 bits)
    // (128-particle groups amortise the walk over more particles; below 2^21 particles
    // they would leave too few groups to fill the GPU)
    const int gsize = c->bh_group >= 0 ? c->bh_group : (n >= (size_t(1) << 21) ? 128 : 64);
    const bool group = mode == 1 && gsize > 0 && nnodes < (size_t(1) << 29);
    if (group) GVS_TRY(group_prepare(c, t, gsize));
    int span = -1;  // profile timing span
    GVS_TRY(prof_begin(c, st, &span));
    if (group) {
        GVS_CUDA(c, cudaMemsetAsync(as<uint32_t>(t->gcount) + 1, 0, 4, st));
        const bool guard = eps == 0.0;
        const float th2 = (float)(theta * theta), e2 = (float)(eps * eps);
        auto launch = [&](auto kern) -> gvs_status {
            int per_sm = 0;
            GVS_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, GW_WARPS * 32, 0));
            kern<<<std::max(1, per_sm) * c->num_sms, GW_WARPS * 32, 0, st>>>(
                as<int2>(t->groups), as<uint32_t>(t->gcount), as<float4>(t->krec), as<float4>(t->pos32), th2, e2,
                n, nnodes, as<int4>(t->meta), as<float4>(t->cm32), tab, c->bh_budget, out, err_ptr(c));
            return GVS_OK;
        };
        if (gsize == 128) GVS_TRY(guard ? launch(k_walk_group<4, true>) : launch(k_walk_group<4, false>));
        else if (gsize == 64) GVS_TRY(guard ? launch(k_walk_group<2, true>) : launch(k_walk_group<2, false>));
        else GVS_TRY(guard ? launch(k_walk_group<1, true>) : launch(k_walk_group<1, false>));
        c->prof.launches += 2;
    } else if (mode == 0)
        k_walk<0><<<nblk(n, 128), 128, 0, st>>>(n, nnodes, as<int4>(t->meta), nullptr, as<double4>(t->cm64),
                                                nullptr, as<double>(t->sx), as<double>(t->sy), as<double>(t->sz),
                                                as<double>(t->sm), tab, theta * theta, eps * eps,
                                                out, nullptr, nullptr, err_ptr(c));
    else if (mode == 1)
        k_walk<1><<<nblk(n, 128), 128, 0, st>>>(n, nnodes, as<int4>(t->meta), as<float4>(t->cm32), nullptr,
                                                as<float4>(t->pos32), as<double>(t->sx), as<double>(t->sy),
                                                as<double>(t->sz), as<double>(t->sm), tab, theta * theta, eps * eps,
                                                out, nullptr, nullptr, err_ptr(c));
    else
        k_walk<2><<<nblk(n, 128), 128, 0, st>>>(n, nnodes, nullptr, nullptr, as<double4>(t->cm64),
                                                as<float4>(t->pos32), as<double>(t->sx), as<double>(t->sy),
                                                as<double>(t->sz), as<double>(t->sm), tab, theta * theta, eps * eps,
                                                out, as<float4>(t->pos32lo), as<float4>(t->mrec), err_ptr(c));
    c->prof.launches += 1;
    GVS_TRY(check_launch(c, "tree walk"));
    if (c->prof.on) {
        GVS_TRY(prof_end(c, span, st, &c->prof.force_ms));
        c->prof.force_launches += 1;
    }
    return GVS_OK;
}

// ---- accessors used by the SPH neighbour search and the tests ------------------
gvs_status tree_view(Ctx *c, TreeView *v) {
    GVS_TRY(tree_build(c));
    Tree *t = tree_of(c);
    v->n = t->n;
    v->nnodes = t->nnodes;
    v->level = as<uint8_t>(t->level);
    v->first = as<uint32_t>(t->first);
    v->cnt = as<uint32_t>(t->cnt);
    v->skip = as<uint32_t>(t->skip);
    v->perm = as<uint32_t>(t->perm);
    v->parent = as<uint32_t>(t->parent);
    v->leaf_of = as<uint32_t>(t->leaf_of);
    if (t->centres_version != t->version) {
        const size_t nn = t->nnodes, n = t->n;
        GVS_CUDA(c, ensure(c, t->boxx, nn * 8));
        GVS_CUDA(c, ensure(c, t->boxy, nn * 8));
        GVS_CUDA(c, ensure(c, t->boxz, nn * 8));
        k_centres<<<nblk(n), 256, 0, c->stream>>>(as<uint64_t>(t->khi), as<uint64_t>(t->klo), as<int>(t->delta),
                                                  as<uint32_t>(t->off), n, as<double>(t->bb), as<double>(t->boxx),
                                                  as<double>(t->boxy), as<double>(t->boxz));
        c->prof.launches += 1;
        GVS_TRY(check_launch(c, "cell centres"));
        t->centres_version = t->version;
    }
    v->bx = as<double>(t->boxx);
    v->by = as<double>(t->boxy);
    v->bz = as<double>(t->boxz);
    v->sx = as<double>(t->sx);
    v->sy = as<double>(t->sy);
    v->sz = as<double>(t->sz);
    v->root_hw = t->root[3];
    return GVS_OK;
}

// Host copy of the tree arrays (for tests): returns node count.
gvs_status tree_export(Ctx *c, size_t cap, uint8_t *level, uint32_t *first, uint32_t *cnt, uint32_t *skip,
                       double *mass, double *com, uint32_t *perm, uint64_t *keys, size_t *nnodes) {
    GVS_TRY(tree_build(c));
    Tree *t = tree_of(c);
    GVS_TRY(tree_moments64(c, t));
    *nnodes = t->nnodes;
    if (cap < t->nnodes) return GVS_OK;
    cudaStream_t st = c->stream;
    const size_t nn = t->nnodes, n = t->n;
    if (level) GVS_CUDA(c, cudaMemcpyAsync(level, t->level.ptr, nn, cudaMemcpyDeviceToHost, st));
    if (first) GVS_CUDA(c, cudaMemcpyAsync(first, t->first.ptr, nn * 4, cudaMemcpyDeviceToHost, st));
    if (cnt) GVS_CUDA(c, cudaMemcpyAsync(cnt, t->cnt.ptr, nn * 4, cudaMemcpyDeviceToHost, st));
    if (skip) GVS_CUDA(c, cudaMemcpyAsync(skip, t->skip.ptr, nn * 4, cudaMemcpyDeviceToHost, st));
    if (mass) GVS_CUDA(c, cudaMemcpyAsync(mass, t->mass.ptr, nn * 8, cudaMemcpyDeviceToHost, st));
    if (com) {
        GVS_CUDA(c, cudaMemcpyAsync(com, t->comx.ptr, nn * 8, cudaMemcpyDeviceToHost, st));
        GVS_CUDA(c, cudaMemcpyAsync(com + nn, t->comy.ptr, nn * 8, cudaMemcpyDeviceToHost, st));
        GVS_CUDA(c, cudaMemcpyAsync(com + 2 * nn, t->comz.ptr, nn * 8, cudaMemcpyDeviceToHost, st));
    }
    if (perm) GVS_CUDA(c, cudaMemcpyAsync(perm, t->perm.ptr, n * 4, cudaMemcpyDeviceToHost, st));
    if (keys) {
        GVS_CUDA(c, cudaMemcpyAsync(keys, t->khi.ptr, n * 8, cudaMemcpyDeviceToHost, st));
        GVS_CUDA(c, cudaMemcpyAsync(keys + n, t->klo.ptr, n * 8, cudaMemcpyDeviceToHost, st));
    }
    GVS_CUDA(c, cudaStreamSynchronize(st));
    return GVS_OK;
}

GVS_CHECKED_UNIT(bh)

}  // namespace gvs
