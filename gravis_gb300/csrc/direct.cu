// direct.cu -- all-pairs softened gravity (BruteForce, crates/sim-core/src/gravity.rs:47-80).
//
// Four forms, one per GVS_PREC_* mode:
//
//  FP64_EXACT  one thread per target i, j ascending over the caller's order,
//              IEEE f64 with no FMA contraction (__dadd_rn/__dmul_rn/__dsqrt_rn/
//              __ddiv_rn).  For every target this performs exactly the
//              operations of the reference loop in the same order (the j<i
//              terms of the symmetric loop equal the gather terms with dx
//              negated, and negation is exact), so results are bit-identical.
//
//  FP64        the tiled kernel below in f64 (double4 j-tiles, FMA, rsqrt
//              refined in f64): the FP64 form of the mixed kernel, used for
//              the "mixed vs FP64" throughput ratio.
//
//  FP32        f32 absolute positions, plain f32 accumulation.
//
//  MIXED       particles are put in Hilbert order and cut into tiles of TJ
//              (= the block size, 128 by default); each tile stores its centre
//              in f64 (as an f32 hi+lo pair) and its members as f32 offsets
//              from that centre (plus the f32 residual of each offset).  For target i and source
//              tile J the kernel forms x_i - c_J = (c_I - c_J) + off_i from the
//              hi/lo pairs, so pair separations are computed from small numbers
//              and keep ~f32 relative precision even in the dense core.  Tiles
//              whose bounding boxes nearly touch the target tile (Chebyshev
//              centre distance < half the sum of the radii) add the residuals
//              (float-float separations), which keeps close pairs accurate.  The
//              per-tile partial force is accumulated in f32 and folded into a
//              (hi, lo) two-sum accumulator, so summation error does not grow
//              with N.  Pair arithmetic uses packed f32x2 FMA/ADD/MUL (two
//              targets per instruction) and one MUFU rsqrt per pair.
//
// Tiled kernels: a block owns NT*IPT consecutive targets (sorted order) and a
// contiguous range of source tiles (grid.y = j-split).  Source tiles stream
// into shared memory through a ring of cp.async.bulk copies completed on
// mbarriers; one elected thread issues them.  Each block writes per-split
// partial sums; a deterministic reduce kernel adds the splits in fixed order
// and scatters the f64 result to the caller's order.
#include "gvs_internal.cuh"

namespace gvs {

namespace {

constexpr int TJ64 = 64;              // particles per f64 tile

// ---------------------------------------------------------------------------
// bounding box (f64 min/max), two passes
// ---------------------------------------------------------------------------
__global__ void k_bbox_part(const double *__restrict__ x, const double *__restrict__ y,
                            const double *__restrict__ z, size_t n, double *__restrict__ part) {
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        double v[3] = {x[i], y[i], z[i]};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            mn[d] = fmin(mn[d], v[d]);
            mx[d] = fmax(mx[d], v[d]);
        }
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        for (int o = 16; o > 0; o >>= 1) {
            mn[d] = fmin(mn[d], __shfl_xor_sync(0xFFFFFFFFu, mn[d], o));
            mx[d] = fmax(mx[d], __shfl_xor_sync(0xFFFFFFFFu, mx[d], o));
        }
    }
    __shared__ double s[32][6];
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0)
        for (int d = 0; d < 3; ++d) { s[w][d] = mn[d]; s[w][3 + d] = mx[d]; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int ww = 1; ww < (int)(blockDim.x >> 5); ++ww)
            for (int d = 0; d < 3; ++d) {
                s[0][d] = fmin(s[0][d], s[ww][d]);
                s[0][3 + d] = fmax(s[0][3 + d], s[ww][3 + d]);
            }
        for (int k = 0; k < 6; ++k) part[blockIdx.x * 6 + k] = s[0][k];
    }
}

// One block of 256 threads folds the per-block parts into part[0..5].
__global__ void __launch_bounds__(256) k_bbox_final(double *part, int nparts) {
    double v[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    for (int b = threadIdx.x; b < nparts; b += blockDim.x)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            v[d] = fmin(v[d], part[b * 6 + d]);
            v[3 + d] = fmax(v[3 + d], part[b * 6 + 3 + d]);
        }
#pragma unroll
    for (int d = 0; d < 3; ++d)
        for (int o = 16; o > 0; o >>= 1) {
            v[d] = fmin(v[d], __shfl_xor_sync(0xFFFFFFFFu, v[d], o));
            v[3 + d] = fmax(v[3 + d], __shfl_xor_sync(0xFFFFFFFFu, v[3 + d], o));
        }
    __shared__ double s[8][6];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 6; ++k) s[w][k] = v[k];
    __syncthreads();  // every thread has read its parts before part[0..5] is written
    if (threadIdx.x == 0) {
        for (int ww = 1; ww < (int)(blockDim.x >> 5); ++ww)
            for (int d = 0; d < 3; ++d) {
                s[0][d] = fmin(s[0][d], s[ww][d]);
                s[0][3 + d] = fmax(s[0][3 + d], s[ww][3 + d]);
            }
        for (int k = 0; k < 6; ++k) part[k] = s[0][k];
    }
}

__global__ void k_hilbert(const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z,
                          size_t n, const double *__restrict__ bb, uint64_t *__restrict__ keys,
                          uint32_t *__restrict__ idx) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double ext = fmax(fmax(bb[3] - bb[0], bb[4] - bb[1]), bb[5] - bb[2]);
    double inv = ext > 0.0 ? 2097151.99 / ext : 0.0;
    uint32_t q[3];
    double v[3] = {x[i], y[i], z[i]};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        double t = (v[d] - bb[d]) * inv;
        t = fmin(fmax(t, 0.0), 2097151.0);
        q[d] = (uint32_t)t;
    }
    keys[i] = hilbert_key(q[0], q[1], q[2]);
    idx[i] = (uint32_t)i;
}

// Small systems (n <= SMALL_ORDER_MAX): the whole Hilbert ordering in one block --
// bounding box, keys (k_hilbert's formula), and a bitonic sort of (key, index)
// pairs in shared memory.  (key, index) pairs are distinct, so the sorted order is
// the stable radix sort's; the permutation is the one the multi-kernel path gives,
// from one launch instead of ~27 (which dominate a step of a thousand particles).
constexpr int SMALL_ORDER_MAX = 8192;

__global__ void __launch_bounds__(1024) k_small_order(const double *__restrict__ x, const double *__restrict__ y,
                                                      const double *__restrict__ z, int n, int P,
                                                      uint32_t *__restrict__ perm) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint64_t *key = reinterpret_cast<uint64_t *>(smem_raw);
    uint32_t *idx = reinterpret_cast<uint32_t *>(key + P);
    __shared__ double red[32][6];
    __shared__ double bb[6];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = tid; i < n; i += blockDim.x) {
        const double v[3] = {x[i], y[i], z[i]};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            mn[d] = fmin(mn[d], v[d]);
            mx[d] = fmax(mx[d], v[d]);
        }
    }
#pragma unroll
    for (int d = 0; d < 3; ++d)
        for (int o = 16; o > 0; o >>= 1) {
            mn[d] = fmin(mn[d], __shfl_xor_sync(0xFFFFFFFFu, mn[d], o));
            mx[d] = fmax(mx[d], __shfl_xor_sync(0xFFFFFFFFu, mx[d], o));
        }
    if (lane == 0)
        for (int d = 0; d < 3; ++d) red[w][d] = mn[d], red[w][3 + d] = mx[d];
    __syncthreads();
    if (tid < 6) {
        double v = red[0][tid];
        for (int ww = 1; ww < (int)(blockDim.x >> 5); ++ww) v = tid < 3 ? fmin(v, red[ww][tid]) : fmax(v, red[ww][tid]);
        bb[tid] = v;
    }
    __syncthreads();
    const double ext = fmax(fmax(bb[3] - bb[0], bb[4] - bb[1]), bb[5] - bb[2]);
    const double inv = ext > 0.0 ? 2097151.99 / ext : 0.0;
    for (int i = tid; i < P; i += blockDim.x) {
        uint64_t k = ~0ull;
        if (i < n) {
            uint32_t q[3];
            const double v[3] = {x[i], y[i], z[i]};
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                double t = (v[d] - bb[d]) * inv;
                t = fmin(fmax(t, 0.0), 2097151.0);
                q[d] = (uint32_t)t;
            }
            k = hilbert_key(q[0], q[1], q[2]);
        }
        key[i] = k;
        idx[i] = (uint32_t)i;
    }
    __syncthreads();
    if (P == (int)blockDim.x) {
        // one element per thread: stages whose partner is in the same warp (j < 32)
        // exchange through registers; the others through shared memory
        uint64_t mk = key[tid];
        uint32_t mi = idx[tid];
        for (int k = 2; k <= P; k <<= 1)
            for (int j = k >> 1; j > 0; j >>= 1) {
                uint64_t pk_;
                uint32_t pi_;
                if (j >= 32) {
                    __syncthreads();
                    key[tid] = mk;
                    idx[tid] = mi;
                    __syncthreads();
                    pk_ = key[tid ^ j];
                    pi_ = idx[tid ^ j];
                } else {
                    pk_ = __shfl_xor_sync(0xFFFFFFFFu, mk, j);
                    pi_ = __shfl_xor_sync(0xFFFFFFFFu, mi, j);
                }
                const bool mine_gt = mk > pk_ || (mk == pk_ && mi > pi_);
                const bool lower = (tid & j) == 0, asc = (tid & k) == 0;
                // the lower slot keeps the smaller pair in an ascending run, the larger in a descending one
                if ((lower == asc) == mine_gt) {
                    mk = pk_;
                    mi = pi_;
                }
            }
        if (tid < n) perm[tid] = mi;
        return;
    }
    for (int k = 2; k <= P; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = tid; i < P; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) {
                    const uint64_t ka = key[i], kb = key[l];
                    const uint32_t ia = idx[i], ib = idx[l];
                    const bool gt = ka > kb || (ka == kb && ia > ib);
                    if (((i & k) == 0) == gt) {
                        key[i] = kb; key[l] = ka;
                        idx[i] = ib; idx[l] = ia;
                    }
                }
            }
            __syncthreads();
        }
    for (int i = tid; i < n; i += blockDim.x) perm[i] = idx[i];
}

// ---------------------------------------------------------------------------
// packing of source tiles
// ---------------------------------------------------------------------------
// Tile t holds sorted slots [t*TJ, (t+1)*TJ) in tile_f4(TJ) = 2 + 4*TJ float4:
//   [0]            centre hi (x, y, z, r)   r = max |offset| over members (f32, rounded up)
//   [1]            centre lo (x, y, z, 0)
//   [2+2k, 3+2k]   member k offset hi: (x,x,y,y) (z,z,m,m)
//   [2+2TJ+2k, ..] member k offset lo: (x,x,y,y) (z,z,0,0)
//   [2+4TJ+c]      chunk c (members 32c .. 32c+31) box of the hi offsets:
//                  (centre x, y, z, half-extent), Chebyshev; half-extent -1e30
//                  when the chunk has no member (padding only)
// MIXED: the centre c is an f32 value, the midpoint of the members' f32-rounded
// bounding box (its lo word is 0; the pair kernel still reads hi + lo, so a
// centre that needs both words would work unchanged); each member stores
// off = x - c, taken in f64, as f32 hi + f32 lo (hi + lo = x - c to ~2^-48).
// The fast path reads only hi; tiles close to the targets also use lo.
// FP32: centre 0, members as rounded absolute positions, lo = 0.
// Components are stored twice so the pair kernel reads ready-made f32x2
// broadcast pairs.  Padding slots sit at the centre with zero mass.
__host__ __device__ constexpr int tile_f4(int tj) { return 2 + 4 * tj + tj / 32; }
__host__ __device__ constexpr int chunk_box(int tj) { return 2 + 4 * tj; }

// A (32 targets, 32 sources) block takes the float-float path when the
// Chebyshev distance of the two boxes' centres is below NEAR_KAPPA times the sum
// of their half-extents.  In f32 the separation of a far pair carries an error
// of about 2^-24 (|x_i - c_J| + |off_j|); below this distance that is no longer
// small against the separation itself.  1.5 keeps every tested Plummer system
// (N = 100 .. 2^20, softening down to 0.01) at or below 3e-7 relative RMS.
constexpr float NEAR_KAPPA = 1.5f;

// map (optional, batched ensembles): slot -> caller index, or PAD_FLAG | anchor
// for padding (the slot then takes the position of the tile's first slot).
constexpr uint32_t PAD_FLAG = 0x80000000u;

template <int TJ, bool MIXED>
__global__ void __launch_bounds__(TJ) k_pack32(const double *__restrict__ X, const double *__restrict__ Y,
                                               const double *__restrict__ Z, const double *__restrict__ M,
                                               const uint32_t *__restrict__ perm, size_t n,
                                               float4 *__restrict__ pack, const uint32_t *__restrict__ map) {
    constexpr int TF4 = tile_f4(TJ);
    __shared__ float red[TJ / 32][6];
    __shared__ float rred[TJ / 32];
    const int t = blockIdx.x, tid = threadIdx.x;
    const size_t s = (size_t)t * TJ + tid;
    bool valid;
    uint32_t o;
    if (map) {
        const uint32_t raw = map[s];
        valid = !(raw & PAD_FLAG);
        o = valid ? raw : (map[(size_t)t * TJ] & ~PAD_FLAG);
    } else {
        valid = s < n;
        o = perm[valid ? s : std::min((size_t)t * TJ, n - 1)];
    }
    if (!CHK_IDX(o, n)) {  // n: the resident state's length (both paths)
        o = 0;
        valid = false;
    }
    // tiles without any member (target-side padding) get a negative radius,
    // so they never trigger the near-field path of the real tile they are paired with
    const int nvalid = __syncthreads_count(valid);
    double p[3] = {X[o], Y[o], Z[o]};
    const double mass = valid ? M[o] : 0.0;
    double c[3] = {0.0, 0.0, 0.0};
    float chi[3] = {0.f, 0.f, 0.f}, clo[3] = {0.f, 0.f, 0.f};
    if (MIXED) {
        // The centre only has to lie near the middle of the tile: it is the f32
        // midpoint of the f32-rounded extent (f32 arithmetic; f64 throughput is a
        // small fraction of f32 on this part), and the offsets below are taken
        // from it exactly in f64.  Its lo part is therefore zero.
        float mn[3], mx[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) mn[d] = mx[d] = __double2float_rn(p[d]);
#pragma unroll
        for (int d = 0; d < 3; ++d)
            for (int off = 16; off > 0; off >>= 1) {
                mn[d] = fminf(mn[d], __shfl_xor_sync(0xFFFFFFFFu, mn[d], off));
                mx[d] = fmaxf(mx[d], __shfl_xor_sync(0xFFFFFFFFu, mx[d], off));
            }
        if ((tid & 31) == 0)
            for (int d = 0; d < 3; ++d) { red[tid >> 5][d] = mn[d]; red[tid >> 5][3 + d] = mx[d]; }
        __syncthreads();
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            float lo = red[0][d], hi = red[0][3 + d];
            for (int w = 1; w < TJ / 32; ++w) { lo = fminf(lo, red[w][d]); hi = fmaxf(hi, red[w][3 + d]); }
            chi[d] = 0.5f * lo + 0.5f * hi;  // no overflow for any finite extent
            c[d] = (double)chi[d];
        }
    }
    float oh[3], ol[3];
    float rad = 0.f;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double e = p[d] - c[d];
        oh[d] = valid ? __double2float_rn(e) : 0.f;
        ol[d] = (valid && MIXED) ? __double2float_rn(e - (double)oh[d]) : 0.f;
        rad = fmaxf(rad, fabsf(oh[d]));
    }
    for (int off = 16; off > 0; off >>= 1) rad = fmaxf(rad, __shfl_xor_sync(0xFFFFFFFFu, rad, off));
    if ((tid & 31) == 0) rred[tid >> 5] = rad;
    __syncthreads();
    float4 *tile = pack + (size_t)t * TF4;
    if (tid == 0) {
        float r = rred[0];
        for (int w = 1; w < TJ / 32; ++w) r = fmaxf(r, rred[w]);
        tile[0] = make_float4(chi[0], chi[1], chi[2], nvalid > 0 ? r * 1.0001f : -1e30f);
        tile[1] = make_float4(clo[0], clo[1], clo[2], 0.f);
    }
    {
        // box of this warp's chunk: members only (padding slots carry no mass)
        float bmn[3], bmx[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            bmn[d] = valid ? oh[d] : 3.0e38f;
            bmx[d] = valid ? oh[d] : -3.0e38f;
            for (int off = 16; off > 0; off >>= 1) {
                bmn[d] = fminf(bmn[d], __shfl_xor_sync(0xFFFFFFFFu, bmn[d], off));
                bmx[d] = fmaxf(bmx[d], __shfl_xor_sync(0xFFFFFFFFu, bmx[d], off));
            }
        }
        const bool any = __any_sync(0xFFFFFFFFu, valid);
        if ((tid & 31) == 0) {
            float4 box = make_float4(0.f, 0.f, 0.f, -1e30f);
            if (any) {
                float h = 0.f;
                float cb[3];
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    cb[d] = 0.5f * bmn[d] + 0.5f * bmx[d];
                    h = fmaxf(h, fmaxf(bmx[d] - cb[d], cb[d] - bmn[d]));
                }
                box = make_float4(cb[0], cb[1], cb[2], h * 1.0001f + 1e-30f);
            }
            tile[chunk_box(TJ) + (tid >> 5)] = box;
        }
    }
    const float mf = (float)mass;
    tile[2 + 2 * tid] = make_float4(oh[0], oh[0], oh[1], oh[1]);
    tile[3 + 2 * tid] = make_float4(oh[2], oh[2], mf, mf);
    tile[2 + 2 * TJ + 2 * tid] = make_float4(ol[0], ol[0], ol[1], ol[1]);
    tile[3 + 2 * TJ + 2 * tid] = make_float4(ol[2], ol[2], 0.f, 0.f);
}

__global__ void k_pack64(const double *__restrict__ X, const double *__restrict__ Y, const double *__restrict__ Z,
                         const double *__restrict__ M, const uint32_t *__restrict__ perm, size_t n, size_t npad,
                         double4 *__restrict__ pack) {
    size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= npad) return;
    bool valid = s < n;
    uint32_t o = perm[valid ? s : (s / TJ64) * TJ64 < n ? (s / TJ64) * TJ64 : 0];
    if (!CHK_IDX(o, n)) {
        o = 0;
        valid = false;
    }
    pack[s] = make_double4(X[o], Y[o], Z[o], valid ? M[o] : 0.0);
}

// Sources [j0, j0 + NJ) of a tile against NP target pairs.  nx.. hold
// -(x_i - c_J) per pair.  Pairs whose bit is set in MASK also add the f32 lo
// parts of both sides (float-float separations): sources close to the
// targets, where f32 offsets alone would lose relative accuracy.
template <int TJ, int NP, int MASK, bool GUARD, int UNR = 4, int NJ = TJ>
__device__ __forceinline__ void tile_pairs(const float4 *__restrict__ tile, const f2 *nx, const f2 *ny, const f2 *nz,
                                           const f2 *nxl, const f2 *nyl, const f2 *nzl, f2 e2, f2 *accx,
                                           f2 *accy, f2 *accz, int j0 = 0) {
    const float4 *jd = tile + 2 + 2 * j0;
    const float4 *jl = tile + 2 + 2 * TJ + 2 * j0;
#pragma unroll (UNR)
    for (int j = 0; j < NJ; ++j) {
        // two 16-byte broadcast loads per source; each float4 holds two ready f32x2 pairs
        const float4 a = jd[2 * j], b = jd[2 * j + 1];
        const f2 xj = pk(a.x, a.y), yj = pk(a.z, a.w), zj = pk(b.x, b.y), mj = pk(b.z, b.w);
        f2 xl = 0ull, yl = 0ull, zl = 0ull;
        if (MASK) {
            const float4 c = jl[2 * j], d = jl[2 * j + 1];
            xl = pk(c.x, c.y); yl = pk(c.z, c.w); zl = pk(d.x, d.y);
        }
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            f2 dx = add2(xj, nx[p]);
            f2 dy = add2(yj, ny[p]);
            f2 dz = add2(zj, nz[p]);
            if ((MASK >> p) & 1) {
                dx = add2(dx, add2(xl, nxl[p]));
                dy = add2(dy, add2(yl, nyl[p]));
                dz = add2(dz, add2(zl, nzl[p]));
            }
            f2 r2 = fma2(dx, dx, e2);
            r2 = fma2(dy, dy, r2);
            r2 = fma2(dz, dz, r2);
            float ra, rb;
            upk(r2, ra, rb);
            if (GUARD) { ra = fmaxf(ra, 1e-24f); rb = fmaxf(rb, 1e-24f); }
            const f2 ri = pk(rsqrt_approx(ra), rsqrt_approx(rb));
            f2 sm = mul2(mj, ri);
            const f2 ri2 = mul2(ri, ri);
            sm = mul2(sm, ri2);
            accx[p] = fma2(sm, dx, accx[p]);
            accy[p] = fma2(sm, dy, accy[p]);
            accz[p] = fma2(sm, dz, accz[p]);
        }
    }
}

// -(c_I + off_i - c_J) as an f32 hi + lo pair, from the f32 hi/lo parts of the
// two centres and of the offset (two-sum at each step, error ~2^-48 relative).
__device__ __forceinline__ void ff_rel(float cih, float cil, float cjh, float cjl, float oh, float ol, float &nh,
                                       float &nl) {
    const float th = __fsub_rn(cih, cjh);
    const float b1 = __fsub_rn(th, cih);
    const float te = __fadd_rn(__fsub_rn(cih, __fsub_rn(th, b1)), __fsub_rn(-cjh, b1));
    const float dl = __fadd_rn(te, __fsub_rn(cil, cjl));
    const float sh = __fadd_rn(th, oh);
    const float b2 = __fsub_rn(sh, th);
    const float se = __fadd_rn(__fsub_rn(th, __fsub_rn(sh, b2)), __fsub_rn(oh, b2));
    nh = -sh;
    nl = -__fadd_rn(__fadd_rn(se, dl), ol);
}

// ---------------------------------------------------------------------------
// tiled f32 kernel (FP32 and MIXED)
// ---------------------------------------------------------------------------
// Block size NT equals the tile size, so target k (k = 0..IPT-1) of every
// thread lies in tile blockIdx.x*IPT + k: the target-side centres are uniform
// over the block and live in shared memory.  Thread t owns targets
// i = blockIdx.x*NT*IPT + k*NT + t; NP = IPT/2 packed pairs (k = 2p, 2p+1).
// Per source tile J and pair p: d = (c_I - c_J) from the hi/lo pairs, then
// -(x_i - c_J) = -(d + off_i) as one f32x2 vector; per source particle j:
// 3 ADD2 + 3 FMA2 (r^2) + 2 MUFU.RSQ + 3 MUL2 + 3 FMA2 (accumulate).
// One work item of the tiled f32 kernel: the IPT target tiles starting at
// tile tgt0 against the source tiles [t0, t0 + nt); writes the item's partial
// sums to dst[c * npad + slot].  The mbarrier ring is shared by all items of
// a CTA: `phase` counts the tiles the CTA has consumed so far, so stage and
// parity continue across items.  Returns false if a bounded wait gave up.
template <int NT, int NP, int NSTAGE, bool MIXED, bool GUARD, int UNR = 4>
__device__ __forceinline__ bool direct_item(const float4 *__restrict__ pack, int tgt0, int t0, int nt, float eps2,
                                            double *__restrict__ dst, size_t npad, unsigned *__restrict__ err,
                                            float4 *smem, uint64_t *bar, float4 (*ci)[2], float4 (*wbox)[2 * NP],
                                            unsigned &phase, unsigned &near_tiles) {
    constexpr int TJ = NT;
    constexpr int IPT = 2 * NP;
    constexpr int TF4 = tile_f4(TJ);
    constexpr int NCH = TJ / 32;  // source chunks per tile
    static_assert(NCH * NP <= 32, "one lane per (source chunk, target pair)");
    constexpr unsigned TILE_BYTES = TF4 * 16;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const size_t ibase = (size_t)tgt0 * TJ;
    if (tid < IPT) {
        const float4 *tp = pack + ((size_t)tgt0 + tid) * TF4;
        ci[tid][0] = __ldg(tp);
        ci[tid][1] = __ldg(tp + 1);
    }
    // warp w's targets in target tile k are that tile's chunk w: its box is stored there
    if (tid < (NT / 32) * IPT)
        wbox[tid / IPT][tid % IPT] = __ldg(pack + ((size_t)tgt0 + tid % IPT) * TF4 + chunk_box(TJ) + tid / IPT);
    __syncthreads();
    if (tid == 0) {
        for (int s = 0; s < NSTAGE && s < nt; ++s) {
            const unsigned st = (phase + s) % NSTAGE;
            mbar_arrive_expect_tx(&bar[st], TILE_BYTES);
            bulk_g2s(smem + st * TF4, pack + (size_t)(t0 + s) * TF4, TILE_BYTES, &bar[st]);
        }
    }

    // target offsets from their own tile centre (hi and lo), packed by pair
    f2 ox[NP], oy[NP], oz[NP], oxl[NP], oyl[NP], ozl[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        float v[2][6];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const float4 *tp = pack + ((size_t)tgt0 + 2 * p + q) * TF4;
            const float4 a = __ldg(tp + 2 + 2 * tid), b = __ldg(tp + 3 + 2 * tid);
            v[q][0] = a.x; v[q][1] = a.z; v[q][2] = b.x;
            if (MIXED) {
                const float4 al = __ldg(tp + 2 + 2 * TJ + 2 * tid), bl = __ldg(tp + 3 + 2 * TJ + 2 * tid);
                v[q][3] = al.x; v[q][4] = al.z; v[q][5] = bl.x;
            } else {
                v[q][3] = v[q][4] = v[q][5] = 0.f;
            }
        }
        ox[p] = pk(v[0][0], v[1][0]);
        oy[p] = pk(v[0][1], v[1][1]);
        oz[p] = pk(v[0][2], v[1][2]);
        oxl[p] = pk(v[0][3], v[1][3]);
        oyl[p] = pk(v[0][4], v[1][4]);
        ozl[p] = pk(v[0][5], v[1][5]);
    }

    f2 accx[NP], accy[NP], accz[NP], hx[NP], hy[NP], hz[NP], lx[NP], ly[NP], lz[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) accx[p] = accy[p] = accz[p] = hx[p] = hy[p] = hz[p] = lx[p] = ly[p] = lz[p] = 0ull;
    const f2 e2 = pk(eps2, eps2);

    int it = 0;
    bool bail = false;
    for (; it < nt; ++it) {
        const int s = (int)((phase + it) % NSTAGE);
        const unsigned parity = ((phase + it) / NSTAGE) & 1u;
        // A thread whose wait gave up still runs the tile (on stale data, discarded):
        // the one barrier at the end of the tile both frees stage s and spreads the bail.
        const bool ok = mbar_wait_bounded(&bar[s], parity, err);
        const float4 *tile = smem + s * TF4;
        f2 nx[NP], ny[NP], nz[NP], nxl[NP], nyl[NP], nzl[NP];
        unsigned mask = 0;  // bit p * NCH + c: target pair p against source chunk c is near
        if (MIXED) {
            const float4 jh = tile[0], jo = tile[1];
            // near-field test, one lane per (source chunk c, target pair p), on the
            // boxes of this warp's 32 targets and of the chunk's 32 sources
            bool near = false;
            if (lane < NCH * NP) {
                const int c = lane % NCH, p = lane / NCH;
                const float4 sb = tile[chunk_box(TJ) + c];
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const float4 h = ci[2 * p + q][0], l = ci[2 * p + q][1], tb = wbox[warp][2 * p + q];
                    const float ddx = ((h.x - jh.x) + (l.x - jo.x)) + (tb.x - sb.x);
                    const float ddy = ((h.y - jh.y) + (l.y - jo.y)) + (tb.y - sb.y);
                    const float ddz = ((h.z - jh.z) + (l.z - jo.z)) + (tb.z - sb.z);
                    const float dist = fmaxf(fabsf(ddx), fmaxf(fabsf(ddy), fabsf(ddz)));
                    near = near || (dist < NEAR_KAPPA * (tb.w + sb.w));
                }
            }
            mask = __ballot_sync(0xFFFFFFFFu, near);
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                if ((mask >> (p * NCH)) & ((1u << NCH) - 1u)) {
                    float o[2][6], hh[2][3], ll[2][3];
                    upk(ox[p], o[0][0], o[1][0]); upk(oy[p], o[0][1], o[1][1]); upk(oz[p], o[0][2], o[1][2]);
                    upk(oxl[p], o[0][3], o[1][3]); upk(oyl[p], o[0][4], o[1][4]); upk(ozl[p], o[0][5], o[1][5]);
#pragma unroll
                    for (int q = 0; q < 2; ++q) {
                        const float4 h = ci[2 * p + q][0], l = ci[2 * p + q][1];
                        ff_rel(h.x, l.x, jh.x, jo.x, o[q][0], o[q][3], hh[q][0], ll[q][0]);
                        ff_rel(h.y, l.y, jh.y, jo.y, o[q][1], o[q][4], hh[q][1], ll[q][1]);
                        ff_rel(h.z, l.z, jh.z, jo.z, o[q][2], o[q][5], hh[q][2], ll[q][2]);
                    }
                    nx[p] = pk(hh[0][0], hh[1][0]); nxl[p] = pk(ll[0][0], ll[1][0]);
                    ny[p] = pk(hh[0][1], hh[1][1]); nyl[p] = pk(ll[0][1], ll[1][1]);
                    nz[p] = pk(hh[0][2], hh[1][2]); nzl[p] = pk(ll[0][2], ll[1][2]);
                } else {
                    const float4 h0 = ci[2 * p][0], l0 = ci[2 * p][1], h1 = ci[2 * p + 1][0], l1 = ci[2 * p + 1][1];
                    // -(c_I - c_J) per lane, then minus the target offset
                    const f2 dx = pk(-((h0.x - jh.x) + (l0.x - jo.x)), -((h1.x - jh.x) + (l1.x - jo.x)));
                    const f2 dy = pk(-((h0.y - jh.y) + (l0.y - jo.y)), -((h1.y - jh.y) + (l1.y - jo.y)));
                    const f2 dz = pk(-((h0.z - jh.z) + (l0.z - jo.z)), -((h1.z - jh.z) + (l1.z - jo.z)));
                    nx[p] = sub2(dx, ox[p]);
                    ny[p] = sub2(dy, oy[p]);
                    nz[p] = sub2(dz, oz[p]);
                    nxl[p] = nyl[p] = nzl[p] = 0ull;
                }
            }
        } else {
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                nx[p] = sub2(0ull, ox[p]);
                ny[p] = sub2(0ull, oy[p]);
                nz[p] = sub2(0ull, oz[p]);
                nxl[p] = nyl[p] = nzl[p] = 0ull;
            }
        }
        if (lane == 0) near_tiles += (unsigned)__popc(mask);
        if (!MIXED || mask == 0) {
            tile_pairs<TJ, NP, 0, GUARD, UNR>(tile, nx, ny, nz, nxl, nyl, nzl, e2, accx, accy, accz);
        } else {
            // chunk by chunk: far pairs on the plain path, near ones with the lo parts
            // (a pair flagged in some chunk has its lo parts; they are zero otherwise)
#pragma unroll 1
            for (int c = 0; c < NCH; ++c) {
                unsigned cm = 0;
#pragma unroll
                for (int p = 0; p < NP; ++p) cm |= ((mask >> (p * NCH + c)) & 1u) << p;
                if (cm == 0)
                    tile_pairs<TJ, NP, 0, GUARD, UNR, 32>(tile, nx, ny, nz, nxl, nyl, nzl, e2, accx, accy, accz, 32 * c);
                else if (NP == 2 && cm == 1)
                    tile_pairs<TJ, NP, 1, GUARD, UNR, 32>(tile, nx, ny, nz, nxl, nyl, nzl, e2, accx, accy, accz, 32 * c);
                else if (NP == 2 && cm == 2)
                    tile_pairs<TJ, NP, 2, GUARD, UNR, 32>(tile, nx, ny, nz, nxl, nyl, nzl, e2, accx, accy, accz, 32 * c);
                else
                    tile_pairs<TJ, NP, (1 << NP) - 1, GUARD, UNR, 32>(tile, nx, ny, nz, nxl, nyl, nzl, e2, accx,
                                                                      accy, accz, 32 * c);
            }
        }
        if (MIXED) {
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                two_sum2(hx[p], lx[p], accx[p]);
                two_sum2(hy[p], ly[p], accy[p]);
                two_sum2(hz[p], lz[p], accz[p]);
                accx[p] = accy[p] = accz[p] = 0ull;
            }
        }
        if (__syncthreads_or(!ok)) { bail = true; break; }  // every thread is done with stage s
        if (tid == 0 && it + NSTAGE < nt) {
            mbar_arrive_expect_tx(&bar[s], TILE_BYTES);
            bulk_g2s(smem + s * TF4, pack + (size_t)(t0 + it + NSTAGE) * TF4, TILE_BYTES, &bar[s]);
        }
    }
    if (bail) {
        // drain copies still in flight before the CTA exits (bounded)
        if (tid == 0)
            for (int j = it; j < nt && j < it + NSTAGE; ++j)
                mbar_wait_bounded(&bar[(phase + j) % NSTAGE], ((phase + j) / NSTAGE) & 1u, err);
        return false;
    }
    phase += (unsigned)nt;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        float v[3][2][2];  // component, lane, (hi, lo)
        if (MIXED) {
            upk(hx[p], v[0][0][0], v[0][1][0]); upk(lx[p], v[0][0][1], v[0][1][1]);
            upk(hy[p], v[1][0][0], v[1][1][0]); upk(ly[p], v[1][0][1], v[1][1][1]);
            upk(hz[p], v[2][0][0], v[2][1][0]); upk(lz[p], v[2][0][1], v[2][1][1]);
        } else {
            upk(accx[p], v[0][0][0], v[0][1][0]);
            upk(accy[p], v[1][0][0], v[1][1][0]);
            upk(accz[p], v[2][0][0], v[2][1][0]);
            for (int c = 0; c < 3; ++c) v[c][0][1] = v[c][1][1] = 0.f;
        }
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const size_t i = ibase + (size_t)(2 * p + q) * NT + tid;
#pragma unroll
            for (int c = 0; c < 3; ++c) dst[(size_t)c * npad + i] = (double)v[c][q][0] + (double)v[c][q][1];
        }
    }
    return true;
}

template <int NT, int NP, int NSTAGE, bool MIXED, bool GUARD, int MINB, int UNR>
__global__ void __launch_bounds__(NT, MINB) k_direct32(const float4 *__restrict__ pack, int ntiles, int tiles_per_split,
                                                 float eps2, double *__restrict__ partial, size_t npad,
                                                 unsigned *__restrict__ err,
                                                 unsigned long long *__restrict__ near_count) {
    constexpr int IPT = 2 * NP;
    extern __shared__ __align__(128) float4 smem[];
    __shared__ __align__(8) uint64_t bar[NSTAGE];
    __shared__ float4 ci[IPT][2];          // target-tile centres (hi, lo)
    __shared__ float4 wbox[NT / 32][IPT];  // per warp: box of its targets in each target tile
    if (threadIdx.x == 0) {
        for (int s = 0; s < NSTAGE; ++s) mbar_init(&bar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    const int t0 = blockIdx.y * tiles_per_split;
    const int nt = max(0, min(ntiles, t0 + tiles_per_split) - t0);
    unsigned phase = 0, near_tiles = 0;
    const bool ok = direct_item<NT, NP, NSTAGE, MIXED, GUARD, UNR>(pack, (int)blockIdx.x * IPT, t0, nt, eps2,
                                                             partial + (size_t)blockIdx.y * 3 * npad, npad, err,
                                                             smem, bar, ci, wbox, phase, near_tiles);
    if (ok && (threadIdx.x & 31) == 0 && near_count) atomicAdd(near_count, (unsigned long long)near_tiles);
}

// Persistent form for batched ensembles: each CTA takes work items
// (target tile, first source tile, source tile count, partial slot) from a
// queue counter until it is empty.  Items never wait on each other.
template <int NT, int NP, int NSTAGE, bool MIXED, bool GUARD, int MINB, int UNR>
__global__ void __launch_bounds__(NT, MINB) k_direct32_items(const float4 *__restrict__ pack,
                                                       const int4 *__restrict__ items, int nitems,
                                                       unsigned *__restrict__ counter, float eps2,
                                                       double *__restrict__ partial, size_t npad,
                                                       unsigned *__restrict__ err,
                                                       unsigned long long *__restrict__ near_count, int ntiles,
                                                       int nsplit) {
    constexpr int IPT = 2 * NP;
    extern __shared__ __align__(128) float4 smem[];
    __shared__ __align__(8) uint64_t bar[NSTAGE];
    __shared__ float4 ci[IPT][2];
    __shared__ float4 wbox[NT / 32][IPT];
    __shared__ int item_s;
    if (threadIdx.x == 0) {
        for (int s = 0; s < NSTAGE; ++s) mbar_init(&bar[s], 1);
        fence_mbar_init();
    }
    unsigned phase = 0, near_tiles = 0;
    for (;;) {
        if (threadIdx.x == 0) item_s = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int k = item_s;
        __syncthreads();
        if (k >= nitems) break;
        const int4 w = items[k];
        if (!CHK(w.x >= 0 && w.x < ntiles && w.y >= 0 && w.z > 0 && w.y + w.z <= ntiles && w.w >= 0 &&
                     w.w < nsplit, DERR_BOUNDS))
            continue;  // block-uniform: every thread read the same item
        if (!direct_item<NT, NP, NSTAGE, MIXED, GUARD, UNR>(pack, w.x, w.y, w.z, eps2, partial + (size_t)w.w * 3 * npad,
                                                       npad, err, smem, bar, ci, wbox, phase, near_tiles))
            return;
    }
    if ((threadIdx.x & 31) == 0 && near_count) atomicAdd(near_count, (unsigned long long)near_tiles);
}

// ---------------------------------------------------------------------------
// tiled f64 kernel (FP64): same tiling, double4 tiles, f64 rsqrt
// ---------------------------------------------------------------------------
template <int NT, int IPT, int NSTAGE, bool GUARD>
__global__ void __launch_bounds__(NT) k_direct64(const double4 *__restrict__ pack, int ntiles, int tiles_per_split,
                                                 double eps2, double *__restrict__ partial, size_t npad,
                                                 unsigned *__restrict__ err) {
    constexpr unsigned TILE_BYTES = TJ64 * 32;
    extern __shared__ __align__(128) double4 smem64[];
    __shared__ __align__(8) uint64_t bar[NSTAGE];
    const int tid = threadIdx.x;
    const size_t ibase = (size_t)blockIdx.x * NT * IPT;
    const int t0 = blockIdx.y * tiles_per_split;
    const int t1 = min(ntiles, t0 + tiles_per_split);
    const int nt = max(0, t1 - t0);
    double xi[IPT], yi[IPT], zi[IPT], ax[IPT], ay[IPT], az[IPT];
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        double4 v = pack[ibase + (size_t)k * NT + tid];
        xi[k] = v.x; yi[k] = v.y; zi[k] = v.z;
        ax[k] = ay[k] = az[k] = 0.0;
    }
    if (tid == 0) {
        for (int s = 0; s < NSTAGE; ++s) mbar_init(&bar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0)
        for (int s = 0; s < NSTAGE && s < nt; ++s) {
            mbar_arrive_expect_tx(&bar[s], TILE_BYTES);
            bulk_g2s(smem64 + s * TJ64, pack + (size_t)(t0 + s) * TJ64, TILE_BYTES, &bar[s]);
        }
    int it = 0;
    bool bail = false;
    for (; it < nt; ++it) {
        const int s = it % NSTAGE;
        bool ok = mbar_wait_bounded(&bar[s], (unsigned)(it / NSTAGE) & 1u, err);
        if (__syncthreads_or(!ok)) { bail = true; break; }
        const double4 *tile = smem64 + s * TJ64;
#pragma unroll 2
        for (int j = 0; j < TJ64; ++j) {
            const double4 q = tile[j];
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                double dx = q.x - xi[k], dy = q.y - yi[k], dz = q.z - zi[k];
                double r2 = fma(dz, dz, fma(dy, dy, fma(dx, dx, eps2)));
                if (GUARD) r2 = fmax(r2, 1e-200);
                double ri = rsqrt(r2);
                double sm = q.w * ri * ri * ri;
                ax[k] = fma(sm, dx, ax[k]);
                ay[k] = fma(sm, dy, ay[k]);
                az[k] = fma(sm, dz, az[k]);
            }
        }
        __syncthreads();
        if (tid == 0 && it + NSTAGE < nt) {
            mbar_arrive_expect_tx(&bar[s], TILE_BYTES);
            bulk_g2s(smem64 + s * TJ64, pack + (size_t)(t0 + it + NSTAGE) * TJ64, TILE_BYTES, &bar[s]);
        }
    }
    if (bail) {
        if (tid == 0)
            for (int j = it; j < nt && j < it + NSTAGE; ++j)
                mbar_wait_bounded(&bar[j % NSTAGE], (unsigned)(j / NSTAGE) & 1u, err);
        return;
    }
    double *dst = partial + (size_t)blockIdx.y * 3 * npad;
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        size_t i = ibase + (size_t)k * NT + tid;
        dst[i] = ax[k];
        dst[npad + i] = ay[k];
        dst[2 * npad + i] = az[k];
    }
}

// Adds the nsplit partials in fixed order and scatters to caller order.
__global__ void k_reduce(const double *__restrict__ partial, int nsplit, size_t npad, size_t n,
                         const uint32_t *__restrict__ perm, double *__restrict__ AX, double *__restrict__ AY,
                         double *__restrict__ AZ, int accumulate) {
    size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    double r[3] = {0.0, 0.0, 0.0};
    for (int js = 0; js < nsplit; ++js)
#pragma unroll
        for (int c = 0; c < 3; ++c) r[c] += partial[((size_t)js * 3 + c) * npad + s];
    uint32_t o = perm[s];
    if (!CHK_IDX(o, n)) return;
    if (accumulate) {
        AX[o] += r[0]; AY[o] += r[1]; AZ[o] += r[2];
    } else {
        AX[o] = r[0]; AY[o] = r[1]; AZ[o] = r[2];
    }
}

// ---------------------------------------------------------------------------
// fused force + vector-Jacobian product (the adjoint's all-pairs kernel)
// ---------------------------------------------------------------------------
// For the softened force a_i = sum_j m_j d_ij s^-3/2 (d_ij = x_j - x_i,
// s = |d|^2 + eps^2) and an adjoint vector w (one 3-vector per particle):
//   g_k  = sum_i (da_i/dx_k)^T w_i = sum_j T(d_kj) (m_k w_j - m_j w_k),
//          T(d) = s^-3/2 I - 3 s^-5/2 d d^T          (symmetric, even in d)
//   gm_k = sum_i w_i . da_i/dm_k = - sum_j (w_j . d_kj) s^-3/2
// Per source j and target k (packed by pairs of targets) the kernel forms
// r3 = s^-3/2, r5 = s^-5/2 once and accumulates
//   a  += m_j r3 d,  S += m_j r3,  A += r3 w_j,  B += r5 (w_j.d) d,
//   C  += m_j r5 (w_k.d) d,  gm -= r3 (w_j.d)
// then g = m_k (A - 3 B) - w_k S + 3 C per tile (linear in the sums), folded
// into two-sum accumulators with a.  The forces come out of the same pass
// because the reverse-time sweep needs a(x) at exactly the points where it
// applies the VJP.  Tiles, near-field path and bulk-copy ring as k_direct32;
// the adjoint vectors stream in a second tile of (wx,wx,wy,wy)(wz,wz,0,0).
__host__ __device__ constexpr int wtile_f4(int tj) { return 2 * tj; }

// OWN: the source tile is one of the block's own target tiles; there the
// explicit u = m_k w_j - m_j w_k form is used, which is exactly zero for the
// self pair (the split A/S form would leave the rounding of two large
// self terms, m_k eps^-3 w_k, that should cancel).
template <int TJ, int NP, int MASK, bool GUARD, bool OWN, int NJ = TJ>
__device__ __forceinline__ void tile_vjp(const float4 *__restrict__ tile, const float4 *__restrict__ wt,
                                         const f2 *nx, const f2 *ny, const f2 *nz, const f2 *nxl, const f2 *nyl,
                                         const f2 *nzl, const f2 *wkx, const f2 *wky, const f2 *wkz, const f2 *mk,
                                         f2 e2, f2 *ax, f2 *ay, f2 *az, f2 *S, f2 *Ax, f2 *Ay, f2 *Az, f2 *Bx,
                                         f2 *By, f2 *Bz, f2 *Cx, f2 *Cy, f2 *Cz, f2 *Gx, f2 *Gy, f2 *Gz, f2 *gm,
                                         int j0 = 0) {
    const f2 mthree = pk(-3.f, -3.f);
    const float4 *jd = tile + 2 + 2 * j0;
    const float4 *jl = tile + 2 + 2 * TJ + 2 * j0;
    const float4 *jw = wt + 2 * j0;
#pragma unroll 2
    for (int j = 0; j < NJ; ++j) {
        const float4 a = jd[2 * j], b = jd[2 * j + 1], wa = jw[2 * j], wb = jw[2 * j + 1];
        const f2 xj = pk(a.x, a.y), yj = pk(a.z, a.w), zj = pk(b.x, b.y), mj = pk(b.z, b.w);
        const f2 wx = pk(wa.x, wa.y), wy = pk(wa.z, wa.w), wz = pk(wb.x, wb.y);
        f2 xl = 0ull, yl = 0ull, zl = 0ull;
        if (MASK) {
            const float4 c = jl[2 * j], d = jl[2 * j + 1];
            xl = pk(c.x, c.y); yl = pk(c.z, c.w); zl = pk(d.x, d.y);
        }
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            f2 dx = add2(xj, nx[p]), dy = add2(yj, ny[p]), dz = add2(zj, nz[p]);
            if ((MASK >> p) & 1) {
                dx = add2(dx, add2(xl, nxl[p]));
                dy = add2(dy, add2(yl, nyl[p]));
                dz = add2(dz, add2(zl, nzl[p]));
            }
            f2 r2 = fma2(dx, dx, e2);
            r2 = fma2(dy, dy, r2);
            r2 = fma2(dz, dz, r2);
            float ra, rb;
            upk(r2, ra, rb);
            if (GUARD) { ra = fmaxf(ra, 1e-24f); rb = fmaxf(rb, 1e-24f); }
            const f2 ri = pk(rsqrt_approx(ra), rsqrt_approx(rb));
            const f2 ri2 = mul2(ri, ri);
            const f2 r3 = mul2(ri, ri2);
            const f2 r5 = mul2(r3, ri2);
            const f2 mr3 = mul2(mj, r3);
            ax[p] = fma2(mr3, dx, ax[p]);
            ay[p] = fma2(mr3, dy, ay[p]);
            az[p] = fma2(mr3, dz, az[p]);
            const f2 dw = fma2(wz, dz, fma2(wy, dy, mul2(wx, dx)));
            gm[p] = fma2(r3, dw, gm[p]);
            if (OWN) {
                const f2 ux = sub2(mul2(mk[p], wx), mul2(mj, wkx[p]));
                const f2 uy = sub2(mul2(mk[p], wy), mul2(mj, wky[p]));
                const f2 uz = sub2(mul2(mk[p], wz), mul2(mj, wkz[p]));
                const f2 du = fma2(uz, dz, fma2(uy, dy, mul2(ux, dx)));
                const f2 c = mul2(mthree, mul2(r5, du));
                Gx[p] = fma2(c, dx, fma2(r3, ux, Gx[p]));
                Gy[p] = fma2(c, dy, fma2(r3, uy, Gy[p]));
                Gz[p] = fma2(c, dz, fma2(r3, uz, Gz[p]));
            } else {
                S[p] = add2(S[p], mr3);
                Ax[p] = fma2(r3, wx, Ax[p]);
                Ay[p] = fma2(r3, wy, Ay[p]);
                Az[p] = fma2(r3, wz, Az[p]);
                const f2 b = mul2(r5, dw);
                Bx[p] = fma2(b, dx, Bx[p]);
                By[p] = fma2(b, dy, By[p]);
                Bz[p] = fma2(b, dz, Bz[p]);
                const f2 dwk = fma2(wkz[p], dz, fma2(wky[p], dy, mul2(wkx[p], dx)));
                const f2 cc = mul2(mul2(mj, r5), dwk);
                Cx[p] = fma2(cc, dx, Cx[p]);
                Cy[p] = fma2(cc, dy, Cy[p]);
                Cz[p] = fma2(cc, dz, Cz[p]);
            }
        }
    }
}

// Partials per split: [split][7][npad] = a (3), g (3), gm (1), in sorted order.
template <int NT, int NP, int NSTAGE, bool GUARD>
__global__ void __launch_bounds__(NT) k_force_vjp32(const float4 *__restrict__ pack, const float4 *__restrict__ wpack,
                                                    int ntiles, int tiles_per_split, float eps2,
                                                    double *__restrict__ partial, size_t npad,
                                                    unsigned *__restrict__ err) {
    constexpr int TJ = NT;
    constexpr int IPT = 2 * NP;
    constexpr int TF4 = tile_f4(TJ);
    constexpr int WF4 = wtile_f4(TJ);
    constexpr unsigned TILE_BYTES = TF4 * 16, WTILE_BYTES = WF4 * 16;
    extern __shared__ __align__(128) float4 smem_v[];
    float4 *spos = smem_v;                  // NSTAGE position tiles
    float4 *sw = smem_v + NSTAGE * TF4;     // NSTAGE adjoint-vector tiles
    __shared__ __align__(8) uint64_t bar[NSTAGE];
    __shared__ float4 ci[IPT][2];
    __shared__ float4 wbox[NT / 32][IPT];  // per warp: box of its targets in each target tile
    constexpr int NCH = TJ / 32;
    static_assert(NCH * NP <= 32, "one lane per (source chunk, target pair)");

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const size_t ibase = (size_t)blockIdx.x * NT * IPT;
    const int t0 = blockIdx.y * tiles_per_split;
    const int nt = max(0, min(ntiles, t0 + tiles_per_split) - t0);
    if (tid == 0) {
        for (int s = 0; s < NSTAGE; ++s) mbar_init(&bar[s], 1);
        fence_mbar_init();
    }
    if (tid < IPT) {
        const float4 *tp = pack + ((size_t)blockIdx.x * IPT + tid) * TF4;
        ci[tid][0] = __ldg(tp);
        ci[tid][1] = __ldg(tp + 1);
    }
    if (tid < (NT / 32) * IPT)
        wbox[tid / IPT][tid % IPT] =
            __ldg(pack + ((size_t)blockIdx.x * IPT + tid % IPT) * TF4 + chunk_box(TJ) + tid / IPT);
    __syncthreads();
    if (tid == 0)
        for (int s = 0; s < NSTAGE && s < nt; ++s) {
            mbar_arrive_expect_tx(&bar[s], TILE_BYTES + WTILE_BYTES);
            bulk_g2s(spos + s * TF4, pack + (size_t)(t0 + s) * TF4, TILE_BYTES, &bar[s]);
            bulk_g2s(sw + s * WF4, wpack + (size_t)(t0 + s) * WF4, WTILE_BYTES, &bar[s]);
        }
    // target data: offsets (hi, lo), own adjoint vector, mass
    f2 ox[NP], oy[NP], oz[NP], oxl[NP], oyl[NP], ozl[NP], wkx[NP], wky[NP], wkz[NP], mk[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        float v[2][10];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const size_t tile = (size_t)blockIdx.x * IPT + 2 * p + q;
            const float4 *tp = pack + tile * TF4;
            const float4 a = __ldg(tp + 2 + 2 * tid), b = __ldg(tp + 3 + 2 * tid);
            const float4 al = __ldg(tp + 2 + 2 * TJ + 2 * tid), bl = __ldg(tp + 3 + 2 * TJ + 2 * tid);
            const float4 wa = __ldg(wpack + tile * WF4 + 2 * tid), wb = __ldg(wpack + tile * WF4 + 2 * tid + 1);
            v[q][0] = a.x; v[q][1] = a.z; v[q][2] = b.x; v[q][3] = al.x; v[q][4] = al.z; v[q][5] = bl.x;
            v[q][6] = wa.x; v[q][7] = wa.z; v[q][8] = wb.x; v[q][9] = b.z;
        }
        ox[p] = pk(v[0][0], v[1][0]); oy[p] = pk(v[0][1], v[1][1]); oz[p] = pk(v[0][2], v[1][2]);
        oxl[p] = pk(v[0][3], v[1][3]); oyl[p] = pk(v[0][4], v[1][4]); ozl[p] = pk(v[0][5], v[1][5]);
        wkx[p] = pk(v[0][6], v[1][6]); wky[p] = pk(v[0][7], v[1][7]); wkz[p] = pk(v[0][8], v[1][8]);
        mk[p] = pk(v[0][9], v[1][9]);
    }
    f2 ax[NP], ay[NP], az[NP], S[NP], Ax[NP], Ay[NP], Az[NP], Bx[NP], By[NP], Bz[NP], Cx[NP], Cy[NP], Cz[NP], gm[NP];
    f2 Gx[NP], Gy[NP], Gz[NP];
    f2 hi[NP][7], lo[NP][7];
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        ax[p] = ay[p] = az[p] = S[p] = Ax[p] = Ay[p] = Az[p] = Bx[p] = By[p] = Bz[p] = Cx[p] = Cy[p] = Cz[p] = gm[p] =
            0ull;
        Gx[p] = Gy[p] = Gz[p] = 0ull;
#pragma unroll
        for (int k = 0; k < 7; ++k) hi[p][k] = lo[p][k] = 0ull;
    }
    const f2 e2 = pk(eps2, eps2);
    const f2 three = pk(3.f, 3.f);
    int it = 0;
    bool bail = false;
    for (; it < nt; ++it) {
        const int s = it % NSTAGE;
        const bool ok = mbar_wait_bounded(&bar[s], (unsigned)(it / NSTAGE) & 1u, err);
        if (__syncthreads_or(!ok)) { bail = true; break; }
        const float4 *tile = spos + s * TF4;
        const float4 jh = tile[0], jo = tile[1];
        f2 nx[NP], ny[NP], nz[NP], nxl[NP], nyl[NP], nzl[NP];
        // near-field test as in direct_item: one lane per (source chunk, target pair)
        bool near = false;
        if (lane < NCH * NP) {
            const int c = lane % NCH, p = lane / NCH;
            const float4 sb = tile[chunk_box(TJ) + c];
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const float4 h = ci[2 * p + q][0], l = ci[2 * p + q][1], tb = wbox[warp][2 * p + q];
                const float ddx = ((h.x - jh.x) + (l.x - jo.x)) + (tb.x - sb.x);
                const float ddy = ((h.y - jh.y) + (l.y - jo.y)) + (tb.y - sb.y);
                const float ddz = ((h.z - jh.z) + (l.z - jo.z)) + (tb.z - sb.z);
                const float dist = fmaxf(fabsf(ddx), fmaxf(fabsf(ddy), fabsf(ddz)));
                near = near || (dist < NEAR_KAPPA * (tb.w + sb.w));
            }
        }
        const unsigned cmask = __ballot_sync(0xFFFFFFFFu, near);
        int mask = 0;  // pair p has some near chunk
#pragma unroll
        for (int p = 0; p < NP; ++p)
            if ((cmask >> (p * NCH)) & ((1u << NCH) - 1u)) mask |= 1 << p;
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            if ((mask >> p) & 1) {
                float o[2][6], hh[2][3], ll[2][3];
                upk(ox[p], o[0][0], o[1][0]); upk(oy[p], o[0][1], o[1][1]); upk(oz[p], o[0][2], o[1][2]);
                upk(oxl[p], o[0][3], o[1][3]); upk(oyl[p], o[0][4], o[1][4]); upk(ozl[p], o[0][5], o[1][5]);
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const float4 h = ci[2 * p + q][0], l = ci[2 * p + q][1];
                    ff_rel(h.x, l.x, jh.x, jo.x, o[q][0], o[q][3], hh[q][0], ll[q][0]);
                    ff_rel(h.y, l.y, jh.y, jo.y, o[q][1], o[q][4], hh[q][1], ll[q][1]);
                    ff_rel(h.z, l.z, jh.z, jo.z, o[q][2], o[q][5], hh[q][2], ll[q][2]);
                }
                nx[p] = pk(hh[0][0], hh[1][0]); nxl[p] = pk(ll[0][0], ll[1][0]);
                ny[p] = pk(hh[0][1], hh[1][1]); nyl[p] = pk(ll[0][1], ll[1][1]);
                nz[p] = pk(hh[0][2], hh[1][2]); nzl[p] = pk(ll[0][2], ll[1][2]);
            } else {
                const float4 h0 = ci[2 * p][0], l0 = ci[2 * p][1], h1 = ci[2 * p + 1][0], l1 = ci[2 * p + 1][1];
                nx[p] = sub2(pk(-((h0.x - jh.x) + (l0.x - jo.x)), -((h1.x - jh.x) + (l1.x - jo.x))), ox[p]);
                ny[p] = sub2(pk(-((h0.y - jh.y) + (l0.y - jo.y)), -((h1.y - jh.y) + (l1.y - jo.y))), oy[p]);
                nz[p] = sub2(pk(-((h0.z - jh.z) + (l0.z - jo.z)), -((h1.z - jh.z) + (l1.z - jo.z))), oz[p]);
                nxl[p] = nyl[p] = nzl[p] = 0ull;
            }
        }
        const float4 *wt = sw + s * WF4;
        constexpr int ALL = NP == 1 ? 1 : 3;
        const int J = t0 + it;
        const bool own = J >= (int)blockIdx.x * IPT && J < ((int)blockIdx.x + 1) * IPT;
        if (own) {
            if (mask != ALL) {  // every lane is near its own tile: switch all pairs to float-float
#pragma unroll
                for (int p = 0; p < NP; ++p)
                    if (!((mask >> p) & 1)) {
                        float o[2][6], hh[2][3], ll[2][3];
                        upk(ox[p], o[0][0], o[1][0]); upk(oy[p], o[0][1], o[1][1]); upk(oz[p], o[0][2], o[1][2]);
                        upk(oxl[p], o[0][3], o[1][3]); upk(oyl[p], o[0][4], o[1][4]); upk(ozl[p], o[0][5], o[1][5]);
#pragma unroll
                        for (int q = 0; q < 2; ++q) {
                            const float4 h = ci[2 * p + q][0], l = ci[2 * p + q][1];
                            ff_rel(h.x, l.x, jh.x, jo.x, o[q][0], o[q][3], hh[q][0], ll[q][0]);
                            ff_rel(h.y, l.y, jh.y, jo.y, o[q][1], o[q][4], hh[q][1], ll[q][1]);
                            ff_rel(h.z, l.z, jh.z, jo.z, o[q][2], o[q][5], hh[q][2], ll[q][2]);
                        }
                        nx[p] = pk(hh[0][0], hh[1][0]); nxl[p] = pk(ll[0][0], ll[1][0]);
                        ny[p] = pk(hh[0][1], hh[1][1]); nyl[p] = pk(ll[0][1], ll[1][1]);
                        nz[p] = pk(hh[0][2], hh[1][2]); nzl[p] = pk(ll[0][2], ll[1][2]);
                    }
            }
            tile_vjp<TJ, NP, ALL, GUARD, true>(tile, wt, nx, ny, nz, nxl, nyl, nzl, wkx, wky, wkz, mk, e2, ax, ay, az,
                                               S, Ax, Ay, Az, Bx, By, Bz, Cx, Cy, Cz, Gx, Gy, Gz, gm);
        } else if (mask == 0) {
            tile_vjp<TJ, NP, 0, GUARD, false>(tile, wt, nx, ny, nz, nxl, nyl, nzl, wkx, wky, wkz, mk, e2, ax, ay, az,
                                              S, Ax, Ay, Az, Bx, By, Bz, Cx, Cy, Cz, Gx, Gy, Gz, gm);
        } else {
            // chunk by chunk: a near chunk takes every pair on the float-float path
            // (pairs without a near chunk have zero lo parts)
#pragma unroll 1
            for (int c = 0; c < NCH; ++c) {
                unsigned any = 0;
#pragma unroll
                for (int p = 0; p < NP; ++p) any |= (cmask >> (p * NCH + c)) & 1u;
                if (any)
                    tile_vjp<TJ, NP, ALL, GUARD, false, 32>(tile, wt, nx, ny, nz, nxl, nyl, nzl, wkx, wky, wkz, mk,
                                                            e2, ax, ay, az, S, Ax, Ay, Az, Bx, By, Bz, Cx, Cy, Cz,
                                                            Gx, Gy, Gz, gm, 32 * c);
                else
                    tile_vjp<TJ, NP, 0, GUARD, false, 32>(tile, wt, nx, ny, nz, nxl, nyl, nzl, wkx, wky, wkz, mk, e2,
                                                          ax, ay, az, S, Ax, Ay, Az, Bx, By, Bz, Cx, Cy, Cz, Gx, Gy,
                                                          Gz, gm, 32 * c);
            }
        }
        // g = m_k (A - 3 B) - w_k S + 3 C for this tile, then fold into (hi, lo)
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            const f2 gx = add2(Gx[p], fma2(three, Cx[p], sub2(mul2(mk[p], sub2(Ax[p], mul2(three, Bx[p]))),
                                                               mul2(wkx[p], S[p]))));
            const f2 gy = add2(Gy[p], fma2(three, Cy[p], sub2(mul2(mk[p], sub2(Ay[p], mul2(three, By[p]))),
                                                               mul2(wky[p], S[p]))));
            const f2 gz = add2(Gz[p], fma2(three, Cz[p], sub2(mul2(mk[p], sub2(Az[p], mul2(three, Bz[p]))),
                                                               mul2(wkz[p], S[p]))));
            const f2 v[7] = {ax[p], ay[p], az[p], gx, gy, gz, sub2(0ull, gm[p])};
#pragma unroll
            for (int k = 0; k < 7; ++k) two_sum2(hi[p][k], lo[p][k], v[k]);
            ax[p] = ay[p] = az[p] = S[p] = Ax[p] = Ay[p] = Az[p] = Bx[p] = By[p] = Bz[p] = Cx[p] = Cy[p] = Cz[p] =
                gm[p] = 0ull;
            Gx[p] = Gy[p] = Gz[p] = 0ull;
        }
        __syncthreads();
        if (tid == 0 && it + NSTAGE < nt) {
            mbar_arrive_expect_tx(&bar[s], TILE_BYTES + WTILE_BYTES);
            bulk_g2s(spos + s * TF4, pack + (size_t)(t0 + it + NSTAGE) * TF4, TILE_BYTES, &bar[s]);
            bulk_g2s(sw + s * WF4, wpack + (size_t)(t0 + it + NSTAGE) * WF4, WTILE_BYTES, &bar[s]);
        }
    }
    if (bail) {
        if (tid == 0)
            for (int j = it; j < nt && j < it + NSTAGE; ++j)
                mbar_wait_bounded(&bar[j % NSTAGE], (unsigned)(j / NSTAGE) & 1u, err);
        return;
    }
    double *dst = partial + (size_t)blockIdx.y * 7 * npad;
#pragma unroll
    for (int p = 0; p < NP; ++p)
#pragma unroll
        for (int k = 0; k < 7; ++k) {
            float h0, h1, l0, l1;
            upk(hi[p][k], h0, h1);
            upk(lo[p][k], l0, l1);
            dst[(size_t)k * npad + ibase + (size_t)(2 * p) * NT + tid] = (double)h0 + (double)l0;
            dst[(size_t)k * npad + ibase + (size_t)(2 * p + 1) * NT + tid] = (double)h1 + (double)l1;
        }
}

// Adjoint vectors in sorted tile order: slot s of tile t at [t*WF4 + 2k].
template <int TJ>
__global__ void k_pack_w(const double *__restrict__ wx, const double *__restrict__ wy, const double *__restrict__ wz,
                         double scale, const uint32_t *__restrict__ perm, size_t n, size_t nslots,
                         float4 *__restrict__ wpack) {
    const size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nslots) return;
    float a = 0.f, b = 0.f, c = 0.f;
    if (s < n) {
        const uint32_t o = perm[s];
        if (CHK_IDX(o, n)) { a = (float)(scale * wx[o]); b = (float)(scale * wy[o]); c = (float)(scale * wz[o]); }
    }
    const size_t t = s / TJ, k = s % TJ;
    wpack[t * wtile_f4(TJ) + 2 * k] = make_float4(a, a, b, b);
    wpack[t * wtile_f4(TJ) + 2 * k + 1] = make_float4(c, c, 0.f, 0.f);
}

// f64 form of the fused kernel (reference gradients): double4 tiles of (x, y, z, m)
// and (wx, wy, wz, 0), one target per thread pair of accumulator sets.
template <int NT, int NSTAGE>
__global__ void __launch_bounds__(NT) k_force_vjp64(const double4 *__restrict__ pack, const double4 *__restrict__ wpack,
                                                    int ntiles, int tiles_per_split, double eps2,
                                                    double *__restrict__ partial, size_t npad) {
    __shared__ double4 sp[TJ64], sw[TJ64];
    const int tid = threadIdx.x;
    const size_t i = (size_t)blockIdx.x * NT + tid;
    const int t0 = blockIdx.y * tiles_per_split;
    const int t1 = min(ntiles, t0 + tiles_per_split);
    const double4 me = pack[i], wme = wpack[i];
    double a[3] = {0, 0, 0}, g[3] = {0, 0, 0}, gm = 0.0;
    for (int t = t0; t < t1; ++t) {
        __syncthreads();
        for (int k = tid; k < TJ64; k += NT) {
            sp[k] = pack[(size_t)t * TJ64 + k];
            sw[k] = wpack[(size_t)t * TJ64 + k];
        }
        __syncthreads();
        for (int j = 0; j < TJ64; ++j) {
            const double4 q = sp[j], w = sw[j];
            const double dx = q.x - me.x, dy = q.y - me.y, dz = q.z - me.z;
            const double s = fma(dz, dz, fma(dy, dy, fma(dx, dx, eps2)));
            if (s <= 0.0) continue;  // only the self pair at eps = 0
            const double ri = rsqrt(s), r3 = ri * ri * ri, r5 = r3 * ri * ri;
            const double mr3 = q.w * r3;
            a[0] = fma(mr3, dx, a[0]); a[1] = fma(mr3, dy, a[1]); a[2] = fma(mr3, dz, a[2]);
            const double ux = me.w * w.x - q.w * wme.x, uy = me.w * w.y - q.w * wme.y, uz = me.w * w.z - q.w * wme.z;
            const double du = ux * dx + uy * dy + uz * dz;
            const double c = 3.0 * r5 * du;
            g[0] += r3 * ux - c * dx; g[1] += r3 * uy - c * dy; g[2] += r3 * uz - c * dz;
            gm -= r3 * (w.x * dx + w.y * dy + w.z * dz);
        }
    }
    double *dst = partial + (size_t)blockIdx.y * 7 * npad;
    const double v[7] = {a[0], a[1], a[2], g[0], g[1], g[2], gm};
    for (int k = 0; k < 7; ++k) dst[(size_t)k * npad + i] = v[k];
}

__global__ void k_pack_w64(const double *__restrict__ wx, const double *__restrict__ wy, const double *__restrict__ wz,
                           double scale, const uint32_t *__restrict__ perm, size_t n, size_t nslots,
                           double4 *__restrict__ wpack) {
    const size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nslots) return;
    double a = 0, b = 0, c = 0;
    if (s < n) {
        const uint32_t o = perm[s];
        if (CHK_IDX(o, n)) { a = scale * wx[o]; b = scale * wy[o]; c = scale * wz[o]; }
    }
    wpack[s] = make_double4(a, b, c, 0.0);
}

// Sums the split partials of the fused kernel: a overwrites, g and gm accumulate (scaled).
__global__ void k_reduce_vjp(const double *__restrict__ partial, int nsplit, size_t npad, size_t n,
                             const uint32_t *__restrict__ perm, double *__restrict__ AX, double *__restrict__ AY,
                             double *__restrict__ AZ, double *__restrict__ GX, double *__restrict__ GY,
                             double *__restrict__ GZ, double *__restrict__ GM) {
    const size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    double r[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int js = 0; js < nsplit; ++js)
#pragma unroll
        for (int k = 0; k < 7; ++k) r[k] += partial[((size_t)js * 7 + k) * npad + s];
    const uint32_t o = perm[s];
    if (!CHK_IDX(o, n)) return;
    AX[o] = r[0]; AY[o] = r[1]; AZ[o] = r[2];
    GX[o] += r[3]; GY[o] += r[4]; GZ[o] += r[5];
    GM[o] += r[6];
}

// ---------------------------------------------------------------------------
// FP64_EXACT: the reference's arithmetic, one target per thread
// ---------------------------------------------------------------------------
// Small systems in FP64_EXACT: one thread per target leaves most of the GPU idle
// (a thousand targets are 32 warps), and GB300 runs f64 at a small fraction of
// f32.  The terms of the sum are independent; only their addition is ordered.  So
// a source chunk's terms (the reference's operations for pair (i, j), unchanged)
// are computed by N x C threads, and then every target adds its chunk of terms
// in ascending j (skipping j = i) onto its running sum: the same operations in
// the same order, bit for bit, with all SMs computing the terms.
constexpr size_t EXACT_SPLIT_MAX = 40000;            // larger systems fill the GPU with targets alone
constexpr size_t EXACT_TERMS_BYTES = size_t(192) << 20;  // term buffer per chunk

__global__ void k_exact_terms(const double *__restrict__ X, const double *__restrict__ Y,
                              const double *__restrict__ Z, const double *__restrict__ M, size_t n, size_t j0,
                              double eps2, double *__restrict__ TX, double *__restrict__ TY,
                              double *__restrict__ TZ) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t jj = blockIdx.y, j = j0 + jj, o = jj * n + i;
    if (j == i) {  // never added (the sum skips j = i)
        TX[o] = TY[o] = TZ[o] = 0.0;
        return;
    }
    const double xi = X[i], yi = Y[i], zi = Z[i];
    const double dx = __dsub_rn(X[j], xi), dy = __dsub_rn(Y[j], yi), dz = __dsub_rn(Z[j], zi);
    const double r2 = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)), eps2);
    const double inv_r3 = __ddiv_rn(1.0, __dmul_rn(r2, __dsqrt_rn(r2)));
    const double f = __dmul_rn(M[j], inv_r3);
    TX[o] = __dmul_rn(f, dx);
    TY[o] = __dmul_rn(f, dy);
    TZ[o] = __dmul_rn(f, dz);
}

// Adds a chunk's terms in ascending j onto each target's running sum (launched as
// 8-thread blocks: a thousand serial sums then spread over 125 SMs' f64 pipes).
// The sum is a serial chain, so its loads are issued 16 terms ahead of it.
__global__ void k_exact_sum(size_t n, size_t j0, int C, const double *__restrict__ TX,
                            const double *__restrict__ TY, const double *__restrict__ TZ, double *__restrict__ S) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double sx = S[i], sy = S[n + i], sz = S[2 * n + i];
    constexpr int B = 16;  // terms loaded together, then added one by one in order
    int jj = 0;
    for (; jj + B <= C; jj += B) {
        double tx[B], ty[B], tz[B];
#pragma unroll
        for (int u = 0; u < B; ++u) {
            const size_t o = (size_t)(jj + u) * n + i;
            tx[u] = TX[o]; ty[u] = TY[o]; tz[u] = TZ[o];
        }
#pragma unroll
        for (int u = 0; u < B; ++u) {
            if (j0 + (size_t)(jj + u) == i) continue;
            sx = __dadd_rn(sx, tx[u]);
            sy = __dadd_rn(sy, ty[u]);
            sz = __dadd_rn(sz, tz[u]);
        }
    }
    for (; jj < C; ++jj) {
        if (j0 + (size_t)jj == i) continue;
        const size_t o = (size_t)jj * n + i;
        sx = __dadd_rn(sx, TX[o]);
        sy = __dadd_rn(sy, TY[o]);
        sz = __dadd_rn(sz, TZ[o]);
    }
    S[i] = sx; S[n + i] = sy; S[2 * n + i] = sz;
}

__global__ void k_exact_store(size_t n, const double *__restrict__ S, double *__restrict__ AX,
                              double *__restrict__ AY, double *__restrict__ AZ, int accumulate) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (accumulate) {
        AX[i] = __dadd_rn(AX[i], S[i]); AY[i] = __dadd_rn(AY[i], S[n + i]); AZ[i] = __dadd_rn(AZ[i], S[2 * n + i]);
    } else {
        AX[i] = S[i]; AY[i] = S[n + i]; AZ[i] = S[2 * n + i];
    }
}

constexpr int EX_NT = 128;

__global__ void __launch_bounds__(EX_NT) k_direct_exact(const double *__restrict__ X, const double *__restrict__ Y,
                                                        const double *__restrict__ Z, const double *__restrict__ M,
                                                        size_t n, double eps2, double *__restrict__ AX,
                                                        double *__restrict__ AY, double *__restrict__ AZ,
                                                        int accumulate, const int64_t *__restrict__ targets,
                                                        size_t ntargets) {
    __shared__ double4 tile[EX_NT];
    const size_t k = (size_t)blockIdx.x * EX_NT + threadIdx.x;
    const size_t nt = targets ? ntargets : n;
    const bool active = k < nt;
    const size_t i = active ? (targets ? (size_t)targets[k] : k) : 0;
    const double xi = X[i], yi = Y[i], zi = Z[i];
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (size_t j0 = 0; j0 < n; j0 += EX_NT) {
        const size_t jl = j0 + threadIdx.x;
        __syncthreads();
        if (jl < n) tile[threadIdx.x] = make_double4(X[jl], Y[jl], Z[jl], M[jl]);
        __syncthreads();
        const int jn = (int)min((size_t)EX_NT, n - j0);
        for (int jj = 0; jj < jn; ++jj) {
            const size_t j = j0 + jj;
            if (j == i) continue;
            const double4 q = tile[jj];
            const double dx = __dsub_rn(q.x, xi), dy = __dsub_rn(q.y, yi), dz = __dsub_rn(q.z, zi);
            const double r2 = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)),
                                        eps2);
            const double inv_r3 = __ddiv_rn(1.0, __dmul_rn(r2, __dsqrt_rn(r2)));
            const double f = __dmul_rn(q.w, inv_r3);
            sx = __dadd_rn(sx, __dmul_rn(f, dx));
            sy = __dadd_rn(sy, __dmul_rn(f, dy));
            sz = __dadd_rn(sz, __dmul_rn(f, dz));
        }
    }
    if (!active) return;
    const size_t o = targets ? k : i;
    if (accumulate) {
        AX[o] = __dadd_rn(AX[o], sx); AY[o] = __dadd_rn(AY[o], sy); AZ[o] = __dadd_rn(AZ[o], sz);
    } else {
        AX[o] = sx; AY[o] = sy; AZ[o] = sz;
    }
}

template <class T>
void set_smem(T kernel, int bytes) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

// f64 min/max of the resident positions into dev_out6 = (min x, min y, min z, max x, max y, max z).
// min/max are exact, so the result equals the reference's sequential scan
// (BoundingBox::containing, crates/sim-core/src/octree.rs:14-44).
gvs_status bbox_minmax(Ctx *c, double *dev_out6, DevBuf &part_buf) {
    const size_t n = c->n;
    const int nb = std::min(c->num_sms * 4, std::max(1, ceil_div((long long)n, 256)));
    GVS_CUDA(c, ensure(c, part_buf, (size_t)nb * 6 * sizeof(double)));
    double *bb = as<double>(part_buf);
    k_bbox_part<<<nb, 256, 0, c->stream>>>(as<double>(c->x), as<double>(c->y), as<double>(c->z), n, bb);
    k_bbox_final<<<1, 256, 0, c->stream>>>(bb, nb);
    c->prof.launches += 2;
    GVS_CUDA(c, cudaMemcpyAsync(dev_out6, bb, 6 * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    return check_launch(c, "bounding box");
}

// Hilbert order of the resident positions: c->perm[s] = caller index of sorted slot s.
gvs_status spatial_order(Ctx *c) {
    const size_t n = c->n;
    if (n <= (size_t)SMALL_ORDER_MAX) {
        GVS_CUDA(c, ensure(c, c->perm, n * 4));
        int P = 32;
        while (P < (int)n) P <<= 1;
        const int smem = P * (int)(sizeof(uint64_t) + sizeof(uint32_t));
        set_smem(k_small_order, smem);
        // up to 1024 particles: one thread per padded slot (register stages); beyond, 1024 threads
        k_small_order<<<1, std::min(P, 1024), smem, c->stream>>>(as<double>(c->x), as<double>(c->y),
                                                                 as<double>(c->z), (int)n, P, as<uint32_t>(c->perm));
        c->prof.launches += 1;
        return check_launch(c, "small-system order");
    }
    const int nb = std::min(c->num_sms * 4, std::max(1, ceil_div((long long)n, 256)));
    GVS_CUDA(c, ensure(c, c->bbox_part, (size_t)nb * 6 * sizeof(double)));
    GVS_CUDA(c, ensure(c, c->keys, n * 8));
    GVS_CUDA(c, ensure(c, c->keys_alt, n * 8));
    GVS_CUDA(c, ensure(c, c->perm, n * 4));
    GVS_CUDA(c, ensure(c, c->perm_alt, n * 4));
    double *bb = as<double>(c->bbox_part);
    k_bbox_part<<<nb, 256, 0, c->stream>>>(as<double>(c->x), as<double>(c->y), as<double>(c->z), n, bb);
    k_bbox_final<<<1, 256, 0, c->stream>>>(bb, nb);
    k_hilbert<<<ceil_div((long long)n, 256), 256, 0, c->stream>>>(as<double>(c->x), as<double>(c->y),
                                                                  as<double>(c->z), n, bb, as<uint64_t>(c->keys),
                                                                  as<uint32_t>(c->perm));
    c->prof.launches += 3;
    GVS_TRY(check_launch(c, "hilbert keys"));
    uint64_t *ko;
    uint32_t *vo;
    GVS_TRY(radix_sort_u64(c, as<uint64_t>(c->keys), as<uint32_t>(c->perm), as<uint64_t>(c->keys_alt),
                           as<uint32_t>(c->perm_alt), n, 0, 64, &ko, &vo));
    if (vo != as<uint32_t>(c->perm)) {
        std::swap(c->perm, c->perm_alt);
        std::swap(c->keys, c->keys_alt);
    }
    return GVS_OK;
}

namespace {

struct Launch32 {
    int nt, np, nsplit;
};

// Chooses the j-split: at least ~4 waves of resident blocks, then the split
// whose last wave is fullest (every block costs the same, so a ragged last
// wave idles SMs), preferring fewer splits on ties.
int auto_split(Ctx *c, int iblocks, int ntiles, int blocks_per_sm) {
    const long long conc = (long long)c->num_sms * std::max(1, blocks_per_sm);
    const int lo = std::max(1, (int)((4 * conc + iblocks - 1) / iblocks));
    // splits of at least 4 source tiles amortise the partial sums; a system too small
    // to fill one wave that way (a few thousand particles) splits down to single tiles
    const int cap = (long long)iblocks * std::max(1, ntiles / 4) < conc ? ntiles : std::max(1, ntiles / 4);
    int best = std::min(lo, cap);
    double best_eff = -1.0;
    for (int ns = best; ns <= std::min(64, std::max(best, cap)); ++ns) {
        const int tps = ceil_div(ntiles, ns);
        const long long total = (long long)iblocks * ceil_div(ntiles, tps);
        const double waves = (double)total / conc;
        const double eff = waves / std::ceil(waves);
        if (eff > best_eff + 1e-3) { best_eff = eff; best = ns; }
    }
    return best;
}

template <int NT, int NP, bool MIXED, bool GUARD, int MINB = 1, int UNR = 4>
gvs_status launch32_t(Ctx *c, float eps2, int nsplit_req, double **partial_out, int *nsplit_out, size_t *npad_out) {
    constexpr int NSTAGE = 3;
    constexpr int TJ = NT;
    constexpr int IPT = 2 * NP;
    constexpr int TF4 = tile_f4(TJ);
    const size_t n = c->n;
    const int ntiles = ceil_div((long long)n, TJ);
    const size_t per_block = (size_t)NT * IPT;
    const int iblocks = ceil_div((long long)n, (long long)per_block);
    const size_t npad = (size_t)iblocks * per_block;
    const int ntiles_pad = (int)(npad / TJ);  // >= ntiles
    GVS_CUDA(c, ensure(c, c->jpack32, (size_t)ntiles_pad * TF4 * sizeof(float4)));
    // target-side padding tiles (beyond ntiles) are packed too: zero mass, never reduced
    k_pack32<TJ, MIXED><<<ntiles_pad, TJ, 0, c->stream>>>(as<double>(c->x), as<double>(c->y), as<double>(c->z),
                                                           as<double>(c->m), as<uint32_t>(c->perm), n,
                                                           as<float4>(c->jpack32), nullptr);
    c->prof.launches += 1;
    const int smem = NSTAGE * TF4 * (int)sizeof(float4);
    auto kern = k_direct32<NT, NP, NSTAGE, MIXED, GUARD, MINB, UNR>;
    set_smem(kern, smem);
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, smem);
    const int nsplit = nsplit_req > 0 ? std::min(nsplit_req, ntiles) : auto_split(c, iblocks, ntiles, std::max(1, per_sm));
    const int tps = ceil_div(ntiles, nsplit);
    const int nsplit_eff = ceil_div(ntiles, tps);
    GVS_CUDA(c, ensure(c, c->partial, (size_t)nsplit_eff * 3 * npad * sizeof(double)));
    dim3 grid(iblocks, nsplit_eff);
    int span = -1;  // profile timing span
    GVS_TRY(prof_begin(c, c->stream, &span));
    unsigned long long *nearc = reinterpret_cast<unsigned long long *>(err_ptr(c) + EW_NEAR_TILES);
    kern<<<grid, NT, smem, c->stream>>>(as<float4>(c->jpack32), ntiles, tps, eps2, as<double>(c->partial), npad,
                                        err_ptr(c), nearc);
    c->prof.launches += 1;
    GVS_TRY(check_launch(c, "direct f32 kernel"));
    if (c->prof.on) {
        GVS_TRY(prof_end(c, span, c->stream, &c->prof.force_ms));
        c->prof.force_launches += 1;
        c->prof.force_flops += 20.0 * (double)n * (double)n;
        c->prof.force_bytes += (double)nsplit_eff * (double)npad * 24.0 + (double)iblocks * nsplit_eff * tps *
                                                                              (double)TF4 * 16.0;
        // near-field decisions: per warp, source tile, 32-source chunk and target pair
        c->prof.tile_visits += (double)iblocks * (double)ntiles * (NT / 32) * (TJ / 32) * NP;
    }
    *partial_out = as<double>(c->partial);
    *nsplit_out = nsplit_eff;
    *npad_out = npad;
    return GVS_OK;
}

template <bool MIXED, bool GUARD>
gvs_status launch32(Ctx *c, float eps2, double **partial, int *nsplit, size_t *npad) {
    const long long bucket = 63 - __builtin_clzll((unsigned long long)std::max<size_t>(c->n, 1));
    for (const auto &e : c->tune_cache)
        if (e.first == bucket) c->tune = e.second;
    Tune t = c->tune;
    if (!direct_shape_eligible(c->n, t.nthreads)) {
        t.nthreads = 128;  // every unroll of the 128-thread, 4-target shape is compiled
        t.minb = 4;
    }
#define GVS_L32(NT_, NP_, MB_, U_)                                                        \
    if (t.nthreads == NT_ && t.ipt == 2 * NP_ && t.minb == MB_ && t.unroll == U_)          \
        return launch32_t<NT_, NP_, MIXED, GUARD, MB_, U_>(c, eps2, t.nsplit, partial, nsplit, npad);
    GVS_L32(128, 2, 4, 2)
    GVS_L32(128, 2, 4, 4)
    GVS_L32(128, 2, 4, 8)
    GVS_L32(128, 2, 4, 16)
    GVS_L32(256, 2, 2, 4)
    GVS_L32(256, 2, 2, 8)
    GVS_L32(256, 2, 2, 16)
    GVS_L32(512, 2, 1, 8)
    GVS_L32(512, 2, 1, 2)
#undef GVS_L32
    // default shape (Tune's defaults)
    return launch32_t<256, 2, MIXED, GUARD, 2, 2>(c, eps2, t.nsplit, partial, nsplit, npad);
}

gvs_status launch64(Ctx *c, double eps2, double **partial_out, int *nsplit_out, size_t *npad_out) {
    constexpr int NT = 128, IPT = 2, NSTAGE = 4;
    const size_t n = c->n;
    const size_t per_block = (size_t)NT * IPT;
    const int iblocks = ceil_div((long long)n, (long long)per_block);
    const size_t npad = (size_t)iblocks * per_block;
    const int ntiles = ceil_div((long long)n, TJ64);
    const size_t nslots = std::max(npad, (size_t)ntiles * TJ64);
    GVS_CUDA(c, ensure(c, c->jpack64, nslots * sizeof(double4)));
    k_pack64<<<ceil_div((long long)nslots, 256), 256, 0, c->stream>>>(as<double>(c->x), as<double>(c->y),
                                                                      as<double>(c->z), as<double>(c->m),
                                                                      as<uint32_t>(c->perm), n, nslots,
                                                                      as<double4>(c->jpack64));
    c->prof.launches += 1;
    const int nsplit = auto_split(c, iblocks, ntiles, 4);
    const int tps = ceil_div(ntiles, nsplit);
    const int nsplit_eff = ceil_div(ntiles, tps);
    GVS_CUDA(c, ensure(c, c->partial, (size_t)nsplit_eff * 3 * npad * sizeof(double)));
    const int smem = NSTAGE * TJ64 * (int)sizeof(double4);
    auto kern = eps2 > 0.0 ? k_direct64<NT, IPT, NSTAGE, false> : k_direct64<NT, IPT, NSTAGE, true>;
    set_smem(kern, smem);
    int span = -1;  // profile timing span
    GVS_TRY(prof_begin(c, c->stream, &span));
    kern<<<dim3(iblocks, nsplit_eff), NT, smem, c->stream>>>(as<double4>(c->jpack64), ntiles, tps, eps2,
                                                              as<double>(c->partial), npad, err_ptr(c));
    c->prof.launches += 1;
    GVS_TRY(check_launch(c, "direct f64 kernel"));
    if (c->prof.on) {
        GVS_TRY(prof_end(c, span, c->stream, &c->prof.force_ms));
        c->prof.force_launches += 1;
        c->prof.force_flops += 20.0 * (double)n * (double)n;
    }
    *partial_out = as<double>(c->partial);
    *nsplit_out = nsplit_eff;
    *npad_out = npad;
    return GVS_OK;
}

}  // namespace

gvs_status direct_forces(Ctx *c, int precision, double eps, bool accumulate) {
    const size_t n = c->n;
    if (n == 0) return GVS_OK;
    const double eps2 = eps * eps;
    if (precision == GVS_PREC_FP64_EXACT) {
        int span = -1;  // profile timing span
        GVS_TRY(prof_begin(c, c->stream, &span));
        if (n <= EXACT_SPLIT_MAX) {
            const int C = (int)std::max<size_t>(1, std::min<size_t>(n, EXACT_TERMS_BYTES / (24 * n)));
            GVS_CUDA(c, ensure(c, c->exact_terms, (size_t)C * n * 24));
            GVS_CUDA(c, ensure(c, c->exact_sums, n * 24));
            GVS_CUDA(c, cudaMemsetAsync(c->exact_sums.ptr, 0, n * 24, c->stream));
            double *T = as<double>(c->exact_terms);
            for (size_t j0 = 0; j0 < n; j0 += (size_t)C) {
                const int cc = (int)std::min<size_t>((size_t)C, n - j0);
                k_exact_terms<<<dim3(ceil_div((long long)n, 128), cc), 128, 0, c->stream>>>(
                    as<double>(c->x), as<double>(c->y), as<double>(c->z), as<double>(c->m), n, j0, eps2, T,
                    T + (size_t)cc * n, T + 2 * (size_t)cc * n);
                k_exact_sum<<<ceil_div((long long)n, 8), 8, 0, c->stream>>>(
                    n, j0, cc, T, T + (size_t)cc * n, T + 2 * (size_t)cc * n, as<double>(c->exact_sums));
                c->prof.launches += 2;
            }
            k_exact_store<<<ceil_div((long long)n, 256), 256, 0, c->stream>>>(
                n, as<double>(c->exact_sums), as<double>(c->ax), as<double>(c->ay), as<double>(c->az),
                accumulate ? 1 : 0);
            c->prof.launches += 1;
        } else {
            k_direct_exact<<<ceil_div((long long)n, EX_NT), EX_NT, 0, c->stream>>>(
                as<double>(c->x), as<double>(c->y), as<double>(c->z), as<double>(c->m), n, eps2, as<double>(c->ax),
                as<double>(c->ay), as<double>(c->az), accumulate ? 1 : 0, nullptr, 0);
            c->prof.launches += 1;
        }
        GVS_TRY(check_launch(c, "direct exact kernel"));
        if (c->prof.on) {
            GVS_TRY(prof_end(c, span, c->stream, &c->prof.force_ms));
            c->prof.force_launches += 1;
            c->prof.force_flops += 20.0 * (double)n * (double)(n - 1);
        }
        return GVS_OK;
    }
    GVS_TRY(spatial_order(c));
    double *partial = nullptr;
    int nsplit = 0;
    size_t npad = 0;
    if (precision == GVS_PREC_FP64) {
        GVS_TRY(launch64(c, eps2, &partial, &nsplit, &npad));
    } else {
        const float e2 = (float)eps2;
        const bool guard = !(e2 > 0.f);
        const bool mixed = precision == GVS_PREC_MIXED;
        if (mixed && !guard) GVS_TRY((launch32<true, false>(c, e2, &partial, &nsplit, &npad)));
        else if (mixed) GVS_TRY((launch32<true, true>(c, e2, &partial, &nsplit, &npad)));
        else if (!guard) GVS_TRY((launch32<false, false>(c, e2, &partial, &nsplit, &npad)));
        else GVS_TRY((launch32<false, true>(c, e2, &partial, &nsplit, &npad)));
    }
    k_reduce<<<ceil_div((long long)n, 256), 256, 0, c->stream>>>(partial, nsplit, npad, n, as<uint32_t>(c->perm),
                                                                  as<double>(c->ax), as<double>(c->ay),
                                                                  as<double>(c->az), accumulate ? 1 : 0);
    c->prof.launches += 1;
    return check_launch(c, "direct reduce");
}

// Fused forces + VJP on the resident positions with adjoint vectors scale * w
// (device arrays in caller order): a <- forces (overwrites the resident
// accelerations), g += VJP_x, gm += VJP_m.  MIXED / FP32 use the f32 tile
// kernel, FP64 / FP64_EXACT the f64 one.
gvs_status direct_force_vjp(Ctx *c, int precision, double eps, const double *wx, const double *wy, const double *wz,
                            double scale, double *gx, double *gy, double *gz, double *gm) {
    const size_t n = c->n;
    if (n == 0) return GVS_OK;
    GVS_TRY(spatial_order(c));
    cudaStream_t st = c->stream;
    const double eps2 = eps * eps;
    double *partial = nullptr;
    int nsplit_eff = 1;
    size_t npad = 0;
    int span = -1;  // profile timing span
    if (precision == GVS_PREC_MIXED || precision == GVS_PREC_FP32) {
        constexpr int NT = 128, NP = 1, NSTAGE = 3, TJ = NT, IPT = 2 * NP;
        constexpr int TF4 = tile_f4(TJ), WF4 = wtile_f4(TJ);
        const int ntiles = ceil_div((long long)n, TJ);
        const int iblocks = ceil_div((long long)n, (long long)NT * IPT);
        npad = (size_t)iblocks * NT * IPT;
        const int ntiles_pad = (int)(npad / TJ);
        GVS_CUDA(c, ensure(c, c->jpack32, (size_t)ntiles_pad * TF4 * sizeof(float4)));
        GVS_CUDA(c, ensure(c, c->scratch_a, (size_t)ntiles_pad * WF4 * sizeof(float4)));
        k_pack32<TJ, true><<<ntiles_pad, TJ, 0, st>>>(as<double>(c->x), as<double>(c->y), as<double>(c->z),
                                                      as<double>(c->m), as<uint32_t>(c->perm), n,
                                                      as<float4>(c->jpack32), nullptr);
        k_pack_w<TJ><<<ceil_div((long long)npad, 256), 256, 0, st>>>(wx, wy, wz, scale, as<uint32_t>(c->perm), n,
                                                                     npad, as<float4>(c->scratch_a));
        c->prof.launches += 2;
        const int smem = NSTAGE * (TF4 + WF4) * (int)sizeof(float4);
        const float e2 = (float)eps2;
        const bool guard = !(e2 > 0.f);
        auto kern = guard ? k_force_vjp32<NT, NP, NSTAGE, true> : k_force_vjp32<NT, NP, NSTAGE, false>;
        set_smem(kern, smem);
        int per_sm = 1;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, smem);
        const int nsplit = auto_split(c, iblocks, ntiles, std::max(1, per_sm));
        const int tps = ceil_div(ntiles, nsplit);
        nsplit_eff = ceil_div(ntiles, tps);
        GVS_CUDA(c, ensure(c, c->partial, (size_t)nsplit_eff * 7 * npad * sizeof(double)));
        partial = as<double>(c->partial);
        GVS_TRY(prof_begin(c, st, &span));
        kern<<<dim3(iblocks, nsplit_eff), NT, smem, st>>>(as<float4>(c->jpack32), as<float4>(c->scratch_a), ntiles,
                                                          tps, e2, partial, npad, err_ptr(c));
    } else {
        constexpr int NT = 128, NSTAGE = 1;
        const int ntiles = ceil_div((long long)n, TJ64);
        const int iblocks = ceil_div((long long)n, NT);
        npad = (size_t)iblocks * NT;
        const size_t nslots = std::max(npad, (size_t)ntiles * TJ64);
        GVS_CUDA(c, ensure(c, c->jpack64, nslots * sizeof(double4)));
        GVS_CUDA(c, ensure(c, c->scratch_a, nslots * sizeof(double4)));
        k_pack64<<<ceil_div((long long)nslots, 256), 256, 0, st>>>(as<double>(c->x), as<double>(c->y),
                                                                   as<double>(c->z), as<double>(c->m),
                                                                   as<uint32_t>(c->perm), n, nslots,
                                                                   as<double4>(c->jpack64));
        k_pack_w64<<<ceil_div((long long)nslots, 256), 256, 0, st>>>(wx, wy, wz, scale, as<uint32_t>(c->perm), n,
                                                                     nslots, as<double4>(c->scratch_a));
        c->prof.launches += 2;
        const int nsplit = auto_split(c, iblocks, ntiles, 4);
        const int tps = ceil_div(ntiles, nsplit);
        nsplit_eff = ceil_div(ntiles, tps);
        GVS_CUDA(c, ensure(c, c->partial, (size_t)nsplit_eff * 7 * npad * sizeof(double)));
        partial = as<double>(c->partial);
        GVS_TRY(prof_begin(c, st, &span));
        k_force_vjp64<NT, NSTAGE><<<dim3(iblocks, nsplit_eff), NT, 0, st>>>(
            as<double4>(c->jpack64), as<double4>(c->scratch_a), ntiles, tps, eps2, partial, npad);
    }
    c->prof.launches += 1;
    GVS_TRY(check_launch(c, "force+VJP kernel"));
    if (c->prof.on) {
        GVS_TRY(prof_end(c, span, st, &c->prof.vjp_ms));
        c->prof.vjp_launches += 1;
    }
    k_reduce_vjp<<<ceil_div((long long)n, 256), 256, 0, st>>>(partial, nsplit_eff, npad, n, as<uint32_t>(c->perm),
                                                              as<double>(c->ax), as<double>(c->ay), as<double>(c->az),
                                                              gx, gy, gz, gm);
    c->prof.launches += 1;
    return check_launch(c, "force+VJP reduce");
}

// ---- batched ensembles: map-driven packing and the persistent item kernel ----
// (tile size 128 = block size, 2 target pairs per thread, as the default single-system shape)
constexpr int ENS_TJ = 128, ENS_NP = 2, ENS_NSTAGE = 3, ENS_UNR = 2;

gvs_status ens_pack(Ctx *c, int ntiles, const uint32_t *map, float4 *pack) {
    k_pack32<ENS_TJ, true><<<ntiles, ENS_TJ, 0, c->stream>>>(as<double>(c->x), as<double>(c->y), as<double>(c->z),
                                                            as<double>(c->m), nullptr, c->n, pack, map);
    c->prof.launches += 1;
    return check_launch(c, "ensemble pack");
}

int ens_tile_float4s() { return tile_f4(ENS_TJ); }
int ens_tile() { return ENS_TJ; }
int ens_targets_per_block() { return ENS_TJ * 2 * ENS_NP; }

gvs_status ens_pairs(Ctx *c, const float4 *pack, const int4 *items, int nitems, unsigned *counter, float eps2,
                     double *partial, size_t npad, int ntiles, int nsplit) {
    const int smem = ENS_NSTAGE * tile_f4(ENS_TJ) * (int)sizeof(float4);
    const bool guard = !(eps2 > 0.f);
    auto kern = guard ? k_direct32_items<ENS_TJ, ENS_NP, ENS_NSTAGE, true, true, 4, ENS_UNR>
                      : k_direct32_items<ENS_TJ, ENS_NP, ENS_NSTAGE, true, false, 4, ENS_UNR>;
    set_smem(kern, smem);
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, ENS_TJ, smem);
    const int grid = std::max(1, std::min(nitems, c->num_sms * std::max(1, per_sm)));
    GVS_CUDA(c, cudaMemsetAsync(counter, 0, sizeof(unsigned), c->stream));
    unsigned long long *nearc = reinterpret_cast<unsigned long long *>(err_ptr(c) + EW_NEAR_TILES);
    kern<<<grid, ENS_TJ, smem, c->stream>>>(pack, items, nitems, counter, eps2, partial, npad, err_ptr(c), nearc,
                                            ntiles, nsplit);
    c->prof.launches += 1;
    return check_launch(c, "ensemble pair kernel");
}

// Times every compiled (block size, targets per thread) variant of the f32
// pair kernel on the resident state and keeps the fastest for this N bucket.
// Compiled shapes of the f32 pair kernel: (block size, targets per thread, min blocks per
// SM, source-loop unroll).  The first is the default.
static const int kShapes[][4] = {{256, 4, 2, 2},  {128, 4, 4, 4},  {128, 4, 4, 2},  {128, 4, 4, 8}, {128, 4, 4, 16},
                                 {256, 4, 2, 4},  {256, 4, 2, 8},  {256, 4, 2, 16}, {512, 4, 1, 8}, {512, 4, 1, 2}};

// Mixed-precision accuracy needs tiles that are small against the system: a tile
// size above n/64 (fewer than 64 tiles) let the f32 offsets of close pairs in
// tiles that are not flagged near lose up to 1e-5 relative in measurements on
// Plummer spheres, so such shapes fall back to 128-particle tiles.
bool direct_shape_eligible(size_t n, int nthreads) { return nthreads <= 128 || n >= (size_t)nthreads * 64; }

bool direct_shape_compiled(int nthreads, int ipt, int minb, int unroll) {
    for (const auto &cd : kShapes)
        if (cd[0] == nthreads && cd[1] == ipt && cd[2] == minb && cd[3] == unroll) return true;
    return false;
}

void set_direct_shape(Ctx *c, int nthreads, int ipt, int minb, int unroll) {
    c->tune.nthreads = nthreads;
    c->tune.ipt = ipt;
    c->tune.minb = minb;
    c->tune.unroll = unroll;
    c->tune.nsplit = 0;
    c->tune_cache.clear();  // a fixed shape overrides earlier autotune choices
}

gvs_status autotune_direct(Ctx *c, int precision, double eps, int *best_nt, int *best_ipt, double *best_ms) {
    // (block size, targets per thread, min blocks per SM, source-loop unroll)
    const auto &cand = kShapes;
    const bool was_on = c->prof.on;
    Tune best = c->tune;
    double best_t = 1e300;
    c->tune_report.clear();
    for (const auto &cd : cand) {
        if (!direct_shape_eligible(c->n, cd[0])) continue;
        c->tune.nthreads = cd[0];
        c->tune.ipt = cd[1];
        c->tune.minb = cd[2];
        c->tune.unroll = cd[3];
        c->tune.nsplit = 0;
        GVS_TRY(direct_forces(c, precision, eps, false));  // warm (also builds the order)
        c->prof.on = true;
        GVS_TRY(prof_settle(c));
        const double ms0 = c->prof.force_ms;
        for (int r = 0; r < 2; ++r) GVS_TRY(direct_forces(c, precision, eps, false));
        GVS_TRY(prof_settle(c));
        const double t = (c->prof.force_ms - ms0) / 2.0;
        c->prof.on = was_on;
        c->tune_report.push_back({c->tune, t});
        if (t < best_t) {
            best_t = t;
            best = c->tune;
        }
    }
    c->tune = best;
    long long bucket = 63 - __builtin_clzll((unsigned long long)std::max<size_t>(c->n, 1));
    bool found = false;
    for (auto &e : c->tune_cache)
        if (e.first == bucket) { e.second = best; found = true; }
    if (!found) c->tune_cache.push_back({bucket, best});
    if (best_nt) *best_nt = best.nthreads;
    if (best_ipt) *best_ipt = best.ipt;
    if (best_ms) *best_ms = best_t;
    return GVS_OK;
}

// FP64_EXACT accelerations of selected targets (accuracy probes at large N).
gvs_status direct_forces_subset(Ctx *c, int precision, double eps, const int64_t *idx_dev, size_t nidx,
                                double *out_dev) {
    (void)precision;
    if (nidx == 0) return GVS_OK;
    k_direct_exact<<<ceil_div((long long)nidx, EX_NT), EX_NT, 0, c->stream>>>(
        as<double>(c->x), as<double>(c->y), as<double>(c->z), as<double>(c->m), c->n, eps * eps, out_dev,
        out_dev + nidx, out_dev + 2 * nidx, 0, idx_dev, nidx);
    c->prof.launches += 1;
    return check_launch(c, "direct subset kernel");
}

GVS_CHECKED_UNIT(direct)

}  // namespace gvs
