// gvs_internal.cuh -- shared definitions for the gravis GB300 engine (sm_103a).
//
// The engine keeps one context per (caller, device): a CUDA stream, the
// particle state resident in HBM as f64 structure-of-arrays in the caller's
// order (the same 18 arrays as sim-core's Particles), and the scratch that the
// force paths need (spatial sort, packed j-tiles, per-split partial sums,
// octree arrays, SPH neighbour lists).  Every C-ABI call validates its
// arguments, runs on the context's stream and returns a gvs_status.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/gvs.h"

namespace gvs {

// ---------------------------------------------------------------------------
// device error word (bit flags written by kernels, read by the host)
// ---------------------------------------------------------------------------
enum DeviceError : unsigned {
    DERR_MBAR_TIMEOUT = 1u << 0,   // an mbarrier wait hit its iteration cap
    DERR_STACK_OVERFLOW = 1u << 1, // tree walk stack exhausted
    DERR_NEIGH_OVERFLOW = 1u << 2, // SPH neighbour buffer too small
    DERR_NAN = 1u << 3,            // non-finite value detected
    DERR_TREE = 1u << 4,           // tree build invariant violated
    DERR_BOUNDS = 1u << 5,         // checked build: index out of range
    DERR_SPIN_TIMEOUT = 1u << 6,   // a radix-sort look-back wait hit its cap
};

// Layout of the context's device word area (err_word, 64 u32): word 0 holds the
// DeviceError flags; the rest are counters that kernels add to and the profile
// reads (u64 counters take two aligned words).
enum ErrWordSlot : int {
    EW_FLAGS = 0,
    EW_NEAR_TILES = 8,      // u64: float-float near-field blocks of the f32 pair kernel
    EW_SPH_REDO = 10,       // mixed SPH particles rerun on the f64 path
    EW_BH_ITERS = 12,       // u64: BH group-walk iterations
    EW_BH_GROUPS = 14,      // BH groups walked
    EW_BH_FALLBACKS = 15,   // ... of which walked per particle
    EW_BH_TERMS = 16,       // u64: BH group-walk terms evaluated for real particles
    EW_WALK_TERMS = 18,     // u64: terms summed by the per-particle BH walks (f64, mixed, f32)
    EW_PROFILE_END = 20,    // profile counters: [EW_NEAR_TILES, EW_PROFILE_END)
    EW_NEIGH_WORK = 22,     // work counter of the SPH neighbour search
};

// ---------------------------------------------------------------------------
// a growable device buffer owned by the context
// ---------------------------------------------------------------------------
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
};

struct Ctx;
cudaError_t ensure(Ctx *c, DevBuf &b, size_t bytes);  // grows, never shrinks
template <class T> T *as(DevBuf &b) { return reinterpret_cast<T *>(b.ptr); }

// Profiling counters of one context (kernel time of the dominant kernels).
struct Prof {
    bool on = false;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    // timed spans: event pairs recorded on the kernels' streams and read at the next
    // settle (profile read), so that timing never blocks the host between launches
    std::vector<cudaEvent_t> pool;
    std::vector<std::pair<int, double *>> spans;  // (first event of the pair, where its ms go)
    int used = 0;
    double force_ms = 0.0;   // summed device time of force kernels
    long long force_launches = 0;
    long long launches = 0;  // every kernel this context launched
    double force_bytes = 0;  // algorithmic bytes moved by timed force kernels
    double force_flops = 0;  // algorithmic flops (20 per pair interaction)
    double tile_visits = 0;  // (warp, source tile, 32-source chunk, target pair) blocks of the f32 pair kernel
    double vjp_ms = 0;       // device time of the fused force + VJP kernels
    long long vjp_launches = 0;
};

struct Tune {
    int ipt = 4;       // i-particles per thread
    int nthreads = 256;
    int nsplit = 0;    // 0 = automatic
    int minb = 2;      // __launch_bounds__ minimum blocks per SM (register cap)
    int unroll = 2;    // source-loop unroll of the pair kernel
};

struct Ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    // a second stream for work that runs beside the main stream's (gravity beside the
    // SPH pass of a step), forked and joined with the two events
    cudaStream_t side = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    cudaEvent_t sph_join = nullptr;  // set while an SPH pass must wait for it before adding its accelerations
    std::string last_error;

    // resident state, caller order, capacity >= n
    size_t n = 0, cap = 0;
    DevBuf x, y, z, vx, vy, vz, ax, ay, az, m;
    DevBuf ptype, u, h, alpha, rho, pres, cs, du_dt, omega, div_v, max_mu, dalpha_dt;
    bool has_gas = false;

    // direct-sum scratch
    DevBuf keys, keys_alt, perm, perm_alt, sort_hist, bbox_part;
    DevBuf sort_state;  // radix sort: digit histograms, tile counters, look-back status
    DevBuf jpack32, jpack64, partial;
    DevBuf exact_terms, exact_sums;  // FP64_EXACT for small systems: a source chunk's terms, running sums
    // generic scratch
    DevBuf scratch_a, scratch_b, err_word, red_part, l2_flush;

    // host staging (pinned)
    void *pinned = nullptr;
    size_t pinned_bytes = 0;

    // tree / BH / SPH state lives in its own struct (bh.cu / sph.cu)
    void *tree = nullptr;
    void *sph = nullptr;
    void *ens = nullptr;
    void *adj = nullptr;

    Prof prof;
    Tune tune;
    int bh_group = -1;    // FP32 Barnes-Hut: particles per walk group (32, 64, 128), 0 = per-particle
                          // walk, -1 = 128 from 2^21 particles, else 64
    int bh_budget = 1024; // group-walk iterations before a group is walked per particle
    unsigned long long alloc_gen = 0;  // bumped whenever ensure() (re)allocates a buffer

    // One direct-sum KDK step captured as a CUDA graph, replayed by gvs_kdk_steps.
    // Valid while the step's parameters, n, the kernel shape and every buffer
    // address (alloc_gen) are the ones it was captured with.
    struct StepGraph {
        cudaGraphExec_t exec = nullptr;
        int precision = -1, nt = 0, ipt = 0, minb = 0, unroll = 0;
        double eps = 0.0, dt = 0.0;
        size_t n = 0;
        unsigned long long gen = 0;
        long long launches = 0;  // kernel launches in one replay
        bool disabled = false;   // capture failed once: stay eager
    } sgraph;
    std::vector<std::pair<long long, Tune>> tune_cache;  // (n bucket, choice)
    std::vector<std::pair<Tune, double>> tune_report;   // last autotune: every candidate and its ms

    // fault injection: GVS_FAULT / gvs_set_fault ("alloc", "launch", "nan@K")
    int fault_kind = 0;  // 0 none, 1 alloc, 2 launch, 3 nan
    long long fault_step = -1;
    long long step_counter = 0;
    unsigned long long pos_version = 0;  // bumped whenever resident positions change
    double peak_by_variant[3] = {0.0, 0.0, 0.0};  // FP32 probe: scalar, packed, mixed (TFLOP/s)
};

// Records an error message on the context and returns the status.
gvs_status fail(Ctx *c, gvs_status s, const char *fmt, ...);
gvs_status cuda_fail(Ctx *c, cudaError_t e, const char *what);
gvs_status check_launch(Ctx *c, const char *what);
gvs_status read_device_errors(Ctx *c);  // syncs the stream; DEVICE_ERROR if any flag
// Profile timing: prof_begin records the start of a span on `st` (slot -1 when the
// profile is off), prof_end its end, whose device time is added to *acc at the next
// prof_settle (which waits for every recorded span; gvs_profile_read calls it).
gvs_status prof_begin(Ctx *c, cudaStream_t st, int *slot);
gvs_status prof_end(Ctx *c, int slot, cudaStream_t st, double *acc);
gvs_status prof_settle(Ctx *c);

#define GVS_CUDA(c, expr)                                                  \
    do {                                                                   \
        cudaError_t _e = (expr);                                           \
        if (_e != cudaSuccess) return ::gvs::cuda_fail((c), _e, #expr);    \
    } while (0)

#define GVS_TRY(expr)                          \
    do {                                       \
        gvs_status _s = (expr);                \
        if (_s != GVS_OK) return _s;           \
    } while (0)

inline unsigned *err_ptr(Ctx *c) { return as<unsigned>(c->err_word); }

// ---------------------------------------------------------------------------
// checked build (-DGVS_CHECKED, built as libgvs_checked.so)
// ---------------------------------------------------------------------------
// Kernels test each index they compute -- through a permutation, a tree link, a
// leaf or neighbour slot, a work item -- against the array it indexes.  A bad
// index sets DERR_BOUNDS in this translation unit's flag word and the access is
// skipped (no kernel traps); the tree build also verifies its invariants
// (DERR_TREE).  read_device_errors gathers every unit's flags into the
// context's error word.  In the normal build CHK_IDX and CHK are `true` and the
// tests compile away.
#ifdef GVS_CHECKED
static __device__ unsigned g_checked_flags;
__device__ __forceinline__ bool chk_fail(unsigned bit) {
    atomicOr(&g_checked_flags, bit);
    return false;
}
#define CHK_IDX(i, bound) (((size_t)(i) < (size_t)(bound)) ? true : ::gvs::chk_fail((unsigned)::gvs::DERR_BOUNDS))
#define CHK(cond, bit) ((cond) ? true : ::gvs::chk_fail((unsigned)(bit)))
// Reads and clears this translation unit's flag word (host side).
static inline unsigned checked_take(cudaStream_t st) {
    unsigned v = 0;
    static const unsigned zero = 0;
    if (cudaMemcpyFromSymbolAsync(&v, g_checked_flags, sizeof v, 0, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyToSymbolAsync(g_checked_flags, &zero, sizeof zero, 0, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return DERR_BOUNDS;
    return v;
}
#define GVS_CHECKED_UNIT(name) \
    unsigned checked_take_##name(cudaStream_t st) { return checked_take(st); }
unsigned checked_take_bh(cudaStream_t st);
unsigned checked_take_direct(cudaStream_t st);
unsigned checked_take_sph(cudaStream_t st);
unsigned checked_take_ensemble(cudaStream_t st);
unsigned checked_take_sort(cudaStream_t st);
constexpr bool kChecked = true;
#else
#define CHK_IDX(i, bound) true
#define CHK(cond, bit) true
#define GVS_CHECKED_UNIT(name)
constexpr bool kChecked = false;
#endif

// ---------------------------------------------------------------------------
// PTX helpers: mbarrier + untiled bulk copy (cp.async.bulk), sm_90+ / sm_103a
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: returns false (and sets the error flag) after `cap` polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, unsigned parity, unsigned *err,
                                                  unsigned cap = 1u << 22) {
    for (unsigned it = 0; it < cap; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    if (err) atomicOr(err, (unsigned)DERR_MBAR_TIMEOUT);
    return false;
}

// 1-D bulk copy global -> this CTA's shared memory, completing on `bar`.
// Both addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst_smem, const void *src_gmem, unsigned bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst_smem)),
        "l"(src_gmem), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ float rsqrt_approx(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Error-free transformation (Knuth two-sum): s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    float bp = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
}

// f32x2 helpers (packed two-lane f32 arithmetic, sm_100+)
typedef unsigned long long f2;  // two f32 lanes in one 64-bit register pair

__device__ __forceinline__ f2 pk(float a, float b) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void upk(f2 v, float &a, float &b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ f2 add2(f2 a, f2 b) {
    f2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
    f2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
    f2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
    f2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

// (hi, lo) += v, lane-wise, with Knuth's two-sum (error-free for hi + v).
__device__ __forceinline__ void two_sum2(f2 &hi, f2 &lo, f2 v) {
    const f2 s = add2(hi, v);
    const f2 bp = sub2(s, hi);
    const f2 e = add2(sub2(hi, sub2(s, bp)), sub2(v, bp));
    lo = add2(lo, e);
    hi = s;
}

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// 63-bit Hilbert key of a point quantised to 21 bits per axis (Skilling's
// transpose method, "Programming the Hilbert curve", AIP Conf. Proc. 707, 2004).
// The bounding box of a Plummer sphere is set by a few outliers (r ~ 1e3 at
// N = 2^20), so 21 bits are needed to resolve the core; Hilbert rather than
// Morton order because consecutive runs of a Hilbert curve stay contiguous,
// which keeps the 128-particle tiles (and their f32 offsets) small.
__device__ __forceinline__ uint64_t hilbert_key(uint32_t x0, uint32_t x1, uint32_t x2) {
    uint32_t X[3] = {x0, x1, x2};
    const uint32_t M = 1u << 20;
    for (uint32_t Q = M; Q > 1; Q >>= 1) {
        const uint32_t P = Q - 1;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            if (X[i] & Q) {
                X[0] ^= P;
            } else {
                const uint32_t t = (X[0] ^ X[i]) & P;
                X[0] ^= t;
                X[i] ^= t;
            }
        }
    }
    X[1] ^= X[0];
    X[2] ^= X[1];
    uint32_t t = 0;
    for (uint32_t Q = M; Q > 1; Q >>= 1)
        if (X[2] & Q) t ^= Q - 1;
    X[0] ^= t; X[1] ^= t; X[2] ^= t;
    uint64_t key = 0;
    for (int b = 20; b >= 0; --b)
#pragma unroll
        for (int i = 0; i < 3; ++i) key = (key << 1) | ((X[i] >> b) & 1u);
    return key;
}


// ---------------------------------------------------------------------------
// subsystem entry points (defined in the .cu files)
// ---------------------------------------------------------------------------
// sort.cu
gvs_status radix_sort_u64(Ctx *c, uint64_t *keys, uint32_t *vals, uint64_t *keys_alt, uint32_t *vals_alt, size_t n,
                          int begin_bit, int end_bit, uint64_t **keys_out, uint32_t **vals_out);
gvs_status exclusive_scan_u32(Ctx *c, const uint32_t *in, uint32_t *out, size_t n, uint32_t *total_dev);
// direct.cu
gvs_status direct_forces(Ctx *c, int precision, double eps, bool accumulate);
gvs_status direct_force_vjp(Ctx *c, int precision, double eps, const double *wx, const double *wy, const double *wz,
                            double scale, double *gx, double *gy, double *gz, double *gm);
gvs_status direct_forces_subset(Ctx *c, int precision, double eps, const int64_t *idx_dev, size_t nidx,
                                double *out_dev);
gvs_status spatial_order(Ctx *c);
gvs_status bbox_minmax(Ctx *c, double *dev_out6, DevBuf &part_buf);
bool direct_shape_compiled(int nthreads, int ipt, int minb, int unroll);
bool direct_shape_eligible(size_t n, int nthreads);
void set_direct_shape(Ctx *c, int nthreads, int ipt, int minb, int unroll);
gvs_status autotune_direct(Ctx *c, int precision, double eps, int *best_nt, int *best_ipt, double *best_ms);
// kdk.cu
gvs_status kick(Ctx *c, double half_dt);
gvs_status kick_drift(Ctx *c, double half_dt, double dt);
gvs_status clear_acc(Ctx *c);
// n <= 32, FP64_EXACT direct sum: nsteps whole KDK steps in one launch (bit-identical)
bool kdk_tiny_eligible(const Ctx *c);
gvs_status kdk_tiny_exact(Ctx *c, double eps, double dt, long long nsteps);
// diag.cu
gvs_status diagnostics(Ctx *c, double eps, int with_potential, gvs_diag *out);
// bh.cu
gvs_status bh_forces(Ctx *c, double eps, double theta, int precision, bool accumulate);
gvs_status tree_build(Ctx *c);
void tree_free(Ctx *c);
// Read-only view of the octree of the resident positions (device pointers).
// Nodes are in depth-first pre-order; node k covers sorted slots
// [first[k], first[k] + count) and its subtree ends at node skip[k].
struct TreeView {
    size_t n, nnodes;
    const uint8_t *level;
    const uint32_t *first, *cnt, *skip, *perm, *parent, *leaf_of;  // leaf_of[j]: the leaf holding particle j
    const double *bx, *by, *bz, *sx, *sy, *sz;  // cell centres; sorted positions
    double root_hw;                              // half width at depth 0 (depth L: root_hw * 2^-L)
};
gvs_status tree_view(Ctx *c, TreeView *v);
gvs_status tree_export(Ctx *c, size_t cap, uint8_t *level, uint32_t *first, uint32_t *cnt, uint32_t *skip,
                       double *mass, double *com, uint32_t *perm, uint64_t *keys, size_t *nnodes);
// sph.cu
gvs_status sph_compute(Ctx *c, const gvs_sph_params *prm);
gvs_status sph_timestep(Ctx *c, const gvs_sph_params *prm, double *dt_out);
gvs_status sph_step(Ctx *c, const gvs_sph_params *prm, int algo, int precision, double eps, double theta, double dt,
                    double *dt_next);
gvs_status sph_neighbors_export(Ctx *c, size_t cap, uint32_t *start, uint32_t *count, uint32_t *idx, size_t *total);
void sph_free(Ctx *c);

// ics_dev.cu: PlummerSphere::generate on the device into the resident x..m (n allocated)
gvs_status ic_plummer_device(Ctx *c, size_t n, uint64_t seed, double a, double total_mass);
gvs_status ic_collision_device(Ctx *c, size_t n, uint64_t seed, double separation);
// adjoint.cu
void adj_free(Ctx *c);
// ensemble.cu
void ens_free(Ctx *c);

// forces on resident state according to the algorithm selector
gvs_status gravity(Ctx *c, int algo, int precision, double eps, double theta, bool accumulate);

}  // namespace gvs
