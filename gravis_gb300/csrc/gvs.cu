// gvs.cu -- context management and the C ABI entry points of libgvs.so.
//
// The entry points mirror sim-core's hot-path interfaces:
//   GravitySolver::compute_accelerations  (crates/sim-core/src/gravity.rs:6-10)
//   LeapfrogKDK::step                      (crates/sim-core/src/integrator.rs:42-76)
//   diagnostics::compute                   (crates/sim-core/src/diagnostics.rs:37-48)
// Every call validates its arguments before touching the device, runs on the
// context's stream, and reports failures as a gvs_status plus a message.
#include <stdarg.h>
#include <stdlib.h>

#include <algorithm>

#include "gvs_internal.cuh"

namespace gvs {

static char g_last_error[512] = "";

cudaError_t ensure(Ctx *c, DevBuf &b, size_t bytes) {
    if (bytes <= b.bytes && b.ptr) return cudaSuccess;
    if (c->fault_kind == 1) return cudaErrorMemoryAllocation;  // injected
    if (b.ptr) {
        cudaError_t e = cudaFree(b.ptr);  // synchronises: no kernel still uses it
        if (e != cudaSuccess) return e;
        b.ptr = nullptr;
        b.bytes = 0;
    }
    size_t want = std::max<size_t>(bytes, 256);
    c->alloc_gen++;
    cudaError_t e = cudaMalloc(&b.ptr, want);
    if (e != cudaSuccess) {
        b.ptr = nullptr;
        return e;
    }
    b.bytes = want;
    return cudaSuccess;
}

gvs_status fail(Ctx *c, gvs_status s, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->last_error = buf;
    snprintf(g_last_error, sizeof g_last_error, "%s", buf);
    return s;
}

gvs_status cuda_fail(Ctx *c, cudaError_t e, const char *what) {
    gvs_status s = (e == cudaErrorMemoryAllocation) ? GVS_ERR_OOM : GVS_ERR_LAUNCH;
    if (c && c->fault_kind == 1 && e == cudaErrorMemoryAllocation) s = GVS_ERR_INJECTED;
    return fail(c, s, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

gvs_status check_launch(Ctx *c, const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(c, e, what);
    return GVS_OK;
}

// Moves the checked build's per-unit flags into the context's error word.
static gvs_status gather_checked_flags(Ctx *c) {
#ifdef GVS_CHECKED
    cudaStream_t st = c->stream;
    const unsigned f = checked_take_bh(st) | checked_take_direct(st) | checked_take_sph(st) |
                       checked_take_ensemble(st) | checked_take_sort(st);
    if (f) {
        unsigned w = 0;
        GVS_CUDA(c, cudaMemcpy(&w, c->err_word.ptr, sizeof w, cudaMemcpyDeviceToHost));
        w |= f;
        GVS_CUDA(c, cudaMemcpy(c->err_word.ptr, &w, sizeof w, cudaMemcpyHostToDevice));
    }
#else
    (void)c;
#endif
    return GVS_OK;
}

gvs_status read_device_errors(Ctx *c) {
    unsigned flags = 0;
    GVS_CUDA(c, cudaStreamSynchronize(c->stream));
    GVS_TRY(gather_checked_flags(c));
    GVS_CUDA(c, cudaMemcpyAsync(&flags, c->err_word.ptr, sizeof flags, cudaMemcpyDeviceToHost, c->stream));
    GVS_CUDA(c, cudaStreamSynchronize(c->stream));
    if (flags) {
        GVS_CUDA(c, cudaMemsetAsync(c->err_word.ptr, 0, sizeof(unsigned), c->stream));
        gvs_status s = (flags & (DERR_MBAR_TIMEOUT | DERR_SPIN_TIMEOUT)) ? GVS_ERR_TIMEOUT : GVS_ERR_DEVICE;
        return fail(c, s, "device error word 0x%x (1 mbarrier timeout, 2 stack overflow, 4 neighbour overflow, "
                          "8 non-finite, 16 tree invariant, 32 index out of range, 64 sort look-back timeout)",
                    flags);
    }
    return GVS_OK;
}

gvs_status gravity(Ctx *c, int algo, int precision, double eps, double theta, bool accumulate) {
    if (c->fault_kind == 2) return fail(c, GVS_ERR_INJECTED, "injected launch fault");
    switch (algo) {
    case GVS_ALGO_NONE:
        return accumulate ? GVS_OK : clear_acc(c);
    case GVS_ALGO_DIRECT:
        return direct_forces(c, precision, eps, accumulate);
    case GVS_ALGO_BH:
        return bh_forces(c, eps, theta, precision, accumulate);
    default:
        return fail(c, GVS_ERR_INVALID_ARG, "unknown gravity algorithm %d", algo);
    }
}

static gvs_status upload(Ctx *c, DevBuf &b, const void *src, size_t bytes) {
    GVS_CUDA(c, ensure(c, b, bytes));
    if (src) GVS_CUDA(c, cudaMemcpyAsync(b.ptr, src, bytes, cudaMemcpyHostToDevice, c->stream));
    return GVS_OK;
}

static gvs_status download(Ctx *c, void *dst, DevBuf &b, size_t bytes) {
    if (!dst || bytes == 0) return GVS_OK;
    GVS_CUDA(c, cudaMemcpyAsync(dst, b.ptr, bytes, cudaMemcpyDeviceToHost, c->stream));
    return GVS_OK;
}

static gvs_status alloc_state(Ctx *c, size_t n) {
    c->pos_version++;
    const size_t b = std::max<size_t>(n, 1) * sizeof(double);
    DevBuf *f64s[] = {&c->x, &c->y, &c->z, &c->vx, &c->vy, &c->vz, &c->ax, &c->ay, &c->az, &c->m,
                      &c->u, &c->h, &c->alpha, &c->rho, &c->pres, &c->cs, &c->du_dt, &c->omega,
                      &c->div_v, &c->max_mu, &c->dalpha_dt};
    for (DevBuf *d : f64s) GVS_CUDA(c, ensure(c, *d, b));
    GVS_CUDA(c, ensure(c, c->ptype, std::max<size_t>(n, 1)));
    c->n = n;
    return GVS_OK;
}

static bool nan_fault_due(Ctx *c) {
    return c->fault_kind == 3 && c->fault_step >= 0 && c->step_counter == c->fault_step;
}

// One KDK step on the resident state (integrator.rs:42-76).
static gvs_status kdk_one(Ctx *c, int algo, int precision, double eps, double theta, double dt) {
    const double half = 0.5 * dt;
    GVS_TRY(kick_drift(c, half, dt));  // half-kick, drift, clear_accelerations
    GVS_TRY(gravity(c, algo, precision, eps, theta, /*accumulate=*/false));
    GVS_TRY(kick(c, half));
    c->step_counter++;
    return GVS_OK;
}

gvs_status prof_begin(Ctx *c, cudaStream_t st, int *slot) {
    *slot = -1;
    if (!c->prof.on) return GVS_OK;
    Prof &p = c->prof;
    if (p.used + 2 > (int)p.pool.size()) {
        if (p.pool.size() >= 1024) {
            GVS_TRY(prof_settle(c));  // a long run without a read: settle, then reuse the pool
        } else {
            for (int k = 0; k < 2; ++k) {
                cudaEvent_t e = nullptr;
                GVS_CUDA(c, cudaEventCreate(&e));
                p.pool.push_back(e);
            }
        }
    }
    *slot = p.used;
    p.used += 2;
    GVS_CUDA(c, cudaEventRecord(p.pool[(size_t)*slot], st));
    return GVS_OK;
}

gvs_status prof_end(Ctx *c, int slot, cudaStream_t st, double *acc) {
    if (slot < 0) return GVS_OK;
    GVS_CUDA(c, cudaEventRecord(c->prof.pool[(size_t)slot + 1], st));
    c->prof.spans.emplace_back(slot, acc);
    return GVS_OK;
}

gvs_status prof_settle(Ctx *c) {
    Prof &p = c->prof;
    for (const auto &sp : p.spans) {
        GVS_CUDA(c, cudaEventSynchronize(p.pool[(size_t)sp.first + 1]));
        float ms = 0.f;
        GVS_CUDA(c, cudaEventElapsedTime(&ms, p.pool[(size_t)sp.first], p.pool[(size_t)sp.first + 1]));
        *sp.second += ms;
    }
    p.spans.clear();
    p.used = 0;
    return GVS_OK;
}

}  // namespace gvs

using namespace gvs;

struct gvs_ctx : public Ctx {};

struct StepGraphKey {
    int precision;
    double eps, dt;
    size_t n;
    Tune tune;
};

static bool sgraph_valid(Ctx *c, const StepGraphKey &k) {
    const auto &g = c->sgraph;
    return g.exec && g.precision == k.precision && g.eps == k.eps && g.dt == k.dt && g.n == k.n &&
           g.gen == c->alloc_gen && g.nt == k.tune.nthreads && g.ipt == k.tune.ipt && g.minb == k.tune.minb &&
           g.unroll == k.tune.unroll;
}

// Captures one kdk_one into c->sgraph; on a capture error the context stays eager.
static gvs_status sgraph_capture(Ctx *c, const StepGraphKey &k, int algo, double theta) {
    auto &g = c->sgraph;
    if (g.exec) { cudaGraphExecDestroy(g.exec); g.exec = nullptr; }
    const unsigned long long gen0 = c->alloc_gen;
    const long long l0 = c->prof.launches;
    const long long step0 = c->step_counter;
    const unsigned long long pv0 = c->pos_version;
    if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        g.disabled = true;
        return GVS_OK;
    }
    const gvs_status st = kdk_one(c, algo, k.precision, k.eps, theta, k.dt);
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
    // the captured step has not run: undo its host-side bookkeeping
    g.launches = c->prof.launches - l0;
    c->prof.launches = l0;
    c->step_counter = step0;
    c->pos_version = pv0;
    if (st != GVS_OK || e != cudaSuccess || c->alloc_gen != gen0) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        g.disabled = true;  // the eager loop takes over
        return GVS_OK;
    }
    const cudaError_t ei = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) {
        g.exec = nullptr;
        cudaGetLastError();
        g.disabled = true;
        return GVS_OK;
    }
    g.precision = k.precision;
    g.eps = k.eps;
    g.dt = k.dt;
    g.n = k.n;
    g.gen = c->alloc_gen;
    // the shape the step ran with (the per-n autotune choice may have replaced c->tune)
    g.nt = c->tune.nthreads;
    g.ipt = c->tune.ipt;
    g.minb = c->tune.minb;
    g.unroll = c->tune.unroll;
    return GVS_OK;
}

static gvs_status check_ctx(const gvs_ctx *ctx) {
    if (!ctx) {
        snprintf(g_last_error, sizeof g_last_error, "null context");
        return GVS_ERR_INVALID_ARG;
    }
    return GVS_OK;
}

extern "C" {

const char *gvs_version(void) {
    return kChecked ? "gravis-gb300 0.1.0 (sm_103a, checked)" : "gravis-gb300 0.1.0 (sm_103a)";
}

gvs_status gvs_create(gvs_ctx **out, int device) {
    if (!out) return fail(nullptr, GVS_ERR_INVALID_ARG, "gvs_create: out is NULL");
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return fail(nullptr, GVS_ERR_NO_DEVICE, "no CUDA device (%s)", cudaGetErrorString(e));
    if (device < 0 || device >= ndev) return fail(nullptr, GVS_ERR_INVALID_ARG, "device %d out of range", device);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess)
        return fail(nullptr, GVS_ERR_NO_DEVICE, "cannot query device %d", device);
    if (prop.major < 10)
        return fail(nullptr, GVS_ERR_NO_DEVICE, "device %d is sm_%d%d; this build targets sm_103a", device,
                    prop.major, prop.minor);
    if (cudaSetDevice(device) != cudaSuccess) return fail(nullptr, GVS_ERR_NO_DEVICE, "cudaSetDevice failed");
    gvs_ctx *c = new gvs_ctx();
    c->device = device;
    c->num_sms = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->join_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&c->prof.ev[0]) != cudaSuccess || cudaEventCreate(&c->prof.ev[1]) != cudaSuccess) {
        gvs_destroy(c);  // releases whichever streams and events were created
        return fail(nullptr, GVS_ERR_LAUNCH, "stream/event creation failed");
    }
    if (ensure(c, c->err_word, 256) != cudaSuccess ||
        cudaMemsetAsync(c->err_word.ptr, 0, 256, c->stream) != cudaSuccess) {
        gvs_destroy(c);
        return fail(nullptr, GVS_ERR_OOM, "cannot allocate the device error word");
    }
    if (const char *f = getenv("GVS_FAULT")) gvs_set_fault(c, f);
    *out = c;
    return GVS_OK;
}

gvs_status gvs_destroy(gvs_ctx *c) {
    if (!c) return GVS_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->side) cudaStreamSynchronize(c->side);
    if (c->sgraph.exec) cudaGraphExecDestroy(c->sgraph.exec);
    tree_free(c);
    sph_free(c);
    adj_free(c);
    ens_free(c);
    DevBuf *all[] = {&c->x, &c->y, &c->z, &c->vx, &c->vy, &c->vz, &c->ax, &c->ay, &c->az, &c->m,
                     &c->ptype, &c->u, &c->h, &c->alpha, &c->rho, &c->pres, &c->cs, &c->du_dt, &c->omega,
                     &c->div_v, &c->max_mu, &c->dalpha_dt, &c->keys, &c->keys_alt, &c->perm, &c->perm_alt,
                     &c->exact_terms, &c->exact_sums,
                     &c->sort_hist, &c->sort_state, &c->bbox_part, &c->jpack32, &c->jpack64, &c->partial, &c->scratch_a,
                     &c->scratch_b, &c->err_word, &c->red_part, &c->l2_flush};
    for (DevBuf *b : all)
        if (b->ptr) cudaFree(b->ptr);
    if (c->pinned) cudaFreeHost(c->pinned);
    for (int k = 0; k < 2; ++k)
        if (c->prof.ev[k]) cudaEventDestroy(c->prof.ev[k]);
    for (cudaEvent_t e : c->prof.pool) cudaEventDestroy(e);
    if (c->fork_ev) cudaEventDestroy(c->fork_ev);
    if (c->join_ev) cudaEventDestroy(c->join_ev);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return GVS_OK;
}

gvs_status gvs_last_error(const gvs_ctx *c, char *buf, size_t len) {
    if (!buf || len == 0) return GVS_ERR_INVALID_ARG;
    const char *msg = c ? c->last_error.c_str() : g_last_error;
    snprintf(buf, len, "%s", msg);
    return GVS_OK;
}

gvs_status gvs_set_fault(gvs_ctx *c, const char *spec) {
    GVS_TRY(check_ctx(c));
    if (!spec) return fail(c, GVS_ERR_INVALID_ARG, "fault spec is NULL");
    if (!strcmp(spec, "none") || !*spec) {
        c->fault_kind = 0;
    } else if (!strcmp(spec, "alloc")) {
        c->fault_kind = 1;
    } else if (!strcmp(spec, "launch")) {
        c->fault_kind = 2;
    } else if (!strncmp(spec, "nan@", 4)) {
        char *end = nullptr;
        long long k = strtoll(spec + 4, &end, 10);
        if (!end || *end || k < 0) return fail(c, GVS_ERR_INVALID_ARG, "bad fault spec '%s'", spec);
        c->fault_kind = 3;
        c->fault_step = k;
        c->step_counter = 0;
    } else {
        return fail(c, GVS_ERR_INVALID_ARG, "unknown fault spec '%s' (none|alloc|launch|nan@K)", spec);
    }
    return GVS_OK;
}

gvs_status gvs_sync(gvs_ctx *c) {
    GVS_TRY(check_ctx(c));
    GVS_CUDA(c, cudaStreamSynchronize(c->stream));
    return read_device_errors(c);
}

gvs_status gvs_device_errors(gvs_ctx *c, unsigned *flags) {
    GVS_TRY(check_ctx(c));
    if (!flags) return fail(c, GVS_ERR_INVALID_ARG, "flags is NULL");
    GVS_CUDA(c, cudaStreamSynchronize(c->stream));
    GVS_TRY(gather_checked_flags(c));
    GVS_CUDA(c, cudaMemcpyAsync(flags, c->err_word.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    GVS_CUDA(c, cudaStreamSynchronize(c->stream));
    GVS_CUDA(c, cudaMemsetAsync(c->err_word.ptr, 0, sizeof(unsigned), c->stream));
    return GVS_OK;
}

size_t gvs_count(const gvs_ctx *c) { return c ? c->n : 0; }

gvs_status gvs_set_state(gvs_ctx *c, size_t n, const double *x, const double *y, const double *z, const double *vx,
                         const double *vy, const double *vz, const double *mass, const uint8_t *ptype,
                         const double *u, const double *h, const double *alpha) {
    GVS_TRY(check_ctx(c));
    if (!x || !y || !z || !vx || !vy || !vz || !mass) return fail(c, GVS_ERR_INVALID_ARG, "null state array");
    if (n > 0xFFFFFFF0ull) return fail(c, GVS_ERR_INVALID_ARG, "n = %zu exceeds 32-bit indexing", n);
    if (c->fault_kind == 1) return fail(c, GVS_ERR_INJECTED, "injected allocation fault");
    cudaSetDevice(c->device);
    GVS_TRY(alloc_state(c, n));
    const size_t b = n * sizeof(double);
    GVS_TRY(upload(c, c->x, x, b)); GVS_TRY(upload(c, c->y, y, b)); GVS_TRY(upload(c, c->z, z, b));
    GVS_TRY(upload(c, c->vx, vx, b)); GVS_TRY(upload(c, c->vy, vy, b)); GVS_TRY(upload(c, c->vz, vz, b));
    GVS_TRY(upload(c, c->m, mass, b));
    c->pos_version++;
    GVS_TRY(clear_acc(c));
    c->has_gas = ptype != nullptr;
    if (ptype) GVS_CUDA(c, cudaMemcpyAsync(c->ptype.ptr, ptype, n, cudaMemcpyHostToDevice, c->stream));
    else GVS_CUDA(c, cudaMemsetAsync(c->ptype.ptr, 0, std::max<size_t>(n, 1), c->stream));
    DevBuf *zero[] = {&c->rho, &c->pres, &c->cs, &c->du_dt, &c->div_v, &c->max_mu, &c->dalpha_dt};
    for (DevBuf *d : zero) GVS_CUDA(c, cudaMemsetAsync(d->ptr, 0, std::max<size_t>(b, 8), c->stream));
    if (u) GVS_TRY(upload(c, c->u, u, b)); else GVS_CUDA(c, cudaMemsetAsync(c->u.ptr, 0, std::max<size_t>(b, 8), c->stream));
    if (h) GVS_TRY(upload(c, c->h, h, b)); else GVS_CUDA(c, cudaMemsetAsync(c->h.ptr, 0, std::max<size_t>(b, 8), c->stream));
    if (alpha) GVS_TRY(upload(c, c->alpha, alpha, b));
    else GVS_CUDA(c, cudaMemsetAsync(c->alpha.ptr, 0, std::max<size_t>(b, 8), c->stream));
    c->step_counter = 0;
    GVS_CUDA(c, cudaStreamSynchronize(c->stream));
    return GVS_OK;
}

// The resident state of an n-particle gas-free system with zero accelerations, whose
// x..m a device generator then fills.
static gvs_status device_ics_prepare(gvs_ctx *c, size_t n) {
    if (c->fault_kind == 1) return fail(c, GVS_ERR_INJECTED, "injected allocation fault");
    cudaSetDevice(c->device);
    GVS_TRY(alloc_state(c, n));
    const size_t b = n * sizeof(double);
    c->pos_version++;
    GVS_TRY(clear_acc(c));
    c->has_gas = false;
    GVS_CUDA(c, cudaMemsetAsync(c->ptype.ptr, 0, n, c->stream));
    DevBuf *zero[] = {&c->rho, &c->pres, &c->cs, &c->du_dt, &c->div_v, &c->max_mu, &c->dalpha_dt, &c->u, &c->h,
                      &c->alpha};
    for (DevBuf *d : zero) GVS_CUDA(c, cudaMemsetAsync(d->ptr, 0, b, c->stream));
    c->step_counter = 0;
    return GVS_OK;
}

gvs_status gvs_ic_plummer_device(gvs_ctx *c, size_t n, uint64_t seed, double scale_radius, double total_mass) {
    GVS_TRY(check_ctx(c));
    if (n == 0 || !(scale_radius > 0.0) || !(total_mass > 0.0))
        return fail(c, GVS_ERR_INVALID_ARG, "need n >= 1, scale_radius > 0, total_mass > 0");
    if (n > (size_t(1) << 27)) return fail(c, GVS_ERR_INVALID_ARG, "device Plummer ICs: n = %zu above 2^27", n);
    GVS_TRY(device_ics_prepare(c, n));
    GVS_TRY(ic_plummer_device(c, n, seed, scale_radius, total_mass));
    return read_device_errors(c);
}

gvs_status gvs_ic_collision_device(gvs_ctx *c, size_t n, uint64_t seed, double separation) {
    GVS_TRY(check_ctx(c));
    if (n < 2 || !(separation > 0.0)) return fail(c, GVS_ERR_INVALID_ARG, "need n >= 2, separation > 0");
    if (n > (size_t(1) << 27)) return fail(c, GVS_ERR_INVALID_ARG, "device collision ICs: n = %zu above 2^27", n);
    GVS_TRY(device_ics_prepare(c, n));
    GVS_TRY(ic_collision_device(c, n, seed, separation));
    return read_device_errors(c);
}

gvs_status gvs_get_state(gvs_ctx *c, double *x, double *y, double *z, double *vx, double *vy, double *vz, double *ax,
                         double *ay, double *az) {
    GVS_TRY(check_ctx(c));
    const size_t b = c->n * sizeof(double);
    GVS_TRY(download(c, x, c->x, b)); GVS_TRY(download(c, y, c->y, b)); GVS_TRY(download(c, z, c->z, b));
    GVS_TRY(download(c, vx, c->vx, b)); GVS_TRY(download(c, vy, c->vy, b)); GVS_TRY(download(c, vz, c->vz, b));
    GVS_TRY(download(c, ax, c->ax, b)); GVS_TRY(download(c, ay, c->ay, b)); GVS_TRY(download(c, az, c->az, b));
    GVS_CUDA(c, cudaStreamSynchronize(c->stream));
    return read_device_errors(c);
}

gvs_status gvs_set_accelerations(gvs_ctx *c, const double *ax, const double *ay, const double *az) {
    GVS_TRY(check_ctx(c));
    if (!ax || !ay || !az) return fail(c, GVS_ERR_INVALID_ARG, "null acceleration array");
    const size_t b = c->n * sizeof(double);
    GVS_TRY(upload(c, c->ax, ax, b)); GVS_TRY(upload(c, c->ay, ay, b)); GVS_TRY(upload(c, c->az, az, b));
    GVS_CUDA(c, cudaStreamSynchronize(c->stream));
    return GVS_OK;
}

gvs_status gvs_set_gas(gvs_ctx *c, const double *density, const double *pressure, const double *u,
                       const double *du_dt, const double *h, const double *sound_speed, const double *alpha) {
    GVS_TRY(check_ctx(c));
    const size_t b = c->n * sizeof(double);
    if (density) GVS_TRY(upload(c, c->rho, density, b));
    if (pressure) GVS_TRY(upload(c, c->pres, pressure, b));
    if (u) GVS_TRY(upload(c, c->u, u, b));
    if (du_dt) GVS_TRY(upload(c, c->du_dt, du_dt, b));
    if (h) GVS_TRY(upload(c, c->h, h, b));
    if (sound_speed) GVS_TRY(upload(c, c->cs, sound_speed, b));
    if (alpha) GVS_TRY(upload(c, c->alpha, alpha, b));
    GVS_CUDA(c, cudaStreamSynchronize(c->stream));
    return GVS_OK;
}

gvs_status gvs_get_gas(gvs_ctx *c, double *density, double *pressure, double *u, double *du_dt, double *h,
                       double *sound_speed, double *alpha) {
    GVS_TRY(check_ctx(c));
    const size_t b = c->n * sizeof(double);
    GVS_TRY(download(c, density, c->rho, b)); GVS_TRY(download(c, pressure, c->pres, b));
    GVS_TRY(download(c, u, c->u, b)); GVS_TRY(download(c, du_dt, c->du_dt, b));
    GVS_TRY(download(c, h, c->h, b)); GVS_TRY(download(c, sound_speed, c->cs, b));
    GVS_TRY(download(c, alpha, c->alpha, b));
    GVS_CUDA(c, cudaStreamSynchronize(c->stream));
    return read_device_errors(c);
}

static gvs_status check_prec_algo(gvs_ctx *c, int algo, int precision, double eps, double theta) {
    if (algo < GVS_ALGO_NONE || algo > GVS_ALGO_BH) return fail(c, GVS_ERR_INVALID_ARG, "bad algo %d", algo);
    if (precision < GVS_PREC_FP64_EXACT || precision > GVS_PREC_MIXED)
        return fail(c, GVS_ERR_INVALID_ARG, "bad precision %d", precision);
    if (!(eps >= 0.0)) return fail(c, GVS_ERR_INVALID_ARG, "softening must be >= 0 (got %g)", eps);
    if (algo == GVS_ALGO_BH && !(theta >= 0.0)) return fail(c, GVS_ERR_INVALID_ARG, "theta must be >= 0");
    return GVS_OK;
}

static gvs_status gravity_host(gvs_ctx *c, int algo, size_t n, const double *x, const double *y, const double *z,
                               const double *mass, double eps, double theta, int precision, double *ax, double *ay,
                               double *az) {
    GVS_TRY(check_ctx(c));
    if (!x || !y || !z || !mass || !ax || !ay || !az) return fail(c, GVS_ERR_INVALID_ARG, "null array");
    GVS_TRY(check_prec_algo(c, algo, precision, eps, theta));
    if (n > 0xFFFFFFF0ull) return fail(c, GVS_ERR_INVALID_ARG, "n too large");
    if (n == 0) return GVS_OK;
    cudaSetDevice(c->device);
    if (c->n != n) GVS_TRY(alloc_state(c, n));
    const size_t b = n * sizeof(double);
    GVS_TRY(upload(c, c->x, x, b)); GVS_TRY(upload(c, c->y, y, b)); GVS_TRY(upload(c, c->z, z, b));
    GVS_TRY(upload(c, c->m, mass, b));
    c->pos_version++;
    // accumulate semantics: upload the caller's a, add forces, download
    GVS_TRY(upload(c, c->ax, ax, b)); GVS_TRY(upload(c, c->ay, ay, b)); GVS_TRY(upload(c, c->az, az, b));
    GVS_TRY(gravity(c, algo, precision, eps, theta, true));
    GVS_TRY(download(c, ax, c->ax, b)); GVS_TRY(download(c, ay, c->ay, b)); GVS_TRY(download(c, az, c->az, b));
    GVS_CUDA(c, cudaStreamSynchronize(c->stream));
    return read_device_errors(c);
}

gvs_status gvs_gravity_direct(gvs_ctx *c, size_t n, const double *x, const double *y, const double *z,
                              const double *mass, double eps, int precision, double *ax, double *ay, double *az) {
    return gravity_host(c, GVS_ALGO_DIRECT, n, x, y, z, mass, eps, 0.0, precision, ax, ay, az);
}

gvs_status gvs_gravity_bh(gvs_ctx *c, size_t n, const double *x, const double *y, const double *z,
                          const double *mass, double eps, double theta, int precision, double *ax, double *ay,
                          double *az) {
    return gravity_host(c, GVS_ALGO_BH, n, x, y, z, mass, eps, theta, precision, ax, ay, az);
}

gvs_status gvs_tree_export(gvs_ctx *c, size_t cap, size_t *nnodes, uint8_t *level, uint32_t *first, uint32_t *count,
                           uint32_t *skip, double *mass, double *com, uint32_t *order, uint64_t *keys) {
    GVS_TRY(check_ctx(c));
    if (!nnodes) return fail(c, GVS_ERR_INVALID_ARG, "nnodes is NULL");
    if (c->n == 0) return fail(c, GVS_ERR_STATE, "no particles");
    cudaSetDevice(c->device);
    GVS_TRY(tree_export(c, cap, level, first, count, skip, mass, com, order, keys, nnodes));
    return read_device_errors(c);
}

gvs_status gvs_compute_forces(gvs_ctx *c, int algo, int precision, double eps, double theta) {
    GVS_TRY(check_ctx(c));
    GVS_TRY(check_prec_algo(c, algo, precision, eps, theta));
    cudaSetDevice(c->device);
    GVS_TRY(gravity(c, algo, precision, eps, theta, false));
    return GVS_OK;
}

gvs_status gvs_kdk_steps(gvs_ctx *c, int algo, int precision, double eps, double theta, double dt,
                         long long nsteps) {
    GVS_TRY(check_ctx(c));
    GVS_TRY(check_prec_algo(c, algo, precision, eps, theta));
    if (!(dt > 0.0) || nsteps < 0) return fail(c, GVS_ERR_INVALID_ARG, "dt must be > 0 and nsteps >= 0");
    cudaSetDevice(c->device);
    // Systems of at most 32 particles with the exact f64 sum run whole
    // trajectories in one launch (one warp); the result is the same bit for bit.
    if (algo == GVS_ALGO_DIRECT && precision == GVS_PREC_FP64_EXACT && kdk_tiny_eligible(c) && !c->prof.on &&
        c->fault_kind == 0 && nsteps >= 2)
        return kdk_tiny_exact(c, eps, dt, nsteps);
    // Direct-sum steps replay one captured step: the step is a fixed chain of
    // kernels with no host synchronisation (unless kernel timing is on).
    const bool graph = algo == GVS_ALGO_DIRECT && !c->prof.on && c->fault_kind == 0 && !c->sgraph.disabled &&
                       nsteps >= 2;
    long long s = 0;
    if (graph) {
        StepGraphKey key{precision, eps, dt, c->n, c->tune};
        if (!sgraph_valid(c, key)) {
            GVS_TRY(kdk_one(c, algo, precision, eps, theta, dt));  // allocates what the step needs
            ++s;
            GVS_TRY(sgraph_capture(c, key, algo, theta));
        }
        if (c->sgraph.exec) {
            for (; s < nsteps; ++s) {
                GVS_CUDA(c, cudaGraphLaunch(c->sgraph.exec, c->stream));
                c->prof.launches += c->sgraph.launches;
                c->step_counter++;
                c->pos_version++;
            }
            return GVS_OK;
        }
    }
    for (; s < nsteps; ++s) {
        if (nan_fault_due(c)) return fail(c, GVS_ERR_INJECTED, "injected non-finite fault at step %lld", s);
        GVS_TRY(kdk_one(c, algo, precision, eps, theta, dt));
    }
    return GVS_OK;
}

gvs_status gvs_kdk_step_host(gvs_ctx *c, size_t n, double *x, double *y, double *z, double *vx, double *vy,
                             double *vz, double *ax, double *ay, double *az, const double *mass, int algo,
                             int precision, double eps, double theta, double dt) {
    GVS_TRY(check_ctx(c));
    if (!x || !y || !z || !vx || !vy || !vz || !ax || !ay || !az || !mass)
        return fail(c, GVS_ERR_INVALID_ARG, "null array");
    GVS_TRY(check_prec_algo(c, algo, precision, eps, theta));
    if (!(dt > 0.0)) return fail(c, GVS_ERR_INVALID_ARG, "dt must be > 0");
    if (n > 0xFFFFFFF0ull) return fail(c, GVS_ERR_INVALID_ARG, "n too large");
    if (n == 0) return GVS_OK;
    cudaSetDevice(c->device);
    if (c->n != n) GVS_TRY(alloc_state(c, n));
    const size_t b = n * sizeof(double);
    GVS_TRY(upload(c, c->x, x, b)); GVS_TRY(upload(c, c->y, y, b)); GVS_TRY(upload(c, c->z, z, b));
    GVS_TRY(upload(c, c->vx, vx, b)); GVS_TRY(upload(c, c->vy, vy, b)); GVS_TRY(upload(c, c->vz, vz, b));
    GVS_TRY(upload(c, c->ax, ax, b)); GVS_TRY(upload(c, c->ay, ay, b)); GVS_TRY(upload(c, c->az, az, b));
    GVS_TRY(upload(c, c->m, mass, b));
    c->pos_version++;
    if (nan_fault_due(c)) return fail(c, GVS_ERR_INJECTED, "injected non-finite fault");
    GVS_TRY(kdk_one(c, algo, precision, eps, theta, dt));
    GVS_TRY(download(c, x, c->x, b)); GVS_TRY(download(c, y, c->y, b)); GVS_TRY(download(c, z, c->z, b));
    GVS_TRY(download(c, vx, c->vx, b)); GVS_TRY(download(c, vy, c->vy, b)); GVS_TRY(download(c, vz, c->vz, b));
    GVS_TRY(download(c, ax, c->ax, b)); GVS_TRY(download(c, ay, c->ay, b)); GVS_TRY(download(c, az, c->az, b));
    GVS_CUDA(c, cudaStreamSynchronize(c->stream));
    return read_device_errors(c);
}

gvs_status gvs_diagnostics(gvs_ctx *c, double eps, int with_potential, gvs_diag *out) {
    GVS_TRY(check_ctx(c));
    if (!out) return fail(c, GVS_ERR_INVALID_ARG, "out is NULL");
    if (!(eps >= 0.0)) return fail(c, GVS_ERR_INVALID_ARG, "softening must be >= 0");
    cudaSetDevice(c->device);
    GVS_TRY(diagnostics(c, eps, with_potential, out));
    return read_device_errors(c);
}

gvs_status gvs_direct_subset(gvs_ctx *c, int precision, double eps, const int64_t *idx, size_t nidx, double *oax,
                             double *oay, double *oaz) {
    GVS_TRY(check_ctx(c));
    if (!idx || !oax || !oay || !oaz) return fail(c, GVS_ERR_INVALID_ARG, "null array");
    for (size_t k = 0; k < nidx; ++k)
        if (idx[k] < 0 || (size_t)idx[k] >= c->n) return fail(c, GVS_ERR_INVALID_ARG, "target index out of range");
    if (nidx == 0) return GVS_OK;
    cudaSetDevice(c->device);
    GVS_CUDA(c, ensure(c, c->scratch_a, nidx * sizeof(int64_t)));
    GVS_CUDA(c, ensure(c, c->scratch_b, 3 * nidx * sizeof(double)));
    GVS_CUDA(c, cudaMemcpyAsync(c->scratch_a.ptr, idx, nidx * sizeof(int64_t), cudaMemcpyHostToDevice, c->stream));
    GVS_TRY(direct_forces_subset(c, precision, eps, as<int64_t>(c->scratch_a), nidx, as<double>(c->scratch_b)));
    double *d = as<double>(c->scratch_b);
    GVS_CUDA(c, cudaMemcpyAsync(oax, d, nidx * 8, cudaMemcpyDeviceToHost, c->stream));
    GVS_CUDA(c, cudaMemcpyAsync(oay, d + nidx, nidx * 8, cudaMemcpyDeviceToHost, c->stream));
    GVS_CUDA(c, cudaMemcpyAsync(oaz, d + 2 * nidx, nidx * 8, cudaMemcpyDeviceToHost, c->stream));
    GVS_CUDA(c, cudaStreamSynchronize(c->stream));
    return read_device_errors(c);
}

gvs_status gvs_autotune_direct(gvs_ctx *c, int precision, double eps, int *nthreads, int *ipt, double *ms) {
    GVS_TRY(check_ctx(c));
    if (precision != GVS_PREC_MIXED && precision != GVS_PREC_FP32)
        return fail(c, GVS_ERR_INVALID_ARG, "autotune covers the f32 pair kernel (FP32 / MIXED)");
    if (!(eps >= 0.0)) return fail(c, GVS_ERR_INVALID_ARG, "softening must be >= 0");
    if (c->n == 0) return fail(c, GVS_ERR_STATE, "no particles");
    cudaSetDevice(c->device);
    GVS_TRY(autotune_direct(c, precision, eps, nthreads, ipt, ms));
    return read_device_errors(c);
}

gvs_status gvs_set_direct_shape(gvs_ctx *c, int nthreads, int ipt, int min_blocks, int unroll) {
    GVS_TRY(check_ctx(c));
    if (!direct_shape_compiled(nthreads, ipt, min_blocks, unroll))
        return fail(c, GVS_ERR_INVALID_ARG, "pair-kernel shape (%d, %d, %d, %d) is not compiled", nthreads, ipt,
                    min_blocks, unroll);
    set_direct_shape(c, nthreads, ipt, min_blocks, unroll);
    return GVS_OK;
}

gvs_status gvs_set_bh_walk(gvs_ctx *c, int group_size, int budget) {
    GVS_TRY(check_ctx(c));
    if (group_size != -1 && group_size != 0 && group_size != 32 && group_size != 64 && group_size != 128)
        return fail(c, GVS_ERR_INVALID_ARG,
                    "BH walk group size must be -1 (automatic), 0 (per-particle), 32, 64 or 128, got %d",
                    group_size);
    if (budget < 0) return fail(c, GVS_ERR_INVALID_ARG, "BH group-walk budget must be >= 0, got %d", budget);
    c->bh_group = group_size;
    c->bh_budget = budget > 0 ? budget : 1024;
    return GVS_OK;
}

gvs_status gvs_autotune_report(gvs_ctx *c, int cap, int *count, int *nthreads, int *ipt, int *min_blocks,
                               int *unroll, double *ms) {
    GVS_TRY(check_ctx(c));
    if (!count) return fail(c, GVS_ERR_INVALID_ARG, "count is NULL");
    *count = (int)c->tune_report.size();
    if (cap < *count) return GVS_OK;
    for (int k = 0; k < *count; ++k) {
        const auto &e = c->tune_report[(size_t)k];
        if (nthreads) nthreads[k] = e.first.nthreads;
        if (ipt) ipt[k] = e.first.ipt;
        if (min_blocks) min_blocks[k] = e.first.minb;
        if (unroll) unroll[k] = e.first.unroll;
        if (ms) ms[k] = e.second;
    }
    return GVS_OK;
}

// ---- SPH ---------------------------------------------------------------------------

gvs_status gvs_sph_params_default(gvs_sph_params *p) {
    if (!p) return GVS_ERR_INVALID_ARG;
    p->gamma = 5.0 / 3.0;   // solver.rs:43
    p->eta = 1.2;           // solver.rs:44
    p->cfl_factor = 0.3;    // solver.rs:46
    p->force_factor = 0.25; // solver.rs:47
    p->h_max = INFINITY;    // solver.rs:48
    p->beta_visc = 2.0;     // forces.rs:34
    p->alpha_min = 0.1;     // forces.rs:35
    p->alpha_max = 2.0;     // forces.rs:36
    p->alpha_cond = 1.0;    // forces.rs:37
    p->sigma_visc = 0.1;    // forces.rs:38
    p->precision = GVS_PREC_FP64_EXACT;
    return GVS_OK;
}

static gvs_status check_sph(gvs_ctx *c, const gvs_sph_params *p) {
    GVS_TRY(check_ctx(c));
    if (!p) return fail(c, GVS_ERR_INVALID_ARG, "SPH parameters are NULL");
    if (!(p->gamma > 1.0) || !(p->eta > 0.0) || !(p->cfl_factor > 0.0) || !(p->force_factor > 0.0) ||
        !(p->alpha_min <= p->alpha_max))
        return fail(c, GVS_ERR_INVALID_ARG, "invalid SPH parameters");
    if (p->precision != GVS_PREC_FP64_EXACT && p->precision != GVS_PREC_FP64 && p->precision != GVS_PREC_MIXED)
        return fail(c, GVS_ERR_INVALID_ARG, "SPH precision must be FP64_EXACT, FP64 or MIXED");
    if (!c->has_gas) return fail(c, GVS_ERR_STATE, "no gas particles uploaded (ptype/u/h/alpha were NULL)");
    cudaSetDevice(c->device);
    return GVS_OK;
}

gvs_status gvs_sph_compute(gvs_ctx *c, const gvs_sph_params *p, double *omega, double *div_v, double *max_mu,
                           double *dalpha_dt) {
    GVS_TRY(check_sph(c, p));
    GVS_TRY(sph_compute(c, p));
    const size_t b = c->n * sizeof(double);
    GVS_TRY(download(c, omega, c->omega, b)); GVS_TRY(download(c, div_v, c->div_v, b));
    GVS_TRY(download(c, max_mu, c->max_mu, b)); GVS_TRY(download(c, dalpha_dt, c->dalpha_dt, b));
    GVS_CUDA(c, cudaStreamSynchronize(c->stream));
    return read_device_errors(c);
}

gvs_status gvs_sph_timestep(gvs_ctx *c, const gvs_sph_params *p, double *dt) {
    GVS_TRY(check_sph(c, p));
    if (!dt) return fail(c, GVS_ERR_INVALID_ARG, "dt is NULL");
    GVS_TRY(sph_timestep(c, p, dt));
    return read_device_errors(c);
}

gvs_status gvs_sph_step(gvs_ctx *c, const gvs_sph_params *p, int algo, int precision, double eps, double theta,
                        double dt, double *dt_next) {
    GVS_TRY(check_sph(c, p));
    GVS_TRY(check_prec_algo(c, algo, precision, eps, theta));
    if (!(dt > 0.0) || !dt_next) return fail(c, GVS_ERR_INVALID_ARG, "dt must be > 0 and dt_next non-NULL");
    if (nan_fault_due(c)) return fail(c, GVS_ERR_INJECTED, "injected non-finite fault");
    GVS_TRY(sph_step(c, p, algo, precision, eps, theta, dt, dt_next));
    return read_device_errors(c);
}

gvs_status gvs_sph_neighbors(gvs_ctx *c, size_t cap, size_t *total, uint32_t *start, uint32_t *count,
                             uint32_t *idx) {
    GVS_TRY(check_ctx(c));
    if (!total) return fail(c, GVS_ERR_INVALID_ARG, "total is NULL");
    cudaSetDevice(c->device);
    return sph_neighbors_export(c, cap, start, count, idx, total);
}

// ---- profiling -----------------------------------------------------------------

struct EventSlots {
    cudaEvent_t ev[16] = {};
};

gvs_status gvs_profile_enable(gvs_ctx *c, int on) {
    GVS_TRY(check_ctx(c));
    GVS_TRY(prof_settle(c));  // spans of the previous profile go to the counters reset below
    c->prof.on = on != 0;
    c->prof.force_ms = 0.0;
    c->prof.force_launches = 0;
    c->prof.launches = 0;
    c->prof.force_flops = 0.0;
    c->prof.force_bytes = 0.0;
    c->prof.tile_visits = 0.0;
    c->prof.vjp_ms = 0.0;
    c->prof.vjp_launches = 0;
    GVS_CUDA(c, cudaMemsetAsync(err_ptr(c) + EW_NEAR_TILES, 0, (EW_PROFILE_END - EW_NEAR_TILES) * sizeof(unsigned),
                                c->stream));
    return GVS_OK;
}

gvs_status gvs_profile_read(gvs_ctx *c, gvs_profile *out) {
    GVS_TRY(check_ctx(c));
    if (!out) return fail(c, GVS_ERR_INVALID_ARG, "out is NULL");
    GVS_CUDA(c, cudaStreamSynchronize(c->stream));
    GVS_TRY(prof_settle(c));
    out->force_ms = c->prof.force_ms;
    out->force_launches = c->prof.force_launches;
    out->launches = c->prof.launches;
    out->force_flops = c->prof.force_flops;
    out->force_bytes = c->prof.force_bytes;
    out->vjp_ms = c->prof.vjp_ms;
    out->vjp_launches = c->prof.vjp_launches;
    unsigned long long nearc = 0;
    GVS_CUDA(c, cudaMemcpy(&nearc, err_ptr(c) + EW_NEAR_TILES, sizeof nearc, cudaMemcpyDeviceToHost));
    out->near_tile_visits = (double)nearc;
    out->tile_visits = c->prof.tile_visits;
    unsigned redo = 0;
    GVS_CUDA(c, cudaMemcpy(&redo, err_ptr(c) + EW_SPH_REDO, sizeof redo, cudaMemcpyDeviceToHost));
    out->sph_f64_redo = redo;
    unsigned words[4] = {0, 0, 0, 0};  // group walk: iterations (u64), groups, fallbacks
    GVS_CUDA(c, cudaMemcpy(words, err_ptr(c) + EW_BH_ITERS, sizeof words, cudaMemcpyDeviceToHost));
    out->bh_group_iterations = (long long)((unsigned long long)words[0] | ((unsigned long long)words[1] << 32));
    out->bh_groups = words[2];
    out->bh_group_fallbacks = words[3];
    unsigned long long pairs = 0;
    GVS_CUDA(c, cudaMemcpy(&pairs, err_ptr(c) + EW_BH_TERMS, sizeof pairs, cudaMemcpyDeviceToHost));
    out->bh_group_interactions = (long long)pairs;
    unsigned long long wt = 0;
    GVS_CUDA(c, cudaMemcpy(&wt, err_ptr(c) + EW_WALK_TERMS, sizeof wt, cudaMemcpyDeviceToHost));
    out->bh_walk_terms = (long long)wt;
    return GVS_OK;
}

gvs_status gvs_stream(gvs_ctx *c, void **stream) {
    GVS_TRY(check_ctx(c));
    if (!stream) return fail(c, GVS_ERR_INVALID_ARG, "stream is NULL");
    *stream = static_cast<void *>(c->stream);
    return GVS_OK;
}

static std::vector<std::pair<const gvs_ctx *, EventSlots>> g_slots;

static cudaEvent_t *slots_for(gvs_ctx *c) {
    for (auto &p : g_slots)
        if (p.first == c) return p.second.ev;
    g_slots.push_back({c, EventSlots()});
    return g_slots.back().second.ev;
}

gvs_status gvs_event_record(gvs_ctx *c, int slot) {
    GVS_TRY(check_ctx(c));
    if (slot < 0 || slot >= 16) return fail(c, GVS_ERR_INVALID_ARG, "event slot out of range");
    cudaEvent_t *ev = slots_for(c);
    if (!ev[slot]) GVS_CUDA(c, cudaEventCreate(&ev[slot]));
    GVS_CUDA(c, cudaEventRecord(ev[slot], c->stream));
    return GVS_OK;
}

gvs_status gvs_event_elapsed(gvs_ctx *c, int a, int b, float *ms) {
    GVS_TRY(check_ctx(c));
    if (a < 0 || a >= 16 || b < 0 || b >= 16 || !ms) return fail(c, GVS_ERR_INVALID_ARG, "bad event slots");
    cudaEvent_t *ev = slots_for(c);
    if (!ev[a] || !ev[b]) return fail(c, GVS_ERR_STATE, "event slot not recorded");
    GVS_CUDA(c, cudaEventSynchronize(ev[b]));
    GVS_CUDA(c, cudaEventElapsedTime(ms, ev[a], ev[b]));
    return GVS_OK;
}

gvs_status gvs_l2_flush(gvs_ctx *c) {
    GVS_TRY(check_ctx(c));
    const size_t bytes = 512ull << 20;  // 4x the 129 MB L2
    GVS_CUDA(c, ensure(c, c->l2_flush, bytes));
    GVS_CUDA(c, cudaMemsetAsync(c->l2_flush.ptr, (int)(c->step_counter & 0xFF), bytes, c->stream));
    return GVS_OK;
}

}  // extern "C"

// ---- FP32 throughput probe ----------------------------------------------------------
namespace {
constexpr int PEAK_ITERS = 4096;

__global__ void k_fp32_peak_scalar(float *out, float a, float b) {
    float r[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) r[k] = (float)(threadIdx.x + k);
    for (int it = 0; it < PEAK_ITERS; ++it)
#pragma unroll
        for (int k = 0; k < 16; ++k) r[k] = fmaf(r[k], a, b);
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 16; ++k) s += r[k];
    if (s == 12345.678f) out[0] = s;
}

__global__ void k_fp32_peak_packed(float *out, float a, float b) {
    unsigned long long r[8], av, bv;
    asm("mov.b64 %0, {%1, %1};" : "=l"(av) : "f"(a));
    asm("mov.b64 %0, {%1, %1};" : "=l"(bv) : "f"(b));
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        float x = (float)(threadIdx.x + k), y = x + 0.5f;
        asm("mov.b64 %0, {%1, %2};" : "=l"(r[k]) : "f"(x), "f"(y));
    }
    for (int it = 0; it < PEAK_ITERS; ++it)
#pragma unroll
        for (int k = 0; k < 8; ++k) asm volatile("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(r[k]) : "l"(av), "l"(bv));
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        float x, y;
        asm("mov.b64 {%0, %1}, %2;" : "=f"(x), "=f"(y) : "l"(r[k]));
        s += x + y;
    }
    if (s == 12345.678f) out[0] = s;
}

// Packed and scalar chains interleaved one to one: on sm_10x the packed FMA runs
// on the heavy FP32 pipe and a scalar FMA can go to the lite pipe in the same
// cycles, so this stream can exceed either pure form.  The scalar chains use
// distinct multipliers so they cannot be merged into packed instructions.
__global__ void k_fp32_peak_mixed(float *out, float a, float b) {
    unsigned long long r[8], av, bv;
    float s_[8], m_[8];
    asm("mov.b64 %0, {%1, %1};" : "=l"(av) : "f"(a));
    asm("mov.b64 %0, {%1, %1};" : "=l"(bv) : "f"(b));
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        float x = (float)(threadIdx.x + k), y = x + 0.5f;
        asm("mov.b64 %0, {%1, %2};" : "=l"(r[k]) : "f"(x), "f"(y));
        s_[k] = x + 0.25f;
        m_[k] = a - 1e-4f * (float)k;
    }
    for (int it = 0; it < PEAK_ITERS; ++it)
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            asm volatile("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(r[k]) : "l"(av), "l"(bv));
            asm volatile("fma.rn.f32 %0, %0, %1, %2;" : "+f"(s_[k]) : "f"(m_[k]), "f"(b));
        }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        float x, y;
        asm("mov.b64 {%0, %1}, %2;" : "=f"(x), "=f"(y) : "l"(r[k]));
        s += x + y + s_[k];
    }
    if (s == 12345.678f) out[0] = s;
}
}  // namespace

// Self-test of the bounded-wait path: one thread waits on an mbarrier that
// nothing arrives at, for `cap` polls, then sets the timeout flag and returns.
__global__ void k_wait_probe(unsigned *err, unsigned cap) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x != 0) return;
    mbar_init(&bar, 1);
    fence_mbar_init();
    mbar_wait_bounded(&bar, 0u, err, cap);
}

extern "C" gvs_status gvs_check_bounded_wait(gvs_ctx *c, unsigned polls) {
    GVS_TRY(check_ctx(c));
    if (polls == 0 || polls > (1u << 20)) return fail(c, GVS_ERR_INVALID_ARG, "polls must be in [1, 2^20]");
    cudaSetDevice(c->device);
    k_wait_probe<<<1, 32, 0, c->stream>>>(err_ptr(c), polls);
    c->prof.launches += 1;
    GVS_TRY(check_launch(c, "bounded-wait probe"));
    return read_device_errors(c);  // GVS_ERR_TIMEOUT expected; the word is cleared
}

extern "C" gvs_status gvs_measure_fp32_peak(gvs_ctx *c, double *tflops) {
    GVS_TRY(check_ctx(c));
    if (!tflops) return fail(c, GVS_ERR_INVALID_ARG, "tflops is NULL");
    cudaSetDevice(c->device);
    GVS_CUDA(c, ensure(c, c->scratch_b, 64));
    const int blocks = c->num_sms * 8, threads = 256;
    double best = 0.0;
    for (int variant = 0; variant < 3; ++variant) {
        for (int rep = 0; rep < 3; ++rep) {
            GVS_CUDA(c, cudaEventRecord(c->prof.ev[0], c->stream));
            if (variant == 0)
                k_fp32_peak_scalar<<<blocks, threads, 0, c->stream>>>(as<float>(c->scratch_b), 0.999f, 0.001f);
            else if (variant == 1)
                k_fp32_peak_packed<<<blocks, threads, 0, c->stream>>>(as<float>(c->scratch_b), 0.999f, 0.001f);
            else
                k_fp32_peak_mixed<<<blocks, threads, 0, c->stream>>>(as<float>(c->scratch_b), 0.999f, 0.001f);
            GVS_CUDA(c, cudaEventRecord(c->prof.ev[1], c->stream));
            GVS_TRY(check_launch(c, "fp32 peak probe"));
            GVS_CUDA(c, cudaEventSynchronize(c->prof.ev[1]));
            float ms = 0.f;
            GVS_CUDA(c, cudaEventElapsedTime(&ms, c->prof.ev[0], c->prof.ev[1]));
            // lane FMAs per thread per iteration: 16 scalar, 8 x 2 packed, 8 x 2 + 8 mixed
            const double fmas = variant == 2 ? 24.0 : 16.0;
            const double flops = 2.0 * fmas * PEAK_ITERS * (double)blocks * threads;
            const double tf = ms > 0.f ? flops / (ms * 1e-3) / 1e12 : 0.0;
            c->peak_by_variant[variant] = std::max(rep == 0 ? 0.0 : c->peak_by_variant[variant], tf);
            best = std::max(best, tf);
        }
    }
    *tflops = best;
    return GVS_OK;
}

extern "C" gvs_status gvs_fp32_peak_variants(gvs_ctx *c, double *scalar, double *packed, double *mixed) {
    GVS_TRY(check_ctx(c));
    if (scalar) *scalar = c->peak_by_variant[0];
    if (packed) *packed = c->peak_by_variant[1];
    if (mixed) *mixed = c->peak_by_variant[2];
    return GVS_OK;
}
