// lsg_solvers.cu — host side of liblsg: work-array cache, the solver loops
// and the native C ABI declared in include/lsg.h.
//
// The loops restate the control flow of the reference solvers with device-
// resident state:
//   lsg_aar   MPI_REAL/AAR.c:37-177       lsg_pgr / lsg_pl2r  PGR.c:35-173, PL2R.c:35-172
//   lsg_cg    MPI_REAL/CG.c:33-175        lsg_aar_mixed       FP64 refinement around FP32 AAR
// Iteration numbering, history column selection ((iter-2)%m for AAR written
// one launch early as (iter-1)%m; (iter-2+m)%m for PGR/PL2R), the residual
// check only at extrapolation steps and the reported count follow the
// reference.  Convergence is decided on the device (DevCtrl::done); the host
// enqueues `check_every` extrapolation cycles ahead and reads the flag
// through pinned memory, so the GPU never idles waiting for the host.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdarg>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <type_traits>
#include <vector>

#include "lsg_internal.cuh"
#include "lsg_host.h"

namespace lsg {

// ---------------------------------------------------------------- errors

static thread_local int t_last_status = LSG_OK;
static thread_local char t_last_error[512] = "";

int set_error(int status, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_last_error, sizeof(t_last_error), fmt, ap);
    va_end(ap);
    t_last_status = status;
    return status;
}

void set_last_status(int st) { t_last_status = st; if (st == LSG_OK) t_last_error[0] = 0; }
int last_status() { return t_last_status; }
const char *last_error() { return t_last_error; }

#define LSG_CUDA(call)                                                                       \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return cudaGetLastError(), /* clear it for later launches */                     \
                   set_error(e_ == cudaErrorMemoryAllocation ? LSG_NO_MEMORY : LSG_CUDA_ERROR, \
                             "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

// ---------------------------------------------------------------- FP64 stencil arithmetic

// 0: double-float sums on the FP32 pipe (default); 1: FP64 arithmetic.
static std::atomic<int> g_fp64_arith{[] {
    const char *e = getenv("LSG_FP64_ARITH");
    return (e && e[0] == '1') ? 1 : 0;
}()};
int fp64_exact() { return g_fp64_arith.load(std::memory_order_relaxed); }

// Form of the FP32 AAR's Richardson passes: 0 = the residual ring where it
// applies, 1 = the lean form (three residual buffers, H and DF stored),
// 2 = the x-carrying recurrence.  LSG_AAR_FORM sets the initial value.
static std::atomic<int> g_aar_form{[] {
    const char *e = getenv("LSG_AAR_FORM");
    const int v = e ? atoi(e) : 0;
    return v >= 0 && v <= 2 ? v : 0;
}()};
int aar_form() { return g_aar_form.load(std::memory_order_relaxed); }
int fp64_exact_for(double tol) { return (fp64_exact() || tol < kDfMinTol) ? 1 : 0; }

// ---------------------------------------------------------------- device info

int sm_count() {
    static std::mutex mu;
    static std::map<int, int> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> g(mu);
    auto it = cache.find(dev);
    if (it != cache.end()) return it->second;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 152;
    cache[dev] = sms;
    return sms;
}

// Resident stencil blocks on the device (one wave).
template <typename T>
static int stencil_slots(int sms) {
    static int bpsm = 0;  // per vector type, resolved on first use
    if (bpsm == 0) bpsm = Kernels<T>::stencil_blocks_per_sm();
    return sms * bpsm;
}

// ---------------------------------------------------------------- work arrays

// One allocation per (device, element size, grid points, history depth):
//   xalt, r0, r1, rs             four vectors (ping-pong partners; rs: the
//                                cycle-start residual of the lean FP32 AAR)
//   dx[m], df[m]                 the history, column j at offset j*n
//   ring[m + 1]                  FP32 keys with m <= 8: the residual ring of the AAR
//   partials                     per-block FP64 sums
//   ctrl                         DevCtrl
// The mixed solver adds r32 / e32 (float) on an FP64 key.
struct Workspace {
    std::mutex mu;
    int device = 0;
    size_t es = 0;
    long long n = 0;
    int m = 0;
    char *base = nullptr;
    void *xalt = nullptr, *r0 = nullptr, *r1 = nullptr, *rs = nullptr, *dx = nullptr, *df = nullptr;
    void *ring = nullptr;     // FP32 keys: the residual ring, m + 1 slots ring_ss elements apart
    long long ring_ss = 0;
    float *r32 = nullptr, *e32 = nullptr;
    double *partials = nullptr;
    long long partials_cap = 0;
    DevCtrl *ctrl = nullptr;
    DevCtrl *hctrl = nullptr;  // pinned, two slots
    cudaEvent_t ev[2] = {nullptr, nullptr};
    ~Workspace() {
        if (base) cudaFree(base);
        if (hctrl) cudaFreeHost(hctrl);
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
    }
};

static std::mutex g_ws_mu;
static std::map<std::tuple<int, size_t, long long, int, int>, std::unique_ptr<Workspace>> g_ws;

static size_t align_up(size_t v) { return (v + 255) & ~(size_t)255; }

long long partials_needed(long long n, int m, int sms) {
    long long cap = 0;
    // stencil launches (worst case over both tile shapes and lz >= 1 planes)
    const long long bx = (long long)sms * 8;
    cap = std::max(cap, bx);
    // grid-stride reductions use <= 4*sms blocks; a Gram launch (<= 8 resident
    // 256-thread blocks per SM) writes up to m*m+m values per block
    cap = std::max(cap, (long long)8 * sms * (m * m + m));
    (void)n;
    return cap;
}

// Fetches (creating on first use) the work arrays; returned locked.
static int get_workspace(size_t es, long long n, int m, bool mixed, const Geom &g,
                         Workspace **out, std::unique_lock<std::mutex> *lock) {
    int dev = 0;
    cudaGetDevice(&dev);
    const int sms = sm_count();
    Workspace *ws;
    {
        std::lock_guard<std::mutex> gl(g_ws_mu);
        auto key = std::make_tuple(dev, es, n, m, mixed ? 1 : 0);
        auto &slot = g_ws[key];
        if (!slot) slot.reset(new Workspace());
        ws = slot.get();
    }
    *lock = std::unique_lock<std::mutex>(ws->mu);
    if (ws->base) { *out = ws; return LSG_OK; }
    // Partials: stencil grids for this geometry plus the reduction grids.
    long long cap = partials_needed(n, m, sms);
    cap = std::max(cap, stencil_blocks<double>(g, choose_lz<double>(g, stencil_slots<double>(sms))));
    cap = std::max(cap, stencil_blocks<float>(g, choose_lz<float>(g, stencil_slots<float>(sms))));
    cap = std::max(cap, Kernels<float>::paired_plan(g, nullptr));
    if (es == sizeof(cplx<double>) || es == sizeof(cplx<float>)) {  // complex: (re, im) partials
        cap = std::max(cap, 2 * stencil_blocks<cplx<double>>(g, choose_lz<cplx<double>>(g, stencil_slots<cplx<double>>(sms))));
        cap = std::max(cap, 2 * stencil_blocks<cplx<float>>(g, choose_lz<cplx<float>>(g, stencil_slots<cplx<float>>(sms))));
    }
    const size_t vec = align_up((size_t)n * es);
    size_t bytes = 0;
    const size_t o_xalt = bytes; bytes += vec;
    const size_t o_r0 = bytes; bytes += vec;
    const size_t o_r1 = bytes; bytes += vec;
    const size_t o_rs = bytes; bytes += vec;
    const size_t o_dx = bytes; bytes += align_up((size_t)n * es * (size_t)m);
    const size_t o_df = bytes; bytes += align_up((size_t)n * es * (size_t)m);
    size_t o_ring = 0;
    const bool with_ring = es == 4 && !mixed && m >= 1 && m <= kRingMaxM;
    if (with_ring) { o_ring = bytes; bytes += vec * (size_t)(m + 1); }
    size_t o_r32 = 0, o_e32 = 0;
    if (mixed) {  // FP32 (or complex64) correction, half the outer element size
        o_r32 = bytes; bytes += align_up((size_t)n * (es / 2));
        o_e32 = bytes; bytes += align_up((size_t)n * (es / 2));
    }
    const size_t o_part = bytes; bytes += align_up((size_t)cap * 8);
    const size_t o_ctrl = bytes; bytes += align_up(sizeof(DevCtrl));
    char *base = nullptr;
    cudaError_t e = cudaMalloc(&base, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(LSG_NO_MEMORY, "cudaMalloc of %zu bytes for work arrays failed: %s", bytes,
                         cudaGetErrorString(e));
    }
    DevCtrl *h = nullptr;
    e = cudaMallocHost(&h, 2 * sizeof(DevCtrl));
    if (e != cudaSuccess) {
        cudaFree(base);
        return set_error(LSG_NO_MEMORY, "cudaMallocHost failed: %s", cudaGetErrorString(e));
    }
    ws->device = dev;
    ws->es = es;
    ws->n = n;
    ws->m = m;
    ws->base = base;
    ws->xalt = base + o_xalt;
    ws->r0 = base + o_r0;
    ws->r1 = base + o_r1;
    ws->rs = base + o_rs;
    ws->dx = base + o_dx;
    ws->df = base + o_df;
    if (with_ring) {
        ws->ring = base + o_ring;
        ws->ring_ss = (long long)(vec / es);
    }
    if (mixed) {
        ws->r32 = (float *)(base + o_r32);
        ws->e32 = (float *)(base + o_e32);
    }
    ws->partials = (double *)(base + o_part);
    ws->partials_cap = cap;
    ws->ctrl = (DevCtrl *)(base + o_ctrl);
    ws->hctrl = h;
    cudaEventCreateWithFlags(&ws->ev[0], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&ws->ev[1], cudaEventDisableTiming);
    *out = ws;
    return LSG_OK;
}

static void release_csr_extras();

int release_workspaces() {
    cudaDeviceSynchronize();
    {
        std::lock_guard<std::mutex> gl(g_ws_mu);
        g_ws.clear();
    }
    release_csr_extras();
    release_icc();
    release_gmres_workspaces();
    return release_batch_workspaces();
}

// ---------------------------------------------------------------- operator

// system.c:480-498: c_0 = -sum_p 2/p^2; c_p = 2 (-1)^(p+1) (R!/(R-p)!) / ((R+p)!/R!) / p^2,
// with the same product order so the values match the reference bit for bit.
int lap_coefficient(int radius, double *c) {
    c[0] = 0.0;
    for (int p = 1; p <= radius; p++) c[0] += -(2.0 / (p * p));
    for (int p = 1; p <= radius; p++) {
        double nr = 1, dr = 1;
        for (int i = radius - p + 1; i <= radius; i++) nr *= i;
        for (int i = radius + 1; i <= radius + p; i++) dr *= i;
        c[p] = 2 * std::pow(-1.0, p + 1) * (nr / dr) / (p * p);
    }
    for (int p = radius + 1; p <= LSG_MAX_RADIUS; p++) c[p] = 0.0;
    return LSG_OK;
}

int check_operator(const lsg_operator *op) {
    if (!op) return set_error(LSG_BAD_ARG, "operator is NULL");
    for (int d = 0; d < 3; d++)
        if (op->n[d] < 1) return set_error(LSG_BAD_ARG, "grid size n[%d] = %d < 1", d, op->n[d]);
    if ((long long)op->n[0] * op->n[1] * op->n[2] > 4294967295LL)
        return set_error(LSG_BAD_ARG, "grid of %lld points exceeds 2^32-1",
                         (long long)op->n[0] * op->n[1] * op->n[2]);
    if (op->radius < 1 || op->radius > LSG_MAX_RADIUS)
        return set_error(LSG_BAD_ARG, "radius %d outside 1..%d", op->radius, LSG_MAX_RADIUS);
    return LSG_OK;
}

double jacobi_diag(const lsg_operator *op) { return op->a * (3 * op->coeff[0]) + op->sigma; }

int check_params(const lsg_params *prm, bool history) {
    if (!prm) return set_error(LSG_BAD_ARG, "params is NULL");
    if (prm->max_iter < 0) return set_error(LSG_BAD_ARG, "max_iter %d < 0", prm->max_iter);
    if (!(prm->tol >= 0)) return set_error(LSG_BAD_ARG, "tol must be >= 0");
    if (history) {
        if (prm->m < 1 || prm->m > LSG_MAX_M)
            return set_error(LSG_BAD_ARG, "history depth m = %d outside 1..%d", prm->m, LSG_MAX_M);
        if (prm->p < 1) return set_error(LSG_BAD_ARG, "period p = %d < 1", prm->p);
    }
    return LSG_OK;
}

// ---------------------------------------------------------------- solve driver helpers

// ---------------------------------------------------------------- profiling

// Per-class device time from CUDA events recorded on the solve's stream
// around each launch (lsg_profile).  Events come from a pool reused across
// solves; totals are folded in after the solve's final stream synchronize.
static std::mutex g_prof_mu;
static bool g_prof_on = false;
static lsg_kernel_stats g_prof;
static std::vector<cudaEvent_t> g_ev_pool;

struct ProfRec {
    int cls;
    cudaEvent_t a, b;
};

struct Run {
    cudaStream_t s;
    int sms;
    long long launches = 0;
    bool prof = false;
    size_t ev_used = 0;
    std::vector<ProfRec> recs;
    Run(cudaStream_t s_, int sms_) : s(s_), sms(sms_) {
        std::lock_guard<std::mutex> g(g_prof_mu);
        prof = g_prof_on;
    }
    cudaEvent_t event() {
        // only the thread holding the profile flag draws events; the pool is
        // guarded by g_prof_mu
        std::lock_guard<std::mutex> g(g_prof_mu);
        if (ev_used == g_ev_pool.size()) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
            g_ev_pool.push_back(e);
        }
        return g_ev_pool[ev_used++];
    }
    // Accumulates recorded launch times; call after the stream is idle.
    void flush() {
        if (!prof) return;
        std::lock_guard<std::mutex> g(g_prof_mu);
        for (const ProfRec &r : recs) {
            float ms = 0.f;
            if (r.a && r.b && cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
                g_prof.launches[r.cls]++;
                g_prof.ms[r.cls] += ms;
            }
        }
        recs.clear();
        ev_used = 0;
    }
};

// Readers of the per-translation-unit bounds words (bounds-checked build).
std::vector<unsigned long long (*)()> &bounds_readers() {
    static std::vector<unsigned long long (*)()> v;
    return v;
}
int register_bounds_reader(unsigned long long (*read)()) {
    bounds_readers().push_back(read);
    return 0;
}

// Tracing: with LSG_NVTX=1 in the environment every solve and every kernel
// launch sits in an NVTX range (the solver's name; the kernel class), for
// profiler timelines and `ncu --nvtx --nvtx-include "<class>/"` filters.
static bool trace_on() {
    static const bool on = [] {
        const char *e = getenv("LSG_NVTX");
        return e && e[0] == '1';
    }();
    return on;
}
struct TraceRange {
    bool on;
    explicit TraceRange(const char *name) : on(trace_on()) {
        if (on) nvtxRangePushA(name);
    }
    ~TraceRange() {
        if (on) nvtxRangePop();
    }
};
static const char *const kClassNames[LSG_K_CLASSES] = {"richardson", "residual", "gram",   "update",
                                                       "small",      "cg",       "refine", "precond"};

#define LSG_KC(cls, call)                                                                    \
    do {                                                                                     \
        TraceRange tr_(kClassNames[cls]);                                                    \
        cudaEvent_t ea_ = nullptr;                                                           \
        if (R.prof && (ea_ = R.event()) != nullptr) cudaEventRecord(ea_, R.s);               \
        cudaError_t e_ = (call);                                                             \
        R.launches++;                                                                        \
        if (e_ != cudaSuccess)                                                               \
            return cudaGetLastError(),                                                       \
                   set_error(LSG_CUDA_ERROR, "launch %s: %s", #call, cudaGetErrorString(e_)); \
        if (ea_) {                                                                           \
            cudaEvent_t eb_ = R.event();                                                     \
            if (eb_) { cudaEventRecord(eb_, R.s); R.recs.push_back({cls, ea_, eb_}); }       \
        }                                                                                    \
    } while (0)

static int reduce_blocks(long long n, int sms) {
    long long b = (n + 255) / 256;
    return (int)std::max<long long>(1, std::min<long long>(b, 4LL * sms));
}

// Initial DevCtrl contents.  relres starts at tol + 1 as in AAR.c:76, so a
// solve stopped before its first check reports the reference's value.
DevCtrl ctrl_init(double tol, int stall_limit) {
    DevCtrl c;
    memset(&c, 0, sizeof(c));
    c.relres = tol + 1.0;
    c.best = INFINITY;
    c.stall_limit = stall_limit;
    return c;
}

// Enqueues cycles through `enqueue_iter(it)` with a pipelined convergence read
// every `per_check` checkpoints; `is_check(it)` marks iterations that end with
// a device-side convergence test.  Returns after the solve stopped.
template <class Enq, class IsCheck>
static int pipelined_loop(Run &R, Workspace *ws, int first_iter, int max_iter, int per_check,
                          Enq &&enqueue_iter, IsCheck &&is_check) {
    int it = first_iter;
    int batch = 0;
    bool stop = false;
    while (!stop) {
        int checks = 0;
        while (it <= max_iter && checks < per_check) {
            int rc = enqueue_iter(it);
            if (rc != LSG_OK) return rc;
            if (is_check(it)) checks++;
            it++;
        }
        const int slot = batch & 1;
        LSG_CUDA(cudaMemcpyAsync(ws->hctrl + slot, ws->ctrl, sizeof(DevCtrl), cudaMemcpyDeviceToHost, R.s));
        LSG_CUDA(cudaEventRecord(ws->ev[slot], R.s));
        if (batch > 0) {
            const int prev = slot ^ 1;
            LSG_CUDA(cudaEventSynchronize(ws->ev[prev]));
            if (ws->hctrl[prev].done) stop = true;
        }
        if (it > max_iter) stop = true;
        batch++;
    }
    LSG_CUDA(cudaStreamSynchronize(R.s));
    return LSG_OK;
}

static int default_per_check(const lsg_params *prm, long long n) {
    if (prm->check_every > 0) return prm->check_every;
    return n >= (1LL << 21) ? 2 : 8;
}

static void fill_result(lsg_result *res, const DevCtrl &c, int max_iter, double seconds,
                        long long launches) {
    if (!res) return;
    res->iters = c.done ? c.iters : max_iter;
    res->rhs_norm = c.rhs_norm;
    res->relres = c.rhs_norm > 0 ? c.relres / c.rhs_norm : c.relres;
    if (c.status == LSG_NAN_DETECTED) res->status = LSG_NAN_DETECTED;
    else if (c.df_range) res->status = LSG_RANGE;
    else if (c.status == LSG_TIMEOUT) res->status = LSG_TIMEOUT;
    else if (c.done && !c.stalled && !(c.relres > c.tol_abs)) res->status = LSG_OK;
    else res->status = (c.status == LSG_SVD_NO_CONVERGENCE) ? LSG_SVD_NO_CONVERGENCE : LSG_NOT_CONVERGED;
    res->seconds = seconds;
    res->launches = launches;
    res->svd_fallbacks = c.svd_fallbacks;
}

static double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// ---------------------------------------------------------------- AAR

// Number of Richardson (non-extrapolation) iterations among 1..last: the
// parity of the r (and, in the reference form, x) ping-pong after `last`.
static long long richardson_count(int last, int p) {
    if (last < 1) return 0;
    return last - last / p + (p == 1 ? 1 : 0);
}

// The AAR iteration (AAR.c:91-148) as a resumable object: enqueue(it) issues
// iteration `it`; the caller drives it with pipelined_loop and may pause it
// (the device sets ctrl->done) and resume from any iteration.
//   FP64 follows the reference's true-residual form: x and r ping-pong.
//   FP32 uses the residual recurrence: x in place, only r ping-pongs, and
//   b is not read after the initial residual.  When a cycle's Richardson
//   columns all stay in the history (p - 1 <= m) the Richardson passes leave
//   x out ("lean"): r rotates through three buffers so the cycle-start
//   residual survives, and the extrapolation rebuilds x from it.
template <typename T>
struct AarLoop {
    using S = typename ScalarOf<T>::type;
    static constexpr bool recur = std::is_same<typename RealOf<T>::type, float>::value;
    static constexpr int W = AccWidth<T>::value;
    Run &R;
    const lsg_params *prm;
    Workspace *ws;
    const T *b;
    long long n;
    int m, p;
    Weights<T> w;
    S cf;
    StencilLaunch L;     // residual passes
    StencilLaunch Lr;    // Richardson passes (autotuned shape when cached, or the paired march)
    StencilLaunch Lres;  // extrapolation-step residual of the recurrence form
    int sb, sbr, rb, gb; // stencil blocks of L and of Lres (partial sums)
    T *X[2];
    T *Rv[3];
    T *DX, *DF;
    DevCtrl *ctrl;
    double *part;
    bool lean = false;
    int xc = 0, rc = 0, rsc = 0;  // rsc: buffer of the cycle-start residual (lean)
    // residual ring (RingWindow): r_k in slot k mod (m + 1) of RG
    bool ring = false;
    T *RG = nullptr;
    long long rss = 0;
    std::vector<int> replaced;  // iterations whose residual a mixed solve overwrote
    int fold_it = 0;            // x holds the Richardson steps up to this iteration

    AarLoop(Run &R_, const lsg_operator *op, const lsg_params *prm_, T *x, const T *b_, Workspace *ws_)
        : R(R_), prm(prm_), ws(ws_), b(b_) {
        const Geom g = make_geom(op->n);
        n = g.n;
        m = prm->m;
        p = prm->p;
        const int form = aar_form();
        lean = recur && m <= 32 && p - 1 <= m && form != 2;
        if constexpr (std::is_same<T, float>::value)
            ring = lean && form == 0 && ws->ring && m <= kRingMaxM && n % 4 == 0 && ws->ring_ss % 4 == 0 &&
                   (((uintptr_t)x | (uintptr_t)ws->xalt | (uintptr_t)ws->dx | (uintptr_t)ws->df) & 15u) == 0;
        w = make_weights<T>(op);
        cf = jacobi_factor<T>(op);
        const int lz = choose_lz<T>(g, stencil_slots<T>(R.sms));
        L = StencilLaunch{g, lz, R.s};  // paired -1: untuned
        L.exact = fp64_exact_for(prm->tol);
        Lr = rich_launch<T>(op, L);      // a tuned shape sets paired to 0 (classic) or 1
        L.paired = 0;
        Lres = L;
        sb = (int)stencil_blocks<T>(g, lz);
        sbr = sb;
        // FP32 recurrence passes: the two-columns-per-lane march when the grid
        // and every vector allow 8-byte pairs
        int plz = 0;
        const long long pb = Kernels<T>::paired_plan(g, &plz);
        const uintptr_t al = (uintptr_t)x | (uintptr_t)ws->xalt | (uintptr_t)ws->r0 | (uintptr_t)ws->r1 |
                             (uintptr_t)ws->rs | (uintptr_t)ws->dx | (uintptr_t)ws->df;
        const bool pairable = recur && pb > 0 && op->radius == 6 && g.nx % 2 == 0 && (al & 7u) == 0;
        if (pairable) {
            if (Lr.paired == -1) {  // untuned: the paired march
                Lr.paired = 1;
                Lr.lz = plz;
                if (ring) Kernels<T>::ring_paired_plan(g, &Lr.lz);
            }
            Lres.paired = 1;
            Lres.lz = plz;
            sbr = (int)pb;
        } else if (Lr.paired >= 1) {  // tuned paired shape the vectors cannot take
            Lr = L;
        }
        if (Lr.paired == -1) Lr.paired = 0;
        rb = reduce_blocks(n, R.sms);
        gb = Kernels<T>::gram_grid(GRAM_SYM, m, n, R.sms);
        X[0] = x;
        X[1] = (T *)ws->xalt;
        Rv[0] = (T *)ws->r0;
        Rv[1] = (T *)ws->r1;
        Rv[2] = (T *)ws->rs;
        DX = (T *)ws->dx;
        DF = (T *)ws->df;
        ctrl = ws->ctrl;
        part = ws->partials;
        if (ring) {
            RG = (T *)ws->ring;
            rss = ws->ring_ss;
        }
    }
    bool is_anderson(int it) const { return it % p == 0 && it > 1; }
    T *slot_ptr(int k) const { return RG + (size_t)(k % (m + 1)) * (size_t)rss; }
    bool was_replaced(int k) const { return std::find(replaced.begin(), replaced.end(), k) != replaced.end(); }
    // The ring's view at extrapolation iteration `it` (or, for a fold after
    // iteration it - 1, of the columns up to it - 1).
    RingWindow window(int it) const {
        RingWindow rw{};
        const int M1 = m + 1;
        for (int t = 0; t <= m; t++) {
            const int k = it - m - 1 + t;
            rw.slot[t] = ((k % M1) + M1) % M1;
        }
        rw.s0 = (it - 1) % m;
        int la = 0;  // the last extrapolation before it
        for (int k = it - 1; k >= 1; k--)
            if (is_anderson(k)) { la = k; break; }
        for (int t = 0; t < m; t++) {
            const int k = it - m + t;
            if (k < 1) continue;
            const bool ext = is_anderson(k), rep = was_replaced(k);
            rw.valid |= 1u << t;
            if (ext || rep) rw.hmem |= 1u << t;
            if (rep) rw.dfmem |= 1u << t;
            if (!ext && k > la && k > fold_it) rw.cyc |= 1u << t;
        }
        rw.e0 = rw.e1 = -1;
        for (int t = 0; t < m; t++)
            if ((rw.hmem >> t) & 1u) {
                if (rw.e0 < 0) rw.e0 = t;
                else if (rw.e1 < 0) rw.e1 = t;
            }
        return rw;
    }
    // The residual the iteration continues from after iterations 1..last (a
    // mixed solve replaces it with the FP64 residual).
    T *residual_after(int last) {
        if (ring) return slot_ptr(last);
        sync_parity(last);
        return Rv[rc];
    }
    // Before that residual is overwritten, the ring keeps its column: DF (and,
    // for a Richardson column, H) go to the history arrays.
    int prepare_replace(int last) {
        if (!ring || last < 1 || was_replaced(last)) return LSG_OK;
        const size_t col = (size_t)((last - 1) % m) * (size_t)n;
        LSG_KC(LSG_K_REFINE, Kernels<T>::ring_store_column(slot_ptr(last - 1), slot_ptr(last), DF + col,
                                                           is_anderson(last) ? nullptr : DX + col,
                                                           prm->omega * cf, prm->beta, cf, n, R.s));
        replaced.push_back(last);
        return LSG_OK;
    }
    // r buffers holding the residual (and, lean, the cycle-start residual)
    // after iteration `last`
    void sync_parity(int last) {
        if (lean) {
            lean_buffers(last, p, &rsc, &rc);
            xc = 0;
            return;
        }
        const long long rich = richardson_count(last, p);
        rc = (int)(rich & 1);
        xc = recur ? 0 : rc;
    }
    unsigned cycle_mask(int last) const { return lean_mask(last, p, m); }
    // A lean solve that stopped after Richardson iteration `last` has not
    // added that cycle's steps to x yet: fold them in.
    int finish(int last) {
        if (!lean || last < 1 || is_anderson(last)) return LSG_OK;
        if (ring) {
            if (last <= fold_it) return LSG_OK;
            LSG_KC(LSG_K_UPDATE, Kernels<T>::ring_fold(m, window(last + 1), RG, rss, X[0], prm->omega * cf, n, R.s));
            fold_it = last;
            return LSG_OK;
        }
        sync_parity(last);
        LSG_KC(LSG_K_UPDATE, Kernels<T>::recur_fold(m, X[0], Rv[rc], Rv[rsc], DX, prm->beta, cf, n,
                                                    cycle_mask(last), R.s));
        return LSG_OK;
    }
    int reset_history() {
        LSG_CUDA(cudaMemsetAsync(DX, 0, sizeof(T) * (size_t)n * m, R.s));
        LSG_CUDA(cudaMemsetAsync(DF, 0, sizeof(T) * (size_t)n * m, R.s));
        return LSG_OK;
    }
    int enqueue(int it) {
        const int col = (it - 1) % m;  // the reference writes this column at iteration it+1
        T *dxc = DX + (size_t)col * n, *dfc = DF + (size_t)col * n;
        if constexpr (std::is_same<T, float>::value) {
          if (ring) {
            if (is_anderson(it)) {
                const RingWindow rw = window(it);
                LSG_KC(LSG_K_GRAM, Kernels<T>::ring_gram(m, rw, RG, rss, DF, cf, n, part, gb, ctrl, R.s));
                LSG_KC(LSG_K_SMALL, finalize_gram_solve(part, gb, GRAM_SYM, m, cf, ctrl, R.s));
                T *step = (T *)ws->xalt;  // the residual pass reads it as its stencil input
                LSG_KC(LSG_K_UPDATE, Kernels<T>::ring_update(m, rw, RG, rss, DX, X[0], step, prm->omega * cf,
                                                             prm->beta, cf, n, ctrl, R.s));
                LSG_KC(LSG_K_RESIDUAL, Kernels<T>::ring_residual(Lres, w, step, slot_ptr(it - 1), slot_ptr(it), dxc,
                                                                 cf, prm->beta, part, ctrl));
                LSG_KC(LSG_K_SMALL, finalize_norm(part, sbr, ctrl, NF_CHECK, prm->tol, it, R.s, W));
            } else {
                LSG_KC(LSG_K_RICHARDSON, Kernels<T>::ring_richardson(Lr, w, slot_ptr(it - 1), slot_ptr(it),
                                                                     prm->omega * cf, ctrl));
            }
            return LSG_OK;
          }
        }
        if (is_anderson(it)) {
            LSG_KC(LSG_K_GRAM, Kernels<T>::gram(GRAM_SYM, m, DX, DF, Rv[rc], n, part, gb, ctrl, R.s, L.exact));
            if constexpr (IsCplx<T>::value)
                LSG_KC(LSG_K_SMALL, finalize_gram_solve_c(part, gb, m, cf, ctrl, R.s));
            else
                LSG_KC(LSG_K_SMALL, finalize_gram_solve(part, gb, GRAM_SYM, m, cf, ctrl, R.s));
            if (recur) {
                // the step goes to the spare vector: the residual reads it as its stencil input
                T *step = (T *)ws->xalt;
                if (lean)
                    LSG_KC(LSG_K_UPDATE, Kernels<T>::aar_update_lean(m, X[0], Rv[rc], Rv[rsc], DX, step, prm->beta,
                                                                     cf, n, cycle_mask(it - 1), ctrl, R.s));
                else
                    LSG_KC(LSG_K_UPDATE, Kernels<T>::aar_update(m, X[0], Rv[rc], DX, step, prm->beta, cf, n, ctrl, R.s));
                LSG_KC(LSG_K_RESIDUAL, Kernels<T>::residual_recur(Lres, w, step, Rv[rc], dfc, dxc, cf, prm->beta, part, ctrl));
                rsc = rc;
            } else {
                LSG_KC(LSG_K_UPDATE, Kernels<T>::aar_update(m, X[xc], Rv[rc], DX, dxc, prm->beta, cf, n, ctrl, R.s));
                LSG_KC(LSG_K_RESIDUAL, Kernels<T>::residual(L, w, RES_ANDERSON, X[xc], b, Rv[rc], dfc, dxc, cf,
                                                            prm->beta, part, ctrl));
            }
            LSG_KC(LSG_K_SMALL, finalize_norm(part, recur ? sbr : sb, ctrl, NF_CHECK, prm->tol, it, R.s, W));
        } else if (lean) {
            const int t = lean_target(rsc, rc);
            LSG_KC(LSG_K_RICHARDSON, Kernels<T>::richardson_lean(Lr, w, Rv[rc], Rv[t], dxc, dfc, prm->omega * cf,
                                                                 cf, prm->beta, ctrl));
            rc = t;
        } else if (recur) {
            LSG_KC(LSG_K_RICHARDSON, Kernels<T>::richardson_recur(Lr, w, Rv[rc], X[0], Rv[rc ^ 1], dxc, dfc,
                                                                  prm->omega * cf, cf, prm->beta, ctrl));
            rc ^= 1;
        } else {
            LSG_KC(LSG_K_RICHARDSON, Kernels<T>::richardson(Lr, w, RICH_AAR, X[xc], Rv[rc], b, X[xc ^ 1], Rv[rc ^ 1],
                                                            dxc, dfc, prm->omega * cf, cf, prm->beta, ctrl));
            xc ^= 1;
            rc ^= 1;
        }
        return LSG_OK;
    }
    // Runs iterations first..max_iter until the device pauses or stops.
    int run(int first) {
        auto enq = [this](int it) { return enqueue(it); };
        auto chk = [this](int it) { return is_anderson(it); };
        return pipelined_loop(R, ws, first, prm->max_iter, default_per_check(prm, n), enq, chk);
    }
};

// AAR.c:37-177.  x (in/out) and b are device arrays of n values of T.
template <typename T>
int aar_core(Run &R, const lsg_operator *op, const lsg_params *prm, T *x, const T *b,
             Workspace *ws, DevCtrl *out) {
    AarLoop<T> A(R, op, prm, x, b, ws);
    ws->hctrl[0] = ctrl_init(prm->tol, 0);
    LSG_CUDA(cudaMemcpyAsync(A.ctrl, ws->hctrl, sizeof(DevCtrl), cudaMemcpyHostToDevice, R.s));
    int rc = A.reset_history();
    if (rc) return rc;
    // ||b|| and tol *= ||b|| (AAR.c:78-79); f = b - A x (AAR.c:80-82).
    LSG_KC(LSG_K_UPDATE, Kernels<T>::norm2(b, A.n, A.part, A.rb, A.ctrl, R.s));
    LSG_KC(LSG_K_SMALL, finalize_norm(A.part, A.rb, A.ctrl, NF_RHS, prm->tol, 0, R.s, AarLoop<T>::W));
    LSG_KC(LSG_K_RESIDUAL, Kernels<T>::residual(A.L, A.w, RES_INIT, x, b, A.residual_after(0), nullptr, nullptr,
                                                A.cf, 0.0, A.part, A.ctrl));
    rc = A.run(1);
    if (rc != LSG_OK) return rc;
    DevCtrl c;
    LSG_CUDA(cudaMemcpy(&c, A.ctrl, sizeof(DevCtrl), cudaMemcpyDeviceToHost));
    // Where the last iterate lives: in the reference form x moved to the other
    // buffer at every Richardson iteration up to the final one.
    const int last = c.done ? c.iters : prm->max_iter;
    if (!AarLoop<T>::recur && (richardson_count(last, prm->p) & 1))
        LSG_CUDA(cudaMemcpyAsync(x, A.X[1], sizeof(T) * (size_t)A.n, cudaMemcpyDeviceToDevice, R.s));
    if (!c.done) {
        rc = A.finish(last);
        if (rc != LSG_OK) return rc;
    }
    LSG_CUDA(cudaStreamSynchronize(R.s));
    *out = c;
    return LSG_OK;
}

// PGR.c:35-173 (galerkin) and PL2R.c:35-172.
template <typename T>
int prich_core(Run &R, bool galerkin, const lsg_operator *op, const lsg_params *prm, T *x,
               const T *b, Workspace *ws, DevCtrl *out) {
    const Geom g = make_geom(op->n);
    const long long n = g.n;
    const int m = prm->m, p = prm->p, max_iter = prm->max_iter;
    const Weights<T> w = make_weights<T>(op);
    const double cf = op->precond ? 1.0 / jacobi_diag(op) : 1.0;
    const int lz = choose_lz<T>(g, stencil_slots<T>(R.sms));
    StencilLaunch L{g, lz, R.s};
    L.exact = fp64_exact_for(prm->tol);
    StencilLaunch Lr = rich_launch<T>(op, L);
    if (Lr.paired >= 1) Lr = L;  // the paired march serves the AAR recurrence passes only
    Lr.paired = 0;
    const int rb = reduce_blocks(n, R.sms);
    T *X[2] = {x, (T *)ws->xalt};
    T *Rv[2] = {(T *)ws->r0, (T *)ws->r1};
    T *DX = (T *)ws->dx, *DF = (T *)ws->df;
    DevCtrl *ctrl = ws->ctrl;
    double *part = ws->partials;
    const int kind = galerkin ? GRAM_GALERKIN : GRAM_SYM;
    const int gb = Kernels<T>::gram_grid(kind, m, n, R.sms);

    ws->hctrl[0] = ctrl_init(prm->tol, 0);
    LSG_CUDA(cudaMemcpyAsync(ctrl, ws->hctrl, sizeof(DevCtrl), cudaMemcpyHostToDevice, R.s));
    LSG_CUDA(cudaMemsetAsync(DX, 0, sizeof(T) * (size_t)n * m, R.s));
    LSG_CUDA(cudaMemsetAsync(DF, 0, sizeof(T) * (size_t)n * m, R.s));
    LSG_KC(LSG_K_UPDATE, Kernels<T>::norm2(b, n, part, rb, ctrl, R.s));
    LSG_KC(LSG_K_SMALL, finalize_norm(part, rb, ctrl, NF_RHS, prm->tol, 0, R.s));
    LSG_KC(LSG_K_RESIDUAL, Kernels<T>::residual(L, w, RES_INIT, X[0], b, Rv[0], nullptr, nullptr, cf, 0.0, part, ctrl));

    int cur = 0;
    auto is_proj = [p](int it) { return it % p == 0; };
    auto enqueue = [&](int it) -> int {
        const int col = (it - 2 + m) % m;
        LSG_KC(LSG_K_RICHARDSON, Kernels<T>::richardson(Lr, w, RICH_PGR, X[cur], Rv[cur], b, X[cur ^ 1], Rv[cur ^ 1],
                                      DX + (size_t)col * n, DF + (size_t)col * n, prm->omega * cf,
                                      cf, 0.0, ctrl));
        cur ^= 1;
        if (is_proj(it)) {
            LSG_KC(LSG_K_GRAM, Kernels<T>::gram(kind, m, DX, DF, Rv[cur], n, part, gb, ctrl, R.s, L.exact));
            LSG_KC(LSG_K_SMALL, finalize_gram_solve(part, gb, kind, m, 1.0, ctrl, R.s));
            LSG_KC(LSG_K_UPDATE, Kernels<T>::proj_update(m, col, X[cur], Rv[cur], DX, DF, n, part, rb, ctrl, R.s));
            LSG_KC(LSG_K_SMALL, finalize_norm(part, rb, ctrl, NF_CHECK, prm->tol, it, R.s));
        }
        return LSG_OK;
    };
    int rc = pipelined_loop(R, ws, 1, max_iter, default_per_check(prm, n), enqueue, is_proj);
    if (rc != LSG_OK) return rc;
    DevCtrl c;
    LSG_CUDA(cudaMemcpy(&c, ctrl, sizeof(DevCtrl), cudaMemcpyDeviceToHost));
    const int last = c.done ? c.iters : max_iter;
    if (last & 1) LSG_CUDA(cudaMemcpyAsync(x, X[1], sizeof(T) * (size_t)n, cudaMemcpyDeviceToDevice, R.s));
    LSG_CUDA(cudaStreamSynchronize(R.s));
    *out = c;
    return LSG_OK;
}

// CG.c:33-175.  Work vectors: r = r0, d ping-pong = (r1, xalt), q = dx[0].
template <typename T>
int cg_core(Run &R, const lsg_operator *op, const lsg_params *prm, T *x, const T *b,
            Workspace *ws, DevCtrl *out) {
    const Geom g = make_geom(op->n);
    const long long n = g.n;
    const int max_iter = prm->max_iter;
    const Weights<T> w = make_weights<T>(op);
    const double cf = op->precond ? 1.0 / jacobi_diag(op) : 1.0;
    const int lz = choose_lz<T>(g, stencil_slots<T>(R.sms));
    StencilLaunch L{g, lz, R.s};
    L.exact = fp64_exact_for(prm->tol);
    const int sb = (int)stencil_blocks<T>(g, lz);
    const int rb = reduce_blocks(n, R.sms);
    T *r = (T *)ws->r0;
    T *D[2] = {(T *)ws->r1, (T *)ws->xalt};
    T *q = (T *)ws->dx;
    DevCtrl *ctrl = ws->ctrl;
    double *part = ws->partials;

    ws->hctrl[0] = ctrl_init(prm->tol, 0);
    LSG_CUDA(cudaMemcpyAsync(ctrl, ws->hctrl, sizeof(DevCtrl), cudaMemcpyHostToDevice, R.s));
    LSG_CUDA(cudaMemsetAsync(D[0], 0, sizeof(T) * (size_t)n, R.s));
    LSG_KC(LSG_K_UPDATE, Kernels<T>::norm2(b, n, part, rb, ctrl, R.s));
    LSG_KC(LSG_K_SMALL, finalize_norm(part, rb, ctrl, NF_RHS, prm->tol, 0, R.s));
    // r = b - A x; d = M^-1 r; delta = r.d; relres = ||r|| (CG.c:65-89)
    LSG_KC(LSG_K_RESIDUAL, Kernels<T>::residual(L, w, RES_INIT, x, b, r, nullptr, nullptr, cf, 0.0, part, ctrl));
    LSG_KC(LSG_K_SMALL, finalize_cg(part, sb, ctrl, 2, cf, op->precond, 0, max_iter, R.s));

    int cur = 0;
    auto always = [](int) { return true; };
    auto enqueue = [&](int it) -> int {  // it = iter_count + 1
        const int ic = it - 1;           // iter_count at the top of the loop body
        LSG_KC(LSG_K_CG, Kernels<T>::cg_direction(L, w, r, D[cur], D[cur ^ 1], q, cf, part, ctrl));
        cur ^= 1;
        LSG_KC(LSG_K_SMALL, finalize_cg(part, sb, ctrl, 0, cf, op->precond, it, max_iter, R.s));
        if (ic % 50 == 0) {  // restart with the true residual (CG.c:109-120)
            LSG_KC(LSG_K_UPDATE, Kernels<T>::cg_step(x, r, D[cur], q, n, 1, part, rb, ctrl, R.s));
            LSG_KC(LSG_K_RESIDUAL, Kernels<T>::residual(L, w, RES_INIT, x, b, r, nullptr, nullptr, cf, 0.0, part, ctrl));
            LSG_KC(LSG_K_SMALL, finalize_cg(part, sb, ctrl, 1, cf, op->precond, it, max_iter, R.s));
        } else {
            LSG_KC(LSG_K_UPDATE, Kernels<T>::cg_step(x, r, D[cur], q, n, 0, part, rb, ctrl, R.s));
            LSG_KC(LSG_K_SMALL, finalize_cg(part, rb, ctrl, 1, cf, op->precond, it, max_iter, R.s));
        }
        return LSG_OK;
    };
    const int per = prm->check_every > 0 ? prm->check_every : (n >= (1LL << 21) ? 8 : 32);
    int rc = pipelined_loop(R, ws, 1, max_iter, per, enqueue, always);
    if (rc != LSG_OK) return rc;
    DevCtrl c;
    LSG_CUDA(cudaMemcpy(&c, ctrl, sizeof(DevCtrl), cudaMemcpyDeviceToHost));
    *out = c;
    return LSG_OK;
}

// ---------------------------------------------------------------- dispatch

template <typename T>
static int solve_t(int solver, const lsg_operator *op, const lsg_params *prm, void *d_x,
                   const void *d_b, lsg_result *res, cudaStream_t s) {
    static const char *const names[4] = {"lsg_aar", "lsg_pgr", "lsg_pl2r", "lsg_cg"};
    TraceRange trace(names[solver & 3]);
    const double t0 = now_s();
    const Geom g = make_geom(op->n);
    Workspace *ws = nullptr;
    std::unique_lock<std::mutex> lk;
    const int mh = solver == 3 ? 1 : prm->m;
    if (IsCplx<T>::value && solver != 0)
        return set_error(LSG_UNSUPPORTED, "complex vectors: only AAR is provided (PETSC_COMPLEX/AAR_Complex.c)");
    if (IsCplx<T>::value && 2 * prm->m > LSG_MAX_M)
        return set_error(LSG_BAD_ARG, "complex AAR: m = %d > %d", prm->m, LSG_MAX_M / 2);
    int rc = get_workspace(sizeof(T), g.n, mh, false, g, &ws, &lk);
    if (rc != LSG_OK) return rc;
    Run R(s, sm_count());
    DevCtrl c;
    if constexpr (IsCplx<T>::value) {
        rc = aar_core<T>(R, op, prm, (T *)d_x, (const T *)d_b, ws, &c);
    } else {
        switch (solver) {
        case 0: rc = aar_core<T>(R, op, prm, (T *)d_x, (const T *)d_b, ws, &c); break;
        case 1: rc = prich_core<T>(R, true, op, prm, (T *)d_x, (const T *)d_b, ws, &c); break;
        case 2: rc = prich_core<T>(R, false, op, prm, (T *)d_x, (const T *)d_b, ws, &c); break;
        default: rc = cg_core<T>(R, op, prm, (T *)d_x, (const T *)d_b, ws, &c); break;
        }
    }
    if (rc != LSG_OK) return rc;
    R.flush();
    lsg_result tmp;
    fill_result(&tmp, c, prm->max_iter, now_s() - t0, R.launches);
    tmp.outer_iters = 0;
    tmp.inner_iters = 0;
    if (res) *res = tmp;
    set_last_status(tmp.status);
    return tmp.status;
}

int solve(int solver, const lsg_operator *op, const lsg_params *prm, int dtype, void *d_x,
          const void *d_b, lsg_result *res, cudaStream_t s) {
    int rc = check_operator(op);
    if (rc) return rc;
    rc = check_params(prm, solver != 3);
    if (rc) return rc;
    if (!d_x || !d_b) return set_error(LSG_BAD_ARG, "NULL vector");
    if (dtype == LSG_F64) return solve_t<double>(solver, op, prm, d_x, d_b, res, s);
    if (dtype == LSG_F32) return solve_t<float>(solver, op, prm, d_x, d_b, res, s);
    if (dtype == LSG_C128) return solve_t<cplx<double>>(solver, op, prm, d_x, d_b, res, s);
    if (dtype == LSG_C64) return solve_t<cplx<float>>(solver, op, prm, d_x, d_b, res, s);
    return set_error(LSG_BAD_ARG, "unknown dtype %d", dtype);
}

// ---------------------------------------------------------------- mixed precision

// FP32 AAR with FP64 residual replacement.  One FP32 AAR iteration runs on the
// correction e (x = x64 + e), its residual carried by the FP32 recurrence.
// Whenever the FP32 residual has fallen by the factor rho = inner_tol since
// the last replacement (or stalls, or passes tol), the device pauses the
// iteration; the host then folds e into x64 (x64 += e, e = 0), recomputes
// r = b - A x64 in FP64, stores it as the FP32 residual and resumes -- with the
// Anderson history intact, so no iterations are spent rebuilding it.  FP64
// is used only for that residual, x64, the reductions and the m x m solve.
// Convergence is decided on the FP64 residual.
template <typename T64, typename T32>
int solve_mixed_t(const lsg_operator *op, const lsg_params *prm, T64 *x, const T64 *b,
                  lsg_result *res, cudaStream_t s) {
    constexpr int W = AccWidth<T64>::value;
    TraceRange trace("lsg_aar_mixed");
    const double t0 = now_s();
    int rc = check_operator(op);
    if (rc) return rc;
    rc = check_params(prm, true);
    if (rc) return rc;
    if (IsCplx<T64>::value && 2 * prm->m > LSG_MAX_M)
        return set_error(LSG_BAD_ARG, "complex AAR: m = %d > %d", prm->m, LSG_MAX_M / 2);
    if (!x || !b) return set_error(LSG_BAD_ARG, "NULL vector");
    const Geom g = make_geom(op->n);
    const long long n = g.n;
    Workspace *wo = nullptr, *wi = nullptr;
    std::unique_lock<std::mutex> lo, li;
    rc = get_workspace(sizeof(T64), n, 1, true, g, &wo, &lo);  // outer: e32, partials, ctrl
    if (rc) return rc;
    rc = get_workspace(sizeof(T32), n, prm->m, false, g, &wi, &li);  // FP32 AAR work arrays
    if (rc) return rc;
    Run R(s, sm_count());
    const Weights<T64> w64 = make_weights<T64>(op);
    const int lz = choose_lz<T64>(g, stencil_slots<T64>(R.sms));
    StencilLaunch L64{g, lz, s};
    L64.exact = fp64_exact_for(prm->tol);
    const int sb64 = (int)stencil_blocks<T64>(g, lz);
    const int rb = reduce_blocks(n, R.sms);
    DevCtrl *octrl = wo->ctrl;
    double *opart = wo->partials;
    const int max_outer = prm->max_outer > 0 ? prm->max_outer : 50;
    const double rho = prm->inner_tol > 0 ? prm->inner_tol : 3e-4;
    T32 *e32 = (T32 *)wo->e32;
    AarLoop<T32> A(R, op, prm, e32, nullptr, wi);

    wo->hctrl[0] = ctrl_init(prm->tol, 0);
    wo->hctrl[0].x_zero = 1;
    LSG_CUDA(cudaMemcpyAsync(octrl, wo->hctrl, sizeof(DevCtrl), cudaMemcpyHostToDevice, s));
    LSG_CUDA(cudaMemsetAsync(e32, 0, sizeof(T32) * (size_t)n, s));
    // x0 = 0 (the usual start): the first residual needs no stencil pass
    LSG_KC(LSG_K_REFINE, zero_check<T64>(x, n, octrl, s));
    rc = A.reset_history();
    if (rc) return rc;
    LSG_KC(LSG_K_UPDATE, Kernels<T64>::norm2(b, n, opart, rb, octrl, s));
    LSG_KC(LSG_K_SMALL, finalize_norm(opart, rb, octrl, NF_RHS, prm->tol, 0, s, W));
    // the constant mode decouples when the shift is non-zero (deflate_x)
    const double sig_re = op->sigma, sig_im = IsCplx<T64>::value ? op->sigma_im : 0.0;
    const bool deflate = sig_re != 0.0 || sig_im != 0.0;
    if (deflate) {
        LSG_KC(LSG_K_REFINE, rhs_mean<T64>(b, n, opart, octrl, s));
        R.launches += 1;  // sum + finalize
    }

    int status = LSG_NOT_CONVERGED, replacements = 0, it = 1, iters = 0;
    double frac_run = 1.0;
    int misses_run = 0;
    DevCtrl co, ci;
    for (;;) {
        // r = b - A x64 in FP64, stored as the FP32 residual the iteration continues from
        rc = A.prepare_replace(it - 1);
        if (rc != LSG_OK) return rc;
        T32 *r32 = A.residual_after(it - 1);
        if (deflate) {
            LSG_KC(LSG_K_REFINE, deflate_x<T64>(x, n, opart, octrl, sig_re, sig_im, s));
            R.launches += 2;  // sum + finalize + shift
        }
        const int first = it == 1 ? 1 : 0;
        LSG_KC(LSG_K_REFINE, (ir_residual<T64, T32>(L64, w64, x, b, r32, opart, octrl, first)));
        if (first)
            LSG_KC(LSG_K_REFINE, (ir_residual_const<T64, T32>(b, r32, n, opart, sb64, octrl, sig_re, sig_im, s)));
        LSG_KC(LSG_K_SMALL, finalize_norm(opart, sb64, octrl, NF_CHECK, prm->tol, it - 1, s, W));
        LSG_CUDA(cudaMemcpyAsync(&wo->hctrl[0], octrl, sizeof(DevCtrl), cudaMemcpyDeviceToHost, s));
        LSG_CUDA(cudaStreamSynchronize(s));
        co = wo->hctrl[0];
        if (co.status == LSG_NAN_DETECTED) { status = LSG_NAN_DETECTED; break; }
        if (co.df_range) { status = LSG_RANGE; break; }
        if (co.done) { status = LSG_OK; break; }
        if (it > prm->max_iter || replacements >= max_outer) break;
        // resume (or start) the FP32 iteration with its next pause target
        if (it == 1) {
            ci = ctrl_init(prm->tol, 12);
        } else {
            ci.done = 0;
            ci.stall = 0;
            ci.stalled = 0;
            ci.best = INFINITY;
        }
        ci.tol_abs = next_target(&frac_run, &misses_run, rho, co.relres, ci.relres, co.tol_abs, it == 1);
        ci.rhs_norm = co.rhs_norm;
        wi->hctrl[0] = ci;
        LSG_CUDA(cudaMemcpyAsync(A.ctrl, wi->hctrl, sizeof(DevCtrl), cudaMemcpyHostToDevice, s));
        rc = A.run(it);
        if (rc != LSG_OK) return rc;
        LSG_CUDA(cudaMemcpy(&ci, A.ctrl, sizeof(DevCtrl), cudaMemcpyDeviceToHost));
        if (ci.status == LSG_NAN_DETECTED) { status = LSG_NAN_DETECTED; break; }
        if (ci.status == LSG_TIMEOUT) { status = LSG_TIMEOUT; break; }
        iters = ci.done ? ci.iters : prm->max_iter;
        if (!ci.done) {
            rc = A.finish(iters);
            if (rc != LSG_OK) return rc;
        }
        // fold the correction into x64 (e = 0 afterwards) and replace the residual
        LSG_KC(LSG_K_REFINE, (ir_correct<T64, T32>(x, e32, n, s)));
        replacements++;
        it = iters + 1;
    }
    LSG_CUDA(cudaStreamSynchronize(s));
    R.flush();
    if (res) {
        res->iters = iters;
        res->inner_iters = iters;
        res->outer_iters = replacements;
        res->rhs_norm = co.rhs_norm;
        res->relres = co.rhs_norm > 0 ? co.relres / co.rhs_norm : co.relres;
        res->status = status;
        res->seconds = now_s() - t0;
        res->launches = R.launches;
        res->svd_fallbacks = ci.svd_fallbacks;
    }
    set_last_status(status);
    return status;
}

int solve_mixed(const lsg_operator *op, const lsg_params *prm, double *x, const double *b,
                lsg_result *res, cudaStream_t s) {
    return solve_mixed_t<double, float>(op, prm, x, b, res, s);
}

int solve_mixed_c(const lsg_operator *op, const lsg_params *prm, void *x, const void *b,
                  lsg_result *res, cudaStream_t s) {
    return solve_mixed_t<cplx<double>, cplx<float>>(op, prm, (cplx<double> *)x, (const cplx<double> *)b,
                                                    res, s);
}

// ---------------------------------------------------------------- block ICC(0) AAR

// AAR.c:37-177 with f = M^-1 r, M the block ICC(0) factor (PETSC_REAL/AAR_Real.c
// pc = 1).  f is materialised by the preconditioner pass, which also completes
// the history column of the previous iteration (DF_c = f - f_old, H_c = step +
// beta DF_c, c = (it-2) % m); a Richardson iteration is then one stencil pass
// (x2 = x + omega f, r = b - A x2, the step into column (it-1) % m), an
// Anderson iteration the Gram of (DF, f), the m x m solve, the update
// x += beta f - sum H_j s_j (unit Jacobi factor) and the residual pass.
int solve_icc(const lsg_operator *op, const lsg_params *prm, const int block[3], double *x, const double *b,
              lsg_result *res, cudaStream_t s) {
    TraceRange trace("lsg_aar_icc");
    const double t0 = now_s();
    int rc = check_operator(op);
    if (rc) return rc;
    rc = check_params(prm, true);
    if (rc) return rc;
    if (!x || !b || !block) return set_error(LSG_BAD_ARG, "NULL argument");
    if (op->radius > 6) return set_error(LSG_UNSUPPORTED, "block ICC(0): radius %d > 6", op->radius);
    for (int a = 0; a < 3; a++)
        if (block[a] < 1 || block[a] > 255 || op->n[a] % block[a] != 0)
            return set_error(LSG_BAD_ARG, "block ICC(0): box side %d does not divide the grid side %d", block[a],
                             op->n[a]);
    if ((long long)block[0] * block[1] * block[2] > 4096)
        return set_error(LSG_BAD_ARG, "block ICC(0): a box holds at most 4096 points");
    const Geom g = make_geom(op->n);
    const long long n = g.n;
    const int m = prm->m, p = prm->p;
    Workspace *ws = nullptr;
    std::unique_lock<std::mutex> lk;
    rc = get_workspace(sizeof(double), n, m, false, g, &ws, &lk);
    if (rc) return rc;
    const IccFactor *F = nullptr;
    rc = icc_get(op, block, &F, nullptr);
    if (rc) return rc;
    Run R(s, sm_count());
    const Weights<double> w = make_weights<double>(op);
    const int lz = choose_lz<double>(g, stencil_slots<double>(R.sms));
    StencilLaunch L{g, lz, s};
    L.exact = fp64_exact_for(prm->tol);
    StencilLaunch Lr = rich_launch<double>(op, L);
    if (Lr.paired >= 1) Lr = L;
    Lr.paired = 0;
    Lr.exact = L.exact;
    const int sb = (int)stencil_blocks<double>(g, lz);
    const int rb = reduce_blocks(n, R.sms);
    const int gb = Kernels<double>::gram_grid(GRAM_SYM, m, n, R.sms);
    double *X[2] = {x, (double *)ws->xalt};
    double *r = (double *)ws->r0;
    double *Fv[2] = {(double *)ws->r1, (double *)ws->rs};
    double *H = (double *)ws->dx, *DF = (double *)ws->df;
    DevCtrl *ctrl = ws->ctrl;
    double *part = ws->partials;
    ws->hctrl[0] = ctrl_init(prm->tol, 0);
    LSG_CUDA(cudaMemcpyAsync(ctrl, ws->hctrl, sizeof(DevCtrl), cudaMemcpyHostToDevice, s));
    LSG_CUDA(cudaMemsetAsync(H, 0, sizeof(double) * (size_t)n * m, s));
    LSG_CUDA(cudaMemsetAsync(DF, 0, sizeof(double) * (size_t)n * m, s));
    LSG_KC(LSG_K_UPDATE, Kernels<double>::norm2(b, n, part, rb, ctrl, s));
    LSG_KC(LSG_K_SMALL, finalize_norm(part, rb, ctrl, NF_RHS, prm->tol, 0, s));
    LSG_KC(LSG_K_RESIDUAL, Kernels<double>::residual(L, w, RES_INIT, x, b, r, nullptr, nullptr, 1.0, 0.0, part, ctrl));
    int xc = 0, fc = 0;
    auto is_anderson = [p](int it) { return it % p == 0 && it > 1; };
    auto enqueue = [&](int it) -> int {
        const int cprev = ((it - 2) % m + m) % m;
        LSG_KC(LSG_K_PRECOND, icc_apply(F, g, r, Fv[fc ^ 1], Fv[fc], DF + (size_t)cprev * n, H + (size_t)cprev * n,
                                        prm->beta, it > 1 ? 1 : 0, ctrl, L.exact, s));
        fc ^= 1;
        const double *f = Fv[fc];
        double *hcol = H + (size_t)((it - 1) % m) * n;
        if (is_anderson(it)) {
            LSG_KC(LSG_K_GRAM, Kernels<double>::gram(GRAM_SYM, m, H, DF, f, n, part, gb, ctrl, s, L.exact));
            LSG_KC(LSG_K_SMALL, finalize_gram_solve(part, gb, GRAM_SYM, m, 1.0, ctrl, s));
            LSG_KC(LSG_K_UPDATE, Kernels<double>::aar_update(m, X[xc], f, H, hcol, prm->beta, 1.0, n, ctrl, s));
            LSG_KC(LSG_K_RESIDUAL, Kernels<double>::residual(L, w, RES_INIT, X[xc], b, r, nullptr, nullptr, 1.0, 0.0,
                                                             part, ctrl));
            LSG_KC(LSG_K_SMALL, finalize_norm(part, sb, ctrl, NF_CHECK, prm->tol, it, s));
        } else {
            LSG_KC(LSG_K_RICHARDSON, rich_prec(Lr, w, X[xc], f, b, X[xc ^ 1], r, hcol, prm->omega, ctrl));
            xc ^= 1;
        }
        return LSG_OK;
    };
    rc = pipelined_loop(R, ws, 1, prm->max_iter, default_per_check(prm, n), enqueue, is_anderson);
    if (rc != LSG_OK) return rc;
    DevCtrl c;
    LSG_CUDA(cudaMemcpy(&c, ctrl, sizeof(DevCtrl), cudaMemcpyDeviceToHost));
    const int last = c.done ? c.iters : prm->max_iter;
    if (richardson_count(last, p) & 1)
        LSG_CUDA(cudaMemcpyAsync(x, X[1], sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, s));
    LSG_CUDA(cudaStreamSynchronize(s));
    R.flush();
    lsg_result tmp;
    fill_result(&tmp, c, prm->max_iter, now_s() - t0, R.launches);
    tmp.outer_iters = 0;
    tmp.inner_iters = 0;
    if (res) *res = tmp;
    set_last_status(tmp.status);
    return tmp.status;
}

int apply(const lsg_operator *op, int dtype, const void *d_x, void *d_y, cudaStream_t s) {
    int rc = check_operator(op);
    if (rc) return rc;
    if (!d_x || !d_y) return set_error(LSG_BAD_ARG, "NULL vector");
    const Geom g = make_geom(op->n);
    const int sms = sm_count();
    if (dtype == LSG_F64) {
        const StencilLaunch L{g, choose_lz<double>(g, stencil_slots<double>(sms)), s};
        LSG_CUDA(Kernels<double>::residual(L, make_weights<double>(op), RES_APPLY, (const double *)d_x,
                                           nullptr, (double *)d_y, nullptr, nullptr, 1.0, 0.0, nullptr, nullptr));
    } else if (dtype == LSG_F32) {
        const StencilLaunch L{g, choose_lz<float>(g, stencil_slots<float>(sms)), s};
        LSG_CUDA(Kernels<float>::residual(L, make_weights<float>(op), RES_APPLY, (const float *)d_x,
                                          nullptr, (float *)d_y, nullptr, nullptr, 1.0, 0.0, nullptr, nullptr));
    } else if (dtype == LSG_C128) {
        const StencilLaunch L{g, choose_lz<cplx<double>>(g, stencil_slots<cplx<double>>(sms)), s};
        LSG_CUDA(Kernels<cplx<double>>::residual(L, make_weights<cplx<double>>(op), RES_APPLY,
                                                 (const cplx<double> *)d_x, nullptr, (cplx<double> *)d_y,
                                                 nullptr, nullptr, cplx<double>(1.0, 0.0), 0.0, nullptr, nullptr));
    } else if (dtype == LSG_C64) {
        const StencilLaunch L{g, choose_lz<cplx<float>>(g, stencil_slots<cplx<float>>(sms)), s};
        LSG_CUDA(Kernels<cplx<float>>::residual(L, make_weights<cplx<float>>(op), RES_APPLY,
                                                (const cplx<float> *)d_x, nullptr, (cplx<float> *)d_y,
                                                nullptr, nullptr, cplx<double>(1.0, 0.0), 0.0, nullptr, nullptr));
    } else {
        return set_error(LSG_BAD_ARG, "unknown dtype %d", dtype);
    }
    return LSG_OK;
}

// ---------------------------------------------------------------- general sparse operator

// Per-(device, n) extras of the CSR path: D^-1, the preconditioned residual f
// and a flag word for the structure checks.
struct CsrExtra {
    double *base = nullptr;
    double *dinv = nullptr, *f = nullptr;
    int *flag = nullptr;
    ~CsrExtra() {
        if (base) cudaFree(base);
    }
};
static std::mutex g_csr_mu;
static std::map<std::pair<int, long long>, std::unique_ptr<CsrExtra>> g_csr;

static void release_csr_extras() {
    std::lock_guard<std::mutex> g(g_csr_mu);
    g_csr.clear();
}

static int csr_view(const lsg_csr *A, CsrView *v) {
    if (!A) return set_error(LSG_BAD_ARG, "matrix is NULL");
    if (A->n < 1) return set_error(LSG_BAD_ARG, "matrix size n = %d < 1", A->n);
    if (A->nnz < 1 || A->nnz > 2147483647LL)
        return set_error(LSG_BAD_ARG, "nnz = %lld outside 1..2^31-1 (32-bit row offsets)", A->nnz);
    if (!A->row_ptr || !A->col || !A->val) return set_error(LSG_BAD_ARG, "NULL CSR array");
    v->n = A->n;
    v->nnz = A->nnz;
    v->rp = A->row_ptr;
    v->col = A->col;
    v->val = A->val;
    const int lpr = A->lanes_per_row;
    if (lpr != 0 && lpr != 1 && lpr != 4 && lpr != 8 && lpr != 16 && lpr != 32)
        return set_error(LSG_BAD_ARG, "lanes_per_row %d is not 0, 1, 4, 8, 16 or 32", lpr);
    v->group = lpr ? lpr : csr_group(*v);
    return LSG_OK;
}

// Checks the caller's row offsets, then (only if they are sound) the column
// indices; returns LSG_BAD_ARG on a malformed matrix before any gather runs.
static int csr_validate(const CsrView &A, CsrExtra *ex, cudaStream_t s) {
    const int blocks = (int)std::max<long long>(1, std::min<long long>((A.nnz + 255) / 256, 4LL * sm_count()));
    for (int phase = 0; phase < 2; phase++) {
        int bad = 0;
        LSG_CUDA(cudaMemsetAsync(ex->flag, 0, sizeof(int), s));
        LSG_CUDA(csr_check(A, phase, ex->flag, blocks, s));
        LSG_CUDA(cudaMemcpyAsync(&bad, ex->flag, sizeof(int), cudaMemcpyDeviceToHost, s));
        LSG_CUDA(cudaStreamSynchronize(s));
        if (bad)
            return set_error(LSG_BAD_ARG, phase == 0 ? "CSR row offsets are not 0 .. nnz non-decreasing"
                                                     : "CSR column index outside 0..n-1");
    }
    return LSG_OK;
}

static int csr_extra(long long n, CsrExtra **out) {
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> g(g_csr_mu);
    auto &slot = g_csr[std::make_pair(dev, n)];
    if (!slot) slot.reset(new CsrExtra());
    CsrExtra *ex = slot.get();
    if (!ex->base) {
        const size_t vb = align_up((size_t)n * 8);
        cudaError_t e = cudaMalloc(&ex->base, 2 * vb + 256);
        if (e != cudaSuccess) {
            cudaGetLastError();
            ex->base = nullptr;
            return set_error(LSG_NO_MEMORY, "CSR work arrays: %s", cudaGetErrorString(e));
        }
        ex->dinv = ex->base;
        ex->f = (double *)((char *)ex->base + vb);
        ex->flag = (int *)((char *)ex->base + 2 * vb);
    }
    *out = ex;
    return LSG_OK;
}

// AAR.c:37-177 on a general matrix: the reference-form iteration of AarLoop
// with CSR passes; the extrapolation step materialises f = D^-1 r and reuses
// the Gram, m x m solve and update kernels with a unit Jacobi factor.
int solve_csr(const lsg_csr *Ain, const lsg_params *prm, double *x, const double *b, lsg_result *res,
              cudaStream_t s) {
    TraceRange trace("lsg_aar_csr");
    const double t0 = now_s();
    CsrView A;
    int rc = csr_view(Ain, &A);
    if (rc) return rc;
    rc = check_params(prm, true);
    if (rc) return rc;
    if (prm->m > 8) return set_error(LSG_UNSUPPORTED, "CSR AAR: history depth m = %d > 8", prm->m);
    if (!x || !b) return set_error(LSG_BAD_ARG, "NULL vector");
    const long long n = A.n;
    CsrExtra *ex = nullptr;
    rc = csr_extra(n, &ex);
    if (rc) return rc;
    rc = csr_validate(A, ex, s);
    if (rc) return rc;
    const int nn[3] = {A.n, 1, 1};
    const Geom g = make_geom(nn);
    Workspace *ws = nullptr;
    std::unique_lock<std::mutex> lk;
    rc = get_workspace(sizeof(double), n, prm->m, false, g, &ws, &lk);
    if (rc) return rc;
    Run R(s, sm_count());
    const int m = prm->m, p = prm->p;
    const int cb = (int)std::max<long long>(1, std::min<long long>((n * A.group + 255) / 256, 8LL * R.sms));
    const int rb = reduce_blocks(n, R.sms);
    const int gb = Kernels<double>::gram_grid(GRAM_SYM, m, n, R.sms);
    double *X[2] = {x, (double *)ws->xalt};
    double *Rv[2] = {(double *)ws->r0, (double *)ws->r1};
    double *DX = (double *)ws->dx, *DF = (double *)ws->df;
    DevCtrl *ctrl = ws->ctrl;
    double *part = ws->partials;
    int bad = 0;
    LSG_CUDA(cudaMemsetAsync(ex->flag, 0, sizeof(int), s));
    LSG_KC(LSG_K_SMALL, csr_diag(A, ex->dinv, Ain->precond ? 1 : 0, ex->flag, cb, s));
    LSG_CUDA(cudaMemcpyAsync(&bad, ex->flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    LSG_CUDA(cudaStreamSynchronize(s));
    if (bad) return set_error(LSG_BAD_ARG, "zero diagonal entry: Jacobi preconditioning undefined");
    ws->hctrl[0] = ctrl_init(prm->tol, 0);
    LSG_CUDA(cudaMemcpyAsync(ctrl, ws->hctrl, sizeof(DevCtrl), cudaMemcpyHostToDevice, s));
    LSG_CUDA(cudaMemsetAsync(DX, 0, sizeof(double) * (size_t)n * m, s));
    LSG_CUDA(cudaMemsetAsync(DF, 0, sizeof(double) * (size_t)n * m, s));
    LSG_KC(LSG_K_UPDATE, Kernels<double>::norm2(b, n, part, rb, ctrl, s));
    LSG_KC(LSG_K_SMALL, finalize_norm(part, rb, ctrl, NF_RHS, prm->tol, 0, s));
    LSG_KC(LSG_K_RESIDUAL, csr_residual(A, RES_INIT, x, b, Rv[0], nullptr, nullptr, ex->dinv, 0.0, part, cb, ctrl, s));
    int xc = 0, rcur = 0;
    auto is_anderson = [p](int it) { return it % p == 0 && it > 1; };
    auto enqueue = [&](int it) -> int {
        const int col = (it - 1) % m;
        double *dxc = DX + (size_t)col * n, *dfc = DF + (size_t)col * n;
        if (is_anderson(it)) {
            LSG_KC(LSG_K_UPDATE, csr_scale(ex->dinv, Rv[rcur], ex->f, n, rb, ctrl, s));
            LSG_KC(LSG_K_GRAM, Kernels<double>::gram(GRAM_SYM, m, DX, DF, ex->f, n, part, gb, ctrl, s));
            LSG_KC(LSG_K_SMALL, finalize_gram_solve(part, gb, GRAM_SYM, m, 1.0, ctrl, s));
            LSG_KC(LSG_K_UPDATE, Kernels<double>::aar_update(m, X[xc], ex->f, DX, dxc, prm->beta, 1.0, n, ctrl, s));
            LSG_KC(LSG_K_RESIDUAL, csr_residual(A, RES_ANDERSON, X[xc], b, Rv[rcur], dfc, dxc, ex->dinv, prm->beta,
                                                part, cb, ctrl, s));
            LSG_KC(LSG_K_SMALL, finalize_norm(part, cb, ctrl, NF_CHECK, prm->tol, it, s));
        } else {
            LSG_KC(LSG_K_RICHARDSON, csr_richardson(A, X[xc], Rv[rcur], b, X[xc ^ 1], Rv[rcur ^ 1], dxc, dfc,
                                                    ex->dinv, prm->omega, prm->beta, cb, ctrl, s));
            xc ^= 1;
            rcur ^= 1;
        }
        return LSG_OK;
    };
    rc = pipelined_loop(R, ws, 1, prm->max_iter, default_per_check(prm, n), enqueue, is_anderson);
    if (rc != LSG_OK) return rc;
    DevCtrl c;
    LSG_CUDA(cudaMemcpy(&c, ctrl, sizeof(DevCtrl), cudaMemcpyDeviceToHost));
    const int last = c.done ? c.iters : prm->max_iter;
    if (richardson_count(last, p) & 1)
        LSG_CUDA(cudaMemcpyAsync(x, X[1], sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, s));
    LSG_CUDA(cudaStreamSynchronize(s));
    R.flush();
    lsg_result tmp;
    fill_result(&tmp, c, prm->max_iter, now_s() - t0, R.launches);
    tmp.outer_iters = 0;
    tmp.inner_iters = 0;
    if (res) *res = tmp;
    set_last_status(tmp.status);
    return tmp.status;
}

int apply_csr(const lsg_csr *Ain, const double *x, double *y, cudaStream_t s) {
    CsrView A;
    int rc = csr_view(Ain, &A);
    if (rc) return rc;
    if (!x || !y) return set_error(LSG_BAD_ARG, "NULL vector");
    CsrExtra *ex = nullptr;
    rc = csr_extra(A.n, &ex);
    if (rc) return rc;
    rc = csr_validate(A, ex, s);
    if (rc) return rc;
    const int cb = (int)std::max<long long>(1, std::min<long long>(((long long)A.n * A.group + 255) / 256,
                                                                   8LL * sm_count()));
    LSG_CUDA(csr_residual(A, RES_APPLY, x, nullptr, y, nullptr, nullptr, nullptr, 0.0, nullptr, cb, nullptr, s));
    return LSG_OK;
}

int pinv(const double *A, const double *b, double *x, int m, cudaStream_t s) {
    if (m < 1 || m > LSG_MAX_M) return set_error(LSG_BAD_ARG, "m = %d outside 1..%d", m, LSG_MAX_M);
    if (!A || !b || !x) return set_error(LSG_BAD_ARG, "NULL pointer");
    int *dst = nullptr;
    LSG_CUDA(cudaMallocAsync((void **)&dst, sizeof(int), s));
    LSG_CUDA(pinv_solve_dev(A, b, x, m, dst, s));
    int st = 0;
    LSG_CUDA(cudaMemcpyAsync(&st, dst, sizeof(int), cudaMemcpyDeviceToHost, s));
    LSG_CUDA(cudaFreeAsync(dst, s));
    LSG_CUDA(cudaStreamSynchronize(s));
    return st;
}

}  // namespace lsg

// ---------------------------------------------------------------- C ABI

extern "C" {

int lsg_lap_coefficient(int radius, double *c) {
    if (radius < 1 || radius > LSG_MAX_RADIUS || !c) return lsg::set_error(LSG_BAD_ARG, "bad radius");
    return lsg::lap_coefficient(radius, c);
}

int lsg_operator_init(lsg_operator *op, int nx, int ny, int nz, int radius, double a, double sigma,
                      int precond) {
    if (!op) return lsg::set_error(LSG_BAD_ARG, "operator is NULL");
    memset(op, 0, sizeof(*op));
    op->n[0] = nx; op->n[1] = ny; op->n[2] = nz;
    op->radius = radius;
    op->a = a;
    op->sigma = sigma;
    op->precond = precond;
    int rc = lsg_lap_coefficient(radius, op->coeff);
    if (rc) return rc;
    return lsg::check_operator(op);
}

void lsg_params_default(lsg_params *prm) {
    if (!prm) return;
    memset(prm, 0, sizeof(*prm));
    prm->omega = 0.6;
    prm->beta = 0.6;
    prm->m = 7;
    prm->p = 6;
    prm->max_iter = 100000;
    prm->tol = 1e-8;
    prm->inner_tol = 3e-4;
    prm->max_outer = 50;
}

int lsg_apply(const lsg_operator *op, int dtype, const void *d_x, void *d_y, void *stream) {
    return lsg::apply(op, dtype, d_x, d_y, (cudaStream_t)stream);
}

int lsg_aar(const lsg_operator *op, const lsg_params *prm, int dtype, void *d_x, const void *d_b,
            lsg_result *res, void *stream) {
    return lsg::solve(0, op, prm, dtype, d_x, d_b, res, (cudaStream_t)stream);
}
int lsg_pgr(const lsg_operator *op, const lsg_params *prm, int dtype, void *d_x, const void *d_b,
            lsg_result *res, void *stream) {
    return lsg::solve(1, op, prm, dtype, d_x, d_b, res, (cudaStream_t)stream);
}
int lsg_pl2r(const lsg_operator *op, const lsg_params *prm, int dtype, void *d_x, const void *d_b,
             lsg_result *res, void *stream) {
    return lsg::solve(2, op, prm, dtype, d_x, d_b, res, (cudaStream_t)stream);
}
int lsg_cg(const lsg_operator *op, const lsg_params *prm, int dtype, void *d_x, const void *d_b,
           lsg_result *res, void *stream) {
    return lsg::solve(3, op, prm, dtype, d_x, d_b, res, (cudaStream_t)stream);
}
int lsg_aar_mixed(const lsg_operator *op, const lsg_params *prm, double *d_x, const double *d_b,
                  lsg_result *res, void *stream) {
    return lsg::solve_mixed(op, prm, d_x, d_b, res, (cudaStream_t)stream);
}
int lsg_aar_mixed_c(const lsg_operator *op, const lsg_params *prm, void *d_x, const void *d_b,
                    lsg_result *res, void *stream) {
    return lsg::solve_mixed_c(op, prm, d_x, d_b, res, (cudaStream_t)stream);
}
int lsg_aar_csr(const lsg_csr *A, const lsg_params *prm, double *d_x, const double *d_b, lsg_result *res,
                void *stream) {
    return lsg::solve_csr(A, prm, d_x, d_b, res, (cudaStream_t)stream);
}
int lsg_apply_csr(const lsg_csr *A, const double *d_x, double *d_y, void *stream) {
    return lsg::apply_csr(A, d_x, d_y, (cudaStream_t)stream);
}
int lsg_pinv_solve(const double *d_A, const double *d_b, double *d_x, int m, void *stream) {
    return lsg::pinv(d_A, d_b, d_x, m, (cudaStream_t)stream);
}
int lsg_release_workspaces(void) { return lsg::release_workspaces(); }
int lsg_aar_icc(const lsg_operator *op, const lsg_params *prm, const int block[3], double *d_x, const double *d_b,
                lsg_result *res, void *stream) {
    return lsg::solve_icc(op, prm, block, d_x, d_b, res, (cudaStream_t)stream);
}

int lsg_profile(int on) {
    std::lock_guard<std::mutex> g(lsg::g_prof_mu);
    if (on) memset(&lsg::g_prof, 0, sizeof(lsg::g_prof));
    lsg::g_prof_on = on != 0;
    return LSG_OK;
}

int lsg_profile_read(lsg_kernel_stats *stats) {
    if (!stats) return lsg::set_error(LSG_BAD_ARG, "NULL stats");
    std::lock_guard<std::mutex> g(lsg::g_prof_mu);
    *stats = lsg::g_prof;
    return LSG_OK;
}
int lsg_last_status(void) { return lsg::last_status(); }

int lsg_bounds_errors(long long *first_bad) {
#ifdef LSG_BOUNDS
    unsigned long long first = 0;
    for (auto read : lsg::bounds_readers()) {
        const unsigned long long v = read();
        if (v && !first) first = v;
    }
    if (first_bad) *first_bad = first ? (long long)(first - 1) : -1;
    return LSG_OK;
#else
    if (first_bad) *first_bad = -1;
    return LSG_UNSUPPORTED;
#endif
}
const char *lsg_last_error(void) { return lsg::last_error(); }

const char *lsg_status_string(int st) {
    switch (st) {
    case LSG_OK: return "ok";
    case LSG_NOT_CONVERGED: return "not converged";
    case LSG_NAN_DETECTED: return "NaN or Inf detected";
    case LSG_BAD_ARG: return "bad argument";
    case LSG_CUDA_ERROR: return "CUDA error";
    case LSG_TIMEOUT: return "device wait timed out";
    case LSG_UNSUPPORTED: return "unsupported";
    case LSG_NO_MEMORY: return "out of device memory";
    case LSG_SVD_NO_CONVERGENCE: return "SVD sweep limit reached";
    case LSG_RANGE: return "value beyond the double-float stencil range";
    default: return "unknown status";
    }
}

const char *lsg_version(void) { return "lsg 0.1 (sm_103a)"; }

int lsg_set_fp64_arith(int mode) { return lsg::g_fp64_arith.exchange(mode ? 1 : 0); }

int lsg_set_aar_form(int form) {
    if (form < 0 || form > 2) return -1;
    return lsg::g_aar_form.exchange(form);
}

}  // extern "C"
