// lsg_krylov.cu — restarted GMRES(m), the Krylov comparator the reference
// runs against AAR (PETSC_REAL/main.c:84-122: KSPGMRES, default restart 30,
// classical Gram-Schmidt, Jacobi preconditioning, rtol on the preconditioned
// residual).  PETSc is not part of this build: the algorithm is Saad and
// Schultz's GMRES(m) with left preconditioning, restated here.
//
// With the scalar Jacobi preconditioner M^-1 = cf (the stencil's diagonal is
// constant) the Arnoldi process runs on cf A.  Basis vectors are kept
// unnormalised, w_i with scale s_i = 1 / ||w_i|| held on the device, so no
// pass rewrites a vector it is reading:
//   z      = cf A (s_j w_j)                 stencil pass (weights scaled by cf)
//   h_ij   = s_i (w_i . z),  i <= j         one multi-dot pass over the basis
//   z     -= sum_i h_ij s_i w_i, ||z||^2     one update pass;  w_{j+1} = z
//   Givens rotations of the Hessenberg column and the residual estimate
//   |g_{j+1}| on one device thread; the cycle ends when |g_{j+1}| <= rtol
//   ||M^-1 b||, after m steps, at max_iter or on breakdown.
// At the end of a cycle y solves the triangular system, x += sum y_i s_i w_i,
// and the true residual r = b - A x (also the next cycle's w_0) decides
// convergence, so the reported relres is ||b - A x|| / ||b||.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>
#include <vector>

#include "lsg_kernels.cuh"
#include "lsg_host.h"

namespace lsg {

constexpr int kMaxAug = 4;  // LGMRES: error approximations kept (PETSc's default is 2)

// Slots of the error approximations used in one LGMRES cycle, newest first.
struct AugSlots {
    int slot[kMaxAug];
};

// S: double for real vectors, cplx<double> for complex ones (Hermitian
// inner products, complex Hessenberg matrix and Givens rotations).
template <typename S>
struct GmresState {
    int k;           // Arnoldi steps completed in this cycle
    int cycle_done;  // 1: this cycle has ended
    int iters;       // Arnoldi steps in total
    int pad;
    S s[LSG_MAX_M + 1];                  // basis scales: v_i = s_i w_i (|s_i| = 1 / ||w_i||)
    S coef[LSG_MAX_M + 1];               // h_ij s_i (Arnoldi), y_i s_i (cycle end)
    S H[(LSG_MAX_M + 1) * LSG_MAX_M];    // Hessenberg matrix, H[i * LSG_MAX_M + j]
    double cs[LSG_MAX_M];
    S sn[LSG_MAX_M], g[LSG_MAX_M + 1];
    S zs[kMaxAug + 1];                   // LGMRES: scales of the error approximations z = zs_l Z_l
};

template <typename S>
__device__ __forceinline__ bool cycle_over(const GmresState<S> *st, const DevCtrl *c) {
    return solve_done(c) || *(volatile const int *)&st->cycle_done;
}

// Scalar helpers shared by the real and complex forms.
__device__ __forceinline__ double sconj(double a) { return a; }
__device__ __forceinline__ cplx<double> sconj(cplx<double> a) { return conj(a); }
__device__ __forceinline__ double sabs(double a) { return fabs(a); }
__device__ __forceinline__ double sabs(cplx<double> a) { return hypot(a.x, a.y); }
__device__ __forceinline__ double sdiv(double a, double b) { return a / b; }
__device__ __forceinline__ cplx<double> sdiv(cplx<double> a, cplx<double> b) {
    const double d = b.x * b.x + b.y * b.y;
    return cplx<double>((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

// z = (cf A)(s_j w_j): the stencil input is w_j scaled by s_j, read at init.
template <typename T>
struct ArnoldiOp {
    static constexpr int NACC = 0;
    using Raw = T;
    using Ctr = NoCtr;
    const T *w;
    T *z;
    const GmresState<typename ScalarOf<T>::type> *st;
    int j;
    T scale;
    double *partials;
    const DevCtrl *ctrl;
    int zslot = -1;  // LGMRES: >= 0 when the input is error approximation zslot (scale zs)
    __device__ bool skip() const { return cycle_over(st, ctrl); }
    __device__ void init() { scale = (T)(zslot < 0 ? st->s[j] : st->zs[zslot]); }
    __device__ __forceinline__ Raw fetch(unsigned i) const { return ldg(w + i); }
    __device__ __forceinline__ T value(const Raw &v) const { return v * scale; }
    __device__ __forceinline__ Ctr fetch_center(unsigned) const { return Ctr{}; }
    __device__ __forceinline__ void store(unsigned i, T, T au, const Ctr &, Acc<T> *) const { z[i] = au; }
};

constexpr int kDotChunk = 8;

// Partial dot products w_i . z for i in chunk blockIdx.y (8 basis vectors per
// chunk, z read once per chunk).
template <typename T>
__global__ void __launch_bounds__(kReduceThreads) gmres_dots_kernel(const T *__restrict__ V, long long ld, int cnt,
                                                                    const T *__restrict__ z, long long n,
                                                                    double *partials,
                                                                    const GmresState<typename ScalarOf<T>::type> *st,
                                                                    const DevCtrl *ctrl) {
    __shared__ double red[kDotChunk * (kReduceThreads / 32) * AccWidth<T>::value];
    if (cycle_over(st, ctrl)) return;
    const int i0 = blockIdx.y * kDotChunk;
    const int nq = min(kDotChunk, cnt - i0);
    Acc<T> acc[kDotChunk];
#pragma unroll
    for (int q = 0; q < kDotChunk; q++) acc[q].zero();
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
        const T zt = ldg(z + t);
#pragma unroll
        for (int q = 0; q < kDotChunk; q++)
            if (q < nq) acc[q].add_prod(ldg(V + (long long)(i0 + q) * ld + t), zt);
    }
    block_reduce_store<kDotChunk>(acc, red,
                                  partials + ((long long)blockIdx.y * gridDim.x + blockIdx.x) * kDotChunk *
                                                 AccWidth<T>::value);
}

// Column j of H from the dot partials: h_ij = conj(s_i) (w_i^H z) = v_i^H z;
// coef_i = h_ij s_i.
template <typename S>
__global__ void gmres_fin_dots_kernel(const double *partials, int nblk, int j, GmresState<S> *st,
                                      const DevCtrl *ctrl) {
    constexpr int W = sizeof(S) / sizeof(double);
    if (cycle_over(st, ctrl)) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int i = warp; i <= j; i += nw) {
        const int c = i / kDotChunk, q = i % kDotChunk;
        double t[W];
        for (int u = 0; u < W; u++) {
            double v = 0.0;
            for (int b = lane; b < nblk; b += 32)
                v += partials[(((long long)c * nblk + b) * kDotChunk + q) * W + u];
            t[u] = warp_sum(v);
        }
        if (lane == 0) {
            S dot;
            if constexpr (W == 1) dot = t[0];
            else dot = S(t[0], t[1]);
            const S h = sconj(st->s[i]) * dot;
            st->H[i * LSG_MAX_M + j] = h;
            st->coef[i] = h * st->s[i];
        }
    }
}

// z -= sum_{i < cnt} coef_i w_i (coefficients from the state); ||z||^2 partials.
// With accumulate_x: x += sum coef_i w_i instead (cycle end), no norm.
template <typename T>
__global__ void __launch_bounds__(kReduceThreads) gmres_combine_kernel(const T *__restrict__ V, long long ld,
                                                                       int cnt, T *z, long long n,
                                                                       double *partials,
                                                                       const GmresState<typename ScalarOf<T>::type> *st,
                                                                       const DevCtrl *ctrl, int accumulate_x) {
    __shared__ double red[(kReduceThreads / 32) * AccWidth<T>::value];
    __shared__ T c[LSG_MAX_M + 1];
    if (accumulate_x ? solve_done(ctrl) : cycle_over(st, ctrl)) return;
    const int k = accumulate_x ? st->k : cnt;
    if (threadIdx.x < k) c[threadIdx.x] = (T)st->coef[threadIdx.x];
    __syncthreads();
    Acc<T> acc;
    acc.zero();
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
        T a = T(0);
        for (int i = 0; i < k; i++) a = fma(c[i], ldg(V + (long long)i * ld + t), a);
        if (accumulate_x) {
            z[t] += a;
        } else {
            const T v = z[t] - a;
            z[t] = v;
            acc.add_prod(v, v);
        }
    }
    if (!accumulate_x) {
        Acc<T> a1[1] = {acc};
        block_reduce_store<1>(a1, red, partials + blockIdx.x * AccWidth<T>::value);
    }
}

// Step j's Hessenberg column: ||z||, previous rotations, the new rotation,
// the residual estimate and the cycle-end test.
// Complex form: rotations G = [[c, s], [-conj(s), c]] with c real (c = |a| /
// rho, s = (a / |a|) b / rho for the pair (a, b = ||z||), rho = sqrt(|a|^2 + b^2)).
template <typename S>
__global__ void gmres_fin_step_kernel(const double *partials, int nblk, int j, int m, double acf,
                                      int max_iter, GmresState<S> *st, DevCtrl *ctrl) {
    constexpr int W = sizeof(S) / sizeof(double);
    __shared__ double red[32];
    if (cycle_over(st, ctrl)) return;
    double sum = 0.0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) sum += partials[(long long)b * W];
    sum = warp_sum(sum);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x != 0) return;
    double tot = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) tot += red[w];
    const double eta = sqrt(tot);
    S *H = st->H;
    H[(j + 1) * LSG_MAX_M + j] = S(eta);
    st->s[j + 1] = S(eta > 0.0 ? 1.0 / eta : 0.0);
    double r;
    if constexpr (W == 1) {
        for (int i = 0; i < j; i++) {
            const double a = H[i * LSG_MAX_M + j], b = H[(i + 1) * LSG_MAX_M + j];
            H[i * LSG_MAX_M + j] = st->cs[i] * a + st->sn[i] * b;
            H[(i + 1) * LSG_MAX_M + j] = -st->sn[i] * a + st->cs[i] * b;
        }
        const double a = H[j * LSG_MAX_M + j], b = eta;
        r = hypot(a, b);
        const double c = r > 0.0 ? a / r : 1.0, s = r > 0.0 ? b / r : 0.0;
        st->cs[j] = c;
        st->sn[j] = s;
        H[j * LSG_MAX_M + j] = r;
        H[(j + 1) * LSG_MAX_M + j] = 0.0;
        st->g[j + 1] = -s * st->g[j];
        st->g[j] = c * st->g[j];
    } else {
        for (int i = 0; i < j; i++) {
            const S a = H[i * LSG_MAX_M + j], b = H[(i + 1) * LSG_MAX_M + j];
            H[i * LSG_MAX_M + j] = st->cs[i] * a + st->sn[i] * b;
            H[(i + 1) * LSG_MAX_M + j] = st->cs[i] * b - sconj(st->sn[i]) * a;
        }
        const S a = H[j * LSG_MAX_M + j];
        const double aa = sabs(a), b = eta;
        r = hypot(aa, b);
        const S ph = aa > 0.0 ? S(a.x / aa, a.y / aa) : S(1.0, 0.0);  // a / |a|
        const double c = r > 0.0 ? aa / r : 1.0;
        const S s = r > 0.0 ? (b / r) * ph : S(0.0, 0.0);
        st->cs[j] = c;
        st->sn[j] = s;
        H[j * LSG_MAX_M + j] = r * ph;
        H[(j + 1) * LSG_MAX_M + j] = S(0.0, 0.0);
        st->g[j + 1] = -(sconj(s) * st->g[j]);
        st->g[j] = c * st->g[j];
    }
    st->k = j + 1;
    st->iters++;
    const double est = sabs(st->g[j + 1]);
    ctrl->relres = est / acf;  // estimate of ||b - A x||
    if (!isfinite(est) || !isfinite(r)) {
        ctrl->status = LSG_NAN_DETECTED;
        ctrl->done = 1;
        ctrl->iters = st->iters;
        return;
    }
    // converged estimate, m steps, iteration limit, or breakdown (w_{j+1} = 0)
    if (est <= ctrl->tol_abs * acf || j + 1 == m || st->iters >= max_iter || !(eta > 0.0)) st->cycle_done = 1;
}

// y = R^-1 g (back substitution on the rotated Hessenberg); coef_i = y_i s_i.
// LGMRES (mk < m): the steps from mk on took error approximation aug.slot[i -
// mk] as their input, so their coefficient is y_i zs_slot.
template <typename S>
__global__ void gmres_solve_y_kernel(GmresState<S> *st, const DevCtrl *ctrl, int mk, AugSlots aug) {
    if (solve_done(ctrl) || threadIdx.x != 0) return;
    const int k = st->k;
    S y[LSG_MAX_M];
    for (int i = k - 1; i >= 0; i--) {
        S t = st->g[i];
        for (int l = i + 1; l < k; l++) t = t - st->H[i * LSG_MAX_M + l] * y[l];
        const S d = st->H[i * LSG_MAX_M + i];
        y[i] = sabs(d) != 0.0 ? sdiv(t, d) : S(0.0);
    }
    for (int i = 0; i < k; i++) st->coef[i] = y[i] * (i < mk ? st->s[i] : st->zs[aug.slot[i - mk]]);
}

// LGMRES cycle end: delta = sum_{i < min(k, mk)} coef_i w_i + sum_{i >= mk}
// coef_i Z_slot(i - mk) (= W y), written to the free slot zf; x += delta;
// ||delta||^2 partials.
template <typename T>
__global__ void __launch_bounds__(kReduceThreads) lgmres_delta_kernel(const T *__restrict__ V, long long ld,
                                                                      T *Z, int mk, AugSlots aug, int zf, T *x,
                                                                      long long n, double *partials,
                                                                      const GmresState<typename ScalarOf<T>::type> *st,
                                                                      const DevCtrl *ctrl) {
    __shared__ double red[(kReduceThreads / 32) * AccWidth<T>::value];
    __shared__ T c[LSG_MAX_M + 1];
    if (solve_done(ctrl)) return;
    const int k = st->k;
    const int kv = k < mk ? k : mk;
    if (threadIdx.x < k) c[threadIdx.x] = (T)st->coef[threadIdx.x];
    __syncthreads();
    Acc<T> acc;
    acc.zero();
    T *zo = Z + (long long)zf * ld;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
        T a = T(0);
        for (int i = 0; i < kv; i++) a = fma(c[i], ldg(V + (long long)i * ld + t), a);
        for (int i = mk; i < k; i++) a = fma(c[i], ldg(Z + (long long)aug.slot[i - mk] * ld + t), a);
        zo[t] = a;
        x[t] += a;
        acc.add_prod(a, a);
    }
    Acc<T> a1[1] = {acc};
    block_reduce_store<1>(a1, red, partials + blockIdx.x * AccWidth<T>::value);
}

// zs[zf] = 1 / ||delta|| (0 for a zero update).
template <typename S>
__global__ void lgmres_znorm_kernel(const double *partials, int nblk, int zf, GmresState<S> *st,
                                    const DevCtrl *ctrl) {
    constexpr int W = sizeof(S) / sizeof(double);
    __shared__ double red[32];
    if (solve_done(ctrl)) return;
    double sum = 0.0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) sum += partials[(long long)b * W];
    sum = warp_sum(sum);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x != 0) return;
    double tot = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) tot += red[w];
    const double nd = sqrt(tot);
    st->zs[zf] = S(nd > 0.0 ? 1.0 / nd : 0.0);
}

// After r = b - A x (the new w_0): convergence on the true residual, else a
// new cycle from w_0 = r, s_0 = (cf / |cf|) / ||r|| (v_0 = cf r / ||cf r||),
// g_0 = |cf| ||r||.
template <typename S>
__global__ void gmres_restart_kernel(const double *partials, int nblk, S cf, int max_iter, GmresState<S> *st,
                                     DevCtrl *ctrl) {
    constexpr int W = sizeof(S) / sizeof(double);
    __shared__ double red[32];
    if (solve_done(ctrl)) return;
    double sum = 0.0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) sum += partials[(long long)b * W];
    sum = warp_sum(sum);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x != 0) return;
    double tot = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) tot += red[w];
    const double nr = sqrt(tot);
    ctrl->relres = nr;
    if (!isfinite(nr)) {
        ctrl->status = LSG_NAN_DETECTED;
        ctrl->done = 1;
        ctrl->iters = st->iters;
        return;
    }
    if (!(nr > ctrl->tol_abs) || st->iters >= max_iter) {
        ctrl->done = 1;
        ctrl->iters = st->iters;
        return;
    }
    const double acf = sabs(cf);
    st->s[0] = (1.0 / nr) * sdiv(cf, S(acf));
    st->g[0] = S(acf * nr);
    st->k = 0;
    st->cycle_done = 0;
}

// ---------------------------------------------------------------- host

struct GmresWs {
    std::mutex mu;
    char *base = nullptr;
    void *V = nullptr;
    long long ld = 0;
    double *partials = nullptr;
    DevCtrl *ctrl = nullptr;
    void *st = nullptr;  // GmresState<double> or GmresState<cplx<double>>
    DevCtrl *hctrl = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    ~GmresWs() {
        if (base) cudaFree(base);
        if (hctrl) cudaFreeHost(hctrl);
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
    }
};

static std::mutex g_gws_mu;
// keyed by (device, element size, doubled for complex, n, m): FP64 and
// complex64 vectors have the same size but different solver-state layouts
static std::map<std::tuple<int, size_t, long long, int>, std::unique_ptr<GmresWs>> g_gws;

int release_gmres_workspaces() {
    std::lock_guard<std::mutex> g(g_gws_mu);
    g_gws.clear();
    return LSG_OK;
}

#define LSG_GCUDA(call)                                                                      \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return cudaGetLastError(), /* clear it for later launches */                     \
                   set_error(e_ == cudaErrorMemoryAllocation ? LSG_NO_MEMORY : LSG_CUDA_ERROR, \
                             "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

// aug > 0: LGMRES(m, aug) -- each cycle runs m - aug Krylov steps and then one
// step on each of the last min(cycles, aug) error approximations (newest
// first), kept in aug + 1 slots Z after the basis.
template <typename T>
static int gmres_t(const lsg_operator *op, const lsg_params *prm, T *x, const T *b, lsg_result *res,
                   cudaStream_t s, int aug = 0) {
    using S = typename ScalarOf<T>::type;
    using State = GmresState<S>;
    const double t0 = std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
    const Geom g = make_geom(op->n);
    const long long n = g.n;
    const int m = prm->m;
    const int sms = sm_count();
    const int rb = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 4LL * sms));
    const int nchunk = (m + 1 + kDotChunk - 1) / kDotChunk;
    StencilLaunch L{g, choose_lz<T>(g, sms * Kernels<T>::stencil_blocks_per_sm()), s};
    L.exact = fp64_exact_for(prm->tol);
    const long long sb = stencil_blocks<T>(g, L.lz);
    int dev = 0;
    cudaGetDevice(&dev);
    GmresWs *ws;
    {
        std::lock_guard<std::mutex> gl(g_gws_mu);
        auto &slot = g_gws[std::make_tuple(dev, (size_t)(sizeof(T) * (IsCplx<T>::value ? 2 : 1)), n, m | (aug << 8))];
        if (!slot) slot.reset(new GmresWs());
        ws = slot.get();
    }
    std::unique_lock<std::mutex> lk(ws->mu);
    if (!ws->base) {
        const long long ld = (long long)((((size_t)n * sizeof(T) + 255) & ~(size_t)255) / sizeof(T));
        const long long pcap = std::max<long long>((long long)rb * nchunk * kDotChunk, sb) * AccWidth<T>::value;
        const size_t vbytes = (size_t)ld * sizeof(T) * (size_t)(m + 1 + (aug > 0 ? aug + 1 : 0));
        const size_t pbytes = ((size_t)pcap * 8 + 255) & ~(size_t)255;
        const size_t cbytes = (sizeof(DevCtrl) + 255) & ~(size_t)255;
        cudaError_t e = cudaMalloc(&ws->base, vbytes + pbytes + cbytes + sizeof(State));
        if (e != cudaSuccess) {
            cudaGetLastError();
            ws->base = nullptr;
            return set_error(LSG_NO_MEMORY, "GMRES work arrays: %s", cudaGetErrorString(e));
        }
        ws->V = ws->base;
        ws->ld = ld;
        ws->partials = (double *)(ws->base + vbytes);
        ws->ctrl = (DevCtrl *)(ws->base + vbytes + pbytes);
        ws->st = ws->base + vbytes + pbytes + cbytes;
        LSG_GCUDA(cudaMallocHost(&ws->hctrl, 2 * sizeof(DevCtrl)));
        LSG_GCUDA(cudaEventCreateWithFlags(&ws->ev[0], cudaEventDisableTiming));
        LSG_GCUDA(cudaEventCreateWithFlags(&ws->ev[1], cudaEventDisableTiming));
    }
    T *V = (T *)ws->V;
    const long long ld = ws->ld;
    DevCtrl *ctrl = ws->ctrl;
    State *st = (State *)ws->st;
    double *part = ws->partials;
    const Weights<T> w = make_weights<T>(op);
    const S cf = jacobi_factor<T>(op);
    Weights<T> wcf = w;  // weights of cf A
    for (int p = 0; p <= op->radius; p++) wcf.w[p] = (T)(cf * (S)w.w[p]);
    refresh_df_weights(wcf);
    double acf;
    if constexpr (IsCplx<T>::value) acf = std::hypot(cf.x, cf.y);
    else acf = std::fabs(cf);
    long long launches = 0;

    ws->hctrl[0] = ctrl_init(prm->tol, 0);
    LSG_GCUDA(cudaMemcpyAsync(ctrl, ws->hctrl, sizeof(DevCtrl), cudaMemcpyHostToDevice, s));
    LSG_GCUDA(cudaMemsetAsync(st, 0, sizeof(State), s));
    auto chk = [&](cudaError_t e) -> int {
        launches++;
        return e == cudaSuccess ? LSG_OK : set_error(LSG_CUDA_ERROR, "GMRES launch: %s", cudaGetErrorString(e));
    };
#define LSG_GK(call) do { int rc_ = chk(call); if (rc_) return rc_; } while (0)
    LSG_GK(Kernels<T>::norm2(b, n, part, rb, ctrl, s));
    LSG_GK(finalize_norm(part, rb, ctrl, NF_RHS, prm->tol, 0, s, AccWidth<T>::value));
    auto restart = [&]() -> int {
        LSG_GK(Kernels<T>::residual(L, w, RES_INIT, x, b, V, nullptr, nullptr, 1.0, 0.0, part, ctrl));
        gmres_restart_kernel<S><<<1, 256, 0, s>>>(part, (int)sb, cf, prm->max_iter, st, ctrl);
        LSG_GK(cudaGetLastError());
        return LSG_OK;
    };
    int rc = restart();
    if (rc) return rc;
    // LGMRES: the error approximations' slots, newest first
    T *Z = V + (long long)(m + 1) * ld;
    const int mk = m - aug;
    std::vector<int> zorder;
    auto cycle = [&](int) -> int {
        const int na = std::min((int)zorder.size(), aug);
        const int steps = mk + na;
        AugSlots as{};
        for (int l = 0; l < na; l++) as.slot[l] = zorder[l];
        for (int j = 0; j < steps; j++) {
            T *wj = V + (long long)j * ld, *z = V + (long long)(j + 1) * ld;
            ArnoldiOp<T> aop{wj, z, st, j, T(0), nullptr, ctrl};
            if (j >= mk) {
                aop.w = Z + (long long)as.slot[j - mk] * ld;
                aop.zslot = as.slot[j - mk];
            }
            LSG_GK(launch_stencil<T>(L, wcf, aop));
            const int nc = (j + 1 + kDotChunk - 1) / kDotChunk;
            gmres_dots_kernel<T><<<dim3(rb, nc), kReduceThreads, 0, s>>>(V, ld, j + 1, z, n, part, st, ctrl);
            LSG_GK(cudaGetLastError());
            gmres_fin_dots_kernel<S><<<1, 256, 0, s>>>(part, rb, j, st, ctrl);
            LSG_GK(cudaGetLastError());
            gmres_combine_kernel<T><<<rb, kReduceThreads, 0, s>>>(V, ld, j + 1, z, n, part, st, ctrl, 0);
            LSG_GK(cudaGetLastError());
            gmres_fin_step_kernel<S><<<1, 256, 0, s>>>(part, rb, j, steps, acf, prm->max_iter, st, ctrl);
            LSG_GK(cudaGetLastError());
        }
        gmres_solve_y_kernel<S><<<1, 32, 0, s>>>(st, ctrl, aug > 0 ? mk : m + 1, as);
        LSG_GK(cudaGetLastError());
        if (aug > 0) {
            // x += W y, kept (scaled to unit norm) as the newest error approximation
            int zf = 0;
            while (std::find(zorder.begin(), zorder.begin() + na, zf) != zorder.begin() + na) zf++;
            lgmres_delta_kernel<T><<<rb, kReduceThreads, 0, s>>>(V, ld, Z, mk, as, zf, x, n, part, st, ctrl);
            LSG_GK(cudaGetLastError());
            lgmres_znorm_kernel<S><<<1, 256, 0, s>>>(part, rb, zf, st, ctrl);
            LSG_GK(cudaGetLastError());
            zorder.insert(zorder.begin(), zf);
            if ((int)zorder.size() > aug) zorder.resize(aug);
        } else {
            gmres_combine_kernel<T><<<rb, kReduceThreads, 0, s>>>(V, ld, m, x, n, part, st, ctrl, 1);
            LSG_GK(cudaGetLastError());
        }
        return restart();
    };
#undef LSG_GK
    // one cycle per "iteration" of the pipelined loop, convergence read every cycle
    int c = 0, batch = 0;
    const int max_cycles = prm->max_iter / std::max(1, m - aug) + 2;
    bool stop = false;
    while (!stop) {
        rc = cycle(c++);
        if (rc) return rc;
        const int slot = batch & 1;
        LSG_GCUDA(cudaMemcpyAsync(ws->hctrl + slot, ctrl, sizeof(DevCtrl), cudaMemcpyDeviceToHost, s));
        LSG_GCUDA(cudaEventRecord(ws->ev[slot], s));
        if (batch > 0) {
            LSG_GCUDA(cudaEventSynchronize(ws->ev[slot ^ 1]));
            if (ws->hctrl[slot ^ 1].done) stop = true;
        }
        if (c >= max_cycles) stop = true;
        batch++;
    }
    LSG_GCUDA(cudaStreamSynchronize(s));
    DevCtrl hc;
    State hs;
    LSG_GCUDA(cudaMemcpy(&hc, ctrl, sizeof(DevCtrl), cudaMemcpyDeviceToHost));
    LSG_GCUDA(cudaMemcpy(&hs, st, sizeof(State), cudaMemcpyDeviceToHost));
    lsg_result r;
    memset(&r, 0, sizeof(r));
    r.iters = hc.done ? hc.iters : hs.iters;
    r.rhs_norm = hc.rhs_norm;
    r.relres = hc.rhs_norm > 0 ? hc.relres / hc.rhs_norm : hc.relres;
    if (hc.status == LSG_NAN_DETECTED) r.status = LSG_NAN_DETECTED;
    else if (hc.df_range) r.status = LSG_RANGE;
    else if (hc.done && !(hc.relres > hc.tol_abs)) r.status = LSG_OK;
    else r.status = LSG_NOT_CONVERGED;
    r.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count() - t0;
    r.launches = launches;
    if (res) *res = r;
    set_last_status(r.status);
    return r.status;
}

// ---------------------------------------------------------------- COCG (BiCG on complex-symmetric A)
//
// The reference runs PETSc's KSPBICG on its complex shifted operator
// (PETSC_COMPLEX/main.c:150-175).  A = a Lap + sigma I is complex symmetric
// (A^T = A), and BiCG started with the shadow residual conj(r_0) keeps every
// shadow iterate the conjugate of the primal one, so it reduces to conjugate
// orthogonal CG (van der Vorst & Melissen 1990): CG with the bilinear form
// u^T v, one operator application per step.  Jacobi preconditioned (complex
// cf); convergence on ||r||_2 / ||b||_2 every step.

struct CocgState {
    cplx<double> alpha, beta, rho;
};

// d = cf r + beta d_old at every stencil point, q = A d, partial d^T q.
template <typename T>
struct CocgDirOp {
    static constexpr int NACC = 1;
    using Raw = Pair<T>;  // (r, d_old)
    using Ctr = NoCtr;
    const T *r;
    const T *d_old;
    T *d_new;
    T *q;
    T cf;
    T beta;
    double *partials;
    const DevCtrl *ctrl;
    const CocgState *st;
    __device__ bool skip() const { return solve_done(ctrl); }
    __device__ void init() { beta = T(st->beta); }
    __device__ __forceinline__ Raw fetch(unsigned i) const { return Raw{ldg(r + i), ldg(d_old + i)}; }
    __device__ __forceinline__ T value(const Raw &v) const { return fma(beta, v.b, cf * v.a); }
    __device__ __forceinline__ Ctr fetch_center(unsigned) const { return Ctr{}; }
    __device__ __forceinline__ void store(unsigned i, T u, T au, const Ctr &, Acc<T> *acc) const {
        d_new[i] = u;
        q[i] = au;
        acc[0].add_prod(conj(u), au);  // the accumulator conjugates its first factor: u^T q
    }
};

// x += alpha d; r -= alpha q; partials (||r||^2, r^T r) per block (4 reals).
template <typename T>
__global__ void __launch_bounds__(kReduceThreads) cocg_step_kernel(T *__restrict__ x, T *__restrict__ r,
                                                                   const T *__restrict__ d,
                                                                   const T *__restrict__ q, long long n,
                                                                   double *partials, const CocgState *st,
                                                                   const DevCtrl *ctrl) {
    __shared__ double red[2 * (kReduceThreads / 32) * 2];
    if (solve_done(ctrl)) return;
    const T alpha = T(st->alpha);
    Acc<T> acc[2];
    acc[0].zero();
    acc[1].zero();
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        x[i] = fma(alpha, ldg(d + i), x[i]);
        const T rn = fma(-alpha, ldg(q + i), r[i]);
        r[i] = rn;
        acc[0].add_prod(rn, rn);        // |r|^2 (real part)
        acc[1].add_prod(conj(rn), rn);  // r^T r
    }
    block_reduce_store<2>(acc, red, partials + (long long)blockIdx.x * 4);
}

__device__ __forceinline__ double cocg_sum(const double *partials, int nblk, int stride, int off, double *red) {
    double t = 0.0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) t += partials[(long long)b * stride + off];
    t = warp_sum(t);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
    __syncthreads();
    double tot = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) tot += red[w];
    __syncthreads();
    return tot;
}

__device__ __forceinline__ cplx<double> cdiv(cplx<double> a, cplx<double> b) {
    const double d = b.x * b.x + b.y * b.y;
    return cplx<double>((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

// alpha = rho / (d^T q).
__global__ void cocg_alpha_kernel(const double *partials, int nblk, CocgState *st, DevCtrl *ctrl, int iter) {
    __shared__ double red[32];
    if (solve_done(ctrl)) return;
    const double re = cocg_sum(partials, nblk, 2, 0, red);
    const double im = cocg_sum(partials, nblk, 2, 1, red);
    if (threadIdx.x != 0) return;
    st->alpha = cdiv(st->rho, cplx<double>(re, im));
    if (!isfinite(st->alpha.x) || !isfinite(st->alpha.y)) {
        ctrl->status = LSG_NAN_DETECTED;
        ctrl->done = 1;
        ctrl->iters = iter;
    }
}

// After the update of step `iter` (0: the initial residual): ||r||, rho_new =
// cf r^T r, beta = rho_new / rho, convergence.
__global__ void cocg_fin_kernel(const double *partials, int nblk, CocgState *st, DevCtrl *ctrl, cplx<double> cf,
                                int iter, int max_iter) {
    __shared__ double red[32];
    if (solve_done(ctrl)) return;
    const double nn = cocg_sum(partials, nblk, 4, 0, red);
    const double re = cocg_sum(partials, nblk, 4, 2, red);
    const double im = cocg_sum(partials, nblk, 4, 3, red);
    if (threadIdx.x != 0) return;
    const cplx<double> rho_new = cf * cplx<double>(re, im);
    st->beta = iter == 0 ? cplx<double>(0.0, 0.0) : cdiv(rho_new, st->rho);
    st->rho = rho_new;
    const double nr = sqrt(nn);
    ctrl->relres = nr;
    if (!isfinite(nr)) {
        ctrl->status = LSG_NAN_DETECTED;
        ctrl->done = 1;
        ctrl->iters = iter;
    } else if (!(nr > ctrl->tol_abs) || iter >= max_iter) {
        ctrl->done = 1;
        ctrl->iters = iter;
    }
}

template <typename T>
static int cocg_t(const lsg_operator *op, const lsg_params *prm, T *x, const T *b, lsg_result *res,
                  cudaStream_t s) {
    const double t0 = std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
    const Geom g = make_geom(op->n);
    const long long n = g.n;
    const int sms = sm_count();
    const int rb = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 4LL * sms));
    StencilLaunch L{g, choose_lz<T>(g, sms * Kernels<T>::stencil_blocks_per_sm()), s};
    const long long sb = stencil_blocks<T>(g, L.lz);
    int dev = 0;
    cudaGetDevice(&dev);
    GmresWs *ws;
    const int mcols = 3;  // r, d ping-pong and q in the basis storage
    {
        std::lock_guard<std::mutex> gl(g_gws_mu);
        auto &slot = g_gws[std::make_tuple(dev, (size_t)(sizeof(T) * (IsCplx<T>::value ? 2 : 1)), n, -mcols)];
        if (!slot) slot.reset(new GmresWs());
        ws = slot.get();
    }
    std::unique_lock<std::mutex> lk(ws->mu);
    if (!ws->base) {
        const long long ld = (long long)((((size_t)n * sizeof(T) + 255) & ~(size_t)255) / sizeof(T));
        const long long pcap = std::max<long long>((long long)rb * 4, sb * 2);
        const size_t vbytes = (size_t)ld * sizeof(T) * (size_t)(mcols + 1);
        const size_t pbytes = ((size_t)pcap * 8 + 255) & ~(size_t)255;
        const size_t cbytes = (sizeof(DevCtrl) + 255) & ~(size_t)255;
        cudaError_t e = cudaMalloc(&ws->base, vbytes + pbytes + cbytes + sizeof(CocgState));
        if (e != cudaSuccess) {
            cudaGetLastError();
            ws->base = nullptr;
            return set_error(LSG_NO_MEMORY, "COCG work arrays: %s", cudaGetErrorString(e));
        }
        ws->V = ws->base;
        ws->ld = ld;
        ws->partials = (double *)(ws->base + vbytes);
        ws->ctrl = (DevCtrl *)(ws->base + vbytes + pbytes);
        ws->st = ws->base + vbytes + pbytes + cbytes;
        LSG_GCUDA(cudaMallocHost(&ws->hctrl, 2 * sizeof(DevCtrl)));
        LSG_GCUDA(cudaEventCreateWithFlags(&ws->ev[0], cudaEventDisableTiming));
        LSG_GCUDA(cudaEventCreateWithFlags(&ws->ev[1], cudaEventDisableTiming));
    }
    T *V = (T *)ws->V;
    const long long ld = ws->ld;
    T *r = V, *D[2] = {V + ld, V + 2 * ld}, *q = V + 3 * ld;
    DevCtrl *ctrl = ws->ctrl;
    CocgState *st = (CocgState *)ws->st;
    double *part = ws->partials;
    const Weights<T> w = make_weights<T>(op);
    const cplx<double> cf = jacobi_factor<T>(op);
    long long launches = 0;
    ws->hctrl[0] = ctrl_init(prm->tol, 0);
    LSG_GCUDA(cudaMemcpyAsync(ctrl, ws->hctrl, sizeof(DevCtrl), cudaMemcpyHostToDevice, s));
    LSG_GCUDA(cudaMemsetAsync(st, 0, sizeof(CocgState), s));
    LSG_GCUDA(cudaMemsetAsync(D[0], 0, sizeof(T) * (size_t)ld * 2, s));  // d and the other d buffer
    LSG_GCUDA(cudaMemsetAsync(q, 0, sizeof(T) * (size_t)n, s));
    auto chk = [&](cudaError_t e) -> int {
        launches++;
        return e == cudaSuccess ? LSG_OK : set_error(LSG_CUDA_ERROR, "COCG launch: %s", cudaGetErrorString(e));
    };
#define LSG_CK(call) do { int rc_ = chk(call); if (rc_) return rc_; } while (0)
    LSG_CK(Kernels<T>::norm2(b, n, part, rb, ctrl, s));
    LSG_CK(finalize_norm(part, rb, ctrl, NF_RHS, prm->tol, 0, s, 2));
    LSG_CK(Kernels<T>::residual(L, w, RES_INIT, x, b, r, nullptr, nullptr, cplx<double>(1.0, 0.0), 0.0, part, ctrl));
    // with alpha = 0 the step kernel only measures ||r||^2 and r^T r
    cocg_step_kernel<T><<<rb, kReduceThreads, 0, s>>>(x, r, D[0], q, n, part, st, ctrl);
    LSG_CK(cudaGetLastError());
    cocg_fin_kernel<<<1, 256, 0, s>>>(part, rb, st, ctrl, cf, 0, prm->max_iter);
    LSG_CK(cudaGetLastError());
    int cur = 0, it = 0, batch = 0;
    bool stop = prm->max_iter <= 0;
    const int per = prm->check_every > 0 ? prm->check_every : (n >= (1LL << 21) ? 8 : 32);
    while (!stop) {
        for (int k = 0; k < per && it < prm->max_iter; k++) {
            it++;
            CocgDirOp<T> op2{r, D[cur], D[cur ^ 1], q, T(cf), T(0.0), part, ctrl, st};
            LSG_CK(launch_stencil<T>(L, w, op2));
            cur ^= 1;
            cocg_alpha_kernel<<<1, 256, 0, s>>>(part, (int)sb, st, ctrl, it);
            LSG_CK(cudaGetLastError());
            cocg_step_kernel<T><<<rb, kReduceThreads, 0, s>>>(x, r, D[cur], q, n, part, st, ctrl);
            LSG_CK(cudaGetLastError());
            cocg_fin_kernel<<<1, 256, 0, s>>>(part, rb, st, ctrl, cf, it, prm->max_iter);
            LSG_CK(cudaGetLastError());
        }
        const int slot = batch & 1;
        LSG_GCUDA(cudaMemcpyAsync(ws->hctrl + slot, ctrl, sizeof(DevCtrl), cudaMemcpyDeviceToHost, s));
        LSG_GCUDA(cudaEventRecord(ws->ev[slot], s));
        if (batch > 0) {
            LSG_GCUDA(cudaEventSynchronize(ws->ev[slot ^ 1]));
            if (ws->hctrl[slot ^ 1].done) stop = true;
        }
        if (it >= prm->max_iter) stop = true;
        batch++;
    }
#undef LSG_CK
    LSG_GCUDA(cudaStreamSynchronize(s));
    DevCtrl hc;
    LSG_GCUDA(cudaMemcpy(&hc, ctrl, sizeof(DevCtrl), cudaMemcpyDeviceToHost));
    lsg_result rr;
    memset(&rr, 0, sizeof(rr));
    rr.iters = hc.done ? hc.iters : prm->max_iter;
    rr.rhs_norm = hc.rhs_norm;
    rr.relres = hc.rhs_norm > 0 ? hc.relres / hc.rhs_norm : hc.relres;
    if (hc.status == LSG_NAN_DETECTED) rr.status = LSG_NAN_DETECTED;
    else if (hc.done && !(hc.relres > hc.tol_abs)) rr.status = LSG_OK;
    else rr.status = LSG_NOT_CONVERGED;
    rr.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count() - t0;
    rr.launches = launches;
    if (res) *res = rr;
    set_last_status(rr.status);
    return rr.status;
}

int cocg(const lsg_operator *op, const lsg_params *prm, int dtype, void *d_x, const void *d_b, lsg_result *res,
         cudaStream_t s) {
    int rc = check_operator(op);
    if (rc) return rc;
    rc = check_params(prm, false);
    if (rc) return rc;
    if (!d_x || !d_b) return set_error(LSG_BAD_ARG, "NULL vector");
    if (dtype == LSG_C128)
        return cocg_t<cplx<double>>(op, prm, (cplx<double> *)d_x, (const cplx<double> *)d_b, res, s);
    if (dtype == LSG_C64) return cocg_t<cplx<float>>(op, prm, (cplx<float> *)d_x, (const cplx<float> *)d_b, res, s);
    return set_error(LSG_UNSUPPORTED, "COCG: complex vectors only (real symmetric problems: lsg_cg)");
}

int gmres(const lsg_operator *op, const lsg_params *prm, int dtype, void *d_x, const void *d_b, lsg_result *res,
          cudaStream_t s, int aug) {
    int rc = check_operator(op);
    if (rc) return rc;
    rc = check_params(prm, true);
    if (rc) return rc;
    if (!d_x || !d_b) return set_error(LSG_BAD_ARG, "NULL vector");
    if (aug < 0 || aug > kMaxAug || (aug > 0 && aug >= prm->m))
        return set_error(LSG_BAD_ARG, "LGMRES: augmentation %d outside 1..min(%d, m - 1)", aug, kMaxAug);
    if (dtype == LSG_F64) return gmres_t<double>(op, prm, (double *)d_x, (const double *)d_b, res, s, aug);
    if (dtype == LSG_F32) return gmres_t<float>(op, prm, (float *)d_x, (const float *)d_b, res, s, aug);
    if (dtype == LSG_C128)
        return gmres_t<cplx<double>>(op, prm, (cplx<double> *)d_x, (const cplx<double> *)d_b, res, s, aug);
    if (dtype == LSG_C64)
        return gmres_t<cplx<float>>(op, prm, (cplx<float> *)d_x, (const cplx<float> *)d_b, res, s, aug);
    return set_error(LSG_BAD_ARG, "GMRES: unknown dtype %d", dtype);
}

}  // namespace lsg

extern "C" int lsg_gmres(const lsg_operator *op, const lsg_params *prm, int dtype, void *d_x, const void *d_b,
                         lsg_result *res, void *stream) {
    return lsg::gmres(op, prm, dtype, d_x, d_b, res, (cudaStream_t)stream, 0);
}

extern "C" int lsg_lgmres(const lsg_operator *op, const lsg_params *prm, int aug, int dtype, void *d_x,
                          const void *d_b, lsg_result *res, void *stream) {
    return lsg::gmres(op, prm, dtype, d_x, d_b, res, (cudaStream_t)stream, aug);
}

extern "C" int lsg_cocg(const lsg_operator *op, const lsg_params *prm, int dtype, void *d_x, const void *d_b,
                        lsg_result *res, void *stream) {
    return lsg::cocg(op, prm, dtype, d_x, d_b, res, (cudaStream_t)stream);
}
