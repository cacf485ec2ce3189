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

#include "lsg_kernels.cuh"
#include "lsg_host.h"

namespace lsg {

struct GmresState {
    int k;           // Arnoldi steps completed in this cycle
    int cycle_done;  // 1: this cycle has ended
    int iters;       // Arnoldi steps in total
    int pad;
    double s[LSG_MAX_M + 1];                  // 1 / ||w_i||
    double coef[LSG_MAX_M + 1];               // h_ij s_i (Arnoldi), y_i s_i (cycle end)
    double H[(LSG_MAX_M + 1) * LSG_MAX_M];    // Hessenberg matrix, H[i * LSG_MAX_M + j]
    double cs[LSG_MAX_M], sn[LSG_MAX_M], g[LSG_MAX_M + 1];
};

__device__ __forceinline__ bool cycle_over(const GmresState *st, const DevCtrl *c) {
    return solve_done(c) || *(volatile const int *)&st->cycle_done;
}

// z = (cf A)(s_j w_j): the stencil input is w_j scaled by s_j, read at init.
template <typename T>
struct ArnoldiOp {
    static constexpr int NACC = 0;
    using Raw = T;
    using Ctr = NoCtr;
    const T *w;
    T *z;
    const GmresState *st;
    int j;
    T scale;
    double *partials;
    const DevCtrl *ctrl;
    __device__ bool skip() const { return cycle_over(st, ctrl); }
    __device__ void init() { scale = (T)st->s[j]; }
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
                                                                    double *partials, const GmresState *st,
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
                                  partials + ((long long)blockIdx.y * gridDim.x + blockIdx.x) * kDotChunk);
}

// Column j of H from the dot partials; coef_i = h_ij s_i.
__global__ void gmres_fin_dots_kernel(const double *partials, int nblk, int j, GmresState *st,
                                      const DevCtrl *ctrl) {
    if (cycle_over(st, ctrl)) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int i = warp; i <= j; i += nw) {
        const int c = i / kDotChunk, q = i % kDotChunk;
        double t = 0.0;
        for (int b = lane; b < nblk; b += 32) t += partials[((long long)c * nblk + b) * kDotChunk + q];
        t = warp_sum(t);
        if (lane == 0) {
            const double h = st->s[i] * t;
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
                                                                       double *partials, const GmresState *st,
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
__global__ void gmres_fin_step_kernel(const double *partials, int nblk, int j, int m, double acf,
                                      int max_iter, GmresState *st, DevCtrl *ctrl) {
    __shared__ double red[32];
    if (cycle_over(st, ctrl)) return;
    double sum = 0.0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) sum += partials[b];
    sum = warp_sum(sum);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x != 0) return;
    double tot = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) tot += red[w];
    const double eta = sqrt(tot);
    double *H = st->H;
    H[(j + 1) * LSG_MAX_M + j] = eta;
    st->s[j + 1] = eta > 0.0 ? 1.0 / eta : 0.0;
    for (int i = 0; i < j; i++) {
        const double a = H[i * LSG_MAX_M + j], b = H[(i + 1) * LSG_MAX_M + j];
        H[i * LSG_MAX_M + j] = st->cs[i] * a + st->sn[i] * b;
        H[(i + 1) * LSG_MAX_M + j] = -st->sn[i] * a + st->cs[i] * b;
    }
    const double a = H[j * LSG_MAX_M + j], b = eta;
    const double r = hypot(a, b);
    const double c = r > 0.0 ? a / r : 1.0, s = r > 0.0 ? b / r : 0.0;
    st->cs[j] = c;
    st->sn[j] = s;
    H[j * LSG_MAX_M + j] = r;
    H[(j + 1) * LSG_MAX_M + j] = 0.0;
    st->g[j + 1] = -s * st->g[j];
    st->g[j] = c * st->g[j];
    st->k = j + 1;
    st->iters++;
    const double est = fabs(st->g[j + 1]);
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
__global__ void gmres_solve_y_kernel(GmresState *st, const DevCtrl *ctrl) {
    if (solve_done(ctrl) || threadIdx.x != 0) return;
    const int k = st->k;
    double y[LSG_MAX_M];
    for (int i = k - 1; i >= 0; i--) {
        double t = st->g[i];
        for (int l = i + 1; l < k; l++) t -= st->H[i * LSG_MAX_M + l] * y[l];
        const double d = st->H[i * LSG_MAX_M + i];
        y[i] = d != 0.0 ? t / d : 0.0;
    }
    for (int i = 0; i < k; i++) st->coef[i] = y[i] * st->s[i];
}

// After r = b - A x (the new w_0): convergence on the true residual, else a
// new cycle from w_0 = r, s_0 = sign(cf) / ||r||, g_0 = |cf| ||r||.
__global__ void gmres_restart_kernel(const double *partials, int nblk, double cf, int max_iter, GmresState *st,
                                     DevCtrl *ctrl) {
    __shared__ double red[32];
    if (solve_done(ctrl)) return;
    double sum = 0.0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) sum += partials[b];
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
    st->s[0] = (cf < 0 ? -1.0 : 1.0) / nr;
    st->g[0] = fabs(cf) * nr;
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
    GmresState *st = nullptr;
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
            return set_error(e_ == cudaErrorMemoryAllocation ? LSG_NO_MEMORY : LSG_CUDA_ERROR, \
                             "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

template <typename T>
static int gmres_t(const lsg_operator *op, const lsg_params *prm, T *x, const T *b, lsg_result *res,
                   cudaStream_t s) {
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
        auto &slot = g_gws[std::make_tuple(dev, sizeof(T), n, m)];
        if (!slot) slot.reset(new GmresWs());
        ws = slot.get();
    }
    std::unique_lock<std::mutex> lk(ws->mu);
    if (!ws->base) {
        const long long ld = (long long)((((size_t)n * sizeof(T) + 255) & ~(size_t)255) / sizeof(T));
        const long long pcap = std::max<long long>((long long)rb * nchunk * kDotChunk, sb) * AccWidth<T>::value;
        const size_t vbytes = (size_t)ld * sizeof(T) * (size_t)(m + 1);
        const size_t pbytes = ((size_t)pcap * 8 + 255) & ~(size_t)255;
        const size_t cbytes = (sizeof(DevCtrl) + 255) & ~(size_t)255;
        cudaError_t e = cudaMalloc(&ws->base, vbytes + pbytes + cbytes + sizeof(GmresState));
        if (e != cudaSuccess) {
            cudaGetLastError();
            ws->base = nullptr;
            return set_error(LSG_NO_MEMORY, "GMRES work arrays: %s", cudaGetErrorString(e));
        }
        ws->V = ws->base;
        ws->ld = ld;
        ws->partials = (double *)(ws->base + vbytes);
        ws->ctrl = (DevCtrl *)(ws->base + vbytes + pbytes);
        ws->st = (GmresState *)(ws->base + vbytes + pbytes + cbytes);
        LSG_GCUDA(cudaMallocHost(&ws->hctrl, 2 * sizeof(DevCtrl)));
        LSG_GCUDA(cudaEventCreateWithFlags(&ws->ev[0], cudaEventDisableTiming));
        LSG_GCUDA(cudaEventCreateWithFlags(&ws->ev[1], cudaEventDisableTiming));
    }
    T *V = (T *)ws->V;
    const long long ld = ws->ld;
    DevCtrl *ctrl = ws->ctrl;
    GmresState *st = ws->st;
    double *part = ws->partials;
    const Weights<T> w = make_weights<T>(op);
    const double cf = op->precond ? 1.0 / jacobi_diag(op) : 1.0;
    Weights<T> wcf = w;  // weights of cf A
    for (int p = 0; p <= op->radius; p++) wcf.w[p] = (T)(cf * (double)w.w[p]);
    refresh_df_weights(wcf);
    const double acf = std::fabs(cf);
    long long launches = 0;

    ws->hctrl[0] = ctrl_init(prm->tol, 0);
    LSG_GCUDA(cudaMemcpyAsync(ctrl, ws->hctrl, sizeof(DevCtrl), cudaMemcpyHostToDevice, s));
    LSG_GCUDA(cudaMemsetAsync(st, 0, sizeof(GmresState), s));
    auto chk = [&](cudaError_t e) -> int {
        launches++;
        return e == cudaSuccess ? LSG_OK : set_error(LSG_CUDA_ERROR, "GMRES launch: %s", cudaGetErrorString(e));
    };
#define LSG_GK(call) do { int rc_ = chk(call); if (rc_) return rc_; } while (0)
    LSG_GK(Kernels<T>::norm2(b, n, part, rb, ctrl, s));
    LSG_GK(finalize_norm(part, rb, ctrl, NF_RHS, prm->tol, 0, s));
    auto restart = [&]() -> int {
        LSG_GK(Kernels<T>::residual(L, w, RES_INIT, x, b, V, nullptr, nullptr, 1.0, 0.0, part, ctrl));
        gmres_restart_kernel<<<1, 256, 0, s>>>(part, (int)sb, cf, prm->max_iter, st, ctrl);
        LSG_GK(cudaGetLastError());
        return LSG_OK;
    };
    int rc = restart();
    if (rc) return rc;
    auto cycle = [&](int) -> int {
        for (int j = 0; j < m; j++) {
            T *wj = V + (long long)j * ld, *z = V + (long long)(j + 1) * ld;
            ArnoldiOp<T> aop{wj, z, st, j, T(0), nullptr, ctrl};
            LSG_GK(launch_stencil<T>(L, wcf, aop));
            const int nc = (j + 1 + kDotChunk - 1) / kDotChunk;
            gmres_dots_kernel<T><<<dim3(rb, nc), kReduceThreads, 0, s>>>(V, ld, j + 1, z, n, part, st, ctrl);
            LSG_GK(cudaGetLastError());
            gmres_fin_dots_kernel<<<1, 256, 0, s>>>(part, rb, j, st, ctrl);
            LSG_GK(cudaGetLastError());
            gmres_combine_kernel<T><<<rb, kReduceThreads, 0, s>>>(V, ld, j + 1, z, n, part, st, ctrl, 0);
            LSG_GK(cudaGetLastError());
            gmres_fin_step_kernel<<<1, 256, 0, s>>>(part, rb, j, m, acf, prm->max_iter, st, ctrl);
            LSG_GK(cudaGetLastError());
        }
        gmres_solve_y_kernel<<<1, 32, 0, s>>>(st, ctrl);
        LSG_GK(cudaGetLastError());
        gmres_combine_kernel<T><<<rb, kReduceThreads, 0, s>>>(V, ld, m, x, n, part, st, ctrl, 1);
        LSG_GK(cudaGetLastError());
        return restart();
    };
#undef LSG_GK
    // one cycle per "iteration" of the pipelined loop, convergence read every cycle
    int c = 0, batch = 0;
    const int max_cycles = prm->max_iter / std::max(1, m) + 2;
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
    GmresState hs;
    LSG_GCUDA(cudaMemcpy(&hc, ctrl, sizeof(DevCtrl), cudaMemcpyDeviceToHost));
    LSG_GCUDA(cudaMemcpy(&hs, st, sizeof(GmresState), cudaMemcpyDeviceToHost));
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

int gmres(const lsg_operator *op, const lsg_params *prm, int dtype, void *d_x, const void *d_b, lsg_result *res,
          cudaStream_t s) {
    int rc = check_operator(op);
    if (rc) return rc;
    rc = check_params(prm, true);
    if (rc) return rc;
    if (!d_x || !d_b) return set_error(LSG_BAD_ARG, "NULL vector");
    if (dtype == LSG_F64) return gmres_t<double>(op, prm, (double *)d_x, (const double *)d_b, res, s);
    if (dtype == LSG_F32) return gmres_t<float>(op, prm, (float *)d_x, (const float *)d_b, res, s);
    return set_error(LSG_UNSUPPORTED, "GMRES: dtype %d (real FP64 / FP32 only)", dtype);
}

}  // namespace lsg

extern "C" int lsg_gmres(const lsg_operator *op, const lsg_params *prm, int dtype, void *d_x, const void *d_b,
                         lsg_result *res, void *stream) {
    return lsg::gmres(op, prm, dtype, d_x, d_b, res, (cudaStream_t)stream);
}
