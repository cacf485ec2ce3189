// lsg_icc.cu — block-Jacobi ICC(0) preconditioner for the FP64 AAR.
//
// The reference's PETSc drivers select it with pc = 1
// (PETSC_REAL/AAR_Real.c:58-61, PETSC_COMPLEX/AAR_Complex.c:63-66): PCICC on
// each rank's diagonal block of A (MatGetDiagonalBlock), applied to the
// rank's part of the residual (AAR_Real.c:100-103).  Here the blocks are the
// (bx, by, bz) boxes that tile the periodic grid -- the subdomains a
// Cartesian rank grid would own -- and every coupling that leaves a box, the
// periodic wrap included, is dropped.  The operator has constant
// coefficients, so all boxes share one block matrix and one factor.
//
// Factor (host, once per operator and box shape): incomplete L D L^T with the
// sparsity of A's lower triangle (zero fill; Meijerink & van der Vorst 1977),
// natural order x fastest.  Two rows of the star stencil share lower
// neighbours only along their common axis, so
//   l(i, i-pe) = (w_p - sum_{q>p} l(i, i-qe) l(i-pe, i-qe) d(i-qe)) / d(i-pe)
//   d(i)       = w_0 (1 + shift) - sum_{axis,p} l(i, i-pe)^2 d(i-pe),
// with the shift 0, 1e-3, 2e-3, ... (Manteuffel's remedy) that keeps every
// pivot positive; PETSc's ICC shifts the diagonal for the same reason.
//
// Apply (device): one CTA per box; the box's residual is staged in shared
// memory and both triangular solves run as wavefronts over the levels
// cx + cy + cz (every lower neighbour of a point lies on a lower level), one
// barrier per level.  The kernel also completes the AAR history: with
// f = M^-1 r, DF_c = f - f_old and H_c = step + beta DF_c, where H_c held the
// previous step x - x_old (AAR.c:96-102 with the preconditioned residual).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>
#include <type_traits>
#include <vector>

#include "lsg_kernels.cuh"
#include "lsg_host.h"

namespace lsg {

constexpr int kIccSlots = 18;  // 3 axes x 6 lower neighbours
constexpr int kIccMaxPoints = 4096;
constexpr int kIccThreads = 128;

// ---------------------------------------------------------------- host factor

int icc_factor_host(const int block[3], const double *w, int radius, double shift, double *L, double *d) {
    const int bx = block[0], by = block[1], bz = block[2];
    const int n = bx * by * bz;
    const int strides[3] = {1, bx, bx * by};
    for (int i = 0; i < n * kIccSlots; i++) L[i] = 0.0;
    for (int i = 0; i < n; i++) {
        const int c[3] = {i % bx, (i / bx) % by, i / (bx * by)};
        double acc = w[0] * (1.0 + shift);
        for (int a = 0; a < 3; a++) {
            for (int p = radius; p >= 1; p--) {  // farthest first: its terms feed the nearer ones
                if (c[a] < p) continue;
                const int k = i - p * strides[a];
                double t = w[p];
                for (int q = radius; q > p; q--) {
                    if (c[a] < q) continue;
                    const int tt = i - q * strides[a];
                    t = t - L[(size_t)i * kIccSlots + 6 * a + q - 1] * L[(size_t)k * kIccSlots + 6 * a + (q - p) - 1] *
                                d[tt];
                }
                L[(size_t)i * kIccSlots + 6 * a + p - 1] = t / d[k];
            }
        }
        for (int a = 0; a < 3; a++)
            for (int p = 1; p <= radius; p++)
                if (c[a] >= p) {
                    const int k = i - p * strides[a];
                    const double l = L[(size_t)i * kIccSlots + 6 * a + p - 1];
                    acc = acc - l * l * d[k];
                }
        if (!(acc > 0.0)) return 1;
        d[i] = acc;
    }
    return 0;
}

// ---------------------------------------------------------------- device factor

struct IccFactor {
    int bx, by, bz, nb, nlev, radius;
    double shift;
    double *L = nullptr;      // nb x 18
    double *dinv = nullptr;   // nb: 1 / d
    float2 *Lf = nullptr;     // the same as double-float pairs (double-float apply)
    float2 *dinvf = nullptr;
    int *order = nullptr;     // point indices sorted by level (natural order within a level)
    int *lev = nullptr;       // nlev + 1 offsets into order
    int *coord = nullptr;     // cx | cy << 8 | cz << 16
    void *base = nullptr;
    ~IccFactor() {
        if (base) cudaFree(base);
    }
};

struct IccView {
    const double *L, *dinv;
    const float2 *Lf, *dinvf;
    const int *order, *lev, *coord;
    int bx, by, bz, nb, nlev, radius;
};

static std::mutex g_icc_mu;
static std::map<std::tuple<int, int, int, int, int, std::vector<double>>, std::unique_ptr<IccFactor>> g_icc;

void release_icc() {
    std::lock_guard<std::mutex> g(g_icc_mu);
    g_icc.clear();
}

int icc_get(const lsg_operator *op, const int block[3], const IccFactor **out, double *shift_out) {
    const int bx = block[0], by = block[1], bz = block[2];
    const Weights<double> w = make_weights<double>(op);
    std::vector<double> wv(w.w, w.w + op->radius + 1);
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> g(g_icc_mu);
    auto key = std::make_tuple(dev, bx, by, bz, op->radius, wv);
    auto &slot = g_icc[key];
    if (slot) {
        *out = slot.get();
        if (shift_out) *shift_out = slot->shift;
        return LSG_OK;
    }
    const int nb = bx * by * bz;
    std::vector<double> L((size_t)nb * kIccSlots), d(nb);
    double shift = 0.0;
    int fail = 1;
    for (int k = 0; k < 40 && fail; k++) {
        fail = icc_factor_host(block, w.w, op->radius, shift, L.data(), d.data());
        if (fail) shift = shift == 0.0 ? 1e-3 : 2.0 * shift;
    }
    if (fail) return set_error(LSG_NAN_DETECTED, "block ICC(0): no positive factor with a diagonal shift");
    std::vector<double> dinv(nb);
    for (int i = 0; i < nb; i++) dinv[i] = 1.0 / d[i];
    const int nlev = bx + by + bz - 2;
    std::vector<int> lev(nlev + 1, 0), order(nb), coord(nb);
    for (int i = 0; i < nb; i++) {
        const int cx = i % bx, cy = (i / bx) % by, cz = i / (bx * by);
        coord[i] = cx | (cy << 8) | (cz << 16);
        lev[cx + cy + cz + 1]++;
    }
    for (int l = 0; l < nlev; l++) lev[l + 1] += lev[l];
    {
        std::vector<int> fill(lev.begin(), lev.end() - 1);
        for (int i = 0; i < nb; i++) {
            const int l = (i % bx) + ((i / bx) % by) + i / (bx * by);
            order[fill[l]++] = i;
        }
    }
    std::unique_ptr<IccFactor> F(new IccFactor());
    const size_t bL = (size_t)nb * kIccSlots * 8, bD = (size_t)nb * 8, bO = (size_t)nb * 4,
                 bV = (size_t)(nlev + 1) * 4, bC = (size_t)nb * 4;
    auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
    std::vector<float2> Lf((size_t)nb * kIccSlots), dinvf(nb);
    for (size_t i = 0; i < Lf.size(); i++) Lf[i] = df_weight(L[i]);
    for (int i = 0; i < nb; i++) dinvf[i] = df_weight(dinv[i]);
    char *base = nullptr;
    const size_t oLf = al(bL) + al(bD) + al(bO) + al(bV) + al(bC), oDf = oLf + al(bL);
    cudaError_t e = cudaMalloc(&base, oDf + al(bD));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(LSG_NO_MEMORY, "block ICC(0) factor: %s", cudaGetErrorString(e));
    }
    F->base = base;
    F->L = (double *)base;
    F->dinv = (double *)(base + al(bL));
    F->order = (int *)(base + al(bL) + al(bD));
    F->lev = (int *)(base + al(bL) + al(bD) + al(bO));
    F->coord = (int *)(base + al(bL) + al(bD) + al(bO) + al(bV));
    F->Lf = (float2 *)(base + oLf);
    F->dinvf = (float2 *)(base + oDf);
    e = cudaMemcpy(F->L, L.data(), bL, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(F->dinv, dinv.data(), bD, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(F->order, order.data(), bO, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(F->lev, lev.data(), bV, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(F->coord, coord.data(), bC, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(F->Lf, Lf.data(), bL, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(F->dinvf, dinvf.data(), bD, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return set_error(LSG_CUDA_ERROR, "block ICC(0) upload: %s", cudaGetErrorString(e));
    F->bx = bx;
    F->by = by;
    F->bz = bz;
    F->nb = nb;
    F->nlev = nlev;
    F->radius = op->radius;
    F->shift = shift;
    slot = std::move(F);
    *out = slot.get();
    if (shift_out) *shift_out = shift;
    return LSG_OK;
}

// ---------------------------------------------------------------- apply

// acc - l y for double-float acc, l, y (l y by the FMA two-product; the lo
// word left unnormalised until the point's sum is complete).
__device__ __forceinline__ float2 df_fnms(float2 acc, float2 l, float2 y) {
    const float p = __fmul_rn(l.x, y.x);
    float e = __fmaf_rn(l.x, y.x, -p);
    e = __fmaf_rn(l.x, y.y, e);
    e = __fmaf_rn(l.y, y.x, e);
    float s, t;
    df_two_sum(acc.x, -p, s, t);
    return make_float2(s, __fadd_rn(__fsub_rn(acc.y, e), t));
}

__device__ __forceinline__ float2 df_norm(float2 v) {
    const float h = __fadd_rn(v.x, v.y);
    return make_float2(h, __fsub_rn(v.y, __fsub_rn(h, v.x)));
}

__device__ __forceinline__ void icc_apply_df(const IccView &F, const Geom &g, const double *__restrict__ r,
                                             double *__restrict__ f, const double *__restrict__ f_old,
                                             double *__restrict__ df, double *__restrict__ hc, double beta,
                                             int hist, const DevCtrl *ctrl, float2 *y) {
    const int ks = ctrl ? df_shift_for(ctrl->rhs_norm) : 0;
    bool bad = false;
    const int nbx = g.nx / F.bx, nby = g.ny / F.by;
    const int box = blockIdx.x;
    const int ox = (box % nbx) * F.bx, oy = ((box / nbx) % nby) * F.by, oz = (box / (nbx * nby)) * F.bz;
    const int st[3] = {1, F.bx, F.bx * F.by};
    const int dim[3] = {F.bx, F.by, F.bz};
    auto gidx = [&](int cw) -> long long {
        return (long long)(ox + (cw & 0xff)) +
               (long long)g.nx * ((oy + ((cw >> 8) & 0xff)) + (long long)g.ny * (oz + (cw >> 16)));
    };
    for (int i = threadIdx.x; i < F.nb; i += blockDim.x) y[i] = df_split(r[gidx(F.coord[i])], ks, bad);
    __syncthreads();
    for (int l = 0; l < F.nlev; l++) {
        for (int t = F.lev[l] + threadIdx.x; t < F.lev[l + 1]; t += blockDim.x) {
            const int i = F.order[t];
            const int cw = F.coord[i];
            const int c[3] = {cw & 0xff, (cw >> 8) & 0xff, cw >> 16};
            const float2 *Li = F.Lf + (size_t)i * kIccSlots;
            float2 acc = y[i];
#pragma unroll
            for (int a = 0; a < 3; a++)
                for (int p = 1; p <= F.radius; p++)
                    if (c[a] >= p) acc = df_fnms(acc, Li[6 * a + p - 1], y[i - p * st[a]]);
            y[i] = df_norm(acc);
        }
        __syncthreads();
    }
    for (int l = F.nlev - 1; l >= 0; l--) {
        for (int t = F.lev[l] + threadIdx.x; t < F.lev[l + 1]; t += blockDim.x) {
            const int i = F.order[t];
            const int cw = F.coord[i];
            const int c[3] = {cw & 0xff, (cw >> 8) & 0xff, cw >> 16};
            float2 acc = df_mul(y[i], F.dinvf[i]);
#pragma unroll
            for (int a = 0; a < 3; a++)
                for (int p = 1; p <= F.radius; p++)
                    if (c[a] + p < dim[a]) {
                        const int j = i + p * st[a];
                        acc = df_fnms(acc, F.Lf[(size_t)j * kIccSlots + 6 * a + p - 1], y[j]);
                    }
            y[i] = df_norm(acc);
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < F.nb; i += blockDim.x) {
        const long long gi = gidx(F.coord[i]);
        const double fv = df_to_double(y[i], ks);
        f[gi] = fv;
        if (hist) {
            const double d = fv - f_old[gi];
            df[gi] = d;
            hc[gi] = fma(beta, d, hc[gi]);
        }
    }
    if (__syncthreads_or(bad ? 1 : 0) && threadIdx.x == 0 && ctrl)
        atomicOr(&const_cast<DevCtrl *>(ctrl)->df_range, 1);
}

// f = (L D L^T)^-1 r on box blockIdx.x; hist: also DF = f - f_old and
// hc = hc + beta DF.  Sums in the fixed order axis x, y, z and p = 1..radius.
// DFM: the solves in double-float arithmetic (the residual split into pairs
// scaled by 2^k as in the stencil passes; f rounded to doubles once).
template <bool DFM>
__global__ void __launch_bounds__(kIccThreads) icc_apply_kernel(IccView F, Geom g, const double *__restrict__ r,
                                                                 double *__restrict__ f,
                                                                 const double *__restrict__ f_old,
                                                                 double *__restrict__ df, double *__restrict__ hc,
                                                                 double beta, int hist, const DevCtrl *ctrl) {
    extern __shared__ double ysm[];
    if (solve_done(ctrl)) return;
    if constexpr (DFM) {
        icc_apply_df(F, g, r, f, f_old, df, hc, beta, hist, ctrl, reinterpret_cast<float2 *>(ysm));
        return;
    }
    double *y = ysm;
    const int nbx = g.nx / F.bx, nby = g.ny / F.by;
    const int box = blockIdx.x;
    const int ox = (box % nbx) * F.bx, oy = ((box / nbx) % nby) * F.by, oz = (box / (nbx * nby)) * F.bz;
    const int st[3] = {1, F.bx, F.bx * F.by};
    const int dim[3] = {F.bx, F.by, F.bz};
    auto gidx = [&](int cw) -> long long {
        return (long long)(ox + (cw & 0xff)) +
               (long long)g.nx * ((oy + ((cw >> 8) & 0xff)) + (long long)g.ny * (oz + (cw >> 16)));
    };
    for (int i = threadIdx.x; i < F.nb; i += blockDim.x) y[i] = r[gidx(F.coord[i])];
    __syncthreads();
    // forward: y_i = r_i - sum l(i, k) y_k over the lower neighbours k
    for (int l = 0; l < F.nlev; l++) {
        for (int t = F.lev[l] + threadIdx.x; t < F.lev[l + 1]; t += blockDim.x) {
            const int i = F.order[t];
            const int cw = F.coord[i];
            const int c[3] = {cw & 0xff, (cw >> 8) & 0xff, cw >> 16};
            const double *Li = F.L + (size_t)i * kIccSlots;
            double acc = y[i];
#pragma unroll
            for (int a = 0; a < 3; a++)
                for (int p = 1; p <= F.radius; p++)
                    if (c[a] >= p) acc = fma(-Li[6 * a + p - 1], y[i - p * st[a]], acc);
            y[i] = acc;
        }
        __syncthreads();
    }
    // backward: x_i = y_i / d_i - sum l(j, i) x_j over the upper neighbours j
    for (int l = F.nlev - 1; l >= 0; l--) {
        for (int t = F.lev[l] + threadIdx.x; t < F.lev[l + 1]; t += blockDim.x) {
            const int i = F.order[t];
            const int cw = F.coord[i];
            const int c[3] = {cw & 0xff, (cw >> 8) & 0xff, cw >> 16};
            double acc = y[i] * F.dinv[i];
#pragma unroll
            for (int a = 0; a < 3; a++)
                for (int p = 1; p <= F.radius; p++)
                    if (c[a] + p < dim[a]) {
                        const int j = i + p * st[a];
                        acc = fma(-F.L[(size_t)j * kIccSlots + 6 * a + p - 1], y[j], acc);
                    }
            y[i] = acc;
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < F.nb; i += blockDim.x) {
        const long long gi = gidx(F.coord[i]);
        const double fv = y[i];
        f[gi] = fv;
        if (hist) {
            const double d = fv - f_old[gi];
            df[gi] = d;
            hc[gi] = fma(beta, d, hc[gi]);
        }
    }
}

// ---- the same apply with the factor staged in shared memory once per CTA
// and one warp per box: a CTA loads L (slot-major, so a warp's points hit
// distinct banks), 1/d, the level order and the coordinates once; each warp
// then solves boxes on its own, its wavefront levels separated by warp
// barriers only, with the box's vector in its own shared-memory slice.  The
// per-point sums are the ones of icc_apply_kernel, in the same order, so the
// result is the same bit for bit.
constexpr int kIccWarps = 32;  // warps per CTA (fewer when the box's slices do not fit)

template <typename V>
__device__ __forceinline__ V icc_fnms(V acc, V l, V y);
template <>
__device__ __forceinline__ float2 icc_fnms<float2>(float2 acc, float2 l, float2 y) { return df_fnms(acc, l, y); }
template <>
__device__ __forceinline__ double icc_fnms<double>(double acc, double l, double y) { return fma(-l, y, acc); }

// DFM: double-float pairs (V = float2), else FP64 (V = double).
template <bool DFM>
__global__ void __launch_bounds__(32 * kIccWarps) icc_apply_smem_kernel(IccView F, Geom g, const double *__restrict__ r,
                                                                        double *__restrict__ f,
                                                                        const double *__restrict__ f_old,
                                                                        double *__restrict__ df,
                                                                        double *__restrict__ hc, double beta, int hist,
                                                                        int nboxes, const DevCtrl *ctrl) {
    using V = typename std::conditional<DFM, float2, double>::type;
    extern __shared__ __align__(16) unsigned char icc_sm[];
    if (solve_done(ctrl)) return;
    const int nb = F.nb, nlev = F.nlev, R = F.radius;
    const int nw = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    V *Ls = reinterpret_cast<V *>(icc_sm);               // 18 x nb, slot-major
    V *Ds = Ls + (size_t)nb * kIccSlots;                  // nb: 1 / d
    V *Yall = Ds + nb;                                    // nw x nb
    int *ord = reinterpret_cast<int *>(Yall + (size_t)nw * nb);
    int *crd = ord + nb;
    int *lvl = crd + nb;                                  // nlev + 1
    const V *Lg = DFM ? reinterpret_cast<const V *>(F.Lf) : reinterpret_cast<const V *>(F.L);
    const V *Dg = DFM ? reinterpret_cast<const V *>(F.dinvf) : reinterpret_cast<const V *>(F.dinv);
    for (int k = threadIdx.x; k < nb * kIccSlots; k += blockDim.x) {
        const int i = k / kIccSlots, sl = k - i * kIccSlots;
        Ls[(size_t)sl * nb + i] = Lg[k];
    }
    for (int k = threadIdx.x; k < nb; k += blockDim.x) {
        Ds[k] = Dg[k];
        ord[k] = F.order[k];
        crd[k] = F.coord[k];
    }
    for (int k = threadIdx.x; k <= nlev; k += blockDim.x) lvl[k] = F.lev[k];
    const int ks = (DFM && ctrl) ? df_shift_for(ctrl->rhs_norm) : 0;
    bool bad = false;
    const int nbx = g.nx / F.bx, nby = g.ny / F.by;
    const int st[3] = {1, F.bx, F.bx * F.by};
    const int dim[3] = {F.bx, F.by, F.bz};
    V *y = Yall + (size_t)warp * nb;
    __syncthreads();
    for (int box = blockIdx.x * nw + warp; box < nboxes; box += gridDim.x * nw) {
        const int ox = (box % nbx) * F.bx, oy = ((box / nbx) % nby) * F.by, oz = (box / (nbx * nby)) * F.bz;
        auto gidx = [&](int cw) -> long long {
            return (long long)(ox + (cw & 0xff)) +
                   (long long)g.nx * ((oy + ((cw >> 8) & 0xff)) + (long long)g.ny * (oz + (cw >> 16)));
        };
        for (int i = lane; i < nb; i += 32) {
            const double rv = r[gidx(crd[i])];
            if constexpr (DFM) y[i] = df_split(rv, ks, bad);
            else y[i] = rv;
        }
        __syncwarp();
        // forward: y_i = r_i - sum l(i, k) y_k over the lower neighbours k
        for (int l = 0; l < nlev; l++) {
            for (int t = lvl[l] + lane; t < lvl[l + 1]; t += 32) {
                const int i = ord[t];
                const int cw = crd[i];
                const int c[3] = {cw & 0xff, (cw >> 8) & 0xff, cw >> 16};
                V acc = y[i];
#pragma unroll
                for (int a = 0; a < 3; a++)
#pragma unroll
                    for (int p = 1; p <= 6; p++)
                        if (p <= R && c[a] >= p)
                            acc = icc_fnms<V>(acc, Ls[(size_t)(6 * a + p - 1) * nb + i], y[i - p * st[a]]);
                if constexpr (DFM) y[i] = df_norm(acc);
                else y[i] = acc;
            }
            __syncwarp();
        }
        // backward: x_i = y_i / d_i - sum l(j, i) x_j over the upper neighbours j
        for (int l = nlev - 1; l >= 0; l--) {
            for (int t = lvl[l] + lane; t < lvl[l + 1]; t += 32) {
                const int i = ord[t];
                const int cw = crd[i];
                const int c[3] = {cw & 0xff, (cw >> 8) & 0xff, cw >> 16};
                V acc;
                if constexpr (DFM) acc = df_mul(y[i], Ds[i]);
                else acc = y[i] * Ds[i];
#pragma unroll
                for (int a = 0; a < 3; a++)
#pragma unroll
                    for (int p = 1; p <= 6; p++)
                        if (p <= R && c[a] + p < dim[a]) {
                            const int j = i + p * st[a];
                            acc = icc_fnms<V>(acc, Ls[(size_t)(6 * a + p - 1) * nb + j], y[j]);
                        }
                if constexpr (DFM) y[i] = df_norm(acc);
                else y[i] = acc;
            }
            __syncwarp();
        }
        for (int i = lane; i < nb; i += 32) {
            const long long gi = gidx(crd[i]);
            double fv;
            if constexpr (DFM) fv = df_to_double(y[i], ks);
            else fv = y[i];
            f[gi] = fv;
            if (hist) {
                const double d = fv - f_old[gi];
                df[gi] = d;
                hc[gi] = fma(beta, d, hc[gi]);
            }
        }
        __syncwarp();  // y is reused by the warp's next box
    }
    if (DFM && __syncthreads_or(bad ? 1 : 0) && threadIdx.x == 0 && ctrl)
        atomicOr(&const_cast<DevCtrl *>(ctrl)->df_range, 1);
}

// Shared memory of icc_apply_smem_kernel with nw warps.
static size_t icc_smem_bytes(const IccFactor *F, int nw) {
    return (size_t)F->nb * kIccSlots * 8 + (size_t)F->nb * 8 + (size_t)nw * F->nb * 8 + (size_t)F->nb * 8 +
           (size_t)(F->nlev + 1) * 4;
}
constexpr size_t kIccSmemMax = 220 * 1024;

cudaError_t icc_apply(const IccFactor *F, const Geom &g, const double *r, double *f, const double *f_old,
                      double *df, double *hc, double beta, int hist, const DevCtrl *ctrl, int exact, cudaStream_t s) {
    const IccView v{F->L, F->dinv, F->Lf, F->dinvf, F->order, F->lev, F->coord, F->bx, F->by, F->bz, F->nb,
                    F->nlev, F->radius};
    const long long boxes = (long long)(g.nx / F->bx) * (g.ny / F->by) * (g.nz / F->bz);
    int nw = kIccWarps;
    while (nw > 4 && icc_smem_bytes(F, nw) > kIccSmemMax) nw /= 2;
    const size_t sm2 = icc_smem_bytes(F, nw);
    if (sm2 <= kIccSmemMax && boxes < (1LL << 30)) {
        // the factor staged once per CTA, one warp per box
        auto launch = [&](auto kern) -> cudaError_t {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2);
            if (e != cudaSuccess) return e;
            int occ = 0;
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 32 * nw, sm2);
            if (e != cudaSuccess) return e;
            const long long need = (boxes + nw - 1) / nw;
            const unsigned grid = (unsigned)std::max<long long>(
                1, std::min<long long>(need, (long long)sm_count() * std::max(1, occ)));
            kern<<<grid, 32 * nw, sm2, s>>>(v, g, r, f, f_old, df, hc, beta, hist, (int)boxes, ctrl);
            return cudaGetLastError();
        };
        return exact ? launch(icc_apply_smem_kernel<false>) : launch(icc_apply_smem_kernel<true>);
    }
    const size_t smem = (size_t)F->nb * sizeof(double);
    if (exact)
        icc_apply_kernel<false><<<(unsigned)boxes, kIccThreads, smem, s>>>(v, g, r, f, f_old, df, hc, beta, hist, ctrl);
    else
        icc_apply_kernel<true><<<(unsigned)boxes, kIccThreads, smem, s>>>(v, g, r, f, f_old, df, hc, beta, hist, ctrl);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- Richardson step with a materialised f

// u = x + omega f at every stencil point (f = M^-1 r from the preconditioner
// pass); r2 = b - A u, x2 = u, and the step omega f into the history column
// (completed with beta DF by the next preconditioner pass).  AAR.c:134-139.
struct RichPrecOp {
    static constexpr int NACC = 0;
    static constexpr bool DF = true;
    using Raw = Pair<double>;     // (x, f)
    using Ctr = Triple<double>;   // (b, x, f) at the centre
    const double *x;
    const double *f;
    const double *b;
    double *x2;
    double *r2;
    double *hn;
    double c;  // omega
    double *partials;
    const DevCtrl *ctrl;
    float2 cp;
    __device__ bool skip() const { return solve_done(ctrl); }
    __device__ void init() { cp = df_weight(c); }
    __device__ __forceinline__ Raw fetch(unsigned i) const { return Raw{ldg(x + i), ldg(f + i)}; }
    __device__ __forceinline__ double value(const Raw &v) const { return fma(c, v.b, v.a); }
    __device__ __forceinline__ Ctr fetch_center(unsigned i) const { return Ctr{ldg(b + i), ldg(x + i), ldg(f + i)}; }
    __device__ __forceinline__ void store(unsigned i, double u, double au, const Ctr &cc, Acc<double> *) const {
        x2[i] = u;
        r2[i] = cc.a - au;
        hn[i] = c * cc.c;
    }
    static constexpr bool VALUE_DF = true;
    __device__ __forceinline__ float2 value_df(const Raw &v, int k, bool &bad) const {
        return df_split(fma(c, v.b, v.a), k, bad);  // u = x + omega f in FP64, split once
    }
    static constexpr bool STORE_DF = true;
    // A u rounded to a double once, then the FP64 epilogue of store().
    __device__ __forceinline__ void store_df(unsigned i, float2, float2 au, const Ctr &cc, int k,
                                             Acc<double> *acc) const {
        store(i, fma(c, cc.c, cc.b), df_to_double(au, k), cc, acc);
    }
};

cudaError_t rich_prec(const StencilLaunch &L, const Weights<double> &w, const double *x, const double *f,
                      const double *b, double *x2, double *r2, double *hn, double omega, const DevCtrl *ctrl) {
    RichPrecOp op{x, f, b, x2, r2, hn, omega, nullptr, ctrl};
    return launch_stencil<double>(L, w, op);
}

}  // namespace lsg

extern "C" int lsg_icc_factor(const lsg_operator *op, const int block[3], double *L, double *d, double *shift) {
    if (!op || !block || !L || !d) return lsg::set_error(LSG_BAD_ARG, "lsg_icc_factor: NULL argument");
    if (op->radius < 1 || op->radius > 6)
        return lsg::set_error(LSG_UNSUPPORTED, "block ICC(0): radius %d outside 1..6", op->radius);
    if (block[0] < 1 || block[1] < 1 || block[2] < 1 || block[0] > 255 || block[1] > 255 || block[2] > 255 ||
        (long long)block[0] * block[1] * block[2] > lsg::kIccMaxPoints)
        return lsg::set_error(LSG_BAD_ARG, "block ICC(0): box %d x %d x %d outside 1..255 per side, <= %d points",
                              block[0], block[1], block[2], lsg::kIccMaxPoints);
    const lsg::Weights<double> w = lsg::make_weights<double>(op);
    double s = 0.0;
    for (int k = 0; k < 40; k++) {
        if (!lsg::icc_factor_host(block, w.w, op->radius, s, L, d)) {
            if (shift) *shift = s;
            return LSG_OK;
        }
        s = s == 0.0 ? 1e-3 : 2.0 * s;
    }
    return lsg::set_error(LSG_NAN_DETECTED, "block ICC(0): no positive factor with a diagonal shift");
}
