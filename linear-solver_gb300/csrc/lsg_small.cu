// lsg_small.cu — the kernels that turn per-block partial sums into the
// scalars a solve needs, and the m x m pseudo-inverse solve.
//
//   finalize_norm        ||v|| from partials; convergence test     tools.c:18-28, AAR.c:91,123
//   finalize_gram_solve  Gram assembly + s = pinv(G) h             AAR.c:212-223; PGR.c:206-217;
//                                                                  PL2R.c:206-217; tools.c:52-105
//   finalize_cg          alpha / beta / delta / relres             CG.c:100-104, 131-148
//
// The pseudo-inverse keeps the reference's semantics: with A = U W V^T,
//     x = V diag(1/w_j) V^T b,   terms with w_j < m * wmax * 2.22044605e-16 dropped
// (tools.c:325-335 assign V to U before forming the product, exact for the
// symmetric Gram of AAR / PL2R; for PGR's DX^T DF it is (A^T A)^{+1/2} b).
// The SVD is a one-sided (Hestenes) Jacobi iteration, written here from the
// mathematics: rotate column pairs of G = A V until they are orthogonal; then
// w_j = ||G(:,j)|| and V holds the right singular vectors.  Lanes own rows,
// so the column dot products are warp reductions.  The sweep count is bounded
// and exhaustion is reported as LSG_SVD_NO_CONVERGENCE (the reference exits
// the process after 250 iterations, tools.c:270).
#include <mutex>

#include "lsg_internal.cuh"
#include "lsg_host.h"

namespace lsg {

constexpr int kFinThreads = 256;
constexpr int kFinWarps = kFinThreads / 32;
constexpr int kMaxSweeps = 60;
constexpr double kPinvEps = 2.22044605e-16;

__device__ __forceinline__ bool ctrl_done(const DevCtrl *c) { return *(volatile const int *)&c->done; }

// Sum of partials[k*stride + off] over k < nparts, block-wide, deterministic.
__device__ double block_sum_partials(const double *partials, int nparts, int stride, int off,
                                     double *red) {
    double s = 0.0;
    for (int k = threadIdx.x; k < nparts; k += blockDim.x) s += partials[(long long)k * stride + off];
    s = warp_sum(s);
    const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[w] = s;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < nw ? red[threadIdx.x] : 0.0;
        t = warp_sum(t);
    }
    return t;  // valid in warp 0
}

__device__ void finalize_norm_body(const double *partials, int nparts, DevCtrl *ctrl, int mode,
                                   double tol, int iter, int width) {
    __shared__ double red[32];
    const double s = block_sum_partials(partials, nparts, width, 0, red);
    if (threadIdx.x != 0) return;
    const double v = sqrt(s);
    if (mode == NF_RHS) {
        ctrl->rhs_norm = v;
        ctrl->tol_abs = tol * v;
        if (!isfinite(v)) { ctrl->status = LSG_NAN_DETECTED; ctrl->done = 1; ctrl->iters = 0; }
        return;
    }
    ctrl->relres = v;
    if (mode == NF_CHECK) {
        if (!isfinite(v)) {
            ctrl->status = LSG_NAN_DETECTED;
            ctrl->done = 1;
            ctrl->iters = iter;
        } else if (!(v > ctrl->tol_abs)) {  // the loop test of AAR.c:91 fails
            ctrl->done = 1;
            ctrl->iters = iter;
        } else if (ctrl->stall_limit > 0) {
            if (v < 0.7 * ctrl->best) {
                ctrl->best = v;
                ctrl->stall = 0;
            } else if (++ctrl->stall >= ctrl->stall_limit) {
                ctrl->done = 1;
                ctrl->stalled = 1;
                ctrl->iters = iter;
            }
        }
    }
}

__global__ void finalize_norm_kernel(const double *partials, int nparts, DevCtrl *ctrl, int mode,
                                     double tol, int iter, int width) {
    if (mode != NF_RHS && ctrl_done(ctrl)) return;
    finalize_norm_body(partials, nparts, ctrl, mode, tol, iter, width);
}

// ---------------------------------------------------------------- m x m solve

// Stopping test of the Jacobi sweeps: a column pair counts as orthogonal once
// gamma^2 <= (kJacobiTol)^2 * alpha * beta.
constexpr double kJacobiTol = 8 * kPinvEps;

// x = V diag(1/w) V^T b from the converged G = A V (lane j of the warp owns
// column j); shared by both Jacobi variants.  ld: leading dimension of G, V.
__device__ void pinv_apply(const double *G, const double *V, int ld, const double *b, double *x,
                           int m, double scale, double cut) {
    const int lane = threadIdx.x & 31;
    double w = 0.0;
    if (lane < m) {
        for (int k = 0; k < m; k++) w = fma(G[k * ld + lane], G[k * ld + lane], w);
        w = sqrt(w);
    }
    double wmax = lane < m ? w : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) wmax = fmax(wmax, __shfl_xor_sync(0xffffffffu, wmax, o));
    const double wmin = cut * wmax;
    double tj = 0.0;  // (V^T b)_j / w_j on lane j
    if (lane < m && w >= wmin && w > 0.0) {
        for (int i = 0; i < m; i++) tj = fma(V[i * ld + lane], b[i], tj);
        tj /= w;
    }
    double xi = 0.0;
    for (int j = 0; j < m; j++) {
        const double t = __shfl_sync(0xffffffffu, tj, j);
        if (lane < m) xi = fma(V[lane * ld + j], t, xi);
    }
    if (lane < m) x[lane] = xi * scale;
}

// General case, m <= 32: one warp, lane k owns row k, column pairs visited
// cyclically with the rotation computed in FP64.  Returns 0 on convergence,
// LSG_SVD_NO_CONVERGENCE otherwise.
__device__ int warp_pinv(double *G, double *V, const double *b, double *x, int m, double cut) {
    const int lane = threadIdx.x & 31;
    for (int i = lane; i < m * m; i += 32) V[i] = (i / m == i % m) ? 1.0 : 0.0;
    __syncwarp();
    bool rotated = true;
    int sweep = 0;
    for (; sweep < kMaxSweeps && rotated; sweep++) {
        rotated = false;
        for (int i = 0; i < m - 1; i++) {
            for (int j = i + 1; j < m; j++) {
                double gi = 0.0, gj = 0.0;
                if (lane < m) { gi = G[lane * m + i]; gj = G[lane * m + j]; }
                double al = gi * gi, be = gj * gj, ga = gi * gj;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    al += __shfl_xor_sync(0xffffffffu, al, o);
                    be += __shfl_xor_sync(0xffffffffu, be, o);
                    ga += __shfl_xor_sync(0xffffffffu, ga, o);
                }
                if (ga == 0.0 || ga * ga <= kJacobiTol * kJacobiTol * al * be) continue;
                rotated = true;
                const double zeta = (be - al) / (2.0 * ga);
                double t;
                if (fabs(zeta) > 1e150) t = 0.5 / zeta;
                else t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                const double c = 1.0 / sqrt(1.0 + t * t);
                const double s = c * t;
                if (lane < m) {
                    G[lane * m + i] = c * gi - s * gj;
                    G[lane * m + j] = s * gi + c * gj;
                    const double vi = V[lane * m + i], vj = V[lane * m + j];
                    V[lane * m + i] = c * vi - s * vj;
                    V[lane * m + j] = s * vi + c * vj;
                }
                __syncwarp();
            }
        }
    }
    pinv_apply(G, V, m, b, x, m, 1.0, cut);
    return rotated ? LSG_SVD_NO_CONVERGENCE : 0;
}

// Fast case, m <= 8: the columns (padded to an even count M2) are paired by
// the round-robin ("circle") schedule, so each round rotates M2/2 disjoint
// pairs at once; lane = 8*q + row works on pair q, row `row`.  G is scaled by
// a power of two so its largest entry is O(1) (exact; undone at the end); the
// rotation angle is then computed in FP32 and (c, s) re-normalised to
// c^2 + s^2 = 1 in FP64 by two Newton steps, so each rotation stays exactly
// orthogonal in FP64 while its angle is accurate to ~1e-7 -- a pair left
// slightly non-orthogonal is finished by the next sweep.  Pairs whose FP32
// angle would underflow use the FP64 formula.  G, V: 8 x 8, row-major, ld 8,
// rows and columns >= m zero.
__device__ int warp_pinv8(double *G, double *V, const double *b, double *x, int m, double cut) {
    const int lane = threadIdx.x & 31;
    const int q = lane >> 3, row = lane & 7;
    const int M2 = m + (m & 1);
    // power-of-two normalisation
    double amax = 0.0;
    for (int k = lane; k < 64; k += 32) amax = fmax(amax, fabs(G[k]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    int e = 0;
    if (amax > 0.0) frexp(amax, &e);
    for (int k = lane; k < 64; k += 32) {
        G[k] = ldexp(G[k], -e);
        V[k] = ((k >> 3) == (k & 7)) ? 1.0 : 0.0;
    }
    __syncwarp();
    int sweep = 0;
    bool any = true;
    for (; sweep < kMaxSweeps && any; sweep++) {
        bool rotated = false;
        for (int r = 0; r < M2 - 1; r++) {
            int i = -1, j = -1;
            if (q < M2 / 2) {
                const int pa = q, pb = M2 - 1 - q;
                const int ca = pa == 0 ? 0 : 1 + (pa - 1 + r) % (M2 - 1);
                const int cb = pb == 0 ? 0 : 1 + (pb - 1 + r) % (M2 - 1);
                i = min(ca, cb);
                j = max(ca, cb);
            }
            const bool active = i >= 0 && j < m;
            double gi = 0.0, gj = 0.0, vi = 0.0, vj = 0.0;
            if (active) {
                gi = G[row * 8 + i]; gj = G[row * 8 + j];
                vi = V[row * 8 + i]; vj = V[row * 8 + j];
            }
            double al = gi * gi, be = gj * gj, ga = gi * gj;
#pragma unroll
            for (int o = 1; o < 8; o <<= 1) {
                al += __shfl_xor_sync(0xffffffffu, al, o);
                be += __shfl_xor_sync(0xffffffffu, be, o);
                ga += __shfl_xor_sync(0xffffffffu, ga, o);
            }
            if (active && ga != 0.0 && ga * ga > kJacobiTol * kJacobiTol * al * be) {
                rotated = true;
                double c, s;
                const float num = (float)(be - al), den = (float)(2.0 * ga);
                if (den != 0.0f) {
                    const float z = num / den;
                    const float az = fabsf(z);
                    const float t = az < 1e18f ? copysignf(1.0f, z) / (az + sqrtf(1.0f + z * z)) : 0.5f / z;
                    const float cf = rsqrtf(1.0f + t * t);
                    c = (double)cf;
                    s = (double)(cf * t);
#pragma unroll
                    for (int it = 0; it < 2; it++) {
                        const double k = fma(-0.5, fma(c, c, s * s), 1.5);
                        c *= k;
                        s *= k;
                    }
                } else {
                    const double zeta = (be - al) / (2.0 * ga);
                    const double t = fabs(zeta) > 1e150 ? 0.5 / zeta
                                   : (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                    c = 1.0 / sqrt(1.0 + t * t);
                    s = c * t;
                }
                G[row * 8 + i] = c * gi - s * gj;
                G[row * 8 + j] = s * gi + c * gj;
                V[row * 8 + i] = c * vi - s * vj;
                V[row * 8 + j] = s * vi + c * vj;
            }
            __syncwarp();
        }
        any = __any_sync(0xffffffffu, rotated);
    }
    pinv_apply(G, V, 8, b, x, m, ldexp(1.0, -e), cut);
    return any ? LSG_SVD_NO_CONVERGENCE : 0;
}

// 1/d in FP64 from an FP32 seed and two Newton steps (no FP64 divide).
__device__ __forceinline__ double rcp_newton(double d) {
    double r = (double)(1.0f / (float)d);
    r = r * fma(-d, r, 2.0);
    r = r * fma(-d, r, 2.0);
    return r;
}

// Fast path for a symmetric positive semi-definite G (the AAR / PL2R Gram):
// x = G^-1 h by a lane-parallel LDL^T factorisation, taken only when it is
// provably what the reference's truncated pseudo-inverse returns.  Rows and
// columns of G that are exactly zero (history columns not yet written) have
// exactly-zero singular values, which the reference drops; they are dropped
// here too and x is 0 there.  For the rest, kappa_2(G) <= trace(G) *
// trace(G^-1); when that bound is below 1 / (100 m eps) no singular value can
// fall under the cutoff m * wmax * eps (MPI_REAL/tools.c:331-335), so the
// pseudo-inverse is the inverse.  Returns false (caller falls back to the
// Jacobi SVD) when G is not of that kind.  G: m x m row-major (ld m) in shared
// memory; Ls, Wi: m x m shared scratch; dd: m doubles.  One warp.
__device__ bool warp_ldl_solve(const double *G, const double *h, double *x, int m, double *Ls,
                               double *Wi, double *dd, double cut) {
    const int lane = threadIdx.x & 31;
    const unsigned full = 0xffffffffu;
    bool act = false, bad = false;
    double trg = 0.0;
    if (lane < m) {
        const double gii = G[lane * m + lane];
        act = gii != 0.0;
        bad = gii < 0.0 || !isfinite(gii);
        if (!act)
            for (int j = 0; j < m; j++) bad |= G[lane * m + j] != 0.0 || G[j * m + lane] != 0.0;
        trg = gii;
    }
    if (__any_sync(full, bad)) return false;
    const unsigned amask = __ballot_sync(full, act);
    if (amask == 0) {  // G = 0: the reference's pinv returns 0
        if (lane < m) x[lane] = 0.0;
        return true;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) trg += __shfl_xor_sync(full, trg, o);
    // Work on sc * G with sc a power of two making the trace O(1), so every
    // pivot lies in the range where the FP32-seeded reciprocal is valid
    // (an out-of-range pivot gives a non-finite bound and the fallback).
    int ex = 0;
    frexp(trg, &ex);
    const double sc = ldexp(1.0, -ex);
    trg *= sc;
    for (int k = lane; k < m * m; k += 32) Ls[k] = 0.0;
    __syncwarp();
    // LDL^T over the active indices: lane r holds row r of L, and Wi (free
    // until the bound below) row r of -L(r, t) d_t, formed once per entry.
    double rinv = 0.0;  // lane j: 1 / d_j
    for (int j = 0; j < m; j++) {
        if (!((amask >> j) & 1u)) continue;
        double acc = 0.0;
        if (lane < m && act) {
            acc = G[lane * m + j] * sc;
            for (int t = 0; t < j; t++)
                if ((amask >> t) & 1u) acc = fma(Wi[lane * m + t], Ls[j * m + t], acc);
        }
        const double dj = __shfl_sync(full, acc, j);
        if (!(dj > 0.0)) return false;
        const double inv = rcp_newton(dj);
        if (lane == j) { dd[j] = dj; Ls[j * m + j] = 1.0; rinv = inv; }
        if (lane < m && lane > j && act) {
            const double l = acc * inv;
            Ls[lane * m + j] = l;
            Wi[lane * m + j] = -l * dj;
        }
        __syncwarp();
    }
    // kappa bound: trace(G^-1) = sum_k (1/d_k) ||row k of L^-1||^2.  Lane c
    // builds column c of L^-1 by forward substitution.
    if (lane < m) {
        for (int r = 0; r < m; r++) {
            double v = (r == lane) ? 1.0 : 0.0;
            if (((amask >> r) & 1u) && r > lane)
                for (int t = lane; t < r; t++) v = fma(-Ls[r * m + t], Wi[t * m + lane], v);
            Wi[r * m + lane] = ((amask >> r) & 1u) ? v : 0.0;
        }
    }
    __syncwarp();
    double tri = 0.0;
    if (lane < m && act) {
        double rn = 0.0;
        for (int c = 0; c < m; c++) rn = fma(Wi[lane * m + c], Wi[lane * m + c], rn);
        tri = rn * rinv;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) tri += __shfl_xor_sync(full, tri, o);
    if (!(trg * tri * (100.0 * cut) < 1.0)) return false;
    // Solve L z = h, z /= d, L^T x = z.
    double sv = (lane < m && act) ? h[lane] : 0.0;
    for (int t = 0; t < m; t++) {
        if (!((amask >> t) & 1u)) continue;
        const double zt = __shfl_sync(full, sv, t);
        if (lane < m && lane > t && act) sv = fma(-Ls[lane * m + t], zt, sv);
    }
    sv *= rinv;
    for (int t = m - 1; t >= 0; t--) {
        if (!((amask >> t) & 1u)) continue;
        const double xt = __shfl_sync(full, sv, t);
        if (lane < m && lane < t && act) sv = fma(-Ls[t * m + lane], xt, sv);
    }
    if (lane < m) x[lane] = act ? sv * sc : 0.0;
    return true;
}

// Dispatch on m; G (m x m row-major) is overwritten.  Gs / Vs: 8 x 8 staging
// for the fast path.  Called by one full warp.
__device__ int warp_pinv_any(double *G, double *V, const double *b, double *x, int m, double *Gs,
                             double *Vs, double cut) {
    const int lane = threadIdx.x & 31;
    if (m <= 8) {
        for (int k = lane; k < 64; k += 32) {
            const int r = k >> 3, c = k & 7;
            Gs[k] = (r < m && c < m) ? G[r * m + c] : 0.0;
        }
        __syncwarp();
        return warp_pinv8(Gs, Vs, b, x, m, cut);
    }
    return warp_pinv(G, V, b, x, m, cut);
}

// Sums nv values over nparts block partials (row k: values of block k): value
// v = warp + q * nwarps is one warp's, lanes striding over the rows, each lane
// adding its rows in increasing order, then a warp sum.  A warp keeps its
// (up to kSumVals) values' loads in flight together, two rows at a time,
// since the partials are L2-resident and the loop is latency-bound.
constexpr int kSumVals = 6;
__device__ __forceinline__ void sum_gram_partials(const double *__restrict__ partials, int nparts, int nv,
                                                  double *vals, int *bad) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int v0 = warp; v0 < nv; v0 += nw * kSumVals) {
        double t[kSumVals];
#pragma unroll
        for (int q = 0; q < kSumVals; q++) t[q] = 0.0;
        int k = lane;
        for (; k + 32 < nparts; k += 64) {
            const double *ra = partials + (long long)k * nv, *rb = ra + 32LL * nv;
            double a[kSumVals], b[kSumVals];
#pragma unroll
            for (int q = 0; q < kSumVals; q++) {
                const int v = v0 + q * nw;
                a[q] = v < nv ? __ldcg(ra + v) : 0.0;
                b[q] = v < nv ? __ldcg(rb + v) : 0.0;
            }
#pragma unroll
            for (int q = 0; q < kSumVals; q++) {
                t[q] += a[q];
                t[q] += b[q];
            }
        }
        if (k < nparts) {
            const double *ra = partials + (long long)k * nv;
#pragma unroll
            for (int q = 0; q < kSumVals; q++) {
                const int v = v0 + q * nw;
                if (v < nv) t[q] += __ldcg(ra + v);
            }
        }
#pragma unroll
        for (int q = 0; q < kSumVals; q++) {
            const int v = v0 + q * nw;
            const double tv = warp_sum(t[q]);
            if (lane == 0 && v < nv) {
                vals[v] = tv;
                if (!isfinite(tv)) *bad = 1;
            }
        }
    }
}

// Assembles G (m x m) and h from the summed values and solves s = pinv(G) h
// into ctrl->s (one warp); bad: a value was not finite.
__device__ void gram_solve_tail(const double *vals, int bad, int kind, int m, double hscale, DevCtrl *ctrl) {
    __shared__ double G[LSG_MAX_M * LSG_MAX_M], V[LSG_MAX_M * LSG_MAX_M];
    __shared__ double Gs[LSG_MAX_M * LSG_MAX_M], Vs[64];
    __shared__ double h[LSG_MAX_M], s[LSG_MAX_M], dd[LSG_MAX_M];
    const int nv = gram_values(kind, m);
    const int np = nv - m;
    if (threadIdx.x < 32) {
        // Assemble G (row-major) and h.
        if (kind == GRAM_SYM) {
            for (int k = threadIdx.x; k < np; k += 32) {
                int j = 0;
                while ((j + 1) * (j + 2) / 2 <= k) j++;
                const int a = k - j * (j + 1) / 2;
                G[a * m + j] = vals[k];
                G[j * m + a] = vals[k];
            }
        } else {
            for (int k = threadIdx.x; k < np; k += 32) G[k] = vals[k];  // (a, j) = DX_a . DF_j
        }
        for (int j = threadIdx.x; j < m; j += 32) h[j] = vals[np + j] * hscale;
        __syncwarp();
        int st = 0;
        if (!bad) {
            // symmetric PSD Gram: LDL^T when provably equal to the truncated pinv
            const double cut = m * kPinvEps;  // MPI_REAL/tools.c:331-335
            const bool fast = kind == GRAM_SYM && warp_ldl_solve(G, h, s, m, V, Gs + 0, dd, cut);
            if (!fast) {
                if (kind == GRAM_SYM && threadIdx.x == 0) ctrl->svd_fallbacks++;
                st = warp_pinv_any(G, V, h, s, m, Gs, Vs, cut);
            }
        }
        __syncwarp();
        if (threadIdx.x < m) ctrl->s[threadIdx.x] = bad ? 0.0 : s[threadIdx.x];
        if (threadIdx.x == 0) {
            if (bad) { ctrl->status = LSG_NAN_DETECTED; ctrl->done = 1; }
            else if (st) ctrl->status = st;  // reported, the solve continues
        }
    }
}

__device__ void gram_solve_body(const double *partials, int nparts, int kind, int m, double hscale,
                                DevCtrl *ctrl) {
    __shared__ double vals[LSG_MAX_M * LSG_MAX_M + LSG_MAX_M];
    __shared__ int bad;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    sum_gram_partials(partials, nparts, gram_values(kind, m), vals, &bad);
    __syncthreads();
    gram_solve_tail(vals, bad, kind, m, hscale, ctrl);
}

// The Gram sums of a single solve spread over ceil(nv / 8) blocks: the FP64
// pipe issues one warp instruction per ~64 cycles on each SM partition, so
// one block summing all nv values over the block partials is slower than the
// small solve after it.  Warp w of block b sums value v = 8 b + w over rows
// lane, lane + 32, ... (four loads in flight) and then across the warp, the
// order of sum_gram_partials, so the totals equal the one-block totals bit for
// bit.  Lane 0 stores the total in row 0 of its column, which no other warp
// reads.  Returns true in the last block to finish: a ticket in the control
// block, which that block resets to 0 for the next launch.
__device__ bool sum_gram_spread(double *partials, int nparts, int nv, DevCtrl *ctrl) {
    __shared__ int last;
    const int lane = threadIdx.x & 31;
    const int v = blockIdx.x * (int)(blockDim.x >> 5) + (int)(threadIdx.x >> 5);
    if (v < nv) {
        const double *col = partials + v;
        double t = 0.0;
        int k = lane;
        for (; k + 96 < nparts; k += 128) {
            const double a0 = __ldcg(col + (long long)k * nv), a1 = __ldcg(col + (long long)(k + 32) * nv);
            const double a2 = __ldcg(col + (long long)(k + 64) * nv), a3 = __ldcg(col + (long long)(k + 96) * nv);
            t += a0;
            t += a1;
            t += a2;
            t += a3;
        }
        for (; k < nparts; k += 32) t += __ldcg(col + (long long)k * nv);
        t = warp_sum(t);
        if (lane == 0) __stcg(partials + v, t);
    }
    __threadfence();  // the totals are visible device-wide before the ticket
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned ticket = atomicAdd(&ctrl->fin_ticket, 1u);
        last = ticket == gridDim.x - 1;
        if (last) ctrl->fin_ticket = 0;
    }
    __syncthreads();
    return last != 0;
}

// The last block's read of the totals (through L2: other blocks stored them).
__device__ void load_gram_totals(const double *partials, int nv, double *vals, int *bad) {
    if (threadIdx.x == 0) *bad = 0;
    __syncthreads();
    for (int v = threadIdx.x; v < nv; v += blockDim.x) {
        const double t = __ldcg(partials + v);
        vals[v] = t;
        if (!isfinite(t)) *bad = 1;
    }
    __syncthreads();
}

__global__ void finalize_gram_solve_kernel(double *partials, int nparts, int kind, int m, double hscale,
                                           DevCtrl *ctrl) {
    __shared__ double vals[LSG_MAX_M * LSG_MAX_M + LSG_MAX_M];
    __shared__ int bad;
    if (ctrl_done(ctrl)) return;
    const int nv = gram_values(kind, m);
    if (!sum_gram_spread(partials, nparts, nv, ctrl)) return;
    load_gram_totals(partials, nv, vals, &bad);
    gram_solve_tail(vals, bad, kind, m, hscale, ctrl);
}

// Complex Hermitian Gram: from the summed (re, im) values, builds the real
// 2m x 2m representation [[A, -B], [B, A]] of G = A + iB (same singular
// values, each twice) and right-hand side [Re h; Im h], and solves it with
// zgelsd's cutoff sigma < eps * sigma_max (PETSC_COMPLEX/AAR_Complex.c:239,
// rcond = -1).
__device__ void gram_solve_c_tail(const double *vals, int bad, int m, double hre, double him, DevCtrl *ctrl) {
    constexpr int M2MAX = LSG_MAX_M;
    __shared__ double G[M2MAX * M2MAX], V[M2MAX * M2MAX], W[M2MAX * M2MAX];
    __shared__ double Gs[64], Vs[64];
    __shared__ double h[M2MAX], s[M2MAX], dd[M2MAX];
    const int np = (m * (m + 1)) / 2;
    const int m2 = 2 * m;
    if (threadIdx.x < 32) {
        for (int k = threadIdx.x; k < np; k += 32) {
            int j = 0;
            while ((j + 1) * (j + 2) / 2 <= k) j++;
            const int a = k - j * (j + 1) / 2;
            const double re = vals[2 * k];  // G(a, j) = DF_a^H DF_j, real on the diagonal
            const double im = a == j ? 0.0 : vals[2 * k + 1];
            // A(a,j) = re, B(a,j) = im; A(j,a) = re, B(j,a) = -im
            G[a * m2 + j] = re;           G[j * m2 + a] = re;
            G[(a + m) * m2 + j + m] = re; G[(j + m) * m2 + a + m] = re;
            G[a * m2 + j + m] = -im;      G[j * m2 + a + m] = im;
            G[(a + m) * m2 + j] = im;     G[(j + m) * m2 + a] = -im;
        }
        for (int j = threadIdx.x; j < m; j += 32) {
            const double re = vals[2 * (np + j)], im = vals[2 * (np + j) + 1];
            h[j] = hre * re - him * im;
            h[j + m] = hre * im + him * re;
        }
        __syncwarp();
        int st = 0;
        if (!bad) {
            const double cut = kPinvEps;
            if (!warp_ldl_solve(G, h, s, m2, V, W, dd, cut)) {
                if (threadIdx.x == 0) ctrl->svd_fallbacks++;
                st = warp_pinv_any(G, V, h, s, m2, Gs, Vs, cut);
            }
        }
        __syncwarp();
        for (int j = threadIdx.x; j < m; j += 32) {
            ctrl->s[2 * j] = bad ? 0.0 : s[j];
            ctrl->s[2 * j + 1] = bad ? 0.0 : s[j + m];
        }
        if (threadIdx.x == 0) {
            if (bad) { ctrl->status = LSG_NAN_DETECTED; ctrl->done = 1; }
            else if (st) ctrl->status = st;
        }
    }
}

__device__ void gram_solve_c_body(const double *partials, int nparts, int m, double hre, double him,
                                  DevCtrl *ctrl) {
    __shared__ double vals[2 * (LSG_MAX_M * LSG_MAX_M + LSG_MAX_M)];
    __shared__ int bad;
    const int nvr = m * (m + 1) + 2 * m;  // reals per block partial: 2 (m (m + 1) / 2 + m)
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    sum_gram_partials(partials, nparts, nvr, vals, &bad);
    __syncthreads();
    gram_solve_c_tail(vals, bad, m, hre, him, ctrl);
}

// One solve's complex Gram, its sums spread as in finalize_gram_solve_kernel.
__global__ void finalize_gram_solve_c_kernel(double *partials, int nparts, int m, double hre, double him,
                                             DevCtrl *ctrl) {
    __shared__ double vals[2 * (LSG_MAX_M * LSG_MAX_M + LSG_MAX_M)];
    __shared__ int bad;
    if (ctrl_done(ctrl)) return;
    const int nvr = m * (m + 1) + 2 * m;
    if (!sum_gram_spread(partials, nparts, nvr, ctrl)) return;
    load_gram_totals(partials, nvr, vals, &bad);
    gram_solve_c_tail(vals, bad, m, hre, him, ctrl);
}

// ---------------------------------------------------------------- batched finalize
// One block per active instance (amap[blockIdx.x]); the iteration number comes
// from the batch clock as in the batched stencil passes.

__global__ void batch_finalize_norm_kernel(BArgs a, const int *amap, int kind, double tol, int width) {
    const int i = amap[blockIdx.x];
    const BCtl &C = a.ctl[i];
    const int it = a.clk->it0 + a.k + 1;
    switch (kind) {
    case BF_RHS:
        finalize_norm_body(C.part, C.ublocks, C.ctrl, NF_RHS, tol, 0, width);
        break;
    case BF_RHS_OUTER:
        finalize_norm_body(C.part, C.ublocks, C.octrl, NF_RHS, tol, 0, width);
        break;
    case BF_CHECK:
        if (it > a.max_iter || ctrl_done(C.ctrl)) return;
        finalize_norm_body(C.part, C.sblocks, C.ctrl, NF_CHECK, tol, it, width);
        break;
    default:  // BF_REPLACE
        if (ctrl_done(C.octrl) || !(a.gate == 1 || ctrl_done(C.ctrl))) return;
        finalize_norm_body(C.part, C.sblocks, C.octrl, NF_CHECK, tol, it, width);
    }
}

__global__ void batch_finalize_gram_kernel(BArgs a, const int *amap, int cplx_gram) {
    const int i = amap[blockIdx.x];
    const BCtl &C = a.ctl[i];
    const int it = a.clk->it0 + a.k + 1;
    if (it > a.max_iter || ctrl_done(C.ctrl)) return;
    if (cplx_gram) gram_solve_c_body(C.part, C.ublocks, a.m, C.hre, C.him, C.ctrl);
    else gram_solve_body(C.part, C.ublocks, GRAM_SYM, a.m, C.hre, C.ctrl);
}

// Thread per active instance.  A paused FP32 iteration whose FP64 residual
// did not meet tol resumes with the target max(tol_abs, rho * relres) and a
// fresh stall record -- or the instance stops: NaN in the FP32 iteration, or
// max_outer runs used.
__global__ void batch_resume_kernel(BArgs a, const int *amap, int nact, double rho, int max_outer) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nact) return;
    const BCtl &C = a.ctl[amap[t]];
    DevCtrl *in = C.ctrl, *out = C.octrl;
    if (out->done || !in->done) return;
    const int it = a.clk->it0 + a.k + 1;
    if (in->status == LSG_NAN_DETECTED) {
        out->status = LSG_NAN_DETECTED;
        out->done = 1;
        out->iters = it;
        return;
    }
    if (out->restarts >= max_outer) {
        out->done = 1;
        out->iters = it;
        return;
    }
    const double target =
        next_target(&out->tol_frac, &out->floor_misses, rho, out->relres, in->relres, out->tol_abs,
                    out->restarts == 0);
    out->restarts++;
    in->stall = 0;
    in->stalled = 0;
    in->best = __longlong_as_double(0x7ff0000000000000LL);  // +inf
    in->tol_abs = target;
    in->rhs_norm = out->rhs_norm;
    __threadfence();
    in->done = 0;
}

__global__ void batch_tick_kernel(BClock *clk, const BCtl *ctl, int count, int p, int mixed) {
    __shared__ int red[32];
    int *flags = reinterpret_cast<int *>(clk + 1);
    int c = 0;
    for (int i = threadIdx.x; i < count; i += blockDim.x) {
        const DevCtrl *d = mixed ? ctl[i].octrl : ctl[i].ctrl;
        const int f = ctrl_done(d) ? 1 : 0;
        flags[i] = f;
        c += f;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int tot = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) tot += red[w];
        clk->ndone = tot;
        clk->it0 += p;
    }
}

__global__ void finalize_cg_kernel(const double *partials, int nparts, DevCtrl *ctrl, int mode,
                                   double cf, int precond, int iter, int max_iter) {
    __shared__ double red[32];
    if (ctrl_done(ctrl)) return;
    const double sum = block_sum_partials(partials, nparts, 1, 0, red);
    if (threadIdx.x != 0) return;
    if (mode == 0) {  // alpha = delta / (d . q)
        ctrl->dq = sum;
        ctrl->alpha = ctrl->delta / sum;
        if (!isfinite(ctrl->alpha)) { ctrl->status = LSG_NAN_DETECTED; ctrl->done = 1; ctrl->iters = iter; }
        return;
    }
    // mode 1: after the residual update of iteration `iter` (1-based count);
    // mode 2: initial residual (iter = 0).
    const double delta_new = precond ? cf * sum : sum;
    const double relres = sqrt(sum);
    const double delta_old = ctrl->delta;
    ctrl->delta = delta_new;
    ctrl->relres = relres;
    ctrl->beta = mode == 2 ? 0.0 : delta_new / delta_old;
    if (!isfinite(relres)) {
        ctrl->status = LSG_NAN_DETECTED;
        ctrl->done = 1;
        ctrl->iters = iter;
    } else if (!(relres > ctrl->tol_abs) || iter >= max_iter) {
        ctrl->done = 1;
        ctrl->iters = iter;
    }
}

__global__ void pinv_kernel(const double *A, const double *b, double *x, int m, int *status) {
    __shared__ double G[LSG_MAX_M * LSG_MAX_M], V[LSG_MAX_M * LSG_MAX_M], h[LSG_MAX_M], s[LSG_MAX_M];
    __shared__ double Gs[64], Vs[64];
    for (int i = threadIdx.x; i < m * m; i += 32) G[i] = A[i];
    for (int i = threadIdx.x; i < m; i += 32) h[i] = b[i];
    __syncwarp();
    const int st = warp_pinv_any(G, V, h, s, m, Gs, Vs, m * kPinvEps);
    __syncwarp();
    if (threadIdx.x < m) x[threadIdx.x] = s[threadIdx.x];
    if (threadIdx.x == 0 && status) *status = st;
}

// ---------------------------------------------------------------- launchers

cudaError_t finalize_norm(const double *partials, int nparts, DevCtrl *ctrl, int mode, double tol,
                          int iter, cudaStream_t s, int width) {
    finalize_norm_kernel<<<1, kFinThreads, 0, s>>>(partials, nparts, ctrl, mode, tol, iter, width);
    return cudaGetLastError();
}

cudaError_t finalize_gram_solve(double *partials, int nparts, int kind, int m, double hscale, DevCtrl *ctrl,
                                cudaStream_t s) {
    const int blocks = (gram_values(kind, m) + kFinWarps - 1) / kFinWarps;
    finalize_gram_solve_kernel<<<blocks, kFinThreads, 0, s>>>(partials, nparts, kind, m, hscale, ctrl);
    return cudaGetLastError();
}

cudaError_t finalize_gram_solve_c(double *partials, int nparts, int m, cplx<double> hscale, DevCtrl *ctrl,
                                  cudaStream_t s) {
    if (2 * m > LSG_MAX_M) return cudaErrorInvalidValue;
    const int blocks = (m * (m + 1) + 2 * m + kFinWarps - 1) / kFinWarps;
    finalize_gram_solve_c_kernel<<<blocks, kFinThreads, 0, s>>>(partials, nparts, m, hscale.x, hscale.y, ctrl);
    return cudaGetLastError();
}

cudaError_t finalize_cg(const double *partials, int nparts, DevCtrl *ctrl, int mode, double cf,
                        int precond, int iter, int max_iter, cudaStream_t s) {
    finalize_cg_kernel<<<1, kFinThreads, 0, s>>>(partials, nparts, ctrl, mode, cf, precond, iter, max_iter);
    return cudaGetLastError();
}

cudaError_t batch_finalize_norm(const BArgs &a, const int *amap, int nact, int kind, double tol,
                                int width, cudaStream_t s) {
    if (nact <= 0) return cudaSuccess;
    batch_finalize_norm_kernel<<<nact, kFinThreads, 0, s>>>(a, amap, kind, tol, width);
    return cudaGetLastError();
}

cudaError_t batch_finalize_gram(const BArgs &a, const int *amap, int nact, bool complex_gram,
                                cudaStream_t s) {
    if (nact <= 0) return cudaSuccess;
    if (complex_gram && 2 * a.m > LSG_MAX_M) return cudaErrorInvalidValue;
    batch_finalize_gram_kernel<<<nact, kFinThreads, 0, s>>>(a, amap, complex_gram ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t batch_resume(const BArgs &a, const int *amap, int nact, double rho, int max_outer,
                         cudaStream_t s) {
    if (nact <= 0) return cudaSuccess;
    batch_resume_kernel<<<(nact + 127) / 128, 128, 0, s>>>(a, amap, nact, rho, max_outer);
    return cudaGetLastError();
}

cudaError_t batch_tick(BClock *clk, const BCtl *ctl, int count, int p, bool mixed, cudaStream_t s) {
    batch_tick_kernel<<<1, 256, 0, s>>>(clk, ctl, count, p, mixed ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t pinv_solve_dev(const double *A, const double *b, double *x, int m, int *status,
                           cudaStream_t s) {
    pinv_kernel<<<1, 32, 0, s>>>(A, b, x, m, status);
    return cudaGetLastError();
}

}  // namespace lsg

// ---------------------------------------------------------------- allocation-free pinv solve
//
// lsg_pinv_solve_noalloc: the m x m pseudo-inverse solve for callers that must
// not allocate device memory.  lsg_pinv_solve allocates the kernel's status
// word with cudaMallocAsync on every call; this variant keeps it in the
// file-scope array below instead.  Callers that cannot call cudaMalloc
// include code that runs while the device memory is already owned by an
// external pool (an application allocator or a memory-capped MPS client,
// where a new allocation fails or breaks its budget) and latency-bound
// loops that call the small solve every few iterations and cannot afford an
// allocation round trip each time.
//
// The scratch is LSG_PINV_NOALLOC_SCRATCH_INTS ints (256 bytes), held on
// every GPU that loads the library until the process exits.  Every call
// shares it and it keeps the last call's contents, so the status word is
// cleared on the call's stream before each launch; calls that overlap on the
// GPU (different streams, or threads) race on it.  The device address of the
// array is looked up once per device by the first call made with that device
// current.  The address is cached for the life of the process: after cudaDeviceReset (a new
// primary context) it would be stale, so the call is not to be used after a
// device reset.  Each call waits for its stream: the status word is read back
// before the call returns.

#define LSG_PINV_NOALLOC_SCRATCH_INTS 64
static __device__ __align__(256) int g_pinv_noalloc_scratch[LSG_PINV_NOALLOC_SCRATCH_INTS];

namespace {

std::mutex g_noalloc_mu;
constexpr int kNoallocMaxDevices = 64;
int *g_noalloc_addr[kNoallocMaxDevices];

}  // namespace

extern "C" int lsg_pinv_solve_noalloc(const double *d_A, const double *d_b, double *d_x, int m,
                                      void *stream) {
    if (m < 1 || m > LSG_MAX_M)
        return lsg::set_error(LSG_BAD_ARG,
                              "lsg_pinv_solve_noalloc: m = %d outside 1..%d (the allocation-free "
                              "solve keeps its m x m work in shared memory)", m, LSG_MAX_M);
    if (!d_A || !d_b || !d_x) return lsg::set_error(LSG_BAD_ARG, "lsg_pinv_solve_noalloc: NULL pointer");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return lsg::set_error(LSG_CUDA_ERROR, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kNoallocMaxDevices)
        return lsg::set_error(LSG_UNSUPPORTED, "lsg_pinv_solve_noalloc: device %d beyond %d", dev,
                              kNoallocMaxDevices);
    int *scratch = nullptr;
    {
        std::lock_guard<std::mutex> g(g_noalloc_mu);
        if (!g_noalloc_addr[dev]) {
            // One-time set-up on this device (current): the host-side name of the
            // array is not a device address, so ask the runtime for it.
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_pinv_noalloc_scratch);
            if (e != cudaSuccess)
                return lsg::set_error(LSG_CUDA_ERROR, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            g_noalloc_addr[dev] = (int *)p;
        }
        scratch = g_noalloc_addr[dev];
    }
    cudaStream_t s = (cudaStream_t)stream;
    e = cudaMemsetAsync(scratch, 0, sizeof(int), s);
    if (e != cudaSuccess) return lsg::set_error(LSG_CUDA_ERROR, "cudaMemsetAsync: %s", cudaGetErrorString(e));
    lsg::pinv_kernel<<<1, 32, 0, s>>>(d_A, d_b, d_x, m, scratch);
    e = cudaGetLastError();
    if (e != cudaSuccess) return lsg::set_error(LSG_CUDA_ERROR, "pinv launch: %s", cudaGetErrorString(e));
    int st = 0;
    e = cudaMemcpyAsync(&st, scratch, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return lsg::set_error(LSG_CUDA_ERROR, "status read: %s", cudaGetErrorString(e));
    return st;
}

