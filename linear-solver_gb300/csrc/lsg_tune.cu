// lsg_tune.cu — autotuner of the stencil launch shape.
//
// The Richardson pass is ~5/6 of an AAR solve's stencil passes.  Its launch
// shape -- the xy tile (32 x TY columns per block, rows per thread, launch
// bounds) and the z-march depth (planes per block, hence z chunks and waves)
// -- is picked per vector type and grid by timing every candidate on the
// device: each tile variant at its one-wave depth, half and twice that, the
// full column and the wave-balanced depth of the cost model in choose_lz.  Entries are cached per (device, vector type, grid); solves
// use a cached entry when one exists (mode 1, the default), may tune grids
// they meet for the first time (mode 2), or ignore the cache (mode 0).  The
// cache can be saved to and loaded from a text file.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "lsg_internal.cuh"
#include "lsg_host.h"

namespace lsg {

using TuneKey = std::tuple<int, int, int, int, int>;  // device, dtype, nx, ny, nz
static std::mutex g_tune_mu;
static std::map<TuneKey, TuneEntry> g_tune;
static int g_tune_mode = -1;

int tune_mode() {
    std::lock_guard<std::mutex> g(g_tune_mu);
    if (g_tune_mode < 0) {
        const char *e = getenv("LSG_AUTOTUNE");
        g_tune_mode = (e && *e) ? std::max(0, std::min(2, atoi(e))) : 1;
    }
    return g_tune_mode;
}

void set_tune_mode(int mode) {
    std::lock_guard<std::mutex> g(g_tune_mu);
    g_tune_mode = std::max(0, std::min(2, mode));
}

static TuneKey tune_key(int dtype, const Geom &g) {
    int dev = 0;
    cudaGetDevice(&dev);
    return TuneKey{dev, dtype, g.nx, g.ny, g.nz};
}

bool tune_lookup(int dtype, const Geom &g, TuneEntry *e) {
    if (tune_mode() == 0) return false;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(tune_key(dtype, g));
    if (it == g_tune.end()) return false;
    *e = it->second;
    return true;
}

template <typename T> static int dtype_of();
template <> int dtype_of<double>() { return LSG_F64; }
template <> int dtype_of<float>() { return LSG_F32; }
template <> int dtype_of<cplx<double>>() { return LSG_C128; }
template <> int dtype_of<cplx<float>>() { return LSG_C64; }

// Fills the tuner's scratch vectors with values in [-0.5, 0.5) (a hash of the
// index), so the passes time the arithmetic of real data (zeros take the
// double-float split's flush path).
template <typename T>
__global__ void tune_fill_kernel(T *v, long long n) {
    using R = typename RealOf<T>::type;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        unsigned h = (unsigned)i * 2654435761u;
        h ^= h >> 15;
        h *= 2246822519u;
        h ^= h >> 13;
        const R a = (R)((double)h * (1.0 / 4294967296.0) - 0.5);
        if constexpr (IsCplx<T>::value) v[i] = T(a, (R)0.25 * a);
        else v[i] = a;
    }
}

// Times `reps` launches of the Richardson pass in shape (tile, lz); ms per launch.
// FP32 vectors time the pass of the AAR form in use: the residual ring's
// (r' only) by default, else the lean recurrence pass (x left out).
template <typename T>
static int time_rich(const StencilLaunch &L, const Weights<T> &w, T *v, long long n, const DevCtrl *ctrl,
                     cudaEvent_t e0, cudaEvent_t e1, float *ms) {
    constexpr bool recur = std::is_same<typename RealOf<T>::type, float>::value;
    using S = typename ScalarOf<T>::type;
    const S c = S(0.5), cf = S(1.0);
    T *x = v, *r = v + n, *r2 = v + 2 * n, *dx = v + 3 * n, *df = v + 4 * n, *x2 = v + 5 * n;
    const T *b = v + 6 * n;
    auto launch = [&]() -> cudaError_t {
        if constexpr (std::is_same<T, float>::value)
            if (aar_form() == 0) return Kernels<T>::ring_richardson(L, w, r, r2, c, ctrl);
        if (recur) return Kernels<T>::richardson_lean(L, w, r, r2, dx, df, c, cf, 0.5, ctrl);
        return Kernels<T>::richardson(L, w, RICH_AAR, x, r, b, x2, r2, dx, df, c, cf, 0.5, ctrl);
    };
    for (int k = 0; k < 2; k++)
        if (launch() != cudaSuccess) return set_error(LSG_CUDA_ERROR, "autotune launch failed");
    const int reps = 5;
    cudaEventRecord(e0, L.stream);
    for (int k = 0; k < reps; k++) launch();
    cudaEventRecord(e1, L.stream);
    cudaError_t e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) return set_error(LSG_CUDA_ERROR, "autotune: %s", cudaGetErrorString(e));
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    *ms = t / reps;
    return LSG_OK;
}

// Tunes the Richardson pass of `op` for vector type T on `stream`.
template <typename T>
static int tune_t(const lsg_operator *op, cudaStream_t s, TuneEntry *out, int *ncand) {
    const Geom g = make_geom(op->n);
    const long long n = g.n;
    const Weights<T> w = make_weights<T>(op);
    const int sms = sm_count();
    // scratch: x r r2 dx df x2 b (contiguous, n values each) and a control
    // block that never stops the pass
    const size_t vb = (size_t)n * sizeof(T);
    const size_t cb = (7 * vb + 255) & ~(size_t)255;
    char *buf = nullptr;
    cudaError_t e = cudaMalloc(&buf, cb + 256);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(LSG_NO_MEMORY, "autotune scratch of %zu bytes: %s", cb, cudaGetErrorString(e));
    }
    T *v = (T *)buf;
    DevCtrl *ctrl = (DevCtrl *)(buf + cb);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int rc = LSG_OK;
    if (cudaMemsetAsync(buf, 0, cb + 256, s) != cudaSuccess) rc = set_error(LSG_CUDA_ERROR, "autotune memset");
    tune_fill_kernel<T><<<sms * 4, 256, 0, s>>>(v, 7 * n);
    if (cudaGetLastError() != cudaSuccess) rc = set_error(LSG_CUDA_ERROR, "autotune fill");
    TuneEntry best;
    best.tile = 0;
    const int lz_default = choose_lz<T>(g, sms * Kernels<T>::stencil_blocks_per_sm(0));
    best.lz = lz_default;
    best.us = 1e30;
    best.us_default = 0;
    int count = 0;
    for (int var = 0; var < kTileVariants && rc == LSG_OK; var++) {
        const int slots = sms * Kernels<T>::stencil_blocks_per_sm(var);
        const int lz1 = one_wave_lz(g, tile_var_rows<T>(var), slots);
        std::vector<int> cands{lz1, std::max(8, lz1 / 2), std::min(g.nz, 2 * lz1), g.nz,
                               balanced_lz(g, tile_var_rows<T>(var), slots, FillCost<T>::value)};
        if (var == 0) cands.push_back(lz_default);
        std::sort(cands.begin(), cands.end());
        cands.erase(std::unique(cands.begin(), cands.end()), cands.end());
        for (int lz : cands) {
            if (lz < 1 || lz > g.nz) continue;
            StencilLaunch L{g, lz, s, var};
            L.exact = fp64_exact();
            float ms = 0.f;
            rc = time_rich<T>(L, w, v, n, ctrl, e0, e1, &ms);
            if (rc != LSG_OK) break;
            count++;
            const double us = 1000.0 * ms;
            if (var == 0 && lz == lz_default) best.us_default = us;
            if (us < best.us) {
                best.us = us;
                best.tile = var;
                best.lz = lz;
            }
        }
    }
    // the paired march of the FP32 recurrence pass in its two shapes (tile
    // codes kTilePaired, kTilePaired2) x the same kinds of z depth
    int plz = 0;
    if (rc == LSG_OK && Kernels<T>::paired_plan(g, &plz) > 0 && std::is_same<T, float>::value &&
        g.nx % 2 == 0) {
        for (int shape = 1; shape <= 3 && rc == LSG_OK; shape++) {
            const int rows = shape == 1 ? kPairBY * kPairNY : shape == 2 ? kPair2BY * kPair2NY : kPair3BY * kPair3NY;
            const int slots = sms * Kernels<T>::paired_blocks_per_sm(shape);
            const long long bxy = (long long)((g.nx + 63) / 64) * ((g.ny + rows - 1) / rows);
            const long long chunks = std::max<long long>(1, bxy >= slots ? 1 : slots / bxy);
            const int lz1 = std::max(8, std::min(g.nz, (int)((g.nz + chunks - 1) / chunks)));
            std::vector<int> cands{lz1, std::max(8, lz1 / 2), std::min(g.nz, 2 * lz1), g.nz,
                                   balanced_lz(g, rows, slots, FillCost<T>::value, 64)};
            if (shape == 1) cands.push_back(plz);
            std::sort(cands.begin(), cands.end());
            cands.erase(std::unique(cands.begin(), cands.end()), cands.end());
            for (int lz : cands) {
                if (lz < 1 || lz > g.nz) continue;
                StencilLaunch L{g, lz, s, 0};
                L.paired = shape;
                float ms = 0.f;
                rc = time_rich<T>(L, w, v, n, ctrl, e0, e1, &ms);
                if (rc != LSG_OK) break;
                count++;
                const double us = 1000.0 * ms;
                if (shape == 1 && lz == plz) best.us_default = us;  // the untuned solve runs this one
                if (us < best.us) {
                    best.us = us;
                    best.tile = shape == 1 ? kTilePaired : shape == 2 ? kTilePaired2 : kTilePaired3;
                    best.lz = lz;
                }
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamSynchronize(s);
    cudaFree(buf);
    if (rc != LSG_OK) return rc;
    *out = best;
    *ncand = count;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[tune_key(dtype_of<T>(), g)] = best;
    return LSG_OK;
}

int autotune(const lsg_operator *op, int dtype, TuneEntry *out, int *ncand, cudaStream_t s) {
    int rc = check_operator(op);
    if (rc) return rc;
    if (op->radius != 6) return set_error(LSG_UNSUPPORTED, "autotune: tile variants exist for radius 6 only");
    switch (dtype) {
    case LSG_F64: return tune_t<double>(op, s, out, ncand);
    case LSG_F32: return tune_t<float>(op, s, out, ncand);
    case LSG_C128: return tune_t<cplx<double>>(op, s, out, ncand);
    case LSG_C64: return tune_t<cplx<float>>(op, s, out, ncand);
    default: return set_error(LSG_BAD_ARG, "unknown dtype %d", dtype);
    }
}

// Launch shape of the Richardson pass: the cached entry, a fresh tuning in
// mode 2, or the default shape `L`.
template <typename T>
StencilLaunch rich_launch(const lsg_operator *op, const StencilLaunch &L) {
    if (op->radius != 6) return L;
    const Geom g = make_geom(op->n);
    TuneEntry e;
    if (!tune_lookup(dtype_of<T>(), g, &e)) {
        if (tune_mode() != 2) return L;
        int nc = 0;
        if (tune_t<T>(op, L.stream, &e, &nc) != LSG_OK) {
            set_last_status(LSG_OK);
            return L;
        }
    }
    StencilLaunch r = L;
    if (e.tile == kTilePaired || e.tile == kTilePaired2 || e.tile == kTilePaired3) {
        r.tile = 0;
        r.paired = e.tile == kTilePaired ? 1 : e.tile == kTilePaired2 ? 2 : 3;
    } else {
        r.tile = e.tile;
        r.paired = 0;  // a tuned classic shape
    }
    r.lz = e.lz;
    return r;
}
template StencilLaunch rich_launch<double>(const lsg_operator *, const StencilLaunch &);
template StencilLaunch rich_launch<float>(const lsg_operator *, const StencilLaunch &);
template StencilLaunch rich_launch<cplx<double>>(const lsg_operator *, const StencilLaunch &);
template StencilLaunch rich_launch<cplx<float>>(const lsg_operator *, const StencilLaunch &);

int tune_save(const char *path) {
    if (!path) return set_error(LSG_BAD_ARG, "NULL path");
    FILE *f = fopen(path, "w");
    if (!f) return set_error(LSG_BAD_ARG, "cannot write %s", path);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    fprintf(f, "# lsg autotune cache: device dtype nx ny nz tile lz us us_default\n");
    for (const auto &kv : g_tune) {
        const TuneKey &k = kv.first;
        const TuneEntry &e = kv.second;
        fprintf(f, "%d %d %d %d %d %d %d %.3f %.3f\n", std::get<0>(k), std::get<1>(k), std::get<2>(k),
                std::get<3>(k), std::get<4>(k), e.tile, e.lz, e.us, e.us_default);
    }
    fclose(f);
    return LSG_OK;
}

int tune_load(const char *path, int *count) {
    if (!path) return set_error(LSG_BAD_ARG, "NULL path");
    FILE *f = fopen(path, "r");
    if (!f) return set_error(LSG_BAD_ARG, "cannot read %s", path);
    char line[256];
    int loaded = 0;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    while (fgets(line, sizeof(line), f)) {
        if (line[0] == '#') continue;
        int dev, dt, nx, ny, nz, tile, lz;
        double us, usd;
        if (sscanf(line, "%d %d %d %d %d %d %d %lf %lf", &dev, &dt, &nx, &ny, &nz, &tile, &lz, &us, &usd) != 9)
            continue;
        if (tile < 0 || (tile >= kTileVariants && tile != kTilePaired && tile != kTilePaired2 && tile != kTilePaired3) ||
            lz < 1 ||
            lz > nz)
            continue;
        g_tune[TuneKey{dev, dt, nx, ny, nz}] = TuneEntry{tile, lz, us, usd};
        loaded++;
    }
    fclose(f);
    if (count) *count = loaded;
    return LSG_OK;
}

}  // namespace lsg

extern "C" {

int lsg_autotune(const lsg_operator *op, int dtype, lsg_tune_info *info, void *stream) {
    lsg::TuneEntry e;
    int nc = 0;
    const int rc = lsg::autotune(op, dtype, &e, &nc, (cudaStream_t)stream);
    if (rc != LSG_OK) return rc;
    if (info) {
        int by = 0, ny = 0;
        auto shape = [&](auto tag) {
            using T = decltype(tag);
            if (e.tile == lsg::kTilePaired) {  // 32 x 8 threads, 2 rows x 2 columns each
                by = lsg::kPairBY;
                ny = lsg::kPairNY;
                return;
            }
            if (e.tile == lsg::kTilePaired2) {  // 32 x 4 threads, 2 rows x 2 columns each
                by = lsg::kPair2BY;
                ny = lsg::kPair2NY;
                return;
            }
            if (e.tile == lsg::kTilePaired3) {  // 32 x 8 threads, 4 rows x 2 columns each
                by = lsg::kPair3BY;
                ny = lsg::kPair3NY;
                return;
            }
            switch (e.tile) {
            case 1: by = lsg::TileVar<T, 1>::BY; ny = lsg::TileVar<T, 1>::NY; break;
            case 2: by = lsg::TileVar<T, 2>::BY; ny = lsg::TileVar<T, 2>::NY; break;
            default: by = lsg::TileVar<T, 0>::BY; ny = lsg::TileVar<T, 0>::NY;
            }
        };
        if (dtype == LSG_F64) shape(double());
        else if (dtype == LSG_F32) shape(float());
        else if (dtype == LSG_C128) shape(lsg::cplx<double>());
        else shape(lsg::cplx<float>());
        info->tile = e.tile;
        info->threads_y = by;
        info->rows_per_thread = ny;
        info->lz = e.lz;
        info->us_best = e.us;
        info->us_default = e.us_default;
        info->candidates = nc;
    }
    return LSG_OK;
}

int lsg_set_autotune(int mode) {
    if (mode < 0 || mode > 2) return lsg::set_error(LSG_BAD_ARG, "autotune mode %d outside 0..2", mode);
    lsg::set_tune_mode(mode);
    return LSG_OK;
}

int lsg_autotune_save(const char *path) { return lsg::tune_save(path); }
int lsg_autotune_load(const char *path, int *count) { return lsg::tune_load(path, count); }

}  // extern "C"
