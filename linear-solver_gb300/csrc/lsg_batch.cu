// lsg_batch.cu — batched AAR: many independent solves (own grid size, shift
// and coefficients; shared omega, beta, m, p, tol) in lockstep on one stream.
//
// Every pass is ONE launch over all active instances (lsg_batch.cuh), and one
// extrapolation cycle -- p-1 Richardson passes, the Gram / m x m solve /
// update / residual of the extrapolation iteration, the convergence tests,
// for mixed solves the FP64 residual replacement of paused instances, and a
// clock tick -- is captured once as a CUDA graph and replayed.  The
// iteration number, history column and ping-pong parity live on the device
// (BClock), so the replayed graph needs no parameter updates.
//
// Each instance follows the single-solve iteration of lsg_solvers.cu exactly
// (AAR.c:37-177 numbering; mixed: the FP32 iteration paused when its residual
// fell by rho, FP64 residual replacement, resumed with the history kept), so a
// batched instance reproduces its single solve up to the summation order of
// the reductions.  Instances that finish are skipped through their control
// blocks; when the active set has shrunk enough, the launch plan (blocks per
// instance, z planes per stencil block) is rebuilt for the remaining ones and
// the cycle re-captured, so the GPU stays filled to the last instance.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>
#include <vector>

#include "lsg_internal.cuh"
#include "lsg_host.h"

namespace lsg {

#define LSG_BCUDA(call)                                                                      \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return cudaGetLastError(), /* clear it for later launches */                     \
                   set_error(e_ == cudaErrorMemoryAllocation ? LSG_NO_MEMORY : LSG_CUDA_ERROR, \
                             "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

static size_t al256(size_t v) { return (v + 255) & ~(size_t)255; }

// Launch plan of the active instances.
struct BPlan {
    std::vector<int> act;     // active instances
    int var = 0;              // tile variant of the stencil passes
    int sgrid = 0, ugrid = 0;
    int pgrid = 0;            // paired-march Richardson blocks (0: the one-column march)
    long long points = 0;     // grid points of the active instances
};

// Work arrays, tables and the captured cycle of one batch shape.
struct BatchWs {
    std::mutex mu;
    int count = 0;
    char *base = nullptr;         // device: vectors, partials, control blocks, tables
    char *host = nullptr;         // pinned mirrors of the tables
    size_t inst_bytes = 0;
    BCtl *d_ctl = nullptr, *h_ctl = nullptr;
    void *d_inst = nullptr, *h_inst = nullptr;
    int *d_smap = nullptr, *h_smap = nullptr;
    int *d_umap = nullptr, *h_umap = nullptr;
    int *d_pmap = nullptr, *h_pmap = nullptr;  // FP32: paired-march Richardson blocks
    int *d_amap = nullptr, *h_amap = nullptr;
    BClock *d_clk = nullptr, *h_clk = nullptr;  // BClock + count done flags; host: 2 slots
    DevCtrl *d_ctrl = nullptr, *h_ctrl = nullptr;  // 2 per instance: ctrl, octrl
    size_t clk_bytes = 0;
    long long smap_cap = 0, umap_cap = 0, pmap_cap = 0;
    int paired = 0;               // this solve's Richardson passes run the paired march
    std::vector<char *> vec;      // per instance: xalt r0 r1 dx[m] df[m] (e) (FP32: rs)
    std::vector<double *> part;
    std::vector<long long> part_cap;
    int tuned = 0;               // 1: tile variant and z-depth scale measured for this batch
    int tvar = 0;
    double tscale = 1.0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaEvent_t join = nullptr;
    cudaGraphExec_t exec = nullptr;
    ~BatchWs() {
        if (exec) cudaGraphExecDestroy(exec);
        if (base) cudaFree(base);
        if (host) cudaFreeHost(host);
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
        if (join) cudaEventDestroy(join);
        if (stream) cudaStreamDestroy(stream);
    }
};

using BKey = std::tuple<int, int, int, int, std::vector<long long>>;
static std::mutex g_bws_mu;
static std::map<BKey, std::unique_ptr<BatchWs>> g_bws;

int release_batch_workspaces() {
    std::lock_guard<std::mutex> g(g_bws_mu);
    g_bws.clear();
    return LSG_OK;
}

// Stencil tiles of one instance.
static void tiles_of(const Geom &g, int ty, int *tx, int *tyn) {
    *tx = (g.nx + 31) / 32;
    *tyn = (g.ny + ty - 1) / ty;
}

// Upper bound of the stencil blocks of one instance over all plans (z chunks of >= 8 planes).
static long long max_sblocks(const Geom &g, int ty) {
    int tx, tyn;
    tiles_of(g, ty, &tx, &tyn);
    const int lzmin = std::min(8, g.nz);
    return (long long)tx * tyn * ((g.nz + lzmin - 1) / lzmin);
}

// Paired-march tiles of one instance (64 columns x kPairBY * kPairNY rows)
// and their upper bound over all plans.
static void ptiles_of(const Geom &g, int *tx, int *tyn) {
    *tx = (g.nx + 63) / 64;
    *tyn = (g.ny + kPairBY * kPairNY - 1) / (kPairBY * kPairNY);
}
static long long max_pblocks(const Geom &g) {
    int tx, tyn;
    ptiles_of(g, &tx, &tyn);
    const int lzmin = std::min(8, g.nz);
    return (long long)tx * tyn * ((g.nz + lzmin - 1) / lzmin);
}

static const int kUcapPerSm = 8;

// lsg_set_batch_march: 1 (default) lets FP32 batches run the paired march.
static std::atomic<int> g_batch_paired{1};
static bool batch_paired_enabled() { return g_batch_paired.load(std::memory_order_relaxed) != 0; }  // point-local blocks (256 threads) per SM over the batch

template <typename T>
static int batch_ws_get(const std::vector<Geom> &geo, int m, bool mixed, bool generic, BatchWs **out,
                        std::unique_lock<std::mutex> *lock) {
    int dev = 0;
    cudaGetDevice(&dev);
    const int count = (int)geo.size();
    std::vector<long long> shape;
    for (const Geom &g : geo) { shape.push_back(g.nx); shape.push_back(g.ny); shape.push_back(g.nz); }
    BKey key{dev, (int)sizeof(T) * (IsCplx<T>::value ? -1 : 1), m, (mixed ? 2 : 0) + (generic ? 1 : 0), shape};
    BatchWs *ws;
    {
        std::lock_guard<std::mutex> g(g_bws_mu);
        auto &slot = g_bws[key];
        if (!slot) slot.reset(new BatchWs());
        ws = slot.get();
    }
    *lock = std::unique_lock<std::mutex>(ws->mu);
    if (ws->base) { *out = ws; return LSG_OK; }

    const int sms = sm_count();
    int ty = BatchKernels<T>::tile_y(generic, 0);  // fewest rows over the variants: most blocks
    for (int v = 1; v < kTileVariants && !generic; v++) ty = std::min(ty, BatchKernels<T>::tile_y(false, v));
    const int W = AccWidth<T>::value;
    const long long nvmax = (long long)(m * (m + 1)) / 2 + m;
    const long long ucap = (long long)kUcapPerSm * sms;
    const size_t es = sizeof(T);
    const int nvec = 3 + 2 * m + (mixed ? 1 : 0) + (IsRecur<T>::value ? 1 : 0);
    size_t bytes = 0;
    std::vector<size_t> o_vec(count), o_part(count);
    ws->part_cap.resize(count);
    long long smap_cap = 0, pmap_cap = 0;
    for (int i = 0; i < count; i++) {
        if (std::is_same<T, float>::value) pmap_cap += max_pblocks(geo[i]);
        o_vec[i] = bytes;
        bytes += (size_t)nvec * al256((size_t)geo[i].n * es);
        const long long sb = max_sblocks(geo[i], ty);
        const long long ub = std::min<long long>((geo[i].n + 255) / 256, ucap);
        ws->part_cap[i] = std::max(sb * W, ub * nvmax * W);
        smap_cap += sb;
    }
    for (int i = 0; i < count; i++) {
        o_part[i] = bytes;
        bytes += al256((size_t)ws->part_cap[i] * 8);
    }
    ws->smap_cap = smap_cap;
    ws->pmap_cap = pmap_cap;
    ws->umap_cap = ucap + count;
    ws->inst_bytes = sizeof(BInst<T>) * count;
    ws->clk_bytes = al256(sizeof(BClock) + sizeof(int) * count);
    const size_t o_ctrl = bytes; bytes += al256(sizeof(DevCtrl) * 2 * count);
    const size_t o_ctl = bytes; bytes += al256(sizeof(BCtl) * count);
    const size_t o_inst = bytes; bytes += al256(ws->inst_bytes);
    const size_t o_smap = bytes; bytes += al256(sizeof(int) * smap_cap);
    const size_t o_umap = bytes; bytes += al256(sizeof(int) * ws->umap_cap);
    const size_t o_pmap = bytes; bytes += al256(sizeof(int) * pmap_cap);
    const size_t o_amap = bytes; bytes += al256(sizeof(int) * count);
    const size_t o_clk = bytes; bytes += ws->clk_bytes;
    cudaError_t e = cudaMalloc(&ws->base, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        ws->base = nullptr;
        return set_error(LSG_NO_MEMORY, "cudaMalloc of %zu bytes for the batch failed: %s", bytes,
                         cudaGetErrorString(e));
    }
    // pinned mirrors: ctrl, ctl, inst, smap, umap, amap, clk x 2
    const size_t hb_ctrl = 0;
    size_t hbytes = al256(sizeof(DevCtrl) * 2 * count);
    const size_t hb_ctl = hbytes; hbytes += al256(sizeof(BCtl) * count);
    const size_t hb_inst = hbytes; hbytes += al256(ws->inst_bytes);
    const size_t hb_smap = hbytes; hbytes += al256(sizeof(int) * smap_cap);
    const size_t hb_umap = hbytes; hbytes += al256(sizeof(int) * ws->umap_cap);
    const size_t hb_pmap = hbytes; hbytes += al256(sizeof(int) * pmap_cap);
    const size_t hb_amap = hbytes; hbytes += al256(sizeof(int) * count);
    const size_t hb_clk = hbytes; hbytes += 2 * ws->clk_bytes;
    e = cudaMallocHost(&ws->host, hbytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        cudaFree(ws->base);
        ws->base = nullptr;
        ws->host = nullptr;
        return set_error(LSG_NO_MEMORY, "cudaMallocHost of %zu bytes failed: %s", hbytes, cudaGetErrorString(e));
    }
    ws->count = count;
    ws->vec.resize(count);
    ws->part.resize(count);
    for (int i = 0; i < count; i++) {
        ws->vec[i] = ws->base + o_vec[i];
        ws->part[i] = (double *)(ws->base + o_part[i]);
    }
    ws->d_ctrl = (DevCtrl *)(ws->base + o_ctrl);
    ws->d_ctl = (BCtl *)(ws->base + o_ctl);
    ws->d_inst = ws->base + o_inst;
    ws->d_smap = (int *)(ws->base + o_smap);
    ws->d_umap = (int *)(ws->base + o_umap);
    ws->d_pmap = (int *)(ws->base + o_pmap);
    ws->d_amap = (int *)(ws->base + o_amap);
    ws->d_clk = (BClock *)(ws->base + o_clk);
    ws->h_ctrl = (DevCtrl *)(ws->host + hb_ctrl);
    ws->h_ctl = (BCtl *)(ws->host + hb_ctl);
    ws->h_inst = ws->host + hb_inst;
    ws->h_smap = (int *)(ws->host + hb_smap);
    ws->h_umap = (int *)(ws->host + hb_umap);
    ws->h_pmap = (int *)(ws->host + hb_pmap);
    ws->h_amap = (int *)(ws->host + hb_amap);
    ws->h_clk = (BClock *)(ws->host + hb_clk);
    LSG_BCUDA(cudaStreamCreateWithFlags(&ws->stream, cudaStreamNonBlocking));
    LSG_BCUDA(cudaEventCreateWithFlags(&ws->ev[0], cudaEventDisableTiming));
    LSG_BCUDA(cudaEventCreateWithFlags(&ws->ev[1], cudaEventDisableTiming));
    LSG_BCUDA(cudaEventCreateWithFlags(&ws->join, cudaEventDisableTiming));
    *out = ws;
    return LSG_OK;
}

// Host clock slot k (BClock followed by `count` done flags).
static BClock *clk_slot(BatchWs *ws, int k) { return (BClock *)((char *)ws->h_clk + k * ws->clk_bytes); }
static const int *clk_flags(const BClock *c) { return (const int *)(c + 1); }

// Splits the active instances' work over one launch: point-local passes get
// blocks in proportion to the instance sizes (at least one each); stencil
// passes use the tile grid of each instance with z chunks of a common depth,
// chosen so that all blocks fit in one wave of resident blocks when possible
// (a partial second wave would double the time of its blocks).
template <typename T>
static void make_plan(BatchWs *ws, const std::vector<Geom> &geo, const std::vector<int> &act, bool generic,
                      int var, int slots, double lscale, BPlan *plan) {
    const int ty = BatchKernels<T>::tile_y(generic, var);
    const int sms = sm_count();
    BInst<T> *hi = (BInst<T> *)ws->h_inst;
    plan->act = act;
    plan->points = 0;
    long long bxy_sum = 0, cols = 0;
    int maxnz = 1;
    for (int i : act) {
        int tx, tyn;
        tiles_of(geo[i], ty, &tx, &tyn);
        hi[i].tx = tx;
        hi[i].ty = tyn;
        bxy_sum += (long long)tx * tyn;
        cols += (long long)tx * tyn * geo[i].nz;
        maxnz = std::max(maxnz, geo[i].nz);
        plan->points += geo[i].n;
    }
    int L = maxnz;
    if (bxy_sum < slots) {
        L = (int)std::max<long long>(8, (cols + slots - 1) / slots);
        auto blocks_at = [&](int l) {
            long long b = 0;
            for (int i : act) b += (long long)hi[i].tx * hi[i].ty * ((geo[i].nz + std::min(l, geo[i].nz) - 1) / std::min(l, geo[i].nz));
            return b;
        };
        while (L < maxnz && blocks_at(L) > slots) L++;
        L = std::max(8, std::min(maxnz, (int)(L * lscale + 0.5)));
    }
    plan->var = var;
    int sb0 = 0;
    for (int i : act) {
        const int lz = std::min(L, geo[i].nz);
        hi[i].lz = lz;
        const int nb = hi[i].tx * hi[i].ty * ((geo[i].nz + lz - 1) / lz);
        ws->h_ctl[i].sblk0 = sb0;
        ws->h_ctl[i].sblocks = nb;
        for (int b = 0; b < nb; b++) ws->h_smap[sb0 + b] = i;
        sb0 += nb;
    }
    plan->sgrid = sb0;
    // FP32 Richardson passes: the paired march's own tile grid, its z depth
    // chosen by the same one-wave rule
    plan->pgrid = 0;
    if (ws->paired) {
        const int pslots = sms * std::max(1, BatchKernels<T>::paired_blocks_per_sm());
        long long pxy = 0, pcols = 0;
        for (int i : act) {
            ptiles_of(geo[i], &hi[i].ptx, &hi[i].pty);
            pxy += (long long)hi[i].ptx * hi[i].pty;
            pcols += (long long)hi[i].ptx * hi[i].pty * geo[i].nz;
        }
        int Lp = maxnz;
        if (pxy < pslots) {
            Lp = (int)std::max<long long>(8, (pcols + pslots - 1) / pslots);
            auto pblocks_at = [&](int l) {
                long long b = 0;
                for (int i : act) {
                    const int lz = std::min(l, geo[i].nz);
                    b += (long long)hi[i].ptx * hi[i].pty * ((geo[i].nz + lz - 1) / lz);
                }
                return b;
            };
            while (Lp < maxnz && pblocks_at(Lp) > pslots) Lp++;
            Lp = std::max(8, std::min(maxnz, (int)(Lp * lscale + 0.5)));
        }
        int pb0 = 0;
        for (int i : act) {
            const int lz = std::min(Lp, geo[i].nz);
            hi[i].plz = lz;
            const int nb = hi[i].ptx * hi[i].pty * ((geo[i].nz + lz - 1) / lz);
            ws->h_ctl[i].pblk0 = pb0;
            ws->h_ctl[i].pblocks = nb;
            for (int b = 0; b < nb; b++) ws->h_pmap[pb0 + b] = i;
            pb0 += nb;
        }
        plan->pgrid = pb0;
    }
    long long need = 0;
    for (int i : act) need += (geo[i].n + 255) / 256;
    const long long U = std::min<long long>(need, (long long)kUcapPerSm * sms);
    int ub0 = 0;
    for (int i : act) {
        long long u = (long long)((double)U * (double)geo[i].n / (double)std::max<long long>(1, plan->points));
        u = std::max<long long>(1, std::min<long long>(u, (geo[i].n + 255) / 256));
        ws->h_ctl[i].ublk0 = ub0;
        ws->h_ctl[i].ublocks = (int)u;
        for (long long b = 0; b < u; b++) ws->h_umap[ub0 + b] = i;
        ub0 += (int)u;
    }
    plan->ugrid = ub0;
    for (size_t k = 0; k < act.size(); k++) ws->h_amap[k] = act[k];
}

template <typename T>
static int upload_tables(BatchWs *ws, const BPlan &plan) {
    cudaStream_t s = ws->stream;
    LSG_BCUDA(cudaMemcpyAsync(ws->d_ctl, ws->h_ctl, sizeof(BCtl) * ws->count, cudaMemcpyHostToDevice, s));
    LSG_BCUDA(cudaMemcpyAsync(ws->d_inst, ws->h_inst, ws->inst_bytes, cudaMemcpyHostToDevice, s));
    if (plan.sgrid > 0)
        LSG_BCUDA(cudaMemcpyAsync(ws->d_smap, ws->h_smap, sizeof(int) * plan.sgrid, cudaMemcpyHostToDevice, s));
    if (plan.ugrid > 0)
        LSG_BCUDA(cudaMemcpyAsync(ws->d_umap, ws->h_umap, sizeof(int) * plan.ugrid, cudaMemcpyHostToDevice, s));
    if (plan.pgrid > 0)
        LSG_BCUDA(cudaMemcpyAsync(ws->d_pmap, ws->h_pmap, sizeof(int) * plan.pgrid, cudaMemcpyHostToDevice, s));
    if (!plan.act.empty())
        LSG_BCUDA(cudaMemcpyAsync(ws->d_amap, ws->h_amap, sizeof(int) * plan.act.size(), cudaMemcpyHostToDevice, s));
    return LSG_OK;
}

// Launch wrappers of one batch solve.
template <typename T>
struct BatchRun {
    BatchWs *ws;
    const lsg_params *prm;
    bool mixed, generic;
    double rho;
    int max_outer;
    BPlan plan;
    long long launches = 0;
    bool deflating = false;  // mixed: some instance has a non-zero shift

    BArgs args(const int *map, int k, int gate = 0) const {
        BArgs a;
        a.ctl = ws->d_ctl;
        a.map = map;
        a.clk = ws->d_clk;
        a.k = k;
        a.m = prm->m;
        a.p = prm->p;
        a.max_iter = prm->max_iter;
        a.beta = prm->beta;
        a.gate = gate;
        a.lean = IsRecur<T>::value && prm->p - 1 <= prm->m;
        a.exact = fp64_exact_for(prm->tol);
        return a;
    }
    const BInst<T> *tab() const { return (const BInst<T> *)ws->d_inst; }
    int nact() const { return (int)plan.act.size(); }

#define LSG_BL(call)                                                                          \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        launches++;                                                                           \
        if (e_ != cudaSuccess)                                                                \
            return set_error(LSG_CUDA_ERROR, "batched launch %s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

    // r = b - A x64 of paused (gate 0) or all unfinished (gate 1) instances,
    // after iteration it0 + k + 1; resumes the paused ones (gate 0).
    int refine(int k, int gate) {
        cudaStream_t s = ws->stream;
        const int W = AccWidth<T>::value;
        if (gate == 1) LSG_BL(BatchKernels<T>::fold(tab(), args(ws->d_umap, k, 1), plan.ugrid, s));
        LSG_BL(BatchKernels<T>::ir_correct(tab(), args(ws->d_umap, k, gate), plan.ugrid, s));
        if (deflating) {
            LSG_BL(BatchKernels<T>::mean_deflate(tab(), args(ws->d_umap, k, gate), plan.ugrid, args(nullptr, k, gate),
                                                 ws->d_amap, nact(), 1, s));
            launches += 2;
        }
        LSG_BL(BatchKernels<T>::ir_residual(tab(), args(ws->d_smap, k, gate), plan.sgrid, generic, plan.var, s));
        LSG_BL(batch_finalize_norm(args(nullptr, k, gate), ws->d_amap, nact(), BF_REPLACE, prm->tol, W, s));
        if (gate == 0) LSG_BL(batch_resume(args(nullptr, k, 0), ws->d_amap, nact(), rho, max_outer, s));
        return LSG_OK;
    }
    int richardson(int k) {
        if (plan.pgrid > 0)
            LSG_BL(BatchKernels<T>::richardson_paired(tab(), args(ws->d_pmap, k), plan.pgrid, ws->stream));
        else
            LSG_BL(BatchKernels<T>::richardson(tab(), args(ws->d_smap, k), plan.sgrid, generic, plan.var, ws->stream));
        return LSG_OK;
    }
    // One extrapolation cycle (iterations it0+1 .. it0+p) and the clock tick.
    int cycle() {
        cudaStream_t s = ws->stream;
        const int p = prm->p, W = AccWidth<T>::value;
        for (int k = 0; k + 1 < p; k++) {
            int rc = richardson(k);
            if (rc) return rc;
        }
        const int k = p - 1;
        LSG_BL(BatchKernels<T>::gram(tab(), args(ws->d_umap, k), plan.ugrid, s));
        LSG_BL(batch_finalize_gram(args(nullptr, k), ws->d_amap, nact(), IsCplx<T>::value, s));
        LSG_BL(BatchKernels<T>::update(tab(), args(ws->d_umap, k), plan.ugrid, s));
        LSG_BL(BatchKernels<T>::residual_anderson(tab(), args(ws->d_smap, k), plan.sgrid, generic, plan.var, s));
        LSG_BL(batch_finalize_norm(args(nullptr, k), ws->d_amap, nact(), BF_CHECK, prm->tol, W, s));
        if (mixed) {
            int rc = refine(k, 0);
            if (rc) return rc;
        }
        LSG_BL(batch_tick(ws->d_clk, ws->d_ctl, ws->count, p, mixed, s));
        return LSG_OK;
    }
    // Captures one cycle as a graph (replacing the previous one).
    int capture() {
        if (ws->exec) {
            cudaGraphExecDestroy(ws->exec);
            ws->exec = nullptr;
        }
        LSG_BCUDA(cudaStreamBeginCapture(ws->stream, cudaStreamCaptureModeThreadLocal));
        const long long l0 = launches;
        int rc = cycle();
        cudaGraph_t graph = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(ws->stream, &graph);
        launches = l0;
        if (rc != LSG_OK) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (ce != cudaSuccess) return set_error(LSG_CUDA_ERROR, "cycle capture: %s", cudaGetErrorString(ce));
        const cudaError_t ie = cudaGraphInstantiate(&ws->exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) {
            ws->exec = nullptr;
            return set_error(LSG_CUDA_ERROR, "cycle graph instantiation: %s", cudaGetErrorString(ie));
        }
        return LSG_OK;
    }
    long long per_cycle() const { return (prm->p - 1) + 5 + (mixed ? 4 : 0) + 1; }
};

// Batch autotuner: times the batched Richardson pass (every instance active)
// for each tile variant at the one-wave z depth, half and twice it, and keeps
// the fastest for this batch shape.  Runs before the solve state exists: the
// control blocks are set to "running", and the FP32 plain form (x updated in
// place) writes its iterate to the spare vector instead of the caller's x.
template <typename T>
static int tune_batch(BatchWs *ws, const std::vector<Geom> &geo, const std::vector<int> &act,
                      const lsg_params *prm, bool mixed) {
    const int count = ws->count;
    cudaStream_t s = ws->stream;
    BInst<T> *hi = (BInst<T> *)ws->h_inst;
    std::vector<T *> xsave(count);
    const bool redirect = !mixed && std::is_same<typename RealOf<T>::type, float>::value;
    for (int i = 0; i < count; i++) {
        xsave[i] = hi[i].x;
        if (redirect) hi[i].x = hi[i].xalt;
    }
    std::vector<DevCtrl> run(2 * count, ctrl_init(prm->tol, 0));
    LSG_BCUDA(cudaMemcpyAsync(ws->d_ctrl, run.data(), sizeof(DevCtrl) * 2 * count, cudaMemcpyHostToDevice, s));
    LSG_BCUDA(cudaMemsetAsync(ws->d_clk, 0, ws->clk_bytes, s));
    cudaEvent_t e0, e1;
    LSG_BCUDA(cudaEventCreate(&e0));
    LSG_BCUDA(cudaEventCreate(&e1));
    BatchRun<T> B{ws, prm, mixed, false, 0.0, 0, BPlan(), 0};
    float best = 1e30f;
    int rc = LSG_OK;
    static const double scales[3] = {1.0, 0.5, 2.0};
    for (int var = 0; var < kTileVariants && rc == LSG_OK; var++) {
        const int slots = sm_count() * BatchKernels<T>::stencil_blocks_per_sm(false, var);
        for (double sc : scales) {
            make_plan<T>(ws, geo, act, false, var, slots, sc, &B.plan);
            rc = upload_tables<T>(ws, B.plan);
            if (rc) break;
            for (int k = 0; k < 2 && rc == LSG_OK; k++) rc = B.richardson(0);
            if (rc) break;
            cudaEventRecord(e0, s);
            for (int k = 0; k < 5 && rc == LSG_OK; k++) rc = B.richardson(0);
            cudaEventRecord(e1, s);
            if (rc) break;
            if (cudaEventSynchronize(e1) != cudaSuccess) {
                rc = set_error(LSG_CUDA_ERROR, "batch autotune: %s", cudaGetErrorString(cudaGetLastError()));
                break;
            }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) {
                best = ms;
                ws->tvar = var;
                ws->tscale = sc;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (int i = 0; i < count; i++) hi[i].x = xsave[i];
    if (rc == LSG_OK) ws->tuned = 1;
    return rc;
}

template <typename T>
static int batch_solve(const lsg_operator *ops, int count, const lsg_params *prm, bool mixed, void *const *xs,
                       const void *const *bs, lsg_result *res, cudaStream_t us) {
    using TW = typename WideOf<T>::type;
    const double t0 = std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
    if (count < 1) return set_error(LSG_BAD_ARG, "batch count %d < 1", count);
    if (!ops || !xs || !bs) return set_error(LSG_BAD_ARG, "NULL batch array");
    int rc = check_params(prm, true);
    if (rc) return rc;
    if (prm->m > 8) return set_error(LSG_UNSUPPORTED, "batched AAR: history depth m = %d > 8", prm->m);
    bool generic = false;
    std::vector<Geom> geo(count);
    for (int i = 0; i < count; i++) {
        rc = check_operator(&ops[i]);
        if (rc) return set_error(rc, "instance %d: %s", i, last_error());
        if (!xs[i] || !bs[i]) return set_error(LSG_BAD_ARG, "instance %d: NULL vector", i);
        if (ops[i].radius != 6) generic = true;
        geo[i] = make_geom(ops[i].n);
    }
    BatchWs *ws = nullptr;
    std::unique_lock<std::mutex> lk;
    rc = batch_ws_get<T>(geo, prm->m, mixed, generic, &ws, &lk);
    if (rc) return rc;
    const int m = prm->m, p = prm->p;
    const size_t es = sizeof(T);
    // Instance records.
    BInst<T> *hi = (BInst<T> *)ws->h_inst;
    bool deflating = false;
    for (int i = 0; i < count; i++) {
        BInst<T> &I = hi[i];
        memset((void *)&I, 0, sizeof(I));
        I.g = geo[i];
        constexpr int VN = IsCplx<T>::value ? 0 : (int)(16 / sizeof(T));
        // x is the caller's vector (the rest are work arrays): 16-byte loads only when it is aligned
        I.vec = VN > 0 && geo[i].n % VN == 0 && (((uintptr_t)xs[i]) & 15u) == 0;
        I.w = make_weights<T>(&ops[i]);
        I.w64 = make_weights<TW>(&ops[i]);
        const typename ScalarOf<T>::type cf = jacobi_factor<T>(&ops[i]);
        I.cf = T(cf);
        I.c = T(prm->omega * cf);
        const size_t vb = al256((size_t)geo[i].n * es);
        char *v = ws->vec[i];
        I.xalt = (T *)(v);
        I.r0 = (T *)(v + vb);
        I.r1 = (T *)(v + 2 * vb);
        I.dx = (T *)(v + 3 * vb);
        I.df = (T *)(v + (3 + m) * vb);
        if (IsRecur<T>::value) I.rs = (T *)(v + (3 + 2 * m + (mixed ? 1 : 0)) * vb);
        if (mixed) {
            I.x = (T *)(v + (3 + 2 * m) * vb);
            I.b = nullptr;
            I.x64 = (TW *)xs[i];
            I.b64 = (const TW *)bs[i];
        } else {
            I.x = (T *)xs[i];
            I.b = (const T *)bs[i];
        }
        BCtl &C = ws->h_ctl[i];
        memset(&C, 0, sizeof(C));
        C.ctrl = ws->d_ctrl + 2 * i;
        C.octrl = mixed ? ws->d_ctrl + 2 * i + 1 : nullptr;
        C.part = ws->part[i];
        C.n = geo[i].n;
        if constexpr (IsCplx<T>::value) {
            C.hre = cf.x;
            C.him = cf.y;
        } else {
            C.hre = cf;
        }
        C.sig_re = ops[i].sigma;
        C.sig_im = IsCplx<T>::value ? ops[i].sigma_im : 0.0;
        if (mixed && (C.sig_re != 0.0 || C.sig_im != 0.0)) deflating = true;
        ws->h_ctrl[2 * i] = ctrl_init(prm->tol, mixed ? 12 : 0);
        ws->h_ctrl[2 * i + 1] = ctrl_init(prm->tol, 0);
        if (mixed) ws->h_ctrl[2 * i].done = 1;  // opens the first refinement pass
    }
    cudaStream_t s = ws->stream;
    LSG_BCUDA(cudaEventRecord(ws->join, us));
    LSG_BCUDA(cudaStreamWaitEvent(s, ws->join, 0));
    std::vector<int> act(count);
    for (int i = 0; i < count; i++) act[i] = i;
    ws->paired = 0;  // the tuner times the one-column march
    if (!generic && !ws->tuned && tune_mode() == 2) {
        rc = tune_batch<T>(ws, geo, act, prm, mixed);
        if (rc) return rc;
    }
    LSG_BCUDA(cudaMemcpyAsync(ws->d_ctrl, ws->h_ctrl, sizeof(DevCtrl) * 2 * count, cudaMemcpyHostToDevice, s));
    LSG_BCUDA(cudaMemsetAsync(ws->d_clk, 0, ws->clk_bytes, s));
    for (int i = 0; i < count; i++) {
        const size_t vb = al256((size_t)geo[i].n * es);
        LSG_BCUDA(cudaMemsetAsync(hi[i].dx, 0, 2 * (size_t)m * vb, s));  // dx, df contiguous
        if (mixed) LSG_BCUDA(cudaMemsetAsync(hi[i].x, 0, vb, s));
    }
    // FP32: the Richardson passes take the paired march when every grid has an
    // even nx (its pairs never straddle the wrap) and the vectors it touches
    // are 8-byte aligned (the work arrays are; x is the caller's)
    if constexpr (std::is_same<T, float>::value) {
        bool ok = !generic && batch_paired_enabled();
        for (int i = 0; i < count && ok; i++) ok = geo[i].nx % 2 == 0 && (((uintptr_t)hi[i].x) & 7u) == 0;
        ws->paired = ok ? 1 : 0;
    }
    const int var = generic ? 0 : ws->tvar;
    const double lscale = generic ? 1.0 : ws->tscale;
    const int slots = sm_count() * BatchKernels<T>::stencil_blocks_per_sm(generic, var);
    BatchRun<T> B{ws, prm, mixed, generic, prm->inner_tol > 0 ? prm->inner_tol : 3e-4,
                  prm->max_outer > 0 ? prm->max_outer : 50, BPlan(), 0};
    B.deflating = deflating;
    make_plan<T>(ws, geo, act, generic, var, slots, lscale, &B.plan);
    rc = upload_tables<T>(ws, B.plan);
    if (rc) return rc;
    const int W = AccWidth<T>::value;
    // ||b||, tol *= ||b|| (AAR.c:78-79); r = b - A x (AAR.c:80-82) or the first FP64 residual.
    if (mixed) {
        {
            cudaError_t e = BatchKernels<T>::norm2_rhs(B.tab(), B.args(ws->d_umap, -1), B.plan.ugrid, true, s);
            if (e != cudaSuccess) return set_error(LSG_CUDA_ERROR, "batched rhs norm: %s", cudaGetErrorString(e));
            e = batch_finalize_norm(B.args(nullptr, -1), ws->d_amap, B.nact(), BF_RHS_OUTER, prm->tol,
                                    AccWidth<TW>::value, s);
            if (e != cudaSuccess) return set_error(LSG_CUDA_ERROR, "batched rhs norm: %s", cudaGetErrorString(e));
            B.launches += 2;
            if (B.deflating) {  // mean(b64) of the instances with a shift
                e = BatchKernels<T>::mean_deflate(B.tab(), B.args(ws->d_umap, -1), B.plan.ugrid, B.args(nullptr, -1),
                                                  ws->d_amap, B.nact(), 0, s);
                if (e != cudaSuccess) return set_error(LSG_CUDA_ERROR, "batched rhs mean: %s", cudaGetErrorString(e));
                B.launches += 2;
            }
        }
        rc = B.refine(-1, 0);
        if (rc) return rc;
    } else {
        cudaError_t e = BatchKernels<T>::norm2_rhs(B.tab(), B.args(ws->d_umap, -1), B.plan.ugrid, false, s);
        if (e == cudaSuccess)
            e = batch_finalize_norm(B.args(nullptr, -1), ws->d_amap, B.nact(), BF_RHS, prm->tol, W, s);
        if (e == cudaSuccess)
            e = BatchKernels<T>::residual_init(B.tab(), B.args(ws->d_smap, -1), B.plan.sgrid, generic, B.plan.var, s);
        if (e != cudaSuccess) return set_error(LSG_CUDA_ERROR, "batched initial residual: %s", cudaGetErrorString(e));
        B.launches += 3;
    }
    int it0 = 0;  // host copy of the clock
    if (p == 1 && prm->max_iter >= 1) {
        // iteration 1 is a Richardson iteration (AAR.c:109 needs iter > 1)
        rc = B.richardson(0);
        if (rc) return rc;
        LSG_BCUDA(batch_tick(ws->d_clk, ws->d_ctl, count, 1, mixed, s));
        B.launches++;
        it0 = 1;
    }
    rc = B.capture();
    if (rc) return rc;
    const int per_check = prm->check_every > 0 ? prm->check_every : (B.plan.points >= (1LL << 21) ? 2 : 8);
    int batch = 0;
    bool stop = it0 >= prm->max_iter;
    long long planned_points = B.plan.points;
    while (!stop) {
        for (int c = 0; c < per_check && it0 < prm->max_iter; c++) {
            LSG_BCUDA(cudaGraphLaunch(ws->exec, s));
            B.launches += B.per_cycle();
            it0 += p;
        }
        const int slot = batch & 1;
        LSG_BCUDA(cudaMemcpyAsync(clk_slot(ws, slot), ws->d_clk, ws->clk_bytes, cudaMemcpyDeviceToHost, s));
        LSG_BCUDA(cudaEventRecord(ws->ev[slot], s));
        if (batch > 0) {
            const int prev = slot ^ 1;
            LSG_BCUDA(cudaEventSynchronize(ws->ev[prev]));
            const BClock *ck = clk_slot(ws, prev);
            if (ck->ndone >= count) stop = true;
            if (!stop) {
                // re-plan once the unfinished instances hold <= 60% of the planned points
                long long live = 0;
                const int *fl = clk_flags(ck);
                for (int i = 0; i < count; i++)
                    if (!fl[i]) live += geo[i].n;
                if (live > 0 && live * 10 <= planned_points * 6) {
                    LSG_BCUDA(cudaStreamSynchronize(s));
                    LSG_BCUDA(cudaMemcpy(clk_slot(ws, prev), ws->d_clk, ws->clk_bytes, cudaMemcpyDeviceToHost));
                    const int *f2 = clk_flags(clk_slot(ws, prev));
                    std::vector<int> a2;
                    for (int i = 0; i < count; i++)
                        if (!f2[i]) a2.push_back(i);
                    if (a2.empty()) {
                        stop = true;
                    } else {
                        make_plan<T>(ws, geo, a2, generic, var, slots, lscale, &B.plan);
                        rc = upload_tables<T>(ws, B.plan);
                        if (rc) return rc;
                        rc = B.capture();
                        if (rc) return rc;
                        planned_points = B.plan.points;
                    }
                }
            }
        }
        if (it0 >= prm->max_iter) stop = true;
        batch++;
    }
    LSG_BCUDA(cudaStreamSynchronize(s));
    if (mixed && it0 >= prm->max_iter) {
        // max_iter reached: fold the corrections of the unfinished instances and
        // take their true residual after the last iteration
        rc = B.refine(prm->max_iter - it0 - 1, 1);
        if (rc) return rc;
    } else if (it0 >= prm->max_iter) {
        // a lean batch stopped between extrapolations: add the cycle's steps to x
        const cudaError_t e = BatchKernels<T>::fold(B.tab(), B.args(ws->d_umap, prm->max_iter - it0 - 1, 1),
                                                    B.plan.ugrid, s);
        if (e != cudaSuccess) return set_error(LSG_CUDA_ERROR, "batched fold: %s", cudaGetErrorString(e));
        B.launches++;
    }
    LSG_BCUDA(cudaMemcpyAsync(ws->h_ctrl, ws->d_ctrl, sizeof(DevCtrl) * 2 * count, cudaMemcpyDeviceToHost, s));
    LSG_BCUDA(cudaStreamSynchronize(s));
    // Where the last iterate lives (reference form: x ping-pongs with xalt).
    if (!mixed && !std::is_same<typename RealOf<T>::type, float>::value) {
        for (int i = 0; i < count; i++) {
            const DevCtrl &c = ws->h_ctrl[2 * i];
            const int last = c.done ? c.iters : prm->max_iter;
            if (richardson_parity(last, p))
                LSG_BCUDA(cudaMemcpyAsync(xs[i], hi[i].xalt, es * (size_t)geo[i].n, cudaMemcpyDeviceToDevice, s));
        }
    }
    LSG_BCUDA(cudaEventRecord(ws->join, s));
    LSG_BCUDA(cudaStreamWaitEvent(us, ws->join, 0));
    LSG_BCUDA(cudaStreamSynchronize(s));
    const double secs =
        std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count() - t0;
    int worst = LSG_OK;
    for (int i = 0; i < count; i++) {
        lsg_result r;
        memset(&r, 0, sizeof(r));
        const DevCtrl &c = ws->h_ctrl[2 * i];
        const DevCtrl &o = mixed ? ws->h_ctrl[2 * i + 1] : c;
        r.rhs_norm = o.rhs_norm;
        r.relres = o.rhs_norm > 0 ? o.relres / o.rhs_norm : o.relres;
        const bool ok = o.done && !o.stalled && !(o.relres > o.tol_abs) && o.status != LSG_NAN_DETECTED;
        r.iters = o.done ? o.iters : prm->max_iter;
        if (o.status == LSG_NAN_DETECTED || c.status == LSG_NAN_DETECTED) r.status = LSG_NAN_DETECTED;
        else if (o.df_range || c.df_range) r.status = LSG_RANGE;
        else if (ok) r.status = LSG_OK;
        else r.status = (c.status == LSG_SVD_NO_CONVERGENCE) ? LSG_SVD_NO_CONVERGENCE : LSG_NOT_CONVERGED;
        if (mixed) {
            r.outer_iters = o.restarts;
            r.inner_iters = r.iters;
        }
        r.seconds = secs;
        r.launches = B.launches;
        r.svd_fallbacks = c.svd_fallbacks;
        if (res) res[i] = r;
        if (r.status != LSG_OK && worst == LSG_OK) worst = r.status;
    }
    set_last_status(worst);
    return worst;
}

int solve_batched(const lsg_operator *ops, int count, const lsg_params *prm, int dtype, void *const *xs,
                  const void *const *bs, lsg_result *res, cudaStream_t s) {
    if (dtype == LSG_F64) return batch_solve<double>(ops, count, prm, false, xs, bs, res, s);
    if (dtype == LSG_F32) return batch_solve<float>(ops, count, prm, false, xs, bs, res, s);
    if (dtype == LSG_C128) return batch_solve<cplx<double>>(ops, count, prm, false, xs, bs, res, s);
    if (dtype == LSG_C64) return batch_solve<cplx<float>>(ops, count, prm, false, xs, bs, res, s);
    return set_error(LSG_BAD_ARG, "unknown dtype %d", dtype);
}

int solve_mixed_batched(const lsg_operator *ops, int count, const lsg_params *prm, int dtype, void *const *xs,
                        const void *const *bs, lsg_result *res, cudaStream_t s) {
    if (dtype == LSG_F64) return batch_solve<float>(ops, count, prm, true, xs, bs, res, s);
    if (dtype == LSG_C128) return batch_solve<cplx<float>>(ops, count, prm, true, xs, bs, res, s);
    return set_error(LSG_BAD_ARG, "mixed batched AAR: dtype %d is not LSG_F64 or LSG_C128", dtype);
}

}  // namespace lsg

extern "C" {

int lsg_set_batch_march(int paired) { return lsg::g_batch_paired.exchange(paired ? 1 : 0); }

int lsg_aar_batched(const lsg_operator *ops, int count, const lsg_params *prm, int dtype, void *const *d_x,
                    const void *const *d_b, lsg_result *res, void *stream) {
    return lsg::solve_batched(ops, count, prm, dtype, d_x, d_b, res, (cudaStream_t)stream);
}

int lsg_aar_mixed_batched(const lsg_operator *ops, int count, const lsg_params *prm, int dtype,
                          void *const *d_x, const void *const *d_b, lsg_result *res, void *stream) {
    return lsg::solve_mixed_batched(ops, count, prm, dtype, d_x, d_b, res, (cudaStream_t)stream);
}

}  // extern "C"
