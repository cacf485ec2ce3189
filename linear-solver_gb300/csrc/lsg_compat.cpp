// lsg_compat.cpp — the reference's own entry points (AAR, PGR, PL2R, CG) on
// host buffers, so MPI_REAL/main.c and system.c link against liblsg unchanged.
//
//   AAR   MPI_REAL/AAR.c:37   (AAR.h:18-22)     PGR   MPI_REAL/PGR.c:35  (PGR.h:18-22)
//   PL2R  MPI_REAL/PL2R.c:35  (PL2R.h:18-22)    CG    MPI_REAL/CG.c:33   (CG.h:18-21)
//
// Each call copies x and rhs to the GPU, runs the device solver and copies x
// back.  The host callbacks are identified, never called: the reference
// operator (system.c:80-213) and Jacobi preconditioner (system.c:222-227)
// are recognised by address (the process's Lap_Vec_mult / Precondition
// symbols, or registered addresses).  A user operator runs on the GPU when its
// callback was bound to the CSR form of its matrix (AAR only); anything else
// is refused.  Reports are
// printed in the reference's format (AAR.c:151-159, PGR.c:145-153,
// PL2R.c:144-152, CG.c:157-165).
#include <dlfcn.h>

#include <chrono>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/lsg_compat.h"
#include "lsg_host.h"

namespace {

std::mutex g_mu;
void *g_ops[8];
int g_nops = 0;
void *g_pcs[8];
int g_npcs = 0;
int g_verbose = 1;
int g_mode = 0;  // 0 FP64 (reference semantics), 1 mixed-precision AAR
thread_local lsg_result t_result;

// Device staging buffers reused across calls of the same size.
struct Staging {
    double *x = nullptr, *b = nullptr;
    long long n = 0;
} g_stage;
// Two copy streams: x and rhs go to the device concurrently.
cudaStream_t g_copy[2] = {nullptr, nullptr};

// Operators bound to a CSR copy of their matrix (lsg_register_operator_csr).
struct CsrBinding {
    void *fn = nullptr;
    int n = 0;
    long long nnz = 0;
    int *rp = nullptr, *col = nullptr;
    double *val = nullptr;
};
CsrBinding g_csr_ops[8];
int g_ncsr = 0;

const CsrBinding *csr_binding(void *fn) {
    std::lock_guard<std::mutex> g(g_mu);
    for (int i = 0; i < g_ncsr; i++)
        if (g_csr_ops[i].fn == fn) return &g_csr_ops[i];
    return nullptr;
}

bool listed(void *fn, void *const *list, int count) {
    for (int i = 0; i < count; i++)
        if (list[i] == fn) return true;
    return false;
}

bool is_reference_operator(void *fn) {
    if (!fn) return false;
    {
        std::lock_guard<std::mutex> g(g_mu);
        if (listed(fn, g_ops, g_nops)) return true;
    }
    void *sym = dlsym(RTLD_DEFAULT, "Lap_Vec_mult");
    return sym != nullptr && sym == fn;
}

// 0: none, 1: Jacobi, -1: unknown callback
int precondition_kind(void *fn) {
    if (!fn) return 0;
    {
        std::lock_guard<std::mutex> g(g_mu);
        if (listed(fn, g_pcs, g_npcs)) return 1;
    }
    void *sym = dlsym(RTLD_DEFAULT, "Precondition");
    return (sym != nullptr && sym == fn) ? 1 : -1;
}

int fail(const char *who, int status, const char *msg) {
    lsg::set_error(status, "%s", msg);
    fprintf(stderr, "%s (liblsg): %s\n", who, msg);
    memset(&t_result, 0, sizeof(t_result));
    t_result.status = status;
    return status;
}

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Shared body of the four entry points.  solver: 0 AAR, 1 PGR, 2 PL2R, 3 CG.
void run_compat(const char *who, int solver, POISSON *system, void *lap, void *pc, double a,
                double *x, double *rhs, double omega, double beta, int m, int p, int max_iter,
                double tol, int Np) {
    if (!system || !x || !rhs) { fail(who, LSG_BAD_ARG, "NULL system, x or rhs"); return; }
    const CsrBinding *csr = csr_binding(lap);
    if (!csr && !is_reference_operator(lap)) {
        fail(who, LSG_UNSUPPORTED,
             "Lap_Vec_mult is not the reference periodic FD operator; register it with "
             "lsg_register_operator_callback (no CPU fallback)");
        return;
    }
    const int pk = precondition_kind(pc);
    if (pk < 0) {
        fail(who, LSG_UNSUPPORTED,
             "Precondition is not the reference Jacobi preconditioner; register it with "
             "lsg_register_precondition_callback (no CPU fallback)");
        return;
    }
    for (int d = 0; d < 3; d++) {
        if (system->psize[d] != system->ssize[d]) {
            fail(who, LSG_UNSUPPORTED,
                 "distributed domain (psize != ssize): run one rank per GPU with the whole grid");
            return;
        }
    }
    const long long n = (long long)system->psize[0] * system->psize[1] * system->psize[2];
    if (n != Np || Np <= 0) { fail(who, LSG_BAD_ARG, "Np does not match psize"); return; }
    if (csr && (solver != 0 || csr->n != n)) {
        fail(who, csr->n != n ? LSG_BAD_ARG : LSG_UNSUPPORTED,
             csr->n != n ? "registered CSR matrix size differs from Np"
                         : "a registered CSR operator serves AAR only");
        return;
    }
    if (!csr && (system->FDn < 1 || system->FDn > LSG_MAX_RADIUS || !system->coeff_lap)) {
        fail(who, LSG_UNSUPPORTED, "FDn outside 1..8 or coeff_lap missing");
        return;
    }
    lsg_operator op;
    memset(&op, 0, sizeof(op));
    for (int d = 0; d < 3; d++) op.n[d] = system->psize[d];
    op.radius = csr ? 1 : system->FDn;
    for (int k = 0; k <= op.radius && !csr; k++) op.coeff[k] = system->coeff_lap[k];
    op.a = a;
    op.sigma = 0.0;
    op.precond = pk;
    lsg_params prm;
    lsg_params_default(&prm);
    prm.omega = omega;
    prm.beta = beta;
    prm.m = m;
    prm.p = p;
    prm.max_iter = max_iter;
    prm.tol = tol;

    std::lock_guard<std::mutex> g(g_mu);
    if (g_stage.n != n) {
        if (g_stage.x) cudaFree(g_stage.x);
        if (g_stage.b) cudaFree(g_stage.b);
        g_stage = Staging();
        if (cudaMalloc(&g_stage.x, sizeof(double) * n) != cudaSuccess ||
            cudaMalloc(&g_stage.b, sizeof(double) * n) != cudaSuccess) {
            cudaGetLastError();
            if (g_stage.x) cudaFree(g_stage.x);
            g_stage = Staging();
            fail(who, LSG_NO_MEMORY, "device allocation for x/rhs failed");
            return;
        }
        g_stage.n = n;
    }
    for (auto &c : g_copy)
        if (!c && cudaStreamCreateWithFlags(&c, cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            c = nullptr;
        }
    if (cudaMemcpyAsync(g_stage.x, x, sizeof(double) * n, cudaMemcpyHostToDevice, g_copy[0]) != cudaSuccess ||
        cudaMemcpyAsync(g_stage.b, rhs, sizeof(double) * n, cudaMemcpyHostToDevice, g_copy[1]) != cudaSuccess ||
        cudaStreamSynchronize(g_copy[0]) != cudaSuccess || cudaStreamSynchronize(g_copy[1]) != cudaSuccess) {
        fail(who, LSG_CUDA_ERROR, "host to device copy failed");
        return;
    }
    lsg_result res;
    memset(&res, 0, sizeof(res));
    const double t0 = now_s();
    int st;
    if (csr) {
        const lsg_csr A{csr->n, csr->nnz, csr->rp, csr->col, csr->val, pk, 0};
        st = lsg::solve_csr(&A, &prm, g_stage.x, g_stage.b, &res, nullptr);
    } else {
        st = (solver == 0 && g_mode == 1) ? lsg::solve_mixed(&op, &prm, g_stage.x, g_stage.b, &res, nullptr)
                                          : lsg::solve(solver, &op, &prm, LSG_F64, g_stage.x, g_stage.b, &res,
                                                       nullptr);
    }
    const double t1 = now_s();
    if (st == LSG_BAD_ARG || st == LSG_CUDA_ERROR || st == LSG_NO_MEMORY || st == LSG_UNSUPPORTED) {
        fail(who, st, lsg::last_error());
        return;
    }
    if (cudaMemcpy(x, g_stage.x, sizeof(double) * n, cudaMemcpyDeviceToHost) != cudaSuccess) {
        fail(who, LSG_CUDA_ERROR, "device to host copy failed");
        return;
    }
    t_result = res;
    lsg::set_last_status(res.status);
    if (!g_verbose) return;
    // The reference's report: its loop variable is iters+1 for the Richardson
    // family (AAR.c:152) and equal to iters for CG (CG.c:158).
    const bool converged = res.status == LSG_OK;
    const int loopvar = solver == 3 ? res.iters : res.iters + 1;
    if (loopvar < max_iter && converged)
        printf("%s converged!:  Iterations = %d, Relative Residual = %g, Time = %.4f sec\n", who,
               res.iters, res.relres, t1 - t0);
    if (loopvar >= max_iter) {
        printf("WARNING: %s exceeded maximum iterations.\n", who);
        printf("%s:  Iterations = %d, Relative Residual = %g, Time = %.4f sec \n", who, res.iters,
               res.relres, t1 - t0);
    }
    if (res.status == LSG_NAN_DETECTED) fprintf(stderr, "%s (liblsg): residual became NaN/Inf\n", who);
}

}  // namespace

extern "C" {

void AAR(POISSON *system, lsg_lap_fn Lap_Vec_mult, lsg_precond_fn Precondition, double a,
         double *x, double *rhs, double omega, double beta, int m, int p, int max_iter,
         double tol, int Np, LSG_MPI_COMM comm) {
    (void)comm;
    run_compat("AAR", 0, system, (void *)Lap_Vec_mult, (void *)Precondition, a, x, rhs, omega,
               beta, m, p, max_iter, tol, Np);
}

void PGR(POISSON *system, lsg_lap_fn Lap_Vec_mult, lsg_precond_fn Precondition, double a,
         double *x, double *rhs, double omega, int m, int p, int max_iter, double tol, int Np,
         LSG_MPI_COMM comm) {
    (void)comm;
    run_compat("PGR", 1, system, (void *)Lap_Vec_mult, (void *)Precondition, a, x, rhs, omega,
               0.0, m, p, max_iter, tol, Np);
}

void PL2R(POISSON *system, lsg_lap_fn Lap_Vec_mult, lsg_precond_fn Precondition, double a,
          double *x, double *rhs, double omega, int m, int p, int max_iter, double tol, int Np,
          LSG_MPI_COMM comm) {
    (void)comm;
    run_compat("PL2R", 2, system, (void *)Lap_Vec_mult, (void *)Precondition, a, x, rhs, omega,
               0.0, m, p, max_iter, tol, Np);
}

void CG(POISSON *system, lsg_lap_fn Lap_Vec_mult, lsg_precond_fn Precondition, double a,
        double *x, double *b, int max_iter, double tol, int Np, LSG_MPI_COMM comm) {
    (void)comm;
    run_compat("CG", 3, system, (void *)Lap_Vec_mult, (void *)Precondition, a, x, b, 0.0, 0.0,
               1, 1, max_iter, tol, Np);
}

int lsg_register_operator_callback(void *fn) {
    if (!fn) return lsg::set_error(LSG_BAD_ARG, "NULL callback");
    std::lock_guard<std::mutex> g(g_mu);
    if (listed(fn, g_ops, g_nops)) return LSG_OK;
    if (g_nops >= 8) return lsg::set_error(LSG_BAD_ARG, "too many registered operators");
    g_ops[g_nops++] = fn;
    return LSG_OK;
}

int lsg_register_operator_csr(void *fn, int n, long long nnz, const int *row_ptr, const int *col,
                              const double *val) {
    if (!fn || !row_ptr || !col || !val) return lsg::set_error(LSG_BAD_ARG, "NULL callback or CSR array");
    if (n < 1 || nnz < 1 || nnz > 2147483647LL) return lsg::set_error(LSG_BAD_ARG, "bad CSR sizes");
    if (row_ptr[0] != 0 || (long long)row_ptr[n] != nnz)
        return lsg::set_error(LSG_BAD_ARG, "CSR row offsets must run from 0 to nnz");
    for (int i = 0; i < n; i++)
        if (row_ptr[i + 1] < row_ptr[i]) return lsg::set_error(LSG_BAD_ARG, "CSR row offsets decrease");
    for (long long k = 0; k < nnz; k++)
        if (col[k] < 0 || col[k] >= n) return lsg::set_error(LSG_BAD_ARG, "CSR column index outside 0..n-1");
    std::lock_guard<std::mutex> g(g_mu);
    CsrBinding *slot = nullptr;
    for (int i = 0; i < g_ncsr; i++)
        if (g_csr_ops[i].fn == fn) slot = &g_csr_ops[i];
    if (!slot) {
        if (g_ncsr >= 8) return lsg::set_error(LSG_BAD_ARG, "too many registered CSR operators");
        slot = &g_csr_ops[g_ncsr++];
    }
    if (slot->rp) cudaFree(slot->rp);
    if (slot->col) cudaFree(slot->col);
    if (slot->val) cudaFree(slot->val);
    *slot = CsrBinding();
    if (cudaMalloc(&slot->rp, sizeof(int) * (size_t)(n + 1)) != cudaSuccess ||
        cudaMalloc(&slot->col, sizeof(int) * (size_t)nnz) != cudaSuccess ||
        cudaMalloc(&slot->val, sizeof(double) * (size_t)nnz) != cudaSuccess) {
        cudaGetLastError();
        return lsg::set_error(LSG_NO_MEMORY, "device copy of the CSR matrix");
    }
    if (cudaMemcpy(slot->rp, row_ptr, sizeof(int) * (size_t)(n + 1), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(slot->col, col, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(slot->val, val, sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice) != cudaSuccess)
        return lsg::set_error(LSG_CUDA_ERROR, "copy of the CSR matrix");
    slot->fn = fn;
    slot->n = n;
    slot->nnz = nnz;
    return LSG_OK;
}

int lsg_register_precondition_callback(void *fn) {
    if (!fn) return lsg::set_error(LSG_BAD_ARG, "NULL callback");
    std::lock_guard<std::mutex> g(g_mu);
    if (listed(fn, g_pcs, g_npcs)) return LSG_OK;
    if (g_npcs >= 8) return lsg::set_error(LSG_BAD_ARG, "too many registered preconditioners");
    g_pcs[g_npcs++] = fn;
    return LSG_OK;
}

void lsg_set_verbose(int on) { g_verbose = on; }

void lsg_set_compat_mode(int mode) { g_mode = mode == 1 ? 1 : 0; }

void lsg_last_result(lsg_result *res) {
    if (res) *res = t_result;
}

}  // extern "C"
