// noalloc.cu -- a CG solve that allocates nothing.
//
// pfg_linear_solver_crs_noalloc is the LinearSolver plug-in of
// pfg_linear_solver_crs for callers that cannot allocate device memory: hosts
// whose device memory is owned by another runtime or a fixed-budget pool, and
// code that must not call cudaMalloc/cudaFree while other work is queued.  The
// caller passes the CRS matrix, right-hand side and solution in device memory;
// every work vector, the reduction partials and the solver scalars live in
// one file-scope __device__ array of fixed size (kNaMaxDof DOF).  CUDA loads
// this file's module, and with it the array, on a device the first time the
// entry point runs there (lazy module loading, the default), and the device
// keeps it until the process exits.  Callers that must not allocate at all
// while they solve make one set-up call (n = 0) per device first, or run with
// CUDA_MODULE_LOADING=EAGER, which loads every module when the context is made.
#include <chrono>
#include <cmath>
#include <mutex>

#include "bsr.cuh"

namespace pfg {

constexpr int64_t kNaMaxDof = 262144;    // largest system the static scratch holds
constexpr int kNaMaxCtas = 1024;         // reduction partials per kernel
constexpr int kNaThreads = 256;
// r, z, p, q, D^-1 (5 vectors) + partials (3 per CTA) + scalars
constexpr int64_t kNaScratch = 5 * kNaMaxDof + 3 * kNaMaxCtas + 64;

static __device__ __align__(256) double g_noalloc_scratch[kNaScratch];

struct NaState {
    double rho, rr, bb, pq, alpha, beta;
    double iter, done;
    unsigned int ticket, pad;
};

// ---- kernels over the caller's 1-based CRS (the reference's own arrays)
// row sums of one warp: y_i = sum_k val(k) v(col(k)), k in row_ptr(i)-1 .. row_ptr(i+1)-2
__device__ __forceinline__ double na_row(const int64_t *rp, const int32_t *ci, const double *val, const double *v,
                                         int64_t i, int lane)
{
    double s = 0.0;
    for (int64_t k = rp[i] - 1 + lane; k < rp[i + 1] - 1; k += 32) s = fma(val[k], v[ci[k] - 1], s);
    return warp_sum(s);
}

// r = b - A x, D^-1 (point Jacobi or identity), z = D^-1 r; rr, bb, rho = r.z
__global__ void __launch_bounds__(kNaThreads)
    k_na_start(const int64_t *rp, const int32_t *ci, const double *val, const double *b, const double *x, int64_t n,
               int jacobi, double *r, double *z, double *dinv, double *p, double *partials, NaState *S)
{
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    double acc[3] = {0.0, 0.0, 0.0};
    for (int64_t i = w0; i < n; i += nw) {
        const double ax = na_row(rp, ci, val, x, i, lane);
        double d = 0.0;
        for (int64_t k = rp[i] - 1 + lane; k < rp[i + 1] - 1; k += 32)
            if (ci[k] - 1 == i) d = val[k];
        d = warp_sum(d);
        if (lane == 0) {
            const double ri = b[i] - ax;
            const double di = (jacobi && d != 0.0) ? 1.0 / d : 1.0;
            r[i] = ri;
            dinv[i] = di;
            z[i] = di * ri;
            p[i] = 0.0;
            acc[0] = fma(ri, ri, acc[0]);
            acc[1] = fma(b[i], b[i], acc[1]);
            acc[2] = fma(ri, di * ri, acc[2]);
        }
    }
    double tot[3];
    if (grid_sum<3>(acc, partials, &S->ticket, tot)) {
        S->rr = tot[0];
        S->bb = tot[1];
        S->rho = tot[2];
        S->beta = 0.0;
    }
}

// p = z + beta p
__global__ void k_na_dir(int64_t n, const double *z, double *p, const NaState *S)
{
    if (S->done != 0.0) return;
    const double beta = S->beta;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = fma(beta, p[i], z[i]);
}

// q = A p; alpha = rho / (p.q)
__global__ void __launch_bounds__(kNaThreads)
    k_na_spmv(const int64_t *rp, const int32_t *ci, const double *val, int64_t n, const double *p, double *q,
              double *partials, NaState *S)
{
    if (S->done != 0.0) return;
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    double acc[1] = {0.0};
    for (int64_t i = w0; i < n; i += nw) {
        const double qi = na_row(rp, ci, val, p, i, lane);
        if (lane == 0) {
            q[i] = qi;
            acc[0] = fma(p[i], qi, acc[0]);
        }
    }
    double tot[1];
    if (grid_sum<1>(acc, partials, &S->ticket, tot)) {
        S->pq = tot[0];
        if (!(tot[0] > 0.0) || !isfinite(tot[0])) {
            S->done = -1.0;  // breakdown: p.Ap <= 0
        } else {
            S->alpha = S->rho / tot[0];
        }
    }
}

// x += alpha p; r -= alpha q; z = D^-1 r; rho' = r.z; rr = r.r; stop test
__global__ void __launch_bounds__(kNaThreads)
    k_na_update(int64_t n, double *x, double *r, double *z, const double *p, const double *q, const double *dinv,
                double *partials, NaState *S, double tol, int itrmax)
{
    if (S->done != 0.0) return;
    const double alpha = S->alpha;
    double acc[2] = {0.0, 0.0};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] = fma(alpha, p[i], x[i]);
        const double ri = fma(-alpha, q[i], r[i]);
        r[i] = ri;
        const double zi = dinv[i] * ri;
        z[i] = zi;
        acc[0] = fma(ri, zi, acc[0]);
        acc[1] = fma(ri, ri, acc[1]);
    }
    double tot[2];
    if (grid_sum<2>(acc, partials, &S->ticket, tot)) {
        S->beta = tot[0] / S->rho;
        S->rho = tot[0];
        S->rr = tot[1];
        S->iter += 1.0;
        if (sqrt(tot[1]) <= tol * sqrt(S->bb)) S->done = 1.0;
        else if (S->iter >= itrmax) S->done = 2.0;
        if (!isfinite(tot[0]) || !isfinite(tot[1])) S->done = -2.0;
    }
}

// Device address of the scratch array on the current device.  Looked up on
// every call rather than cached: after a context reset the module is loaded
// again at another address, and once the module is loaded the lookup itself
// allocates nothing.  The first lookup on a device is what loads this file's
// module there (CUDA loads modules lazily by default), placing the array.
static double *scratch_address()
{
    void *p = nullptr;
    PFG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    return (double *)p;
}

}  // namespace pfg

using namespace pfg;

extern "C" int pfg_linear_solver_crs_noalloc(const int64_t *d_row_ptr, const int32_t *d_col_idx, const double *d_val,
                                             const double *d_rhs, double *d_x, int64_t n, const pfg_solve_opts *opts,
                                             pfg_info *info, void *stream)
{
    static std::mutex call_mu;  // one solve at a time: every call shares the scratch
    int status = PFG_OK;
    NaState h{};
    const int rc = guard([&] {
        PFG_CHECK(n >= 0, PFG_E_ARG, "n must not be negative");
        if (n == 0) {  // set-up only: load the module and place the array on this device
            std::lock_guard<std::mutex> lk(call_mu);
            (void)scratch_address();
            return;
        }
        PFG_CHECK(d_row_ptr && d_col_idx && d_val && d_rhs && d_x, PFG_E_ARG, "NULL argument");
        PFG_CHECK(n <= kNaMaxDof, PFG_E_ARG,
                  "pfg_linear_solver_crs_noalloc: n = " + std::to_string(n) + " exceeds the static scratch limit of " +
                      std::to_string(kNaMaxDof) + " DOF; use pfg_linear_solver_crs");
        pfg_solve_opts d;
        pfg_solve_opts_default(&d);
        d.algorithm = PFG_ALG_CG;
        d.precond = PFG_PC_JACOBI;
        d.stop_rule = PFG_STOP_TRUE_RELATIVE;
        if (!opts) opts = &d;
        PFG_CHECK(opts->algorithm == PFG_ALG_CG && opts->precision == PFG_PREC_FP64, PFG_E_UNSUPPORTED,
                  "pfg_linear_solver_crs_noalloc: FP64 CG only");
        PFG_CHECK(opts->precond == PFG_PC_NONE || opts->precond == PFG_PC_JACOBI, PFG_E_UNSUPPORTED,
                  "pfg_linear_solver_crs_noalloc: point Jacobi or no preconditioner");
        PFG_CHECK(opts->stop_rule == PFG_STOP_TRUE_RELATIVE, PFG_E_UNSUPPORTED,
                  "pfg_linear_solver_crs_noalloc: stop rule PFG_STOP_TRUE_RELATIVE only");
        const double tol = opts->relative_er > 0 ? opts->relative_er : 1e-10;
        const int itrmax = opts->itrmax > 0 ? opts->itrmax : 100000;
        cudaStream_t st = (cudaStream_t)stream;
        std::lock_guard<std::mutex> lk(call_mu);
        double *base = scratch_address();
        double *r = base, *z = base + kNaMaxDof, *p = base + 2 * kNaMaxDof, *q = base + 3 * kNaMaxDof;
        double *dinv = base + 4 * kNaMaxDof, *partials = base + 5 * kNaMaxDof;
        NaState *S = (NaState *)(partials + 3 * kNaMaxCtas);
        // the scratch keeps the previous call's contents: clear the scalars
        // and the reduction ticket, which must start at zero
        PFG_CUDA(cudaMemsetAsync(S, 0, sizeof(NaState), st));
        int sms = 1;
        int dev = 0;
        PFG_CUDA(cudaGetDevice(&dev));
        PFG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        const int gw = (int)std::min<int64_t>(std::min<int64_t>((n + 7) / 8, (int64_t)sms * 4), kNaMaxCtas);
        const int gv = (int)std::min<int64_t>(std::min<int64_t>((n + kNaThreads - 1) / kNaThreads, (int64_t)sms * 4),
                                              kNaMaxCtas);
        const auto t0 = std::chrono::steady_clock::now();
        auto read = [&]() {
            PFG_CUDA(cudaMemcpyAsync(&h, S, sizeof(NaState), cudaMemcpyDeviceToHost, st));
            PFG_CUDA(cudaStreamSynchronize(st));
        };
        int launches = 0;
        double iters = 0.0;
        // CG from the true residual; when the recursive residual meets the
        // tolerance, recompute b - A x and restart if it does not (at most 5 times)
        for (int restart = 0; restart < 6; ++restart) {
            k_na_start<<<gw, kNaThreads, 0, st>>>(d_row_ptr, d_col_idx, d_val, d_rhs, d_x, n,
                                                  opts->precond == PFG_PC_JACOBI, r, z, dinv, p, partials, S);
            PFG_CUDA(cudaGetLastError());
            ++launches;
            read();
            if (std::sqrt(h.rr) <= tol * std::sqrt(h.bb) || restart == 5 || iters >= itrmax) break;
            const double zero[2] = {iters, 0.0};  // keep the iteration count, clear done
            PFG_CUDA(cudaMemcpyAsync(&S->iter, zero, 2 * sizeof(double), cudaMemcpyHostToDevice, st));
            for (;;) {
                for (int it = 0; it < 16; ++it) {
                    k_na_dir<<<gv, kNaThreads, 0, st>>>(n, z, p, S);
                    k_na_spmv<<<gw, kNaThreads, 0, st>>>(d_row_ptr, d_col_idx, d_val, n, p, q, partials, S);
                    k_na_update<<<gv, kNaThreads, 0, st>>>(n, d_x, r, z, p, q, dinv, partials, S, tol, itrmax);
                    launches += 3;
                }
                PFG_CUDA(cudaGetLastError());
                read();
                if (h.done != 0.0) break;
            }
            iters = h.iter;
            if (h.done < 0.0) break;  // breakdown
        }
        const double ms =
            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        const bool conv = std::sqrt(h.rr) <= tol * std::sqrt(h.bb);
        status = h.done < 0.0 ? PFG_E_BREAKDOWN : (conv ? PFG_OK : PFG_W_NOT_CONVERGED);
        h.iter = iters;
        if (info) {
            info->status = status;
            info->iterations = (int32_t)h.iter;
            info->replacements = 0;
            info->kernel_launches = launches;
            info->rel_residual = h.bb > 0 ? std::sqrt(h.rr / h.bb) : std::sqrt(h.rr);
            info->iter_residual = info->rel_residual;
            info->solve_ms = ms;
            info->fallback = 0;
        }
    });
    if (rc != PFG_OK) return rc;
    if (status == PFG_E_BREAKDOWN) set_last_error("CG breakdown (p.Ap <= 0 or non-finite)");
    if (status == PFG_W_NOT_CONVERGED) set_last_error("not converged within itrmax");
    return status;
}
