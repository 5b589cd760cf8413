// batch.cu -- persistent batched CG over many independent systems (batch.cuh).
//
// One launch solves every bound system.  Each CTA (or each cluster of CTAs,
// for the largest systems) takes the next job from an atomic queue and runs a
// complete preconditioned CG on it, with team-local reductions and no grid-wide
// synchronisation; when the queue is empty the CTA retires.  Jobs are ordered
// by estimated cost (the iteration count of the previous solve of the same
// system, when there was one), so the longest systems start first.
//
// Team step of one CG iteration (each warp of the team owns whole 32-row
// slices of the system's sliced-ELL matrix; the thread that computes q for a
// row also updates that row's x, r, z and p, so only the dot products and the
// complete direction vector need team-wide synchronisation):
//   q = K p, <p,q>        -> team reduction 1 (alpha)
//   x, r, z, <r,z>, <r,r>  -> team reduction 2 (beta, stop test)
//   p = z + beta p        -> team barrier (p complete before the next gathers)
// Vectors written during the launch are gathered with ld.global.cg (L2, not the
// SM's L1, which is not coherent across the cluster's SMs); the matrix, the
// right-hand side and the preconditioner are read-only in the launch.
#include <cooperative_groups.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <mutex>
#include <numeric>
#include <vector>

#include "batch.cuh"

namespace cg = cooperative_groups;

namespace pfg {
namespace {

constexpr int kMaxCluster = 8;
constexpr int kAbortEvery = 64;   // iterations between two reads of the abort flag
// Mixed precision hands a system over to FP64 CG (from its current x) after
// kMaxFailures FP32 passes in a row that broke down, overflowed or diverged
// (|r| grew kDiverge-fold over its smallest value in the pass), or kMaxStall
// replacements in a row that did not cut the FP64 residual by 10 %: the FP32
// copy of a system conditioned beyond FP32 is not positive definite.
constexpr int kMaxFailures = 2;
constexpr int kMaxStall = 3;
constexpr float kDiverge = 1.0e3f;

struct TeamShared {
    double slot[2][kMaxCluster][4];   // CTA totals of team reductions, one row per rank (every CTA holds all)
    double wpart[2][32][4];           // per-warp partials (FP64), double-buffered
    float wpart32[2][32][4];          // per-warp compensated partials (s, c pairs), double-buffered
    int job;
};

struct Team {
    int rank;   // CTA rank in the team
    int size;   // CTAs in the team (1: a single CTA, no cluster barrier)
    int nred;   // reductions done on this job (alternates the double buffers)
};

__device__ __forceinline__ void team_sync(const Team &tm)
{
    if (tm.size > 1)
        cg::this_cluster().sync();
    else
        __syncthreads();
}

// Team-wide sums of NV FP64 values with one CTA barrier (plus one cluster
// barrier in a cluster team).  Every warp forms the CTA total from the warp
// partials with the same butterfly; in a cluster, lane r of warp 0 pushes the
// CTA total into row `rank` of CTA r's slot table (distributed shared memory),
// and after the cluster barrier every warp adds its own CTA's copy of the table
// in rank order -- all threads of the team get the same bits and no thread
// reads remote shared memory.  The buffers alternate between consecutive
// reductions: a buffer is rewritten two reductions later, after every thread
// has passed the barrier of the reduction in between, i.e. after every thread
// has read it.
template <int NV>
__device__ __forceinline__ void team_sum(double (&v)[NV], Team &tm, TeamShared &sh)
{
    static_assert(NV <= 4, "at most 4 values per reduction");
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int buf = tm.nred++ & 1;
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = warp_sum(v[k]);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) sh.wpart[buf][wid][k] = v[k];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = warp_sum(lane < nw ? sh.wpart[buf][lane][k] : 0.0);
    if (tm.size > 1) {
        cg::cluster_group cl = cg::this_cluster();
        if (wid == 0 && lane < tm.size) {
            double *dst = cl.map_shared_rank(&sh.slot[buf][tm.rank][0], lane);
#pragma unroll
            for (int k = 0; k < NV; ++k) dst[k] = v[k];
        }
        cl.sync();
#pragma unroll
        for (int k = 0; k < NV; ++k) v[k] = warp_sum(lane < tm.size ? sh.slot[buf][lane][k] : 0.0);
    }
}

__device__ __forceinline__ void comp_warp_merge(Comp32 &t)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float s2 = __shfl_xor_sync(0xffffffffu, t.s, o);
        const float c2 = __shfl_xor_sync(0xffffffffu, t.c, o);
        comp_merge(t, s2, c2);
    }
}

// Team-wide compensated FP32 sums (Dot2 accumulators), rounded to float at the
// end; same structure as team_sum.
template <int NV>
__device__ __forceinline__ void team_sum_comp(Comp32 (&v)[NV], float (&tot)[NV], Team &tm, TeamShared &sh)
{
    static_assert(NV <= 2, "at most 2 compensated values per reduction");
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int buf = tm.nred++ & 1;
#pragma unroll
    for (int k = 0; k < NV; ++k) comp_warp_merge(v[k]);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            sh.wpart32[buf][wid][2 * k] = v[k].s;
            sh.wpart32[buf][wid][2 * k + 1] = v[k].c;
        }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        v[k].s = lane < nw ? sh.wpart32[buf][lane][2 * k] : 0.f;
        v[k].c = lane < nw ? sh.wpart32[buf][lane][2 * k + 1] : 0.f;
        comp_warp_merge(v[k]);
    }
    if (tm.size > 1) {
        cg::cluster_group cl = cg::this_cluster();
        if (wid == 0 && lane < tm.size) {
            double *dst = cl.map_shared_rank(&sh.slot[buf][tm.rank][0], lane);
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                dst[2 * k] = (double)v[k].s;
                dst[2 * k + 1] = (double)v[k].c;
            }
        }
        cl.sync();
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            v[k].s = lane < tm.size ? (float)sh.slot[buf][lane][2 * k] : 0.f;
            v[k].c = lane < tm.size ? (float)sh.slot[buf][lane][2 * k + 1] : 0.f;
            comp_warp_merge(v[k]);
        }
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) tot[k] = __fadd_rn(v[k].s, v[k].c);
}

// Abort flag of the batch, read by rank 0 and agreed on by the team.
__device__ __forceinline__ bool team_abort(const BatchParams &P, Team &tm, TeamShared &sh)
{
    double f[1] = {(P.abort && tm.rank == 0 && threadIdx.x == 0) ? (double)(*P.abort != 0) : 0.0};
    team_sum<1>(f, tm, sh);
    return f[0] != 0.0;
}

template <typename T>
__device__ __forceinline__ void precond3(int pc, const T *__restrict__ dinv, int64_t row, const T (&r)[3],
                                         T (&z)[3])
{
    if (pc == PFG_PC_NONE) {
#pragma unroll
        for (int i = 0; i < 3; ++i) z[i] = r[i];
        return;
    }
    const T *D = dinv + row * 9;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        T s = T(0);
#pragma unroll
        for (int j = 0; j < 3; ++j) s = fma(__ldg(D + i * 3 + j), r[j], s);
        z[i] = s;
    }
}

// Gather of block column c of a vector written during the launch (L2 path).
template <typename T>
struct GatherCG {
    const T *v;
    __device__ __forceinline__ void operator()(int c, T (&xv)[3]) const
    {
        const T *q = v + 3 * (int64_t)c;
        xv[0] = __ldcg(q);
        xv[1] = __ldcg(q + 1);
        xv[2] = __ldcg(q + 2);
    }
};

struct Span {
    int64_t w0, nw;   // first warp of this thread's warp in the team, warps in the team
};

__device__ __forceinline__ Span team_span(const Team &tm, int warps_per_cta)
{
    return Span{(int64_t)tm.rank * warps_per_cta + (threadIdx.x >> 5), (int64_t)tm.size * warps_per_cta};
}

// Sum of squares of r = b - K x (FP64) over the team, r written out.
__device__ double residual64(const BatchMesh &D, const Span &sp, Team &tm, TeamShared &sh)
{
    // Local copies of the descriptor's pointers: stores through them cannot
    // alias the descriptor, so it is not re-read after every store.
    const int lane = threadIdx.x & 31;
    const SellView<double> A = D.A64;
    const double *__restrict__ b = D.b;
    const double *__restrict__ x = D.x;
    double *__restrict__ r = D.r64;
    double acc[1] = {0.0};
    for (int64_t s = sp.w0; s < A.ns; s += sp.nw) {
        double y[3];
        sell_row_product<3>(A, s, lane, GatherCG<double>{x}, y);
        const int64_t row = s * 32 + lane;
        if (row < A.nb) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const int64_t i = 3 * row + k;
                const double rv = __ldg(b + i) - y[k];
                r[i] = rv;
                acc[0] = fma(rv, rv, acc[0]);
            }
        }
    }
    team_sum<1>(acc, tm, sh);
    return acc[0];
}

// Gather of block column c of the candidate solution x + x32.
struct GatherSum {
    const double *x;
    const float *x32;
    __device__ __forceinline__ void operator()(int c, double (&xv)[3]) const
    {
        const int64_t j = 3 * (int64_t)c;
#pragma unroll
        for (int k = 0; k < 3; ++k) xv[k] = __ldcg(x + j + k) + (double)__ldcg(x32 + j + k);
    }
};

// Sum of squares of b - K (x + x32) over the team; the candidate residual is
// written to q64 (unused by the mixed iterations), r64 keeps the residual of x.
__device__ double candidate_residual(const BatchMesh &D, const Span &sp, Team &tm, TeamShared &sh)
{
    const int lane = threadIdx.x & 31;
    const SellView<double> A = D.A64;
    const double *__restrict__ b = D.b;
    double *__restrict__ q = D.q64;
    const GatherSum src{D.x, D.x32};
    double acc[1] = {0.0};
    for (int64_t s = sp.w0; s < A.ns; s += sp.nw) {
        double y[3];
        sell_row_product<3>(A, s, lane, src, y);
        const int64_t row = s * 32 + lane;
        if (row < A.nb) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const int64_t i = 3 * row + k;
                const double rv = __ldg(b + i) - y[k];
                q[i] = rv;
                acc[0] = fma(rv, rv, acc[0]);
            }
        }
    }
    team_sum<1>(acc, tm, sh);
    return acc[0];
}

__device__ void restore_fixed_rows(const BatchMesh &D, const Span &sp, int64_t nb)
{
    const uint8_t *__restrict__ fixed = D.fixed;
    const double *__restrict__ fixval = D.fixval;
    double *__restrict__ x = D.x;
    if (!fixed) return;
    const int lane = threadIdx.x & 31;
    for (int64_t s = sp.w0; s * 32 < nb; s += sp.nw) {
        const int64_t row = s * 32 + lane;
        if (row < nb)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const int64_t i = 3 * row + k;
                if (fixed[i]) x[i] = fixval[i];
            }
    }
}

// ------------------------------------------------------------- FP64 CG
// Preconditioned CG on K x = b from the current x, counting on from `it`:
//   q = K p, <p,q>                      -> team reduction (alpha)
//   x += a p, r -= a q, z = M^-1 r, <r,z>, <r,r>   -> team reduction (beta, stop)
//   p = z + b p                         -> team barrier (p complete for the gathers)
// (The Chronopoulos-Gear form, one reduction per iteration, measured 8 % slower
// here: its extra live vectors cost registers the SpMV needs.)  A recursive
// residual at the tolerance is confirmed on the true residual, restarting from
// it otherwise (at most P.max_restarts).  Returns the status; `rel` = true
// |b - Kx| / |b| at exit.
template <int NT>
__device__ int cg64(const BatchParams &P, const BatchMesh &D, Team &tm, TeamShared &sh, int &it, int &restarts,
                    double &rel)
{
    const SellView<double> A = D.A64;
    const int64_t nb = A.nb;
    const int lane = threadIdx.x & 31;
    const Span sp = team_span(tm, NT / 32);
    const int pc = P.precond;
    const bool lead = tm.rank == 0 && threadIdx.x == 0;

    // r = b - K x0, z = M^-1 r, p = z
    double a3[3] = {0.0, 0.0, 0.0};
    {
        const double *__restrict__ b = D.b;
        const double *__restrict__ x = D.x;
        double *__restrict__ r = D.r64;
        double *__restrict__ z = D.z64;
        double *__restrict__ p = D.p64;
        const double *__restrict__ dinv = D.dinv64;
        for (int64_t s = sp.w0; s < A.ns; s += sp.nw) {
            double y[3];
            sell_row_product<3>(A, s, lane, GatherCG<double>{x}, y);
            const int64_t row = s * 32 + lane;
            if (row < nb) {
                double rv[3], zv[3];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const double bi = __ldg(b + 3 * row + k);
                    rv[k] = bi - y[k];
                    a3[2] = fma(bi, bi, a3[2]);
                }
                precond3<double>(pc, dinv, row, rv, zv);
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const int64_t i = 3 * row + k;
                    r[i] = rv[k];
                    z[i] = zv[k];
                    p[i] = zv[k];
                    a3[0] = fma(rv[k], zv[k], a3[0]);
                    a3[1] = fma(rv[k], rv[k], a3[1]);
                }
            }
        }
    }
    team_sum<3>(a3, tm, sh);  // also completes p for the first gathers
    double rho = a3[0];
    const double bb = a3[2];
    const double tol_b = P.tol * sqrt(bb);
    int status = PFG_OK;
    rel = bb > 0.0 ? sqrt(a3[1] / bb) : 0.0;
    if (sqrt(a3[1]) <= tol_b) return PFG_OK;
    for (;;) {
        if (it >= P.itrmax) {
            status = PFG_W_NOT_CONVERGED;
            break;
        }
        // q = K p, <p, q>; the abort flag rides along every kAbortEvery iterations
        double a2[2] = {0.0, 0.0};
        if (P.abort && lead && it % kAbortEvery == 0) a2[1] = (double)(*P.abort != 0);
        {
            const double *__restrict__ p = D.p64;
            double *__restrict__ q = D.q64;
            for (int64_t s = sp.w0; s < A.ns; s += sp.nw) {
                double y[3];
                sell_row_product<3>(A, s, lane, GatherCG<double>{p}, y);
                const int64_t row = s * 32 + lane;
                if (row < nb)
#pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        const int64_t i = 3 * row + k;
                        q[i] = y[k];
                        a2[0] = fma(p[i], y[k], a2[0]);
                    }
            }
        }
        team_sum<2>(a2, tm, sh);
        if (a2[1] != 0.0) {
            status = PFG_E_ABORTED;
            break;
        }
        if (!(a2[0] > 0.0) || !isfinite(a2[0])) {
            status = PFG_E_BREAKDOWN;
            break;
        }
        const double alpha = rho / a2[0];
        // x += alpha p, r -= alpha q, z = M^-1 r, <r, z>, <r, r>
        double a4[2] = {0.0, 0.0};
        {
            double *__restrict__ x = D.x;
            double *__restrict__ r = D.r64;
            double *__restrict__ z = D.z64;
            const double *__restrict__ p = D.p64;
            const double *__restrict__ q = D.q64;
            const double *__restrict__ dinv = D.dinv64;
            for (int64_t s = sp.w0; s * 32 < nb; s += sp.nw) {
                const int64_t row = s * 32 + lane;
                if (row >= nb) continue;
                double rv[3], zv[3];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const int64_t i = 3 * row + k;
                    x[i] = fma(alpha, p[i], x[i]);
                    rv[k] = fma(-alpha, q[i], r[i]);
                    r[i] = rv[k];
                }
                precond3<double>(pc, dinv, row, rv, zv);
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    z[3 * row + k] = zv[k];
                    a4[0] = fma(rv[k], zv[k], a4[0]);
                    a4[1] = fma(rv[k], rv[k], a4[1]);
                }
            }
        }
        team_sum<2>(a4, tm, sh);  // x complete for a true residual
        ++it;
        if (!isfinite(a4[0]) || !isfinite(a4[1])) {
            status = PFG_E_NONFINITE;
            break;
        }
        double beta;
        if (sqrt(a4[1]) <= tol_b) {
            // recursive residual converged: confirm on the true residual
            const double rt = residual64(D, sp, tm, sh);
            rel = bb > 0.0 ? sqrt(rt / bb) : 0.0;
            if (sqrt(rt) <= tol_b) return PFG_OK;
            if (restarts >= P.max_restarts) {
                status = PFG_W_NOT_CONVERGED;
                break;
            }
            ++restarts;
            // restart from the true residual (r64 holds it): z = M^-1 r, p = z
            double ar[1] = {0.0};
            {
                const double *__restrict__ r = D.r64;
                double *__restrict__ z = D.z64;
                const double *__restrict__ dinv = D.dinv64;
                for (int64_t s = sp.w0; s * 32 < nb; s += sp.nw) {
                    const int64_t row = s * 32 + lane;
                    if (row >= nb) continue;
                    double rv[3], zv[3];
#pragma unroll
                    for (int k = 0; k < 3; ++k) rv[k] = r[3 * row + k];
                    precond3<double>(pc, dinv, row, rv, zv);
#pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        z[3 * row + k] = zv[k];
                        ar[0] = fma(rv[k], zv[k], ar[0]);
                    }
                }
            }
            team_sum<1>(ar, tm, sh);
            rho = ar[0];
            beta = 0.0;
        } else {
            beta = a4[0] / rho;
            rho = a4[0];
        }
        // p = z + beta p (p = z after a restart)
        {
            double *__restrict__ p = D.p64;
            const double *__restrict__ z = D.z64;
            for (int64_t s = sp.w0; s * 32 < nb; s += sp.nw) {
                const int64_t row = s * 32 + lane;
                if (row >= nb) continue;
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const int64_t i = 3 * row + k;
                    p[i] = beta == 0.0 ? z[i] : fma(beta, p[i], z[i]);
                }
            }
        }
        team_sync(tm);
    }
    const double rt = residual64(D, sp, tm, sh);
    rel = bb > 0.0 ? sqrt(rt / bb) : 0.0;
    return status;
}

__device__ void finish_job(const BatchParams &P, int m, const BatchMesh &D, Team &tm, int status, int it,
                           int reps, int fallback, double rel)
{
    restore_fixed_rows(D, team_span(tm, blockDim.x / 32), D.A64.nb);
    if (tm.rank == 0 && threadIdx.x == 0) {
        BatchOut o;
        o.status = status;
        o.iterations = it;
        o.replacements = reps;
        o.team_size = tm.size;
        o.fallback = fallback;
        o.rel_residual = rel;
        P.out[m] = o;
    }
}

template <int NT>
__device__ void solve_fp64(const BatchParams &P, int m, Team &tm, TeamShared &sh, int fallback)
{
    const BatchMesh &D = P.mesh[m];
    int it = 0, restarts = 0;
    double rel = 0.0;
    const int status = cg64<NT>(P, D, tm, sh, it, restarts, rel);
    finish_job(P, m, D, tm, status, it, restarts, fallback, rel);
}

// ------------------------------------------- FP32 CG with FP64 replacement
template <int NT>
__device__ void solve_mixed(const BatchParams &P, int m, Team &tm, TeamShared &sh)
{
    const BatchMesh &D = P.mesh[m];
    const SellView<float> A = D.A32;
    const int64_t nb = A.nb;
    const int lane = threadIdx.x & 31;
    const Span sp = team_span(tm, NT / 32);
    const int pc = P.precond;

    // FP64 residual of x0 and |b|
    double a2[2] = {0.0, 0.0};
    for (int64_t s = sp.w0; s < D.A64.ns; s += sp.nw) {
        double y[3];
        sell_row_product<3>(D.A64, s, lane, GatherCG<double>{D.x}, y);
        const int64_t row = s * 32 + lane;
        if (row < nb)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const int64_t i = 3 * row + k;
                const double bi = __ldg(D.b + i);
                const double rv = bi - y[k];
                D.r64[i] = rv;
                D.x32[i] = 0.f;
                a2[0] = fma(rv, rv, a2[0]);
                a2[1] = fma(bi, bi, a2[1]);
            }
    }
    team_sum<2>(a2, tm, sh);
    const double bb = a2[1];
    const double tol_b = P.tol * sqrt(bb);
    double rel = bb > 0.0 ? sqrt(a2[0] / bb) : 0.0;
    int it = 0, reps = 0, status = PFG_OK, failures = 0, stall = 0, fallback = 0;
    double best_rt = a2[0], cur_rt = a2[0];
    bool converged = sqrt(a2[0]) <= tol_b;
    bool restart = true;   // the first pass starts from p = z
    float rho = 0.f, rmax = 0.f, rmin = 0.f;
    while (!converged) {
        // (re)start from the FP64 residual: r32 = r64, z = M^-1 r, beta keeps p unless a restart
        {
            Comp32 c2[2] = {Comp32{0.f, 0.f}, Comp32{0.f, 0.f}};
            for (int64_t s = sp.w0; s * 32 < nb; s += sp.nw) {
                const int64_t row = s * 32 + lane;
                if (row >= nb) continue;
                float rv[3], zv[3];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    rv[k] = (float)D.r64[3 * row + k];
                    D.r32[3 * row + k] = rv[k];
                }
                precond3<float>(pc, D.dinv32, row, rv, zv);
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    D.z32[3 * row + k] = zv[k];
                    comp_add_prod(c2[0], rv[k], zv[k]);
                    comp_add_prod(c2[1], rv[k], rv[k]);
                }
            }
            float t2[2];
            team_sum_comp<2>(c2, t2, tm, sh);
            const float beta = (!restart && rho != 0.f && isfinite(t2[0])) ? t2[0] / rho : 0.f;
            rho = t2[0];
            rmax = sqrtf(t2[1]);
            rmin = rmax;
            for (int64_t s = sp.w0; s * 32 < nb; s += sp.nw) {
                const int64_t row = s * 32 + lane;
                if (row >= nb) continue;
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const int64_t i = 3 * row + k;
                    D.p32[i] = beta == 0.f ? D.z32[i] : fmaf(beta, D.p32[i], D.z32[i]);
                }
            }
            team_sync(tm);
        }
        // FP32 iterations until the residual fell by delta (or trouble)
        bool poisoned = false, broke = false, diverged = false;
        for (;;) {
            if (it >= P.itrmax) break;
            if (P.abort && it % kAbortEvery == 0 && team_abort(P, tm, sh)) {
                status = PFG_E_ABORTED;
                break;
            }
            Comp32 c1[1] = {Comp32{0.f, 0.f}};
            for (int64_t s = sp.w0; s < A.ns; s += sp.nw) {
                float y[3];
                sell_row_product<3>(A, s, lane, GatherCG<float>{D.p32}, y);
                const int64_t row = s * 32 + lane;
                if (row < nb)
#pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        const int64_t i = 3 * row + k;
                        D.q32[i] = y[k];
                        comp_add_prod(c1[0], D.p32[i], y[k]);
                    }
            }
            float pq[1];
            team_sum_comp<1>(c1, pq, tm, sh);
            if (!(pq[0] > 0.f) || !isfinite(pq[0])) {
                broke = true;
                break;
            }
            const float alpha = rho / pq[0];
            Comp32 c2[2] = {Comp32{0.f, 0.f}, Comp32{0.f, 0.f}};
            for (int64_t s = sp.w0; s * 32 < nb; s += sp.nw) {
                const int64_t row = s * 32 + lane;
                if (row >= nb) continue;
                float rv[3], zv[3];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const int64_t i = 3 * row + k;
                    D.x32[i] = fmaf(alpha, D.p32[i], D.x32[i]);
                    rv[k] = fmaf(-alpha, D.q32[i], D.r32[i]);
                    D.r32[i] = rv[k];
                }
                precond3<float>(pc, D.dinv32, row, rv, zv);
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    D.z32[3 * row + k] = zv[k];
                    comp_add_prod(c2[0], rv[k], zv[k]);
                    comp_add_prod(c2[1], rv[k], rv[k]);
                }
            }
            float t2[2];
            team_sum_comp<2>(c2, t2, tm, sh);
            ++it;
            if (!isfinite(t2[0]) || !isfinite(t2[1])) {
                poisoned = true;
                break;
            }
            const float rn = sqrtf(t2[1]);
            rmax = fmaxf(rmax, rn);
            rmin = fminf(rmin, rn);
            if (rn > kDiverge * rmin) {
                diverged = true;
                break;
            }
            if ((double)rn < P.delta * (double)rmax || (double)rn <= tol_b) {
                // residual replacement; the restart block recomputes rho and
                // keeps the direction through beta = rho_new / rho
                break;
            }
            const float beta = t2[0] / rho;
            rho = t2[0];
            for (int64_t s = sp.w0; s * 32 < nb; s += sp.nw) {
                const int64_t row = s * 32 + lane;
                if (row >= nb) continue;
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const int64_t i = 3 * row + k;
                    D.p32[i] = fmaf(beta, D.p32[i], D.z32[i]);
                }
            }
            team_sync(tm);
        }
        // Keep the FP32 correction only if it lowers the FP64 residual: the
        // candidate b - K (x + x32) goes to q64; on acceptance it becomes r64
        // and x32 is folded into x, otherwise x and r64 stay as they were.
        bool accepted = false;
        double rt = cur_rt;
        if (!poisoned) {
            rt = candidate_residual(D, sp, tm, sh);
            accepted = isfinite(rt) && rt < cur_rt;
        }
        for (int64_t s = sp.w0; s * 32 < nb; s += sp.nw) {
            const int64_t row = s * 32 + lane;
            if (row >= nb) continue;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const int64_t i = 3 * row + k;
                if (accepted) {
                    D.x[i] += (double)D.x32[i];
                    D.r64[i] = D.q64[i];
                }
                D.x32[i] = 0.f;
            }
        }
        team_sync(tm);
        ++reps;
        if (accepted) cur_rt = rt;
        rt = cur_rt;
        rel = bb > 0.0 ? sqrt(rt / bb) : 0.0;
        if (status == PFG_E_ABORTED) break;
        if (sqrt(rt) <= tol_b) {
            converged = true;
            break;
        }
        if (it >= P.itrmax) {
            status = PFG_W_NOT_CONVERGED;
            break;
        }
        if (rt < 0.81 * best_rt) {
            best_rt = rt;
            stall = 0;
        } else {
            ++stall;
        }
        restart = poisoned || broke || diverged || !accepted;
        failures = restart ? failures + 1 : 0;
        if (failures >= kMaxFailures || stall >= kMaxStall) {
            // FP32 cannot carry this system: FP64 CG from the current x
            fallback = 1;
            int restarts = 0;
            status = cg64<NT>(P, D, tm, sh, it, restarts, rel);
            break;
        }
    }
    finish_job(P, m, D, tm, status, it, reps, fallback, rel);
}

template <bool MIXED, int NT>
__device__ __forceinline__ void solve_job(const BatchParams &P, int m, Team &tm, TeamShared &sh)
{
    if (MIXED && !(P.force64 && P.force64[m]))
        solve_mixed<NT>(P, m, tm, sh);
    else
        solve_fp64<NT>(P, m, tm, sh, MIXED ? 2 : 0);
}

template <bool MIXED, int NT>
__global__ void __launch_bounds__(NT, 1) k_batch_cg(BatchParams P)
{
    __shared__ TeamShared sh;
    if (P.cluster > 1) {
        // team phase: the cluster takes jobs together
        cg::cluster_group cl = cg::this_cluster();
        const int rank = (int)cl.block_rank();
        for (;;) {
            if (rank == 0 && threadIdx.x == 0) sh.job = (int)atomicAdd(P.queue, 1u);
            cl.sync();
            const int job = *cl.map_shared_rank(&sh.job, 0);
            cl.sync();  // every CTA has read the job before rank 0 overwrites it
            if (job >= P.n_team) break;
            Team tm{rank, P.cluster, 0};
            solve_job<MIXED, NT>(P, P.order[job], tm, sh);
        }
    }
    // single-CTA phase
    const int n_solo = P.n_total - P.n_team;
    for (;;) {
        if (threadIdx.x == 0) sh.job = (int)atomicAdd(P.queue + 1, 1u);
        __syncthreads();
        const int job = sh.job;
        __syncthreads();
        if (job >= n_solo) break;
        Team tm{0, 1, 0};
        solve_job<MIXED, NT>(P, P.order[P.n_team + job], tm, sh);
    }
}

}  // namespace
}  // namespace pfg

// ------------------------------------------------------------------ host side
namespace pfg {
namespace {

const void *batch_kernel(bool mixed, int threads)
{
    if (mixed) {
        if (threads == 256) return (const void *)k_batch_cg<true, 256>;
        if (threads == 512) return (const void *)k_batch_cg<true, 512>;
        return (const void *)k_batch_cg<true, 1024>;
    }
    if (threads == 256) return (const void *)k_batch_cg<false, 256>;
    if (threads == 512) return (const void *)k_batch_cg<false, 512>;
    return (const void *)k_batch_cg<false, 1024>;
}

int device_sms()
{
    int dev = 0, n = 0;
    PFG_CUDA(cudaGetDevice(&dev));
    PFG_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
    return n;
}

void fill_launch(cudaLaunchConfig_t &lc, cudaLaunchAttribute &attr, int grid, int threads, int cluster,
                 cudaStream_t st)
{
    memset(&lc, 0, sizeof(lc));
    lc.gridDim = dim3((unsigned)grid, 1, 1);
    lc.blockDim = dim3((unsigned)threads, 1, 1);
    lc.dynamicSmemBytes = 0;
    lc.stream = st;
    lc.attrs = nullptr;
    lc.numAttrs = 0;
    if (cluster > 1) {
        attr.id = cudaLaunchAttributeClusterDimension;
        attr.val.clusterDim.x = (unsigned)cluster;
        attr.val.clusterDim.y = 1;
        attr.val.clusterDim.z = 1;
        lc.attrs = &attr;
        lc.numAttrs = 1;
    }
}

// Persistent grid: as many CTAs (or clusters) as can be resident at once.
int persistent_grid(bool mixed, int threads, int cluster)
{
    const void *fn = batch_kernel(mixed, threads);
    const int sms = device_sms();
    if (cluster <= 1) {
        int per_sm = 0;
        PFG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0));
        return std::max(per_sm, 0) * sms;
    }
    cudaLaunchConfig_t lc;
    cudaLaunchAttribute attr;
    fill_launch(lc, attr, cluster * sms, threads, cluster, nullptr);
    int clusters = 0;
    PFG_CUDA(cudaOccupancyMaxActiveClusters(&clusters, fn, &lc));
    return std::max(clusters, 0) * cluster;
}

bool valid_config(const pfg_batch_config &c)
{
    return (c.threads == 256 || c.threads == 512 || c.threads == 1024) &&
           (c.cluster == 1 || c.cluster == 2 || c.cluster == 4 || c.cluster == 8) && c.team_fraction >= 0.0 &&
           c.team_fraction <= 1.0;
}

uint64_t mix(uint64_t h, uint64_t v)
{
    h ^= v + 0x9e3779b97f4a7c15ULL + (h << 6) + (h >> 2);
    return h;
}

}  // namespace
}  // namespace pfg

using namespace pfg;

struct pfg_batch {
    std::mutex mu;
    int device = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    std::vector<pfg_solver *> handles;
    std::vector<BatchSource> src;
    std::vector<int64_t> ndof, off;   // DOF of each system and its offset in the pooled vectors
    int64_t total = 0;                // pooled length (each system padded to 32 values)
    DevBuf<double> v64;               // x | r | p | q | z | s, `total` values each
    DevBuf<float> v32;                // x32 | r32 | p32 | q32 | z32
    DevBuf<double> d64;               // block-Jacobi inverses, 3 * total
    DevBuf<float> d32;
    int dinv_kind = -1;               // preconditioner the inverses hold
    DevBuf<BatchMesh> meshes;
    DevBuf<BatchOut> out;
    DevBuf<int> order;
    DevBuf<unsigned> queue;
    std::vector<double> work;         // matrix blocks of each system (work per iteration)
    std::vector<int> last_iters;      // iterations of the previous solve (0: none yet)
    std::vector<int> iters64;         // iterations of the last FP64 solve of each system (0: none)
    std::vector<uint8_t> force64;     // mixed: systems to solve in FP64 (learned)
    DevBuf<uint8_t> force64_d;
    pfg_batch_config cfg{512, 4, 0.25};
    bool tuned = false;
    int *abort_h = nullptr;           // host-mapped abort flag
    int *abort_d = nullptr;
    cudaGraphExec_t graph = nullptr;
    uint64_t graph_key = 0;
    std::vector<BatchOut> out_h;

    ~pfg_batch()
    {
        if (graph) cudaGraphExecDestroy(graph);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (abort_h) cudaFreeHost(abort_h);
        if (st) cudaStreamDestroy(st);
    }
};

namespace {

void need(bool c, int code, const char *msg)
{
    if (!c) throw Error(code, msg);
}

struct RunSpec {
    bool mixed;
    int precond, itrmax;
    double tol, delta;
    int debug;
};

RunSpec run_spec(const pfg_solve_opts *opts)
{
    pfg_solve_opts o;
    if (opts)
        o = *opts;
    else {
        pfg_solve_opts_default(&o);
        o.algorithm = PFG_ALG_CG;
        o.precision = PFG_PREC_MIXED;
        o.precond = PFG_PC_BLOCK_JACOBI;
    }
    need(o.algorithm == PFG_ALG_CG, PFG_E_UNSUPPORTED,
         "batched solves run CG (the bound systems are symmetric positive definite)");
    need(o.precision == PFG_PREC_FP64 || o.precision == PFG_PREC_MIXED, PFG_E_ARG, "precision");
    need(o.precond == PFG_PC_NONE || o.precond == PFG_PC_JACOBI || o.precond == PFG_PC_BLOCK_JACOBI, PFG_E_ARG,
         "precond");
    need(o.itrmax > 0 && o.relative_er > 0.0, PFG_E_ARG, "itrmax and relative_er must be positive");
    need(o.reliable_delta > 0.0 && o.reliable_delta < 1.0, PFG_E_ARG, "reliable_delta must lie in (0, 1)");
    return RunSpec{o.precision == PFG_PREC_MIXED, o.precond, o.itrmax, o.relative_er, o.reliable_delta, o.debug};
}

// Launches one batched solve with configuration c (graph replay when the
// captured one matches); returns the device milliseconds of the launch.
double run_batch(pfg_batch *b, const RunSpec &rs, const pfg_batch_config &c)
{
    const int count = (int)b->src.size();
    // block-Jacobi inverses for the requested preconditioner
    if (rs.precond != PFG_PC_NONE && b->dinv_kind != rs.precond) {
        for (int m = 0; m < count; ++m)
            block_jacobi(*b->src[m].K, rs.precond, b->d64.p + 3 * b->off[m], b->d32.p + 3 * b->off[m], b->st);
        b->dinv_kind = rs.precond;
    }
    // longest estimated work first: blocks x iterations (previous solve, else sqrt of the rows)
    std::vector<int> ord((size_t)count);
    std::iota(ord.begin(), ord.end(), 0);
    std::vector<double> cost((size_t)count);
    for (int m = 0; m < count; ++m) {
        const double it = b->last_iters[m] > 0 ? (double)b->last_iters[m] : std::sqrt((double)b->ndof[m]);
        cost[m] = b->work[m] * it;
    }
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int d) { return cost[a] > cost[d]; });
    int n_team = 0;
    if (c.cluster > 1) n_team = std::min(count, (int)std::lround(c.team_fraction * count));
    PFG_CUDA(cudaMemcpyAsync(b->order.p, ord.data(), count * sizeof(int), cudaMemcpyHostToDevice, b->st));

    const int grid = persistent_grid(rs.mixed, c.threads, c.cluster);
    need(grid > 0, PFG_E_UNSUPPORTED, "batched kernel configuration cannot be resident on this GPU");
    BatchParams P;
    P.mesh = b->meshes.p;
    P.out = b->out.p;
    P.order = b->order.p;
    P.n_team = n_team;
    P.n_total = count;
    P.cluster = c.cluster;
    P.queue = b->queue.p;
    P.precond = rs.precond;
    P.itrmax = rs.itrmax;
    P.max_restarts = 5;
    P.tol = rs.tol;
    P.delta = rs.delta;
    P.abort = b->abort_d;
    P.force64 = rs.mixed ? b->force64_d.p : nullptr;
    if (rs.mixed)
        PFG_CUDA(cudaMemcpyAsync(b->force64_d.p, b->force64.data(), count, cudaMemcpyHostToDevice, b->st));

    uint64_t key = 0x51ab;
    for (uint64_t v : {(uint64_t)rs.mixed, (uint64_t)rs.precond, (uint64_t)rs.itrmax, (uint64_t)c.threads,
                       (uint64_t)c.cluster, (uint64_t)n_team, (uint64_t)count, (uint64_t)grid,
                       (uint64_t)(uintptr_t)b->meshes.p, (uint64_t)(uintptr_t)b->v64.p,
                       (uint64_t)(uintptr_t)b->abort_d, (uint64_t)(uintptr_t)b->force64_d.p})
        key = mix(key, v);
    uint64_t tb, db;
    memcpy(&tb, &rs.tol, 8);
    memcpy(&db, &rs.delta, 8);
    key = mix(mix(key, tb), db);
    if (!b->graph || b->graph_key != key) {
        if (b->graph) cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
        cudaGraph_t g;
        PFG_CUDA(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
        // x0 = 0 for every system, empty job queues, then the persistent kernel
        cudaMemsetAsync(b->v64.p, 0, b->total * sizeof(double), b->st);
        cudaMemsetAsync(b->queue.p, 0, 2 * sizeof(unsigned), b->st);
        cudaLaunchConfig_t lc;
        cudaLaunchAttribute attr;
        fill_launch(lc, attr, grid, c.threads, c.cluster, b->st);
        void *args[] = {&P};
        const cudaError_t le = cudaLaunchKernelExC(&lc, batch_kernel(rs.mixed, c.threads), args);
        const cudaError_t ce = cudaStreamEndCapture(b->st, &g);
        PFG_CUDA(le);
        PFG_CUDA(ce);
        const cudaError_t ie = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        PFG_CUDA(ie);
        b->graph_key = key;
    }
    PFG_CUDA(cudaEventRecord(b->e0, b->st));
    PFG_CUDA(cudaGraphLaunch(b->graph, b->st));
    PFG_CUDA(cudaEventRecord(b->e1, b->st));
    b->out_h.resize((size_t)count);
    PFG_CUDA(cudaMemcpyAsync(b->out_h.data(), b->out.p, count * sizeof(BatchOut), cudaMemcpyDeviceToHost, b->st));
    PFG_CUDA(cudaStreamSynchronize(b->st));
    PFG_CUDA(cudaGetLastError());
    float ms = 0.f;
    PFG_CUDA(cudaEventElapsedTime(&ms, b->e0, b->e1));
    for (int m = 0; m < count; ++m) {
        const BatchOut &o = b->out_h[m];
        b->last_iters[m] = std::max(o.iterations, 1);
        if (!rs.mixed || o.fallback == 2) {
            if (o.status == PFG_OK) b->iters64[m] = o.iterations;
        } else if (o.fallback == 1) {
            b->force64[m] = 1;  // the FP32 operator failed on this system
        } else if (b->iters64[m] > 0 && o.iterations > 3 * b->iters64[m] / 2) {
            b->force64[m] = 1;  // FP32 needs 1.5x the FP64 iterations: no gain
        }
    }
    return (double)ms;
}

}  // namespace

extern "C" {

int pfg_batch_create(pfg_batch **out)
{
    return guard([&] {
        need(out != nullptr, PFG_E_ARG, "NULL batch pointer");
        pfg_batch *b = new pfg_batch();
        try {
            PFG_CUDA(cudaGetDevice(&b->device));
            PFG_CUDA(cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking));
            PFG_CUDA(cudaEventCreate(&b->e0));
            PFG_CUDA(cudaEventCreate(&b->e1));
            PFG_CUDA(cudaHostAlloc((void **)&b->abort_h, sizeof(int), cudaHostAllocMapped));
            *b->abort_h = 0;
            PFG_CUDA(cudaHostGetDevicePointer((void **)&b->abort_d, b->abort_h, 0));
            b->queue.alloc(2);
        } catch (...) {
            delete b;
            throw;
        }
        *out = b;
    });
}

int pfg_batch_destroy(pfg_batch *b)
{
    return guard([&] {
        if (!b) return;
        {
            std::lock_guard<std::mutex> lk(b->mu);
            if (b->st) cudaStreamSynchronize(b->st);
        }
        delete b;
    });
}

int pfg_batch_set(pfg_batch *b, int64_t count, pfg_solver *const *handles)
{
    return guard([&] {
        need(b && handles && count > 0, PFG_E_ARG, "batch, handles and count > 0 required");
        need(count <= (int64_t)1 << 24, PFG_E_ARG, "too many systems in one batch");
        std::lock_guard<std::mutex> lk(b->mu);
        int dev = 0;
        PFG_CUDA(cudaGetDevice(&dev));
        need(dev == b->device, PFG_E_STATE, "batch used on another device than it was created on");
        std::vector<BatchSource> src((size_t)count);
        for (int64_t m = 0; m < count; ++m) {
            src[m] = batch_bind(handles[m]);
            need(src[m].device == b->device, PFG_E_ARG, "batch member on another device");
        }
        b->handles.assign(handles, handles + count);
        b->src = std::move(src);
        b->ndof.resize((size_t)count);
        b->off.resize((size_t)count);
        b->work.resize((size_t)count);
        b->last_iters.assign((size_t)count, 0);
        b->iters64.assign((size_t)count, 0);
        b->force64.assign((size_t)count, 0);
        b->force64_d.resize((size_t)count);
        int64_t tot = 0;
        for (int64_t m = 0; m < count; ++m) {
            const DevMatrix &K = *b->src[m].K;
            b->ndof[m] = K.ndof();
            b->off[m] = tot;
            b->work[m] = (double)K.nnzb;
            tot += (K.ndof() + 31) / 32 * 32;
        }
        b->total = tot;
        b->v64.resize((size_t)tot * 6);
        b->v32.resize((size_t)tot * 5);
        b->d64.resize((size_t)tot * 3);
        b->d32.resize((size_t)tot * 3);
        b->dinv_kind = -1;
        std::vector<BatchMesh> hm((size_t)count);
        for (int64_t m = 0; m < count; ++m) {
            const BatchSource &s = b->src[m];
            BatchMesh &d = hm[m];
            const int64_t o = b->off[m];
            d.A64 = s.K->sell<double>();
            d.A32 = s.K->sell<float>();
            d.b = s.b;
            d.fixed = s.fixed;
            d.fixval = s.fixval;
            d.x = b->v64.p + o;
            d.r64 = b->v64.p + tot + o;
            d.p64 = b->v64.p + 2 * tot + o;
            d.q64 = b->v64.p + 3 * tot + o;
            d.z64 = b->v64.p + 4 * tot + o;
            d.s64 = b->v64.p + 5 * tot + o;
            d.x32 = b->v32.p + o;
            d.r32 = b->v32.p + tot + o;
            d.p32 = b->v32.p + 2 * tot + o;
            d.q32 = b->v32.p + 3 * tot + o;
            d.z32 = b->v32.p + 4 * tot + o;
            d.dinv64 = b->d64.p + 3 * o;
            d.dinv32 = b->d32.p + 3 * o;
        }
        b->meshes.resize((size_t)count);
        b->out.resize((size_t)count);
        b->order.resize((size_t)count);
        PFG_CUDA(cudaMemcpyAsync(b->meshes.p, hm.data(), count * sizeof(BatchMesh), cudaMemcpyHostToDevice, b->st));
        PFG_CUDA(cudaMemsetAsync(b->out.p, 0, count * sizeof(BatchOut), b->st));
        PFG_CUDA(cudaStreamSynchronize(b->st));
        if (b->graph) cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    });
}

int pfg_batch_set_config(pfg_batch *b, const pfg_batch_config *cfg)
{
    return guard([&] {
        need(b && cfg, PFG_E_ARG, "NULL argument");
        need(valid_config(*cfg), PFG_E_ARG, "threads 256/512/1024, cluster 1/2/4/8, team_fraction in [0, 1]");
        std::lock_guard<std::mutex> lk(b->mu);
        b->cfg = *cfg;
    });
}

int pfg_batch_get_config(pfg_batch *b, pfg_batch_config *cfg, int32_t *tuned)
{
    return guard([&] {
        need(b && cfg, PFG_E_ARG, "NULL argument");
        std::lock_guard<std::mutex> lk(b->mu);
        *cfg = b->cfg;
        if (tuned) *tuned = b->tuned ? 1 : 0;
    });
}

int pfg_batch_solve(pfg_batch *b, const pfg_solve_opts *opts, double *const *x_out, pfg_info *infos,
                    pfg_batch_info *binfo)
{
    int worst = PFG_OK;
    const int rc = guard([&] {
        need(b != nullptr, PFG_E_ARG, "NULL batch");
        std::lock_guard<std::mutex> lk(b->mu);
        need(!b->src.empty(), PFG_E_STATE, "solve before pfg_batch_set");
        const RunSpec rs = run_spec(opts);
        const double ms = run_batch(b, rs, b->cfg);
        const int count = (int)b->src.size();
        int64_t tot_it = 0;
        int max_it = 0, fallbacks = 0;
        double max_rel = 0.0;
        for (int m = 0; m < count; ++m) {
            const BatchOut &o = b->out_h[m];
            if (x_out && x_out[m])
                PFG_CUDA(cudaMemcpyAsync(x_out[m], b->v64.p + b->off[m], b->ndof[m] * sizeof(double),
                                         cudaMemcpyDeviceToHost, b->st));
            if (infos) {
                pfg_info &in = infos[m];
                memset(&in, 0, sizeof(in));
                in.status = o.status;
                in.iterations = o.iterations;
                in.replacements = o.replacements;
                in.kernel_launches = 1;
                in.rel_residual = o.rel_residual;
                in.iter_residual = o.rel_residual;
                in.solve_ms = ms;
                in.fallback = o.fallback;
            }
            tot_it += o.iterations;
            max_it = std::max(max_it, o.iterations);
            max_rel = std::max(max_rel, o.rel_residual);
            fallbacks += o.fallback != 0;
            if (o.status < 0 && (worst >= 0)) worst = o.status;
            if (o.status > 0 && worst == PFG_OK) worst = o.status;
        }
        PFG_CUDA(cudaStreamSynchronize(b->st));
        if (binfo) {
            memset(binfo, 0, sizeof(*binfo));
            binfo->config = b->cfg;
            binfo->launches = 1;
            binfo->max_iterations = max_it;
            binfo->total_iterations = tot_it;
            binfo->max_rel_residual = max_rel;
            binfo->solve_ms = ms;
            binfo->fallbacks = fallbacks;
        }
        if (worst < 0) {
            set_last_error("a batched system ended with status " + std::to_string(worst));
        }
    });
    if (rc != PFG_OK) return rc;
    return worst;
}

int pfg_batch_get_x(pfg_batch *b, int64_t index, double *x_out)
{
    return guard([&] {
        need(b && x_out, PFG_E_ARG, "NULL argument");
        std::lock_guard<std::mutex> lk(b->mu);
        need(index >= 0 && index < (int64_t)b->src.size(), PFG_E_ARG, "index out of range");
        PFG_CUDA(cudaMemcpyAsync(x_out, b->v64.p + b->off[index], b->ndof[index] * sizeof(double),
                                 cudaMemcpyDeviceToHost, b->st));
        PFG_CUDA(cudaStreamSynchronize(b->st));
    });
}

int pfg_batch_tune(pfg_batch *b, const pfg_solve_opts *opts, pfg_batch_config *best, double *best_ms)
{
    return guard([&] {
        need(b != nullptr, PFG_E_ARG, "NULL batch");
        std::lock_guard<std::mutex> lk(b->mu);
        need(!b->src.empty(), PFG_E_STATE, "tune before pfg_batch_set");
        const RunSpec rs = run_spec(opts);
        // one untimed solve fills the iteration counts the job order uses
        run_batch(b, rs, b->cfg);
        pfg_batch_config cur = b->cfg, top = b->cfg;
        double top_ms = 1e300;
        auto trial = [&](const pfg_batch_config &c) {
            if (!valid_config(c)) return;
            if (persistent_grid(rs.mixed, c.threads, c.cluster) <= 0) return;
            const double ms = run_batch(b, rs, c);
            if (rs.debug)
                fprintf(stderr, "[pfg] batch tune: threads %d cluster %d team share %.4f: %.2f ms\n", c.threads,
                        c.cluster, c.team_fraction, ms);
            if (ms < top_ms) {
                top_ms = ms;
                top = c;
            }
        };
        // stage 1: CTA size (block rows per CTA tile) x team size; stage 2: team share
        for (int nt : {256, 512, 1024})
            for (int cl : {1, 2, 4, 8}) {
                pfg_batch_config c = cur;
                c.threads = nt;
                c.cluster = cl;
                c.team_fraction = cl > 1 ? 0.125 : 0.0;
                trial(c);
            }
        cur = top;
        if (cur.cluster > 1)
            for (double f : {0.0625, 0.25, 0.5, 1.0}) {
                pfg_batch_config c = cur;
                c.team_fraction = f;
                trial(c);
            }
        b->cfg = top;
        b->tuned = true;
        if (best) *best = top;
        if (best_ms) *best_ms = top_ms;
    });
}

int pfg_batch_abort_flag(pfg_batch *b, volatile int32_t **flag)
{
    return guard([&] {
        need(b && flag, PFG_E_ARG, "NULL argument");
        *flag = (volatile int32_t *)b->abort_h;
    });
}

}  // extern "C"
