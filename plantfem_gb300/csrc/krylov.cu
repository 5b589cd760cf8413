// krylov.cu -- CG and BiCGSTAB on the device, FP64 and mixed precision.
//
// Restates bicgstab_CRS_2 (FEMSolverClass.f90:2199-2298) and adds CG for the
// symmetric eliminated system.  Design:
//   * every scalar (rho, alpha, beta, c1..c3, norms) lives in device memory
//     (KState); the last CTA of each fused reduction computes the next scalars,
//     so one iteration is 2 (CG) or 3 (BiCGSTAB) kernel launches and no host
//     round trip;
//   * the direction update p = z + beta p (CG) or p = r + beta (p - c3 y)
//     (BiCGSTAB) is fused into the SpMV that consumes p: the gathered source
//     value of every block column is formed on the fly, the owning warp writes
//     the row's new p to a ping-pong buffer;
//   * a chunk of iterations is captured once into a CUDA graph and replayed;
//     kernels return at entry once KState says done (or, mixed precision, that
//     a residual replacement is due), and the host checks KState once per chunk;
//   * mixed precision: matrix, vectors and dots in FP32 (dots compensated,
//     Dot2 of Ogita-Rump-Oishi); the solution is accumulated in FP64 and the
//     FP32 residual is replaced by the FP64 residual b - A x (FP64 SpMV) each
//     time it dropped by reliable_delta ("reliable updates", Sleijpen & van der
//     Vorst 1996, as used for mixed-precision CG by Clark et al. 2010).  The
//     stop test is always on that FP64 residual.
#include <cmath>
#include <mutex>
#include <unordered_map>

#include "krylov.cuh"
#include "ilu.cuh"
#include "bulk.cuh"

namespace pfg {

static int g_sm_count = 0;

static int sm_count()
{
    if (g_sm_count == 0) {
        int dev = 0;
        PFG_CUDA(cudaGetDevice(&dev));
        PFG_CUDA(cudaDeviceGetAttribute(&g_sm_count, cudaDevAttrMultiProcessorCount, dev));
        if (g_sm_count <= 0) g_sm_count = 1;
    }
    return g_sm_count;
}

constexpr int kThreads = 256;  // 8 warps per CTA for every row kernel
constexpr int kWarps = kThreads / 32;

int Krylov::row_grid(int64_t nb)
{
    // Persistent-style grid: a fixed number of resident CTAs per SM, each warp
    // striding over block rows.  6 CTAs x 256 threads keeps 48 warps per SM.
    int64_t want = (nb + kWarps - 1) / kWarps;
    int64_t cap = (int64_t)sm_count() * 6;
    return (int)std::max<int64_t>(1, std::min(want, cap));
}

// Grid of exactly the CTAs that are resident at once (occupancy query, cached
// per kernel), capped by the work: one wave, every warp striding over units.
template <typename K>
static int resident_grid(K kern, int64_t warps_needed)
{
    static std::mutex mu;
    static std::unordered_map<const void *, int> cache;
    int per_sm = 0;
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find((const void *)kern);
        if (it == cache.end()) {
            PFG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, 0));
            cache[(const void *)kern] = per_sm;
        } else {
            per_sm = it->second;
        }
    }
    const int64_t want = (warps_needed + kWarps - 1) / kWarps;
    return (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)std::max(per_sm, 1) * sm_count()));
}

template <int BS, typename T>
__device__ __forceinline__ T pick(const T (&y)[BS], int i)
{
    T v = y[0];
#pragma unroll
    for (int k = 1; k < BS; ++k) v = (i == k) ? y[k] : v;
    return v;
}

// ---------------------------------------------------------------- reductions
template <typename T>
struct Acc;
template <>
struct Acc<double> {
    using type = double;
    __device__ static double zero() { return 0.0; }
    __device__ static void add(double &a, double x, double y) { a = fma(x, y, a); }
};
template <>
struct Acc<float> {
    using type = Comp32;
    __device__ static Comp32 zero() { return Comp32{0.f, 0.f}; }
    __device__ static void add(Comp32 &a, float x, float y) { comp_add_prod(a, x, y); }
};

template <int NV>
__device__ __forceinline__ bool grid_total(double (&v)[NV], double *pd, float *, unsigned *ticket,
                                           double (&tot)[NV])
{
    return grid_sum<NV>(v, pd, ticket, tot);
}
template <int NV>
__device__ __forceinline__ bool grid_total(Comp32 (&v)[NV], double *, float *pf, unsigned *ticket,
                                           float (&tot)[NV])
{
    return grid_sum_comp<NV>(v, pf, ticket, tot);
}

__device__ __forceinline__ bool finite_d(double x) { return isfinite(x); }

// *bits = max(*bits, v) for non-negative floats (their bit patterns order as
// unsigned integers); one atomic per CTA (every thread of the CTA calls this).
// A non-finite v is kept as +inf.
__device__ __forceinline__ void track_abs_max(float v, unsigned *bits)
{
    __shared__ float wmax[32];
    if (!(v <= 3.0e38f)) v = __int_as_float(0x7f800000);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if ((threadIdx.x & 31) == 0) wmax[w] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        float m = wmax[0];
        for (int k = 1; k < nw; ++k) m = fmaxf(m, wmax[k]);
        atomicMax(bits, __float_as_uint(m));
    }
}

// ------------------------------------------------------------ plain kernels
template <int BS, typename T>
__global__ void __launch_bounds__(kThreads) k_spmv(BsrView<T> A, const T *__restrict__ x, T *__restrict__ y)
{
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t row = w0; row < A.nb; row += nw) {
        T acc[BS];
        auto src = [&](int c, T(&xv)[BS]) {
#pragma unroll
            for (int i = 0; i < BS; ++i) xv[i] = __ldg(x + (int64_t)BS * c + i);
        };
        bsr_row_product<BS>(A, row, lane, src, acc);
        if (lane < BS) y[(int64_t)BS * row + lane] = pick<BS>(acc, lane);
    }
}

// Slice loop of the sliced-ELL kernels: warp w takes slices w, w + nw, ...;
// lane l owns block row 32 s + l.
#define PFG_SLICE_LOOP(A)                                                          \
    const int lane = threadIdx.x & 31;                                             \
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;      \
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;                     \
    for (int64_t s = w0; s < (A).ns; s += nw)

// y = A x on the sliced copy (plain SpMV, profiling and the FP32 entry point).
template <int BS, typename T>
__global__ void __launch_bounds__(kThreads) k_spmv_sell(SellView<T> A, const T *__restrict__ x, T *__restrict__ y)
{
    PFG_SLICE_LOOP(A)
    {
        T acc[BS];
        auto src = [&](int c, T(&xv)[BS]) {
#pragma unroll
            for (int i = 0; i < BS; ++i) xv[i] = __ldg(x + (int64_t)BS * c + i);
        };
        sell_row_product<BS>(A, s, lane, src, acc);
        const int64_t row = s * 32 + lane;
        if (row < A.nb)
#pragma unroll
            for (int i = 0; i < BS; ++i) y[BS * row + i] = acc[i];
    }
}

// r = b - A x in FP64; totals: true_rr = r.r and bb = b.b into KState.
template <int BS>
__global__ void __launch_bounds__(kThreads) k_residual64(SellView<double> A, const double *__restrict__ b,
                                                         const double *__restrict__ x, double *__restrict__ r,
                                                         KState *S, double *partials, unsigned *ticket)
{
    double acc[2] = {0.0, 0.0};
    PFG_SLICE_LOOP(A)
    {
        double y[BS];
        auto src = [&](int c, double(&xv)[BS]) {
#pragma unroll
            for (int i = 0; i < BS; ++i) xv[i] = __ldg(x + (int64_t)BS * c + i);
        };
        sell_row_product<BS>(A, s, lane, src, y);
        const int64_t row = s * 32 + lane;
        if (row < A.nb) {
#pragma unroll
            for (int k = 0; k < BS; ++k) {
                const int64_t i = (int64_t)BS * row + k;
                const double bi = b[i];
                const double ri = bi - y[k];
                r[i] = ri;
                acc[0] = fma(ri, ri, acc[0]);
                acc[1] = fma(bi, bi, acc[1]);
            }
        }
    }
    double tot[2];
    if (grid_sum<2>(acc, partials, ticket, tot)) {
        S->true_rr = tot[0];
        S->bb = tot[1];
    }
}

template <int BS, typename T>
__device__ __forceinline__ void pc_apply(int pc, const T *__restrict__ dinv, int64_t row, const T (&r)[BS],
                                         T (&z)[BS])
{
    if (pc == PFG_PC_NONE) {
#pragma unroll
        for (int i = 0; i < BS; ++i) z[i] = r[i];
        return;
    }
    const T *D = dinv + row * (BS * BS);
#pragma unroll
    for (int i = 0; i < BS; ++i) {
        T s = T(0);
#pragma unroll
        for (int j = 0; j < BS; ++j) s = fma(__ldg(D + i * BS + j), r[j], s);
        z[i] = s;
    }
}

// Inverse of the diagonal block of every block row (block Jacobi), or of the
// diagonal entries only (point Jacobi).  A zero pivot keeps the identity, as
// JacobiPreconditionerCRS skips rows with A_kk == 0 (FEMSolverClass.f90:2519).
template <int BS>
__global__ void k_precond(BsrView<double> A, int pc, double *__restrict__ d64, float *__restrict__ d32)
{
    for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < A.nb;
         row += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = A.rp[row];
        const int nblk = (int)(A.rp[row + 1] - s);
        double D[BS * BS];
#pragma unroll
        for (int e = 0; e < BS * BS; ++e) D[e] = 0.0;
        for (int k = 0; k < nblk; ++k)
            if (A.col[s + k] == row) {
#pragma unroll
                for (int e = 0; e < BS * BS; ++e) D[e] = A.val[s * BS * BS + (int64_t)e * nblk + k];
                break;
            }
        double Inv[BS * BS];
#pragma unroll
        for (int e = 0; e < BS * BS; ++e) Inv[e] = 0.0;
        if (pc == PFG_PC_JACOBI || BS == 1) {
#pragma unroll
            for (int i = 0; i < BS; ++i) Inv[i * BS + i] = D[i * BS + i] != 0.0 ? 1.0 / D[i * BS + i] : 1.0;
        } else {
            // 3x3 inverse by cofactors
            const double a = D[0], b = D[1], c = D[2], d = D[3], e = D[4], f = D[5], g = D[6], h = D[7],
                         k = D[8];
            const double c0 = e * k - f * h, c1 = f * g - d * k, c2 = d * h - e * g;
            const double det = a * c0 + b * c1 + c * c2;
            if (det != 0.0 && isfinite(det)) {
                const double id = 1.0 / det;
                Inv[0] = c0 * id;
                Inv[1] = (c * h - b * k) * id;
                Inv[2] = (b * f - c * e) * id;
                Inv[3] = c1 * id;
                Inv[4] = (a * k - c * g) * id;
                Inv[5] = (c * d - a * f) * id;
                Inv[6] = c2 * id;
                Inv[7] = (b * g - a * h) * id;
                Inv[8] = (a * e - b * d) * id;
            } else {
#pragma unroll
                for (int i = 0; i < BS; ++i) Inv[i * BS + i] = D[i * BS + i] != 0.0 ? 1.0 / D[i * BS + i] : 1.0;
            }
        }
#pragma unroll
        for (int e = 0; e < BS * BS; ++e) {
            d64[row * BS * BS + e] = Inv[e];
            if (d32) d32[row * BS * BS + e] = (float)Inv[e];
        }
    }
}

__global__ void k_to_f32(const double *__restrict__ a, float *__restrict__ b, int64_t n)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

// ------------------------------------------------------------------ CG kernels
template <typename T>
__device__ __forceinline__ T st_beta(const KState *S);
template <>
__device__ __forceinline__ double st_beta<double>(const KState *S) { return S->beta; }
template <>
__device__ __forceinline__ float st_beta<float>(const KState *S) { return S->beta32; }
template <typename T>
__device__ __forceinline__ T st_alpha(const KState *S);
template <>
__device__ __forceinline__ double st_alpha<double>(const KState *S) { return S->alpha; }
template <>
__device__ __forceinline__ float st_alpha<float>(const KState *S) { return S->alpha32; }

// q = A p_new, p_new = z + beta p_old formed on the fly; pq = p_new . q;
// fin: alpha = rho / pq.
template <int BS, typename T>
__global__ void __launch_bounds__(kThreads)
    k_cg_spmv(SellView<T> A, const T *__restrict__ z, T *pA, T *pB, T *__restrict__ q, KState *S, double *pd,
              float *pf, unsigned *ticket)
{
    if (S->done | S->need_update) return;
    const T beta = st_beta<T>(S);
    const int par = S->parity;
    const T *pold = par ? pB : pA;
    T *pnew = par ? pA : pB;
    typename Acc<T>::type acc[1] = {Acc<T>::zero()};
    PFG_SLICE_LOOP(A)
    {
        T y[BS];
        auto src = [&](int c, T(&xv)[BS]) {
#pragma unroll
            for (int i = 0; i < BS; ++i) {
                const int64_t j = (int64_t)BS * c + i;
                xv[i] = fma(beta, __ldg(pold + j), __ldg(z + j));
            }
        };
        sell_row_product<BS>(A, s, lane, src, y);
        const int64_t row = s * 32 + lane;
        if (row < A.nb) {
#pragma unroll
            for (int k = 0; k < BS; ++k) {
                const int64_t i = (int64_t)BS * row + k;
                const T pn = fma(beta, pold[i], z[i]);
                pnew[i] = pn;
                q[i] = y[k];
                Acc<T>::add(acc[0], pn, y[k]);
            }
        }
    }
    T tot[1];
    if (grid_total<1>(acc, pd, pf, ticket, tot)) {
        const double pq = (double)tot[0];
        if (!(pq > 0.0) || !finite_d(pq)) {
            S->status = PFG_E_BREAKDOWN;
            S->done = 1;
        } else if (sizeof(T) == 8) {
            S->pq = pq;
            S->alpha = S->rho / pq;
        } else {
            S->alpha32 = (float)(S->rho32 / tot[0]);
        }
    }
}

// Unfused forms.  Forming p = z + beta p inside the gather recomputes it for
// every block that references a node (27 times in a hex mesh): free in FP32,
// but it doubles the FP64 pipe work of the FP64 SpMV, which is already
// FP64-bound on GB300.  So the direction update can also run as its own
// streaming pass, in place, followed by a plain gather.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_cg_dir(int64_t n, const T *__restrict__ z, T *__restrict__ p, KState *S)
{
    if (S->done | S->need_update) return;
    const T beta = st_beta<T>(S);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = fma(beta, p[i], z[i]);
}

// q = A p; pq = p.q; fin: alpha = rho / pq.
template <int BS, typename T>
__global__ void __launch_bounds__(kThreads)
    k_cg_spmv_u(SellView<T> A, const T *__restrict__ p, T *__restrict__ q, KState *S, double *pd, float *pf,
                unsigned *ticket)
{
    if (S->done | S->need_update) return;
    typename Acc<T>::type acc[1] = {Acc<T>::zero()};
    PFG_SLICE_LOOP(A)
    {
        T y[BS];
        auto src = [&](int c, T(&xv)[BS]) {
#pragma unroll
            for (int i = 0; i < BS; ++i) xv[i] = __ldg(p + (int64_t)BS * c + i);
        };
        sell_row_product<BS>(A, s, lane, src, y);
        const int64_t row = s * 32 + lane;
        if (row < A.nb) {
#pragma unroll
            for (int k = 0; k < BS; ++k) {
                const int64_t i = (int64_t)BS * row + k;
                q[i] = y[k];
                Acc<T>::add(acc[0], p[i], y[k]);
            }
        }
    }
    T tot[1];
    if (grid_total<1>(acc, pd, pf, ticket, tot)) {
        const double pq = (double)tot[0];
        if (!(pq > 0.0) || !finite_d(pq)) {
            S->status = PFG_E_BREAKDOWN;
            S->done = 1;
        } else if (sizeof(T) == 8) {
            S->pq = pq;
            S->alpha = S->rho / pq;
        } else {
            S->alpha32 = (float)(S->rho32 / tot[0]);
        }
    }
}

// The end of a CG update pass: the grid totals rho' = <r, z> and <r, r>, then
// (last CTA only) fin (FP64): beta = rho'/rho, stop test on the recursive
// residual; fin (FP32): the same, or request a residual replacement.
template <typename T>
__device__ __forceinline__ void cg_update_tail(typename Acc<T>::type (&acc)[2], KState *S, double *pd, float *pf,
                                               unsigned *ticket, double tol, double delta, int itrmax)
{
    T tot[2];
    if (grid_total<2>(acc, pd, pf, ticket, tot)) {
        S->iter += 1;
        S->parity ^= 1;
        const double rho_n = (double)tot[0], rr = (double)tot[1];
        if (!finite_d(rho_n) || !finite_d(rr)) {
            if (sizeof(T) == 8) {
                S->status = PFG_E_NONFINITE;
                S->done = 1;
            } else {  // FP32 overflow: restart from the FP64 residual
                S->need_update = 1;
                S->breakdowns += 1;
                S->poisoned = 1;
            }
            return;
        }
        if (sizeof(T) == 8) {
            S->rr = rr;
            S->beta = rho_n / S->rho;
            S->rho = rho_n;
            if (sqrt(rr) <= tol * sqrt(S->bb)) S->done = 1;
        } else {
            const float rn = sqrtf((float)rr);
            S->rr32 = (float)rr;
            S->rmax32 = fmaxf(S->rmax32, rn);
            S->rmin32 = fminf(S->rmin32, rn);
            // replace on progress (delta), at the tolerance, or when the FP32
            // recursion diverges (1000x above its minimum since the last
            // replacement); the host keeps the correction only if it lowers
            // the FP64 residual
            if ((double)rn < delta * (double)S->rmax32 || (double)rn <= tol * sqrt(S->bb) ||
                rn > 1000.f * S->rmin32) {
                S->need_update = 1;  // replacement recomputes rho and beta
            } else {
                S->beta32 = (float)(rho_n / (double)S->rho32);
                S->rho32 = (float)rho_n;
            }
        }
        if (S->iter >= itrmax && !S->done) {
            S->status = PFG_W_NOT_CONVERGED;
            S->done = 1;
        }
    }
}

// x += alpha p_new; r -= alpha q; z = M^-1 r; rho' = r.z; rr = r.r.
template <int BS, typename T, int QS = BS>
__global__ void __launch_bounds__(kThreads)
    k_cg_update(int64_t nb, T *__restrict__ x, T *__restrict__ r, T *__restrict__ z, const T *pA, const T *pB,
                T *__restrict__ q, const T *__restrict__ dinv, int pc, KState *S, double *pd, float *pf,
                unsigned *ticket, double tol, double delta, int itrmax)
{
    if (S->done | S->need_update) return;
    const T alpha = st_alpha<T>(S);
    const T *pnew = S->parity ? pA : pB;
    typename Acc<T>::type acc[2] = {Acc<T>::zero(), Acc<T>::zero()};
    for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < nb;
         row += (int64_t)gridDim.x * blockDim.x) {
        T rv[BS], zv[BS];
#pragma unroll
        for (int i = 0; i < BS; ++i) {
            const int64_t j = (int64_t)BS * row + i;
            x[j] = fma(alpha, pnew[j], x[j]);
            rv[i] = fma(-alpha, q[(int64_t)QS * row + i], r[j]);
            r[j] = rv[i];
        }
        // the symmetric product's accumulator (QS = 4): cleared for the next
        // product after the row's reads, as scalars (one 16-byte read and
        // clear of the row at once made the 3.09M-DOF mixed CG 323 ms instead
        // of 258 ms)
        if (QS == 4) {
#pragma unroll
            for (int i = 0; i < 4; ++i) q[4 * row + i] = T(0);
        }
        pc_apply<BS, T>(pc, dinv, row, rv, zv);
#pragma unroll
        for (int i = 0; i < BS; ++i) {
            z[(int64_t)BS * row + i] = zv[i];
            Acc<T>::add(acc[0], rv[i], zv[i]);
            Acc<T>::add(acc[1], rv[i], rv[i]);
        }
    }
    cg_update_tail<T>(acc, S, pd, pf, ticket, tol, delta, itrmax);
}

// (Re)start of CG from the residual r: z = M^-1 r, rho = r.z, beta = 0.
// FP32 version also folds in the residual replacement bookkeeping.
template <int BS, typename T>
__global__ void __launch_bounds__(kThreads)
    k_cg_restart(int64_t nb, const T *__restrict__ r, T *__restrict__ z, const T *__restrict__ dinv, int pc,
                 KState *S, double *pd, float *pf, unsigned *ticket, int keep_direction)
{
    typename Acc<T>::type acc[2] = {Acc<T>::zero(), Acc<T>::zero()};
    for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < nb;
         row += (int64_t)gridDim.x * blockDim.x) {
        T rv[BS], zv[BS];
#pragma unroll
        for (int i = 0; i < BS; ++i) rv[i] = r[(int64_t)BS * row + i];
        pc_apply<BS, T>(pc, dinv, row, rv, zv);
#pragma unroll
        for (int i = 0; i < BS; ++i) {
            z[(int64_t)BS * row + i] = zv[i];
            Acc<T>::add(acc[0], rv[i], zv[i]);
            Acc<T>::add(acc[1], rv[i], rv[i]);
        }
    }
    T tot[2];
    if (grid_total<2>(acc, pd, pf, ticket, tot)) {
        if (sizeof(T) == 8) {
            S->rho = (double)tot[0];
            S->rr = (double)tot[1];
            S->beta = 0.0;
        } else {
            const float rho_n = tot[0];
            S->beta32 = (keep_direction && S->rho32 != 0.f) ? rho_n / S->rho32 : 0.f;
            S->rho32 = rho_n;
            S->rr32 = tot[1];
            S->rmax32 = sqrtf(tot[1]);
            S->rmin32 = S->rmax32;
            S->need_update = 0;
            S->xmax_bits = 0u;
        }
    }
}

// ------------------------------------------------------------ BiCGSTAB kernels
// FP64: the reference stops ("Bicgstab devide by zero", FEMSolverClass.f90:2266,2295).
// FP32 inner iteration of the mixed solver: restart from the FP64 residual
// instead; the host gives up after repeated breakdowns without progress.
__device__ __forceinline__ void bicg_breakdown(KState *S, bool f64)
{
    if (f64) {
        S->status = PFG_E_BREAKDOWN;
        S->done = 1;
    } else {
        S->need_update = 1;
        S->breakdowns += 1;
    }
}

// y_new = A p_new, p_new = r + beta (p_old - c3 y_old) on the fly; c2 = r0.y_new;
// fin: alpha = c1 / c2  (FEMSolverClass.f90:2236-2248, 2296).
template <int BS, typename T>
__global__ void __launch_bounds__(kThreads)
    k_bicg_spmv1(SellView<T> A, const T *__restrict__ r, const T *__restrict__ r0, T *pA, T *pB, T *yA, T *yB,
                 KState *S, double *pd, float *pf, unsigned *ticket)
{
    if (S->done | S->need_update) return;
    const bool f64 = sizeof(T) == 8;
    const T beta = f64 ? (T)S->beta : (T)S->beta32;
    const T c3 = f64 ? (T)S->c3 : (T)S->c3_32;
    const int par = S->parity;
    const T *pold = par ? pB : pA;
    T *pnew = par ? pA : pB;
    const T *yold = par ? yB : yA;
    T *ynew = par ? yA : yB;
    typename Acc<T>::type acc[1] = {Acc<T>::zero()};
    PFG_SLICE_LOOP(A)
    {
        T y[BS];
        auto src = [&](int c, T(&xv)[BS]) {
#pragma unroll
            for (int i = 0; i < BS; ++i) {
                const int64_t j = (int64_t)BS * c + i;
                xv[i] = fma(beta, fma(-c3, __ldg(yold + j), __ldg(pold + j)), __ldg(r + j));
            }
        };
        sell_row_product<BS>(A, s, lane, src, y);
        const int64_t row = s * 32 + lane;
        if (row < A.nb) {
#pragma unroll
            for (int k = 0; k < BS; ++k) {
                const int64_t i = (int64_t)BS * row + k;
                const T pn = fma(beta, fma(-c3, yold[i], pold[i]), r[i]);
                pnew[i] = pn;
                ynew[i] = y[k];
                Acc<T>::add(acc[0], r0[i], y[k]);
            }
        }
    }
    T tot[1];
    if (grid_total<1>(acc, pd, pf, ticket, tot)) {
        const double c2 = (double)tot[0];
        if (c2 == 0.0 || !finite_d(c2)) {
            bicg_breakdown(S, f64);
        } else if (f64) {
            S->c2 = c2;
            S->alpha = S->c1 / c2;
        } else {
            S->c2_32 = tot[0];
            S->alpha32 = S->c1_32 / tot[0];
        }
    }
}

// v = A e, e = r - alpha y_new on the fly; ev = e.v, vv = v.v; fin: c3 = ev/vv
// (FEMSolverClass.f90:2254-2267).
template <int BS, typename T>
__global__ void __launch_bounds__(kThreads)
    k_bicg_spmv2(SellView<T> A, const T *__restrict__ r, const T *yA, const T *yB, T *__restrict__ e,
                 T *__restrict__ v, KState *S, double *pd, float *pf, unsigned *ticket)
{
    if (S->done | S->need_update) return;
    const bool f64 = sizeof(T) == 8;
    const T alpha = f64 ? (T)S->alpha : (T)S->alpha32;
    const T *ynew = S->parity ? yA : yB;
    typename Acc<T>::type acc[2] = {Acc<T>::zero(), Acc<T>::zero()};
    PFG_SLICE_LOOP(A)
    {
        T y[BS];
        auto src = [&](int c, T(&xv)[BS]) {
#pragma unroll
            for (int i = 0; i < BS; ++i) {
                const int64_t j = (int64_t)BS * c + i;
                xv[i] = fma(-alpha, __ldg(ynew + j), __ldg(r + j));
            }
        };
        sell_row_product<BS>(A, s, lane, src, y);
        const int64_t row = s * 32 + lane;
        if (row < A.nb) {
#pragma unroll
            for (int k = 0; k < BS; ++k) {
                const int64_t i = (int64_t)BS * row + k;
                const T ei = fma(-alpha, ynew[i], r[i]);
                e[i] = ei;
                v[i] = y[k];
                Acc<T>::add(acc[0], ei, y[k]);
                Acc<T>::add(acc[1], y[k], y[k]);
            }
        }
    }
    T tot[2];
    if (grid_total<2>(acc, pd, pf, ticket, tot)) {
        const double vv = (double)tot[1];
        if (vv == 0.0 || !finite_d(vv) || !finite_d((double)tot[0])) {
            bicg_breakdown(S, f64);
        } else if (f64) {
            S->ev = (double)tot[0];
            S->vv = vv;
            S->c3 = (double)tot[0] / vv;
        } else {
            S->c3_32 = tot[0] / tot[1];
        }
    }
}

// x += alpha p_new + c3 e; r = e - c3 v; rr = r.r; c1' = r0.r; stop rules and
// beta = c1' / (c2 c3) (FEMSolverClass.f90:2268-2296).
template <int BS, typename T>
__global__ void __launch_bounds__(kThreads)
    k_bicg_update(int64_t nb, T *__restrict__ x, T *__restrict__ r, const T *__restrict__ r0, const T *pA,
                  const T *pB, const T *__restrict__ e, const T *__restrict__ eh, const T *__restrict__ v, KState *S,
                  double *pd, float *pf, unsigned *ticket, int stop_rule, double er0, double tol, double delta,
                  int itrmax)
{
    if (S->done | S->need_update) return;
    const bool f64 = sizeof(T) == 8;
    const T alpha = f64 ? (T)S->alpha : (T)S->alpha32;
    const T c3 = f64 ? (T)S->c3 : (T)S->c3_32;
    const T *pnew = S->parity ? pA : pB;
    typename Acc<T>::type acc[2] = {Acc<T>::zero(), Acc<T>::zero()};
    const int64_t n = nb * BS;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const T ei = e[i];
        x[i] = x[i] + alpha * pnew[i] + c3 * eh[i];
        const T ri = fma(-c3, v[i], ei);
        r[i] = ri;
        Acc<T>::add(acc[0], ri, ri);
        Acc<T>::add(acc[1], r0[i], ri);
    }
    T tot[2];
    if (grid_total<2>(acc, pd, pf, ticket, tot)) {
        S->iter += 1;
        S->parity ^= 1;
        const double rr = (double)tot[0], c1n = (double)tot[1];
        if (!finite_d(rr) || !finite_d(c1n)) {
            if (f64) {
                S->status = PFG_E_NONFINITE;
                S->done = 1;
            } else {
                bicg_breakdown(S, false);  // FP32 overflow: restart from the FP64 residual
                S->poisoned = 1;
            }
            return;
        }
        if (f64) {
            S->rr = rr;
            if (S->iter == 1) S->rr1 = rr;
            bool stop;
            if (stop_rule == PFG_STOP_REFERENCE)
                stop = (sqrt(rr / S->rr1) < tol) || (sqrt(rr) < er0);
            else
                stop = sqrt(rr) <= tol * sqrt(S->bb);
            if (stop) {
                S->done = 1;
            } else {
                const double c2c3 = S->c2 * S->c3;
                if (c2c3 == 0.0) {
                    S->status = PFG_E_BREAKDOWN;
                    S->done = 1;
                } else {
                    S->beta = c1n / c2c3;
                    S->c1 = c1n;
                }
            }
        } else {
            const float rn = sqrtf((float)rr);
            S->rr32 = (float)rr;
            S->rmax32 = fmaxf(S->rmax32, rn);
            S->rmin32 = fminf(S->rmin32, rn);
            // replace on progress (delta), at the tolerance, or when the FP32
            // recursion diverges (1000x above its minimum since the last
            // replacement) before it can spoil the FP64 solution
            if ((double)rn < delta * (double)S->rmax32 || (double)rn <= tol * sqrt(S->bb) ||
                rn > 1000.f * S->rmin32) {
                S->need_update = 1;
            } else {
                const float c2c3 = S->c2_32 * S->c3_32;
                if (c2c3 == 0.f) {
                    bicg_breakdown(S, false);
                } else {
                    S->beta32 = (float)c1n / c2c3;
                    S->c1_32 = (float)c1n;
                    S->breakdowns = 0;
                }
            }
        }
        if (S->iter >= itrmax && !S->done) {
            S->status = PFG_W_NOT_CONVERGED;
            S->done = 1;
        }
    }
}

// Unfused BiCGSTAB passes: p = r + beta (p - c3 y) in place; e = r - alpha y;
// plain-gather SpMVs y = A ph (c2 = r0.y) and v = A eh (ev = e.v, vv).  With
// right preconditioning ph = M^-1 p and eh = M^-1 e (block Jacobi, one block
// row per thread) and x advances along ph and eh; without it ph = p, eh = e.
template <int BS, typename T>
__global__ void __launch_bounds__(kThreads)
    k_bicg_dir(int64_t nb, const T *__restrict__ r, T *__restrict__ p, const T *__restrict__ y, T *__restrict__ ph,
               const T *__restrict__ dinv, int pc, KState *S, bool track_max = false)
{
    if (S->done | S->need_update) return;
    const bool f64 = sizeof(T) == 8;
    const T beta = f64 ? (T)S->beta : (T)S->beta32;
    const T c3 = f64 ? (T)S->c3 : (T)S->c3_32;
    float vmax = 0.f;
    for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < nb;
         row += (int64_t)gridDim.x * blockDim.x) {
        T pv[BS], hv[BS];
#pragma unroll
        for (int i = 0; i < BS; ++i) {
            const int64_t j = (int64_t)BS * row + i;
            pv[i] = fma(beta, fma(-c3, y[j], p[j]), r[j]);
            p[j] = pv[i];
        }
        if (pc != PFG_PC_NONE) {
            pc_apply<BS, T>(pc, dinv, row, pv, hv);
#pragma unroll
            for (int i = 0; i < BS; ++i) ph[(int64_t)BS * row + i] = hv[i];
        }
        if (track_max)
#pragma unroll
            for (int i = 0; i < BS; ++i) vmax = fmaxf(vmax, fabsf((float)(pc != PFG_PC_NONE ? hv[i] : pv[i])));
    }
    if (track_max) track_abs_max(vmax, &S->xmax_bits);
}

template <int BS, typename T>
__global__ void __launch_bounds__(kThreads)
    k_bicg_e(int64_t nb, const T *__restrict__ r, const T *__restrict__ y, T *__restrict__ e, T *__restrict__ eh,
             const T *__restrict__ dinv, int pc, KState *S, bool track_max = false)
{
    if (S->done | S->need_update) return;
    const T alpha = sizeof(T) == 8 ? (T)S->alpha : (T)S->alpha32;
    float vmax = 0.f;
    for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < nb;
         row += (int64_t)gridDim.x * blockDim.x) {
        T ev[BS], hv[BS];
#pragma unroll
        for (int i = 0; i < BS; ++i) {
            const int64_t j = (int64_t)BS * row + i;
            ev[i] = fma(-alpha, y[j], r[j]);
            e[j] = ev[i];
        }
        if (pc != PFG_PC_NONE) {
            pc_apply<BS, T>(pc, dinv, row, ev, hv);
#pragma unroll
            for (int i = 0; i < BS; ++i) eh[(int64_t)BS * row + i] = hv[i];
        }
        if (track_max)
#pragma unroll
            for (int i = 0; i < BS; ++i) vmax = fmaxf(vmax, fabsf((float)(pc != PFG_PC_NONE ? hv[i] : ev[i])));
    }
    if (track_max) track_abs_max(vmax, &S->xmax_bits);
}

template <int BS, typename T>
__global__ void __launch_bounds__(kThreads)
    k_bicg_spmv1_u(SellView<T> A, const T *__restrict__ p, const T *__restrict__ r0, T *__restrict__ y, KState *S,
                   double *pd, float *pf, unsigned *ticket)
{
    if (S->done | S->need_update) return;
    const bool f64 = sizeof(T) == 8;
    typename Acc<T>::type acc[1] = {Acc<T>::zero()};
    PFG_SLICE_LOOP(A)
    {
        T yv[BS];
        auto src = [&](int c, T(&xv)[BS]) {
#pragma unroll
            for (int i = 0; i < BS; ++i) xv[i] = __ldg(p + (int64_t)BS * c + i);
        };
        sell_row_product<BS>(A, s, lane, src, yv);
        const int64_t row = s * 32 + lane;
        if (row < A.nb) {
#pragma unroll
            for (int k = 0; k < BS; ++k) {
                const int64_t i = (int64_t)BS * row + k;
                y[i] = yv[k];
                Acc<T>::add(acc[0], r0[i], yv[k]);
            }
        }
    }
    T tot[1];
    if (grid_total<1>(acc, pd, pf, ticket, tot)) {
        const double c2 = (double)tot[0];
        if (c2 == 0.0 || !finite_d(c2)) {
            bicg_breakdown(S, f64);
        } else if (f64) {
            S->c2 = c2;
            S->alpha = S->c1 / c2;
        } else {
            S->c2_32 = tot[0];
            S->alpha32 = S->c1_32 / tot[0];
        }
    }
}

template <int BS, typename T>
__global__ void __launch_bounds__(kThreads)
    k_bicg_spmv2_u(SellView<T> A, const T *__restrict__ eh, const T *__restrict__ e, T *__restrict__ v, KState *S,
                   double *pd, float *pf, unsigned *ticket)
{
    if (S->done | S->need_update) return;
    const bool f64 = sizeof(T) == 8;
    typename Acc<T>::type acc[2] = {Acc<T>::zero(), Acc<T>::zero()};
    PFG_SLICE_LOOP(A)
    {
        T yv[BS];
        auto src = [&](int c, T(&xv)[BS]) {
#pragma unroll
            for (int i = 0; i < BS; ++i) xv[i] = __ldg(eh + (int64_t)BS * c + i);
        };
        sell_row_product<BS>(A, s, lane, src, yv);
        const int64_t row = s * 32 + lane;
        if (row < A.nb) {
#pragma unroll
            for (int k = 0; k < BS; ++k) {
                const int64_t i = (int64_t)BS * row + k;
                v[i] = yv[k];
                Acc<T>::add(acc[0], e[i], yv[k]);
                Acc<T>::add(acc[1], yv[k], yv[k]);
            }
        }
    }
    T tot[2];
    if (grid_total<2>(acc, pd, pf, ticket, tot)) {
        const double vv = (double)tot[1];
        if (vv == 0.0 || !finite_d(vv) || !finite_d((double)tot[0])) {
            bicg_breakdown(S, f64);
        } else if (f64) {
            S->ev = (double)tot[0];
            S->vv = vv;
            S->c3 = (double)tot[0] / vv;
        } else {
            S->c3_32 = tot[0] / tot[1];
        }
    }
}

// BiCGSTAB (re)start from r: r0 = r (first start only), c1 = r0.r, beta = 0.
// keep_direction != 0 (mixed replacement): keep p, y and r0, beta = c1'/(c2 c3).
template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_bicg_restart(int64_t n, const T *__restrict__ r, T *__restrict__ r0, KState *S, double *pd, float *pf,
                   unsigned *ticket, int set_r0, int keep_direction)
{
    typename Acc<T>::type acc[3] = {Acc<T>::zero(), Acc<T>::zero(), Acc<T>::zero()};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const T ri = r[i];
        if (set_r0) r0[i] = ri;
        const T r0i = set_r0 ? ri : r0[i];
        Acc<T>::add(acc[0], r0i, ri);
        Acc<T>::add(acc[1], ri, ri);
        Acc<T>::add(acc[2], r0i, r0i);
    }
    T tot[3];
    if (grid_total<3>(acc, pd, pf, ticket, tot)) {
        if (sizeof(T) == 8) {
            S->c1 = (double)tot[0];
            S->rr = (double)tot[1];
            S->beta = 0.0;
            S->c3 = 0.0;
        } else {
            const float c1n = tot[0];
            const float c2c3 = S->c2_32 * S->c3_32;
            S->beta32 = (keep_direction && c2c3 != 0.f) ? c1n / c2c3 : 0.f;
            if (!keep_direction) S->c3_32 = 0.f;
            S->c1_32 = c1n;
            S->rr32 = tot[1];
            S->r0r0_32 = tot[2];
            S->rmax32 = sqrtf(tot[1]);
            S->rmin32 = S->rmax32;
            S->need_update = 0;
            S->xmax_bits = 0u;
        }
    }
}

// ------------------------------------------- symmetric storage (FP32 inner)
// The FP32 inner iterations of a symmetric matrix can read only its upper
// half: each stored block (i, j), j >= i, is applied as A_ij x_j to row i and,
// for j > i, as A_ij^T x_i to row j.  The transposed products are scattered
// with 16-byte vector reductions (red.global.add.v4.f32) into a 4-per-node
// accumulator that stays in L2; half the matrix bytes for 1 + (upper blocks)
// reductions per row.  The summation order of a row's contributions is that
// of the reductions, so FP32 inner results vary in their last bits from run
// to run (the FP64 residual and the stop test are computed as always).  This
// form serves the mixed CG, whose iteration count does not follow those bits
// (1841-1842 iterations on the 3.09M-DOF system); the mixed BiCGSTAB, whose
// count does, uses the reproducible fixed-point form below.
// (no "memory" clobber: the kernels that use it never read the accumulator, so
// the compiler may keep issuing the next slots' loads across a reduction)
__device__ __forceinline__ void red_add_v4(float *a, float x, float y, float z)
{
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(a), "f"(x), "f"(y), "f"(z), "f"(0.f));
}

// y4 += A x from the upper half U (y4: 4 floats per block row, zero on entry)
__global__ void __launch_bounds__(kThreads)
    k_spmv_sym(SellView<float> U, const float *__restrict__ x, float *__restrict__ y4, const KState *S)
{
    if (S && (S->done | S->need_update)) return;
    PFG_SLICE_LOOP(U)
    {
        const int64_t row = s * 32 + lane;
        const bool live = row < U.nb;
        float xi[3];
#pragma unroll
        for (int t = 0; t < 3; ++t) xi[t] = live ? __ldg(x + 3 * row + t) : 0.f;
        const int64_t b0 = U.sptr[s];
        const int w = (int)(U.sptr[s + 1] - b0);
        const int *cp = U.col + b0 * 32 + lane;
        const float *vp = U.val + b0 * 32 * 9 + lane;
        float acc[3] = {0.f, 0.f, 0.f};
#pragma unroll 2
        for (int k = 0; k < w; ++k) {
            const int c = ld_stream(cp + (int64_t)k * 32);
            float a[9];
#pragma unroll
            for (int e = 0; e < 9; ++e) a[e] = ld_stream(vp + ((int64_t)k * 9 + e) * 32);
            float xj[3];
#pragma unroll
            for (int t = 0; t < 3; ++t) xj[t] = __ldg(x + 3 * (int64_t)c + t);
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int t = 0; t < 3; ++t) acc[r] = fmaf(a[3 * r + t], xj[t], acc[r]);
            if (live && c != row) {
                float tv[3];
#pragma unroll
                for (int t = 0; t < 3; ++t) tv[t] = fmaf(a[t], xi[0], fmaf(a[3 + t], xi[1], a[6 + t] * xi[2]));
                red_add_v4(y4 + 4 * (int64_t)c, tv[0], tv[1], tv[2]);
            }
        }
        if (live) red_add_v4(y4 + 4 * row, acc[0], acc[1], acc[2]);
    }
}

// CG form: q4 += A p from the upper half and <p, A p> in the same pass,
// fin: alpha = rho / <p, Ap>.  With acc_i = sum over the row's stored blocks
// (j >= i) of A_ij p_j, symmetry gives <p, Ap> = sum_i (2 p_i.acc_i - p_i^T A_ii p_i),
// so the reduction does not wait for the scattered transposes.
template <int UNR, int MINB>
__global__ void __launch_bounds__(kThreads, MINB)
    k_cg_spmv_sym_t(SellView<float> U, const float *__restrict__ p, float *__restrict__ q4, KState *S, double *pd,
                    float *pf, unsigned *ticket)
{
    if (S->done | S->need_update) return;
    Comp32 dot[1] = {Comp32{0.f, 0.f}};
    PFG_SLICE_LOOP(U)
    {
        const int64_t row = s * 32 + lane;
        const bool live = row < U.nb;
        float xi[3];
#pragma unroll
        for (int t = 0; t < 3; ++t) xi[t] = live ? __ldg(p + 3 * row + t) : 0.f;
        const int64_t b0 = U.sptr[s];
        const int w = (int)(U.sptr[s + 1] - b0);
        const int *cp = U.col + b0 * 32 + lane;
        const float *vp = U.val + b0 * 32 * 9 + lane;
        float acc[3] = {0.f, 0.f, 0.f}, dg[3] = {0.f, 0.f, 0.f};
#pragma unroll UNR
        for (int k = 0; k < w; ++k) {
            const int c = ld_stream(cp + (int64_t)k * 32);
            float a[9];
#pragma unroll
            for (int e = 0; e < 9; ++e) a[e] = ld_stream(vp + ((int64_t)k * 9 + e) * 32);
            float xj[3];
#pragma unroll
            for (int t = 0; t < 3; ++t) xj[t] = __ldg(p + 3 * (int64_t)c + t);
            float bx[3];
#pragma unroll
            for (int r = 0; r < 3; ++r) bx[r] = fmaf(a[3 * r], xj[0], fmaf(a[3 * r + 1], xj[1], a[3 * r + 2] * xj[2]));
#pragma unroll
            for (int r = 0; r < 3; ++r) acc[r] += bx[r];
            if (c == row) {  // the diagonal block (and zero padding)
#pragma unroll
                for (int r = 0; r < 3; ++r) dg[r] += bx[r];
            } else if (live) {
                float tv[3];
#pragma unroll
                for (int t = 0; t < 3; ++t) tv[t] = fmaf(a[t], xi[0], fmaf(a[3 + t], xi[1], a[6 + t] * xi[2]));
                red_add_v4(q4 + 4 * (int64_t)c, tv[0], tv[1], tv[2]);
            }
        }
        if (live) {
            red_add_v4(q4 + 4 * row, acc[0], acc[1], acc[2]);
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                comp_add_prod(dot[0], 2.f * xi[r], acc[r]);
                comp_add_prod(dot[0], -xi[r], dg[r]);
            }
        }
    }
    float tot[1];
    if (grid_total<1>(dot, pd, pf, ticket, tot)) {
        const double pq = (double)tot[0];
        if (!(pq > 0.0) || !finite_d(pq)) {
            S->status = PFG_E_BREAKDOWN;
            S->done = 1;
        } else {
            S->alpha32 = (float)(S->rho32 / tot[0]);
        }
    }
}

// Register-pipelined form (loads of two slots per loop step in flight,
// 63 registers, 4 CTAs per SM): 0.1015-0.1036 ms per launch at 3.09M DOF, kept
// as a profiling reference for the bulk-staged form below that the solves use.
// (One slot at 5 CTAs: 0.1036 ms; three slots at 3 CTAs: 0.107 ms; an L2
// evict-first policy on its loads: 0.117 ms.)

// Bulk-staged form of the CG product, the one the solves use.  The column
// and value planes of a warp's slices are streamed into a ring of NST
// shared-memory stages of CH slots each by the bulk copy engine
// (cp.async.bulk, completion counted on one mbarrier per stage), so the bytes
// in flight no longer depend on how many loads the warp's registers can hold;
// the lanes read the staged planes (consecutive lanes, consecutive words: no
// bank conflicts) and gather p as above.  A slot of a slice is 32 columns
// (128 B) and 9 x 32 values (1152 B), contiguous in the sliced layout, so a
// stage is two copies.  The copies carry an L2 evict-first policy: the
// streamed matrix (0.6 GB at 3.09M DOF) then leaves p and the accumulator
// (29 MB) resident in L2 for the gathers and the transposed reductions.  A
// stage that does not complete within the wait limit stops the warp with
// PFG_E_INTERNAL (after waiting, again bounded, for its copies in flight).
// Measured per launch at 3.09M DOF (GB300): CH 2, NST 4 (82 KB of stages per
// CTA, 2 CTAs per SM) 0.0959 ms; CH 3, NST 3: 0.098 ms; CH 4, NST 2: 0.100 ms;
// CH 2, NST 5: 0.101 ms; CH 1, NST 6: 0.104 ms; CH 2, NST 4 without the L2
// policy: 0.102 ms.
template <int CH, int NST>
struct SymBulk {
    static constexpr int kColB = CH * 32 * 4;
    static constexpr int kValB = CH * 32 * 9 * 4;
    static constexpr int kStageB = kColB + kValB;
    static constexpr int kBarB = ((kWarps * NST * 8 + 127) / 128) * 128;
    static constexpr int kSmem = kBarB + kWarps * NST * kStageB;
};

// One warp's ring of stages over the slices w0, w0 + nw, ... of U (empty
// slices skipped).  Chunks are consumed in the order they are produced:
// chunk c sits in stage c % NST, and its barrier completes phase c / NST.
template <int CH, int NST, bool EVF>
struct SliceStager {
    using L = SymBulk<CH, NST>;
    SellView<float> U;
    uint64_t *bar;
    unsigned char *stages;
    int64_t nw, ps, pb0;
    int pw, pk, lane;
    unsigned pidx, cidx;
    uint64_t pol;

    __device__ void init(unsigned char *dsm, const SellView<float> &u, int64_t w0, int64_t nw_)
    {
        U = u;
        lane = threadIdx.x & 31;
        const int wid = threadIdx.x >> 5;
        bar = reinterpret_cast<uint64_t *>(dsm) + wid * NST;
        stages = dsm + L::kBarB + (size_t)wid * NST * L::kStageB;
        if (lane == 0) {
#pragma unroll
            for (int i = 0; i < NST; ++i) mbar_init(bar + i, 1);
            fence_proxy_async_smem();
        }
        __syncwarp();
        pol = EVF ? l2_evict_first_policy() : 0ull;
        nw = nw_;
        ps = w0;
        pidx = cidx = 0;
        seek();
#pragma unroll
        for (int i = 0; i < NST; ++i) produce();
    }
    __device__ void seek()  // first non-empty slice at or after ps
    {
        for (; ps < U.ns; ps += nw) {
            pb0 = U.sptr[ps];
            pw = (int)(U.sptr[ps + 1] - pb0);
            if (pw > 0) break;
        }
        pk = 0;
    }
    __device__ void produce()
    {
        if (ps >= U.ns) return;
        const int st = (int)(pidx % NST);
        const int nsl = min(CH, pw - pk);
        if (lane == 0) {
            unsigned char *dst = stages + st * L::kStageB;
            const int *cs = U.col + (pb0 + pk) * 32;
            const float *vs = U.val + (pb0 + pk) * 288;
            mbar_arrive_expect_tx(bar + st, (unsigned)nsl * 1280u);
            if (EVF) {
                bulk_g2s_hint(dst, cs, (unsigned)nsl * 128u, bar + st, pol);
                bulk_g2s_hint(dst + L::kColB, vs, (unsigned)nsl * 1152u, bar + st, pol);
            } else {
                bulk_g2s(dst, cs, (unsigned)nsl * 128u, bar + st);
                bulk_g2s(dst + L::kColB, vs, (unsigned)nsl * 1152u, bar + st);
            }
        }
        ++pidx;
        pk += nsl;
        if (pk >= pw) {
            ps += nw;
            seek();
        }
    }
    // Waits for the next chunk (false: it did not complete within the limit).
    __device__ bool wait(const int *&cols, const float *&vals)
    {
        const int st = (int)(cidx % NST);
        if (!__all_sync(0xffffffffu, mbar_wait(bar + st, (cidx / NST) & 1u))) return false;
        cols = reinterpret_cast<const int *>(stages + st * L::kStageB);
        vals = reinterpret_cast<const float *>(stages + st * L::kStageB + L::kColB);
        return true;
    }
    // Every lane has read the chunk: refill its stage with the next one.
    __device__ void release()
    {
        __syncwarp();
        if (lane == 0) fence_proxy_async_smem();
        produce();
        ++cidx;
    }
    // After a failed wait: wait (bounded) for the copies still in flight.
    __device__ void drain()
    {
        for (; cidx != pidx; ++cidx) (void)mbar_wait(bar + cidx % NST, (cidx / NST) & 1u);
    }
};

// FUSE: the direction update p = z + beta p rides in the product (as
// k_cg_spmv does for the full copy): p_old is pA or pB by S->parity, every
// gather forms z_j + beta p_old,j (the same FP32 fma as k_cg_dir, so the same
// bits) and the lane that owns a row stores its p_new in the other buffer;
// without FUSE, p = pA and z, pB are unused.
template <int CH, int NST, bool EVF, bool FUSE>
__global__ void __launch_bounds__(kThreads)
    k_cg_spmv_symb(SellView<float> U, const float *__restrict__ z, const float *pA, float *pB,
                   float *__restrict__ q4, KState *S, double *pd, float *pf, unsigned *ticket)
{
    extern __shared__ __align__(128) unsigned char dsm[];
    if (S->done | S->need_update) return;
    const float beta = FUSE ? S->beta32 : 0.f;
    const int par = FUSE ? S->parity : 0;
    const float *p = (FUSE && par) ? pB : pA;                    // p (FUSE: p_old)
    float *pnew = FUSE ? (par ? const_cast<float *>(pA) : pB) : nullptr;
    auto pval = [&](int64_t i) { return FUSE ? fmaf(beta, __ldg(p + i), __ldg(z + i)) : __ldg(p + i); };
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    SliceStager<CH, NST, EVF> sg;
    sg.init(dsm, U, w0, nw);

    Comp32 dot[1] = {Comp32{0.f, 0.f}};
    bool ok = true;
    for (int64_t s = w0; ok && s < U.ns; s += nw) {
        const int64_t b0 = U.sptr[s];
        const int w = (int)(U.sptr[s + 1] - b0);
        if (w <= 0) continue;
        const int64_t row = s * 32 + lane;
        const bool live = row < U.nb;
        float xi[3];
#pragma unroll
        for (int t = 0; t < 3; ++t) xi[t] = live ? pval(3 * row + t) : 0.f;
        if (FUSE && live)
#pragma unroll
            for (int t = 0; t < 3; ++t) pnew[3 * row + t] = xi[t];
        float acc[3] = {0.f, 0.f, 0.f}, dg[3] = {0.f, 0.f, 0.f};
        for (int k = 0; k < w; k += CH) {
            const int *cs;
            const float *vs;
            if (!sg.wait(cs, vs)) {
                ok = false;
                break;
            }
            const int nsl = min(CH, w - k);
            int c[CH];
            float xj[CH][3];
#pragma unroll
            for (int j = 0; j < CH; ++j)
                if (j < nsl) {
                    c[j] = cs[j * 32 + lane];
#pragma unroll
                    for (int t = 0; t < 3; ++t) xj[j][t] = pval(3 * (int64_t)c[j] + t);
                }
#pragma unroll
            for (int j = 0; j < CH; ++j)
                if (j < nsl) {
                    float a[9];
#pragma unroll
                    for (int e = 0; e < 9; ++e) a[e] = vs[(j * 9 + e) * 32 + lane];
                    float bx[3];
#pragma unroll
                    for (int r = 0; r < 3; ++r)
                        bx[r] = fmaf(a[3 * r], xj[j][0], fmaf(a[3 * r + 1], xj[j][1], a[3 * r + 2] * xj[j][2]));
#pragma unroll
                    for (int r = 0; r < 3; ++r) acc[r] += bx[r];
                    if (c[j] == row) {
#pragma unroll
                        for (int r = 0; r < 3; ++r) dg[r] += bx[r];
                    } else if (live) {
                        float tv[3];
#pragma unroll
                        for (int t = 0; t < 3; ++t) tv[t] = fmaf(a[t], xi[0], fmaf(a[3 + t], xi[1], a[6 + t] * xi[2]));
                        red_add_v4(q4 + 4 * (int64_t)c[j], tv[0], tv[1], tv[2]);
                    }
                }
            sg.release();
        }
        if (ok && live) {
            red_add_v4(q4 + 4 * row, acc[0], acc[1], acc[2]);
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                comp_add_prod(dot[0], 2.f * xi[r], acc[r]);
                comp_add_prod(dot[0], -xi[r], dg[r]);
            }
        }
    }
    if (!ok) {
        if (lane == 0) {
            S->status = PFG_E_INTERNAL;
            S->done = 1;
        }
        sg.drain();
    }
    float tot[1];
    if (grid_total<1>(dot, pd, pf, ticket, tot) && !S->done) {
        const double pq = (double)tot[0];
        if (!(pq > 0.0) || !finite_d(pq)) {
            S->status = PFG_E_BREAKDOWN;
            S->done = 1;
        } else {
            S->alpha32 = (float)(S->rho32 / tot[0]);
        }
    }
}

constexpr int kSymbSlots = 2, kSymbStages = 4;
using SymbLayout = SymBulk<kSymbSlots, kSymbStages>;
#define k_cg_spmv_sym k_cg_spmv_symb<kSymbSlots, kSymbStages, true, false>
#define k_cg_spmv_sym_fused k_cg_spmv_symb<kSymbSlots, kSymbStages, true, true>

// Grid of a bulk-staged kernel: its resident CTAs with `smem` bytes of
// dynamic shared memory each, capped by the slices.  The first call per
// kernel raises the kernel's dynamic shared-memory limit, so it is made before
// any graph capture.
template <typename K>
static int staged_grid(K kern, int smem, int64_t ns)
{
    static std::mutex mu;
    static std::unordered_map<const void *, int> cache;
    int per_sm = 0;
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find((const void *)kern);
        if (it == cache.end()) {
            PFG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
            PFG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem));
            cache[(const void *)kern] = per_sm;
        } else {
            per_sm = it->second;
        }
    }
    const int64_t want = (ns + kWarps - 1) / kWarps;
    return (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)std::max(per_sm, 1) * sm_count()));
}

// fuse: z, pA, pB as k_cg_spmv_symb's FUSE form; else p = pA
static void launch_cg_spmv_sym(bool fuse, const SellView<float> &U, const float *z, const float *pA, float *pB,
                               float *q4, KState *S, double *pd, float *pf, unsigned *tk, cudaStream_t st)
{
    if (fuse)
        k_cg_spmv_sym_fused<<<staged_grid(k_cg_spmv_sym_fused, SymbLayout::kSmem, U.ns), kThreads, SymbLayout::kSmem,
                              st>>>(U, z, pA, pB, q4, S, pd, pf, tk);
    else
        k_cg_spmv_sym<<<staged_grid(k_cg_spmv_sym, SymbLayout::kSmem, U.ns), kThreads, SymbLayout::kSmem, st>>>(
            U, nullptr, pA, nullptr, q4, S, pd, pf, tk);
}

// Reproducible form of the symmetric product (the BiCGSTAB inner iterations,
// whose iteration count follows every rounding difference).  Each row's own
// stored blocks are summed in FP32 by the lane that owns the row, in slot
// order, and stored to y; the scattered transposes are converted to 64-bit
// fixed point and added with integer reductions, which give the same total in
// any order.  The quantum is a power of two chosen per product from a bound on
// every partial sum, |sum| <= (max row sum of |A|) * max|x| < 2^61 / scale,
// so no accumulator overflows; x's maximum comes from the kernel that wrote
// x (KState::xmax_bits).  Terms smaller than the quantum (2^-61 of the bound)
// are rounded to it.  k_symfx_finish adds the two parts in a fixed order.
// Measured on the 3.09M-DOF system: 0.113 ms per product against 0.105 ms for
// the FP32 vector reductions (an ordered gather of the transposes through a
// transposed index, also reproducible, took 0.14-0.26 ms: latency-bound).
__device__ __forceinline__ void red_add_u64(unsigned long long *a, long long v)
{
    asm volatile("red.global.add.u64 [%0], %1;" ::"l"(a), "l"(v));
}

// Exponent k of the fixed-point scale 2^k for a product whose partial sums are
// bounded by rowsum * max|x|: bound * 2^k < 2^61.
__device__ __forceinline__ int symfx_exponent(float rowsum, unsigned xmax_bits)
{
    const float bound = rowsum * __uint_as_float(xmax_bits);
    if (!(bound > 0.f)) return 126;
    if (!isfinite(bound)) return -67;
    return min(126, 61 - (ilogbf(bound) + 1));
}

// y = (own stored blocks) x; acc64[t nb + c] += fixed-point transposes (three
// planes: a warp's reductions of one component cover consecutive words; the
// three components of a row in one sector made the reductions twice as slow)
template <int UNR, int MINB>
__global__ void __launch_bounds__(kThreads, MINB)
    k_spmv_symfx_t(SellView<float> U, const float *__restrict__ x, float *__restrict__ y,
                   unsigned long long *__restrict__ acc64, float rowsum, const KState *S)
{
    if (S->done | S->need_update) return;
    const float scale = exp2f((float)symfx_exponent(rowsum, S->xmax_bits));
    PFG_SLICE_LOOP(U)
    {
        const int64_t row = s * 32 + lane;
        const bool live = row < U.nb;
        float xi[3];
#pragma unroll
        for (int t = 0; t < 3; ++t) xi[t] = live ? __ldg(x + 3 * row + t) : 0.f;
        const int64_t b0 = U.sptr[s];
        const int w = (int)(U.sptr[s + 1] - b0);
        const int *cp = U.col + b0 * 32 + lane;
        const float *vp = U.val + b0 * 32 * 9 + lane;
        float acc[3] = {0.f, 0.f, 0.f};
#pragma unroll UNR
        for (int k = 0; k < w; ++k) {
            const int c = ld_stream(cp + (int64_t)k * 32);
            float a[9];
#pragma unroll
            for (int e = 0; e < 9; ++e) a[e] = ld_stream(vp + ((int64_t)k * 9 + e) * 32);
            float xj[3];
#pragma unroll
            for (int t = 0; t < 3; ++t) xj[t] = __ldg(x + 3 * (int64_t)c + t);
#pragma unroll
            for (int r = 0; r < 3; ++r) acc[r] += fmaf(a[3 * r], xj[0], fmaf(a[3 * r + 1], xj[1], a[3 * r + 2] * xj[2]));
            if (live && c != row) {
#pragma unroll
                for (int t = 0; t < 3; ++t) {
                    const float tv = fmaf(a[t], xi[0], fmaf(a[3 + t], xi[1], a[6 + t] * xi[2]));
                    red_add_u64(acc64 + (int64_t)t * U.nb + c, __float2ll_rn(tv * scale));
                }
            }
        }
        if (live)
#pragma unroll
            for (int t = 0; t < 3; ++t) y[3 * row + t] = acc[t];
    }
}
// one slot per loop step at 5 CTAs per SM: 0.113 ms per launch at 3.09M DOF
// (two slots at 4 CTAs: 0.127 ms)

// The same product with the matrix planes staged in shared memory by bulk
// copies (SliceStager, as k_cg_spmv_symb).  Each lane sums its row's own
// blocks in slot order, as above, so the results are the same bits.
template <int CH, int NST, bool EVF>
__global__ void __launch_bounds__(kThreads)
    k_spmv_symfxb(SellView<float> U, const float *__restrict__ x, float *__restrict__ y,
                  unsigned long long *__restrict__ acc64, float rowsum, KState *S)
{
    extern __shared__ __align__(128) unsigned char dsm[];
    if (S->done | S->need_update) return;
    const float scale = exp2f((float)symfx_exponent(rowsum, S->xmax_bits));
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    SliceStager<CH, NST, EVF> sg;
    sg.init(dsm, U, w0, nw);
    bool ok = true;
    for (int64_t s = w0; ok && s < U.ns; s += nw) {
        const int64_t b0 = U.sptr[s];
        const int w = (int)(U.sptr[s + 1] - b0);
        if (w <= 0) continue;
        const int64_t row = s * 32 + lane;
        const bool live = row < U.nb;
        float xi[3];
#pragma unroll
        for (int t = 0; t < 3; ++t) xi[t] = live ? __ldg(x + 3 * row + t) : 0.f;
        float acc[3] = {0.f, 0.f, 0.f};
        for (int k = 0; k < w; k += CH) {
            const int *cs;
            const float *vs;
            if (!sg.wait(cs, vs)) {
                ok = false;
                break;
            }
            const int nsl = min(CH, w - k);
            int c[CH];
            float xj[CH][3];
#pragma unroll
            for (int j = 0; j < CH; ++j)
                if (j < nsl) {
                    c[j] = cs[j * 32 + lane];
#pragma unroll
                    for (int t = 0; t < 3; ++t) xj[j][t] = __ldg(x + 3 * (int64_t)c[j] + t);
                }
#pragma unroll
            for (int j = 0; j < CH; ++j)
                if (j < nsl) {
                    float a[9];
#pragma unroll
                    for (int e = 0; e < 9; ++e) a[e] = vs[(j * 9 + e) * 32 + lane];
#pragma unroll
                    for (int r = 0; r < 3; ++r)
                        acc[r] += fmaf(a[3 * r], xj[j][0], fmaf(a[3 * r + 1], xj[j][1], a[3 * r + 2] * xj[j][2]));
                    if (live && c[j] != row) {
#pragma unroll
                        for (int t = 0; t < 3; ++t) {
                            const float tv = fmaf(a[t], xi[0], fmaf(a[3 + t], xi[1], a[6 + t] * xi[2]));
                            red_add_u64(acc64 + (int64_t)t * U.nb + c[j], __float2ll_rn(tv * scale));
                        }
                    }
                }
            sg.release();
        }
        if (ok && live)
#pragma unroll
            for (int t = 0; t < 3; ++t) y[3 * row + t] = acc[t];
    }
    if (!ok) {
        if (lane == 0) {
            S->status = PFG_E_INTERNAL;
            S->done = 1;
        }
        sg.drain();
    }
}
#define k_spmv_symfx k_spmv_symfxb<kSymbSlots, kSymbStages, true>

static void launch_spmv_symfx(const SellView<float> &U, const float *x, float *y, unsigned long long *acc64,
                              float rowsum, KState *S, cudaStream_t st)
{
    k_spmv_symfx<<<staged_grid(k_spmv_symfx, SymbLayout::kSmem, U.ns), kThreads, SymbLayout::kSmem, st>>>(
        U, x, y, acc64, rowsum, S);
}

// y += acc64 / scale (acc64 = 0 for the next product), then the dot products
// and scalar updates of the BiCGSTAB products:
//   mode 1:  <a, y>          -> c2 = <r0, y>, alpha = c1 / c2
//   mode 2:  <a, y>, <y, y>  -> c3 = <e, v> / <v, v>
// and xmax_bits = 0 for the next vector's maximum.  A thread per scalar entry
// with four entries in flight (a thread per block row with its three entries
// in turn was latency-bound: 88 us against 19 us at 3.09M DOF).
__global__ void __launch_bounds__(kThreads)
    k_symfx_finish(int64_t nb, float *__restrict__ y, unsigned long long *__restrict__ acc64,
                   const float *__restrict__ a, float rowsum, int mode, KState *S, double *pd, float *pf,
                   unsigned *ticket)
{
    if (S->done | S->need_update) return;
    const float inv = exp2f((float)-symfx_exponent(rowsum, S->xmax_bits));
    Comp32 acc[2] = {Comp32{0.f, 0.f}, Comp32{0.f, 0.f}};
    const int64_t n = 3 * nb;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i0 < n; i0 += 4 * stride) {
        long long qv[4];
        float yv[4], av[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int64_t i = i0 + u * stride;
            if (i < n) {
                const int64_t row = i / 3;
                qv[u] = (long long)acc64[(i - 3 * row) * nb + row];
                yv[u] = y[i];
                av[u] = a[i];
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int64_t i = i0 + u * stride;
            if (i < n) {
                const int64_t row = i / 3;
                acc64[(i - 3 * row) * nb + row] = 0ull;
                const float v = yv[u] + (float)qv[u] * inv;
                y[i] = v;
                comp_add_prod(acc[0], av[u], v);
                if (mode == 2) comp_add_prod(acc[1], v, v);
            }
        }
    }
    float tot[2];
    if (grid_total<2>(acc, pd, pf, ticket, tot)) {
        S->xmax_bits = 0u;  // every CTA read it at its start
        if (mode == 1) {
            const double c2 = (double)tot[0];
            if (c2 == 0.0 || !finite_d(c2)) {
                bicg_breakdown(S, false);
            } else {
                S->c2_32 = tot[0];
                S->alpha32 = S->c1_32 / tot[0];
            }
        } else {
            const double vv = (double)tot[1];
            if (vv == 0.0 || !finite_d(vv) || !finite_d((double)tot[0]))
                bicg_breakdown(S, false);
            else
                S->c3_32 = tot[0] / tot[1];
        }
    }
}

// --------------------------------------------------- mixed-precision plumbing
// x64 += x32, x32 = 0 (fold the FP32 correction into the FP64 solution).
__global__ void k_fold(int64_t n, double *__restrict__ x64, float *__restrict__ x32)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x64[i] += (double)x32[i];
        x32[i] = 0.f;
    }
}

// r32 = (float) r64 after the FP64 residual; decides convergence on it.
__global__ void k_replace(int64_t n, const double *__restrict__ r64, float *__restrict__ r32, KState *S,
                          double tol)
{
    const bool conv = sqrt(S->true_rr) <= tol * sqrt(S->bb);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        r32[i] = (float)r64[i];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        S->replacements += 1;
        if (conv) S->done = 1;
    }
}

// ------------------------------------------------------------------- host side
Krylov::Krylov()
{
    PFG_CUDA(cudaMallocHost((void **)&host_state_, sizeof(KState)));
    memset(host_state_, 0, sizeof(KState));
}

Krylov::~Krylov()
{
    if (graph_) cudaGraphExecDestroy(graph_);
    if (host_state_) cudaFreeHost(host_state_);
}

const Ilu0 &Krylov::ilu_factor(const DevMatrix &A, bool sorted, cudaStream_t st)
{
    if (!ilu_) ilu_.reset(new Ilu0());
    ilu_->factor(A, sorted, st);
    return *ilu_;
}

const Ilu0 *Krylov::ilu_held() const { return ilu_ && ilu_->ready() ? ilu_.get() : nullptr; }

void Krylov::ilu_reset()
{
    if (ilu_) ilu_->reset();
}

template <int BS, typename T>
static void launch_spmv(const DevMatrix &A, BsrView<T> v, const T *x, T *y, cudaStream_t st)
{
    if (A.nb == 0) return;
    k_spmv<BS, T><<<Krylov::row_grid(A.nb), kThreads, 0, st>>>(v, x, y);
    PFG_CUDA(cudaGetLastError());
}

void Krylov::spmv64(const DevMatrix &A, const double *x, double *y, cudaStream_t st)
{
    if (A.bs == 3)
        launch_spmv<3, double>(A, A.view<double>(), x, y, st);
    else
        launch_spmv<1, double>(A, A.view<double>(), x, y, st);
}

void Krylov::spmv64_sliced(DevMatrix &A, const double *x, double *y, cudaStream_t st)
{
    if (A.nb == 0) return;
    build_sell(A, true, false, st);
    if (A.bs == 3)
        k_spmv_sell<3, double><<<resident_grid(k_spmv_sell<3, double>, A.ns), kThreads, 0, st>>>(A.sell<double>(), x,
                                                                                                 y);
    else
        k_spmv_sell<1, double><<<resident_grid(k_spmv_sell<1, double>, A.ns), kThreads, 0, st>>>(A.sell<double>(), x,
                                                                                                 y);
    PFG_CUDA(cudaGetLastError());
}

void Krylov::spmv32(const DevMatrix &A, const float *x, float *y, cudaStream_t st)
{
    PFG_CHECK(A.v32_valid, PFG_E_STATE, "FP32 matrix copy not built");
    if (A.bs == 3)
        launch_spmv<3, float>(A, A.view<float>(), x, y, st);
    else
        launch_spmv<1, float>(A, A.view<float>(), x, y, st);
}

void Krylov::make_v32(DevMatrix &A, cudaStream_t st)
{
    const int64_t nv = A.nnzb * A.bs * A.bs;
    A.v32.ensure((size_t)std::max<int64_t>(nv, 1));
    if (nv) {
        k_to_f32<<<grid_for(nv, 256, sm_count() * 8), 256, 0, st>>>(A.v64.p, A.v32.p, nv);
        PFG_CUDA(cudaGetLastError());
    }
    A.v32_valid = true;
}

void Krylov::prepare(const DevMatrix &A, const KConfig &cfg, cudaStream_t st)
{
    const int64_t n = A.ndof();
    const bool mixed = cfg.precision == PFG_PREC_MIXED;
    n_ = n;
    bs_ = A.bs;
    const size_t nn = (size_t)std::max<int64_t>(n, 1);
    r_.ensure(nn);
    z_.ensure(nn);
    pA_.ensure(nn);
    pB_.ensure(nn);
    q_.ensure(nn);
    if (!mixed && cfg.algorithm == PFG_ALG_BICGSTAB) {
        r0_.ensure(nn);
        yA_.ensure(nn);
        yB_.ensure(nn);
        e_.ensure(nn);
        v_.ensure(nn);
        if (cfg.precond != PFG_PC_NONE) {
            ph_.ensure(nn);
            eh_.ensure(nn);
        }
    }
    if (mixed) {
        r32_.ensure(nn);
        z32_.ensure(nn);
        pA32_.ensure(nn);
        pB32_.ensure(nn);
        q32_.ensure(nn);
        x32_.ensure(nn);
        xb_.ensure(nn);
        if (cfg.algorithm == PFG_ALG_BICGSTAB) {
            r032_.ensure(nn);
            yA32_.ensure(nn);
            yB32_.ensure(nn);
            e32_.ensure(nn);
            v32_.ensure(nn);
            if (cfg.precond != PFG_PC_NONE) {
                ph32_.ensure(nn);
                eh32_.ensure(nn);
            }
        }
    }
    // one partial per CTA and reduced value: bound by the most CTAs that can be
    // resident (2048 threads per SM / kThreads)
    const int g = sm_count() * (2048 / kThreads);
    partials_.ensure((size_t)g * 4 + 8);
    partials32_.ensure((size_t)g * 8 + 16);
    if (!ticket_.p) {
        ticket_.alloc(1);
        PFG_CUDA(cudaMemsetAsync(ticket_.p, 0, sizeof(unsigned), st));
    }
    if (!state_.p) state_.alloc(1);
    PFG_CUDA(cudaMemsetAsync(state_.p, 0, sizeof(KState), st));
    (void)st;
}

void block_jacobi_inverse(const DevMatrix &A, int pc, double *d64, cudaStream_t st)
{
    const int g = grid_for(A.nb, 256, sm_count() * 8);
    if (A.bs == 3)
        k_precond<3><<<g, 256, 0, st>>>(A.view<double>(), pc, d64, nullptr);
    else
        k_precond<1><<<g, 256, 0, st>>>(A.view<double>(), pc, d64, nullptr);
    PFG_CUDA(cudaGetLastError());
}

void block_jacobi(const DevMatrix &A, int precond, double *d64, float *d32, cudaStream_t st)
{
    if (precond == PFG_PC_NONE || A.nb == 0) return;
    const int g = grid_for(A.nb, 256, sm_count() * 8);
    if (A.bs == 3)
        k_precond<3><<<g, 256, 0, st>>>(A.view<double>(), precond, d64, d32);
    else
        k_precond<1><<<g, 256, 0, st>>>(A.view<double>(), precond, d64, d32);
    PFG_CUDA(cudaGetLastError());
}

void Krylov::build_precond(const DevMatrix &A, int precond, bool fp32, cudaStream_t st)
{
    if (precond == PFG_PC_NONE || is_ilu(precond)) return;
    const size_t m = (size_t)std::max<int64_t>(A.nb * A.bs * A.bs, 1);
    dinv_.ensure(m);
    if (fp32) dinv32_.ensure(m);
    block_jacobi(A, precond, dinv_.p, fp32 ? dinv32_.p : nullptr, st);
    ++launches_;
}

void Krylov::read_state(KState &h, cudaStream_t st)
{
    PFG_CUDA(cudaMemcpyAsync(host_state_, state_.p, sizeof(KState), cudaMemcpyDeviceToHost, st));
    PFG_CUDA(cudaStreamSynchronize(st));
    h = *host_state_;
}

double Krylov::true_residual(const DevMatrix &A, const double *b, const double *x, double *r, cudaStream_t st)
{
    PFG_CHECK(A.s64_valid, PFG_E_INTERNAL, "sliced FP64 copy not built");
    const int g = A.bs == 3 ? resident_grid(k_residual64<3>, A.ns) : resident_grid(k_residual64<1>, A.ns);
    if (A.bs == 3)
        k_residual64<3><<<g, kThreads, 0, st>>>(A.sell<double>(), b, x, r, state_.p, partials_.p, ticket_.p);
    else
        k_residual64<1><<<g, kThreads, 0, st>>>(A.sell<double>(), b, x, r, state_.p, partials_.p, ticket_.p);
    PFG_CUDA(cudaGetLastError());
    ++launches_;
    KState h;
    read_state(h, st);
    const double bn = sqrt(h.bb);
    return bn > 0 ? sqrt(h.true_rr) / bn : sqrt(h.true_rr);
}

// Capture `body` (a sequence of kernel launches on `st`) into an executable graph.
template <typename F>
static cudaGraphExec_t capture(cudaStream_t st, F &&body)
{
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    PFG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    try {
        body();
    } catch (...) {
        cudaStreamEndCapture(st, &g);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    PFG_CUDA(cudaStreamEndCapture(st, &g));
    cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    PFG_CUDA(e);
    return ge;
}

static uint64_t mix_key(std::initializer_list<uint64_t> v)
{
    uint64_t h = 1469598103934665603ull;
    for (uint64_t x : v) {
        h ^= x + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
    }
    return h;
}

uint64_t Krylov::graph_key(int kind, const DevMatrix &A, const void *x, const KConfig &cfg) const
{
    auto u = [](const void *p) { return (uint64_t)(uintptr_t)p; };
    auto d = [](double v) {
        uint64_t b;
        memcpy(&b, &v, sizeof b);
        return b;
    };
    return mix_key({(uint64_t)kind, (uint64_t)A.bs, (uint64_t)A.nb, (uint64_t)A.nnzb, u(A.rp.p), u(A.col.p),
                    u(A.v64.p), u(A.v32.p), u(x), u(r_.p), u(r0_.p), u(z_.p), u(pA_.p), u(pB_.p), u(q_.p),
                    u(yA_.p), u(yB_.p), u(e_.p), u(v_.p), u(dinv_.p), u(r32_.p), u(r032_.p), u(z32_.p),
                    u(pA32_.p), u(pB32_.p), u(q32_.p), u(yA32_.p), u(yB32_.p), u(e32_.p), u(v32_.p), u(x32_.p),
                    u(dinv32_.p), u(ph_.p), u(eh_.p), u(ph32_.p), u(eh32_.p), u(partials_.p), u(partials32_.p), u(ticket_.p), u(state_.p),
                    (uint64_t)cfg.precond, (uint64_t)cfg.stop_rule, (uint64_t)cfg.graph_chunk, (uint64_t)cfg.itrmax,
                    (uint64_t)cfg.fuse, (uint64_t)cfg.storage, u(y4_.p), u(fx_.p), u(A.sptr_u.p), u(A.scol_u.p),
                    u(A.s32_u.p), d((double)A.sym_rowsum), d(cfg.relative_er), d(cfg.er0), d(cfg.reliable_delta),
                    ilu_ ? ilu_->generation() : 0, u(ilu_ ? ilu_->lu() : nullptr)});
}

// One chunk of CG iterations.  fuse: p = z + beta p formed inside the SpMV
// gather (ping-pong pA/pB), else a streaming pass updates p (= pA) in place.
template <int BS, typename T>
static int cg_chunk(const SellView<T> &A, bool fuse, int chunk, int64_t nb, T *x, T *r, T *z, T *pA, T *pB, T *q,
                    const T *dinv, int pc, KState *S, double *pd, float *pf, unsigned *tk, double tol, double delta,
                    int itrmax, cudaStream_t st)
{
    const int64_t n = nb * BS;
    const int gu = resident_grid(k_cg_update<BS, T>, (nb + 31) / 32);
    if (fuse) {
        const int gs = resident_grid(k_cg_spmv<BS, T>, A.ns);
        for (int it = 0; it < chunk; ++it) {
            k_cg_spmv<BS, T><<<gs, kThreads, 0, st>>>(A, z, pA, pB, q, S, pd, pf, tk);
            k_cg_update<BS, T><<<gu, kThreads, 0, st>>>(nb, x, r, z, pA, pB, q, dinv, pc, S, pd, pf, tk, tol, delta,
                                                        itrmax);
        }
    } else {
        const int gs = resident_grid(k_cg_spmv_u<BS, T>, A.ns);
        const int gd = resident_grid(k_cg_dir<T>, (n + 31) / 32);
        for (int it = 0; it < chunk; ++it) {
            k_cg_dir<T><<<gd, kThreads, 0, st>>>(n, z, pA, S);
            k_cg_spmv_u<BS, T><<<gs, kThreads, 0, st>>>(A, pA, q, S, pd, pf, tk);
            k_cg_update<BS, T><<<gu, kThreads, 0, st>>>(nb, x, r, z, pA, pA, q, dinv, pc, S, pd, pf, tk, tol, delta,
                                                        itrmax);
        }
    }
    PFG_CUDA(cudaGetLastError());
    return (fuse ? 2 : 3) * chunk;
}

// One chunk of BiCGSTAB iterations (bicgstab_CRS_2's loop body).  fuse: the
// direction and e updates ride in the SpMV gathers (ping-pong p and y), else
// two streaming passes update p and e in place (p = pA, y = yA).
template <int BS, typename T>
static int bicg_chunk(const SellView<T> &A, bool fuse, int chunk, int64_t nb, T *x, T *r, T *r0, T *pA, T *pB,
                      T *yA, T *yB, T *e, T *v, T *ph, T *eh, const T *dinv, int pc, KState *S, double *pd,
                      float *pf, unsigned *tk, int stop_rule, double er0, double tol, double delta, int itrmax,
                      cudaStream_t st)
{
    const int64_t n = nb * BS;
    const int64_t nvec = (n + 31) / 32;
    const int g3 = resident_grid(k_bicg_update<BS, T>, nvec);
    if (fuse) {
        const int g1 = resident_grid(k_bicg_spmv1<BS, T>, A.ns);
        const int g2 = resident_grid(k_bicg_spmv2<BS, T>, A.ns);
        for (int it = 0; it < chunk; ++it) {
            k_bicg_spmv1<BS, T><<<g1, kThreads, 0, st>>>(A, r, r0, pA, pB, yA, yB, S, pd, pf, tk);
            k_bicg_spmv2<BS, T><<<g2, kThreads, 0, st>>>(A, r, yA, yB, e, v, S, pd, pf, tk);
            k_bicg_update<BS, T><<<g3, kThreads, 0, st>>>(nb, x, r, r0, pA, pB, e, e, v, S, pd, pf, tk, stop_rule,
                                                          er0, tol, delta, itrmax);
        }
    } else {
        T *phat = pc != PFG_PC_NONE ? ph : pA;
        T *ehat = pc != PFG_PC_NONE ? eh : e;
        const int g1 = resident_grid(k_bicg_spmv1_u<BS, T>, A.ns);
        const int g2 = resident_grid(k_bicg_spmv2_u<BS, T>, A.ns);
        const int gd = resident_grid(k_bicg_dir<BS, T>, (nb + 31) / 32);
        const int ge = resident_grid(k_bicg_e<BS, T>, (nb + 31) / 32);
        for (int it = 0; it < chunk; ++it) {
            k_bicg_dir<BS, T><<<gd, kThreads, 0, st>>>(nb, r, pA, yA, ph, dinv, pc, S);
            k_bicg_spmv1_u<BS, T><<<g1, kThreads, 0, st>>>(A, phat, r0, yA, S, pd, pf, tk);
            k_bicg_e<BS, T><<<ge, kThreads, 0, st>>>(nb, r, yA, e, eh, dinv, pc, S);
            k_bicg_spmv2_u<BS, T><<<g2, kThreads, 0, st>>>(A, ehat, e, v, S, pd, pf, tk);
            k_bicg_update<BS, T><<<g3, kThreads, 0, st>>>(nb, x, r, r0, phat, phat, e, ehat, v, S, pd, pf, tk,
                                                          stop_rule, er0, tol, delta, itrmax);
        }
    }
    PFG_CUDA(cudaGetLastError());
    return (fuse ? 3 : 5) * chunk;
}

// One chunk of ILU(0)-preconditioned FP64 BiCGSTAB iterations
// (bicgstab_CRS_ILU's loop body, LinearSolverClass.f90:4140-4228): the
// direction and e passes without a preconditioner, ph = M^-1 p and
// eh = M^-1 e by the level-scheduled sweep, the products y = A ph and
// v = A eh, and the update x += alpha ph + c3 eh.
template <int BS>
static int bicg_chunk_ilu(const SellView<double> &A, const Ilu0 &ilu, int chunk, int64_t nb, double *x, double *r,
                          double *r0, double *p, double *y, double *e, double *v, double *ph, double *eh, KState *S,
                          double *pd, float *pf, unsigned *tk, int stop_rule, double er0, double tol, int itrmax,
                          cudaStream_t st)
{
    const int64_t n = nb * BS;
    const int g3 = resident_grid(k_bicg_update<BS, double>, (n + 31) / 32);
    const int g1 = resident_grid(k_bicg_spmv1_u<BS, double>, A.ns);
    const int g2 = resident_grid(k_bicg_spmv2_u<BS, double>, A.ns);
    const int gd = resident_grid(k_bicg_dir<BS, double>, (nb + 31) / 32);
    const int ge = resident_grid(k_bicg_e<BS, double>, (nb + 31) / 32);
    int nk = 0;
    for (int it = 0; it < chunk; ++it) {
        k_bicg_dir<BS, double><<<gd, kThreads, 0, st>>>(nb, r, p, y, ph, nullptr, PFG_PC_NONE, S);
        nk += ilu.apply(p, ph, S, st);
        k_bicg_spmv1_u<BS, double><<<g1, kThreads, 0, st>>>(A, ph, r0, y, S, pd, pf, tk);
        k_bicg_e<BS, double><<<ge, kThreads, 0, st>>>(nb, r, y, e, eh, nullptr, PFG_PC_NONE, S);
        nk += ilu.apply(e, eh, S, st);
        k_bicg_spmv2_u<BS, double><<<g2, kThreads, 0, st>>>(A, eh, e, v, S, pd, pf, tk);
        k_bicg_update<BS, double><<<g3, kThreads, 0, st>>>(nb, x, r, r0, ph, ph, e, eh, v, S, pd, pf, tk, stop_rule,
                                                          er0, tol, 0.1, itrmax);
        nk += 5;
    }
    PFG_CUDA(cudaGetLastError());
    return nk;
}

// One chunk of FP32 CG iterations with the symmetric (upper-half) matrix:
// dir, product into q4 with <p, Ap> and alpha, update (reads and clears q4).
static int cg_chunk_sym(const SellView<float> &U, bool fuse, int chunk, int64_t nb, float *x, float *r, float *z,
                        float *pA, float *pB, float *q4, const float *dinv, int pc, KState *S, double *pd, float *pf,
                        unsigned *tk, double tol, double delta, int itrmax, cudaStream_t st)
{
    const int64_t n = nb * 3;
    const int gd = resident_grid(k_cg_dir<float>, (n + 31) / 32);
    const int gu = resident_grid(k_cg_update<3, float, 4>, (nb + 31) / 32);
    for (int it = 0; it < chunk; ++it) {
        if (fuse) {  // direction update inside the product (ping-pong pA / pB)
            launch_cg_spmv_sym(true, U, z, pA, pB, q4, S, pd, pf, tk, st);
            k_cg_update<3, float, 4><<<gu, kThreads, 0, st>>>(nb, x, r, z, pA, pB, q4, dinv, pc, S, pd, pf, tk, tol,
                                                              delta, itrmax);
        } else {
            k_cg_dir<float><<<gd, kThreads, 0, st>>>(n, z, pA, S);
            launch_cg_spmv_sym(false, U, nullptr, pA, nullptr, q4, S, pd, pf, tk, st);
            k_cg_update<3, float, 4><<<gu, kThreads, 0, st>>>(nb, x, r, z, pA, pA, q4, dinv, pc, S, pd, pf, tk, tol,
                                                              delta, itrmax);
        }
    }
    PFG_CUDA(cudaGetLastError());
    return (fuse ? 2 : 3) * chunk;
}

// One chunk of FP32 BiCGSTAB iterations with the symmetric matrix (the
// separate-pass structure of bicg_chunk): each product is the reproducible
// fixed-point form (k_spmv_symfx + k_symfx_finish), and the direction and e
// passes record the maximum of the vector the next product reads.
static int bicg_chunk_sym(const SellView<float> &U, float rowsum, int chunk, int64_t nb, float *x, float *r,
                          float *r0, float *p, float *y, float *e, float *v, float *ph, float *eh,
                          unsigned long long *fx, const float *dinv, int pc, KState *S, double *pd, float *pf,
                          unsigned *tk, double er0, double tol, double delta, int itrmax, cudaStream_t st)
{
    const int64_t nvec = (nb * 3 + 31) / 32;
    float *phat = pc != PFG_PC_NONE ? ph : p;
    float *ehat = pc != PFG_PC_NONE ? eh : e;
    const int gd = resident_grid(k_bicg_dir<3, float>, (nb + 31) / 32);
    const int ge = resident_grid(k_bicg_e<3, float>, (nb + 31) / 32);
    const int gf = resident_grid(k_symfx_finish, (3 * nb + 127) / 128);
    const int g3 = resident_grid(k_bicg_update<3, float>, nvec);
    for (int it = 0; it < chunk; ++it) {
        k_bicg_dir<3, float><<<gd, kThreads, 0, st>>>(nb, r, p, y, ph, dinv, pc, S, true);
        launch_spmv_symfx(U, phat, y, fx, rowsum, S, st);
        k_symfx_finish<<<gf, kThreads, 0, st>>>(nb, y, fx, r0, rowsum, 1, S, pd, pf, tk);
        k_bicg_e<3, float><<<ge, kThreads, 0, st>>>(nb, r, y, e, eh, dinv, pc, S, true);
        launch_spmv_symfx(U, ehat, v, fx, rowsum, S, st);
        k_symfx_finish<<<gf, kThreads, 0, st>>>(nb, v, fx, e, rowsum, 2, S, pd, pf, tk);
        k_bicg_update<3, float><<<g3, kThreads, 0, st>>>(nb, x, r, r0, phat, phat, e, ehat, v, S, pd, pf, tk,
                                                         PFG_STOP_TRUE_RELATIVE, er0, tol, delta, itrmax);
    }
    PFG_CUDA(cudaGetLastError());
    return 7 * chunk;
}

SolveResult Krylov::solve(DevMatrix &A, const double *b, double *x, const KConfig &cfg_in, cudaStream_t st)
{
    KConfig cfg = cfg_in;
    PFG_CHECK(A.nb > 0, PFG_E_STATE, "empty matrix");
    PFG_CHECK(cfg.algorithm == PFG_ALG_CG || cfg.algorithm == PFG_ALG_BICGSTAB, PFG_E_ARG, "unknown algorithm");
    PFG_CHECK(cfg.precision == PFG_PREC_FP64 || cfg.precision == PFG_PREC_MIXED, PFG_E_ARG, "unknown precision");
    PFG_CHECK(cfg.precond >= PFG_PC_NONE && cfg.precond <= PFG_PC_ILU0_SORTED, PFG_E_ARG, "unknown precond");
    PFG_CHECK(!is_ilu(cfg.precond) || (cfg.algorithm == PFG_ALG_BICGSTAB && cfg.precision == PFG_PREC_FP64),
              PFG_E_UNSUPPORTED, "ILU(0) preconditions FP64 BiCGSTAB only (bicgstab_CRS_ILU)");
    if (cfg.itrmax <= 0) cfg.itrmax = 100000;
    if (cfg.graph_chunk <= 0) cfg.graph_chunk = 32;
    if (cfg.precision == PFG_PREC_MIXED) cfg.stop_rule = PFG_STOP_TRUE_RELATIVE;
    PFG_CHECK(cfg.storage == PFG_STORAGE_FULL || cfg.storage == PFG_STORAGE_SYMMETRIC, PFG_E_ARG, "unknown storage");
    // the symmetric copy serves the FP32 inner iterations of 3x3-block systems
    if (cfg.precision != PFG_PREC_MIXED || A.bs != 3) cfg.storage = PFG_STORAGE_FULL;
    if (cfg.reliable_delta <= 0.0 || cfg.reliable_delta >= 1.0) cfg.reliable_delta = 0.1;
    // update_mode 0 (auto): separate streaming passes.  Measured on GB300 at
    // 3.09M DOF: FP64 CG 894 ms separate vs 1165 ms fused (the fused gather
    // doubles the work of the FP64-pipe-bound SpMV), FP32 CG 430 vs 448 ms;
    // mixed CG from the symmetric copy 257.6-259.1 vs 255.3-257.0 ms (the
    // gathers of z and p_old cost about what the direction pass saves).
    // Preconditioned BiCGSTAB exists only in the separate form.
    if (cfg.fuse != 0 && cfg.fuse != 1) cfg.fuse = 0;
    if (cfg.algorithm == PFG_ALG_BICGSTAB && cfg.precond != PFG_PC_NONE) cfg.fuse = 0;
    prepare(A, cfg, st);
    launches_ = 0;
    // the Krylov kernels read the sliced copy: FP64 always (residuals), FP32
    // for the mixed inner iterations
    // the symmetric-storage inner iterations read only the upper-half FP32 copy
    build_sell(A, true, cfg.precision == PFG_PREC_MIXED && cfg.storage != PFG_STORAGE_SYMMETRIC, st);
    cudaEvent_t e0, e1;
    PFG_CUDA(cudaEventCreate(&e0));
    PFG_CUDA(cudaEventCreate(&e1));
    PFG_CUDA(cudaEventRecord(e0, st));
    SolveResult res;
    try {
        if (cfg.precision == PFG_PREC_MIXED) {
            res = run_mixed(A, b, x, cfg, st);
            if (res.fallback) {
                // The FP32 copy of the operator failed (repeated breakdowns or
                // overflow, or FP64 residuals that stopped falling: a system
                // whose conditioning is beyond FP32).  Finish in FP64 from the
                // current x, within what is left of itrmax.
                KConfig c64 = cfg;
                c64.precision = PFG_PREC_FP64;
                c64.stop_rule = PFG_STOP_TRUE_RELATIVE;
                c64.itrmax = std::max(1, cfg.itrmax - res.iterations);
                prepare(A, c64, st);
                SolveResult r2 = cfg.algorithm == PFG_ALG_CG ? run_cg64(A, b, x, c64, st)
                                                             : run_bicgstab64(A, b, x, c64, st);
                r2.iterations += res.iterations;
                r2.replacements = res.replacements;
                r2.fallback = 1;
                res = r2;
            }
        } else if (cfg.algorithm == PFG_ALG_CG)
            res = run_cg64(A, b, x, cfg, st);
        else
            res = run_bicgstab64(A, b, x, cfg, st);
    } catch (...) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
    }
    PFG_CUDA(cudaEventRecord(e1, st));
    PFG_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    res.ms = ms;
    res.launches = launches_;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return res;
}

SolveResult Krylov::run_cg64(DevMatrix &A, const double *b, double *x, const KConfig &cfg, cudaStream_t st)
{
    SolveResult res;
    build_precond(A, cfg.precond, false, st);
    const int64_t n = A.ndof();
    const int g = row_grid(A.nb);
    const uint64_t key = graph_key(1, A, x, cfg);
    if (!graph_ || graph_key_ != key) {
        if (graph_) cudaGraphExecDestroy(graph_);
        graph_ = nullptr;
        int nk = 0;
        auto body = [&]() {
            nk = A.bs == 3 ? cg_chunk<3, double>(A.sell<double>(), cfg.fuse != 0, cfg.graph_chunk, A.nb, x, r_.p,
                                                 z_.p, pA_.p, pB_.p, q_.p, dinv_.p, cfg.precond, state_.p,
                                                 partials_.p, partials32_.p, ticket_.p, cfg.relative_er,
                                                 cfg.reliable_delta, cfg.itrmax, st)
                           : cg_chunk<1, double>(A.sell<double>(), cfg.fuse != 0, cfg.graph_chunk, A.nb, x, r_.p,
                                                 z_.p, pA_.p, pB_.p, q_.p, dinv_.p, cfg.precond, state_.p,
                                                 partials_.p, partials32_.p, ticket_.p, cfg.relative_er,
                                                 cfg.reliable_delta, cfg.itrmax, st);
        };
        graph_ = capture(st, body);
        graph_key_ = key;
        graph_kernels_ = nk;
    }
    bool fresh = false;  // res.rel_residual is the true residual of the current x
    for (int restart = 0; restart < 20; ++restart) {
        // r = b - A x (true residual), restart the recurrences from it
        double rel = true_residual(A, b, x, r_.p, st);
        res.rel_residual = rel;
        if (rel <= cfg.relative_er) {
            fresh = true;
            break;
        }
        PFG_CUDA(cudaMemsetAsync(pA_.p, 0, n * sizeof(double), st));
        PFG_CUDA(cudaMemsetAsync(pB_.p, 0, n * sizeof(double), st));
        if (A.bs == 3)
            k_cg_restart<3, double><<<g, kThreads, 0, st>>>(A.nb, r_.p, z_.p, dinv_.p, cfg.precond, state_.p,
                                                            partials_.p, partials32_.p, ticket_.p, 0);
        else
            k_cg_restart<1, double><<<g, kThreads, 0, st>>>(A.nb, r_.p, z_.p, dinv_.p, cfg.precond, state_.p,
                                                            partials_.p, partials32_.p, ticket_.p, 0);
        PFG_CUDA(cudaGetLastError());
        ++launches_;
        KState h;
        for (;;) {
            PFG_CUDA(cudaGraphLaunch(graph_, st));
            launches_ += graph_kernels_;
            read_state(h, st);
            if (cfg.debug != 0) fprintf(stderr, "[pfg] CG64 iter %d |r|/|b| %.3e\n", h.iter, sqrt(h.rr / h.bb));
            if (h.done) break;
        }
        res.iterations = h.iter;
        res.iter_residual = sqrt(h.rr / h.bb);
        if (h.status != PFG_OK) {
            res.status = h.status;
            res.rel_residual = true_residual(A, b, x, r_.p, st);
            return res;
        }
        // clear done, keep the iteration count for itrmax
        int zero = 0;
        PFG_CUDA(cudaMemcpyAsync(&state_.p->done, &zero, sizeof(int), cudaMemcpyHostToDevice, st));
    }
    if (!fresh) res.rel_residual = true_residual(A, b, x, r_.p, st);
    if (res.rel_residual > cfg.relative_er && res.status == PFG_OK) res.status = PFG_W_NOT_CONVERGED;
    return res;
}

SolveResult Krylov::run_bicgstab64(DevMatrix &A, const double *b, double *x, const KConfig &cfg, cudaStream_t st)
{
    SolveResult res;
    build_precond(A, cfg.precond, false, st);
    const bool ilu = is_ilu(cfg.precond);
    if (ilu) {
        ilu_factor(A, cfg.precond == PFG_PC_ILU0_SORTED, st);
        ++launches_;
    }
    const int64_t n = A.ndof();
    const int g = row_grid(A.nb);
    const uint64_t key = graph_key(2, A, x, cfg);
    if (!graph_ || graph_key_ != key) {
        if (graph_) cudaGraphExecDestroy(graph_);
        graph_ = nullptr;
        int nk = 0;
        // an ILU iteration captures two sweeps of one launch per level: a
        // few thousand graph nodes per chunk at most
        const int ilu_chunk =
            ilu ? std::max(1, std::min(cfg.graph_chunk, 4096 / (5 + 2 * ilu_->levels()))) : cfg.graph_chunk;
        auto body = [&]() {
            if (ilu) {
                nk = A.bs == 3 ? bicg_chunk_ilu<3>(A.sell<double>(), *ilu_, ilu_chunk, A.nb, x, r_.p, r0_.p, pA_.p,
                                                   yA_.p, e_.p, v_.p, ph_.p, eh_.p, state_.p, partials_.p,
                                                   partials32_.p, ticket_.p, cfg.stop_rule, cfg.er0,
                                                   cfg.relative_er, cfg.itrmax, st)
                               : bicg_chunk_ilu<1>(A.sell<double>(), *ilu_, ilu_chunk, A.nb, x, r_.p, r0_.p, pA_.p,
                                                   yA_.p, e_.p, v_.p, ph_.p, eh_.p, state_.p, partials_.p,
                                                   partials32_.p, ticket_.p, cfg.stop_rule, cfg.er0,
                                                   cfg.relative_er, cfg.itrmax, st);
                return;
            }
            nk = A.bs == 3 ? bicg_chunk<3, double>(A.sell<double>(), cfg.fuse != 0, cfg.graph_chunk, A.nb, x, r_.p,
                                                   r0_.p, pA_.p, pB_.p, yA_.p, yB_.p, e_.p, v_.p, ph_.p, eh_.p,
                                                   dinv_.p, cfg.precond, state_.p,
                                                   partials_.p, partials32_.p, ticket_.p, cfg.stop_rule, cfg.er0,
                                                   cfg.relative_er, cfg.reliable_delta, cfg.itrmax, st)
                           : bicg_chunk<1, double>(A.sell<double>(), cfg.fuse != 0, cfg.graph_chunk, A.nb, x, r_.p,
                                                   r0_.p, pA_.p, pB_.p, yA_.p, yB_.p, e_.p, v_.p, ph_.p, eh_.p,
                                                   dinv_.p, cfg.precond, state_.p,
                                                   partials_.p, partials32_.p, ticket_.p, cfg.stop_rule, cfg.er0,
                                                   cfg.relative_er, cfg.reliable_delta, cfg.itrmax, st);
        };
        graph_ = capture(st, body);
        graph_key_ = key;
        graph_kernels_ = nk;
    }
    const int max_restarts = cfg.stop_rule == PFG_STOP_REFERENCE ? 1 : 20;
    bool fresh = false;  // res.rel_residual is the true residual of the current x
    for (int restart = 0; restart < max_restarts; ++restart) {
        double rel = true_residual(A, b, x, r_.p, st);
        res.rel_residual = rel;
        fresh = true;
        if (cfg.stop_rule == PFG_STOP_TRUE_RELATIVE && rel <= cfg.relative_er) break;
        // bicgstab_CRS_ILU returns before its loop when |r|^2 < er0 (:4150)
        if (ilu && cfg.stop_rule == PFG_STOP_REFERENCE && host_state_->true_rr < cfg.er0) break;
        fresh = false;
        PFG_CUDA(cudaMemsetAsync(pA_.p, 0, n * sizeof(double), st));
        PFG_CUDA(cudaMemsetAsync(pB_.p, 0, n * sizeof(double), st));
        PFG_CUDA(cudaMemsetAsync(yA_.p, 0, n * sizeof(double), st));
        PFG_CUDA(cudaMemsetAsync(yB_.p, 0, n * sizeof(double), st));
        k_bicg_restart<double><<<g, kThreads, 0, st>>>(n, r_.p, r0_.p, state_.p, partials_.p, partials32_.p,
                                                       ticket_.p, 1, 0);
        PFG_CUDA(cudaGetLastError());
        ++launches_;
        KState h;
        for (;;) {
            PFG_CUDA(cudaGraphLaunch(graph_, st));
            launches_ += graph_kernels_;
            read_state(h, st);
            if (cfg.debug != 0) fprintf(stderr, "[pfg] BiCGSTAB64 iter %d |r| %.3e\n", h.iter, sqrt(h.rr));
            if (h.done) break;
        }
        res.iterations = h.iter;
        res.iter_residual = cfg.stop_rule == PFG_STOP_REFERENCE ? sqrt(h.rr / (h.rr1 > 0 ? h.rr1 : 1.0))
                                                                : sqrt(h.rr / h.bb);
        if (h.status != PFG_OK) {
            res.status = h.status;
            break;
        }
        int zero = 0;
        PFG_CUDA(cudaMemcpyAsync(&state_.p->done, &zero, sizeof(int), cudaMemcpyHostToDevice, st));
    }
    if (!fresh) res.rel_residual = true_residual(A, b, x, r_.p, st);
    if (cfg.stop_rule == PFG_STOP_TRUE_RELATIVE && res.rel_residual > cfg.relative_er && res.status == PFG_OK)
        res.status = PFG_W_NOT_CONVERGED;
    return res;
}

// Replacements in a row whose FP64 residual did not fall by 10 %, and FP32
// passes in a row whose correction was rejected, before the mixed solve hands
// over to FP64 (BiCGSTAB's residual is erratic: it gets more room).
constexpr int kMixedStallCG = 4, kMixedStallBiCG = 8;
constexpr int kMixedRejectCG = 2, kMixedRejectBiCG = 2;

SolveResult Krylov::run_mixed(DevMatrix &A, const double *b, double *x, const KConfig &cfg, cudaStream_t st)
{
    SolveResult res;
    const bool cg = cfg.algorithm == PFG_ALG_CG;
    // the FP32 sliced copies come from the FP64 values (build_sell,
    // build_sell_upper): no FP32 block-row copy is needed here
    build_precond(A, cfg.precond, true, st);
    const int64_t n = A.ndof();
    const int g = row_grid(A.nb);
    const int gv = grid_for(n, 256, sm_count() * 8);
    const bool sym = cfg.storage == PFG_STORAGE_SYMMETRIC;
    if (sym) {
        // upper half (checked symmetric) and its zeroed accumulator: 4 floats
        // per row (CG) or three fixed-point planes (BiCGSTAB)
        build_sell_upper(A, st);
        if (cg) {
            y4_.ensure((size_t)A.nb * 4);
            PFG_CUDA(cudaMemsetAsync(y4_.p, 0, (size_t)A.nb * 4 * sizeof(float), st));
        } else {
            fx_.ensure((size_t)A.nb * 3);
            PFG_CUDA(cudaMemsetAsync(fx_.p, 0, (size_t)A.nb * 3 * sizeof(unsigned long long), st));
        }
    }
    if (sym) {  // (the first call per kernel sets a kernel attribute: outside capture)
        staged_grid(k_cg_spmv_sym, SymbLayout::kSmem, A.ns_u);
        staged_grid(k_cg_spmv_sym_fused, SymbLayout::kSmem, A.ns_u);
        staged_grid(k_spmv_symfx, SymbLayout::kSmem, A.ns_u);
    }
    const uint64_t key = graph_key(cg ? 3 : 4, A, x, cfg);
    if (!graph_ || graph_key_ != key) {
        if (graph_) cudaGraphExecDestroy(graph_);
        graph_ = nullptr;
        int nk = 0;
        auto body = [&]() {
            const bool fz = cfg.fuse != 0;
            const int ch = cfg.graph_chunk;
            if (sym && cg)
                nk = cg_chunk_sym(sell_upper(A), fz, ch, A.nb, x32_.p, r32_.p, z32_.p, pA32_.p, pB32_.p, y4_.p,
                                  dinv32_.p,
                                  cfg.precond, state_.p, partials_.p, partials32_.p, ticket_.p, cfg.relative_er,
                                  cfg.reliable_delta, cfg.itrmax, st);
            else if (sym)
                nk = bicg_chunk_sym(sell_upper(A), A.sym_rowsum, ch, A.nb, x32_.p, r32_.p, r032_.p, pA32_.p,
                                    yA32_.p, e32_.p, v32_.p, ph32_.p, eh32_.p, fx_.p, dinv32_.p, cfg.precond,
                                    state_.p, partials_.p, partials32_.p, ticket_.p, cfg.er0, cfg.relative_er,
                                    cfg.reliable_delta, cfg.itrmax, st);
            else if (cg)
                nk = A.bs == 3 ? cg_chunk<3, float>(A.sell<float>(), fz, ch, A.nb, x32_.p, r32_.p, z32_.p, pA32_.p,
                                                    pB32_.p, q32_.p, dinv32_.p, cfg.precond, state_.p, partials_.p,
                                                    partials32_.p, ticket_.p, cfg.relative_er, cfg.reliable_delta,
                                                    cfg.itrmax, st)
                               : cg_chunk<1, float>(A.sell<float>(), fz, ch, A.nb, x32_.p, r32_.p, z32_.p, pA32_.p,
                                                    pB32_.p, q32_.p, dinv32_.p, cfg.precond, state_.p, partials_.p,
                                                    partials32_.p, ticket_.p, cfg.relative_er, cfg.reliable_delta,
                                                    cfg.itrmax, st);
            else
                nk = A.bs == 3 ? bicg_chunk<3, float>(A.sell<float>(), fz, ch, A.nb, x32_.p, r32_.p, r032_.p,
                                                      pA32_.p, pB32_.p, yA32_.p, yB32_.p, e32_.p, v32_.p, ph32_.p,
                                                      eh32_.p, dinv32_.p, cfg.precond, state_.p,
                                                      partials_.p, partials32_.p, ticket_.p, PFG_STOP_TRUE_RELATIVE,
                                                      cfg.er0, cfg.relative_er, cfg.reliable_delta, cfg.itrmax, st)
                               : bicg_chunk<1, float>(A.sell<float>(), fz, ch, A.nb, x32_.p, r32_.p, r032_.p,
                                                      pA32_.p, pB32_.p, yA32_.p, yB32_.p, e32_.p, v32_.p, ph32_.p,
                                                      eh32_.p, dinv32_.p, cfg.precond, state_.p,
                                                      partials_.p, partials32_.p, ticket_.p, PFG_STOP_TRUE_RELATIVE,
                                                      cfg.er0, cfg.relative_er, cfg.reliable_delta, cfg.itrmax, st);
        };
        graph_ = capture(st, body);
        graph_key_ = key;
        graph_kernels_ = nk;
    }
    // initial FP64 residual and first replacement
    PFG_CUDA(cudaMemsetAsync(x32_.p, 0, n * sizeof(float), st));
    PFG_CUDA(cudaMemsetAsync(pA32_.p, 0, n * sizeof(float), st));
    PFG_CUDA(cudaMemsetAsync(pB32_.p, 0, n * sizeof(float), st));
    if (!cg) {
        PFG_CUDA(cudaMemsetAsync(yA32_.p, 0, n * sizeof(float), st));
        PFG_CUDA(cudaMemsetAsync(yB32_.p, 0, n * sizeof(float), st));
    }
    bool first = true;
    KState h;
    memset(&h, 0, sizeof(h));
    double best_rel = 0.0, prev_rel = 0.0;
    int stall = 0, failures = 0;
    for (;;) {
        // residual replacement: x64 += x32; r64 = b - A64 x64; r32 = r64.
        // The FP32 correction is kept only if it lowers the FP64 residual
        // (x is backed up before the fold); an overflowed one is dropped.
        bool rejected = false;
        if (!first) {
            if (h.poisoned) {
                PFG_CUDA(cudaMemsetAsync(x32_.p, 0, n * sizeof(float), st));
                const int zero = 0;
                PFG_CUDA(cudaMemcpyAsync(&state_.p->poisoned, &zero, sizeof(int), cudaMemcpyHostToDevice, st));
                rejected = true;
            } else {
                PFG_CUDA(cudaMemcpyAsync(xb_.p, x, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
                k_fold<<<gv, 256, 0, st>>>(n, x, x32_.p);
                PFG_CUDA(cudaGetLastError());
                ++launches_;
            }
        }
        double rel = true_residual(A, b, x, r_.p, st);
        // CG's true residual falls from pass to pass; BiCGSTAB's does not
        // have to (a pass may raise it a little and the next still carry on),
        // so a BiCGSTAB correction is dropped when it raises it tenfold.
        // Measured on the 3.09M-DOF system (ten solves each): dropping only
        // thousandfold rises let 300-660-fold rises through, each costing
        // hundreds of iterations to climb back (median 983 ms, worst 1264);
        // tenfold: median 787 ms, worst 983 ms.
        const double growth = cg ? 1.0 : 10.0;
        if (!first && !rejected && !(rel < growth * prev_rel)) {
            if (cfg.debug != 0)
                fprintf(stderr, "[pfg] mixed iter %d: correction raised |b-Ax|/|b| %.3e -> %.3e\n", h.iter, prev_rel,
                        rel);
            PFG_CUDA(cudaMemcpyAsync(x, xb_.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
            rel = true_residual(A, b, x, r_.p, st);
            rejected = true;
        } else if (!first && rejected && cfg.debug != 0) {
            fprintf(stderr, "[pfg] mixed iter %d: FP32 pass overflowed (breakdowns %d)\n", h.iter, h.breakdowns);
        }
        prev_rel = rel;
        failures = rejected ? failures + 1 : 0;
        // A rejected CG pass restarts from the same state and would fail the
        // same way; within 100x of the target FP64 finishes in a few
        // iterations.  A rejected BiCGSTAB pass is retried from a full
        // restart (r0 = r, p = r) and hands over after two rejections in a
        // row: its FP64 finish restarts the Krylov space (~200-470 iterations
        // from 1e-9..1e-7 on the 3.09M-DOF system).
        if (rejected && rel < 100.0 * cfg.relative_er && cg) failures = std::max(failures, kMixedRejectCG);
        if (cfg.debug != 0 && rejected)
            fprintf(stderr, "[pfg] mixed iter %d: FP32 correction rejected (|b-Ax|/|b| %.3e)\n", h.iter, rel);
        if (failures >= (cg ? kMixedRejectCG : kMixedRejectBiCG) && rel > cfg.relative_er) {
            // FP32 passes in a row made no progress: finish in FP64
            if (cfg.debug != 0) fprintf(stderr, "[pfg] mixed: hand-over to FP64 after rejected corrections\n");
            res.fallback = 1;
            res.iterations = h.iter;
            res.replacements = h.replacements;
            res.rel_residual = rel;
            return res;
        }
        res.rel_residual = rel;
        // FP64 residuals that stopped falling (10 % per replacement) while
        // above the target: the FP32 operator has reached its accuracy
        if (first || rel < 0.9 * best_rel) {
            best_rel = rel;
            stall = 0;
        } else if (++stall >= (cg ? kMixedStallCG : kMixedStallBiCG) && rel > cfg.relative_er) {
            if (cfg.debug != 0) fprintf(stderr, "[pfg] mixed: hand-over to FP64 after stalled residuals\n");
            res.fallback = 1;
            res.iterations = h.iter;
            res.replacements = h.replacements;
            return res;
        }
        k_replace<<<gv, 256, 0, st>>>(n, r_.p, r32_.p, state_.p, cfg.relative_er);
        PFG_CUDA(cudaGetLastError());
        launches_ += 2;  // k_replace and the restart below
        if (cg) {
            // a rejected pass restarts from p = z (its direction may be spoilt)
            const int keep = (first || rejected) ? 0 : 1;
            if (rejected) {
                PFG_CUDA(cudaMemsetAsync(pA32_.p, 0, n * sizeof(float), st));
                PFG_CUDA(cudaMemsetAsync(pB32_.p, 0, n * sizeof(float), st));
            }
            if (A.bs == 3)
                k_cg_restart<3, float><<<g, kThreads, 0, st>>>(A.nb, r32_.p, z32_.p, dinv32_.p, cfg.precond,
                                                               state_.p, partials_.p, partials32_.p, ticket_.p,
                                                               keep);
            else
                k_cg_restart<1, float><<<g, kThreads, 0, st>>>(A.nb, r32_.p, z32_.p, dinv32_.p, cfg.precond,
                                                               state_.p, partials_.p, partials32_.p, ticket_.p,
                                                               keep);
        } else {
            // Keep the search direction and the shadow residual r0 while r0.r
            // still carries FP32 digits (|cos(r0, r)| > 1e-3); otherwise, or
            // after a breakdown, restart with r0 = r and p = r.  Keeping the
            // first r0 for good makes r0.r lose every FP32 digit once |r| has
            // dropped by many orders.
            bool full = first || rejected || h.breakdowns > 0;
            if (!full) {
                k_bicg_restart<float><<<g, kThreads, 0, st>>>(n, r32_.p, r032_.p, state_.p, partials_.p,
                                                              partials32_.p, ticket_.p, 0, 1);
                PFG_CUDA(cudaGetLastError());
                ++launches_;
                read_state(h, st);
                const double den = std::sqrt((double)h.rr32 * (double)h.r0r0_32);
                full = !(den > 0.0 && std::fabs((double)h.c1_32) > 1e-3 * den);
            }
            if (full) {
                PFG_CUDA(cudaMemsetAsync(pA32_.p, 0, n * sizeof(float), st));
                PFG_CUDA(cudaMemsetAsync(pB32_.p, 0, n * sizeof(float), st));
                PFG_CUDA(cudaMemsetAsync(yA32_.p, 0, n * sizeof(float), st));
                PFG_CUDA(cudaMemsetAsync(yB32_.p, 0, n * sizeof(float), st));
                k_bicg_restart<float><<<g, kThreads, 0, st>>>(n, r32_.p, r032_.p, state_.p, partials_.p,
                                                              partials32_.p, ticket_.p, 1, 0);
            }
        }
        PFG_CUDA(cudaGetLastError());
        first = false;
        read_state(h, st);
        if (h.breakdowns > 3 && !h.done) {
            // repeated FP32 breakdowns with no completed iteration in between:
            // x holds the folded solution, the caller finishes in FP64
            res.fallback = 1;
            res.iterations = h.iter;
            res.replacements = h.replacements;
            return res;
        }
        if (cfg.debug != 0)
            fprintf(stderr, "[pfg] mixed iter %d replacement %d |b-Ax|/|b| %.3e\n", h.iter, h.replacements, rel);
        if (h.done) break;
        for (;;) {
            PFG_CUDA(cudaGraphLaunch(graph_, st));
            launches_ += graph_kernels_;
            read_state(h, st);
            if (h.done || h.need_update) break;
        }
        if (h.done && h.status != PFG_OK) {
            // fold what was computed, report the true residual
            k_fold<<<gv, 256, 0, st>>>(n, x, x32_.p);
            PFG_CUDA(cudaGetLastError());
            ++launches_;
            res.rel_residual = true_residual(A, b, x, r_.p, st);
            break;
        }
    }
    res.status = h.status;
    res.iterations = h.iter;
    res.replacements = h.replacements;
    res.iter_residual = sqrt((double)h.rr32 / (h.bb > 0 ? h.bb : 1.0));
    if (res.status == PFG_OK && res.rel_residual > cfg.relative_er) res.status = PFG_W_NOT_CONVERGED;
    return res;
}

__global__ void k_fill(float *a, int64_t n, float v)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        a[i] = v;
}
__global__ void k_fill(double *a, int64_t n, double v)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        a[i] = v;
}

void Krylov::profile(DevMatrix &A, int kernel, int reps, cudaStream_t st, double &ms, double &bytes)
{
    PFG_CHECK(kernel >= 0 && kernel <= 12 && reps > 0, PFG_E_ARG, "bad profile request");
    if (kernel == 9) {
        // one D^-1 L^-1 sweep of the held ILU(0) factor (factored in
        // ascending column order if none is held)
        if (!ilu_ || !ilu_->ready()) ilu_factor(A, true, st);
        const int64_t nd = A.ndof();
        DevBuf<double> v(nd), o(nd);
        k_fill<<<grid_for(nd, 256, sm_count() * 8), 256, 0, st>>>(v.p, nd, 1.0);
        for (int w = 0; w < 3; ++w) ilu_->apply(v.p, o.p, nullptr, st);
        cudaEvent_t e0, e1;
        PFG_CUDA(cudaEventCreate(&e0));
        PFG_CUDA(cudaEventCreate(&e1));
        PFG_CUDA(cudaEventRecord(e0, st));
        for (int r = 0; r < reps; ++r) ilu_->apply(v.p, o.p, nullptr, st);
        PFG_CUDA(cudaEventRecord(e1, st));
        PFG_CUDA(cudaEventSynchronize(e1));
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        ms = (double)t / reps;
        bytes = ilu_->sweep_bytes();
        return;
    }
    PFG_CHECK(kernel < 7 || A.bs == 3, PFG_E_UNSUPPORTED, "the symmetric product is built for 3x3 blocks");
    const int64_t n = A.ndof();
    const double bs2 = (double)(A.bs * A.bs);
    // algorithmic bytes: values and block columns once, row pointers (int64)
    // once, source vector once, result once -- padding slots are overhead
    const double idx = (double)A.nnzb * 4.0 + (double)(A.nb + 1) * 8.0;
    const bool f64 = kernel == 0 || kernel == 3 || kernel == 6;
    if (kernel == 4 && !A.v32_valid) make_v32(A, st);
    if (kernel <= 2 || kernel == 5 || kernel == 6) build_sell(A, f64, !f64, st);
    if (kernel >= 7) {
        build_sell_upper(A, st);
        y4_.ensure((size_t)A.nb * 4);
        PFG_CUDA(cudaMemsetAsync(y4_.p, 0, (size_t)A.nb * 4 * sizeof(float), st));
    }
    if (kernel == 10 || kernel == 12) {
        fx_.ensure((size_t)A.nb * 3);
        PFG_CUDA(cudaMemsetAsync(fx_.p, 0, (size_t)A.nb * 3 * sizeof(unsigned long long), st));
    }
    const int gv = grid_for(n, 256, sm_count() * 8);
    const int gb = row_grid(A.nb);
    DevBuf<double> x64, y64;
    DevBuf<float> x32, y32, p32, q32;
    KState hs;
    memset(&hs, 0, sizeof(hs));
    hs.rho32 = 1.0f;
    hs.xmax_bits = 0x3f800000u;  // max |x| = 1 (x is filled with ones)
    hs.beta32 = 0.5f;
    if (!state_.p) state_.alloc(1);
    if (!ticket_.p) {
        ticket_.alloc(1);
        PFG_CUDA(cudaMemsetAsync(ticket_.p, 0, sizeof(unsigned), st));
    }
    const int g0 = A.bs == 3 ? resident_grid(k_spmv_sell<3, double>, A.ns) : resident_grid(k_spmv_sell<1, double>, A.ns);
    const int g1 = A.bs == 3 ? resident_grid(k_spmv_sell<3, float>, A.ns) : resident_grid(k_spmv_sell<1, float>, A.ns);
    const int g2 = A.bs == 3 ? resident_grid(k_cg_spmv<3, float>, A.ns) : resident_grid(k_cg_spmv<1, float>, A.ns);
    const int g5 = A.bs == 3 ? resident_grid(k_cg_spmv_u<3, float>, A.ns) : resident_grid(k_cg_spmv_u<1, float>, A.ns);
    const int g6 = A.bs == 3 ? resident_grid(k_cg_spmv_u<3, double>, A.ns) : resident_grid(k_cg_spmv_u<1, double>, A.ns);
    partials_.ensure((size_t)sm_count() * (2048 / kThreads) * 4 + 8);
    partials32_.ensure((size_t)sm_count() * (2048 / kThreads) * 8 + 16);
    PFG_CUDA(cudaMemcpyAsync(state_.p, &hs, sizeof(KState), cudaMemcpyHostToDevice, st));
    auto launch = [&]() {
        switch (kernel) {
        case 0:
            if (A.bs == 3) k_spmv_sell<3, double><<<g0, kThreads, 0, st>>>(A.sell<double>(), x64.p, y64.p);
            else k_spmv_sell<1, double><<<g0, kThreads, 0, st>>>(A.sell<double>(), x64.p, y64.p);
            break;
        case 1:
            if (A.bs == 3) k_spmv_sell<3, float><<<g1, kThreads, 0, st>>>(A.sell<float>(), x32.p, y32.p);
            else k_spmv_sell<1, float><<<g1, kThreads, 0, st>>>(A.sell<float>(), x32.p, y32.p);
            break;
        case 2:
            if (A.bs == 3)
                k_cg_spmv<3, float><<<g2, kThreads, 0, st>>>(A.sell<float>(), x32.p, p32.p, y32.p, q32.p, state_.p,
                                                             partials_.p, partials32_.p, ticket_.p);
            else
                k_cg_spmv<1, float><<<g2, kThreads, 0, st>>>(A.sell<float>(), x32.p, p32.p, y32.p, q32.p, state_.p,
                                                             partials_.p, partials32_.p, ticket_.p);
            break;
        case 5:
            if (A.bs == 3)
                k_cg_spmv_u<3, float><<<g5, kThreads, 0, st>>>(A.sell<float>(), x32.p, y32.p, state_.p, partials_.p,
                                                               partials32_.p, ticket_.p);
            else
                k_cg_spmv_u<1, float><<<g5, kThreads, 0, st>>>(A.sell<float>(), x32.p, y32.p, state_.p, partials_.p,
                                                               partials32_.p, ticket_.p);
            break;
        case 6:
            if (A.bs == 3)
                k_cg_spmv_u<3, double><<<g6, kThreads, 0, st>>>(A.sell<double>(), x64.p, y64.p, state_.p, partials_.p,
                                                                partials32_.p, ticket_.p);
            else
                k_cg_spmv_u<1, double><<<g6, kThreads, 0, st>>>(A.sell<double>(), x64.p, y64.p, state_.p, partials_.p,
                                                                partials32_.p, ticket_.p);
            break;
        case 7:
            k_spmv_sym<<<resident_grid(k_spmv_sym, A.ns_u), kThreads, 0, st>>>(sell_upper(A), x32.p, y4_.p,
                                                                              nullptr);
            break;
        case 8:
            launch_cg_spmv_sym(false, sell_upper(A), nullptr, x32.p, nullptr, y4_.p, state_.p, partials_.p,
                               partials32_.p, ticket_.p, st);
            break;
        case 11:
            k_cg_spmv_sym_t<2, 4><<<resident_grid(k_cg_spmv_sym_t<2, 4>, A.ns_u), kThreads, 0, st>>>(
                sell_upper(A), x32.p, y4_.p, state_.p, partials_.p, partials32_.p, ticket_.p);
            break;
        case 10:  // (its finish pass, which adds and clears the transposes, is not part of the launch)
            launch_spmv_symfx(sell_upper(A), x32.p, y32.p, fx_.p, A.sym_rowsum, state_.p, st);
            break;
        case 12:
            k_spmv_symfx_t<1, 5><<<resident_grid(k_spmv_symfx_t<1, 5>, A.ns_u), kThreads, 0, st>>>(
                sell_upper(A), x32.p, y32.p, fx_.p, A.sym_rowsum, state_.p);
            break;
        case 3:
            if (A.bs == 3) k_spmv<3, double><<<gb, kThreads, 0, st>>>(A.view<double>(), x64.p, y64.p);
            else k_spmv<1, double><<<gb, kThreads, 0, st>>>(A.view<double>(), x64.p, y64.p);
            break;
        default:
            if (A.bs == 3) k_spmv<3, float><<<gb, kThreads, 0, st>>>(A.view<float>(), x32.p, y32.p);
            else k_spmv<1, float><<<gb, kThreads, 0, st>>>(A.view<float>(), x32.p, y32.p);
        }
    };
    if (f64) {
        x64.alloc((size_t)n);
        y64.alloc((size_t)n);
        k_fill<<<gv, 256, 0, st>>>(x64.p, n, 1.0);
        bytes = (double)A.nnzb * bs2 * 8.0 + idx + 2.0 * (double)n * 8.0;
    } else {
        x32.alloc((size_t)n);
        y32.alloc((size_t)n);
        k_fill<<<gv, 256, 0, st>>>(x32.p, n, 1.0f);
        bytes = (double)A.nnzb * bs2 * 4.0 + idx + 2.0 * (double)n * 4.0;
        if (kernel >= 7 && kernel != 9)  // the upper half: (nnzb + nb) / 2 blocks of a symmetric pattern
            bytes = (double)(A.nnzb + A.nb) / 2.0 * (bs2 * 4.0 + 4.0) + (double)(A.nb + 1) * 8.0 +
                    2.0 * (double)n * 4.0;
        if (kernel == 2) {
            p32.alloc((size_t)n);
            q32.alloc((size_t)n);
            k_fill<<<gv, 256, 0, st>>>(p32.p, n, 1.0f);
            bytes += 2.0 * (double)n * 4.0;  // p_old read, p_new write on top of the SpMV
        }
    }
    PFG_CUDA(cudaGetLastError());
    for (int w = 0; w < 3; ++w) launch();  // warm-up
    cudaEvent_t e0, e1;
    PFG_CUDA(cudaEventCreate(&e0));
    PFG_CUDA(cudaEventCreate(&e1));
    PFG_CUDA(cudaEventRecord(e0, st));
    for (int r = 0; r < reps; ++r) launch();
    PFG_CUDA(cudaEventRecord(e1, st));
    PFG_CUDA(cudaEventSynchronize(e1));
    PFG_CUDA(cudaGetLastError());
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ms = (double)t / reps;
    if (kernel == 2 || kernel == 5 || kernel == 6 || kernel == 8 || kernel == 11) {
        KState h;
        read_state(h, st);
        PFG_CHECK(!h.done, PFG_E_BREAKDOWN, "profiled CG SpMV hit p.Ap <= 0 (matrix not positive definite)");
    }
}

}  // namespace pfg
