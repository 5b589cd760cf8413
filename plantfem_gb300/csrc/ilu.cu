// ilu.cu -- level-scheduled ILU(0) factorization and D^-1 L^-1 sweep.
#include <algorithm>
#include <climits>

#include "ilu.cuh"

namespace pfg {

namespace {

constexpr int kIluWarps = 4;  // warps (block rows) per CTA

// Warp-private working set of the factorization: the block row being
// factored, the entries of one earlier block row K at this row's block
// columns, the two rows' block columns and the visiting order.
template <int BS>
struct IluRow {
    double rowv[kIluMaxBlocks * BS * BS];
    double kv[kIluMaxBlocks * BS * BS];
    int cols[kIluMaxBlocks];
    int kcols[kIluMaxBlocks];
    int seq[kIluMaxBlocks];
};

// ILUCRS(0) (SparseClass.f90:1629-1792) for the block rows of one level.
// Scalar row i = BS*I + d visits its entries k < i in turn (stored order, or
// ascending column order when `sorted`):
//     l = a(i,k) / U(k,k);  a(i,k) = l;  a(i,j) -= l * a(k,j) for j > k in row i,
// a(k,j) being 0 where row k stores no entry j.  Rows k of earlier block rows
// are final (earlier levels).  The rows d of this block row are independent
// until the diagonal block: the entries before it in visiting order are
// processed for all d at once (one load of each row K's entries), the rest
// row after row, since row d's steps against the diagonal block need rows
// e < d complete.  Values live in shared memory in the matrix's layout:
// entry (r, c) of block b at [(r*BS + c) * nb_I + b].
template <int BS>
__global__ void __launch_bounds__(32 * kIluWarps)
    k_ilu_factor(const int64_t *__restrict__ rp, const int *__restrict__ col, double *lu, double *udiag,
                 const int *__restrict__ order, int64_t start, int count, int sorted)
{
    constexpr int BB = BS * BS;
    __shared__ IluRow<BS> sm_all[kIluWarps];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int idx = blockIdx.x * kIluWarps + w;
    if (idx >= count) return;  // the whole warp leaves together
    IluRow<BS> &sm = sm_all[w];
    const int I = order[start + idx];
    const int64_t base = rp[I];
    const int nbI = (int)(rp[I + 1] - base);
    if (nbI > kIluMaxBlocks) return;  // refused on the host before any launch
    double *gI = lu + BB * base;
    for (int t = lane; t < nbI * BB; t += 32) sm.rowv[t] = gI[t];
    for (int b = lane; b < nbI; b += 32) sm.cols[b] = col[base + b];
    __syncwarp();
    for (int b = lane; b < nbI; b += 32) {
        int r = b;
        if (sorted) {
            const int c = sm.cols[b];
            r = 0;
            for (int q = 0; q < nbI; ++q) {
                const int cq = sm.cols[q];
                r += (cq < c) || (cq == c && q < b);
            }
        }
        sm.seq[r] = b;
    }
    __syncwarp();
    int pdiag = -1;
    for (int q = 0; q < nbI; ++q)
        if (sm.cols[sm.seq[q]] == I) {
            pdiag = q;
            break;
        }

    // kv <- row K's values at this row's block columns (0 where K has none)
    auto load_k = [&](int K) {
        const int64_t kb = rp[K];
        const int nbK = (int)(rp[K + 1] - kb);
        for (int t = lane; t < nbK; t += 32) sm.kcols[t] = col[kb + t];
        __syncwarp();
        const double *gK = lu + BB * kb;
        for (int b2 = lane; b2 < nbI; b2 += 32) {
            const int J = sm.cols[b2];
            int pos = -1;
            for (int q = 0; q < nbK; ++q)
                if (sm.kcols[q] == J) {
                    pos = q;
                    break;
                }
#pragma unroll
            for (int rc = 0; rc < BB; ++rc) sm.kv[rc * nbI + b2] = pos >= 0 ? gK[rc * nbK + pos] : 0.0;
        }
        __syncwarp();
    };
    // one k step of scalar row d: k = BS*K + e, stored as entry e of block b;
    // src holds row k's values at this row's columns, dk = U(k,k)
    auto step = [&](int d, int b, int K, int e, const double *src, double dk) {
        const int k = BS * K + e;
        const double l = sm.rowv[(d * BS + e) * nbI + b] / dk;
        __syncwarp();
        if (lane == 0) sm.rowv[(d * BS + e) * nbI + b] = l;
        for (int b2 = lane; b2 < nbI; b2 += 32) {
            const int J = sm.cols[b2];
#pragma unroll
            for (int e2 = 0; e2 < BS; ++e2)
                if (BS * J + e2 > k) {
                    // a + (-(l * a_kj)) rounded as written (no contraction),
                    // so the factor matches a serial restatement bit for bit
                    double &a = sm.rowv[(d * BS + e2) * nbI + b2];
                    a = __dadd_rn(a, -__dmul_rn(l, src[(e * BS + e2) * nbI + b2]));
                }
        }
        __syncwarp();
    };
    auto earlier_block = [&](int b, int K, int d_lo, int d_hi) {
        load_k(K);
        double dk[BS];
#pragma unroll
        for (int e = 0; e < BS; ++e) dk[e] = udiag[(int64_t)BS * K + e];
        for (int d = d_lo; d < d_hi; ++d)
#pragma unroll 1
            for (int e = 0; e < BS; ++e) step(d, b, K, e, sm.kv, dk[e]);
    };

    const int qend = pdiag >= 0 ? pdiag : nbI;
    for (int q = 0; q < qend; ++q) {
        const int b = sm.seq[q];
        const int K = sm.cols[b];
        if (K < I) earlier_block(b, K, 0, BS);
    }
    if (pdiag >= 0) {
        const int bd = sm.seq[pdiag];
        for (int d = 0; d < BS; ++d) {
            for (int e = 0; e < d; ++e) step(d, bd, I, e, sm.rowv, sm.rowv[(e * BS + e) * nbI + bd]);
            for (int q = pdiag + 1; q < nbI; ++q) {
                const int b = sm.seq[q];
                const int K = sm.cols[b];
                if (K < I) earlier_block(b, K, d, d + 1);
            }
        }
    }
    __syncwarp();
    for (int t = lane; t < nbI * BB; t += 32) gI[t] = sm.rowv[t];
    if (lane < BS)
        udiag[(int64_t)BS * I + lane] = pdiag >= 0 ? sm.rowv[(lane * BS + lane) * nbI + sm.seq[pdiag]] : 0.0;
}

// Sweep layout, built once per factor: the rows in level order, each with
// its blocks J < I (block columns, and values transposed within the row as in
// the matrix: entry (r, c) of block b at val[BB*off + (r*BS + c)*m + b]), and
// per row the strictly lower part of its diagonal block and 1 / U(i,i) (1 for
// a zero U(i,i), as ILU_matvecCRS reads it).  Each row then needs one load of
// its (I, m, off) before its values, instead of order -> row pointer ->
// block columns -> values.
template <int BS>
constexpr int diag_stride() { return BS == 3 ? 8 : 1; }  // [l10 l20 l21 r0 r1 r2 - -] or [r0]

// UPPER: the same layout for the backward solve, with the blocks J > I, the
// strictly upper part of the diagonal block ([u01 u02 u12 q0 q1 q2 - -] or
// [q0]) and q = 1 / U(i,i) as the reference divides (a zero U(i,i) gives inf).
template <int BS, bool UPPER>
__global__ void __launch_bounds__(32 * kIluWarps)
    k_ilu_sweep_layout(const int64_t *__restrict__ rp, const int *__restrict__ col, const double *__restrict__ lu,
                       const double *__restrict__ udiag, const int *__restrict__ order,
                       const int64_t *__restrict__ sw_off, int64_t nb, int2 *__restrict__ sw_row,
                       int *__restrict__ sw_col, double *__restrict__ sw_val, double *__restrict__ sw_diag)
{
    constexpr int BB = BS * BS, SD = diag_stride<BS>();
    const int lane = threadIdx.x & 31;
    const int64_t p = (int64_t)blockIdx.x * kIluWarps + (threadIdx.x >> 5);
    if (p >= nb) return;
    const int I = order[p];
    const int64_t base = rp[I];
    const int nbI = (int)(rp[I + 1] - base);
    const int64_t off = sw_off[p];
    const int m = (int)(sw_off[p + 1] - off);
    if (lane == 0) sw_row[p] = make_int2(I, m);
    int carry = 0;
    for (int b0 = 0; b0 < nbI; b0 += 32) {
        const int b = b0 + lane;
        const int J = b < nbI ? col[base + b] : (UPPER ? -1 : INT_MAX);
        const bool take = UPPER ? J > I : J < I;
        const unsigned sel = __ballot_sync(0xffffffffu, take);
        if (take) {
            const int r = carry + __popc(sel & ((1u << lane) - 1u));
            sw_col[off + r] = J;
#pragma unroll
            for (int rc = 0; rc < BB; ++rc) sw_val[BB * off + (int64_t)rc * m + r] = lu[BB * base + (int64_t)rc * nbI + b];
        } else if (J == I && BS == 3) {
            const int e0 = UPPER ? 0 * BS + 1 : 1 * BS + 0;
            const int e1 = UPPER ? 0 * BS + 2 : 2 * BS + 0;
            const int e2 = UPPER ? 1 * BS + 2 : 2 * BS + 1;
            sw_diag[SD * p + 0] = lu[BB * base + (int64_t)e0 * nbI + b];
            sw_diag[SD * p + 1] = lu[BB * base + (int64_t)e1 * nbI + b];
            sw_diag[SD * p + 2] = lu[BB * base + (int64_t)e2 * nbI + b];
        }
        carry += __popc(sel);
    }
    if (lane < BS) {
        const double d = udiag[(int64_t)BS * I + lane];
        sw_diag[SD * p + (BS == 3 ? 3 : 0) + lane] = UPPER ? 1.0 / d : (d == 0.0 ? 1.0 : 1.0 / d);
    }
}

// Lanes per block row in the sweep, and block slots a lane loads before the
// wait (rows with more than kSweepLanes * kSweepSlots blocks J < I load the
// rest after it).  GB300 runs a warp-wide FP64 instruction in 16 cycles of
// its SM's FP64 pipe, which the widest levels saturate: eight lanes per row
// (a structured hex mesh has 13 blocks J < I per row) keep most lanes of
// every FP64 instruction busy and cut the reduction to three rounds.
constexpr int kSweepLanes = 8;
constexpr int kSweepSlots = 2;
constexpr int kSweepRows = kIluWarps * 32 / kSweepLanes;  // block rows per CTA

// ILU_matvecCRS (SparseClass.f90:1795-1852) as executed, for the block rows
// of one level: t_i = v_i - sum_{k<i} L(i,k) t_k, out_i = t_i / U(i,i) (taken
// as 1 for a zero U(i,i)).  kSweepLanes lanes sum a row's blocks J < I, the
// first of them finishes the BS rows through the diagonal block's strictly
// lower part.
//
// Levels after the first of at most kIluEarlyRows block rows run as
// programmatically dependent grids: a level's grid is scheduled once every CTA
// of the level before it is past its own wait, loads what does not depend on
// that level (its row, block columns, factor values, v) and waits
// (griddepcontrol.wait: the previous grid complete, its writes visible) only
// before it reads t, through L2 (ld.global.cg).  The first level launches
// plainly, after the pass that wrote v.  Larger levels launch plainly too (the
// wait is then a no-op): early launch slowed the widest levels of a 100^3
// sweep (up to ~2500 block rows) in measurement.
template <int BS>
__global__ void __launch_bounds__(32 * kIluWarps)
    k_ilu_lower(const int2 *__restrict__ sw_row, const int64_t *__restrict__ sw_off, const int *__restrict__ sw_col,
                const double *__restrict__ sw_val, const double *__restrict__ sw_diag, int64_t start, int count,
                const double *v, double *t, double *out, const KState *S)
{
    constexpr int BB = BS * BS, SD = diag_stride<BS>();
    const int sub = threadIdx.x % kSweepLanes;
    const int idx = blockIdx.x * kSweepRows + threadIdx.x / kSweepLanes;
    const bool active = idx < count;  // the same for the row's lanes
    int I = 0, m = 0;
    int64_t off = 0;
    int J[kSweepSlots];
    double gv[kSweepSlots][BB];
    double dd[SD], vI[BS];
#pragma unroll
    for (int q = 0; q < kSweepSlots; ++q) J[q] = -1;
    if (active) {
        const int64_t p = start + idx;
        const int2 rm = sw_row[p];
        off = sw_off[p];
        I = rm.x;
        m = rm.y;
#pragma unroll
        for (int q = 0; q < kSweepSlots; ++q) {
            const int b = sub + kSweepLanes * q;
            if (b < m) {
                J[q] = sw_col[off + b];
#pragma unroll
                for (int rc = 0; rc < BB; ++rc) gv[q][rc] = sw_val[BB * off + (int64_t)rc * m + b];
            }
        }
        if (sub == 0) {
#pragma unroll
            for (int k = 0; k < SD; ++k) dd[k] = sw_diag[SD * p + k];
#pragma unroll
            for (int d = 0; d < BS; ++d) vI[d] = __ldcg(v + (int64_t)BS * I + d);
        }
    }
    asm volatile("griddepcontrol.wait;" ::: "memory");
    // only now may the next level's grid be scheduled: one level ahead at most
    asm volatile("griddepcontrol.launch_dependents;");
    if (S != nullptr && (S->done | S->need_update)) return;  // the same for the whole grid
    double acc[BS];
#pragma unroll
    for (int d = 0; d < BS; ++d) acc[d] = 0.0;
#pragma unroll
    for (int q = 0; q < kSweepSlots; ++q) {
        if (J[q] >= 0) {
            double tj[BS];
#pragma unroll
            for (int e = 0; e < BS; ++e) tj[e] = __ldcg(t + (int64_t)BS * J[q] + e);
#pragma unroll
            for (int d = 0; d < BS; ++d)
#pragma unroll
                for (int e = 0; e < BS; ++e) acc[d] = fma(gv[q][d * BS + e], tj[e], acc[d]);
        }
    }
    for (int b = sub + kSweepLanes * kSweepSlots; b < m; b += kSweepLanes) {
        const int Jb = sw_col[off + b];
        double tj[BS];
#pragma unroll
        for (int e = 0; e < BS; ++e) tj[e] = __ldcg(t + (int64_t)BS * Jb + e);
#pragma unroll
        for (int d = 0; d < BS; ++d)
#pragma unroll
            for (int e = 0; e < BS; ++e)
                acc[d] = fma(sw_val[BB * off + (int64_t)(d * BS + e) * m + b], tj[e], acc[d]);
    }
    // every lane takes part (inactive rows add zeros): xor partners stay in the row's lanes
#pragma unroll
    for (int o = kSweepLanes / 2; o > 0; o >>= 1) {
#pragma unroll
        for (int d = 0; d < BS; ++d) acc[d] += __shfl_xor_sync(0xffffffffu, acc[d], o);
    }
    if (active && sub == 0) {
        if constexpr (BS == 3) {
            const double t0 = vI[0] - acc[0];
            const double t1 = vI[1] - acc[1] - dd[0] * t0;
            const double t2 = vI[2] - acc[2] - dd[1] * t0 - dd[2] * t1;
            double *tr = t + (int64_t)3 * I, *orow = out + (int64_t)3 * I;
            tr[0] = t0;
            tr[1] = t1;
            tr[2] = t2;
            orow[0] = t0 * dd[3];
            orow[1] = t1 * dd[4];
            orow[2] = t2 * dd[5];
        } else {
            const double t0 = vI[0] - acc[0];
            t[I] = t0;
            out[I] = t0 * dd[0];
        }
    }
}

// The backward half of ILUCRS(0, RHS) (SparseClass.f90:1663-1677) for the block
// rows of one level of the upper dependency order, in place on x (which holds
// y_i / U(i,i) from the forward sweep): x_i -= (sum_{j>i} U(i,j) x_j) / U(i,i).
// Same lane layout and launch scheme as k_ilu_lower; x_j (j > i) is final
// from earlier levels, read through L2 after the wait.
template <int BS>
__global__ void __launch_bounds__(32 * kIluWarps)
    k_ilu_upper(const int2 *__restrict__ sw_row, const int64_t *__restrict__ sw_off, const int *__restrict__ sw_col,
                const double *__restrict__ sw_val, const double *__restrict__ sw_diag, int64_t start, int count,
                double *x)
{
    constexpr int BB = BS * BS, SD = diag_stride<BS>();
    const int sub = threadIdx.x % kSweepLanes;
    const int idx = blockIdx.x * kSweepRows + threadIdx.x / kSweepLanes;
    const bool active = idx < count;
    int I = 0, m = 0;
    int64_t off = 0;
    int J[kSweepSlots];
    double gv[kSweepSlots][BB];
    double dd[SD], yI[BS];
#pragma unroll
    for (int q = 0; q < kSweepSlots; ++q) J[q] = -1;
    if (active) {
        const int64_t p = start + idx;
        const int2 rm = sw_row[p];
        off = sw_off[p];
        I = rm.x;
        m = rm.y;
#pragma unroll
        for (int q = 0; q < kSweepSlots; ++q) {
            const int b = sub + kSweepLanes * q;
            if (b < m) {
                J[q] = sw_col[off + b];
#pragma unroll
                for (int rc = 0; rc < BB; ++rc) gv[q][rc] = sw_val[BB * off + (int64_t)rc * m + b];
            }
        }
        if (sub == 0) {
#pragma unroll
            for (int k = 0; k < SD; ++k) dd[k] = sw_diag[SD * p + k];
#pragma unroll
            for (int d = 0; d < BS; ++d) yI[d] = __ldcg(x + (int64_t)BS * I + d);  // from the forward sweep
        }
    }
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;");
    double acc[BS];
#pragma unroll
    for (int d = 0; d < BS; ++d) acc[d] = 0.0;
#pragma unroll
    for (int q = 0; q < kSweepSlots; ++q) {
        if (J[q] >= 0) {
            double xj[BS];
#pragma unroll
            for (int e = 0; e < BS; ++e) xj[e] = __ldcg(x + (int64_t)BS * J[q] + e);
#pragma unroll
            for (int d = 0; d < BS; ++d)
#pragma unroll
                for (int e = 0; e < BS; ++e) acc[d] = fma(gv[q][d * BS + e], xj[e], acc[d]);
        }
    }
    for (int b = sub + kSweepLanes * kSweepSlots; b < m; b += kSweepLanes) {
        const int Jb = sw_col[off + b];
        double xj[BS];
#pragma unroll
        for (int e = 0; e < BS; ++e) xj[e] = __ldcg(x + (int64_t)BS * Jb + e);
#pragma unroll
        for (int d = 0; d < BS; ++d)
#pragma unroll
            for (int e = 0; e < BS; ++e)
                acc[d] = fma(sw_val[BB * off + (int64_t)(d * BS + e) * m + b], xj[e], acc[d]);
    }
#pragma unroll
    for (int o = kSweepLanes / 2; o > 0; o >>= 1) {
#pragma unroll
        for (int d = 0; d < BS; ++d) acc[d] += __shfl_xor_sync(0xffffffffu, acc[d], o);
    }
    if (active && sub == 0) {
        if constexpr (BS == 3) {
            const double x2 = yI[2] - acc[2] * dd[5];
            const double x1 = yI[1] - (acc[1] + dd[2] * x2) * dd[4];
            const double x0 = yI[0] - (acc[0] + dd[0] * x1 + dd[1] * x2) * dd[3];
            double *xr = x + (int64_t)3 * I;
            xr[0] = x0;
            xr[1] = x1;
            xr[2] = x2;
        } else {
            x[I] = yI[0] - acc[0] * dd[0];
        }
    }
}

// Levels of at most this many block rows launch early (see k_ilu_lower).
constexpr int kIluEarlyRows = 1024;

// One level of the sweep on st, programmatically dependent when it is not
// the first and is small.
template <int BS>
void launch_lower(int grid, bool early, const int2 *sw_row, const int64_t *sw_off, const int *sw_col,
                  const double *sw_val, const double *sw_diag, int64_t start, int count, const double *v, double *t,
                  double *out, const KState *S, cudaStream_t st)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(32 * kIluWarps);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = early ? 1 : 0;
    PFG_CUDA(cudaLaunchKernelEx(&cfg, k_ilu_lower<BS>, sw_row, sw_off, sw_col, sw_val, sw_diag, start, count, v, t,
                                out, S));
}

// One level of the backward sweep, launched like launch_lower.
template <int BS>
void launch_upper(int grid, bool early, const int2 *sw_row, const int64_t *sw_off, const int *sw_col,
                  const double *sw_val, const double *sw_diag, int64_t start, int count, double *x, cudaStream_t st)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(32 * kIluWarps);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = early ? 1 : 0;
    PFG_CUDA(cudaLaunchKernelEx(&cfg, k_ilu_upper<BS>, sw_row, sw_off, sw_col, sw_val, sw_diag, start, count, x));
}

int ilu_grid(int64_t count) { return (int)((count + kIluWarps - 1) / kIluWarps); }

}  // namespace

void Ilu0::factor(const DevMatrix &A, bool sorted, cudaStream_t st)
{
    PFG_CHECK(A.nb > 0 && (A.bs == 1 || A.bs == 3), PFG_E_STATE, "ILU(0): no matrix");
    if (ready_ && sorted == sorted_ && A.pattern_gen == pattern_gen_ && A.bs == bs_ && A.nb == nb_ &&
        A.nnzb == nnzb_ && A.rp.p == rp_ && A.col.p == col_)
        return;
    ready_ = false;
    // levels from the block pattern (host pass, once per pattern)
    std::vector<int64_t> rp((size_t)A.nb + 1);
    std::vector<int> col((size_t)std::max<int64_t>(A.nnzb, 1));
    PFG_CUDA(cudaMemcpyAsync(rp.data(), A.rp.p, rp.size() * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    PFG_CUDA(cudaMemcpyAsync(col.data(), A.col.p, (size_t)A.nnzb * sizeof(int), cudaMemcpyDeviceToHost, st));
    PFG_CUDA(cudaStreamSynchronize(st));
    std::vector<int> lvl((size_t)A.nb);
    int nl = 0;
    for (int64_t I = 0; I < A.nb; ++I) {
        PFG_CHECK(rp[I + 1] - rp[I] <= kIluMaxBlocks, PFG_E_UNSUPPORTED,
                  "ILU(0): a row stores more than 64 blocks");
        int L = 0;
        for (int64_t q = rp[I]; q < rp[I + 1]; ++q)
            if (col[q] < I) L = std::max(L, lvl[col[q]] + 1);
        lvl[I] = L;
        nl = std::max(nl, L + 1);
    }
    lptr_.assign((size_t)nl + 1, 0);
    for (int64_t I = 0; I < A.nb; ++I) ++lptr_[(size_t)lvl[I] + 1];
    for (int L = 0; L < nl; ++L) lptr_[L + 1] += lptr_[L];
    std::vector<int> order((size_t)A.nb);
    {
        std::vector<int64_t> fill(lptr_.begin(), lptr_.end() - 1);
        for (int64_t I = 0; I < A.nb; ++I) order[(size_t)fill[lvl[I]]++] = (int)I;
    }
    const int64_t n = A.ndof();
    order_.resize((size_t)A.nb);
    lu_.resize(A.v64.n);
    udiag_.resize((size_t)n);
    t_.resize((size_t)n);
    PFG_CUDA(cudaMemcpyAsync(order_.p, order.data(), order.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    PFG_CUDA(cudaMemcpyAsync(lu_.p, A.v64.p, A.v64.bytes(), cudaMemcpyDeviceToDevice, st));
    PFG_CUDA(cudaMemsetAsync(udiag_.p, 0, (size_t)n * sizeof(double), st));
    for (int L = 0; L < nl; ++L) {
        const int64_t cnt = lptr_[L + 1] - lptr_[L];
        if (A.bs == 3)
            k_ilu_factor<3><<<ilu_grid(cnt), 32 * kIluWarps, 0, st>>>(A.rp.p, A.col.p, lu_.p, udiag_.p, order_.p,
                                                                     lptr_[L], (int)cnt, sorted ? 1 : 0);
        else
            k_ilu_factor<1><<<ilu_grid(cnt), 32 * kIluWarps, 0, st>>>(A.rp.p, A.col.p, lu_.p, udiag_.p, order_.p,
                                                                     lptr_[L], (int)cnt, sorted ? 1 : 0);
    }
    PFG_CUDA(cudaGetLastError());
    // the sweep layout: rows in level order with their blocks J < I
    std::vector<int64_t> off((size_t)A.nb + 1, 0);
    for (int64_t q = 0; q < A.nb; ++q) {
        const int I = order[(size_t)q];
        int m = 0;
        for (int64_t k = rp[I]; k < rp[I + 1]; ++k) m += col[k] < I;
        off[(size_t)q + 1] = off[(size_t)q] + m;
    }
    const int64_t nlow = off[(size_t)A.nb];
    sw_off_.resize((size_t)A.nb + 1);
    sw_row_.resize((size_t)A.nb);
    sw_col_.resize((size_t)std::max<int64_t>(nlow, 1));
    sw_val_.resize((size_t)std::max<int64_t>(nlow * A.bs * A.bs, 1));
    sw_diag_.resize((size_t)A.nb * (A.bs == 3 ? 8 : 1));
    PFG_CUDA(cudaMemcpyAsync(sw_off_.p, off.data(), off.size() * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    // a row without a stored diagonal block keeps zero lower entries there
    PFG_CUDA(cudaMemsetAsync(sw_diag_.p, 0, sw_diag_.bytes(), st));
    if (A.bs == 3)
        k_ilu_sweep_layout<3, false><<<ilu_grid(A.nb), 32 * kIluWarps, 0, st>>>(A.rp.p, A.col.p, lu_.p, udiag_.p, order_.p,
                                                                        sw_off_.p, A.nb, sw_row_.p, sw_col_.p,
                                                                        sw_val_.p, sw_diag_.p);
    else
        k_ilu_sweep_layout<1, false><<<ilu_grid(A.nb), 32 * kIluWarps, 0, st>>>(A.rp.p, A.col.p, lu_.p, udiag_.p, order_.p,
                                                                        sw_off_.p, A.nb, sw_row_.p, sw_col_.p,
                                                                        sw_val_.p, sw_diag_.p);
    PFG_CUDA(cudaGetLastError());
    // backward solve (ILUCRS with RHS): levels of the upper dependencies
    // (row I waits for the rows J > I it stores) and the same layout of its
    // blocks J > I
    {
        std::vector<int> ulvl((size_t)A.nb);
        int nu = 0;
        for (int64_t I = A.nb - 1; I >= 0; --I) {
            int L = 0;
            for (int64_t q = rp[I]; q < rp[I + 1]; ++q)
                if (col[q] > I) L = std::max(L, ulvl[col[q]] + 1);
            ulvl[I] = L;
            nu = std::max(nu, L + 1);
        }
        uptr_.assign((size_t)nu + 1, 0);
        for (int64_t I = 0; I < A.nb; ++I) ++uptr_[(size_t)ulvl[I] + 1];
        for (int L = 0; L < nu; ++L) uptr_[L + 1] += uptr_[L];
        std::vector<int> uorder((size_t)A.nb);
        std::vector<int64_t> fill(uptr_.begin(), uptr_.end() - 1);
        for (int64_t I = A.nb - 1; I >= 0; --I) uorder[(size_t)fill[ulvl[I]]++] = (int)I;
        std::vector<int64_t> uoff((size_t)A.nb + 1, 0);
        for (int64_t q = 0; q < A.nb; ++q) {
            const int I = uorder[(size_t)q];
            int m = 0;
            for (int64_t k = rp[I]; k < rp[I + 1]; ++k) m += col[k] > I;
            uoff[(size_t)q + 1] = uoff[(size_t)q] + m;
        }
        const int64_t nup = uoff[(size_t)A.nb];
        uorder_.resize((size_t)A.nb);
        su_off_.resize((size_t)A.nb + 1);
        su_row_.resize((size_t)A.nb);
        su_col_.resize((size_t)std::max<int64_t>(nup, 1));
        su_val_.resize((size_t)std::max<int64_t>(nup * A.bs * A.bs, 1));
        su_diag_.resize((size_t)A.nb * (A.bs == 3 ? 8 : 1));
        PFG_CUDA(cudaMemcpyAsync(uorder_.p, uorder.data(), uorder.size() * sizeof(int), cudaMemcpyHostToDevice, st));
        PFG_CUDA(cudaMemcpyAsync(su_off_.p, uoff.data(), uoff.size() * sizeof(int64_t), cudaMemcpyHostToDevice, st));
        PFG_CUDA(cudaMemsetAsync(su_diag_.p, 0, su_diag_.bytes(), st));
        if (A.bs == 3)
            k_ilu_sweep_layout<3, true><<<ilu_grid(A.nb), 32 * kIluWarps, 0, st>>>(
                A.rp.p, A.col.p, lu_.p, udiag_.p, uorder_.p, su_off_.p, A.nb, su_row_.p, su_col_.p, su_val_.p,
                su_diag_.p);
        else
            k_ilu_sweep_layout<1, true><<<ilu_grid(A.nb), 32 * kIluWarps, 0, st>>>(
                A.rp.p, A.col.p, lu_.p, udiag_.p, uorder_.p, su_off_.p, A.nb, su_row_.p, su_col_.p, su_val_.p,
                su_diag_.p);
        PFG_CUDA(cudaGetLastError());
    }
    PFG_CUDA(cudaStreamSynchronize(st));
    sweep_bytes_ = (double)nlow * (A.bs * A.bs * 8.0 + 4.0) +
                   (double)A.nb * (8.0 + 8.0 + 8.0 * (A.bs == 3 ? 8 : 1)) + 4.0 * (double)n * 8.0;
    bs_ = A.bs;
    nb_ = A.nb;
    nnzb_ = A.nnzb;
    rp_ = A.rp.p;
    col_ = A.col.p;
    pattern_gen_ = A.pattern_gen;
    sorted_ = sorted;
    ++gen_;
    ready_ = true;
}

void Ilu0::solve(const double *rhs, double *x, cudaStream_t st) const
{
    apply(rhs, x, nullptr, st);  // x = D'^-1 L^-1 rhs (D' = U's diagonal, 0 read as 1)
    const int nu = (int)uptr_.size() - 1;
    for (int L = 0; L < nu; ++L) {
        const int64_t cnt = uptr_[L + 1] - uptr_[L];
        const bool early = L > 0 && cnt <= kIluEarlyRows;
        const int grid = (int)((cnt + kSweepRows - 1) / kSweepRows);
        if (bs_ == 3)
            launch_upper<3>(grid, early, su_row_.p, su_off_.p, su_col_.p, su_val_.p, su_diag_.p, uptr_[L], (int)cnt,
                            x, st);
        else
            launch_upper<1>(grid, early, su_row_.p, su_off_.p, su_col_.p, su_val_.p, su_diag_.p, uptr_[L], (int)cnt,
                            x, st);
    }
    PFG_CUDA(cudaGetLastError());
}

int Ilu0::apply(const double *v, double *out, const KState *S, cudaStream_t st) const
{
    PFG_CHECK(ready_, PFG_E_STATE, "ILU(0): not factored");
    const int nl = levels();
    for (int L = 0; L < nl; ++L) {
        const int64_t cnt = lptr_[L + 1] - lptr_[L];
        const bool early = L > 0 && cnt <= kIluEarlyRows;
        const int grid = (int)((cnt + kSweepRows - 1) / kSweepRows);
        if (bs_ == 3)
            launch_lower<3>(grid, early, sw_row_.p, sw_off_.p, sw_col_.p, sw_val_.p, sw_diag_.p, lptr_[L],
                            (int)cnt, v, t_.p, out, S, st);
        else
            launch_lower<1>(grid, early, sw_row_.p, sw_off_.p, sw_col_.p, sw_val_.p, sw_diag_.p, lptr_[L],
                            (int)cnt, v, t_.p, out, S, st);
    }
    PFG_CUDA(cudaGetLastError());
    return nl;
}

}  // namespace pfg
