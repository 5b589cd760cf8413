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

// ILU_matvecCRS (SparseClass.f90:1795-1852) as executed, for the block rows
// of one level: t_i = v_i - sum_{k<i} L(i,k) t_k, out_i = t_i / U(i,i) (1 for
// a zero U(i,i)).  The lanes sum the blocks J < I, lane 0 finishes the BS
// rows through the diagonal block's strictly lower part.
//
// Small levels run as a chain of programmatically dependent launches: a
// level's grid is scheduled once every CTA of the level before it is past its
// own wait, loads what does not depend on that level (its rows, block columns
// and factor entries) and waits (griddepcontrol.wait: the previous grid
// complete and its writes visible) only before it reads v and t.  t is read
// through L2 (ld.global.cg).  Large levels launch plainly (the wait is then a
// no-op): measured on GB300, early launch cut a 60^3 sweep (levels of <= ~900
// block rows) from 3.87 to 2.85 ms but slowed the 100^3 one (levels of up to
// ~2500) from 8.66 to 9.47 ms.
template <int BS>
__global__ void __launch_bounds__(32 * kIluWarps)
    k_ilu_lower(const int64_t *__restrict__ rp, const int *__restrict__ col, const double *__restrict__ lu,
                const double *__restrict__ udiag, const int *__restrict__ order, int64_t start, int count,
                const double *v, double *t, double *out, const KState *S)
{
    constexpr int BB = BS * BS;
    constexpr int NS = kIluMaxBlocks / 32;  // block slots per lane
    const int lane = threadIdx.x & 31;
    const int idx = blockIdx.x * kIluWarps + (threadIdx.x >> 5);
    const bool active = idx < count;  // the same for the whole warp
    int I = 0, bd = -1;
    int J[NS];
    double gv[NS][BB];
    double ld[BS > 1 ? BS * BS : 1], dg[BS];
    if (active) {
        I = order[start + idx];
        const int64_t base = rp[I];
        const int nbI = (int)(rp[I + 1] - base);
        const double *g = lu + BB * base;
#pragma unroll
        for (int q = 0; q < NS; ++q) {
            const int b = lane + 32 * q;
            J[q] = b < nbI ? col[base + b] : INT_MAX;
            if (J[q] < I) {
#pragma unroll
                for (int rc = 0; rc < BB; ++rc) gv[q][rc] = g[rc * nbI + b];
            } else if (J[q] == I) {
                bd = b;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) bd = max(bd, __shfl_xor_sync(0xffffffffu, bd, o));
        if (lane == 0) {
#pragma unroll
            for (int d = 0; d < BS; ++d) {
                dg[d] = udiag[(int64_t)BS * I + d];
#pragma unroll
                for (int e = 0; e < d; ++e) ld[d * BS + e] = bd >= 0 ? g[(d * BS + e) * nbI + bd] : 0.0;
            }
        }
    }
    asm volatile("griddepcontrol.wait;" ::: "memory");
    // only now may the next level's grid be scheduled: one level ahead at most
    asm volatile("griddepcontrol.launch_dependents;");
    if (!active) return;
    if (S != nullptr && (S->done | S->need_update)) return;
    double acc[BS];
#pragma unroll
    for (int d = 0; d < BS; ++d) acc[d] = 0.0;
#pragma unroll
    for (int q = 0; q < NS; ++q) {
        if (J[q] < I) {
            double tj[BS];
#pragma unroll
            for (int e = 0; e < BS; ++e) tj[e] = __ldcg(t + (int64_t)BS * J[q] + e);
#pragma unroll
            for (int d = 0; d < BS; ++d)
#pragma unroll
                for (int e = 0; e < BS; ++e) acc[d] = fma(gv[q][d * BS + e], tj[e], acc[d]);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int d = 0; d < BS; ++d) acc[d] += __shfl_xor_sync(0xffffffffu, acc[d], o);
    }
    if (lane == 0) {
        double tv[BS];
#pragma unroll
        for (int d = 0; d < BS; ++d) {
            double s = __ldcg(v + (int64_t)BS * I + d) - acc[d];
#pragma unroll
            for (int e = 0; e < d; ++e) s -= ld[d * BS + e] * tv[e];
            tv[d] = s;
            t[(int64_t)BS * I + d] = s;
            out[(int64_t)BS * I + d] = s / (dg[d] == 0.0 ? 1.0 : dg[d]);
        }
    }
}

// Levels of at most this many block rows launch early (see k_ilu_lower).
constexpr int kIluEarlyRows = 1024;

// One level of the sweep on st, programmatically dependent when it is small.
template <int BS>
void launch_lower(int grid, const int64_t *rp, const int *col, const double *lu, const double *udiag,
                  const int *order, int64_t start, int count, const double *v, double *t, double *out,
                  const KState *S, cudaStream_t st)
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
    cfg.numAttrs = count <= kIluEarlyRows ? 1 : 0;
    PFG_CUDA(cudaLaunchKernelEx(&cfg, k_ilu_lower<BS>, rp, col, lu, udiag, order, start, count, v, t, out, S));
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
    int64_t lower = 0;
    for (int64_t I = 0; I < A.nb; ++I) {
        PFG_CHECK(rp[I + 1] - rp[I] <= kIluMaxBlocks, PFG_E_UNSUPPORTED,
                  "ILU(0): a row stores more than 64 blocks");
        int L = 0;
        for (int64_t q = rp[I]; q < rp[I + 1]; ++q) {
            if (col[q] < I) L = std::max(L, lvl[col[q]] + 1);
            lower += col[q] <= I;
        }
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
    sweep_bytes_ = (double)lower * (A.bs * A.bs * 8.0 + 4.0) + (double)A.nb * (8.0 + 4.0) + 5.0 * (double)n * 8.0;
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
    PFG_CUDA(cudaStreamSynchronize(st));
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

int Ilu0::apply(const double *v, double *out, const KState *S, cudaStream_t st) const
{
    PFG_CHECK(ready_, PFG_E_STATE, "ILU(0): not factored");
    const int nl = levels();
    for (int L = 0; L < nl; ++L) {
        const int64_t cnt = lptr_[L + 1] - lptr_[L];
        if (bs_ == 3)
            launch_lower<3>(ilu_grid(cnt), rp_, col_, lu_.p, udiag_.p, order_.p, lptr_[L], (int)cnt, v, t_.p, out, S,
                            st);
        else
            launch_lower<1>(ilu_grid(cnt), rp_, col_, lu_.p, udiag_.p, order_.p, lptr_[L], (int)cnt, v, t_.p, out, S,
                            st);
    }
    PFG_CUDA(cudaGetLastError());
    return nl;
}

}  // namespace pfg
