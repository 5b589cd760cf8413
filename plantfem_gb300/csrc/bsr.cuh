// bsr.cuh -- the block-row matrix layout of the library and its row products.
//
// A matrix is stored as BS x BS blocks (BS = 3 for the 3-DOF elasticity
// systems assembled from hex8 meshes, BS = 1 for arbitrary scalar CRS
// matrices handed in by a caller).  It is the 3x3-BCRS re-layout of plantFEM's
// scalar CRS (FEMDomainClass.f90:10780-10836 expands a node graph into exactly
// such 3x3 blocks):
//
//   rp[nb+1]   int64  block-row pointer, 0-based
//   col[nnzb]  int32  block column (node id, 0-based) in first-appearance order
//   val[nnzb*BS*BS]   values; block row i occupies val[BS*BS*rp[i] ...) and is
//                     stored *transposed within the row*: entry (r, c) of the
//                     k-th block of the row sits at
//                        val[BS*BS*rp[i] + (r*BS + c) * nblk_i + k]
//
// The transposed-within-row order lets the warp that owns a block row read
// each of the BS*BS entry planes with one coalesced load instruction (lane k
// reads block k), with no per-value index arithmetic and no shuffles between
// loads; only the three row sums are reduced across the warp at the end.
#pragma once

#include "pfg_common.cuh"

namespace pfg {

template <typename T>
struct BsrView {
    int64_t nb;        // number of block rows (= block columns)
    int64_t nnzb;      // number of stored blocks
    const int64_t *rp;
    const int *col;
    const T *val;
};

// y[0..BS) = sum over the blocks of block row `row` of A(row, c) * src(c).
// Executed by a full warp; every lane returns the complete sums.
// Src: __device__ void operator()(int c, T (&x)[BS]) const, the BS source
// values of block column c (may compute them on the fly from several vectors).
template <int BS, typename T, typename Src>
__device__ __forceinline__ void bsr_row_product(const BsrView<T> &A, int64_t row, int lane, const Src &src,
                                                T (&y)[BS])
{
    const int64_t s = A.rp[row];
    const int nblk = (int)(A.rp[row + 1] - s);
    const T *v = A.val + s * (BS * BS);
#pragma unroll
    for (int r = 0; r < BS; ++r) y[r] = T(0);
    for (int b = lane; b < nblk; b += 32) {
        T a[BS * BS];
        const int c = ld_stream(A.col + s + b);
#pragma unroll
        for (int e = 0; e < BS * BS; ++e) a[e] = ld_stream(v + (int64_t)e * nblk + b);
        T xv[BS];
        src(c, xv);
#pragma unroll
        for (int r = 0; r < BS; ++r)
#pragma unroll
            for (int cc = 0; cc < BS; ++cc) y[r] = fma(a[r * BS + cc], xv[cc], y[r]);
    }
#pragma unroll
    for (int r = 0; r < BS; ++r) y[r] = warp_sum(y[r]);
}

// ------------------------------------------------------------- grid reduction
// Deterministic two-stage reduction of NV values: each CTA reduces its
// threads' values in a fixed tree, writes them to partials[blockIdx * NV + k],
// and the last CTA to arrive (atomic ticket) sums the partials in CTA order
// and runs `fin` with the totals on thread 0.  The ticket is reset for reuse.
struct GridTicket {
    unsigned int *counter;
};

template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double *smem /* >= NV * 32 */)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = warp_sum(v[k]);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) smem[k * 32 + wid] = v[k];
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double t = lane < nw ? smem[k * 32 + lane] : 0.0;
            v[k] = warp_sum(t);
        }
    }
}

template <int NV>
__device__ __forceinline__ void block_sum_comp(Comp32 (&v)[NV], float *smem /* >= 2 * NV * 32 */)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            float s2 = __shfl_xor_sync(0xffffffffu, v[k].s, o);
            float c2 = __shfl_xor_sync(0xffffffffu, v[k].c, o);
            comp_merge(v[k], s2, c2);
        }
    }
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            smem[(2 * k) * 32 + wid] = v[k].s;
            smem[(2 * k + 1) * 32 + wid] = v[k].c;
        }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            Comp32 t;
            t.s = lane < nw ? smem[(2 * k) * 32 + lane] : 0.f;
            t.c = lane < nw ? smem[(2 * k + 1) * 32 + lane] : 0.f;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                float s2 = __shfl_xor_sync(0xffffffffu, t.s, o);
                float c2 = __shfl_xor_sync(0xffffffffu, t.c, o);
                comp_merge(t, s2, c2);
            }
            v[k] = t;
        }
    }
}

// Returns true on thread 0 of the last CTA; totals[] then holds the grid sums.
template <int NV>
__device__ __forceinline__ bool grid_sum(double (&v)[NV], double *partials, unsigned int *counter,
                                         double (&totals)[NV])
{
    __shared__ double smem[NV * 32];
    __shared__ bool last;
    block_sum<NV>(v, smem);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) partials[(int64_t)blockIdx.x * NV + k] = v[k];
        __threadfence();
        unsigned int t = atomicAdd(counter, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return false;
    // last CTA: warp 0 sums partials in a fixed order
    __threadfence();
    if (threadIdx.x < 32) {
        double acc[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += 32)
#pragma unroll
            for (int k = 0; k < NV; ++k) acc[k] += *((volatile double *)&partials[(int64_t)b * NV + k]);
#pragma unroll
        for (int k = 0; k < NV; ++k) totals[k] = warp_sum(acc[k]);
    }
    if (threadIdx.x == 0) *counter = 0u;
    return threadIdx.x == 0;
}

template <int NV>
__device__ __forceinline__ bool grid_sum_comp(Comp32 (&v)[NV], float *partials, unsigned int *counter,
                                              float (&totals)[NV])
{
    __shared__ float smem[2 * NV * 32];
    __shared__ bool last;
    block_sum_comp<NV>(v, smem);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            partials[((int64_t)blockIdx.x * NV + k) * 2] = v[k].s;
            partials[((int64_t)blockIdx.x * NV + k) * 2 + 1] = v[k].c;
        }
        __threadfence();
        unsigned int t = atomicAdd(counter, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    if (threadIdx.x < 32) {
        Comp32 acc[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] = Comp32{0.f, 0.f};
        for (int b = threadIdx.x; b < (int)gridDim.x; b += 32)
#pragma unroll
            for (int k = 0; k < NV; ++k)
                comp_merge(acc[k], *((volatile float *)&partials[((int64_t)b * NV + k) * 2]),
                           *((volatile float *)&partials[((int64_t)b * NV + k) * 2 + 1]));
#pragma unroll
        for (int k = 0; k < NV; ++k) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                float s2 = __shfl_xor_sync(0xffffffffu, acc[k].s, o);
                float c2 = __shfl_xor_sync(0xffffffffu, acc[k].c, o);
                comp_merge(acc[k], s2, c2);
            }
            totals[k] = acc[k].s + acc[k].c;
        }
    }
    if (threadIdx.x == 0) *counter = 0u;
    return threadIdx.x == 0;
}

}  // namespace pfg
