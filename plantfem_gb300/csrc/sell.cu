// sell.cu -- block-row (BCRS) -> sliced-ELL conversion on the device.
#include "assembly.cuh"

namespace pfg {

// width of each slice = longest block row in it
__global__ void k_sell_widths(int64_t nb, int64_t ns, const int64_t *__restrict__ rp, int64_t *__restrict__ width)
{
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += (int64_t)gridDim.x * blockDim.x) {
        int64_t w = 0;
        for (int l = 0; l < 32; ++l) {
            const int64_t row = s * 32 + l;
            if (row < nb) w = max(w, rp[row + 1] - rp[row]);
        }
        width[s] = w;
    }
}

// one thread per (slice, lane): block columns, padding points at the row itself
__global__ void k_sell_pattern(int64_t nb, int64_t ns, const int64_t *__restrict__ rp, const int *__restrict__ bcol,
                               const int64_t *__restrict__ sptr, int *__restrict__ scol)
{
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < ns * 32; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = t >> 5;
        const int l = (int)(t & 31);
        const int64_t row = t;
        const int64_t b0 = sptr[s], w = sptr[s + 1] - b0;
        const int64_t r0 = row < nb ? rp[row] : 0;
        const int64_t nblk = row < nb ? rp[row + 1] - r0 : 0;
        const int self = row < nb ? (int)row : 0;
        for (int64_t k = 0; k < w; ++k) scol[(b0 + k) * 32 + l] = k < nblk ? bcol[r0 + k] : self;
    }
}

template <int BS, typename T>
__global__ void k_sell_values(int64_t nb, int64_t ns, const int64_t *__restrict__ rp, const double *__restrict__ v64,
                              const int64_t *__restrict__ sptr, T *__restrict__ sval)
{
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < ns * 32; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = t >> 5;
        const int l = (int)(t & 31);
        const int64_t row = t;
        const int64_t b0 = sptr[s], w = sptr[s + 1] - b0;
        const int64_t r0 = row < nb ? rp[row] : 0;
        const int64_t nblk = row < nb ? rp[row + 1] - r0 : 0;
        const double *src = v64 + r0 * (BS * BS);
        for (int64_t k = 0; k < w; ++k)
#pragma unroll
            for (int e = 0; e < BS * BS; ++e)
                sval[((b0 + k) * (BS * BS) + e) * 32 + l] = k < nblk ? (T)src[(int64_t)e * nblk + k] : T(0);
    }
}

void build_sell(DevMatrix &A, bool want64, bool want32, cudaStream_t st)
{
    PFG_CHECK(A.nb > 0, PFG_E_STATE, "empty matrix");
    const int g = grid_for(A.nb, 256, 152 * 16);
    if (!A.sell_pattern) {
        A.ns = (A.nb + 31) / 32;
        DevBuf<int64_t> width((size_t)A.ns + 1);
        PFG_CUDA(cudaMemsetAsync(width.p, 0, (A.ns + 1) * sizeof(int64_t), st));
        k_sell_widths<<<grid_for(A.ns, 256, 152 * 16), 256, 0, st>>>(A.nb, A.ns, A.rp.p, width.p);
        PFG_CUDA(cudaGetLastError());
        A.sptr.resize((size_t)A.ns + 1);
        const int64_t slots = exclusive_scan(width.p, A.sptr.p, A.ns + 1, st);
        A.scol.resize((size_t)std::max<int64_t>(slots * 32, 1));
        k_sell_pattern<<<g, 256, 0, st>>>(A.nb, A.ns, A.rp.p, A.col.p, A.sptr.p, A.scol.p);
        PFG_CUDA(cudaGetLastError());
        A.sell_pattern = true;
        A.s64_valid = A.s32_valid = false;
    }
    int64_t slots = 0;
    PFG_CUDA(cudaMemcpyAsync(&slots, A.sptr.p + A.ns, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    PFG_CUDA(cudaStreamSynchronize(st));
    const size_t nv = (size_t)std::max<int64_t>(slots * 32 * A.bs * A.bs, 1);
    if (want64 && !A.s64_valid) {
        A.s64.resize(nv);
        if (A.bs == 3)
            k_sell_values<3, double><<<g, 256, 0, st>>>(A.nb, A.ns, A.rp.p, A.v64.p, A.sptr.p, A.s64.p);
        else
            k_sell_values<1, double><<<g, 256, 0, st>>>(A.nb, A.ns, A.rp.p, A.v64.p, A.sptr.p, A.s64.p);
        PFG_CUDA(cudaGetLastError());
        A.s64_valid = true;
    }
    if (want32 && !A.s32_valid) {
        A.s32.resize(nv);
        if (A.bs == 3)
            k_sell_values<3, float><<<g, 256, 0, st>>>(A.nb, A.ns, A.rp.p, A.v64.p, A.sptr.p, A.s32.p);
        else
            k_sell_values<1, float><<<g, 256, 0, st>>>(A.nb, A.ns, A.rp.p, A.v64.p, A.sptr.p, A.s32.p);
        PFG_CUDA(cudaGetLastError());
        A.s32_valid = true;
    }
}

}  // namespace pfg
