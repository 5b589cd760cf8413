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

// ------------------------------------------------- upper half (symmetric storage)
// width of each slice = most upper blocks (column >= row) of a row in it
__global__ void k_sellu_widths(int64_t nb, int64_t ns, const int64_t *__restrict__ rp, const int *__restrict__ bcol,
                               int64_t *__restrict__ width)
{
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += (int64_t)gridDim.x * blockDim.x) {
        int64_t w = 0;
        for (int l = 0; l < 32; ++l) {
            const int64_t row = s * 32 + l;
            if (row >= nb) break;
            int64_t c = 0;
            for (int64_t k = rp[row]; k < rp[row + 1]; ++k) c += bcol[k] >= row;
            w = max(w, c);
        }
        width[s] = w;
    }
}

// columns (and FP32 values) of the upper blocks of each row, in the row's
// order; padding slots point at the row itself with zero values
__global__ void k_sellu_fill(int64_t nb, int64_t ns, const int64_t *__restrict__ rp, const int *__restrict__ bcol,
                             const double *__restrict__ v64, const int64_t *__restrict__ sptr, int *__restrict__ scol,
                             float *__restrict__ sval)
{
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < ns * 32; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = t >> 5;
        const int l = (int)(t & 31);
        const int64_t row = t;
        const int64_t b0 = sptr[s], w = sptr[s + 1] - b0;
        const int64_t r0 = row < nb ? rp[row] : 0;
        const int64_t nblk = row < nb ? rp[row + 1] - r0 : 0;
        const int self = row < nb ? (int)row : 0;
        int64_t slot = 0;
        for (int64_t k = 0; k < nblk; ++k) {
            const int c = bcol[r0 + k];
            if (c < row) continue;
            scol[(b0 + slot) * 32 + l] = c;
            for (int e = 0; e < 9; ++e)
                sval[((b0 + slot) * 9 + e) * 32 + l] = (float)v64[r0 * 9 + (int64_t)e * nblk + k];
            ++slot;
        }
        for (; slot < w; ++slot) {
            scol[(b0 + slot) * 32 + l] = self;
            for (int e = 0; e < 9; ++e) sval[((b0 + slot) * 9 + e) * 32 + l] = 0.f;
        }
    }
}

// Counts the upper blocks (i, j) whose transpose partner (j, i) is missing or
// differs by more than 1e-9 relative (plus 1e-12 of the diagonal scale of the
// two rows: assembly rounding leaves noise in entries that cancel to zero).
__global__ void k_sym_check(int64_t nb, const int64_t *__restrict__ rp, const int *__restrict__ bcol,
                            const double *__restrict__ v64, unsigned long long *__restrict__ bad)
{
    auto entry = [&](int64_t row, int64_t k, int e) {
        const int64_t r0 = rp[row];
        return v64[r0 * 9 + (int64_t)e * (rp[row + 1] - r0) + k];
    };
    auto diag_scale = [&](int64_t row) {
        double m = 0.0;
        for (int64_t k = rp[row]; k < rp[row + 1]; ++k)
            if (bcol[k] == row)
                for (int e = 0; e < 9; e += 4) m = fmax(m, fabs(entry(row, k - rp[row], e)));
        return m;
    };
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += (int64_t)gridDim.x * blockDim.x) {
        const double di = diag_scale(i);
        for (int64_t k = rp[i]; k < rp[i + 1]; ++k) {
            const int64_t j = bcol[k];
            if (j <= i) continue;
            int64_t kk = -1;
            for (int64_t q = rp[j]; q < rp[j + 1]; ++q)
                if (bcol[q] == i) {
                    kk = q - rp[j];
                    break;
                }
            if (kk < 0) {
                atomicAdd(bad, 1ull);
                continue;
            }
            const double scale = 1e-12 * fmax(di, diag_scale(j));
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) {
                    const double a = entry(i, k - rp[i], 3 * r + c), b = entry(j, kk, 3 * c + r);
                    if (!(fabs(a - b) <= 1e-9 * fmax(fabs(a), fabs(b)) + scale)) {
                        atomicAdd(bad, 1ull);
                        r = 3;
                        break;
                    }
                }
        }
    }
}

void build_sell_upper(DevMatrix &A, cudaStream_t st)
{
    PFG_CHECK(A.nb > 0, PFG_E_STATE, "empty matrix");
    PFG_CHECK(A.bs == 3, PFG_E_UNSUPPORTED, "symmetric storage is built for 3x3-block matrices");
    if (A.sell_u_pattern && A.s32_u_valid) return;
    const int g = grid_for(A.nb, 256, 152 * 16);
    // the values (pattern included) changed: check the symmetry once
    {
        DevBuf<unsigned long long> bad(1);
        PFG_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(unsigned long long), st));
        k_sym_check<<<g, 256, 0, st>>>(A.nb, A.rp.p, A.col.p, A.v64.p, bad.p);
        PFG_CUDA(cudaGetLastError());
        unsigned long long nbad = 0;
        PFG_CUDA(cudaMemcpyAsync(&nbad, bad.p, sizeof nbad, cudaMemcpyDeviceToHost, st));
        PFG_CUDA(cudaStreamSynchronize(st));
        PFG_CHECK(nbad == 0, PFG_E_ARG,
                  "symmetric storage needs a symmetric matrix: " + std::to_string(nbad) +
                      " blocks differ from their transposes");
    }
    if (!A.sell_u_pattern) {
        A.ns_u = (A.nb + 31) / 32;
        DevBuf<int64_t> width((size_t)A.ns_u + 1);
        PFG_CUDA(cudaMemsetAsync(width.p, 0, (A.ns_u + 1) * sizeof(int64_t), st));
        k_sellu_widths<<<grid_for(A.ns_u, 256, 152 * 16), 256, 0, st>>>(A.nb, A.ns_u, A.rp.p, A.col.p, width.p);
        PFG_CUDA(cudaGetLastError());
        A.sptr_u.resize((size_t)A.ns_u + 1);
        const int64_t slots = exclusive_scan(width.p, A.sptr_u.p, A.ns_u + 1, st);
        A.scol_u.resize((size_t)std::max<int64_t>(slots * 32, 1));
        A.s32_u.resize((size_t)std::max<int64_t>(slots * 32 * 9, 1));
        A.sell_u_pattern = true;
    }
    k_sellu_fill<<<g, 256, 0, st>>>(A.nb, A.ns_u, A.rp.p, A.col.p, A.v64.p, A.sptr_u.p, A.scol_u.p, A.s32_u.p);
    PFG_CUDA(cudaGetLastError());
    A.s32_u_valid = true;
}

}  // namespace pfg
