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

// Slice values, one warp per slice (lane = row of the slice), one entry plane
// (r, c) and up to kTileK slots at a time through shared memory: each row's
// plane is read as one contiguous run of its blocks (block row layout,
// bsr.cuh) and written back slot by slot as 32 consecutive lanes.
constexpr int kTileK = 64;
constexpr int kTileWarps = 2;

template <int BS, typename T>
__global__ void __launch_bounds__(32 * kTileWarps)
    k_sell_values(int64_t nb, int64_t ns, const int64_t *__restrict__ rp, const double *__restrict__ v64,
                  const int64_t *__restrict__ sptr, T *__restrict__ sval)
{
    constexpr int BB = BS * BS;
    __shared__ T tile[kTileWarps][32][kTileK + 1];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int64_t s = (int64_t)blockIdx.x * kTileWarps + w; s < ns; s += (int64_t)gridDim.x * kTileWarps) {
        const int64_t b0 = sptr[s];
        const int wdt = (int)(sptr[s + 1] - b0);
        const int64_t row = s * 32 + lane;
        const int64_t r0 = row < nb ? rp[row] : 0;
        const int nblk = row < nb ? (int)(rp[row + 1] - r0) : 0;
        for (int e = 0; e < BB; ++e)
            for (int kc = 0; kc < wdt; kc += kTileK) {
                for (int l = 0; l < 32; ++l) {
                    const int64_t r0l = __shfl_sync(0xffffffffu, r0, l);
                    const int nl = __shfl_sync(0xffffffffu, nblk, l);
                    for (int kk = lane; kk < kTileK; kk += 32) {
                        const int k = kc + kk;
                        tile[w][l][kk] = k < nl ? (T)v64[r0l * BB + (int64_t)e * nl + k] : T(0);
                    }
                }
                __syncwarp();
                const int kend = min(kTileK, wdt - kc);
                for (int kk = 0; kk < kend; ++kk) sval[((b0 + kc + kk) * BB + e) * 32 + lane] = tile[w][lane][kk];
                __syncwarp();
            }
    }
}

static int tile_grid(int64_t ns) { return (int)std::min<int64_t>((ns + kTileWarps - 1) / kTileWarps, sm_count_device() * 32); }

void build_sell(DevMatrix &A, bool want64, bool want32, cudaStream_t st)
{
    PFG_CHECK(A.nb > 0, PFG_E_STATE, "empty matrix");
    const int g = grid_for(A.nb, 256, sm_count_device() * 16);
    if (!A.sell_pattern) {
        A.ns = (A.nb + 31) / 32;
        DevBuf<int64_t> width((size_t)A.ns + 1);
        PFG_CUDA(cudaMemsetAsync(width.p, 0, (A.ns + 1) * sizeof(int64_t), st));
        k_sell_widths<<<grid_for(A.ns, 256, sm_count_device() * 16), 256, 0, st>>>(A.nb, A.ns, A.rp.p, width.p);
        PFG_CUDA(cudaGetLastError());
        A.sptr.resize((size_t)A.ns + 1);
        const int64_t slots = exclusive_scan(width.p, A.sptr.p, A.ns + 1, st);
        A.scol.resize((size_t)std::max<int64_t>(slots * 32, 1));
        k_sell_pattern<<<g, 256, 0, st>>>(A.nb, A.ns, A.rp.p, A.col.p, A.sptr.p, A.scol.p);
        PFG_CUDA(cudaGetLastError());
        A.sell_pattern = true;
        A.s64_valid = A.s32_valid = false;
    }
    if (!(want64 && !A.s64_valid) && !(want32 && !A.s32_valid)) return;  // up to date: no host round trip
    int64_t slots = 0;
    PFG_CUDA(cudaMemcpyAsync(&slots, A.sptr.p + A.ns, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    PFG_CUDA(cudaStreamSynchronize(st));
    const size_t nv = (size_t)std::max<int64_t>(slots * 32 * A.bs * A.bs, 1);
    if (want64 && !A.s64_valid) {
        A.s64.resize(nv);
        if (A.bs == 3)
            k_sell_values<3, double><<<tile_grid(A.ns), 32 * kTileWarps, 0, st>>>(A.nb, A.ns, A.rp.p, A.v64.p,
                                                                               A.sptr.p, A.s64.p);
        else
            k_sell_values<1, double><<<tile_grid(A.ns), 32 * kTileWarps, 0, st>>>(A.nb, A.ns, A.rp.p, A.v64.p,
                                                                               A.sptr.p, A.s64.p);
        PFG_CUDA(cudaGetLastError());
        A.s64_valid = true;
    }
    if (want32 && !A.s32_valid) {
        A.s32.resize(nv);
        if (A.bs == 3)
            k_sell_values<3, float><<<tile_grid(A.ns), 32 * kTileWarps, 0, st>>>(A.nb, A.ns, A.rp.p, A.v64.p,
                                                                              A.sptr.p, A.s32.p);
        else
            k_sell_values<1, float><<<tile_grid(A.ns), 32 * kTileWarps, 0, st>>>(A.nb, A.ns, A.rp.p, A.v64.p,
                                                                              A.sptr.p, A.s32.p);
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

// Columns and FP32 values of the upper blocks (column >= row) of each row, in
// the row's order; padding slots point at the row itself with zero values.
// One warp per slice, kTileK slots at a time: per row, the ballot prefix of
// "upper" over its blocks gives each upper block its slot (kept in shared
// memory), then each entry plane is gathered row by row and written back slot
// by slot as 32 consecutive lanes.
__global__ void __launch_bounds__(32 * kTileWarps)
    k_sellu_fill(int64_t nb, int64_t ns, const int64_t *__restrict__ rp, const int *__restrict__ bcol,
                 const double *__restrict__ v64, const int64_t *__restrict__ sptr, int *__restrict__ scol,
                 float *__restrict__ sval)
{
    __shared__ short kmap[kTileWarps][32][kTileK];
    __shared__ int ucnt[kTileWarps][32];
    __shared__ float tile[kTileWarps][32][kTileK + 1];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int64_t s = (int64_t)blockIdx.x * kTileWarps + w; s < ns; s += (int64_t)gridDim.x * kTileWarps) {
        const int64_t b0 = sptr[s];
        const int wdt = (int)(sptr[s + 1] - b0);
        const int64_t row = s * 32 + lane;
        const int64_t r0 = row < nb ? rp[row] : 0;
        const int nblk = row < nb ? (int)(rp[row + 1] - r0) : 0;
        for (int kc = 0; kc < wdt; kc += kTileK) {
            // slots [kc, kc + kTileK) of every row: which of its blocks fill them
            for (int l = 0; l < 32; ++l) {
                const int64_t r0l = __shfl_sync(0xffffffffu, r0, l);
                const int nl = __shfl_sync(0xffffffffu, nblk, l);
                const int64_t rowl = s * 32 + l;
                int base = 0;
                for (int k0 = 0; k0 < nl; k0 += 32) {
                    const int k = k0 + lane;
                    const bool up = k < nl && bcol[r0l + k] >= rowl;
                    const unsigned bal = __ballot_sync(0xffffffffu, up);
                    const int pos = base + __popc(bal & ((1u << lane) - 1u)) - kc;
                    if (up && pos >= 0 && pos < kTileK) kmap[w][l][pos] = (short)k;
                    base += __popc(bal);
                }
                if (lane == 0) ucnt[w][l] = min(max(base - kc, 0), kTileK);
            }
            __syncwarp();
            const int kend = min(kTileK, wdt - kc);
            const int mine = ucnt[w][lane];
            for (int kk = 0; kk < kend; ++kk)
                scol[(b0 + kc + kk) * 32 + lane] = kk < mine ? bcol[r0 + kmap[w][lane][kk]] : (row < nb ? (int)row : 0);
            for (int e = 0; e < 9; ++e) {
                for (int l = 0; l < 32; ++l) {
                    const int64_t r0l = __shfl_sync(0xffffffffu, r0, l);
                    const int nl = __shfl_sync(0xffffffffu, nblk, l);
                    const int cl = ucnt[w][l];
                    for (int kk = lane; kk < kTileK; kk += 32)
                        tile[w][l][kk] = kk < cl ? (float)v64[r0l * 9 + (int64_t)e * nl + kmap[w][l][kk]] : 0.f;
                }
                __syncwarp();
                for (int kk = 0; kk < kend; ++kk) sval[((b0 + kc + kk) * 9 + e) * 32 + lane] = tile[w][lane][kk];
                __syncwarp();
            }
        }
    }
}

// Counts the upper blocks (i, j) whose transpose partner (j, i) is missing or
// differs by more than 1e-9 relative (plus 1e-12 of the diagonal scale of the
// two rows: assembly rounding leaves noise in entries that cancel to zero).
// One warp per row i, a lane per block (i, j): the lane finds (j, i) and row
// j's diagonal block in one pass over row j's block columns.
__global__ void k_sym_check(int64_t nb, const int64_t *__restrict__ rp, const int *__restrict__ bcol,
                            const double *__restrict__ v64, unsigned long long *__restrict__ bad)
{
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = w0; i < nb; i += nw) {
        const int64_t ri = rp[i];
        const int ni = (int)(rp[i + 1] - ri);
        // |diagonal entries| of row i's diagonal block
        double di = 0.0;
        for (int k = lane; k < ni; k += 32)
            if (bcol[ri + k] == i)
                for (int e = 0; e < 9; e += 4) di = fmax(di, fabs(v64[ri * 9 + (int64_t)e * ni + k]));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) di = fmax(di, __shfl_xor_sync(0xffffffffu, di, o));
        unsigned long long nbad = 0;
        for (int k = lane; k < ni; k += 32) {
            const int64_t j = bcol[ri + k];
            if (j <= i) continue;
            const int64_t rj = rp[j];
            const int nj = (int)(rp[j + 1] - rj);
            int kk = -1;
            double dj = 0.0;
            for (int q = 0; q < nj; ++q) {
                const int64_t c = bcol[rj + q];
                if (c == i && kk < 0) kk = q;
                if (c == j)
                    for (int e = 0; e < 9; e += 4) dj = fmax(dj, fabs(v64[rj * 9 + (int64_t)e * nj + q]));
            }
            if (kk < 0) {
                ++nbad;
                continue;
            }
            const double scale = 1e-12 * fmax(di, dj);
            bool ok = true;
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const double a = v64[ri * 9 + (int64_t)(3 * r + c) * ni + k];
                    const double b = v64[rj * 9 + (int64_t)(3 * c + r) * nj + kk];
                    ok = ok && fabs(a - b) <= 1e-9 * fmax(fabs(a), fabs(b)) + scale;
                }
            nbad += !ok;
        }
        if (nbad) atomicAdd(bad, nbad);
    }
}

// max over scalar rows of sum_j |a_ij| (as FP32 bits), a warp per block row:
// the bound the fixed-point symmetric product sizes its quantum from.
__global__ void k_rowsum_max(int64_t nb, const int64_t *__restrict__ rp, const double *__restrict__ v64,
                             unsigned *__restrict__ out)
{
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    float best = 0.f;
    for (int64_t i = w0; i < nb; i += nw) {
        const int64_t r0 = rp[i];
        const int n = (int)(rp[i + 1] - r0);
        float sum[3] = {0.f, 0.f, 0.f};
        for (int k = lane; k < n; k += 32)
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int c = 0; c < 3; ++c) sum[r] += fabsf((float)v64[r0 * 9 + (int64_t)(3 * r + c) * n + k]);
#pragma unroll
        for (int r = 0; r < 3; ++r) best = fmaxf(best, warp_sum(sum[r]));
    }
    if (lane == 0) atomicMax(out, __float_as_uint(best));
}

void build_sell_upper(DevMatrix &A, cudaStream_t st)
{
    PFG_CHECK(A.nb > 0, PFG_E_STATE, "empty matrix");
    PFG_CHECK(A.bs == 3, PFG_E_UNSUPPORTED, "symmetric storage is built for 3x3-block matrices");
    if (A.sell_u_pattern && A.s32_u_valid) return;
    const int g = grid_for(A.nb, 256, sm_count_device() * 16);
    // the values (pattern included) changed: check the symmetry once
    {
        DevBuf<unsigned long long> bad(2);  // [0] asymmetric blocks, [1] low word: row-sum bound bits
        PFG_CUDA(cudaMemsetAsync(bad.p, 0, 2 * sizeof(unsigned long long), st));
        k_sym_check<<<g, 256, 0, st>>>(A.nb, A.rp.p, A.col.p, A.v64.p, bad.p);
        k_rowsum_max<<<g, 256, 0, st>>>(A.nb, A.rp.p, A.v64.p, reinterpret_cast<unsigned *>(bad.p + 1));
        PFG_CUDA(cudaGetLastError());
        unsigned long long hb[2] = {0, 0};
        PFG_CUDA(cudaMemcpyAsync(hb, bad.p, sizeof hb, cudaMemcpyDeviceToHost, st));
        PFG_CUDA(cudaStreamSynchronize(st));
        const unsigned long long nbad = hb[0];
        const unsigned rs_bits = (unsigned)(hb[1] & 0xffffffffull);  // little-endian low word
        memcpy(&A.sym_rowsum, &rs_bits, sizeof rs_bits);
        PFG_CHECK(nbad == 0, PFG_E_ARG,
                  "symmetric storage needs a symmetric matrix: " + std::to_string(nbad) +
                      " blocks differ from their transposes");
    }
    if (!A.sell_u_pattern) {
        A.ns_u = (A.nb + 31) / 32;
        DevBuf<int64_t> width((size_t)A.ns_u + 1);
        PFG_CUDA(cudaMemsetAsync(width.p, 0, (A.ns_u + 1) * sizeof(int64_t), st));
        k_sellu_widths<<<grid_for(A.ns_u, 256, sm_count_device() * 16), 256, 0, st>>>(A.nb, A.ns_u, A.rp.p, A.col.p, width.p);
        PFG_CUDA(cudaGetLastError());
        A.sptr_u.resize((size_t)A.ns_u + 1);
        const int64_t slots = exclusive_scan(width.p, A.sptr_u.p, A.ns_u + 1, st);
        A.scol_u.resize((size_t)std::max<int64_t>(slots * 32, 1));
        A.s32_u.resize((size_t)std::max<int64_t>(slots * 32 * 9, 1));
        A.sell_u_pattern = true;
    }
    k_sellu_fill<<<tile_grid(A.ns_u), 32 * kTileWarps, 0, st>>>(A.nb, A.ns_u, A.rp.p, A.col.p, A.v64.p, A.sptr_u.p,
                                                               A.scol_u.p, A.s32_u.p);
    PFG_CUDA(cudaGetLastError());
    A.s32_u_valid = true;
}

}  // namespace pfg
