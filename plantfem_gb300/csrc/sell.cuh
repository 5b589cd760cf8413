// sell.cuh -- sliced-ELL copy of the 3x3-block matrix for the Krylov loop.
//
// Block rows are grouped in slices of 32 consecutive rows (one warp, one lane
// per block row).  A slice is padded to the longest row in it and stored
// "slot-major": for slot k of slice s, the 32 block columns are contiguous,
// and so are the 32 values of each of the BS*BS block entries:
//
//   sptr[ns+1]                    int64  first slot of each slice
//   col[(sptr[s] + k) * 32 + l]   int32  block column of slot k of row 32 s + l
//   val[((sptr[s] + k) * BS*BS + e) * 32 + l]   entry e = r*BS + c of that block
//
// Padding slots point at the row itself with zero values.  A warp therefore
// reads every value plane with one fully coalesced 128-byte (FP32) or
// 256-byte (FP64) load, each lane owns its block row's BS sums (no shuffles),
// and the 10 loads of a slot are independent of each other, so a thread keeps
// many loads in flight.  The copy is built from the block-row (BCRS) layout on
// the device; BCRS stays the layout of assembly, elimination and CRS export.
#pragma once

#include "pfg_common.cuh"

namespace pfg {

template <typename T>
struct SellView {
    int64_t nb;   // block rows
    int64_t ns;   // slices
    const int64_t *sptr;
    const int *col;
    const T *val;
};

// Lane `lane` of the warp that owns slice s: y[0..BS) = row (32 s + lane) of
// A times src.  Src as in bsr_row_product.
template <int BS, typename T, typename Src>
__device__ __forceinline__ void sell_row_product(const SellView<T> &A, int64_t s, int lane, const Src &src,
                                                 T (&y)[BS])
{
    const int64_t b0 = A.sptr[s];
    const int w = (int)(A.sptr[s + 1] - b0);
    const int *cp = A.col + b0 * 32 + lane;
    const T *vp = A.val + b0 * 32 * (BS * BS) + lane;
#pragma unroll
    for (int r = 0; r < BS; ++r) y[r] = T(0);
#pragma unroll 3
    for (int k = 0; k < w; ++k) {
        T a[BS * BS];
        const int c = ld_stream(cp + (int64_t)k * 32);
#pragma unroll
        for (int e = 0; e < BS * BS; ++e) a[e] = ld_stream(vp + ((int64_t)k * (BS * BS) + e) * 32);
        T xv[BS];
        src(c, xv);
#pragma unroll
        for (int r = 0; r < BS; ++r)
#pragma unroll
            for (int cc = 0; cc < BS; ++cc) y[r] = fma(a[r * BS + cc], xv[cc], y[r]);
    }
}

}  // namespace pfg
