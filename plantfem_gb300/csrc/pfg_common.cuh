// pfg_common.cuh -- shared definitions of the plantfem_gb300 CUDA library.
//
// Error model: every entry point of the C ABI returns an int status (PFG_OK or
// a negative PFG_E* code) and never exits the process; the message of the
// last failure on the calling thread is kept for pfg_last_error().
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "pfg.h"

namespace pfg {

// Raised inside the library, turned into a status code at the C boundary.
struct Error : public std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string &msg);

#define PFG_CUDA(call)                                                                        \
    do {                                                                                      \
        cudaError_t _e = (call);                                                              \
        if (_e != cudaSuccess) {                                                              \
            throw ::pfg::Error(PFG_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e) + \
                                               " (" + __FILE__ + ":" + std::to_string(__LINE__) + ")"); \
        }                                                                                     \
    } while (0)

#define PFG_CHECK(cond, code, msg)                        \
    do {                                                  \
        if (!(cond)) throw ::pfg::Error((code), (msg));   \
    } while (0)

// Wraps a C-ABI body: converts exceptions into status codes.
template <typename F>
int guard(F &&f)
{
    try {
        f();
        return PFG_OK;
    } catch (const Error &e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::bad_alloc &) {
        set_last_error("host allocation failed");
        return PFG_E_NOMEM;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return PFG_E_INTERNAL;
    }
}

// Owning device buffer (cudaMalloc / cudaFree), movable, not copyable.
template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    explicit DevBuf(size_t count) { alloc(count); }
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    DevBuf &operator=(DevBuf &&o) noexcept
    {
        if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
        return *this;
    }
    ~DevBuf() { release(); }
    void alloc(size_t count)
    {
        release();
        if (count == 0) return;
        cudaError_t e = cudaMalloc((void **)&p, count * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            (void)cudaGetLastError();
            throw Error(PFG_E_NOMEM, "cudaMalloc of " + std::to_string(count * sizeof(T)) + " bytes failed: " +
                                         cudaGetErrorString(e));
        }
        n = count;
    }
    void ensure(size_t count)
    {
        if (n < count) alloc(count);
    }
    // Exactly `count` elements; keeps the allocation (and its address) when
    // the size is unchanged, so captured CUDA graphs stay valid.
    void resize(size_t count)
    {
        if (n != count) alloc(count);
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    size_t bytes() const { return n * sizeof(T); }
    T *get() const { return p; }
};

// Streaming multiprocessors of the current device (cached per device).
inline int sm_count_device()
{
    static int cache[64] = {0};
    int dev = 0;
    PFG_CUDA(cudaGetDevice(&dev));
    PFG_CHECK(dev >= 0 && dev < 64, PFG_E_UNSUPPORTED, "device ordinal above 63");
    if (cache[dev] == 0) {
        int v = 0;
        PFG_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev));
        cache[dev] = v > 0 ? v : 1;
    }
    return cache[dev];
}

// Blocks for `work` items, at most `cap` (default: 16 per SM of the device).
inline int grid_for(int64_t work, int per_block, int cap = 0)
{
    if (cap <= 0) cap = sm_count_device() * 16;
    int64_t g = (work + per_block - 1) / per_block;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (int)g;
}

// ---------------------------------------------------------------- device utils
template <typename T>
__device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Streaming load of matrix data that is read once per sweep: read-only path,
// not allocated in L1, so L1 keeps the gathered source vector.
__device__ __forceinline__ float ld_stream(const float *p)
{
    float v;
    asm("ld.global.nc.L1::no_allocate.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ double ld_stream(const double *p)
{
    double v;
    asm("ld.global.nc.L1::no_allocate.f64 %0, [%1];" : "=d"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ int ld_stream(const int *p)
{
    int v;
    asm("ld.global.nc.L1::no_allocate.s32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

// Error-free transformation of a sum (Knuth TwoSum), used by the compensated
// FP32 dot products (Ogita, Rump & Oishi, "Accurate sum and dot product",
// SIAM J. Sci. Comput. 26(6), 2005).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    // explicit round-to-nearest intrinsics: no contraction into FMA allowed here
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (hi, lo) pair accumulator for Dot2: products split exactly with FMA.
struct Comp32 {
    float s, c;
};
__device__ __forceinline__ void comp_add_prod(Comp32 &acc, float a, float b)
{
    float p = __fmul_rn(a, b);
    float pe = fmaf(a, b, -p);  // exact low part of a*b
    float s, e;
    two_sum(acc.s, p, s, e);
    acc.s = s;
    acc.c = __fadd_rn(acc.c, __fadd_rn(e, pe));
}
__device__ __forceinline__ void comp_merge(Comp32 &acc, float s2, float c2)
{
    float s, e;
    two_sum(acc.s, s2, s, e);
    acc.s = s;
    acc.c = __fadd_rn(acc.c, __fadd_rn(e, c2));
}

}  // namespace pfg
