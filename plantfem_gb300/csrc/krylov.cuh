// krylov.cuh -- device-resident CG / BiCGSTAB on the block-row layout.
//
// The host-level solver objects are declared here and implemented in
// krylov.cu; the FEMSolver handle (femsolver.cu) owns one of each.
#pragma once

#include <atomic>
#include <memory>

#include "bsr.cuh"
#include "sell.cuh"

namespace pfg {

// Scalars of one solve, resident in device memory.  Kernels read what they
// need at entry and the last CTA of each reduction writes the new values, so
// no scalar ever travels to the host inside the iteration loop.
struct KState {
    // FP64 recurrences
    double rho, rho_prev, alpha, beta, pq, rr, bb, rr1, c1, c2, c3, ev, vv;
    // FP32 recurrences of the mixed-precision inner iteration
    float rho32, alpha32, beta32, rr32, c1_32, c2_32, c3_32, rmax32, rmin32, r0r0_32;
    double true_rr;        // |b - A x|^2 in FP64 at the last residual replacement
    int iter;              // inner iterations done
    int done;              // 1 = stop (converged, breakdown or itrmax)
    int need_update;       // mixed: 1 = fold x32 into x64 and replace r
    int parity;            // which of the ping-pong buffers holds the current p
    int status;            // PFG_OK, PFG_E_BREAKDOWN, PFG_W_NOT_CONVERGED
    int replacements;      // mixed: number of FP64 residual replacements
    int breakdowns;        // mixed BiCGSTAB: FP32 breakdowns since the last completed iteration
    int poisoned;          // mixed: an FP32 update produced a non-finite value; drop x32
    unsigned xmax_bits;    // max |v| (float bits) of the vector the next fixed-point symmetric product reads
};

struct KConfig {
    int algorithm;     // PFG_ALG_*
    int precision;     // PFG_PREC_*
    int precond;       // PFG_PC_*
    int stop_rule;     // PFG_STOP_*
    int itrmax;
    double er0, relative_er, reliable_delta;
    int graph_chunk;
    int debug;
    int fuse;  // 1: vector updates ride in the SpMV gathers, 0: separate streaming passes
    int storage = 0;  // mixed: 0 full FP32 copy, 1 upper half of a symmetric matrix (PFG_STORAGE_*)
};

struct SolveResult {
    int status = PFG_OK;
    int iterations = 0;
    int replacements = 0;
    int launches = 0;  // kernels launched by the solve, inside graphs included
    double rel_residual = 0.0;
    double iter_residual = 0.0;
    double ms = 0.0;
    int fallback = 0;  // mixed: the FP32 inner iterations failed, finished in FP64
};

// Matrix owned on the device in the block-row layout.  v32 is the FP32 copy
// used by the mixed-precision inner iterations (built on demand).
struct DevMatrix {
    int bs = 3;
    int64_t nb = 0, nnzb = 0;
    DevBuf<int64_t> rp;
    DevBuf<int> col;
    DevBuf<double> v64;
    DevBuf<float> v32;
    bool v32_valid = false;
    // sliced-ELL copy read by the Krylov kernels (sell.cuh), rebuilt on demand
    int64_t ns = 0;
    DevBuf<int64_t> sptr;
    DevBuf<int> scol;
    DevBuf<double> s64;
    DevBuf<float> s32;
    bool sell_pattern = false, s64_valid = false, s32_valid = false;
    // Upper half (block column >= block row) of a symmetric 3x3-block matrix,
    // sliced like the full copy, FP32 values: the symmetric-storage inner
    // iterations read half the matrix bytes (sell.cu, krylov.cu k_spmv_sym).
    int64_t ns_u = 0;
    DevBuf<int64_t> sptr_u;
    DevBuf<int> scol_u;
    DevBuf<float> s32_u;
    bool sell_u_pattern = false, s32_u_valid = false;
    float sym_rowsum = 0.f;  // max over scalar rows of sum |a_ij| (FP32), set with s32_u

    // bumped whenever rp/col change: keys factors derived from the pattern
    uint64_t pattern_gen = 0;

    int64_t ndof() const { return nb * bs; }
    // v64 changed: every derived copy is stale
    void values_changed() { v32_valid = s64_valid = s32_valid = s32_u_valid = false; }
    // rp/col changed too
    void pattern_changed()
    {
        values_changed();
        sell_pattern = sell_u_pattern = false;
        pattern_gen = next_pattern_gen();
    }
    // process-wide counter: no two patterns (of any matrix) share a value
    static uint64_t next_pattern_gen()
    {
        static std::atomic<uint64_t> counter{0};
        return ++counter;
    }
    template <typename T>
    BsrView<T> view() const;
    template <typename T>
    SellView<T> sell() const;
};
template <>
inline BsrView<double> DevMatrix::view<double>() const { return BsrView<double>{nb, nnzb, rp.p, col.p, v64.p}; }
template <>
inline BsrView<float> DevMatrix::view<float>() const { return BsrView<float>{nb, nnzb, rp.p, col.p, v32.p}; }
template <>
inline SellView<double> DevMatrix::sell<double>() const { return SellView<double>{nb, ns, sptr.p, scol.p, s64.p}; }
template <>
inline SellView<float> DevMatrix::sell<float>() const { return SellView<float>{nb, ns, sptr.p, scol.p, s32.p}; }

// Build (or refresh) the sliced-ELL copy: pattern once, FP64 and/or FP32
// values when stale.  Implemented in sell.cu.
void build_sell(DevMatrix &A, bool want64, bool want32, cudaStream_t st);

// Build (or refresh) the FP32 upper-half sliced copy of a 3x3-block matrix;
// checks once per value change that the matrix is symmetric (blockwise, to
// 1e-9 relative) and throws PFG_E_ARG if it is not.  Implemented in sell.cu.
void build_sell_upper(DevMatrix &A, cudaStream_t st);
inline SellView<float> sell_upper(const DevMatrix &A)
{
    return SellView<float>{A.nb, A.ns_u, A.sptr_u.p, A.scol_u.p, A.s32_u.p};
}

// Inverse of every diagonal block (PFG_PC_BLOCK_JACOBI) or diagonal entry
// (PFG_PC_JACOBI) of A into d64 (and d32 unless null), BS*BS values per block
// row.  Implemented in krylov.cu.
void block_jacobi(const DevMatrix &A, int precond, double *d64, float *d32, cudaStream_t st);

class Ilu0;

inline bool is_ilu(int precond) { return precond == PFG_PC_ILU0 || precond == PFG_PC_ILU0_SORTED; }

class Krylov {
  public:
    Krylov();
    ~Krylov();
    // Solve A x = b (device vectors of length A.ndof()); x holds x0 on entry.
    SolveResult solve(DevMatrix &A, const double *b, double *x, const KConfig &cfg, cudaStream_t st);
    // y = A x in FP64 / FP32 (plain SpMV, used by the C ABI and the tests).
    static void spmv64(const DevMatrix &A, const double *x, double *y, cudaStream_t st);
    // y = A x in FP64 from the sliced copy (built on first use and kept while
    // the values stay): the form for a matrix that is applied many times.
    static void spmv64_sliced(DevMatrix &A, const double *x, double *y, cudaStream_t st);
    static void spmv32(const DevMatrix &A, const float *x, float *y, cudaStream_t st);
    static void make_v32(DevMatrix &A, cudaStream_t st);
    // Grid size used for the row loops (a multiple of the SM count).
    static int row_grid(int64_t nb);
    // Mean ms per launch of one kernel over `reps` launches (CUDA events on st)
    // and the algorithmic bytes of one launch.  kernel: 0 FP64 sliced SpMV,
    // 1 FP32 sliced SpMV, 2 FP32 CG SpMV with fused direction update (sliced),
    // 3 FP64 block-row SpMV, 4 FP32 block-row SpMV.
    void profile(DevMatrix &A, int kernel, int reps, cudaStream_t st, double &ms, double &bytes);
    // The ILU(0) factor kept for PFG_PC_ILU0* solves (ilu.cuh); factored from
    // A (if not held for A's pattern and this column order) by ilu_factor.
    const Ilu0 &ilu_factor(const DevMatrix &A, bool sorted, cudaStream_t st);
    // The factor held now (null if none).
    const Ilu0 *ilu_held() const;
    void ilu_reset();

  private:
    void prepare(const DevMatrix &A, const KConfig &cfg, cudaStream_t st);
    void build_precond(const DevMatrix &A, int precond, bool fp32, cudaStream_t st);
    SolveResult run_cg64(DevMatrix &A, const double *b, double *x, const KConfig &cfg, cudaStream_t st);
    SolveResult run_bicgstab64(DevMatrix &A, const double *b, double *x, const KConfig &cfg, cudaStream_t st);
    SolveResult run_mixed(DevMatrix &A, const double *b, double *x, const KConfig &cfg, cudaStream_t st);
    void read_state(KState &h, cudaStream_t st);
    // Hash of everything a captured chunk graph bakes in: every device pointer
    // its kernels receive and the configuration scalars.
    uint64_t graph_key(int kind, const DevMatrix &A, const void *x, const KConfig &cfg) const;
    double true_residual(const DevMatrix &A, const double *b, const double *x, double *r, cudaStream_t st);

    int64_t n_ = 0;
    int bs_ = 3;
    // FP64 work vectors
    DevBuf<double> r_, r0_, z_, pA_, pB_, q_, yA_, yB_, e_, v_, dinv_, ph_, eh_;
    DevBuf<double> xb_;  // mixed: x before the fold of an FP32 correction
    DevBuf<float> y4_;   // symmetric storage: 4-per-row product accumulator (CG)
    DevBuf<unsigned long long> fx_;  // symmetric storage: fixed-point transposes, 3 planes of nb (BiCGSTAB)
    // FP32 work vectors
    DevBuf<float> r32_, r032_, z32_, pA32_, pB32_, q32_, yA32_, yB32_, e32_, v32_, x32_, dinv32_, ph32_, eh32_;
    DevBuf<double> partials_;
    DevBuf<float> partials32_;
    DevBuf<unsigned int> ticket_;
    DevBuf<KState> state_;
    KState *host_state_ = nullptr;  // pinned mirror
    // cached CUDA graphs of one chunk of iterations
    cudaGraphExec_t graph_ = nullptr;
    uint64_t graph_key_ = 0;
    int graph_kernels_ = 0;  // kernels captured in graph_
    std::unique_ptr<Ilu0> ilu_;
    int launches_ = 0;       // launch count of the current solve
};

}  // namespace pfg
