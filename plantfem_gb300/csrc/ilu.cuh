// ilu.cuh -- ILU(0) preconditioner of BiCGSTAB (preconditioning="ILU").
//
// plantFEM's FEMSolver_%solve(preconditioning="ILU" | "incompleteLU")
// (FEMSolverClass.f90:1777-1784) runs bicgstab_CRS_ILU
// (LinearSolverClass.f90:4104-4230): BiCGSTAB right-preconditioned by the
// ILU(0) factor of the eliminated matrix (ILUCRS, SparseClass.f90:1629-1792),
// applied by ILU_matvecCRS (SparseClass.f90:1795-1852).  That routine's
// backward sweep puts every row's saved value back at the end of the row, so
// the operator it applies is D^-1 L^-1 (L the unit lower factor, D the
// factor's diagonal with 0 read as 1); this object applies the same operator.
//
// Both the factorization and the forward sweep are recurrences over the
// rows.  Block row I depends on the block rows J < I it stores, so the rows
// are grouped into levels (level = 1 + the deepest level it depends on) and
// every level is one launch over its rows: one warp per block row, the BS
// scalar rows of a block row handled in order by that warp.  A Cube3D mesh
// of n^3 elements has 7n + 1 levels of about (n+1)^3 / (7n) block rows.
//
// The factor is kept across solves for the same pattern, as FEMSolver_
// keeps ILU_MATRIX (the reference reuses it even after the values change);
// pfg_ilu_reset drops it.
#pragma once

#include <vector>

#include "krylov.cuh"

namespace pfg {

// Most stored blocks in a block row the kernels handle (hex8 meshes: 27).
constexpr int kIluMaxBlocks = 64;

class Ilu0 {
  public:
    // Factor A's FP64 values unless the factor of A's pattern with the same
    // column order is held already.  sorted = false visits the entries k < i
    // of each row in stored order (ILUCRS exactly); true in ascending column
    // order (the order ILUCRS asks for, SparseClass.f90:1671).  Throws
    // PFG_E_UNSUPPORTED for rows longer than kIluMaxBlocks blocks.
    void factor(const DevMatrix &A, bool sorted, cudaStream_t st);
    void reset() { ready_ = false; }
    bool ready() const { return ready_; }
    int levels() const { return (int)lptr_.size() - 1; }
    // Bumped by every factorization (captured graphs bake the level launches in).
    uint64_t generation() const { return gen_; }
    // out = D^-1 L^-1 v on st, one launch per level; the launches return at
    // entry once S says the solve is done (S may be null).  Returns the count.
    int apply(const double *v, double *out, const KState *S, cudaStream_t st) const;
    // x = the solve of ILUCRS(0, RHS) (SparseClass.f90:1647-1679) with this
    // factor: the forward sweep above, then the backward substitution with U
    // (one launch per level of the upper dependencies).  rhs and x distinct.
    void solve(const double *rhs, double *x, cudaStream_t st) const;
    // Factor values in the matrix's block-row layout and the U diagonal.
    const double *lu() const { return lu_.p; }
    const double *udiag() const { return udiag_.p; }
    // Algorithmic bytes of one apply: the blocks J < I (values and block
    // columns) and the per-row entries of the sweep layout once, v, t
    // written and gathered once, out.
    double sweep_bytes() const { return sweep_bytes_; }

  private:
    bool ready_ = false, sorted_ = false;
    int bs_ = 3;
    int64_t nb_ = 0, nnzb_ = 0;
    uint64_t pattern_gen_ = 0, gen_ = 0;
    double sweep_bytes_ = 0.0;
    const int64_t *rp_ = nullptr;
    const int *col_ = nullptr;
    DevBuf<double> lu_, udiag_, t_;
    DevBuf<int> order_;           // block rows grouped by level, ascending within a level
    // sweep layout (ilu.cu): per level-ordered row (I, number of blocks J < I),
    // offset of its blocks, their block columns and values, diagonal-block
    // lower part and 1 / U(i,i)
    DevBuf<int2> sw_row_;
    DevBuf<int64_t> sw_off_;
    DevBuf<int> sw_col_;
    DevBuf<double> sw_val_, sw_diag_;
    // the same for the backward solve: rows by levels of their blocks J > I
    std::vector<int64_t> uptr_;
    DevBuf<int> uorder_;
    DevBuf<int2> su_row_;
    DevBuf<int64_t> su_off_;
    DevBuf<int> su_col_;
    DevBuf<double> su_val_, su_diag_;
    std::vector<int64_t> lptr_;   // level L holds order_[lptr_[L] .. lptr_[L+1])
};

}  // namespace pfg
