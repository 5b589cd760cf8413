// lobpcg.cuh -- block LOBPCG for K x = lambda M x on the device.
//
// Restates LOBPCG_CRS (SparseClass.f90:2008-2239) for FEMSolver_%eig
// (FEMSolverClass.f90:1384-1541), GB300 form:
//   * block vectors live in panels of 8 columns, each panel row-major
//     (n x 8): the SpMM gathers 8 contiguous values per DOF, the Gram and
//     linear-combination passes read 32 rows x 8 values contiguously per warp;
//   * K and M are read through the sliced-ELL copy (one thread per block row
//     and panel); fixed DOFs (fix_eig) are masked out of every block vector,
//     which equals the row/column removal of reduce_crs_matrix
//     (LinearSolverClass.f90:3824-3947) without re-laying out the matrices;
//   * Rayleigh-Ritz on [X W P]: the Gram matrices S^T K S and S^T M S are
//     reduced on the device (deterministic, FP64; from FP32 vectors with
//     compensated FP32 sums), the small generalized eigenproblem is solved on
//     the host in FP64 (Householder tridiagonalisation + implicit QL), with a
//     rank-revealing choice of basis instead of the reference's Euclidean
//     Gram-Schmidt (which loses rank);
//   * mixed precision: FP32 panels and SpMM until the residuals reach the
//     FP32 floor, then FP64 iterations from that start to the tolerance.
#pragma once

#include "krylov.cuh"

namespace pfg {

struct EigConfig {
    int nev = 5;            // wanted eigenpairs (LOBPCG_NUM_MODE)
    int block = 0;          // block size k >= nev (0: nev)
    int max_itr = 100000;   // LOBPCG_MAX_ITR
    double tol = 1e-6;      // LOBPCG_TOL
    int precision = PFG_PREC_FP64;
    int precond = PFG_PC_BLOCK_JACOBI;
    int stop_rule = 1;      // 0: reference max|R|/max|R_1| < tol, 1: per-pair relative residual
    uint64_t seed = 1;
    double tol_fp32 = 1e-4; // mixed: leave the FP32 phase at this relative residual
    int debug = 0;
};

struct EigResult {
    int status = PFG_OK;
    int iterations = 0;      // total (FP32 + FP64 phase)
    int iterations_fp32 = 0;
    double max_rel_residual = 0.0;
    double ms = 0.0;
    int launches = 0;
};

// Solve on the device.  K, M share the block pattern (built from one mesh);
// fixed[ndof] (device, may be null) masks DOFs out.  lambda (host, nev) and
// X (device, ndof x nev column-major, may be null) receive the result.
EigResult lobpcg_solve(DevMatrix &K, DevMatrix &M, const uint8_t *fixed, const EigConfig &cfg, double *lambda,
                       double *X, cudaStream_t st);

// Lowest eigenpairs of the symmetric-definite pencil (A, B), dense, m x m
// column-major, FP64 on the host, with B's numerically null directions
// dropped (relative threshold rank_tol).  Returns the number of pairs (<= k)
// written to lam and C (m x k column-major).
int small_generalized_eig(int m, const double *A, const double *B, int k, double rank_tol, double *lam, double *C);

// The dense branch of FEMSolver_%eig (dense_eig.cu): every eigenpair of
// A z = lambda B z for dense row-major N x N device matrices (both destroyed;
// B symmetric positive definite, else PFG_E_ARG).  w (host, N): eigenvalues
// in the order of Z's columns (unsorted); Z (device, N x N row-major): the
// B-orthonormal eigenvectors as columns.  *sweeps: Jacobi sweeps done.
constexpr int kDenseEigMax = 4096;
int dense_generalized_eig(int N, double *A, double *B, double *w, double *Z, int *sweeps, cudaStream_t st);
__global__ void k_dense_from_blocks(int64_t nb, int bs, const int64_t *__restrict__ rp, const int *__restrict__ col,
                                    const double *__restrict__ v, const int *__restrict__ map, int N,
                                    double *__restrict__ D);

}  // namespace pfg
