// batch.cuh -- many independent elasticity systems in one persistent launch.
//
// plantFEM solves one organ mesh per FEMSolver_ object and calls
// FEMSolver_%solve on each in turn (FEMSolverClass.f90:1707 onwards).  A batch
// binds the handles of many such systems (each assembled and fixed as usual)
// and solves all of them with one persistent kernel:
//
//   * every system keeps its own sliced-ELL matrix (sell.cuh) and is solved by
//     a *team*: either a thread-block cluster of CS CTAs (large systems, the
//     first `n_team` jobs) or a single CTA (the rest);
//   * jobs are taken from two atomic queues, largest estimated cost first
//     (longest-processing-time order), so uneven sizes and iteration counts
//     are balanced dynamically while the launch runs;
//   * team-wide dot products are reduced deterministically: per-CTA partials go
//     to rank 0's shared memory (distributed shared memory), every CTA sums
//     them in rank order after a cluster barrier, so all CTAs take identical
//     control decisions;
//   * FP64 CG, or FP32 CG with compensated dots and FP64 residual replacement
//     (reliable updates), block-Jacobi preconditioned, to a true relative
//     residual |b - Kx| / |b| <= tol.
//
// The launch configuration (threads per CTA, cluster size, share of team jobs)
// is picked by a measuring autotuner (batch.cu).
#pragma once

#include "krylov.cuh"

namespace pfg {

// What a bound handle contributes (filled by batch_bind in femsolver.cu).
struct BatchSource {
    DevMatrix *K = nullptr;           // eliminated matrix with valid SELL FP64/FP32 copies
    const double *b = nullptr;        // eliminated right-hand side
    const uint8_t *fixed = nullptr;   // Dirichlet mask (null: no fixed DOFs)
    const double *fixval = nullptr;   // prescribed values
    int device = 0;
};

// Device descriptor of one system.
struct BatchMesh {
    SellView<double> A64;
    SellView<float> A32;
    const double *b;
    const uint8_t *fixed;
    const double *fixval;
    double *x;                            // x0 in, solution out
    double *r64, *p64, *q64, *z64, *s64;  // FP64 work vectors (CG: r, p, w, u, s)
    float *x32, *r32, *p32, *q32, *z32;   // FP32 work vectors
    const double *dinv64;                 // block-Jacobi inverses (9 per block row)
    const float *dinv32;
};

// Per-system result written by the kernel.
struct BatchOut {
    int status;
    int iterations;
    int replacements;   // FP64 residual replacements (mixed) / true-residual restarts (FP64)
    int team_size;      // CTAs that solved it
    int fallback;       // mixed: 0 FP32 inner iterations, 1 handed over to FP64 in this solve,
                        // 2 solved in FP64 because an earlier solve of it needed FP64
    double rel_residual;   // true |b - Kx| / |b|
};

struct BatchParams {
    const BatchMesh *mesh;
    BatchOut *out;
    const int *order;         // job order: team jobs, then single-CTA jobs
    int n_team;               // first n_team jobs are solved by a whole cluster
    int n_total;
    int cluster;              // CTAs per cluster (1: no cluster launch)
    unsigned *queue;          // [0] team queue, [1] single-CTA queue (zero at launch)
    int precond;              // PFG_PC_NONE / PFG_PC_JACOBI / PFG_PC_BLOCK_JACOBI
    int itrmax;
    int max_restarts;
    double tol;
    double delta;             // reliable-update threshold (mixed)
    const volatile int *abort;   // host-mapped abort flag (null: none)
    const uint8_t *force64;      // mixed: per system, 1 = solve in FP64 (learned from earlier solves)
};

// femsolver.cu: eliminate, refresh the sliced copies and describe the handle.
BatchSource batch_bind(::pfg_solver *h);

}  // namespace pfg
