/*
 * pfg.h -- C ABI of plantfem_gb300, the GB300-native (sm_103a) linear-elastic
 * hex8 solve path of plantFEM.
 *
 * Every entry point is a plain C function over plain pointers and sizes; no
 * C++ or torch types cross this boundary.  Functions return 0 (PFG_OK) on
 * success, a positive PFG_W_* warning, or a negative PFG_E_* error code; the
 * text of the last error on the calling thread is pfg_last_error().  Nothing
 * here exits the process (the reference prints and `stop`s instead).
 *
 * Numbering follows the reference: node, element and DOF ids passed in are
 * 1-based; CRS arrays are 1-based int64 row pointers and int32 column indices
 * in first-appearance column order, exactly as FEMSolver_%CRS_Index_Row /
 * CRS_Index_Col (FEMSolverClass.f90:25-27).  Mesh arrays are Fortran
 * column-major: NodCoord(nn,3) and ElemNod(ne,8).
 *
 * Each declaration names the reference routine it replaces (file:line inside
 * the plantFEM tree).
 */
#ifndef PFG_H
#define PFG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ----------------------------------------------------------- status codes */
#define PFG_OK 0
#define PFG_W_NOT_CONVERGED 1   /* itrmax reached ("[ERROR] LOBPCG NOT CONVERGED", SparseClass.f90:2237) */
#define PFG_E_ARG (-1)          /* bad argument (size, NULL, out of range) */
#define PFG_E_STATE (-2)        /* call order (e.g. solve before setCRS) */
#define PFG_E_MISSING_SLOT (-3) /* fill-in request, FEMSolverClass.f90:1040-1047 */
#define PFG_E_BREAKDOWN (-4)    /* "Bicgstab devide by zero", FEMSolverClass.f90:2266,2295 */
#define PFG_E_NOMEM (-5)        /* device or host allocation failed */
#define PFG_E_CUDA (-6)         /* CUDA runtime error */
#define PFG_E_DETJ (-7)         /* zero-volume element, "Bmat,detJ=0" FEMDomainClass.f90:12285 */
#define PFG_E_INTERNAL (-8)
#define PFG_E_UNSUPPORTED (-9)
#define PFG_E_NONFINITE (-10)   /* NaN/Inf in the input or in a Krylov scalar */
#define PFG_E_ABORTED (-11)     /* a batched solve saw its abort flag set */

/* ----------------------------------------------------------- solve options */
#define PFG_ALG_BICGSTAB 0      /* bicgstab_CRS_2, FEMSolverClass.f90:2199-2298 (reference default) */
#define PFG_ALG_CG 1            /* conjugate gradients (K is symmetric after elimination) */

#define PFG_PREC_FP64 0         /* every operation in FP64 (the plain drop-in) */
#define PFG_PREC_MIXED 1        /* FP32 inner iterations, FP64 residual replacement */

/* Storage of the FP32 copy the mixed inner iterations read (no reference
 * counterpart; the reference keeps one FP64 CRS). */
#define PFG_STORAGE_FULL 0       /* every block: deterministic, works for any matrix */
#define PFG_STORAGE_SYMMETRIC 1  /* upper half of a symmetric 3x3-block matrix: half the bytes per
                                    product; checked symmetric (else PFG_E_ARG); the FP32 sums'
                                    order, hence their last bits, varies from run to run */

#define PFG_PC_NONE 0           /* unpreconditioned, as the reference */
#define PFG_PC_JACOBI 1         /* point Jacobi (JacobiPreconditionerCRS, FEMSolverClass.f90:2508-2529) */
#define PFG_PC_BLOCK_JACOBI 2   /* inverse of each 3x3 diagonal node block */
/* ILU(0) (FEMSolver_%solve(preconditioning="ILU"|"incompleteLU"),
 * FEMSolverClass.f90:1777-1784 -> bicgstab_CRS_ILU, LinearSolverClass.f90:4104-4230):
 * BiCGSTAB only, FP64 only, right-preconditioned by D^-1 L^-1 of the ILU(0)
 * factor (ILU_matvecCRS, SparseClass.f90:1795-1852, as it executes).  The
 * factor is taken once per pattern and kept across solves (ILU_MATRIX);
 * pfg_ilu_reset drops it. */
#define PFG_PC_ILU0 3           /* ILUCRS exactly: each row's k in stored column order */
#define PFG_PC_ILU0_SORTED 4    /* ILUCRS with each row's k in ascending column order (the order
                                   SparseClass.f90:1671 asks for; equal to PFG_PC_ILU0 for rows
                                   whose columns are sorted) */

#define PFG_STOP_REFERENCE 0    /* sqrt(rr/rr_1) < relative_er or sqrt(rr) < er0, FEMSolverClass.f90:2275-2289 */
#define PFG_STOP_TRUE_RELATIVE 1 /* |b - A x| / |b| <= relative_er, with |b - A x| recomputed in FP64 */

typedef struct pfg_solve_opts {
    int32_t algorithm;       /* PFG_ALG_* */
    int32_t precision;       /* PFG_PREC_* */
    int32_t precond;         /* PFG_PC_* */
    int32_t stop_rule;       /* PFG_STOP_* (mixed precision always uses TRUE_RELATIVE) */
    int32_t itrmax;          /* FEMSolver_%itrmax, default 100000 (FEMSolverClass.f90:69) */
    int32_t graph_chunk;     /* iterations per captured CUDA graph launch, default 32 */
    double er0;              /* FEMSolver_%er0, default 1e-10 (FEMSolverClass.f90:70) */
    double relative_er;      /* FEMSolver_%relative_er, default 1e-10 (FEMSolverClass.f90:71) */
    double reliable_delta;   /* mixed: replace the FP32 residual by the FP64 one whenever it fell
                                by this factor since the last replacement; default 0.1 */
    int32_t debug;           /* FEMSolver_%debug: print the residual per graph chunk */
    int32_t update_mode;     /* 0 auto, 1 vector updates fused into the SpMV gathers,
                                2 separate streaming passes (see krylov.cu) */
    int32_t storage;         /* mixed: PFG_STORAGE_FULL (default) or PFG_STORAGE_SYMMETRIC */
} pfg_solve_opts;

typedef struct pfg_info {
    int32_t status;          /* PFG_OK, PFG_W_NOT_CONVERGED or PFG_E_BREAKDOWN */
    int32_t iterations;      /* Krylov iterations */
    int32_t replacements;    /* mixed: FP64 residual replacements */
    int32_t kernel_launches; /* kernels this call launched (directly or inside CUDA graphs) */
    double rel_residual;     /* |b - A x| / |b| recomputed in FP64 at exit */
    double iter_residual;    /* recursive residual the stop rule saw */
    double solve_ms;         /* device time of the solve */
    int32_t fallback;        /* mixed: 1 when the FP32 inner iterations failed (breakdown,
                                overflow, or FP64 residuals that stopped falling) and the
                                solve finished in FP64 from the current x */
} pfg_info;

/* Fill opts with the reference's defaults (BiCGSTAB, FP64, no preconditioner,
 * reference stop rule, itrmax 100000, er0 = relative_er = 1e-10). */
void pfg_solve_opts_default(pfg_solve_opts *opts);

const char *pfg_last_error(void);
const char *pfg_version(void);

/* --------------------------------------------------------------- handle */
typedef struct pfg_solver pfg_solver;

/* FEMSolver_%init(NumDomain=1) (FEMSolverClass.f90:174-327) on the current
 * CUDA device.  One handle = one stream; calls on a handle are serialised. */
int pfg_create(pfg_solver **h);
/* FEMSolver_%remove() (FEMSolverClass.f90:1827-1889): frees everything. */
int pfg_destroy(pfg_solver *h);

/* FEMSolver_%setDomain(FEMDomain, DomainID=1) (FEMSolverClass.f90:329-419):
 * copies the hex8 mesh to the device.  nodcoord: NodCoord(nn,3) column-major;
 * elemnod: ElemNod(ne,nne) column-major, 1-based, nne must be 8. */
int pfg_set_mesh(pfg_solver *h, int64_t nn, const double *nodcoord, int64_t ne, int32_t nne,
                 const int32_t *elemnod);

/* FEMSolver_%setCRS(DOF) (FEMSolverClass.f90:439-898, single-domain branch
 * :677-694 -> ZeroMatrix_as_CRS FEMDomainClass.f90:10581-10840): builds the
 * sparsity pattern on the device; values and RHS start at zero.  dof must be 3. */
int pfg_set_crs(pfg_solver *h, int32_t dof);

/* FEMSolver_%setCRS(CRS_) (FEMSolverClass.f90:421-429): adopt a caller CRS
 * (1-based).  Matrices with the 3x3 node-block structure of ZeroMatrix are
 * stored as 3x3 blocks, any other matrix as 1x1 blocks. */
int pfg_set_crs_arrays(pfg_solver *h, int64_t n, const int64_t *row_ptr, const int32_t *col_idx,
                       const double *val);

/* Size of the scalar CRS of the working matrix (n rows, nnz entries). */
int pfg_get_crs_size(pfg_solver *h, int64_t *n, int64_t *nnz);
/* FEMSolver_%getCRS() (FEMSolverClass.f90:2690-2727) / the public CRS_Index_Row,
 * CRS_Index_Col, CRS_val fields: copy the working matrix out as 1-based scalar
 * CRS in the reference's column order.  Any pointer may be NULL. */
int pfg_get_crs(pfg_solver *h, int64_t *row_ptr, int32_t *col_idx, double *val);

/* FEMSolver_%setRHS(RHS) (FEMSolverClass.f90:431-437). */
int pfg_set_rhs(pfg_solver *h, int64_t n, const double *rhs);
/* Copy the current RHS (after elimination, if a solve ran) out. */
int pfg_get_rhs(pfg_solver *h, int64_t n, double *rhs);

/* FEMSolver_%setMatrix(DomainID, ElementID, DOF, Matrix) (FEMSolverClass.f90:901-911
 * -> setValue :1020-1057): add a 24x24 column-major element matrix.  Additions are
 * buffered on the host and scattered on the device at the next call that reads
 * the matrix. */
int pfg_set_matrix(pfg_solver *h, int32_t domain_id, int32_t element_id, int32_t dof, const double *matrix);
/* Batched form: count element matrices, element_ids 1-based, matrices count*576. */
int pfg_set_matrices(pfg_solver *h, int64_t count, const int32_t *element_ids, const double *matrices);
/* FEMSolver_%setVector(DomainID, ElementID, DOF, Vector) (FEMSolverClass.f90:913-920,
 * setValue :1059-1069): add a 24-entry element vector to the RHS. */
int pfg_set_vector(pfg_solver *h, int32_t domain_id, int32_t element_id, int32_t dof, const double *vector);

/* Element loop + scatter of StiffnessMatrixFEMDomain(ElementID, E, v)
 * (FEMDomainClass.f90:11457-11515) over all elements, on the device, with
 * graph-coloured atomic-free scatter; the whole-matrix form of
 * StiffnessMatrix_as_CRS (FEMDomainClass.f90:11123-11232).  E, nu: ne values
 * (or 1 value broadcast when n_prop == 1).  Adds into the working matrix. */
int pfg_assemble_stiffness(pfg_solver *h, int64_t n_prop, const double *E, const double *nu);
/* Same for MassMatrixFEMDomain(ElementID, Density, DOF=3) (FEMDomainClass.f90:10874-10952);
 * lumped != 0 applies the row lumping of :10940-10948. */
int pfg_assemble_mass(pfg_solver *h, int64_t n_prop, const double *rho, int32_t lumped);
/* Same for MassVectorFEMDomain(ElementID, Density, DOF=3, Accel) (FEMDomainClass.f90:10993-11073)
 * summed into the RHS, as the tutorials' setVector loop does. */
int pfg_assemble_body_force(pfg_solver *h, int64_t n_prop, const double *rho, const double accel[3]);

/* FEMSolver_%zeros() (FEMSolverClass.f90:1310-1322): zero values and RHS. */
int pfg_zeros(pfg_solver *h);

/* FEMSolver_%fix(DomainID, IDs, FixValue | FixValues) (FEMSolverClass.f90:1073-1136):
 * mark 1-based DOF ids fixed; values NULL -> every id gets `value`.  Ids < 1 or
 * beyond the system size are skipped, as the reference's first call does. */
int pfg_fix(pfg_solver *h, int64_t n, const int32_t *ids, const double *values, double value);

/* The Dirichlet elimination that FEMSolver_%solve performs before its Krylov
 * solve (FEMSolverClass.f90:1707-1756), on its own: afterwards the stored
 * matrix and RHS are the eliminated system (pfg_dev_solve solves it). */
int pfg_eliminate(pfg_solver *h);

/* getElementCauchyStress(displacement, E, v, option) (FEMDomainClass.f90:15249-15330,
 * StressMatrix :11912-12035): cell-averaged Cauchy stress of every element from the
 * node-interleaved displacement (3*nn, host).  option 0: full 3x3 tensors (out: ne*9,
 * row-major); otherwise one value per element (out: ne), the reference's options
 * (:15310-15362): 1 I1 = trace, 2 p = trace/3, 3 I2 = (tr(S)^2 - tr(S S))/2,
 * 4 I3 = det S, 5 / 6 / 7 the same three of the deviator S - tr(S)/3 I (J1, J2,
 * J3), 10 + 3 (i-1) + (j-1) the component S(i, j) (the (i, j) form).  E, v:
 * n_prop = 1 or ne values. */
int pfg_element_stress(pfg_solver *h, const double *displacement, int64_t n_prop, const double *E, const double *v,
                       int32_t option, double *out);

/* x = FEMSolver_%solve() (FEMSolverClass.f90:1697-1825): Dirichlet elimination
 * (mutates the stored matrix and RHS in place, as the reference), Krylov solve,
 * x(fixed) = value.  opts NULL -> pfg_solve_opts_default.  x0 may be NULL.
 * x_out receives n values; info may be NULL. */
int pfg_solve(pfg_solver *h, const pfg_solve_opts *opts, const double *x0, double *x_out, pfg_info *info);

/* Drop the ILU(0) factor the handle keeps for PFG_PC_ILU0* solves (the
 * reference keeps FEMSolver_%ILU_MATRIX for good, FEMSolverClass.f90:67,
 * LinearSolverClass.f90:4126-4135): the next ILU solve factors again. */
int pfg_ilu_reset(pfg_solver *h);

/* ILUCRS(0) (SparseClass.f90:1629-1792) of the working matrix as it is now
 * (call pfg_eliminate first for the matrix pfg_solve factors), unless the
 * handle holds the factor of this pattern for the same order already.
 * sorted: 0 stored column order (PFG_PC_ILU0), 1 ascending (PFG_PC_ILU0_SORTED).
 * lu_out (may be NULL): nnz values on the pattern pfg_get_crs returns, unit
 * lower factor strictly below the diagonal, U on and above it. */
int pfg_ilu_factor(pfg_solver *h, int32_t sorted, double *lu_out);

/* out = D^-1 L^-1 v with the held factor (ILU_matvecCRS, SparseClass.f90:1795-1852,
 * as it executes); factors in ascending order first if none is held.  Host
 * vectors of pfg ndof values. */
int pfg_ilu_apply(pfg_solver *h, const double *v, double *out);

/* CRS_%ILU(0, RHS) (ILUCRS's RHS branch, SparseClass.f90:1647-1679): x = the
 * solve with the held factor (taken in ascending order first if none is held):
 * forward substitution with L, division by U's diagonal where nonzero, then
 * backward substitution with U.  The reference factors its matrix in place
 * first; here the handle's matrix is left as it is.  Host vectors. */
int pfg_ilu_solve(pfg_solver *h, const double *rhs, double *x);

/* ------------------------------------------------------------- eigenproblem */
/* FEMSolver_%keepThisMatrixAs(As) (FEMSolverClass.f90:1544-1604): copy the
 * working matrix into a named slot ("A" = stiffness, "B" = mass for eig); at
 * most 10 names, an existing name is overwritten. */
int pfg_keep_this_matrix_as(pfg_solver *h, const char *name);

/* FEMSolver_%fix_eig(IDs) (FEMSolverClass.f90:1607-1628): 1-based DOF ids whose
 * amplitude is zero in eig; accumulated, duplicates ignored. */
/* FEMSolver_%loadMatrix(from) (FEMSolverClass.f90:1203-1222): the matrix kept
 * under `name` becomes the working matrix again (pattern and values). */
int pfg_load_matrix(pfg_solver *h, const char *name);
int pfg_fix_eig(pfg_solver *h, int64_t n, const int32_t *ids);

#define PFG_EIG_STOP_REFERENCE 0 /* max|R| / max|R at iteration 1| < tol, SparseClass.f90:2218-2234 */
#define PFG_EIG_STOP_RESIDUAL 1  /* every wanted pair |K x - lambda M x| / (lambda |M x|) < tol */

typedef struct pfg_eig_opts {
    int32_t block_size;      /* LOBPCG block k >= num_eigen (<= 32); 0: num_eigen as the reference */
    int32_t max_itr;         /* FEMSolver_%LOBPCG_MAX_ITR, default 100000 */
    double tol;              /* FEMSolver_%LOBPCG_TOL, default 1e-6 */
    int32_t precision;       /* PFG_PREC_FP64 or PFG_PREC_MIXED (FP32 phase, then FP64) */
    int32_t precond;         /* PFG_PC_BLOCK_JACOBI (default) or PFG_PC_JACOBI / PFG_PC_NONE */
    int32_t stop_rule;       /* PFG_EIG_STOP_*, default PFG_EIG_STOP_RESIDUAL */
    int32_t debug;
    uint64_t seed;           /* start block (the reference's random%randn is unseeded) */
    double tol_fp32;         /* mixed: FP32 phase ends at this relative residual, default 1e-4 */
} pfg_eig_opts;

void pfg_eig_opts_default(pfg_eig_opts *opts);

/* FEMSolver_%eig(num_eigen, eigen_value, eigen_vectors) with use_LOBPCG
 * (FEMSolverClass.f90:1384-1541 -> LOBPCG_CRS SparseClass.f90:2008-2239):
 * lowest num_eigen pairs of A x = lambda B x (the slots kept as "A" and "B")
 * with the fix_eig DOFs removed.  eigen_value[num_eigen] ascending;
 * eigen_vectors (may be NULL): ndof x num_eigen column-major, B-orthonormal,
 * zero at the fixed DOFs (as the reference scatters them back, :1498-1539).
 * info->iterations = LOBPCG iterations, info->rel_residual = largest relative
 * residual of the wanted pairs. */
int pfg_eig(pfg_solver *h, const pfg_eig_opts *opts, int32_t num_eigen, double *eigen_value, double *eigen_vectors,
            pfg_info *info);

/* The dense branch of FEMSolver_%eig (use_LOBPCG = .false., the reference's
 * default; FEMSolverClass.f90:1384-1541 with DSPGVD at :1470-1500): every
 * eigenpair of A z = lambda B z for the matrices kept as "A" and "B", with the
 * fix_eig DOFs removed (reduce_crs_matrix order), computed in FP64 on the GPU
 * (Cholesky of B, C = L^-1 A L^-T, cyclic Jacobi, back substitution).
 * num_eigen <= 0: all N pairs (N from pfg_eig_reduced_size), else the lowest
 * min(num_eigen, N).  eigen_value ascending; eigen_vectors (may be NULL):
 * ndof x count column-major, B-orthonormal, zero at the fixed DOFs.  At most
 * 4096 unknowns (PFG_E_UNSUPPORTED above: the packed dense problem grows as
 * N^2); B not positive definite: PFG_E_ARG.  info->iterations = Jacobi sweeps. */
int pfg_eig_dense(pfg_solver *h, int32_t num_eigen, double *eigen_value, double *eigen_vectors, pfg_info *info);
/* Size N of the fix_eig-reduced eigenproblem of the matrices kept as "A"/"B". */
int pfg_eig_reduced_size(pfg_solver *h, int64_t *n);

/* ------------------------------------------------ reference-signature plug-ins */
/* crs_spmv_real64(val, row_ptr, col_idx, old_vector, new_vector, n, col_size)
 * (SparseClass-c.c:53-65, bound at SparseClass.f90:38-51): new_vector += A *
 * old_vector on the GPU; host arrays, 1-based row_ptr/col_idx.  The argument
 * list is the reference's, but the reference binds a void C function as a
 * Fortran subroutine while these return an int status: the Fortran interface
 * block declares them as integer(c_int) functions (rewritten, not renamed). */
int pfg_crs_spmv_real64(const double *val, const int64_t *row_ptr, const int32_t *col_idx,
                        const double *old_vector, double *new_vector, size_t n, size_t col_size);
/* crs_spmv_real32 (SparseClass-c.c:38-50, bound at SparseClass.f90:25-36). */
int pfg_crs_spmv_real32(const float *val, const int64_t *row_ptr, const int32_t *col_idx,
                        const float *old_vector, float *new_vector, size_t n, size_t col_size);

/* The user-solver hook of FEMSolver_%solve(LinearSolver=..., x0) (FEMSolverClass.f90:1632-1662):
 * subroutine LinearSolver(row_ptr, col_idx, val, rhs, x) over host CRS arrays
 * (1-based), x in/out (x0 on entry).  n = size(rhs), nnz = size(val). */
int pfg_linear_solver_crs(const int64_t *row_ptr, const int32_t *col_idx, const double *val, const double *rhs,
                          double *x, int64_t n, int64_t nnz, const pfg_solve_opts *opts, pfg_info *info);

/* Allocation-free variant of pfg_linear_solver_crs.  No counterpart in the
 * reference: it exists for callers that cannot allocate device memory, such as
 * a host program whose GPU memory is owned by another runtime or a fixed-size
 * pool, or code that must not call cudaMalloc/cudaFree (which synchronise the
 * device) while other work is queued.  The caller passes the 1-based CRS
 * arrays, rhs and x (x0 on entry, solution on exit) in DEVICE memory; this
 * call allocates nothing -- no cudaMalloc, cudaFree or allocating library
 * routine.  Its work vectors and reduction scratch live in one static device
 * array sized for at most 262,144 unknowns (about 10.5 MB); larger n is
 * rejected with PFG_E_ARG.  CUDA loads that array (with this entry point's
 * kernels) on a device the first time the entry point runs there, because
 * modules load lazily by default, and keeps it until the process exits.  So a
 * caller that must not allocate during its solves makes one set-up call per
 * device first -- n = 0, every pointer may be NULL, nothing is solved -- with
 * that device current and before any stream capture, or runs with
 * CUDA_MODULE_LOADING=EAGER.  FP64 conjugate gradients only, point Jacobi or
 * no preconditioner, stop rule PFG_STOP_TRUE_RELATIVE only (others return
 * PFG_E_UNSUPPORTED; opts NULL: CG + Jacobi, true relative residual 1e-10).
 * Every call shares the one array and finds the previous call's contents in
 * it (the solver clears what must start at zero); calls are serialised and
 * each returns after its stream has finished, but work from another caller
 * that overlaps it on the GPU would race.  stream may be NULL. */
int pfg_linear_solver_crs_noalloc(const int64_t *d_row_ptr, const int32_t *d_col_idx, const double *d_val,
                                  const double *d_rhs, double *d_x, int64_t n, const pfg_solve_opts *opts,
                                  pfg_info *info, void *stream);

/* ------------------------------------------------ device-pointer entry points */
/* For callers that already hold device memory (the PyTorch binding): the same
 * operations over device pointers on a caller stream (cudaStream_t as void*). */
/* y = K x (FP64) with the handle's working matrix. */
int pfg_dev_spmv(pfg_solver *h, const double *d_x, double *d_y, void *stream);
/* Solve with the handle's (already eliminated) matrix: d_b -> d_x (x0 on entry). */
int pfg_dev_solve(pfg_solver *h, const pfg_solve_opts *opts, const double *d_b, double *d_x, pfg_info *info,
                  void *stream);

/* Device-array forms used by the PyTorch binding (stream NULL: the handle's own
 * stream, after the caller's work on the legacy default stream). */
/* StiffnessMatrix loop with device E / v (n_prop = 1 or ne values); adds into K. */
int pfg_dev_assemble_stiffness(pfg_solver *h, int64_t n_prop, const double *d_E, const double *d_nu, void *stream);
/* setRHS from device memory. */
int pfg_dev_set_rhs(pfg_solver *h, int64_t n, const double *d_rhs, void *stream);
/* Adjoint sensitivity of a per-element Young's modulus (no reference counterpart:
 * the reference has no adjoint).  For K(E) u = f and an adjoint solution lambda
 * of K lambda = dL/du (zero at fixed DOFs), writes dL/dE_e = -lambda_e^T
 * (dK_e/dE_e) u_e for every element, with dK_e/dE_e the element stiffness at
 * E = 1 (StiffnessMatrixFEMDomain is linear in E).  u, lambda: 3*nn device arrays. */
int pfg_dev_adjoint_grad_E(pfg_solver *h, const double *d_u, const double *d_lambda, int64_t n_prop,
                           const double *d_nu, double *d_grad, void *stream);

/* ------------------------------------------------ Newmark-beta time stepping */
/* SeismicAnalysis_%LinearReyleighNewmark (SeismicAnalysisClass.f90:1255-1436;
 * formulas getNewmarkBetaMatrix/Vector and updateVelocity/AccelNewmarkBeta,
 * :1464-1535) on the GPU.  The reference rebuilds and re-solves the element
 * matrices every step; here the stiffness kept as "A" and the consistent mass
 * kept as "B" (pfg_keep_this_matrix_as) are combined once into
 *   A_eff = M / (b dt^2) + g / (b dt) C + K,   C = alpha M + beta K (Rayleigh),
 * which replaces the handle's working matrix, with the handle's fixes
 * eliminated (prescribed displacements held at every step).  Each step forms
 *   R = M a_ext + M (u/(b dt^2) + v/(b dt) + (1/(2b) - 1) a)
 *     + C (g/(b dt) u + (g/b - 1) v + dt (g/(2b) - 1) a)
 * with two SpMVs, solves A_eff u' = R from u (warm start) and updates v, a.
 * u, v, a start at zero (fixed values in u). */
typedef struct pfg_newmark_params {
    double dt;               /* SeismicAnalysis_%dt, default 1 */
    double newmark_beta;     /* default 0.25 */
    double newmark_gamma;    /* default 0.5 */
    double rayleigh_alpha;   /* SeismicAnalysis_%alpha, default 0.524 */
    double rayleigh_beta;    /* SeismicAnalysis_%beta, default 0.00129 */
} pfg_newmark_params;

void pfg_newmark_params_default(pfg_newmark_params *p);
int pfg_newmark_setup(pfg_solver *h, const pfg_newmark_params *p);
/* Initial state (host arrays of 3 nn, each may be NULL to keep it). */
int pfg_newmark_set_state(pfg_solver *h, int64_t n, const double *u, const double *v, const double *a);
/* One time step: a_ext (external acceleration, F = M a_ext; NULL = 0); opts
 * NULL: CG + block Jacobi to the true relative residual 1e-10 (A_eff is
 * symmetric positive definite).  u_out, v_out, a_out: NULL or host arrays. */
int pfg_newmark_step(pfg_solver *h, const pfg_solve_opts *opts, int64_t n, const double *a_ext, double *u_out,
                     double *v_out, double *a_out, pfg_info *info);

/* ------------------------------------------------------------ batched solves */
/* No single reference call: plantFEM solves one organ mesh per FEMSolver_
 * object and calls FEMSolver_%solve on each in turn (FEMSolverClass.f90:1707
 * onwards, one mesh at a time).  A batch takes many such handles -- each set
 * up exactly as for pfg_solve: setCRS, assembly, fix -- and solves all of them
 * in ONE persistent kernel launch (replayed from a CUDA graph): each system is
 * solved by one CTA, or by a thread-block cluster for the largest ones, taking
 * jobs from an atomic queue in order of decreasing estimated cost.  Handles
 * must hold 3-DOF (3x3-block) systems on the batch's device, must outlive the
 * batch's use of them and must not be used while a batched solve runs; re-bind
 * (pfg_batch_set) after changing any of them. */
typedef struct pfg_batch pfg_batch;

typedef struct pfg_batch_config {
    int32_t threads;       /* threads per CTA (256, 512 or 1024): block rows of one CTA tile */
    int32_t cluster;       /* CTAs that solve one large system together (1, 2, 4 or 8) */
    double team_fraction;  /* share of the systems, largest estimated cost first, solved by a
                              whole cluster; the rest are solved by single CTAs */
} pfg_batch_config;

typedef struct pfg_batch_info {
    pfg_batch_config config;   /* configuration used */
    int32_t launches;          /* kernel launches of the solve (the persistent kernel: 1) */
    int32_t max_iterations;    /* largest CG iteration count of any system */
    int64_t total_iterations;  /* sum over the systems */
    double max_rel_residual;   /* largest true |b - Kx| / |b| */
    double solve_ms;           /* device time of the launch (CUDA events) */
    int32_t fallbacks;         /* mixed: systems solved in FP64 (pfg_info.fallback != 0) */
} pfg_batch_info;

int pfg_batch_create(pfg_batch **out);
int pfg_batch_destroy(pfg_batch *b);
/* Bind `count` handles: applies each handle's Dirichlet elimination as
 * pfg_solve does, builds the sliced matrix copies, pools the work vectors. */
int pfg_batch_set(pfg_batch *b, int64_t count, pfg_solver *const *handles);
/* Solve every bound system from x0 = 0 to the true relative residual
 * opts->relative_er.  opts->algorithm must be PFG_ALG_CG (the systems are
 * symmetric positive definite; others: PFG_E_UNSUPPORTED); precision FP64 or
 * MIXED (FP32 CG with compensated dots and FP64 residual replacement);
 * precond NONE, JACOBI or BLOCK_JACOBI; itrmax per system.  opts NULL: mixed,
 * block Jacobi, 1e-10.  x_out NULL, or `count` host arrays (3 nn each) that
 * receive the solutions with the fixed values restored; infos NULL or `count`
 * records.  A mixed solve keeps an FP32 correction only when it lowers the
 * FP64 residual and hands a system over to FP64 CG when FP32 fails on it
 * (infos[m].fallback = 1); the batch remembers those systems, and the ones
 * whose FP32 iterations exceed 1.5x their FP64 iterations, and solves them in
 * FP64 from the next mixed solve on (fallback = 2) until pfg_batch_set.
 * Returns PFG_OK, the first negative status of any system, or
 * PFG_W_NOT_CONVERGED. */
int pfg_batch_solve(pfg_batch *b, const pfg_solve_opts *opts, double *const *x_out, pfg_info *infos,
                    pfg_batch_info *binfo);
/* Solution of system `index` of the last batched solve. */
int pfg_batch_get_x(pfg_batch *b, int64_t index, double *x_out);
/* Launch configuration by hand (checked), and the one in use. */
int pfg_batch_set_config(pfg_batch *b, const pfg_batch_config *cfg);
int pfg_batch_get_config(pfg_batch *b, pfg_batch_config *cfg, int32_t *tuned);
/* Autotuner: times full batched solves of the bound systems with `opts` over
 * candidate configurations (threads per CTA x cluster size, then the team
 * share of the best), keeps the fastest for later solves and returns it;
 * opts->debug prints every candidate's time. */
int pfg_batch_tune(pfg_batch *b, const pfg_solve_opts *opts, pfg_batch_config *best, double *best_ms);
/* Host address of the batch's abort flag (host-mapped memory, 0 at creation).
 * Setting it to 1 from any host thread makes every team retire its system with
 * PFG_E_ABORTED at its next check (every 64 iterations); the caller resets it. */
int pfg_batch_abort_flag(pfg_batch *b, volatile int32_t **flag);

/* ------------------------------------------------------------ instrumentation */
/* No counterpart in the reference (it has only wall-clock timers, TimeClass.f90).
 * Times `reps` back-to-back launches of one kernel on the handle's matrix with
 * CUDA events on the handle's stream and returns the mean milliseconds per
 * launch and the algorithmic bytes one launch moves.  kernel: 0 = FP64 block
 * SpMV, 1 = FP32 block SpMV, 2 = the FP32 CG SpMV with the fused direction
 * update, 3 / 4 = FP64 / FP32 warp-per-row BCRS SpMV, 5 / 6 = the FP32 / FP64
 * CG SpMV with the p.q reduction (the dominant kernels of the mixed and FP64
 * solves with streaming update passes, the default), 7 = the FP32 product from
 * the upper half of a symmetric matrix (PFG_STORAGE_SYMMETRIC), 8 = its CG form
 * with the fused p.Ap (the dominant kernel of the symmetric-storage mixed CG:
 * matrix planes staged in shared memory by bulk copies), 9 = one D^-1 L^-1
 * sweep of the held ILU(0) factor (all its level launches; the factor is taken
 * in ascending column order first if none is held), 10 = the reproducible FP32
 * symmetric product of the mixed BiCGSTAB (own blocks in FP32, transposes in
 * 64-bit fixed point, matrix planes staged like 8's; its finish pass is not
 * part of the launch), 11 / 12 = kernels 8 / 10 in their register-pipelined
 * form (no staging; for comparison).  Kernels 2, 5, 6, 8 and 11 need a
 * symmetric positive definite (eliminated) matrix, 7, 10 and 12 a symmetric
 * one. */
int pfg_profile_kernel(pfg_solver *h, int32_t kernel, int32_t reps, double *ms_per_launch, double *bytes_per_launch);

#ifdef __cplusplus
}
#endif
#endif /* PFG_H */
