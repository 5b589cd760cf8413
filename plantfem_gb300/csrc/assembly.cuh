// assembly.cuh -- hex8 mesh on the device: sparsity pattern, colouring,
// element integration with coloured scatter, Dirichlet elimination, CRS
// import/export.  Implemented in assembly.cu.
#pragma once

#include "krylov.cuh"

namespace pfg {

struct DevMesh {
    int64_t nn = 0, ne = 0;
    DevBuf<double> xyz;          // SoA: x[nn], y[nn], z[nn]
    DevBuf<int> conn;            // SoA: conn[a * ne + e], 0-based node ids, a = 0..7
    std::vector<int> conn_host;  // same, on the host (colouring, setMatrix slots)
    // elements grouped by colour: no two elements of one colour share a node
    DevBuf<int> color_elems;
    std::vector<int64_t> color_ptr;
    // per element, the slot of each of its 64 blocks in the CRS rows of the
    // pattern with generation slots_gen (built by the first assembly)
    mutable DevBuf<uint16_t> slots;
    mutable uint64_t slots_gen = 0;
};

// Build the node-graph pattern in the reference's first-appearance order
// (ZeroMatrix_as_CRS, FEMDomainClass.f90:10655-10836) on the device and set up
// an all-zero 3x3-block matrix with it.
void build_pattern(const DevMesh &m, DevMatrix &K, cudaStream_t st);

// Greedy element colouring on the host (first fit in element order).
void color_elements(DevMesh &m, cudaStream_t st);

// kind: 0 stiffness (p0 = E, p1 = nu), 1 consistent mass (p0 = rho), 2 lumped
// mass.  p0/p1 are device arrays of ne values, or of 1 value when `broadcast`.
// Adds into K.v64 (coloured, atomic-free).  Throws PFG_E_DETJ on detJ == 0.
void assemble_elements(const DevMesh &m, DevMatrix &K, int kind, const double *p0, const double *p1, bool broadcast,
                       cudaStream_t st);
// Body force rho * sum_gp N accel detJ added into rhs (device, 3*nn).
void assemble_body_force(const DevMesh &m, double *rhs, const double *rho, bool broadcast, const double accel[3],
                         cudaStream_t st);
// Add count user element matrices (24x24 column-major, device) for 0-based
// element ids (device) into K (atomic adds: repeated ids are allowed).
void scatter_element_matrices(const DevMesh &m, DevMatrix &K, int64_t count, const int *ids, const double *mats,
                              cudaStream_t st);
// Add element vectors (24 each) into rhs.
void scatter_element_vectors(const DevMesh &m, double *rhs, int64_t count, const int *ids, const double *vecs,
                             cudaStream_t st);
// Per-element 24x24 stiffness (column-major) into out[ne*576] (no scatter).
void element_stiffness(const DevMesh &m, const double *E, const double *nu, bool broadcast, double *out,
                       cudaStream_t st);
// Cell-averaged Cauchy stress (ne x 9, row-major 3x3) from a 3*nn displacement.
void element_stress(const DevMesh &m, const double *disp, const double *E, const double *nu, bool broadcast,
                    double *out, cudaStream_t st);
// One value per element from the stress tensors (ne x 9, device): the options
// of getElementCauchyStress (1 I1, 2 p, 3 I2, 4 I3, 5 J1, 6 J2, 7 J3,
// 10 + 3 (i-1) + (j-1) component (i, j)); out: ne values (device).
void element_stress_option(int64_t ne, const double *S, int option, double *out, cudaStream_t st);
// Adjoint sensitivity g_e = -lambda_e^T (dK_e/dE_e) u_e for every element.
void adjoint_grad_E(const DevMesh &m, const double *u, const double *lam, const double *nu, bool broadcast,
                    double *grad, cudaStream_t st);

// Dirichlet elimination of FEMSolver_%solve (FEMSolverClass.f90:1707-1756)
// on the device, in place: rhs_i -= K_ij u_j for fixed j (every row), then
// rhs(fixed) = value, zero fixed rows and columns, unit diagonal.
void apply_dirichlet(DevMatrix &K, double *rhs, const uint8_t *fixed, const double *fixval, cudaStream_t st);
// x(fixed) = value (FEMSolverClass.f90:1814-1823).
void restore_fixed(int64_t n, double *x, const uint8_t *fixed, const double *fixval, cudaStream_t st);

// Scalar CRS (1-based, device arrays) -> block layout.  Detects the 3x3
// node-block structure of ZeroMatrix; otherwise stores 1x1 blocks.
// allow_blocks == false always stores 1x1 blocks; val may then be NULL (values
// filled by the caller).
void import_crs(int64_t n, int64_t nnz, const int64_t *row_ptr, const int32_t *col_idx, const double *val,
                DevMatrix &K, cudaStream_t st, bool allow_blocks = true);
// Block layout -> scalar CRS (1-based, device arrays, reference column order).
void export_crs(const DevMatrix &K, int64_t *row_ptr, int32_t *col_idx, double *val, cudaStream_t st);
// Values in the matrix's block-row layout (bval, K's pattern) -> scalar CRS
// values in the order export_crs writes (device pointers).
void export_values(const DevMatrix &K, const double *bval, double *val, cudaStream_t st);

// Exclusive prefix sum of n int64 values (out may alias in); returns the total.
int64_t exclusive_scan(const int64_t *in, int64_t *out, int64_t n, cudaStream_t st);

}  // namespace pfg
