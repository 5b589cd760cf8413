/*
 * oracle.c -- CPU restatement of plantFEM's linear-elastic hex8 solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the GPU library in
 * plantfem_gb300/ is compared against.  Nothing in the product path links,
 * loads or calls it; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline use it.
 *
 * Every routine restates one reference routine, cited by file:line inside the
 * plantFEM source tree.  Conventions follow the reference exactly:
 *   - NodCoord(nn,3) and ElemNod(ne,8) are Fortran column-major arrays,
 *     ElemNod holds 1-based node ids;
 *   - CRS row_ptr is int64 and 1-based, col_idx is int32 and 1-based, column
 *     order inside a row is first-appearance order (not sorted);
 *   - element matrices are 24x24 column-major, local DOF = 3*(a-1)+d.
 *
 * Pinning: orc_crs_spmv_real64 is checked bit-for-bit against the reference's
 * own C SpMV (src/SparseClass/SparseClass-c.c:53-65) compiled into
 * oracle/_ref; the pattern builders are checked against each other the way
 * Tutorial/fem/CRS_Zero_Matrix.f90:10-29 does; the full solve path is checked
 * against the gravity-bar known answer of
 * Tutorial/fem/benchmark_bar_in_gravity_field.f90:63-67.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NNE 8
#define NGP 8

/* ------------------------------------------------------------------------ */
/* A1  Cube3D structured mesh                                                 */
/* MeshClass.f90:6745-6805 (rectangular2D) + :6992-7087 (Convert2Dto3D)      */
/* ------------------------------------------------------------------------ */
void orc_cube3d(int nx, int ny, int nz, double lx, double ly, double lz,
                double *nodcoord, int32_t *elemnod)
{
    int64_t nn2 = (int64_t)(nx + 1) * (ny + 1);
    int64_t nn = nn2 * (nz + 1);
    int64_t ne2 = (int64_t)nx * ny;
    int64_t ne = ne2 * nz;
    /* 2-D nodes: x fastest, coordinate = len/num * (i-1)  (MeshClass.f90:6762-6768) */
    for (int k = 0; k <= nz; ++k) {
        for (int j = 0; j <= ny; ++j) {
            for (int i = 0; i <= nx; ++i) {
                int64_t n = (int64_t)k * nn2 + (int64_t)j * (nx + 1) + i;
                nodcoord[n] = lx / (double)nx * (double)i;
                nodcoord[nn + n] = ly / (double)ny * (double)j;
                /* Convert2Dto3D: Tn/NumOfLayer*(j-1)  (MeshClass.f90:7041) */
                nodcoord[2 * nn + n] = lz / (double)nz * (double)k;
            }
        }
    }
    /* 2-D quads (MeshClass.f90:6794-6803) then layers (MeshClass.f90:7062-7068) */
    for (int k = 0; k < nz; ++k) {
        for (int j = 0; j < ny; ++j) {
            for (int i = 0; i < nx; ++i) {
                int64_t e = (int64_t)k * ne2 + (int64_t)j * nx + i;
                int32_t q[4];
                q[0] = (i + 1) + j * (nx + 1);
                q[1] = (i + 2) + j * (nx + 1);
                q[2] = nx + 2 + (i + 1) + j * (nx + 1);
                q[3] = nx + 1 + (i + 1) + j * (nx + 1);
                for (int a = 0; a < 4; ++a) {
                    elemnod[(int64_t)a * ne + e] = q[a] + (int32_t)(nn2 * k);
                    elemnod[(int64_t)(a + 4) * ne + e] = q[a] + (int32_t)(nn2 * (k + 1));
                }
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* A2  hex8 shape functions                                                   */
/* ShapeFunctionClass.f90:517-545 (Gauss points, weights 1.0),                */
/* :780-787 (N), :1094-1119 (dN/dxi), :1459-1480 (Jmat = dNdgzi*ElemCoord)    */
/* ------------------------------------------------------------------------ */
static const double GP = 0.57735026918962576;
static const double GPX[NGP] = {-1, 1, 1, -1, -1, 1, 1, -1};
static const double GPY[NGP] = {-1, -1, 1, 1, -1, -1, 1, 1};
static const double GPZ[NGP] = {-1, -1, -1, -1, 1, 1, 1, 1};
static const double SX[NNE] = {-1, 1, 1, -1, -1, 1, 1, -1};
static const double SY[NNE] = {-1, -1, 1, 1, -1, -1, 1, 1};
static const double SZ[NNE] = {-1, -1, -1, -1, 1, 1, 1, 1};

static void orc_gauss_point(int gp, double g[3])
{
    g[0] = GPX[gp] * GP;
    g[1] = GPY[gp] * GP;
    g[2] = GPZ[gp] * GP;
}

static void orc_shape_N(const double g[3], double N[NNE])
{
    for (int a = 0; a < NNE; ++a)
        N[a] = 0.125 * (1.0 + SX[a] * g[0]) * (1.0 + SY[a] * g[1]) * (1.0 + SZ[a] * g[2]);
}

/* dN(3,8): dN[i*8+a] = dN_a / dxi_i */
static void orc_shape_dN(const double g[3], double dN[3 * NNE])
{
    for (int a = 0; a < NNE; ++a) {
        dN[0 * NNE + a] = 0.125 * SX[a] * (1.0 + SY[a] * g[1]) * (1.0 + SZ[a] * g[2]);
        dN[1 * NNE + a] = 0.125 * SY[a] * (1.0 + SX[a] * g[0]) * (1.0 + SZ[a] * g[2]);
        dN[2 * NNE + a] = 0.125 * SZ[a] * (1.0 + SX[a] * g[0]) * (1.0 + SY[a] * g[1]);
    }
}

/* det_mat_real64: cofactor expansion along the first column (MathClass.f90:1460-1476) */
static double orc_det3(const double J[3][3])
{
    double m0 = J[1][1] * J[2][2] - J[2][1] * J[1][2];
    double m1 = J[0][1] * J[2][2] - J[2][1] * J[0][2];
    double m2 = J[0][1] * J[1][2] - J[1][1] * J[0][2];
    return J[0][0] * m0 - J[1][0] * m1 + J[2][0] * m2;
}

/* inverse_rank_2 for n=3 (MathClass.f90:1584-1593) */
static void orc_inv3(const double A[3][3], double Ai[3][3])
{
    double d = 1.0 / orc_det3(A);
    Ai[0][0] = d * (A[1][1] * A[2][2] - A[1][2] * A[2][1]);
    Ai[0][1] = d * (A[0][2] * A[2][1] - A[0][1] * A[2][2]);
    Ai[0][2] = d * (A[0][1] * A[1][2] - A[0][2] * A[1][1]);
    Ai[1][0] = d * (A[1][2] * A[2][0] - A[1][0] * A[2][2]);
    Ai[1][1] = d * (A[0][0] * A[2][2] - A[0][2] * A[2][0]);
    Ai[1][2] = d * (A[0][2] * A[1][0] - A[0][0] * A[1][2]);
    Ai[2][0] = d * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
    Ai[2][1] = d * (A[0][1] * A[2][0] - A[0][0] * A[2][1]);
    Ai[2][2] = d * (A[0][0] * A[1][1] - A[0][1] * A[1][0]);
}

/* Per Gauss point: J (ShapeFunctionClass.f90:1476), detJ, and the derivative
 * matrix JPsy = transpose(matmul(transpose(dNdgzi), Jin)) exactly as
 * BMatrixFEMDomain computes it (FEMDomainClass.f90:12287-12289), i.e.
 * JPsy = J^-T dN/dxi.  Returns detJ; status via *ok. */
static double orc_gp_geometry(const double xe[NNE][3], int gp, double JPsy[3][NNE], double N[NNE], int *ok)
{
    double g[3], dN[3 * NNE], J[3][3], Jin[3][3];
    orc_gauss_point(gp, g);
    orc_shape_dN(g, dN);
    if (N) orc_shape_N(g, N);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            for (int a = 0; a < NNE; ++a) s += dN[i * NNE + a] * xe[a][j];
            J[i][j] = s;
        }
    double detJ = orc_det3(J);
    if (detJ == 0.0) { *ok = 0; return 0.0; }
    orc_inv3(J, Jin);
    for (int p = 0; p < 3; ++p)
        for (int q = 0; q < NNE; ++q) {
            double s = 0.0;
            for (int r = 0; r < 3; ++r) s += dN[r * NNE + q] * Jin[r][p];
            JPsy[p][q] = s;
        }
    *ok = 1;
    return detJ;
}

/* A3  B matrix, 3-D branch (FEMDomainClass.f90:12283-12305), Bmat(6,24) */
static void orc_bmatrix(const double JPsy[3][NNE], double B[6][24])
{
    memset(B, 0, sizeof(double) * 6 * 24);
    for (int q = 0; q < NNE; ++q) {
        for (int p = 0; p < 3; ++p) B[p][3 * q + p] = JPsy[p][q];
        B[3][3 * q + 0] = JPsy[1][q];
        B[3][3 * q + 1] = JPsy[0][q];
        B[4][3 * q + 1] = JPsy[2][q];
        B[4][3 * q + 2] = JPsy[1][q];
        B[5][3 * q + 0] = JPsy[2][q];
        B[5][3 * q + 2] = JPsy[0][q];
    }
}

/* A4  isotropic D (FEMDomainClass.f90:11600-11641) */
static void orc_dmatrix(double E, double v, double D[6][6])
{
    double mu = E / 2.0 / (1.0 + v);
    double lambda = v * E / (1.0 + v) / (1.0 - 2.0 * v);
    memset(D, 0, sizeof(double) * 36);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) D[i][j] = lambda;
    for (int i = 0; i < 3; ++i) D[i][i] = 2.0 * mu + lambda;
    for (int i = 3; i < 6; ++i) D[i][i] = mu;
}

static void orc_gather_coords(const double *nodcoord, int64_t nn, const int32_t *elemnod, int64_t ne,
                              int64_t e, double xe[NNE][3])
{
    for (int a = 0; a < NNE; ++a) {
        int64_t node = elemnod[(int64_t)a * ne + e] - 1;
        for (int d = 0; d < 3; ++d) xe[a][d] = nodcoord[(int64_t)d * nn + node];
    }
}

/* A5  StiffnessMatrixFEMDomain (FEMDomainClass.f90:11457-11515):
 * Ke = sum_gp B^T D B detJ (Gauss weights are 1.0 and not multiplied).
 * Ke is 24x24 column-major.  Returns 0, or -1 when detJ == 0 (the reference
 * stops with "Bmat,detJ=0", FEMDomainClass.f90:12285). */
int orc_hex8_stiffness(const double *xe_flat, double E, double v, double *Ke)
{
    const double (*xe)[3] = (const double (*)[3])xe_flat;
    double D[6][6], B[6][24], JPsy[3][NNE], DB[6][24];
    orc_dmatrix(E, v, D);
    memset(Ke, 0, sizeof(double) * 576);
    for (int gp = 0; gp < NGP; ++gp) {
        int ok;
        double detJ = orc_gp_geometry(xe, gp, JPsy, NULL, &ok);
        if (!ok) return -1;
        orc_bmatrix(JPsy, B);
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 24; ++j) {
                double s = 0.0;
                for (int k = 0; k < 6; ++k) s += D[i][k] * B[k][j];
                DB[i][j] = s;
            }
        for (int col = 0; col < 24; ++col)
            for (int row = 0; row < 24; ++row) {
                double s = 0.0;
                for (int k = 0; k < 6; ++k) s += B[k][row] * DB[k][col];
                Ke[col * 24 + row] += s * detJ;
            }
    }
    return 0;
}

/* A6  MassMatrixFEMDomain (FEMDomainClass.f90:10874-10952): consistent mass
 * rho * sum_gp Nmat Nmat^T detJ with Nmat = N (x) I3; optional row lumping
 * (:10940-10948). */
int orc_hex8_mass(const double *xe_flat, double rho, int lumped, double *Me)
{
    const double (*xe)[3] = (const double (*)[3])xe_flat;
    double JPsy[3][NNE], N[NNE];
    memset(Me, 0, sizeof(double) * 576);
    for (int gp = 0; gp < NGP; ++gp) {
        int ok;
        double detJ = orc_gp_geometry(xe, gp, JPsy, N, &ok);
        if (!ok) return -1;
        for (int a = 0; a < NNE; ++a)
            for (int b = 0; b < NNE; ++b)
                for (int d = 0; d < 3; ++d)
                    Me[(3 * b + d) * 24 + 3 * a + d] += N[a] * N[b] * detJ;
    }
    for (int i = 0; i < 576; ++i) Me[i] *= rho;
    if (lumped) {
        for (int i = 0; i < 24; ++i) {
            double s = 0.0;
            for (int j = 0; j < 24; ++j) s += Me[j * 24 + i];
            for (int j = 0; j < 24; ++j) Me[j * 24 + i] = 0.0;
            Me[i * 24 + i] = s;
        }
    }
    return 0;
}

/* A7  MassVectorFEMDomain (FEMDomainClass.f90:10993-11073): body force
 * rho * sum_gp Nmat accel detJ. */
int orc_hex8_mass_vector(const double *xe_flat, double rho, const double accel[3], double *Fe)
{
    const double (*xe)[3] = (const double (*)[3])xe_flat;
    double JPsy[3][NNE], N[NNE];
    memset(Fe, 0, sizeof(double) * 24);
    for (int gp = 0; gp < NGP; ++gp) {
        int ok;
        double detJ = orc_gp_geometry(xe, gp, JPsy, N, &ok);
        if (!ok) return -1;
        for (int a = 0; a < NNE; ++a)
            for (int d = 0; d < 3; ++d) Fe[3 * a + d] += N[a] * accel[d] * detJ;
    }
    for (int i = 0; i < 24; ++i) Fe[i] *= rho;
    return 0;
}

/* StressMatrixFEMDomain without GaussPoint (FEMDomainClass.f90:11912-12035):
 * cell-averaged Cauchy stress, sigma = mean_gp D B u_e.  S is 3x3 row-major. */
int orc_hex8_stress(const double *xe_flat, const double *ue, double E, double v, double *S)
{
    const double (*xe)[3] = (const double (*)[3])xe_flat;
    double D[6][6], B[6][24], JPsy[3][NNE], eps[6], sig[6];
    orc_dmatrix(E, v, D);
    memset(S, 0, sizeof(double) * 9);
    for (int gp = 0; gp < NGP; ++gp) {
        int ok;
        orc_gp_geometry(xe, gp, JPsy, NULL, &ok);
        if (!ok) return -1;
        orc_bmatrix(JPsy, B);
        for (int i = 0; i < 6; ++i) {
            double s = 0.0;
            for (int j = 0; j < 24; ++j) s += B[i][j] * ue[j];
            eps[i] = s;
        }
        for (int i = 0; i < 6; ++i) {
            double s = 0.0;
            for (int j = 0; j < 6; ++j) s += D[i][j] * eps[j];
            sig[i] = s;
        }
        S[0] += sig[0]; S[4] += sig[1]; S[8] += sig[2];
        S[1] += sig[3]; S[5] += sig[4]; S[2] += sig[5];
        S[3] += sig[3]; S[7] += sig[4]; S[6] += sig[5];
    }
    for (int i = 0; i < 9; ++i) S[i] /= (double)NGP;
    return 0;
}

/* Whole-mesh wrappers (one element at a time, as the reference's element loops do) */
int orc_element_stiffness_all(int64_t nn, int64_t ne, const double *nodcoord, const int32_t *elemnod,
                              const double *E, const double *v, double *Ke_all)
{
    int err = 0;
#pragma omp parallel for reduction(| : err)
    for (int64_t e = 0; e < ne; ++e) {
        double xe[NNE][3];
        orc_gather_coords(nodcoord, nn, elemnod, ne, e, xe);
        err |= orc_hex8_stiffness(&xe[0][0], E[e], v[e], Ke_all + e * 576) != 0;
    }
    return err ? -1 : 0;
}

int orc_element_stress_all(int64_t nn, int64_t ne, const double *nodcoord, const int32_t *elemnod,
                           const double *disp, const double *E, const double *v, double *S_all)
{
    int err = 0;
#pragma omp parallel for reduction(| : err)
    for (int64_t e = 0; e < ne; ++e) {
        double xe[NNE][3], ue[24];
        orc_gather_coords(nodcoord, nn, elemnod, ne, e, xe);
        for (int a = 0; a < NNE; ++a) {
            int64_t node = elemnod[(int64_t)a * ne + e] - 1;
            /* reshape(displacement, nn, nd) is plantFEM's own row-major reshape
             * (ArrayClass.f90:5328-5344), so Disp(node, d) = displacement(3(node-1)+d) */
            for (int d = 0; d < 3; ++d) ue[3 * a + d] = disp[3 * node + d];
        }
        err |= orc_hex8_stress(&xe[0][0], ue, E[e], v[e], S_all + e * 9) != 0;
    }
    return err ? -1 : 0;
}

/* ------------------------------------------------------------------------ */
/* A8  ZeroMatrix_as_CRS, ELL path (FEMDomainClass.f90:10655-10836)           */
/* Column order per node row: elements in ascending id that touch the node    */
/* (:10680-10686), their 8 nodes in local order (:10689-10698), duplicates    */
/* dropped keeping the first (:10703-10718) and compacted (:10722-10736).     */
/* DOF expansion (:10780-10836).  Two calls: fill=0 counts and returns nnz,   */
/* fill=1 writes row_ptr (n*dof+1, 1-based) and col_idx (nnz, 1-based).       */
/* ------------------------------------------------------------------------ */
static int64_t orc_node_graph(int64_t nn, int64_t ne, int nne, const int32_t *elemnod,
                              int64_t **node_ptr_out, int32_t **node_col_out)
{
    int64_t *cnt = calloc(nn + 1, sizeof(int64_t));
    for (int64_t e = 0; e < ne; ++e)
        for (int a = 0; a < nne; ++a) cnt[elemnod[(int64_t)a * ne + e] - 1 + 1]++;
    int64_t *eptr = malloc((nn + 1) * sizeof(int64_t));
    eptr[0] = 0;
    for (int64_t i = 0; i < nn; ++i) eptr[i + 1] = eptr[i] + cnt[i + 1];
    int32_t *elist = malloc((eptr[nn] + 1) * sizeof(int32_t));
    int64_t *fillp = malloc(nn * sizeof(int64_t));
    for (int64_t i = 0; i < nn; ++i) fillp[i] = eptr[i];
    /* ELL_elem(node, count) = element id, ascending element order (:10680-10686) */
    for (int64_t e = 0; e < ne; ++e)
        for (int a = 0; a < nne; ++a) {
            int64_t node = elemnod[(int64_t)a * ne + e] - 1;
            elist[fillp[node]++] = (int32_t)e;
        }
    int64_t *nptr = malloc((nn + 1) * sizeof(int64_t));
    int64_t cap = 0;
    for (int64_t i = 0; i < nn; ++i) cap += (eptr[i + 1] - eptr[i]) * nne;
    int32_t *ncol = malloc((cap + 1) * sizeof(int32_t));
    int32_t *cand = malloc((size_t)(64 * nne + 64) * sizeof(int32_t));
    int64_t pos = 0;
    nptr[0] = 0;
    for (int64_t i = 0; i < nn; ++i) {
        int64_t m = 0;
        int64_t ncand = (eptr[i + 1] - eptr[i]) * nne;
        int32_t *c = ncand <= 64 * nne + 64 ? cand : malloc(ncand * sizeof(int32_t));
        for (int64_t j = eptr[i]; j < eptr[i + 1]; ++j)
            for (int k = 0; k < nne; ++k) c[m++] = elemnod[(int64_t)k * ne + elist[j]];
        /* (iii) zero later duplicates; (iv) shift zero to right */
        for (int64_t j = 0; j < m; ++j) {
            if (c[j] == 0) continue;
            for (int64_t k = j + 1; k < m; ++k)
                if (c[j] == c[k]) c[k] = 0;
        }
        for (int64_t j = 0; j < m; ++j)
            if (c[j] != 0) ncol[pos++] = c[j];
        nptr[i + 1] = pos;
        if (c != cand) free(c);
    }
    free(cand); free(fillp); free(elist); free(eptr); free(cnt);
    *node_ptr_out = nptr;
    *node_col_out = ncol;
    return pos;
}

static int64_t orc_expand_dof(int64_t nn, int dof, const int64_t *nptr, const int32_t *ncol,
                              int64_t *row_ptr, int32_t *col_idx)
{
    int64_t nnz = nptr[nn] * dof * dof;
    if (!row_ptr) return nnz;
    /* row pointers (:10785-10796) */
    row_ptr[0] = 1;
    for (int64_t i = 0; i < nn; ++i)
        for (int j = 0; j < dof; ++j)
            row_ptr[dof * i + j + 1] = row_ptr[dof * i + j] + dof * (nptr[i + 1] - nptr[i]);
    /* column indices (:10805-10828) */
    int64_t m = 0;
    for (int64_t i = 0; i < nn; ++i)
        for (int k = 0; k < dof; ++k)
            for (int64_t j = nptr[i]; j < nptr[i + 1]; ++j)
                for (int l = 1; l <= dof; ++l) col_idx[m++] = dof * (ncol[j] - 1) + l;
    return nnz;
}

int64_t orc_zero_matrix(int64_t nn, int64_t ne, int nne, const int32_t *elemnod, int dof,
                        int64_t *row_ptr, int32_t *col_idx)
{
    int64_t *nptr;
    int32_t *ncol;
    orc_node_graph(nn, ne, nne, elemnod, &nptr, &ncol);
    int64_t nnz = orc_expand_dof(nn, dof, nptr, ncol, row_ptr, col_idx);
    free(nptr); free(ncol);
    return nnz;
}

/* Legacy COO path of ZeroMatrix (FEMDomainClass.f90:10597-10653): COO%add per
 * (element, local a, local b) appends a new column at the end of row node_a
 * (SparseClass.f90:450-500), then COO%to_CRS (:358-409), then the same DOF
 * expansion.  Must give the same arrays as the ELL path. */
int64_t orc_zero_matrix_legacy(int64_t nn, int64_t ne, int nne, const int32_t *elemnod, int dof,
                               int64_t *row_ptr, int32_t *col_idx)
{
    int64_t *len = calloc(nn, sizeof(int64_t));
    int64_t *capv = malloc(nn * sizeof(int64_t));
    int32_t **rows = malloc(nn * sizeof(int32_t *));
    for (int64_t i = 0; i < nn; ++i) { capv[i] = 8; rows[i] = malloc(8 * sizeof(int32_t)); }
    for (int64_t e = 0; e < ne; ++e)
        for (int a = 0; a < nne; ++a)
            for (int b = 0; b < nne; ++b) {
                int64_t r = elemnod[(int64_t)a * ne + e] - 1;
                int32_t c = elemnod[(int64_t)b * ne + e];
                int dup = 0;
                for (int64_t k = 0; k < len[r]; ++k)
                    if (rows[r][k] == c) { dup = 1; break; }
                if (dup) continue;
                if (len[r] == capv[r]) { capv[r] *= 2; rows[r] = realloc(rows[r], capv[r] * sizeof(int32_t)); }
                rows[r][len[r]++] = c;
            }
    int64_t *nptr = malloc((nn + 1) * sizeof(int64_t));
    nptr[0] = 0;
    for (int64_t i = 0; i < nn; ++i) nptr[i + 1] = nptr[i] + len[i];
    int32_t *ncol = malloc((nptr[nn] + 1) * sizeof(int32_t));
    for (int64_t i = 0; i < nn; ++i) {
        memcpy(ncol + nptr[i], rows[i], len[i] * sizeof(int32_t));
        free(rows[i]);
    }
    free(rows); free(capv); free(len);
    int64_t nnz = orc_expand_dof(nn, dof, nptr, ncol, row_ptr, col_idx);
    free(nptr); free(ncol);
    return nnz;
}

/* ------------------------------------------------------------------------ */
/* A10 setValue (FEMSolverClass.f90:1020-1069): linear search of the column in */
/* the row, then CRS_val += Ke (serial: the reference's atomic is commented   */
/* out at :1051, so the oracle assembles one element at a time).             */
/* Returns -1 when a slot is missing (the reference stops, :1040-1047).       */
/* ------------------------------------------------------------------------ */
int orc_set_matrix(const int64_t *row_ptr, const int32_t *col_idx, double *val,
                   int64_t ne, const int32_t *elemnod, int64_t e, int dof, const double *Ke)
{
    for (int i = 0; i < NNE; ++i)
        for (int j = 1; j <= dof; ++j) {
            int64_t row_id = (int64_t)dof * (elemnod[(int64_t)i * ne + e] - 1) + j;
            for (int ii = 0; ii < NNE; ++ii)
                for (int jj = 1; jj <= dof; ++jj) {
                    int64_t col_id = (int64_t)dof * (elemnod[(int64_t)ii * ne + e] - 1) + jj;
                    int64_t id = -1;
                    for (int64_t k = row_ptr[row_id - 1]; k < row_ptr[row_id]; ++k)
                        if (col_idx[k - 1] == col_id) { id = k; break; }
                    if (id < 0) return -1;
                    int er = dof * i + j, ec = dof * ii + jj;
                    val[id - 1] += Ke[(int64_t)(ec - 1) * (NNE * dof) + (er - 1)];
                }
        }
    return 0;
}

int orc_set_vector(double *rhs, int64_t ne, const int32_t *elemnod, int64_t e, int dof, const double *Fe)
{
    for (int i = 0; i < NNE; ++i)
        for (int j = 1; j <= dof; ++j) {
            int64_t row_id = (int64_t)dof * (elemnod[(int64_t)i * ne + e] - 1) + j;
            rhs[row_id - 1] += Fe[dof * i + j - 1];
        }
    return 0;
}

/* Serial element loop + scatter, the oracle form of the tutorials' setMatrix
 * loop (Tutorial/fem/simpleDeformationByFEMSolver.f90:17-32). kind 0 =
 * stiffness (prop0=E, prop1=nu), kind 1 = consistent mass (prop0=rho). */
int orc_assemble(int64_t nn, int64_t ne, const double *nodcoord, const int32_t *elemnod, int kind,
                 const double *prop0, const double *prop1, const int64_t *row_ptr, const int32_t *col_idx,
                 double *val)
{
    double Ke[576], xe[NNE][3];
    for (int64_t e = 0; e < ne; ++e) {
        orc_gather_coords(nodcoord, nn, elemnod, ne, e, xe);
        int rc = kind == 0 ? orc_hex8_stiffness(&xe[0][0], prop0[e], prop1[e], Ke)
                           : orc_hex8_mass(&xe[0][0], prop0[e], 0, Ke);
        if (rc) return -1;
        if (orc_set_matrix(row_ptr, col_idx, val, ne, elemnod, e, 3, Ke)) return -2;
    }
    return 0;
}

int orc_assemble_body_force(int64_t nn, int64_t ne, const double *nodcoord, const int32_t *elemnod,
                            const double *rho, const double accel[3], double *rhs)
{
    double Fe[24], xe[NNE][3];
    for (int64_t e = 0; e < ne; ++e) {
        orc_gather_coords(nodcoord, nn, elemnod, ne, e, xe);
        if (orc_hex8_mass_vector(&xe[0][0], rho[e], accel, Fe)) return -1;
        orc_set_vector(rhs, ne, elemnod, e, 3, Fe);
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* A12 Dirichlet elimination inside solve (FEMSolverClass.f90:1707-1756):     */
/* RHS(i) -= val*fix_value(col) for every row, RHS(fixed) = value, zero the   */
/* fixed rows and columns, unit diagonal on fixed rows.  Mutates val/rhs.     */
/* ------------------------------------------------------------------------ */
void orc_apply_fix(int64_t n, const int64_t *row_ptr, const int32_t *col_idx, double *val,
                   double *rhs, const uint8_t *fixed, const double *fixval)
{
    for (int64_t i = 0; i < n; ++i)
        for (int64_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
            int64_t c = col_idx[k - 1] - 1;
            if (fixed[c]) rhs[i] = rhs[i] - val[k - 1] * fixval[c];
        }
    for (int64_t i = 0; i < n; ++i)
        if (fixed[i]) rhs[i] = fixval[i];
    for (int64_t i = 0; i < n; ++i)
        for (int64_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
            if (fixed[i]) val[k - 1] = 0.0;
            if (fixed[col_idx[k - 1] - 1]) val[k - 1] = 0.0;
        }
    for (int64_t i = 0; i < n; ++i)
        if (fixed[i])
            for (int64_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k)
                if (col_idx[k - 1] - 1 == i) val[k - 1] = 1.0;
}

/* ------------------------------------------------------------------------ */
/* A14/A15 SpMV                                                                */
/* ------------------------------------------------------------------------ */
/* crs_spmv_real64 restated (SparseClass-c.c:53-65): accumulates
 * new_vector[row] += val*old_vector[col]; row_ptr/col_idx 1-based. */
void orc_crs_spmv_real64(const double *val, const int64_t *row_ptr, const int32_t *col_idx,
                         const double *old_vector, double *new_vector, size_t n, size_t col_size)
{
    (void)col_size;
#pragma omp parallel for schedule(static)
    for (int64_t row = 0; row < (int64_t)n; ++row)
        for (int64_t col = row_ptr[row]; col < row_ptr[row + 1]; ++col)
            new_vector[row] = new_vector[row] + val[col - 1] * old_vector[col_idx[col - 1] - 1];
}

/* sub_crs_matvec_generic (LinearSolverClass.f90:3728-3777): zero new_vector,
 * OMP over rows with an atomic add per nonzero.  atomic=0 gives the same
 * per-row summation order without the atomic. */
void orc_sub_crs_matvec(int64_t n, const int64_t *row_ptr, const int32_t *col_idx, const double *val,
                        const double *x, double *y, int atomic)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) y[i] = 0.0;
    if (atomic) {
#pragma omp parallel for schedule(static)
        for (int64_t row = 0; row < n; ++row)
            for (int64_t k = row_ptr[row]; k < row_ptr[row + 1]; ++k) {
                double t = val[k - 1] * x[col_idx[k - 1] - 1];
#pragma omp atomic
                y[row] += t;
            }
    } else {
#pragma omp parallel for schedule(static)
        for (int64_t row = 0; row < n; ++row) {
            double s = y[row];
            for (int64_t k = row_ptr[row]; k < row_ptr[row + 1]; ++k) s = s + val[k - 1] * x[col_idx[k - 1] - 1];
            y[row] = s;
        }
    }
}

static double orc_dot(int64_t n, const double *a, const double *b)
{
    double s = 0.0; /* Fortran dot_product, serial (FEMSolverClass.f90:2243) */
    for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

/* ------------------------------------------------------------------------ */
/* A13 bicgstab_CRS_2 (FEMSolverClass.f90:2199-2298), restated step by step.  */
/* Stop when sqrt(rr/rr_1) < relative_er (rr_1 = |r|^2 after iteration 1) or */
/* sqrt(rr) < er0.  Returns 0 on exit by a criterion, 1 if itrmax reached,   */
/* -1 on vv == 0 or c2*c3 == 0 (the reference stops with "Bicgstab devide by  */
/* zero").  *iters receives the iteration count.                             */
/* ------------------------------------------------------------------------ */
int orc_bicgstab_crs2(int64_t n, const int64_t *row_ptr, const int32_t *col_idx, const double *a,
                      double *x, const double *b, int itrmax, double er0, double relative_er,
                      int atomic, int *iters)
{
    double *r = malloc(n * sizeof(double)), *r0 = malloc(n * sizeof(double));
    double *p = malloc(n * sizeof(double)), *y = malloc(n * sizeof(double));
    double *e = malloc(n * sizeof(double)), *v = malloc(n * sizeof(double));
    double *ax = malloc(n * sizeof(double));
    int rc = 1, itr;
    double c1, c2, c3, alp, bet, ev, vv, rr, re_er0 = 1.0;
    orc_sub_crs_matvec(n, row_ptr, col_idx, a, x, ax, atomic);
    for (int64_t i = 0; i < n; ++i) r[i] = b[i] - ax[i];
    c1 = orc_dot(n, r, r);
    for (int64_t i = 0; i < n; ++i) { p[i] = r[i]; r0[i] = r[i]; }
    for (itr = 1; itr <= itrmax; ++itr) {
        c1 = orc_dot(n, r0, r);
        orc_sub_crs_matvec(n, row_ptr, col_idx, a, p, y, atomic);
        c2 = orc_dot(n, r0, y);
        alp = c1 / c2;
        for (int64_t i = 0; i < n; ++i) e[i] = r[i] - alp * y[i];
        orc_sub_crs_matvec(n, row_ptr, col_idx, a, e, v, atomic);
        ev = orc_dot(n, e, v);
        vv = orc_dot(n, v, v);
        if (vv == 0.0) { rc = -1; break; }
        c3 = ev / vv;
        for (int64_t i = 0; i < n; ++i) {
            x[i] = x[i] + alp * p[i] + c3 * e[i];
            r[i] = e[i] - c3 * v[i];
        }
        rr = orc_dot(n, r, r);
        if (itr == 1) re_er0 = rr;
        if (sqrt(rr / re_er0) < relative_er) { rc = 0; break; }
        if (sqrt(rr) < er0) { rc = 0; break; }
        c1 = orc_dot(n, r0, r);
        bet = c1 / (c2 * c3);
        if (c2 * c3 == 0.0) { rc = -1; break; }
        for (int64_t i = 0; i < n; ++i) p[i] = r[i] + bet * (p[i] - c3 * y[i]);
    }
    if (iters) *iters = itr > itrmax ? itrmax : itr;
    free(r); free(r0); free(p); free(y); free(e); free(v); free(ax);
    return rc;
}

/* FP64 oracle solve of the eliminated (symmetric positive definite) system:
 * Jacobi-preconditioned CG stopped on the TRUE relative residual
 * |b - A x| / |b| <= tol (recomputed whenever the recursive residual says so).
 * This is the "tolerance 1e-12" FP64 oracle the GPU solutions are compared
 * with; the algorithmic restatement of the reference solver is
 * orc_bicgstab_crs2.  Returns 0 converged, 1 not converged. */
int orc_pcg(int64_t n, const int64_t *row_ptr, const int32_t *col_idx, const double *a, double *x,
            const double *b, int maxit, double tol, int *iters, double *relres)
{
    double *r = malloc(n * sizeof(double)), *z = malloc(n * sizeof(double));
    double *p = malloc(n * sizeof(double)), *q = malloc(n * sizeof(double));
    double *dinv = malloc(n * sizeof(double));
    for (int64_t i = 0; i < n; ++i) {
        double d = 0.0;
        for (int64_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k)
            if (col_idx[k - 1] - 1 == i) d = a[k - 1];
        dinv[i] = d != 0.0 ? 1.0 / d : 1.0;
    }
    double bnorm = sqrt(orc_dot(n, b, b));
    if (bnorm == 0.0) bnorm = 1.0;
    int it = 0, rc = 1;
    double res = 0.0;
    for (int restart = 0; restart < 50 && it < maxit; ++restart) {
        orc_sub_crs_matvec(n, row_ptr, col_idx, a, x, q, 0);
        for (int64_t i = 0; i < n; ++i) r[i] = b[i] - q[i];
        res = sqrt(orc_dot(n, r, r)) / bnorm;
        if (res <= tol) { rc = 0; break; }
        for (int64_t i = 0; i < n; ++i) { z[i] = dinv[i] * r[i]; p[i] = z[i]; }
        double rho = orc_dot(n, r, z);
        for (; it < maxit; ++it) {
            orc_sub_crs_matvec(n, row_ptr, col_idx, a, p, q, 0);
            double alpha = rho / orc_dot(n, p, q);
            for (int64_t i = 0; i < n; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
            double rn = sqrt(orc_dot(n, r, r)) / bnorm;
            if (rn <= 0.5 * tol) { ++it; break; }
            for (int64_t i = 0; i < n; ++i) z[i] = dinv[i] * r[i];
            double rho1 = orc_dot(n, r, z);
            double beta = rho1 / rho;
            rho = rho1;
            for (int64_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
        }
    }
    if (rc != 0) {
        orc_sub_crs_matvec(n, row_ptr, col_idx, a, x, q, 0);
        for (int64_t i = 0; i < n; ++i) r[i] = b[i] - q[i];
        res = sqrt(orc_dot(n, r, r)) / bnorm;
        if (res <= tol) rc = 0;
    }
    if (iters) *iters = it;
    if (relres) *relres = res;
    free(r); free(z); free(p); free(q); free(dinv);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* A16 reduce_crs_matrix (LinearSolverClass.f90:3824-3947): drop the listed    */
/* rows and columns (1-based ids, any order, duplicates allowed), keep order. */
/* Two calls like orc_zero_matrix: out arrays NULL returns the new nnz.       */
/* ------------------------------------------------------------------------ */
int64_t orc_reduce_crs(int64_t n, const int64_t *row_ptr, const int32_t *col_idx, const double *val,
                       int64_t nrem, const int32_t *remove_ids, int64_t *new_row_ptr,
                       int32_t *new_col_idx, double *new_val)
{
    int32_t *newid = malloc(n * sizeof(int32_t));
    uint8_t *rm = calloc(n, 1);
    for (int64_t k = 0; k < nrem; ++k)
        if (remove_ids[k] >= 1 && remove_ids[k] <= n) rm[remove_ids[k] - 1] = 1;
    int32_t id = 0;
    for (int64_t i = 0; i < n; ++i) newid[i] = rm[i] ? -1 : ++id;
    int64_t m = 0, r = 0;
    if (new_row_ptr) new_row_ptr[0] = 1;
    for (int64_t i = 0; i < n; ++i) {
        if (rm[i]) continue;
        for (int64_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
            int32_t c = newid[col_idx[k - 1] - 1];
            if (c < 0) continue;
            if (new_col_idx) { new_col_idx[m] = c; new_val[m] = val[k - 1]; }
            ++m;
        }
        ++r;
        if (new_row_ptr) new_row_ptr[r] = m + 1;
    }
    free(newid); free(rm);
    return m;
}

/* CRS_%matmul of a block of vectors (crs_matvec_generic_SparseClass,       */
/* SparseClass.f90:834-943, applied column by column as LOBPCG_CRS does):     */
/* Y(i, :) = sum_k val(k) X(col(k), :), X and Y row-major n x m.  Each column */
/* of Y is the same row sum, in the same order, as orc_sub_crs_matvec's.      */
void orc_crs_spmm(int64_t n, const int64_t *row_ptr, const int32_t *col_idx, const double *val, int64_t m,
                  const double *X, double *Y)
{
#pragma omp parallel
    {
        double *acc = malloc((size_t)m * sizeof(double));
#pragma omp for schedule(static)
        for (int64_t row = 0; row < n; ++row) {
            for (int64_t j = 0; j < m; ++j) acc[j] = 0.0;
            for (int64_t k = row_ptr[row]; k < row_ptr[row + 1]; ++k) {
                const double a = val[k - 1];
                const double *xr = X + (int64_t)(col_idx[k - 1] - 1) * m;
                for (int64_t j = 0; j < m; ++j) acc[j] = acc[j] + a * xr[j];
            }
            for (int64_t j = 0; j < m; ++j) Y[row * m + j] = acc[j];
        }
        free(acc);
    }
}

/* GramSchmidt (SparseClass.f90:2243-2275): column-sequential modified
 * Gram-Schmidt of the n x m column-major V in place; a column that is zero on
 * entry is skipped, each other column is projected off the columns before it
 * one at a time (nai = v_j . viold, viold = viold - nai v_j) and normalised.
 * The projection off v_j and the dot with v_{j+1} share one pass over viold;
 * the dots are OpenMP reductions (summation order differs from a sequential
 * loop in the last bits only). */
void orc_gram_schmidt(int64_t n, int64_t m, double *V)
{
    double *viold = malloc((size_t)n * sizeof(double));
    for (int64_t i = 0; i < m; ++i) {
        double *vi = V + i * n;
        double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
        for (int64_t k = 0; k < n; ++k) {
            viold[k] = vi[k];
            s += vi[k] * vi[k];
        }
        if (s == 0.0) continue;
        double nai = 0.0;
        if (i > 0) {
            const double *v0 = V;
#pragma omp parallel for reduction(+ : nai) schedule(static)
            for (int64_t k = 0; k < n; ++k) nai += v0[k] * viold[k];
        }
        for (int64_t j = 0; j < i; ++j) {
            const double *vj = V + j * n;
            const double *vn = j + 1 < i ? V + (j + 1) * n : viold;  /* next dot, or |viold|^2 */
            const double a = nai;
            double t = 0.0;
#pragma omp parallel for reduction(+ : t) schedule(static)
            for (int64_t k = 0; k < n; ++k) {
                const double v = viold[k] - a * vj[k];
                viold[k] = v;
                t += vn[k] * v;
            }
            nai = t;
        }
        /* here nai = |viold|^2 (for i > 0: the last pass dotted viold with itself) */
        const double nrm = i > 0 ? sqrt(nai) : sqrt(s);
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < n; ++k) vi[k] = viold[k] / nrm;
    }
    free(viold);
}

/* The same for a row-major n x m V (numpy's C order): transposed into a
 * column-major scratch T (n m doubles; NULL: allocated here) in 64-row tiles
 * (OpenMP), orthogonalised, and transposed back.  A caller that repeats the
 * call passes its own T: fresh pages of a large allocation cost more to
 * fault in than the whole orthogonalisation. */
void orc_gram_schmidt_rm(int64_t n, int64_t m, double *V, double *scratch)
{
    double *T = scratch ? scratch : malloc((size_t)n * (size_t)m * sizeof(double));
#pragma omp parallel for schedule(static)
    for (int64_t r0 = 0; r0 < n; r0 += 64) {
        const int64_t r1 = r0 + 64 < n ? r0 + 64 : n;
        for (int64_t c = 0; c < m; ++c)
            for (int64_t r = r0; r < r1; ++r) T[c * n + r] = V[r * m + c];
    }
    orc_gram_schmidt(n, m, T);
#pragma omp parallel for schedule(static)
    for (int64_t r0 = 0; r0 < n; r0 += 64) {
        const int64_t r1 = r0 + 64 < n ? r0 + 64 : n;
        for (int64_t r = r0; r < r1; ++r)
            for (int64_t c = 0; c < m; ++c) V[r * m + c] = T[c * n + r];
    }
    if (!scratch) free(T);
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* A18 ILUCRS(fill_in_order = 0) (SparseClass.f90:1629-1792, case (0)): the  */
/* in-place incomplete LU factorization on the CRS pattern.  diag_vec starts */
/* as the matrix diagonal (diagCRS :1597-1626, 0 where a row stores none);    */
/* for rows i = 2..n, every entry k < i of row i in turn:                     */
/*     A_ik = get(i,k) / diag_vec(k);  update(i,k) = A_ik;                    */
/*     add(i,j, -A_ik * get(k,j)) for the entries j >= k+1 of row i;          */
/*     diag_vec(i) = get(i,i).                                                 */
/* get of an entry row k does not store is 0 (getCRS :1542-1560).  The k of a */
/* row are visited in the row's STORED column order (:1664-1672; the comment */
/* there asks for sorted columns): sorted = 0 restates that, sorted != 0     */
/* visits them in ascending column order, which is the same thing for rows  */
/* whose columns are sorted and the textbook ILU(0) for any row.             */
/* ------------------------------------------------------------------------ */
void orc_ilu0(int64_t n, const int64_t *row_ptr, const int32_t *col_idx, double *val, int sorted)
{
    double *diag = calloc((size_t)n, sizeof(double));
    int64_t *posk = malloc((size_t)n * sizeof(int64_t));
    int64_t maxlen = 0;
    for (int64_t i = 0; i < n; ++i) {
        posk[i] = -1;
        const int64_t s = row_ptr[i] - 1, e = row_ptr[i + 1] - 1;
        if (e - s > maxlen) maxlen = e - s;
        for (int64_t q = s; q < e; ++q)
            if (col_idx[q] - 1 == i) { diag[i] = val[q]; break; }
    }
    int64_t *seq = malloc((size_t)(maxlen > 0 ? maxlen : 1) * sizeof(int64_t));
    for (int64_t i = 1; i < n; ++i) {
        const int64_t s = row_ptr[i] - 1, e = row_ptr[i + 1] - 1, len = e - s;
        for (int64_t q = 0; q < len; ++q) seq[q] = s + q;
        if (sorted) /* insertion sort of the entry positions by column (stable) */
            for (int64_t q = 1; q < len; ++q) {
                const int64_t t = seq[q];
                int64_t r = q;
                while (r > 0 && col_idx[seq[r - 1]] > col_idx[t]) { seq[r] = seq[r - 1]; --r; }
                seq[r] = t;
            }
        for (int64_t qq = 0; qq < len; ++qq) {
            const int64_t kk = seq[qq];
            const int64_t k = col_idx[kk] - 1;
            if (k >= i) continue;
            const double a_ik = val[kk] / diag[k];
            val[kk] = a_ik;
            const int64_t ks = row_ptr[k] - 1, ke = row_ptr[k + 1] - 1;
            for (int64_t q = ke - 1; q >= ks; --q) posk[col_idx[q] - 1] = q; /* first match wins */
            for (int64_t jj = s; jj < e; ++jj) {
                const int64_t j = col_idx[jj] - 1;
                if (j < k + 1) continue;
                const double a_kj = posk[j] >= 0 ? val[posk[j]] : 0.0;
                val[jj] = val[jj] + (-(a_ik * a_kj));
            }
            for (int64_t q = ks; q < ke; ++q) posk[col_idx[q] - 1] = -1;
            double d = 0.0;
            for (int64_t q = s; q < e; ++q)
                if (col_idx[q] - 1 == i) { d = val[q]; break; }
            diag[i] = d;
        }
    }
    free(seq);
    free(posk);
    free(diag);
}

/* ILU_matvecCRS (SparseClass.f90:1795-1852) as it executes on an ILU(0)      */
/* factor: forward substitution with the unit lower factor (:1803-1817),      */
/* then division by the factor's diagonal, 0 taken as 1 (:1820-1828).  The    */
/* loop written as the backward substitution (:1830-1849) ends each row by   */
/* storing back the value it saved before the row's loop, so it leaves the   */
/* vector as it was: the operator applied is D^-1 L^-1.                       */
void orc_ilu_apply(int64_t n, const int64_t *row_ptr, const int32_t *col_idx, const double *lu,
                   const double *v, double *out)
{
    for (int64_t i = 0; i < n; ++i) out[i] = v[i];
    for (int64_t i = 1; i < n; ++i) {
        double s = out[i];
        for (int64_t q = row_ptr[i] - 1; q < row_ptr[i + 1] - 1; ++q)
            if (col_idx[q] - 1 < i) s = s - lu[q] * out[col_idx[q] - 1];
        out[i] = s;
    }
    for (int64_t i = 0; i < n; ++i) {
        double d = 0.0;
        for (int64_t q = row_ptr[i] - 1; q < row_ptr[i + 1] - 1; ++q)
            if (col_idx[q] - 1 == i) { d = lu[q]; break; }
        if (d == 0.0) d = 1.0;
        out[i] = out[i] / d;
    }
}

/* bicgstab_CRS_ILU (LinearSolverClass.f90:4104-4230): BiCGSTAB right-       */
/* preconditioned by the ILU(0) factor lu (orc_ilu0): y = A M^-1 p and        */
/* v = A M^-1 e through sub_crs_matvec's precondition argument (:3751-3763), */
/* x += alp M^-1 p + c3 M^-1 e.  Returns at once when |r0|^2 < er0 (:4150);  */
/* stop rules, return codes and *iters as orc_bicgstab_crs2.                  */
int orc_bicgstab_ilu(int64_t n, const int64_t *row_ptr, const int32_t *col_idx, const double *a,
                     const double *lu, double *x, const double *b, int itrmax, double er0, double relative_er,
                     int *iters)
{
    double *r = malloc(n * sizeof(double)), *r0 = malloc(n * sizeof(double));
    double *p = malloc(n * sizeof(double)), *y = malloc(n * sizeof(double));
    double *e = malloc(n * sizeof(double)), *v = malloc(n * sizeof(double));
    double *pd = malloc(n * sizeof(double)), *ps = malloc(n * sizeof(double));
    int rc = 1, itr = 0;
    double c1, c2, c3, alp, bet, ev, vv, rr, re_er0 = 1.0;
    orc_sub_crs_matvec(n, row_ptr, col_idx, a, x, y, 0);
    for (int64_t i = 0; i < n; ++i) r[i] = b[i] - y[i];
    c1 = orc_dot(n, r, r);
    if (c1 < er0) {
        rc = 0;
        goto done;
    }
    for (int64_t i = 0; i < n; ++i) { p[i] = r[i]; r0[i] = r[i]; }
    for (itr = 1; itr <= itrmax; ++itr) {
        c1 = orc_dot(n, r0, r);
        orc_ilu_apply(n, row_ptr, col_idx, lu, p, pd);
        orc_sub_crs_matvec(n, row_ptr, col_idx, a, pd, y, 0);
        c2 = orc_dot(n, r0, y);
        alp = c1 / c2;
        for (int64_t i = 0; i < n; ++i) e[i] = r[i] - alp * y[i];
        orc_ilu_apply(n, row_ptr, col_idx, lu, e, ps);
        orc_sub_crs_matvec(n, row_ptr, col_idx, a, ps, v, 0);
        ev = orc_dot(n, e, v);
        vv = orc_dot(n, v, v);
        if (vv == 0.0) { rc = -1; break; }
        c3 = ev / vv;
        for (int64_t i = 0; i < n; ++i) {
            x[i] = x[i] + alp * pd[i] + c3 * ps[i];
            r[i] = e[i] - c3 * v[i];
        }
        rr = orc_dot(n, r, r);
        if (itr == 1) re_er0 = rr;
        if (sqrt(rr / re_er0) < relative_er) { rc = 0; break; }
        if (sqrt(rr) < er0) { rc = 0; break; }
        c1 = orc_dot(n, r0, r);
        bet = c1 / (c2 * c3);
        if (c2 * c3 == 0.0) { rc = -1; break; }
        for (int64_t i = 0; i < n; ++i) p[i] = r[i] + bet * (p[i] - c3 * y[i]);
    }
done:
    if (iters) *iters = itr > itrmax ? itrmax : itr;
    free(r); free(r0); free(p); free(y); free(e); free(v); free(pd); free(ps);
    return rc;
}

/* ILUCRS(0, RHS) (SparseClass.f90:1647-1679), the solve with an ILU(0) factor   */
/* lu (orc_ilu0), in place on rhs: forward substitution with the unit lower    */
/* factor; rhs(i) /= U(i,i) where U(i,i) != 0; then for i = n..1,              */
/* rhs(i) -= U(i,j)/U(i,i) rhs(j) over the entries j > i (this loop divides by */
/* a zero U(i,i), as the reference does).                                      */
void orc_ilu_solve(int64_t n, const int64_t *row_ptr, const int32_t *col_idx, const double *lu, double *rhs)
{
    double *d = calloc((size_t)n, sizeof(double));
    for (int64_t i = 0; i < n; ++i)
        for (int64_t q = row_ptr[i] - 1; q < row_ptr[i + 1] - 1; ++q)
            if (col_idx[q] - 1 == i) { d[i] = lu[q]; break; }
    for (int64_t i = 1; i < n; ++i)
        for (int64_t q = row_ptr[i] - 1; q < row_ptr[i + 1] - 1; ++q)
            if (col_idx[q] - 1 < i) rhs[i] = rhs[i] - lu[q] * rhs[col_idx[q] - 1];
    for (int64_t i = n - 1; i >= 0; --i)
        if (d[i] != 0.0) rhs[i] = rhs[i] / d[i];
    for (int64_t i = n - 1; i >= 0; --i)
        for (int64_t q = row_ptr[i] - 1; q < row_ptr[i + 1] - 1; ++q)
            if (col_idx[q] - 1 > i) rhs[i] = rhs[i] - lu[q] / d[i] * rhs[col_idx[q] - 1];
    free(d);
}
