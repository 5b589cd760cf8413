// assembly.cu -- pattern, colouring, hex8 element kernels and Dirichlet
// elimination on the device.
#include <algorithm>

#include "assembly.cuh"

namespace pfg {

// ------------------------------------------------------------------- scan
// Exclusive scan of int64 in tiles of 2048 (256 threads x 8), recursing on the
// tile totals.
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void k_scan_tiles(const int64_t *__restrict__ in, int64_t *__restrict__ out, int64_t n,
                             int64_t *__restrict__ tile_sums)
{
    __shared__ int64_t s[kScanThreads];
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int64_t v[kScanItems];
    int64_t run = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t i = base + k;
        const int64_t x = i < n ? in[i] : 0;
        v[k] = run;  // exclusive within the thread
        run += x;
    }
    s[threadIdx.x] = run;
    __syncthreads();
    // Hillis-Steele inclusive scan of the thread totals
    for (int o = 1; o < kScanThreads; o <<= 1) {
        int64_t t = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
        __syncthreads();
        s[threadIdx.x] += t;
        __syncthreads();
    }
    const int64_t prefix = threadIdx.x > 0 ? s[threadIdx.x - 1] : 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t i = base + k;
        if (i < n) out[i] = v[k] + prefix;
    }
    if (threadIdx.x == kScanThreads - 1) tile_sums[blockIdx.x] = s[kScanThreads - 1];
}

__global__ void k_scan_add(int64_t *__restrict__ out, int64_t n, const int64_t *__restrict__ tile_prefix)
{
    const int64_t i = (int64_t)blockIdx.x * kScanTile + threadIdx.x;
    const int64_t add = tile_prefix[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t j = i + (int64_t)k * kScanThreads;
        if (j < n) out[j] += add;
    }
}

int64_t exclusive_scan(const int64_t *in, int64_t *out, int64_t n, cudaStream_t st)
{
    if (n <= 0) return 0;
    const int64_t tiles = (n + kScanTile - 1) / kScanTile;
    DevBuf<int64_t> sums((size_t)tiles + 1);
    k_scan_tiles<<<(unsigned)tiles, kScanThreads, 0, st>>>(in, out, n, sums.p);
    PFG_CUDA(cudaGetLastError());
    int64_t total = 0;
    if (tiles == 1) {
        PFG_CUDA(cudaMemcpyAsync(&total, sums.p, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        PFG_CUDA(cudaStreamSynchronize(st));
        return total;
    }
    DevBuf<int64_t> pref((size_t)tiles);
    total = exclusive_scan(sums.p, pref.p, tiles, st);
    k_scan_add<<<(unsigned)tiles, kScanThreads, 0, st>>>(out, n, pref.p);
    PFG_CUDA(cudaGetLastError());
    PFG_CUDA(cudaStreamSynchronize(st));
    return total;
}

// ---------------------------------------------------------------- pattern
constexpr int kMaxRow = 128;  // unique node neighbours per node supported

__global__ void k_count_incidence(const int *__restrict__ conn, int64_t ne, unsigned long long *cnt)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ne * 8; i += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&cnt[conn[i]], 1ull);
}

__global__ void k_fill_incidence(const int *__restrict__ conn, int64_t ne, const int64_t *__restrict__ eptr,
                                 unsigned long long *cursor, int *__restrict__ elist)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ne * 8; i += (int64_t)gridDim.x * blockDim.x) {
        const int node = conn[i];
        const int64_t e = i % ne;
        const unsigned long long pos = atomicAdd(&cursor[node], 1ull);
        elist[eptr[node] + (int64_t)pos] = (int)e;
    }
}

// Elements touching a node in ascending element id (ELL_elem, FEMDomainClass.f90:10680-10686).
__global__ void k_sort_incidence(int64_t nn, const int64_t *__restrict__ eptr, int *__restrict__ elist)
{
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nn; v += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = eptr[v], e = eptr[v + 1];
        for (int64_t i = s + 1; i < e; ++i) {
            const int key = elist[i];
            int64_t j = i - 1;
            while (j >= s && elist[j] > key) {
                elist[j + 1] = elist[j];
                --j;
            }
            elist[j + 1] = key;
        }
    }
}

// Candidate columns = nodes of those elements in local order, first
// occurrence kept (FEMDomainClass.f90:10689-10736).  fill == 0 counts.
__global__ void k_node_graph(int64_t nn, const int *__restrict__ conn, int64_t ne, const int64_t *__restrict__ eptr,
                             const int *__restrict__ elist, int64_t *__restrict__ cnt, const int64_t *__restrict__ rp,
                             int *__restrict__ col, int fill, int *err)
{
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nn; v += (int64_t)gridDim.x * blockDim.x) {
        int acc[kMaxRow];
        int m = 0;
        for (int64_t j = eptr[v]; j < eptr[v + 1]; ++j) {
            const int e = elist[j];
            for (int a = 0; a < 8; ++a) {
                const int c = conn[(int64_t)a * ne + e];
                bool dup = false;
                for (int k = 0; k < m; ++k)
                    if (acc[k] == c) { dup = true; break; }
                if (dup) continue;
                if (m >= kMaxRow) { *err = 1; break; }
                acc[m++] = c;
            }
        }
        if (!fill) {
            cnt[v] = m;
        } else {
            const int64_t s = rp[v];
            for (int k = 0; k < m; ++k) col[s + k] = acc[k];
        }
    }
}

void build_pattern(const DevMesh &m, DevMatrix &K, cudaStream_t st)
{
    PFG_CHECK(m.nn > 0 && m.ne > 0, PFG_E_STATE, "no mesh: call setDomain (pfg_set_mesh) first");
    const int64_t nn = m.nn, ne = m.ne;
    DevBuf<unsigned long long> cnt((size_t)nn + 1);
    DevBuf<int64_t> eptr((size_t)nn + 1);
    PFG_CUDA(cudaMemsetAsync(cnt.p, 0, (nn + 1) * sizeof(unsigned long long), st));
    const int g = grid_for(ne * 8, 256, sm_count_device() * 16);
    k_count_incidence<<<g, 256, 0, st>>>(m.conn.p, ne, cnt.p);
    PFG_CUDA(cudaGetLastError());
    const int64_t ninc = exclusive_scan((const int64_t *)cnt.p, eptr.p, nn + 1, st);
    PFG_CHECK(ninc == ne * 8, PFG_E_INTERNAL, "incidence count mismatch");
    DevBuf<int> elist((size_t)ninc);
    PFG_CUDA(cudaMemsetAsync(cnt.p, 0, (nn + 1) * sizeof(unsigned long long), st));
    k_fill_incidence<<<g, 256, 0, st>>>(m.conn.p, ne, eptr.p, cnt.p, elist.p);
    const int gn = grid_for(nn, 128, sm_count_device() * 16);
    k_sort_incidence<<<gn, 128, 0, st>>>(nn, eptr.p, elist.p);
    PFG_CUDA(cudaGetLastError());
    DevBuf<int64_t> ncnt((size_t)nn + 1);
    DevBuf<int> err(1);
    PFG_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
    PFG_CUDA(cudaMemsetAsync(ncnt.p, 0, (nn + 1) * sizeof(int64_t), st));
    k_node_graph<<<gn, 128, 0, st>>>(nn, m.conn.p, ne, eptr.p, elist.p, ncnt.p, nullptr, nullptr, 0, err.p);
    PFG_CUDA(cudaGetLastError());
    K.bs = 3;
    K.nb = nn;
    K.rp.alloc((size_t)nn + 1);
    const int64_t nnzb = exclusive_scan(ncnt.p, K.rp.p, nn + 1, st);
    int herr = 0;
    PFG_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    PFG_CUDA(cudaStreamSynchronize(st));
    PFG_CHECK(herr == 0, PFG_E_UNSUPPORTED, "a node has more than 128 neighbouring nodes");
    PFG_CHECK(nnzb < (int64_t)INT32_MAX, PFG_E_UNSUPPORTED, "more than 2^31 blocks");
    K.nnzb = nnzb;
    K.col.alloc((size_t)nnzb);
    k_node_graph<<<gn, 128, 0, st>>>(nn, m.conn.p, ne, eptr.p, elist.p, nullptr, K.rp.p, K.col.p, 1, err.p);
    PFG_CUDA(cudaGetLastError());
    K.v64.alloc((size_t)nnzb * 9);
    PFG_CUDA(cudaMemsetAsync(K.v64.p, 0, (size_t)nnzb * 9 * sizeof(double), st));
    // new pattern: every derived copy (FP32, sliced) is stale
    K.pattern_changed();
    PFG_CUDA(cudaStreamSynchronize(st));
}

void color_elements(DevMesh &m, cudaStream_t st)
{
    const int64_t nn = m.nn, ne = m.ne;
    const std::vector<int> &cn = m.conn_host;
    std::vector<int64_t> ptr((size_t)nn + 1, 0);
    for (int64_t i = 0; i < ne * 8; ++i) ptr[(size_t)cn[(size_t)i] + 1]++;
    for (int64_t v = 0; v < nn; ++v) ptr[(size_t)v + 1] += ptr[(size_t)v];
    std::vector<int> lst((size_t)ne * 8);
    std::vector<int64_t> cur(ptr.begin(), ptr.end() - 1);
    for (int64_t e = 0; e < ne; ++e)
        for (int a = 0; a < 8; ++a) {
            const int v = cn[(size_t)(a * ne + e)];
            lst[(size_t)cur[(size_t)v]++] = (int)e;
        }
    std::vector<int> color((size_t)ne, -1);
    int ncol = 0;
    for (int64_t e = 0; e < ne; ++e) {
        uint64_t used = 0;
        for (int a = 0; a < 8; ++a) {
            const int v = cn[(size_t)(a * ne + e)];
            for (int64_t k = ptr[(size_t)v]; k < ptr[(size_t)v + 1]; ++k) {
                const int f = lst[(size_t)k];
                if (f < e && color[(size_t)f] >= 0 && color[(size_t)f] < 64) used |= 1ull << color[(size_t)f];
            }
        }
        int c = 0;
        while (c < 64 && (used >> c) & 1ull) ++c;
        PFG_CHECK(c < 64, PFG_E_UNSUPPORTED, "element colouring needs more than 64 colours");
        color[(size_t)e] = c;
        ncol = std::max(ncol, c + 1);
    }
    m.color_ptr.assign((size_t)ncol + 1, 0);
    for (int64_t e = 0; e < ne; ++e) m.color_ptr[(size_t)color[(size_t)e] + 1]++;
    for (int c = 0; c < ncol; ++c) m.color_ptr[(size_t)c + 1] += m.color_ptr[(size_t)c];
    std::vector<int> byc((size_t)ne);
    std::vector<int64_t> cc(m.color_ptr.begin(), m.color_ptr.end() - 1);
    for (int64_t e = 0; e < ne; ++e) byc[(size_t)cc[(size_t)color[(size_t)e]]++] = (int)e;
    m.color_elems.alloc((size_t)ne);
    PFG_CUDA(cudaMemcpyAsync(m.color_elems.p, byc.data(), (size_t)ne * sizeof(int), cudaMemcpyHostToDevice, st));
    PFG_CUDA(cudaStreamSynchronize(st));
}

// ------------------------------------------------------------ element math
// Gauss points of ShapeFunctionClass.f90:517-545 (order as listed there,
// weights 1.0) and the node signs of the hex8 shape functions (:1094-1119).
__constant__ double c_sgx[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
__constant__ double c_sgy[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
__constant__ double c_sgz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
#define PFG_GP 0.57735026918962576

__device__ __forceinline__ double shape_N(int a, int gp)
{
    const double g0 = c_sgx[gp] * PFG_GP, g1 = c_sgy[gp] * PFG_GP, g2 = c_sgz[gp] * PFG_GP;
    return 0.125 * (1.0 + c_sgx[a] * g0) * (1.0 + c_sgy[a] * g1) * (1.0 + c_sgz[a] * g2);
}

// J = dN/dxi * ElemCoord (ShapeFunctionClass.f90:1476), detJ by cofactors
// along the first column (MathClass.f90:1460-1476), inverse_rank_2
// (MathClass.f90:1584-1593), and G[a][p] = JPsy(p, a) with
// JPsy = transpose(matmul(transpose(dNdgzi), Jin)) (FEMDomainClass.f90:12289).
__device__ __forceinline__ double gp_geometry_dn(const double (*xe)[3], const double (*dN)[8], double (*G)[3]);

// dN/dxi at Gauss point gp (3 x 8), the values gp_geometry computes.
__device__ __forceinline__ void gp_dshape(int gp, double (*dN)[8])
{
    const double g0 = c_sgx[gp] * PFG_GP, g1 = c_sgy[gp] * PFG_GP, g2 = c_sgz[gp] * PFG_GP;
#pragma unroll
    for (int a = 0; a < 8; ++a) {
        dN[0][a] = 0.125 * c_sgx[a] * (1.0 + c_sgy[a] * g1) * (1.0 + c_sgz[a] * g2);
        dN[1][a] = 0.125 * c_sgy[a] * (1.0 + c_sgx[a] * g0) * (1.0 + c_sgz[a] * g2);
        dN[2][a] = 0.125 * c_sgz[a] * (1.0 + c_sgx[a] * g0) * (1.0 + c_sgy[a] * g1);
    }
}

__device__ __forceinline__ double gp_geometry(const double (*xe)[3], int gp, double (*G)[3])
{
    double dN[3][8];
    gp_dshape(gp, dN);
    return gp_geometry_dn(xe, dN, G);
}

// gp_geometry with dN/dxi given (the element kernel keeps the eight Gauss
// points' tables in shared memory: they are the same for every element).
__device__ __forceinline__ double gp_geometry_dn(const double (*xe)[3], const double (*dN)[8], double (*G)[3])
{
    double J[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
#pragma unroll
            for (int a = 0; a < 8; ++a) s = fma(dN[i][a], xe[a][j], s);
            J[i][j] = s;
        }
    const double m0 = J[1][1] * J[2][2] - J[2][1] * J[1][2];
    const double m1 = J[0][1] * J[2][2] - J[2][1] * J[0][2];
    const double m2 = J[0][1] * J[1][2] - J[1][1] * J[0][2];
    const double det = J[0][0] * m0 - J[1][0] * m1 + J[2][0] * m2;
    if (det == 0.0) return 0.0;
    const double d = 1.0 / det;
    double Ji[3][3];
    Ji[0][0] = d * (J[1][1] * J[2][2] - J[1][2] * J[2][1]);
    Ji[0][1] = d * (J[0][2] * J[2][1] - J[0][1] * J[2][2]);
    Ji[0][2] = d * (J[0][1] * J[1][2] - J[0][2] * J[1][1]);
    Ji[1][0] = d * (J[1][2] * J[2][0] - J[1][0] * J[2][2]);
    Ji[1][1] = d * (J[0][0] * J[2][2] - J[0][2] * J[2][0]);
    Ji[1][2] = d * (J[0][2] * J[1][0] - J[0][0] * J[1][2]);
    Ji[2][0] = d * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    Ji[2][1] = d * (J[0][1] * J[2][0] - J[0][0] * J[2][1]);
    Ji[2][2] = d * (J[0][0] * J[1][1] - J[0][1] * J[1][0]);
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int p = 0; p < 3; ++p) G[a][p] = dN[0][a] * Ji[0][p] + dN[1][a] * Ji[1][p] + dN[2][a] * Ji[2][p];
    return det;
}

// Isotropic Lame constants of DMatrixFEMDomain (FEMDomainClass.f90:11608-11609).
__device__ __forceinline__ void lame(double E, double v, double &lambda, double &mu)
{
    mu = E / 2.0 / (1.0 + v);
    lambda = v * E / (1.0 + v) / (1.0 - 2.0 * v);
}

__device__ __forceinline__ int64_t find_slot(const int64_t *__restrict__ rp, const int *__restrict__ col, int row,
                                             int c, int &nblk)
{
    const int64_t s = rp[row];
    nblk = (int)(rp[row + 1] - s);
    for (int k = 0; k < nblk; ++k)
        if (col[s + k] == c) return k;
    return -1;
}

// Element matrices, four threads per element.  Stiffness: B^T D B detJ summed
// over the Gauss points (FEMDomainClass.f90:11504-11511).  With the Lame
// constants of the element and P_ab = sum_gp detJ g_a g_b^T (g_a the
// gradient of N_a through the reference's J^-T form), the 3x3 block is
// K_ab = lambda P_ab + mu P_ab^T + mu tr(P_ab) I, the product with B of
// :12283-12305 and D of :11626-11637 written out.  Mass: rho sum_gp N_a N_b
// detJ I3 (FEMDomainClass.f90:10934-10936); row-lumped (:10940-10948): the
// row sums on the diagonal blocks.  Only the 36 blocks b >= a are computed
// (K and M are symmetric); each is added at (a, b) and, transposed, at (b, a).
// Thread s of an element takes block rows s and 7 - s (nine blocks each).
// Node coordinates, gradients and detJ of the eight Gauss points live in
// shared memory (the four threads compute two Gauss points each); the slot
// of every block in its CRS row comes from the element's slot map (built
// once per pattern), so the scatter does no search.  FP64-bound: about 4.5k
// DFMA per stiffness element.
constexpr int kEPC = 16;  // elements per CTA

template <int GPU, int MINB>
__global__ void __launch_bounds__(4 * kEPC, MINB)
    k_element_matrix(int64_t n_el, const int *__restrict__ elems, const double *__restrict__ xyz, int64_t nn,
                     const int *__restrict__ conn, int64_t ne, int kind, const double *__restrict__ p0,
                     const double *__restrict__ p1, int bcast, const int64_t *__restrict__ rp,
                     const uint16_t *__restrict__ slots, double *__restrict__ val, int mode, double *__restrict__ out,
                     int *err)
{
    __shared__ double sX[kEPC][8][3];
    __shared__ double sH[kEPC][8][8][3];  // [element][gp][node][dim]: sqrt|detJ| g (G itself where detJ <= 0)
    __shared__ double sW[kEPC][8];
    __shared__ double sDN[8][3][8];       // dN/dxi per Gauss point
    __shared__ int sNode[kEPC][8];
    __shared__ int sPos[kEPC];            // every detJ of the element > 0
    const int q = threadIdx.x >> 2, sub = threadIdx.x & 3;
    for (int gp = threadIdx.x; gp < 8; gp += blockDim.x) gp_dshape(gp, sDN[gp]);
    __syncthreads();
    for (int64_t base = (int64_t)blockIdx.x * kEPC; base < n_el; base += (int64_t)gridDim.x * kEPC) {
        const int64_t li = base + q;
        const bool valid = li < n_el;
        const int e = valid ? (elems ? elems[li] : (int)li) : 0;
        if (valid)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int v = sub + 4 * h;
                const int node = conn[(int64_t)v * ne + e];
                sNode[q][v] = node;
                sX[q][v][0] = xyz[node];
                sX[q][v][1] = xyz[nn + node];
                sX[q][v][2] = xyz[2 * nn + node];
            }
        __syncwarp();
        bool pos = true;
        if (valid)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int gp = sub + 4 * h;
                const double det = gp_geometry_dn(sX[q], sDN[gp], sH[q][gp]);
                sW[q][gp] = det;
                if (det == 0.0) *err = 1;
                pos = pos && det > 0.0;
            }
        {  // the element's four lanes (a quad of the warp) agree on whether every detJ > 0
            int pv = pos ? 1 : 0;
            pv &= __shfl_xor_sync(0xffffffffu, pv, 1);
            pv &= __shfl_xor_sync(0xffffffffu, pv, 2);
            pos = pv != 0;
        }
        __syncwarp();
        if (valid && kind == 0) {
            // P_ab = sum_gp detJ g_a g_b^T = sum_gp h_a h_b^T with h = sqrt(detJ) g when
            // every detJ > 0; otherwise G stays and each term takes its detJ
            if (sub == 0) sPos[q] = pos ? 1 : 0;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int gp = sub + 4 * h;
                if (pos) {
                    const double r = sqrt(sW[q][gp]);
#pragma unroll
                    for (int v = 0; v < 8; ++v)
#pragma unroll
                        for (int d = 0; d < 3; ++d) sH[q][gp][v][d] *= r;
                }
            }
        }
        __syncwarp();
        if (valid) {
            double lam = 0.0, mu = 0.0, rho = 0.0;
            if (kind == 0)
                lame(bcast ? p0[0] : p0[e], bcast ? p1[0] : p1[e], lam, mu);
            else
                rho = bcast ? p0[0] : p0[e];
            const uint16_t *sl = slots ? slots + (int64_t)e * 64 : nullptr;
#pragma unroll 1
            for (int h = 0; h < 2; ++h) {
                const int a = h == 0 ? sub : 7 - sub;
#pragma unroll 1
                for (int b = a; b < 8; ++b) {
                    double K[3][3];
                    if (kind == 0) {
                        double P[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
                        if (sPos[q]) {
#pragma unroll GPU
                            for (int gp = 0; gp < 8; ++gp) {
                                const double ha[3] = {sH[q][gp][a][0], sH[q][gp][a][1], sH[q][gp][a][2]};
                                const double hb[3] = {sH[q][gp][b][0], sH[q][gp][b][1], sH[q][gp][b][2]};
#pragma unroll
                                for (int i = 0; i < 3; ++i)
#pragma unroll
                                    for (int j = 0; j < 3; ++j) P[i][j] = fma(ha[i], hb[j], P[i][j]);
                            }
                        } else {
                            for (int gp = 0; gp < 8; ++gp) {
                                const double w = sW[q][gp];
                                const double wa[3] = {w * sH[q][gp][a][0], w * sH[q][gp][a][1], w * sH[q][gp][a][2]};
                                const double gb[3] = {sH[q][gp][b][0], sH[q][gp][b][1], sH[q][gp][b][2]};
#pragma unroll
                                for (int i = 0; i < 3; ++i)
#pragma unroll
                                    for (int j = 0; j < 3; ++j) P[i][j] = fma(wa[i], gb[j], P[i][j]);
                            }
                        }
                        const double mt = mu * (P[0][0] + P[1][1] + P[2][2]);
#pragma unroll
                        for (int i = 0; i < 3; ++i)
#pragma unroll
                            for (int j = 0; j < 3; ++j)
                                K[i][j] = fma(lam, P[i][j], mu * P[j][i]) + (i == j ? mt : 0.0);
                    } else {
                        double m = 0.0;
                        if (kind == 1) {
#pragma unroll
                            for (int gp = 0; gp < 8; ++gp) m += shape_N(a, gp) * shape_N(b, gp) * sW[q][gp];
                            m *= rho;
                        } else if (a == b) {
                            for (int bb = 0; bb < 8; ++bb) {
                                double mb = 0.0;
#pragma unroll
                                for (int gp = 0; gp < 8; ++gp) mb += shape_N(a, gp) * shape_N(bb, gp) * sW[q][gp];
                                m += rho * mb;
                            }
                        }
#pragma unroll
                        for (int i = 0; i < 3; ++i)
#pragma unroll
                            for (int j = 0; j < 3; ++j) K[i][j] = (i == j) ? m : 0.0;
                        if (kind == 2 && a != b && mode == 0) continue;  // lumped: diagonal blocks only
                    }
                    if (mode == 1) {
                        double *o = out + (int64_t)e * 576;
#pragma unroll
                        for (int i = 0; i < 3; ++i)
#pragma unroll
                            for (int j = 0; j < 3; ++j) {
                                o[(3 * b + j) * 24 + 3 * a + i] = K[i][j];
                                if (a != b) o[(3 * a + i) * 24 + 3 * b + j] = K[i][j];
                            }
                        continue;
                    }
                    {
                        const int ra = sNode[q][a];
                        const int64_t r0 = rp[ra];
                        const int nblk = (int)(rp[ra + 1] - r0);
                        double *v = val + r0 * 9 + sl[a * 8 + b];
#pragma unroll
                        for (int i = 0; i < 3; ++i)
#pragma unroll
                            for (int j = 0; j < 3; ++j) v[(int64_t)(3 * i + j) * nblk] += K[i][j];
                    }
                    if (a != b) {
                        const int rb = sNode[q][b];
                        const int64_t r0 = rp[rb];
                        const int nblk = (int)(rp[rb + 1] - r0);
                        double *v = val + r0 * 9 + sl[b * 8 + a];
#pragma unroll
                        for (int i = 0; i < 3; ++i)
#pragma unroll
                            for (int j = 0; j < 3; ++j) v[(int64_t)(3 * j + i) * nblk] += K[i][j];
                    }
                }
            }
        }
        __syncwarp();
    }
}

// Slot map of the coloured assembly: slots[e * 64 + a * 8 + b] = position of
// block column node(b) in block row node(a).  A thread per (element, a).
// err = 2: a block has no slot (not the mesh's pattern); 3: a row longer than
// 65,535 blocks.
__global__ void k_slot_map(int64_t ne, const int *__restrict__ conn, const int64_t *__restrict__ rp,
                           const int *__restrict__ col, uint16_t *__restrict__ slots, int *err)
{
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < ne * 8;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = t >> 3;
        const int a = (int)(t & 7);
        const int row = conn[(int64_t)a * ne + e];
        const int64_t r0 = rp[row];
        const int n = (int)(rp[row + 1] - r0);
        if (n > 65535) *err = 3;
        for (int b = 0; b < 8; ++b) {
            const int c = conn[(int64_t)b * ne + e];
            int k = 0;
            while (k < n && col[r0 + k] != c) ++k;
            if (k == n) *err = 2;
            slots[e * 64 + a * 8 + b] = (uint16_t)(k < n ? k : 0);
        }
    }
}

static void check_err(DevBuf<int> &err, cudaStream_t st)
{
    int h = 0;
    PFG_CUDA(cudaMemcpyAsync(&h, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    PFG_CUDA(cudaStreamSynchronize(st));
    PFG_CHECK(h != 1, PFG_E_DETJ, "element with detJ == 0 (the reference stops with \"Bmat,detJ=0\")");
    PFG_CHECK(h != 2, PFG_E_MISSING_SLOT, "no CRS slot for an element block (fill-in request)");
}

static void ensure_slot_map(const DevMesh &m, const DevMatrix &K, cudaStream_t st)
{
    if (m.slots_gen == K.pattern_gen && m.slots.p) return;
    m.slots.resize((size_t)m.ne * 64);
    DevBuf<int> err(1);
    PFG_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
    k_slot_map<<<grid_for(m.ne * 8, 256), 256, 0, st>>>(m.ne, m.conn.p, K.rp.p, K.col.p, m.slots.p, err.p);
    PFG_CUDA(cudaGetLastError());
    int h = 0;
    PFG_CUDA(cudaMemcpyAsync(&h, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    PFG_CUDA(cudaStreamSynchronize(st));
    PFG_CHECK(h != 2, PFG_E_MISSING_SLOT, "no CRS slot for an element block (fill-in request)");
    PFG_CHECK(h != 3, PFG_E_UNSUPPORTED, "a CRS block row longer than 65,535 blocks");
    m.slots_gen = K.pattern_gen;
}

template <typename Kern>
static int element_grid(Kern kern, int64_t n)
{
    int per_sm = 0;
    PFG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 4 * kEPC, 0));
    if (per_sm <= 0) per_sm = 1;
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + kEPC - 1) / kEPC, (int64_t)per_sm * sm_count_device()));
}

// The element kernel's configuration: Gauss-point loop unrolled 4x, at least
// 6 CTAs per SM (168 registers).  Measured at 100^3 (1M elements, 8 colour
// launches): 22.1 ms against 23.2 ms fully unrolled (252 registers) and
// 27.1 ms at 128 registers (spills).
using ElementKernel = void (*)(int64_t, const int *, const double *, int64_t, const int *, int64_t, int,
                               const double *, const double *, int, const int64_t *, const uint16_t *, double *, int,
                               double *, int *);
static const ElementKernel kElementKernel = k_element_matrix<4, 6>;

template <typename... Args>
static void launch_element_matrix(int64_t n, cudaStream_t st, Args... args)
{
    kElementKernel<<<element_grid(kElementKernel, n), 4 * kEPC, 0, st>>>(n, args...);
}

void assemble_elements(const DevMesh &m, DevMatrix &K, int kind, const double *p0, const double *p1, bool broadcast,
                       cudaStream_t st)
{
    PFG_CHECK(K.bs == 3 && K.nb == m.nn, PFG_E_STATE, "pattern not built for this mesh (call setCRS(DOF=3))");
    PFG_CHECK(!m.color_ptr.empty(), PFG_E_STATE, "mesh not coloured");
    ensure_slot_map(m, K, st);
    DevBuf<int> err(1);
    PFG_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
    for (size_t c = 0; c + 1 < m.color_ptr.size(); ++c) {
        const int64_t n = m.color_ptr[c + 1] - m.color_ptr[c];
        if (n == 0) continue;
        launch_element_matrix(n, st, (const int *)(m.color_elems.p + m.color_ptr[c]), (const double *)m.xyz.p,
                              m.nn, (const int *)m.conn.p, m.ne, kind, p0, p1, broadcast ? 1 : 0,
                              (const int64_t *)K.rp.p, (const uint16_t *)m.slots.p, K.v64.p, 0, (double *)nullptr,
                              err.p);
        PFG_CUDA(cudaGetLastError());
    }
    K.values_changed();
    check_err(err, st);
}

void element_stiffness(const DevMesh &m, const double *E, const double *nu, bool broadcast, double *out,
                       cudaStream_t st)
{
    DevBuf<int> err(1);
    PFG_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
    launch_element_matrix(m.ne, st, (const int *)nullptr, (const double *)m.xyz.p, m.nn, (const int *)m.conn.p,
                          m.ne, 0, E, nu, broadcast ? 1 : 0, (const int64_t *)nullptr, (const uint16_t *)nullptr,
                          (double *)nullptr, 1, out, err.p);
    PFG_CUDA(cudaGetLastError());
    check_err(err, st);
}

// Body force per element, scattered per colour (MassVectorFEMDomain, FEMDomainClass.f90:11063-11070).
__global__ void k_body_force(int64_t n_el, const int *__restrict__ elems, const double *__restrict__ xyz, int64_t nn,
                             const int *__restrict__ conn, int64_t ne, const double *__restrict__ rho, int bcast,
                             double ax, double ay, double az, double *__restrict__ rhs, int *err)
{
    for (int64_t li = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; li < n_el; li += (int64_t)gridDim.x * blockDim.x) {
        const int e = elems[li];
        double xe[8][3];
        int node[8];
#pragma unroll
        for (int a = 0; a < 8; ++a) {
            const int v = conn[(int64_t)a * ne + e];
            node[a] = v;
            xe[a][0] = xyz[v];
            xe[a][1] = xyz[nn + v];
            xe[a][2] = xyz[2 * nn + v];
        }
        double f[8];
#pragma unroll
        for (int a = 0; a < 8; ++a) f[a] = 0.0;
        for (int gp = 0; gp < 8; ++gp) {
            double G[8][3];
            const double det = gp_geometry(xe, gp, G);
            if (det == 0.0) *err = 1;
#pragma unroll
            for (int a = 0; a < 8; ++a) f[a] += shape_N(a, gp) * det;
        }
        const double r = bcast ? rho[0] : rho[e];
#pragma unroll
        for (int a = 0; a < 8; ++a) {
            rhs[3 * (int64_t)node[a] + 0] += r * (f[a] * ax);
            rhs[3 * (int64_t)node[a] + 1] += r * (f[a] * ay);
            rhs[3 * (int64_t)node[a] + 2] += r * (f[a] * az);
        }
    }
}

void assemble_body_force(const DevMesh &m, double *rhs, const double *rho, bool broadcast, const double accel[3],
                         cudaStream_t st)
{
    PFG_CHECK(!m.color_ptr.empty(), PFG_E_STATE, "mesh not coloured");
    DevBuf<int> err(1);
    PFG_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
    for (size_t c = 0; c + 1 < m.color_ptr.size(); ++c) {
        const int64_t n = m.color_ptr[c + 1] - m.color_ptr[c];
        if (n == 0) continue;
        k_body_force<<<grid_for(n, 128, sm_count_device() * 16), 128, 0, st>>>(n, m.color_elems.p + m.color_ptr[c], m.xyz.p, m.nn,
                                                                 m.conn.p, m.ne, rho, broadcast ? 1 : 0, accel[0],
                                                                 accel[1], accel[2], rhs, err.p);
        PFG_CUDA(cudaGetLastError());
    }
    check_err(err, st);
}

// User element matrices (24x24 column-major): atomic adds, since a batch may
// repeat an element or hold elements that share nodes.
__global__ void k_scatter_mats(int64_t count, const int *__restrict__ ids, const double *__restrict__ mats,
                               const int *__restrict__ conn, int64_t ne, const int64_t *__restrict__ rp,
                               const int *__restrict__ col, double *__restrict__ val, int *err)
{
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < count * 64; w += (int64_t)gridDim.x * blockDim.x) {
        const int64_t q = w >> 6;
        const int a = (int)(w & 63) >> 3, b = (int)(w & 7);
        const int e = ids[q];
        if (e < 0 || e >= ne) { *err = 3; continue; }
        const int ra = conn[(int64_t)a * ne + e], rb = conn[(int64_t)b * ne + e];
        int nblk;
        const int64_t k = find_slot(rp, col, ra, rb, nblk);
        if (k < 0) { *err = 2; continue; }
        double *v = val + rp[ra] * 9 + k;
        const double *M = mats + q * 576;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) atomicAdd(v + (int64_t)(3 * i + j) * nblk, M[(3 * b + j) * 24 + 3 * a + i]);
    }
}

void scatter_element_matrices(const DevMesh &m, DevMatrix &K, int64_t count, const int *ids, const double *mats,
                              cudaStream_t st)
{
    if (count == 0) return;
    PFG_CHECK(K.bs == 3 && K.nb == m.nn, PFG_E_STATE, "pattern not built for this mesh (call setCRS(DOF=3))");
    DevBuf<int> err(1);
    PFG_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
    k_scatter_mats<<<grid_for(count * 64, 256, sm_count_device() * 16), 256, 0, st>>>(count, ids, mats, m.conn.p, m.ne, K.rp.p,
                                                                        K.col.p, K.v64.p, err.p);
    PFG_CUDA(cudaGetLastError());
    K.values_changed();
    int h = 0;
    PFG_CUDA(cudaMemcpyAsync(&h, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    PFG_CUDA(cudaStreamSynchronize(st));
    PFG_CHECK(h != 3, PFG_E_ARG, "element id out of range");
    PFG_CHECK(h != 2, PFG_E_MISSING_SLOT, "no CRS slot for an element block (fill-in request)");
}

__global__ void k_scatter_vecs(int64_t count, const int *__restrict__ ids, const double *__restrict__ vecs,
                               const int *__restrict__ conn, int64_t ne, double *__restrict__ rhs, int *err)
{
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < count * 24; w += (int64_t)gridDim.x * blockDim.x) {
        const int64_t q = w / 24;
        const int l = (int)(w % 24);
        const int e = ids[q];
        if (e < 0 || e >= ne) { *err = 3; continue; }
        const int v = conn[(int64_t)(l / 3) * ne + e];
        atomicAdd(rhs + 3 * (int64_t)v + (l % 3), vecs[q * 24 + l]);
    }
}

void scatter_element_vectors(const DevMesh &m, double *rhs, int64_t count, const int *ids, const double *vecs,
                             cudaStream_t st)
{
    if (count == 0) return;
    DevBuf<int> err(1);
    PFG_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
    k_scatter_vecs<<<grid_for(count * 24, 256, sm_count_device() * 16), 256, 0, st>>>(count, ids, vecs, m.conn.p, m.ne, rhs, err.p);
    PFG_CUDA(cudaGetLastError());
    int h = 0;
    PFG_CUDA(cudaMemcpyAsync(&h, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    PFG_CUDA(cudaStreamSynchronize(st));
    PFG_CHECK(h != 3, PFG_E_ARG, "element id out of range");
}

// Strain vector of the reference's B rows (FEMDomainClass.f90:12292-12303):
// [exx, eyy, ezz, gxy, gyz, gzx] at one Gauss point.
__device__ __forceinline__ void strain(const double (*G)[3], const double (*u)[3], double (&eps)[6])
{
#pragma unroll
    for (int k = 0; k < 6; ++k) eps[k] = 0.0;
#pragma unroll
    for (int a = 0; a < 8; ++a) {
        eps[0] += G[a][0] * u[a][0];
        eps[1] += G[a][1] * u[a][1];
        eps[2] += G[a][2] * u[a][2];
        eps[3] += G[a][1] * u[a][0] + G[a][0] * u[a][1];
        eps[4] += G[a][2] * u[a][1] + G[a][1] * u[a][2];
        eps[5] += G[a][2] * u[a][0] + G[a][0] * u[a][2];
    }
}

// StressMatrixFEMDomain without GaussPoint (FEMDomainClass.f90:11985-12032):
// mean over the Gauss points of D B u_e; disp node-interleaved (plantFEM's
// row-major reshape, ArrayClass.f90:5328-5344).
__global__ void k_stress(int64_t ne, const double *__restrict__ xyz, int64_t nn, const int *__restrict__ conn,
                         const double *__restrict__ disp, const double *__restrict__ E, const double *__restrict__ nu,
                         int bcast, double *__restrict__ out, int *err)
{
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
        double xe[8][3], ue[8][3];
#pragma unroll
        for (int a = 0; a < 8; ++a) {
            const int v = conn[(int64_t)a * ne + e];
            xe[a][0] = xyz[v];
            xe[a][1] = xyz[nn + v];
            xe[a][2] = xyz[2 * nn + v];
            ue[a][0] = disp[3 * (int64_t)v];
            ue[a][1] = disp[3 * (int64_t)v + 1];
            ue[a][2] = disp[3 * (int64_t)v + 2];
        }
        double lam, mu;
        lame(bcast ? E[0] : E[e], bcast ? nu[0] : nu[e], lam, mu);
        double S[6] = {0, 0, 0, 0, 0, 0};
        for (int gp = 0; gp < 8; ++gp) {
            double G[8][3], eps[6];
            if (gp_geometry(xe, gp, G) == 0.0) *err = 1;
            strain(G, ue, eps);
            const double tr = eps[0] + eps[1] + eps[2];
            S[0] += lam * tr + 2.0 * mu * eps[0];
            S[1] += lam * tr + 2.0 * mu * eps[1];
            S[2] += lam * tr + 2.0 * mu * eps[2];
            S[3] += mu * eps[3];
            S[4] += mu * eps[4];
            S[5] += mu * eps[5];
        }
        double *o = out + e * 9;
        o[0] = S[0] / 8.0; o[4] = S[1] / 8.0; o[8] = S[2] / 8.0;
        o[1] = o[3] = S[3] / 8.0;
        o[5] = o[7] = S[4] / 8.0;
        o[2] = o[6] = S[5] / 8.0;
    }
}

// One number per element from its cell-averaged stress tensor S (row-major),
// the options of getElementCauchyStress (FEMDomainClass.f90:15310-15362):
// 1 I1 = tr S, 2 p = tr S / 3, 3 I2 = (tr(S)^2 - tr(S S)) / 2, 4 I3 = det S
// (cofactors along the first column, det_mat of MathClass.f90:1460-1476),
// 5-7 the same three of the deviator s = S - tr(S)/3 I (J1 = tr s, J2, J3),
// 10 + 3 (i-1) + (j-1): the component S(i, j).  Other codes leave 0, as the
// reference's select case does for an unknown option.
__device__ __forceinline__ double det3_first_column(const double *a)
{
    return a[0] * (a[4] * a[8] - a[7] * a[5]) - a[3] * (a[1] * a[8] - a[7] * a[2]) +
           a[6] * (a[1] * a[5] - a[4] * a[2]);
}

__global__ void k_stress_option(int64_t ne, const double *__restrict__ S, int option, double *__restrict__ out)
{
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
        double a[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) a[k] = S[e * 9 + k];
        double r = 0.0;
        if (option >= 10 && option <= 18) {
            r = a[option - 10];
        } else if (option >= 1 && option <= 7) {
            double tr = a[0] + a[4] + a[8];
            if (option >= 5) {  // the deviator
                const double m = tr / 3.0;
                a[0] -= m;
                a[4] -= m;
                a[8] -= m;
                tr = a[0] + a[4] + a[8];
            }
            const int inv = option >= 5 ? option - 4 : (option == 2 ? 0 : (option == 1 ? 1 : option - 1));
            if (inv == 0) {
                r = tr / 3.0;
            } else if (inv == 1) {
                r = tr;
            } else if (inv == 2) {
                double trss = 0.0;  // tr(S S)
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int k = 0; k < 3; ++k) trss += a[3 * i + k] * a[3 * k + i];
                r = (tr * tr - trss) * 0.5;
            } else {
                r = det3_first_column(a);
            }
        }
        out[e] = r;
    }
}

void element_stress_option(int64_t ne, const double *S, int option, double *out, cudaStream_t st)
{
    k_stress_option<<<grid_for(ne, 256), 256, 0, st>>>(ne, S, option, out);
    PFG_CUDA(cudaGetLastError());
}

void element_stress(const DevMesh &m, const double *disp, const double *E, const double *nu, bool broadcast,
                    double *out, cudaStream_t st)
{
    DevBuf<int> err(1);
    PFG_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
    k_stress<<<grid_for(m.ne, 128, sm_count_device() * 16), 128, 0, st>>>(m.ne, m.xyz.p, m.nn, m.conn.p, disp, E, nu,
                                                            broadcast ? 1 : 0, out, err.p);
    PFG_CUDA(cudaGetLastError());
    check_err(err, st);
}

// g_e = -lambda_e^T (K_e / E_e) u_e = -sum_gp detJ eps(lambda)^T D(1, nu) eps(u).
__global__ void k_adjoint_grad(int64_t ne, const double *__restrict__ xyz, int64_t nn, const int *__restrict__ conn,
                               const double *__restrict__ u, const double *__restrict__ lm,
                               const double *__restrict__ nu, int bcast, double *__restrict__ grad, int *err)
{
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
        double xe[8][3], ue[8][3], le[8][3];
#pragma unroll
        for (int a = 0; a < 8; ++a) {
            const int v = conn[(int64_t)a * ne + e];
            xe[a][0] = xyz[v];
            xe[a][1] = xyz[nn + v];
            xe[a][2] = xyz[2 * nn + v];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                ue[a][d] = u[3 * (int64_t)v + d];
                le[a][d] = lm[3 * (int64_t)v + d];
            }
        }
        double lam, mu;
        lame(1.0, bcast ? nu[0] : nu[e], lam, mu);
        double s = 0.0;
        for (int gp = 0; gp < 8; ++gp) {
            double G[8][3], eu[6], el[6];
            const double det = gp_geometry(xe, gp, G);
            if (det == 0.0) *err = 1;
            strain(G, ue, eu);
            strain(G, le, el);
            const double tru = eu[0] + eu[1] + eu[2], trl = el[0] + el[1] + el[2];
            const double w = lam * tru * trl + 2.0 * mu * (eu[0] * el[0] + eu[1] * el[1] + eu[2] * el[2]) +
                             mu * (eu[3] * el[3] + eu[4] * el[4] + eu[5] * el[5]);
            s += det * w;
        }
        grad[e] = -s;
    }
}

void adjoint_grad_E(const DevMesh &m, const double *u, const double *lam, const double *nu, bool broadcast,
                    double *grad, cudaStream_t st)
{
    DevBuf<int> err(1);
    PFG_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
    k_adjoint_grad<<<grid_for(m.ne, 128, sm_count_device() * 16), 128, 0, st>>>(m.ne, m.xyz.p, m.nn, m.conn.p, u, lam, nu,
                                                                  broadcast ? 1 : 0, grad, err.p);
    PFG_CUDA(cudaGetLastError());
    check_err(err, st);
}

// --------------------------------------------------- Dirichlet elimination
// One thread per block row.  The lift keeps the reference's order (row entries
// in column order) and rounding (separate multiply and subtract).
template <int BS>
__global__ void k_dirichlet(int64_t nb, const int64_t *__restrict__ rp, const int *__restrict__ col,
                            double *__restrict__ val, double *__restrict__ rhs, const uint8_t *__restrict__ fixed,
                            const double *__restrict__ fixval)
{
    for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < nb; row += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = rp[row];
        const int nblk = (int)(rp[row + 1] - s);
        double *v = val + s * BS * BS;
#pragma unroll
        for (int r = 0; r < BS; ++r) {
            const int64_t i = (int64_t)BS * row + r;
            const bool fi = fixed[i] != 0;
            double acc = rhs[i];
            for (int k = 0; k < nblk; ++k) {
                const int c = col[s + k];
#pragma unroll
                for (int cc = 0; cc < BS; ++cc) {
                    const int64_t j = (int64_t)BS * c + cc;
                    double &a = v[(int64_t)(r * BS + cc) * nblk + k];
                    const bool fj = fixed[j] != 0;
                    if (fj) acc = __dsub_rn(acc, __dmul_rn(a, fixval[j]));
                    if (fi || fj) a = (fi && i == j) ? 1.0 : 0.0;
                }
            }
            rhs[i] = fi ? fixval[i] : acc;
        }
    }
}

void apply_dirichlet(DevMatrix &K, double *rhs, const uint8_t *fixed, const double *fixval, cudaStream_t st)
{
    const int g = grid_for(K.nb, 128, sm_count_device() * 16);
    if (K.bs == 3)
        k_dirichlet<3><<<g, 128, 0, st>>>(K.nb, K.rp.p, K.col.p, K.v64.p, rhs, fixed, fixval);
    else
        k_dirichlet<1><<<g, 128, 0, st>>>(K.nb, K.rp.p, K.col.p, K.v64.p, rhs, fixed, fixval);
    PFG_CUDA(cudaGetLastError());
    K.values_changed();
}

__global__ void k_restore_fixed(int64_t n, double *x, const uint8_t *fixed, const double *fixval)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (fixed[i]) x[i] = fixval[i];
}

void restore_fixed(int64_t n, double *x, const uint8_t *fixed, const double *fixval, cudaStream_t st)
{
    k_restore_fixed<<<grid_for(n, 256, sm_count_device() * 8), 256, 0, st>>>(n, x, fixed, fixval);
    PFG_CUDA(cudaGetLastError());
}

// ------------------------------------------------------------ CRS in / out
// 3x3 node-block structure check: rows 3I..3I+2 have equal length L = 3*nblk
// and row 3I+r holds [3c+1, 3c+2, 3c+3] for the same node sequence c.
// A scalar CRS is taken as 3x3 blocks when every node row I has three scalar
// rows 3I..3I+2 of equal length L (a multiple of 3), starting at a multiple of
// 9 entries, and each group of three columns reads 3c+1, 3c+2, 3c+3 in all
// three rows (the layout FEMDomainClass.f90:10780-10836 produces).  The three
// rows of node row I are then one contiguous run of 3L entries.  One warp per
// node row, lanes over the run (coalesced).
__global__ void k_check_blocks(int64_t nb, const int64_t *__restrict__ row_ptr, const int32_t *__restrict__ col_idx,
                               int64_t n, int *ok)
{
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t I = w0; I < nb; I += nw) {
        const int64_t s0 = row_ptr[3 * I] - 1;
        const int64_t L = row_ptr[3 * I + 1] - row_ptr[3 * I];
        bool good = (L % 3) == 0 && (s0 % 9) == 0 && row_ptr[3 * I + 2] - row_ptr[3 * I + 1] == L &&
                    row_ptr[3 * I + 3] - row_ptr[3 * I + 2] == L;
        if (good) {
            for (int64_t t = lane; t < 3 * L; t += 32) {
                const int64_t q = t % L, k = q / 3, cc = q % 3;
                const int32_t c0 = col_idx[s0 + 3 * k];
                if ((c0 - 1) % 3 != 0 || c0 < 1 || c0 > n || col_idx[s0 + t] != c0 + (int32_t)cc) good = false;
            }
        }
        if (__any_sync(0xffffffffu, !good) && lane == 0) *ok = 0;
    }
}

// Scalar CRS (checked by k_check_blocks) -> the block-row layout (bsr.cuh):
// node row I's run of 9 nblk values, entry t = r (3 nblk) + 3k + c, lands at
// bval[9 bs + (3r + c) nblk + k].  One warp per node row: coalesced reads,
// writes inside the row's own 72 nblk bytes.
__global__ void k_import_b3(int64_t nb, const int64_t *__restrict__ row_ptr, const int32_t *__restrict__ col_idx,
                            const double *__restrict__ val, int64_t *__restrict__ rp, int *__restrict__ bcol,
                            double *__restrict__ bval)
{
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t I = w0; I < nb; I += nw) {
        const int64_t s0 = row_ptr[3 * I] - 1;
        const int nblk = (int)((row_ptr[3 * I + 1] - row_ptr[3 * I]) / 3);
        const int64_t bs = s0 / 9;
        if (lane == 0) {
            rp[I] = bs;
            if (I == nb - 1) rp[nb] = bs + nblk;
        }
        for (int k = lane; k < nblk; k += 32) bcol[bs + k] = (col_idx[s0 + 3 * k] - 1) / 3;
        if (val == nullptr) continue;
        const int run = 3 * nblk;
        for (int t = lane; t < 3 * run; t += 32) {
            const int r = t / run, q = t - r * run, k = q / 3, c = q - 3 * k;
            bval[bs * 9 + (int64_t)(3 * r + c) * nblk + k] = val[s0 + t];
        }
    }
}

__global__ void k_import_b1(int64_t n, const int64_t *__restrict__ row_ptr, const int32_t *__restrict__ col_idx,
                            int64_t nnz, int64_t *__restrict__ rp, int *__restrict__ bcol, int *bad)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += (int64_t)gridDim.x * blockDim.x) {
        rp[i] = row_ptr[i] - 1;
        if (i > 0 && row_ptr[i] < row_ptr[i - 1]) *bad = 1;
    }
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x) {
        const int32_t c = col_idx[k];
        if (c < 1 || c > n) *bad = 1;
        bcol[k] = c - 1;
    }
}

void import_crs(int64_t n, int64_t nnz, const int64_t *row_ptr, const int32_t *col_idx, const double *val,
                DevMatrix &K, cudaStream_t st, bool allow_blocks)
{
    PFG_CHECK(n > 0, PFG_E_ARG, "empty CRS");
    DevBuf<int> ok(1);
    int hok = 0;
    if (allow_blocks && n % 3 == 0 && val != nullptr) {
        hok = 1;
        PFG_CUDA(cudaMemcpyAsync(ok.p, &hok, sizeof(int), cudaMemcpyHostToDevice, st));
        k_check_blocks<<<grid_for(n / 3, 256, sm_count_device() * 16), 256, 0, st>>>(n / 3, row_ptr, col_idx, n, ok.p);
        PFG_CUDA(cudaGetLastError());
        PFG_CUDA(cudaMemcpyAsync(&hok, ok.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        PFG_CUDA(cudaStreamSynchronize(st));
    }
    // keep the FP32 buffer (and its address): it is rebuilt from v64 on demand
    K.pattern_changed();
    if (hok) {
        const int64_t nb = n / 3;
        K.bs = 3;
        K.nb = nb;
        K.nnzb = nnz / 9;
        K.rp.resize((size_t)nb + 1);
        K.col.resize((size_t)std::max<int64_t>(K.nnzb, 1));
        K.v64.resize((size_t)std::max<int64_t>(nnz, 1));
        k_import_b3<<<grid_for(nb, 128, sm_count_device() * 16), 128, 0, st>>>(nb, row_ptr, col_idx, val, K.rp.p, K.col.p,
                                                                 K.v64.p);
        PFG_CUDA(cudaGetLastError());
    } else {
        K.bs = 1;
        K.nb = n;
        K.nnzb = nnz;
        K.rp.resize((size_t)n + 1);
        K.col.resize((size_t)std::max<int64_t>(nnz, 1));
        K.v64.resize((size_t)std::max<int64_t>(nnz, 1));
        int zero = 0;
        PFG_CUDA(cudaMemcpyAsync(ok.p, &zero, sizeof(int), cudaMemcpyHostToDevice, st));
        k_import_b1<<<grid_for(std::max(n + 1, nnz), 256, sm_count_device() * 16), 256, 0, st>>>(n, row_ptr, col_idx, nnz, K.rp.p,
                                                                                   K.col.p, ok.p);
        PFG_CUDA(cudaGetLastError());
        if (nnz && val) PFG_CUDA(cudaMemcpyAsync(K.v64.p, val, nnz * sizeof(double), cudaMemcpyDeviceToDevice, st));
        int bad = 0;
        PFG_CUDA(cudaMemcpyAsync(&bad, ok.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        PFG_CUDA(cudaStreamSynchronize(st));
        PFG_CHECK(!bad, PFG_E_ARG, "CRS row_ptr not monotone or col_idx out of 1..n");
    }
}

__global__ void k_export_b3(int64_t nb, const int64_t *__restrict__ rp, const int *__restrict__ bcol,
                            const double *__restrict__ bval, int64_t *__restrict__ row_ptr, int32_t *__restrict__ col_idx,
                            double *__restrict__ val)
{
    for (int64_t I = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; I < nb; I += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = rp[I];
        const int nblk = (int)(rp[I + 1] - s);
        for (int r = 0; r < 3; ++r) {
            // row 3I+r starts at 9 s + 3 r nblk (FEMDomainClass.f90:10785-10796)
            const int64_t o = 9 * s + (int64_t)3 * r * nblk;
            if (row_ptr) {
                row_ptr[3 * I + r] = o + 1;
                if (I == nb - 1 && r == 2) row_ptr[3 * nb] = 9 * (s + nblk) + 1;
            }
            for (int k = 0; k < nblk; ++k)
                for (int c = 0; c < 3; ++c) {
                    if (col_idx) col_idx[o + 3 * k + c] = 3 * bcol[s + k] + c + 1;
                    if (val) val[o + 3 * k + c] = bval[9 * s + (int64_t)(3 * r + c) * nblk + k];
                }
        }
    }
}

__global__ void k_export_b1(int64_t n, int64_t nnz, const int64_t *__restrict__ rp, const int *__restrict__ bcol,
                            int64_t *__restrict__ row_ptr, int32_t *__restrict__ col_idx)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += (int64_t)gridDim.x * blockDim.x)
        if (row_ptr) row_ptr[i] = rp[i] + 1;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x)
        if (col_idx) col_idx[k] = bcol[k] + 1;
}

void export_values(const DevMatrix &K, const double *bval, double *val, cudaStream_t st)
{
    if (K.bs == 3)
        k_export_b3<<<grid_for(K.nb, 128, sm_count_device() * 16), 128, 0, st>>>(K.nb, K.rp.p, K.col.p, bval, nullptr, nullptr,
                                                                   val);
    else if (K.nnzb)
        PFG_CUDA(cudaMemcpyAsync(val, bval, K.nnzb * sizeof(double), cudaMemcpyDeviceToDevice, st));
    PFG_CUDA(cudaGetLastError());
}

void export_crs(const DevMatrix &K, int64_t *row_ptr, int32_t *col_idx, double *val, cudaStream_t st)
{
    if (K.bs == 3) {
        k_export_b3<<<grid_for(K.nb, 128, sm_count_device() * 16), 128, 0, st>>>(K.nb, K.rp.p, K.col.p, K.v64.p, row_ptr, col_idx,
                                                                   val);
    } else {
        k_export_b1<<<grid_for(std::max(K.nb + 1, K.nnzb), 256, sm_count_device() * 16), 256, 0, st>>>(K.nb, K.nnzb, K.rp.p,
                                                                                        K.col.p, row_ptr, col_idx);
        if (val && K.nnzb)
            PFG_CUDA(cudaMemcpyAsync(val, K.v64.p, K.nnzb * sizeof(double), cudaMemcpyDeviceToDevice, st));
    }
    PFG_CUDA(cudaGetLastError());
}

}  // namespace pfg
