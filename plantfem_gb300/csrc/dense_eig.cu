// dense_eig.cu -- the dense branch of FEMSolver_%eig on the device.
//
// With use_LOBPCG = .false. (the reference's default, FEMSolverClass.f90:73),
// eigFEMSolver (:1384-1541) drops the fix_eig DOFs from A and B
// (reduce_crs_matrix), packs both upper triangles and calls LAPACK DSPGVD
// (ITYPE = 1, JOBZ = 'V', UPLO = 'U'): every eigenpair of A z = lambda B z,
// ascending, B-orthonormal vectors, scattered back with zeros at the fixed
// DOFs.  Here the same problem is solved in FP64 on the GPU by a method of
// our own choosing (DSPGVD is an un-vendored LAPACK routine):
//   1. Cholesky factor B = L L^T (right-looking, one launch pair per column);
//   2. C = L^-1 A L^-T by two forward substitutions (C = L^-1 (L^-1 A)^T, A
//      symmetric), a thread per right-hand side;
//   3. C = Q diag(lambda) Q^T by the cyclic Jacobi method with a round-robin
//      ("tournament") ordering, so every step rotates N/2 disjoint pairs at
//      once (Jacobi 1846; parallel ordering after Brent & Luk 1985), with
//      Rutishauser's rotation formulas (Golub & Van Loan, Matrix
//      Computations, sec. 8.5);
//   4. Z = L^-T Q by back substitution; pairs sorted ascending.
// All matrices are dense row-major N x N in device memory; N is bounded
// (kDenseEigMax), as the reference's packed dense problem is.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "lobpcg.cuh"

namespace pfg {

// ---------------------------------------------------------------- assembly
// Dense reduced matrix from a block matrix: entry (3i+r, 3j+c) of block
// (i, j) goes to (map[3i+r], map[3j+c]) when neither DOF is fixed (map < 0).
__global__ void k_dense_from_blocks(int64_t nb, int bs, const int64_t *__restrict__ rp, const int *__restrict__ col,
                                    const double *__restrict__ v, const int *__restrict__ map, int N,
                                    double *__restrict__ D)
{
    const int bs2 = bs * bs;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r0 = rp[i];
        const int nblk = (int)(rp[i + 1] - r0);
        for (int k = 0; k < nblk; ++k) {
            const int j = col[r0 + k];
            for (int e = 0; e < bs2; ++e) {
                const int r = e / bs, c = e % bs;
                const int nr = map[(int64_t)bs * i + r], nc = map[(int64_t)bs * j + c];
                if (nr >= 0 && nc >= 0) D[(int64_t)nr * N + nc] = v[r0 * bs2 + (int64_t)e * nblk + k];
            }
        }
    }
}

// ---------------------------------------------------------------- Cholesky
// Step k, part 1: trailing update of the lower triangle, B_ij -= B_ik B_jk / B_kk
// for k < j <= i (column k still unscaled).  err = 1 if B_kk <= 0.
__global__ void k_chol_update(int N, int k, double *__restrict__ B, int *err)
{
    const double d = B[(int64_t)k * N + k];
    if (!(d > 0.0)) {
        if (blockIdx.x == 0 && threadIdx.x == 0) *err = 1;
        return;
    }
    const int64_t m = N - 1 - k;  // trailing size
    const int64_t total = m * (m + 1) / 2;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        // t -> (ii, jj) with 0 <= jj <= ii < m, row-major over the lower triangle
        int64_t ii = (int64_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
        while (ii * (ii + 1) / 2 > t) --ii;
        while ((ii + 1) * (ii + 2) / 2 <= t) ++ii;
        const int64_t jj = t - ii * (ii + 1) / 2;
        const int64_t i = k + 1 + ii, j = k + 1 + jj;
        B[i * N + j] -= B[i * N + k] * B[j * N + k] / d;
    }
}

// Step k, part 2: L_kk = sqrt(B_kk), L_ik = B_ik / L_kk for i > k.
__global__ void k_chol_scale(int N, int k, double *__restrict__ B)
{
    const double d = B[(int64_t)k * N + k];
    if (!(d > 0.0)) return;
    const double s = sqrt(d);
    for (int64_t i = k + 1 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N;
         i += (int64_t)gridDim.x * blockDim.x)
        B[i * N + k] /= s;
    if (blockIdx.x == 0 && threadIdx.x == 0) B[(int64_t)k * N + k] = s;
}

// ------------------------------------------------------ triangular solves
// Y = L^-1 Y in place, a thread per column j (row-major: the threads of a
// warp read one row's consecutive entries; L_ik is the same for all).
__global__ void k_forward_subst(int N, const double *__restrict__ L, double *__restrict__ Y)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    for (int i = 0; i < N; ++i) {
        double s = Y[(int64_t)i * N + j];
        const double *Li = L + (int64_t)i * N;
        for (int k = 0; k < i; ++k) s = fma(-Li[k], Y[(int64_t)k * N + j], s);
        Y[(int64_t)i * N + j] = s / Li[i];
    }
}

// Z = L^-T Z in place (back substitution with L's columns), a thread per column.
__global__ void k_backward_subst_t(int N, const double *__restrict__ L, double *__restrict__ Z)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    for (int i = N - 1; i >= 0; --i) {
        double s = Z[(int64_t)i * N + j];
        for (int k = i + 1; k < N; ++k) s = fma(-L[(int64_t)k * N + i], Z[(int64_t)k * N + j], s);
        Z[(int64_t)i * N + j] = s / L[(int64_t)i * N + i];
    }
}

__global__ void k_transpose(int N, const double *__restrict__ X, double *__restrict__ Y)
{
    __shared__ double t[32][33];
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int i = by + r, j = bx + threadIdx.x;
        if (i < N && j < N) t[r][threadIdx.x] = X[(int64_t)i * N + j];
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int i = bx + r, j = by + threadIdx.x;
        if (i < N && j < N) Y[(int64_t)i * N + j] = t[threadIdx.x][r];
    }
}

// C = (C + C^T) / 2 (upper and lower written from the same pair) and V = I.
__global__ void k_symmetrize_identity(int N, double *__restrict__ C, double *__restrict__ V)
{
    const int64_t total = (int64_t)N * N;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / N, j = t % N;
        V[t] = (i == j) ? 1.0 : 0.0;
        if (j > i) {
            const double a = 0.5 * (C[i * N + j] + C[j * N + i]);
            C[i * N + j] = a;
            C[j * N + i] = a;
        }
    }
}

// ---------------------------------------------------------------- Jacobi
// Round-robin ("tournament") ordering of M (even) indices: at step t pair i is
// (a_i, b_i) with a_0 = t mod (M-1), b_0 = M-1, a_i = (t+i) mod (M-1),
// b_i = (t-i) mod (M-1); over M-1 steps every pair meets once.  The matrix
// is kept in pair order: positions 2i, 2i+1 hold a_i, b_i, so a step reads
// its 2x2 blocks contiguously and writes them to the next step's positions.
__device__ __forceinline__ int rr_member(int M, int t, int pos)
{
    const int i = pos >> 1, K = M - 1;
    if (i == 0) return (pos & 1) ? K : t % K;
    return (pos & 1) ? (t - i + K) % K : (t + i) % K;
}
__device__ __forceinline__ int rr_position(int M, int t, int x)
{
    const int K = M - 1;
    if (x == K) return 1;
    const int d = ((x - t) % K + K) % K;
    if (d == 0) return 0;
    if (d <= M / 2 - 1) return 2 * d;
    return 2 * (K - d) + 1;
}

// Cp[rr_position(0, x)][rr_position(0, y)] = C[x][y] (0 for the padding index
// of an odd N); V[k][rr_position(0, x)] = (k == x).
__global__ void k_jacobi_init(int N, int M, const double *__restrict__ C, double *__restrict__ Cp,
                              double *__restrict__ V)
{
    const int64_t total = (int64_t)M * M;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(t / M), y = (int)(t % M);
        const double v = (x < N && y < N) ? C[(int64_t)x * N + y] : 0.0;
        Cp[(int64_t)rr_position(M, 0, x) * M + rr_position(M, 0, y)] = v;
        if (x < N) V[(int64_t)x * M + rr_position(M, 0, y)] = (x == y) ? 1.0 : 0.0;
    }
}

// Rotation of every pair: J = [[c, s], [-s, c]] on (a_i, b_i) zeroes
// (J^T C J)_ab (Rutishauser: theta = (C_bb - C_aa) / (2 C_ab),
// t = sign(theta) / (|theta| + sqrt(theta^2 + 1)), c = 1 / sqrt(t^2 + 1), s = t c;
// Golub & Van Loan, Matrix Computations, sec. 8.5).
__global__ void k_jacobi_angles(int M, const double *__restrict__ Cp, double *__restrict__ cs)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M / 2) return;
    const double app = Cp[(int64_t)(2 * i) * M + 2 * i], aqq = Cp[(int64_t)(2 * i + 1) * M + 2 * i + 1];
    const double apq = Cp[(int64_t)(2 * i) * M + 2 * i + 1];
    double c = 1.0, s = 0.0;
    if (apq != 0.0 && fabs(apq) > 1e-300) {
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(fma(theta, theta, 1.0)));
        c = 1.0 / sqrt(fma(t, t, 1.0));
        s = t * c;
    }
    cs[2 * i] = c;
    cs[2 * i + 1] = s;
}

// One step: the 2x2 block of row pair a and column pair b becomes
// J_a^T C_ab J_b (the rotations of all pairs at once, J block diagonal),
// written at step t+1's positions; V's columns likewise (V <- V J).
__global__ void k_jacobi_step(int N, int M, int t, const double *__restrict__ Cp, double *__restrict__ Cn,
                              const double *__restrict__ V, double *__restrict__ Vn, const double *__restrict__ cs)
{
    const int P = M / 2;
    const int64_t nc = (int64_t)P * P, nv = (int64_t)N * P;
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < nc + nv;
         u += (int64_t)gridDim.x * blockDim.x) {
        if (u < nc) {
            const int a = (int)(u / P), b = (int)(u % P);
            const double ca = cs[2 * a], sa = cs[2 * a + 1], cb = cs[2 * b], sb = cs[2 * b + 1];
            const double2 r0 = *reinterpret_cast<const double2 *>(Cp + (int64_t)(2 * a) * M + 2 * b);
            const double2 r1 = *reinterpret_cast<const double2 *>(Cp + (int64_t)(2 * a + 1) * M + 2 * b);
            // rows: J_a^T
            const double y00 = ca * r0.x - sa * r1.x, y01 = ca * r0.y - sa * r1.y;
            const double y10 = sa * r0.x + ca * r1.x, y11 = sa * r0.y + ca * r1.y;
            // columns: J_b
            const double z00 = cb * y00 - sb * y01, z01 = sb * y00 + cb * y01;
            const double z10 = cb * y10 - sb * y11, z11 = sb * y10 + cb * y11;
            const int ra = rr_position(M, t + 1, rr_member(M, t, 2 * a));
            const int rb = rr_position(M, t + 1, rr_member(M, t, 2 * a + 1));
            const int qa = rr_position(M, t + 1, rr_member(M, t, 2 * b));
            const int qb = rr_position(M, t + 1, rr_member(M, t, 2 * b + 1));
            Cn[(int64_t)ra * M + qa] = z00;
            Cn[(int64_t)ra * M + qb] = z01;
            Cn[(int64_t)rb * M + qa] = z10;
            Cn[(int64_t)rb * M + qb] = z11;
        } else {
            const int64_t w = u - nc;
            const int k = (int)(w / P), b = (int)(w % P);
            const double cb = cs[2 * b], sb = cs[2 * b + 1];
            const double2 v = *reinterpret_cast<const double2 *>(V + (int64_t)k * M + 2 * b);
            const int qa = rr_position(M, t + 1, rr_member(M, t, 2 * b));
            const int qb = rr_position(M, t + 1, rr_member(M, t, 2 * b + 1));
            Vn[(int64_t)k * M + qa] = cb * v.x - sb * v.y;
            Vn[(int64_t)k * M + qb] = sb * v.x + cb * v.y;
        }
    }
}

// off = sum_{i != j} C_ij^2, dia = sum_i C_ii^2 of an M x M matrix (atomic adds
// of per-CTA sums; only compared with a threshold)
__global__ void k_offdiag(int M, const double *__restrict__ C, double *__restrict__ out)
{
    __shared__ double so[256], sd[256];
    double o = 0.0, d = 0.0;
    const int64_t total = (int64_t)M * M;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const double v = C[t];
        if (t / M == t % M) d += v * v;
        else o += v * v;
    }
    so[threadIdx.x] = o;
    sd[threadIdx.x] = d;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            so[threadIdx.x] += so[threadIdx.x + w];
            sd[threadIdx.x] += sd[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        atomicAdd(out, so[0]);
        atomicAdd(out + 1, sd[0]);
    }
}

// Eigenpairs out of the pair-order layout of step 0: w[x] = Cp[pos][pos],
// Q[r][x] = V[r][pos] with pos = rr_position(0, x), x < N.
__global__ void k_jacobi_extract(int N, int M, const double *__restrict__ Cp, const double *__restrict__ V,
                                 double *__restrict__ w, double *__restrict__ Q)
{
    const int64_t total = (int64_t)N * N;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(t / N), x = (int)(t % N);
        const int pos = rr_position(M, 0, x);
        Q[t] = V[(int64_t)r * M + pos];
        if (r == 0) w[x] = Cp[(int64_t)pos * M + pos];
    }
}

int dense_generalized_eig(int N, double *A, double *B, double *w, double *Z, int *sweeps, cudaStream_t st)
{
    PFG_CHECK(N >= 1 && N <= kDenseEigMax, PFG_E_UNSUPPORTED,
              "dense eig: " + std::to_string(N) + " unknowns, the dense branch handles at most " +
                  std::to_string(kDenseEigMax) + " (set use_LOBPCG for larger problems)");
    DevBuf<int> err(1);
    PFG_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
    // 1. B = L L^T
    for (int k = 0; k < N; ++k) {
        const int64_t m = N - 1 - k;
        if (m > 0) k_chol_update<<<grid_for(m * (m + 1) / 2, 256), 256, 0, st>>>(N, k, B, err.p);
        k_chol_scale<<<grid_for(std::max<int64_t>(m, 1), 256), 256, 0, st>>>(N, k, B);
    }
    PFG_CUDA(cudaGetLastError());
    int h_err = 0;
    PFG_CUDA(cudaMemcpyAsync(&h_err, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    PFG_CUDA(cudaStreamSynchronize(st));
    PFG_CHECK(h_err == 0, PFG_E_ARG, "dense eig: B is not positive definite (DSPGVD would report INFO > N)");
    // 2. C = L^-1 (L^-1 A)^T
    const int gt = (N + 127) / 128;
    k_forward_subst<<<gt, 128, 0, st>>>(N, B, A);
    dim3 tb(32, 8), tg((N + 31) / 32, (N + 31) / 32);
    k_transpose<<<tg, tb, 0, st>>>(N, A, Z);  // Z as scratch
    k_forward_subst<<<gt, 128, 0, st>>>(N, B, Z);
    k_symmetrize_identity<<<grid_for((int64_t)N * N, 256), 256, 0, st>>>(N, Z, A);  // C = Z (A: scratch)
    // 3. cyclic Jacobi in pair order (M = N rounded up to even)
    const int M = N + (N & 1);
    DevBuf<double> Cp((size_t)M * M), Cn((size_t)M * M), Vp((size_t)N * M), Vn((size_t)N * M), cs((size_t)M),
        norms(2);
    k_jacobi_init<<<grid_for((int64_t)M * M, 256), 256, 0, st>>>(N, M, Z, Cp.p, Vp.p);
    const int P = M / 2;
    const int gs = grid_for((int64_t)P * P + (int64_t)N * P, 256);
    int sweep = 0;
    for (; sweep < 40 && M > 2; ++sweep) {
        PFG_CUDA(cudaMemsetAsync(norms.p, 0, 2 * sizeof(double), st));
        k_offdiag<<<grid_for((int64_t)M * M, 256, sm_count_device() * 4), 256, 0, st>>>(M, Cp.p, norms.p);
        double hn[2];
        PFG_CUDA(cudaMemcpyAsync(hn, norms.p, sizeof hn, cudaMemcpyDeviceToHost, st));
        PFG_CUDA(cudaStreamSynchronize(st));
        if (!(hn[0] > 1e-30 * hn[1]) || !std::isfinite(hn[0])) break;
        for (int t = 0; t < M - 1; ++t) {  // a sweep returns the layout to step 0's
            k_jacobi_angles<<<(P + 127) / 128, 128, 0, st>>>(M, Cp.p, cs.p);
            k_jacobi_step<<<gs, 256, 0, st>>>(N, M, t, Cp.p, Cn.p, Vp.p, Vn.p, cs.p);
            std::swap(Cp.p, Cn.p);
            std::swap(Vp.p, Vn.p);
        }
        PFG_CUDA(cudaGetLastError());
    }
    if (M == 2 && N == 2) {  // one rotation of a 2 x 2 problem
        k_jacobi_angles<<<1, 128, 0, st>>>(M, Cp.p, cs.p);
        k_jacobi_step<<<gs, 256, 0, st>>>(N, M, 0, Cp.p, Cn.p, Vp.p, Vn.p, cs.p);
        std::swap(Cp.p, Cn.p);
        std::swap(Vp.p, Vn.p);
        sweep = 1;
    }
    if (sweeps) *sweeps = sweep;
    DevBuf<double> dw((size_t)N);
    k_jacobi_extract<<<grid_for((int64_t)N * N, 256), 256, 0, st>>>(N, M, Cp.p, Vp.p, dw.p, A);
    // 4. Z = L^-T Q (Q in A's buffer)
    k_backward_subst_t<<<gt, 128, 0, st>>>(N, B, A);
    PFG_CUDA(cudaGetLastError());
    PFG_CUDA(cudaMemcpyAsync(w, dw.p, (size_t)N * sizeof(double), cudaMemcpyDeviceToHost, st));
    PFG_CUDA(cudaMemcpyAsync(Z, A, (size_t)N * N * sizeof(double), cudaMemcpyDeviceToDevice, st));
    PFG_CUDA(cudaStreamSynchronize(st));
    return N;
}

}  // namespace pfg
