// lobpcg.cu -- block LOBPCG on the device (see lobpcg.cuh).
#include <algorithm>
#include <cmath>
#include <type_traits>
#include <vector>

#include "lobpcg.cuh"

namespace pfg {

// ===================================================================== host
// Symmetric eigensolver for the small Rayleigh-Ritz problems: Householder
// reduction to tridiagonal form with accumulated transformations, then the
// implicit QL iteration with shifts (Bowdler, Martin, Reinsch & Wilkinson,
// Numer. Math. 11 (1968), the method of EISPACK's tql2).  A is n x n column-
// major, replaced by the eigenvectors; w receives the eigenvalues ascending.
static void sym_eig(int n, std::vector<double> &A, std::vector<double> &w)
{
    auto a = [&](int i, int j) -> double & { return A[(size_t)j * n + i]; };
    std::vector<double> Q((size_t)n * n, 0.0), d(n), e(n, 0.0), v(n), p(n), q(n);
    for (int i = 0; i < n; ++i) Q[(size_t)i * n + i] = 1.0;
    // Householder: zero column j below the subdiagonal
    for (int j = 0; j + 2 < n; ++j) {
        double alpha = 0.0;
        for (int i = j + 1; i < n; ++i) alpha += a(i, j) * a(i, j);
        alpha = std::sqrt(alpha);
        if (alpha == 0.0) continue;
        if (a(j + 1, j) > 0) alpha = -alpha;
        // v = x - alpha e1 on rows j+1..n-1
        for (int i = 0; i < n; ++i) v[i] = 0.0;
        for (int i = j + 1; i < n; ++i) v[i] = a(i, j);
        v[j + 1] -= alpha;
        double vv = 0.0;
        for (int i = j + 1; i < n; ++i) vv += v[i] * v[i];
        if (vv == 0.0) continue;
        const double beta = 2.0 / vv;
        // A <- H A H with H = I - beta v v^T:  p = beta A v, K = beta/2 v^T p, q = p - K v,
        // A <- A - v q^T - q v^T.  Columns < j are reduced already (zero below
        // their subdiagonal), so p, q and the update live in rows/columns >= j.
        for (int i = j; i < n; ++i) {
            double s = 0.0;
            for (int l = j + 1; l < n; ++l) s += a(i, l) * v[l];
            p[i] = beta * s;
        }
        double K = 0.0;
        for (int i = j + 1; i < n; ++i) K += v[i] * p[i];
        K *= 0.5 * beta;
        for (int i = j; i < n; ++i) q[i] = p[i] - K * v[i];
        for (int c = j; c < n; ++c)
            for (int r = j; r < n; ++r) a(r, c) -= v[r] * q[c] + q[r] * v[c];
        // Q <- Q H = Q - beta (Q v) v^T, column by column (contiguous)
        for (int r = 0; r < n; ++r) p[r] = 0.0;
        for (int l = j + 1; l < n; ++l) {
            const double vl = v[l];
            const double *ql = &Q[(size_t)l * n];
            for (int r = 0; r < n; ++r) p[r] += ql[r] * vl;
        }
        for (int l = j + 1; l < n; ++l) {
            const double bv = beta * v[l];
            double *ql = &Q[(size_t)l * n];
            for (int r = 0; r < n; ++r) ql[r] -= p[r] * bv;
        }
    }
    for (int i = 0; i < n; ++i) d[i] = a(i, i);
    for (int i = 0; i + 1 < n; ++i) e[i] = a(i + 1, i);
    e[n - 1] = 0.0;
    // implicit QL on (d, e), rotations applied to the columns of Q
    const double eps = 2.220446049250313e-16;
    for (int l = 0; l < n; ++l) {
        for (int iter = 0; iter < 200; ++iter) {
            int m = l;
            for (; m < n - 1; ++m) {
                const double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
                if (std::fabs(e[m]) <= eps * dd) break;
            }
            if (m == l) break;
            // sqrt(x*x + y*y) in place of hypot: the matrices are scaled to
            // unit diagonal (B) or come from it (A'), far from overflow
            double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
            double r = std::sqrt(g * g + 1.0);
            g = d[m] - d[l] + e[l] / (g + (g >= 0 ? r : -r));
            double s = 1.0, c = 1.0, pp = 0.0;
            int i = m - 1;
            bool underflow = false;
            for (; i >= l; --i) {
                const double f = s * e[i], b = c * e[i];
                r = std::sqrt(f * f + g * g);
                e[i + 1] = r;
                if (r == 0.0) {
                    d[i + 1] -= pp;
                    e[m] = 0.0;
                    underflow = true;
                    break;
                }
                s = f / r;
                c = g / r;
                g = d[i + 1] - pp;
                r = (d[i] - g) * s + 2.0 * c * b;
                pp = s * r;
                d[i + 1] = g + pp;
                g = c * r - b;
                double *qi = &Q[(size_t)i * n], *qi1 = &Q[(size_t)(i + 1) * n];
                for (int k = 0; k < n; ++k) {
                    const double t = qi1[k];
                    qi1[k] = s * qi[k] + c * t;
                    qi[k] = c * qi[k] - s * t;
                }
            }
            if (underflow) continue;
            d[l] -= pp;
            e[l] = g;
            e[m] = 0.0;
        }
    }
    // sort ascending
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](int x, int y) { return d[x] < d[y]; });
    w.assign(n, 0.0);
    for (int i = 0; i < n; ++i) {
        w[i] = d[idx[i]];
        for (int r = 0; r < n; ++r) A[(size_t)i * n + r] = Q[(size_t)idx[i] * n + r];
    }
}

// The lowest k eigenpairs of a symmetric A (n x n, column-major; destroyed):
// Householder reduction to tridiagonal T = Q^T A Q without accumulating Q,
// T's eigenvalues by the implicit QL iteration without vectors (tql1), the k
// wanted eigenvectors of T by inverse iteration (Peters & Wilkinson, "The
// calculation of specified eigenvectors by inverse iteration", Handbook for
// Automatic Computation II (1971); the scheme of LAPACK's dstein: tridiagonal
// LU with partial pivoting, tiny pivots replaced by eps ||T||, shifts of
// coincident eigenvalues spread by 10 eps ||T||, modified Gram-Schmidt against
// the earlier vectors of a cluster, i.e. of eigenvalues within 1e-3 ||T||),
// and the back transformation Q y by the stored reflectors.  About a third of
// the work of sym_eig at n = 72, k = 24 (no n x n accumulation of Q).
// w: all n eigenvalues ascending; Y: n x k, column j the eigenvector of w[j].
static void sym_eig_lowest(int n, std::vector<double> &A, int k, std::vector<double> &w, std::vector<double> &Y)
{
    auto a = [&](int i, int j) -> double & { return A[(size_t)j * n + i]; };
    std::vector<double> d(n), e(n, 0.0), V((size_t)n * n, 0.0), beta(n, 0.0), v(n), p(n), q(n);
    for (int j = 0; j + 2 < n; ++j) {
        double alpha = 0.0;
        for (int i = j + 1; i < n; ++i) alpha += a(i, j) * a(i, j);
        alpha = std::sqrt(alpha);
        if (alpha == 0.0) continue;
        if (a(j + 1, j) > 0) alpha = -alpha;
        for (int i = 0; i < n; ++i) v[i] = 0.0;
        for (int i = j + 1; i < n; ++i) v[i] = a(i, j);
        v[j + 1] -= alpha;
        double vv = 0.0;
        for (int i = j + 1; i < n; ++i) vv += v[i] * v[i];
        if (vv == 0.0) continue;
        const double bt = 2.0 / vv;
        // p = beta A v as a sum of columns (contiguous, vectorisable loops)
        for (int i = j; i < n; ++i) p[i] = 0.0;
        for (int l = j + 1; l < n; ++l) {
            const double vl = bt * v[l];
            const double *al = &A[(size_t)l * n];
            for (int i = j; i < n; ++i) p[i] += al[i] * vl;
        }
        double K = 0.0;
        for (int i = j + 1; i < n; ++i) K += v[i] * p[i];
        K *= 0.5 * bt;
        for (int i = j; i < n; ++i) q[i] = p[i] - K * v[i];
        for (int c = j; c < n; ++c)
            for (int r = j; r < n; ++r) a(r, c) -= v[r] * q[c] + q[r] * v[c];
        for (int i = j + 1; i < n; ++i) V[(size_t)j * n + i] = v[i];
        beta[j] = bt;
    }
    double tnorm = 0.0;
    for (int i = 0; i < n; ++i) {
        d[i] = a(i, i);
        if (i + 1 < n) e[i] = a(i + 1, i);
    }
    for (int i = 0; i < n; ++i)
        tnorm = std::max(tnorm, std::fabs(d[i]) + (i > 0 ? std::fabs(e[i - 1]) : 0.0) + std::fabs(e[i]));
    // eigenvalues: implicit QL on copies of (d, e), no vectors
    const double eps = 2.220446049250313e-16;
    {
        std::vector<double> dd = d, ee = e;
        ee[n - 1] = 0.0;
        for (int l = 0; l < n; ++l) {
            for (int iter = 0; iter < 200; ++iter) {
                int m = l;
                for (; m < n - 1; ++m) {
                    const double s = std::fabs(dd[m]) + std::fabs(dd[m + 1]);
                    if (std::fabs(ee[m]) <= eps * s) break;
                }
                if (m == l) break;
                double g = (dd[l + 1] - dd[l]) / (2.0 * ee[l]);
                double r = std::sqrt(g * g + 1.0);
                g = dd[m] - dd[l] + ee[l] / (g + (g >= 0 ? r : -r));
                double s = 1.0, c = 1.0, pp = 0.0;
                bool underflow = false;
                for (int i = m - 1; i >= l; --i) {
                    const double f = s * ee[i], b = c * ee[i];
                    r = std::sqrt(f * f + g * g);
                    ee[i + 1] = r;
                    if (r == 0.0) {
                        dd[i + 1] -= pp;
                        ee[m] = 0.0;
                        underflow = true;
                        break;
                    }
                    s = f / r;
                    c = g / r;
                    g = dd[i + 1] - pp;
                    r = (dd[i] - g) * s + 2.0 * c * b;
                    pp = s * r;
                    dd[i + 1] = g + pp;
                    g = c * r - b;
                }
                if (underflow) continue;
                dd[l] -= pp;
                ee[l] = g;
                ee[m] = 0.0;
            }
        }
        std::sort(dd.begin(), dd.end());
        w = dd;
    }
    // inverse iteration for the k lowest
    const int kk = std::min(k, n);
    Y.assign((size_t)n * kk, 0.0);
    const double tiny = eps * std::max(tnorm, 1e-300);
    const double ortol = 1e-3 * tnorm, pertol = 10.0 * eps * tnorm;
    std::vector<double> dl(n), dg(n), du(n), du2(n), x(n), Yt((size_t)n * kk);  // Yt: T's eigenvectors
    std::vector<char> piv(n);
    int cluster0 = 0;
    double prev = 0.0;
    for (int j = 0; j < kk; ++j) {
        double lam = w[j];
        if (j > 0) {
            if (w[j] - w[j - 1] > ortol) cluster0 = j;
            if (lam <= prev + pertol) lam = prev + pertol;  // distinct shifts inside a cluster
        }
        prev = lam;
        // LU of T - lam I with partial pivoting (U: diagonal dg, superdiagonals du, du2)
        for (int i = 0; i < n; ++i) {
            dg[i] = d[i] - lam;
            dl[i] = du[i] = (i + 1 < n) ? e[i] : 0.0;
            du2[i] = 0.0;
        }
        for (int i = 0; i + 1 < n; ++i) {
            if (std::fabs(dg[i]) >= std::fabs(dl[i])) {
                piv[i] = 0;
                if (std::fabs(dg[i]) < tiny) dg[i] = dg[i] < 0 ? -tiny : tiny;
                const double f = dl[i] / dg[i];
                dl[i] = f;
                dg[i + 1] -= f * du[i];
            } else {
                piv[i] = 1;
                const double f = dg[i] / dl[i];
                dg[i] = dl[i];
                dl[i] = f;
                const double t = du[i];
                du[i] = dg[i + 1];
                dg[i + 1] = t - f * dg[i + 1];
                if (i + 2 < n) {
                    du2[i] = du[i + 1];
                    du[i + 1] = -f * du[i + 1];
                }
            }
        }
        if (std::fabs(dg[n - 1]) < tiny) dg[n - 1] = dg[n - 1] < 0 ? -tiny : tiny;
        for (int i = 0; i < n; ++i) dg[i] = 1.0 / dg[i];  // pivots kept as reciprocals for the solves
        // start: a fixed pseudo-random vector (different per j)
        for (int i = 0; i < n; ++i) {
            uint64_t h = (uint64_t)(j + 1) * 0x9e3779b97f4a7c15ull ^ ((uint64_t)i * 0xbf58476d1ce4e5b9ull);
            h ^= h >> 31;
            h *= 0x94d049bb133111ebull;
            h ^= h >> 29;
            x[i] = (double)(h >> 11) * (2.0 / 9007199254740992.0) - 1.0;
        }
        for (int it = 0; it < 3; ++it) {
            for (int i = 0; i + 1 < n; ++i) {  // L^-1 (with the row interchanges)
                if (piv[i]) std::swap(x[i], x[i + 1]);
                x[i + 1] -= dl[i] * x[i];
            }
            for (int i = n - 1; i >= 0; --i) {  // U^-1
                double t = x[i];
                if (i + 1 < n) t -= du[i] * x[i + 1];
                if (i + 2 < n) t -= du2[i] * x[i + 2];
                x[i] = t * dg[i];
            }
            for (int c = cluster0; c < j; ++c) {  // orthogonal to the cluster's earlier vectors
                const double *yc = &Yt[(size_t)c * n];
                double s = 0.0;
                for (int i = 0; i < n; ++i) s += yc[i] * x[i];
                for (int i = 0; i < n; ++i) x[i] -= s * yc[i];
            }
            double nrm = 0.0;
            for (int i = 0; i < n; ++i) nrm += x[i] * x[i];
            nrm = std::sqrt(nrm);
            if (!(nrm > 0.0) || !std::isfinite(nrm)) nrm = 1.0;
            for (int i = 0; i < n; ++i) x[i] /= nrm;
        }
        std::copy(x.begin(), x.end(), Yt.begin() + (size_t)j * n);
    }
    // back transformation of all kk vectors at once, y <- H_0 (H_1 (... (H_{n-3} y))):
    // the block is held row-major (n x kk), so each reflector's dot products
    // and updates run along contiguous rows of kk values
    std::vector<double> Xr((size_t)n * kk), sv(kk);
    for (int c = 0; c < kk; ++c)
        for (int i = 0; i < n; ++i) Xr[(size_t)i * kk + c] = Yt[(size_t)c * n + i];
    for (int jj = n - 3; jj >= 0; --jj) {
        if (beta[jj] == 0.0) continue;
        const double *vj = &V[(size_t)jj * n];
        for (int c = 0; c < kk; ++c) sv[c] = 0.0;
        for (int i = jj + 1; i < n; ++i) {
            const double vi = vj[i];
            const double *xi = &Xr[(size_t)i * kk];
            for (int c = 0; c < kk; ++c) sv[c] += vi * xi[c];
        }
        for (int c = 0; c < kk; ++c) sv[c] *= beta[jj];
        for (int i = jj + 1; i < n; ++i) {
            const double vi = vj[i];
            double *xi = &Xr[(size_t)i * kk];
            for (int c = 0; c < kk; ++c) xi[c] -= sv[c] * vi;
        }
    }
    for (int c = 0; c < kk; ++c)
        for (int i = 0; i < n; ++i) Y[(size_t)c * n + i] = Xr[(size_t)i * kk + c];
}

// B = L L^T (lower L, column-major, in place of B's lower triangle) when every
// pivot exceeds rank_tol times the largest diagonal entry; false otherwise.
static bool cholesky_well_posed(int m, std::vector<double> &B, double rank_tol)
{
    double dmax = 0.0;
    for (int i = 0; i < m; ++i) dmax = std::max(dmax, B[(size_t)i * m + i]);
    if (!(dmax > 0.0)) return false;
    // right-looking: scale column j, then update the trailing columns (each
    // update a contiguous column axpy)
    for (int j = 0; j < m; ++j) {
        double *bj = &B[(size_t)j * m];
        const double d = bj[j];
        if (!(d > rank_tol * dmax)) return false;
        const double ljj = std::sqrt(d);
        bj[j] = ljj;
        const double inv = 1.0 / ljj;
        for (int i = j + 1; i < m; ++i) bj[i] *= inv;
        for (int c = j + 1; c < m; ++c) {
            double *bc = &B[(size_t)c * m];
            const double f = bj[c];
            for (int i = c; i < m; ++i) bc[i] -= bj[i] * f;
        }
    }
    return true;
}

int small_generalized_eig(int m, const double *Ain, const double *Bin, int k, double rank_tol, double *lam, double *C)
{
    // scale to unit diagonal, then keep B's numerically nonzero directions
    std::vector<double> s(m);
    for (int i = 0; i < m; ++i) {
        const double b = Bin[(size_t)i * m + i];
        s[i] = (b > 0 && std::isfinite(b)) ? 1.0 / std::sqrt(b) : 0.0;
    }
    std::vector<double> B((size_t)m * m), w;
    for (int j = 0; j < m; ++j)
        for (int i = 0; i < m; ++i)
            B[(size_t)j * m + i] = 0.5 * (Bin[(size_t)j * m + i] + Bin[(size_t)i * m + j]) * s[i] * s[j];
    {
        // Well-posed B (no pivot at or below rank_tol of the largest: the
        // usual case): A' = L^-1 (S A S) L^-T and C = S L^-T Y, a Cholesky
        // and two triangular solves instead of B's eigendecomposition.
        // Otherwise B's eigendecomposition below drops its null directions.
        std::vector<double> L = B;
        if (cholesky_well_posed(m, L, rank_tol)) {
            // Block forward substitution X <- L^-1 X on a row-major m x w
            // block: each step scales row q and subtracts it from the rows
            // below, whole rows at a time (contiguous, vectorisable).
            auto block_lsolve = [&](double *X, int w) {
                for (int q = 0; q < m; ++q) {
                    const double *lq = &L[(size_t)q * m];  // column q of L
                    double *xq = X + (size_t)q * w;
                    const double inv = 1.0 / lq[q];
                    for (int c = 0; c < w; ++c) xq[c] *= inv;
                    for (int i = q + 1; i < m; ++i) {
                        const double f = lq[i];
                        double *xi = X + (size_t)i * w;
                        for (int c = 0; c < w; ++c) xi[c] -= f * xq[c];
                    }
                }
            };
            // W = L^-1 (S A S); A' = W L^-T = (L^-1 W^T)^T (symmetric)
            std::vector<double> W((size_t)m * m), Ap((size_t)m * m);
            for (int r = 0; r < m; ++r)
                for (int c = 0; c < m; ++c)
                    W[(size_t)r * m + c] = 0.5 * (Ain[(size_t)c * m + r] + Ain[(size_t)r * m + c]) * s[r] * s[c];
            block_lsolve(W.data(), m);
            for (int r = 0; r < m; ++r)
                for (int c = 0; c < m; ++c) Ap[(size_t)r * m + c] = W[(size_t)c * m + r];
            block_lsolve(Ap.data(), m);
            for (int c = 0; c < m; ++c)  // symmetrise
                for (int r = 0; r < c; ++r) {
                    const double v = 0.5 * (Ap[(size_t)c * m + r] + Ap[(size_t)r * m + c]);
                    Ap[(size_t)c * m + r] = Ap[(size_t)r * m + c] = v;
                }
            std::vector<double> mu, Y;
            const int kk = std::min(k, m);
            sym_eig_lowest(m, Ap, kk, mu, Y);
            // C = S L^-T Y: block back substitution on the row-major m x kk
            // block of the eigenvectors
            std::vector<double> Cb((size_t)m * kk);
            for (int j2 = 0; j2 < kk; ++j2)
                for (int r = 0; r < m; ++r) Cb[(size_t)r * kk + j2] = Y[(size_t)j2 * m + r];
            for (int r = m - 1; r >= 0; --r) {
                double *cr = &Cb[(size_t)r * kk];
                const double inv = 1.0 / L[(size_t)r * m + r];
                for (int c = 0; c < kk; ++c) cr[c] *= inv;
                for (int q = 0; q < r; ++q) {
                    const double f = L[(size_t)q * m + r];  // L(r, q) = L^T(q, r)
                    double *cq = &Cb[(size_t)q * kk];
                    for (int c = 0; c < kk; ++c) cq[c] -= f * cr[c];
                }
            }
            for (int j2 = 0; j2 < kk; ++j2) {
                lam[j2] = mu[j2];
                for (int r = 0; r < m; ++r) C[(size_t)j2 * m + r] = Cb[(size_t)r * kk + j2] * s[r];
            }
            return kk;
        }
    }
    sym_eig(m, B, w);
    const double wmax = w[m - 1];
    if (!(wmax > 0)) return 0;
    std::vector<int> keep;
    for (int i = 0; i < m; ++i)
        if (w[i] > rank_tol * wmax) keep.push_back(i);
    const int r = (int)keep.size();
    // T = S Q_keep Theta^-1/2  (m x r)
    std::vector<double> T((size_t)m * r);
    for (int c = 0; c < r; ++c) {
        const double f = 1.0 / std::sqrt(w[keep[c]]);
        for (int i = 0; i < m; ++i) T[(size_t)c * m + i] = s[i] * B[(size_t)keep[c] * m + i] * f;
    }
    // A' = T^T A T
    std::vector<double> AT((size_t)m * r), Ap((size_t)r * r);
    for (int c = 0; c < r; ++c)
        for (int i = 0; i < m; ++i) {
            double acc = 0.0;
            for (int l = 0; l < m; ++l) acc += 0.5 * (Ain[(size_t)l * m + i] + Ain[(size_t)i * m + l]) * T[(size_t)c * m + l];
            AT[(size_t)c * m + i] = acc;
        }
    for (int c = 0; c < r; ++c)
        for (int i = 0; i < r; ++i) {
            double acc = 0.0;
            for (int l = 0; l < m; ++l) acc += T[(size_t)i * m + l] * AT[(size_t)c * m + l];
            Ap[(size_t)c * r + i] = acc;
        }
    for (int c = 0; c < r; ++c)
        for (int i = 0; i < c; ++i) {
            const double v = 0.5 * (Ap[(size_t)c * r + i] + Ap[(size_t)i * r + c]);
            Ap[(size_t)c * r + i] = Ap[(size_t)i * r + c] = v;
        }
    std::vector<double> mu;
    sym_eig(r, Ap, mu);
    const int kk = std::min(k, r);
    for (int j = 0; j < kk; ++j) {
        lam[j] = mu[j];
        for (int i = 0; i < m; ++i) {
            double acc = 0.0;
            for (int l = 0; l < r; ++l) acc += T[(size_t)l * m + i] * Ap[(size_t)j * r + l];
            C[(size_t)j * m + i] = acc;
        }
    }
    return kk;
}

// =================================================================== device
constexpr int kT = 256;
constexpr int PW = 8;  // panel width

template <typename T>
__device__ __forceinline__ const T *panel_row(const T *base, int64_t n, int q, int64_t row)
{
    return base + ((int64_t)q * n + row) * PW;
}

// A panel row (PW = 8 consecutive values, 32 or 64 bytes, aligned to its
// size) moved with 16-byte accesses: one gather instruction per 16 bytes
// instead of one per value.
__device__ __forceinline__ void ld_row(const float *p, float (&v)[PW])
{
#pragma unroll
    for (int u = 0; u < 2; ++u) {
        const float4 w = __ldg(reinterpret_cast<const float4 *>(p) + u);
        v[4 * u] = w.x;
        v[4 * u + 1] = w.y;
        v[4 * u + 2] = w.z;
        v[4 * u + 3] = w.w;
    }
}
__device__ __forceinline__ void ld_row(const double *p, double (&v)[PW])
{
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const double2 w = __ldg(reinterpret_cast<const double2 *>(p) + u);
        v[2 * u] = w.x;
        v[2 * u + 1] = w.y;
    }
}
__device__ __forceinline__ void ld_row(const float2 *p, float2 (&v)[PW])
{
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const float4 w = __ldg(reinterpret_cast<const float4 *>(p) + u);
        v[2 * u] = make_float2(w.x, w.y);
        v[2 * u + 1] = make_float2(w.z, w.w);
    }
}
__device__ __forceinline__ void st_row(float *p, const float (&v)[PW])
{
#pragma unroll
    for (int u = 0; u < 2; ++u)
        reinterpret_cast<float4 *>(p)[u] = make_float4(v[4 * u], v[4 * u + 1], v[4 * u + 2], v[4 * u + 3]);
}
__device__ __forceinline__ void st_row(double *p, const double (&v)[PW])
{
#pragma unroll
    for (int u = 0; u < 4; ++u) reinterpret_cast<double2 *>(p)[u] = make_double2(v[2 * u], v[2 * u + 1]);
}
__device__ __forceinline__ void st_row(float2 *p, const float2 (&v)[PW])
{
#pragma unroll
    for (int u = 0; u < 4; ++u)
        reinterpret_cast<float4 *>(p)[u] = make_float4(v[2 * u].x, v[2 * u].y, v[2 * u + 1].x, v[2 * u + 1].y);
}
// The same from shared memory (plain loads: __ldg is for global memory).
__device__ __forceinline__ void lds_row(const float *p, float (&v)[PW])
{
#pragma unroll
    for (int u = 0; u < 2; ++u) {
        const float4 w = reinterpret_cast<const float4 *>(p)[u];
        v[4 * u] = w.x;
        v[4 * u + 1] = w.y;
        v[4 * u + 2] = w.z;
        v[4 * u + 3] = w.w;
    }
}
__device__ __forceinline__ void lds_row(const double *p, double (&v)[PW])
{
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const double2 w = reinterpret_cast<const double2 *>(p)[u];
        v[2 * u] = w.x;
        v[2 * u + 1] = w.y;
    }
}
__device__ __forceinline__ void lds_row(const float2 *p, float2 (&v)[PW])
{
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const float4 w = reinterpret_cast<const float4 *>(p)[u];
        v[2 * u] = make_float2(w.x, w.y);
        v[2 * u + 1] = make_float2(w.z, w.w);
    }
}

// Double-FP32 ("double-float") arithmetic on the FP32 pipe, for the second
// phase of the mixed LOBPCG (its Gram, SpMM and linear combinations of FP64
// panels): GB300's FP64 pipe is about 1/30 of its FP32 pipe, and the FP64
// forms of these kernels ran on it (the Gram at 0.92 TFLOP/s).  Each FP64 value is split into hi + lo floats (exact to
// 48 bits); a product's rounding error comes exactly from an FMA (Dekker's
// product), the cross terms hi*lo are added to it, and each sum keeps its
// rounding error by TwoSum (Knuth); the pair (hi, lo) accumulates one CTA's
// rows and the partial sums are added in FP64 (Hida, Li & Bailey 2001, "Algorithms
// for quad-double precision", double-double addition and multiplication).
// Explicit _rn intrinsics keep the compiler from contracting the error-free
// steps into FMAs.  Relative error about n_cta * 2^-48 per partial sum.
struct DFAcc {
    float hi, lo;
    __device__ void zero() { hi = lo = 0.f; }
    __device__ void add(float2 a, float2 b)
    {
        const float p = __fmul_rn(a.x, b.x);
        float e = fmaf(a.x, b.x, -p);
        e = fmaf(a.x, b.y, e);
        e = fmaf(a.y, b.x, e);
        const float t = __fadd_rn(hi, p);
        const float z = __fsub_rn(t, hi);
        const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, z)), __fsub_rn(p, z));
        hi = t;
        lo = __fadd_rn(lo, __fadd_rn(err, e));
    }
    __device__ double get() const { return (double)hi + (double)lo; }
    // the sum as a normalised (hi, lo) pair: TwoSum of the two parts (FP32 only)
    __device__ float2 get2() const
    {
        const float s = __fadd_rn(hi, lo);
        const float z = __fsub_rn(s, hi);
        return make_float2(s, __fadd_rn(__fsub_rn(hi, __fsub_rn(s, z)), __fsub_rn(lo, z)));
    }
};

__device__ __forceinline__ float2 df_split(double x)
{
    const float h = __double2float_rn(x);
    return make_float2(h, __double2float_rn(x - (double)h));
}

__device__ __forceinline__ double df_value(float2 v) { return (double)v.x + (double)v.y; }

// a + b of two double-float numbers (TwoSum of the heads, the tails added,
// renormalised by a second TwoSum)
__device__ __forceinline__ float2 df_add(float2 a, float2 b)
{
    const float s = __fadd_rn(a.x, b.x);
    const float z = __fsub_rn(s, a.x);
    float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, z)), __fsub_rn(b.x, z));
    e = __fadd_rn(e, __fadd_rn(a.y, b.y));
    const float t = __fadd_rn(s, e);
    const float z2 = __fsub_rn(t, s);
    return make_float2(t, __fadd_rn(__fsub_rn(s, __fsub_rn(t, z2)), __fsub_rn(e, z2)));
}

// Y = A X for every panel (one warp per (slice, panel), one lane per block
// row); rows of fixed DOFs are zeroed (the reduce_crs_matrix restriction).
template <int BS, typename T>
__global__ void __launch_bounds__(kT) k_spmm(SellView<T> A, int np, const T *__restrict__ X, T *__restrict__ Y,
                                             const uint8_t *__restrict__ fixed)
{
    const int lane = threadIdx.x & 31;
    const int64_t n = A.nb * BS;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t u = w0; u < A.ns * np; u += nw) {
        const int64_t s = u / np;
        const int q = (int)(u - s * np);
        const int64_t b0 = A.sptr[s];
        const int wdt = (int)(A.sptr[s + 1] - b0);
        const int *cp = A.col + b0 * 32 + lane;
        const T *vp = A.val + b0 * 32 * (BS * BS) + lane;
        T acc[BS][PW];
#pragma unroll
        for (int r = 0; r < BS; ++r)
#pragma unroll
            for (int c = 0; c < PW; ++c) acc[r][c] = T(0);
        for (int k = 0; k < wdt; ++k) {
            const int col = ld_stream(cp + (int64_t)k * 32);
            T a[BS * BS];
#pragma unroll
            for (int e = 0; e < BS * BS; ++e) a[e] = ld_stream(vp + ((int64_t)k * (BS * BS) + e) * 32);
#pragma unroll
            for (int cc = 0; cc < BS; ++cc) {
                T xv[PW];
                ld_row(panel_row(X, n, q, (int64_t)BS * col + cc), xv);
#pragma unroll
                for (int r = 0; r < BS; ++r)
#pragma unroll
                    for (int c = 0; c < PW; ++c) acc[r][c] = fma(a[r * BS + cc], xv[c], acc[r][c]);
            }
        }
        const int64_t row = s * 32 + lane;
        if (row < A.nb) {
#pragma unroll
            for (int r = 0; r < BS; ++r) {
                const int64_t i = (int64_t)BS * row + r;
                if (fixed && fixed[i])
#pragma unroll
                    for (int c = 0; c < PW; ++c) acc[r][c] = T(0);
                st_row(Y + ((int64_t)q * n + i) * PW, acc[r]);
            }
        }
    }
}

// ---- double-float forms of the SpMM and the linear combinations (mixed
// second phase).  That phase keeps its panels and images as (hi, lo) float
// pairs: the producers (SpMM, linear combinations, preconditioner, residual)
// write pairs, so the inner loops are FP32 arithmetic only and no conversion
// pass runs per iteration; only the matrices' FP64 values are split, once
// (k_to_df).  Splitting FP64 operands where they are used put a conversion
// per use on the FP64 pipe and was slower than FP64 itself; converting them
// in a pass before every use cost 16 % of a double-float iteration.
__global__ void k_to_df(int64_t len, const double *__restrict__ a, float2 *__restrict__ b)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = df_split(a[i]);
}

// Y = A X with A's sliced values (vdf, A's slot layout), the panels X and Y in
// double-float.  Layout and warp mapping as k_spmm.
template <int BS>
__global__ void __launch_bounds__(kT) k_spmm_df(SellView<double> A, const float2 *__restrict__ vdf, int np,
                                                const float2 *__restrict__ X, float2 *__restrict__ Y,
                                                const uint8_t *__restrict__ fixed)
{
    const int lane = threadIdx.x & 31;
    const int64_t n = A.nb * BS;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t u = w0; u < A.ns * np; u += nw) {
        const int64_t s = u / np;
        const int q = (int)(u - s * np);
        const int64_t b0 = A.sptr[s];
        const int wdt = (int)(A.sptr[s + 1] - b0);
        const int *cp = A.col + b0 * 32 + lane;
        const float2 *vp = vdf + b0 * 32 * (BS * BS) + lane;
        DFAcc acc[BS][PW];
#pragma unroll
        for (int r = 0; r < BS; ++r)
#pragma unroll
            for (int c = 0; c < PW; ++c) acc[r][c].zero();
        for (int k = 0; k < wdt; ++k) {
            const int col = ld_stream(cp + (int64_t)k * 32);
            float2 a[BS * BS];
#pragma unroll
            for (int e = 0; e < BS * BS; ++e) a[e] = __ldg(vp + ((int64_t)k * (BS * BS) + e) * 32);
#pragma unroll
            for (int cc = 0; cc < BS; ++cc) {
                float2 xv[PW];
                ld_row(panel_row(X, n, q, (int64_t)BS * col + cc), xv);
#pragma unroll
                for (int r = 0; r < BS; ++r)
#pragma unroll
                    for (int c = 0; c < PW; ++c) acc[r][c].add(a[r * BS + cc], xv[c]);
            }
        }
        const int64_t row = s * 32 + lane;
        if (row < A.nb) {
#pragma unroll
            for (int r = 0; r < BS; ++r) {
                const int64_t i = (int64_t)BS * row + r;
                const bool f = fixed && fixed[i];
                float2 yv[PW];
#pragma unroll
                for (int c = 0; c < PW; ++c) yv[c] = f ? make_float2(0.f, 0.f) : acc[r][c].get2();
                st_row(Y + ((int64_t)q * n + i) * PW, yv);
            }
        }
    }
}

// k_lincomb with the blocks, the coefficients and the results in double-float.
__global__ void __launch_bounds__(kT)
    k_lincomb_df(int64_t n, int k, int nblk, const float2 *__restrict__ X, const float2 *__restrict__ W,
                 const float2 *__restrict__ P, const double *__restrict__ C, float2 *__restrict__ Xn,
                 float2 *__restrict__ Pn)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    float2 *sC = (float2 *)smraw;
    const int m = nblk * k;
    const int np = (k + PW - 1) / PW;
    const int kp = np * PW;
    for (int e = threadIdx.x; e < m * kp; e += blockDim.x) {
        const int r = e / kp, j = e - r * kp;
        sC[e] = j < k ? df_split(C[(int64_t)j * m + r]) : make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < n; row += (int64_t)gridDim.x * blockDim.x) {
        for (int qo = 0; qo < np; ++qo) {
            DFAcc ax[PW], ap[PW];
#pragma unroll
            for (int c = 0; c < PW; ++c) {
                ax[c].zero();
                ap[c].zero();
            }
            for (int b = 0; b < nblk; ++b) {
                for (int qi = 0; qi < np; ++qi) {
                    float2 v[PW];
                    ld_row(panel_row(b == 0 ? X : (b == 1 ? W : P), n, qi, row), v);
#pragma unroll
                    for (int c = 0; c < PW; ++c) {
                        const int i = qi * PW + c;
                        if (i >= k) break;
                        float2 cr[PW];
                        lds_row(sC + (int64_t)(b * k + i) * kp + qo * PW, cr);
#pragma unroll
                        for (int o = 0; o < PW; ++o) {
                            if (b == 0)
                                ax[o].add(v[c], cr[o]);
                            else
                                ap[o].add(v[c], cr[o]);
                        }
                    }
                }
            }
            float2 pv[PW], xv[PW];
#pragma unroll
            for (int o = 0; o < PW; ++o) {
                pv[o] = ap[o].get2();
                xv[o] = df_add(ax[o].get2(), pv[o]);
            }
            st_row(Pn + ((int64_t)qo * n + row) * PW, pv);
            st_row(Xn + ((int64_t)qo * n + row) * PW, xv);
        }
    }
}

struct F64Acc {
    double v;
    __device__ void zero() { v = 0.0; }
    __device__ void add(double a, double b) { v = fma(a, b, v); }
    __device__ double get() const { return v; }
};
// FP32 panels (the mixed first phase): plain FP32 multiply-adds per thread
// over its CTA's rows (about n / 300 terms), partial sums added in FP64.
struct F32Acc {
    float v;
    __device__ void zero() { v = 0.f; }
    __device__ void add(float a, float b) { v = fmaf(a, b, v); }
    __device__ double get() const { return (double)v; }
};

// Staged operand type and accumulator of the Gram kernel per storage type:
// FP32 panels (FP32 sums), FP64 panels (FP64 sums), double-float panels
// (double-float sums; DF = true).
template <typename T, bool DF>
struct GramArith;
template <>
struct GramArith<float, false> {
    using Stage = float;
    using Acc = F32Acc;
    __device__ static float stage(float x) { return x; }
    __device__ static float none() { return 0.f; }
};
template <>
struct GramArith<double, false> {
    using Stage = double;
    using Acc = F64Acc;
    __device__ static double stage(double x) { return x; }
    __device__ static double none() { return 0.0; }
};
template <>
struct GramArith<float2, true> {  // panels already in double-float (mixed second phase)
    using Stage = float2;
    using Acc = DFAcc;
    __device__ static float2 stage(float2 x) { return x; }
    __device__ static float2 none() { return make_float2(0.f, 0.f); }
};

constexpr int kGramRows = 32;  // rows staged in shared memory per step
constexpr int kGramSub = 4;    // each thread owns a 4 x 4 sub-tile of both Gram matrices

// Shared-memory tile of the Gram staging: kGramRows rows of one 8-column
// panel, row-major, followed by 64 bytes of padding so that consecutive tiles
// start 16 banks apart (the 16-byte loads of the threads of a quarter warp,
// which read two neighbouring tiles, then hit distinct banks).
template <typename St>
__host__ __device__ constexpr int gram_tile_elems()
{
    return kGramRows * PW + 64 / (int)sizeof(St);
}

// 16-byte moves of staged values: global (T) -> shared (St), 16 bytes of
// source per call.
__device__ __forceinline__ void gram_stage16(const float *src, float *dst)
{
    *reinterpret_cast<float4 *>(dst) = __ldg(reinterpret_cast<const float4 *>(src));
}
__device__ __forceinline__ void gram_stage16(const double *src, double *dst)
{
    *reinterpret_cast<double2 *>(dst) = __ldg(reinterpret_cast<const double2 *>(src));
}
__device__ __forceinline__ void gram_stage16(const float2 *src, float2 *dst)
{
    *reinterpret_cast<float4 *>(dst) = __ldg(reinterpret_cast<const float4 *>(src));
}
// four consecutive staged values (16- or 32-byte aligned)
__device__ __forceinline__ void gram_lds4(const float *p, float (&v)[kGramSub])
{
    const float4 w = *reinterpret_cast<const float4 *>(p);
    v[0] = w.x;
    v[1] = w.y;
    v[2] = w.z;
    v[3] = w.w;
}
__device__ __forceinline__ void gram_lds4(const double *p, double (&v)[kGramSub])
{
    const double2 a = reinterpret_cast<const double2 *>(p)[0], b = reinterpret_cast<const double2 *>(p)[1];
    v[0] = a.x;
    v[1] = a.y;
    v[2] = b.x;
    v[3] = b.y;
}
__device__ __forceinline__ void gram_lds4(const float2 *p, float2 (&v)[kGramSub])
{
    const float4 a = reinterpret_cast<const float4 *>(p)[0], b = reinterpret_cast<const float4 *>(p)[1];
    v[0] = make_float2(a.x, a.y);
    v[1] = make_float2(a.z, a.w);
    v[2] = make_float2(b.x, b.y);
    v[3] = make_float2(b.z, b.w);
}

// Upper triangles of S^T (K S) and S^T (M S), S = [X W P] (nblk blocks of k
// columns, each padded to kp = 8 np columns): each CTA reduces a contiguous
// row range and writes its partial sums (FP64) to part[cta][2 * npairs], pair
// p = (i, j), i <= j, numbered row by row over the upper triangle of the
// m = nblk k real columns.
//
// Register-tiled outer products: the padded m_p x m_p matrix is cut into 8 x 8
// tiles; the upper-triangle tiles (I <= J) are split into four 4 x 4 sub-tiles,
// one per thread (4 * T (T + 1) / 2 threads for T = m_p / 8 tile columns, at
// most 312).  A step stages kGramRows rows of every panel of S, K S and M S
// into shared memory, one panel tile after another: the rows of a panel are
// contiguous in global memory, so each warp copies whole tiles with 16-byte
// loads.  Per staged row a thread reads its 4 values of S and 4 of each image
// with 16-byte shared loads and does 32 multiply-adds: FP32 for FP32 panels
// (per CTA row range; the ranges are summed in FP64), FP64 for FP64 panels,
// or double-float (DF: double-float panels of the mixed mode's second phase)
// on the FP32 pipe.  Padding columns are staged as they are
// stored and their sums are not written; the sub-tile below the diagonal of
// a diagonal tile is computed and not written.
template <typename T, bool DF>
__global__ void __launch_bounds__(320)
    k_gram(int64_t n, int k, int nblk, const T *S0, const T *S1, const T *S2, const T *K0, const T *K1, const T *K2,
           const T *M0, const T *M1, const T *M2, double *part)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    const int kp = (k + PW - 1) / PW * PW;
    const int np = kp / PW;
    const int mp = nblk * kp;
    const int m = nblk * k;
    const int npairs = m * (m + 1) / 2;
    const int tiles = mp / PW;
    const int ntasks = kGramSub * tiles * (tiles + 1) / 2;
    using Ar = GramArith<T, DF>;
    using St = typename Ar::Stage;
    constexpr int TE = gram_tile_elems<St>();
    St *sS = (St *)smraw;  // [3][tiles][TE]: S, K S, M S
    const bool active = (int)threadIdx.x < ntasks;
    int ti = 0, tj = 0, oi = 0, oj = 0;
    if (active) {
        const int tp = threadIdx.x >> 2, sub = threadIdx.x & 3;
        int I = 0, rem = tp;
        while (rem >= tiles - I) {
            rem -= tiles - I;
            ++I;
        }
        ti = I;
        tj = I + rem;
        oi = kGramSub * (sub >> 1);
        oj = kGramSub * (sub & 1);
    }
    typename Ar::Acc aA[kGramSub][kGramSub], aB[kGramSub][kGramSub];
#pragma unroll
    for (int a = 0; a < kGramSub; ++a)
#pragma unroll
        for (int b = 0; b < kGramSub; ++b) {
            aA[a][b].zero();
            aB[a][b].zero();
        }
    const int64_t per = (n + gridDim.x - 1) / gridDim.x;
    const int64_t r0 = (int64_t)blockIdx.x * per, r1 = min(n, r0 + per);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    constexpr int kPer16 = 16 / (int)sizeof(T);  // source values per 16-byte move
    const St *pS = sS + ti * TE + oi, *pK = sS + (tiles + tj) * TE + oj, *pM = sS + (2 * tiles + tj) * TE + oj;
    for (int64_t t0 = r0; t0 < r1; t0 += kGramRows) {
        const int rows = (int)((r1 - t0) < (int64_t)kGramRows ? (r1 - t0) : (int64_t)kGramRows);
        const int units = rows * PW / kPer16;  // 16-byte moves per tile
        __syncthreads();
        for (int ta = wid; ta < 3 * tiles; ta += nwarps) {
            const int mat = ta / tiles, t = ta - mat * tiles;
            const int b = t / np, q = t - b * np;
            const T *base = mat == 0 ? (b == 0 ? S0 : (b == 1 ? S1 : S2))
                                     : (mat == 1 ? (b == 0 ? K0 : (b == 1 ? K1 : K2)) : (b == 0 ? M0 : (b == 1 ? M1 : M2)));
            const T *src = base + ((int64_t)q * n + t0) * PW;
            St *dst = sS + ta * TE;
            for (int u = lane; u < units; u += 32) gram_stage16(src + u * kPer16, dst + u * kPer16);
        }
        __syncthreads();
        if (active) {
            for (int r = 0; r < rows; ++r) {
                St si[kGramSub], yk[kGramSub], ym[kGramSub];
                gram_lds4(pS + r * PW, si);
                gram_lds4(pK + r * PW, yk);
                gram_lds4(pM + r * PW, ym);
#pragma unroll
                for (int a = 0; a < kGramSub; ++a)
#pragma unroll
                    for (int b = 0; b < kGramSub; ++b) {
                        aA[a][b].add(si[a], yk[b]);
                        aB[a][b].add(si[a], ym[b]);
                    }
            }
        }
    }
    if (!active) return;
#pragma unroll
    for (int a = 0; a < kGramSub; ++a)
#pragma unroll
        for (int b = 0; b < kGramSub; ++b) {
            const int pi = PW * ti + oi + a, pj = PW * tj + oj + b;  // padded columns
            const int bi = pi / kp, ci = pi - bi * kp, bj = pj / kp, cj = pj - bj * kp;
            if (ci >= k || cj >= k) continue;
            const int i = bi * k + ci, j = bj * k + cj;
            if (i > j) continue;
            const int p = i * m - i * (i - 1) / 2 + (j - i);
            part[(int64_t)blockIdx.x * 2 * npairs + p] = aA[a][b].get();
            part[(int64_t)blockIdx.x * 2 * npairs + npairs + p] = aB[a][b].get();
        }
}

// Sum the per-CTA partials in CTA order (deterministic).
__global__ void k_reduce_parts(const double *__restrict__ part, int nparts, int len, double *__restrict__ out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int b = 0; b < nparts; ++b) s += part[(int64_t)b * len + i];
        out[i] = s;
    }
}

// Pn = W C_w + P C_p ; Xn = X C_x + Pn   (C: m x k column-major, FP64).
// A thread per row and output panel.  The coefficients are staged transposed,
// sC[(b k + i) kp + j] with j padded to kp by zeros, so the 8 coefficients of
// one input value for one output panel are a 16-byte-aligned row of shared
// memory (2 or 4 vector loads per 8 multiply-adds); the input and output rows
// move with 16-byte accesses.
template <typename T>
__global__ void __launch_bounds__(kT)
    k_lincomb(int64_t n, int k, int nblk, const T *__restrict__ X, const T *__restrict__ W, const T *__restrict__ P,
              const double *__restrict__ C, T *__restrict__ Xn, T *__restrict__ Pn)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    T *sC = (T *)smraw;
    const int m = nblk * k;
    const int np = (k + PW - 1) / PW;
    const int kp = np * PW;
    for (int e = threadIdx.x; e < m * kp; e += blockDim.x) {
        const int r = e / kp, j = e - r * kp;
        sC[e] = j < k ? (T)C[(int64_t)j * m + r] : T(0);
    }
    __syncthreads();
    for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < n; row += (int64_t)gridDim.x * blockDim.x) {
        for (int qo = 0; qo < np; ++qo) {
            T ax[PW], ap[PW];
#pragma unroll
            for (int c = 0; c < PW; ++c) ax[c] = ap[c] = T(0);
            for (int b = 0; b < nblk; ++b) {
                for (int qi = 0; qi < np; ++qi) {
                    T v[PW];
                    ld_row(panel_row(b == 0 ? X : (b == 1 ? W : P), n, qi, row), v);
#pragma unroll
                    for (int c = 0; c < PW; ++c) {
                        const int i = qi * PW + c;
                        if (i >= k) break;
                        T cr[PW];
                        lds_row(sC + (int64_t)(b * k + i) * kp + qo * PW, cr);
#pragma unroll
                        for (int o = 0; o < PW; ++o) {
                            if (b == 0)
                                ax[o] = fma(v[c], cr[o], ax[o]);
                            else
                                ap[o] = fma(v[c], cr[o], ap[o]);
                        }
                    }
                }
            }
#pragma unroll
            for (int o = 0; o < PW; ++o) ax[o] += ap[o];
            st_row(Pn + ((int64_t)qo * n + row) * PW, ap);
            st_row(Xn + ((int64_t)qo * n + row) * PW, ax);
        }
    }
}

// R = KX - MX diag(lam); per column: |R_j|^2, |MX_j|^2, max|R_j|  -> part[cta][3k]
// (entry 3 j + {0, 1, 2} of CTA x's row).  CTA (x, q) takes the rows of panel
// q, so a thread's sums are 3 x 8 registers and its rows move as vectors.
template <typename T>
__global__ void __launch_bounds__(kT)
    k_residual(int64_t n, int k, const T *__restrict__ KX, const T *__restrict__ MX, const double *__restrict__ lam,
               T *__restrict__ R, double *part)
{
    __shared__ double sred[3 * PW][kT / 32];
    const int q = blockIdx.y;
    double rr[PW], mm[PW], mx[PW];
    T lq[PW];
#pragma unroll
    for (int c = 0; c < PW; ++c) {
        rr[c] = mm[c] = mx[c] = 0.0;
        lq[c] = q * PW + c < k ? (T)lam[q * PW + c] : T(0);
    }
    for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < n; row += (int64_t)gridDim.x * blockDim.x) {
        const int64_t off = ((int64_t)q * n + row) * PW;
        T kv[PW], mv[PW];
        ld_row(KX + off, kv);
        ld_row(MX + off, mv);
#pragma unroll
        for (int c = 0; c < PW; ++c) {
            if (q * PW + c >= k) {
                kv[c] = T(0);
                continue;
            }
            const T r = kv[c] - mv[c] * lq[c];
            kv[c] = r;
            const double rd = (double)r, md = (double)mv[c];
            rr[c] = fma(rd, rd, rr[c]);
            mm[c] = fma(md, md, mm[c]);
            mx[c] = fmax(mx[c], fabs(rd));
        }
        st_row(R + off, kv);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < PW; ++c) {
        double a = warp_sum(rr[c]), b = warp_sum(mm[c]), m = mx[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) {
            sred[3 * c][wid] = a;
            sred[3 * c + 1][wid] = b;
            sred[3 * c + 2][wid] = m;
        }
    }
    __syncthreads();
    if (threadIdx.x < 3 * PW) {
        const int c = threadIdx.x / 3, t = threadIdx.x % 3;
        if (q * PW + c < k) {
            double v = 0.0;
            for (int w = 0; w < (int)(blockDim.x / 32); ++w) v = t == 2 ? fmax(v, sred[3 * c + t][w]) : v + sred[3 * c + t][w];
            part[(int64_t)blockIdx.x * 3 * k + 3 * (q * PW + c) + t] = v;
        }
    }
}

// k_residual for double-float panels: R = KX - MX diag(lam) in double-float
// arithmetic on the FP32 pipe (lam split once per column); the sums of
// |r|^2 and |m|^2 and max|r| take the leading floats (seven digits are all a
// residual norm needs) into FP64 accumulators (no FP32 underflow of squares
// for badly scaled systems), reduced across threads as in k_residual.
__global__ void __launch_bounds__(kT)
    k_residual_df(int64_t n, int k, const float2 *__restrict__ KX, const float2 *__restrict__ MX,
                  const double *__restrict__ lam, float2 *__restrict__ R, double *part)
{
    __shared__ double sred[3 * PW][kT / 32];
    const int q = blockIdx.y;
    double rr[PW], mm[PW], mx[PW];
    float2 lq[PW];
#pragma unroll
    for (int c = 0; c < PW; ++c) {
        rr[c] = mm[c] = mx[c] = 0.0;
        lq[c] = q * PW + c < k ? df_split(-lam[q * PW + c]) : make_float2(0.f, 0.f);
    }
    for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < n; row += (int64_t)gridDim.x * blockDim.x) {
        const int64_t off = ((int64_t)q * n + row) * PW;
        float2 kv[PW], mv[PW];
        ld_row(KX + off, kv);
        ld_row(MX + off, mv);
#pragma unroll
        for (int c = 0; c < PW; ++c) {
            if (q * PW + c >= k) {
                kv[c] = make_float2(0.f, 0.f);
                continue;
            }
            DFAcc a;  // k + m (-lam)
            a.hi = kv[c].x;
            a.lo = kv[c].y;
            a.add(mv[c], lq[c]);
            const float2 r = a.get2();
            kv[c] = r;
            const double rd = (double)r.x, md = (double)mv[c].x;
            rr[c] = fma(rd, rd, rr[c]);
            mm[c] = fma(md, md, mm[c]);
            mx[c] = fmax(mx[c], fabs(rd));
        }
        st_row(R + off, kv);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < PW; ++c) {
        double a = warp_sum(rr[c]), b = warp_sum(mm[c]), m = mx[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) {
            sred[3 * c][wid] = a;
            sred[3 * c + 1][wid] = b;
            sred[3 * c + 2][wid] = m;
        }
    }
    __syncthreads();
    if (threadIdx.x < 3 * PW) {
        const int c = threadIdx.x / 3, t = threadIdx.x % 3;
        if (q * PW + c < k) {
            double v = 0.0;
            for (int w = 0; w < (int)(blockDim.x / 32); ++w) v = t == 2 ? fmax(v, sred[3 * c + t][w]) : v + sred[3 * c + t][w];
            part[(int64_t)blockIdx.x * 3 * k + 3 * (q * PW + c) + t] = v;
        }
    }
}

// k_eig_precond for double-float panels, in double-float arithmetic (the
// block inverse split once per node).
template <int BS>
__global__ void __launch_bounds__(kT)
    k_eig_precond_df(int64_t nb, int k, const double *__restrict__ dinv, int pc, const float2 *__restrict__ R,
                     float2 *__restrict__ W, const uint8_t *__restrict__ fixed)
{
    const int np = (k + PW - 1) / PW;
    const int64_t n = nb * BS;
    for (int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; node < nb;
         node += (int64_t)gridDim.x * blockDim.x) {
        float2 D[BS * BS];
#pragma unroll
        for (int e = 0; e < BS * BS; ++e)
            D[e] = pc == PFG_PC_NONE ? make_float2(e % (BS + 1) == 0 ? 1.f : 0.f, 0.f)
                                     : df_split(dinv[node * BS * BS + e]);
        for (int q = 0; q < np; ++q) {
            float2 rv[BS][PW];
#pragma unroll
            for (int i = 0; i < BS; ++i) ld_row(panel_row(R, n, q, (int64_t)BS * node + i), rv[i]);
#pragma unroll
            for (int i = 0; i < BS; ++i) {
                const bool f = fixed && fixed[(int64_t)BS * node + i];
                float2 wv[PW];
#pragma unroll
                for (int c = 0; c < PW; ++c) {
                    DFAcc a;
                    a.zero();
#pragma unroll
                    for (int j = 0; j < BS; ++j) a.add(D[BS * i + j], rv[j][c]);
                    wv[c] = f ? make_float2(0.f, 0.f) : a.get2();
                }
                st_row(W + ((int64_t)q * n + (int64_t)BS * node + i) * PW, wv);
            }
        }
    }
}

// W = T R: block Jacobi (BS x BS diagonal blocks of K) per node and column;
// fixed DOFs zeroed.
template <int BS, typename T>
__global__ void __launch_bounds__(kT)
    k_eig_precond(int64_t nb, int k, const double *__restrict__ dinv, int pc, const T *__restrict__ R,
                  T *__restrict__ W, const uint8_t *__restrict__ fixed)
{
    const int np = (k + PW - 1) / PW;
    const int64_t n = nb * BS;
    for (int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; node < nb;
         node += (int64_t)gridDim.x * blockDim.x) {
        // the phase's own precision: FP32 panels take the block inverse in FP32
        using W_t = typename std::conditional<std::is_same<T, float>::value, float, double>::type;
        W_t D[BS * BS];
#pragma unroll
        for (int e = 0; e < BS * BS; ++e)
            D[e] = pc == PFG_PC_NONE ? (e % (BS + 1) == 0 ? W_t(1) : W_t(0)) : (W_t)dinv[node * BS * BS + e];
        for (int q = 0; q < np; ++q) {
            T rv[BS][PW];
#pragma unroll
            for (int i = 0; i < BS; ++i) ld_row(panel_row(R, n, q, (int64_t)BS * node + i), rv[i]);
#pragma unroll
            for (int i = 0; i < BS; ++i) {
                const bool f = fixed && fixed[(int64_t)BS * node + i];
                T wv[PW];
#pragma unroll
                for (int c = 0; c < PW; ++c) {
                    W_t v = W_t(0);
#pragma unroll
                    for (int j = 0; j < BS; ++j) v += D[BS * i + j] * (W_t)rv[j][c];
                    wv[c] = f ? T(0) : (T)v;
                }
                st_row(W + ((int64_t)q * n + (int64_t)BS * node + i) * PW, wv);
            }
        }
    }
}

__device__ __forceinline__ uint64_t splitmix(uint64_t x)
{
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

// X = uniform(-1, 1) from (seed, row, column); padding columns and fixed rows 0.
template <typename T>
__global__ void k_random(int64_t n, int k, uint64_t seed, T *__restrict__ X, const uint8_t *__restrict__ fixed)
{
    const int np = (k + PW - 1) / PW;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n * np * PW;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % PW);
        const int64_t row = (i / PW) % n;
        const int q = (int)(i / (PW * n));
        const int j = q * PW + c;
        const uint64_t h = splitmix(seed * 0x100000001b3ull ^ splitmix((uint64_t)row * 131 + (uint64_t)j));
        const double u = (double)(h >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
        X[i] = (j < k && !(fixed && fixed[row])) ? (T)u : T(0);
    }
}

__device__ __forceinline__ float2 to_df32(float x) { return make_float2(x, 0.f); }
__device__ __forceinline__ double to_f64(float x) { return (double)x; }
__device__ __forceinline__ double to_f64(double x) { return x; }
__device__ __forceinline__ double to_f64(float2 x) { return df_value(x); }

// FP32 panels -> double-float panels (the start of the mixed second phase)
__global__ void k_f32_to_df(int64_t len, const float *__restrict__ a, float2 *__restrict__ b)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = to_df32(a[i]);
}

// first nev columns of X (panels) -> column-major n x nev (FP64)
template <typename T>
__global__ void k_unpanel(int64_t n, int nev, const T *__restrict__ X, double *__restrict__ out)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n * nev; i += (int64_t)gridDim.x * blockDim.x) {
        const int j = (int)(i / n);
        const int64_t row = i - (int64_t)j * n;
        out[i] = to_f64(X[((int64_t)(j / PW) * n + row) * PW + (j % PW)]);
    }
}

// ===================================================================== driver
namespace {

int g_sms = 0;
int sms()
{
    if (!g_sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_sms <= 0) g_sms = 1;
    }
    return g_sms;
}

template <typename T>
struct Blocks {
    DevBuf<T> X, W, P, KX, KW, KP, MX, MW, MP, Xn, Pn, KXn, KPn, MXn, MPn, R;
    void alloc(size_t len)
    {
        for (DevBuf<T> *b : {&X, &W, &P, &KX, &KW, &KP, &MX, &MW, &MP, &Xn, &Pn, &KXn, &KPn, &MXn, &MPn, &R})
            b->resize(len);
    }
};

struct Ctx {
    int64_t n, nb;
    int bs;
    int k, kp, np;
    cudaStream_t st;
    const uint8_t *fixed;
    DevBuf<float2> df_K, df_M;  // the sliced FP64 matrix values as double-float pairs (mixed second phase)
    const DevMatrix *dfK = nullptr, *dfM = nullptr;
    int launches = 0;
    DevBuf<double> part, gram, C, lam_d, dinv;
    std::vector<double> hg, hC, hlam;
    int ngrid;
};

template <typename T>
SellView<T> sell_of(const DevMatrix &A)
{
    if constexpr (std::is_same<T, double>::value)
        return A.sell<double>();
    else
        return A.sell<float>();
}

// A's sliced FP64 values as double-float pairs (converted once per phase).
static const float2 *df_values(Ctx &c, const DevMatrix &A)
{
    const bool isK = &A == c.dfK;
    PFG_CHECK(isK || &A == c.dfM, PFG_E_INTERNAL, "double-float values of an unexpected matrix");
    return isK ? c.df_K.p : c.df_M.p;
}

static void to_df(Ctx &c, const double *a, float2 *b, int64_t len)
{
    k_to_df<<<grid_for(len, 256, sms() * 8), 256, 0, c.st>>>(len, a, b);
    PFG_CUDA(cudaGetLastError());
    ++c.launches;
}

// Y = A X, panels in double-float, A's values as double-float pairs.
static void spmm_df(Ctx &c, const DevMatrix &A, const float2 *X, float2 *Y)
{
    const SellView<double> v = A.sell<double>();
    int per = 0;
    if (A.bs == 3)
        PFG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_spmm_df<3>, kT, 0));
    else
        PFG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_spmm_df<1>, kT, 0));
    const int64_t warps = A.ns * c.np;
    const int g = (int)std::max<int64_t>(1, std::min<int64_t>((warps + 7) / 8, (int64_t)std::max(per, 1) * sms()));
    if (A.bs == 3)
        k_spmm_df<3><<<g, kT, 0, c.st>>>(v, df_values(c, A), c.np, X, Y, c.fixed);
    else
        k_spmm_df<1><<<g, kT, 0, c.st>>>(v, df_values(c, A), c.np, X, Y, c.fixed);
    PFG_CUDA(cudaGetLastError());
    ++c.launches;
}

template <typename T>
void spmm(Ctx &c, const DevMatrix &A, const T *X, T *Y)
{
    if constexpr (std::is_same<T, float2>::value) {
        spmm_df(c, A, X, Y);
    } else {
        const SellView<T> v = sell_of<T>(A);
        int per = 0;
        if (A.bs == 3)
            PFG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_spmm<3, T>, kT, 0));
        else
            PFG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_spmm<1, T>, kT, 0));
        const int64_t warps = A.ns * c.np;
        const int g =
            (int)std::max<int64_t>(1, std::min<int64_t>((warps + 7) / 8, (int64_t)std::max(per, 1) * sms()));
        if (A.bs == 3)
            k_spmm<3, T><<<g, kT, 0, c.st>>>(v, c.np, X, Y, c.fixed);
        else
            k_spmm<1, T><<<g, kT, 0, c.st>>>(v, c.np, X, Y, c.fixed);
        PFG_CUDA(cudaGetLastError());
        ++c.launches;
    }
}

// KX = K X and MX = M X
template <typename T>
void spmm_pair(Ctx &c, const DevMatrix &K, const DevMatrix &M, const T *X, T *KX, T *MX)
{
    spmm<T>(c, K, X, KX);
    spmm<T>(c, M, X, MX);
}

template <typename T>
void gram(Ctx &c, int nblk, const Blocks<T> &B, std::vector<double> &GA, std::vector<double> &GB)
{
    const int m = nblk * c.k;
    const int npairs = m * (m + 1) / 2;
    const int mp = nblk * c.kp;
    const int tiles = mp / PW;
    const int threads = (kGramSub * tiles * (tiles + 1) / 2 + 31) / 32 * 32;
    // staged tiles: 3 matrices x tiles; a double-float value is 8 bytes like a double
    const size_t smem = (size_t)3 * tiles * (kGramRows * PW + 64 / sizeof(T)) * sizeof(T);
    const int g = c.ngrid;
    c.part.ensure((size_t)g * 2 * npairs);
    c.gram.ensure((size_t)2 * npairs);
    // float2: double-float panels (mixed second phase); float: FP32; double: IEEE FP64
    constexpr bool kDF = std::is_same<T, float2>::value;
    auto kern = k_gram<T, kDF>;
    PFG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<g, threads, smem, c.st>>>(c.n, c.k, nblk, B.X.p, B.W.p, B.P.p, B.KX.p, B.KW.p, B.KP.p, B.MX.p, B.MW.p,
                                     B.MP.p, c.part.p);
    k_reduce_parts<<<grid_for(2 * npairs, 256, 64), 256, 0, c.st>>>(c.part.p, g, 2 * npairs, c.gram.p);
    PFG_CUDA(cudaGetLastError());
    c.launches += 2;
    c.hg.resize((size_t)2 * npairs);
    PFG_CUDA(cudaMemcpyAsync(c.hg.data(), c.gram.p, 2 * npairs * sizeof(double), cudaMemcpyDeviceToHost, c.st));
    PFG_CUDA(cudaStreamSynchronize(c.st));
    GA.assign((size_t)m * m, 0.0);
    GB.assign((size_t)m * m, 0.0);
    int p = 0;
    for (int i = 0; i < m; ++i)
        for (int j = i; j < m; ++j, ++p) {
            GA[(size_t)j * m + i] = GA[(size_t)i * m + j] = c.hg[p];
            GB[(size_t)j * m + i] = GB[(size_t)i * m + j] = c.hg[npairs + p];
        }
}

template <typename T>
void lincomb(Ctx &c, int nblk, const T *X, const T *W, const T *P, T *Xn, T *Pn)
{
    const int m = nblk * c.k;
    const size_t smem = (size_t)m * c.kp * sizeof(T);  // (a double-float coefficient is 8 bytes too)
    if constexpr (std::is_same<T, float2>::value) {
        PFG_CUDA(cudaFuncSetAttribute(k_lincomb_df, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_lincomb_df<<<grid_for(c.n, kT, sms() * 8), kT, smem, c.st>>>(c.n, c.k, nblk, X, W, P, c.C.p, Xn, Pn);
    } else {
        PFG_CUDA(cudaFuncSetAttribute(k_lincomb<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_lincomb<T><<<grid_for(c.n, kT, sms() * 8), kT, smem, c.st>>>(c.n, c.k, nblk, X, W, P, c.C.p, Xn, Pn);
    }
    PFG_CUDA(cudaGetLastError());
    ++c.launches;
}

// Rayleigh-Ritz on nblk blocks: C, lam on the device; returns pairs found.
template <typename T>
int rayleigh_ritz(Ctx &c, int nblk, const Blocks<T> &B, double rank_tol)
{
    std::vector<double> GA, GB;
    gram<T>(c, nblk, B, GA, GB);
    const int m = nblk * c.k;
    c.hC.assign((size_t)m * c.k, 0.0);
    c.hlam.assign(c.k, 0.0);
    const int got = small_generalized_eig(m, GA.data(), GB.data(), c.k, rank_tol, c.hlam.data(), c.hC.data());
    if (got < c.k) return got;
    c.C.ensure((size_t)m * c.k);
    c.lam_d.ensure((size_t)c.k);
    PFG_CUDA(cudaMemcpyAsync(c.C.p, c.hC.data(), (size_t)m * c.k * sizeof(double), cudaMemcpyHostToDevice, c.st));
    PFG_CUDA(cudaMemcpyAsync(c.lam_d.p, c.hlam.data(), c.k * sizeof(double), cudaMemcpyHostToDevice, c.st));
    return got;
}

template <typename T>
void apply_rr(Ctx &c, int nblk, Blocks<T> &B)
{
    lincomb<T>(c, nblk, B.X.p, B.W.p, B.P.p, B.Xn.p, B.Pn.p);
    lincomb<T>(c, nblk, B.KX.p, B.KW.p, B.KP.p, B.KXn.p, B.KPn.p);
    lincomb<T>(c, nblk, B.MX.p, B.MW.p, B.MP.p, B.MXn.p, B.MPn.p);
    std::swap(B.X, B.Xn);
    std::swap(B.P, B.Pn);
    std::swap(B.KX, B.KXn);
    std::swap(B.KP, B.KPn);
    std::swap(B.MX, B.MXn);
    std::swap(B.MP, B.MPn);
}

struct ResInfo {
    std::vector<double> rel, maxabs;
};

template <typename T>
ResInfo residuals(Ctx &c, Blocks<T> &B)
{
    const int g = std::min(c.ngrid, 1024);
    c.part.ensure((size_t)g * 3 * c.k);
    if constexpr (std::is_same<T, float2>::value)
        k_residual_df<<<dim3(g, c.np), kT, 0, c.st>>>(c.n, c.k, B.KX.p, B.MX.p, c.lam_d.p, B.R.p, c.part.p);
    else
        k_residual<T><<<dim3(g, c.np), kT, 0, c.st>>>(c.n, c.k, B.KX.p, B.MX.p, c.lam_d.p, B.R.p, c.part.p);
    PFG_CUDA(cudaGetLastError());
    ++c.launches;
    std::vector<double> h((size_t)g * 3 * c.k);
    PFG_CUDA(cudaMemcpyAsync(h.data(), c.part.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c.st));
    PFG_CUDA(cudaStreamSynchronize(c.st));
    ResInfo ri;
    ri.rel.assign(c.k, 0.0);
    ri.maxabs.assign(c.k, 0.0);
    for (int j = 0; j < c.k; ++j) {
        double rr = 0, mm = 0, mx = 0;
        for (int b = 0; b < g; ++b) {
            rr += h[(size_t)b * 3 * c.k + 3 * j];
            mm += h[(size_t)b * 3 * c.k + 3 * j + 1];
            mx = std::max(mx, h[(size_t)b * 3 * c.k + 3 * j + 2]);
        }
        const double den = std::fabs(c.hlam[j]) * std::sqrt(mm);
        ri.rel[j] = den > 0 ? std::sqrt(rr) / den : std::sqrt(rr);
        ri.maxabs[j] = mx;
    }
    return ri;
}

constexpr int kRefreshImages = 10;
constexpr int kFp32Stall = 50;

// One precision phase.  start: 0 random, 1 X already holds a start block.
template <typename T>
int phase(Ctx &c, DevMatrix &K, DevMatrix &M, Blocks<T> &B, const EigConfig &cfg, bool fp32_phase, int start,
          int &iters_left, int &iters_done, double &max_rel, double &ref_r1)
{
    const size_t len = (size_t)c.n * c.kp;
    if constexpr (!std::is_same<T, float2>::value) {
        if (start == 0) {
            k_random<T><<<grid_for((int64_t)len, 256, sms() * 8), 256, 0, c.st>>>(c.n, c.k, cfg.seed, B.X.p,
                                                                                 c.fixed);
            PFG_CUDA(cudaGetLastError());
            ++c.launches;
        }
    }
    const double rank_tol = fp32_phase ? 1e-9 : 1e-13;
    spmm<T>(c, K, B.X.p, B.KX.p);
    spmm<T>(c, M, B.X.p, B.MX.p);
    // Rayleigh-Ritz on X alone (X of LOBPCG_CRS, SparseClass.f90:2063-2067)
    if (rayleigh_ritz<T>(c, 1, B, rank_tol) < c.k) throw Error(PFG_E_BREAKDOWN, "LOBPCG: start block is rank deficient");
    apply_rr<T>(c, 1, B);
    bool haveP = false;
    double best = 1e300, best_lsum = 1e300;
    int since_best = 0, since_refresh = 0;
    for (;;) {
        ResInfo ri = residuals<T>(c, B);
        max_rel = 0.0;
        double maxabs = 0.0;
        for (int j = 0; j < cfg.nev; ++j) {
            max_rel = std::max(max_rel, ri.rel[j]);
            maxabs = std::max(maxabs, ri.maxabs[j]);
        }
        if (ref_r1 < 0) ref_r1 = maxabs;
        if (cfg.debug)
            fprintf(stderr, "[pfg] LOBPCG %s it %d max rel residual %.3e lambda_1 %.9e\n", fp32_phase ? "fp32" : "fp64",
                    iters_done, max_rel, c.hlam[0]);
        const bool conv = cfg.stop_rule == 0 ? (maxabs / (ref_r1 > 0 ? ref_r1 : 1.0) < cfg.tol) : (max_rel < cfg.tol);
        if (conv) return 1;
        if (fp32_phase) {
            if (max_rel < cfg.tol_fp32) return 0;
            // FP32 floor: neither the mean log residual of the wanted pairs
            // (by 10 %) nor the sum of their Ritz values (by more than FP32
            // noise, 1e-6 relative) fell for kFp32Stall iterations.  From a
            // random start the Ritz values fall for many iterations while the
            // relative residuals grow, so the residuals alone are no signal.
            double mlog = 0.0, lsum = 0.0;
            for (int j = 0; j < cfg.nev; ++j) {
                mlog += std::log(std::max(ri.rel[j], 1e-300));
                lsum += c.hlam[j];
            }
            mlog /= cfg.nev;
            const bool res_down = mlog < best - std::log(1.1);
            const bool lam_down = lsum < best_lsum - 1e-6 * std::fabs(best_lsum);
            if (res_down) best = mlog;
            if (lam_down) best_lsum = lsum;
            if (res_down || lam_down) {
                since_best = 0;
            } else if (++since_best > kFp32Stall) {
                return 0;
            }
        }
        if (iters_left <= 0) return -1;
        --iters_left;
        ++iters_done;
        // W = T R, its images
        const int gp = grid_for(c.nb, kT, sms() * 8);
        if constexpr (std::is_same<T, float2>::value) {
            if (c.bs == 3)
                k_eig_precond_df<3><<<gp, kT, 0, c.st>>>(c.nb, c.k, c.dinv.p, cfg.precond, B.R.p, B.W.p, c.fixed);
            else
                k_eig_precond_df<1><<<gp, kT, 0, c.st>>>(c.nb, c.k, c.dinv.p, cfg.precond, B.R.p, B.W.p, c.fixed);
        } else {
            if (c.bs == 3)
                k_eig_precond<3, T><<<gp, kT, 0, c.st>>>(c.nb, c.k, c.dinv.p, cfg.precond, B.R.p, B.W.p, c.fixed);
            else
                k_eig_precond<1, T><<<gp, kT, 0, c.st>>>(c.nb, c.k, c.dinv.p, cfg.precond, B.R.p, B.W.p, c.fixed);
        }
        PFG_CUDA(cudaGetLastError());
        ++c.launches;
        spmm_pair<T>(c, K, M, B.W.p, B.KW.p, B.MW.p);
        int nblk = haveP ? 3 : 2;
        int got = rayleigh_ritz<T>(c, nblk, B, rank_tol);
        if (got < c.k && nblk == 3) {
            nblk = 2;  // P became dependent: drop it this iteration
            got = rayleigh_ritz<T>(c, nblk, B, rank_tol);
        }
        if (got < c.k) throw Error(PFG_E_BREAKDOWN, "LOBPCG: Rayleigh-Ritz basis lost rank");
        apply_rr<T>(c, nblk, B);
        haveP = true;
        // The images KX, MX, KP, MP follow X and P through the same linear
        // combinations; recompute them from X and P every kRefreshImages
        // iterations so rounding in those updates cannot drift the residuals
        // R = KX - MX Lambda away from the true ones (without this the FP64
        // phase stalled near 3e-3 on the 60^3 cantilever).
        if (++since_refresh >= kRefreshImages) {
            since_refresh = 0;
            spmm_pair<T>(c, K, M, B.X.p, B.KX.p, B.MX.p);
            spmm_pair<T>(c, K, M, B.P.p, B.KP.p, B.MP.p);
        }
    }
}

}  // namespace

// Block Jacobi (3x3 node blocks) inverse of K, FP64, for the LOBPCG preconditioner.
void block_jacobi_inverse(const DevMatrix &A, int pc, double *d64, cudaStream_t st);

EigResult lobpcg_solve(DevMatrix &K, DevMatrix &M, const uint8_t *fixed, const EigConfig &cfg_in, double *lambda,
                       double *Xout, cudaStream_t st)
{
    EigConfig cfg = cfg_in;
    PFG_CHECK(K.bs == M.bs && K.nb == M.nb, PFG_E_ARG, "eig: A and B must have the same size and block structure");
    if (cfg.block < cfg.nev) cfg.block = cfg.nev;
    PFG_CHECK(cfg.nev >= 1 && cfg.block <= 32, PFG_E_ARG, "eig: need 1 <= num_eigen <= block size <= 32");
    Ctx c;
    c.n = K.ndof();
    c.nb = K.nb;
    c.bs = K.bs;
    c.k = cfg.block;
    c.kp = (c.k + PW - 1) / PW * PW;
    c.np = c.kp / PW;
    c.st = st;
    c.fixed = fixed;
    c.ngrid = sms() * 2;
    PFG_CHECK(c.n >= 3 * c.k, PFG_E_ARG, "eig: block size too large for the system");
    EigResult res;
    cudaEvent_t e0, e1;
    PFG_CUDA(cudaEventCreate(&e0));
    PFG_CUDA(cudaEventCreate(&e1));
    PFG_CUDA(cudaEventRecord(e0, st));
    c.dinv.ensure((size_t)c.nb * c.bs * c.bs);
    block_jacobi_inverse(K, cfg.precond == PFG_PC_NONE ? PFG_PC_BLOCK_JACOBI : cfg.precond, c.dinv.p, st);
    ++c.launches;
    const size_t len = (size_t)c.n * c.kp;
    int iters_left = cfg.max_itr, iters_done = 0, rc = -1;
    double max_rel = 0.0, ref_r1 = -1.0;
    build_sell(K, true, cfg.precision == PFG_PREC_MIXED, st);
    build_sell(M, true, cfg.precision == PFG_PREC_MIXED, st);
    Blocks<double> B64;
    Blocks<float2> Bdf;
    if (cfg.precision == PFG_PREC_MIXED) {
        // FP32 phase, then the second phase with the panels, images, SpMM,
        // Gram and linear combinations in double-float on the FP32 pipe (the
        // matrices' FP64 values split once here)
        {
            Blocks<float> B32;
            B32.alloc(len);
            double r1 = -1.0;
            rc = phase<float>(c, K, M, B32, cfg, true, 0, iters_left, iters_done, max_rel, r1);
            res.iterations_fp32 = iters_done;
            Bdf.alloc(len);
            k_f32_to_df<<<grid_for((int64_t)len, 256, sms() * 8), 256, 0, st>>>((int64_t)len, B32.X.p, Bdf.X.p);
            PFG_CUDA(cudaGetLastError());
            ++c.launches;
        }
        c.dfK = &K;
        c.dfM = &M;
        c.df_K.resize(K.s64.n);
        c.df_M.resize(M.s64.n);
        to_df(c, K.s64.p, c.df_K.p, (int64_t)K.s64.n);
        to_df(c, M.s64.p, c.df_M.p, (int64_t)M.s64.n);
        rc = phase<float2>(c, K, M, Bdf, cfg, false, 1, iters_left, iters_done, max_rel, ref_r1);
    } else {
        B64.alloc(len);
        rc = phase<double>(c, K, M, B64, cfg, false, 0, iters_left, iters_done, max_rel, ref_r1);
    }
    res.iterations = iters_done;
    res.max_rel_residual = max_rel;
    res.status = rc == 1 ? PFG_OK : PFG_W_NOT_CONVERGED;
    for (int j = 0; j < cfg.nev; ++j) lambda[j] = c.hlam[j];
    if (Xout) {
        if (cfg.precision == PFG_PREC_MIXED)
            k_unpanel<float2><<<grid_for(c.n * cfg.nev, 256, sms() * 8), 256, 0, st>>>(c.n, cfg.nev, Bdf.X.p, Xout);
        else
            k_unpanel<double><<<grid_for(c.n * cfg.nev, 256, sms() * 8), 256, 0, st>>>(c.n, cfg.nev, B64.X.p, Xout);
        PFG_CUDA(cudaGetLastError());
        ++c.launches;
    }
    PFG_CUDA(cudaEventRecord(e1, st));
    PFG_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    res.ms = ms;
    res.launches = c.launches;
    return res;
}

}  // namespace pfg
