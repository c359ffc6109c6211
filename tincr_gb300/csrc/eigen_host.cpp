// Dense symmetric eigensolver for the Davidson subspace matrix (host, FP64).
//
// Householder reduction to tridiagonal form followed by the implicit-shift QL iteration, with
// accumulated transformations (the method of Wilkinson & Reinsch, "Handbook for Automatic
// Computation, Vol. II: Linear Algebra", routines tred2/tql2).  Only the upper triangle of the
// input is read, like `eigh(UPLO::Upper)` in tincr's Davidson (src/excited_states/solvers/davidson.rs:93).
// The subspace is at most 15 * n_roots wide, so this stays a small host step between device phases.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

namespace tincr {

// a: n x n row-major (upper triangle read); w: eigenvalues ascending; z: n x n row-major with the
// eigenvector of w[k] in column k.  Returns false if the QL iteration did not converge.
bool eigh_upper(int n, const double *a, double *w, double *z) {
    std::vector<double> V((size_t)n * n), d(n), e(n);
    auto v = [&](int i, int j) -> double & { return V[(size_t)i * n + j]; };
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) v(i, j) = (i <= j) ? a[(size_t)i * n + j] : a[(size_t)j * n + i];
    for (int j = 0; j < n; ++j) d[j] = v(n - 1, j);

    // Householder tridiagonalisation (tred2)
    for (int i = n - 1; i > 0; --i) {
        double scale = 0.0, h = 0.0;
        for (int k = 0; k < i; ++k) scale += std::fabs(d[k]);
        if (scale == 0.0) {
            e[i] = d[i - 1];
            for (int j = 0; j < i; ++j) {
                d[j] = v(i - 1, j);
                v(i, j) = 0.0;
                v(j, i) = 0.0;
            }
        } else {
            for (int k = 0; k < i; ++k) {
                d[k] /= scale;
                h += d[k] * d[k];
            }
            double f = d[i - 1];
            double g = std::sqrt(h);
            if (f > 0) g = -g;
            e[i] = scale * g;
            h -= f * g;
            d[i - 1] = f - g;
            for (int j = 0; j < i; ++j) e[j] = 0.0;
            for (int j = 0; j < i; ++j) {
                f = d[j];
                v(j, i) = f;
                g = e[j] + v(j, j) * f;
                for (int k = j + 1; k <= i - 1; ++k) {
                    g += v(k, j) * d[k];
                    e[k] += v(k, j) * f;
                }
                e[j] = g;
            }
            f = 0.0;
            for (int j = 0; j < i; ++j) {
                e[j] /= h;
                f += e[j] * d[j];
            }
            double hh = f / (h + h);
            for (int j = 0; j < i; ++j) e[j] -= hh * d[j];
            for (int j = 0; j < i; ++j) {
                f = d[j];
                g = e[j];
                for (int k = j; k <= i - 1; ++k) v(k, j) -= (f * e[k] + g * d[k]);
                d[j] = v(i - 1, j);
                v(i, j) = 0.0;
            }
        }
        d[i] = h;
    }
    // accumulate transformations
    for (int i = 0; i < n - 1; ++i) {
        v(n - 1, i) = v(i, i);
        v(i, i) = 1.0;
        double h = d[i + 1];
        if (h != 0.0) {
            for (int k = 0; k <= i; ++k) d[k] = v(k, i + 1) / h;
            for (int j = 0; j <= i; ++j) {
                double g = 0.0;
                for (int k = 0; k <= i; ++k) g += v(k, i + 1) * v(k, j);
                for (int k = 0; k <= i; ++k) v(k, j) -= g * d[k];
            }
        }
        for (int k = 0; k <= i; ++k) v(k, i + 1) = 0.0;
    }
    for (int j = 0; j < n; ++j) {
        d[j] = v(n - 1, j);
        v(n - 1, j) = 0.0;
    }
    v(n - 1, n - 1) = 1.0;
    e[0] = 0.0;

    // implicit QL (tql2)
    for (int i = 1; i < n; ++i) e[i - 1] = e[i];
    e[n - 1] = 0.0;
    double f = 0.0, tst1 = 0.0;
    const double eps = std::ldexp(1.0, -52);
    for (int l = 0; l < n; ++l) {
        tst1 = std::max(tst1, std::fabs(d[l]) + std::fabs(e[l]));
        int m = l;
        while (m < n) {
            if (std::fabs(e[m]) <= eps * tst1) break;
            ++m;
        }
        if (m > l) {
            int iter = 0;
            do {
                if (++iter > 60) return false;
                double g = d[l];
                double p = (d[l + 1] - g) / (2.0 * e[l]);
                double r = std::hypot(p, 1.0);
                if (p < 0) r = -r;
                d[l] = e[l] / (p + r);
                d[l + 1] = e[l] * (p + r);
                double dl1 = d[l + 1];
                double h = g - d[l];
                for (int i = l + 2; i < n; ++i) d[i] -= h;
                f += h;
                p = d[m];
                double c = 1.0, c2 = c, c3 = c;
                double el1 = e[l + 1];
                double s = 0.0, s2 = 0.0;
                for (int i = m - 1; i >= l; --i) {
                    c3 = c2;
                    c2 = c;
                    s2 = s;
                    g = c * e[i];
                    h = c * p;
                    r = std::hypot(p, e[i]);
                    e[i + 1] = s * r;
                    s = e[i] / r;
                    c = p / r;
                    p = c * d[i] - s * g;
                    d[i + 1] = h + s * (c * g + s * d[i]);
                    for (int k = 0; k < n; ++k) {
                        h = v(k, i + 1);
                        v(k, i + 1) = s * v(k, i) + c * h;
                        v(k, i) = c * v(k, i) - s * h;
                    }
                }
                p = -s * s2 * c3 * el1 * e[l] / dl1;
                e[l] = s * p;
                d[l] = c * p;
            } while (std::fabs(e[l]) > eps * tst1);
        }
        d[l] = d[l] + f;
        e[l] = 0.0;
    }
    // sort ascending
    std::vector<int> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return d[x] < d[y]; });
    for (int k = 0; k < n; ++k) {
        w[k] = d[idx[k]];
        for (int i = 0; i < n; ++i) z[(size_t)i * n + k] = v(i, idx[k]);
    }
    return true;
}

// ----------------------------------------------------------------------------------------------
// The k lowest eigenpairs only: Householder tridiagonalisation without accumulating Q (the
// reflection vectors are kept), bisection on Sturm counts for the k smallest eigenvalues, inverse
// iteration with partial-pivoting LU of T - w I for their eigenvectors, Gram-Schmidt among them
// (separates (near-)degenerate roots) and back-transformation through the k vectors.  About
// (4/3) n^3 flops against the full decomposition's ~9 n^3; Davidson needs n_roots << n pairs.
// a: n x n row-major (upper triangle read); w: k eigenvalues ascending; y: y[r * n + i] = component
// i of eigenvector r.  Returns false on non-finite input.
// ----------------------------------------------------------------------------------------------

namespace {

int sturm_count(const std::vector<double> &d, const std::vector<double> &e, int n, double x, double pivmin) {
    int c = 0;
    double q = d[0] - x;
    if (std::fabs(q) < pivmin) q = -pivmin;
    if (q < 0.0) ++c;
    for (int i = 1; i < n; ++i) {
        q = d[i] - x - e[i - 1] * e[i - 1] / q;
        if (std::fabs(q) < pivmin) q = -pivmin;
        if (q < 0.0) ++c;
    }
    return c;
}

}  // namespace

bool eigh_lowest_upper(int n, const double *a, int k, double *w, double *y) {
    if (n <= 0 || k <= 0 || k > n) return false;
    std::vector<double> A((size_t)n * n), d(n), e(n, 0.0), beta(n, 0.0), p(n);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            const double x = (i <= j) ? a[(size_t)i * n + j] : a[(size_t)j * n + i];
            if (!std::isfinite(x)) return false;
            A[(size_t)i * n + j] = x;
        }
    // 1. T = Q^T A Q; reflection k acts on rows/columns k+1..n-1, its vector u kept in column k
    //    below the diagonal (stored transposed in row k to the right of the diagonal for contiguous
    //    access)
    // rows of the matrix-vector product and of the rank-2 update are spread over host threads for
    // large subspaces; every row is computed by one thread in a fixed order (deterministic)
    const bool par = n >= 256;
    double bet_s = 0.0;
    bool skip = false;
#pragma omp parallel num_threads(8) if (par)
    for (int c = 0; c + 2 < n; ++c) {
        const int n1 = n - c - 1;
        double *u = &A[(size_t)c * n + c + 1];            // row c, columns c+1.. (= column c by symmetry)
#pragma omp single
        {
            const double x0 = u[0];
            double s2 = 0.0;
            for (int i = 1; i < n1; ++i) s2 += u[i] * u[i];
            d[c] = A[(size_t)c * n + c];
            skip = s2 == 0.0;
            if (skip) {
                beta[c] = 0.0;
                e[c] = x0;
            } else {
                const double nx = std::sqrt(x0 * x0 + s2);
                const double alpha = x0 > 0.0 ? -nx : nx;
                bet_s = 1.0 / (alpha * (alpha - x0));
                u[0] = x0 - alpha;
                beta[c] = bet_s;
                e[c] = alpha;
            }
        }
        if (skip) continue;   // every thread sees the same flag after the single's barrier
        const double bet = bet_s;
        // p = bet A' u over the trailing block (symmetric, full storage kept up to date)
#pragma omp for schedule(static)
        for (int i = 0; i < n1; ++i) {
            const double *row = &A[(size_t)(c + 1 + i) * n + c + 1];
            double acc = 0.0;
            for (int j = 0; j < n1; ++j) acc += row[j] * u[j];
            p[i] = bet * acc;
        }
#pragma omp single
        {
            double up = 0.0;
            for (int i = 0; i < n1; ++i) up += u[i] * p[i];
            const double K = 0.5 * bet * up;
            for (int i = 0; i < n1; ++i) p[i] -= K * u[i];
        }
#pragma omp for schedule(static)
        for (int i = 0; i < n1; ++i) {
            double *row = &A[(size_t)(c + 1 + i) * n + c + 1];
            const double ui = u[i], pi = p[i];
            for (int j = 0; j < n1; ++j) row[j] -= ui * p[j] + pi * u[j];
        }
    }
    if (n >= 2) {
        d[n - 2] = A[(size_t)(n - 2) * n + n - 2];
        e[n - 2] = A[(size_t)(n - 2) * n + n - 1];
    }
    d[n - 1] = A[(size_t)(n - 1) * n + n - 1];
    e[n - 1] = 0.0;
    // 2. eigenvalues by bisection
    double lo = 1e300, hi = -1e300, emax2 = 0.0;
    for (int i = 0; i < n; ++i) {
        const double r = std::fabs(e[i]) + (i > 0 ? std::fabs(e[i - 1]) : 0.0);
        lo = std::min(lo, d[i] - r);
        hi = std::max(hi, d[i] + r);
        emax2 = std::max(emax2, e[i] * e[i]);
    }
    const double eps = 2.220446049250313e-16;
    const double tnorm = std::max(std::fabs(lo), std::fabs(hi));
    const double pivmin = 2.2250738585072014e-308 * std::max(1.0, emax2);
    lo -= 2.0 * eps * tnorm + 2.0 * pivmin;
    hi += 2.0 * eps * tnorm + 2.0 * pivmin;
    double left = lo;   // eigenvalue r lies above the previous one
    for (int r = 0; r < k; ++r) {
        double x_lo = left, x_hi = hi;
        for (int it = 0; it < 200; ++it) {
            if (x_hi - x_lo <= 2.0 * eps * std::max(std::fabs(x_lo), std::fabs(x_hi)) + 4.0 * pivmin) break;
            const double mid = 0.5 * (x_lo + x_hi);
            if (sturm_count(d, e, n, mid, pivmin) > r) x_hi = mid;
            else x_lo = mid;
        }
        w[r] = 0.5 * (x_lo + x_hi);
        left = x_lo;
    }
    // 3. inverse iteration on T - w I (LU with partial pivoting)
    std::vector<double> dl(n), dd(n), du(n), du2(n), z(n);
    std::vector<char> swp(n);
    const double tiny = eps * std::max(tnorm, 1e-300);
    for (int r = 0; r < k; ++r) {
        for (int i = 0; i < n; ++i) {
            dd[i] = d[i] - w[r];
            dl[i] = e[i];
            du[i] = e[i];
            du2[i] = 0.0;
            swp[i] = 0;
        }
        for (int i = 0; i + 1 < n; ++i) {
            if (std::fabs(dd[i]) >= std::fabs(dl[i])) {
                if (std::fabs(dd[i]) < tiny) dd[i] = dd[i] < 0.0 ? -tiny : tiny;
                const double l = dl[i] / dd[i];
                dl[i] = l;
                dd[i + 1] -= l * du[i];
            } else {
                const double l = dd[i] / dl[i];
                dd[i] = dl[i];
                dl[i] = l;
                const double t = du[i];
                du[i] = dd[i + 1];
                dd[i + 1] = t - l * dd[i + 1];
                if (i + 2 < n) {
                    du2[i] = du[i + 1];
                    du[i + 1] = -l * du[i + 1];
                }
                swp[i] = 1;
            }
        }
        if (std::fabs(dd[n - 1]) < tiny) dd[n - 1] = dd[n - 1] < 0.0 ? -tiny : tiny;
        for (int i = 0; i < n; ++i) z[i] = 1.0 + 0.5 * (double)((i * (r + 1) * 7919 + 13 * r) % 97) / 97.0;
        for (int it = 0; it < 3; ++it) {
            for (int i = 0; i + 1 < n; ++i) {
                if (swp[i]) std::swap(z[i], z[i + 1]);
                z[i + 1] -= dl[i] * z[i];
            }
            for (int i = n - 1; i >= 0; --i) {
                double s = z[i];
                if (i + 1 < n) s -= du[i] * z[i + 1];
                if (i + 2 < n) s -= du2[i] * z[i + 2];
                z[i] = s / dd[i];
            }
            double nrm = 0.0;
            for (int i = 0; i < n; ++i) nrm += z[i] * z[i];
            nrm = 1.0 / std::sqrt(nrm);
            for (int i = 0; i < n; ++i) z[i] *= nrm;
        }
        // Gram-Schmidt against the lower roots (twice)
        for (int pass = 0; pass < 2; ++pass)
            for (int q = 0; q < r; ++q) {
                const double *yq = y + (size_t)q * n;   // still in the tridiagonal basis
                double s = 0.0;
                for (int i = 0; i < n; ++i) s += yq[i] * z[i];
                for (int i = 0; i < n; ++i) z[i] -= s * yq[i];
            }
        double nrm = 0.0;
        for (int i = 0; i < n; ++i) nrm += z[i] * z[i];
        nrm = 1.0 / std::sqrt(nrm);
        for (int i = 0; i < n; ++i) y[(size_t)r * n + i] = z[i] * nrm;
    }
    // 4. back-transformation y = H_0 ... H_{n-3} z
    for (int r = 0; r < k; ++r) {
        double *yr = y + (size_t)r * n;
        for (int c = n - 3; c >= 0; --c) {
            if (beta[c] == 0.0) continue;
            const int n1 = n - c - 1;
            const double *u = &A[(size_t)c * n + c + 1];
            double s = 0.0;
            for (int i = 0; i < n1; ++i) s += u[i] * yr[c + 1 + i];
            s *= beta[c];
            for (int i = 0; i < n1; ++i) yr[c + 1 + i] -= s * u[i];
        }
    }
    for (int r = 0; r < k; ++r)
        if (!std::isfinite(w[r])) return false;
    return true;
}

}  // namespace tincr
