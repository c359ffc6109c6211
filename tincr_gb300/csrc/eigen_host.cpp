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

}  // namespace tincr
