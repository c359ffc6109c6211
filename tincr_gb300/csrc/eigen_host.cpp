// Dense symmetric eigensolver for the Davidson subspace matrix (host, FP64).
//
// Householder reduction to tridiagonal form followed by the implicit-shift QL iteration, with
// accumulated transformations (the method of Wilkinson & Reinsch, "Handbook for Automatic
// Computation, Vol. II: Linear Algebra", routines tred2/tql2).  eigh_upper follows the structure of
// the public-domain JAMA transcription of those two routines (JAMA: A Java Matrix Package, NIST and
// The MathWorks, 1999, class EigenvalueDecomposition, methods tred2 and tql2), with row-major
// storage and the input read from the upper triangle.  Only the upper triangle of the
// input is read, like `eigh(UPLO::Upper)` in tincr's Davidson (src/excited_states/solvers/davidson.rs:93).
// The subspace is at most 15 * n_roots wide, so this stays a small host step between device phases.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

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
// iteration with partial-pivoting LU of T - w I for their eigenvectors, Gram-Schmidt within clusters
// of close roots and back-transformation through the k vectors.  About (4/3) n^3 flops against the
// full decomposition's ~9 n^3; Davidson needs n_roots << n pairs.
// a: n x n row-major (upper triangle read); w: k eigenvalues ascending; y: y[r * n + i] = component
// i of eigenvector r.  Returns false on non-finite input.
//
// Threads: the tridiagonalisation deals rows to the team in blocks of eight, two barriers per
// reflection; bisection, inverse iteration and back-transformation run one root per task.  Every
// value is computed by one thread in a fixed order, so results do not depend on the thread count.
// ----------------------------------------------------------------------------------------------

namespace {

// Number of eigenvalues of T (diagonal d, squared off-diagonal bsq) below x: the sign changes of the
// leading principal minors N_i = (d_i - x) N_{i-1} - e_{i-1}^2 N_{i-2} (a division-free recurrence,
// backward stable like the pivot form: each step's rounding is a relative perturbation of d_i - x
// and of e_{i-1}^2).  An exact zero becomes a tiny value of the opposite sign; both terms are
// rescaled by a power of two when the newest leaves [2^-400, 2^400].  Counted at SLICE points at
// once: independent recurrences interleaved, so that their floating-point latencies overlap.  The
// range test reads the exponent bits; the exact rescaling exponent comes from ilogb in the rare
// branch that needs it.
constexpr int SLICE = 4;   // points per multisection step

void sturm_count_multi(const double *d, const double *bsq, int n, const double *x, int *cnt) {
    double n0[SLICE], n1[SLICE];
    for (int q = 0; q < SLICE; ++q) {
        n0[q] = 1.0;
        n1[q] = d[0] - x[q];
        if (n1[q] == 0.0) n1[q] = -0x1p-100;
        cnt[q] = std::signbit(n1[q]) ? 1 : 0;
    }
    for (int i = 1; i < n; ++i) {
        const double di = d[i], bi = bsq[i - 1];
        for (int q = 0; q < SLICE; ++q) {
            double n2 = (di - x[q]) * n1[q] - bi * n0[q];
            unsigned long long bits;
            std::memcpy(&bits, &n2, sizeof bits);
            const int bex = (int)((bits >> 52) & 0x7ff);   // biased exponent (0: zero or subnormal)
            if (n2 == 0.0) {
                n2 = -0x1p-100 * n1[q];
            } else if (bex > 1023 + 400 || bex < 1023 - 400) {
                const double sc = std::ldexp(1.0, -std::ilogb(n2));
                n1[q] *= sc;
                n2 *= sc;
            }
            cnt[q] += std::signbit(n1[q]) != std::signbit(n2) ? 1 : 0;
            n0[q] = n1[q];
            n1[q] = n2;
        }
    }
}

// threads for the tridiagonalisation: the per-step barrier pays off from n ~ 128.  Eight threads come
// within 10% of twelve and sixteen on a 16-core Grace host and leave cores to the CUDA driver and
// the caller, so a preempted thread does not stall every barrier.
int tridiag_threads(int n) {
#ifdef _OPENMP
    return n >= 128 ? std::min(8, omp_get_max_threads()) : 1;
#else
    (void)n;
    return 1;
#endif
}

// a . b with eight independent partial sums (vectorisable, fixed order)
inline double dot8(const double *a, const double *b, int len) {
    double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int j = 0;
    for (; j + 8 <= len; j += 8)
        for (int t = 0; t < 8; ++t) s[t] += a[j + t] * b[j + t];
    double r = ((s[0] + s[1]) + (s[2] + s[3])) + ((s[4] + s[5]) + (s[6] + s[7]));
    for (; j < len; ++j) r += a[j] * b[j];
    return r;
}

}  // namespace

bool eigh_lowest_upper(int n, const double *a, int k, double *w, double *y) {
    if (n <= 0 || k <= 0 || k > n) return false;
    std::vector<double> A((size_t)n * n), d(n), e(n, 0.0), beta(n, 0.0), p(n), uv(2 * (size_t)n), bsq(n);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            const double x = (i <= j) ? a[(size_t)i * n + j] : a[(size_t)j * n + i];
            if (!std::isfinite(x)) return false;
            A[(size_t)i * n + j] = x;
        }
    // 1. T = Q^T A Q.  Reflection c acts on rows/columns c+1..n-1; its vector u (with u_0 = x0 - alpha)
    //    replaces row c to the right of the diagonal (= column c below it), where the back-
    //    transformation reads it.  The full symmetric trailing block is kept up to date.
    //    Rows are dealt to threads in blocks of eight (one cache line of p per thread).  One barrier
    //    and one pass over the owned rows per step: after the barrier, K = beta u.p / 2 and
    //    q = p - K u on every thread; row c+1 is formed privately by every thread from the old values
    //    (the same arithmetic, so the same bits), which gives the next reflection u' without a
    //    second barrier; then each owned row gets rows -= u q^T + q u^T and, in the same pass, its
    //    entry of the next p' = beta' A'' u' and of u'.p' (buffers of the step's parity).  The owner
    //    of row c+1 stores it after the next barrier, when no thread reads the old row.
    const int T = tridiag_threads(n);
    std::vector<double> part(2 * 64, 0.0), pp(2 * (size_t)n);
    // the reflection of row c from its updated entries row[c..n-1] (row[0] = the diagonal):
    // writes u (row[1..], with u_0 = x0 - alpha) and returns beta (0: nothing to reflect)
    auto reflect = [](double *row, int n1, double &dc, double &ec) {
        const double x0 = row[1];
        double s2 = 0.0;
        for (int i = 2; i <= n1; ++i) s2 += row[i] * row[i];
        dc = row[0];
        if (s2 == 0.0) {
            ec = x0;
            return 0.0;
        }
        const double nx = std::sqrt(x0 * x0 + s2);
        const double alpha = x0 > 0.0 ? -nx : nx;
        ec = alpha;
        row[1] = x0 - alpha;
        return 1.0 / (alpha * (alpha - x0));
    };
    if (n >= 3) {
#pragma omp parallel num_threads(T) if (T > 1)
    {
#ifdef _OPENMP
        const int nt = omp_get_num_threads(), me = omp_get_thread_num();
#else
        const int nt = 1, me = 0;
#endif
        std::vector<double> q(n), nxt(n), cur(n);   // cur: row c (u in cur[1..]), nxt: row c+1 being formed
        for (int j = 0; j < n; ++j) cur[j] = A[j];  // row 0 (c = 0)
        double d0, e0;
        double bet = reflect(cur.data(), n - 1, d0, e0);   // the same on every thread
        if (me == 0) {
            d[0] = d0;
            e[0] = e0;
        }
        // row this thread owns whose reflection it still has to store (row 0: thread 0, after the
        // first barrier, since every thread copies the old row 0 first)
        int pending = me == 0 ? 0 : -1;
        // p = beta A' u of step 0 on the owned rows (later steps form theirs while updating)
        if (bet != 0.0) {
            double up = 0.0;
            for (int i = 1; i < n; ++i) {
                if ((i >> 3) % nt != me) continue;
                pp[i] = bet * dot8(&A[(size_t)i * n + 1], cur.data() + 1, n - 1);
                up += cur[i] * pp[i];
            }
            part[me] = up;
        }
        for (int c = 0; c + 2 < n; ++c) {
            const double *u = cur.data() - c;   // u[i] for i = c+1..n-1
            const double *p = pp.data() + (size_t)(c & 1) * n;
            const double *pt = part.data() + (c & 1) * 64;
            double *pn = pp.data() + (size_t)((c + 1) & 1) * n;
            double *ptn = part.data() + ((c + 1) & 1) * 64;
#pragma omp barrier
            if (pending >= 0) {   // row c, formed in the previous step: past the barrier nobody reads it
                for (int j = c; j < n; ++j) A[(size_t)c * n + j] = cur[j - c];
                pending = -1;
            }
            // row c+1 (columns c+1..n-1) after this step's update, on every thread
            const int r = c + 1;
            double K = 0.0;
            if (bet != 0.0) {
                double ut = 0.0;
                for (int t = 0; t < nt; ++t) ut += pt[t];
                K = 0.5 * bet * ut;
                for (int j = c + 1; j < n; ++j) q[j] = p[j] - K * u[j];
                const double ur = u[r], qr = q[r];
                for (int j = r; j < n; ++j) nxt[j - r] = A[(size_t)r * n + j] - (ur * q[j] + qr * u[j]);
            } else {
                for (int j = r; j < n; ++j) nxt[j - r] = A[(size_t)r * n + j];
            }
            double dr = 0.0, er = 0.0, betn = 0.0;
            if (c + 3 < n) betn = reflect(nxt.data(), n - r - 1, dr, er);
            // owned rows c+2..: this step's update and, in the same pass, the next step's p
            const double *un = nxt.data() - r;   // next u[i] for i = r+1..n-1
            double upn = 0.0;
            for (int i = c + 2; i < n; ++i) {
                if ((i >> 3) % nt != me) continue;
                double *row = &A[(size_t)i * n];
                if (bet != 0.0) {
                    const double ui = u[i], qi = q[i];
                    row[c + 1] -= ui * q[c + 1] + qi * u[c + 1];
                    if (betn != 0.0) {
                        double acc = 0.0;
#pragma omp simd reduction(+ : acc)
                        for (int j = c + 2; j < n; ++j) {
                            const double x = row[j] - (ui * q[j] + qi * u[j]);
                            row[j] = x;
                            acc += x * un[j];
                        }
                        pn[i] = betn * acc;
                        upn += un[i] * pn[i];
                    } else {
#pragma omp simd
                        for (int j = c + 2; j < n; ++j) row[j] -= ui * q[j] + qi * u[j];
                    }
                } else if (betn != 0.0) {
                    pn[i] = betn * dot8(row + c + 2, un + c + 2, n - c - 2);
                    upn += un[i] * pn[i];
                }
            }
            ptn[me] = upn;
            if (me == 0) {
                beta[c] = bet;
                if (c + 3 < n) { d[r] = dr; e[r] = er; }
            }
            std::swap(cur, nxt);   // cur = row c+1, cur[0] its diagonal
            bet = betn;
            if ((r >> 3) % nt == me) pending = r;
        }
        if (pending >= 0) {
            const int r = pending;
            for (int j = r; j < n; ++j) A[(size_t)r * n + j] = cur[j - r];
        }
    }
    }
    if (n >= 2) {
        d[n - 2] = A[(size_t)(n - 2) * n + n - 2];
        e[n - 2] = A[(size_t)(n - 2) * n + n - 1];
    }
    d[n - 1] = A[(size_t)(n - 1) * n + n - 1];
    e[n - 1] = 0.0;
    // 2. eigenvalues by bisection, one root per task
    double lo = 1e300, hi = -1e300, emax2 = 0.0;
    for (int i = 0; i < n; ++i) {
        const double r = std::fabs(e[i]) + (i > 0 ? std::fabs(e[i - 1]) : 0.0);
        lo = std::min(lo, d[i] - r);
        hi = std::max(hi, d[i] + r);
        emax2 = std::max(emax2, e[i] * e[i]);
        bsq[i] = e[i] * e[i];
    }
    const double eps = 2.220446049250313e-16;
    const double tnorm = std::max(std::fabs(lo), std::fabs(hi));
    const double pivmin = 2.2250738585072014e-308 * std::max(1.0, emax2);
    lo -= 2.0 * eps * tnorm + 2.0 * pivmin;
    hi += 2.0 * eps * tnorm + 2.0 * pivmin;
    const bool par_roots = k >= 4 && n >= 48;
    const double tiny = eps * std::max(tnorm, 1e-300);
    const double ortol = 1e-3 * tnorm;
    // one parallel region for the root phases (each region start wakes the team)
#ifdef _OPENMP
    const int root_threads = std::min(12, omp_get_max_threads());
#else
    const int root_threads = 1;
#endif
#pragma omp parallel num_threads(root_threads) if (par_roots)
    {
#pragma omp for schedule(dynamic, 1)
    for (int r = 0; r < k; ++r) {
        // multisection: SLICE interior points per step cut [x_lo, x_hi] into SLICE + 1 parts
        double x_lo = lo, x_hi = hi;
        for (int it = 0; it < 200; ++it) {
            if (x_hi - x_lo <= 2.0 * eps * std::max(std::fabs(x_lo), std::fabs(x_hi)) + 4.0 * pivmin) break;
            double xs[SLICE];
            int cs[SLICE];
            const double h = (x_hi - x_lo) / (SLICE + 1);
            for (int q = 0; q < SLICE; ++q) xs[q] = x_lo + h * (q + 1);
            sturm_count_multi(d.data(), bsq.data(), n, xs, cs);
            int f = 0;   // first point with more than r eigenvalues below it
            while (f < SLICE && cs[f] <= r) ++f;
            const double a = f > 0 ? xs[f - 1] : x_lo, b = f < SLICE ? xs[f] : x_hi;
            if (!(a > x_lo || b < x_hi)) break;   // no representable progress left
            x_lo = a;
            x_hi = b;
        }
        w[r] = 0.5 * (x_lo + x_hi);
    }
    // 3. inverse iteration on T - w I (LU with partial pivoting), one root per task; y holds the
    //    eigenvectors of T until the back-transformation
#pragma omp for schedule(dynamic, 1)
    for (int r = 0; r < k; ++r) {
        std::vector<double> dl(n), dd(n), du(n), du2(n);
        std::vector<char> swp(n);
        double *z = y + (size_t)r * n;
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
    }
    // Gram-Schmidt (twice) against the lower roots of the same cluster: roots closer than 1e-3 |T|
    // (the criterion of LAPACK's dstein); separated roots are orthogonal to rounding already
#pragma omp single
    for (int r = 1, r0 = 0; r < k; ++r) {
        if (w[r] - w[r - 1] > ortol) {
            r0 = r;
            continue;
        }
        double *z = y + (size_t)r * n;
        for (int pass = 0; pass < 2; ++pass)
            for (int q = r0; q < r; ++q) {
                const double *yq = y + (size_t)q * n;
                double s = 0.0;
                for (int i = 0; i < n; ++i) s += yq[i] * z[i];
                for (int i = 0; i < n; ++i) z[i] -= s * yq[i];
            }
        double nrm = 0.0;
        for (int i = 0; i < n; ++i) nrm += z[i] * z[i];
        nrm = 1.0 / std::sqrt(nrm);
        for (int i = 0; i < n; ++i) z[i] *= nrm;
    }
    // 4. back-transformation y = H_0 ... H_{n-3} z, one root per task
#pragma omp for schedule(dynamic, 1)
    for (int r = 0; r < k; ++r) {
        double *yr = y + (size_t)r * n;
        for (int c = n - 3; c >= 0; --c) {
            if (beta[c] == 0.0) continue;
            const int n1 = n - c - 1;
            const double *u = &A[(size_t)c * n + c + 1];
            double s = 0.0;
#pragma omp simd reduction(+ : s)
            for (int i = 0; i < n1; ++i) s += u[i] * yr[c + 1 + i];
            s *= beta[c];
#pragma omp simd
            for (int i = 0; i < n1; ++i) yr[c + 1 + i] -= s * u[i];
        }
    }
    }   // omp parallel
    for (int r = 0; r < k; ++r)
        if (!std::isfinite(w[r])) return false;
    return true;
}

}  // namespace tincr
