// Slater-Koster rules, cubic B-spline evaluation and gamma-function derivatives for the pairwise
// atom kernels (host and device).
//
// Splines: FITPACK representation (knots t[0..nt), coefficients c[0..nt-4), degree 3) as produced
// by `splrep` (tincr: Rusty-FITPACK `splrep` in src/initialization/parameters.rs:215-243).  The
// value and first derivative come from the Cox-de Boor recursion for the four non-zero cubic
// B-splines on the knot interval [t_l, t_{l+1}) (de Boor, "A Practical Guide to Splines", 1978),
// the derivative through the degree-2 basis: s'(x) = sum_i 3 (c_i - c_{i-1}) / (t_{i+3} - t_i) N_{i,2}(x).
// Outside [t_3, t_{nt-4}] the spline is taken as zero (value and derivative), or, with `extrapolate`,
// beyond t_{nt-4} as the polynomial piece of the last interval (FITPACK splev with ext = 0).
//
// SK rules: s and p orbitals, real harmonics m = -1, 0, +1 -> y, z, x, integrals in slot order
// ss_sigma, sp_sigma, ps_sigma, pp_pi, pp_sigma (src/param/slako_transformations.rs:57-680).  The
// gradient with respect to the inter-centre vector r = pos2 - pos1 is
//     d/dr_c [P(u) V(r)] = (grad_u P . (e_c - u_c u)) V / r + P V'(r) u_c
// which is the quantity tincr's `slako_transformation_gradients` (:682-6404) hard-codes.
#pragma once

#include <math.h>

#ifdef __CUDACC__
#define TINCR_HD __host__ __device__ __forceinline__
#else
#define TINCR_HD inline
#endif

namespace tincr {

constexpr int SK_SLOTS = 5;

// Four cubic B-spline values (and degree-2 values for the derivative) at x on interval l.
// Returns false when x is outside the spline's support [t_3, t_{nt-4}], unless `extrapolate` and
// x > t_{nt-4}: then the last interval's four B-splines, whose Cox-de Boor polynomials continue
// past its end (the boundary piece of the spline).
TINCR_HD bool bspline3_basis(const double *t, int nt, double x, int &l, double N3[4], double N2[3],
                             bool extrapolate = false) {
    const int k = 3;
    const int lo = k, hi = nt - k - 1;          // valid intervals l in [lo, hi-1], x in [t_lo, t_hi]
    if (!(x >= t[lo] && (x <= t[hi] || extrapolate))) return false;
    int a = lo, b = hi - 1;
    // binary search for t[l] <= x < t[l+1], with x == t[hi] in the last interval
    while (a < b) {
        int mid = (a + b + 1) >> 1;
        if (t[mid] <= x) a = mid; else b = mid - 1;
    }
    l = a;
    while (l > lo && t[l] == t[l + 1]) --l;
    // Cox-de Boor: N[j] for degree d, j = 0..d over B-splines l-d..l
    double N[4] = {1.0, 0.0, 0.0, 0.0};
    double left[4], right[4];
    for (int d = 1; d <= k; ++d) {
        left[d] = x - t[l + 1 - d];
        right[d] = t[l + d] - x;
        double saved = 0.0;
        for (int r = 0; r < d; ++r) {
            double den = right[r + 1] + left[d - r];
            double temp = den != 0.0 ? N[r] / den : 0.0;
            N[r] = saved + right[r + 1] * temp;
            saved = left[d - r] * temp;
        }
        N[d] = saved;
        if (d == 2) {
            N2[0] = N[0];
            N2[1] = N[1];
            N2[2] = N[2];
        }
    }
    for (int j = 0; j < 4; ++j) N3[j] = N[j];
    return true;
}

// value and derivative of one spline from a precomputed basis on interval l
TINCR_HD void bspline3_eval(const double *t, const double *c, int l, const double N3[4], const double N2[3],
                            double &val, double &der) {
    // B-splines of degree 3 non-zero on [t_l, t_{l+1}): indices l-3 .. l
    val = c[l - 3] * N3[0] + c[l - 2] * N3[1] + c[l - 1] * N3[2] + c[l] * N3[3];
    // derivative: degree-2 B-splines l-2 .. l with coefficients 3 (c_i - c_{i-1}) / (t_{i+3} - t_i)
    double d = 0.0;
    for (int j = 0; j < 3; ++j) {
        int i = l - 2 + j;
        double den = t[i + 3] - t[i];
        if (den != 0.0) d += 3.0 * (c[i] - c[i - 1]) / den * N2[j];
    }
    der = d;
}

// Cartesian axis of a real p orbital: m = -1 -> y (1), 0 -> z (2), +1 -> x (0)
TINCR_HD int p_axis(int m) { return m == -1 ? 1 : (m == 0 ? 2 : 0); }

// Value of one SK matrix element and its gradient w.r.t. r (vector from centre 1 to 2).
// u: direction cosines, r: distance, v/dv: integrals and r-derivatives in slot order.
TINCR_HD void sk_element(int l1, int m1, int l2, int m2, const double u[3], double r, const double v[SK_SLOTS],
                         const double dv[SK_SLOTS], double &val, double g[3]) {
    // angular factors: up to two terms (slot, P, grad_u P)
    int slot[2];
    double P[2];
    double gu[2][3] = {{0, 0, 0}, {0, 0, 0}};
    int nt = 0;
    if (l1 == 0 && l2 == 0) {
        slot[0] = 0; P[0] = 1.0; nt = 1;
    } else if (l1 == 0 && l2 == 1) {
        int c = p_axis(m2);
        slot[0] = 1; P[0] = u[c]; gu[0][c] = 1.0; nt = 1;
    } else if (l1 == 1 && l2 == 0) {
        int c = p_axis(m1);
        slot[0] = 2; P[0] = u[c]; gu[0][c] = 1.0; nt = 1;
    } else {
        int c1 = p_axis(m1), c2 = p_axis(m2);
        if (c1 == c2) {
            int o0 = (c1 + 1) % 3, o1 = (c1 + 2) % 3;
            if (o0 > o1) { int tmp = o0; o0 = o1; o1 = tmp; }
            slot[0] = 3; P[0] = u[o0] * u[o0] + u[o1] * u[o1];
            gu[0][o0] = 2.0 * u[o0]; gu[0][o1] = 2.0 * u[o1];
            slot[1] = 4; P[1] = u[c1] * u[c1]; gu[1][c1] = 2.0 * u[c1];
        } else {
            double p = u[c1] * u[c2];
            slot[0] = 3; P[0] = -p; gu[0][c1] = -u[c2]; gu[0][c2] = -u[c1];
            slot[1] = 4; P[1] = p; gu[1][c1] = u[c2]; gu[1][c2] = u[c1];
        }
        nt = 2;
    }
    val = 0.0;
    g[0] = g[1] = g[2] = 0.0;
    for (int t = 0; t < nt; ++t) {
        double V = v[slot[t]], dV = dv[slot[t]];
        val += P[t] * V;
        double gdotu = gu[t][0] * u[0] + gu[t][1] * u[1] + gu[t][2] * u[2];
        for (int c = 0; c < 3; ++c) g[c] += (gu[t][c] - gdotu * u[c]) * V / r + P[t] * dV * u[c];
    }
}

// Value of one SK matrix element (the value part of sk_element).
TINCR_HD double sk_value(int l1, int m1, int l2, int m2, const double u[3], const double v[SK_SLOTS]) {
    if (l1 == 0 && l2 == 0) return v[0];
    if (l1 == 0) return u[p_axis(m2)] * v[1];
    if (l2 == 0) return u[p_axis(m1)] * v[2];
    const int c1 = p_axis(m1), c2 = p_axis(m2);
    if (c1 == c2) {
        const int o0 = c1 == 0 ? 1 : 0, o1 = c1 == 2 ? 1 : 2;   // the other two axes, ascending
        return (u[o0] * u[o0] + u[o1] * u[o1]) * v[3] + u[c1] * u[c1] * v[4];
    }
    return u[c1] * u[c2] * (-v[3] + v[4]);
}

// d gamma / d r for the Gaussian gamma function, C = 1/sqrt(2 (sA^2 + sB^2 + R_lr^2 / 2))
// (src/scc/gamma_approximation.rs:126-137).  Uses CUDA's erf and exp.
TINCR_HD double gamma_deriv(double r, double c) {
    const double two_over_sqrt_pi = 1.1283791670955126;   // 2 / sqrt(pi)
    return two_over_sqrt_pi * c * exp(-(c * r) * (c * r)) / r - erf(c * r) / (r * r);
}

}  // namespace tincr
