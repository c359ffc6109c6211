// Analytic ground-state and TDA excited-state gradients on the GPU (adjoint form).
//
// tincr contracts dense derivative tensors dS/dR, dH0/dR, dgamma_AO/dR, dgamma_lr_AO/dR and the
// Fock-derivative tensors f_v[V] / f_lr[V] ([3N, n, n] each; src/gradients/excited_state.rs:259-487,
// ground_state.rs:12-137, helpers.rs:47-188) with densities.  Every one of those terms is linear in
// the four derivative tensors, so the whole gradient is
//     grad[c] = <dS[c], PS> + <dH0[c], PH> + <dgamma_AO[c], QG> + <dgamma_lr_AO[c], QL>  (+ repulsion)
// for four dense n x n "adjoint" matrices built once with a few n^3 GEMMs:
//     <f_v[V][c], Y>  = 1/4 (<dS[c], Pv(V,Y)> + <dgamma[c], Qv(V,Y)>)
//     <f_lr[V][c], Y> = 1/4 (<dS[c], Plr(V,Y)> + <dgamma_lr[c], Qlr(V,Y)>)
// (formulas at plr_adjoint / pv_adjoint below).  dS/dR and dH0/dR are non-zero only in the rows and
// columns of the moving atom, and dgamma_AO only on atom-pair blocks, so the contraction is one
// pairwise-atom kernel that evaluates the Slater-Koster and gamma derivatives on the fly from the
// spline tables: O(N^2) work instead of O(N n^2) storage and O(N n^3) flops.
//
// The H-type contractions (Hav, H+) and the Z-vector operator are AO-direct (Ctx::ao_contract).
#include <algorithm>
#include <cmath>
#include <vector>

#include "ops.cuh"
#include "sk_math.cuh"
#include "tda.cuh"

namespace tincr {

// ----------------------------------------------------------------------------------------------
// elementwise and reduction kernels
// ----------------------------------------------------------------------------------------------

#define GRID_STRIDE(t, total) \
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < (total); t += (long long)gridDim.x * blockDim.x)

// out = a*A + b*B + c*C (any of B, C may be null)
__global__ void axpby3_kernel(long long len, double a, const double *A, double b, const double *B, double c,
                              const double *Cm, double *out) {
    GRID_STRIDE(t, len) {
        double v = a * A[t];
        if (B) v += b * B[t];
        if (Cm) v += c * Cm[t];
        out[t] = v;
    }
}

// out[i][j] = A[i][j] * col[j] (col scaling) or row[i] * A[i][j]
__global__ void scale_rc_kernel(int rows, int cols, const double *A, const double *row, const double *col, double *out) {
    GRID_STRIDE(t, (long long)rows * cols) {
        int i = int(t / cols), j = int(t % cols);
        double v = A[t];
        if (row) v *= row[i];
        if (col) v *= col[j];
        out[t] = v;
    }
}

// out[a][b] = G[a][b] * (trans ? A[b][a] : A[a][b])
__global__ void hadamard_kernel(int n, const double *G, const double *A, int trans, double *out) {
    GRID_STRIDE(t, (long long)n * n) {
        int a = int(t / n), b = int(t % n);
        out[t] = G[t] * (trans ? A[(long long)b * n + a] : A[t]);
    }
}

// sym[a][b] = P[a][b] + P[b][a]
__global__ void symmetrize_kernel(int n, const double *P, double *sym) {
    GRID_STRIDE(t, (long long)n * n) {
        int a = int(t / n), b = int(t % n);
        sym[t] = P[t] + P[(long long)b * n + a];
    }
}

// right-hand side of the Z-vector equation: R[i][a] = q_ai[a][i] - q_ia[i][a]
__global__ void zrhs_kernel(int o, int v, const double *qai, const double *qia, double *R) {
    GRID_STRIDE(t, (long long)o * v) {
        int i = int(t / v), a = int(t % v);
        R[t] = qai[(long long)a * o + i] - qia[t];
    }
}

// out = X / (e_a - e_i)
__global__ void zguess_kernel(long long ov, const double *R, const double *omega, double *out) {
    GRID_STRIDE(t, ov) out[t] = R[t] / omega[t];
}

// upper-triangular W of the excited gradient (excited_state.rs:352-388, into_triangular(Upper)):
//   W_ij = q_ij + H[Z]_ij (diag halved), W_ia = q_ai^T + e_i Z_ia, W_ab = q_ab (diag halved), W_ai dropped
__global__ void w_assemble_kernel(int o, int v, const double *wij, const double *qai, const double *Z,
                                  const double *eo, const double *qab, double *W) {
    int m = o + v;
    GRID_STRIDE(t, (long long)m * m) {
        int p = int(t / m), q = int(t % m);
        double val = 0.0;
        if (q >= p) {
            if (q < o) {
                val = wij[(long long)p * o + q];
                if (p == q) val *= 0.5;
            } else if (p < o) {
                int a = q - o;
                val = qai[(long long)a * o + p] + eo[p] * Z[(long long)p * v + a];
            } else {
                int a = p - o, b = q - o;
                val = qab[(long long)a * v + b];
                if (a == b) val *= 0.5;
            }
        }
        W[t] = val;
    }
}

// sv[b] = sum_a S[a][b] (V[a][b] + V[b][a]),  r[a] = sum_b S[a][b] (Y[a][b] + Y[b][a])  (S symmetric)
__global__ void fv_vectors_kernel(int n, const double *S, const double *V, const double *Y, double *sv, double *r) {
    GRID_STRIDE(t, 2LL * n) {
        int k = int(t % n);
        const double *s = S + (long long)k * n;
        double acc = 0.0;
        if (t < n) {
            for (int a = 0; a < n; ++a) acc += s[a] * (V[(long long)a * n + k] + V[(long long)k * n + a]);
            sv[k] = acc;
        } else {
            for (int b = 0; b < n; ++b) acc += s[b] * (Y[(long long)k * n + b] + Y[(long long)b * n + k]);
            r[k] = acc;
        }
    }
}

// per-atom sums of an AO vector and their gamma products:  out_ao[mu] = sum_B g[A(mu)][B] sum_{nu in B} x[nu]
__global__ void atom_gamma_kernel(int n, int n_atoms, const int *ao_off, const int *ao_atom, const double *g,
                                  const double *x1, const double *x2, double *xa1, double *xa2, double *gx1,
                                  double *gx2) {
    extern __shared__ double sh[];
    double *s1 = sh, *s2 = sh + n_atoms;
    for (int A = threadIdx.x; A < n_atoms; A += blockDim.x) {
        double a1 = 0.0, a2 = 0.0;
        for (int mu = ao_off[A]; mu < ao_off[A + 1]; ++mu) {
            a1 += x1[mu];
            a2 += x2[mu];
        }
        s1[A] = a1;
        s2[A] = a2;
        xa1[A] = a1;
        xa2[A] = a2;
    }
    __syncthreads();
    for (int mu = threadIdx.x; mu < n; mu += blockDim.x) {
        const double *gr = g + (long long)ao_atom[mu] * n_atoms;
        double a1 = 0.0, a2 = 0.0;
        for (int B = 0; B < n_atoms; ++B) {
            a1 += gr[B] * s1[B];
            a2 += gr[B] * s2[B];
        }
        gx1[mu] = a1;
        gx2[mu] = a2;
    }
}

// PS[a][b] += scale ((gsv_a + gsv_b) Y_ab + (V_ab + V_ba) gr_b)     (Pv adjoint of f_v)
// QG[A][B] += scale rA_A svA_B                                         (Qv = r sv^T, atom blocks)
__global__ void pv_accumulate_kernel(int n, int n_atoms, double scale, const double *V, const double *Y,
                                     const double *gsv, const double *gr, double *PS) {
    GRID_STRIDE(t, (long long)n * n) {
        int a = int(t / n), b = int(t % n);
        PS[t] += scale * ((gsv[a] + gsv[b]) * Y[t] + (V[t] + V[(long long)b * n + a]) * gr[b]);
    }
}

__global__ void outer_accumulate_kernel(int n_atoms, double scale, const double *x, const double *y, double *Q) {
    GRID_STRIDE(t, (long long)n_atoms * n_atoms) {
        int A = int(t / n_atoms), B = int(t % n_atoms);
        Q[t] += scale * x[A] * y[B];
    }
}

// Qlr = (s v^T s) o Y + (s v^T) o (Y s) + (s v) o (Y^T s) + v o (s Y^T s)
__global__ void qlr_kernel(long long len, const double *svts, const double *Y, const double *svt, const double *Ys,
                           const double *sv, const double *Yts, const double *v, const double *sYts, double *Q) {
    GRID_STRIDE(t, len) Q[t] = svts[t] * Y[t] + svt[t] * Ys[t] + sv[t] * Yts[t] + v[t] * sYts[t];
}

// Qblk[A][B] += scale * sum_{a in A, b in B} Q[a][b]
__global__ void block_sum_kernel(int n, int n_atoms, const int *ao_off, const double *Q, double scale, double *Qblk) {
    GRID_STRIDE(t, (long long)n_atoms * n_atoms) {
        int A = int(t / n_atoms), B = int(t % n_atoms);
        double s = 0.0;
        for (int a = ao_off[A]; a < ao_off[A + 1]; ++a)
            for (int b = ao_off[B]; b < ao_off[B + 1]; ++b) s += Q[(long long)a * n + b];
        Qblk[t] += scale * s;
    }
}

// PS[a][b] += scale * 1/2 (esp_A(a) + esp_A(b)) P[a][b]   (ground-state Coulomb term)
__global__ void coulomb_p_kernel(int n, const int *ao_atom, const double *esp, const double *P, double scale, double *PS) {
    GRID_STRIDE(t, (long long)n * n) {
        int a = int(t / n), b = int(t % n);
        PS[t] += scale * 0.5 * (esp[ao_atom[a]] + esp[ao_atom[b]]) * P[t];
    }
}

// single-block dot product
__global__ void dot_kernel(long long len, const double *a, const double *b, double *out) {
    __shared__ double red[32];
    double s = 0.0;
    for (long long x = threadIdx.x; x < len; x += blockDim.x) s += a[x] * b[x];
    for (int off = 16; off; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        for (int off = 16; off; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
        if (threadIdx.x == 0) *out = s;
    }
}

// x += alpha p ; r -= alpha Ap
__global__ void cg_update_kernel(long long len, double alpha, const double *p, const double *Ap, double *x, double *r) {
    GRID_STRIDE(t, len) {
        x[t] += alpha * p[t];
        r[t] -= alpha * Ap[t];
    }
}

// the same update with alpha = rr / pAp formed on the device (pAp left there by dot_kernel)
// Device-side CG state: s[0] = r.r (r.z when preconditioned), s[1] = p.Ap, s[2] = the new r.r,
// s[3] = beta, s[4] = the new r.z; flag[0] = 0 while running, 1 once converged, 2 on a non-finite
// step; flag[1] = iterations done.  Every thread forms alpha from the same two values, so all take
// the same decision.

// x += alpha p ; r -= alpha Ap, alpha = r.r / p.Ap (skipped once the recursion has stopped)
__global__ void cg_update_dev_kernel(long long len, const double *s, const int *flag, const double *p,
                                     const double *Ap, double *x, double *r) {
    if (flag[0] != 0) return;
    const double alpha = s[0] / s[1];
    if (!isfinite(alpha)) return;   // cg_check_kernel records it
    GRID_STRIDE(t, len) {
        x[t] += alpha * p[t];
        r[t] -= alpha * Ap[t];
    }
}

// the convergence test of helpers.rs:1146-1223 (r.r <= conv) and the next beta
__global__ void cg_check_kernel(double *s, int *flag, double conv, int precond) {
    if (flag[0] != 0) return;
    flag[1] += 1;
    if (!isfinite(s[0] / s[1])) {
        flag[0] = 2;
    } else if (s[2] <= conv) {
        flag[0] = 1;
    } else {
        const double next = precond ? s[4] : s[2];
        s[3] = next / s[0];
        s[0] = next;
    }
}

// p = beta p + r (skipped once the recursion has stopped)
__global__ void cg_dir_kernel(long long len, const double *s, const int *flag, double *p, const double *r) {
    if (flag[0] != 0) return;
    const double beta = s[3];
    GRID_STRIDE(t, len) p[t] = beta * p[t] + r[t];
}

// batched transpose of k matrices rows x cols
__global__ void transpose_batched_kernel(int k, int rows, int cols, const double *in, double *out) {
    GRID_STRIDE(t, (long long)k * rows * cols) {
        long long per = (long long)rows * cols;
        int b = int(t / per);
        long long e = t % per;
        int r = int(e / cols), c = int(e % cols);
        out[b * per + (long long)c * rows + r] = in[t];
    }
}

// ----------------------------------------------------------------------------------------------
// pairwise-atom gradient kernel
// ----------------------------------------------------------------------------------------------

struct PairArgs {
    int n_atoms, n_orb, n_kinds, n_knots;
    const double *xyz;
    const int *kind, *ao_off;
    const int *kind_norb, *kind_l, *kind_m;      // [n_kinds], [n_kinds*4], [n_kinds*4]
    const int *kind_z;
    const double *sigma;                         // per kind: 1 / (U sqrt(pi))
    const double *knots, *coef;                  // SK splines: coef[((a*nk+b)*2+sh)*5+slot][n_knots]
    const double *Ssym, *Hsym;                   // n x n symmetrised adjoints (may be null)
    const double *QG, *QL;                       // N x N symmetrised atom-block adjoints (may be null)
    double r_lr;
    int orientation;                             // 0: tincr's (centre 1 by Z, then by the moving atom), 1: by index
    int sk_extrapolate;                          // SK splines beyond the grid: boundary polynomial (1) or zero (0)
    // repulsion (ground state only)
    int rep_ntmax;
    const int *rep_nt;
    const double *rep_knots, *rep_coef, *rep_dmax;
    double *grad;                                // [3N] (written)
};

__global__ void __launch_bounds__(128) pair_gradient_kernel(PairArgs a) {
    const int i = blockIdx.x;
    const double xi = a.xyz[3 * i], yi = a.xyz[3 * i + 1], zi = a.xyz[3 * i + 2];
    const int ki = a.kind[i];
    double g0 = 0.0, g1 = 0.0, g2 = 0.0;
    for (int j = threadIdx.x; j < a.n_atoms; j += blockDim.x) {
        if (j == i) continue;
        const int kj = a.kind[j];
        double dx = a.xyz[3 * j] - xi, dy = a.xyz[3 * j + 1] - yi, dz = a.xyz[3 * j + 2] - zi;
        double r = sqrt(dx * dx + dy * dy + dz * dz);
        double e[3] = {-dx / r, -dy / r, -dz / r};   // (R_i - R_j) / r
        // ---- Slater-Koster terms (src/scc/h0_and_s.rs:196-300) ----
        if ((a.Ssym || a.Hsym) && r < 30.0) {
            int zi_ = a.kind_z[ki], zj_ = a.kind_z[kj];
            bool c1_is_i = zi_ < zj_ || (zi_ == zj_ && (a.orientation == 0 || i < j));
            int c1 = c1_is_i ? i : j, c2 = c1_is_i ? j : i;
            int k1 = a.kind[c1], k2 = a.kind[c2];
            double rv[3] = {a.xyz[3 * c2] - a.xyz[3 * c1], a.xyz[3 * c2 + 1] - a.xyz[3 * c1 + 1],
                            a.xyz[3 * c2 + 2] - a.xyz[3 * c1 + 2]};
            double u[3] = {rv[0] / r, rv[1] / r, rv[2] / r};
            int l;
            double N3[4], N2[3];
            double vS[SK_SLOTS] = {0, 0, 0, 0, 0}, dS[SK_SLOTS] = {0, 0, 0, 0, 0};
            double vH[SK_SLOTS] = {0, 0, 0, 0, 0}, dH[SK_SLOTS] = {0, 0, 0, 0, 0};
            if (bspline3_basis(a.knots, a.n_knots, r, l, N3, N2, a.sk_extrapolate != 0)) {
                const double *cS = a.coef + (long long)((k1 * a.n_kinds + k2) * 2 + 0) * SK_SLOTS * a.n_knots;
                const double *cH = a.coef + (long long)((k1 * a.n_kinds + k2) * 2 + 1) * SK_SLOTS * a.n_knots;
                for (int s = 0; s < SK_SLOTS; ++s) {
                    bspline3_eval(a.knots, cS + (long long)s * a.n_knots, l, N3, N2, vS[s], dS[s]);
                    bspline3_eval(a.knots, cH + (long long)s * a.n_knots, l, N3, N2, vH[s], dH[s]);
                }
            }
            // d/dR_i = -d/dr when i is centre 1 (r = R_j - R_i), +d/dr otherwise
            double sgn = c1_is_i ? -1.0 : 1.0;
            int n1 = a.kind_norb[k1], n2 = a.kind_norb[k2];
            int off1 = a.ao_off[c1], off2 = a.ao_off[c2];
            for (int p = 0; p < n1; ++p) {
                int lp = a.kind_l[k1 * 4 + p], mp = a.kind_m[k1 * 4 + p];
                for (int q = 0; q < n2; ++q) {
                    int lq = a.kind_l[k2 * 4 + q], mq = a.kind_m[k2 * 4 + q];
                    long long idx = (long long)(off1 + p) * a.n_orb + (off2 + q);
                    double val, gr[3];
                    if (a.Ssym) {
                        sk_element(lp, mp, lq, mq, u, r, vS, dS, val, gr);
                        double w = sgn * a.Ssym[idx];
                        g0 += w * gr[0]; g1 += w * gr[1]; g2 += w * gr[2];
                    }
                    if (a.Hsym) {
                        sk_element(lp, mp, lq, mq, u, r, vH, dH, val, gr);
                        double w = sgn * a.Hsym[idx];
                        g0 += w * gr[0]; g1 += w * gr[1]; g2 += w * gr[2];
                    }
                }
            }
        }
        // ---- gamma terms (gamma_approximation.rs:256-282, :392-423) ----
        if (a.QG || a.QL) {
            double si = a.sigma[ki], sj = a.sigma[kj];
            double w = 0.0;
            if (a.QG) {
                double c = 1.0 / sqrt(2.0 * (si * si + sj * sj));
                w += gamma_deriv(r, c) * a.QG[(long long)i * a.n_atoms + j];
            }
            if (a.QL) {
                double c = 1.0 / sqrt(2.0 * (si * si + sj * sj + 0.5 * a.r_lr * a.r_lr));
                w += gamma_deriv(r, c) * a.QL[(long long)i * a.n_atoms + j];
            }
            g0 += w * e[0]; g1 += w * e[1]; g2 += w * e[2];
        }
        // ---- repulsion (gradients/helpers.rs:843-868) ----
        if (a.rep_nt) {
            int pk = ki * a.n_kinds + kj;
            if (r <= a.rep_dmax[pk]) {
                int l;
                double N3[4], N2[3], v, d = 0.0;
                const double *t = a.rep_knots + (long long)pk * a.rep_ntmax;
                if (bspline3_basis(t, a.rep_nt[pk], r, l, N3, N2))
                    bspline3_eval(t, a.rep_coef + (long long)pk * a.rep_ntmax, l, N3, N2, v, d);
                g0 += d * e[0]; g1 += d * e[1]; g2 += d * e[2];
            }
        }
    }
    __shared__ double red[3][4];
    for (int off = 16; off; off >>= 1) {
        g0 += __shfl_down_sync(0xffffffffu, g0, off);
        g1 += __shfl_down_sync(0xffffffffu, g1, off);
        g2 += __shfl_down_sync(0xffffffffu, g2, off);
    }
    int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) { red[0][w] = g0; red[1][w] = g1; red[2][w] = g2; }
    __syncthreads();
    if (threadIdx.x < 3) {
        double s = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[threadIdx.x][k];
        a.grad[3 * i + threadIdx.x] = s;
    }
}

// ----------------------------------------------------------------------------------------------
// host side
// ----------------------------------------------------------------------------------------------

static int gridn(long long work, int n_sm) {
    long long b = (work + 255) / 256;
    return int(std::max<long long>(1, std::min<long long>(b, 32LL * n_sm)));
}

#define EW(kernel, work, ...)                                                      \
    do {                                                                           \
        kernel<<<gridn((work), n_sm), 256, 0, stream>>>(__VA_ARGS__);              \
        count_launch(stream, #kernel);                                             \
        check_launch(#kernel);                                                     \
    } while (0)

void Ctx::set_parameters(int n_kinds_, const int *kind_z, const int *kind_norb, const int *kind_l, const int *kind_m,
                         const double *kind_hubbard, const double *kind_occ, int n_knots_, const double *knots,
                         const double *coef, int rep_ntmax_, const int *rep_nt, const double *rep_knots,
                         const double *rep_coef, const double *rep_dmax) {
    if (n_kinds_ <= 0 || n_knots_ < 8 || !kind_z || !kind_norb || !kind_l || !kind_m || !kind_hubbard || !kind_occ ||
        !knots || !coef)
        fail(TINCR_BAD_ARG, "set_parameters: bad arguments");
    for (int k = 0; k < n_kinds_; ++k)
        if (kind_norb[k] < 1 || kind_norb[k] > 4) fail(TINCR_BAD_ARG, "set_parameters: only s and p shells");
    n_kinds = n_kinds_;
    n_knots = n_knots_;
    h_kind_z.assign(kind_z, kind_z + n_kinds);
    h_kind_norb.assign(kind_norb, kind_norb + n_kinds);
    h_kind_occ.assign(kind_occ, kind_occ + 4 * n_kinds);
    std::vector<double> sig(n_kinds);
    for (int k = 0; k < n_kinds; ++k) sig[k] = 1.0 / (kind_hubbard[k] * 1.7724538509055159);
    auto up = [&](auto &d, const auto *h, size_t cnt) {
        d.alloc(cnt);
        TINCR_CUDA(cudaMemcpyAsync(d.p, h, cnt * sizeof(*h), cudaMemcpyHostToDevice, stream));
    };
    up(d_kind_z, kind_z, n_kinds);
    up(d_kind_norb, kind_norb, n_kinds);
    up(d_kind_l, kind_l, 4 * (size_t)n_kinds);
    up(d_kind_m, kind_m, 4 * (size_t)n_kinds);
    up(d_sigma, sig.data(), n_kinds);
    up(d_knots, knots, n_knots);
    up(d_coef, coef, (size_t)n_kinds * n_kinds * 2 * SK_SLOTS * n_knots);
    rep_ntmax = 0;
    if (rep_nt && rep_knots && rep_coef && rep_dmax && rep_ntmax_ > 0) {
        rep_ntmax = rep_ntmax_;
        up(d_rep_nt, rep_nt, (size_t)n_kinds * n_kinds);
        up(d_rep_knots, rep_knots, (size_t)n_kinds * n_kinds * rep_ntmax);
        up(d_rep_coef, rep_coef, (size_t)n_kinds * n_kinds * rep_ntmax);
        up(d_rep_dmax, rep_dmax, (size_t)n_kinds * n_kinds);
    }
    sync();
    params_ready = true;
}

// PS += scale_p * Plr(v, Y);  QLblk += scale_q * blocks(Qlr(v, Y))      (gamma = gamma_lr_AO)
//   Plr = (g o Y) s v + (g o (Y s)) v + Y ((s v) o g) + Y s (g o v) + v s (g o Y) + ((v s) o g) Y
//         + (g o (Y^T s)) v^T + Y^T s (g o v^T)
//   Qlr = (s v^T s) o Y + (s v^T) o (Y s) + (s v) o (Y^T s) + v o (s Y^T s)
// so that <f_lr[v][c], Y> = 1/4 (<dS[c], Plr> + <dgamma_lr_AO[c], Qlr>)  (helpers.rs:130-188).
void Ctx::plr_adjoint(const double *v, const double *Y, double scale_p, double scale_q, double *PS, double *QLblk) {
    const int n = n_orb;
    const size_t nn = (size_t)n * n;
    gw.reserve(14 * nn);
    double *sv = gw.p, *Ys = sv + nn, *vs = Ys + nn, *Yts = vs + nn, *svt = Yts + nn, *svts = svt + nn, *sYt = svts + nn,
           *sYts = sYt + nn, *h1 = sYts + nn, *h2 = h1 + nn, *Q = h2 + nn;
    const double *s = dS_.p, *g = d_glr_ao.p;
    auto mm = [&](bool ta, bool tb, const double *A, const double *B, double *C, double alpha, double beta) {
        if (prec == TINCR_PREC_BF16X3) {   // mixed form: the dense adjoint contractions on the tensor cores
            gemm_mixed(ta, tb, n, n, n, A, n, B, n, C, n, alpha, beta);
            return;
        }
        int slot = prof_begin(TINCR_KF_GRADIENT);
        EpiStore e{C, 0, n, alpha, beta};
        if (!ta && !tb) gemm_f64<false, false>(stream, n, n, n, A, n, 0, B, n, 0, 1, e);
        else if (ta && !tb) gemm_f64<true, false>(stream, n, n, n, A, n, 0, B, n, 0, 1, e);
        else if (!ta && tb) gemm_f64<false, true>(stream, n, n, n, A, n, 0, B, n, 0, 1, e);
        else gemm_f64<true, true>(stream, n, n, n, A, n, 0, B, n, 0, 1, e);
        prof_end(slot, 2.0 * n * (double)n * n, 24.0 * nn);
    };
    mm(false, false, s, v, sv, 1.0, 0.0);        // s v
    mm(false, false, Y, s, Ys, 1.0, 0.0);        // Y s
    mm(false, false, v, s, vs, 1.0, 0.0);        // v s
    mm(true, false, Y, s, Yts, 1.0, 0.0);        // Y^T s
    mm(false, true, s, v, svt, 1.0, 0.0);        // s v^T
    mm(false, false, svt, s, svts, 1.0, 0.0);    // s v^T s
    mm(false, true, s, Y, sYt, 1.0, 0.0);        // s Y^T
    mm(false, false, sYt, s, sYts, 1.0, 0.0);    // s Y^T s
    // P terms accumulate into PS with factor scale_p
    EW(hadamard_kernel, nn, n, g, Y, 0, h1);                 // g o Y
    mm(false, false, h1, sv, PS, scale_p, 1.0);              // (g o Y) s v
    mm(false, false, vs, h1, PS, scale_p, 1.0);              // v s (g o Y)
    EW(hadamard_kernel, nn, n, g, Ys, 0, h2);                // g o (Y s)
    mm(false, false, h2, v, PS, scale_p, 1.0);               // (g o (Y s)) v
    EW(hadamard_kernel, nn, n, g, sv, 0, h2);                // (s v) o g
    mm(false, false, Y, h2, PS, scale_p, 1.0);               // Y ((s v) o g)
    EW(hadamard_kernel, nn, n, g, v, 0, h2);                 // g o v
    mm(false, false, Ys, h2, PS, scale_p, 1.0);              // Y s (g o v)
    EW(hadamard_kernel, nn, n, g, vs, 0, h2);                // (v s) o g
    mm(false, false, h2, Y, PS, scale_p, 1.0);               // ((v s) o g) Y
    EW(hadamard_kernel, nn, n, g, Yts, 0, h2);               // g o (Y^T s)
    mm(false, true, h2, v, PS, scale_p, 1.0);                // (g o (Y^T s)) v^T
    EW(hadamard_kernel, nn, n, g, v, 1, h2);                 // g o v^T
    mm(false, false, Yts, h2, PS, scale_p, 1.0);             // Y^T s (g o v^T)
    // Q
    EW(qlr_kernel, nn, (long long)nn, svts, Y, svt, Ys, sv, Yts, v, sYts, Q);
    EW(block_sum_kernel, (long long)n_atoms * n_atoms, n, n_atoms, d_ao_off.p, Q, scale_q, QLblk);
}

// PS += scale * Pv(V, Y);  QGblk += scale * blocks(r sv^T)   (gamma = gamma_AO), with
//   Pv = (gsv_a + gsv_b) Y_ab + (V + V^T)_ab (gamma r)_b,  sv = colsum(S o (V + V^T)), r = rowsum(S o (Y + Y^T))
// so that <f_v[V][c], Y> = 1/4 (<dS[c], Pv> + <dgamma_AO[c], r sv^T>)  (helpers.rs:47-80).
void Ctx::pv_adjoint(const double *V, const double *Y, double scale, double *PS, double *QGblk) {
    const int n = n_orb;
    gv.reserve(4 * (size_t)n + 2 * (size_t)n_atoms);
    double *sv = gv.p, *r = sv + n, *gsv = r + n, *gr = gsv + n, *svA = gr + n, *rA = svA + n_atoms;
    EW(fv_vectors_kernel, 2LL * n, n, dS_.p, V, Y, sv, r);
    atom_gamma_kernel<<<1, 256, 2 * n_atoms * sizeof(double), stream>>>(n, n_atoms, d_ao_off.p, d_ao_atom.p, d_gamma.p,
                                                                         sv, r, svA, rA, gsv, gr);
    count_launch(stream, "atom_gamma");
    check_launch("atom_gamma");
    EW(pv_accumulate_kernel, (long long)n * n, n, n_atoms, scale, V, Y, gsv, gr, PS);
    // blocks of (r sv^T): sum_{a in A} r_a * sum_{b in B} sv_b
    EW(outer_accumulate_kernel, (long long)n_atoms * n_atoms, n_atoms, scale, rA, svA, QGblk);
}

// CG on (operator) Z = R  (helpers.rs:1130-1223): x0 = R / omega, stop when r.r <= conv.
int Ctx::zvector_cg(int variant, const double *R, double *Z, int max_iter, double conv, int *iters) {
    const long long len = ov;
    gcg.reserve(5 * (size_t)len + 8);
    double *r = gcg.p, *p = r + len, *Ap = p + len, *tmp = Ap + len, *Xt = tmp + len, *dots = Xt + len;
    int h_flag[2] = {0, 0};
    auto op = [&](const double *x, double *out) {
        // tincr: TDA matrix A for LC (mult_av_lc: 2 Coulomb - exchange), A+B without exchange otherwise
        // (mult_av_nolc: 4 Coulomb).  Exact variant with LC: (A+B) = 4 Coulomb - (ij|ab) - (ib|ja).
        double ac = (lc && variant == TINCR_GRAD_REFERENCE) ? 1.0 : 2.0;
        ao_contract(1, BLK_OCC, BLK_VIRT, x, BLK_OCC, BLK_VIRT, lc ? -0.25 : 0.0, ac, out, 1.0, 0.0, x);
        if (lc && variant == TINCR_GRAD_EXACT) {
            EW(transpose_batched_kernel, len, 1, n_occ, n_virt, x, Xt);
            ao_contract(1, BLK_VIRT, BLK_OCC, Xt, BLK_OCC, BLK_VIRT, -0.25, 0.0, out, 1.0, 1.0, nullptr);
        }
    };
    auto dot_dev = [&](const double *a, const double *b, double *out) {   // out on the device, no sync
        dot_kernel<<<1, 1024, 0, stream>>>(len, a, b, out);
        count_launch(stream, "dot");
        check_launch("dot");
    };
    EW(zguess_kernel, len, len, R, d_omega.p, Z);          // bs = R / omega
    int *flag = reinterpret_cast<int *>(dots + 6);
    // CG from the current Z (tincr: helpers.rs:1146-1223); the convergence test is FP64 on r.r.  The
    // recursion runs on the device (alpha, beta and the test in device scalars); the host reads
    // the flag every CG_SYNC iterations, and the iterations queued after convergence change nothing.
    // The mixed form preconditions with diag(omega), the dominant part of the operator's diagonal
    // (tincr's CG is unpreconditioned): the same stopping rule on the same residual, so Z agrees to
    // that tolerance, in fewer iterations.  The FP64 form keeps tincr's recursion.
    constexpr int CG_SYNC = 4;
    double *zr = tmp;   // preconditioned residual
    auto run = [&](int limit, int *done) {
        const bool pre = prec == TINCR_PREC_BF16X3;
        const double *dir = pre ? zr : r;
        op(Z, Ap);
        EW(axpby3_kernel, len, len, 1.0, R, -1.0, Ap, 0.0, nullptr, r);   // r = R - A Z
        if (pre) EW(zguess_kernel, len, len, r, d_omega.p, zr);
        TINCR_CUDA(cudaMemcpyAsync(p, dir, len * sizeof(double), cudaMemcpyDeviceToDevice, stream));
        dot_dev(r, dir, dots);
        TINCR_CUDA(cudaMemsetAsync(flag, 0, 2 * sizeof(int), stream));
        int queued = 0;
        while (queued < limit) {
            const int batch = std::min(CG_SYNC, limit - queued);
            for (int q = 0; q < batch; ++q) {
                op(p, Ap);
                dot_dev(p, Ap, dots + 1);
                EW(cg_update_dev_kernel, len, len, dots, flag, p, Ap, Z, r);
                dot_dev(r, r, dots + 2);
                if (pre) {
                    EW(zguess_kernel, len, len, r, d_omega.p, zr);
                    dot_dev(r, zr, dots + 4);
                }
                cg_check_kernel<<<1, 1, 0, stream>>>(dots, flag, conv, pre ? 1 : 0);
                count_launch(stream, "cg_check");
                check_launch("cg_check");
                EW(cg_dir_kernel, len, len, dots, flag, p, dir);
            }
            queued += batch;
            TINCR_CUDA(cudaMemcpyAsync(h_flag, flag, 2 * sizeof(int), cudaMemcpyDeviceToHost, stream));
            sync();
            if (h_flag[0] == 2) fail(TINCR_NONFINITE, "Z-vector CG: non-finite step");
            if (h_flag[0] == 1) break;
        }
        *done = h_flag[1];
        return h_flag[0] == 1 ? TINCR_OK : TINCR_CG_MAXITER;
    };
    int it = 0, status;
    if (prec == TINCR_PREC_BF16X3) {
        // mixed products; if the recursion stalls on the mixed operator, FP64 CG continues from Z
        status = run(std::min(max_iter, 200), &it);
        if (status != TINCR_OK) {
            prec = TINCR_PREC_FP64;
            int it2 = 0;
            status = run(std::max(1, max_iter - it), &it2);
            it += it2;
            prec = TINCR_PREC_BF16X3;
        }
    } else {
        status = run(max_iter, &it);
    }
    if (iters) *iters = it;
    return status;
}

int Ctx::gradient(const int *atom_kind, double r_lr_, const double *P, const double *h_coul_x, const double *dq,
                  int state, int variant, double *grad_gs, double *grad_exc, int *cg_iters) {
    if (!ready) fail(TINCR_BAD_ARG, "gradient: tincr_tda_setup first");
    if (!params_ready) fail(TINCR_BAD_ARG, "gradient: tincr_set_parameters first");
    if (!atom_kind || !P || !dq) fail(TINCR_BAD_ARG, "gradient: null input");
    if (grad_exc && (state < 0 || state >= solved_roots)) fail(TINCR_BAD_ARG, "gradient: state not solved");
    if (grad_gs && !h_coul_x) fail(TINCR_BAD_ARG, "gradient: h_coul_x needed for the ground-state gradient");
    const bool sk_extrapolate = (variant & TINCR_GRAD_SK_EXTRAPOLATE) != 0;
    variant &= ~TINCR_GRAD_SK_EXTRAPOLATE;
    if (variant != TINCR_GRAD_REFERENCE && variant != TINCR_GRAD_EXACT) fail(TINCR_BAD_ARG, "gradient: variant");
    for (int A = 0; A < n_atoms; ++A) {
        int k = atom_kind[A];
        if (k < 0 || k >= n_kinds) fail(TINCR_BAD_ARG, "gradient: atom kind out of range");
        if (h_kind_norb[k] != h_ao_off[A + 1] - h_ao_off[A]) fail(TINCR_BAD_ARG, "gradient: kind/orbital mismatch");
    }
    const int n = n_orb, o = n_occ, v = n_virt, N = n_atoms;
    const size_t nn = (size_t)n * n;
    g_launches = 0;
    prec = solve_prec;   // the contractions follow the precision the roots were solved with
    TINCR_CUDA(cudaEventRecord(ev0, stream));
    DevBuf<int> dkind(N);
    TINCR_CUDA(cudaMemcpyAsync(dkind.p, atom_kind, N * sizeof(int), cudaMemcpyHostToDevice, stream));
    // dP = P - P0
    std::vector<double> hp0(n);
    for (int A = 0; A < N; ++A)
        for (int mu = h_ao_off[A]; mu < h_ao_off[A + 1]; ++mu) hp0[mu] = h_kind_occ[4 * atom_kind[A] + (mu - h_ao_off[A])];
    DevBuf<double> dPm(nn), dDP(nn), dqd(N);
    TINCR_CUDA(cudaMemcpyAsync(dPm.p, P, nn * sizeof(double), cudaMemcpyHostToDevice, stream));
    TINCR_CUDA(cudaMemcpyAsync(dqd.p, dq, N * sizeof(double), cudaMemcpyHostToDevice, stream));
    {
        std::vector<double> dp(P, P + nn);
        for (int mu = 0; mu < n; ++mu) dp[(size_t)mu * n + mu] -= hp0[mu];
        TINCR_CUDA(cudaMemcpyAsync(dDP.p, dp.data(), nn * sizeof(double), cudaMemcpyHostToDevice, stream));
        sync();
    }
    DevBuf<double> PS(nn), PH(nn), Ssym(nn), Hsym(nn), QG((size_t)N * N), QL((size_t)N * N), QGs((size_t)N * N),
        QLs((size_t)N * N), dgrad(3 * (size_t)N);
    PairArgs pa{};
    pa.n_atoms = N; pa.n_orb = n; pa.n_kinds = n_kinds; pa.n_knots = n_knots;
    pa.xyz = d_xyz.p; pa.kind = dkind.p; pa.ao_off = d_ao_off.p;
    pa.kind_norb = d_kind_norb.p; pa.kind_l = d_kind_l.p; pa.kind_m = d_kind_m.p; pa.kind_z = d_kind_z.p;
    pa.sigma = d_sigma.p; pa.knots = d_knots.p; pa.coef = d_coef.p;
    pa.r_lr = r_lr_;
    pa.orientation = variant == TINCR_GRAD_EXACT ? 1 : 0;
    pa.sk_extrapolate = sk_extrapolate ? 1 : 0;
    auto run_pairs = [&](bool rep, double *out_host) {
        EW(symmetrize_kernel, nn, n, PS.p, Ssym.p);
        EW(symmetrize_kernel, nn, n, PH.p, Hsym.p);
        EW(symmetrize_kernel, (long long)N * N, N, QG.p, QGs.p);
        EW(symmetrize_kernel, (long long)N * N, N, QL.p, QLs.p);
        pa.Ssym = Ssym.p; pa.Hsym = Hsym.p; pa.QG = QGs.p; pa.QL = lc ? QLs.p : nullptr;
        pa.rep_nt = (rep && rep_ntmax > 0) ? d_rep_nt.p : nullptr;
        pa.rep_ntmax = rep_ntmax; pa.rep_knots = d_rep_knots.p; pa.rep_coef = d_rep_coef.p; pa.rep_dmax = d_rep_dmax.p;
        pa.grad = dgrad.p;
        int slot = prof_begin(TINCR_KF_GRADIENT);
        pair_gradient_kernel<<<N, 128, 0, stream>>>(pa);
        count_launch(stream, "pair_gradient");
        check_launch("pair_gradient");
        prof_end(slot, 0.0, 8.0 * (4.0 * nn + 4.0 * N * N));
        TINCR_CUDA(cudaMemcpyAsync(out_host, dgrad.p, 3 * (size_t)N * sizeof(double), cudaMemcpyDeviceToHost, stream));
        sync();
    };
    auto mm = [&](bool ta, bool tb, int M, int Nn, int K, const double *A, int lda, const double *B, int ldb, double *C,
                  int ldc, double alpha, double beta) {
        if (prec == TINCR_PREC_BF16X3) {
            gemm_mixed(ta, tb, M, Nn, K, A, lda, B, ldb, C, ldc, alpha, beta);
            return;
        }
        EpiStore e{C, 0, ldc, alpha, beta};
        int slot = prof_begin(TINCR_KF_GRADIENT);
        if (!ta && !tb) gemm_f64<false, false>(stream, M, Nn, K, A, lda, 0, B, ldb, 0, 1, e);
        else if (ta && !tb) gemm_f64<true, false>(stream, M, Nn, K, A, lda, 0, B, ldb, 0, 1, e);
        else if (!ta && tb) gemm_f64<false, true>(stream, M, Nn, K, A, lda, 0, B, ldb, 0, 1, e);
        else gemm_f64<true, true>(stream, M, Nn, K, A, lda, 0, B, ldb, 0, 1, e);
        prof_end(slot, 2.0 * M * (double)Nn * K, 8.0 * ((double)M * K + (double)K * Nn + (double)M * Nn));
    };

    // ---------------- ground state (ground_state.rs:12-137) ----------------
    if (grad_gs) {
        TINCR_CUDA(cudaMemsetAsync(PS.p, 0, nn * sizeof(double), stream));
        TINCR_CUDA(cudaMemsetAsync(QG.p, 0, (size_t)N * N * sizeof(double), stream));
        TINCR_CUDA(cudaMemsetAsync(QL.p, 0, (size_t)N * N * sizeof(double), stream));
        TINCR_CUDA(cudaMemcpyAsync(PH.p, dPm.p, nn * sizeof(double), cudaMemcpyDeviceToDevice, stream));  // dH0 . P
        // - dS . W with W = 1/2 P H P
        DevBuf<double> dH(nn), tmp(nn);
        TINCR_CUDA(cudaMemcpyAsync(dH.p, h_coul_x, nn * sizeof(double), cudaMemcpyHostToDevice, stream));
        mm(false, false, n, n, n, dPm.p, n, dH.p, n, tmp.p, n, 1.0, 0.0);
        mm(false, false, n, n, n, tmp.p, n, dPm.p, n, PS.p, n, -0.5, 1.0);
        // + dS . (1/2 (esp_a + esp_b) P), esp = gamma dq
        std::vector<double> hdq(dq, dq + N), hg(h_gamma), esp(N, 0.0);
        for (int A = 0; A < N; ++A)
            for (int B = 0; B < N; ++B) esp[A] += hg[(size_t)A * N + B] * hdq[B];
        DevBuf<double> desp(N);
        TINCR_CUDA(cudaMemcpyAsync(desp.p, esp.data(), N * sizeof(double), cudaMemcpyHostToDevice, stream));
        EW(coulomb_p_kernel, nn, n, d_ao_atom.p, desp.p, dPm.p, 1.0, PS.p);
        // + dq . dgamma . dq: QG = 1/2 dq dq^T so that the symmetrised block is dq_i dq_j
        EW(outer_accumulate_kernel, (long long)N * N, N, 0.5, dqd.p, dqd.p, QG.p);
        // - 1/4 <f_lr(dP), dP>
        if (lc) plr_adjoint(dDP.p, dDP.p, -0.25 * 0.25, -0.25 * 0.25, PS.p, QL.p);
        run_pairs(true, grad_gs);
    }

    // ---------------- excited state (excited_state.rs:56-487) ----------------
    if (grad_exc) {
        const double omega_state = h_energies[state];
        const double *X = dR.p + (long long)state * ov;      // [o x v]
        std::vector<double> eo(h_orbe.begin(), h_orbe.begin() + o), ev(h_orbe.begin() + o, h_orbe.begin() + o + v);
        DevBuf<double> deo(o), dev_(v);
        TINCR_CUDA(cudaMemcpyAsync(deo.p, eo.data(), o * sizeof(double), cudaMemcpyHostToDevice, stream));
        TINCR_CUDA(cudaMemcpyAsync(dev_.p, ev.data(), v * sizeof(double), cudaMemcpyHostToDevice, stream));
        const size_t oo = (size_t)o * o, vv = (size_t)v * v;
        DevBuf<double> Tij(oo), Tab(vv), Vij(oo), Vab(vv), tmpov(ov), gij(oo), qij(oo), qab(vv), hx(vv), qia(ov),
            hq(oo), qai(ov), Rz(ov), Z(ov), wz(oo), Xt(ov);
        mm(false, true, o, o, v, X, v, X, v, Tij.p, o, 1.0, 0.0);                 // X X^T
        mm(true, false, v, v, o, X, v, X, v, Tab.p, v, 1.0, 0.0);                 // X^T X
        EW(scale_rc_kernel, ov, o, v, X, nullptr, dev_.p, tmpov.p);             // X e_v
        mm(false, true, o, o, v, tmpov.p, v, X, v, Vij.p, o, 2.0, 0.0);           // 2 X e_v X^T
        EW(scale_rc_kernel, ov, o, v, X, deo.p, nullptr, tmpov.p);              // e_o X
        mm(true, false, v, v, o, tmpov.p, v, X, v, Vab.p, v, 2.0, 0.0);           // 2 X^T e_o X
        // Hav / h_a_nolr:  2 (2 Coulomb - exchange)  ->  ac = 2, ax = -1/2 (LC)
        const double hax = lc ? -0.5 : 0.0;
        ao_contract(1, BLK_VIRT, BLK_VIRT, Tab.p, BLK_OCC, BLK_OCC, hax, 2.0, gij.p, 1.0, 0.0, nullptr);
        ao_contract(1, BLK_OCC, BLK_OCC, Tij.p, BLK_OCC, BLK_OCC, hax, 2.0, gij.p, -1.0, 1.0, nullptr);
        EW(axpby3_kernel, oo, (long long)oo, 2.0 * omega_state, Tij.p, -1.0, Vij.p, 1.0, gij.p, qij.p);
        EW(axpby3_kernel, vv, (long long)vv, 2.0 * omega_state, Tab.p, 1.0, Vab.p, 0.0, nullptr, qab.p);
        ao_contract(1, BLK_OCC, BLK_VIRT, X, BLK_VIRT, BLK_VIRT, hax, 2.0, hx.p, 1.0, 0.0, nullptr);
        mm(false, true, o, v, v, X, v, hx.p, v, qia.p, v, 1.0, 0.0);               // X hx^T
        ao_contract(1, BLK_VIRT, BLK_VIRT, Tab.p, BLK_OCC, BLK_VIRT, hax, 2.0, qia.p, 1.0, 1.0, nullptr);
        ao_contract(1, BLK_OCC, BLK_OCC, Tij.p, BLK_OCC, BLK_VIRT, hax, 2.0, qia.p, -1.0, 1.0, nullptr);
        ao_contract(1, BLK_OCC, BLK_VIRT, X, BLK_OCC, BLK_OCC, hax, 2.0, hq.p, 1.0, 0.0, nullptr);
        mm(true, false, v, o, o, X, v, hq.p, o, qai.p, o, 1.0, 0.0);               // X^T hq  [v x o]
        EW(zrhs_kernel, ov, o, v, qai.p, qia.p, Rz.p);
        int cgi = 0;
        int cg_status = zvector_cg(variant, Rz.p, Z.p, 10000, 1.0e-19, &cgi);
        if (cg_iters) *cg_iters = cgi;
        last_cg_status = cg_status;
        // W_ij = q_ij + H[Z]_ij
        if (lc && variant == TINCR_GRAD_EXACT) {
            // H+[Z]: 4 Coulomb - (ij|kb) Z - (ib|jk) Z
            ao_contract(1, BLK_OCC, BLK_VIRT, Z.p, BLK_OCC, BLK_OCC, -0.25, 2.0, wz.p, 1.0, 0.0, nullptr);
            EW(transpose_batched_kernel, ov, 1, o, v, Z.p, Xt.p);
            ao_contract(1, BLK_VIRT, BLK_OCC, Xt.p, BLK_OCC, BLK_OCC, -0.25, 0.0, wz.p, 1.0, 1.0, nullptr);
        } else {
            ao_contract(1, BLK_OCC, BLK_VIRT, Z.p, BLK_OCC, BLK_OCC, hax, 2.0, wz.p, 1.0, 0.0, nullptr);
        }
        EW(axpby3_kernel, oo, (long long)oo, 1.0, qij.p, 1.0, wz.p, 0.0, nullptr, wz.p);
        const int m = o + v;
        DevBuf<double> W((size_t)m * m), CW((size_t)n * m), Wao(nn), Mao(nn), Xao(nn), t1((size_t)n * std::max(o, v));
        EW(w_assemble_kernel, (long long)m * m, o, v, wz.p, qai.p, Z.p, deo.p, qab.p, W.p);
        // W_AO = C triu(W) C^T   (C restricted to the o+v active MOs)
        mm(false, false, n, m, m, dC.p, n, W.p, m, CW.p, m, 1.0, 0.0);
        mm(false, true, n, n, m, CW.p, m, dC.p, n, Wao.p, n, 1.0, 0.0);
        // M = Cv T_ab Cv^T - Co T_ij Co^T + Co Z Cv^T
        mm(false, false, n, v, v, dC.p + o, n, Tab.p, v, t1.p, v, 1.0, 0.0);
        mm(false, true, n, n, v, t1.p, v, dC.p + o, n, Mao.p, n, 1.0, 0.0);
        mm(false, false, n, o, o, dC.p, n, Tij.p, o, t1.p, o, 1.0, 0.0);
        mm(false, true, n, n, o, t1.p, o, dC.p, n, Mao.p, n, -1.0, 1.0);
        mm(false, false, n, v, o, dC.p, n, Z.p, v, t1.p, v, 1.0, 0.0);
        mm(false, true, n, n, v, t1.p, v, dC.p + o, n, Mao.p, n, 1.0, 1.0);
        // X_AO = Co X Cv^T
        mm(false, false, n, v, o, dC.p, n, X, v, t1.p, v, 1.0, 0.0);
        mm(false, true, n, n, v, t1.p, v, dC.p + o, n, Xao.p, n, 1.0, 0.0);
        // adjoints:  dH0 . M ;  - dS . W_AO ;  f_v(dP).M ; 2 f_v(X_AO).X_AO ; LC: -1/2 f_lr(dP).M - f_lr(X_AO^T).X_AO
        TINCR_CUDA(cudaMemcpyAsync(PH.p, Mao.p, nn * sizeof(double), cudaMemcpyDeviceToDevice, stream));
        EW(axpby3_kernel, nn, (long long)nn, -1.0, Wao.p, 0.0, nullptr, 0.0, nullptr, PS.p);
        TINCR_CUDA(cudaMemsetAsync(QG.p, 0, (size_t)N * N * sizeof(double), stream));
        TINCR_CUDA(cudaMemsetAsync(QL.p, 0, (size_t)N * N * sizeof(double), stream));
        pv_adjoint(dDP.p, Mao.p, 0.25, PS.p, QG.p);
        pv_adjoint(Xao.p, Xao.p, 0.5, PS.p, QG.p);
        if (lc) {
            plr_adjoint(dDP.p, Mao.p, -0.125, -0.125, PS.p, QL.p);
            DevBuf<double> XaoT(nn);
            EW(transpose_batched_kernel, nn, 1, n, n, Xao.p, XaoT.p);
            plr_adjoint(XaoT.p, Xao.p, -0.25, -0.25, PS.p, QL.p);
        }
        run_pairs(false, grad_exc);
    }
    TINCR_CUDA(cudaEventRecord(ev1, stream));
    sync();
    float ms = 0.f;
    TINCR_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    last_ms = ms;
    last_launches = g_launches;
    prof_resolve();
    return (grad_exc && last_cg_status != TINCR_OK) ? last_cg_status : TINCR_OK;
}

}  // namespace tincr
