// RPA / Casida excited states on the GPU (FP64).
//
// tincr states the Casida problem densely (src/excited_states/casida.rs:6-80, with A and B from
// src/excited_states/a_and_b.rs:5-163, singlets, closed shell: df/2 = 1):
//     A = omega + 2 q_ov^T gamma q_ov - K,   B = 2 q_ov^T gamma q_ov - K',
//     K_{ia,jb} = (ij|ab)_lr, K'_{ia,jb} = (ib|ja)_lr (Mulliken charges, gamma_lr),
//     (A-B)^1/2 (A+B) (A-B)^1/2 F = Omega^2 F,  X+Y = (A-B)^1/2 F / sqrt(Omega),  X-Y = (A+B)(X+Y) / Omega.
// Here the lowest n_roots come from a Davidson on the pair of products (A+B) V and (A-B) V
// (Stratmann, Scuseria, Frisch, J. Chem. Phys. 109, 8218 (1998)): in the basis V the projected
// M+ = V^T (A+B) V and M- = V^T (A-B) V give the same symmetric problem
// M- M+ (X+Y) = Omega^2 (X+Y), whose solutions are Ritz pairs of the full one; the residuals
// (A+B)(X+Y) - Omega (X-Y) and (A-B)(X-Y) - Omega (X+Y) are preconditioned by (Omega - omega)^-1 and
// both added to the basis.  The products use the AO-direct contractions of the TDA (Ctx::ao_contract):
//     (A-B) V = omega o V - K[V] + K'[V],   (A+B) V = (A-B) V + 4 J[V] - 2 K'[V],
// two exchange contractions (K with V, K' with V^T) and one Coulomb contraction per block of vectors.
// The subspace problem (m <= 15 n_roots) is solved on the host: a Cholesky factor L of M-, then the
// lowest roots of L^T M+ L (eigen_host.cpp).
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "ops.cuh"
#include "tda.cuh"

namespace tincr {

namespace {

__global__ void rpa_transpose_kernel(int k, int rows, int cols, const double *__restrict__ in, double *__restrict__ out) {
    const long long len = (long long)rows * cols;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < (long long)k * len;
         t += (long long)gridDim.x * blockDim.x) {
        const long long b = t / len, e = t - b * len;
        const int r = (int)(e / cols), c = (int)(e - (long long)r * cols);
        out[b * len + (long long)c * rows + r] = in[t];
    }
}

// P += T, M -= T
__global__ void rpa_pm_kernel(long long len, const double *__restrict__ T, double *P, double *M) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < len; t += (long long)gridDim.x * blockDim.x) {
        P[t] += T[t];
        M[t] -= T[t];
    }
}

// out = omega o V (k vectors)
__global__ void rpa_omega_kernel(long long ov, int k, const double *__restrict__ omega, const double *__restrict__ V,
                                 double *out) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ov * k; t += (long long)gridDim.x * blockDim.x)
        out[t] = omega[t % ov] * V[t];
}

// T_j = R_{idx[j]} / (w_j - omega), |w_j - omega| < 1e-4 -> 1 (tincr's preconditioner, solvers/mod.rs:373-380)
__global__ void rpa_precondition_kernel(long long ov, int k, const int *__restrict__ idx, const double *__restrict__ w,
                                        const double *__restrict__ R, const double *__restrict__ omega, double *T) {
    const int j = blockIdx.y;
    const double *r = R + (long long)idx[j] * ov;
    const double wj = w[j];
    for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < ov; x += (long long)gridDim.x * blockDim.x) {
        double d = wj - omega[x];
        if (fabs(d) < 1.0e-4) d = 1.0;
        T[(long long)j * ov + x] = r[x] / d;
    }
}

__global__ void rpa_scale_copy_kernel(long long n, const double *__restrict__ in, double s, double *out) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        out[t] = s * in[t];
}

__global__ void rpa_unit_kernel(int k, long long ov, const int *__restrict__ pos, double *V) {
    for (int r = threadIdx.x; r < k; r += blockDim.x) V[(long long)r * ov + pos[r]] = 1.0;
}

int grid_of(long long work, int n_sm) {
    return (int)std::max<long long>(1, std::min<long long>((work + 255) / 256, 32LL * n_sm));
}

// C = A B (host, n x n row-major)
void host_mm(int n, const double *A, const double *B, double *C) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        double *c = C + (size_t)i * n;
        std::fill(c, c + n, 0.0);
        for (int k = 0; k < n; ++k) {
            const double a = A[(size_t)i * n + k];
            const double *b = B + (size_t)k * n;
            for (int j = 0; j < n; ++j) c[j] += a * b[j];
        }
    }
}

// C[i][j] = A_i . B_j over vectors of length len (rows of A and B), i < M, j < N, into C (ldc):
// split over the long dimension, partial sums added atomically into the zeroed C
void dots(Ctx &c, int M, int N, long long len, const double *A, const double *B, double *C, int ldc) {
    if (M <= 0 || N <= 0) return;
    TINCR_CUDA(cudaMemset2DAsync(C, (size_t)ldc * sizeof(double), 0, (size_t)N * sizeof(double), M, c.stream));
    const int sk = pick_splitk(M, N, (int)len, 1, c.n_sm);
    pgemm<false, true>(c, TINCR_KF_SUBSPACE, M, N, (int)len, A, (int)len, 0, B, (int)len, 0, 1,
                       EpiAtomicAdd{C, 0, ldc, 1.0}, sk);
}

}  // namespace

// P = (A+B) V, M = (A-B) V for k vectors (vector-major, device)
void Ctx::rpa_products(int k, const double *V, double *P, double *M) {
    const long long len = ov * k;
    if (!lc) {   // no exchange: (A-B) = omega, (A+B) = omega + 4 J
        rpa_omega_kernel<<<grid_of(len, n_sm), 256, 0, stream>>>(ov, k, d_omega.p, V, M);
        count_launch(stream, "rpa_omega");
        check_launch("rpa_omega");
        ao_contract(k, BLK_OCC, BLK_VIRT, V, BLK_OCC, BLK_VIRT, 0.0, 2.0, P, 1.0, 0.0, V);
        return;
    }
    // M = omega o V - K[V];  P = M + 4 J[V]
    ao_contract(k, BLK_OCC, BLK_VIRT, V, BLK_OCC, BLK_VIRT, -0.25, 0.0, M, 1.0, 0.0, V);
    TINCR_CUDA(cudaMemcpyAsync(P, M, (size_t)len * sizeof(double), cudaMemcpyDeviceToDevice, stream));
    ao_contract(k, BLK_OCC, BLK_VIRT, V, BLK_OCC, BLK_VIRT, 0.0, 2.0, P, 1.0, 1.0, nullptr);
    // T = -K'[V] from V^T (v x o blocks): P += T, M -= T
    rpa_w1.reserve((size_t)len);
    rpa_w2.reserve((size_t)len);
    rpa_transpose_kernel<<<grid_of(len, n_sm), 256, 0, stream>>>(k, n_occ, n_virt, V, rpa_w1.p);
    count_launch(stream, "rpa_transpose");
    check_launch("rpa_transpose");
    ao_contract(k, BLK_VIRT, BLK_OCC, rpa_w1.p, BLK_OCC, BLK_VIRT, -0.25, 0.0, rpa_w2.p, 1.0, 0.0, nullptr);
    rpa_pm_kernel<<<grid_of(len, n_sm), 256, 0, stream>>>(len, rpa_w2.p, P, M);
    count_launch(stream, "rpa_pm");
    check_launch("rpa_pm");
}

int Ctx::rpa_solve(int n_roots, int max_iter, double tol, double *energies, double *xpy_out, double *xmy_out,
                   double *osc, int *iterations) {
    if (!ready) fail(TINCR_BAD_ARG, "tincr_tda_setup must be called first");
    if (n_roots <= 0 || n_roots > ov || max_iter <= 0 || !(tol > 0.0) || !energies)
        fail(TINCR_BAD_ARG, "rpa_solve: bad arguments");
    g_launches = 0;
    prec = TINCR_PREC_FP64;
    TINCR_CUDA(cudaEventRecord(ev0, stream));
    const int max_space = std::max(15 * n_roots, 2 * n_roots + 2);
    const int mmax = max_space + 2 * n_roots;
    DevBuf<double> V((size_t)mmax * ov), P((size_t)mmax * ov), M((size_t)mmax * ov);
    DevBuf<double> XpY((size_t)n_roots * ov), XmY((size_t)n_roots * ov), R1((size_t)n_roots * ov),
        R2((size_t)n_roots * ov), T((size_t)2 * n_roots * ov);
    DevBuf<double> dproj((size_t)mmax * mmax), dsub((size_t)2 * n_roots * mmax), dw(2 * n_roots), dnorm(2 * n_roots),
        dc((size_t)2 * n_roots * mmax);
    DevBuf<int> didx(2 * n_roots);
    // guess: unit vectors on the n_roots smallest omega (solvers/utils.rs:17-26)
    {
        std::vector<int> order(ov);
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return h_omega[a] < h_omega[b]; });
        std::vector<int> pos(order.begin(), order.begin() + n_roots);
        TINCR_CUDA(cudaMemcpyAsync(didx.p, pos.data(), n_roots * sizeof(int), cudaMemcpyHostToDevice, stream));
        TINCR_CUDA(cudaMemsetAsync(V.p, 0, (size_t)n_roots * ov * sizeof(double), stream));
        rpa_unit_kernel<<<1, 256, 0, stream>>>(n_roots, ov, didx.p, V.p);
        count_launch(stream, "rpa_unit");
        check_launch("rpa_unit");
    }
    int m = n_roots, m_done = 0;
    std::vector<double> hp, hm;        // projected M+ and M- (m x m, row-major), kept between iterations
    std::vector<double> om(n_roots), errs(n_roots), nrm(2 * n_roots);
    int status = TINCR_NOT_CONVERGED, it_done = 0;
    // Gram-Schmidt of k candidate rows T against V[0:m] (twice, as a block) and among themselves;
    // rows of norm <= 1e-8 after that are dropped.  Appends to V, returns the new m.
    auto append = [&](int k, double *Tc) {
        for (int pass = 0; pass < 2 && m > 0; ++pass) {
            dots(*this, k, m, ov, Tc, V.p, dc.p, m);
            pgemm<false, false>(*this, TINCR_KF_SUBSPACE, k, (int)ov, m, dc.p, m, 0, V.p, (int)ov, 0, 1,
                                EpiStore{Tc, 0, (int)ov, -1.0, 1.0});
        }
        const int m0 = m;
        for (int j = 0; j < k; ++j) {
            double *t = Tc + (long long)j * ov;
            for (int pass = 0; pass < 2 && m > m0; ++pass) {
                const int acc = m - m0;
                dots(*this, 1, acc, ov, t, V.p + (long long)m0 * ov, dc.p, acc);
                pgemm<false, false>(*this, TINCR_KF_SUBSPACE, 1, (int)ov, acc, dc.p, acc, 0, V.p + (long long)m0 * ov,
                                    (int)ov, 0, 1, EpiStore{t, 0, (int)ov, -1.0, 1.0});
            }
            row_norms(1, ov, t, ov, dnorm.p);
            double nv = 0.0;
            TINCR_CUDA(cudaMemcpyAsync(&nv, dnorm.p, sizeof(double), cudaMemcpyDeviceToHost, stream));
            sync();
            if (!std::isfinite(nv)) fail(TINCR_NONFINITE, "rpa_solve: non-finite correction vector");
            if (nv > 1.0e-8 && m < mmax) {
                rpa_scale_copy_kernel<<<grid_of(ov, n_sm), 256, 0, stream>>>(ov, t, 1.0 / nv, V.p + (long long)m * ov);
                count_launch(stream, "rpa_scale_copy");
                check_launch("rpa_scale_copy");
                ++m;
            }
        }
    };
    std::vector<double> xs, ys;   // subspace X+Y and X-Y, [n_roots x m]
    for (int it = 0; it < max_iter; ++it) {
        it_done = it + 1;
        // 1. products of the new basis vectors; new columns of M+ and M-
        const int knew = m - m_done;
        if (knew > 0) {
            rpa_products(knew, V.p + (long long)m_done * ov, P.p + (long long)m_done * ov, M.p + (long long)m_done * ov);
            std::vector<double> blk((size_t)m * knew);
            std::vector<double> hp2((size_t)m * m), hm2((size_t)m * m);
            for (int i = 0; i < m_done; ++i)
                for (int j = 0; j < m_done; ++j) {
                    hp2[(size_t)i * m + j] = hp[(size_t)i * m_done + j];
                    hm2[(size_t)i * m + j] = hm[(size_t)i * m_done + j];
                }
            for (int which = 0; which < 2; ++which) {
                const double *Y = (which == 0 ? P.p : M.p) + (long long)m_done * ov;
                // blk[i][j] = V_i . Y_j, i < m, j < knew
                dots(*this, m, knew, ov, V.p, Y, dproj.p, knew);
                TINCR_CUDA(cudaMemcpyAsync(blk.data(), dproj.p, blk.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                           stream));
                sync();
                std::vector<double> &h = which == 0 ? hp2 : hm2;
                for (int i = 0; i < m; ++i)
                    for (int j = 0; j < knew; ++j) {
                        h[(size_t)i * m + m_done + j] = blk[(size_t)i * knew + j];
                        h[(size_t)(m_done + j) * m + i] = blk[(size_t)i * knew + j];
                    }
            }
            hp.swap(hp2);
            hm.swap(hm2);
            m_done = m;
        }
        // 2. subspace problem: with M- = L L^T, L^T M+ L t = Omega^2 t (similar to M- M+), and
        //    X+Y = L t / sqrt(Omega), X-Y = M+ (X+Y) / Omega, so that (X+Y)^T (X-Y) = 1
        for (double v : hp)
            if (!std::isfinite(v)) fail(TINCR_NONFINITE, "rpa_solve: non-finite projected matrix");
        std::vector<double> L((size_t)m * m, 0.0), tmp((size_t)m * m), H((size_t)m * m);
        for (int j = 0; j < m; ++j) {   // Cholesky, lower triangle, row-major
            double d = hm[(size_t)j * m + j];
            for (int q = 0; q < j; ++q) d -= L[(size_t)j * m + q] * L[(size_t)j * m + q];
            if (!(d > 0.0)) fail(TINCR_NONFINITE, "rpa_solve: A - B is not positive definite in the subspace");
            const double ljj = std::sqrt(d);
            L[(size_t)j * m + j] = ljj;
#pragma omp parallel for schedule(static) if (m > 64)
            for (int i = j + 1; i < m; ++i) {
                double v = hm[(size_t)i * m + j];
                for (int q = 0; q < j; ++q) v -= L[(size_t)i * m + q] * L[(size_t)j * m + q];
                L[(size_t)i * m + j] = v / ljj;
            }
        }
        host_mm(m, hp.data(), L.data(), tmp.data());          // M+ L
#pragma omp parallel for schedule(static)
        for (int i = 0; i < m; ++i)                           // H = L^T (M+ L)
            for (int j = 0; j < m; ++j) {
                double v = 0.0;
                for (int q = i; q < m; ++q) v += L[(size_t)q * m + i] * tmp[(size_t)q * m + j];
                H[(size_t)i * m + j] = v;
            }
        std::vector<double> w2(n_roots), tt((size_t)n_roots * m);
        if (!eigh_lowest_upper(m, H.data(), n_roots, w2.data(), tt.data()))
            fail(TINCR_NONFINITE, "rpa_solve: subspace eigensolver failed");
        xs.assign((size_t)n_roots * m, 0.0);
        ys.assign((size_t)n_roots * m, 0.0);
        for (int r = 0; r < n_roots; ++r) {
            if (!(w2[r] > 0.0)) fail(TINCR_NONFINITE, "rpa_solve: non-positive Omega^2");
            om[r] = std::sqrt(w2[r]);
            const double f = 1.0 / std::sqrt(om[r]);
            for (int i = 0; i < m; ++i) {   // (X+Y) = L t / sqrt(Omega)
                double v = 0.0;
                for (int q = 0; q <= i; ++q) v += L[(size_t)i * m + q] * tt[(size_t)r * m + q];
                xs[(size_t)r * m + i] = f * v;
            }
            for (int i = 0; i < m; ++i) {   // (X-Y) = M+ (X+Y) / Omega
                double v = 0.0;
                for (int q = 0; q < m; ++q) v += hp[(size_t)i * m + q] * xs[(size_t)r * m + q];
                ys[(size_t)r * m + i] = v / om[r];
            }
        }
        // 3. full-space vectors and residuals R1 = (A+B)(X+Y) - Omega (X-Y), R2 = (A-B)(X-Y) - Omega (X+Y)
        TINCR_CUDA(cudaMemcpyAsync(dsub.p, xs.data(), xs.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
        TINCR_CUDA(cudaMemcpyAsync(dsub.p + (size_t)n_roots * m, ys.data(), ys.size() * sizeof(double),
                                   cudaMemcpyHostToDevice, stream));
        TINCR_CUDA(cudaMemcpyAsync(dw.p, om.data(), n_roots * sizeof(double), cudaMemcpyHostToDevice, stream));
        const double *dxs = dsub.p, *dys = dsub.p + (size_t)n_roots * m;
        pgemm<false, false>(*this, TINCR_KF_SUBSPACE, n_roots, (int)ov, m, dxs, m, 0, V.p, (int)ov, 0, 1,
                            EpiStore{XpY.p, 0, (int)ov, 1.0, 0.0});
        pgemm<false, false>(*this, TINCR_KF_SUBSPACE, n_roots, (int)ov, m, dys, m, 0, V.p, (int)ov, 0, 1,
                            EpiStore{XmY.p, 0, (int)ov, 1.0, 0.0});
        pgemm<false, false>(*this, TINCR_KF_SUBSPACE, n_roots, (int)ov, m, dxs, m, 0, P.p, (int)ov, 0, 1,
                            EpiResidual{R1.p, XmY.p, dw.p, ov});
        pgemm<false, false>(*this, TINCR_KF_SUBSPACE, n_roots, (int)ov, m, dys, m, 0, M.p, (int)ov, 0, 1,
                            EpiResidual{R2.p, XpY.p, dw.p, ov});
        row_norms(n_roots, ov, R1.p, ov, dnorm.p);
        row_norms(n_roots, ov, R2.p, ov, dnorm.p + n_roots);
        TINCR_CUDA(cudaMemcpyAsync(nrm.data(), dnorm.p, 2 * n_roots * sizeof(double), cudaMemcpyDeviceToHost, stream));
        sync();
        std::vector<int> idx;
        std::vector<double> wsel;
        for (int r = 0; r < n_roots; ++r) {
            errs[r] = std::max(nrm[r], nrm[n_roots + r]);
            if (!std::isfinite(errs[r])) fail(TINCR_NONFINITE, "rpa_solve: non-finite residual");
            if (errs[r] >= tol) {
                idx.push_back(r);
                wsel.push_back(om[r]);
            }
        }
        last_max_residual = *std::max_element(errs.begin(), errs.end());
        if (idx.empty() && it > 0) {
            status = TINCR_OK;
            break;
        }
        if (it == max_iter - 1) break;
        const int kadd = (int)idx.size();
        if (m + 2 * kadd > max_space) {
            // collapse onto the current X+Y and X-Y
            TINCR_CUDA(cudaMemcpyAsync(T.p, XpY.p, (size_t)n_roots * ov * sizeof(double), cudaMemcpyDeviceToDevice, stream));
            TINCR_CUDA(cudaMemcpyAsync(T.p + (size_t)n_roots * ov, XmY.p, (size_t)n_roots * ov * sizeof(double),
                                       cudaMemcpyDeviceToDevice, stream));
            m = 0;
            m_done = 0;
            hp.clear();
            hm.clear();
            append(2 * n_roots, T.p);
            ++last_collapses;
            continue;
        }
        if (kadd > 0) {
            TINCR_CUDA(cudaMemcpyAsync(didx.p, idx.data(), kadd * sizeof(int), cudaMemcpyHostToDevice, stream));
            TINCR_CUDA(cudaMemcpyAsync(dw.p, wsel.data(), kadd * sizeof(double), cudaMemcpyHostToDevice, stream));
            dim3 g(grid_of(ov, n_sm), kadd);
            rpa_precondition_kernel<<<g, 256, 0, stream>>>(ov, kadd, didx.p, dw.p, R1.p, d_omega.p, T.p);
            rpa_precondition_kernel<<<g, 256, 0, stream>>>(ov, kadd, didx.p, dw.p, R2.p, d_omega.p,
                                                           T.p + (long long)kadd * ov);
            count_launch(stream, "rpa_precondition");
            count_launch(stream, "rpa_precondition");
            check_launch("rpa_precondition");
            append(2 * kadd, T.p);
        }
    }
    TINCR_CUDA(cudaEventRecord(ev1, stream));
    for (int r = 0; r < n_roots; ++r) energies[r] = om[r];
    DevBuf<double> tr((size_t)ov * n_roots);
    if (xpy_out) {
        launch_transpose(n_roots, (int)ov, XpY.p, tr.p);
        TINCR_CUDA(cudaMemcpyAsync(xpy_out, tr.p, (size_t)ov * n_roots * sizeof(double), cudaMemcpyDeviceToHost, stream));
        sync();
    }
    if (xmy_out) {
        launch_transpose(n_roots, (int)ov, XmY.p, tr.p);
        TINCR_CUDA(cudaMemcpyAsync(xmy_out, tr.p, (size_t)ov * n_roots * sizeof(double), cudaMemcpyDeviceToHost, stream));
        sync();
    }
    if (osc) {
        // transition charges of X+Y and f = 2/3 Omega |mu|^2 (the TDA's moments, tda/moments.rs:7-24)
        std::vector<double> qt((size_t)n_roots * n_atoms);
        DevBuf<double> dy((size_t)n_roots * n_atoms);
        const int keep = solve_prec;
        solve_prec = TINCR_PREC_FP64;
        qtrans_dev(n_roots, XpY.p, dy.p);
        solve_prec = keep;
        TINCR_CUDA(cudaMemcpyAsync(qt.data(), dy.p, qt.size() * sizeof(double), cudaMemcpyDeviceToHost, stream));
        sync();
        for (int r = 0; r < n_roots; ++r) {
            double mu[3] = {0, 0, 0};
            for (int A = 0; A < n_atoms; ++A)
                for (int c = 0; c < 3; ++c) mu[c] += h_xyz[(size_t)A * 3 + c] * qt[(size_t)r * n_atoms + A];
            osc[r] = 2.0 / 3.0 * om[r] * (mu[0] * mu[0] + mu[1] * mu[1] + mu[2] * mu[2]);
        }
    }
    sync();
    if (iterations) *iterations = it_done;
    float ms = 0.f;
    TINCR_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    last_ms = ms;
    last_launches = g_launches;
    return status;
}

}  // namespace tincr
