// Mixed-precision AO-direct contraction (TINCR_PREC_BF16X3): the four GEMMs of Ctx::ao_contract
// on three-plane split-BF16 operands with FP32 tensor-core accumulation (planes.cuh); omega o X is
// added in FP64.
//
//   VT  = split(V^T)                                  [|S| x |R|]   planes
//   H   = [C_R;SC_R] V                                [2n x |S|]    planes             (step 1)
//   F   = ax gamma_lr o (H [C_S;SC_S]^T)              [2n x 2n]     planes             (step 2)
//         with the Coulomb diagonals y of M captured from the same accumulator
//   z   = ac gamma y                                  FP64, then an FP32 copy
//   GT  = (F [SC_Q;C_Q] + diag(z, z) [C_Q;SC_Q])^T    [|Q| x 2n]    planes             (step 4)
//   out = [SC_P;C_P]^T G  (+ omega o X)               [|P| x |Q|]   FP64               (step 5)
// The epilogues run in FP32 on FP32 copies of gamma_lr and [C;SC] (GB300's FP64 pipe is too narrow
// for per-element conversions).  Without exchange, H is also kept in FP64 for the Coulomb
// diagonals and the Coulomb part of G is split like an operand.
#include <algorithm>

#include "gemm_tc.cuh"
#include "kernels.cuh"
#include "ops.cuh"
#include "planes.cuh"
#include "tda.cuh"

namespace tincr {

static int grid_of(long long work, int n_sm) {
    long long b = (work + 255) / 256;
    return int(std::max<long long>(1, std::min<long long>(b, 32LL * n_sm)));
}

static __global__ void to_float_kernel(long long len, const double *__restrict__ x, float *y) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < len; t += (long long)gridDim.x * blockDim.x)
        y[t] = (float)x[t];
}

static void to_float(Ctx &c, long long len, const double *x, float *y) {
    to_float_kernel<<<grid_of(len, c.n_sm), 256, 0, c.stream>>>(len, x, y);
    count_launch(c.stream, "to_float");
    check_launch("to_float");
}

// constant planes of a system: [C_o;SC_o], [C_v;SC_v] (K = block) and [SC_o;C_o]^T, [SC_v;C_v]^T (K = 2n)
void Ctx::prepare_planes() {
    if (planes_ready) return;
    const int n = n_orb;
    const long long k2 = pad64(2LL * n);
    for (int blk = 0; blk < 2; ++blk) {
        const int w = bsz(blk);
        const long long kp = pad64(w);
        const long long ps1 = 2LL * n * kp, ps2 = (long long)w * k2;
        cst[blk].alloc((size_t)N_PLANES * ps1);
        split_planes_kernel<<<grid_of(ps1, n_sm), 256, 0, stream>>>(1, 2 * n, w, stk(blk), w, 0, 0, cst[blk].p, ps1, kp,
                                                                    0);
        count_launch(stream, "split_planes");
        check_launch("split_planes");
        cswT[blk].alloc((size_t)N_PLANES * ps2);
        split_planes_kernel<<<grid_of(ps2, n_sm), 256, 0, stream>>>(1, w, 2 * n, swp(blk), w, 0, 1, cswT[blk].p, ps2, k2,
                                                                    0);
        count_launch(stream, "split_planes");
        check_launch("split_planes");
        stk32[blk].alloc((size_t)2 * n * w);
        to_float(*this, 2LL * n * w, stk(blk), stk32[blk].p);
    }
    if (lc) {
        glr32.alloc((size_t)n * n);
        to_float(*this, (long long)n * n, d_glr_ao.p, glr32.p);
    }
    planes_ready = true;
}

template <class Epi>
static void plane_gemm(Ctx &c, int family, int M, int N, long long Kpad, PlaneOperand A, PlaneOperand B, int batch,
                       Epi epi, int K_alg) {
    int slot = c.prof_begin(family);
    if (c.use_tc)
        gemm_planes_tc(c.stream, M, N, (int)Kpad, A, B, batch, epi, c.d_tc_err.p, c.n_sm,
                       c.tc_first_wait_ns < 0 ? TC_WAIT_NS : (unsigned long long)c.tc_first_wait_ns);
    else gemm_planes_mma(c.stream, M, N, (int)Kpad, A, B, batch, epi);
    double nb = batch;
    // algorithmic: FP64-equivalent flops of the contraction (counted once) and bytes of the three
    // BF16 planes of each operand read and of the result written once
    c.prof_end(slot, 2.0 * M * (double)N * K_alg * nb,
               6.0 * ((double)M * K_alg * (A.sb ? nb : 1.0) + (double)N * K_alg * (B.sb ? nb : 1.0)) +
                   6.0 * M * (double)N * nb);
}

void Ctx::ao_contract_mixed(int k, int R, int S, const double *V, int P, int Q, double ax, double ac, double *out,
                            double alpha, double beta, const double *Xomega) {
    prepare_planes();
    if (use_tc) tc_err_ensure();
    const int n = n_orb;
    const int nr = bsz(R), ns = bsz(S), np = bsz(P), nq = bsz(Q);
    const bool exch = ax != 0.0 && lc;
    const long long kr = pad64(nr), ks = pad64(ns), k2 = pad64(2LL * n);
    // one plane of each per-vector operand (elements)
    const size_t per_plane = (size_t)ns * kr + (size_t)2 * n * ks + (exch ? (size_t)2 * n * k2 : 0) + (size_t)nq * k2;
    const size_t per_f64 = (size_t)2 * n * ns + (size_t)2 * n * nq + 3 * (size_t)n;
    const size_t budget = (size_t)768 << 20;
    const int kc_max =
        (int)std::max<size_t>(1, std::min<size_t>(64, budget / (per_plane * N_PLANES * 2 + per_f64 * 8)));
    const size_t plane = per_plane * kc_max;   // elements of one plane of all per-vector operands
    const long long key = (long long)(((R * 2 + S) * 2 + Q) * 2 + (exch ? 1 : 0)) * 1000003LL + n;
    if (mx_bf16.n < N_PLANES * plane || mx_key != key) {
        mx_bf16.reserve(N_PLANES * plane);
        TINCR_CUDA(cudaMemsetAsync(mx_bf16.p, 0, mx_bf16.n * sizeof(bf16), stream));   // K padding stays zero
        mx_key = key;
    }
    mx_f64.reserve(per_f64 * kc_max);
    mx_f32.reserve((size_t)kc_max * n);
    float *z32 = mx_f32.p;
    // plane 0 of each operand; plane q lies q * plane elements further
    bf16 *VT = mx_bf16.p;
    bf16 *Hp = VT + (size_t)kc_max * ns * kr;
    bf16 *Fp = Hp + (size_t)kc_max * 2 * n * ks;
    bf16 *GTp = Fp + (exch ? (size_t)kc_max * 2 * n * k2 : 0);
    const long long ps = (long long)plane;
    double *H64 = mx_f64.p, *Gc = H64 + (size_t)kc_max * 2 * n * ns, *d3 = Gc + (size_t)kc_max * 2 * n * nq;
    double *d2 = d3 + (size_t)kc_max * n, *z = d2 + (size_t)kc_max * n;
    const long long ps_r = 2LL * n * kr, ps_s = 2LL * n * ks, ps_t = (long long)nq * k2, ps_p = (long long)np * k2;

    for (int c0 = 0; c0 < k; c0 += kc_max) {
        const int kc = std::min(kc_max, k - c0);
        const double *Vc = V + (long long)c0 * nr * ns;
        // V^T planes (K = |R|)
        split_planes_kernel<<<grid_of((long long)kc * ns * kr, n_sm), 256, 0, stream>>>(
            kc, ns, nr, Vc, ns, (long long)nr * ns, 1, VT, ps, kr, (long long)ns * kr);
        count_launch(stream, "split_planes");
        check_launch("split_planes");
        if (exch) {
            // step 1: H = [C_R;SC_R] V (planes only)
            plane_gemm(*this, TINCR_KF_AO_TRANSFORM, 2 * n, ns, kr, PlaneOperand{cst[R].p, ps_r, kr, 0},
                       PlaneOperand{VT, ps, kr, (long long)ns * kr}, kc,
                       EpiPlaneH{nullptr, 0, 0, Hp, ps, ks, 2LL * n * ks}, nr);
            // step 2: F = ax gamma_lr o (H [C_S;SC_S]^T), Coulomb diagonals of M captured
            plane_gemm(*this, TINCR_KF_AO_EXCHANGE, 2 * n, 2 * n, ks, PlaneOperand{Hp, ps, ks, 2LL * n * ks},
                       PlaneOperand{cst[S].p, ps_s, ks, 0}, kc,
                       EpiPlaneF{glr32.p, n, (float)ax, Fp, ps, k2, 2LL * n * k2, ac != 0.0 ? d3 : nullptr, d2}, ns);
            if (ac != 0.0) {
                // z = ac gamma y (FP64), then an FP32 copy for the step-4 epilogue
                launch_coulomb(stream, kc, n, n_atoms, d_ao_off.p, d_gamma.p, d3, d2, z, nullptr, nullptr, ac);
                to_float(*this, (long long)kc * n, z, z32);
            }
            // step 4: G^T = (F [SC_Q;C_Q] + diag(z, z) [C_Q;SC_Q])^T
            plane_gemm(*this, TINCR_KF_AO_EXCHANGE, 2 * n, nq, k2, PlaneOperand{Fp, ps, k2, 2LL * n * k2},
                       PlaneOperand{cswT[Q].p, ps_t, k2, 0}, kc,
                       EpiPlaneGT{ac != 0.0 ? z32 : nullptr, stk32[Q].p, n, nq, GTp, ps, k2, (long long)nq * k2}, 2 * n);
        } else {
            // step 1 with an FP64 copy of H for the Coulomb diagonals
            plane_gemm(*this, TINCR_KF_AO_TRANSFORM, 2 * n, ns, kr, PlaneOperand{cst[R].p, ps_r, kr, 0},
                       PlaneOperand{VT, ps, kr, (long long)ns * kr}, kc,
                       EpiPlaneH{H64, ns, 2LL * n * ns, Hp, ps, ks, 2LL * n * ks}, nr);
            if (ac != 0.0) {
                dim3 g(ceil_div(2LL * n * 32, 256), kc);
                diag_dots_kernel<<<g, 256, 0, stream>>>(n, ns, H64, ns, 2LL * n * ns, stk(S), d3, d2);
                count_launch(stream, "diag_dots");
                check_launch("diag_dots");
                launch_coulomb(stream, kc, n, n_atoms, d_ao_off.p, d_gamma.p, d3, d2, z, nullptr, nullptr, ac);
                dim3 g2(grid_of(2LL * n * nq, n_sm), kc);
                scale_rows_kernel<<<g2, 256, 0, stream>>>(n, nq, z, stk(Q), Gc);
                count_launch(stream, "scale_rows");
                check_launch("scale_rows");
            } else {
                TINCR_CUDA(cudaMemsetAsync(Gc, 0, (size_t)kc * 2 * n * nq * sizeof(double), stream));
            }
            split_planes_kernel<<<grid_of((long long)kc * nq * k2, n_sm), 256, 0, stream>>>(
                kc, nq, 2 * n, Gc, nq, 2LL * n * nq, 1, GTp, ps, k2, (long long)nq * k2);
            count_launch(stream, "split_planes");
            check_launch("split_planes");
        }
        // step 5: out = [SC_P;C_P]^T G (+ omega o X)
        plane_gemm(*this, TINCR_KF_AO_TRANSFORM, np, nq, k2, PlaneOperand{cswT[P].p, ps_p, k2, 0},
                   PlaneOperand{GTp, ps, k2, (long long)nq * k2}, kc,
                   EpiPlaneOut{out + (long long)c0 * np * nq, nq, (long long)np * nq, Xomega ? d_omega.p : nullptr,
                               Xomega ? Xomega + (long long)c0 * np * nq : nullptr, alpha, beta},
                   2 * n);
    }
    if (use_tc) tc_err_watch();   // reported by the next sync()
}

// Transition charges of k vectors X (q_ov X per atom) in the mixed form: H = [C_o; SC_o] X_b for all
// vectors as one three-plane split-BF16 GEMM (M = 2n, N = k v, K = o), then the AO-block diagonals
// and the atomic sums in FP64 (diag_dots_kernel, launch_coulomb).
void Ctx::qtrans_mixed(int k, const double *X, double *y_out) {
    const int n = n_orb, o = n_occ, v = n_virt;
    if (use_tc) tc_err_ensure();
    const long long kp = pad64(o);
    const long long pa = 2LL * n * kp, pb = (long long)k * v * kp;
    mg_bf16.reserve((size_t)N_PLANES * (pa + pb));
    bf16 *Ap = mg_bf16.p, *Bp = Ap + N_PLANES * pa;
    split_planes_kernel<<<grid_of(pa, n_sm), 256, 0, stream>>>(1, 2 * n, o, dLst.p, o, 0, 0, Ap, pa, kp, 0);
    count_launch(stream, "split_planes");
    check_launch("split_planes");
    // B rows (b, a) = X_b[:, a] (K = i): the transposed planes of each vector, one after the other
    split_planes_kernel<<<grid_of(pb, n_sm), 256, 0, stream>>>(k, v, o, X, v, ov, 1, Bp, pb, kp, (long long)v * kp);
    count_launch(stream, "split_planes");
    check_launch("split_planes");
    const long long nh = (long long)k * v;
    wsH.reserve((size_t)2 * n * nh);
    wsd3.reserve((size_t)k * n);
    wsd2.reserve((size_t)k * n);
    plane_gemm(*this, TINCR_KF_AO_TRANSFORM, 2 * n, (int)nh, kp, PlaneOperand{Ap, pa, kp, 0},
               PlaneOperand{Bp, pb, kp, 0}, 1, EpiPlaneOut{wsH.p, nh, 0, nullptr, nullptr, 1.0, 0.0}, o);
    dim3 g(ceil_div(2LL * n * 32, 256), k);
    diag_dots_kernel<<<g, 256, 0, stream>>>(n, v, wsH.p, nh, v, dRv.p, wsd3.p, wsd2.p);
    count_launch(stream, "diag_dots");
    check_launch("diag_dots");
    launch_coulomb(stream, k, n, n_atoms, d_ao_off.p, d_gamma.p, wsd3.p, wsd2.p, nullptr, nullptr, y_out, 1.0);
    if (use_tc) tc_err_watch();
}

// C = alpha op(A) op(B) + beta C (row-major FP64 in and out) on the three-plane tensor-core GEMM:
// op(A) is M x K (A[m*lda + k], or A[k*lda + m] when ta), op(B) is K x N (B[k*ldb + n], or
// B[n*ldb + k] when tb).  The operands are split into planes per call (K padded to 64).
void Ctx::gemm_mixed(bool ta, bool tb, int M, int N, int K, const double *A, int lda, const double *B, int ldb,
                     double *C, int ldc, double alpha, double beta) {
    if (M <= 0 || N <= 0 || K <= 0) return;
    if (use_tc) tc_err_ensure();
    const long long kp = pad64(K);
    const long long pa = (long long)M * kp, pb = (long long)N * kp;
    if (mg_bf16.n < (size_t)N_PLANES * (pa + pb) || mg_key != kp) {
        mg_bf16.reserve((size_t)N_PLANES * (pa + pb));
        mg_key = kp;
    }
    bf16 *Ap = mg_bf16.p, *Bp = Ap + N_PLANES * pa;
    // planes are written for every K column (padding included), so no memset is needed
    split_planes_kernel<<<grid_of(pa, n_sm), 256, 0, stream>>>(1, M, K, A, lda, 0, ta ? 1 : 0, Ap, pa, kp, 0);
    count_launch(stream, "split_planes");
    check_launch("split_planes");
    split_planes_kernel<<<grid_of(pb, n_sm), 256, 0, stream>>>(1, N, K, B, ldb, 0, tb ? 0 : 1, Bp, pb, kp, 0);
    count_launch(stream, "split_planes");
    check_launch("split_planes");
    plane_gemm(*this, TINCR_KF_GRADIENT, M, N, kp, PlaneOperand{Ap, pa, kp, 0}, PlaneOperand{Bp, pb, kp, 0}, 1,
               EpiPlaneOut{C, ldc, 0, nullptr, nullptr, alpha, beta}, K);
    if (use_tc) tc_err_watch();   // reported by the next sync()
}

}  // namespace tincr
