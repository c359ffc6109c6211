// Mixed-precision AO-direct contraction (TINCR_PREC_BF16X3): the four GEMMs of Ctx::ao_contract
// on split-BF16 planes with FP32 tensor-core accumulation.  The Coulomb diagonals (y = q_ov X per
// atom) are taken in FP64 from the FP64 copy of H, and the omega o X term is added in FP64.
//
//   VT  = split(V^T)                                  [|S| x |R|]   planes
//   H   = [C_R;SC_R] V                                [2n x |S|]    FP64 + planes      (step 1)
//   z   = ac gamma y,  Gc = diag(z, z) [C_Q;SC_Q]      FP64 (Coulomb part of G)
//   F   = ax gamma_lr o (H [C_S;SC_S]^T)              [2n x 2n]     planes             (step 2)
//   GT  = (F [SC_Q;C_Q] + Gc)^T                       [|Q| x 2n]    planes             (step 4)
//   out = [SC_P;C_P]^T G  (+ omega o X)               [|P| x |Q|]   FP64               (step 5)
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

// constant planes of a system: [C_o;SC_o], [C_v;SC_v] (K = block) and [SC_o;C_o]^T, [SC_v;C_v]^T (K = 2n)
void Ctx::prepare_planes() {
    if (planes_ready) return;
    const int n = n_orb;
    const long long k2 = pad64(2LL * n);
    for (int blk = 0; blk < 2; ++blk) {
        int w = bsz(blk);
        long long kp = pad64(w);
        cst_hi[blk].alloc((size_t)2 * n * kp);
        cst_lo[blk].alloc((size_t)2 * n * kp);
        split_planes_kernel<<<grid_of(2LL * n * kp, n_sm), 256, 0, stream>>>(1, 2 * n, w, stk(blk), w, 0, 0, cst_hi[blk].p,
                                                                             cst_lo[blk].p, kp, 0);
        count_launch(stream, "split_planes");
        check_launch("split_planes");
        cswT_hi[blk].alloc((size_t)w * k2);
        cswT_lo[blk].alloc((size_t)w * k2);
        split_planes_kernel<<<grid_of((long long)w * k2, n_sm), 256, 0, stream>>>(1, w, 2 * n, swp(blk), w, 0, 1,
                                                                                  cswT_hi[blk].p, cswT_lo[blk].p, k2, 0);
        count_launch(stream, "split_planes");
        check_launch("split_planes");
    }
    planes_ready = true;
}

template <class Epi>
static void plane_gemm(Ctx &c, int family, int M, int N, long long Kpad, PlaneOperand A, PlaneOperand B, int batch,
                       Epi epi, int K_alg) {
    int slot = c.prof_begin(family);
    if (c.use_tc) gemm_planes_tc(c.stream, M, N, (int)Kpad, A, B, batch, epi, c.d_tc_err.p);
    else gemm_planes_mma(c.stream, M, N, (int)Kpad, A, B, batch, epi);
    double nb = batch;
    // algorithmic: FP64-equivalent flops of the contraction and bytes of BF16 planes read / written once
    c.prof_end(slot, 2.0 * M * (double)N * K_alg * nb,
               4.0 * ((double)M * K_alg * (A.sb ? nb : 1.0) + (double)N * K_alg * (B.sb ? nb : 1.0)) + 4.0 * M * (double)N * nb);
}

void Ctx::ao_contract_mixed(int k, int R, int S, const double *V, int P, int Q, double ax, double ac, double *out,
                            double alpha, double beta, const double *Xomega) {
    prepare_planes();
    if (use_tc && !d_tc_err.p) {
        d_tc_err.alloc(1);
        TINCR_CUDA(cudaMemsetAsync(d_tc_err.p, 0, sizeof(int), stream));
    }
    const int n = n_orb;
    const int nr = bsz(R), ns = bsz(S), np = bsz(P), nq = bsz(Q);
    const bool exch = ax != 0.0 && lc;
    const long long kr = pad64(nr), ks = pad64(ns), k2 = pad64(2LL * n);
    // workspace per vector (elements)
    const size_t per_bf16 = (size_t)ns * kr + (size_t)2 * n * ks + (exch ? (size_t)2 * n * k2 : 0) + (size_t)nq * k2;
    const size_t per_f64 = (size_t)2 * n * ns + (size_t)2 * n * nq + 3 * (size_t)n;
    const size_t budget = (size_t)768 << 20;
    int kc_max = (int)std::max<size_t>(1, std::min<size_t>(64, budget / (per_bf16 * 4 + per_f64 * 8)));
    const size_t need16 = per_bf16 * kc_max;
    if (mx_bf16.n < 2 * need16 || mx_key != (long long)(((R * 2 + S) * 2 + Q) * 2 + (exch ? 1 : 0)) * 1000003LL + n) {
        mx_bf16.reserve(2 * need16);
        TINCR_CUDA(cudaMemsetAsync(mx_bf16.p, 0, mx_bf16.n * sizeof(bf16), stream));   // K padding stays zero
        mx_key = (long long)(((R * 2 + S) * 2 + Q) * 2 + (exch ? 1 : 0)) * 1000003LL + n;
    }
    mx_f64.reserve(per_f64 * kc_max);
    bf16 *b0 = mx_bf16.p;
    bf16 *VTh = b0, *VTl = VTh + (size_t)kc_max * ns * kr;
    bf16 *Hh = VTl + (size_t)kc_max * ns * kr, *Hl = Hh + (size_t)kc_max * 2 * n * ks;
    bf16 *Fh = Hl + (size_t)kc_max * 2 * n * ks, *Fl = Fh + (exch ? (size_t)kc_max * 2 * n * k2 : 0);
    bf16 *GTh = Fl + (exch ? (size_t)kc_max * 2 * n * k2 : 0), *GTl = GTh + (size_t)kc_max * nq * k2;
    double *H64 = mx_f64.p, *Gc = H64 + (size_t)kc_max * 2 * n * ns, *d3 = Gc + (size_t)kc_max * 2 * n * nq;
    double *d2 = d3 + (size_t)kc_max * n, *z = d2 + (size_t)kc_max * n;

    for (int c0 = 0; c0 < k; c0 += kc_max) {
        const int kc = std::min(kc_max, k - c0);
        const double *Vc = V + (long long)c0 * nr * ns;
        // V^T planes (K = |R|)
        split_planes_kernel<<<grid_of((long long)kc * ns * kr, n_sm), 256, 0, stream>>>(
            kc, ns, nr, Vc, ns, (long long)nr * ns, 1, VTh, VTl, kr, (long long)ns * kr);
        count_launch(stream, "split_planes");
        check_launch("split_planes");
        // step 1: H = [C_R;SC_R] V
        plane_gemm(*this, TINCR_KF_AO_TRANSFORM, 2 * n, ns, kr, PlaneOperand{cst_hi[R].p, cst_lo[R].p, kr, 0},
                   PlaneOperand{VTh, VTl, kr, (long long)ns * kr}, kc,
                   EpiPlaneH{H64, ns, 2LL * n * ns, Hh, Hl, ks, 2LL * n * ks}, nr);
        // Coulomb in FP64
        if (ac != 0.0) {
            dim3 g(ceil_div(2LL * n * 32, 256), kc);
            diag_dots_kernel<<<g, 256, 0, stream>>>(n, ns, H64, stk(S), d3, d2);
            count_launch(stream, "diag_dots");
            check_launch("diag_dots");
            coulomb_kernel<<<kc, 256, n_atoms * sizeof(double), stream>>>(n, n_atoms, d_ao_off.p, d_gamma.p, d3, d2, z,
                                                                           nullptr, nullptr, ac);
            count_launch(stream, "coulomb");
            check_launch("coulomb");
            dim3 g2(grid_of(2LL * n * nq, n_sm), kc);
            scale_rows_kernel<<<g2, 256, 0, stream>>>(n, nq, z, stk(Q), Gc);
            count_launch(stream, "scale_rows");
            check_launch("scale_rows");
        }
        if (exch) {
            // step 2: F = ax gamma_lr o (H [C_S;SC_S]^T)
            plane_gemm(*this, TINCR_KF_AO_EXCHANGE, 2 * n, 2 * n, ks, PlaneOperand{Hh, Hl, ks, 2LL * n * ks},
                       PlaneOperand{cst_hi[S].p, cst_lo[S].p, ks, 0}, kc,
                       EpiPlaneF{d_glr_ao.p, n, (float)ax, Fh, Fl, k2, 2LL * n * k2}, ns);
            // step 4: G^T = (F [SC_Q;C_Q] + Gc)^T
            plane_gemm(*this, TINCR_KF_AO_EXCHANGE, 2 * n, nq, k2, PlaneOperand{Fh, Fl, k2, 2LL * n * k2},
                       PlaneOperand{cswT_hi[Q].p, cswT_lo[Q].p, k2, 0}, kc,
                       EpiPlaneGT{ac != 0.0 ? Gc : nullptr, nq, 2LL * n * nq, GTh, GTl, k2, (long long)nq * k2}, 2 * n);
        } else {
            if (ac == 0.0) TINCR_CUDA(cudaMemsetAsync(Gc, 0, (size_t)kc * 2 * n * nq * sizeof(double), stream));
            split_planes_kernel<<<grid_of((long long)kc * nq * k2, n_sm), 256, 0, stream>>>(
                kc, nq, 2 * n, Gc, nq, 2LL * n * nq, 1, GTh, GTl, k2, (long long)nq * k2);
            count_launch(stream, "split_planes");
            check_launch("split_planes");
        }
        // step 5: out = [SC_P;C_P]^T G (+ omega o X)
        plane_gemm(*this, TINCR_KF_AO_TRANSFORM, np, nq, k2, PlaneOperand{cswT_hi[P].p, cswT_lo[P].p, k2, 0},
                   PlaneOperand{GTh, GTl, k2, (long long)nq * k2}, kc,
                   EpiPlaneOut{out + (long long)c0 * np * nq, nq, (long long)np * nq, Xomega ? d_omega.p : nullptr,
                               Xomega ? Xomega + (long long)c0 * np * nq : nullptr, alpha, beta},
                   2 * n);
    }
    if (use_tc) {
        int e = 0;
        TINCR_CUDA(cudaMemcpyAsync(&e, d_tc_err.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
        sync();
        if (e) {
            TINCR_CUDA(cudaMemsetAsync(d_tc_err.p, 0, sizeof(int), stream));
            fail(TINCR_CUDA_ERR, "tensor-core GEMM: a pipeline wait timed out (code " + std::to_string(e) + ")");
        }
    }
}

}  // namespace tincr
