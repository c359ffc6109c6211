// GEMM epilogues of the linear-response path and the timed GEMM launcher.
#pragma once

#include "gemm_f64.cuh"
#include "tda.cuh"

namespace tincr {

// M -> F = scale * (G o M) for the LC products, capturing the two diagonals used by the Coulomb
// term before scaling (M3 = Co X SCv^T: block (0,1); M2 = SCo X Cv^T: block (1,0)).
struct EpiLcHadamard {
    double *F;
    const double *G;   // n x n, gamma_lr in the AO basis
    double *d3, *d2;   // [batch][n]
    int n;
    double scale;
    __device__ __forceinline__ void operator()(int b, int r, int c, double acc) const {
        int n2 = 2 * n;
        int rr = r < n ? r : r - n, cc = c < n ? c : c - n;
        if (r < n && c == r + n) d3[(long long)b * n + r] = acc;
        if (r >= n && c == r - n) d2[(long long)b * n + c] = acc;
        F[(long long)b * n2 * n2 + (long long)r * n2 + c] = scale * G[(long long)rr * n + cc] * acc;
    }
};

// AX_b[i][a] = acc + omega[i*v+a] * X_b[i][a]
struct EpiOmega {
    double *out;
    const double *omega;
    const double *X;
    long long ov;
    int v;
    __device__ __forceinline__ void operator()(int b, int i, int a, double acc) const {
        long long k = (long long)i * v + a;
        out[b * ov + k] = acc + omega[k] * X[b * ov + k];
    }
};

// Rk[r][x] = acc - u[r] * R[r][x]
struct EpiResidual {
    double *Rk;
    const double *R;
    const double *u;
    long long ld;
    __device__ __forceinline__ void operator()(int, int r, int x, double acc) const {
        long long k = (long long)r * ld + x;
        Rk[k] = acc - u[r] * R[k];
    }
};

// GEMM launch with optional event timing; bytes = algorithmic traffic (operands once + result)
template <bool TA, bool TB, class Epi>
static void pgemm(Ctx &c, int family, int M, int N, int K, const double *A, int lda, long long sA, const double *B,
                  int ldb, long long sB, int batch, Epi epi, int splitk = 1) {
    int slot = c.prof_begin(family);
    gemm_f64<TA, TB>(c.stream, M, N, K, A, lda, sA, B, ldb, sB, batch, epi, splitk);
    double nb = (double)batch;
    double bytes = 8.0 * ((double)M * K * (sA ? nb : 1.0) + (double)K * N * (sB ? nb : 1.0) + (double)M * N * nb);
    c.prof_end(slot, 2.0 * M * (double)N * K * nb, bytes);
}

}  // namespace tincr
