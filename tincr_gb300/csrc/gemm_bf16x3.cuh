// Split-BF16 tensor-core GEMM with FP64 operands and FP64 epilogues (mixed-precision form).
//
// Each FP64 operand element x is split into x_hi = bf16(x) and x_lo = bf16(x - x_hi) while it is
// staged into shared memory; the product is accumulated as  A_hi B_hi + A_hi B_lo + A_lo B_hi
// (the lo*lo term, ~2^-16 relative, is dropped) with BF16 MMAs that accumulate in FP32.  The FP32
// partial sum of every 32-deep K slice is folded into FP64 registers, so FP32 rounding acts on
// 32-term sums only.  Same interface and epilogue functors as gemm_f64 (row-major, optional
// transposes, batch over blockIdx.z, split-K with an accumulating epilogue).
//
// Tile: 64 x 128 per 256-thread CTA, 8 warps as 2 (m) x 4 (n), each warp 32 x 32 =
// 2 x 4 m16n8k16 tiles (FP64 fold-in accumulators keep the warp tile small); shared tiles hold
// hi and lo parts K-contiguous with a padded row stride (40 bf16) so the 32-bit fragment loads
// of a warp hit 32 distinct banks.
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"

namespace tincr {

constexpr int XB_M = 64, XB_N = 128, XB_K = 32, XB_T = 256, XB_LD = XB_K + 8;

__device__ __forceinline__ void split_bf16(double x, __nv_bfloat16 &hi, __nv_bfloat16 &lo) {
    float xf = (float)x;
    hi = __float2bfloat16_rn(xf);
    lo = __float2bfloat16_rn((float)(x - (double)__bfloat162float(hi)));
}

__device__ __forceinline__ void mma_bf16_16816(float c[4], const unsigned a[4], const unsigned b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <bool TA, bool TB, class Epi>
__global__ void __launch_bounds__(XB_T)
gemm_bf16x3_kernel(int M, int N, int K, int k_chunk, int splitk, const double *__restrict__ A, int lda, long long sA,
                   const double *__restrict__ B, int ldb, long long sB, Epi epi) {
    __shared__ __align__(16) __nv_bfloat16 Ah[XB_M * XB_LD], Al[XB_M * XB_LD];
    __shared__ __align__(16) __nv_bfloat16 Bh[XB_N * XB_LD], Bl[XB_N * XB_LD];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp >> 2, wn = warp & 3;          // warp tile origin: (32 wm, 32 wn)
    const int g = lane >> 2, tg = lane & 3;
    const int zb = blockIdx.z / splitk, zk = blockIdx.z % splitk;
    const int m0 = blockIdx.y * XB_M, n0 = blockIdx.x * XB_N;
    const int kbeg = zk * k_chunk;
    const int kend = min(K, kbeg + k_chunk);
    A += zb * sA;
    B += zb * sB;

    double acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.0;

    for (int k0 = kbeg; k0 < kend; k0 += XB_K) {
        // stage A (128 x 32) and B (128 x 32) K-contiguous, split into hi / lo
#pragma unroll 4
        for (int e = tid; e < XB_M * XB_K; e += XB_T) {
            int m, k;
            if (!TA) { m = e / XB_K; k = e % XB_K; }
            else     { k = e / XB_M; m = e % XB_M; }
            int gm = m0 + m, gk = k0 + k;
            double x = (gm < M && gk < kend) ? (TA ? A[(long long)gk * lda + gm] : A[(long long)gm * lda + gk]) : 0.0;
            split_bf16(x, Ah[m * XB_LD + k], Al[m * XB_LD + k]);
        }
#pragma unroll 4
        for (int e = tid; e < XB_N * XB_K; e += XB_T) {
            int n, k;
            if (TB) { n = e / XB_K; k = e % XB_K; }
            else    { k = e / XB_N; n = e % XB_N; }
            int gn = n0 + n, gk = k0 + k;
            double x = (gn < N && gk < kend) ? (TB ? B[(long long)gn * ldb + gk] : B[(long long)gk * ldb + gn]) : 0.0;
            split_bf16(x, Bh[n * XB_LD + k], Bl[n * XB_LD + k]);
        }
        __syncthreads();
        float c[2][4][4];
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j)
#pragma unroll
                for (int e = 0; e < 4; ++e) c[i][j][e] = 0.f;
#pragma unroll
        for (int kk = 0; kk < XB_K; kk += 16) {
            unsigned ah[2][4], al[2][4], bh[4][2], bl[4][2];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                int r = wm * 32 + i * 16 + g;
                const __nv_bfloat16 *ph = Ah + r * XB_LD + kk + tg * 2;
                const __nv_bfloat16 *pl = Al + r * XB_LD + kk + tg * 2;
                ah[i][0] = *(const unsigned *)(ph);
                ah[i][1] = *(const unsigned *)(ph + 8 * XB_LD);
                ah[i][2] = *(const unsigned *)(ph + 8);
                ah[i][3] = *(const unsigned *)(ph + 8 * XB_LD + 8);
                al[i][0] = *(const unsigned *)(pl);
                al[i][1] = *(const unsigned *)(pl + 8 * XB_LD);
                al[i][2] = *(const unsigned *)(pl + 8);
                al[i][3] = *(const unsigned *)(pl + 8 * XB_LD + 8);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                int cidx = wn * 32 + j * 8 + g;
                const __nv_bfloat16 *ph = Bh + cidx * XB_LD + kk + tg * 2;
                const __nv_bfloat16 *pl = Bl + cidx * XB_LD + kk + tg * 2;
                bh[j][0] = *(const unsigned *)(ph);
                bh[j][1] = *(const unsigned *)(ph + 8);
                bl[j][0] = *(const unsigned *)(pl);
                bl[j][1] = *(const unsigned *)(pl + 8);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    mma_bf16_16816(c[i][j], ah[i], bh[j]);
                    mma_bf16_16816(c[i][j], ah[i], bl[j]);
                    mma_bf16_16816(c[i][j], al[i], bh[j]);
                }
        }
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j)
#pragma unroll
                for (int e = 0; e < 4; ++e) acc[i][j][e] += (double)c[i][j][e];
        __syncthreads();
    }
    // epilogue: fragment (i, j): rows g / g+8, cols 2 tg, 2 tg + 1
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                int m = m0 + wm * 32 + i * 16 + g + (e >= 2 ? 8 : 0);
                int n = n0 + wn * 32 + j * 8 + tg * 2 + (e & 1);
                if (m < M && n < N) epi(zb, m, n, acc[i][j][e]);
            }
}

template <bool TA, bool TB, class Epi>
void gemm_bf16x3(cudaStream_t st, int M, int N, int K, const double *A, int lda, long long sA, const double *B,
                 int ldb, long long sB, int batch, Epi epi, int splitk = 1) {
    if (M <= 0 || N <= 0 || batch <= 0) return;
    if (splitk < 1) splitk = 1;
    int k_chunk = (K + splitk - 1) / splitk;
    k_chunk = ((k_chunk + XB_K - 1) / XB_K) * XB_K;
    if (k_chunk <= 0) k_chunk = XB_K;
    splitk = (K + k_chunk - 1) / k_chunk;
    if (splitk < 1) splitk = 1;
    dim3 grid(ceil_div(N, XB_N), ceil_div(M, XB_M), batch * splitk);
    gemm_bf16x3_kernel<TA, TB, Epi><<<grid, XB_T, 0, st>>>(M, N, K, k_chunk, splitk, A, lda, sA, B, ldb, sB, epi);
    count_launch(st, "gemm_bf16x3");
    check_launch("gemm_bf16x3");
}

}  // namespace tincr
