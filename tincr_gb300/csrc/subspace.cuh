// Tall-skinny FP64 products of the Davidson subspace (davidson.rs:86-176), without tile padding.
//
// All subspace operations multiply a few (<= 32) long vectors with up to 15 * n_roots long vectors
// of length L = n_occ * n_virt.  A square-tiled GEMM pads the short dimension to its tile and, on
// GB300's FP64 pipe (~2 DFMA per SM clock), pays for the padding in time; these kernels keep the
// short dimension exact.
//
// skinny_dots:  C[i][j] += sum_x A[i][x] B[j][x]   (i < M, j < NB <= 32), L split across CTAs,
//               32 x NB output block per CTA staged through shared memory, FP64 atomics into C.
// skinny_comb:  Out[r][x] = epi(r, x, sum_i Y[r][i] V[i][x])   (r < R <= 32), one column per
//               thread, Y staged in shared memory by 64-wide i chunks, coalesced reads of V rows.
#pragma once

#include "common.cuh"

namespace tincr {

constexpr int SK_ROWS = 32, SK_COLS = 64, SK_T = 256;

// C[M x nb] += A[M x L] . B[nb x L]^T ; rows of B at or beyond nb are read as zero.
template <int NB>
__global__ void __launch_bounds__(SK_T)
skinny_dots_guard_kernel(int M, int nb, int L, int l_chunk, const double *__restrict__ A, long long lda,
                         const double *__restrict__ B, long long ldb, double *C, int ldc) {
    __shared__ double As[SK_ROWS][SK_COLS + 1];
    __shared__ double Bs[NB][SK_COLS + 1];
    const int i0 = blockIdx.y * SK_ROWS;
    const int x_beg = blockIdx.x * l_chunk;
    const int x_end = min(L, x_beg + l_chunk);
    const int ti = threadIdx.x & 31, tj = threadIdx.x >> 5;
    constexpr int PER = NB / 8;
    double acc[PER];
#pragma unroll
    for (int k = 0; k < PER; ++k) acc[k] = 0.0;
    for (int xs = x_beg; xs < x_end; xs += SK_COLS) {
        for (int e = threadIdx.x; e < SK_ROWS * SK_COLS; e += SK_T) {
            int r = e / SK_COLS, c = e % SK_COLS;
            int gi = i0 + r, gx = xs + c;
            As[r][c] = (gi < M && gx < x_end) ? A[(long long)gi * lda + gx] : 0.0;
        }
        for (int e = threadIdx.x; e < NB * SK_COLS; e += SK_T) {
            int r = e / SK_COLS, c = e % SK_COLS;
            int gx = xs + c;
            Bs[r][c] = (r < nb && gx < x_end) ? B[(long long)r * ldb + gx] : 0.0;
        }
        __syncthreads();
#pragma unroll 8
        for (int c = 0; c < SK_COLS; ++c) {
            double a = As[ti][c];
#pragma unroll
            for (int k = 0; k < PER; ++k) acc[k] = fma(a, Bs[tj + 8 * k][c], acc[k]);
        }
        __syncthreads();
    }
    int gi = i0 + ti;
    if (gi < M)
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            int j = tj + 8 * k;
            if (j < nb) atomicAdd(C + (long long)gi * ldc + j, acc[k]);
        }
}

// Out[r][x] = epi(r, x, sum_{i < m} Y(r, i) V[i][x]),  r < R (template, <= 32),
// Y(r, i) = Y[r * ysr + i * ysi] (row-major [rows x m]: ysr = m, ysi = 1; transposed: ysr = 1, ysi = rows)
template <int R, class Epi>
__global__ void __launch_bounds__(SK_T)
skinny_comb_kernel(int m, long long L, const double *__restrict__ Y, long long ysr, long long ysi,
                   const double *__restrict__ V, long long ldv, int rows, Epi epi) {
    __shared__ double Ys[R][64];
    double acc[R];
#pragma unroll
    for (int r = 0; r < R; ++r) acc[r] = 0.0;
    const long long x = blockIdx.x * (long long)SK_T + threadIdx.x;
    for (int i0 = 0; i0 < m; i0 += 64) {
        const int ic = min(64, m - i0);
        __syncthreads();
        for (int e = threadIdx.x; e < R * 64; e += SK_T) {
            int r = e / 64, c = e % 64;
            Ys[r][c] = (r < rows && c < ic) ? Y[(long long)r * ysr + (long long)(i0 + c) * ysi] : 0.0;
        }
        __syncthreads();
        if (x < L) {
            for (int c = 0; c < ic; ++c) {
                double v = V[(long long)(i0 + c) * ldv + x];
#pragma unroll
                for (int r = 0; r < R; ++r) acc[r] = fma(Ys[r][c], v, acc[r]);
            }
        }
    }
    if (x < L)
#pragma unroll
        for (int r = 0; r < R; ++r)
            if (r < rows) epi(r, x, acc[r]);
}

// Epilogues of skinny_comb
struct CombStore {              // Out[r][x] = alpha acc + beta Out[r][x]
    double *out;
    long long ld;
    double alpha, beta;
    __device__ __forceinline__ void operator()(int r, long long x, double acc) const {
        double *p = out + (long long)r * ld + x;
        *p = beta == 0.0 ? alpha * acc : alpha * acc + beta * (*p);
    }
};

struct CombResidual {           // Rk[r][x] = acc - u[r] R[r][x]
    double *Rk;
    const double *R;
    const double *u;
    long long ld;
    __device__ __forceinline__ void operator()(int r, long long x, double acc) const {
        long long k = (long long)r * ld + x;
        Rk[k] = acc - u[r] * R[k];
    }
};

// launchers ----------------------------------------------------------------------------------

inline void skinny_dots(cudaStream_t st, int n_sm, int M, int nb, long long L, const double *A, long long lda,
                        const double *B, long long ldb, double *C, int ldc) {
    if (M <= 0 || nb <= 0 || L <= 0) return;
    int my = ceil_div(M, SK_ROWS);
    long long want = 2LL * n_sm;                       // CTAs in flight
    long long chunks = std::max<long long>(1, std::min<long long>(want / my + 1, (L + 1023) / 1024));
    int l_chunk = (int)(((L + chunks - 1) / chunks + SK_COLS - 1) / SK_COLS * SK_COLS);
    int gx = (int)((L + l_chunk - 1) / l_chunk);
    dim3 grid(gx, my);
    // the FP64 pipe is the bound: the instantiation closest above nb wastes the fewest FMAs
    if (nb <= 8) skinny_dots_guard_kernel<8><<<grid, SK_T, 0, st>>>(M, nb, (int)L, l_chunk, A, lda, B, ldb, C, ldc);
    else if (nb <= 16) skinny_dots_guard_kernel<16><<<grid, SK_T, 0, st>>>(M, nb, (int)L, l_chunk, A, lda, B, ldb, C, ldc);
    else if (nb <= 24) skinny_dots_guard_kernel<24><<<grid, SK_T, 0, st>>>(M, nb, (int)L, l_chunk, A, lda, B, ldb, C, ldc);
    else if (nb <= 32) skinny_dots_guard_kernel<32><<<grid, SK_T, 0, st>>>(M, nb, (int)L, l_chunk, A, lda, B, ldb, C, ldc);
    else fail(TINCR_BAD_ARG, "skinny_dots: more than 32 short rows");
    count_launch(st, "skinny_dots");
    check_launch("skinny_dots");
}

template <class Epi>
inline void skinny_comb(cudaStream_t st, int rows, int m, long long L, const double *Y, long long ysr, long long ysi,
                        const double *V, long long ldv, Epi epi) {
    if (rows <= 0 || L <= 0) return;
    dim3 grid((unsigned)((L + SK_T - 1) / SK_T));
    // the FP64 pipe is the bound: rows are padded to the next multiple of 4 only
#define TINCR_SKINNY_COMB(R) skinny_comb_kernel<R, Epi><<<grid, SK_T, 0, st>>>(m, L, Y, ysr, ysi, V, ldv, rows, epi)
    if (rows <= 4) TINCR_SKINNY_COMB(4);
    else if (rows <= 8) TINCR_SKINNY_COMB(8);
    else if (rows <= 12) TINCR_SKINNY_COMB(12);
    else if (rows <= 16) TINCR_SKINNY_COMB(16);
    else if (rows <= 20) TINCR_SKINNY_COMB(20);
    else if (rows <= 24) TINCR_SKINNY_COMB(24);
    else if (rows <= 28) TINCR_SKINNY_COMB(28);
    else if (rows <= 32) TINCR_SKINNY_COMB(32);
    else fail(TINCR_BAD_ARG, "skinny_comb: more than 32 output rows");
#undef TINCR_SKINNY_COMB
    count_launch(st, "skinny_comb");
    check_launch("skinny_comb");
}

}  // namespace tincr
