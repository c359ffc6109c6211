// Batched FP64 GEMM with fused epilogues (SIMT, shared-memory tiled).
//
// C_b(m, n) = epi( sum_k op(A_b)(m, k) * op(B_b)(k, n) ) for b in [0, batch), row-major storage:
//   op(A)(m, k) = TA ? A[k*lda + m] : A[m*lda + k]
//   op(B)(k, n) = TB ? B[n*ldb + k] : B[k*ldb + n]
// A 64x64 output tile per 256-thread CTA, 16-deep k slices staged through shared memory with a
// register prefetch of the next slice.  Split-K over blockIdx.z (for the tall-skinny subspace
// products, whose K is the full singles space) hands partial sums to an accumulating epilogue.
//
// GB300's FP64 rate (about 2 DFMA per SM clock) makes every FP64 contraction of this path
// DFMA-bound; the tile keeps 16 independent accumulators per thread and 8 warps per CTA so the
// FP64 pipe stays busy, and shared-memory reads are broadcast (A) or conflict free (B).
#pragma once

#include "common.cuh"

namespace tincr {

constexpr int GB_M = 64, GB_N = 64, GB_K = 16, GB_T = 256;

// Plain store: C = alpha * acc + beta * C
struct EpiStore {
    double *C;
    long long sC;
    int ldc;
    double alpha, beta;
    __device__ __forceinline__ void operator()(int b, int m, int n, double acc) const {
        double *p = C + b * sC + (long long)m * ldc + n;
        *p = (beta == 0.0) ? alpha * acc : alpha * acc + beta * (*p);
    }
};

// Accumulate (split-K partial sums): C += alpha * acc
struct EpiAtomicAdd {
    double *C;
    long long sC;
    int ldc;
    double alpha;
    __device__ __forceinline__ void operator()(int b, int m, int n, double acc) const {
        atomicAdd(C + b * sC + (long long)m * ldc + n, alpha * acc);
    }
};

// One 64 x 64 output tile over k in [kbeg, kend): acc[i][j] holds C(m0 + ty + 16 i, n0 + tx + 16 j)
// for thread (tx, ty) = (tid & 15, tid >> 4).  All 256 threads of the CTA take part.
template <bool TA, bool TB>
__device__ __forceinline__ void gemm_f64_tile(int M, int N, int kbeg, int kend, const double *__restrict__ A, int lda,
                                              const double *__restrict__ B, int ldb, int m0, int n0,
                                              double (&As)[GB_K][GB_M + 1], double (&Bs)[GB_K][GB_N + 1],
                                              double (&acc)[4][4]) {
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

    double ra[4], rb[4];
    auto load = [&](int k0) {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            int m, k;
            if (!TA) { m = tid >> 2; k = ((tid & 3) << 2) + e; }
            else     { k = tid >> 4; m = ((tid & 15) << 2) + e; }
            int gm = m0 + m, gk = k0 + k;
            ra[e] = (gm < M && gk < kend) ? (TA ? A[(long long)gk * lda + gm] : A[(long long)gm * lda + gk]) : 0.0;
            int n, kb;
            if (!TB) { kb = tid >> 4; n = ((tid & 15) << 2) + e; }
            else     { n = tid >> 2; kb = ((tid & 3) << 2) + e; }
            int gn = n0 + n, gkb = k0 + kb;
            rb[e] = (gn < N && gkb < kend) ? (TB ? B[(long long)gn * ldb + gkb] : B[(long long)gkb * ldb + gn]) : 0.0;
        }
    };
    auto store = [&]() {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            int m, k;
            if (!TA) { m = tid >> 2; k = ((tid & 3) << 2) + e; }
            else     { k = tid >> 4; m = ((tid & 15) << 2) + e; }
            As[k][m] = ra[e];
            int n, kb;
            if (!TB) { kb = tid >> 4; n = ((tid & 15) << 2) + e; }
            else     { n = tid >> 2; kb = ((tid & 3) << 2) + e; }
            Bs[kb][n] = rb[e];
        }
    };

    if (kbeg < kend) {
        load(kbeg);
        for (int k0 = kbeg; k0 < kend; k0 += GB_K) {
            __syncthreads();
            store();
            __syncthreads();
            if (k0 + GB_K < kend) load(k0 + GB_K);
#pragma unroll
            for (int kk = 0; kk < GB_K; ++kk) {
                double a[4], b[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
                for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
            }
        }
    }
}

template <bool TA, bool TB, class Epi>
__global__ void __launch_bounds__(GB_T)
gemm_f64_kernel(int M, int N, int K, int k_chunk, int splitk, const double *__restrict__ A, int lda,
                long long sA, const double *__restrict__ B, int ldb, long long sB, Epi epi) {
    __shared__ double As[GB_K][GB_M + 1];
    __shared__ double Bs[GB_K][GB_N + 1];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int zb = blockIdx.z / splitk, zk = blockIdx.z % splitk;
    const int m0 = blockIdx.y * GB_M, n0 = blockIdx.x * GB_N;
    const int kbeg = zk * k_chunk;
    const int kend = min(K, kbeg + k_chunk);
    double acc[4][4];
    gemm_f64_tile<TA, TB>(M, N, kbeg, kend, A + zb * sA, lda, B + zb * sB, ldb, m0, n0, As, Bs, acc);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        int m = m0 + ty + 16 * i;
        if (m >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int n = n0 + tx + 16 * j;
            if (n < N) epi(zb, m, n, acc[i][j]);
        }
    }
}

// Launch helper.  splitk > 1 requires an accumulating epilogue.
template <bool TA, bool TB, class Epi>
void gemm_f64(cudaStream_t st, int M, int N, int K, const double *A, int lda, long long sA,
              const double *B, int ldb, long long sB, int batch, Epi epi, int splitk = 1) {
    if (M <= 0 || N <= 0 || batch <= 0) return;
    if (splitk < 1) splitk = 1;
    int k_chunk = (K + splitk - 1) / splitk;
    k_chunk = ((k_chunk + GB_K - 1) / GB_K) * GB_K;
    if (k_chunk <= 0) k_chunk = GB_K;
    splitk = (K + k_chunk - 1) / k_chunk;
    if (splitk < 1) splitk = 1;
    dim3 grid(ceil_div(N, GB_N), ceil_div(M, GB_M), batch * splitk);
    gemm_f64_kernel<TA, TB, Epi><<<grid, GB_T, 0, st>>>(M, N, K, k_chunk, splitk, A, lda, sA, B, ldb, sB, epi);
    count_launch(st, "gemm_f64");
    check_launch("gemm_f64");
}

// Split-K factor that fills the GPU for a small M x N output with a long K.
inline int pick_splitk(int M, int N, int K, int batch, int n_sm) {
    long long tiles = (long long)ceil_div(M, GB_M) * ceil_div(N, GB_N) * batch;
    long long want = 4LL * n_sm;
    if (tiles >= want) return 1;
    long long s = (want + tiles - 1) / tiles;
    long long max_s = (K + 255) / 256;   // keep at least 256 k per split
    if (s > max_s) s = max_s;
    return s < 1 ? 1 : int(s);
}

}  // namespace tincr
