// Split-BF16 operand planes and the plane GEMM of the mixed-precision A.X product.
//
// A value x is carried as two BF16 numbers, hi = bf16(x) and lo = bf16(x - hi) (16 significant
// bits together; the dropped lo*lo product is ~2^-16 relative).  The GEMM
//     C[M x N] = A[M x K] B[N x K]^T,   A = A_hi + A_lo, B = B_hi + B_lo,
// is accumulated as A_hi B_hi + A_hi B_lo + A_lo B_hi in FP32 on the tensor cores.  Operands are
// K-contiguous planes with a padded leading dimension (multiple of 64 elements, padding zero), so
// every GEMM of the chain reads only BF16 and no FP64 instruction sits in the inner loop (GB300's
// FP64 pipe is ~1/1000 of its BF16 tensor rate).  The producing epilogues write the next GEMM's
// planes directly.
//
// This file holds the split kernel, the epilogue functors and a warp-level MMA implementation of
// the plane GEMM (128 x 128 CTA tile, 8 warps of 64 x 32, 32-deep K slices double-buffered with
// cp.async).  gemm_tc.cuh implements the same GEMM with tcgen05 + TMA.  Both fold the tensor-core
// sum into FP32 running sums every 64 elements of K: the tensor core's own accumulation is
// one-sided over long chains, the CUDA-core adds round to nearest.
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"

namespace tincr {

typedef __nv_bfloat16 bf16;

inline long long pad64(long long k) { return (k + 63) / 64 * 64; }

__device__ __forceinline__ void split_f32(float x, bf16 &hi, bf16 &lo) {
    hi = __float2bfloat16_rn(x);
    lo = __float2bfloat16_rn(x - __bfloat162float(hi));
}

// planes[b][r][c] (ld ldp, padding zeroed) from src[b][r][c] (or src[b][c][r] when trans) in FP64
__global__ void split_planes_kernel(int batch, int rows, int cols, const double *__restrict__ src, long long lds,
                                    long long sbs, int trans, bf16 *hi, bf16 *lo, long long ldp, long long sbp) {
    long long per = (long long)rows * ldp;
    long long total = per * batch;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        int b = int(t / per);
        long long e = t % per;
        int r = int(e / ldp), c = int(e % ldp);
        float x = 0.f;
        if (c < cols) x = (float)(trans ? src[b * sbs + (long long)c * lds + r] : src[b * sbs + (long long)r * lds + c]);
        bf16 h, l;
        split_f32(x, h, l);
        hi[b * sbp + e] = h;
        lo[b * sbp + e] = l;
    }
}

// ---------------------------------------------------------------------------------------------
// epilogues: operator()(b, m, n, float acc) for one element, run8(b, m, n, N, F8) for columns
// n .. n+7 of row m (n a multiple of 8, columns >= N skipped)
// ---------------------------------------------------------------------------------------------

struct F8 {
    float x[8];
};

// 8 consecutive split values as two 16-byte stores (plane rows are 64-element padded, so aligned)
__device__ __forceinline__ void store_split8(bf16 *hi, bf16 *lo, const float (&v)[8]) {
    __align__(16) bf16 h[8], l[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) split_f32(v[j], h[j], l[j]);
    *reinterpret_cast<uint4 *>(hi) = *reinterpret_cast<const uint4 *>(h);
    *reinterpret_cast<uint4 *>(lo) = *reinterpret_cast<const uint4 *>(l);
}

// H = acc: FP64 copy (for the Coulomb diagonals) and planes for the next GEMM
struct EpiPlaneH {
    double *H;           // [b][m][ldh]
    long long ldh, sbh;
    bf16 *hi, *lo;       // [b][m][ldp]
    long long ldp, sbp;
    __device__ __forceinline__ void operator()(int b, int m, int n, float acc) const {
        H[b * sbh + (long long)m * ldh + n] = (double)acc;
        bf16 h, l;
        split_f32(acc, h, l);
        hi[b * sbp + (long long)m * ldp + n] = h;
        lo[b * sbp + (long long)m * ldp + n] = l;
    }
    __device__ __forceinline__ void run8(int b, int m, int n, int N, const F8 &v) const {
        if (n + 8 <= N) {
            double *h64 = H + b * sbh + (long long)m * ldh + n;
#pragma unroll
            for (int j = 0; j < 8; ++j) h64[j] = (double)v.x[j];
            store_split8(hi + b * sbp + (long long)m * ldp + n, lo + b * sbp + (long long)m * ldp + n, v.x);
        } else {
#pragma unroll
            for (int j = 0; j < 8; ++j)
                if (n + j < N) (*this)(b, m, n + j, v.x[j]);
        }
    }
};

// F = ax * gamma_lr o M  as planes (row m, column n of the 2n x 2n block matrix)
struct EpiPlaneF {
    const double *G;     // n x n gamma_lr in the AO basis
    int n;
    float ax;
    bf16 *hi, *lo;
    long long ldp, sbp;
    __device__ __forceinline__ void operator()(int b, int m, int c, float acc) const {
        int rr = m < n ? m : m - n, cc = c < n ? c : c - n;
        float v = ax * (float)G[(long long)rr * n + cc] * acc;
        bf16 h, l;
        split_f32(v, h, l);
        hi[b * sbp + (long long)m * ldp + c] = h;
        lo[b * sbp + (long long)m * ldp + c] = l;
    }
    __device__ __forceinline__ void run8(int b, int m, int c, int N, const F8 &v) const {
        if (c + 8 <= N) {
            const int rr = m < n ? m : m - n;
            float w[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int cc = c + j < n ? c + j : c + j - n;
                w[j] = ax * (float)G[(long long)rr * n + cc] * v.x[j];
            }
            store_split8(hi + b * sbp + (long long)m * ldp + c, lo + b * sbp + (long long)m * ldp + c, w);
        } else {
#pragma unroll
            for (int j = 0; j < 8; ++j)
                if (c + j < N) (*this)(b, m, c + j, v.x[j]);
        }
    }
};

// G = acc (+ Gc, the FP64 Coulomb part) written transposed as planes: GT[b][n][m]
struct EpiPlaneGT {
    const double *Gc;    // [b][m][ldg] or null
    long long ldg, sbg;
    bf16 *hi, *lo;
    long long ldp, sbp;
    __device__ __forceinline__ void operator()(int b, int m, int n, float acc) const {
        float g = acc;
        if (Gc) g += (float)Gc[b * sbg + (long long)m * ldg + n];
        bf16 h, l;
        split_f32(g, h, l);
        hi[b * sbp + (long long)n * ldp + m] = h;
        lo[b * sbp + (long long)n * ldp + m] = l;
    }
    __device__ __forceinline__ void run8(int b, int m, int n, int N, const F8 &v) const {
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (n + j < N) (*this)(b, m, n + j, v.x[j]);
    }
};

// out = acc + omega o X (A.X) or alpha acc + beta out, FP64
struct EpiPlaneOut {
    double *out;
    long long ld, sb;
    const double *omega;  // null: no diagonal term
    const double *X;
    double alpha, beta;
    __device__ __forceinline__ void operator()(int b, int m, int n, float acc) const {
        long long k = (long long)m * ld + n;
        double *p = out + b * sb + k;
        if (omega) *p = (double)acc + omega[k] * X[b * sb + k];
        else *p = beta == 0.0 ? alpha * (double)acc : alpha * (double)acc + beta * (*p);
    }
    __device__ __forceinline__ void run8(int b, int m, int n, int N, const F8 &v) const {
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (n + j < N) (*this)(b, m, n + j, v.x[j]);
    }
};

// ---------------------------------------------------------------------------------------------
// warp-MMA plane GEMM
// ---------------------------------------------------------------------------------------------

constexpr int PG_M = 128, PG_N = 128, PG_K = 32, PG_T = 256, PG_LD = PG_K + 8;
constexpr int PG_TILE = PG_M * PG_LD;                 // bf16 per (rows x K-slice) tile incl. padding
constexpr int PG_SMEM = 2 * 4 * PG_TILE * 2;          // 2 stages x {Ahi, Alo, Bhi, Blo} x bytes

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, int src_bytes) {
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(src_bytes));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::); }

__device__ __forceinline__ void mma_bf16(float c[4], const unsigned a[4], const unsigned b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

struct PlaneOperand {
    const bf16 *hi, *lo;
    long long ld;        // elements, multiple of 8
    long long sb;        // batch stride (elements), 0 = shared
};

template <class Epi>
__global__ void __launch_bounds__(PG_T)
gemm_planes_mma_kernel(int M, int N, int Kpad, PlaneOperand A, PlaneOperand B, Epi epi) {
    extern __shared__ __align__(16) unsigned char pg_smem[];
    bf16 *sm = reinterpret_cast<bf16 *>(pg_smem);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp >> 2, wn = warp & 3;            // warp tile origin (64 wm, 32 wn)
    const int g = lane >> 2, tg = lane & 3;
    const int b = blockIdx.z;
    const int m0 = blockIdx.y * PG_M, n0 = blockIdx.x * PG_N;
    const bf16 *Ah = A.hi + b * A.sb, *Al = A.lo + b * A.sb, *Bh = B.hi + b * B.sb, *Bl = B.lo + b * B.sb;

    auto stage_ptr = [&](int s, int which) { return sm + (s * 4 + which) * PG_TILE; };
    // one stage: 4 tiles of 128 rows x 32 bf16 = 4 x 512 chunks of 16 B; 256 threads x 8 chunks
    auto load_stage = [&](int s, int k0) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            int idx = tid + q * PG_T;          // 0 .. 2047
            int which = idx >> 9;              // 0 Ahi, 1 Alo, 2 Bhi, 3 Blo
            int within = idx & 511;
            int r = within >> 2, c = (within & 3) * 8;
            const bf16 *base;
            long long ld;
            int row0, lim;
            if (which < 2) { base = which == 0 ? Ah : Al; ld = A.ld; row0 = m0; lim = M; }
            else           { base = which == 2 ? Bh : Bl; ld = B.ld; row0 = n0; lim = N; }
            int gr = row0 + r;
            const bf16 *src = base + (long long)(gr < lim ? gr : 0) * ld + k0 + c;
            cp_async16(stage_ptr(s, which) + r * PG_LD + c, src, gr < lim ? 16 : 0);
        }
        cp_async_commit();
    };

    // acc: FP32 running sums (round-to-nearest adds); part: the tensor-core sum of one 64-deep K block
    float acc[4][4][4], part[4][4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[i][j][e] = part[i][j][e] = 0.f;

    const int nk = Kpad / PG_K;
    load_stage(0, 0);
    for (int kb = 0; kb < nk; ++kb) {
        const int s = kb & 1;
        cp_async_wait_all();
        __syncthreads();
        if (kb + 1 < nk) load_stage(s ^ 1, (kb + 1) * PG_K);
        const bf16 *sAh = stage_ptr(s, 0), *sAl = stage_ptr(s, 1), *sBh = stage_ptr(s, 2), *sBl = stage_ptr(s, 3);
#pragma unroll
        for (int kk = 0; kk < PG_K; kk += 16) {
            unsigned ah[4][4], al[4][4], bh[4][2], bl[4][2];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                int r = wm * 64 + i * 16 + g;
                const bf16 *ph = sAh + r * PG_LD + kk + tg * 2;
                const bf16 *pl = sAl + r * PG_LD + kk + tg * 2;
                ah[i][0] = *(const unsigned *)(ph);
                ah[i][1] = *(const unsigned *)(ph + 8 * PG_LD);
                ah[i][2] = *(const unsigned *)(ph + 8);
                ah[i][3] = *(const unsigned *)(ph + 8 * PG_LD + 8);
                al[i][0] = *(const unsigned *)(pl);
                al[i][1] = *(const unsigned *)(pl + 8 * PG_LD);
                al[i][2] = *(const unsigned *)(pl + 8);
                al[i][3] = *(const unsigned *)(pl + 8 * PG_LD + 8);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                int c = wn * 32 + j * 8 + g;
                const bf16 *ph = sBh + c * PG_LD + kk + tg * 2;
                const bf16 *pl = sBl + c * PG_LD + kk + tg * 2;
                bh[j][0] = *(const unsigned *)(ph);
                bh[j][1] = *(const unsigned *)(ph + 8);
                bl[j][0] = *(const unsigned *)(pl);
                bl[j][1] = *(const unsigned *)(pl + 8);
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    mma_bf16(part[i][j], ah[i], bh[j]);
                    mma_bf16(part[i][j], ah[i], bl[j]);
                    mma_bf16(part[i][j], al[i], bh[j]);
                }
        }
        if ((kb & 1) || kb + 1 == nk) {
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j)
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        acc[i][j][e] += part[i][j][e];
                        part[i][j][e] = 0.f;
                    }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                int m = m0 + wm * 64 + i * 16 + g + (e >= 2 ? 8 : 0);
                int n = n0 + wn * 32 + j * 8 + tg * 2 + (e & 1);
                if (m < M && n < N) epi(b, m, n, acc[i][j][e]);
            }
}

template <class Epi>
void gemm_planes_mma(cudaStream_t st, int M, int N, int Kpad, PlaneOperand A, PlaneOperand B, int batch, Epi epi) {
    if (M <= 0 || N <= 0 || batch <= 0) return;
    if (Kpad % PG_K) fail(TINCR_BAD_ARG, "gemm_planes: K not padded");
    static bool attr = false;
    if (!attr) {
        TINCR_CUDA(cudaFuncSetAttribute(gemm_planes_mma_kernel<Epi>, cudaFuncAttributeMaxDynamicSharedMemorySize, PG_SMEM));
        attr = true;
    }
    dim3 grid(ceil_div(N, PG_N), ceil_div(M, PG_M), batch);
    gemm_planes_mma_kernel<Epi><<<grid, PG_T, PG_SMEM, st>>>(M, N, Kpad, A, B, epi);
    count_launch(st, "gemm_planes_mma");
    check_launch("gemm_planes_mma");
}

}  // namespace tincr
