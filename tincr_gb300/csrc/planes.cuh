// Split-BF16 operand planes and the plane GEMM of the mixed-precision A.X product.
//
// A value x (FP32) is carried as three BF16 numbers: hi = bf16(x), mid = bf16(x - hi),
// lo = bf16(x - hi - mid).  The two differences are exact in FP32 and the three planes hold x's 24
// significant bits.  The GEMM
//     C[M x N] = A[M x K] B[N x K]^T,   A = A0 + A1 + A2, B = B0 + B1 + B2 (plane 0 = hi),
// is accumulated as A0B0 + A0B1 + A1B0 + A0B2 + A2B0 + A1B1 in FP32 on the tensor cores (the
// dropped products are below 2^-24 relative), which gives FP32-level products from BF16 tensor
// cores.  The tensor-core sum of every 64 elements of K is folded into FP32 running sums with
// round-to-nearest adds on the CUDA cores.  Operands are K-contiguous planes with a padded
// leading dimension (padding zero): the three planes of an operand lie `ps` elements apart in one
// buffer, so every GEMM of the chain reads only BF16 and no FP64 instruction sits in the inner
// loop (GB300's FP64 pipe is ~1/1000 of its BF16 tensor rate).  The producing epilogues write the
// next GEMM's planes directly.
//
// This file holds the split kernel, the epilogue functors and a warp-level MMA implementation of
// the plane GEMM (128 x 128 CTA tile, 8 warps of 64 x 32, 32-deep K slices double-buffered with
// cp.async).  gemm_tc.cuh implements the same GEMM with tcgen05 + TMA.
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"

namespace tincr {

typedef __nv_bfloat16 bf16;

constexpr int N_PLANES = 3;

inline long long pad64(long long k) { return (k + 63) / 64 * 64; }

__device__ __forceinline__ void split3(float x, bf16 &h, bf16 &m, bf16 &l) {
    h = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(h);
    m = __float2bfloat16_rn(r1);
    l = __float2bfloat16_rn(r1 - __bfloat162float(m));
}

// x split into the three planes at p[k], p[k + ps], p[k + 2 ps]
__device__ __forceinline__ void store3(bf16 *p, long long ps, long long k, float x) {
    bf16 h, m, l;
    split3(x, h, m, l);
    p[k] = h;
    p[k + ps] = m;
    p[k + 2 * ps] = l;
}

// planes[b][r][c] (ld ldp, padding zeroed) from src[b][r][c] (or src[b][c][r] when trans) in FP64
static __global__ void split_planes_kernel(int batch, int rows, int cols, const double *__restrict__ src, long long lds,
                                           long long sbs, int trans, bf16 *dst, long long ps, long long ldp,
                                           long long sbp) {
    long long per = (long long)rows * ldp;
    long long total = per * batch;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        int b = int(t / per);
        long long e = t % per;
        int r = int(e / ldp), c = int(e % ldp);
        float x = 0.f;
        if (c < cols) x = (float)(trans ? src[b * sbs + (long long)c * lds + r] : src[b * sbs + (long long)r * lds + c]);
        store3(dst, ps, b * sbp + e, x);
    }
}

// ---------------------------------------------------------------------------------------------
// epilogues: operator()(b, m, n, float acc) for one element, run8(b, m, n, N, F8) for columns
// n .. n+7 of row m (n a multiple of 8, columns >= N skipped)
// ---------------------------------------------------------------------------------------------

struct F8 {
    float x[8];
};

// 8 consecutive values as three 16-byte stores (plane rows are 64-element padded, so aligned)
__device__ __forceinline__ void store3_8(bf16 *p, long long ps, const float (&v)[8]) {
    __align__(16) bf16 h[8], m[8], l[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) split3(v[j], h[j], m[j], l[j]);
    *reinterpret_cast<uint4 *>(p) = *reinterpret_cast<const uint4 *>(h);
    *reinterpret_cast<uint4 *>(p + ps) = *reinterpret_cast<const uint4 *>(m);
    *reinterpret_cast<uint4 *>(p + 2 * ps) = *reinterpret_cast<const uint4 *>(l);
}

// H = acc: planes for the next GEMM and, when H is set, an FP64 copy (Coulomb diagonals of the
// products without exchange)
struct EpiPlaneH {
    double *H;           // [b][m][ldh] or null
    long long ldh, sbh;
    bf16 *p;             // planes [b][m][ldp], plane stride ps
    long long ps, ldp, sbp;
    __device__ __forceinline__ void operator()(int b, int m, int n, float acc) const {
        if (H) H[b * sbh + (long long)m * ldh + n] = (double)acc;
        store3(p, ps, b * sbp + (long long)m * ldp + n, acc);
    }
    __device__ __forceinline__ void run8(int b, int m, int n, int N, const F8 &v) const {
        if (n + 8 <= N) {
            if (H) {
                double *h64 = H + b * sbh + (long long)m * ldh + n;
#pragma unroll
                for (int j = 0; j < 8; ++j) h64[j] = (double)v.x[j];
            }
            store3_8(p + b * sbp + (long long)m * ldp + n, ps, v.x);
        } else {
#pragma unroll
            for (int j = 0; j < 8; ++j)
                if (n + j < N) (*this)(b, m, n + j, v.x[j]);
        }
    }
};

// F = ax * gamma_lr o M  as planes (row m, column c of the 2n x 2n block matrix), FP32 throughout;
// the Coulomb diagonals M[mu][n+mu] -> d3 and M[n+mu][mu] -> d2 are captured when d3 is set
struct EpiPlaneF {
    const float *G;      // n x n gamma_lr in the AO basis (FP32 copy)
    int n;
    float ax;
    bf16 *p;
    long long ps, ldp, sbp;
    double *d3, *d2;     // [b][n] or null
    __device__ __forceinline__ void diag(int b, int m, int c, float acc) const {
        if (d3) {
            if (m < n && c == m + n) d3[(long long)b * n + m] = (double)acc;
            if (m >= n && c == m - n) d2[(long long)b * n + c] = (double)acc;
        }
    }
    __device__ __forceinline__ void operator()(int b, int m, int c, float acc) const {
        int rr = m < n ? m : m - n, cc = c < n ? c : c - n;
        diag(b, m, c, acc);
        store3(p, ps, b * sbp + (long long)m * ldp + c, ax * G[(long long)rr * n + cc] * acc);
    }
    __device__ __forceinline__ void run8(int b, int m, int c, int N, const F8 &v) const {
        if (c + 8 <= N) {
            const int rr = m < n ? m : m - n;
            const int dc = m < n ? m + n : m - n;   // column of the captured diagonal element
            if (d3 && dc >= c && dc < c + 8) {
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    if (c + j == dc) diag(b, m, c + j, v.x[j]);
            }
            float w[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int cc = c + j < n ? c + j : c + j - n;
                w[j] = ax * G[(long long)rr * n + cc] * v.x[j];
            }
            store3_8(p + b * sbp + (long long)m * ldp + c, ps, w);
        } else {
#pragma unroll
            for (int j = 0; j < 8; ++j)
                if (c + j < N) (*this)(b, m, c + j, v.x[j]);
        }
    }
};

// G = acc + diag(z, z) [C_Q;SC_Q] (the Coulomb part, FP32), written transposed as planes: GT[b][n][m]
struct EpiPlaneGT {
    const float *z;      // [b][n_ao] Coulomb potential per AO, or null
    const float *rv;     // [C_Q;SC_Q], 2 n_ao x ldr (FP32 copy)
    int n_ao, ldr;
    bf16 *p;
    long long ps, ldp, sbp;
    __device__ __forceinline__ void operator()(int b, int m, int n, float acc) const {
        float g = acc;
        if (z) g += z[(long long)b * n_ao + (m < n_ao ? m : m - n_ao)] * rv[(long long)m * ldr + n];
        store3(p, ps, b * sbp + (long long)n * ldp + m, g);
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
constexpr int PG_TILE = PG_M * PG_LD;                      // bf16 per (rows x K-slice) tile incl. padding
constexpr int PG_SMEM = 2 * 2 * N_PLANES * PG_TILE * 2;   // 2 stages x {A, B} x planes x bytes

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

// the six plane products of one m16n8k16 step: (0,0) (0,1) (1,0) (0,2) (2,0) (1,1)
__device__ __forceinline__ void mma_split6(float c[4], const unsigned (&a)[N_PLANES][4],
                                           const unsigned (&b)[N_PLANES][2]) {
    mma_bf16(c, a[0], b[0]);
    mma_bf16(c, a[0], b[1]);
    mma_bf16(c, a[1], b[0]);
    mma_bf16(c, a[0], b[2]);
    mma_bf16(c, a[2], b[0]);
    mma_bf16(c, a[1], b[1]);
}

struct PlaneOperand {
    const bf16 *p;       // plane 0; plane q at p + q * ps
    long long ps;
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
    const bf16 *Ab = A.p + b * A.sb, *Bb = B.p + b * B.sb;

    // tile `which`: 0..2 = A planes, 3..5 = B planes
    auto stage_ptr = [&](int s, int which) { return sm + (s * 2 * N_PLANES + which) * PG_TILE; };
    // one stage: 6 tiles of 128 rows x 32 bf16 = 6 x 512 chunks of 16 B; 256 threads x 12 chunks
    auto load_stage = [&](int s, int k0) {
#pragma unroll
        for (int q = 0; q < 12; ++q) {
            int idx = tid + q * PG_T;          // 0 .. 3071
            int which = idx >> 9;
            int within = idx & 511;
            int r = within >> 2, c = (within & 3) * 8;
            const bf16 *base;
            long long ld;
            int row0, lim;
            if (which < N_PLANES) { base = Ab + which * A.ps; ld = A.ld; row0 = m0; lim = M; }
            else                  { base = Bb + (which - N_PLANES) * B.ps; ld = B.ld; row0 = n0; lim = N; }
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
#pragma unroll
        for (int kk = 0; kk < PG_K; kk += 16) {
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                unsigned af[N_PLANES][4];
#pragma unroll
                for (int q = 0; q < N_PLANES; ++q) {
                    const bf16 *pa = stage_ptr(s, q) + (wm * 64 + i * 16 + g) * PG_LD + kk + tg * 2;
                    af[q][0] = *(const unsigned *)(pa);
                    af[q][1] = *(const unsigned *)(pa + 8 * PG_LD);
                    af[q][2] = *(const unsigned *)(pa + 8);
                    af[q][3] = *(const unsigned *)(pa + 8 * PG_LD + 8);
                }
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    unsigned bf[N_PLANES][2];
#pragma unroll
                    for (int q = 0; q < N_PLANES; ++q) {
                        const bf16 *pb = stage_ptr(s, N_PLANES + q) + (wn * 32 + j * 8 + g) * PG_LD + kk + tg * 2;
                        bf[q][0] = *(const unsigned *)(pb);
                        bf[q][1] = *(const unsigned *)(pb + 8);
                    }
                    mma_split6(part[i][j], af, bf);
                }
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
