// FP64-accurate GEMMs on the 5th-generation tensor cores: exact fixed-point digits.
//
// A row x[0..K) of an operand with |x_k| < 2^E is carried as the integers X_k = trunc(|x_k| 2^(56-E))
// (|X_k| < 2^56) written as eight 7-bit digits, X_k = sum_s D_{k,s} 2^(7(7-s)), each digit with the
// sign of x_k (|D| <= 127, exact in bf16).  A dot product of two such rows is
//     2^(Ea+Eb-112) sum_{s,t} 2^(7(14-s-t)) sum_k D^a_{k,s} D^b_{k,t},
// and its 36 digit products with s + t <= 7 run as bf16 tcgen05 MMAs: the (g + 1) products of one
// level g = s + t accumulate in one FP32 TMEM accumulator.  The eight 32-column level accumulators
// are adjacent, and the B planes lie one after the other in shared memory, so one MMA of A plane s
// against B planes 0 .. 7-s (N = 32 (8 - s)) with its accumulator address shifted by s levels adds
// every product of A plane s to its level: eight MMAs per 16 k instead of 36.  Over a chunk of 128 k a level sum is an
// integer below 8 * 128 * 127^2 < 2^24, so the accumulator holds it exactly whatever the order and
// rounding of the hardware sums.  After each chunk the CUDA cores convert the eight level sums to
// integers and add them into two int64 accumulators per output, H = sum_{g<=3} G_g 2^(7(3-g)) and
// L = sum_{g>=4} G_g 2^(7(7-g)); the result is (H 2^28 + L) 2^(Ea+Eb-63).  The error is the
// truncation of each operand to 2^-56 of its row bound (at most 2^-55 (max|a| sum|b| + sum|a| max|b|))
// plus the dropped levels s + t >= 8, below 2^-51 max|a| max|b| per term and present only where both
// operands carry low digits: a fixed-point error at FP64 scale, relative to the row maxima rather
// than to each term.  All sums are exact integers, so the result does not depend on the K order or
// on a split-K reduction (int64 atomics).
// This is the fixed-point splitting of Ozaki, Ogita, Oishi and Rump ("Error-free transformations
// of matrix multiplication by using fast routines of matrix multiplication and its applications",
// Numer. Algorithms 59, 2012) with 7-bit digits sized for exact FP32 tensor-core accumulation.
//
// Operands are eight digit planes, K-major, in tiles of RT rows (128 for A, 32 for B) x 64 k, so
// that every TMA box is one contiguous block per plane (DgOperand, dg_off); K padded to 64 and rows
// to RT with zeros.  CTA = 320 threads, one 128-row x 32-column output tile at a time
// (persistent over tiles), K consumed in 64-element blocks, each block in two half-stages
// (A planes 0-3 with B planes 0-7, then A planes 4-7 with B planes 0-3) through a 2-buffer ring:
//   * warp 8 / lane 0: TMA producer (A box 64 x 128 x 4 planes, B box 64 x 32 x 8 planes, 128-byte
//     swizzle);
//   * warp 9 / lane 0: MMA issuer (M = 128, N = 32 (8 - s), K = 16), the eight level accumulators of
//     a 128-K chunk in one of two TMEM sets (2 x 8 x 32 = 512 columns), ping-pong between chunks;
//   * warps 0-7: integer folds (warp w: TMEM lanes 32 (w % 4).., columns 16 (w / 4)..), then the
//     epilogue functor on the tile's (H, L).
// Every mbarrier wait is bounded (2 s); on expiry the thread records an error code and leaves its
// loop, the MMA issuer waits (bounded) for its MMAs in flight, the producer for its loads, and the
// CTA frees its TMEM and returns.
#pragma once

#include "gemm_tc.cuh"

namespace tincr {

constexpr int DG_M = 128, DG_N = 32, DG_K = 64, DG_T = 320, DG_PLANES = 8, DG_LEVELS = 8;
constexpr int DG_ATILE = DG_M * DG_K * 2;                        // 16 KB: one A plane of a K block
constexpr int DG_BTILE = DG_N * DG_K * 2;                        // 4 KB: one B plane of a K block
constexpr int DG_BUF = 4 * DG_ATILE + DG_PLANES * DG_BTILE;      // 96 KB half-stage
constexpr int DG_SMEM = 2 * DG_BUF + 1024 + 256;
constexpr int DG_COLS = 2 * DG_LEVELS * DG_N;                    // 512 TMEM columns
// instruction descriptor, kind::f16, D = F32, A = B = BF16, both K-major, M = 128, N = n (16 <= n <= 256)
__device__ __forceinline__ uint32_t dg_idesc(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(DG_M >> 4) << 24);
}

__device__ __forceinline__ void dg_mma(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

// Signed 7-bit digits of x for the row bound 2^E (|x| < 2^E): d[s] = sign(x) ((X >> 7(7-s)) & 127),
// X = trunc(|x| 2^(56-E)), returned as bf16 bit patterns.  Zero and subnormal x give zero digits.
__device__ __forceinline__ void dg_digits(double x, int E, unsigned short (&d)[DG_PLANES]) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const int ex = (int)((bits >> 52) & 0x7ff);
    unsigned long long X = 0;
    if (ex != 0 && ex != 0x7ff) {
        const unsigned long long mant = (bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
        const int rs = 1019 + E - ex;   // X = mant * 2^(ex - 1075 + 56 - E) = mant >> rs
        if (rs < -3) X = (1ull << 56) - 1;   // x above the bound (not produced by a correct bound)
        else if (rs < 0) X = mant << (-rs);  // |x| within 2^3 of the bound
        else if (rs < 64) X = mant >> rs;
    }
    const unsigned short sg = (unsigned short)((bits >> 48) & 0x8000u);
#pragma unroll
    for (int s = 0; s < DG_PLANES; ++s) {
        const unsigned D = (unsigned)(X >> (7 * (DG_PLANES - 1 - s))) & 127u;
        // D as float: 2^23 + D has D in its low mantissa bits; subtract 2^23 (exact), take the top half
        const float f = __uint_as_float(0x4B000000u | D) - 8388608.0f;
        d[s] = (unsigned short)(__float_as_uint(f) >> 16) | (D ? sg : (unsigned short)0);
    }
}

// bound exponent of a row: the smallest E with max |x| < 2^E (0 for a zero row), from the bit
// pattern of max |x| (integer compare of non-negative doubles)
__device__ __forceinline__ int dg_bound_exp(unsigned long long maxbits) {
    if (maxbits == 0) return 0;
    int e;
    frexp(__longlong_as_double((long long)maxbits), &e);
    return e;
}

// Eight digit planes in tiles: element (plane p, row r, k) at
//   p * rows_pad * Kpad + (r / RT) * RT * Kpad + (k / 64) * RT * 64 + (r % RT) * 64 + k % 64,
// RT = 2^rt_shift (128 for A operands, 32 for B operands), rows_pad a multiple of RT, Kpad of 64.
struct DgOperand {
    bf16 *p;
    long long rows_pad, Kpad;
    int rt_shift;
};

__host__ __device__ __forceinline__ long long dg_off(const DgOperand &o, int plane, long long r, long long k) {
    const long long rt = 1LL << o.rt_shift;
    return (long long)plane * o.rows_pad * o.Kpad + (r >> o.rt_shift) * rt * o.Kpad + (k >> 6) * rt * 64 +
           (r & (rt - 1)) * 64 + (k & 63);
}

__device__ __forceinline__ void tma_load_5d(void *dst, const CUtensorMap *map, int c2, int c3, int c4, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
        "%6}], [%7];\n" ::"r"(smem_u32(dst)),
        "l"((uint64_t)map), "r"(0), "r"(0), "r"(c2), "r"(c3), "r"(c4), "r"(smem_u32(bar))
        : "memory");
}

struct DgTiles {
    int n_mt;   // 128-row tiles of A
    int n_ks;   // K splits
    int nkb;    // K blocks of 64
    __device__ __forceinline__ int count() const { return n_mt * n_ks; }
    __device__ __forceinline__ void decode(int t, int &mt, int &kb0, int &kb1) const {
        mt = t % n_mt;
        const int ks = t / n_mt;
        kb0 = (int)((long long)ks * nkb / n_ks);
        kb1 = (int)((long long)(ks + 1) * nkb / n_ks);
    }
};

template <class Epi>
__global__ void __launch_bounds__(DG_T, 1)
gemm_digits_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                   const __grid_constant__ CUtensorMap mapB4, DgTiles tl, int nbt, Epi epi, int *err) {
    extern __shared__ unsigned char dg_raw[];
    unsigned char *smem = (unsigned char *)(((uintptr_t)dg_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + 2 * DG_BUF);
    uint64_t *empty = full + 2;
    uint64_t *accf = empty + 2;   // accumulator set a holds a finished chunk
    uint64_t *acce = accf + 2;    // accumulator set a has been folded
    uint64_t *done = acce + 2;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ntiles = tl.count();

    if (threadIdx.x == 0) {
        for (int s = 0; s < 2; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
            mbar_init(&accf[s], 1);
            mbar_init(&acce[s], 8);   // one arrival per folding warp
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                     "r"(DG_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 8) {
        if (lane == 0) {
            int q = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
                int mt, kb0, kb1;
                tl.decode(t, mt, kb0, kb1);
                for (int kb = kb0; kb < kb1 && ok; ++kb)
                    for (int h = 0; h < 2; ++h, ++q) {
                        const int s = q & 1;
                        if (q >= 2 && !mbar_wait(&empty[s], ((q >> 1) & 1) ^ 1)) {
                            atomicExch(err, 1);
                            ok = false;
                            break;
                        }
                        unsigned char *st = smem + s * DG_BUF;
                        // the second half (A planes 4-7) pairs only with B planes 0-3
                        mbar_expect_tx(&full[s], 4 * DG_ATILE + (h ? 4 : DG_PLANES) * DG_BTILE);
                        tma_load_5d(st, &mapA, kb, mt, 4 * h, &full[s]);
                        tma_load_5d(st + 4 * DG_ATILE, h ? &mapB4 : &mapB, kb, nbt, 0, &full[s]);
                    }
            }
            if (!ok)   // loads still in flight land before the CTA exits
                for (int r = (q > 2 ? q - 2 : 0); r < q; ++r) mbar_wait(&full[r & 1], (r >> 1) & 1);
        }
    } else if (warp == 9) {
        if (lane == 0) {
            int q = 0, c = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
                int mt, kb0, kb1;
                tl.decode(t, mt, kb0, kb1);
                for (int kc = kb0; kc < kb1 && ok; kc += 2, ++c) {
                    const int a = c & 1;
                    if (c >= 2 && !mbar_wait(&acce[a], ((c >> 1) - 1) & 1)) {
                        atomicExch(err, 3);
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                    unsigned started = 0;
                    const int kend = kc + 2 < kb1 ? kc + 2 : kb1;
                    for (int kb = kc; kb < kend && ok; ++kb)
                        for (int h = 0; h < 2; ++h, ++q) {
                            const int s = q & 1;
                            if (!mbar_wait(&full[s], (q >> 1) & 1)) {
                                atomicExch(err, 2);
                                ok = false;
                                break;
                            }
                            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                            const uint32_t base = smem_u32(smem + s * DG_BUF);
#pragma unroll
                            for (int si = 0; si < 4; ++si) {
                                const int sa = 4 * h + si;   // A plane; B planes 0 .. 7 - sa, levels sa .. 7
                                const uint32_t d = tmem + (uint32_t)(a * DG_LEVELS * DG_N + sa * DG_N);
                                const uint32_t idesc = dg_idesc(DG_N * (DG_LEVELS - sa));
#pragma unroll
                                for (int kk = 0; kk < DG_K / 16; ++kk) {
                                    const uint64_t ad = tc_desc(base + si * DG_ATILE + kk * 32);
                                    const uint64_t bd = tc_desc(base + 4 * DG_ATILE + kk * 32);
                                    // the first MMA of a chunk (A plane 0, N = 256) initialises all eight levels
                                    dg_mma(d, ad, bd, idesc, (started | (kk > 0 ? 1u : 0u)));
                                }
                                started = 1u;
                            }
                            tc_commit(&empty[s]);
                        }
                    if (ok) tc_commit(&accf[a]);
                }
            }
            tc_commit(done);
            mbar_wait(done, 0);   // no MMA is in flight once the issuer leaves (also after a failure)
        }
    } else {
        // folding warps 0-7: row 32 (warp % 4) + lane of the tile, columns 16 (warp / 4) .. + 15
        const int quarter = warp & 3, half = warp >> 2;
        long long H[16], L[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) H[j] = L[j] = 0;
        int c = 0;
        bool ok = true;
        for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
            int mt, kb0, kb1;
            tl.decode(t, mt, kb0, kb1);
            for (int kc = kb0; kc < kb1; kc += 2, ++c) {
                const int a = c & 1;
                ok = __all_sync(0xffffffffu, mbar_wait(&accf[a], (c >> 1) & 1));
                if (!ok) {
                    if (lane == 0) atomicExch(err, 4);
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t t0 =
                    tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(a * DG_LEVELS * DG_N + half * 16);
#pragma unroll
                for (int lg = 0; lg < DG_LEVELS; lg += 4) {
                    uint32_t r0[16], r1[16], r2[16], r3[16];
                    tmem_ld16(t0 + (uint32_t)((lg + 0) * DG_N), r0);
                    tmem_ld16(t0 + (uint32_t)((lg + 1) * DG_N), r1);
                    tmem_ld16(t0 + (uint32_t)((lg + 2) * DG_N), r2);
                    tmem_ld16(t0 + (uint32_t)((lg + 3) * DG_N), r3);
                    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        // exact integers below 2^24 in magnitude
                        const long long v = ((((long long)__float2int_rz(__uint_as_float(r0[j])) << 7) +
                                              (long long)__float2int_rz(__uint_as_float(r1[j])))
                                                 << 14) +
                                            ((long long)__float2int_rz(__uint_as_float(r2[j])) << 7) +
                                            (long long)__float2int_rz(__uint_as_float(r3[j]));
                        if (lg == 0) H[j] += v;
                        else L[j] += v;
                    }
                }
                asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(&acce[a]);
            }
            if (!ok) break;
            if (kb1 > kb0) epi(mt * DG_M + quarter * 32 + lane, half * 16, H, L);
#pragma unroll
            for (int j = 0; j < 16; ++j) H[j] = L[j] = 0;
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(DG_COLS));
    }
}

// (H 2^28 + L) 2^(E - 63) as a double (one rounding: both conversions are exact, |H|, |L| < 2^53)
__device__ __forceinline__ double dg_value(long long H, long long L, double scale) {
    return fma((double)H, 268435456.0, (double)L) * scale;
}

// split-K partial sums: exact int64 atomics into acc[(row * ldn + col) * 2 + {0, 1}] (rows < M, cols < N)
struct DgEpiAtomic {
    unsigned long long *acc;
    int M, N, ldn;
    __device__ __forceinline__ void operator()(int row, int col0, const long long (&H)[16],
                                               const long long (&L)[16]) const {
        if (row >= M) return;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const int col = col0 + j;
            if (col < N && (H[j] | L[j])) {
                unsigned long long *p = acc + 2 * ((long long)row * ldn + col);
                atomicAdd(p, (unsigned long long)H[j]);
                atomicAdd(p + 1, (unsigned long long)L[j]);
            }
        }
    }
};

// linear combinations: value v of output (row = x, col = r) with scale[r] = 2^(Eb[r] - 63);
// mode 0: out[r][x] = v;  1: out[r][x] = v - u[r] R[r][x] (residual);  2: out[r][x] -= v
struct DgEpiComb {
    double *out;
    long long ld;
    const double *scale;
    int M, N, mode;
    const double *R;
    const double *u;
    __device__ __forceinline__ void operator()(int row, int col0, const long long (&H)[16],
                                               const long long (&L)[16]) const {
        if (row >= M) return;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const int col = col0 + j;
            if (col >= N) continue;
            const double v = dg_value(H[j], L[j], scale[col]);
            double *p = out + (long long)col * ld + row;
            if (mode == 0) *p = v;
            else if (mode == 1) *p = v - u[col] * R[(long long)col * ld + row];
            else *p -= v;
        }
    }
};

// 5-D map over a tiled digit operand: (k % 64, r % RT, k / 64, r / RT, plane), box 64 x RT x 1 x 1 x planes
inline CUtensorMap digit_map(const DgOperand &o, int box_planes) {
    const long long rt = 1LL << o.rt_shift;
    if (((uintptr_t)o.p & 15) || o.Kpad % DG_K || o.rows_pad % rt || o.Kpad <= 0 || o.rows_pad <= 0)
        fail(TINCR_BAD_ARG, "digit_map: layout");
    CUtensorMap m;
    cuuint64_t dims[5] = {64, (cuuint64_t)rt, (cuuint64_t)(o.Kpad / 64), (cuuint64_t)(o.rows_pad / rt), DG_PLANES};
    cuuint64_t strides[4] = {64 * 2, (cuuint64_t)(rt * 64 * 2), (cuuint64_t)(rt * o.Kpad * 2),
                             (cuuint64_t)(o.rows_pad * o.Kpad * 2)};
    cuuint32_t box[5] = {64, (cuuint32_t)rt, 1, 1, (cuuint32_t)box_planes};
    cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    CUresult r = tensor_map_encoder()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, o.p, dims, strides, box, estr,
                                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) fail(TINCR_CUDA_ERR, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
    return m;
}

// C tile loop over A rows [0, M) (128-row tiles) and the 32 B rows of row tile nbt, K = 64 nkb (at
// most the operands' Kpad) split into n_ks ranges; persistent grid of at most n_sm CTAs.
template <class Epi>
void gemm_digits(cudaStream_t st, int n_sm, int M, int nkb, int n_ks, const DgOperand &A, const DgOperand &B, int nbt,
                 Epi epi, int *d_err) {
    if (M <= 0 || nkb <= 0) return;
    if (A.rt_shift != 7 || B.rt_shift != 5 || (long long)nkb * DG_K > A.Kpad || (long long)nkb * DG_K > B.Kpad ||
        M > A.rows_pad || (nbt + 1) * 32LL > B.rows_pad)
        fail(TINCR_BAD_ARG, "gemm_digits: operand layout");
    const CUtensorMap ma = digit_map(A, 4);
    const CUtensorMap mb = digit_map(B, DG_PLANES);
    const CUtensorMap mb4 = digit_map(B, 4);
    static bool attr = false;
    if (!attr) {
        TINCR_CUDA(cudaFuncSetAttribute(gemm_digits_kernel<Epi>, cudaFuncAttributeMaxDynamicSharedMemorySize, DG_SMEM));
        attr = true;
    }
    DgTiles tl{ceil_div(M, DG_M), std::max(1, std::min(n_ks, nkb)), nkb};
    const int ntiles = tl.n_mt * tl.n_ks;
    gemm_digits_kernel<Epi><<<std::min(ntiles, n_sm), DG_T, DG_SMEM, st>>>(ma, mb, mb4, tl, nbt, epi, d_err);
    count_launch(st, "gemm_digits");
    check_launch("gemm_digits");
}

}  // namespace tincr
