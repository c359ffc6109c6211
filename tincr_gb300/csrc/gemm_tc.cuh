// Plane GEMM on the 5th-generation tensor cores: tcgen05.mma with TMEM accumulators, TMA loads.
//
// C[M x N] = A[M x K] B[N x K]^T with A and B in three split-BF16 planes each (planes.cuh),
// accumulated as the six plane products A0B0 + A0B1 + A1B0 + A0B2 + A2B0 + A1B1.
//
// Persistent: at most one CTA per SM, each walking the 128 x 128 output tiles t = blockIdx.x,
// + gridDim.x, ... (all roles in the same order), so the loads and MMAs of a tile's first K blocks
// overlap the previous tile's epilogue.  CTA = 320 threads, K consumed in 64-element (128-byte) blocks:
//   * warp 8 / lane 0: TMA producer, six boxes (A0, A1, A2, B0, B1, B2; 128 rows x 64 bf16, 128-byte
//     swizzle) per stage into a 2-stage ring, completion on the stage's "full" mbarrier;
//   * warp 9 / lane 0: MMA issuer, 4 K=16 steps x 6 products per block (tcgen05.mma.cta_group::1
//     .kind::f16, M = N = 128) into one of two TMEM accumulator pairs (ping-pong): the hi x hi product
//     in one accumulator, the five smaller products in the other; tcgen05.commit to the stage's
//     "empty" and the pair's "full" mbarrier;
//   * warps 0-7: fold each K block's pair into FP32 running sums held in registers (warp w owns
//     TMEM lanes 32 (w % 4) .. + 31 = tile rows, one row per thread, and columns 64 (w / 4) .. + 63),
//     then the epilogue functor.
// The dominant accumulator takes only 4 MMAs per block before the CUDA cores add it with
// round-to-nearest, and the small products accumulate apart from it, which keeps long K (up to
// 2 n_orb) from building up a one-sided accumulation error; the fold overlaps the next block's MMAs.
// Every mbarrier wait is bounded (2 s); on expiry the thread records an error code and leaves its
// loop, the MMA issuer waits (bounded) for its MMAs in flight, the producer for its loads, and the
// CTA frees its TMEM and returns.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>

#include "planes.cuh"

namespace tincr {

constexpr int TC_M = 128, TC_N = 128, TC_K = 64, TC_STAGES = 2, TC_T = 320;
constexpr int TC_FOLD_WARPS = 8;                         // warps 0-7 fold and run the epilogue
constexpr int TC_TILE = TC_M * TC_K * 2;                  // 16 KB (128 rows x 128 bytes)
constexpr int TC_STAGE = 2 * N_PLANES * TC_TILE;          // A0, A1, A2, B0, B1, B2
constexpr int TC_SMEM = TC_STAGES * TC_STAGE + 1024 + 256;
constexpr int TC_COLS = 4 * TC_N;                         // two ping-pong pairs {hi x hi, other products}
constexpr unsigned long long TC_WAIT_NS = 2000000000ull;  // a wait gives up after 2 s

// instruction descriptor, kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16 (bits 7-9, 10-12 = 1),
// both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28
constexpr uint32_t TC_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TC_N >> 3) << 17) |
                              ((uint32_t)(TC_M >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 bytes apart
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;                 // leading byte offset (unused for swizzled K-major), 16 B
    d |= (uint64_t)(1024 >> 4) << 32;       // stride byte offset: 1024 B between 8-row groups
    d |= (uint64_t)1 << 46;                 // descriptor version for tcgen05
    d |= (uint64_t)2 << 61;                 // swizzle: 128 B
    return d;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
    return t;
}
// bounded wait for the completion of the phase with the given parity; false on timeout.  A limit of
// 0 gives up without polling (the test hook of the failure path, see gemm_planes_tc_kernel).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity,
                                          unsigned long long limit_ns = TC_WAIT_NS) {
    if (limit_ns == 0) return false;
    uint32_t a = smem_u32(bar);
    const unsigned long long t0 = global_ns();
    for (unsigned it = 0;; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if ((it & 63) == 63 && global_ns() - t0 > limit_ns) return false;
    }
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];\n" ::"r"(smem_u32(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
        "l"(adesc), "l"(bdesc), "r"(TC_IDESC), "r"(accumulate));
}

__device__ __forceinline__ void tc_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
}

// tensor maps of the three A planes, then the three B planes
struct TcMaps {
    CUtensorMap m[2 * N_PLANES];
};

template <class Epi>
__global__ void __launch_bounds__(TC_T, 1)
gemm_planes_tc_kernel(const __grid_constant__ TcMaps maps, int M, int N, int Kpad, int a_batched, int b_batched,
                      int batch, Epi epi, int *err, unsigned long long first_wait_ns) {
    extern __shared__ unsigned char tc_raw[];
    unsigned char *smem = (unsigned char *)(((uintptr_t)tc_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + TC_STAGES * TC_STAGE);
    uint64_t *empty = full + TC_STAGES;
    uint64_t *accf = empty + TC_STAGES;      // accumulator a holds a finished K block
    uint64_t *acce = accf + 2;               // accumulator a has been folded
    uint64_t *done = acce + 2;               // every MMA issued has completed
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nk = Kpad / TC_K;
    const int tiles_n = (N + TC_N - 1) / TC_N, tiles_m = (M + TC_M - 1) / TC_M;
    const int n_tiles = tiles_n * tiles_m * batch;
    // tile t = (b tiles_m + mt) tiles_n + nt; this CTA takes t = blockIdx.x, + gridDim.x, ...  Every
    // role walks the same tiles and K blocks; g counts this CTA's K blocks over all its tiles and
    // gives the stage (g % TC_STAGES), the accumulator pair (g & 1) and the barrier phases.

    if (threadIdx.x == 0) {
        for (int s = 0; s < TC_STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(&accf[a], 1);
            mbar_init(&acce[a], TC_FOLD_WARPS);   // one arrival per folding warp
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                     "r"(TC_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == TC_FOLD_WARPS) {
        if (lane == 0) {
            long long g = 0, issued = 0;
            bool ok = true;
            for (int t = blockIdx.x; ok && t < n_tiles; t += gridDim.x) {
                const int nt = t % tiles_n, mt = (t / tiles_n) % tiles_m, b = t / (tiles_n * tiles_m);
                const int m0 = mt * TC_M, n0 = nt * TC_N;
                for (int kb = 0; kb < nk; ++kb, ++g) {
                    const int s = (int)(g % TC_STAGES);
                    if (g >= TC_STAGES && !mbar_wait(&empty[s], (unsigned)((g / TC_STAGES) & 1) ^ 1u)) {
                        atomicExch(err, 1);
                        ok = false;
                        break;
                    }
                    unsigned char *st = smem + s * TC_STAGE;
                    mbar_expect_tx(&full[s], TC_STAGE);
#pragma unroll
                    for (int q = 0; q < N_PLANES; ++q) {
                        tma_load_3d(st + q * TC_TILE, &maps.m[q], kb * TC_K, m0, a_batched ? b : 0, &full[s]);
                        tma_load_3d(st + (N_PLANES + q) * TC_TILE, &maps.m[N_PLANES + q], kb * TC_K, n0,
                                    b_batched ? b : 0, &full[s]);
                    }
                    issued = g + 1;
                }
            }
            if (!ok)   // loads still in flight land before the CTA exits
                for (long long h = (issued > TC_STAGES ? issued - TC_STAGES : 0); h < issued; ++h)
                    mbar_wait(&full[h % TC_STAGES], (unsigned)((h / TC_STAGES) & 1));
        }
    } else if (warp == TC_FOLD_WARPS + 1) {
        if (lane == 0) {
            long long g = 0;
            bool ok = true;
            for (int t = blockIdx.x; ok && t < n_tiles; t += gridDim.x) {
                for (int kb = 0; kb < nk; ++kb, ++g) {
                    const int s = (int)(g % TC_STAGES), a = (int)(g & 1);
                    // first_wait_ns limits the first of these waits (TC_WAIT_NS unless a test shortens it
                    // to exercise the recovery: the producer drains its loads, the fold warps give up)
                    if (!mbar_wait(&full[s], (unsigned)((g / TC_STAGES) & 1), g == 0 ? first_wait_ns : TC_WAIT_NS)) {
                        atomicExch(err, 2);
                        ok = false;
                        break;
                    }
                    if (g >= 2 && !mbar_wait(&acce[a], (unsigned)(((g >> 1) - 1) & 1))) {
                        atomicExch(err, 3);
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                    const uint32_t base = smem_u32(smem + s * TC_STAGE);
                    const uint32_t dm = tmem + (uint32_t)(a * 2 * TC_N), dx = dm + (uint32_t)TC_N;
#pragma unroll
                    for (int kk = 0; kk < TC_K / 16; ++kk) {
                        const uint32_t off = kk * 32;   // 16 bf16 = 32 bytes along K
                        const uint64_t a0 = tc_desc(base + 0 * TC_TILE + off), a1 = tc_desc(base + 1 * TC_TILE + off),
                                       a2 = tc_desc(base + 2 * TC_TILE + off);
                        const uint64_t b0 = tc_desc(base + 3 * TC_TILE + off), b1 = tc_desc(base + 4 * TC_TILE + off),
                                       b2 = tc_desc(base + 5 * TC_TILE + off);
                        tc_mma(dm, a0, b0, kk > 0 ? 1u : 0u);
                        tc_mma(dx, a0, b1, kk > 0 ? 1u : 0u);
                        tc_mma(dx, a1, b0, 1u);
                        tc_mma(dx, a0, b2, 1u);
                        tc_mma(dx, a2, b0, 1u);
                        tc_mma(dx, a1, b1, 1u);
                    }
                    tc_commit(&empty[s]);
                    tc_commit(&accf[a]);
                }
            }
            tc_commit(done);
            mbar_wait(done, 0);   // no MMA is in flight once the issuer leaves (also after a failure)
        }
    } else {
        // folding warps 0-7: row m0 + 32 (warp % 4) + lane (TMEM lane quarter of the warp), columns
        // n0 + 64 (warp / 4) .. + 63: two warps per lane quarter halve the fold and epilogue per thread.
        // A tile's epilogue runs while the MMAs of the next tile's first K blocks proceed.
        constexpr int HN = TC_N / 2;
        const int quarter = warp & 3, half = warp >> 2;
        long long g = 0;
        bool ok = true;
        for (int t = blockIdx.x; ok && t < n_tiles; t += gridDim.x) {
            const int nt = t % tiles_n, mt = (t / tiles_n) % tiles_m, b = t / (tiles_n * tiles_m);
            const int m0 = mt * TC_M, n0 = nt * TC_N;
            float sum[HN];
#pragma unroll
            for (int j = 0; j < HN; ++j) sum[j] = 0.f;
            for (int kb = 0; kb < nk; ++kb, ++g) {
                const int a = (int)(g & 1);
                ok = __all_sync(0xffffffffu, mbar_wait(&accf[a], (unsigned)((g >> 1) & 1)));
                if (!ok) {
                    if (lane == 0) atomicExch(err, 4);
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t t0 =
                    tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(a * 2 * TC_N) + (uint32_t)(half * HN);
#pragma unroll
                for (int c0 = 0; c0 < HN; c0 += 16) {
                    uint32_t rm[16], rx[16];
                    tmem_ld16(t0 + (uint32_t)c0, rm);
                    tmem_ld16(t0 + (uint32_t)(TC_N + c0), rx);
                    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
                    for (int j = 0; j < 16; ++j) sum[c0 + j] += __uint_as_float(rm[j]) + __uint_as_float(rx[j]);
                }
                asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(&acce[a]);
            }
            const int row = m0 + quarter * 32 + lane;
            if (ok && row < M) {
#pragma unroll
                for (int c0 = 0; c0 < HN; c0 += 8) {
                    F8 v;
#pragma unroll
                    for (int j = 0; j < 8; ++j) v.x[j] = sum[c0 + j];
                    epi.run8(b, row, n0 + half * HN + c0, N, v);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TC_COLS));
    }
}

// ---------------------------------------------------------------------------------------------
// host: tensor maps and launch
// ---------------------------------------------------------------------------------------------

inline PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        TINCR_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
        if (!p || q != cudaDriverEntryPointSuccess) fail(TINCR_CUDA_ERR, "cuTensorMapEncodeTiled not available");
        fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// 3-D map over bf16 planes [batch][rows][ld] with logical extent [batch][rows][Kpad], box 64 x 128
inline CUtensorMap plane_map(const bf16 *base, int rows, long long Kpad, long long ld, long long sb, int batch) {
    if (((uintptr_t)base & 15) || (ld * 2) % 16 || (sb * 2) % 16 || Kpad % TC_K)
        fail(TINCR_BAD_ARG, "plane_map: alignment");
    CUtensorMap m;
    cuuint64_t dims[3] = {(cuuint64_t)Kpad, (cuuint64_t)rows, (cuuint64_t)(sb ? batch : 1)};
    cuuint64_t strides[2] = {(cuuint64_t)(ld * 2), (cuuint64_t)((sb ? sb : ld * rows) * 2)};
    cuuint32_t box[3] = {TC_K, TC_M, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = tensor_map_encoder()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<bf16 *>(base), dims, strides,
                                      box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) fail(TINCR_CUDA_ERR, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
    return m;
}

template <class Epi>
void gemm_planes_tc(cudaStream_t st, int M, int N, int Kpad, PlaneOperand A, PlaneOperand B, int batch, Epi epi,
                    int *d_err, int n_sm, unsigned long long first_wait_ns = TC_WAIT_NS) {
    if (M <= 0 || N <= 0 || batch <= 0) return;
    if (Kpad <= 0 || Kpad % TC_K) fail(TINCR_BAD_ARG, "gemm_planes_tc: K not padded to 64");
    TcMaps maps;
    for (int q = 0; q < N_PLANES; ++q) {
        maps.m[q] = plane_map(A.p + q * A.ps, M, Kpad, A.ld, A.sb, batch);
        maps.m[N_PLANES + q] = plane_map(B.p + q * B.ps, N, Kpad, B.ld, B.sb, batch);
    }
    static bool attr = false;
    if (!attr) {
        TINCR_CUDA(cudaFuncSetAttribute(gemm_planes_tc_kernel<Epi>, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM));
        attr = true;
    }
    // persistent: at most one CTA per SM (the shared memory allows one), each walking its tiles
    const long long n_tiles = (long long)ceil_div(N, TC_N) * ceil_div(M, TC_M) * batch;
    if (n_tiles > (1LL << 31) - 1) fail(TINCR_BAD_ARG, "gemm_planes_tc: too many tiles");
    const int grid = (int)std::min<long long>(n_tiles, std::max(1, n_sm));
    gemm_planes_tc_kernel<Epi><<<grid, TC_T, TC_SMEM, st>>>(maps, M, N, Kpad, A.sb ? 1 : 0, B.sb ? 1 : 0, batch, epi,
                                                            d_err, first_wait_ns);
    count_launch(st, "gemm_planes_tc");
    check_launch("gemm_planes_tc");
}

}  // namespace tincr
