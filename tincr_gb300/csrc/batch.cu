// Batched LE / CT TDA: tincr's per-monomer TDA loop (src/fmo/lcmo/basis.rs:462-465, Monomer::
// prepare_tda / run_tda in src/excited_states/tda/monomer.rs:8-53, mod.rs:18-70) and the CT pair
// loop (basis.rs:170-238, PairChargeTransfer::prepare_ct_tda / run_ct_tda in
// src/excited_states/tda/ct_pair.rs:12-180) as one device-resident lockstep block Davidson.
//
// Per iteration (a CUDA graph replayed until no instance is running; heavy and light instances are
// two concurrent branches of it):
//   1. H  = [C_o;SC_o] X                      grouped GEMM (FP64 tiles, or split-BF16 planes in the
//                                             mixed form), tiles over (instance, vector)
//   2. F  = -1/4 gamma_lr o (H [C_v;SC_v]^T)  grouped GEMM with the Hadamard epilogue (LC instances),
//      or the two Coulomb diagonals only     (non-LC instances)
//   3. y = q_ov X per atom, z = gamma y       one CTA per (instance, vector)
//   4. G  = F [SC_v;C_v]                      grouped GEMM (LC) or row scaling by z (non-LC)
//   5. AX = [SC_o;C_o]^T G + omega o X        grouped GEMM with the omega epilogue
//   6. subspace step                          a 4-CTA cluster per heavy instance, one CTA per light
//      one: projections, FP64 eigensolver (Householder, multisection, inverse iteration), Ritz
//      vectors and residuals, convergence test, preconditioning, Gram-Schmidt, collapse
//      (davidson.rs:83-178)
// Every CTA of steps 1-6 reads its instance's state first and returns when the instance has
// converged or has no new vector in that slot.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <map>
#include <mutex>
#include <numeric>
#include <tuple>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include <cooperative_groups.h>

#include "batch.cuh"
#include "gemm_f64.cuh"
#include "planes.cuh"
#include "tda.cuh"

namespace tincr {

namespace cg = cooperative_groups;

constexpr int BT_T = 256;
constexpr int BT_MAXR = 6;   // roots per instance (subspace up to 90, its projected matrix in shared memory)

struct BtArrays {
    const BtInst *inst;
    BtState *state;
    double *C, *SC, *S, *blk, *glr, *gam, *omega, *V, *AV, *R, *Rk, *T, *sub, *H, *F, *D, *u, *err, *Y;
    bf16 *P;           // split-BF16 planes (mixed form): plane q of element k at P[k + q * ps]
    long long ps;
    float *glr32, *blk32, *D32;   // FP32 copies of glr, blk and D (z slots) for the plane epilogues
    const int *ao_off, *ao_atom;
    int *active;
    double tol;
};

enum BtMode { BT_FP64 = 0, BT_FINAL = 1, BT_MIXED = 2 };

// ----------------------------------------------------------------------------------------------
// grouped FP64 GEMM over static tiles {instance, vector, tile row, tile column}
// ----------------------------------------------------------------------------------------------

struct BtOp {
    int M, N, K, lda, ldb;
    const double *A, *B;
    const BtInst *in;
    int I, b;
    const double *X;   // trial vector of this (instance, vector)
};

// The trial vector of slot b: a new column of the basis (products) or a Ritz vector (final pass).
__device__ __forceinline__ bool bt_vector(const BtArrays &a, const BtInst &in, int I, int b, bool final_pass,
                                          const double **X) {
    if (final_pass) {
        if (b >= in.nr) return false;
        *X = a.R + in.off_r + (long long)b * in.ov;
        return true;
    }
    const BtState &s = a.state[I];
    if (s.status != BT_RUNNING || b >= s.m - s.m_done) return false;
    *X = a.V + in.off_v + (long long)(s.m_done + b) * in.ov;
    return true;
}

// SC = S C (set-up)
struct BtStepSC {
    BtArrays a;
    __device__ bool setup(int I, int, BtOp &op) const {
        const BtInst &in = a.inst[I];
        op.in = &a.inst[I];
        op.M = in.n; op.N = in.o + in.v; op.K = in.n;
        op.A = a.S + in.off_s; op.lda = in.n;
        op.B = a.C + in.off_c; op.ldb = in.o + in.v;
        return true;
    }
    __device__ void epi(const BtOp &op, int m, int n, double acc) const {
        a.SC[op.in->off_c + (long long)m * (op.in->o + op.in->v) + n] = acc;
    }
};

// SC = S C for every instance in FP32 on the CUDA cores (mixed form): S and C rounded to FP32,
// FP32 sums over n <= a few hundred terms, relative error ~1e-7, the accuracy the [C; SC] planes
// of the mixed products carry anyway.  64 x 64 tile per CTA (tile table of BtStepSC), 4 x 4 per thread.
__global__ void __launch_bounds__(GB_T) bt_sc32_kernel(const int4 *__restrict__ tiles, BtArrays a) {
    __shared__ float As[GB_K][GB_M + 1];
    __shared__ float Bs[GB_K][GB_N + 1];
    const int4 t = tiles[blockIdx.x];
    const BtInst &in = a.inst[t.x];
    const int n = in.n, w = in.o + in.v;
    const double *S = a.S + in.off_s, *C = a.C + in.off_c;
    const int m0 = t.z * GB_M, n0 = t.w * GB_N;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    for (int k0 = 0; k0 < n; k0 += GB_K) {
        for (int e = threadIdx.x; e < GB_K * GB_M; e += GB_T) {
            const int kk = e % GB_K, mm = e / GB_K;   // A[m][k] = S[m0 + mm][k0 + kk]
            const int gm = m0 + mm, gk = k0 + kk;
            As[kk][mm] = (gm < n && gk < n) ? (float)S[(long long)gm * n + gk] : 0.f;
        }
        for (int e = threadIdx.x; e < GB_K * GB_N; e += GB_T) {
            const int nn = e % GB_N, kk = e / GB_N;   // B[k][n] = C[k0 + kk][n0 + nn]
            const int gk = k0 + kk, gn = n0 + nn;
            Bs[kk][nn] = (gk < n && gn < w) ? (float)C[(long long)gk * w + gn] : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GB_K; ++kk) {
            float av[4], bv[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) av[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int m = m0 + ty + 16 * i;
        if (m >= n) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int c = n0 + tx + 16 * j;
            if (c < w) a.SC[in.off_c + (long long)m * w + c] = (double)acc[i][j];
        }
    }
}

// 1. H_b = [C_o;SC_o] X_b   (2n x v)
struct BtStep1 {
    BtArrays a;
    bool final_pass;
    __device__ bool setup(int I, int b, BtOp &op) const {
        const BtInst &in = a.inst[I];
        const double *X;
        if (!bt_vector(a, in, I, b, final_pass, &X)) return false;
        op.in = &a.inst[I]; op.I = I; op.b = b;
        op.M = 2 * in.n; op.N = in.v; op.K = in.o;
        op.A = a.blk + in.off_blk; op.lda = in.o;
        op.B = X; op.ldb = in.v;
        return true;
    }
    __device__ void epi(const BtOp &op, int m, int n, double acc) const {
        const BtInst &in = *op.in;
        a.H[in.off_h + (long long)op.b * 2 * in.n * in.v + (long long)m * in.v + n] = acc;
    }
};

// 2. F_b = -1/4 gamma_lr o (H_b [C_v;SC_v]^T) with the Coulomb diagonals captured (LC instances)
struct BtStep2 {
    BtArrays a;
    __device__ bool setup(int I, int b, BtOp &op) const {
        const BtInst &in = a.inst[I];
        const double *X;
        if (!in.lc || !bt_vector(a, in, I, b, false, &X)) return false;
        op.in = &a.inst[I]; op.I = I; op.b = b;
        op.M = 2 * in.n; op.N = 2 * in.n; op.K = in.v;
        op.A = a.H + in.off_h + (long long)b * 2 * in.n * in.v; op.lda = in.v;
        op.B = a.blk + in.off_blk + 2LL * in.n * in.o; op.ldb = in.v;   // [C_v;SC_v], used transposed
        return true;
    }
    __device__ void epi(const BtOp &op, int r, int c, double acc) const {
        const BtInst &in = *op.in;
        const int n = in.n, n2 = 2 * n;
        const int rr = r < n ? r : r - n, cc = c < n ? c : c - n;
        if (!in.nh) {   // Coulomb diagonals (bt_diag_kernel for block-structured instances)
            double *d = a.D + in.off_d;
            if (r < n && c == r + n) d[(long long)op.b * n + r] = acc;
            if (r >= n && c == r - n) d[(long long)(in.nr + op.b) * n + c] = acc;
        }
        a.F[in.off_f + (long long)op.b * n2 * n2 + (long long)r * n2 + c] =
            -0.25 * a.glr[in.off_glr + (long long)rr * n + cc] * acc;
    }
};

// 4. G_b = F_b [SC_v;C_v]   (2n x v, written over H_b); block-structured instances add the Coulomb
//    term z o [C_v;SC_v] here instead of through F's diagonals (their F tiles there are skipped)
struct BtStep4 {
    BtArrays a;
    __device__ bool setup(int I, int b, BtOp &op) const {
        const BtInst &in = a.inst[I];
        const double *X;
        if (!in.lc || !bt_vector(a, in, I, b, false, &X)) return false;
        op.in = &a.inst[I]; op.I = I; op.b = b;
        const int n2 = 2 * in.n;
        op.M = n2; op.N = in.v; op.K = n2;
        op.A = a.F + in.off_f + (long long)b * n2 * n2; op.lda = n2;
        op.B = a.blk + in.off_blk + (long long)n2 * (2 * in.o + in.v); op.ldb = in.v;   // [SC_v;C_v]
        return true;
    }
    __device__ void epi(const BtOp &op, int m, int n, double acc) const {
        const BtInst &in = *op.in;
        if (in.nh) {
            const int nn = in.n;
            acc += a.D[in.off_d + (long long)(2 * in.nr + op.b) * nn + (m < nn ? m : m - nn)] *
                   a.blk[in.off_blk + 2LL * nn * in.o + (long long)m * in.v + n];
        }
        a.H[in.off_h + (long long)op.b * 2 * in.n * in.v + (long long)m * in.v + n] = acc;
    }
};

// 5. AX_b = [SC_o;C_o]^T G_b + omega o X_b   (o x v)
struct BtStep5 {
    BtArrays a;
    __device__ bool setup(int I, int b, BtOp &op) const {
        const BtInst &in = a.inst[I];
        const double *X;
        if (!bt_vector(a, in, I, b, false, &X)) return false;
        op.in = &a.inst[I]; op.I = I; op.b = b; op.X = X;
        const int n2 = 2 * in.n;
        op.M = in.o; op.N = in.v; op.K = in.nh ? in.n + in.nh : n2;   // rows n+nh.. of G meet C_o = 0
        op.A = a.blk + in.off_blk + (long long)n2 * (in.o + in.v); op.lda = in.o;        // [SC_o;C_o], transposed
        op.B = a.H + in.off_h + (long long)b * n2 * in.v; op.ldb = in.v;
        return true;
    }
    __device__ void epi(const BtOp &op, int m, int n, double acc) const {
        const BtInst &in = *op.in;
        const long long k = (long long)m * in.v + n;
        const BtState &s = a.state[op.I];
        a.AV[in.off_v + (long long)(s.m_done + op.b) * in.ov + k] = acc + a.omega[in.off_omega + k] * op.X[k];
    }
};

template <bool TA, bool TB, class Step>
__global__ void __launch_bounds__(GB_T) bt_gemm_kernel(const int4 *__restrict__ tiles, Step step) {
    __shared__ double As[GB_K][GB_M + 1];
    __shared__ double Bs[GB_K][GB_N + 1];
    const int4 t = tiles[blockIdx.x];
    BtOp op;
    if (!step.setup(t.x, t.y, op)) return;   // uniform over the CTA
    const int m0 = t.z * GB_M, n0 = t.w * GB_N;
    double acc[4][4];
    gemm_f64_tile<TA, TB>(op.M, op.N, 0, op.K, op.A, op.lda, op.B, op.ldb, m0, n0, As, Bs, acc);
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int m = m0 + ty + 16 * i;
        if (m >= op.M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int n = n0 + tx + 16 * j;
            if (n < op.N) step.epi(op, m, n, acc[i][j]);
        }
    }
}

// ----------------------------------------------------------------------------------------------
// elementwise / small grouped kernels: grid (vector slot, instance)
// ----------------------------------------------------------------------------------------------

// [C_o;SC_o], [C_v;SC_v], [SC_o;C_o], [SC_v;C_v] of every instance (set-up)
__global__ void bt_pack_kernel(BtArrays a) {
    const BtInst in = a.inst[blockIdx.x];
    const int n = in.n, o = in.o, v = in.v, w = o + v;
    const double *C = a.C + in.off_c, *SC = a.SC + in.off_c;
    double *lst = a.blk + in.off_blk, *rv = lst + 2LL * n * o, *lsw = rv + 2LL * n * v, *rsw = lsw + 2LL * n * o;
    const long long total = 2LL * n * w;
    for (long long t = threadIdx.x; t < total; t += blockDim.x) {
        const int r = int(t / w), c = int(t % w);
        const int mu = r < n ? r : r - n;
        const double cv = C[(long long)mu * w + c], sv = SC[(long long)mu * w + c];
        if (c < o) {
            lst[(long long)r * o + c] = r < n ? cv : sv;
            lsw[(long long)r * o + c] = r < n ? sv : cv;
        } else {
            rv[(long long)r * v + c - o] = r < n ? cv : sv;
            rsw[(long long)r * v + c - o] = r < n ? sv : cv;
        }
    }
}

// gamma_lr in the AO basis from the atom-pair matrix (stored in place of gamma_lr atomwise) (set-up)
__global__ void bt_expand_kernel(BtArrays a, const double *__restrict__ glr_atoms, const long long *__restrict__ off_atoms) {
    const BtInst in = a.inst[blockIdx.x];
    if (!in.lc) return;
    const int *ao_atom = a.ao_atom + in.off_aoatom;
    const double *g = glr_atoms + off_atoms[blockIdx.x];
    const long long total = (long long)in.n * in.n;
    for (long long t = threadIdx.x; t < total; t += blockDim.x) {
        const int mu = int(t / in.n), nu = int(t % in.n);
        a.glr[in.off_glr + t] = g[(long long)ao_atom[mu] * in.N + ao_atom[nu]];
    }
}

// FP32 copies of gamma_lr (AO) and the packed blocks for the mixed form's epilogues (set-up)
__global__ void bt_f32_copies_kernel(BtArrays a) {
    const BtInst in = a.inst[blockIdx.x];
    const long long nb = 2LL * in.n * 2 * (in.o + in.v);
    for (long long t = threadIdx.x; t < nb; t += blockDim.x) a.blk32[in.off_blk + t] = (float)a.blk[in.off_blk + t];
    if (in.lc)
        for (long long t = threadIdx.x; t < (long long)in.n * in.n; t += blockDim.x)
            a.glr32[in.off_glr + t] = (float)a.glr[in.off_glr + t];
}

// unit vectors on the nr smallest omega (solvers/utils.rs:17-26), state reset
__global__ void bt_guess_kernel(BtArrays a, const int *__restrict__ pos) {
    const int I = blockIdx.x;
    const BtInst in = a.inst[I];
    double *V = a.V + in.off_v;
    for (long long t = threadIdx.x; t < (long long)in.nr * in.ov; t += blockDim.x) V[t] = 0.0;
    __syncthreads();
    if (threadIdx.x < in.nr) V[(long long)threadIdx.x * in.ov + pos[in.off_u + threadIdx.x]] = 1.0;
    if (threadIdx.x == 0) {
        BtState s{};
        s.m = in.nr;
        s.m_done = 0;
        s.dim_sub = in.nr;
        s.status = BT_RUNNING;
        a.state[I] = s;
    }
}

// Coulomb diagonals d3_mu = M[mu][n+mu], d2_mu = M[n+mu][mu] of M = H [C_v;SC_v]^T, one warp per row
// (non-LC and, in the mixed form, block-structured instances in the products, every instance in the
// final pass)
__global__ void bt_diag_kernel(BtArrays a, int mode, int I0) {
    const int I = I0 + blockIdx.y, b = blockIdx.x;
    const BtInst in = a.inst[I];
    const double *X;
    if (!bt_vector(a, in, I, b, mode == BT_FINAL, &X)) return;
    // the exchange GEMM's epilogue captures them for LC instances, unless it skips their blocks
    if (mode != BT_FINAL && in.lc && !in.nh) return;
    const int n = in.n, v = in.v;
    const double *H = a.H + in.off_h + (long long)b * 2 * n * v;
    const double *rv = a.blk + in.off_blk + 2LL * n * in.o;
    double *d = a.D + in.off_d;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int r = warp; r < 2 * n; r += blockDim.x >> 5) {
        const int mu = r < n ? r : r - n;
        const double *h = H + (long long)r * v;
        const double *q = rv + (long long)(r < n ? n + mu : mu) * v;
        double s = 0.0;
        for (int x = lane; x < v; x += 32) s += h[x] * q[x];
        for (int off = 16; off; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
        if (lane == 0) d[(long long)((r < n ? 0 : in.nr) + b) * n + mu] = s;
    }
}

// y_A = 1/2 sum_{mu in A}(d3 + d2) (= q_ov X per atom), z = gamma y; z onto F's off-diagonal-block
// diagonals (FP64 form, LC) or kept per AO (non-LC, and the mixed form); in the final pass y is the
// transition charge of the root.
__global__ void bt_coulomb_kernel(BtArrays a, int mode, int I0) {
    extern __shared__ double ysh[];
    const int I = I0 + blockIdx.y, b = blockIdx.x;
    const BtInst in = a.inst[I];
    const double *X;
    const bool final_pass = mode == BT_FINAL;
    if (!bt_vector(a, in, I, b, final_pass, &X)) return;
    const int n = in.n, N = in.N;
    const int *ao_off = a.ao_off + in.off_ao;
    const double *d3 = a.D + in.off_d + (long long)b * n, *d2 = a.D + in.off_d + (long long)(in.nr + b) * n;
    for (int A = threadIdx.x; A < N; A += blockDim.x) {
        double s = 0.0;
        for (int mu = ao_off[A]; mu < ao_off[A + 1]; ++mu) s += d3[mu] + d2[mu];
        ysh[A] = 0.5 * s;
        if (final_pass) a.Y[in.off_y + (long long)b * N + A] = 0.5 * s;
    }
    if (final_pass) return;
    __syncthreads();
    const double *gam = a.gam + in.off_gam;
    const int n2 = 2 * n;
    for (int A = threadIdx.x; A < N; A += blockDim.x) {
        double z = 0.0;
        for (int B = 0; B < N; ++B) z += gam[(long long)A * N + B] * ysh[B];
        for (int mu = ao_off[A]; mu < ao_off[A + 1]; ++mu) {
            if (in.lc && mode == BT_FP64 && !in.nh) {
                double *f = a.F + in.off_f + (long long)b * n2 * n2;
                f[(long long)mu * n2 + n + mu] += z;
                f[(long long)(n + mu) * n2 + mu] += z;
            } else {
                a.D[in.off_d + (long long)(2 * in.nr + b) * n + mu] = z;
                if (mode == BT_MIXED) a.D32[in.off_d + (long long)(2 * in.nr + b) * n + mu] = (float)z;
            }
        }
    }
}

// non-LC: G_b = diag(z, z) [C_v;SC_v]  (written over H_b)
__global__ void bt_scale_rows_kernel(BtArrays a, int I0) {
    const int I = I0 + blockIdx.y, b = blockIdx.x;
    const BtInst in = a.inst[I];
    const double *X;
    if (in.lc || !bt_vector(a, in, I, b, false, &X)) return;
    const int n = in.n, v = in.v;
    const double *z = a.D + in.off_d + (long long)(2 * in.nr + b) * n;
    const double *rv = a.blk + in.off_blk + 2LL * n * in.o;
    double *G = a.H + in.off_h + (long long)b * 2 * n * v;
    for (long long t = threadIdx.x; t < 2LL * n * v; t += blockDim.x) {
        const int r = int(t / v);
        G[t] = z[r < n ? r : r - n] * rv[t];
    }
}

// ----------------------------------------------------------------------------------------------
// mixed form: grouped three-plane split-BF16 GEMM (BM x BN tiles, warp MMA, six plane products,
// FP32 folded every 32 of K).  The tile shape of each instance and product step is chosen by the
// autotuner below, keyed on the instance's shape.
// ----------------------------------------------------------------------------------------------

inline int pad32(int k) { return (k + 31) / 32 * 32; }

struct BtPlaneOp {
    int M, N, Kpad, lda, ldb;
    const bf16 *A, *B;   // plane 0 (plane q at + q * ps)
    const BtInst *in;
    int I, b;
    const double *X;
};

constexpr int BP_T = 128, BP_K = 32, BP_LD = BP_K + 8;
// tile shapes (rows of A x rows of B per CTA) the autotuner chooses from
constexpr int BP_SHAPES = 4;
constexpr int BP_BM[BP_SHAPES] = {64, 64, 32, 32};
constexpr int BP_BN[BP_SHAPES] = {64, 32, 64, 32};
constexpr int bp_smem(int bm, int bn) { return 2 * N_PLANES * (bm + bn) * BP_LD * 2; }   // 2 stages, bytes

// Four warps in a 2 x 2 arrangement, each computing a (BM/2) x (BN/2) block from m16n8k16 MMAs.
// Every output element sees the same K order (32-deep slices, two MMA k-steps each, folded after
// every slice) whatever the tile shape, so the results do not depend on the shape.
template <class Step, int BM, int BN>
__global__ void __launch_bounds__(BP_T) bt_plane_kernel(const int4 *__restrict__ tiles, Step step) {
    constexpr int MI = BM / 32, NJ = BN / 16;          // 16-row and 8-column fragments per warp
    constexpr int STAGE = N_PLANES * (BM + BN) * BP_LD;
    constexpr int CHUNKS = N_PLANES * (BM + BN) * (BP_K / 8);   // 16-byte pieces per stage
    static_assert(CHUNKS % BP_T == 0, "stage load must divide evenly over the CTA");
    extern __shared__ __align__(16) unsigned char bp_raw[];
    bf16 *sm = reinterpret_cast<bf16 *>(bp_raw);
    const int4 t = tiles[blockIdx.x];
    BtPlaneOp op;
    if (!step.setup(t.x, t.y, op)) return;   // uniform over the CTA
    const long long ps = step.a.ps;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp >> 1, wn = warp & 1, g = lane >> 2, tg = lane & 3;
    const int m0 = t.z * BM, n0 = t.w * BN;
    auto tileA = [&](int s, int q) { return sm + s * STAGE + q * BM * BP_LD; };
    auto tileB = [&](int s, int q) { return sm + s * STAGE + N_PLANES * BM * BP_LD + q * BN * BP_LD; };
    auto load_stage = [&](int s, int k0) {
#pragma unroll
        for (int q = 0; q < CHUNKS / BP_T; ++q) {
            const int idx = tid + q * BP_T;
            const int row = idx >> 2, c = (idx & 3) * 8;   // row of the stacked A planes, then B planes
            const bf16 *base;
            bf16 *dst;
            int ld, gr, lim;
            if (row < N_PLANES * BM) {
                const int pl = row / BM, r = row % BM;
                base = op.A + pl * ps; ld = op.lda; gr = m0 + r; lim = op.M; dst = tileA(s, pl) + r * BP_LD + c;
            } else {
                const int pl = (row - N_PLANES * BM) / BN, r = (row - N_PLANES * BM) % BN;
                base = op.B + pl * ps; ld = op.ldb; gr = n0 + r; lim = op.N; dst = tileB(s, pl) + r * BP_LD + c;
            }
            cp_async16(dst, base + (long long)(gr < lim ? gr : 0) * ld + k0 + c, gr < lim ? 16 : 0);
        }
        cp_async_commit();
    };
    // acc: FP32 running sums; pm: the hi x hi product of one 32-deep K slice, px: the five smaller
    // plane products (kept apart so that the tensor core's accumulation of the small terms cannot
    // shift the dominant one); both folded into acc with round-to-nearest adds every slice
    float acc[MI][NJ][4], pm[MI][NJ][4], px[MI][NJ][4];
#pragma unroll
    for (int i = 0; i < MI; ++i)
#pragma unroll
        for (int j = 0; j < NJ; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[i][j][e] = pm[i][j][e] = px[i][j][e] = 0.f;
    const int nk = op.Kpad / BP_K;
    load_stage(0, 0);
    for (int kb = 0; kb < nk; ++kb) {
        const int s = kb & 1;
        cp_async_wait_all();
        __syncthreads();
        if (kb + 1 < nk) load_stage(s ^ 1, (kb + 1) * BP_K);
#pragma unroll
        for (int kk = 0; kk < BP_K; kk += 16) {
            unsigned af[MI][N_PLANES][4];
#pragma unroll
            for (int i = 0; i < MI; ++i)
#pragma unroll
                for (int q = 0; q < N_PLANES; ++q) {
                    const bf16 *pa = tileA(s, q) + (wm * (BM / 2) + i * 16 + g) * BP_LD + kk + tg * 2;
                    af[i][q][0] = *(const unsigned *)(pa);
                    af[i][q][1] = *(const unsigned *)(pa + 8 * BP_LD);
                    af[i][q][2] = *(const unsigned *)(pa + 8);
                    af[i][q][3] = *(const unsigned *)(pa + 8 * BP_LD + 8);
                }
#pragma unroll
            for (int j = 0; j < NJ; ++j) {
                unsigned bf[N_PLANES][2];
#pragma unroll
                for (int q = 0; q < N_PLANES; ++q) {
                    const bf16 *pb = tileB(s, q) + (wn * (BN / 2) + j * 8 + g) * BP_LD + kk + tg * 2;
                    bf[q][0] = *(const unsigned *)(pb);
                    bf[q][1] = *(const unsigned *)(pb + 8);
                }
#pragma unroll
                for (int i = 0; i < MI; ++i) {
                    mma_bf16(pm[i][j], af[i][0], bf[0]);
                    mma_bf16(px[i][j], af[i][0], bf[1]);
                    mma_bf16(px[i][j], af[i][1], bf[0]);
                    mma_bf16(px[i][j], af[i][0], bf[2]);
                    mma_bf16(px[i][j], af[i][2], bf[0]);
                    mma_bf16(px[i][j], af[i][1], bf[1]);
                }
            }
        }
#pragma unroll
        for (int i = 0; i < MI; ++i)
#pragma unroll
            for (int j = 0; j < NJ; ++j)
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    acc[i][j][e] += pm[i][j][e] + px[i][j][e];
                    pm[i][j][e] = px[i][j][e] = 0.f;
                }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < MI; ++i)
#pragma unroll
        for (int j = 0; j < NJ; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int m = m0 + wm * (BM / 2) + i * 16 + g + (e >= 2 ? 8 : 0);
                const int n = n0 + wn * (BN / 2) + j * 8 + tg * 2 + (e & 1);
                if (m < op.M && n < op.N) step.epi(op, m, n, acc[i][j][e]);
            }
}

__device__ __forceinline__ void bt_split_store(const BtArrays &a, long long k, float x) { store3(a.P, a.ps, k, x); }

// plane pointers of an instance
__device__ __forceinline__ long long bt_pc_rv(const BtInst &in) { return in.off_pc + 2LL * in.n * in.ko; }
__device__ __forceinline__ long long bt_pc_rswt(const BtInst &in) { return bt_pc_rv(in) + 2LL * in.n * in.kv; }
__device__ __forceinline__ long long bt_pc_lswt(const BtInst &in) { return bt_pc_rswt(in) + (long long)in.v * in.k2; }
__device__ __forceinline__ long long bt_pv_slot(const BtInst &in, int b) {
    return in.off_pv + (long long)b * ((long long)in.v * in.ko + 2LL * in.n * in.kv + 2LL * in.n * in.k2 +
                                       (long long)in.v * in.k2);
}
__device__ __forceinline__ long long bt_pv_h(const BtInst &in, int b) { return bt_pv_slot(in, b) + (long long)in.v * in.ko; }
__device__ __forceinline__ long long bt_pv_f(const BtInst &in, int b) { return bt_pv_h(in, b) + 2LL * in.n * in.kv; }
__device__ __forceinline__ long long bt_pv_gt(const BtInst &in, int b) { return bt_pv_f(in, b) + 2LL * in.n * in.k2; }

// constant planes of every instance (set-up of the mixed form)
__global__ void bt_const_planes_kernel(BtArrays a) {
    const BtInst in = a.inst[blockIdx.x];
    const int n = in.n, o = in.o, v = in.v, n2 = 2 * n;
    const double *lst = a.blk + in.off_blk, *rv = lst + 2LL * n * o, *lsw = rv + 2LL * n * v, *rsw = lsw + 2LL * n * o;
    for (long long t = threadIdx.x; t < (long long)n2 * o; t += blockDim.x) {
        const int r = int(t / o), c = int(t % o);
        bt_split_store(a, in.off_pc + (long long)r * in.ko + c, (float)lst[t]);
        bt_split_store(a, bt_pc_lswt(in) + (long long)c * in.k2 + r, (float)lsw[t]);
    }
    for (long long t = threadIdx.x; t < (long long)n2 * v; t += blockDim.x) {
        const int r = int(t / v), c = int(t % v);
        bt_split_store(a, bt_pc_rv(in) + (long long)r * in.kv + c, (float)rv[t]);
        bt_split_store(a, bt_pc_rswt(in) + (long long)c * in.k2 + r, (float)rsw[t]);
    }
}

// X^T planes of the new trial vectors (or of the Ritz vectors in the final pass)
__global__ void bt_split_x_kernel(BtArrays a, int I0, int final_pass) {
    const int I = I0 + blockIdx.y, b = blockIdx.x;
    const BtInst in = a.inst[I];
    const double *X;
    if (!bt_vector(a, in, I, b, final_pass != 0, &X)) return;
    const long long base = bt_pv_slot(in, b);
    for (long long t = threadIdx.x; t < in.ov; t += blockDim.x) {
        const int i = int(t / in.v), x = int(t % in.v);
        bt_split_store(a, base + (long long)x * in.ko + i, (float)X[t]);
    }
}

// 1. H = [C_o;SC_o] X: FP64 copy (Coulomb diagonals) and planes
struct BtP1 {
    BtArrays a;
    bool final_pass;   // Ritz vectors: the transition charges after convergence
    __device__ bool setup(int I, int b, BtPlaneOp &op) const {
        const BtInst &in = a.inst[I];
        const double *X;
        if (!bt_vector(a, in, I, b, final_pass, &X)) return false;
        op.in = &a.inst[I]; op.I = I; op.b = b;
        op.M = 2 * in.n; op.N = in.v; op.Kpad = in.ko;
        op.A = a.P + in.off_pc; op.lda = in.ko;
        op.B = a.P + bt_pv_slot(in, b); op.ldb = in.ko;
        return true;
    }
    __device__ void epi(const BtPlaneOp &op, int m, int n, float acc) const {
        const BtInst &in = *op.in;
        if (final_pass || !in.lc || in.nh)
            a.H[in.off_h + (long long)op.b * 2 * in.n * in.v + (long long)m * in.v + n] = (double)acc;
        bt_split_store(a, bt_pv_h(in, op.b) + (long long)m * in.kv + n, acc);
    }
};

// 2. F = -1/4 gamma_lr o (H [C_v;SC_v]^T) as planes (LC instances)
struct BtP2 {
    BtArrays a;
    __device__ bool setup(int I, int b, BtPlaneOp &op) const {
        const BtInst &in = a.inst[I];
        const double *X;
        if (!in.lc || !bt_vector(a, in, I, b, false, &X)) return false;
        op.in = &a.inst[I]; op.I = I; op.b = b;
        op.M = 2 * in.n; op.N = 2 * in.n; op.Kpad = in.kv;
        op.A = a.P + bt_pv_h(in, b); op.lda = in.kv;
        op.B = a.P + bt_pc_rv(in); op.ldb = in.kv;
        return true;
    }
    __device__ void epi(const BtPlaneOp &op, int r, int c, float acc) const {
        const BtInst &in = *op.in;
        const int n = in.n;
        const int rr = r < n ? r : r - n, cc = c < n ? c : c - n;
        if (!in.nh) {   // Coulomb diagonals of M from the same accumulator (bt_diag_kernel otherwise)
            double *d = a.D + in.off_d;
            if (r < n && c == r + n) d[(long long)op.b * n + r] = (double)acc;
            if (r >= n && c == r - n) d[(long long)(in.nr + op.b) * n + c] = (double)acc;
        }
        const float f = -0.25f * a.glr32[in.off_glr + (long long)rr * n + cc] * acc;
        bt_split_store(a, bt_pv_f(in, op.b) + (long long)r * in.k2 + c, f);
    }
};

// 4. G = F [SC_v;C_v] + diag(z, z) [C_v;SC_v], written transposed as planes (LC instances)
struct BtP4 {
    BtArrays a;
    __device__ bool setup(int I, int b, BtPlaneOp &op) const {
        const BtInst &in = a.inst[I];
        const double *X;
        if (!in.lc || !bt_vector(a, in, I, b, false, &X)) return false;
        op.in = &a.inst[I]; op.I = I; op.b = b;
        op.M = 2 * in.n; op.N = in.v; op.Kpad = in.k2;
        op.A = a.P + bt_pv_f(in, b); op.lda = in.k2;
        op.B = a.P + bt_pc_rswt(in); op.ldb = in.k2;
        return true;
    }
    __device__ void epi(const BtPlaneOp &op, int r, int x, float acc) const {
        const BtInst &in = *op.in;
        const int n = in.n;
        const float z = a.D32[in.off_d + (long long)(2 * in.nr + op.b) * n + (r < n ? r : r - n)];
        const float rv = a.blk32[in.off_blk + 2LL * n * in.o + (long long)r * in.v + x];
        bt_split_store(a, bt_pv_gt(in, op.b) + (long long)x * in.k2 + r, acc + z * rv);
    }
};

// non-LC: G = diag(z, z) [C_v;SC_v] as transposed planes
__global__ void bt_gt_nolc_kernel(BtArrays a, int I0) {
    const int I = I0 + blockIdx.y, b = blockIdx.x;
    const BtInst in = a.inst[I];
    const double *X;
    if (in.lc || !bt_vector(a, in, I, b, false, &X)) return;
    const int n = in.n, v = in.v;
    const double *z = a.D + in.off_d + (long long)(2 * in.nr + b) * n;
    const double *rv = a.blk + in.off_blk + 2LL * n * in.o;
    for (long long t = threadIdx.x; t < 2LL * n * v; t += blockDim.x) {
        const int r = int(t / v), x = int(t % v);
        bt_split_store(a, bt_pv_gt(in, b) + (long long)x * in.k2 + r, (float)(z[r < n ? r : r - n] * rv[t]));
    }
}

// 5. AX = [SC_o;C_o]^T G + omega o X
struct BtP5 {
    BtArrays a;
    __device__ bool setup(int I, int b, BtPlaneOp &op) const {
        const BtInst &in = a.inst[I];
        const double *X;
        if (!bt_vector(a, in, I, b, false, &X)) return false;
        op.in = &a.inst[I]; op.I = I; op.b = b; op.X = X;
        op.M = in.o; op.N = in.v; op.Kpad = in.nh ? in.k5 : in.k2;   // rows n+nh.. of G meet C_o = 0
        op.A = a.P + bt_pc_lswt(in); op.lda = in.k2;
        op.B = a.P + bt_pv_gt(in, b); op.ldb = in.k2;
        return true;
    }
    __device__ void epi(const BtPlaneOp &op, int m, int n, float acc) const {
        const BtInst &in = *op.in;
        const long long k = (long long)m * in.v + n;
        const BtState &s = a.state[op.I];
        a.AV[in.off_v + (long long)(s.m_done + op.b) * in.ov + k] = (double)acc + a.omega[in.off_omega + k] * op.X[k];
    }
};

// restart every instance from its Ritz vectors (FP64 polish after the mixed phase)
__global__ void bt_restart_kernel(BtArrays a) {
    const int I = blockIdx.x;
    const BtInst in = a.inst[I];
    const BtState old = a.state[I];
    if (old.status == BT_NONFINITE) return;
    double *V = a.V + in.off_v;
    const double *R = a.R + in.off_r;
    for (long long t = threadIdx.x; t < (long long)in.nr * in.ov; t += blockDim.x) V[t] = R[t];
    if (threadIdx.x == 0) {
        BtState s{};
        s.m = in.nr;
        s.m_done = 0;
        s.dim_sub = in.nr;
        s.iter = old.iter;
        s.status = BT_RUNNING;
        s.products = old.products;
        s.collapses = old.collapses;
        s.first_stop = 1;
        a.state[I] = s;
    }
}

// Device-side control of the iteration loop (a CUDA graph WHILE node replays one iteration until
// no instance runs).  loop[0] = iterations run in the current phase, loop[1] = its limit,
// loop[2] = iterations of the phase before (the mixed phase, when an FP64 phase follows it).
__global__ void bt_loop_init_kernel(int *loop, int limit, int after_prev) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int prev = after_prev ? loop[0] : 0;
    loop[2] = prev;
    loop[1] = after_prev ? max(1, limit - prev) : max(1, limit);
    loop[0] = 0;
}

// End of one iteration: count it and keep the loop going while an instance runs and the limit is
// not reached (the same rule as a host loop reading the running count after every iteration).
__global__ void bt_loop_next_kernel(const int *active, int *loop, cudaGraphConditionalHandle handle) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int its = loop[0] + 1;
    loop[0] = its;
    cudaGraphSetConditional(handle, (*active > 0 && its < loop[1]) ? 1u : 0u);
}

// ----------------------------------------------------------------------------------------------
// subspace step
// ----------------------------------------------------------------------------------------------

// sum over the CTA of NV values per thread; every thread receives the totals.  The warp partials
// are added by NV lanes of warp 0 only (GB300's FP64 unit takes ~64 cycles per warp instruction, so
// the adds are not repeated in every warp).  red: (BT_T / 32 + 1) * NV doubles.
template <int NV>
__device__ __forceinline__ void bt_block_sum(double (&v)[NV], double *red) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int q = 0; q < NV; ++q)
        for (int off = 16; off; off >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], off);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) red[warp * NV + q] = v[q];
    __syncthreads();
    double *tot = red + (BT_T / 32) * NV;
    if (threadIdx.x < NV) {
        double s = 0.0;
        for (int w = 0; w < BT_T / 32; ++w) s += red[w * NV + threadIdx.x];
        tot[threadIdx.x] = s;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NV; ++q) v[q] = tot[q];
    __syncthreads();
}

// sum over the CTA of eight values per thread; every thread receives the totals.  Within a warp the
// eight sums are reduced by halving exchanges (lanes 0-15 keep values 0-3 and receive them from lanes
// 16-31, and so on): 9 shuffle-adds instead of 40.  red: (BT_T / 32 + 1) * 8 doubles.
__device__ __forceinline__ void bt_block_sum8(double (&v)[8], double *red) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool h16 = lane & 16, h8 = lane & 8, h4 = lane & 4;
    double a[4], b[2], c;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const double send = h16 ? v[q] : v[q + 4], keep = h16 ? v[q + 4] : v[q];
        a[q] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const double send = h8 ? a[q] : a[q + 2], keep = h8 ? a[q + 2] : a[q];
        b[q] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
    {
        const double send = h4 ? b[0] : b[1], keep = h4 ? b[1] : b[0];
        c = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
    c += __shfl_xor_sync(0xffffffffu, c, 2);
    c += __shfl_xor_sync(0xffffffffu, c, 1);
    // lane L now holds the warp total of value (L >> 2) & 7
    __syncthreads();
    if ((lane & 3) == 0) red[warp * 8 + ((lane >> 2) & 7)] = c;
    __syncthreads();
    double *tot = red + (BT_T / 32) * 8;
    if (threadIdx.x < 8) {
        double s = 0.0;
        for (int w = 0; w < BT_T / 32; ++w) s += red[w * 8 + threadIdx.x];
        tot[threadIdx.x] = s;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = tot[q];
    __syncthreads();
}

// Number of eigenvalues of the symmetric tridiagonal (d, squared off-diagonal esq) below x: the
// sign changes of the leading principal minors N_i = (d_i - x) N_{i-1} - e_{i-1}^2 N_{i-2}, a
// division-free recurrence (3 FP64 operations per row instead of a division), rescaled by a power
// of two when N_i leaves [2^-400, 2^400]; an exact zero becomes a tiny value of the other sign.
__device__ __forceinline__ int bt_sturm(const double *d, const double *esq, int m, double x) {
    double n0 = 1.0, n1 = d[0] - x;
    if (n1 == 0.0) n1 = -0x1p-100;
    int c = __double2hiint(n1) < 0;
    for (int i = 1; i < m; ++i) {
        double n2 = fma(d[i] - x, n1, -(esq[i - 1] * n0));
        const long long bits = __double_as_longlong(n2);
        if ((bits << 1) == 0) {
            n2 = -0x1p-100 * n1;
        } else {
            const int ex = (int)((bits >> 52) & 0x7ff);
            if ((ex > 1023 + 400 || ex < 1023 - 400) && ex < 2047) {
                const double sc = __longlong_as_double((long long)(2046 - ex) << 52);   // 2^(1023 - ex)
                n1 *= sc;
                n2 *= sc;
            }
        }
        c += (int)(((unsigned)__double2hiint(n1) ^ (unsigned)__double2hiint(n2)) >> 31);
        n0 = n1;
        n1 = n2;
    }
    return c;
}

// Lowest nr eigenpairs of the symmetric m x m matrix A (shared memory, overwritten), all in FP64:
// Householder reduction to tridiagonal form T = Q^T A Q (Householder vectors kept in A's lower
// triangle), the nr smallest eigenvalues of T by warp multisection on Sturm counts (one warp per
// root, 33 points per step), their eigenvectors by inverse iteration on T (LU with partial
// pivoting), Gram-Schmidt among them, and the back-transformation y = Q z.
// Out: w[r] ascending; Y[r * m + i] orthonormal eigenvectors.  W: scratch of 4 m + 5 nr m doubles.
__device__ void bt_eig_lowest(int m, int nr, double *A, double *W, double *w, double *red) {
    double *d = W, *e = d + m, *beta = e + m, *p = beta + m, *Y = p + m, *F = Y + (size_t)nr * m;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // 1. tridiagonalisation (one reflection per column k, acting on rows/columns k+1..m-1).  Four
    //    barriers per column; the FP64 latency chains are kept short: the column norm, the
    //    reflection scalars and u^T p on warp 0 alone (shuffle reductions, no cross-warp step), and
    //    p = bet A' u with G threads per row (G = 8, 4, 2 for trailing blocks up to 32, 64, 128 rows).
    for (int k = 0; k + 2 < m; ++k) {
        const int n1 = m - k - 1;
        double *u = A + (size_t)(k + 1) * m + k;   // u_i = u[i * m], i < n1 (column k below the diagonal)
        if (warp == 0) {
            double s2 = 0.0;
            for (int i = 1 + lane; i < n1; i += 32) s2 += u[(size_t)i * m] * u[(size_t)i * m];
            for (int off = 16; off; off >>= 1) s2 += __shfl_xor_sync(0xffffffffu, s2, off);
            if (lane == 0) {   // H = I - bet u u^T, u = x - alpha e_1
                const double x0 = u[0];
                d[k] = A[(size_t)k * m + k];
                if (s2 == 0.0) {
                    beta[k] = 0.0;
                    e[k] = x0;
                } else {
                    const double nx = sqrt(x0 * x0 + s2);
                    const double alpha = x0 > 0.0 ? -nx : nx;
                    u[0] = x0 - alpha;
                    beta[k] = 1.0 / (alpha * (alpha - x0));
                    e[k] = alpha;
                }
            }
        }
        __syncthreads();
        const double bet = beta[k];
        if (bet == 0.0) continue;   // the same in every thread
        {
            const int G = n1 <= 32 ? 8 : n1 <= 64 ? 4 : 2;
            const int row = tid / G, sub = tid % G;
            double acc = 0.0;
            if (row < n1) {
                const double *ar = A + (size_t)(k + 1 + row) * m + (k + 1);
                for (int j = sub; j < n1; j += G) acc += ar[j] * u[(size_t)j * m];
            }
            for (int off = G >> 1; off; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
            if (sub == 0 && row < n1) p[row] = bet * acc;
        }
        __syncthreads();
        if (warp == 0) {   // q = p - K u, K = bet u^T p / 2
            double up = 0.0;
            for (int i = lane; i < n1; i += 32) up += u[(size_t)i * m] * p[i];
            for (int off = 16; off; off >>= 1) up += __shfl_xor_sync(0xffffffffu, up, off);
            const double K = 0.5 * bet * up;
            for (int i = lane; i < n1; i += 32) p[i] -= K * u[(size_t)i * m];
        }
        __syncthreads();
        for (int t = tid; t < n1 * n1; t += BT_T) {          // A' -= u q^T + q u^T
            const int i = t / n1, j = t % n1;
            A[(size_t)(k + 1 + i) * m + (k + 1 + j)] -= u[(size_t)i * m] * p[j] + p[i] * u[(size_t)j * m];
        }
        __syncthreads();
    }
    if (tid == 0) {
        if (m >= 2) {
            d[m - 2] = A[(m - 2) * m + m - 2];
            e[m - 2] = A[(m - 1) * m + m - 2];
        }
        d[m - 1] = A[(m - 1) * m + m - 1];
        e[m - 1] = 0.0;
    }
    __syncthreads();
    // 2. eigenvalues: Gershgorin interval (warp 0), then multisection per root; p holds e^2
    if (warp == 0) {
        double glo = 1e300, ghi = -1e300, emax2 = 0.0;
        for (int i = lane; i < m; i += 32) {
            const double r = fabs(e[i]) + (i > 0 ? fabs(e[i - 1]) : 0.0);
            glo = fmin(glo, d[i] - r);
            ghi = fmax(ghi, d[i] + r);
            p[i] = e[i] * e[i];
            emax2 = fmax(emax2, p[i]);
        }
        for (int off = 16; off; off >>= 1) {
            glo = fmin(glo, __shfl_xor_sync(0xffffffffu, glo, off));
            ghi = fmax(ghi, __shfl_xor_sync(0xffffffffu, ghi, off));
            emax2 = fmax(emax2, __shfl_xor_sync(0xffffffffu, emax2, off));
        }
        if (lane == 0) {
            red[0] = glo;
            red[1] = ghi;
            red[2] = emax2;
        }
    }
    __syncthreads();
    const double eps = 2.220446049250313e-16;
    const double tnorm = fmax(fabs(red[0]), fabs(red[1]));
    const double pivmin = 2.2250738585072014e-308 * fmax(1.0, red[2]);
    const double lo = red[0] - (2.0 * eps * tnorm + 2.0 * pivmin);
    const double hi = red[1] + (2.0 * eps * tnorm + 2.0 * pivmin);
    if (warp < nr) {
        const int r = warp;
        double a = lo, b = hi;
        for (int it = 0; it < 64; ++it) {
            if (b - a <= 2.0 * eps * fmax(fabs(a), fabs(b)) + 4.0 * pivmin) break;
            const double h = (b - a) * (1.0 / 33.0);
            const double x = a + h * (lane + 1);
            const unsigned ball = __ballot_sync(0xffffffffu, bt_sturm(d, p, m, x) > r);
            if (ball == 0u) {
                a = __shfl_sync(0xffffffffu, x, 31);
            } else {
                const int f = __ffs(ball) - 1;
                const double xf = __shfl_sync(0xffffffffu, x, f);
                const double xp = __shfl_sync(0xffffffffu, x, f > 0 ? f - 1 : 0);
                if (f > 0) a = xp;
                b = xf;
            }
        }
        if (lane == 0) w[r] = 0.5 * (a + b);
    }
    __syncthreads();
    // 3. inverse iteration for each root (lane 0 of warp r), on T - w_r I
    if (warp < nr && lane == 0) {
        const int r = warp;
        const double lam = w[r];
        double *z = Y + (size_t)r * m;
        double *dl = F + (size_t)r * 4 * m, *dd = dl + m, *du = dd + m, *du2 = du + m;
        const double tiny = eps * fmax(tnorm, 1e-300);
        for (int i = 0; i < m; ++i) {
            dd[i] = d[i] - lam;
            dl[i] = e[i];
            du[i] = e[i];
            du2[i] = 0.0;
        }
        unsigned long long swp = 0, swp2 = 0;   // row interchanges (bit i)
        // dd[i] receives the reciprocal of pivot i (one division per row; the solves only multiply)
        for (int i = 0; i + 1 < m; ++i) {
            if (fabs(dd[i]) >= fabs(dl[i])) {
                if (fabs(dd[i]) < tiny) dd[i] = dd[i] < 0.0 ? -tiny : tiny;
                const double rp = 1.0 / dd[i];
                const double l = dl[i] * rp;
                dd[i] = rp;
                dl[i] = l;
                dd[i + 1] -= l * du[i];
            } else {
                const double rp = 1.0 / dl[i];
                const double l = dd[i] * rp;
                dd[i] = rp;
                dl[i] = l;
                const double t = du[i];
                du[i] = dd[i + 1];
                dd[i + 1] = t - l * dd[i + 1];
                if (i + 2 < m) {
                    du2[i] = du[i + 1];
                    du[i + 1] = -l * du[i + 1];
                }
                if (i < 64) swp |= 1ull << i; else swp2 |= 1ull << (i - 64);
            }
        }
        if (fabs(dd[m - 1]) < tiny) dd[m - 1] = dd[m - 1] < 0.0 ? -tiny : tiny;
        dd[m - 1] = 1.0 / dd[m - 1];
        for (int i = 0; i < m; ++i) z[i] = 1.0 + 0.5 * (double)((i * (r + 1) * 7919 + 13 * r) % 97) / 97.0;
        for (int it = 0; it < 3; ++it) {
            for (int i = 0; i + 1 < m; ++i) {            // L^-1 with the interchanges
                const bool sw = i < 64 ? ((swp >> i) & 1ull) : ((swp2 >> (i - 64)) & 1ull);
                if (sw) { const double t = z[i]; z[i] = z[i + 1]; z[i + 1] = t; }
                z[i + 1] -= dl[i] * z[i];
            }
            for (int i = m - 1; i >= 0; --i) {           // U^-1
                double s = z[i];
                if (i + 1 < m) s -= du[i] * z[i + 1];
                if (i + 2 < m) s -= du2[i] * z[i + 2];
                z[i] = s * dd[i];
            }
            double nrm = 0.0;
            for (int i = 0; i < m; ++i) nrm += z[i] * z[i];
            nrm = 1.0 / sqrt(nrm);
            for (int i = 0; i < m; ++i) z[i] *= nrm;
        }
    }
    __syncthreads();
    // Gram-Schmidt of the roots in ascending order (separates vectors of (near-)degenerate roots),
    // warp 0 with lanes over the components
    if (warp == 0) {
        for (int r = 1; r < nr; ++r) {
            double *z = Y + (size_t)r * m;
            for (int pass = 0; pass < 2; ++pass)
                for (int q = 0; q < r; ++q) {
                    const double *y = Y + (size_t)q * m;
                    double s = 0.0;
                    for (int i = lane; i < m; i += 32) s += y[i] * z[i];
                    for (int off = 16; off; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
                    for (int i = lane; i < m; i += 32) z[i] -= s * y[i];
                    __syncwarp();
                }
            double nrm = 0.0;
            for (int i = lane; i < m; i += 32) nrm += z[i] * z[i];
            for (int off = 16; off; off >>= 1) nrm += __shfl_xor_sync(0xffffffffu, nrm, off);
            nrm = 1.0 / sqrt(nrm);
            for (int i = lane; i < m; i += 32) z[i] *= nrm;
            __syncwarp();
        }
    }
    __syncthreads();
    // 4. back-transformation y = H_0 H_1 ... H_{m-3} z (warp r, reflections in reverse order)
    if (warp < nr) {
        double *z = Y + (size_t)warp * m;
        for (int k = m - 3; k >= 0; --k) {
            const double bet = beta[k];
            if (bet == 0.0) continue;
            const int n1 = m - k - 1;
            double s = 0.0;
            for (int i = lane; i < n1; i += 32) s += A[(k + 1 + i) * m + k] * z[k + 1 + i];
            for (int off = 16; off; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
            for (int i = lane; i < n1; i += 32) z[k + 1 + i] -= bet * s * A[(k + 1 + i) * m + k];
            __syncwarp();
        }
    }
    __syncthreads();
}

// The subspace step runs on thread-block clusters of BT_CL CTAs.  A heavy instance (several roots
// on a long vector) takes a whole cluster: its CTAs own interleaved blocks of BT_T components of
// every ov-long vector and combine their partial sums through distributed shared memory (added in
// rank order, so every CTA holds the same bits and takes the same decisions); the small
// eigenproblem is solved by the cluster's first CTA and copied by the others.  Light instances (one CT root) take one CTA each, four to a
// cluster, where splitting would repeat the eigensolver more than it divides the vector work.
constexpr int BT_CL = 4;

// shared memory of the subspace kernel for subspaces up to mmax: the projected matrix, eigensolver
// scratch (4 m + 5 nr m <= mmax^2 doubles since mmax = 15 nr), reductions, Gram-Schmidt dots, two
// cluster exchange buffers and the new projected columns
inline size_t bt_subspace_smem(int mmax) {
    const size_t cb = (size_t)mmax * BT_MAXR + 8;
    return (2 * (size_t)mmax * mmax + 8 * BT_MAXR * (BT_T / 32) + mmax + BT_MAXR + 16 + BT_MAXR + 3 * cb) *
           sizeof(double);
}

// Sum over the cluster's CTAs of the n values each CTA holds in `mine` (shared memory): out[k] =
// the partials of ranks 0, 1, ... added in that order, so every CTA receives the same bits (a CTA
// working alone copies its values).  Callers alternate between two `mine` buffers: a CTA writes a
// buffer again only after the next call's cluster barrier, which every CTA reaches after its reads
// of this call.
__device__ __forceinline__ void bt_cluster_sum(const cg::cluster_group &cl, bool coop, double *mine, int n,
                                               double *out) {
    if (coop) cl.sync();
    else __syncthreads();
    for (int k = threadIdx.x; k < n; k += BT_T) {
        double s = mine[k];
        if (coop) {
            s = 0.0;
#pragma unroll
            for (int r = 0; r < BT_CL; ++r) s += *cl.map_shared_rank(mine + k, r);
        }
        out[k] = s;
    }
    __syncthreads();
}

// heavy instances (about nr^2 ov FP64 work per iteration at or above this) take a whole cluster in
// the subspace step
constexpr long long BT_HEAVY = 8192;

// Ritz vectors and residuals of NR roots over this CTA's components (x0, x0 + xs, ...);
// sq[r] += |Rk_r|^2 partials
template <int NR>
__device__ __forceinline__ void bt_ritz(int m, long long ov, long long x0, long long xs, const double *V,
                                        const double *AV, const double *Yev, const double *u, double *R, double *Rk,
                                        double (&sq)[BT_MAXR]) {
    for (long long x = x0; x < ov; x += xs) {
        double rv[NR], av[NR];
#pragma unroll
        for (int r = 0; r < NR; ++r) rv[r] = av[r] = 0.0;
        for (int i = 0; i < m; ++i) {
            const double vi = V[(long long)i * ov + x], ai = AV[(long long)i * ov + x];
#pragma unroll
            for (int r = 0; r < NR; ++r) {
                const double y = Yev[r * m + i];
                rv[r] += y * vi;
                av[r] += y * ai;
            }
        }
#pragma unroll
        for (int r = 0; r < NR; ++r) {
            const double rk = av[r] - u[r] * rv[r];
            R[(long long)r * ov + x] = rv[r];
            Rk[(long long)r * ov + x] = rk;
            sq[r] += rk * rk;
        }
    }
}

// cl_inst[c]: the work of cluster c, {I, -1, -1, -1} with .y = -2 for one heavy instance I on the
// whole cluster, or up to four light instances (-1 = none), one per CTA
__global__ void __cluster_dims__(BT_CL, 1, 1) __launch_bounds__(BT_T)
    bt_subspace_kernel(BtArrays a, const int4 *__restrict__ cl_inst) {
    const cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const int4 cw = cl_inst[blockIdx.x / BT_CL];
    const bool coop = cw.y == -2;
    const int I = coop ? cw.x : rank == 0 ? cw.x : rank == 1 ? cw.y : rank == 2 ? cw.z : cw.w;
    if (I < 0) return;                     // light cluster with fewer than four instances
    const int part_rank = coop ? rank : 0, ncl = coop ? BT_CL : 1;
    const bool lead = part_rank == 0;      // writes the instance's shared results
    const int tid = threadIdx.x;
    const BtInst in = a.inst[I];
    __shared__ BtState st;
    __shared__ int s_sel[BT_MAXR], s_nsel, s_action, s_mcur;
    __shared__ double s_u[BT_MAXR], s_err[BT_MAXR], s_sq[BT_MAXR], s_nrm;
    if (tid == 0) st = a.state[I];
    __syncthreads();
    if (st.status != BT_RUNNING) return;   // the same state in every CTA of a heavy instance's cluster
    const long long ov = in.ov;
    const long long x0 = (long long)part_rank * BT_T + tid, xs = (long long)ncl * BT_T;   // this CTA's components
    const int nr = in.nr, mmax = in.mmax;
    double *V = a.V + in.off_v, *AV = a.AV + in.off_v;
    double *R = a.R + in.off_r, *Rk = a.Rk + in.off_r, *T = a.T + in.off_r;
    double *P = a.sub + in.off_sub;
    const double *om = a.omega + in.off_omega;
    const int m = st.m, m_done = st.m_done;

    extern __shared__ double smem[];
    const size_t cbn = (size_t)mmax * BT_MAXR + 8;
    double *A = smem, *Z = A + (size_t)mmax * mmax;
    double *red = Z + (size_t)mmax * mmax;
    double *cdot = red + 8 * BT_MAXR * (BT_T / 32);
    double *wev = cdot + mmax + BT_MAXR + 16;
    double *cbuf[2] = {wev + BT_MAXR, wev + BT_MAXR + cbn};
    double *pnew = cbuf[1] + cbn;
    int ph = 0;   // exchange buffer of the next cluster sum

    // 1. new columns of the projected matrix: P[i][j] = V_i . AV_j, j in [m_done, m), one warp per
    //    entry over this CTA's components, summed over the cluster
    const int kn = m - m_done;
    {
        const int warp = tid >> 5, lane = tid & 31, nw = BT_T / 32;
        double *part = cbuf[ph];
        for (int e = warp; e < m * kn; e += nw) {
            const int i = e / kn, j = m_done + e % kn;
            const double *x = V + (long long)i * ov, *y = AV + (long long)j * ov;
            double s = 0.0;
            for (long long b0 = (long long)part_rank * BT_T; b0 < ov; b0 += xs)
                for (int l = lane; l < BT_T; l += 32) {
                    const long long t = b0 + l;
                    if (t < ov) s += x[t] * y[t];
                }
            for (int off = 16; off; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
            if (lane == 0) part[e] = s;
        }
        bt_cluster_sum(cl, coop, part, m * kn, pnew);
        ph ^= 1;
    }
    if (lead)
        for (int e = tid; e < m * kn; e += BT_T) P[(long long)(e / kn) * mmax + m_done + e % kn] = pnew[e];
    // 2. eigenpairs of the upper triangle (davidson.rs:89-93): old columns from the previous
    //    iterations, new ones from this step.  The lead CTA solves; the other CTAs of a heavy
    //    instance's cluster copy its eigenpairs.
    double *Yev = Z + 4 * m;   // eigenvector r at Yev[r * m + i]
    if (lead) {
        for (int e = tid; e < m * m; e += BT_T) {
            const int i = e / m, j = e % m, lo = i < j ? i : j, hi = i < j ? j : i;
            A[e] = hi >= m_done ? pnew[lo * kn + hi - m_done] : P[(long long)lo * mmax + hi];
        }
        __syncthreads();
        bt_eig_lowest(m, nr, A, Z, wev, red);
    }
    if (coop) {
        cl.sync();   // the lead's eigenpairs are final (it does not write them again in this step)
        if (!lead) {
            const double *yr = cl.map_shared_rank(Yev, 0), *wr = cl.map_shared_rank(wev, 0);
            for (int e = tid; e < nr * m; e += BT_T) Yev[e] = yr[e];
            if (tid < nr) wev[tid] = wr[tid];
        }
    }
    if (tid < nr) s_u[tid] = wev[tid];
    __syncthreads();
    // 3. Ritz vectors R_r = sum_i y_ir V_i and residuals Rk_r = sum_i y_ir AV_i - u_r R_r (:101-107),
    //    with the loop over roots instantiated for this instance's count (no predicated FP64 work)
    double sq[BT_MAXR];
#pragma unroll
    for (int r = 0; r < BT_MAXR; ++r) sq[r] = 0.0;
    switch (nr) {
    case 1: bt_ritz<1>(m, ov, x0, xs, V, AV, Yev, s_u, R, Rk, sq); break;
    case 2: bt_ritz<2>(m, ov, x0, xs, V, AV, Yev, s_u, R, Rk, sq); break;
    case 3: bt_ritz<3>(m, ov, x0, xs, V, AV, Yev, s_u, R, Rk, sq); break;
    case 4: bt_ritz<4>(m, ov, x0, xs, V, AV, Yev, s_u, R, Rk, sq); break;
    case 5: bt_ritz<5>(m, ov, x0, xs, V, AV, Yev, s_u, R, Rk, sq); break;
    default: bt_ritz<BT_MAXR>(m, ov, x0, xs, V, AV, Yev, s_u, R, Rk, sq); break;
    }
    bt_block_sum<BT_MAXR>(sq, red);
    if (tid < BT_MAXR) cbuf[ph][tid] = sq[tid];
    bt_cluster_sum(cl, coop, cbuf[ph], BT_MAXR, s_sq);
    ph ^= 1;
    // 4. convergence and the next action (:109-178), taken identically by every CTA
    if (tid == 0) {
        st.products += m - m_done;
        int cvd = 0;
        bool finite = true;
        double mx = 0.0;
        for (int r = 0; r < nr; ++r) {
            const double e = sqrt(s_sq[r]);
            s_err[r] = e;
            if (lead) {
                a.u[in.off_u + r] = s_u[r];
                a.err[in.off_u + r] = e;
            }
            if (!isfinite(e) || !isfinite(s_u[r])) finite = false;
            if (e < a.tol) ++cvd;
            mx = fmax(mx, e);
        }
        st.max_res = mx;
        const int lft = nr - cvd;
        const int it = st.iter;
        st.iter = it + 1;
        s_action = 0;
        if (!finite) {
            st.status = BT_NONFINITE;
        } else if (lft == 0 && (it > 0 || st.first_stop)) {
            st.status = BT_CONVERGED;
        } else if (it == in.max_iter - 1) {
            st.status = BT_MAXITER;
        } else if (st.dim_sub + lft <= mmax) {
            int k = 0;
            for (int r = 0; r < nr; ++r)
                if (s_err[r] > a.tol) s_sel[k++] = r;   // roots to expand (:150-157); reuses s_sel
            s_nsel = k;
            st.dim_sub += lft;
            s_action = 1;
        } else {
            s_action = 2;
        }
        st.m_done = m;
        s_mcur = m;
    }
    __syncthreads();
    if (s_action == 1) {
        // 5. preconditioned residuals (solvers/mod.rs:373-380), then classical Gram-Schmidt of each
        //    against the growing basis with tincr's 1e-8 drop rule (:162-168)
        const int kadd = s_nsel;
        for (int j = 0; j < kadd; ++j) {
            const int r = s_sel[j];
            const double w = s_u[r];
            for (long long x = x0; x < ov; x += xs) {
                double d = w - om[x];
                if (fabs(d) < 1.0e-4) d = 1.0;
                T[(long long)j * ov + x] = Rk[(long long)r * ov + x] / d;
            }
        }
        __syncthreads();
        for (int j = 0; j < kadd; ++j) {
            double *t = T + (long long)j * ov;
            const int mc = s_mcur;
            double *part = cbuf[ph];
            for (int i0 = 0; i0 < mc; i0 += 8) {
                double c8[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) c8[q] = 0.0;
                for (long long x = x0; x < ov; x += xs) {
                    const double tx = t[x];
#pragma unroll
                    for (int q = 0; q < 8; ++q)
                        if (i0 + q < mc) c8[q] += V[(long long)(i0 + q) * ov + x] * tx;
                }
                bt_block_sum8(c8, red);
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    if (tid == q) part[i0 + q] = c8[q];
            }
            bt_cluster_sum(cl, coop, part, mc, cdot);
            ph ^= 1;
            double nr2[1] = {0.0};
            for (long long x = x0; x < ov; x += xs) {
                double s = t[x];
                for (int i = 0; i < mc; ++i) s -= cdot[i] * V[(long long)i * ov + x];
                t[x] = s;
                nr2[0] += s * s;
            }
            bt_block_sum<1>(nr2, red);
            if (tid == 0) cbuf[ph][0] = nr2[0];
            bt_cluster_sum(cl, coop, cbuf[ph], 1, &s_nrm);
            ph ^= 1;
            const double nrm = sqrt(s_nrm);
            if (!isfinite(nrm)) {
                if (tid == 0) st.status = BT_NONFINITE;
                break;
            }
            if (nrm > 1.0e-8 && mc < mmax) {
                const double inv = 1.0 / nrm;
                for (long long x = x0; x < ov; x += xs) V[(long long)mc * ov + x] = t[x] * inv;
                __syncthreads();
                if (tid == 0) s_mcur = mc + 1;
            }
            __syncthreads();
        }
        if (tid == 0) st.m = s_mcur;
    } else if (s_action == 2) {
        // 6. collapse onto the Ritz vectors (:172-176), this CTA's components
        for (int r = 0; r < nr; ++r)
            for (long long x = x0; x < ov; x += xs) V[(long long)r * ov + x] = R[(long long)r * ov + x];
        if (tid == 0) {
            st.dim_sub = nr;
            st.m = nr;
            st.m_done = 0;
            st.collapses += 1;
        }
    }
    if (coop) cl.sync();   // no CTA leaves while another may still read its exchange buffers
    if (tid == 0 && lead) {
        a.state[I] = st;
        if (st.status == BT_RUNNING) atomicAdd(a.active, 1);
    }
}

// ----------------------------------------------------------------------------------------------
// host
// ----------------------------------------------------------------------------------------------

// the four plane GEMM steps of the mixed product
enum BpStep { BP_P1 = 0, BP_P2 = 1, BP_P4 = 2, BP_P5 = 3, BP_STEPS = 4 };

struct BatchWork {
    std::vector<BtInst> h;
    PinnedBuf pinC, pinS, pinG, pinGlr, pinOm;   // staging of the instance inputs
    DevBuf<BtInst> inst;
    DevBuf<BtState> state;
    DevBuf<double> C, SC, S, blk, glr, glr_atoms, gam, omega, V, AV, R, Rk, T, sub, H, F, D, u, err, Y;
    DevBuf<int> ao_off, ao_atom, pos, active;
    DevBuf<int> loop;                                  // device loop control (bt_loop_init_kernel)
    DevBuf<long long> off_glr_atoms;
    DevBuf<int4> t_sc;
    // Instances run in two groups, heavy (several roots on long vectors) then light, whose
    // iterations are two concurrent branches of the iteration graph; per group:
    DevBuf<int4> t1[2], t2[2], t4[2], t5[2];           // FP64 product tiles
    size_t nt1[2] = {}, nt2[2] = {}, nt4[2] = {}, nt5[2] = {};
    DevBuf<int4> pt[2][BP_STEPS][BP_SHAPES];           // plane GEMM tiles per product step and tile shape
    size_t npt[2][BP_STEPS][BP_SHAPES] = {};
    DevBuf<int4> cl_inst[2];                           // work of each cluster of the subspace step
    DevBuf<int4> tune_tiles[BP_SHAPES];
    DevBuf<bf16> Pl;
    DevBuf<float> glr32, blk32, D32;
    cudaStream_t hi = nullptr, side = nullptr;         // branches of the heavy (high priority) and light groups
    cudaEvent_t fork = nullptr, join_hi = nullptr, join_side = nullptr;
    ~BatchWork() {
        if (fork) cudaEventDestroy(fork);
        if (join_hi) cudaEventDestroy(join_hi);
        if (join_side) cudaEventDestroy(join_side);
        if (hi) cudaStreamDestroy(hi);
        if (side) cudaStreamDestroy(side);
    }
};

template <class T>
static void upload_any(cudaStream_t st, DevBuf<T> &d, const std::vector<T> &h) {
    d.reserve(std::max<size_t>(1, h.size()));
    if (!h.empty()) TINCR_CUDA(cudaMemcpyAsync(d.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, st));
}

template <bool TA, bool TB, class Step>
static void bt_launch(Ctx &c, cudaStream_t st, const DevBuf<int4> &tiles, size_t n_tiles, const Step &step, int family,
                      double flops) {
    if (n_tiles == 0) return;
    int slot = c.prof_begin(family);
    bt_gemm_kernel<TA, TB, Step><<<(unsigned)n_tiles, GB_T, 0, st>>>(tiles.p, step);
    count_launch(st, "bt_gemm");
    check_launch("bt_gemm");
    c.prof_end(slot, flops, 0.0);
}

template <class Step, int BM, int BN>
static void bp_launch(cudaStream_t st, const int4 *tiles, size_t n, const Step &step) {
    static const bool attr = [] {
        TINCR_CUDA(cudaFuncSetAttribute(bt_plane_kernel<Step, BM, BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        bp_smem(BM, BN)));
        return true;
    }();
    (void)attr;
    bt_plane_kernel<Step, BM, BN><<<(unsigned)n, BP_T, bp_smem(BM, BN), st>>>(tiles, step);
    count_launch(st, "bt_plane");
    check_launch("bt_plane");
}

template <class Step>
static void bp_launch_shape(cudaStream_t st, int shape, const int4 *tiles, size_t n, const Step &step) {
    if (n == 0) return;
    switch (shape) {
    case 0: bp_launch<Step, 64, 64>(st, tiles, n, step); break;
    case 1: bp_launch<Step, 64, 32>(st, tiles, n, step); break;
    case 2: bp_launch<Step, 32, 64>(st, tiles, n, step); break;
    default: bp_launch<Step, 32, 32>(st, tiles, n, step); break;
    }
}

// one plane step: a launch per tile shape in use
template <class Step>
static void bt_plane_launch(Ctx &c, cudaStream_t st, BatchWork &w, int g, int p, const Step &step, int family) {
    for (int sh = 0; sh < BP_SHAPES; ++sh) {
        if (w.npt[g][p][sh] == 0) continue;
        const int slot = c.prof_begin(family);
        bp_launch_shape(st, sh, w.pt[g][p][sh].p, w.npt[g][p][sh], step);
        c.prof_end(slot, 0.0, 0.0);
    }
}

// ----------------------------------------------------------------------------------------------
// autotuner of the plane GEMM tile shapes
// ----------------------------------------------------------------------------------------------
// The instances of an FMO batch come in a few shapes (monomers of each ring count, pairs of them).
// For each shape (atoms, AOs, occupied, virtual, long-range flag) and each plane step, the tuner
// times the four tile shapes on the batch's own instances of that shape, all vector slots, the
// tile list repeated until the 64 x 64 grid has at least four CTAs per SM, and keeps the fastest
// (64 x 64 unless another is more than 2% faster).  Smaller tiles waste less of a tile on
// 96 - 204-row operands; larger ones load less per output.  The table lives for the process.

struct BpKey {
    int device, n_atoms, n_orb, n_occ, n_virt, lc;
    bool operator<(const BpKey &o) const {
        return std::tie(device, n_atoms, n_orb, n_occ, n_virt, lc) <
               std::tie(o.device, o.n_atoms, o.n_orb, o.n_occ, o.n_virt, o.lc);
    }
};
struct BpChoice {
    int shape[BP_STEPS];                 // -1: the step does not run for this shape
    double us[BP_STEPS][BP_SHAPES];      // measured time of each candidate per repetition of the tiles, us
};
static std::mutex g_bp_mu;
static std::map<BpKey, BpChoice> g_bp_table;

static BpKey bp_key(int device, const BtInst &b) { return BpKey{device, b.N, b.n, b.o, b.v, b.lc}; }

static bool bp_step_runs(const BtInst &b, int p) { return (p != BP_P2 && p != BP_P4) || b.lc; }

// Does [lo, hi) meet [a0, a1) or [b0, b1)?
static bool bp_meets(int lo, int hi, int a0, int a1, int b0, int b1) {
    return (lo < a1 && hi > a0) || (lo < b1 && hi > b0);
}

// Tiles of every vector slot of instance I for step p in tile shape sh.  With the block structure
// of a CT dimer (C_o zero on AOs >= nh, C_v zero on AOs < nh) the tiles that only hold zeros, or
// values that the next step multiplies by zeros, are left out (their planes keep the zeros they
// were cleared to):
//   H = [C_o;SC_o] X: rows nh..n-1 are zero;
//   F: only rows {mu, n+mu : mu < nh} and columns {nu, n+nu : nu >= nh} reach AX, the other rows
//      of M are zero or meet C_o = 0 in AX, the other columns are zero or meet C_v = 0 in G;
//   G = F [SC_v;C_v] + z: rows n+nh.. meet C_o = 0 in AX (which stops its K there).
static void bp_tiles(const BtInst &b, int I, int p, int sh, std::vector<int4> &out) {
    if (!bp_step_runs(b, p)) return;
    const int n = b.n, n2 = 2 * n, nh = b.nh, BM = BP_BM[sh], BN = BP_BN[sh];
    const int M = p == BP_P5 ? b.o : n2, N = p == BP_P2 ? n2 : b.v;
    for (int s = 0; s < b.nr; ++s)
        for (int tm = 0; tm < ceil_div(M, BM); ++tm)
            for (int tn = 0; tn < ceil_div(N, BN); ++tn) {
                if (nh) {
                    const int r0 = tm * BM, r1 = r0 + BM, c0 = tn * BN, c1 = c0 + BN;
                    if (p == BP_P1 && !bp_meets(r0, r1, 0, nh, n, n2)) continue;
                    if (p == BP_P2 && !(bp_meets(r0, r1, 0, nh, n, n + nh) && bp_meets(c0, c1, nh, n, n + nh, n2)))
                        continue;
                    if (p == BP_P4 && r0 >= n + nh) continue;
                }
                out.push_back(make_int4(I, s, tm, tn));
            }
}

// forced shape from TINCR_GB300_BATCH_TILES (64x64, 64x32, 32x64, 32x32), or -1 for the tuner
static int bp_forced_shape() {
    const char *e = getenv("TINCR_GB300_BATCH_TILES");
    if (!e || !*e || !strcmp(e, "auto")) return -1;
    for (int sh = 0; sh < BP_SHAPES; ++sh) {
        char name[16];
        snprintf(name, sizeof name, "%dx%d", BP_BM[sh], BP_BN[sh]);
        if (!strcmp(e, name)) return sh;
    }
    fail(TINCR_BAD_ARG, std::string("TINCR_GB300_BATCH_TILES: unknown tile shape ") + e);
    return -1;
}

template <class Step>
static void bp_probe(cudaStream_t st, int sh, const int4 *tiles, size_t n, const Step &step) {
    bp_launch_shape(st, sh, tiles, n, step);
}

// Tune every instance shape of the batch missing from the table.  Runs after the guesses and before
// the first iteration: everything the probes write (H, F, G planes, Coulomb diagonals, the products of
// the guesses) is written again by the first iteration before it is read.
static void bp_autotune(Ctx &c, BatchWork &w, const BtArrays &a, int n_sm) {
    std::map<BpKey, std::vector<int>> todo;
    {
        std::lock_guard<std::mutex> lk(g_bp_mu);
        for (int I = 0; I < (int)w.h.size(); ++I) {
            const BpKey k = bp_key(c.device, w.h[I]);
            if (!g_bp_table.count(k)) todo[k].push_back(I);
        }
    }
    if (todo.empty()) return;
    constexpr int REPS = 3;
    std::vector<cudaEvent_t> ev(2 * BP_STEPS * BP_SHAPES * (REPS + 1));
    for (auto &e : ev) TINCR_CUDA(cudaEventCreate(&e));
    for (auto &kv : todo) {
        const BtInst &b0 = w.h[kv.second[0]];
        BpChoice ch{};
        for (int p = 0; p < BP_STEPS; ++p) {
            ch.shape[p] = -1;
            if (!bp_step_runs(b0, p)) continue;
            std::vector<int4> base0;
            for (int I : kv.second) bp_tiles(w.h[I], I, p, 0, base0);
            const size_t reps = std::min<size_t>(64, std::max<size_t>(1, (4 * (size_t)n_sm + base0.size() - 1) / base0.size()));
            size_t cnt[BP_SHAPES];
            for (int sh = 0; sh < BP_SHAPES; ++sh) {
                std::vector<int4> one, all;
                for (int I : kv.second) bp_tiles(w.h[I], I, p, sh, one);
                for (size_t r = 0; r < reps; ++r) all.insert(all.end(), one.begin(), one.end());
                cnt[sh] = all.size();
                upload_any(c.stream, w.tune_tiles[sh], all);
            }
            for (int sh = 0; sh < BP_SHAPES; ++sh)
                for (int r = 0; r <= REPS; ++r) {   // r = 0 warms up
                    cudaEvent_t *e = &ev[2 * ((p * BP_SHAPES + sh) * (REPS + 1) + r)];
                    TINCR_CUDA(cudaEventRecord(e[0], c.stream));
                    const int4 *t = w.tune_tiles[sh].p;
                    switch (p) {
                    case BP_P1: bp_probe(c.stream, sh, t, cnt[sh], BtP1{a, false}); break;
                    case BP_P2: bp_probe(c.stream, sh, t, cnt[sh], BtP2{a}); break;
                    case BP_P4: bp_probe(c.stream, sh, t, cnt[sh], BtP4{a}); break;
                    default: bp_probe(c.stream, sh, t, cnt[sh], BtP5{a}); break;
                    }
                    TINCR_CUDA(cudaEventRecord(e[1], c.stream));
                }
            c.sync();   // the tile lists of the next step reuse the buffers
            float best = 0.f;
            for (int sh = 0; sh < BP_SHAPES; ++sh) {
                float t = 1e30f;
                for (int r = 1; r <= REPS; ++r) {
                    cudaEvent_t *e = &ev[2 * ((p * BP_SHAPES + sh) * (REPS + 1) + r)];
                    float ms = 0.f;
                    TINCR_CUDA(cudaEventElapsedTime(&ms, e[0], e[1]));
                    t = std::min(t, ms);
                }
                ch.us[p][sh] = 1000.0 * t / (double)reps;
                if (sh == 0 || t < 0.98f * best) {
                    best = t;
                    ch.shape[p] = sh;
                }
            }
        }
        std::lock_guard<std::mutex> lk(g_bp_mu);
        g_bp_table[kv.first] = ch;
    }
    for (auto &e : ev) cudaEventDestroy(e);
}

int bp_table_entries(int capacity, int *entries, double *us) {
    std::lock_guard<std::mutex> lk(g_bp_mu);
    int n = 0;
    for (const auto &kv : g_bp_table) {
        if (n < capacity) {
            const BpKey &k = kv.first;
            const BpChoice &ch = kv.second;
            if (entries) {
                int *e = entries + 9 * n;
                e[0] = k.n_atoms; e[1] = k.n_orb; e[2] = k.n_occ; e[3] = k.n_virt; e[4] = k.lc;
                for (int p = 0; p < BP_STEPS; ++p) e[5 + p] = ch.shape[p];
            }
            if (us)
                for (int p = 0; p < BP_STEPS; ++p)
                    for (int sh = 0; sh < BP_SHAPES; ++sh) us[(n * BP_STEPS + p) * BP_SHAPES + sh] = ch.us[p][sh];
        }
        ++n;
    }
    return n;
}

int Ctx::solve_batch(int n_inst, const tincr_tda_instance *hin, int max_iter, double tol, int precision,
                     tincr_tda_result *res) {
    if (n_inst <= 0 || !hin || !res || max_iter <= 0 || !(tol > 0.0)) fail(TINCR_BAD_ARG, "solve_batch: bad arguments");
    if (precision != TINCR_PREC_FP64 && precision != TINCR_PREC_BF16X3) fail(TINCR_BAD_ARG, "solve_batch: unknown precision");
    const bool mixed = precision == TINCR_PREC_BF16X3;
    g_launches = 0;
    if (!batch) batch = new BatchWork();
    BatchWork &w = *batch;
    w.h.assign(n_inst, BtInst{});
    // internal order: heavy instances first (group 0), then light ones (group 1); order[I] is the
    // caller's index of internal instance I
    std::vector<int> order;
    order.reserve(n_inst);
    int g_lo[3] = {0, 0, n_inst};   // group g holds internal instances [g_lo[g], g_lo[g + 1])
    for (int pass = 0; pass < 2; ++pass)
        for (int k = 0; k < n_inst; ++k) {
            const long long nr = hin[k].n_roots, ov = (long long)hin[k].n_occ * hin[k].n_virt;
            if ((nr * nr * ov >= BT_HEAVY) == (pass == 0)) order.push_back(k);
        }
    for (int k = 0; k < n_inst; ++k) {
        const long long nr = hin[k].n_roots, ov = (long long)hin[k].n_occ * hin[k].n_virt;
        if (nr * nr * ov >= BT_HEAVY) ++g_lo[1];
    }
    std::vector<int> hAo, hAoAtom, hPos;
    std::vector<long long> hGlrOff(n_inst, 0), offPos(n_inst, 0);
    long long o_c = 0, o_s = 0, o_blk = 0, o_glr = 0, o_gam = 0, o_om = 0, o_v = 0, o_r = 0, o_sub = 0, o_h = 0, o_f = 0,
              o_d = 0, o_u = 0, o_y = 0, o_glra = 0, o_pos = 0;
    long long o_pc = 0, o_pv = 0;
    int o_ao = 0, o_aoatom = 0, mmax_all = 1, nr_max = 1, nmax_atoms = 1;
    // pass 1: validation and the packed offsets of every instance
    for (int I = 0; I < n_inst; ++I) {
        const tincr_tda_instance &q = hin[order[I]];
        if (q.n_atoms <= 0 || q.n_orb <= 0 || q.n_occ <= 0 || q.n_virt <= 0 || q.n_occ + q.n_virt > q.n_orb ||
            q.n_roots <= 0 || q.n_roots > BT_MAXR || (long long)q.n_roots > (long long)q.n_occ * q.n_virt ||
            !q.orbs_per_atom || !q.c || !q.s || !q.orbe || !q.gamma || !q.xyz)
            fail(TINCR_BAD_ARG, "solve_batch: instance " + std::to_string(order[I]) + " is malformed (n_roots <= 6)");
        BtInst &b = w.h[I];
        b.n = q.n_orb; b.o = q.n_occ; b.v = q.n_virt; b.N = q.n_atoms;
        b.nr = q.n_roots; b.mmax = 15 * q.n_roots; b.lc = q.gamma_lr != nullptr; b.max_iter = max_iter;
        b.ov = (long long)b.o * b.v;
        const int n = b.n, w_ = b.o + b.v, N = b.N;
        int sum = 0;
        for (int A = 0; A < N; ++A) {
            if (q.orbs_per_atom[A] <= 0) fail(TINCR_BAD_ARG, "solve_batch: orbs_per_atom must be positive");
            sum += q.orbs_per_atom[A];
        }
        if (sum != n) fail(TINCR_BAD_ARG, "solve_batch: orbs_per_atom does not add up to n_orb");
        b.off_c = o_c; o_c += (long long)n * w_;
        b.off_s = o_s; o_s += (long long)n * n;
        b.off_blk = o_blk; o_blk += 2LL * n * 2 * w_;
        b.off_glr = o_glr; if (b.lc) o_glr += (long long)n * n;
        b.off_gam = o_gam; o_gam += (long long)N * N;
        b.off_omega = o_om; o_om += b.ov;
        b.off_v = o_v; o_v += (long long)b.mmax * b.ov;
        b.off_r = o_r; o_r += (long long)b.nr * b.ov;
        b.off_sub = o_sub; o_sub += (long long)b.mmax * b.mmax;
        b.off_h = o_h; o_h += (long long)b.nr * 2 * n * b.v;
        b.off_f = o_f; if (b.lc) o_f += (long long)b.nr * 4 * n * n;
        b.off_d = o_d; o_d += 3LL * b.nr * n;
        b.off_u = o_u; o_u += b.nr;
        b.off_y = o_y; o_y += (long long)b.nr * N;
        b.ko = pad32(b.o); b.kv = pad32(b.v); b.k2 = pad32(2 * n);
        b.off_pc = o_pc; o_pc += 2LL * n * b.ko + 2LL * n * b.kv + (long long)b.v * b.k2 + (long long)b.o * b.k2;
        b.off_pv = o_pv;
        o_pv += (long long)b.nr * ((long long)b.v * b.ko + 2LL * n * b.kv + 2LL * n * b.k2 + (long long)b.v * b.k2);
        b.off_ao = o_ao; o_ao += N + 1;
        b.off_aoatom = o_aoatom; o_aoatom += n;
        if (b.lc) { hGlrOff[I] = o_glra; o_glra += (long long)N * N; }
        offPos[I] = o_pos; o_pos += b.nr;
        mmax_all = std::max(mmax_all, b.mmax);
        nr_max = std::max(nr_max, b.nr);
        nmax_atoms = std::max(nmax_atoms, N);
    }
    // pass 2, one instance per task: copies into the page-locked staging buffers with the finiteness
    // check, orbital-energy differences and the guess positions
    w.pinC.reserve(o_c);
    w.pinS.reserve(o_s);
    w.pinG.reserve(o_gam);
    w.pinGlr.reserve(o_glra);
    w.pinOm.reserve(o_om);
    hAo.resize(o_ao);
    hAoAtom.resize(o_aoatom);
    hPos.resize(o_pos);
    std::vector<unsigned char> bad(n_inst, 0);
#pragma omp parallel for schedule(dynamic, 4) num_threads(12)
    for (int I = 0; I < n_inst; ++I) {
        const tincr_tda_instance &q = hin[order[I]];
        BtInst &b = w.h[I];
        const int n = b.n, w_ = b.o + b.v, N = b.N;
        auto copy = [&](double *dst, const double *src, size_t cnt, unsigned char flag) {
            bool ok = true;
            for (size_t k = 0; k < cnt; ++k) {
                const double x = src[k];
                ok &= std::isfinite(x);
                dst[k] = x;
            }
            if (!ok) bad[I] |= flag;
        };
        copy(w.pinC.p + b.off_c, q.c, (size_t)n * w_, 1);
        // block structure of a CT dimer: occupied MOs only on AOs < nh, virtual MOs only on AOs >= nh
        {
            int hi_o = 0, lo_v = n;
            for (int mu = 0; mu < n; ++mu) {
                const double *row = q.c + (size_t)mu * w_;
                for (int k = 0; k < b.o; ++k)
                    if (row[k] != 0.0) { hi_o = mu + 1; break; }
                if (lo_v == n)
                    for (int k = b.o; k < w_; ++k)
                        if (row[k] != 0.0) { lo_v = mu; break; }
            }
            b.nh = (hi_o > 0 && hi_o < n && hi_o <= lo_v) ? hi_o : 0;
            b.k5 = b.nh ? pad32(n + b.nh) : b.k2;
        }
        copy(w.pinS.p + b.off_s, q.s, (size_t)n * n, 2);
        copy(w.pinG.p + b.off_gam, q.gamma, (size_t)N * N, 4);
        if (b.lc) copy(w.pinGlr.p + hGlrOff[I], q.gamma_lr, (size_t)N * N, 8);
        for (int k = 0; k < w_; ++k)
            if (!std::isfinite(q.orbe[k])) bad[I] |= 16;
        int off = 0;
        for (int A = 0; A < N; ++A) {
            hAo[b.off_ao + A] = off;
            for (int k = 0; k < q.orbs_per_atom[A]; ++k) hAoAtom[b.off_aoatom + off + k] = A;
            off += q.orbs_per_atom[A];
        }
        hAo[b.off_ao + N] = off;
        // omega_ia = e_a - e_i (excited_states/utils.rs:8-22) and the guess positions (stable ties)
        double *om = w.pinOm.p + b.off_omega;
        for (int i = 0; i < b.o; ++i)
            for (int x = 0; x < b.v; ++x) om[(size_t)i * b.v + x] = q.orbe[b.o + x] - q.orbe[i];
        std::vector<int> ord(b.ov);
        std::iota(ord.begin(), ord.end(), 0);
        std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return om[x] < om[y]; });
        for (int r = 0; r < b.nr; ++r) hPos[offPos[I] + r] = ord[r];
    }
    for (int I = 0; I < n_inst; ++I)
        if (bad[I]) {
            static const char *names[5] = {"c", "s", "gamma", "gamma_lr", "orbe"};
            int f = 0;
            while (!((bad[I] >> f) & 1)) ++f;
            fail(TINCR_NONFINITE, "solve_batch: instance " + std::to_string(order[I]) + ": non-finite value in " + names[f]);
        }
    // device arrays
    auto upload_pinned = [&](DevBuf<double> &d, const PinnedBuf &h, long long count) {
        d.reserve(std::max<long long>(1, count));
        if (count > 0)
            TINCR_CUDA(cudaMemcpyAsync(d.p, h.p, (size_t)count * sizeof(double), cudaMemcpyHostToDevice, stream));
    };
    upload_any(stream, w.inst, w.h);
    w.state.reserve(n_inst);
    upload_pinned(w.C, w.pinC, o_c);
    w.SC.reserve(std::max<long long>(1, o_c));
    upload_pinned(w.S, w.pinS, o_s);
    w.blk.reserve(std::max<long long>(1, o_blk));
    w.glr.reserve(std::max<long long>(1, o_glr));
    upload_pinned(w.glr_atoms, w.pinGlr, o_glra);
    upload_any(stream, w.off_glr_atoms, hGlrOff);
    upload_pinned(w.gam, w.pinG, o_gam);
    upload_pinned(w.omega, w.pinOm, o_om);
    w.V.reserve(o_v);
    w.AV.reserve(o_v);
    w.R.reserve(o_r);
    w.Rk.reserve(o_r);
    w.T.reserve(o_r);
    w.sub.reserve(o_sub);
    w.H.reserve(o_h);
    // the mixed form leaves the zero rows of block-structured H out: they must read as zeros
    if (mixed) TINCR_CUDA(cudaMemsetAsync(w.H.p, 0, o_h * sizeof(double), stream));
    w.F.reserve(std::max<long long>(1, o_f));
    // the FP64 exchange leaves the zero tiles of block-structured F out: they must read as zeros
    if (!(mixed && tol >= MIXED_TOL_FLOOR) && o_f > 0) TINCR_CUDA(cudaMemsetAsync(w.F.p, 0, o_f * sizeof(double), stream));
    w.D.reserve(o_d);
    w.u.reserve(o_u);
    w.err.reserve(o_u);
    w.Y.reserve(o_y);
    upload_any(stream, w.ao_off, hAo);
    upload_any(stream, w.ao_atom, hAoAtom);
    upload_any(stream, w.pos, hPos);
    w.active.reserve(1);
    w.loop.reserve(3);

    // clusters of the subspace step: each heavy instance on one cluster, the light ones four to a
    // cluster; per group, roots per instance (grid of the per-vector kernels)
    static_assert(BT_CL == 4, "a cluster's work is one int4");
    unsigned sub_grid[2] = {0, 0};
    int nr_grp[2] = {1, 1};
    for (int g = 0; g < 2; ++g) {
        std::vector<int4> cw;
        for (int I = g_lo[g]; I < g_lo[g + 1]; ++I) nr_grp[g] = std::max(nr_grp[g], w.h[I].nr);
        if (g == 0) {
            for (int I = g_lo[0]; I < g_lo[1]; ++I) cw.push_back(make_int4(I, -2, -2, -2));
        } else {
            for (int k = g_lo[1]; k < g_lo[2]; k += BT_CL) {
                int v[BT_CL];
                for (int r = 0; r < BT_CL; ++r) v[r] = k + r < g_lo[2] ? k + r : -1;
                cw.push_back(make_int4(v[0], v[1], v[2], v[3]));
            }
        }
        sub_grid[g] = (unsigned)(cw.size() * BT_CL);
        if (!cw.empty()) upload_any(stream, w.cl_inst[g], cw);
    }

    // static tile tables (the FP64 product tables only when an FP64 product runs)
    const bool fp64_products = !(mixed && tol >= MIXED_TOL_FLOOR);
    std::vector<int4> tsc, t1[2], t2[2], t4[2], t5[2];
    for (int I = 0; I < n_inst; ++I) {
        const BtInst &b = w.h[I];
        const int n2 = 2 * b.n, g = I < g_lo[1] ? 0 : 1;
        for (int tm = 0; tm < ceil_div(b.n, GB_M); ++tm)
            for (int tn = 0; tn < ceil_div(b.o + b.v, GB_N); ++tn) tsc.push_back(make_int4(I, 0, tm, tn));
        for (int s = 0; s < (fp64_products ? b.nr : 0); ++s) {
            for (int tm = 0; tm < ceil_div(n2, GB_M); ++tm)
                for (int tn = 0; tn < ceil_div(b.v, GB_N); ++tn) {
                    t1[g].push_back(make_int4(I, s, tm, tn));
                    if (b.lc && !(b.nh && tm * GB_M >= b.n + b.nh)) t4[g].push_back(make_int4(I, s, tm, tn));
                }
            // with the block structure: F tiles that only hold zeros or values multiplied by zeros
            // are left out (as in the plane steps), G rows from n+nh are not needed
            if (b.lc)
                for (int tm = 0; tm < ceil_div(n2, GB_M); ++tm)
                    for (int tn = 0; tn < ceil_div(n2, GB_N); ++tn) {
                        const int r0 = tm * GB_M, c0 = tn * GB_N;
                        if (b.nh && !(bp_meets(r0, r0 + GB_M, 0, b.nh, b.n, b.n + b.nh) &&
                                      bp_meets(c0, c0 + GB_N, b.nh, b.n, b.n + b.nh, n2)))
                            continue;
                        t2[g].push_back(make_int4(I, s, tm, tn));
                    }
            for (int tm = 0; tm < ceil_div(b.o, GB_M); ++tm)
                for (int tn = 0; tn < ceil_div(b.v, GB_N); ++tn) t5[g].push_back(make_int4(I, s, tm, tn));
        }
    }
    upload_any(stream, w.t_sc, tsc);
    for (int g = 0; g < 2; ++g) {
        w.nt1[g] = t1[g].size(); w.nt2[g] = t2[g].size(); w.nt4[g] = t4[g].size(); w.nt5[g] = t5[g].size();
        if (w.nt1[g]) upload_any(stream, w.t1[g], t1[g]);
        if (w.nt2[g]) upload_any(stream, w.t2[g], t2[g]);
        if (w.nt4[g]) upload_any(stream, w.t4[g], t4[g]);
        if (w.nt5[g]) upload_any(stream, w.t5[g], t5[g]);
    }
    // split-BF16 planes of the mixed form (their tile tables follow the guesses and the autotuner)
    if (mixed) {
        w.Pl.reserve(N_PLANES * (o_pc + o_pv));
        TINCR_CUDA(cudaMemsetAsync(w.Pl.p, 0, N_PLANES * (o_pc + o_pv) * sizeof(bf16), stream));   // K padding stays zero
        for (auto &b : w.h) b.off_pv += o_pc;
        upload_any(stream, w.inst, w.h);
    }

    BtArrays a{};
    a.inst = w.inst.p; a.state = w.state.p;
    a.C = w.C.p; a.SC = w.SC.p; a.S = w.S.p; a.blk = w.blk.p; a.glr = w.glr.p; a.gam = w.gam.p; a.omega = w.omega.p;
    a.V = w.V.p; a.AV = w.AV.p; a.R = w.R.p; a.Rk = w.Rk.p; a.T = w.T.p; a.sub = w.sub.p; a.H = w.H.p; a.F = w.F.p;
    a.D = w.D.p; a.u = w.u.p; a.err = w.err.p; a.Y = w.Y.p; a.ao_off = w.ao_off.p; a.ao_atom = w.ao_atom.p;
    a.active = w.active.p; a.tol = tol;
    a.P = mixed ? w.Pl.p : nullptr;
    a.ps = o_pc + o_pv;
    if (mixed) {
        w.glr32.reserve(std::max<long long>(1, o_glr));
        w.blk32.reserve(std::max<long long>(1, o_blk));
        w.D32.reserve(o_d);
    }
    a.glr32 = mixed ? w.glr32.p : nullptr;
    a.blk32 = mixed ? w.blk32.p : nullptr;
    a.D32 = mixed ? w.D32.p : nullptr;

    TINCR_CUDA(cudaEventRecord(ev0, stream));
    // set-up: SC, packed blocks, gamma_lr in the AO basis, guesses
    // FP32 S C serves the mixed operator; a solve that finishes with FP64 iterations (tolerance below
    // the mixed floor) needs the FP64 product for them
    if (mixed && tol >= MIXED_TOL_FLOOR) {
        const int slot = prof_begin(TINCR_KF_OTHER);
        bt_sc32_kernel<<<(unsigned)tsc.size(), GB_T, 0, stream>>>(w.t_sc.p, a);
        count_launch(stream, "bt_sc32");
        check_launch("bt_sc32");
        prof_end(slot, 0.0, 0.0);
    } else {
        bt_launch<false, false>(*this, stream, w.t_sc, tsc.size(), BtStepSC{a}, TINCR_KF_OTHER, 0.0);
    }
    bt_pack_kernel<<<n_inst, BT_T, 0, stream>>>(a);
    count_launch(stream, "bt_pack");
    check_launch("bt_pack");
    if (o_glra > 0) {
        bt_expand_kernel<<<n_inst, BT_T, 0, stream>>>(a, w.glr_atoms.p, w.off_glr_atoms.p);
        count_launch(stream, "bt_expand");
        check_launch("bt_expand");
    }
    if (mixed) {
        bt_const_planes_kernel<<<n_inst, BT_T, 0, stream>>>(a);
        count_launch(stream, "bt_const_planes");
        check_launch("bt_const_planes");
        bt_f32_copies_kernel<<<n_inst, BT_T, 0, stream>>>(a);
        count_launch(stream, "bt_f32_copies");
        check_launch("bt_f32_copies");
    }
    bt_guess_kernel<<<n_inst, BT_T, 0, stream>>>(a, w.pos.p);
    count_launch(stream, "bt_guess");
    check_launch("bt_guess");
    const dim3 gv(nr_max, n_inst);
    const dim3 gvg[2] = {dim3(nr_grp[0], g_lo[1] - g_lo[0]), dim3(nr_grp[1], g_lo[2] - g_lo[1])};
    if (mixed) {
        // tile shape of every instance and plane step: forced, or from the autotuner's table
        const int forced = bp_forced_shape();
        if (forced < 0) {
            TINCR_CUDA(cudaMemsetAsync(w.D32.p, 0, o_d * sizeof(float), stream));
            bt_split_x_kernel<<<gv, BT_T, 0, stream>>>(a, 0, 0);
            count_launch(stream, "bt_split_x");
            check_launch("bt_split_x");
            bp_autotune(*this, w, a, n_sm);
        }
        std::vector<int4> pt[2][BP_STEPS][BP_SHAPES];
        {
            std::lock_guard<std::mutex> lk(g_bp_mu);
            for (int I = 0; I < n_inst; ++I) {
                const BpChoice *ch = forced < 0 ? &g_bp_table.at(bp_key(device, w.h[I])) : nullptr;
                const int g = I < g_lo[1] ? 0 : 1;
                for (int p = 0; p < BP_STEPS; ++p) {
                    const int sh = ch ? ch->shape[p] : forced;
                    if (sh >= 0) bp_tiles(w.h[I], I, p, sh, pt[g][p][sh]);
                }
            }
        }
        for (int g = 0; g < 2; ++g)
            for (int p = 0; p < BP_STEPS; ++p)
                for (int sh = 0; sh < BP_SHAPES; ++sh) {
                    w.npt[g][p][sh] = pt[g][p][sh].size();
                    if (!pt[g][p][sh].empty()) upload_any(stream, w.pt[g][p][sh], pt[g][p][sh]);
                }
    }

    const size_t sub_smem = bt_subspace_smem(mmax_all);
    TINCR_CUDA(cudaFuncSetAttribute(bt_subspace_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sub_smem));
    const size_t coul_smem = (size_t)nmax_atoms * sizeof(double);
    if (coul_smem > 48 * 1024)
        TINCR_CUDA(cudaFuncSetAttribute(bt_coulomb_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)coul_smem));
    if (!w.side) {
        int least = 0, greatest = 0;
        TINCR_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        TINCR_CUDA(cudaStreamCreateWithPriority(&w.hi, cudaStreamNonBlocking, greatest));
        TINCR_CUDA(cudaStreamCreateWithPriority(&w.side, cudaStreamNonBlocking, least));
        TINCR_CUDA(cudaEventCreateWithFlags(&w.fork, cudaEventDisableTiming));
        TINCR_CUDA(cudaEventCreateWithFlags(&w.join_hi, cudaEventDisableTiming));
        TINCR_CUDA(cudaEventCreateWithFlags(&w.join_side, cudaEventDisableTiming));
    }

    // one Davidson iteration of the running instances of group g on stream st
    auto iteration = [&](cudaStream_t st, int g) {
        if (g_lo[g] == g_lo[g + 1]) return;
        const int I0 = g_lo[g];
        bt_launch<false, false>(*this, st, w.t1[g], w.nt1[g], BtStep1{a, false}, TINCR_KF_AO_TRANSFORM, 0.0);
        bt_launch<false, true>(*this, st, w.t2[g], w.nt2[g], BtStep2{a}, TINCR_KF_AO_EXCHANGE, 0.0);
        bt_diag_kernel<<<gvg[g], BT_T, 0, st>>>(a, 0, I0);
        count_launch(st, "bt_diag");
        check_launch("bt_diag");
        bt_coulomb_kernel<<<gvg[g], BT_T, coul_smem, st>>>(a, 0, I0);
        count_launch(st, "bt_coulomb");
        check_launch("bt_coulomb");
        bt_launch<false, false>(*this, st, w.t4[g], w.nt4[g], BtStep4{a}, TINCR_KF_AO_EXCHANGE, 0.0);
        bt_scale_rows_kernel<<<gvg[g], BT_T, 0, st>>>(a, I0);
        count_launch(st, "bt_scale_rows");
        check_launch("bt_scale_rows");
        bt_launch<true, false>(*this, st, w.t5[g], w.nt5[g], BtStep5{a}, TINCR_KF_AO_TRANSFORM, 0.0);
        bt_subspace_kernel<<<sub_grid[g], BT_T, sub_smem, st>>>(a, w.cl_inst[g].p);
        count_launch(st, "bt_subspace");
        check_launch("bt_subspace");
    };
    // the mixed-form iteration: split-BF16 plane GEMMs, FP64 Coulomb diagonals and subspace step
    auto iteration_mixed = [&](cudaStream_t st, int g) {
        if (g_lo[g] == g_lo[g + 1]) return;
        const int I0 = g_lo[g];
        bt_split_x_kernel<<<gvg[g], BT_T, 0, st>>>(a, I0, 0);
        count_launch(st, "bt_split_x");
        check_launch("bt_split_x");
        bt_plane_launch(*this, st, w, g, BP_P1, BtP1{a, false}, TINCR_KF_AO_TRANSFORM);
        bt_plane_launch(*this, st, w, g, BP_P2, BtP2{a}, TINCR_KF_AO_EXCHANGE);   // + LC Coulomb diagonals
        bt_diag_kernel<<<gvg[g], BT_T, 0, st>>>(a, BT_MIXED, I0);                  // non-LC Coulomb diagonals
        count_launch(st, "bt_diag");
        check_launch("bt_diag");
        bt_coulomb_kernel<<<gvg[g], BT_T, coul_smem, st>>>(a, BT_MIXED, I0);
        count_launch(st, "bt_coulomb");
        check_launch("bt_coulomb");
        bt_plane_launch(*this, st, w, g, BP_P4, BtP4{a}, TINCR_KF_AO_EXCHANGE);
        bt_gt_nolc_kernel<<<gvg[g], BT_T, 0, st>>>(a, I0);
        count_launch(st, "bt_gt_nolc");
        check_launch("bt_gt_nolc");
        bt_plane_launch(*this, st, w, g, BP_P5, BtP5{a}, TINCR_KF_AO_TRANSFORM);
        bt_subspace_kernel<<<sub_grid[g], BT_T, sub_smem, st>>>(a, w.cl_inst[g].p);
        count_launch(st, "bt_subspace");
        check_launch("bt_subspace");
    };
    // One iteration of both groups.  The groups are independent, so in the graph they are two
    // concurrent branches: the heavy group, whose iterations are more and whose subspace step is
    // bound by the latency of its small eigenproblems, at high priority, and the light group at low
    // priority filling the SMs the heavy one leaves.  With kernel timing on, both run in turn on the
    // main stream.
    auto both = [&](const std::function<void(cudaStream_t, int)> &body, bool fork) {
        TINCR_CUDA(cudaMemsetAsync(w.active.p, 0, sizeof(int), stream));
        if (fork) {
            TINCR_CUDA(cudaEventRecord(w.fork, stream));
            TINCR_CUDA(cudaStreamWaitEvent(w.hi, w.fork, 0));
            TINCR_CUDA(cudaStreamWaitEvent(w.side, w.fork, 0));
            body(w.hi, 0);
            body(w.side, 1);
            TINCR_CUDA(cudaEventRecord(w.join_hi, w.hi));
            TINCR_CUDA(cudaEventRecord(w.join_side, w.side));
            TINCR_CUDA(cudaStreamWaitEvent(stream, w.join_hi, 0));
            TINCR_CUDA(cudaStreamWaitEvent(stream, w.join_side, 0));
        } else {
            body(stream, 0);
            body(stream, 1);
        }
    };
    // Run an iteration function until no instance is running or the limit is reached.  Without
    // kernel timing the whole loop is one CUDA graph: a WHILE node whose body is one iteration of
    // both groups followed by bt_loop_next_kernel, which decides on the device whether the body runs
    // again, so no host round trip separates the iterations.  With kernel timing on (per-family
    // events), the iterations run from the host one by one.  `after_prev`: the limit counts the
    // iterations of the previous loop (limit - previous, at least 1).  Returns the launches of one
    // iteration (for the launch count, finished once the iteration counts are read back).
    auto run_loop = [&](const std::function<void(cudaStream_t, int)> &body, int limit, bool after_prev) {
        long long per_iter = 0;
        if (!profiling) {
            bt_loop_init_kernel<<<1, 1, 0, stream>>>(w.loop.p, limit, after_prev ? 1 : 0);
            count_launch(stream, "bt_loop_init");
            check_launch("bt_loop_init");
            cudaGraph_t graph = nullptr;
            cudaGraphExec_t exec = nullptr;
            TINCR_CUDA(cudaGraphCreate(&graph, 0));
            cudaGraphConditionalHandle handle;
            TINCR_CUDA(cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault));
            cudaGraphNodeParams cp{};
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = handle;
            cp.conditional.type = cudaGraphCondTypeWhile;
            cp.conditional.size = 1;
            cudaGraphNode_t node;
            TINCR_CUDA(cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp));
            cudaGraph_t body_graph = cp.conditional.phGraph_out[0];
            TINCR_CUDA(cudaStreamBeginCaptureToGraph(stream, body_graph, nullptr, nullptr, 0,
                                                     cudaStreamCaptureModeThreadLocal));
            const long long before = g_launches;
            both(body, true);
            bt_loop_next_kernel<<<1, 1, 0, stream>>>(w.active.p, w.loop.p, handle);
            count_launch(stream, "bt_loop_next");
            check_launch("bt_loop_next");
            per_iter = g_launches - before;
            g_launches = before;
            cudaGraph_t captured = nullptr;
            TINCR_CUDA(cudaStreamEndCapture(stream, &captured));
            TINCR_CUDA(cudaGraphInstantiate(&exec, graph, cudaGraphInstantiateFlagUseNodePriority));
            cudaGraphDestroy(graph);
            TINCR_CUDA(cudaGraphLaunch(exec, stream));
            // freed once the launch completes
            cudaGraphExecDestroy(exec);
        } else {
            int its = 0, active = n_inst, prev = 0;
            if (after_prev) {
                TINCR_CUDA(cudaMemcpyAsync(&prev, w.loop.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
                sync();
                limit = std::max(1, limit - prev);
            }
            while (active > 0 && its < limit) {
                both(body, false);
                ++its;
                TINCR_CUDA(cudaMemcpyAsync(&active, w.active.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
                sync();
            }
            const int rec[3] = {its, limit, prev};
            TINCR_CUDA(cudaMemcpyAsync(w.loop.p, rec, sizeof(rec), cudaMemcpyHostToDevice, stream));
            sync();
        }
        return per_iter;
    };
    long long per_iter_first = 0, per_iter_second = 0;
    if (mixed && tol >= MIXED_TOL_FLOOR) {
        per_iter_first = run_loop(iteration_mixed, max_iter, false);
    } else if (mixed) {
        // the mixed operator resolves residuals down to MIXED_TOL_FLOOR: the mixed phase stops there
        a.tol = MIXED_TOL_FLOOR;
        per_iter_first = run_loop(iteration_mixed, max_iter, false);
        a.tol = tol;
        // FP64 polish: every instance restarts from its mixed Ritz vectors on the FP64 operator and
        // may stop at its first Rayleigh-Ritz step; convergence and energies are those of FP64.  The
        // polish may take max_iter minus the mixed iterations (at least 1), counted on the device.
        bt_restart_kernel<<<n_inst, BT_T, 0, stream>>>(a);
        count_launch(stream, "bt_restart");
        check_launch("bt_restart");
        per_iter_second = run_loop(iteration, max_iter, true);
    } else {
        per_iter_first = run_loop(iteration, max_iter, false);
    }
    // final pass: transition charges of the Ritz vectors (H = [C_o;SC_o] R, then its Coulomb
    // diagonals); a mixed solve forms H with the plane GEMM (its S C is FP32-accurate either way)
    for (int g = 0; g < 2; ++g) {
        if (g_lo[g] == g_lo[g + 1]) continue;
        if (mixed && tol >= MIXED_TOL_FLOOR) {
            bt_split_x_kernel<<<gvg[g], BT_T, 0, stream>>>(a, g_lo[g], 1);
            count_launch(stream, "bt_split_x");
            check_launch("bt_split_x");
            bt_plane_launch(*this, stream, w, g, BP_P1, BtP1{a, true}, TINCR_KF_OTHER);
        } else {
            bt_launch<false, false>(*this, stream, w.t1[g], w.nt1[g], BtStep1{a, true}, TINCR_KF_OTHER, 0.0);
        }
    }
    bt_diag_kernel<<<gv, BT_T, 0, stream>>>(a, 1, 0);
    count_launch(stream, "bt_diag");
    check_launch("bt_diag");
    bt_coulomb_kernel<<<gv, BT_T, coul_smem, stream>>>(a, 1, 0);
    count_launch(stream, "bt_coulomb");
    check_launch("bt_coulomb");
    TINCR_CUDA(cudaEventRecord(ev1, stream));

    // results
    std::vector<BtState> hs(n_inst);
    std::vector<double> hu(o_u), hR(o_r), hY(o_y);
    TINCR_CUDA(cudaMemcpyAsync(hs.data(), w.state.p, n_inst * sizeof(BtState), cudaMemcpyDeviceToHost, stream));
    TINCR_CUDA(cudaMemcpyAsync(hu.data(), w.u.p, o_u * sizeof(double), cudaMemcpyDeviceToHost, stream));
    TINCR_CUDA(cudaMemcpyAsync(hR.data(), w.R.p, o_r * sizeof(double), cudaMemcpyDeviceToHost, stream));
    TINCR_CUDA(cudaMemcpyAsync(hY.data(), w.Y.p, o_y * sizeof(double), cudaMemcpyDeviceToHost, stream));
    int loop_rec[3] = {0, 0, 0};
    TINCR_CUDA(cudaMemcpyAsync(loop_rec, w.loop.p, sizeof(loop_rec), cudaMemcpyDeviceToHost, stream));
    sync();
    // launches of the device loop(s): iterations of the last loop in loop_rec[0], of the loop before
    // it (mixed phase followed by the FP64 polish) in loop_rec[2]
    if (per_iter_second > 0)
        g_launches += per_iter_first * loop_rec[2] + per_iter_second * loop_rec[0];
    else
        g_launches += per_iter_first * loop_rec[0];
    int worst = TINCR_OK;
    last_products = 0;
    for (int I = 0; I < n_inst; ++I) {
        const BtState &s = hs[I];
        tincr_tda_result &o = res[order[I]];
        o.iterations = s.iter;
        o.status = s.status == BT_CONVERGED ? TINCR_OK
                 : s.status == BT_NONFINITE ? TINCR_NONFINITE : TINCR_NOT_CONVERGED;
        if (o.status == TINCR_NONFINITE) worst = TINCR_NONFINITE;
        else if (o.status == TINCR_NOT_CONVERGED && worst == TINCR_OK) worst = TINCR_NOT_CONVERGED;
        last_products += s.products;
    }
    // per-instance outputs, one task per instance (the coefficients are transposed to tincr's layout)
#pragma omp parallel for schedule(dynamic, 4) num_threads(12)
    for (int I = 0; I < n_inst; ++I) {
        const BtInst &b = w.h[I];
        const tincr_tda_instance &q = hin[order[I]];
        tincr_tda_result &o = res[order[I]];
        const double *u = hu.data() + b.off_u, *Rr = hR.data() + b.off_r, *Y = hY.data() + b.off_y;
        if (o.energies)
            for (int r = 0; r < b.nr; ++r) o.energies[r] = u[r];
        if (o.coefficients)
            for (long long x = 0; x < b.ov; ++x)
                for (int r = 0; r < b.nr; ++r) o.coefficients[x * b.nr + r] = Rr[(long long)r * b.ov + x];
        if (o.q_trans)
            for (int A = 0; A < b.N; ++A)
                for (int r = 0; r < b.nr; ++r) o.q_trans[(size_t)A * b.nr + r] = Y[(size_t)r * b.N + A];
        // Mulliken transition dipoles and oscillator strengths (tda/moments.rs:7-24)
        for (int r = 0; r < b.nr; ++r) {
            double mu[3] = {0.0, 0.0, 0.0};
            for (int A = 0; A < b.N; ++A)
                for (int c = 0; c < 3; ++c) mu[c] += q.xyz[(size_t)A * 3 + c] * Y[(size_t)r * b.N + A];
            if (o.tr_dip)
                for (int c = 0; c < 3; ++c) o.tr_dip[(size_t)c * b.nr + r] = mu[c];
            if (o.osc) o.osc[r] = 2.0 / 3.0 * u[r] * (mu[0] * mu[0] + mu[1] * mu[1] + mu[2] * mu[2]);
        }
    }
    float ms = 0.f;
    TINCR_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    last_ms = ms;
    last_launches = g_launches;
    prof_resolve();
    return worst;
}

void release_batch(BatchWork *w) { delete w; }

}  // namespace tincr
