// Batched LE / CT TDA: tincr's per-monomer TDA loop (src/fmo/lcmo/basis.rs:462-465, Monomer::
// prepare_tda / run_tda in src/excited_states/tda/monomer.rs:8-53, mod.rs:18-70) and the CT pair
// loop (basis.rs:170-238, PairChargeTransfer::prepare_ct_tda / run_ct_tda in
// src/excited_states/tda/ct_pair.rs:12-180) as one device-resident lockstep block Davidson.
//
// Per iteration (a CUDA graph replayed until no instance is running):
//   1. H  = [C_o;SC_o] X                      grouped FP64 GEMM, tiles over (instance, vector)
//   2. F  = -1/4 gamma_lr o (H [C_v;SC_v]^T)  grouped GEMM with the Hadamard epilogue (LC instances),
//      or the two Coulomb diagonals only     (non-LC instances)
//   3. y = q_ov X per atom, z = gamma y       one CTA per (instance, vector)
//   4. G  = F [SC_v;C_v]                      grouped GEMM (LC) or row scaling by z (non-LC)
//   5. AX = [SC_o;C_o]^T G + omega o X        grouped GEMM with the omega epilogue
//   6. subspace step                          one CTA per instance: projections, FP64 Jacobi
//      eigensolver, Ritz vectors and residuals, convergence test, preconditioning, Gram-Schmidt,
//      collapse (davidson.rs:83-178)
// Every CTA of steps 1-6 reads its instance's state first and returns when the instance has
// converged or has no new vector in that slot.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "batch.cuh"
#include "gemm_f64.cuh"
#include "tda.cuh"

namespace tincr {

constexpr int BT_T = 256;
constexpr int BT_MAXR = 6;   // roots per instance (subspace up to 90, Jacobi in shared memory)

struct BtArrays {
    const BtInst *inst;
    BtState *state;
    double *C, *SC, *S, *blk, *glr, *gam, *omega, *V, *AV, *R, *Rk, *T, *sub, *H, *F, *D, *u, *err, *Y;
    const int *ao_off, *ao_atom;
    int *active;
    double tol;
};

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
        double *d = a.D + in.off_d;
        if (r < n && c == r + n) d[(long long)op.b * n + r] = acc;
        if (r >= n && c == r - n) d[(long long)(in.nr + op.b) * n + c] = acc;
        a.F[in.off_f + (long long)op.b * n2 * n2 + (long long)r * n2 + c] =
            -0.25 * a.glr[in.off_glr + (long long)rr * n + cc] * acc;
    }
};

// 4. G_b = F_b [SC_v;C_v]   (2n x v, written over H_b)
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
        op.M = in.o; op.N = in.v; op.K = n2;
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
// (non-LC instances in the products, every instance in the final pass)
__global__ void bt_diag_kernel(BtArrays a, int final_pass) {
    const int I = blockIdx.y, b = blockIdx.x;
    const BtInst in = a.inst[I];
    const double *X;
    if (!bt_vector(a, in, I, b, final_pass != 0, &X)) return;
    if (!final_pass && in.lc) return;
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
// diagonals (LC) or kept per AO (non-LC); in the final pass y is the transition charge of the root.
__global__ void bt_coulomb_kernel(BtArrays a, int final_pass) {
    extern __shared__ double ysh[];
    const int I = blockIdx.y, b = blockIdx.x;
    const BtInst in = a.inst[I];
    const double *X;
    if (!bt_vector(a, in, I, b, final_pass != 0, &X)) return;
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
            if (in.lc) {
                double *f = a.F + in.off_f + (long long)b * n2 * n2;
                f[(long long)mu * n2 + n + mu] += z;
                f[(long long)(n + mu) * n2 + mu] += z;
            } else {
                a.D[in.off_d + (long long)(2 * in.nr + b) * n + mu] = z;
            }
        }
    }
}

// non-LC: G_b = diag(z, z) [C_v;SC_v]  (written over H_b)
__global__ void bt_scale_rows_kernel(BtArrays a) {
    const int I = blockIdx.y, b = blockIdx.x;
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
// subspace step: one CTA per instance
// ----------------------------------------------------------------------------------------------

// sum over the CTA of NV values per thread; every thread receives the totals
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
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double s = 0.0;
        for (int w = 0; w < BT_T / 32; ++w) s += red[w * NV + q];
        v[q] = s;
    }
    __syncthreads();
}

__device__ __forceinline__ int bt_rr(int pos, int step, int mm) {
    return pos == 0 ? 0 : 1 + (pos - 1 + step) % (mm - 1);
}

// Cyclic Jacobi with the round-robin parallel ordering: A (m x m, symmetric) is diagonalised in
// place, Z receives the eigenvectors as columns.  Stops when the off-diagonal Frobenius norm is
// below 1e-14 of the total.
__device__ void bt_jacobi(int m, double *A, double *Z, double *cs, int *pq, double *red) {
    const int tid = threadIdx.x;
    for (int e = tid; e < m * m; e += BT_T) Z[e] = (e / m == e % m) ? 1.0 : 0.0;
    __syncthreads();
    if (m == 1) return;
    const int mm = (m + 1) & ~1, np = mm / 2;
    for (int sweep = 0; sweep < 40; ++sweep) {
        double s2[2] = {0.0, 0.0};
        for (int e = tid; e < m * m; e += BT_T) {
            const double x2 = A[e] * A[e];
            if (e / m == e % m) s2[1] += x2;
            else s2[0] += x2;
        }
        bt_block_sum<2>(s2, red);
        if (s2[0] <= 1e-28 * (s2[0] + s2[1])) break;
        for (int step = 0; step < mm - 1; ++step) {
            for (int k = tid; k < np; k += BT_T) {
                int p = bt_rr(k, step, mm), q = bt_rr(mm - 1 - k, step, mm);
                if (p > q) { const int t = p; p = q; q = t; }
                double c = 1.0, s = 0.0;
                if (q < m) {
                    const double apq = A[p * m + q];
                    if (apq != 0.0) {
                        const double theta = (A[q * m + q] - A[p * m + p]) / (2.0 * apq);
                        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                        c = 1.0 / sqrt(t * t + 1.0);
                        s = t * c;
                    }
                }
                cs[2 * k] = c;
                cs[2 * k + 1] = s;
                pq[2 * k] = p;
                pq[2 * k + 1] = q;
            }
            __syncthreads();
            for (int e = tid; e < np * m; e += BT_T) {   // A <- A J, Z <- Z J (columns p, q)
                const int k = e / m, r = e % m, p = pq[2 * k], q = pq[2 * k + 1];
                if (q >= m) continue;
                const double c = cs[2 * k], s = cs[2 * k + 1];
                const double ap = A[r * m + p], aq = A[r * m + q];
                A[r * m + p] = c * ap - s * aq;
                A[r * m + q] = s * ap + c * aq;
                const double zp = Z[r * m + p], zq = Z[r * m + q];
                Z[r * m + p] = c * zp - s * zq;
                Z[r * m + q] = s * zp + c * zq;
            }
            __syncthreads();
            for (int e = tid; e < np * m; e += BT_T) {   // A <- J^T A (rows p, q)
                const int k = e / m, r = e % m, p = pq[2 * k], q = pq[2 * k + 1];
                if (q >= m) continue;
                const double c = cs[2 * k], s = cs[2 * k + 1];
                const double ap = A[p * m + r], aq = A[q * m + r];
                A[p * m + r] = c * ap - s * aq;
                A[q * m + r] = s * ap + c * aq;
            }
            __syncthreads();
            for (int k = tid; k < np; k += BT_T) {
                const int p = pq[2 * k], q = pq[2 * k + 1];
                if (q < m) A[p * m + q] = A[q * m + p] = 0.0;
            }
            __syncthreads();
        }
    }
}

// shared memory of the subspace kernel (doubles) for subspaces up to mmax
inline size_t bt_subspace_smem(int mmax) {
    const size_t mm = (size_t)mmax + 1;
    return (2 * (size_t)mmax * mmax + 8 * BT_MAXR * (BT_T / 32) + 2 * mm + mmax + BT_MAXR + 16) * sizeof(double) +
           (2 * mm + BT_MAXR + 8) * sizeof(int);
}

__global__ void __launch_bounds__(BT_T) bt_subspace_kernel(BtArrays a) {
    const int I = blockIdx.x;
    const int tid = threadIdx.x;
    const BtInst in = a.inst[I];
    __shared__ BtState st;
    __shared__ int s_sel[BT_MAXR], s_nsel, s_action, s_mcur;
    __shared__ double s_u[BT_MAXR], s_err[BT_MAXR];
    if (tid == 0) st = a.state[I];
    __syncthreads();
    if (st.status != BT_RUNNING) return;
    const long long ov = in.ov;
    const int nr = in.nr, mmax = in.mmax;
    double *V = a.V + in.off_v, *AV = a.AV + in.off_v;
    double *R = a.R + in.off_r, *Rk = a.Rk + in.off_r, *T = a.T + in.off_r;
    double *P = a.sub + in.off_sub;
    const double *om = a.omega + in.off_omega;
    const int m = st.m, m_done = st.m_done;

    extern __shared__ double smem[];
    double *A = smem, *Z = A + (size_t)mmax * mmax;
    double *red = Z + (size_t)mmax * mmax;
    double *cs = red + 8 * BT_MAXR * (BT_T / 32);
    double *cdot = cs + 2 * (mmax + 1);
    int *pq = reinterpret_cast<int *>(cdot + mmax + BT_MAXR + 16);

    // 1. new columns of the projected matrix: P[i][j] = V_i . AV_j, j in [m_done, m)
    {
        const int warp = tid >> 5, lane = tid & 31, nw = BT_T / 32;
        const int kn = m - m_done;
        for (int e = warp; e < m * kn; e += nw) {
            const int i = e / kn, j = m_done + e % kn;
            const double *x = V + (long long)i * ov, *y = AV + (long long)j * ov;
            double s = 0.0;
            for (long long t = lane; t < ov; t += 32) s += x[t] * y[t];
            for (int off = 16; off; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
            if (lane == 0) P[(long long)i * mmax + j] = s;
        }
    }
    __syncthreads();
    // 2. eigenpairs of the upper triangle (davidson.rs:89-93)
    for (int e = tid; e < m * m; e += BT_T) {
        const int i = e / m, j = e % m;
        A[e] = i <= j ? P[(long long)i * mmax + j] : P[(long long)j * mmax + i];
    }
    __syncthreads();
    bt_jacobi(m, A, Z, cs, pq, red);
    if (tid == 0) {
        // the nr smallest eigenvalues in ascending order (ties: lower index first)
        unsigned long long used = 0, used2 = 0;
        for (int r = 0; r < nr; ++r) {
            int best = -1;
            for (int i = 0; i < m; ++i) {
                const bool u = i < 64 ? ((used >> i) & 1ull) : ((used2 >> (i - 64)) & 1ull);
                if (u) continue;
                if (best < 0 || A[i * m + i] < A[best * m + best]) best = i;
            }
            if (best < 64) used |= 1ull << best; else used2 |= 1ull << (best - 64);
            s_sel[r] = best;
            s_u[r] = A[best * m + best];
        }
    }
    __syncthreads();
    // 3. Ritz vectors R_r = sum_i y_ir V_i and residuals Rk_r = sum_i y_ir AV_i - u_r R_r (:101-107)
    double sq[BT_MAXR];
#pragma unroll
    for (int r = 0; r < BT_MAXR; ++r) sq[r] = 0.0;
    for (long long x = tid; x < ov; x += BT_T) {
        double rv[BT_MAXR], av[BT_MAXR];
#pragma unroll
        for (int r = 0; r < BT_MAXR; ++r) rv[r] = av[r] = 0.0;
        for (int i = 0; i < m; ++i) {
            const double vi = V[(long long)i * ov + x], ai = AV[(long long)i * ov + x];
#pragma unroll
            for (int r = 0; r < BT_MAXR; ++r)
                if (r < nr) {
                    const double y = Z[i * m + s_sel[r]];
                    rv[r] += y * vi;
                    av[r] += y * ai;
                }
        }
#pragma unroll
        for (int r = 0; r < BT_MAXR; ++r)
            if (r < nr) {
                const double rk = av[r] - s_u[r] * rv[r];
                R[(long long)r * ov + x] = rv[r];
                Rk[(long long)r * ov + x] = rk;
                sq[r] += rk * rk;
            }
    }
    bt_block_sum<BT_MAXR>(sq, red);
    // 4. convergence and the next action (:109-178)
    if (tid == 0) {
        st.products += m - m_done;
        int cvd = 0;
        bool finite = true;
        double mx = 0.0;
        for (int r = 0; r < nr; ++r) {
            const double e = sqrt(sq[r]);
            s_err[r] = e;
            a.u[in.off_u + r] = s_u[r];
            a.err[in.off_u + r] = e;
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
        } else if (lft == 0 && it > 0) {
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
            for (long long x = tid; x < ov; x += BT_T) {
                double d = w - om[x];
                if (fabs(d) < 1.0e-4) d = 1.0;
                T[(long long)j * ov + x] = Rk[(long long)r * ov + x] / d;
            }
        }
        __syncthreads();
        for (int j = 0; j < kadd; ++j) {
            double *t = T + (long long)j * ov;
            const int mc = s_mcur;
            for (int i0 = 0; i0 < mc; i0 += 8) {
                double c8[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) c8[q] = 0.0;
                for (long long x = tid; x < ov; x += BT_T) {
                    const double tx = t[x];
#pragma unroll
                    for (int q = 0; q < 8; ++q)
                        if (i0 + q < mc) c8[q] += V[(long long)(i0 + q) * ov + x] * tx;
                }
                bt_block_sum<8>(c8, red);
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    if (tid == q) cdot[i0 + q] = c8[q];
            }
            __syncthreads();
            double nr2[1] = {0.0};
            for (long long x = tid; x < ov; x += BT_T) {
                double s = t[x];
                for (int i = 0; i < mc; ++i) s -= cdot[i] * V[(long long)i * ov + x];
                t[x] = s;
                nr2[0] += s * s;
            }
            bt_block_sum<1>(nr2, red);
            const double nrm = sqrt(nr2[0]);
            if (!isfinite(nrm)) {
                if (tid == 0) st.status = BT_NONFINITE;
                break;
            }
            if (nrm > 1.0e-8 && mc < mmax) {
                const double inv = 1.0 / nrm;
                for (long long x = tid; x < ov; x += BT_T) V[(long long)mc * ov + x] = t[x] * inv;
                __syncthreads();
                if (tid == 0) s_mcur = mc + 1;
            }
            __syncthreads();
        }
        if (tid == 0) st.m = s_mcur;
    } else if (s_action == 2) {
        // 6. collapse onto the Ritz vectors (:172-176)
        for (long long x = tid; x < (long long)nr * ov; x += BT_T) V[x] = R[x];
        if (tid == 0) {
            st.dim_sub = nr;
            st.m = nr;
            st.m_done = 0;
            st.collapses += 1;
        }
    }
    __syncthreads();
    if (tid == 0) {
        a.state[I] = st;
        if (st.status == BT_RUNNING) atomicAdd(a.active, 1);
    }
}

// ----------------------------------------------------------------------------------------------
// host
// ----------------------------------------------------------------------------------------------

struct BatchWork {
    std::vector<BtInst> h;
    DevBuf<BtInst> inst;
    DevBuf<BtState> state;
    DevBuf<double> C, SC, S, blk, glr, glr_atoms, gam, omega, V, AV, R, Rk, T, sub, H, F, D, u, err, Y;
    DevBuf<int> ao_off, ao_atom, pos, active;
    DevBuf<long long> off_glr_atoms;
    DevBuf<int4> t_sc, t1, t2, t4, t5;
    cudaGraphExec_t graph = nullptr;
    ~BatchWork() {
        if (graph) cudaGraphExecDestroy(graph);
    }
};

static void upload_vec(cudaStream_t st, DevBuf<double> &d, const std::vector<double> &h) {
    d.reserve(std::max<size_t>(1, h.size()));
    if (!h.empty()) TINCR_CUDA(cudaMemcpyAsync(d.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, st));
}

template <class T>
static void upload_any(cudaStream_t st, DevBuf<T> &d, const std::vector<T> &h) {
    d.reserve(std::max<size_t>(1, h.size()));
    if (!h.empty()) TINCR_CUDA(cudaMemcpyAsync(d.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, st));
}

template <bool TA, bool TB, class Step>
static void bt_launch(Ctx &c, const DevBuf<int4> &tiles, size_t n_tiles, const Step &step, int family, double flops) {
    if (n_tiles == 0) return;
    int slot = c.prof_begin(family);
    bt_gemm_kernel<TA, TB, Step><<<(unsigned)n_tiles, GB_T, 0, c.stream>>>(tiles.p, step);
    count_launch(c.stream, "bt_gemm");
    check_launch("bt_gemm");
    c.prof_end(slot, flops, 0.0);
}

int Ctx::solve_batch(int n_inst, const tincr_tda_instance *hin, int max_iter, double tol, int precision,
                     tincr_tda_result *res) {
    if (n_inst <= 0 || !hin || !res || max_iter <= 0 || !(tol > 0.0)) fail(TINCR_BAD_ARG, "solve_batch: bad arguments");
    if (precision != TINCR_PREC_FP64) fail(TINCR_BAD_ARG, "solve_batch: only TINCR_PREC_FP64 is implemented");
    g_launches = 0;
    if (!batch) batch = new BatchWork();
    BatchWork &w = *batch;
    w.h.assign(n_inst, BtInst{});
    std::vector<double> hC, hS, hG, hGlr, hOm;
    std::vector<int> hAo, hAoAtom, hPos;
    std::vector<long long> hGlrOff(n_inst, 0);
    long long o_c = 0, o_s = 0, o_blk = 0, o_glr = 0, o_gam = 0, o_om = 0, o_v = 0, o_r = 0, o_sub = 0, o_h = 0, o_f = 0,
              o_d = 0, o_u = 0, o_y = 0;
    int o_ao = 0, o_aoatom = 0, mmax_all = 1, nr_max = 1, nmax_atoms = 1;
    for (int I = 0; I < n_inst; ++I) {
        const tincr_tda_instance &q = hin[I];
        if (q.n_atoms <= 0 || q.n_orb <= 0 || q.n_occ <= 0 || q.n_virt <= 0 || q.n_occ + q.n_virt > q.n_orb ||
            q.n_roots <= 0 || q.n_roots > BT_MAXR || (long long)q.n_roots > (long long)q.n_occ * q.n_virt ||
            !q.orbs_per_atom || !q.c || !q.s || !q.orbe || !q.gamma || !q.xyz)
            fail(TINCR_BAD_ARG, "solve_batch: instance " + std::to_string(I) + " is malformed (n_roots <= 6)");
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
        b.off_ao = o_ao; o_ao += N + 1;
        b.off_aoatom = o_aoatom; o_aoatom += n;
        mmax_all = std::max(mmax_all, b.mmax);
        nr_max = std::max(nr_max, b.nr);
        nmax_atoms = std::max(nmax_atoms, N);
        // host-side copies into the packed arrays
        check_finite(q.c, (size_t)n * w_, "c");
        check_finite(q.s, (size_t)n * n, "s");
        check_finite(q.orbe, (size_t)w_, "orbe");
        check_finite(q.gamma, (size_t)N * N, "gamma");
        hC.insert(hC.end(), q.c, q.c + (size_t)n * w_);
        hS.insert(hS.end(), q.s, q.s + (size_t)n * n);
        hG.insert(hG.end(), q.gamma, q.gamma + (size_t)N * N);
        if (b.lc) {
            check_finite(q.gamma_lr, (size_t)N * N, "gamma_lr");
            hGlrOff[I] = (long long)hGlr.size();
            hGlr.insert(hGlr.end(), q.gamma_lr, q.gamma_lr + (size_t)N * N);
        }
        int off = 0;
        for (int A = 0; A < N; ++A) {
            hAo.push_back(off);
            for (int k = 0; k < q.orbs_per_atom[A]; ++k) hAoAtom.push_back(A);
            off += q.orbs_per_atom[A];
        }
        hAo.push_back(off);
        // omega_ia = e_a - e_i (excited_states/utils.rs:8-22) and the guess positions (stable ties)
        std::vector<double> om(b.ov);
        for (int i = 0; i < b.o; ++i)
            for (int x = 0; x < b.v; ++x) om[(size_t)i * b.v + x] = q.orbe[b.o + x] - q.orbe[i];
        hOm.insert(hOm.end(), om.begin(), om.end());
        std::vector<int> ord(b.ov);
        std::iota(ord.begin(), ord.end(), 0);
        std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return om[x] < om[y]; });
        for (int r = 0; r < b.nr; ++r) hPos.push_back(ord[r]);
    }
    // device arrays
    upload_any(stream, w.inst, w.h);
    w.state.reserve(n_inst);
    upload_vec(stream, w.C, hC);
    w.SC.reserve(std::max<long long>(1, o_c));
    upload_vec(stream, w.S, hS);
    w.blk.reserve(std::max<long long>(1, o_blk));
    w.glr.reserve(std::max<long long>(1, o_glr));
    upload_vec(stream, w.glr_atoms, hGlr);
    upload_any(stream, w.off_glr_atoms, hGlrOff);
    upload_vec(stream, w.gam, hG);
    upload_vec(stream, w.omega, hOm);
    w.V.reserve(o_v);
    w.AV.reserve(o_v);
    w.R.reserve(o_r);
    w.Rk.reserve(o_r);
    w.T.reserve(o_r);
    w.sub.reserve(o_sub);
    w.H.reserve(o_h);
    w.F.reserve(std::max<long long>(1, o_f));
    w.D.reserve(o_d);
    w.u.reserve(o_u);
    w.err.reserve(o_u);
    w.Y.reserve(o_y);
    upload_any(stream, w.ao_off, hAo);
    upload_any(stream, w.ao_atom, hAoAtom);
    upload_any(stream, w.pos, hPos);
    w.active.reserve(1);

    // static tile tables
    std::vector<int4> tsc, t1, t2, t4, t5;
    for (int I = 0; I < n_inst; ++I) {
        const BtInst &b = w.h[I];
        const int n2 = 2 * b.n;
        for (int tm = 0; tm < ceil_div(b.n, GB_M); ++tm)
            for (int tn = 0; tn < ceil_div(b.o + b.v, GB_N); ++tn) tsc.push_back(make_int4(I, 0, tm, tn));
        for (int s = 0; s < b.nr; ++s) {
            for (int tm = 0; tm < ceil_div(n2, GB_M); ++tm)
                for (int tn = 0; tn < ceil_div(b.v, GB_N); ++tn) {
                    t1.push_back(make_int4(I, s, tm, tn));
                    if (b.lc) t4.push_back(make_int4(I, s, tm, tn));
                }
            if (b.lc)
                for (int tm = 0; tm < ceil_div(n2, GB_M); ++tm)
                    for (int tn = 0; tn < ceil_div(n2, GB_N); ++tn) t2.push_back(make_int4(I, s, tm, tn));
            for (int tm = 0; tm < ceil_div(b.o, GB_M); ++tm)
                for (int tn = 0; tn < ceil_div(b.v, GB_N); ++tn) t5.push_back(make_int4(I, s, tm, tn));
        }
    }
    upload_any(stream, w.t_sc, tsc);
    upload_any(stream, w.t1, t1);
    upload_any(stream, w.t2, t2);
    upload_any(stream, w.t4, t4);
    upload_any(stream, w.t5, t5);

    BtArrays a{};
    a.inst = w.inst.p; a.state = w.state.p;
    a.C = w.C.p; a.SC = w.SC.p; a.S = w.S.p; a.blk = w.blk.p; a.glr = w.glr.p; a.gam = w.gam.p; a.omega = w.omega.p;
    a.V = w.V.p; a.AV = w.AV.p; a.R = w.R.p; a.Rk = w.Rk.p; a.T = w.T.p; a.sub = w.sub.p; a.H = w.H.p; a.F = w.F.p;
    a.D = w.D.p; a.u = w.u.p; a.err = w.err.p; a.Y = w.Y.p; a.ao_off = w.ao_off.p; a.ao_atom = w.ao_atom.p;
    a.active = w.active.p; a.tol = tol;

    TINCR_CUDA(cudaEventRecord(ev0, stream));
    // set-up: SC, packed blocks, gamma_lr in the AO basis, guesses
    bt_launch<false, false>(*this, w.t_sc, tsc.size(), BtStepSC{a}, TINCR_KF_OTHER, 0.0);
    bt_pack_kernel<<<n_inst, BT_T, 0, stream>>>(a);
    count_launch(stream, "bt_pack");
    check_launch("bt_pack");
    if (!hGlr.empty()) {
        bt_expand_kernel<<<n_inst, BT_T, 0, stream>>>(a, w.glr_atoms.p, w.off_glr_atoms.p);
        count_launch(stream, "bt_expand");
        check_launch("bt_expand");
    }
    bt_guess_kernel<<<n_inst, BT_T, 0, stream>>>(a, w.pos.p);
    count_launch(stream, "bt_guess");
    check_launch("bt_guess");

    const size_t sub_smem = bt_subspace_smem(mmax_all);
    TINCR_CUDA(cudaFuncSetAttribute(bt_subspace_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sub_smem));
    const size_t coul_smem = (size_t)nmax_atoms * sizeof(double);
    if (coul_smem > 48 * 1024)
        TINCR_CUDA(cudaFuncSetAttribute(bt_coulomb_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)coul_smem));
    const dim3 gv(nr_max, n_inst);

    // one Davidson iteration of every running instance (captured once as a graph)
    auto iteration = [&]() {
        bt_launch<false, false>(*this, w.t1, t1.size(), BtStep1{a, false}, TINCR_KF_AO_TRANSFORM, 0.0);
        bt_launch<false, true>(*this, w.t2, t2.size(), BtStep2{a}, TINCR_KF_AO_EXCHANGE, 0.0);
        bt_diag_kernel<<<gv, BT_T, 0, stream>>>(a, 0);
        count_launch(stream, "bt_diag");
        check_launch("bt_diag");
        bt_coulomb_kernel<<<gv, BT_T, coul_smem, stream>>>(a, 0);
        count_launch(stream, "bt_coulomb");
        check_launch("bt_coulomb");
        bt_launch<false, false>(*this, w.t4, t4.size(), BtStep4{a}, TINCR_KF_AO_EXCHANGE, 0.0);
        bt_scale_rows_kernel<<<gv, BT_T, 0, stream>>>(a);
        count_launch(stream, "bt_scale_rows");
        check_launch("bt_scale_rows");
        bt_launch<true, false>(*this, w.t5, t5.size(), BtStep5{a}, TINCR_KF_AO_TRANSFORM, 0.0);
        TINCR_CUDA(cudaMemsetAsync(w.active.p, 0, sizeof(int), stream));
        bt_subspace_kernel<<<n_inst, BT_T, sub_smem, stream>>>(a);
        count_launch(stream, "bt_subspace");
        check_launch("bt_subspace");
    };
    int iters = 0, active = n_inst;
    const bool use_graph = !profiling;
    cudaGraphExec_t exec = nullptr;
    if (use_graph) {
        cudaGraph_t g = nullptr;
        TINCR_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        long long before = g_launches;
        iteration();
        const long long per_iter = g_launches - before;
        g_launches = before;
        TINCR_CUDA(cudaStreamEndCapture(stream, &g));
        TINCR_CUDA(cudaGraphInstantiate(&exec, g, 0));
        cudaGraphDestroy(g);
        while (active > 0 && iters < max_iter) {
            TINCR_CUDA(cudaGraphLaunch(exec, stream));
            g_launches += per_iter;
            ++iters;
            TINCR_CUDA(cudaMemcpyAsync(&active, w.active.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
            sync();
        }
        cudaGraphExecDestroy(exec);
    } else {
        while (active > 0 && iters < max_iter) {
            iteration();
            ++iters;
            TINCR_CUDA(cudaMemcpyAsync(&active, w.active.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
            sync();
        }
    }
    // final pass: transition charges of the Ritz vectors
    bt_launch<false, false>(*this, w.t1, t1.size(), BtStep1{a, true}, TINCR_KF_OTHER, 0.0);
    bt_diag_kernel<<<gv, BT_T, 0, stream>>>(a, 1);
    count_launch(stream, "bt_diag");
    check_launch("bt_diag");
    bt_coulomb_kernel<<<gv, BT_T, coul_smem, stream>>>(a, 1);
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
    sync();
    int worst = TINCR_OK;
    last_products = 0;
    for (int I = 0; I < n_inst; ++I) {
        const BtInst &b = w.h[I];
        const tincr_tda_instance &q = hin[I];
        tincr_tda_result &o = res[I];
        const BtState &s = hs[I];
        o.iterations = s.iter;
        o.status = s.status == BT_CONVERGED ? TINCR_OK
                 : s.status == BT_NONFINITE ? TINCR_NONFINITE : TINCR_NOT_CONVERGED;
        if (o.status == TINCR_NONFINITE) worst = TINCR_NONFINITE;
        else if (o.status == TINCR_NOT_CONVERGED && worst == TINCR_OK) worst = TINCR_NOT_CONVERGED;
        last_products += s.products;
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
