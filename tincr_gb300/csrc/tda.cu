// Linear-response TDA / LC-TDA on the GPU: transition charges, the AO-direct A.X product and the
// block Davidson solver.
//
// AO-direct product.  tincr's Mulliken transition charges are
//     q^A_pq = 1/2 sum_{mu in A} (C_mu,p (SC)_mu,q + (SC)_mu,p C_mu,q)
// (src/excited_states/transition_charges.rs:8-98), so every contraction q.gamma.q of the CIS
// matrix (src/excited_states/solvers/mod.rs:280-369) can be carried out in the AO basis without
// ever forming q_ov / q_oo / q_vv.  With Co, Cv the occupied / virtual MO coefficients and
// SCo = (S C)_occ, SCv = (S C)_virt, for one trial vector X [o x v]:
//     H  = [Co; SCo] X                      [2n x v]
//     M  = H [Cv; SCv]^T                    [2n x 2n] = [[Co X Cv^T, Co X SCv^T], [SCo X Cv^T, SCo X SCv^T]]
//     y_A = 1/2 sum_{mu in A} (M[mu, n+mu] + M[n+mu, mu])         ( = (q_ov X)_A )
//     z   = gamma y,  z_mu = z_{A(mu)}
//     F  = -1/4 (gamma_lr_AO o M)  +  z on the diagonals of the two off-diagonal blocks
//     AX = omega o X + [SCo; Co]^T F [SCv; Cv]
// which equals omega o X + 2 q_ov^T gamma q_ov X - K_lr X exactly (K_lr the long-range exchange
// sum_jb (ij|ab)_lr X_jb).  Cost per vector 8 n o v + 16 n^2 v instead of 2 N o v (o + v).
// Without long-range correction F is diagonal-only and the two n^2 v products drop out.
#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <vector>

#include <cooperative_groups.h>

#include "common.cuh"
#include "kernels.cuh"
#include "gemm_f64.cuh"
#include "ops.cuh"
#include "subspace.cuh"
#include "tda.cuh"

namespace cg = cooperative_groups;

namespace tincr {

thread_local long long g_launches = 0;

[[noreturn]] void fail(int status, const std::string &msg) { throw Error{status, msg}; }

void check_cuda(cudaError_t e, const char *what) {
    if (e != cudaSuccess) fail(TINCR_CUDA_ERR, std::string(what) + ": " + cudaGetErrorString(e));
}

void check_launch(const char *name) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) fail(TINCR_CUDA_ERR, std::string("launch ") + name + ": " + cudaGetErrorString(e));
}

bool eigh_upper(int n, const double *a, double *w, double *z);

// ----------------------------------------------------------------------------------------------
// small kernels
// ----------------------------------------------------------------------------------------------

// Lst = [Co; SCo] (2n x o), Rv = [Cv; SCv] (2n x v), Lsw = [SCo; Co], Rsw = [SCv; Cv]
__global__ void pack_blocks_kernel(int n, int o, int v, const double *__restrict__ C, const double *__restrict__ SC,
                                   double *Lst, double *Rv, double *Lsw, double *Rsw) {
    long long total = 2LL * n * (o + v);
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        int r = int(t / (o + v));
        int c = int(t % (o + v));
        int mu = r < n ? r : r - n;
        double cv = C[(long long)mu * n + c];
        double sv = SC[(long long)mu * n + c];
        if (c < o) {
            Lst[(long long)r * o + c] = r < n ? cv : sv;
            Lsw[(long long)r * o + c] = r < n ? sv : cv;
        } else {
            int a = c - o;
            Rv[(long long)r * v + a] = r < n ? cv : sv;
            Rsw[(long long)r * v + a] = r < n ? sv : cv;
        }
    }
}

// out[mu][nu] = g[A(mu)][A(nu)]
__global__ void expand_ao_kernel(int n, int n_atoms, const int *__restrict__ ao_atom, const double *__restrict__ g,
                                 double *out) {
    long long total = (long long)n * n;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        int mu = int(t / n), nu = int(t % n);
        out[t] = g[(long long)ao_atom[mu] * n_atoms + ao_atom[nu]];
    }
}

// q^A_pq = 1/2 sum_{mu in A} (C_mu,p SC_mu,q + SC_mu,p C_mu,q) for p in [p0, p0+np), q in [q0, q0+nq)
// (transition_charges.rs:38-95).  One thread per output element, q fastest (coalesced stores).
__global__ void trans_charges_kernel(int n, int n_atoms, const int *__restrict__ ao_off, const double *__restrict__ C,
                                     const double *__restrict__ SC, int p0, int np, int q0, int nq, double *out) {
    int A = blockIdx.y;
    long long per = (long long)np * nq;
    int mu0 = ao_off[A], mu1 = ao_off[A + 1];
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < per; t += (long long)gridDim.x * blockDim.x) {
        int p = int(t / nq) + p0, q = int(t % nq) + q0;
        double s = 0.0;
        for (int mu = mu0; mu < mu1; ++mu) {
            const double *c = C + (long long)mu * n;
            const double *sc = SC + (long long)mu * n;
            s += 0.5 * (c[p] * sc[q] + c[q] * sc[p]);
        }
        out[(long long)A * per + t] = s;
    }
}

// Diagonals of the AO blocks without forming them: with H_b = [C_R; SC_R] V_b and St = [C_S; SC_S],
// d3[b][mu] = sum_s H_b[mu][s] St[n+mu][s], d2[b][mu] = sum_s H_b[n+mu][s] St[mu][s];
// row m of H_b at H + b * sbh + m * ldh
__global__ void diag_dots_kernel(int n, int v, const double *__restrict__ H, long long ldh, long long sbh,
                                 const double *__restrict__ Rv, double *d3, double *d2) {
    int b = blockIdx.y;
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= 2 * n) return;
    int mu = warp < n ? warp : warp - n;
    const double *h = H + (long long)b * sbh + (long long)warp * ldh;
    const double *r = Rv + (long long)(warp < n ? n + mu : mu) * v;
    double s = 0.0;
    for (int a = lane; a < v; a += 32) s += h[a] * r[a];
    for (int off = 16; off; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if (lane == 0) (warp < n ? d3 : d2)[(long long)b * n + mu] = s;
}

// Coulomb: y_A = 1/2 sum_{mu in A}(d3 + d2); z = gamma y; zao_mu = z_{A(mu)}.  Grid (atoms / 8,
// vectors): every CTA forms y of its vector, each warp one z_A.  Optionally adds zao to F's
// off-diagonal-block diagonals (LC) and writes y (transition charges).
__global__ void __launch_bounds__(256)
coulomb_kernel(int n, int n_atoms, const int *__restrict__ ao_off, const double *__restrict__ gamma,
               const double *__restrict__ d3, const double *__restrict__ d2, double *zao, double *F, double *y_out,
               double scale) {
    extern __shared__ double sh[];
    double *y = sh;            // [n_atoms]
    const int b = blockIdx.y;
    const double *D3 = d3 + (long long)b * n, *D2 = d2 + (long long)b * n;
    for (int A = threadIdx.x; A < n_atoms; A += blockDim.x) {
        double s = 0.0;
        for (int mu = ao_off[A]; mu < ao_off[A + 1]; ++mu) s += D3[mu] + D2[mu];
        y[A] = 0.5 * s;
        if (y_out && blockIdx.x == 0) y_out[(long long)b * n_atoms + A] = 0.5 * s;
    }
    __syncthreads();
    // one warp per atom: z_A = scale sum_B gamma_AB y_B (coalesced gamma row)
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int A = blockIdx.x * COULOMB_ATOMS + warp;
    if (A >= n_atoms) return;
    const double *g = gamma + (long long)A * n_atoms;
    double z = 0.0;
    for (int B = lane; B < n_atoms; B += 32) z += g[B] * y[B];
    for (int off = 16; off; off >>= 1) z += __shfl_xor_sync(0xffffffffu, z, off);
    z *= scale;
    const int n2 = 2 * n;
    for (int mu = ao_off[A] + lane; mu < ao_off[A + 1]; mu += 32) {
        if (zao) zao[(long long)b * n + mu] = z;
        if (F) {
            double *f = F + (long long)b * n2 * n2;
            f[(long long)mu * n2 + n + mu] += z;
            f[(long long)(n + mu) * n2 + mu] += z;
        }
    }
}

void launch_coulomb(cudaStream_t st, int kc, int n, int n_atoms, const int *ao_off, const double *gamma,
                    const double *d3, const double *d2, double *zao, double *F, double *y_out, double scale) {
    dim3 g(ceil_div(n_atoms, COULOMB_ATOMS), kc);
    coulomb_kernel<<<g, 32 * COULOMB_ATOMS, n_atoms * sizeof(double), st>>>(n, n_atoms, ao_off, gamma, d3, d2, zao, F,
                                                                            y_out, scale);
    count_launch(st, "coulomb");
    check_launch("coulomb");
}

// F diagonal-only (no exchange term): G_b = F_b [SC_Q; C_Q] = diag(z, z) [C_Q; SC_Q]
__global__ void scale_rows_kernel(int n, int v, const double *__restrict__ zao, const double *__restrict__ Rv,
                                  double *G) {
    int b = blockIdx.y;
    long long total = 2LL * n * v;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        int r = int(t / v);
        int mu = r < n ? r : r - n;
        // row r < n pairs with Cv (Rv row mu); row n+mu pairs with SCv (Rv row n+mu)
        G[(long long)b * total + t] = zao[(long long)b * n + mu] * Rv[t];
    }
}

// out[r][x] = in[x][r] (dense transpose, rows x cols -> cols x rows)
__global__ void transpose_kernel(int rows, int cols, const double *__restrict__ in, double *out) {
    __shared__ double tile[32][33];
    int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += 8) {
        int r = by + j, c = bx + threadIdx.x;
        if (r < rows && c < cols) tile[j][threadIdx.x] = in[(long long)r * cols + c];
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += 8) {
        int r = bx + j, c = by + threadIdx.x;
        if (r < cols && c < rows) out[(long long)r * rows + c] = tile[threadIdx.x][j];
    }
}

// row norms: out[r] = ||A[r]||_2 (one CTA per row)

// T[j][x] = Rk[idx_j][x] / denom with denom = w_j - omega[x], |denom| < 1e-4 -> 1 (solvers/mod.rs:373-380)
__global__ void precondition_kernel(long long ov, int k, const int *__restrict__ idx, const double *__restrict__ w,
                                    const double *__restrict__ Rk, const double *__restrict__ omega, double *T) {
    int j = blockIdx.y;
    const double *r = Rk + (long long)idx[j] * ov;
    double wj = w[j];
    for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < ov; x += (long long)gridDim.x * blockDim.x) {
        double d = wj - omega[x];
        if (fabs(d) < 1.0e-4) d = 1.0;
        T[(long long)j * ov + x] = r[x] / d;
    }
}

// Deterministic multi-CTA row norms: partial[r][c] = sum of A[r][x]^2 over chunk c (pass 1),
// out[r] = sqrt(sum_c partial[r][c]) in chunk order (pass 2).
__global__ void row_sq_partial_kernel(long long len, int chunks, const double *__restrict__ A, long long lda,
                                      double *partial) {
    __shared__ double red[32];
    const int r = blockIdx.y, c = blockIdx.x;
    const long long per = (len + chunks - 1) / chunks;
    const long long x0 = (long long)c * per, x1 = x0 + per < len ? x0 + per : len;
    const double *a = A + (long long)r * lda;
    double s = 0.0;
    for (long long x = x0 + threadIdx.x; x < x1; x += blockDim.x) s += a[x] * a[x];
    for (int off = 16; off; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        for (int off = 16; off; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
        if (threadIdx.x == 0) partial[(long long)r * chunks + c] = s;
    }
}

__global__ void row_sq_finish_kernel(int rows, int chunks, const double *__restrict__ partial, double *out) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    double s = 0.0;
    for (int c = 0; c < chunks; ++c) s += partial[(long long)r * chunks + c];
    out[r] = sqrt(s);
}

// Sequential Gram-Schmidt of the kadd correction vectors T against the vectors accepted in this step
// (davidson.rs:162-168): t -= sum_i (q_i . t) q_i over the accepted q_i, then accept t / |t| when
// |t| > 1e-8 (and the basis has room), else drop it.  One cooperative launch, one grid barrier per
// vector: the pass that forms t'_j = t_j - sum_i c_i q_i (into its destination row) and |t'_j|^2
// also accumulates the dots of the next vector t_{j+1} with every accepted q_i and with t'_j, so the
// accepted rows are read once per vector.  After the barrier every CTA reduces the partial sums in
// the same fixed order and takes the same decision; when t'_j is accepted its dot with t_{j+1} joins
// the next coefficients.  Normalisation is deferred: an accepted row is kept as t' with the factor
// 1/|t'|, which the coefficients apply, and every accepted row is scaled in place at the end.
// state[0]: m out; state[1]: 1 if a norm was not finite.  part: [2][gridDim.x][GS_SLOTS] doubles.
constexpr int GS_MAX = 32, GS_SLOTS = GS_MAX + 2;
__global__ void __launch_bounds__(256) seq_gs_kernel(int kadd, long long ov, int m0, int mmax, double *V, double *T,
                                                     double *part, int *state) {
    cg::grid_group grid = cg::this_grid();
    __shared__ double c[GS_MAX], sc[GS_MAX], tot[GS_SLOTS];
    __shared__ double red[8][GS_SLOTS];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long x0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    int m = m0;
    bool finite = true;
    int ncoef = 0;   // coefficients c[0 .. ncoef) of the current vector (its dots with the accepted rows)
    for (int j = 0; j < kadd && finite; ++j) {
        const int acc = m - m0;
        const double *t = T + (long long)j * ov;
        const double *tn = j + 1 < kadd ? T + (long long)(j + 1) * ov : nullptr;
        double *dst = m < mmax ? V + (long long)m * ov : T + (long long)j * ov;
        double d[GS_MAX + 1];
#pragma unroll
        for (int i = 0; i <= GS_MAX; ++i) d[i] = 0.0;
        double sq = 0.0;
        for (long long x = x0; x < ov; x += stride) {
            double v = t[x];
            const double tnx = tn ? tn[x] : 0.0;
#pragma unroll
            for (int i = 0; i < GS_MAX; ++i)
                if (i < acc) {
                    const double q = V[(long long)(m0 + i) * ov + x];
                    if (i < ncoef) v -= c[i] * q;
                    d[i] += q * tnx;
                }
            dst[x] = v;
            sq += v * v;
            d[GS_MAX] += v * tnx;
        }
        // block partials: slots 0 .. acc-1 (dots with q_i), GS_MAX (dot with t'_j), GS_MAX + 1 (|t'_j|^2).
        // The 32 dot slots are reduced over the warp by halving exchanges (lane L ends with slot L:
        // 31 shuffle-adds instead of 160; GB300's FP64 unit takes ~64 cycles per warp instruction).
        double *pb = part + ((long long)(j & 1) * gridDim.x + blockIdx.x) * GS_SLOTS;
        {
            double a16[16], a8[8], a4[4], a2[2];
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                const bool h = lane & 16;
                a16[q] = (h ? d[q + 16] : d[q]) + __shfl_xor_sync(0xffffffffu, h ? d[q] : d[q + 16], 16);
            }
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const bool h = lane & 8;
                a8[q] = (h ? a16[q + 8] : a16[q]) + __shfl_xor_sync(0xffffffffu, h ? a16[q] : a16[q + 8], 8);
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const bool h = lane & 4;
                a4[q] = (h ? a8[q + 4] : a8[q]) + __shfl_xor_sync(0xffffffffu, h ? a8[q] : a8[q + 4], 4);
            }
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const bool h = lane & 2;
                a2[q] = (h ? a4[q + 2] : a4[q]) + __shfl_xor_sync(0xffffffffu, h ? a4[q] : a4[q + 2], 2);
            }
            const bool h = lane & 1;
            red[warp][lane] = (h ? a2[1] : a2[0]) + __shfl_xor_sync(0xffffffffu, h ? a2[0] : a2[1], 1);
            double vc = d[GS_MAX], vs = sq;
            for (int off = 16; off; off >>= 1) {
                vc += __shfl_xor_sync(0xffffffffu, vc, off);
                vs += __shfl_xor_sync(0xffffffffu, vs, off);
            }
            if (lane == 0) {
                red[warp][GS_MAX] = vc;
                red[warp][GS_MAX + 1] = vs;
            }
        }
        __syncthreads();
        if (threadIdx.x < GS_SLOTS && (threadIdx.x < acc || threadIdx.x >= GS_MAX)) {
            double v = 0.0;
            for (int w = 0; w < 8; ++w) v += red[w][threadIdx.x];
            pb[threadIdx.x] = v;
        }
        grid.sync();
        // every CTA: the sums over the CTAs of the used slots, in a fixed order (warp w takes slots
        // w, w + 8, ...: lanes stride over the CTAs, then a shuffle tree), so every CTA holds the same
        // totals; then the norm of t'_j, accept or drop, and the next vector's coefficients
        const double *pj = part + (long long)(j & 1) * gridDim.x * GS_SLOTS;
        for (int i = warp; i < GS_SLOTS; i += 8) {
            if (!(i < acc || i >= GS_MAX)) continue;   // uniform over the warp
            double v = 0.0;
            for (int b = lane; b < (int)gridDim.x; b += 32) v += pj[(long long)b * GS_SLOTS + i];
            for (int off = 16; off; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            if (lane == 0) tot[i] = v;
        }
        __syncthreads();
        const double nrm = sqrt(tot[GS_MAX + 1]);
        if (!isfinite(nrm)) {
            if (blockIdx.x == 0 && threadIdx.x == 0) state[1] = 1;
            finite = false;   // every CTA sees the same norm
            break;
        }
        const bool accept = nrm > 1.0e-8 && m < mmax;
        __syncthreads();   // c and sc of this vector are no longer read
        if (threadIdx.x < acc || (accept && threadIdx.x == acc)) {
            const int i = threadIdx.x;
            const double v = tot[i < acc ? i : GS_MAX];
            const double f = i < acc ? sc[i] : 1.0 / nrm;
            if (i == acc) sc[i] = f;
            c[i] = v * f * f;   // (q_i . t_{j+1}) / |t'_i|^2 with the unscaled row t'_i
        }
        __syncthreads();
        if (accept) ++m;
        ncoef = m - m0;
        // part[(j + 1) & 1] is written next; every CTA has passed the barrier of vector j - 1, whose
        // partials (same parity) it read before that barrier's successor
    }
    // scale the accepted rows
    for (int i = 0; i < m - m0; ++i) {
        double *q = V + (long long)(m0 + i) * ov;
        const double f = sc[i];
        for (long long x = x0; x < ov; x += stride) q[x] *= f;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) state[0] = m;
}

// dst = src * s  (vector scaled copy)
__global__ void scale_copy_kernel(long long len, const double *__restrict__ src, double s, double *dst) {
    for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < len; x += (long long)gridDim.x * blockDim.x)
        dst[x] = src[x] * s;
}

// unit vectors: V[j][pos[j]] = 1 (V pre-zeroed)
__global__ void unit_vectors_kernel(int k, long long ov, const int *__restrict__ pos, double *V) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < k) V[(long long)j * ov + pos[j]] = 1.0;
}

// ----------------------------------------------------------------------------------------------
// profiling
// ----------------------------------------------------------------------------------------------

int Ctx::prof_begin(int family) {
    if (!profiling) return -1;
    cudaEvent_t a, b;
    if (event_pool.size() >= 2) {
        a = event_pool.back(); event_pool.pop_back();
        b = event_pool.back(); event_pool.pop_back();
    } else {
        TINCR_CUDA(cudaEventCreate(&a));
        TINCR_CUDA(cudaEventCreate(&b));
    }
    TINCR_CUDA(cudaEventRecord(a, stream));
    pending.push_back({family, a, b, 0.0, 0.0});
    return (int)pending.size() - 1;
}

void Ctx::prof_end(int slot, double flops, double bytes) {
    if (slot < 0) return;
    TINCR_CUDA(cudaEventRecord(pending[slot].b, stream));
    pending[slot].flops = flops;
    pending[slot].bytes = bytes;
}

void Ctx::prof_resolve() {
    for (auto &p : pending) {
        float ms = 0.f;
        TINCR_CUDA(cudaEventElapsedTime(&ms, p.a, p.b));
        KernelStats &s = stats[p.family];
        s.ms += ms;
        s.launches += 1;
        s.flops += p.flops;
        s.bytes += p.bytes;
        event_pool.push_back(p.a);
        event_pool.push_back(p.b);
    }
    pending.clear();
}

// ----------------------------------------------------------------------------------------------
// launch helpers
// ----------------------------------------------------------------------------------------------

static int grid_for(long long work, int threads, int n_sm) {
    long long b = (work + threads - 1) / threads;
    long long cap = 32LL * n_sm;
    return int(std::max<long long>(1, std::min(b, cap)));
}

void Ctx::launch_transpose(int rows, int cols, const double *in, double *out) {
    dim3 grid(ceil_div(cols, 32), ceil_div(rows, 32));
    transpose_kernel<<<grid, dim3(32, 8), 0, stream>>>(rows, cols, in, out);
    count_launch(stream, "transpose");
    check_launch("transpose");
}

// ----------------------------------------------------------------------------------------------
// context
// ----------------------------------------------------------------------------------------------

Ctx::Ctx(int dev) : device(dev) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= dev || dev < 0)
        fail(TINCR_NO_DEVICE, "no CUDA device " + std::to_string(dev));
    TINCR_CUDA(cudaSetDevice(dev));
    cudaDeviceProp prop{};
    TINCR_CUDA(cudaGetDeviceProperties(&prop, dev));
    if (prop.major != 10 || prop.minor != 3)
        fail(TINCR_NO_DEVICE, std::string("device is not sm_103: ") + prop.name);
    n_sm = prop.multiProcessorCount;
    TINCR_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    TINCR_CUDA(cudaEventCreate(&ev0));
    TINCR_CUDA(cudaEventCreate(&ev1));
    // co-resident grid of the cooperative Gram-Schmidt kernel (0: cooperative launch unavailable)
    int coop = 0, per_sm = 0;
    TINCR_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    TINCR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, seq_gs_kernel, 256, 0));
    coop_grid = coop ? std::min(1, per_sm) * n_sm : 0;
    // plane GEMM of the mixed-precision contraction: tcgen05 (default) or warp MMA
    const char *pg = std::getenv("TINCR_GB300_PLANE_GEMM");
    if (pg && std::string(pg) == "mma") use_tc = false;
    // Davidson subspace eigensolver: host (default) or the thread-block cluster kernel
    const char *se = std::getenv("TINCR_GB300_SUBSPACE_EIG");
    if (se && std::string(se) == "cluster") eig_cluster_on = true;
    // subspace products of the mixed Davidson: digit GEMMs on the tensor cores (default) or FP64
    const char *sg = std::getenv("TINCR_GB300_SUBSPACE_GEMM");
    if (sg && std::string(sg) == "fp64") use_digits = false;
}

Ctx::~Ctx() {
    cudaSetDevice(device);
    release_batch(batch);
    if (h_tc_err) cudaFreeHost(h_tc_err);
    for (auto &p : pending) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
    for (auto e : event_pool) cudaEventDestroy(e);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
}

// Every host synchronisation also reports a bounded-wait failure of the tensor-core kernels queued
// before it (tc_err_watch), so those launches need no synchronisation of their own.
void Ctx::sync() {
    TINCR_CUDA(cudaStreamSynchronize(stream));
    if (h_tc_err && *h_tc_err) {
        const int e = *h_tc_err;
        *h_tc_err = 0;
        TINCR_CUDA(cudaMemsetAsync(d_tc_err.p, 0, sizeof(int), stream));
        TINCR_CUDA(cudaStreamSynchronize(stream));
        fail(TINCR_CUDA_ERR, "tensor-core GEMM: a pipeline wait timed out (code " + std::to_string(e) + ")");
    }
}

void Ctx::tc_err_ensure() {
    if (d_tc_err.p) return;
    d_tc_err.alloc(1);
    TINCR_CUDA(cudaMemsetAsync(d_tc_err.p, 0, sizeof(int), stream));
    if (!h_tc_err) {
        TINCR_CUDA(cudaMallocHost(&h_tc_err, sizeof(int)));
        *h_tc_err = 0;
    }
}

void Ctx::tc_err_watch() {
    if (d_tc_err.p && h_tc_err)
        TINCR_CUDA(cudaMemcpyAsync(h_tc_err, d_tc_err.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
}

// norms of `rows` vectors of length len (stride lda) into out[rows], spread over the whole GPU
void Ctx::row_norms(int rows, long long len, const double *A, long long lda, double *out) {
    const int chunks = (int)std::max<long long>(1, std::min<long long>((4LL * n_sm + rows - 1) / rows, (len + 2047) / 2048));
    norm_partial.reserve((size_t)rows * chunks);
    row_sq_partial_kernel<<<dim3(chunks, rows), 256, 0, stream>>>(len, chunks, A, lda, norm_partial.p);
    count_launch(stream, "row_sq_partial");
    check_launch("row_sq_partial");
    row_sq_finish_kernel<<<ceil_div(rows, 128), 128, 0, stream>>>(rows, chunks, norm_partial.p, out);
    count_launch(stream, "row_sq_finish");
    check_launch("row_sq_finish");
}

template <class T>
static void upload(cudaStream_t st, DevBuf<T> &d, const T *h, size_t n) {
    d.alloc(n);
    TINCR_CUDA(cudaMemcpyAsync(d.p, h, n * sizeof(T), cudaMemcpyHostToDevice, st));
}

void check_finite(const double *p, size_t n, const char *what) {
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(p[i])) fail(TINCR_NONFINITE, std::string("non-finite value in ") + what);
}

// S C on the device (FP64 GEMM)
void Ctx::upload_mo(int n, const double *C, const double *S) {
    upload(stream, dC, C, (size_t)n * n);
    upload(stream, dS_, S, (size_t)n * n);
    dSC.alloc((size_t)n * n);
    gemm_f64<false, false>(stream, n, n, n, dS_.p, n, 0, dC.p, n, 0, 1, EpiStore{dSC.p, 0, n, 1.0, 0.0});
    sync();
}

void Ctx::set_atoms(int n_atoms_, const int *orbs_per_atom, int n_orb_) {
    if (n_atoms_ <= 0 || n_orb_ <= 0 || !orbs_per_atom) fail(TINCR_BAD_ARG, "empty system");
    std::vector<int> off(n_atoms_ + 1, 0), atom_of(n_orb_);
    for (int a = 0; a < n_atoms_; ++a) {
        if (orbs_per_atom[a] <= 0) fail(TINCR_BAD_ARG, "orbs_per_atom must be positive");
        off[a + 1] = off[a] + orbs_per_atom[a];
    }
    if (off[n_atoms_] != n_orb_) fail(TINCR_BAD_ARG, "sum(orbs_per_atom) != n_orb");
    for (int a = 0; a < n_atoms_; ++a)
        for (int mu = off[a]; mu < off[a + 1]; ++mu) atom_of[mu] = a;
    n_atoms = n_atoms_;
    n_orb = n_orb_;
    h_ao_off = off;
    upload(stream, d_ao_off, off.data(), off.size());
    upload(stream, d_ao_atom, atom_of.data(), atom_of.size());
}

void Ctx::trans_charges(int n_atoms_, const int *opa, int n, const double *C, const double *S, int occ0, int no,
                        int virt0, int nv, double *q_ov, double *q_oo, double *q_vv) {
    if (!C || !S || no <= 0 || nv <= 0 || occ0 < 0 || virt0 < 0 || occ0 + no > n || virt0 + nv > n)
        fail(TINCR_BAD_ARG, "trans_charges: bad orbital ranges");
    check_finite(C, (size_t)n * n, "C");
    check_finite(S, (size_t)n * n, "S");
    set_atoms(n_atoms_, opa, n);
    upload_mo(n, C, S);
    struct Job { double *host; int p0, np, q0, nq; };
    Job jobs[3] = {{q_ov, occ0, no, virt0, nv}, {q_oo, occ0, no, occ0, no}, {q_vv, virt0, nv, virt0, nv}};
    for (auto &j : jobs) {
        if (!j.host) continue;
        size_t cnt = (size_t)n_atoms * j.np * j.nq;
        DevBuf<double> out(cnt);
        dim3 grid(grid_for((long long)j.np * j.nq, 256, n_sm) / std::max(1, std::min(n_atoms, 32)) + 1, n_atoms);
        trans_charges_kernel<<<grid, 256, 0, stream>>>(n, n_atoms, d_ao_off.p, dC.p, dSC.p, j.p0, j.np, j.q0, j.nq, out.p);
        count_launch(stream, "trans_charges");
        check_launch("trans_charges");
        TINCR_CUDA(cudaMemcpyAsync(j.host, out.p, cnt * sizeof(double), cudaMemcpyDeviceToHost, stream));
        sync();
    }
}

void Ctx::tda_setup(int n_atoms_, const int *opa, int n, const double *C, const double *S, const double *orbe,
                    int no, int nv, const double *gamma, const double *gamma_lr, const double *xyz) {
    if (!C || !S || !orbe || !gamma || !xyz) fail(TINCR_BAD_ARG, "tda_setup: null input");
    if (no <= 0 || nv <= 0 || no + nv > n) fail(TINCR_BAD_ARG, "tda_setup: bad n_occ/n_virt");
    check_finite(C, (size_t)n * n, "C");
    check_finite(S, (size_t)n * n, "S");
    check_finite(orbe, n, "orbe");
    check_finite(gamma, (size_t)n_atoms_ * n_atoms_, "gamma");
    if (gamma_lr) check_finite(gamma_lr, (size_t)n_atoms_ * n_atoms_, "gamma_lr");
    set_atoms(n_atoms_, opa, n);
    if ((size_t)n_atoms * sizeof(double) > 48 * 1024)
        fail(TINCR_BAD_ARG, "tda_setup: more than 6144 atoms in one system is not supported");
    n_occ = no;
    n_virt = nv;
    ov = (long long)no * nv;
    lc = gamma_lr != nullptr;
    upload_mo(n, C, S);
    planes_ready = false;
    mx_key = -1;
    h_xyz.assign(xyz, xyz + 3 * (size_t)n_atoms);
    upload(stream, d_xyz, xyz, 3 * (size_t)n_atoms);
    h_gamma.assign(gamma, gamma + (size_t)n_atoms * n_atoms);
    h_orbe.assign(orbe, orbe + n);
    solved_roots = 0;
    h_omega.resize(ov);
    for (int i = 0; i < no; ++i)
        for (int a = 0; a < nv; ++a) h_omega[(size_t)i * nv + a] = orbe[no + a] - orbe[i];   // utils.rs:8-22
    upload(stream, d_omega, h_omega.data(), (size_t)ov);
    upload(stream, d_gamma, gamma, (size_t)n_atoms * n_atoms);
    dLst.alloc((size_t)2 * n * no);
    dLsw.alloc((size_t)2 * n * no);
    dRv.alloc((size_t)2 * n * nv);
    dRsw.alloc((size_t)2 * n * nv);
    pack_blocks_kernel<<<grid_for(2LL * n * (no + nv), 256, n_sm), 256, 0, stream>>>(n, no, nv, dC.p, dSC.p, dLst.p,
                                                                                      dRv.p, dLsw.p, dRsw.p);
    count_launch(stream, "pack_blocks");
    check_launch("pack_blocks");
    if (lc) {
        DevBuf<double> glr;
        upload(stream, glr, gamma_lr, (size_t)n_atoms * n_atoms);
        d_glr_ao.alloc((size_t)n * n);
        expand_ao_kernel<<<grid_for((long long)n * n, 256, n_sm), 256, 0, stream>>>(n, n_atoms, d_ao_atom.p, glr.p, d_glr_ao.p);
        count_launch(stream, "expand_ao");
        check_launch("expand_ao");
        sync();
    } else {
        d_glr_ao.release();
    }
    sync();
    ready = true;
}

// Workspace for a chunk of kc vectors.
int Ctx::product_chunk() const {
    size_t per = (size_t)2 * n_orb * n_virt * 2 + 2 * (size_t)n_orb;      // H, G, d3, d2 (+zao)
    if (lc) per += (size_t)4 * n_orb * n_orb;                              // F
    size_t budget = (size_t)768 << 20;                                      // bytes of workspace
    long long kc = (long long)(budget / (per * sizeof(double)));
    return (int)std::max<long long>(1, std::min<long long>(kc, 64));
}

// Generic AO-direct contraction of the Mulliken two-electron integrals, for k right-hand sides:
//   out_b[p][q] = alpha * ( ac * 2 J[V_b]_pq + ax * 4 K[V_b]_pq ) (+ beta * out_b or + omega o X_b)
// with J[V]_pq = sum_A q^A_pq (gamma y)_A, y_A = sum_rs q^A_rs V_rs (Coulomb, gamma) and
// K[V]_pq = sum_rs (pr|qs)_lr V_rs (exchange, gamma_lr), p in block P, q in Q, r in R, s in S.
// Implemented as  [SC_P; C_P]^T (ax gamma_lr o M + ac D(z)) [SC_Q; C_Q],  M = [C_R; SC_R] V [C_S; SC_S]^T.
void Ctx::ao_contract(int k, int R, int S, const double *V, int P, int Q, double ax, double ac, double *out,
                      double alpha, double beta, const double *Xomega) {
    if (prec == TINCR_PREC_BF16X3) {
        ao_contract_mixed(k, R, S, V, P, Q, ax, ac, out, alpha, beta, Xomega);
        return;
    }
    const int n = n_orb;
    const int nr = bsz(R), ns = bsz(S), np = bsz(P), nq = bsz(Q);
    const bool exch = ax != 0.0 && lc;
    const int kc_max = product_chunk();
    const int wmax = std::max(n_occ, n_virt);
    wsH.reserve((size_t)kc_max * 2 * n * wmax);
    wsG.reserve((size_t)kc_max * 2 * n * wmax);
    wsd3.reserve((size_t)kc_max * n);
    wsd2.reserve((size_t)kc_max * n);
    wsz.reserve((size_t)kc_max * n);
    if (exch) wsF.reserve((size_t)kc_max * 4 * n * n);
    for (int c0 = 0; c0 < k; c0 += kc_max) {
        int kc = std::min(kc_max, k - c0);
        const double *Vc = V + (long long)c0 * nr * ns;
        // 1. H_b = [C_R; SC_R] V_b
        pgemm<false, false>(*this, TINCR_KF_AO_TRANSFORM, 2 * n, ns, nr, stk(R), nr, 0, Vc, ns, (long long)nr * ns, kc,
                            EpiStore{wsH.p, 2LL * n * ns, ns, 1.0, 0.0});
        if (exch) {
            // 2. F_b = ax gamma_lr o (H_b [C_S; SC_S]^T), diagonals captured for the Coulomb term
            pgemm<false, true>(*this, TINCR_KF_AO_EXCHANGE, 2 * n, 2 * n, ns, wsH.p, ns, 2LL * n * ns, stk(S), ns, 0, kc,
                               EpiLcHadamard{wsF.p, d_glr_ao.p, wsd3.p, wsd2.p, n, ax});
        } else if (ac != 0.0) {
            dim3 g(ceil_div(2LL * n * 32, 256), kc);
            diag_dots_kernel<<<g, 256, 0, stream>>>(n, ns, wsH.p, ns, 2LL * n * ns, stk(S), wsd3.p, wsd2.p);
            count_launch(stream, "diag_dots");
            check_launch("diag_dots");
        }
        // 3. Coulomb: z = ac gamma y on the diagonals of F's off-diagonal blocks (or as a row scale)
        if (ac != 0.0) {
            launch_coulomb(stream, kc, n, n_atoms, d_ao_off.p, d_gamma.p, wsd3.p, wsd2.p, exch ? nullptr : wsz.p,
                           exch ? wsF.p : nullptr, nullptr, ac);
        }
        // 4. G_b = F_b [SC_Q; C_Q]
        if (exch) {
            pgemm<false, false>(*this, TINCR_KF_AO_EXCHANGE, 2 * n, nq, 2 * n, wsF.p, 2 * n, 4LL * n * n, swp(Q), nq, 0,
                                kc, EpiStore{wsG.p, 2LL * n * nq, nq, 1.0, 0.0});
        } else if (ac != 0.0) {
            dim3 g(grid_for(2LL * n * nq, 256, n_sm), kc);
            scale_rows_kernel<<<g, 256, 0, stream>>>(n, nq, wsz.p, stk(Q), wsG.p);
            count_launch(stream, "scale_rows");
            check_launch("scale_rows");
        } else {
            TINCR_CUDA(cudaMemsetAsync(wsG.p, 0, (size_t)kc * 2 * n * nq * sizeof(double), stream));
        }
        // 5. out_b = [SC_P; C_P]^T G_b  (+ omega o X_b, or alpha/beta)
        double *outc = out + (long long)c0 * np * nq;
        if (Xomega) {
            pgemm<true, false>(*this, TINCR_KF_AO_TRANSFORM, np, nq, 2 * n, swp(P), np, 0, wsG.p, nq, 2LL * n * nq, kc,
                               EpiOmega{outc, d_omega.p, Xomega + (long long)c0 * np * nq, (long long)np * nq, nq});
        } else {
            pgemm<true, false>(*this, TINCR_KF_AO_TRANSFORM, np, nq, 2 * n, swp(P), np, 0, wsG.p, nq, 2LL * n * nq, kc,
                               EpiStore{outc, (long long)np * nq, nq, alpha, beta});
        }
    }
}

// AX (k x ov) for X (k x ov), both device, vector-major:
//   AX = omega o X + 2 J[X] - K[X]   (solvers/mod.rs:307-361)
void Ctx::products_dev(int k, const double *X, double *AX, double *) {
    ao_contract(k, BLK_OCC, BLK_VIRT, X, BLK_OCC, BLK_VIRT, lc ? -0.25 : 0.0, 1.0, AX, 1.0, 0.0, X);
}

// q_ov X per atom only (transition charges of the vectors): steps 1 and the diagonal dots.
void Ctx::qtrans_dev(int k, const double *X, double *y_out) {
    if (solve_prec == TINCR_PREC_BF16X3) {   // mixed form: the half transform on the tensor cores
        qtrans_mixed(k, X, y_out);
        return;
    }
    const int n = n_orb, o = n_occ, v = n_virt;
    const int kc_max = product_chunk();
    wsH.reserve((size_t)kc_max * 2 * n * v);
    wsd3.reserve((size_t)kc_max * n);
    wsd2.reserve((size_t)kc_max * n);
    for (int c0 = 0; c0 < k; c0 += kc_max) {
        int kc = std::min(kc_max, k - c0);
        gemm_f64<false, false>(stream, 2 * n, v, o, dLst.p, o, 0, X + (long long)c0 * ov, v, ov, kc,
                               EpiStore{wsH.p, 2LL * n * v, v, 1.0, 0.0});
        dim3 g(ceil_div(2LL * n * 32, 256), kc);
        diag_dots_kernel<<<g, 256, 0, stream>>>(n, v, wsH.p, v, 2LL * n * v, dRv.p, wsd3.p, wsd2.p);
        count_launch(stream, "diag_dots");
        check_launch("diag_dots");
        launch_coulomb(stream, kc, n, n_atoms, d_ao_off.p, d_gamma.p, wsd3.p, wsd2.p, nullptr, nullptr,
                       y_out + (long long)c0 * n_atoms, 1.0);
    }
}

void Ctx::products(int k, const double *X, double *AX, int precision) {
    if (!ready) fail(TINCR_BAD_ARG, "tincr_tda_setup must be called first");
    if (k <= 0 || !X || !AX) fail(TINCR_BAD_ARG, "products: bad arguments");
    if (precision != TINCR_PREC_FP64 && precision != TINCR_PREC_BF16X3) fail(TINCR_BAD_ARG, "products: unknown precision");
    prec = precision;
    check_finite(X, (size_t)ov * k, "X");
    g_launches = 0;
    DevBuf<double> dXin((size_t)ov * k), dX((size_t)ov * k), dAX((size_t)ov * k);
    TINCR_CUDA(cudaMemcpyAsync(dXin.p, X, (size_t)ov * k * sizeof(double), cudaMemcpyHostToDevice, stream));
    TINCR_CUDA(cudaEventRecord(ev0, stream));
    launch_transpose((int)ov, k, dXin.p, dX.p);          // [ov x k] -> [k x ov]
    products_dev(k, dX.p, dAX.p, nullptr);
    launch_transpose(k, (int)ov, dAX.p, dXin.p);          // back to [ov x k]
    TINCR_CUDA(cudaEventRecord(ev1, stream));
    TINCR_CUDA(cudaMemcpyAsync(AX, dXin.p, (size_t)ov * k * sizeof(double), cudaMemcpyDeviceToHost, stream));
    sync();
    float ms = 0.f;
    TINCR_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    last_ms = ms;
    last_launches = g_launches;
    prof_resolve();
}

void Ctx::set_states(int n_roots, const double *energies, const double *coefficients) {
    if (!ready) fail(TINCR_BAD_ARG, "tincr_tda_setup must be called first");
    if (n_roots <= 0 || n_roots > ov || !energies || !coefficients) fail(TINCR_BAD_ARG, "set_states: bad arguments");
    check_finite(energies, n_roots, "energies");
    check_finite(coefficients, (size_t)ov * n_roots, "coefficients");
    DevBuf<double> tmp((size_t)ov * n_roots);
    dR.reserve((size_t)n_roots * ov);
    TINCR_CUDA(cudaMemcpyAsync(tmp.p, coefficients, (size_t)ov * n_roots * sizeof(double), cudaMemcpyHostToDevice, stream));
    launch_transpose((int)ov, n_roots, tmp.p, dR.p);     // [ov x n_roots] -> [n_roots x ov]
    sync();
    h_energies.assign(energies, energies + n_roots);
    solved_roots = n_roots;
    solve_prec = TINCR_PREC_FP64;
}

// ----------------------------------------------------------------------------------------------
// Davidson (src/excited_states/solvers/davidson.rs:53-185)
// ----------------------------------------------------------------------------------------------

// Block Davidson on the current operator (precision `prec`).  Initial subspace: unit vectors on the
// n_roots smallest omega (tincr's guess), or the rows of dR (Ritz vectors of an earlier run), in which
// case the run may stop at its first iteration.  Leaves Ritz values in u and Ritz vectors in dR.
int Ctx::davidson(int n_roots, int max_iter, double tol, bool from_ritz, std::vector<double> &u, int *it_out) {
    const int max_space = 15 * n_roots;                        // davidson.rs:74
    const int mmax = std::max(max_space, n_roots);
    dV.reserve((size_t)mmax * ov);
    dAV.reserve((size_t)mmax * ov);
    dR.reserve((size_t)n_roots * ov);
    dRk.reserve((size_t)n_roots * ov);
    dT.reserve((size_t)n_roots * ov);
    DevBuf<double> dYt((size_t)n_roots * mmax), du(n_roots), dnorm(n_roots), dw(n_roots),
        dc((size_t)mmax * n_roots + 64);
    DevBuf<int> didx(n_roots);
    dAp.reserve((size_t)mmax * mmax);
    eig_err.reserve(1);
    // mixed form: subspace products as FP64-accurate digit GEMMs (digits.cu)
    const bool dg = prec == TINCR_PREC_BF16X3 && use_digits && n_roots <= 32;
    if (dg) dg_reserve(mmax);
    TINCR_CUDA(cudaMemsetAsync(eig_err.p, 0, sizeof(int), stream));
    u.assign(n_roots, 0.0);
    if (from_ritz) {
        TINCR_CUDA(cudaMemcpyAsync(dV.p, dR.p, (size_t)n_roots * ov * sizeof(double), cudaMemcpyDeviceToDevice, stream));
        // the Ritz vectors of an orthonormal basis are unit vectors; anything else is a broken run
        row_norms(n_roots, ov, dV.p, ov, dnorm.p);
        std::vector<double> nr(n_roots);
        TINCR_CUDA(cudaMemcpyAsync(nr.data(), dnorm.p, n_roots * sizeof(double), cudaMemcpyDeviceToHost, stream));
        sync();
        for (int r = 0; r < n_roots; ++r)
            if (!(std::fabs(nr[r] - 1.0) < 1e-6))
                fail(TINCR_NONFINITE, "Ritz vector " + std::to_string(r) + " has norm " + std::to_string(nr[r]));
    } else {
        // unit vectors on the n_roots smallest omega (solvers/utils.rs:17-26, stable ties)
        std::vector<int> order(ov);
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return h_omega[a] < h_omega[b]; });
        std::vector<int> pos(order.begin(), order.begin() + n_roots);
        DevBuf<int> dpos(n_roots);
        TINCR_CUDA(cudaMemcpyAsync(dpos.p, pos.data(), n_roots * sizeof(int), cudaMemcpyHostToDevice, stream));
        TINCR_CUDA(cudaMemsetAsync(dV.p, 0, (size_t)n_roots * ov * sizeof(double), stream));
        unit_vectors_kernel<<<1, 256, 0, stream>>>(n_roots, ov, dpos.p, dV.p);
        count_launch(stream, "unit_vectors");
        check_launch("unit_vectors");
        sync();
    }
    if (dg) dg_add_rows(false, 0, n_roots, dV.p);
    int m = n_roots;            // columns of the guess
    int m_done = 0;             // columns with products (product cache)
    int dim_sub = n_roots;      // tincr's dim_sub bookkeeping
    const int dim_sub_origin = n_roots;
    std::vector<double> aproj;  // host copy of the projected matrix (host eigensolver only)
    std::vector<double> w(mmax);
    std::vector<double> errs(n_roots);
    int status = TINCR_NOT_CONVERGED;
    int it_done = 0;
    for (int it = 0; it < max_iter; ++it) {
        it_done = it + 1;
        // 1. products for the new columns (cache reset after a collapse: m_done = 0)
        if (m > m_done) {
            products_dev(m - m_done, dV.p + (long long)m_done * ov, dAV.p + (long long)m_done * ov, nullptr);
            last_products += m - m_done;
            if (dg) dg_add_rows(true, m_done, m - m_done, dAV.p + (long long)m_done * ov);
        }
        // 1.1 projected matrix, new columns only: P[:, mold:m] = V[0:m] AV[mold:m]^T, kept on the device
        //     (leading dimension mmax; the old columns stay valid until a collapse)
        int knew = m - m_done;
        const int mold = m_done;
        if (knew > 0 && dg) {
            dg_project(m, mold, knew, dAp.p, mmax);
        } else if (knew > 0) {
            TINCR_CUDA(cudaMemset2DAsync(dAp.p + mold, (size_t)mmax * sizeof(double), 0, (size_t)knew * sizeof(double),
                                         m, stream));
            if (knew <= 32) {
                int slot = prof_begin(TINCR_KF_SUBSPACE);
                skinny_dots(stream, n_sm, m, knew, ov, dV.p, ov, dAV.p + (long long)mold * ov, ov, dAp.p + mold, mmax);
                prof_end(slot, 2.0 * m * (double)knew * ov, 8.0 * (double)(m + knew) * ov);
            } else {
                int sk = pick_splitk(m, knew, (int)ov, 1, n_sm);
                pgemm<false, true>(*this, TINCR_KF_SUBSPACE, m, knew, (int)ov, dV.p, (int)ov, 0,
                                   dAV.p + (long long)mold * ov, (int)ov, 0, 1, EpiAtomicAdd{dAp.p + mold, 0, mmax, 1.0}, sk);
            }
        }
        m_done = m;
        // 2. the n_roots lowest eigenpairs of the subspace matrix (upper triangle): on the host
        //    (eigen_host.cpp), or on one thread-block cluster (eig_cluster.cu) when selected and it fits
        bool on_device = eig_cluster_on && eig_cluster(*this, m, n_roots, dAp.p, mmax, du.p, dYt.p, eig_err.p);
        if (!on_device) {
            aproj.resize((size_t)m * m);
            TINCR_CUDA(cudaMemcpy2DAsync(aproj.data(), (size_t)m * sizeof(double), dAp.p, (size_t)mmax * sizeof(double),
                                         (size_t)m * sizeof(double), m, cudaMemcpyDeviceToHost, stream));
            sync();
            const auto th0 = std::chrono::steady_clock::now();
            std::vector<double> yt((size_t)n_roots * m);
            if (!eigh_lowest_upper(m, aproj.data(), n_roots, w.data(), yt.data()))
                fail(TINCR_NONFINITE, "subspace eigensolver failed");
            if (profiling) {
                KernelStats &hs = stats[TINCR_KF_HOST];
                hs.ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - th0).count();
                hs.launches += 1;
                hs.flops += 4.0 / 3.0 * (double)m * m * m;
            }
            for (int r = 0; r < n_roots; ++r) u[r] = w[r];
            for (int r = 0; r < n_roots; ++r)
                if (!std::isfinite(u[r])) fail(TINCR_NONFINITE, "non-finite Ritz value");
            TINCR_CUDA(cudaMemcpyAsync(dYt.p, yt.data(), yt.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
            TINCR_CUDA(cudaMemcpyAsync(du.p, u.data(), n_roots * sizeof(double), cudaMemcpyHostToDevice, stream));
        }
        // 3.1 Ritz vectors R = Y^T V ; 3.2 residuals Rk = Y^T AV - u o R
        if (dg) {
            dg_ritz(n_roots, m, dYt.p, dR.p, dRk.p, du.p);
        } else if (n_roots <= 32) {
            int slot = prof_begin(TINCR_KF_SUBSPACE);
            skinny_comb(stream, n_roots, m, ov, dYt.p, m, 1, dV.p, ov, CombStore{dR.p, ov, 1.0, 0.0});
            skinny_comb(stream, n_roots, m, ov, dYt.p, m, 1, dAV.p, ov, CombResidual{dRk.p, dR.p, du.p, ov});
            prof_end(slot, 4.0 * n_roots * (double)m * ov, 8.0 * (2.0 * m + 3.0 * n_roots) * ov);
        } else {
            pgemm<false, false>(*this, TINCR_KF_SUBSPACE, n_roots, (int)ov, m, dYt.p, m, 0, dV.p, (int)ov, 0, 1,
                                EpiStore{dR.p, 0, (int)ov, 1.0, 0.0});
            pgemm<false, false>(*this, TINCR_KF_SUBSPACE, n_roots, (int)ov, m, dYt.p, m, 0, dAV.p, (int)ov, 0, 1,
                                EpiResidual{dRk.p, dR.p, du.p, ov});
        }
        row_norms(n_roots, ov, dRk.p, ov, dnorm.p);
        TINCR_CUDA(cudaMemcpyAsync(errs.data(), dnorm.p, n_roots * sizeof(double), cudaMemcpyDeviceToHost, stream));
        int eig_bad = 0, dg_err[2] = {0, 0};
        if (on_device) {
            TINCR_CUDA(cudaMemcpyAsync(u.data(), du.p, n_roots * sizeof(double), cudaMemcpyDeviceToHost, stream));
            TINCR_CUDA(cudaMemcpyAsync(&eig_bad, eig_err.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
        }
        if (dg) {
            TINCR_CUDA(cudaMemcpyAsync(&dg_err[0], d_tc_err.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
            TINCR_CUDA(cudaMemcpyAsync(&dg_err[1], dg_bad.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
        }
        sync();
        if (eig_bad) fail(TINCR_NONFINITE, "subspace eigensolver: non-finite projected matrix or Ritz pairs");
        if (dg_err[0] || dg_err[1]) dg_check();
        int roots_cvd = 0;
        for (int r = 0; r < n_roots; ++r) {
            if (!std::isfinite(errs[r])) fail(TINCR_NONFINITE, "non-finite residual");
            if (errs[r] < tol) ++roots_cvd;
        }
        int roots_lft = n_roots - roots_cvd;
        last_max_residual = *std::max_element(errs.begin(), errs.end());
        last_history.push_back({it, m, last_max_residual, roots_lft, prec});
        if (roots_lft == 0 && (it > 0 || from_ritz)) {         // davidson.rs:121
            status = TINCR_OK;
            break;
        }
        if (it == max_iter - 1) break;
        if (dim_sub + roots_lft <= max_space) {                // davidson.rs:146
            std::vector<int> idx;
            std::vector<double> wsel;
            for (int r = 0; r < n_roots; ++r)
                if (errs[r] > tol) { idx.push_back(r); wsel.push_back(u[r]); }
            int kadd = (int)idx.size();
            dim_sub += roots_lft;
            if (kadd > 0) {
                TINCR_CUDA(cudaMemcpyAsync(didx.p, idx.data(), kadd * sizeof(int), cudaMemcpyHostToDevice, stream));
                TINCR_CUDA(cudaMemcpyAsync(dw.p, wsel.data(), kadd * sizeof(double), cudaMemcpyHostToDevice, stream));
                dim3 g(grid_for(ov, 256, n_sm) / std::max(1, kadd) + 1, kadd);
                precondition_kernel<<<g, 256, 0, stream>>>(ov, kadd, didx.p, dw.p, dRk.p, d_omega.p, dT.p);
                count_launch(stream, "precondition");
                check_launch("precondition");
                // orthogonalise against the current basis in one block: T -= (T V^T) V
                if (dg) {
                    dg_ortho(kadd, m, dT.p, dc.p);
                } else if (kadd <= 32) {
                    TINCR_CUDA(cudaMemsetAsync(dc.p, 0, (size_t)kadd * m * sizeof(double), stream));
                    // c = V T^T  [m x kadd];  T -= c^T V
                    int slot = prof_begin(TINCR_KF_SUBSPACE);
                    skinny_dots(stream, n_sm, m, kadd, ov, dV.p, ov, dT.p, ov, dc.p, kadd);
                    skinny_comb(stream, kadd, m, ov, dc.p, 1, kadd, dV.p, ov, CombStore{dT.p, ov, -1.0, 1.0});
                    prof_end(slot, 4.0 * kadd * (double)m * ov, 8.0 * (2.0 * m + 3.0 * kadd) * ov);
                } else {
                    TINCR_CUDA(cudaMemsetAsync(dc.p, 0, (size_t)kadd * m * sizeof(double), stream));
                    int sk = pick_splitk(kadd, m, (int)ov, 1, n_sm);
                    pgemm<false, true>(*this, TINCR_KF_SUBSPACE, kadd, m, (int)ov, dT.p, (int)ov, 0, dV.p, (int)ov, 0, 1,
                                       EpiAtomicAdd{dc.p, 0, m, 1.0}, sk);
                    pgemm<false, false>(*this, TINCR_KF_SUBSPACE, kadd, (int)ov, m, dc.p, m, 0, dV.p, (int)ov, 0, 1,
                                        EpiStore{dT.p, 0, (int)ov, -1.0, 1.0});
                }
                // then sequentially against the vectors accepted in this step (davidson.rs:162-168)
                if (kadd <= 32 && coop_grid > 0) {
                    int slot = prof_begin(TINCR_KF_SUBSPACE);
                    gs_part.reserve((size_t)2 * coop_grid * GS_SLOTS);
                    gs_state.reserve(2);
                    int hstate[2] = {m, 0};
                    TINCR_CUDA(cudaMemcpyAsync(gs_state.p, hstate, 2 * sizeof(int), cudaMemcpyHostToDevice, stream));
                    int a_kadd = kadd, a_m0 = m, a_mmax = mmax;
                    long long a_ov = ov;
                    double *a_V = dV.p, *a_T = dT.p, *a_part = gs_part.p;
                    int *a_state = gs_state.p;
                    void *args[] = {&a_kadd, &a_ov, &a_m0, &a_mmax, &a_V, &a_T, &a_part, &a_state};
                    TINCR_CUDA(cudaLaunchCooperativeKernel((const void *)seq_gs_kernel, dim3(coop_grid), dim3(256), args,
                                                           0, stream));
                    count_launch(stream, "seq_gs");
                    prof_end(slot, 4.0 * kadd * (double)kadd * ov / 2.0, 8.0 * (kadd * (kadd + 3.0) / 2.0) * ov);
                    TINCR_CUDA(cudaMemcpyAsync(hstate, gs_state.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, stream));
                    sync();
                    if (hstate[1]) fail(TINCR_NONFINITE, "non-finite correction vector");
                    if (dg) dg_add_rows(false, m, hstate[0] - m, dV.p + (long long)m * ov);
                    m = hstate[0];
                } else {
                    const int m0 = m;
                    for (int j = 0; j < kadd; ++j) {
                        double *t = dT.p + (long long)j * ov;
                        int acc = m - m0;
                        if (acc > 0) {
                            TINCR_CUDA(cudaMemsetAsync(dc.p, 0, acc * sizeof(double), stream));
                            // c = Q t  [acc x 1] over the vectors accepted in this step;  t -= c^T Q
                            int slot = prof_begin(TINCR_KF_SUBSPACE);
                            skinny_dots(stream, n_sm, acc, 1, ov, dV.p + (long long)m0 * ov, ov, t, ov, dc.p, 1);
                            skinny_comb(stream, 1, acc, ov, dc.p, acc, 1, dV.p + (long long)m0 * ov, ov,
                                        CombStore{t, ov, -1.0, 1.0});
                            prof_end(slot, 4.0 * acc * (double)ov, 8.0 * (acc + 2.0) * ov);
                        }
                        row_norms(1, ov, t, ov, dnorm.p);
                        double nrm = 0.0;
                        TINCR_CUDA(cudaMemcpyAsync(&nrm, dnorm.p, sizeof(double), cudaMemcpyDeviceToHost, stream));
                        sync();
                        if (!std::isfinite(nrm)) fail(TINCR_NONFINITE, "non-finite correction vector");
                        if (nrm > 1.0e-8 && m < mmax) {
                            scale_copy_kernel<<<grid_for(ov, 256, n_sm), 256, 0, stream>>>(ov, t, 1.0 / nrm,
                                                                                           dV.p + (long long)m * ov);
                            count_launch(stream, "scale_copy");
                            check_launch("scale_copy");
                            ++m;
                        }
                    }
                    if (dg) dg_add_rows(false, m0, m - m0, dV.p + (long long)m0 * ov);
                }
            }
        } else {                                               // collapse, davidson.rs:172-176
            dim_sub = dim_sub_origin;
            ++last_collapses;
            TINCR_CUDA(cudaMemcpyAsync(dV.p, dR.p, (size_t)dim_sub * ov * sizeof(double), cudaMemcpyDeviceToDevice, stream));
            m = dim_sub;
            if (dg) dg_add_rows(false, 0, dim_sub, dV.p);
            m_done = 0;
            aproj.clear();
        }
    }
    *it_out = it_done;
    return status;
}

int Ctx::solve(int n_roots, int max_iter, double tol, int precision, double *energies, double *coefficients,
               double *osc, double *tr_dip, double *q_trans, int *iterations) {
    if (!ready) fail(TINCR_BAD_ARG, "tincr_tda_setup must be called first");
    if (n_roots <= 0 || n_roots > ov || max_iter <= 0 || !(tol > 0.0)) fail(TINCR_BAD_ARG, "solve: bad arguments");
    if (!energies || !coefficients) fail(TINCR_BAD_ARG, "solve: null outputs");
    if (precision != TINCR_PREC_FP64 && precision != TINCR_PREC_BF16X3) fail(TINCR_BAD_ARG, "solve: unknown precision");
    g_launches = 0;
    last_products = 0;
    last_collapses = 0;
    last_history.clear();
    TINCR_CUDA(cudaEventRecord(ev0, stream));
    std::vector<double> u;
    int it_done = 0;
    prec = precision;
    solve_prec = precision;
    // the mixed operator resolves residuals down to MIXED_TOL_FLOOR; below that the mixed phase
    // stops there and FP64 iterations take over
    const bool polish = precision == TINCR_PREC_BF16X3 && tol < MIXED_TOL_FLOOR;
    int status = davidson(n_roots, max_iter, polish ? MIXED_TOL_FLOOR : tol, false, u, &it_done);
    if (polish) {
        // FP64 polish for tolerances below the mixed operator's resolution: Davidson on the FP64
        // operator from the mixed Ritz vectors, which may stop at its first Rayleigh-Ritz step.
        prec = TINCR_PREC_FP64;
        int it2 = 0;
        status = davidson(n_roots, std::max(1, max_iter - it_done), tol, true, u, &it2);
        it_done += it2;
    }
    // results: energies, coefficients [ov x n_roots], transition charges, dipoles, oscillator strengths
    TINCR_CUDA(cudaEventRecord(ev1, stream));
    for (int r = 0; r < n_roots; ++r) energies[r] = u[r];
    h_energies.assign(u.begin(), u.end());
    solved_roots = n_roots;
    DevBuf<double> dCo((size_t)ov * n_roots);
    launch_transpose(n_roots, (int)ov, dR.p, dCo.p);
    TINCR_CUDA(cudaMemcpyAsync(coefficients, dCo.p, (size_t)ov * n_roots * sizeof(double), cudaMemcpyDeviceToHost, stream));
    std::vector<double> qt((size_t)n_roots * n_atoms);
    {
        DevBuf<double> dy((size_t)n_roots * n_atoms);
        qtrans_dev(n_roots, dR.p, dy.p);
        TINCR_CUDA(cudaMemcpyAsync(qt.data(), dy.p, qt.size() * sizeof(double), cudaMemcpyDeviceToHost, stream));
    }
    sync();
    // tda/mod.rs:91-97, moments.rs:7-24
    for (int r = 0; r < n_roots; ++r) {
        double mu[3] = {0, 0, 0};
        for (int A = 0; A < n_atoms; ++A)
            for (int c = 0; c < 3; ++c) mu[c] += h_xyz[(size_t)A * 3 + c] * qt[(size_t)r * n_atoms + A];
        if (tr_dip)
            for (int c = 0; c < 3; ++c) tr_dip[(size_t)c * n_roots + r] = mu[c];
        if (osc) osc[r] = 2.0 / 3.0 * u[r] * (mu[0] * mu[0] + mu[1] * mu[1] + mu[2] * mu[2]);
    }
    if (q_trans)
        for (int A = 0; A < n_atoms; ++A)
            for (int r = 0; r < n_roots; ++r) q_trans[(size_t)A * n_roots + r] = qt[(size_t)r * n_atoms + A];
    if (iterations) *iterations = it_done;
    float ms = 0.f;
    TINCR_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    last_ms = ms;
    last_launches = g_launches;
    prof_resolve();
    return status;
}

}  // namespace tincr
