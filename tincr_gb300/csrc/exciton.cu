// FMO exciton Hamiltonian in the diabatic LE / CT basis and its lowest states (tincr_exciton_states).
//
// tincr builds the matrix element by element on rayon threads (SuperSystem::
// create_exciton_hamiltonian_new, src/fmo/lcmo/basis.rs:449-503; couplings in
// src/fmo/lcmo/integrals.rs), rebuilding the Mulliken transition charges between the orbitals of
// two monomers for every element.  Here the matrix is assembled on the GPU in a few grouped passes:
//   * Coulomb: W = gamma Q over all atoms, then 2 q_s . W_t for every element (block-sparse Q: each
//     state's charges live on one or two monomers);
//   * exchange: the charges are never stored.  With Mulliken charges
//     q^A_pq = 1/2 sum_{mu in A} (C_mu p (S C)_mu q + (S C)_mu p C_mu q) over the AOs of the one or
//     two monomers involved, sum_i q^A_ij b_ia is a sum over mu in A of two outer products of per-AO
//     rows, and exchange = sum_{A, B} gamma_lr[A, B] sum_{a, j} U^A_aj W^B_aj.  The state-dependent
//     rows come from batched small GEMMs; V = gamma_lr W is formed once per group of elements that
//     share their second state and monomers, in one CTA per tile of (a, j), which then serves the
//     group's elements (see "exchange integrals" below);
//   * one-electron LE-CT terms through the LCMO Fock matrix (src/fmo/lcmo/hamiltonian.rs:12-152),
//     whose needed blocks F'_{xy} = (x^T F x)_{xy}, x = 3/2 I - 1/2 S_total, come from block-sparse
//     products over the real pairs around x and y (batched small GEMMs);
//   * the lowest roots by tincr's Davidson on the dense matrix (davidson.rs:53-185 with the engine
//     of solvers/mod.rs:36-51: H X, preconditioner r / (w - diag H)), products on the device, the
//     small subspace eigenproblem on the host (eigen_host.cpp).
// Precision: TINCR_PREC_FP64 runs every contraction in FP64; TINCR_PREC_BF16X3 runs the exchange
// jobs and the LCMO GEMMs in FP32 on the CUDA cores (GB300's FP64 rate is 1/64 of FP32); Coulomb,
// the matrix itself and the Davidson stay FP64 in both.
#include <algorithm>
#include <cmath>
#include <map>
#include <unordered_map>
#include <vector>

#include "tda.cuh"

namespace tincr {

namespace {

// ----------------------------------------------------------------------------------------------
// batched small GEMMs: C[m, n] += alpha sum_k A(m, k) d(k) B(k, n), strided addressing; B == null:
// C[m, n] += alpha A(m, n) (A addressed with sam, sak as the m and n strides)
// ----------------------------------------------------------------------------------------------

struct GemmJob {
    const double *A, *B, *d;
    double *C;
    long long sam, sak, sbk, sbn, ldc;
    int M, N, K;
    double alpha;
};

constexpr int XG_T = 256, XG_KC = 16;   // 256 threads; K in chunks of 16

// TILE x TILE output tile, (TILE / 16)^2 outputs per thread: 64 for FP32 (4 x 4 register blocks),
// 32 for FP64 (more CTAs for the narrow FP64 pipe)
template <class T, int TILE>
__global__ void __launch_bounds__(XG_T) ex_gemm_kernel(const GemmJob *__restrict__ jobs, const int4 *__restrict__ tiles) {
    constexpr int R = TILE / 16, PER = TILE * XG_KC / XG_T;
    __shared__ T As[XG_KC][TILE + 4], Bs[XG_KC][TILE + 4];   // [k][m], [k][n]
    const int4 tl = tiles[blockIdx.x];
    const GemmJob J = jobs[tl.x];
    const int m0 = tl.y * TILE, n0 = tl.z * TILE;
    const int tr = threadIdx.x >> 4, tc = threadIdx.x & 15;   // rows m0 + R tr + i, columns n0 + R tc + j
    if (!J.B) {   // elementwise add
        for (int e = threadIdx.x; e < TILE * TILE; e += XG_T) {
            const int m = m0 + e / TILE, n = n0 + e % TILE;
            if (m < J.M && n < J.N) atomicAdd(J.C + m * J.ldc + n, J.alpha * J.A[m * J.sam + n * J.sak]);
        }
        return;
    }
    T acc[R][R];
#pragma unroll
    for (int i = 0; i < R; ++i)
#pragma unroll
        for (int j = 0; j < R; ++j) acc[i][j] = T(0);
    for (int k0 = 0; k0 < J.K; k0 += XG_KC) {
        // A chunk [TILE m x 16 k] and B chunk [16 k x TILE n], PER elements of each per thread
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int e = threadIdx.x + q * XG_T;
            const int mm = e >> 4, kk = e & 15;   // A: consecutive threads along k
            const int m = m0 + mm, k = k0 + kk;
            T v = T(0);
            if (m < J.M && k < J.K) {
                double x = J.A[m * J.sam + k * J.sak];
                if (J.d) x *= J.d[k];
                v = (T)x;
            }
            As[kk][mm] = v;
            const int kb = e / TILE, nn = e % TILE;   // B: consecutive threads along n
            const int k2 = k0 + kb, n = n0 + nn;
            Bs[kb][nn] = (k2 < J.K && n < J.N) ? (T)J.B[k2 * J.sbk + n * J.sbn] : T(0);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < XG_KC; ++kk) {
            T a[R], b[R];
#pragma unroll
            for (int i = 0; i < R; ++i) a[i] = As[kk][R * tr + i];
#pragma unroll
            for (int j = 0; j < R; ++j) b[j] = Bs[kk][R * tc + j];
#pragma unroll
            for (int i = 0; i < R; ++i)
#pragma unroll
                for (int j = 0; j < R; ++j) acc[i][j] += a[i] * b[j];
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < R; ++i)
#pragma unroll
        for (int j = 0; j < R; ++j) {
            const int m = m0 + R * tr + i, n = n0 + R * tc + j;
            if (m < J.M && n < J.N) atomicAdd(J.C + m * J.ldc + n, J.alpha * (double)acc[i][j]);
        }
}

struct GemmBatch {
    std::vector<GemmJob> jobs;
    std::vector<int4> tiles;
    void gemm(int M, int N, int K, const double *A, long long sam, long long sak, const double *B, long long sbk,
              long long sbn, double *C, long long ldc, double alpha, const double *d = nullptr) {
        if (M <= 0 || N <= 0 || K <= 0) return;
        jobs.push_back(GemmJob{A, B, d, C, sam, sak, sbk, sbn, ldc, M, N, K, alpha});
    }
    // C[m, n] += alpha A(m, n)
    void add(int M, int N, const double *A, long long sam, long long san, double *C, long long ldc, double alpha) {
        if (M <= 0 || N <= 0) return;
        jobs.push_back(GemmJob{A, nullptr, nullptr, C, sam, san, 0, 0, ldc, M, N, 1, alpha});
    }
    void run(Ctx &c, bool fp32, DevBuf<GemmJob> &dj, DevBuf<int4> &dt, int family) {
        if (jobs.empty()) return;
        const int tile = fp32 ? 64 : 32;
        tiles.clear();
        for (int j = 0; j < (int)jobs.size(); ++j)
            for (int tm = 0; tm < ceil_div(jobs[j].M, tile); ++tm)
                for (int tn = 0; tn < ceil_div(jobs[j].N, tile); ++tn) tiles.push_back(make_int4(j, tm, tn, 0));
        dj.reserve(jobs.size());
        dt.reserve(tiles.size());
        TINCR_CUDA(cudaMemcpyAsync(dj.p, jobs.data(), jobs.size() * sizeof(GemmJob), cudaMemcpyHostToDevice, c.stream));
        TINCR_CUDA(cudaMemcpyAsync(dt.p, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice, c.stream));
        double flops = 0.0;
        for (const GemmJob &j : jobs) flops += j.B ? 2.0 * j.M * j.N * j.K : (double)j.M * j.N;
        const int slot = c.prof_begin(family);
        for (size_t t0 = 0; t0 < tiles.size(); t0 += 1u << 20) {   // grid limit
            const unsigned nb = (unsigned)std::min<size_t>(tiles.size() - t0, 1u << 20);
            if (fp32)
                ex_gemm_kernel<float, 64><<<nb, XG_T, 0, c.stream>>>(dj.p, dt.p + t0);
            else
                ex_gemm_kernel<double, 32><<<nb, XG_T, 0, c.stream>>>(dj.p, dt.p + t0);
            count_launch(c.stream, "ex_gemm");
        }
        check_launch("ex_gemm");
        c.prof_end(slot, flops, 0.0);
        // the host vectors must outlive the copies: wait before they are reused or freed
        c.sync();
        jobs.clear();
        tiles.clear();
    }
};

// ----------------------------------------------------------------------------------------------
// states and Coulomb couplings
// ----------------------------------------------------------------------------------------------

// A diabatic state: LE on monomer m (hole = electron = m) or CT with hole h and electron l; its
// transition charges on the atoms [a0, a0 + n0) and, for CT, [a1, a1 + n1) (global atom indices).
struct ExState {
    int kind;            // 0 LE, 1 CT
    int hole, elec;      // monomers
    int a0, n0, a1, n1;  // atom ranges of the charges
    long long q_off;     // charges in dq
    double energy;
};

// W[t * n_atoms + A] = sum_{B in atoms(t)} gamma[A, B] q_t[B]; one CTA per state
__global__ void ex_coul_w_kernel(int n_atoms, const ExState *__restrict__ st, const double *__restrict__ q,
                                 const double *__restrict__ gamma, double *W) {
    const ExState s = st[blockIdx.x];
    for (int A = threadIdx.x; A < n_atoms; A += blockDim.x) {
        double acc = 0.0;
        const double *g = gamma + (long long)A * n_atoms;
        for (int b = 0; b < s.n0; ++b) acc += g[s.a0 + b] * q[s.q_off + b];
        for (int b = 0; b < s.n1; ++b) acc += g[s.a1 + b] * q[s.q_off + s.n0 + b];
        W[(long long)blockIdx.x * n_atoms + A] = acc;
    }
}

// H[s, t] (t > s) = 2 q_s . W_t, except between LE states of one monomer and CT states of one
// directed pair (zero, integrals.rs:21-24, :67-70); H[s, s] = the state's energy
__global__ void ex_coul_h_kernel(int n_states, int n_atoms, const ExState *__restrict__ st,
                                 const double *__restrict__ q, const double *__restrict__ W, double *H) {
    const int s = blockIdx.x;
    const ExState a = st[s];
    for (int t = s + threadIdx.x; t < n_states; t += blockDim.x) {
        double v = 0.0;
        if (t == s) {
            v = a.energy;
        } else {
            const ExState b = st[t];
            const bool same = a.kind == b.kind && a.hole == b.hole && a.elec == b.elec;
            if (!same) {
                const double *w = W + (long long)t * n_atoms;
                double acc = 0.0;
                for (int x = 0; x < a.n0; ++x) acc += q[a.q_off + x] * w[a.a0 + x];
                for (int x = 0; x < a.n1; ++x) acc += q[a.q_off + a.n0 + x] * w[a.a1 + x];
                v = 2.0 * acc;
            }
        }
        H[(long long)s * n_states + t] = v;
    }
}

// H[t, s] = H[s, t] for t > s (tincr fills the lower triangle from the upper one, basis.rs:495)
__global__ void ex_symmetrize_kernel(int n, double *H) {
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= (long long)n * n) return;
    const int r = (int)(idx / n), c = (int)(idx % n);
    if (r > c) H[idx] = H[(long long)c * n + r];
}

// ----------------------------------------------------------------------------------------------
// exchange integrals
// ----------------------------------------------------------------------------------------------
//
// An element (s, t) pairs occupied-side charges q^A_ij between columns P = [p0, p0 + np) of monomer
// x1's C and Q = [q0, q0 + nq) of y1's C (atoms A of {x1, y1}) with virtual-side charges q^B_ab
// between columns P' = [pa0, pa0 + na) of x2 and Q' = [qb0, qb0 + nb) of y2 (atoms B of {x2, y2}),
// through the state vectors b1(i, a) of s and b2(j, b) of t:
//   exchange = sum_{A, B} gamma_lr[A, B] sum_{a, j} U^A_aj W^B_aj,
//   U^A_aj = sum_i q^A_ij b1(i, a) = 1/2 sum_{mu in A} (L1c[mu, a] R1s[mu, j] + L1s[mu, a] R1c[mu, j]),
//   W^B_aj = sum_b q^B_ab b2(j, b) = 1/2 sum_{nu in B} (L2c[nu, a] R2s[nu, j] + L2s[nu, a] R2c[nu, j]),
// with per-AO rows L1c = C_P b1, L1s = (S C)_P b1 (state s), R1c = C_Q, R1s = (S C)_Q, L2c = C_P',
// L2s = (S C)_P', R2c = C_Q' b2^T, R2s = (S C)_Q' b2^T (state t); on the other monomer of a pair,
// C is zero and S C is the cross product S_yx C_x.  The passes:
//   1. side-1 arrays L1c, L1s per (state s, partner monomer) and side-2 arrays R2c, R2s per (state t,
//      monomer set): batched small GEMMs (ex_gemm_kernel) into FP64 scratch;
//   2. one CTA per side-2 group and ta x tj tile of (a, j) (ta tj <= 128) (ex_vu_kernel): the tile's
//      L2 / R2 rows staged in shared memory, W formed there, then the gamma block in the staging area
//      and V^A_aj = sum_B gamma_lr[A, B] W^B_aj accumulated in registers per block of atoms A and kept
//      in shared memory; then for each element (s, t) of the group, s's L1 rows and the R1 rows
//      staged, sum_A U^A_aj V^A_aj, block sum, added to H.
// A side-2 group (t, its monomers, the side-1 monomers) serves every s paired with it: the four LE
// states of a monomer against one LE or CT state share V, which is formed once.

// Per-monomer device views: C and S C ([n x n], row-major, columns = MOs), atom range, AO offsets.
struct ExMono {
    const double *C, *SC;
    const int *ao_off;   // [n_atoms + 1], local
    int n, n_atoms, atom0;
};

// side-1 group: the occupied-side arrays of one state against one partner monomer
struct ExS1 {
    int x1, y1;                      // monomers (y1 == x1: one monomer)
    int p0, np, q0, na;              // columns P of x1, Q of y1 (start), a extent
    const double *X1;                // b1(i, a) = X1[(i1 + i) * ld1 + a1 + a]
    int ld1, i1, a1;
    const double *cross_yx1;         // S_y1x1 C_x1 [n_y1 x n_x1] (two monomers)
    const double *cross_xy1;         // S_x1y1 C_y1 [n_x1 x n_y1] (two monomers)
    long long own;                   // rows of x1: L1c at own, L1s at own + n_x1 na, [mu][a] (per state)
    long long crs;                   // rows of y1: L1s at crs, [mu - n_x1][a] (per state and y1; L1c = 0)
};

// side-2 group: the virtual-side arrays and V of one state against one monomer set
struct ExS2 {
    int x1, y1;                      // side-1 monomers: the atoms A of V
    int x2, y2;
    int pa0, na, qb0, nb, nq;
    int ta, tj;                      // tile sides over a and j (ta tj <= XJ_T)
    const double *X2;                // b2(j, b) = X2[(j2 + j) * ld2 + b2 + b]
    int ld2, j2, b2;
    const double *cross_xy2, *cross_yx2;
    long long own;                   // rows of y2 (x2 = y2: all rows): R2c at own, R2s at own + n_y2 nq, [nu][j]
    long long crs;                   // rows of x2 when x2 != y2: R2s at crs, [nu][j] (per state and x2; R2c = 0)
};

struct ExEl {
    int s, t;                        // matrix element (s < t)
    int k1, k2;                      // side-1 and side-2 groups
};

constexpr int XJ_T = 128;            // threads per CTA: the largest (a, j) tile
constexpr int XJ_TS = 16;            // largest tile side
constexpr int XJ_AO = 2 * 102 + 4;   // AOs of two monomers (largest supported monomer: 102 AOs)
constexpr int XJ_ATOMS = 80;         // atoms of two monomers (largest supported monomer: 40 atoms)

__device__ __forceinline__ int ex_nao(const ExMono &x, const ExMono &y, bool two) { return x.n + (two ? y.n : 0); }
__device__ __forceinline__ int ex_nat(const ExMono &x, const ExMono &y, bool two) {
    return x.n_atoms + (two ? y.n_atoms : 0);
}

// Shared memory of ex_vu_kernel, by phase (every array [row][tile column]; byte offsets):
//   A: W [0, W) | L2 / R2 staging [W, W + ST)
//   B: W [0, W) | gamma block [W, W + G) | V [W + G, W + G + V)
//   C: L1 / R1 staging [0, ST) | V
// The staged rows hold (C, S C) pairs side by side, so one vector load fetches both.
// FP64: 215 KB, FP32: 108 KB.
template <class T> struct ExPair;
template <> struct ExPair<float> { using type = float2; };
template <> struct ExPair<double> { using type = double2; };

template <class T>
struct ExVUSmem {
    static constexpr size_t W_BYTES = sizeof(T) * XJ_ATOMS * XJ_T;
    static constexpr size_t ST_BYTES = sizeof(T) * 4 * XJ_AO * XJ_TS;
    static constexpr size_t G_BYTES = sizeof(T) * XJ_ATOMS * XJ_ATOMS;
    static constexpr size_t V_OFF = W_BYTES + G_BYTES;
    static constexpr size_t V_BYTES = sizeof(T) * XJ_ATOMS * XJ_T;
    static constexpr size_t END =
        W_BYTES + ST_BYTES > V_OFF + V_BYTES ? W_BYTES + ST_BYTES : V_OFF + V_BYTES;
    static constexpr size_t BYTES = END + sizeof(double) * (XJ_T / 32);
    static_assert(ST_BYTES <= V_OFF, "the side-1 staging of phase C would overlap V");
    static_assert(BYTES <= 227 * 1024, "over the shared memory of one CTA");
};

// one CTA per (side-2 group, ta x tj tile of (a, j)):
//   V^A_aj = sum_B gamma_lr[A, B] W^B_aj, then for every element (s, t) of the group
//   H[s, t] -= sum_A sum_aj U^A_aj(s) V^A_aj
template <class T>
__global__ void __launch_bounds__(XJ_T) ex_vu_kernel(const int4 *__restrict__ tiles, const ExS2 *__restrict__ keys,
                                                     const int *__restrict__ el_begin, const ExEl *__restrict__ els,
                                                     const ExS1 *__restrict__ k1s, const ExMono *__restrict__ mono,
                                                     const double *__restrict__ gamma_lr, int n_atoms_total,
                                                     const double *__restrict__ scr, double *H, int n_states) {
    constexpr int CH = sizeof(T) == 4 ? 16 : 8;   // atoms A per register block
    using L = ExVUSmem<T>;
    extern __shared__ __align__(16) unsigned char xv_raw[];
    using T2 = typename ExPair<T>::type;   // (C, S C) of one row and column
    T(*W)[XJ_T] = reinterpret_cast<T(*)[XJ_T]>(xv_raw);
    T2(*L2)[XJ_TS] = reinterpret_cast<T2(*)[XJ_TS]>(xv_raw + L::W_BYTES);
    T2(*R2)[XJ_TS] = L2 + XJ_AO;
    T(*G)[XJ_ATOMS] = reinterpret_cast<T(*)[XJ_ATOMS]>(xv_raw + L::W_BYTES);
    T(*V)[XJ_T] = reinterpret_cast<T(*)[XJ_T]>(xv_raw + L::V_OFF);
    T2(*L1)[XJ_TS] = reinterpret_cast<T2(*)[XJ_TS]>(xv_raw);
    T2(*R1)[XJ_TS] = L1 + XJ_AO;
    double *red = reinterpret_cast<double *>(xv_raw + L::END);

    const int4 tl = tiles[blockIdx.x];
    const ExS2 K = keys[tl.x];
    const int a0 = tl.y, j0 = tl.z, ta = K.ta, tj = K.tj;
    const ExMono m1x = mono[K.x1], m1y = mono[K.y1], m2x = mono[K.x2], m2y = mono[K.y2];
    const bool two1 = K.x1 != K.y1, two2 = K.x2 != K.y2;
    const int nat1 = ex_nat(m1x, m1y, two1), nat2 = ex_nat(m2x, m2y, two2);
    const int nao1 = ex_nao(m1x, m1y, two1), nao2 = ex_nao(m2x, m2y, two2);
    const int al = threadIdx.x / tj, jl = threadIdx.x % tj;
    const bool active = threadIdx.x < ta * tj && a0 + al < K.na && j0 + jl < K.nq;

    // ---- phase A: L2 = C_P', (S C)_P' (S_y2x2 C_x2 on y2) and R2 (side-2 scratch); W ----
#pragma unroll 4
    for (int e = threadIdx.x; e < nao2 * ta; e += XJ_T) {
        const int nu = e / ta, q = e % ta;
        T c = T(0), sc = T(0);
        if (a0 + q < K.na) {
            const int col = K.pa0 + a0 + q;
            if (nu < m2x.n) {
                c = (T)m2x.C[(long long)nu * m2x.n + col];
                sc = (T)m2x.SC[(long long)nu * m2x.n + col];
            } else {
                sc = (T)K.cross_yx2[(long long)(nu - m2x.n) * m2x.n + col];
            }
        }
        L2[nu][q] = T2{c, sc};
    }
    {
        const int ny2 = two2 ? m2y.n : m2x.n;   // rows held by the per-state part
        const double *rc = scr + K.own, *rs = rc + (long long)ny2 * K.nq;
#pragma unroll 4
        for (int e = threadIdx.x; e < nao2 * tj; e += XJ_T) {
            const int nu = e / tj, q = e % tj;
            T c = T(0), sc = T(0);
            if (j0 + q < K.nq) {
                const int j = j0 + q;
                if (!two2) {
                    c = (T)rc[(long long)nu * K.nq + j];
                    sc = (T)rs[(long long)nu * K.nq + j];
                } else if (nu < m2x.n) {
                    sc = (T)scr[K.crs + (long long)nu * K.nq + j];
                } else {
                    c = (T)rc[(long long)(nu - m2x.n) * K.nq + j];
                    sc = (T)rs[(long long)(nu - m2x.n) * K.nq + j];
                }
            }
            R2[nu][q] = T2{c, sc};
        }
    }
    __syncthreads();
    for (int B = 0; B < nat2; ++B) {
        const bool onx = B < m2x.n_atoms;
        const ExMono &mb = onx ? m2x : m2y;
        const int bl = onx ? B : B - m2x.n_atoms;
        const int base = onx ? 0 : m2x.n;
        T w = T(0);
        if (active)
            for (int nu = base + mb.ao_off[bl]; nu < base + mb.ao_off[bl + 1]; ++nu) {
                const T2 l = L2[nu][al], r = R2[nu][jl];
                w += l.x * r.y + l.y * r.x;
            }
        W[B][threadIdx.x] = T(0.5) * w;
    }
    __syncthreads();   // the staged rows are dead: the gamma block takes their place

    // ---- phase B: gamma block, V = gamma W ----
    const int nA = (nat1 + CH - 1) / CH * CH;
#pragma unroll 4
    for (int e = threadIdx.x; e < nat2 * nA; e += XJ_T) {
        const int B = e / nA, A = e % nA;
        T g = T(0);
        if (A < nat1) {
            const int gA = A < m1x.n_atoms ? m1x.atom0 + A : m1y.atom0 + (A - m1x.n_atoms);
            const int gB = B < m2x.n_atoms ? m2x.atom0 + B : m2y.atom0 + (B - m2x.n_atoms);
            g = (T)gamma_lr[(long long)gB * n_atoms_total + gA];   // gamma_lr is symmetric: A runs along a row
        }
        G[B][A] = g;
    }
    __syncthreads();
    for (int A0 = 0; A0 < nat1; A0 += CH) {
        T acc[CH];
#pragma unroll
        for (int k = 0; k < CH; ++k) acc[k] = T(0);
        for (int B = 0; B < nat2; ++B) {
            const T w = W[B][threadIdx.x];
#pragma unroll
            for (int k = 0; k < CH; ++k) acc[k] += G[B][A0 + k] * w;
        }
#pragma unroll
        for (int k = 0; k < CH; ++k)
            if (A0 + k < nat1) V[A0 + k][threadIdx.x] = acc[k];
    }
    __syncthreads();   // W and the gamma block are dead: the side-1 rows take their place

    // ---- phase C: per element, L1 (side-1 scratch), R1 = C_Q, (S C)_Q (S_x1y1 C_y1 on x1); U . V ----
    const int eb = el_begin[tl.x], ee = el_begin[tl.x + 1];
    for (int ei = eb; ei < ee; ++ei) {
        const ExEl E = els[ei];
        const ExS1 K1 = k1s[E.k1];
        const double *l1c = scr + K1.own, *l1s = l1c + (long long)m1x.n * K1.na;
#pragma unroll 4
        for (int e = threadIdx.x; e < nao1 * ta; e += XJ_T) {
            const int mu = e / ta, q = e % ta;
            T c = T(0), sc = T(0);
            if (a0 + q < K1.na) {
                const int a = a0 + q;
                if (mu < m1x.n) {
                    c = (T)l1c[(long long)mu * K1.na + a];
                    sc = (T)l1s[(long long)mu * K1.na + a];
                } else {
                    sc = (T)scr[K1.crs + (long long)(mu - m1x.n) * K1.na + a];
                }
            }
            L1[mu][q] = T2{c, sc};
        }
        if (ei == eb) {   // the same columns Q of y1 for every element of the group
#pragma unroll 4
            for (int e = threadIdx.x; e < nao1 * tj; e += XJ_T) {
                const int mu = e / tj, q = e % tj;
                T c = T(0), sc = T(0);
                if (j0 + q < K.nq) {
                    const int col = K1.q0 + j0 + q;
                    if (!two1) {
                        c = (T)m1x.C[(long long)mu * m1x.n + col];
                        sc = (T)m1x.SC[(long long)mu * m1x.n + col];
                    } else if (mu < m1x.n) {
                        sc = (T)K1.cross_xy1[(long long)mu * m1y.n + col];
                    } else {
                        c = (T)m1y.C[(long long)(mu - m1x.n) * m1y.n + col];
                        sc = (T)m1y.SC[(long long)(mu - m1x.n) * m1y.n + col];
                    }
                }
                R1[mu][q] = T2{c, sc};
            }
        }
        __syncthreads();
        T acc = T(0);
        if (active) {
            for (int A = 0; A < nat1; ++A) {
                const bool onx = A < m1x.n_atoms;
                const ExMono &ma = onx ? m1x : m1y;
                const int aloc = onx ? A : A - m1x.n_atoms;
                const int base = onx ? 0 : m1x.n;
                T u = T(0);
                for (int mu = base + ma.ao_off[aloc]; mu < base + ma.ao_off[aloc + 1]; ++mu) {
                    const T2 l = L1[mu][al], r = R1[mu][jl];
                    u += l.x * r.y + l.y * r.x;
                }
                acc += u * V[A][threadIdx.x];
            }
            acc *= T(0.5);
        }
        double d = (double)acc;
        for (int o = 16; o; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = d;
        __syncthreads();   // also: the next element's staging overwrites L1 only after every thread is done
        if (threadIdx.x == 0) {
            double tot = 0.0;
            for (int w = 0; w < XJ_T / 32; ++w) tot += red[w];
            atomicAdd(H + (long long)E.s * n_states + E.t, -tot);
        }
    }
}

// ----------------------------------------------------------------------------------------------
// one-electron LE-CT couplings (integrals.rs:542-600)
// ----------------------------------------------------------------------------------------------

// le on the CT's electron monomer: -sum_{ij} F'[l_i, h_j] (X_le X_ct^T)_ij (occupied blocks);
// le on the CT's hole monomer: +sum_{ab} F'[h_a, l_b] (X_le^T X_ct)_ab (virtual blocks).
// F'[p, q] of monomer p-block x and q-block y: Fb[p * fp + q * fq].
struct Ex1eJob {
    int s, t;           // LE state, CT state
    int on_elec;        // 1: LE monomer = electron monomer of the CT
    const double *Xl, *Xc;
    int ol, vl, oc, vc; // LE: o x v, CT: o_h x v_l
    const double *F;
    long long fp, fq;   // strides of F'[row of the LE monomer, column of the other monomer]
    int r0, c0;         // MO offsets of the used blocks (0 for occupied, n_occ for virtual)
};

__global__ void ex_1e_kernel(const Ex1eJob *__restrict__ jobs, double *H, int n_states) {
    __shared__ double red[8];
    const Ex1eJob J = jobs[blockIdx.x];
    double acc = 0.0;
    if (J.on_elec) {
        // t_ij = sum_a Xl[i, a] Xc[j, a], i < ol, j < oc
        for (int e = threadIdx.x; e < J.ol * J.oc; e += blockDim.x) {
            const int i = e / J.oc, j = e % J.oc;
            double t = 0.0;
            for (int a = 0; a < J.vl; ++a) t += J.Xl[(long long)i * J.vl + a] * J.Xc[(long long)j * J.vc + a];
            acc -= J.F[(long long)(J.r0 + i) * J.fp + (long long)(J.c0 + j) * J.fq] * t;
        }
    } else {
        // t_ab = sum_i Xl[i, a] Xc[i, b], a < vl, b < vc
        for (int e = threadIdx.x; e < J.vl * J.vc; e += blockDim.x) {
            const int a = e / J.vc, b = e % J.vc;
            double t = 0.0;
            for (int i = 0; i < J.ol; ++i) t += J.Xl[(long long)i * J.vl + a] * J.Xc[(long long)i * J.vc + b];
            acc += J.F[(long long)(J.r0 + a) * J.fp + (long long)(J.c0 + b) * J.fq] * t;
        }
    }
    for (int off = 16; off; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
        atomicAdd(H + (long long)J.s * n_states + J.t, tot);
    }
}

// ----------------------------------------------------------------------------------------------
// Davidson on the dense exciton matrix: small kernels
// ----------------------------------------------------------------------------------------------

// rk[r] -= u[r] ritz[r] (rows of length n)
__global__ void ex_residual_kernel(int k, int n, const double *__restrict__ u, const double *__restrict__ ritz,
                                   double *rk) {
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= (long long)k * n) return;
    rk[idx] -= u[idx / n] * ritz[idx];
}

// out = r / (w - diag(H)) (the dense engine's preconditioner, solvers/mod.rs:45-47)
__global__ void ex_precondition_kernel(int n, const double *__restrict__ r, double w, const double *__restrict__ H,
                                       double *out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x < n) out[x] = r[x] / (w - H[(long long)x * n + x]);
}

__global__ void ex_row_norms_kernel(int k, int n, const double *__restrict__ a, double *out) {
    __shared__ double red[8];
    const double *row = a + (long long)blockIdx.x * n;
    double s = 0.0;
    for (int x = threadIdx.x; x < n; x += blockDim.x) s += row[x] * row[x];
    for (int off = 16; off; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        out[blockIdx.x] = sqrt(t);
    }
}

// *nrm = sqrt(sum of the k partial sums), added in a fixed order
__global__ void ex_norm_finish_kernel(int k, const double *__restrict__ part, double *nrm) {
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < k; ++i) t += part[i];
        *nrm = sqrt(t);
    }
}

// out[i, x] = sum_k A[i, k] B[k, x] (k in order), one thread per output; A [M x K], B [K x N], out [M x N]
// row-major (the Davidson's new products H v_i, Ritz vectors and Y^T AV)
// out[i][x] = sum_k A[i][k] B[k][x] split over K: part[s][i][x] = sum over chunk s of k (gridDim.z = S
// chunks), then
// ex_rowprod_sum_kernel adds the S partial sums in chunk order (fixed order: a row's value does not
// depend on the other rows of the launch)
__global__ void ex_rowprod_part_kernel(int N, int K, const double *__restrict__ A, const double *__restrict__ B,
                                       double *__restrict__ part) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y, sc = blockIdx.z, S = gridDim.z;
    if (x >= N) return;
    const int k0 = (int)((long long)K * sc / S), k1 = (int)((long long)K * (sc + 1) / S);
    const double *a = A + (long long)i * K;
    double acc = 0.0;
    for (int k = k0; k < k1; ++k) acc += a[k] * B[(long long)k * N + x];
    part[((long long)sc * gridDim.y + i) * N + x] = acc;
}

__global__ void ex_rowprod_sum_kernel(long long len, int S, const double *__restrict__ part, double *__restrict__ out) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= len) return;
    double acc = 0.0;
    for (int sc = 0; sc < S; ++sc) acc += part[(long long)sc * len + t];
    out[t] = acc;
}

// C[i, j] = A_i . B_j (rows of length K), one warp per entry (lane-strided sums, fixed shuffle order)
__global__ void ex_dotmat_kernel(int M, int N, int K, const double *__restrict__ A, const double *__restrict__ B,
                                 double *C) {
    const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= (long long)M * N) return;
    const int i = (int)(w / N), j = (int)(w % N);
    const double *a = A + (long long)i * K, *b = B + (long long)j * K;
    double acc = 0.0;
    for (int k = lane; k < K; k += 32) acc += a[k] * b[k];
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) C[(long long)i * N + j] = acc;
}

// the Davidson's growing basis with its size m in device memory: c[i] = V_i . v for i < *m
__global__ void ex_dots_dev_kernel(const int *__restrict__ m, int n, const double *__restrict__ V,
                                   const double *__restrict__ v, double *c) {
    if ((int)blockIdx.x >= *m) return;
    __shared__ double red[8];
    const double *row = V + (long long)blockIdx.x * n;
    double s = 0.0;
    for (int x = threadIdx.x; x < n; x += blockDim.x) s += row[x] * v[x];
    for (int off = 16; off; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        c[blockIdx.x] = t;
    }
}

// v -= c^T V for i < *m, one thread per component; each CTA's sum of squares into part[]
// part2[s][x] = sum over chunk s of i < *m of c[i] V[i][x] (gridDim.y = S chunks)
__global__ void ex_orth_part_kernel(const int *__restrict__ m, int n, const double *__restrict__ V,
                                    const double *__restrict__ c, double *__restrict__ part2) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, sc = blockIdx.y, S = gridDim.y, mm = *m;
    if (x >= n) return;
    const int i0 = (int)((long long)mm * sc / S), i1 = (int)((long long)mm * (sc + 1) / S);
    double acc = 0.0;
    for (int i = i0; i < i1; ++i) acc += c[i] * V[(long long)i * n + x];
    part2[(long long)sc * n + x] = acc;
}

// v -= sum of the S partial sums (chunk order), with the block partial sums of |v|^2
__global__ void ex_orth_finish_kernel(int n, int S, const double *__restrict__ part2, double *v, double *part) {
    __shared__ double red[8];
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    double s = 0.0;
    if (x < n) {
        double acc = 0.0;
        for (int sc = 0; sc < S; ++sc) acc += part2[(long long)sc * n + x];
        const double y = v[x] - acc;
        v[x] = y;
        s = y * y;
    }
    for (int off = 16; off; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        part[blockIdx.x] = t;
    }
}

// tincr's drop rule (davidson.rs:162-168): the correction joins the basis as row *m when its norm
// exceeds 1e-8 (and the basis has room); ex_count_kernel then advances *m
__global__ void ex_append_kernel(int n, const double *__restrict__ nrm, const int *__restrict__ m, int cap,
                                 const double *__restrict__ t, double *V) {
    const double r = *nrm;
    const int mm = *m;
    if (!(r > 1.0e-8) || mm >= cap) return;
    const double f = 1.0 / r;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x < n) V[(long long)mm * n + x] = t[x] * f;
}

__global__ void ex_count_kernel(const double *__restrict__ nrm, int *m, int cap) {
    if (threadIdx.x == 0 && *nrm > 1.0e-8 && *m < cap) ++*m;
}

__global__ void ex_set_int_kernel(int *p, int v) {
    if (threadIdx.x == 0) *p = v;
}

__global__ void ex_diag_kernel(int n, const double *__restrict__ H, double *d) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x < n) d[x] = H[(long long)x * n + x];
}

}  // namespace

// ----------------------------------------------------------------------------------------------
// host driver
// ----------------------------------------------------------------------------------------------

namespace {

struct PairKey {
    int i, j;
    bool operator<(const PairKey &o) const { return i != o.i ? i < o.i : j < o.j; }
};

template <class T>
static void upload_vec(cudaStream_t st, DevBuf<T> &d, const std::vector<T> &h) {
    d.alloc(std::max<size_t>(1, h.size()));
    if (!h.empty()) TINCR_CUDA(cudaMemcpyAsync(d.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, st));
}

}  // namespace

int Ctx::exciton_states(int n_mono, const tincr_exciton_monomer *mono, int n_pairs, const tincr_exciton_pair *pairs,
                        int n_ct, const tincr_exciton_ct *cts, int n_atoms_total, const double *gamma,
                        const double *gamma_lr, int precision, int n_roots, double tol, int max_iter, double *h_out,
                        double *energies, double *vectors, int *iterations) {
    if (n_mono <= 0 || !mono || n_atoms_total <= 0 || !gamma || !gamma_lr || n_roots <= 0 || max_iter <= 0 ||
        !energies || (n_ct > 0 && !cts) || (n_pairs > 0 && !pairs))
        fail(TINCR_BAD_ARG, "exciton_states: bad arguments");
    if (precision != TINCR_PREC_FP64 && precision != TINCR_PREC_BF16X3)
        fail(TINCR_BAD_ARG, "exciton_states: unknown precision");
    const bool fp32 = precision == TINCR_PREC_BF16X3;
    constexpr int ACTIVE = 10;   // restricted active space of the LE-CT / CT-CT exchange (settings.rs:110-118)
    TINCR_CUDA(cudaEventRecord(ev0, stream));
    g_launches = 0;

    // ---- monomers: C, S C, AO offsets; states ----
    std::vector<int> atom0(n_mono), nao(n_mono), no(n_mono);
    int atoms_sum = 0;
    for (int k = 0; k < n_mono; ++k) {
        const tincr_exciton_monomer &m = mono[k];
        if (m.n_atoms <= 0 || m.n_orb <= 0 || m.n_occ <= 0 || m.n_occ >= m.n_orb || !m.orbs_per_atom || !m.c || !m.s ||
            !m.orbe || m.n_le < 0 || (m.n_le > 0 && (!m.le_energies || !m.le_coefficients || !m.le_q_trans)))
            fail(TINCR_BAD_ARG, "exciton_states: bad monomer " + std::to_string(k));
        if (m.n_orb > 102 || m.n_atoms > XJ_ATOMS / 2)
            fail(TINCR_BAD_ARG, "exciton_states: monomers of up to 102 AOs and 40 atoms are supported");
        if (m.n_occ < ACTIVE || m.n_orb - m.n_occ < ACTIVE)
            fail(TINCR_BAD_ARG, "exciton_states: a monomer has fewer than 10 occupied or virtual orbitals");
        atom0[k] = atoms_sum;
        atoms_sum += m.n_atoms;
        nao[k] = m.n_orb;
        no[k] = m.n_occ;
        check_finite(m.c, (size_t)m.n_orb * m.n_orb, "monomer C");
        check_finite(m.s, (size_t)m.n_orb * m.n_orb, "monomer S");
    }
    if (atoms_sum != n_atoms_total) fail(TINCR_BAD_ARG, "exciton_states: atom count differs from the monomers'");

    // concatenated C, S, orbital energies, AO offsets
    std::vector<long long> offC(n_mono + 1, 0), offAo(n_mono + 1, 0);
    for (int k = 0; k < n_mono; ++k) {
        offC[k + 1] = offC[k] + (long long)nao[k] * nao[k];
        offAo[k + 1] = offAo[k] + mono[k].n_atoms + 1;
    }
    std::vector<double> hC(offC[n_mono]), hS(offC[n_mono]);
    std::vector<int> hAo(offAo[n_mono]);
    for (int k = 0; k < n_mono; ++k) {
        std::copy(mono[k].c, mono[k].c + (size_t)nao[k] * nao[k], hC.begin() + offC[k]);
        std::copy(mono[k].s, mono[k].s + (size_t)nao[k] * nao[k], hS.begin() + offC[k]);
        int acc = 0;
        for (int a = 0; a < mono[k].n_atoms; ++a) {
            hAo[offAo[k] + a] = acc;
            acc += mono[k].orbs_per_atom[a];
        }
        hAo[offAo[k] + mono[k].n_atoms] = acc;
        if (acc != nao[k]) fail(TINCR_BAD_ARG, "exciton_states: orbitals per atom do not add up to n_orb");
    }
    DevBuf<double> dC, dS, dSC, dG, dGlr;
    DevBuf<int> dAo;
    upload_vec(stream, dC, hC);
    upload_vec(stream, dS, hS);
    upload_vec(stream, dAo, hAo);
    dSC.alloc(hC.size());
    TINCR_CUDA(cudaMemsetAsync(dSC.p, 0, hC.size() * sizeof(double), stream));
    // the large inputs (gamma, gamma_lr, the real pairs' dimer orbitals) go through the context's
    // page-locked staging buffer: parallel host copies, then one DMA each
    const size_t n_g = (size_t)n_atoms_total * n_atoms_total;
    size_t pin_need = 2 * n_g + 1;   // (+1: the Davidson's basis size read back)
    for (int p = 0; p < n_pairs; ++p)   // overlap blocks (pairs with bad indices are rejected below)
        if (pairs[p].i >= 0 && pairs[p].i < n_mono && pairs[p].j >= 0 && pairs[p].j < n_mono)
            pin_need += (size_t)nao[pairs[p].i] * nao[pairs[p].j];
    for (int p = 0; p < n_pairs; ++p)   // (pairs with bad indices are rejected below)
        if (pairs[p].real && pairs[p].i >= 0 && pairs[p].i < n_mono && pairs[p].j >= 0 && pairs[p].j < n_mono) {
            const size_t nij = (size_t)nao[pairs[p].i] + nao[pairs[p].j];
            pin_need += nij * nij + nij;
        }
    for (int k = 0; k < n_mono; ++k)   // LE charges and CI vectors
        pin_need += (size_t)std::max(0, mono[k].n_le) * (mono[k].n_atoms + (size_t)no[k] * (nao[k] - no[k]));
    for (int c = 0; c < n_ct; ++c)     // CT charges and CI vectors (states with bad indices are rejected below)
        if (cts && cts[c].h >= 0 && cts[c].h < n_mono && cts[c].l >= 0 && cts[c].l < n_mono)
            pin_need += (size_t)mono[cts[c].h].n_atoms + mono[cts[c].l].n_atoms +
                        (size_t)no[cts[c].h] * (nao[cts[c].l] - no[cts[c].l]);
    ex_pin.reserve(pin_need);
    size_t pin_used = 0;
    auto stage = [&](double *dst, const double *src, size_t n, const char *what) {
        double *h = ex_pin.p + pin_used;
        pin_used += n;
        const long long chunk = 1 << 18, nc = ((long long)n + chunk - 1) / chunk;
        long long bad = 0;
#pragma omp parallel for schedule(static) num_threads(8) reduction(+ : bad)
        for (long long c = 0; c < nc; ++c) {
            const size_t a = (size_t)c * chunk, b = std::min(n, a + (size_t)chunk);
            for (size_t x = a; x < b; ++x) {
                h[x] = src[x];
                bad += !std::isfinite(src[x]);
            }
        }
        if (bad) fail(TINCR_NONFINITE, std::string("non-finite value in ") + what);
        TINCR_CUDA(cudaMemcpyAsync(dst, h, n * sizeof(double), cudaMemcpyHostToDevice, stream));
    };
    dG.alloc(n_g);
    dGlr.alloc(n_g);
    stage(dG.p, gamma, n_g, "gamma");
    stage(dGlr.p, gamma_lr, n_g, "gamma_lr");

    // pairs: type, S_xy, dimer SCC
    std::map<PairKey, int> pidx;
    for (int p = 0; p < n_pairs; ++p) {
        const tincr_exciton_pair &q = pairs[p];
        if (q.i < 0 || q.j <= q.i || q.j >= n_mono || !q.s_ij) fail(TINCR_BAD_ARG, "exciton_states: bad pair");
        if (q.real && (!q.pair_orbs || !q.pair_orbe)) fail(TINCR_BAD_ARG, "exciton_states: real pair without its SCC");
        pidx[PairKey{q.i, q.j}] = p;
    }
    // dense pair lookup: the pair index of monomers (a, b), -1 when not listed
    std::vector<int> pdense((size_t)n_mono * n_mono, -1);
    for (auto &kv : pidx) {
        pdense[(size_t)kv.first.i * n_mono + kv.first.j] = kv.second;
        pdense[(size_t)kv.first.j * n_mono + kv.first.i] = kv.second;
    }
    auto is_real = [&](int a, int b) {
        if (a == b) return false;
        const int p = pdense[(size_t)a * n_mono + b];
        return p >= 0 && pairs[p].real != 0;
    };
    // cross products S_xy C_y (n_x x n_y) and S_yx C_x (n_y x n_x) of every listed pair
    std::vector<long long> offX(n_pairs + 1, 0);
    for (int p = 0; p < n_pairs; ++p) offX[p + 1] = offX[p] + 2LL * nao[pairs[p].i] * nao[pairs[p].j];
    std::vector<long long> offSxy(n_pairs + 1, 0);
    for (int p = 0; p < n_pairs; ++p) offSxy[p + 1] = offSxy[p] + (long long)nao[pairs[p].i] * nao[pairs[p].j];
    // the overlap blocks, packed in parallel into the staging buffer (finiteness checked there), one DMA
    if (pin_used + offSxy[n_pairs] > ex_pin.n) {   // (counted above; growing drops the staged copies)
        sync();
        ex_pin.reserve(pin_used + offSxy[n_pairs] + 1);
    }
    double *hSxy = ex_pin.p + pin_used;
    pin_used += offSxy[n_pairs];
    int bad_overlap = -1;
#pragma omp parallel for schedule(dynamic, 8) num_threads(8)
    for (int p = 0; p < n_pairs; ++p) {
        const long long sz = offSxy[p + 1] - offSxy[p];
        bool ok = true;
        for (long long x = 0; x < sz; ++x) {
            hSxy[offSxy[p] + x] = pairs[p].s_ij[x];
            ok = ok && std::isfinite(pairs[p].s_ij[x]);
        }
        if (!ok) {
#pragma omp critical
            bad_overlap = p;
        }
    }
    if (bad_overlap >= 0) fail(TINCR_NONFINITE, "non-finite value in pair overlap");
    DevBuf<double> dSxy, dCross;
    dSxy.alloc(std::max<long long>(1, offSxy[n_pairs]));
    if (offSxy[n_pairs])
        TINCR_CUDA(cudaMemcpyAsync(dSxy.p, hSxy, offSxy[n_pairs] * sizeof(double), cudaMemcpyHostToDevice, stream));
    dCross.alloc(std::max<long long>(1, offX[n_pairs]));
    TINCR_CUDA(cudaMemsetAsync(dCross.p, 0, dCross.n * sizeof(double), stream));
    auto cross = [&](int x, int y) -> const double * {   // S_xy C_y, [n_x x n_y]
        if (x == y) return nullptr;
        const int p = pdense[(size_t)x * n_mono + y];
        if (p < 0) return nullptr;
        const long long half = (long long)nao[pairs[p].i] * nao[pairs[p].j];
        return dCross.p + offX[p] + (x == pairs[p].i ? 0 : half);
    };

    DevBuf<GemmJob> dJobs;
    DevBuf<int4> dTiles;
    GemmBatch gb;
    // S C per monomer and the cross products (FP64 in both precisions: they feed every exchange job)
    for (int k = 0; k < n_mono; ++k) {
        const int n = nao[k];
        gb.gemm(n, n, n, dS.p + offC[k], n, 1, dC.p + offC[k], n, 1, dSC.p + offC[k], n, 1.0);
    }
    for (int p = 0; p < n_pairs; ++p) {
        const int i = pairs[p].i, j = pairs[p].j, ni = nao[i], nj = nao[j];
        const double *sij = dSxy.p + offSxy[p];
        // S_ij C_j [ni x nj]
        gb.gemm(ni, nj, nj, sij, nj, 1, dC.p + offC[j], nj, 1, dCross.p + offX[p], nj, 1.0);
        // S_ji C_i = S_ij^T C_i [nj x ni]
        gb.gemm(nj, ni, ni, sij, 1, nj, dC.p + offC[i], ni, 1, dCross.p + offX[p] + (long long)ni * nj, ni, 1.0);
    }
    gb.run(*this, false, dJobs, dTiles, TINCR_KF_OTHER);

    // states in the basis order: LE (monomer-major), then the CT states as given.  Offsets first, then
    // the charges and CI vectors gathered in parallel into the staging buffer (one DMA each)
    std::vector<ExState> hst;
    std::vector<long long> xoff;
    struct Src {
        const double *q, *x;         // charges [atoms x n] and coefficients [o v x n], column `col` of n
        int n, col, nq;
        long long nx;
    };
    std::vector<Src> src;
    long long nq_tot = 0, nx_tot = 0;
    for (int k = 0; k < n_mono; ++k) {
        const tincr_exciton_monomer &m = mono[k];
        const long long ov = (long long)m.n_occ * (m.n_orb - m.n_occ);
        for (int r = 0; r < m.n_le; ++r) {
            hst.push_back(ExState{0, k, k, atom0[k], m.n_atoms, 0, 0, nq_tot, m.le_energies[r]});
            xoff.push_back(nx_tot);
            src.push_back(Src{m.le_q_trans, m.le_coefficients, m.n_le, r, m.n_atoms, ov});
            nq_tot += m.n_atoms;
            nx_tot += ov;
        }
    }
    for (int c = 0; c < n_ct; ++c) {
        const tincr_exciton_ct &q = cts[c];
        if (q.h < 0 || q.h >= n_mono || q.l < 0 || q.l >= n_mono || q.h == q.l || q.n_ct <= 0 || q.state < 0 ||
            q.state >= q.n_ct || !q.energies || !q.coefficients || !q.q_tr)
            fail(TINCR_BAD_ARG, "exciton_states: bad CT state");
        if (pdense[(size_t)q.h * n_mono + q.l] < 0) fail(TINCR_BAD_ARG, "exciton_states: CT state of an unlisted pair");
        const long long ov = (long long)no[q.h] * (nao[q.l] - no[q.l]);
        const int nh = mono[q.h].n_atoms, nl = mono[q.l].n_atoms;
        hst.push_back(ExState{1, q.h, q.l, atom0[q.h], nh, atom0[q.l], nl, nq_tot, q.energies[q.state]});
        xoff.push_back(nx_tot);
        src.push_back(Src{q.q_tr, q.coefficients, q.n_ct, q.state, nh + nl, ov});
        nq_tot += nh + nl;
        nx_tot += ov;
    }
    const int ns = (int)hst.size();
    if (ns < n_roots) fail(TINCR_BAD_ARG, "exciton_states: fewer basis states than roots");
    if (pin_used + nq_tot + nx_tot > ex_pin.n) {   // (counted above; growing drops the staged gamma copies)
        sync();
        ex_pin.reserve(pin_used + nq_tot + nx_tot);
    }
    double *hq = ex_pin.p + pin_used, *hX = hq + nq_tot;
    long long bad = 0;
#pragma omp parallel for schedule(dynamic, 8) num_threads(8) reduction(+ : bad)
    for (int t = 0; t < ns; ++t) {
        const Src &r = src[t];
        double *qo = hq + hst[t].q_off, *xo = hX + xoff[t];
        for (int a = 0; a < r.nq; ++a) {
            qo[a] = r.q[(size_t)a * r.n + r.col];
            bad += !std::isfinite(qo[a]);
        }
        for (long long x = 0; x < r.nx; ++x) {
            xo[x] = r.x[x * r.n + r.col];
            bad += !std::isfinite(xo[x]);
        }
    }
    if (bad) fail(TINCR_NONFINITE, "non-finite value in transition charges or CI coefficients");
    DevBuf<ExState> dst;
    DevBuf<double> dq, dX, dW, dH;
    upload_vec(stream, dst, hst);
    dq.alloc(std::max<long long>(1, nq_tot));
    dX.alloc(std::max<long long>(1, nx_tot));
    if (nq_tot) TINCR_CUDA(cudaMemcpyAsync(dq.p, hq, nq_tot * sizeof(double), cudaMemcpyHostToDevice, stream));
    if (nx_tot) TINCR_CUDA(cudaMemcpyAsync(dX.p, hX, nx_tot * sizeof(double), cudaMemcpyHostToDevice, stream));
    pin_used += nq_tot + nx_tot;
    dW.alloc((size_t)ns * n_atoms_total);
    dH.alloc((size_t)ns * ns);

    // ---- Coulomb and diagonal ----
    {
        const int slot = prof_begin(TINCR_KF_OTHER);
        ex_coul_w_kernel<<<ns, 256, 0, stream>>>(n_atoms_total, dst.p, dq.p, dG.p, dW.p);
        count_launch(stream, "ex_coul_w");
        check_launch("ex_coul_w");
        ex_coul_h_kernel<<<ns, 256, 0, stream>>>(ns, n_atoms_total, dst.p, dq.p, dW.p, dH.p);
        count_launch(stream, "ex_coul_h");
        check_launch("ex_coul_h");
        prof_end(slot, 4.0 * ns * (double)n_atoms_total * 40.0, 0.0);
    }

    // ---- exchange integrals (see the kernels: side-1 groups, side-2 groups with V, elements) ----
    std::vector<ExMono> hm(n_mono);
    for (int k = 0; k < n_mono; ++k)
        hm[k] = ExMono{dC.p + offC[k], dSC.p + offC[k], dAo.p + offAo[k], nao[k], mono[k].n_atoms, atom0[k]};
    DevBuf<ExMono> dm;
    upload_vec(stream, dm, hm);
    auto nao_of = [&](int x, int y) { return (long long)nao[x] + (x != y ? nao[y] : 0); };
    auto nat_of = [&](int x, int y) { return (long long)mono[x].n_atoms + (x != y ? mono[y].n_atoms : 0); };
    std::vector<ExS1> k1v;
    std::vector<ExS2> k2v;
    std::vector<ExEl> elv;
    // side arrays in one FP64 scratch: per state, the rows on its own monomer (C b, S C b), and per
    // state and partner monomer, the cross rows (S_yx C_x b); each computed once and shared by every
    // group that reads it
    struct SideJob {
        int kind;                    // 0: own side 1, 1: cross side 1, 2: own side 2, 3: cross side 2
        int x, y;                    // monomer of the columns; monomer of the rows (cross) or x
        int c0, nc, nout;            // columns [c0, c0 + nc) contracted; output columns (a or j)
        const double *X;             // the state vector and its addressing (side 1: b1(i, a); side 2: b2(j, b))
        int ld, r0;
        long long off;
    };
    std::vector<SideJob> sjobs;
    long long scr = 0;
    std::unordered_map<long long, long long> side_tab;
    side_tab.reserve((size_t)8 * ns + 1024);
    elv.reserve((size_t)64 * ns);
    k2v.reserve((size_t)32 * ns);
    auto side_of = [&](int kind, int state, int mono_key, int variant, int x, int y, int c0, int nc, int nout,
                       const double *X, int ld, int r0, long long rows) -> long long {
        const long long key = (((long long)kind * ns + state) * (n_mono + 1) + mono_key) * 2 + variant;
        auto it = side_tab.find(key);
        if (it != side_tab.end()) return it->second;
        const long long off = scr;
        scr += rows * nout;
        sjobs.push_back(SideJob{kind, x, y, c0, nc, nout, X, ld, r0, off});
        side_tab.emplace(key, off);
        return off;
    };
    auto k1_of = [&](int state, int variant, int x1, int y1, int p0, int np, int q0, int na, const double *X1, int ld1,
                     int i1) -> int {
        ExS1 K;
        K.x1 = x1; K.y1 = y1; K.p0 = p0; K.np = np; K.q0 = q0; K.na = na;
        K.X1 = X1; K.ld1 = ld1; K.i1 = i1; K.a1 = 0;
        K.cross_yx1 = x1 != y1 ? cross(y1, x1) : nullptr;
        K.cross_xy1 = x1 != y1 ? cross(x1, y1) : nullptr;
        K.own = side_of(0, state, n_mono, variant, x1, x1, p0, np, na, X1, ld1, i1, 2LL * nao[x1]);
        K.crs = x1 != y1 ? side_of(1, state, y1, variant, x1, y1, p0, np, na, X1, ld1, i1, nao[y1]) : -1;
        k1v.push_back(K);
        return (int)k1v.size() - 1;
    };
    // group tables keyed by (state, monomer): LE-LE side 1 (s, partner), LE-LE side 2 (t, side-1
    // monomer), LE-CT side 1 (LE state, CT hole), LE-CT side 2 (CT state, LE monomer), CT-CT side 1
    // (s, hole of t)
    std::vector<int> tab[5];
    for (auto &v : tab) v.assign((size_t)ns * n_mono, -1);
    auto k1_cached = [&](int which, int state, int partner, int variant, int x1, int y1, int p0, int np, int q0, int na,
                         const double *X1, int ld1, int i1) -> int {
        int &id = tab[which][(size_t)state * n_mono + partner];
        if (id < 0) id = k1_of(state, variant, x1, y1, p0, np, q0, na, X1, ld1, i1);
        return id;
    };
    auto k2_of = [&](int which, int state, int key, int variant, int x1, int y1, int x2, int y2, int pa0, int na,
                     int qb0, int nb, int nq, const double *X2, int ld2, int j2) -> int {
        int *slot = which >= 0 ? &tab[which][(size_t)state * n_mono + key] : nullptr;
        if (slot && *slot >= 0) return *slot;
        ExS2 K;
        K.x1 = x1; K.y1 = y1; K.x2 = x2; K.y2 = y2;
        K.pa0 = pa0; K.na = na; K.qb0 = qb0; K.nb = nb; K.nq = nq;
        auto side = [](int n) {   // near-equal parts of at most XJ_TS
            const int parts = (n + XJ_TS - 1) / XJ_TS;
            return (n + parts - 1) / parts;
        };
        K.ta = side(na);
        K.tj = side(nq);
        while (K.ta * K.tj > XJ_T) {
            if (K.ta >= K.tj) --K.ta; else --K.tj;
        }
        K.X2 = X2; K.ld2 = ld2; K.j2 = j2; K.b2 = 0;
        K.cross_xy2 = x2 != y2 ? cross(x2, y2) : nullptr;
        K.cross_yx2 = x2 != y2 ? cross(y2, x2) : nullptr;
        K.own = side_of(2, state, n_mono, variant, y2, y2, qb0, nb, nq, X2, ld2, j2, 2LL * nao[y2]);
        K.crs = x2 != y2 ? side_of(3, state, x2, variant, y2, x2, qb0, nb, nq, X2, ld2, j2, nao[x2]) : -1;
        const int id = (int)k2v.size();
        k2v.push_back(K);
        if (slot) *slot = id;
        return id;
    };
    auto listed = [&](int a, int b) { return a == b || cross(a, b) != nullptr; };
    // the elements that carry an exchange term, from neighbour lists (real pairs) rather than from all
    // pairs of states
    std::vector<std::vector<int>> nbr(n_mono);
    for (int p = 0; p < n_pairs; ++p)
        if (pairs[p].real) {
            nbr[pairs[p].i].push_back(pairs[p].j);
            nbr[pairs[p].j].push_back(pairs[p].i);
        }
    for (auto &v : nbr) std::sort(v.begin(), v.end());
    std::vector<int> le0(n_mono + 1, 0);   // LE states of monomer k: [le0[k], le0[k + 1])
    for (int k = 0; k < n_mono; ++k) le0[k + 1] = le0[k] + mono[k].n_le;
    const int n_le_states = le0[n_mono];
    std::unordered_map<long long, std::vector<int>> ct_at;   // (hole, electron) -> CT states
    for (int t = n_le_states; t < ns; ++t) ct_at[(long long)hst[t].hole * n_mono + hst[t].elec].push_back(t);
    // le_le (integrals.rs:81-169): exchange for real pairs, full orbital spaces
    for (int I = 0; I < n_mono; ++I)
        for (int Jm : nbr[I]) {
            if (Jm < I) continue;
            const int oI = no[I], vI = nao[I] - oI, oJ = no[Jm], vJ = nao[Jm] - oJ;
            for (int s = le0[I]; s < le0[I + 1]; ++s)
                for (int t = le0[Jm]; t < le0[Jm + 1]; ++t) {
                    const int k1 = k1_cached(0, s, Jm, 0, I, Jm, 0, oI, 0, vI, dX.p + xoff[s], vI, 0);
                    const int k2 = k2_of(1, t, I, 0, I, Jm, I, Jm, oI, vI, oJ, vJ, oJ, dX.p + xoff[t], vJ, 0);
                    elv.push_back(ExEl{s, t, k1, k2});
                }
        }
    // le_ct_2e_new (integrals.rs:602-727): exchange when the LE monomer is the hole, the electron or a
    // real-pair neighbour of either; restricted active spaces.  A pair that is not listed is an ESD
    // pair, whose AO overlap is zero (its atoms are farther apart than the Slater-Koster tables
    // reach): its charges, and the integral, vanish.
    std::vector<int> cand;
    for (int ct = n_le_states; ct < ns; ++ct) {
        const int h = hst[ct].hole, l = hst[ct].elec;
        cand.assign({h, l});
        cand.insert(cand.end(), nbr[h].begin(), nbr[h].end());
        cand.insert(cand.end(), nbr[l].begin(), nbr[l].end());
        std::sort(cand.begin(), cand.end());
        cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
        const int oh = no[h], vl = nao[l] - no[l];
        for (int I : cand) {
            if (!listed(I, h) || !listed(I, l)) continue;
            const int oI = no[I], vI = nao[I] - oI;
            for (int le = le0[I]; le < le0[I + 1]; ++le) {
                const int k1 = k1_cached(2, le, h, 1, I, h, oI - ACTIVE, ACTIVE, oh - ACTIVE, ACTIVE, dX.p + xoff[le],
                                         vI, oI - ACTIVE);
                const int k2 = k2_of(3, ct, I, 1, I, h, I, l, oI, ACTIVE, no[l], ACTIVE, ACTIVE, dX.p + xoff[ct], vl,
                                     oh - ACTIVE);
                elv.push_back(ExEl{le, ct, k1, k2});
            }
        }
    }
    // ct_ct_new (integrals.rs:733-878): exchange when the holes and the electrons are each on the same
    // monomer or on a real pair (but not both the same pair); restricted active spaces
    for (int s = n_le_states; s < ns; ++s) {
        const int h1 = hst[s].hole, l1 = hst[s].elec, v1 = nao[l1] - no[l1];
        for (int hi = -1; hi < (int)nbr[h1].size(); ++hi) {
            const int h2 = hi < 0 ? h1 : nbr[h1][hi];
            for (int li = -1; li < (int)nbr[l1].size(); ++li) {
                const int l2 = li < 0 ? l1 : nbr[l1][li];
                if (h2 == l2) continue;
                auto it = ct_at.find((long long)h2 * n_mono + l2);
                if (it == ct_at.end()) continue;
                const int v2 = nao[l2] - no[l2];
                for (int t : it->second) {
                    if (t <= s || (h1 == h2 && l1 == l2)) continue;
                    const int k1 = k1_cached(4, s, h2, 1, h1, h2, no[h1] - ACTIVE, ACTIVE, no[h2] - ACTIVE, ACTIVE,
                                             dX.p + xoff[s], v1, no[h1] - ACTIVE);
                    const int k2 = k2_of(-1, t, 0, 1, h1, h2, l1, l2, no[l1], ACTIVE, no[l2], ACTIVE, ACTIVE,
                                         dX.p + xoff[t], v2, no[h2] - ACTIVE);
                    elv.push_back(ExEl{s, t, k1, k2});
                }
            }
        }
    }
    for (auto &v : tab) std::vector<int>().swap(v);
    auto run_exchange = [&](auto zero) {
        using T = decltype(zero);
        if (elv.empty()) return;
        // side arrays (FP64 scratch) by batched GEMMs
        DevBuf<double> d1;
        d1.alloc(std::max<long long>(1, scr));
        TINCR_CUDA(cudaMemsetAsync(d1.p, 0, d1.n * sizeof(double), stream));
        for (const SideJob &J : sjobs) {
            const int nx = nao[J.x], ny = nao[J.y];
            double *out = d1.p + J.off;
            if (J.kind <= 1) {   // side 1: rows x C_P b1 or rows of y (S_yx C_x)_P b1; B(i, a) = X[(r0 + i) ld + a]
                const double *B = J.X + (long long)J.r0 * J.ld;
                if (J.kind == 0) {
                    gb.gemm(nx, J.nout, J.nc, dC.p + offC[J.x] + J.c0, nx, 1, B, J.ld, 1, out, J.nout, 1.0);
                    gb.gemm(nx, J.nout, J.nc, dSC.p + offC[J.x] + J.c0, nx, 1, B, J.ld, 1, out + (long long)nx * J.nout,
                            J.nout, 1.0);
                } else {
                    gb.gemm(ny, J.nout, J.nc, cross(J.y, J.x) + J.c0, nx, 1, B, J.ld, 1, out, J.nout, 1.0);
                }
            } else {             // side 2: rows of x C_Q' b2^T or rows of y (S_yx C_x)_Q' b2^T; B(b, j) = X[(r0 + j) ld + b]
                const double *B = J.X + (long long)J.r0 * J.ld;
                if (J.kind == 2) {
                    gb.gemm(nx, J.nout, J.nc, dC.p + offC[J.x] + J.c0, nx, 1, B, 1, J.ld, out, J.nout, 1.0);
                    gb.gemm(nx, J.nout, J.nc, dSC.p + offC[J.x] + J.c0, nx, 1, B, 1, J.ld, out + (long long)nx * J.nout,
                            J.nout, 1.0);
                } else {
                    gb.gemm(ny, J.nout, J.nc, cross(J.y, J.x) + J.c0, nx, 1, B, 1, J.ld, out, J.nout, 1.0);
                }
            }
        }
        gb.run(*this, sizeof(T) == 4, dJobs, dTiles, TINCR_KF_AO_EXCHANGE);
        // elements grouped by side-2 group (a stable counting sort); one CTA per (group, tile) forms V
        // and serves the group's elements
        std::vector<int> el_begin(k2v.size() + 1, 0);
        for (const ExEl &E : elv) ++el_begin[E.k2 + 1];
        for (size_t k = 0; k < k2v.size(); ++k) el_begin[k + 1] += el_begin[k];
        {
            std::vector<ExEl> sorted(elv.size());
            std::vector<int> fill(el_begin.begin(), el_begin.end() - 1);
            for (const ExEl &E : elv) sorted[fill[E.k2]++] = E;
            elv.swap(sorted);
        }
        std::vector<int4> vt;
        double fl = 0.0;
        for (int k = 0; k < (int)k2v.size(); ++k) {
            const ExS2 &K = k2v[k];
            if (el_begin[k + 1] == el_begin[k]) continue;
            for (int a0 = 0; a0 < K.na; a0 += K.ta)
                for (int j0 = 0; j0 < K.nq; j0 += K.tj) vt.push_back(make_int4(k, a0, j0, 0));
            fl += (2.0 * nat_of(K.x1, K.y1) * nat_of(K.x2, K.y2) +
                   4.0 * nao_of(K.x1, K.y1) * (el_begin[k + 1] - el_begin[k])) * K.na * K.nq;
        }
        DevBuf<ExS1> dk1;
        DevBuf<ExS2> dk2;
        DevBuf<ExEl> del;
        DevBuf<int> deb;
        DevBuf<int4> dvt;
        upload_vec(stream, dk1, k1v);
        upload_vec(stream, dk2, k2v);
        upload_vec(stream, del, elv);
        upload_vec(stream, deb, el_begin);
        upload_vec(stream, dvt, vt);
        static bool attr[2] = {false, false};
        if (!attr[sizeof(T) == 4]) {
            TINCR_CUDA(cudaFuncSetAttribute(ex_vu_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)ExVUSmem<T>::BYTES));
            attr[sizeof(T) == 4] = true;
        }
        const int slot = prof_begin(TINCR_KF_AO_EXCHANGE);
        for (size_t t0 = 0; t0 < vt.size(); t0 += 1u << 20) {   // grid limit
            const unsigned nb = (unsigned)std::min<size_t>(vt.size() - t0, 1u << 20);
            ex_vu_kernel<T><<<nb, XJ_T, ExVUSmem<T>::BYTES, stream>>>(dvt.p + t0, dk2.p, deb.p, del.p, dk1.p, dm.p,
                                                                       dGlr.p, n_atoms_total, d1.p, dH.p, ns);
            count_launch(stream, "ex_vu");
            check_launch("ex_vu");
        }
        sync();   // the host lists above must outlive their uploads
        prof_end(slot, fl, 0.0);
    };
    if (fp32)
        run_exchange(0.0f);
    else
        run_exchange(0.0);

    // ---- LCMO Fock blocks and one-electron LE-CT couplings ----
    // blocks F'_{xy} (x < y) of every CT pair, from the real pairs' dimer orbitals
    std::vector<std::pair<int, int>> ctp;
    for (int c = 0; c < n_ct; ++c) {
        const int x = std::min(cts[c].h, cts[c].l), y = std::max(cts[c].h, cts[c].l);
        if (std::find(ctp.begin(), ctp.end(), std::make_pair(x, y)) == ctp.end()) ctp.emplace_back(x, y);
    }
    std::vector<std::vector<int>> nb(n_mono);   // real-pair neighbours
    for (int p = 0; p < n_pairs; ++p)
        if (pairs[p].real) {
            nb[pairs[p].i].push_back(pairs[p].j);
            nb[pairs[p].j].push_back(pairs[p].i);
        }
    DevBuf<double> dFp;   // F'_{xy} of the CT pairs
    std::map<PairKey, long long> fp_off;
    std::vector<Ex1eJob> e1;
    if (!ctp.empty()) {
        // per real pair: s_pr [ni x nij], s_qr [nj x nij], s_pq [ni x nj]; F blocks: diagonal F_kk,
        // off-diagonal F_ij (i < j) of real pairs
        std::vector<int> rp;
        for (int p = 0; p < n_pairs; ++p)
            if (pairs[p].real) rp.push_back(p);
        std::map<int, long long> o_spr, o_sqr, o_spq, o_fij, o_po, o_pe;
        long long nspr = 0, nspq = 0, nfij = 0, npo = 0, npe = 0;
        for (int p : rp) {
            const int ni = nao[pairs[p].i], nj = nao[pairs[p].j], nij = ni + nj;
            o_spr[p] = nspr; nspr += (long long)ni * nij;
            o_sqr[p] = nspr; nspr += (long long)nj * nij;
            o_spq[p] = nspq; nspq += (long long)ni * nj;
            o_fij[p] = nfij; nfij += (long long)ni * nj;
            o_po[p] = npo; npo += (long long)nij * nij;
            o_pe[p] = npe; npe += nij;
        }
        // dimer orbitals and energies: packed in parallel into the staging buffer, one DMA each
        double *hPo = ex_pin.p + pin_used;
        pin_used += npo;
        double *hPe = ex_pin.p + pin_used;
        pin_used += npe;
        int bad_pair = -1;
#pragma omp parallel for schedule(dynamic, 4) num_threads(8)
        for (int r = 0; r < (int)rp.size(); ++r) {
            const int p = rp[r];
            const size_t nij = (size_t)nao[pairs[p].i] + nao[pairs[p].j];
            const double *po = pairs[p].pair_orbs, *pe = pairs[p].pair_orbe;
            bool ok = true;
            for (size_t x = 0; x < nij * nij; ++x) ok = ok && std::isfinite(po[x]);
            for (size_t x = 0; x < nij; ++x) ok = ok && std::isfinite(pe[x]);
            if (!ok) {
#pragma omp critical
                bad_pair = p;
            }
            std::copy(po, po + nij * nij, hPo + o_po.at(p));
            std::copy(pe, pe + nij, hPe + o_pe.at(p));
        }
        if (bad_pair >= 0) fail(TINCR_NONFINITE, "non-finite value in pair orbitals of pair " + std::to_string(bad_pair));
        DevBuf<double> dPo, dPe, dSpr, dSpq, dFd, dFij;
        dPo.alloc(std::max<long long>(1, npo));
        dPe.alloc(std::max<long long>(1, npe));
        if (npo) TINCR_CUDA(cudaMemcpyAsync(dPo.p, hPo, npo * sizeof(double), cudaMemcpyHostToDevice, stream));
        if (npe) TINCR_CUDA(cudaMemcpyAsync(dPe.p, hPe, npe * sizeof(double), cudaMemcpyHostToDevice, stream));
        dSpr.alloc(std::max<long long>(1, nspr));
        dSpq.alloc(std::max<long long>(1, nspq));
        dFij.alloc(std::max<long long>(1, nfij));
        dFd.alloc(std::max<size_t>(1, hC.size()));   // F_kk, laid out like C
        TINCR_CUDA(cudaMemsetAsync(dSpr.p, 0, dSpr.n * sizeof(double), stream));
        TINCR_CUDA(cudaMemsetAsync(dSpq.p, 0, dSpq.n * sizeof(double), stream));
        TINCR_CUDA(cudaMemsetAsync(dFij.p, 0, dFij.n * sizeof(double), stream));
        // F_kk starts at (1 - real pairs of k) diag(e_k): every pair adds f_aa - diag(e_k)
        {
            std::vector<double> hFd(hC.size(), 0.0);
            std::vector<int> npk(n_mono, 0);
            for (int p : rp) {
                ++npk[pairs[p].i];
                ++npk[pairs[p].j];
            }
            for (int k = 0; k < n_mono; ++k)
                for (int a = 0; a < nao[k]; ++a)
                    hFd[offC[k] + (long long)a * nao[k] + a] = (1.0 - npk[k]) * mono[k].orbe[a];
            TINCR_CUDA(cudaMemcpyAsync(dFd.p, hFd.data(), hFd.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
            sync();
        }
        // stage 1: s_pr = (S_ii C_i)^T C_ij[0:ni] + (S_ji C_i)^T C_ij[ni:], s_qr = (S_ij C_j)^T C_ij[0:ni] +
        // (S_jj C_j)^T C_ij[ni:], s_pq = C_i^T (S_ij C_j)  (hamiltonian.rs:61-70)
        for (int p : rp) {
            const int i = pairs[p].i, j = pairs[p].j, ni = nao[i], nj = nao[j], nij = ni + nj;
            const double *po = dPo.p + o_po[p];
            gb.gemm(ni, nij, ni, dSC.p + offC[i], 1, ni, po, nij, 1, dSpr.p + o_spr[p], nij, 1.0);
            gb.gemm(ni, nij, nj, cross(j, i), 1, ni, po + (long long)ni * nij, nij, 1, dSpr.p + o_spr[p], nij, 1.0);
            gb.gemm(nj, nij, ni, cross(i, j), 1, nj, po, nij, 1, dSpr.p + o_sqr[p], nij, 1.0);
            gb.gemm(nj, nij, nj, dSC.p + offC[j], 1, nj, po + (long long)ni * nij, nij, 1, dSpr.p + o_sqr[p], nij, 1.0);
            gb.gemm(ni, nj, ni, dC.p + offC[i], 1, ni, cross(i, j), nj, 1, dSpq.p + o_spq[p], nj, 1.0);
        }
        gb.run(*this, fp32, dJobs, dTiles, TINCR_KF_OTHER);
        // stage 2: F_ii += s_pr diag(e) s_pr^T, F_jj += s_qr diag(e) s_qr^T, F_ij = s_pr diag(e) s_qr^T
        for (int p : rp) {
            const int i = pairs[p].i, j = pairs[p].j, ni = nao[i], nj = nao[j], nij = ni + nj;
            const double *spr = dSpr.p + o_spr[p], *sqr = dSpr.p + o_sqr[p], *e = dPe.p + o_pe[p];
            gb.gemm(ni, ni, nij, spr, nij, 1, spr, 1, nij, dFd.p + offC[i], ni, 1.0, e);
            gb.gemm(nj, nj, nij, sqr, nij, 1, sqr, 1, nij, dFd.p + offC[j], nj, 1.0, e);
            gb.gemm(ni, nj, nij, spr, nij, 1, sqr, 1, nij, dFij.p + o_fij[p], nj, 1.0, e);
        }
        gb.run(*this, fp32, dJobs, dTiles, TINCR_KF_OTHER);
        // block accessors of F and of S_off (the MO overlaps between monomers of real pairs)
        struct Blk {
            const double *p;
            long long sr, sc;   // element (r, c) at p[r * sr + c * sc]
        };
        auto Fb = [&](int k, int m) -> Blk {
            if (k == m) return Blk{dFd.p + offC[k], nao[k], 1};
            auto it = pidx.find(PairKey{std::min(k, m), std::max(k, m)});
            const int p = it->second;
            const double *b = dFij.p + o_fij[p];
            if (k < m) return Blk{b, nao[m], 1};
            return Blk{b, 1, nao[k]};
        };
        auto Sb = [&](int k, int m) -> Blk {   // S_total block (k, m), k != m real pair
            auto it = pidx.find(PairKey{std::min(k, m), std::max(k, m)});
            const int p = it->second;
            const double *b = dSpq.p + o_spq[p];
            if (k < m) return Blk{b, nao[m], 1};
            return Blk{b, 1, nao[k]};
        };
        // stage 3: FX_{k, y} = F_ky - 1/2 sum_{m real neighbour of y, F_km != 0} F_km S_my for k in {x} + nb(x)
        std::map<PairKey, long long> fx_off;
        long long nfx = 0;
        for (auto &xy : ctp) {
            std::vector<int> ks = {xy.first};
            ks.insert(ks.end(), nb[xy.first].begin(), nb[xy.first].end());
            for (int k : ks)
                if (!fx_off.count(PairKey{k, xy.second})) {
                    fx_off[PairKey{k, xy.second}] = nfx;
                    nfx += (long long)nao[k] * nao[xy.second];
                }
        }
        DevBuf<double> dFX;
        dFX.alloc(std::max<long long>(1, nfx));
        TINCR_CUDA(cudaMemsetAsync(dFX.p, 0, dFX.n * sizeof(double), stream));
        for (auto &kv : fx_off) {
            const int k = kv.first.i, y = kv.first.j;
            double *out = dFX.p + kv.second;
            const int nk = nao[k], ny = nao[y];
            if (k == y || is_real(k, y)) {
                const Blk f = Fb(k, y);
                gb.add(nk, ny, f.p, f.sr, f.sc, out, ny, 1.0);
            }
            for (int m : nb[y]) {
                if (!(m == k || is_real(k, m))) continue;
                const Blk f = Fb(k, m), s = Sb(m, y);
                gb.gemm(nk, ny, nao[m], f.p, f.sr, f.sc, s.p, s.sr, s.sc, out, ny, -0.5);
            }
        }
        gb.run(*this, fp32, dJobs, dTiles, TINCR_KF_OTHER);
        // stage 4: F'_{xy} = FX_{xy} - 1/2 sum_{k real neighbour of x} S_kx^T FX_{ky}
        long long nfp = 0;
        for (auto &xy : ctp) {
            fp_off[PairKey{xy.first, xy.second}] = nfp;
            nfp += (long long)nao[xy.first] * nao[xy.second];
        }
        dFp.alloc(std::max<long long>(1, nfp));
        TINCR_CUDA(cudaMemsetAsync(dFp.p, 0, dFp.n * sizeof(double), stream));
        for (auto &xy : ctp) {
            const int x = xy.first, y = xy.second, nx = nao[x], ny = nao[y];
            double *out = dFp.p + fp_off[PairKey{x, y}];
            gb.add(nx, ny, dFX.p + fx_off[PairKey{x, y}], ny, 1, out, ny, 1.0);
            for (int k : nb[x]) {
                const Blk s = Sb(k, x);   // (k, x) block; S_kx^T element (r, c) = s(c, r)
                gb.gemm(nx, ny, nao[k], s.p, s.sc, s.sr, dFX.p + fx_off[PairKey{k, y}], ny, 1, out, ny, -0.5);
            }
        }
        gb.run(*this, fp32, dJobs, dTiles, TINCR_KF_OTHER);
        // one-electron jobs: every LE state on the hole or the electron monomer of a CT state
        for (int t = 0; t < ns; ++t) {
            if (hst[t].kind != 1) continue;
            const int h = hst[t].hole, l = hst[t].elec;
            const int x = std::min(h, l), y = std::max(h, l);
            const double *F = dFp.p + fp_off[PairKey{x, y}];
            for (int s = 0; s < ns; ++s) {
                if (hst[s].kind != 0 || (hst[s].hole != h && hst[s].hole != l)) continue;
                const int I = hst[s].hole;
                Ex1eJob J;
                J.s = std::min(s, t);
                J.t = std::max(s, t);
                J.Xl = dX.p + xoff[s];
                J.Xc = dX.p + xoff[t];
                J.ol = no[I]; J.vl = nao[I] - no[I]; J.oc = no[h]; J.vc = nao[l] - no[l];
                J.F = F;
                // F'[row in I's MOs, column in the other monomer's MOs]: stored block (x, y), n_x x n_y
                if (I == x) { J.fp = nao[y]; J.fq = 1; } else { J.fp = 1; J.fq = nao[y]; }
                if (I == l) {   // occupied blocks
                    J.on_elec = 1;
                    J.r0 = 0;
                    J.c0 = 0;
                } else {        // virtual blocks
                    J.on_elec = 0;
                    J.r0 = no[I];
                    J.c0 = no[l];
                }
                e1.push_back(J);
            }
        }
    }
    if (!e1.empty()) {
        DevBuf<Ex1eJob> de1;
        upload_vec(stream, de1, e1);
        ex_1e_kernel<<<(unsigned)e1.size(), 256, 0, stream>>>(de1.p, dH.p, ns);
        count_launch(stream, "ex_1e");
        check_launch("ex_1e");
        sync();
    }
    ex_symmetrize_kernel<<<ceil_div((long long)ns * ns, 256), 256, 0, stream>>>(ns, dH.p);
    count_launch(stream, "ex_symmetrize");
    check_launch("ex_symmetrize");
    if (h_out) TINCR_CUDA(cudaMemcpyAsync(h_out, dH.p, (size_t)ns * ns * sizeof(double), cudaMemcpyDeviceToHost, stream));
    sync();

    // ---- lowest roots: tincr's Davidson on the dense matrix (basis.rs:497-503) ----
    const int nr = n_roots, max_space = 15 * nr;
    std::vector<double> hdiag(ns);
    DevBuf<double> dd;
    dd.alloc(ns);
    ex_diag_kernel<<<ceil_div(ns, 256), 256, 0, stream>>>(ns, dH.p, dd.p);
    count_launch(stream, "ex_diag");
    TINCR_CUDA(cudaMemcpyAsync(hdiag.data(), dd.p, ns * sizeof(double), cudaMemcpyDeviceToHost, stream));
    sync();
    std::vector<int> order(ns);
    for (int x = 0; x < ns; ++x) order[x] = x;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return hdiag[a] < hdiag[b]; });
    const int cap = max_space + nr;
    DevBuf<double> dV, dAV, dAp, dY, dRitz, dRk, dU, dNrm, dT, dc, dPart, dPart2, dRp;
    dPart.alloc(ceil_div(ns, 256));
    // the long sums split over CTAs in chunks of at least 64 terms (at most 16 chunks); the chunk
    // count depends on the sum's length only, so a row's value does not depend on its launch
    const int xb = ceil_div(ns, 256);
    auto chunks = [](int K) { return std::max(1, std::min(16, K / 64)); };
    const int S_orth = chunks(cap);
    dPart2.alloc((size_t)S_orth * ns);
    auto rowprod = [&](int rows, int K, const double *A, const double *B, double *out) {
        const int S = chunks(K);
        dRp.reserve((size_t)S * rows * ns);
        ex_rowprod_part_kernel<<<dim3(xb, rows, S), 256, 0, stream>>>(ns, K, A, B, dRp.p);
        count_launch(stream, "ex_rowprod_part");
        ex_rowprod_sum_kernel<<<ceil_div((long long)rows * ns, 256), 256, 0, stream>>>((long long)rows * ns, S, dRp.p,
                                                                                     out);
        count_launch(stream, "ex_rowprod_sum");
        check_launch("ex_rowprod");
    };
    DevBuf<int> dM;   // the basis size while corrections join it
    dM.alloc(1);
    int *hM = reinterpret_cast<int *>(ex_pin.p + pin_used);   // one int of the page-locked staging buffer
    dV.alloc((size_t)cap * ns);
    dAV.alloc((size_t)cap * ns);
    dAp.alloc((size_t)cap * cap);
    dY.alloc((size_t)nr * cap);
    dRitz.alloc((size_t)nr * ns);
    dRk.alloc((size_t)nr * ns);
    dU.alloc(nr);
    dNrm.alloc(std::max(nr, 1) + 1);
    dT.alloc(ns);
    dc.alloc(cap);
    {
        std::vector<double> g((size_t)nr * ns, 0.0);   // initial_subspace (solvers/utils.rs:17-26)
        for (int r = 0; r < nr; ++r) g[(size_t)r * ns + order[r]] = 1.0;
        TINCR_CUDA(cudaMemcpyAsync(dV.p, g.data(), g.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
        sync();
    }
    int m = nr, dim_sub = nr, it = 0, status = TINCR_NOT_CONVERGED;
    int n_av = 0;   // rows of AV that hold H v_i for the current basis
    std::vector<double> ap, w(nr), yt, err(nr), u(nr);
    for (it = 0; it < max_iter; ++it) {
        // products of the subspace vectors and the projection.  tincr's dense engine multiplies every
        // vector again (solvers/mod.rs:36-51); the rows of earlier vectors are unchanged (each row of the
        // product is formed on its own, in the same order), so only the new vectors are multiplied
        const int sub_slot = prof_begin(TINCR_KF_SUBSPACE);
        if (n_av < m) {   // (H is symmetric: row i of V H is H v_i)
            rowprod(m - n_av, ns, dV.p + (size_t)n_av * ns, dH.p, dAV.p + (size_t)n_av * ns);
            n_av = m;
        }
        ex_dotmat_kernel<<<ceil_div((long long)m * m * 32, 256), 256, 0, stream>>>(m, m, ns, dV.p, dAV.p, dAp.p);
        count_launch(stream, "ex_dotmat");
        check_launch("ex_dotmat");
        prof_end(sub_slot, 2.0 * m * (double)m * ns, 0.0);
        ap.resize((size_t)m * m);
        TINCR_CUDA(cudaMemcpyAsync(ap.data(), dAp.p, ap.size() * sizeof(double), cudaMemcpyDeviceToHost, stream));
        sync();
        yt.assign((size_t)nr * m, 0.0);
        if (!eigh_lowest_upper(m, ap.data(), nr, w.data(), yt.data()))
            fail(TINCR_NONFINITE, "exciton_states: subspace eigensolver failed");
        for (int r = 0; r < nr; ++r) u[r] = w[r];
        TINCR_CUDA(cudaMemcpyAsync(dY.p, yt.data(), yt.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
        TINCR_CUDA(cudaMemcpyAsync(dU.p, u.data(), nr * sizeof(double), cudaMemcpyHostToDevice, stream));
        rowprod(nr, m, dY.p, dV.p, dRitz.p);
        rowprod(nr, m, dY.p, dAV.p, dRk.p);
        ex_residual_kernel<<<ceil_div((long long)nr * ns, 256), 256, 0, stream>>>(nr, ns, dU.p, dRitz.p, dRk.p);
        count_launch(stream, "ex_residual");
        ex_row_norms_kernel<<<nr, 256, 0, stream>>>(nr, ns, dRk.p, dNrm.p);
        count_launch(stream, "ex_row_norms");
        TINCR_CUDA(cudaMemcpyAsync(err.data(), dNrm.p, nr * sizeof(double), cudaMemcpyDeviceToHost, stream));
        sync();
        int cvd = 0;
        for (int r = 0; r < nr; ++r) {
            if (!std::isfinite(err[r])) fail(TINCR_NONFINITE, "exciton_states: non-finite residual");
            if (err[r] < tol) ++cvd;
        }
        const int lft = nr - cvd;
        if (lft == 0 && it > 0) {
            status = TINCR_OK;
            ++it;
            break;
        }
        if (dim_sub + lft <= max_space) {
            dim_sub += lft;
            // the corrections in order, each orthogonalised against the basis so far (which grows on
            // the device, so no host round trip separates them); the basis size comes back once
            ex_set_int_kernel<<<1, 32, 0, stream>>>(dM.p, m);
            count_launch(stream, "ex_set_int");
            const int m_max = std::min(cap, m + lft);
            for (int r = 0; r < nr; ++r) {
                if (!(err[r] > tol)) continue;
                ex_precondition_kernel<<<ceil_div(ns, 256), 256, 0, stream>>>(ns, dRk.p + (size_t)r * ns, u[r], dH.p,
                                                                             dT.p);
                count_launch(stream, "ex_precondition");
                ex_dots_dev_kernel<<<m_max, 256, 0, stream>>>(dM.p, ns, dV.p, dT.p, dc.p);
                count_launch(stream, "ex_dots");
                ex_orth_part_kernel<<<dim3(xb, S_orth), 256, 0, stream>>>(dM.p, ns, dV.p, dc.p, dPart2.p);
                count_launch(stream, "ex_orth_part");
                ex_orth_finish_kernel<<<xb, 256, 0, stream>>>(ns, S_orth, dPart2.p, dT.p, dPart.p);
                count_launch(stream, "ex_orth_finish");
                ex_norm_finish_kernel<<<1, 32, 0, stream>>>(ceil_div(ns, 256), dPart.p, dNrm.p + nr);
                count_launch(stream, "ex_norm_finish");
                ex_append_kernel<<<ceil_div(ns, 256), 256, 0, stream>>>(ns, dNrm.p + nr, dM.p, cap, dT.p, dV.p);
                count_launch(stream, "ex_append");
                ex_count_kernel<<<1, 32, 0, stream>>>(dNrm.p + nr, dM.p, cap);
                count_launch(stream, "ex_count");
            }
            check_launch("ex_append");
            TINCR_CUDA(cudaMemcpyAsync(hM, dM.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
            sync();
            m = *hM;
        } else {
            dim_sub = nr;
            TINCR_CUDA(cudaMemcpyAsync(dV.p, dRitz.p, (size_t)nr * ns * sizeof(double), cudaMemcpyDeviceToDevice, stream));
            m = nr;
            n_av = 0;
        }
    }
    for (int r = 0; r < nr; ++r) energies[r] = u[r];
    if (vectors) {
        std::vector<double> rv((size_t)nr * ns);
        TINCR_CUDA(cudaMemcpyAsync(rv.data(), dRitz.p, rv.size() * sizeof(double), cudaMemcpyDeviceToHost, stream));
        sync();
        for (int x = 0; x < ns; ++x)
            for (int r = 0; r < nr; ++r) vectors[(size_t)x * nr + r] = rv[(size_t)r * ns + x];
    }
    if (iterations) *iterations = it;
    TINCR_CUDA(cudaEventRecord(ev1, stream));
    sync();
    float ms = 0.f;
    TINCR_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    last_ms = ms;
    last_launches = g_launches;
    prof_resolve();
    return status;
}

}  // namespace tincr
