// FMO exciton Hamiltonian in the diabatic LE / CT basis and its lowest states (tincr_exciton_states).
//
// tincr builds the matrix element by element on rayon threads (SuperSystem::
// create_exciton_hamiltonian_new, src/fmo/lcmo/basis.rs:449-503; couplings in
// src/fmo/lcmo/integrals.rs), rebuilding the Mulliken transition charges between the orbitals of
// two monomers for every element.  Here the matrix is assembled on the GPU in a few grouped passes:
//   * Coulomb: W = gamma Q over all atoms, then 2 q_s . W_t for every element (block-sparse Q: each
//     state's charges live on one or two monomers);
//   * exchange: one CTA per (element, tile of the (a, j) index pairs).  The charges are never
//     stored: with Mulliken charges q^A_pq = 1/2 sum_{mu in A} (C_mu p (S C)_mu q + (S C)_mu p C_mu q)
//     over the AOs of the one or two monomers involved, sum_i q^A_ij b_ia is a sum over mu in A of
//     two outer products of per-AO rows, so each job forms four small [AO x tile] arrays from C, S C
//     (per monomer) and S_xy C_y (per pair), then
//       exchange = sum_{A, B} gamma_lr[A, B] sum_{a, j} U^A_aj W^B_aj;
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

constexpr int XG_T = 256, XG_TILE = 32;

template <class T>
__global__ void __launch_bounds__(XG_T) ex_gemm_kernel(const GemmJob *__restrict__ jobs, const int4 *__restrict__ tiles) {
    __shared__ T As[XG_TILE][XG_TILE + 1], Bs[XG_TILE][XG_TILE + 1];
    const int4 tl = tiles[blockIdx.x];
    const GemmJob J = jobs[tl.x];
    const int m0 = tl.y * XG_TILE, n0 = tl.z * XG_TILE;
    const int tr = threadIdx.x & 31, tc = (threadIdx.x >> 5) * 4;
    if (!J.B) {   // elementwise add
        for (int q = 0; q < 4; ++q) {
            const int m = m0 + tr, n = n0 + tc + q;
            if (m < J.M && n < J.N) atomicAdd(J.C + m * J.ldc + n, J.alpha * J.A[m * J.sam + n * J.sak]);
        }
        return;
    }
    T acc[4] = {T(0), T(0), T(0), T(0)};
    for (int k0 = 0; k0 < J.K; k0 += XG_TILE) {
        for (int e = threadIdx.x; e < XG_TILE * XG_TILE; e += XG_T) {
            const int mm = e >> 5, kk = e & 31;
            const int m = m0 + mm, k = k0 + kk;
            T v = T(0);
            if (m < J.M && k < J.K) {
                double x = J.A[m * J.sam + k * J.sak];
                if (J.d) x *= J.d[k];
                v = (T)x;
            }
            As[mm][kk] = v;
            const int kb = e >> 5, nn = e & 31;
            const int k2 = k0 + kb, n = n0 + nn;
            Bs[kb][nn] = (k2 < J.K && n < J.N) ? (T)J.B[k2 * J.sbk + n * J.sbn] : T(0);
        }
        __syncthreads();
#pragma unroll 8
        for (int kk = 0; kk < XG_TILE; ++kk) {
            const T a = As[tr][kk];
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[q] += a * Bs[kk][tc + q];
        }
        __syncthreads();
    }
    for (int q = 0; q < 4; ++q) {
        const int m = m0 + tr, n = n0 + tc + q;
        if (m < J.M && n < J.N) atomicAdd(J.C + m * J.ldc + n, J.alpha * (double)acc[q]);
    }
}

struct GemmBatch {
    std::vector<GemmJob> jobs;
    std::vector<int4> tiles;
    void gemm(int M, int N, int K, const double *A, long long sam, long long sak, const double *B, long long sbk,
              long long sbn, double *C, long long ldc, double alpha, const double *d = nullptr) {
        if (M <= 0 || N <= 0 || K <= 0) return;
        const int j = (int)jobs.size();
        jobs.push_back(GemmJob{A, B, d, C, sam, sak, sbk, sbn, ldc, M, N, K, alpha});
        for (int tm = 0; tm < ceil_div(M, XG_TILE); ++tm)
            for (int tn = 0; tn < ceil_div(N, XG_TILE); ++tn) tiles.push_back(make_int4(j, tm, tn, 0));
    }
    // C[m, n] += alpha A(m, n)
    void add(int M, int N, const double *A, long long sam, long long san, double *C, long long ldc, double alpha) {
        if (M <= 0 || N <= 0) return;
        const int j = (int)jobs.size();
        jobs.push_back(GemmJob{A, nullptr, nullptr, C, sam, san, 0, 0, ldc, M, N, 1, alpha});
        for (int tm = 0; tm < ceil_div(M, XG_TILE); ++tm)
            for (int tn = 0; tn < ceil_div(N, XG_TILE); ++tn) tiles.push_back(make_int4(j, tm, tn, 0));
    }
    void run(Ctx &c, bool fp32, DevBuf<GemmJob> &dj, DevBuf<int4> &dt, int family) {
        if (tiles.empty()) return;
        dj.reserve(jobs.size());
        dt.reserve(tiles.size());
        TINCR_CUDA(cudaMemcpyAsync(dj.p, jobs.data(), jobs.size() * sizeof(GemmJob), cudaMemcpyHostToDevice, c.stream));
        TINCR_CUDA(cudaMemcpyAsync(dt.p, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice, c.stream));
        double flops = 0.0;
        for (const GemmJob &j : jobs) flops += j.B ? 2.0 * j.M * j.N * j.K : (double)j.M * j.N;
        const int slot = c.prof_begin(family);
        if (fp32)
            ex_gemm_kernel<float><<<(unsigned)tiles.size(), XG_T, 0, c.stream>>>(dj.p, dt.p);
        else
            ex_gemm_kernel<double><<<(unsigned)tiles.size(), XG_T, 0, c.stream>>>(dj.p, dt.p);
        count_launch(c.stream, "ex_gemm");
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
// exchange jobs
// ----------------------------------------------------------------------------------------------

// Per-monomer device views: C and S C ([n x n], row-major, columns = MOs), atom range, AO offsets.
struct ExMono {
    const double *C, *SC;
    const int *ao_off;   // [n_atoms + 1], local
    int n, n_atoms, atom0;
};

// One exchange tile: element (s, t); side 1 holds the charges between the occupied columns P of
// monomer x1 and Q of y1, side 2 between the virtual columns P' of x2 and Q' of y2.
//   b1(i, a) = X1[(i1 + i) * ld1 + a1 + a]  (state s: i over P, a over P')
//   b2(j, b) = X2[(j2 + j) * ld2 + b2 + b]  (state t: j over Q, b over Q')
// The tile covers a in [ta0, ta0 + ta), j in [tj0, tj0 + tj), ta * tj <= XJ_T.
struct ExJob {
    int s, t;
    int x1, y1, x2, y2;
    int p0, np, q0, pa0, qb0, nb;
    int ta0, ta, tj0, tj;
    const double *X1, *X2;
    int ld1, i1, a1, ld2, j2, b2;
    const double *cross_xy1, *cross_yx1;   // S_x1y1 C_y1 [n_x1 x n_y1], S_y1x1 C_x1 [n_y1 x n_x1] (x1 != y1)
    const double *cross_xy2, *cross_yx2;   // the same for x2, y2
};

constexpr int XJ_T = 128;          // threads = the largest (a, j) tile
constexpr int XJ_TMAX = 16;        // largest tile side
constexpr int XJ_AO = 2 * 102 + 4; // AOs of two monomers (largest supported monomer: 102 AOs)
constexpr int XJ_ATOMS = 80;       // atoms of two monomers

template <class T>
struct XjSmem {
    T L1[XJ_AO][XJ_TMAX], L2[XJ_AO][XJ_TMAX];   // Lc, Ls (side 1) or L'c, L's (side 2)
    T R1[XJ_AO][XJ_TMAX], R2[XJ_AO][XJ_TMAX];   // Rc, Rs (side 1) or R'c, R's (side 2)
    T V[XJ_ATOMS][XJ_T];                        // V^A = sum_B gamma_lr[A, B] W^B per (a, j)
    T red[XJ_T / 32];
};

// AO row mu of the fragment {x, y} (x's AOs first; y only when y != x): monomer and local row
__device__ __forceinline__ void frag_row(const ExMono &mx, const ExMono &my, bool two, int mu, int &which, int &row) {
    if (!two || mu < mx.n) {
        which = 0;
        row = mu;
    } else {
        which = 1;
        row = mu - mx.n;
    }
}

template <class T>
__global__ void __launch_bounds__(XJ_T) ex_exchange_kernel(const ExJob *__restrict__ jobs, const ExMono *__restrict__ mono,
                                                           const double *__restrict__ gamma_lr, int n_atoms_total,
                                                           double *H, int n_states) {
    extern __shared__ __align__(16) unsigned char xj_raw[];
    XjSmem<T> &sm = *reinterpret_cast<XjSmem<T> *>(xj_raw);
    const ExJob J = jobs[blockIdx.x];
    const int tid = threadIdx.x;
    const int ntile = J.ta * J.tj;
    const int my_a = tid / J.tj, my_j = tid % J.tj;
    const bool active = tid < ntile;

    // ---- side 2 (virtual charges): L'c = P', L's = S P', R'c = Q' b2^T, R's = (S Q') b2^T ----
    const ExMono m2x = mono[J.x2], m2y = mono[J.y2];
    const bool two2 = J.x2 != J.y2;
    const int nao2 = m2x.n + (two2 ? m2y.n : 0);
    for (int e = tid; e < nao2 * J.ta; e += XJ_T) {
        const int mu = e / J.ta, a = e % J.ta;
        int w, r;
        frag_row(m2x, m2y, two2, mu, w, r);
        const int col = J.pa0 + J.ta0 + a;
        T lc = T(0), ls = T(0);
        if (w == 0) {
            lc = (T)m2x.C[(long long)r * m2x.n + col];
            ls = (T)m2x.SC[(long long)r * m2x.n + col];
        } else {
            ls = (T)J.cross_yx2[(long long)r * m2x.n + col];
        }
        sm.L1[mu][a] = lc;
        sm.L2[mu][a] = ls;
    }
    for (int e = tid; e < nao2 * J.tj; e += XJ_T) {
        const int mu = e / J.tj, jj = e % J.tj;
        int w, r;
        frag_row(m2x, m2y, two2, mu, w, r);
        const double *brow = J.X2 + (long long)(J.j2 + J.tj0 + jj) * J.ld2 + J.b2;
        T rc = T(0), rs = T(0);
        for (int b = 0; b < J.nb; ++b) {
            const int col = J.qb0 + b;
            const T bb = (T)brow[b];
            if (two2) {
                if (w == 1) {
                    rc += (T)m2y.C[(long long)r * m2y.n + col] * bb;
                    rs += (T)m2y.SC[(long long)r * m2y.n + col] * bb;
                } else {
                    rs += (T)J.cross_xy2[(long long)r * m2y.n + col] * bb;
                }
            } else {
                rc += (T)m2x.C[(long long)r * m2x.n + col] * bb;
                rs += (T)m2x.SC[(long long)r * m2x.n + col] * bb;
            }
        }
        sm.R1[mu][jj] = rc;
        sm.R2[mu][jj] = rs;
    }
    // atoms of side 1 (for V's rows)
    const ExMono m1x = mono[J.x1], m1y = mono[J.y1];
    const bool two1 = J.x1 != J.y1;
    const int nat1 = m1x.n_atoms + (two1 ? m1y.n_atoms : 0);
    const int nat2 = m2x.n_atoms + (two2 ? m2y.n_atoms : 0);
    __syncthreads();
    // V^A = sum_B gamma_lr[A, B] W^B, W^B_aj = 1/2 sum_{nu in B} (L'c R's + L's R'c)
    if (active) {
        for (int A = 0; A < nat1; ++A) sm.V[A][tid] = T(0);
        for (int B = 0; B < nat2; ++B) {
            const ExMono &mb = (B < m2x.n_atoms) ? m2x : m2y;
            const int bl = (B < m2x.n_atoms) ? B : B - m2x.n_atoms;
            const int base = (B < m2x.n_atoms) ? 0 : m2x.n;
            T wv = T(0);
            for (int nu = mb.ao_off[bl]; nu < mb.ao_off[bl + 1]; ++nu)
                wv += sm.L1[base + nu][my_a] * sm.R2[base + nu][my_j] + sm.L2[base + nu][my_a] * sm.R1[base + nu][my_j];
            wv *= T(0.5);
            const int gB = mb.atom0 + bl;
            for (int A = 0; A < nat1; ++A) {
                const int gA = (A < m1x.n_atoms) ? m1x.atom0 + A : m1y.atom0 + (A - m1x.n_atoms);
                sm.V[A][tid] += (T)gamma_lr[(long long)gA * n_atoms_total + gB] * wv;
            }
        }
    }
    __syncthreads();
    // ---- side 1 (occupied charges): Lc = P b1, Ls = (S P) b1, Rc = Q, Rs = S Q ----
    const int nao1 = m1x.n + (two1 ? m1y.n : 0);
    for (int e = tid; e < nao1 * J.ta; e += XJ_T) {
        const int mu = e / J.ta, a = e % J.ta;
        int w, r;
        frag_row(m1x, m1y, two1, mu, w, r);
        T lc = T(0), ls = T(0);
        for (int i = 0; i < J.np; ++i) {
            const int col = J.p0 + i;
            const T bb = (T)J.X1[(long long)(J.i1 + i) * J.ld1 + J.a1 + J.ta0 + a];
            if (w == 0) {
                lc += (T)m1x.C[(long long)r * m1x.n + col] * bb;
                ls += (T)m1x.SC[(long long)r * m1x.n + col] * bb;
            } else {
                ls += (T)J.cross_yx1[(long long)r * m1x.n + col] * bb;
            }
        }
        sm.L1[mu][a] = lc;
        sm.L2[mu][a] = ls;
    }
    for (int e = tid; e < nao1 * J.tj; e += XJ_T) {
        const int mu = e / J.tj, jj = e % J.tj;
        int w, r;
        frag_row(m1x, m1y, two1, mu, w, r);
        const int col = J.q0 + J.tj0 + jj;
        T rc = T(0), rs = T(0);
        if (two1) {
            if (w == 1) {
                rc = (T)m1y.C[(long long)r * m1y.n + col];
                rs = (T)m1y.SC[(long long)r * m1y.n + col];
            } else {
                rs = (T)J.cross_xy1[(long long)r * m1y.n + col];
            }
        } else {
            rc = (T)m1x.C[(long long)r * m1x.n + col];
            rs = (T)m1x.SC[(long long)r * m1x.n + col];
        }
        sm.R1[mu][jj] = rc;
        sm.R2[mu][jj] = rs;
    }
    __syncthreads();
    T acc = T(0);
    if (active) {
        for (int A = 0; A < nat1; ++A) {
            const ExMono &ma = (A < m1x.n_atoms) ? m1x : m1y;
            const int al = (A < m1x.n_atoms) ? A : A - m1x.n_atoms;
            const int base = (A < m1x.n_atoms) ? 0 : m1x.n;
            T u = T(0);
            for (int mu = ma.ao_off[al]; mu < ma.ao_off[al + 1]; ++mu)
                u += sm.L1[base + mu][my_a] * sm.R2[base + mu][my_j] + sm.L2[base + mu][my_a] * sm.R1[base + mu][my_j];
            acc += T(0.5) * u * sm.V[A][tid];
        }
    }
    for (int off = 16; off; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if ((tid & 31) == 0) sm.red[tid >> 5] = acc;
    __syncthreads();
    if (tid == 0) {
        double tot = 0.0;
        for (int w = 0; w < XJ_T / 32; ++w) tot += (double)sm.red[w];
        atomicAdd(H + (long long)J.s * n_states + J.t, -tot);
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

// v -= c^T V (c: m coefficients), then the norm into *nrm (one CTA)
__global__ void ex_orth_update_kernel(int m, int n, const double *__restrict__ V, const double *__restrict__ c,
                                      double *v, double *nrm) {
    __shared__ double red[8];
    double s = 0.0;
    for (int x = threadIdx.x; x < n; x += blockDim.x) {
        double y = v[x];
        for (int i = 0; i < m; ++i) y -= c[i] * V[(long long)i * n + x];
        v[x] = y;
        s += y * y;
    }
    for (int off = 16; off; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        *nrm = sqrt(t);
    }
}

// c[i] = V_i . v (one CTA per i)
__global__ void ex_dots_kernel(int m, int n, const double *__restrict__ V, const double *__restrict__ v, double *c) {
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

__global__ void ex_scale_kernel(int n, double f, const double *__restrict__ in, double *out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x < n) out[x] = in[x] * f;
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
    check_finite(gamma, (size_t)n_atoms_total * n_atoms_total, "gamma");
    check_finite(gamma_lr, (size_t)n_atoms_total * n_atoms_total, "gamma_lr");

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
    dG.alloc((size_t)n_atoms_total * n_atoms_total);
    dGlr.alloc((size_t)n_atoms_total * n_atoms_total);
    TINCR_CUDA(cudaMemcpyAsync(dG.p, gamma, dG.n * sizeof(double), cudaMemcpyHostToDevice, stream));
    TINCR_CUDA(cudaMemcpyAsync(dGlr.p, gamma_lr, dGlr.n * sizeof(double), cudaMemcpyHostToDevice, stream));

    // pairs: type, S_xy, dimer SCC
    std::map<PairKey, int> pidx;
    for (int p = 0; p < n_pairs; ++p) {
        const tincr_exciton_pair &q = pairs[p];
        if (q.i < 0 || q.j <= q.i || q.j >= n_mono || !q.s_ij) fail(TINCR_BAD_ARG, "exciton_states: bad pair");
        if (q.real && (!q.pair_orbs || !q.pair_orbe)) fail(TINCR_BAD_ARG, "exciton_states: real pair without its SCC");
        pidx[PairKey{q.i, q.j}] = p;
    }
    auto is_real = [&](int a, int b) {
        if (a == b) return false;
        auto it = pidx.find(PairKey{std::min(a, b), std::max(a, b)});
        return it != pidx.end() && pairs[it->second].real != 0;
    };
    // cross products S_xy C_y (n_x x n_y) and S_yx C_x (n_y x n_x) of every listed pair
    std::vector<long long> offX(n_pairs + 1, 0);
    for (int p = 0; p < n_pairs; ++p) offX[p + 1] = offX[p] + 2LL * nao[pairs[p].i] * nao[pairs[p].j];
    std::vector<double> hSxy(offX[n_pairs] / 2 + 1);
    std::vector<long long> offSxy(n_pairs + 1, 0);
    for (int p = 0; p < n_pairs; ++p) {
        const long long sz = (long long)nao[pairs[p].i] * nao[pairs[p].j];
        offSxy[p + 1] = offSxy[p] + sz;
        check_finite(pairs[p].s_ij, (size_t)sz, "pair overlap");
        std::copy(pairs[p].s_ij, pairs[p].s_ij + sz, hSxy.begin() + offSxy[p]);
    }
    DevBuf<double> dSxy, dCross;
    upload_vec(stream, dSxy, hSxy);
    dCross.alloc(std::max<long long>(1, offX[n_pairs]));
    TINCR_CUDA(cudaMemsetAsync(dCross.p, 0, dCross.n * sizeof(double), stream));
    auto cross = [&](int x, int y) -> const double * {   // S_xy C_y, [n_x x n_y]
        auto it = pidx.find(PairKey{std::min(x, y), std::max(x, y)});
        if (it == pidx.end()) return nullptr;
        const int p = it->second;
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

    // states in the basis order: LE (monomer-major), then the CT states as given
    std::vector<ExState> hst;
    std::vector<double> hq, hX;
    std::vector<long long> xoff;
    for (int k = 0; k < n_mono; ++k) {
        const tincr_exciton_monomer &m = mono[k];
        const int o = m.n_occ, v = m.n_orb - m.n_occ;
        for (int r = 0; r < m.n_le; ++r) {
            ExState s{0, k, k, atom0[k], m.n_atoms, 0, 0, (long long)hq.size(), m.le_energies[r]};
            for (int a = 0; a < m.n_atoms; ++a) hq.push_back(m.le_q_trans[(size_t)a * m.n_le + r]);
            xoff.push_back((long long)hX.size());
            for (long long x = 0; x < (long long)o * v; ++x) hX.push_back(m.le_coefficients[x * m.n_le + r]);
            hst.push_back(s);
        }
    }
    for (int c = 0; c < n_ct; ++c) {
        const tincr_exciton_ct &q = cts[c];
        if (q.h < 0 || q.h >= n_mono || q.l < 0 || q.l >= n_mono || q.h == q.l || q.n_ct <= 0 || q.state < 0 ||
            q.state >= q.n_ct || !q.energies || !q.coefficients || !q.q_tr)
            fail(TINCR_BAD_ARG, "exciton_states: bad CT state");
        if (!pidx.count(PairKey{std::min(q.h, q.l), std::max(q.h, q.l)}))
            fail(TINCR_BAD_ARG, "exciton_states: CT state of an unlisted pair");
        const int oh = no[q.h], vl = nao[q.l] - no[q.l];
        const int nh = mono[q.h].n_atoms, nl = mono[q.l].n_atoms;
        ExState s{1, q.h, q.l, atom0[q.h], nh, atom0[q.l], nl, (long long)hq.size(), q.energies[q.state]};
        for (int a = 0; a < nh + nl; ++a) hq.push_back(q.q_tr[(size_t)a * q.n_ct + q.state]);
        xoff.push_back((long long)hX.size());
        for (long long x = 0; x < (long long)oh * vl; ++x) hX.push_back(q.coefficients[x * q.n_ct + q.state]);
        hst.push_back(s);
    }
    const int ns = (int)hst.size();
    if (ns < n_roots) fail(TINCR_BAD_ARG, "exciton_states: fewer basis states than roots");
    check_finite(hq.data(), hq.size(), "transition charges");
    check_finite(hX.data(), hX.size(), "CI coefficients");
    DevBuf<ExState> dst;
    DevBuf<double> dq, dX, dW, dH;
    upload_vec(stream, dst, hst);
    upload_vec(stream, dq, hq);
    upload_vec(stream, dX, hX);
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

    // ---- exchange jobs ----
    std::vector<ExMono> hm(n_mono);
    for (int k = 0; k < n_mono; ++k)
        hm[k] = ExMono{dC.p + offC[k], dSC.p + offC[k], dAo.p + offAo[k], nao[k], mono[k].n_atoms, atom0[k]};
    DevBuf<ExMono> dm;
    upload_vec(stream, dm, hm);
    std::vector<ExJob> xj;
    auto tile_side = [](int n, int &t) { t = n <= XJ_TMAX ? n : (n + ((n + XJ_TMAX - 1) / XJ_TMAX) - 1) / ((n + XJ_TMAX - 1) / XJ_TMAX); };
    auto add_job = [&](int s, int t, int x1, int y1, int x2, int y2, int p0, int np, int q0, int nq, int pa0, int na,
                       int qb0, int nb, const double *X1, int ld1, int i1, int a1, const double *X2, int ld2, int j2,
                       int b2) {
        int ta, tj;
        tile_side(na, ta);
        tile_side(nq, tj);
        while (ta * tj > XJ_T) {
            if (ta >= tj) --ta; else --tj;
        }
        for (int a0 = 0; a0 < na; a0 += ta)
            for (int j0 = 0; j0 < nq; j0 += tj) {
                ExJob J;
                J.s = s; J.t = t; J.x1 = x1; J.y1 = y1; J.x2 = x2; J.y2 = y2;
                J.p0 = p0; J.np = np; J.q0 = q0; J.pa0 = pa0; J.qb0 = qb0; J.nb = nb;
                J.ta0 = a0; J.ta = std::min(ta, na - a0); J.tj0 = j0; J.tj = std::min(tj, nq - j0);
                J.X1 = X1; J.X2 = X2; J.ld1 = ld1; J.i1 = i1; J.a1 = a1; J.ld2 = ld2; J.j2 = j2; J.b2 = b2;
                J.cross_xy1 = x1 != y1 ? cross(x1, y1) : nullptr;
                J.cross_yx1 = x1 != y1 ? cross(y1, x1) : nullptr;
                J.cross_xy2 = x2 != y2 ? cross(x2, y2) : nullptr;
                J.cross_yx2 = x2 != y2 ? cross(y2, x2) : nullptr;
                // a pair that is not listed is an ESD pair, whose AO overlap is zero (its atoms are
                // farther apart than the Slater-Koster tables reach): its charges, and the integral,
                // vanish
                if ((x1 != y1 && !J.cross_xy1) || (x2 != y2 && !J.cross_xy2)) continue;
                xj.push_back(J);
            }
    };
    auto near = [&](int a, int b) { return a == b || is_real(a, b); };   // pair type Pair or None
    for (int s = 0; s < ns; ++s)
        for (int t = s + 1; t < ns; ++t) {
            const ExState &A = hst[s], &B = hst[t];
            const double *Xs = dX.p + xoff[s], *Xt = dX.p + xoff[t];
            if (A.kind == 0 && B.kind == 0) {
                // le_le (integrals.rs:81-169): exchange for real pairs, full orbital spaces
                if (A.hole == B.hole || !is_real(A.hole, B.hole)) continue;
                const int I = A.hole, Jm = B.hole, oI = no[I], vI = nao[I] - oI, oJ = no[Jm], vJ = nao[Jm] - oJ;
                add_job(s, t, I, Jm, I, Jm, 0, oI, 0, oJ, oI, vI, oJ, vJ, Xs, vI, 0, 0, Xt, vJ, 0, 0);
            } else if (A.kind == 0 || B.kind == 0) {
                // le_ct_2e_new (integrals.rs:602-727): exchange when the LE monomer is the hole, the
                // electron or a real-pair neighbour of either; restricted active spaces
                const int le = A.kind == 0 ? s : t, ct = A.kind == 0 ? t : s;
                const ExState &L = hst[le], &C = hst[ct];
                const int I = L.hole, h = C.hole, l = C.elec;
                if (!(near(I, h) || near(I, l))) continue;
                const int oI = no[I], vI = nao[I] - oI, oh = no[h], vl = nao[l] - no[l];
                const int out_s = std::min(le, ct), out_t = std::max(le, ct);
                add_job(out_s, out_t, I, h, I, l, oI - ACTIVE, ACTIVE, oh - ACTIVE, ACTIVE, oI, ACTIVE, no[l], ACTIVE,
                        dX.p + xoff[le], vI, oI - ACTIVE, 0, dX.p + xoff[ct], vl, oh - ACTIVE, 0);
            } else {
                // ct_ct_new (integrals.rs:733-878): exchange when the holes and the electrons are each on
                // the same monomer or on a real pair; restricted active spaces
                if (A.hole == B.hole && A.elec == B.elec) continue;
                if (!(near(A.hole, B.hole) && near(A.elec, B.elec))) continue;
                const int h1 = A.hole, l1 = A.elec, h2 = B.hole, l2 = B.elec;
                const int v1 = nao[l1] - no[l1], v2 = nao[l2] - no[l2];
                add_job(s, t, h1, h2, l1, l2, no[h1] - ACTIVE, ACTIVE, no[h2] - ACTIVE, ACTIVE, no[l1], ACTIVE, no[l2],
                        ACTIVE, Xs, v1, no[h1] - ACTIVE, 0, Xt, v2, no[h2] - ACTIVE, 0);
            }
        }
    if (!xj.empty()) {
        DevBuf<ExJob> dxj;
        upload_vec(stream, dxj, xj);
        const size_t smem = fp32 ? sizeof(XjSmem<float>) : sizeof(XjSmem<double>);
        static bool attr = false;
        if (!attr) {
            TINCR_CUDA(cudaFuncSetAttribute(ex_exchange_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)sizeof(XjSmem<float>)));
            TINCR_CUDA(cudaFuncSetAttribute(ex_exchange_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)sizeof(XjSmem<double>)));
            attr = true;
        }
        const int slot = prof_begin(TINCR_KF_AO_EXCHANGE);
        for (size_t j0 = 0; j0 < xj.size(); j0 += 1u << 20) {   // grid limit
            const unsigned nb = (unsigned)std::min<size_t>(xj.size() - j0, 1u << 20);
            if (fp32)
                ex_exchange_kernel<float><<<nb, XJ_T, smem, stream>>>(dxj.p + j0, dm.p, dGlr.p, n_atoms_total, dH.p, ns);
            else
                ex_exchange_kernel<double><<<nb, XJ_T, smem, stream>>>(dxj.p + j0, dm.p, dGlr.p, n_atoms_total, dH.p, ns);
            count_launch(stream, "ex_exchange");
            check_launch("ex_exchange");
        }
        double fl = 0.0;
        for (const ExJob &J : xj) {
            const double n1 = hm[J.x1].n_atoms + (J.x1 != J.y1 ? hm[J.y1].n_atoms : 0);
            const double n2 = hm[J.x2].n_atoms + (J.x2 != J.y2 ? hm[J.y2].n_atoms : 0);
            fl += 2.0 * J.ta * J.tj * n1 * n2;
        }
        prof_end(slot, fl, 0.0);
        sync();
    }

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
        std::vector<double> hPo(std::max<long long>(1, npo)), hPe(std::max<long long>(1, npe));
        for (int p : rp) {
            const int nij = nao[pairs[p].i] + nao[pairs[p].j];
            check_finite(pairs[p].pair_orbs, (size_t)nij * nij, "pair orbitals");
            check_finite(pairs[p].pair_orbe, (size_t)nij, "pair orbital energies");
            std::copy(pairs[p].pair_orbs, pairs[p].pair_orbs + (size_t)nij * nij, hPo.begin() + o_po[p]);
            std::copy(pairs[p].pair_orbe, pairs[p].pair_orbe + nij, hPe.begin() + o_pe[p]);
        }
        DevBuf<double> dPo, dPe, dSpr, dSpq, dFd, dFij;
        upload_vec(stream, dPo, hPo);
        upload_vec(stream, dPe, hPe);
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
    DevBuf<double> dV, dAV, dAp, dY, dRitz, dRk, dU, dNrm, dT, dc;
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
    std::vector<double> ap, w(nr), yt, err(nr), u(nr);
    for (it = 0; it < max_iter; ++it) {
        // products of every subspace vector (the dense engine has no cache) and the projection
        TINCR_CUDA(cudaMemsetAsync(dAV.p, 0, (size_t)m * ns * sizeof(double), stream));
        TINCR_CUDA(cudaMemsetAsync(dAp.p, 0, (size_t)m * m * sizeof(double), stream));
        gb.gemm(m, ns, ns, dV.p, ns, 1, dH.p, ns, 1, dAV.p, ns, 1.0);
        gb.run(*this, false, dJobs, dTiles, TINCR_KF_SUBSPACE);
        gb.gemm(m, m, ns, dV.p, ns, 1, dAV.p, 1, ns, dAp.p, m, 1.0);
        gb.run(*this, false, dJobs, dTiles, TINCR_KF_SUBSPACE);
        ap.resize((size_t)m * m);
        TINCR_CUDA(cudaMemcpyAsync(ap.data(), dAp.p, ap.size() * sizeof(double), cudaMemcpyDeviceToHost, stream));
        sync();
        yt.assign((size_t)nr * m, 0.0);
        if (!eigh_lowest_upper(m, ap.data(), nr, w.data(), yt.data()))
            fail(TINCR_NONFINITE, "exciton_states: subspace eigensolver failed");
        for (int r = 0; r < nr; ++r) u[r] = w[r];
        TINCR_CUDA(cudaMemcpyAsync(dY.p, yt.data(), yt.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
        TINCR_CUDA(cudaMemcpyAsync(dU.p, u.data(), nr * sizeof(double), cudaMemcpyHostToDevice, stream));
        TINCR_CUDA(cudaMemsetAsync(dRitz.p, 0, (size_t)nr * ns * sizeof(double), stream));
        TINCR_CUDA(cudaMemsetAsync(dRk.p, 0, (size_t)nr * ns * sizeof(double), stream));
        gb.gemm(nr, ns, m, dY.p, m, 1, dV.p, ns, 1, dRitz.p, ns, 1.0);
        gb.gemm(nr, ns, m, dY.p, m, 1, dAV.p, ns, 1, dRk.p, ns, 1.0);
        gb.run(*this, false, dJobs, dTiles, TINCR_KF_SUBSPACE);
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
            for (int r = 0; r < nr; ++r) {
                if (!(err[r] > tol)) continue;
                ex_precondition_kernel<<<ceil_div(ns, 256), 256, 0, stream>>>(ns, dRk.p + (size_t)r * ns, u[r], dH.p,
                                                                             dT.p);
                count_launch(stream, "ex_precondition");
                ex_dots_kernel<<<m, 256, 0, stream>>>(m, ns, dV.p, dT.p, dc.p);
                count_launch(stream, "ex_dots");
                ex_orth_update_kernel<<<1, 256, 0, stream>>>(m, ns, dV.p, dc.p, dT.p, dNrm.p + nr);
                count_launch(stream, "ex_orth_update");
                double nrm = 0.0;
                TINCR_CUDA(cudaMemcpyAsync(&nrm, dNrm.p + nr, sizeof(double), cudaMemcpyDeviceToHost, stream));
                sync();
                if (nrm > 1.0e-8 && m < cap) {
                    ex_scale_kernel<<<ceil_div(ns, 256), 256, 0, stream>>>(ns, 1.0 / nrm, dT.p, dV.p + (size_t)m * ns);
                    count_launch(stream, "ex_scale");
                    ++m;
                }
            }
        } else {
            dim_sub = nr;
            TINCR_CUDA(cudaMemcpyAsync(dV.p, dRitz.p, (size_t)nr * ns * sizeof(double), cudaMemcpyDeviceToDevice, stream));
            m = nr;
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
