// Batched SCC ground states (restricted closed shell, long-range corrected or not), one system per CTA.
//
// Follows tincr's SCC routine (src/scc/scc_routine.rs:121-290) together with the inputs it builds
// first: overlap S and H0 from the Slater-Koster splines (src/scc/h0_and_s.rs:92-182), the Gaussian
// gamma matrices (src/scc/gamma_approximation.rs:75-124, :175-193), the neutral-atom reference density
// (src/scc/helpers.rs:218-229), the long-range exchange Hamiltonian (src/scc/helpers.rs:111-155), the
// Loewdin orthogonalisation X = S^-1/2 (scc_routine.rs:172-174) and the repulsive energy.
// Convergence: the largest element of the commutator X^T (F P S - S P F) X below tol, with DIIS on the
// Fock matrix (up to 8 iterates).  tincr mixes Mulliken charges with Broyden's method and stops at an
// rms charge change of 1e-5: the same stationary density, reached here to a tighter test.
//
// Layout.  A persistent grid (two CTAs per SM) takes systems from a counter, largest first.  A CTA
// keeps its system's matrices in a private slot of global memory (a few MB, L2-resident) and runs
// every step itself:
//  * GEMMs on tiles of 16 x 16 outputs, one per thread (FP64) or 32 x 32, 2 x 2 per thread (FP32).
//    GB300 issues 2 FP64 FMAs per SM and clock against 128 FP32 FMAs, so the FP64 GEMMs are bound by
//    the FP64 pipe and small tiles keep the padding of n = 48..256 matrices small;
//  * eigenpairs: Householder tridiagonalisation, Sturm-count bisection with one thread per root,
//    inverse iteration with one thread per root (LU with partial pivoting), Gram-Schmidt inside
//    clusters of close roots (LAPACK dstein's criterion, 1e-3 of the tridiagonal's norm), and the
//    back-transformation by the stored reflections;
//  * the Fock build, Mulliken charges, DIIS and the energy as CTA-wide element loops and reductions.
// With TINCR_SCC_FP32_START the iterations run in FP32 until the commutator is below 1e-5 (at most
// 60 of them), then continue in FP64 from that density with a fresh DIIS history: the stationary
// point, the convergence test and the final orbitals are FP64 either way.
// Every loop is bounded (max_iter, 80 bisection steps, 3 inverse iterations); there is no
// inter-CTA waiting.  Non-finite values end the system's iterations and are reported.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "common.cuh"
#include "sk_math.cuh"
#include "tda.cuh"

namespace tincr {

namespace {

constexpr int SC_T = 256, SC_W = SC_T / 32;
constexpr int SC_NMAX = 256;           // orbitals (and atoms) per system
constexpr int SC_DIIS = 8;             // DIIS history
constexpr int SC_FP32_MAX = 20;        // FP32 iterations at most before the FP64 phase
constexpr double SC_FP32_SWITCH = 1e-5;
constexpr double SC_PROXIMITY = 30.0;  // bohr: Slater-Koster pairs farther apart are zero (tincr's PROXIMITY_CUTOFF)
constexpr int SC_SLOTS_PER_SM = 2;

struct ScArgs {
    int n_sys;
    const tincr_scc_system *sys;
    const int *order;                  // systems in the order they are taken
    const int *kind;
    const double *xyz;
    const double *p_start;             // packed n x n blocks or null
    const double *s_in, *h0_in, *gam_in, *glr_in;   // caller-supplied inputs or null
    // parameter tables
    int n_kinds, n_knots, sk_extrapolate;
    const int *kind_z, *kind_norb, *kind_l, *kind_m;
    const double *kind_occ, *kind_energy, *sigma, *knots, *coef;
    int rep_ntmax;
    const int *rep_nt;
    const double *rep_knots, *rep_coef, *rep_dmax;
    int lc;
    double r_lr, tol, level_shift;
    int max_iter, fp32_start;
    // outputs (null: not wanted)
    double *orbe, *orbs, *p, *dq, *energy, *s_out, *h0_out, *hcx, *residual;
    int *iterations, *converged, *status;
    // slots
    unsigned char *ws;
    long long slot_bytes, nn_max, at2_max, npad;
    int *next;
};

// shared memory of one CTA
struct ScShared {
    alignas(16) double gemm[2 * 16 * 17];               // GEMM tiles (FP64 16 x 17, FP32 16 x 33 each)
    double d[SC_NMAX], e[SC_NMAX], beta[SC_NMAX], esq[SC_NMAX], vp[SC_NMAX], vu[SC_NMAX], vs[SC_NMAX];
    double w[SC_NMAX];                                   // eigenvalues
    double qao[SC_NMAX], dq[SC_NMAX], esp[SC_NMAX];
    double red[SC_W * SC_DIIS + SC_DIIS + 8];
    double B[SC_DIIS][SC_DIIS];
    double coef[SC_DIIS + 1];
    double lin[(SC_DIIS + 1) * (SC_DIIS + 2)];
    int kind[SC_NMAX], ao_off[SC_NMAX + 1];
    short ao_atom[SC_NMAX];
    int sys_id, flag;
};

// ---------------------------------------------------------------------------------------------
// CTA-wide reductions (every thread receives the result)
// ---------------------------------------------------------------------------------------------

__device__ double sc_sum(double v, ScShared &sm) {
    for (int off = 16; off; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sm.red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    for (int w = 0; w < SC_W; ++w) s += sm.red[w];
    __syncthreads();
    return s;
}

__device__ double sc_max(double v, ScShared &sm) {
    for (int off = 16; off; off >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, off));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sm.red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = sm.red[0];
    for (int w = 1; w < SC_W; ++w) s = fmax(s, sm.red[w]);
    __syncthreads();
    return s;
}

// m sums (m <= SC_DIIS) at once; out in sm.red[SC_W * SC_DIIS + r]
__device__ void sc_sums(double *v, int m, ScShared &sm) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int r = 0; r < m; ++r) {
        double x = v[r];
        for (int off = 16; off; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
        if (lane == 0) sm.red[warp * SC_DIIS + r] = x;
    }
    __syncthreads();
    if (threadIdx.x < m) {
        double s = 0.0;
        for (int w = 0; w < SC_W; ++w) s += sm.red[w * SC_DIIS + threadIdx.x];
        sm.red[SC_W * SC_DIIS + threadIdx.x] = s;
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------------------------
// CTA GEMM: C = alpha op(A) op(B) + beta C, row-major, op(A) M x K, op(B) K x N (beta = 0: C not read).
// Tiles of TL = 16 R outputs square; thread (ty, tx) computes rows R ty + i, columns R tx + j.
// ---------------------------------------------------------------------------------------------

template <class T, int R>
__device__ void sc_gemm(int M, int N, int K, T alpha, const T *A, int lda, bool ta, const T *B, int ldb, bool tb,
                        T beta, T *C, int ldc, ScShared &sm, bool sym) {
    constexpr int TL = 16 * R;
    T(*As)[TL + 1] = reinterpret_cast<T(*)[TL + 1]>(sm.gemm);
    T(*Bs)[TL + 1] = reinterpret_cast<T(*)[TL + 1]>(reinterpret_cast<T *>(sm.gemm) + 16 * (TL + 1));
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
    const int tm = (M + TL - 1) / TL, tn = (N + TL - 1) / TL;
    for (int t = 0; t < tm * tn; ++t) {
        if (sym && t / tn < t % tn) continue;   // symmetric result: tiles on and below the diagonal only
        const int m0 = (t / tn) * TL, n0 = (t % tn) * TL;
        T acc[R][R];
#pragma unroll
        for (int i = 0; i < R; ++i)
#pragma unroll
            for (int j = 0; j < R; ++j) acc[i][j] = T(0);
        for (int k0 = 0; k0 < K; k0 += 16) {
#pragma unroll
            for (int q = 0; q < R; ++q) {
                const int e = tid + q * SC_T;   // 0 .. 16 TL - 1
                if (!ta) {
                    const int mm = e >> 4, kk = e & 15;
                    const int m = m0 + mm, k = k0 + kk;
                    As[kk][mm] = (m < M && k < K) ? A[(long long)m * lda + k] : T(0);
                } else {
                    const int kk = e / TL, mm = e % TL;
                    const int m = m0 + mm, k = k0 + kk;
                    As[kk][mm] = (m < M && k < K) ? A[(long long)k * lda + m] : T(0);
                }
                if (!tb) {
                    const int kk = e / TL, nn = e % TL;
                    const int n = n0 + nn, k = k0 + kk;
                    Bs[kk][nn] = (n < N && k < K) ? B[(long long)k * ldb + n] : T(0);
                } else {
                    const int nn = e >> 4, kk = e & 15;
                    const int n = n0 + nn, k = k0 + kk;
                    Bs[kk][nn] = (n < N && k < K) ? B[(long long)n * ldb + k] : T(0);
                }
            }
            __syncthreads();
#pragma unroll
            for (int kk = 0; kk < 16; ++kk) {
                T a[R], b[R];
#pragma unroll
                for (int i = 0; i < R; ++i) a[i] = As[kk][R * ty + i];
#pragma unroll
                for (int j = 0; j < R; ++j) b[j] = Bs[kk][R * tx + j];
#pragma unroll
                for (int i = 0; i < R; ++i)
#pragma unroll
                    for (int j = 0; j < R; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
            }
            __syncthreads();
        }
#pragma unroll
        for (int i = 0; i < R; ++i)
#pragma unroll
            for (int j = 0; j < R; ++j) {
                const int m = m0 + R * ty + i, n = n0 + R * tx + j;
                if (m < M && n < N) {
                    T *c = C + (long long)m * ldc + n;
                    *c = beta == T(0) ? alpha * acc[i][j] : fma(alpha, acc[i][j], beta * *c);
                }
            }
    }
    __syncthreads();
    if (sym) {   // upper triangle from the lower one (C and, with beta != 0, its old value symmetric)
        for (long long e = tid; e < (long long)M * M; e += SC_T) {
            const int i = (int)(e / M), j = (int)(e - (long long)i * M);
            if (i < j) C[(long long)i * ldc + j] = C[(long long)j * ldc + i];
        }
        __syncthreads();
    }
}

template <class T> struct ScTile;
template <> struct ScTile<double> { static constexpr int R = 1; };
template <> struct ScTile<float> { static constexpr int R = 2; };

template <class T>
__device__ __forceinline__ void gemm(int M, int N, int K, T alpha, const T *A, int lda, bool ta, const T *B, int ldb,
                                     bool tb, T beta, T *C, int ldc, ScShared &sm) {
    sc_gemm<T, ScTile<T>::R>(M, N, K, alpha, A, lda, ta, B, ldb, tb, beta, C, ldc, sm, false);
}

// the same for a product known to be symmetric (M == N): the tiles below the diagonal are computed
// and mirrored
template <class T>
__device__ __forceinline__ void gemm_sym(int M, int K, T alpha, const T *A, int lda, bool ta, const T *B, int ldb,
                                         bool tb, T beta, T *C, int ldc, ScShared &sm) {
    sc_gemm<T, ScTile<T>::R>(M, M, K, alpha, A, lda, ta, B, ldb, tb, beta, C, ldc, sm, true);
}

// ---------------------------------------------------------------------------------------------
// Symmetric eigenproblem
// ---------------------------------------------------------------------------------------------

template <class T> struct ScEps;
template <> struct ScEps<double> {
    static constexpr double eps = 2.220446049250313e-16, tiny = 2.2250738585072014e-308;
};
template <> struct ScEps<float> {
    static constexpr double eps = 1.1920928955078125e-07, tiny = 1.1754943508222875e-38;
};

// number of eigenvalues of the tridiagonal (d, squared off-diagonal esq) below x: sign changes of
// the leading principal minors N_i = (d_i - x) N_{i-1} - esq_{i-1} N_{i-2} (no division), rescaled
// by a power of two when |N_i| leaves [2^-L, 2^L]; an exact zero becomes a tiny value of the
// opposite sign
__device__ __forceinline__ int sc_sturm(const double *d, const double *esq, int n, double x) {
    double n0 = 1.0, n1 = d[0] - x;
    if (n1 == 0.0) n1 = -0x1p-100;
    int c = __double2hiint(n1) < 0;
    for (int i = 1; i < n; ++i) {
        double n2 = fma(d[i] - x, n1, -(esq[i - 1] * n0));
        const long long bits = __double_as_longlong(n2);
        if ((bits << 1) == 0) {
            n2 = -0x1p-100 * n1;
        } else {
            const int ex = (int)((bits >> 52) & 0x7ff);
            if ((ex > 1023 + 400 || ex < 1023 - 400) && ex < 2047) {
                const double s = __longlong_as_double((long long)(2046 - ex) << 52);
                n1 *= s;
                n2 *= s;
            }
        }
        c += (int)(((unsigned)__double2hiint(n1) ^ (unsigned)__double2hiint(n2)) >> 31);
        n0 = n1;
        n1 = n2;
    }
    return c;
}

__device__ __forceinline__ int sc_sturm(const float *d, const float *esq, int n, float x) {
    float n0 = 1.0f, n1 = d[0] - x;
    if (n1 == 0.0f) n1 = -0x1p-40f;
    int c = __float_as_int(n1) < 0;
    for (int i = 1; i < n; ++i) {
        float n2 = fmaf(d[i] - x, n1, -(esq[i - 1] * n0));
        const int bits = __float_as_int(n2);
        if ((bits << 1) == 0) {
            n2 = -0x1p-40f * n1;
        } else {
            const int ex = (bits >> 23) & 0xff;
            if ((ex > 127 + 40 || ex < 127 - 40) && ex < 255) {
                const float s = __int_as_float((254 - ex) << 23);   // 2^(127 - ex)
                n1 *= s;
                n2 *= s;
            }
        }
        c += (int)(((unsigned)__float_as_int(n1) ^ (unsigned)__float_as_int(n2)) >> 31);
        n0 = n1;
        n1 = n2;
    }
    return c;
}

// Lowest nr eigenpairs of the symmetric n x n matrix A (row-major, overwritten: row k keeps the
// k-th Householder vector in columns k+1..n-1).  Eigenvalues ascending into sm.w (as double),
// eigenvectors into Z [n x nr] row-major (column r = eigenvector r).  ws: 4 n nr elements, piv: n nr
// bytes.  Returns false on a non-finite value.
template <class T>
__device__ bool sc_eigh(int n, int nr, T *A, T *Z, T *ws, unsigned char *piv, ScShared &sm) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    T *d = reinterpret_cast<T *>(sm.d), *e = reinterpret_cast<T *>(sm.e), *beta = reinterpret_cast<T *>(sm.beta);
    T *esq = reinterpret_cast<T *>(sm.esq), *p = reinterpret_cast<T *>(sm.vp), *u = reinterpret_cast<T *>(sm.vu);
    T *s = reinterpret_cast<T *>(sm.vs);
    // 1. tridiagonalisation: H_k = I - beta_k u u^T acting on rows / columns k+1..n-1
    for (int k = 0; k + 2 < n; ++k) {
        const int n1 = n - k - 1;
        T *row = A + (long long)k * n + (k + 1);
        if (warp == 0) {
            T s2 = T(0);
            for (int i = 1 + lane; i < n1; i += 32) s2 += row[i] * row[i];
            for (int off = 16; off; off >>= 1) s2 += __shfl_xor_sync(0xffffffffu, s2, off);
            const T x0 = row[0];
            T bet = T(0), alpha = x0;
            if (s2 != T(0)) {
                const T nx = sqrt(x0 * x0 + s2);
                alpha = x0 > T(0) ? -nx : nx;
                bet = T(1) / (alpha * (alpha - x0));
            }
            for (int i = 1 + lane; i < n1; i += 32) u[i] = row[i];
            if (lane == 0) {
                d[k] = A[(long long)k * n + k];
                e[k] = alpha;
                beta[k] = bet;
                u[0] = x0 - alpha;
                row[0] = x0 - alpha;
            }
        }
        __syncthreads();
        const T bet = beta[k];
        if (bet == T(0)) continue;   // the same in every thread
        {   // p = bet A' u, G lanes per row
            const int G = n1 >= 64 ? 32 : (n1 >= 16 ? 8 : 2);
            const int rows_per_pass = SC_T / G;
            const int sub = tid % G;
            for (int base = 0; base < n1; base += rows_per_pass) {   // the same trip count in every thread
                const int r0 = base + tid / G;
                T acc = T(0);
                if (r0 < n1) {
                    const T *ar = A + (long long)(k + 1 + r0) * n + (k + 1);
                    for (int j = sub; j < n1; j += G) acc = fma(ar[j], u[j], acc);
                }
                for (int off = G >> 1; off; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
                if (sub == 0 && r0 < n1) p[r0] = bet * acc;
            }
        }
        __syncthreads();
        if (warp == 0) {   // q = p - (bet u.p / 2) u
            T up = T(0);
            for (int i = lane; i < n1; i += 32) up += u[i] * p[i];
            for (int off = 16; off; off >>= 1) up += __shfl_xor_sync(0xffffffffu, up, off);
            const T K = T(0.5) * bet * up;
            for (int i = lane; i < n1; i += 32) p[i] -= K * u[i];
        }
        __syncthreads();
        for (int t = tid; t < n1 * n1; t += SC_T) {   // A' -= u q^T + q u^T
            const int i = t / n1, j = t - i * n1;
            T *a = A + (long long)(k + 1 + i) * n + (k + 1 + j);
            *a = fma(-u[i], p[j], fma(-p[i], u[j], *a));
        }
        __syncthreads();
    }
    if (tid == 0) {
        if (n >= 2) {
            d[n - 2] = A[(long long)(n - 2) * n + n - 2];
            e[n - 2] = A[(long long)(n - 2) * n + n - 1];
            beta[n - 2] = T(0);
        }
        d[n - 1] = A[(long long)(n - 1) * n + n - 1];
        e[n - 1] = T(0);
        beta[n - 1] = T(0);
    }
    __syncthreads();
    // 2. Gershgorin interval, e^2, finiteness
    double glo = 1e300, ghi = -1e300, emax2 = 0.0;
    bool fin = true;
    for (int i = tid; i < n; i += SC_T) {
        const double r = fabs((double)e[i]) + (i > 0 ? fabs((double)e[i - 1]) : 0.0);
        glo = fmin(glo, (double)d[i] - r);
        ghi = fmax(ghi, (double)d[i] + r);
        esq[i] = e[i] * e[i];
        emax2 = fmax(emax2, (double)esq[i]);
        fin = fin && isfinite((double)d[i]) && isfinite((double)e[i]);
    }
    glo = -sc_max(-glo, sm);
    ghi = sc_max(ghi, sm);
    emax2 = sc_max(emax2, sm);
    if (sc_max(fin ? 0.0 : 1.0, sm) != 0.0) return false;
    const double eps = ScEps<T>::eps;
    const double tnorm = fmax(fabs(glo), fabs(ghi));
    const double pivmin = ScEps<T>::tiny * fmax(1.0, emax2) * 4.0;
    // 3. eigenvalue r by bisection on Sturm counts, one thread per root
    for (int r = tid; r < nr; r += SC_T) {
        T a = (T)(glo - (2.0 * eps * tnorm + 2.0 * pivmin)), b = (T)(ghi + (2.0 * eps * tnorm + 2.0 * pivmin));
        for (int it = 0; it < 80; ++it) {
            const T mid = T(0.5) * (a + b);
            if (!(b - a > T(2.0 * eps) * fmax(fabs(a), fabs(b)) + T(pivmin)) || mid <= a || mid >= b) break;
            if (sc_sturm(d, esq, n, mid) > r) b = mid; else a = mid;
        }
        sm.w[r] = 0.5 * ((double)a + (double)b);
    }
    __syncthreads();
    // 4. inverse iteration, one thread per root: LU of T - w_r I with partial pivoting (factors
    //    interleaved over the roots, [i * nr + r], so a warp's accesses are contiguous), then three
    //    solves from a fixed start vector; the recurrences run in registers
    const T tiny = (T)(eps * fmax(tnorm, 1e-30));
    for (int r = tid; r < nr; r += SC_T) {
        const T lam = (T)sm.w[r];
        T *__restrict__ DL = ws;
        T *__restrict__ DD = ws + (long long)n * nr;
        T *__restrict__ DU = ws + 2LL * n * nr;
        T *__restrict__ DU2 = ws + 3LL * n * nr;
        unsigned char *__restrict__ PV = piv;
        T *__restrict__ Zr = Z;
#define IX(i) ((long long)(i) * nr + r)
        T cdd = d[0] - lam, cdu = e[0];
        for (int i = 0; i + 1 < n; ++i) {
            const T li = e[i], dn = d[i + 1] - lam, un = e[i + 1];
            if (fabs(cdd) >= fabs(li)) {
                const T dv = fabs(cdd) < tiny ? (cdd < T(0) ? -tiny : tiny) : cdd;
                const T rp = T(1) / dv, l = li * rp;
                DD[IX(i)] = rp;
                DL[IX(i)] = l;
                DU[IX(i)] = cdu;
                DU2[IX(i)] = T(0);
                PV[IX(i)] = 0;
                cdd = dn - l * cdu;
                cdu = un;
            } else {
                const T rp = T(1) / li, l = cdd * rp;
                DD[IX(i)] = rp;
                DL[IX(i)] = l;
                DU[IX(i)] = dn;
                DU2[IX(i)] = i + 2 < n ? un : T(0);
                PV[IX(i)] = 1;
                cdd = cdu - l * dn;
                cdu = -l * un;
            }
        }
        DD[IX(n - 1)] = T(1) / (fabs(cdd) < tiny ? (cdd < T(0) ? -tiny : tiny) : cdd);
        DU[IX(n - 1)] = T(0);
        DU2[IX(n - 1)] = T(0);
        for (int it = 0; it < 3; ++it) {
            // L^-1 with the interchanges (the start vector is generated in the first pass)
            auto start = [&](int i) { return T(1) + T(0.5) * (T)((i * (r + 1) * 7919 + 13 * r) % 97) / T(97); };
            T zc = it == 0 ? start(0) : Zr[IX(0)];
#pragma unroll 4
            for (int i = 0; i + 1 < n; ++i) {
                T zn = it == 0 ? start(i + 1) : Zr[IX(i + 1)];
                if (PV[IX(i)]) { const T t = zc; zc = zn; zn = t; }
                zn -= DL[IX(i)] * zc;
                Zr[IX(i)] = zc;
                zc = zn;
            }
            Zr[IX(n - 1)] = zc;
            // U^-1 and the norm
            T z1 = T(0), z2 = T(0), nrm = T(0);
#pragma unroll 4
            for (int i = n - 1; i >= 0; --i) {
                T v = Zr[IX(i)] - DU[IX(i)] * z1 - DU2[IX(i)] * z2;
                v *= DD[IX(i)];
                Zr[IX(i)] = v;
                nrm = fma(v, v, nrm);
                z2 = z1;
                z1 = v;
            }
            nrm = T(1) / sqrt(nrm);
#pragma unroll 4
            for (int i = 0; i < n; ++i) Zr[IX(i)] *= nrm;
        }
#undef IX
    }
    __syncthreads();
    // 5. Gram-Schmidt (twice) inside clusters of roots closer than 1e-3 |T| (warp 0, ascending)
    if (warp == 0) {
        const double ortol = 1e-3 * tnorm;
        int c0 = 0;
        for (int r = 1; r < nr; ++r) {
            if (sm.w[r] - sm.w[r - 1] > ortol) {
                c0 = r;
                continue;
            }
            for (int pass = 0; pass < 2; ++pass)
                for (int q = c0; q < r; ++q) {
                    T dot = T(0);
                    for (int i = lane; i < n; i += 32) dot += Z[(long long)i * nr + q] * Z[(long long)i * nr + r];
                    for (int off = 16; off; off >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, off);
                    for (int i = lane; i < n; i += 32) Z[(long long)i * nr + r] -= dot * Z[(long long)i * nr + q];
                    __syncwarp();
                }
            T nrm = T(0);
            for (int i = lane; i < n; i += 32) nrm += Z[(long long)i * nr + r] * Z[(long long)i * nr + r];
            for (int off = 16; off; off >>= 1) nrm += __shfl_xor_sync(0xffffffffu, nrm, off);
            nrm = T(1) / sqrt(nrm);
            for (int i = lane; i < n; i += 32) Z[(long long)i * nr + r] *= nrm;
            __syncwarp();
        }
    }
    __syncthreads();
    // 6. back-transformation Z <- H_0 ... H_{n-3} Z
    for (int k = n - 3; k >= 0; --k) {
        const T bet = beta[k];
        if (bet == T(0)) continue;
        const int n1 = n - k - 1;
        const T *uk = A + (long long)k * n + (k + 1);
        for (int r = tid; r < nr; r += SC_T) {
            T acc = T(0);
            for (int i = 0; i < n1; ++i) acc = fma(uk[i], Z[(long long)(k + 1 + i) * nr + r], acc);
            s[r] = bet * acc;
        }
        __syncthreads();
        for (int t = tid; t < n1 * nr; t += SC_T) {
            const int i = t / nr, r = t - i * nr;
            T *z = Z + (long long)(k + 1 + i) * nr + r;
            *z = fma(-s[r], uk[i], *z);
        }
        __syncthreads();
    }
    return true;
}

// ---------------------------------------------------------------------------------------------
// per-slot storage
// ---------------------------------------------------------------------------------------------

// FP64 inputs of the current system (S, H0, X = S^-1/2, Sh = S^1/2, gamma, gamma_lr, reference
// occupations p0) followed by the work area (29 n^2 doubles), used as T elements by the phase that
// runs (the FP32 phase keeps FP32 copies of the inputs in it), and the pivot flags (n^2 bytes).
struct ScSlot {
    double *S, *H0, *X, *Sh, *gam, *glr, *p0;
    unsigned char *work;
    unsigned char *piv;
};

constexpr int SC_WORK = 29;   // n x n blocks of the work area

__host__ __device__ inline long long sc_slot_doubles(long long nn, long long at2, long long npad) {
    return 4 * nn + 2 * at2 + npad + SC_WORK * nn;
}

__device__ ScSlot sc_slot(const ScArgs &a, int slot) {
    double *f = reinterpret_cast<double *>(a.ws + (long long)slot * a.slot_bytes);
    ScSlot s;
    s.S = f;
    s.H0 = f + a.nn_max;
    s.X = f + 2 * a.nn_max;
    s.Sh = f + 3 * a.nn_max;
    s.gam = f + 4 * a.nn_max;
    s.glr = s.gam + a.at2_max;
    s.p0 = s.glr + a.at2_max;
    s.work = reinterpret_cast<unsigned char *>(s.p0 + a.npad);
    s.piv = s.work + SC_WORK * a.nn_max * (long long)sizeof(double);
    return s;
}

template <class T> struct ScWork {
    T *S, *H0, *X, *Sh, *gam, *glr;     // inputs in T (FP64: the slot's arrays)
    T *F, *Fp, *P, *Pp, *T1, *T2, *T3, *EA, *Z, *W;   // n x n each (W: 4 n x n)
    T *Fh, *Eh;                         // SC_DIIS n x n each
};

template <class T>
__device__ ScWork<T> sc_work(const ScSlot &s, long long nn) {
    ScWork<T> w;
    T *b = reinterpret_cast<T *>(s.work);
    w.F = b; w.Fp = b + nn; w.P = b + 2 * nn; w.Pp = b + 3 * nn; w.T1 = b + 4 * nn; w.T2 = b + 5 * nn;
    w.T3 = b + 6 * nn; w.EA = b + 7 * nn; w.Z = b + 8 * nn; w.W = b + 9 * nn;
    w.Fh = b + 13 * nn; w.Eh = b + (13 + SC_DIIS) * nn;
    return w;
}

// ---------------------------------------------------------------------------------------------
// system set-up: AO tables, S, H0, gamma, gamma_lr, repulsion (FP64)
// ---------------------------------------------------------------------------------------------

__device__ double sc_setup(const ScArgs &a, const tincr_scc_system &sy, const ScSlot &sl, ScShared &sm) {
    const int tid = threadIdx.x, N = sy.n_atoms, n = sy.n_orb;
    const int *kind = a.kind + sy.atom_off;
    const double *xyz = a.xyz + 3 * sy.atom_off;
    for (int A = tid; A < N; A += SC_T) sm.kind[A] = kind[A];
    __syncthreads();
    if (tid == 0) {
        int o = 0;
        for (int A = 0; A < N; ++A) {
            sm.ao_off[A] = o;
            o += a.kind_norb[sm.kind[A]];
        }
        sm.ao_off[N] = o;
    }
    __syncthreads();
    for (int A = tid; A < N; A += SC_T)
        for (int mu = sm.ao_off[A]; mu < sm.ao_off[A + 1]; ++mu) sm.ao_atom[mu] = (short)A;
    __syncthreads();
    const long long nn = (long long)n * n;
    for (long long t = tid; t < nn; t += SC_T) {
        const int mu = (int)(t / n), nu = (int)(t - (long long)mu * n);
        double sv = 0.0, hv = 0.0;
        if (mu == nu) {
            const int A = sm.ao_atom[mu];
            sv = 1.0;
            hv = a.kind_energy[4 * sm.kind[A] + (mu - sm.ao_off[A])];
        }
        sl.S[t] = a.s_in ? a.s_in[sy.mat_off + t] : sv;
        sl.H0[t] = a.h0_in ? a.h0_in[sy.mat_off + t] : hv;
    }
    __syncthreads();
    const bool build_sk = !a.s_in || !a.h0_in;
    // atom pairs A < B
    double erep = 0.0;
    for (int t = tid; t < N * N; t += SC_T) {
        const int A = t / N, B = t - A * N;
        const int kA = sm.kind[A], kB = sm.kind[B];
        const double dx = xyz[3 * B] - xyz[3 * A], dy = xyz[3 * B + 1] - xyz[3 * A + 1], dz = xyz[3 * B + 2] - xyz[3 * A + 2];
        const double r = sqrt(dx * dx + dy * dy + dz * dz);
        // gamma (gamma_approximation.rs:75-124, diagonal :175-193)
        {
            const double sA = a.sigma[kA], sB = a.sigma[kB];
            double g, gl = 0.0;
            if (A == B) {
                g = 1.0 / sqrt(3.141592653589793 * sA * sA);
                if (a.lc) gl = 1.0 / sqrt(3.141592653589793 * (sA * sA + 0.25 * a.r_lr * a.r_lr));
            } else {
                g = erf(r / sqrt(2.0 * (sA * sA + sB * sB))) / r;
                if (a.lc) gl = erf(r / sqrt(2.0 * (sA * sA + sB * sB + 0.5 * a.r_lr * a.r_lr))) / r;
            }
            sl.gam[t] = a.gam_in ? a.gam_in[sy.pair_off + t] : g;
            sl.glr[t] = a.lc ? (a.glr_in ? a.glr_in[sy.pair_off + t] : gl) : 0.0;
        }
        if (A >= B) continue;
        // repulsion (pairs within the spline's range)
        if (a.rep_nt) {
            const int pk = kA * a.n_kinds + kB;
            if (r <= a.rep_dmax[pk]) {
                int l;
                double N3[4], N2[3], v = 0.0, dv;
                const double *tk = a.rep_knots + (long long)pk * a.rep_ntmax;
                if (bspline3_basis(tk, a.rep_nt[pk], r, l, N3, N2))
                    bspline3_eval(tk, a.rep_coef + (long long)pk * a.rep_ntmax, l, N3, N2, v, dv);
                erep += v;
            }
        }
        // Slater-Koster block: centre 1 the lower Z, ties by index (h0_and_s.rs:92-182)
        if (!build_sk || r >= SC_PROXIMITY) continue;
        const bool swap = a.kind_z[kA] > a.kind_z[kB];
        const int c1 = swap ? B : A, c2 = swap ? A : B;
        const int k1 = sm.kind[c1], k2 = sm.kind[c2];
        const double sg = swap ? -1.0 : 1.0;
        const double u[3] = {sg * dx / r, sg * dy / r, sg * dz / r};
        double vS[SK_SLOTS] = {0, 0, 0, 0, 0}, vH[SK_SLOTS] = {0, 0, 0, 0, 0}, dS[SK_SLOTS], dH[SK_SLOTS];
        int l;
        double N3[4], N2[3];
        if (bspline3_basis(a.knots, a.n_knots, r, l, N3, N2, a.sk_extrapolate != 0)) {
            const double *cS = a.coef + (long long)((k1 * a.n_kinds + k2) * 2 + 0) * SK_SLOTS * a.n_knots;
            const double *cH = a.coef + (long long)((k1 * a.n_kinds + k2) * 2 + 1) * SK_SLOTS * a.n_knots;
            for (int q = 0; q < SK_SLOTS; ++q) {
                bspline3_eval(a.knots, cS + (long long)q * a.n_knots, l, N3, N2, vS[q], dS[q]);
                bspline3_eval(a.knots, cH + (long long)q * a.n_knots, l, N3, N2, vH[q], dH[q]);
            }
        }
        const int n1 = a.kind_norb[k1], n2 = a.kind_norb[k2];
        for (int pp = 0; pp < n1; ++pp)
            for (int qq = 0; qq < n2; ++qq) {
                const int l1 = a.kind_l[4 * k1 + pp], m1 = a.kind_m[4 * k1 + pp];
                const int l2 = a.kind_l[4 * k2 + qq], m2 = a.kind_m[4 * k2 + qq];
                const double sv = sk_value(l1, m1, l2, m2, u, vS), hv = sk_value(l1, m1, l2, m2, u, vH);
                const int mu = sm.ao_off[c1] + pp, nu = sm.ao_off[c2] + qq;
                if (!a.s_in) {
                    sl.S[(long long)mu * n + nu] = sv;
                    sl.S[(long long)nu * n + mu] = sv;
                }
                if (!a.h0_in) {
                    sl.H0[(long long)mu * n + nu] = hv;
                    sl.H0[(long long)nu * n + mu] = hv;
                }
            }
    }
    const double e = sc_sum(erep, sm);   // synchronises
    return e;
}

// ---------------------------------------------------------------------------------------------
// SCC pieces
// ---------------------------------------------------------------------------------------------

// Mulliken charge differences of dP = P - diag(p0) into sm.dq (double), esp = gamma dq into sm.esp
template <class T>
__device__ void sc_charges(int n, int N, const T *P, const T *S, const T *gam, const double *p0, ScShared &sm) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int mu = warp; mu < n; mu += SC_W) {
        T acc = T(0);
        const T *pr = P + (long long)mu * n, *sr = S + (long long)mu * n;
        for (int nu = lane; nu < n; nu += 32) acc = fma(pr[nu], sr[nu], acc);
        for (int off = 16; off; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
        if (lane == 0) sm.qao[mu] = (double)acc - p0[mu];   // S_mumu = 1
    }
    __syncthreads();
    for (int A = tid; A < N; A += SC_T) {
        double q = 0.0;
        for (int mu = sm.ao_off[A]; mu < sm.ao_off[A + 1]; ++mu) q += sm.qao[mu];
        sm.dq[A] = q;
    }
    __syncthreads();
    for (int A = tid; A < N; A += SC_T) {
        double s = 0.0;
        for (int B = 0; B < N; ++B) s = fma((double)gam[(long long)A * N + B], sm.dq[B], s);
        sm.esp[A] = s;
    }
    __syncthreads();
}

// F = H0 + 1/2 S o (esp_mu + esp_nu) [+ H^x(dP)]  (scc_routine.rs:176-183; helpers.rs:111-155)
template <class T>
__device__ void sc_fock(int n, int N, bool lc, const ScWork<T> &w, const double *p0, ScShared &sm) {
    const int tid = threadIdx.x;
    const long long nn = (long long)n * n;
    for (long long t = tid; t < nn; t += SC_T) {
        const int mu = (int)(t / n), nu = (int)(t - (long long)mu * n);
        const T es = (T)(0.5 * (sm.esp[sm.ao_atom[mu]] + sm.esp[sm.ao_atom[nu]]));
        w.F[t] = fma(es, w.S[t], w.H0[t]);
    }
    if (!lc) {
        __syncthreads();
        return;
    }
    T *dP = w.W, *hx = w.W + nn, *tmp = w.W + 2 * nn;
    for (long long t = tid; t < nn; t += SC_T) {
        const int mu = (int)(t / n), nu = (int)(t - (long long)mu * n);
        dP[t] = w.P[t] - (mu == nu ? (T)p0[mu] : T(0));
    }
    __syncthreads();
#define GLR(mu, nu) w.glr[(long long)sm.ao_atom[mu] * N + sm.ao_atom[nu]]
    gemm<T>(n, n, n, T(1), w.S, n, false, dP, n, false, T(0), w.T1, n, sm);   // S dP
    for (long long t = tid; t < nn; t += SC_T) {
        const int mu = (int)(t / n), nu = (int)(t - (long long)mu * n);
        tmp[t] = GLR(mu, nu) * w.T1[t];
    }
    __syncthreads();
    gemm<T>(n, n, n, T(1), tmp, n, false, w.S, n, false, T(0), w.T2, n, sm);   // (g o S dP) S
    gemm_sym<T>(n, n, T(1), w.T1, n, false, w.S, n, false, T(0), w.T3, n, sm);   // S dP S
    for (long long t = tid; t < nn; t += SC_T) {
        const int mu = (int)(t / n), nu = (int)(t - (long long)mu * n);
        const T g = GLR(mu, nu);
        hx[t] = w.T2[t] + w.T2[(long long)nu * n + mu] + g * w.T3[t];
        tmp[t] = dP[t] * g;
    }
    __syncthreads();
    gemm<T>(n, n, n, T(1), w.S, n, false, tmp, n, false, T(0), w.T1, n, sm);   // S (dP o g)
    gemm_sym<T>(n, n, T(1), w.T1, n, false, w.S, n, false, T(1), hx, n, sm);    // + S (dP o g) S
    for (long long t = tid; t < nn; t += SC_T) {
        const int mu = (int)(t / n), nu = (int)(t - (long long)mu * n);
        w.F[t] += T(-0.0625) * (hx[t] + hx[(long long)nu * n + mu]);
    }
#undef GLR
    __syncthreads();
}

// solve the DIIS equations (m + 1 unknowns, the last the multiplier) on thread 0; sm.coef
__device__ void sc_diis_solve(int m, int cur, ScShared &sm) {
    if (threadIdx.x == 0) {
        const int q = m + 1, ld = q + 1;
        double *L = sm.lin;
        for (int i = 0; i < q; ++i) {
            for (int j = 0; j < q; ++j) L[i * ld + j] = (i < m && j < m) ? sm.B[i][j] : (i == m && j == m ? 0.0 : -1.0);
            L[i * ld + q] = i == m ? -1.0 : 0.0;
        }
        bool ok = true;
        for (int c = 0; c < q && ok; ++c) {
            int pr = c;
            for (int i = c + 1; i < q; ++i)
                if (fabs(L[i * ld + c]) > fabs(L[pr * ld + c])) pr = i;
            if (!(fabs(L[pr * ld + c]) > 0.0)) { ok = false; break; }
            if (pr != c)
                for (int j = 0; j <= q; ++j) { const double t = L[c * ld + j]; L[c * ld + j] = L[pr * ld + j]; L[pr * ld + j] = t; }
            for (int i = c + 1; i < q; ++i) {
                const double f = L[i * ld + c] / L[c * ld + c];
                for (int j = c; j <= q; ++j) L[i * ld + j] -= f * L[c * ld + j];
            }
        }
        if (ok) {
            for (int i = q - 1; i >= 0; --i) {
                double v = L[i * ld + q];
                for (int j = i + 1; j < q; ++j) v -= L[i * ld + j] * sm.coef[j];
                sm.coef[i] = v / L[i * ld + i];
            }
            for (int i = 0; i < m; ++i) ok = ok && isfinite(sm.coef[i]);
        }
        if (!ok)
            for (int i = 0; i < m; ++i) sm.coef[i] = i == cur ? 1.0 : 0.0;
    }
    __syncthreads();
}

struct ScState {
    int it;            // iterations done (both phases)
    bool converged;
    double errn;
    bool finite;
};

// SCC iterations in arithmetic T from the AO density in w.P: at most `limit` iterations; stops when
// the commutator is below `stop` (after at least one diagonalisation in total).  On return w.F and
// w.Fp hold the Fock matrix of the last iterate (from its density) and st.errn its commutator.
// `hist`: DIIS entries so far (in w.Fh / w.Eh and sm.B); the entry of the last iterate is stored in
// slot hist % SC_DIIS but not counted, so the next phase's first iterate replaces it.
template <class T>
__device__ void sc_iterate(const ScArgs &a, const tincr_scc_system &sy, const ScWork<T> &w, unsigned char *piv,
                           const double *p0, int limit, double stop, ScState &st, int &hist, ScShared &sm) {
    const int tid = threadIdx.x, n = sy.n_orb, N = sy.n_atoms, o = sy.n_occ;
    const long long nn = (long long)n * n;
    // P' = S^1/2 P S^1/2 of the starting density
    gemm<T>(n, n, n, T(1), w.Sh, n, false, w.P, n, false, T(0), w.T1, n, sm);
    gemm_sym<T>(n, n, T(1), w.T1, n, false, w.Sh, n, false, T(0), w.Pp, n, sm);
    for (int k = 0; k < limit; ++k) {
        ++st.it;
        sc_charges<T>(n, N, w.P, w.S, w.gam, p0, sm);
        sc_fock<T>(n, N, a.lc != 0, w, p0, sm);
        // F' = X F X, E' = F' P' - P' F'
        gemm<T>(n, n, n, T(1), w.X, n, false, w.F, n, false, T(0), w.T1, n, sm);
        gemm_sym<T>(n, n, T(1), w.T1, n, false, w.X, n, false, T(0), w.Fp, n, sm);
        gemm<T>(n, n, n, T(1), w.Fp, n, false, w.Pp, n, false, T(0), w.T1, n, sm);
        const int cur = hist % SC_DIIS;
        T *Fc = w.Fh + cur * nn, *Ec = w.Eh + cur * nn;
        double emax = 0.0;
        bool fin = true;
        for (long long t = tid; t < nn; t += SC_T) {
            const int mu = (int)(t / n), nu = (int)(t - (long long)mu * n);
            const T ev = w.T1[t] - w.T1[(long long)nu * n + mu];
            Ec[t] = ev;
            Fc[t] = w.Fp[t];
            emax = fmax(emax, fabs((double)ev));
            fin = fin && isfinite((double)w.Fp[t]);
        }
        st.errn = sc_max(emax, sm);
        if (sc_max(fin && isfinite(st.errn) ? 0.0 : 1.0, sm) != 0.0) {
            st.finite = false;
            return;
        }
        if (st.it > 1 && st.errn < stop) {
            st.converged = true;
            return;
        }
        if (k + 1 == limit) return;   // the Fock matrix of this iterate is the result
        ++hist;
        const int m = hist < SC_DIIS ? hist : SC_DIIS;
        // new row of the DIIS matrix: <E_i, E_cur>
        {
            double v[SC_DIIS];
            for (int i = 0; i < m; ++i) v[i] = 0.0;
            for (long long t = tid; t < nn; t += SC_T) {
                const double ec = (double)Ec[t];
                for (int i = 0; i < m; ++i) v[i] = fma((double)w.Eh[i * nn + t], ec, v[i]);
            }
            sc_sums(v, m, sm);
            if (tid < m) {
                sm.B[tid][cur] = sm.red[SC_W * SC_DIIS + tid];
                sm.B[cur][tid] = sm.red[SC_W * SC_DIIS + tid];
            }
            __syncthreads();
        }
        // F'_use = sum c_i F'_i (+ level shift (I - P'/2))
        if (m > 1) {
            sc_diis_solve(m, cur, sm);
        } else if (tid == 0) {
            sm.coef[cur] = 1.0;
        }
        __syncthreads();
        for (long long t = tid; t < nn; t += SC_T) {
            T v = T(0);
            if (m > 1) {
                for (int i = 0; i < m; ++i) v = fma((T)sm.coef[i], w.Fh[i * nn + t], v);
            } else {
                v = Fc[t];
            }
            if (a.level_shift != 0.0) {
                const int mu = (int)(t / n), nu = (int)(t - (long long)mu * n);
                v += (T)a.level_shift * ((mu == nu ? T(1) : T(0)) - T(0.5) * w.Pp[t]);
            }
            w.EA[t] = v;
        }
        __syncthreads();
        if (!sc_eigh<T>(n, o, w.EA, w.Z, w.W, piv, sm)) {
            st.finite = false;
            return;
        }
        // P' = 2 Z Z^T, C_o = X Z, P = 2 C_o C_o^T
        gemm_sym<T>(n, o, T(2), w.Z, o, false, w.Z, o, true, T(0), w.Pp, n, sm);
        gemm<T>(n, o, n, T(1), w.X, n, false, w.Z, o, false, T(0), w.T2, o, sm);
        gemm_sym<T>(n, o, T(2), w.T2, o, false, w.T2, o, true, T(0), w.P, n, sm);
    }
}

__global__ void __launch_bounds__(SC_T, SC_SLOTS_PER_SM) scc_kernel(ScArgs a) {
    __shared__ ScShared sm;
    const int tid = threadIdx.x;
    const ScSlot sl = sc_slot(a, blockIdx.x);
    for (int guard = 0; guard < a.n_sys; ++guard) {
        if (tid == 0) sm.sys_id = atomicAdd(a.next, 1);
        __syncthreads();
        const int q = sm.sys_id;
        __syncthreads();
        if (q >= a.n_sys) break;
        const int id = a.order[q];
        const tincr_scc_system sy = a.sys[id];
        const int n = sy.n_orb, N = sy.n_atoms, o = sy.n_occ;
        const long long nn = (long long)n * n, NN = (long long)N * N;
        const double erep = sc_setup(a, sy, sl, sm);
        const double *p0 = sl.p0;
        for (int mu = tid; mu < n; mu += SC_T) {
            const int A = sm.ao_atom[mu];
            sl.p0[mu] = a.kind_occ[4 * sm.kind[A] + (mu - sm.ao_off[A])];
        }
        ScState st{0, false, 0.0, true};
        ScWork<double> w = sc_work<double>(sl, nn);
        w.S = sl.S; w.H0 = sl.H0; w.X = sl.X; w.Sh = sl.Sh; w.gam = sl.gam; w.glr = sl.glr;
        // X = S^-1/2 and S^1/2 from the eigenpairs of S (scc_routine.rs:172-174)
        for (long long t = tid; t < nn; t += SC_T) w.EA[t] = w.S[t];
        __syncthreads();
        bool ok = sc_eigh<double>(n, n, w.EA, w.Z, w.Fh, sl.piv, sm);
        if (ok) {
            double bad = 0.0;
            for (int r = tid; r < n; r += SC_T) bad = fmax(bad, sm.w[r] > 0.0 ? 0.0 : 1.0);
            ok = sc_max(bad, sm) == 0.0;
        }
        const double *ps = a.p_start ? a.p_start + sy.mat_off : nullptr;
        auto start_density = [&]() {
            for (long long t = tid; t < nn; t += SC_T) {
                const int mu = (int)(t / n), nu = (int)(t - (long long)mu * n);
                w.P[t] = ps ? ps[t] : (mu == nu ? p0[mu] : 0.0);
            }
            __syncthreads();
        };
        if (ok) {
            for (long long t = tid; t < nn; t += SC_T) {
                const int r = (int)(t % n);
                w.T1[t] = w.Z[t] / sqrt(sm.w[r]);
                w.T2[t] = w.Z[t] * sqrt(sm.w[r]);
            }
            __syncthreads();
            gemm_sym<double>(n, n, 1.0, w.T1, n, false, w.Z, n, true, 0.0, w.X, n, sm);
            gemm_sym<double>(n, n, 1.0, w.T2, n, false, w.Z, n, true, 0.0, w.Sh, n, sm);
            start_density();
        }
        int remaining = a.max_iter, hist = 0;
        if (ok && a.fp32_start) {
            // FP32 phase: its work arrays at the start of the work area, FP32 copies of the inputs
            // after them (the FP64 density in w.P does not overlap either)
            ScWork<float> wf = sc_work<float>(sl, nn);
            float *cp = reinterpret_cast<float *>(sl.work) + (13 + 2 * SC_DIIS) * nn;
            wf.S = cp; wf.H0 = cp + nn; wf.X = cp + 2 * nn; wf.Sh = cp + 3 * nn; wf.gam = cp + 4 * nn;
            wf.glr = wf.gam + NN;
            for (long long t = tid; t < nn; t += SC_T) {
                wf.S[t] = (float)w.S[t];
                wf.H0[t] = (float)w.H0[t];
                wf.X[t] = (float)w.X[t];
                wf.Sh[t] = (float)w.Sh[t];
                wf.P[t] = (float)w.P[t];
            }
            for (long long t = tid; t < NN; t += SC_T) {
                wf.gam[t] = (float)w.gam[t];
                wf.glr[t] = (float)w.glr[t];
            }
            __syncthreads();
            const int lim = remaining < SC_FP32_MAX ? remaining : SC_FP32_MAX;
            ScState sf{0, false, 0.0, true};
            sc_iterate<float>(a, sy, wf, sl.piv, p0, lim, fmax(a.tol, SC_FP32_SWITCH), sf, hist, sm);
            if (sf.finite) {
                // continue in FP64 from the density of the FP32 phase's last diagonalisation, with
                // its DIIS history: E' first (FP64 slots beyond every FP32 array), then F' (FP64
                // slots over the FP32 E' and input copies, which are done with)
                for (long long t = tid; t < nn; t += SC_T) w.P[t] = (double)wf.P[t];
                const int m = hist + 1 < SC_DIIS ? hist + 1 : SC_DIIS;
                for (long long t = tid; t < m * nn; t += SC_T) w.Eh[t] = (double)wf.Eh[t];
                __syncthreads();
                for (long long t = tid; t < m * nn; t += SC_T) w.Fh[t] = (double)wf.Fh[t];
                __syncthreads();
            } else {
                start_density();
                hist = 0;
            }
            st.it = sf.it;
            remaining -= sf.it;
            if (remaining < 1) remaining = 1;
        }
        if (ok) {
            sc_iterate<double>(a, sy, w, sl.piv, p0, remaining, a.tol, st, hist, sm);
            if (!st.finite && a.fp32_start) {
                // the continuation from the FP32 phase failed: max_iter FP64 iterations from the
                // start, with a fresh DIIS history (the iteration count goes on)
                start_density();
                hist = 0;
                st = ScState{st.it, false, 0.0, true};
                sc_iterate<double>(a, sy, w, sl.piv, p0, a.max_iter, a.tol, st, hist, sm);
            }
            ok = st.finite;
        }
        double energy = 0.0;
        if (ok) {
            // orbitals of the last Fock matrix (scc_routine.rs:187-192)
            for (long long t = tid; t < nn; t += SC_T) w.EA[t] = w.Fp[t];
            __syncthreads();
            ok = sc_eigh<double>(n, n, w.EA, w.Z, w.Fh, sl.piv, sm);
        }
        if (ok) {
            double *C = a.orbs + sy.mat_off;
            gemm<double>(n, n, n, 1.0, w.X, n, false, w.Z, n, false, 0.0, C, n, sm);
            gemm_sym<double>(n, o, 2.0, C, n, false, C, n, true, 0.0, w.P, n, sm);
            sc_charges<double>(n, N, w.P, w.S, w.gam, p0, sm);
            // E = sum P o H0 + 1/2 dq gamma dq [- 1/8 (sum (S dP S) o dP o g_lr + sum (S dP) o (dP S) o g_lr)]
            double e1 = 0.0;
            for (long long t = tid; t < nn; t += SC_T) e1 = fma(w.P[t], w.H0[t], e1);
            double e2 = 0.0;
            for (int A = tid; A < N; A += SC_T) e2 += 0.5 * sm.dq[A] * sm.esp[A];
            double e3 = 0.0;
            if (a.lc) {
                double *dP = w.W;
                for (long long t = tid; t < nn; t += SC_T) {
                    const int mu = (int)(t / n), nu = (int)(t - (long long)mu * n);
                    dP[t] = w.P[t] - (mu == nu ? p0[mu] : 0.0);
                }
                __syncthreads();
                gemm<double>(n, n, n, 1.0, w.S, n, false, dP, n, false, 0.0, w.T1, n, sm);
                gemm_sym<double>(n, n, 1.0, w.T1, n, false, w.S, n, false, 0.0, w.T2, n, sm);
                for (long long t = tid; t < nn; t += SC_T) {
                    const int mu = (int)(t / n), nu = (int)(t - (long long)mu * n);
                    const double g = w.glr[(long long)sm.ao_atom[mu] * N + sm.ao_atom[nu]];
                    e3 += g * (w.T2[t] * dP[t] + w.T1[t] * w.T1[(long long)nu * n + mu]);
                }
                e3 *= -0.125;
            }
            energy = sc_sum(e1 + e2 + e3, sm) + erep;
            for (int r = tid; r < n; r += SC_T) a.orbe[sy.orb_off + r] = sm.w[r];
            for (int A = tid; A < N; A += SC_T) a.dq[sy.atom_off + A] = sm.dq[A];
            for (long long t = tid; t < nn; t += SC_T) {
                if (a.p) a.p[sy.mat_off + t] = w.P[t];
                if (a.s_out) a.s_out[sy.mat_off + t] = w.S[t];
                if (a.h0_out) a.h0_out[sy.mat_off + t] = w.H0[t];
                if (a.hcx) a.hcx[sy.mat_off + t] = w.F[t];
            }
        }
        if (tid == 0) {
            a.iterations[id] = st.it;
            a.converged[id] = (ok && st.converged) ? 1 : 0;
            a.residual[id] = ok ? st.errn : NAN;
            a.energy[id] = ok ? energy : NAN;
            a.status[id] = ok ? TINCR_OK : TINCR_NONFINITE;
        }
        __syncthreads();
    }
}

}  // namespace

int Ctx::scc_batch(int n_sys, const tincr_scc_system *sys, const int *kinds, const double *xyz,
                   const double *kind_energy, const tincr_scc_inputs *given, const double *p_start, double r_lr,
                   int flags, double tol, int max_iter,
                   double level_shift, double *orbe, double *orbs, double *p_out, double *dq, double *energy,
                   double *s_out, double *h0_out, double *hcx_out, int *iterations, int *converged,
                   double *residual) {
    if (!params_ready) fail(TINCR_BAD_ARG, "scc_batch: tincr_set_parameters first");
    if (n_sys < 1 || !sys || !kinds || !xyz || !kind_energy || !orbe || !orbs || !energy || !iterations ||
        !converged || !residual)
        fail(TINCR_BAD_ARG, "scc_batch: bad arguments");
    if (!(tol > 0.0) || max_iter < 1 || !std::isfinite(level_shift) || level_shift < 0.0)
        fail(TINCR_BAD_ARG, "scc_batch: tol > 0, max_iter >= 1, level_shift >= 0");
    const bool lc = (flags & TINCR_SCC_LC) != 0;
    if (lc && !(r_lr > 0.0)) fail(TINCR_BAD_ARG, "scc_batch: LC needs r_lr > 0");
    if (flags & ~(TINCR_SCC_LC | TINCR_SCC_SK_EXTRAPOLATE | TINCR_SCC_FP32_START))
        fail(TINCR_BAD_ARG, "scc_batch: unknown flags");
    long long n_at_tot = 0, n_orb_tot = 0, n_mat_tot = 0, n_pair_tot = 0;
    int nmax = 0, Nmax = 0;
    for (int i = 0; i < n_sys; ++i) {
        const tincr_scc_system &s = sys[i];
        if (s.n_atoms < 1 || s.n_atoms > SC_NMAX || s.n_orb < 2 || s.n_orb > SC_NMAX || s.n_occ < 1 ||
            s.n_occ > s.n_orb || s.atom_off < 0 || s.orb_off < 0 || s.mat_off < 0 || s.pair_off < 0)
            fail(TINCR_BAD_ARG, "scc_batch: system " + std::to_string(i) + ": sizes or offsets out of range "
                                "(2 <= n_orb <= 256, 1 <= n_atoms <= 256, 1 <= n_occ <= n_orb)");
        int no = 0;
        for (int A = 0; A < s.n_atoms; ++A) {
            const int k = kinds[s.atom_off + A];
            if (k < 0 || k >= n_kinds) fail(TINCR_BAD_ARG, "scc_batch: atom kind out of range");
            no += h_kind_norb[k];
        }
        if (no != s.n_orb) fail(TINCR_BAD_ARG, "scc_batch: n_orb does not match the atoms' orbitals");
        n_at_tot = std::max(n_at_tot, s.atom_off + s.n_atoms);
        n_orb_tot = std::max(n_orb_tot, s.orb_off + s.n_orb);
        n_mat_tot = std::max(n_mat_tot, s.mat_off + (long long)s.n_orb * s.n_orb);
        n_pair_tot = std::max(n_pair_tot, s.pair_off + (long long)s.n_atoms * s.n_atoms);
        nmax = std::max(nmax, s.n_orb);
        Nmax = std::max(Nmax, s.n_atoms);
    }
    for (long long i = 0; i < 3 * n_at_tot; ++i)
        if (!std::isfinite(xyz[i])) fail(TINCR_NONFINITE, "scc_batch: non-finite coordinates");
    for (int i = 0; i < 4 * n_kinds; ++i)
        if (!std::isfinite(kind_energy[i])) fail(TINCR_NONFINITE, "scc_batch: non-finite orbital energies");
    auto finite = [](const double *x, long long len, const char *what) {
        if (x)
            for (long long i = 0; i < len; ++i)
                if (!std::isfinite(x[i])) fail(TINCR_NONFINITE, std::string("scc_batch: non-finite ") + what);
    };
    const tincr_scc_inputs none{nullptr, nullptr, nullptr, nullptr};
    const tincr_scc_inputs &gv = given ? *given : none;
    finite(p_start, n_mat_tot, "starting density");
    finite(gv.s, n_mat_tot, "S");
    finite(gv.h0, n_mat_tot, "H0");
    finite(gv.gamma, n_pair_tot, "gamma");
    finite(gv.gamma_lr, lc ? n_pair_tot : 0, "gamma_lr");
    // largest systems first
    std::vector<int> order(n_sys);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return sys[x].n_orb > sys[y].n_orb; });
    // device copies
    DevBuf<tincr_scc_system> d_sys(n_sys);
    DevBuf<int> d_order(n_sys), d_kind(n_at_tot), d_ints(4 * (size_t)n_sys + 1);
    DevBuf<double> d_xyz3(3 * n_at_tot), d_ke(4 * (size_t)n_kinds), d_occ(4 * (size_t)n_kinds);
    DevBuf<double> d_ps(p_start ? n_mat_tot : 0), d_orbe(n_orb_tot), d_orbs(n_mat_tot), d_dq(n_at_tot);
    DevBuf<double> d_p(p_out ? n_mat_tot : 0), d_s(s_out ? n_mat_tot : 0), d_h0(h0_out ? n_mat_tot : 0);
    DevBuf<double> d_hcx(hcx_out ? n_mat_tot : 0), d_sc(2 * (size_t)n_sys);
    DevBuf<double> d_sin(gv.s ? n_mat_tot : 0), d_h0in(gv.h0 ? n_mat_tot : 0);
    DevBuf<double> d_gin(gv.gamma ? n_pair_tot : 0), d_glrin(gv.gamma_lr && lc ? n_pair_tot : 0);
    auto up = [&](void *dst, const void *src, size_t bytes) {
        TINCR_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream));
    };
    up(d_sys.p, sys, sizeof(tincr_scc_system) * n_sys);
    up(d_order.p, order.data(), sizeof(int) * n_sys);
    up(d_kind.p, kinds, sizeof(int) * n_at_tot);
    up(d_xyz3.p, xyz, sizeof(double) * 3 * n_at_tot);
    up(d_ke.p, kind_energy, sizeof(double) * 4 * n_kinds);
    up(d_occ.p, h_kind_occ.data(), sizeof(double) * 4 * n_kinds);
    if (p_start) up(d_ps.p, p_start, sizeof(double) * n_mat_tot);
    if (gv.s) up(d_sin.p, gv.s, sizeof(double) * n_mat_tot);
    if (gv.h0) up(d_h0in.p, gv.h0, sizeof(double) * n_mat_tot);
    if (gv.gamma) up(d_gin.p, gv.gamma, sizeof(double) * n_pair_tot);
    if (gv.gamma_lr && lc) up(d_glrin.p, gv.gamma_lr, sizeof(double) * n_pair_tot);
    TINCR_CUDA(cudaMemsetAsync(d_ints.p, 0, sizeof(int) * (4 * (size_t)n_sys + 1), stream));
    // slots
    const long long nn_max = (long long)nmax * nmax, at2_max = (long long)Nmax * Nmax, npad = (nmax + 31) / 32 * 32;
    const long long slot_bytes =
        (sc_slot_doubles(nn_max, at2_max, npad) * (long long)sizeof(double) + nn_max + 255) / 256 * 256;
    const int n_slots = std::min(n_sys, SC_SLOTS_PER_SM * n_sm);
    scc_ws.reserve((size_t)(slot_bytes * n_slots));
    ScArgs a{};
    a.n_sys = n_sys;
    a.sys = d_sys.p;
    a.order = d_order.p;
    a.kind = d_kind.p;
    a.xyz = d_xyz3.p;
    a.p_start = p_start ? d_ps.p : nullptr;
    a.s_in = gv.s ? d_sin.p : nullptr;
    a.h0_in = gv.h0 ? d_h0in.p : nullptr;
    a.gam_in = gv.gamma ? d_gin.p : nullptr;
    a.glr_in = gv.gamma_lr && lc ? d_glrin.p : nullptr;
    a.n_kinds = n_kinds;
    a.n_knots = n_knots;
    a.sk_extrapolate = (flags & TINCR_SCC_SK_EXTRAPOLATE) ? 1 : 0;
    a.kind_z = d_kind_z.p;
    a.kind_norb = d_kind_norb.p;
    a.kind_l = d_kind_l.p;
    a.kind_m = d_kind_m.p;
    a.kind_occ = d_occ.p;
    a.kind_energy = d_ke.p;
    a.sigma = d_sigma.p;
    a.knots = d_knots.p;
    a.coef = d_coef.p;
    a.rep_ntmax = rep_ntmax;
    a.rep_nt = rep_ntmax > 0 ? d_rep_nt.p : nullptr;
    a.rep_knots = d_rep_knots.p;
    a.rep_coef = d_rep_coef.p;
    a.rep_dmax = d_rep_dmax.p;
    a.lc = lc ? 1 : 0;
    a.r_lr = lc ? r_lr : 0.0;
    a.tol = tol;
    a.level_shift = level_shift;
    a.max_iter = max_iter;
    a.fp32_start = (flags & TINCR_SCC_FP32_START) ? 1 : 0;
    a.orbe = d_orbe.p;
    a.orbs = d_orbs.p;
    a.p = p_out ? d_p.p : nullptr;
    a.dq = d_dq.p;
    a.energy = d_sc.p;
    a.residual = d_sc.p + n_sys;
    a.s_out = s_out ? d_s.p : nullptr;
    a.h0_out = h0_out ? d_h0.p : nullptr;
    a.hcx = hcx_out ? d_hcx.p : nullptr;
    a.iterations = d_ints.p;
    a.converged = d_ints.p + n_sys;
    a.status = d_ints.p + 2 * n_sys;
    a.next = d_ints.p + 4 * n_sys;
    a.ws = scc_ws.p;
    a.slot_bytes = slot_bytes;
    a.nn_max = nn_max;
    a.at2_max = at2_max;
    a.npad = npad;
    TINCR_CUDA(cudaEventRecord(ev0, stream));
    g_launches = 0;
    scc_kernel<<<n_slots, SC_T, 0, stream>>>(a);
    count_launch(stream, "scc_kernel");
    check_launch("scc_kernel");
    TINCR_CUDA(cudaEventRecord(ev1, stream));
    auto down = [&](void *dst, const void *src, size_t bytes) {
        TINCR_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, stream));
    };
    std::vector<int> ints(3 * (size_t)n_sys);
    std::vector<double> sc(2 * (size_t)n_sys);
    down(ints.data(), d_ints.p, sizeof(int) * 3 * n_sys);
    down(sc.data(), d_sc.p, sizeof(double) * 2 * n_sys);
    down(orbe, d_orbe.p, sizeof(double) * n_orb_tot);
    down(orbs, d_orbs.p, sizeof(double) * n_mat_tot);
    if (dq) down(dq, d_dq.p, sizeof(double) * n_at_tot);
    if (p_out) down(p_out, d_p.p, sizeof(double) * n_mat_tot);
    if (s_out) down(s_out, d_s.p, sizeof(double) * n_mat_tot);
    if (h0_out) down(h0_out, d_h0.p, sizeof(double) * n_mat_tot);
    if (hcx_out) down(hcx_out, d_hcx.p, sizeof(double) * n_mat_tot);
    sync();
    float ms = 0.f;
    TINCR_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    last_ms = ms;
    last_launches = g_launches;
    int rc = TINCR_OK;
    for (int i = 0; i < n_sys; ++i) {
        iterations[i] = ints[i];
        converged[i] = ints[n_sys + i];
        energy[i] = sc[i];
        residual[i] = sc[n_sys + i];
        if (ints[2 * n_sys + i] == TINCR_NONFINITE) rc = TINCR_NONFINITE;
        else if (!ints[n_sys + i] && rc == TINCR_OK) rc = TINCR_NOT_CONVERGED;
    }
    if (rc == TINCR_NONFINITE) err = "scc_batch: non-finite value in an SCC iteration (see the per-system residual)";
    else if (rc == TINCR_NOT_CONVERGED) err = "scc_batch: some systems did not converge (see converged[])";
    return rc;
}

}  // namespace tincr
