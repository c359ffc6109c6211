// Lowest k eigenpairs of the Davidson subspace matrix on one thread-block cluster (FP64).
//
// Same steps as the host solver eigen_host.cpp:eigh_lowest_upper (Householder tridiagonalisation,
// Sturm-count bisection, inverse iteration, Gram-Schmidt, back-transformation), laid out for a cluster
// of R = 16 (or 8) CTAs that talk through distributed shared memory.  This keeps the projected matrix
// and the Ritz vectors on the device: tincr's Davidson (src/excited_states/solvers/davidson.rs:93,
// `eigh(UPLO::Upper)`) needs the n_roots lowest pairs of an m x m matrix every iteration, m <= 15 n_roots.
//
//  1. Tridiagonalisation.  Row i of the matrix lives on CTA i % R, so every CTA keeps a share of the
//     shrinking trailing block.  Step c needs two cluster barriers: (A) the owners of column c write
//     their entries into every CTA's copy of u together with partial |x|^2 sums; (B) the owners of
//     p = beta K u write p into every copy together with partial u.p sums.  Each CTA then forms
//     q = p - (beta u.p / 2) u itself and updates its rows.  Buffers alternate with the step parity,
//     so a CTA that runs ahead never overwrites data a slower CTA still reads.  Partial sums are added
//     in rank order, so every CTA takes the same branch with the same values.  The reflection vectors
//     go to global memory (U, row c = u_c), where the back-transformation reads them.
//  2. Eigenvalues: one warp per root, 32-point multisection on Sturm counts.  The count is the number
//     of sign changes of the leading principal minors N_i = (d_i - x) N_{i-1} - e_{i-1}^2 N_{i-2}
//     (a division-free recurrence: 3 FP64 operations per row instead of a division), rescaled by a
//     power of two when N_i leaves [2^-400, 2^400].
//  3. Eigenvectors of T: inverse iteration with partial-pivoting LU of T - w I (three solves from the
//     host solver's start vector), one lane per root.  Roots closer than 1e-3 |T| form a cluster that
//     one CTA handles, re-orthogonalising them by Gram-Schmidt (twice) in ascending order (the
//     criterion of LAPACK's dstein); separated roots come out orthogonal to rounding.
//  4. Back-transformation y = H_0 ... H_{m-3} z: one warp per root, reflections read from U.
// Every loop is bounded; a non-finite input or result sets *err.
#include <cooperative_groups.h>

#include <algorithm>

#include "common.cuh"
#include "tda.cuh"

namespace cg = cooperative_groups;

namespace tincr {

namespace {

constexpr int EC_T = 256, EC_W = EC_T / 32, EC_RMAX = 16, EC_KMAX = 64, EC_IIC = 8;

struct EcLayout {
    int rows;                                                        // owned rows per CTA, ceil(m / R)
    size_t region, ub, pb, q, red, d, e, bsq, beta, w, scr, total;   // offsets in doubles
};

// region: the owned rows (rows x m) during the reduction, then the inverse-iteration workspace
// (5 interleaved m x iic arrays + m x iic flag bytes), then one m-vector per warp.
__host__ __device__ inline EcLayout ec_layout(int m, int R, int iic) {
    EcLayout L;
    L.rows = (m + R - 1) / R;
    size_t reg = (size_t)L.rows * m;
    reg = reg > (size_t)EC_W * m ? reg : (size_t)EC_W * m;
    const size_t ii = 5 * (size_t)m * iic + ((size_t)m * iic + 7) / 8;
    reg = reg > ii ? reg : ii;
    size_t o = 0;
    L.region = o; o += reg;
    L.ub = o; o += 2 * (size_t)m;
    L.pb = o; o += 2 * (size_t)m;
    L.q = o; o += m;
    L.red = o; o += 4 * EC_RMAX;
    L.d = o; o += m;
    L.e = o; o += m;
    L.bsq = o; o += m;
    L.beta = o; o += m;
    L.w = o; o += EC_KMAX;
    L.scr = o; o += EC_W;
    L.total = o;
    return L;
}

__device__ __forceinline__ double ec_warp_sum(double v) {
    for (int off = 16; off; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// number of eigenvalues of T (diagonal d, squared off-diagonal bsq) below x
__device__ __forceinline__ int ec_count(const double *d, const double *bsq, int m, double x) {
    double n0 = 1.0, n1 = d[0] - x;
    if (n1 == 0.0) n1 = -0x1p-100;
    int c = __double2hiint(n1) < 0;
    for (int i = 1; i < m; ++i) {
        double n2 = fma(d[i] - x, n1, -(bsq[i - 1] * n0));
        const long long bits = __double_as_longlong(n2);
        if ((bits << 1) == 0) {
            n2 = -0x1p-100 * n1;   // an exact zero: a tiny value of the opposite sign
        } else {
            const int ex = (int)((bits >> 52) & 0x7ff);
            if ((ex > 1023 + 400 || ex < 1023 - 400) && ex < 2047) {
                const double s = __longlong_as_double((long long)(2046 - ex) << 52);   // 2^(1023 - ex)
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

__global__ void __launch_bounds__(EC_T, 1)
eig_cluster_kernel(int m, int k, int iic, const double *__restrict__ P, int ldp, double *__restrict__ w_out,
                   double *__restrict__ Y, double *__restrict__ U, double *__restrict__ Zg, int *__restrict__ err) {
    cg::cluster_group cluster = cg::this_cluster();
    extern __shared__ __align__(16) double sm[];
    const int R = (int)cluster.num_blocks();
    const int me = (int)cluster.block_rank();
    const EcLayout L = ec_layout(m, R, iic);
    const int rows = L.rows;
    double *A = sm + L.region, *ub = sm + L.ub, *pb = sm + L.pb, *qv = sm + L.q, *red = sm + L.red;
    double *dv = sm + L.d, *ev = sm + L.e, *bsq = sm + L.bsq, *bv = sm + L.beta, *wv = sm + L.w, *scr = sm + L.scr;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    bool bad = false;
    for (int t = tid; t < rows * m; t += EC_T) {
        const int li = t / m, j = t - li * m, i = me + R * li;
        double v = 0.0;
        if (i < m) v = i <= j ? P[(size_t)i * ldp + j] : P[(size_t)j * ldp + i];
        if (!isfinite(v)) bad = true;
        A[t] = v;
    }
    if (bad) atomicExch(err, 1);
    cluster.sync();   // every CTA of the cluster runs before any remote shared-memory access

    // ---- 1. tridiagonalisation ----
    for (int c = 0; c + 2 < m; ++c) {
        const int b = c & 1;
        double *u = ub + (size_t)b * m, *p = pb + (size_t)b * m;
        double *ra = red + b * EC_RMAX, *rp = red + (2 + b) * EC_RMAX;
        // (A) column c of the owned rows into every CTA's u; partial |x|^2 over rows >= c + 2; d[c]
        for (int t = tid; t < rows * R; t += EC_T) {
            const int li = t / R, r = t - li * R, i = me + R * li;
            if (i >= c + 1 && i < m) *cluster.map_shared_rank(u + i, r) = A[(size_t)li * m + c];
        }
        if (warp == 0) {
            double s = 0.0;
            for (int li = lane; li < rows; li += 32) {
                const int i = me + R * li;
                if (i >= c + 2 && i < m) {
                    const double x = A[(size_t)li * m + c];
                    s = fma(x, x, s);
                }
            }
            s = ec_warp_sum(s);
            if (lane < R) *cluster.map_shared_rank(ra + me, lane) = s;
        }
        if (c % R == me && warp == 1 && lane < R) *cluster.map_shared_rank(dv + c, lane) = A[(size_t)(c / R) * m + c];
        cluster.sync();
        double s2 = 0.0;
        for (int r = 0; r < R; ++r) s2 += ra[r];
        const double x0 = u[c + 1];
        if (s2 == 0.0) {   // the same on every CTA
            if (tid == 0) {
                bv[c] = 0.0;
                ev[c] = x0;
            }
            continue;
        }
        const double nx = sqrt(x0 * x0 + s2);
        const double alpha = x0 > 0.0 ? -nx : nx;
        const double bet = 1.0 / (alpha * (alpha - x0));
        __syncthreads();   // every thread has read u[c + 1]
        if (tid == 0) {
            u[c + 1] = x0 - alpha;
            bv[c] = bet;
            ev[c] = alpha;
        }
        __syncthreads();
        if (c % R == me)
            for (int j = c + 1 + tid; j < m; j += EC_T) U[(size_t)c * m + j] = u[j];
        // (B) p = beta K u on the owned rows into every CTA's p; partial u.p
        double upw = 0.0;
        for (int li = warp; li < rows; li += EC_W) {
            const int i = me + R * li;
            if (i < c + 1 || i >= m) continue;   // warp-uniform
            const double *row = A + (size_t)li * m;
            double acc = 0.0;
            for (int j = c + 1 + lane; j < m; j += 32) acc = fma(row[j], u[j], acc);
            const double pi = bet * ec_warp_sum(acc);
            if (lane < R) *cluster.map_shared_rank(p + i, lane) = pi;
            upw = fma(pi, u[i], upw);
        }
        if (lane == 0) scr[warp] = upw;
        __syncthreads();
        if (tid < R) {
            double up = 0.0;
            for (int w = 0; w < EC_W; ++w) up += scr[w];
            *cluster.map_shared_rank(rp + me, tid) = up;
        }
        cluster.sync();
        // (C) q = p - K u with K = beta u.p / 2;  rows -= u q^T + q u^T
        double up = 0.0;
        for (int r = 0; r < R; ++r) up += rp[r];
        const double K = 0.5 * bet * up;
        for (int j = c + 1 + tid; j < m; j += EC_T) qv[j] = p[j] - K * u[j];
        __syncthreads();
        for (int li = warp; li < rows; li += EC_W) {
            const int i = me + R * li;
            if (i < c + 1 || i >= m) continue;
            double *row = A + (size_t)li * m;
            const double ui = u[i], qi = qv[i];
            for (int j = c + 1 + lane; j < m; j += 32) row[j] -= ui * qv[j] + qi * u[j];
        }
        __syncthreads();
    }
    // the trailing 2 x 2 block
    if (warp == 0 && lane < R) {
        if (m >= 2 && (m - 2) % R == me) {
            const double *row = A + (size_t)((m - 2) / R) * m;
            *cluster.map_shared_rank(dv + m - 2, lane) = row[m - 2];
            *cluster.map_shared_rank(ev + m - 2, lane) = row[m - 1];
        }
        if ((m - 1) % R == me) *cluster.map_shared_rank(dv + m - 1, lane) = A[(size_t)((m - 1) / R) * m + m - 1];
    }
    if (tid == 0) ev[m - 1] = 0.0;
    __threadfence();
    cluster.sync();

    // ---- 2. eigenvalues by multisection ----
    for (int i = tid; i < m; i += EC_T) bsq[i] = ev[i] * ev[i];
    if (warp == 0) {
        double lo = 1e300, hi = -1e300, emax2 = 0.0;
        for (int i = lane; i < m; i += 32) {
            const double r = fabs(ev[i]) + (i > 0 ? fabs(ev[i - 1]) : 0.0);
            lo = fmin(lo, dv[i] - r);
            hi = fmax(hi, dv[i] + r);
            emax2 = fmax(emax2, ev[i] * ev[i]);
        }
        for (int off = 16; off; off >>= 1) {
            lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, off));
            hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, off));
            emax2 = fmax(emax2, __shfl_xor_sync(0xffffffffu, emax2, off));
        }
        if (lane == 0) {
            scr[0] = lo;
            scr[1] = hi;
            scr[2] = emax2;
        }
    }
    __syncthreads();
    const double eps = 2.220446049250313e-16;
    const double tnorm = fmax(fabs(scr[0]), fabs(scr[1]));
    const double pivmin = 2.2250738585072014e-308 * fmax(1.0, scr[2]);
    const double lo = scr[0] - (2.0 * eps * tnorm + 2.0 * pivmin);
    const double hi = scr[1] + (2.0 * eps * tnorm + 2.0 * pivmin);
    {
        const int r = me + R * warp;
        if (r < k) {
            double a = lo, bb = hi;
            for (int it = 0; it < 64; ++it) {
                if (!(bb - a > 2.0 * eps * fmax(fabs(a), fabs(bb)) + 4.0 * pivmin)) break;   // warp-uniform
                const double h = (bb - a) * (1.0 / 33.0);
                const double x = fma(h, (double)(lane + 1), a);
                const unsigned ball = __ballot_sync(0xffffffffu, ec_count(dv, bsq, m, x) > r);
                if (ball == 0u) {
                    a = __shfl_sync(0xffffffffu, x, 31);
                } else {
                    const int f = __ffs(ball) - 1;
                    const double xf = __shfl_sync(0xffffffffu, x, f);
                    const double xp = __shfl_sync(0xffffffffu, x, f > 0 ? f - 1 : 0);
                    if (f > 0) a = xp;
                    bb = xf;
                }
            }
            if (lane < R) *cluster.map_shared_rank(wv + r, lane) = 0.5 * (a + bb);
        }
    }
    cluster.sync();

    // ---- 3. eigenvectors of T, by clusters of close roots ----
    {
        const double ortol = 1e-3 * tnorm;
        const double tiny = eps * fmax(tnorm, 1e-300);
        int jc = 0;
        for (int r0 = 0; r0 < k; ++jc) {
            int r1 = r0 + 1;
            while (r1 < k && wv[r1] - wv[r1 - 1] <= ortol) ++r1;
            if (jc % R == me && warp == 0) {
                for (int c0 = r0; c0 < r1; c0 += iic) {
                    const int nc = min(iic, r1 - c0);
                    if (lane < nc) {
                        const int r = c0 + lane;
                        const size_t mi = (size_t)m * iic;
                        double *DL = A + lane, *RD = A + mi + lane, *DU = A + 2 * mi + lane, *DU2 = A + 3 * mi + lane;
                        double *Z = A + 4 * mi + lane;
                        unsigned char *F = reinterpret_cast<unsigned char *>(A + 5 * mi) + lane;
                        const double lam = wv[r];
                        double ddc = dv[0] - lam, duc = ev[0];
                        for (int i = 0; i + 1 < m; ++i) {
                            const double dli = ev[i], ddn = dv[i + 1] - lam, dun = ev[i + 1];
                            const size_t o = (size_t)i * iic;
                            if (fabs(ddc) >= fabs(dli)) {
                                if (fabs(ddc) < tiny) ddc = ddc < 0.0 ? -tiny : tiny;
                                const double l = dli / ddc;
                                DL[o] = l;
                                RD[o] = 1.0 / ddc;
                                DU[o] = duc;
                                DU2[o] = 0.0;
                                F[o] = 0;
                                ddc = ddn - l * duc;
                                duc = dun;
                            } else {   // rows i and i + 1 interchanged
                                const double l = ddc / dli;
                                RD[o] = 1.0 / dli;
                                DL[o] = l;
                                DU[o] = ddn;
                                F[o] = 1;
                                ddc = duc - l * ddn;
                                if (i + 2 < m) {
                                    DU2[o] = dun;
                                    duc = -l * dun;
                                } else {
                                    DU2[o] = 0.0;
                                    duc = dun;
                                }
                            }
                        }
                        if (fabs(ddc) < tiny) ddc = ddc < 0.0 ? -tiny : tiny;
                        RD[(size_t)(m - 1) * iic] = 1.0 / ddc;
                        for (int i = 0; i < m; ++i)
                            Z[(size_t)i * iic] = 1.0 + 0.5 * (double)((i * (r + 1) * 7919 + 13 * r) % 97) / 97.0;
                        for (int it = 0; it < 3; ++it) {
                            for (int i = 0; i + 1 < m; ++i) {
                                const size_t o = (size_t)i * iic;
                                double zi = Z[o];
                                double zn = Z[o + iic];
                                if (F[o]) {
                                    const double t = zi;
                                    zi = zn;
                                    zn = t;
                                    Z[o] = zi;
                                }
                                Z[o + iic] = zn - DL[o] * zi;
                            }
                            double nrm = 0.0, z1 = 0.0, z2 = 0.0;
                            for (int i = m - 1; i >= 0; --i) {
                                const size_t o = (size_t)i * iic;
                                double s = Z[o];
                                if (i + 1 < m) s -= DU[o] * z1;
                                if (i + 2 < m) s -= DU2[o] * z2;
                                s *= RD[o];
                                Z[o] = s;
                                nrm = fma(s, s, nrm);
                                z2 = z1;
                                z1 = s;
                            }
                            const double sc = 1.0 / sqrt(nrm);
                            for (int i = 0; i < m; ++i) Z[(size_t)i * iic] *= sc;
                        }
                        for (int i = 0; i < m; ++i) Zg[(size_t)r * m + i] = Z[(size_t)i * iic];
                    }
                    __syncwarp();
                }
                // Gram-Schmidt (twice) within the cluster, ascending
                for (int r = r0 + 1; r < r1; ++r) {
                    double *z = Zg + (size_t)r * m;
                    for (int pass = 0; pass < 2; ++pass)
                        for (int q = r0; q < r; ++q) {
                            const double *y = Zg + (size_t)q * m;
                            double s = 0.0;
                            for (int i = lane; i < m; i += 32) s = fma(y[i], z[i], s);
                            s = ec_warp_sum(s);
                            for (int i = lane; i < m; i += 32) z[i] -= s * y[i];
                            __syncwarp();
                        }
                    double nr = 0.0;
                    for (int i = lane; i < m; i += 32) nr = fma(z[i], z[i], nr);
                    nr = 1.0 / sqrt(ec_warp_sum(nr));
                    for (int i = lane; i < m; i += 32) z[i] *= nr;
                    __syncwarp();
                }
            }
            r0 = r1;
        }
    }
    __threadfence();
    cluster.sync();   // the last cluster barrier: no shared-memory access across CTAs after it

    // ---- 4. back-transformation, one warp per root ----
    {
        const int r = me + R * warp;
        if (r < k) {
            double *y = A + (size_t)warp * m;
            for (int i = lane; i < m; i += 32) y[i] = Zg[(size_t)r * m + i];
            __syncwarp();
            for (int c = m - 3; c >= 0; --c) {
                const double bet = bv[c];
                if (bet == 0.0) continue;
                const double *uc = U + (size_t)c * m;
                double s = 0.0;
                for (int i = c + 1 + lane; i < m; i += 32) s = fma(uc[i], y[i], s);
                s = ec_warp_sum(s) * bet;
                for (int i = c + 1 + lane; i < m; i += 32) y[i] -= s * uc[i];
                __syncwarp();
            }
            bool nf = false;
            for (int i = lane; i < m; i += 32) {
                Y[(size_t)r * m + i] = y[i];
                nf |= !isfinite(y[i]);
            }
            if (lane == 0) {
                w_out[r] = wv[r];
                nf |= !isfinite(wv[r]);
            }
            if (nf) atomicExch(err, 1);
        }
    }
}

struct EcConfig {
    int R = 0;             // cluster size, 0 = not available
    size_t max_smem = 0;
};

EcConfig ec_config(int device) {
    static EcConfig cfg[64];
    static bool done[64] = {};
    if (device < 0 || device >= 64) return EcConfig{};
    if (done[device]) return cfg[device];
    done[device] = true;
    EcConfig c;
    int optin = 0;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device) != cudaSuccess ||
        cudaFuncSetAttribute(eig_cluster_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
        cudaFuncSetAttribute(eig_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin) != cudaSuccess) {
        cudaGetLastError();
        return cfg[device] = c;
    }
    c.max_smem = (size_t)optin;
    for (int R : {EC_RMAX, 8}) {
        cudaLaunchConfig_t lc = {};
        lc.gridDim = dim3(R);
        lc.blockDim = dim3(EC_T);
        lc.dynamicSmemBytes = (size_t)optin;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = R;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        lc.attrs = at;
        lc.numAttrs = 1;
        int nclusters = 0;
        if (cudaOccupancyMaxActiveClusters(&nclusters, eig_cluster_kernel, &lc) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        if (nclusters >= 1) {
            c.R = R;
            break;
        }
    }
    return cfg[device] = c;
}

}  // namespace

// Launch on one cluster.  Returns false (nothing launched) when the cluster form is unavailable or the
// subspace does not fit its shared memory; the caller then uses the host solver.
bool eig_cluster(Ctx &c, int m, int k, const double *P, int ldp, double *w, double *Y, int *err) {
    if (m < 1 || k < 1 || k > m || k > EC_KMAX) return false;
    const EcConfig cfg = ec_config(c.device);
    if (cfg.R == 0) return false;
    const int R = cfg.R;
    if (k > R * EC_W) return false;
    int iic = std::min(EC_IIC, k);
    size_t smem = ec_layout(m, R, iic).total * sizeof(double);
    while (smem > cfg.max_smem && iic > 1) {
        --iic;
        smem = ec_layout(m, R, iic).total * sizeof(double);
    }
    if (smem > cfg.max_smem) return false;
    c.eig_U.reserve((size_t)m * m);
    c.eig_Z.reserve((size_t)k * m);
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3(R);
    lc.blockDim = dim3(EC_T);
    lc.dynamicSmemBytes = smem;
    lc.stream = c.stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = R;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    lc.attrs = at;
    lc.numAttrs = 1;
    const int slot = c.prof_begin(TINCR_KF_EIGEN);
    TINCR_CUDA(cudaLaunchKernelEx(&lc, eig_cluster_kernel, m, k, iic, P, ldp, w, Y, c.eig_U.p, c.eig_Z.p, err));
    count_launch(c.stream, "eig_cluster");
    check_launch("eig_cluster");
    c.prof_end(slot, 4.0 / 3.0 * (double)m * m * m + 4.0 * (double)k * m * m, 8.0 * (double)m * m);
    return true;
}

bool subspace_eigh(Ctx &c, int m, int k, const double *a_host, double *w, double *y, int *used_device) {
    *used_device = 0;
    if (c.eig_cluster_on) {
        DevBuf<double> dA((size_t)m * m), dw(k), dy((size_t)k * m);
        DevBuf<int> derr(1);
        TINCR_CUDA(cudaMemcpyAsync(dA.p, a_host, (size_t)m * m * sizeof(double), cudaMemcpyHostToDevice, c.stream));
        TINCR_CUDA(cudaMemsetAsync(derr.p, 0, sizeof(int), c.stream));
        if (eig_cluster(c, m, k, dA.p, m, dw.p, dy.p, derr.p)) {
            int bad = 0;
            TINCR_CUDA(cudaMemcpyAsync(w, dw.p, k * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
            TINCR_CUDA(cudaMemcpyAsync(y, dy.p, (size_t)k * m * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
            TINCR_CUDA(cudaMemcpyAsync(&bad, derr.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
            c.sync();
            *used_device = 1;
            return bad == 0;
        }
        c.sync();
    }
    return eigh_lowest_upper(m, a_host, k, w, y);
}

}  // namespace tincr
