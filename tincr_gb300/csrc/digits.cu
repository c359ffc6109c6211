// Mixed-precision Davidson subspace products on the tensor cores, FP64-accurate (digits.cuh).
//
// The mixed form keeps the Davidson subspace arithmetic at FP64 accuracy (projection V AV^T, Ritz
// vectors and residuals, orthogonalisation against the basis) but GB300's FP64 pipe (~1.2 TFLOP/s)
// makes those skinny products the bulk of a solve.  Here they run as digit GEMMs:
//   * every basis vector V_i and product AV_i is cut into digits once, when it joins the basis, with
//     its own bound exponent: a row layout [plane][i][x] (the projection and orthogonalisation
//     dots, K = x) and a column layout [plane][x][i] (the Ritz and correction combinations, K = i);
//   * dots  c_ij = V_i . B_j  read both operands' digits, split K over the SMs, add exact int64
//     partial sums with atomics and scale by 2^(E_i + E_j);
//   * combinations  out_r(x) = sum_i V_i(x) Y_ir  use V_i(x) / 2^E_i (all below 1, one bound for the
//     whole column) and fold 2^E_i into the small coefficient matrix Y, whose digits are cut per call.
// The FP64 basis itself is kept (the A.X products, the sequential Gram-Schmidt and the outputs use it).
#include "digits.cuh"
#include "tda.cuh"

namespace tincr {

namespace {

__device__ __forceinline__ unsigned long long abs_bits(double x) {
    return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}

// block-wide maximum of non-negative 64-bit patterns (blockDim.x = 256)
__device__ __forceinline__ unsigned long long block_max_u64(unsigned long long v, unsigned long long *red) {
    for (int off = 16; off; off >>= 1) {
        const unsigned long long o = __shfl_xor_sync(0xffffffffu, v, off);
        v = o > v ? o : v;
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    unsigned long long m = 0;
    for (int w = 0; w < 8; ++w) m = red[w] > m ? red[w] : m;
    __syncthreads();
    return m;
}

// mx[r] = max over k of |src[r][k]| as a bit pattern (atomicMax; mx zeroed), grid (chunks, rows)
__global__ void __launch_bounds__(256) dg_row_max_kernel(long long K, const double *__restrict__ src, long long lds,
                                                        unsigned long long *mx) {
    __shared__ unsigned long long red[8];
    const int r = blockIdx.y;
    unsigned long long v = 0;
    for (long long k = blockIdx.x * 256LL + threadIdx.x; k < K; k += (long long)gridDim.x * 256) {
        const unsigned long long b = abs_bits(src[(long long)r * lds + k]);
        v = b > v ? b : v;
    }
    v = block_max_u64(v, red);
    if (threadIdx.x == 0 && v) atomicMax(mx + r, v);
}

constexpr int DS_K = 64;   // k values per CTA of the split

// Digits of rows r < nr of src (row maxima mx[r] from dg_row_max_kernel), k < K, DS_K values of k per
// CTA: the bound exponents go to E[e0 + r] (CTA 0; *bad on inf/NaN); digits to
//   row layout     element (p, drow + r, k) of `rowop`   (when rowop.p)
//   column layout  element (p, k, dcol + r) of `colop`   (when colop.p; staged through shared memory
//                  so that consecutive threads write consecutive r)
__global__ void __launch_bounds__(256) dg_split_kernel(int nr, long long K, const double *__restrict__ src, long long lds,
                                                      const unsigned long long *__restrict__ mx, int *E, int e0, int *bad,
                                                      DgOperand rowop, int drow, DgOperand colop, int dcol) {
    __shared__ unsigned short sd[DG_PLANES][DS_K][33];
    __shared__ int sE[32];
    if (threadIdx.x < nr) {
        const unsigned long long b = mx[threadIdx.x];
        const bool nonfinite = b >= 0x7FF0000000000000ull;
        sE[threadIdx.x] = nonfinite ? 0 : dg_bound_exp(b);
        if (blockIdx.x == 0) {
            E[e0 + threadIdx.x] = sE[threadIdx.x];
            if (nonfinite) atomicExch(bad, 1);
        }
    }
    __syncthreads();
    unsigned short *o = reinterpret_cast<unsigned short *>(rowop.p);
    unsigned short *oT = reinterpret_cast<unsigned short *>(colop.p);
    const long long k0 = blockIdx.x * (long long)DS_K;
    for (int idx = threadIdx.x; idx < nr * DS_K; idx += 256) {
        const int r = idx / DS_K, kk = idx % DS_K;
        const long long k = k0 + kk;
        unsigned short d[DG_PLANES];
        if (k < K) {
            dg_digits(src[(long long)r * lds + k], sE[r], d);
        } else {
#pragma unroll
            for (int p = 0; p < DG_PLANES; ++p) d[p] = 0;
        }
        if (o && k < K)
#pragma unroll
            for (int p = 0; p < DG_PLANES; ++p) o[dg_off(rowop, p, drow + r, k)] = d[p];
#pragma unroll
        for (int p = 0; p < DG_PLANES; ++p) sd[p][kk][r] = d[p];
    }
    if (!oT) return;   // the same for every thread of the grid
    __syncthreads();
    const int per = DS_K * nr;
    for (int idx = threadIdx.x; idx < DG_PLANES * per; idx += 256) {
        const int p = idx / per, rem = idx % per, kk = rem / nr, r = rem % nr;
        const long long k = k0 + kk;
        if (k < K) oT[dg_off(colop, p, k, dcol + r)] = sd[p][kk][r];
    }
}

// digits of nr <= 32 rows (length K, stride lds) with their bound exponents
static void dg_split_rows(Ctx &c, int nr, long long K, const double *src, long long lds, int *E, int e0,
                          const DgOperand &rowop, int drow, const DgOperand &colop, int dcol) {
    if (nr <= 0) return;
    if (nr > 32) fail(TINCR_BAD_ARG, "dg_split_rows: more than 32 rows");
    TINCR_CUDA(cudaMemsetAsync(c.dg_mx.p, 0, 32 * sizeof(unsigned long long), c.stream));
    const int chunks = (int)std::min<long long>(32, (K + 4095) / 4096);
    dg_row_max_kernel<<<dim3(chunks, nr), 256, 0, c.stream>>>(K, src, lds, c.dg_mx.p);
    count_launch(c.stream, "dg_row_max");
    check_launch("dg_row_max");
    dg_split_kernel<<<ceil_div(K, DS_K), 256, 0, c.stream>>>(nr, K, src, lds, c.dg_mx.p, E, e0, c.dg_bad.p, rowop, drow,
                                                             colop, dcol);
    count_launch(c.stream, "dg_split");
    check_launch("dg_split");
}

}  // namespace

inline long long pad128(long long r) { return (r + 127) / 128 * 128; }
static const DgOperand kNoOperand{nullptr, 0, 0, 0};

namespace {

// Coefficient digits of a combination: Y(r, i) = Y[r * ysr + i * ysi] 2^(Erow[i]) for r < k, i < m,
// cut with one bound per r into the tiled operand out (zero for i >= m and for rows k..31);
// scale[r] = 2^(Eb_r - 63).  One CTA per r < 32.
__global__ void __launch_bounds__(256) dg_comb_b_kernel(int k, int m, const double *__restrict__ Y, long long ysr,
                                                       long long ysi, const int *__restrict__ Erow, DgOperand out,
                                                       double *scale) {
    __shared__ unsigned long long red[8];
    const int r = blockIdx.x;
    unsigned long long mx = 0;
    if (r < k)
        for (int i = threadIdx.x; i < m; i += 256) {
            const unsigned long long b = abs_bits(ldexp(Y[r * ysr + i * ysi], Erow[i]));
            mx = b > mx ? b : mx;
        }
    mx = block_max_u64(mx, red);
    const int E = mx >= 0x7FF0000000000000ull ? 0 : dg_bound_exp(mx);
    unsigned short *o = reinterpret_cast<unsigned short *>(out.p);
    for (long long i = threadIdx.x; i < out.Kpad; i += 256) {
        const double v = (r < k && i < m) ? ldexp(Y[r * ysr + i * ysi], Erow[i]) : 0.0;
        unsigned short d[DG_PLANES];
        dg_digits(v, E, d);
#pragma unroll
        for (int p = 0; p < DG_PLANES; ++p) o[dg_off(out, p, r, i)] = d[p];
    }
    if (threadIdx.x == 0) scale[r] = ldexp(1.0, E - 63);
}

// out[i * ldo + j] = (H 2^28 + L) 2^(Ea[i] + Eb[j] - 63), i < M, j < N
__global__ void dg_finalize_kernel(int M, int N, const unsigned long long *__restrict__ acc, int ldn,
                                   const int *__restrict__ Ea, const int *__restrict__ Eb, double *out, long long ldo) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= M * N) return;
    const int i = t / N, j = t % N;
    const unsigned long long *p = acc + 2 * ((long long)i * ldn + j);
    out[(long long)i * ldo + j] = dg_value((long long)p[0], (long long)p[1], ldexp(1.0, Ea[i] + Eb[j] - 63));
}

}  // namespace

void Ctx::dg_reserve(int mmax) {
    const long long ovp = pad64(ov), mpad = pad64(mmax);
    if (dg_mmax >= mmax && dg_ovp == ovp) return;
    dg_mmax = mmax;
    dg_ovp = ovp;
    dg_mpad = mpad;
    dg_V.alloc((size_t)DG_PLANES * pad128(mmax) * ovp);
    dg_VT.alloc((size_t)DG_PLANES * pad128(ov) * mpad);
    dg_AVT.alloc((size_t)DG_PLANES * pad128(ov) * mpad);
    dg_B.alloc((size_t)DG_PLANES * DG_N * ovp);
    dg_C.alloc((size_t)DG_PLANES * DG_N * mpad);
    dg_eV.alloc(mmax);
    dg_eAV.alloc(mmax);
    dg_eB.alloc(DG_N);
    dg_scale.alloc(DG_N);
    dg_acc.alloc((size_t)mpad * DG_N * 2);
    dg_bad.alloc(1);
    dg_mx.alloc(32);
    // padding (K beyond ov or m, unused rows) stays zero
    TINCR_CUDA(cudaMemsetAsync(dg_V.p, 0, dg_V.n * sizeof(bf16), stream));
    TINCR_CUDA(cudaMemsetAsync(dg_VT.p, 0, dg_VT.n * sizeof(bf16), stream));
    TINCR_CUDA(cudaMemsetAsync(dg_AVT.p, 0, dg_AVT.n * sizeof(bf16), stream));
    TINCR_CUDA(cudaMemsetAsync(dg_B.p, 0, dg_B.n * sizeof(bf16), stream));
    TINCR_CUDA(cudaMemsetAsync(dg_C.p, 0, dg_C.n * sizeof(bf16), stream));
    TINCR_CUDA(cudaMemsetAsync(dg_bad.p, 0, sizeof(int), stream));
    tc_err_ensure();
}

// the tiled digit operands of the basis
static DgOperand opV(const Ctx &c) { return DgOperand{c.dg_V.p, pad128(c.dg_mmax), c.dg_ovp, 7}; }
static DgOperand opVT(const Ctx &c, bool av) { return DgOperand{av ? c.dg_AVT.p : c.dg_VT.p, pad128(c.ov), c.dg_mpad, 7}; }
static DgOperand opB(const Ctx &c) { return DgOperand{c.dg_B.p, DG_N, c.dg_ovp, 5}; }
static DgOperand opC(const Ctx &c) { return DgOperand{c.dg_C.p, DG_N, c.dg_mpad, 5}; }

// rows i0 .. i0+n-1 of V (av = false) or AV (av = true) join the basis: bound exponents and digits;
// AV rows also go to the row-layout B operand (rows 0..n-1) of the next projection
void Ctx::dg_add_rows(bool av, int i0, int n, const double *rows) {
    if (n <= 0) return;
    if (n > DG_N || i0 + n > dg_mmax) fail(TINCR_BAD_ARG, "dg_add_rows: too many rows");
    if (av) {
        dg_split_rows(*this, n, ov, rows, ov, dg_eAV.p, i0, opB(*this), 0, opVT(*this, true), i0);
        TINCR_CUDA(cudaMemcpyAsync(dg_eB.p, dg_eAV.p + i0, n * sizeof(int), cudaMemcpyDeviceToDevice, stream));
    } else {
        dg_split_rows(*this, n, ov, rows, ov, dg_eV.p, i0, opV(*this), i0, opVT(*this, false), i0);
    }
}

// dots A_i . B_j over x (A = V rows 0..m-1, B = dg_B rows 0..n-1) into out[i * ldo + j]
static void dg_dots(Ctx &c, int m, int n, double *out, long long ldo) {
    TINCR_CUDA(cudaMemsetAsync(c.dg_acc.p, 0, (size_t)m * DG_N * 2 * sizeof(unsigned long long), c.stream));
    const int nkb = (int)(c.dg_ovp / DG_K);
    const int n_mt = ceil_div(m, DG_M);
    const int slot = c.prof_begin(TINCR_KF_DIGITS);
    gemm_digits(c.stream, c.n_sm, m, nkb, std::max(1, c.n_sm / n_mt), opV(c), opB(c), 0, DgEpiAtomic{c.dg_acc.p, m, n, DG_N},
                c.d_tc_err.p);
    dg_finalize_kernel<<<ceil_div((long long)m * n, 256), 256, 0, c.stream>>>(m, n, c.dg_acc.p, DG_N, c.dg_eV.p, c.dg_eB.p,
                                                                             out, ldo);
    count_launch(c.stream, "dg_finalize");
    check_launch("dg_finalize");
    // algorithmic bytes: the digit planes of both operands read once and the int64 sums
    c.prof_end(slot, 2.0 * m * (double)n * c.ov, 2.0 * DG_PLANES * (double)(m + DG_N) * c.dg_ovp + 16.0 * m * n);
}

// combination out_r(x) (mode of DgEpiComb) = sum_{i < m} A_i(x) Y(r, i), r < k, A = V (or AV) columns
static void dg_comb(Ctx &c, bool av, int k, int m, const double *Y, long long ysr, long long ysi, double *out, int mode,
                    const double *R, const double *u) {
    dg_comb_b_kernel<<<DG_N, 256, 0, c.stream>>>(k, m, Y, ysr, ysi, av ? c.dg_eAV.p : c.dg_eV.p, opC(c), c.dg_scale.p);
    count_launch(c.stream, "dg_comb_b");
    check_launch("dg_comb_b");
    const int slot = c.prof_begin(TINCR_KF_DIGITS);
    const int nkb = ceil_div(m, DG_K);
    gemm_digits(c.stream, c.n_sm, (int)c.ov, nkb, 1, opVT(c, av), opC(c), 0,
                DgEpiComb{out, c.ov, c.dg_scale.p, (int)c.ov, k, mode, R, u}, c.d_tc_err.p);
    // algorithmic bytes: the digit planes of both operands (K padded to 64) read once and the FP64
    // output written (read as well for the residual and the update)
    c.prof_end(slot, 2.0 * k * (double)m * c.ov,
               2.0 * DG_PLANES * 64.0 * nkb * ((double)c.ov + DG_N) + 8.0 * k * c.ov * (mode ? 2 : 1));
}

void Ctx::dg_project(int m, int mold, int knew, double *P, int ldp) { dg_dots(*this, m, knew, P + mold, ldp); }

void Ctx::dg_ritz(int k, int m, const double *Yt, double *R, double *Rk, const double *u) {
    dg_comb(*this, false, k, m, Yt, m, 1, R, 0, nullptr, nullptr);
    dg_comb(*this, true, k, m, Yt, m, 1, Rk, 1, R, u);
}

void Ctx::dg_ortho(int kadd, int m, double *T, double *cbuf) {
    // T rows: bound exponents and row digits (the B operand of the dots)
    dg_split_rows(*this, kadd, ov, T, ov, dg_eB.p, 0, opB(*this), 0, kNoOperand, 0);
    // c = V T^T [m x kadd];  T -= c^T V
    dg_dots(*this, m, kadd, cbuf, kadd);
    dg_comb(*this, false, kadd, m, cbuf, 1, kadd, T, 2, nullptr, nullptr);
}

// 0 when the digit kernels reported no error; resets the error words
int Ctx::dg_check() {
    int e[2] = {0, 0};
    TINCR_CUDA(cudaMemcpyAsync(&e[0], d_tc_err.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
    TINCR_CUDA(cudaMemcpyAsync(&e[1], dg_bad.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
    sync();
    if (e[0]) {
        TINCR_CUDA(cudaMemsetAsync(d_tc_err.p, 0, sizeof(int), stream));
        fail(TINCR_CUDA_ERR, "digit GEMM: bounded wait expired (code " + std::to_string(e[0]) + ")");
    }
    if (e[1]) {
        TINCR_CUDA(cudaMemsetAsync(dg_bad.p, 0, sizeof(int), stream));
        fail(TINCR_NONFINITE, "non-finite vector in the Davidson basis");
    }
    return 0;
}

// C[M x N] = A[M x K] B[N x K]^T through the digit GEMM (host arrays; N <= 32): the dots form
// (split K, int64 atomics) for the tests of the C ABI.
void Ctx::gemm_f64_digits(int M, int N, int K, const double *A, const double *B, double *C) {
    if (M <= 0 || N <= 0 || N > DG_N || K <= 0) fail(TINCR_BAD_ARG, "gemm_f64_digits: bad sizes");
    const long long Kp = pad64(K);
    DevBuf<double> dA((size_t)M * K), dB((size_t)N * K), dC((size_t)M * N);
    DevBuf<bf16> pa((size_t)DG_PLANES * pad128(M) * Kp), pb((size_t)DG_PLANES * DG_N * Kp);
    DevBuf<int> ea(M), eb(DG_N);
    DevBuf<unsigned long long> acc((size_t)M * DG_N * 2);
    tc_err_ensure();
    if (!dg_bad.p) {
        dg_bad.alloc(1);
        TINCR_CUDA(cudaMemsetAsync(dg_bad.p, 0, sizeof(int), stream));
    }
    if (!dg_mx.p) dg_mx.alloc(32);
    TINCR_CUDA(cudaMemcpyAsync(dA.p, A, (size_t)M * K * sizeof(double), cudaMemcpyHostToDevice, stream));
    TINCR_CUDA(cudaMemcpyAsync(dB.p, B, (size_t)N * K * sizeof(double), cudaMemcpyHostToDevice, stream));
    TINCR_CUDA(cudaMemsetAsync(pa.p, 0, pa.n * sizeof(bf16), stream));
    TINCR_CUDA(cudaMemsetAsync(pb.p, 0, pb.n * sizeof(bf16), stream));
    TINCR_CUDA(cudaMemsetAsync(acc.p, 0, acc.n * sizeof(unsigned long long), stream));
    const DgOperand oa{pa.p, pad128(M), Kp, 7}, ob{pb.p, DG_N, Kp, 5};
    for (int r0 = 0; r0 < M; r0 += DG_N)
        dg_split_rows(*this, std::min(DG_N, M - r0), K, dA.p + (long long)r0 * K, K, ea.p, r0, oa, r0, kNoOperand, 0);
    dg_split_rows(*this, N, K, dB.p, K, eb.p, 0, ob, 0, kNoOperand, 0);
    const int nkb = (int)(Kp / DG_K), n_mt = ceil_div(M, DG_M);
    gemm_digits(stream, n_sm, M, nkb, std::max(1, n_sm / n_mt), oa, ob, 0, DgEpiAtomic{acc.p, M, N, DG_N}, d_tc_err.p);
    dg_finalize_kernel<<<ceil_div((long long)M * N, 256), 256, 0, stream>>>(M, N, acc.p, DG_N, ea.p, eb.p, dC.p, N);
    check_launch("dg_finalize");
    dg_check();
    TINCR_CUDA(cudaMemcpyAsync(C, dC.p, (size_t)M * N * sizeof(double), cudaMemcpyDeviceToHost, stream));
    sync();
}

}  // namespace tincr
