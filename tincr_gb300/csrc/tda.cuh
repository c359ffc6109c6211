// Device context of one molecular system (see tda.cu).
#pragma once

#include <cuda_bf16.h>

#include <vector>

#include "common.cuh"

namespace tincr {

struct DavidsonStep {
    int iter;
    int n_sub;
    double max_residual;
    int roots_left;
    int prec;
};

// Per-kernel-family device timing (CUDA events on the library stream), enabled on request.
struct KernelStats {
    double ms = 0.0;
    long long launches = 0;
    double flops = 0.0;
    double bytes = 0.0;
};

enum Blk { BLK_OCC = 0, BLK_VIRT = 1 };

// Residual tolerances at or above this are met by the mixed (three-plane split-BF16) operator alone;
// tighter tolerances make a TINCR_PREC_BF16X3 solve finish with FP64 Davidson iterations.
constexpr double MIXED_TOL_FLOOR = 1e-6;

struct BatchWork;                      // batched LE / CT TDA workspace (batch.cu)
void release_batch(BatchWork *w);
// entries of the batch tile-shape autotuner's table (9 ints and 16 times each); returns the count
int bp_table_entries(int capacity, int *entries, double *us);

struct Ctx {
    int device = 0;
    int n_sm = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // device address of noalloc.cu's fixed scratch array in this context, looked up by the first
    // tincr_tda_products_noalloc call on the context (nullptr until then)
    double *noalloc_scratch = nullptr;
    std::string err;
    double last_ms = 0.0;
    long long last_launches = 0;
    std::vector<DavidsonStep> last_history;
    long long last_products = 0;
    int last_collapses = 0;
    double last_max_residual = 0.0;

    // profiling
    bool profiling = false;
    struct Pending {
        int family;
        cudaEvent_t a, b;
        double flops, bytes;
    };
    std::vector<Pending> pending;
    std::vector<cudaEvent_t> event_pool;
    KernelStats stats[8];
    int prof_begin(int family);                 // returns slot or -1
    void prof_end(int slot, double flops, double bytes);
    void prof_resolve();                        // after a sync: fold pending events into stats

    // system
    bool ready = false;
    bool lc = false;
    int n_atoms = 0, n_orb = 0, n_occ = 0, n_virt = 0;
    long long ov = 0;
    std::vector<int> h_ao_off;
    std::vector<double> h_xyz, h_omega;
    DevBuf<int> d_ao_off, d_ao_atom;
    DevBuf<double> dC, dSC, d_omega, d_gamma, d_glr_ao;
    DevBuf<double> dLst, dRv, dLsw, dRsw;     // [Co;SCo], [Cv;SCv], [SCo;Co], [SCv;Cv]

    std::vector<double> h_gamma, h_orbe, h_energies;
    int solved_roots = 0;
    DevBuf<double> dS_, d_xyz;

    // parameters for the gradient (SK splines, gamma, repulsion)
    bool params_ready = false;
    int n_kinds = 0, n_knots = 0, rep_ntmax = 0;
    std::vector<int> h_kind_z, h_kind_norb;
    std::vector<double> h_kind_occ;
    DevBuf<int> d_kind_z, d_kind_norb, d_kind_l, d_kind_m, d_rep_nt;
    DevBuf<double> d_sigma, d_knots, d_coef, d_rep_knots, d_rep_coef, d_rep_dmax;
    DevBuf<double> gw, gv, gcg;            // gradient workspaces
    int last_cg_status = TINCR_OK;

    int prec = TINCR_PREC_FP64;           // arithmetic of the contractions in ao_contract
    int solve_prec = TINCR_PREC_FP64;     // precision the current roots were solved with (gradient follows)

    // split-BF16 planes of the mixed-precision contraction (mixed.cu)
    bool planes_ready = false;
    bool use_tc = true;                   // tcgen05 plane GEMM; false: warp-MMA plane GEMM
    DevBuf<__nv_bfloat16> cst[2], cswT[2], mx_bf16;   // three planes each (planes.cuh)
    DevBuf<float> glr32, stk32[2], mx_f32;             // FP32 copies for the plane epilogues
    DevBuf<__nv_bfloat16> mg_bf16;                     // planes of gemm_mixed
    long long mg_key = -1;
    DevBuf<double> mx_f64;
    long long mx_key = -1;
    DevBuf<int> d_tc_err;                 // error word of the tensor-core kernels' bounded waits
    long long tc_first_wait_ns = -1;      // limit of the plane GEMM's first MMA-side wait (-1: the default)
    int *h_tc_err = nullptr;              // pinned copy, refreshed after tensor-core launches, read by sync()
    void tc_err_ensure();                 // allocate and clear d_tc_err
    void tc_err_watch();                  // queue the copy of d_tc_err to h_tc_err (checked at the next sync)

    // product workspace
    DevBuf<double> wsH, wsF, wsG, wsd3, wsd2, wsz;
    // Davidson state
    DevBuf<double> dV, dAV, dR, dRk, dT;
    DevBuf<double> dAp;                   // projected matrix V AV^T (upper triangle, leading dimension = capacity)
    DevBuf<double> eig_U, eig_Z;          // reflection vectors and tridiagonal eigenvectors (eig_cluster.cu)
    DevBuf<int> eig_err;
    bool eig_cluster_on = false;          // subspace eigensolver on a thread-block cluster instead of the host
    // FP64-accurate digit GEMMs for the subspace products of the mixed Davidson (digits.cu)
    bool use_digits = true;
    DevBuf<__nv_bfloat16> dg_V, dg_VT, dg_AVT, dg_B, dg_C;   // basis digits (row, column layouts), operands
    DevBuf<int> dg_eV, dg_eAV, dg_eB, dg_bad;
    DevBuf<double> dg_scale;
    DevBuf<unsigned long long> dg_acc, dg_mx;
    int dg_mmax = 0;
    long long dg_ovp = 0, dg_mpad = 0;
    void dg_reserve(int mmax);
    void dg_add_rows(bool av, int i0, int n, const double *rows);
    void dg_project(int m, int mold, int knew, double *P, int ldp);
    void dg_ritz(int k, int m, const double *Yt, double *R, double *Rk, const double *u);
    void dg_ortho(int kadd, int m, double *T, double *cbuf);
    int dg_check();
    void gemm_f64_digits(int M, int N, int K, const double *A, const double *B, double *C);
    BatchWork *batch = nullptr;
    PinnedBuf ex_pin;                     // staging of the exciton Hamiltonian's large inputs
    DevBuf<unsigned char> scc_ws;         // per-CTA slots of the batched SCC (scc.cu)
    DevBuf<double> rpa_w1, rpa_w2;        // transposed vectors and K' products of the RPA (rpa.cu)

    explicit Ctx(int dev);
    ~Ctx();
    void sync();
    DevBuf<double> norm_partial, gs_part;
    DevBuf<int> gs_state;
    int coop_grid = 0;                    // CTAs of the cooperative Gram-Schmidt launch
    void row_norms(int rows, long long len, const double *A, long long lda, double *out);
    void launch_transpose(int rows, int cols, const double *in, double *out);
    void set_atoms(int n_atoms, const int *orbs_per_atom, int n_orb);
    void upload_mo(int n, const double *C, const double *S);
    int product_chunk() const;

    void trans_charges(int n_atoms, const int *opa, int n, const double *C, const double *S, int occ0, int no,
                       int virt0, int nv, double *q_ov, double *q_oo, double *q_vv);
    void tda_setup(int n_atoms, const int *opa, int n, const double *C, const double *S, const double *orbe, int no,
                   int nv, const double *gamma, const double *gamma_lr, const double *xyz);
    const double *stk(int b) const { return b == BLK_OCC ? dLst.p : dRv.p; }    // [C_B; SC_B]
    const double *swp(int b) const { return b == BLK_OCC ? dLsw.p : dRsw.p; }   // [SC_B; C_B]
    int bsz(int b) const { return b == BLK_OCC ? n_occ : n_virt; }
    void ao_contract(int k, int R, int S, const double *V, int P, int Q, double ax, double ac, double *out,
                     double alpha, double beta, const double *Xomega);
    void prepare_planes();
    void gemm_mixed(bool ta, bool tb, int M, int N, int K, const double *A, int lda, const double *B, int ldb,
                    double *C, int ldc, double alpha, double beta);
    void ao_contract_mixed(int k, int R, int S, const double *V, int P, int Q, double ax, double ac, double *out,
                           double alpha, double beta, const double *Xomega);
    void products_dev(int k, const double *X, double *AX, double *y_out);
    void qtrans_dev(int k, const double *X, double *y_out);
    void qtrans_mixed(int k, const double *X, double *y_out);
    void products(int k, const double *X, double *AX, int precision);
    void set_parameters(int n_kinds, const int *kind_z, const int *kind_norb, const int *kind_l, const int *kind_m,
                        const double *kind_hubbard, const double *kind_occ, int n_knots, const double *knots,
                        const double *coef, int rep_ntmax, const int *rep_nt, const double *rep_knots,
                        const double *rep_coef, const double *rep_dmax);
    void plr_adjoint(const double *v, const double *Y, double scale_p, double scale_q, double *PS, double *QLblk);
    void pv_adjoint(const double *V, const double *Y, double scale, double *PS, double *QGblk);
    int zvector_cg(int variant, const double *R, double *Z, int max_iter, double conv, int *iters);
    int gradient(const int *atom_kind, double r_lr, const double *P, const double *h_coul_x, const double *dq,
                 int state, int variant, double *grad_gs, double *grad_exc, int *cg_iters);
    void set_states(int n_roots, const double *energies, const double *coefficients);
    int solve(int n_roots, int max_iter, double tol, int precision, double *energies, double *coefficients,
              double *osc, double *tr_dip, double *q_trans, int *iterations);
    int davidson(int n_roots, int max_iter, double tol, bool from_ritz, std::vector<double> &u, int *it_out);
    int solve_batch(int n_inst, const tincr_tda_instance *inst, int max_iter, double tol, int precision,
                    tincr_tda_result *res);
    void rpa_products(int k, const double *V, double *P, double *M);
    int rpa_solve(int n_roots, int max_iter, double tol, double *energies, double *xpy, double *xmy, double *osc,
                  int *iterations);
    int scc_batch(int n_sys, const tincr_scc_system *sys, const int *kinds, const double *xyz,
                  const double *kind_energy, const tincr_scc_inputs *given, const double *p_start, double r_lr,
                  int flags, double tol, int max_iter,
                  double level_shift, double *orbe, double *orbs, double *p_out, double *dq, double *energy,
                  double *s_out, double *h0_out, double *hcx_out, int *iterations, int *converged, double *residual);
    int exciton_states(int n_mono, const tincr_exciton_monomer *mono, int n_pairs, const tincr_exciton_pair *pairs,
                       int n_ct, const tincr_exciton_ct *cts, int n_atoms_total, const double *gamma,
                       const double *gamma_lr, int precision, int n_roots, double tol, int max_iter, double *h_out,
                       double *energies, double *vectors, int *iterations);
};

// Lowest k eigenpairs of the m x m matrix P (upper triangle, leading dimension ldp) on one thread-block
// cluster (eig_cluster.cu): w[k] ascending, Y[r * m + i]; *err set on non-finite data.  Returns false
// without launching when the subspace does not fit the cluster's shared memory.
bool eig_cluster(Ctx &c, int m, int k, const double *P, int ldp, double *w, double *Y, int *err);
// host solver (eigen_host.cpp)
bool eigh_lowest_upper(int n, const double *a, int k, double *w, double *y);
// subspace eigenpairs with the context's solver: the host (default) or the cluster kernel when it
// is selected and the matrix fits (tincr_subspace_eigh)
bool subspace_eigh(Ctx &c, int m, int k, const double *a_host, double *w, double *y, int *used_device);

// A.X product with caller-owned device buffers and fixed device scratch (noalloc.cu)
void products_noalloc(Ctx &c, int k, const double *X, double *AX);

}  // namespace tincr
