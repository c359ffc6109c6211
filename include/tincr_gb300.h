/*
 * tincr_gb300 — C ABI of the GB300 (sm_103a) linear-response excited-state path of tincr.
 *
 * One context owns one GPU and the device-resident state of one molecular system (MO coefficients,
 * overlap, gamma matrices, Davidson subspace).  Every array crossing this boundary is a HOST
 * pointer to C-order (row-major) float64 data unless stated otherwise; the library copies in and
 * out.  Every call returns a tincr_status; tincr_last_error() gives a message for the last failure.
 *
 * Each entry point names the tincr interface it replaces (file:line inside the tincr project).
 * Calls on one context are not thread safe; distinct contexts are independent (the per-instance
 * reentrancy that tincr's rayon-parallel `Monomer::run_tda` calls need, src/fmo/lcmo/basis.rs:462).
 */
#ifndef TINCR_GB300_H
#define TINCR_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tincr_ctx tincr_ctx;

typedef enum {
    TINCR_OK = 0,
    TINCR_NOT_CONVERGED = 1, /* Davidson reached max_iter (DavidsonError, solvers/davidson.rs:28-37) */
    TINCR_NONFINITE = 2,     /* NaN/Inf found in inputs or in an iterate                          */
    TINCR_BAD_ARG = 3,       /* wrong sizes, null pointers, call order                            */
    TINCR_CUDA_ERR = 4,      /* CUDA runtime error                                                 */
    TINCR_NO_DEVICE = 5,     /* no usable sm_103 device                                            */
    TINCR_CG_MAXITER = 6     /* Z-vector CG hit its iteration cap (helpers.rs:1146 stops silently) */
} tincr_status;

/* Arithmetic of the two-electron contractions (Coulomb + long-range exchange) of A.X.
 * Subspace Rayleigh-Ritz, orthogonalisation, residual norms and CG scalars are always FP64.
 * TINCR_PREC_BF16X3: the four GEMMs of the AO-direct product run on tensor cores with every operand
 * split into three BF16 planes (x = hi + mid + lo holds x's FP32 value; six plane products per
 * MMA step) and FP32 accumulation folded every 64 elements of K: products to about 1e-7 relative.
 * The Coulomb diagonals and omega o X stay FP64.  For a residual tolerance below 1e-6 the solve
 * ends with FP64 Davidson iterations started from the mixed Ritz vectors (usually one
 * Rayleigh-Ritz step), so the convergence test and the energies are then those of FP64.
 * Setting the environment variable TINCR_GB300_PLANE_GEMM=mma before tincr_ctx_create selects
 * the warp-MMA implementation of the single-system plane GEMM instead of tcgen05. */
typedef enum {
    TINCR_PREC_FP64 = 0,      /* plain FP64 drop-in                                             */
    TINCR_PREC_BF16X3 = 1     /* three-plane split-BF16 tensor-core products, FP64 subspace       */
} tincr_precision;

/* ---- context --------------------------------------------------------------------------------- */

/* Create a context on CUDA device `device`.  Fails with TINCR_NO_DEVICE if it is not sm_103. */
int tincr_ctx_create(tincr_ctx **out, int device);
int tincr_ctx_destroy(tincr_ctx *ctx);
const char *tincr_last_error(const tincr_ctx *ctx);
/* Device time (ms, CUDA events) of the last tincr_tda_solve / tincr_tda_products call and the
 * number of kernels it launched. */
int tincr_last_timing(const tincr_ctx *ctx, double *ms, long long *kernel_launches);

/* Replaces `set_ci_eigenvalues` / `set_ci_coefficients` (src/properties/setter.rs): install
 * excitation energies [n_roots] and CI vectors [n_occ*n_virt, n_roots] computed elsewhere (for
 * example by a caller's own solver) as the roots the gradient of this context works on. */
int tincr_tda_set_states(tincr_ctx *ctx, int n_roots, const double *energies, const double *coefficients);

/* No counterpart in tincr: declare the precision that the installed roots were solved with, which
 * the gradient's contractions then use (tincr_tda_set_states resets it to TINCR_PREC_FP64; a
 * mixed tincr_tda_solve sets TINCR_PREC_BF16X3).  For roots taken from a mixed
 * tincr_tda_solve_batch. */
int tincr_set_precision(tincr_ctx *ctx, int precision);

/* Statistics of the last tincr_tda_solve: A.X products evaluated (tincr's compute_products
 * columns), subspace collapses and the final largest residual norm. */
int tincr_last_solve_stats(const tincr_ctx *ctx, long long *n_products, int *n_collapses, double *max_residual);

/* Per-iteration record of the last tincr_tda_solve (tincr logs the same quantities to stdout in
 * src/excited_states/solvers/davidson.rs:123-143): iteration index within its phase, subspace size,
 * largest residual norm, roots not yet converged and the precision of the phase (a TINCR_PREC_BF16X3
 * solve runs a mixed phase, then, for tolerances below 1e-6, an FP64 phase).  Up to `capacity` records are written to each
 * non-NULL array; *n_steps receives the total count. */
int tincr_davidson_history(const tincr_ctx *ctx, int capacity, int *n_steps, int *iter, int *n_sub,
                           double *max_residual, int *roots_left, int *precision);

/* The k lowest eigenpairs of a symmetric m x m matrix, as the Davidson loop computes them every iteration
 * (the Rayleigh-Ritz step, `eigh(UPLO::Upper)` in src/excited_states/solvers/davidson.rs:93).  Only the
 * upper triangle of `a` (row-major, host memory) is read.  The solver is the context's: the host
 * (default; OpenMP threads) or, when the environment variable TINCR_GB300_SUBSPACE_EIG=cluster was set
 * at context creation, one thread-block cluster of the device if the matrix fits its shared memory
 * (m up to about 600 with 16 CTAs).  w [k] ascending; y [k*m], y[r*m + i] = component i of
 * eigenvector r (unit length); *on_device (may be NULL) receives 1 when the cluster kernel ran.
 * Non-finite input: TINCR_NONFINITE. */
int tincr_subspace_eigh(tincr_ctx *ctx, int m, int k, const double *a, double *w, double *y, int *on_device);

/* C = A B^T (A [M*K], B [N*K], C [M*N], row-major host arrays, 1 <= N <= 32) on the tensor cores with
 * FP64-class accuracy: every row is cut into eight exact 7-bit digits under its own power-of-two bound,
 * the digit products run as bf16 MMAs with exact FP32 sums over 128-element chunks and exact int64
 * sums beyond (the same GEMM as the subspace products of the mixed Davidson).  Non-finite input:
 * TINCR_NONFINITE. */
int tincr_gemm_fp64_tensor(tincr_ctx *ctx, int M, int N, int K, const double *A, const double *B, double *C);

/* Kernel families timed with CUDA events when profiling is on. */
typedef enum {
    TINCR_KF_AO_EXCHANGE = 0,  /* the two n^2 v contractions of the LC exchange (A.X steps 2 and 4) */
    TINCR_KF_AO_TRANSFORM = 1, /* MO<->AO half transforms of A.X (steps 1 and 5)                    */
    TINCR_KF_SUBSPACE = 2,     /* Davidson projections, Ritz vectors, residuals, orthogonalisation  */
    TINCR_KF_GRADIENT = 3,     /* gradient: pairwise-atom derivative kernel and adjoint GEMMs        */
    TINCR_KF_OTHER = 4,        /* Coulomb, packing, transition charges, small kernels              */
    TINCR_KF_HOST = 5,         /* host time of the Davidson subspace eigensolver (not a kernel)      */
    TINCR_KF_EIGEN = 6,        /* the subspace eigensolver on one thread-block cluster               */
    TINCR_KF_DIGITS = 7,       /* FP64-accurate digit GEMMs of the mixed Davidson subspace products  */
    TINCR_KF_COUNT = 8
} tincr_kernel_family;

/* Turn per-family kernel timing on (1) or off (0); turning it on clears the statistics. */
int tincr_set_profiling(tincr_ctx *ctx, int enable);
/* Test hook of the failure path, no counterpart in tincr.  Every mbarrier wait of the tcgen05 plane
 * GEMM gives up after 2 s, records an error code, drains the copies and MMAs it has in flight, frees
 * its TMEM and returns; the next host synchronisation of the call reports TINCR_CUDA_ERR.  This sets
 * the limit of the first wait of the MMA issuer for this context's later launches: 0 gives up at
 * once (the other waits of the CTA keep their 2 s limit and run out in turn), a negative value
 * restores the default. */
int tincr_debug_tc_first_wait(tincr_ctx *ctx, long long limit_ns);
/* Accumulated device ms, launches, algorithmic FLOPs and algorithmic bytes of one family. */
int tincr_kernel_stats(const tincr_ctx *ctx, int family, double *ms, long long *launches, double *flops,
                       double *bytes);

/* ---- transition charges ---------------------------------------------------------------------- */

/* Replaces `trans_charges(n_atoms, atoms, orbs, s, occ_indices, virt_indices)`
 * (src/excited_states/transition_charges.rs:8-98).  Occupied and virtual orbitals are the
 * contiguous MO ranges [occ0, occ0+n_occ) and [virt0, virt0+n_virt).
 *   orbs_per_atom [n_atoms]; C, S [n_orb*n_orb];
 *   q_ov [n_atoms*n_occ*n_virt] (index A*o*v + i*v + a), q_oo [n_atoms*o*o], q_vv [n_atoms*v*v];
 *   any of q_ov/q_oo/q_vv may be NULL when not wanted. */
int tincr_trans_charges(tincr_ctx *ctx, int n_atoms, const int *orbs_per_atom, int n_orb,
                        const double *C, const double *S, int occ0, int n_occ, int virt0, int n_virt,
                        double *q_ov, double *q_oo, double *q_vv);

/* ---- TDA / LC-TDA ------------------------------------------------------------------------------ */

/* Load one system's ground state onto the device: the inputs `System::prepare_tda`
 * (src/excited_states/tda/system.rs:10-52) reads from Properties.
 *   C, S [n_orb*n_orb]; orbe [n_orb]; gamma [n_atoms*n_atoms];
 *   gamma_lr [n_atoms*n_atoms] or NULL for a calculation without long-range correction;
 *   xyz [n_atoms*3] bohr (for transition dipoles, src/excited_states/tda/moments.rs:7-15).
 * The occupied block is MOs [0, n_occ), the virtual block [n_occ, n_occ+n_virt)
 * (src/initialization/system.rs:132-140). */
int tincr_tda_setup(tincr_ctx *ctx, int n_atoms, const int *orbs_per_atom, int n_orb,
                    const double *C, const double *S, const double *orbe, int n_occ, int n_virt,
                    const double *gamma, const double *gamma_lr, const double *xyz);

/* Replaces `DavidsonEngine::compute_products` for a System/Monomer
 * (src/excited_states/solvers/mod.rs:280-369, :59-148):
 *   AX = omega o X + 2 q_ov^T gamma q_ov X - K_lr X
 * X and AX are [n_occ*n_virt, k] (column j = trial vector j, tincr's guess layout).  Unlike the
 * trait, no product cache is kept here: the caller passes exactly the vectors to multiply. */
int tincr_tda_products(tincr_ctx *ctx, int k, const double *X, double *AX, int precision);

/* Replaces `System::run_tda(n_roots, max_iter, tolerance)` (src/excited_states/tda/mod.rs:74-131)
 * with `Davidson::new` (src/excited_states/solvers/davidson.rs:53-185) and `initial_subspace`
 * (solvers/utils.rs:17-26) on the device.
 *   energies [n_roots]; coefficients [n_occ*n_virt, n_roots] (tincr's ci_coefficients layout);
 *   osc [n_roots] oscillator strengths; tr_dip [3*n_roots] (row c = x,y,z component);
 *   q_trans [n_atoms*n_roots] or NULL; iterations: Davidson iterations done.
 * Returns TINCR_NOT_CONVERGED when max_iter is reached (tincr unwraps a DavidsonError). */
int tincr_tda_solve(tincr_ctx *ctx, int n_roots, int max_iter, double tolerance, int precision,
                    double *energies, double *coefficients, double *osc, double *tr_dip,
                    double *q_trans, int *iterations);

/* ---- batched LE / CT TDA (FMO) ------------------------------------------------------------ */

/* One small TDA problem of a batch: an FMO monomer (tincr's Monomer::prepare_tda / run_tda,
 * src/excited_states/tda/monomer.rs:8-53, tda/mod.rs:18-70) or one direction of a charge-transfer
 * pair (PairChargeTransfer::prepare_ct_tda / run_ct_tda, src/excited_states/tda/ct_pair.rs:12-180).
 * A CT pair direction is passed as the dimer: atoms of the hole monomer then of the electron
 * monomer, the dimer overlap S, the dimer gamma / gamma_lr, and c = [C_occ | C_virt] where C_occ
 * holds the hole monomer's occupied MOs (zero on the electron monomer's AOs) and C_virt the
 * electron monomer's virtual MOs (zero on the hole monomer's AOs).  With that c, the Mulliken
 * transition charges of the dimer equal tincr's pair charges (calculate_q_ov, :81-127, with q_oo
 * of the hole and q_vv of the electron monomer), so the same A.X applies. */
typedef struct {
    int n_atoms, n_orb, n_occ, n_virt;
    int n_roots;                 /* 1..6 */
    const int *orbs_per_atom;    /* [n_atoms] */
    const double *c;             /* [n_orb x (n_occ + n_virt)]: occupied MOs, then virtual MOs */
    const double *s;             /* [n_orb x n_orb] */
    const double *orbe;          /* [n_occ + n_virt]: occupied, then virtual orbital energies */
    const double *gamma;         /* [n_atoms x n_atoms] */
    const double *gamma_lr;      /* [n_atoms x n_atoms], NULL without long-range correction */
    const double *xyz;           /* [n_atoms x 3] bohr, for the transition dipoles */
} tincr_tda_instance;

/* Results of one instance; any output pointer may be NULL. */
typedef struct {
    double *energies;            /* [n_roots] */
    double *coefficients;        /* [n_occ*n_virt x n_roots] (tincr's ci_coefficients layout) */
    double *osc;                 /* [n_roots] */
    double *tr_dip;              /* [3 x n_roots] */
    double *q_trans;             /* [n_atoms x n_roots] */
    int iterations;              /* Davidson iterations of this instance */
    int status;                  /* TINCR_OK, TINCR_NOT_CONVERGED or TINCR_NONFINITE */
} tincr_tda_result;

/* Replaces the per-monomer TDA loop of SuperSystem::create_exciton_hamiltonian_new
 * (src/fmo/lcmo/basis.rs:462-465, rayon over monomers) and the CT pair TDAs of
 * create_diab_basis_new (basis.rs:170-238): every instance runs tincr's block Davidson
 * (davidson.rs:53-185, guesses of solvers/utils.rs:17-26) with its own convergence, all on the
 * device in lockstep.  Returns TINCR_OK when every instance converged, otherwise the worst
 * instance status (per-instance status in res[i].status); tincr unwraps a DavidsonError instead. */
int tincr_tda_solve_batch(tincr_ctx *ctx, int n_inst, const tincr_tda_instance *inst, int max_iter,
                          double tolerance, int precision, tincr_tda_result *res);

/* ---- FMO exciton Hamiltonian ------------------------------------------------------------------ */

/* One monomer of the aggregate with its locally excited (LE) roots. */
typedef struct {
    int n_atoms, n_orb, n_occ;       /* atoms; AOs (= MOs); occupied MOs (the first n_occ)          */
    const int *orbs_per_atom;        /* [n_atoms]                                                     */
    const double *c;                 /* [n_orb x n_orb] MO coefficients, columns = MOs                */
    const double *s;                 /* [n_orb x n_orb] AO overlap                                    */
    const double *orbe;              /* [n_orb] orbital energies                                      */
    int n_le;                        /* LE roots of the monomer in the basis                          */
    const double *le_energies;       /* [n_le]                                                        */
    const double *le_coefficients;   /* [n_occ*n_virt x n_le] (tincr's ci_coefficients layout)        */
    const double *le_q_trans;        /* [n_atoms x n_le] transition charges                           */
} tincr_exciton_monomer;

/* A monomer pair that is a real pair (tincr's get_pair_type, src/fmo/pair.rs:35-53) or carries CT
 * states.  Pairs not listed are ESD pairs: Coulomb couplings only, and zero AO overlap (their atoms
 * are farther apart than the Slater-Koster tables reach), so the exchange integrals that need their
 * overlap vanish. */
typedef struct {
    int i, j;                        /* monomers, i < j                                               */
    int real;                        /* 1: real pair (exchange couplings, LCMO Fock block), 0: ESD     */
    const double *s_ij;              /* [n_orb_i x n_orb_j] AO overlap between the two monomers       */
    const double *pair_orbs;         /* real pairs: [n_ij x n_ij] dimer MO coefficients (AOs of i, j) */
    const double *pair_orbe;         /* real pairs: [n_ij] dimer orbital energies                     */
} tincr_exciton_pair;

/* One charge-transfer basis state: root `state` of the pair TDA with the hole on monomer h and the
 * electron on monomer l. */
typedef struct {
    int h, l;
    int state;                       /* root index in this direction's results                        */
    int n_ct;                        /* roots of this direction                                       */
    const double *energies;          /* [n_ct]                                                        */
    const double *coefficients;      /* [n_occ(h)*n_virt(l) x n_ct]                                   */
    const double *q_tr;              /* [(n_atoms(h) + n_atoms(l)) x n_ct], h's atoms first            */
} tincr_exciton_ct;

/* Replaces SuperSystem::create_exciton_hamiltonian_new (src/fmo/lcmo/basis.rs:449-503): the exciton
 * matrix in the diabatic basis (every monomer's LE roots in monomer order, then the CT states as
 * given), with tincr's couplings (exciton_coupling, src/fmo/lcmo/integrals.rs:17-79: le_le, le_ct_new
 * with the LCMO Fock matrix of src/fmo/lcmo/hamiltonian.rs:12-152, ct_ct_new; restricted active space
 * of 10 occupied and 10 virtual orbitals for the LE-CT and CT-CT exchange), then its lowest n_roots
 * roots by tincr's Davidson on the dense matrix (guess from the diagonal, residual tolerance tol).
 * gamma / gamma_lr: [n_atoms x n_atoms] atomwise matrices of the whole aggregate, monomers' atoms in
 * monomer order.  precision: TINCR_PREC_FP64, or TINCR_PREC_BF16X3 (exchange integrals and LCMO GEMMs
 * in FP32; matrix and Davidson in FP64).  Monomers of up to 102 AOs and 40 atoms, with at least 10
 * occupied and 10 virtual orbitals.  h_out ([dim x dim]) and vectors ([dim x n_roots]) may be NULL.
 * Returns TINCR_NOT_CONVERGED when max_iter is reached. */
int tincr_exciton_states(tincr_ctx *ctx, int n_monomers, const tincr_exciton_monomer *monomers, int n_pairs,
                         const tincr_exciton_pair *pairs, int n_ct, const tincr_exciton_ct *ct, int n_atoms,
                         const double *gamma, const double *gamma_lr, int precision, int n_roots, double tol,
                         int max_iter, double *h_out, double *energies, double *vectors, int *iterations);

/* The tile shapes of the batch's mixed-form plane GEMMs, as chosen by the autotuner.  No counterpart
 * in tincr (rayon runs one monomer per thread).  The first TINCR_PREC_BF16X3 batch that contains an
 * instance shape (n_atoms, n_orb, n_occ, n_virt, long-range flag) times the four tile shapes
 * 64x64, 64x32, 32x64 and 32x32 (rows x columns of the output per CTA) for each of its four plane
 * GEMM steps (H = [C_o;SC_o]X, F, G, AX) on that shape's instances and keeps the fastest; later
 * batches reuse the choice (the table lives for the process).  TINCR_GB300_BATCH_TILES=<shape>
 * forces one shape and skips the tuner.  Results do not depend on the shape.
 * Writes up to `capacity` entries: entries[9 i ..] = n_atoms, n_orb, n_occ, n_virt, lc, then the
 * chosen shape index (0-3 in the order above, -1 when the step does not run: F and G without
 * long-range correction) for the four steps; us[16 i + 4 step + shape] (may be NULL) = measured
 * microseconds per repetition of that shape's tiles.  *n_entries = the table's size. */
int tincr_batch_tile_table(const tincr_ctx *ctx, int capacity, int *n_entries, int *entries, double *us);

/* A.X product that allocates no device memory.  No counterpart in tincr: it exists for callers
 * that own all device memory themselves (pool or arena allocators of an MD or FMO driver) or that
 * cannot accept the implicit device synchronisation of cudaMalloc/cudaFree between their kernels.
 * X_dev and AX_dev are caller-owned DEVICE buffers (device or managed memory of the context's GPU;
 * anything else is rejected with TINCR_BAD_ARG) of k trial vectors, vector-major
 * [k][n_occ*n_virt] (element i*n_virt + a of each vector); the operator is the one set by
 * tincr_tda_setup, FP64.  Temporaries live in one file-scope device array of 32 MiB (held by every
 * GPU that loads the library until exit); systems needing more than that per trial vector
 * (8 (4 n v + 3 n) bytes, + 32 n^2 bytes with long-range correction, n = n_orb, v = n_virt) are
 * rejected with TINCR_BAD_ARG.  The first call on a tincr context looks up that array's device
 * address (make it before any stream capture).  The array exists once per CUDA context, so all
 * calls in one CUDA context (normally the device's primary context) share it: calls whose GPU work
 * overlaps race and must be serialised by the caller.  Ordering: the call runs after all work queued
 * before it on the legacy default stream (and so on every blocking stream); writes of X_dev and
 * uses of AX_dev on the caller's non-blocking streams must be complete before the call.
 * Synchronises the context's stream before returning. */
int tincr_tda_products_noalloc(tincr_ctx *ctx, int k, const double *X_dev, double *AX_dev);

/* ---- analytic gradients ---------------------------------------------------------------------- */

typedef enum {
    /* tincr's formulas: Z-vector with the TDA matrix A for LC (mult_av_lc, helpers.rs:1384-1438),
     * Hav for W_ij[Z], same-element SK derivatives with the moving atom as centre 1 (h0_and_s.rs:218) */
    TINCR_GRAD_REFERENCE = 0,
    /* derivative of the energies tincr computes: (A+B) Z-vector and H+[Z] for LC, SK derivatives
     * in the centre order H0 is built with (lower index first for same-element pairs) */
    TINCR_GRAD_EXACT = 1,
    /* flag, OR-ed into either variant: the Slater-Koster splines beyond their grid up to 30 bohr are
     * the boundary polynomial piece (FITPACK splev with ext = 0, which tincr's splev_uniform
     * evaluates there, h0_and_s.rs:110, :215) instead of zero; the caller's S, H0 and SCC must
     * follow the same rule */
    TINCR_GRAD_SK_EXTRAPOLATE = 16
} tincr_grad_variant;

/* Parameter tables for the gradient kernels (the SK splines, gamma and repulsion tincr's
 * SlaterKoster / RepulsivePotential / GammaFunction hold; src/initialization/parameters.rs:127-372).
 *   kind_z [n_kinds] atomic numbers; kind_norb [n_kinds] (1 or 4); kind_l, kind_m [n_kinds*4]
 *   quantum numbers of each orbital (s, p_y, p_z, p_x order); kind_hubbard [n_kinds];
 *   kind_occ [n_kinds*4] reference (neutral atom) occupations per orbital (P0);
 *   sk_knots [n_knots] common FITPACK knot vector of every SK spline;
 *   sk_coef [n_kinds][n_kinds][2 (S, H0)][5 (ss_s, sp_s, ps_s, pp_p, pp_s)][n_knots]: entry (a, b)
 *   has centre 1 of kind a (used for z_a <= z_b), unused integrals zero;
 *   rep_nt [n_kinds*n_kinds], rep_knots / rep_coef [n_kinds*n_kinds*rep_ntmax], rep_dmax
 *   [n_kinds*n_kinds]: repulsive spline per kind pair (both orders filled); may be NULL. */
int tincr_set_parameters(tincr_ctx *ctx, int n_kinds, const int *kind_z, const int *kind_norb,
                         const int *kind_l, const int *kind_m, const double *kind_hubbard,
                         const double *kind_occ, int n_knots, const double *sk_knots,
                         const double *sk_coef, int rep_ntmax, const int *rep_nt,
                         const double *rep_knots, const double *rep_coef, const double *rep_dmax);

/* Replaces `System::ground_state_gradient(true)` (src/gradients/ground_state.rs:12-137) and
 * `System::tda_gradient_lc(state)` / `tda_gradient_nolc(state)` (src/gradients/excited_state.rs:
 * 56-487) for the system of the last tincr_tda_setup and the roots of the last tincr_tda_solve.
 * LC is on when tincr_tda_setup got gamma_lr; r_lr is its long-range radius (bohr).
 *   atom_kind [n_atoms] index into the parameter tables; P [n_orb*n_orb] SCC density matrix;
 *   h_coul_x [n_orb*n_orb] final SCC Hamiltonian (for the energy-weighted density, ground_state.rs:77);
 *   dq [n_atoms] Mulliken charge differences; state: root index;
 *   grad_gs [3*n_atoms] ground-state gradient or NULL; grad_exc [3*n_atoms] gradient of the
 *   excitation energy of `state` or NULL (total S_n gradient = grad_gs + grad_exc);
 *   cg_iterations: Z-vector CG iterations (or NULL).  Returns TINCR_CG_MAXITER when the CG did
 *   not reach r.r <= 1e-19 in 10000 iterations (gradient still written).
 * The two-electron contractions (Z-vector products included) use the precision the roots were
 * solved with: TINCR_PREC_BF16X3 after a mixed tincr_tda_solve, FP64 after an FP64 solve or
 * tincr_tda_set_states.  The CG's convergence test is FP64; a mixed CG that stalls after 200
 * iterations continues in FP64 from its current Z. */
int tincr_gradient(tincr_ctx *ctx, const int *atom_kind, double r_lr, const double *P,
                   const double *h_coul_x, const double *dq, int state, int variant,
                   double *grad_gs, double *grad_exc, int *cg_iterations);

/* ---- RPA / Casida ----------------------------------------------------------------------------- */

/* Replaces tincr's Casida solver (src/excited_states/casida.rs:6-80, with A and B from
 * src/excited_states/a_and_b.rs:5-163: singlets, closed shell) for the system of the last
 * tincr_tda_setup, in FP64: the lowest n_roots of (A-B)^1/2 (A+B) (A-B)^1/2 F = Omega^2 F with
 * A = omega + 2 (ia|jb) - (ij|ab)_lr and B = 2 (ia|jb) - (ib|ja)_lr (Mulliken charges), by a Davidson
 * on the products (A+B) V and (A-B) V (Stratmann, Scuseria, Frisch, J. Chem. Phys. 109, 8218 (1998)).
 * Converged when both residuals (A+B)(X+Y) - Omega (X-Y) and (A-B)(X-Y) - Omega (X+Y) of every root
 * are below tol (2-norm).  tincr's RPA path is not reachable in its current tree (casida.rs and
 * a_and_b.rs are no longer compiled); the gradient that reads X+Y and X-Y is
 * src/gradients/excited_state.rs:489-983.
 * Out: energies [n_roots] Omega; xpy, xmy [ov x n_roots] (or NULL) X+Y and X-Y with
 * (X+Y)^T (X-Y) = 1; osc [n_roots] (or NULL) 2/3 Omega |mu|^2 with mu from the transition charges of
 * X+Y; iterations.  Returns TINCR_NOT_CONVERGED when max_iter is reached. */
int tincr_rpa_solve(tincr_ctx *ctx, int n_roots, int max_iter, double tol, double *energies, double *xpy,
                    double *xmy, double *osc, int *iterations);

/* ---- SCC ground states --------------------------------------------------------------------- */

typedef enum {
    TINCR_SCC_LC = 1,              /* long-range corrected (gamma_lr with radius r_lr)                 */
    TINCR_SCC_SK_EXTRAPOLATE = 2,  /* SK splines beyond their grid: boundary polynomial, not zero      */
    TINCR_SCC_FP32_START = 4       /* FP32 iterations until the commutator is below 1e-5, then FP64    */
} tincr_scc_flags;

/* One system of a batched SCC.  Offsets index the packed arrays of tincr_scc_batch. */
typedef struct {
    int n_atoms;                   /* 1..256                                                          */
    int n_orb;                     /* 2..256: the atoms' orbitals (kind_norb), checked                */
    int n_occ;                     /* doubly occupied orbitals (n_elec / 2; closed shell)             */
    int pad;
    long long atom_off;            /* first atom in kinds[] / dq[] (xyz: 3 * atom_off)                */
    long long orb_off;             /* first orbital energy in orbe[]                                  */
    long long mat_off;             /* first element of the n_orb x n_orb blocks (orbs, P, S, ...)     */
    long long pair_off;            /* first element of the n_atoms x n_atoms blocks (given gammas)    */
} tincr_scc_system;

/* Inputs the caller supplies instead of the ones tincr_scc_batch builds (each may be NULL):
 * packed S / H0 blocks at mat_off, atomwise gamma / gamma_lr blocks at pair_off. */
typedef struct {
    const double *s, *h0, *gamma, *gamma_lr;
} tincr_scc_inputs;

/* Replaces tincr's SCC for many independent systems at once (System::run_scc, src/scc/
 * scc_routine.rs:121-290, with h0_and_s, src/scc/h0_and_s.rs:92-182, the gamma matrices,
 * src/scc/gamma_approximation.rs:75-193, and the LC exchange Hamiltonian, src/scc/helpers.rs:
 * 111-155): FMO monomers and pairs (src/fmo/scc/), displaced geometries of a numerical gradient.
 * Uses the context's parameter tables (tincr_set_parameters, kind indices into them).
 *   kinds [atoms], xyz [3 * atoms] bohr; kind_energy [n_kinds*4] on-site orbital energies (H0 diagonal);
 *   given: S, H0, gamma, gamma_lr supplied by the caller (NULL, or NULL members: built here);
 *   p_start: packed n_orb x n_orb starting densities or NULL (the neutral-atom reference density);
 *   flags: tincr_scc_flags; r_lr: long-range radius with TINCR_SCC_LC;
 *   tol: convergence when the largest element of X^T (F P S - S P F) X is below tol (X = S^-1/2),
 *   tincr's stationary density; DIIS on the Fock matrix; max_iter iterations at most;
 *   level_shift >= 0 adds level_shift (S - S P S / 2) to the matrix that is diagonalised.
 * Out: orbe [orbitals] ascending, orbs [n_orb x n_orb blocks] (column i = orbital i), P (or NULL),
 *   dq [atoms] Mulliken charge differences, energy [n_sys] total SCC energy (electronic + repulsive),
 *   s_out / h0_out / h_coul_x (converged F, the input tincr_gradient takes) or NULL;
 *   iterations, converged (0/1) and residual (commutator of the last iterate) [n_sys].
 * Returns TINCR_NOT_CONVERGED when some system missed tol in max_iter iterations (its outputs are
 * those of the last Fock matrix), TINCR_NONFINITE when an iterate was not finite. */
int tincr_scc_batch(tincr_ctx *ctx, int n_sys, const tincr_scc_system *systems, const int *kinds,
                    const double *xyz, const double *kind_energy, const tincr_scc_inputs *given,
                    const double *p_start, double r_lr,
                    int flags, double tol, int max_iter, double level_shift, double *orbe, double *orbs,
                    double *P, double *dq, double *energy, double *s_out, double *h0_out,
                    double *h_coul_x, int *iterations, int *converged, double *residual);

#ifdef __cplusplus
}
#endif

#endif /* TINCR_GB300_H */
