// Batched TDA over many small independent instances: FMO monomers (locally excited states) and
// charge-transfer pair directions (hole on one monomer, electron on another).
//
// Every instance is a small system in the AO-direct form of tda.cu (a CT pair direction is the
// dimer with the hole monomer's occupied MOs and the electron monomer's virtual MOs, which gives
// tincr's pair transition charges exactly).  All instances step through tincr's block Davidson in
// lockstep on the device: each iteration is a fixed sequence of grouped kernels over static tile
// tables, and each CTA first reads its instance's state, so converged instances drop out without
// any host decision (per-instance convergence masking).  The iteration is captured once as a CUDA
// graph and replayed.
#pragma once

#include "common.cuh"

namespace tincr {

enum BtStatus { BT_RUNNING = 0, BT_CONVERGED = 1, BT_MAXITER = 2, BT_NONFINITE = 3 };

// Static description of one instance; offsets are element offsets into the packed arrays.
struct BtInst {
    int n, o, v, N;          // AOs, occupied, virtual, atoms
    int nr, mmax;            // roots, largest subspace (15 nr, davidson.rs:74)
    int lc;                  // long-range exchange on
    int max_iter;
    long long ov;
    long long off_c;         // C [n x (o+v)], SC [n x (o+v)]
    long long off_s;         // S [n x n]
    long long off_blk;       // [C_o;SC_o] 2n x o | [C_v;SC_v] 2n x v | [SC_o;C_o] 2n x o | [SC_v;C_v] 2n x v
    long long off_glr;       // gamma_lr in the AO basis [n x n]
    long long off_gam;       // gamma [N x N]
    long long off_omega;     // omega [ov]
    long long off_v;         // V, AV [mmax x ov]
    long long off_r;         // R, Rk, T [nr x ov]
    long long off_sub;       // projected matrix [mmax x mmax]
    long long off_h;         // H, G [nr x 2n x v]
    long long off_f;         // F [nr x 4 n^2]
    long long off_d;         // d3, d2, z [3 x nr x n]
    long long off_u;         // Ritz values, residual norms [nr]
    long long off_y;         // transition charges of the roots [nr x N]
    int off_ao;              // ao_off [N + 1]
    int off_aoatom;          // AO -> atom [n]
    // split-BF16 planes of the mixed form (K padded to 32 elements: ko = pad(o), kv = pad(v),
    // k2 = pad(2n)); hi and lo planes share the offsets
    int ko, kv, k2;
    long long off_pc;        // [C_o;SC_o] 2n x ko | [C_v;SC_v] 2n x kv | [SC_v;C_v]^T v x k2 | [SC_o;C_o]^T o x k2
    long long off_pv;        // per slot: X^T v x ko | H 2n x kv | F 2n x k2 | G^T v x k2
    // Block structure of a CT pair direction's dimer: occupied MOs vanish on AOs >= nh and virtual
    // MOs on AOs < nh (0: no such structure).  The mixed form then skips the product blocks that
    // are zero or multiplied by zeros; k5 = pad(n + nh) is the K of the last product step.
    int nh, k5;
};

// Dynamic Davidson state of one instance (davidson.rs:53-185 bookkeeping).
struct BtState {
    int m;            // columns of the guess
    int m_done;       // columns with products
    int dim_sub;      // tincr's dim_sub
    int iter;         // iterations done
    int status;       // BtStatus
    int products;     // A.X products evaluated
    int collapses;
    int first_stop;   // may stop at iteration 0 (FP64 polish started from Ritz vectors)
    double max_res;   // largest residual of the last iteration
};

}  // namespace tincr
