// extern "C" boundary: turns tincr::Error exceptions into tincr_status codes.
#include <cstring>
#include <new>

#include "tda.cuh"

struct tincr_ctx {
    tincr::Ctx *impl = nullptr;
    std::string err;
};

namespace {

template <class F>
int guarded(tincr_ctx *ctx, F &&f) {
    if (!ctx || !ctx->impl) return TINCR_BAD_ARG;
    try {
        TINCR_CUDA(cudaSetDevice(ctx->impl->device));
        ctx->impl->err.clear();
        int rc = f(*ctx->impl);
        // a status returned without an exception carries the message the call left, if any
        ctx->err = rc == TINCR_OK ? std::string() : ctx->impl->err;
        return rc;
    } catch (const tincr::Error &e) {
        ctx->err = e.msg;
        return e.status;
    } catch (const std::bad_alloc &) {
        ctx->err = "host allocation failed";
        return TINCR_BAD_ARG;
    }
}

}  // namespace

extern "C" {

int tincr_ctx_create(tincr_ctx **out, int device) {
    if (!out) return TINCR_BAD_ARG;
    *out = nullptr;
    try {
        auto *c = new tincr_ctx;
        c->impl = new tincr::Ctx(device);
        *out = c;
        return TINCR_OK;
    } catch (const tincr::Error &e) {
        return e.status;
    } catch (...) {
        return TINCR_BAD_ARG;
    }
}

int tincr_ctx_destroy(tincr_ctx *ctx) {
    if (!ctx) return TINCR_BAD_ARG;
    delete ctx->impl;
    delete ctx;
    return TINCR_OK;
}

const char *tincr_last_error(const tincr_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int tincr_last_timing(const tincr_ctx *ctx, double *ms, long long *kernel_launches) {
    if (!ctx || !ctx->impl) return TINCR_BAD_ARG;
    if (ms) *ms = ctx->impl->last_ms;
    if (kernel_launches) *kernel_launches = ctx->impl->last_launches;
    return TINCR_OK;
}

int tincr_tda_set_states(tincr_ctx *ctx, int n_roots, const double *energies, const double *coefficients) {
    return guarded(ctx, [&](tincr::Ctx &c) {
        c.set_states(n_roots, energies, coefficients);
        return TINCR_OK;
    });
}

int tincr_last_solve_stats(const tincr_ctx *ctx, long long *n_products, int *n_collapses, double *max_residual) {
    if (!ctx || !ctx->impl) return TINCR_BAD_ARG;
    if (n_products) *n_products = ctx->impl->last_products;
    if (n_collapses) *n_collapses = ctx->impl->last_collapses;
    if (max_residual) *max_residual = ctx->impl->last_max_residual;
    return TINCR_OK;
}

int tincr_set_precision(tincr_ctx *ctx, int precision) {
    return guarded(ctx, [&](tincr::Ctx &c) {
        if (precision != TINCR_PREC_FP64 && precision != TINCR_PREC_BF16X3)
            tincr::fail(TINCR_BAD_ARG, "set_precision: unknown precision");
        c.solve_prec = precision;
        return TINCR_OK;
    });
}

int tincr_subspace_eigh(tincr_ctx *ctx, int m, int k, const double *a, double *w, double *y, int *on_device) {
    return guarded(ctx, [&](tincr::Ctx &c) {
        if (m < 1 || k < 1 || k > m || !a || !w || !y) tincr::fail(TINCR_BAD_ARG, "subspace_eigh: bad arguments");
        int used = 0;
        if (!tincr::subspace_eigh(c, m, k, a, w, y, &used)) tincr::fail(TINCR_NONFINITE, "subspace_eigh: non-finite data");
        if (on_device) *on_device = used;
        return TINCR_OK;
    });
}

int tincr_gemm_fp64_tensor(tincr_ctx *ctx, int M, int N, int K, const double *A, const double *B, double *C) {
    return guarded(ctx, [&](tincr::Ctx &c) {
        if (!A || !B || !C) tincr::fail(TINCR_BAD_ARG, "gemm_fp64_tensor: null argument");
        c.gemm_f64_digits(M, N, K, A, B, C);
        return TINCR_OK;
    });
}

int tincr_davidson_history(const tincr_ctx *ctx, int capacity, int *n_steps, int *iter, int *n_sub,
                           double *max_residual, int *roots_left, int *precision) {
    if (!ctx || !ctx->impl || capacity < 0) return TINCR_BAD_ARG;
    const auto &h = ctx->impl->last_history;
    if (n_steps) *n_steps = (int)h.size();
    for (int i = 0; i < capacity && i < (int)h.size(); ++i) {
        if (iter) iter[i] = h[i].iter;
        if (n_sub) n_sub[i] = h[i].n_sub;
        if (max_residual) max_residual[i] = h[i].max_residual;
        if (roots_left) roots_left[i] = h[i].roots_left;
        if (precision) precision[i] = h[i].prec;
    }
    return TINCR_OK;
}

int tincr_debug_tc_first_wait(tincr_ctx *ctx, long long limit_ns) {
    return guarded(ctx, [&](tincr::Ctx &c) {
        c.tc_first_wait_ns = limit_ns < 0 ? -1 : limit_ns;
        return TINCR_OK;
    });
}

int tincr_set_profiling(tincr_ctx *ctx, int enable) {
    return guarded(ctx, [&](tincr::Ctx &c) {
        c.sync();
        c.prof_resolve();
        c.profiling = enable != 0;
        if (c.profiling)
            for (auto &s : c.stats) s = tincr::KernelStats{};
        return TINCR_OK;
    });
}

int tincr_kernel_stats(const tincr_ctx *ctx, int family, double *ms, long long *launches, double *flops,
                       double *bytes) {
    if (!ctx || !ctx->impl || family < 0 || family >= TINCR_KF_COUNT) return TINCR_BAD_ARG;
    const tincr::KernelStats &s = ctx->impl->stats[family];
    if (ms) *ms = s.ms;
    if (launches) *launches = s.launches;
    if (flops) *flops = s.flops;
    if (bytes) *bytes = s.bytes;
    return TINCR_OK;
}

int tincr_trans_charges(tincr_ctx *ctx, int n_atoms, const int *orbs_per_atom, int n_orb, const double *C,
                        const double *S, int occ0, int n_occ, int virt0, int n_virt, double *q_ov, double *q_oo,
                        double *q_vv) {
    return guarded(ctx, [&](tincr::Ctx &c) {
        c.trans_charges(n_atoms, orbs_per_atom, n_orb, C, S, occ0, n_occ, virt0, n_virt, q_ov, q_oo, q_vv);
        return TINCR_OK;
    });
}

int tincr_tda_setup(tincr_ctx *ctx, int n_atoms, const int *orbs_per_atom, int n_orb, const double *C,
                    const double *S, const double *orbe, int n_occ, int n_virt, const double *gamma,
                    const double *gamma_lr, const double *xyz) {
    return guarded(ctx, [&](tincr::Ctx &c) {
        c.tda_setup(n_atoms, orbs_per_atom, n_orb, C, S, orbe, n_occ, n_virt, gamma, gamma_lr, xyz);
        return TINCR_OK;
    });
}

int tincr_tda_products(tincr_ctx *ctx, int k, const double *X, double *AX, int precision) {
    return guarded(ctx, [&](tincr::Ctx &c) {
        c.products(k, X, AX, precision);
        return TINCR_OK;
    });
}

int tincr_exciton_states(tincr_ctx *ctx, int n_monomers, const tincr_exciton_monomer *monomers, int n_pairs,
                         const tincr_exciton_pair *pairs, int n_ct, const tincr_exciton_ct *ct, int n_atoms,
                         const double *gamma, const double *gamma_lr, int precision, int n_roots, double tol,
                         int max_iter, double *h_out, double *energies, double *vectors, int *iterations) {
    return guarded(ctx, [&](tincr::Ctx &c) {
        return c.exciton_states(n_monomers, monomers, n_pairs, pairs, n_ct, ct, n_atoms, gamma, gamma_lr, precision,
                                n_roots, tol, max_iter, h_out, energies, vectors, iterations);
    });
}

int tincr_rpa_solve(tincr_ctx *ctx, int n_roots, int max_iter, double tol, double *energies, double *xpy,
                    double *xmy, double *osc, int *iterations) {
    return guarded(ctx, [&](tincr::Ctx &c) { return c.rpa_solve(n_roots, max_iter, tol, energies, xpy, xmy, osc, iterations); });
}

int tincr_scc_batch(tincr_ctx *ctx, int n_sys, const tincr_scc_system *systems, const int *kinds, const double *xyz,
                    const double *kind_energy, const tincr_scc_inputs *given, const double *p_start, double r_lr,
                    int flags, double tol, int max_iter, double level_shift, double *orbe, double *orbs, double *P, double *dq, double *energy,
                    double *s_out, double *h0_out, double *h_coul_x, int *iterations, int *converged,
                    double *residual) {
    return guarded(ctx, [&](tincr::Ctx &c) {
        return c.scc_batch(n_sys, systems, kinds, xyz, kind_energy, given, p_start, r_lr, flags, tol, max_iter, level_shift,
                           orbe, orbs, P, dq, energy, s_out, h0_out, h_coul_x, iterations, converged, residual);
    });
}

int tincr_tda_products_noalloc(tincr_ctx *ctx, int k, const double *X_dev, double *AX_dev) {
    return guarded(ctx, [&](tincr::Ctx &c) {
        tincr::products_noalloc(c, k, X_dev, AX_dev);
        return TINCR_OK;
    });
}

int tincr_tda_solve(tincr_ctx *ctx, int n_roots, int max_iter, double tolerance, int precision, double *energies,
                    double *coefficients, double *osc, double *tr_dip, double *q_trans, int *iterations) {
    return guarded(ctx, [&](tincr::Ctx &c) {
        c.last_history.clear();
        return c.solve(n_roots, max_iter, tolerance, precision, energies, coefficients, osc, tr_dip, q_trans,
                       iterations);
    });
}

int tincr_tda_solve_batch(tincr_ctx *ctx, int n_inst, const tincr_tda_instance *inst, int max_iter, double tolerance,
                          int precision, tincr_tda_result *res) {
    return guarded(ctx, [&](tincr::Ctx &c) { return c.solve_batch(n_inst, inst, max_iter, tolerance, precision, res); });
}

int tincr_batch_tile_table(const tincr_ctx *ctx, int capacity, int *n_entries, int *entries, double *us) {
    if (!ctx || !ctx->impl || capacity < 0 || !n_entries) return TINCR_BAD_ARG;
    *n_entries = tincr::bp_table_entries(capacity, entries, us);
    return TINCR_OK;
}

int tincr_set_parameters(tincr_ctx *ctx, int n_kinds, const int *kind_z, const int *kind_norb, const int *kind_l,
                         const int *kind_m, const double *kind_hubbard, const double *kind_occ, int n_knots,
                         const double *sk_knots, const double *sk_coef, int rep_ntmax, const int *rep_nt,
                         const double *rep_knots, const double *rep_coef, const double *rep_dmax) {
    return guarded(ctx, [&](tincr::Ctx &c) {
        c.set_parameters(n_kinds, kind_z, kind_norb, kind_l, kind_m, kind_hubbard, kind_occ, n_knots, sk_knots, sk_coef,
                         rep_ntmax, rep_nt, rep_knots, rep_coef, rep_dmax);
        return TINCR_OK;
    });
}

int tincr_gradient(tincr_ctx *ctx, const int *atom_kind, double r_lr, const double *P, const double *h_coul_x,
                   const double *dq, int state, int variant, double *grad_gs, double *grad_exc, int *cg_iterations) {
    return guarded(ctx, [&](tincr::Ctx &c) {
        return c.gradient(atom_kind, r_lr, P, h_coul_x, dq, state, variant, grad_gs, grad_exc, cg_iterations);
    });
}

}  // extern "C"
