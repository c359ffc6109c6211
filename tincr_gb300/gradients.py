"""Host-side mirror of tincr's analytic gradients, computed on the GPU through the C ABI.

Mirrors `System::ground_state_gradient(true)` (src/gradients/ground_state.rs:12-137) and
`System::tda_gradient_lc(state)` / `tda_gradient_nolc(state)` (src/gradients/excited_state.rs:56-487):
results are [3N] arrays, index 3*atom + xyz, Hartree/bohr.  The excited-state system must have
been solved (`ExcitedStateSystem.run_tda`) on the same context; `state` indexes its roots.

variant="reference" reproduces tincr's formulas; variant="exact" is the derivative of the
energies tincr computes (it differs for LC-TDA and for same-element Slater-Koster pairs; see
include/tincr_gb300.h).
"""

import numpy as np

from . import _lib
from ._lib import dptr, f64, iptr
from .params import SK_INTEGRALS

VARIANTS = {"reference": _lib.GRAD_REFERENCE, "exact": _lib.GRAD_EXACT}


def parameter_tables(params, numbers):
    """Kind tables for `tincr_set_parameters` from a ParamSet and the atoms' atomic numbers.

    Returns (tables dict, atom_kind [N] int32)."""
    zs = sorted(set(int(z) for z in numbers))
    kind_of = {z: k for k, z in enumerate(zs)}
    nk = len(zs)
    knots = np.ascontiguousarray(params.sk_knots, dtype=np.float64)
    nt = len(knots)
    kind_norb = np.zeros(nk, np.int32)
    kind_l = np.zeros(4 * nk, np.int32)
    kind_m = np.zeros(4 * nk, np.int32)
    hub = np.zeros(nk)
    occ = np.zeros(4 * nk)
    for k, z in enumerate(zs):
        el = params.element(z)
        kind_norb[k] = el.n_orbs
        kind_l[4 * k:4 * k + el.n_orbs] = el.l
        kind_m[4 * k:4 * k + el.n_orbs] = el.m
        hub[k] = el.hubbard
        occ[4 * k:4 * k + el.n_orbs] = el.occ
    coef = np.zeros((nk, nk, 2, len(SK_INTEGRALS), nt))
    for a, za in enumerate(zs):
        for b, zb in enumerate(zs):
            if za > zb:
                continue
            coef[a, b, 0, :, :] = params.sk_coef[(za, zb, "s")][:, :nt]
            coef[a, b, 1, :, :] = params.sk_coef[(za, zb, "h")][:, :nt]
    rep = {}
    for a, za in enumerate(zs):
        for b, zb in enumerate(zs):
            rep[(a, b)] = params.rep[tuple(sorted((za, zb)))]
    ntmax = max(len(t) for t, _, _ in rep.values())
    rep_nt = np.zeros(nk * nk, np.int32)
    rep_t = np.zeros((nk * nk, ntmax))
    rep_c = np.zeros((nk * nk, ntmax))
    rep_d = np.zeros(nk * nk)
    for (a, b), (t, c, dmax) in rep.items():
        i = a * nk + b
        rep_nt[i] = len(t)
        rep_t[i, :len(t)] = t
        rep_c[i, :len(c)] = c
        rep_d[i] = dmax
    tables = dict(n_kinds=nk, kind_z=np.array(zs, np.int32), kind_norb=kind_norb, kind_l=kind_l, kind_m=kind_m,
                  kind_hubbard=hub, kind_occ=occ, knots=knots, coef=np.ascontiguousarray(coef), rep_ntmax=ntmax,
                  rep_nt=rep_nt, rep_knots=rep_t, rep_coef=rep_c, rep_dmax=rep_d)
    atom_kind = np.array([kind_of[int(z)] for z in numbers], np.int32)
    return tables, atom_kind


def set_parameters(ctx, tables):
    t = tables
    ctx.check(ctx.lib.tincr_set_parameters(
        ctx.h, int(t["n_kinds"]), iptr(t["kind_z"]), iptr(t["kind_norb"]), iptr(t["kind_l"]), iptr(t["kind_m"]),
        dptr(t["kind_hubbard"]), dptr(t["kind_occ"]), len(t["knots"]), dptr(t["knots"]), dptr(t["coef"]),
        int(t["rep_ntmax"]), iptr(t["rep_nt"]), dptr(t["rep_knots"]), dptr(t["rep_coef"]), dptr(t["rep_dmax"])))


class GradientSystem:
    """Gradients of a solved `ExcitedStateSystem`.

    sysm: groundstate.System (atomic numbers, parameter set, r_lr); gs: groundstate.GroundState."""

    def __init__(self, es, sysm, gs):
        self.es = es
        self.ctx = es.ctx
        self.sysm = sysm
        self.p = f64(gs.p)
        self.h = f64(gs.h_coul_x)
        self.dq = f64(gs.dq)
        self.tables, self.atom_kind = parameter_tables(sysm.params, sysm.numbers)
        self.r_lr = float(sysm.r_lr) if es.gamma_lr is not None else 0.0
        set_parameters(self.ctx, self.tables)
        self.last_cg_iterations = None

    def _run(self, state, variant, want_gs, want_exc):
        n3 = 3 * self.sysm.n_atoms
        ggs = np.empty(n3) if want_gs else None
        gex = np.empty(n3) if want_exc else None
        it = _lib.C.c_int(0)
        code = VARIANTS[variant]
        if getattr(self.sysm, "sk_tail", "zero") == "extrapolate":   # the ground state's SK tail rule
            code |= _lib.GRAD_SK_EXTRAPOLATE
        rc = self.ctx.lib.tincr_gradient(self.ctx.h, iptr(self.atom_kind), self.r_lr, dptr(self.p), dptr(self.h),
                                         dptr(self.dq), int(state), code, dptr(ggs), dptr(gex), _lib.C.byref(it))
        self.ctx.check(rc, allow=(_lib.OK, _lib.CG_MAXITER))
        self.last_cg_iterations = it.value
        return ggs, gex

    def ground_state_gradient(self, variant="reference"):
        return self._run(0, variant, True, False)[0]

    def tda_gradient(self, state, variant="reference"):
        """Gradient of the excitation energy of `state` (add the ground-state gradient for S_n)."""
        return self._run(state, variant, False, True)[1]

    def both(self, state, variant="reference"):
        return self._run(state, variant, True, True)
