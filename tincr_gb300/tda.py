"""Host-side mirror of tincr's excited-state interface, running on the GPU through the C ABI.

Mirrors `System::prepare_tda` (src/excited_states/tda/system.rs:10-52), the `DavidsonEngine`
trait (src/excited_states/solvers/mod.rs:20-34) and `System::run_tda`
(src/excited_states/tda/mod.rs:74-131), with the same argument meaning and result layouts:
ci_coefficients is [n_occ*n_virt, n_roots], q_trans [n_atoms, n_roots], tr_dipoles [3, n_roots].
A non-converged Davidson raises, like tincr's `.unwrap()` of a `DavidsonError`.
"""

import numpy as np

from . import _lib
from ._lib import dptr, f64, iptr


def trans_charges(ctx, orbs_per_atom, orbs, s, occ_indices, virt_indices):
    """`trans_charges` (src/excited_states/transition_charges.rs:8-98) on the GPU.

    Returns (q_ov [N, o*v], q_oo [N, o*o], q_vv [N, v*v])."""
    opa = np.ascontiguousarray(orbs_per_atom, dtype=np.int32)
    n_atoms = len(opa)
    orbs, s = f64(orbs), f64(s)
    n = orbs.shape[0]
    occ0, no = int(occ_indices[0]), len(occ_indices)
    virt0, nv = int(virt_indices[0]), len(virt_indices)
    q_ov = np.empty((n_atoms, no * nv))
    q_oo = np.empty((n_atoms, no * no))
    q_vv = np.empty((n_atoms, nv * nv))
    ctx.check(ctx.lib.tincr_trans_charges(ctx.h, n_atoms, iptr(opa), n, dptr(orbs), dptr(s), occ0, no, virt0, nv,
                                          dptr(q_ov), dptr(q_oo), dptr(q_vv)))
    return q_ov, q_oo, q_vv


class DavidsonError(RuntimeError):
    """Davidson did not converge (tincr's `DavidsonError`, solvers/davidson.rs:28-37)."""


class ExcitedStateSystem:
    """TDA / LC-TDA of one system on one GPU.

    orbs_per_atom [N], orbs C [n, n], s [n, n], orbe [n], n_occ / n_virt (occupied = first n_occ MOs),
    gamma [N, N], gamma_lr [N, N] or None (no long-range correction), xyz [N, 3] bohr.
    """

    def __init__(self, ctx, orbs_per_atom, orbs, s, orbe, n_occ, n_virt, gamma, gamma_lr, xyz):
        self.ctx = ctx
        self.opa = np.ascontiguousarray(orbs_per_atom, dtype=np.int32)
        self.n_atoms = len(self.opa)
        self.orbs, self.s, self.orbe = f64(orbs), f64(s), f64(orbe)
        self.n_orb = self.orbs.shape[0]
        self.n_occ, self.n_virt = int(n_occ), int(n_virt)
        self.gamma, self.gamma_lr = f64(gamma), f64(gamma_lr)
        self.xyz = f64(xyz)
        self.prepared = False
        self.properties = {}

    @classmethod
    def from_ground_state(cls, ctx, sysm, gs, lc=None):
        lc = sysm.lc if lc is None else lc
        return cls(ctx, sysm.orbs_per_atom, gs.orbs, gs.s, gs.orbe, sysm.n_occ, sysm.n_virt, gs.gamma,
                   gs.gamma_lr if lc else None, sysm.xyz)

    @property
    def dim(self):
        return self.n_occ * self.n_virt

    def prepare_tda(self):
        """Upload C, S, orbital energies and gamma matrices (`prepare_tda`); computes S C,
        omega = e_a - e_i and the AO-basis gamma_lr on the device."""
        c = self.ctx
        c.check(c.lib.tincr_tda_setup(c.h, self.n_atoms, iptr(self.opa), self.n_orb, dptr(self.orbs), dptr(self.s),
                                      dptr(self.orbe), self.n_occ, self.n_virt, dptr(self.gamma),
                                      dptr(self.gamma_lr), dptr(self.xyz)))
        self.prepared = True

    def compute_products(self, x, precision=_lib.PREC_FP64):
        """A.X for the columns of x [o*v, k] (`DavidsonEngine::compute_products`, without the cache)."""
        if not self.prepared:
            self.prepare_tda()
        x = f64(np.atleast_2d(x.T).T if x.ndim == 1 else x)
        out = np.empty_like(x)
        self.ctx.check(self.ctx.lib.tincr_tda_products(self.ctx.h, x.shape[1], dptr(x), dptr(out), int(precision)))
        return out

    def set_states(self, energies, coefficients):
        """Install roots computed elsewhere (`set_ci_eigenvalues` / `set_ci_coefficients`)."""
        if not self.prepared:
            self.prepare_tda()
        e = f64(np.atleast_1d(energies))
        x = f64(coefficients.reshape(self.dim, -1))
        self.ctx.check(self.ctx.lib.tincr_tda_set_states(self.ctx.h, len(e), dptr(e), dptr(x)))
        self.properties.update(ci_eigenvalues=e, ci_coefficients=x)

    def set_precision(self, precision):
        """Precision the installed roots were solved with; the gradient's contractions follow it."""
        self.ctx.check(self.ctx.lib.tincr_set_precision(self.ctx.h, int(precision)))

    def run_tda(self, n_roots, max_iter, tolerance, precision=_lib.PREC_FP64, raise_on_failure=True):
        """`System::run_tda(n_roots, max_iter, tolerance)`; results are stored in `properties`
        (ci_eigenvalues, ci_coefficients, q_trans, tr_dipoles, oscillator_strengths) and returned."""
        if not self.prepared:
            self.prepare_tda()
        n_roots = int(n_roots)
        e = np.empty(n_roots)
        x = np.empty((self.dim, n_roots))
        f = np.empty(n_roots)
        mu = np.empty((3, n_roots))
        qt = np.empty((self.n_atoms, n_roots))
        it = _lib.C.c_int(0)
        rc = self.ctx.lib.tincr_tda_solve(self.ctx.h, n_roots, int(max_iter), float(tolerance), int(precision),
                                          dptr(e), dptr(x), dptr(f), dptr(mu), dptr(qt), _lib.C.byref(it))
        self.ctx.check(rc, allow=(_lib.OK, _lib.NOT_CONVERGED))
        if rc == _lib.NOT_CONVERGED and raise_on_failure:
            raise DavidsonError("Davidson Algorithm did not converge!")
        self.properties.update(ci_eigenvalues=e, ci_coefficients=x, q_trans=qt, tr_dipoles=mu,
                               oscillator_strengths=f, davidson_iterations=it.value,
                               **self.ctx.last_solve_stats())
        return self.properties

    def run_rpa(self, n_roots, max_iter, tolerance, raise_on_failure=True):
        """RPA / Casida excited states (tincr's `casida`, src/excited_states/casida.rs:6-80, solved by
        a Davidson on (A+B) V and (A-B) V, FP64; `tincr_rpa_solve`).  Stores and returns
        rpa_eigenvalues [n_roots], XpY and XmY [dim x n_roots] ((X+Y)^T (X-Y) = 1, tincr's XpY / XmY)
        and rpa_oscillator_strengths."""
        if not self.prepared:
            self.prepare_tda()
        n_roots = int(n_roots)
        e = np.empty(n_roots)
        xpy = np.empty((self.dim, n_roots))
        xmy = np.empty((self.dim, n_roots))
        f = np.empty(n_roots)
        it = _lib.C.c_int(0)
        rc = self.ctx.lib.tincr_rpa_solve(self.ctx.h, n_roots, int(max_iter), float(tolerance), dptr(e), dptr(xpy),
                                          dptr(xmy), dptr(f), _lib.C.byref(it))
        self.ctx.check(rc, allow=(_lib.OK, _lib.NOT_CONVERGED))
        if rc == _lib.NOT_CONVERGED and raise_on_failure:
            raise DavidsonError("RPA Davidson did not converge!")
        self.properties.update(rpa_eigenvalues=e, XpY=xpy, XmY=xmy, rpa_oscillator_strengths=f,
                               rpa_iterations=it.value)
        return self.properties
