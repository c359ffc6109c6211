"""Oracle: transition charges, TDA/LC-TDA product engine, block Davidson, dense TDA, moments.

Test infrastructure only (see oracle/__init__.py).
"""

import numpy as np


def trans_charges(ao_atom_offsets, orbs, s, occ_indices, virt_indices):
    """Mulliken transition charges (`src/excited_states/transition_charges.rs:8-98`).

    q^A_pq = 1/2 sum_{mu in A} (C_mu p (SC)_mu q + C_mu q (SC)_mu p), written as
    q_ov [N, o*v] (index i*v + a), q_oo [N, o*o], q_vv [N, v*v].
    `ao_atom_offsets` is [N+1] (first AO of each atom, then n_orb).
    """
    sc = s @ orbs                                    # `:35`
    o0, o1 = occ_indices[0], occ_indices[-1] + 1
    v0, v1 = virt_indices[0], virt_indices[-1] + 1
    n_atoms = len(ao_atom_offsets) - 1
    no, nv = o1 - o0, v1 - v0
    q_ov = np.zeros((n_atoms, no * nv))
    q_oo = np.zeros((n_atoms, no * no))
    q_vv = np.zeros((n_atoms, nv * nv))
    for a in range(n_atoms):
        mu = slice(ao_atom_offsets[a], ao_atom_offsets[a + 1])
        co, cv = orbs[mu, o0:o1], orbs[mu, v0:v1]
        so, sv = sc[mu, o0:o1], sc[mu, v0:v1]
        q_ov[a] = (0.5 * (co.T @ sv + so.T @ cv)).reshape(-1)      # `:58`
        q_oo[a] = (0.5 * (co.T @ so + so.T @ co)).reshape(-1)      # `:70`
        q_vv[a] = (0.5 * (cv.T @ sv + sv.T @ cv)).reshape(-1)      # `:90`
    return q_ov, q_oo, q_vv


def orbe_differences(orbe_occ, orbe_virt):
    """omega_ia = e_a - e_i, occupied-major (`src/excited_states/utils.rs:8-22`)."""
    return (orbe_virt[None, :] - orbe_occ[:, None]).reshape(-1)


def initial_subspace(diag, dim):
    """Unit vectors on the `dim` smallest diagonal entries (`solvers/utils.rs:17-26`).

    tincr sorts with an unstable sort; ties are broken here by index (stable sort), and the GPU
    path uses the same rule.
    """
    order = np.argsort(diag, kind="stable")
    mtx = np.zeros((len(diag), dim))
    for idx, i in enumerate(order[:dim]):
        mtx[i, idx] = 1.0
    return mtx


class TdaEngine:
    """`DavidsonEngine` for a `System` (`src/excited_states/solvers/mod.rs:278-385`) with its
    `ProductCache` (`excited_states/utils.rs:29-66`)."""

    def __init__(self, omega, q_ov, gamma, q_oo=None, q_vv=None, gamma_lr=None, n_occ=None, n_virt=None):
        self.omega = omega
        self.q_ov = q_ov
        self.gamma = gamma
        self.q_oo = q_oo
        self.q_vv = q_vv
        self.gamma_lr = gamma_lr
        self.n_occ = n_occ
        self.n_virt = n_virt
        self.cache = None
        self.n_products = 0   # number of A.x products evaluated (for statistics)

    def apply(self, x):
        """A.X for the columns of x, no caching (`:307-361`)."""
        fock = self.omega[:, None] * x                                        # `:307-308`
        two_el = 2.0 * self.q_ov.T @ (self.gamma @ (self.q_ov @ x))           # `:311`
        if self.gamma_lr is not None:
            n_atoms = self.gamma.shape[0]
            no, nv = self.n_occ, self.n_virt
            gamma_oo = (self.gamma_lr @ self.q_oo).reshape(n_atoms * no, no)  # `:328-331`
            q_vv_r = self.q_vv.reshape(n_atoms * nv, nv)
            k_x = np.zeros_like(two_el)
            for i in range(x.shape[1]):                                        # `:335-358`
                xi = x[:, i].reshape(no, nv)
                t = (xi @ q_vv_r.T).reshape(no, n_atoms, nv).transpose(1, 0, 2).reshape(n_atoms * no, nv)
                k_x[:, i] = (gamma_oo.T @ t).reshape(-1)
            two_el = two_el - k_x                                              # `:360`
        self.n_products += x.shape[1]
        return fock + two_el

    def compute_products(self, x):
        """Products of the CIS matrix with the subspace vectors; only new columns are computed
        and the cache is reset when the subspace was collapsed (`:282-302`, `:365`)."""
        n_prod = x.shape[1]
        n_old = 0 if self.cache is None else self.cache.shape[1]
        if n_prod <= n_old:
            self.cache = None
            comp = x
        else:
            comp = x[:, n_old:]
        new = self.apply(comp)
        self.cache = new if self.cache is None else np.concatenate([self.cache, new], axis=1)
        return self.cache.copy()

    def precondition(self, r_k, w_k):
        """r / (w - omega) with |denominator| < 1e-4 replaced by 1 (`:373-380`)."""
        denom = w_k - self.omega
        denom = np.where(np.abs(denom) < 1e-4, 1.0, denom)
        return r_k / denom

    def get_size(self):
        return len(self.omega)


def ct_pair_q_ov(ao_off_h, ao_off_l, orbs_h, orbs_l, s_hl, n_occ_h, n_occ_l):
    """Transition charges of a charge-transfer pair, hole on H and electron on L
    (`PairChargeTransfer::calculate_q_ov`, `src/excited_states/tda/ct_pair.rs:81-127`).

    s_hl is the overlap block between H's and L's AOs; returns q_ov [N_H + N_L, o_H * v_L]."""
    occs = orbs_h[:, :n_occ_h]
    virts = orbs_l[:, n_occ_l:]
    s_c_l = s_hl @ virts                 # `:88`
    s_c_h = s_hl.T @ occs                # `:90`
    nh, nl = len(ao_off_h) - 1, len(ao_off_l) - 1
    q = np.zeros((nh + nl, occs.shape[1], virts.shape[1]))
    for a in range(nh):                  # `:104-113`
        mu = slice(ao_off_h[a], ao_off_h[a + 1])
        q[a] = occs[mu].T @ s_c_l[mu]
    for b in range(nl):                  # `:115-124`
        mu = slice(ao_off_l[b], ao_off_l[b + 1])
        q[nh + b] = s_c_h[mu].T @ virts[mu]
    return 0.5 * q.reshape(nh + nl, -1)


class CtEngine(TdaEngine):
    """`DavidsonEngine` for a `PairChargeTransfer` (`src/excited_states/solvers/mod.rs:166-276`):
    the exchange couples q_oo of the hole monomer H with q_vv of the electron monomer L through
    the H x L block of gamma_lr."""

    def __init__(self, omega, q_ov, gamma, q_oo_h, q_vv_l, gamma_lr_hl, n_occ, n_virt):
        super().__init__(omega, q_ov, gamma, q_oo_h, q_vv_l, gamma_lr_hl, n_occ, n_virt)

    def apply(self, x):
        fock = self.omega[:, None] * x                                        # `:198-199`
        two_el = 2.0 * self.q_ov.T @ (self.gamma @ (self.q_ov @ x))           # `:202`
        no, nv = self.n_occ, self.n_virt
        nl = self.gamma_lr.shape[1]
        gamma_oo = (self.gamma_lr.T @ self.q_oo).reshape(nl * no, no)        # `:219-222`
        q_vv_r = self.q_vv.reshape(nl * nv, nv)
        k_x = np.zeros_like(two_el)
        for i in range(x.shape[1]):                                            # `:226-248`
            xi = x[:, i].reshape(no, nv)
            t = (xi @ q_vv_r.T).reshape(no, nl, nv).transpose(1, 0, 2).reshape(nl * no, nv)
            k_x[:, i] = (gamma_oo.T @ t).reshape(-1)
        self.n_products += x.shape[1]
        return fock + two_el - k_x                                             # `:250`


def run_tda_engine(eng, xyz, n_roots, max_iter, tolerance, history=None, reorthogonalize=False):
    """`run_tda` / `run_ct_tda` around an existing engine: Davidson from `initial_subspace`,
    transition charges, Mulliken dipoles, oscillator strengths (ct_pair.rs:129-180)."""
    guess = initial_subspace(eng.omega, n_roots)
    e, x, iters = davidson(eng, guess, n_roots, tolerance, max_iter, history=history,
                           reorthogonalize=reorthogonalize)
    q_trans = eng.q_ov @ x
    mu = mulliken_dipoles(q_trans, xyz)
    return dict(energies=e, coefficients=x, q_trans=q_trans, tr_dipoles=mu, f=oscillator_strength(e, mu),
                iterations=iters, n_products=eng.n_products)


class DavidsonError(RuntimeError):
    """`DavidsonError` (`solvers/davidson.rs:28-37`)."""


def davidson(engine, guess, n_roots, tolerance, max_iter, history=None, reorthogonalize=False):
    """Block Davidson (`src/excited_states/solvers/davidson.rs:53-185`).

    Returns (eigenvalues [n_roots], eigenvectors [dim, n_roots], iterations).

    tincr orthogonalises each correction against the basis with one classical Gram-Schmidt pass
    (`:162-168`).  When a correction lies almost in the span of the basis, one pass leaves it with a
    component of order (machine epsilon x its norm / the remainder's norm) inside that span, the
    basis stops being orthonormal, and the Rayleigh-Ritz step can return spurious Ritz values near
    zero (Rayleigh quotients of near-null combinations of nearly dependent columns) with small
    residuals, which pass the convergence test.  `reorthogonalize=True` repeats the pass once
    ("twice is enough"), which keeps the basis orthonormal to rounding; it is not tincr's statement
    and serves to compute converged reference roots where the single pass fails.
    """
    steps = davidson_steps(engine, guess, n_roots, tolerance, max_iter, history=history,
                           reorthogonalize=reorthogonalize)
    while True:
        try:
            next(steps)
        except StopIteration as done:
            return done.value


def davidson_steps(engine, guess, n_roots, tolerance, max_iter, history=None, reorthogonalize=False):
    """`davidson` as a generator: yields the iteration index after every iteration that does not
    end the solve; the generator's return value is (eigenvalues, eigenvectors, iterations).  Lets a
    caller time or interleave the iterations of one solve."""
    dim = engine.get_size()
    guess = np.array(guess, dtype=np.float64)
    dim_sub_origin = guess.shape[1]
    dim_sub = dim_sub_origin
    max_space = 15 * n_roots                                                   # `:74`
    for i in range(max_iter):                                                  # `:83`
        ax = engine.compute_products(guess)                                    # `:86`
        a_proj = guess.T @ ax                                                  # `:89`
        u, v = np.linalg.eigh(a_proj, UPLO="U")                                # `:93`
        u = u[:n_roots]
        v = v[:, :n_roots]
        ritz = guess @ v                                                       # `:101`
        rk = ax @ v - ritz * u[None, :]                                        # `:104`
        errors = np.linalg.norm(rk, axis=0)                                    # `:107`
        roots_cvd = int(np.sum(errors < tolerance))                            # `:115-117`
        roots_lft = n_roots - roots_cvd
        if history is not None:
            history.append(dict(iter=i, n_sub=guess.shape[1], max_res=float(errors.max()),
                                roots_left=roots_lft))
        if roots_lft == 0 and i > 0:                                           # `:121`
            return u.copy(), np.ascontiguousarray(ritz[:, :n_roots]), i + 1
        if dim_sub + roots_lft <= max_space:                                   # `:146`
            add = [engine.precondition(rk[:, idx], u[idx])
                   for idx in range(n_roots) if errors[idx] > tolerance]       # `:150-157`
            dim_sub += roots_lft
            for vec in add:                                                    # `:162-168`
                orth = vec - guess @ (guess.T @ vec)
                if reorthogonalize:
                    orth = orth - guess @ (guess.T @ orth)
                nrm = np.linalg.norm(orth)
                if nrm > 1.0e-8:
                    guess = np.concatenate([guess, (orth / nrm)[:, None]], axis=1)
        else:                                                                  # `:172-176`
            dim_sub = dim_sub_origin
            guess = ritz[:, :dim_sub].copy()
        yield i
    raise DavidsonError("Davidson Algorithm did not converge!")


def tda_full_matrix(omega, q_ov, gamma, q_oo=None, q_vv=None, gamma_lr=None, n_occ=None, n_virt=None):
    """Dense CIS matrix A = diag(omega) + 2 q_ov^T gamma q_ov - K_lr (`tda/mod.rs:133-215`)."""
    a = np.diag(omega) + 2.0 * q_ov.T @ (gamma @ q_ov)
    if gamma_lr is not None:
        no, nv = n_occ, n_virt
        k = (q_oo.T @ (gamma_lr @ q_vv)).reshape(no, no, nv, nv).transpose(0, 2, 1, 3).reshape(no * nv, no * nv)
        a = a - k
    return a


def mulliken_dipoles(q_trans, xyz):
    """Transition dipoles mu = xyz^T q_trans (`tda/moments.rs:7-15`)."""
    return xyz.T @ q_trans


def oscillator_strength(energies, tr_dipoles):
    """f = 2/3 E |mu|^2 (`tda/moments.rs:17-24`)."""
    return 2.0 / 3.0 * energies * np.einsum("ki,ki->i", tr_dipoles, tr_dipoles)


def run_tda(omega, q_ov, gamma, xyz, n_roots, max_iter, tolerance, q_oo=None, q_vv=None, gamma_lr=None,
            n_occ=None, n_virt=None, history=None, reorthogonalize=False):
    """`System::run_tda` (`src/excited_states/tda/mod.rs:74-131`) without the file output.

    Returns dict(energies, coefficients [o*v, n_roots], q_trans, tr_dipoles, f, iterations, n_products).
    """
    eng = TdaEngine(omega, q_ov, gamma, q_oo, q_vv, gamma_lr, n_occ, n_virt)
    guess = initial_subspace(omega, n_roots)
    e, x, iters = davidson(eng, guess, n_roots, tolerance, max_iter, history=history,
                           reorthogonalize=reorthogonalize)
    q_trans = q_ov @ x
    mu = mulliken_dipoles(q_trans, xyz)
    f = oscillator_strength(e, mu)
    return dict(energies=e, coefficients=x, q_trans=q_trans, tr_dipoles=mu, f=f, iterations=iters,
                n_products=eng.n_products)
