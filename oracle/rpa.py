"""Oracle: RPA / Casida excited states in tincr's dense statement (test infrastructure only, see
oracle/__init__.py).

Follows `build_a_matrix` / `build_b_matrix` (src/excited_states/a_and_b.rs:5-163; singlets, closed
shell: the occupation differences df = 2 make df/2 = 1) and `casida` (src/excited_states/casida.rs:
6-80).  tincr no longer compiles these files; the B builder is pinned through its sum with A, the
(A+B).v known answer of tincr's tests (not_refactored_tests/solver.rs:1478-1634)."""

import numpy as np


def a_b_matrices(omega, q_ov, gamma, q_oo=None, q_vv=None, gamma_lr=None, n_occ=None, n_virt=None):
    """Dense A and B [o*v, o*v] (index i*v + a):
    A = omega + 2 q_ov^T gamma q_ov - K_A^lr, K_A^lr_{ia,jb} = sum_AB q_A^{ij} gamma_lr q_B^{ab} (a_and_b.rs:18-53);
    B = 2 q_ov^T gamma q_ov - K_B^lr, K_B^lr_{ia,jb} = sum_AB q_A^{ib} gamma_lr q_B^{ja} (:97-130)."""
    n_atoms = q_ov.shape[0]
    no, nv = int(n_occ), int(n_virt)
    q = q_ov.reshape(n_atoms, no * nv)
    k2 = 2.0 * q.T @ (gamma @ q)
    a = np.diag(np.asarray(omega).reshape(-1)) + k2
    b = k2.copy()
    if gamma_lr is not None:
        ka = (q_oo.reshape(n_atoms, no * no).T @ (gamma_lr @ q_vv.reshape(n_atoms, nv * nv)))
        a -= ka.reshape(no, no, nv, nv).transpose(0, 2, 1, 3).reshape(no * nv, no * nv)
        qq = q_ov.reshape(n_atoms, no, nv)
        t = np.tensordot(gamma_lr, qq, axes=(1, 0))                   # t[A, k, j] = sum_B g_AB q_B^{kj}
        kb = np.einsum("ail,akj->ijkl", qq, t)                        # sum_A q_A^{il} t[A, k, j]
        b -= kb.reshape(no * nv, no * nv)
    return a, b


def casida(a, b):
    """(A-B)^1/2 (A+B) (A-B)^1/2 F = Omega^2 F (casida.rs:41-63); X+Y = (A-B)^1/2 F / sqrt(Omega),
    X-Y = (A+B)(X+Y) / Omega (:65-71).  The square root is the diagonal one when A-B is diagonal to
    1e-10 (`:46-53`), the symmetric one otherwise.  Returns (Omega ascending, X+Y, X-Y), columns = roots."""
    amb, apb = a - b, a + b
    off = np.linalg.norm(np.diag(np.diag(amb)) - amb)
    if off < 1.0e-10:
        sq = np.diag(np.sqrt(np.diag(amb)))
    else:
        w, u = np.linalg.eigh(amb)
        sq = (u * np.sqrt(w)) @ u.T
    r = sq @ apb @ sq
    om2, f = np.linalg.eigh(r)
    om = np.sqrt(om2)
    xpy = sq @ f / np.sqrt(om)
    xmy = apb @ xpy / om
    return om, xpy, xmy
