"""Oracle: ground-state and TDA excited-state analytic gradients in tincr's dense form.

Restates `src/gradients/ground_state.rs:12-137`, `src/gradients/excited_state.rs:11-487` and the
helpers of `src/gradients/helpers.rs` (f_v `:47-80`, f_lr `:130-188`, h_a_nolr `:361-378`,
Hav `:631-831`, repulsive gradient `:843-868`, tda_zvector_no_lc `:1053-1128`, tda_zvector_lc
`:1130-1223`, mult_av_nolc `:1351-1382`, mult_av_lc `:1384-1438`) and the gamma derivatives of
`src/scc/gamma_approximation.rs:126-171`, `:256-282`, `:392-423`.  Every contraction keeps tincr's
reshapes (C order, like ndarray's `into_shape` on standard-layout arrays).

Test infrastructure only (see oracle/__init__.py).
"""

import numpy as np
from scipy.interpolate import splev
from scipy.special import erf

from . import slako

PI_SQRT = 1.7724538509055159


# ----------------------------------------------------------------------------------------------
# gamma derivatives
# ----------------------------------------------------------------------------------------------

def gamma_c(hubbard, r_lr):
    """C_AB of the Gaussian gamma function (`gamma_approximation.rs:29-73`)."""
    sigma = 1.0 / (np.asarray(hubbard) * PI_SQRT)
    return 1.0 / np.sqrt(2.0 * (sigma[:, None] ** 2 + sigma[None, :] ** 2 + 0.5 * r_lr ** 2))


def gamma_gradients_atomwise(xyz, c):
    """dgamma [3N, N, N], filled only at [3i+k, i, j] = e_ij[k] dgamma/dr(r_ij), e_ij = (R_i - R_j)/r
    (`gamma_approximation.rs:256-282`, derivative `:126-137`)."""
    n = len(xyz)
    g1 = np.zeros((3 * n, n, n))
    for i in range(n):
        g1[3 * i:3 * i + 3] = gamma_gradient_rows(i, xyz, c)
    return g1


def gamma_gradient_rows(i, xyz, c):
    """Rows 3i..3i+2 of `gamma_gradients_atomwise`: [3, N, N], nonzero only in row i."""
    n = len(xyz)
    g1 = np.zeros((3, n, n))
    for j in range(n):
        if i == j:
            continue
        rv = xyz[i] - xyz[j]
        r = np.linalg.norm(rv)
        cv = c[i, j]
        dg = 2.0 * cv / PI_SQRT * np.exp(-(cv * r) ** 2) / r - erf(cv * r) / r ** 2
        g1[:, i, j] = rv / r * dg
    return g1


def gamma_gradients_ao(g1, ao_atom):
    """AO expansion [3N, n_orb, n_orb] (`gamma_approximation.rs:425-454`)."""
    n_atoms = g1.shape[1]
    n_orb = len(ao_atom)
    g1_ao = np.zeros((3 * n_atoms, n_orb, n_orb))
    for i in range(n_atoms):
        g1_ao[3 * i:3 * i + 3] = gamma_gradient_ao_rows(i, g1[3 * i:3 * i + 3], ao_atom)
    return g1_ao


def gamma_gradient_ao_rows(i, g1_rows, ao_atom):
    """Rows 3i..3i+2 of `gamma_gradients_ao` from the atomwise rows [3, N, N] of atom i."""
    n_atoms = g1_rows.shape[1]
    n_orb = len(ao_atom)
    out = np.zeros((3, n_orb, n_orb))
    mu = np.where(ao_atom == i)[0]
    for j in range(n_atoms):
        if i == j:
            continue
        nu = np.where(ao_atom == j)[0]
        for k in range(3):
            out[k][np.ix_(mu, nu)] = g1_rows[k, i, j]
            out[k][np.ix_(nu, mu)] = g1_rows[k, i, j]
    return out


# ----------------------------------------------------------------------------------------------
# Fock-derivative tensors
# ----------------------------------------------------------------------------------------------

def f_v(v, s, grad_s, g0_ao, g1_ao, n_atoms, n_orb):
    """Coulomb response dF[V] [3N, n_orb, n_orb] (`gradients/helpers.rs:47-80`)."""
    vp = v + v.T
    sv = (s * vp).sum(axis=0)
    gsv = g0_ao @ sv
    out = np.zeros((3 * n_atoms, n_orb, n_orb))
    for nc in range(3 * n_atoms):
        ds = grad_s[nc]
        dg = g1_ao[nc]
        gdsv = g0_ao @ (ds * vp).sum(axis=0)
        dgsv = dg @ sv
        d_f = ds * (gsv[:, None] + gsv[None, :]) + s * (dgsv[:, None] + gdsv[:, None] + dgsv[None, :] + gdsv[None, :])
        out[nc] = 0.25 * d_f
    return out


def f_lr(v, s, grad_s, g0_lr_ao, g1_lr_ao, n_atoms, n_orb):
    """Long-range exchange response dF_lr[V] [3N, n_orb, n_orb] (`gradients/helpers.rs:130-188`)."""
    sv = s @ v
    v_t = v.T
    sv_t = s @ v_t
    gv = g0_lr_ao * v
    t_sv = sv.T
    svg_t = (sv * g0_lr_ao).T
    sgv_t = (s @ gv).T
    out = np.zeros((3 * n_atoms, n_orb, n_orb))
    for nc in range(3 * n_atoms):
        d_s = grad_s[nc]
        d_g = g1_lr_ao[nc]
        d_sv_t = d_s @ v_t
        d_sv = d_s @ v
        d_gv = d_g * v
        d_f = g0_lr_ao * (d_s @ t_sv)
        d_f = d_f + (d_sv_t * g0_lr_ao) @ s
        d_f = d_f + d_s @ svg_t
        d_f = d_f + d_s @ sgv_t
        d_f = d_f + g0_lr_ao * (s @ d_sv.T)
        d_f = d_f + (sv_t * g0_lr_ao) @ d_s.T
        d_f = d_f + s @ (d_sv * g0_lr_ao).T
        d_f = d_f + s @ (d_s @ gv).T
        d_f = d_f + d_g * (s @ t_sv)
        d_f = d_f + (sv_t * d_g) @ s
        d_f = d_f + s @ (sv * d_g).T
        d_f = d_f + s @ (s @ d_gv).T
        out[nc] = 0.25 * d_f
    return out


# ----------------------------------------------------------------------------------------------
# H-type contractions
# ----------------------------------------------------------------------------------------------

def h_a_nolr(g0, q_pq, q_rs, v_rs):
    """4 q_pq^T gamma q_rs . v (`gradients/helpers.rs:361-378`)."""
    n_at = q_pq.shape[0]
    tmp = q_rs.reshape(n_at, -1) @ v_rs.reshape(-1)
    tmp2 = g0 @ tmp
    return 4.0 * (tmp2 @ q_pq.reshape(n_at, -1)).reshape(q_pq.shape[1], q_pq.shape[2])


class Hav:
    """`Hav` (`gradients/helpers.rs:631-831`): Coulomb (x2) minus one LR exchange term, times 2."""

    def __init__(self, q_ov, q_vv, q_oo):
        self.qov, self.qvv, self.qoo = q_ov, q_vv, q_oo
        self.qvo = np.ascontiguousarray(q_ov.transpose(0, 2, 1))
        self.n_at, self.no, self.nv = q_ov.shape

    def compute(self, g0, g0_lr, v, kind):
        f = {"tab": self._tab, "tij": self._tij, "qia_x": self._qia_x, "qia_tab": self._qia_tab,
             "qia_tij": self._qia_tij, "qai": self._qai_or_wij, "wij": self._qai_or_wij}[kind]
        return 2.0 * f(g0, g0_lr, v)

    def _tab(self, g0, g0_lr, v):
        N, o, nv = self.n_at, self.no, self.nv
        tmp = self.qvv.reshape(N, nv * nv) @ v.reshape(-1)
        hp = 2.0 * ((g0 @ tmp) @ self.qoo.reshape(N, o * o)).reshape(o, o)
        tmp = (self.qov.reshape(N * o, nv) @ v.T).reshape(N, o, nv)
        tmp2 = (g0_lr @ tmp.reshape(N, o * nv)).reshape(N, o, nv)
        t2s = tmp2.transpose(0, 2, 1).reshape(N * nv, o)
        qs = self.qov.transpose(1, 0, 2).reshape(o, N * nv)
        return hp - qs @ t2s

    def _tij(self, g0, g0_lr, v):
        N, o = self.n_at, self.no
        tmp = self.qoo.reshape(N, o * o) @ v.reshape(-1)
        hp = 2.0 * ((g0 @ tmp) @ self.qoo.reshape(N, o * o)).reshape(o, o)
        tmp = (self.qoo.reshape(N * o, o) @ v.T).reshape(N, o, o)
        tmp2 = (g0_lr @ tmp.reshape(N, o * o)).reshape(N, o, o)
        t2s = tmp2.transpose(0, 2, 1).reshape(N * o, o)
        qs = self.qoo.transpose(1, 0, 2).reshape(o, N * o)
        return hp - qs @ t2s

    def _qia_x(self, g0, g0_lr, v):
        N, o, nv = self.n_at, self.no, self.nv
        tmp = self.qov.reshape(N, o * nv) @ v.reshape(-1)
        hp = 2.0 * ((g0 @ tmp) @ self.qvv.reshape(N, nv * nv)).reshape(nv, nv)
        tmp = (self.qvv.reshape(N * nv, nv) @ v.T).reshape(N, nv, o)
        tmp2 = (g0_lr @ tmp.reshape(N, nv * o)).reshape(N, nv, o)
        t2s = tmp2.transpose(0, 2, 1).reshape(N * o, nv)
        qs = self.qvo.transpose(1, 0, 2).reshape(nv, N * o)
        return hp - qs @ t2s

    def _qia_tab(self, g0, g0_lr, v):
        N, o, nv = self.n_at, self.no, self.nv
        tmp = self.qvv.reshape(N, nv * nv) @ v.reshape(-1)
        hp = 2.0 * ((g0 @ tmp) @ self.qov.reshape(N, o * nv)).reshape(o, nv)
        tmp = (self.qvv.reshape(N * nv, nv) @ v.T).reshape(N, nv, nv)
        tmp2 = (g0_lr @ tmp.reshape(N, nv * nv)).reshape(N, nv, nv)
        t2s = tmp2.transpose(0, 2, 1).reshape(N * nv, nv)
        qs = self.qov.transpose(1, 0, 2).reshape(o, N * nv)
        return hp - qs @ t2s

    def _qia_tij(self, g0, g0_lr, v):
        N, o, nv = self.n_at, self.no, self.nv
        tmp = self.qoo.reshape(N, o * o) @ v.reshape(-1)
        hp = 2.0 * ((g0 @ tmp) @ self.qov.reshape(N, o * nv)).reshape(o, nv)
        tmp = (self.qvo.reshape(N * nv, o) @ v.T).reshape(N, nv, o)
        tmp2 = (g0_lr @ tmp.reshape(N, nv * o)).reshape(N, nv, o)
        t2s = tmp2.transpose(0, 2, 1).reshape(N * o, nv)
        qs = self.qoo.transpose(1, 0, 2).reshape(o, N * o)
        return hp - qs @ t2s

    def _qai_or_wij(self, g0, g0_lr, v):
        N, o, nv = self.n_at, self.no, self.nv
        tmp = self.qov.reshape(N, o * nv) @ v.reshape(-1)
        hp = 2.0 * ((g0 @ tmp) @ self.qoo.reshape(N, o * o)).reshape(o, o)
        tmp = (self.qov.reshape(N * o, nv) @ v.T).reshape(N, o, o)
        tmp2 = (g0_lr @ tmp.reshape(N, o * o)).reshape(N, o, o)
        t2s = tmp2.transpose(0, 2, 1).reshape(N * o, o)
        qs = self.qoo.transpose(1, 0, 2).reshape(o, N * o)
        return hp - qs @ t2s


# ----------------------------------------------------------------------------------------------
# Z-vector
# ----------------------------------------------------------------------------------------------

def mult_av_nolc(g0, q_ov, omega, v):
    """omega o v + 4 q_ov^T gamma q_ov . v (`gradients/helpers.rs:1351-1382`)."""
    N = q_ov.shape[0]
    q = q_ov.reshape(N, -1)
    return omega * v + 4.0 * ((g0 @ (q @ v.reshape(-1))) @ q).reshape(v.shape)


def mult_av_lc(g0, g0_lr, q_ov, q_oo, q_vv, omega, v):
    """omega o v + 2 Coulomb - LR exchange (`gradients/helpers.rs:1384-1438`)."""
    N, no, nv = q_ov.shape
    q = q_ov.reshape(N, -1)
    u = omega * v + 2.0 * ((g0 @ (q @ v.reshape(-1))) @ q).reshape(no, nv)
    tmp31 = (q_vv.reshape(N * nv, nv) @ v.T).reshape(N, nv, no)
    tmp32 = (g0_lr @ tmp31.reshape(N, nv * no)).reshape(N, nv, no).swapaxes(1, 2)
    tmp33 = q_oo.reshape(N * no, no).T @ np.ascontiguousarray(tmp32).reshape(N * no, nv)
    return u - tmp33


def mult_apb_lc(g0, g0_lr, q_ov, q_oo, q_vv, omega, v):
    """(A+B).v for LC: omega o v + 4 Coulomb - (ij|ab) - (ib|ja) exchange, the operator of
    `mult_apb_v` (`gradients/helpers.rs:1225-1307`).  Used by the exact-gradient variant."""
    N, no, nv = q_ov.shape
    u = mult_av_lc(g0, g0_lr, q_ov, q_oo, q_vv, omega, v)
    q = q_ov.reshape(N, -1)
    u = u + 2.0 * ((g0 @ (q @ v.reshape(-1))) @ q).reshape(no, nv)
    t41 = (np.ascontiguousarray(q_ov.transpose(0, 2, 1)).reshape(N * nv, no) @ v).reshape(N, nv, nv)
    t42 = (g0_lr @ t41.reshape(N, nv * nv)).reshape(N, nv, nv).swapaxes(1, 2)
    t43 = np.ascontiguousarray(q_ov.transpose(1, 0, 2)).reshape(no, N * nv) @ np.ascontiguousarray(t42).reshape(N * nv, nv)
    return u - t43


def hplus_wij(g0, g0_lr, q_ov, q_oo, v):
    """H+[v] projected on the occupied block with both exchange terms (`Hplus::hplus_qai_or_wij`,
    `gradients/helpers.rs:588-618`).  Used by the exact-gradient variant."""
    N, no, nv = q_ov.shape
    tmp = q_ov.reshape(N, no * nv) @ v.reshape(-1)
    hp = 4.0 * ((g0 @ tmp) @ q_oo.reshape(N, no * no)).reshape(no, no)
    tmp = (q_ov.reshape(N * no, nv) @ v.T).reshape(N, no, no)
    tmp2 = (g0_lr @ tmp.reshape(N, no * no)).reshape(N, no, no)
    hp -= q_oo.transpose(1, 0, 2).reshape(no, N * no) @ tmp2.transpose(0, 2, 1).reshape(N * no, no)
    tmp = (q_oo.reshape(N * no, no) @ v).reshape(N, no, nv)
    tmp2 = (g0_lr @ tmp.reshape(N, no * nv)).reshape(N, no, nv)
    hp -= q_ov.transpose(1, 0, 2).reshape(no, N * nv) @ tmp2.transpose(0, 2, 1).reshape(N * nv, no)
    return hp


def cg_zvector(apply, a_diag, r_matrix, conv=1.0e-19, maxiter=10000, stats=None):
    """Conjugate gradient of `tda_zvector_lc`/`tda_zvector_no_lc` (`helpers.rs:1130-1223`)."""
    kmax = r_matrix.size
    bs = r_matrix / a_diag
    rhs = r_matrix.reshape(kmax).copy()
    rkm1 = rhs - apply(bs).reshape(kmax)
    rhs_2 = bs.reshape(kmax).copy()
    pkm1 = rkm1.copy()
    it = 0
    for it in range(maxiter):
        apk = apply(pkm1.reshape(r_matrix.shape)).reshape(kmax)
        tmp1 = rkm1 @ rkm1
        tmp2 = pkm1 @ apk
        rhs_2 = rhs_2 + (tmp1 / tmp2) * pkm1
        rkm1 = rkm1 - (tmp1 / tmp2) * apk
        tmp2 = rkm1 @ rkm1
        if tmp2 <= conv:
            break
        pkm1 = (tmp2 / tmp1) * pkm1 + rkm1
    if stats is not None:
        stats["cg_iterations"] = it + 1
    return rhs_2.reshape(r_matrix.shape)


# ----------------------------------------------------------------------------------------------
# derivative tensors of one geometry
# ----------------------------------------------------------------------------------------------

def derivative_tensors(numbers, xyz, ao_offset, ao_atom, hubbard, r_lr, params, orientation="reference",
                       sk_tail="zero"):
    """dS, dH0 [3N, n, n], dgamma (atomwise) and dgamma_AO, dgamma_lr_AO (`ground_state.rs:22-37`,
    `:97-106`, `excited_state.rs:35-53`); `sk_tail` as in `slako.sk_block`."""
    grad_s, grad_h0 = slako.h0_and_s_gradients(numbers, xyz, ao_offset, params, orientation=orientation,
                                               sk_tail=sk_tail)
    g1 = gamma_gradients_atomwise(xyz, gamma_c(hubbard, 0.0))
    g1_ao = gamma_gradients_ao(g1, ao_atom)
    out = dict(grad_s=grad_s, grad_h0=grad_h0, grad_gamma=g1, grad_gamma_ao=g1_ao)
    if r_lr > 0.0:
        g1lr = gamma_gradients_atomwise(xyz, gamma_c(hubbard, r_lr))
        out["grad_gamma_lr"] = g1lr
        out["grad_gamma_lr_ao"] = gamma_gradients_ao(g1lr, ao_atom)
    return out


def gradient_v_rep(numbers, xyz, params):
    """Repulsive-potential gradient (`gradients/helpers.rs:843-868`)."""
    n = len(numbers)
    grad = np.zeros(3 * n)
    for i in range(n):
        for j in range(n):
            if i == j:
                continue
            rv = xyz[i] - xyz[j]
            r = np.linalg.norm(rv)
            za, zb = sorted((int(numbers[i]), int(numbers[j])))
            t, c, dmax = params.rep[(za, zb)]
            d = float(splev(r, (t, c, 3), der=1)) if r <= dmax else 0.0
            grad[3 * i:3 * i + 3] += rv / r * d
    return grad


def ground_state_gradient(inp, der, lc):
    """`System::ground_state_gradient` (`src/gradients/ground_state.rs:12-137`).

    inp: dict with p, p0, h_coul_x, gamma, dq, s, ao_atom, numbers, xyz, params, gamma_lr_ao (LC).
    Returns (gradient [3N], f_lr_dmd0 or None).
    """
    n_atoms = len(inp["numbers"])
    gd = ground_state_densities(inp)
    return ground_state_contract(inp, der, gd, lc, n_atoms,
                                 gradient_v_rep(inp["numbers"], inp["xyz"], inp["params"]))


def ground_state_densities(inp):
    """The coordinate-independent operands of the ground-state gradient (`ground_state.rs:40-96`)."""
    p = inp["p"]
    ao_atom = inp["ao_atom"]
    esp = inp["gamma"] @ inp["dq"]
    esp_ao = esp[ao_atom]
    coulomb_mat = (esp_ao[:, None] + esp_ao[None, :]) * 0.5
    dq = inp["dq"]
    return dict(p_flat=p.reshape(-1), coulomb_x_p=(p * coulomb_mat).reshape(-1),
                dq_x_dq=(dq[:, None] * dq[None, :]).reshape(-1),
                w=0.5 * (p @ inp["h_coul_x"] @ p).reshape(-1), diff_p=p - inp["p0"])


def ground_state_contract(inp, der, gd, lc, n_atoms, v_rep):
    """Contraction of the derivative tensors `der` (all 3N rows, or the rows of one atom with
    n_atoms = 1) with the ground-state operands `gd` (`ground_state.rs:97-136`); `v_rep` is the
    repulsive gradient of the same rows.  Returns (gradient rows, f_lr_dmd0 rows or None)."""
    n_orb = inp["p"].shape[0]
    gs2 = der["grad_s"].reshape(3 * n_atoms, -1)
    gh2 = der["grad_h0"].reshape(3 * n_atoms, -1)
    grad = gh2 @ gd["p_flat"]
    grad -= gs2 @ gd["w"]
    grad += gs2 @ gd["coulomb_x_p"]
    grad += der["grad_gamma"].reshape(3 * n_atoms, -1) @ gd["dq_x_dq"]
    grad = grad + v_rep
    flr_dmd0 = None
    if lc:
        diff_p = gd["diff_p"]
        flr_dmd0 = f_lr(diff_p, inp["s"], der["grad_s"], inp["gamma_lr_ao"], der["grad_gamma_lr_ao"],
                        n_atoms, n_orb)
        grad = grad - 0.25 * flr_dmd0.reshape(3 * n_atoms, -1) @ diff_p.reshape(-1)
    return grad, flr_dmd0


def tda_gradient(inp, der, state, lc, flr_dmd0=None, stats=None, variant="reference"):
    """`tda_gradient_lc` / `tda_gradient_nolc` (`src/gradients/excited_state.rs:56-487`):
    `tda_gradient_densities`, then `tda_gradient_contract` over all 3N derivative rows."""
    d = tda_gradient_densities(inp, state, lc, stats=stats, variant=variant)
    return tda_gradient_contract(inp, der, d, lc, flr_dmd0, inp["q_ov"].shape[0])


def tda_gradient_densities(inp, state, lc, stats=None, variant="reference"):
    """The coordinate-independent part of `tda_gradient_lc` / `tda_gradient_nolc`
    (`src/gradients/excited_state.rs:56-430`): Z-vector, W, and the AO densities the derivative
    tensors are contracted with.  Returns dict(diff_p, m = T_vv - T_oo + Z_AO, w_ao, x_ao).

    variant="reference" follows tincr exactly.  For LC, tincr solves the Z-vector equation with
    the TDA matrix A (`mult_av_lc`, 2 Coulomb - one exchange) and uses Hav for W_ij[Z]; the
    derivative of the LC-TDA excitation energy needs (A+B) and H+[Z] instead (both exchange
    terms, Z is not symmetric).  variant="exact" makes those two replacements, which brings the
    LC gradient onto central finite differences; non-LC is identical in both variants.

    inp: dict with orbe, occ, virt (index arrays), omega_state/ci_eigenvalues, ci_coefficients
    [o*v, n_states], q_ov, q_oo, q_vv, gamma, gamma_lr, p, p0, s, orbs, gamma_ao, gamma_lr_ao.
    """
    orbe = inp["orbe"]
    occ, virt = inp["occ"], inp["virt"]
    orbe_occ, orbe_virt = orbe[occ], orbe[virt]
    ei, ea = np.diag(orbe_occ), np.diag(orbe_virt)
    no, nv = len(occ), len(virt)
    omega_state = inp["ci_eigenvalues"][state]
    n_states = inp["ci_coefficients"].shape[1]
    xs = np.ascontiguousarray(inp["ci_coefficients"].T).reshape(n_states, no, nv)[state]
    u_ab = 2.0 * xs.T @ xs
    u_ij = 2.0 * xs @ xs.T
    v_ab = 2.0 * (ei @ xs).T @ xs
    v_ij = 2.0 * xs @ ea @ xs.T
    t_ab = xs.T @ xs
    t_ij = xs @ xs.T
    n_atoms = inp["q_ov"].shape[0]
    qov = inp["q_ov"].reshape(n_atoms, no, nv)
    qoo = inp["q_oo"].reshape(n_atoms, no, no)
    qvv = inp["q_vv"].reshape(n_atoms, nv, nv)
    g0 = inp["gamma"]
    omega_input = orbe_virt[None, :] - orbe_occ[:, None]
    if lc:
        g0_lr = inp["gamma_lr"]
        hav = Hav(qov, qvv, qoo)
        g_ij = hav.compute(g0, g0_lr, t_ab, "tab") - hav.compute(g0, g0_lr, t_ij, "tij")
        q_ij = omega_state * u_ij - v_ij + g_ij
        q_ab = omega_state * u_ab + v_ab
        q_ia = xs @ hav.compute(g0, g0_lr, xs, "qia_x").T
        q_ia = q_ia + hav.compute(g0, g0_lr, t_ab, "qia_tab")
        q_ia = q_ia - hav.compute(g0, g0_lr, t_ij, "qia_tij")
        q_ai = xs.T @ hav.compute(g0, g0_lr, xs, "qai")
        r_ia = q_ai.T - q_ia
        zop = mult_apb_lc if variant == "exact" else mult_av_lc
        z_ia = cg_zvector(lambda v: zop(g0, g0_lr, qov, qoo, qvv, omega_input, v),
                          omega_input, r_ia, stats=stats)
        if variant == "exact":
            w_ij = q_ij + hplus_wij(g0, g0_lr, qov, qoo, z_ia)
        else:
            w_ij = q_ij + hav.compute(g0, g0_lr, z_ia, "wij")
    else:
        g_ij = h_a_nolr(g0, qoo, qvv, t_ab) - h_a_nolr(g0, qoo, qoo, t_ij)
        q_ij = omega_state * u_ij - v_ij + g_ij
        q_ab = omega_state * u_ab + v_ab
        q_ia = xs @ h_a_nolr(g0, qvv, qov, xs).T
        q_ia = q_ia + h_a_nolr(g0, qov, qvv, t_ab)
        q_ia = q_ia - h_a_nolr(g0, qov, qoo, t_ij)
        q_ai = xs.T @ h_a_nolr(g0, qoo, qov, xs)
        r_ia = q_ai.T - q_ia
        z_ia = cg_zvector(lambda v: mult_av_nolc(g0, qov, omega_input, v), omega_input, r_ia, stats=stats)
        w_ij = q_ij + h_a_nolr(g0, qoo, qov, z_ia)
    w_ij = w_ij.copy()
    w_ij[np.diag_indices(no)] /= 2.0
    w_ia = q_ai.T + ei @ z_ia
    w_ai = q_ai + (ei @ z_ia).T
    w_ab = q_ab.copy()
    w_ab[np.diag_indices(nv)] /= 2.0
    w = np.zeros((no + nv, no + nv))
    w[:no, :no] = w_ij
    w[:no, no:] = w_ia
    w[no:, :no] = w_ai
    w[no:, no:] = w_ab
    orbs = inp["orbs"]
    c_o = orbs[:, occ]
    c_v = orbs[:, virt]
    t_oo = c_o @ t_ij @ c_o.T
    t_vv = c_v @ t_ab @ c_v.T
    z_ao = c_o @ z_ia @ c_v.T
    w_ao = orbs @ np.triu(w) @ orbs.T
    x_ao = c_o @ xs @ c_v.T
    if stats is not None:
        stats["z_ia"] = z_ia
        stats["w"] = w
    return dict(diff_p=inp["p"] - inp["p0"], m=(t_vv - t_oo + z_ao).reshape(-1), w_ao=w_ao, x_ao=x_ao)


def tda_gradient_contract(inp, der, d, lc, flr_dmd0, n_atoms):
    """Contraction of the derivative tensors `der` (all 3N rows, or the rows of one atom with
    n_atoms = 1) with the densities of `tda_gradient_densities` (`excited_state.rs:432-486`, LC;
    `:232-256`, non-LC); flr_dmd0 holds f_lr(P - P0) for the same rows (LC)."""
    n_orb = inp["s"].shape[0]
    s = inp["s"]
    diff_p, m, w_ao, x_ao = d["diff_p"], d["m"], d["w_ao"], d["x_ao"]
    f_dmd0 = f_v(diff_p, s, der["grad_s"], inp["gamma_ao"], der["grad_gamma_ao"], n_atoms, n_orb)
    grad_h = der["grad_h0"] + f_dmd0
    if lc:
        grad_h = grad_h - 0.5 * flr_dmd0
    f = f_v(x_ao, s, der["grad_s"], inp["gamma_ao"], der["grad_gamma_ao"], n_atoms, n_orb)
    grad = grad_h.reshape(3 * n_atoms, -1) @ m
    grad = grad - der["grad_s"].reshape(3 * n_atoms, -1) @ w_ao.reshape(-1)
    grad = grad + 2.0 * f.reshape(3 * n_atoms, -1) @ x_ao.reshape(-1)
    if lc:
        flr_p = f_lr(x_ao.T, s, der["grad_s"], inp["gamma_lr_ao"], der["grad_gamma_lr_ao"], n_atoms, n_orb)
        grad = grad - flr_p.reshape(3 * n_atoms, -1) @ x_ao.reshape(-1)
    return grad


# ----------------------------------------------------------------------------------------------
# the same gradients one atom at a time (memory O(n_orb^2) instead of O(3N n_orb^2))
# ----------------------------------------------------------------------------------------------

class AtomRows:
    """Derivative-tensor rows of one atom at a time: the 3-row blocks of `derivative_tensors`
    (dS, dH0, dgamma, dgamma_AO, dgamma_lr_AO) for atom i, built on request."""

    def __init__(self, numbers, xyz, ao_offset, ao_atom, hubbard, r_lr, params, orientation="reference",
                 sk_tail="zero"):
        self.numbers, self.xyz, self.ao_offset, self.ao_atom = numbers, xyz, ao_offset, ao_atom
        self.params, self.orientation, self.r_lr, self.sk_tail = params, orientation, r_lr, sk_tail
        self.c0 = gamma_c(hubbard, 0.0)
        self.clr = gamma_c(hubbard, r_lr) if r_lr > 0.0 else None
        self.v_rep = gradient_v_rep(numbers, xyz, params)

    def __call__(self, i):
        gs, gh = slako.h0_and_s_gradient_rows(i, self.numbers, self.xyz, self.ao_offset, self.params,
                                              orientation=self.orientation, sk_tail=self.sk_tail)
        g1 = gamma_gradient_rows(i, self.xyz, self.c0)
        out = dict(grad_s=gs, grad_h0=gh, grad_gamma=g1, grad_gamma_ao=gamma_gradient_ao_rows(i, g1, self.ao_atom))
        if self.clr is not None:
            g1lr = gamma_gradient_rows(i, self.xyz, self.clr)
            out["grad_gamma_lr"] = g1lr
            out["grad_gamma_lr_ao"] = gamma_gradient_ao_rows(i, g1lr, self.ao_atom)
        return out


def gradient_rows(inp, rows, i, gd, d, lc):
    """Ground-state and excitation gradient of atom i (3 components each) from its derivative rows:
    the same formulas as `ground_state_gradient` and `tda_gradient`, with the operands `gd`
    (`ground_state_densities`) and `d` (`tda_gradient_densities`, or None for the ground state
    only)."""
    blk = rows(i)
    g, flr = ground_state_contract(inp, blk, gd, lc, 1, rows.v_rep[3 * i:3 * i + 3])
    x = None if d is None else tda_gradient_contract(inp, blk, d, lc, flr, 1)
    return g, x


def gradients_by_atom(inp, rows, state, lc, variant="reference", stats=None):
    """Ground-state and excitation gradients [3N] each, atom by atom (`gradient_rows`), equal to
    `ground_state_gradient` + `tda_gradient` without the [3N, n_orb, n_orb] tensors."""
    gd = ground_state_densities(inp)
    d = tda_gradient_densities(inp, state, lc, stats=stats, variant=variant)
    n_atoms = len(inp["numbers"])
    ggs, gex = np.zeros(3 * n_atoms), np.zeros(3 * n_atoms)
    for i in range(n_atoms):
        ggs[3 * i:3 * i + 3], gex[3 * i:3 * i + 3] = gradient_rows(inp, rows, i, gd, d, lc)
    return ggs, gex
