"""Oracle: Slater-Koster matrix elements and their Cartesian gradients (s and p orbitals).

Restates `src/param/slako_transformations.rs` (`directional_cosines` `:35-55`,
`slako_transformation` `:57-680`, `slako_transformation_gradients` `:682-6404`) for l <= 1 and the
dense assembly of `src/scc/h0_and_s.rs:92-300`.  The gradient rules are the analytic derivative of
the value rules with respect to the inter-centre vector r = pos2 - pos1:

    d/dr_c [P(u) V(r)] = (grad_u P . (e_c - u_c u)) V / r + P V'(r) u_c,   u = r/|r|

which is what tincr's hard-coded expressions evaluate.  Splines are FITPACK cubic splines
(SciPy's FITPACK binding) from the shipped parameter set, evaluated as zero beyond the last grid
point (10 bohr): tincr's behaviour there comes from Rusty-FITPACK's `splev_uniform`, which no
fixture pins, and FITPACK's polynomial extrapolation would make S indefinite beyond ~15 bohr.

Test infrastructure only (see oracle/__init__.py).
"""

import numpy as np
from scipy.interpolate import splev

PROXIMITY_CUTOFF = 30.0
_AX = {-1: 1, 0: 2, 1: 0}   # m -> Cartesian axis of the real p orbital (y, z, x)


def _terms(l1, m1, l2, m2, u):
    """Angular factors: list of (slot, P(u), grad_u P) for one orbital pair."""
    e = np.eye(3)
    n = u.shape[0]
    if l1 == 0 and l2 == 0:
        return [(0, np.ones(n), np.zeros((n, 3)))]
    if l1 == 0 and l2 == 1:
        c = _AX[m2]
        return [(1, u[:, c], np.tile(e[c], (n, 1)))]
    if l1 == 1 and l2 == 0:
        c = _AX[m1]
        return [(2, u[:, c], np.tile(e[c], (n, 1)))]
    c1, c2 = _AX[m1], _AX[m2]
    if c1 == c2:
        o = [k for k in range(3) if k != c1]
        p_pi = u[:, o[0]] ** 2 + u[:, o[1]] ** 2
        g_pi = 2.0 * u[:, o[0], None] * e[o[0]] + 2.0 * u[:, o[1], None] * e[o[1]]
        p_si = u[:, c1] ** 2
        g_si = 2.0 * u[:, c1, None] * e[c1]
        return [(3, p_pi, g_pi), (4, p_si, g_si)]
    p = u[:, c1] * u[:, c2]
    g = u[:, c2, None] * e[c1] + u[:, c1, None] * e[c2]
    return [(3, -p, -g), (4, p, g)]


def sk_block(knots, coef, present, l_a, m_a, l_b, m_b, rvec, grad=False, sk_tail="zero"):
    """Matrix elements (and gradients w.r.t. rvec) between all orbitals of centre 1 (l_a, m_a)
    and centre 2 (l_b, m_b) for a batch of inter-centre vectors rvec [n, 3].  Beyond the spline grid
    the integrals are zero (sk_tail="zero") or the boundary polynomial piece (sk_tail="extrapolate",
    FITPACK splev with ext = 0, which tincr's splev_uniform evaluates up to 30 bohr).

    Returns val [n, na, nb] and, if grad, g [n, 3, na, nb].
    """
    r = np.linalg.norm(rvec, axis=1)
    u = rvec / r[:, None]
    n = len(r)
    v = np.zeros((5, n))
    dv = np.zeros((5, n))
    slot_of = {0: 0, 2: 1, 4: 2, 5: 3, 6: 4}
    for idx in present:
        s = slot_of[idx]
        ext = 0 if sk_tail == "extrapolate" else 1
        v[s] = splev(r, (knots, coef[s], 3), ext=ext)
        dv[s] = splev(r, (knots, coef[s], 3), der=1, ext=ext)
    na, nb = len(l_a), len(l_b)
    val = np.zeros((n, na, nb))
    g = np.zeros((n, 3, na, nb)) if grad else None
    proj = np.eye(3)[None, :, :] - u[:, :, None] * u[:, None, :]        # [n, c, d]
    for p in range(na):
        for q in range(nb):
            for slot, pu, gu in _terms(int(l_a[p]), int(m_a[p]), int(l_b[q]), int(m_b[q]), u):
                val[:, p, q] += pu * v[slot]
                if grad:
                    g[:, :, p, q] += (np.einsum("nd,ncd->nc", gu, proj) * (v[slot] / r)[:, None]
                                      + (pu * dv[slot])[:, None] * u)
    return val, g


def h0_and_s_gradients(numbers, xyz, ao_offset, params, orientation="reference", sk_tail="zero"):
    """Dense dS/dR and dH0/dR [3N, n_orb, n_orb] (`src/scc/h0_and_s.rs:196-300`).

    Entry [3i+c, mu, nu] (and [3i+c, nu, mu]) holds d S_{mu nu} / d R_{i,c} for mu on atom i and
    nu on atom j != i within the proximity cutoff.

    orientation="reference" reproduces tincr: for a same-element pair the derivative with respect
    to atom i is taken with atom i as centre 1, for both atoms of the pair.  tincr's homonuclear H0
    tables are not swap symmetric (sp_sigma != -ps_sigma), so that derivative differs from the
    derivative of the H0 that `h0_and_s` builds (centre 1 = lower index) for the higher-index atom.
    orientation="index" uses the lower-index atom as centre 1 for same-element pairs, i.e. the
    exact derivative of H0 as built.
    """
    n_atoms = len(numbers)
    n_orb = int(ao_offset[-1])
    gs = np.zeros((3 * n_atoms, n_orb, n_orb))
    gh = np.zeros((3 * n_atoms, n_orb, n_orb))
    for i in range(n_atoms):
        h0_and_s_gradient_rows(i, numbers, xyz, ao_offset, params, orientation,
                               out_s=gs[3 * i:3 * i + 3], out_h=gh[3 * i:3 * i + 3], sk_tail=sk_tail)
    return gs, gh


def h0_and_s_gradient_rows(i, numbers, xyz, ao_offset, params, orientation="reference", out_s=None, out_h=None,
                           sk_tail="zero"):
    """Rows 3i..3i+2 of the dense dS/dR and dH0/dR of `h0_and_s_gradients` (the loop body of
    `src/scc/h0_and_s.rs:203-296` for one atom i): [3, n_orb, n_orb] each, written into out_s /
    out_h when given (zeros elsewhere).  The partner atoms j are evaluated in batches of the same
    element and centre order (one spline evaluation per batch)."""
    n_atoms = len(numbers)
    n_orb = int(ao_offset[-1])
    gs = np.zeros((3, n_orb, n_orb)) if out_s is None else out_s
    gh = np.zeros((3, n_orb, n_orb)) if out_h is None else out_h
    ei = params.element(numbers[i])
    zi = int(numbers[i])
    groups = {}
    for j in range(n_atoms):
        if i == j:
            continue
        d = xyz[j] - xyz[i]
        if np.linalg.norm(d) >= PROXIMITY_CUTOFF:
            continue
        zj = int(numbers[j])
        centre1_is_i = zi < zj or (zi == zj and (orientation == "reference" or i < j))
        groups.setdefault((zj, centre1_is_i), []).append(j)
    mu = slice(ao_offset[i], ao_offset[i + 1])
    for (zj, centre1_is_i), js in groups.items():
        ej = params.element(zj)
        d = xyz[js] - xyz[i][None, :]
        if centre1_is_i:
            # gradient w.r.t. r = pos_j - pos_i, turned into d/dR_i by a minus sign (`:218-248`)
            key = (zi, zj)
            _, gS = sk_block(params.sk_knots, params.sk_coef[key + ("s",)], params.sk_present[key],
                             ei.l, ei.m, ej.l, ej.m, d, grad=True, sk_tail=sk_tail)
            _, gH = sk_block(params.sk_knots, params.sk_coef[key + ("h",)], params.sk_present[key],
                             ei.l, ei.m, ej.l, ej.m, d, grad=True, sk_tail=sk_tail)
            bs_all, bh_all = -gS, -gH
        else:
            # centres swapped: r = pos_i - pos_j, orbitals (j, i) (`:249-277`)
            key = (zj, zi)
            _, gS = sk_block(params.sk_knots, params.sk_coef[key + ("s",)], params.sk_present[key],
                             ej.l, ej.m, ei.l, ei.m, -d, grad=True, sk_tail=sk_tail)
            _, gH = sk_block(params.sk_knots, params.sk_coef[key + ("h",)], params.sk_present[key],
                             ej.l, ej.m, ei.l, ei.m, -d, grad=True, sk_tail=sk_tail)
            bs_all, bh_all = gS.transpose(0, 1, 3, 2), gH.transpose(0, 1, 3, 2)
        for t, j in enumerate(js):
            nu = slice(ao_offset[j], ao_offset[j + 1])
            bs, bh = bs_all[t], bh_all[t]
            gs[:, mu, nu] = bs
            gs[:, nu, mu] = bs.transpose(0, 2, 1)
            gh[:, mu, nu] = bh
            gh[:, nu, mu] = bh.transpose(0, 2, 1)
    return gs, gh


def h0_and_s(numbers, xyz, ao_offset, ao_energy, params, sk_tail="zero"):
    """Dense S and H0 (`src/scc/h0_and_s.rs:92-182`), used to cross-check the host producer and
    for finite differences of the SK gradients."""
    n_atoms = len(numbers)
    n_orb = int(ao_offset[-1])
    S = np.eye(n_orb)
    H = np.diag(np.asarray(ao_energy, dtype=np.float64))
    for i in range(n_atoms):
        for j in range(i + 1, n_atoms):
            d = xyz[j] - xyz[i]
            if np.linalg.norm(d) >= PROXIMITY_CUTOFF:
                continue
            zi, zj = int(numbers[i]), int(numbers[j])
            ei, ej = params.element(zi), params.element(zj)
            if zi <= zj:
                key = (zi, zj)
                vs, _ = sk_block(params.sk_knots, params.sk_coef[key + ("s",)], params.sk_present[key],
                                 ei.l, ei.m, ej.l, ej.m, d[None, :], sk_tail=sk_tail)
                vh, _ = sk_block(params.sk_knots, params.sk_coef[key + ("h",)], params.sk_present[key],
                                 ei.l, ei.m, ej.l, ej.m, d[None, :], sk_tail=sk_tail)
                bs, bh = vs[0], vh[0]
            else:
                key = (zj, zi)
                vs, _ = sk_block(params.sk_knots, params.sk_coef[key + ("s",)], params.sk_present[key],
                                 ej.l, ej.m, ei.l, ei.m, -d[None, :], sk_tail=sk_tail)
                vh, _ = sk_block(params.sk_knots, params.sk_coef[key + ("h",)], params.sk_present[key],
                                 ej.l, ej.m, ei.l, ei.m, -d[None, :], sk_tail=sk_tail)
                bs, bh = vs[0].T, vh[0].T
            mu = slice(ao_offset[i], ao_offset[i + 1])
            nu = slice(ao_offset[j], ao_offset[j + 1])
            S[mu, nu] = bs
            S[nu, mu] = bs.T
            H[mu, nu] = bh
            H[nu, mu] = bh.T
    return S, H
