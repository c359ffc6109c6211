"""Oracle: tincr's FMO exciton Hamiltonian in the diabatic LE / CT basis and its lowest states.

Restates `SuperSystem::create_exciton_hamiltonian_new` (src/fmo/lcmo/basis.rs:449-503) with
`build_lcmo_fock_matrix` (src/fmo/lcmo/hamiltonian.rs:12-152), the basis of
`create_diab_basis_new` (basis.rs:180-238: n_le LE states per monomer, then for each CT pair the
n_ct states of both directions) and the couplings of `exciton_coupling`
(src/fmo/lcmo/integrals.rs:17-79): `le_le` (:81-169), `le_ct_new` = `le_ct_1e_new` (:542-600) +
`le_ct_2e_new` (:602-727), `ct_ct_new` (:733-878), with the transition charges of
src/fmo/lcmo/lcmo_trans_charges.rs (`q_lele` :21-86, `q_lect` :276-426, `q_ctct` :428-586) and the
gamma blocks of src/fmo/supersystem.rs:343-371.  The lowest roots come from tincr's Davidson on the
dense matrix (engine src/excited_states/solvers/mod.rs:36-51: H X, preconditioner r / (w - diag H)).

tincr's defaults apply: restricted active space on, 10 occupied and 10 virtual orbitals next to the
gap for the exchange integrals of LE-CT and CT-CT couplings (src/io/settings.rs:110-118); the
LE-LE exchange uses the full spaces.  Pair types follow `get_pair_type` (src/fmo/pair.rs:35-53): a
monomer pair is a real pair when some atom pair is closer than 2 x the sum of their van der Waals
radii (src/constants.rs:1389, UFF radii in bohr), otherwise it is an ESD pair (no exchange); a
monomer with itself has type None.

Two statements of the reference are index slips that this restatement does not copy (tincr as
written reads another monomer's orbitals or charges there, or fails on an out-of-range index when
the monomers differ in size, as the acenes of the benchmark aggregate do):
* `q_ctct` for the occupied orbitals (lcmo_trans_charges.rs:485-494) forms the charges on the
  second hole monomer's atoms from the FIRST hole monomer's coefficients (`occs_ct_a.row(mu)` where
  the electron branch, :571, uses the second set); here the second set is used, as in `q_lele`
  and in the electron branch.
* `ct_ct_new` with a common electron monomer (integrals.rs:789-800) takes q_vv, atom count and
  virtual count from the HOLE monomer of the first state (`self.monomers[state_1.m_h]`); here from
  the common electron monomer, whose virtual orbitals the integral couples.

Test infrastructure only (see oracle/__init__.py).
"""

import numpy as np

from . import tda as OT

# Sums of UFF van der Waals radii in bohr for H, C, N, O (src/constants.rs:1389, VDW_SUM[i][j])
VDW_SUM_BOHR = {(1, 1): 5.454, (1, 6): 6.366, (1, 7): 6.185, (1, 8): 6.128, (6, 6): 7.279, (6, 7): 7.098,
                (6, 8): 7.041, (7, 7): 6.916, (7, 8): 6.860, (8, 8): 6.803}
ACTIVE_LE = 10      # src/io/settings.rs:110-112
ACTIVE_CT = 10      # src/io/settings.rs:113-115


def pair_type(numbers_a, xyz_a, numbers_b, xyz_b, vdw_scaling=2.0):
    """'pair' when some atom pair is closer than vdw_scaling x their vdW sum, else 'esd'
    (`get_pair_type`, src/fmo/pair.rs:35-53)."""
    for za, ra in zip(numbers_a, xyz_a):
        d = np.linalg.norm(xyz_b - ra[None, :], axis=1)
        lim = np.array([vdw_scaling * VDW_SUM_BOHR[tuple(sorted((int(za), int(zb))))] for zb in numbers_b])
        if np.any(d < lim):
            return "pair"
    return "esd"


class Frag:
    """What the couplings read of one monomer: atoms in the aggregate (global indices), AO offsets
    of its atoms (local), MO coefficients C [n, n] and energies, occupied count, transition charges
    q_ov / q_oo / q_vv [N, .] (`trans_charges` with the monomer's S) and xyz."""

    def __init__(self, index, atoms, ao_offset, orbs, orbe, s, n_occ, xyz, numbers):
        self.index = index
        self.atoms = np.asarray(atoms)
        self.ao_offset = np.asarray(ao_offset)
        self.orbs, self.orbe, self.s = orbs, orbe, s
        self.n_atoms = len(self.atoms)
        self.n_orb = orbs.shape[0]
        self.n_occ = n_occ
        self.n_virt = self.n_orb - n_occ
        self.xyz, self.numbers = xyz, numbers
        occ, virt = np.arange(n_occ), np.arange(n_occ, self.n_orb)
        self.q_ov, self.q_oo, self.q_vv = OT.trans_charges(self.ao_offset, orbs, s, occ, virt)
        self.occs = orbs[:, :n_occ]
        self.virts = orbs[:, n_occ:]


class Aggregate:
    """The supersystem data the exciton Hamiltonian reads.

    frags: list of Frag (monomer order); s_block(I, J): AO overlap between monomers I and J;
    gamma / gamma_lr: atomwise gamma matrices of the whole aggregate (global atom order);
    pair_types: {(I, J), I < J: 'pair' | 'esd'}; pair_scc: {(I, J): (orbs_IJ, orbe_IJ)} for every
    real pair (ground state of the dimer, AO order I then J)."""

    def __init__(self, frags, s_block, gamma, gamma_lr, pair_types, pair_scc):
        self.frags = frags
        self.s_block = s_block
        self.gamma, self.gamma_lr = gamma, gamma_lr
        self.pair_types = pair_types
        self.pair_scc = pair_scc

    def type_of_pair(self, i, j):
        """`Properties::type_of_pair` (src/properties/getter.rs:583-591): None for i == j."""
        if i == j:
            return None
        return self.pair_types[(min(i, j), max(i, j))]

    def g(self, a, b, lr):
        """`gamma_a_b` (supersystem.rs:347-353): gamma block between the atoms of monomers a, b."""
        m = self.gamma_lr if lr else self.gamma
        return m[np.ix_(self.frags[a].atoms, self.frags[b].atoms)]

    def g_ab_c(self, a, b, c, lr):
        """`gamma_ab_c` (supersystem.rs:355-361): [N_a + N_b, N_c]."""
        return np.concatenate([self.g(a, c, lr), self.g(b, c, lr)], axis=0)

    def g_ab_cd(self, a, b, c, d, lr):
        """`gamma_ab_cd` (supersystem.rs:363-371): [N_a + N_b, N_c + N_d]."""
        return np.block([[self.g(a, c, lr), self.g(a, d, lr)], [self.g(b, c, lr), self.g(b, d, lr)]])


# ----------------------------------------------------------------------------------------------
# LCMO Fock matrix
# ----------------------------------------------------------------------------------------------

def lcmo_fock(agg):
    """`build_lcmo_fock_matrix` (src/fmo/lcmo/hamiltonian.rs:12-152): the Fock matrix in the basis
    of all monomer MOs (monomer order), diagonal blocks diag(e_I) corrected by every real pair,
    off-diagonal blocks sum_r e_r <p^I|r^IJ><r^IJ|q^J>, then the first-order Loewdin
    transformation x^T F x with x = 3/2 I - 1/2 S_total (S_total: MO overlaps between monomers).
    Returns (F', MO offsets of the monomers)."""
    frags = agg.frags
    off = np.concatenate([[0], np.cumsum([f.n_orb for f in frags])])
    dim = int(off[-1])
    fock = np.zeros((dim, dim))
    s_total = np.eye(dim)
    for f in frags:
        sl = slice(off[f.index], off[f.index + 1])
        fock[sl, sl] = np.diag(f.orbe)
    for (i, j), t in sorted(agg.pair_types.items()):
        if t != "pair":
            continue
        fi, fj = frags[i], frags[j]
        orbs_ij, orbe_ij = agg.pair_scc[(i, j)]
        ni = fi.n_orb
        s_pair = np.block([[fi.s, agg.s_block(i, j)], [agg.s_block(j, i), fj.s]])
        s_pr = (fi.orbs.T @ s_pair[:ni, :]) @ orbs_ij
        s_qr = (fj.orbs.T @ s_pair[ni:, :]) @ orbs_ij
        s_pq = (fi.orbs.T @ s_pair[:ni, ni:]) @ fj.orbs
        si, sj = slice(off[i], off[i + 1]), slice(off[j], off[j + 1])
        s_total[si, sj] = s_pq
        s_total[sj, si] = s_pq.T
        f_aa = (s_pr * orbe_ij) @ s_pr.T
        f_bb = (s_qr * orbe_ij) @ s_qr.T
        f_ab = (s_pr * orbe_ij) @ s_qr.T
        f_ba = (s_qr * orbe_ij) @ s_pr.T
        fock[si, si] += f_aa - np.diag(fi.orbe)
        fock[sj, sj] += f_bb - np.diag(fj.orbe)
        fock[si, sj] += f_ab
        fock[sj, si] += f_ba
    x = 1.5 * np.eye(dim) - 0.5 * s_total
    return (x.T @ fock) @ x, off


class LcmoFockBlocks:
    """Blocks of the LCMO Fock matrix F' = x^T F x (`lcmo_fock`) without the dense matrix, for
    aggregates whose MO space is too large to hold it: x = I - 1/2 S_off, with S_off and F nonzero only
    on the diagonal blocks and between the monomers of real pairs, so
        F'_xy = sum_{k in {x} + nb(x)} sum_{m in {y} + nb(y)} x_kx^T F_km x_my,
    x_kx = I for k == x and -1/2 S_kx otherwise (nb = real-pair neighbours).  The same sums of the
    same pair quantities as the dense form (hamiltonian.rs:12-152), block by block; blocks cached."""

    def __init__(self, agg):
        self.agg = agg
        n = len(agg.frags)
        self.nb = [[] for _ in range(n)]
        for (i, j), t in agg.pair_types.items():
            if t == "pair":
                self.nb[i].append(j)
                self.nb[j].append(i)
        self._pair = {}
        self._f = {}
        self._fp = {}

    def _pair_terms(self, i, j):
        """(s_pq, f_aa, f_bb, f_ab) of the real pair i < j (hamiltonian.rs:46-110)."""
        key = (i, j)
        if key not in self._pair:
            agg = self.agg
            fi, fj = agg.frags[i], agg.frags[j]
            orbs_ij, orbe_ij = agg.pair_scc[(i, j)]
            ni = fi.n_orb
            s_pair = np.block([[fi.s, agg.s_block(i, j)], [agg.s_block(j, i), fj.s]])
            s_pr = (fi.orbs.T @ s_pair[:ni, :]) @ orbs_ij
            s_qr = (fj.orbs.T @ s_pair[ni:, :]) @ orbs_ij
            s_pq = (fi.orbs.T @ s_pair[:ni, ni:]) @ fj.orbs
            self._pair[key] = (s_pq, (s_pr * orbe_ij) @ s_pr.T, (s_qr * orbe_ij) @ s_qr.T,
                               (s_pr * orbe_ij) @ s_qr.T)
        return self._pair[key]

    def s(self, k, m):
        """MO overlap block S_km of a real pair (k != m)."""
        s_pq = self._pair_terms(min(k, m), max(k, m))[0]
        return s_pq if k < m else s_pq.T

    def f(self, k, m):
        """Block F_km before the transformation (zero unless k == m or k, m is a real pair)."""
        key = (k, m)
        if key not in self._f:
            frags = self.agg.frags
            if k == m:
                out = np.diag(frags[k].orbe).astype(float)
                for o in self.nb[k]:
                    _, f_aa, f_bb, _ = self._pair_terms(min(k, o), max(k, o))
                    out = out + (f_aa if k < o else f_bb) - np.diag(frags[k].orbe)
            elif m in self.nb[k]:
                f_ab = self._pair_terms(min(k, m), max(k, m))[3]
                out = f_ab if k < m else f_ab.T
            else:
                out = None
            self._f[key] = out
        return self._f[key]

    def __call__(self, x, y):
        key = (x, y)
        if key not in self._fp:
            frags = self.agg.frags
            out = np.zeros((frags[x].n_orb, frags[y].n_orb))
            for k in [x] + self.nb[x]:
                xk = None if k == x else -0.5 * self.s(k, x)
                for m in [y] + self.nb[y]:
                    fkm = self.f(k, m)
                    if fkm is None:
                        continue
                    t = fkm if m == y else fkm @ (-0.5 * self.s(m, y))
                    out += t if xk is None else xk.T @ t
            self._fp[key] = out
        return self._fp[key]


# ----------------------------------------------------------------------------------------------
# diabatic basis states
# ----------------------------------------------------------------------------------------------

class LE:
    """A locally excited state (`LocallyExcited`, basis.rs): monomer, root n, energy, TDM [o, v],
    q_trans = q_ov . X [N]."""

    def __init__(self, frag, n, energy, x):
        self.m, self.n, self.energy = frag.index, n, energy
        self.tdm = x.reshape(frag.n_occ, frag.n_virt)
        self.q_trans = frag.q_ov @ x


class CT:
    """A pair charge-transfer state (`ChargeTransferPair`, basis.rs:604-612): hole monomer m_h,
    electron monomer m_l, root n, energy, TDM [o_h, v_l], q_tr [N_h + N_l]."""

    def __init__(self, m_h, m_l, n, energy, x, q_tr, o_h, v_l):
        self.m_h, self.m_l, self.n, self.energy = m_h, m_l, n, energy
        self.tdm = x.reshape(o_h, v_l)
        self.q_tr = q_tr


def diabatic_basis(agg, le_results, ct_results, ct_pairs, n_le, n_ct):
    """`create_diab_basis_new` (basis.rs:180-238): n_le LE states of every monomer, then for every
    CT pair (I, J) in order, for n < n_ct: the state I -> J, then J -> I.
    le_results[I] = (energies, coefficients [o v, roots]); ct_results[(h, l)] = (energies,
    coefficients [o_h v_l, roots], q_tr [N_h + N_l, roots])."""
    states = []
    for f in agg.frags:
        e, c = le_results[f.index]
        for n in range(n_le):
            states.append(LE(f, n, float(e[n]), c[:, n]))
    for i, j in ct_pairs:
        for n in range(n_ct):
            for h, l in ((i, j), (j, i)):
                e, c, q = ct_results[(h, l)]
                states.append(CT(h, l, n, float(e[n]), c[:, n], q[:, n], agg.frags[h].n_occ,
                                 agg.frags[l].n_virt))
    return states


def aggregate_of(monomers, setup):
    """The Aggregate of an FMO set-up: `monomers` carry .index, .system (ao_offset, n_occ, n_atoms,
    xyz, numbers) and .ground (orbs, orbe, s); `setup` carries .real {(I, J): bool}, .s_block(I, J),
    .gamma, .gamma_lr and .pair_scc (the host set-up of the GPU path provides these)."""
    frags = []
    off = 0
    for m in monomers:
        sy, g = m.system, m.ground
        frags.append(Frag(m.index, np.arange(off, off + sy.n_atoms), sy.ao_offset, g.orbs, g.orbe, g.s, sy.n_occ,
                          sy.xyz, sy.numbers))
        off += sy.n_atoms
    types = {k: ("pair" if v else "esd") for k, v in setup.real.items()}
    return Aggregate(frags, setup.s_block, setup.gamma, setup.gamma_lr, types, setup.pair_scc)


def basis_of(agg, labels, results, ct_pairs, n_le, n_ct):
    """`diabatic_basis` from a solved work list: labels[k] = ("LE", I) or ("CT", h, l), results[k]
    a dict with energies, coefficients and (CT) q_trans."""
    le, ct = {}, {}
    for k, lab in enumerate(labels):
        r = results[k]
        if lab[0] == "LE":
            le[lab[1]] = (r["energies"], r["coefficients"])
        else:
            ct[(lab[1], lab[2])] = (r["energies"], r["coefficients"], r["q_trans"])
    return diabatic_basis(agg, le, ct, ct_pairs, n_le, n_ct)


# ----------------------------------------------------------------------------------------------
# transition charges between orbitals of two monomers
# ----------------------------------------------------------------------------------------------

def q_between(fa, fb, ca, cb, s_ab):
    """Mulliken transition charges between orbitals ca (columns, on monomer a's AOs) and cb (on b's
    AOs) with the AO overlap s_ab between a and b: [N_a + N_b, ncol(ca), ncol(cb)], the charges on a's
    atoms first (`q_lele` :21-86, `q_lect` :276-426, `q_ctct` :428-586)."""
    sc_b = s_ab @ cb          # on a's AOs
    sc_a = s_ab.T @ ca        # on b's AOs
    q = np.zeros((fa.n_atoms + fb.n_atoms, ca.shape[1], cb.shape[1]))
    for A in range(fa.n_atoms):
        mu = slice(fa.ao_offset[A], fa.ao_offset[A + 1])
        q[A] = ca[mu].T @ sc_b[mu]
    for B in range(fb.n_atoms):
        mu = slice(fb.ao_offset[B], fb.ao_offset[B + 1])
        q[fa.n_atoms + B] = sc_a[mu].T @ cb[mu]
    return 0.5 * q


def exchange_contract(q_ij, q_ab, b_ia, b_jb, gamma_lr):
    """tincr's exchange contraction (integrals.rs:137-166 and its copies):
    trace(ab_bjb . bia_ij^T . gamma_lr) with bia_ij[A, a j] = sum_i q_ij[A, i, j] b_ia[i, a] and
    ab_bjb[B, a j] = sum_b q_ab[B, a, b] b_jb[j, b]."""
    na_ij, n_i, n_j = q_ij.shape
    na_ab, n_a, n_b = q_ab.shape
    bia_ij = (np.ascontiguousarray(q_ij.transpose(0, 2, 1)).reshape(na_ij * n_j, n_i) @ b_ia) \
        .reshape(na_ij, n_j, n_a).transpose(0, 2, 1).reshape(na_ij, n_a * n_j)
    ab_bjb = (q_ab.reshape(na_ab * n_a, n_b) @ b_jb.T).reshape(na_ab, n_a * n_j)
    return float(np.trace(ab_bjb @ bia_ij.T @ gamma_lr))


# ----------------------------------------------------------------------------------------------
# couplings
# ----------------------------------------------------------------------------------------------

def le_le(agg, a, b):
    """`le_le` (integrals.rs:81-169): 2 Coulomb - exchange (exchange for real pairs only, full
    orbital spaces, dimer gamma_lr)."""
    fa, fb = agg.frags[a.m], agg.frags[b.m]
    coulomb = a.q_trans @ agg.g(a.m, b.m, False) @ b.q_trans
    exchange = 0.0
    if agg.type_of_pair(a.m, b.m) == "pair":
        s_ab = agg.s_block(a.m, b.m)
        q_ij = q_between(fa, fb, fa.occs, fb.occs, s_ab)
        q_ab = q_between(fa, fb, fa.virts, fb.virts, s_ab)
        exchange = exchange_contract(q_ij, q_ab, a.tdm, b.tdm, agg.g_ab_cd(a.m, b.m, a.m, b.m, True))
    return 2.0 * coulomb - exchange


def fock_block(fock, off, i, j):
    """MO block (monomer i, monomer j) of the LCMO Fock matrix: `fock` is the dense matrix of
    `lcmo_fock` (with its offsets `off`) or a callable (i, j) -> block, such as `LcmoFockBlocks`."""
    if callable(fock):
        return fock(i, j)
    return fock[off[i]:off[i + 1], off[j]:off[j + 1]]


def le_ct_1e(agg, fock, off, le, ct):
    """`le_ct_1e_new` (integrals.rs:542-600): one-electron coupling through the LCMO Fock matrix
    when the LE monomer carries the CT state's electron (occupied block, minus sign) or hole
    (virtual block)."""
    fi = agg.frags[le.m]
    if le.m == ct.m_l:
        fh = agg.frags[ct.m_h]
        f_ij = fock_block(fock, off, le.m, ct.m_h)[:fi.n_occ, :fh.n_occ]
        t_ij = le.tdm @ ct.tdm.T
        return -float(np.sum(f_ij * t_ij))
    if le.m == ct.m_h:
        fl = agg.frags[ct.m_l]
        f_ab = fock_block(fock, off, le.m, ct.m_l)[fi.n_occ:, fl.n_occ:]
        t_ab = le.tdm.T @ ct.tdm
        return float(np.sum(f_ab * t_ab))
    return 0.0


def le_ct_2e(agg, le, ct):
    """`le_ct_2e_new` (integrals.rs:602-727): 2 Coulomb - exchange in the restricted active space."""
    fi = agg.frags[le.m]
    fh, fl = agg.frags[ct.m_h], agg.frags[ct.m_l]
    coulomb = le.q_trans @ (agg.g_ab_c(ct.m_h, ct.m_l, le.m, False).T @ ct.q_tr)
    t_h, t_l = agg.type_of_pair(le.m, ct.m_h), agg.type_of_pair(le.m, ct.m_l)
    exchange = 0.0
    if t_h in ("pair", None) or t_l in ("pair", None):
        no = fi.n_occ
        if le.m == ct.m_h:
            q_ij = fi.q_oo.reshape(fi.n_atoms, no, no)[:, no - ACTIVE_LE:, no - ACTIVE_CT:]
        else:
            q_ij = q_between(fi, fh, fi.occs[:, no - ACTIVE_LE:], fh.occs[:, fh.n_occ - ACTIVE_CT:],
                             agg.s_block(le.m, ct.m_h))
        if le.m == ct.m_l:
            q_ab = fi.q_vv.reshape(fi.n_atoms, fi.n_virt, fi.n_virt)[:, :ACTIVE_LE, :ACTIVE_CT]
        else:
            q_ab = q_between(fi, fl, fi.virts[:, :ACTIVE_LE], fl.virts[:, :ACTIVE_CT], agg.s_block(le.m, ct.m_l))
        if le.m == ct.m_h:
            glr = agg.g_ab_c(le.m, ct.m_l, le.m, True).T
        elif le.m == ct.m_l:
            glr = agg.g_ab_c(le.m, ct.m_h, le.m, True)
        else:
            glr = agg.g_ab_cd(le.m, ct.m_h, le.m, ct.m_l, True)
        b_ia = le.tdm[no - ACTIVE_LE:, :ACTIVE_LE]
        b_jb = ct.tdm[fh.n_occ - ACTIVE_CT:, :ACTIVE_CT]
        exchange = exchange_contract(q_ij, q_ab, b_ia, b_jb, glr)
    return 2.0 * coulomb - exchange


def ct_ct(agg, s1, s2):
    """`ct_ct_new` (integrals.rs:733-878): 2 Coulomb - exchange in the restricted active space (the
    exchange when the hole monomers and the electron monomers are each the same monomer or a real
    pair, but not both the same)."""
    coulomb = s1.q_tr @ agg.g_ab_cd(s1.m_h, s1.m_l, s2.m_h, s2.m_l, False) @ s2.q_tr
    t_hh, t_ll = agg.type_of_pair(s1.m_h, s2.m_h), agg.type_of_pair(s1.m_l, s2.m_l)
    exchange = 0.0
    if t_hh in ("pair", None) and t_ll in ("pair", None):
        fh1, fh2 = agg.frags[s1.m_h], agg.frags[s2.m_h]
        fl1, fl2 = agg.frags[s1.m_l], agg.frags[s2.m_l]
        if s1.m_h == s2.m_h:
            no = fh1.n_occ
            q_ij = fh1.q_oo.reshape(fh1.n_atoms, no, no)[:, no - ACTIVE_CT:, no - ACTIVE_CT:]
        else:
            q_ij = q_between(fh1, fh2, fh1.occs[:, fh1.n_occ - ACTIVE_CT:], fh2.occs[:, fh2.n_occ - ACTIVE_CT:],
                             agg.s_block(s1.m_h, s2.m_h))
        if s1.m_l == s2.m_l:
            nv = fl1.n_virt
            q_ab = fl1.q_vv.reshape(fl1.n_atoms, nv, nv)[:, :ACTIVE_CT, :ACTIVE_CT]
        else:
            q_ab = q_between(fl1, fl2, fl1.virts[:, :ACTIVE_CT], fl2.virts[:, :ACTIVE_CT],
                             agg.s_block(s1.m_l, s2.m_l))
        if s1.m_h == s2.m_h:
            glr = agg.g_ab_c(s1.m_l, s2.m_l, s1.m_h, True).T
        elif s1.m_l == s2.m_l:
            glr = agg.g_ab_c(s1.m_h, s2.m_h, s1.m_l, True)
        else:
            glr = agg.g_ab_cd(s1.m_h, s2.m_h, s1.m_l, s2.m_l, True)
        b_ia = s1.tdm[fh1.n_occ - ACTIVE_CT:, :ACTIVE_CT]
        b_jb = s2.tdm[fh2.n_occ - ACTIVE_CT:, :ACTIVE_CT]
        exchange = exchange_contract(q_ij, q_ab, b_ia, b_jb, glr)
    return 2.0 * coulomb - exchange


def exciton_coupling(agg, fock, off, a, b):
    """`exciton_coupling` (integrals.rs:17-79) for the LE and pair-CT states."""
    if isinstance(a, LE) and isinstance(b, LE):
        if a.m == b.m:
            return a.energy if a.n == b.n else 0.0
        return le_le(agg, a, b)
    if isinstance(a, LE):
        return le_ct_1e(agg, fock, off, a, b) + le_ct_2e(agg, a, b)
    if isinstance(b, LE):
        return le_ct_1e(agg, fock, off, b, a) + le_ct_2e(agg, b, a)
    if a.m_h == b.m_h and a.m_l == b.m_l:
        return a.energy if a.n == b.n else 0.0
    return ct_ct(agg, a, b)


def exciton_hamiltonian(agg, states, fock=None, off=None):
    """The exciton matrix (basis.rs:471-495): the upper triangle element by element, then
    H + H^T - diag(H)."""
    if fock is None:
        fock, off = lcmo_fock(agg)
    dim = len(states)
    h = np.zeros((dim, dim))
    for i in range(dim):
        for j in range(i, dim):
            h[i, j] = exciton_coupling(agg, fock, off, states[i], states[j])
    return h + h.T - np.diag(np.diag(h))


_ROWS = {}


def _rows_init(agg, states, fock, off):
    _ROWS.update(agg=agg, states=states, fock=fock, off=off)


def _row(i):
    st = _ROWS["states"]
    return i, [exciton_coupling(_ROWS["agg"], _ROWS["fock"], _ROWS["off"], st[i], st[j]) for j in range(i, len(st))]


def exciton_hamiltonian_rows(agg, states, workers, fock=None, off=None):
    """`exciton_hamiltonian` with the rows of the upper triangle shared out to `workers` processes,
    as tincr shares them out to rayon threads (`states.par_iter()`, basis.rs:479-487).  Every element
    is the same function of the same inputs, so the matrix equals the serial one.  The workers are
    spawned with one BLAS thread each; the caller must run under a `__main__` guard."""
    if fock is None:
        fock, off = lcmo_fock(agg)
    dim = len(states)
    if workers <= 1:
        return exciton_hamiltonian(agg, states, fock, off)
    import multiprocessing as mp
    import os
    from concurrent.futures import ProcessPoolExecutor
    names = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")
    saved = {k: os.environ.get(k) for k in names}
    os.environ.update({k: "1" for k in names})
    h = np.zeros((dim, dim))
    try:
        with ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn"), initializer=_rows_init,
                                 initargs=(agg, states, fock, off)) as ex:
            # long rows first, so the short ones fill in at the end
            for i, row in ex.map(_row, range(dim), chunksize=max(1, dim // (16 * workers))):
                h[i, i:] = row
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    return h + h.T - np.diag(np.diag(h))


class DenseEngine:
    """Davidson engine of a dense matrix (src/excited_states/solvers/mod.rs:36-51)."""

    def __init__(self, h):
        self.h = h
        self.d = np.diag(h).copy()

    def compute_products(self, x):
        return self.h @ x

    def precondition(self, r_k, w_k):
        return r_k / (w_k - self.d)

    def get_size(self):
        return self.h.shape[0]


def exciton_states(h, n_roots, tol=1e-4, max_iter=100):
    """Lowest roots of the exciton matrix by tincr's Davidson (basis.rs:497-503):
    (energies, eigenvectors [dim, n_roots], iterations)."""
    guess = OT.initial_subspace(np.diag(h), n_roots)
    return OT.davidson(DenseEngine(h), guess, n_roots, tol, max_iter)
