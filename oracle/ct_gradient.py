"""Oracle: gradient of a charge-transfer state of a monomer pair (tincr's CT terms of the FMO
exciton-state gradient).

tincr differentiates a CT state I -> J as an excited state of the dimer IJ: it writes the CT
amplitudes, given over the hole monomer's occupied and the electron monomer's virtual orbitals, in
the dimer's own orbitals and takes the dimer's TDA gradient at that single state, with the CT
energy as its excitation energy.  Restated here:

* `monomer_pair_overlaps`: the overlaps between the monomers' and the dimer's orbitals,
  S_I,IJ = C_I^T S[I rows, :] C_IJ and S_J,IJ = C_J^T S[J rows, :] C_IJ
  (`build_lcmo_fock_matrix`, src/fmo/lcmo/hamiltonian.rs:61-64, stored by `set_overlap_i_ij` /
  `set_overlap_j_ij` at :89-90);
* `ct_amplitudes_in_pair`: X_IJ = S_h,IJ[occ_h, occ_IJ]^T X_CT S_l,IJ[virt_l, virt_IJ]
  (`Pair::prepare_charge_transfer_gradient`, src/fmo/gradients/ct_state_new.rs:115-150, for the
  pair-TDA CT states of `create_diab_basis_new`; `Pair::prepare_ct_state`,
  src/fmo/gradients/excited_state.rs:1166-1212, for the single hole -> electron orbital pairs of
  `create_diab_basis`, whose X_CT is `ct_unit_amplitudes`);
* `ct_state_gradient`: `Pair::tda_gradient_lc(0)` (src/fmo/gradients/excited_state.rs:1470-1713)
  with ci_eigenvalues = [E_CT] and ci_coefficients = X_IJ.  That routine is
  `System::tda_gradient_lc` (src/gradients/excited_state.rs:259-487) on the pair's quantities: its
  r_ia round trip through a Fortran-ordered copy (:1556-1557) returns r_ia itself, and it forms
  f_lr(P - P0) inline where the system version reads it from its properties.  The dimer quantities
  are those of `Pair::prepare_lcmo_gradient` (src/fmo/gradients/pair.rs:220-350): the dimer's S,
  gamma, gamma_lr, their derivatives and the transition charges of the dimer's orbitals.

The pair's gamma there is assembled from the monomers' blocks and `gamma_atomwise_ab` over
`pair_atoms[0..n_I]` and `pair_atoms[n_J..]` (pair.rs:244-250), which is the dimer's gamma only when
both monomers have the same atom count (otherwise the block does not fit and the assignment fails);
this restatement uses the dimer's gamma, which equals tincr's wherever tincr's runs.

Test infrastructure only (see oracle/__init__.py).
"""

import numpy as np

from . import gradients as OG
from . import tda as OT


def monomer_pair_overlaps(c_i, c_j, c_ij, s_pair, n_orb_i):
    """(S_I,IJ [n_I, n_IJ], S_J,IJ [n_J, n_IJ]) of hamiltonian.rs:61-64; monomer I's AOs come
    first in the dimer."""
    s_i = c_i.T @ s_pair[:n_orb_i, :] @ c_ij
    s_j = c_j.T @ s_pair[n_orb_i:, :] @ c_ij
    return s_i, s_j


def ct_unit_amplitudes(n_occ_h, n_virt_l, ct_ind_h, ct_ind_l):
    """X_CT of the single orbital pair of `prepare_ct_state` (excited_state.rs:1176-1179): one at
    (HOMO - ct_ind_h of the hole monomer, LUMO + ct_ind_l of the electron monomer)."""
    x = np.zeros((n_occ_h, n_virt_l))
    x[n_occ_h - 1 - ct_ind_h, ct_ind_l] = 1.0
    return x


def ct_amplitudes_in_pair(s_i_ij, s_j_ij, n_occ_i, n_occ_j, n_occ, x_ct, hole_i):
    """X_IJ [n_occ, n_virt] of ct_state_new.rs:115-150 (hole on I when hole_i, else on J); x_ct is
    [n_occ_h, n_virt_l] over the hole monomer's occupied and the electron monomer's virtual
    orbitals."""
    if hole_i:
        return s_i_ij[:n_occ_i, :n_occ].T @ (x_ct @ s_j_ij[n_occ_j:, n_occ:])
    return s_j_ij[:n_occ_j, :n_occ].T @ (x_ct @ s_i_ij[n_occ_i:, n_occ:])


def ct_state_gradient(sy, g, n_orb_i, c_i, c_j, n_occ_i, n_occ_j, x_ct, energy, hole_i, lc=True):
    """Gradient [3 N_IJ] of the CT state (dimer atom order, monomer I first) for the dimer system
    `sy` (groundstate.System) with ground state `g` (orbitals, density, S, gamma, gamma_lr).
    Returns (gradient, X_IJ)."""
    s_i, s_j = monomer_pair_overlaps(c_i, c_j, g.orbs, g.s, n_orb_i)
    x = ct_amplitudes_in_pair(s_i, s_j, n_occ_i, n_occ_j, sy.n_occ, x_ct, hole_i)
    occ, virt = sy.occ_indices, sy.virt_indices
    qov, qoo, qvv = OT.trans_charges(sy.ao_offset, g.orbs, g.s, occ, virt)
    ao = lambda m: m[np.ix_(sy.ao_atom, sy.ao_atom)]
    inp = dict(p=g.p, p0=g.p0, h_coul_x=g.h_coul_x, gamma=g.gamma, dq=g.dq, s=g.s, ao_atom=sy.ao_atom,
               numbers=sy.numbers, xyz=sy.xyz, params=sy.params, gamma_lr_ao=ao(g.gamma_lr) if lc else None,
               orbe=g.orbe, occ=occ, virt=virt, ci_eigenvalues=np.array([float(energy)]),
               ci_coefficients=x.reshape(-1, 1), q_ov=qov, q_oo=qoo, q_vv=qvv,
               gamma_lr=g.gamma_lr if lc else None, orbs=g.orbs, gamma_ao=ao(g.gamma))
    der = OG.derivative_tensors(sy.numbers, sy.xyz, sy.ao_offset, sy.ao_atom, sy.hubbard,
                                sy.r_lr if lc else 0.0, sy.params)
    flr = None
    if lc:
        n = sy.n_orbs
        flr = OG.f_lr(g.p - g.p0, g.s, der["grad_s"], inp["gamma_lr_ao"], der["grad_gamma_lr_ao"], sy.n_atoms, n)
    return OG.tda_gradient(inp, der, 0, lc, flr_dmd0=flr), x
