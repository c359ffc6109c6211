"""CT-state gradient: the oracle's restatement of tincr's amplitude projection and the host side of
`fmo.ct_state_gradients` (no GPU).

* known answer: with dimer orbitals that are the two monomers' orbitals side by side (any column
  order), the projected amplitudes are the CT amplitudes placed at the dimer's occupied orbitals of
  the hole monomer and virtual orbitals of the electron monomer, in both hole directions;
* the host projection of `fmo.ct_amplitudes_in_pair` equals the oracle's on a water-ammonia pair
  with its SCC ground state (1e-13), for pair-TDA-like amplitudes and tincr's single-orbital CT;
* two monomers beyond the Slater-Koster range: the dimer's orbitals stay on one monomer each, and
  the projected amplitudes vanish on every orbital of the wrong monomer (1e-13);
* tincr's single-orbital convention (HOMO - k of the hole, LUMO + l of the electron);
* the oracle's CT gradient is translation invariant (sum over atoms below 1e-12);
* the host logic of `fmo.exciton_gradient`: the basis order of `exciton_states`, no terms below
  the threshold, argument checks;
* against central differences of the lowest pair-TDA CT energy (tincr's own check of this
  gradient): within 5 % / 2 % of the largest component at 5.5 / 10 bohr, the gap being the
  monomer-orbital response that the dimer gradient leaves out."""

import numpy as np
import pytest

from cases import golden
from oracle import ct_gradient as OCT
from tincr_gb300 import fmo
from tincr_gb300 import groundstate as gs
from tincr_gb300.params import NUMBERS


def test_projection_known_answer():
    rng = np.random.default_rng(7)
    ni, nj, oi, oj = 5, 4, 2, 1
    c_i = np.linalg.qr(rng.standard_normal((ni, ni)))[0]
    c_j = np.linalg.qr(rng.standard_normal((nj, nj)))[0]
    # dimer orbitals: occupied (I occ, J occ) then virtual (J virt, I virt), in a shuffled order
    cols = [("i", k) for k in range(oi)] + [("j", k) for k in range(oj)]
    cols = [cols[1], cols[2], cols[0]]
    vcols = [("j", k) for k in range(oj, nj)] + [("i", k) for k in range(oi, ni)]
    vcols = vcols[::-1]
    c_ij = np.zeros((ni + nj, ni + nj))
    for n, (m, k) in enumerate(cols + vcols):
        if m == "i":
            c_ij[:ni, n] = c_i[:, k]
        else:
            c_ij[ni:, n] = c_j[:, k]
    s = np.eye(ni + nj)
    s_i, s_j = OCT.monomer_pair_overlaps(c_i, c_j, c_ij, s, ni)
    no = oi + oj
    for hole_i in (True, False):
        oh, vl = (oi, nj - oj) if hole_i else (oj, ni - oi)
        x_ct = rng.standard_normal((oh, vl))
        x = OCT.ct_amplitudes_in_pair(s_i, s_j, oi, oj, no, x_ct, hole_i)
        want = np.zeros((no, ni + nj - no))
        hm, lm = ("i", "j") if hole_i else ("j", "i")
        lo = oj if hole_i else oi
        for a, col in enumerate(cols):
            for b, vcol in enumerate(vcols):
                if col[0] == hm and vcol[0] == lm:
                    want[a, b] = x_ct[col[1], vcol[1] - lo]
        assert np.abs(x - want).max() < 1e-14


def _pair(shift_bohr):
    mols = []
    for name in ("h2o", "ammonia"):
        d = golden(name)
        mols.append((np.array([NUMBERS[s] for s in d["symbols"]], np.int32), d["xyz_angstrom"] / 0.529177210903))
    z = np.concatenate([mols[0][0], mols[1][0]])
    x = np.concatenate([mols[0][1], mols[1][1] + np.array([0.0, 0.0, shift_bohr])])
    mono = np.concatenate([np.zeros(len(mols[0][0]), int), np.ones(len(mols[1][0]), int)])
    mons = fmo.build_monomers(z, x, mono, lc=True)
    sy = gs.build_system(z, x, lc=True)
    g = gs.run_scc(sy, tol=1e-11,
                   p_start=np.block([[mons[0].ground.p, np.zeros((mons[0].system.n_orbs, mons[1].system.n_orbs))],
                                     [np.zeros((mons[1].system.n_orbs, mons[0].system.n_orbs)), mons[1].ground.p]]))
    assert g.converged
    return mons, sy, g


def test_host_projection_matches_oracle():
    mons, sy, g = _pair(5.5)
    mi, mj = mons
    rng = np.random.default_rng(3)
    for hole_i in (True, False):
        mh, ml = (mi, mj) if hole_i else (mj, mi)
        for x_ct in (rng.standard_normal((mh.system.n_occ, ml.system.n_virt)),
                     fmo.ct_unit_amplitudes(mons, mh.index, ml.index, 1, 0)):
            got = fmo.ct_amplitudes_in_pair(mi, mj, sy, g, x_ct, hole_i)
            s_i, s_j = OCT.monomer_pair_overlaps(mi.ground.orbs, mj.ground.orbs, g.orbs, g.s, mi.system.n_orbs)
            want = OCT.ct_amplitudes_in_pair(s_i, s_j, mi.system.n_occ, mj.system.n_occ, sy.n_occ, x_ct, hole_i)
            assert got.shape == (sy.n_occ, sy.n_virt)
            assert np.abs(got - want).max() < 1e-13


def test_projection_of_separated_monomers_stays_on_them():
    mons, sy, g = _pair(60.0)
    mi, mj = mons
    ni = mi.system.n_orbs
    on_i = np.abs(g.orbs[:ni, :]).max(axis=0) > 1e-10
    on_j = np.abs(g.orbs[ni:, :]).max(axis=0) > 1e-10
    assert not np.any(on_i & on_j)          # every dimer orbital lives on one monomer
    no = sy.n_occ
    x_ct = fmo.ct_unit_amplitudes(mons, 0, 1, 0, 0)
    x = fmo.ct_amplitudes_in_pair(mi, mj, sy, g, x_ct, True)
    assert np.abs(x[on_j[:no], :]).max() < 1e-13
    assert np.abs(x[:, on_i[no:]]).max() < 1e-13
    assert abs(np.linalg.norm(x) - 1.0) < 1e-3  # the monomers' orbitals barely change in the dimer


def test_unit_amplitudes_follow_tincr():
    mons, _, _ = _pair(5.5)
    for h, l, k, m in ((0, 1, 0, 0), (0, 1, 2, 1), (1, 0, 1, 1)):
        a = fmo.ct_unit_amplitudes(mons, h, l, k, m)
        b = OCT.ct_unit_amplitudes(mons[h].system.n_occ, mons[l].system.n_virt, k, m)
        assert np.array_equal(a, b)
        assert a[mons[h].system.n_occ - 1 - k, m] == 1.0 and a.sum() == 1.0
    with pytest.raises(ValueError):   # water has two virtual orbitals
        fmo.ct_unit_amplitudes(mons, 1, 0, 0, 2)
    with pytest.raises(ValueError):
        fmo.ct_unit_amplitudes(mons, 0, 1, mons[0].system.n_occ, 0)


def test_oracle_ct_gradient_is_translation_invariant():
    """The CT gradient contracts derivatives of S, H0 and gamma, which depend on relative positions
    only: summed over the atoms it vanishes in each direction."""
    mons, sy, g = _pair(5.5)
    mi, mj = mons
    x_ct = np.random.default_rng(1).standard_normal((mi.system.n_occ, mj.system.n_virt))
    x_ct /= np.linalg.norm(x_ct)
    grad, x = OCT.ct_state_gradient(sy, g, mi.system.n_orbs, mi.ground.orbs, mj.ground.orbs, mi.system.n_occ,
                                    mj.system.n_occ, x_ct, 0.4, True)
    assert grad.shape == (3 * sy.n_atoms,) and np.abs(grad).max() > 1e-3
    assert np.abs(grad.reshape(-1, 3).sum(axis=0)).max() < 1e-12


def test_ct_gradient_argument_checks():
    """tincr's ct_gradient_new takes the lower monomer index first; a CT term needs two monomers and
    amplitudes over the hole's occupied x the electron's virtual orbitals; all checked before any
    GPU work."""
    mons, sy, g = _pair(5.5)
    with pytest.raises(ValueError):
        fmo.ct_gradient(None, mons, 1, 0, 0, 0, 0.3, True)
    with pytest.raises(ValueError):
        fmo.ct_state_gradients(None, mons, [(0, 0, np.zeros((4, 2)), 0.3)])
    with pytest.raises(ValueError):   # water -> ammonia: 4 x 3 amplitudes, not 4 x 2
        fmo.ct_amplitudes_in_pair(mons[0], mons[1], sy, g, np.zeros((4, 2)), True)
    grads, states = fmo.ct_state_gradients(None, mons, [])
    assert grads == [] and states == {}


def test_exciton_basis_order_and_empty_gradient():
    """The basis of `exciton_states` (n_le LE roots per monomer, then (i -> j, n), (j -> i, n) per CT
    pair and root), and an exciton vector with every coefficient at or below the threshold: no term,
    no GPU work, a zero gradient."""
    from cases import fmo_case
    c = fmo_case(3, 1, 1)
    mons, labels = c["monomers"], c["labels"]
    n_le, n_ct = 4, 1
    results = [dict(energies=np.zeros(n_le if lab[0] == "LE" else n_ct), coefficients=None) for lab in labels]
    basis, ct_of = fmo.exciton_basis(labels, results, len(mons), n_le, n_ct, c["pairs"])
    assert len(basis) == len(mons) * n_le + 2 * n_ct * len(c["pairs"])
    assert basis[:n_le] == [("LE", 0, r) for r in range(n_le)]
    i, j = c["pairs"][0]
    assert basis[len(mons) * n_le:len(mons) * n_le + 2] == [("CT", i, j, 0), ("CT", j, i, 0)]
    assert set(ct_of) == {(a, b) for a, b in c["pairs"]} | {(b, a) for a, b in c["pairs"]}

    class _Setup:
        monomers, ct_pairs = mons, c["pairs"]

    v = np.full(len(basis), 0.01)
    grad, n_le_t, n_ct_t, states = fmo.exciton_gradient(None, _Setup, results, labels, n_le, n_ct, v)
    assert n_le_t == 0 and n_ct_t == 0 and states == {}
    assert grad.shape == (3 * sum(m.system.n_atoms for m in mons),) and not grad.any()
    with pytest.raises(ValueError):
        fmo.exciton_gradient(None, _Setup, results, labels, n_le, n_ct, v[:-1])
    assert fmo.run_gradient_jobs([]) == []


def _ct_energy(z, x, mono):
    """Lowest pair-TDA CT energy water -> ammonia (tincr's `new_fmo_ct_energy_wrapper`,
    src/fmo/gradients/numerical.rs:147-189, dense) and its amplitudes, from isolated monomer SCCs."""
    from cases import fmo_oracle_engine
    mons = fmo.build_monomers(z, x, mono, lc=True, scc_tol=1e-12)
    _, labels = fmo.aggregate_instances(mons, [(0, 1)], 1, 3)
    eng, _ = fmo_oracle_engine(dict(monomers=mons, labels=labels, lc=True), labels.index(("CT", 0, 1)))
    a = eng.apply(np.eye(eng.n_occ * eng.n_virt))
    e, v = np.linalg.eigh(0.5 * (a + a.T))
    return e[0], v[:, 0], mons


def test_ct_gradient_against_finite_differences_of_the_ct_energy():
    """tincr checks this gradient against central differences of the lowest pair-TDA CT energy
    (`test_new_charge_transfer_gradient`, numerical.rs:254-265).  The dimer's TDA gradient at the
    projected amplitudes leaves out the response of the monomer orbitals the CT state is built from
    (tincr's CPHF correction), so it matches only to a few per cent at contact, closer at larger
    separation; a wrong projection or sign would be off by the whole gradient."""
    gaps = []
    for shift in (5.5, 10.0):
        mons0, _, _ = _pair(shift)
        z = np.concatenate([m.system.numbers for m in mons0])
        x = np.concatenate([m.system.xyz for m in mons0])
        mono = np.concatenate([np.full(m.system.n_atoms, k) for k, m in enumerate(mons0)])
        e0, v0, mons = _ct_energy(z, x, mono)
        mi, mj = mons
        sy = gs.build_system(z, x, lc=True)
        ni, nj = mi.system.n_orbs, mj.system.n_orbs
        p = np.zeros((ni + nj, ni + nj))
        p[:ni, :ni], p[ni:, ni:] = mi.ground.p, mj.ground.p
        g = gs.run_scc(sy, tol=1e-12, p_start=p)
        grad, _ = OCT.ct_state_gradient(sy, g, ni, mi.ground.orbs, mj.ground.orbs, mi.system.n_occ, mj.system.n_occ,
                                        v0.reshape(mi.system.n_occ, -1), e0, True)
        h = 1e-4
        fd = np.zeros_like(grad)
        for c in range(len(fd)):
            xp, xm = x.copy(), x.copy()
            xp[c // 3, c % 3] += h
            xm[c // 3, c % 3] -= h
            fd[c] = (_ct_energy(z, xp, mono)[0] - _ct_energy(z, xm, mono)[0]) / (2 * h)
        gaps.append(np.abs(grad - fd).max() / np.abs(fd).max())
    assert gaps[0] < 0.05 and gaps[1] < 0.02     # measured: 2.8 % at 5.5 bohr, 1.0 % at 10 bohr
    assert gaps[1] < gaps[0]
