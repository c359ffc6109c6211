"""CPU checks of the exciton-Hamiltonian oracle (oracle/exciton.py, tincr's FMO exciton model) on a
small seeded acene aggregate:

* an LE-LE coupling of a real pair equals X_I^T (A X_J) with A the TDA operator of the dimer in the
  basis of both monomers' orbitals (2 Coulomb - exchange is the off-diagonal block of the dimer's
  A: an independent restatement of `le_le`'s reshapes);
* the matrix element functions give the same value in both orders (the matrix is symmetric before
  tincr fills the lower triangle from the upper one);
* the Davidson on the exciton matrix gives its lowest eigenvalues;
* the LCMO Fock matrix is symmetric and reduces to the orbital energies without real pairs."""

import numpy as np
import pytest

from cases import fmo_case, fmo_oracle_engine
from oracle import exciton as OX
from oracle import tda as OT
from tincr_gb300 import fmo
from tincr_gb300 import groundstate as gs


def _aggregate(nx=3, ny=1, nz=1):
    c = fmo_case(nx, ny, nz)
    mons = c["monomers"]
    setup = fmo.ExcitonSetup(mons, c["pairs"])
    frags = []
    off = 0
    for m in mons:
        sy, g = m.system, m.ground
        frags.append(OX.Frag(m.index, np.arange(off, off + sy.n_atoms), sy.ao_offset, g.orbs, g.orbe, g.s, sy.n_occ,
                             sy.xyz, sy.numbers))
        off += sy.n_atoms
    types = {k: ("pair" if v else "esd") for k, v in setup.real.items()}
    agg = OX.Aggregate(frags, setup.s_block, setup.gamma, setup.gamma_lr, types, setup.pair_scc)
    le, ct = {}, {}
    for k, lab in enumerate(c["labels"]):
        eng, xyz = fmo_oracle_engine(c, k)
        r = OT.run_tda_engine(eng, xyz, c["instances"][k]["n_roots"], 150, 1e-8)
        if lab[0] == "LE":
            le[lab[1]] = (r["energies"], r["coefficients"])
        else:
            ct[(lab[1], lab[2])] = (r["energies"], r["coefficients"], r["q_trans"])
    states = OX.diabatic_basis(agg, le, ct, c["pairs"], 4, 1)
    return c, setup, agg, states


@pytest.fixture(scope="module")
def agg3():
    return _aggregate()


def _dimer_engine(agg, i, j):
    """TDA product engine of the dimer (i, j) in the basis [occ_i, occ_j] x [virt_i, virt_j]."""
    fi, fj = agg.frags[i], agg.frags[j]
    ni, nj = fi.n_orb, fj.n_orb
    c = np.zeros((ni + nj, ni + nj))
    c[:ni, :fi.n_occ] = fi.occs
    c[ni:, fi.n_occ:fi.n_occ + fj.n_occ] = fj.occs
    o = fi.n_occ + fj.n_occ
    c[:ni, o:o + fi.n_virt] = fi.virts
    c[ni:, o + fi.n_virt:] = fj.virts
    e = np.concatenate([fi.orbe[:fi.n_occ], fj.orbe[:fj.n_occ], fi.orbe[fi.n_occ:], fj.orbe[fj.n_occ:]])
    s = np.block([[fi.s, agg.s_block(i, j)], [agg.s_block(j, i), fj.s]])
    ao = np.concatenate([fi.ao_offset[:-1], ni + fj.ao_offset])
    occ, virt = np.arange(o), np.arange(o, ni + nj)
    q_ov, q_oo, q_vv = OT.trans_charges(ao, c, s, occ, virt)
    atoms = np.concatenate([fi.atoms, fj.atoms])
    g, glr = agg.gamma[np.ix_(atoms, atoms)], agg.gamma_lr[np.ix_(atoms, atoms)]
    om = OT.orbe_differences(e[occ], e[virt])
    return OT.TdaEngine(om, q_ov, g, q_oo, q_vv, glr, o, len(virt))


def test_le_le_coupling_is_the_dimer_matrix_block(agg3):
    c, setup, agg, states = agg3
    les = [s for s in states if isinstance(s, OX.LE)]
    checked = 0
    for (i, j), t in agg.pair_types.items():
        if t != "pair":
            continue
        eng = _dimer_engine(agg, i, j)
        fi, fj = agg.frags[i], agg.frags[j]
        v = fi.n_virt + fj.n_virt
        for a in [s for s in les if s.m == i]:
            xa = np.zeros((fi.n_occ + fj.n_occ, v))
            xa[:fi.n_occ, :fi.n_virt] = a.tdm
            for b in [s for s in les if s.m == j]:
                xb = np.zeros_like(xa)
                xb[fi.n_occ:, fi.n_virt:] = b.tdm
                ref = xa.reshape(-1) @ eng.apply(xb.reshape(-1, 1))[:, 0]
                assert abs(OX.le_le(agg, a, b) - ref) < 1e-12
                checked += 1
    assert checked >= 16


def test_couplings_symmetric_and_davidson_roots(agg3):
    c, setup, agg, states = agg3
    fock, off = OX.lcmo_fock(agg)
    assert np.abs(fock - fock.T).max() < 1e-12
    n = len(states)
    for a in range(n):
        for b in range(a + 1, n):
            x = OX.exciton_coupling(agg, fock, off, states[a], states[b])
            y = OX.exciton_coupling(agg, fock, off, states[b], states[a])
            assert abs(x - y) < 1e-12
    h = OX.exciton_hamiltonian(agg, states, fock, off)
    e, v, it = OX.exciton_states(h, 5, tol=1e-8, max_iter=200)
    assert np.abs(e - np.linalg.eigvalsh(h)[:5]).max() < 1e-10


def test_lcmo_fock_without_real_pairs_is_diagonal(agg3):
    c, setup, agg, states = agg3
    esd = OX.Aggregate(agg.frags, agg.s_block, agg.gamma, agg.gamma_lr,
                       {k: "esd" for k in agg.pair_types}, {})
    fock, off = OX.lcmo_fock(esd)
    assert np.allclose(fock, np.diag(np.concatenate([f.orbe for f in agg.frags])), atol=0, rtol=0)


def test_dimer_scc_from_monomer_densities():
    """The exciton set-up starts each dimer SCC from its two monomers' converged densities (tincr
    starts a pair SCC from its monomers' charges); it must reach the ground state the neutral-atom
    start reaches, and an SCC that misses its tolerance must say so (tincr panics there)."""
    c = fmo_case(2, 1, 1)
    a, b = c["monomers"]
    sy = gs.build_system(np.concatenate([a.system.numbers, b.system.numbers]),
                         np.concatenate([a.system.xyz, b.system.xyz]), lc=True, r_lr=a.system.r_lr)
    ref = gs.run_scc(sy, tol=1e-10)
    assert ref.converged
    na = a.system.n_orbs
    p_start = np.zeros_like(ref.p)
    p_start[:na, :na] = a.ground.p
    p_start[na:, na:] = b.ground.p
    g = gs.run_scc(sy, tol=1e-10, p_start=p_start, require_convergence=True)
    assert g.converged and g.iterations < ref.iterations
    assert abs(g.energy - ref.energy) < 1e-9
    assert np.abs(g.orbe - ref.orbe).max() < 1e-8
    assert not gs.run_scc(sy, tol=1e-10, max_iter=2).converged
    with pytest.raises(RuntimeError):
        gs.run_scc(sy, tol=1e-10, max_iter=2, require_convergence=True)
    # the level shift (the fallback for dimers whose occupations swap) keeps the stationary density
    gsh = gs.run_scc(sy, tol=1e-10, p_start=p_start, level_shift=0.5, max_iter=1000, require_convergence=True)
    assert abs(gsh.energy - ref.energy) < 1e-9
    assert np.abs(gsh.orbe - ref.orbe).max() < 1e-8


def test_lcmo_fock_blocks_equal_the_dense_matrix(agg3):
    """The block-by-block LCMO Fock matrix (for aggregates too large for the dense x^T F x) equals
    the dense one on every pair of monomers."""
    c, setup, agg, states = agg3
    fock, off = OX.lcmo_fock(agg)
    fb = OX.LcmoFockBlocks(agg)
    n = len(agg.frags)
    for i in range(n):
        for j in range(n):
            assert np.abs(fb(i, j) - fock[off[i]:off[i + 1], off[j]:off[j + 1]]).max() < 1e-12
    # and the couplings through it
    for a in range(len(states)):
        for b in range(len(states)):
            assert abs(OX.exciton_coupling(agg, fb, None, states[a], states[b]) -
                       OX.exciton_coupling(agg, fock, off, states[a], states[b])) < 1e-12
