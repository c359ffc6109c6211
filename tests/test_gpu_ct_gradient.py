"""CT-state and exciton-state gradients on the GPU (`fmo.ct_state_gradients`, `fmo.ct_gradient`,
`fmo.exciton_gradient`) against the oracle restatement of tincr's pair CT gradient
(oracle/ct_gradient.py) on a small seeded acene aggregate (three acenes, two CT pairs of 132 and 186
orbitals).

Both sides read the same dimer ground states (the batched GPU SCC of `fmo.pair_ground_states`) and
the same CT amplitudes (the GPU batch TDA, FP64, converged to 1e-8):
* every CT direction's lowest pair-TDA state: amplitudes in the dimer's orbitals within 1e-12 of the
  oracle's projection, gradient within 1e-9 Eh/bohr; summed over the atoms it vanishes to 1e-5
  (tincr's same-element SK derivative orientation) and, in the "exact" variant, to 1e-8;
* the same without the long-range correction;
* tincr's `ct_gradient_new` form (single orbital pair, hole on the second monomer);
* the exciton-state gradient of the lowest exciton state: the LE part (`exciton_le_gradient`) plus
  c^2 times the oracle's gradient of every CT basis state, within 1e-9 Eh/bohr."""

import numpy as np
import pytest

from cases import fmo_case
from oracle import ct_gradient as OCT
from tincr_gb300 import _lib
from tincr_gb300 import fmo

pytestmark = pytest.mark.gpu

N_LE, N_CT = 4, 1


@pytest.fixture(scope="module")
def solved(gpu_ctx):
    c = fmo_case(3, 1, 1)
    rc, res = fmo.solve_batch(gpu_ctx, c["instances"], 150, 1e-8, _lib.PREC_FP64)
    assert rc == _lib.OK
    return c, res


def _oracle(mons, states, h, l, x_ct, energy):
    i, j = min(h, l), max(h, l)
    sy, g = states[(i, j)]
    mi, mj = mons[i], mons[j]
    return OCT.ct_state_gradient(sy, g, mi.system.n_orbs, mi.ground.orbs, mj.ground.orbs, mi.system.n_occ,
                                 mj.system.n_occ, x_ct, energy, h == i, lc=sy.lc)


def _ct_terms(c, res, root=0):
    mons = c["monomers"]
    out = []
    for k, lab in enumerate(c["labels"]):
        if lab[0] == "CT":
            h, l = lab[1], lab[2]
            x = np.asarray(res[k]["coefficients"])[:, root].reshape(mons[h].system.n_occ, -1)
            out.append((h, l, x, float(res[k]["energies"][root])))
    return out


def test_ct_state_gradients_match_oracle(gpu_ctx, solved):
    c, res = solved
    mons = c["monomers"]
    terms = _ct_terms(c, res)
    grads, states = fmo.ct_state_gradients(gpu_ctx, mons, terms, n_streams=2)
    assert len(grads) == 4 and set(states) == {(0, 1), (1, 2)}
    for (h, l, x, e), gr in zip(terms, grads):
        i, j = min(h, l), max(h, l)
        want, xp = _oracle(mons, states, h, l, x, e)
        got_x = fmo.ct_amplitudes_in_pair(mons[i], mons[j], *states[(i, j)], x, h == i)
        assert np.abs(got_x - xp).max() < 1e-12
        assert gr.shape == want.shape
        assert np.abs(gr - want).max() < 1e-9, (h, l)
        # tincr's same-element SK derivatives put the moving atom at centre 1 (h0_and_s.rs:218), so the
        # C-C terms of dH0 do not cancel over the atoms (naphthalene: 2e-4 per element; ~1e-6 here)
        assert np.abs(gr.reshape(-1, 3).sum(axis=0)).max() < 1e-5
    # with one centre order per pair (variant "exact") the gradient is translation invariant
    ge, _ = fmo.ct_state_gradients(gpu_ctx, mons, terms[:2], pair_states=states, variant="exact", n_streams=2)
    for gr in ge:
        assert np.abs(gr.reshape(-1, 3).sum(axis=0)).max() < 1e-8


def test_ct_state_gradients_without_lc(gpu_ctx):
    c = fmo_case(3, 1, 1, lc=False)
    rc, res = fmo.solve_batch(gpu_ctx, c["instances"], 150, 1e-8, _lib.PREC_FP64)
    assert rc == _lib.OK
    mons = c["monomers"]
    terms = _ct_terms(c, res)
    grads, states = fmo.ct_state_gradients(gpu_ctx, mons, terms, n_streams=3)
    assert not states[(0, 1)][0].lc
    for (h, l, x, e), gr in zip(terms, grads):
        want, _ = _oracle(mons, states, h, l, x, e)
        assert np.abs(gr - want).max() < 1e-9, (h, l)


def test_ct_gradient_single_orbital_pair(gpu_ctx, solved):
    """tincr's ct_gradient_new(1, 2, ct_ind_i=1, ct_ind_j=0, E, hole_i=false): HOMO of monomer 2 ->
    LUMO + 1 of monomer 1."""
    c, _ = solved
    mons = c["monomers"]
    states = fmo.pair_ground_states(gpu_ctx, mons, [(1, 2)])
    gr = fmo.ct_gradient(gpu_ctx, mons, 1, 2, 1, 0, 0.31, False, pair_states=states)
    x_ct = OCT.ct_unit_amplitudes(mons[2].system.n_occ, mons[1].system.n_virt, 0, 1)
    want, _ = _oracle(mons, states, 2, 1, x_ct, 0.31)
    assert np.abs(gr - want).max() < 1e-9
    with pytest.raises(ValueError):
        fmo.ct_gradient(gpu_ctx, mons, 2, 1, 0, 0, 0.3, True)


def test_exciton_gradient_adds_le_and_ct_terms(gpu_ctx, solved):
    c, res = solved
    mons = c["monomers"]
    setup = fmo.ExcitonSetup(mons, c["pairs"], scc="gpu", ctx=gpu_ctx)
    ex = fmo.exciton_states(gpu_ctx, setup, res, c["labels"], N_LE, N_CT, n_roots=3, tol=1e-8)
    basis, _ = fmo.exciton_basis(c["labels"], res, len(mons), N_LE, N_CT, setup.ct_pairs)
    assert len(basis) == ex["vectors"].shape[0]
    v = ex["vectors"][:, 0]
    grad, n_le_t, n_ct_t, states = fmo.exciton_gradient(gpu_ctx, setup, res, c["labels"], N_LE, N_CT, v,
                                                        threshold=0.0)
    le_part, n_le2, _ = fmo.exciton_le_gradient(mons, res, v, N_LE, threshold=0.0)
    assert n_le_t == n_le2 == len(mons) * N_LE
    assert n_ct_t == 4
    offs = np.concatenate([[0], np.cumsum([m.system.n_atoms for m in mons])])
    want = le_part.copy()
    for b, cb in enumerate(v):
        if basis[b][0] != "CT":
            continue
        _, h, l, n = basis[b]
        k = c["labels"].index(("CT", h, l))
        x = np.asarray(res[k]["coefficients"])[:, n].reshape(mons[h].system.n_occ, -1)
        og, _ = _oracle(mons, states, h, l, x, float(res[k]["energies"][n]))
        i, j = min(h, l), max(h, l)
        ni = 3 * int(offs[i + 1] - offs[i])
        want[3 * offs[i]:3 * offs[i + 1]] += cb ** 2 * og[:ni]
        want[3 * offs[j]:3 * offs[j + 1]] += cb ** 2 * og[ni:]
    assert np.abs(grad - want).max() < 1e-9
    # the default threshold keeps fewer terms; the ones it keeps are the same
    g2, n_le3, n_ct3, _ = fmo.exciton_gradient(gpu_ctx, setup, res, c["labels"], N_LE, N_CT, v, pair_states=states)
    assert n_le3 == int(np.sum(np.abs(v[:len(mons) * N_LE]) > 0.05))
    assert n_ct3 == int(np.sum(np.abs(v[len(mons) * N_LE:]) > 0.05))
    with pytest.raises(ValueError):
        fmo.exciton_gradient(gpu_ctx, setup, res, c["labels"], N_LE, N_CT, v[:-1])
