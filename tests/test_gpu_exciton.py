"""GPU exciton Hamiltonian (tincr_exciton_states) against the oracle restatement of tincr's
create_exciton_hamiltonian_new (oracle/exciton.py) on small seeded acene aggregates.

Both sides read the same LE / CT roots (the GPU batch TDA, FP64, converged to 1e-8), the same
monomer and dimer ground states and the same gamma matrices:
* FP64: every matrix element within 1e-10 Eh, the lowest roots within 1e-8 Eh of the oracle
  matrix's eigenvalues;
* mixed form (exchange integrals and LCMO Fock products in FP32): elements within 1e-6 Eh, roots
  within 1e-6 Eh."""

import numpy as np
import pytest

from cases import fmo_case
from oracle import exciton as OX
from tincr_gb300 import _lib
from tincr_gb300 import fmo

pytestmark = pytest.mark.gpu

N_LE, N_CT, N_ROOTS = 4, 1, 5


def _oracle_matrix(c, setup, labels, res):
    frags = []
    off = 0
    for m in c["monomers"]:
        sy, g = m.system, m.ground
        frags.append(OX.Frag(m.index, np.arange(off, off + sy.n_atoms), sy.ao_offset, g.orbs, g.orbe, g.s, sy.n_occ,
                             sy.xyz, sy.numbers))
        off += sy.n_atoms
    types = {k: ("pair" if v else "esd") for k, v in setup.real.items()}
    agg = OX.Aggregate(frags, setup.s_block, setup.gamma, setup.gamma_lr, types, setup.pair_scc)
    le, ct = {}, {}
    for k, lab in enumerate(labels):
        r = res[k]
        if lab[0] == "LE":
            le[lab[1]] = (r["energies"], r["coefficients"])
        else:
            ct[(lab[1], lab[2])] = (r["energies"], r["coefficients"], r["q_trans"])
    states = OX.diabatic_basis(agg, le, ct, setup.ct_pairs, N_LE, N_CT)
    return OX.exciton_hamiltonian(agg, states)


@pytest.fixture(scope="module", params=[(3, 1, 1), (2, 2, 1)])
def aggregate(request, gpu_ctx):
    c = fmo_case(*request.param)
    setup = fmo.ExcitonSetup(c["monomers"], c["pairs"])
    rc, res = fmo.solve_batch(gpu_ctx, c["instances"], 150, 1e-8, _lib.PREC_FP64)
    assert rc == _lib.OK
    h_ref = _oracle_matrix(c, setup, c["labels"], res)
    return c, setup, res, h_ref


@pytest.mark.parametrize("prec,bar_h,bar_e", [(_lib.PREC_FP64, 1e-10, 1e-8), (_lib.PREC_BF16X3, 1e-6, 1e-6)])
def test_exciton_matrix_and_roots_match_oracle(gpu_ctx, aggregate, prec, bar_h, bar_e):
    c, setup, res, h_ref = aggregate
    out = fmo.exciton_states(gpu_ctx, setup, res, c["labels"], N_LE, N_CT, n_roots=N_ROOTS, tol=1e-8,
                             max_iter=200, precision=prec, want_matrix=True)
    assert out["status"] == _lib.OK
    assert out["matrix"].shape == h_ref.shape
    assert np.abs(out["matrix"] - h_ref).max() < bar_h
    e_ref = np.linalg.eigvalsh(h_ref)[:N_ROOTS]
    assert np.abs(out["energies"] - e_ref).max() < bar_e
    # the returned vectors are eigenvectors of the oracle matrix to the same accuracy
    v = out["vectors"]
    assert np.abs(h_ref @ v - v * out["energies"]).max() < 1e-6


def test_exciton_rejects_bad_input(gpu_ctx, aggregate):
    c, setup, res, h_ref = aggregate
    with pytest.raises(_lib.TincrError) as e:
        fmo.exciton_states(gpu_ctx, setup, res, c["labels"], N_LE, N_CT, n_roots=10 ** 6)
    assert e.value.status == _lib.BAD_ARG
