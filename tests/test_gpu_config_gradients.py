"""Excited-state gradients on the two single-molecule benchmark geometries, through the adjoint /
Z-vector path.

* C20H22 all-trans polyene (planar, C=C 1.34 A, C-C 1.46 A, C-H 1.09 A; 102 orbitals, 51 x 51
  singles), plain DFTB: the lowest 10 roots (residual < 1e-6) plus the analytic S1 gradient.
* Decacene C42H24 (ideal hexagons, C-C 1.40 A, C-H 1.08 A; 192 orbitals, 96 x 96 singles): the
  lowest 3 TDA states, DFTB and LC-DFTB (omega = 0.3 bohr^-1), FP64 and mixed.

Checks:
* "reference" variant (tincr's formulas) against the oracle's analytic gradient of the same roots
  (`gradients/excited_state.rs`, `gradients/ground_state.rs`): 1e-9 Eh/bohr.
* "exact" variant against central finite differences (+-1e-4 bohr, every coordinate) of the
  excitation energies, each displaced geometry solved by an SCC and the GPU FP64 Davidson (residual
  1e-8; tincr's Davidson stalls near 4e-9 on decacene, where the 1e-8 drop rule of its Gram-Schmidt
  rejects every correction): 1e-5 Eh/bohr.  The polyene's displaced SCCs run on the host, the
  decacene's as one batched GPU SCC.
* mixed form: energies within 1e-6 Eh and gradients within 1e-5 Eh/bohr of the FP64 form.
"""

import numpy as np
import pytest

from oracle import gradients as OG
from oracle import tda as OT
from tincr_gb300 import geometry as G
from tincr_gb300 import gradients as GR
from tincr_gb300 import groundstate as gs
from tincr_gb300 import tda as T

from cases import displaced_scc

pytestmark = pytest.mark.gpu

FD_STEP = 1e-4


def _molecule(name, lc):
    z, x = G.polyene(20) if name == "polyene" else G.acene(10)
    sy = gs.build_system(z, G.to_bohr(x), lc=lc)
    return sy, gs.run_scc(sy, tol=1e-11)


def _solve(ctx, sy, g, lc, n_roots, precision=T._lib.PREC_FP64, tol=1e-8):
    es = T.ExcitedStateSystem.from_ground_state(ctx, sy, g, lc=lc)
    es.run_tda(n_roots, 450, tol, precision=precision)
    return es


def _oracle_inputs(sy, g, e, x):
    occ, virt = sy.occ_indices, sy.virt_indices
    qov, qoo, qvv = OT.trans_charges(sy.ao_offset, g.orbs, g.s, occ, virt)
    der = OG.derivative_tensors(sy.numbers, sy.xyz, sy.ao_offset, sy.ao_atom, sy.hubbard, sy.r_lr, sy.params,
                                orientation="reference")
    inp = dict(p=g.p, p0=g.p0, h_coul_x=g.h_coul_x, gamma=g.gamma, dq=g.dq, s=g.s, ao_atom=sy.ao_atom,
               numbers=sy.numbers, xyz=sy.xyz, params=sy.params, gamma_lr_ao=gs.atom_to_ao(sy, g.gamma_lr),
               orbe=g.orbe, occ=occ, virt=virt, ci_eigenvalues=e, ci_coefficients=x, q_ov=qov, q_oo=qoo,
               q_vv=qvv, gamma_lr=g.gamma_lr, orbs=g.orbs, gamma_ao=gs.atom_to_ao(sy, g.gamma))
    return inp, der


def _finite_differences(ctx, sy, lc, n_roots):
    """Central differences of the n_roots lowest excitation energies, [n_roots, 3N]."""
    disp = displaced_scc(sy.numbers, sy.xyz, lc, FD_STEP)
    fd = np.zeros((n_roots, sy.xyz.size))
    for c, pair in enumerate(disp):
        e = []
        for sgn, a in zip((1.0, -1.0), pair):
            xyz = sy.xyz.copy()
            xyz[c // 3, c % 3] += sgn * FD_STEP
            d = T.ExcitedStateSystem(ctx, sy.orbs_per_atom, a["orbs"], a["s"], a["orbe"], sy.n_occ, sy.n_virt,
                                     a["gamma"], a["gamma_lr"], xyz)
            e.append(d.run_tda(n_roots, 450, 1e-8)["ci_eigenvalues"].copy())
        fd[:, c] = (e[0] - e[1]) / (2 * FD_STEP)
    return fd


def test_polyene_ten_roots_and_s1_gradient(gpu_ctx):
    sy, g = _molecule("polyene", lc=False)
    es = _solve(gpu_ctx, sy, g, False, 10, tol=1e-6)
    e, x = es.properties["ci_eigenvalues"].copy(), es.properties["ci_coefficients"].copy()
    occ, virt = sy.occ_indices, sy.virt_indices
    qov, _, _ = OT.trans_charges(sy.ao_offset, g.orbs, g.s, occ, virt)
    om = OT.orbe_differences(g.orbe[occ], g.orbe[virt])
    ref = OT.run_tda(om, qov, g.gamma, sy.xyz, 10, 450, 1e-6)
    assert np.abs(e - ref["energies"]).max() < 1e-8
    gr = GR.GradientSystem(es, sy, g)
    inp, der = _oracle_inputs(sy, g, e, x)
    ogs, flr = OG.ground_state_gradient(inp, der, False)
    oex = OG.tda_gradient(inp, der, 0, False, flr_dmd0=flr, variant="reference")
    ggs, gex = gr.both(0, "reference")
    print("polyene S1: |d grad_gs| %.1e |d grad_exc| %.1e" % (np.abs(ggs - ogs).max(), np.abs(gex - oex).max()))
    assert np.abs(ggs - ogs).max() < 1e-9 and np.abs(gex - oex).max() < 1e-9
    # the exact variant against finite differences of the S1 excitation energy (roots to 1e-8)
    es8 = _solve(gpu_ctx, sy, g, False, 1)
    ana = GR.GradientSystem(es8, sy, g).tda_gradient(0, "exact")
    fd = _finite_differences(gpu_ctx, sy, False, 1)[0]
    print("polyene S1 exact gradient vs FD: %.1e" % np.abs(ana - fd).max())
    assert np.abs(ana - fd).max() < 1e-5


@pytest.mark.parametrize("lc", [True, False])
def test_decacene_reference_gradients_match_oracle(gpu_ctx, lc):
    sy, g = _molecule("decacene", lc)
    es = _solve(gpu_ctx, sy, g, lc, 3)
    e, x = es.properties["ci_eigenvalues"].copy(), es.properties["ci_coefficients"].copy()
    gr = GR.GradientSystem(es, sy, g)
    inp, der = _oracle_inputs(sy, g, e, x)
    ogs, flr = OG.ground_state_gradient(inp, der, lc)
    for state in range(3):
        ggs, gex = gr.both(state, "reference")
        oex = OG.tda_gradient(inp, der, state, lc, flr_dmd0=flr, variant="reference")
        print("decacene lc=%s state %d: |d grad_gs| %.1e |d grad_exc| %.1e" %
              (lc, state, np.abs(ggs - ogs).max(), np.abs(gex - oex).max()))
        assert np.abs(ggs - ogs).max() < 1e-9
        assert np.abs(gex - oex).max() < 1e-9


@pytest.mark.parametrize("lc", [True, False])
def test_decacene_exact_gradients_match_finite_differences(gpu_ctx, lc):
    """All 198 coordinates: the 396 displaced SCCs as one batched GPU SCC (tincr_gb300.numerical)."""
    from tincr_gb300 import numerical as NUM
    sy, g = _molecule("decacene", lc)
    es = _solve(gpu_ctx, sy, g, lc, 3)
    gr = GR.GradientSystem(es, sy, g)
    ana = np.array([gr.tda_gradient(s, "exact") for s in range(3)])
    _, fd = NUM.fd_gradient(gpu_ctx, sy, n_roots=3, h=FD_STEP)
    err = np.abs(ana - fd).max(axis=1)
    print("decacene lc=%s exact gradient vs FD, per state:" % lc, " ".join("%.1e" % v for v in err))
    assert err.max() < 1e-5


@pytest.mark.parametrize("lc", [True, False])
def test_decacene_mixed_within_bar(gpu_ctx, lc):
    sy, g = _molecule("decacene", lc)
    out = {}
    for prec in (T._lib.PREC_FP64, T._lib.PREC_BF16X3):
        es = _solve(gpu_ctx, sy, g, lc, 3, precision=prec, tol=1e-6)
        gr = GR.GradientSystem(es, sy, g)
        out[prec] = (es.properties["ci_eigenvalues"].copy(),
                     np.array([gr.tda_gradient(s, "exact") for s in range(3)]))
    de = np.abs(out[T._lib.PREC_FP64][0] - out[T._lib.PREC_BF16X3][0]).max()
    dg = np.abs(out[T._lib.PREC_FP64][1] - out[T._lib.PREC_BF16X3][1]).max(axis=1)
    print("decacene lc=%s mixed: |dE| %.1e Eh, |d grad| per state %s Eh/bohr" %
          (lc, de, " ".join("%.1e" % v for v in dg)))
    assert de < 1e-6
    assert dg.max() < 1e-5
