"""GPU parity tests of the analytic gradients through the C ABI.

* variant "reference" against the oracle's dense restatement of tincr's gradient code
  (ground_state.rs / excited_state.rs) on the same roots (installed with tincr_tda_set_states):
  1e-9 Eh/bohr; and the full chain GPU Davidson -> gradient at 1e-6 Eh/bohr.
* variant "exact" against the oracle's exact variant, and against central finite differences of
  the excitation energy (+-1e-4 bohr): 1e-5 Eh/bohr, the gradient accuracy target.
"""

import numpy as np
import pytest

from oracle import gradients as OG
from oracle import tda as OT
from tincr_gb300 import geometry as G
from tincr_gb300 import gradients as GR
from tincr_gb300 import groundstate as gs
from tincr_gb300 import tda as T
from tincr_gb300.params import NUMBERS

from cases import golden

pytestmark = pytest.mark.gpu


def _molecule(name):
    if name in ("h2o", "ammonia", "benzene", "uracil"):
        d = golden(name)
        return np.array([NUMBERS[s] for s in d["symbols"]]), d["xyz_angstrom"] / 0.529177210903
    if name == "naphthalene":
        z, x = G.acene(2)
        return z, G.to_bohr(x)
    if name == "polyene8":
        z, x = G.polyene(8)
        return z, G.to_bohr(x)
    if name == "water8":
        z, x = G.water_cluster(2, 2, 2)
        return z, G.to_bohr(x)
    raise KeyError(name)


def _oracle(sy, g, lc, state, variant, n_roots):
    occ, virt = sy.occ_indices, sy.virt_indices
    qov, qoo, qvv = OT.trans_charges(sy.ao_offset, g.orbs, g.s, occ, virt)
    om = OT.orbe_differences(g.orbe[occ], g.orbe[virt])
    a = OT.tda_full_matrix(om, qov, g.gamma, qoo, qvv, g.gamma_lr if lc else None, sy.n_occ, sy.n_virt)
    e, x = np.linalg.eigh(a)
    orient = "reference" if variant == "reference" else "index"
    der = OG.derivative_tensors(sy.numbers, sy.xyz, sy.ao_offset, sy.ao_atom, sy.hubbard, sy.r_lr, sy.params,
                                orientation=orient)
    inp = dict(p=g.p, p0=g.p0, h_coul_x=g.h_coul_x, gamma=g.gamma, dq=g.dq, s=g.s, ao_atom=sy.ao_atom,
               numbers=sy.numbers, xyz=sy.xyz, params=sy.params, gamma_lr_ao=gs.atom_to_ao(sy, g.gamma_lr),
               orbe=g.orbe, occ=occ, virt=virt, ci_eigenvalues=e[:n_roots], ci_coefficients=x[:, :n_roots],
               q_ov=qov, q_oo=qoo, q_vv=qvv, gamma_lr=g.gamma_lr, orbs=g.orbs, gamma_ao=gs.atom_to_ao(sy, g.gamma))
    ggs, flr = OG.ground_state_gradient(inp, der, lc)
    gex = OG.tda_gradient(inp, der, state, lc, flr_dmd0=flr, variant=variant)
    return ggs, gex, e, x


def _gpu(ctx, sy, g, lc, state, variant, n_roots, states=None):
    """GPU gradient; `states` = (energies, vectors) installs given roots, else the GPU Davidson solves."""
    es = T.ExcitedStateSystem.from_ground_state(ctx, sy, g, lc=lc)
    if states is None:
        es.run_tda(n_roots, 300, 1e-8)
    else:
        es.set_states(*states)
    gr = GR.GradientSystem(es, sy, g)
    ggs, gex = gr.both(state, variant)
    return ggs, gex, es.properties["ci_eigenvalues"], gr.last_cg_iterations


@pytest.mark.parametrize("name", ["h2o", "uracil", "naphthalene", "water8"])
@pytest.mark.parametrize("lc", [True, False])
@pytest.mark.parametrize("variant", ["reference", "exact"])
def test_gradients_match_oracle(gpu_ctx, name, lc, variant):
    z, x = _molecule(name)
    sy = gs.build_system(z, x, lc=lc)
    g = gs.run_scc(sy, tol=1e-11)
    n_roots = min(3, sy.n_occ * sy.n_virt)
    ogs, oex, oe, ox = _oracle(sy, g, lc, 0, variant, n_roots)
    ggs, gex, ge, cg = _gpu(gpu_ctx, sy, g, lc, 0, variant, n_roots, states=(oe[:n_roots], ox[:, :n_roots]))
    assert np.abs(ggs - ogs).max() < 1e-9
    assert np.abs(gex - oex).max() < 1e-9
    assert cg > 0


@pytest.mark.parametrize("lc", [True, False])
def test_gradient_after_gpu_davidson(gpu_ctx, lc):
    """Full GPU chain: Davidson roots (residual 1e-8) -> gradient, against the dense oracle."""
    z, x = _molecule("naphthalene")
    sy = gs.build_system(z, x, lc=lc)
    g = gs.run_scc(sy, tol=1e-11)
    ogs, oex, oe, _ = _oracle(sy, g, lc, 0, "reference", 3)
    ggs, gex, ge, _ = _gpu(gpu_ctx, sy, g, lc, 0, "reference", 3)
    assert abs(ge[0] - oe[0]) < 1e-10
    assert np.abs(gex - oex).max() < 1e-6


@pytest.mark.parametrize("lc", [True, False])
def test_exact_gradient_matches_finite_differences(gpu_ctx, lc):
    """Central differences (+-1e-4 bohr) of the lowest excitation energy on water, all coordinates."""
    z, x = _molecule("h2o")
    sy = gs.build_system(z, x, lc=lc)
    g = gs.run_scc(sy, tol=1e-11)
    _, _, oe, ox = _oracle(sy, g, lc, 0, "exact", 3)
    _, gex, _, _ = _gpu(gpu_ctx, sy, g, lc, 0, "exact", 3, states=(oe[:3], ox[:, :3]))

    def e0(xyz):
        s2 = gs.build_system(z, xyz, lc=lc)
        g2 = gs.run_scc(s2, tol=1e-11)
        occ, virt = s2.occ_indices, s2.virt_indices
        qov, qoo, qvv = OT.trans_charges(s2.ao_offset, g2.orbs, g2.s, occ, virt)
        om = OT.orbe_differences(g2.orbe[occ], g2.orbe[virt])
        a = OT.tda_full_matrix(om, qov, g2.gamma, qoo, qvv, g2.gamma_lr if lc else None, s2.n_occ, s2.n_virt)
        return np.linalg.eigvalsh(a)[0]

    h = 1e-4
    fd = np.zeros_like(gex)
    for c in range(len(fd)):
        xp, xm = x.copy(), x.copy()
        xp[c // 3, c % 3] += h
        xm[c // 3, c % 3] -= h
        fd[c] = (e0(xp) - e0(xm)) / (2 * h)
    assert np.abs(gex - fd).max() < 1e-5


def test_gradient_call_order_and_arguments(gpu_ctx):
    from tincr_gb300 import _lib
    z, x = _molecule("h2o")
    sy = gs.build_system(z, x, lc=True)
    g = gs.run_scc(sy)
    es = T.ExcitedStateSystem.from_ground_state(gpu_ctx, sy, g)
    es.run_tda(2, 100, 1e-8)
    gr = GR.GradientSystem(es, sy, g)
    with pytest.raises(_lib.TincrError) as e:
        gr.tda_gradient(5)                 # only 2 roots solved
    assert e.value.status == _lib.BAD_ARG
    bad = gr.atom_kind.copy()
    bad[0] = 7
    gr.atom_kind = bad
    with pytest.raises(_lib.TincrError) as e:
        gr.tda_gradient(0)
    assert e.value.status == _lib.BAD_ARG


@pytest.mark.parametrize("name,lc,variant", [("water8", True, "reference"), ("naphthalene", True, "exact"),
                                             ("polyene8", False, "reference")])
def test_mixed_gradient_within_bar(gpu_ctx, name, lc, variant):
    """After a mixed solve the gradient's contractions and Z-vector run mixed: S1 gradient within
    1e-5 Eh/bohr (the gradient accuracy target) of the gradient after an FP64 solve of the same roots."""
    z, x = _molecule(name)
    sy = gs.build_system(z, x, lc=lc)
    g = gs.run_scc(sy, tol=1e-11)
    out = {}
    for prec in (T._lib.PREC_FP64, T._lib.PREC_BF16X3):
        es = T.ExcitedStateSystem.from_ground_state(gpu_ctx, sy, g)
        es.run_tda(3, 300, 1e-6, precision=prec)
        gr = GR.GradientSystem(es, sy, g)
        out[prec] = gr.both(0, variant)
    d_gs = np.abs(out[T._lib.PREC_FP64][0] - out[T._lib.PREC_BF16X3][0]).max()
    d_ex = np.abs(out[T._lib.PREC_FP64][1] - out[T._lib.PREC_BF16X3][1]).max()
    print("%s mixed gradient: |d grad_gs| %.2e |d grad_exc| %.2e Eh/bohr" % (name, d_gs, d_ex))
    assert d_gs < 1e-5 and d_ex < 1e-5
