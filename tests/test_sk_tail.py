"""Slater-Koster splines beyond their grid (10 bohr).  tincr evaluates them up to 30 bohr
(src/scc/h0_and_s.rs:110, :215) with Rusty-FITPACK's splev_uniform, i.e. the boundary polynomial
piece past the last knot (FITPACK splev, ext = 0).  The default here takes them as zero; the
`sk_tail="extrapolate"` mode evaluates the boundary piece in the host S / H0 (and so the SCC), the
oracle's dense derivatives and the GPU gradient kernel (flag TINCR_GRAD_SK_EXTRAPOLATE).

On water and ammonia 12 bohr apart (pairs at 9.5-14 bohr, S stays positive definite):
* CPU: the host S / H0 equal the oracle's; the oracle's dS/dR and dH0/dR are the central
  differences of its S and H0; the two tail rules differ.
* GPU: the gradient with the flag equals the oracle's with extrapolated derivative tensors
  (REFERENCE variant, 1e-9 Eh/bohr) and central differences of the excitation energy computed with
  extrapolated S / H0 throughout (EXACT variant, 1e-5 Eh/bohr).
On this pair the extrapolated tails move S1 by 3.1e-5 Eh and its excitation gradient by up to
3.7e-3 Eh/bohr."""

import numpy as np
import pytest

from cases import fixture_case
from oracle import gradients as OG
from oracle import slako as OS
from oracle import tda as OT
from tincr_gb300 import groundstate as gs

D = 12.0   # bohr between the two water molecules


def _dimer():
    """Water and ammonia 12 bohr apart (two different molecules: no degenerate pair of local
    excitations, so the lowest root is a smooth function of the geometry)."""
    a, b = fixture_case("h2o", True), fixture_case("ammonia", True)
    za, xa = np.asarray(a["numbers"]), np.asarray(a["xyz"])
    zb, xb = np.asarray(b["numbers"]), np.asarray(b["xyz"])
    xb = xb - xb.mean(axis=0) + xa.mean(axis=0) + np.array([D, 0.3, -0.2])
    return np.concatenate([za, zb]), np.concatenate([xa, xb])


def test_extrapolated_tables_consistent():
    z, x = _dimer()
    sy0 = gs.build_system(z, x, lc=True)
    sy = gs.build_system(z, x, lc=True, sk_tail="extrapolate")
    s0, h0 = gs.h0_and_s(sy0)
    s, h = gs.h0_and_s(sy)
    assert np.abs(s - s0).max() > 1e-4 and np.abs(h - h0).max() > 1e-4   # the rule matters here
    assert np.linalg.eigvalsh(s).min() > 0.3
    so, ho = OS.h0_and_s(sy.numbers, sy.xyz, sy.ao_offset, sy.ao_energy, sy.params, sk_tail="extrapolate")
    assert np.abs(so - s).max() < 1e-14 and np.abs(ho - h).max() < 1e-14
    gS, gH = OS.h0_and_s_gradients(sy.numbers, sy.xyz, sy.ao_offset, sy.params, orientation="index",
                                   sk_tail="extrapolate")
    step = 1e-5
    for a, c in ((0, 0), (3, 0), (4, 1), (5, 2)):   # atoms on both molecules
        xp, xm = sy.xyz.copy(), sy.xyz.copy()
        xp[a, c] += step
        xm[a, c] -= step
        sp, hp = OS.h0_and_s(sy.numbers, xp, sy.ao_offset, sy.ao_energy, sy.params, sk_tail="extrapolate")
        sm, hm = OS.h0_and_s(sy.numbers, xm, sy.ao_offset, sy.ao_energy, sy.params, sk_tail="extrapolate")
        assert np.abs((sp - sm) / (2 * step) - gS[3 * a + c]).max() < 1e-7
        assert np.abs((hp - hm) / (2 * step) - gH[3 * a + c]).max() < 1e-7


def _ground(z, x, tail):
    sy = gs.build_system(z, x, lc=True, sk_tail=tail)
    return sy, gs.run_scc(sy, tol=1e-11, require_convergence=True)


def _oracle_gradient(sy, g, state, variant, n_roots=3):
    occ, virt = sy.occ_indices, sy.virt_indices
    qov, qoo, qvv = OT.trans_charges(sy.ao_offset, g.orbs, g.s, occ, virt)
    om = OT.orbe_differences(g.orbe[occ], g.orbe[virt])
    e, xv = np.linalg.eigh(OT.tda_full_matrix(om, qov, g.gamma, qoo, qvv, g.gamma_lr, sy.n_occ, sy.n_virt))
    der = OG.derivative_tensors(sy.numbers, sy.xyz, sy.ao_offset, sy.ao_atom, sy.hubbard, sy.r_lr, sy.params,
                                orientation="reference" if variant == "reference" else "index", sk_tail=sy.sk_tail)
    import cases
    inp = cases.oracle_gradient_inputs(sy, g, True, e[:n_roots], xv[:, :n_roots], (qov, qoo, qvv))
    ggs, flr = OG.ground_state_gradient(inp, der, True)
    gex = OG.tda_gradient(inp, der, state, True, flr_dmd0=flr, variant=variant)
    return ggs, gex, e[:n_roots], xv[:, :n_roots]


def _excitation(z, x, state):
    sy, g = _ground(z, x, "extrapolate")
    occ, virt = sy.occ_indices, sy.virt_indices
    qov, qoo, qvv = OT.trans_charges(sy.ao_offset, g.orbs, g.s, occ, virt)
    om = OT.orbe_differences(g.orbe[occ], g.orbe[virt])
    return np.linalg.eigvalsh(OT.tda_full_matrix(om, qov, g.gamma, qoo, qvv, g.gamma_lr, sy.n_occ, sy.n_virt))[state]


@pytest.mark.gpu
def test_gpu_gradient_with_extrapolated_tails(gpu_ctx):
    from tincr_gb300 import gradients as GR
    from tincr_gb300 import tda as T
    z, x = _dimer()
    sy, g = _ground(z, x, "extrapolate")
    ggs_o, gex_o, e, xv = _oracle_gradient(sy, g, 0, "reference")
    es = T.ExcitedStateSystem.from_ground_state(gpu_ctx, sy, g)
    es.set_states(e, xv)
    ggs, gex = GR.GradientSystem(es, sy, g).both(0, "reference")
    assert np.abs(ggs - ggs_o).max() < 1e-9
    assert np.abs(gex - gex_o).max() < 1e-9
    # the derivative of the excitation energy (exact variant) against central differences
    _, gex_x = GR.GradientSystem(es, sy, g).both(0, "exact")
    step = 2e-5   # (1e-4 leaves a truncation error of 1.3e-5 on this pair, with either tail rule)
    for a, c in ((0, 0), (3, 0), (4, 1), (5, 2)):
        xp, xm = sy.xyz.copy(), sy.xyz.copy()
        xp[a, c] += step
        xm[a, c] -= step
        fd = (_excitation(z, xp, 0) - _excitation(z, xm, 0)) / (2 * step)
        assert abs(fd - gex_x[3 * a + c]) < 1e-5
    # without the flag (zero tails) the same roots give another gradient: the rule is in effect
    sy0 = gs.build_system(z, x, lc=True)
    _, gex0 = GR.GradientSystem(es, sy0, g).both(0, "reference")
    assert np.abs(gex0 - gex).max() > 1e-6
