"""Batched LE / CT TDA (FMO monomers and charge-transfer pair directions).

CPU: the dimer formulation that the GPU batch uses for a CT pair (Mulliken charges of the dimer
with C = [C_H,occ | C_L,virt]) reproduces tincr's pair engine (`calculate_q_ov` + the H x L
exchange of solvers/mod.rs:166-276) to rounding.
GPU: `tincr_tda_solve_batch` against the oracle engines instance by instance: energies within
1e-10 Eh, |overlap| of the eigenvectors 1 within 1e-7, oscillator strengths within 1e-8, the same
Davidson iteration counts, with convergence masks (instances finishing at different iterations).
"""

import numpy as np
import pytest

from cases import fmo_case, fmo_oracle_engine
from oracle import tda as OT
from tincr_gb300 import _lib
from tincr_gb300 import fmo


def _dimer_engine(q):
    """TdaEngine of the dimer formulation of an instance dict."""
    ao = np.concatenate([[0], np.cumsum(q["opa"])])
    no, nv = q["n_occ"], q["n_virt"]
    qov, qoo, qvv = OT.trans_charges(ao, q["c"], q["s"], np.arange(no), np.arange(no, no + nv))
    om = OT.orbe_differences(q["orbe"][:no], q["orbe"][no:])
    return OT.TdaEngine(om, qov, q["gamma"], qoo, qvv, q["gamma_lr"], no, nv)


def test_ct_dimer_formulation_equals_pair_engine():
    case = fmo_case(2, 1, 1)
    assert case["pairs"], "the two stacked acenes must form a CT pair"
    for k, lab in enumerate(case["labels"]):
        if lab[0] != "CT":
            continue
        q = case["instances"][k]
        ref, _ = fmo_oracle_engine(case, k)
        dim = _dimer_engine(q)
        x = np.random.default_rng(k).standard_normal((q["n_occ"] * q["n_virt"], 3))
        a, b = ref.apply(x), dim.apply(x)
        assert np.abs(a - b).max() < 1e-12 * np.abs(a).max()
        assert np.abs(ref.omega - dim.omega).max() == 0.0


def test_aggregate_work_list():
    case = fmo_case(3, 1, 1)
    n_mon = len(case["monomers"])
    assert [lab[0] for lab in case["labels"]].count("LE") == n_mon
    assert len(case["instances"]) == n_mon + 2 * len(case["pairs"])
    for q in case["instances"]:
        assert q["c"].shape == (q["n_orb"], q["n_occ"] + q["n_virt"])
        assert q["orbe"].shape == (q["n_occ"] + q["n_virt"],)


def _oracle(case, k, tol, max_iter):
    eng, xyz = fmo_oracle_engine(case, k)
    q = case["instances"][k]
    return OT.run_tda_engine(eng, xyz, q["n_roots"], max_iter, tol)


@pytest.mark.gpu
@pytest.mark.parametrize("tol", [1e-4, 1e-8])
def test_batch_matches_oracle(gpu_ctx, tol):
    case = fmo_case(3, 1, 1)
    rc, res = fmo.solve_batch(gpu_ctx, case["instances"], max_iter=150, tol=tol)
    assert rc == _lib.OK
    iters = set()
    for k, r in enumerate(res):
        ref = _oracle(case, k, tol, 150)
        assert r["status"] == _lib.OK
        e_tol = 1e-10 if tol < 1e-6 else 1e-8
        assert np.abs(r["energies"] - ref["energies"]).max() < e_tol, case["labels"][k]
        if tol < 1e-6:
            ov = np.abs(np.einsum("xr,xr->r", r["coefficients"], ref["coefficients"]))
            assert np.abs(ov - 1.0).max() < 1e-7
            assert np.abs(r["osc"] - ref["f"]).max() < 1e-8
            sgn = np.sign(np.einsum("xr,xr->r", r["coefficients"], ref["coefficients"]))
            assert np.abs(r["q_trans"] * sgn - ref["q_trans"]).max() < 1e-8
        assert r["iterations"] == ref["iterations"], case["labels"][k]
        iters.add(r["iterations"])
    assert len(iters) > 1     # instances converged at different iterations: the masks were exercised


@pytest.mark.gpu
def test_batch_single_instance_equals_system_solver(gpu_ctx):
    """A one-instance batch gives the single-system solver's roots."""
    from tincr_gb300 import tda as T
    case = fmo_case(2, 1, 1)
    q = case["instances"][0]
    rc, res = fmo.solve_batch(gpu_ctx, [q], max_iter=100, tol=1e-8)
    m = case["monomers"][0]
    es = T.ExcitedStateSystem.from_ground_state(gpu_ctx, m.system, m.ground)
    ref = es.run_tda(q["n_roots"], 100, 1e-8)
    assert np.abs(res[0]["energies"] - ref["ci_eigenvalues"]).max() < 1e-10
    assert res[0]["iterations"] == ref["davidson_iterations"]


@pytest.mark.gpu
def test_batch_not_converged_and_bad_input(gpu_ctx):
    case = fmo_case(2, 1, 1)
    rc, res = fmo.solve_batch(gpu_ctx, case["instances"], max_iter=2, tol=1e-12)
    assert rc == _lib.NOT_CONVERGED
    assert all(r["status"] == _lib.NOT_CONVERGED and r["iterations"] == 2 for r in res)
    bad = dict(case["instances"][0])
    bad["n_roots"] = 7
    with pytest.raises(_lib.TincrError) as e:
        fmo.solve_batch(gpu_ctx, [bad])
    assert e.value.status == _lib.BAD_ARG
    bad = dict(case["instances"][0])
    bad["s"] = bad["s"].copy()
    bad["s"][0, 1] = np.nan
    with pytest.raises(_lib.TincrError) as e:
        fmo.solve_batch(gpu_ctx, [bad])
    assert e.value.status == _lib.NONFINITE


@pytest.mark.gpu
def test_batch_mixed_within_bar(gpu_ctx):
    """Mixed form (three-plane split-BF16 GEMMs, FP64 subspace): every root of every instance within
    1e-6 Eh of the FP64 batch (the mixed-form target)."""
    case = fmo_case(3, 1, 1)
    rc64, r64 = fmo.solve_batch(gpu_ctx, case["instances"], max_iter=150, tol=1e-6)
    rcm, rm = fmo.solve_batch(gpu_ctx, case["instances"], max_iter=150, tol=1e-6, precision=_lib.PREC_BF16X3)
    assert rc64 == _lib.OK and rcm == _lib.OK
    err = max(np.abs(a["energies"] - b["energies"]).max() for a, b in zip(r64, rm))
    print("mixed batch: max |dE| = %.2e Eh" % err)
    assert err < 1e-6
    dq, dosc = 0.0, 0.0
    for a, b in zip(r64, rm):
        ovs = np.einsum("xr,xr->r", a["coefficients"], b["coefficients"])
        assert np.abs(np.abs(ovs) - 1.0).max() < 1e-6
        # transition charges (sign of each root aligned) and oscillator strengths of the roots
        dq = max(dq, np.abs(a["q_trans"] - b["q_trans"] * np.sign(ovs)[None, :]).max())
        dosc = max(dosc, np.abs(a["osc"] - b["osc"]).max())
    print("mixed batch: max |dq_trans| = %.2e, max |d osc| = %.2e" % (dq, dosc))
    assert dq < 1e-5 and dosc < 1e-6


@pytest.mark.gpu
def test_batch_mixed_tight_tolerance(gpu_ctx):
    """Tolerance 1e-8 (below the mixed operator's 1e-6 floor): the mixed batch finishes with FP64
    iterations and matches the FP64 batch to 1e-10 Eh."""
    case = fmo_case(3, 1, 1)
    _, r64 = fmo.solve_batch(gpu_ctx, case["instances"], max_iter=150, tol=1e-8)
    rcm, rm = fmo.solve_batch(gpu_ctx, case["instances"], max_iter=150, tol=1e-8, precision=_lib.PREC_BF16X3)
    if rcm != _lib.OK:
        print("statuses", [r["status"] for r in rm], "iterations", [r["iterations"] for r in rm],
              "fp64 iterations", [r["iterations"] for r in r64])
    assert rcm == _lib.OK
    assert max(np.abs(a["energies"] - b["energies"]).max() for a, b in zip(r64, rm)) < 1e-10


@pytest.mark.gpu
def test_le_gradients_concurrent_match_single_context(gpu_ctx):
    """LE gradients on several concurrent contexts equal the single-context gradients (to 1e-12
    Eh/bohr) and, for one monomer, the oracle's tincr-formula gradient (to 1e-8 Eh/bohr)."""
    from oracle import gradients as OG
    from tincr_gb300 import gradients as GR
    from tincr_gb300 import groundstate as gs
    from tincr_gb300 import tda as T
    case = fmo_case(3, 1, 1)
    n_mon = len(case["monomers"])
    rc, res = fmo.solve_batch(gpu_ctx, case["instances"][:n_mon], max_iter=150, tol=1e-8)
    states = [0] * n_mon
    conc = fmo.le_gradients(case["monomers"], res, states, n_streams=3)
    for k, m in enumerate(case["monomers"]):
        es = T.ExcitedStateSystem.from_ground_state(gpu_ctx, m.system, m.ground)
        es.set_states(res[k]["energies"], res[k]["coefficients"])
        g1 = GR.GradientSystem(es, m.system, m.ground).tda_gradient(0)
        assert np.abs(conc[k] - g1).max() < 1e-12
    # oracle for the smallest monomer
    k = int(np.argmin([m.system.n_orbs for m in case["monomers"]]))
    m = case["monomers"][k]
    sy, g = m.system, m.ground
    from oracle import tda as OT
    qov, qoo, qvv = OT.trans_charges(sy.ao_offset, g.orbs, g.s, sy.occ_indices, sy.virt_indices)
    der = OG.derivative_tensors(sy.numbers, sy.xyz, sy.ao_offset, sy.ao_atom, sy.hubbard, sy.r_lr, sy.params)
    inp = dict(p=g.p, p0=g.p0, h_coul_x=g.h_coul_x, gamma=g.gamma, dq=g.dq, s=g.s, ao_atom=sy.ao_atom,
               numbers=sy.numbers, xyz=sy.xyz, params=sy.params, gamma_lr_ao=gs.atom_to_ao(sy, g.gamma_lr),
               orbe=g.orbe, occ=sy.occ_indices, virt=sy.virt_indices, ci_eigenvalues=res[k]["energies"],
               ci_coefficients=res[k]["coefficients"], q_ov=qov, q_oo=qoo, q_vv=qvv, gamma_lr=g.gamma_lr,
               orbs=g.orbs, gamma_ao=gs.atom_to_ao(sy, g.gamma))
    _, flr = OG.ground_state_gradient(inp, der, True)
    ref = OG.tda_gradient(inp, der, 0, True, flr_dmd0=flr)
    assert np.abs(conc[k] - ref).max() < 1e-8


@pytest.mark.gpu
def test_batch_tile_autotuner(gpu_ctx, monkeypatch):
    """The mixed batch's plane GEMM tile shapes: the autotuner records a choice for every instance
    shape of the batch, and every forced tile shape gives the same energies, vectors and iteration
    counts (each output element sees the same K order whatever the shape)."""
    case = fmo_case(3, 1, 1)
    monkeypatch.delenv("TINCR_GB300_BATCH_TILES", raising=False)
    rc, ra = fmo.solve_batch(gpu_ctx, case["instances"], max_iter=150, tol=1e-6, precision=_lib.PREC_BF16X3)
    assert rc == _lib.OK
    table = gpu_ctx.batch_tile_table()
    keys = {(t["n_atoms"], t["n_orb"], t["n_occ"], t["n_virt"]) for t in table}
    for q in case["instances"]:
        assert (q["n_atoms"], q["n_orb"], q["n_occ"], q["n_virt"]) in keys
    for t in table:
        assert t["shapes"]["H"] in gpu_ctx.TILE_SHAPES and t["shapes"]["AX"] in gpu_ctx.TILE_SHAPES
        assert (t["shapes"]["F"] is None) == (not t["lc"])
        for st, times in t["us"].items():
            assert all(v > 0 for v in times.values())
        print("tiles", t["n_atoms"], t["n_orb"], t["n_occ"], t["n_virt"], t["shapes"])
    for shape in gpu_ctx.TILE_SHAPES:
        monkeypatch.setenv("TINCR_GB300_BATCH_TILES", shape)
        rc, rb = fmo.solve_batch(gpu_ctx, case["instances"], max_iter=150, tol=1e-6, precision=_lib.PREC_BF16X3)
        assert rc == _lib.OK
        for a, b in zip(ra, rb):
            assert a["iterations"] == b["iterations"]
            assert np.array_equal(a["energies"], b["energies"])
            assert np.array_equal(np.abs(a["coefficients"]), np.abs(b["coefficients"]))
    monkeypatch.setenv("TINCR_GB300_BATCH_TILES", "48x48")
    with pytest.raises(_lib.TincrError) as e:
        fmo.solve_batch(gpu_ctx, case["instances"], precision=_lib.PREC_BF16X3)
    assert e.value.status == _lib.BAD_ARG
