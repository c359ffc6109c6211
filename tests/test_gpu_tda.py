"""GPU parity tests: transition charges, A.X products and the Davidson solver through the C ABI,
against the oracle on the same inputs.

Tolerances: FP64 path, so transition charges and products agree to a few ulp-scale relative
errors (1e-12 relative); Davidson energies to 1e-10 Eh (the FP64 target is 1e-8) and
eigenvectors up to sign (|overlap| = 1 within 1e-7)."""

import numpy as np
import pytest

from cases import fixture_case, golden, oracle_inputs, synthetic_case
from oracle import tda as OT
from tincr_gb300 import _lib
from tincr_gb300 import tda as T

pytestmark = pytest.mark.gpu

FIXTURES = ["h2o", "ammonia", "benzene", "uracil", "h2"]


def _case(name, lc):
    if name in FIXTURES:
        return fixture_case(name, lc)
    return synthetic_case(name, lc)


def _solver(ctx, c):
    return T.ExcitedStateSystem(ctx, c["opa"], c["orbs"], c["s"], c["orbe"], c["n_occ"], c["n_virt"], c["gamma"],
                                c["gamma_lr"], c["xyz"])


@pytest.mark.parametrize("name", ["h2o", "benzene", "uracil", "polyene8", "water8"])
def test_trans_charges_match_oracle(gpu_ctx, name):
    c = _case(name, True)
    no, nv = c["n_occ"], c["n_virt"]
    q = T.trans_charges(gpu_ctx, c["opa"], c["orbs"], c["s"], np.arange(no), np.arange(no, no + nv))
    ref = OT.trans_charges(c["ao_offset"], c["orbs"], c["s"], np.arange(no), np.arange(no, no + nv))
    for a, b in zip(q, ref):
        assert a.shape == b.shape
        assert np.abs(a - b).max() < 1e-13


def test_trans_charges_partial_ranges(gpu_ctx):
    """Non-default orbital ranges (an active space) and one NULL output."""
    c = _case("uracil", True)
    occ, virt = np.arange(10, 18), np.arange(21, 27)
    q_ov, q_oo, q_vv = T.trans_charges(gpu_ctx, c["opa"], c["orbs"], c["s"], occ, virt)
    ref = OT.trans_charges(c["ao_offset"], c["orbs"], c["s"], occ, virt)
    assert np.abs(q_ov - ref[0]).max() < 1e-13
    assert np.abs(q_oo - ref[1]).max() < 1e-13
    assert np.abs(q_vv - ref[2]).max() < 1e-13


@pytest.mark.parametrize("name", ["h2o", "benzene", "uracil", "polyene8", "water8", "h2"])
@pytest.mark.parametrize("lc", [True, False])
def test_products_match_oracle(gpu_ctx, name, lc):
    c = _case(name, lc)
    o = oracle_inputs(c)
    eng = OT.TdaEngine(o["omega"], o["q_ov"], o["gamma"], o["q_oo"], o["q_vv"], o["gamma_lr"], o["n_occ"],
                       o["n_virt"])
    rng = np.random.default_rng(11)
    x = rng.standard_normal((c["n_occ"] * c["n_virt"], 5))
    ref = eng.apply(x)
    s = _solver(gpu_ctx, c)
    out = s.compute_products(x)
    assert np.abs(out - ref).max() < 1e-12 * max(1.0, np.abs(ref).max())


def _oracle_tda(c, n_roots, tol, max_iter=200):
    o = oracle_inputs(c)
    return OT.run_tda(o["omega"], o["q_ov"], o["gamma"], c["xyz"], n_roots, max_iter, tol, o["q_oo"], o["q_vv"],
                      o["gamma_lr"], o["n_occ"], o["n_virt"])


def _check_solution(gpu, ref, e_tol=1e-10):
    assert np.abs(gpu["ci_eigenvalues"] - ref["energies"]).max() < e_tol
    ov = np.abs(np.einsum("xr,xr->r", gpu["ci_coefficients"], ref["coefficients"]))
    assert np.abs(ov - 1.0).max() < 1e-7
    assert np.abs(gpu["oscillator_strengths"] - ref["f"]).max() < 1e-8
    # q_trans and dipoles change sign with the eigenvector: compare with the sign of the overlap
    sgn = np.sign(np.einsum("xr,xr->r", gpu["ci_coefficients"], ref["coefficients"]))
    assert np.abs(gpu["q_trans"] * sgn - ref["q_trans"]).max() < 1e-8
    assert np.abs(gpu["tr_dipoles"] * sgn - ref["tr_dipoles"]).max() < 1e-7


@pytest.mark.parametrize("name", ["h2o", "benzene", "uracil", "water8"])
@pytest.mark.parametrize("lc", [True, False])
def test_davidson_matches_oracle(gpu_ctx, name, lc):
    c = _case(name, lc)
    nr = min(4, c["n_occ"] * c["n_virt"])
    ref = _oracle_tda(c, nr, 1e-7)
    gpu = _solver(gpu_ctx, c).run_tda(nr, 200, 1e-7)
    _check_solution(gpu, ref)
    assert gpu["davidson_iterations"] == ref["iterations"]


@pytest.mark.parametrize("name,lc", [("uracil", True), ("water8", True), ("polyene8", False)])
def test_davidson_history_matches_oracle(gpu_ctx, name, lc):
    """Iteration by iteration, the FP64 solve has the oracle's subspace size and number of
    unconverged roots, and its largest residual agrees to 1e-8."""
    c = _case(name, lc)
    o = oracle_inputs(c)
    hist = []
    OT.run_tda(o["omega"], o["q_ov"], o["gamma"], c["xyz"], 4, 200, 1e-7, o["q_oo"], o["q_vv"], o["gamma_lr"],
               o["n_occ"], o["n_virt"], history=hist)
    _solver(gpu_ctx, c).run_tda(4, 200, 1e-7)
    gh = gpu_ctx.davidson_history()
    assert [h["n_sub"] for h in gh] == [h["n_sub"] for h in hist]
    assert [h["roots_left"] for h in gh] == [h["roots_left"] for h in hist]
    assert all(h["precision"] == _lib.PREC_FP64 for h in gh)
    assert max(abs(a["max_residual"] - b["max_res"]) for a, b in zip(gh, hist)) < 1e-8


def test_polyene_ten_roots_plain_fp64(gpu_ctx):
    """C20H22 all-trans polyene, non-LC DFTB, lowest 10 roots with residual < 1e-6."""
    c = synthetic_case("polyene", lc=False)
    ref = _oracle_tda(c, 10, 1e-6)
    gpu = _solver(gpu_ctx, c).run_tda(10, 450, 1e-6)
    _check_solution(gpu, ref, e_tol=1e-8)


def test_all_roots_known_answer_water(gpu_ctx):
    """n_roots equal to the full singles dimension (8) on tincr's water known answer
    (not_refactored_tests/solver.rs:32-198): energies to 1e-10."""
    from tincr_gb300 import groundstate as gs
    from cases import FIXTURE_BOHR
    k = golden("kat_excited_energies_tda_routine")
    sy = gs.build_system([8, 1, 1], k["positions"] / FIXTURE_BOHR, lc=True)
    sy.hubbard = np.array([0.4467609798860577, 0.47201583989641355, 0.47201583989641355])
    s = T.ExcitedStateSystem(gpu_ctx, [4, 1, 1], k["orbs"], k["S"], k["orbe"], 4, 2, gs.gamma_atomwise(sy, 0.0),
                             gs.gamma_atomwise(sy, 3.03), sy.xyz)
    res = s.run_tda(8, 50, 1e-10)
    assert np.abs(res["ci_eigenvalues"] - k["omega_ref_out"]).max() < 1e-10


def test_single_excitation_space(gpu_ctx):
    """H2: one occupied, one virtual orbital (smallest possible problem)."""
    c = _case("h2", True)
    ref = _oracle_tda(c, 1, 1e-10)
    gpu = _solver(gpu_ctx, c).run_tda(1, 10, 1e-10)
    assert abs(gpu["ci_eigenvalues"][0] - ref["energies"][0]) < 1e-12


def test_collapse_path(gpu_ctx):
    """One root on a 27-water cluster: the subspace reaches 15 vectors and collapses twice
    (davidson.rs:172-176) before the residual drops below 1e-6."""
    c = synthetic_case("water27", True)
    hist = []
    o = oracle_inputs(c)
    ref = OT.run_tda(o["omega"], o["q_ov"], o["gamma"], c["xyz"], 1, 200, 1e-6, o["q_oo"], o["q_vv"], o["gamma_lr"],
                     o["n_occ"], o["n_virt"], history=hist)
    assert [h["n_sub"] for h in hist].count(1) >= 2      # collapsed at least once after the start
    gpu = _solver(gpu_ctx, c).run_tda(1, 200, 1e-6)
    assert abs(gpu["ci_eigenvalues"][0] - ref["energies"][0]) < 1e-9
    assert abs(gpu["davidson_iterations"] - ref["iterations"]) <= 2


def test_not_converged_and_bad_arguments(gpu_ctx):
    c = _case("uracil", True)
    s = _solver(gpu_ctx, c)
    with pytest.raises(T.DavidsonError):
        s.run_tda(4, 1, 1e-12)
    res = s.run_tda(4, 1, 1e-12, raise_on_failure=False)
    assert res["davidson_iterations"] == 1
    with pytest.raises(_lib.TincrError) as e:
        s.run_tda(0, 10, 1e-6)
    assert e.value.status == _lib.BAD_ARG
    bad = dict(c)
    bad["orbs"] = c["orbs"].copy()
    bad["orbs"][3, 2] = np.nan
    with pytest.raises(_lib.TincrError) as e:
        _solver(gpu_ctx, bad).prepare_tda()
    assert e.value.status == _lib.NONFINITE
    with pytest.raises(_lib.TincrError) as e:
        T.ExcitedStateSystem(gpu_ctx, [1, 1], c["orbs"], c["s"], c["orbe"], c["n_occ"], c["n_virt"], c["gamma"],
                             c["gamma_lr"], c["xyz"]).prepare_tda()
    assert e.value.status == _lib.BAD_ARG


@pytest.mark.parametrize("plane", ["tc", "mma"])
@pytest.mark.parametrize("name,lc", [("h2o", True), ("uracil", True), ("uracil", False), ("polyene8", True)])
def test_mixed_plane_gemms_match_fp64(monkeypatch, name, lc, plane):
    """Both plane GEMMs (tcgen05 + TMA, warp MMA) give the same three-plane split-BF16 A.X, within
    1e-6 of the FP64 product relative to max |A.X|, with and without the long-range exchange."""
    monkeypatch.setenv("TINCR_GB300_PLANE_GEMM", plane)
    ctx = _lib.Context(0)
    try:
        c = _case(name, lc)
        s = _solver(ctx, c)
        x = np.random.default_rng(11).standard_normal((c["n_occ"] * c["n_virt"], 5))
        ref = s.compute_products(x)
        mix = s.compute_products(x, precision=_lib.PREC_BF16X3)
        assert np.abs(mix - ref).max() < 1e-6 * np.abs(ref).max()
    finally:
        ctx.close()


@pytest.mark.parametrize("name", ["uracil", "water27"])
def test_mixed_products_close_to_fp64(gpu_ctx, name):
    """Split-BF16 contractions: A.X within 1e-6 of the FP64 product (relative to max |A.X|)."""
    c = _case(name, True)
    s = _solver(gpu_ctx, c)
    x = np.random.default_rng(5).standard_normal((c["n_occ"] * c["n_virt"], 4))
    ref = s.compute_products(x)
    mix = s.compute_products(x, precision=_lib.PREC_BF16X3)
    assert np.abs(mix - ref).max() < 1e-6 * np.abs(ref).max()


@pytest.mark.parametrize("plane", ["tc", "mma"])
@pytest.mark.parametrize("name", ["water27", "uracil"])
def test_mixed_davidson_energies_within_bar(monkeypatch, name, plane):
    """Mixed form at tolerance 1e-6 (mixed operator only): every root within 1e-6 Eh of the FP64 GPU
    roots (the mixed-form target), with either plane GEMM."""
    monkeypatch.setenv("TINCR_GB300_PLANE_GEMM", plane)
    ctx = _lib.Context(0)
    try:
        c = _case(name, True)
        ref = _solver(ctx, c).run_tda(6, 300, 1e-6)
        e_ref = ref["ci_eigenvalues"].copy()
        s = _solver(ctx, c)
        mix = s.run_tda(6, 300, 1e-6, precision=_lib.PREC_BF16X3)
        err = np.abs(mix["ci_eigenvalues"] - e_ref)
        print("%s %s per-root |dE| (Eh):" % (name, plane), " ".join("%.2e" % e for e in err))
        hist = ctx.davidson_history()
        if err.max() >= 1e-6:
            print("mixed energies", mix["ci_eigenvalues"])
            for h in hist:
                print(h)
        assert err.max() < 1e-6
        assert all(h["precision"] == _lib.PREC_BF16X3 for h in hist)
    finally:
        ctx.close()


def test_mixed_davidson_tight_tolerance_finishes_in_fp64(gpu_ctx):
    """Below the mixed operator's resolution (tolerance 1e-8) the solve ends with FP64 iterations:
    energies within 1e-10 Eh of the FP64 solve and the last residual is that of the FP64 operator."""
    c = _case("water27", True)
    ref = _solver(gpu_ctx, c).run_tda(4, 300, 1e-8)
    mix = _solver(gpu_ctx, c).run_tda(4, 300, 1e-8, precision=_lib.PREC_BF16X3)
    hist = gpu_ctx.davidson_history()
    assert hist[0]["precision"] == _lib.PREC_BF16X3 and hist[-1]["precision"] == _lib.PREC_FP64
    assert hist[-1]["max_residual"] < 1e-8
    assert np.abs(mix["ci_eigenvalues"] - ref["ci_eigenvalues"]).max() < 1e-10
