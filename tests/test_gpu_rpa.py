"""RPA / Casida on the GPU (`tincr_rpa_solve`, `ExcitedStateSystem.run_rpa`) against the oracle's
dense Casida statement (oracle/rpa.py, tincr's casida.rs / a_and_b.rs): LC and non-LC systems, the
lowest roots within 1e-9 Eh, X+Y and X-Y within 1e-5 (up to sign), oscillator strengths within 1e-7
(the vectors are converged to a residual of 1e-7),
(X+Y)^T (X-Y) = 1; a TDA solve on the same context is unaffected."""

import numpy as np
import pytest

from cases import oracle_inputs, synthetic_case
from oracle import rpa as OR
from tincr_gb300 import _lib
from tincr_gb300 import tda as T

pytestmark = pytest.mark.gpu


def _system(ctx, c):
    return T.ExcitedStateSystem(ctx, c["opa"], c["orbs"], c["s"], c["orbe"], c["n_occ"], c["n_virt"], c["gamma"],
                                c["gamma_lr"], c["xyz"])


def _signs(x):
    idx = np.argmax(np.abs(x), axis=0)
    return np.sign(x[idx, np.arange(x.shape[1])])


@pytest.mark.parametrize("name,lc", [("water8", True), ("polyene8", False), ("naphthalene", True),
                                     ("polyene8", True)])
def test_rpa_matches_dense_casida(gpu_ctx, name, lc):
    c = synthetic_case(name, lc=lc)
    o = oracle_inputs(c)
    a, b = OR.a_b_matrices(o["omega"], o["q_ov"], o["gamma"], o["q_oo"], o["q_vv"], o["gamma_lr"], o["n_occ"],
                           o["n_virt"])
    om, xpy, xmy = OR.casida(a, b)
    k = 6
    es = _system(gpu_ctx, c)
    r = es.run_rpa(k, 100, 1e-7)
    e = r["rpa_eigenvalues"]
    assert np.abs(e - om[:k]).max() < 1e-9, (e, om[:k])
    gp, gm = r["XpY"], r["XmY"]
    assert np.abs(np.einsum("xi,xi->i", gp, gm) - 1.0).max() < 1e-9
    s = _signs(xpy[:, :k]) * _signs(gp)
    assert np.abs(gp * s - xpy[:, :k]).max() < 1e-5
    assert np.abs(gm * s - xmy[:, :k]).max() < 1e-5
    # oscillator strengths: 2/3 Omega |xyz^T q_ov (X+Y)|^2
    mu = c["xyz"].T @ (o["q_ov"] @ xpy[:, :k])
    f = 2.0 / 3.0 * om[:k] * np.einsum("ci,ci->i", mu, mu)
    assert np.abs(r["rpa_oscillator_strengths"] - f).max() < 1e-7


def test_rpa_leaves_tda_state(gpu_ctx):
    c = synthetic_case("water8", lc=True)
    es = _system(gpu_ctx, c)
    before = es.run_tda(4, 100, 1e-8)["ci_eigenvalues"].copy()
    es.run_rpa(4, 100, 1e-7)
    assert np.all(es.properties["rpa_eigenvalues"] <= before + 1e-10)
    after = es.run_tda(4, 100, 1e-8)["ci_eigenvalues"]
    assert np.abs(after - before).max() < 1e-12


def test_rpa_iteration_cap(gpu_ctx):
    c = synthetic_case("water27", lc=True)
    es = _system(gpu_ctx, c)
    with pytest.raises(T.DavidsonError):
        es.run_rpa(6, 1, 1e-9)
    r = es.run_rpa(6, 1, 1e-9, raise_on_failure=False)
    assert r["rpa_iterations"] == 1


def test_rpa_arguments(gpu_ctx):
    """Bad arguments come back as BAD_ARG; one root of the smallest fixture system (water) against
    the dense Casida statement."""
    c = synthetic_case("water8", lc=True)
    es = _system(gpu_ctx, c)
    for n_roots, max_iter, tol in ((0, 10, 1e-6), (3, 0, 1e-6), (3, 10, 0.0), (10 ** 6, 10, 1e-6)):
        with pytest.raises(_lib.TincrError) as e:
            es.run_rpa(n_roots, max_iter, tol)
        assert e.value.status == _lib.BAD_ARG
    o = oracle_inputs(c)
    a, b = OR.a_b_matrices(o["omega"], o["q_ov"], o["gamma"], o["q_oo"], o["q_vv"], o["gamma_lr"], o["n_occ"],
                           o["n_virt"])
    om, _, _ = OR.casida(a, b)
    assert abs(es.run_rpa(1, 100, 1e-8)["rpa_eigenvalues"][0] - om[0]) < 1e-10
