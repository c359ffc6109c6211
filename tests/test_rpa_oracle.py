"""The RPA / Casida oracle (oracle/rpa.py): its A equals the TDA's dense A, its A + B reproduces
tincr's (A+B).v known answer, and its Casida solutions satisfy the RPA equations; with B = 0 the
roots are the TDA's."""

import numpy as np
import pytest

from cases import golden, oracle_inputs, synthetic_case
from oracle import rpa as OR
from oracle import tda as OT


def test_a_plus_b_matches_known_answer():
    d = golden("kat_test_apbv_fortran")
    q_ov, q_oo, q_vv = d["qtrans_ov"], d["qtrans_oo"], d["qtrans_vv"]
    n_atoms, no, nv = q_ov.shape
    a, b = OR.a_b_matrices(d["omega0"].reshape(-1), q_ov, d["gamma"], q_oo, q_vv, d["gamma_lr"], no, nv)
    bs = d["bs"]
    out = np.stack([((a + b) @ bs[:, :, k].reshape(-1)).reshape(no, nv) for k in range(bs.shape[2])], axis=2)
    assert np.abs(out - d["bp_ref"]).max() < 1e-14


@pytest.mark.parametrize("name,lc", [("water8", True), ("polyene8", False)])
def test_casida_solves_rpa_equations(name, lc):
    o = oracle_inputs(synthetic_case(name, lc=lc))
    a, b = OR.a_b_matrices(o["omega"], o["q_ov"], o["gamma"], o["q_oo"], o["q_vv"], o["gamma_lr"], o["n_occ"],
                           o["n_virt"])
    assert np.abs(a - OT.tda_full_matrix(o["omega"], o["q_ov"], o["gamma"], o["q_oo"], o["q_vv"], o["gamma_lr"],
                                         o["n_occ"], o["n_virt"])).max() < 1e-13
    assert np.abs(b - b.T).max() < 1e-13
    om, xpy, xmy = OR.casida(a, b)
    k = 6
    assert np.abs((a + b) @ xpy[:, :k] - xmy[:, :k] * om[:k]).max() < 1e-11
    assert np.abs((a - b) @ xmy[:, :k] - xpy[:, :k] * om[:k]).max() < 1e-11
    assert np.abs(np.einsum("xi,xi->i", xpy[:, :k], xmy[:, :k]) - 1.0).max() < 1e-11
    # RPA lies below TDA (the B coupling lowers the roots) and B = 0 gives the TDA roots
    tda = np.linalg.eigvalsh(a)
    assert np.all(om[:k] <= tda[:k] + 1e-12)
    om0, _, _ = OR.casida(a, np.zeros_like(b))
    assert np.abs(om0[:k] - tda[:k]).max() < 1e-11
