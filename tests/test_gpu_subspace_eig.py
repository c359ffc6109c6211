"""Subspace eigensolvers of the Davidson loop (the Rayleigh-Ritz step, `eigh(UPLO::Upper)` in
src/excited_states/solvers/davidson.rs:93) through `tincr_subspace_eigh`: the host solver (default)
and the thread-block-cluster kernel (TINCR_GB300_SUBSPACE_EIG=cluster) give the k lowest
eigenpairs of LAPACK (numpy.linalg.eigh) on random symmetric matrices with separated, clustered and
exactly degenerate spectra; only the upper triangle is read; non-finite input is an error; matrices
too wide for the cluster's shared memory go to the host solver.  A Davidson solve with the cluster
kernel takes the same iterations and gives the same roots as with the host solver."""

import os

import numpy as np
import pytest

from cases import synthetic_case
from tincr_gb300 import _lib
from tincr_gb300 import tda as T

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cluster_ctx(gpu_ctx):
    old = os.environ.get("TINCR_GB300_SUBSPACE_EIG")
    os.environ["TINCR_GB300_SUBSPACE_EIG"] = "cluster"
    try:
        ctx = _lib.Context(0)
    finally:
        if old is None:
            del os.environ["TINCR_GB300_SUBSPACE_EIG"]
        else:
            os.environ["TINCR_GB300_SUBSPACE_EIG"] = old
    yield ctx
    ctx.close()


def _matrix(rng, m, kind):
    q, _ = np.linalg.qr(rng.standard_normal((m, m)))
    if kind == "random":
        ev = np.sort(rng.standard_normal(m))
    elif kind == "davidson":                   # a positive spectrum with close low roots, like a TDA subspace
        ev = np.sort(0.6 + 0.4 * rng.random(m))
        ev[: min(m, 8)] = 0.69 + 1e-4 * np.arange(min(m, 8))
    else:                                      # exact and near degeneracies
        ev = np.sort(rng.standard_normal(m))
        if m >= 6:
            ev[1] = ev[0]
            ev[3] = ev[2] + 1e-10
            ev[5] = ev[4] + 1e-6
    a = (q * ev) @ q.T
    return 0.5 * (a + a.T), ev


def _check(a, k, w, y, tol_w=1e-12):
    ref = np.linalg.eigvalsh(a)[:k]
    scale = max(1.0, np.abs(ref).max())
    assert np.abs(w - ref).max() < tol_w * scale
    assert np.abs(a @ y.T - y.T * w).max() < 1e-11 * scale
    assert np.abs(y @ y.T - np.eye(k)).max() < 1e-11


@pytest.mark.parametrize("m,k", [(1, 1), (2, 1), (3, 2), (17, 5), (64, 20), (150, 10), (300, 20), (450, 30)])
@pytest.mark.parametrize("kind", ["random", "davidson", "degenerate"])
@pytest.mark.parametrize("solver", ["host", "cluster"])
def test_eigh_matches_lapack(gpu_ctx, cluster_ctx, m, k, kind, solver):
    ctx = cluster_ctx if solver == "cluster" else gpu_ctx
    rng = np.random.default_rng(1000 * m + k)
    a, _ = _matrix(rng, m, kind)
    w, y, on_dev = ctx.subspace_eigh(a, k)
    assert on_dev == (solver == "cluster")
    _check(a, k, w, y)


def test_upper_triangle_only(cluster_ctx):
    rng = np.random.default_rng(3)
    a, _ = _matrix(rng, 120, "random")
    garbage = np.triu(a) + np.tril(rng.standard_normal((120, 120)) * 5.0, -1)
    w, y, on_dev = cluster_ctx.subspace_eigh(garbage, 12)
    assert on_dev
    _check(a, 12, w, y)


@pytest.mark.parametrize("solver", ["host", "cluster"])
def test_nonfinite_and_bad_arguments(gpu_ctx, cluster_ctx, solver):
    ctx = cluster_ctx if solver == "cluster" else gpu_ctx
    rng = np.random.default_rng(4)
    a, _ = _matrix(rng, 40, "random")
    a[3, 7] = np.nan
    with pytest.raises(_lib.TincrError) as e:
        ctx.subspace_eigh(a, 4)
    assert e.value.status == _lib.NONFINITE
    with pytest.raises(_lib.TincrError) as e:
        ctx.subspace_eigh(np.eye(3), 4)
    assert e.value.status == _lib.BAD_ARG
    # the context stays usable
    w, _, _ = ctx.subspace_eigh(np.diag([3.0, 1.0, 2.0]), 2)
    assert np.allclose(w, [1.0, 2.0], atol=1e-14)


def test_wide_subspace_uses_host(cluster_ctx):
    rng = np.random.default_rng(5)
    a, _ = _matrix(rng, 900, "davidson")
    w, y, on_dev = cluster_ctx.subspace_eigh(a, 20)
    assert not on_dev
    _check(a, 20, w, y)


def test_davidson_host_and_cluster_eigensolvers_agree(gpu_ctx, cluster_ctx):
    """water27 LC-TDA, 8 roots: the same Davidson iterations and subspace sizes, roots within 1e-11 Eh."""
    c = synthetic_case("water27", True)

    def run(ctx):
        s = T.ExcitedStateSystem(ctx, c["opa"], c["orbs"], c["s"], c["orbe"], c["n_occ"], c["n_virt"], c["gamma"],
                                 c["gamma_lr"], c["xyz"])
        r = s.run_tda(8, 200, 1e-7)
        return r, ctx.davidson_history()

    host, hh = run(gpu_ctx)
    dev, hd = run(cluster_ctx)
    assert dev["davidson_iterations"] == host["davidson_iterations"]
    assert [h["n_sub"] for h in hd] == [h["n_sub"] for h in hh]
    assert np.abs(dev["ci_eigenvalues"] - host["ci_eigenvalues"]).max() < 1e-11
    ov = np.abs(np.einsum("xr,xr->r", dev["ci_coefficients"], host["ci_coefficients"]))
    assert np.abs(ov - 1.0).max() < 1e-8
