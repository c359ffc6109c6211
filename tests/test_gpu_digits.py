"""FP64-accurate digit GEMM on the tensor cores (`tincr_gemm_fp64_tensor`, the subspace products of
the mixed Davidson): C = A B^T against an extended-precision reference (numpy long double),
within 2^-51 of the fixed-point error scale max|a| sum|b| + sum|a| max|b| + K max|a| max|b|, on Gaussian,
localised and cancelling data, ragged sizes, K split over the SMs; zero rows; non-finite input.
The mixed Davidson with the digit GEMMs takes the same iterations as with FP64 subspace products."""

import numpy as np
import pytest

from cases import synthetic_case
from tincr_gb300 import _lib
from tincr_gb300 import tda as T

pytestmark = pytest.mark.gpu


def _exact(a, b):
    """A B^T in extended precision (long double: at least 64-bit significands, products of two 53-bit
    significands are rounded at 2^-64 relative or better)."""
    la, lb = a.astype(np.longdouble), b.astype(np.longdouble)
    return (la @ lb.T).astype(np.float64)


def _bound(a, b):
    """Error scale of the fixed-point digits: truncation of each operand to 2^-56 of its row bound
    (max|a| sum|b| + sum|a| max|b|) and the dropped digit levels (up to K max|a| max|b|)."""
    ma, mb = np.abs(a).max(1)[:, None], np.abs(b).max(1)[None, :]
    return ma * np.abs(b).sum(1)[None, :] + np.abs(a).sum(1)[:, None] * mb + a.shape[1] * ma * mb


def _data(rng, m, k, kind):
    x = rng.standard_normal((m, k))
    if kind == "localized":
        x *= np.exp(-np.arange(k) / max(1, k / 8))[None, :]
        x[:, :3] *= 1e3
    elif kind == "wide":
        x *= 10.0 ** rng.uniform(-8, 8, (m, 1))
    return x


@pytest.mark.parametrize("M,N,K", [(1, 1, 1), (5, 3, 70), (128, 32, 640), (200, 17, 1000), (300, 20, 2100)])
@pytest.mark.parametrize("kind", ["gauss", "localized", "wide"])
def test_digit_gemm_exact_reference(gpu_ctx, M, N, K, kind):
    rng = np.random.default_rng(M * 7 + N * 3 + K)
    a, b = _data(rng, M, K, kind), _data(rng, N, K, kind)
    if kind == "gauss" and M > 1:
        b[0] = a[0] * (1 + 1e-9 * rng.standard_normal(K))   # near-cancelling pair
        b[0, ::2] *= -1
    c = gpu_ctx.gemm_fp64_tensor(a, b)
    ref = _exact(a, b)
    err = np.abs(c - ref) / _bound(a, b)
    print("max error / bound = %.2e" % err.max())
    assert err.max() < 2.0 ** -51


def test_digit_gemm_long_k_against_fp64(gpu_ctx):
    """K = 131072 (the water128 singles space), split over the SMs: within FP64 rounding of numpy."""
    rng = np.random.default_rng(9)
    a, b = rng.standard_normal((150, 131072)), rng.standard_normal((20, 131072))
    c = gpu_ctx.gemm_fp64_tensor(a, b)
    assert np.abs(c - a @ b.T).max() < 1e-16 * _bound(a, b).max() * 4


def test_digit_gemm_zero_rows_and_nonfinite(gpu_ctx):
    a = np.zeros((3, 100))
    a[1, 5] = 2.5
    b = np.ones((2, 100))
    c = gpu_ctx.gemm_fp64_tensor(a, b)
    assert np.array_equal(c, np.array([[0.0, 0.0], [2.5, 2.5], [0.0, 0.0]]))
    a[2, 7] = np.inf
    with pytest.raises(_lib.TincrError) as e:
        gpu_ctx.gemm_fp64_tensor(a, b)
    assert e.value.status == _lib.NONFINITE
    c = gpu_ctx.gemm_fp64_tensor(np.eye(4), np.eye(4))   # usable afterwards
    assert np.array_equal(c, np.eye(4))


def test_mixed_davidson_digit_and_fp64_subspace_agree(gpu_ctx, monkeypatch):
    """water27 LC-TDA, 6 roots to residual 1e-5, mixed form: the subspace products as digit GEMMs or
    in FP64 give the same Davidson history and roots within 1e-7 Eh (both carry the mixed A.X
    operator's error; the mixed-form target against FP64 is 1e-6 Eh)."""
    c = synthetic_case("water27", True)

    def run(ctx):
        s = T.ExcitedStateSystem(ctx, c["opa"], c["orbs"], c["s"], c["orbe"], c["n_occ"], c["n_virt"], c["gamma"],
                                 c["gamma_lr"], c["xyz"])
        r = s.run_tda(6, 200, 1e-5, precision=_lib.PREC_BF16X3)
        return r, ctx.davidson_history()

    dg, hd = run(gpu_ctx)
    monkeypatch.setenv("TINCR_GB300_SUBSPACE_GEMM", "fp64")
    ctx = _lib.Context(0)
    try:
        f64, hf = run(ctx)
    finally:
        ctx.close()
    print("iterations", len(hd), len(hf), "max |dE| %.2e" % np.abs(dg["ci_eigenvalues"] - f64["ci_eigenvalues"]).max())
    assert [h["n_sub"] for h in hd] == [h["n_sub"] for h in hf]
    assert np.abs(dg["ci_eigenvalues"] - f64["ci_eigenvalues"]).max() < 1e-7
