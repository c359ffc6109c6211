"""GPU test of tincr_tda_products_noalloc, the A.X product that allocates no device memory.

It serves callers that own all device memory themselves (an MD or FMO driver with its own pool
allocator) or cannot accept cudaMalloc/cudaFree synchronisation between their kernels.  The test
calls it through the C ABI with caller-owned device buffers and checks it against the regular
entry point (tincr_tda_products) at the FP64 product tolerance of the other tests, on two calls in
a row, and checks that a system too large for the fixed scratch array is rejected.

Collected last on purpose (file name) so that a failure here stops a -x run only after every
other test has run."""

import ctypes

import numpy as np
import pytest

from cases import fixture_case, synthetic_case
from tincr_gb300 import _lib
from tincr_gb300 import tda as T

pytestmark = pytest.mark.gpu


def _noalloc(ctx, x_vecmajor):
    import torch
    xd = torch.from_numpy(np.ascontiguousarray(x_vecmajor)).to("cuda")
    ad = torch.empty_like(xd)
    torch.cuda.synchronize()
    rc = ctx.lib.tincr_tda_products_noalloc(ctx.h, xd.shape[0], ctypes.c_void_p(xd.data_ptr()),
                                            ctypes.c_void_p(ad.data_ptr()))
    ctx.check(rc)
    torch.cuda.synchronize()
    return ad.cpu().numpy()


@pytest.mark.parametrize("name,lc", [("uracil", True), ("uracil", False), ("water27", True)])
def test_noalloc_products_match_regular_entry_point(gpu_ctx, name, lc):
    pytest.importorskip("torch")
    c = fixture_case(name, lc) if name == "uracil" else synthetic_case(name, lc)
    s = T.ExcitedStateSystem(gpu_ctx, c["opa"], c["orbs"], c["s"], c["orbe"], c["n_occ"], c["n_virt"], c["gamma"],
                             c["gamma_lr"], c["xyz"])
    s.prepare_tda()
    rng = np.random.default_rng(7)
    for k in (3, 2):                         # two calls in a row, different vectors and counts
        x = rng.standard_normal((s.dim, k))
        ref = s.compute_products(x)          # [ov, k]
        out = _noalloc(gpu_ctx, x.T).T       # device buffers are vector-major [k, ov]
        assert np.abs(out - ref).max() < 1e-12 * max(1.0, np.abs(ref).max())


def test_noalloc_rejects_systems_beyond_the_scratch_size(gpu_ctx):
    pytest.importorskip("torch")
    n_atoms, n = 384, 1536                   # 4 n^2 doubles of exchange scratch alone exceed 32 MiB
    opa = np.full(n_atoms, 4, np.int32)
    eye = np.eye(n)
    s = T.ExcitedStateSystem(gpu_ctx, opa, eye, eye, np.arange(n, dtype=float), 1024, 512, np.eye(n_atoms),
                             0.5 * np.eye(n_atoms), np.zeros((n_atoms, 3)))
    s.prepare_tda()
    with pytest.raises(_lib.TincrError) as e:
        _noalloc(gpu_ctx, np.zeros((1, s.dim)))
    assert e.value.status == _lib.BAD_ARG
    assert "scratch" in str(e.value)
