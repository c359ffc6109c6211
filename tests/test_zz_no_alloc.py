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
    """Copy the vectors to the device on torch's default stream and call the entry point at once:
    the call orders itself after the legacy default stream, so no host synchronisation is needed
    before it (it synchronises its own stream before returning)."""
    import torch
    xd = torch.from_numpy(np.ascontiguousarray(x_vecmajor)).to("cuda")
    ad = torch.empty_like(xd)
    rc = ctx.lib.tincr_tda_products_noalloc(ctx.h, xd.shape[0], ctypes.c_void_p(xd.data_ptr()),
                                            ctypes.c_void_p(ad.data_ptr()))
    ctx.check(rc)
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


def test_noalloc_rejects_host_pointers(gpu_ctx):
    """A host buffer passed in place of device memory is refused before any kernel runs."""
    pytest.importorskip("torch")
    import torch
    c = fixture_case("uracil", True)
    s = T.ExcitedStateSystem(gpu_ctx, c["opa"], c["orbs"], c["s"], c["orbe"], c["n_occ"], c["n_virt"], c["gamma"],
                             c["gamma_lr"], c["xyz"])
    s.prepare_tda()
    host = np.zeros((1, s.dim))
    dev = torch.zeros((1, s.dim), dtype=torch.float64, device="cuda")
    for x_ptr, ax_ptr in ((host.ctypes.data, dev.data_ptr()), (dev.data_ptr(), host.ctypes.data)):
        rc = gpu_ctx.lib.tincr_tda_products_noalloc(gpu_ctx.h, 1, ctypes.c_void_p(x_ptr), ctypes.c_void_p(ax_ptr))
        assert rc == _lib.BAD_ARG
        assert "device memory" in gpu_ctx.lib.tincr_last_error(gpu_ctx.h).decode()
    # the context is still usable afterwards
    x = np.random.default_rng(1).standard_normal((s.dim, 1))
    ref = s.compute_products(x)
    assert np.abs(_noalloc(gpu_ctx, x.T).T - ref).max() < 1e-12 * max(1.0, np.abs(ref).max())
