"""Failure path of the bounded device waits: a tcgen05 plane GEMM whose pipeline wait runs out.

Every mbarrier wait of the tensor-core kernels gives up after a limit (2 s), records an error code,
drains the copies and MMAs it has in flight, frees its TMEM and returns, so the GPU and the CUDA
context stay usable and the host reports TINCR_CUDA_ERR at the call's next synchronisation.  The test
hook tincr_debug_tc_first_wait sets the limit of the MMA issuer's first wait to 0 (it gives up
without waiting, the other waits of the CTA then run out after their 2 s), which makes the path run
on purpose, with no invalid kernel, address or trap: the call must fail with TINCR_CUDA_ERR, and the
same context (after the hook is reset) and a fresh one must give the normal product again."""

import numpy as np
import pytest

from cases import fixture_case
from tincr_gb300 import _lib
from tincr_gb300 import tda as T

pytestmark = pytest.mark.gpu


def _system(ctx):
    c = fixture_case("uracil", True)
    s = T.ExcitedStateSystem(ctx, c["opa"], c["orbs"], c["s"], c["orbe"], c["n_occ"], c["n_virt"], c["gamma"],
                             c["gamma_lr"], c["xyz"])
    s.prepare_tda()
    return s


def test_plane_gemm_wait_runs_out_and_is_reported(monkeypatch):
    monkeypatch.setenv("TINCR_GB300_PLANE_GEMM", "tc")
    ctx = _lib.Context(0)
    try:
        s = _system(ctx)
        x = np.random.default_rng(5).standard_normal((s.dim, 1))
        ref = s.compute_products(x, precision=_lib.PREC_BF16X3)
        ctx.check(ctx.lib.tincr_debug_tc_first_wait(ctx.h, 0))
        with pytest.raises(_lib.TincrError) as e:
            s.compute_products(x, precision=_lib.PREC_BF16X3)
        assert e.value.status == _lib.CUDA_ERR
        assert "timed out" in str(e.value)
        ctx.check(ctx.lib.tincr_debug_tc_first_wait(ctx.h, -1))
        again = s.compute_products(x, precision=_lib.PREC_BF16X3)
        assert np.array_equal(again, ref)
    finally:
        ctx.close()
    fresh = _lib.Context(0)
    try:
        s = _system(fresh)
        assert np.array_equal(s.compute_products(x, precision=_lib.PREC_BF16X3), ref)
    finally:
        fresh.close()
