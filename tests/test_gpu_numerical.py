"""Finite-difference gradients with the batched GPU SCC (tincr_gb300/numerical.py, tincr's
gradients/numerical.rs): against the analytic gradients of the "exact" variant (the derivative of
the energies computed), and against central differences whose displaced SCCs run on the host."""

import numpy as np
import pytest

from cases import displaced_scc
from tincr_gb300 import geometry as G
from tincr_gb300 import gradients as GR
from tincr_gb300 import groundstate as gs
from tincr_gb300 import numerical as NUM
from tincr_gb300 import tda as T

pytestmark = pytest.mark.gpu


def _water_ammonia(lc):
    zw, xw = G.water_cluster(1, 1, 1)
    za = np.array([7, 1, 1, 1], np.int32)
    xa = np.array([[0.0, 0.0, 0.0], [0.94, 0.0, -0.38], [-0.47, 0.81, -0.38], [-0.47, -0.81, -0.38]])
    z = np.concatenate([zw, za])
    x = np.concatenate([xw, xa + np.array([2.9, 0.4, 0.3])])
    sy = gs.build_system(z, G.to_bohr(x), lc=lc)
    return sy, gs.run_scc(sy, tol=1e-11)


@pytest.mark.parametrize("lc", [True, False])
def test_fd_gradient_matches_exact_analytic(gpu_ctx, lc):
    sy, g = _water_ammonia(lc)
    es = T.ExcitedStateSystem.from_ground_state(gpu_ctx, sy, g)
    es.run_tda(2, 450, 1e-8)
    ggs, gex = GR.GradientSystem(es, sy, g).both(0, "exact")
    fd_gs, fd_exc = NUM.fd_gradient(gpu_ctx, sy, n_roots=1, h=1e-4)
    print("lc=%s: |FD - analytic| ground %.1e, S1 excitation %.1e" %
          (lc, np.abs(fd_gs - ggs).max(), np.abs(fd_exc[0] - gex).max()))
    assert np.abs(fd_gs - ggs).max() < 1e-6
    assert np.abs(fd_exc[0] - gex).max() < 1e-5


def test_fd_gradient_equals_host_scc_differences(gpu_ctx):
    sy, g = _water_ammonia(True)
    coords = [0, 4, 11, 19]
    _, fd = NUM.fd_gradient(gpu_ctx, sy, n_roots=2, h=1e-4, coords=coords)
    disp = displaced_scc(sy.numbers, sy.xyz, True, 1e-4)
    for c in coords:
        e = []
        for sgn, a in zip((1.0, -1.0), disp[c]):
            xyz = sy.xyz.copy()
            xyz[c // 3, c % 3] += sgn * 1e-4
            d = T.ExcitedStateSystem(gpu_ctx, sy.orbs_per_atom, a["orbs"], a["s"], a["orbe"], sy.n_occ, sy.n_virt,
                                     a["gamma"], a["gamma_lr"], xyz)
            e.append(d.run_tda(2, 450, 1e-8)["ci_eigenvalues"].copy())
        host = (e[0] - e[1]) / 2e-4
        assert np.abs(fd[:, c] - host).max() < 1e-7, c


def test_ridders_extrapolation(gpu_ctx):
    """Ridders' method (tincr's ridders_method constants) on a few coordinates: within 1e-6 of the
    analytic exact ground-state gradient, and no farther from it than the single central difference."""
    sy, g = _water_ammonia(True)
    es = T.ExcitedStateSystem.from_ground_state(gpu_ctx, sy, g)
    es.run_tda(1, 450, 1e-8)
    ggs, _ = GR.GradientSystem(es, sy, g).both(0, "exact")
    coords = [1, 7, 13]
    r_gs, _ = NUM.fd_gradient(gpu_ctx, sy, h=1e-3, coords=coords, ridders=4)
    c_gs, _ = NUM.fd_gradient(gpu_ctx, sy, h=1e-3, coords=coords)
    for c in coords:
        assert abs(r_gs[c] - ggs[c]) < 1e-6
        assert abs(r_gs[c] - ggs[c]) <= abs(c_gs[c] - ggs[c]) + 1e-9
