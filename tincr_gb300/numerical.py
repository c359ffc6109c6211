"""Finite-difference gradients on the GPU: every displaced geometry's SCC in one batched GPU SCC.

tincr checks its analytic gradients against numerical derivatives of the SCC energy and of the TDA
excitation energies (src/gradients/numerical.rs: `gs_gradient_wrapper`, `tda_gradient_wrapper`,
`finite_difference`, `ridders_method`): one SCC, and one TDA, per displaced geometry.  Here the
6N displaced geometries (+h and -h along every Cartesian coordinate) run as one `tincr_scc_batch`
call, and their TDAs as one batched TDA on the GPU from those ground states.  The derivatives are central
differences with one step (tincr's `finite_difference`); `ridders` adds Ridders' extrapolation
over a fixed ladder of steps h, h/1.4, h/1.4^2, ... (the constants of `ridders_method`), all
levels evaluated in the same batch."""

import numpy as np

from . import _lib
from . import groundstate as gs
from . import scc as gscc
from . import tda as T


def _displaced(sysm, coords, steps):
    systems, index = [], []
    for c in coords:
        for h in steps:
            for sgn in (1.0, -1.0):
                xyz = sysm.xyz.copy()
                xyz[c // 3, c % 3] += sgn * h
                systems.append(gs.build_system(sysm.numbers, xyz, lc=sysm.lc, r_lr=sysm.r_lr if sysm.lc else 0.0,
                                               params=sysm.params, sk_tail=sysm.sk_tail))
                index.append((c, h, sgn))
    return systems, index


def energies_at(ctx, systems, n_roots=0, scc_tol=1e-11, tda_tol=1e-8, max_iter=450, fp32_start=False):
    """SCC energies (batched GPU SCC) and, with n_roots > 0, the n_roots lowest TDA excitation
    energies (FP64) of every system: all systems in one batched TDA (`tincr_tda_solve_batch`, the
    FMO batch, tincr's Davidson per instance) for up to 6 roots, one GPU Davidson per system above.
    Returns (e_scc [n], e_exc [n, n_roots])."""
    grounds, _ = gscc.scc_batch(ctx, systems, tol=scc_tol, fp32_start=fp32_start, require_convergence=True)
    e_scc = np.array([g.energy for g in grounds])
    e_exc = np.zeros((len(systems), n_roots))
    if 0 < n_roots <= 6:
        from . import fmo
        inst = []
        for sy, g in zip(systems, grounds):
            no, nv = sy.n_occ, sy.n_virt
            inst.append(dict(n_atoms=sy.n_atoms, n_orb=sy.n_orbs, n_occ=no, n_virt=nv, n_roots=n_roots,
                             opa=sy.orbs_per_atom.astype(np.int32), c=g.orbs[:, :no + nv], s=g.s,
                             orbe=g.orbe[:no + nv], gamma=g.gamma, gamma_lr=g.gamma_lr if sy.lc else None, xyz=sy.xyz))
        rc, res = fmo.solve_batch(ctx, inst, max_iter, tda_tol, _lib.PREC_FP64)
        if rc != _lib.OK:
            raise T.DavidsonError("batched Davidson did not converge for every displaced geometry")
        e_exc = np.array([r["energies"] for r in res])
    elif n_roots > 6:
        for k, (sy, g) in enumerate(zip(systems, grounds)):
            es = T.ExcitedStateSystem.from_ground_state(ctx, sy, g)
            e_exc[k] = es.run_tda(n_roots, max_iter, tda_tol, precision=_lib.PREC_FP64)["ci_eigenvalues"]
    return e_scc, e_exc


def fd_gradient(ctx, sysm, n_roots=0, h=1e-4, coords=None, ridders=0, scc_tol=1e-11, tda_tol=1e-8,
                fp32_start=False):
    """Numerical gradients of the SCC energy and of the n_roots lowest excitation energies of `sysm`
    over the Cartesian coordinates `coords` (default: all 3N), in Hartree/bohr.

    ridders = 0: central differences with step h.  ridders = L > 0: Ridders' extrapolation as
    tincr's `ridders_method` (src/gradients/numerical.rs:90-157: con = 1.4, safe = 2, Neville tableau
    over the steps h / 1.4^k, k <= L, the estimate of the smallest error so far in each row, the
    early stop when the diagonal grows by safe x error below 1e-5); all L + 1 steps are evaluated in
    the same batch.  Returns (grad_scc [3N], grad_exc [n_roots, 3N]); coordinates outside `coords`
    are NaN."""
    n3 = sysm.xyz.size
    coords = list(range(n3)) if coords is None else [int(c) for c in coords]
    con = 1.4
    steps = [h / con ** k for k in range(int(ridders) + 1)]
    systems, index = _displaced(sysm, coords, steps)
    e_scc, e_exc = energies_at(ctx, systems, n_roots, scc_tol, tda_tol, fp32_start=fp32_start)
    vals = np.concatenate([e_scc[:, None], e_exc], axis=1)   # [systems, 1 + n_roots]
    pos = {key: k for k, key in enumerate(index)}
    out = np.full((1 + n_roots, n3), np.nan)
    for c in coords:
        d = [(vals[pos[(c, s, 1.0)]] - vals[pos[(c, s, -1.0)]]) / (2.0 * s) for s in steps]
        if ridders == 0:
            out[:, c] = d[0]
            continue
        for q in range(1 + n_roots):   # ridders_method, quantity by quantity
            tab = [[d[0][q]]]
            err, est = 0.0, d[0][q]
            for i in range(1, len(steps)):
                tab.append([d[i][q]])
                fac = con * con
                for j in range(1, i + 1):
                    tab[i].append((tab[i][j - 1] * fac - tab[i - 1][j - 1]) / (fac - 1.0))
                    fac *= con * con
                    cur = max(abs(tab[i][j] - tab[i][j - 1]), abs(tab[i][j] - tab[i - 1][j - 1]))
                    if j == 1 or cur <= err:
                        err, est = cur, tab[i][j]
                if abs(tab[i][i] - tab[i - 1][i - 1]) >= 2.0 * err and err < 1.0e-5:
                    break
            out[q, c] = est
    return out[0], out[1:]
