"""Batched SCC ground states on the GPU through the C ABI (`tincr_scc_batch`).

Mirrors tincr's SCC (`System::run_scc`, src/scc/scc_routine.rs:121-290, with `h0_and_s`,
src/scc/h0_and_s.rs:92-182, the gamma matrices and the LC exchange Hamiltonian) for many independent
systems at once: FMO monomers and pairs, displaced geometries.  The result of each system is a
`groundstate.GroundState`, the same record the host SCC (`groundstate.run_scc`) returns: S, H0,
orbitals, orbital energies, density, Mulliken charge differences, the converged Fock matrix and the
energy come from the GPU; gamma / gamma_lr (inputs of the later TDA) are the atomwise matrices of
`groundstate.gamma_atomwise`.

The convergence test is the host SCC's: the largest element of X^T (F P S - S P F) X below `tol`
(X = S^-1/2), with DIIS on the Fock matrix.  `fp32_start` runs the first iterations in FP32 until
that commutator is below 1e-5 and finishes in FP64 (the result is FP64 either way)."""

import numpy as np

from . import _lib
from . import groundstate as gs
from ._lib import dptr, iptr
from .gradients import parameter_tables, set_parameters

SYSTEM_DTYPE = np.dtype([("n_atoms", np.int32), ("n_orb", np.int32), ("n_occ", np.int32), ("pad", np.int32),
                         ("atom_off", np.int64), ("orb_off", np.int64), ("mat_off", np.int64),
                         ("pair_off", np.int64)])


class _Inputs(_lib.C.Structure):
    _fields_ = [("s", _lib.C.c_void_p), ("h0", _lib.C.c_void_p), ("gamma", _lib.C.c_void_p),
                ("gamma_lr", _lib.C.c_void_p)]


def _common(systems, attr):
    vals = {getattr(s, attr) if attr != "params" else id(s.params) for s in systems}
    if len(vals) != 1:
        raise ValueError("scc_batch: all systems must share %s" % attr)


def scc_batch(ctx, systems, tol=1e-10, max_iter=250, p_start=None, level_shift=0.0, fp32_start=False,
              given=None, require_convergence=False, full=True):
    """SCC ground states of `systems` (groundstate.System, sharing parameters, LC setting and SK tail
    rule) on the GPU.  `p_start`: None or a list with a starting density (or None) per system;
    `given`: None or a list of dicts with any of "s", "h0", "gamma", "gamma_lr" per system, used
    instead of the matrices the GPU builds.  `full=False` returns only the orbitals, orbital
    energies, charges and energy (the density, S, H0 and Fock matrix are None and not copied back).
    Returns (list of GroundState, status); with
    `require_convergence` a system that misses `tol` raises (tincr panics, src/fmo/scc/pair.rs:234-240)."""
    systems = list(systems)
    if not systems:
        return [], _lib.OK
    for attr in ("lc", "r_lr", "sk_tail", "params"):
        _common(systems, attr)
    s0 = systems[0]
    for sy in systems:
        if sy.n_elec % 2:
            raise ValueError("scc_batch: closed-shell systems only (odd electron count)")
    numbers = np.concatenate([sy.numbers for sy in systems])
    tables, kinds = parameter_tables(s0.params, numbers)
    set_parameters(ctx, tables)
    kind_energy = np.zeros(4 * tables["n_kinds"])
    for k, z in enumerate(tables["kind_z"]):
        el = s0.params.element(int(z))
        kind_energy[4 * k:4 * k + el.n_orbs] = el.energy
    n = len(systems)
    rec = np.zeros(n, SYSTEM_DTYPE)
    a = o = m = pr = 0
    for i, sy in enumerate(systems):
        rec[i] = (sy.n_atoms, sy.n_orbs, sy.n_elec // 2, 0, a, o, m, pr)
        a += sy.n_atoms
        o += sy.n_orbs
        m += sy.n_orbs ** 2
        pr += sy.n_atoms ** 2
    xyz = np.ascontiguousarray(np.concatenate([sy.xyz for sy in systems]).reshape(-1), dtype=np.float64)
    kinds = np.ascontiguousarray(kinds, dtype=np.int32)

    def packed(blocks, size):
        out = np.zeros(size)
        for i, b in enumerate(blocks):
            off = int(rec[i]["mat_off"]) if size == m else int(rec[i]["pair_off"])
            out[off:off + b.size] = np.asarray(b, dtype=np.float64).reshape(-1)
        return out

    ps = None
    if p_start is not None:
        ps = packed([p if p is not None else np.diag(sy.ao_occ.astype(np.float64))
                     for p, sy in zip(p_start, systems)], m)
    keep = []
    inputs = None
    if given is not None:
        inputs = _Inputs()
        for key, size in (("s", m), ("h0", m), ("gamma", pr), ("gamma_lr", pr)):
            if all(key in g for g in given):
                arr = packed([g[key] for g in given], size)
                keep.append(arr)
                setattr(inputs, key, arr.ctypes.data)
            elif any(key in g for g in given):
                raise ValueError("scc_batch: %s given for some systems only" % key)
    flags = (_lib.SCC_LC if s0.lc else 0) | (_lib.SCC_SK_EXTRAPOLATE if s0.sk_tail == "extrapolate" else 0) | \
        (_lib.SCC_FP32_START if fp32_start else 0)
    orbe, orbs, dq = np.zeros(o), np.zeros(m), np.zeros(a)
    p, s_out, h0_out, hcx = (np.zeros(m), np.zeros(m), np.zeros(m), np.zeros(m)) if full else (None,) * 4
    energy, res = np.zeros(n), np.zeros(n)
    its, conv = np.zeros(n, np.int32), np.zeros(n, np.int32)
    rc = ctx.lib.tincr_scc_batch(
        ctx.h, n, rec.ctypes.data, iptr(kinds), dptr(xyz), dptr(kind_energy),
        _lib.C.byref(inputs) if inputs is not None else None, dptr(ps), float(s0.r_lr if s0.lc else 0.0), flags,
        float(tol), int(max_iter), float(level_shift), dptr(orbe), dptr(orbs), dptr(p), dptr(dq), dptr(energy),
        dptr(s_out), dptr(h0_out), dptr(hcx), iptr(its), iptr(conv), dptr(res))
    ctx.check(rc, allow=(_lib.OK, _lib.NOT_CONVERGED))
    out = []
    for i, sy in enumerate(systems):
        no, mo, ao, nb = sy.n_orbs, int(rec[i]["mat_off"]), int(rec[i]["orb_off"]), int(rec[i]["atom_off"])
        blk = lambda x: None if x is None else x[mo:mo + no * no].reshape(no, no).copy()
        if not full:
            gam = glr = None
        elif given is not None and "gamma" in given[i]:
            gam = np.array(given[i]["gamma"], dtype=np.float64)
        else:
            gam = gs.gamma_atomwise(sy, 0.0)
        if not full:
            pass
        elif not sy.lc:
            glr = np.zeros_like(gam)
        elif given is not None and "gamma_lr" in given[i]:
            glr = np.array(given[i]["gamma_lr"], dtype=np.float64)
        else:
            glr = gs.gamma_atomwise(sy, sy.r_lr)
        out.append(gs.GroundState(
            s=blk(s_out), h0=blk(h0_out), gamma=gam, gamma_lr=glr, orbs=blk(orbs), orbe=orbe[ao:ao + no].copy(),
            p=blk(p), p0=np.diag(sy.ao_occ.astype(np.float64)) if full else None, dq=dq[nb:nb + sy.n_atoms].copy(),
            h_coul_x=blk(hcx),
            energy=float(energy[i]), iterations=int(its[i]), converged=bool(conv[i]), residual=float(res[i])))
    if require_convergence and rc == _lib.NOT_CONVERGED:
        bad = [i for i in range(n) if not conv[i]]
        raise RuntimeError("SCC not converged to %g in %d iterations: systems %s" % (tol, max_iter, bad[:20]))
    return out, rc


def last_ms(ctx):
    """Device time (ms) of the last tincr_scc_batch call (CUDA events around the kernel)."""
    return ctx.last_timing()[0]
