"""Host-side mirror of tincr's FMO excited-state set-up for the batched GPU TDA.

tincr (src/fmo/lcmo/basis.rs:449-533) runs one TDA per monomer (n_le locally excited roots,
max_iter 50, tolerance 1e-4; `Monomer::run_tda`) and, for the diabatic basis, one TDA per direction
of every monomer pair (n_ct roots, max_iter 150, tolerance 1e-4; `PairChargeTransfer::run_ct_tda`,
src/excited_states/tda/ct_pair.rs).  Here every such problem becomes one `tincr_tda_instance` and
the whole set is solved by `tincr_tda_solve_batch` in one call.

A CT pair direction (hole on monomer H, electron on monomer L) is passed as the dimer with
orbital block C = [C_H,occ (on H's AOs) | C_L,virt (on L's AOs)], the dimer overlap, gamma and
gamma_lr.  The dimer's Mulliken transition charges for that C are exactly tincr's pair charges:
q_ov from `calculate_q_ov` (ct_pair.rs:81-127, S_HL blocks), q_oo of H and q_vv of L (they vanish
on the other monomer's atoms), so A.X needs no special case.

The monomer ground states come from the host SCC of the isolated monomers (tincr's FMO SCC adds
the electrostatic embedding of the other monomers, src/fmo/scc; that step precedes the TDA path).
"""

import os
import weakref

import numpy as np

from . import _lib
from . import groundstate as gs
from ._lib import C as ct


class Monomer:
    """One fragment: its atoms in the aggregate, its System and its SCC ground state."""

    def __init__(self, index, atoms, system, ground):
        self.index = index
        self.atoms = atoms
        self.system = system
        self.ground = ground


def _monomer_scc(args):
    """Host SCC of one monomer (top-level for a spawn process pool)."""
    sy, tol = args
    return gs.run_scc(sy, tol=tol, require_convergence=True)


def build_monomers(numbers, xyz_bohr, monomer_of_atom, lc=True, r_lr=gs.LONG_RANGE_RADIUS, scc_tol=1e-10, workers=1,
                   scc="host", ctx=None):
    """Monomers by construction (one per distinct `monomer_of_atom` value), each with an SCC ground
    state: on the host (`workers` > 1: in a spawn process pool, one BLAS thread per worker) or, with
    scc="gpu", all monomers in one batched GPU SCC on `ctx` (tincr_scc_batch)."""
    systems = []
    for k in np.unique(monomer_of_atom):
        at = np.nonzero(monomer_of_atom == k)[0]
        systems.append((int(k), at, gs.build_system(numbers[at], xyz_bohr[at], lc=lc, r_lr=r_lr)))
    if scc == "gpu":
        from . import scc as gscc
        grounds, _ = gscc.scc_batch(ctx, [sy for _, _, sy in systems], tol=scc_tol, require_convergence=True)
    elif scc == "host":
        jobs = [(sy, scc_tol) for _, _, sy in systems]
        grounds = _pool_map(_monomer_scc, jobs, workers)
    else:
        raise ValueError("scc must be 'host' or 'gpu'")
    return [Monomer(k, at, sy, g) for (k, at, sy), g in zip(systems, grounds)]


def _pool_map(fn, jobs, workers, chunksize=4):
    """map(fn, jobs), in a spawn process pool when workers > 1 (the caller needs a __main__
    guard).  One BLAS thread per worker: the workers already fill the cores, and a full-width BLAS
    pool in each of them would oversubscribe the host."""
    if workers <= 1 or len(jobs) <= 1:
        return [fn(a) for a in jobs]
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    names = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")
    saved = {k: os.environ.get(k) for k in names}
    os.environ.update({k: "1" for k in names})
    try:
        with ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
            return list(ex.map(fn, jobs, chunksize=chunksize))
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def candidate_pairs(monomers, reach_bohr):
    """Pairs (I, J), I < J, whose bounding spheres (centroid, largest centroid-atom distance) come
    closer than `reach_bohr`: a superset of the pairs with an atom pair closer than that, found
    without the atom-by-atom distances of every pair of a large aggregate."""
    cen = np.array([m.system.xyz.mean(axis=0) for m in monomers])
    rad = np.array([np.linalg.norm(m.system.xyz - c, axis=1).max() for m, c in zip(monomers, cen)])
    d = np.linalg.norm(cen[:, None, :] - cen[None, :, :], axis=-1) - rad[:, None] - rad[None, :]
    i, j = np.nonzero(np.triu(d < reach_bohr, 1))
    return list(zip(i.tolist(), j.tolist()))


def close_pairs(monomers, cutoff_bohr):
    """Pairs (I, J), I < J, whose smallest interatomic distance is below the cutoff."""
    out = []
    for i, j in candidate_pairs(monomers, cutoff_bohr):
        a, b = monomers[i], monomers[j]
        d = np.linalg.norm(a.system.xyz[:, None, :] - b.system.xyz[None, :, :], axis=-1).min()
        if d < cutoff_bohr:
            out.append((i, j))
    return out


def monomer_instance(m, n_roots):
    """Instance of `Monomer::prepare_tda` / `run_tda` (tda/monomer.rs:8-53)."""
    sy, g = m.system, m.ground
    no, nv = sy.n_occ, sy.n_virt
    return dict(n_atoms=sy.n_atoms, n_orb=sy.n_orbs, n_occ=no, n_virt=nv, n_roots=n_roots,
                opa=sy.orbs_per_atom.astype(np.int32), c=g.orbs[:, :no + nv], s=g.s, orbe=g.orbe[:no + nv],
                gamma=g.gamma, gamma_lr=g.gamma_lr if sy.lc else None, xyz=sy.xyz)


class Dimer:
    """Overlap and gamma matrices of two monomers' atoms (H's atoms first)."""

    def __init__(self, mh, ml):
        sy = gs.build_system(np.concatenate([mh.system.numbers, ml.system.numbers]),
                             np.concatenate([mh.system.xyz, ml.system.xyz]), lc=mh.system.lc, r_lr=mh.system.r_lr)
        self.system = sy
        self.s, _ = gs.h0_and_s(sy)
        self.gamma = gs.gamma_atomwise(sy, 0.0)
        self.gamma_lr = gs.gamma_atomwise(sy, sy.r_lr) if sy.lc else None


def ct_instance(mh, ml, dimer, n_roots):
    """Instance of `PairChargeTransfer::prepare_ct_tda` (ct_pair.rs:12-79): hole on mh, electron on ml."""
    nh, nl = mh.system.n_orbs, ml.system.n_orbs
    oh, ol = mh.system.n_occ, ml.system.n_occ
    vl = ml.system.n_virt
    c = np.zeros((nh + nl, oh + vl))
    c[:nh, :oh] = mh.ground.orbs[:, :oh]
    c[nh:, oh:] = ml.ground.orbs[:, ol:ol + vl]
    orbe = np.concatenate([mh.ground.orbe[:oh], ml.ground.orbe[ol:ol + vl]])
    sy = dimer.system
    return dict(n_atoms=sy.n_atoms, n_orb=sy.n_orbs, n_occ=oh, n_virt=vl, n_roots=n_roots,
                opa=sy.orbs_per_atom.astype(np.int32), c=c, s=dimer.s, orbe=orbe, gamma=dimer.gamma,
                gamma_lr=dimer.gamma_lr, xyz=sy.xyz)


def aggregate_instances(monomers, pairs, n_le, n_ct):
    """tincr's FMO excited-state work list: every monomer (n_le roots), then both directions of
    every pair (n_ct roots): (I -> J) and (J -> I) (basis.rs:170-238)."""
    inst, labels = [], []
    for m in monomers:
        inst.append(monomer_instance(m, n_le))
        labels.append(("LE", m.index))
    for i, j in pairs:
        inst.append(ct_instance(monomers[i], monomers[j], Dimer(monomers[i], monomers[j]), n_ct))
        labels.append(("CT", monomers[i].index, monomers[j].index))
        inst.append(ct_instance(monomers[j], monomers[i], Dimer(monomers[j], monomers[i]), n_ct))
        labels.append(("CT", monomers[j].index, monomers[i].index))
    return inst, labels


class _Instance(ct.Structure):
    _fields_ = [("n_atoms", ct.c_int), ("n_orb", ct.c_int), ("n_occ", ct.c_int), ("n_virt", ct.c_int),
                ("n_roots", ct.c_int), ("orbs_per_atom", ct.POINTER(ct.c_int)), ("c", ct.POINTER(ct.c_double)),
                ("s", ct.POINTER(ct.c_double)), ("orbe", ct.POINTER(ct.c_double)),
                ("gamma", ct.POINTER(ct.c_double)), ("gamma_lr", ct.POINTER(ct.c_double)),
                ("xyz", ct.POINTER(ct.c_double))]


class _Result(ct.Structure):
    _fields_ = [("energies", ct.POINTER(ct.c_double)), ("coefficients", ct.POINTER(ct.c_double)),
                ("osc", ct.POINTER(ct.c_double)), ("tr_dip", ct.POINTER(ct.c_double)),
                ("q_trans", ct.POINTER(ct.c_double)), ("iterations", ct.c_int), ("status", ct.c_int)]


# tincr_tda_instance / tincr_tda_result as numpy records (same layout as the C structs: five ints and
# padding to the pointer alignment, then seven pointers; five pointers, then two ints), so that a
# batch of hundreds of instances is marshalled with array operations
_INST_DT = np.dtype([("dims", np.int32, 5), ("pad", np.int32), ("ptr", np.uint64, 7)])
_RES_DT = np.dtype([("ptr", np.uint64, 5), ("iterations", np.int32), ("status", np.int32)])
assert _INST_DT.itemsize == ct.sizeof(_Instance) and _RES_DT.itemsize == ct.sizeof(_Result)


def _f64(a):
    return a if (a.dtype == np.float64 and a.flags.c_contiguous) else np.ascontiguousarray(a, dtype=np.float64)


_ADDR = {}   # id(array) -> (weak reference, data address): the lookup numpy makes costs microseconds


def _addr(a):
    if a is None:
        return 0
    hit = _ADDR.get(id(a))
    if hit is not None and hit[0]() is a:
        return hit[1]
    ptr = a.__array_interface__["data"][0]
    if len(_ADDR) > 65536:
        _ADDR.clear()
    _ADDR[id(a)] = (weakref.ref(a), ptr)
    return ptr


def solve_batch(ctx, instances, max_iter=50, tol=1e-4, precision=_lib.PREC_FP64):
    """Run `tincr_tda_solve_batch`; returns (status, list of result dicts)."""
    n = len(instances)
    keep = []
    arr = np.zeros(n, _INST_DT)
    for k, q in enumerate(instances):
        c, s_, orbe, gam, xyz = _f64(q["c"]), _f64(q["s"]), _f64(q["orbe"]), _f64(q["gamma"]), _f64(q["xyz"])
        glr = None if q["gamma_lr"] is None else _f64(q["gamma_lr"])
        opa = q["opa"] if (q["opa"].dtype == np.int32 and q["opa"].flags.c_contiguous) else \
            np.ascontiguousarray(q["opa"], dtype=np.int32)
        keep.append((c, s_, orbe, gam, xyz, glr, opa))
        arr[k] = ((q["n_atoms"], q["n_orb"], q["n_occ"], q["n_virt"], q["n_roots"]), 0,
                  (_addr(opa), _addr(c), _addr(s_), _addr(orbe), _addr(gam), _addr(glr), _addr(xyz)))
    dims = arr["dims"].astype(np.int64)
    nr, ov, na = dims[:, 4], dims[:, 2] * dims[:, 3], dims[:, 0]
    # one block per output kind, instance k at its offset
    sizes = np.stack([nr, ov * nr, nr, 3 * nr, na * nr])
    offs = np.concatenate([np.zeros((5, 1), np.int64), np.cumsum(sizes, axis=1)], axis=1)
    blocks = [np.zeros(int(offs[j, -1])) for j in range(5)]
    res = np.zeros(n, _RES_DT)
    for j in range(5):
        res["ptr"][:, j] = _addr(blocks[j]) + 8 * offs[j, :-1].astype(np.uint64)
    rc = ctx.lib.tincr_tda_solve_batch(ctx.h, n, arr.ctypes.data, int(max_iter), float(tol), int(precision),
                                       res.ctypes.data)
    ctx.check(rc, allow=(_lib.OK, _lib.NOT_CONVERGED))
    outs = []
    e, cf, osc, td, qt = blocks
    o0 = offs[:, :-1].tolist()
    o1 = offs[:, 1:].tolist()
    its, sts = res["iterations"].tolist(), res["status"].tolist()
    for k in range(n):
        r_, v_, a_ = int(nr[k]), int(ov[k]), int(na[k])
        outs.append(dict(energies=e[o0[0][k]:o1[0][k]], coefficients=cf[o0[1][k]:o1[1][k]].reshape(v_, r_),
                         osc=osc[o0[2][k]:o1[2][k]], tr_dip=td[o0[3][k]:o1[3][k]].reshape(3, r_),
                         q_trans=qt[o0[4][k]:o1[4][k]].reshape(a_, r_), iterations=its[k], status=sts[k]))
    return rc, outs


def instance_cost(q):
    """Estimated work of one instance: n_roots o v (o + v), the exchange contraction of tincr's
    product per trial vector (the quantity the work list is balanced on)."""
    o, v = int(q["n_occ"]), int(q["n_virt"])
    return int(q["n_roots"]) * o * v * (o + v)


def shard_instances(instances, world, rank):
    """Indices (ascending) of the instances rank `rank` of `world` solves: longest-processing-time
    assignment by `instance_cost` (the most expensive instance first to the least loaded rank, ties
    to the lower rank), the same on every rank without communication."""
    if world <= 1:
        return list(range(len(instances)))
    load = [0] * world
    owner = [0] * len(instances)
    for k in sorted(range(len(instances)), key=lambda k: (-instance_cost(instances[k]), k)):
        r = min(range(world), key=lambda x: (load[x], x))
        owner[k] = r
        load[r] += instance_cost(instances[k])
    return [k for k in range(len(instances)) if owner[k] == rank]


# order in which statuses of different ranks are folded into one (later = worse)
_SEVERITY = {_lib.OK: 0, _lib.NOT_CONVERGED: 1, _lib.CG_MAXITER: 2, _lib.NONFINITE: 3, _lib.BAD_ARG: 4,
             _lib.CUDA_ERR: 5, _lib.NO_DEVICE: 6}


def worst_status(codes):
    """The most severe of several status codes (unknown codes rank above every known one)."""
    worst = _lib.OK
    for c in codes:
        if _SEVERITY.get(c, 99) > _SEVERITY.get(worst, 99):
            worst = c
    return worst


def solve_batch_sharded(ctx, instances, world, rank, allgather=None, solver=None, **kw):
    """The FMO work list split over `world` ranks (one GPU each): every rank solves its shard with
    `solve_batch` (or `solver`), then one all-gather of the per-instance results (energies,
    coefficients, transition charges, dipoles, oscillator strengths) gives every rank the whole
    list, in the caller's order, as the exciton Hamiltonian needs it.

    `allgather(obj) -> list of every rank's obj, in rank order` is the caller's collective (for
    instance torch.distributed.all_gather_object over gloo: the results are host arrays); it is
    required when world > 1, so this module needs no communication library of its own.

    Every rank takes part in the all-gather even when its own solve failed: a rank whose solver
    raised sends its status and message instead of results, and after the collective every rank
    raises the same error (a TincrError with the most severe status of the failed ranks, or a
    RuntimeError when a rank failed outside the library).  No rank is left waiting in the
    collective for one that raised.  Returns (worst status over all ranks, list of result dicts)."""
    solver = solver or solve_batch
    mine = shard_instances(instances, world, rank)
    failure = None
    try:
        rc, out = solver(ctx, [instances[k] for k in mine], **kw) if mine else (_lib.OK, [])
    except _lib.TincrError as e:
        if world <= 1:
            raise
        rc, out, failure = e.status, None, (e.status, "rank %d: %s" % (rank, e))
    except Exception as e:   # noqa: BLE001 - reported to every rank below, then raised there
        if world <= 1:
            raise
        rc, out, failure = None, None, (None, "rank %d: %s: %s" % (rank, type(e).__name__, e))
    if world <= 1:
        return rc, out
    if allgather is None:
        raise ValueError("solve_batch_sharded: world > 1 needs an allgather collective")
    parts = allgather((mine, rc, out, failure))
    failures = [p[3] for p in parts if p[3] is not None]
    if failures:
        msg = "; ".join(m for _, m in failures)
        codes = [s for s, _ in failures if s is not None]
        if len(codes) == len(failures):
            raise _lib.TincrError(worst_status(codes), msg)
        raise RuntimeError("sharded FMO solve failed: " + msg)
    full = [None] * len(instances)
    for idx, _, out_r, _ in parts:
        for k, o in zip(idx, out_r):
            full[k] = o
    return worst_status(p[1] for p in parts), full


def run_gradient_jobs(jobs, n_streams=8, contexts=None, variant="reference"):
    """Excitation-energy gradients of independent systems on the GPU.  jobs: list of (system, ground
    state, energies [k], coefficients [o*v, k], state, precision): the roots of each system are
    installed with `tincr_tda_set_states` (tincr's `set_ci_eigenvalues` / `set_ci_coefficients`) and
    `tincr_gradient` gives the gradient of root `state`.  The jobs are spread over `n_streams`
    contexts (or `contexts`), each driven by its own host thread, which take the next job from a
    shared list ordered by system size, largest first, so that their kernels overlap on the device
    and the longest jobs start first.  Returns a list of [3 N] arrays in job order."""
    import threading
    from concurrent.futures import ThreadPoolExecutor
    from . import gradients as GR
    from . import tda as T
    out = [None] * len(jobs)
    if not jobs:
        return out
    own = contexts is None
    ctxs = contexts if not own else [_lib.Context(0) for _ in range(min(n_streams, len(jobs)))]
    lanes = min(len(ctxs), len(jobs))
    order = sorted(range(len(jobs)), key=lambda k: -jobs[k][0].n_orbs)
    lock = threading.Lock()
    nxt = [0]

    def work(lane):
        c = ctxs[lane]
        while True:
            with lock:
                if nxt[0] >= len(order):
                    return
                k = order[nxt[0]]
                nxt[0] += 1
            sy, g, e, x, state, prec = jobs[k]
            es = T.ExcitedStateSystem.from_ground_state(c, sy, g)
            es.prepare_tda()
            es.set_states(np.atleast_1d(np.asarray(e, dtype=np.float64)), np.asarray(x, dtype=np.float64))
            es.set_precision(prec)
            out[k] = GR.GradientSystem(es, sy, g).tda_gradient(int(state), variant)

    try:
        with ThreadPoolExecutor(max_workers=lanes) as ex:
            for f in [ex.submit(work, lane) for lane in range(lanes)]:
                f.result()
    finally:
        if own:
            for c in ctxs:
                c.close()
    return out


def le_gradients(monomers, results, states, n_streams=8, variant="reference", contexts=None,
                 precision=_lib.PREC_FP64):
    """Excitation-energy gradients of locally excited states, the LE terms of tincr's FMO exciton
    gradient (`SuperSystem::fmo_cis_gradient`, src/fmo/lcmo/cis_gradient.rs:118-126, which adds
    c^2 * `Monomer::tda_gradient_lc(n)` per contributing LE state; src/fmo/gradients/excited_state.rs:
    299-542).  For monomer k the gradient of root states[k] of results[k] (its batch TDA result) is
    computed on the GPU (`run_gradient_jobs`: the monomers spread over `n_streams` contexts, each
    driven by its own host thread, as tincr runs the monomers on rayon threads).

    `precision` is the precision the results were solved with; the gradients' contractions follow it.
    Entries of `states` that are None are skipped.  Returns a list of [3 N_k] arrays (Hartree/bohr,
    atom order of the monomer) or None."""
    ks = [k for k in range(len(monomers)) if states[k] is not None]
    jobs = [(monomers[k].system, monomers[k].ground, results[k]["energies"], results[k]["coefficients"],
             int(states[k]), precision) for k in ks]
    got = run_gradient_jobs(jobs, n_streams=n_streams, contexts=contexts, variant=variant)
    out = [None] * len(monomers)
    for k, g in zip(ks, got):
        out[k] = g
    return out


def exciton_le_gradient(monomers, results, vector, n_le, threshold=0.05, n_ct_states=0, **kw):
    """The LE terms of tincr's exciton-state gradient (`SuperSystem::fmo_cis_gradient`,
    src/fmo/lcmo/cis_gradient.rs:10-166): for every LE basis state with |c| > threshold in the
    exciton eigenvector `vector` (basis order: n_le LE states per monomer first), c^2 times that LE
    state's excitation gradient, added on the monomer's atoms.  The CT basis states' terms
    (`ct_gradient_new`, cis_gradient.rs:127-163) are not part of this function; their number above
    the threshold is returned so that a caller can report it.

    `results` are the batch TDA results of the monomers (LE instances, monomer order); the keyword
    arguments go to `le_gradients`.  Returns (gradient [3 N_total] in the aggregate's atom order,
    number of LE terms, number of CT terms above the threshold)."""
    n_mon = len(monomers)
    terms = []
    for b, c in enumerate(np.asarray(vector)):
        if abs(c) > threshold and b < n_mon * n_le:
            terms.append((b // n_le, b % n_le, float(c) ** 2))
    n_ct = int(np.sum(np.abs(np.asarray(vector)[n_mon * n_le:n_mon * n_le + n_ct_states]) > threshold))
    offs = np.concatenate([[0], np.cumsum([m.system.n_atoms for m in monomers])])
    grad = np.zeros(3 * int(offs[-1]))
    pending = list(terms)
    while pending:   # one state per monomer per round
        seen, batch, rest = set(), [], []
        for t in pending:
            (rest if t[0] in seen else batch).append(t)
            seen.add(t[0])
        pending = rest
        states = [None] * n_mon
        for k, r, _ in batch:
            states[k] = r
        g = le_gradients(monomers, results[:n_mon], states, **kw)
        for k, r, w in batch:
            grad[3 * offs[k]:3 * offs[k + 1]] += w * g[k]
    return grad, len(terms), n_ct


# ----------------------------------------------------------------------------------------------
# exciton Hamiltonian inputs (upstream of the couplings: pair types, overlaps, gamma, pair SCC)
# ----------------------------------------------------------------------------------------------

# Sums of van der Waals radii in bohr for H, C, N, O: tincr's VDW_SUM table (UFF radii,
# src/constants.rs:1389)
VDW_SUM_BOHR = {(1, 1): 5.454, (1, 6): 6.366, (1, 7): 6.185, (1, 8): 6.128, (6, 6): 7.279, (6, 7): 7.098,
                (6, 8): 7.041, (7, 7): 6.916, (7, 8): 6.860, (8, 8): 6.803}


def is_real_pair(ma, mb, vdw_scaling=2.0):
    """tincr's `get_pair_type` (src/fmo/pair.rs:35-53): a real pair when some atom pair is closer than
    vdw_scaling times the sum of its van der Waals radii, otherwise an ESD pair."""
    za, zb = ma.system.numbers, mb.system.numbers
    lim = np.array([[VDW_SUM_BOHR[(min(int(x), int(y)), max(int(x), int(y)))] for y in zb] for x in za])
    d = np.linalg.norm(ma.system.xyz[:, None, :] - mb.system.xyz[None, :, :], axis=-1)
    return bool(np.any(d < vdw_scaling * lim))


def _dimer_scc(args):
    """Host SCC of one dimer (top-level for a spawn process pool): returns (orbs, orbe).  It starts
    from the block-diagonal density of the two converged monomers, as tincr starts a pair SCC from
    its monomers' charges (src/fmo/scc/pair.rs:112-124), and raises if it does not converge (tincr
    panics, pair.rs:234-240): from the neutral-atom density a few dimers of a dense aggregate stall
    past the iteration limit, and an unconverged dimer would hand machine-dependent orbitals to the
    LCMO Fock matrix."""
    z, xyz, lc, r_lr, tol, p_start, isolated = args
    sy = gs.build_system(z, xyz, lc=lc, r_lr=r_lr)
    g = gs.run_scc(sy, tol=tol, p_start=p_start)
    if not g.converged:
        # some dimers of the benchmark lattices overlap (H-H contacts under 0.5 A) and their DIIS swaps
        # occupations; a level shift of the virtual space settles some of them on a stationary density
        g = gs.run_scc(sy, tol=tol, p_start=p_start, level_shift=0.5, max_iter=1000,
                       require_convergence=isolated is None)
    if not g.converged:
        # the caller's policy for a dimer without a stationary ground state: the isolated monomers'
        # orbitals (block diagonal) and energies as its pair ground state
        (ca, ea), (cb, eb) = isolated
        orbs = np.zeros((len(ea) + len(eb), len(ea) + len(eb)))
        orbs[:len(ea), :len(ea)] = ca
        orbs[len(ea):, len(ea):] = cb
        return orbs, np.concatenate([ea, eb]), False
    return g.orbs, g.orbe, True


def _dimer_scc_gpu(ctx, jobs):
    """The dimer SCCs of `jobs` (the arguments of `_dimer_scc`) as batched GPU SCCs: DIIS from the
    monomers' densities, then the dimers that missed the tolerance again with a level shift of 0.5 and
    up to 1000 iterations, then the caller's policy for the rest (the isolated monomers' orbitals, or
    an error).  Returns (orbs, orbe, converged) per job."""
    from . import scc as gscc
    systems = [gs.build_system(z, xyz, lc=lc, r_lr=r_lr) for z, xyz, lc, r_lr, _, _, _ in jobs]
    tol = jobs[0][4]
    grounds, _ = gscc.scc_batch(ctx, systems, tol=tol, p_start=[j[5] for j in jobs], full=False)
    retry = [k for k, g in enumerate(grounds) if not g.converged]
    if retry:
        again, _ = gscc.scc_batch(ctx, [systems[k] for k in retry], tol=tol, max_iter=1000, level_shift=0.5,
                                  p_start=[jobs[k][5] for k in retry], full=False)
        for k, g in zip(retry, again):
            grounds[k] = g
    out = []
    for (z, xyz, lc, r_lr, _, _, isolated), g in zip(jobs, grounds):
        if g.converged:
            out.append((g.orbs, g.orbe, True))
        elif isolated is None:
            raise RuntimeError("dimer SCC not converged to %g with a level shift either" % tol)
        else:
            (ca, ea), (cb, eb) = isolated
            orbs = np.zeros((len(ea) + len(eb), len(ea) + len(eb)))
            orbs[:len(ea), :len(ea)] = ca
            orbs[len(ea):, len(ea):] = cb
            out.append((orbs, np.concatenate([ea, eb]), False))
    return out


class ExcitonSetup:
    """Everything the exciton Hamiltonian reads besides the LE / CT roots, produced on the host
    (tincr's SuperSystem holds the same: src/fmo/supersystem.rs:248-305, src/fmo/pair.rs):

    * pair types of every monomer pair (real pair / ESD, `is_real_pair`);
    * the AO overlap blocks S_IJ between the monomers of every real pair and of every CT pair;
    * the atomwise gamma and gamma_lr of the whole aggregate;
    * the ground state (MO coefficients, energies) of every real pair's dimer, for the LCMO Fock
      matrix (tincr's FMO pair SCC; here the isolated dimer, like the monomers).
    `workers` > 1 runs the dimer SCCs in a spawn process pool; scc="gpu" runs them as one batched
    GPU SCC on `ctx` (tincr_scc_batch), with the same starts, retry and policy.  A dimer SCC that does
    not converge, neither by DIIS from the monomers' densities nor with a level shift, raises (tincr
    panics) unless `unconverged="isolated"`, which gives such a dimer the isolated monomers' orbitals
    and energies as its pair ground state; `unconverged_pairs` lists those dimers."""

    def __init__(self, monomers, ct_pairs, lc=True, scc_tol=1e-10, workers=1, unconverged="raise", scc="host",
                 ctx=None):
        self.monomers = monomers
        self.ct_pairs = list(ct_pairs)
        n = len(monomers)
        self.real = {(i, j): False for i in range(n) for j in range(i + 1, n)}
        reach = 2.0 * max(VDW_SUM_BOHR.values())   # no atom pair farther apart than this is a real pair
        for i, j in candidate_pairs(monomers, reach):
            self.real[(i, j)] = is_real_pair(monomers[i], monomers[j])
        sy0 = monomers[0].system
        self.lc, self.r_lr = lc, sy0.r_lr
        z = np.concatenate([m.system.numbers for m in monomers])
        xyz = np.concatenate([m.system.xyz for m in monomers])
        self.atom_offset = np.concatenate([[0], np.cumsum([m.system.n_atoms for m in monomers])]).astype(np.int64)
        big = gs.build_system(z, xyz, lc=lc, r_lr=self.r_lr)
        self.gamma = gs.gamma_atomwise(big, 0.0)
        self.gamma_lr = gs.gamma_atomwise(big, self.r_lr) if lc else np.zeros_like(self.gamma)
        need = sorted(set(k for k, v in self.real.items() if v) | set(tuple(sorted(p)) for p in self.ct_pairs))
        self.s_blocks = {}
        for i, j in need:
            mi, mj = monomers[i], monomers[j]
            sy = gs.build_system(np.concatenate([mi.system.numbers, mj.system.numbers]),
                                 np.concatenate([mi.system.xyz, mj.system.xyz]), lc=lc, r_lr=self.r_lr)
            s, _ = gs.h0_and_s(sy)
            ni = mi.system.n_orbs
            self.s_blocks[(i, j)] = np.ascontiguousarray(s[:ni, ni:])
        jobs = []
        self.real_pairs = sorted(k for k, v in self.real.items() if v)
        for i, j in self.real_pairs:
            mi, mj = monomers[i], monomers[j]
            ni, nj = mi.system.n_orbs, mj.system.n_orbs
            p_start = np.zeros((ni + nj, ni + nj))
            p_start[:ni, :ni] = mi.ground.p
            p_start[ni:, ni:] = mj.ground.p
            iso = ((mi.ground.orbs, mi.ground.orbe), (mj.ground.orbs, mj.ground.orbe)) \
                if unconverged == "isolated" else None
            jobs.append((np.concatenate([mi.system.numbers, mj.system.numbers]),
                         np.concatenate([mi.system.xyz, mj.system.xyz]), lc, self.r_lr, scc_tol, p_start, iso))
        if scc == "gpu":
            out = _dimer_scc_gpu(ctx, jobs)
        elif scc == "host":
            out = _pool_map(_dimer_scc, jobs, workers)
        else:
            raise ValueError("scc must be 'host' or 'gpu'")
        self.pair_scc = {k: (o[0], o[1]) for k, o in zip(self.real_pairs, out)}
        self.unconverged_pairs = [k for k, o in zip(self.real_pairs, out) if not o[2]]

    def s_block(self, i, j):
        """AO overlap between monomers i and j (rows i).  Pairs without a stored block are ESD pairs
        whose atoms are all farther apart than the Slater-Koster grid reaches: their overlap is zero."""
        key = (min(i, j), max(i, j))
        if key not in self.s_blocks:
            mi, mj = self.monomers[i], self.monomers[j]
            d = np.linalg.norm(mi.system.xyz[:, None, :] - mj.system.xyz[None, :, :], axis=-1).min()
            if d <= float(np.max(mi.system.params.sk_knots)):
                raise KeyError("overlap of pair %s not computed" % (key,))
            return np.zeros((mi.system.n_orbs, mj.system.n_orbs))
        if i < j:
            return self.s_blocks[(i, j)]
        return self.s_blocks[(j, i)].T


class _ExMonomer(ct.Structure):
    _fields_ = [("n_atoms", ct.c_int), ("n_orb", ct.c_int), ("n_occ", ct.c_int),
                ("orbs_per_atom", ct.POINTER(ct.c_int)), ("c", ct.POINTER(ct.c_double)), ("s", ct.POINTER(ct.c_double)),
                ("orbe", ct.POINTER(ct.c_double)), ("n_le", ct.c_int), ("le_energies", ct.POINTER(ct.c_double)),
                ("le_coefficients", ct.POINTER(ct.c_double)), ("le_q_trans", ct.POINTER(ct.c_double))]


class _ExPair(ct.Structure):
    _fields_ = [("i", ct.c_int), ("j", ct.c_int), ("real", ct.c_int), ("s_ij", ct.POINTER(ct.c_double)),
                ("pair_orbs", ct.POINTER(ct.c_double)), ("pair_orbe", ct.POINTER(ct.c_double))]


class _ExCT(ct.Structure):
    _fields_ = [("h", ct.c_int), ("l", ct.c_int), ("state", ct.c_int), ("n_ct", ct.c_int),
                ("energies", ct.POINTER(ct.c_double)), ("coefficients", ct.POINTER(ct.c_double)),
                ("q_tr", ct.POINTER(ct.c_double))]


def _dp(a):
    return None if a is None else a.ctypes.data_as(ct.POINTER(ct.c_double))


def exciton_states(ctx, setup, results, labels, n_le, n_ct, n_roots=10, tol=1e-4, max_iter=100,
                   precision=_lib.PREC_FP64, want_matrix=False):
    """tincr's exciton Hamiltonian and its lowest roots on the GPU (`tincr_exciton_states`;
    SuperSystem::create_exciton_hamiltonian_new, src/fmo/lcmo/basis.rs:449-503).

    `results` / `labels`: the batch TDA results of the work list of `aggregate_instances` (LE
    instances of every monomer, then both directions of every CT pair of `setup.ct_pairs`).  The basis
    is n_le LE roots per monomer, then for every CT pair and root n < n_ct the states I -> J and
    J -> I (basis.rs:180-238).  Returns dict(energies [n_roots], vectors [dim, n_roots], iterations,
    status, matrix [dim, dim] when want_matrix)."""
    mons = setup.monomers
    keep = []
    le_of = {}
    ct_of = {}
    for k, lab in enumerate(labels):
        if lab[0] == "LE":
            le_of[lab[1]] = results[k]
        else:
            ct_of[(lab[1], lab[2])] = results[k]
    marr = (_ExMonomer * len(mons))()
    for k, m in enumerate(mons):
        sy, g = m.system, m.ground
        r = le_of[m.index]
        opa = np.ascontiguousarray(sy.orbs_per_atom, dtype=np.int32)
        e = _f64(np.asarray(r["energies"])[:n_le])
        cf = _f64(np.asarray(r["coefficients"])[:, :n_le])
        qt = _f64(np.asarray(r["q_trans"])[:, :n_le])
        c, s, orbe = _f64(g.orbs), _f64(g.s), _f64(g.orbe)
        keep += [opa, e, cf, qt, c, s, orbe]
        marr[k] = _ExMonomer(sy.n_atoms, sy.n_orbs, sy.n_occ, opa.ctypes.data_as(ct.POINTER(ct.c_int)), _dp(c),
                             _dp(s), _dp(orbe), n_le, _dp(e), _dp(cf), _dp(qt))
    plist = sorted(set(setup.real_pairs) | set(tuple(sorted(p)) for p in setup.ct_pairs))
    parr = (_ExPair * max(1, len(plist)))()
    for k, (i, j) in enumerate(plist):
        sij = _f64(setup.s_block(i, j))
        real = bool(setup.real.get((i, j), False))
        po, pe = (setup.pair_scc[(i, j)] if real else (None, None))
        po = None if po is None else _f64(po)
        pe = None if pe is None else _f64(pe)
        keep += [sij, po, pe]
        parr[k] = _ExPair(i, j, int(real), _dp(sij), _dp(po), _dp(pe))
    states = []
    for i, j in setup.ct_pairs:
        for n in range(n_ct):
            for h, l in ((i, j), (j, i)):
                states.append((h, l, n))
    carr = (_ExCT * max(1, len(states)))()
    for k, (h, l, n) in enumerate(states):
        r = ct_of[(h, l)]
        e, cf, qt = _f64(np.asarray(r["energies"])), _f64(np.asarray(r["coefficients"])), _f64(np.asarray(r["q_trans"]))
        keep += [e, cf, qt]
        carr[k] = _ExCT(h, l, n, len(e), _dp(e), _dp(cf), _dp(qt))
    dim = sum(n_le for _ in mons) + len(states)
    energies = np.zeros(n_roots)
    vectors = np.zeros((dim, n_roots))
    mat = np.zeros((dim, dim)) if want_matrix else None
    its = ct.c_int(0)
    g, glr = _f64(setup.gamma), _f64(setup.gamma_lr)
    rc = ctx.lib.tincr_exciton_states(ctx.h, len(mons), ct.addressof(marr), len(plist), ct.addressof(parr),
                                      len(states), ct.addressof(carr), g.shape[0], _dp(g), _dp(glr), int(precision),
                                      int(n_roots), float(tol), int(max_iter), _dp(mat), _dp(energies), _dp(vectors),
                                      ct.byref(its))
    ctx.check(rc, allow=(_lib.OK, _lib.NOT_CONVERGED))
    out = dict(energies=energies, vectors=vectors, iterations=its.value, status=rc)
    if want_matrix:
        out["matrix"] = mat
    return out


# ----------------------------------------------------------------------------------------------
# CT-state gradients and the exciton-state gradient
# ----------------------------------------------------------------------------------------------

def pair_ground_states(ctx, monomers, pairs, scc_tol=1e-10):
    """Full SCC ground states (orbitals, density, S, gammas, converged Fock matrix) of the dimers of
    `pairs` ((i, j) with monomer i's atoms first), which the CT-state gradients differentiate: one
    batched GPU SCC (`tincr_scc_batch`) from the block-diagonal density of the two monomers, then the
    dimers that missed the tolerance again with a level shift of 0.5 and up to 1000 iterations (the
    starts and retry of the exciton set-up's dimer SCCs).  tincr takes a real pair's SCC from its FMO
    pair SCC (src/fmo/scc/pair.rs) and runs the SCC of an ESD pair for its CT gradient
    (`new_charge_transfer_pair_gradient`, src/fmo/gradients/ct_state_new.rs:56-58).  Returns
    {(i, j): (System, GroundState)}; a dimer without a converged ground state raises (tincr panics,
    pair.rs:234-240)."""
    from . import scc as gscc
    pairs = list(dict.fromkeys((int(i), int(j)) for i, j in pairs))
    if not pairs:
        return {}
    systems, starts = [], []
    for i, j in pairs:
        mi, mj = monomers[i], monomers[j]
        systems.append(gs.build_system(np.concatenate([mi.system.numbers, mj.system.numbers]),
                                       np.concatenate([mi.system.xyz, mj.system.xyz]), lc=mi.system.lc,
                                       r_lr=mi.system.r_lr))
        ni, nj = mi.system.n_orbs, mj.system.n_orbs
        p = np.zeros((ni + nj, ni + nj))
        p[:ni, :ni] = mi.ground.p
        p[ni:, ni:] = mj.ground.p
        starts.append(p)
    grounds, _ = gscc.scc_batch(ctx, systems, tol=scc_tol, p_start=starts)
    retry = [k for k, g in enumerate(grounds) if not g.converged]
    if retry:
        again, _ = gscc.scc_batch(ctx, [systems[k] for k in retry], tol=scc_tol, max_iter=1000, level_shift=0.5,
                                  p_start=[starts[k] for k in retry])
        for k, g in zip(retry, again):
            grounds[k] = g
    bad = [pairs[k] for k, g in enumerate(grounds) if not g.converged]
    if bad:
        raise RuntimeError("dimer SCC not converged to %g for the CT gradient of pairs %s" % (scc_tol, bad[:10]))
    return {key: (sy, g) for key, sy, g in zip(pairs, systems, grounds)}


def ct_amplitudes_in_pair(mi, mj, sy, g, x_ct, hole_i):
    """The CT amplitudes x_ct [n_occ(hole), n_virt(electron)], given over the hole monomer's occupied
    and the electron monomer's virtual orbitals, in the orbitals of the dimer (monomer mi's atoms
    first; hole on mi when hole_i): X_IJ = S_h,IJ[occ_h, occ_IJ]^T x_ct S_l,IJ[virt_l, virt_IJ] with
    S_I,IJ = C_I^T S[I rows, :] C_IJ (`Pair::prepare_charge_transfer_gradient`,
    src/fmo/gradients/ct_state_new.rs:115-150; overlaps of src/fmo/lcmo/hamiltonian.rs:61-64).
    Returns X_IJ [n_occ(IJ), n_virt(IJ)]."""
    ni = mi.system.n_orbs
    no = sy.n_occ
    s_h = mi if hole_i else mj
    s_l = mj if hole_i else mi
    rows_h = slice(0, ni) if hole_i else slice(ni, None)
    rows_l = slice(ni, None) if hole_i else slice(0, ni)
    oh, ol = s_h.system.n_occ, s_l.system.n_occ
    x_ct = np.asarray(x_ct, dtype=np.float64)
    if x_ct.size != oh * s_l.system.n_virt:
        raise ValueError("ct_amplitudes_in_pair: %d amplitudes for %d occupied x %d virtual orbitals"
                         % (x_ct.size, oh, s_l.system.n_virt))
    x_ct = x_ct.reshape(oh, -1)
    occ_h = s_h.ground.orbs[:, :oh].T @ g.s[rows_h, :] @ g.orbs[:, :no]         # [oh, no]
    virt_l = s_l.ground.orbs[:, ol:].T @ g.s[rows_l, :] @ g.orbs[:, no:]        # [vl, nv]
    return occ_h.T @ (x_ct @ virt_l)


def _ct_jobs(monomers, terms, states, precision):
    """Gradient jobs (`run_gradient_jobs`) of CT terms (hole, electron, x_ct, energy): the dimer
    (lower monomer index first), its ground state from `states`, the CT energy and the amplitudes in
    the dimer's orbitals as its one root."""
    jobs = []
    for h, l, x_ct, energy in terms:
        i, j = min(int(h), int(l)), max(int(h), int(l))
        sy, g = states[(i, j)]
        x = ct_amplitudes_in_pair(monomers[i], monomers[j], sy, g, x_ct, int(h) == i)
        jobs.append((sy, g, np.array([float(energy)]), x.reshape(-1, 1), 0, precision))
    return jobs


def ct_state_gradients(ctx, monomers, terms, pair_states=None, n_streams=8, contexts=None, variant="reference",
                       precision=_lib.PREC_FP64, scc_tol=1e-10):
    """Excitation-energy gradients of charge-transfer states, each the TDA gradient of its dimer at
    one state (tincr's `new_charge_transfer_pair_gradient`, src/fmo/gradients/ct_state_new.rs:13-70,
    and `ct_gradient_new`, src/fmo/lcmo/ct_gradient.rs:116-172: `Pair::tda_gradient_lc(0)`,
    src/fmo/gradients/excited_state.rs:1470-1713, with ci_eigenvalues = [E_CT] and the CT amplitudes
    in the dimer's orbitals as ci_coefficients).

    terms: list of (hole, electron, x_ct, energy): monomer indices, amplitudes
    [n_occ(hole), n_virt(electron)] and the CT energy.  The dimer of a term is the pair
    (min, max) of its monomers, lower index first; its ground state comes from `pair_states` (as
    `pair_ground_states` returns) or from one batched GPU SCC of all dimers needed.  The gradients
    run on the GPU (`run_gradient_jobs`); `precision` is the precision the amplitudes were solved
    with.  Returns (list of gradients [3 (N_I + N_J)] in the dimer's atom order, pair_states)."""
    if any(int(h) == int(l) for h, l, _, _ in terms):
        raise ValueError("ct_state_gradients: a CT term needs two different monomers")
    keys = [(min(int(h), int(l)), max(int(h), int(l))) for h, l, _, _ in terms]
    need = [k for k in dict.fromkeys(keys) if pair_states is None or k not in pair_states]
    states = dict(pair_states or {})
    if need:
        states.update(pair_ground_states(ctx, monomers, need, scc_tol))
    jobs = _ct_jobs(monomers, terms, states, precision)
    return run_gradient_jobs(jobs, n_streams=n_streams, contexts=contexts, variant=variant), states


def ct_unit_amplitudes(monomers, hole, electron, ct_ind_h, ct_ind_l):
    """Amplitudes of the single orbital pair HOMO - ct_ind_h (hole monomer) -> LUMO + ct_ind_l
    (electron monomer), tincr's CT basis states of `create_diab_basis` (src/fmo/lcmo/basis.rs:24-141)
    as `Pair::prepare_ct_state` writes them (src/fmo/gradients/excited_state.rs:1176-1179)."""
    oh, vl = monomers[hole].system.n_occ, monomers[electron].system.n_virt
    if not (0 <= int(ct_ind_h) < oh and 0 <= int(ct_ind_l) < vl):
        raise ValueError("ct_unit_amplitudes: orbital offsets (%d, %d) outside %d occupied / %d virtual orbitals"
                         % (int(ct_ind_h), int(ct_ind_l), oh, vl))
    x = np.zeros((oh, vl))
    x[oh - 1 - int(ct_ind_h), int(ct_ind_l)] = 1.0
    return x


def ct_gradient(ctx, monomers, index_i, index_j, ct_ind_i, ct_ind_j, ct_energy, hole_i, **kw):
    """tincr's `SuperSystem::ct_gradient_new(index_i, index_j, ct_ind_i, ct_ind_j, ct_energy, hole_i)`
    (src/fmo/lcmo/ct_gradient.rs:116-172) for index_i < index_j: the gradient [3 (N_i + N_j)]
    (monomer index_i's atoms first) of the single-orbital CT state hole -> electron, the hole on
    index_i when hole_i (orbital HOMO - ct_ind_i of index_i -> LUMO + ct_ind_j of index_j), else on
    index_j (HOMO - ct_ind_j of index_j -> LUMO + ct_ind_i of index_i), with excitation energy
    ct_energy.  For an ESD pair tincr's routine takes the non-LC gradient (`tda_gradient_nolc`, :169)
    with the pair's SCC call commented out (:164-165); here every pair has its dimer SCC and the
    gradient follows the LC setting, as `new_charge_transfer_pair_gradient` does for both pair types.
    Keyword arguments go to `ct_state_gradients`."""
    if not index_i < index_j:
        raise ValueError("ct_gradient: index_i < index_j (tincr's argument order)")
    if hole_i:
        term = (index_i, index_j, ct_unit_amplitudes(monomers, index_i, index_j, ct_ind_i, ct_ind_j), ct_energy)
    else:
        term = (index_j, index_i, ct_unit_amplitudes(monomers, index_j, index_i, ct_ind_j, ct_ind_i), ct_energy)
    grads, _ = ct_state_gradients(ctx, monomers, [term], **kw)
    return grads[0]


def exciton_basis(labels, results, n_mon, n_le, n_ct, ct_pairs):
    """The diabatic basis of `exciton_states` as a list: ("LE", monomer, root) for the n_le roots of
    every monomer, then for every CT pair (i, j) and root n < n_ct the states ("CT", i, j, n) and
    ("CT", j, i, n) (hole, electron, root; src/fmo/lcmo/basis.rs:180-238).  Returns the list and a
    dict (hole, electron) -> batch TDA result of that CT direction."""
    ct_of = {}
    for k, lab in enumerate(labels):
        if lab[0] == "CT":
            ct_of[(lab[1], lab[2])] = results[k]
    basis = [("LE", m, r) for m in range(n_mon) for r in range(n_le)]
    for i, j in ct_pairs:
        for n in range(n_ct):
            basis.append(("CT", i, j, n))
            basis.append(("CT", j, i, n))
    return basis, ct_of


def exciton_gradient(ctx, setup, results, labels, n_le, n_ct, vector, threshold=0.05, contexts=None,
                     precision=_lib.PREC_FP64, variant="reference", scc_tol=1e-10, pair_states=None):
    """Gradient of an exciton state's excitation energy, tincr's `SuperSystem::fmo_cis_gradient`
    (src/fmo/lcmo/cis_gradient.rs:10-166) over the basis of `exciton_states`: for every basis state
    whose coefficient in `vector` exceeds `threshold` in magnitude, c^2 times that state's gradient,
    added on its atoms.  An LE state contributes its monomer's TDA gradient at that root
    (cis_gradient.rs:118-126), a CT state the gradient of its dimer at that state (the pair-TDA CT
    state with its amplitudes and energy, as `new_charge_transfer_pair_gradient` takes them; the
    dimers' ground states from `pair_states` or one batched GPU SCC).  All terms form one job list
    for `run_gradient_jobs`.  tincr's routine expands the state in the single-orbital CT basis of
    `create_diab_basis` and reads the eigenvectors from properties that neither exciton Hamiltonian
    stores (basis.rs:445-446), so it cannot run as written; this one uses the basis the energies come
    from.  No CPHF term is added, as in `fmo_cis_gradient` (tincr adds `calculate_cphf_correction` in
    its Ehrenfest gradient, src/dynamics/helpers.rs:248, and its numerical CT test,
    src/fmo/gradients/numerical.rs:120).

    Returns (gradient [3 N_total] in the aggregate's atom order, number of LE terms, number of CT
    terms, pair_states)."""
    mons = setup.monomers
    n_mon = len(mons)
    vector = np.asarray(vector, dtype=np.float64)
    basis, ct_of = exciton_basis(labels, results, n_mon, n_le, n_ct, setup.ct_pairs)
    if len(basis) != len(vector):
        raise ValueError("exciton_gradient: vector of %d entries for a basis of %d states" % (len(vector), len(basis)))
    le_of = {lab[1]: results[k] for k, lab in enumerate(labels) if lab[0] == "LE"}
    le_terms, ct_terms, ct_w = [], [], []
    for b, c in enumerate(vector):
        if abs(c) <= threshold:
            continue
        st = basis[b]
        if st[0] == "LE":
            le_terms.append((st[1], st[2], float(c) ** 2))
        else:
            _, h, l, n = st
            r = ct_of[(h, l)]
            x = np.asarray(r["coefficients"])[:, n].reshape(mons[h].system.n_occ, -1)
            ct_terms.append((h, l, x, float(np.asarray(r["energies"])[n])))
            ct_w.append(float(c) ** 2)
    keys = [(min(h, l), max(h, l)) for h, l, _, _ in ct_terms]
    need = [k for k in dict.fromkeys(keys) if pair_states is None or k not in pair_states]
    pair_states = dict(pair_states or {})
    if need:
        pair_states.update(pair_ground_states(ctx, mons, need, scc_tol))
    # every term, LE and CT, in one job list over the same contexts
    jobs = [(mons[m].system, mons[m].ground, le_of[mons[m].index]["energies"], le_of[mons[m].index]["coefficients"],
             r, precision) for m, r, _ in le_terms]
    jobs += _ct_jobs(mons, ct_terms, pair_states, precision)
    grads = run_gradient_jobs(jobs, contexts=contexts, variant=variant)
    offs = np.concatenate([[0], np.cumsum([m.system.n_atoms for m in mons])])
    grad = np.zeros(3 * int(offs[-1]))
    for (m, _, w), gle in zip(le_terms, grads):
        grad[3 * offs[m]:3 * offs[m + 1]] += w * gle
    for (h, l, _, _), w, gct in zip(ct_terms, ct_w, grads[len(le_terms):]):
        i, j = min(h, l), max(h, l)
        ni = 3 * int(offs[i + 1] - offs[i])
        grad[3 * offs[i]:3 * offs[i + 1]] += w * gct[:ni]
        grad[3 * offs[j]:3 * offs[j + 1]] += w * gct[ni:]
    return grad, len(le_terms), len(ct_terms), pair_states
