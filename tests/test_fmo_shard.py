"""Multi-rank FMO work list (CPU, gloo, world size 2): the shards cover every instance once, are
balanced by estimated cost, and the all-gather returns the whole result list in the caller's order
on every rank.  The per-rank solver is a stand-in that derives each result from its instance, so no
GPU is needed; the GPU batch itself is covered by test_fmo.py."""

import os
import socket

import numpy as np
import pytest

from tincr_gb300 import _lib
from tincr_gb300 import fmo


def _instances(n=23, seed=5):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        o, v = int(rng.integers(8, 52)), int(rng.integers(8, 52))
        out.append(dict(n_occ=o, n_virt=v, n_roots=int(rng.choice([1, 4])), tag=k))
    return out


def _fake_solver(ctx, inst, **kw):
    return _lib.OK, [dict(energies=np.array([0.1 * q["tag"]]), tag=q["tag"]) for q in inst]


def test_shards_cover_and_balance():
    inst = _instances()
    for world in (1, 2, 3, 4):
        shards = [fmo.shard_instances(inst, world, r) for r in range(world)]
        flat = sorted(k for s in shards for k in s)
        assert flat == list(range(len(inst)))
        loads = [sum(fmo.instance_cost(inst[k]) for k in s) for s in shards]
        # LPT: the largest load exceeds the mean by at most the largest single instance
        assert max(loads) - sum(loads) / world <= max(fmo.instance_cost(q) for q in inst)


def _gloo_allgather(world):
    import torch.distributed as dist

    def gather(obj):
        parts = [None] * world
        dist.all_gather_object(parts, obj)
        return parts
    return gather


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        inst = _instances()
        rc, full = fmo.solve_batch_sharded(None, inst, world, rank, allgather=_gloo_allgather(world),
                                           solver=_fake_solver)
        q.put((rank, rc, [r["tag"] for r in full], [float(r["energies"][0]) for r in full]))
    finally:
        dist.destroy_process_group()


def _failing_solver(ctx, inst, **kw):
    """Rank 1's shard raises as the library does for a non-finite input; rank 0's shard reports
    NOT_CONVERGED."""
    import torch.distributed as dist
    if dist.get_rank() == 1:
        raise _lib.TincrError(_lib.NONFINITE, "planted non-finite input")
    return _lib.NOT_CONVERGED, [dict(energies=np.array([0.0]), tag=q["tag"]) for q in inst]


def _failing_rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        try:
            fmo.solve_batch_sharded(None, _instances(), world, rank, allgather=_gloo_allgather(world),
                                    solver=_failing_solver)
            q.put((rank, None, "no error"))
        except _lib.TincrError as e:
            q.put((rank, e.status, str(e)))
    finally:
        dist.destroy_process_group()


def test_sharded_results_gathered_in_order():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    n = len(_instances())
    for rank, rc, tags, es in got:
        assert rc == _lib.OK
        assert tags == list(range(n))
        assert np.allclose(es, 0.1 * np.arange(n))


def test_failed_shard_raises_on_every_rank():
    """A rank whose solve raises still joins the all-gather; every rank then raises the same error
    (the most severe status), so no rank waits in the collective for the failed one."""
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_failing_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, status, msg in got:
        assert status == _lib.NONFINITE, msg
        assert "planted non-finite input" in msg and "rank 1" in msg


def test_worst_status_folds_every_code():
    assert fmo.worst_status([]) == _lib.OK
    assert fmo.worst_status([_lib.OK, _lib.NOT_CONVERGED]) == _lib.NOT_CONVERGED
    assert fmo.worst_status([_lib.NOT_CONVERGED, _lib.CG_MAXITER, _lib.OK]) == _lib.CG_MAXITER
    assert fmo.worst_status([_lib.CUDA_ERR, _lib.NONFINITE, _lib.BAD_ARG]) == _lib.CUDA_ERR
    assert fmo.worst_status([_lib.OK, 42]) == 42


def _bench_rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        q.put((rank, bench.barrier_and_max(1.5 + rank, world)))
    finally:
        dist.destroy_process_group()


def test_bench_timing_is_max_over_ranks():
    """bench.py's N > 1 path (replicas of the single-system step): barrier, then the slowest rank's
    time on every rank."""
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_bench_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [v for _, v in got] == [2.5, 2.5]


def test_batch_marshalling_layout():
    """fmo.solve_batch marshals instances and result buffers as records with the C structs' layout:
    a stand-in for the library reads every instance through its pointers and writes every result,
    and each value lands in the right instance's arrays."""
    import ctypes as ct
    rng = np.random.default_rng(3)
    inst = []
    for k in range(7):
        na, o, v, nr = 2 + k % 3, 3 + k, 2 + (k * 2) % 5, 1 + k % 4
        n = o + v + 1
        inst.append(dict(n_atoms=na, n_orb=n, n_occ=o, n_virt=v, n_roots=nr,
                         opa=np.full(na, 1, np.int32), c=rng.standard_normal((n, o + v)),
                         s=rng.standard_normal((n, n)), orbe=rng.standard_normal(o + v),
                         gamma=rng.standard_normal((na, na)),
                         gamma_lr=None if k % 2 else rng.standard_normal((na, na)),
                         xyz=rng.standard_normal((na, 3))))

    class Lib:
        def tincr_tda_solve_batch(self, h, n, arr_addr, max_iter, tol, prec, res_addr):
            arr = (fmo._Instance * n).from_address(arr_addr)
            res = (fmo._Result * n).from_address(res_addr)
            for k in range(n):
                q = arr[k]
                o, v, nr, na = q.n_occ, q.n_virt, q.n_roots, q.n_atoms
                assert q.c[0] == inst[k]["c"][0, 0] and q.s[1] == inst[k]["s"].reshape(-1)[1]
                assert q.orbe[o + v - 1] == inst[k]["orbe"][-1] and q.xyz[3 * na - 1] == inst[k]["xyz"][-1, -1]
                assert bool(q.gamma_lr) == (inst[k]["gamma_lr"] is not None)
                r = res[k]
                for i in range(nr):
                    r.energies[i] = 100 * k + i
                    r.osc[i] = -k
                for i in range(o * v * nr):
                    r.coefficients[i] = k + 1e-3 * i
                for i in range(3 * nr):
                    r.tr_dip[i] = 7 * k
                for i in range(na * nr):
                    r.q_trans[i] = 11 * k + i
                r.iterations = 5 + k
                r.status = 0
            return 0

    class Ctx:
        lib = Lib()
        h = None

        def check(self, rc, allow=()):
            assert rc in allow

    rc, out = fmo.solve_batch(Ctx(), inst, 50, 1e-4, _lib.PREC_BF16X3)
    assert rc == _lib.OK
    for k, (q, r) in enumerate(zip(inst, out)):
        nr, ov = q["n_roots"], q["n_occ"] * q["n_virt"]
        assert np.array_equal(r["energies"], 100 * k + np.arange(nr))
        assert r["coefficients"].shape == (ov, nr)
        assert np.allclose(r["coefficients"].reshape(-1), k + 1e-3 * np.arange(ov * nr))
        assert np.all(r["osc"] == -k) and np.all(r["tr_dip"] == 7 * k) and r["tr_dip"].shape == (3, nr)
        assert np.array_equal(r["q_trans"].reshape(-1), 11 * k + np.arange(q["n_atoms"] * nr))
        assert r["iterations"] == 5 + k and r["status"] == 0
