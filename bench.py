"""Benchmark of the linear-response excited-state path on one GB300 (or N replicas).

Workload (one "step"): LC-TDA of the (H2O)128 water cluster (768 orbitals, 512 occupied x 256
virtual, omega = 0.3 bohr^-1 i.e. R_lr = 3.3333 bohr), lowest 20 roots with tincr's `sp` job
settings (max_iter 450, residual tolerance 1e-4; src/main.rs:124): transition charges / AO setup,
block Davidson, oscillator strengths.  Geometry: seeded synthetic cluster (tincr_gb300.geometry);
the ground state (C, S, orbital energies, gamma matrices) is prepared once on the host and is not
part of a step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64|bf16x3] [--impl reference]

`value` is device time per step (CUDA events on the library stream, inputs resident in HBM);
`e2e` is the same step through the C ABI with host buffers (setup upload + solve + result copy).
`--impl reference` times the CPU restatement of tincr's algorithm (the oracle, numpy + the host
BLAS with all host threads) on a bounded sample of the same workload and scales it to one step.
Under torchrun (N > 1) every rank runs an independent replica (the path does not shard one
system); rank 0 prints the JSON line with the max over ranks.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "LC-TDA roots+S1 grad wall s (mixed vs FP64 GPU, <=1e-6 Eh); FMO monomers/s"
N_ROOTS, MAX_ITER, TOL = 20, 450, 1e-4
R_LR = 1.0 / 0.3


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def barrier_and_max(value, world):
    """Barrier + max over ranks (gloo on CPU tensors: our GPU work never enters torch)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload():
    from tincr_gb300 import geometry as G
    from tincr_gb300 import groundstate as gs
    z, x = G.water_cluster(8, 4, 4)
    sy = gs.build_system(z, G.to_bohr(x), lc=True, r_lr=R_LR)
    g = gs.run_scc(sy, tol=1e-9)
    return sy, g


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for ln in open(self.path):
                p = [v.strip() for v in ln.split(",")]
                if len(p) < 9:
                    continue
                try:
                    sm.append(float(p[1]))
                    mx.append(float(p[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, p[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        except OSError:
            pass
        finally:
            if self.path and os.path.exists(self.path):
                os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def l2_flush(buf):
    """Write a buffer larger than L2 (129 MB) between timed steps."""
    buf.zero_()


def run_gpu(args):
    rank, world, local = dist_env()
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    from tincr_gb300 import _lib, build
    from tincr_gb300 import tda as T
    build.build()
    prec = {"fp64": _lib.PREC_FP64, "bf16x3": _lib.PREC_BF16X3}[args.precision]
    sy, g = workload()
    ctx = _lib.Context(local)
    es = T.ExcitedStateSystem.from_ground_state(ctx, sy, g)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    # pinned host copies of the step inputs for the end-to-end leg
    host_in = [es.orbs, es.s, es.orbe, es.gamma, es.gamma_lr, es.xyz]
    h2d_bytes = sum(a.nbytes for a in host_in) + es.opa.nbytes
    d2h_bytes = 8 * (N_ROOTS * (1 + es.dim + 1 + 3 + es.n_atoms))

    def step():
        es.run_tda(N_ROOTS, MAX_ITER, TOL, precision=prec)
        return ctx.last_timing()

    es.prepare_tda()
    for _ in range(args.warmup):
        l2_flush(flush)
        torch.cuda.synchronize()
        step()
    # device-timed region: inputs resident (prepare_tda done), Davidson + moments per step
    ctx.set_profiling(True)
    dev_ms, launches, iters = [], 0, []
    n_products_total = 0
    barrier_and_max(0.0, world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            l2_flush(flush)
            torch.cuda.synchronize()
            ms, nl = step()
            dev_ms.append(ms)
            launches += nl
            iters.append(es.properties["davidson_iterations"])
            n_products_total += es.properties["n_products"]
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    stats = {f: ctx.kernel_stats(f) for f in range(4)}
    ctx.set_profiling(False)
    # end-to-end leg: the public call sequence with host buffers (setup upload + solve + download)
    e2e = []
    for _ in range(args.steps):
        l2_flush(flush)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        es2 = T.ExcitedStateSystem(ctx, es.opa, es.orbs, es.s, es.orbe, es.n_occ, es.n_virt, es.gamma,
                                   es.gamma_lr, es.xyz)
        es2.prepare_tda()
        es2.run_tda(N_ROOTS, MAX_ITER, TOL, precision=prec)
        e2e.append(time.perf_counter() - t0)
    step_s = barrier_and_max(float(np.mean(dev_ms)) / 1e3, world)
    e2e_s = barrier_and_max(float(np.mean(e2e)), world)
    energies = es.properties["ci_eigenvalues"]
    out = None
    if rank == 0:
        peaks = {}
        pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
        if os.path.exists(pk):
            peaks = json.load(open(pk))
        ex = stats[_lib.KF_AO_EXCHANGE]
        if prec == _lib.PREC_FP64:
            # FP64 runs on the DFMA pipe; no measured FP64 peak exists, use the nominal GB300 rate
            achieved = ex["flops"] / (ex["ms"] / 1e3) / 1e12 if ex["ms"] > 0 else None
            peak, peak_note = 1.25, "nominal FP64 1.25 TFLOP/s (no measured FP64 peak)"
            bound, unit = "fp64", "TFLOP/s"
        else:
            achieved = ex["flops"] / (ex["ms"] / 1e3) / 1e12 if ex["ms"] > 0 else None
            peak = peaks.get("bf16_tflops", 1900.0)
            peak_note = "measured bf16_tflops" if "bf16_tflops" in peaks else "fallback 1.9 PFLOP/s"
            bound, unit = "tensor", "TFLOP/s"
        # DRAM bytes per launch of the exchange family: ncu bytes per product vector (full-size
        # capture, profiles/) times the vectors per launch of this solve (2 launches per chunk)
        traffic = None
        tf = os.path.join(ROOT, "profiles", "ao_exchange_traffic.json")
        if os.path.exists(tf) and ex["launches"] > 0:
            rec = json.load(open(tf)).get(args.precision)
            if rec:
                vec_per_launch = 2.0 * n_products_total / ex["launches"]
                traffic = rec["dram_bytes_per_vector"] * vec_per_launch / 2.0
        cpu = cpu_baseline(sy, g, sum(iters) / len(iters), es) if args.cpu_baseline else None
        out = {
            "metric": METRIC, "value": step_s, "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if prec == _lib.PREC_FP64 else "bf16x3+f64",
            "data": "synthetic (seeded (H2O)128 cluster, host SCC ground state)",
            "config": {"workload": "water128-lctda-20roots", "n_orb": int(sy.n_orbs), "n_occ": int(sy.n_occ),
                       "n_virt": int(sy.n_virt), "n_roots": N_ROOTS, "tol": TOL, "max_iter": MAX_ITER,
                       "r_lr_bohr": R_LR, "precision": args.precision, "l2": "flushed (256 MB write) between steps",
                       "parallelism": "replicas" if world > 1 else "single-gpu",
                       "davidson_iterations": iters[-1]},
            "e2e": {"value": e2e_s, "unit": "s", "h2d_bytes_per_step": int(h2d_bytes),
                    "d2h_bytes_per_step": int(d2h_bytes)},
            "gpu_launches": int(launches),
            "roofline": {"bound": bound, "achieved": achieved, "peak": peak, "unit": unit,
                         "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                         "algorithmic_flops_per_launch": ex["flops"] / max(1, ex["launches"]),
                         "algorithmic_bytes_per_launch": ex["bytes"] / max(1, ex["launches"]),
                         "kernel": "AO-exchange contractions (gemm_f64, A.X steps 2 and 4)",
                         "peak_source": peak_note,
                         "kernel_ms_per_step": ex["ms"] / args.steps,
                         "kernel_share_of_step": ex["ms"] / max(1e-9, sum(dev_ms))},
            "kernel_families_ms_per_step": {n: stats[f]["ms"] / args.steps for f, n in
                                            enumerate(["ao_exchange", "ao_transform", "subspace", "other"])},
            "cpu_baseline": cpu,
            "clocks": clocks.summary(),
            "lowest_energies_eh": [float(e) for e in energies[:3]],
            "wall_s": wall,
        }
    return out


def cpu_sample(sy, g, n_products, n_iters, sample_vectors=2):
    """Time tincr's reference-form algorithm (oracle, numpy + host BLAS) on a bounded sample:
    transition charges + `sample_vectors` A.X products + one Davidson subspace step at full
    size, scaled to the products and iterations of one full solve."""
    from oracle import tda as OT
    t0 = time.perf_counter()
    occ, virt = sy.occ_indices, sy.virt_indices
    qov, qoo, qvv = OT.trans_charges(sy.ao_offset, g.orbs, g.s, occ, virt)
    om = OT.orbe_differences(g.orbe[occ], g.orbe[virt])
    t_setup = time.perf_counter() - t0
    eng = OT.TdaEngine(om, qov, g.gamma, qoo, qvv, g.gamma_lr, sy.n_occ, sy.n_virt)
    rng = np.random.default_rng(0)
    x = rng.standard_normal((len(om), sample_vectors))
    t0 = time.perf_counter()
    ax = eng.apply(x)
    t_prod = (time.perf_counter() - t0) / sample_vectors
    # one subspace step with a half-full subspace (projection, eigh, Ritz, residuals)
    m = min(15 * N_ROOTS, 150)
    v = rng.standard_normal((len(om), m))
    av = rng.standard_normal((len(om), m))
    t0 = time.perf_counter()
    a = v.T @ av
    w, y = np.linalg.eigh(a, UPLO="U")
    ritz = v @ y[:, :N_ROOTS]
    rk = av @ y[:, :N_ROOTS] - ritz * w[:N_ROOTS]
    np.linalg.norm(rk, axis=0)
    t_sub = time.perf_counter() - t0
    total = t_setup + n_products * t_prod + n_iters * t_sub
    threads = os.cpu_count()
    sample = ("trans_charges + %d reference-form A.X products (%.2f s each) + one subspace step at m=%d, "
              "scaled to %d products and %d Davidson iterations" % (sample_vectors, t_prod, m, n_products, n_iters))
    return total, threads, sample


def cpu_baseline(sy, g, n_iters, es):
    n_products = int(es.properties["n_products"])
    total, threads, sample = cpu_sample(sy, g, n_products, int(n_iters))
    return {"value": total, "unit": "s", "cores": threads, "kind": "port", "sample": sample}


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return None
    sy, g = workload()
    # product count of the GPU solve at these settings (same algorithm, same guesses)
    n_products = args.ref_products
    vals = []
    sample = ""
    threads = os.cpu_count()
    for _ in range(args.warmup):
        cpu_sample(sy, g, n_products, args.ref_iters, sample_vectors=1)
    for _ in range(args.steps):
        total, threads, sample = cpu_sample(sy, g, n_products, args.ref_iters, sample_vectors=1)
        vals.append(total)
    v = float(np.mean(vals))
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": v * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded (H2O)128 cluster, host SCC ground state)",
            "config": {"workload": "water128-lctda-20roots", "n_roots": N_ROOTS, "tol": TOL, "max_iter": MAX_ITER},
            "cpu_baseline": {"value": v, "unit": "s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_products(args):
    """Profiling helper: set up the workload and evaluate A.X for `--k` random trial vectors once
    (used for ncu captures of the product kernels on the full-size system)."""
    from tincr_gb300 import _lib, build
    from tincr_gb300 import tda as T
    build.build()
    sy, g = workload()
    ctx = _lib.Context(0)
    es = T.ExcitedStateSystem.from_ground_state(ctx, sy, g)
    es.prepare_tda()
    x = np.random.default_rng(0).standard_normal((es.dim, args.k))
    prec = {"fp64": _lib.PREC_FP64, "bf16x3": _lib.PREC_BF16X3}[args.precision]
    for _ in range(max(1, args.steps)):
        ax = es.compute_products(x, precision=prec)
    ms, nl = ctx.last_timing()
    print(json.dumps({"mode": "products", "k": args.k, "ms": ms, "launches": nl,
                      "checksum": float(np.abs(ax).sum())}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "bf16x3"])
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--ref-products", type=int, default=420)
    ap.add_argument("--ref-iters", type=int, default=20)
    ap.add_argument("--mode", default="solve", choices=["solve", "products"])
    ap.add_argument("--k", type=int, default=4)
    args = ap.parse_args()
    if args.mode == "products":
        run_products(args)
        return
    out = run_reference(args) if args.impl == "reference" else run_gpu(args)
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
