"""Benchmark of the linear-response excited-state path on one GB300 (or N replicas).

Workload (one "step"): LC-TDA of the (H2O)128 water cluster (768 orbitals, 512 occupied x 256
virtual, omega = 0.3 bohr^-1 i.e. R_lr = 3.3333 bohr), lowest 20 roots with tincr's `sp` job
settings (max_iter 450, residual tolerance 1e-4; src/main.rs:124), then the analytic gradient of
S1 (ground-state + excitation gradient, tincr's formulas: Z-vector, derivative contractions).
Geometry: seeded synthetic cluster (tincr_gb300.geometry); the ground state (C, S, P, orbital
energies, gamma matrices) is prepared once on the host and is not part of a step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--precision bf16x3|fp64] [--impl reference]

The default precision is the mixed form (split-BF16 tensor-core products, FP64 convergence); the
run also times the plain FP64 form of the same step and reports it under "fp64_gpu" with the
largest energy and gradient differences between the two.
`value` is device time per step (CUDA events on the library stream, inputs resident in HBM);
`e2e` is the same step through the C ABI with host buffers (setup upload, solve, parameter upload,
gradient, result copies).
`cpu_baseline` (this arm) times the CPU restatement of tincr's algorithm (the oracle, numpy + the
host BLAS with all host threads) on a bounded sample of the water step, scaled to the step's counts;
the FMO work list is timed in full.  `--impl reference` runs the complete CPU step once, measured
(Davidson to convergence with its own iteration count, then the S1 gradients), and the whole FMO work
list.  `parity` holds the per-root errors against the oracle's results on the same inputs
(tests/golden/water128.npz, acene64.npz).
`--mode acene512` runs the 512-acene aggregate (8 x 8 x 8 lattice: batched TDA, exciton states,
the LE terms of the lowest exciton state's gradient) once per form with sampled oracle checks.
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
PRECISIONS = {"fp64": 0, "bf16x3": 1}   # tincr_precision values
FMO_N_LE, FMO_N_CT, FMO_TOL, FMO_MAX_ITER = 4, 1, 1e-4, 150
# exciton states: tincr's Davidson on the exciton matrix (src/fmo/lcmo/basis.rs:500: tolerance 1e-4,
# 100 iterations), the lowest 10 states
FMO_N_EXCITON, FMO_EX_TOL, FMO_EX_MAX_ITER = 10, 1e-4, 100
R_LR = 1.0 / 0.3
SCC_TOL = 1e-10   # the SCC's commutator tolerance (host and GPU)


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
    from tincr_gb300 import gradients as GR
    from tincr_gb300 import tda as T
    build.build()
    prec = PRECISIONS[args.precision]
    sy, g = workload()
    ctx = _lib.Context(local)
    es = T.ExcitedStateSystem.from_ground_state(ctx, sy, g)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    # page-locked host copies of the step inputs for the end-to-end leg (torch's pinned allocator,
    # viewed as numpy arrays; `keep` holds the tensors)
    keep = []

    def pinned(a):
        a = np.ascontiguousarray(a)
        t = torch.empty(a.shape, dtype=torch.float64 if a.dtype == np.float64 else torch.int32, pin_memory=True)
        keep.append(t)
        v = t.numpy()
        v[...] = a
        return v

    host_in = [pinned(a) for a in (es.orbs, es.s, es.orbe, es.gamma, es.gamma_lr, es.xyz)]
    opa_pin = pinned(es.opa.astype(np.int32))
    import dataclasses
    g_pin = dataclasses.replace(g, p=pinned(g.p), h_coul_x=pinned(g.h_coul_x), dq=pinned(g.dq))
    h2d_bytes = sum(a.nbytes for a in host_in) + es.opa.nbytes
    es.prepare_tda()
    gr = GR.GradientSystem(es, sy, g)
    h2d_bytes += gr.p.nbytes + gr.h.nbytes + gr.dq.nbytes + gr.atom_kind.nbytes
    h2d_bytes += sum(np.asarray(v).nbytes for v in gr.tables.values() if isinstance(v, np.ndarray))
    d2h_bytes = 8 * (N_ROOTS * (1 + es.dim + 1 + 3 + es.n_atoms)) + 2 * 8 * 3 * sy.n_atoms

    def step(p):
        """One step: lowest N_ROOTS roots, then the S1 (ground + excitation) gradient."""
        r = es.run_tda(N_ROOTS, MAX_ITER, TOL, precision=p)
        ms1, nl1 = ctx.last_timing()
        ggs, gex = gr.both(0, "reference")
        ms2, nl2 = ctx.last_timing()
        return ms1 + ms2, nl1 + nl2, r, ggs + gex

    def timed(p, warm, steps, profile):
        for _ in range(warm):
            l2_flush(flush)
            torch.cuda.synchronize()
            step(p)
        if profile:
            ctx.set_profiling(True)
        dev_ms, launches, iters, prods = [], 0, [], 0
        barrier_and_max(0.0, world)
        torch.cuda.synchronize()
        for _ in range(steps):
            l2_flush(flush)
            torch.cuda.synchronize()
            ms, nl, r, grad = step(p)
            dev_ms.append(ms)
            launches += nl
            iters.append(r["davidson_iterations"])
            prods += es.properties["n_products"]
        torch.cuda.synchronize()
        stats = {f: ctx.kernel_stats(f) for f in range(_lib.KF_COUNT)} if profile else None
        if profile:
            ctx.set_profiling(False)
        return dict(dev_ms=dev_ms, launches=launches, iters=iters, products=prods, stats=stats,
                    energies=r["ci_eigenvalues"].copy(), f=r["oscillator_strengths"].copy(), grad=grad.copy(),
                    cg=gr.last_cg_iterations)

    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        main = timed(prec, args.warmup, args.steps, False)
        wall = time.perf_counter() - t0
    # kernel-family breakdown from one more step with per-family CUDA events (kept out of the timed
    # steps: the events and their host bookkeeping perturb the step a little)
    main["stats"] = timed(prec, 0, 1, True)["stats"]
    # end-to-end leg: the public call sequence with host buffers (setup upload, solve, parameter
    # upload, gradient, result copies) for a system handed over from the host
    e2e = []
    for _ in range(args.steps):
        l2_flush(flush)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        orbs_h, s_h, orbe_h, gam_h, glr_h, xyz_h = host_in
        es2 = T.ExcitedStateSystem(ctx, opa_pin, orbs_h, s_h, orbe_h, es.n_occ, es.n_virt, gam_h, glr_h, xyz_h)
        es2.prepare_tda()
        es2.run_tda(N_ROOTS, MAX_ITER, TOL, precision=prec)
        gr2 = GR.GradientSystem(es2, sy, g_pin)
        gr2.both(0, "reference")
        e2e.append(time.perf_counter() - t0)
    # the plain FP64 form of the same step, for the mixed-vs-FP64 comparison
    ref64 = None
    if prec != _lib.PREC_FP64 and args.compare_fp64:
        es.prepare_tda()
        gr = GR.GradientSystem(es, sy, g)
        ref64 = timed(_lib.PREC_FP64, 1, max(1, min(args.steps, 2)), False)
    step_s = barrier_and_max(float(np.mean(main["dev_ms"])) / 1e3, world)
    e2e_s = barrier_and_max(float(np.mean(e2e)), world)
    if rank != 0:
        return None
    stats = main["stats"]
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    step_ms = float(np.mean(main["dev_ms"]))
    ex = stats[_lib.KF_AO_EXCHANGE]
    achieved = ex["flops"] / (ex["ms"] / 1e3) / 1e12 if ex["ms"] > 0 else None
    if prec == _lib.PREC_FP64:
        # FP64 runs on the DFMA pipe; no measured FP64 peak exists, use the nominal GB300 rate
        peak, peak_note = 1.25, "nominal FP64 1.25 TFLOP/s (no measured FP64 peak)"
        bound, kernel = "fp64", "AO-exchange contractions (gemm_f64, A.X steps 2 and 4)"
    else:
        peak = peaks.get("bf16_tflops", 1900.0)
        peak_note = ("measured bf16_tflops" if "bf16_tflops" in peaks else "fallback 1.9 PFLOP/s") + \
            "; achieved counts the algorithmic 2MNK once, the tensor pipe executes 6 split-BF16 plane products per MAC"
        bound, kernel = "tensor", "AO-exchange contractions (gemm_planes_tc, tcgen05 split-BF16, A.X steps 2 and 4)"
    # DRAM bytes per launch of the exchange family: ncu bytes per product vector (capture in
    # profiles/) times the vectors per launch of this step (2 launches per chunk)
    traffic = None
    tf = os.path.join(ROOT, "profiles", "ao_exchange_traffic.json")
    if os.path.exists(tf) and ex["launches"] > 0:
        rec = json.load(open(tf)).get(args.precision)
        if rec:
            vec_per_launch = 2.0 * (main["products"] / args.steps) / ex["launches"]   # stats: one step
            traffic = rec["dram_bytes_per_vector"] * vec_per_launch / 2.0
    roof_ex = {"bound": bound, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
               "frac": (achieved / peak) if achieved else None, "traffic": traffic,
               "algorithmic_flops_per_launch": ex["flops"] / max(1, ex["launches"]),
               "algorithmic_bytes_per_launch": ex["bytes"] / max(1, ex["launches"]),
               "kernel": kernel, "peak_source": peak_note,
               "kernel_ms_per_step": ex["ms"], "kernel_share_of_step": ex["ms"] / max(1e-9, step_ms),
               "launches_per_step": ex["launches"]}
    # the digit GEMMs of the mixed Davidson subspace products: HBM-bound (digit planes read once)
    roof_dg = None
    dg = stats.get(_lib.KF_DIGITS) if _lib.KF_COUNT > _lib.KF_DIGITS else None
    if dg and dg["launches"] > 0 and dg["ms"] > 0:
        gbs = dg["bytes"] / (dg["ms"] / 1e3) / 1e9
        hbm = peaks.get("hbm_gbs", 6800.0)
        dg_traffic = None
        tf = os.path.join(ROOT, "profiles", "gemm_digits_traffic.json")
        if os.path.exists(tf):
            ratio = json.load(open(tf)).get("dram_over_algorithmic")
            if ratio:
                dg_traffic = ratio * dg["bytes"] / dg["launches"]
        roof_dg = {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                   "traffic": dg_traffic,
                   "algorithmic_bytes_per_launch": dg["bytes"] / dg["launches"],
                   "algorithmic_flops_per_launch": dg["flops"] / dg["launches"],
                   "kernel": "subspace digit GEMMs (gemm_digits, tcgen05 bf16 digit products of FP64 operands: "
                             "projection, Ritz vectors, residuals, orthogonalisation)",
                   "peak_source": ("measured hbm_gbs" if "hbm_gbs" in peaks else "fallback 6.8 TB/s") +
                                  "; algorithmic bytes = the 8 bf16 digit planes of both operands read once + "
                                  "the FP64 output (the FP64 operands themselves are half that)",
                   "kernel_ms_per_step": dg["ms"], "kernel_share_of_step": dg["ms"] / max(1e-9, step_ms),
                   "launches_per_step": dg["launches"]}
    # the dominant kernel of the step carries the roofline; the other is reported beside it
    roofline, roofline_other = roof_ex, roof_dg
    if roof_dg and roof_dg["kernel_ms_per_step"] > roof_ex["kernel_ms_per_step"]:
        roofline, roofline_other = roof_dg, roof_ex
    cpu = cpu_baseline(sy, g, float(np.mean(main["iters"])), main["products"] / args.steps, main["cg"]) \
        if args.cpu_baseline else None
    fams = ["ao_exchange", "ao_transform", "subspace", "gradient", "other", "host_subspace_eigensolver",
            "subspace_eigensolver", "subspace_digit_gemm"][:_lib.KF_COUNT]
    out = {
        "metric": METRIC, "value": step_s, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if prec == _lib.PREC_FP64 else "bf16x3+f64",
        "data": "synthetic (seeded (H2O)128 cluster, host SCC ground state)",
        "config": workload_config(sy, world),
        "precision": args.precision,
        "counts": {"davidson_iterations": main["iters"][-1], "products": int(main["products"] / args.steps),
                   "zvector_cg_iterations": main["cg"]},
        "e2e": {"value": e2e_s, "unit": "s", "h2d_bytes_per_step": int(h2d_bytes),
                "d2h_bytes_per_step": int(d2h_bytes)},
        "gpu_launches": int(main["launches"]),
        "roofline": roofline,
        "roofline_other_kernel": roofline_other,
        "kernel_families_ms_per_step": {n: stats[f]["ms"] for f, n in enumerate(fams)},
        "cpu_baseline": cpu,
        "clocks": clocks.summary(),
        "lowest_energies_eh": [float(e) for e in main["energies"][:3]],
        "wall_s": wall,
    }
    out["parity"] = water_parity(g, main, ref64)
    if args.fmo:
        out["fmo"], mons = run_fmo(args, ctx)
        if world == 1 and args.next_rows:
            out["scc"] = _guarded(lambda: scc_measure(ctx, mons, args.cpu_baseline))
    if world == 1 and args.next_rows:
        out["rpa"] = _guarded(lambda: rpa_measure(ctx, sy, g))
        out["fd"] = _guarded(lambda: fd_measure(ctx))
    if ref64 is not None:
        out["fp64_gpu"] = {"value": float(np.mean(ref64["dev_ms"])) / 1e3, "unit": "s",
                           "speedup_of_mixed": float(np.mean(ref64["dev_ms"])) / max(1e-9, float(np.mean(main["dev_ms"]))),
                           "max_abs_energy_err_eh": float(np.abs(main["energies"] - ref64["energies"]).max()),
                           "max_abs_grad_err_eh_per_bohr": float(np.abs(main["grad"] - ref64["grad"]).max())}
    return out


def golden(name):
    """A committed oracle fixture of the benchmark workloads (tests/golden/make_bench_fixtures.py)."""
    path = os.path.join(ROOT, "tests", "golden", name + ".npz")
    return np.load(path) if os.path.exists(path) else None


def water_parity(g, main, ref64):
    """Per-root errors of this run against the oracle's results on the same inputs (computed once on
    the CPU, tests/golden/water128.npz): energies and oscillator strengths per root, the largest S1
    gradient error, for the timed precision and for the FP64 form."""
    fx = golden("water128")
    if fx is None:
        return {"unavailable": "fixture tests/golden/water128.npz missing"}
    d_orbe = float(np.abs(g.orbe - fx["orbe"]).max())
    if d_orbe > 1e-8:
        return {"unavailable": "ground state differs from the fixture's (orbital energies %.1e)" % d_orbe}
    ref_g = fx["grad_ground"] + fx["grad_excited"]
    out = {"oracle": "tests/golden/water128.npz: numpy restatement of tincr on the same inputs, roots converged to "
                     "residual %g (%d Davidson iterations, %d products, corrections re-orthogonalised)"
                     % (float(fx["tol"]), int(fx["iterations"]), int(fx["n_products"])),
           "bars": {"fp64_energy_eh": 1e-8, "mixed_energy_eh": 1e-6, "gradient_eh_per_bohr": 1e-5},
           "per_root_energy_err_eh": [float(x) for x in np.abs(main["energies"] - fx["energies"])],
           "per_root_f_err": [float(x) for x in np.abs(main["f"] - fx["f"])],
           "max_grad_err_eh_per_bohr": float(np.abs(main["grad"] - ref_g).max())}
    if ref64 is not None:
        out["fp64_per_root_energy_err_eh"] = [float(x) for x in np.abs(ref64["energies"] - fx["energies"])]
        out["fp64_max_f_err"] = float(np.abs(ref64["f"] - fx["f"]).max())
        out["fp64_max_grad_err_eh_per_bohr"] = float(np.abs(ref64["grad"] - ref_g).max())
        out["fp64_davidson_iterations"] = int(ref64["iters"][-1])
    return out


def fmo_workload():
    """64-acene FMO aggregate: 4 x 4 x 4 lattice (3.6 / 5.0 / 14 A), ring counts drawn from {2..5},
    +-15 deg in-plane rotation, +-0.1 A jitter (seeded); LC, monomer SCC on the host; CT pairs with a
    smallest interatomic distance below 4.5 A; 4 LE roots per monomer, 1 CT root per pair direction."""
    from tincr_gb300 import fmo
    from tincr_gb300 import geometry as G
    from tincr_gb300 import groundstate as gs
    z, x, mono = G.acene_lattice(4, 4, 4)
    mons = fmo.build_monomers(z, G.to_bohr(x), mono, lc=True)
    pairs = fmo.close_pairs(mons, 4.5 / gs.P.BOHR_TO_ANGS)
    inst, labels = fmo.aggregate_instances(mons, pairs, FMO_N_LE, FMO_N_CT)
    return mons, pairs, inst, labels


def _cpu_helpers():
    """The oracle and its input builders (test infrastructure, used only by the CPU legs)."""
    tests = os.path.join(ROOT, "tests")
    if tests not in sys.path:
        sys.path.insert(0, tests)
    import cases
    from oracle import gradients as OG
    from oracle import tda as OT
    return cases, OG, OT


def fmo_cpu_reference(mons, pairs, inst, labels, setup):
    """tincr's FMO step on the CPU, measured in full: the TDA of every instance of the work list
    with tincr's engines (oracle `TdaEngine` per monomer, `CtEngine` per pair direction; numpy +
    the host BLAS); the exciton Hamiltonian over those states (LCMO Fock matrix, then the matrix
    rows shared out to one process per host core, as tincr shares them out to rayon threads,
    src/fmo/lcmo/basis.rs:479-487) and its lowest 10 roots by tincr's Davidson; then the LE
    excitation gradient of the aggregate's lowest LE root (dense derivative tensors, Z-vector,
    f_v / f_lr contractions).  `setup` (pair types, overlaps, gamma, dimer ground states) is the
    host set-up the GPU arm also reads, not timed.  Returns (seconds, description, exciton energies)."""
    cases, OG, OT = _cpu_helpers()
    from oracle import exciton as OX
    case = dict(monomers=mons, labels=labels, lc=True)
    t0 = time.perf_counter()
    res = []
    for k, q in enumerate(inst):
        eng, xyz = cases.fmo_oracle_engine(case, k)
        res.append(OT.run_tda_engine(eng, xyz, q["n_roots"], FMO_MAX_ITER, FMO_TOL))
    t_tda = time.perf_counter() - t0
    t0 = time.perf_counter()
    agg = OX.aggregate_of(mons, setup)
    states = OX.basis_of(agg, labels, res, setup.ct_pairs, FMO_N_LE, FMO_N_CT)
    h = OX.exciton_hamiltonian_rows(agg, states, os.cpu_count() or 1)
    ex = OX.exciton_states(h, FMO_N_EXCITON, FMO_EX_TOL, FMO_EX_MAX_ITER)
    t_ex = time.perf_counter() - t0
    t0 = time.perf_counter()
    n_mon = len(mons)
    k1 = int(np.argmin([res[k]["energies"][0] for k in range(n_mon)]))
    sy, g = mons[k1].system, mons[k1].ground
    q = OT.trans_charges(sy.ao_offset, g.orbs, g.s, sy.occ_indices, sy.virt_indices)
    inp = cases.oracle_gradient_inputs(sy, g, True, res[k1]["energies"], res[k1]["coefficients"], q)
    der = OG.derivative_tensors(sy.numbers, sy.xyz, sy.ao_offset, sy.ao_atom, sy.hubbard, sy.r_lr, sy.params)
    _, flr = OG.ground_state_gradient(inp, der, True)
    OG.tda_gradient(inp, der, 0, True, flr_dmd0=flr)
    t_grad = time.perf_counter() - t0
    n_le = sum(1 for l in labels if l[0] == "LE")
    sample = ("measured in full: oracle TDA of all %d instances (%d LE, %d CT; %.2f s) + the exciton Hamiltonian "
              "(%d states, rows on %d processes) and its lowest %d roots (%.2f s) + the LE gradient of the lowest LE "
              "root (monomer %d, %.2f s)" % (len(inst), n_le, len(inst) - n_le, t_tda, len(states),
                                              os.cpu_count() or 1, FMO_N_EXCITON, t_ex, k1, t_grad))
    return t_tda + t_ex + t_grad, sample, np.asarray(ex[0])


def ctx_device(ctx):
    return int(os.environ.get("LOCAL_RANK", "0"))


def tile_summary(table):
    """How many instance shapes chose each tile shape, per plane GEMM step of the mixed batch."""
    out = {"instance_shapes": len(table)}
    for st in ("H", "F", "G", "AX"):
        cnt = {}
        for t in table:
            sh = t["shapes"][st]
            if sh is not None:
                cnt[sh] = cnt.get(sh, 0) + 1
        out[st] = cnt
    return out


def exciton_gradient_measure(ctx, setup, labels, mixed, fp64):
    """Gradient of the lowest exciton state (`fmo.exciton_gradient`: c^2-weighted LE gradients of
    the monomers and CT-state gradients of the dimers, every basis state with |c| > 0.05), outside
    the timed FMO step: the first call includes the batched GPU SCC of the dimers it needs, the second
    reuses those ground states.  Mixed and FP64 forms, each from its own batch and exciton roots."""
    from tincr_gb300 import _lib
    from tincr_gb300 import fmo
    ctxs = [_lib.Context(ctx_device(ctx)) for _ in range(8)]
    out = {"terms_threshold": 0.05}
    grads = {}
    try:
        pst = None
        for name, prec, (r, ex) in (("bf16x3", _lib.PREC_BF16X3, mixed), ("fp64", _lib.PREC_FP64, fp64)):
            v = ex["vectors"][:, 0]
            t0 = time.perf_counter()
            g, n_le, n_ct, pst = fmo.exciton_gradient(ctx, setup, r, labels, FMO_N_LE, FMO_N_CT, v, contexts=ctxs,
                                                      precision=prec, pair_states=pst)
            t_first = time.perf_counter() - t0
            t0 = time.perf_counter()
            g, n_le, n_ct, pst = fmo.exciton_gradient(ctx, setup, r, labels, FMO_N_LE, FMO_N_CT, v, contexts=ctxs,
                                                      precision=prec, pair_states=pst)
            grads[name] = g
            out[name] = {"le_terms": n_le, "ct_terms": n_ct, "wall_ms": (time.perf_counter() - t0) * 1e3,
                         "first_call_wall_ms": t_first * 1e3, "dimer_scc_pairs": len(pst),
                         "gradient_norm": float(np.linalg.norm(g))}
        out["max_abs_err_mixed_vs_fp64_eh_per_bohr"] = float(np.abs(grads["bf16x3"] - grads["fp64"]).max())
    except Exception as e:   # a dimer without a stationary SCC ground state: reported, not fatal
        out["error"] = "%s: %s" % (type(e).__name__, e)
    finally:
        for c in ctxs:
            c.close()
    return out


def run_fmo(args, ctx):
    """The 64-acene FMO step, mixed and FP64 forms (monomers/s): batched LE / CT TDA of the work
    list, the exciton Hamiltonian and its lowest 10 states, and the S1 LE gradient.  Returns the
    JSON record and the monomers (their ground states serve the SCC measurement)."""
    from tincr_gb300 import _lib
    from tincr_gb300 import fmo
    t0 = time.perf_counter()
    mons, pairs, inst, labels = fmo_workload()
    t_setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    setup = fmo.ExcitonSetup(mons, pairs, workers=min(16, os.cpu_count() or 1))
    t_exsetup = time.perf_counter() - t0
    out = {"workload": "acene64-fmo-le4-ct1-exciton10", "monomers": len(mons), "ct_pairs": len(pairs),
           "instances": len(inst), "tol": FMO_TOL, "max_iter": FMO_MAX_ITER,
           "exciton": {"n_states": FMO_N_EXCITON, "tol": FMO_EX_TOL, "max_iter": FMO_EX_MAX_ITER,
                       "basis": "%d LE per monomer + %d CT per pair direction" % (FMO_N_LE, FMO_N_CT),
                       "real_pairs": len(setup.real_pairs)},
           "host_setup_s": t_setup, "host_exciton_setup_s": t_exsetup}
    res = {}
    gctx = _lib.Context(ctx_device(ctx))
    n_mon = len(mons)

    def fmo_step(prec):
        """Batched LE / CT TDA; the exciton Hamiltonian over those states and its lowest 10 roots;
        then the gradient of S1, the lowest LE root of the aggregate (its LE gradient, c = 1; the
        lowest exciton state's gradient with its CT terms is measured after the steps,
        `exciton_gradient_measure`)."""
        rc, r = fmo.solve_batch(ctx, inst, FMO_MAX_ITER, FMO_TOL, prec)
        t_batch = ctx.last_timing()[0] / 1e3
        ex = fmo.exciton_states(ctx, setup, r, labels, FMO_N_LE, FMO_N_CT, n_roots=FMO_N_EXCITON, tol=FMO_EX_TOL,
                                max_iter=FMO_EX_MAX_ITER, precision=prec)
        t_ex = ctx.last_timing()[0] / 1e3
        k1 = int(np.argmin([r[k]["energies"][0] for k in range(n_mon)]))
        states = [None] * n_mon
        states[k1] = 0
        g = fmo.le_gradients(mons, r[:n_mon], states, contexts=[gctx], precision=prec)
        t_grad = gctx.last_timing()[0] / 1e3
        return rc, r, g[k1], k1, t_batch, t_grad, ex, t_ex

    for name, prec in (("bf16x3", _lib.PREC_BF16X3), ("fp64", _lib.PREC_FP64)):
        for _ in range(max(1, args.warmup)):
            fmo_step(prec)
        dev, wall, tb, tg, te = [], [], [], [], []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            rc, r, g1, k1, t_batch, t_grad, ex, t_ex = fmo_step(prec)
            wall.append(time.perf_counter() - t0)
            dev.append(t_batch + t_ex + t_grad)
            tb.append(t_batch)
            tg.append(t_grad)
            te.append(t_ex)
        res[name] = (float(np.mean(dev)), float(np.mean(wall)), rc, r, g1, k1, float(np.mean(tb)), float(np.mean(tg)),
                     ex, float(np.mean(te)))
    gctx.close()
    dm, wm, rcm, rm, gm, km, tbm, tgm, exm, tem = res["bf16x3"]
    d64, w64, rc64, r64, g64, k64, tb64, tg64, ex64, te64 = res["fp64"]
    out["exciton_gradient"] = exciton_gradient_measure(ctx, setup, labels, (rm, exm), (r64, ex64))
    out["exciton"].update({
        "energies_eh": [float(e) for e in exm["energies"]], "davidson_iterations": int(exm["iterations"]),
        "status_ok": bool(exm["status"] == _lib.OK and ex64["status"] == _lib.OK),
        "max_abs_energy_err_vs_fp64_eh": float(np.abs(exm["energies"] - ex64["energies"]).max())})
    out.update({
        "value_monomers_per_s": len(mons) / dm, "unit": "monomers/s",
        "step_ms": dm * 1e3, "batch_tda_ms": tbm * 1e3, "exciton_ms": tem * 1e3, "s1_gradient_ms": tgm * 1e3,
        "instances_per_s": len(inst) / tbm,
        "e2e": {"value": len(mons) / wm, "unit": "monomers/s", "wall_ms": wm * 1e3},
        "fp64_gpu": {"value": len(mons) / d64, "step_ms": d64 * 1e3, "batch_tda_ms": tb64 * 1e3,
                     "exciton_ms": te64 * 1e3, "s1_gradient_ms": tg64 * 1e3, "e2e_wall_ms": w64 * 1e3},
        "speedup_mixed_vs_fp64": d64 / dm,
        "status_ok": bool(rcm == _lib.OK and rc64 == _lib.OK),
        "max_abs_energy_err_eh": float(max(np.abs(a["energies"] - b["energies"]).max() for a, b in zip(rm, r64))),
        "s1_monomer": km,
        "max_abs_s1_grad_err_eh_per_bohr": float(np.abs(gm - g64).max()) if km == k64 else None,
        "davidson_iterations_max": int(max(x["iterations"] for x in rm)),
        "plane_tile_autotuner": tile_summary(ctx.batch_tile_table()),
    })
    fx = golden("acene64")
    if fx is not None:
        orbe = np.concatenate([m.ground.orbe for m in mons])
        if np.abs(orbe - fx["monomer_orbe"]).max() <= 1e-8:
            em = np.concatenate([r["energies"] for r in rm])
            e64 = np.concatenate([r["energies"] for r in r64])
            out["parity"] = {
                "oracle": "tests/golden/acene64.npz: oracle engines on every instance, same inputs",
                "mixed_max_energy_err_eh": float(np.abs(em - fx["energies"]).max()),
                "fp64_max_energy_err_eh": float(np.abs(e64 - fx["energies"]).max()),
                "fp64_iterations_equal": [r["iterations"] for r in r64] == fx["iterations"].tolist(),
                "mixed_s1_le_grad_err_eh_per_bohr": float(np.abs(gm - fx["s1_le_gradient"]).max())
                if km == int(fx["s1_monomer"]) else None,
                "fp64_s1_le_grad_err_eh_per_bohr": float(np.abs(g64 - fx["s1_le_gradient"]).max())
                if k64 == int(fx["s1_monomer"]) else None}
            if "exciton_energies" in fx.files:
                out["parity"]["exciton_oracle"] = ("oracle exciton Hamiltonian over the oracle's LE / CT roots, "
                                                   "its Davidson at the same settings")
                out["parity"]["mixed_exciton_energy_err_eh"] = [
                    float(x) for x in np.abs(exm["energies"] - fx["exciton_energies"])]
                out["parity"]["fp64_exciton_max_energy_err_eh"] = float(
                    np.abs(ex64["energies"] - fx["exciton_energies"]).max())
    if args.cpu_baseline:
        total, sample, _ = fmo_cpu_reference(mons, pairs, inst, labels, setup)
        out["cpu_baseline"] = {"value": len(mons) / total, "unit": "monomers/s", "step_s": total,
                               "cores": os.cpu_count(), "kind": "port", "sample": sample}
    return out, mons


def cpu_sample(sy, g, n_products, n_iters, cg_iters, sample_vectors=2):
    """Time tincr's reference-form algorithm (oracle, numpy + host BLAS) on a bounded sample of one
    step and scale it to the whole step.

    TDA: transition charges + `sample_vectors` A.X products + one Davidson subspace step at full
    size, scaled to the products and iterations of one solve.  Gradient (tincr's dense formulas,
    src/gradients/helpers.rs:47-188): the f_v and f_lr loop bodies for the 3 coordinates of one atom
    at full size (dense dS / dgamma operands, which is how tincr multiplies them), scaled to 3N
    coordinates and their two calls each, plus `cg_iters` Z-vector products and the [3N, n^2]
    contractions.  The construction of the derivative tensors themselves is not counted."""
    from oracle import gradients as OG
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
    eng.apply(x)
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
    del qov, qoo, qvv, eng, v, av
    # gradient sample: one atom's 3 coordinates of f_lr and f_v, and of the [3N, n^2] contractions
    n, N = g.s.shape[0], sy.n_atoms
    ds = rng.standard_normal((3, n, n))
    dg = rng.standard_normal((3, n, n))
    vm = rng.standard_normal((n, n))
    glr_ao = g.gamma_lr[np.ix_(sy.ao_atom, sy.ao_atom)]
    g_ao = g.gamma[np.ix_(sy.ao_atom, sy.ao_atom)]
    t0 = time.perf_counter()
    OG.f_lr(vm, g.s, ds, glr_ao, dg, 1, n)
    t_flr = time.perf_counter() - t0
    t0 = time.perf_counter()
    OG.f_v(vm, g.s, ds, g_ao, dg, 1, n)
    t_fv = time.perf_counter() - t0
    t0 = time.perf_counter()
    ds.reshape(3, -1) @ vm.reshape(-1)
    t_mv = time.perf_counter() - t0
    t_grad = N * (2.0 * t_flr + 2.0 * t_fv + 6.0 * t_mv) + cg_iters * t_prod
    total = t_setup + n_products * t_prod + n_iters * t_sub + t_grad
    threads = os.cpu_count()
    sample = ("TDA: trans_charges + %d reference-form A.X products (%.2f s each) + one subspace step at m=%d, "
              "scaled to %d products and %d Davidson iterations; S1 gradient: f_lr (%.2f s) and f_v (%.2f s) "
              "on 3 of %d coordinates, scaled to all coordinates x 2 calls, + %d Z-vector products "
              "(derivative-tensor construction not counted)"
              % (sample_vectors, t_prod, m, n_products, n_iters, t_flr, t_fv, 3 * N, cg_iters))
    return total, threads, sample


def cpu_baseline(sy, g, n_iters, n_products, cg_iters):
    total, threads, sample = cpu_sample(sy, g, int(n_products), int(round(n_iters)), int(cg_iters))
    out = {"value": total, "unit": "s", "cores": threads, "kind": "port", "sample": sample}
    out["single_thread"] = cpu_single_thread(int(n_products), int(round(n_iters)), int(cg_iters))
    return out


def cpu_single_thread(n_products, n_iters, cg_iters):
    """The same sample with one thread: a child process whose BLAS and OpenMP pools have one thread
    (set before numpy loads), one A.X product in the sample."""
    import subprocess
    import sys
    env = dict(os.environ, OMP_NUM_THREADS="1", OPENBLAS_NUM_THREADS="1", MKL_NUM_THREADS="1")
    cmd = [sys.executable, os.path.abspath(__file__), "--mode", "cpu-sample", "--ref-products", str(n_products),
           "--ref-iters", str(n_iters), "--ref-cg", str(cg_iters)]
    try:
        r = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=600)
        d = json.loads(r.stdout.strip().splitlines()[-1])
        return {"value": d["value"], "unit": "s", "cores": 1}
    except Exception as e:   # the baseline is reported, not required
        return {"unavailable": str(e)[:200]}


def run_cpu_sample(args):
    """--mode cpu-sample: the CPU sample of one step in this process (no GPU), one A.X product."""
    sy, g = workload()
    total, threads, sample = cpu_sample(sy, g, args.ref_products, args.ref_iters, args.ref_cg, sample_vectors=1)
    print(json.dumps({"value": total, "threads": threads, "sample": sample}))


def cpu_reference_step(sy, g):
    """tincr's complete step on the CPU, measured: the oracle (numpy + the host BLAS, all host
    threads) runs transition charges, the Davidson to convergence at the bench settings (its own
    products and iterations; tincr's `System::run_tda`, src/excited_states/tda/mod.rs:74-131), the
    moments, then the S1 ground-state and excitation gradients of tincr's formulas
    (src/gradients/ground_state.rs:12-137, src/gradients/excited_state.rs:56-487), with the
    derivative-tensor rows of one atom at a time built on the way (the same per-coordinate f_v /
    f_lr work as tincr's loops, src/gradients/helpers.rs:47-188, without holding [3N, n, n]).
    The Davidson orthogonalises each correction twice: with tincr's single Gram-Schmidt pass the
    restated solve of this cluster loses the orthogonality of its basis after the subspace collapse
    and stops at spurious near-zero roots (oracle.tda.davidson); the second pass costs one more
    matrix-vector pass per correction, under 1% of the step, and gives the roots the GPU path finds."""
    cases, OG, OT = _cpu_helpers()
    occ, virt = sy.occ_indices, sy.virt_indices
    t0 = time.perf_counter()
    q = OT.trans_charges(sy.ao_offset, g.orbs, g.s, occ, virt)
    om = OT.orbe_differences(g.orbe[occ], g.orbe[virt])
    eng = OT.TdaEngine(om, q[0], g.gamma, q[1], q[2], g.gamma_lr, sy.n_occ, sy.n_virt)
    r = OT.run_tda_engine(eng, sy.xyz, N_ROOTS, MAX_ITER, TOL, reorthogonalize=True)
    t_tda = time.perf_counter() - t0
    t0 = time.perf_counter()
    inp = cases.oracle_gradient_inputs(sy, g, True, r["energies"], r["coefficients"], q)
    del eng, q
    rows = OG.AtomRows(sy.numbers, sy.xyz, sy.ao_offset, sy.ao_atom, sy.hubbard, sy.r_lr, sy.params)
    st = {}
    OG.gradients_by_atom(inp, rows, 0, True, stats=st)
    t_grad = time.perf_counter() - t0
    return dict(seconds=t_tda + t_grad, tda_s=t_tda, gradient_s=t_grad, davidson_iterations=int(r["iterations"]),
                products=int(r["n_products"]), zvector_cg_iterations=int(st.get("cg_iterations", 0)),
                lowest_energies_eh=[float(e) for e in r["energies"][:3]])


def workload_config(sy, world):
    """The `config` object of both arms (the workload: what is computed, not how)."""
    return {"workload": "water128-lctda-20roots+S1grad", "n_orb": int(sy.n_orbs), "n_occ": int(sy.n_occ),
            "n_virt": int(sy.n_virt), "n_roots": N_ROOTS, "tol": TOL, "max_iter": MAX_ITER, "r_lr_bohr": R_LR,
            "gradient": "S1, tincr formulas", "l2": "GPU arm: flushed (256 MB write) between steps",
            "parallelism": "replicas" if world > 1 else "single-gpu"}


def run_reference(args):
    """`--impl reference`: tincr's algorithm on the host CPU (the oracle port; tincr itself is
    Rust and cannot be built here).  Rank 0 alone works.  Warm-up: `--warmup` reference-form A.X
    products.  Timed: the complete step once, measured end to end (`cpu_reference_step`); its wall
    time is the line's value, spread evenly over the `--steps` steps of the line (ms_per_step), so
    the steps' total equals the time the run actually took.  The FMO object times the whole
    64-acene work list and the S1 LE gradient the same way."""
    rank, world, local = dist_env()
    if rank != 0:
        return None
    cases, OG, OT = _cpu_helpers()
    sy, g = workload()
    q = OT.trans_charges(sy.ao_offset, g.orbs, g.s, sy.occ_indices, sy.virt_indices)
    om = OT.orbe_differences(g.orbe[sy.occ_indices], g.orbe[sy.virt_indices])
    eng = OT.TdaEngine(om, q[0], g.gamma, q[1], q[2], g.gamma_lr, sy.n_occ, sy.n_virt)
    x = np.random.default_rng(0).standard_normal((len(om), 1))
    for _ in range(args.warmup):
        eng.apply(x)
    del eng, q
    rec = cpu_reference_step(sy, g)
    v = rec["seconds"]
    threads = os.cpu_count()
    sample = ("measured in full, once: trans_charges + Davidson to convergence (%d iterations, %d reference-form A.X "
              "products, corrections orthogonalised twice, %.1f s) + S1 ground-state and excitation gradients atom by atom (Z-vector %d CG iterations, "
              "derivative rows and f_v / f_lr per coordinate, %.1f s); the wall time is spread evenly over the %d "
              "steps" % (rec["davidson_iterations"], rec["products"], rec["tda_s"], rec["zvector_cg_iterations"],
                         rec["gradient_s"], args.steps))
    fmo_ref = None
    if args.fmo:
        from tincr_gb300 import fmo
        mons, pairs, inst, labels = fmo_workload()
        setup = fmo.ExcitonSetup(mons, pairs, workers=os.cpu_count() or 1)
        total, fsample, _ = fmo_cpu_reference(mons, pairs, inst, labels, setup)
        fmo_ref = {"workload": "acene64-fmo-le4-ct1-exciton10", "value_monomers_per_s": len(mons) / total,
                   "unit": "monomers/s", "step_s": total, "cores": threads, "kind": "port", "sample": fsample}
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": v * 1e3 / max(1, args.steps), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded (H2O)128 cluster, host SCC ground state)",
            "config": workload_config(sy, world),
            "counts": {k: rec[k] for k in ("davidson_iterations", "products", "zvector_cg_iterations")},
            "lowest_energies_eh": rec["lowest_energies_eh"],
            "cpu_baseline": {"value": v, "unit": "s", "cores": threads, "kind": "port", "sample": sample,
                             "tda_s": rec["tda_s"], "gradient_s": rec["gradient_s"]},
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "fmo": fmo_ref}


def run_fmo_once(args):
    """Profiling helper: the 64-acene FMO work list solved once by the batched TDA (`--steps`
    repetitions after one warm-up), without kernel timing (so the CUDA-graph iteration runs)."""
    from tincr_gb300 import _lib, build
    from tincr_gb300 import fmo
    build.build()
    mons, pairs, inst, labels = fmo_workload()
    ctx = _lib.Context(0)
    prec = PRECISIONS[args.precision]
    fmo.solve_batch(ctx, inst, FMO_MAX_ITER, FMO_TOL, prec)
    for _ in range(max(1, args.steps)):
        rc, r = fmo.solve_batch(ctx, inst, FMO_MAX_ITER, FMO_TOL, prec)
    ms, nl = ctx.last_timing()
    print(json.dumps({"mode": "fmo", "precision": args.precision, "instances": len(inst), "status": rc, "ms": ms,
                      "launches": nl, "plane_tile_autotuner": tile_summary(ctx.batch_tile_table()),
                      "plane_tile_table": ctx.batch_tile_table()}))
    ctx.close()


def run_fmo_exciton_once(args):
    """Profiling helper: the 64-acene work list solved once by the batched TDA, then the exciton
    Hamiltonian and its lowest 10 states once (`--precision`), without kernel timing."""
    from tincr_gb300 import _lib, build
    from tincr_gb300 import fmo
    build.build()
    mons, pairs, inst, labels = fmo_workload()
    setup = fmo.ExcitonSetup(mons, pairs, workers=os.cpu_count() or 1)
    ctx = _lib.Context(0)
    prec = PRECISIONS[args.precision]
    rc, r = fmo.solve_batch(ctx, inst, FMO_MAX_ITER, FMO_TOL, prec)
    ex = fmo.exciton_states(ctx, setup, r, labels, FMO_N_LE, FMO_N_CT, n_roots=FMO_N_EXCITON, tol=FMO_EX_TOL,
                            max_iter=FMO_EX_MAX_ITER, precision=prec)
    ms, nl = ctx.last_timing()
    print(json.dumps({"mode": "fmo-exciton", "precision": args.precision, "states": int(len(ex["vectors"])),
                      "status": ex["status"], "ms": ms, "launches": nl,
                      "energies_eh": [float(e) for e in ex["energies"]]}))
    ctx.close()


def run_fmo_exgrad_once(args):
    """Profiling helper: the 64-acene work list solved once by the batched TDA, its exciton states,
    then the gradient of the lowest exciton state (`fmo.exciton_gradient`, LE and CT terms) twice
    (`--precision`); the second call, which reuses the dimer ground states of the first, runs between
    cudaProfilerStart and cudaProfilerStop (for `ncu --profile-from-start off`)."""
    import torch
    from tincr_gb300 import _lib, build
    from tincr_gb300 import fmo
    build.build()
    mons, pairs, inst, labels = fmo_workload()
    setup = fmo.ExcitonSetup(mons, pairs, workers=min(16, os.cpu_count() or 1))
    ctx = _lib.Context(0)
    prec = PRECISIONS[args.precision]
    rc, r = fmo.solve_batch(ctx, inst, FMO_MAX_ITER, FMO_TOL, prec)
    ex = fmo.exciton_states(ctx, setup, r, labels, FMO_N_LE, FMO_N_CT, n_roots=FMO_N_EXCITON, tol=FMO_EX_TOL,
                            max_iter=FMO_EX_MAX_ITER, precision=prec)
    ctxs = [_lib.Context(0) for _ in range(8)]
    v = ex["vectors"][:, 0]
    g, n_le, n_ct, pst = fmo.exciton_gradient(ctx, setup, r, labels, FMO_N_LE, FMO_N_CT, v, contexts=ctxs,
                                              precision=prec)
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    t0 = time.perf_counter()
    g, n_le, n_ct, pst = fmo.exciton_gradient(ctx, setup, r, labels, FMO_N_LE, FMO_N_CT, v, contexts=ctxs,
                                              precision=prec, pair_states=pst)
    wall = time.perf_counter() - t0
    torch.cuda.profiler.stop()
    print(json.dumps({"mode": "fmo-exgrad", "precision": args.precision, "batch_status": rc, "le_terms": n_le,
                      "ct_terms": n_ct, "dimers": len(pst), "wall_ms": wall * 1e3,
                      "gradient_norm": float(np.linalg.norm(g))}))
    for c in ctxs:
        c.close()
    ctx.close()


def scc_dimers(mons):
    """The real-pair dimers of the 64-acene FMO set-up (529 systems of 96-204 orbitals) with their
    starting densities, the block-diagonal densities of their monomers (tincr starts a pair SCC from
    its monomers' charges, src/fmo/scc/pair.rs:112-124)."""
    from tincr_gb300 import fmo
    from tincr_gb300 import groundstate as gs
    reach = 2.0 * max(fmo.VDW_SUM_BOHR.values())
    dims, starts = [], []
    for i, j in fmo.candidate_pairs(mons, reach):
        if not fmo.is_real_pair(mons[i], mons[j]):
            continue
        mi, mj = mons[i], mons[j]
        dims.append(gs.build_system(np.concatenate([mi.system.numbers, mj.system.numbers]),
                                    np.concatenate([mi.system.xyz, mj.system.xyz]), lc=True, r_lr=mi.system.r_lr))
        ni, nj = mi.system.n_orbs, mj.system.n_orbs
        p = np.zeros((ni + nj, ni + nj))
        p[:ni, :ni] = mi.ground.p
        p[ni:, ni:] = mj.ground.p
        starts.append(p)
    return dims, starts


def _scc_host_job(args):
    from tincr_gb300 import groundstate as gs
    sy, p = args
    return gs.run_scc(sy, tol=SCC_TOL, p_start=p).iterations


def _scc_gemm_flops(systems, grounds):
    """FP64 flops of the SCC's GEMMs per system and iteration (LC: 10 n^3 for the exchange
    Hamiltonian, 4 n^3 for X F X, 2 n^3 for F'P', 6 n^2 n_occ for the densities) over the iterations
    run, plus the start (X, S^1/2, P': 8 n^3) and the end (orbitals, density, LC energy: 6 n^3):
    the dense count (the kernel forms the symmetric products from their lower-triangle tiles)."""
    f = 0.0
    for sy, g in zip(systems, grounds):
        n, o = float(sy.n_orbs), float(sy.n_elec // 2)
        per = (10 * n ** 3 if sy.lc else 0.0) + 6 * n ** 3 + 6 * n * n * o
        f += g.iterations * per + 8 * n ** 3 + 6 * n ** 3
    return f


def scc_measure(ctx, mons, cpu_baseline=True, scc_set="all"):
    """Batched GPU SCC (tincr_scc_batch) on the 64-acene FMO set-up: the 64 monomers, then the 529
    real-pair dimers, in FP64 and with the FP32 start; device time (CUDA events around the kernel),
    wall time through the Python API (host packing and copies included), the FP64 GEMM rate against
    GB300's nominal FP64 peak (1.25 TFLOP/s: no FP64 figure is measured for this machine), agreement with
    the host SCC, and the host SCC on all host cores (process pool) as the CPU baseline."""
    from tincr_gb300 import fmo
    from tincr_gb300 import scc as gscc
    dims, starts = scc_dimers(mons)
    sets = [("monomers", [m.system for m in mons], None)]
    if scc_set == "all":
        sets.append(("dimers", dims, starts))
    gscc.scc_batch(ctx, sets[0][1], tol=SCC_TOL)   # warm-up: allocation of the slots
    out = {"metric": "batched SCC seconds", "tol": SCC_TOL}
    for name, systems, st in sets:
        for fp32 in (False, True):
            t0 = time.perf_counter()
            g, rc = gscc.scc_batch(ctx, systems, tol=SCC_TOL, p_start=st, fp32_start=fp32)
            wall = time.perf_counter() - t0
            ms = ctx.last_timing()[0]
            its = [x.iterations for x in g]
            rec = {"systems": len(systems), "n_orb": [min(s.n_orbs for s in systems), max(s.n_orbs for s in systems)],
                   "status": int(rc), "kernel_ms": ms, "wall_ms": 1e3 * wall, "iterations_mean": float(np.mean(its)),
                   "iterations_max": int(max(its)), "unconverged": int(sum(not x.converged for x in g))}
            if not fp32:
                fl = _scc_gemm_flops(systems, g)
                rec["fp64_gemm_tflop"] = fl / 1e12
                rec["fp64_gemm_tflops"] = fl / (ms * 1e-3) / 1e12
                rec["fp64_frac_of_nominal"] = rec["fp64_gemm_tflops"] / 1.25
            if name == "monomers":
                rec["max_abs_orbe_diff_vs_host"] = float(max(np.abs(x.orbe - m.ground.orbe).max()
                                                             for x, m in zip(g, mons)))
            out["%s_%s" % (name, "fp32start" if fp32 else "fp64")] = rec
    if cpu_baseline:
        # host SCC restatement on all host cores: the monomers in full, a bounded sample of dimers
        cores = os.cpu_count() or 1
        t0 = time.perf_counter()
        fmo._pool_map(_scc_host_job, [(m.system, None) for m in mons], cores)
        t_mon = time.perf_counter() - t0
        k = min(len(dims), 4 * cores)
        t0 = time.perf_counter()
        fmo._pool_map(_scc_host_job, list(zip(dims[:k], starts[:k])), cores)
        t_dim = (time.perf_counter() - t0) * len(dims) / k
        out["cpu_baseline"] = {"kind": "port", "cores": cores, "monomers_s": t_mon, "dimers_s": t_dim,
                               "sample": "host SCC (groundstate.run_scc, numpy) in a spawn pool of %d processes: "
                                         "all %d monomers; %d of %d dimers, scaled" % (cores, len(mons), k, len(dims))}
    return out


def run_scc_bench(args):
    """--mode scc: `scc_measure` on its own; prints one JSON line."""
    from tincr_gb300 import _lib, build
    build.build()
    mons, pairs, inst, labels = fmo_workload()
    ctx = _lib.Context(0)
    out = {"mode": "scc"}
    out.update(scc_measure(ctx, mons, args.cpu_baseline, args.scc_set))
    print(json.dumps(out))
    ctx.close()


def rpa_measure(ctx, sy, g):
    """RPA / Casida (tincr_rpa_solve, FP64) on the (H2O)128 LC workload: the lowest N_ROOTS roots to
    the bench residual, timed with CUDA events, beside the FP64 TDA solve of the same roots."""
    from tincr_gb300 import _lib
    from tincr_gb300 import tda as T
    es = T.ExcitedStateSystem.from_ground_state(ctx, sy, g)
    es.prepare_tda()
    out = {"workload": "water128-lc-20roots", "tol": TOL}
    r = es.run_rpa(N_ROOTS, MAX_ITER, TOL)
    out["rpa_ms"] = ctx.last_timing()[0]
    out["rpa_iterations"] = int(r["rpa_iterations"])
    r = es.run_tda(N_ROOTS, MAX_ITER, TOL, precision=_lib.PREC_FP64)
    out["tda_fp64_ms"] = ctx.last_timing()[0]
    out["tda_iterations"] = int(r["davidson_iterations"])
    d = es.properties["rpa_eigenvalues"] - r["ci_eigenvalues"]
    out["rpa_minus_tda_eh"] = {"min": float(d.min()), "max": float(d.max())}
    return out


def run_rpa_bench(args):
    """--mode rpa: `rpa_measure` on its own; prints one JSON line."""
    from tincr_gb300 import _lib, build
    build.build()
    sy, g = workload()
    ctx = _lib.Context(0)
    out = {"mode": "rpa"}
    out.update(rpa_measure(ctx, sy, g))
    print(json.dumps(out))
    ctx.close()


def _scc_energy_job(sy):
    from tincr_gb300 import groundstate as gs
    return gs.run_scc(sy, tol=1e-11).energy


def fd_measure(ctx):
    """Numerical S1 gradient of decacene (C42H24, LC, all 198 coordinates, +-1e-4 bohr; tincr's
    gradients/numerical.rs check): the 396 displaced SCCs as one batched GPU SCC, then each
    geometry's TDA (3 roots, FP64) on the GPU; the host SCC of a sample of the displaced geometries
    on all host cores beside it, and the largest difference from the analytic exact-variant gradient."""
    from tincr_gb300 import fmo
    from tincr_gb300 import geometry as G
    from tincr_gb300 import gradients as GR
    from tincr_gb300 import groundstate as gs
    from tincr_gb300 import numerical as NUM
    from tincr_gb300 import scc as gscc
    from tincr_gb300 import tda as T
    z, x = G.acene(10)
    sy = gs.build_system(z, G.to_bohr(x), lc=True)
    g = gs.run_scc(sy, tol=1e-11)
    systems, _ = NUM._displaced(sy, range(sy.xyz.size), [1e-4])
    t0 = time.perf_counter()
    gscc.scc_batch(ctx, systems, tol=1e-11, require_convergence=True)
    scc_wall = time.perf_counter() - t0
    scc_ms = ctx.last_timing()[0]
    t0 = time.perf_counter()
    _, fd = NUM.fd_gradient(ctx, sy, n_roots=1, h=1e-4)
    fd_wall = time.perf_counter() - t0
    es = T.ExcitedStateSystem.from_ground_state(ctx, sy, g)
    es.run_tda(3, 450, 1e-8)
    ana = GR.GradientSystem(es, sy, g).tda_gradient(0, "exact")
    cores = os.cpu_count() or 1
    k = min(len(systems), 2 * cores)
    t0 = time.perf_counter()
    fmo._pool_map(_scc_energy_job, systems[:k], cores)
    host_scc = (time.perf_counter() - t0) * len(systems) / k
    return {"workload": "decacene-lc-s1-fd-198coords", "displaced_sccs": len(systems),
            "scc_batch_kernel_ms": scc_ms, "scc_batch_wall_s": scc_wall, "fd_gradient_wall_s": fd_wall,
            "max_abs_fd_minus_analytic_eh_per_bohr": float(np.abs(fd[0] - ana).max()),
            "cpu_baseline": {"kind": "port", "cores": cores, "displaced_sccs_s": host_scc,
                             "sample": "host SCC (groundstate.run_scc) of %d of the %d displaced geometries in a "
                                       "spawn pool of %d processes, scaled" % (k, len(systems), cores)}}


def _guarded(fn):
    """The result of fn(), or the error it raised (the extra measurements must not cost the main line)."""
    try:
        return fn()
    except Exception as e:   # reported in the JSON line, not hidden
        return {"error": "%s: %s" % (type(e).__name__, e)}


def fmo512_workload(workers, scc="host", ctx=None):
    """512-acene FMO aggregate: the 64-acene recipe on an 8 x 8 x 8 lattice (13812 atoms); monomer
    SCCs on the host (a process pool) or as one batched GPU SCC (scc="gpu")."""
    from tincr_gb300 import fmo
    from tincr_gb300 import geometry as G
    from tincr_gb300 import groundstate as gs
    z, x, mono = G.acene_lattice(8, 8, 8)
    mons = fmo.build_monomers(z, G.to_bohr(x), mono, lc=True, workers=workers, scc=scc, ctx=ctx)
    pairs = fmo.close_pairs(mons, 4.5 / gs.P.BOHR_TO_ANGS)
    inst, labels = fmo.aggregate_instances(mons, pairs, FMO_N_LE, FMO_N_CT)
    return mons, pairs, inst, labels


def acene512_parity(mons, setup, inst, labels, r64, rmx, h64, hmx, e64, emx, n_sample=32, n_elem=100, seed=512):
    """Sampled checks of the 512-acene step against the oracle (too large for it in full):
    the TDA of n_sample random instances (oracle engines); n_elem random matrix elements of each kind
    (LE-LE, LE-CT, CT-CT) among those that carry an exchange term, plus n_elem random pairs of
    states, from the oracle couplings (LCMO Fock block by block) on the GPU roots of the same form;
    the lowest roots of the GPU FP64 matrix by dense diagonalisation against the GPU Davidson's."""
    cases, OG, OT = _cpu_helpers()
    from oracle import exciton as OX
    rng = np.random.default_rng(seed)
    out = {}
    case = dict(monomers=mons, labels=labels, lc=True)
    n_mon = len(mons)
    pick = np.concatenate([rng.choice(n_mon, n_sample // 4, replace=False),
                           n_mon + rng.choice(len(inst) - n_mon, n_sample - n_sample // 4, replace=False)])
    d64, dmx = 0.0, 0.0
    for k in pick:
        eng, xyz = cases.fmo_oracle_engine(case, int(k))
        r = OT.run_tda_engine(eng, xyz, inst[k]["n_roots"], FMO_MAX_ITER, FMO_TOL)
        d64 = max(d64, float(np.abs(r64[k]["energies"] - r["energies"]).max()))
        dmx = max(dmx, float(np.abs(rmx[k]["energies"] - r["energies"]).max()))
    out["tda_sample"] = {"instances": int(len(pick)), "fp64_max_energy_err_eh": d64, "mixed_max_energy_err_eh": dmx}
    agg = OX.aggregate_of(mons, setup)
    states = OX.basis_of(agg, labels, r64, setup.ct_pairs, FMO_N_LE, FMO_N_CT)
    # the mixed matrix is built from the mixed roots: near-degenerate roots of an instance can come
    # out as another rotation of the same subspace, so its elements are checked on those roots
    states_mx = OX.basis_of(agg, labels, rmx, setup.ct_pairs, FMO_N_LE, FMO_N_CT)
    fb = OX.LcmoFockBlocks(agg)
    near = lambda a, b: a == b or agg.type_of_pair(a, b) == "pair"
    le = [i for i, st in enumerate(states) if isinstance(st, OX.LE)]
    ct = [i for i, st in enumerate(states) if isinstance(st, OX.CT)]
    mon = lambda st: (st.m,) if isinstance(st, OX.LE) else (st.m_h, st.m_l)
    chosen = {"le_le": [], "le_ct": [], "ct_ct": [], "any": []}
    tries = 0
    while min(len(v) for v in chosen.values()) < n_elem and tries < 200000:
        tries += 1
        i, j = (int(v) for v in rng.choice(len(states), 2, replace=False))
        a, b = states[i], states[j]
        if len(chosen["any"]) < n_elem:
            chosen["any"].append((i, j))
        if isinstance(a, OX.LE) and isinstance(b, OX.LE):
            kind, ok = "le_le", a.m != b.m and near(a.m, b.m)
        elif isinstance(a, OX.LE) or isinstance(b, OX.LE):
            L, C = (a, b) if isinstance(a, OX.LE) else (b, a)
            kind, ok = "le_ct", near(L.m, C.m_h) or near(L.m, C.m_l)
        else:
            kind, ok = "ct_ct", mon(a) != mon(b) and near(a.m_h, b.m_h) and near(a.m_l, b.m_l)
        if ok and len(chosen[kind]) < n_elem:
            chosen[kind].append((i, j))
    # targeted draws for kinds that random pairs rarely hit
    for _ in range(20 * n_elem):
        if len(chosen["le_le"]) >= n_elem:
            break
        i = int(rng.choice(le))
        nb = [j for j in le if states[j].m != states[i].m and near(states[j].m, states[i].m)]
        if nb:
            chosen["le_le"].append((i, int(rng.choice(nb))))
    for _ in range(20 * n_elem):
        if len(chosen["ct_ct"]) >= n_elem:
            break
        i = int(rng.choice(ct))
        nb = [j for j in ct if mon(states[j]) != mon(states[i]) and near(states[j].m_h, states[i].m_h)
              and near(states[j].m_l, states[i].m_l)]
        if nb:
            chosen["ct_ct"].append((i, int(rng.choice(nb))))
    el = {}
    for kind, pairs_ in chosen.items():
        e64k, emxk = 0.0, 0.0
        for i, j in pairs_:
            e64k = max(e64k, abs(h64[i, j] - OX.exciton_coupling(agg, fb, None, states[i], states[j])))
            emxk = max(emxk, abs(hmx[i, j] - OX.exciton_coupling(agg, fb, None, states_mx[i], states_mx[j])))
        el[kind] = {"elements": len(pairs_), "fp64_max_err_eh": e64k, "mixed_max_err_eh": emxk}
    out["matrix_sample"] = el
    w = np.linalg.eigvalsh(h64)[:FMO_N_EXCITON]
    out["roots"] = {"dense_eigenvalues_of_gpu_fp64_matrix_eh": [float(x) for x in w],
                    "fp64_davidson_max_err_eh": float(np.abs(e64 - w).max()),
                    "mixed_davidson_max_err_eh": float(np.abs(emx - w).max())}
    return out


def run_fmo512(args):
    """--mode acene512: the 512-acene aggregate once per form (batched TDA of the work list, the
    exciton Hamiltonian and its lowest 10 states, the gradient of the lowest exciton state with its
    LE and CT terms), with sampled oracle checks (`acene512_parity`).  Prints one JSON line."""
    from tincr_gb300 import _lib, build
    from tincr_gb300 import fmo
    build.build()
    workers = os.cpu_count() or 1
    ctx = _lib.Context(0)
    t0 = time.perf_counter()
    mons, pairs, inst, labels = fmo512_workload(workers, scc=args.setup_scc, ctx=ctx)
    t_w = time.perf_counter() - t0
    t0 = time.perf_counter()
    # the 8 x 8 x 8 lattice puts some acenes into each other (H-H contacts down to 0.2 A); the SCC of
    # 5-8 of those dimers has no stable stationary point, and they take the isolated monomers' orbitals
    setup = fmo.ExcitonSetup(mons, pairs, workers=workers, unconverged="isolated", scc=args.setup_scc, ctx=ctx)
    t_s = time.perf_counter() - t0
    gctxs = [_lib.Context(0) for _ in range(8)]
    n_mon = len(mons)
    out = {"mode": "acene512", "workload": "acene512-fmo-le4-ct1-exciton10", "monomers": n_mon,
           "atoms": int(sum(m.system.n_atoms for m in mons)), "ct_pairs": len(pairs), "instances": len(inst),
           "real_pairs": len(setup.real_pairs), "dimers_without_scc_solution": [list(k) for k in setup.unconverged_pairs],
           "setup_scc": args.setup_scc, "host_setup_s": t_w, "host_exciton_setup_s": t_s}
    runs = {}
    pst = None   # dimer ground states of the CT gradient terms, shared by both forms
    for name, prec in (("bf16x3", _lib.PREC_BF16X3), ("fp64", _lib.PREC_FP64)):
        fmo.solve_batch(ctx, inst, FMO_MAX_ITER, FMO_TOL, prec)   # warm-up (tile autotuner, graphs)
        t0 = time.perf_counter()
        rc, r = fmo.solve_batch(ctx, inst, FMO_MAX_ITER, FMO_TOL, prec)
        t_b = ctx.last_timing()[0]
        ex = fmo.exciton_states(ctx, setup, r, labels, FMO_N_LE, FMO_N_CT, n_roots=FMO_N_EXCITON, tol=FMO_EX_TOL,
                                max_iter=FMO_EX_MAX_ITER, precision=prec)
        t_e = ctx.last_timing()[0]
        g_err = None
        tg0 = time.perf_counter()
        try:   # LE and CT terms; the CT terms' dimer SCCs run inside (batched GPU SCC)
            g, n_le_t, n_ct_t, pst = fmo.exciton_gradient(ctx, setup, r, labels, FMO_N_LE, FMO_N_CT,
                                                          ex["vectors"][:, 0], contexts=gctxs, precision=prec,
                                                          pair_states=pst)
        except RuntimeError as e:   # a CT term on a dimer without an SCC solution: LE terms only
            g_err = str(e)
            g, n_le_t, n_ct_t = fmo.exciton_le_gradient(mons, r, ex["vectors"][:, 0], FMO_N_LE,
                                                        n_ct_states=len(ex["vectors"]) - n_mon * FMO_N_LE,
                                                        contexts=gctxs, precision=prec)
        t_g = time.perf_counter() - tg0
        wall = time.perf_counter() - t0
        # the matrix itself (473 MB) for the checks, outside the timed calls
        ex["matrix"] = fmo.exciton_states(ctx, setup, r, labels, FMO_N_LE, FMO_N_CT, n_roots=FMO_N_EXCITON,
                                          tol=FMO_EX_TOL, max_iter=FMO_EX_MAX_ITER, precision=prec,
                                          want_matrix=True)["matrix"]
        runs[name] = (rc, r, ex, g)
        out[name] = {"batch_tda_ms": t_b, "exciton_ms": t_e, "wall_s": wall, "status_ok": rc == _lib.OK,
                     "exciton_states": int(len(ex["vectors"])), "exciton_iterations": int(ex["iterations"]),
                     "exciton_energies_eh": [float(e) for e in ex["energies"]],
                     "lowest_state_le_gradient_terms": n_le_t, "lowest_state_ct_gradient_terms": n_ct_t,
                     "exciton_gradient_norm": float(np.linalg.norm(g)), "exciton_gradient_s": t_g,
                     "dimer_scc_pairs": len(pst or {})}
        if g_err is not None:
            out[name]["exciton_gradient_error"] = g_err
    for c in gctxs:
        c.close()
    ctx.close()
    (_, r64, ex64, g64), (_, rmx, exmx, gmx) = runs["fp64"], runs["bf16x3"]
    out["mixed_vs_fp64"] = {
        "max_instance_energy_err_eh": float(max(np.abs(a["energies"] - b["energies"]).max() for a, b in zip(rmx, r64))),
        "max_exciton_energy_err_eh": float(np.abs(exmx["energies"] - ex64["energies"]).max()),
        "max_exciton_gradient_err_eh_per_bohr": float(np.abs(gmx - g64).max()),
        "speedup_batch_plus_exciton": (out["fp64"]["batch_tda_ms"] + out["fp64"]["exciton_ms"]) /
                                      (out["bf16x3"]["batch_tda_ms"] + out["bf16x3"]["exciton_ms"])}
    t0 = time.perf_counter()
    out["parity"] = acene512_parity(mons, setup, inst, labels, r64, rmx, ex64["matrix"], exmx["matrix"],
                                    ex64["energies"], exmx["energies"])
    out["parity"]["oracle_s"] = time.perf_counter() - t0
    print(json.dumps(out))


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
    prec = PRECISIONS[args.precision]
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
    ap.add_argument("--precision", default="bf16x3", choices=sorted(PRECISIONS))
    ap.add_argument("--no-compare-fp64", dest="compare_fp64", action="store_false")
    ap.add_argument("--no-fmo", dest="fmo", action="store_false")
    ap.add_argument("--no-next-rows", dest="next_rows", action="store_false",
                    help="skip the batched SCC and RPA measurements of the single-GPU run")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    # counts of the step a `--mode cpu-sample` child scales its sample to (passed by the GPU arm)
    ap.add_argument("--ref-products", type=int, default=None)
    ap.add_argument("--ref-iters", type=int, default=None)
    ap.add_argument("--ref-cg", type=int, default=None)
    ap.add_argument("--mode", default="solve",
                    choices=["solve", "products", "fmo", "fmo-exciton", "fmo-exgrad", "cpu-sample", "acene512", "scc",
                             "rpa"])
    ap.add_argument("--scc-set", default="all", choices=["all", "monomers"])
    ap.add_argument("--setup-scc", default="host", choices=["host", "gpu"],
                    help="--mode acene512: SCCs of the set-up on the host (process pool) or batched on the GPU")
    ap.add_argument("--k", type=int, default=4)
    args = ap.parse_args()
    if args.mode == "products":
        run_products(args)
        return
    if args.mode == "fmo":
        run_fmo_once(args)
        return
    if args.mode == "acene512":
        run_fmo512(args)
        return
    if args.mode == "fmo-exciton":
        run_fmo_exciton_once(args)
        return
    if args.mode == "fmo-exgrad":
        run_fmo_exgrad_once(args)
        return
    if args.mode == "scc":
        run_scc_bench(args)
        return
    if args.mode == "rpa":
        run_rpa_bench(args)
        return
    if args.mode == "cpu-sample":
        if None in (args.ref_products, args.ref_iters, args.ref_cg):
            ap.error("--mode cpu-sample needs --ref-products, --ref-iters and --ref-cg")
        run_cpu_sample(args)
        return
    out = run_reference(args) if args.impl == "reference" else run_gpu(args)
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
