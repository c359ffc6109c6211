"""Oracle results on the two benchmark workloads, saved as fixtures for the GPU parity tests.

    python tests/golden/make_bench_fixtures.py [water128] [acene64]

Both workloads are the seeded synthetic systems `bench.py` times (`bench.workload`,
`bench.fmo_workload`), with the host SCC ground state.  The oracle (numpy restatement of tincr) runs
on this machine's CPU, once:

* water128.npz: (H2O)128 LC-TDA (768 orbitals, 512 x 256, R_lr = 1/0.3 bohr), the lowest 20 roots
  converged to residual 1e-6 (max_iter 450): per-root energies, oscillator strengths,
  transition-dipole norms, Davidson iterations and products (tincr's `System::run_tda`,
  src/excited_states/tda/mod.rs:74-131).  The Davidson takes its corrections through two
  Gram-Schmidt passes: with tincr's single pass the restated solve loses the orthogonality of its
  basis after the subspace collapse and returns spurious near-zero roots on this cluster (see
  oracle.tda.davidson), so the reference roots are the converged eigenpairs, which any correct
  solver approaches whatever its history.  Then the S1 ground-state and excitation
  gradients of tincr's formulas (src/gradients/ground_state.rs:12-137,
  src/gradients/excited_state.rs:56-487), evaluated atom by atom; and the S1 CI vector in a
  sign-canonical MO basis (every MO column's largest-magnitude AO coefficient positive), so that a
  test can install the oracle's root on a ground state whose eigenvector signs came out otherwise.
  The orbital energies are stored as an input check.
* acene64.npz: the 64-acene FMO work list (64 monomers x 4 LE roots, both directions of the 284
  pairs closer than 4.5 A x 1 CT root; tolerance 1e-4, max_iter 150): per-instance energies,
  oscillator strengths and Davidson iterations of the oracle engines (`TdaEngine` for a monomer,
  `CtEngine` for a pair direction: src/excited_states/solvers/mod.rs:59-269, davidson.rs:53-185),
  the excitation gradient of the lowest LE root of the aggregate (tincr's
  `Monomer::tda_gradient_lc`, src/fmo/gradients/excited_state.rs:299-542), and the lowest 10
  roots of the exciton Hamiltonian over those LE / CT states (oracle.exciton: LCMO Fock matrix,
  couplings, tincr's Davidson at tolerance 1e-4 and 100 iterations, src/fmo/lcmo/basis.rs:449-503),
  with the host set-up of the pair types, overlaps, gamma matrices and dimer ground states
  (`fmo.ExcitonSetup`).  Monomer orbital energies are stored as an input check.
"""

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))


# residual tolerance of the water reference roots: converged far below the bench's 1e-4, so that the
# Ritz values are the eigenvalues to ~1e-11 Eh whatever history a solver takes to them
WATER_TOL = 1e-6


def canonical_signs(c):
    """+1/-1 per MO column: the sign of the column's largest-magnitude coefficient."""
    idx = np.argmax(np.abs(c), axis=0)
    return np.sign(c[idx, np.arange(c.shape[1])])


def water128():
    import bench
    from cases import oracle_gradient_inputs
    from oracle import gradients as OG
    from oracle import tda as OT
    sy, g = bench.workload()
    occ, virt = sy.occ_indices, sy.virt_indices
    t0 = time.perf_counter()
    q = OT.trans_charges(sy.ao_offset, g.orbs, g.s, occ, virt)
    om = OT.orbe_differences(g.orbe[occ], g.orbe[virt])
    res = OT.run_tda(om, q[0], g.gamma, sy.xyz, bench.N_ROOTS, bench.MAX_ITER, WATER_TOL, q_oo=q[1], q_vv=q[2],
                     gamma_lr=g.gamma_lr, n_occ=sy.n_occ, n_virt=sy.n_virt, reorthogonalize=True)
    t_tda = time.perf_counter() - t0
    print("water128 TDA: %d iterations, %d products, %.1f s" % (res["iterations"], res["n_products"], t_tda))
    t0 = time.perf_counter()
    inp = oracle_gradient_inputs(sy, g, True, res["energies"], res["coefficients"], q)
    del q
    rows = OG.AtomRows(sy.numbers, sy.xyz, sy.ao_offset, sy.ao_atom, sy.hubbard, sy.r_lr, sy.params)
    ggs, gex = OG.gradients_by_atom(inp, rows, 0, True)
    t_grad = time.perf_counter() - t0
    print("water128 S1 gradient: %.1f s, |g| = %.6f" % (t_grad, np.abs(ggs + gex).max()))
    sg = canonical_signs(g.orbs)
    x1 = res["coefficients"][:, 0].reshape(sy.n_occ, sy.n_virt)
    x1c = sg[occ][:, None] * sg[virt][None, :] * x1
    np.savez_compressed(os.path.join(HERE, "water128.npz"),
                        orbe=g.orbe, energies=res["energies"], f=res["f"],
                        tr_dipole_norms=np.linalg.norm(res["tr_dipoles"], axis=0),
                        iterations=res["iterations"], n_products=res["n_products"],
                        grad_ground=ggs, grad_excited=gex, s1_vector_canonical=x1c.reshape(-1),
                        n_roots=bench.N_ROOTS, tol=WATER_TOL, max_iter=bench.MAX_ITER,
                        oracle_seconds=np.array([t_tda, t_grad]))


def acene64():
    import bench
    from cases import fmo_oracle_engine, oracle_gradient_inputs
    from oracle import gradients as OG
    from oracle import tda as OT
    from oracle import exciton as OX
    from tincr_gb300 import fmo
    mons, pairs, inst, labels = bench.fmo_workload()
    t0 = time.perf_counter()
    e, f, its, nr, res = [], [], [], [], []
    case = dict(monomers=mons, labels=labels, lc=True)
    for k, q in enumerate(inst):
        eng, _ = fmo_oracle_engine(case, k)
        r = OT.run_tda_engine(eng, q["xyz"], q["n_roots"], bench.FMO_MAX_ITER, bench.FMO_TOL)
        e.append(r["energies"])
        f.append(r["f"])
        its.append(r["iterations"])
        nr.append(q["n_roots"])
        res.append(r)
    t_tda = time.perf_counter() - t0
    setup = fmo.ExcitonSetup(mons, pairs, workers=os.cpu_count() or 1)
    t0 = time.perf_counter()
    agg = OX.aggregate_of(mons, setup)
    states = OX.basis_of(agg, labels, res, setup.ct_pairs, bench.FMO_N_LE, bench.FMO_N_CT)
    h = OX.exciton_hamiltonian_rows(agg, states, os.cpu_count() or 1)
    ex_e, _, ex_it = OX.exciton_states(h, bench.FMO_N_EXCITON, bench.FMO_EX_TOL, bench.FMO_EX_MAX_ITER)
    t_ex = time.perf_counter() - t0
    print("acene64 exciton: %d states, %d Davidson iterations, %.1f s, lowest %.8f Eh"
          % (len(states), ex_it, t_ex, ex_e[0]))
    n_mon = len(mons)
    k1 = int(np.argmin([e[k][0] for k in range(n_mon)]))
    m = mons[k1]
    sy, g = m.system, m.ground
    t0 = time.perf_counter()
    q = OT.trans_charges(sy.ao_offset, g.orbs, g.s, sy.occ_indices, sy.virt_indices)
    om = OT.orbe_differences(g.orbe[sy.occ_indices], g.orbe[sy.virt_indices])
    eng = OT.TdaEngine(om, q[0], g.gamma, q[1], q[2], g.gamma_lr, sy.n_occ, sy.n_virt)
    r = OT.run_tda_engine(eng, sy.xyz, bench.FMO_N_LE, bench.FMO_MAX_ITER, bench.FMO_TOL)
    inp = oracle_gradient_inputs(sy, g, True, r["energies"], r["coefficients"], q)
    der = OG.derivative_tensors(sy.numbers, sy.xyz, sy.ao_offset, sy.ao_atom, sy.hubbard, sy.r_lr, sy.params)
    _, flr = OG.ground_state_gradient(inp, der, True)
    gex = OG.tda_gradient(inp, der, 0, True, flr_dmd0=flr)
    t_grad = time.perf_counter() - t0
    print("acene64: %d instances in %.1f s, S1 monomer %d, LE gradient %.2f s"
          % (len(inst), t_tda, k1, t_grad))
    np.savez_compressed(os.path.join(HERE, "acene64.npz"),
                        energies=np.concatenate(e), f=np.concatenate(f), iterations=np.array(its),
                        n_roots=np.array(nr), kinds=np.array([0 if l[0] == "LE" else 1 for l in labels]),
                        monomer_orbe=np.concatenate([mm.ground.orbe for mm in mons]),
                        s1_monomer=k1, s1_le_gradient=gex, tol=bench.FMO_TOL, max_iter=bench.FMO_MAX_ITER,
                        exciton_energies=ex_e, exciton_iterations=ex_it, exciton_dim=len(states),
                        oracle_seconds=np.array([t_tda, t_grad, t_ex]))


if __name__ == "__main__":
    which = sys.argv[1:] or ["water128", "acene64"]
    for w in which:
        {"water128": water128, "acene64": acene64}[w]()
    print("bench fixtures written to", HERE)
