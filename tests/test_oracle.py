"""CPU tests: the oracle pinned against tincr's golden data and known answers, and the formulas
the GPU path relies on.  No GPU needed."""

import numpy as np
import pytest

from cases import FIXTURE_BOHR, fixture_case, golden, oracle_inputs, synthetic_case
from oracle import gradients as OG
from oracle import slako as OS
from oracle import tda as OT
from tincr_gb300 import groundstate as gs
from tincr_gb300.params import NUMBERS

MOLS = ["h2o", "ammonia", "benzene", "uracil"]


def _fixture_system(mol):
    d = golden(mol)
    nums = [NUMBERS[s] for s in d["symbols"]]
    sy = gs.build_system(nums, d["xyz_angstrom"] / FIXTURE_BOHR, lc=True)
    # the fixtures were produced with an older parameter set: take Hubbard U from their gamma diagonal
    sy.hubbard = np.diag(d["gamma_atomwise"]).copy()
    return d, sy


@pytest.mark.parametrize("mol", MOLS + ["h2"])
def test_gamma_matches_fixtures(mol):
    """gamma, gamma_lr (R_lr = 3.03) and their AO expansions (gamma_approximation.rs tests, 1e-15)."""
    d, sy = _fixture_system(mol)
    assert np.abs(gs.gamma_atomwise(sy, 0.0) - d["gamma_atomwise"]).max() < 1e-15
    assert np.abs(gs.gamma_atomwise(sy, 3.03) - d["gamma_atomwise_lc"]).max() < 1e-15
    assert np.abs(gs.atom_to_ao(sy, d["gamma_atomwise"]) - d["gamma_ao_wise"]).max() < 1e-15
    assert np.abs(gs.atom_to_ao(sy, d["gamma_atomwise_lc"]) - d["gamma_ao_wise_lc"]).max() < 1e-15


@pytest.mark.parametrize("mol", MOLS)
def test_gamma_gradients_match_fixtures(mol):
    """d gamma / dR atomwise [3N, N, N] and AO-wise [3N, n, n] (gamma_approximation.rs:256-454)."""
    d, sy = _fixture_system(mol)
    n = sy.n_atoms
    for r_lr, suffix in ((0.0, ""), (3.03, "_lc")):
        g1 = OG.gamma_gradients_atomwise(sy.xyz, OG.gamma_c(sy.hubbard, r_lr))
        ref = d["gamma_atomwise_grad" + suffix].reshape(3 * n, n, n)
        assert np.abs(g1 - ref).max() < 1e-14
        g1ao = OG.gamma_gradients_ao(g1, sy.ao_atom)
        ref_ao = d["gamma_ao_wise_grad" + suffix].reshape(3 * n, sy.n_orbs, sy.n_orbs)
        assert np.abs(g1ao - ref_ao).max() < 1e-14


def test_tda_known_answer_water():
    """Water LC-TDA from explicit S, orbital energies and C (not_refactored_tests/solver.rs:32-198, 1e-10)."""
    k = golden("kat_excited_energies_tda_routine")
    sy = gs.build_system([8, 1, 1], k["positions"] / FIXTURE_BOHR, lc=True)
    sy.hubbard = np.array([0.4467609798860577, 0.47201583989641355, 0.47201583989641355])
    g, glr = gs.gamma_atomwise(sy, 0.0), gs.gamma_atomwise(sy, 3.03)
    occ, virt = np.arange(4), np.arange(4, 6)
    qov, qoo, qvv = OT.trans_charges(sy.ao_offset, k["orbs"], k["S"], occ, virt)
    om = OT.orbe_differences(k["orbe"][:4], k["orbe"][4:])
    a = OT.tda_full_matrix(om, qov, g, qoo, qvv, glr, 4, 2)
    assert np.abs(np.linalg.eigvalsh(a) - k["omega_ref_out"]).max() < 1e-10
    # the Davidson solver on all 8 roots reproduces the same energies
    eng = OT.TdaEngine(om, qov, g, qoo, qvv, glr, 4, 2)
    e, x, _ = OT.davidson(eng, OT.initial_subspace(om, 8), 8, 1e-10, 50)
    assert np.abs(e - k["omega_ref_out"]).max() < 1e-10


def test_tda_known_answer_2x2():
    """2x2 active-space LC-TDA from explicit gamma, gamma_lr and q's (solver.rs:887-1005, 1e-14)."""
    t = golden("kat_tda_routine")
    qov, qoo, qvv = (t[k].reshape(3, -1) for k in ("q_trans_ov", "q_trans_oo", "q_trans_vv"))
    a = OT.tda_full_matrix(t["omega_0"].reshape(-1), qov, t["gamma"], qoo, qvv, t["gamma_lr"], 2, 2)
    e, v = np.linalg.eigh(a)
    assert np.abs(e - t["omega_ref"]).max() < 1e-14
    # eigenvectors up to sign: tincr stores c_ij [state, i, a]
    ref = t["c_ij_ref"].reshape(4, 4)
    assert np.abs(np.abs(np.einsum("ks,sk->s", ref, v)) - 1.0).max() < 1e-12


@pytest.mark.parametrize("mol", ["h2o", "benzene", "uracil"])
@pytest.mark.parametrize("lc", [True, False])
def test_davidson_matches_dense(mol, lc):
    """Davidson roots are eigenvalues of the dense CIS matrix (tincr's tda/system.rs:105-159 check).

    With tincr's unit-vector guess (solvers/utils.rs:17-26) a root whose symmetry has no overlap
    with the guess space is never reached (benzene, D6h), so the check is that every converged root
    is an exact eigenvalue, and that the lowest root is the true lowest one."""
    c = fixture_case(mol, lc)
    o = oracle_inputs(c)
    nr = min(4, c["n_occ"] * c["n_virt"])
    res = OT.run_tda(o["omega"], o["q_ov"], o["gamma"], c["xyz"], nr, 100, 1e-8, o["q_oo"], o["q_vv"],
                     o["gamma_lr"], o["n_occ"], o["n_virt"])
    a = OT.tda_full_matrix(o["omega"], o["q_ov"], o["gamma"], o["q_oo"], o["q_vv"], o["gamma_lr"],
                           o["n_occ"], o["n_virt"])
    dense = np.linalg.eigvalsh(a)
    assert max(np.abs(dense - e).min() for e in res["energies"]) < 1e-10
    assert abs(res["energies"][0] - dense[0]) < 1e-10


def test_ao_direct_products_equal_reference_form():
    """The AO-basis factorisation used by the GPU path equals tincr's q-based A.X
    (solvers/mod.rs:280-369) on uracil with long-range correction."""
    c = fixture_case("uracil", lc=True)
    o = oracle_inputs(c)
    eng = OT.TdaEngine(o["omega"], o["q_ov"], o["gamma"], o["q_oo"], o["q_vv"], o["gamma_lr"], o["n_occ"], o["n_virt"])
    rng = np.random.default_rng(3)
    x = rng.standard_normal((c["n_occ"] * c["n_virt"], 3))
    ref = eng.apply(x)
    n, no, nv = c["orbs"].shape[0], c["n_occ"], c["n_virt"]
    C = c["orbs"]
    sc = c["s"] @ C
    ao_atom = np.repeat(np.arange(len(c["opa"])), c["opa"])
    glr = c["gamma_lr"][np.ix_(ao_atom, ao_atom)]
    lst = np.concatenate([C[:, :no], sc[:, :no]])
    rv = np.concatenate([C[:, no:], sc[:, no:]])
    lsw = np.concatenate([sc[:, :no], C[:, :no]])
    rsw = np.concatenate([sc[:, no:], C[:, no:]])
    out = np.zeros_like(ref)
    idx = np.arange(n)
    for b in range(x.shape[1]):
        xb = x[:, b].reshape(no, nv)
        m = (lst @ xb) @ rv.T
        y = np.bincount(ao_atom, weights=0.5 * (m[idx, n + idx] + m[n + idx, idx]))
        z = (c["gamma"] @ y)[ao_atom]
        f = -0.25 * np.tile(glr, (2, 2)) * m
        f[idx, n + idx] += z
        f[n + idx, idx] += z
        out[:, b] = (lsw.T @ f @ rsw + o["omega"].reshape(no, nv) * xb).reshape(-1)
    assert np.abs(out - ref).max() < 1e-13 * np.abs(ref).max()


def test_sk_overlap_angular_structure_vs_fixture():
    """Orbital order (s, p_y, p_z, p_x) and the s-p rule S = u_m V_sp on tincr's benzene S fixture:
    for each H-C pair the three p elements are proportional to the direction cosines."""
    d = golden("benzene")
    sy = gs.system_from_symbols(list(d["symbols"]), d["xyz_angstrom"])
    S = d["S"]
    checked = 0
    for h in np.where(sy.numbers == 1)[0]:
        for c in np.where(sy.numbers == 6)[0]:
            u = sy.xyz[c] - sy.xyz[h]
            u /= np.linalg.norm(u)
            p = S[sy.ao_offset[h], sy.ao_offset[c] + 1:sy.ao_offset[c] + 4]   # (y, z, x)
            v = p / np.array([u[1], u[2], u[0]])
            finite = np.abs(np.array([u[1], u[2], u[0]])) > 1e-3
            if finite.sum() >= 2:
                assert np.ptp(v[finite]) < 1e-8 * max(1.0, np.abs(v[finite]).max())
                checked += 1
    assert checked > 10


def test_sk_host_and_oracle_agree_and_gradients_match_fd():
    d = golden("uracil")
    sy = gs.system_from_symbols(list(d["symbols"]), d["xyz_angstrom"])
    S, H = gs.h0_and_s(sy)
    S2, H2 = OS.h0_and_s(sy.numbers, sy.xyz, sy.ao_offset, sy.ao_energy, sy.params)
    assert np.abs(S - S2).max() < 1e-15 and np.abs(H - H2).max() < 1e-15
    gS, gH = OS.h0_and_s_gradients(sy.numbers, sy.xyz, sy.ao_offset, sy.params, orientation="index")
    h = 1e-5
    for c in range(0, 3 * sy.n_atoms, 5):
        xp, xm = sy.xyz.copy(), sy.xyz.copy()
        xp[c // 3, c % 3] += h
        xm[c // 3, c % 3] -= h
        Sp, Hp = OS.h0_and_s(sy.numbers, xp, sy.ao_offset, sy.ao_energy, sy.params)
        Sm, Hm = OS.h0_and_s(sy.numbers, xm, sy.ao_offset, sy.ao_energy, sy.params)
        assert np.abs((Sp - Sm) / (2 * h) - gS[c]).max() < 1e-8
        assert np.abs((Hp - Hm) / (2 * h) - gH[c]).max() < 1e-8


def _exc_energy(numbers, xyz, lc, state=0):
    sy = gs.build_system(numbers, xyz, lc=lc)
    g = gs.run_scc(sy, tol=1e-11)
    occ, virt = sy.occ_indices, sy.virt_indices
    qov, qoo, qvv = OT.trans_charges(sy.ao_offset, g.orbs, g.s, occ, virt)
    om = OT.orbe_differences(g.orbe[occ], g.orbe[virt])
    a = OT.tda_full_matrix(om, qov, g.gamma, qoo, qvv, g.gamma_lr if lc else None, sy.n_occ, sy.n_virt)
    return np.linalg.eigvalsh(a)[state]


def oracle_gradient(numbers, xyz, lc, state=0, variant="exact", orientation="index", n_roots=3):
    sy = gs.build_system(numbers, xyz, lc=lc)
    g = gs.run_scc(sy, tol=1e-11)
    occ, virt = sy.occ_indices, sy.virt_indices
    qov, qoo, qvv = OT.trans_charges(sy.ao_offset, g.orbs, g.s, occ, virt)
    om = OT.orbe_differences(g.orbe[occ], g.orbe[virt])
    a = OT.tda_full_matrix(om, qov, g.gamma, qoo, qvv, g.gamma_lr if lc else None, sy.n_occ, sy.n_virt)
    e, x = np.linalg.eigh(a)
    der = OG.derivative_tensors(sy.numbers, sy.xyz, sy.ao_offset, sy.ao_atom, sy.hubbard, sy.r_lr, sy.params,
                                orientation=orientation)
    inp = dict(p=g.p, p0=g.p0, h_coul_x=g.h_coul_x, gamma=g.gamma, dq=g.dq, s=g.s, ao_atom=sy.ao_atom,
               numbers=sy.numbers, xyz=sy.xyz, params=sy.params, gamma_lr_ao=gs.atom_to_ao(sy, g.gamma_lr),
               orbe=g.orbe, occ=occ, virt=virt, ci_eigenvalues=e[:n_roots], ci_coefficients=x[:, :n_roots],
               q_ov=qov, q_oo=qoo, q_vv=qvv, gamma_lr=g.gamma_lr, orbs=g.orbs, gamma_ao=gs.atom_to_ao(sy, g.gamma))
    grad_gs, flr = OG.ground_state_gradient(inp, der, lc)
    grad_exc = OG.tda_gradient(inp, der, state, lc, flr_dmd0=flr, variant=variant)
    return grad_gs, grad_exc, sy


@pytest.mark.parametrize("lc", [True, False])
def test_excited_gradient_exact_variant_matches_fd(lc):
    """Analytic excitation-energy gradient against central differences (+-1e-4 bohr) on water
    (gradients/numerical.rs design)."""
    d = golden("h2o")
    nums = np.array([NUMBERS[s] for s in d["symbols"]])
    xyz = d["xyz_angstrom"] / 0.529177210903
    _, ge, sy = oracle_gradient(nums, xyz, lc)
    h = 1e-4
    fd = np.zeros_like(ge)
    for c in range(len(fd)):
        xp, xm = xyz.copy(), xyz.copy()
        xp[c // 3, c % 3] += h
        xm[c // 3, c % 3] -= h
        fd[c] = (_exc_energy(nums, xp, lc) - _exc_energy(nums, xm, lc)) / (2 * h)
    assert np.abs(ge - fd).max() < 1e-5


def test_reference_lc_gradient_differs_from_fd_by_zvector_operator():
    """tincr's LC-TDA gradient (Z-vector with the TDA matrix A) is not the derivative of the LC-TDA
    energy; the exact variant ((A+B), H+[Z]) is.  Records the size of that difference on water."""
    d = golden("h2o")
    nums = np.array([NUMBERS[s] for s in d["symbols"]])
    xyz = d["xyz_angstrom"] / 0.529177210903
    _, g_ref, _ = oracle_gradient(nums, xyz, True, variant="reference")
    _, g_ex, _ = oracle_gradient(nums, xyz, True, variant="exact")
    diff = np.abs(g_ref - g_ex).max()
    assert 1e-5 < diff < 1e-2
    _, g_ref_nolc, _ = oracle_gradient(nums, xyz, False, variant="reference")
    _, g_ex_nolc, _ = oracle_gradient(nums, xyz, False, variant="exact")
    assert np.abs(g_ref_nolc - g_ex_nolc).max() < 1e-14


def test_apb_product_known_answer():
    """(A+B).v with long-range exchange on tincr's 2 x 2 active-space known answer
    (not_refactored_tests/solver.rs:1478-1634, `test_apbv_fortran`: four unit trial vectors, the
    stored products bp_ref): the operator of the exact-variant Z-vector, to rounding."""
    d = golden("kat_test_apbv_fortran")
    bs = d["bs"]
    out = np.stack([OG.mult_apb_lc(d["gamma"], d["gamma_lr"], d["qtrans_ov"], d["qtrans_oo"], d["qtrans_vv"],
                                   d["omega0"], bs[:, :, k]) for k in range(bs.shape[2])], axis=2)
    assert np.abs(out - d["bp_ref"]).max() < 1e-14


@pytest.mark.parametrize("name,lc,variant", [("naphthalene", True, "reference"), ("naphthalene", False, "reference"),
                                             ("water8", True, "exact")])
def test_gradient_by_atom_equals_dense(name, lc, variant):
    """The atom-by-atom oracle gradient (one atom's derivative rows at a time, used at benchmark
    sizes where the [3N, n, n] tensors do not fit) equals the dense restatement."""
    from cases import oracle_gradient_inputs
    from oracle import gradients as OG
    from oracle import tda as OT
    from tincr_gb300 import geometry as G
    from tincr_gb300 import groundstate as gs
    z, x = G.acene(2) if name == "naphthalene" else G.water_cluster(2, 2, 2)
    sy = gs.build_system(z, G.to_bohr(x), lc=lc)
    g = gs.run_scc(sy, tol=1e-10)
    occ, virt = sy.occ_indices, sy.virt_indices
    q = OT.trans_charges(sy.ao_offset, g.orbs, g.s, occ, virt)
    om = OT.orbe_differences(g.orbe[occ], g.orbe[virt])
    a = OT.tda_full_matrix(om, q[0], g.gamma, q[1], q[2], g.gamma_lr if lc else None, sy.n_occ, sy.n_virt)
    e, xv = np.linalg.eigh(a)
    inp = oracle_gradient_inputs(sy, g, lc, e[:3], xv[:, :3], q)
    orient = "reference" if variant == "reference" else "index"
    der = OG.derivative_tensors(sy.numbers, sy.xyz, sy.ao_offset, sy.ao_atom, sy.hubbard, sy.r_lr, sy.params,
                                orientation=orient)
    ggs, flr = OG.ground_state_gradient(inp, der, lc)
    gex = OG.tda_gradient(inp, der, 1, lc, flr_dmd0=flr, variant=variant)
    rows = OG.AtomRows(sy.numbers, sy.xyz, sy.ao_offset, sy.ao_atom, sy.hubbard, sy.r_lr, sy.params,
                       orientation=orient)
    ggs2, gex2 = OG.gradients_by_atom(inp, rows, 1, lc, variant=variant)
    assert np.abs(ggs2 - ggs).max() < 1e-13
    assert np.abs(gex2 - gex).max() < 1e-13
