"""Batched SCC ground states on the GPU (`tincr_scc_batch`, tincr_gb300/scc.py).

* tincr's own SCC fixtures (tests/data of the reference: water, ammonia, benzene, uracil; LC): with
  the fixtures' S, H0 and gammas given, the GPU SCC reproduces the stored orbital energies, density
  and charges within tincr's convergence (it stops at an rms charge change of 1e-5), and equals the
  host SCC restatement on the same inputs at 1e-9.
* built inputs: the GPU's S and H0 equal the host's h0_and_s at 1e-14, and its converged ground
  state (orbital energies, density, charges, Fock matrix, energy, orbitals up to sign) equals the
  host SCC (`groundstate.run_scc`) on acenes, a polyene and a water cluster, LC and not, in one
  batch of mixed sizes, with the FP32 start, a level shift, a starting density and the extrapolated
  SK tails.
* failure reporting: an iteration cap, wrong sizes and non-finite coordinates."""

import numpy as np
import pytest

from cases import FIXTURE_BOHR, golden
from tincr_gb300 import _lib
from tincr_gb300 import geometry as G
from tincr_gb300 import groundstate as gs
from tincr_gb300 import scc
from tincr_gb300.params import NUMBERS

pytestmark = pytest.mark.gpu

MOLS = ["h2o", "ammonia", "benzene", "uracil"]


def _fixture(mol):
    d = golden(mol)
    z = np.array([NUMBERS[s] for s in d["symbols"]], np.int32)
    sy = gs.build_system(z, d["xyz_angstrom"] / FIXTURE_BOHR, lc=True)
    given = dict(s=np.array(d["S"]), h0=np.array(d["H0"]), gamma=np.array(d["gamma_atomwise"]),
                 gamma_lr=np.array(d["gamma_atomwise_lc"]))
    return sy, given, d


def _host_with(sy, given, tol):
    """host SCC restatement with the given S, H0 and gammas"""
    orig = gs.gamma_atomwise
    gs.gamma_atomwise = lambda s, r: np.array(given["gamma_lr"] if r > 0 else given["gamma"])
    try:
        return gs.run_scc(sy, tol=tol, s_h0=(given["s"], given["h0"]))
    finally:
        gs.gamma_atomwise = orig


def test_scc_reproduces_tincr_fixtures(gpu_ctx):
    items = [_fixture(m) for m in MOLS]
    out, rc = scc.scc_batch(gpu_ctx, [sy for sy, _, _ in items], tol=1e-11, given=[g for _, g, _ in items])
    assert rc == _lib.OK
    # tincr's fixtures: its SCC stops at an rms charge change of 1e-5, the bars cover that
    bars = {"h2o": 1e-7, "ammonia": 1e-7, "benzene": 1e-7, "uracil": 2e-5}
    for (sy, given, d), g, mol in zip(items, out, MOLS):
        assert g.converged and g.residual < 1e-11
        assert np.abs(g.orbe - d["orbe_after_scc"][:, 0]).max() < bars[mol], mol
        assert np.abs(g.p - d["P_after_scc"]).max() < 10 * bars[mol], mol
        assert np.abs(g.dq - d["dq_after_scc"][:, 0]).max() < 10 * bars[mol], mol
        h = _host_with(sy, given, 1e-11)
        assert np.abs(g.orbe - h.orbe).max() < 1e-9, mol
        assert np.abs(g.p - h.p).max() < 1e-9, mol
        assert np.abs(g.h_coul_x - h.h_coul_x).max() < 1e-9, mol
        assert abs(g.energy - h.energy) < 1e-9, mol


def _systems(lc, sk_tail="zero"):
    out = []
    for k in (2, 3, 5):
        z, x = G.acene(k)
        out.append(gs.build_system(z, G.to_bohr(x), lc=lc, sk_tail=sk_tail))
    z, x = G.polyene(20)
    out.append(gs.build_system(z, G.to_bohr(x), lc=lc, sk_tail=sk_tail))
    z, x = G.water_cluster(3, 3, 3)
    out.append(gs.build_system(z, G.to_bohr(x), lc=lc, sk_tail=sk_tail))
    return out


def _compare(g, h, tag):
    assert g.converged, tag
    # spline values agree to rounding (the extrapolated tails reach O(1e-2) with O(1e-14) rounding)
    assert np.abs(g.s - h.s).max() < 1e-13, tag
    assert np.abs(g.h0 - h.h0).max() < 1e-13, tag
    assert np.abs(g.orbe - h.orbe).max() < 1e-9, tag
    assert np.abs(g.p - h.p).max() < 1e-8, tag
    assert np.abs(g.dq - h.dq).max() < 1e-8, tag
    assert np.abs(g.h_coul_x - h.h_coul_x).max() < 1e-8, tag
    assert abs(g.energy - h.energy) < 1e-8, tag
    # orbitals up to sign, where the orbital energy is separated from its neighbours
    gap = np.minimum(np.diff(h.orbe, prepend=-np.inf), np.diff(h.orbe, append=np.inf))
    sep = gap > 1e-4
    sgn = np.sign(np.einsum("ij,ij->j", g.orbs, h.orbs))   # the sign of each orbital's overlap
    assert np.abs(g.orbs[:, sep] * sgn[sep] - h.orbs[:, sep]).max() < 1e-6, tag


@pytest.mark.parametrize("lc", [True, False])
@pytest.mark.parametrize("fp32", [False, True])
def test_scc_batch_matches_host(gpu_ctx, lc, fp32):
    systems = _systems(lc)
    out, rc = scc.scc_batch(gpu_ctx, systems, tol=1e-10, fp32_start=fp32)
    assert rc == _lib.OK
    for sy, g in zip(systems, out):
        h = gs.run_scc(sy, tol=1e-10)
        _compare(g, h, (sy.n_orbs, lc, fp32))


def test_scc_level_shift_start_density_and_sk_tails(gpu_ctx):
    # a naphthalene dimer 3.6 A apart from the block-diagonal monomer density, with a level shift,
    # and the extrapolated SK tails
    z, x = G.acene(2)
    xb = G.to_bohr(x)
    mono = gs.build_system(z, xb, lc=True, sk_tail="extrapolate")
    gm = gs.run_scc(mono, tol=1e-10)
    z2 = np.concatenate([z, z])
    x2 = np.concatenate([xb, xb + np.array([0.0, 0.0, 3.6 / 0.529177210903])])
    dim = gs.build_system(z2, x2, lc=True, sk_tail="extrapolate")
    n = mono.n_orbs
    p_start = np.zeros((2 * n, 2 * n))
    p_start[:n, :n] = gm.p
    p_start[n:, n:] = gm.p
    out, rc = scc.scc_batch(gpu_ctx, [dim], tol=1e-10, p_start=[p_start], level_shift=0.5)
    assert rc == _lib.OK
    h = gs.run_scc(dim, tol=1e-10, p_start=p_start, level_shift=0.5)
    _compare(out[0], h, "dimer")


def test_scc_reports_failures(gpu_ctx):
    systems = _systems(True)[:2]
    out, rc = scc.scc_batch(gpu_ctx, systems, tol=1e-10, max_iter=2)
    assert rc == _lib.NOT_CONVERGED
    assert not any(g.converged for g in out)
    assert all(g.iterations == 2 for g in out)
    with pytest.raises(RuntimeError):
        scc.scc_batch(gpu_ctx, systems, tol=1e-10, max_iter=2, require_convergence=True)
    bad = gs.build_system(systems[0].numbers, systems[0].xyz.copy(), lc=True)
    bad.xyz[0, 0] = np.nan
    with pytest.raises(_lib.TincrError) as e:
        scc.scc_batch(gpu_ctx, [bad], tol=1e-10)
    assert e.value.status == _lib.NONFINITE
    zb, xb = G.water_cluster(6, 6, 2)
    big = gs.build_system(zb, G.to_bohr(xb), lc=True)
    with pytest.raises(_lib.TincrError) as e:   # 432 orbitals: above the 256 of one CTA's slot
        scc.scc_batch(gpu_ctx, [big], tol=1e-10)
    assert e.value.status == _lib.BAD_ARG
    # the context still works
    out, rc = scc.scc_batch(gpu_ctx, systems[:1], tol=1e-10)
    assert rc == _lib.OK


def test_fmo_setup_on_gpu_matches_host(gpu_ctx):
    """build_monomers(scc="gpu") and ExcitonSetup(scc="gpu") (batched dimer SCCs from the monomers'
    densities) give the host set-up's ground states."""
    from cases import fmo_case
    from tincr_gb300 import fmo
    case = fmo_case(3, 2, 1)
    mons = case["monomers"]
    z = np.concatenate([m.system.numbers for m in mons])
    x = np.concatenate([m.system.xyz for m in mons])
    mono = np.concatenate([np.full(m.system.n_atoms, k) for k, m in enumerate(mons)])
    gm = fmo.build_monomers(z, x, mono, lc=True, scc="gpu", ctx=gpu_ctx)
    for a, b in zip(gm, mons):
        assert np.abs(a.ground.orbe - b.ground.orbe).max() < 1e-9
        assert np.abs(a.ground.p - b.ground.p).max() < 1e-8
    host = fmo.ExcitonSetup(mons, case["pairs"])
    dev = fmo.ExcitonSetup(mons, case["pairs"], scc="gpu", ctx=gpu_ctx)
    assert host.real_pairs == dev.real_pairs and host.real_pairs
    for k in host.real_pairs:
        assert np.abs(host.pair_scc[k][1] - dev.pair_scc[k][1]).max() < 1e-9


def test_scc_edge_cases(gpu_ctx):
    """The largest system one CTA takes (a water cluster of 252 orbitals) equals the host SCC; a
    two-orbital system (H2); an empty batch and a non-finite starting density are rejected."""
    z, x = G.water_cluster(7, 3, 2)            # 42 waters: 252 orbitals, 126 atoms
    big = gs.build_system(z, G.to_bohr(x), lc=True)
    assert big.n_orbs == 252
    h2 = gs.build_system(np.array([1, 1], np.int32), np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 1.4]]), lc=True)
    out, rc = scc.scc_batch(gpu_ctx, [big, h2], tol=1e-10)
    assert rc == _lib.OK
    for sy, g in zip((big, h2), out):
        _compare(g, gs.run_scc(sy, tol=1e-10), sy.n_orbs)
    out, rc = scc.scc_batch(gpu_ctx, [], tol=1e-10)
    assert out == [] and rc == _lib.OK
    p = np.diag(h2.ao_occ.astype(np.float64))
    p[0, 1] = np.nan
    with pytest.raises(_lib.TincrError) as e:
        scc.scc_batch(gpu_ctx, [h2], tol=1e-10, p_start=[p])
    assert e.value.status == _lib.NONFINITE
    with pytest.raises(ValueError):   # open shell
        scc.scc_batch(gpu_ctx, [gs.build_system(np.array([1], np.int32), np.zeros((1, 3)), lc=True)])
