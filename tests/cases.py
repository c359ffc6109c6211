"""Input cases shared by the tests: golden-fixture ground states and seeded synthetic systems."""

import os

import numpy as np

from tincr_gb300 import geometry as G
from tincr_gb300 import groundstate as gs
from tincr_gb300.params import NUMBERS

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# the fixtures of tincr's tests/data were generated with this bohr radius
FIXTURE_BOHR = 0.529177249


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def fixture_case(mol, lc=True):
    """Ground state exactly as stored in tincr's tests/data/<mol> fixtures."""
    d = golden(mol)
    numbers = np.array([NUMBERS[s] for s in d["symbols"]], dtype=np.int32)
    sy = gs.build_system(numbers, d["xyz_angstrom"] / FIXTURE_BOHR, lc=lc)
    n_occ = int(np.sum(d["occupation"][:, 0] > 0))
    return dict(
        name=mol, numbers=numbers, xyz=sy.xyz, opa=d["orbs_per_atom"][:, 0].astype(np.int32),
        ao_offset=np.concatenate([[0], np.cumsum(d["orbs_per_atom"][:, 0].astype(np.int64))]),
        orbs=np.ascontiguousarray(d["orbs_after_scc"]), s=np.ascontiguousarray(d["S"]),
        orbe=d["orbe_after_scc"][:, 0].copy(), n_occ=n_occ, n_virt=sy.n_orbs - n_occ,
        gamma=np.ascontiguousarray(d["gamma_atomwise"]),
        gamma_lr=np.ascontiguousarray(d["gamma_atomwise_lc"]) if lc else None)


_SYN = {}


def synthetic_case(name, lc=True, r_lr=gs.LONG_RANGE_RADIUS):
    """Seeded synthetic system with a host SCC ground state (cached per process)."""
    key = (name, lc, r_lr)
    if key in _SYN:
        return _SYN[key]
    if name == "polyene":
        z, x = G.polyene(20)
    elif name == "polyene8":
        z, x = G.polyene(8)
    elif name == "decacene":
        z, x = G.acene(10)
    elif name == "naphthalene":
        z, x = G.acene(2)
    elif name.startswith("water"):
        n = {"water8": (2, 2, 2), "water27": (3, 3, 3), "water128": (8, 4, 4)}[name]
        z, x = G.water_cluster(*n)
    else:
        raise KeyError(name)
    sy = gs.build_system(z, G.to_bohr(x), lc=lc, r_lr=r_lr)
    g = gs.run_scc(sy)
    case = dict(name=name, numbers=sy.numbers, xyz=sy.xyz, opa=sy.orbs_per_atom.astype(np.int32),
                ao_offset=sy.ao_offset, orbs=g.orbs, s=g.s, orbe=g.orbe, n_occ=sy.n_occ, n_virt=sy.n_virt,
                gamma=g.gamma, gamma_lr=g.gamma_lr if lc else None, system=sy, ground=g)
    _SYN[key] = case
    return case


def oracle_inputs(case):
    """q's, omega and engine arguments of the oracle for a case."""
    from oracle import tda
    no, nv = case["n_occ"], case["n_virt"]
    occ = np.arange(no)
    virt = np.arange(no, no + nv)
    qov, qoo, qvv = tda.trans_charges(case["ao_offset"], case["orbs"], case["s"], occ, virt)
    om = tda.orbe_differences(case["orbe"][occ], case["orbe"][virt])
    return dict(omega=om, q_ov=qov, q_oo=qoo, q_vv=qvv, gamma=case["gamma"], gamma_lr=case["gamma_lr"],
                n_occ=no, n_virt=nv)


_FMO = {}


def fmo_case(nx=3, ny=1, nz=1, lc=True, n_le=4, n_ct=1, cutoff_angstrom=4.5, seed=20240064):
    """Small seeded acene aggregate (the 4.5 A CT cutoff and ring counts of the FMO benchmark) with
    its batched work list: every monomer, both directions of every close pair."""
    from tincr_gb300 import fmo
    key = (nx, ny, nz, lc, n_le, n_ct, cutoff_angstrom, seed)
    if key in _FMO:
        return _FMO[key]
    z, x, mono = G.acene_lattice(nx, ny, nz, seed=seed)
    mons = fmo.build_monomers(z, G.to_bohr(x), mono, lc=lc)
    pairs = fmo.close_pairs(mons, cutoff_angstrom / gs.P.BOHR_TO_ANGS)
    inst, labels = fmo.aggregate_instances(mons, pairs, n_le, n_ct)
    case = dict(monomers=mons, pairs=pairs, instances=inst, labels=labels, lc=lc)
    _FMO[key] = case
    return case


def fmo_oracle_engine(case, k):
    """Oracle engine of instance k: TdaEngine of the monomer (LE) or CtEngine of the pair (CT)."""
    from oracle import tda as OT
    lab = case["labels"][k]
    mons = {m.index: m for m in case["monomers"]}
    if lab[0] == "LE":
        m = mons[lab[1]]
        sy, g = m.system, m.ground
        qov, qoo, qvv = OT.trans_charges(sy.ao_offset, g.orbs, g.s, sy.occ_indices, sy.virt_indices)
        om = OT.orbe_differences(g.orbe[sy.occ_indices], g.orbe[sy.virt_indices])
        eng = OT.TdaEngine(om, qov, g.gamma, qoo, qvv, g.gamma_lr if case["lc"] else None, sy.n_occ, sy.n_virt)
        return eng, sy.xyz
    mh, ml = mons[lab[1]], mons[lab[2]]
    from tincr_gb300 import fmo
    d = fmo.Dimer(mh, ml)
    nh = mh.system.n_orbs
    sh, sl = mh.system, ml.system
    qov = OT.ct_pair_q_ov(sh.ao_offset, sl.ao_offset, mh.ground.orbs, ml.ground.orbs, d.s[:nh, nh:], sh.n_occ,
                          sl.n_occ)
    _, qoo_h, _ = OT.trans_charges(sh.ao_offset, mh.ground.orbs, mh.ground.s, sh.occ_indices, sh.virt_indices)
    _, _, qvv_l = OT.trans_charges(sl.ao_offset, ml.ground.orbs, ml.ground.s, sl.occ_indices, sl.virt_indices)
    om = OT.orbe_differences(mh.ground.orbe[sh.occ_indices], ml.ground.orbe[sl.virt_indices])
    na = sh.n_atoms
    glr = d.gamma_lr[:na, na:] if case["lc"] else np.zeros((na, sl.n_atoms))
    eng = OT.CtEngine(om, qov, d.gamma, qoo_h, qvv_l, glr, sh.n_occ, sl.n_virt)
    return eng, d.system.xyz


def scc_arrays(args):
    """Host SCC of one geometry -> the arrays a TDA set-up needs.  `args` = (numbers, xyz in bohr,
    lc); top-level so that a spawn process pool can run it."""
    z, xyz, lc = args
    sy = gs.build_system(z, xyz, lc=lc)
    g = gs.run_scc(sy, tol=1e-11)
    return dict(orbs=g.orbs, s=g.s, orbe=g.orbe, gamma=g.gamma, gamma_lr=g.gamma_lr if lc else None)


def displaced_scc(z, xyz, lc, h):
    """SCC ground states at xyz + h e_c and xyz - h e_c for every Cartesian coordinate c, run in a
    spawn process pool with one BLAS thread per worker.  Returns [(plus, minus)] per coordinate."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    jobs = []
    for c in range(xyz.size):
        for sgn in (1.0, -1.0):
            x = xyz.copy()
            x[c // 3, c % 3] += sgn * h
            jobs.append((z, x, lc))
    keys = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")
    saved = {k: os.environ.get(k) for k in keys}
    os.environ.update({k: "1" for k in keys})
    try:
        with ProcessPoolExecutor(max_workers=min(16, os.cpu_count() or 1),
                                 mp_context=mp.get_context("spawn")) as ex:
            out = list(ex.map(scc_arrays, jobs, chunksize=4))
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    return [(out[2 * c], out[2 * c + 1]) for c in range(xyz.size)]


def oracle_gradient_inputs(sy, g, lc, energies, coefficients, q=None):
    """The `inp` dict of the oracle gradients for a host system `sy` with ground state `g` and the
    roots (energies [n], coefficients [o*v, n]); q = (q_ov, q_oo, q_vv) when already computed."""
    from oracle import tda as OT
    occ, virt = sy.occ_indices, sy.virt_indices
    qov, qoo, qvv = q if q is not None else OT.trans_charges(sy.ao_offset, g.orbs, g.s, occ, virt)
    return dict(p=g.p, p0=g.p0, h_coul_x=g.h_coul_x, gamma=g.gamma, dq=g.dq, s=g.s, ao_atom=sy.ao_atom,
                numbers=sy.numbers, xyz=sy.xyz, params=sy.params,
                gamma_lr_ao=gs.atom_to_ao(sy, g.gamma_lr) if lc else None,
                orbe=g.orbe, occ=occ, virt=virt, ci_eigenvalues=np.asarray(energies),
                ci_coefficients=np.asarray(coefficients), q_ov=qov, q_oo=qoo, q_vv=qvv,
                gamma_lr=g.gamma_lr if lc else None, orbs=g.orbs, gamma_ao=gs.atom_to_ao(sy, g.gamma))
