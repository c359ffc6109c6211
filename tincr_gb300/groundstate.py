"""Host-side DFTB ground state: the upstream producer of the excited-state path's inputs.

The linear-response path (transition charges, Davidson TDA, analytic gradient) consumes the
converged ground state: MO coefficients C, orbital energies, overlap S, the gamma matrices and
the density matrices.  In tincr these come from `System::from` (`src/initialization/system.rs:74-240`),
`prepare_scc` and `run_scc` (`src/scc/scc_routine.rs:73-290`).  This module produces the same
quantities on the host so that tests and benchmarks can feed the GPU path; it is not part of the
timed path.

Conventions follow tincr:
* orbitals per atom in the order of `Atom::from` (s, then p with m = -1, 0, +1 i.e. y, z, x);
* occupied orbitals are the first n_elec/2 MOs (`system.rs:132-140`);
* SK integrals are zero beyond the last grid point of the table (10 bohr).  tincr evaluates its
  splines up to PROXIMITY_CUTOFF = 30 bohr (`h0_and_s.rs:110`) through Rusty-FITPACK's
  `splev_uniform`, whose behaviour outside the knot range no tincr fixture pins (all fixture
  distances are below 9.6 bohr).  Polynomial extrapolation of the end piece (FITPACK ext=0) grows
  to O(0.1-1) at 20-30 bohr and makes S indefinite for extended molecules, so the tail is taken as
  zero by default, the rule tincr itself applies to its repulsive splines (`parameters.rs:345-372`);
  `build_system(sk_tail="extrapolate")` evaluates the end piece instead, as FITPACK's splev does;
* S and H0 by the Slater-Koster rules of `src/param/slako_transformations.rs:57-680` (s and p
  orbitals) on the pair ordering of `src/scc/h0_and_s.rs:92-182`: the atom with the smaller atomic
  number is centre 1 and the direction vector points from centre 1 to centre 2;
* gamma from Gaussian charge distributions (`src/scc/gamma_approximation.rs:29-193`), the
  long-range (screened) gamma with the same formula and R_lr;
* SCC Hamiltonian H = H0 + H1 o S (+ LC exchange) (`scc_routine.rs:173-180`, `scc/helpers.rs:111-155`,
  `:232-255`).  Convergence is driven with DIIS to a tight threshold instead of tincr's Broyden
  mixer: both reach the same fixed point, and the tight threshold keeps the inputs of the
  finite-difference checks noise free.
"""

from dataclasses import dataclass

import numpy as np
from scipy.interpolate import splev
from scipy.special import erf

from . import params as P

# PROXIMITY_CUTOFF of tincr (`src/defaults.rs:40`), bohr
PROXIMITY_CUTOFF = 30.0
# LONG_RANGE_RADIUS default (`src/defaults.rs:39`), bohr
LONG_RANGE_RADIUS = 3.03
PI_SQRT = 1.7724538509055159


@dataclass
class System:
    numbers: np.ndarray      # [N] atomic numbers
    xyz: np.ndarray          # [N, 3] bohr
    n_atoms: int
    n_orbs: int
    orbs_per_atom: np.ndarray   # [N]
    ao_offset: np.ndarray       # [N+1]
    ao_atom: np.ndarray         # [n_orbs] atom of each AO
    ao_l: np.ndarray
    ao_m: np.ndarray
    ao_energy: np.ndarray
    ao_occ: np.ndarray
    n_elec: int
    occ_indices: np.ndarray
    virt_indices: np.ndarray
    hubbard: np.ndarray         # [N]
    r_lr: float                 # long-range radius (0 = LC off)
    lc: bool
    params: P.ParamSet
    # Slater-Koster splines beyond their grid (10 bohr) up to PROXIMITY_CUTOFF: "zero", or
    # "extrapolate" with the boundary polynomial piece, FITPACK's splev rule (ext = 0), which is what
    # tincr's splev_uniform evaluates there (h0_and_s.rs:110)
    sk_tail: str = "zero"

    @property
    def n_occ(self):
        return len(self.occ_indices)

    @property
    def n_virt(self):
        return len(self.virt_indices)


def build_system(numbers, xyz_bohr, lc=True, r_lr=LONG_RANGE_RADIUS, params=None, sk_tail="zero"):
    """Create a `System` from atomic numbers and bohr coordinates (`system.rs:74-240`)."""
    if sk_tail not in ("zero", "extrapolate"):
        raise ValueError("sk_tail must be 'zero' or 'extrapolate'")
    ps = params or P.load()
    numbers = np.asarray(numbers, dtype=np.int32)
    xyz = np.ascontiguousarray(np.asarray(xyz_bohr, dtype=np.float64).reshape(-1, 3))
    n_atoms = len(numbers)
    opa = np.array([ps.element(z).n_orbs for z in numbers], dtype=np.int64)
    off = np.zeros(n_atoms + 1, dtype=np.int64)
    off[1:] = np.cumsum(opa)
    n_orbs = int(off[-1])
    ao_atom = np.repeat(np.arange(n_atoms), opa)
    ao_l = np.concatenate([ps.element(z).l for z in numbers])
    ao_m = np.concatenate([ps.element(z).m for z in numbers])
    ao_e = np.concatenate([ps.element(z).energy for z in numbers])
    ao_occ = np.concatenate([ps.element(z).occ for z in numbers])
    n_elec = int(sum(ps.element(z).n_elec for z in numbers))
    idx = np.arange(n_orbs)
    occ = idx[idx < n_elec // 2]
    virt = idx[idx >= n_elec // 2]
    hub = np.array([ps.element(z).hubbard for z in numbers])
    return System(numbers=numbers, xyz=xyz, n_atoms=n_atoms, n_orbs=n_orbs, orbs_per_atom=opa,
                  ao_offset=off, ao_atom=ao_atom, ao_l=ao_l, ao_m=ao_m, ao_energy=ao_e, ao_occ=ao_occ,
                  n_elec=n_elec, occ_indices=occ, virt_indices=virt, hubbard=hub,
                  r_lr=float(r_lr) if lc else 0.0, lc=bool(lc), params=ps, sk_tail=sk_tail)


def system_from_symbols(symbols, xyz_angstrom, **kw):
    nums = [P.NUMBERS[s.capitalize()] for s in symbols]
    return build_system(nums, np.asarray(xyz_angstrom) / P.BOHR_TO_ANGS, **kw)


# ----------------------------------------------------------------------------------------------
# Slater-Koster rules (s and p orbitals)
# ----------------------------------------------------------------------------------------------

def _dir(u, m):
    # real spherical harmonics of l=1: m=-1 -> y, m=0 -> z, m=+1 -> x
    return u[..., {-1: 1, 0: 2, 1: 0}[m]]


def sk_value(l1, m1, l2, m2, u, v):
    """Value of one SK matrix element (`slako_transformations.rs:83-680`, s/p cases).

    u: [..., 3] direction cosines from centre 1 to centre 2; v: [5, ...] integrals in SK_INTEGRALS
    slot order (ss_sigma, sp_sigma, ps_sigma, pp_pi, pp_sigma).
    """
    if l1 == 0 and l2 == 0:
        return v[0]
    if l1 == 0 and l2 == 1:
        return _dir(u, m2) * v[1]
    if l1 == 1 and l2 == 0:
        return _dir(u, m1) * v[2]
    if l1 == 1 and l2 == 1:
        if m1 == m2:
            c = {-1: 1, 0: 2, 1: 0}[m1]
            o = [k for k in range(3) if k != c]
            return (u[..., o[0]] ** 2 + u[..., o[1]] ** 2) * v[3] + u[..., c] ** 2 * v[4]
        return _dir(u, m1) * _dir(u, m2) * (-v[3] + v[4])
    raise ValueError("only s and p orbitals are parameterised")


def _pair_list(sysm):
    """Pairs (a, b), a != b, a < b in index, within the proximity cutoff, oriented so that
    Z_a <= Z_b (centre 1 = a)."""
    n = sysm.n_atoms
    ii, jj = np.triu_indices(n, 1)
    d = np.linalg.norm(sysm.xyz[jj] - sysm.xyz[ii], axis=1)
    keep = d < PROXIMITY_CUTOFF
    ii, jj = ii[keep], jj[keep]
    zi, zj = sysm.numbers[ii], sysm.numbers[jj]
    swap = zi > zj
    a = np.where(swap, jj, ii)
    b = np.where(swap, ii, jj)
    return a, b


def h0_and_s(sysm):
    """Overlap S and H0 (`src/scc/h0_and_s.rs:92-182`)."""
    ps = sysm.params
    n = sysm.n_orbs
    S = np.zeros((n, n))
    H0 = np.zeros((n, n))
    a, b = _pair_list(sysm)
    za, zb = sysm.numbers[a], sysm.numbers[b]
    knots = ps.sk_knots
    ext = 0 if sysm.sk_tail == "extrapolate" else 1
    for zA in np.unique(za):
        for zB in np.unique(zb[za == zA]):
            sel = (za == zA) & (zb == zB)
            A, B = a[sel], b[sel]
            rv = sysm.xyz[B] - sysm.xyz[A]
            r = np.linalg.norm(rv, axis=1)
            u = rv / r[:, None]
            vs = np.zeros((5, len(r)))
            vh = np.zeros((5, len(r)))
            cs = ps.sk_coef[(int(zA), int(zB), "s")]
            ch = ps.sk_coef[(int(zA), int(zB), "h")]
            for slot, idx in enumerate(P.SK_INTEGRALS):
                if idx in ps.sk_present[(int(zA), int(zB))]:
                    vs[slot] = splev(r, (knots, cs[slot], 3), ext=ext)
                    vh[slot] = splev(r, (knots, ch[slot], 3), ext=ext)
            eA, eB = ps.element(zA), ps.element(zB)
            for p1 in range(eA.n_orbs):
                for p2 in range(eB.n_orbs):
                    l1, m1, l2, m2 = int(eA.l[p1]), int(eA.m[p1]), int(eB.l[p2]), int(eB.m[p2])
                    mu = sysm.ao_offset[A] + p1
                    nu = sysm.ao_offset[B] + p2
                    sv = sk_value(l1, m1, l2, m2, u, vs)
                    hv = sk_value(l1, m1, l2, m2, u, vh)
                    S[mu, nu] = sv
                    S[nu, mu] = sv
                    H0[mu, nu] = hv
                    H0[nu, mu] = hv
    d = np.arange(n)
    S[d, d] = 1.0
    H0[d, d] = sysm.ao_energy
    return S, H0


# ----------------------------------------------------------------------------------------------
# gamma matrices
# ----------------------------------------------------------------------------------------------

def gamma_params(sysm, r_lr):
    """sigma_A and C_AB of the Gaussian gamma function (`gamma_approximation.rs:29-73`)."""
    sigma = 1.0 / (sysm.hubbard * PI_SQRT)
    c = 1.0 / np.sqrt(2.0 * (sigma[:, None] ** 2 + sigma[None, :] ** 2 + 0.5 * r_lr ** 2))
    return sigma, c


def gamma_atomwise(sysm, r_lr):
    """gamma_AB = erf(C_AB r)/r, diagonal 1/sqrt(pi (sigma^2 + r_lr^2/4)) (`:75-124`, `:175-193`)."""
    sigma, c = gamma_params(sysm, r_lr)
    d = np.linalg.norm(sysm.xyz[:, None, :] - sysm.xyz[None, :, :], axis=-1)
    n = sysm.n_atoms
    g = np.zeros((n, n))
    off = ~np.eye(n, dtype=bool)
    g[off] = erf(c[off] * d[off]) / d[off]
    g[np.arange(n), np.arange(n)] = 1.0 / np.sqrt(np.pi * (sigma ** 2 + 0.25 * r_lr ** 2))
    return g


def atom_to_ao(sysm, g):
    """Expand an atom-pair matrix to AO pairs (`gamma_ao_wise_from_gamma_atomwise`, `:366-390`)."""
    return g[np.ix_(sysm.ao_atom, sysm.ao_atom)]


# ----------------------------------------------------------------------------------------------
# SCC
# ----------------------------------------------------------------------------------------------

def density_matrix_ref(sysm):
    """Neutral-atom reference density P0 (`scc/helpers.rs:218-229`)."""
    return np.diag(sysm.ao_occ.astype(np.float64))


def mulliken(sysm, p, s):
    """Mulliken atomic populations of p (`scc/mulliken.rs:9-25`)."""
    q_ao = np.einsum("ij,ji->i", s, p)
    return np.bincount(sysm.ao_atom, weights=q_ao, minlength=sysm.n_atoms)


def lc_exact_exchange(s, g0_lr_ao, dp):
    """Long-range exchange Hamiltonian H^x[dP] (`scc/helpers.rs:111-155`)."""
    s_dp = s @ dp
    tmp = (g0_lr_ao * s_dp) @ s
    hx = tmp + tmp.T
    hx = hx + g0_lr_ao * (s_dp @ s)
    hx = hx + (s @ (dp * g0_lr_ao)) @ s
    hx *= -0.125
    return 0.5 * (hx + hx.T)


def repulsive_energy(sysm):
    ps = sysm.params
    e = 0.0
    for i in range(sysm.n_atoms):
        for j in range(i + 1, sysm.n_atoms):
            za, zb = sorted((int(sysm.numbers[i]), int(sysm.numbers[j])))
            t, c, dmax = ps.rep[(za, zb)]
            r = np.linalg.norm(sysm.xyz[i] - sysm.xyz[j])
            if r <= dmax:
                e += float(splev(r, (t, c, 3)))
    return e


@dataclass
class GroundState:
    s: np.ndarray
    h0: np.ndarray
    gamma: np.ndarray
    gamma_lr: np.ndarray       # zeros when LC is off
    orbs: np.ndarray
    orbe: np.ndarray
    p: np.ndarray
    p0: np.ndarray
    dq: np.ndarray
    h_coul_x: np.ndarray       # converged SCC Hamiltonian (H0 + H1 o S + H^x)
    energy: float
    iterations: int
    converged: bool = True
    residual: float = 0.0      # largest |[F, P]| element (orthogonalised basis) of the last iterate


def run_scc(sysm, tol=1e-10, max_iter=250, s_h0=None, p_start=None, require_convergence=False, level_shift=0.0):
    """Restricted closed-shell SCC to ||[F, P]|| < tol, from the reference (neutral-atom) density or
    from `p_start` (tincr starts a pair SCC from its monomers' charges, src/fmo/scc/pair.rs:112-124).
    The result's `converged` says whether the test was met within max_iter iterations; with
    `require_convergence` a miss raises RuntimeError (tincr panics there, pair.rs:234-240).
    `level_shift` > 0 raises the virtual orbitals of the matrix that is diagonalised by that much
    (F + shift (S - S P S / 2) for the current density P): a stationary density is unchanged, but
    an aufbau occupation that swaps between near-degenerate orbitals from one iteration to the next
    settles."""
    s, h0 = s_h0 if s_h0 is not None else h0_and_s(sysm)
    gamma = gamma_atomwise(sysm, 0.0)
    gamma_lr = gamma_atomwise(sysm, sysm.r_lr) if sysm.lc else np.zeros_like(gamma)
    g_lr_ao = atom_to_ao(sysm, gamma_lr) if sysm.lc else None
    p0 = density_matrix_ref(sysm)
    w, v = np.linalg.eigh(s)
    x = (v / np.sqrt(w)) @ v.T
    n_occ = sysm.n_elec // 2
    p = p0.copy() if p_start is None else np.array(p_start, dtype=float)
    hist_f, hist_e = [], []
    it = 0
    converged = False
    orbs = orbe = f = None
    for it in range(1, max_iter + 1):
        dp = p - p0
        dq = mulliken(sysm, dp, s)
        esp = gamma @ dq
        esp_ao = esp[sysm.ao_atom]
        f = h0 + 0.5 * (esp_ao[:, None] + esp_ao[None, :]) * s
        if sysm.lc:
            f = f + lc_exact_exchange(s, g_lr_ao, dp)
        err = x.T @ (f @ p @ s - s @ p @ f) @ x
        errn = np.abs(err).max()
        hist_f.append(f)
        hist_e.append(err)
        if len(hist_f) > 8:
            hist_f.pop(0)
            hist_e.pop(0)
        if it > 1 and errn < tol:
            converged = True
            break
        m = len(hist_f)
        if m > 1:
            bmat = -np.ones((m + 1, m + 1))
            bmat[m, m] = 0.0
            for i in range(m):
                for j in range(m):
                    bmat[i, j] = np.vdot(hist_e[i], hist_e[j])
            rhs = np.zeros(m + 1)
            rhs[m] = -1.0
            try:
                coef = np.linalg.solve(bmat, rhs)[:m]
                f_use = sum(c * fi for c, fi in zip(coef, hist_f))
            except np.linalg.LinAlgError:
                f_use = f
        else:
            f_use = f
        if level_shift:
            f_use = f_use + level_shift * (s - 0.5 * s @ p @ s)
        orbe, cp = np.linalg.eigh(x.T @ f_use @ x)
        orbs = x @ cp
        occ_c = orbs[:, :n_occ]
        p = 2.0 * occ_c @ occ_c.T
    if require_convergence and not converged:
        raise RuntimeError("SCC not converged to %g in %d iterations" % (tol, max_iter))
    # final diagonalisation of the converged Fock matrix
    orbe, cp = np.linalg.eigh(x.T @ f @ x)
    orbs = x @ cp
    occ_c = orbs[:, :n_occ]
    p = 2.0 * occ_c @ occ_c.T
    dq = mulliken(sysm, p - p0, s)
    e_el = float(np.sum(p * h0) + 0.5 * dq @ gamma @ dq)
    if sysm.lc:
        dp = p - p0
        e_el += -0.125 * float(np.sum((s @ dp @ s) * dp * g_lr_ao) + np.sum((s @ dp) * (dp @ s) * g_lr_ao))
    return GroundState(s=s, h0=h0, gamma=gamma, gamma_lr=gamma_lr, orbs=np.ascontiguousarray(orbs),
                       orbe=orbe, p=p, p0=p0, dq=dq, h_coul_x=f, energy=e_el + repulsive_energy(sysm),
                       iterations=it, converged=converged, residual=float(errn))
