"""H/C/N/O DFTB parameter set: pseudo-atom data, Slater-Koster splines, repulsive splines.

The data file `data/hcno_params.npz` is produced by `data/make_params.py` from tincr's RON tables.
Element data follow `Atom::from(Element)` (`src/initialization/atom.rs:58-95`); Slater-Koster
tables follow `SlaterKosterTable` (`src/initialization/parameters.rs:161-244`): one table per
element pair ordered by atomic number, integrals keyed 0 ss_sigma, 2 sp_sigma, 4 ps_sigma,
5 pp_pi, 6 pp_sigma, every integral splined with FITPACK cubic interpolation (s=0) on one
shared 250-point grid from 0 to 10 bohr.
"""

import os
from dataclasses import dataclass, field

import numpy as np

_DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "hcno_params.npz")

SYMBOLS = {1: "H", 6: "C", 7: "N", 8: "O"}
NUMBERS = {v: k for k, v in SYMBOLS.items()}
# index of each SK integral inside a packed coefficient block
SK_INTEGRALS = (0, 2, 4, 5, 6)
SK_SLOT = {idx: k for k, idx in enumerate(SK_INTEGRALS)}

# BOHR_TO_ANGS of tincr (`src/constants.rs:4`)
BOHR_TO_ANGS = 0.529177210903


@dataclass
class Element:
    z: int
    hubbard: float
    l: np.ndarray
    m: np.ndarray
    energy: np.ndarray
    occ: np.ndarray
    n_elec: int

    @property
    def n_orbs(self):
        return len(self.l)


@dataclass
class ParamSet:
    elements: dict
    sk_knots: np.ndarray            # [254] knot vector shared by every SK spline
    sk_coef: dict                   # (za, zb, 's'|'h') -> [5, n_coef] coefficients, slot order SK_INTEGRALS
    sk_present: dict                # (za, zb) -> tuple of integral indices tabulated
    rep: dict = field(default_factory=dict)  # (za, zb) -> (t, c, dmax)

    def element(self, z):
        return self.elements[int(z)]


_CACHE = {}


def load(path=_DATA):
    """Load (and cache) the parameter set."""
    if path in _CACHE:
        return _CACHE[path]
    d = np.load(path)
    elements = {}
    for z in d["elements"]:
        z = int(z)
        elements[z] = Element(z=z, hubbard=float(d["el%d_hubbard" % z]), l=d["el%d_l" % z],
                              m=d["el%d_m" % z], energy=d["el%d_energy" % z], occ=d["el%d_occ" % z],
                              n_elec=int(d["el%d_nelec" % z]))
    knots = d["sk_knots"]
    ncoef = len(knots)
    sk_coef, sk_present, rep = {}, {}, {}
    zs = sorted(elements)
    for ia, za in enumerate(zs):
        for zb in zs[ia:]:
            present = []
            for kind in ("s", "h"):
                block = np.zeros((len(SK_INTEGRALS), ncoef))
                for idx in SK_INTEGRALS:
                    key = "sk_%d_%d_%s_%d_c" % (za, zb, kind, idx)
                    if key in d.files:
                        block[SK_SLOT[idx]] = d[key]
                        if kind == "s":
                            present.append(idx)
                sk_coef[(za, zb, kind)] = block
            sk_present[(za, zb)] = tuple(present)
            key = "rep_%d_%d" % (za, zb)
            rep[(za, zb)] = (d[key + "_t"], d[key + "_c"], float(d[key + "_grid"][-1]))
    ps = ParamSet(elements=elements, sk_knots=knots, sk_coef=sk_coef, sk_present=sk_present, rep=rep)
    _CACHE[path] = ps
    return ps
