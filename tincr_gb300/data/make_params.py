"""Convert tincr's H/C/N/O parameter set (RON) into the compact `hcno_params.npz` shipped here.

Run once where the tincr sources are available:

    python tincr_gb300/data/make_params.py /path/to/tincr

What is extracted, and from where (paths inside the tincr project):

* pseudo atoms (`src/param/slaterkoster/{confined,free}_pseudo_atom/<el>.ron`), combined the way
  `Atom::from(Element)` does (`src/initialization/atom.rs:58-95`): Hubbard U from the confined atom,
  orbital energies from the free atom, one orbital per m in -l..l (order s, p(m=-1), p(m=0),
  p(m=+1)), occupation = shell occupation / (2l+1);
* Slater-Koster tables (`src/param/slaterkoster/slako_tables/<a>_<b>.ron`, element pair ordered by
  atomic number as in `SlaterKosterTable::new`, `src/initialization/parameters.rs:191-213`): the
  distance grid and the tabulated S and H0 integrals keyed by integral index
  (0 ss_sigma, 2 sp_sigma, 4 ps_sigma, 5 pp_pi, 6 pp_sigma);
* repulsive potentials (`src/param/repulsive_potential/reppot_tables/<a>_<b>.ron`,
  `src/initialization/parameters.rs:301-372`).

The cubic interpolating splines (FITPACK `splrep`, k=3, s=0; tincr calls Rusty-FITPACK's `splrep`
with all defaults at `parameters.rs:222`, `:237`, `:325`) are computed with SciPy's FITPACK
binding and stored as knots + coefficients, so no spline fitting happens at run time.
"""

import os
import sys

import numpy as np
from scipy.interpolate import splrep

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import ron  # noqa: E402

ELEMENTS = {1: "h", 6: "c", 7: "n", 8: "o"}


def _atom(src, z):
    sym = ELEMENTS[z]
    base = os.path.join(src, "src", "param", "slaterkoster")
    conf = ron.loads(open(os.path.join(base, "confined_pseudo_atom", sym + ".ron")).read())
    free = ron.loads(open(os.path.join(base, "free_pseudo_atom", sym + ".ron")).read())
    ls, ms, es, occ = [], [], [], []
    n_elec = 0
    for i, j in zip(conf["valence_orbitals"], free["valence_orbitals"]):
        l = conf["angular_momenta"][i]
        e = free["energies"][j]
        for m in range(-l, l + 1):
            ls.append(l)
            ms.append(m)
            es.append(e)
            occ.append(conf["orbital_occupation"][i] / (2 * l + 1))
        n_elec += conf["orbital_occupation"][i]
    return dict(hubbard=float(conf["hubbard_u"]), l=np.array(ls, np.int32), m=np.array(ms, np.int32),
                energy=np.array(es), occ=np.array(occ), n_elec=n_elec)


def main(src, out):
    arrs = {}
    zs = sorted(ELEMENTS)
    arrs["elements"] = np.array(zs, np.int32)
    for z in zs:
        a = _atom(src, z)
        arrs["el%d_hubbard" % z] = np.array(a["hubbard"])
        arrs["el%d_l" % z] = a["l"]
        arrs["el%d_m" % z] = a["m"]
        arrs["el%d_energy" % z] = a["energy"]
        arrs["el%d_occ" % z] = a["occ"]
        arrs["el%d_nelec" % z] = np.array(a["n_elec"], np.int32)
    grid = None
    for ia, za in enumerate(zs):
        for zb in zs[ia:]:
            fn = os.path.join(src, "src", "param", "slaterkoster", "slako_tables",
                              "%s_%s.ron" % (ELEMENTS[za], ELEMENTS[zb]))
            tab = ron.loads(open(fn).read())
            d = np.array(tab["d"], dtype=np.float64)
            if grid is None:
                grid = d
            assert np.array_equal(grid, d), "all SK tables are expected on one grid"
            for kind in ("s", "h"):
                for (l1, l2, idx), vals in tab[kind].items():
                    y = np.array(vals, dtype=np.float64)
                    t, c, k = splrep(d, y)
                    key = "sk_%d_%d_%s_%d" % (za, zb, kind, idx)
                    arrs[key + "_y"] = y
                    arrs[key + "_c"] = np.asarray(c, np.float64)
                    arrs["sk_knots"] = np.asarray(t, np.float64)
            rfn = os.path.join(src, "src", "param", "repulsive_potential", "reppot_tables",
                               "%s_%s.ron" % (ELEMENTS[za], ELEMENTS[zb]))
            rep = ron.loads(open(rfn).read())
            rd = np.array(rep["d"], np.float64)
            ry = np.array(rep["vrep"], np.float64)
            t, c, k = splrep(rd, ry)
            key = "rep_%d_%d" % (za, zb)
            arrs[key + "_grid"] = rd
            arrs[key + "_y"] = ry
            arrs[key + "_t"] = np.asarray(t, np.float64)
            arrs[key + "_c"] = np.asarray(c, np.float64)
    arrs["sk_grid"] = grid
    np.savez_compressed(out, **arrs)


if __name__ == "__main__":
    if len(sys.argv) not in (2, 3):
        sys.exit("usage: python make_params.py <path of the tincr source tree> [output .npz]")
    src = sys.argv[1]
    out = sys.argv[2] if len(sys.argv) > 2 else os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                                              "hcno_params.npz")
    main(src, out)
    print("wrote", out)
