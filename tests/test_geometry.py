"""CPU tests: the seeded synthetic geometries follow the benchmark recipes (bond lengths, angles,
lattice, jitter bounds) and give the stated orbital and electron counts."""

import numpy as np

from tincr_gb300 import geometry as G
from tincr_gb300 import groundstate as gs


def _pairs_within(xyz, lo, hi):
    d = np.linalg.norm(xyz[:, None, :] - xyz[None, :, :], axis=2)
    i, j = np.where(np.triu((d > lo) & (d < hi), 1))
    return d[i, j]


def test_polyene_c20h22():
    z, x = G.polyene(20)
    assert (z == 6).sum() == 20 and (z == 1).sum() == 22
    assert np.abs(x[:, 2]).max() == 0.0                              # planar
    c = x[z == 6]
    bonds = np.linalg.norm(np.diff(c, axis=0), axis=1)
    assert np.allclose(bonds[0::2], 1.34) and np.allclose(bonds[1::2], 1.46)
    for i in range(1, 19):                                           # 120 degrees at every inner C
        u, v = c[i - 1] - c[i], c[i + 1] - c[i]
        assert np.isclose(np.degrees(np.arccos(u @ v / np.linalg.norm(u) / np.linalg.norm(v))), 120.0)
    ch = _pairs_within(x, 1.0, 1.2)
    assert len(ch) == 22 and np.allclose(ch, 1.09)
    sy = gs.build_system(z, G.to_bohr(x), lc=False)
    assert (sy.n_orbs, sy.n_occ, sy.n_virt) == (102, 51, 51)


def test_water128_cluster():
    z, x = G.water_cluster(8, 4, 4)
    assert len(z) == 384 and (z == 8).sum() == 128
    mol = x.reshape(128, 3, 3)
    oh = np.linalg.norm(mol[:, 1:] - mol[:, :1], axis=2)
    assert np.allclose(oh, 0.9572)
    u, v = mol[:, 1] - mol[:, 0], mol[:, 2] - mol[:, 0]
    ang = np.degrees(np.arccos(np.einsum("ij,ij->i", u, v) / (oh[:, 0] * oh[:, 1])))
    assert np.allclose(ang, 104.52)
    lattice = np.array([[i, j, k] for i in range(8) for j in range(4) for k in range(4)]) * 3.0
    assert np.abs(mol[:, 0] - lattice).max() <= 0.2                   # O on the 3.0 A lattice +- 0.2 A
    sy = gs.build_system(z, G.to_bohr(x), lc=True)
    assert (sy.n_orbs, sy.n_occ, sy.n_virt) == (768, 512, 256)


def test_decacene():
    z, x = G.acene(10)
    assert (z == 6).sum() == 42 and (z == 1).sum() == 24
    assert np.abs(x[:, 0]).max() == 0.0                              # planar (yz)
    cc = _pairs_within(x[z == 6], 1.2, 1.5)
    assert np.allclose(cc, 1.40, atol=1e-6)
    ch = _pairs_within(x, 1.0, 1.2)
    assert len(ch) == 24 and np.allclose(ch, 1.08, atol=1e-6)
    sy = gs.build_system(z, G.to_bohr(x), lc=True)
    assert (sy.n_orbs, sy.n_occ, sy.n_virt) == (192, 96, 96)


def test_acene_aggregate():
    z, x, mono = G.acene_lattice(4, 4, 4)
    assert mono.max() + 1 == 64
    norb = {2: 48, 3: 66, 4: 84, 5: 102}
    seen = set()
    for m in range(64):
        zm = z[mono == m]
        rings = ((zm == 6).sum() - 2) // 4
        assert rings in norb
        seen.add(rings)
        sy = gs.build_system(zm, G.to_bohr(x[mono == m]), lc=True)
        assert sy.n_orbs == norb[rings] and sy.n_occ == sy.n_virt
    assert seen == {2, 3, 4, 5}
