"""Seeded synthetic geometries of the benchmark structures (Angstrom; atomic numbers).

* `polyene(n_c)`: planar all-trans CnH(n+2), C=C 1.34, C-C 1.46, C-H 1.09 Angstrom, 120 degrees.
* `water_cluster(nx, ny, nz)`: H2O (O-H 0.9572 Angstrom, H-O-H 104.52 degrees) on a cubic lattice
  of 3.0 Angstrom, uniform random orientation (seeded quaternion) and +-0.2 Angstrom uniform jitter.
* `acene(n_rings)`: linear acene, ideal hexagons, C-C 1.40, C-H 1.08 Angstrom, long axis along z.
* `acene_lattice(...)`: acene aggregate on an x/y/z lattice (3.6 / 5.0 / 14 Angstrom), ring counts
  uniform in {2..5}, in-plane rotation +-15 degrees, +-0.1 Angstrom jitter.  Monomers are defined
  by construction (molecule index), not by bond-graph fragmentation.

All random draws use numpy's PCG64 with an explicit seed.
"""

import numpy as np

from .params import BOHR_TO_ANGS


def polyene(n_c=20):
    pos = [np.zeros(2)]
    for k in range(n_c - 1):
        b = 1.34 if k % 2 == 0 else 1.46
        th = np.deg2rad(30.0 if k % 2 == 0 else -30.0)
        pos.append(pos[-1] + b * np.array([np.cos(th), np.sin(th)]))
    c = np.array(pos)
    hs = []
    for i in range(n_c):
        nb = [c[j] for j in (i - 1, i + 1) if 0 <= j < n_c]
        if len(nb) == 2:
            d = (c[i] - nb[0]) / np.linalg.norm(c[i] - nb[0]) + (c[i] - nb[1]) / np.linalg.norm(c[i] - nb[1])
            hs.append(c[i] + 1.09 * d / np.linalg.norm(d))
        else:
            u = (c[i] - nb[0]) / np.linalg.norm(c[i] - nb[0])
            for ang in (60.0, -60.0):
                a = np.deg2rad(ang)
                r = np.array([[np.cos(a), -np.sin(a)], [np.sin(a), np.cos(a)]])
                hs.append(c[i] + 1.09 * (r @ u))
    xyz = np.concatenate([np.c_[c, np.zeros(n_c)], np.c_[np.array(hs), np.zeros(len(hs))]])
    z = np.array([6] * n_c + [1] * len(hs), dtype=np.int32)
    return z, xyz


def _random_rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def water_cluster(nx=8, ny=4, nz=4, spacing=3.0, jitter=0.2, seed=20240128):
    rng = np.random.Generator(np.random.PCG64(seed))
    r, th = 0.9572, np.deg2rad(104.52)
    mol = np.array([[0.0, 0.0, 0.0],
                    [r * np.sin(th / 2), r * np.cos(th / 2), 0.0],
                    [-r * np.sin(th / 2), r * np.cos(th / 2), 0.0]])
    xyz, z = [], []
    for i in range(nx):
        for j in range(ny):
            for k in range(nz):
                rot = _random_rotation(rng)
                shift = np.array([i, j, k]) * spacing + rng.uniform(-jitter, jitter, size=3)
                xyz.append(mol @ rot.T + shift)
                z += [8, 1, 1]
    return np.array(z, dtype=np.int32), np.concatenate(xyz)


def acene(n_rings):
    """Linear acene with n_rings fused hexagons; long axis along z, molecular plane yz."""
    a = 1.40
    h = a * np.sqrt(3.0) / 2.0
    carb = {}
    # ring k centred at z = 2 h k; vertices at angles 0, 60, ..., 300 degrees (y = a cos, z = a sin)
    for k in range(n_rings):
        cz = 2.0 * h * k
        for v in range(6):
            ang = np.deg2rad(60.0 * v)
            p = (round(a * np.cos(ang), 6), round(cz + a * np.sin(ang), 6))
            carb[p] = True
    c = np.array(sorted(carb.keys(), key=lambda p: (p[1], p[0])))
    hs = []
    for i, p in enumerate(c):
        d = np.linalg.norm(c - p, axis=1)
        nb = c[(d > 0.1) & (d < 1.5)]
        if len(nb) == 2:
            u = (p - nb[0]) / np.linalg.norm(p - nb[0]) + (p - nb[1]) / np.linalg.norm(p - nb[1])
            hs.append(p + 1.08 * u / np.linalg.norm(u))
    c3 = np.c_[np.zeros(len(c)), c]
    h3 = np.c_[np.zeros(len(hs)), np.array(hs)]
    xyz = np.concatenate([c3, h3])
    xyz[:, 2] -= xyz[:, 2].mean()
    return np.array([6] * len(c) + [1] * len(hs), dtype=np.int32), xyz


def acene_lattice(nx=4, ny=4, nz=4, spacing=(3.6, 5.0, 14.0), jitter=0.1, rot_deg=15.0, seed=20240064):
    """Returns (numbers, xyz, monomer_index) for an acene aggregate."""
    rng = np.random.Generator(np.random.PCG64(seed))
    zs, xyz, mono = [], [], []
    m = 0
    for i in range(nx):
        for j in range(ny):
            for k in range(nz):
                nr = int(rng.integers(2, 6))
                z, x = acene(nr)
                ang = np.deg2rad(rng.uniform(-rot_deg, rot_deg))
                rot = np.array([[1, 0, 0], [0, np.cos(ang), -np.sin(ang)], [0, np.sin(ang), np.cos(ang)]])
                x = x @ rot.T + np.array([i * spacing[0], j * spacing[1], k * spacing[2]])
                x = x + rng.uniform(-jitter, jitter, size=x.shape)
                zs.append(z)
                xyz.append(x)
                mono += [m] * len(z)
                m += 1
    return np.concatenate(zs), np.concatenate(xyz), np.array(mono, dtype=np.int32)


def to_bohr(xyz_angstrom):
    return np.asarray(xyz_angstrom) / BOHR_TO_ANGS
