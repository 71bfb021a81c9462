"""Synthetic tetrahedral meshes (the workload generator, not part of the path).

``kuhn_box`` splits an nx x ny x nz grid of hexahedra into 6 tetrahedra each
(the Kuhn / Freudenthal split along the cube diagonal), the unit-cube-style
mesh Feel++ builds with ``unitCube()`` / gmsh in its tests, here generated
deterministically:

* vertex (i, j, k) has id ``(i*(ny+1) + j)*(nz+1) + k`` (x slowest, z fastest);
* cells are visited in the same (i, j, k) order; cell tetrahedra follow the 6
  permutations (a, b, c) of the axes in lexicographic order, tetrahedron
  ``[c0, c0+e_a, c0+e_a+e_b, c0+e_a+e_b+e_c]`` (half of them negatively oriented,
  which Feel++ accepts since J = |det K|);
* interior vertices are moved by U(-a h, a h) per coordinate (numpy PCG64 with
  the given seed), h the cell size along that axis;
* an optional per-element coefficient is lognormal(0, 1) from a second seed.
"""
import itertools

import numpy as np

PERMS = list(itertools.permutations(range(3)))


def kuhn_box(nx, ny=None, nz=None, lengths=(1.0, 1.0, 1.0), perturb=0.0, seed=1234):
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    Lx, Ly, Lz = lengths
    ii, jj, kk = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    hx, hy, hz = Lx / nx, Ly / ny, Lz / nz
    xyz = np.stack([ii * hx, jj * hy, kk * hz], axis=-1).reshape(-1, 3).astype(np.float64)
    if perturb > 0:
        rng = np.random.default_rng(seed)
        d = rng.uniform(-1.0, 1.0, size=xyz.shape) * (perturb * np.array([hx, hy, hz]))
        interior = ((ii > 0) & (ii < nx) & (jj > 0) & (jj < ny) & (kk > 0) & (kk < nz)).reshape(-1)
        xyz[interior] += d[interior]

    def vid(i, j, k):
        return (i * (ny + 1) + j) * (nz + 1) + k

    ci, cj, ck = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ci, cj, ck = ci.reshape(-1), cj.reshape(-1), ck.reshape(-1)
    unit = np.eye(3, dtype=np.int64)
    tets = np.zeros((ci.size, 6, 4), dtype=np.int64)
    for t, (a, b, c) in enumerate(PERMS):
        steps = [np.zeros(3, dtype=np.int64), unit[a], unit[a] + unit[b], unit[a] + unit[b] + unit[c]]
        for v, s in enumerate(steps):
            tets[:, t, v] = vid(ci + s[0], cj + s[1], ck + s[2])
    return xyz, tets.reshape(-1, 4).astype(np.int32)


def lognormal_kappa(nt, seed=5678):
    rng = np.random.default_rng(seed)
    return rng.lognormal(0.0, 1.0, size=nt)


def unit_cube(n, perturb=0.0, seed=1234):
    return kuhn_box(n, perturb=perturb, seed=seed)
