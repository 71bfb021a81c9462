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


def hex_box(nx, ny=None, nz=None, lengths=(1.0, 1.0, 1.0), perturb=0.0, seed=1234):
    """Structured hexahedral mesh of [0,Lx]x[0,Ly]x[0,Lz] (the grid of MeshStructured): the vertices and
    their interior perturbation as in kuhn_box, one hexahedron per cell in the reference vertex order
    (z = -1 face (0,0,0) (1,0,0) (1,1,0) (0,1,0), then the z = +1 face)."""
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
    corners = ((0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1))
    hexes = np.stack([vid(ci + a, cj + b, ck + c) for a, b, c in corners], axis=1)
    return xyz, hexes.astype(np.int32)


def lognormal_kappa(nt, seed=5678):
    rng = np.random.default_rng(seed)
    return rng.lognormal(0.0, 1.0, size=nt)


def unit_cube(n, perturb=0.0, seed=1234):
    return kuhn_box(n, perturb=perturb, seed=seed)


# local edges of a tetrahedron in the reference dof order (vertex pairs)
EDGE_VERTS = ((1, 2), (2, 0), (0, 1), (0, 3), (1, 3), (2, 3))


def bulge_map(xyz, amp):
    """Smooth map of the unit cube onto a curved domain: x + amp (sin pi y sin pi z, sin pi z sin pi x,
    sin pi x sin pi y); every face of the cube bulges outwards or inwards."""
    x, y, z = xyz[..., 0], xyz[..., 1], xyz[..., 2]
    s = np.sin
    return np.stack([x + amp * s(np.pi * y) * s(np.pi * z), y + amp * s(np.pi * z) * s(np.pi * x),
                     z + amp * s(np.pi * x) * s(np.pi * y)], axis=-1)


def curved_box(n, amp=0.1, perturb=0.0, seed=1234):
    """Kuhn mesh of the unit cube mapped by bulge_map, as curved (P2-geometry) tetrahedra: vertices and
    edge nodes are images of the straight mesh's vertices and edge midpoints. Returns xyz (V x 3),
    tets (T x 4) and ho (T x 6 x 3, the edge nodes in EDGE_VERTS order)."""
    xyz0, tets = kuhn_box(n, perturb=perturb, seed=seed)
    mids = np.stack([0.5 * (xyz0[tets[:, a]] + xyz0[tets[:, b]]) for a, b in EDGE_VERTS], axis=1)
    return bulge_map(xyz0, amp), tets, bulge_map(mids, amp)
