"""Hexahedra (Q1/Q2) without a GPU: the oracle against known answers, then the library's host set-up
(first-encounter dof table, Gauss rule and basis tables) against the oracle."""
import ctypes as C

import numpy as np
import pytest

from feelpp_gb300 import meshgen
from oracle import hexoracle as ho


def unit_cube_hex():
    xyz = ho.HEX_VERTS * 0.5 + 0.5          # [0,1]^3 in the reference vertex order
    return xyz, np.arange(8, dtype=np.int32)[None, :]


def test_q1_unit_cube_matrices():
    """Q1 on the unit cube: stiffness 1/3 on the diagonal, 0 along an edge, -1/12 across a face or the body
    diagonal; mass = tensor product of the 1D mass [1/3 1/6; 1/6 1/3] (known closed forms)."""
    xyz, hexes = unit_cube_hex()
    K = ho.element_matrices(1, xyz, hexes)[0]
    Mm = ho.element_matrices(1, xyz, hexes, kappa_const=0.0, mass=1.0)[0]
    P = ho.HEX_VERTS
    for i in range(8):
        for j in range(8):
            d = int(np.sum(P[i] != P[j]))        # coordinates in which the vertices differ
            kexp = {0: 1.0 / 3.0, 1: 0.0, 2: -1.0 / 12.0, 3: -1.0 / 12.0}[d]
            mexp = (1.0 / 3.0) ** (3 - d) * (1.0 / 6.0) ** d
            assert abs(K[i, j] - kexp) < 1e-14
            assert abs(Mm[i, j] - mexp) < 1e-15


@pytest.mark.parametrize("order", [1, 2])
def test_oracle_consistency(order):
    """Laplacian rows sum to zero, the mass matrix sums to the volume and reproduces quadratic
    moments, the constant load integrates to c |Omega|, on perturbed hexahedra."""
    xyz, hexes = meshgen.hex_box(3, perturb=0.2)
    N, l2g = ho.dof_table(hexes, order)
    Ke = ho.element_matrices(order, xyz, hexes, kappa=meshgen.lognormal_kappa(len(hexes)))
    assert np.abs(Ke.sum(axis=2)).max() < 1e-13 * np.abs(Ke).max()
    Me = ho.element_matrices(order, xyz, hexes, kappa_const=0.0, mass=1.0, qdeg=2 * order + 1)
    assert abs(Me.sum() - 1.0) < 1e-13
    F = ho.rhs(order, xyz, hexes, l2g, N, fkind=2, c=2.5)
    assert abs(F.sum() - 2.5) < 1e-13
    # Q2 interpolates x^2 exactly: 1^T M (x^2 at the dofs) = int x^2 over the (straight-sided) cube
    if order == 2:
        xs, hs = meshgen.hex_box(3)
        N2, l2 = ho.dof_table(hs, 2)
        pts = ho.dof_points(2)
        gphi, _ = ho.tabulate(1, pts)
        X = np.zeros(N2)
        for e, h in enumerate(hs):
            p = gphi @ xs[h]                     # physical positions of the element's dof points
            X[l2[e]] = p[:, 0] ** 2
        M2 = ho.element_matrices(2, xs, hs, kappa_const=0.0, mass=1.0)
        tot = sum((M2[e].sum(axis=0) * X[l2[e]]).sum() for e in range(len(hs)))
        assert abs(tot - 1.0 / 3.0) < 1e-13


def test_gauss_rule_exactness():
    """(o+1)//2+1 points per direction integrate x^a y^b z^c exactly for a, b, c <= 2 m - 1"""
    for qdeg in range(1, 7):
        pts, w = ho.quadrature(qdeg)
        m = (qdeg + 1) // 2 + 1
        for a in range(2 * m):
            exact = 0.0 if a % 2 else 2.0 / (a + 1)
            got = np.sum(w * pts[:, 0] ** a * pts[:, 1] ** 0 * pts[:, 2] ** 0) / 4.0
            assert abs(got - exact) < 1e-14


def test_dof_table_first_encounter():
    """two cells sharing a face: the second cell reuses 4 vertex, 4 edge and 1 face dofs"""
    xyz, hexes = meshgen.hex_box(2, 1, 1)
    N1, l1 = ho.dof_table(hexes, 1)
    N2, l2 = ho.dof_table(hexes, 2)
    assert N1 == 12 and N2 == 5 * 3 * 3
    assert list(l1[0]) == list(range(8)) and list(l2[0]) == list(range(27))
    shared = set(l2[0]) & set(l2[1])
    assert len(shared) == 9


@pytest.mark.parametrize("order", [1, 2])
def test_host_dof_table_matches_oracle(fgpu_lib, order):
    xyz, hexes = meshgen.hex_box(4, 3, 2, perturb=0.1)
    n = ho.nloc(order)
    l2g = np.zeros((len(hexes), n), dtype=np.int32)
    nd = C.c_int64()
    rc = fgpu_lib.fgpu_host_hex_dof_table(len(xyz), len(hexes), hexes.ctypes.data_as(C.c_void_p), order,
                                          l2g.ctypes.data_as(C.c_void_p), C.byref(nd))
    assert rc == 0
    N, l2o = ho.dof_table(hexes, order)
    assert nd.value == N and np.array_equal(l2g, l2o)


@pytest.mark.parametrize("order,qdeg", [(1, 2), (1, 6), (2, 4), (2, 3)])
def test_host_ref_tables_match_oracle(fgpu_lib, order, qdeg):
    nq = C.c_int()
    assert fgpu_lib.fgpu_host_hex_ref_tables(order, qdeg, None, None, None, None, None, C.byref(nq)) == 0
    n = ho.nloc(order)
    Q = nq.value
    nodes, qx, qw = np.zeros((n, 3)), np.zeros((Q, 3)), np.zeros(Q)
    phi, dphi = np.zeros((Q, n)), np.zeros((Q, n, 3))
    p = [a.ctypes.data_as(C.c_void_p) for a in (nodes, qx, qw, phi, dphi)]
    assert fgpu_lib.fgpu_host_hex_ref_tables(order, qdeg, *p, C.byref(nq)) == 0
    pts, w = ho.quadrature(qdeg)
    assert Q == len(w)
    assert np.abs(qx - pts).max() < 1e-15 and np.abs(qw - w).max() < 1e-15
    assert np.array_equal(nodes, ho.dof_points(order))
    ph, dph = ho.tabulate(order, pts)
    assert np.abs(phi - ph).max() < 1e-14 and np.abs(dphi - dph).max() < 1e-14


def test_host_rejects_bad_input(fgpu_lib):
    xyz, hexes = meshgen.hex_box(1)
    bad = hexes.copy()
    bad[0, 3] = 99
    assert fgpu_lib.fgpu_host_hex_dof_table(len(xyz), 1, bad.ctypes.data_as(C.c_void_p), 1, None, None) != 0
    assert fgpu_lib.fgpu_host_hex_dof_table(len(xyz), 1, hexes.ctypes.data_as(C.c_void_p), 3, None, None) != 0
