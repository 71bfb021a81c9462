"""Host-side logic of the product (dof numbering, sparsity pattern, reference
tables) against the oracle; CPU only (host-only C-ABI queries)."""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import mesh


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def product_dofs(lib, xyz, tets, order, ncomp):
    T = len(tets)
    nl = (order + 1) * (order + 2) * (order + 3) // 6 * ncomp
    l2g = np.zeros((T, nl), dtype=np.int32)
    nd = C.c_int64()
    assert lib.fgpu_host_dof_table(len(xyz), T, _p(tets), order, ncomp, _p(l2g), C.byref(nd)) == 0
    return int(nd.value), l2g


def product_pattern(lib, xyz, tets, order, ncomp, N):
    ia = np.zeros(N + 1, dtype=np.int64)
    nnz = C.c_int64()
    assert lib.fgpu_host_pattern(len(xyz), len(tets), _p(tets), order, ncomp, _p(ia), None, C.byref(nnz)) == 0
    ja = np.zeros(nnz.value, dtype=np.int32)
    assert lib.fgpu_host_pattern(len(xyz), len(tets), _p(tets), order, ncomp, _p(ia), _p(ja), C.byref(nnz)) == 0
    return ia, ja


CASES = [(1, 1), (2, 1), (3, 1), (1, 3), (2, 3)]


@pytest.mark.parametrize("order,ncomp", CASES)
@pytest.mark.parametrize("n,perturb", [(1, 0.0), (3, 0.2), (5, 0.15)])
def test_dof_table_and_pattern_bit_exact(fgpu_lib, oracle, order, ncomp, n, perturb):
    xyz, tets = mesh(n, perturb=perturb)
    N, l2g = product_dofs(fgpu_lib, xyz, tets, order, ncomp)
    No, l2g_o = oracle.dof_table(tets, order, ncomp)
    assert N == No
    assert np.array_equal(l2g, l2g_o)
    ia, ja = product_pattern(fgpu_lib, xyz, tets, order, ncomp, N)
    ia_o, ja_o = oracle.pattern(No, l2g_o)
    assert np.array_equal(ia, ia_o) and np.array_equal(ja, ja_o)


@pytest.mark.parametrize("order", [1, 2, 3])
def test_shuffled_mesh_numbering(fgpu_lib, oracle, order):
    # element order and vertex ids permuted: first-encounter numbering and edge
    # permutations must still agree with the restated DofTable rules
    xyz, tets = mesh(3, perturb=0.1)
    rng = np.random.default_rng(7)
    perm_v = rng.permutation(len(xyz))
    inv = np.empty_like(perm_v)
    inv[perm_v] = np.arange(len(xyz))
    xyz2 = xyz[perm_v]
    tets2 = inv[tets][rng.permutation(len(tets))].astype(np.int32)
    tets2 = np.ascontiguousarray(tets2[:, rng.permutation(4)])
    N, l2g = product_dofs(fgpu_lib, xyz2, tets2, order, 1)
    No, l2g_o = oracle.dof_table(tets2, order, 1)
    assert N == No and np.array_equal(l2g, l2g_o)
    ia, ja = product_pattern(fgpu_lib, xyz2, tets2, order, 1, N)
    ia_o, ja_o = oracle.pattern(No, l2g_o)
    assert np.array_equal(ia, ia_o) and np.array_equal(ja, ja_o)


def test_single_element(fgpu_lib, oracle):
    tets = np.array([[0, 1, 2, 3]], dtype=np.int32)
    xyz = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=float)
    for order in (1, 2, 3):
        N, l2g = product_dofs(fgpu_lib, xyz, tets, order, 1)
        assert N == (order + 1) * (order + 2) * (order + 3) // 6
        assert np.array_equal(l2g[0], np.arange(N))


def test_bad_inputs_rejected(fgpu_lib):
    tets = np.array([[0, 1, 2, 7]], dtype=np.int32)   # vertex 7 out of range for nv = 4
    l2g = np.zeros((1, 4), dtype=np.int32)
    nd = C.c_int64()
    assert fgpu_lib.fgpu_host_dof_table(4, 1, _p(tets), 1, 1, _p(l2g), C.byref(nd)) == 1
    tets = np.array([[0, 1, 1, 3]], dtype=np.int32)   # repeated vertex
    assert fgpu_lib.fgpu_host_dof_table(4, 1, _p(tets), 1, 1, _p(l2g), C.byref(nd)) == 1
    assert fgpu_lib.fgpu_host_dof_table(4, 1, _p(tets), 4, 1, _p(l2g), C.byref(nd)) == 1   # order 4 unsupported
    assert fgpu_lib.fgpu_host_dof_table(4, 0, _p(tets), 1, 1, _p(l2g), C.byref(nd)) == 1   # empty mesh


@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("qdeg", [2, 4, 6])
def test_reference_tables_match_oracle_basis(fgpu_lib, oracle, order, qdeg):
    n = (order + 1) * (order + 2) * (order + 3) // 6
    Q = C.c_int()
    assert fgpu_lib.fgpu_host_ref_tables(order, qdeg, None, None, None, None, None, C.byref(Q)) == 0
    nodes = np.zeros((n, 3))
    phi = np.zeros((Q.value, n))
    dphi = np.zeros((Q.value, n, 3))
    S = np.zeros((9, n, n))
    M = np.zeros((n, n))
    fgpu_lib.fgpu_host_ref_tables(order, qdeg, _p(nodes), _p(phi), _p(dphi), _p(S), _p(M), C.byref(Q))
    assert np.abs(nodes - oracle.nodes(order)).max() < 1e-15 * 4
    q = oracle.quad(qdeg)
    ph, dph = oracle.tabulate(order, q[:, :3])
    assert np.abs(phi - ph).max() < 1e-14
    assert np.abs(dphi - dph).max() < 1e-13
    # reference tensors = quadrature sums of the oracle tabulation
    w = q[:, 3]
    S_o = np.einsum("q,qia,qjb->abij", w, dph, dph).reshape(9, n, n)
    M_o = np.einsum("q,qi,qj->ij", w, ph, ph)
    assert np.abs(S - S_o).max() < 1e-13 * max(1.0, np.abs(S_o).max())
    assert np.abs(M - M_o).max() < 1e-14
