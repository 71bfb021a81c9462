"""Smoothed-aggregation AMG set-up (host logic, CPU only) against its definition:
Galerkin coarse operators A_{l+1} = P^T A_l P, prolongators P = (I - omega D^-1 A) P0 with
P0(i, agg(i)) = 1/sqrt(|agg|) and omega = 4/(3 lmax), aggregation covering every coupled row,
lmax estimates against scipy, the dense coarsest inverse, and independence of the thread count."""
import ctypes as C

import numpy as np
import pytest

from feelpp_gb300 import _ffi
from tests.helpers import mesh, oracle_system

sp = pytest.importorskip("scipy.sparse")
spla = pytest.importorskip("scipy.sparse.linalg")


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class Hier:
    def __init__(self, lib, ia, ja, a, nthreads=1, **cfg):
        self.lib = lib
        c = _ffi.AmgCfg(cfg.get("threshold", 0.0), cfg.get("max_levels", 0), cfg.get("coarse_eq_lim", 0),
                        cfg.get("agg_smooths", 0), 0)
        h = C.c_void_p()
        ia, ja, a = (np.ascontiguousarray(ia, np.int64), np.ascontiguousarray(ja, np.int32),
                     np.ascontiguousarray(a, np.float64))
        assert lib.fgpu_amg_host_build(len(ia) - 1, _p(ia), _p(ja), _p(a), C.byref(c), nthreads, C.byref(h)) == 0
        self.h = h

    def __del__(self):
        self.lib.fgpu_amg_host_destroy(self.h)

    def nlevels(self):
        return self.lib.fgpu_amg_host_levels(self.h)

    def level(self, l):
        n, nnz, pnnz, pcols = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        lmax = C.c_double()
        assert self.lib.fgpu_amg_host_level(self.h, l, C.byref(n), C.byref(nnz), C.byref(pnnz), C.byref(pcols),
                                            C.byref(lmax)) == 0
        n, nnz, pnnz, pcols = n.value, nnz.value, pnnz.value, pcols.value
        ia = np.zeros(n + 1, np.int64)
        ja = np.zeros(nnz, np.int32)
        a = np.zeros(nnz)
        pia = np.zeros(n + 1, np.int64)
        pja = np.zeros(max(pnnz, 1), np.int32)
        pa = np.zeros(max(pnnz, 1))
        agg = np.zeros(max(n, 1), np.int32)
        last = l == self.nlevels() - 1
        assert self.lib.fgpu_amg_host_export(self.h, l, _p(ia), _p(ja), _p(a), None if last else _p(pia),
                                             None if last else _p(pja), None if last else _p(pa),
                                             None if last else _p(agg)) == 0
        A = sp.csr_matrix((a, ja, ia), shape=(n, n))
        P = None if last else sp.csr_matrix((pa[:pnnz], pja[:pnnz], pia), shape=(n, pcols))
        return A, P, (None if last else agg[:n]), lmax.value


def laplacian(oracle, n, order, dirichlet=True):
    xyz, tets = mesh(n, perturb=0.15)
    N, l2g, ia, ja, val = oracle_system(oracle, xyz, tets, order, mass=0.0)
    if dirichlet:
        b = np.zeros(N)
        mask = oracle.boundary_mask(order, xyz, tets, l2g, N)
        oracle.dirichlet(ia, ja, val, b, mask, mode=1)        # in place
    return ia, ja, val


@pytest.mark.parametrize("order,n", [(1, 8), (2, 4), (3, 3)])
def test_galerkin_hierarchy(fgpu_lib, oracle, order, n):
    ia, ja, val = laplacian(oracle, n, order)
    H = Hier(fgpu_lib, ia, ja, val, coarse_eq_lim=30)
    L = H.nlevels()
    assert L >= 2
    prev = None
    for l in range(L):
        A, P, agg, lmax = H.level(l)
        if l == 0:
            A0 = sp.csr_matrix((val, ja, ia), shape=A.shape)
            assert (A - A0).count_nonzero() == 0
        if prev is not None:
            Ap, Pp = prev
            G = (Pp.T @ Ap @ Pp).tocsr()
            assert abs(A - G).max() <= 1e-12 * abs(G).max()
        # lmax(D^-1 A) against scipy (Lanczos lower bound within a few percent)
        d = A.diagonal()
        S = sp.diags(1 / np.sqrt(d)) @ A @ sp.diags(1 / np.sqrt(d))
        true = spla.eigsh(S, k=1, which="LA", return_eigenvectors=False)[0] if A.shape[0] > 8 else np.linalg.eigvalsh(S.toarray()).max()
        assert 0.85 * true <= lmax <= true * (1 + 1e-8)
        if P is not None:
            coupled = np.asarray(abs(A - sp.diags(d)).sum(axis=1)).ravel() > 0     # nonzero off-diagonal couplings
            assert np.all(agg[coupled] >= 0) and np.all(agg[~coupled] == -1)
            nagg = P.shape[1]
            assert set(agg[agg >= 0]) == set(range(nagg))
            size = np.bincount(agg[agg >= 0], minlength=nagg)
            rows = np.nonzero(agg >= 0)[0]
            P0 = sp.csr_matrix((1 / np.sqrt(size[agg[rows]]), (rows, agg[rows])), shape=P.shape)
            omega = 4.0 / (3.0 * lmax)
            Pdef = (P0 - omega * sp.diags(1 / d) @ A @ P0).tocsr()
            assert abs(P - Pdef).max() <= 1e-13 * abs(Pdef).max()
            assert nagg < A.shape[0]
        prev = (A, P)
    assert H.level(L - 1)[0].shape[0] <= 30 or L == 10


def test_coarse_inverse_and_threads(fgpu_lib, oracle):
    ia, ja, val = laplacian(oracle, 6, 2)
    H1 = Hier(fgpu_lib, ia, ja, val, nthreads=1, coarse_eq_lim=60)
    H4 = Hier(fgpu_lib, ia, ja, val, nthreads=4, coarse_eq_lim=60)
    assert H1.nlevels() == H4.nlevels()
    for l in range(H1.nlevels()):
        A1, P1, g1, m1 = H1.level(l)
        A4, P4, g4, m4 = H4.level(l)
        assert np.array_equal(A1.data, A4.data) and np.array_equal(A1.indices, A4.indices) and m1 == m4
        if P1 is not None:
            assert np.array_equal(P1.data, P4.data) and np.array_equal(g1, g4)
    Ac = H1.level(H1.nlevels() - 1)[0].toarray()
    inv = np.zeros(Ac.size)
    assert fgpu_lib.fgpu_amg_host_coarse_inverse(H1.h, _p(inv)) == 1
    assert np.abs(inv.reshape(Ac.shape) @ Ac - np.eye(len(Ac))).max() <= 1e-10


def test_unsmoothed_and_threshold(fgpu_lib, oracle):
    ia, ja, val = laplacian(oracle, 6, 1)
    H = Hier(fgpu_lib, ia, ja, val, agg_smooths=-1, coarse_eq_lim=20)
    A, P, agg, _ = H.level(0)
    # unsmoothed: P = P0, one entry per aggregated row, orthonormal columns
    assert np.all(np.diff(P.indptr) <= 1)
    assert np.allclose((P.T @ P).toarray(), np.eye(P.shape[1]), atol=1e-14)
    # a strength threshold drops weak couplings: never more aggregates than rows, and the
    # Galerkin identity still holds
    Ht = Hier(fgpu_lib, ia, ja, val, threshold=0.2, coarse_eq_lim=20)
    A0, P0, _, _ = Ht.level(0)
    A1 = Ht.level(1)[0]
    G = (P0.T @ A0 @ P0).tocsr()
    assert abs(A1 - G).max() <= 1e-12 * abs(G).max()


def _elasticity_beam(oracle, n):
    """clamped P1 elasticity beam of [0,4]x[0,1]^2 (lambda 1, mu 0.5), its rigid body modes at the nodes"""
    xyz, tets = mesh(n, perturb=0.1, lengths=(4.0, 1.0, 1.0))
    N, l2g, ia, ja, val = oracle_system(oracle, xyz, tets, 1, ncomp=3, kind=1, lam=1.0, mu=0.5)
    # P1 nodes are the mesh vertices: node coordinates through the scalar dof table
    Ns, l2s = oracle.dof_table(tets, 1)
    X = np.zeros((Ns, 3))
    X[l2s.ravel()] = xyz[tets.ravel()]
    mask = np.zeros(N, dtype=np.uint8)
    mask[(3 * np.nonzero(X[:, 0] <= 1e-12)[0][:, None] + np.arange(3)).ravel()] = 1
    oracle.dirichlet(ia, ja, val, np.zeros(N), mask, mode=1)
    c = X.mean(axis=0)
    x, y, z = (X - c).T
    o, one = np.zeros(Ns), np.ones(Ns)
    modes = [(one, o, o), (o, one, o), (o, o, one), (-y, x, o), (o, -z, y), (z, o, -x)]
    B = np.stack([np.stack(m, axis=1).ravel() for m in modes])        # 6 x N, node-major dofs
    return ia, ja, val, B, mask


def _nns_hier(lib, ia, ja, a, B, **cfg):
    c = _ffi.AmgCfg(cfg.get("threshold", 0.0), cfg.get("max_levels", 0), cfg.get("coarse_eq_lim", 0), cfg.get("agg_smooths", 0), 0)
    Bc = np.ascontiguousarray(B, np.float64)
    c.block_size, c.nns_count, c.nns_host = 3, len(B), Bc.ctypes.data
    h = C.c_void_p()
    ia, ja, a = np.ascontiguousarray(ia, np.int64), np.ascontiguousarray(ja, np.int32), np.ascontiguousarray(a, np.float64)
    assert lib.fgpu_amg_host_build(len(ia) - 1, _p(ia), _p(ja), _p(a), C.byref(c), 2, C.byref(h)) == 0
    H = Hier.__new__(Hier)
    H.lib, H.h = lib, h
    return H


def test_rigid_body_near_null_space(fgpu_lib, oracle):
    """Aggregation by nodes, the tentative prolongator spans the rigid body modes on each aggregate
    (orthonormal columns), and the Galerkin identity holds on every level."""
    ia, ja, val, B, mask = _elasticity_beam(oracle, 6)
    Hu = _nns_hier(fgpu_lib, ia, ja, val, B, agg_smooths=-1, coarse_eq_lim=60)
    A, P, agg, _ = Hu.level(0)
    assert np.array_equal(agg[0::3], agg[1::3]) and np.array_equal(agg[0::3], agg[2::3])     # whole nodes
    assert np.allclose((P.T @ P).toarray(), np.eye(P.shape[1]), atol=1e-13)
    rows = agg >= 0
    Bt = B.T * rows[:, None]
    assert np.abs(Bt - P @ (P.T @ Bt)).max() <= 1e-10 * np.abs(Bt).max()
    nagg = agg.max() + 1
    assert 3 * nagg <= P.shape[1] <= 6 * nagg
    H = _nns_hier(fgpu_lib, ia, ja, val, B, coarse_eq_lim=60)
    prev = None
    for l in range(H.nlevels()):
        A, P, agg, lmax = H.level(l)
        if prev is not None:
            Ap, Pp = prev
            G = (Pp.T @ Ap @ Pp).tocsr()
            assert abs(A - G).max() <= 1e-12 * abs(G).max()
        prev = (A, P)
    assert H.nlevels() >= 2


@pytest.mark.parametrize("seed,nodes,bs,density", [(0, 40, 3, 0.05), (1, 25, 2, 0.2), (2, 60, 3, 0.01)])
def test_node_graph_of_symmetrised_graph(seed, nodes, bs, density):
    """The device set-up of a level with a near null space symmetrises the node graph of the strength
    graph, N(S) + N(S)^T, instead of taking the node graph of the symmetrised dof graph, N(S + S^T): the
    two are the same sorted node rows (a node pair is coupled when some dof pair of theirs is, in
    either direction). Checked on random non-symmetric dof graphs with bs dofs per node."""
    rng = np.random.default_rng(seed)
    n = nodes * bs
    S = sp.random(n, n, density=density, random_state=rng, format="csr")
    S.data[:] = 1.0
    S.setdiag(0.0)
    S.eliminate_zeros()
    node = np.arange(n) // bs
    inc = sp.csr_matrix((np.ones(n), (node, np.arange(n))), shape=(nodes, n))   # node x dof incidence

    def node_graph(G):
        N = (inc @ G @ inc.T).tocsr()
        N.setdiag(0.0)
        N.eliminate_zeros()
        N.data[:] = 1.0
        N.sort_indices()
        return N

    a = node_graph(S + S.T)
    NS = node_graph(S)
    b = (NS + NS.T).tocsr()
    b.data[:] = 1.0
    b.sort_indices()
    assert np.array_equal(a.indptr, b.indptr) and np.array_equal(a.indices, b.indices)
