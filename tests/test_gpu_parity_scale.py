"""Parity with the oracle at the configurations' sizes (run on a GB300).

Full comparisons (pattern bit-exact, every value within |a - b| <= 1e-12 |b| + 1e-14 max|A|):
P2 on the 32^3 cube with lognormal kappa, P3 on 20^3, vector P2 elasticity on a 16x4x4 beam of
[0,4]x[0,1]^2, and a batch of uneven P1-P3 problems. At the headline 64^3 size the dof table is
compared in full, and a seeded sample of 10^4 rows of the P2 and P3 matrices is compared entry by
entry: the oracle assembles only the elements incident to the sampled rows (in element order, so
those rows receive every contribution in the reference's order) into the device pattern, and the
sampled rows' columns are checked against the rows the GraphCSR rule gives (sorted union of the
incident elements' dofs)."""
import numpy as np
import pytest

import feelpp_gb300 as fpp
from feelpp_gb300 import meshgen
from tests.helpers import assert_values_close, oracle_system

pytestmark = pytest.mark.gpu


def _device(env, xyz, tets, order, kappa, mass=1.0, ncomp=1, elasticity=None):
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.FunctionSpace(M, order, ncomp)
    u, v = V.element(), V.element()
    a = fpp.form2(test=V, trial=V)
    if elasticity is not None:
        a.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.stress(u, *elasticity), fpp.grad(v))))
    else:
        a.assign(fpp.integrate(fpp.elements(M), kappa * fpp.inner(fpp.gradt(u), fpp.grad(v)) + mass * fpp.idt(u) * fpp.id(v)))
    return M, V, a


@pytest.mark.parametrize("order,n", [(2, 32), (3, 20)])
def test_full_parity_lognormal_kappa(env, oracle, order, n):
    xyz, tets = meshgen.kuhn_box(n, perturb=0.15, seed=1234)
    kappa = meshgen.lognormal_kappa(len(tets), seed=5678)
    M, V, a = _device(env, xyz, tets, order, kappa)
    N, l2g, ia, ja, val = oracle_system(oracle, xyz, tets, order, kappa=kappa, mass=1.0)
    assert V.ndof == N and np.array_equal(V.dof_l2g(), l2g)
    dia, dja, dval = a.csr()
    assert np.array_equal(dia, ia) and np.array_equal(dja, ja)
    assert_values_close(dval, val, what="P%d %d^3" % (order, n))


def test_full_parity_elasticity_beam(env, oracle):
    xyz, tets = meshgen.kuhn_box(16, 4, 4, lengths=(4.0, 1.0, 1.0), perturb=0.1, seed=1234)
    M, V, a = _device(env, xyz, tets, 2, None, ncomp=3, elasticity=(1.0, 0.5))
    N, l2g, ia, ja, val = oracle_system(oracle, xyz, tets, 2, ncomp=3, kind=1, lam=1.0, mu=0.5)
    assert V.ndof == N and np.array_equal(V.dof_l2g(), l2g)
    dia, dja, dval = a.csr()
    assert np.array_equal(dia, ia) and np.array_equal(dja, ja)
    assert_values_close(dval, val, what="vector P2 elasticity 16x4x4 beam")


def test_batch_uneven_orders_against_oracle(env, oracle):
    rng = np.random.default_rng(4321)
    specs = [(int(rng.integers(3, 11)), int(rng.integers(1, 4))) for _ in range(12)]
    probs = []
    for k, (n, order) in enumerate(specs):
        xyz, tets = meshgen.kuhn_box(n, perturb=0.15, seed=1234 + k)
        kappa = meshgen.lognormal_kappa(len(tets), seed=5678 + k)
        M = fpp.Mesh(xyz, tets, env=env)
        V = fpp.Pch(M, order)
        u, v = V.element(), V.element()
        integral = fpp.integrate(fpp.elements(M), kappa * fpp.inner(fpp.gradt(u), fpp.grad(v)) + fpp.idt(u) * fpp.id(v))
        probs.append((xyz, tets, kappa, order, fpp.form2(test=V, trial=V), integral))
    batch = fpp.Batch([p[4] for p in probs], [p[5] for p in probs])
    batch.assemble()
    for xyz, tets, kappa, order, a, _ in probs:
        N, l2g, ia, ja, val = oracle_system(oracle, xyz, tets, order, kappa=kappa, mass=1.0)
        dia, dja, dval = a.csr()
        assert np.array_equal(dia, ia) and np.array_equal(dja, ja)
        assert_values_close(dval, val, what="batched P%d, %d tets" % (order, len(tets)))


@pytest.mark.parametrize("order", [2, 3])
def test_sampled_rows_at_64(env, oracle, order):
    n, nsample = 64, 10000
    xyz, tets = meshgen.kuhn_box(n, perturb=0.15, seed=1234)
    kappa = meshgen.lognormal_kappa(len(tets), seed=5678)
    M, V, a = _device(env, xyz, tets, order, kappa)
    N, l2g = oracle.dof_table(tets, order)
    assert V.ndof == N and np.array_equal(V.dof_l2g(), l2g)
    closed = {2: 230 * n ** 3 + 138 * n ** 2 + 24 * n + 1, 3: 1311 * n ** 3 + 459 * n ** 2 + 45 * n + 1}[order]
    dia, dja, dval = a.csr()
    assert a.nnz == closed
    rows = np.sort(np.random.default_rng(99).choice(N, size=nsample, replace=False))
    sel = np.zeros(N, dtype=bool)
    sel[rows] = True
    el = np.nonzero(sel[l2g].any(axis=1))[0]           # elements incident to a sampled row, in element order
    # GraphCSR rows: sorted union of the dofs of the elements incident to the row
    sub = l2g[el].astype(np.int64)
    keys = []
    for i in range(sub.shape[1]):
        m = sel[sub[:, i]]
        keys.append((sub[m, i][:, None] * N + sub[m]).reshape(-1))
    key = np.unique(np.concatenate(keys))
    kr, kc = key // N, key % N
    for r in rows[:: max(1, nsample // 2000)]:         # 2000 rows checked column by column
        assert np.array_equal(dja[dia[r]:dia[r + 1]], kc[np.searchsorted(kr, r):np.searchsorted(kr, r, side="right")])
    counts = np.bincount(kr, minlength=N)[rows]
    assert np.array_equal(counts, np.diff(dia)[rows])
    val = oracle.assemble(order, xyz, tets[el], l2g[el], dia, dja, kappa=kappa[el], mass=1.0, nthreads=1)
    idx = np.concatenate([np.arange(dia[r], dia[r + 1]) for r in rows])
    assert_values_close(dval[idx], val[idx], what="P%d 64^3, %d sampled rows" % (order, nsample))
