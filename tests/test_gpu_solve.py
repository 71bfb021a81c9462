"""Device CG / Jacobi solves against the oracle (run on a GB300)."""
import numpy as np
import pytest

import feelpp_gb300 as fpp
from tests.helpers import mesh, oracle_system

pytestmark = pytest.mark.gpu


def poisson(env, n, order, perturb=0.2, mode="elimination_symmetric"):
    xyz, tets = mesh(n, perturb=perturb)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, order)
    u, v = V.element(), V.element()
    a = fpp.form2(test=V, trial=V)
    a.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.gradt(u), fpp.grad(v))))
    l = fpp.form1(test=V)
    l.assign(fpp.integrate(fpp.elements(M), fpp.sine_source() * fpp.id(v)))
    a += fpp.on(fpp.boundaryfaces(M), rhs=l, element=u, expr=0.0, type=mode)
    return xyz, tets, M, V, u, a, l


@pytest.mark.parametrize("order,n", [(1, 16), (2, 8), (3, 5)])
def test_pcg_matches_oracle(env, oracle, order, n):
    xyz, tets, M, V, u, a, l = poisson(env, n, order)
    st = a.solve(rhs=l, solution=u, rtol=1e-10)
    assert st["rel_residual"] <= 1e-10
    N, l2g, ia, ja, val = oracle_system(oracle, xyz, tets, order, mass=0.0)
    b = oracle.rhs(order, xyz, tets, l2g, N, fkind=0)
    mask = oracle.boundary_mask(order, xyz, tets, l2g, N)
    oracle.dirichlet(ia, ja, val, b, mask, mode=1)
    x, it, res = oracle.pcg(ia, ja, val, b, rtol=1e-10)
    ud = u.to_numpy()
    assert np.linalg.norm(ud - x) <= 1e-8 * np.linalg.norm(x)
    # same Krylov method and preconditioner: iteration counts agree closely
    assert abs(st["iterations"] - it) <= max(2, 0.02 * it)


@pytest.mark.parametrize("order,n", [(2, 12), (3, 8)])
def test_mixed_precision_refinement_reaches_1e10(env, oracle, order, n):
    xyz, tets, M, V, u, a, l = poisson(env, n, order)
    st = a.solve(rhs=l, solution=u, rtol=1e-10, mixed=True)
    assert st["rel_residual"] <= 1e-10 and st["outer"] >= 2
    u64 = V.element()
    st64 = a.solve(rhs=l, solution=u64, rtol=1e-10)
    x32, x64 = u.to_numpy(), u64.to_numpy()
    assert np.linalg.norm(x32 - x64) <= 1e-8 * np.linalg.norm(x64)
    # reliable updates keep the Krylov space: the binary32 iteration count stays
    # close to the binary64 one (a restarted refinement needs about twice as many)
    assert st["iterations"] <= 1.25 * st64["iterations"] + 16
    # discretisation error within 1% of the FP64 solve's
    N, l2g = oracle.dof_table(tets, order)
    e32 = oracle.errors(order, xyz, tets, l2g, x32, 2 * order + 2 if 2 * order + 2 <= 8 else 8)
    e64 = oracle.errors(order, xyz, tets, l2g, x64, 2 * order + 2 if 2 * order + 2 <= 8 else 8)
    assert abs(e32[0] - e64[0]) <= 0.01 * e64[0]


@pytest.mark.parametrize("order,n", [(1, 16), (2, 8)])
def test_df64_solve_matches_f64(env, oracle, order, n):
    xyz, tets, M, V, u, a, l = poisson(env, n, order)
    st = a.solve(rhs=l, solution=u, rtol=1e-10, arith="df64")
    assert st["rel_residual"] <= 1e-9
    u64 = V.element()
    a.solve(rhs=l, solution=u64, rtol=1e-10)
    x, x64 = u.to_numpy(), u64.to_numpy()
    assert np.linalg.norm(x - x64) <= 1e-8 * np.linalg.norm(x64)


def test_manufactured_solution_rates(env, oracle):
    errs = []
    for n in (8, 16):
        xyz, tets, M, V, u, a, l = poisson(env, n, 2, perturb=0.0)
        a.solve(rhs=l, solution=u, rtol=1e-12)
        N, l2g = oracle.dof_table(tets, 2)
        errs.append(oracle.errors(2, xyz, tets, l2g, u.to_numpy(), 8))
    assert np.log2(errs[0][0] / errs[1][0]) > 2.7   # L2 ~ h^3
    assert np.log2(errs[0][1] / errs[1][1]) > 1.8   # H1 ~ h^2


@pytest.mark.parametrize("order", [1, 2, 3])
def test_device_error_norms_match_oracle(env, oracle, order):
    xyz, tets, M, V, u, a, l = poisson(env, 5, order)
    a.solve(rhs=l, solution=u, rtol=1e-12)
    q = min(2 * order + 2, 8)
    l2, h1 = u.errors_sine(q)
    N, l2g = oracle.dof_table(tets, order)
    ol2, oh1 = oracle.errors(order, xyz, tets, l2g, u.to_numpy(), q)
    assert abs(l2 - ol2) <= 1e-10 * ol2 and abs(h1 - oh1) <= 1e-10 * oh1


def test_elasticity_solve(env, oracle):
    xyz, tets = mesh(4, perturb=0.0, lengths=(4.0, 1.0, 1.0))
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pchv(M, 2)
    u, v = V.element(), V.element()
    a = fpp.form2(test=V, trial=V)
    a.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.stress(u, 1.0, 0.5), fpp.grad(v))))
    l = fpp.form1(test=V)
    l.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.cst_vec(0, 0, -1), fpp.id(v))))
    a += fpp.on(fpp.markedfaces(M, 0.0), rhs=l, element=u, expr=0.0, type="elimination_symmetric")
    st = a.solve(rhs=l, solution=u, rtol=1e-10, mixed=True)
    assert st["rel_residual"] <= 1e-10
    N, l2g, ia, ja, val = oracle_system(oracle, xyz, tets, 2, ncomp=3, kind=1, lam=1.0, mu=0.5)
    b = oracle.rhs(2, xyz, tets, l2g, N, fkind=1, fc=(0, 0, -1), ncomp=3)
    mask = oracle.boundary_mask(2, xyz, tets, l2g, N, ncomp=3, xplane=0.0)
    oracle.dirichlet(ia, ja, val, b, mask, mode=1)
    x, it, res = oracle.pcg(ia, ja, val, b, rtol=1e-12, maxit=100000)
    assert np.linalg.norm(u.to_numpy() - x) <= 1e-8 * np.linalg.norm(x)
    assert x.reshape(-1, 3)[:, 2].min() < 0          # the beam sags under (0, 0, -1)


def test_matrix_mult(env, oracle):
    xyz, tets, M, V, u, a, l = poisson(env, 6, 3)
    x = np.random.default_rng(0).standard_normal(V.ndof)
    xv, yv = V.element(), V.element()
    xv.upload(x)
    a.mult(xv, yv)
    ia, ja, val = a.csr()
    y = oracle.spmv(ia, ja, val, x)
    assert np.abs(yv.to_numpy() - y).max() <= 1e-13 * np.abs(y).max()


def _jacobi_lmax(ia, ja, val):
    """lambda_max of D^-1 A (as D^-1/2 A D^-1/2) for the small test systems."""
    import scipy.sparse as sp
    from scipy.sparse.linalg import eigsh
    n = len(ia) - 1
    A = sp.csr_matrix((val, ja, ia), shape=(n, n))
    d = 1.0 / np.sqrt(A.diagonal())
    S = sp.diags(d) @ A @ sp.diags(d)
    return float(eigsh(S, k=1, which="LA", return_eigenvectors=False)[0])


@pytest.mark.parametrize("order,n,degree", [(2, 8, 3), (3, 6, 4)])
def test_cheb_jacobi_pcg(env, oracle, order, n, degree):
    """Chebyshev-Jacobi PCG: same converged solution as the oracle's Jacobi PCG,
    fewer iterations, and a lambda_max estimate (x1.1) just above the true one."""
    xyz, tets, M, V, u, a, l = poisson(env, n, order)
    st = a.solve(rhs=l, solution=u, rtol=1e-10, pc="cheb_jacobi", cheb_degree=degree)
    assert st["rel_residual"] <= 1e-10
    w = V.element()
    stj = a.solve(rhs=l, solution=w, rtol=1e-10)
    assert st["iterations"] * 1.5 <= stj["iterations"]
    ia, ja, val = a.csr()
    lt = _jacobi_lmax(ia, ja, val)
    assert 0.98 * lt <= st["eig_max"] <= 1.15 * lt
    N, l2g, oia, oja, oval = oracle_system(oracle, xyz, tets, order, mass=0.0)
    b = oracle.rhs(order, xyz, tets, l2g, N, fkind=0)
    mask = oracle.boundary_mask(order, xyz, tets, l2g, N)
    oracle.dirichlet(oia, oja, oval, b, mask, mode=1)
    x, it, res = oracle.pcg(oia, oja, oval, b, rtol=1e-12)
    assert np.linalg.norm(u.to_numpy() - x) <= 1e-8 * np.linalg.norm(x)


def test_cheb_jacobi_mixed(env):
    xyz, tets, M, V, u, a, l = poisson(env, 10, 2)
    st = a.solve(rhs=l, solution=u, rtol=1e-10, mixed=True, pc="cheb_jacobi")
    assert st["rel_residual"] <= 1e-10 and st["outer"] >= 2
    w = V.element()
    stj = a.solve(rhs=l, solution=w, rtol=1e-10)
    assert np.linalg.norm(u.to_numpy() - w.to_numpy()) <= 1e-8 * np.linalg.norm(w.to_numpy())
    assert st["iterations"] * 1.5 <= stj["iterations"]


def test_bad_pc_name(env):
    xyz, tets, M, V, u, a, l = poisson(env, 3, 1)
    with pytest.raises(ValueError):
        a.solve(rhs=l, solution=u, pc="ilu")


def test_stiff_elasticity_true_residual(env):
    """A slender clamped beam (vector P2, 12x12x12 cells on [0,4]x[0,1]^2) is stiff enough
    for the CG recurrence residual to drift from b - A x: both solves must still stop on
    the true residual (residual replacement), and the mixed one must not return a worse
    iterate than FP64 would (best-iterate folding, FP64 fallback on binary32 stagnation)."""
    xyz, tets = mesh(12, perturb=0.1, lengths=(4.0, 1.0, 1.0))
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pchv(M, 2)
    u, v = V.element(), V.element()
    a = fpp.form2(test=V, trial=V)
    a.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.stress(u, 1.0, 0.5), fpp.grad(v))))
    l = fpp.form1(test=V)
    l.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.cst_vec(0, 0, -1), fpp.id(v))))
    a += fpp.on(fpp.markedfaces(M, 0.0), rhs=l, element=u, expr=0.0, type="elimination_symmetric")
    st64 = a.solve(rhs=l, solution=u, rtol=1e-10)
    assert st64["rel_residual"] <= 1e-10
    w = V.element()
    stm = a.solve(rhs=l, solution=w, rtol=1e-10, mixed=True)
    assert stm["rel_residual"] <= 1e-10
    x64, xm = u.to_numpy(), w.to_numpy()
    assert np.linalg.norm(xm - x64) <= 1e-6 * np.linalg.norm(x64)
