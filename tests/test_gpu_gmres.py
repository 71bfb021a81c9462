"""GMRES (the reference's default ksp-type) on a GB300: the non-symmetric system of the default on()
elimination and a non-symmetric Nitsche form, against the oracle and a sparse direct solve; Jacobi and
AMG right preconditioning, restarts, the iteration limit, a zero right-hand side, determinism."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import feelpp_gb300 as fpp
from feelpp_gb300 import meshgen

pytestmark = pytest.mark.gpu


def poisson(env, n, order, on_type):
    xyz, tets = meshgen.kuhn_box(n, perturb=0.15)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, order)
    u, v = V.element(), V.element()
    a = fpp.form2(test=V, trial=V)
    a.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.gradt(u), fpp.grad(v))))
    l = fpp.form1(test=V)
    l.assign(fpp.integrate(fpp.elements(M), fpp.sine_source() * fpp.id(v)))
    a += fpp.on(fpp.boundaryfaces(M), rhs=l, element=u, expr=0.0, type=on_type)
    return xyz, tets, M, V, a, l


def test_gmres_on_nonsymmetric_elimination(env, oracle):
    order = 2
    xyz, tets, M, V, a, l = poisson(env, 6, order, "elimination")
    ia, ja, val = a.csr()
    A = sp.csr_matrix((val, ja, ia))
    assert abs(A - A.T).max() > 0.1          # the elimination keeps the columns: not symmetric
    u = V.element()
    st = a.solve(rhs=l, solution=u, rtol=1e-10, ksp="gmres", pc="jacobi")
    assert st["rel_residual"] <= 1e-10
    # same solution as the symmetric elimination solved by the oracle's CG
    N, l2g = oracle.dof_table(tets, order)
    ia2, ja2 = oracle.pattern(N, l2g)
    val2 = oracle.assemble(order, xyz, tets, l2g, ia2, ja2, mass=0.0)
    b = oracle.rhs(order, xyz, tets, l2g, N)
    mask = oracle.boundary_mask(order, xyz, tets, l2g, N)
    oracle.dirichlet(ia2, ja2, val2, b, mask, mode=1)
    x, _, _ = oracle.pcg(ia2, ja2, val2, b, rtol=1e-12)
    assert np.linalg.norm(u.to_numpy() - x) <= 1e-8 * np.linalg.norm(x)
    # AMG right preconditioning: fewer iterations, same solution
    w = V.element()
    sg = a.solve(rhs=l, solution=w, rtol=1e-10, ksp="gmres", pc="gamg")
    assert sg["rel_residual"] <= 1e-10 and sg["iterations"] < st["iterations"]
    assert np.linalg.norm(w.to_numpy() - x) <= 1e-8 * np.linalg.norm(x)
    # deterministic
    u2 = V.element()
    a.solve(rhs=l, solution=u2, rtol=1e-10, ksp="gmres", pc="jacobi")
    assert np.array_equal(u2.to_numpy(), u.to_numpy())


def test_gmres_nonsymmetric_nitsche(env):
    """-int (grad u.n) v + int (grad v.n) u + gamma/h int u v: the non-symmetric Nitsche variant"""
    from feelpp_gb300 import N, hFace
    xyz, tets = meshgen.kuhn_box(5, perturb=0.1)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, 2)
    u, v = V.element(), V.element()
    bf = fpp.boundaryfaces(M)
    a = fpp.form2(test=V, trial=V)
    a.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.gradt(u), fpp.grad(v)) + 0.1 * fpp.idt(u) * fpp.id(v)))
    a += fpp.integrate(bf, -fpp.inner(fpp.gradt(u) * N(), fpp.id(v)) + fpp.inner(fpp.grad(v) * N(), fpp.idt(u))
                       + 10.0 * fpp.idt(u) * fpp.id(v) / hFace())
    l = fpp.form1(test=V)
    l.assign(fpp.integrate(fpp.elements(M), fpp.sine_source() * fpp.id(v)))
    ia, ja, val = a.csr()
    A = sp.csr_matrix((val, ja, ia))
    assert abs(A - A.T).max() > 1e-3
    xd = spla.spsolve(A.tocsc(), l.to_numpy())
    for pc in ("jacobi", "none"):
        w = V.element()
        st = a.solve(rhs=l, solution=w, rtol=1e-11, ksp="gmres", pc=pc, restart=40)
        assert st["rel_residual"] <= 1e-11
        assert np.linalg.norm(w.to_numpy() - xd) <= 1e-8 * np.linalg.norm(xd)


def test_gmres_restarts_limit_and_zero_rhs(env):
    xyz, tets, M, V, a, l = poisson(env, 4, 2, "elimination_symmetric")
    u = V.element()
    st = a.solve(rhs=l, solution=u, rtol=1e-10, ksp="gmres", pc="jacobi", restart=5)
    assert st["rel_residual"] <= 1e-10 and st["outer"] > 1
    w = V.element()
    with pytest.raises(fpp.FgpuError) as ei:
        a.solve(rhs=l, solution=w, rtol=1e-10, maxit=3, ksp="gmres", pc="jacobi")
    assert ei.value.code == 5
    z = fpp.form1(test=V)
    x0 = V.element()
    st0 = a.solve(rhs=z, solution=x0, rtol=1e-10, ksp="gmres")
    assert st0["iterations"] == 0 and not np.any(x0.to_numpy())
    with pytest.raises(ValueError):
        a.solve(rhs=l, solution=w, ksp="bicg")
    with pytest.raises(fpp.FgpuError):
        a.solve(rhs=l, solution=w, ksp="gmres", pc="cheb_jacobi")
