"""Matrix-free operator and matrix-free CG against the assembled CSR (run on a GB300)."""
import numpy as np
import pytest

import feelpp_gb300 as fpp
from feelpp_gb300 import meshgen
from tests.helpers import mesh

pytestmark = pytest.mark.gpu

TOL = {"f64": 1e-13, "df64": 1e-12, "f32": 2e-6}


def system(env, n, order, with_dirichlet=True):
    xyz, tets = mesh(n, perturb=0.15)
    kappa = meshgen.lognormal_kappa(len(tets))
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, order)
    u, v = V.element(), V.element()
    integral = fpp.integrate(fpp.elements(M), kappa * fpp.inner(fpp.gradt(u), fpp.grad(v)) + 0.5 * (fpp.idt(u) * fpp.id(v)))
    a = fpp.form2(test=V, trial=V)
    a.assign(integral)
    l = fpp.form1(test=V)
    l.assign(fpp.integrate(fpp.elements(M), fpp.sine_source() * fpp.id(v)))
    if with_dirichlet:
        a += fpp.on(fpp.boundaryfaces(M), rhs=l, element=u, expr=0.0, type="elimination_symmetric")
    return xyz, tets, M, V, integral, a, l


@pytest.mark.parametrize("order,n", [(1, 8), (2, 6), (3, 4)])
@pytest.mark.parametrize("prec", ["f64", "df64", "f32"])
def test_operator_apply_matches_csr(env, order, n, prec):
    xyz, tets, M, V, integral, a, l = system(env, n, order)
    op = fpp.operator(V, integral, precision=prec)
    op.set_dirichlet(V.boundary_dofs())
    x = np.random.default_rng(5).standard_normal(V.ndof)
    xv, yv, zv = V.element(), V.element(), V.element()
    xv.upload(x)
    op.apply(xv, yv)
    a.mult(xv, zv)
    y, z = yv.to_numpy(), zv.to_numpy()
    assert np.abs(y - z).max() <= TOL[prec] * np.abs(z).max()


def test_operator_without_dirichlet(env):
    xyz, tets, M, V, integral, a, l = system(env, 5, 2, with_dirichlet=False)
    op = fpp.operator(V, integral, precision="f64")
    x = np.random.default_rng(6).standard_normal(V.ndof)
    xv, yv, zv = V.element(), V.element(), V.element()
    xv.upload(x)
    op.apply(xv, yv)
    a.mult(xv, zv)
    assert np.abs(yv.to_numpy() - zv.to_numpy()).max() <= 1e-13 * np.abs(zv.to_numpy()).max()


@pytest.mark.parametrize("order,n", [(2, 8), (3, 6)])
def test_mixed_matfree_solve(env, order, n):
    xyz, tets, M, V, integral, a, l = system(env, n, order)
    op64 = fpp.operator(V, integral, precision="f64")
    op32 = fpp.operator(V, integral, precision="f32")
    bd = V.boundary_dofs()
    op64.set_dirichlet(bd)
    op32.set_dirichlet(bd)
    u = V.element()
    st = op64.solve(l, u, rtol=1e-10, inner=op32)
    assert st["rel_residual"] <= 1e-10 and st["outer"] >= 2
    w = V.element()
    st64 = a.solve(rhs=l, solution=w, rtol=1e-10)
    assert st["iterations"] <= 1.25 * st64["iterations"] + 16
    a.solve(rhs=l, solution=w, rtol=1e-11)
    x, xr = u.to_numpy(), w.to_numpy()
    assert np.linalg.norm(x - xr) <= 1e-8 * np.linalg.norm(xr)


def test_plain_matfree_solve_df64(env):
    xyz, tets, M, V, integral, a, l = system(env, 6, 2)
    op = fpp.operator(V, integral, precision="df64")
    op.set_dirichlet(V.boundary_dofs())
    u = V.element()
    st = op.solve(l, u, rtol=1e-10)
    assert st["rel_residual"] <= 1e-9
    w = V.element()
    a.solve(rhs=l, solution=w, rtol=1e-11)
    assert np.linalg.norm(u.to_numpy() - w.to_numpy()) <= 1e-7 * np.linalg.norm(w.to_numpy())


def test_mixed_matfree_cheb_jacobi(env):
    xyz, tets, M, V, integral, a, l = system(env, 6, 3)
    op64 = fpp.operator(V, integral, precision="f64")
    op32 = fpp.operator(V, integral, precision="f32")
    bd = V.boundary_dofs()
    op64.set_dirichlet(bd)
    op32.set_dirichlet(bd)
    u = V.element()
    st = op64.solve(l, u, rtol=1e-10, inner=op32, pc="cheb_jacobi", cheb_degree=3)
    assert st["rel_residual"] <= 1e-10 and st["eig_max"] > 1.0
    w = V.element()
    stj = op64.solve(l, w, rtol=1e-10, inner=op32)
    assert st["iterations"] * 1.5 <= stj["iterations"]
    assert np.linalg.norm(u.to_numpy() - w.to_numpy()) <= 1e-8 * np.linalg.norm(w.to_numpy())


@pytest.mark.parametrize("order,n,dirichlet", [(1, 8, True), (2, 6, True), (3, 4, False)])
def test_colour_scatter_apply(env, order, n, dirichlet):
    xyz, tets, M, V, integral, a, l = system(env, n, order, with_dirichlet=dirichlet)
    opg = fpp.operator(V, integral, precision="f32")
    opc = fpp.operator(V, integral, precision="f32")
    opc.set_algo("colour")
    if dirichlet:
        opg.set_dirichlet(V.boundary_dofs())
        opc.set_dirichlet(V.boundary_dofs())
    x = np.random.default_rng(7).standard_normal(V.ndof)
    xv, yg, yc, zv = V.element(), V.element(), V.element(), V.element()
    xv.upload(x)
    opg.apply(xv, yg)
    opc.apply(xv, yc)
    a.mult(xv, zv)
    z = zv.to_numpy()
    assert np.abs(yc.to_numpy() - z).max() <= TOL["f32"] * np.abs(z).max()
    assert np.abs(yc.to_numpy() - yg.to_numpy()).max() <= TOL["f32"] * np.abs(z).max()
    # the colour order is fixed: two applies give the same bits
    y2 = V.element()
    opc.apply(xv, y2)
    assert np.array_equal(y2.to_numpy(), yc.to_numpy())


def test_colour_scatter_mixed_solve(env):
    xyz, tets, M, V, integral, a, l = system(env, 6, 3)
    op64 = fpp.operator(V, integral, precision="f64")
    op32 = fpp.operator(V, integral, precision="f32")
    op32.set_algo("colour")
    bd = V.boundary_dofs()
    op64.set_dirichlet(bd)
    op32.set_dirichlet(bd)
    u = V.element()
    st = op64.solve(l, u, rtol=1e-10, inner=op32)
    assert st["rel_residual"] <= 1e-10
    w = V.element()
    a.solve(rhs=l, solution=w, rtol=1e-11)
    assert np.linalg.norm(u.to_numpy() - w.to_numpy()) <= 1e-8 * np.linalg.norm(w.to_numpy())


def test_colour_scatter_rejects_f64(env):
    xyz, tets, M, V, integral, a, l = system(env, 4, 1)
    op = fpp.operator(V, integral, precision="f64")
    with pytest.raises(Exception):
        op.set_algo("colour")
