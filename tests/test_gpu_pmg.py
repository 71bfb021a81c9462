"""p-multigrid (matrix-free order-p smoothing, assembled P1 coarse level with AMG) for the matrix-free
CG on a GB300: convergence to the FP64 residual tolerance, the same solution as the assembled FP64 solve,
and far fewer iterations than Jacobi."""
import numpy as np
import pytest

import feelpp_gb300 as fpp
from feelpp_gb300 import meshgen
from tests.helpers import mesh

pytestmark = pytest.mark.gpu


def problem(env, n, order, kappa=None):
    xyz, tets = mesh(n, perturb=0.15)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, order)
    V1 = fpp.Pch(M, 1)
    u, v = V.element(), V.element()
    u1, v1 = V1.element(), V1.element()
    k = 1.0 if kappa is None else kappa
    integral = fpp.integrate(fpp.elements(M), k * fpp.inner(fpp.gradt(u), fpp.grad(v)))
    l = fpp.form1(test=V)
    l.assign(fpp.integrate(fpp.elements(M), fpp.sine_source() * fpp.id(v)))
    bd = V.boundary_dofs()
    lv = l.to_numpy()
    lv[bd] = 0.0
    l.vec.upload(lv)
    op64 = fpp.operator(V, integral, precision="f64")
    op32 = fpp.operator(V, integral, precision="f32")
    op64.set_dirichlet(bd)
    op32.set_dirichlet(bd)
    a1 = fpp.form2(test=V1, trial=V1)
    a1.assign(fpp.integrate(fpp.elements(M), k * fpp.inner(fpp.gradt(u1), fpp.grad(v1))))
    l1 = fpp.form1(test=V1)
    a1 += fpp.on(fpp.boundaryfaces(M), rhs=l1, element=u1, expr=0.0, type="elimination_symmetric")
    # assembled FP64 reference solve of the order-p system
    a = fpp.form2(test=V, trial=V)
    a.assign(integral)
    lc = fpp.form1(test=V)
    lc.assign(fpp.integrate(fpp.elements(M), fpp.sine_source() * fpp.id(v)))
    a += fpp.on(fpp.boundaryfaces(M), rhs=lc, element=u, expr=0.0, type="elimination_symmetric")
    return xyz, tets, M, V, l, op64, op32, a1, a, lc


@pytest.mark.parametrize("order,n", [(2, 8), (3, 6)])
def test_pmg_mixed_matfree(env, order, n):
    xyz, tets, M, V, l, op64, op32, a1, a, lc = problem(env, n, order)
    u = V.element()
    st = op64.solve(l, u, rtol=1e-10, inner=op32, pc="pmg", coarse=a1)
    assert st["rel_residual"] <= 1e-10
    assert st["pmg"]["lmax"] > 1.0 and st["pmg"]["coarse_rows"] == (n + 1) ** 3
    w = V.element()
    stj = op64.solve(l, w, rtol=1e-10, inner=op32)
    assert st["iterations"] <= 0.35 * stj["iterations"]
    ws = V.element()
    a.solve(rhs=lc, solution=ws, rtol=1e-12)
    assert np.linalg.norm(u.to_numpy() - ws.to_numpy()) <= 1e-8 * np.linalg.norm(ws.to_numpy())


def test_pmg_plain_df64_and_kappa(env):
    xyz, tets = mesh(6, perturb=0.15)
    kappa = meshgen.lognormal_kappa(len(tets))
    xyz, tets, M, V, l, op64, op32, a1, a, lc = problem(env, 6, 3, kappa=kappa)
    u = V.element()
    st = op64.solve(l, u, rtol=1e-10, pc="pmg", coarse=a1, smoother=op32)
    assert st["rel_residual"] <= 1e-10
    ws = V.element()
    a.solve(rhs=lc, solution=ws, rtol=1e-12)
    assert np.linalg.norm(u.to_numpy() - ws.to_numpy()) <= 1e-8 * np.linalg.norm(ws.to_numpy())
    # the preconditioner is deterministic: a second solve gives the same bits
    u2 = V.element()
    op64.solve(l, u2, rtol=1e-10, pc="pmg", coarse=a1, smoother=op32)
    assert np.array_equal(u2.to_numpy(), u.to_numpy())
