"""Boundary-face integrals against the oracle (run on a GB300):
form2 = integrate(boundaryfaces | markedfaces, alpha*idt(u)*id(v)) and
form1 = integrate(boundaryfaces | markedfaces, g*id(v)), scalar P1-P3."""
import numpy as np
import pytest

import feelpp_gb300 as fpp
from tests.helpers import assert_values_close, mesh

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("marked", [False, True])
def test_face_mass_and_load(env, oracle, order, marked):
    xyz, tets = mesh(4, perturb=0.2)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, order)
    u, v = V.element(), V.element()
    rng = fpp.markedfaces(M, 0.0) if marked else fpp.boundaryfaces(M)
    a = fpp.form2(test=V, trial=V)
    a.assign(fpp.integrate(rng, 2.5 * (fpp.idt(u) * fpp.id(v))))
    l = fpp.form1(test=V)
    l.assign(fpp.integrate(rng, 3.0 * fpp.id(v)))
    N, l2g = oracle.dof_table(tets, order)
    ia, ja = oracle.pattern(N, l2g)
    val = oracle.face_matrix(order, xyz, tets, l2g, ia, ja, 2.5, xplane=0.0 if marked else None)
    F = oracle.face_load(order, xyz, tets, l2g, N, 3.0, xplane=0.0 if marked else None)
    dia, dja, dval = a.csr()
    assert np.array_equal(dia, ia) and np.array_equal(dja, ja)
    assert_values_close(dval, val, what="face mass")
    assert_values_close(l.to_numpy(), F, what="face load")
    area = 1.0 if marked else 6.0
    assert abs(dval.sum() - 2.5 * area) < 1e-11 and abs(l.to_numpy().sum() - 3.0 * area) < 1e-11


def test_robin_plus_volume_form(env, oracle):
    """a = kappa grad.grad + alpha (boundary) u v, assembled as a volume '=' then a face '+='."""
    from tests.helpers import oracle_system
    xyz, tets = mesh(3, perturb=0.1)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, 2)
    u, v = V.element(), V.element()
    a = fpp.form2(test=V, trial=V)
    a.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.gradt(u), fpp.grad(v))))
    a += fpp.integrate(fpp.boundaryfaces(M), 0.7 * (fpp.idt(u) * fpp.id(v)))
    N, l2g, ia, ja, val = oracle_system(oracle, xyz, tets, 2, mass=0.0)
    oracle.face_matrix(2, xyz, tets, l2g, ia, ja, 0.7, val=val)
    assert_values_close(a.values(), val, what="volume + Robin")
    # the Robin term makes the pure-Neumann Laplacian definite: CG solves it
    l = fpp.form1(test=V)
    l.assign(fpp.integrate(fpp.boundaryfaces(M), 1.0 * fpp.id(v)))
    w = V.element()
    st = a.solve(rhs=l, solution=w, rtol=1e-10)
    assert st["rel_residual"] <= 1e-10
    # u = 1/0.7 solves -lap u = 0, du/dn + 0.7 u = 1
    assert np.allclose(w.to_numpy(), 1.0 / 0.7, rtol=1e-8)


@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("marked", [False, True])
def test_nitsche_face_terms(env, oracle, order, marked):
    """The weak-Dirichlet terms of cg_laplacian.hpp, written as there, against the oracle:
    -inner(k*gradt(u)*N(), id(v)) - inner(k*grad(v)*N(), idt(u)) + 2*k*idt(u)*id(v)/hFace() and
    -inner(k*grad(v)*N(), g) + 2*k*g*id(v)/hFace(), plus a Robin term in the same integral."""
    from feelpp_gb300 import N, hFace
    k, g, alpha = 1.3, 0.4, 0.25
    xyz, tets = mesh(3, perturb=0.2)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, order)
    u, v = V.element(), V.element()
    rng = fpp.markedfaces(M, 0.0) if marked else fpp.boundaryfaces(M)
    a = fpp.form2(test=V, trial=V)
    a.assign(fpp.integrate(rng, -fpp.inner(k * fpp.gradt(u) * N(), fpp.id(v)) - fpp.inner(k * fpp.grad(v) * N(), fpp.idt(u))
                           + 2 * k * fpp.idt(u) * fpp.id(v) / hFace() + alpha * fpp.idt(u) * fpp.id(v)))
    l = fpp.form1(test=V)
    l.assign(fpp.integrate(rng, -fpp.inner(k * fpp.grad(v) * N(), g) + 2 * k * g * fpp.id(v) / hFace()))
    Nd, l2g = oracle.dof_table(tets, order)
    ia, ja = oracle.pattern(Nd, l2g)
    xp = 0.0 if marked else None
    val = oracle.face_terms_matrix(order, xyz, tets, l2g, ia, ja, mass=alpha, mass_h=2 * k, dn_trial=-k, dn_test=-k, xplane=xp)
    F = oracle.face_terms_load(order, xyz, tets, l2g, Nd, g_h=2 * k * g, g_dn=-k * g, xplane=xp)
    dia, dja, dval = a.csr()
    assert np.array_equal(dia, ia) and np.array_equal(dja, ja)
    assert_values_close(dval, val, what="Nitsche face matrix")
    assert_values_close(l.to_numpy(), F, what="Nitsche face load")
    # deterministic: a second assembly gives the same bits
    a2 = fpp.form2(test=V, trial=V)
    a2.assign(fpp.integrate(rng, -fpp.inner(k * fpp.gradt(u) * N(), fpp.id(v)) - fpp.inner(k * fpp.grad(v) * N(), fpp.idt(u))
                            + 2 * k * fpp.idt(u) * fpp.id(v) / hFace() + alpha * fpp.idt(u) * fpp.id(v)))
    assert np.array_equal(a2.values(), dval)


def test_nitsche_weak_dirichlet_solve(env, oracle):
    """Symmetric Nitsche Poisson (gamma = 20): g = c, f = 0 gives u = c; with the sine source and g = 0
    the L2 error is within a few percent of the strongly imposed (on()) solution's."""
    from feelpp_gb300 import N, hFace
    k, gamma, c, order = 1.0, 20.0, 0.7, 2
    xyz, tets = mesh(6, perturb=0.1)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, order)
    u, v = V.element(), V.element()
    bf = fpp.boundaryfaces(M)
    a = fpp.form2(test=V, trial=V)
    a.assign(fpp.integrate(fpp.elements(M), fpp.inner(k * fpp.gradt(u), fpp.grad(v))))
    a += fpp.integrate(bf, -fpp.inner(k * fpp.gradt(u) * N(), fpp.id(v)) - fpp.inner(k * fpp.grad(v) * N(), fpp.idt(u))
                       + gamma * k * fpp.idt(u) * fpp.id(v) / hFace())
    l = fpp.form1(test=V)
    l.assign(fpp.integrate(bf, -fpp.inner(k * fpp.grad(v) * N(), c) + gamma * k * c * fpp.id(v) / hFace()))
    w = V.element()
    st = a.solve(rhs=l, solution=w, rtol=1e-12)
    assert st["rel_residual"] <= 1e-12
    assert np.abs(w.to_numpy() - c).max() <= 1e-9
    ls = fpp.form1(test=V)
    ls.assign(fpp.integrate(fpp.elements(M), fpp.sine_source() * fpp.id(v)))
    ws = V.element()
    st = a.solve(rhs=ls, solution=ws, rtol=1e-10)
    e_weak = ws.errors_sine(6)[0]
    b = fpp.form2(test=V, trial=V)
    b.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.gradt(u), fpp.grad(v))))
    lb = fpp.form1(test=V)
    lb.assign(fpp.integrate(fpp.elements(M), fpp.sine_source() * fpp.id(v)))
    b += fpp.on(bf, rhs=lb, element=u, expr=0.0, type="elimination_symmetric")
    wb = V.element()
    b.solve(rhs=lb, solution=wb, rtol=1e-10)
    e_strong = wb.errors_sine(6)[0]
    assert e_weak <= 3.0 * e_strong
