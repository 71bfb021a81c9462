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
