"""Curved (P2-geometry) tetrahedra on a GB300 against the oracle: Laplace/mass matrices (FP64 and FP32),
load vectors, the affine limit, a solve on a curved domain, and the paths that refuse curved meshes."""
import numpy as np
import pytest

import feelpp_gb300 as fpp
from feelpp_gb300 import meshgen
from tests.helpers import assert_values_close

pytestmark = pytest.mark.gpu


def curved(env, n, order, amp=0.1, perturb=0.1):
    xyz, tets, ho = meshgen.curved_box(n, amp=amp, perturb=perturb)
    M = fpp.Mesh(xyz, tets, env=env, ho=ho)
    V = fpp.Pch(M, order)
    return xyz, tets, ho, M, V


@pytest.mark.parametrize("order", [1, 2, 3])
def test_curved_matrix_and_load_match_oracle(env, oracle, order):
    xyz, tets, ho, M, V = curved(env, 4, order)
    kappa = meshgen.lognormal_kappa(len(tets))
    u, v = V.element(), V.element()
    a = fpp.form2(test=V, trial=V)
    a.assign(fpp.integrate(fpp.elements(M), kappa * fpp.inner(fpp.gradt(u), fpp.grad(v)) + 0.7 * fpp.idt(u) * fpp.id(v)))
    l = fpp.form1(test=V)
    l.assign(fpp.integrate(fpp.elements(M), fpp.sine_source() * fpp.id(v)))
    N, l2g = oracle.dof_table(tets, order)
    ia, ja = oracle.pattern(N, l2g)
    val = oracle.assemble_ho(order, xyz, tets, ho, l2g, ia, ja, kappa=kappa, mass=0.7)
    dia, dja, dval = a.csr()
    assert np.array_equal(dia, ia) and np.array_equal(dja, ja)
    assert_values_close(dval, val, what="curved Laplace/mass")
    F = oracle.rhs_ho(order, xyz, tets, ho, l2g, N)
    assert_values_close(l.to_numpy(), F, what="curved load vector")
    # binary32 matrices within single-precision rounding
    a32 = fpp.form2(test=V, trial=V, precision="f32")
    a32.assign(fpp.integrate(fpp.elements(M), kappa * fpp.inner(fpp.gradt(u), fpp.grad(v)) + 0.7 * fpp.idt(u) * fpp.id(v)))
    v32 = a32.values()
    assert np.abs(v32 - val).max() <= 2e-5 * np.abs(val).max()
    # deterministic
    a2 = fpp.form2(test=V, trial=V)
    a2.assign(fpp.integrate(fpp.elements(M), kappa * fpp.inner(fpp.gradt(u), fpp.grad(v)) + 0.7 * fpp.idt(u) * fpp.id(v)))
    assert np.array_equal(a2.values(), dval)


def test_straight_edges_equal_affine(env):
    xyz, tets, ho = meshgen.curved_box(4, amp=0.0, perturb=0.2)
    for order in (1, 2, 3):
        Ma = fpp.Mesh(xyz, tets, env=env)
        Mc = fpp.Mesh(xyz, tets, env=env, ho=ho)
        vals = []
        for M in (Ma, Mc):
            V = fpp.Pch(M, order)
            u, v = V.element(), V.element()
            a = fpp.form2(test=V, trial=V)
            a.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.gradt(u), fpp.grad(v)) + fpp.idt(u) * fpp.id(v),
                                   quad=2 * order + 2))
            vals.append(a.values())
        assert np.abs(vals[1] - vals[0]).max() <= 1e-12 * np.abs(vals[0]).max()


def test_curved_poisson_solve(env, oracle):
    order = 2
    xyz, tets, ho, M, V = curved(env, 6, order)
    u, v = V.element(), V.element()
    a = fpp.form2(test=V, trial=V)
    a.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.gradt(u), fpp.grad(v))))
    l = fpp.form1(test=V)
    l.assign(fpp.integrate(fpp.elements(M), fpp.cst(1.0) * fpp.id(v)))
    a += fpp.on(fpp.boundaryfaces(M), rhs=l, element=u, expr=0.0, type="elimination_symmetric")
    st = a.solve(rhs=l, solution=u, rtol=1e-10)
    assert st["rel_residual"] <= 1e-10
    N, l2g = oracle.dof_table(tets, order)
    ia, ja = oracle.pattern(N, l2g)
    val = oracle.assemble_ho(order, xyz, tets, ho, l2g, ia, ja, mass=0.0)
    b = oracle.rhs_ho(order, xyz, tets, ho, l2g, N, fkind=2, c=1.0)
    mask = oracle.boundary_mask(order, xyz, tets, l2g, N)
    oracle.dirichlet(ia, ja, val, b, mask, mode=1)
    x, it, res = oracle.pcg(ia, ja, val, b, rtol=1e-12)
    assert np.linalg.norm(u.to_numpy() - x) <= 1e-8 * np.linalg.norm(x)
    # AMG works on the curved system as on any SPD matrix
    w = V.element()
    sg = a.solve(rhs=l, solution=w, rtol=1e-10, pc="gamg")
    assert sg["rel_residual"] <= 1e-10


def test_curved_refusals(env):
    xyz, tets, ho, M, V = curved(env, 2, 1)
    u, v = V.element(), V.element()
    a = fpp.form2(test=V, trial=V)
    with pytest.raises(fpp.FgpuError):
        a.assign(fpp.integrate(fpp.boundaryfaces(M), 1.0 * fpp.idt(u) * fpp.id(v)))
    with pytest.raises(fpp.FgpuError):
        fpp.operator(V, fpp.integrate(fpp.elements(M), fpp.inner(fpp.gradt(u), fpp.grad(v))), precision="f32")
    # back to affine: face integrals work again
    M.set_ho_nodes(None)
    a.assign(fpp.integrate(fpp.boundaryfaces(M), 1.0 * fpp.idt(u) * fpp.id(v)))
