"""Time-dependent reassembly replayed from a captured CUDA graph (run on a GB300).

Backward Euler for the heat equation, (M + dt kappa(t) K) u^{n+1} = M u^n + dt F,
with kappa(t) = 1 + 0.5 sin t held in a device scalar: the captured step
(reassembly, right-hand side, Dirichlet rows) must reproduce the eager step, and
the reassembled matrix must match the oracle's M + dt kappa(t) K."""
import math

import numpy as np
import pytest

import feelpp_gb300 as fpp
from tests.helpers import assert_values_close, mesh, oracle_system

pytestmark = pytest.mark.gpu


def heat_setup(env, n=4, order=2):
    xyz, tets = mesh(n, perturb=0.15)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, order)
    u, v = V.element(), V.element()
    mass = fpp.form2(test=V, trial=V)
    mass.assign(fpp.integrate(fpp.elements(M), fpp.idt(u) * fpp.id(v)))
    F = fpp.form1(test=V)
    F.assign(fpp.integrate(fpp.elements(M), fpp.sine_source() * fpp.id(v)))
    bc = fpp.DirichletBC(V, V.boundary_dofs())
    return xyz, tets, M, V, u, v, mass, F, bc


def test_graph_reassembly_follows_device_scalar(env, oracle):
    xyz, tets, M, V, u, v, mass, F, bc = heat_setup(env)
    dt = 0.05
    kt = fpp.DeviceScalar(env, 1.0)
    A = fpp.form2(test=V, trial=V)
    step_integral = fpp.integrate(fpp.elements(M), dt * kt * fpp.inner(fpp.gradt(u), fpp.grad(v)) + fpp.idt(u) * fpp.id(v))
    A.assign(step_integral)                      # eager call first (allocates the records)
    with fpp.capture(env) as g:
        A.assign(step_integral)
    for t in (0.3, 1.7):
        kt.set(1.0 + 0.5 * math.sin(t))
        g.launch()
        N, l2g, ia, ja, val = oracle_system(oracle, xyz, tets, 2, kappa=None, mass=1.0)
        ref = oracle.assemble(2, xyz, tets, l2g, ia, ja, kappa_const=dt * (1.0 + 0.5 * math.sin(t)), mass=1.0)
        assert_values_close(A.values(), ref, what="M + dt kappa(t) K at t=%g" % t)


def test_backward_euler_graph_equals_eager(env):
    xyz, tets, M, V, u, v, mass, F, bc = heat_setup(env)
    dt, nsteps = 0.05, 6
    kt = fpp.DeviceScalar(env, 1.0)
    A = fpp.form2(test=V, trial=V)
    integral = fpp.integrate(fpp.elements(M), dt * kt * fpp.inner(fpp.gradt(u), fpp.grad(v)) + fpp.idt(u) * fpp.id(v))
    b = V.element()

    def step_ops(un):
        A.assign(integral)
        mass.mult(un, b)
        b.axpby(dt, F.vec, 1.0)
        A.apply_bc(bc, rhs=b)

    def run(use_graph):
        un = V.element()
        un.zero()
        step_ops(un)                              # eager warm-up (first calls allocate)
        g = None
        if use_graph:
            with fpp.capture(env) as g:
                step_ops(un)
        hist = []
        for k in range(nsteps):
            kt.set(1.0 + 0.5 * math.sin((k + 1) * dt))
            if use_graph:
                g.launch()
            else:
                step_ops(un)
            A.solve(rhs=b, solution=un, rtol=1e-12)
            hist.append(un.to_numpy().copy())
        return hist

    eager = run(False)
    graph = run(True)
    for e, gr in zip(eager, graph):
        assert np.array_equal(e, gr)
    assert np.linalg.norm(eager[-1]) > 0


def test_capture_rejects_sync_calls(env):
    xyz, tets, M, V, u, v, mass, F, bc = heat_setup(env, n=2, order=1)
    w = V.element()
    with pytest.raises(fpp.FgpuError):
        with fpp.capture(env):
            mass.solve(rhs=F, solution=w)
    # the context is usable afterwards
    mass.mult(F.vec, w)
    assert np.isfinite(w.to_numpy()).all()


def test_bc_apply_equals_on(env):
    xyz, tets, M, V, u, v, mass, F, bc = heat_setup(env, n=3, order=2)
    a1 = fpp.form2(test=V, trial=V)
    a2 = fpp.form2(test=V, trial=V)
    integral = fpp.integrate(fpp.elements(M), fpp.inner(fpp.gradt(u), fpp.grad(v)))
    a1.assign(integral)
    a2.assign(integral)
    l1, l2 = fpp.form1(test=V), fpp.form1(test=V)
    for l in (l1, l2):
        l.assign(fpp.integrate(fpp.elements(M), fpp.sine_source() * fpp.id(v)))
    a1 += fpp.on(fpp.boundaryfaces(M), rhs=l1, element=u, expr=0.0, type="elimination_symmetric")
    a2.apply_bc(bc, rhs=l2, type="elimination_symmetric")
    assert np.array_equal(a1.values(), a2.values())
    assert np.array_equal(l1.to_numpy(), l2.to_numpy())
