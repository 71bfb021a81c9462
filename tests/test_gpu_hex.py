"""Hexahedral meshes on a GB300 against the oracle: Q1/Q2 dof tables, patterns, Laplace/mass matrices
(FP64 and FP32) and load vectors on perturbed hexahedra, boundary dofs, a Poisson solve (CG and AMG),
the EnSight export, and the paths that refuse hexahedra."""
import numpy as np
import pytest

import feelpp_gb300 as fpp
from feelpp_gb300 import meshgen
from oracle import hexoracle as ho
from tests.helpers import assert_values_close

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("order", [1, 2])
def test_hex_matrix_and_load_match_oracle(env, oracle, order):
    xyz, hexes = meshgen.hex_box(5, 4, 3, perturb=0.2)
    kappa = meshgen.lognormal_kappa(len(hexes))
    M = fpp.Mesh(xyz, hexes, env=env)
    V = fpp.Pch(M, order)
    N, l2g = ho.dof_table(hexes, order)
    assert V.ndof == N and np.array_equal(V.dof_l2g(), l2g)
    u, v = V.element(), V.element()
    expr = kappa * fpp.inner(fpp.gradt(u), fpp.grad(v)) + 0.7 * fpp.idt(u) * fpp.id(v)
    a = fpp.form2(test=V, trial=V)
    a.assign(fpp.integrate(fpp.elements(M), expr))
    ia, ja = oracle.pattern(N, l2g)
    dia, dja, dval = a.csr()
    assert np.array_equal(dia, ia) and np.array_equal(dja, ja)
    val = ho.assemble(order, xyz, hexes, l2g, ia, ja, kappa=kappa, mass=0.7)
    assert_values_close(dval, val, what="hex Laplace/mass")
    l = fpp.form1(test=V)
    l.assign(fpp.integrate(fpp.elements(M), fpp.sine_source() * fpp.id(v)))
    assert_values_close(l.to_numpy(), ho.rhs(order, xyz, hexes, l2g, N), what="hex load vector")
    # explicit quadrature degree
    a3 = fpp.form2(test=V, trial=V)
    a3.assign(fpp.integrate(fpp.elements(M), expr, quad=3))
    assert_values_close(a3.values(), ho.assemble(order, xyz, hexes, l2g, ia, ja, kappa=kappa, mass=0.7, qdeg=3),
                        what="hex matrix, degree 3")
    # binary32 within single-precision rounding; deterministic
    a32 = fpp.form2(test=V, trial=V, precision="f32")
    a32.assign(fpp.integrate(fpp.elements(M), expr))
    assert np.abs(a32.values() - val).max() <= 2e-5 * np.abs(val).max()
    a2 = fpp.form2(test=V, trial=V)
    a2.assign(fpp.integrate(fpp.elements(M), expr))
    assert np.array_equal(a2.values(), dval)


@pytest.mark.parametrize("order", [1, 2])
def test_hex_boundary_dofs(env, order):
    xyz, hexes = meshgen.hex_box(3, 4, 2, perturb=0.1)
    M = fpp.Mesh(xyz, hexes, env=env)
    V = fpp.Pch(M, order)
    N, l2g = ho.dof_table(hexes, order)
    mask = ho.boundary_mask(order, hexes, l2g, N)
    assert np.array_equal(np.sort(V.boundary_dofs()), np.flatnonzero(mask))


def test_hex_poisson_solve(env, oracle):
    order = 2
    xyz, hexes = meshgen.hex_box(6, perturb=0.15)
    M = fpp.Mesh(xyz, hexes, env=env)
    V = fpp.Pch(M, order)
    u, v = V.element(), V.element()
    a = fpp.form2(test=V, trial=V)
    a.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.gradt(u), fpp.grad(v))))
    l = fpp.form1(test=V)
    l.assign(fpp.integrate(fpp.elements(M), fpp.sine_source() * fpp.id(v)))
    a += fpp.on(fpp.boundaryfaces(M), rhs=l, element=u, expr=0.0, type="elimination_symmetric")
    st = a.solve(rhs=l, solution=u, rtol=1e-10)
    assert st["rel_residual"] <= 1e-10
    N, l2g = ho.dof_table(hexes, order)
    ia, ja = oracle.pattern(N, l2g)
    val = ho.assemble(order, xyz, hexes, l2g, ia, ja)
    b = ho.rhs(order, xyz, hexes, l2g, N)
    mask = ho.boundary_mask(order, hexes, l2g, N)
    oracle.dirichlet(ia, ja, val, b, mask, mode=1)
    x, it, res = oracle.pcg(ia, ja, val, b, rtol=1e-12)
    assert np.linalg.norm(u.to_numpy() - x) <= 1e-8 * np.linalg.norm(x)
    # the discrete solution approximates sin(pi x) sin(pi y) sin(pi z) at the vertices
    vx = np.zeros(N)
    vx[l2g[:, :8].reshape(-1)] = 1
    pv = np.zeros((N, 3))
    pv[l2g[:, :8].reshape(-1)] = xyz[hexes.reshape(-1)]
    ex = np.sin(np.pi * pv[:, 0]) * np.sin(np.pi * pv[:, 1]) * np.sin(np.pi * pv[:, 2])
    assert np.abs(u.to_numpy()[vx > 0] - ex[vx > 0]).max() < 2e-3
    w = V.element()
    sg = a.solve(rhs=l, solution=w, rtol=1e-10, pc="gamg")
    assert sg["rel_residual"] <= 1e-10
    assert np.linalg.norm(w.to_numpy() - x) <= 1e-7 * np.linalg.norm(x)


def test_hex_export(env, tmp_path):
    xyz, hexes = meshgen.hex_box(3, 2, 2)
    M = fpp.Mesh(xyz, hexes, env=env)
    V = fpp.Pch(M, 2)
    u = V.element()
    vals = np.arange(V.ndof, dtype=np.float64)
    u.upload(vals)
    prefix = str(tmp_path / "hexout")
    fpp.export_ensight(V, prefix, {"u": u})
    geo = open(prefix + ".geo", "rb").read()
    assert b"hexa8" in geo
    off = geo.index(b"hexa8") + 80
    ne = int(np.frombuffer(geo[off:off + 4], dtype=np.int32)[0])
    conn = np.frombuffer(geo[off + 4:off + 4 + 4 * 8 * ne], dtype=np.int32).reshape(ne, 8)
    assert ne == len(hexes) and np.array_equal(conn, hexes + 1)
    scl = open(prefix + ".u.scl", "rb").read()
    f = np.frombuffer(scl[3 * 80 + 4:], dtype=np.float32)
    _, l2g = ho.dof_table(hexes, 2)
    expect = np.zeros(len(xyz))
    expect[hexes.reshape(-1)] = vals[l2g[:, :8].reshape(-1)]
    assert np.array_equal(f, expect.astype(np.float32))


def test_hex_refusals(env):
    xyz, hexes = meshgen.hex_box(2)
    M = fpp.Mesh(xyz, hexes, env=env)
    with pytest.raises(fpp.FgpuError):
        fpp.Pch(M, 3)
    with pytest.raises(fpp.FgpuError):
        fpp.Pchv(M, 1)
    V = fpp.Pch(M, 1)
    u, v = V.element(), V.element()
    a = fpp.form2(test=V, trial=V)
    with pytest.raises(fpp.FgpuError):
        a.assign(fpp.integrate(fpp.boundaryfaces(M), 1.0 * fpp.idt(u) * fpp.id(v)))
    with pytest.raises(fpp.FgpuError):
        fpp.operator(V, fpp.integrate(fpp.elements(M), fpp.inner(fpp.gradt(u), fpp.grad(v))), precision="f32")
    with pytest.raises(fpp.FgpuError):
        a.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.gradt(u), fpp.grad(v)), quad=9))
    with pytest.raises(fpp.FgpuError):
        M.set_ho_nodes(np.zeros((len(hexes), 6, 3)))
    with pytest.raises(ValueError):
        fpp.Mesh(xyz, hexes[:, :6], env=env)
