"""Edge cases on a GB300 against the oracle: the smallest meshes (one tetrahedron, one hexahedron),
vertices no element uses, negatively oriented elements, an empty Dirichlet set, a zero right-hand side,
and inputs the library must refuse without touching the device."""
import ctypes as C

import numpy as np
import pytest

import feelpp_gb300 as fpp
from feelpp_gb300 import _ffi, meshgen
from oracle import hexoracle
from tests.helpers import assert_values_close

pytestmark = pytest.mark.gpu


def laplace_mass(M, V, kappa=None):
    u, v = V.element(), V.element()
    k = 1.0 if kappa is None else kappa
    a = fpp.form2(test=V, trial=V)
    a.assign(fpp.integrate(fpp.elements(M), k * fpp.inner(fpp.gradt(u), fpp.grad(v)) + 0.5 * fpp.idt(u) * fpp.id(v)))
    return a


@pytest.mark.parametrize("order", [1, 2, 3])
def test_single_tetrahedron(env, oracle, order):
    xyz = np.array([[0.1, 0.0, 0.0], [1.0, 0.2, 0.0], [0.0, 1.0, 0.1], [0.2, 0.1, 0.9]])
    tets = np.array([[0, 1, 2, 3]], dtype=np.int32)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, order)
    a = laplace_mass(M, V)
    N, l2g = oracle.dof_table(tets, order)
    ia, ja = oracle.pattern(N, l2g)
    assert V.ndof == N and a.nnz == N * N
    val = oracle.assemble(order, xyz, tets, l2g, ia, ja, kappa_const=1.0, mass=0.5)
    assert_values_close(a.values(), val, what="one tetrahedron")


@pytest.mark.parametrize("order", [1, 2])
def test_single_hexahedron(env, order):
    xyz = hexoracle.HEX_VERTS * np.array([0.5, 0.7, 0.4]) + 0.05 * np.sin(np.arange(24)).reshape(8, 3)
    hexes = np.arange(8, dtype=np.int32)[None, :]
    M = fpp.Mesh(xyz, hexes, env=env)
    V = fpp.Pch(M, order)
    a = laplace_mass(M, V)
    N, l2g = hexoracle.dof_table(hexes, order)
    ia = np.arange(N + 1, dtype=np.int64) * N
    ja = np.tile(np.arange(N, dtype=np.int32), N)
    val = hexoracle.assemble(order, xyz, hexes, l2g, ia, ja, mass=0.5)
    assert_values_close(a.values(), val, what="one hexahedron")


def test_unused_vertices_and_negative_orientation(env, oracle):
    """vertices no element references get no dof; elements with det K < 0 integrate with |det K|"""
    xyz, tets = meshgen.kuhn_box(3, perturb=0.2)
    extra = np.array([[5.0, 5.0, 5.0], [6.0, 6.0, 6.0]])
    xyz2 = np.vstack([extra, xyz])                  # two unused vertices first: every id shifts by 2
    tets2 = tets + 2
    tets2[::2] = tets2[::2][:, [1, 0, 2, 3]]        # every other element negatively oriented
    kappa = meshgen.lognormal_kappa(len(tets))
    for order in (1, 2, 3):
        M = fpp.Mesh(xyz2, tets2, env=env)
        V = fpp.Pch(M, order)
        a = laplace_mass(M, V, kappa)
        N, l2g = oracle.dof_table(tets2, order)
        ia, ja = oracle.pattern(N, l2g)
        assert V.ndof == N
        val = oracle.assemble(order, xyz2, tets2, l2g, ia, ja, kappa=kappa, mass=0.5)
        assert_values_close(a.values(), val, what="unused vertices, mixed orientation P%d" % order)


def test_empty_dirichlet_and_zero_rhs(env, oracle):
    xyz, tets = meshgen.kuhn_box(4, perturb=0.1)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, 2)
    a = laplace_mass(M, V)
    before = a.values()
    l = fpp.form1(test=V)
    env.check(env.lib.fgpu_dirichlet(env.h, a.h, l.vec.h, 0, None, None, 1, 1.0))
    assert np.array_equal(a.values(), before)
    u = V.element()
    st = a.solve(rhs=l, solution=u, rtol=1e-10)
    assert st["iterations"] == 0 and not np.any(u.to_numpy())


def test_refused_inputs(env):
    lib = env.lib
    xyz = np.zeros((4, 3))
    tets = np.array([[0, 1, 2, 4]], dtype=np.int32)
    h = C.c_void_p()
    p = lambda a: a.ctypes.data_as(C.c_void_p)   # noqa: E731
    assert _ffi.ERROR_NAMES[lib.fgpu_mesh_upload(env.h, 4, p(xyz), 1, p(tets), C.byref(h))] == "FGPU_ERR_OUT_OF_RANGE"
    assert _ffi.ERROR_NAMES[lib.fgpu_mesh_upload(env.h, 4, p(xyz), 0, p(tets), C.byref(h))] == "FGPU_ERR_INVALID"
    neg = np.array([[0, 1, 2, -1]], dtype=np.int32)
    assert _ffi.ERROR_NAMES[lib.fgpu_mesh_upload(env.h, 4, p(xyz), 1, p(neg), C.byref(h))] == "FGPU_ERR_OUT_OF_RANGE"
    hexes = np.array([[0, 1, 2, 3, 0, 1, 2, 9]], dtype=np.int32)
    assert _ffi.ERROR_NAMES[lib.fgpu_mesh_upload_hex(env.h, 4, p(xyz), 1, p(hexes), C.byref(h))] == "FGPU_ERR_OUT_OF_RANGE"
    good = np.array([[0, 1, 2, 3]], dtype=np.int32)
    xyz[1, 0] = xyz[2, 1] = xyz[3, 2] = 1.0
    M = fpp.Mesh(xyz, good, env=env)
    with pytest.raises(fpp.FgpuError):
        fpp.Pch(M, 4)
    with pytest.raises(fpp.FgpuError):
        fpp.FunctionSpace(M, 1, 2)
    # the context is still usable
    V = fpp.Pch(M, 1)
    assert laplace_mass(M, V).nnz == 16
