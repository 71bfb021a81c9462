"""Allocation-free load-vector entry point (fgpu_assemble_vector_noalloc).

It serves callers that cannot allocate device memory when they assemble (the
application's pool allocator owns the device memory, or allocation is not
allowed after set-up). Its output must equal the regular fgpu_assemble_vector
result, call after call, even though the shared static scratch keeps the
previous call's contents. This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

import feelpp_gb300 as fpp
from feelpp_gb300 import _ffi, meshgen
from tests.helpers import assert_values_close, mesh

pytestmark = pytest.mark.gpu


def _desc(kind, c=(0.0, 0.0, 0.0), q=0):
    d = _ffi.RhsDesc()
    d.kind = kind
    for k in range(3):
        d.c[k] = c[k]
    d.quad_degree = q
    return d


def _regular(V, src):
    v = V.element()
    l = fpp.form1(test=V)
    l.assign(fpp.integrate(fpp.elements(V.mesh), src * fpp.id(v)))
    return l.to_numpy()


def _noalloc(env, V, desc, out):
    import torch
    dptr = C.c_void_p()
    env.check(env.lib.fgpu_vector_device(out.h, C.byref(dptr)))
    env.sync()                                   # the caller's stream must come after the context's work
    s = torch.cuda.Stream()
    rc = env.lib.fgpu_assemble_vector_noalloc(V.h, C.byref(desc), dptr, 0, C.c_void_p(s.cuda_stream))
    env.check(rc)
    torch.cuda.synchronize()
    return out.to_numpy()


def _device_ptr(env, out):
    dptr = C.c_void_p()
    env.check(env.lib.fgpu_vector_device(out.h, C.byref(dptr)))
    return dptr


@pytest.mark.parametrize("order", [1, 2, 3])
def test_noalloc_matches_regular_twice(env, order):
    xyz, tets = mesh(6, perturb=0.2)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, order)
    ref_sine = _regular(V, fpp.sine_source())
    ref_const = _regular(V, 2.5)
    out = fpp.DeviceVector(env, V.ndof)
    got1 = _noalloc(env, V, _desc(_ffi.RHS_SINE), out)
    assert_values_close(got1, ref_sine, what="no-alloc load vector, first call")
    # second call, other source: the scratch still holds the first call's values
    got2 = _noalloc(env, V, _desc(_ffi.RHS_CONST, (2.5, 0.0, 0.0)), out)
    assert_values_close(got2, ref_const, what="no-alloc load vector, second call")


def test_noalloc_vector_space(env):
    xyz, tets = mesh(4, perturb=0.1, lengths=(4.0, 1.0, 1.0))
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pchv(M, 2)
    ref = _regular(V, fpp.cst_vec(0.0, 0.0, -1.0))
    out = fpp.DeviceVector(env, V.ndof)
    for _ in range(2):
        got = _noalloc(env, V, _desc(_ffi.RHS_CONST_VEC, (0.0, 0.0, -1.0)), out)
        assert_values_close(got, ref, what="no-alloc vector load")


def test_noalloc_rejects_oversized(env):
    xyz, tets = mesh(26)                      # 105 456 tets x 20 local dofs > 2^21
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, 3)
    out = fpp.DeviceVector(env, V.ndof)
    dptr = C.c_void_p()
    env.check(env.lib.fgpu_vector_device(out.h, C.byref(dptr)))
    rc = env.lib.fgpu_assemble_vector_noalloc(V.h, C.byref(_desc(_ffi.RHS_SINE)), dptr, 0, None)
    assert rc == 1
    assert b"FGPU_NOALLOC_MAX_ELEMENT_VALUES" in env.lib.fgpu_last_error(env.h)


def test_noalloc_allocates_no_device_memory(env):
    """The property the entry point exists for: once the first call has set the
    device up, further calls leave the device's free memory unchanged."""
    import torch
    xyz, tets = mesh(8, perturb=0.2)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, 2)
    out = fpp.DeviceVector(env, V.ndof)
    ref = _regular(V, fpp.sine_source())
    _noalloc(env, V, _desc(_ffi.RHS_SINE), out)             # first call: set-up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    got = _noalloc(env, V, _desc(_ffi.RHS_SINE), out)
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, "the call changed free device memory by %d bytes" % (free0 - free1)
    assert_values_close(got, ref, what="no-alloc load vector after set-up")


def test_noalloc_refuses_hexahedra(env):
    xyz, hexes = meshgen.hex_box(3, 3, 3, perturb=0.1)
    M = fpp.Mesh(xyz, hexes, env=env)
    V = fpp.Pch(M, 1)
    out = fpp.DeviceVector(env, V.ndof)
    rc = env.lib.fgpu_assemble_vector_noalloc(V.h, C.byref(_desc(_ffi.RHS_SINE)), _device_ptr(env, out), 0, None)
    assert rc == 1
    assert b"tetrahedral meshes only" in env.lib.fgpu_last_error(env.h)


def test_noalloc_refuses_face_source(env):
    xyz, tets = mesh(3)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, 1)
    out = fpp.DeviceVector(env, V.ndof)
    rc = env.lib.fgpu_assemble_vector_noalloc(V.h, C.byref(_desc(_ffi.RHS_FACE, (1.0, 0.0, 0.0))),
                                              _device_ptr(env, out), 0, None)
    assert rc == 1
    assert b"FGPU_RHS_FACE" in env.lib.fgpu_last_error(env.h)
