"""Tensor-core (tcgen05) element phase of the binary32 matrix-free operator (run on a GB300).

3xTF32 (hi*hi + hi*lo + lo*hi) keeps binary32-level accuracy: the tolerance is
4e-6 relative to sum |a_k b_k| per GEMM entry, and 2e-6 of max |y| for the operator."""
import ctypes as C

import numpy as np
import pytest

import feelpp_gb300 as fpp
from tests.test_gpu_matfree import system

pytestmark = pytest.mark.gpu


def test_tc_selftest_gemm(env):
    rng = np.random.default_rng(11)
    A = rng.standard_normal((128, 24)).astype(np.float32)
    B = rng.standard_normal((144, 24)).astype(np.float32)
    D = np.zeros((128, 144), dtype=np.float32)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    env.check(env.lib.fgpu_tc_selftest(env.h, p(A), p(B), p(D)))
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64).T
    assert np.all(np.abs(D - ref) <= 4e-6 * scale), np.abs(D - ref).max()


@pytest.mark.parametrize("order,n", [(2, 6), (3, 4), (3, 7), (2, 24), (3, 20)])
def test_operator_apply_tensor_cores(env, order, n):
    """(the larger meshes give every CTA of the pipelined kernel three or more tiles, so both buffers are
    reused)"""
    xyz, tets, M, V, integral, a, l = system(env, n, order)
    op = fpp.operator(V, integral, precision="f32")
    op.use_tensor_cores(True)
    op.set_dirichlet(V.boundary_dofs())
    x = np.random.default_rng(5).standard_normal(V.ndof)
    xv, yv, zv = V.element(), V.element(), V.element()
    xv.upload(x)
    op.apply(xv, yv)
    a.mult(xv, zv)
    y, z = yv.to_numpy(), zv.to_numpy()
    assert np.abs(y - z).max() <= 2e-6 * np.abs(z).max()


def test_mixed_matfree_solve_tensor_cores(env):
    xyz, tets, M, V, integral, a, l = system(env, 6, 3)
    op64 = fpp.operator(V, integral, precision="f64")
    op32 = fpp.operator(V, integral, precision="f32")
    op32.use_tensor_cores(True)
    bd = V.boundary_dofs()
    op64.set_dirichlet(bd)
    op32.set_dirichlet(bd)
    u = V.element()
    st = op64.solve(l, u, rtol=1e-10, inner=op32)
    assert st["rel_residual"] <= 1e-10
    w = V.element()
    a.solve(rhs=l, solution=w, rtol=1e-11)
    assert np.linalg.norm(u.to_numpy() - w.to_numpy()) <= 1e-8 * np.linalg.norm(w.to_numpy())
