"""Streamed assembly (FGPU_ALGO_STREAMED: scalar Laplace/mass forms on affine tetrahedra in one
persistent launch) on a GB300: the same arithmetic and summation order as the two-phase assembly, so the
values must be bit-identical to it, and within the FP64 parity tolerance of the oracle. Long thin
meshes make the ring of element slots wrap many times (element tasks waiting for the gather tasks
that still read the slots they overwrite)."""
import ctypes as C

import numpy as np
import pytest

import feelpp_gb300 as fpp
from feelpp_gb300 import _ffi, meshgen
from tests.helpers import assert_values_close, oracle_system

pytestmark = pytest.mark.gpu


def _assemble(env, M, V, kappa, algo, precision="f64", mass=0.7, accumulate_twice=False):
    u, v = V.element(), V.element()
    a = fpp.form2(test=V, trial=V, precision=precision)
    a.algo = algo
    integral = fpp.integrate(fpp.elements(M), kappa * fpp.inner(fpp.gradt(u), fpp.grad(v)) + mass * fpp.idt(u) * fpp.id(v))
    a.assign(integral)
    if accumulate_twice:
        a += integral
    return a


CASES = [
    # (order, nx, ny, nz): cubes and long bars (the bars wrap the ring of element slots)
    (1, 12, 12, 12), (2, 8, 8, 8), (3, 5, 5, 5),
    (1, 160, 3, 3), (2, 96, 3, 3), (3, 64, 2, 3),
]


@pytest.mark.parametrize("order,nx,ny,nz", CASES)
def test_streamed_equals_two_phase_bits_and_oracle(env, oracle, order, nx, ny, nz):
    xyz, tets = meshgen.kuhn_box(nx, ny, nz, lengths=(nx / 8.0, ny / 8.0, nz / 8.0), perturb=0.15, seed=77)
    kappa = meshgen.lognormal_kappa(len(tets), seed=78)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, order)
    s = _assemble(env, M, V, kappa, _ffi.ALGO_STREAMED)
    t = _assemble(env, M, V, kappa, _ffi.ALGO_TWO_PHASE)
    sv, tv = s.values(), t.values()
    assert np.array_equal(sv, tv), "streamed and two-phase differ in %d entries" % int((sv != tv).sum())
    N, l2g, ia, ja, val = oracle_system(oracle, xyz, tets, order, kappa=kappa, mass=0.7)
    dia, dja, _ = s.csr()
    assert np.array_equal(dia, ia) and np.array_equal(dja, ja)
    assert_values_close(sv, val, what="streamed P%d %dx%dx%d" % (order, nx, ny, nz))
    # repeated launches give the same bits (the control block is reset per launch)
    s.assign(fpp.integrate(fpp.elements(M), kappa * fpp.inner(fpp.gradt(V.element()), fpp.grad(V.element()))
                           + 0.7 * fpp.idt(V.element()) * fpp.id(V.element())))
    assert np.array_equal(s.values(), tv)


@pytest.mark.parametrize("order", [1, 2, 3])
def test_streamed_fp32_and_accumulate_equal_two_phase(env, order):
    xyz, tets = meshgen.kuhn_box(48 if order == 1 else 40, 3, 3, lengths=(6.0, 0.4, 0.4), perturb=0.1, seed=5)
    kappa = meshgen.lognormal_kappa(len(tets), seed=6)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, order)
    for precision in ("f64", "f32"):
        s = _assemble(env, M, V, kappa, _ffi.ALGO_STREAMED, precision=precision, accumulate_twice=True)
        t = _assemble(env, M, V, kappa, _ffi.ALGO_TWO_PHASE, precision=precision, accumulate_twice=True)
        assert np.array_equal(s.values(), t.values()), precision


def test_auto_is_two_phase_and_matches_streamed(env):
    xyz, tets = meshgen.kuhn_box(10, perturb=0.2, seed=3)
    kappa = meshgen.lognormal_kappa(len(tets), seed=4)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, 2)
    a = _assemble(env, M, V, kappa, _ffi.ALGO_AUTO)
    u, v = V.element(), V.element()
    l0 = env.launches()
    a.assign(fpp.integrate(fpp.elements(M), kappa * fpp.inner(fpp.gradt(u), fpp.grad(v)) + 0.7 * fpp.idt(u) * fpp.id(v)))
    assert env.launches() - l0 == 2          # element matrices (geometry inside), gather
    s = _assemble(env, M, V, kappa, _ffi.ALGO_STREAMED)
    assert np.array_equal(a.values(), s.values())


def test_auto_bits_do_not_depend_on_free_memory(env):
    """AUTO chooses from the form and the mesh only: a large foreign allocation changes nothing."""
    import torch
    xyz, tets = meshgen.kuhn_box(12, perturb=0.2, seed=8)
    kappa = meshgen.lognormal_kappa(len(tets), seed=9)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, 2)
    ref = _assemble(env, M, V, kappa, _ffi.ALGO_AUTO).values()
    free, _ = torch.cuda.mem_get_info()
    hog = torch.empty(int(free * 0.9) // 8, dtype=torch.float64, device="cuda")
    try:
        got = _assemble(env, M, V, kappa, _ffi.ALGO_AUTO).values()
    finally:
        del hog
        torch.cuda.empty_cache()
    assert np.array_equal(got, ref)


def test_streamed_host_transfer_equals_device_values(env):
    import torch
    xyz, tets = meshgen.kuhn_box(20, 6, 6, lengths=(2.0, 0.6, 0.6), perturb=0.15, seed=10)
    kappa = meshgen.lognormal_kappa(len(tets), seed=11)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, 2)
    a = _assemble(env, M, V, kappa, _ffi.ALGO_TWO_PHASE)
    ref = a.values()
    h = torch.zeros(a.nnz, dtype=torch.float64).pin_memory()
    d = _ffi.FormDesc()
    d.kind, d.kappa, d.mass, d.quad_degree, d.algo = _ffi.FORM_LAPLACE_MASS, 0.0, 0.7, 0, _ffi.ALGO_STREAMED
    d.kappa_elem = kappa.ctypes.data_as(C.c_void_p)
    for mode in ("auto", "copy"):
        env.set_host_transfer(mode)
        h.zero_()
        env.check(env.lib.fgpu_assemble_matrix_host(env.h, a.h, C.byref(d), C.c_void_p(h.data_ptr())))
        assert np.array_equal(h.numpy(), ref), mode
    env.set_host_transfer("auto")


def test_auto_bits_same_eager_and_captured(env):
    """AUTO never switches algorithm inside a graph capture: replayed values equal eager ones."""
    xyz, tets = meshgen.kuhn_box(9, perturb=0.2, seed=12)
    kappa = meshgen.lognormal_kappa(len(tets), seed=13)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, 3)
    u, v = V.element(), V.element()
    a = fpp.form2(test=V, trial=V)
    kt = fpp.DeviceScalar(env, 1.0)
    integral = fpp.integrate(fpp.elements(M), kt * fpp.inner(fpp.gradt(u), fpp.grad(v)) + 0.7 * fpp.idt(u) * fpp.id(v))
    a.assign(integral)
    eager = a.values()
    with fpp.capture(env) as g:
        a.assign(integral)
    a.zero()
    g.launch()
    assert np.array_equal(a.values(), eager)
