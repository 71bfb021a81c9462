"""Device assembly parity against the oracle (run on a GB300).

Tolerances: the plain FP64 path must match per entry within
|a - b| <= 1e-12 |b| + 1e-14 max|A| (helpers.RTOL_F64 / ATOL_F64); the FP32 path
is reported against the FP64 oracle and must stay within 2e-5 relative to the
largest entry of its row block."""
import numpy as np
import pytest

import feelpp_gb300 as fpp
from feelpp_gb300 import meshgen
from tests.helpers import assert_values_close, mesh, oracle_system

pytestmark = pytest.mark.gpu


def device_matrix(env, xyz, tets, order, kappa=1.0, mass=1.0, ncomp=1, elasticity=None, precision="f64"):
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.FunctionSpace(M, order, ncomp)
    u, v = V.element(), V.element()
    a = fpp.form2(test=V, trial=V, precision=precision)
    if elasticity is not None:
        a.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.stress(u, *elasticity), fpp.grad(v))))
    else:
        expr = kappa * fpp.inner(fpp.gradt(u), fpp.grad(v))
        if mass:
            expr = expr + mass * (fpp.idt(u) * fpp.id(v))
        a.assign(fpp.integrate(fpp.elements(M), expr))
    return M, V, a


def test_p1_unit_cube_16_plain_fp64(env, oracle):
    """P1 Laplacian stiffness + mass on the 16^3 Kuhn cube (24 576 tets), perturbed 0.2h."""
    xyz, tets = mesh(16, perturb=0.2)
    M, V, a = device_matrix(env, xyz, tets, 1)
    assert V.ndof == 4913 and a.nnz == 66961
    N, l2g, ia, ja, val = oracle_system(oracle, xyz, tets, 1, mass=1.0)
    assert np.array_equal(V.dof_l2g(), l2g)
    dia, dja, dval = a.csr()
    assert np.array_equal(dia, ia) and np.array_equal(dja, ja)
    assert_values_close(dval, val)


@pytest.mark.parametrize("order,n", [(1, 6), (2, 6), (3, 4)])
def test_lognormal_kappa_parity(env, oracle, order, n):
    xyz, tets = mesh(n, perturb=0.15)
    kappa = meshgen.lognormal_kappa(len(tets))
    M, V, a = device_matrix(env, xyz, tets, order, kappa=kappa, mass=1.0)
    N, l2g, ia, ja, val = oracle_system(oracle, xyz, tets, order, kappa=kappa, mass=1.0)
    dia, dja, dval = a.csr()
    assert np.array_equal(dia, ia) and np.array_equal(dja, ja)
    assert_values_close(dval, val)


@pytest.mark.parametrize("order,n", [(2, 6), (3, 4)])
def test_fp32_assembly_error_vs_fp64_oracle(env, oracle, order, n):
    xyz, tets = mesh(n, perturb=0.15)
    kappa = meshgen.lognormal_kappa(len(tets))
    M, V, a = device_matrix(env, xyz, tets, order, kappa=kappa, mass=1.0, precision="f32")
    N, l2g, ia, ja, val = oracle_system(oracle, xyz, tets, order, kappa=kappa, mass=1.0)
    dval = a.values()
    scale = np.abs(val).max()
    err = np.abs(dval - val) / scale
    assert err.max() < 2e-5, err.max()


def test_elasticity_p2_parity(env, oracle):
    xyz, tets = mesh(3, perturb=0.1, lengths=(4.0, 1.0, 1.0))
    M, V, a = device_matrix(env, xyz, tets, 2, ncomp=3, elasticity=(1.0, 0.5))
    N, l2g, ia, ja, val = oracle_system(oracle, xyz, tets, 2, ncomp=3, kind=1, lam=1.0, mu=0.5)
    assert np.array_equal(V.dof_l2g(), l2g)
    dia, dja, dval = a.csr()
    assert np.array_equal(dia, ia) and np.array_equal(dja, ja)
    assert_values_close(dval, val)


def test_elasticity_p1_parity(env, oracle):
    xyz, tets = mesh(4, perturb=0.2)
    M, V, a = device_matrix(env, xyz, tets, 1, ncomp=3, elasticity=(2.0, 0.3))
    N, l2g, ia, ja, val = oracle_system(oracle, xyz, tets, 1, ncomp=3, kind=1, lam=2.0, mu=0.3)
    dia, dja, dval = a.csr()
    assert np.array_equal(dja, ja)
    assert_values_close(dval, val)


def test_accumulate_and_reassign(env, oracle):
    xyz, tets = mesh(4, perturb=0.2)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, 2)
    u, v = V.element(), V.element()
    a = fpp.form2(test=V, trial=V)
    a += fpp.integrate(fpp.elements(M), fpp.inner(fpp.gradt(u), fpp.grad(v)))
    a += fpp.integrate(fpp.elements(M), fpp.idt(u) * fpp.id(v))
    N, l2g, ia, ja, val = oracle_system(oracle, xyz, tets, 2, mass=1.0)
    assert_values_close(a.values(), val)
    a.assign(fpp.integrate(fpp.elements(M), 2.0 * fpp.inner(fpp.gradt(u), fpp.grad(v))))
    N, l2g, ia, ja, val2 = oracle_system(oracle, xyz, tets, 2, kappa=np.full(len(tets), 2.0), mass=0.0)
    assert_values_close(a.values(), val2)


@pytest.mark.parametrize("order", [1, 2, 3])
def test_load_vector_parity(env, oracle, order):
    xyz, tets = mesh(4, perturb=0.2)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, order)
    v = V.element()
    l = fpp.form1(test=V)
    l.assign(fpp.integrate(fpp.elements(M), fpp.sine_source() * fpp.id(v)))
    N, l2g = oracle.dof_table(tets, order)
    F = oracle.rhs(order, xyz, tets, l2g, N, fkind=0)
    assert_values_close(l.to_numpy(), F, what="load vector")


def test_vector_load_parity(env, oracle):
    xyz, tets = mesh(3, perturb=0.1, lengths=(4.0, 1.0, 1.0))
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pchv(M, 2)
    v = V.element()
    l = fpp.form1(test=V)
    l.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.cst_vec(0, 0, -1), fpp.id(v))))
    N, l2g = oracle.dof_table(tets, 2, 3)
    F = oracle.rhs(2, xyz, tets, l2g, N, fkind=1, fc=(0.0, 0.0, -1.0), ncomp=3)
    assert_values_close(l.to_numpy(), F, what="vector load")


@pytest.mark.parametrize("mode_name,mode", [("elimination", 0), ("elimination_symmetric", 1),
                                            ("elimination_keep_diagonal", 2)])
def test_dirichlet_modes(env, oracle, mode_name, mode):
    xyz, tets = mesh(4, perturb=0.2)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, 2)
    u, v = V.element(), V.element()
    a = fpp.form2(test=V, trial=V)
    a.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.gradt(u), fpp.grad(v))))
    l = fpp.form1(test=V)
    l.assign(fpp.integrate(fpp.elements(M), fpp.sine_source() * fpp.id(v)))
    a += fpp.on(fpp.boundaryfaces(M), rhs=l, element=u, expr=0.25, type=mode_name)
    N, l2g, ia, ja, val = oracle_system(oracle, xyz, tets, 2, mass=0.0)
    b = oracle.rhs(2, xyz, tets, l2g, N, fkind=0)
    mask = oracle.boundary_mask(2, xyz, tets, l2g, N)
    assert np.array_equal(np.sort(V.boundary_dofs()), np.nonzero(mask)[0])
    oracle.dirichlet(ia, ja, val, b, mask, g=np.full(N, 0.25), mode=mode)
    assert_values_close(a.values(), val, what="matrix after on()")
    assert_values_close(l.to_numpy(), b, what="rhs after on()")


@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("order,n,frac,precision", [(2, 8, 0.2, "f64"), (1, 20, 0.05, "f64"), (3, 5, 0.5, "f64"),
                                                    (2, 8, 0.2, "f32")])
def test_dirichlet_scattered_rows(env, oracle, mode, order, n, frac, precision):
    """on() over a seeded random subset of the dofs (rows eliminated anywhere in the numbering, groups of
    32 rows with none, some or all of them eliminated, rows longer than 32 entries), random values g, a
    random right-hand side and diag = 2.5, on FP64 and FP32 matrices."""
    xyz, tets = mesh(n, perturb=0.2)
    M, V, a = device_matrix(env, xyz, tets, order, kappa=1.0, mass=0.5, precision=precision)
    ia, ja, val = a.csr()
    N = len(ia) - 1
    rng = np.random.default_rng(100 + mode + 10 * order)
    dofs = np.sort(rng.choice(N, size=max(1, int(frac * N)), replace=False)).astype(np.int32)
    dofs[: min(64, len(dofs))] = np.arange(min(64, len(dofs)), dtype=np.int32)   # the first two groups eliminated
    dofs = np.unique(dofs)
    g = rng.standard_normal(len(dofs))
    b0 = rng.standard_normal(N)
    rhs = V.element()
    rhs.upload(b0)
    bc = fpp.DirichletBC(V, dofs, g)
    a.apply_bc(bc, rhs=rhs, type={0: "elimination", 1: "elimination_symmetric", 2: "elimination_keep_diagonal"}[mode],
               diag=2.5)
    mask = np.zeros(N, np.uint8)
    mask[dofs] = 1
    gg = np.zeros(N)
    gg[dofs] = g
    b = b0.copy()
    oracle.dirichlet(ia, ja, val, b, mask, g=gg, mode=mode, diag=2.5)
    got = a.values()
    if precision == "f32":
        val = val.astype(np.float32).astype(np.float64)
    assert np.array_equal(got == 0.0, val == 0.0)
    assert_values_close(got, val, what="matrix after on()")
    assert_values_close(rhs.to_numpy(), b, what="rhs after on()")


def test_bad_element_reported(env):
    xyz = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0], [0, 0, 1]], dtype=float)
    tets = np.array([[0, 1, 2, 3], [0, 1, 2, 4]], dtype=np.int32)   # first tet is flat (det K = 0)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, 1)
    u, v = V.element(), V.element()
    a = fpp.form2(test=V, trial=V)
    with pytest.raises(fpp.FgpuError) as ei:
        a.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.gradt(u), fpp.grad(v))))
    assert ei.value.code == 3
    # the context stays usable
    xyz2, tets2 = mesh(2)
    M2, V2, a2 = device_matrix(env, xyz2, tets2, 1)
    assert a2.nnz > 0


def test_p2_large_properties(env):
    """P2 on 40^3 (384 000 tets, nnz 15.0 M): size-independent checks on the full matrix."""
    import scipy.sparse as sp
    n = 40
    xyz, tets = mesh(n, perturb=0.15)
    M, V, a = device_matrix(env, xyz, tets, 2, kappa=1.0, mass=0.0)
    assert V.ndof == (2 * n + 1) ** 3 and a.nnz == 230 * n ** 3 + 138 * n ** 2 + 24 * n + 1
    ia, ja, val = a.csr()
    A = sp.csr_matrix((val, ja, ia), shape=(V.ndof, V.ndof))
    scale = np.abs(val).max()
    assert np.abs(A @ np.ones(V.ndof)).max() < 1e-11 * scale            # constants in the kernel
    assert abs(A - A.T).max() < 1e-14 * scale                           # symmetric
    Mm, Vm, m = device_matrix(env, xyz, tets, 2, kappa=0.0, mass=1.0)
    assert abs(m.values().sum() - 1.0) < 1e-11                          # 1^T M 1 = |Omega|


def test_deterministic_repeat(env):
    xyz, tets = mesh(8, perturb=0.2)
    kappa = meshgen.lognormal_kappa(len(tets))
    M, V, a = device_matrix(env, xyz, tets, 3, kappa=kappa)
    v1 = a.values()
    u, v = V.element(), V.element()
    a.assign(fpp.integrate(fpp.elements(M), kappa * fpp.inner(fpp.gradt(u), fpp.grad(v)) + fpp.idt(u) * fpp.id(v)))
    assert np.array_equal(v1, a.values())


@pytest.mark.parametrize("order,n", [(1, 6), (2, 4), (3, 3)])
@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_two_phase_equals_fused_gather(env, order, n, precision):
    """Element matrices buffered (upper triangles) then summed per CSR entry in element order
    agree with the fused row-owner gather (which sums per slot) to rounding, for '=' and '+=';
    AUTO is the two-phase path here."""
    from feelpp_gb300 import _ffi
    xyz, tets = mesh(n, perturb=0.2)
    kappa = meshgen.lognormal_kappa(len(tets))
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, order)
    u, v = V.element(), V.element()
    integral = fpp.integrate(fpp.elements(M), kappa * fpp.inner(fpp.gradt(u), fpp.grad(v)) + 0.7 * (fpp.idt(u) * fpp.id(v)))
    got = []
    for algo in (_ffi.ALGO_GATHER, _ffi.ALGO_TWO_PHASE, _ffi.ALGO_AUTO):
        a = fpp.form2(test=V, trial=V, precision=precision)
        a.algo = algo
        a.assign(integral)
        a += integral
        got.append(a.values())
    assert np.array_equal(got[1], got[2])
    tol = 1e-6 if precision == "f32" else 1e-14
    assert_values_close(got[1], got[0], rtol=tol, atol=tol, what="two-phase vs fused")


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_elasticity_two_phase_vs_native(env, order, precision):
    """Vector elasticity: df64 / binary32 two-phase blocks against the row-owner gather
    (native FP64 / binary32 arithmetic), same pattern, values to rounding."""
    from feelpp_gb300 import _ffi
    xyz, tets = mesh(3, perturb=0.2, lengths=(2.0, 1.0, 1.0))
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pchv(M, order)
    u, v = V.element(), V.element()
    integral = fpp.integrate(fpp.elements(M), fpp.inner(fpp.stress(u, 1.3, 0.6), fpp.grad(v)))
    got = []
    for algo in (_ffi.ALGO_GATHER, _ffi.ALGO_TWO_PHASE):
        a = fpp.form2(test=V, trial=V, precision=precision)
        a.algo = algo
        a.assign(integral)
        a += integral
        got.append(a.values())
    tol = 2e-6 if precision == "f32" else 1e-13
    assert_values_close(got[1], got[0], rtol=tol, atol=tol, what="elasticity two-phase vs gather")


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_assemble_matrix_host(env, precision):
    """fgpu_assemble_matrix_host (pipelined gather + copies for FP64, assemble-then-copy otherwise) gives the
    values of fgpu_assemble_matrix followed by a copy."""
    import ctypes as C
    from feelpp_gb300 import _ffi, fe
    xyz, tets = mesh(8, perturb=0.2)
    kappa = meshgen.lognormal_kappa(len(tets))
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, 2)
    u, v = V.element(), V.element()
    integral = fpp.integrate(fpp.elements(M), kappa * fpp.inner(fpp.gradt(u), fpp.grad(v)) + fpp.idt(u) * fpp.id(v))
    a = fpp.form2(test=V, trial=V, precision=precision)
    a.assign(integral)
    ref = a.values().astype(np.float64)
    d, karr = fe.Form2._desc_of(integral, _ffi.ALGO_AUTO)
    d.kappa_elem = karr.ctypes.data_as(C.c_void_p)
    out = np.zeros(a.nnz)
    a.zero()
    env.check(env.lib.fgpu_assemble_matrix_host(env.h, a.h, C.byref(d), out.ctypes.data_as(C.c_void_p)))
    assert np.array_equal(out, ref)
    assert np.array_equal(a.values().astype(np.float64), ref)


@pytest.mark.parametrize("mode", ["auto", "direct", "copy"])
def test_assemble_matrix_host_transfer_modes(env, mode):
    """Host-output assembly into a page-locked buffer: direct stores from the gather kernel and copy-engine
    ranges give the device values bit for bit; direct stores refuse a pageable buffer."""
    import ctypes as C
    import torch
    from feelpp_gb300 import _ffi, fe
    xyz, tets = mesh(10, perturb=0.2)
    kappa = meshgen.lognormal_kappa(len(tets))
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, 2)
    u, v = V.element(), V.element()
    integral = fpp.integrate(fpp.elements(M), kappa * fpp.inner(fpp.gradt(u), fpp.grad(v)) + fpp.idt(u) * fpp.id(v))
    a = fpp.form2(test=V, trial=V)
    a.assign(integral)
    ref = a.values()
    d, karr = fe.Form2._desc_of(integral, _ffi.ALGO_AUTO)
    d.kappa_elem = karr.ctypes.data_as(C.c_void_p)
    pinned = torch.zeros(a.nnz, dtype=torch.float64).pin_memory()
    env.set_host_transfer(mode)
    try:
        a.zero()
        env.check(env.lib.fgpu_assemble_matrix_host(env.h, a.h, C.byref(d), C.c_void_p(pinned.data_ptr())))
        assert np.array_equal(pinned.numpy(), ref)
        assert np.array_equal(a.values(), ref)
        pageable = np.zeros(a.nnz)
        rc = env.lib.fgpu_assemble_matrix_host(env.h, a.h, C.byref(d), pageable.ctypes.data_as(C.c_void_p))
        if mode == "direct":
            assert _ffi.ERROR_NAMES.get(rc) == "FGPU_ERR_INVALID"
        else:
            assert rc == 0 and np.array_equal(pageable, ref)
    finally:
        env.set_host_transfer("auto")
