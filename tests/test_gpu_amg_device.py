"""Smoothed-aggregation AMG set-up on the device (the default of fgpu_amg_create), run on a GB300:
the device-built hierarchy equals the host set-up's bit for bit (every level operator, prolongator,
aggregate map and lambda_max estimate, and the dense coarsest inverse), for scalar P1-P3 Laplacians
with a lognormal coefficient, vector P1 elasticity, unsmoothed aggregation and a non-zero strength
threshold; and CG + AMG gives the same iterations and the same solution bits with either set-up."""
import ctypes as C

import numpy as np
import pytest

import feelpp_gb300 as fpp
from feelpp_gb300 import _ffi, meshgen
from tests.helpers import mesh

pytestmark = pytest.mark.gpu


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _levels(lib, h):
    """every level of a fgpu_amg_host object: (A (ia, ja, a), P (ia, ja, a) or None, agg, lmax)"""
    out = []
    nl = lib.fgpu_amg_host_levels(h)
    for l in range(nl):
        n, nnz, pnnz, pcols = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        lmax = C.c_double()
        assert lib.fgpu_amg_host_level(h, l, C.byref(n), C.byref(nnz), C.byref(pnnz), C.byref(pcols), C.byref(lmax)) == 0
        n, nnz, pnnz = n.value, nnz.value, pnnz.value
        ia, ja, a = np.zeros(n + 1, np.int64), np.zeros(max(nnz, 1), np.int32), np.zeros(max(nnz, 1))
        last = l == nl - 1
        pia, pja, pa = np.zeros(n + 1, np.int64), np.zeros(max(pnnz, 1), np.int32), np.zeros(max(pnnz, 1))
        agg = np.zeros(max(n, 1), np.int32)
        assert lib.fgpu_amg_host_export(h, l, _p(ia), _p(ja), _p(a), None if last else _p(pia), None if last else _p(pja),
                                        None if last else _p(pa), None if last else _p(agg)) == 0
        P = None if last else (pia, pja[:pnnz], pa[:pnnz], pcols.value)
        out.append(((ia, ja[:nnz], a[:nnz]), P, None if last else agg[:n], lmax.value))
    inv_n = out[-1][0][0].size - 1
    inv = np.zeros(max(inv_n * inv_n, 1))
    has_inv = lib.fgpu_amg_host_coarse_inverse(h, _p(inv))
    return out, (inv if has_inv == 1 else None)


def _host_and_device(env, form, **cfg):
    lib = env.lib
    c = _ffi.AmgCfg(cfg.get("threshold", 0.0), cfg.get("max_levels", 0), cfg.get("coarse_eq_lim", 0), cfg.get("agg_smooths", 0),
                    0, 0)
    ia, ja, a = form.csr()
    ia, ja, a = np.ascontiguousarray(ia, np.int64), np.ascontiguousarray(ja, np.int32), np.ascontiguousarray(a, np.float64)
    hh, hd = C.c_void_p(), C.c_void_p()
    assert lib.fgpu_amg_host_build(len(ia) - 1, _p(ia), _p(ja), _p(a), C.byref(c), 4, C.byref(hh)) == 0
    env.check(lib.fgpu_amg_device_build(env.h, form.h, C.byref(c), C.byref(hd)))
    try:
        host = _levels(lib, hh)
        dev = _levels(lib, hd)
        ndev = lib.fgpu_amg_host_device_levels(hd)
    finally:
        lib.fgpu_amg_host_destroy(hh)
        lib.fgpu_amg_host_destroy(hd)
    return host, dev, ndev


def _assert_same(host, dev):
    (hl, hinv), (dl, dinv) = host, dev
    assert len(hl) == len(dl)
    for l, (h, d) in enumerate(zip(hl, dl)):
        for x, y in zip(h[0], d[0]):
            assert np.array_equal(x, y), "level %d operator" % l
        assert (h[1] is None) == (d[1] is None)
        if h[1] is not None:
            for x, y in zip(h[1][:3], d[1][:3]):
                assert np.array_equal(x, y), "level %d prolongator" % l
            assert h[1][3] == d[1][3]
            assert np.array_equal(h[2], d[2]), "level %d aggregates" % l
        assert h[3] == d[3], "level %d lambda_max" % l
    assert (hinv is None) == (dinv is None)
    if hinv is not None:
        assert np.array_equal(hinv, dinv)


def poisson(env, n, order, kappa=True, perturb=0.15):
    xyz, tets = mesh(n, perturb=perturb)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, order)
    u, v = V.element(), V.element()
    k = meshgen.lognormal_kappa(len(tets), seed=5) if kappa else 1.0
    a = fpp.form2(test=V, trial=V)
    a.assign(fpp.integrate(fpp.elements(M), k * fpp.inner(fpp.gradt(u), fpp.grad(v))))
    l = fpp.form1(test=V)
    l.assign(fpp.integrate(fpp.elements(M), fpp.sine_source() * fpp.id(v)))
    a += fpp.on(fpp.boundaryfaces(M), rhs=l, element=u, expr=0.0, type="elimination_symmetric")
    return V, a, l


@pytest.mark.parametrize("order,n", [(1, 28), (2, 16), (3, 11)])
def test_device_hierarchy_equals_host(env, order, n):
    V, a, l = poisson(env, n, order)
    host, dev, ndev = _host_and_device(env, a)
    assert ndev >= 1                                   # the fine level (> 16384 rows) was built on the device
    _assert_same(host, dev)


@pytest.mark.parametrize("cfg", [dict(agg_smooths=-1), dict(threshold=0.05), dict(coarse_eq_lim=200, max_levels=3)])
def test_device_hierarchy_options(env, cfg):
    V, a, l = poisson(env, 16, 2)
    host, dev, ndev = _host_and_device(env, a, **cfg)
    assert ndev >= 1
    _assert_same(host, dev)


def test_device_hierarchy_elasticity(env):
    xyz, tets = meshgen.kuhn_box(20, lengths=(4.0, 1.0, 1.0), perturb=0.1, seed=3)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pchv(M, 1)
    u, v = V.element(), V.element()
    a = fpp.form2(test=V, trial=V)
    a.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.stress(u, 1.0, 0.5), fpp.grad(v))))
    l = fpp.form1(test=V)
    l.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.cst_vec(0, 0, -1), fpp.id(v))))
    a += fpp.on(fpp.markedfaces(M, 0.0), rhs=l, element=u, expr=0.0, type="elimination_symmetric")
    host, dev, ndev = _host_and_device(env, a)
    assert ndev >= 1
    _assert_same(host, dev)


def test_device_setup_gives_the_host_solve(env):
    V, a, l = poisson(env, 20, 2)
    wd, wh = V.element(), V.element()
    sd = a.solve(rhs=l, solution=wd, rtol=1e-10, pc="gamg")
    sh = a.solve(rhs=l, solution=wh, rtol=1e-10, pc="gamg", gamg=dict(setup_on_host=True))
    assert sd["rel_residual"] <= 1e-10
    assert sd["iterations"] == sh["iterations"]
    assert np.array_equal(wd.to_numpy(), wh.to_numpy())
    assert sd["gamg"]["levels"] == sh["gamg"]["levels"] and sd["gamg"]["nnz"] == sh["gamg"]["nnz"]


def _beam(env, n, order, clamp=True):
    xyz, tets = meshgen.kuhn_box(n, lengths=(4.0, 1.0, 1.0), perturb=0.1, seed=3)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pchv(M, order)
    u, v = V.element(), V.element()
    a = fpp.form2(test=V, trial=V)
    a.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.stress(u, 1.0, 0.5), fpp.grad(v))))
    l = fpp.form1(test=V)
    l.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.cst_vec(0, 0, -1), fpp.id(v))))
    if clamp:
        a += fpp.on(fpp.markedfaces(M, 0.0), rhs=l, element=u, expr=0.0, type="elimination_symmetric")
    return V, a, l


@pytest.mark.parametrize("order", [1, 2])
def test_rigid_body_modes_are_null_vectors(env, order):
    """the six modes at the dof nodes lie in the kernel of the unconstrained elasticity operator"""
    V, a, l = _beam(env, 3, order, clamp=False)
    ia, ja, val = a.csr()
    import scipy.sparse as sp
    A = sp.csr_matrix((val, ja, ia), shape=(len(ia) - 1,) * 2)
    for m in V.rigid_body_modes():
        x = m.to_numpy()
        assert np.abs(A @ x).max() <= 1e-11 * abs(A).max() * np.abs(x).max()


@pytest.mark.parametrize("order,n", [(1, 20), (2, 10)])
def test_device_hierarchy_equals_host_rigid_body(env, order, n):
    V, a, l = _beam(env, n, order)
    modes = V.rigid_body_modes()
    lib = env.lib
    arr = (C.c_void_p * 6)(*[m.h.value for m in modes])
    B = np.stack([m.to_numpy() for m in modes])
    c = _ffi.AmgCfg(0.0, 0, 0, 0, 0, 0)
    c.block_size, c.nns_count, c.nns = 3, 6, C.cast(arr, C.c_void_p)
    Bc = np.ascontiguousarray(B)
    c.nns_host = Bc.ctypes.data
    ia, ja, val = a.csr()
    ia, ja, val = np.ascontiguousarray(ia, np.int64), np.ascontiguousarray(ja, np.int32), np.ascontiguousarray(val)
    hh, hd = C.c_void_p(), C.c_void_p()
    assert lib.fgpu_amg_host_build(len(ia) - 1, _p(ia), _p(ja), _p(val), C.byref(c), 4, C.byref(hh)) == 0
    env.check(lib.fgpu_amg_device_build(env.h, a.h, C.byref(c), C.byref(hd)))
    try:
        host, dev, ndev = _levels(lib, hh), _levels(lib, hd), lib.fgpu_amg_host_device_levels(hd)
    finally:
        lib.fgpu_amg_host_destroy(hh)
        lib.fgpu_amg_host_destroy(hd)
    assert ndev >= 1
    _assert_same(host, dev)
    agg = dev[0][0][2]
    assert np.array_equal(agg[0::3], agg[1::3]) and np.array_equal(agg[0::3], agg[2::3])


def test_rigid_body_amg_solves_elasticity(env):
    """CG + AMG on the clamped P2 beam (to 1e-8: binary64 CG stalls near 1e-9 on this beam, the
    double-double refinement goes further): the rigid body near null space cuts the iterations several
    times against the constant one, to the same solution"""
    V, a, l = _beam(env, 12, 2)
    w0, w1 = V.element(), V.element()
    s0 = a.solve(rhs=l, solution=w0, rtol=1e-8, pc="gamg")
    s1 = a.solve(rhs=l, solution=w1, rtol=1e-8, pc="gamg", gamg=dict(near_null_space="rigid"))
    assert s0["rel_residual"] <= 1e-8 and s1["rel_residual"] <= 1e-8
    assert s1["iterations"] * 3 <= s0["iterations"]
    x0, x1 = w0.to_numpy(), w1.to_numpy()
    assert np.linalg.norm(x1 - x0) <= 1e-5 * np.linalg.norm(x0)
    sh = a.solve(rhs=l, solution=V.element(), rtol=1e-8, pc="gamg", gamg=dict(near_null_space="rigid", setup_on_host=True))
    assert sh["iterations"] == s1["iterations"]
    # the double-double refinement with the rigid-body AMG inner solve reaches 1e-12
    wd = V.element()
    sd = a.solve_refined(rhs=l, solution=wd, rtol=1e-12, pc="gamg", gamg=dict(near_null_space="rigid"))
    assert sd["rel_residual"] <= 1e-12
