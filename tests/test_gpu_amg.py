"""CG preconditioned by the smoothed-aggregation AMG V-cycle (pc-type=gamg) on a GB300:
convergence to the FP64 residual tolerance, the same solution as CG + Jacobi, far fewer
iterations, determinism, rebuild after reassembly."""
import numpy as np
import pytest

import feelpp_gb300 as fpp
from feelpp_gb300 import meshgen
from tests.helpers import mesh

pytestmark = pytest.mark.gpu


def poisson(env, n, order, kappa=None, perturb=0.15):
    xyz, tets = mesh(n, perturb=perturb)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, order)
    u, v = V.element(), V.element()
    k = 1.0 if kappa is None else kappa
    a = fpp.form2(test=V, trial=V)
    a.assign(fpp.integrate(fpp.elements(M), k * fpp.inner(fpp.gradt(u), fpp.grad(v))))
    l = fpp.form1(test=V)
    l.assign(fpp.integrate(fpp.elements(M), fpp.sine_source() * fpp.id(v)))
    a += fpp.on(fpp.boundaryfaces(M), rhs=l, element=u, expr=0.0, type="elimination_symmetric")
    return M, V, u, v, a, l


@pytest.mark.parametrize("order,n", [(1, 16), (2, 10), (3, 6)])
def test_gamg_matches_jacobi(env, order, n):
    M, V, u, v, a, l = poisson(env, n, order)
    w = V.element()
    st = a.solve(rhs=l, solution=w, rtol=1e-10, pc="gamg")
    assert st["rel_residual"] <= 1e-10
    info = st["gamg"]
    assert info["levels"] >= 2 and all(info["rows"][k + 1] < info["rows"][k] for k in range(info["levels"] - 1))
    wj = V.element()
    stj = a.solve(rhs=l, solution=wj, rtol=1e-12)
    assert st["iterations"] <= 0.35 * stj["iterations"]
    x, xj = w.to_numpy(), wj.to_numpy()
    assert np.linalg.norm(x - xj) <= 1e-8 * np.linalg.norm(xj)
    # the V-cycle is a fixed sequence of deterministic kernels: a second solve gives the same bits
    w2 = V.element()
    a.solve(rhs=l, solution=w2, rtol=1e-10, pc="gamg")
    assert np.array_equal(w2.to_numpy(), x)


def test_gamg_lognormal_kappa_and_rebuild(env):
    xyz, tets = mesh(10, perturb=0.15)
    kappa = meshgen.lognormal_kappa(len(tets))
    M, V, u, v, a, l = poisson(env, 10, 2, kappa=kappa)
    w = V.element()
    st = a.solve(rhs=l, solution=w, rtol=1e-10, pc="gamg")
    assert st["rel_residual"] <= 1e-10
    setup0 = a.gamg().info()["setup_ms"]
    assert setup0 > 0
    # reassemble with another coefficient: the hierarchy is rebuilt before the next solve
    a.assign(fpp.integrate(fpp.elements(M), (2.0 * kappa) * fpp.inner(fpp.gradt(u), fpp.grad(v))))
    a += fpp.on(fpp.boundaryfaces(M), rhs=l, element=u, expr=0.0, type="elimination_symmetric")
    w2 = V.element()
    st2 = a.solve(rhs=l, solution=w2, rtol=1e-10, pc="gamg")
    assert st2["rel_residual"] <= 1e-10
    assert np.linalg.norm(w2.to_numpy() - 0.5 * w.to_numpy()) <= 1e-8 * np.linalg.norm(w.to_numpy())


def test_gamg_df64_and_options(env):
    M, V, u, v, a, l = poisson(env, 10, 2)
    w = V.element()
    st = a.solve(rhs=l, solution=w, rtol=1e-10, pc="gamg", arith="df64")
    assert st["rel_residual"] <= 1e-10
    w2 = V.element()
    st2 = a.solve(rhs=l, solution=w2, rtol=1e-10, pc="gamg",
                  gamg=dict(agg_smooths=-1, smoother_degree=4, coarse_eq_lim=200))
    assert st2["rel_residual"] <= 1e-10
    assert np.linalg.norm(w2.to_numpy() - w.to_numpy()) <= 1e-7 * np.linalg.norm(w.to_numpy())


def test_gamg_rejected_without_hierarchy(env):
    M, V, u, v, a, l = poisson(env, 4, 1)
    import ctypes as C
    from feelpp_gb300 import _ffi, fe
    cfg = fe._solver_cfg(1e-10, 100, "gamg", False, 0.1, 16, "f64", 0, 0.0)
    st = _ffi.SolveStats()
    w = V.element()
    rc = env.lib.fgpu_solve_cg(env.h, a.h, None, l.vec.h, w.h, C.byref(cfg), C.byref(st))
    assert _ffi.ERROR_NAMES[rc] == "FGPU_ERR_INVALID"


def test_gamg_one_level_dense(env):
    """Below coarse-eq-lim rows the hierarchy is one dense level: the V-cycle is the (binary32) inverse,
    and CG converges in a handful of iterations."""
    M, V, u, v, a, l = poisson(env, 6, 1)
    w = V.element()
    st = a.solve(rhs=l, solution=w, rtol=1e-10, pc="gamg")
    assert st["gamg"]["levels"] == 1 and st["rel_residual"] <= 1e-10 and st["iterations"] <= 6


def test_gamg_hierarchy_kept_across_reassembly(env):
    """reuse=True keeps the hierarchy of the first assembly as the preconditioner of later ones (time
    stepping): CG still converges to the current matrix's solution"""
    xyz, tets = mesh(10, perturb=0.15)
    kappa = meshgen.lognormal_kappa(len(tets))
    M, V, u, v, a, l = poisson(env, 10, 2, kappa=kappa)
    w = V.element()
    a.solve(rhs=l, solution=w, rtol=1e-10, pc="gamg")
    amg0 = a.gamg()
    a.assign(fpp.integrate(fpp.elements(M), (1.5 * kappa) * fpp.inner(fpp.gradt(u), fpp.grad(v))))
    a += fpp.on(fpp.boundaryfaces(M), rhs=l, element=u, expr=0.0, type="elimination_symmetric")
    w2 = V.element()
    st = a.solve(rhs=l, solution=w2, rtol=1e-10, pc="gamg", gamg={"reuse": True})
    assert a.gamg(reuse=True) is amg0
    assert st["rel_residual"] <= 1e-10
    assert np.linalg.norm(w2.to_numpy() - w.to_numpy() / 1.5) <= 1e-8 * np.linalg.norm(w.to_numpy())
