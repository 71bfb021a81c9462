"""Iterative refinement with a double-double residual (fgpu_solve_cg_refine_dd) on a GB300: the
clamped vector P2 elasticity beam of [0,4]x[0,1]^2 (body force (0,0,-1), lambda 1, mu 0.5) solved
below the binary64 floor of its residual; the residual of the double-double solution is checked in
extended precision on the host (numpy longdouble: 80-bit on x86, IEEE quad on Arm), and the
displacement against the oracle's FP64 PCG."""
import numpy as np
import pytest

import feelpp_gb300 as fpp
from feelpp_gb300 import meshgen

pytestmark = pytest.mark.gpu


def _beam(env, n):
    xyz, tets = meshgen.kuhn_box(n, lengths=(4.0, 1.0, 1.0), perturb=0.1, seed=1234)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pchv(M, 2)
    u, v = V.element(), V.element()
    a = fpp.form2(test=V, trial=V)
    a.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.stress(u, 1.0, 0.5), fpp.grad(v))))
    l = fpp.form1(test=V)
    l.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.cst_vec(0, 0, -1), fpp.id(v))))
    a += fpp.on(fpp.markedfaces(M, 0.0), rhs=l, element=u, expr=0.0, type="elimination_symmetric")
    return V, a, l


def _residual_ext(ia, ja, val, b, xh, xl):
    ld = np.longdouble
    x = xh.astype(ld) + xl.astype(ld)
    prod = val.astype(ld) * x[ja]
    ax = np.add.reduceat(prod, ia[:-1].astype(np.int64)) if len(prod) else np.zeros(len(b), dtype=ld)
    r = b.astype(ld) - ax
    return float(np.sqrt(np.sum(r * r)) / np.sqrt(np.sum(b.astype(ld) ** 2)))


@pytest.mark.parametrize("pc,mixed", [("jacobi", False), ("jacobi", True), ("gamg", False)])
def test_refined_beam_below_binary64_floor(env, oracle, pc, mixed):
    V, a, l = _beam(env, 12)
    ia, ja, val = a.csr()
    b = l.to_numpy()
    x, xl = V.element(), V.element()
    st = a.solve_refined(rhs=l, solution=x, solution_lo=xl, rtol=1e-13, pc=pc, mixed=mixed)
    assert st["rel_residual"] <= 1e-13 and st["outer"] >= 2
    xh, xlo = x.to_numpy(), xl.to_numpy()
    if np.finfo(np.longdouble).eps < np.finfo(np.float64).eps:
        assert _residual_ext(ia, ja, val, b, xh, xlo) <= 2e-13
    # the oracle's FP64 PCG on the same system
    xo, it, res = oracle.pcg(ia, ja, val, b, rtol=1e-11, maxit=200000)
    assert np.linalg.norm(xh - xo) <= 1e-8 * np.linalg.norm(xo)


def test_plain_binary64_cg_stalls_where_refinement_converges(env):
    """The binary64 CG cannot certify rtol 1e-13 on the beam (its recomputed residual has a floor near
    u ||A|| ||x|| / ||b||); the refined solve reaches it."""
    V, a, l = _beam(env, 12)
    x = V.element()
    with pytest.raises(fpp.FgpuError):
        a.solve(rhs=l, solution=x, rtol=1e-13, maxit=20000)
    x2, xl2 = V.element(), V.element()
    st = a.solve_refined(rhs=l, solution=x2, solution_lo=xl2, rtol=1e-13)
    assert st["rel_residual"] <= 1e-13
