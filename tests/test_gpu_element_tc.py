"""FP64-accurate element matrices of the affine Laplace/mass form on the bf16 tensor cores (tcgen05
kind::f16, the coefficients and reference tensors cut into exact 8-bit slices; the FGPU_TC_DF64 bit of
fgpu_set_tensor_cores), run on a GB300: the two-phase assembly with them agrees with the CUDA-core df64
element kernel and with native binary64 arithmetic to 1e-13 of each row's largest entry over P1-P3,
ragged last tiles, several tiles per block, mass-only and stiffness-only forms and meshes scaled by
1e3; with kappa spread over eight orders of magnitude between neighbouring elements on a mesh scaled by
1e-3 (stiffness and mass terms of one row up to 1e12 apart) the shared row and column scales of the
slices leave 1e-10 of the row's largest entry, still inside the suite's FP64 parity tolerance; and it
repeats bit for bit."""
import ctypes as C

import numpy as np
import pytest

import feelpp_gb300 as fpp
from feelpp_gb300 import _ffi, meshgen
from tests.helpers import assert_values_close

pytestmark = pytest.mark.gpu


def _assemble(env, V, kappa_elem, kappa, mass, algo=_ffi.ALGO_TWO_PHASE, tc=True):
    import torch
    env.set_tensor_cores(True, df64=tc)
    try:
        d = _ffi.FormDesc()
        d.kind, d.kappa, d.mass, d.quad_degree, d.algo = _ffi.FORM_LAPLACE_MASS, kappa, mass, 0, algo
        kp = None
        if kappa_elem is not None:
            kt = torch.as_tensor(np.ascontiguousarray(kappa_elem, np.float64), device="cuda")
            kp = C.c_void_p(kt.data_ptr())
        a = fpp.form2(test=V, trial=V)
        env.check(env.lib.fgpu_assemble_matrix_dev(env.h, a.h, C.byref(d), kp, 0))
        torch.cuda.synchronize()
        ia, ja, val = a.csr()
        return np.asarray(ia), val
    finally:
        env.set_tensor_cores(True)


def _row_rel(ia, x, ref):
    """largest |x - ref| of each row over that row's largest |ref|"""
    d = np.abs(x - ref)
    r = np.abs(ref)
    rows = np.repeat(np.arange(len(ia) - 1), np.diff(ia))
    dm = np.zeros(len(ia) - 1)
    rm = np.zeros(len(ia) - 1)
    np.maximum.at(dm, rows, d)
    np.maximum.at(rm, rows, r)
    return float((dm / np.where(rm > 0, rm, 1.0)).max())


@pytest.mark.parametrize("order,n", [(1, 9), (2, 7), (3, 5), (2, 24), (3, 13)])
def test_tc_elements_match_cuda_cores_and_native_fp64(env, order, n):
    xyz, tets = meshgen.kuhn_box(n, perturb=0.15, seed=11)
    kappa = meshgen.lognormal_kappa(len(tets), seed=12)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, order)
    ia, tc = _assemble(env, V, kappa, 0.0, 0.7)
    _, cc = _assemble(env, V, kappa, 0.0, 0.7, tc=False)
    _, nat = _assemble(env, V, kappa, 0.0, 0.7, algo=_ffi.ALGO_GATHER_NATIVE_F64)
    assert _row_rel(ia, tc, nat) <= 1e-13
    assert _row_rel(ia, cc, nat) <= 1e-13
    assert np.abs(tc - cc).max() <= 1e-13 * np.abs(nat).max()
    _, again = _assemble(env, V, kappa, 0.0, 0.7)
    assert np.array_equal(again, tc)


@pytest.mark.parametrize("kappa_sigma,scale,mass,row_tol", [(3.0, 1e-3, 1.0, 1e-10), (0.5, 1e3, 1e-4, 1e-13),
                                                            (0.0, 1.0, 0.0, 1e-13), (-1.0, 1.0, 2.0, 1e-13)])
def test_tc_elements_dynamic_range(env, kappa_sigma, scale, mass, row_tol):
    """kappa over many orders of magnitude, tiny and huge meshes (mass against stiffness terms 1e-6 to
    1e6 apart), stiffness only, and mass only (kappa_sigma < 0: kappa = 0)"""
    xyz, tets = meshgen.kuhn_box(10, perturb=0.2, seed=13)
    xyz = xyz * scale
    rng = np.random.default_rng(14)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, 2)
    if kappa_sigma < 0:
        kappa, kc = None, 0.0
    else:
        kappa, kc = np.exp(kappa_sigma * rng.standard_normal(len(tets))), 0.0
    ia, tc = _assemble(env, V, kappa, kc, mass)
    _, nat = _assemble(env, V, kappa, kc, mass, algo=_ffi.ALGO_GATHER_NATIVE_F64)
    _, cc = _assemble(env, V, kappa, kc, mass, tc=False)
    assert np.abs(nat).max() > 0
    assert _row_rel(ia, tc, nat) <= row_tol
    assert _row_rel(ia, cc, nat) <= 1e-13
    assert_values_close(tc, nat, what="tensor-core df64 elements")
