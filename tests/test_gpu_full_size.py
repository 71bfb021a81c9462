"""Size-independent properties at the full configuration sizes on a GB300: the P2 and P3 assemblies on the
64^3 Kuhn mesh (1 572 864 tetrahedra; 60.9 M and 345.6 M entries) with lognormal kappa. The closed-form dof
and entry counts of the COUPLED pattern, sorted rows with a diagonal, zero row sums of the Laplacian,
symmetry, 1^T M 1 = |Omega|, bit-identical repeated assembly, and the FP32 assembly within single-precision
rounding of the FP64 one."""
import numpy as np
import pytest

import feelpp_gb300 as fpp
from feelpp_gb300 import meshgen

pytestmark = pytest.mark.gpu

N_MESH = 64


@pytest.fixture(scope="module")
def mesh64(env):
    xyz, tets = meshgen.kuhn_box(N_MESH, perturb=0.15, seed=1234)
    kappa = meshgen.lognormal_kappa(len(tets), seed=5678)
    return fpp.Mesh(xyz, tets, env=env), kappa


def nnz_formula(order, n):
    return {2: 230 * n ** 3 + 138 * n ** 2 + 24 * n + 1, 3: 1311 * n ** 3 + 459 * n ** 2 + 45 * n + 1}[order]


@pytest.mark.parametrize("order", [2, 3])
def test_full_size_properties(mesh64, order):
    import scipy.sparse as sp
    M, kappa = mesh64
    n = N_MESH
    V = fpp.Pch(M, order)
    assert V.ndof == (order * n + 1) ** 3
    u, v = V.element(), V.element()
    a = fpp.form2(test=V, trial=V)
    a.assign(fpp.integrate(fpp.elements(M), kappa * fpp.inner(fpp.gradt(u), fpp.grad(v))))
    assert a.nnz == nnz_formula(order, n)
    ia, ja, val = a.csr()
    rows = np.repeat(np.arange(V.ndof, dtype=np.int64), np.diff(ia))
    # sorted columns in every row, and the diagonal present
    inrow = np.diff(ja.astype(np.int64)) > 0
    assert np.all(inrow | (np.diff(rows) > 0))
    assert np.count_nonzero(ja == rows) == V.ndof
    A = sp.csr_matrix((val, ja, ia), shape=(V.ndof, V.ndof))
    scale = np.abs(val).max()
    assert np.abs(A @ np.ones(V.ndof)).max() < 1e-11 * scale          # constants in the kernel
    if order == 2:
        assert abs(A - A.T).max() < 1e-14 * scale                     # symmetric
    # repeated assembly: the same bits
    a.assign(fpp.integrate(fpp.elements(M), kappa * fpp.inner(fpp.gradt(u), fpp.grad(v))))
    assert np.array_equal(a.values(), val)
    # binary32 within single-precision rounding of the binary64 values
    a32 = fpp.form2(test=V, trial=V, precision="f32")
    a32.assign(fpp.integrate(fpp.elements(M), kappa * fpp.inner(fpp.gradt(u), fpp.grad(v))))
    assert np.abs(a32.values() - val).max() <= 2e-5 * scale
    del a32, A
    m = fpp.form2(test=V, trial=V)
    m.assign(fpp.integrate(fpp.elements(M), fpp.idt(u) * fpp.id(v)))
    assert abs(m.values().sum() - 1.0) < 1e-10                         # 1^T M 1 = |Omega|
