"""Binary32 quadrature-form element matrices on the tensor cores (tcgen05 kind::tf32, 3xTF32) for curved
(P2-geometry) tetrahedra P1-P3 and Q1/Q2 hexahedra, run on a GB300: within 2e-5 of the largest entry of
the FP64 oracle, within binary32 rounding of the CUDA-core binary32 kernel, repeatable bit for bit, and
over several tiles per block (meshes larger than 128 x the number of blocks)."""
import numpy as np
import pytest

import feelpp_gb300 as fpp
from feelpp_gb300 import meshgen
from oracle import hexoracle as ho_orc

pytestmark = pytest.mark.gpu


def _assemble32(env, M, V, kappa, tc):
    env.set_tensor_cores(tc)
    try:
        u, v = V.element(), V.element()
        a = fpp.form2(test=V, trial=V, precision="f32")
        a.assign(fpp.integrate(fpp.elements(M), kappa * fpp.inner(fpp.gradt(u), fpp.grad(v)) + 0.7 * fpp.idt(u) * fpp.id(v)))
        return a.values()
    finally:
        env.set_tensor_cores(True)


@pytest.mark.parametrize("order,n", [(1, 6), (2, 5), (3, 4), (2, 24)])
def test_curved_tc_matches_oracle_and_cuda_cores(env, oracle, order, n):
    xyz, tets, ho = meshgen.curved_box(n, amp=0.1, perturb=0.1)
    M = fpp.Mesh(xyz, tets, env=env, ho=ho)
    V = fpp.Pch(M, order)
    kappa = meshgen.lognormal_kappa(len(tets))
    tc = _assemble32(env, M, V, kappa, True)
    cc = _assemble32(env, M, V, kappa, False)
    if n <= 6:
        N, l2g = oracle.dof_table(tets, order)
        ia, ja = oracle.pattern(N, l2g)
        val = oracle.assemble_ho(order, xyz, tets, ho, l2g, ia, ja, kappa=kappa, mass=0.7)
        assert np.abs(tc - val).max() <= 2e-5 * np.abs(val).max()
        assert np.abs(cc - val).max() <= 2e-5 * np.abs(val).max()
    # both binary32 paths sum 24-43 points in binary32 in different orders
    assert np.abs(tc - cc).max() <= 1e-5 * np.abs(cc).max()
    assert np.array_equal(_assemble32(env, M, V, kappa, True), tc)


@pytest.mark.parametrize("order,n", [(1, 5), (2, 4), (2, 16)])
def test_hex_tc_matches_oracle_and_cuda_cores(env, order, n):
    xyz, hexes = meshgen.hex_box(n, n, n, perturb=0.2)
    kappa = meshgen.lognormal_kappa(len(hexes))
    M = fpp.Mesh(xyz, hexes, env=env)
    V = fpp.Pch(M, order)
    tc = _assemble32(env, M, V, kappa, True)
    cc = _assemble32(env, M, V, kappa, False)
    assert np.abs(tc - cc).max() <= 1e-5 * np.abs(cc).max()
    if n <= 5:
        N, l2g = ho_orc.dof_table(hexes, order)
        import oracle.pyoracle as orc
        ia, ja = orc.pattern(N, l2g)
        val = ho_orc.assemble(order, xyz, hexes, l2g, ia, ja, kappa=kappa, mass=0.7)
        assert np.abs(tc - val).max() <= 2e-5 * np.abs(val).max()
