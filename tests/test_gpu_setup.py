"""Device-built dof tables, incidence and patterns against the host build (run on a GB300).

The device set-up (first-encounter numbering as a weighted scan over entity keys,
hash-table edge/face identification, per-row bitonic sorts) must give the same
arrays as the host restatement of Feel++'s DofTable / Stencil bit for bit, also on
meshes whose element order and vertex ids are shuffled (so that first encounters
and edge orientations are irregular)."""
import numpy as np
import pytest

import feelpp_gb300 as fpp
from feelpp_gb300 import meshgen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env_host(fgpu_lib):
    return fpp.Environment(host_setup=True)


def _shuffled(n, seed):
    xyz, tets = meshgen.kuhn_box(n, perturb=0.1, seed=seed)
    rng = np.random.default_rng(seed)
    vperm = rng.permutation(len(xyz))              # new id of old vertex v: vperm[v]
    xyz2 = np.empty_like(xyz)
    xyz2[vperm] = xyz
    tets2 = vperm[tets].astype(np.int32)
    tets2 = tets2[rng.permutation(len(tets2))]
    # rotate the vertex order of some elements (same orientation class is not needed here)
    return xyz2, np.ascontiguousarray(tets2)


@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("shuffle", [False, True])
def test_device_setup_equals_host(env, env_host, order, shuffle):
    xyz, tets = _shuffled(5, 11 + order) if shuffle else meshgen.kuhn_box(5, perturb=0.1, seed=3)
    out = []
    for e in (env, env_host):
        M = fpp.Mesh(xyz, tets, env=e)
        V = fpp.Pch(M, order)
        a = fpp.form2(test=V, trial=V)
        ia, ja, _ = a.csr()
        out.append((V.ndof, V.dof_l2g(), ia, ja, V.boundary_dofs()))
    (nd, l2g, ia, ja, bd), (nh, l2gh, iah, jah, bdh) = out
    assert nd == nh
    assert np.array_equal(l2g, l2gh)
    assert np.array_equal(ia, iah) and np.array_equal(ja, jah)
    assert np.array_equal(np.sort(bd), np.sort(bdh))


def test_device_setup_vector_space(env, env_host):
    xyz, tets = _shuffled(4, 5)
    got = []
    for e in (env, env_host):
        M = fpp.Mesh(xyz, tets, env=e)
        V = fpp.Pchv(M, 2)
        a = fpp.form2(test=V, trial=V)
        got.append(a.csr()[:2] + (V.dof_l2g(),))
    for x, y in zip(got[0], got[1]):
        assert np.array_equal(x, y)


def test_device_setup_assembly_matches_oracle_on_shuffled_mesh(env, oracle):
    from tests.helpers import assert_values_close, oracle_system
    xyz, tets = _shuffled(4, 21)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, 3)
    u, v = V.element(), V.element()
    a = fpp.form2(test=V, trial=V)
    a.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.gradt(u), fpp.grad(v)) + fpp.idt(u) * fpp.id(v)))
    N, l2g, ia, ja, val = oracle_system(oracle, xyz, tets, 3, mass=1.0)
    assert np.array_equal(V.dof_l2g(), l2g)
    dia, dja, dval = a.csr()
    assert np.array_equal(dia, ia) and np.array_equal(dja, ja)
    assert_values_close(dval, val)


@pytest.mark.parametrize("order", [1, 2, 3])
def test_boundary_dofs_device_match_oracle(env, oracle, order):
    """Boundary dofs found on the device (face hash with occurrence counts) equal the oracle's, for the
    whole boundary and for a marked plane; repeated queries and moved coordinates stay right."""
    from tests.helpers import mesh
    xyz, tets = mesh(5, perturb=0.2)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, order)
    N, l2g = oracle.dof_table(tets, order)
    for xplane in (None, 0.0):
        mask = oracle.boundary_mask(order, xyz, tets, l2g, N, xplane=xplane)
        got = V.boundary_dofs(xplane)
        assert np.array_equal(got, np.nonzero(mask)[0])
        assert np.array_equal(V.boundary_dofs(xplane), got)
    # moving the mesh changes which faces lie on x <= 0
    xyz2 = xyz.copy()
    xyz2[:, 0] -= 0.5
    M.set_coords(xyz2)
    mask = oracle.boundary_mask(order, xyz2, tets, l2g, N, xplane=0.0)
    assert np.array_equal(V.boundary_dofs(0.0), np.nonzero(mask)[0])
