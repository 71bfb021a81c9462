"""EnSight Gold export of device results (run on a GB300): the files parse back to the mesh and to the
vertex values of the fields."""
import numpy as np
import pytest

import feelpp_gb300 as fpp
from tests.helpers import mesh

pytestmark = pytest.mark.gpu


def read_str(f):
    return f.read(80).split(b"\x00")[0].decode().strip()


def read_geo(path):
    with open(path, "rb") as f:
        assert read_str(f) == "C Binary"
        read_str(f), read_str(f)
        assert read_str(f) == "node id off" and read_str(f) == "element id off"
        assert read_str(f) == "part"
        assert np.frombuffer(f.read(4), np.int32)[0] == 1
        read_str(f)
        assert read_str(f) == "coordinates"
        nv = int(np.frombuffer(f.read(4), np.int32)[0])
        xyz = np.frombuffer(f.read(12 * nv), np.float32).reshape(3, nv).T
        assert read_str(f) == "tetra4"
        nt = int(np.frombuffer(f.read(4), np.int32)[0])
        conn = np.frombuffer(f.read(16 * nt), np.int32).reshape(nt, 4)
        assert f.read() == b""
    return xyz, conn


def read_scl(path, nv):
    with open(path, "rb") as f:
        read_str(f)
        assert read_str(f) == "part" and np.frombuffer(f.read(4), np.int32)[0] == 1
        assert read_str(f) == "coordinates"
        v = np.frombuffer(f.read(4 * nv), np.float32)
        assert f.read() == b""
    return v


@pytest.mark.parametrize("order", [1, 3])
def test_export_ensight(env, oracle, tmp_path, order):
    xyz, tets = mesh(4, perturb=0.2)
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, order)
    u = V.element()
    x = np.random.default_rng(3).standard_normal(V.ndof)
    u.upload(x)
    w = V.element()
    w.upload(2.0 * x + 1.0)
    prefix = tmp_path / "sol"
    fpp.export_ensight(V, prefix, {"u": u, "w2": w})
    case = (tmp_path / "sol.case").read_text()
    assert "type: ensight gold" in case and "model: sol.geo" in case and "scalar per node: u sol.u.scl" in case
    gx, conn = read_geo(tmp_path / "sol.geo")
    assert np.array_equal(gx, xyz.astype(np.float32)) and np.array_equal(conn, tets + 1)
    N, l2g = oracle.dof_table(tets, order)
    vdof = np.zeros(len(xyz), dtype=np.int64)
    vdof[tets.reshape(-1)] = l2g[:, :4].reshape(-1)
    assert np.array_equal(read_scl(tmp_path / "sol.u.scl", len(xyz)), x[vdof].astype(np.float32))
    assert np.array_equal(read_scl(tmp_path / "sol.w2.scl", len(xyz)), (2.0 * x + 1.0)[vdof].astype(np.float32))
    with pytest.raises(fpp.FgpuError):
        fpp.export_ensight(V, prefix, {"bad name": u})
