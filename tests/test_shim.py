"""The C++ shim (include/fgpu_feel.hpp): a Feel++-style program written with form2 / integrate /
on / solve compiles and links against the C-ABI library on the CPU; on a GB300 it runs and gives
the same CSR arrays, load vector and solution as the Python front end, and the oracle's pattern
and values."""
import os
import subprocess
import sys
import tempfile

import numpy as np
import pytest

from tests.conftest import ROOT
from tests.helpers import assert_values_close, oracle_system

sys.path.insert(0, os.path.join(ROOT, "tests", "cpp"))


def test_shim_program_compiles_and_links(fgpu_lib):
    import build_shim
    exe = build_shim.build()
    assert os.access(exe, os.X_OK)


def _write_input(path, xyz, tets, kappa):
    with open(path, "wb") as f:
        np.array([len(xyz), len(tets)], dtype=np.int64).tofile(f)
        np.ascontiguousarray(xyz, dtype=np.float64).tofile(f)
        np.ascontiguousarray(tets, dtype=np.int32).tofile(f)
        np.ascontiguousarray(kappa, dtype=np.float64).tofile(f)


def _read_output(path):
    raw = open(path, "rb").read()
    off = 0

    def take(dtype, n):
        nonlocal off
        a = np.frombuffer(raw, dtype=dtype, count=n, offset=off)
        off += a.nbytes
        return a
    nrows, nnz = take(np.int64, 2)
    out = {"ia": take(np.int32, nrows + 1), "ja": take(np.int32, nnz), "val": take(np.float64, nnz),
           "load": take(np.float64, nrows), "u": take(np.float64, nrows)}
    out["iterations"] = int(take(np.int64, 1)[0])
    out["rel_residual"], out["l2"], out["h1"] = take(np.float64, 3)
    return out


@pytest.mark.gpu
def test_shim_poisson_matches_python_front_end_and_oracle(env, oracle):
    import build_shim
    import feelpp_gb300 as fpp
    from feelpp_gb300 import meshgen
    exe = build_shim.build()
    xyz, tets = meshgen.kuhn_box(6, perturb=0.15, seed=1234)
    kappa = meshgen.lognormal_kappa(len(tets), seed=5678)
    with tempfile.TemporaryDirectory() as d:
        fin, fout = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        _write_input(fin, xyz, tets, kappa)
        r = subprocess.run([exe, fin, fout, "--ksp-type", "cg", "--pc-type", "jacobi", "--on.type", "elimination_symmetric",
                            "--ksp-rtol", "1e-10"], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        got = _read_output(fout)
    # the oracle: GraphCSR pattern and FP64 values
    N, l2g, ia, ja, val = oracle_system(oracle, xyz, tets, 2, kappa=kappa, mass=1.0)
    assert np.array_equal(got["ia"].astype(np.int64), ia) and np.array_equal(got["ja"], ja)
    assert_values_close(got["val"], val, what="shim P2 matrix")
    F = oracle.rhs(2, xyz, tets, l2g, N, fkind=0)
    assert_values_close(got["load"], F, what="shim load vector")
    # the Python front end on the same device, same calls: identical bits
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, 2)
    u, v = V.element(), V.element()
    a = fpp.form2(test=V, trial=V)
    a.assign(fpp.integrate(fpp.elements(M), kappa * fpp.inner(fpp.gradt(u), fpp.grad(v)) + fpp.idt(u) * fpp.id(v)))
    assert np.array_equal(a.values(), got["val"])
    l = fpp.form1(test=V)
    l.assign(fpp.integrate(fpp.elements(M), fpp.sine_source() * fpp.id(v)))
    a += fpp.on(fpp.boundaryfaces(M), rhs=l, element=u, expr=0.0, type="elimination_symmetric")
    st = a.solve(rhs=l, solution=u, rtol=1e-10)
    assert got["iterations"] == st["iterations"] and got["rel_residual"] <= 1e-10
    np.testing.assert_allclose(got["u"], u.to_numpy(), rtol=0, atol=1e-12 * np.abs(got["u"]).max())
    l2, h1 = u.errors_sine()
    assert abs(got["l2"] - l2) <= 1e-12 * l2


@pytest.mark.gpu
def test_shim_defaults_are_feelpp_defaults(env):
    """Without options the shim uses Feel++'s defaults: on.type=elimination (non-symmetric) and
    ksp-type=gmres; the solve still reaches the tolerance."""
    import build_shim
    from feelpp_gb300 import meshgen
    exe = build_shim.build()
    xyz, tets = meshgen.kuhn_box(4, perturb=0.1, seed=3)
    kappa = np.ones(len(tets))
    with tempfile.TemporaryDirectory() as d:
        fin, fout = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        _write_input(fin, xyz, tets, kappa)
        r = subprocess.run([exe, fin, fout], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        got = _read_output(fout)
    assert got["rel_residual"] <= 1e-10 and got["iterations"] > 0
