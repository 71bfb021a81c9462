"""Batched assembly of independent problems and CUDA-graph replay (run on a GB300).

A batch runs the same kernels' bodies as the single-problem paths (the two-phase
element/gather-map kernels, or the fused row-owner gather), with the same records,
maps and tables, so every batched matrix must equal the matrix assembled alone by
the same algorithm bit for bit; one problem per order is also checked against the
oracle at the FP64 tolerance."""
import numpy as np
import pytest

import feelpp_gb300 as fpp
from feelpp_gb300 import meshgen
from tests.helpers import assert_values_close, mesh, oracle_system

pytestmark = pytest.mark.gpu


def _problems(env, specs, precision="f64"):
    out = []
    for k, (n, order) in enumerate(specs):
        xyz, tets = meshgen.kuhn_box(n, perturb=0.15, seed=100 + k)
        kappa = meshgen.lognormal_kappa(len(tets), seed=200 + k)
        M = fpp.Mesh(xyz, tets, env=env)
        V = fpp.Pch(M, order)
        u, v = V.element(), V.element()
        integral = fpp.integrate(fpp.elements(M), kappa * fpp.inner(fpp.gradt(u), fpp.grad(v)) + fpp.idt(u) * fpp.id(v))
        a = fpp.form2(test=V, trial=V, precision=precision)
        out.append((xyz, tets, kappa, M, V, integral, a))
    return out


SPECS = [(3, 1), (5, 2), (2, 3), (7, 1), (4, 3), (3, 2), (6, 2), (1, 1), (2, 2), (3, 3)]


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("algo", ["two_phase", "gather"])
def test_batch_equals_single_assembly(env, precision, algo):
    from feelpp_gb300 import _ffi
    probs = _problems(env, SPECS, precision)
    batch = fpp.Batch([p[6] for p in probs], [p[5] for p in probs])
    batch.set_algo(algo)
    batch.assemble()
    cfg = batch.launch_config()
    assert cfg["tuned"] and cfg["threads"] in (128, 256) and cfg["two_phase"] == (algo == "two_phase")
    got = [p[6].values().copy() for p in probs]
    for (xyz, tets, kappa, M, V, integral, a), g in zip(probs, got):
        a.zero()
        a.algo = _ffi.ALGO_TWO_PHASE if algo == "two_phase" else _ffi.ALGO_GATHER
        a.assign(integral)
        assert np.array_equal(g, a.values())
        a.algo = _ffi.ALGO_AUTO
    # '+=' doubles every value (the df64 path adds the stored binary64 value as a
    # double-float: 2^-48 relative; binary32 storage: one rounding)
    batch.assemble(accumulate=True)
    for (xyz, tets, kappa, M, V, integral, a), g in zip(probs, got):
        np.testing.assert_allclose(a.values(), 2 * g, rtol=1e-6 if precision == "f32" else 1e-13, atol=0)


def test_batch_matches_oracle(env, oracle):
    probs = _problems(env, [(4, 1), (3, 2), (2, 3)])
    batch = fpp.Batch([p[6] for p in probs], [p[5] for p in probs])
    batch.assemble()
    for (xyz, tets, kappa, M, V, integral, a), order in zip(probs, (1, 2, 3)):
        N, l2g, ia, ja, val = oracle_system(oracle, xyz, tets, order, kappa=kappa, mass=1.0)
        assert_values_close(a.values(), val, what="batched P%d" % order)


def test_batch_pinned_launch_and_graph(env):
    probs = _problems(env, SPECS[:5])
    batch = fpp.Batch([p[6] for p in probs], [p[5] for p in probs])
    batch.set_launch(128, 4)
    batch.assemble()
    ref = [p[6].values().copy() for p in probs]
    for p in probs:
        p[6].zero()
    with fpp.capture(env) as g:
        batch.assemble()
    for p in probs:                       # capture records, it does not run
        assert not p[6].values().any()
    g.launch(3)
    for p, r in zip(probs, ref):
        assert np.array_equal(p[6].values(), r)


def test_batch_rejects_mixed_precision(env):
    probs = _problems(env, [(2, 1)], "f64") + _problems(env, [(2, 1)], "f32")
    with pytest.raises(fpp.FgpuError):
        fpp.Batch([p[6] for p in probs], [p[5] for p in probs])
