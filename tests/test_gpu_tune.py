"""Launch-shape autotuner (run on a GB300): the two-phase assembly's shapes (threads per block, blocks
per SM, contributions per load batch) are timed on the first assembly of a key, the picks are
appended to the cache file named in fgpu_config.tune_cache and read back by a later context, and
the tuned shapes give the same bits as the fixed default shapes."""
import os
import tempfile

import numpy as np
import pytest

import feelpp_gb300 as fpp
from feelpp_gb300 import meshgen

pytestmark = pytest.mark.gpu


def _assemble(env, xyz, tets, kappa, order, precision):
    M = fpp.Mesh(xyz, tets, env=env)
    V = fpp.Pch(M, order)
    u, v = V.element(), V.element()
    a = fpp.form2(test=V, trial=V, precision=precision)
    a.assign(fpp.integrate(fpp.elements(M), kappa * fpp.inner(fpp.gradt(u), fpp.grad(v)) + fpp.idt(u) * fpp.id(v)))
    return a


@pytest.mark.parametrize("order,n", [(1, 20), (2, 12), (3, 8)])
def test_tuned_shapes_keep_the_bits_and_persist(order, n):
    xyz, tets = meshgen.kuhn_box(n, perturb=0.15, seed=21)
    kappa = meshgen.lognormal_kappa(len(tets), seed=22)
    with tempfile.TemporaryDirectory() as d:
        cache = os.path.join(d, "tune.txt")
        fixed = fpp.Environment(tune=False)
        tuned = fpp.Environment(tune=True, tune_cache=cache)
        for precision in ("f64", "f32"):
            ref = _assemble(fixed, xyz, tets, kappa, order, precision).values()
            l0 = tuned.launches()
            got = _assemble(tuned, xyz, tets, kappa, order, precision).values()
            assert tuned.launches() - l0 > 100                 # the candidates were timed
            assert np.array_equal(got, ref)
        lines = open(cache).read().split("\n")
        keys = [ln.split()[0] for ln in lines if ln.startswith("two_phase|")]
        assert any("|P%d|f64|" % order in k for k in keys) and any("|P%d|f32|" % order in k for k in keys)
        for ln in lines:
            if ln.startswith("two_phase|"):
                th, bp, gth, gbp, batch, pipe = map(int, ln.split()[1:])
                assert th in (128, 256) and bp in (4, 8, 16, 32) and gth in (128, 256)
                assert gbp in ((2, 4, 6, 8, 12, 16) if pipe else (8, 16, 32, 64))
                assert batch in (2, 4, 8) and pipe in (0, 1)
        # a later context reads the picks: no timing on its first assembly
        later = fpp.Environment(tune=True, tune_cache=cache)
        l0 = later.launches()
        again = _assemble(later, xyz, tets, kappa, order, "f64").values()
        assert later.launches() - l0 < 50
        assert np.array_equal(again, _assemble(fixed, xyz, tets, kappa, order, "f64").values())
        # the plain and the software-pipelined gather, whichever the tuner picked: the same bits
        for pipe in (0, 1):
            forced = os.path.join(d, "forced%d.txt" % pipe)
            with open(forced, "w") as f:
                for ln in lines:
                    if ln.startswith("two_phase|"):
                        f.write(" ".join(ln.split()[:6] + [str(pipe)]) + "\n")
            env_h = fpp.Environment(tune=True, tune_cache=forced)
            for precision in ("f64", "f32"):
                got = _assemble(env_h, xyz, tets, kappa, order, precision).values()
                assert np.array_equal(got, _assemble(fixed, xyz, tets, kappa, order, precision).values())


def test_cg_spmv_pick_is_recorded():
    xyz, tets = meshgen.kuhn_box(10, perturb=0.15, seed=23)
    with tempfile.TemporaryDirectory() as d:
        cache = os.path.join(d, "tune.txt")
        env = fpp.Environment(tune=True, tune_cache=cache)
        M = fpp.Mesh(xyz, tets, env=env)
        V = fpp.Pch(M, 2)
        u, v = V.element(), V.element()
        a = fpp.form2(test=V, trial=V)
        a.assign(fpp.integrate(fpp.elements(M), fpp.inner(fpp.gradt(u), fpp.grad(v))))
        l = fpp.form1(test=V)
        l.assign(fpp.integrate(fpp.elements(M), fpp.sine_source() * fpp.id(v)))
        a += fpp.on(fpp.boundaryfaces(M), rhs=l, element=u, expr=0.0, type="elimination_symmetric")
        st = a.solve(rhs=l, solution=u, rtol=1e-10)
        assert st["rel_residual"] <= 1e-10
        picks = [ln.split() for ln in open(cache) if ln.startswith("spmv|")]
        assert picks and int(picks[-1][1]) in (0, 4, 8, 16, 32)
