"""Shared helpers for the parity tests (meshes, oracle assembly, tolerances)."""
import numpy as np

from feelpp_gb300 import meshgen

# Plain FP64 path: per-entry |a - b| <= RTOL * |b| + ATOL * max|A| (the absolute
# floor covers entries that cancel to ~0; both sides sum the same terms in
# different orders).
RTOL_F64 = 1e-12
ATOL_F64 = 1e-14


def mesh(n, perturb=0.2, seed=1234, lengths=(1.0, 1.0, 1.0)):
    return meshgen.kuhn_box(n, lengths=lengths, perturb=perturb, seed=seed)


def oracle_system(oracle, xyz, tets, order, kappa=None, mass=1.0, ncomp=1, kind=0, lam=1.0, mu=0.5, qdeg=None):
    N, l2g = oracle.dof_table(tets, order, ncomp)
    ia, ja = oracle.pattern(N, l2g)
    val = oracle.assemble(order, xyz, tets, l2g, ia, ja, kind=kind, kappa=kappa, mass=mass, lam=lam, mu=mu,
                          qdeg=qdeg, ncomp=ncomp)
    return N, l2g, ia, ja, val


def assert_values_close(got, ref, rtol=RTOL_F64, atol=ATOL_F64, what="values"):
    scale = np.abs(ref).max()
    err = np.abs(got - ref)
    bad = err > rtol * np.abs(ref) + atol * scale
    assert not bad.any(), "%s: %d entries differ, worst abs %.3e (scale %.3e)" % (what, bad.sum(), err.max(), scale)
