"""ctypes bindings of the oracle library (test infrastructure only).

Every function mirrors one ``orc_*`` entry point of ``oracle/oracle.cpp``;
arrays are numpy arrays (float64 / int32 / int64, C-contiguous).
"""
import ctypes as C
import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        P = C.c_void_p
        i64, i32, f64 = C.c_int64, C.c_int, C.c_double
        sig = {
            "orc_version": (i32, []),
            "orc_quad": (i32, [i32, P]),
            "orc_nodes": (i32, [i32, P]),
            "orc_gll": (i32, [i32, P]),
            "orc_tabulate": (i32, [i32, i32, P, P, P]),
            "orc_dof_table": (i64, [i64, P, i32, i32, P]),
            "orc_pattern": (i32, [i64, i64, i32, P, P, P]),
            "orc_geometry": (i32, [P, i64, P, P, P, P]),
            "orc_assemble": (i32, [i32, i32, i32, P, i64, P, P, i32, P, f64, f64, f64, f64, i64, P, P, P, i32, i64]),
            "orc_rhs": (i32, [i32, i32, i32, P, i64, P, P, i32, P, P]),
            "orc_assemble_ho": (i32, [i32, i32, P, i64, P, P, P, P, f64, f64, P, P, P]),
            "orc_rhs_ho": (i32, [i32, i32, P, i64, P, P, P, i32, P, P]),
            "orc_boundary_mask": (i32, [i32, i32, P, i64, P, P, i32, f64, i64, P]),
            "orc_dirichlet": (i32, [i64, P, P, P, P, P, P, i32, f64]),
            "orc_spmv": (i32, [i64, P, P, P, P, P]),
            "orc_pcg": (i32, [i64, P, P, P, P, P, f64, i32, P, i32]),
            "orc_errors": (i32, [i32, i32, P, i64, P, P, P, P, P]),
            "orc_num_threads": (i32, []),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def nloc(order):
    return (order + 1) * (order + 2) * (order + 3) // 6


def quad(deg):
    n = lib().orc_quad(deg, None)
    out = np.zeros((n, 4))
    lib().orc_quad(deg, _p(out))
    return out


def nodes(order):
    out = np.zeros((nloc(order), 3))
    lib().orc_nodes(order, _p(out))
    return out


def gll(n):
    out = np.zeros(n)
    lib().orc_gll(n, _p(out))
    return out


def tabulate(order, pts):
    pts = _c(pts, np.float64)
    n = nloc(order)
    phi = np.zeros((len(pts), n))
    dphi = np.zeros((len(pts), n, 3))
    lib().orc_tabulate(order, len(pts), _p(pts), _p(phi), _p(dphi))
    return phi, dphi


def dof_table(tets, order, ncomp=1):
    tets = _c(tets, np.int32)
    T = len(tets)
    l2g = np.zeros((T, nloc(order) * ncomp), dtype=np.int32)
    N = lib().orc_dof_table(T, _p(tets), order, ncomp, _p(l2g))
    return int(N), l2g


def pattern(N, l2g):
    l2g = _c(l2g, np.int32)
    ia = np.zeros(N + 1, dtype=np.int64)
    lib().orc_pattern(N, l2g.shape[0], l2g.shape[1], _p(l2g), _p(ia), None)
    ja = np.zeros(int(ia[-1]), dtype=np.int32)
    lib().orc_pattern(N, l2g.shape[0], l2g.shape[1], _p(l2g), _p(ia), _p(ja))
    return ia, ja


def geometry(xyz, tets):
    xyz = _c(xyz, np.float64)
    tets = _c(tets, np.int32)
    T = len(tets)
    J = np.zeros(T)
    B = np.zeros((T, 3, 3))
    d = np.zeros(T)
    lib().orc_geometry(_p(xyz), T, _p(tets), _p(J), _p(B), _p(d))
    return J, B, d


def assemble(order, xyz, tets, l2g, ia, ja, kind=0, kappa=None, kappa_const=1.0, mass=0.0,
             lam=1.0, mu=0.5, qdeg=None, ncomp=1, nthreads=1, val=None):
    xyz = _c(xyz, np.float64)
    tets = _c(tets, np.int32)
    l2g = _c(l2g, np.int32)
    if qdeg is None:
        qdeg = 2 * order
    N = len(ia) - 1
    if val is None:
        val = np.zeros(len(ja))
    kap = None if kappa is None else _c(kappa, np.float64)
    rc = lib().orc_assemble(order, ncomp, qdeg, _p(xyz), len(tets), _p(tets), _p(l2g), kind, _p(kap),
                            kappa_const, mass, lam, mu, N, _p(ia), _p(ja), _p(val), nthreads, len(xyz))
    if rc != 0:
        raise RuntimeError("orc_assemble failed: %d" % rc)
    return val


def rhs(order, xyz, tets, l2g, N, fkind=0, fc=(0.0, 0.0, 0.0), qdeg=None, ncomp=1):
    xyz = _c(xyz, np.float64)
    tets = _c(tets, np.int32)
    l2g = _c(l2g, np.int32)
    if qdeg is None:
        qdeg = 2 * order
    F = np.zeros(N)
    fcv = np.array(fc, dtype=np.float64)
    rc = lib().orc_rhs(order, ncomp, qdeg, _p(xyz), len(tets), _p(tets), _p(l2g), fkind, _p(fcv), _p(F))
    if rc != 0:
        raise RuntimeError("orc_rhs failed: %d" % rc)
    return F


def boundary_mask(order, xyz, tets, l2g, N, ncomp=1, xplane=None):
    xyz = _c(xyz, np.float64)
    tets = _c(tets, np.int32)
    l2g = _c(l2g, np.int32)
    mask = np.zeros(N, dtype=np.uint8)
    lib().orc_boundary_mask(order, ncomp, _p(xyz), len(tets), _p(tets), _p(l2g),
                            0 if xplane is None else 1, 0.0 if xplane is None else xplane, N, _p(mask))
    return mask


def dirichlet(ia, ja, val, b, mask, g=None, mode=0, diag=1.0):
    N = len(ia) - 1
    gg = None if g is None else _c(g, np.float64)
    lib().orc_dirichlet(N, _p(ia), _p(ja), _p(val), _p(b), _p(mask), _p(gg), mode, diag)


def spmv(ia, ja, val, x):
    y = np.zeros(len(ia) - 1)
    lib().orc_spmv(len(ia) - 1, _p(ia), _p(ja), _p(val), _p(_c(x, np.float64)), _p(y))
    return y


def pcg(ia, ja, val, b, rtol=1e-10, maxit=10000, nthreads=1):
    N = len(ia) - 1
    x = np.zeros(N)
    res = np.zeros(1)
    it = lib().orc_pcg(N, _p(ia), _p(ja), _p(val), _p(_c(b, np.float64)), _p(x), rtol, maxit, _p(res), nthreads)
    return x, int(it), float(res[0])


def errors(order, xyz, tets, l2g, u, qdeg):
    l2 = np.zeros(1)
    h1 = np.zeros(1)
    rc = lib().orc_errors(order, qdeg, _p(_c(xyz, np.float64)), len(tets), _p(_c(tets, np.int32)),
                          _p(_c(l2g, np.int32)), _p(_c(u, np.float64)), _p(l2), _p(h1))
    if rc != 0:
        raise RuntimeError("orc_errors failed")
    return float(l2[0]), float(h1[0])


def num_threads():
    return lib().orc_num_threads()


# ---------------------------------------------------------------------------
# Boundary-face integrals (integrator.hpp MESH_FACES, :786-795), restated with
# numpy on top of the oracle's basis tabulation: boundary faces are the faces
# of one element (found by counting sorted vertex triples), visited in element
# order; each face integral uses a collapsed Gauss-Legendre rule (numpy's
# leggauss, 6 x 6 points, exact far beyond the degree-6 integrands) in the
# element's reference coordinates, scaled by the physical face area (affine
# faces). Face blocks are added like MatSetValues(ADD_VALUES).
# ---------------------------------------------------------------------------
_REF_VERTS = np.array([[-1.0, -1.0, -1.0], [1.0, -1.0, -1.0], [-1.0, 1.0, -1.0], [-1.0, -1.0, 1.0]])
_FACE_VERTS = np.array([[1, 2, 3], [0, 2, 3], [0, 1, 3], [0, 1, 2]])


def boundary_faces(xyz, tets, xplane=None):
    """(element, local face) of the faces of exactly one element, in element order; with xplane only
    those whose three vertices have x <= xplane + 1e-12."""
    counts = {}
    keys = []
    for e, t in enumerate(tets):
        for f in range(4):
            k = tuple(sorted(int(t[v]) for v in _FACE_VERTS[f]))
            keys.append(k)
            counts[k] = counts.get(k, 0) + 1
    out = []
    for idx, k in enumerate(keys):
        if counts[k] != 1:
            continue
        e, f = divmod(idx, 4)
        if xplane is not None and not all(xyz[v, 0] <= xplane + 1e-12 for v in k):
            continue
        out.append((e, f))
    return out


def _face_rule(f, npts=6):
    g, w = np.polynomial.legendre.leggauss(npts)
    u = (g + 1) / 2
    wu = w / 2
    A, B, C = _REF_VERTS[_FACE_VERTS[f]]
    pts, wts = [], []
    for i in range(npts):
        for j in range(npts):
            s, t = u[i], u[j] * (1 - u[i])
            pts.append(A + s * (B - A) + t * (C - A))
            wts.append(wu[i] * wu[j] * (1 - u[i]))
    wts = np.array(wts)
    return np.array(pts), wts / wts.sum()          # weights per unit face area


def _face_area(xyz, tets, e, f):
    P = xyz[tets[e][_FACE_VERTS[f]]]
    return 0.5 * np.linalg.norm(np.cross(P[1] - P[0], P[2] - P[0]))


def face_matrix(order, xyz, tets, l2g, ia, ja, alpha, xplane=None, val=None):
    """val (nnz) += alpha int_faces phi_i phi_j, scattered into the CSR (ia, ja)."""
    val = np.zeros(len(ja)) if val is None else val
    tab = {}
    for e, f in boundary_faces(xyz, tets, xplane):
        if f not in tab:
            pts, w = _face_rule(f)
            phi, _ = tabulate(order, pts)
            tab[f] = (phi * w[:, None]).T @ phi
        blk = alpha * _face_area(xyz, tets, e, f) * tab[f]
        dofs = l2g[e]
        for a, r in enumerate(dofs):
            cols = ja[ia[r]:ia[r + 1]]
            for b, c in enumerate(dofs):
                val[ia[r] + np.searchsorted(cols, c)] += blk[a, b]
    return val


def face_load(order, xyz, tets, l2g, N, g, xplane=None):
    """F (N) = g int_faces phi_i."""
    F = np.zeros(N)
    tab = {}
    for e, f in boundary_faces(xyz, tets, xplane):
        if f not in tab:
            pts, w = _face_rule(f)
            phi, _ = tabulate(order, pts)
            tab[f] = w @ phi
        F[l2g[e]] += g * _face_area(xyz, tets, e, f) * tab[f]
    return F


def _face_normal_h(xyz, tets, e, f):
    """Unit outward normal and hFace (longest face edge, feelpp/feel/feelmesh/geond.hpp:737-757)."""
    P = xyz[tets[e][_FACE_VERTS[f]]]
    c = np.cross(P[1] - P[0], P[2] - P[0])
    nrm = c / np.linalg.norm(c)
    if np.dot(nrm, xyz[tets[e][f]] - P[0]) > 0:
        nrm = -nrm
    h = max(np.linalg.norm(P[1] - P[0]), np.linalg.norm(P[2] - P[0]), np.linalg.norm(P[2] - P[1]))
    return nrm, h


def face_terms_matrix(order, xyz, tets, l2g, ia, ja, mass=0.0, mass_h=0.0, dn_trial=0.0, dn_test=0.0, xplane=None,
                      val=None):
    """val (nnz) += int_faces mass u v + mass_h u v / hFace + dn_trial (grad u . N) v + dn_test (grad v . N) u,
    by quadrature in physical space (gradients B grad_ref, B from the oracle's geometry)."""
    val = np.zeros(len(ja)) if val is None else val
    _, Bs, _ = geometry(xyz, tets)
    for e, f in boundary_faces(xyz, tets, xplane):
        pts, w = _face_rule(f)
        phi, dref = tabulate(order, pts)                       # (q, n), (q, n, 3)
        grad = np.einsum("da,qna->qnd", Bs[e], dref)          # physical gradients
        nrm, h = _face_normal_h(xyz, tets, e, f)
        dn = grad @ nrm                                        # (q, n)
        A = _face_area(xyz, tets, e, f)
        blk = (mass + mass_h / h) * (phi * w[:, None]).T @ phi
        blk += dn_trial * (phi * w[:, None]).T @ dn            # (i, j): phi_i (grad phi_j . n)
        blk += dn_test * (dn * w[:, None]).T @ phi             # (i, j): (grad phi_i . n) phi_j
        blk *= A
        dofs = l2g[e]
        for a, r in enumerate(dofs):
            cols = ja[ia[r]:ia[r + 1]]
            for b, c in enumerate(dofs):
                val[ia[r] + np.searchsorted(cols, c)] += blk[a, b]
    return val


def face_terms_load(order, xyz, tets, l2g, N, g=0.0, g_h=0.0, g_dn=0.0, xplane=None):
    """F (N) = int_faces g v + g_h v / hFace + g_dn (grad v . N)."""
    F = np.zeros(N)
    _, Bs, _ = geometry(xyz, tets)
    for e, f in boundary_faces(xyz, tets, xplane):
        pts, w = _face_rule(f)
        phi, dref = tabulate(order, pts)
        grad = np.einsum("da,qna->qnd", Bs[e], dref)
        nrm, h = _face_normal_h(xyz, tets, e, f)
        A = _face_area(xyz, tets, e, f)
        F[l2g[e]] += A * ((g + g_h / h) * (w @ phi) + g_dn * (w @ (grad @ nrm)))
    return F


def assemble_ho(order, xyz, tets, ho, l2g, ia, ja, kappa=None, kappa_const=1.0, mass=0.0, qdeg=None):
    """Scalar kappa grad.grad + mass u v on curved (P2-geometry) tetrahedra; ho = T x 6 x 3 edge nodes."""
    qdeg = 2 * order + 2 if qdeg is None else qdeg
    val = np.zeros(len(ja))
    kap = None if kappa is None else _c(kappa, np.float64)
    rc = lib().orc_assemble_ho(order, qdeg, _p(_c(xyz, np.float64)), len(tets), _p(_c(tets, np.int32)),
                               _p(_c(ho, np.float64)), _p(_c(l2g, np.int32)), _p(kap), kappa_const, mass,
                               _p(_c(ia, np.int64)), _p(_c(ja, np.int32)), _p(val))
    if rc != 0:
        raise RuntimeError("orc_assemble_ho failed: %d" % rc)
    return val


def rhs_ho(order, xyz, tets, ho, l2g, N, fkind=0, c=0.0, qdeg=None):
    qdeg = 2 * order + 2 if qdeg is None else qdeg
    F = np.zeros(N)
    fc = np.array([c, 0.0, 0.0])
    rc = lib().orc_rhs_ho(order, qdeg, _p(_c(xyz, np.float64)), len(tets), _p(_c(tets, np.int32)), _p(_c(ho, np.float64)),
                          _p(_c(l2g, np.int32)), fkind, _p(fc), _p(F))
    if rc != 0:
        raise RuntimeError("orc_rhs_ho failed: %d" % rc)
    return F
