"""CPU restatement of the reference's hexahedral (Hypercube<3,1>) Q1/Q2 path, in numpy.

Test infrastructure only (the checker of the device path, never called by the product).

Follows, in the reference:
* reference hexahedron [-1,1]^3 and its vertex order: feelpp/feel/feelmesh/refhypercube.hpp:148-183;
* local edges, faces and the Q2 points on them: feelpp/feel/feelmesh/hypercubeordering.hpp
  (hexa::__e2p_order1/__e2p_order2, __f2p_order1/__f2p_order2): vertex dofs 0-7, edge j -> 8 + j,
  face f -> 20 + f, interior 26;
* dof numbering by first encounter over (element, local dof): feelpp/feel/feeldiscr/doftable.hpp:2364-2455;
* tensor Gauss-Legendre quadrature with (o + 1) // 2 + 1 points per direction, x slowest, weights
  w_i w_j w_l: feelpp/feel/feelpoly/gausshypercube.cpp (GaussHypercube::gaussdegree and operator()<3>);
* trilinear map and K, J, B = K^-T at every quadrature point: feelpp/feel/feelpoly/geomap.hpp:1971-1991;
* element matrix sum_q w_q J_q (kappa grad phi_j . grad phi_i + m phi_j phi_i) and scatter-add into the
  COUPLED CSR pattern: feelpp/feel/feelvf/bilinearformcontext.hpp:552-590, 784-847.

The 1D rule comes from numpy's leggauss and the Lagrange functions from their defining products
(independently of the device set-up, which computes both itself).
"""
import numpy as np

HEX_VERTS = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                      [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], dtype=np.float64)
HEX_EDGES = ((0, 1), (1, 2), (2, 3), (3, 0), (1, 5), (5, 4), (4, 0), (2, 6), (6, 5), (3, 7), (7, 6), (4, 7))
HEX_FACES = ((0, 1, 2, 3), (0, 1, 5, 4), (1, 2, 6, 5), (2, 3, 7, 6), (3, 0, 4, 7), (4, 5, 6, 7))


def nloc(order):
    return {1: 8, 2: 27}[order]


def dof_points(order):
    pts = [HEX_VERTS[v] for v in range(8)]
    if order == 2:
        pts += [0.5 * (HEX_VERTS[a] + HEX_VERTS[b]) for a, b in HEX_EDGES]
        pts += [HEX_VERTS[list(f)].mean(axis=0) for f in HEX_FACES]
        pts.append(np.zeros(3))
    return np.array(pts)


def quadrature(qdeg):
    m = (qdeg + 1) // 2 + 1
    x, w = np.polynomial.legendre.leggauss(m)
    pts, wts = [], []
    for i in range(m):
        for j in range(m):
            for l in range(m):
                pts.append((x[i], x[j], x[l]))
                wts.append(w[i] * w[j] * w[l])
    return np.array(pts), np.array(wts)


def _lagrange_1d(nodes, a, t):
    """value and derivative at t of the 1D Lagrange function of node a over `nodes`"""
    others = [b for b in nodes if b != a]
    den = np.prod([a - b for b in others])
    val = np.prod([t - b for b in others]) / den
    der = 0.0
    for k in range(len(others)):
        der += np.prod([t - b for i, b in enumerate(others) if i != k]) / den
    return val, der


def tabulate(order, pts):
    """phi (Q x n) and reference gradients (Q x n x 3) of the Q_order basis at pts"""
    nodes1 = [-1.0, 1.0] if order == 1 else [-1.0, 0.0, 1.0]
    P = dof_points(order)
    Q, n = len(pts), len(P)
    phi = np.zeros((Q, n))
    dphi = np.zeros((Q, n, 3))
    for q in range(Q):
        for i in range(n):
            v = [_lagrange_1d(nodes1, P[i, c], pts[q, c]) for c in range(3)]
            phi[q, i] = v[0][0] * v[1][0] * v[2][0]
            dphi[q, i] = (v[0][1] * v[1][0] * v[2][0], v[0][0] * v[1][1] * v[2][0], v[0][0] * v[1][0] * v[2][1])
    return phi, dphi


def dof_table(hexes, order):
    """first-encounter numbering: l2g (T x n) and the dof count"""
    hexes = np.asarray(hexes)
    n = nloc(order)
    l2g = np.zeros((len(hexes), n), dtype=np.int32)
    seen = {}
    nxt = 0

    def get(key):
        nonlocal nxt
        if key not in seen:
            seen[key] = nxt
            nxt += 1
        return seen[key]

    for e, h in enumerate(hexes):
        for v in range(8):
            l2g[e, v] = get(("v", int(h[v])))
        if order == 2:
            for j, (a, b) in enumerate(HEX_EDGES):
                l2g[e, 8 + j] = get(("e",) + tuple(sorted((int(h[a]), int(h[b])))))
            for f, fv in enumerate(HEX_FACES):
                l2g[e, 20 + f] = get(("f",) + tuple(sorted(int(h[k]) for k in fv)))
            l2g[e, 26] = get(("i", e))
    return nxt, l2g


def _maps(xyz, hexes, gdphi):
    """per element and point: K (T x Q x 3 x 3), det K, B = K^-T"""
    X = xyz[hexes]                                   # T x 8 x 3
    K = np.einsum("tgr,qgc->tqrc", X, gdphi)         # K[r][c] = sum_g X_g[r] dpsi_g/dxhat_c
    det = np.linalg.det(K)
    B = np.transpose(np.linalg.inv(K), (0, 1, 3, 2))
    return X, K, det, B


def element_matrices(order, xyz, hexes, kappa=None, kappa_const=1.0, mass=0.0, qdeg=None):
    qdeg = 2 * order if qdeg is None else qdeg
    pts, w = quadrature(qdeg)
    phi, dphi = tabulate(order, pts)
    _, gdphi = tabulate(1, pts)
    _, _, det, B = _maps(np.asarray(xyz, dtype=np.float64), np.asarray(hexes), gdphi)
    if np.any(~(np.abs(det) > 0)):
        raise ValueError("degenerate hexahedron")
    kap = np.full(len(hexes), kappa_const) if kappa is None else np.asarray(kappa, dtype=np.float64)
    G = np.einsum("tqia,qja->tqji", B, dphi)          # physical gradients T x Q x n x 3
    wJ = w[None, :] * np.abs(det)                    # T x Q
    Ke = np.einsum("tq,tqia,tqja->tij", wJ * kap[:, None], G, G)
    if mass:
        Ke += mass * np.einsum("tq,qi,qj->tij", wJ, phi, phi)
    return Ke


def assemble(order, xyz, hexes, l2g, ia, ja, kappa=None, kappa_const=1.0, mass=0.0, qdeg=None):
    """CSR values (pattern ia/ja) of kappa grad.grad + mass id.id, element order scatter-add"""
    Ke = element_matrices(order, xyz, hexes, kappa, kappa_const, mass, qdeg)
    val = np.zeros(len(ja))
    for e in range(len(hexes)):
        rows = l2g[e]
        for i, r in enumerate(rows):
            cols = ja[ia[r]:ia[r + 1]]
            pos = ia[r] + np.searchsorted(cols, rows)
            np.add.at(val, pos, Ke[e, i])
    return val


def rhs(order, xyz, hexes, l2g, N, fkind=0, c=0.0, qdeg=None):
    """load vector of f = 3 pi^2 sin(pi x) sin(pi y) sin(pi z) (fkind 0) or f = c (fkind 2)"""
    qdeg = 2 * order if qdeg is None else qdeg
    pts, w = quadrature(qdeg)
    phi, _ = tabulate(order, pts)
    gphi, gdphi = tabulate(1, pts)
    X, _, det, _ = _maps(np.asarray(xyz, dtype=np.float64), np.asarray(hexes), gdphi)
    if fkind == 0:
        p = np.einsum("tgr,qg->tqr", X, gphi)
        f = 3.0 * np.pi ** 2 * np.sin(np.pi * p[..., 0]) * np.sin(np.pi * p[..., 1]) * np.sin(np.pi * p[..., 2])
    else:
        f = np.full(det.shape, float(c))
    Fe = np.einsum("tq,qi->ti", w[None, :] * np.abs(det) * f, phi)
    F = np.zeros(N)
    np.add.at(F, l2g.reshape(-1), Fe.reshape(-1))
    return F


def boundary_mask(order, hexes, l2g, N):
    """dofs on faces that belong to one element"""
    hexes = np.asarray(hexes)
    count = {}
    for h in hexes:
        for fv in HEX_FACES:
            key = tuple(sorted(int(h[k]) for k in fv))
            count[key] = count.get(key, 0) + 1
    mask = np.zeros(N, dtype=np.uint8)
    for e, h in enumerate(hexes):
        for f, fv in enumerate(HEX_FACES):
            if count[tuple(sorted(int(h[k]) for k in fv))] != 1:
                continue
            local = list(fv)
            if order == 2:
                local += [8 + j for j, (a, b) in enumerate(HEX_EDGES) if a in fv and b in fv]
                local.append(20 + f)
            mask[l2g[e, local]] = 1
    return mask
