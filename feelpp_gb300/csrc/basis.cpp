// Lagrange P1-P3 basis on the reference tetrahedron and the reference tensors
// of the affine forms, computed once on the host and kept resident on the device.
//
// Node set: Feel++'s Lagrange<k> on tetrahedra uses PointSetFekete ->
// PointSetWarpBlend (feelpp/feel/feelpoly/fekete.hpp:1251-1262). For k <= 2 the
// warp is inactive and the nodes are equispaced; for k = 3 only the edge points
// are warped (warpblend.hpp:92-115), and the 1D blend/warp composition moves each
// edge point to the Gauss-Lobatto-Legendre position of the 4-point rule
// (+-1/sqrt(5) on [-1,1]); the face points stay at the face centroids. Local
// ordering (equispaced.hpp:118-145): vertices 0..3, then the points of edges
// 0..5 (each oriented from its first to its second vertex), then faces 0..3.
//
// The basis itself is built independently of Feel++'s Dubiner route: monomials
// in xi = (x+1)/2, a Vandermonde solve in long double, and the polynomial
// gradients evaluated exactly. The Lagrange basis of a node set is unique, so
// both routes agree to rounding.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "fgpu_core.h"
#include "quad_tet.h"

namespace fgpu {

const int kEdgeVerts[6][2] = {{1, 2}, {2, 0}, {0, 1}, {0, 3}, {1, 3}, {2, 3}};
const int kFaceVerts[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
static const double kRefVerts[4][3] = {{-1, -1, -1}, {1, -1, -1}, {-1, 1, -1}, {-1, -1, 1}};

bool lagrange_nodes(int order, std::vector<double>& xyz) {
    if (order < 1 || order > 3) return false;
    xyz.clear();
    for (int v = 0; v < 4; ++v)
        for (int d = 0; d < 3; ++d) xyz.push_back(kRefVerts[v][d]);
    if (order == 1) return true;
    std::vector<long double> t;  // positions along an edge in [0,1]
    if (order == 2) {
        t = {0.5L};
    } else {
        long double g = 1.0L / std::sqrt(5.0L);  // interior GLL points of the 4-point rule
        t = {(1.0L - g) / 2.0L, (1.0L + g) / 2.0L};
    }
    for (int e = 0; e < 6; ++e) {
        const double* a = kRefVerts[kEdgeVerts[e][0]];
        const double* b = kRefVerts[kEdgeVerts[e][1]];
        for (long double s : t)
            for (int d = 0; d < 3; ++d) xyz.push_back((double)(a[d] + s * ((long double)b[d] - a[d])));
    }
    if (order == 3)
        for (int f = 0; f < 4; ++f)
            for (int d = 0; d < 3; ++d) {
                long double s = 0;
                for (int k = 0; k < 3; ++k) s += kRefVerts[kFaceVerts[f][k]][d];
                xyz.push_back((double)(s / 3.0L));
            }
    return true;
}

namespace {

typedef long double LD;

struct Mono {
    int a, b, c;
};

std::vector<Mono> monomials(int p) {
    std::vector<Mono> m;
    for (int s = 0; s <= p; ++s)
        for (int a = s; a >= 0; --a)
            for (int b = s - a; b >= 0; --b) m.push_back({a, b, s - a - b});
    return m;
}

LD ipow(LD x, int k) {
    LD r = 1;
    for (int i = 0; i < k; ++i) r *= x;
    return r;
}

// Solve A X = I (n x n) by Gaussian elimination with partial pivoting.
bool invert(std::vector<LD> A, int n, std::vector<LD>& X) {
    X.assign((size_t)n * n, 0);
    for (int i = 0; i < n; ++i) X[(size_t)i * n + i] = 1;
    for (int k = 0; k < n; ++k) {
        int p = k;
        for (int i = k + 1; i < n; ++i)
            if (std::fabs(A[(size_t)i * n + k]) > std::fabs(A[(size_t)p * n + k])) p = i;
        if (A[(size_t)p * n + k] == 0) return false;
        if (p != k)
            for (int j = 0; j < n; ++j) {
                std::swap(A[(size_t)k * n + j], A[(size_t)p * n + j]);
                std::swap(X[(size_t)k * n + j], X[(size_t)p * n + j]);
            }
        LD inv = 1 / A[(size_t)k * n + k];
        for (int i = 0; i < n; ++i) {
            if (i == k) continue;
            LD f = A[(size_t)i * n + k] * inv;
            if (f == 0) continue;
            for (int j = 0; j < n; ++j) {
                A[(size_t)i * n + j] -= f * A[(size_t)k * n + j];
                X[(size_t)i * n + j] -= f * X[(size_t)k * n + j];
            }
        }
    }
    for (int k = 0; k < n; ++k) {
        LD inv = 1 / A[(size_t)k * n + k];
        for (int j = 0; j < n; ++j) X[(size_t)k * n + j] *= inv;
    }
    return true;
}

}  // namespace

namespace {

// Gauss-Legendre rule with k points on [0, 1] (Newton on P_k from the
// Chebyshev-like initial guesses; long double).
void gauss_legendre01(int k, std::vector<LD>& x, std::vector<LD>& w) {
    x.resize(k);
    w.resize(k);
    const LD pi = 3.141592653589793238462643383279502884L;
    for (int i = 0; i < k; ++i) {
        LD t = std::cos(pi * (i + 0.75L) / (k + 0.5L));
        LD dp = 1;
        for (int it = 0; it < 100; ++it) {
            LD p0 = 1, p1 = t;
            for (int m = 2; m <= k; ++m) {
                const LD p2 = ((2 * m - 1) * t * p1 - (m - 1) * p0) / m;
                p0 = p1;
                p1 = p2;
            }
            dp = k * (t * p1 - p0) / (t * t - 1);
            const LD dt = p1 / dp;
            t -= dt;
            if (std::fabs(dt) < 1e-30L) break;
        }
        x[i] = (1 - t) / 2;
        w[i] = 1 / ((1 - t * t) * dp * dp);   // weight on [-1,1] is 2 / ((1 - t^2) P'^2); halved for [0,1]
    }
}

}  // namespace

// Face tables for boundary integrals (integrator.hpp MESH_FACES): for each
// reference face f (vertices kFaceVerts[f]), per unit face area,
//   Mf[f](i, j) = (1/|f|) int_f phi_i phi_j,   Lf[f](i) = (1/|f|) int_f phi_i,
// with a collapsed (Duffy) Gauss-Legendre rule of (p + 2)^2 points on the face
// triangle, exact for the degree-2p integrands. Only the dofs on the face are
// nonzero (fl[f]).
bool build_face_tables(int order, FaceTables& out, std::string& err) {
    if (order < 1 || order > 3) { err = "order must be 1, 2 or 3"; return false; }
    std::vector<double> nodes;
    lagrange_nodes(order, nodes);
    const int n = nloc_of(order);
    std::vector<Mono> mono = monomials(order);
    std::vector<LD> V((size_t)n * n), C;
    for (int k = 0; k < n; ++k) {
        LD x = ((LD)nodes[3 * k] + 1) / 2, y = ((LD)nodes[3 * k + 1] + 1) / 2, z = ((LD)nodes[3 * k + 2] + 1) / 2;
        for (int m = 0; m < n; ++m) V[(size_t)k * n + m] = ipow(x, mono[m].a) * ipow(y, mono[m].b) * ipow(z, mono[m].c);
    }
    if (!invert(V, n, C)) { err = "singular Vandermonde"; return false; }
    const int kq = order + 2;
    std::vector<LD> gx, gw;
    gauss_legendre01(kq, gx, gw);
    out.order = order;
    out.n = n;
    out.Mf.assign((size_t)4 * n * n, 0.0);
    out.Lf.assign((size_t)4 * n, 0.0);
    out.Gf.assign((size_t)4 * 3 * n * n, 0.0);
    out.Df.assign((size_t)4 * 3 * n, 0.0);
    for (int f = 0; f < 4; ++f) {
        LD A[3], E1[3], E2[3];
        for (int d = 0; d < 3; ++d) {
            A[d] = kRefVerts[kFaceVerts[f][0]][d];
            E1[d] = (LD)kRefVerts[kFaceVerts[f][1]][d] - A[d];
            E2[d] = (LD)kRefVerts[kFaceVerts[f][2]][d] - A[d];
        }
        std::vector<LD> M((size_t)n * n, 0), L(n, 0), G((size_t)3 * n * n, 0), D((size_t)3 * n, 0);
        LD wsum = 0;
        std::vector<LD> phi(n), dphi((size_t)3 * n);
        for (int a = 0; a < kq; ++a)
            for (int b = 0; b < kq; ++b) {
                // (s, t) = (u, v (1 - u)) on the unit triangle, jacobian (1 - u)
                const LD u = gx[a], v = gx[b];
                const LD s2 = u, t2 = v * (1 - u), w = gw[a] * gw[b] * (1 - u);
                LD P[3];
                for (int d = 0; d < 3; ++d) P[d] = A[d] + s2 * E1[d] + t2 * E2[d];
                const LD x = (P[0] + 1) / 2, y = (P[1] + 1) / 2, z = (P[2] + 1) / 2;
                for (int i = 0; i < n; ++i) {
                    LD vv = 0, gx = 0, gy = 0, gz = 0;
                    for (int m = 0; m < n; ++m) {
                        const LD c = C[(size_t)m * n + i];
                        if (c == 0) continue;
                        const int ea = mono[m].a, eb = mono[m].b, ec = mono[m].c;
                        vv += c * ipow(x, ea) * ipow(y, eb) * ipow(z, ec);
                        // d/dxhat = (1/2) d/dxi on the [-1,1] reference element
                        if (ea) gx += c * ea * ipow(x, ea - 1) * ipow(y, eb) * ipow(z, ec) / 2;
                        if (eb) gy += c * eb * ipow(x, ea) * ipow(y, eb - 1) * ipow(z, ec) / 2;
                        if (ec) gz += c * ec * ipow(x, ea) * ipow(y, eb) * ipow(z, ec - 1) / 2;
                    }
                    phi[i] = vv;
                    dphi[i] = gx;
                    dphi[(size_t)n + i] = gy;
                    dphi[(size_t)2 * n + i] = gz;
                }
                wsum += w;
                for (int i = 0; i < n; ++i) {
                    L[i] += w * phi[i];
                    for (int j = 0; j < n; ++j) M[(size_t)i * n + j] += w * phi[i] * phi[j];
                    for (int a = 0; a < 3; ++a) {
                        D[(size_t)a * n + i] += w * dphi[(size_t)a * n + i];
                        for (int j = 0; j < n; ++j) G[((size_t)a * n + i) * n + j] += w * phi[i] * dphi[(size_t)a * n + j];
                    }
                }
            }
        // the weights sum to the unit triangle's area 1/2: normalise to unit face area
        for (int i = 0; i < n; ++i) {
            LD li = L[i] / wsum;
            out.Lf[(size_t)f * n + i] = std::fabs(li) < 1e-15L ? 0.0 : (double)li;
            for (int j = 0; j < n; ++j) {
                LD mij = M[(size_t)i * n + j] / wsum;
                out.Mf[((size_t)f * n + i) * n + j] = std::fabs(mij) < 1e-15L ? 0.0 : (double)mij;
            }
            for (int a = 0; a < 3; ++a) {
                const LD di = D[(size_t)a * n + i] / wsum;
                out.Df[((size_t)f * 3 + a) * n + i] = std::fabs(di) < 1e-15L ? 0.0 : (double)di;
                for (int j = 0; j < n; ++j) {
                    const LD g = G[((size_t)a * n + i) * n + j] / wsum;
                    out.Gf[(((size_t)f * 3 + a) * n + i) * n + j] = std::fabs(g) < 1e-15L ? 0.0 : (double)g;
                }
            }
        }
    }
    return true;
}

bool build_ref_tables(int order, int qdeg, RefTables& out, std::string& err) {
    if (order < 1 || order > 3) { err = "order must be 1, 2 or 3"; return false; }
    if (qdeg < 1 || qdeg > kMaxTetRuleDegree) { err = "quadrature degree must be in [1, 8]"; return false; }
    std::vector<double> nodes;
    lagrange_nodes(order, nodes);
    const int n = nloc_of(order);
    std::vector<Mono> mono = monomials(order);
    if ((int)mono.size() != n) { err = "internal: monomial count"; return false; }
    // Vandermonde V[k][m] = mono_m(node_k) in xi = (x+1)/2
    std::vector<LD> V((size_t)n * n), C;
    for (int k = 0; k < n; ++k) {
        LD x = ((LD)nodes[3 * k] + 1) / 2, y = ((LD)nodes[3 * k + 1] + 1) / 2, z = ((LD)nodes[3 * k + 2] + 1) / 2;
        for (int m = 0; m < n; ++m) V[(size_t)k * n + m] = ipow(x, mono[m].a) * ipow(y, mono[m].b) * ipow(z, mono[m].c);
    }
    if (!invert(V, n, C)) { err = "singular Vandermonde"; return false; }
    // phi_i(x) = sum_m C[m][i] mono_m(x)
    const TetRule& R = tet_rules[qdeg];
    const int Q = R.npts;
    out.order = order; out.n = n; out.qdeg = qdeg; out.Q = Q;
    out.nodes = nodes;
    out.qx.resize((size_t)Q * 3); out.qw.resize(Q);
    out.phi.assign((size_t)Q * n, 0); out.dphi.assign((size_t)Q * n * 3, 0);
    std::vector<LD> phi((size_t)Q * n), dphi((size_t)Q * n * 3);
    for (int q = 0; q < Q; ++q) {
        out.qx[3 * q] = R.x[q]; out.qx[3 * q + 1] = R.y[q]; out.qx[3 * q + 2] = R.z[q]; out.qw[q] = R.w[q];
        LD x = ((LD)R.x[q] + 1) / 2, y = ((LD)R.y[q] + 1) / 2, z = ((LD)R.z[q] + 1) / 2;
        for (int i = 0; i < n; ++i) {
            LD v = 0, gx = 0, gy = 0, gz = 0;
            for (int m = 0; m < n; ++m) {
                LD c = C[(size_t)m * n + i];
                if (c == 0) continue;
                int a = mono[m].a, b = mono[m].b, cc = mono[m].c;
                v += c * ipow(x, a) * ipow(y, b) * ipow(z, cc);
                // d/dx = (1/2) d/dxi
                if (a) gx += c * a * ipow(x, a - 1) * ipow(y, b) * ipow(z, cc) / 2;
                if (b) gy += c * b * ipow(x, a) * ipow(y, b - 1) * ipow(z, cc) / 2;
                if (cc) gz += c * cc * ipow(x, a) * ipow(y, b) * ipow(z, cc - 1) / 2;
            }
            phi[(size_t)q * n + i] = v;
            dphi[((size_t)q * n + i) * 3 + 0] = gx;
            dphi[((size_t)q * n + i) * 3 + 1] = gy;
            dphi[((size_t)q * n + i) * 3 + 2] = gz;
        }
    }
    for (size_t k = 0; k < phi.size(); ++k) out.phi[k] = (double)phi[k];
    for (size_t k = 0; k < dphi.size(); ++k) out.dphi[k] = (double)dphi[k];
    // reference tensors with the same rule (Sum_q w_q ...), as the quadrature form
    // of the reference evaluates them (pointsetquadrature.hpp:403-416)
    out.S.assign((size_t)9 * n * n, 0);
    out.M.assign((size_t)n * n, 0);
    std::vector<LD> S((size_t)9 * n * n, 0), M((size_t)n * n, 0);
    for (int q = 0; q < Q; ++q) {
        LD w = R.w[q];
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                M[(size_t)i * n + j] += w * phi[(size_t)q * n + i] * phi[(size_t)q * n + j];
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b)
                        S[((size_t)(a * 3 + b) * n + i) * n + j] +=
                            w * dphi[((size_t)q * n + i) * 3 + a] * dphi[((size_t)q * n + j) * 3 + b];
            }
    }
    for (size_t k = 0; k < S.size(); ++k) out.S[k] = (double)S[k];
    // S_ba(j, i) and S_ab(i, j) are the same integral; make them the same number
    // (the long-double sums round their products in different orders), so that an
    // element matrix can be stored as blocks of its upper triangle
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            for (int i = 0; i < n; ++i)
                for (int j = 0; j < n; ++j) {
                    const bool upper = i < j || (i == j && a <= b);
                    if (!upper) out.S[((size_t)(a * 3 + b) * n + i) * n + j] = out.S[((size_t)(b * 3 + a) * n + j) * n + i];
                }
    for (size_t k = 0; k < M.size(); ++k) out.M[k] = (double)M[k];
    // T7: c0*S00 + c1*S11 + c2*S22 + c3*(S01+S10) + c4*(S02+S20) + c5*(S12+S21) + c6*M
    const int pairs[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
    out.T7.assign((size_t)7 * n * n, 0);
    for (int k = 0; k < 6; ++k) {
        int a = pairs[k][0], b = pairs[k][1];
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                LD v = S[((size_t)(a * 3 + b) * n + i) * n + j];
                if (a != b) v += S[((size_t)(b * 3 + a) * n + i) * n + j];
                out.T7[((size_t)k * n + i) * n + j] = (double)v;
            }
    }
    for (int i = 0; i < n * n; ++i) out.T7[(size_t)6 * n * n + i] = (double)M[i];
    // the tensors are symmetric; make them exactly so (the long-double sums of
    // (i, j) and (j, i) may round apart), so that K_e(i, j) and K_e(j, i) are
    // computed from the same numbers and an element matrix can be stored as its
    // upper triangle
    for (int k = 0; k < 7; ++k)
        for (int i = 0; i < n; ++i)
            for (int j = i + 1; j < n; ++j)
                out.T7[((size_t)k * n + j) * n + i] = out.T7[((size_t)k * n + i) * n + j];
    return true;
}

}  // namespace fgpu
