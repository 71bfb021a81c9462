// Hexahedral meshes (Mesh<Hypercube<3,1>>): Q1 and Q2 Lagrange spaces, host set-up.
//
// Reference element [-1,1]^3 with the vertex order of feelmesh/refhypercube.hpp:148-183
// (0 (-1,-1,-1), 1 (1,-1,-1), 2 (1,1,-1), 3 (-1,1,-1), then the same at z = +1), edges and
// faces as in feelmesh/hypercubeordering.hpp (hexa::__e2p_order1, __f2p_order1; Q2 points
// __e2p_order2 / __f2p_order2: edge j's point is local dof 8 + j, face f's is 20 + f, the
// centre 26). Dofs are numbered by first encounter over (element, local dof), as for
// simplices (doftable.hpp:2364-2455): vertices, then edges, faces and the interior; Q1 and
// Q2 carry at most one dof per edge and face, so no orientation enters.
//
// Quadrature: tensor Gauss-Legendre rule with m = (o + 1) / 2 + 1 points per direction for
// degree o (feelpoly/gausshypercube.cpp: gaussdegree, the points ordered x slowest, z fastest,
// weights w_i w_j w_l). The 1D rule is computed by Newton iteration on the Legendre polynomial
// (roots to machine precision; the reference computes the same rule through gaussjacobi).
#include <algorithm>
#include <cmath>
#include <numeric>
#include <string>
#include <vector>

#include "fgpu_core.h"

namespace fgpu {

const int kHexEdgeVerts[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {1, 5}, {5, 4}, {4, 0}, {2, 6}, {6, 5}, {3, 7}, {7, 6}, {4, 7}};
const int kHexFaceVerts[6][4] = {{0, 1, 2, 3}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}, {4, 5, 6, 7}};
static const double kHexRefVerts[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                          {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};

int hex_nloc(int order) { return order == 1 ? 8 : order == 2 ? 27 : 0; }

namespace {

// ids of keyed entities: slots with equal sorted keys (K ints) share an id; ids follow the
// sorted key order (only identity matters: the dof numbering is by first encounter)
int64_t identify_keys(int64_t nslots, int K, const std::vector<int32_t>& keys, std::vector<int32_t>& ids) {
    std::vector<int64_t> ord(nslots);
    std::iota(ord.begin(), ord.end(), 0);
    auto less = [&](int64_t a, int64_t b) {
        for (int k = 0; k < K; ++k) {
            const int32_t x = keys[a * K + k], y = keys[b * K + k];
            if (x != y) return x < y;
        }
        return a < b;
    };
    std::sort(ord.begin(), ord.end(), less);
    ids.assign(nslots, -1);
    int64_t next = 0;
    for (int64_t k = 0; k < nslots; ++k) {
        bool same = k > 0;
        for (int c = 0; c < K && same; ++c) same = keys[ord[k] * K + c] == keys[ord[k - 1] * K + c];
        if (!same) ++next;
        ids[ord[k]] = (int32_t)(next - 1);
    }
    return next;
}

void hex_entity_ids(int64_t nh, const int32_t* hexes, std::vector<int32_t>& edge_of_slot, std::vector<int32_t>& face_of_slot,
                    int64_t* nedges, int64_t* nfaces) {
    std::vector<int32_t> keys((size_t)nh * 12 * 2);
    for (int64_t e = 0; e < nh; ++e)
        for (int j = 0; j < 12; ++j) {
            int32_t a = hexes[8 * e + kHexEdgeVerts[j][0]], b = hexes[8 * e + kHexEdgeVerts[j][1]];
            keys[(e * 12 + j) * 2] = std::min(a, b);
            keys[(e * 12 + j) * 2 + 1] = std::max(a, b);
        }
    *nedges = identify_keys(nh * 12, 2, keys, edge_of_slot);
    keys.assign((size_t)nh * 6 * 4, 0);
    for (int64_t e = 0; e < nh; ++e)
        for (int f = 0; f < 6; ++f) {
            int32_t v[4];
            for (int k = 0; k < 4; ++k) v[k] = hexes[8 * e + kHexFaceVerts[f][k]];
            std::sort(v, v + 4);
            for (int k = 0; k < 4; ++k) keys[(e * 6 + f) * 4 + k] = v[k];
        }
    *nfaces = identify_keys(nh * 6, 4, keys, face_of_slot);
}

// 1D Gauss-Legendre rule on [-1, 1], m points ascending
void gauss_legendre(int m, std::vector<double>& x, std::vector<double>& w) {
    x.assign(m, 0.0);
    w.assign(m, 0.0);
    const double pi = 3.14159265358979323846;
    for (int i = 0; i < m; ++i) {
        double t = -std::cos(pi * (i + 0.75) / (m + 0.5));   // initial guess, ascending
        double dp = 1.0;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = t;
            for (int k = 2; k <= m; ++k) {
                const double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            const double pm = m == 0 ? 1.0 : p1, pm1 = m == 1 ? 1.0 : p0;
            dp = m * (t * pm - pm1) / (t * t - 1.0);
            const double dt = pm / dp;
            t -= dt;
            if (std::fabs(dt) < 1e-17) break;
        }
        double p0 = 1.0, p1 = t;
        for (int k = 2; k <= m; ++k) {
            const double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
            p0 = p1;
            p1 = p2;
        }
        dp = m * (t * p1 - p0) / (t * t - 1.0);
        x[i] = t;
        w[i] = 2.0 / ((1.0 - t * t) * dp * dp);
    }
}

// 1D Lagrange functions on the nodes {-1, 1} (k = 1) or {-1, 0, 1} (k = 2); a in {-1, 0, 1}
double lag1d(int k, int a, double t) {
    if (k == 1) return 0.5 * (1.0 + a * t);
    if (a == -1) return 0.5 * t * (t - 1.0);
    if (a == 1) return 0.5 * t * (t + 1.0);
    return (1.0 - t) * (1.0 + t);
}
double dlag1d(int k, int a, double t) {
    if (k == 1) return 0.5 * a;
    if (a == -1) return t - 0.5;
    if (a == 1) return t + 0.5;
    return -2.0 * t;
}

}  // namespace

// reference points of the local dofs (n x 3)
void hex_dof_points(int order, std::vector<double>& pts) {
    pts.clear();
    for (int v = 0; v < 8; ++v) pts.insert(pts.end(), kHexRefVerts[v], kHexRefVerts[v] + 3);
    if (order < 2) return;
    for (int j = 0; j < 12; ++j)
        for (int c = 0; c < 3; ++c) pts.push_back(0.5 * (kHexRefVerts[kHexEdgeVerts[j][0]][c] + kHexRefVerts[kHexEdgeVerts[j][1]][c]));
    for (int f = 0; f < 6; ++f)
        for (int c = 0; c < 3; ++c) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += kHexRefVerts[kHexFaceVerts[f][k]][c];
            pts.push_back(0.25 * s);
        }
    pts.insert(pts.end(), {0.0, 0.0, 0.0});
}

bool build_hex_ref_tables(int order, int qdeg, RefTables& R, std::string& err) {
    const int n = hex_nloc(order);
    if (!n) { err = "hexahedra: Q1 and Q2 spaces only"; return false; }
    if (qdeg < 1) qdeg = 2 * order;
    const int m = (qdeg + 1) / 2 + 1;
    R.order = order;
    R.n = n;
    R.qdeg = qdeg;
    R.Q = m * m * m;
    std::vector<double> gx, gw;
    gauss_legendre(m, gx, gw);
    R.qx.clear();
    R.qw.clear();
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j)
            for (int l = 0; l < m; ++l) {
                R.qx.insert(R.qx.end(), {gx[i], gx[j], gx[l]});
                R.qw.push_back(gw[i] * gw[j] * gw[l]);
            }
    hex_dof_points(order, R.nodes);
    R.phi.assign((size_t)R.Q * n, 0.0);
    R.dphi.assign((size_t)R.Q * n * 3, 0.0);
    for (int q = 0; q < R.Q; ++q) {
        const double* x = &R.qx[3 * q];
        for (int i = 0; i < n; ++i) {
            int a[3];
            for (int c = 0; c < 3; ++c) a[c] = (int)std::lround(R.nodes[3 * i + c]);
            const double L[3] = {lag1d(order, a[0], x[0]), lag1d(order, a[1], x[1]), lag1d(order, a[2], x[2])};
            const double D[3] = {dlag1d(order, a[0], x[0]), dlag1d(order, a[1], x[1]), dlag1d(order, a[2], x[2])};
            R.phi[(size_t)q * n + i] = L[0] * L[1] * L[2];
            R.dphi[((size_t)q * n + i) * 3 + 0] = D[0] * L[1] * L[2];
            R.dphi[((size_t)q * n + i) * 3 + 1] = L[0] * D[1] * L[2];
            R.dphi[((size_t)q * n + i) * 3 + 2] = L[0] * L[1] * D[2];
        }
    }
    R.S.clear();
    R.M.clear();
    R.T7.clear();
    return true;
}

bool build_hex_topology(int64_t nv, int64_t nh, const int32_t* hexes, int order, Topology& topo, std::string& err) {
    const int n = hex_nloc(order);
    if (!n) { err = "hexahedra: Q1 and Q2 spaces only"; return false; }
    if (nh >= ((int64_t)1 << 26)) { err = "too many elements for the packed incidence"; return false; }
    topo.order = order;
    topo.n = n;
    topo.l2n.assign((size_t)nh * n, -1);
    topo.edge_rev.clear();
    std::vector<int32_t> vnode(nv, -1), enode, fnode, edge_of_slot, face_of_slot;
    int64_t nedges = 0, nfaces = 0;
    if (order == 2) {
        hex_entity_ids(nh, hexes, edge_of_slot, face_of_slot, &nedges, &nfaces);
        enode.assign(nedges, -1);
        fnode.assign(nfaces, -1);
    }
    int64_t next = 0;
    for (int64_t e = 0; e < nh; ++e) {
        int32_t* out = &topo.l2n[(size_t)e * n];
        for (int v = 0; v < 8; ++v) {
            int32_t& s = vnode[hexes[8 * e + v]];
            if (s < 0) s = (int32_t)next++;
            out[v] = s;
        }
        if (order < 2) continue;
        for (int j = 0; j < 12; ++j) {
            int32_t& s = enode[edge_of_slot[(size_t)e * 12 + j]];
            if (s < 0) s = (int32_t)next++;
            out[8 + j] = s;
        }
        for (int f = 0; f < 6; ++f) {
            int32_t& s = fnode[face_of_slot[(size_t)e * 6 + f]];
            if (s < 0) s = (int32_t)next++;
            out[20 + f] = s;
        }
        out[26] = (int32_t)next++;
    }
    if (next >= (int64_t)1 << 31) { err = "too many dofs for 32-bit indices"; return false; }
    topo.nnodes = next;
    topo.inc_ptr.assign(next + 1, 0);
    for (int64_t k = 0; k < nh * n; ++k) topo.inc_ptr[topo.l2n[k] + 1]++;
    for (int64_t r = 0; r < next; ++r) topo.inc_ptr[r + 1] += topo.inc_ptr[r];
    topo.inc.resize((size_t)nh * n);
    std::vector<int64_t> fill(topo.inc_ptr.begin(), topo.inc_ptr.end() - 1);
    for (int64_t e = 0; e < nh; ++e)
        for (int l = 0; l < n; ++l) topo.inc[fill[topo.l2n[(size_t)e * n + l]]++] = (int32_t)((e << 5) | l);
    return true;
}

// dofs on boundary faces (faces of one element), optionally only faces with every vertex at x <= xmax
bool hex_boundary_nodes(int64_t nh, const int32_t* hexes, const double* xyz, const Topology& topo, int xmax_on, double xmax,
                        std::vector<int32_t>& nodes) {
    std::vector<int32_t> edge_of_slot, face_of_slot;
    int64_t nedges = 0, nfaces = 0;
    hex_entity_ids(nh, hexes, edge_of_slot, face_of_slot, &nedges, &nfaces);
    std::vector<uint8_t> cnt(nfaces, 0);
    for (int64_t s = 0; s < nh * 6; ++s)
        if (cnt[face_of_slot[s]] < 2) cnt[face_of_slot[s]]++;
    const int n = topo.n;
    std::vector<int> fl[6];
    for (int f = 0; f < 6; ++f) {
        for (int k = 0; k < 4; ++k) fl[f].push_back(kHexFaceVerts[f][k]);
        if (topo.order < 2) continue;
        for (int j = 0; j < 12; ++j) {
            bool ina = false, inb = false;
            for (int k = 0; k < 4; ++k) {
                ina |= kHexFaceVerts[f][k] == kHexEdgeVerts[j][0];
                inb |= kHexFaceVerts[f][k] == kHexEdgeVerts[j][1];
            }
            if (ina && inb) fl[f].push_back(8 + j);
        }
        fl[f].push_back(20 + f);
    }
    std::vector<uint8_t> mark(topo.nnodes, 0);
    for (int64_t e = 0; e < nh; ++e)
        for (int f = 0; f < 6; ++f) {
            if (cnt[face_of_slot[e * 6 + f]] != 1) continue;
            if (xmax_on) {
                bool ok = true;
                for (int k = 0; k < 4; ++k) ok = ok && xyz[3 * (int64_t)hexes[8 * e + kHexFaceVerts[f][k]]] <= xmax + 1e-12;
                if (!ok) continue;
            }
            for (int li : fl[f]) mark[topo.l2n[(size_t)e * n + li]] = 1;
        }
    nodes.clear();
    for (int64_t r = 0; r < topo.nnodes; ++r)
        if (mark[r]) nodes.push_back((int32_t)r);
    return true;
}

}  // namespace fgpu
