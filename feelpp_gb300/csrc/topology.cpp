// Host-side topology of a tetrahedral mesh for the device assembly:
// entity identification, Feel++-compatible dof numbering, node incidence,
// sparsity pattern, element colouring and boundary dofs.
//
// Dof numbering follows Feel++'s DofTable exactly (the pattern and the value
// layout of the assembled matrix depend on it):
//  * elements are visited in insertion order (doftable.hpp:2364-2455);
//  * inside an element, vertices 0..3, then edges 0..5, then faces 0..3
//    (doffromelement.hpp:505-530);
//  * an entity dof gets the next free number the first time its key is met
//    (doftable.hpp:1213-1250: map_gdof.try_emplace, next_free_dof += nComponents);
//  * an edge is identified by its two point ids; in an element whose local
//    edge j has id(e2p[j][0]) > id(e2p[j][1]) the edge is REVERSE-permuted
//    (mesh3d.hpp:750-782) and its l-th local dof is the edge slot
//    nDofPerEdge-1-l (doffromelement.hpp:282-333);
//  * a face is identified by its three point ids (one dof per face at P3).
// Entity identification here is bucketed by smallest vertex id instead of a
// hash map, which only changes the internal entity ids, not the dof numbers.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "fgpu_core.h"

namespace fgpu {

namespace {

// Unique ids of keyed entities (edges: 2 vertex ids, faces: 3) grouped by their
// smallest vertex. slot_ids[k] gets the entity id of slot k.
template <int K>
int64_t identify_entities(int64_t nv, int64_t nslots, const int32_t* keys /* nslots x K, sorted asc */,
                          std::vector<int32_t>& slot_ids) {
    std::vector<int64_t> ptr(nv + 1, 0);
    for (int64_t s = 0; s < nslots; ++s) ptr[keys[s * K] + 1]++;
    for (int64_t v = 0; v < nv; ++v) ptr[v + 1] += ptr[v];
    std::vector<int64_t> fill(ptr.begin(), ptr.end() - 1);
    std::vector<int64_t> bucket(nslots);
    for (int64_t s = 0; s < nslots; ++s) bucket[fill[keys[s * K]]++] = s;
    slot_ids.assign(nslots, -1);
    int64_t next = 0;
    std::vector<std::pair<int64_t, int64_t>> tmp;  // (packed rest-of-key, slot)
    for (int64_t v = 0; v < nv; ++v) {
        int64_t b = ptr[v], e = ptr[v + 1];
        if (b == e) continue;
        tmp.clear();
        for (int64_t k = b; k < e; ++k) {
            int64_t s = bucket[k];
            int64_t rest = K == 2 ? (int64_t)keys[s * K + 1] : ((int64_t)keys[s * K + 1] << 32) | (uint32_t)keys[s * K + 2];
            tmp.push_back({rest, s});
        }
        std::sort(tmp.begin(), tmp.end());
        for (size_t k = 0; k < tmp.size(); ++k) {
            if (k == 0 || tmp[k].first != tmp[k - 1].first) ++next;
            slot_ids[tmp[k].second] = (int32_t)(next - 1);
        }
    }
    return next;
}

void edge_keys(int64_t nt, const int32_t* tets, std::vector<int32_t>& keys) {
    keys.resize((size_t)nt * 6 * 2);
    for (int64_t e = 0; e < nt; ++e)
        for (int j = 0; j < 6; ++j) {
            int32_t a = tets[4 * e + kEdgeVerts[j][0]], b = tets[4 * e + kEdgeVerts[j][1]];
            keys[(e * 6 + j) * 2] = std::min(a, b);
            keys[(e * 6 + j) * 2 + 1] = std::max(a, b);
        }
}

void face_keys(int64_t nt, const int32_t* tets, std::vector<int32_t>& keys) {
    keys.resize((size_t)nt * 4 * 3);
    for (int64_t e = 0; e < nt; ++e)
        for (int f = 0; f < 4; ++f) {
            int32_t k[3] = {tets[4 * e + kFaceVerts[f][0]], tets[4 * e + kFaceVerts[f][1]], tets[4 * e + kFaceVerts[f][2]]};
            std::sort(k, k + 3);
            for (int d = 0; d < 3; ++d) keys[(e * 4 + f) * 3 + d] = k[d];
        }
}

template <typename F>
void parallel_for(int64_t n, int nthreads, F&& f) {
    if (nthreads <= 1 || n < 4096) {
        f(0, n);
        return;
    }
    std::vector<std::thread> th;
    int64_t chunk = (n + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; ++t) {
        int64_t b = t * chunk, e = std::min(n, b + chunk);
        if (b >= e) break;
        th.emplace_back([&f, b, e] { f(b, e); });
    }
    for (auto& x : th) x.join();
}

}  // namespace

bool build_topology(int64_t nv, int64_t nt, const int32_t* tets, int order, Topology& topo, std::string& err) {
    if (order < 1 || order > 3) { err = "order must be 1, 2 or 3"; return false; }
    for (int64_t k = 0; k < 4 * nt; ++k)
        if (tets[k] < 0 || tets[k] >= nv) { err = "tetrahedron vertex index out of range"; return false; }
    for (int64_t e = 0; e < nt; ++e) {
        const int32_t* t = tets + 4 * e;
        if (t[0] == t[1] || t[0] == t[2] || t[0] == t[3] || t[1] == t[2] || t[1] == t[3] || t[2] == t[3]) {
            err = "tetrahedron with a repeated vertex";
            return false;
        }
    }
    const int n = nloc_of(order), ndpe = dofs_per_edge(order), ndpf = dofs_per_face(order);
    topo.order = order;
    topo.n = n;
    topo.l2n.assign((size_t)nt * n, -1);
    topo.edge_rev.assign((size_t)nt * 6, 0);
    std::vector<int32_t> edge_of_slot, face_of_slot, keys;
    int64_t nedges = 0, nfaces = 0;
    if (ndpe > 0) {
        edge_keys(nt, tets, keys);
        nedges = identify_entities<2>(nv, nt * 6, keys.data(), edge_of_slot);
    }
    if (ndpf > 0) {
        face_keys(nt, tets, keys);
        nfaces = identify_entities<3>(nv, nt * 4, keys.data(), face_of_slot);
    }
    std::vector<int32_t> vnode(nv, -1), enode((size_t)nedges * std::max(ndpe, 1), -1),
        fnode((size_t)nfaces * std::max(ndpf, 1), -1);
    int64_t next = 0;
    for (int64_t e = 0; e < nt; ++e) {
        const int32_t* t = tets + 4 * e;
        int32_t* out = &topo.l2n[(size_t)e * n];
        int lc = 0;
        for (int i = 0; i < 4; ++i) {
            if (vnode[t[i]] < 0) vnode[t[i]] = (int32_t)next++;
            out[lc++] = vnode[t[i]];
        }
        for (int j = 0; j < 6; ++j) {
            bool rev = t[kEdgeVerts[j][0]] > t[kEdgeVerts[j][1]];
            topo.edge_rev[(size_t)e * 6 + j] = rev;
            if (ndpe == 0) continue;
            int64_t eid = edge_of_slot[(size_t)e * 6 + j];
            for (int l = 0; l < ndpe; ++l) {
                int s = rev ? ndpe - 1 - l : l;
                int32_t& slot = enode[(size_t)eid * ndpe + s];
                if (slot < 0) slot = (int32_t)next++;
                out[lc++] = slot;
            }
        }
        for (int f = 0; f < 4 && ndpf > 0; ++f) {
            int64_t fid = face_of_slot[(size_t)e * 4 + f];
            for (int l = 0; l < ndpf; ++l) {
                int32_t& slot = fnode[(size_t)fid * ndpf + l];
                if (slot < 0) slot = (int32_t)next++;
                out[lc++] = slot;
            }
        }
    }
    if (next >= (int64_t)1 << 31) { err = "too many dofs for 32-bit indices"; return false; }
    topo.nnodes = next;
    // incidence node -> (element << 5 | local), elements ascending
    topo.inc_ptr.assign(next + 1, 0);
    for (int64_t k = 0; k < nt * n; ++k) topo.inc_ptr[topo.l2n[k] + 1]++;
    for (int64_t r = 0; r < next; ++r) topo.inc_ptr[r + 1] += topo.inc_ptr[r];
    if (nt >= ((int64_t)1 << 26)) { err = "too many elements for the packed incidence"; return false; }
    topo.inc.resize((size_t)nt * n);
    std::vector<int64_t> fill(topo.inc_ptr.begin(), topo.inc_ptr.end() - 1);
    for (int64_t e = 0; e < nt; ++e)
        for (int l = 0; l < n; ++l) topo.inc[fill[topo.l2n[(size_t)e * n + l]]++] = (int32_t)((e << 5) | l);
    return true;
}

// Scalar node pattern: row r = sorted union of the nodes of the elements that
// contain r (Stencil::computeGraph, stencil.hpp:1500-1692, COUPLED pattern),
// plus the diagonal (graphcsr.cpp:634-660, always present here because r is a
// node of each of its elements); CSR close (graphcsr.cpp:990-1020).
bool build_node_pattern(const Topology& topo, int64_t nt, NodePattern& pat, int nthreads, std::string& err) {
    (void)nt;
    const int64_t N = topo.nnodes;
    const int n = topo.n;
    pat.nrows = N;
    std::vector<int32_t> cnt(N, 0);
    auto row_cols = [&](int64_t r, std::vector<int32_t>& tmp) {
        tmp.clear();
        for (int64_t k = topo.inc_ptr[r]; k < topo.inc_ptr[r + 1]; ++k) {
            int64_t e = topo.inc[k] >> 5;
            const int32_t* d = &topo.l2n[(size_t)e * n];
            tmp.insert(tmp.end(), d, d + n);
        }
        std::sort(tmp.begin(), tmp.end());
        tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
    };
    parallel_for(N, nthreads, [&](int64_t b, int64_t e) {
        std::vector<int32_t> tmp;
        for (int64_t r = b; r < e; ++r) {
            row_cols(r, tmp);
            cnt[r] = (int32_t)tmp.size();
        }
    });
    pat.ia.assign(N + 1, 0);
    int mx = 0;
    for (int64_t r = 0; r < N; ++r) {
        pat.ia[r + 1] = pat.ia[r] + cnt[r];
        mx = std::max(mx, cnt[r]);
    }
    pat.nnz = pat.ia[N];
    pat.max_row = mx;
    try {
        pat.ja.resize(pat.nnz);
    } catch (...) {
        err = "host allocation of the pattern failed";
        return false;
    }
    parallel_for(N, nthreads, [&](int64_t b, int64_t e) {
        std::vector<int32_t> tmp;
        for (int64_t r = b; r < e; ++r) {
            row_cols(r, tmp);
            std::memcpy(&pat.ja[pat.ia[r]], tmp.data(), tmp.size() * sizeof(int32_t));
        }
    });
    return true;
}

// Greedy colouring: elements sharing a vertex (hence a dof) get different
// colours. Returns the number of colours, or -1 if more than 64 are needed.
int colour_elements(int64_t nv, int64_t nt, const int32_t* tets, std::vector<int32_t>& perm,
                    std::vector<int64_t>& colour_ptr) {
    std::vector<uint64_t> used(nv, 0);
    std::vector<uint8_t> col(nt);
    int nc = 0;
    for (int64_t e = 0; e < nt; ++e) {
        uint64_t m = used[tets[4 * e]] | used[tets[4 * e + 1]] | used[tets[4 * e + 2]] | used[tets[4 * e + 3]];
        int c = 0;
        while (c < 64 && ((m >> c) & 1)) ++c;
        if (c == 64) return -1;
        col[e] = (uint8_t)c;
        nc = std::max(nc, c + 1);
        for (int i = 0; i < 4; ++i) used[tets[4 * e + i]] |= (1ull << c);
    }
    colour_ptr.assign(nc + 1, 0);
    for (int64_t e = 0; e < nt; ++e) colour_ptr[col[e] + 1]++;
    for (int c = 0; c < nc; ++c) colour_ptr[c + 1] += colour_ptr[c];
    std::vector<int64_t> fill(colour_ptr.begin(), colour_ptr.end() - 1);
    perm.resize(nt);
    for (int64_t e = 0; e < nt; ++e) perm[fill[col[e]]++] = (int32_t)e;
    return nc;
}

// Boundary faces (faces of exactly one element) as e * 4 + f, in element order;
// with xmax_on only those whose three vertices have x <= xmax (+1e-12). Then a
// greedy colouring in that order (faces sharing a vertex, or with whole_element
// faces whose elements share a vertex, get different colours): `faces` comes back sorted by colour (stable), colour_ptr delimits
// the colours. Returns the number of colours (-1: more than 64 needed).
int boundary_faces_coloured(int64_t nt, const int32_t* tets, const double* xyz, int xmax_on, double xmax, int whole_element,
                            std::vector<int32_t>& faces, std::vector<int64_t>& colour_ptr) {
    std::vector<int32_t> keys, face_of_slot;
    face_keys(nt, tets, keys);
    int64_t nv = 0;
    for (int64_t k = 0; k < 4 * nt; ++k) nv = std::max<int64_t>(nv, tets[k] + 1);
    const int64_t nf = identify_entities<3>(nv, nt * 4, keys.data(), face_of_slot);
    std::vector<uint8_t> cnt(nf, 0);
    for (int64_t s = 0; s < nt * 4; ++s)
        if (cnt[face_of_slot[s]] < 2) cnt[face_of_slot[s]]++;
    std::vector<int32_t> list;
    for (int64_t e = 0; e < nt; ++e)
        for (int f = 0; f < 4; ++f) {
            if (cnt[face_of_slot[e * 4 + f]] != 1) continue;
            if (xmax_on) {
                bool ok = true;
                for (int v = 0; v < 3; ++v) ok = ok && xyz[3 * (int64_t)tets[4 * e + kFaceVerts[f][v]]] <= xmax + 1e-12;
                if (!ok) continue;
            }
            list.push_back((int32_t)(e * 4 + f));
        }
    std::vector<uint64_t> used(nv, 0);
    std::vector<uint8_t> col(list.size());
    int nc = 0;
    for (size_t k = 0; k < list.size(); ++k) {
        const int64_t e = list[k] >> 2;
        const int f = list[k] & 3;
        // conflicts over the face's vertices, or over all four vertices of its element when the face
        // block couples every element dof (normal-derivative terms)
        int vs[4], nvs = 0;
        if (whole_element) {
            for (int v = 0; v < 4; ++v) vs[nvs++] = tets[4 * e + v];
        } else {
            for (int v = 0; v < 3; ++v) vs[nvs++] = tets[4 * e + kFaceVerts[f][v]];
        }
        uint64_t m = 0;
        for (int v = 0; v < nvs; ++v) m |= used[vs[v]];
        int c = 0;
        while (c < 64 && ((m >> c) & 1)) ++c;
        if (c == 64) return -1;
        col[k] = (uint8_t)c;
        nc = std::max(nc, c + 1);
        for (int v = 0; v < nvs; ++v) used[vs[v]] |= (1ull << c);
    }
    colour_ptr.assign(nc + 1, 0);
    for (size_t k = 0; k < list.size(); ++k) colour_ptr[col[k] + 1]++;
    for (int c = 0; c < nc; ++c) colour_ptr[c + 1] += colour_ptr[c];
    std::vector<int64_t> fill(colour_ptr.begin(), colour_ptr.end() - 1);
    faces.resize(list.size());
    for (size_t k = 0; k < list.size(); ++k) faces[fill[col[k]]++] = list[k];
    return nc;
}

bool boundary_nodes(int64_t nt, const int32_t* tets, const double* xyz, const Topology& topo, int xmax_on,
                    double xmax, std::vector<int32_t>& nodes) {
    std::vector<int32_t> keys, face_of_slot;
    face_keys(nt, tets, keys);
    int64_t nv = 0;
    for (int64_t k = 0; k < 4 * nt; ++k) nv = std::max<int64_t>(nv, tets[k] + 1);
    int64_t nf = identify_entities<3>(nv, nt * 4, keys.data(), face_of_slot);
    std::vector<uint8_t> cnt(nf, 0);
    for (int64_t s = 0; s < nt * 4; ++s)
        if (cnt[face_of_slot[s]] < 2) cnt[face_of_slot[s]]++;
    const int n = topo.n, ndpe = dofs_per_edge(topo.order), ndpf = dofs_per_face(topo.order);
    // local dofs carried by each local face
    std::vector<int> fl[4];
    for (int f = 0; f < 4; ++f) {
        for (int v = 0; v < 3; ++v) fl[f].push_back(kFaceVerts[f][v]);
        for (int j = 0; j < 6; ++j) {
            int a = kEdgeVerts[j][0], b = kEdgeVerts[j][1];
            bool ina = false, inb = false;
            for (int v = 0; v < 3; ++v) {
                ina |= kFaceVerts[f][v] == a;
                inb |= kFaceVerts[f][v] == b;
            }
            if (ina && inb)
                for (int l = 0; l < ndpe; ++l) fl[f].push_back(4 + j * ndpe + l);
        }
        for (int l = 0; l < ndpf; ++l) fl[f].push_back(4 + 6 * ndpe + f * ndpf + l);
    }
    std::vector<uint8_t> mark(topo.nnodes, 0);
    for (int64_t e = 0; e < nt; ++e)
        for (int f = 0; f < 4; ++f) {
            if (cnt[face_of_slot[e * 4 + f]] != 1) continue;
            if (xmax_on) {
                bool ok = true;
                for (int v = 0; v < 3; ++v) ok = ok && xyz[3 * (int64_t)tets[4 * e + kFaceVerts[f][v]]] <= xmax + 1e-12;
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
