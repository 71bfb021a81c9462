// EnSight Gold export of device results (the reference's default exporter
// format, feelpp/feel/feelfilters/exporterensightgold.hpp): the mesh as one
// part of 4-node tetrahedra (or 8-node hexahedra) and nodal scalar fields, in "C Binary" files
// written on the host after one copy of each field from the device.
//
// Files for prefix P: P.case (text), P.geo, and P.<name>.scl per field. The
// geometry carries the vertex coordinates and the element connectivity (1-based,
// insertion order); a field on a Pch<k> space is written at the vertices (the
// vertex dofs), as the reference does for its P1 visualisation of Pk fields.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fgpu_core.h"

namespace {

void put80(FILE* f, const char* s) {
    char buf[80];
    std::memset(buf, ' ', sizeof(buf));
    const size_t n = std::min<size_t>(std::strlen(s), 80);
    std::memcpy(buf, s, n);
    if (n < 80) buf[n] = '\0';
    std::fwrite(buf, 1, 80, f);
}

void put_i32(FILE* f, int32_t v) { std::fwrite(&v, sizeof(v), 1, f); }

bool valid_name(const char* s) {
    if (!s || !*s || std::strlen(s) > 19) return false;
    for (const char* p = s; *p; ++p)
        if (!((*p >= 'a' && *p <= 'z') || (*p >= 'A' && *p <= 'Z') || (*p >= '0' && *p <= '9') || *p == '_')) return false;
    return true;
}

}  // namespace

extern "C" int fgpu_export_ensight(const fgpu_space* V, const char* prefix, int nfields, const char* const* names,
                                   const fgpu_vector* const* fields) {
    if (!V || !prefix || nfields < 0 || (nfields > 0 && (!names || !fields))) return FGPU_ERR_INVALID;
    fgpu_ctx* ctx = V->ctx;
    if (V->ncomp != 1) { ctx->err = "export: scalar spaces only"; return FGPU_ERR_INVALID; }
    for (int k = 0; k < nfields; ++k) {
        if (!valid_name(names[k])) { ctx->err = "export: field names are 1-19 letters, digits or '_'"; return FGPU_ERR_INVALID; }
        if (!fields[k] || fields[k]->n != V->ndof) { ctx->err = "export: field size differs from the space"; return FGPU_ERR_INVALID; }
    }
    fgpu_mesh* M = V->mesh;
    const int64_t nv = M->nv, nt = M->nt;
    const int n = V->n;
    if (nv >= INT32_MAX || nt >= INT32_MAX) { ctx->err = "export: mesh too large for 32-bit EnSight ids"; return FGPU_ERR_INVALID; }
    FGPU_CUDA_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
    if (M->h_xyz_stale) {
        FGPU_CUDA_CHECK(ctx, cudaMemcpy(M->h_xyz.data(), M->d_xyz, M->h_xyz.size() * sizeof(double), cudaMemcpyDeviceToHost));
        M->h_xyz_stale = false;
    }
    // vertex -> its dof (local vertex dofs are the first four of every element)
    std::vector<int32_t> l2n((size_t)nt * n);
    FGPU_CUDA_CHECK(ctx, cudaMemcpy(l2n.data(), V->d_l2n, l2n.size() * sizeof(int32_t), cudaMemcpyDeviceToHost));
    std::vector<int64_t> vdof(nv, -1);
    for (int64_t e = 0; e < nt; ++e)
        for (int v = 0; v < M->cv; ++v) vdof[M->h_tets[(size_t)M->cv * e + v]] = l2n[(size_t)e * n + v];
    const std::string base(prefix);
    std::string stem = base;
    const size_t slash = stem.find_last_of('/');
    if (slash != std::string::npos) stem = stem.substr(slash + 1);
    // geometry
    {
        FILE* f = std::fopen((base + ".geo").c_str(), "wb");
        if (!f) { ctx->err = "export: cannot write " + base + ".geo"; return FGPU_ERR_INVALID; }
        put80(f, "C Binary");
        put80(f, "feelpp_gb300 export");
        put80(f, M->cv == 8 ? "hexahedral mesh" : "tetrahedral mesh");
        put80(f, "node id off");
        put80(f, "element id off");
        put80(f, "part");
        put_i32(f, 1);
        put80(f, "mesh");
        put80(f, "coordinates");
        put_i32(f, (int32_t)nv);
        std::vector<float> c(nv);
        for (int d = 0; d < 3; ++d) {
            for (int64_t i = 0; i < nv; ++i) c[i] = (float)M->h_xyz[3 * i + d];
            std::fwrite(c.data(), sizeof(float), nv, f);
        }
        // EnSight's hexa8 numbers the bottom face counter-clockwise, then the top face: the reference
        // hexahedron's vertex order
        put80(f, M->cv == 8 ? "hexa8" : "tetra4");
        put_i32(f, (int32_t)nt);
        std::vector<int32_t> conn((size_t)nt * M->cv);
        for (size_t k = 0; k < conn.size(); ++k) conn[k] = M->h_tets[k] + 1;
        std::fwrite(conn.data(), sizeof(int32_t), conn.size(), f);
        const bool ok = std::ferror(f) == 0;
        std::fclose(f);
        if (!ok) { ctx->err = "export: write error on " + base + ".geo"; return FGPU_ERR_INVALID; }
    }
    // fields
    std::vector<double> h;
    std::vector<float> vals(nv);
    for (int k = 0; k < nfields; ++k) {
        h.resize(V->ndof);
        FGPU_CUDA_CHECK(ctx, cudaMemcpy(h.data(), fields[k]->d, V->ndof * sizeof(double), cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < nv; ++i) vals[i] = vdof[i] >= 0 ? (float)h[vdof[i]] : 0.0f;
        const std::string fn = base + "." + names[k] + ".scl";
        FILE* f = std::fopen(fn.c_str(), "wb");
        if (!f) { ctx->err = "export: cannot write " + fn; return FGPU_ERR_INVALID; }
        put80(f, names[k]);
        put80(f, "part");
        put_i32(f, 1);
        put80(f, "coordinates");
        std::fwrite(vals.data(), sizeof(float), nv, f);
        const bool ok = std::ferror(f) == 0;
        std::fclose(f);
        if (!ok) { ctx->err = "export: write error on " + fn; return FGPU_ERR_INVALID; }
    }
    // case file
    FILE* f = std::fopen((base + ".case").c_str(), "w");
    if (!f) { ctx->err = "export: cannot write " + base + ".case"; return FGPU_ERR_INVALID; }
    std::fprintf(f, "FORMAT\ntype: ensight gold\n\nGEOMETRY\nmodel: %s.geo\n", stem.c_str());
    if (nfields > 0) {
        std::fprintf(f, "\nVARIABLE\n");
        for (int k = 0; k < nfields; ++k) std::fprintf(f, "scalar per node: %s %s.%s.scl\n", names[k], stem.c_str(), names[k]);
    }
    std::fclose(f);
    return FGPU_OK;
}
