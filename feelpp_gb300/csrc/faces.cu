// Boundary-face integrals on affine tetrahedra and scalar Lagrange spaces,
// feelpp/feel/feelvf/integrator.hpp MESH_FACES (:786-795):
//   form2 += integrate(faces, alpha*idt(u)*id(v))                      (Robin)
//   form2 += integrate(faces, -inner(k*gradt(u)*N(), id(v)) - inner(k*grad(v)*N(), idt(u))
//                             + gamma*k*idt(u)*id(v)/hFace())          (Nitsche weak Dirichlet,
//                                      feelpp/feel/feelpde/cg_laplacian.hpp:70-71)
//   form1 += integrate(faces, g*id(v)), and -inner(k*grad(v)*N(), g) + gamma*k*g*id(v)/hFace()
// with N() the unit outward normal and hFace() the longest edge of the face
// (feelpp/feel/feelmesh/geond.hpp:737-757).
//
// On an affine face the restriction of the element basis is fixed by the local
// face: int_f phi_i phi_j = |f| Mf(i, j), int_f phi_i (grad phi_j . n) =
// |f| sum_a w_a Gf(a, i, j) with w = B^T n (B = K^-T), per-unit-area tables
// computed once (basis.cpp build_face_tables). The faces of a range are found
// and greedily coloured on the host once per space, range and colouring kind
// (faces that share a vertex get different colours; with normal-derivative
// terms, which couple every dof of the element, faces whose elements share a
// vertex); one launch per colour scatters the face blocks into the CSR (or the
// load vector) without two threads ever writing one entry, so the result is
// deterministic without atomics: every entry gets its face contributions in
// colour order.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "fgpu_core.h"

namespace fgpu {

namespace {

struct FaceTablesDev {
    int n = 0, nfl = 0;
    double* d_Mf = nullptr;   // 4 n n
    double* d_Lf = nullptr;   // 4 n
    double* d_Gf = nullptr;   // 4 3 n n
    double* d_Df = nullptr;   // 4 3 n
    int* d_fl = nullptr;      // 4 nfl: local dofs on each face
    uint8_t* d_on = nullptr;  // 4 n: 1 when the local dof lies on the face
};

std::mutex g_face_mutex;
std::map<std::pair<int, int>, FaceTablesDev*> g_face_tabs;

// local dofs carried by each local face: its 3 vertices, the dofs of its 3 edges, its own dofs
std::vector<int> face_dofs(int order, int f) {
    const int ndpe = dofs_per_edge(order), ndpf = dofs_per_face(order);
    std::vector<int> out;
    for (int v = 0; v < 3; ++v) out.push_back(kFaceVerts[f][v]);
    for (int j = 0; j < 6; ++j) {
        const int a = kEdgeVerts[j][0], b = kEdgeVerts[j][1];
        bool ina = false, inb = false;
        for (int v = 0; v < 3; ++v) {
            ina |= kFaceVerts[f][v] == a;
            inb |= kFaceVerts[f][v] == b;
        }
        if (ina && inb)
            for (int l = 0; l < ndpe; ++l) out.push_back(4 + j * ndpe + l);
    }
    for (int l = 0; l < ndpf; ++l) out.push_back(4 + 6 * ndpe + f * ndpf + l);
    return out;
}

FaceTablesDev* get_face_tables(fgpu_ctx* ctx, int order) {
    std::lock_guard<std::mutex> lock(g_face_mutex);
    auto key = std::make_pair(ctx->device, order);
    auto it = g_face_tabs.find(key);
    if (it != g_face_tabs.end()) return it->second;
    FaceTables T;
    std::string err;
    if (!build_face_tables(order, T, err)) { ctx->err = err; return nullptr; }
    FaceTablesDev* D = new FaceTablesDev();
    D->n = T.n;
    std::vector<int> fl;
    std::vector<uint8_t> on((size_t)4 * T.n, 0);
    for (int f = 0; f < 4; ++f) {
        std::vector<int> d = face_dofs(order, f);
        D->nfl = (int)d.size();
        fl.insert(fl.end(), d.begin(), d.end());
        for (int i : d) on[(size_t)f * T.n + i] = 1;
    }
    auto up = [](void** dst, const void* src, size_t bytes) {
        cudaError_t e = cudaMalloc(dst, bytes);
        if (e == cudaSuccess) e = cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
        return e;
    };
    cudaError_t e = up((void**)&D->d_Mf, T.Mf.data(), T.Mf.size() * sizeof(double));
    if (e == cudaSuccess) e = up((void**)&D->d_Lf, T.Lf.data(), T.Lf.size() * sizeof(double));
    if (e == cudaSuccess) e = up((void**)&D->d_Gf, T.Gf.data(), T.Gf.size() * sizeof(double));
    if (e == cudaSuccess) e = up((void**)&D->d_Df, T.Df.data(), T.Df.size() * sizeof(double));
    if (e == cudaSuccess) e = up((void**)&D->d_fl, fl.data(), fl.size() * sizeof(int));
    if (e == cudaSuccess) e = up((void**)&D->d_on, on.data(), on.size());
    if (e != cudaSuccess) {
        cudaGetLastError();
        ctx->err = std::string("face tables: ") + cudaGetErrorString(e);
        delete D;
        return nullptr;
    }
    g_face_tabs[key] = D;
    return D;
}

// per face (one thread each): |f|, hFace = longest face edge, and w = B^T n
// (B = K^-T of the element, n the unit outward normal), so that
// grad phi . n = sum_a w_a dphi/dxhat_a on the face. geo = 5 doubles per face.
__global__ void face_geom_kernel(int64_t nf, const int32_t* __restrict__ faces, const double* __restrict__ xyz,
                                 const int32_t* __restrict__ tets, double* __restrict__ geo) {
    const int fv[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nf; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = faces[k] >> 2;
        const int f = faces[k] & 3;
        double X[4][3];
        for (int v = 0; v < 4; ++v)
            for (int d = 0; d < 3; ++d) X[v][d] = xyz[3 * (int64_t)tets[4 * e + v] + d];
        const double* P0 = X[fv[f][0]];
        const double* P1 = X[fv[f][1]];
        const double* P2 = X[fv[f][2]];
        const double u[3] = {P1[0] - P0[0], P1[1] - P0[1], P1[2] - P0[2]};
        const double v[3] = {P2[0] - P0[0], P2[1] - P0[1], P2[2] - P0[2]};
        const double t[3] = {P2[0] - P1[0], P2[1] - P1[1], P2[2] - P1[2]};
        double c[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
        const double cn = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        const double side = c[0] * (X[f][0] - P0[0]) + c[1] * (X[f][1] - P0[1]) + c[2] * (X[f][2] - P0[2]);
        const double sg = side > 0 ? -1.0 / cn : 1.0 / cn;    // outward: away from the opposite vertex
        const double n[3] = {c[0] * sg, c[1] * sg, c[2] * sg};
        const double hu = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        const double hv = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        const double ht = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
        // K(:, a) = (X_{a+1} - X_0) / 2 on the [-1,1] reference tetrahedron; B(i, j) = cof(i, j) / det
        double K[3][3];
        for (int r = 0; r < 3; ++r)
            for (int a = 0; a < 3; ++a) K[r][a] = 0.5 * (X[a + 1][r] - X[0][r]);
        double cof[3][3];
        cof[0][0] = K[1][1] * K[2][2] - K[1][2] * K[2][1];
        cof[0][1] = K[1][2] * K[2][0] - K[1][0] * K[2][2];
        cof[0][2] = K[1][0] * K[2][1] - K[1][1] * K[2][0];
        cof[1][0] = K[0][2] * K[2][1] - K[0][1] * K[2][2];
        cof[1][1] = K[0][0] * K[2][2] - K[0][2] * K[2][0];
        cof[1][2] = K[0][1] * K[2][0] - K[0][0] * K[2][1];
        cof[2][0] = K[0][1] * K[1][2] - K[0][2] * K[1][1];
        cof[2][1] = K[0][2] * K[1][0] - K[0][0] * K[1][2];
        cof[2][2] = K[0][0] * K[1][1] - K[0][1] * K[1][0];
        const double det = K[0][0] * cof[0][0] + K[0][1] * cof[0][1] + K[0][2] * cof[0][2];
        double* g = geo + 5 * k;
        g[0] = 0.5 * cn;
        g[1] = fmax(hu, fmax(hv, ht));
        for (int a = 0; a < 3; ++a) g[2 + a] = (cof[0][a] * n[0] + cof[1][a] * n[1] + cof[2][a] * n[2]) / det;
    }
}

struct FaceCoefs {
    double mass = 0;      // alpha:   int_f alpha u v
    double mass_h = 0;    // beta:    int_f beta u v / hFace
    double dn_trial = 0;  // int_f c (grad u . n) v
    double dn_test = 0;   // int_f c (grad v . n) u
    bool full() const { return dn_trial != 0.0 || dn_test != 0.0; }
};

// one colour: thread per (face, i, j); over the face's own dofs, or over every
// element dof pair with one index on the face when normal-derivative terms are on
template <typename VT>
__global__ void face_matrix_kernel(int64_t f0, int64_t f1, const int32_t* __restrict__ faces, const double* __restrict__ geo,
                                   const int32_t* __restrict__ l2n, int n, const int64_t* __restrict__ ia,
                                   const uint8_t* __restrict__ pos, const double* __restrict__ Mf, const double* __restrict__ Gf,
                                   const uint8_t* __restrict__ on, const int* __restrict__ fl, int nfl, FaceCoefs c, int full,
                                   VT* __restrict__ val) {
    const int per = full ? n * n : nfl * nfl;
    const int64_t total = (f1 - f0) * per;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = f0 + t / per;
        const int ab = (int)(t % per);
        const int64_t e = faces[k] >> 2;
        const int f = faces[k] & 3;
        int li, lj;
        if (full) {
            li = ab / n;
            lj = ab - li * n;
            if (!on[f * n + li] && !on[f * n + lj]) continue;
        } else {
            li = fl[f * nfl + ab / nfl];
            lj = fl[f * nfl + ab % nfl];
        }
        const double* g = geo + 5 * k;
        double v = (c.mass + c.mass_h / g[1]) * Mf[((int64_t)f * n + li) * n + lj];
        if (full) {
            double dt = 0.0, ds = 0.0;
            for (int a = 0; a < 3; ++a) {
                dt += g[2 + a] * Gf[(((int64_t)f * 3 + a) * n + li) * n + lj];
                ds += g[2 + a] * Gf[(((int64_t)f * 3 + a) * n + lj) * n + li];
            }
            v += c.dn_trial * dt + c.dn_test * ds;
        }
        v *= g[0];
        const int64_t row = l2n[e * n + li];
        VT* out = val + ia[row] + pos[(e * n + li) * n + lj];
        *out = (VT)((double)*out + v);
    }
}

// F_i += |f| ((g + g_h / hFace) Lf(i) + g_dn sum_a w_a Df(a, i))
__global__ void face_load_kernel(int64_t f0, int64_t f1, const int32_t* __restrict__ faces, const double* __restrict__ geo,
                                 const int32_t* __restrict__ l2n, int n, const double* __restrict__ Lf, const double* __restrict__ Df,
                                 const int* __restrict__ fl, int nfl, double gc, double gh, double gdn, int full,
                                 double* __restrict__ rhs) {
    const int per = full ? n : nfl;
    const int64_t total = (f1 - f0) * per;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = f0 + t / per;
        const int a = (int)(t % per);
        const int64_t e = faces[k] >> 2;
        const int f = faces[k] & 3;
        const int li = full ? a : fl[f * nfl + a];
        const double* g = geo + 5 * k;
        double v = (gc + gh / g[1]) * Lf[(int64_t)f * n + li];
        if (full) {
            double d = 0.0;
            for (int b = 0; b < 3; ++b) d += g[2 + b] * Df[((int64_t)f * 3 + b) * n + li];
            v += gdn * d;
        }
        rhs[l2n[e * n + li]] += g[0] * v;
    }
}

int get_face_set(fgpu_ctx* ctx, fgpu_space* V, int range, double xmax, int whole, fgpu_space::FaceSet** out) {
    const int xmax_on = range == FGPU_RANGE_MARKED_FACES ? 1 : 0;
    for (auto& fs : V->face_sets)
        if (fs.xmax_on == xmax_on && (!xmax_on || fs.xmax == xmax) && fs.whole == whole) { *out = &fs; return FGPU_OK; }
    if (ctx->capturing) { ctx->err = "face integrals: assemble once before capturing (face lists)"; return FGPU_ERR_INVALID; }
    fgpu_mesh* M = V->mesh;
    if (M->h_xyz_stale) {
        FGPU_CUDA_CHECK(ctx, cudaMemcpy(M->h_xyz.data(), M->d_xyz, M->h_xyz.size() * sizeof(double), cudaMemcpyDeviceToHost));
        M->h_xyz_stale = false;
    }
    fgpu_space::FaceSet fs;
    fs.xmax_on = xmax_on;
    fs.xmax = xmax;
    fs.whole = whole;
    std::vector<int32_t> faces;
    const int nc = boundary_faces_coloured(M->nt, M->h_tets.data(), M->h_xyz.data(), xmax_on, xmax, whole, faces, fs.colour_ptr);
    if (nc < 0) { ctx->err = "face integrals: more than 64 colours"; return FGPU_ERR_INVALID; }
    if (!faces.empty()) {
        FGPU_CUDA_CHECK(ctx, cudaMalloc(&fs.d_faces, faces.size() * sizeof(int32_t)));
        FGPU_CUDA_CHECK(ctx, cudaMemcpy(fs.d_faces, faces.data(), faces.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    }
    V->face_sets.push_back(fs);
    *out = &V->face_sets.back();
    return FGPU_OK;
}

int face_geometry(fgpu_ctx* ctx, const fgpu_space* V, const fgpu_space::FaceSet& fs, double** d_geo) {
    const int64_t nf = fs.colour_ptr.empty() ? 0 : fs.colour_ptr.back();
    *d_geo = nullptr;
    if (nf == 0) return FGPU_OK;
    if (ctx->capturing) { ctx->err = "face integrals: not capturable"; return FGPU_ERR_INVALID; }
    FGPU_CUDA_CHECK(ctx, cudaMalloc(d_geo, nf * 5 * sizeof(double)));
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((nf + 255) / 256, 152 * 8));
    face_geom_kernel<<<blocks, 256, 0, ctx->stream>>>(nf, fs.d_faces, V->mesh->d_xyz, V->mesh->d_tets, *d_geo);
    ctx->launches++;
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

}  // namespace

int launch_face_matrix(fgpu_ctx* ctx, fgpu_matrix* A, int range, double xmax, double mass, double mass_h, double dn_trial,
                       double dn_test, int accumulate) {
    fgpu_space* V = A->space;
    if (V->ncomp != 1) { ctx->err = "face integrals: scalar spaces only"; return FGPU_ERR_INVALID; }
    if (!V->d_pos) { ctx->err = "face integrals: pattern rows longer than 255 entries"; return FGPU_ERR_INVALID; }
    FaceTablesDev* T = get_face_tables(ctx, V->order);
    if (!T) return FGPU_ERR_INVALID;
    FaceCoefs c;
    c.mass = mass;
    c.mass_h = mass_h;
    c.dn_trial = dn_trial;
    c.dn_test = dn_test;
    const int full = c.full() ? 1 : 0;
    fgpu_space::FaceSet* fs = nullptr;
    int rc = get_face_set(ctx, V, range, xmax, full, &fs);
    if (rc) return rc;
    if (!accumulate) FGPU_CUDA_CHECK(ctx, cudaMemsetAsync(A->d_val, 0, A->nnz * (A->precision == FGPU_F64 ? 8 : 4), ctx->stream));
    double* geo = nullptr;
    rc = face_geometry(ctx, V, *fs, &geo);
    if (rc) return rc;
    const int per = full ? T->n * T->n : T->nfl * T->nfl;
    PendingEvent ev;
    prof_begin(ctx, "assemble_faces", ev);
    for (size_t k = 0; k + 1 < fs->colour_ptr.size(); ++k) {
        const int64_t f0 = fs->colour_ptr[k], f1 = fs->colour_ptr[k + 1];
        const int64_t total = (f1 - f0) * per;
        if (total == 0) continue;
        const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 152 * 8));
        if (A->precision == FGPU_F64)
            face_matrix_kernel<double><<<blocks, 256, 0, ctx->stream>>>(f0, f1, fs->d_faces, geo, V->d_l2n, V->n, A->pattern->d_ia,
                                                                       V->d_pos, T->d_Mf, T->d_Gf, T->d_on, T->d_fl, T->nfl, c, full,
                                                                       (double*)A->d_val);
        else
            face_matrix_kernel<float><<<blocks, 256, 0, ctx->stream>>>(f0, f1, fs->d_faces, geo, V->d_l2n, V->n, A->pattern->d_ia,
                                                                      V->d_pos, T->d_Mf, T->d_Gf, T->d_on, T->d_fl, T->nfl, c, full,
                                                                      (float*)A->d_val);
        ++ctx->launches;
    }
    prof_end(ctx, ev);
    cudaError_t e = cudaGetLastError();
    cudaStreamSynchronize(ctx->stream);
    cudaFree(geo);
    if (e != cudaSuccess) { ctx->err = std::string("face matrix: ") + cudaGetErrorString(e); return FGPU_ERR_CUDA; }
    return FGPU_OK;
}

int launch_face_load(fgpu_ctx* ctx, const fgpu_space* Vc, int range, double xmax, double g, double g_h, double g_dn,
                     double* d_rhs, int accumulate) {
    fgpu_space* V = const_cast<fgpu_space*>(Vc);
    if (V->ncomp != 1) { ctx->err = "face integrals: scalar spaces only"; return FGPU_ERR_INVALID; }
    FaceTablesDev* T = get_face_tables(ctx, V->order);
    if (!T) return FGPU_ERR_INVALID;
    const int full = g_dn != 0.0 ? 1 : 0;
    fgpu_space::FaceSet* fs = nullptr;
    int rc = get_face_set(ctx, V, range, xmax, full, &fs);
    if (rc) return rc;
    if (!accumulate) FGPU_CUDA_CHECK(ctx, cudaMemsetAsync(d_rhs, 0, V->ndof * sizeof(double), ctx->stream));
    double* geo = nullptr;
    rc = face_geometry(ctx, V, *fs, &geo);
    if (rc) return rc;
    const int per = full ? T->n : T->nfl;
    for (size_t k = 0; k + 1 < fs->colour_ptr.size(); ++k) {
        const int64_t f0 = fs->colour_ptr[k], f1 = fs->colour_ptr[k + 1];
        const int64_t total = (f1 - f0) * per;
        if (total == 0) continue;
        const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 152 * 8));
        face_load_kernel<<<blocks, 256, 0, ctx->stream>>>(f0, f1, fs->d_faces, geo, V->d_l2n, V->n, T->d_Lf, T->d_Df, T->d_fl, T->nfl,
                                                         g, g_h, g_dn, full, d_rhs);
        ++ctx->launches;
    }
    cudaError_t e = cudaGetLastError();
    cudaStreamSynchronize(ctx->stream);
    cudaFree(geo);
    if (e != cudaSuccess) { ctx->err = std::string("face load: ") + cudaGetErrorString(e); return FGPU_ERR_CUDA; }
    return FGPU_OK;
}

}  // namespace fgpu
