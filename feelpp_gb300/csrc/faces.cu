// Boundary-face integrals: form2 += integrate(boundaryfaces(mesh) | markedfaces,
// alpha*idt(u)*id(v)) (Robin / impedance terms) and form1 += integrate(faces,
// g*id(v)) (Neumann loads), feelpp/feel/feelvf/integrator.hpp MESH_FACES
// (:786-795) for affine tetrahedra and scalar Lagrange spaces.
//
// On an affine face the restriction of the element basis is fixed by the local
// face, so int_f phi_i phi_j = |f| Mf[local face](i, j) with per-unit-area tables
// computed once (basis.cpp build_face_tables). The faces of a range are found
// and greedily coloured on the host once per space and range (faces that share
// a vertex get different colours); one launch per colour scatters the face
// blocks into the CSR (or the load vector) without two threads ever writing
// one entry, so the result is deterministic without atomics: every entry gets
// its face contributions in colour order.
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
    int* d_fl = nullptr;      // 4 nfl: local dofs on each face
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
    for (int f = 0; f < 4; ++f) {
        std::vector<int> d = face_dofs(order, f);
        D->nfl = (int)d.size();
        fl.insert(fl.end(), d.begin(), d.end());
    }
    cudaError_t e = cudaMalloc(&D->d_Mf, T.Mf.size() * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&D->d_Lf, T.Lf.size() * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&D->d_fl, fl.size() * sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(D->d_Mf, T.Mf.data(), T.Mf.size() * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(D->d_Lf, T.Lf.data(), T.Lf.size() * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(D->d_fl, fl.data(), fl.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaGetLastError();
        ctx->err = std::string("face tables: ") + cudaGetErrorString(e);
        delete D;
        return nullptr;
    }
    g_face_tabs[key] = D;
    return D;
}

// physical face areas |f| (one thread per face)
__global__ void face_area_kernel(int64_t nf, const int32_t* __restrict__ faces, const double* __restrict__ xyz,
                                 const int32_t* __restrict__ tets, double* __restrict__ area) {
    const int fv[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nf; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = faces[k] >> 2;
        const int f = faces[k] & 3;
        const double* A = xyz + 3 * (int64_t)tets[4 * e + fv[f][0]];
        const double* B = xyz + 3 * (int64_t)tets[4 * e + fv[f][1]];
        const double* C = xyz + 3 * (int64_t)tets[4 * e + fv[f][2]];
        const double u[3] = {B[0] - A[0], B[1] - A[1], B[2] - A[2]};
        const double v[3] = {C[0] - A[0], C[1] - A[1], C[2] - A[2]};
        const double c0 = u[1] * v[2] - u[2] * v[1], c1 = u[2] * v[0] - u[0] * v[2], c2 = u[0] * v[1] - u[1] * v[0];
        area[k] = 0.5 * sqrt(c0 * c0 + c1 * c1 + c2 * c2);
    }
}

// one colour: thread per (face, a, b) over the face's local dofs
template <typename VT>
__global__ void face_matrix_kernel(int64_t f0, int64_t f1, const int32_t* __restrict__ faces, const double* __restrict__ area,
                                   const int32_t* __restrict__ l2n, int n, const int64_t* __restrict__ ia,
                                   const uint8_t* __restrict__ pos, const double* __restrict__ Mf, const int* __restrict__ fl,
                                   int nfl, double alpha, VT* __restrict__ val) {
    const int64_t total = (f1 - f0) * nfl * nfl;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = f0 + t / (nfl * nfl);
        const int ab = (int)(t % (nfl * nfl));
        const int64_t e = faces[k] >> 2;
        const int f = faces[k] & 3;
        const int li = fl[f * nfl + ab / nfl], lj = fl[f * nfl + ab % nfl];
        const double v = alpha * area[k] * Mf[((int64_t)f * n + li) * n + lj];
        const int64_t row = l2n[e * n + li];
        VT* out = val + ia[row] + pos[(e * n + li) * n + lj];
        *out = (VT)((double)*out + v);
    }
}

__global__ void face_load_kernel(int64_t f0, int64_t f1, const int32_t* __restrict__ faces, const double* __restrict__ area,
                                 const int32_t* __restrict__ l2n, int n, const double* __restrict__ Lf, const int* __restrict__ fl,
                                 int nfl, double g, double* __restrict__ rhs) {
    const int64_t total = (f1 - f0) * nfl;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = f0 + t / nfl;
        const int a = (int)(t % nfl);
        const int64_t e = faces[k] >> 2;
        const int f = faces[k] & 3;
        const int li = fl[f * nfl + a];
        rhs[l2n[e * n + li]] += g * area[k] * Lf[(int64_t)f * n + li];
    }
}

int get_face_set(fgpu_ctx* ctx, fgpu_space* V, int range, double xmax, fgpu_space::FaceSet** out) {
    const int xmax_on = range == FGPU_RANGE_MARKED_FACES ? 1 : 0;
    for (auto& fs : V->face_sets)
        if (fs.xmax_on == xmax_on && (!xmax_on || fs.xmax == xmax)) { *out = &fs; return FGPU_OK; }
    if (ctx->capturing) { ctx->err = "face integrals: assemble once before capturing (face lists)"; return FGPU_ERR_INVALID; }
    fgpu_mesh* M = V->mesh;
    if (M->h_xyz_stale) {
        FGPU_CUDA_CHECK(ctx, cudaMemcpy(M->h_xyz.data(), M->d_xyz, M->h_xyz.size() * sizeof(double), cudaMemcpyDeviceToHost));
        M->h_xyz_stale = false;
    }
    fgpu_space::FaceSet fs;
    fs.xmax_on = xmax_on;
    fs.xmax = xmax;
    std::vector<int32_t> faces;
    const int nc = boundary_faces_coloured(M->nt, M->h_tets.data(), M->h_xyz.data(), xmax_on, xmax, faces, fs.colour_ptr);
    if (nc < 0) { ctx->err = "face integrals: more than 64 colours"; return FGPU_ERR_INVALID; }
    if (!faces.empty()) {
        FGPU_CUDA_CHECK(ctx, cudaMalloc(&fs.d_faces, faces.size() * sizeof(int32_t)));
        FGPU_CUDA_CHECK(ctx, cudaMemcpy(fs.d_faces, faces.data(), faces.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    }
    V->face_sets.push_back(fs);
    *out = &V->face_sets.back();
    return FGPU_OK;
}

int face_areas(fgpu_ctx* ctx, const fgpu_space* V, const fgpu_space::FaceSet& fs, double** d_area) {
    const int64_t nf = fs.colour_ptr.empty() ? 0 : fs.colour_ptr.back();
    *d_area = nullptr;
    if (nf == 0) return FGPU_OK;
    if (ctx->capturing) { ctx->err = "face integrals: not capturable"; return FGPU_ERR_INVALID; }
    FGPU_CUDA_CHECK(ctx, cudaMalloc(d_area, nf * sizeof(double)));
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((nf + 255) / 256, 152 * 8));
    face_area_kernel<<<blocks, 256, 0, ctx->stream>>>(nf, fs.d_faces, V->mesh->d_xyz, V->mesh->d_tets, *d_area);
    ctx->launches++;
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

}  // namespace

int launch_face_matrix(fgpu_ctx* ctx, fgpu_matrix* A, int range, double xmax, double alpha, int accumulate) {
    fgpu_space* V = A->space;
    if (V->ncomp != 1) { ctx->err = "face integrals: scalar spaces only"; return FGPU_ERR_INVALID; }
    if (!V->d_pos) { ctx->err = "face integrals: pattern rows longer than 255 entries"; return FGPU_ERR_INVALID; }
    FaceTablesDev* T = get_face_tables(ctx, V->order);
    if (!T) return FGPU_ERR_INVALID;
    fgpu_space::FaceSet* fs = nullptr;
    int rc = get_face_set(ctx, V, range, xmax, &fs);
    if (rc) return rc;
    if (!accumulate) FGPU_CUDA_CHECK(ctx, cudaMemsetAsync(A->d_val, 0, A->nnz * (A->precision == FGPU_F64 ? 8 : 4), ctx->stream));
    double* area = nullptr;
    rc = face_areas(ctx, V, *fs, &area);
    if (rc) return rc;
    PendingEvent ev;
    prof_begin(ctx, "assemble_faces", ev);
    for (size_t c = 0; c + 1 < fs->colour_ptr.size(); ++c) {
        const int64_t f0 = fs->colour_ptr[c], f1 = fs->colour_ptr[c + 1];
        const int64_t total = (f1 - f0) * T->nfl * T->nfl;
        if (total == 0) continue;
        const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 152 * 8));
        if (A->precision == FGPU_F64)
            face_matrix_kernel<double><<<blocks, 256, 0, ctx->stream>>>(f0, f1, fs->d_faces, area, V->d_l2n, V->n, A->pattern->d_ia,
                                                                       V->d_pos, T->d_Mf, T->d_fl, T->nfl, alpha, (double*)A->d_val);
        else
            face_matrix_kernel<float><<<blocks, 256, 0, ctx->stream>>>(f0, f1, fs->d_faces, area, V->d_l2n, V->n, A->pattern->d_ia,
                                                                      V->d_pos, T->d_Mf, T->d_fl, T->nfl, alpha, (float*)A->d_val);
        ++ctx->launches;
    }
    prof_end(ctx, ev);
    cudaError_t e = cudaGetLastError();
    cudaStreamSynchronize(ctx->stream);
    cudaFree(area);
    if (e != cudaSuccess) { ctx->err = std::string("face matrix: ") + cudaGetErrorString(e); return FGPU_ERR_CUDA; }
    return FGPU_OK;
}

int launch_face_load(fgpu_ctx* ctx, const fgpu_space* Vc, int range, double xmax, double g, double* d_rhs, int accumulate) {
    fgpu_space* V = const_cast<fgpu_space*>(Vc);
    if (V->ncomp != 1) { ctx->err = "face integrals: scalar spaces only"; return FGPU_ERR_INVALID; }
    FaceTablesDev* T = get_face_tables(ctx, V->order);
    if (!T) return FGPU_ERR_INVALID;
    fgpu_space::FaceSet* fs = nullptr;
    int rc = get_face_set(ctx, V, range, xmax, &fs);
    if (rc) return rc;
    if (!accumulate) FGPU_CUDA_CHECK(ctx, cudaMemsetAsync(d_rhs, 0, V->ndof * sizeof(double), ctx->stream));
    double* area = nullptr;
    rc = face_areas(ctx, V, *fs, &area);
    if (rc) return rc;
    for (size_t c = 0; c + 1 < fs->colour_ptr.size(); ++c) {
        const int64_t f0 = fs->colour_ptr[c], f1 = fs->colour_ptr[c + 1];
        const int64_t total = (f1 - f0) * T->nfl;
        if (total == 0) continue;
        const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 152 * 8));
        face_load_kernel<<<blocks, 256, 0, ctx->stream>>>(f0, f1, fs->d_faces, area, V->d_l2n, V->n, T->d_Lf, T->d_fl, T->nfl, g,
                                                         d_rhs);
        ++ctx->launches;
    }
    cudaError_t e = cudaGetLastError();
    cudaStreamSynchronize(ctx->stream);
    cudaFree(area);
    if (e != cudaSuccess) { ctx->err = std::string("face load: ") + cudaGetErrorString(e); return FGPU_ERR_CUDA; }
    return FGPU_OK;
}

}  // namespace fgpu
