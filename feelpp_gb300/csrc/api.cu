// C-ABI entry points (include/fgpu.h). Host orchestration of the device
// assembly path; every call returns a status code and never throws.
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "df64.h"
#include "fgpu_core.h"

namespace fgpu {
int launch_assemble_elasticity(fgpu_ctx* ctx, fgpu_matrix* A, const DevTables* tab, const double* d_coef, double lam,
                               double mu, int accumulate);
int launch_expand_pattern(fgpu_ctx* ctx, const DevPattern& P, int nc, int64_t* d_ia, int32_t* d_ja);
int launch_norms_sine(fgpu_ctx* ctx, const fgpu_space* V, const DevTables* tab, const double* d_u, double* l2, double* h1);
}  // namespace fgpu

using namespace fgpu;

DevPattern::~DevPattern() {
    cudaFree(d_ia);
    cudaFree(d_ja);
}

namespace {

int set_err(fgpu_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return code;
}

template <typename T>
int dev_alloc(fgpu_ctx* ctx, T** p, size_t count) {
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        return set_err(ctx, FGPU_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    return FGPU_OK;
}

// Resolve pending profiling events (after a stream sync) and check the status word.
int finish(fgpu_ctx* ctx, bool sync = true) {
    if (!sync || ctx->capturing) return FGPU_OK;   // captured calls: the status is checked at graph launch
    int hst = 0;
    cudaError_t e = cudaMemcpyAsync(&hst, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return set_err(ctx, FGPU_ERR_CUDA, std::string("stream: ") + cudaGetErrorString(e));
    for (auto& ev : ctx->pending) {
        float ms = 0;
        cudaEventElapsedTime(&ms, ev.start, ev.stop);
        auto& a = ctx->prof[ev.name];
        a.count++;
        a.total_ms += ms;
        ctx->event_pool.push_back(ev.start);
        ctx->event_pool.push_back(ev.stop);
    }
    ctx->pending.clear();
    if (hst) {
        cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream);
        cudaStreamSynchronize(ctx->stream);
        if (hst & kStatusBadElement) return set_err(ctx, FGPU_ERR_BAD_ELEMENT, "degenerate element: |det K| <= 0 or non-finite");
        if (hst & kStatusMissingEntry) return set_err(ctx, FGPU_ERR_PATTERN, "element column absent from the pattern");
        if (hst & kStatusRowOverflow) return set_err(ctx, FGPU_ERR_INVALID, "pattern row longer than the staging buffer");
        if (hst & kStatusStreamTimeout) return set_err(ctx, FGPU_ERR_CUDA, "streamed assembly: a wait for another task timed out");
        return set_err(ctx, FGPU_ERR_CUDA, "device status " + std::to_string(hst));
    }
    return FGPU_OK;
}

int ensure_pattern(fgpu_space* V) {
    if (V->pattern) return FGPU_OK;
    fgpu_ctx* ctx = V->ctx;
    std::string err;
    if (!ctx->host_setup) {
        auto P = std::make_shared<DevPattern>();
        ctx->err.clear();
        const int rcd = build_pattern_device(ctx, V, *P, V->h_pattern.ia);
        if (rcd == FGPU_OK) {
            V->h_pattern.nrows = P->nrows;
            V->h_pattern.nnz = P->nnz;
            V->h_pattern.max_row = P->max_row;
            V->pattern = P;
            if (P->max_row <= 256) {
                int rc = launch_build_positions(ctx, V);
                if (rc) return rc;
                rc = finish(ctx);
                if (rc) return rc;
            }
            return FGPU_OK;
        }
        if (rcd != FGPU_ERR_INVALID) return rcd;
        ctx->err.clear();                 // rows too long for the device sort: host path
        if (V->topo.inc_ptr.size() != (size_t)V->topo.nnodes + 1 || V->topo.inc.empty()) {
            // the device-built topology keeps no host incidence: fetch it
            V->topo.inc_ptr.resize(V->topo.nnodes + 1);
            V->topo.inc.resize((size_t)V->mesh->nt * V->n);
            FGPU_CUDA_CHECK(ctx, cudaMemcpy(V->topo.inc_ptr.data(), V->d_inc_ptr, V->topo.inc_ptr.size() * sizeof(int64_t), cudaMemcpyDeviceToHost));
            FGPU_CUDA_CHECK(ctx, cudaMemcpy(V->topo.inc.data(), V->d_inc, V->topo.inc.size() * sizeof(int32_t), cudaMemcpyDeviceToHost));
        }
    }
    if (!build_node_pattern(V->topo, V->mesh->nt, V->h_pattern, ctx->host_threads, err))
        return set_err(ctx, FGPU_ERR_ALLOC, err);
    auto P = std::make_shared<DevPattern>();
    P->nrows = V->h_pattern.nrows;
    P->nnz = V->h_pattern.nnz;
    P->max_row = V->h_pattern.max_row;
    int rc = dev_alloc(ctx, &P->d_ia, P->nrows + 1);
    if (!rc) rc = dev_alloc(ctx, &P->d_ja, P->nnz);
    if (rc) return rc;
    FGPU_CUDA_CHECK(ctx, cudaMemcpy(P->d_ia, V->h_pattern.ia.data(), (P->nrows + 1) * sizeof(int64_t), cudaMemcpyHostToDevice));
    FGPU_CUDA_CHECK(ctx, cudaMemcpy(P->d_ja, V->h_pattern.ja.data(), P->nnz * sizeof(int32_t), cudaMemcpyHostToDevice));
    V->pattern = P;
    // the device copy is authoritative; drop the host ja
    std::vector<int32_t>().swap(V->h_pattern.ja);
    if (P->max_row <= 256) {
        rc = launch_build_positions(ctx, V);
        if (rc) return rc;
        rc = finish(ctx);
        if (rc) return rc;
    }
    return FGPU_OK;
}

int form_qdeg(const fgpu_space* V, int q) { return q > 0 ? q : 2 * V->order; }

// calls that allocate, synchronize or read host data back cannot be captured
#define FGPU_NO_CAPTURE(ctx, what)                                                              \
    do {                                                                                        \
        if ((ctx) && (ctx)->capturing) return set_err((ctx), FGPU_ERR_INVALID, what ": not allowed while capturing a graph"); \
    } while (0)

}  // namespace

extern "C" {

int fgpu_create(const fgpu_config* cfg, fgpu_ctx** out) {
    if (!out) return FGPU_ERR_INVALID;
    *out = nullptr;
    fgpu_ctx* ctx = new (std::nothrow) fgpu_ctx();
    if (!ctx) return FGPU_ERR_ALLOC;
    ctx->device = cfg ? cfg->device : 0;
    ctx->profile = cfg ? cfg->profile : 0;
    int ht = cfg ? cfg->host_threads : 0;
    if (ht <= 0) ht = (int)std::max(1u, std::thread::hardware_concurrency());
    ctx->host_threads = ht;
    ctx->host_setup = cfg ? cfg->host_setup : 0;
    ctx->tune = cfg ? cfg->tune : 0;
    if (cfg && cfg->tune_cache) {
        ctx->tune_file = cfg->tune_cache;
        tune_load_cache_file(ctx->tune_file);
    }
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) {
        delete ctx;
        return FGPU_ERR_CUDA;
    }
    if (cfg && cfg->stream) {
        ctx->stream = (cudaStream_t)cfg->stream;
    } else {
        e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
        ctx->own_stream = true;
    }
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_status, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(ctx->d_status, 0, sizeof(int));
    if (e != cudaSuccess) {
        delete ctx;
        return FGPU_ERR_CUDA;
    }
    *out = ctx;
    return FGPU_OK;
}

int fgpu_destroy(fgpu_ctx* ctx) {
    if (!ctx) return FGPU_OK;
    cudaStreamSynchronize(ctx->stream);
    for (auto& ev : ctx->pending) {
        cudaEventDestroy(ev.start);
        cudaEventDestroy(ev.stop);
    }
    for (auto ev : ctx->event_pool) cudaEventDestroy(ev);
    for (int i = 0; i < 4; ++i)
        if (ctx->copy_streams[i]) cudaStreamDestroy(ctx->copy_streams[i]);
    for (int i = 0; i < 5; ++i)
        if (ctx->copy_events[i]) cudaEventDestroy(ctx->copy_events[i]);
    cudaFree(ctx->d_status);
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return FGPU_OK;
}

const char* fgpu_last_error(const fgpu_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int fgpu_sync(fgpu_ctx* ctx) {
    if (!ctx) return FGPU_ERR_INVALID;
    return finish(ctx, true);
}

int64_t fgpu_launch_count(const fgpu_ctx* ctx) { return ctx ? ctx->launches : 0; }

// ---------------------------------------------------------------------------
int fgpu_mesh_upload(fgpu_ctx* ctx, int64_t nv, const double* xyz, int64_t nt, const int32_t* tets, fgpu_mesh** out) {
    FGPU_NO_CAPTURE(ctx, "mesh_upload");
    if (!ctx || !out || !xyz || !tets || nv <= 0 || nt <= 0) return set_err(ctx, FGPU_ERR_INVALID, "mesh_upload: bad arguments");
    *out = nullptr;
    for (int64_t k = 0; k < 4 * nt; ++k)
        if (tets[k] < 0 || tets[k] >= nv) return set_err(ctx, FGPU_ERR_OUT_OF_RANGE, "tetrahedron vertex index out of range");
    fgpu_mesh* M = new (std::nothrow) fgpu_mesh();
    if (!M) return set_err(ctx, FGPU_ERR_ALLOC, "host allocation");
    M->ctx = ctx;
    M->nv = nv;
    M->nt = nt;
    M->h_xyz.assign(xyz, xyz + 3 * nv);
    M->h_tets.assign(tets, tets + 4 * nt);
    int rc = dev_alloc(ctx, &M->d_xyz, 3 * nv);
    if (!rc) rc = dev_alloc(ctx, &M->d_tets, 4 * nt);
    if (rc) { delete M; return rc; }
    cudaMemcpyAsync(M->d_xyz, xyz, 3 * nv * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(M->d_tets, tets, 4 * nt * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        cudaFree(M->d_xyz); cudaFree(M->d_tets); delete M;
        return set_err(ctx, FGPU_ERR_CUDA, cudaGetErrorString(e));
    }
    *out = M;
    return FGPU_OK;
}

int fgpu_mesh_upload_hex(fgpu_ctx* ctx, int64_t nv, const double* xyz, int64_t nh, const int32_t* hexes, fgpu_mesh** out) {
    FGPU_NO_CAPTURE(ctx, "mesh_upload_hex");
    if (!ctx || !out || !xyz || !hexes || nv <= 0 || nh <= 0) return set_err(ctx, FGPU_ERR_INVALID, "mesh_upload_hex: bad arguments");
    *out = nullptr;
    for (int64_t k = 0; k < 8 * nh; ++k)
        if (hexes[k] < 0 || hexes[k] >= nv) return set_err(ctx, FGPU_ERR_OUT_OF_RANGE, "hexahedron vertex index out of range");
    fgpu_mesh* M = new (std::nothrow) fgpu_mesh();
    if (!M) return set_err(ctx, FGPU_ERR_ALLOC, "host allocation");
    M->ctx = ctx;
    M->cv = 8;
    M->nv = nv;
    M->nt = nh;
    M->h_xyz.assign(xyz, xyz + 3 * nv);
    M->h_tets.assign(hexes, hexes + 8 * nh);
    int rc = dev_alloc(ctx, &M->d_xyz, 3 * nv);
    if (!rc) rc = dev_alloc(ctx, &M->d_tets, 8 * nh);
    if (rc) { cudaFree(M->d_xyz); delete M; return rc; }
    cudaMemcpyAsync(M->d_xyz, xyz, 3 * nv * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(M->d_tets, hexes, 8 * nh * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        cudaFree(M->d_xyz); cudaFree(M->d_tets); delete M;
        return set_err(ctx, FGPU_ERR_CUDA, cudaGetErrorString(e));
    }
    *out = M;
    return FGPU_OK;
}

int fgpu_mesh_cell_vertices(const fgpu_mesh* M, int* nverts) {
    if (!M || !nverts) return FGPU_ERR_INVALID;
    *nverts = M->cv;
    return FGPU_OK;
}

int fgpu_mesh_set_coords(fgpu_mesh* M, const double* xyz) {
    if (!M || !xyz) return FGPU_ERR_INVALID;
    fgpu_ctx* ctx = M->ctx;
    FGPU_NO_CAPTURE(ctx, "mesh_set_coords");
    FGPU_CUDA_CHECK(ctx, cudaMemcpyAsync(M->d_xyz, xyz, 3 * M->nv * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    M->h_xyz_stale = true;           // the host copy is refreshed when a host-side query needs it
    M->coords_version++;
    return FGPU_OK;
}

int fgpu_mesh_destroy(fgpu_mesh* M) {
    if (!M) return FGPU_OK;
    cudaFree(M->d_xyz);
    cudaFree(M->d_tets);
    cudaFree(M->d_colour_perm);
    cudaFree(M->d_ho);
    delete M;
    return FGPU_OK;
}

// ---------------------------------------------------------------------------
int fgpu_space_create(fgpu_ctx* ctx, fgpu_mesh* M, int order, int ncomp, fgpu_space** out) {
    FGPU_NO_CAPTURE(ctx, "space_create");
    if (!ctx || !M || !out) return set_err(ctx, FGPU_ERR_INVALID, "space_create: bad arguments");
    if (order < 1 || order > 3) return set_err(ctx, FGPU_ERR_INVALID, "order must be 1, 2 or 3");
    if (ncomp != 1 && ncomp != 3) return set_err(ctx, FGPU_ERR_INVALID, "ncomp must be 1 or 3");
    if (M->cv == 8 && (order > 2 || ncomp != 1)) return set_err(ctx, FGPU_ERR_INVALID, "hexahedra: scalar Q1 and Q2 spaces");
    *out = nullptr;
    fgpu_space* V = new (std::nothrow) fgpu_space();
    if (!V) return set_err(ctx, FGPU_ERR_ALLOC, "host allocation");
    V->ctx = ctx;
    V->mesh = M;
    V->order = order;
    V->ncomp = ncomp;
    V->n = M->cv == 8 ? hex_nloc(order) : nloc_of(order);
    std::string err;
    if (M->cv == 8) {
        if (!build_hex_topology(M->nv, M->nt, M->h_tets.data(), order, V->topo, err)) {
            delete V;
            return set_err(ctx, FGPU_ERR_INVALID, err);
        }
    } else if (!ctx->host_setup) {
        // dof table and incidence on the device; the host path takes the meshes it cannot handle
        ctx->err.clear();
        const int rcd = build_space_device(ctx, V);
        if (rcd == FGPU_OK) {
            V->ndof = V->topo.nnodes * ncomp;
            *out = V;
            return FGPU_OK;
        }
        cudaFree(V->d_l2n); cudaFree(V->d_inc_ptr); cudaFree(V->d_inc);
        V->d_l2n = nullptr; V->d_inc_ptr = nullptr; V->d_inc = nullptr;
        V->topo = Topology();
        V->dev_topology = false;
        if (rcd != FGPU_ERR_INVALID) { delete V; return rcd; }   // bad input or a device error
        ctx->err.clear();                                          // outside the device path's limits
    }
    if (M->cv == 4 && !build_topology(M->nv, M->nt, M->h_tets.data(), order, V->topo, err)) {
        delete V;
        return set_err(ctx, FGPU_ERR_INVALID, err);
    }
    V->ndof = V->topo.nnodes * ncomp;
    int rc = dev_alloc(ctx, &V->d_l2n, V->topo.l2n.size());
    if (!rc) rc = dev_alloc(ctx, &V->d_inc_ptr, V->topo.inc_ptr.size());
    if (!rc) rc = dev_alloc(ctx, &V->d_inc, V->topo.inc.size());
    if (rc) { fgpu_space_destroy(V); return rc; }
    cudaMemcpy(V->d_l2n, V->topo.l2n.data(), V->topo.l2n.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
    cudaMemcpy(V->d_inc_ptr, V->topo.inc_ptr.data(), V->topo.inc_ptr.size() * sizeof(int64_t), cudaMemcpyHostToDevice);
    cudaError_t e = cudaMemcpy(V->d_inc, V->topo.inc.data(), V->topo.inc.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { fgpu_space_destroy(V); return set_err(ctx, FGPU_ERR_CUDA, cudaGetErrorString(e)); }
    *out = V;
    return FGPU_OK;
}

int fgpu_space_ndof(const fgpu_space* V, int64_t* ndof, int* nloc) {
    if (!V) return FGPU_ERR_INVALID;
    if (ndof) *ndof = V->ndof;
    if (nloc) *nloc = V->n * V->ncomp;
    return FGPU_OK;
}

int fgpu_space_l2g(const fgpu_space* V, int32_t* out) {
    if (!V || !out) return FGPU_ERR_INVALID;
    const int n = V->n, nc = V->ncomp;
    const int64_t nt = V->mesh->nt;
    for (int64_t e = 0; e < nt; ++e)
        for (int c = 0; c < nc; ++c)
            for (int l = 0; l < n; ++l)
                out[e * n * nc + (int64_t)n * c + l] = V->topo.l2n[(size_t)e * n + l] * nc + c;
    return FGPU_OK;
}

int fgpu_space_boundary_dofs(const fgpu_space* V, int xmax_on, double xmax, int64_t* count, int32_t* dofs) {
    if (!V || !count) return FGPU_ERR_INVALID;
    std::vector<int32_t> nodes;
    if (V->mesh->h_xyz_stale) {
        FGPU_CUDA_CHECK(V->ctx, cudaMemcpyAsync(V->mesh->h_xyz.data(), V->mesh->d_xyz, V->mesh->h_xyz.size() * sizeof(double),
                                                cudaMemcpyDeviceToHost, V->ctx->stream));
        FGPU_CUDA_CHECK(V->ctx, cudaStreamSynchronize(V->ctx->stream));
        V->mesh->h_xyz_stale = false;
    }
    // the last result is kept (callers ask for the count, then the list)
    fgpu_space* W = const_cast<fgpu_space*>(V);
    if (W->bnd_valid && W->bnd_xmax_on == xmax_on && (!xmax_on || W->bnd_xmax == xmax) && W->bnd_coords == W->mesh->coords_version) {
        nodes = W->bnd_nodes;
    } else {
        if (V->mesh->cv == 8)
            hex_boundary_nodes(V->mesh->nt, V->mesh->h_tets.data(), V->mesh->h_xyz.data(), V->topo, xmax_on, xmax, nodes);
        else if (boundary_nodes_device(V->ctx, V, xmax_on, xmax, nodes) != FGPU_OK)
            boundary_nodes(V->mesh->nt, V->mesh->h_tets.data(), V->mesh->h_xyz.data(), V->topo, xmax_on, xmax, nodes);
        W->bnd_nodes = nodes;
        W->bnd_xmax_on = xmax_on;
        W->bnd_xmax = xmax;
        W->bnd_coords = W->mesh->coords_version;
        W->bnd_valid = true;
    }
    *count = (int64_t)nodes.size() * V->ncomp;
    if (dofs)
        for (size_t k = 0; k < nodes.size(); ++k)
            for (int c = 0; c < V->ncomp; ++c) dofs[k * V->ncomp + c] = nodes[k] * V->ncomp + c;
    return FGPU_OK;
}

int fgpu_space_destroy(fgpu_space* V) {
    if (!V) return FGPU_OK;
    cudaFree(V->d_l2n);
    cudaFree(V->d_inc_ptr);
    cudaFree(V->d_inc);
    for (auto& fs : V->face_sets) cudaFree(fs.d_faces);
    cudaFree(V->d_pos);
    cudaFree(V->d_gptr);
    cudaFree(V->d_gidx);
    stream_plan_free(V->stream_plan);
    delete V;
    return FGPU_OK;
}

// ---------------------------------------------------------------------------
int fgpu_matrix_create(fgpu_ctx* ctx, fgpu_space* test, fgpu_space* trial, int precision, fgpu_matrix** out) {
    FGPU_NO_CAPTURE(ctx, "matrix_create");
    if (!ctx || !test || !out) return set_err(ctx, FGPU_ERR_INVALID, "matrix_create: bad arguments");
    if (trial && trial != test) return set_err(ctx, FGPU_ERR_INVALID, "test and trial spaces must be the same space");
    if (precision != FGPU_F64 && precision != FGPU_F32) return set_err(ctx, FGPU_ERR_INVALID, "bad precision");
    *out = nullptr;
    int rc = ensure_pattern(test);
    if (rc) return rc;
    fgpu_matrix* A = new (std::nothrow) fgpu_matrix();
    if (!A) return set_err(ctx, FGPU_ERR_ALLOC, "host allocation");
    A->ctx = ctx;
    A->space = test;
    A->precision = precision;
    A->ncomp = test->ncomp;
    A->pattern = test->pattern;
    const int nc = test->ncomp;
    A->nrows = test->pattern->nrows * nc;
    A->nnz = test->pattern->nnz * nc * nc;
    if (nc == 1) {
        A->d_ia = test->pattern->d_ia;
        A->d_ja = test->pattern->d_ja;
        A->own_ia_ja = false;
    } else {
        rc = dev_alloc(ctx, &A->d_ia, A->nrows + 1);
        if (!rc) rc = dev_alloc(ctx, &A->d_ja, A->nnz);
        if (rc) { fgpu_matrix_destroy(A); return rc; }
        A->own_ia_ja = true;
        rc = launch_expand_pattern(ctx, *A->pattern, nc, A->d_ia, A->d_ja);
        if (rc) { fgpu_matrix_destroy(A); return rc; }
    }
    rc = dev_alloc(ctx, (char**)&A->d_val, A->nnz * (precision == FGPU_F64 ? 8 : 4));
    if (rc) { fgpu_matrix_destroy(A); return rc; }
    cudaMemsetAsync(A->d_val, 0, A->nnz * (precision == FGPU_F64 ? 8 : 4), ctx->stream);
    rc = finish(ctx);
    if (rc) { fgpu_matrix_destroy(A); return rc; }
    *out = A;
    return FGPU_OK;
}

int fgpu_matrix_create_like(const fgpu_matrix* S, int precision, fgpu_matrix** out) {
    if (S) FGPU_NO_CAPTURE(S->ctx, "matrix_create_like");
    if (!S || !out) return FGPU_ERR_INVALID;
    fgpu_ctx* ctx = S->ctx;
    fgpu_matrix* A = new (std::nothrow) fgpu_matrix();
    if (!A) return FGPU_ERR_ALLOC;
    A->ctx = ctx;
    A->space = S->space;
    A->precision = precision;
    A->ncomp = S->ncomp;
    A->pattern = S->pattern;
    A->nrows = S->nrows;
    A->nnz = S->nnz;
    if (S->ncomp == 1) {
        A->d_ia = S->d_ia;
        A->d_ja = S->d_ja;
    } else {
        int rc = dev_alloc(ctx, &A->d_ia, A->nrows + 1);
        if (!rc) rc = dev_alloc(ctx, &A->d_ja, A->nnz);
        if (rc) { fgpu_matrix_destroy(A); return rc; }
        A->own_ia_ja = true;
        cudaMemcpyAsync(A->d_ia, S->d_ia, (A->nrows + 1) * sizeof(int64_t), cudaMemcpyDeviceToDevice, ctx->stream);
        cudaMemcpyAsync(A->d_ja, S->d_ja, A->nnz * sizeof(int32_t), cudaMemcpyDeviceToDevice, ctx->stream);
    }
    int rc = dev_alloc(ctx, (char**)&A->d_val, A->nnz * (precision == FGPU_F64 ? 8 : 4));
    if (rc) { fgpu_matrix_destroy(A); return rc; }
    cudaMemsetAsync(A->d_val, 0, A->nnz * (precision == FGPU_F64 ? 8 : 4), ctx->stream);
    rc = finish(ctx);
    if (rc) { fgpu_matrix_destroy(A); return rc; }
    *out = A;
    return FGPU_OK;
}

int fgpu_matrix_info(const fgpu_matrix* A, int64_t* nrows, int64_t* nnz, int* precision) {
    if (!A) return FGPU_ERR_INVALID;
    if (nrows) *nrows = A->nrows;
    if (nnz) *nnz = A->nnz;
    if (precision) *precision = A->precision;
    return FGPU_OK;
}

// Device -> host copy of a large array in four chunks on four streams (after the
// work queued on the context stream), so that several copy engines move it.
static int chunked_d2h(fgpu_ctx* ctx, void* host, const void* dev, size_t bytes) {
    if (bytes < ((size_t)16 << 20)) {
        FGPU_CUDA_CHECK(ctx, cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, ctx->stream));
        FGPU_CUDA_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
        return FGPU_OK;
    }
    if (!ctx->copy_streams[0]) {
        for (int i = 0; i < 4; ++i) FGPU_CUDA_CHECK(ctx, cudaStreamCreateWithFlags(&ctx->copy_streams[i], cudaStreamNonBlocking));
        for (int i = 0; i < 5; ++i) FGPU_CUDA_CHECK(ctx, cudaEventCreateWithFlags(&ctx->copy_events[i], cudaEventDisableTiming));
    }
    FGPU_CUDA_CHECK(ctx, cudaEventRecord(ctx->copy_events[4], ctx->stream));
    const size_t chunk = ((bytes / 4) + 255) & ~(size_t)255;
    for (int i = 0; i < 4; ++i) {
        const size_t off = (size_t)i * chunk;
        if (off >= bytes) break;
        const size_t nb = std::min(chunk, bytes - off);
        FGPU_CUDA_CHECK(ctx, cudaStreamWaitEvent(ctx->copy_streams[i], ctx->copy_events[4], 0));
        FGPU_CUDA_CHECK(ctx, cudaMemcpyAsync((char*)host + off, (const char*)dev + off, nb, cudaMemcpyDeviceToHost,
                                             ctx->copy_streams[i]));
    }
    for (int i = 0; i < 4; ++i) FGPU_CUDA_CHECK(ctx, cudaStreamSynchronize(ctx->copy_streams[i]));
    return FGPU_OK;
}

int fgpu_matrix_get_csr(const fgpu_matrix* A, int64_t* ia, int32_t* ja, double* val) {
    if (A) FGPU_NO_CAPTURE(A->ctx, "matrix_get_csr");
    if (!A) return FGPU_ERR_INVALID;
    fgpu_ctx* ctx = A->ctx;
    if (ia) FGPU_CUDA_CHECK(ctx, cudaMemcpyAsync(ia, A->d_ia, (A->nrows + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    if (ja) FGPU_CUDA_CHECK(ctx, cudaMemcpyAsync(ja, A->d_ja, A->nnz * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    FGPU_CUDA_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
    if (val) {
        if (A->precision == FGPU_F64) {
            const int rc = chunked_d2h(ctx, val, A->d_val, A->nnz * sizeof(double));
            if (rc) return rc;
        } else {
            std::vector<float> tmp(A->nnz);
            FGPU_CUDA_CHECK(ctx, cudaMemcpy(tmp.data(), A->d_val, A->nnz * sizeof(float), cudaMemcpyDeviceToHost));
            for (int64_t k = 0; k < A->nnz; ++k) val[k] = tmp[k];
        }
    }
    return FGPU_OK;
}

int fgpu_matrix_get_csr32(const fgpu_matrix* A, int32_t* ia, int32_t* ja, double* val) {
    if (A) FGPU_NO_CAPTURE(A->ctx, "matrix_get_csr32");
    if (!A) return FGPU_ERR_INVALID;
    if (A->nnz > (int64_t)INT32_MAX || A->nrows >= (int64_t)INT32_MAX)
        return set_err(A->ctx, FGPU_ERR_INVALID, "matrix_get_csr32: " + std::to_string(A->nnz) +
                                                     " nonzeros do not fit 32-bit row offsets (use fgpu_matrix_get_csr)");
    if (ia) {
        std::vector<int64_t> ia64(A->nrows + 1);
        int rc = fgpu_matrix_get_csr(A, ia64.data(), nullptr, nullptr);
        if (rc) return rc;
        for (int64_t r = 0; r <= A->nrows; ++r) ia[r] = (int32_t)ia64[r];
    }
    return fgpu_matrix_get_csr(A, nullptr, ja, val);
}

int fgpu_matrix_values_device(const fgpu_matrix* A, void** dptr) {
    if (!A || !dptr) return FGPU_ERR_INVALID;
    *dptr = A->d_val;
    return FGPU_OK;
}

int fgpu_matrix_zero(fgpu_matrix* A) {
    if (!A) return FGPU_ERR_INVALID;
    FGPU_CUDA_CHECK(A->ctx, cudaMemsetAsync(A->d_val, 0, A->nnz * (A->precision == FGPU_F64 ? 8 : 4), A->ctx->stream));
    return FGPU_OK;
}

int fgpu_matrix_convert(const fgpu_matrix* src, fgpu_matrix* dst) {
    if (!src || !dst || src->nnz != dst->nnz || src->pattern != dst->pattern) return FGPU_ERR_INVALID;
    int rc = launch_convert_values(src->ctx, src, dst);
    if (rc) return rc;
    return finish(src->ctx);
}

int fgpu_matrix_destroy(fgpu_matrix* A) {
    if (!A) return FGPU_OK;
    if (A->own_ia_ja) {
        cudaFree(A->d_ia);
        cudaFree(A->d_ja);
    }
    cudaFree(A->d_val);
    cudaFree(A->d_coef);
    cudaFree(A->d_kbuf);
    cudaFree(A->d_kappa_stage);
    delete A;
    return FGPU_OK;
}

// ---------------------------------------------------------------------------
// Algorithm choice for FGPU_ALGO_AUTO, from the form and the mesh only (never
// from free device memory or the capture state), so that AUTO gives the same
// bits whoever else uses the device: the two-phase assembly whenever the space
// has a position table (pattern rows of at most 256 entries), the fused gather
// otherwise. A buffer the chosen path cannot allocate is an error. (The
// streamed assembly gives the two-phase bits with a third of the memory
// traffic, but measured slower at P2/P3 64^3: 2.10 against 1.14 ms, 11.7
// against 4.3 ms; it is latency- and issue-bound, so it is not the default.)
// ---------------------------------------------------------------------------
static int auto_assembly_algo(const fgpu_matrix* A, int kind) {
    (void)kind;
    return A->space->d_pos ? FGPU_ALGO_TWO_PHASE : FGPU_ALGO_GATHER;
}

static int assemble_impl(fgpu_ctx* ctx, fgpu_matrix* A, const fgpu_form_desc* f, const double* d_kappa, int accumulate) {
    if (!ctx || !A || !f) return set_err(ctx, FGPU_ERR_INVALID, "assemble_matrix: bad arguments");
    if (A->space->mesh->cv == 8) {   // hexahedra: quadrature element kernel (trilinear map) + gather map
        if (f->algo != FGPU_ALGO_AUTO && f->algo != FGPU_ALGO_TWO_PHASE)
            return set_err(ctx, FGPU_ERR_INVALID, "hexahedra: two-phase assembly only");
        const int rc = launch_assemble_hex(ctx, A, f, d_kappa, accumulate);
        if (rc) return rc;
        return finish(ctx);
    }
    if (f->range == FGPU_RANGE_BOUNDARY_FACES || f->range == FGPU_RANGE_MARKED_FACES) {
        if (A->space->mesh->d_ho) return set_err(ctx, FGPU_ERR_INVALID, "face integrals: flat faces only (the mesh has curved elements)");
        if (f->kind != FGPU_FORM_LAPLACE_MASS || f->kappa != 0.0 || d_kappa || f->kappa_scale)
            return set_err(ctx, FGPU_ERR_INVALID,
                           "face integrals: terms idt(u)*id(v), idt(u)*id(v)/hFace(), (gradt(u).N)*id(v), (grad(v).N)*idt(u)");
        const int rc = launch_face_matrix(ctx, A, f->range, f->range_xmax, f->mass, f->mass_h, f->dn_trial, f->dn_test, accumulate);
        if (rc) return rc;
        return finish(ctx);
    }
    if (f->range != FGPU_RANGE_ELEMENTS) return set_err(ctx, FGPU_ERR_INVALID, "assemble_matrix: bad range");
    if (f->mass_h != 0.0 || f->dn_trial != 0.0 || f->dn_test != 0.0)
        return set_err(ctx, FGPU_ERR_INVALID, "assemble_matrix: hFace()/N() terms on face ranges only");
    fgpu_space* V = A->space;
    if (V->mesh->d_ho) {             // curved (P2-geometry) elements: quadrature element kernel + gather map
        const int rc = launch_assemble_ho(ctx, A, f, d_kappa, accumulate);
        if (rc) return rc;
        return finish(ctx);
    }
    const int qdeg = form_qdeg(V, f->quad_degree);
    std::string err;
    DevTables* tab = get_dev_tables(V->order, qdeg, err);
    if (!tab) return set_err(ctx, FGPU_ERR_INVALID, err);
    int algo = f->algo;
    if (algo == FGPU_ALGO_AUTO) algo = auto_assembly_algo(A, f->kind);
    if (algo == FGPU_ALGO_STREAMED) {
        if (f->kind != FGPU_FORM_LAPLACE_MASS || A->ncomp != 1)
            return set_err(ctx, FGPU_ERR_INVALID, "FGPU_ALGO_STREAMED: scalar Laplace/mass forms only");
        // geometry fused into the kernel: no coefficient records in device memory
        const int rc = launch_assemble_streamed(ctx, A, tab, d_kappa, f->kappa, f->mass, f->kappa_scale, accumulate, nullptr);
        if (rc == kStreamedUnsupported && f->algo == FGPU_ALGO_AUTO) {
            algo = FGPU_ALGO_TWO_PHASE;             // same values (same arithmetic and order)
        } else {
            if (rc == kStreamedUnsupported)
                return set_err(ctx, FGPU_ERR_INVALID, "FGPU_ALGO_STREAMED: a dof belongs to more elements than a gather task stages");
            if (rc) return rc;
            return finish(ctx);
        }
    }
    const int64_t nt = V->mesh->nt;
    const int rec = f->kind == FGPU_FORM_ELASTICITY ? 16 : 8;
    if (A->coef_cap < nt * rec && ctx->capturing)
        return set_err(ctx, FGPU_ERR_INVALID, "assemble_matrix: assemble once before capturing (record buffer)");
    if (A->coef_cap < nt * rec) {
        cudaFree(A->d_coef);
        A->d_coef = nullptr;
        A->coef_cap = 0;
        int rc = dev_alloc(ctx, &A->d_coef, nt * rec);
        if (rc) return rc;
        A->coef_cap = nt * rec;
    }
    int rc = FGPU_OK;
    if (f->kind == FGPU_FORM_LAPLACE_MASS && !(algo == FGPU_ALGO_GATHER_NATIVE_F64 && A->precision == FGPU_F64)) {
        // FP64 matrices: df64 arithmetic on the FP32 pipes; FP32 matrices: binary32
        if (algo == FGPU_ALGO_TWO_PHASE) {
            // the coefficient records are formed inside the element kernel
            const GeoIn geo{V->mesh->d_xyz, V->mesh->d_tets, d_kappa, f->kappa, f->mass, f->kappa_scale};
            rc = launch_assemble_two_phase(ctx, A, tab, nullptr, &geo, accumulate);
            if (rc) return rc;
            return finish(ctx);
        }
        rc = launch_geometry_df(ctx, V->mesh, d_kappa, f->kappa, f->mass, reinterpret_cast<float4*>(A->d_coef), f->kappa_scale);
        if (rc) return rc;
        rc = launch_assemble_gather_df(ctx, A, tab, reinterpret_cast<const float4*>(A->d_coef), accumulate);
        if (rc) return rc;
        return finish(ctx);
    }
    if (f->kappa_scale) return set_err(ctx, FGPU_ERR_INVALID, "kappa_scale: Laplace/mass forms on the default path only");
    if (f->kind == FGPU_FORM_ELASTICITY && algo == FGPU_ALGO_TWO_PHASE) {
        // df64 (FP64 matrices) or binary32 element blocks, then the gather map
        rc = launch_geometry_el_df(ctx, V->mesh, f->lambda, f->mu, reinterpret_cast<float4*>(A->d_coef));
        if (rc) return rc;
        rc = launch_assemble_elasticity_two_phase(ctx, A, tab, reinterpret_cast<const float4*>(A->d_coef), accumulate);
        if (rc) return rc;
        return finish(ctx);
    }
    rc = launch_geometry(ctx, V->mesh, f->kind, d_kappa, f->kappa, f->mass, f->lambda, f->mu, A->d_coef);
    if (rc) return rc;
    if (f->kind == FGPU_FORM_LAPLACE_MASS) {
        rc = launch_assemble_gather(ctx, A, tab, f->kind, A->d_coef, accumulate);
    } else if (f->kind == FGPU_FORM_ELASTICITY) {
        rc = launch_assemble_elasticity(ctx, A, tab, A->d_coef, f->lambda, f->mu, accumulate);
    } else {
        return set_err(ctx, FGPU_ERR_INVALID, "unknown form kind");
    }
    if (rc) return rc;
    return finish(ctx);
}

int fgpu_assemble_matrix(fgpu_ctx* ctx, fgpu_matrix* A, const fgpu_form_desc* f, int accumulate) {
    if (!ctx || !A || !f) return set_err(ctx, FGPU_ERR_INVALID, "assemble_matrix: bad arguments");
    if (!f->kappa_elem) return assemble_impl(ctx, A, f, nullptr, accumulate);
    FGPU_NO_CAPTURE(ctx, "assemble_matrix with host kappa (use fgpu_assemble_matrix_dev)");
    const int64_t nt = A->space->mesh->nt;
    if (!A->d_kappa_stage) {         // kept with the matrix: no allocation (and no implicit sync) per call
        int rc = dev_alloc(ctx, &A->d_kappa_stage, nt);
        if (rc) return rc;
    }
    FGPU_CUDA_CHECK(ctx, cudaMemcpyAsync(A->d_kappa_stage, f->kappa_elem, nt * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    return assemble_impl(ctx, A, f, A->d_kappa_stage, accumulate);
}

int fgpu_set_tensor_cores(fgpu_ctx* ctx, int mask) {
    if (!ctx || (mask & ~(FGPU_TC_F32 | FGPU_TC_DF64))) return FGPU_ERR_INVALID;
    ctx->tensor_cores = mask;
    return FGPU_OK;
}

int fgpu_set_host_transfer(fgpu_ctx* ctx, int mode) {
    if (!ctx) return FGPU_ERR_INVALID;
    if (mode != FGPU_HOST_TRANSFER_AUTO && mode != FGPU_HOST_TRANSFER_COPY && mode != FGPU_HOST_TRANSFER_DIRECT)
        return set_err(ctx, FGPU_ERR_INVALID, "host transfer mode: AUTO, COPY or DIRECT");
    ctx->host_transfer = mode;
    return FGPU_OK;
}

int fgpu_assemble_matrix_host(fgpu_ctx* ctx, fgpu_matrix* A, const fgpu_form_desc* f, double* host_val) {
    if (!ctx || !A || !f || !host_val) return set_err(ctx, FGPU_ERR_INVALID, "assemble_matrix_host: bad arguments");
    FGPU_NO_CAPTURE(ctx, "assemble_matrix_host");
    fgpu_space* V = A->space;
    const int64_t nt = V->mesh->nt;
    const double* d_kappa = nullptr;
    if (f->kappa_elem) {
        if (!A->d_kappa_stage) {
            int rc = dev_alloc(ctx, &A->d_kappa_stage, nt);
            if (rc) return rc;
        }
        FGPU_CUDA_CHECK(ctx, cudaMemcpyAsync(A->d_kappa_stage, f->kappa_elem, nt * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
        d_kappa = A->d_kappa_stage;
    }
    int algo = f->algo;
    if (algo == FGPU_ALGO_AUTO) algo = auto_assembly_algo(A, f->kind);
    const bool pipelined = f->kind == FGPU_FORM_LAPLACE_MASS && f->range == FGPU_RANGE_ELEMENTS && f->mass_h == 0.0 &&
                           f->dn_trial == 0.0 && f->dn_test == 0.0 && A->precision == FGPU_F64 && A->ncomp == 1 &&
                           !V->mesh->d_ho && V->mesh->cv == 4 && (algo == FGPU_ALGO_TWO_PHASE || algo == FGPU_ALGO_STREAMED);
    if (!pipelined) {
        int rc = assemble_impl(ctx, A, f, d_kappa, 0);
        if (rc) return rc;
        return fgpu_matrix_get_csr(A, nullptr, nullptr, host_val);
    }
    std::string err;
    DevTables* tab = get_dev_tables(V->order, form_qdeg(V, f->quad_degree), err);
    if (!tab) return set_err(ctx, FGPU_ERR_INVALID, err);
    if (algo == FGPU_ALGO_STREAMED && ctx->host_transfer != FGPU_HOST_TRANSFER_COPY) {
        // the streamed kernel stores every value to device memory and to the mapped host buffer
        cudaPointerAttributes pa{};
        double* hdev = nullptr;
        if (cudaPointerGetAttributes(&pa, host_val) == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer)
            hdev = static_cast<double*>(pa.devicePointer);
        else
            cudaGetLastError();
        if (hdev) {
            int rc = launch_assemble_streamed(ctx, A, tab, d_kappa, f->kappa, f->mass, f->kappa_scale, 0, hdev);
            if (rc == FGPU_OK) return finish(ctx);
            if (rc != kStreamedUnsupported) return rc;
        }
        if (ctx->host_transfer == FGPU_HOST_TRANSFER_DIRECT)
            return set_err(ctx, FGPU_ERR_INVALID, "direct host transfer: the host buffer is not page-locked and mapped");
    }
    // copy-engine transfers of ranges of entries overlapping the gather of later ranges (two-phase
    // kernels; the streamed path gives the same bits)
    if (A->coef_cap < nt * 8) {
        cudaFree(A->d_coef);
        A->d_coef = nullptr;
        A->coef_cap = 0;
        int rc = dev_alloc(ctx, &A->d_coef, nt * 8);
        if (rc) return rc;
        A->coef_cap = nt * 8;
    }
    const GeoIn geo{V->mesh->d_xyz, V->mesh->d_tets, d_kappa, f->kappa, f->mass, f->kappa_scale};
    int rc = launch_assemble_two_phase_host(ctx, A, tab, nullptr, &geo, host_val);
    if (rc) return rc;
    return finish(ctx);
}

int fgpu_assemble_matrix_dev(fgpu_ctx* ctx, fgpu_matrix* A, const fgpu_form_desc* f, const double* d_kappa, int accumulate) {
    return assemble_impl(ctx, A, f, d_kappa, accumulate);
}

// ---------------------------------------------------------------------------
int fgpu_vector_create(fgpu_ctx* ctx, int64_t n, fgpu_vector** out) {
    FGPU_NO_CAPTURE(ctx, "vector_create");
    if (!ctx || !out || n < 0) return set_err(ctx, FGPU_ERR_INVALID, "vector_create: bad arguments");
    fgpu_vector* v = new (std::nothrow) fgpu_vector();
    if (!v) return FGPU_ERR_ALLOC;
    v->ctx = ctx;
    v->n = n;
    int rc = dev_alloc(ctx, &v->d, n);
    if (rc) { delete v; return rc; }
    cudaMemsetAsync(v->d, 0, n * sizeof(double), ctx->stream);
    *out = v;
    return FGPU_OK;
}
int fgpu_vector_upload(fgpu_vector* v, const double* host) {
    if (!v || !host) return FGPU_ERR_INVALID;
    FGPU_CUDA_CHECK(v->ctx, cudaMemcpyAsync(v->d, host, v->n * sizeof(double), cudaMemcpyHostToDevice, v->ctx->stream));
    return FGPU_OK;
}
int fgpu_vector_download(const fgpu_vector* v, double* host) {
    if (v) FGPU_NO_CAPTURE(v->ctx, "vector_download");
    if (!v || !host) return FGPU_ERR_INVALID;
    FGPU_CUDA_CHECK(v->ctx, cudaMemcpyAsync(host, v->d, v->n * sizeof(double), cudaMemcpyDeviceToHost, v->ctx->stream));
    FGPU_CUDA_CHECK(v->ctx, cudaStreamSynchronize(v->ctx->stream));
    return FGPU_OK;
}
int fgpu_vector_zero(fgpu_vector* v) {
    if (!v) return FGPU_ERR_INVALID;
    FGPU_CUDA_CHECK(v->ctx, cudaMemsetAsync(v->d, 0, v->n * sizeof(double), v->ctx->stream));
    return FGPU_OK;
}
int fgpu_vector_device(const fgpu_vector* v, double** dptr) {
    if (!v || !dptr) return FGPU_ERR_INVALID;
    *dptr = v->d;
    return FGPU_OK;
}
int fgpu_vector_destroy(fgpu_vector* v) {
    if (!v) return FGPU_OK;
    cudaFree(v->d);
    delete v;
    return FGPU_OK;
}

int fgpu_assemble_vector(fgpu_ctx* ctx, const fgpu_space* V, const fgpu_rhs_desc* rhs, fgpu_vector* out, int accumulate) {
    FGPU_NO_CAPTURE(ctx, "assemble_vector");
    if (!ctx || !V || !rhs || !out || out->n != V->ndof) return set_err(ctx, FGPU_ERR_INVALID, "assemble_vector: bad arguments");
    if (V->mesh->cv == 8) {
        if (rhs->range != FGPU_RANGE_ELEMENTS) return set_err(ctx, FGPU_ERR_INVALID, "hexahedra: load vectors over elements(mesh) only");
        const int rc = launch_rhs_hex(ctx, V, rhs, out->d, accumulate);
        const int rc2 = finish(ctx);
        return rc ? rc : rc2;
    }
    if (rhs->range == FGPU_RANGE_BOUNDARY_FACES || rhs->range == FGPU_RANGE_MARKED_FACES) {
        if (V->mesh->d_ho) return set_err(ctx, FGPU_ERR_INVALID, "face integrals: flat faces only (the mesh has curved elements)");
        if (rhs->kind != FGPU_RHS_CONST && rhs->kind != FGPU_RHS_FACE)
            return set_err(ctx, FGPU_ERR_INVALID, "face integrals: loads FGPU_RHS_CONST or FGPU_RHS_FACE");
        const bool ft = rhs->kind == FGPU_RHS_FACE;
        const int rc = launch_face_load(ctx, V, rhs->range, rhs->range_xmax, rhs->c[0], ft ? rhs->c[1] : 0.0, ft ? rhs->c[2] : 0.0,
                                        out->d, accumulate);
        if (rc) return rc;
        return finish(ctx);
    }
    if (rhs->range != FGPU_RANGE_ELEMENTS) return set_err(ctx, FGPU_ERR_INVALID, "assemble_vector: bad range");
    if (rhs->kind == FGPU_RHS_FACE) return set_err(ctx, FGPU_ERR_INVALID, "assemble_vector: FGPU_RHS_FACE on face ranges only");
    if (V->mesh->d_ho) {
        const int rc = launch_rhs_ho(ctx, V, rhs, out->d, accumulate);
        const int rc2 = finish(ctx);
        return rc ? rc : rc2;
    }
    const int qdeg = form_qdeg(V, rhs->quad_degree);
    std::string err;
    DevTables* tab = get_dev_tables(V->order, qdeg, err);
    if (!tab) return set_err(ctx, FGPU_ERR_INVALID, err);
    double* work = nullptr;
    int rc = dev_alloc(ctx, &work, (size_t)V->mesh->nt * V->n * V->ncomp);
    if (rc) return rc;
    rc = launch_rhs(ctx, V, tab, rhs->kind, rhs->c, out->d, accumulate, work);
    int rc2 = finish(ctx);
    cudaFree(work);
    return rc ? rc : rc2;
}

int fgpu_dirichlet(fgpu_ctx* ctx, fgpu_matrix* A, fgpu_vector* rhs, int64_t ndofs, const int32_t* dofs,
                   const double* values, int mode, double diag) {
    FGPU_NO_CAPTURE(ctx, "dirichlet (use fgpu_bc_apply)");
    if (!ctx || !A || (ndofs > 0 && !dofs)) return set_err(ctx, FGPU_ERR_INVALID, "dirichlet: bad arguments");
    if (mode < 0 || mode > 2) return set_err(ctx, FGPU_ERR_INVALID, "dirichlet: bad mode");
    if (rhs && rhs->n != A->nrows) return set_err(ctx, FGPU_ERR_INVALID, "dirichlet: rhs size");
    std::vector<uint8_t> mask(A->nrows, 0);
    std::vector<double> g;
    if (values) g.assign(A->nrows, 0.0);
    for (int64_t k = 0; k < ndofs; ++k) {
        if (dofs[k] < 0 || dofs[k] >= A->nrows) return set_err(ctx, FGPU_ERR_OUT_OF_RANGE, "dirichlet: dof out of range");
        mask[dofs[k]] = 1;
        if (values) g[dofs[k]] = values[k];
    }
    uint8_t* dm = nullptr;
    double* dg = nullptr;
    int rc = dev_alloc(ctx, &dm, A->nrows);
    if (!rc && values) rc = dev_alloc(ctx, &dg, A->nrows);
    if (rc) { cudaFree(dm); return rc; }
    cudaMemcpyAsync(dm, mask.data(), A->nrows, cudaMemcpyHostToDevice, ctx->stream);
    if (values) cudaMemcpyAsync(dg, g.data(), A->nrows * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    rc = launch_dirichlet(ctx, A, rhs ? rhs->d : nullptr, dm, dg, mode, diag);
    int rc2 = finish(ctx);
    cudaFree(dm);
    cudaFree(dg);
    return rc ? rc : rc2;
}

int fgpu_matrix_mult(fgpu_ctx* ctx, const fgpu_matrix* A, const fgpu_vector* x, fgpu_vector* y) {
    if (!ctx || !A || !x || !y || x->n != A->nrows || y->n != A->nrows) return set_err(ctx, FGPU_ERR_INVALID, "mult: bad arguments");
    int rc = launch_spmv(ctx, A, x->d, y->d, 0.0, nullptr);
    if (rc) return rc;
    return finish(ctx);
}

int fgpu_solve_gmres(fgpu_ctx* ctx, const fgpu_matrix* A, fgpu_amg* amg, const fgpu_vector* b, fgpu_vector* x,
                     const fgpu_solver_cfg* cfg, int restart, fgpu_solve_stats* stats) {
    if (!ctx || !A || !b || !x || !cfg || b->n != A->nrows || x->n != A->nrows)
        return set_err(ctx, FGPU_ERR_INVALID, "solve_gmres: bad arguments");
    FGPU_NO_CAPTURE(ctx, "solve_gmres");
    int rc = finish(ctx);
    if (rc) return rc;
    if (A->ncomp != 1 && A->ncomp != 3) return set_err(ctx, FGPU_ERR_INVALID, "solve_gmres: bad matrix");
    rc = solve_gmres(ctx, A, amg, b->d, x->d, cfg, restart, stats);
    const int rc2 = finish(ctx);
    return rc ? rc : rc2;
}

int fgpu_solve_cg(fgpu_ctx* ctx, const fgpu_matrix* A, const fgpu_matrix* A32, const fgpu_vector* b, fgpu_vector* x,
                  const fgpu_solver_cfg* cfg, fgpu_solve_stats* stats) {
    if (!ctx || !A || !b || !x || !cfg || b->n != A->nrows || x->n != A->nrows)
        return set_err(ctx, FGPU_ERR_INVALID, "solve_cg: bad arguments");
    FGPU_NO_CAPTURE(ctx, "solve_cg");
    int rc = finish(ctx);
    if (rc) return rc;
    if (cfg->pc == FGPU_PC_GAMG) return set_err(ctx, FGPU_ERR_INVALID, "solve_cg: pc gamg runs through fgpu_solve_cg_amg");
    if (!cfg->mixed) return solve_pcg(ctx, A, b->d, x->d, cfg, stats);
    if (A->precision != FGPU_F64) return set_err(ctx, FGPU_ERR_INVALID, "mixed solve needs an FP64 matrix");
    fgpu_matrix* tmp = nullptr;
    const fgpu_matrix* a32 = A32;
    if (!a32) {
        rc = fgpu_matrix_create_like(A, FGPU_F32, &tmp);
        if (rc) return rc;
        rc = launch_convert_values(ctx, A, tmp);
        if (rc) { fgpu_matrix_destroy(tmp); return rc; }
        a32 = tmp;
    }
    rc = solve_pcg_mixed(ctx, A, a32, b->d, x->d, cfg, stats);
    if (tmp) fgpu_matrix_destroy(tmp);
    int rc2 = finish(ctx);
    return rc ? rc : rc2;
}

int fgpu_solve_cg_refine_dd(fgpu_ctx* ctx, const fgpu_matrix* A, fgpu_amg* amg, const fgpu_vector* b, fgpu_vector* x,
                            fgpu_vector* x_lo, const fgpu_solver_cfg* cfg, double inner_reduction, fgpu_solve_stats* stats) {
    if (!ctx || !A || !b || !x || !cfg || b->n != A->nrows || x->n != A->nrows || (x_lo && x_lo->n != A->nrows))
        return set_err(ctx, FGPU_ERR_INVALID, "solve_cg_refine_dd: bad arguments");
    FGPU_NO_CAPTURE(ctx, "solve_cg_refine_dd");
    if (A->precision != FGPU_F64) return set_err(ctx, FGPU_ERR_INVALID, "solve_cg_refine_dd: FP64 matrices");
    if (cfg->pc == FGPU_PC_GAMG && (!amg || cfg->mixed))
        return set_err(ctx, FGPU_ERR_INVALID, "solve_cg_refine_dd: pc gamg needs an AMG of A and a non-mixed inner solve");
    if (cfg->pc != FGPU_PC_GAMG && amg) return set_err(ctx, FGPU_ERR_INVALID, "solve_cg_refine_dd: an AMG is given but pc is not gamg");
    int rc = finish(ctx);
    if (rc) return rc;
    fgpu_matrix* tmp = nullptr;
    if (cfg->mixed) {
        rc = fgpu_matrix_create_like(A, FGPU_F32, &tmp);
        if (rc) return rc;
        rc = launch_convert_values(ctx, A, tmp);
        if (rc) { fgpu_matrix_destroy(tmp); return rc; }
    }
    rc = solve_refine_dd(ctx, A, tmp, cfg->pc == FGPU_PC_GAMG ? amg : nullptr, b->d, x->d, x_lo ? x_lo->d : nullptr, cfg,
                         inner_reduction, stats);
    if (tmp) fgpu_matrix_destroy(tmp);
    const int rc2 = finish(ctx);
    return rc ? rc : rc2;
}

int fgpu_solve_cg_amg(fgpu_ctx* ctx, const fgpu_matrix* A, fgpu_amg* amg, const fgpu_vector* b, fgpu_vector* x,
                      const fgpu_solver_cfg* cfg, fgpu_solve_stats* stats) {
    if (!ctx || !A || !amg || !b || !x || !cfg || b->n != A->nrows || x->n != A->nrows)
        return set_err(ctx, FGPU_ERR_INVALID, "solve_cg_amg: bad arguments");
    if (cfg->mixed) return set_err(ctx, FGPU_ERR_INVALID, "solve_cg_amg: the mixed solver takes Jacobi preconditioners only");
    FGPU_NO_CAPTURE(ctx, "solve_cg_amg");
    int rc = finish(ctx);
    if (rc) return rc;
    rc = solve_pcg(ctx, A, b->d, x->d, cfg, stats, amg);
    const int rc2 = finish(ctx);
    return rc ? rc : rc2;
}

// ---------------------------------------------------------------------------
int fgpu_bc_create(fgpu_ctx* ctx, int64_t n, int64_t ndofs, const int32_t* dofs, const double* values, fgpu_bc** out) {
    if (!ctx || !out || n <= 0 || ndofs < 0 || (ndofs > 0 && !dofs)) return set_err(ctx, FGPU_ERR_INVALID, "bc_create: bad arguments");
    FGPU_NO_CAPTURE(ctx, "bc_create");
    *out = nullptr;
    std::vector<uint8_t> mask(n, 0);
    std::vector<double> g;
    if (values) g.assign(n, 0.0);
    for (int64_t k = 0; k < ndofs; ++k) {
        if (dofs[k] < 0 || dofs[k] >= n) return set_err(ctx, FGPU_ERR_OUT_OF_RANGE, "bc_create: dof out of range");
        mask[dofs[k]] = 1;
        if (values) g[dofs[k]] = values[k];
    }
    fgpu_bc* bc = new (std::nothrow) fgpu_bc();
    if (!bc) return FGPU_ERR_ALLOC;
    bc->ctx = ctx;
    bc->n = n;
    int rc = dev_alloc(ctx, &bc->d_mask, n);
    if (!rc && values) rc = dev_alloc(ctx, &bc->d_g, n);
    if (rc) { fgpu_bc_destroy(bc); return rc; }
    cudaMemcpy(bc->d_mask, mask.data(), n, cudaMemcpyHostToDevice);
    if (values) cudaMemcpy(bc->d_g, g.data(), n * sizeof(double), cudaMemcpyHostToDevice);
    *out = bc;
    return FGPU_OK;
}

int fgpu_bc_apply(fgpu_ctx* ctx, const fgpu_bc* bc, fgpu_matrix* A, fgpu_vector* rhs, int mode, double diag) {
    if (!ctx || !bc || !A || bc->n != A->nrows || (rhs && rhs->n != A->nrows)) return set_err(ctx, FGPU_ERR_INVALID, "bc_apply: bad arguments");
    if (mode < 0 || mode > 2) return set_err(ctx, FGPU_ERR_INVALID, "bc_apply: bad mode");
    int rc = launch_dirichlet(ctx, A, rhs ? rhs->d : nullptr, bc->d_mask, bc->d_g, mode, diag);
    if (rc) return rc;
    return finish(ctx);
}

int fgpu_bc_destroy(fgpu_bc* bc) {
    if (!bc) return FGPU_OK;
    cudaFree(bc->d_mask);
    cudaFree(bc->d_g);
    delete bc;
    return FGPU_OK;
}

int fgpu_vector_axpby(fgpu_ctx* ctx, double a, const fgpu_vector* x, double b, fgpu_vector* y) {
    if (!ctx || !x || !y || x->n != y->n) return set_err(ctx, FGPU_ERR_INVALID, "vector_axpby: bad arguments");
    int rc = launch_axpby(ctx, y->n, a, x->d, b, y->d);
    if (rc) return rc;
    return finish(ctx);
}

int fgpu_vector_copy(fgpu_ctx* ctx, const fgpu_vector* src, fgpu_vector* dst) {
    if (!ctx || !src || !dst || src->n != dst->n) return set_err(ctx, FGPU_ERR_INVALID, "vector_copy: bad arguments");
    FGPU_CUDA_CHECK(ctx, cudaMemcpyAsync(dst->d, src->d, src->n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    return finish(ctx);
}

// ---------------------------------------------------------------------------
int fgpu_graph_begin(fgpu_ctx* ctx) {
    if (!ctx) return FGPU_ERR_INVALID;
    if (ctx->capturing) return set_err(ctx, FGPU_ERR_INVALID, "graph_begin: already capturing");
    int rc = finish(ctx);          // drain pending work and profiling events first
    if (rc) return rc;
    FGPU_CUDA_CHECK(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    ctx->capturing = 1;
    ctx->capture_launches0 = ctx->launches;
    return FGPU_OK;
}

int fgpu_graph_end(fgpu_ctx* ctx, fgpu_graph** out) {
    if (!ctx || !out) return FGPU_ERR_INVALID;
    if (!ctx->capturing) return set_err(ctx, FGPU_ERR_INVALID, "graph_end: not capturing");
    *out = nullptr;
    ctx->capturing = 0;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
    const int64_t nl = ctx->launches - ctx->capture_launches0;
    ctx->launches = ctx->capture_launches0;
    if (e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        return set_err(ctx, FGPU_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    }
    fgpu_graph* g = new (std::nothrow) fgpu_graph();
    if (!g) { cudaGraphDestroy(graph); return FGPU_ERR_ALLOC; }
    g->ctx = ctx;
    g->graph = graph;
    g->launches = nl;
    e = cudaGraphInstantiate(&g->exec, graph, 0);
    if (e != cudaSuccess) {
        fgpu_graph_destroy(g);
        return set_err(ctx, FGPU_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    }
    *out = g;
    return FGPU_OK;
}

int fgpu_graph_launch(fgpu_ctx* ctx, fgpu_graph* g, int count) {
    if (!ctx || !g || g->ctx != ctx || count < 0) return set_err(ctx, FGPU_ERR_INVALID, "graph_launch: bad arguments");
    FGPU_NO_CAPTURE(ctx, "graph_launch");
    for (int k = 0; k < count; ++k) {
        FGPU_CUDA_CHECK(ctx, cudaGraphLaunch(g->exec, ctx->stream));
        ctx->launches += g->launches;
    }
    return finish(ctx);
}

int fgpu_graph_destroy(fgpu_graph* g) {
    if (!g) return FGPU_OK;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
    return FGPU_OK;
}

int fgpu_host_dof_table(int64_t nv, int64_t nt, const int32_t* tets, int order, int ncomp, int32_t* l2g,
                        int64_t* ndof) {
    if (!tets || nv <= 0 || nt <= 0 || (ncomp != 1 && ncomp != 3)) return FGPU_ERR_INVALID;
    Topology topo;
    std::string err;
    if (!build_topology(nv, nt, tets, order, topo, err)) return FGPU_ERR_INVALID;
    if (ndof) *ndof = topo.nnodes * ncomp;
    if (l2g) {
        const int n = topo.n;
        for (int64_t e = 0; e < nt; ++e)
            for (int c = 0; c < ncomp; ++c)
                for (int l = 0; l < n; ++l)
                    l2g[e * n * ncomp + (int64_t)n * c + l] = topo.l2n[(size_t)e * n + l] * ncomp + c;
    }
    return FGPU_OK;
}

int fgpu_host_hex_dof_table(int64_t nv, int64_t nh, const int32_t* hexes, int order, int32_t* l2g, int64_t* ndof) {
    if (!hexes || nv <= 0 || nh <= 0) return FGPU_ERR_INVALID;
    for (int64_t k = 0; k < 8 * nh; ++k)
        if (hexes[k] < 0 || hexes[k] >= nv) return FGPU_ERR_OUT_OF_RANGE;
    Topology topo;
    std::string err;
    if (!build_hex_topology(nv, nh, hexes, order, topo, err)) return FGPU_ERR_INVALID;
    if (ndof) *ndof = topo.nnodes;
    if (l2g) std::copy(topo.l2n.begin(), topo.l2n.end(), l2g);
    return FGPU_OK;
}

int fgpu_host_hex_ref_tables(int order, int qdeg, double* nodes, double* qx, double* qw, double* phi, double* dphi, int* nq) {
    RefTables R;
    std::string err;
    if (!build_hex_ref_tables(order, qdeg, R, err)) return FGPU_ERR_INVALID;
    if (nq) *nq = R.Q;
    if (nodes) std::copy(R.nodes.begin(), R.nodes.end(), nodes);
    if (qx) std::copy(R.qx.begin(), R.qx.end(), qx);
    if (qw) std::copy(R.qw.begin(), R.qw.end(), qw);
    if (phi) std::copy(R.phi.begin(), R.phi.end(), phi);
    if (dphi) std::copy(R.dphi.begin(), R.dphi.end(), dphi);
    return FGPU_OK;
}

int fgpu_host_pattern(int64_t nv, int64_t nt, const int32_t* tets, int order, int ncomp, int64_t* ia, int32_t* ja,
                      int64_t* nnz) {
    if (!tets || !ia || nv <= 0 || nt <= 0 || (ncomp != 1 && ncomp != 3)) return FGPU_ERR_INVALID;
    Topology topo;
    NodePattern P;
    std::string err;
    if (!build_topology(nv, nt, tets, order, topo, err)) return FGPU_ERR_INVALID;
    if (!build_node_pattern(topo, nt, P, (int)std::max(1u, std::thread::hardware_concurrency()), err)) return FGPU_ERR_ALLOC;
    const int nc = ncomp;
    for (int64_t m = 0; m < P.nrows; ++m) {
        int64_t len = P.ia[m + 1] - P.ia[m];
        for (int c = 0; c < nc; ++c) ia[m * nc + c] = (int64_t)nc * nc * P.ia[m] + c * nc * len;
    }
    ia[P.nrows * nc] = (int64_t)nc * nc * P.nnz;
    if (nnz) *nnz = (int64_t)nc * nc * P.nnz;
    if (ja)
        for (int64_t m = 0; m < P.nrows; ++m) {
            int64_t b = P.ia[m], len = P.ia[m + 1] - b;
            for (int c = 0; c < nc; ++c) {
                int64_t o = (int64_t)nc * nc * b + c * nc * len;
                for (int64_t k = 0; k < len; ++k)
                    for (int d = 0; d < nc; ++d) ja[o + k * nc + d] = P.ja[b + k] * nc + d;
            }
        }
    return FGPU_OK;
}

int fgpu_host_ref_tables(int order, int qdeg, double* nodes, double* phi, double* dphi, double* S, double* M,
                         int* npts) {
    RefTables R;
    std::string err;
    if (!build_ref_tables(order, qdeg, R, err)) return FGPU_ERR_INVALID;
    if (npts) *npts = R.Q;
    if (nodes) std::memcpy(nodes, R.nodes.data(), R.nodes.size() * sizeof(double));
    if (phi) std::memcpy(phi, R.phi.data(), R.phi.size() * sizeof(double));
    if (dphi) std::memcpy(dphi, R.dphi.data(), R.dphi.size() * sizeof(double));
    if (S) std::memcpy(S, R.S.data(), R.S.size() * sizeof(double));
    if (M) std::memcpy(M, R.M.data(), R.M.size() * sizeof(double));
    return FGPU_OK;
}

int fgpu_host_df64_ops(int op, int64_t n, const double* a, const double* b, double* out) {
    if (!a || !out || n < 0) return FGPU_ERR_INVALID;
    for (int64_t i = 0; i < n; ++i) {
        df x = d2df(a[i]);
        df y = b ? d2df(b[i]) : df{0.0f, 0.0f};
        df r;
        switch (op) {
            case 0: r = x; break;
            case 1: r = df_add(x, y); break;
            case 2: r = df_mul(x, y); break;
            case 3: r = df_recip(x); break;
            case 4: r = df_sub(x, y); break;
            default: return FGPU_ERR_INVALID;
        }
        out[i] = df2d(r);
    }
    return FGPU_OK;
}

int fgpu_norms_sine(fgpu_ctx* ctx, const fgpu_space* V, const fgpu_vector* u, int quad_degree, double* l2, double* h1) {
    FGPU_NO_CAPTURE(ctx, "norms_sine");
    if (!ctx || !V || !u || !l2 || !h1 || u->n != V->ndof || V->ncomp != 1) return set_err(ctx, FGPU_ERR_INVALID, "norms: bad arguments");
    if (V->mesh->d_ho || V->mesh->cv != 4) return set_err(ctx, FGPU_ERR_INVALID, "norms: affine tetrahedra only");
    std::string err;
    DevTables* tab = get_dev_tables(V->order, quad_degree > 0 ? quad_degree : 2 * V->order, err);
    if (!tab) return set_err(ctx, FGPU_ERR_INVALID, err);
    int rc = finish(ctx);
    if (rc) return rc;
    return launch_norms_sine(ctx, V, tab, u->d, l2, h1);
}

int fgpu_prof_reset(fgpu_ctx* ctx) {
    if (!ctx) return FGPU_ERR_INVALID;
    FGPU_NO_CAPTURE(ctx, "prof_reset");
    finish(ctx);
    ctx->prof.clear();
    return FGPU_OK;
}

int fgpu_prof_get(fgpu_ctx* ctx, const char* name, int64_t* count, double* total_ms) {
    if (!ctx || !name) return FGPU_ERR_INVALID;
    FGPU_NO_CAPTURE(ctx, "prof_get");
    int rc = finish(ctx);
    if (rc) return rc;
    auto it = ctx->prof.find(name);
    if (count) *count = it == ctx->prof.end() ? 0 : it->second.count;
    if (total_ms) *total_ms = it == ctx->prof.end() ? 0.0 : it->second.total_ms;
    return FGPU_OK;
}

}  // extern "C"
