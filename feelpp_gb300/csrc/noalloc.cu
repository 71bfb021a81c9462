// Load-vector assembly that performs no device memory allocation.
//
// Some callers cannot allocate device memory at the time they assemble: a
// host application whose memory manager (a PETSc/Kokkos pool, a framework's
// caching allocator) already owns the device memory and forbids allocations
// outside it, or a caller that must not allocate after initialisation
// (fixed-latency time stepping, code paths that may later be captured into
// CUDA graphs, where cudaMalloc is not allowed). For them this file gives
// fgpu_assemble_vector_noalloc: the same element and gather kernels as
// fgpu_assemble_vector, with the per-element work buffer and the basis /
// quadrature tables held in file-scope __device__ arrays instead of cudaMalloc'ed
// memory. The caller passes the input (a function space already on the device)
// and the output (a device vector).
//
// Limits and behaviour:
//  * the scratch holds FGPU_NOALLOC_MAX_ELEMENT_VALUES doubles (16 MiB); larger
//    problems (elements x local dofs x components) are rejected with
//    FGPU_ERR_INVALID; every GPU that loads the library keeps the 16 MiB (plus
//    the ~64 KiB table) until the process exits;
//  * the first call on a device sets it up (looks up the arrays' device
//    addresses with cudaGetSymbolAddress and copies the tables with cudaMemcpy);
//    make that first call before any stream capture;
//  * all calls share the one scratch array and it keeps the last call's
//    contents; every call overwrites the part it reads, so nothing needs
//    clearing, but calls that overlap on the GPU (different streams, or
//    different host threads on one device) race on it and must be serialised
//    by the caller.
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "fgpu_core.h"
#include "quad_tet.h"

namespace fgpu {
int launch_rhs_raw(cudaStream_t stream, const fgpu_space* V, int Q, const double* qx, const double* qw,
                   const double* phi, int fkind, const double* fc, double* d_out, int accumulate, double* d_work,
                   std::string& err);
}

using namespace fgpu;

namespace {

constexpr int kNoallocTableDoubles = 8192;   // phi, points and weights for orders 1-3, degrees 1-8

static __device__ __align__(256) double g_noalloc_scratch[FGPU_NOALLOC_MAX_ELEMENT_VALUES];
static __device__ __align__(256) double g_noalloc_tables[kNoallocTableDoubles];

struct TableSlot {
    int Q = 0;
    size_t phi = 0, qx = 0, qw = 0;   // offsets into g_noalloc_tables
};

struct DeviceState {
    double* scratch = nullptr;        // device address of g_noalloc_scratch
    double* tables = nullptr;         // device address of g_noalloc_tables
    TableSlot slot[4][kMaxTetRuleDegree + 1];
};

std::mutex g_state_mutex;
std::map<int, DeviceState> g_state;

// Set-up, once per device, with that device current.
int setup_device(int dev, DeviceState*& out, std::string& err) {
    std::lock_guard<std::mutex> lock(g_state_mutex);
    auto it = g_state.find(dev);
    if (it != g_state.end()) {
        out = &it->second;
        return FGPU_OK;
    }
    DeviceState st;
    cudaError_t e = cudaGetSymbolAddress((void**)&st.scratch, g_noalloc_scratch);
    if (e != cudaSuccess) { err = std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e); return FGPU_ERR_CUDA; }
    e = cudaGetSymbolAddress((void**)&st.tables, g_noalloc_tables);
    if (e != cudaSuccess) { err = std::string("cudaGetSymbolAddress(tables): ") + cudaGetErrorString(e); return FGPU_ERR_CUDA; }
    std::vector<double> host;
    for (int order = 1; order <= 3; ++order)
        for (int q = 1; q <= kMaxTetRuleDegree; ++q) {
            RefTables R;
            if (!build_ref_tables(order, q, R, err)) return FGPU_ERR_INVALID;
            TableSlot& s = st.slot[order][q];
            s.Q = R.Q;
            s.phi = host.size(); host.insert(host.end(), R.phi.begin(), R.phi.end());
            s.qx = host.size(); host.insert(host.end(), R.qx.begin(), R.qx.end());
            s.qw = host.size(); host.insert(host.end(), R.qw.begin(), R.qw.end());
        }
    if (host.size() > (size_t)kNoallocTableDoubles) { err = "internal: no-alloc table too small"; return FGPU_ERR_INVALID; }
    e = cudaMemcpy(st.tables, host.data(), host.size() * sizeof(double), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { err = std::string("table copy: ") + cudaGetErrorString(e); return FGPU_ERR_CUDA; }
    auto res = g_state.emplace(dev, st);
    out = &res.first->second;
    return FGPU_OK;
}

}  // namespace

extern "C" int fgpu_assemble_vector_noalloc(const fgpu_space* V, const fgpu_rhs_desc* rhs, double* d_out,
                                            int accumulate, void* stream) {
    if (!V || !rhs || !d_out) return FGPU_ERR_INVALID;
    fgpu_ctx* ctx = V->ctx;
    if (rhs->range != FGPU_RANGE_ELEMENTS) { ctx->err = "noalloc: element integrals only"; return FGPU_ERR_INVALID; }
    if (V->mesh->cv != 4) { ctx->err = "noalloc: tetrahedral meshes only (the space is on hexahedra)"; return FGPU_ERR_INVALID; }
    if (V->mesh->d_ho) { ctx->err = "noalloc: affine elements only"; return FGPU_ERR_INVALID; }
    if (rhs->kind != FGPU_RHS_SINE && rhs->kind != FGPU_RHS_CONST && rhs->kind != FGPU_RHS_CONST_VEC) {
        ctx->err = "noalloc: sources FGPU_RHS_SINE, FGPU_RHS_CONST and FGPU_RHS_CONST_VEC only (FGPU_RHS_FACE is a face-range load)";
        return FGPU_ERR_INVALID;
    }
    const int qdeg = rhs->quad_degree > 0 ? rhs->quad_degree : 2 * V->order;
    if (qdeg < 1 || qdeg > kMaxTetRuleDegree) { ctx->err = "noalloc: quadrature degree must be in [1, 8]"; return FGPU_ERR_INVALID; }
    const int64_t need = V->mesh->nt * (int64_t)V->n * V->ncomp;
    if (need > (int64_t)FGPU_NOALLOC_MAX_ELEMENT_VALUES) {
        ctx->err = "noalloc: elements x local dofs x components = " + std::to_string(need) +
                   " exceeds FGPU_NOALLOC_MAX_ELEMENT_VALUES (" + std::to_string((long long)FGPU_NOALLOC_MAX_ELEMENT_VALUES) + ")";
        return FGPU_ERR_INVALID;
    }
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) { ctx->err = "noalloc: no current device"; return FGPU_ERR_CUDA; }
    if (prev != ctx->device && cudaSetDevice(ctx->device) != cudaSuccess) { ctx->err = "noalloc: cannot select the space's device"; return FGPU_ERR_CUDA; }
    DeviceState* st = nullptr;
    std::string err;
    int rc = setup_device(ctx->device, st, err);
    if (rc == FGPU_OK) {
        const TableSlot& s = st->slot[V->order][qdeg];
        rc = launch_rhs_raw((cudaStream_t)stream, V, s.Q, st->tables + s.qx, st->tables + s.qw, st->tables + s.phi,
                            rhs->kind, rhs->c, d_out, accumulate, st->scratch, err);
        if (rc != FGPU_OK) err = "noalloc: " + err;
        else ctx->launches += 2;
    }
    if (prev != ctx->device) cudaSetDevice(prev);
    if (rc != FGPU_OK) ctx->err = err;
    return rc;
}
