// Batched assembly of many independent problems (C-ABI fgpu_batch_*).
//
// A Feel++ application that assembles many independent problems loops over
// them, each `form2 = integrate(elements(mesh_k), expr_k)` running its own
// element loop (feelpp/feel/feelvf/integrator.hpp:975-1238 per mesh). Here the
// problems' device data (patterns, incidence lists, position tables,
// coefficient records, CSR values) stay where each matrix owns them; the batch
// holds a device table of per-problem descriptors and runs the assembly of all
// problems in a fixed number of launches: when the element buffers and gather
// maps fit in device memory, the two-phase path (geometry, element matrices,
// gather map: three launches; each matrix gets the bits FGPU_ALGO_TWO_PHASE
// gives it alone), else the fused row-owner gather as a persistent kernel with
// a device work queue (two launches; the bits of FGPU_ALGO_GATHER). The launch
// shape (threads per block, and rows per work-queue grab for the fused path)
// is picked by timing the candidates on the first '=' assembly and kept.
#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "fgpu_core.h"

using namespace fgpu;

struct fgpu_batch {
    fgpu_ctx* ctx = nullptr;
    int nprob = 0;
    int f32 = 0;
    int acc_floats = 0;              // per-warp staging floats (max over problems of EPB * maxrow * width)
    int64_t total_rows = 0, total_elems = 0, total_nnz = 0, total_groups = 0;
    bool two_phase = false;          // element buffers + gather maps (else the fused row-owner gather)
    BatchProblem* d_probs = nullptr;
    int64_t* d_row_off = nullptr;
    int64_t* d_elem_off = nullptr;
    int64_t* d_grp_off = nullptr;    // groups of 32 elements per problem (two-phase element kernel)
    int64_t* d_nz_off = nullptr;
    unsigned long long* d_counter = nullptr;
    BatchLaunch launch;
    bool tuned = false;
    std::vector<fgpu_matrix*> mats;
    std::vector<double> tune_ms;     // timings of the candidates (diagnostics)
};

namespace {

int epb_of(int order) { return order == 1 ? 8 : order == 2 ? 3 : 1; }

int batch_err(fgpu_ctx* ctx, int code, const char* msg) {
    if (ctx) ctx->err = msg;
    return code;
}

int batch_finish(fgpu_ctx* ctx) {
    if (ctx->capturing) return FGPU_OK;
    int hst = 0;
    cudaError_t e = cudaMemcpyAsync(&hst, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { ctx->err = std::string("batch: ") + cudaGetErrorString(e); return FGPU_ERR_CUDA; }
    if (hst) {
        cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream);
        cudaStreamSynchronize(ctx->stream);
        if (hst & kStatusBadElement) return batch_err(ctx, FGPU_ERR_BAD_ELEMENT, "degenerate element: |det K| <= 0 or non-finite");
        if (hst & kStatusRowOverflow) return batch_err(ctx, FGPU_ERR_INVALID, "pattern row longer than the staging buffer");
        return batch_err(ctx, FGPU_ERR_CUDA, "device status error in batch assembly");
    }
    return FGPU_OK;
}

int run_gather(fgpu_batch* b, const BatchLaunch& cfg, int accumulate) {
    fgpu_ctx* ctx = b->ctx;
    if (b->two_phase)
        return launch_batch_two_phase(ctx, b->nprob, b->d_probs, b->d_grp_off, b->total_groups, b->d_nz_off, b->total_nnz, b->f32,
                                      cfg.threads, accumulate);
    return launch_batch_gather(ctx, b->nprob, b->d_probs, b->d_row_off, b->total_rows, b->f32, b->acc_floats, b->d_counter, cfg,
                               accumulate);
}

int run(fgpu_batch* b, const BatchLaunch& cfg, int accumulate) {
    if (!b->two_phase) {             // the two-phase element kernel forms the coefficient records itself
        int rc = launch_batch_geometry(b->ctx, b->nprob, b->d_probs, b->d_elem_off, b->total_elems);
        if (rc) return rc;
    }
    return run_gather(b, cfg, accumulate);
}

// Time each launch shape once (plus one warm-up) and keep the fastest.
int tune(fgpu_batch* b) {
    fgpu_ctx* ctx = b->ctx;
    const int threads[] = {128, 256};
    const int chunks[] = {4, 16, 64};
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best = 1e300;
    BatchLaunch pick = b->launch;
    const int save = ctx->profile;
    ctx->profile = 0;
    int rc = FGPU_OK;
    for (int t : threads) {
        for (int c : chunks) {
            if (b->two_phase && c != chunks[0]) continue;   // the two-phase gather has no work queue
            BatchLaunch cfg;
            cfg.threads = t;
            cfg.chunk = c;
            rc = run_gather(b, cfg, 0);
            if (rc) break;
            cudaEventRecord(e0, ctx->stream);
            rc = run_gather(b, cfg, 0);
            cudaEventRecord(e1, ctx->stream);
            if (rc) break;
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            b->tune_ms.push_back(ms);
            if (ms < best) { best = ms; pick = cfg; }
        }
        if (rc) break;
    }
    ctx->profile = save;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    b->launch = pick;
    b->tuned = true;
    return FGPU_OK;
}

}  // namespace

extern "C" {

int fgpu_batch_create(fgpu_ctx* ctx, int nprob, fgpu_matrix* const* mats, const fgpu_form_desc* descs,
                      const double* const* d_kappa, fgpu_batch** out) {
    if (!ctx || nprob <= 0 || !mats || !descs || !out) return batch_err(ctx, FGPU_ERR_INVALID, "batch_create: bad arguments");
    *out = nullptr;
    std::vector<BatchProblem> probs(nprob);
    std::vector<int64_t> row_off(nprob + 1, 0), elem_off(nprob + 1, 0), grp_off(nprob + 1, 0);
    int f32 = -1, acc = 0;
    for (int k = 0; k < nprob; ++k) {
        const fgpu_matrix* A = mats[k];
        const fgpu_form_desc& f = descs[k];
        if (!A) return batch_err(ctx, FGPU_ERR_INVALID, "batch_create: null matrix");
        if (A->ctx != ctx) return batch_err(ctx, FGPU_ERR_INVALID, "batch_create: matrix of another context");
        if (A->space->mesh->d_ho || A->space->mesh->cv != 4)
            return batch_err(ctx, FGPU_ERR_INVALID, "batch_create: affine tetrahedra only");
        const fgpu_space* V = A->space;
        if (f.kind != FGPU_FORM_LAPLACE_MASS || A->ncomp != 1)
            return batch_err(ctx, FGPU_ERR_INVALID, "batch_create: batches hold scalar Laplace/mass forms");
        if (V->order < 1 || V->order > 3) return batch_err(ctx, FGPU_ERR_INVALID, "batch_create: orders 1-3");
        if (f.quad_degree != 0 && f.quad_degree != 2 * V->order)
            return batch_err(ctx, FGPU_ERR_INVALID, "batch_create: quadrature degree must be the default 2p");
        if (!V->d_pos || !A->pattern) return batch_err(ctx, FGPU_ERR_INVALID, "batch_create: matrix without position table");
        if (A->pattern->max_row > 255) return batch_err(ctx, FGPU_ERR_INVALID, "batch_create: pattern rows longer than 255");
        const int mf32 = A->precision == FGPU_F32 ? 1 : 0;
        if (f32 >= 0 && mf32 != f32) return batch_err(ctx, FGPU_ERR_INVALID, "batch_create: all matrices need one precision");
        f32 = mf32;
        if (A->coef_cap < V->mesh->nt * 8) {
            cudaFree(A->d_coef);
            fgpu_matrix* Am = mats[k];
            Am->d_coef = nullptr;
            Am->coef_cap = 0;
            if (cudaMalloc(&Am->d_coef, (size_t)V->mesh->nt * 8 * sizeof(double)) != cudaSuccess)
                return batch_err(ctx, FGPU_ERR_ALLOC, "batch_create: record allocation failed");
            Am->coef_cap = V->mesh->nt * 8;
        }
        BatchProblem& P = probs[k];
        std::memset(&P, 0, sizeof(P));
        P.order = V->order;
        P.n = V->n;
        P.maxrow = A->pattern->max_row;
        P.row0 = row_off[k];
        P.nrows = A->nrows;
        P.elem0 = elem_off[k];
        P.nt = V->mesh->nt;
        P.sia = A->pattern->d_ia;
        P.inc_ptr = V->d_inc_ptr;
        P.inc = V->d_inc;
        P.pos = V->d_pos;
        P.xyz = V->mesh->d_xyz;
        P.tets = V->mesh->d_tets;
        P.kappa = d_kappa ? d_kappa[k] : nullptr;
        P.kappa_c = f.kappa;
        P.mass = f.mass;
        P.rec = reinterpret_cast<float4*>(A->d_coef);
        P.val = A->d_val;
        row_off[k + 1] = row_off[k] + A->nrows;
        elem_off[k + 1] = elem_off[k] + V->mesh->nt;
        grp_off[k + 1] = grp_off[k] + (V->mesh->nt + 31) / 32;
        acc = std::max(acc, epb_of(V->order) * P.maxrow * (mf32 ? 1 : 2));
    }
    // two-phase when every space's gather map and every matrix's element buffer exist or fit
    bool two_phase = true;
    {
        size_t need = 0;
        for (int k = 0; k < nprob; ++k) {
            const fgpu_matrix* A = mats[k];
            const fgpu_space* V = A->space;
            const int n = V->n;
            const size_t kb = (size_t)V->mesh->nt * (n * (n + 1) / 2) * (f32 ? 4 : 8);
            if (A->kbuf_bytes < kb) need += kb;
            if (!V->d_gptr) need += ((size_t)V->mesh->nt * n * n + (size_t)A->pattern->nnz * 2 + 1) * sizeof(uint32_t);
            if ((int64_t)V->mesh->nt * n * n >= (int64_t)UINT32_MAX) two_phase = false;
        }
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) { cudaGetLastError(); two_phase = false; }
        if (need + need / 10 >= free_b) two_phase = false;
    }
    std::vector<int64_t> nz_off(nprob + 1, 0);
    for (int k = 0; k < nprob && two_phase; ++k) {
        fgpu_matrix* A = mats[k];
        fgpu_space* V = A->space;
        const int n = V->n;
        const size_t kb = (size_t)V->mesh->nt * (n * (n + 1) / 2) * (f32 ? 4 : 8);
        if (!V->d_gptr && launch_build_gather_map(ctx, V) != FGPU_OK) { two_phase = false; break; }
        if (A->kbuf_bytes < kb) {
            cudaFree(A->d_kbuf);
            A->d_kbuf = nullptr;
            A->kbuf_bytes = 0;
            if (cudaMalloc(&A->d_kbuf, kb) != cudaSuccess) { cudaGetLastError(); two_phase = false; break; }
            A->kbuf_bytes = kb;
        }
        probs[k].nz0 = nz_off[k];
        probs[k].nnz = A->pattern->nnz;
        probs[k].gptr = V->d_gptr;
        probs[k].gidx = V->d_gidx;
        probs[k].kbuf = A->d_kbuf;
        nz_off[k + 1] = nz_off[k] + A->pattern->nnz;
    }
    ctx->err.clear();
    fgpu_batch* b = new (std::nothrow) fgpu_batch();
    if (!b) return FGPU_ERR_ALLOC;
    b->two_phase = two_phase;
    b->total_nnz = two_phase ? nz_off[nprob] : 0;
    b->ctx = ctx;
    b->nprob = nprob;
    b->f32 = f32;
    b->acc_floats = (acc + 3) & ~3;
    b->total_rows = row_off[nprob];
    b->total_elems = elem_off[nprob];
    b->total_groups = grp_off[nprob];
    b->mats.assign(mats, mats + nprob);
    cudaError_t e = cudaMalloc(&b->d_probs, nprob * sizeof(BatchProblem));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_row_off, (nprob + 1) * sizeof(int64_t));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_elem_off, (nprob + 1) * sizeof(int64_t));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_grp_off, (nprob + 1) * sizeof(int64_t));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_counter, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_nz_off, (nprob + 1) * sizeof(int64_t));
    if (e == cudaSuccess) e = cudaMemcpy(b->d_nz_off, nz_off.data(), (nprob + 1) * sizeof(int64_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_probs, probs.data(), nprob * sizeof(BatchProblem), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_row_off, row_off.data(), (nprob + 1) * sizeof(int64_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_elem_off, elem_off.data(), (nprob + 1) * sizeof(int64_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_grp_off, grp_off.data(), (nprob + 1) * sizeof(int64_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        ctx->err = std::string("batch_create: ") + cudaGetErrorString(e);
        fgpu_batch_destroy(b);
        return FGPU_ERR_ALLOC;
    }
    *out = b;
    return FGPU_OK;
}

int fgpu_batch_assemble(fgpu_ctx* ctx, fgpu_batch* b, int accumulate) {
    if (!ctx || !b || b->ctx != ctx) return batch_err(ctx, FGPU_ERR_INVALID, "batch_assemble: bad arguments");
    if (!b->tuned && !accumulate && !ctx->capturing) {
        // the candidates overwrite the values ('='), so tuning runs only on '=' calls
        int rc = b->two_phase ? FGPU_OK : launch_batch_geometry(ctx, b->nprob, b->d_probs, b->d_elem_off, b->total_elems);
        if (!rc) rc = tune(b);
        if (rc) return rc;
    }
    int rc = run(b, b->launch, accumulate);
    if (rc) return rc;
    return batch_finish(ctx);
}

int fgpu_batch_set_launch(fgpu_batch* b, int threads, int chunk) {
    if (!b || (threads != 128 && threads != 256) || chunk < 1) return FGPU_ERR_INVALID;
    b->launch.threads = threads;
    b->launch.chunk = chunk;
    b->tuned = true;
    return FGPU_OK;
}

int fgpu_batch_set_algo(fgpu_batch* b, int algo) {
    if (!b) return FGPU_ERR_INVALID;
    if (algo == FGPU_ALGO_GATHER) {
        b->two_phase = false;
    } else if (algo == FGPU_ALGO_TWO_PHASE || algo == FGPU_ALGO_AUTO) {
        if (b->total_nnz == 0) return batch_err(b->ctx, FGPU_ERR_INVALID, "batch: no two-phase buffers (device memory)");
        b->two_phase = true;
    } else {
        return batch_err(b->ctx, FGPU_ERR_INVALID, "batch: algorithm must be GATHER, TWO_PHASE or AUTO");
    }
    b->tuned = false;
    return FGPU_OK;
}

int fgpu_batch_get_launch(const fgpu_batch* b, int* threads, int* chunk, int* tuned) {
    if (!b) return FGPU_ERR_INVALID;
    if (threads) *threads = b->launch.threads;
    if (chunk) *chunk = b->two_phase ? 0 : b->launch.chunk;      // 0: two-phase batch (no work queue)
    if (tuned) *tuned = b->tuned ? 1 : 0;
    return FGPU_OK;
}

int fgpu_batch_destroy(fgpu_batch* b) {
    if (!b) return FGPU_OK;
    cudaFree(b->d_probs);
    cudaFree(b->d_row_off);
    cudaFree(b->d_elem_off);
    cudaFree(b->d_grp_off);
    cudaFree(b->d_counter);
    cudaFree(b->d_nz_off);
    delete b;
    return FGPU_OK;
}

}  // extern "C"
