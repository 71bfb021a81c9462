// Sparse matrix-vector product and the CG / Jacobi solve behind
// a.solve(_rhs=l, _solution=u) with --ksp-type=cg --pc-type=jacobi
// (feelpp/feel/feelalg/solverlinearpetsc.cpp:490-570; PETSc KSPCG/PCJACOBI).
//
// Every CG iteration is five kernels (q = A p with the p.q partial sums;
// alpha; x, r, z updates with the r.r / r.z partial sums; beta and the
// convergence test; p update). Reductions are two-stage with a fixed grid, so
// results are bitwise reproducible. A device flag stops the iteration once
// ||r|| <= rtol ||b||; the host replays a captured CUDA graph of
// `check_every` iterations and polls the flag between replays.
//
// The mixed solver keeps FP64 for the outer residual b - A x and the
// solution update, and runs the inner CG on FP32 matrix values and FP32
// vectors (iterative refinement).
#include <cmath>
#include <cstring>
#include <vector>

#include "fgpu_core.h"

namespace fgpu {

static constexpr int kVecBlocks = 2 * 152;
static constexpr int kVecThreads = 256;

struct CGScalars {
    double rz, rz_new, pq, rr, bb, alpha, beta, tol2;
    int it, done, fail, pad;
};

template <int G>
__device__ __forceinline__ double group_sum(double v) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
template <int G>
__device__ __forceinline__ float group_sum(float v) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double block_sum(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    double s = 0;
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += sh[k];
    return s;  // valid on thread 0
}

// y = A x  (mode 0)  or  y = b - A x (mode 1); optional partial sum of dot(w, y) per block.
// AT: accumulation type of a row.
template <typename VT, typename XT, typename AT, int G>
__global__ void __launch_bounds__(256) spmv_kernel(int64_t nrows, const int64_t* __restrict__ ia, const int32_t* __restrict__ ja,
                                                  const VT* __restrict__ val, const XT* __restrict__ x, XT* __restrict__ y,
                                                  int mode, const XT* __restrict__ b, const XT* __restrict__ wdot,
                                                  double* __restrict__ partial, const CGScalars* __restrict__ sc) {
    if (sc && sc->done) return;
    __shared__ double sh[32];
    const int gpb = blockDim.x / G;
    const int g = threadIdx.x / G, lane = threadIdx.x % G;
    double dsum = 0;
    for (int64_t r0 = (int64_t)blockIdx.x * gpb; r0 < nrows; r0 += (int64_t)gridDim.x * gpb) {
        int64_t r = r0 + g;
        AT s = 0;
        if (r < nrows) {
            for (int64_t p = ia[r] + lane; p < ia[r + 1]; p += G) s += (AT)val[p] * (AT)x[ja[p]];
        }
        s = group_sum<G>(s);
        if (r < nrows && lane == 0) {
            AT v = mode == 1 ? (AT)b[r] - s : s;
            y[r] = (XT)v;
            if (wdot) dsum += (double)wdot[r] * (double)(XT)v;
        }
    }
    if (partial) {
        double t = block_sum(dsum, sh);
        if (threadIdx.x == 0) partial[blockIdx.x] = t;
    }
}

template <typename VT, typename XT>
__global__ void diag_inv_kernel(int64_t nrows, const int64_t* __restrict__ ia, const int32_t* __restrict__ ja,
                                const VT* __restrict__ val, XT* __restrict__ dinv, int use_pc) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
        double d = 0;
        for (int64_t p = ia[r]; p < ia[r + 1]; ++p)
            if (ja[p] == r) d = (double)val[p];
        dinv[r] = (XT)((use_pc && d != 0.0) ? 1.0 / d : 1.0);
    }
}

// r = b - A x done by spmv(mode 1); this sets z = dinv r, p = z and partial (r.r, r.z, b.b).
template <typename XT>
__global__ void cg_init_kernel(int64_t n, const XT* __restrict__ b, const XT* __restrict__ r, const XT* __restrict__ dinv,
                               XT* __restrict__ z, XT* __restrict__ p, double* __restrict__ partial) {
    __shared__ double sh[32];
    double rr = 0, rz = 0, bb = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        XT zi = dinv[i] * r[i];
        z[i] = zi;
        p[i] = zi;
        rr += (double)r[i] * (double)r[i];
        rz += (double)r[i] * (double)zi;
        bb += (double)b[i] * (double)b[i];
    }
    double a = block_sum(rr, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = a;
    double c = block_sum(rz, sh);
    if (threadIdx.x == 0) partial[gridDim.x + blockIdx.x] = c;
    double d = block_sum(bb, sh);
    if (threadIdx.x == 0) partial[2 * gridDim.x + blockIdx.x] = d;
}

__global__ void cg_init_scalars(const double* __restrict__ partial, int nb, double rtol, CGScalars* sc) {
    __shared__ double sh[32];
    double a = 0, c = 0, d = 0;
    for (int k = threadIdx.x; k < nb; k += blockDim.x) {
        a += partial[k];
        c += partial[nb + k];
        d += partial[2 * nb + k];
    }
    a = block_sum(a, sh);
    c = block_sum(c, sh);
    d = block_sum(d, sh);
    if (threadIdx.x == 0) {
        sc->rr = a; sc->rz = c; sc->bb = d;
        sc->tol2 = rtol * rtol * d;
        sc->it = 0; sc->fail = 0;
        sc->done = (a <= sc->tol2) ? 1 : 0;
    }
}

__global__ void cg_alpha_kernel(const double* __restrict__ partial, int nb, CGScalars* sc) {
    if (sc->done) return;
    __shared__ double sh[32];
    double a = 0;
    for (int k = threadIdx.x; k < nb; k += blockDim.x) a += partial[k];
    a = block_sum(a, sh);
    if (threadIdx.x == 0) {
        sc->pq = a;
        if (!(a > 0.0)) {
            sc->fail = 1;
            sc->done = 1;
        } else {
            sc->alpha = sc->rz / a;
        }
    }
}

template <typename XT>
__global__ void cg_update_kernel(int64_t n, XT* __restrict__ x, XT* __restrict__ r, XT* __restrict__ z,
                                 const XT* __restrict__ p, const XT* __restrict__ q, const XT* __restrict__ dinv,
                                 double* __restrict__ partial, const CGScalars* __restrict__ sc) {
    if (sc->done) return;
    __shared__ double sh[32];
    const XT alpha = (XT)sc->alpha;
    double rr = 0, rz = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] += alpha * p[i];
        XT ri = r[i] - alpha * q[i];
        r[i] = ri;
        XT zi = dinv[i] * ri;
        z[i] = zi;
        rr += (double)ri * (double)ri;
        rz += (double)ri * (double)zi;
    }
    double a = block_sum(rr, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = a;
    double c = block_sum(rz, sh);
    if (threadIdx.x == 0) partial[gridDim.x + blockIdx.x] = c;
}

__global__ void cg_beta_kernel(const double* __restrict__ partial, int nb, int maxit, CGScalars* sc) {
    if (sc->done) return;
    __shared__ double sh[32];
    double a = 0, c = 0;
    for (int k = threadIdx.x; k < nb; k += blockDim.x) {
        a += partial[k];
        c += partial[nb + k];
    }
    a = block_sum(a, sh);
    c = block_sum(c, sh);
    if (threadIdx.x == 0) {
        sc->rr = a;
        sc->it += 1;
        sc->beta = c / sc->rz;
        sc->rz = c;
        if (a <= sc->tol2) sc->done = 1;
        else if (sc->it >= maxit) { sc->done = 1; sc->fail = 2; }
    }
}

template <typename XT>
__global__ void cg_p_kernel(int64_t n, XT* __restrict__ p, const XT* __restrict__ z, const CGScalars* __restrict__ sc) {
    if (sc->done) return;
    const XT beta = (XT)sc->beta;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = z[i] + beta * p[i];
}

// ---------------------------------------------------------------------------
template <typename VT, typename XT, typename AT>
static void launch_spmv_t(cudaStream_t s, const fgpu_matrix* A, int G, const XT* x, XT* y, int mode, const XT* b,
                          const XT* wdot, double* partial, const CGScalars* sc, int blocks) {
    const VT* val = (const VT*)A->d_val;
    switch (G) {
        case 4: spmv_kernel<VT, XT, AT, 4><<<blocks, 256, 0, s>>>(A->nrows, A->d_ia, A->d_ja, val, x, y, mode, b, wdot, partial, sc); break;
        case 8: spmv_kernel<VT, XT, AT, 8><<<blocks, 256, 0, s>>>(A->nrows, A->d_ia, A->d_ja, val, x, y, mode, b, wdot, partial, sc); break;
        case 16: spmv_kernel<VT, XT, AT, 16><<<blocks, 256, 0, s>>>(A->nrows, A->d_ia, A->d_ja, val, x, y, mode, b, wdot, partial, sc); break;
        default: spmv_kernel<VT, XT, AT, 32><<<blocks, 256, 0, s>>>(A->nrows, A->d_ia, A->d_ja, val, x, y, mode, b, wdot, partial, sc); break;
    }
}

static int spmv_group(const fgpu_matrix* A) {
    double avg = A->nrows ? (double)A->nnz / (double)A->nrows : 1.0;
    if (avg <= 6) return 4;
    if (avg <= 24) return 8;
    if (avg <= 64) return 16;
    return 32;
}

static int spmv_blocks(const fgpu_matrix* A, int G) {
    int64_t need = (A->nrows + (256 / G) - 1) / (256 / G);
    return (int)std::max<int64_t>(1, std::min<int64_t>(need, 152 * 8));
}

int launch_spmv(fgpu_ctx* ctx, const fgpu_matrix* A, const double* x, double* y, double alpha_b, const double* b) {
    (void)alpha_b;
    int G = spmv_group(A);
    int blocks = spmv_blocks(A, G);
    PendingEvent ev;
    prof_begin(ctx, "spmv", ev);
    if (A->precision == FGPU_F32)
        launch_spmv_t<float, double, double>(ctx->stream, A, G, x, y, b ? 1 : 0, b, nullptr, nullptr, nullptr, blocks);
    else
        launch_spmv_t<double, double, double>(ctx->stream, A, G, x, y, b ? 1 : 0, b, nullptr, nullptr, nullptr, blocks);
    prof_end(ctx, ev);
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

// One PCG solve on A (values VT) with vectors XT. b, x are XT device vectors.
template <typename VT, typename XT>
static int pcg_core(fgpu_ctx* ctx, const fgpu_matrix* A, const XT* b, XT* x, double rtol, int maxit, int pc,
                    int check_every, int* iters, int* fail, double* rr_out, double* bb_out) {
    const int64_t n = A->nrows;
    cudaStream_t s = ctx->stream;
    XT *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *dinv = nullptr;
    double* partial = nullptr;
    CGScalars* sc = nullptr;
    CGScalars* hsc = nullptr;
    int rc = FGPU_OK;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    const int G = spmv_group(A);
    const int sblocks = spmv_blocks(A, G);
    const int nbp = std::max(sblocks, kVecBlocks);
    auto cleanup = [&]() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        cudaFree(r); cudaFree(z); cudaFree(p); cudaFree(q); cudaFree(dinv); cudaFree(partial); cudaFree(sc);
        if (hsc) cudaFreeHost(hsc);
    };
#define CK(call)                                                             \
    do {                                                                     \
        cudaError_t e_ = (call);                                             \
        if (e_ != cudaSuccess) {                                             \
            ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);   \
            cleanup();                                                       \
            return FGPU_ERR_CUDA;                                            \
        }                                                                    \
    } while (0)
    CK(cudaMalloc(&r, n * sizeof(XT)));
    CK(cudaMalloc(&z, n * sizeof(XT)));
    CK(cudaMalloc(&p, n * sizeof(XT)));
    CK(cudaMalloc(&q, n * sizeof(XT)));
    CK(cudaMalloc(&dinv, n * sizeof(XT)));
    CK(cudaMalloc(&partial, 3 * nbp * sizeof(double)));
    CK(cudaMalloc(&sc, sizeof(CGScalars)));
    CK(cudaMallocHost(&hsc, sizeof(CGScalars)));
    int dblocks = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, kVecBlocks));
    diag_inv_kernel<VT, XT><<<dblocks, 256, 0, s>>>(n, A->d_ia, A->d_ja, (const VT*)A->d_val, dinv, pc == FGPU_PC_JACOBI);
    launch_spmv_t<VT, XT, XT>(s, A, G, x, r, 1, b, nullptr, nullptr, nullptr, sblocks);
    cg_init_kernel<XT><<<kVecBlocks, kVecThreads, 0, s>>>(n, b, r, dinv, z, p, partial);
    cg_init_scalars<<<1, 256, 0, s>>>(partial, kVecBlocks, rtol, sc);
    ctx->launches += 4;
    CK(cudaGetLastError());
    // capture check_every iterations
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < check_every; ++k) {
        launch_spmv_t<VT, XT, XT>(s, A, G, p, q, 0, nullptr, p, partial, sc, sblocks);
        cg_alpha_kernel<<<1, 256, 0, s>>>(partial, sblocks, sc);
        cg_update_kernel<XT><<<kVecBlocks, kVecThreads, 0, s>>>(n, x, r, z, p, q, dinv, partial, sc);
        cg_beta_kernel<<<1, 256, 0, s>>>(partial, kVecBlocks, maxit, sc);
        cg_p_kernel<XT><<<kVecBlocks, kVecThreads, 0, s>>>(n, p, z, sc);
    }
    {
        cudaError_t e = cudaStreamEndCapture(s, &graph);
        if (e != cudaSuccess) { ctx->err = std::string("graph capture: ") + cudaGetErrorString(e); cleanup(); return FGPU_ERR_CUDA; }
    }
    CK(cudaGraphInstantiate(&exec, graph, 0));
    CK(cudaMemcpyAsync(hsc, sc, sizeof(CGScalars), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    int guard = 0;
    while (!hsc->done) {
        CK(cudaGraphLaunch(exec, s));
        ctx->launches += 5 * check_every;
        CK(cudaMemcpyAsync(hsc, sc, sizeof(CGScalars), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if (++guard > maxit / std::max(check_every, 1) + 2) break;
    }
    *iters = hsc->it;
    *fail = hsc->fail;
    *rr_out = hsc->rr;
    *bb_out = hsc->bb;
    cleanup();
#undef CK
    return rc;
}

template <typename A, typename B>
__global__ void cast_kernel(int64_t n, const A* __restrict__ a, B* __restrict__ b, double scale) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (B)((double)a[i] * scale);
}
__global__ void add_scaled_kernel(int64_t n, double* __restrict__ x, const float* __restrict__ d, double scale) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] += scale * (double)d[i];
}
__global__ void norm2_partial_kernel(int64_t n, const double* __restrict__ v, double* __restrict__ partial) {
    __shared__ double sh[32];
    double s = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) s += v[i] * v[i];
    double t = block_sum(s, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

static int device_norm2(fgpu_ctx* ctx, int64_t n, const double* v, double* partial, double* hpart, double* out) {
    norm2_partial_kernel<<<kVecBlocks, kVecThreads, 0, ctx->stream>>>(n, v, partial);
    ctx->launches++;
    FGPU_CUDA_CHECK(ctx, cudaMemcpyAsync(hpart, partial, kVecBlocks * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    FGPU_CUDA_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
    double s = 0;
    for (int k = 0; k < kVecBlocks; ++k) s += hpart[k];
    *out = std::sqrt(s);
    return FGPU_OK;
}

static int residual_norm(fgpu_ctx* ctx, const fgpu_matrix* A, const double* b, const double* x, double* r, double* partial,
                         double* hpart, double* out) {
    int G = spmv_group(A);
    int blocks = spmv_blocks(A, G);
    if (A->precision == FGPU_F64)
        launch_spmv_t<double, double, double>(ctx->stream, A, G, x, r, 1, b, nullptr, nullptr, nullptr, blocks);
    else
        launch_spmv_t<float, double, double>(ctx->stream, A, G, x, r, 1, b, nullptr, nullptr, nullptr, blocks);
    ctx->launches++;
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return device_norm2(ctx, A->nrows, r, partial, hpart, out);
}

int solve_pcg(fgpu_ctx* ctx, const fgpu_matrix* A, const double* d_b, double* d_x, const fgpu_solver_cfg* cfg,
              fgpu_solve_stats* st) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, ctx->stream);
    int iters = 0, fail = 0;
    double rr = 0, bb = 0;
    int ce = cfg->check_every > 0 ? cfg->check_every : 16;
    int rc = A->precision == FGPU_F64
                 ? pcg_core<double, double>(ctx, A, d_b, d_x, cfg->rtol, cfg->maxit, cfg->pc, ce, &iters, &fail, &rr, &bb)
                 : pcg_core<float, double>(ctx, A, d_b, d_x, cfg->rtol, cfg->maxit, cfg->pc, ce, &iters, &fail, &rr, &bb);
    cudaEventRecord(e1, ctx->stream);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != FGPU_OK) return rc;
    // final residual recomputed in FP64
    double *r = nullptr, *partial = nullptr, *hpart = nullptr;
    FGPU_CUDA_CHECK(ctx, cudaMalloc(&r, A->nrows * sizeof(double)));
    FGPU_CUDA_CHECK(ctx, cudaMalloc(&partial, kVecBlocks * sizeof(double)));
    FGPU_CUDA_CHECK(ctx, cudaMallocHost(&hpart, kVecBlocks * sizeof(double)));
    double rn = 0, bn = std::sqrt(bb);
    rc = residual_norm(ctx, A, d_b, d_x, r, partial, hpart, &rn);
    cudaFree(r); cudaFree(partial); cudaFreeHost(hpart);
    if (rc != FGPU_OK) return rc;
    if (st) {
        st->iterations = iters;
        st->outer = 1;
        st->rel_residual = bn > 0 ? rn / bn : 0.0;
        st->time_ms = ms;
    }
    if (fail == 1) { ctx->err = "CG breakdown: p.Ap <= 0 (matrix not SPD)"; return FGPU_ERR_BREAKDOWN; }
    if (fail == 2) { ctx->err = "CG reached maxit"; return FGPU_ERR_NOT_CONVERGED; }
    return FGPU_OK;
}

int solve_pcg_mixed(fgpu_ctx* ctx, const fgpu_matrix* A64, const fgpu_matrix* A32, const double* d_b, double* d_x,
                    const fgpu_solver_cfg* cfg, fgpu_solve_stats* st) {
    const int64_t n = A64->nrows;
    double *r = nullptr, *partial = nullptr, *hpart = nullptr;
    float *r32 = nullptr, *d32 = nullptr;
    auto cleanup = [&]() { cudaFree(r); cudaFree(partial); cudaFreeHost(hpart); cudaFree(r32); cudaFree(d32); };
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, ctx->stream);
#define CK(call)                                                             \
    do {                                                                     \
        cudaError_t e_ = (call);                                             \
        if (e_ != cudaSuccess) {                                             \
            ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);   \
            cleanup();                                                       \
            return FGPU_ERR_CUDA;                                            \
        }                                                                    \
    } while (0)
    CK(cudaMalloc(&r, n * sizeof(double)));
    CK(cudaMalloc(&partial, kVecBlocks * sizeof(double)));
    CK(cudaMallocHost(&hpart, kVecBlocks * sizeof(double)));
    CK(cudaMalloc(&r32, n * sizeof(float)));
    CK(cudaMalloc(&d32, n * sizeof(float)));
    double bn = 0;
    int rc = device_norm2(ctx, n, d_b, partial, hpart, &bn);
    if (rc) { cleanup(); return rc; }
    double inner = cfg->inner_rtol > 0 ? cfg->inner_rtol : 1e-4;
    int ce = cfg->check_every > 0 ? cfg->check_every : 16;
    int total = 0, outer = 0, fail = 0;
    double rn = 0;
    int vb = kVecBlocks;
    while (true) {
        rc = residual_norm(ctx, A64, d_b, d_x, r, partial, hpart, &rn);
        if (rc) { cleanup(); return rc; }
        if (bn == 0.0 || rn <= cfg->rtol * bn) break;
        if (outer >= 50 || total >= cfg->maxit) { fail = 2; break; }
        // inner: A32 d = r / ||r||
        cast_kernel<double, float><<<vb, 256, 0, ctx->stream>>>(n, r, r32, 1.0 / rn);
        CK(cudaMemsetAsync(d32, 0, n * sizeof(float), ctx->stream));
        ctx->launches++;
        int it = 0, f = 0;
        double rr = 0, bb = 0;
        rc = pcg_core<float, float>(ctx, A32, r32, d32, inner, cfg->maxit - total, cfg->pc, ce, &it, &f, &rr, &bb);
        if (rc) { cleanup(); return rc; }
        total += it;
        ++outer;
        add_scaled_kernel<<<vb, 256, 0, ctx->stream>>>(n, d_x, d32, rn);
        ctx->launches++;
        if (f == 1) { fail = 1; break; }
    }
    cudaEventRecord(e1, ctx->stream);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cleanup();
#undef CK
    if (st) {
        st->iterations = total;
        st->outer = outer;
        st->rel_residual = bn > 0 ? rn / bn : 0.0;
        st->time_ms = ms;
    }
    if (fail == 1) { ctx->err = "CG breakdown in the inner FP32 solve"; return FGPU_ERR_BREAKDOWN; }
    if (fail == 2) { ctx->err = "mixed CG did not reach rtol"; return FGPU_ERR_NOT_CONVERGED; }
    return FGPU_OK;
}

}  // namespace fgpu
