// Sparse matrix-vector product and the CG / Jacobi solve behind
// a.solve(_rhs=l, _solution=u) with --ksp-type=cg --pc-type=jacobi
// (feelpp/feel/feelalg/solverlinearpetsc.cpp:490-570; PETSc KSPCG/PCJACOBI).
//
// Number formats (one templated CG, three policies):
//  * F64  : binary64 values and vectors, native FP64 arithmetic - the plain
//           FP64 path (default for FP64 matrices);
//  * DF64 : double-float (binary32 pairs, ~48 bits) on the FP32 pipes, values
//           converted once per solve with integer operations - faster on GB300
//           (FP64 runs at 1/71 of FP32) but limited to ~2^-48 relative accuracy
//           per operation, so only for moderately conditioned systems;
//  * F32  : binary32 values and vectors (dot products accumulated in df64) -
//           the inner solver of the mixed method, which refines with the
//           binary64 residual b - A x and binary64 solution updates
//           (iterative refinement).
//
// Every CG iteration is three kernels (q = A p with the p.q partial sums; x, r,
// z updates with alpha and the r.r / r.z partial sums; p update with beta and
// the convergence test); each block finishes the two-stage reductions itself
// over a fixed grid in a fixed order, so all blocks see the same scalars and
// results are bitwise reproducible. A device flag stops the iteration once
// ||r|| <= rtol ||b||; the host replays a captured CUDA graph of `check_every`
// iterations and polls the flag between replays.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "cg_driver.cuh"
#include "df64.h"
#include "fgpu_core.h"

namespace fgpu {

// ---------------------------------------------------------------------------
// conversions and small vector kernels
// ---------------------------------------------------------------------------
__global__ void d2df_kernel(int64_t n, const double* __restrict__ a, float2* __restrict__ b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = dfpack(d2df(a[i]));
}
__global__ void df2d_kernel(int64_t n, const float2* __restrict__ a, double* __restrict__ b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = df2d(dfun(a[i]));
}
// ---------------------------------------------------------------------------
template <class PL>
static void launch_spmv_t(cudaStream_t s, const fgpu_matrix* A, const typename PL::V* val, int G, const typename PL::S* x,
                          typename PL::S* y, int mode, const typename PL::S* b, const typename PL::S* wdot,
                          typename PL::D* partial, const CGScalars<PL>* sc, int blocks) {
    switch (G) {
        case 2: spmv_kernel<PL, 2><<<blocks, 256, 0, s>>>(A->nrows, A->d_ia, A->d_ja, val, x, y, mode, b, wdot, partial, sc); break;
        case 4: spmv_kernel<PL, 4><<<blocks, 256, 0, s>>>(A->nrows, A->d_ia, A->d_ja, val, x, y, mode, b, wdot, partial, sc); break;
        case 8: spmv_kernel<PL, 8><<<blocks, 256, 0, s>>>(A->nrows, A->d_ia, A->d_ja, val, x, y, mode, b, wdot, partial, sc); break;
        case 16: spmv_kernel<PL, 16><<<blocks, 256, 0, s>>>(A->nrows, A->d_ia, A->d_ja, val, x, y, mode, b, wdot, partial, sc); break;
        default: spmv_kernel<PL, 32><<<blocks, 256, 0, s>>>(A->nrows, A->d_ia, A->d_ja, val, x, y, mode, b, wdot, partial, sc); break;
    }
}

// lanes per row: short tails of the shuffle reduction matter (FP64 adds run on the slow pipe)
static int spmv_group(const fgpu_matrix* A) {
    double avg = A->nrows ? (double)A->nnz / (double)A->nrows : 1.0;
    if (avg <= 40) return 4;
    if (avg <= 120) return 8;
    return 16;
}

static int spmv_blocks(const fgpu_matrix* A, int G) {
    int64_t need = (A->nrows + (256 / G) - 1) / (256 / G);
    return (int)std::max<int64_t>(1, std::min<int64_t>(need, 152 * 16));
}

// without per-block partial sums the grid does not change the result: one block per 256 / G rows
// (P2 64^3 y = A x: 0.40 against 0.43 ms with the capped grid; 8 lanes per row took 0.48 ms, and each
// lane's entries in explicit batches of 8 with their loads issued together 0.53 ms: 64 registers)
static int spmv_blocks_uncapped(const fgpu_matrix* A, int G) {
    return (int)std::max<int64_t>(1, (A->nrows + (256 / G) - 1) / (256 / G));
}

// lanes per row of y = A x: two for rows of up to 40 entries (one FP64 shuffle-add per lane; P2 64^3:
// 0.36 against 0.40 ms with four), else as in the solver
static int mult_group(const fgpu_matrix* A) {
    const double avg = A->nrows ? (double)A->nnz / (double)A->nrows : 1.0;
    return avg <= 40 ? 2 : spmv_group(A);
}


int launch_spmv(fgpu_ctx* ctx, const fgpu_matrix* A, const double* x, double* y, double alpha_b, const double* b) {
    (void)alpha_b;
    if (A->precision != FGPU_F64) {
        ctx->err = "y = A x with binary64 vectors needs an FP64 matrix";
        return FGPU_ERR_INVALID;
    }
    const int G = mult_group(A);
    PendingEvent ev;
    prof_begin(ctx, "spmv", ev);
    launch_spmv_t<PolF64>(ctx->stream, A, (const double*)A->d_val, G, x, y, b ? 1 : 0, b, nullptr, nullptr, nullptr,
                          spmv_blocks_uncapped(A, G));
    prof_end(ctx, ev);
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

// ===========================================================================
// SELL-C-sigma layout for the CG products (C = 32 rows per slice, rows sorted
// by length inside windows of sigma = 256 rows; entries column-major inside a
// slice). One thread per row: coalesced loads, no cross-lane reductions, and
// the lanes of a warp run the same number of iterations (the slice's longest
// row), so the FP64 pipe issues full warps.
// ===========================================================================


static constexpr int kSellC = 32;
static constexpr int kSellSigma = 256;

// one block (256 threads) per window: bitonic sort of (length desc, row asc)
__global__ void sell_sort_kernel(int64_t nrows, const int64_t* __restrict__ ia, int32_t* __restrict__ perm,
                                 int32_t* __restrict__ slice_len) {
    __shared__ int32_t klen[kSellSigma];
    __shared__ int32_t krow[kSellSigma];
    const int64_t w0 = (int64_t)blockIdx.x * kSellSigma;
    const int t = threadIdx.x;
    const int64_t r = w0 + t;
    klen[t] = r < nrows ? (int32_t)(ia[r + 1] - ia[r]) : -1;
    krow[t] = r < nrows ? (int32_t)r : INT32_MAX;
    __syncthreads();
    for (int k = 2; k <= kSellSigma; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            const int ixj = t ^ j;
            if (ixj > t) {
                // "a before b" when a is longer, ties by row id
                const bool a_first = klen[t] > klen[ixj] || (klen[t] == klen[ixj] && krow[t] < krow[ixj]);
                const bool up = (t & k) == 0;
                if (up != a_first) {
                    int32_t tl = klen[t], tr = krow[t];
                    klen[t] = klen[ixj]; krow[t] = krow[ixj];
                    klen[ixj] = tl; krow[ixj] = tr;
                }
            }
            __syncthreads();
        }
    if (r < nrows) perm[r] = krow[t];
    if ((t % kSellC) == 0) {
        const int64_t s = (w0 + t) / kSellC;
        if (w0 + t < nrows) slice_len[s] = klen[t] < 0 ? 0 : klen[t];
    }
}

__global__ void sell_fill_kernel(int64_t nrows, const int64_t* __restrict__ ia, const int32_t* __restrict__ ja,
                                 const int32_t* __restrict__ perm, const int64_t* __restrict__ slice_ptr,
                                 const int32_t* __restrict__ slice_len, int32_t* __restrict__ col, int32_t* __restrict__ src) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ((nrows + kSellC - 1) / kSellC) * kSellC;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = i / kSellC;
        const int lane = (int)(i - s * kSellC);
        const int L = slice_len[s];
        const int64_t base = slice_ptr[s] + lane;
        int32_t row = -1;
        int64_t b = 0, e = 0;
        if (i < nrows) {
            row = perm[i];
            b = ia[row];
            e = ia[row + 1];
        }
        for (int k = 0; k < L; ++k) {
            const int64_t p = b + k;
            const bool real = row >= 0 && p < e;
            col[base + (int64_t)k * kSellC] = real ? ja[p] : (row >= 0 ? row : 0);
            src[base + (int64_t)k * kSellC] = real ? (int32_t)p : -1;
        }
    }
}

int build_sell(fgpu_ctx* ctx, const fgpu_matrix* A, std::shared_ptr<SellLayout>& out) {
    if (A->nnz >= ((int64_t)1 << 31)) { ctx->err = "SELL layout: more than 2^31 entries"; return FGPU_ERR_INVALID; }
    auto L = std::make_shared<SellLayout>();
    L->nrows = A->nrows;
    L->nslices = (A->nrows + kSellC - 1) / kSellC;
    const int64_t nwin = (A->nrows + kSellSigma - 1) / kSellSigma;
    FGPU_CUDA_CHECK(ctx, cudaMalloc(&L->d_perm, A->nrows * sizeof(int32_t)));
    FGPU_CUDA_CHECK(ctx, cudaMalloc(&L->d_slice_len, L->nslices * sizeof(int32_t)));
    FGPU_CUDA_CHECK(ctx, cudaMalloc(&L->d_slice_ptr, (L->nslices + 1) * sizeof(int64_t)));
    sell_sort_kernel<<<(int)nwin, kSellSigma, 0, ctx->stream>>>(A->nrows, A->d_ia, L->d_perm, L->d_slice_len);
    ctx->launches++;
    std::vector<int32_t> hlen(L->nslices);
    FGPU_CUDA_CHECK(ctx, cudaMemcpyAsync(hlen.data(), L->d_slice_len, L->nslices * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    FGPU_CUDA_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
    std::vector<int64_t> hptr(L->nslices + 1, 0);
    for (int64_t s = 0; s < L->nslices; ++s) hptr[s + 1] = hptr[s] + (int64_t)hlen[s] * kSellC;
    L->nstored = hptr[L->nslices];
    FGPU_CUDA_CHECK(ctx, cudaMemcpyAsync(L->d_slice_ptr, hptr.data(), hptr.size() * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
    FGPU_CUDA_CHECK(ctx, cudaMalloc(&L->d_col, L->nstored * sizeof(int32_t)));
    FGPU_CUDA_CHECK(ctx, cudaMalloc(&L->d_src, L->nstored * sizeof(int32_t)));
    const int64_t tot = L->nslices * kSellC;
    sell_fill_kernel<<<(int)std::max<int64_t>(1, std::min<int64_t>((tot + 255) / 256, 152 * 32)), 256, 0, ctx->stream>>>(
        A->nrows, A->d_ia, A->d_ja, L->d_perm, L->d_slice_ptr, L->d_slice_len, L->d_col, L->d_src);
    ctx->launches++;
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    FGPU_CUDA_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
    out = L;
    return FGPU_OK;
}


// SELL values from CSR values of the same type (padding = 0)
template <class PL>
__global__ void sell_values_kernel(int64_t nstored, const int32_t* __restrict__ src, const typename PL::V* __restrict__ csr,
                                   typename PL::V* __restrict__ out) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nstored; j += (int64_t)gridDim.x * blockDim.x)
        out[j] = src[j] >= 0 ? csr[src[j]] : PL::st(PL::zero());
}

// y = A x (mode 0) or y = b - A x (mode 1) on the SELL layout, one thread per row,
// optional per-block partial of dot(w, y)
template <class PL>
__global__ void __launch_bounds__(256) sell_spmv_kernel(int64_t nrows, int64_t nslices, const int32_t* __restrict__ perm,
                                                       const int64_t* __restrict__ slice_ptr, const int32_t* __restrict__ slice_len,
                                                       const int32_t* __restrict__ col, const typename PL::V* __restrict__ val,
                                                       const typename PL::S* __restrict__ x, typename PL::S* __restrict__ y, int mode,
                                                       const typename PL::S* __restrict__ b, const typename PL::S* __restrict__ wdot,
                                                       typename PL::D* __restrict__ partial, const CGScalars<PL>* __restrict__ sc) {
    if (sc && sc->done) return;
    __shared__ typename PL::D sh[32];
    typename PL::D dsum = PL::dzero();
    const int64_t total = nslices * kSellC;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = i / kSellC;
        const int L = slice_len[s];
        const int64_t base = slice_ptr[s] + (i - s * kSellC);
        typename PL::D accd = PL::dzero();     // row sums in the dot-product type (see spmv_kernel)
        // four entries' loads issued together (memory-level parallelism), summed in entry order
        int k = 0;
        for (; k + 4 <= L; k += 4) {
            const int64_t j = base + (int64_t)k * kSellC;
            const int32_t c0 = col[j], c1 = col[j + kSellC], c2 = col[j + 2 * kSellC], c3 = col[j + 3 * kSellC];
            const typename PL::V v0 = val[j], v1 = val[j + kSellC], v2 = val[j + 2 * kSellC], v3 = val[j + 3 * kSellC];
            const typename PL::S x0 = x[c0], x1 = x[c1], x2 = x[c2], x3 = x[c3];
            accd = PL::dmadd(accd, PL::ldv(v0), PL::ld(x0));
            accd = PL::dmadd(accd, PL::ldv(v1), PL::ld(x1));
            accd = PL::dmadd(accd, PL::ldv(v2), PL::ld(x2));
            accd = PL::dmadd(accd, PL::ldv(v3), PL::ld(x3));
        }
        for (; k < L; ++k) {
            const int64_t j = base + (int64_t)k * kSellC;
            accd = PL::dmadd(accd, PL::ldv(val[j]), PL::ld(x[col[j]]));
        }
        const typename PL::A acc = PL::from_d(accd);
        if (i < nrows) {
            const int32_t row = perm[i];
            const typename PL::S v = PL::st(mode == 1 ? PL::sub(PL::ld(b[row]), acc) : acc);
            y[row] = v;
            if (wdot) dsum = PL::dmadd(dsum, PL::ld(wdot[row]), PL::ld(v));
        }
    }
    if (partial) {
        const typename PL::D t = block_sum<PL>(dsum, sh);
        if (threadIdx.x == 0) partial[blockIdx.x] = t;
    }
}

static int sell_blocks(const SellLayout& L) {
    const int64_t total = L.nslices * kSellC;
    return (int)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 152 * 8));
}


// ---------------------------------------------------------------------------
// SpMV autotuner for the CG: CSR with G lanes per row (G in 4, 8, 16, 32) or
// the SELL layout, timed with CUDA events on the actual matrix (1 warm-up + 3
// timed products per candidate) the first time a (device, number format, rows,
// nonzeros) combination is solved; the choice is cached (0 = SELL, else G).
// ---------------------------------------------------------------------------
static std::mutex g_tune_mutex;
static std::map<std::tuple<std::string, int, int, int64_t, int64_t>, int> g_spmv_tune;

template <class PL>
struct SpmvPlan {
    int G = 4;                         // 0: SELL
    const SellLayout* sell = nullptr;
    typename PL::V* sval = nullptr;    // SELL values (owned)
    ~SpmvPlan() { cudaFree(sval); }
    void launch(cudaStream_t s, const fgpu_matrix* A, const typename PL::V* val, const typename PL::S* x, typename PL::S* y,
                int mode, const typename PL::S* b, const typename PL::S* wdot, typename PL::D* partial,
                const CGScalars<PL>* sc) const {
        if (G == 0)
            sell_spmv_kernel<PL><<<sell_blocks(*sell), 256, 0, s>>>(sell->nrows, sell->nslices, sell->d_perm, sell->d_slice_ptr,
                                                                   sell->d_slice_len, sell->d_col, sval, x, y, mode, b, wdot,
                                                                   partial, sc);
        else
            launch_spmv_t<PL>(s, A, val, G, x, y, mode, b, wdot, partial, sc, spmv_blocks(A, G));
    }
    int blocks(const fgpu_matrix* A) const { return G == 0 ? sell_blocks(*sell) : spmv_blocks(A, G); }
};

template <class PL>
static int plan_spmv(fgpu_ctx* ctx, const fgpu_matrix* A, const typename PL::V* val, const typename PL::S* x,
                     typename PL::S* y, SpmvPlan<PL>& plan) {
    const auto key = std::make_tuple(ctx->tune_file, ctx->device, PL::id, A->nrows, A->nnz);
    const std::string skey = "spmv|" + tune_device_key(ctx->device) + "|pol" + std::to_string(PL::id) + "|" +
                             std::to_string(A->nrows) + "x" + std::to_string(A->nnz);
    int choice = -1;
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        auto it = g_spmv_tune.find(key);
        if (it != g_spmv_tune.end()) choice = it->second;
    }
    std::vector<int> tv;
    if (choice == -1 && tune_lookup(ctx->tune_file, skey, tv) && tv.size() == 1) choice = tv[0];
    if (choice == -1 && ctx->tune != 0) choice = spmv_group(A);
    // SELL layout and values (needed to time it, and to use it)
    bool have_sell = false;
    if (choice == -1 || choice == 0) {
        if (!A->sell) {
            int rc = build_sell(ctx, A, A->sell);
            if (rc != FGPU_OK) A->sell.reset();
        }
        if (A->sell && cudaMalloc(&plan.sval, A->sell->nstored * sizeof(typename PL::V)) == cudaSuccess) {
            const int64_t ns = A->sell->nstored;
            sell_values_kernel<PL><<<(int)std::max<int64_t>(1, std::min<int64_t>((ns + 255) / 256, 152 * 32)), 256, 0, ctx->stream>>>(
                ns, A->sell->d_src, val, plan.sval);
            ctx->launches++;
            plan.sell = A->sell.get();
            have_sell = true;
        } else {
            plan.sval = nullptr;
        }
    }
    if (choice == -1) {
        // median of 5 individually timed products per candidate (a sum of a few products let one slow
        // repetition on a shared GPU decide)
        cudaEvent_t ev[6];
        for (auto& e : ev) cudaEventCreate(&e);
        float best_ms = 1e30f;
        int best = spmv_group(A);
        const int cands[5] = {4, 8, 16, 32, 0};
        for (int c : cands) {
            if (c == 0 && !have_sell) continue;
            SpmvPlan<PL> trial;
            trial.G = c;
            trial.sell = plan.sell;
            trial.sval = plan.sval;
            trial.launch(ctx->stream, A, val, x, y, 0, nullptr, nullptr, nullptr, nullptr);
            for (int rep = 0; rep < 5; ++rep) {
                cudaEventRecord(ev[rep], ctx->stream);
                trial.launch(ctx->stream, A, val, x, y, 0, nullptr, nullptr, nullptr, nullptr);
            }
            cudaEventRecord(ev[5], ctx->stream);
            cudaEventSynchronize(ev[5]);
            trial.sval = nullptr;  // not owned by the trial
            float t[5];
            for (int rep = 0; rep < 5; ++rep) cudaEventElapsedTime(&t[rep], ev[rep], ev[rep + 1]);
            std::sort(t, t + 5);
            ctx->launches += 6;
            if (t[2] < best_ms) { best_ms = t[2]; best = c; }
        }
        for (auto& e : ev) cudaEventDestroy(e);
        choice = best;
        tune_record(ctx->tune_file, skey, {choice});
    }
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        g_spmv_tune[key] = choice;
    }
    if (choice == 0 && !have_sell) choice = spmv_group(A);
    plan.G = choice;
    if (choice != 0 && plan.sval) {
        cudaFree(plan.sval);
        plan.sval = nullptr;
    }
    return FGPU_OK;
}

// One PCG solve with policy PL on values `val`, right-hand side b and solution x
// (initial guess on entry), all in the policy's formats.
// PCG on an assembled matrix: Jacobi diagonal from the matrix, SpMV kernel
// picked by the tuner, iterations in cg_run (cg_driver.cuh).
template <class PL>
static int pcg_core(fgpu_ctx* ctx, const fgpu_matrix* A, const typename PL::V* val, const typename PL::S* b,
                    typename PL::S* x, const CgOptions& o, int pc, CgResult* res, const RefreshFn<PL>* refresh = nullptr,
                    fgpu_amg* amg = nullptr) {
    typedef typename PL::S S;
    const int64_t n = A->nrows;
    const int vb = vec_blocks(n);
    S *dinv = nullptr, *tmp = nullptr;
    if (cudaMalloc(&dinv, n * sizeof(S)) != cudaSuccess || cudaMalloc(&tmp, n * sizeof(S)) != cudaSuccess) {
        cudaFree(dinv);
        ctx->err = "CG: allocation failed";
        return FGPU_ERR_ALLOC;
    }
    diag_inv_kernel<PL><<<vb, 256, 0, ctx->stream>>>(n, A->d_ia, A->d_ja, val, dinv, pc != FGPU_PC_NONE);
    ctx->launches++;
    SpmvPlan<PL> plan;
    plan_spmv<PL>(ctx, A, val, dinv, tmp, plan);
    cudaFree(tmp);
    CgOperator<PL> op;
    op.apply = [&plan, A, val, ctx](const S* xx, S* yy, typename PL::D* partial, const CGScalars<PL>* sc) {
        plan.launch(ctx->stream, A, val, xx, yy, 0, nullptr, partial ? xx : nullptr, partial, sc);
    };
    op.npq = plan.blocks(A);
    op.launches = 1;
    op.graph = true;
    PcHook<PL> hook;
    if (amg) hook = amg_pc_hook<PL>(amg);
    const int rc = cg_run<PL>(ctx, n, op, dinv, b, x, o, res, refresh, amg ? &hook : nullptr);
    cudaFree(dinv);
    return rc;
}

// ||b - A x||_2 in native FP64 (binary64 values and vectors); r receives b - A x.
static int f64_residual(fgpu_ctx* ctx, const fgpu_matrix* A, const double* b, const double* x, double* r, double* partial,
                        double* hpart, double* out) {
    const int G = spmv_group(A);
    launch_spmv_t<PolF64>(ctx->stream, A, (const double*)A->d_val, G, x, r, 1, b, nullptr, nullptr, nullptr, spmv_blocks(A, G));
    const int vb = vec_blocks(A->nrows);
    norm2_partial_kernel<<<vb, 256, 0, ctx->stream>>>(A->nrows, r, partial);
    ctx->launches += 2;
    FGPU_CUDA_CHECK(ctx, cudaMemcpyAsync(hpart, partial, vb * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    FGPU_CUDA_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
    double s = 0;
    for (int k = 0; k < vb; ++k) s += hpart[k];
    *out = std::sqrt(s);
    return FGPU_OK;
}

struct Scratch64 {
    double* r = nullptr;
    double* partial = nullptr;
    double* hpart = nullptr;
    ~Scratch64() { cudaFree(r); cudaFree(partial); cudaFreeHost(hpart); }
    bool alloc(int64_t n) {
        return cudaMalloc(&r, n * sizeof(double)) == cudaSuccess && cudaMalloc(&partial, kVecBlocks * sizeof(double)) == cudaSuccess &&
               cudaMallocHost(&hpart, kVecBlocks * sizeof(double)) == cudaSuccess;
    }
};

int solve_pcg(fgpu_ctx* ctx, const fgpu_matrix* A, const double* d_b, double* d_x, const fgpu_solver_cfg* cfg,
              fgpu_solve_stats* st, fgpu_amg* amg) {
    if (A->precision != FGPU_F64) { ctx->err = "solve needs an FP64 matrix"; return FGPU_ERR_INVALID; }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, ctx->stream);
    CgOptions opt = cg_options(cfg);
    opt.delta = 0.0;             // replace the residual only when the recurrence claims convergence
    CgResult res;
    const int64_t n = A->nrows;
    double rn = 0;
    int rc = FGPU_OK;
    // Residual replacement: when the recurrence residual claims convergence, the
    // true residual b - A x is computed; if it misses rtol (the recurrence drifts
    // on stiff systems) it replaces r and the iteration goes on from p = z.
    Scratch64 R;
    if (!R.alloc(n)) { ctx->err = "solve: allocation failed"; return FGPU_ERR_ALLOC; }
    double bn0 = 0;
    {
        const int vb = vec_blocks(n);
        norm2_partial_kernel<<<vb, 256, 0, ctx->stream>>>(n, d_b, R.partial);
        cudaMemcpyAsync(R.hpart, R.partial, vb * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
        cudaStreamSynchronize(ctx->stream);
        for (int k = 0; k < vb; ++k) bn0 += R.hpart[k];
        bn0 = std::sqrt(bn0);
    }
    int stagnant = 0;
    double rlast = 0;
    auto check_true = [&](const double* xd, double* rout, bool* conv) -> int {
        double r2n = 0;
        const int r2 = f64_residual(ctx, A, d_b, xd, rout, R.partial, R.hpart, &r2n);
        if (r2) return r2;
        *conv = r2n <= cfg->rtol * bn0;
        stagnant = (rlast > 0 && r2n > 0.5 * rlast) ? stagnant + 1 : 0;
        rlast = r2n;
        if (!*conv && stagnant >= 2) return kRefreshStagnated;
        return FGPU_OK;
    };
    RefreshFn<PolF64> refresh64 = [&](double* xd, double* rd, bool* conv) -> int { return check_true(xd, rd, conv); };
    double* xtmp = nullptr;
    RefreshFn<PolDF64> refresh_df = [&](float2* xd, float2* rd, bool* conv) -> int {
        if (!xtmp && cudaMalloc(&xtmp, n * sizeof(double)) != cudaSuccess) { cudaGetLastError(); ctx->err = "solve: allocation failed"; return FGPU_ERR_ALLOC; }
        df2d_kernel<<<vec_blocks(n), 256, 0, ctx->stream>>>(n, xd, xtmp);
        const int r2 = check_true(xtmp, R.r, conv);
        if (r2) return r2;
        d2df_kernel<<<vec_blocks(n), 256, 0, ctx->stream>>>(n, R.r, rd);
        ctx->launches += 2;
        return FGPU_OK;
    };
    if (cfg->arith == FGPU_ARITH_DF64) {
        float2 *val = nullptr, *b = nullptr, *x = nullptr;
        if (cudaMalloc(&val, A->nnz * sizeof(float2)) != cudaSuccess || cudaMalloc(&b, n * sizeof(float2)) != cudaSuccess ||
            cudaMalloc(&x, n * sizeof(float2)) != cudaSuccess) {
            rc = FGPU_ERR_ALLOC;
            ctx->err = "df64 solve: allocation failed";
        } else {
            int64_t nb = std::min<int64_t>((A->nnz + 255) / 256, 152 * 32);
            d2df_kernel<<<(int)std::max<int64_t>(nb, 1), 256, 0, ctx->stream>>>(A->nnz, (const double*)A->d_val, val);
            d2df_kernel<<<vec_blocks(n), 256, 0, ctx->stream>>>(n, d_b, b);
            d2df_kernel<<<vec_blocks(n), 256, 0, ctx->stream>>>(n, d_x, x);
            ctx->launches += 3;
            rc = pcg_core<PolDF64>(ctx, A, val, b, x, opt, cfg->pc, &res, &refresh_df, amg);
            if (rc == FGPU_OK) {
                df2d_kernel<<<vec_blocks(n), 256, 0, ctx->stream>>>(n, x, d_x);
                ctx->launches++;
            }
        }
        cudaFree(val); cudaFree(b); cudaFree(x);
    } else {
        rc = pcg_core<PolF64>(ctx, A, (const double*)A->d_val, d_b, d_x, opt, cfg->pc, &res, &refresh64, amg);
    }
    cudaFree(xtmp);
    if (rc == FGPU_OK)    // final residual recomputed in binary64 from the matrix
        rc = f64_residual(ctx, A, d_b, d_x, R.r, R.partial, R.hpart, &rn);
    cudaEventRecord(e1, ctx->stream);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != FGPU_OK) return rc;
    const double bn = bn0;
    int fail = res.fail;
    if (fail == 0 && rn > cfg->rtol * bn) fail = 2;      // maxit with the recurrence short of rtol
    if (fail == 3) fail = 2;                             // the true residual stopped decreasing
    if (st) {
        st->iterations = res.iters;
        st->outer = 1;
        st->rel_residual = bn > 0 ? rn / bn : 0.0;
        st->time_ms = ms;
        st->eig_max = res.lmax;
        st->fallback = 0;
        st->fallback_iterations = 0;
    }
    if (fail == 1) { ctx->err = "CG breakdown: p.Ap <= 0 (matrix not SPD)"; return FGPU_ERR_BREAKDOWN; }
    if (fail == 2) { ctx->err = "CG reached maxit"; return FGPU_ERR_NOT_CONVERGED; }
    return FGPU_OK;
}

int solve_pcg_mixed(fgpu_ctx* ctx, const fgpu_matrix* A64, const fgpu_matrix* A32, const double* d_b, double* d_x,
                    const fgpu_solver_cfg* cfg, fgpu_solve_stats* st) {
    // Mixed precision with reliable updates: binary32 CG on A32 for the
    // correction (scaled to a unit initial residual), binary64 solution and
    // binary64 residual replacement. A replacement is accepted only when it
    // lowers the binary64 residual (the solution is the best iterate so far);
    // a rejected one, or two in a row that do not halve it, end the binary32
    // phase (stagnation) and the solve finishes in FP64 from the best iterate.
    const int64_t n = A64->nrows;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, ctx->stream);
    int rc = FGPU_OK;
    int fail = 0, fallback = 0, fallback_its = 0;
    CgResult res;
    double rn = 0, bn = 0;
    {
        Scratch64 S;
        float *r32 = nullptr, *x32 = nullptr;
        double *xc = nullptr, *rc64 = nullptr;
        if (!S.alloc(n) || cudaMalloc(&r32, n * sizeof(float)) != cudaSuccess || cudaMalloc(&x32, n * sizeof(float)) != cudaSuccess ||
            cudaMalloc(&xc, n * sizeof(double)) != cudaSuccess || cudaMalloc(&rc64, n * sizeof(double)) != cudaSuccess) {
            cudaGetLastError();
            ctx->err = "mixed solve: allocation failed";
            rc = FGPU_ERR_ALLOC;
        }
        double* rbest = S.r;      // binary64 residual of the current solution
        double* rcand = rc64;
        if (rc == FGPU_OK) {
            const int vb = vec_blocks(n);
            norm2_partial_kernel<<<vb, 256, 0, ctx->stream>>>(n, d_b, S.partial);
            cudaMemcpyAsync(S.hpart, S.partial, vb * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
            cudaStreamSynchronize(ctx->stream);
            double s2 = 0;
            for (int k = 0; k < vb; ++k) s2 += S.hpart[k];
            bn = std::sqrt(s2);
            rc = f64_residual(ctx, A64, d_b, d_x, rbest, S.partial, S.hpart, &rn);
            if (rc == FGPU_OK && !(bn == 0.0 || rn <= cfg->rtol * bn)) {
                const double scale = rn;   // binary32 system scaled to a unit initial residual
                d2f_scaled_kernel<<<vb, 256, 0, ctx->stream>>>(n, rbest, r32, 1.0 / scale);
                cudaMemsetAsync(x32, 0, n * sizeof(float), ctx->stream);
                int stagnant = 0;
                // candidate x + scale x_lo; accepted when its binary64 residual is lower
                auto fold = [&](float* xl, bool* accepted) -> int {
                    cudaMemcpyAsync(xc, d_x, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream);
                    fold_kernel<<<vb, 256, 0, ctx->stream>>>(n, xc, xl, scale);
                    ctx->launches++;
                    double rn_c = 0;
                    const int r2 = f64_residual(ctx, A64, d_b, xc, rcand, S.partial, S.hpart, &rn_c);
                    if (r2) return r2;
                    *accepted = rn_c < rn;
                    if (*accepted) {
                        stagnant = rn_c > 0.5 * rn ? stagnant + 1 : 0;
                        cudaMemcpyAsync(d_x, xc, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream);
                        std::swap(rbest, rcand);
                        rn = rn_c;
                    }
                    return FGPU_OK;
                };
                RefreshFn<PolF32> refresh = [&](float* xl, float* rl, bool* conv) -> int {
                    bool ok = false;
                    const int r2 = fold(xl, &ok);
                    if (r2) return r2;
                    d2f_scaled_kernel<<<vb, 256, 0, ctx->stream>>>(n, rbest, rl, 1.0 / scale);
                    ctx->launches++;
                    *conv = rn <= cfg->rtol * bn;
                    if (!*conv && (!ok || stagnant >= 2)) return kRefreshStagnated;
                    return FGPU_OK;
                };
                CgOptions o32 = cg_options(cfg);
                o32.rtol = cfg->rtol * bn / rn;   // the binary32 system starts from a unit residual
                rc = pcg_core<PolF32>(ctx, A32, (const float*)A32->d_val, r32, x32, o32, cfg->pc, &res, &refresh);
                if (rc == FGPU_OK && !res.true_conv) {
                    bool ok = false;
                    if (res.fail != 3) rc = fold(x32, &ok);       // what the last iterations added, if it helps
                    if (rc == FGPU_OK && rn > cfg->rtol * bn) {
                        if (res.fail != 0 && res.iters < cfg->maxit) {
                            // binary32 breakdown or stagnation (A32 = fl32(A) and binary32
                            // vectors too coarse at this conditioning): finish in FP64
                            // from the best iterate
                            fgpu_solver_cfg c64 = *cfg;
                            c64.mixed = 0;
                            c64.arith = FGPU_ARITH_F64;
                            c64.maxit = cfg->maxit - res.iters;
                            fgpu_solve_stats s64{};
                            const int rc64 = solve_pcg(ctx, A64, d_b, d_x, &c64, &s64);
                            fallback_its = s64.iterations;
                            fallback = 1;
                            if (rc64 == FGPU_ERR_BREAKDOWN) fail = 1;
                            else if (rc64 == FGPU_ERR_NOT_CONVERGED) fail = 2;
                            else rc = rc64;
                            if (rc == FGPU_OK) rc = f64_residual(ctx, A64, d_b, d_x, rbest, S.partial, S.hpart, &rn);
                        } else {
                            fail = res.fail == 1 ? 1 : 2;
                        }
                    }
                }
            }
            cudaStreamSynchronize(ctx->stream);
        }
        cudaFree(r32);
        cudaFree(x32);
        cudaFree(xc);
        cudaFree(rc64);
    }
    cudaEventRecord(e1, ctx->stream);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != FGPU_OK) return rc;
    if (st) {
        st->iterations = res.iters + fallback_its;
        st->outer = res.nrefresh;
        st->rel_residual = bn > 0 ? rn / bn : 0.0;
        st->time_ms = ms;
        st->eig_max = res.lmax;
        st->fallback = fallback;
        st->fallback_iterations = fallback_its;
    }
    if (fail == 1) { ctx->err = "CG breakdown: p.Ap <= 0 (matrix not SPD)"; return FGPU_ERR_BREAKDOWN; }
    if (fail == 2) { ctx->err = "mixed CG did not reach rtol"; return FGPU_ERR_NOT_CONVERGED; }
    return FGPU_OK;
}

}  // namespace fgpu

SellLayout::~SellLayout() {
    cudaFree(d_perm);
    cudaFree(d_slice_ptr);
    cudaFree(d_slice_len);
    cudaFree(d_col);
    cudaFree(d_src);
}
