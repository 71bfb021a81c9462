// Tensor-core (tcgen05) element phase of the binary32 matrix-free operator.
//
// For a tile of 128 elements the element products y_e = sum_k c_k T_k x_e are
// one dense contraction followed by a per-element combination:
//     Z (128 x 7n) = X (128 x n) * [T_0; ...; T_6]^T      (tensor cores)
//     y_e[i]       = sum_k c_{e,k} Z[e][k n + i]            (epilogue, FP32 FMA)
// The contraction runs as tcgen05.mma kind::tf32 with the operands staged in
// shared memory (K-major, no swizzle, 8-row x 16-byte core matrices) and the
// FP32 accumulator in tensor memory; one elected thread issues the MMAs and
// commits them to an mbarrier; the epilogue reads the accumulator back with
// tcgen05.ld (each thread owns one element = one TMEM lane).
// Accuracy: both operands are split into TF32 high and low parts and the
// three products hi*hi + hi*lo + lo*hi are accumulated (3xTF32), which keeps
// binary32-level accuracy.
//
// Every wait is bounded: an mbarrier wait that exceeds its iteration budget
// sets a status bit, the CTA stops issuing work, frees its tensor memory and
// returns.
#include <cstdint>
#include <cstring>
#include <vector>

#include "fgpu_core.h"
#include "tc_ptx.cuh"

namespace fgpu {

constexpr int kTcThreads = 128;              // one thread per element / TMEM lane
constexpr int kTcTmemCols = 256;
constexpr int kStatusTcTimeout = 16;

struct TcShared {
    uint64_t mbar;
    uint32_t tmem_base;
    int bad;
};

// Set-up shared by the kernels below: mbarrier init and TMEM allocation (warp 0).
__device__ __forceinline__ void tc_setup(TcShared* ts) {
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&ts->mbar)), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        ts->bad = 0;
    }
    if ((threadIdx.x >> 5) == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&ts->tmem_base)),
                     "r"(kTcTmemCols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_teardown(TcShared* ts) {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if ((threadIdx.x >> 5) == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(ts->tmem_base), "r"(kTcTmemCols) : "memory");
}

// Issue the 3xTF32 products for one tile (elected thread) and commit.
template <int KPAD, int NMMA>
__device__ __forceinline__ void tc_issue(uint32_t tmem_d, const unsigned char* Ah, const unsigned char* Al,
                                         const unsigned char* Bh, const unsigned char* Bl, void* mbar) {
    constexpr uint32_t idesc = make_idesc_tf32(NMMA);
    constexpr uint32_t lbo = 128, sbo = (KPAD / 4) * 128;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
    for (int s = 0; s < KPAD / 8; ++s) {
        const uint64_t ah = make_sdesc(smem_u32(Ah) + s * 256, lbo, sbo);
        const uint64_t al = make_sdesc(smem_u32(Al) + s * 256, lbo, sbo);
        const uint64_t bh = make_sdesc(smem_u32(Bh) + s * 256, lbo, sbo);
        const uint64_t bl = make_sdesc(smem_u32(Bl) + s * 256, lbo, sbo);
        tc_mma(tmem_d, ah, bh, idesc, s > 0 ? 1u : 0u);
        tc_mma(tmem_d, ah, bl, idesc, 1u);
        tc_mma(tmem_d, al, bh, idesc, 1u);
    }
    tc_commit(mbar);
}

// Operand shapes of the element phase: B = [T_0; ...; T_6] as NMMA x KPAD, A = a tile of x_e as
// 128 x KPAD (tf32 hi and lo parts of each).
template <int N>
struct TcDims {
    static constexpr int KPAD = (N + 7) / 8 * 8;
    static constexpr int NMMA = (7 * N + 15) / 16 * 16;
    static constexpr int BBYTES = NMMA * KPAD * 4;
    static constexpr int ABYTES = kTcTile * KPAD * 4;
    static constexpr int SMEM = 1024 + 2 * BBYTES + 2 * ABYTES + 64;
};


// ---------------------------------------------------------------------------
// Pipelined element phase (one CTA per SM, 384 threads): warps 0-7 write the
// tile's x values (all 256 threads over the 128 x KPAD entries, gathered into
// registers during the previous tile while the next tile's loads are in flight) into
// one of two A buffers, while thread 0 issues the MMAs of the previous tile
// into one of two TMEM accumulators and warps 8-11 (one thread per TMEM lane)
// combine the finished accumulator with the coefficients and write the element
// values. Three mbarriers per buffer: full (256 producer arrivals), mma (the commit of the
// MMAs that read the buffer and fill the accumulator), free (128 consumer
// arrivals, the accumulator may be overwritten). Tile it uses buffer it & 1
// for the (it >> 1)-th time: every wait is on a phase that cannot be overtaken.
// Every wait is bounded; a timeout sets a status bit and a shared flag that
// makes every role leave its loop, and the tensor memory is freed at the end.
// ---------------------------------------------------------------------------
struct TcPipeShared {
    uint64_t full[2], mma[2], freeb[2];
    uint32_t tmem_base;
    volatile int bad;
};

// bounded wait that also gives up when another role has flagged a failure
__device__ __forceinline__ bool mbar_wait_or_bad(void* b, uint32_t phase, int budget, volatile int* bad) {
    uint32_t done = 0;
    for (int it = 0; it < budget; ++it) {
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.b32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(smem_u32(b)), "r"(phase)
            : "memory");
        if (done) return true;
        if ((it & 63) == 63 && *bad) return false;
    }
    return false;
}

template <int N>
struct TcPipeDims {
    static constexpr int KPAD = TcDims<N>::KPAD, NMMA = TcDims<N>::NMMA;
    static constexpr int BBYTES = NMMA * KPAD * 4, ABYTES = kTcTile * KPAD * 4;
    static constexpr int USED = 1024 + 2 * BBYTES + 4 * ABYTES + 256;
    static constexpr int SMEM = USED > 118 * 1024 ? USED : 118 * 1024;   // one CTA per SM (its 512 TMEM columns)
    static constexpr int ACC_STRIDE = 256;                                // TMEM columns between the two accumulators
};

constexpr int kTcProducers = 256;
constexpr int kTcPipeThreads = kTcProducers + 128;

template <int N>
__global__ void __launch_bounds__(kTcPipeThreads) mf_element_tc_pipe_kernel(int64_t nt, const int32_t* __restrict__ l2n,
                                                                 const float4* __restrict__ rec, const float* __restrict__ Tg,
                                                                 const float* __restrict__ x, const uint8_t* __restrict__ mask,
                                                                 float* __restrict__ ye, const int* __restrict__ stop,
                                                                 int* __restrict__ status, int wait_budget) {
    typedef TcPipeDims<N> D;
    if (stop && *stop) return;
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    unsigned char* base = (unsigned char*)(((uintptr_t)tc_smem + 1023) & ~(uintptr_t)1023);
    unsigned char* Bh = base;
    unsigned char* Bl = Bh + D::BBYTES;
    unsigned char* A0 = Bl + D::BBYTES;                     // buffer b: hi at A0 + 2 b ABYTES, lo after it
    TcPipeShared* ps = reinterpret_cast<TcPipeShared*>(A0 + 4 * D::ABYTES);
    const int t = threadIdx.x;
    for (int idx = t; idx < D::NMMA * D::KPAD; idx += blockDim.x) {
        const int n = idx / D::KPAD, j = idx - n * D::KPAD;
        float v = 0.0f;
        if (n < 7 * N && j < N) {
            const int k = n / N, i = n - k * N;
            v = Tg[(k * N + i) * N + j];
        }
        const float h = tf32_hi(v);
        *reinterpret_cast<float*>(Bh + core_off(n, j, D::KPAD)) = h;
        *reinterpret_cast<float*>(Bl + core_off(n, j, D::KPAD)) = v - h;
    }
    if (t == 0) {
        for (int b = 0; b < 2; ++b) {
            mbar_init(&ps->full[b], kTcProducers);
            mbar_init(&ps->mma[b], 1);
            mbar_init(&ps->freeb[b], 128);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        ps->bad = 0;
    }
    if ((t >> 5) == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&ps->tmem_base)), "r"(512)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = ps->tmem_base;
    const int64_t ntiles = (nt + kTcTile - 1) / kTcTile;
    if (t < kTcProducers) {
        // producers; thread 0 also issues the MMAs. Entry p = t + q * 256 of a tile is (row, j) =
        // (p / KPAD, p % KPAD): consecutive threads read consecutive ints of the tile's l2n block
        constexpr int ITER = kTcTile * D::KPAD / kTcProducers;
        static_assert(ITER * kTcProducers == kTcTile * D::KPAD, "tile entries split evenly");
        auto load_tile_idx = [&](int64_t tl, int32_t* d) {
            const int64_t e0 = tl * kTcTile;
#pragma unroll
            for (int q = 0; q < ITER; ++q) {
                const int p = t + q * kTcProducers;
                const int row = p / D::KPAD, j = p - row * D::KPAD;
                d[q] = (tl < ntiles && e0 + row < nt && j < N) ? __ldg(l2n + (e0 + row) * N + j) : -1;
            }
        };
        // x values (and Dirichlet mask bytes) of the entries with indices d; -1 reads nothing
        auto gather = [&](const int32_t* d, float* v, uint32_t* m) {
#pragma unroll
            for (int q = 0; q < ITER; ++q) v[q] = d[q] >= 0 ? __ldg(x + d[q]) : 0.0f;
#pragma unroll
            for (int q = 0; q < ITER; ++q) m[q] = (mask && d[q] >= 0) ? (uint32_t)mask[d[q]] : 0u;
        };
        // three-stage register pipeline: while tile it is written to shared memory from the values
        // gathered during tile it - 1, the x values of tile it + 1 and the indices of tile it + 2 are
        // in flight. (4-byte cp.async copies into shared-memory slots, three tiles ahead, measured
        // slower: 0.74 vs 0.64 ms for the P3 96^3 element phase.)
        int32_t dn[ITER];
        float vc[ITER];
        uint32_t mc[ITER];
        load_tile_idx(blockIdx.x, dn);
        gather(dn, vc, mc);
        load_tile_idx(blockIdx.x + gridDim.x, dn);
        for (int64_t it = 0, tile = blockIdx.x; tile < ntiles; ++it, tile += gridDim.x) {
            const int b = (int)(it & 1);
            const uint32_t u = (uint32_t)(it >> 1);
            unsigned char* Ahb = A0 + 2 * b * D::ABYTES;
            unsigned char* Alb = Ahb + D::ABYTES;
            uint32_t mybad = 0;
            if (u > 0 && !mbar_wait_or_bad(&ps->mma[b], (u - 1) & 1u, wait_budget, &ps->bad)) mybad = 1;
            mybad |= (uint32_t)(ps->bad != 0);
            // barrier over the producers that also ORs their failure flags: all leave together or none
            uint32_t anybad = 0;
            asm volatile("{\n\t.reg .pred pin, pout;\n\tsetp.ne.u32 pin, %1, 0;\n\tbar.red.or.pred pout, 1, %2, pin;\n\t"
                         "selp.u32 %0, 1, 0, pout;\n\t}\n"
                         : "=r"(anybad)
                         : "r"(mybad), "r"(kTcProducers)
                         : "memory");
            if (anybad) { ps->bad = 1; break; }
            // start the next tile's gathers and the indices of the one after
            int32_t dd[ITER];
#pragma unroll
            for (int q = 0; q < ITER; ++q) dd[q] = dn[q];
            float vn[ITER];
            uint32_t mn[ITER];
            gather(dd, vn, mn);
            load_tile_idx(tile + 2 * (int64_t)gridDim.x, dn);
            // this tile's values, all producer threads over the 128 x KPAD entries
#pragma unroll
            for (int q = 0; q < ITER; ++q) {
                const int p = t + q * kTcProducers;
                const int row = p / D::KPAD, j = p - row * D::KPAD;
                const float val = mc[q] ? 0.0f : vc[q];
                const float h = tf32_hi(val);
                *reinterpret_cast<float*>(Ahb + core_off(row, j, D::KPAD)) = h;
                *reinterpret_cast<float*>(Alb + core_off(row, j, D::KPAD)) = val - h;
            }
#pragma unroll
            for (int q = 0; q < ITER; ++q) { vc[q] = vn[q]; mc[q] = mn[q]; }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_arrive(&ps->full[b]);
            if (t == 0) {
                // the issuer does not leave the loop on a timeout: it flags it, and the producers' barrier
                // at the next tile takes everyone out together
                bool ok = mbar_wait_or_bad(&ps->full[b], u & 1u, wait_budget, &ps->bad);
                if (ok && u > 0) ok = mbar_wait_or_bad(&ps->freeb[b], (u - 1) & 1u, wait_budget, &ps->bad);
                if (ok) tc_issue<D::KPAD, D::NMMA>(tmem + (uint32_t)(b * D::ACC_STRIDE), Ahb, Alb, Bh, Bl, &ps->mma[b]);
                else { ps->bad = 1; atomicOr(status, kStatusTcTimeout); }
            }
        }
    } else {
        // consumers: one thread per TMEM lane / element row
        const int r = t - kTcProducers;
        const uint32_t lane_addr = tmem + ((uint32_t)(32 * ((t >> 5) & 3)) << 16);
        for (int64_t it = 0, tile = blockIdx.x; tile < ntiles; ++it, tile += gridDim.x) {
            const int b = (int)(it & 1);
            const uint32_t u = (uint32_t)(it >> 1);
            const int64_t e = tile * kTcTile + r;
            float c[7] = {0, 0, 0, 0, 0, 0, 0};
            if (e < nt) {
                const float4 h0 = __ldg(rec + 4 * e), h1 = __ldg(rec + 4 * e + 1);
                c[0] = h0.x; c[1] = h0.y; c[2] = h0.z; c[3] = h0.w; c[4] = h1.x; c[5] = h1.y; c[6] = h1.z;
            }
            if (!mbar_wait_or_bad(&ps->mma[b], u & 1u, wait_budget, &ps->bad)) {
                ps->bad = 1;
                if (r == 0) atomicOr(status, kStatusTcTimeout);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            float y[N];
#pragma unroll
            for (int i = 0; i < N; ++i) y[i] = 0.0f;
            // the accumulator row in groups of three x16 loads, one wait per group
            constexpr int NB = D::NMMA / 16;
#pragma unroll
            for (int g0 = 0; g0 < NB; g0 += 3) {
                uint32_t z[3][16];
#pragma unroll
                for (int g = 0; g < 3; ++g)
                    if (g0 + g < NB) tmem_ld16_nowait(lane_addr + (uint32_t)(b * D::ACC_STRIDE + (g0 + g) * 16), z[g]);
                tmem_wait_ld();
#pragma unroll
                for (int g = 0; g < 3; ++g)
#pragma unroll
                    for (int q = 0; q < 16; ++q) {
                        const int n = (g0 + g) * 16 + q;
                        if (g0 + g < NB && n < 7 * N) y[n % N] = fmaf(c[n / N], __uint_as_float(z[g][q]), y[n % N]);
                    }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            mbar_arrive(&ps->freeb[b]);
            if (e < nt) {
#pragma unroll
                for (int i = 0; i < N; ++i) ye[(int64_t)i * nt + e] = y[i];
            }
            if (ps->bad) break;
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if ((t >> 5) == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
}

// ---------------------------------------------------------------------------
// Self-test: D (128 x NMMA) = A (128 x KPAD) * B (NMMA x KPAD)^T in 3xTF32 with
// the same staging, descriptors, MMA issue and TMEM read-back as the kernel.
// ---------------------------------------------------------------------------
template <int KPAD, int NMMA>
__global__ void __launch_bounds__(kTcThreads) tc_selftest_kernel(const float* __restrict__ A, const float* __restrict__ B,
                                                                 float* __restrict__ Dout, int* __restrict__ status, int wait_budget) {
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    unsigned char* base = (unsigned char*)(((uintptr_t)tc_smem + 1023) & ~(uintptr_t)1023);
    constexpr int BB = NMMA * KPAD * 4, AB = kTcTile * KPAD * 4;
    unsigned char* Bh = base;
    unsigned char* Bl = Bh + BB;
    unsigned char* Ah = Bl + BB;
    unsigned char* Al = Ah + AB;
    TcShared* ts = reinterpret_cast<TcShared*>(Al + AB);
    const int t = threadIdx.x;
    for (int idx = t; idx < NMMA * KPAD; idx += kTcThreads) {
        const int n = idx / KPAD, j = idx - n * KPAD;
        const float v = B[idx], h = tf32_hi(v);
        *reinterpret_cast<float*>(Bh + core_off(n, j, KPAD)) = h;
        *reinterpret_cast<float*>(Bl + core_off(n, j, KPAD)) = v - h;
    }
    for (int j = 0; j < KPAD; ++j) {
        const float v = A[t * KPAD + j], h = tf32_hi(v);
        *reinterpret_cast<float*>(Ah + core_off(t, j, KPAD)) = h;
        *reinterpret_cast<float*>(Al + core_off(t, j, KPAD)) = v - h;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_setup(ts);
    const uint32_t tmem = ts->tmem_base;
    if (t == 0) tc_issue<KPAD, NMMA>(tmem, Ah, Al, Bh, Bl, &ts->mbar);
    const bool ok = mbar_wait(&ts->mbar, 0, wait_budget);
    if (!ok && t == 0) atomicOr(status, kStatusTcTimeout);
    __syncthreads();
    if (ok) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t la = tmem + ((uint32_t)(32 * (t >> 5)) << 16);
        for (int cb = 0; cb < NMMA; cb += 16) {
            float z[16];
            tmem_ld16(la + cb, z);
            for (int q = 0; q < 16; ++q) Dout[t * NMMA + cb + q] = z[q];
        }
    }
    tc_teardown(ts);
}

static constexpr int kTcWaitBudget = 1 << 22;

int launch_mf_element_tc(fgpu_ctx* ctx, int n, int64_t nt, const int32_t* l2n, const float4* rec, const float* T7f, const float* x,
                         const uint8_t* mask, float* ye, const int* stop) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int64_t ntiles = (nt + kTcTile - 1) / kTcTile;
    const int pgrid = (int)std::max<int64_t>(1, std::min<int64_t>(ntiles, (int64_t)sms));
    if (n == 20) {
        auto k = mf_element_tc_pipe_kernel<20>;
        constexpr int sm = TcPipeDims<20>::SMEM;
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
        k<<<pgrid, kTcPipeThreads, sm, ctx->stream>>>(nt, l2n, rec, T7f, x, mask, ye, stop, ctx->d_status, kTcWaitBudget);
    } else if (n == 10) {
        auto k = mf_element_tc_pipe_kernel<10>;
        constexpr int sm = TcPipeDims<10>::SMEM;
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
        k<<<pgrid, kTcPipeThreads, sm, ctx->stream>>>(nt, l2n, rec, T7f, x, mask, ye, stop, ctx->d_status, kTcWaitBudget);
    } else {
        ctx->err = "tensor-core element phase supports P2 and P3";
        return FGPU_ERR_INVALID;
    }
    ctx->launches++;
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

}  // namespace fgpu

using namespace fgpu;

// D = A * B^T (A: 128 x 24, B: 144 x 24, row-major binary32) through the tcgen05
// path; returns FGPU_OK, or FGPU_ERR_CUDA when the MMA did not complete in time.
extern "C" int fgpu_tc_selftest(fgpu_ctx* ctx, const float* hA, const float* hB, float* hD) {
    if (!ctx || !hA || !hB || !hD) return FGPU_ERR_INVALID;
    constexpr int KPAD = 24, NMMA = 144;
    float *A = nullptr, *B = nullptr, *D = nullptr;
    auto done = [&](int rc) { cudaFree(A); cudaFree(B); cudaFree(D); return rc; };
    if (cudaMalloc(&A, kTcTile * KPAD * 4) != cudaSuccess || cudaMalloc(&B, NMMA * KPAD * 4) != cudaSuccess ||
        cudaMalloc(&D, kTcTile * NMMA * 4) != cudaSuccess)
        return done(FGPU_ERR_ALLOC);
    cudaMemcpy(A, hA, kTcTile * KPAD * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(B, hB, NMMA * KPAD * 4, cudaMemcpyHostToDevice);
    cudaMemset(D, 0, kTcTile * NMMA * 4);
    cudaMemset(ctx->d_status, 0, sizeof(int));
    constexpr int sm = 1024 + 2 * NMMA * KPAD * 4 + 2 * kTcTile * KPAD * 4 + 64;
    auto k = tc_selftest_kernel<KPAD, NMMA>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    k<<<1, kTcThreads, sm, ctx->stream>>>(A, B, D, ctx->d_status, kTcWaitBudget);
    ctx->launches++;
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { ctx->err = cudaGetErrorString(e); return done(FGPU_ERR_CUDA); }
    int st = 0;
    cudaMemcpy(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost);
    cudaMemset(ctx->d_status, 0, sizeof(int));
    if (st & kStatusTcTimeout) { ctx->err = "tcgen05 self-test: MMA completion wait timed out"; return done(FGPU_ERR_CUDA); }
    cudaMemcpy(hD, D, kTcTile * NMMA * 4, cudaMemcpyDeviceToHost);
    return done(FGPU_OK);
}
