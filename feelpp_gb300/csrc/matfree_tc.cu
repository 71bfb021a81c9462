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

namespace fgpu {

constexpr int kTcTile = 128;                 // elements per tile (MMA M)
constexpr int kTcThreads = 128;              // one thread per element / TMEM lane
constexpr int kTcTmemCols = 256;
constexpr int kStatusTcTimeout = 16;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor (K-major, no swizzle): start address, leading
// byte offset (between core matrices along K), stride byte offset (between
// 8-row groups), descriptor version 1, layout type 0.
__device__ __forceinline__ uint64_t make_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor: D f32, A and B tf32, both K-major, M = 128, N = nmma.
__host__ __device__ constexpr uint32_t make_idesc_tf32(int nmma) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(nmma >> 3) << 17) | ((uint32_t)(kTcTile >> 4) << 24);
}

__device__ __forceinline__ float tf32_hi(float x) {
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

// byte offset of (row, k) in a K-major no-swizzle operand with kpad columns (tf32)
__device__ __forceinline__ uint32_t core_off(int row, int k, int kpad) {
    return (uint32_t)((row >> 3) * (kpad / 4) * 128 + (k >> 2) * 128 + (row & 7) * 16 + (k & 3) * 4);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void tc_commit(void* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar)) : "memory");
}

// bounded wait for an mbarrier phase; returns false when the budget ran out
__device__ __forceinline__ bool mbar_wait(void* mbar, uint32_t phase, int budget) {
    uint32_t done = 0;
    for (int it = 0; it < budget; ++it) {
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.b32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(smem_u32(mbar)), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

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

// ---------------------------------------------------------------------------
// Element phase: ye[i][e] = sum_k c_{e,k} (T_k x_e)_i for all elements.
// Shared memory: Bh, Bl (NMMA x KPAD tf32), Ah, Al (128 x KPAD tf32).
// ---------------------------------------------------------------------------
template <int N>
struct TcDims {
    static constexpr int KPAD = (N + 7) / 8 * 8;
    static constexpr int NMMA = (7 * N + 15) / 16 * 16;
    static constexpr int BBYTES = NMMA * KPAD * 4;
    static constexpr int ABYTES = kTcTile * KPAD * 4;
    static constexpr int SMEM = 1024 + 2 * BBYTES + 2 * ABYTES + 64;
};

template <int N>
__global__ void __launch_bounds__(kTcThreads) mf_element_tc_kernel(int64_t nt, const int32_t* __restrict__ l2n,
                                                                   const float4* __restrict__ rec, const float* __restrict__ Tg,
                                                                   const float* __restrict__ x, const uint8_t* __restrict__ mask,
                                                                   float* __restrict__ ye, const int* __restrict__ stop,
                                                                   int* __restrict__ status, int wait_budget) {
    typedef TcDims<N> D;
    if (stop && *stop) return;
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    unsigned char* base = (unsigned char*)(((uintptr_t)tc_smem + 1023) & ~(uintptr_t)1023);
    unsigned char* Bh = base;
    unsigned char* Bl = Bh + D::BBYTES;
    unsigned char* Ah = Bl + D::BBYTES;
    unsigned char* Al = Ah + D::ABYTES;
    TcShared* ts = reinterpret_cast<TcShared*>(Al + D::ABYTES);
    const int t = threadIdx.x;
    // B = [T_0; ...; T_6] as NMMA x KPAD: row n = k N + i, column j -> T_k[i][j]
    for (int idx = t; idx < D::NMMA * D::KPAD; idx += kTcThreads) {
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
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_setup(ts);
    const uint32_t tmem = ts->tmem_base;
    const uint32_t my_lane_addr = tmem + ((uint32_t)(32 * (t >> 5)) << 16);
    uint32_t phase = 0;
    const int64_t ntiles = (nt + kTcTile - 1) / kTcTile;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t e = tile * kTcTile + t;
        float c[7] = {0, 0, 0, 0, 0, 0, 0};
        // gather x_e into A (hi / lo), zero padding
#pragma unroll
        for (int j = 0; j < D::KPAD; ++j) {
            float v = 0.0f;
            if (e < nt && j < N) {
                const int32_t d = l2n[e * N + j];
                v = (mask && mask[d]) ? 0.0f : x[d];
            }
            const float h = tf32_hi(v);
            *reinterpret_cast<float*>(Ah + core_off(t, j, D::KPAD)) = h;
            *reinterpret_cast<float*>(Al + core_off(t, j, D::KPAD)) = v - h;
        }
        if (e < nt) {
            const float4 h0 = __ldg(rec + 4 * e), h1 = __ldg(rec + 4 * e + 1);
            c[0] = h0.x; c[1] = h0.y; c[2] = h0.z; c[3] = h0.w; c[4] = h1.x; c[5] = h1.y; c[6] = h1.z;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        if (t == 0) tc_issue<D::KPAD, D::NMMA>(tmem, Ah, Al, Bh, Bl, &ts->mbar);
        const bool ok = mbar_wait(&ts->mbar, phase, wait_budget);
        phase ^= 1u;
        if (!ok) {
            if (t == 0) atomicOr(status, kStatusTcTimeout);
            ts->bad = 1;
        }
        __syncthreads();
        if (ts->bad) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // epilogue: y_i = sum_k c_k Z[k N + i]
        float y[N];
#pragma unroll
        for (int i = 0; i < N; ++i) y[i] = 0.0f;
#pragma unroll
        for (int cb = 0; cb < D::NMMA; cb += 16) {
            float z[16];
            tmem_ld16(my_lane_addr + cb, z);
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                const int n = cb + q;
                if (n < 7 * N) y[n % N] = fmaf(c[n / N], z[q], y[n % N]);
            }
        }
        if (e < nt) {
#pragma unroll
            for (int i = 0; i < N; ++i) ye[(int64_t)i * nt + e] = y[i];
        }
        // all TMEM reads and smem A reads done before the next tile overwrites them
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
    }
    tc_teardown(ts);
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
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ntiles, 2 * (int64_t)sms));
    if (n == 20) {
        auto k = mf_element_tc_kernel<20>;
        constexpr int sm = TcDims<20>::SMEM;
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
        k<<<grid, kTcThreads, sm, ctx->stream>>>(nt, l2n, rec, T7f, x, mask, ye, stop, ctx->d_status, kTcWaitBudget);
    } else if (n == 10) {
        auto k = mf_element_tc_kernel<10>;
        constexpr int sm = TcDims<10>::SMEM;
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
        k<<<grid, kTcThreads, sm, ctx->stream>>>(nt, l2n, rec, T7f, x, mask, ye, stop, ctx->d_status, kTcWaitBudget);
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
