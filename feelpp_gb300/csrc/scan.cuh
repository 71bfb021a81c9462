// Exclusive scan of uint32 counts on the device (used by the set-up kernels:
// gather maps, device dof tables, patterns). Header-only: every kernel is
// static to the translation unit that includes it.
#pragma once
#include <cstdint>
#include <string>

#include "fgpu_core.h"

namespace fgpu {

// exclusive scan of uint32 counts in chunks of kScanChunk: per-chunk sums, a
// one-block scan of the sums, then the chunks with their offsets
static constexpr int kScanChunk = 4096;
static __global__ void scan_chunk_sums_kernel(int64_t n, const uint32_t* __restrict__ in, unsigned long long* __restrict__ sums) {
    __shared__ unsigned long long sh[32];
    const int64_t c0 = (int64_t)blockIdx.x * kScanChunk;
    unsigned long long s = 0;
    for (int k = threadIdx.x; k < kScanChunk; k += blockDim.x)
        if (c0 + k < n) s += in[c0 + k];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
        sums[blockIdx.x] = t;
    }
}
// one block of 1024 threads: each thread scans a contiguous segment of the sums
static __global__ void __launch_bounds__(1024) scan_sums_kernel(int64_t nchunks, unsigned long long* __restrict__ sums) {
    __shared__ unsigned long long part[1024];
    const int64_t seg = (nchunks + 1023) / 1024;
    const int64_t b = threadIdx.x * seg, e = min(b + seg, nchunks);
    unsigned long long t = 0;
    for (int64_t c = b; c < e; ++c) t += sums[c];
    part[threadIdx.x] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long run = 0;
        for (int k = 0; k < 1024; ++k) {
            const unsigned long long v = part[k];
            part[k] = run;
            run += v;
        }
        sums[nchunks] = run;
    }
    __syncthreads();
    unsigned long long run = part[threadIdx.x];
    for (int64_t c = b; c < e; ++c) {
        const unsigned long long v = sums[c];
        sums[c] = run;
        run += v;
    }
}
static __global__ void scan_chunks_kernel(int64_t n, const uint32_t* __restrict__ in, const unsigned long long* __restrict__ sums,
                                   uint32_t* __restrict__ out) {
    // one warp per chunk, sequential over 32-entry strips with warp prefix sums
    const int64_t c = blockIdx.x;
    const int lane = threadIdx.x;
    unsigned long long run = sums[c];
    for (int64_t b = c * kScanChunk; b < min((c + 1) * kScanChunk, n); b += 32) {
        const int64_t k = b + lane;
        const uint32_t v = k < n ? in[k] : 0u;
        uint32_t x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (k < n) out[k] = (uint32_t)(run + x - v);
        run += __shfl_sync(0xffffffffu, x, 31);
    }
    if (c == gridDim.x - 1 && lane == 0) out[n] = (uint32_t)sums[gridDim.x];
}

// out[0..n]: exclusive prefix sums of in[0..n), out[n] = total (written to *total
// too, after a stream sync). The total must fit in 32 bits.
static int scan_u32(fgpu_ctx* ctx, const uint32_t* in, uint32_t* out, int64_t n, uint64_t* total) {
    const int64_t nchunks = std::max<int64_t>(1, (n + kScanChunk - 1) / kScanChunk);
    unsigned long long* sums = nullptr;
    if (cudaMalloc(&sums, (nchunks + 1) * sizeof(unsigned long long)) != cudaSuccess) {
        cudaGetLastError();
        ctx->err = "scan: allocation failed";
        return FGPU_ERR_ALLOC;
    }
    scan_chunk_sums_kernel<<<(int)nchunks, 256, 0, ctx->stream>>>(n, in, sums);
    scan_sums_kernel<<<1, 1024, 0, ctx->stream>>>(nchunks, sums);
    scan_chunks_kernel<<<(int)nchunks, 32, 0, ctx->stream>>>(n, in, sums, out);
    ctx->launches += 3;
    unsigned long long t = 0;
    cudaMemcpyAsync(&t, sums + nchunks, sizeof(t), cudaMemcpyDeviceToHost, ctx->stream);
    const cudaError_t e = cudaStreamSynchronize(ctx->stream);
    cudaFree(sums);
    if (e != cudaSuccess) { ctx->err = std::string("scan: ") + cudaGetErrorString(e); return FGPU_ERR_CUDA; }
    if (t > 0xFFFFFFFFull) { ctx->err = "scan: total exceeds 32 bits"; return FGPU_ERR_INVALID; }
    if (total) *total = t;
    return FGPU_OK;
}

}  // namespace fgpu
