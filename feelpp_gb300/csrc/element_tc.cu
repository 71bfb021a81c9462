// Element matrices of the affine Laplace/mass form to FP64 accuracy on the bf16
// tensor cores (tcgen05.mma kind::f16), by exact integer slicing (the Ozaki
// scheme).
//
// The upper triangle of an element matrix is K_e(t) = sum_{k<7} c_k(e) T_k(t): the
// element's df64 coefficient record c (kappa J B^T B and mass J) against the seven
// reference tensors T (bilinearformcontext.hpp:585-589 evaluates the same sums
// entry by entry). For a tile of 128 elements this is D (128 x NTRI) = A (128 x 7)
// B^T (7 x NTRI) with a contraction length of 7.
//
// Both operands are cut into seven 8-bit slices. With per-tile exponents s_k (the
// largest coefficient k of the tile), per-row exponents E_m and per-column exponents
// F_t chosen so that every scaled value lies in (-1, 1):
//     c_k(m) = 2^(E_m + s_k)  sum_i a_ik(m) 2^(-8(i+1)),
//     T_k(t) = 2^(F_t - s_k)  sum_j b_jk(t) 2^(-8(j+1)),   a, b integers, |a|, |b| <= 256,
// each slice exactly a bf16 value (the low binary32 of a double-float joins the
// slicing through a TwoSum, so the slices hold it without a rounding). A product
// a b has at most 16 bits and a sum of up to 28 of them at most 21 bits, so the
// sums of the levels l = i + j = 0 .. 3 are exact in the FP32 accumulators of
// tensor memory (one accumulator per level); levels 4 to 7 go into a fifth, whose
// rounding is 2^-24 of a term already 2^-40 below the leading one. The epilogue
// adds the five accumulators of an entry in double-float (three TwoSums) and
// scales by 2^(E_m + F_t). Slicing stops after 56 bits and products past level 7
// are left out. Emulated on the CPU with coefficients three and tables two orders
// of magnitude apart within a row and column, the error stays below 3e-14 of
// sum_k |c_k T_k|, the scale of the CUDA-core df64 kernel's compensated sum (which
// this kernel replaces, with other rounding: the two differ in the last bits).
//
// One CTA of 256 threads per tile: threads 0..127 hold one element each (record,
// row exponent, A slices), threads 0..NCH*NP-1 one table column each (B slices of
// the tile's exponents); per chunk of NP = 16 columns thread 0 issues 34 MMAs
// (M = 128, N = 16, K = 16 of which 7 are used) and commits them to an mbarrier;
// the eight warps read the five accumulators back with tcgen05.ld (warps w and
// w + 4 share the lanes of rows 32 (w % 4) ... and take 8 columns each), form the
// values into a shared-memory staging tile, and the chunk is written out with
// coalesced stores (each element's entries are contiguous in the element buffer).
// Every mbarrier wait is bounded: a timeout sets a status bit, the block leaves at
// the next barrier after waiting (bounded) for its issued products, and frees its
// tensor memory.
#include <algorithm>
#include <cstdint>

#include "asm_device.cuh"
#include "df64.h"
#include "fgpu_core.h"
#include "tc_ptx.cuh"

namespace fgpu {

namespace {

constexpr int kOzThreads = 256;
constexpr int kOzSlices = 7;        // 8-bit slices per operand
constexpr int kOzExact = 4;         // levels 0 .. 3 summed exactly, one accumulator each
constexpr int kOzLevels = 8;        // levels 0 .. 7 (the last four in one accumulator)
constexpr int kOzAcc = kOzExact + 1;
constexpr int kOzWaitBudget = 1 << 22;

template <int N>
struct OzDims {
    static constexpr int NTRI = N * (N + 1) / 2;
    static constexpr int NP = 16;                                   // MMA N of a column chunk
    static constexpr int NCH = (NTRI + NP - 1) / NP;                // chunks
    static constexpr int NCOLS_USED = kOzAcc * NP;
    static constexpr int NCOLS = NCOLS_USED <= 32 ? 32 : NCOLS_USED <= 64 ? 64 : NCOLS_USED <= 128 ? 128 : 256;   // tensor-memory allocation
    static constexpr int ASLICE = kTcTile * 32;                     // one A slice: 128 rows x 16 bf16
    static constexpr int BSLICE = NP * 32;                          // one B slice of one chunk
    static constexpr int STG = NP + 1;                              // staging row stride (float2), padded
    static constexpr int SMEM_USED = 1024 + kOzSlices * ASLICE + NCH * kOzSlices * BSLICE + kTcTile * STG * 8 +
                                     NCH * NP * 4 + kTcTile * 4 + 64 + 64;
    static constexpr int MAXCTA = 512 / NCOLS;                      // tensor-memory allocations that fit an SM
    static constexpr int SMEM_MIN = 228 * 1024 / (MAXCTA + 1) + 1024;
    static constexpr int SMEM = SMEM_USED > SMEM_MIN ? SMEM_USED : SMEM_MIN;
    static_assert(NCH * NP <= kOzThreads, "one thread per table column");
};

struct OzShared {
    uint64_t mma;
    uint32_t tmem;
    int bad;
    int sig[8];
};

__device__ __forceinline__ float pow2i(int e) { return __int_as_float((e + 127) << 23); }   // -126 <= e <= 127

// E with |x| < 2^E for normal x (x = 0 and subnormals: -1000)
__device__ __forceinline__ int exp_above(float x) {
    const int b = (__float_as_int(x) >> 23) & 0xFF;
    return b == 0 ? -1000 : b - 126;
}

// the slices of the double-float h + l, |h + l| < 1: s[i] = a_i 2^-8(i+1) with integers |a_i| <= 256
// (rounded to nearest, so each remainder is within half a unit of the next slice's scale). The low
// part joins at the fourth slice (2^-24 below the first) through a TwoSum; the TwoSum's error joins
// one slice later, where it is below the rounding of the last slice.
__device__ __forceinline__ void oz_slices(float h, float l, float* s) {
    float x = f_mul(h, 256.0f);
    const float y = f_mul(l, 256.0f);
    float e = 0.0f;
    float a[kOzSlices];
#pragma unroll
    for (int i = 0; i < kOzSlices; ++i) {
        if (i == 3) {
            const df m = two_sum(x, f_mul(y, 16777216.0f));
            x = m.hi;
            e = m.lo;
        } else if (i == 4) {
            x = f_fma(e, 256.0f, x);
        }
        a[i] = rintf(x);
        x = f_mul(f_sub(x, a[i]), 256.0f);              // exact: |x - a_i| <= 1/2 (Sterbenz)
    }
    float sc = 1.0f / 256.0f;
#pragma unroll
    for (int i = 0; i < kOzSlices; ++i) {
        s[i] = f_mul(a[i], sc);
        sc = f_mul(sc, 1.0f / 256.0f);
    }
}

__device__ __forceinline__ void tmem_ld8_nowait(uint32_t taddr, uint32_t* r) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    uint32_t r;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}

// byte offset of row r (k = 0..7 half) in a K-major no-swizzle bf16 operand of K = 16
__device__ __forceinline__ uint32_t oz_row_off(int r) { return (uint32_t)((r >> 3) * 256 + (r & 7) * 16); }

// the six slices of the seven values (h_k + l_k) q of one operand row, written as bf16 (K = 0..7 of
// the row; the K = 8..15 half stays zero) into slice i at base + i * stride + off
__device__ __forceinline__ void oz_store_row(const float* h, const float* l, float q, unsigned char* base, int stride,
                                             uint32_t off) {
    uint32_t w[kOzSlices][4];
#pragma unroll
    for (int kp = 0; kp < 4; ++kp) {
        float sa[kOzSlices], sb[kOzSlices];
        oz_slices(f_mul(h[2 * kp], q), f_mul(l[2 * kp], q), sa);
        if (2 * kp + 1 < 7) {
            oz_slices(f_mul(h[2 * kp + 1], q), f_mul(l[2 * kp + 1], q), sb);
        } else {
#pragma unroll
            for (int i = 0; i < kOzSlices; ++i) sb[i] = 0.0f;
        }
#pragma unroll
        for (int i = 0; i < kOzSlices; ++i) w[i][kp] = pack_bf16(sa[i], sb[i]);
    }
#pragma unroll
    for (int i = 0; i < kOzSlices; ++i)
        *reinterpret_cast<uint4*>(base + i * stride + off) = make_uint4(w[i][0], w[i][1], w[i][2], w[i][3]);
}

template <int N>
__global__ void __launch_bounds__(kOzThreads) element_tri_oz_kernel(int64_t nt, const float4* __restrict__ rec,
                                                                   const float* __restrict__ Thg, const float* __restrict__ Tlg,
                                                                   float2* __restrict__ kbuf, int* __restrict__ status, int budget) {
    typedef OzDims<N> D;
    extern __shared__ __align__(1024) unsigned char oz_smem[];
    unsigned char* base = (unsigned char*)(((uintptr_t)oz_smem + 1023) & ~(uintptr_t)1023);
    unsigned char* As = base;                                            // kOzSlices slices of A
    unsigned char* Bs = As + kOzSlices * D::ASLICE;                      // [chunk][slice]
    float2* stg = reinterpret_cast<float2*>(Bs + D::NCH * kOzSlices * D::BSLICE);
    float* fcol = reinterpret_cast<float*>(stg + kTcTile * D::STG);     // 2^F_t per column
    float* erow = fcol + D::NCH * D::NP;                                 // 2^E_m per row
    OzShared* sh = reinterpret_cast<OzShared*>(((uintptr_t)(erow + kTcTile) + 15) & ~(uintptr_t)15);
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;

    // zero both operands once: the K columns 7..15 stay zero
    for (int k = t; k < (kOzSlices * D::ASLICE + D::NCH * kOzSlices * D::BSLICE) / 16; k += kOzThreads)
        reinterpret_cast<uint4*>(As)[k] = make_uint4(0u, 0u, 0u, 0u);
    constexpr int NCOLT = D::NCH * D::NP;
    if (t == 0) {
        mbar_init(&sh->mma, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        sh->bad = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sh->tmem)),
                     "r"(D::NCOLS) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = sh->tmem;
    constexpr uint32_t idesc = make_idesc_bf16(D::NP);
    // epilogue: rows 32 (warp % 4) + lane, columns [col0, col0 + ecols) of each chunk
    constexpr int ECOLS = D::NP / 2;
    const int col0 = (warp >> 2) * ECOLS;
    const bool epi = col0 < D::NP;
    const int erow_m = 32 * (warp & 3) + lane;
    const uint32_t lane_addr = tmem + ((uint32_t)(32 * (warp & 3)) << 16);
    uint32_t phase = 0;
    const int64_t ntiles = (nt + kTcTile - 1) / kTcTile;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t e0 = tile * kTcTile;
        if (t < 8) sh->sig[t] = -1000;
        __syncthreads();
        // the tile's records; per coefficient the largest exponent over the tile
        float ch[7], cl[7];
        const bool row = t < kTcTile;
        const bool live = row && e0 + t < nt;
#pragma unroll
        for (int k = 0; k < 7; ++k) ch[k] = cl[k] = 0.0f;
        if (live) load_record(rec + 4 * (e0 + t), ch, cl, true);
        if (row) {
#pragma unroll
            for (int k = 0; k < 7; ++k) {
                const int m = __reduce_max_sync(0xFFFFFFFFu, exp_above(ch[k]));
                if (lane == 0) atomicMax(&sh->sig[k], m);
            }
        }
        __syncthreads();
        int sig[7];
#pragma unroll
        for (int k = 0; k < 7; ++k) sig[k] = sh->sig[k] < -100 ? -1000 : min(sh->sig[k], 100);
        if (row) {
            // row: u_k = c_k 2^-s_k (|u_k| < 1), E = max_k exponent of u_k, slices of u_k 2^-E
            float uh[7], ul[7];
            int E = -1000;
#pragma unroll
            for (int k = 0; k < 7; ++k) {
                const float p = sig[k] == -1000 ? 0.0f : pow2i(-sig[k]);
                uh[k] = f_mul(ch[k], p);
                ul[k] = f_mul(cl[k], p);
                E = max(E, exp_above(uh[k]));
            }
            E = E == -1000 ? 0 : max(E, -60);
            erow[t] = pow2i(E);
            oz_store_row(uh, ul, pow2i(-E), As, D::ASLICE, oz_row_off(t));
        }
        if (t < NCOLT) {
            // column: v_k = T_k 2^s_k, F = max_k exponent of v_k, slices of v_k 2^-F
            float vh[7], vl[7];
            int F = -1000;
#pragma unroll
            for (int k = 0; k < 7; ++k) {
                const float p = sig[k] == -1000 ? 0.0f : pow2i(sig[k]);
                vh[k] = t < D::NTRI ? f_mul(__ldg(Thg + k * D::NTRI + t), p) : 0.0f;
                vl[k] = t < D::NTRI ? f_mul(__ldg(Tlg + k * D::NTRI + t), p) : 0.0f;
                F = max(F, exp_above(vh[k]));
            }
            F = F == -1000 ? 0 : max(F, -100);
            fcol[t] = pow2i(F);
            const int c = t / D::NP, n = t - c * D::NP;
            oz_store_row(vh, vl, pow2i(-F), Bs + c * kOzSlices * D::BSLICE, D::BSLICE, oz_row_off(n));
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        const float er = erow[erow_m];
        for (int c = 0; c < D::NCH; ++c) {
            if (t == 0) {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                // levels 0..7 of slice pairs (i, j), i + j = level; accumulator min(level, 4)
#pragma unroll
                for (int lv = 0; lv < kOzLevels; ++lv)
#pragma unroll
                    for (int i = 0; i <= lv; ++i) {
                        const int j = lv - i;
                        if (i >= kOzSlices || j >= kOzSlices) continue;
                        const int acc = lv < kOzExact ? lv : kOzExact;
                        const bool first = (lv <= kOzExact) && i == 0;
                        const uint64_t ad = make_sdesc(smem_u32(As + i * D::ASLICE), 128, 256);
                        const uint64_t bd = make_sdesc(smem_u32(Bs + (c * kOzSlices + j) * D::BSLICE), 128, 256);
                        tc_mma_f16(tmem + (uint32_t)(acc * D::NP), ad, bd, idesc, first ? 0u : 1u);
                    }
                tc_commit(&sh->mma);
            }
            if (!mbar_wait(&sh->mma, phase, budget)) {
                if (lane == 0) atomicOr(status, kStatusOzTimeout);
                sh->bad = 1;
            }
            phase ^= 1u;
            __syncthreads();
            if (sh->bad) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            if (epi) {
                // the four accumulators of this warp's rows and columns
#pragma unroll 1
                for (int g = 0; g < ECOLS; g += 8) {
                    uint32_t r0[8], r1[8], r2[8], r3[8], r4[8];
                    const uint32_t a0 = lane_addr + (uint32_t)(col0 + g);
                    tmem_ld8_nowait(a0, r0);
                    tmem_ld8_nowait(a0 + D::NP, r1);
                    tmem_ld8_nowait(a0 + 2 * D::NP, r2);
                    tmem_ld8_nowait(a0 + 3 * D::NP, r3);
                    tmem_ld8_nowait(a0 + 4 * D::NP, r4);
                    tmem_wait_ld();
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const df s1 = two_sum(__uint_as_float(r0[q]), __uint_as_float(r1[q]));
                        const df s2 = two_sum(s1.hi, __uint_as_float(r2[q]));
                        const df s3 = two_sum(s2.hi, __uint_as_float(r3[q]));
                        const float err = f_add(f_add(f_add(s1.lo, s2.lo), s3.lo), __uint_as_float(r4[q]));
                        const df v = quick_two_sum(s3.hi, err);
                        const float f = f_mul(er, fcol[c * D::NP + col0 + g + q]);
                        stg[erow_m * D::STG + col0 + g + q] = make_float2(f_mul(v.hi, f), f_mul(v.lo, f));
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncthreads();
            // write the chunk out: each element's entries c NP .. are contiguous in the buffer (two rows per
            // warp pass, 16 lanes per row)
            const int nv = min(D::NP, D::NTRI - c * D::NP);
            const int half = lane >> 4, j = lane & 15;
            for (int m = 2 * warp + half; m < kTcTile; m += 2 * (kOzThreads / 32)) {
                const int64_t e = e0 + m;
                if (e < nt && j < nv) kbuf[e * D::NTRI + c * D::NP + j] = stg[m * D::STG + j];
            }
            __syncthreads();
        }
        if (sh->bad) break;
    }
    // after a timeout, wait (bounded) for the products this block issued before freeing the tensor memory
    if (t == 0 && sh->bad) mbar_wait(&sh->mma, phase ^ 1u, budget);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(D::NCOLS) : "memory");
}

template <int N>
int launch_oz(fgpu_ctx* ctx, int64_t nt, const float4* rec, const float* Th, const float* Tl, void* kbuf) {
    typedef OzDims<N> D;
    auto kern = element_tri_oz_kernel<N>;
    // resident blocks per SM from registers and shared memory, at most 512 / NCOLS so that the
    // blocks' tensor-memory allocations always fit (the occupancy calculator does not count tensor
    // memory); worked out on the first launch on a device, which runs eagerly (a captured assembly
    // needs an earlier one that made its buffers)
    static int per_sm_dev[64] = {0};
    if (ctx->device < 0 || ctx->device >= 64) { ctx->err = "tensor-core element kernel: device index"; return FGPU_ERR_INVALID; }
    int& per_sm = per_sm_dev[ctx->device];
    if (per_sm == 0) {
        FGPU_CUDA_CHECK(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, D::SMEM));
        cudaFuncAttributes fa{};
        FGPU_CUDA_CHECK(ctx, cudaFuncGetAttributes(&fa, kern));
        int smem_sm = 0, regs_sm = 0;
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, ctx->device);
        cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, ctx->device);
        const int by_smem = smem_sm / (D::SMEM + 1024);
        const int by_regs = regs_sm / (((fa.numRegs + 7) & ~7) * kOzThreads);
        per_sm = std::max(1, std::min(std::min(by_smem, by_regs), D::MAXCTA));
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int64_t ntiles = (nt + kTcTile - 1) / kTcTile;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(ntiles, (int64_t)per_sm * sms));
    kern<<<blocks, kOzThreads, D::SMEM, ctx->stream>>>(nt, rec, Th, Tl, static_cast<float2*>(kbuf), ctx->d_status, kOzWaitBudget);
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

}  // namespace

// df64 element buffer (upper triangles) of the affine Laplace/mass form from the coefficient records
int launch_element_tri_tc(fgpu_ctx* ctx, int order, int64_t nt, const float4* rec, const float* Th, const float* Tl, void* kbuf) {
    switch (order) {
        case 1: return launch_oz<4>(ctx, nt, rec, Th, Tl, kbuf);
        case 2: return launch_oz<10>(ctx, nt, rec, Th, Tl, kbuf);
        case 3: return launch_oz<20>(ctx, nt, rec, Th, Tl, kbuf);
        default: ctx->err = "tensor-core element kernel: orders 1-3"; return FGPU_ERR_INVALID;
    }
}

}  // namespace fgpu
