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
// A persistent CTA per SM with three warp roles, synchronised by mbarriers:
//   * slicer warps 0-3 (one element row per thread, then the table columns) load a
//     tile's records, reduce the tile's coefficient exponents, and write the A and B
//     slices, row and column scales of the tile into one of two operand buffers;
//   * warp 4 (one thread) issues, per chunk of NP entries, 20 MMAs (M = 128, N = NP,
//     K = 16: two slice pairs of one level, 7 coefficients each) into one of three
//     tensor-memory buffers of five
//     accumulators, commits each chunk, and frees the operand buffer of a tile once
//     all its products are done;
//   * epilogue warps 5-12 (warps w and w + 4 share the lanes of rows 32 (w % 4) ...
//     and take half of the chunk's columns each) read the five accumulators back with
//     tcgen05.ld, free the tensor-memory buffer, add the levels in double-float, scale,
//     and store the chunk through a shared-memory staging tile with coalesced stores
//     (each element's entries are contiguous in the element buffer).
// So the slicing of tile i + 1, the products of chunk c + 1 and the epilogue of chunk
// c overlap. Every mbarrier wait is bounded: a timeout sets a status bit and a shared
// flag after which no role waits or issues again (named barriers keep their counts),
// and the tensor memory is freed after a bounded wait for the products in flight.
#include <algorithm>
#include <cstdint>

#include "asm_device.cuh"
#include "df64.h"
#include "fgpu_core.h"
#include "tc_ptx.cuh"

namespace fgpu {

namespace {

constexpr int kOzSlicers = 128;      // warps 0-3
constexpr int kOzMmaWarp = 4;
constexpr int kOzEpiWarp0 = 5;       // warps 5-12
constexpr int kOzEpiThreads = 256;
constexpr int kOzThreads = kOzSlicers + 32 + kOzEpiThreads;
constexpr int kOzSlices = 7;         // 8-bit slices per operand
constexpr int kOzExact = 4;          // levels 0 .. 3 summed exactly, one accumulator each
constexpr int kOzLevels = 8;         // levels 0 .. 7 (the last four in one accumulator)
constexpr int kOzAcc = kOzExact + 1;
constexpr int kOzTmemBufs = 3;
constexpr int kOzWaitBudget = 1 << 22;
constexpr int kOzBarEpi = 1, kOzBarSlice = 2;    // named barriers (0 is __syncthreads)

template <int N>
struct OzDims {
    static constexpr int NTRI = N * (N + 1) / 2;
    static constexpr int NP = NTRI <= 16 ? 16 : 32;                 // MMA N of a column chunk
    static constexpr int NCH = (NTRI + NP - 1) / NP;                // chunks
    static constexpr int NCOLT = NCH * NP;                          // table columns incl. padding
    static constexpr int BUFCOLS = kOzAcc * NP;                     // tensor-memory columns of one buffer
    static constexpr int NCOLS = kOzTmemBufs * BUFCOLS <= 256 ? 256 : 512;
    static constexpr int ASLICE = kTcTile * 32;                     // one A slice: 128 rows x 16 bf16
    static constexpr int BSLICE = NP * 32;                          // one B slice of one chunk
    static constexpr int ABUF = kOzSlices * ASLICE;
    static constexpr int BBUF = NCH * (kOzSlices + 1) * BSLICE;   // B pair buffers 0..7 per chunk
    static constexpr int STG = NP + 1;                              // staging row stride (float2), padded
    static constexpr int STGB = kTcTile * STG * 8;
    static constexpr int SMEM_FIXED = 1024 + 2 * ABUF + 2 * BBUF + 2 * NCOLT * 4 + 2 * kTcTile * 4 + 4 * 8 * 4 + 256;
    static constexpr int NSTG = SMEM_FIXED + 2 * STGB <= 232448 ? 2 : 1;   // staging tiles (two when they fit)
    static constexpr int SMEM_USED = SMEM_FIXED + NSTG * STGB;
    static constexpr int MAXCTA = 512 / NCOLS;
    static_assert(NCOLT <= 2 * kOzSlicers, "two table columns per slicer thread at most");
    static_assert(kOzTmemBufs * BUFCOLS <= NCOLS, "tensor-memory buffers");
};

struct OzShared {
    uint64_t ab_full[2], ab_empty[2], meta_empty[2], tm_full[kOzTmemBufs], tm_empty[kOzTmemBufs];
    uint32_t tmem;
    int bad;
    int sigw[4][8];
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

// the slices of the seven values (h_k + l_k) q of one operand row, as bf16 pairs of slices along K:
// A (shift = +1): buffer p holds slice p in K = 0..7 and slice p + 1 in K = 8..15 (p = 0..6);
// B (shift = -1): buffer p holds slice p in K = 0..7 and slice p - 1 in K = 8..15 (p = 0..7), so that
// one MMA of A buffer i with B buffer j adds the products of the slice pairs (i, j) and (i + 1, j - 1),
// both of level i + j. Missing slices are zero.
template <int SHIFT>
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
    constexpr int NBUF = SHIFT > 0 ? kOzSlices : kOzSlices + 1;
#pragma unroll
    for (int p = 0; p < NBUF; ++p) {
        const int lo = p, hi = p + SHIFT;                       // slices in K = 0..7 and K = 8..15
        const uint4 z = make_uint4(0u, 0u, 0u, 0u);
        const uint4 vlo = lo < kOzSlices ? make_uint4(w[lo < kOzSlices ? lo : 0][0], w[lo < kOzSlices ? lo : 0][1],
                                                      w[lo < kOzSlices ? lo : 0][2], w[lo < kOzSlices ? lo : 0][3]) : z;
        const bool hv = hi >= 0 && hi < kOzSlices;
        const int hc = hv ? hi : 0;
        const uint4 vhi = hv ? make_uint4(w[hc][0], w[hc][1], w[hc][2], w[hc][3]) : z;
        *reinterpret_cast<uint4*>(base + p * stride + off) = vlo;
        *reinterpret_cast<uint4*>(base + p * stride + off + 128) = vhi;
    }
}

__device__ __forceinline__ void named_bar(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }
__device__ __forceinline__ bool oz_bad(const OzShared* sh) { return *(volatile const int*)&sh->bad != 0; }
// bounded wait for an mbarrier phase that lets the thread sleep up to 0.5 us per try (fewer issue slots
// spent polling); returns false when the budget ran out
__device__ __forceinline__ bool mbar_wait_sleep(void* mbar, uint32_t phase, int budget) {
    uint32_t done = 0;
    for (int it = 0; it < budget; ++it) {
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.b32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(smem_u32(mbar)), "r"(phase), "r"(500u)
            : "memory");
        if (done) return true;
    }
    return false;
}
// bounded wait unless a failure was already seen; a timeout raises the status bit and the shared flag
__device__ __forceinline__ void oz_wait(OzShared* sh, uint64_t* bar, uint32_t parity, int budget, int* status) {
    if (oz_bad(sh)) return;
    if (!mbar_wait_sleep(bar, parity, budget)) {
        atomicOr(status, kStatusOzTimeout);
        *(volatile int*)&sh->bad = 1;
    }
}

template <int N>
__global__ void __launch_bounds__(kOzThreads) element_tri_oz_kernel(int64_t nt, const float4* __restrict__ rec,
                                                                   const float* __restrict__ Thg, const float* __restrict__ Tlg,
                                                                   float2* __restrict__ kbuf, int* __restrict__ status, int budget) {
    typedef OzDims<N> D;
    extern __shared__ __align__(1024) unsigned char oz_smem[];
    unsigned char* base = (unsigned char*)(((uintptr_t)oz_smem + 1023) & ~(uintptr_t)1023);
    unsigned char* As = base;                                            // 2 buffers of kOzSlices A slices
    unsigned char* Bs = As + 2 * D::ABUF;                                // 2 buffers of [chunk][slice]
    float2* stg = reinterpret_cast<float2*>(Bs + 2 * D::BBUF);          // NSTG staging tiles
    float* fcol = reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(stg) + D::NSTG * D::STGB);   // [2][NCOLT] 2^F_t
    float* erow = fcol + 2 * D::NCOLT;                                   // [2][128] 2^E_m
    OzShared* sh = reinterpret_cast<OzShared*>(((uintptr_t)(erow + 2 * kTcTile) + 15) & ~(uintptr_t)15);
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;

    // zero all operand buffers once: the K columns 7..15 stay zero
    for (int k = t; k < (2 * D::ABUF + 2 * D::BBUF) / 16; k += kOzThreads) reinterpret_cast<uint4*>(As)[k] = make_uint4(0u, 0u, 0u, 0u);
    if (t == 0) {
        for (int i = 0; i < 2; ++i) {
            mbar_init(&sh->ab_full[i], kOzSlicers);
            mbar_init(&sh->ab_empty[i], 1);
            mbar_init(&sh->meta_empty[i], kOzEpiThreads / 32);
        }
        for (int i = 0; i < kOzTmemBufs; ++i) {
            mbar_init(&sh->tm_full[i], 1);
            mbar_init(&sh->tm_empty[i], kOzEpiThreads / 32);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        sh->bad = 0;
    }
    if (warp == kOzMmaWarp) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sh->tmem)),
                     "r"(D::NCOLS) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = sh->tmem;
    const int64_t ntiles = (nt + kTcTile - 1) / kTcTile;
    const int ntile_mine = blockIdx.x < ntiles ? (int)((ntiles - 1 - blockIdx.x) / gridDim.x + 1) : 0;

    if (warp < kOzSlicers / 32) {
        // ---------------- slicers ----------------
        // the records of a tile are loaded before the wait for its operand buffer (the next tile's
        // right after the current tile's slices are out)
        float nh[7], nl[7];
#pragma unroll
        for (int k = 0; k < 7; ++k) nh[k] = nl[k] = 0.0f;
        if (ntile_mine > 0 && (int64_t)blockIdx.x * kTcTile + t < nt) load_record(rec + 4 * ((int64_t)blockIdx.x * kTcTile + t), nh, nl, true);
        for (int it = 0; it < ntile_mine; ++it) {
            const int s = it & 1;
            float ch[7], cl[7];
#pragma unroll
            for (int k = 0; k < 7; ++k) {
                ch[k] = nh[k];
                cl[k] = nl[k];
                nh[k] = nl[k] = 0.0f;
            }
            const int64_t en = ((int64_t)blockIdx.x + (int64_t)(it + 1) * gridDim.x) * kTcTile + t;
            if (it + 1 < ntile_mine && en < nt) load_record(rec + 4 * en, nh, nl, true);
            if (it >= 2) {
                oz_wait(sh, &sh->ab_empty[s], ((it - 2) >> 1) & 1u, budget, status);
                oz_wait(sh, &sh->meta_empty[s], ((it - 2) >> 1) & 1u, budget, status);
            }
#pragma unroll
            for (int k = 0; k < 7; ++k) {
                const int m = __reduce_max_sync(0xFFFFFFFFu, exp_above(ch[k]));
                if (lane == 0) sh->sigw[warp][k] = m;
            }
            named_bar(kOzBarSlice, kOzSlicers);
            int sig[7];
#pragma unroll
            for (int k = 0; k < 7; ++k) {
                const int m = max(max(sh->sigw[0][k], sh->sigw[1][k]), max(sh->sigw[2][k], sh->sigw[3][k]));
                sig[k] = m < -100 ? -1000 : min(m, 100);
            }
            named_bar(kOzBarSlice, kOzSlicers);          // every slicer has read the exponents
            {
                // row: u_k = c_k 2^-s_k (|u_k| < 1), E = max_k exponent of u_k, slices of u_k 2^-E
                float uh[7], ul[7];
                int E = -1000;
#pragma unroll
                for (int k = 0; k < 7; ++k) {
                    const float pk = sig[k] == -1000 ? 0.0f : pow2i(-sig[k]);
                    uh[k] = f_mul(ch[k], pk);
                    ul[k] = f_mul(cl[k], pk);
                    E = max(E, exp_above(uh[k]));
                }
                E = E == -1000 ? 0 : max(E, -60);
                erow[s * kTcTile + t] = pow2i(E);
                oz_store_row<1>(uh, ul, pow2i(-E), As + s * D::ABUF, D::ASLICE, oz_row_off(t));
            }
            for (int col = t; col < D::NCOLT; col += kOzSlicers) {
                // column: v_k = T_k 2^s_k, F = max_k exponent of v_k, slices of v_k 2^-F
                float vh[7], vl[7];
                int F = -1000;
#pragma unroll
                for (int k = 0; k < 7; ++k) {
                    const float pk = sig[k] == -1000 ? 0.0f : pow2i(sig[k]);
                    vh[k] = col < D::NTRI ? f_mul(__ldg(Thg + k * D::NTRI + col), pk) : 0.0f;
                    vl[k] = col < D::NTRI ? f_mul(__ldg(Tlg + k * D::NTRI + col), pk) : 0.0f;
                    F = max(F, exp_above(vh[k]));
                }
                F = F == -1000 ? 0 : max(F, -100);
                fcol[s * D::NCOLT + col] = pow2i(F);
                const int c = col / D::NP, n = col - c * D::NP;
                oz_store_row<-1>(vh, vl, pow2i(-F), Bs + s * D::BBUF + c * (kOzSlices + 1) * D::BSLICE, D::BSLICE, oz_row_off(n));
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_arrive(&sh->ab_full[s]);
        }
    } else if (warp == kOzMmaWarp) {
        // ---------------- MMA issue (one thread) ----------------
        if (lane == 0) {
            constexpr uint32_t idesc = make_idesc_bf16(D::NP);
            uint32_t q = 0, last = 0xFFFFFFFFu;     // chunk counter, last committed chunk
            for (int it = 0; it < ntile_mine; ++it) {
                const int s = it & 1;
                oz_wait(sh, &sh->ab_full[s], (it >> 1) & 1u, budget, status);
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                for (int c = 0; c < D::NCH; ++c, ++q) {
                    const uint32_t b = q % kOzTmemBufs;
                    if (q >= (uint32_t)kOzTmemBufs) oz_wait(sh, &sh->tm_empty[b], ((q / kOzTmemBufs) - 1) & 1u, budget, status);
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    if (oz_bad(sh)) continue;
                    // descriptors of buffer 0; the others are at a fixed stride (the start address field
                    // holds address / 16 in its low bits, and no buffer crosses 256 KB)
                    const uint64_t ad0 = make_sdesc(smem_u32(As + s * D::ABUF), 128, 256);
                    const uint64_t bd0 = make_sdesc(smem_u32(Bs + s * D::BBUF + c * (kOzSlices + 1) * D::BSLICE), 128, 256);
                    const uint32_t dcol = tmem + b * D::BUFCOLS;
                    // level lv: A pair buffers i = 0, 2, 4, 6 against B pair buffers lv - i (pairs (i, lv - i)
                    // and (i + 1, lv - i - 1)); accumulator min(lv, 4)
#pragma unroll
                    for (int lv = 0; lv < kOzLevels; ++lv)
#pragma unroll
                        for (int i = 0; i <= lv && i < kOzSlices; i += 2) {
                            const int j = lv - i;
                            if (j > kOzSlices) continue;
                            const int acc = lv < kOzExact ? lv : kOzExact;
                            const bool first = (lv <= kOzExact) && i == 0;
                            tc_mma_f16(dcol + (uint32_t)(acc * D::NP), ad0 + (uint64_t)(i * D::ASLICE / 16),
                                       bd0 + (uint64_t)(j * D::BSLICE / 16), idesc, first ? 0u : 1u);
                        }
                    tc_commit(&sh->tm_full[b]);
                    last = q;
                }
                if (!oz_bad(sh)) tc_commit(&sh->ab_empty[s]);    // the tile's products done: its operands are free
            }
            // after a failure, wait (bounded) for the products already issued: the last chunk's commit
            // tracks all of them
            if (oz_bad(sh) && last != 0xFFFFFFFFu) mbar_wait(&sh->tm_full[last % kOzTmemBufs], (last / kOzTmemBufs) & 1u, budget);
        }
        __syncwarp();
    } else {
        // ---------------- epilogue ----------------
        const int ew = warp - kOzEpiWarp0;                      // 0..7
        const int grp = warp & 3;                               // tensor-memory lane group
        constexpr int ECOLS = D::NP / 2;
        const int col0 = (ew >> 2) * ECOLS;
        const int m = 32 * grp + lane;                          // this thread's row
        const uint32_t lane_addr = tmem + ((uint32_t)(32 * grp) << 16);
        uint32_t q = 0;
        for (int it = 0; it < ntile_mine; ++it) {
            const int s = it & 1;
            const int64_t e0 = ((int64_t)blockIdx.x + (int64_t)it * gridDim.x) * kTcTile;
            oz_wait(sh, &sh->ab_full[s], (it >> 1) & 1u, budget, status);   // scales of the tile written
            const float er = erow[s * kTcTile + m];
            for (int c = 0; c < D::NCH; ++c, ++q) {
                const uint32_t b = q % kOzTmemBufs;
                oz_wait(sh, &sh->tm_full[b], (q / kOzTmemBufs) & 1u, budget, status);
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                float2* st = stg + (q % (uint32_t)D::NSTG) * (D::STGB / 8);
                if (__all_sync(0xFFFFFFFFu, !oz_bad(sh))) {          // warp-uniform: tcgen05.ld is .sync.aligned
                    uint32_t r[kOzAcc][ECOLS];
                    const uint32_t a0 = lane_addr + b * D::BUFCOLS + (uint32_t)col0;
#pragma unroll
                    for (int a = 0; a < kOzAcc; ++a) {
                        if constexpr (ECOLS == 16) tmem_ld16_nowait(a0 + a * D::NP, r[a]);
                        else tmem_ld8_nowait(a0 + a * D::NP, r[a]);
                    }
                    tmem_wait_ld();
                    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&sh->tm_empty[b]);
#pragma unroll
                    for (int x = 0; x < ECOLS; ++x) {
                        const df s1 = two_sum(__uint_as_float(r[0][x]), __uint_as_float(r[1][x]));
                        const df s2 = two_sum(s1.hi, __uint_as_float(r[2][x]));
                        const df s3 = two_sum(s2.hi, __uint_as_float(r[3][x]));
                        const float err = f_add(f_add(f_add(s1.lo, s2.lo), s3.lo), __uint_as_float(r[4][x]));
                        const df v = quick_two_sum(s3.hi, err);
                        const float f = f_mul(er, fcol[s * D::NCOLT + c * D::NP + col0 + x]);
                        st[m * D::STG + col0 + x] = make_float2(f_mul(v.hi, f), f_mul(v.lo, f));
                    }
                }
                named_bar(kOzBarEpi, kOzEpiThreads);
                // the chunk out: each element's entries c NP .. are contiguous in the buffer
                const int nv = min(D::NP, D::NTRI - c * D::NP);
                if (D::NP == 32) {
                    for (int row = ew; row < kTcTile; row += kOzEpiThreads / 32) {
                        const int64_t e = e0 + row;
                        if (e < nt && lane < nv && !oz_bad(sh)) kbuf[e * D::NTRI + c * D::NP + lane] = st[row * D::STG + lane];
                    }
                } else {
                    const int half = lane >> 4, j = lane & 15;
                    for (int row = 2 * ew + half; row < kTcTile; row += 2 * (kOzEpiThreads / 32)) {
                        const int64_t e = e0 + row;
                        if (e < nt && j < nv && !oz_bad(sh)) kbuf[e * D::NTRI + c * D::NP + j] = st[row * D::STG + j];
                    }
                }
                if constexpr (D::NSTG == 1) named_bar(kOzBarEpi, kOzEpiThreads);   // the one staging tile is read
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&sh->meta_empty[s]);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == kOzMmaWarp) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(D::NCOLS) : "memory");
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
        FGPU_CUDA_CHECK(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, D::SMEM_USED));
        cudaFuncAttributes fa{};
        FGPU_CUDA_CHECK(ctx, cudaFuncGetAttributes(&fa, kern));
        int smem_sm = 0, regs_sm = 0;
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, ctx->device);
        cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, ctx->device);
        const int by_smem = smem_sm / (D::SMEM_USED + 1024);
        const int by_regs = regs_sm / (((fa.numRegs + 7) & ~7) * kOzThreads);
        per_sm = std::max(1, std::min(std::min(by_smem, by_regs), D::MAXCTA));
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int64_t ntiles = (nt + kTcTile - 1) / kTcTile;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(ntiles, (int64_t)per_sm * sms));
    kern<<<blocks, kOzThreads, D::SMEM_USED, ctx->stream>>>(nt, rec, Th, Tl, static_cast<float2*>(kbuf), ctx->d_status, kOzWaitBudget);
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
