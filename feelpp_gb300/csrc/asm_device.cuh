// Device helpers shared by the affine Laplace/mass assembly kernels (assemble.cu,
// stream_asm.cu): the df64 element coefficient record and the element-matrix
// entries formed from it and the reference tensors.
#pragma once
#include <cstdint>

#include "df64.h"
#include "fgpu_core.h"

namespace fgpu {

enum GatherMode { kModeF32 = 0, kModeDF64 = 1 };

// Element coefficient record, 16 floats (64 B):
//   [c0 c1 c2 c3 | c4 c5 c6 J]  high parts,  [c0 c1 c2 c3 | c4 c5 c6 J]  low parts
// with c_0..5 = kappa * (C^T C)_{00,11,22,01,02,12} / |det K| (= kappa J B^T B, C the
// cofactor matrix of K, B = C / det K), c_6 = mass * |det K|, J = |det K|.
// K's entries are formed in FP64 (9 subtractions of vertex coordinates), the rest
// in df64 (geomap.hpp:1971-1991, 2310-2350). ksc: an extra factor of kappa
// (a time-dependent coefficient read from device memory).
__device__ __forceinline__ void geometry_df_record(int64_t e, const double* __restrict__ xyz, const int32_t* __restrict__ tets,
                                                   const double* __restrict__ kappa, df kc, df mc, df ksc,
                                                   float4* __restrict__ o, int* __restrict__ status) {
    int4 t = *reinterpret_cast<const int4*>(tets + 4 * e);
    const double* X0 = xyz + 3 * (int64_t)t.x;
    const double* Xv[3] = {xyz + 3 * (int64_t)t.y, xyz + 3 * (int64_t)t.z, xyz + 3 * (int64_t)t.w};
    df K[9];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r) K[r * 3 + c] = df_scale(d2df(Xv[c][r] - X0[r]), 0.5f);
    df C[9];
    C[0] = df_sub(df_mul(K[4], K[8]), df_mul(K[5], K[7]));
    C[1] = df_sub(df_mul(K[5], K[6]), df_mul(K[3], K[8]));
    C[2] = df_sub(df_mul(K[3], K[7]), df_mul(K[4], K[6]));
    C[3] = df_sub(df_mul(K[2], K[7]), df_mul(K[1], K[8]));
    C[4] = df_sub(df_mul(K[0], K[8]), df_mul(K[2], K[6]));
    C[5] = df_sub(df_mul(K[1], K[6]), df_mul(K[0], K[7]));
    C[6] = df_sub(df_mul(K[1], K[5]), df_mul(K[2], K[4]));
    C[7] = df_sub(df_mul(K[2], K[3]), df_mul(K[0], K[5]));
    C[8] = df_sub(df_mul(K[0], K[4]), df_mul(K[1], K[3]));
    df det = df_add(df_add(df_mul(K[0], C[0]), df_mul(K[1], C[1])), df_mul(K[2], C[2]));
    df J = det.hi < 0.0f ? df_neg(det) : det;
    if (!(J.hi > 0.0f) || !isfinite(J.hi)) atomicOr(status, kStatusBadElement);
    df inv = df_recip(J);
    df s = df_mul(df_mul(kappa ? d2df(kappa[e]) : kc, ksc), inv);
    const int pa[6] = {0, 1, 2, 0, 0, 1}, pb[6] = {0, 1, 2, 1, 2, 2};
    df c[8];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        df g = df_add(df_add(df_mul(C[pa[k]], C[pb[k]]), df_mul(C[3 + pa[k]], C[3 + pb[k]])), df_mul(C[6 + pa[k]], C[6 + pb[k]]));
        c[k] = df_mul(s, g);
    }
    c[6] = df_mul(mc, J);
    c[7] = J;
    o[0] = make_float4(c[0].hi, c[1].hi, c[2].hi, c[3].hi);
    o[1] = make_float4(c[4].hi, c[5].hi, c[6].hi, c[7].hi);
    o[2] = make_float4(c[0].lo, c[1].lo, c[2].lo, c[3].lo);
    o[3] = make_float4(c[4].lo, c[5].lo, c[6].lo, c[7].lo);
}

// Element-matrix entry K_e(i, j) = sum_k c_k T_k(i, j) (the 7 reference tensors
// of the affine Laplace/mass form) from the element's coefficient record.
// df64: each product c_k T_k is formed exactly (TwoProduct by FMA, plus the
// cross terms of the lo parts) and summed with TwoSum; binary32: an FMA chain.
// (tables Th/Tl of 7 slices of `stride` floats; tix = the entry's index in a slice;
// ch/cl: the record's 7 coefficients, hi and lo parts)
__device__ __forceinline__ df coef_entry_df(const float* ch, const float* cl, const float* __restrict__ Th,
                                            const float* __restrict__ Tl, int stride, int tix) {
    float s = 0.0f, err = 0.0f;
#pragma unroll
    for (int k = 0; k < 7; ++k) {
        const float th = Th[k * stride + tix], tl = Tl[k * stride + tix];
        const float p = f_mul(ch[k], th);
        const float pe = f_fma(ch[k], th, -p);
        err = f_fma(ch[k], tl, err);
        err = f_fma(cl[k], th, err);
        err = f_add(err, pe);
        if (k == 0) {
            s = p;
        } else {
            df t = two_sum(s, p);
            s = t.hi;
            err = f_add(err, t.lo);
        }
    }
    return quick_two_sum(s, err);
}
// the same sum with the entry's table values already in registers (th[k], tl[k])
__device__ __forceinline__ df coef_entry_df_reg(const float* ch, const float* cl, const float* th, const float* tl) {
    float s = 0.0f, err = 0.0f;
#pragma unroll
    for (int k = 0; k < 7; ++k) {
        const float p = f_mul(ch[k], th[k]);
        const float pe = f_fma(ch[k], th[k], -p);
        err = f_fma(ch[k], tl[k], err);
        err = f_fma(cl[k], th[k], err);
        err = f_add(err, pe);
        if (k == 0) {
            s = p;
        } else {
            df t = two_sum(s, p);
            s = t.hi;
            err = f_add(err, t.lo);
        }
    }
    return quick_two_sum(s, err);
}
__device__ __forceinline__ float coef_entry_f(const float* ch, const float* __restrict__ Th, int stride, int tix) {
    float v = 0.0f;
#pragma unroll
    for (int k = 0; k < 7; ++k) v = fmaf(ch[k], Th[k * stride + tix], v);
    return v;
}
__device__ __forceinline__ void load_record(const float4* __restrict__ rp, float* ch, float* cl, bool lo) {
    const float4 h0 = __ldg(rp), h1 = __ldg(rp + 1);
    ch[0] = h0.x; ch[1] = h0.y; ch[2] = h0.z; ch[3] = h0.w; ch[4] = h1.x; ch[5] = h1.y; ch[6] = h1.z;
    if (lo) {
        const float4 l0 = __ldg(rp + 2), l1 = __ldg(rp + 3);
        cl[0] = l0.x; cl[1] = l0.y; cl[2] = l0.z; cl[3] = l0.w; cl[4] = l1.x; cl[5] = l1.y; cl[6] = l1.z;
    }
}
// the same record from shared memory
__device__ __forceinline__ void load_record_shared(const float4* rp, float* ch, float* cl, bool lo) {
    const float4 h0 = rp[0], h1 = rp[1];
    ch[0] = h0.x; ch[1] = h0.y; ch[2] = h0.z; ch[3] = h0.w; ch[4] = h1.x; ch[5] = h1.y; ch[6] = h1.z;
    if (lo) {
        const float4 l0 = rp[2], l1 = rp[3];
        cl[0] = l0.x; cl[1] = l0.y; cl[2] = l0.z; cl[3] = l0.w; cl[4] = l1.x; cl[5] = l1.y; cl[6] = l1.z;
    }
}
}  // namespace fgpu
