// Number policies and the three CG kernels shared by the CSR solver
// (solve.cu) and the matrix-free solver (matfree.cu). See solve.cu for the
// algorithm; everything here is header-only device code.
#pragma once
#include <cstdint>

#include "df64.h"
#include "fgpu_core.h"

namespace fgpu {

static constexpr int kVecBlocks = 152 * 4;
static constexpr int kVecThreads = 256;

// ---------------------------------------------------------------------------
// number policies
//   S: vector storage, V: matrix value storage, A: arithmetic type of vector
//   entries, D: accumulation type of dot products (8 bytes)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 dfpack(df v) { return make_float2(v.hi, v.lo); }
__device__ __forceinline__ df dfun(float2 v) { return df{v.x, v.y}; }

struct PolF64 {
    static constexpr int id = 0;
    typedef double S;
    typedef double V;
    typedef double A;
    typedef double D;
    static __device__ __forceinline__ A ld(S s) { return s; }
    static __device__ __forceinline__ S st(A a) { return a; }
    static __device__ __forceinline__ A ldv(V v) { return v; }
    static __device__ __forceinline__ A zero() { return 0.0; }
    static __device__ __forceinline__ A one() { return 1.0; }
    static __device__ __forceinline__ A add(A a, A b) { return a + b; }
    static __device__ __forceinline__ A sub(A a, A b) { return a - b; }
    static __device__ __forceinline__ A mul(A a, A b) { return a * b; }
    static __device__ __forceinline__ A madd(A s, A a, A b) { return fma(a, b, s); }
    static __device__ __forceinline__ A recip(A a) { return 1.0 / a; }
    static __device__ __forceinline__ bool nonzero(A a) { return a != 0.0; }
    static __device__ __forceinline__ A shfl_xor(A a, int o) { return __shfl_xor_sync(0xffffffffu, a, o); }
    static __device__ __forceinline__ D dzero() { return 0.0; }
    static __device__ __forceinline__ D dadd(D s, D t) { return s + t; }
    static __device__ __forceinline__ D dmadd(D s, A a, A b) { return fma(a, b, s); }
    static __device__ __forceinline__ D dshfl_xor(D a, int o) { return __shfl_xor_sync(0xffffffffu, a, o); }
    static __device__ __forceinline__ bool dpos(D a) { return a > 0.0; }
    static __device__ __forceinline__ bool dle(D a, D b) { return a <= b; }
    static __device__ __forceinline__ D ddiv(D a, D b) { return a / b; }
    static __device__ __forceinline__ D dmul(D a, D b) { return a * b; }
    static __device__ __forceinline__ A from_d(D d) { return d; }
    static __device__ __forceinline__ A neg_from_d(D d) { return -d; }
    static D host_from_double(double x) { return x; }
    static double host_to_double(D d) { return d; }
};

struct PolDF64 {
    static constexpr int id = 1;
    typedef float2 S;
    typedef float2 V;
    typedef df A;
    typedef float2 D;
    static __device__ __forceinline__ A ld(S s) { return dfun(s); }
    static __device__ __forceinline__ S st(A a) { return dfpack(a); }
    static __device__ __forceinline__ A ldv(V v) { return dfun(v); }
    static __device__ __forceinline__ A zero() { return df{0.0f, 0.0f}; }
    static __device__ __forceinline__ A one() { return df{1.0f, 0.0f}; }
    static __device__ __forceinline__ A add(A a, A b) { return df_add(a, b); }
    static __device__ __forceinline__ A sub(A a, A b) { return df_sub(a, b); }
    static __device__ __forceinline__ A mul(A a, A b) { return df_mul(a, b); }
    static __device__ __forceinline__ A madd(A s, A a, A b) { return df_add(s, df_mul(a, b)); }
    static __device__ __forceinline__ A recip(A a) { return df_recip(a); }
    static __device__ __forceinline__ bool nonzero(A a) { return a.hi != 0.0f; }
    static __device__ __forceinline__ A shfl_xor(A a, int o) {
        return df{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)};
    }
    static __device__ __forceinline__ D dzero() { return make_float2(0.0f, 0.0f); }
    static __device__ __forceinline__ D dadd(D s, D t) { return dfpack(df_add(dfun(s), dfun(t))); }
    static __device__ __forceinline__ D dmadd(D s, A a, A b) { return dfpack(df_add(dfun(s), df_mul(a, b))); }
    static __device__ __forceinline__ D dshfl_xor(D a, int o) {
        return make_float2(__shfl_xor_sync(0xffffffffu, a.x, o), __shfl_xor_sync(0xffffffffu, a.y, o));
    }
    static __device__ __forceinline__ bool dpos(D a) { return a.x > 0.0f; }
    static __device__ __forceinline__ bool dle(D a, D b) { return a.x <= b.x; }
    static __device__ __forceinline__ D ddiv(D a, D b) { return dfpack(df_mul(dfun(a), df_recip(dfun(b)))); }
    static __device__ __forceinline__ D dmul(D a, D b) { return dfpack(df_mul(dfun(a), dfun(b))); }
    static __device__ __forceinline__ A from_d(D d) { return dfun(d); }
    static __device__ __forceinline__ A neg_from_d(D d) { return df_neg(dfun(d)); }
    static D host_from_double(double x) { df v = d2df(x); D r; r.x = v.hi; r.y = v.lo; return r; }
    static double host_to_double(D d) { return (double)d.x + (double)d.y; }
};

struct PolF32 {
    static constexpr int id = 2;
    typedef float S;
    typedef float V;
    typedef float A;
    typedef float2 D;
    static __device__ __forceinline__ A ld(S s) { return s; }
    static __device__ __forceinline__ S st(A a) { return a; }
    static __device__ __forceinline__ A ldv(V v) { return v; }
    static __device__ __forceinline__ A zero() { return 0.0f; }
    static __device__ __forceinline__ A one() { return 1.0f; }
    static __device__ __forceinline__ A add(A a, A b) { return f_add(a, b); }
    static __device__ __forceinline__ A sub(A a, A b) { return f_sub(a, b); }
    static __device__ __forceinline__ A mul(A a, A b) { return f_mul(a, b); }
    static __device__ __forceinline__ A madd(A s, A a, A b) { return f_fma(a, b, s); }
    static __device__ __forceinline__ A recip(A a) { return __frcp_rn(a); }
    static __device__ __forceinline__ bool nonzero(A a) { return a != 0.0f; }
    static __device__ __forceinline__ A shfl_xor(A a, int o) { return __shfl_xor_sync(0xffffffffu, a, o); }
    static __device__ __forceinline__ D dzero() { return make_float2(0.0f, 0.0f); }
    static __device__ __forceinline__ D dadd(D s, D t) { return dfpack(df_add(dfun(s), dfun(t))); }
    static __device__ __forceinline__ D dmadd(D s, A a, A b) {
        const float p = f_mul(a, b);
        return dfpack(df_add(dfun(s), df{p, f_fma(a, b, -p)}));
    }
    static __device__ __forceinline__ D dshfl_xor(D a, int o) {
        return make_float2(__shfl_xor_sync(0xffffffffu, a.x, o), __shfl_xor_sync(0xffffffffu, a.y, o));
    }
    static __device__ __forceinline__ bool dpos(D a) { return a.x > 0.0f; }
    static __device__ __forceinline__ bool dle(D a, D b) { return a.x <= b.x; }
    static __device__ __forceinline__ D ddiv(D a, D b) { return dfpack(df_mul(dfun(a), df_recip(dfun(b)))); }
    static __device__ __forceinline__ D dmul(D a, D b) { return dfpack(df_mul(dfun(a), dfun(b))); }
    static __device__ __forceinline__ A from_d(D d) { return f_add(d.x, d.y); }
    static __device__ __forceinline__ A neg_from_d(D d) { return -f_add(d.x, d.y); }
    static D host_from_double(double x) { df v = d2df(x); D r; r.x = v.hi; r.y = v.lo; return r; }
    static double host_to_double(D d) { return (double)d.x + (double)d.y; }
};

template <class PL>
struct CGScalars {
    typename PL::D rz[2];     // r.z of the current iteration, double-buffered by iteration parity
    typename PL::D rr, bb, tol2;
    typename PL::D pq;        // p.Ap of the last iteration (read by the Lanczos estimate)
    int it, done, fail, pad;
};

// Block reduction of a D value (valid on thread 0).
template <class PL>
__device__ __forceinline__ typename PL::D block_sum(typename PL::D v, typename PL::D* sh) {
    for (int o = 16; o > 0; o >>= 1) v = PL::dadd(v, PL::dshfl_xor(v, o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    typename PL::D s = PL::dzero();
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s = PL::dadd(s, sh[k]);
    return s;
}

template <class PL>
__device__ __forceinline__ typename PL::D sum_partials(const typename PL::D* __restrict__ partial, int nb, typename PL::D* sh) {
    typename PL::D a = PL::dzero();
    for (int k = threadIdx.x; k < nb; k += blockDim.x) a = PL::dadd(a, partial[k]);
    return block_sum<PL>(a, sh);
}

// y = A x (mode 0) or y = b - A x (mode 1); optional per-block partial of dot(w, y).
template <class PL, int G>
__global__ void __launch_bounds__(256) spmv_kernel(int64_t nrows, const int64_t* __restrict__ ia, const int32_t* __restrict__ ja,
                                                  const typename PL::V* __restrict__ val, const typename PL::S* __restrict__ x,
                                                  typename PL::S* __restrict__ y, int mode, const typename PL::S* __restrict__ b,
                                                  const typename PL::S* __restrict__ wdot, typename PL::D* __restrict__ partial,
                                                  const CGScalars<PL>* __restrict__ sc) {
    if (sc && sc->done) return;
    __shared__ typename PL::D sh[32];
    const int gpb = blockDim.x / G;
    const int g = threadIdx.x / G, lane = threadIdx.x % G;
    typename PL::D dsum = PL::dzero();
    for (int64_t r0 = (int64_t)blockIdx.x * gpb; r0 < nrows; r0 += (int64_t)gridDim.x * gpb) {
        const int64_t r = r0 + g;
        // row sums accumulate in the dot-product type D (binary64, or df64 for the
        // binary32 and df64 policies): a binary32 row sum of a smooth vector loses
        // up to kappa(A) u32 to cancellation, which stalls CG on stiff systems
        typename PL::D sd = PL::dzero();
        if (r < nrows) {
            const int64_t pe = ia[r + 1];
            for (int64_t p = ia[r] + lane; p < pe; p += G) sd = PL::dmadd(sd, PL::ldv(val[p]), PL::ld(x[ja[p]]));
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) sd = PL::dadd(sd, PL::dshfl_xor(sd, o));
        if (r < nrows && lane == 0) {
            const typename PL::A s = PL::from_d(sd);
            const typename PL::S v = PL::st(mode == 1 ? PL::sub(PL::ld(b[r]), s) : s);
            y[r] = v;
            if (wdot) dsum = PL::dmadd(dsum, PL::ld(wdot[r]), PL::ld(v));
        }
    }
    if (partial) {
        const typename PL::D t = block_sum<PL>(dsum, sh);
        if (threadIdx.x == 0) partial[blockIdx.x] = t;
    }
}

template <class PL>
__global__ void diag_inv_kernel(int64_t nrows, const int64_t* __restrict__ ia, const int32_t* __restrict__ ja,
                                const typename PL::V* __restrict__ val, typename PL::S* __restrict__ dinv, int use_pc) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
        typename PL::A d = PL::zero();
        for (int64_t p = ia[r]; p < ia[r + 1]; ++p)
            if (ja[p] == r) d = PL::ldv(val[p]);
        dinv[r] = PL::st((use_pc && PL::nonzero(d)) ? PL::recip(d) : PL::one());
    }
}

// z = dinv r, p = z, partials (r.r, r.z, b.b)
template <class PL>
__global__ void cg_init_kernel(int64_t n, const typename PL::S* __restrict__ b, const typename PL::S* __restrict__ r,
                               const typename PL::S* __restrict__ dinv, typename PL::S* __restrict__ z,
                               typename PL::S* __restrict__ p, typename PL::D* __restrict__ partial) {
    __shared__ typename PL::D sh[32];
    typename PL::D rr = PL::dzero(), rz = PL::dzero(), bb = PL::dzero();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const typename PL::A ri = PL::ld(r[i]);
        const typename PL::S zs = PL::st(PL::mul(PL::ld(dinv[i]), ri));
        z[i] = zs;
        p[i] = zs;
        rr = PL::dmadd(rr, ri, ri);
        rz = PL::dmadd(rz, ri, PL::ld(zs));
        const typename PL::A bi = PL::ld(b[i]);
        bb = PL::dmadd(bb, bi, bi);
    }
    typename PL::D a = block_sum<PL>(rr, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = a;
    a = block_sum<PL>(rz, sh);
    if (threadIdx.x == 0) partial[gridDim.x + blockIdx.x] = a;
    a = block_sum<PL>(bb, sh);
    if (threadIdx.x == 0) partial[2 * gridDim.x + blockIdx.x] = a;
}

template <class PL>
__global__ void cg_init_scalars(const typename PL::D* __restrict__ partial, int nb, typename PL::D rtol2, CGScalars<PL>* sc) {
    __shared__ typename PL::D sh[32];
    const typename PL::D a = sum_partials<PL>(partial, nb, sh);
    const typename PL::D c = sum_partials<PL>(partial + nb, nb, sh);
    const typename PL::D d = sum_partials<PL>(partial + 2 * nb, nb, sh);
    if (threadIdx.x == 0) {
        sc->rr = a; sc->rz[0] = c; sc->rz[1] = c; sc->bb = d;
        sc->tol2 = PL::dmul(rtol2, d);
        sc->it = 0; sc->fail = 0;
        sc->done = PL::dle(a, sc->tol2) ? 1 : 0;
    }
}

// x += alpha p, r -= alpha q, z = dinv r with alpha = r.z / p.q; every block
// reduces the p.q partials itself in the same fixed order, so all blocks use the
// same alpha and no separate scalar kernel is needed.
template <class PL>
__global__ void cg_update_kernel(int64_t n, typename PL::S* __restrict__ x, typename PL::S* __restrict__ r,
                                 typename PL::S* __restrict__ z, const typename PL::S* __restrict__ p,
                                 const typename PL::S* __restrict__ q, const typename PL::S* __restrict__ dinv,
                                 const typename PL::D* __restrict__ pq_partial, int npq,
                                 typename PL::D* __restrict__ partial, CGScalars<PL>* __restrict__ sc, int parity) {
    if (sc->done) return;
    __shared__ typename PL::D sh[32];
    __shared__ typename PL::D s_alpha;
    __shared__ int s_bad;
    const typename PL::D pq = sum_partials<PL>(pq_partial, npq, sh);
    if (threadIdx.x == 0) {
        s_bad = PL::dpos(pq) ? 0 : 1;
        s_alpha = s_bad ? PL::dzero() : PL::ddiv(sc->rz[parity], pq);
    }
    __syncthreads();
    if (blockIdx.x == 0 && threadIdx.x == 0) sc->pq = pq;
    if (s_bad) {                       // breakdown: p.Ap <= 0 (same decision in every block)
        if (blockIdx.x == 0 && threadIdx.x == 0) { sc->fail = 1; sc->done = 1; }
        return;
    }
    const typename PL::A alpha = PL::from_d(s_alpha), nalpha = PL::neg_from_d(s_alpha);
    typename PL::D rr = PL::dzero(), rz = PL::dzero();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] = PL::st(PL::madd(PL::ld(x[i]), alpha, PL::ld(p[i])));
        const typename PL::A ri = PL::ld(PL::st(PL::madd(PL::ld(r[i]), nalpha, PL::ld(q[i]))));
        r[i] = PL::st(ri);
        const typename PL::A zi = PL::ld(PL::st(PL::mul(PL::ld(dinv[i]), ri)));
        z[i] = PL::st(zi);
        rr = PL::dmadd(rr, ri, ri);
        rz = PL::dmadd(rz, ri, zi);
    }
    typename PL::D a = block_sum<PL>(rr, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = a;
    a = block_sum<PL>(rz, sh);
    if (threadIdx.x == 0) partial[gridDim.x + blockIdx.x] = a;
}

// p = z + beta p with beta = r.z(new) / r.z(old); every block reduces the r.r and
// r.z partials itself. Block 0 alone owns the iteration counter: it records
// r.z(new) in the other parity slot (read by the next iteration only), the
// count and the stop flag. Convergence is decided identically by every block
// from the same sums; the maxit stop is block 0's, the other blocks may still
// update p, which is harmless since no later iteration runs.
template <class PL>
__global__ void cg_p_kernel(int64_t n, typename PL::S* __restrict__ p, const typename PL::S* __restrict__ z,
                            const typename PL::D* __restrict__ partial, int nb, int maxit,
                            CGScalars<PL>* __restrict__ sc, int parity) {
    if (sc->done) return;
    __shared__ typename PL::D sh[32];
    __shared__ typename PL::D s_beta;
    __shared__ int s_conv;
    const typename PL::D rr = sum_partials<PL>(partial, nb, sh);
    const typename PL::D rz = sum_partials<PL>(partial + nb, nb, sh);
    if (threadIdx.x == 0) {
        s_conv = PL::dle(rr, sc->tol2) ? 1 : 0;
        s_beta = PL::ddiv(rz, sc->rz[parity]);
        if (blockIdx.x == 0) {
            const int it = sc->it + 1;
            sc->rr = rr;
            sc->rz[parity ^ 1] = rz;
            sc->it = it;
            if (s_conv) {
                sc->done = 1;
            } else if (it >= maxit) {
                sc->done = 1;
                sc->fail = 2;
            }
        }
    }
    __syncthreads();
    if (s_conv) return;
    const typename PL::A beta = PL::from_d(s_beta);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = PL::st(PL::madd(PL::ld(z[i]), beta, PL::ld(p[i])));
}


static inline int vec_blocks(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, kVecBlocks)); }

// b = binary32(a * scale)
static __global__ void d2f_scaled_kernel(int64_t n, const double* __restrict__ a, float* __restrict__ b, double scale) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const df v = d2df(a[i] * scale);
        b[i] = f_add(v.hi, v.lo);
    }
}
static __global__ void axpy_f_kernel(int64_t n, double* __restrict__ x, const float* __restrict__ d, double scale) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = fma(scale, (double)d[i], x[i]);
}

// After a reliable update replaced r: z = dinv r and the partial sums of r.r, r.z
template <class PL>
__global__ void cg_refresh_kernel(int64_t n, const typename PL::S* __restrict__ r, const typename PL::S* __restrict__ dinv,
                                  typename PL::S* __restrict__ z, typename PL::D* __restrict__ partial,
                                  typename PL::S* __restrict__ p_restart) {
    __shared__ typename PL::D sh[32];
    typename PL::D rr = PL::dzero(), rz = PL::dzero();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const typename PL::A ri = PL::ld(r[i]);
        const typename PL::S zs = PL::st(PL::mul(PL::ld(dinv[i]), ri));
        z[i] = zs;
        if (p_restart) p_restart[i] = zs;
        rr = PL::dmadd(rr, ri, ri);
        rz = PL::dmadd(rz, ri, PL::ld(zs));
    }
    typename PL::D a = block_sum<PL>(rr, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = a;
    a = block_sum<PL>(rz, sh);
    if (threadIdx.x == 0) partial[gridDim.x + blockIdx.x] = a;
}

// New r.r and r.z in both parity slots; iteration count kept. The search
// direction p is kept unless the refresh restarts it (p = z, passed as
// p_restart to cg_refresh_kernel): the last iteration before a converged
// recurrence leaves p without its beta update.
template <class PL>
__global__ void cg_refresh_scalars(const typename PL::D* __restrict__ partial, int nb, CGScalars<PL>* sc) {
    __shared__ typename PL::D sh[32];
    const typename PL::D a = sum_partials<PL>(partial, nb, sh);
    const typename PL::D c = sum_partials<PL>(partial + nb, nb, sh);
    if (threadIdx.x == 0) {
        sc->rr = a;
        sc->rz[0] = c;
        sc->rz[1] = c;
        sc->done = 0;
        sc->fail = 0;
    }
}

// r = b - q
template <class PL>
__global__ void residual_from_q_kernel(int64_t n, const typename PL::S* __restrict__ b, const typename PL::S* __restrict__ q,
                                       typename PL::S* __restrict__ r) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        r[i] = PL::st(PL::sub(PL::ld(b[i]), PL::ld(q[i])));
}

// per-block partial sums of v.v (binary64)
static __global__ void norm2_partial_kernel(int64_t n, const double* __restrict__ v, double* __restrict__ partial) {
    __shared__ double sh[32];
    double s = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) s = fma(v[i], v[i], s);
    const double t = block_sum<PolF64>(s, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

// x_hi += scale * x_lo (binary64 += binary32), x_lo = 0
static __global__ void fold_kernel(int64_t n, double* __restrict__ xh, float* __restrict__ xl, double scale) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        xh[i] = fma(scale, (double)xl[i], xh[i]);
        xl[i] = 0.0f;
    }
}

}  // namespace fgpu
