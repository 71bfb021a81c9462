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
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

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
        typename PL::A s = PL::zero();
        if (r < nrows) {
            const int64_t pe = ia[r + 1];
            for (int64_t p = ia[r] + lane; p < pe; p += G) s = PL::madd(s, PL::ldv(val[p]), PL::ld(x[ja[p]]));
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) s = PL::add(s, PL::shfl_xor(s, o));
        if (r < nrows && lane == 0) {
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
// b = binary32(a * scale)
__global__ void d2f_scaled_kernel(int64_t n, const double* __restrict__ a, float* __restrict__ b, double scale) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const df v = d2df(a[i] * scale);
        b[i] = f_add(v.hi, v.lo);
    }
}
__global__ void axpy_f_kernel(int64_t n, double* __restrict__ x, const float* __restrict__ d, double scale) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = fma(scale, (double)d[i], x[i]);
}
__global__ void norm2_partial_kernel(int64_t n, const double* __restrict__ v, double* __restrict__ partial) {
    __shared__ double sh[32];
    double s = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) s = fma(v[i], v[i], s);
    const double t = block_sum<PolF64>(s, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

// ---------------------------------------------------------------------------
template <class PL>
static void launch_spmv_t(cudaStream_t s, const fgpu_matrix* A, const typename PL::V* val, int G, const typename PL::S* x,
                          typename PL::S* y, int mode, const typename PL::S* b, const typename PL::S* wdot,
                          typename PL::D* partial, const CGScalars<PL>* sc, int blocks) {
    switch (G) {
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

static int vec_blocks(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, kVecBlocks)); }

int launch_spmv(fgpu_ctx* ctx, const fgpu_matrix* A, const double* x, double* y, double alpha_b, const double* b) {
    (void)alpha_b;
    if (A->precision != FGPU_F64) {
        ctx->err = "y = A x with binary64 vectors needs an FP64 matrix";
        return FGPU_ERR_INVALID;
    }
    const int G = spmv_group(A);
    PendingEvent ev;
    prof_begin(ctx, "spmv", ev);
    launch_spmv_t<PolF64>(ctx->stream, A, (const double*)A->d_val, G, x, y, b ? 1 : 0, b, nullptr, nullptr, nullptr,
                          spmv_blocks(A, G));
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
        typename PL::A acc = PL::zero();
        for (int k = 0; k < L; ++k) {
            const int64_t j = base + (int64_t)k * kSellC;
            acc = PL::madd(acc, PL::ldv(val[j]), PL::ld(x[col[j]]));
        }
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
static std::map<std::tuple<int, int, int64_t, int64_t>, int> g_spmv_tune;

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
    const auto key = std::make_tuple(ctx->device, PL::id, A->nrows, A->nnz);
    int choice = -1;
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        auto it = g_spmv_tune.find(key);
        if (it != g_spmv_tune.end()) choice = it->second;
    }
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
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
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
            cudaEventRecord(e0, ctx->stream);
            for (int rep = 0; rep < 3; ++rep) trial.launch(ctx->stream, A, val, x, y, 0, nullptr, nullptr, nullptr, nullptr);
            cudaEventRecord(e1, ctx->stream);
            cudaEventSynchronize(e1);
            trial.sval = nullptr;  // not owned by the trial
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            ctx->launches += 4;
            if (ms < best_ms) { best_ms = ms; best = c; }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        choice = best;
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
template <class PL>
static int pcg_core(fgpu_ctx* ctx, const fgpu_matrix* A, const typename PL::V* val, const typename PL::S* b,
                    typename PL::S* x, double rtol, int maxit, int pc, int check_every, int* iters, int* fail,
                    double* rr_out, double* bb_out) {
    typedef typename PL::S S;
    typedef typename PL::D D;
    const int64_t n = A->nrows;
    cudaStream_t s = ctx->stream;
    S *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *dinv = nullptr;
    D* partial = nullptr;
    D* pq_partial = nullptr;
    CGScalars<PL>* sc = nullptr;
    CGScalars<PL>* hsc = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    SpmvPlan<PL> plan;
    // partial-sum buffers sized for the largest grid any candidate launches
    // (the number of CSR blocks grows with the lanes per row)
    int sblocks = spmv_blocks(A, 32);
    const int vb = vec_blocks(n);
    const int nbp = std::max(sblocks, vb);
    auto cleanup = [&]() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        cudaFree(r); cudaFree(z); cudaFree(p); cudaFree(q); cudaFree(dinv); cudaFree(partial); cudaFree(pq_partial);
        cudaFree(sc);
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
    if (check_every & 1) ++check_every;   // parity of the scalar double buffer repeats per replay
    CK(cudaMalloc(&pq_partial, nbp * sizeof(D)));
    CK(cudaMalloc(&r, n * sizeof(S)));
    CK(cudaMalloc(&z, n * sizeof(S)));
    CK(cudaMalloc(&p, n * sizeof(S)));
    CK(cudaMalloc(&q, n * sizeof(S)));
    CK(cudaMalloc(&dinv, n * sizeof(S)));
    CK(cudaMalloc(&partial, 3 * nbp * sizeof(D)));
    CK(cudaMalloc(&sc, sizeof(CGScalars<PL>)));
    CK(cudaMallocHost(&hsc, sizeof(CGScalars<PL>)));
    diag_inv_kernel<PL><<<vb, 256, 0, s>>>(n, A->d_ia, A->d_ja, val, dinv, pc == FGPU_PC_JACOBI);
    plan_spmv<PL>(ctx, A, val, dinv, q, plan);
    sblocks = plan.blocks(A);
    if (sblocks > nbp) { ctx->err = "internal: partial buffer too small"; cleanup(); return FGPU_ERR_INVALID; }
    plan.launch(s, A, val, x, r, 1, b, nullptr, nullptr, nullptr);
    cg_init_kernel<PL><<<vb, kVecThreads, 0, s>>>(n, b, r, dinv, z, p, partial);
    cg_init_scalars<PL><<<1, 256, 0, s>>>(partial, vb, PL::host_from_double(rtol * rtol), sc);
    ctx->launches += 4;
    CK(cudaGetLastError());
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < check_every; ++k) {
        const int parity = k & 1;
        plan.launch(s, A, val, p, q, 0, nullptr, p, pq_partial, sc);
        cg_update_kernel<PL><<<vb, kVecThreads, 0, s>>>(n, x, r, z, p, q, dinv, pq_partial, sblocks, partial, sc, parity);
        cg_p_kernel<PL><<<vb, kVecThreads, 0, s>>>(n, p, z, partial, vb, maxit, sc, parity);
    }
    {
        cudaError_t e = cudaStreamEndCapture(s, &graph);
        if (e != cudaSuccess) { ctx->err = std::string("graph capture: ") + cudaGetErrorString(e); cleanup(); return FGPU_ERR_CUDA; }
    }
    CK(cudaGraphInstantiate(&exec, graph, 0));
    CK(cudaMemcpyAsync(hsc, sc, sizeof(CGScalars<PL>), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    int guard = 0;
    while (!hsc->done) {
        CK(cudaGraphLaunch(exec, s));
        ctx->launches += 3 * check_every;
        CK(cudaMemcpyAsync(hsc, sc, sizeof(CGScalars<PL>), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if (++guard > maxit / std::max(check_every, 1) + 2) break;
    }
    *iters = hsc->it;
    *fail = hsc->fail;
    *rr_out = PL::host_to_double(hsc->rr);
    *bb_out = PL::host_to_double(hsc->bb);
    cleanup();
#undef CK
    return FGPU_OK;
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
              fgpu_solve_stats* st) {
    if (A->precision != FGPU_F64) { ctx->err = "solve needs an FP64 matrix"; return FGPU_ERR_INVALID; }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, ctx->stream);
    const int ce = cfg->check_every > 0 ? cfg->check_every : 16;
    const int64_t n = A->nrows;
    int iters = 0, fail = 0;
    double rr = 0, bb = 0, rn = 0;
    int rc = FGPU_OK;
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
            rc = pcg_core<PolDF64>(ctx, A, val, b, x, cfg->rtol, cfg->maxit, cfg->pc, ce, &iters, &fail, &rr, &bb);
            if (rc == FGPU_OK) {
                df2d_kernel<<<vec_blocks(n), 256, 0, ctx->stream>>>(n, x, d_x);
                ctx->launches++;
            }
        }
        cudaFree(val); cudaFree(b); cudaFree(x);
    } else {
        rc = pcg_core<PolF64>(ctx, A, (const double*)A->d_val, d_b, d_x, cfg->rtol, cfg->maxit, cfg->pc, ce, &iters, &fail,
                              &rr, &bb);
    }
    if (rc == FGPU_OK) {  // final residual recomputed in binary64 from the matrix
        Scratch64 S;
        if (!S.alloc(n)) { ctx->err = "residual: allocation failed"; rc = FGPU_ERR_ALLOC; }
        else rc = f64_residual(ctx, A, d_b, d_x, S.r, S.partial, S.hpart, &rn);
    }
    cudaEventRecord(e1, ctx->stream);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != FGPU_OK) return rc;
    const double bn = std::sqrt(bb);
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
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, ctx->stream);
    int rc = FGPU_OK;
    int total = 0, outer = 0, fail = 0;
    double rn = 0, bn = 0;
    {
        Scratch64 S;
        float *r32 = nullptr, *d32 = nullptr;
        if (!S.alloc(n) || cudaMalloc(&r32, n * sizeof(float)) != cudaSuccess || cudaMalloc(&d32, n * sizeof(float)) != cudaSuccess) {
            ctx->err = "mixed solve: allocation failed";
            rc = FGPU_ERR_ALLOC;
        }
        if (rc == FGPU_OK) {
            const int vb = vec_blocks(n);
            norm2_partial_kernel<<<vb, 256, 0, ctx->stream>>>(n, d_b, S.partial);
            cudaMemcpyAsync(S.hpart, S.partial, vb * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
            cudaStreamSynchronize(ctx->stream);
            double s = 0;
            for (int k = 0; k < vb; ++k) s += S.hpart[k];
            bn = std::sqrt(s);
            const double inner = cfg->inner_rtol > 0 ? cfg->inner_rtol : 1e-4;
            const int ce = cfg->check_every > 0 ? cfg->check_every : 16;
            while (true) {
                rc = f64_residual(ctx, A64, d_b, d_x, S.r, S.partial, S.hpart, &rn);
                if (rc) break;
                if (bn == 0.0 || rn <= cfg->rtol * bn) break;
                if (outer >= 50 || total >= cfg->maxit) { fail = 2; break; }
                // inner: A32 d = r / ||r|| in binary32
                d2f_scaled_kernel<<<vb, 256, 0, ctx->stream>>>(n, S.r, r32, 1.0 / rn);
                cudaMemsetAsync(d32, 0, n * sizeof(float), ctx->stream);
                ctx->launches++;
                int it = 0, f = 0;
                double rr = 0, bb = 0;
                rc = pcg_core<PolF32>(ctx, A32, (const float*)A32->d_val, r32, d32, inner, cfg->maxit - total, cfg->pc, ce,
                                      &it, &f, &rr, &bb);
                if (rc) break;
                total += it;
                ++outer;
                axpy_f_kernel<<<vb, 256, 0, ctx->stream>>>(n, d_x, d32, rn);
                ctx->launches++;
                if (f == 1) { fail = 1; break; }
            }
            cudaStreamSynchronize(ctx->stream);
        }
        cudaFree(r32);
        cudaFree(d32);
    }
    cudaEventRecord(e1, ctx->stream);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != FGPU_OK) return rc;
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

SellLayout::~SellLayout() {
    cudaFree(d_perm);
    cudaFree(d_slice_ptr);
    cudaFree(d_slice_len);
    cudaFree(d_col);
    cudaFree(d_src);
}
