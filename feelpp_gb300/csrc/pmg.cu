// p-multigrid preconditioner for matrix-free high-order operators.
//
// The reference preconditions its assembled systems with PETSc (Jacobi, GAMG;
// feelpp/feel/feelalg/backend.cpp:955); the matrix-free P2/P3 operator of this
// library has no assembled matrix for an algebraic method, so its multigrid
// takes the geometric route that high-order codes use: the order-p space on a
// mesh contains the P1 space of the same mesh (P1 functions are exactly
// interpolated), the prolongation I: P1 -> Pp is the P1 basis evaluated at the
// Pp nodes, and the coarse operator is the assembled P1 form on the same mesh
// (with exact quadrature it equals the Galerkin product I^T A_p I). One
// V-cycle per CG iteration:
//   x = S(r)                 Chebyshev smoothing in D^-1 A_p from zero (binary32 operator)
//   r_c = I^T (r - A_p x)    restriction of the residual
//   x_c = AMG V-cycle(r_c)   the P1 level (smoothed-aggregation hierarchy, amg.cu)
//   x += I x_c               prolongation
//   x += S(r - A_p x)        post-smoothing
// Dirichlet dofs: their rows of I are zero (fine corrections vanish there) and
// the columns of the coarse Dirichlet vertices are zero (the coarse level sees
// no residual there). The smoother is the Chebyshev polynomial on
// [0.05, 1.1] lmax(D^-1 A_p), lmax from a Lanczos estimate. Every kernel returns
// at once when the CG stop flag is set, so the V-cycle runs inside the CG graph.
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <string>
#include <vector>

#include "cg_driver.cuh"
#include "scan.cuh"

struct fgpu_pmg {
    fgpu_ctx* ctx = nullptr;
    fgpu_operator* op = nullptr;     // binary32 order-p operator (Dirichlet rows set)
    fgpu_amg* amg = nullptr;         // hierarchy of the assembled P1 operator
    int64_t nf = 0, nc = 0;
    int32_t* i_col = nullptr;        // I: nf x nc in ELL form, 4 slots per row (slot-major), columns sorted
    float* i_val = nullptr;          //    (padding: column 0, value 0)
    uint32_t* r_ia = nullptr;        // R = I^T: nc x nf, CSR with rows sorted by fine index
    int32_t* r_ja = nullptr;
    float* r_a = nullptr;
    int rG = 16;
    float* dinv = nullptr;           // 1 / diag(A_p)
    float *rf = nullptr, *x = nullptr, *w = nullptr, *q = nullptr, *d0 = nullptr, *d1 = nullptr, *e = nullptr, *rc = nullptr;
    int degree = 3;
    int coarse_cycles = 4;           // AMG V-cycles per coarse solve (P3 96^3, Chebyshev degree 3: 1 / 2 / 3 / 4
                                     // cycles 62 / 46 / 41 / 40 iterations, 885 / 695 / 554 / 535 ms)
    double lmax = 0;
    float inv_theta = 1.0f;
    std::vector<float> c1, c2;
    int launches_per_cycle = 0;
    double setup_ms = 0;
};

namespace fgpu {

namespace {

template <typename T>
__device__ __forceinline__ float tof(T v);
template <>
__device__ __forceinline__ float tof<double>(double v) { return (float)v; }
template <>
__device__ __forceinline__ float tof<float2>(float2 v) { return v.x + v.y; }
template <>
__device__ __forceinline__ float tof<float>(float v) { return v; }

// pre-smoothing start: rf = (float) r, d0 = D^-1 r / theta, x = d0, w = r
template <typename T>
__global__ void pmg_start_kernel(int64_t n, const T* __restrict__ r, float* __restrict__ rf, const float* __restrict__ dinv,
                                 float inv_theta, float* __restrict__ x, float* __restrict__ w, float* __restrict__ d0,
                                 const int* __restrict__ stop) {
    if (stop && *stop) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float ri = tof<T>(r[i]);
        const float d = dinv[i] * ri * inv_theta;
        rf[i] = ri;
        x[i] = d;
        w[i] = ri;
        d0[i] = d;
    }
}

// one Chebyshev step after q = A d_prev: w -= q; d_new = c1 d_prev + c2 D^-1 w; acc += d_new
// (last step with a target: target += acc + d_new)
__global__ void pmg_cheb_kernel(int64_t n, const float* __restrict__ q, float* __restrict__ w, const float* __restrict__ dprev,
                                float* __restrict__ dnew, const float* __restrict__ dinv, float c1, float c2, float* __restrict__ acc,
                                float* __restrict__ target, int last, const int* __restrict__ stop) {
    if (stop && *stop) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float wi = w[i] - q[i];
        const float dn = fmaf(c1, dprev[i], c2 * dinv[i] * wi);
        if (last && target) {
            target[i] += acc[i] + dn;
        } else {
            acc[i] += dn;
            if (!last) {
                w[i] = wi;
                dnew[i] = dn;
            }
        }
    }
}

// residual w = rf - q; with start: d0 = D^-1 w / theta, e = d0 (post-smoothing start)
__global__ void pmg_resid_kernel(int64_t n, const float* __restrict__ rf, const float* __restrict__ q, float* __restrict__ w,
                                 const float* __restrict__ dinv, float inv_theta, float* __restrict__ d0, float* __restrict__ e,
                                 int start, const int* __restrict__ stop) {
    if (stop && *stop) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float wi = rf[i] - q[i];
        w[i] = wi;
        if (start) {
            const float d = dinv[i] * wi * inv_theta;
            d0[i] = d;
            e[i] = d;
        }
    }
}

// x += I x_c with I in ELL form (thread per fine row, slots in column order)
__global__ void pmg_prolong_kernel(int64_t nf, const int32_t* __restrict__ col, const float* __restrict__ val,
                                   const float* __restrict__ xc, float* __restrict__ x, const int* __restrict__ stop) {
    if (stop && *stop) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nf; i += (int64_t)gridDim.x * blockDim.x) {
        float s = 0.0f;
#pragma unroll
        for (int k = 0; k < 4; ++k) s = fmaf(__ldg(val + k * nf + i), __ldg(xc + __ldg(col + k * nf + i)), s);
        x[i] += s;
    }
}

// ---- device construction of the transfer operators ----
// coarse Dirichlet vertices: the P1 dofs of masked fine vertex nodes (identical writes only)
__global__ void pmg_cmask_kernel(int64_t nt, int n, const int32_t* __restrict__ lf, const int32_t* __restrict__ lc,
                                 const uint8_t* __restrict__ mf, uint8_t* __restrict__ mc) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt * 4; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = t >> 2;
        const int v = (int)(t & 3);
        if (mf && mf[lf[e * n + v]]) mc[lc[e * 4 + v]] = 1;
    }
}

// ELL rows of I: each row is written by the first element of its node's incidence list (one writer,
// so the weights, which other elements would compute from other local coordinates, are fixed); the
// entries (P1 dofs of the element's vertices with a nonzero barycentric weight at the node, Dirichlet
// vertices left out) are sorted by column
__global__ void pmg_ell_kernel(int64_t nt, int n, const int32_t* __restrict__ lf, const int32_t* __restrict__ lc,
                               const int64_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                               const uint8_t* __restrict__ mf, const uint8_t* __restrict__ mc, const float* __restrict__ lam,
                               int64_t nf, int32_t* __restrict__ col, float* __restrict__ val) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt * n; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = t / n;
        const int i = (int)(t - e * n);
        const int64_t row = lf[t];
        if ((int64_t)(inc[inc_ptr[row]] >> 5) != e) continue;
        int32_t c[4] = {0, 0, 0, 0};
        float w[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        int k = 0;
        if (!(mf && mf[row])) {
            for (int v = 0; v < 4; ++v) {
                const float l = lam[i * 4 + v];
                const int32_t cv = lc[e * 4 + v];
                if (l != 0.0f && !mc[cv]) {
                    int p = k++;
                    while (p > 0 && c[p - 1] > cv) { c[p] = c[p - 1]; w[p] = w[p - 1]; --p; }
                    c[p] = cv;
                    w[p] = l;
                }
            }
        }
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            col[s * nf + row] = c[s];
            val[s * nf + row] = w[s];
        }
    }
}

__global__ void pmg_rcount_kernel(int64_t nf, const int32_t* __restrict__ col, const float* __restrict__ val, uint32_t* __restrict__ cnt) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nf; i += (int64_t)gridDim.x * blockDim.x)
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (val[k * nf + i] != 0.0f) atomicAdd(cnt + col[k * nf + i], 1u);
}

__global__ void pmg_rfill_kernel(int64_t nf, const int32_t* __restrict__ col, const float* __restrict__ val, uint32_t* __restrict__ fill,
                                 int32_t* __restrict__ rja, float* __restrict__ ra) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nf; i += (int64_t)gridDim.x * blockDim.x)
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float v = val[k * nf + i];
            if (v == 0.0f) continue;
            const uint32_t p = atomicAdd(fill + col[k * nf + i], 1u);
            rja[p] = (int32_t)i;
            ra[p] = v;
        }
}

// sort every restriction row by fine index (one warp per row, bitonic sort of up to 256 entries in
// shared memory); longer rows set *status
__global__ void __launch_bounds__(256) pmg_rsort_kernel(int64_t nc, const uint32_t* __restrict__ ia, int32_t* __restrict__ ja,
                                                        float* __restrict__ a, int* __restrict__ status) {
    __shared__ int32_t sk[8][256];
    __shared__ float sv[8][256];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int64_t r = (int64_t)blockIdx.x * 8 + w; r < nc; r += (int64_t)gridDim.x * 8) {
        const uint32_t p0 = ia[r], len = ia[r + 1] - p0;
        if (len > 256) {
            if (lane == 0) atomicOr(status, 1);
            continue;
        }
        int m = 1;
        while (m < (int)len) m <<= 1;
        for (int k = lane; k < m; k += 32) {
            sk[w][k] = k < (int)len ? ja[p0 + k] : INT32_MAX;
            sv[w][k] = k < (int)len ? a[p0 + k] : 0.0f;
        }
        __syncwarp();
        for (int size = 2; size <= m; size <<= 1)
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                for (int k = lane; k < m; k += 32) {
                    const int partner = k ^ stride;
                    if (partner > k) {
                        const bool up = (k & size) == 0;
                        const int32_t x = sk[w][k], y = sk[w][partner];
                        if ((x > y) == up) {
                            sk[w][k] = y; sk[w][partner] = x;
                            const float t = sv[w][k]; sv[w][k] = sv[w][partner]; sv[w][partner] = t;
                        }
                    }
                }
                __syncwarp();
            }
        for (int k = lane; k < (int)len; k += 32) {
            ja[p0 + k] = sk[w][k];
            a[p0 + k] = sv[w][k];
        }
        __syncwarp();
    }
}

// y = M x (add = 0) or y += M x (add = 1), G lanes per row; the warp-uniform loop keeps every lane
// at the shuffles
template <int G>
__global__ void __launch_bounds__(256) pmg_csr_kernel(int64_t n, const uint32_t* __restrict__ ia, const int32_t* __restrict__ ja,
                                                      const float* __restrict__ a, const float* __restrict__ x, float* __restrict__ y,
                                                      int add, const int* __restrict__ stop) {
    if (stop && *stop) return;
    const int lane = threadIdx.x & (G - 1);
    const int gw = (threadIdx.x & 31) / G;
    const int64_t groups = (int64_t)gridDim.x * (blockDim.x / G);
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G; i - gw < n; i += groups) {
        const bool valid = i < n;
        const int64_t p0 = valid ? ia[i] : 0, p1 = valid ? ia[i + 1] : 0;
        float s = 0.0f;
        for (int64_t p = p0 + lane; p < p1; p += G) s = fmaf(__ldg(a + p), __ldg(x + __ldg(ja + p)), s);
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, G);
        if (lane == 0 && valid) y[i] = add ? y[i] + s : s;
    }
}

template <class PL>
__global__ void pmg_finish_kernel(int64_t n, const float* __restrict__ x, const typename PL::S* __restrict__ r,
                                  typename PL::S* __restrict__ z, typename PL::D* __restrict__ partial_rz,
                                  typename PL::S* __restrict__ p_out, const CGScalars<PL>* __restrict__ sc) {
    if (sc && sc->done) return;
    __shared__ typename PL::D sh[32];
    typename PL::D rz = PL::dzero();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        typename PL::A zi;
        if constexpr (PL::id == 1) zi = df{x[i], 0.0f};
        else zi = (typename PL::A)x[i];
        const typename PL::S zs = PL::st(zi);
        z[i] = zs;
        if (p_out) p_out[i] = zs;
        rz = PL::dmadd(rz, PL::ld(r[i]), PL::ld(zs));
    }
    const typename PL::D t = block_sum<PL>(rz, sh);
    if (threadIdx.x == 0) partial_rz[blockIdx.x] = t;
}

int vb_of(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 8)); }

int lanes(int64_t n, int64_t nnz) {
    const double m = n > 0 ? (double)nnz / (double)n : 1.0;
    return m <= 4 ? 1 : m <= 12 ? 8 : m <= 24 ? 16 : 32;     // the prolongation's rows have 1 to 4 entries
}

void csr(cudaStream_t st, int G, int64_t n, const uint32_t* ia, const int32_t* ja, const float* a, const float* x, float* y, int add,
         const int* stop) {
    const int per = 256 / G;
    const int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + per - 1) / per, 152 * 16));
    switch (G) {
        case 1: pmg_csr_kernel<1><<<g, 256, 0, st>>>(n, ia, ja, a, x, y, add, stop); break;
        case 4: pmg_csr_kernel<4><<<g, 256, 0, st>>>(n, ia, ja, a, x, y, add, stop); break;
        case 8: pmg_csr_kernel<8><<<g, 256, 0, st>>>(n, ia, ja, a, x, y, add, stop); break;
        case 16: pmg_csr_kernel<16><<<g, 256, 0, st>>>(n, ia, ja, a, x, y, add, stop); break;
        default: pmg_csr_kernel<32><<<g, 256, 0, st>>>(n, ia, ja, a, x, y, add, stop); break;
    }
}

// K - 1 Chebyshev steps accumulating into acc; the last adds acc + d into target when set
int cheb(fgpu_pmg* P, float* acc, float* target, const int* stop) {
    cudaStream_t st = P->ctx->stream;
    int nl = 0;
    for (int k = 1; k < P->degree; ++k) {
        float* dprev = (k & 1) ? P->d0 : P->d1;
        float* dnew = (k & 1) ? P->d1 : P->d0;
        nl += mf_apply_f32_gated(P->ctx, P->op, dprev, P->q, stop);
        const bool last = k == P->degree - 1;
        pmg_cheb_kernel<<<vb_of(P->nf), 256, 0, st>>>(P->nf, P->q, P->w, dprev, dnew, P->dinv, P->c1[k - 1], P->c2[k - 1], acc,
                                                      last ? target : nullptr, last ? 1 : 0, stop);
        ++nl;
    }
    return nl;
}

}  // namespace

template <typename T>
int pmg_vcycle(fgpu_pmg* P, const T* r, const int* stop) {
    cudaStream_t st = P->ctx->stream;
    int nl = 0;
    pmg_start_kernel<T><<<vb_of(P->nf), 256, 0, st>>>(P->nf, r, P->rf, P->dinv, P->inv_theta, P->x, P->w, P->d0, stop);
    ++nl;
    nl += cheb(P, P->x, nullptr, stop);
    nl += mf_apply_f32_gated(P->ctx, P->op, P->x, P->q, stop);
    pmg_resid_kernel<<<vb_of(P->nf), 256, 0, st>>>(P->nf, P->rf, P->q, P->w, P->dinv, P->inv_theta, nullptr, nullptr, 0, stop);
    csr(st, P->rG, P->nc, P->r_ia, P->r_ja, P->r_a, P->w, P->rc, 0, stop);
    nl += 2;
    const float* xc = nullptr;
    nl += amg_vcycle_f32(P->amg, P->rc, stop, &xc, P->coarse_cycles);
    pmg_prolong_kernel<<<vb_of(P->nf), 256, 0, st>>>(P->nf, P->i_col, P->i_val, xc, P->x, stop);
    ++nl;
    nl += mf_apply_f32_gated(P->ctx, P->op, P->x, P->q, stop);
    pmg_resid_kernel<<<vb_of(P->nf), 256, 0, st>>>(P->nf, P->rf, P->q, P->w, P->dinv, P->inv_theta, P->d0, P->e, 1, stop);
    ++nl;
    nl += cheb(P, P->e, P->x, stop);
    return nl;
}

template <class PL>
PcHook<PL> pmg_pc_hook(fgpu_pmg* P) {
    PcHook<PL> h;
    h.apply = [P](const typename PL::S* r, typename PL::S* z, typename PL::D* partial_rz, typename PL::S* p_out,
                  const CGScalars<PL>* gate) {
        const int* stop = gate ? &gate->done : nullptr;
        const int nl = pmg_vcycle<typename PL::S>(P, r, stop);
        pmg_finish_kernel<PL><<<vec_blocks(P->nf), kVecThreads, 0, P->ctx->stream>>>(P->nf, P->x, r, z, partial_rz, p_out, gate);
        P->ctx->launches += nl + 1;
    };
    h.launches = P->launches_per_cycle + 1;
    return h;
}

template PcHook<PolF64> pmg_pc_hook<PolF64>(fgpu_pmg*);
template PcHook<PolDF64> pmg_pc_hook<PolDF64>(fgpu_pmg*);
template PcHook<PolF32> pmg_pc_hook<PolF32>(fgpu_pmg*);

namespace {

__global__ void scale_mul_kernel(int64_t n, const float* __restrict__ a, const float* __restrict__ b, float* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) out[i] = a[i] * b[i];
}

__global__ void dot_partials_kernel(int64_t n, const float* __restrict__ a, const float* __restrict__ b, double* __restrict__ partial) {
    __shared__ double sh[256];
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) s += (double)a[i] * b[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

// w = (w - a v - b vold) / beta-style Lanczos updates on the host-driven loop: out = x - a y - b z
__global__ void axpbypcz_kernel(int64_t n, const float* __restrict__ x, float a, const float* __restrict__ y, float b,
                                const float* __restrict__ z, float* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = x[i] - a * y[i] - b * z[i];
}

__global__ void scale_kernel(int64_t n, const float* __restrict__ x, float s, float* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) out[i] = s * x[i];
}

__global__ void lanczos_init_kernel(int64_t n, const float* __restrict__ dinv, float* __restrict__ s, float* __restrict__ v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        s[i] = sqrtf(fmaxf(dinv[i], 0.0f));
        uint64_t h = (uint64_t)i * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
        h ^= h >> 33; h *= 0xff51afd7ed558ccdull; h ^= h >> 33; h *= 0xc4ceb9fe1a85ec53ull; h ^= h >> 33;
        v[i] = (float)(h >> 40) * (1.0f / 16777216.0f) - 0.5f;
    }
}

__global__ void recip_kernel(int64_t n, const float* __restrict__ d, float* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = d[i] != 0.0f ? 1.0f / d[i] : 0.0f;
}

double dot(fgpu_ctx* ctx, int64_t n, const float* a, const float* b, double* d_part, std::vector<double>& h) {
    const int nb = vb_of(n);
    dot_partials_kernel<<<nb, 256, 0, ctx->stream>>>(n, a, b, d_part);
    cudaMemcpyAsync(h.data(), d_part, nb * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    double s = 0;
    for (int k = 0; k < nb; ++k) s += h[k];
    return s;
}

// lmax of D^-1 A (symmetric form D^-1/2 A D^-1/2) by m Lanczos steps with the binary32 operator
int lanczos_lmax(fgpu_pmg* P, int m, double* out) {
    fgpu_ctx* ctx = P->ctx;
    const int64_t n = P->nf;
    float *s = nullptr, *v = nullptr, *vold = nullptr, *t = nullptr, *u = nullptr;
    double* part = nullptr;
    std::vector<double> h(152 * 8);
    cudaError_t e = cudaMalloc(&s, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&v, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&vold, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&t, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&u, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&part, h.size() * sizeof(double));
    if (e != cudaSuccess) { cudaGetLastError(); ctx->err = "pmg: allocation failed"; cudaFree(s); cudaFree(v); cudaFree(vold); cudaFree(t); cudaFree(u); cudaFree(part); return FGPU_ERR_ALLOC; }
    // s = D^-1/2 (from dinv), v0 pseudo-random (hash of the index), normalised
    lanczos_init_kernel<<<vb_of(n), 256, 0, ctx->stream>>>(n, P->dinv, s, t);
    const double nv = std::sqrt(dot(ctx, n, t, t, part, h));
    scale_kernel<<<vb_of(n), 256, 0, ctx->stream>>>(n, t, (float)(1.0 / nv), v);
    cudaMemsetAsync(vold, 0, n * 4, ctx->stream);
    std::vector<double> al, be;
    double bprev = 0;
    for (int k = 0; k < m; ++k) {
        scale_mul_kernel<<<vb_of(n), 256, 0, ctx->stream>>>(n, s, v, t);          // t = D^-1/2 v
        mf_apply_f32_gated(ctx, P->op, t, u, nullptr);                              // u = A t
        scale_mul_kernel<<<vb_of(n), 256, 0, ctx->stream>>>(n, s, u, t);          // t = D^-1/2 A D^-1/2 v
        const double a = dot(ctx, n, t, v, part, h);
        axpbypcz_kernel<<<vb_of(n), 256, 0, ctx->stream>>>(n, t, (float)a, v, (float)bprev, vold, u);
        const double b = std::sqrt(std::max(dot(ctx, n, u, u, part, h), 0.0));
        al.push_back(a);
        if (b < 1e-10 * std::fabs(a) || k + 1 == m) break;
        be.push_back(b);
        std::swap(v, vold);                                                          // vold = v
        scale_kernel<<<vb_of(n), 256, 0, ctx->stream>>>(n, u, (float)(1.0 / b), v); // v = u / b
        bprev = b;
    }
    cudaError_t e2 = cudaStreamSynchronize(ctx->stream);
    cudaFree(s); cudaFree(v); cudaFree(vold); cudaFree(t); cudaFree(u); cudaFree(part);
    if (e2 != cudaSuccess) { ctx->err = cudaGetErrorString(e2); return FGPU_ERR_CUDA; }
    std::vector<double> off(be.begin(), be.end());
    *out = tridiag_max_eig(al, off);
    return FGPU_OK;
}

template <typename T>
cudaError_t upv(T** dst, const std::vector<T>& v) {
    cudaError_t e = cudaMalloc(dst, std::max<size_t>(v.size(), 1) * sizeof(T));
    if (e == cudaSuccess && !v.empty()) e = cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    return e;
}

void pmg_free(fgpu_pmg* P) {
    cudaFree(P->i_col); cudaFree(P->i_val); cudaFree(P->r_ia); cudaFree(P->r_ja); cudaFree(P->r_a);
    cudaFree(P->dinv); cudaFree(P->rf); cudaFree(P->x); cudaFree(P->w); cudaFree(P->q); cudaFree(P->d0); cudaFree(P->d1);
    cudaFree(P->e); cudaFree(P->rc);
}

}  // namespace

}  // namespace fgpu

using namespace fgpu;

extern "C" int fgpu_pmg_create(fgpu_ctx* ctx, fgpu_operator* op32, const fgpu_matrix* A1, fgpu_amg* amg, const fgpu_pmg_cfg* cfg,
                               fgpu_pmg** out) {
    if (!ctx || !op32 || !A1 || !amg || !out) return FGPU_ERR_INVALID;
    if (ctx->capturing) { ctx->err = "pmg: set-up is not capturable"; return FGPU_ERR_INVALID; }
    *out = nullptr;
    const fgpu_space* Vf = operator_space(op32);
    const fgpu_space* Vc = A1->space;
    if (operator_precision(op32) != FGPU_F32) { ctx->err = "pmg: the smoothing operator must be binary32"; return FGPU_ERR_INVALID; }
    if (Vc->mesh != Vf->mesh || Vc->order != 1 || Vc->ncomp != 1 || Vf->ncomp != 1) {
        ctx->err = "pmg: the coarse matrix must be the P1 form on the operator's mesh";
        return FGPU_ERR_INVALID;
    }
    if (amg_rows(amg) != Vc->ndof) { ctx->err = "pmg: the AMG hierarchy is not the coarse matrix's"; return FGPU_ERR_INVALID; }
    const auto t0 = std::chrono::steady_clock::now();
    fgpu_pmg* P = new fgpu_pmg();
    P->ctx = ctx;
    P->op = op32;
    P->amg = amg;
    P->nf = Vf->ndof;
    P->nc = Vc->ndof;
    if (cfg && cfg->smoother_degree >= 2) P->degree = cfg->smoother_degree;
    if (cfg && cfg->coarse_cycles >= 1) P->coarse_cycles = std::min(cfg->coarse_cycles, 4);
    const int64_t nt = Vf->mesh->nt;
    const int n = Vf->n;
    // barycentric weights of the P1 vertices at the order-p reference nodes ([-1,1]^3 element)
    std::vector<double> nodes;
    lagrange_nodes(Vf->order, nodes);
    std::vector<float> lam((size_t)n * 4);
    for (int i = 0; i < n; ++i) {
        const double x = nodes[3 * i], y = nodes[3 * i + 1], z = nodes[3 * i + 2];
        const double l[4] = {-0.5 * (1 + x + y + z), 0.5 * (1 + x), 0.5 * (1 + y), 0.5 * (1 + z)};
        for (int v = 0; v < 4; ++v) lam[(size_t)i * 4 + v] = std::fabs(l[v]) > 1e-12 ? (float)l[v] : 0.0f;
    }
    float* d_lam = nullptr;
    uint8_t* d_mc = nullptr;
    uint32_t* cnt = nullptr;
    cudaError_t e = upv(&d_lam, lam);
    if (e == cudaSuccess) e = cudaMalloc(&d_mc, std::max<int64_t>(P->nc, 1));
    if (e == cudaSuccess) e = cudaMemsetAsync(d_mc, 0, std::max<int64_t>(P->nc, 1), ctx->stream);
    if (e == cudaSuccess) e = cudaMalloc(&P->i_col, std::max<int64_t>(P->nf, 1) * 4 * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&P->i_val, std::max<int64_t>(P->nf, 1) * 4 * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&cnt, (P->nc + 1) * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&P->r_ia, (P->nc + 1) * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemsetAsync(cnt, 0, (P->nc + 1) * sizeof(uint32_t), ctx->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        cudaFree(d_lam); cudaFree(d_mc); cudaFree(cnt);
        ctx->err = "pmg: allocation failed";
        pmg_free(P); delete P;
        return FGPU_ERR_ALLOC;
    }
    const uint8_t* mf = operator_mask(op32);
    const int g4 = (int)std::max<int64_t>(1, std::min<int64_t>((nt * 4 + 255) / 256, 152 * 32));
    const int gn = (int)std::max<int64_t>(1, std::min<int64_t>((nt * n + 255) / 256, 152 * 32));
    const int gf = (int)std::max<int64_t>(1, std::min<int64_t>((P->nf + 255) / 256, 152 * 32));
    pmg_cmask_kernel<<<g4, 256, 0, ctx->stream>>>(nt, n, Vf->d_l2n, Vc->d_l2n, mf, d_mc);
    pmg_ell_kernel<<<gn, 256, 0, ctx->stream>>>(nt, n, Vf->d_l2n, Vc->d_l2n, Vf->d_inc_ptr, Vf->d_inc, mf, d_mc, d_lam, P->nf,
                                                 P->i_col, P->i_val);
    pmg_rcount_kernel<<<gf, 256, 0, ctx->stream>>>(P->nf, P->i_col, P->i_val, cnt);
    ctx->launches += 3;
    uint64_t nnzr = 0;
    int rc = scan_u32(ctx, cnt, P->r_ia, P->nc, &nnzr);
    if (rc == FGPU_OK) {
        e = cudaMalloc(&P->r_ja, std::max<uint64_t>(nnzr, 1) * sizeof(int32_t));
        if (e == cudaSuccess) e = cudaMalloc(&P->r_a, std::max<uint64_t>(nnzr, 1) * sizeof(float));
        if (e == cudaSuccess) e = cudaMemcpyAsync(cnt, P->r_ia, P->nc * sizeof(uint32_t), cudaMemcpyDeviceToDevice, ctx->stream);
        if (e == cudaSuccess) {
            pmg_rfill_kernel<<<gf, 256, 0, ctx->stream>>>(P->nf, P->i_col, P->i_val, cnt, P->r_ja, P->r_a);
            const int gr = (int)std::max<int64_t>(1, std::min<int64_t>((P->nc + 7) / 8, 152 * 32));
            cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream);
            pmg_rsort_kernel<<<gr, 256, 0, ctx->stream>>>(P->nc, P->r_ia, P->r_ja, P->r_a, ctx->d_status);
            ctx->launches += 2;
            int st = 0;
            e = cudaMemcpyAsync(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
            if (e == cudaSuccess && st) { ctx->err = "pmg: a coarse vertex restricts more than 256 fine dofs"; rc = FGPU_ERR_INVALID; }
        }
        if (e != cudaSuccess) { cudaGetLastError(); ctx->err = std::string("pmg: ") + cudaGetErrorString(e); rc = FGPU_ERR_CUDA; }
    }
    cudaFree(d_lam); cudaFree(d_mc); cudaFree(cnt);
    if (rc) { pmg_free(P); delete P; return rc; }
    P->rG = lanes(P->nc, (int64_t)nnzr);
    float** vecs[8] = {&P->rf, &P->x, &P->w, &P->q, &P->d0, &P->d1, &P->e, &P->dinv};
    for (float** p : vecs)
        if (e == cudaSuccess) e = cudaMalloc(p, std::max<int64_t>(P->nf, 1) * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&P->rc, std::max<int64_t>(P->nc, 1) * sizeof(float));
    if (e != cudaSuccess) { cudaGetLastError(); ctx->err = "pmg: allocation failed"; pmg_free(P); delete P; return FGPU_ERR_ALLOC; }
    // D^-1 of the binary32 operator (Dirichlet rows: 1)
    const float* diag = operator_diag_f32(ctx, op32);
    if (!diag) { pmg_free(P); delete P; return FGPU_ERR_CUDA; }
    recip_kernel<<<vb_of(P->nf), 256, 0, ctx->stream>>>(P->nf, diag, P->dinv);
    ctx->launches++;
    rc = lanczos_lmax(P, 12, &P->lmax);
    if (rc) { pmg_free(P); delete P; return rc; }
    // interval [0.05, 1.1] lmax: at P3 96^3 (degree 3, 4 coarse cycles) the lower end 0.01 / 0.02 / 0.03 /
    // 0.05 / 0.1 / 0.2 / 0.3 lmax gave 62 / 45 / 40 / 37 / 40 / 50 / 55 iterations
    const double emax = 1.1 * P->lmax, emin = 0.05 * P->lmax;
    const double theta = 0.5 * (emax + emin), delta = 0.5 * (emax - emin), sigma = theta / delta;
    double rho = 1.0 / sigma;
    P->inv_theta = (float)(1.0 / theta);
    for (int k = 1; k < P->degree; ++k) {
        const double rn = 1.0 / (2.0 * sigma - rho);
        P->c1.push_back((float)(rn * rho));
        P->c2.push_back((float)(2.0 * rn / delta));
        rho = rn;
    }
    // one V-cycle on a zero residual: checks that the cycle runs and counts its kernels
    cudaMemsetAsync(P->q, 0, P->nf * sizeof(float), ctx->stream);
    cudaMemcpyAsync(P->e, P->q, P->nf * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream);
    const int64_t l0 = ctx->launches;
    P->launches_per_cycle = pmg_vcycle<float>(P, P->e, nullptr);
    ctx->launches = l0 + P->launches_per_cycle;
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { ctx->err = cudaGetErrorString(e); pmg_free(P); delete P; return FGPU_ERR_CUDA; }
    P->setup_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    *out = P;
    return FGPU_OK;
}

extern "C" int fgpu_pmg_info(const fgpu_pmg* P, double* lmax, int64_t* coarse_rows, double* setup_ms) {
    if (!P) return FGPU_ERR_INVALID;
    if (lmax) *lmax = P->lmax;
    if (coarse_rows) *coarse_rows = P->nc;
    if (setup_ms) *setup_ms = P->setup_ms;
    return FGPU_OK;
}

extern "C" int fgpu_pmg_destroy(fgpu_pmg* P) {
    if (!P) return FGPU_OK;
    pmg_free(P);
    delete P;
    return FGPU_OK;
}
