// Matrix-free operator y = A x for the affine Laplace/mass form, and the CG
// that uses it.
//
// Feel++ has no element-level matrix-free kernel: its "matrix-free" notion
// applies form-level operators (MatrixShell::multVector, feelpp/feel/feelalg/
// matrixshell.hpp:49,120; OperatorLinearFree::apply, feelpp/feel/feeldiscr/
// operatorlinearfree.hpp:116-170). This operator is validated against the
// assembled CSR product of the same form (after on() with symmetric
// elimination, which is what its Dirichlet handling reproduces).
//
// Two phases per apply, deterministic and without float atomics:
//  1. element phase: y_e = K_e x_e with K_e = sum_k c_k T_k (the 7 reference
//     tensors of the assembly kernels), x_e gathered through the dof table with
//     Dirichlet dofs masked to zero, written to an element buffer (T x n);
//  2. node phase: y[m] = sum of the element buffer over the elements containing
//     dof m, in increasing element order (the node -> element incidence); a
//     Dirichlet row returns y[m] = x[m].
// Number formats: binary32 (tables and coefficients in binary32, fused
// multiply-adds on the FP32 pipes), df64 (double-float, ~48 bits) and native
// binary64 (FP64 pipe; the reference arithmetic).
#include <cmath>
#include <functional>
#include <cstring>
#include <utility>
#include <vector>

#include "df64.h"
#include "fgpu_core.h"

namespace fgpu {

// ---------------------------------------------------------------------------
// element phase
// ---------------------------------------------------------------------------
// binary32: one thread per element; T (7 n n floats) in shared memory.
// binary32 element phase, EPT elements per thread (each reference-tensor value
// read from shared memory serves EPT FMAs). The warp's 32 EPT elements' l2n
// rows are staged in shared memory with coalesced loads (row stride N + 1: no
// bank conflicts); element values are written local-index-major (coalesced).
template <int N>
struct MfF32Shape {                     // elements per thread, warps per block (measured at P3 96³: four
    static constexpr int EPT = 2;       // elements per thread in 2-warp blocks, 153 registers and 32.7 KB
    static constexpr int WPB = 4;       // of shared memory per block, took 0.95 ms against 0.81 ms)
};

template <int N>
__device__ __forceinline__ void mf_element_f32_body(int64_t nt, const int32_t* __restrict__ l2n, const float4* __restrict__ rec,
                                                    const float* __restrict__ Tg, const float* __restrict__ x,
                                                    const uint8_t* __restrict__ mask, float* __restrict__ ye) {
    constexpr int NT = 7 * N * N;
    constexpr int EPT = MfF32Shape<N>::EPT, WPB = MfF32Shape<N>::WPB;
    constexpr int EW = 32 * EPT;                 // elements per warp pass
    __shared__ float T[NT];
    __shared__ int32_t sl2n[WPB][EW * (N + 1)];
    for (int k = threadIdx.x; k < NT; k += blockDim.x) T[k] = Tg[k];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int32_t* my = sl2n[warp];
    for (int64_t e0 = ((int64_t)blockIdx.x * WPB + warp) * EW; e0 < nt; e0 += (int64_t)gridDim.x * WPB * EW) {
        const int ne = (int)min((int64_t)EW, nt - e0);
        for (int k = lane; k < ne * N; k += 32) {
            const int el = k / N, j = k - el * N;
            my[el * (N + 1) + j] = __ldg(l2n + e0 * N + k);
        }
        __syncwarp();
        // lane handles elements e0 + 32 u + lane, u < EPT
        bool va[EPT];
        float xs[EPT][N];
        float c[EPT][7];
#pragma unroll
        for (int u = 0; u < EPT; ++u) {
            va[u] = lane + 32 * u < ne;
#pragma unroll
            for (int j = 0; j < N; ++j) {
                const int32_t d = va[u] ? my[(lane + 32 * u) * (N + 1) + j] : 0;
                xs[u][j] = (!va[u] || (mask && mask[d])) ? 0.0f : __ldg(x + d);
            }
            const int64_t e = va[u] ? e0 + 32 * u + lane : e0;
            const float4 r0 = __ldg(rec + 4 * e), r1 = __ldg(rec + 4 * e + 1);
            c[u][0] = r0.x; c[u][1] = r0.y; c[u][2] = r0.z; c[u][3] = r0.w; c[u][4] = r1.x; c[u][5] = r1.y; c[u][6] = r1.z;
        }
#pragma unroll 1
        for (int i = 0; i < N; ++i) {
            float acc[EPT];
#pragma unroll
            for (int u = 0; u < EPT; ++u) acc[u] = 0.0f;
#pragma unroll
            for (int k = 0; k < 7; ++k) {
                const float* Tk = T + (k * N + i) * N;
                float sm[EPT];
#pragma unroll
                for (int u = 0; u < EPT; ++u) sm[u] = 0.0f;
#pragma unroll
                for (int j = 0; j < N; ++j) {
                    const float t = Tk[j];
#pragma unroll
                    for (int u = 0; u < EPT; ++u) sm[u] = fmaf(t, xs[u][j], sm[u]);
                }
#pragma unroll
                for (int u = 0; u < EPT; ++u) acc[u] = fmaf(c[u][k], sm[u], acc[u]);
            }
#pragma unroll
            for (int u = 0; u < EPT; ++u)
                if (va[u]) ye[(int64_t)i * nt + e0 + 32 * u + lane] = acc[u];
        }
        __syncwarp();
    }
}

template <int N>
__global__ void __launch_bounds__(128) mf_element_f32_kernel(int64_t nt, const int32_t* __restrict__ l2n, const float4* __restrict__ rec,
                                                            const float* __restrict__ Tg, const float* __restrict__ x,
                                                            const uint8_t* __restrict__ mask, float* __restrict__ ye) {
    mf_element_f32_body<N>(nt, l2n, rec, Tg, x, mask, ye);
}

template <int N>
__global__ void __launch_bounds__(128) mf_element_f32_gated(int64_t nt, const int32_t* __restrict__ l2n, const float4* __restrict__ rec,
                                                           const float* __restrict__ Tg, const float* __restrict__ x,
                                                           const uint8_t* __restrict__ mask, float* __restrict__ ye,
                                                           const int* __restrict__ stop) {
    if (stop && *stop) return;
    mf_element_f32_body<N>(nt, l2n, rec, Tg, x, mask, ye);
}

// launch shape of the binary32 element phase: 32 WPB threads per block, enough blocks for one pass
// grid cap of the binary32 element phase (without it: P2 96^3 0.266 against 0.252 ms, P3 0.784 against 0.793)
constexpr int64_t kMfElemCap = 152 * 32;
template <int N>
static void launch_mf_element_f32(cudaStream_t st, int64_t nt, const int32_t* l2n, const float4* rec, const float* T7f,
                                  const float* x, const uint8_t* mask, float* ye, const int* stop, bool gated) {
    constexpr int WPB = MfF32Shape<N>::WPB, EW = 32 * MfF32Shape<N>::EPT;
    const int64_t per_block = (int64_t)WPB * EW;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((nt + per_block - 1) / per_block, kMfElemCap));
    if (gated) mf_element_f32_gated<N><<<blocks, 32 * WPB, 0, st>>>(nt, l2n, rec, T7f, x, mask, ye, stop);
    else mf_element_f32_kernel<N><<<blocks, 32 * WPB, 0, st>>>(nt, l2n, rec, T7f, x, mask, ye);
}

// native binary64: one thread per element (FP64 pipe), coefficients from the
// binary64 geometry records (8 doubles).
template <int N>
__global__ void __launch_bounds__(128) mf_element_f64_kernel(int64_t nt, const int32_t* __restrict__ l2n, const double* __restrict__ coef,
                                                            const double* __restrict__ Tg, const double* __restrict__ x,
                                                            const uint8_t* __restrict__ mask, double* __restrict__ ye) {
    constexpr int NT = 7 * N * N;
    extern __shared__ double Td[];
    for (int k = threadIdx.x; k < NT; k += blockDim.x) Td[k] = Tg[k];
    __syncthreads();
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nt; e += (int64_t)gridDim.x * blockDim.x) {
        double xe[N];
#pragma unroll
        for (int j = 0; j < N; ++j) {
            const int32_t d = l2n[e * N + j];
            xe[j] = (mask && mask[d]) ? 0.0 : x[d];
        }
        const double* c = coef + 8 * e;
#pragma unroll 1
        for (int i = 0; i < N; ++i) {
            double acc = 0.0;
#pragma unroll 1
            for (int k = 0; k < 7; ++k) {
                const double* Tk = Td + (k * N + i) * N;
                double s = 0.0;
#pragma unroll
                for (int j = 0; j < N; ++j) s = fma(Tk[j], xe[j], s);
                acc = fma(c[k], s, acc);
            }
            ye[(int64_t)i * nt + e] = acc;
        }
    }
}

// df64: one thread per element; x and y in binary64 memory, converted with integer
// operations; products and sums as double-float.
template <int N>
__global__ void __launch_bounds__(128) mf_element_df_kernel(int64_t nt, const int32_t* __restrict__ l2n, const float4* __restrict__ rec,
                                                           const float* __restrict__ Thg, const float* __restrict__ Tlg,
                                                           const double* __restrict__ x, const uint8_t* __restrict__ mask,
                                                           double* __restrict__ ye) {
    constexpr int NT = 7 * N * N;
    extern __shared__ float Tsh[];
    float* Th = Tsh;
    float* Tl = Tsh + NT;
    for (int k = threadIdx.x; k < NT; k += blockDim.x) {
        Th[k] = Thg[k];
        Tl[k] = Tlg[k];
    }
    __syncthreads();
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nt; e += (int64_t)gridDim.x * blockDim.x) {
        df xe[N];
#pragma unroll
        for (int j = 0; j < N; ++j) {
            const int32_t d = l2n[e * N + j];
            xe[j] = (mask && mask[d]) ? df{0.0f, 0.0f} : d2df(x[d]);
        }
        const float4 h0 = __ldg(rec + 4 * e), h1 = __ldg(rec + 4 * e + 1), l0 = __ldg(rec + 4 * e + 2), l1 = __ldg(rec + 4 * e + 3);
        const df c[7] = {{h0.x, l0.x}, {h0.y, l0.y}, {h0.z, l0.z}, {h0.w, l0.w}, {h1.x, l1.x}, {h1.y, l1.y}, {h1.z, l1.z}};
#pragma unroll 1
        for (int i = 0; i < N; ++i) {
            df acc{0.0f, 0.0f};
#pragma unroll 1
            for (int k = 0; k < 7; ++k) {
                const int o = (k * N + i) * N;
                df s{0.0f, 0.0f};
#pragma unroll
                for (int j = 0; j < N; ++j) s = df_add(s, df_mul(df{Th[o + j], Tl[o + j]}, xe[j]));
                acc = df_add(acc, df_mul(c[k], s));
            }
            ye[(int64_t)i * nt + e] = df2d(acc);
        }
    }
}

// ---------------------------------------------------------------------------
// node phase: y[m] = sum_{(e,li) in inc(m)} ye[li][e] (element order); Dirichlet rows y = x.
// Element values are stored local-index-major (ye[i * nt + e]) so that the
// element kernels, one thread per element, write them coalesced.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void mf_gather_kernel(int64_t nnodes, int64_t nt, const int64_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                                 const T* __restrict__ ye, const T* __restrict__ x, const uint8_t* __restrict__ mask,
                                 T* __restrict__ y) {
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < nnodes; m += (int64_t)gridDim.x * blockDim.x) {
        if (mask && mask[m]) {
            y[m] = x[m];
            continue;
        }
        // incident element values in batches of 4 (loads issued together), summed in element order
        T s = 0;
        const int64_t t0 = inc_ptr[m], t1 = inc_ptr[m + 1];
        for (int64_t t = t0; t < t1; t += 4) {
            int32_t code[4];
            T v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) code[u] = t + u < t1 ? __ldg(inc + t + u) : 0;
#pragma unroll
            for (int u = 0; u < 4; ++u) v[u] = t + u < t1 ? __ldg(ye + (int64_t)(code[u] & 31) * nt + (code[u] >> 5)) : T(0);
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (t + u < t1) s += v[u];
        }
        y[m] = s;
    }
}

// binary32 node gather that returns at once when *stop is set (used inside captured graphs)
__global__ void mf_gather_f32_stop_kernel(int64_t nnodes, int64_t nt, const int64_t* __restrict__ inc_ptr,
                                          const int32_t* __restrict__ inc, const float* __restrict__ ye,
                                          const float* __restrict__ x, const uint8_t* __restrict__ mask, float* __restrict__ y,
                                          const int* __restrict__ stop) {
    if (stop && *stop) return;
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < nnodes; m += (int64_t)gridDim.x * blockDim.x) {
        if (mask && mask[m]) {
            y[m] = x[m];
            continue;
        }
        float s = 0.0f;
        const int64_t t0 = inc_ptr[m], t1 = inc_ptr[m + 1];
        for (int64_t t = t0; t < t1; t += 4) {
            int32_t code[4];
            float v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) code[u] = t + u < t1 ? __ldg(inc + t + u) : 0;
#pragma unroll
            for (int u = 0; u < 4; ++u) v[u] = t + u < t1 ? __ldg(ye + (int64_t)(code[u] & 31) * nt + (code[u] >> 5)) : 0.0f;
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (t + u < t1) s += v[u];
        }
        y[m] = s;
    }
}

// df64 summation of binary64 element values (keeps ~48 bits in the node sum)
__global__ void mf_gather_df_kernel(int64_t nnodes, int64_t nt, const int64_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                                    const double* __restrict__ ye, const double* __restrict__ x, const uint8_t* __restrict__ mask,
                                    double* __restrict__ y) {
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < nnodes; m += (int64_t)gridDim.x * blockDim.x) {
        if (mask && mask[m]) {
            y[m] = x[m];
            continue;
        }
        df s{0.0f, 0.0f};
        for (int64_t t = inc_ptr[m]; t < inc_ptr[m + 1]; ++t) {
            const int32_t code = inc[t];
            s = df_add(s, d2df(ye[(int64_t)(code & 31) * nt + (code >> 5)]));
        }
        y[m] = df2d(s);
    }
}

// x with the Dirichlet entries zeroed (the element phase then gathers without
// reading the mask); gated by the CG stop flag
__global__ void mask_copy_f32_kernel(int64_t n, const float* __restrict__ x, const uint8_t* __restrict__ mask, float* __restrict__ xm,
                                     const int* __restrict__ stop) {
    if (stop && *stop) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        xm[i] = mask[i] ? 0.0f : x[i];
}

// ---- graph-coloured scatter (FGPU_ALGO_COLOUR): elements coloured so that two
// elements of a colour share no vertex (hence no dof); per colour, one thread
// per element computes y_e = K_e x_e and adds it into y directly. No element
// buffer and no node phase; every entry of y receives its element
// contributions in colour order (deterministic, no atomics).
template <int N>
__global__ void __launch_bounds__(128) mf_scatter_f32_kernel(int64_t c0, int64_t c1, const int32_t* __restrict__ perm,
                                                             const int32_t* __restrict__ l2n, const float4* __restrict__ rec,
                                                             const float* __restrict__ Tg, const float* __restrict__ xm,
                                                             const uint8_t* __restrict__ mask, float* __restrict__ y,
                                                             const int* __restrict__ stop) {
    if (stop && *stop) return;
    constexpr int NT = 7 * N * N;
    __shared__ float T[NT];
    for (int k = threadIdx.x; k < NT; k += blockDim.x) T[k] = Tg[k];
    __syncthreads();
    for (int64_t k = c0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < c1; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = perm[k];
        int32_t d[N];
        float xe[N];
#pragma unroll
        for (int j = 0; j < N; ++j) {
            d[j] = __ldg(l2n + e * N + j);
            xe[j] = __ldg(xm + d[j]);          // x with the Dirichlet entries zeroed
        }
        const float4 h0 = __ldg(rec + 4 * e), h1 = __ldg(rec + 4 * e + 1);
        const float c[7] = {h0.x, h0.y, h0.z, h0.w, h1.x, h1.y, h1.z};
#pragma unroll 1
        for (int i = 0; i < N; ++i) {
            float acc = 0.0f;
#pragma unroll
            for (int kk = 0; kk < 7; ++kk) {
                const float* Tk = T + (kk * N + i) * N;
                float sum = 0.0f;
#pragma unroll
                for (int j = 0; j < N; ++j) sum = fmaf(Tk[j], xe[j], sum);
                acc = fmaf(c[kk], sum, acc);
            }
            if (!(mask && mask[d[i]])) y[d[i]] += acc;
        }
    }
}

// y = (Dirichlet rows) x, else 0; and the masked copy xm of x
__global__ void scatter_init_f32_kernel(int64_t n, const float* __restrict__ x, const uint8_t* __restrict__ mask,
                                        float* __restrict__ y, float* __restrict__ xm, const int* __restrict__ stop) {
    if (stop && *stop) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const bool m = mask && mask[i];
        y[i] = m ? x[i] : 0.0f;
        xm[i] = m ? 0.0f : x[i];
    }
}

// diagonal of the operator (Jacobi): element diagonals then the node gather
template <typename T>
__global__ void mf_diag_element_kernel(int64_t nt, int N, const float4* __restrict__ rec, const double* __restrict__ T7,
                                       T* __restrict__ ye) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nt; e += (int64_t)gridDim.x * blockDim.x) {
        const float4 h0 = rec[4 * e], h1 = rec[4 * e + 1], l0 = rec[4 * e + 2], l1 = rec[4 * e + 3];
        const double c[7] = {(double)h0.x + l0.x, (double)h0.y + l0.y, (double)h0.z + l0.z, (double)h0.w + l0.w,
                             (double)h1.x + l1.x, (double)h1.y + l1.y, (double)h1.z + l1.z};
        for (int i = 0; i < N; ++i) {
            double s = 0;
            for (int k = 0; k < 7; ++k) s += c[k] * T7[(k * N + i) * N + i];
            ye[(int64_t)i * nt + e] = (T)s;
        }
    }
}

}  // namespace fgpu

// ---------------------------------------------------------------------------
// operator object
// ---------------------------------------------------------------------------
struct fgpu_operator {
    fgpu_ctx* ctx = nullptr;
    fgpu_space* space = nullptr;
    int precision = FGPU_F32;        // FGPU_F32, FGPU_F64 (native) or FGPU_DF64 (double-float)
    int qdeg = 0;
    fgpu::DevTables* tab = nullptr;
    float4* d_rec = nullptr;         // df64 coefficient records (T x 4 float4)
    double* d_coef = nullptr;        // binary64 coefficient records (native FP64 path)
    void* d_ye = nullptr;            // element buffer T x n (float or double)
    uint8_t* d_mask = nullptr;       // Dirichlet mask (nnodes) or null
    void* d_diag = nullptr;          // operator diagonal (float or double)
    float* d_xf = nullptr;           // binary32 copies of x and y for fgpu_operator_apply on binary64 vectors
    float* d_yf = nullptr;
    float* d_xm = nullptr;           // binary32 x with the Dirichlet entries zeroed (element phase input)
    int64_t nt = 0, nnodes = 0;
    int use_tc = 0;                  // binary32 element phase on the tensor cores (tcgen05, P2/P3)
    int tc_chosen = 0;               // use_tc set by fgpu_operator_set_tensor_cores (not the default)
    int algo = FGPU_ALGO_GATHER;     // FGPU_ALGO_GATHER (element buffer + node gather) or FGPU_ALGO_COLOUR
    float* d_xs = nullptr;           // colour scatter: masked copy of x
};

namespace fgpu {
int launch_mf_element_tc(fgpu_ctx* ctx, int n, int64_t nt, const int32_t* l2n, const float4* rec, const float* T7f, const float* x,
                         const uint8_t* mask, float* ye, const int* stop);
int launch_geometry(fgpu_ctx* ctx, const fgpu_mesh* mesh, int kind, const double* d_kappa, double kappa, double mass,
                    double lam, double mu, double* d_coef);

// grid cap of the node gathers: none (one thread per node; blocks are issued in node order, so the
// incident element values a block reads were just read by its neighbours). A cap of 152 x 16 blocks with
// a grid-stride loop took 0.534 against 0.487 ms for the P3 96^3 node phase
constexpr int kMfGatherCap = 1 << 30;

static int blocks_for(int64_t n, int threads, int cap) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads, cap));
}

static int mf_apply_colour_f32(fgpu_ctx* ctx, fgpu_operator* op, const float* x, float* y, const int* stop);

// y = A x; x, y device arrays of nnodes entries in the operator's storage type
// (float for F32, double for F64 / DF64)
int operator_apply(fgpu_ctx* ctx, fgpu_operator* op, const void* x, void* y) {
    const fgpu_space* V = op->space;
    const int n = V->n;
    const int64_t nt = op->nt;
    PendingEvent ev;
    if (op->precision == FGPU_F32 && op->algo == FGPU_ALGO_COLOUR) {
        prof_begin(ctx, "matfree_element", ev);
        ctx->launches += mf_apply_colour_f32(ctx, op, (const float*)x, (float*)y, nullptr);
        prof_end(ctx, ev);
        FGPU_CUDA_CHECK(ctx, cudaGetLastError());
        return FGPU_OK;
    }
    prof_begin(ctx, "matfree_element", ev);
    const int eb = blocks_for(nt, 128, 152 * 16);
    const float* xe = (const float*)x;
    const uint8_t* me = op->d_mask;
    if (op->precision == FGPU_F32 && op->d_mask && op->d_xm) {
        mask_copy_f32_kernel<<<blocks_for(op->nnodes, 256, 152 * 8), 256, 0, ctx->stream>>>(op->nnodes, (const float*)x, op->d_mask,
                                                                                        op->d_xm, nullptr);
        ++ctx->launches;
        xe = op->d_xm;
        me = nullptr;
    }
    if (op->precision == FGPU_F32 && op->use_tc && (n == 10 || n == 20)) {
        int rc = launch_mf_element_tc(ctx, n, nt, V->d_l2n, op->d_rec, op->tab->d_T7f, xe, me, (float*)op->d_ye, nullptr);
        if (rc) return rc;
    } else if (op->precision == FGPU_F32) {
        switch (n) {
            case 4: launch_mf_element_f32<4>(ctx->stream, nt, V->d_l2n, op->d_rec, op->tab->d_T7f, xe, me, (float*)op->d_ye, nullptr, false); break;
            case 10: launch_mf_element_f32<10>(ctx->stream, nt, V->d_l2n, op->d_rec, op->tab->d_T7f, xe, me, (float*)op->d_ye, nullptr, false); break;
            case 20: launch_mf_element_f32<20>(ctx->stream, nt, V->d_l2n, op->d_rec, op->tab->d_T7f, xe, me, (float*)op->d_ye, nullptr, false); break;
            default: return FGPU_ERR_INVALID;
        }
    } else if (op->precision == FGPU_F64) {
        const size_t sm = 7 * n * n * sizeof(double);
        switch (n) {
            case 4: mf_element_f64_kernel<4><<<eb, 128, sm, ctx->stream>>>(nt, V->d_l2n, op->d_coef, op->tab->d_T7, (const double*)x, op->d_mask, (double*)op->d_ye); break;
            case 10: mf_element_f64_kernel<10><<<eb, 128, sm, ctx->stream>>>(nt, V->d_l2n, op->d_coef, op->tab->d_T7, (const double*)x, op->d_mask, (double*)op->d_ye); break;
            case 20: mf_element_f64_kernel<20><<<eb, 128, sm, ctx->stream>>>(nt, V->d_l2n, op->d_coef, op->tab->d_T7, (const double*)x, op->d_mask, (double*)op->d_ye); break;
            default: return FGPU_ERR_INVALID;
        }
    } else {
        const size_t sm = 2 * 7 * n * n * sizeof(float);
        switch (n) {
            case 4: mf_element_df_kernel<4><<<eb, 128, sm, ctx->stream>>>(nt, V->d_l2n, op->d_rec, op->tab->d_T7h, op->tab->d_T7l, (const double*)x, op->d_mask, (double*)op->d_ye); break;
            case 10: mf_element_df_kernel<10><<<eb, 128, sm, ctx->stream>>>(nt, V->d_l2n, op->d_rec, op->tab->d_T7h, op->tab->d_T7l, (const double*)x, op->d_mask, (double*)op->d_ye); break;
            case 20: mf_element_df_kernel<20><<<eb, 128, sm, ctx->stream>>>(nt, V->d_l2n, op->d_rec, op->tab->d_T7h, op->tab->d_T7l, (const double*)x, op->d_mask, (double*)op->d_ye); break;
            default: return FGPU_ERR_INVALID;
        }
    }
    prof_end(ctx, ev);
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    PendingEvent ev2;
    prof_begin(ctx, "matfree_gather", ev2);
    const int gb = blocks_for(op->nnodes, 256, kMfGatherCap);
    if (op->precision == FGPU_F32)
        mf_gather_kernel<float><<<gb, 256, 0, ctx->stream>>>(op->nnodes, op->nt, V->d_inc_ptr, V->d_inc, (const float*)op->d_ye, (const float*)x, op->d_mask, (float*)y);
    else if (op->precision == FGPU_F64)
        mf_gather_kernel<double><<<gb, 256, 0, ctx->stream>>>(op->nnodes, op->nt, V->d_inc_ptr, V->d_inc, (const double*)op->d_ye, (const double*)x, op->d_mask, (double*)y);
    else
        mf_gather_df_kernel<<<gb, 256, 0, ctx->stream>>>(op->nnodes, op->nt, V->d_inc_ptr, V->d_inc, (const double*)op->d_ye, (const double*)x, op->d_mask, (double*)y);
    prof_end(ctx, ev2);
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

int operator_diagonal(fgpu_ctx* ctx, fgpu_operator* op) {
    const fgpu_space* V = op->space;
    const int n = V->n;
    const bool f32 = op->precision == FGPU_F32;
    const size_t es = f32 ? sizeof(float) : sizeof(double);
    if (!op->d_diag) FGPU_CUDA_CHECK(ctx, cudaMalloc(&op->d_diag, op->nnodes * es));
    void* ones = nullptr;
    FGPU_CUDA_CHECK(ctx, cudaMalloc(&ones, op->nnodes * es));
    // Dirichlet rows: diag 1 (x = 1 passes through the mask branch)
    std::vector<char> h(op->nnodes * es);
    if (f32) { float* p = (float*)h.data(); for (int64_t i = 0; i < op->nnodes; ++i) p[i] = 1.0f; }
    else { double* p = (double*)h.data(); for (int64_t i = 0; i < op->nnodes; ++i) p[i] = 1.0; }
    cudaMemcpyAsync(ones, h.data(), h.size(), cudaMemcpyHostToDevice, ctx->stream);
    const int eb = blocks_for(op->nt, 256, 152 * 16);
    if (f32) mf_diag_element_kernel<float><<<eb, 256, 0, ctx->stream>>>(op->nt, n, op->d_rec, op->tab->d_T7, (float*)op->d_ye);
    else mf_diag_element_kernel<double><<<eb, 256, 0, ctx->stream>>>(op->nt, n, op->d_rec, op->tab->d_T7, (double*)op->d_ye);
    const int gb = blocks_for(op->nnodes, 256, kMfGatherCap);
    if (f32) mf_gather_kernel<float><<<gb, 256, 0, ctx->stream>>>(op->nnodes, op->nt, V->d_inc_ptr, V->d_inc, (const float*)op->d_ye, (const float*)ones, op->d_mask, (float*)op->d_diag);
    else mf_gather_kernel<double><<<gb, 256, 0, ctx->stream>>>(op->nnodes, op->nt, V->d_inc_ptr, V->d_inc, (const double*)op->d_ye, (const double*)ones, op->d_mask, (double*)op->d_diag);
    ctx->launches += 2;
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    cudaFree(ones);
    if (e != cudaSuccess) { ctx->err = cudaGetErrorString(e); return FGPU_ERR_CUDA; }
    return FGPU_OK;
}

}  // namespace fgpu

// ===========================================================================
// matrix-free CG
// ===========================================================================
#include "cg_driver.cuh"

namespace fgpu {
// per-block partials of x.y
template <class PL>
__global__ void dot_partial_kernel(int64_t n, const typename PL::S* __restrict__ x, const typename PL::S* __restrict__ y,
                                   typename PL::D* __restrict__ partial, const CGScalars<PL>* __restrict__ sc) {
    if (sc && sc->done) return;
    __shared__ typename PL::D sh[32];
    typename PL::D s = PL::dzero();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s = PL::dmadd(s, PL::ld(x[i]), PL::ld(y[i]));
    const typename PL::D t = block_sum<PL>(s, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

}  // namespace fgpu

namespace fgpu {

// q = A p fused with the p.q partial sums (node phase of the apply)
template <class PL>
__global__ void mf_gather_dot_kernel(int64_t nnodes, int64_t nt, const int64_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                                     const typename PL::S* __restrict__ ye, const typename PL::S* __restrict__ x,
                                     const uint8_t* __restrict__ mask, typename PL::S* __restrict__ y,
                                     typename PL::D* __restrict__ partial, const CGScalars<PL>* __restrict__ sc) {
    if (sc && sc->done) return;
    __shared__ typename PL::D sh[32];
    typename PL::D dsum = PL::dzero();
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < nnodes; m += (int64_t)gridDim.x * blockDim.x) {
        typename PL::S v;
        if (mask && mask[m]) {
            v = x[m];
        } else {
            // incident element values in batches of 4 (loads issued together), summed in element order
            typename PL::A s = PL::zero();
            const int64_t t0 = inc_ptr[m], t1 = inc_ptr[m + 1];
            for (int64_t t = t0; t < t1; t += 4) {
                int32_t code[4];
                typename PL::S w[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) code[u] = t + u < t1 ? __ldg(inc + t + u) : 0;
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (t + u < t1) w[u] = ye[(int64_t)(code[u] & 31) * nt + (code[u] >> 5)];
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (t + u < t1) s = PL::add(s, PL::ld(w[u]));
            }
            v = PL::st(s);
        }
        y[m] = v;
        if (partial) dsum = PL::dmadd(dsum, PL::ld(x[m]), PL::ld(v));
    }
    if (partial) {
        const typename PL::D t = block_sum<PL>(dsum, sh);
        if (threadIdx.x == 0) partial[blockIdx.x] = t;
    }
}

// element phase gated by the CG stop flag (runs inside the captured graph)


template <typename T>
__global__ void copy_cast_kernel(int64_t n, const double* __restrict__ a, T* __restrict__ b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) b[i] = (T)a[i];
}
template <typename T>
__global__ void cast_back_kernel(int64_t n, const T* __restrict__ a, double* __restrict__ b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) b[i] = (double)a[i];
}
template <class PL>
__global__ void dinv_from_diag_kernel(int64_t n, const typename PL::S* __restrict__ d, typename PL::S* __restrict__ dinv, int use_pc) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const typename PL::A v = PL::ld(d[i]);
        dinv[i] = PL::st((use_pc && PL::nonzero(v)) ? PL::recip(v) : PL::one());
    }
}

int operator_apply(fgpu_ctx* ctx, fgpu_operator* op, const void* x, void* y);

// element phase + fused node phase; F32 uses the gated kernel (graph-safe)
// FGPU_ALGO_COLOUR binary32 apply: y = A x, with optional x.y partials
static int mf_apply_colour_f32(fgpu_ctx* ctx, fgpu_operator* op, const float* x, float* y, const int* stop) {
    const fgpu_space* V = op->space;
    const fgpu_mesh* M = V->mesh;
    const int n = V->n;
    int nl = 1;
    scatter_init_f32_kernel<<<blocks_for(op->nnodes, 256, 152 * 8), 256, 0, ctx->stream>>>(op->nnodes, x, op->d_mask, y, op->d_xs, stop);
    for (int c = 0; c < M->ncolours; ++c) {
        const int64_t c0 = M->colour_ptr[c], c1 = M->colour_ptr[c + 1];
        if (c1 <= c0) continue;
        const int b = blocks_for(c1 - c0, 128, 152 * 16);
        switch (n) {
            case 4: mf_scatter_f32_kernel<4><<<b, 128, 0, ctx->stream>>>(c0, c1, M->d_colour_perm, V->d_l2n, op->d_rec, op->tab->d_T7f, op->d_xs, op->d_mask, y, stop); break;
            case 10: mf_scatter_f32_kernel<10><<<b, 128, 0, ctx->stream>>>(c0, c1, M->d_colour_perm, V->d_l2n, op->d_rec, op->tab->d_T7f, op->d_xs, op->d_mask, y, stop); break;
            default: mf_scatter_f32_kernel<20><<<b, 128, 0, ctx->stream>>>(c0, c1, M->d_colour_perm, V->d_l2n, op->d_rec, op->tab->d_T7f, op->d_xs, op->d_mask, y, stop); break;
        }
        ++nl;
    }
    return nl;
}

// returns the number of kernels launched
template <class PL>
static int mf_apply_cg(fgpu_ctx* ctx, fgpu_operator* op, const typename PL::S* x, typename PL::S* y, typename PL::D* partial,
                       const CGScalars<PL>* sc, int gblocks) {
    const fgpu_space* V = op->space;
    const int n = V->n;
    const int eb = blocks_for(op->nt, 128, 152 * 16);
    const int* stop = sc ? &sc->done : nullptr;
    if (op->precision == FGPU_F32 && op->algo == FGPU_ALGO_COLOUR) {
        int nc = mf_apply_colour_f32(ctx, op, (const float*)x, (float*)y, stop);
        if (partial) {
            dot_partial_kernel<PL><<<gblocks, 256, 0, ctx->stream>>>(op->nnodes, x, y, partial, sc);
            ++nc;
        }
        return nc;
    }
    int nl = 2;
    const float* xe = (const float*)x;
    const uint8_t* me = op->d_mask;
    if (op->precision == FGPU_F32 && op->d_mask && op->d_xm) {
        mask_copy_f32_kernel<<<blocks_for(op->nnodes, 256, 152 * 8), 256, 0, ctx->stream>>>(op->nnodes, (const float*)x, op->d_mask,
                                                                                        op->d_xm, stop);
        ++nl;
        xe = op->d_xm;
        me = nullptr;
    }
    if (op->precision == FGPU_F32 && op->use_tc && (n == 10 || n == 20)) {
        launch_mf_element_tc(ctx, n, op->nt, V->d_l2n, op->d_rec, op->tab->d_T7f, xe, me, (float*)op->d_ye, stop);
    } else if (op->precision == FGPU_F32) {
        switch (n) {
            case 4: launch_mf_element_f32<4>(ctx->stream, op->nt, V->d_l2n, op->d_rec, op->tab->d_T7f, xe, me, (float*)op->d_ye, stop, true); break;
            case 10: launch_mf_element_f32<10>(ctx->stream, op->nt, V->d_l2n, op->d_rec, op->tab->d_T7f, xe, me, (float*)op->d_ye, stop, true); break;
            default: launch_mf_element_f32<20>(ctx->stream, op->nt, V->d_l2n, op->d_rec, op->tab->d_T7f, xe, me, (float*)op->d_ye, stop, true); break;
        }
    } else {
        // binary64 element phases (native or df64); not gated: the FP64 matrix-free solve polls every iteration
        const int save = ctx->profile;
        ctx->profile = 0;
        const size_t sm64 = 7 * n * n * sizeof(double), smdf = 2 * 7 * n * n * sizeof(float);
        if (op->precision == FGPU_F64) {
            switch (n) {
                case 4: mf_element_f64_kernel<4><<<eb, 128, sm64, ctx->stream>>>(op->nt, V->d_l2n, op->d_coef, op->tab->d_T7, (const double*)x, op->d_mask, (double*)op->d_ye); break;
                case 10: mf_element_f64_kernel<10><<<eb, 128, sm64, ctx->stream>>>(op->nt, V->d_l2n, op->d_coef, op->tab->d_T7, (const double*)x, op->d_mask, (double*)op->d_ye); break;
                default: mf_element_f64_kernel<20><<<eb, 128, sm64, ctx->stream>>>(op->nt, V->d_l2n, op->d_coef, op->tab->d_T7, (const double*)x, op->d_mask, (double*)op->d_ye); break;
            }
        } else {
            switch (n) {
                case 4: mf_element_df_kernel<4><<<eb, 128, smdf, ctx->stream>>>(op->nt, V->d_l2n, op->d_rec, op->tab->d_T7h, op->tab->d_T7l, (const double*)x, op->d_mask, (double*)op->d_ye); break;
                case 10: mf_element_df_kernel<10><<<eb, 128, smdf, ctx->stream>>>(op->nt, V->d_l2n, op->d_rec, op->tab->d_T7h, op->tab->d_T7l, (const double*)x, op->d_mask, (double*)op->d_ye); break;
                default: mf_element_df_kernel<20><<<eb, 128, smdf, ctx->stream>>>(op->nt, V->d_l2n, op->d_rec, op->tab->d_T7h, op->tab->d_T7l, (const double*)x, op->d_mask, (double*)op->d_ye); break;
            }
        }
        ctx->profile = save;
    }
    // the node phase with one thread per node, then the p.q partials on the CG's block layout (the same
    // partials, hence the same bits, as the fused gather-dot kernel on that small grid, which took 0.82
    // against 0.53 ms for the gather alone at P3 96^3)
    mf_gather_dot_kernel<PL><<<blocks_for(op->nnodes, 256, kMfGatherCap), 256, 0, ctx->stream>>>(
        op->nnodes, op->nt, V->d_inc_ptr, V->d_inc, (const typename PL::S*)op->d_ye, x, op->d_mask, y, nullptr, sc);
    if (partial) {
        dot_partial_kernel<PL><<<gblocks, 256, 0, ctx->stream>>>(op->nnodes, x, y, partial, sc);
        ++nl;
    }
    return nl;
}

// y = A x for a binary32 operator with every kernel gated by *stop (for preconditioners that apply
// the operator inside the CG graph); returns the number of kernels launched
int mf_apply_f32_gated(fgpu_ctx* ctx, fgpu_operator* op, const float* x, float* y, const int* stop) {
    const fgpu_space* V = op->space;
    const int n = V->n;
    if (op->algo == FGPU_ALGO_COLOUR) return mf_apply_colour_f32(ctx, op, x, y, stop);
    int nl = 2;
    const float* xe = x;
    const uint8_t* me = op->d_mask;
    if (op->d_mask && op->d_xm) {
        mask_copy_f32_kernel<<<blocks_for(op->nnodes, 256, 152 * 8), 256, 0, ctx->stream>>>(op->nnodes, x, op->d_mask, op->d_xm, stop);
        ++nl;
        xe = op->d_xm;
        me = nullptr;
    }
    const int eb = blocks_for(op->nt, 128, 152 * 16);
    if (op->use_tc && (n == 10 || n == 20)) {
        launch_mf_element_tc(ctx, n, op->nt, V->d_l2n, op->d_rec, op->tab->d_T7f, xe, me, (float*)op->d_ye, stop);
    } else {
        switch (n) {
            case 4: launch_mf_element_f32<4>(ctx->stream, op->nt, V->d_l2n, op->d_rec, op->tab->d_T7f, xe, me, (float*)op->d_ye, stop, true); break;
            case 10: launch_mf_element_f32<10>(ctx->stream, op->nt, V->d_l2n, op->d_rec, op->tab->d_T7f, xe, me, (float*)op->d_ye, stop, true); break;
            default: launch_mf_element_f32<20>(ctx->stream, op->nt, V->d_l2n, op->d_rec, op->tab->d_T7f, xe, me, (float*)op->d_ye, stop, true); break;
        }
    }
    mf_gather_f32_stop_kernel<<<blocks_for(op->nnodes, 256, kMfGatherCap), 256, 0, ctx->stream>>>(
        op->nnodes, op->nt, V->d_inc_ptr, V->d_inc, (const float*)op->d_ye, x, op->d_mask, y, stop);
    return nl;
}

int64_t operator_nnodes(const fgpu_operator* op) { return op->nnodes; }
int operator_precision(const fgpu_operator* op) { return op->precision; }
const fgpu_space* operator_space(const fgpu_operator* op) { return op->space; }
const uint8_t* operator_mask(const fgpu_operator* op) { return op->d_mask; }
const float* operator_diag_f32(fgpu_ctx* ctx, fgpu_operator* op) {
    if (op->precision != FGPU_F32) return nullptr;
    if (!op->d_diag && operator_diagonal(ctx, op) != FGPU_OK) return nullptr;
    return (const float*)op->d_diag;
}

// Matrix-free PCG with Jacobi or Chebyshev-Jacobi (operator diagonal). The
// binary32 operator's iterations run from a captured graph like the CSR
// solver; the binary64 ones launch per iteration (their element phase is
// long, launch overhead is noise, and it is not gated by the stop flag).
template <class PL>
static int mf_pcg_core(fgpu_ctx* ctx, fgpu_operator* op, const typename PL::S* b, typename PL::S* x, const CgOptions& o, int pc,
                       CgResult* res, const RefreshFn<PL>* refresh = nullptr, fgpu_pmg* pmg = nullptr) {
    typedef typename PL::S S;
    const int64_t n = op->nnodes;
    const int vb = vec_blocks(n);
    S* dinv = nullptr;
    if (cudaMalloc(&dinv, n * sizeof(S)) != cudaSuccess) { ctx->err = "matrix-free CG: allocation failed"; return FGPU_ERR_ALLOC; }
    dinv_from_diag_kernel<PL><<<vb, 256, 0, ctx->stream>>>(n, (const S*)op->d_diag, dinv, pc != FGPU_PC_NONE);
    ctx->launches++;
    CgOperator<PL> A;
    A.apply = [ctx, op, vb](const S* xx, S* yy, typename PL::D* partial, const CGScalars<PL>* sc) {
        mf_apply_cg<PL>(ctx, op, xx, yy, partial, sc, vb);   // cg_run counts the launches of an application
    };
    A.npq = vb;
    if (op->precision == FGPU_F32 && op->algo == FGPU_ALGO_COLOUR) {
        int nc = 0;
        for (int c = 0; c < op->space->mesh->ncolours; ++c)
            if (op->space->mesh->colour_ptr[c + 1] > op->space->mesh->colour_ptr[c]) ++nc;
        A.launches = 2 + nc;          // init, colours, dot
    } else {
        A.launches = (op->precision == FGPU_F32 && op->d_mask && op->d_xm) ? 3 : 2;
    }
    A.graph = op->precision == FGPU_F32;
    PcHook<PL> hook;
    if (pmg) hook = pmg_pc_hook<PL>(pmg);
    const int rc = cg_run<PL>(ctx, n, A, dinv, b, x, o, res, refresh, pmg ? &hook : nullptr);
    cudaFree(dinv);
    return rc;
}

static double host_norm(fgpu_ctx* ctx, int64_t n, const double* d) {
    const int vb = vec_blocks(n);
    double* partial = nullptr;
    std::vector<double> h(vb, 0.0);
    if (cudaMalloc(&partial, vb * sizeof(double)) != cudaSuccess) return NAN;
    norm2_partial_kernel<<<vb, 256, 0, ctx->stream>>>(n, d, partial);
    ctx->launches++;
    cudaMemcpyAsync(h.data(), partial, vb * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    cudaFree(partial);
    double s = 0;
    for (double v : h) s += v;
    return std::sqrt(s);
}

// ||b - A x|| with the binary64 (native or df64) operator
static int mf_residual64(fgpu_ctx* ctx, fgpu_operator* op, const double* b, const double* x, double* r, double* q, double* out) {
    ctx->launches += mf_apply_cg<PolF64>(ctx, op, x, q, nullptr, nullptr, vec_blocks(op->nnodes));
    residual_from_q_kernel<PolF64><<<vec_blocks(op->nnodes), 256, 0, ctx->stream>>>(op->nnodes, b, q, r);
    ctx->launches++;
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    *out = host_norm(ctx, op->nnodes, r);
    return FGPU_OK;
}

// binary64 PCG with residual replacement at each convergence claim of the
// recurrence (q: scratch vector of n doubles)
static int mf_plain_solve(fgpu_ctx* ctx, fgpu_operator* op, const double* d_b, double* d_x, CgOptions o,
                          const fgpu_solver_cfg* cfg, double bn, double* q, CgResult* res, fgpu_pmg* pmg = nullptr) {
    o.delta = 0.0;
    int stagnant = 0;
    double rlast = 0;
    RefreshFn<PolF64> refresh = [&](double* xd, double* rd, bool* conv) -> int {
        double r2n = 0;
        const int r2 = mf_residual64(ctx, op, d_b, xd, rd, q, &r2n);
        if (r2) return r2;
        *conv = r2n <= cfg->rtol * bn;
        stagnant = (rlast > 0 && r2n > 0.5 * rlast) ? stagnant + 1 : 0;
        rlast = r2n;
        if (!*conv && stagnant >= 2) return kRefreshStagnated;
        return FGPU_OK;
    };
    return mf_pcg_core<PolF64>(ctx, op, d_b, d_x, o, cfg->pc, res, &refresh, pmg);
}

int solve_cg_operator(fgpu_ctx* ctx, fgpu_operator* op, fgpu_operator* op32, const double* d_b, double* d_x,
                      const fgpu_solver_cfg* cfg, fgpu_solve_stats* st, fgpu_pmg* pmg) {
    const int64_t n = op->nnodes;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, ctx->stream);
    const CgOptions opt = cg_options(cfg);
    CgResult res;
    int rc = FGPU_OK, fail = 0, fallback = 0, fallback_its = 0;
    double rn = 0, bn = host_norm(ctx, n, d_b);
    double *r = nullptr, *q = nullptr, *xc = nullptr, *r2b = nullptr;
    if (cudaMalloc(&r, n * sizeof(double)) != cudaSuccess || cudaMalloc(&q, n * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&xc, n * sizeof(double)) != cudaSuccess || cudaMalloc(&r2b, n * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(r); cudaFree(q); cudaFree(xc);
        ctx->err = "matrix-free solve: allocation failed";
        return FGPU_ERR_ALLOC;
    }
    const int vb = vec_blocks(n);
    if (!cfg->mixed) {
        if (op->precision == FGPU_F32) { ctx->err = "the plain matrix-free solve needs a binary64 operator"; rc = FGPU_ERR_INVALID; }
        else {
            rc = mf_plain_solve(ctx, op, d_b, d_x, opt, cfg, bn, q, &res, pmg);
            fail = res.fail == 3 ? 2 : res.fail;
        }
    } else {
        if (!op32 || op32->precision != FGPU_F32 || op32->space != op->space) { ctx->err = "mixed matrix-free solve needs a binary32 inner operator on the same space"; rc = FGPU_ERR_INVALID; }
        float *r32 = nullptr, *d32 = nullptr;
        if (rc == FGPU_OK && (cudaMalloc(&r32, n * sizeof(float)) != cudaSuccess || cudaMalloc(&d32, n * sizeof(float)) != cudaSuccess)) {
            cudaGetLastError();
            ctx->err = "mixed matrix-free solve: allocation failed";
            rc = FGPU_ERR_ALLOC;
        }
        // reliable updates: the binary32 CG runs on the residual equation with
        // its own search direction; every delta reduction of its recurrence
        // residual (and at its claimed convergence) the correction is folded
        // into the binary64 solution, when that lowers the binary64 residual,
        // and the residual replaced by b - A64 x. A rejected fold, or two in a
        // row that do not halve the residual, end the binary32 phase.
        double* rbest = r;
        double* rcand = r2b;
        if (rc == FGPU_OK) rc = mf_residual64(ctx, op, d_b, d_x, rbest, q, &rn);
        if (rc == FGPU_OK && !(bn == 0.0 || rn <= cfg->rtol * bn)) {
            const double scale = rn;   // binary32 system scaled to a unit initial residual
            d2f_scaled_kernel<<<vb, 256, 0, ctx->stream>>>(n, rbest, r32, 1.0 / scale);
            cudaMemsetAsync(d32, 0, n * sizeof(float), ctx->stream);
            ctx->launches++;
            int stagnant = 0;
            auto fold = [&](float* xl, bool* accepted) -> int {
                cudaMemcpyAsync(xc, d_x, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream);
                fold_kernel<<<vb, 256, 0, ctx->stream>>>(n, xc, xl, scale);
                ctx->launches++;
                double rn_c = 0;
                const int r2 = mf_residual64(ctx, op, d_b, xc, rcand, q, &rn_c);
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
            CgOptions o32 = opt;
            o32.rtol = cfg->rtol * bn / rn;   // the binary32 system starts from a unit residual
            rc = mf_pcg_core<PolF32>(ctx, op32, r32, d32, o32, cfg->pc, &res, &refresh, pmg);
            if (rc == FGPU_OK && !res.true_conv) {
                bool ok = false;
                if (res.fail != 3) rc = fold(d32, &ok);
                if (rc == FGPU_OK && rn > cfg->rtol * bn) {
                    if (res.fail != 0 && res.iters < cfg->maxit) {
                        // binary32 breakdown or stagnation: finish with the binary64 operator from the best iterate
                        CgResult r64;
                        CgOptions o64 = opt;
                        o64.maxit = cfg->maxit - res.iters;
                        rc = mf_plain_solve(ctx, op, d_b, d_x, o64, cfg, bn, q, &r64, pmg);
                        fallback = 1;
                        fallback_its = r64.iters;
                        if (rc == FGPU_OK) rc = mf_residual64(ctx, op, d_b, d_x, rbest, q, &rn);
                        if (rc == FGPU_OK && r64.fail == 1) fail = 1;
                        else if (rc == FGPU_OK && rn > cfg->rtol * bn) fail = 2;
                    } else {
                        fail = res.fail == 1 ? 1 : 2;
                    }
                }
            }
        }
        cudaFree(r32);
        cudaFree(d32);
    }
    if (rc == FGPU_OK && !cfg->mixed) {
        rc = mf_residual64(ctx, op, d_b, d_x, r, q, &rn);
        if (rc == FGPU_OK && fail == 0 && rn > cfg->rtol * bn) fail = 2;
    }
    cudaFree(r);
    cudaFree(q);
    cudaFree(xc);
    cudaFree(r2b);
    cudaEventRecord(e1, ctx->stream);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != FGPU_OK) return rc;
    if (st) {
        st->iterations = res.iters + fallback_its;
        st->outer = cfg->mixed ? res.nrefresh : 1;
        st->rel_residual = bn > 0 ? rn / bn : 0.0;
        st->time_ms = ms;
        st->eig_max = res.lmax;
        st->fallback = fallback;
        st->fallback_iterations = fallback_its;
    }
    if (fail == 1) { ctx->err = "CG breakdown"; return FGPU_ERR_BREAKDOWN; }
    if (fail == 2) { ctx->err = "matrix-free CG did not reach rtol"; return FGPU_ERR_NOT_CONVERGED; }
    return FGPU_OK;
}

}  // namespace fgpu

// ===========================================================================
// C-ABI
// ===========================================================================
using namespace fgpu;

extern "C" int fgpu_operator_create(fgpu_ctx* ctx, fgpu_space* V, const fgpu_form_desc* f, int precision, fgpu_operator** out) {
    if (!ctx || !V || !f || !out) return FGPU_ERR_INVALID;
    if (f->kind != FGPU_FORM_LAPLACE_MASS || V->ncomp != 1) { ctx->err = "matrix-free operators support the scalar Laplace/mass form"; return FGPU_ERR_INVALID; }
    if (precision != FGPU_F32 && precision != FGPU_F64 && precision != FGPU_DF64) { ctx->err = "bad operator precision"; return FGPU_ERR_INVALID; }
    if (V->mesh->d_ho) { ctx->err = "matrix-free operators: affine elements only"; return FGPU_ERR_INVALID; }
    *out = nullptr;
    std::string err;
    DevTables* tab = get_dev_tables(V->order, f->quad_degree > 0 ? f->quad_degree : 2 * V->order, err);
    if (!tab) { ctx->err = err; return FGPU_ERR_INVALID; }
    fgpu_operator* op = new fgpu_operator();
    op->ctx = ctx;
    op->space = V;
    op->precision = precision;
    op->tab = tab;
    op->nt = V->mesh->nt;
    op->nnodes = V->topo.nnodes;
    // default element phase: the tensor cores for binary32 P3 (faster there: 0.64 against 0.79 ms at
    // 96^3), the CUDA cores for P2 (0.25 against 0.44 ms)
    op->use_tc = (precision == FGPU_F32 && V->n == 20 && V->ncomp == 1 && V->mesh->cv == 4) ? 1 : 0;
    double* dk = nullptr;
    auto fail = [&](int code, const char* msg) {
        ctx->err = msg;
        cudaFree(dk);
        fgpu_operator_destroy(op);
        return code;
    };
    if (f->kappa_elem) {
        if (cudaMalloc(&dk, op->nt * sizeof(double)) != cudaSuccess) return fail(FGPU_ERR_ALLOC, "operator: allocation failed");
        cudaMemcpyAsync(dk, f->kappa_elem, op->nt * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    }
    const size_t es = precision == FGPU_F32 ? sizeof(float) : sizeof(double);
    if (cudaMalloc(&op->d_rec, op->nt * 4 * sizeof(float4)) != cudaSuccess ||
        cudaMalloc(&op->d_ye, op->nt * V->n * es) != cudaSuccess)
        return fail(FGPU_ERR_ALLOC, "operator: allocation failed");
    int rc = launch_geometry_df(ctx, V->mesh, dk, f->kappa, f->mass, op->d_rec);
    if (!rc && precision == FGPU_F64) {
        if (cudaMalloc(&op->d_coef, op->nt * 8 * sizeof(double)) != cudaSuccess) return fail(FGPU_ERR_ALLOC, "operator: allocation failed");
        rc = launch_geometry(ctx, V->mesh, FGPU_FORM_LAPLACE_MASS, dk, f->kappa, f->mass, 0, 0, op->d_coef);
    }
    if (!rc) rc = operator_diagonal(ctx, op);
    cudaStreamSynchronize(ctx->stream);
    cudaFree(dk);
    dk = nullptr;
    if (rc) { fgpu_operator_destroy(op); return rc; }
    *out = op;
    return FGPU_OK;
}

extern "C" int fgpu_operator_set_dirichlet(fgpu_operator* op, int64_t ndofs, const int32_t* dofs) {
    if (!op || (ndofs > 0 && !dofs)) return FGPU_ERR_INVALID;
    fgpu_ctx* ctx = op->ctx;
    std::vector<uint8_t> m(op->nnodes, 0);
    for (int64_t k = 0; k < ndofs; ++k) {
        if (dofs[k] < 0 || dofs[k] >= op->nnodes) { ctx->err = "dirichlet dof out of range"; return FGPU_ERR_OUT_OF_RANGE; }
        m[dofs[k]] = 1;
    }
    if (!op->d_mask) FGPU_CUDA_CHECK(ctx, cudaMalloc(&op->d_mask, op->nnodes));
    if (op->precision == FGPU_F32 && !op->d_xm) FGPU_CUDA_CHECK(ctx, cudaMalloc(&op->d_xm, op->nnodes * sizeof(float)));
    FGPU_CUDA_CHECK(ctx, cudaMemcpyAsync(op->d_mask, m.data(), op->nnodes, cudaMemcpyHostToDevice, ctx->stream));
    int rc = operator_diagonal(ctx, op);
    if (rc) return rc;
    FGPU_CUDA_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
    return FGPU_OK;
}

extern "C" int fgpu_operator_apply(fgpu_ctx* ctx, fgpu_operator* op, const fgpu_vector* x, fgpu_vector* y) {
    if (!ctx || !op || !x || !y || x->n != op->nnodes || y->n != op->nnodes) return FGPU_ERR_INVALID;
    int rc;
    if (op->precision == FGPU_F32) {
        // the binary32 copies stay with the operator (no allocation per apply)
        if (!op->d_xf && (cudaMalloc(&op->d_xf, op->nnodes * 4) != cudaSuccess ||
                          cudaMalloc(&op->d_yf, op->nnodes * 4) != cudaSuccess)) {
            cudaFree(op->d_xf);
            op->d_xf = nullptr;
            ctx->err = "apply: allocation failed";
            return FGPU_ERR_ALLOC;
        }
        const int vb = vec_blocks(op->nnodes);
        copy_cast_kernel<float><<<vb, 256, 0, ctx->stream>>>(op->nnodes, x->d, op->d_xf);
        rc = operator_apply(ctx, op, op->d_xf, op->d_yf);
        cast_back_kernel<float><<<vb, 256, 0, ctx->stream>>>(op->nnodes, op->d_yf, y->d);
        ctx->launches += 2;
    } else {
        rc = operator_apply(ctx, op, x->d, y->d);
    }
    // completion and the device status word (bounded tensor-core waits report through it)
    int hst = 0;
    cudaError_t e = cudaMemcpyAsync(&hst, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (!rc && e != cudaSuccess) { ctx->err = cudaGetErrorString(e); rc = FGPU_ERR_CUDA; }
    if (e == cudaSuccess && hst) {
        cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream);
        cudaStreamSynchronize(ctx->stream);
        if (!rc) { ctx->err = "apply: device status " + std::to_string(hst); rc = FGPU_ERR_CUDA; }
    }
    return rc;
}

extern "C" int fgpu_operator_set_tensor_cores(fgpu_operator* op, int on) {
    if (!op) return FGPU_ERR_INVALID;
    if (on && (op->precision != FGPU_F32 || (op->space->n != 10 && op->space->n != 20))) {
        op->ctx->err = "tensor-core element phase: binary32 operators of P2 or P3 only";
        return FGPU_ERR_INVALID;
    }
    op->use_tc = on ? 1 : 0;
    op->tc_chosen = 1;
    return FGPU_OK;
}

extern "C" int fgpu_operator_set_algo(fgpu_operator* op, int algo) {
    if (!op) return FGPU_ERR_INVALID;
    fgpu_ctx* ctx = op->ctx;
    if (algo == FGPU_ALGO_GATHER || algo == FGPU_ALGO_AUTO) { op->algo = FGPU_ALGO_GATHER; return FGPU_OK; }
    if (algo != FGPU_ALGO_COLOUR) { ctx->err = "operator: algorithm must be GATHER or COLOUR"; return FGPU_ERR_INVALID; }
    if (op->precision == FGPU_F32 && op->use_tc && !op->tc_chosen) op->use_tc = 0;   // the P3 default gives way
    if (op->precision != FGPU_F32 || op->use_tc) { ctx->err = "colour scatter: binary32 CUDA-core operators only"; return FGPU_ERR_INVALID; }
    fgpu_mesh* M = op->space->mesh;
    if (!M->d_colour_perm) {
        std::vector<int32_t> perm;
        const int nc = colour_elements(M->nv, M->nt, M->h_tets.data(), perm, M->colour_ptr);
        if (nc < 0) { ctx->err = "colour scatter: more than 64 colours"; return FGPU_ERR_INVALID; }
        FGPU_CUDA_CHECK(ctx, cudaMalloc(&M->d_colour_perm, perm.size() * sizeof(int32_t)));
        FGPU_CUDA_CHECK(ctx, cudaMemcpy(M->d_colour_perm, perm.data(), perm.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
        M->ncolours = nc;
    }
    if (!op->d_xs) FGPU_CUDA_CHECK(ctx, cudaMalloc(&op->d_xs, op->nnodes * sizeof(float)));
    op->algo = FGPU_ALGO_COLOUR;
    return FGPU_OK;
}

extern "C" int fgpu_operator_destroy(fgpu_operator* op) {
    if (!op) return FGPU_OK;
    cudaFree(op->d_rec);
    cudaFree(op->d_coef);
    cudaFree(op->d_ye);
    cudaFree(op->d_mask);
    cudaFree(op->d_diag);
    cudaFree(op->d_xf);
    cudaFree(op->d_yf);
    cudaFree(op->d_xm);
    cudaFree(op->d_xs);
    delete op;
    return FGPU_OK;
}

extern "C" int fgpu_solve_cg_operator(fgpu_ctx* ctx, fgpu_operator* op, fgpu_operator* op32, const fgpu_vector* b, fgpu_vector* x,
                                      const fgpu_solver_cfg* cfg, fgpu_solve_stats* stats) {
    if (!ctx || !op || !b || !x || !cfg || b->n != op->nnodes || x->n != op->nnodes) return FGPU_ERR_INVALID;
    if (cfg->pc == FGPU_PC_PMG) { ctx->err = "solve_cg_operator: pc pmg runs through fgpu_solve_cg_operator_pmg"; return FGPU_ERR_INVALID; }
    int rc = solve_cg_operator(ctx, op, op32, b->d, x->d, cfg, stats, nullptr);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (!rc && e != cudaSuccess) { ctx->err = cudaGetErrorString(e); rc = FGPU_ERR_CUDA; }
    return rc;
}

extern "C" int fgpu_solve_cg_operator_pmg(fgpu_ctx* ctx, fgpu_operator* op, fgpu_operator* op32, fgpu_pmg* pmg, const fgpu_vector* b,
                                          fgpu_vector* x, const fgpu_solver_cfg* cfg, fgpu_solve_stats* stats) {
    if (!ctx || !op || !pmg || !b || !x || !cfg || b->n != op->nnodes || x->n != op->nnodes) return FGPU_ERR_INVALID;
    int rc = solve_cg_operator(ctx, op, op32, b->d, x->d, cfg, stats, pmg);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (!rc && e != cudaSuccess) { ctx->err = cudaGetErrorString(e); rc = FGPU_ERR_CUDA; }
    return rc;
}
