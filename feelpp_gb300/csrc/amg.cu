// Smoothed-aggregation AMG preconditioner on the device: the hierarchy is
// built on the host (amg_setup.cpp) from the assembled FP64 matrix, then
// every level lives in HBM in binary32 (values; the fine level reuses the
// matrix's own row pointers and column indices) and one V-cycle runs as a
// fixed sequence of kernels that the CG driver captures into its CUDA graph.
//
// V-cycle (PETSc PCMG multiplicative, one pre- and one post-smoothing; the
// reference's levels use Richardson/SOR, feelpp/feel/feelalg/backend.cpp:
// 836-845, which is sequential by nature; here the level smoother is the
// Chebyshev polynomial in D^-1 A on [0.1, 1.1] lmax, PETSc GAMG's own default,
// so the preconditioner stays a fixed symmetric linear operator):
//   x_l = S_l(b_l)                      pre-smoothing from zero
//   b_{l+1} = R_l (b_l - A_l x_l)       restriction of the residual
//   x_{l+1} = V(l+1)                    (coarsest: dense inverse, or smoothing)
//   x_l += P_l x_{l+1}                  prolongation
//   x_l += S_l(b_l - A_l x_l)           post-smoothing
// The CG iterations stay in the solver's arithmetic (FP64); only the
// preconditioner runs in binary32.
//
// Each level operator is stored in SELL-C-sigma form (32-row slices, rows
// sorted by length inside 256-row windows, entries column-major: one thread
// per row, coalesced loads) and applied by one kernel per sweep with the
// smoother/residual update fused into its epilogue; prolongators and
// restrictions stay in CSR with G lanes per row (G from the mean row length).
// Every row is summed in a fixed order, so a V-cycle is deterministic.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <string>
#include <vector>

#include "cg_driver.cuh"

struct fgpu_amg {
    fgpu_ctx* ctx = nullptr;
    const fgpu_matrix* A = nullptr;
    struct Level {
        int64_t n = 0, nnz = 0;
        float* dinv = nullptr;
        // the level operator in SELL-C-sigma form (C = 32, sigma = 256): one thread per row,
        // entries column-major inside each 32-row slice
        int64_t nslices = 0;
        int64_t* s_ptr = nullptr;
        int32_t* s_len = nullptr;
        int32_t* s_perm = nullptr;
        int32_t* s_col = nullptr;
        float* s_val = nullptr;
        int64_t* p_ia = nullptr;     // P_l: n x n_{l+1}
        int32_t* p_ja = nullptr;
        float* p_a = nullptr;
        int64_t p_nnz = 0;
        int pG = 4;
        int64_t* r_ia = nullptr;     // R_l = P_l^T: n_{l+1} x n
        int32_t* r_ja = nullptr;
        float* r_a = nullptr;
        int64_t r_nnz = 0;
        int rG = 8;
        float *x = nullptr, *b = nullptr, *w = nullptr, *d0 = nullptr, *d1 = nullptr, *e = nullptr;
        float inv_theta = 1.0f;
        std::vector<float> c1, c2;   // Chebyshev steps 1..K-1
        double lmax = 0;
    };
    std::vector<Level> L;
    float* coarse_inv = nullptr;     // dense inverse of the coarsest operator (or null: smoothing)
    int degree = 3;                  // Chebyshev degree of the level smoothers
    int coarse_degree = 12;          // coarsest-level smoothing degree without a dense inverse
    double setup_ms = 0;
    int device_levels = 0;           // levels whose set-up ran on the device
    fgpu::AmgSetupTimes times;       // set-up phases (device set-up; the host set-up reports tail and layout)
    int launches_per_cycle = 0;
    fgpu_amg_cfg cfg{};              // (its vector pointers cleared: the near null space is kept below)
    fgpu::AmgNns nns;                // near null space (m = 0: none)
    float* xacc = nullptr;           // repeated cycles (amg_vcycle_f32 with cycles > 1): accumulated solution
    float* tres = nullptr;           //                                                   and residual
};

namespace fgpu {

namespace {

enum AmgMode { kResid = 0, kResidStart = 1, kCheb = 2, kPlain = 3, kAdd = 4 };

struct AmgSweep {
    int64_t n = 0;
    const int64_t* ia = nullptr;
    const int32_t* ja = nullptr;
    const float* a = nullptr;
    const float* x = nullptr;        // SpMV input
    const float* b = nullptr;
    const float* dinv = nullptr;
    float* w = nullptr;
    const float* dprev = nullptr;
    float* dnew = nullptr;
    float* acc = nullptr;
    float* out = nullptr;            // kResid / kPlain / kAdd output; kCheb last step target (or null)
    float c1 = 0, c2 = 0, inv_theta = 1;
    int last = 0;
};

template <int MODE>
__device__ __forceinline__ void amg_epilogue(const AmgSweep& s, int64_t i, float acc) {
    if (MODE == kResid) {
        s.out[i] = s.b[i] - acc;
    } else if (MODE == kResidStart) {
        const float wi = s.b[i] - acc;
        const float d = s.dinv[i] * wi * s.inv_theta;
        s.w[i] = wi;
        s.dnew[i] = d;
        s.acc[i] = d;
    } else if (MODE == kCheb) {
        const float wi = s.w[i] - acc;
        const float dn = fmaf(s.c1, s.dprev[i], s.c2 * s.dinv[i] * wi);
        if (s.last && s.out) {
            s.out[i] += s.acc[i] + dn;
        } else {
            s.acc[i] += dn;
            if (!s.last) {
                s.w[i] = wi;
                s.dnew[i] = dn;
            }
        }
    } else if (MODE == kPlain) {
        s.out[i] = acc;
    } else {
        s.out[i] += acc;
    }
}

struct AmgSell {
    int64_t nslices = 0;
    const int64_t* ptr = nullptr;
    const int32_t* len = nullptr;
    const int32_t* perm = nullptr;
    const int32_t* col = nullptr;
    const float* val = nullptr;
};

// row i (in sorted order) of a SELL sweep: the entries of its slice column, four loads issued together
// (memory-level parallelism), summed in entry order, then the epilogue on the original row
template <int MODE>
__device__ __forceinline__ void sell_row(const AmgSweep& s, const AmgSell& m, int64_t i) {
    const int64_t sl = i >> 5;
    const int L = __ldg(m.len + sl);
    const int64_t base = __ldg(m.ptr + sl) + (i & 31);
    float acc = 0.0f;
    int k = 0;
    for (; k + 4 <= L; k += 4) {
        const int64_t j = base + (int64_t)k * 32;
        const int32_t c0 = __ldg(m.col + j), c1 = __ldg(m.col + j + 32), c2 = __ldg(m.col + j + 64), c3 = __ldg(m.col + j + 96);
        const float v0 = __ldg(m.val + j), v1 = __ldg(m.val + j + 32), v2 = __ldg(m.val + j + 64), v3 = __ldg(m.val + j + 96);
        const float x0 = __ldg(s.x + c0), x1 = __ldg(s.x + c1), x2 = __ldg(s.x + c2), x3 = __ldg(s.x + c3);
        acc = fmaf(v0, x0, acc);
        acc = fmaf(v1, x1, acc);
        acc = fmaf(v2, x2, acc);
        acc = fmaf(v3, x3, acc);
    }
    for (; k < L; ++k) {
        const int64_t j = base + (int64_t)k * 32;
        acc = fmaf(__ldg(m.val + j), __ldg(s.x + __ldg(m.col + j)), acc);
    }
    if (i < s.n) amg_epilogue<MODE>(s, __ldg(m.perm + i), acc);
}

// one sweep of a level operator in SELL form: thread per (sorted) row, then the epilogue on the
// original row; every lane of a warp belongs to one slice, so the entry loop is warp-uniform
template <int MODE>
__global__ void __launch_bounds__(128) amg_sell_kernel(AmgSweep s, AmgSell m, const int* __restrict__ stop) {
    if (stop && *stop) return;
    const int64_t total = m.nslices * 32;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
        sell_row<MODE>(s, m, i);
}

// the same sweep for levels with few rows: a block of W warps per slice, warp w summing the entries
// k = w, w + W, ... of the slice's 32 rows (coalesced like the one-thread-per-row kernel), the W
// partial sums of a row then added in warp order; a level of 25 K rows has ~800 slices, so the
// one-thread-per-row kernel would run 25 K threads through rows of ~60 dependent loads each
template <int MODE, int W>
__global__ void __launch_bounds__(32 * W) amg_sell_split_kernel(AmgSweep s, AmgSell m, const int* __restrict__ stop) {
    if (stop && *stop) return;
    __shared__ float part[W][32];
    const int r = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int64_t sl = blockIdx.x; sl < m.nslices; sl += gridDim.x) {
        const int L = __ldg(m.len + sl);
        const int64_t base = __ldg(m.ptr + sl) + r;
        float acc = 0.0f;
        for (int k = w; k < L; k += W) {
            const int64_t j = base + (int64_t)k * 32;
            acc = fmaf(__ldg(m.val + j), __ldg(s.x + __ldg(m.col + j)), acc);
        }
        part[w][r] = acc;
        __syncthreads();
        if (w == 0) {
            float t = part[0][r];
#pragma unroll
            for (int q = 1; q < W; ++q) t += part[q][r];
            const int64_t i = sl * 32 + r;
            if (i < s.n) amg_epilogue<MODE>(s, __ldg(m.perm + i), t);
        }
        __syncthreads();
    }
}

// one sweep of a CSR operator (the prolongators and restrictions): s_i = sum_j a_ij x_j with G lanes
// per row, then the mode's epilogue
template <int G, int MODE>
__global__ void __launch_bounds__(256) amg_sweep_kernel(AmgSweep s, const int* __restrict__ stop) {
    if (stop && *stop) return;
    const int lane = threadIdx.x & (G - 1);
    const int gw = (threadIdx.x & 31) / G;                 // group within the warp
    const int64_t groups = (int64_t)gridDim.x * (blockDim.x / G);
    // the loop condition is uniform over the warp (its first group's row), so
    // every lane reaches the full-warp shuffles; rows past n contribute nothing
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G; i - gw < s.n; i += groups) {
        const bool valid = i < s.n;
        const int64_t p0 = valid ? s.ia[i] : 0, p1 = valid ? s.ia[i + 1] : 0;
        float acc = 0.0f;
        for (int64_t p = p0 + lane; p < p1; p += G) acc = fmaf(__ldg(s.a + p), __ldg(s.x + __ldg(s.ja + p)), acc);
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, G);
        if (lane != 0 || !valid) continue;
        amg_epilogue<MODE>(s, i, acc);
    }
}

__device__ __forceinline__ float to_f32(double v) { return (float)v; }
__device__ __forceinline__ float to_f32(float2 v) { return v.x + v.y; }
__device__ __forceinline__ float to_f32(float v) { return v; }

// pre-smoothing start from zero: b = (float) r (fine level) or b as is; d0 = D^-1 b / theta; x = d0; w = b
template <typename T>
__global__ void amg_start_kernel(int64_t n, const T* __restrict__ bin, float* __restrict__ b, const float* __restrict__ dinv,
                                 float inv_theta, float* __restrict__ x, float* __restrict__ w, float* __restrict__ d0,
                                 const int* __restrict__ stop) {
    if (stop && *stop) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float bi = to_f32(bin[i]);
        if (b != (const float*)bin) b[i] = bi;
        const float d = dinv[i] * bi * inv_theta;
        x[i] = d;
        w[i] = bi;
        d0[i] = d;
    }
}

// coarsest level: x = Ainv b, one warp per row (fixed lane order)
__global__ void amg_dense_kernel(int64_t n, const float* __restrict__ M, const float* __restrict__ b, float* __restrict__ x,
                                 const int* __restrict__ stop) {
    if (stop && *stop) return;
    const int lane = threadIdx.x & 31;
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32; i < n; i += (int64_t)gridDim.x * blockDim.x / 32) {
        float acc = 0.0f;
        for (int64_t j = lane; j < n; j += 32) acc = fmaf(M[i * n + j], b[j], acc);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) x[i] = acc;
    }
}

// z = x0 in the solver's storage, per-block r.z partials (the layout of the CG kernels), p = z when asked
template <class PL>
__global__ void amg_finish_kernel(int64_t n, const float* __restrict__ x0, const typename PL::S* __restrict__ r,
                                  typename PL::S* __restrict__ z, typename PL::D* __restrict__ partial_rz,
                                  typename PL::S* __restrict__ p_out, const CGScalars<PL>* __restrict__ sc) {
    if (sc && sc->done) return;
    __shared__ typename PL::D sh[32];
    typename PL::D rz = PL::dzero();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        typename PL::A zi;
        if constexpr (PL::id == 1) zi = df{x0[i], 0.0f};
        else zi = (typename PL::A)x0[i];
        const typename PL::S zs = PL::st(zi);
        z[i] = zs;
        if (p_out) p_out[i] = zs;
        rz = PL::dmadd(rz, PL::ld(r[i]), PL::ld(zs));
    }
    const typename PL::D t = block_sum<PL>(rz, sh);
    if (threadIdx.x == 0) partial_rz[blockIdx.x] = t;
}

int lanes_for(int64_t n, int64_t nnz) {
    const double m = n > 0 ? (double)nnz / (double)n : 1.0;
    return m <= 6 ? 4 : m <= 12 ? 8 : m <= 24 ? 16 : 32;
}

// grid cap of the CSR sweeps (prolongators, restrictions); one thread group per row without a cap took
// 1.225 against 1.214 ms per P2 64^3 CG + AMG iteration
constexpr int64_t kAmgSweepCap = 152 * 16;
int grid_for(int64_t rows, int G) {
    const int64_t per = 256 / G;
    return (int)std::max<int64_t>(1, std::min<int64_t>((rows + per - 1) / per, kAmgSweepCap));
}

template <int MODE>
void sweep(cudaStream_t st, int G, const AmgSweep& s, const int* stop) {
    const int g = grid_for(s.n, G);
    switch (G) {
        case 4: amg_sweep_kernel<4, MODE><<<g, 256, 0, st>>>(s, stop); break;
        case 8: amg_sweep_kernel<8, MODE><<<g, 256, 0, st>>>(s, stop); break;
        case 16: amg_sweep_kernel<16, MODE><<<g, 256, 0, st>>>(s, stop); break;
        default: amg_sweep_kernel<32, MODE><<<g, 256, 0, st>>>(s, stop); break;
    }
}

// levels with fewer rows than this run the split-slice sweep (152 SMs x 1024 threads: the one-thread-
// per-row kernel would not fill the GPU once)
constexpr int64_t kSellSplitRows = 152 * 1024;

template <int MODE>
void sell_sweep(cudaStream_t st, const fgpu_amg::Level& V, const AmgSweep& s, const int* stop) {
    AmgSell m;
    m.nslices = V.nslices;
    m.ptr = V.s_ptr;
    m.len = V.s_len;
    m.perm = V.s_perm;
    m.col = V.s_col;
    m.val = V.s_val;
    if (V.nslices * 32 < kSellSplitRows) {
        // few rows: eight warps per slice (the rows are long on the coarse levels)
        amg_sell_split_kernel<MODE, 8><<<(int)std::max<int64_t>(1, V.nslices), 256, 0, st>>>(s, m, stop);
        return;
    }
    // one thread per slot, no grid-stride loop: slices differ in length, and many short-lived blocks
    // keep the SMs fuller than a few long-lived ones (measured: 46 % warps active with two waves). Blocks
    // of 128 threads (4 slices): CG + AMG iterations 1.21 / 6.45 ms at P2 / P3 64^3, against 1.28 / 6.86 ms
    // with 256 and 1.29 / 6.68 ms with 64; persistent warps taking four slices at a time from an atomic
    // counter: 1.35 / 6.93 ms
    const int g = (int)std::max<int64_t>(1, (V.nslices * 32 + 127) / 128);
    amg_sell_kernel<MODE><<<g, 128, 0, st>>>(s, m, stop);
}

int vblocks(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 8)); }

// Chebyshev steps 1..K-1 on level l accumulating into acc; the last step adds acc + d into target when set
int cheb_steps(cudaStream_t st, fgpu_amg::Level& V, int K, float* acc, float* target, const int* stop) {
    int nl = 0;
    for (int k = 1; k < K; ++k) {
        AmgSweep s;
        s.n = V.n;
        s.dprev = (k & 1) ? V.d0 : V.d1;
        s.dnew = (k & 1) ? V.d1 : V.d0;
        s.x = s.dprev;
        s.dinv = V.dinv;
        s.w = V.w;
        s.acc = acc;
        s.c1 = V.c1[k - 1];
        s.c2 = V.c2[k - 1];
        s.last = k == K - 1;
        s.out = s.last ? target : nullptr;
        sell_sweep<kCheb>(st, V, s, stop);
        ++nl;
    }
    return nl;
}

}  // namespace

// One V-cycle: level-0 right-hand side r (solver storage S), result in L[0].x.
template <typename T>
int amg_vcycle(fgpu_amg* M, const T* r, const int* stop) {
    cudaStream_t st = M->ctx->stream;
    const int nlev = (int)M->L.size();
    const int K = M->degree;
    int nl = 0;
    for (int l = 0; l < nlev; ++l) {
        fgpu_amg::Level& V = M->L[l];
        const bool coarsest = l == nlev - 1;
        if (coarsest && M->coarse_inv) {
            if (l == 0) {            // one-level hierarchy: the right-hand side still has to reach V.b
                amg_start_kernel<T><<<vblocks(V.n), 256, 0, st>>>(V.n, r, V.b, V.dinv, V.inv_theta, V.x, V.w, V.d0, stop);
                ++nl;
            }
            const int g = (int)std::max<int64_t>(1, std::min<int64_t>((V.n * 32 + 255) / 256, 152 * 8));
            amg_dense_kernel<<<g, 256, 0, st>>>(V.n, M->coarse_inv, V.b, V.x, stop);
            ++nl;
            break;
        }
        const int Kl = coarsest ? M->coarse_degree : K;
        if (l == 0) amg_start_kernel<T><<<vblocks(V.n), 256, 0, st>>>(V.n, r, V.b, V.dinv, V.inv_theta, V.x, V.w, V.d0, stop);
        else amg_start_kernel<float><<<vblocks(V.n), 256, 0, st>>>(V.n, V.b, V.b, V.dinv, V.inv_theta, V.x, V.w, V.d0, stop);
        ++nl;
        if (coarsest) {
            // Chebyshev coefficients of the coarsest level are sized for coarse_degree
            nl += cheb_steps(st, V, Kl, V.x, nullptr, stop);
            break;
        }
        nl += cheb_steps(st, V, Kl, V.x, nullptr, stop);
        AmgSweep s;
        s.n = V.n; s.x = V.x; s.b = V.b; s.out = V.w;
        sell_sweep<kResid>(st, V, s, stop);
        fgpu_amg::Level& C = M->L[l + 1];
        AmgSweep rs;
        rs.n = C.n; rs.ia = V.r_ia; rs.ja = V.r_ja; rs.a = V.r_a; rs.x = V.w; rs.out = C.b;
        sweep<kPlain>(st, V.rG, rs, stop);
        nl += 2;
    }
    for (int l = nlev - 2; l >= 0; --l) {
        fgpu_amg::Level& V = M->L[l];
        fgpu_amg::Level& C = M->L[l + 1];
        AmgSweep ps;
        ps.n = V.n; ps.ia = V.p_ia; ps.ja = V.p_ja; ps.a = V.p_a; ps.x = C.x; ps.out = V.x;
        sweep<kAdd>(st, V.pG, ps, stop);
        AmgSweep s;
        s.n = V.n; s.x = V.x; s.b = V.b; s.dinv = V.dinv; s.w = V.w; s.dnew = V.d0;
        s.acc = V.e; s.inv_theta = V.inv_theta;
        sell_sweep<kResidStart>(st, V, s, stop);
        nl += 2 + cheb_steps(st, V, M->degree, V.e, V.x, stop);
    }
    return nl;
}

template int amg_vcycle<double>(fgpu_amg*, const double*, const int*);

__global__ void amg_add_kernel(int64_t n, const float* __restrict__ a, float* __restrict__ acc, int first,
                               const int* __restrict__ stop) {
    if (stop && *stop) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        acc[i] = first ? a[i] : acc[i] + a[i];
}

// `cycles` V-cycles for A_0 x = r from x = 0 (each further cycle on the residual of the sum so far)
int amg_vcycle_f32(fgpu_amg* M, const float* r, const int* stop, const float** x, int cycles) {
    int nl = amg_vcycle<float>(M, r, stop);
    *x = M->L[0].x;
    if (cycles <= 1) return nl;
    fgpu_amg::Level& V = M->L[0];
    cudaStream_t st = M->ctx->stream;
    if (!M->xacc) {
        if (cudaMalloc(&M->xacc, V.n * sizeof(float)) != cudaSuccess || cudaMalloc(&M->tres, V.n * sizeof(float)) != cudaSuccess) {
            cudaGetLastError();
            return nl;                // no room: one cycle
        }
    }
    amg_add_kernel<<<vblocks(V.n), 256, 0, st>>>(V.n, V.x, M->xacc, 1, stop);
    ++nl;
    for (int c = 1; c < cycles; ++c) {
        AmgSweep s;
        s.n = V.n; s.x = M->xacc; s.b = r; s.out = M->tres;
        if (M->L.size() > 1 || !M->coarse_inv) sell_sweep<kResid>(st, V, s, stop);
        else return nl;               // one dense level: the first cycle was already exact
        nl += 1 + amg_vcycle<float>(M, M->tres, stop);
        amg_add_kernel<<<vblocks(V.n), 256, 0, st>>>(V.n, V.x, M->xacc, 0, stop);
        ++nl;
    }
    *x = M->xacc;
    return nl;
}

int64_t amg_rows(const fgpu_amg* M) { return M->L.empty() ? 0 : M->L[0].n; }
const fgpu_ctx* amg_context(const fgpu_amg* M) { return M->ctx; }
template int amg_vcycle<float2>(fgpu_amg*, const float2*, const int*);
template int amg_vcycle<float>(fgpu_amg*, const float*, const int*);

// PcHook for the CG driver: z = V(r), r.z partials, optional p = z
template <class PL>
PcHook<PL> amg_pc_hook(fgpu_amg* M) {
    PcHook<PL> h;
    h.apply = [M](const typename PL::S* r, typename PL::S* z, typename PL::D* partial_rz, typename PL::S* p_out,
                  const CGScalars<PL>* gate) {
        const int* stop = gate ? &gate->done : nullptr;
        int nl = amg_vcycle<typename PL::S>(M, r, stop);
        amg_finish_kernel<PL><<<vec_blocks(M->L[0].n), kVecThreads, 0, M->ctx->stream>>>(M->L[0].n, M->L[0].x, r, z, partial_rz, p_out,
                                                                                        gate);
        M->ctx->launches += nl + 1;
    };
    h.launches = M->launches_per_cycle + 1;
    return h;
}

template PcHook<PolF64> amg_pc_hook<PolF64>(fgpu_amg*);
template PcHook<PolDF64> amg_pc_hook<PolDF64>(fgpu_amg*);
template PcHook<PolF32> amg_pc_hook<PolF32>(fgpu_amg*);

namespace {

void free_level(fgpu_amg::Level& V) {
    cudaFree(V.dinv);
    cudaFree(V.s_ptr); cudaFree(V.s_len); cudaFree(V.s_perm); cudaFree(V.s_col); cudaFree(V.s_val);
    cudaFree(V.p_ia); cudaFree(V.p_ja); cudaFree(V.p_a); cudaFree(V.r_ia); cudaFree(V.r_ja); cudaFree(V.r_a);
    cudaFree(V.x); cudaFree(V.b); cudaFree(V.w); cudaFree(V.d0); cudaFree(V.d1); cudaFree(V.e);
    V = fgpu_amg::Level();
}

void cheb_coefs(fgpu_amg::Level& V, int K) {
    // [0.05, 1.1] lmax (PETSc's GAMG Chebyshev default is [0.1, 1.1]): CG + AMG to 1e-10 at P3 64^3 in
    // 64 iterations against 68 (0.2: 77); P2 64^3 36 in both
    const double emax = 1.1 * V.lmax, emin = 0.05 * V.lmax;
    const double theta = 0.5 * (emax + emin), delta = 0.5 * (emax - emin), sigma = theta / delta;
    double rho = 1.0 / sigma;
    V.inv_theta = (float)(1.0 / theta);
    V.c1.clear();
    V.c2.clear();
    for (int k = 1; k < K; ++k) {
        const double rn = 1.0 / (2.0 * sigma - rho);
        V.c1.push_back((float)(rn * rho));
        V.c2.push_back((float)(2.0 * rn / delta));
        rho = rn;
    }
}

template <typename T>
cudaError_t upload(T** dst, const T* src, size_t n) {
    cudaError_t e = cudaMalloc(dst, std::max<size_t>(n, 1) * sizeof(T));
    if (e == cudaSuccess && n) e = cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice);
    return e;
}

// SELL-C-sigma of a host CSR: rows sorted by length (descending, ties by row) inside windows
// of 256 rows, slices of 32 rows padded to their longest row (padding: column = the row, value 0)
cudaError_t upload_sell(fgpu_amg::Level& V, const HostCsr& A) {
    constexpr int kC = 32, kSigma = 256;
    const int64_t n = A.nrows;
    V.nslices = (n + kC - 1) / kC;
    std::vector<int32_t> perm(n), len(V.nslices, 0);
    for (int64_t w0 = 0; w0 < n; w0 += kSigma) {
        const int64_t w1 = std::min<int64_t>(n, w0 + kSigma);
        for (int64_t r = w0; r < w1; ++r) perm[r] = (int32_t)r;
        std::sort(perm.begin() + w0, perm.begin() + w1, [&](int32_t a, int32_t b) {
            const int64_t la = A.ia[a + 1] - A.ia[a], lb = A.ia[b + 1] - A.ia[b];
            return la != lb ? la > lb : a < b;
        });
    }
    std::vector<int64_t> ptr(V.nslices + 1, 0);
    for (int64_t sl = 0; sl < V.nslices; ++sl) {
        int64_t L = 0;
        for (int64_t i = sl * kC; i < std::min<int64_t>(n, (sl + 1) * kC); ++i) L = std::max<int64_t>(L, A.ia[perm[i] + 1] - A.ia[perm[i]]);
        len[sl] = (int32_t)L;
        ptr[sl + 1] = ptr[sl] + L * kC;
    }
    std::vector<int32_t> col(ptr[V.nslices]);
    std::vector<float> val(ptr[V.nslices]);
    for (int64_t i = 0; i < V.nslices * kC; ++i) {
        const int64_t sl = i / kC;
        const int64_t base = ptr[sl] + (i - sl * kC);
        const int32_t row = i < n ? perm[i] : -1;
        const int64_t b = row >= 0 ? A.ia[row] : 0, e = row >= 0 ? A.ia[row + 1] : 0;
        for (int64_t k = 0; k < len[sl]; ++k) {
            const int64_t p = b + k;
            const bool real = p < e;
            col[base + k * kC] = real ? A.ja[p] : (row >= 0 ? row : 0);
            val[base + k * kC] = real ? (float)A.a[p] : 0.0f;
        }
    }
    cudaError_t e = upload(&V.s_ptr, ptr.data(), ptr.size());
    if (e == cudaSuccess) e = upload(&V.s_len, len.data(), len.size());
    if (e == cudaSuccess) e = upload(&V.s_perm, perm.data(), perm.size());
    if (e == cudaSuccess) e = upload(&V.s_col, col.data(), col.size());
    if (e == cudaSuccess) e = upload(&V.s_val, val.data(), val.size());
    return e;
}

// level 0 from the device matrix: binary32 SELL values through the layout's CSR positions, and
// binary32 1 / a_ii (the same roundings as the host path: (float)a, (float)(1.0 / a))
__global__ void amg_sell_values_kernel(int64_t nstored, const int32_t* __restrict__ src, const double* __restrict__ csr,
                                       float* __restrict__ out) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nstored; j += (int64_t)gridDim.x * blockDim.x)
        out[j] = src[j] >= 0 ? (float)csr[src[j]] : 0.0f;
}

__global__ void amg_dinv_kernel(int64_t n, const int64_t* __restrict__ ia, const int32_t* __restrict__ ja,
                                const double* __restrict__ val, float* __restrict__ dinv) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        int64_t lo = ia[r], hi = ia[r + 1];
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (ja[mid] < r) lo = mid + 1; else hi = mid;
        }
        dinv[r] = (lo < ia[r + 1] && ja[lo] == r) ? (float)(1.0 / val[lo]) : 0.0f;
    }
}

// the fine level's SELL operator and diagonal built on the device from A (the host path's layout:
// C = 32, sigma = 256, rows sorted by length descending then index, padding columns = the row)
int upload_level0_device(fgpu_ctx* ctx, const fgpu_matrix* A, fgpu_amg::Level& V) {
    std::shared_ptr<SellLayout> L;
    int rc = build_sell(ctx, A, L);
    if (rc) return rc;
    V.nslices = L->nslices;
    V.s_ptr = L->d_slice_ptr; L->d_slice_ptr = nullptr;
    V.s_len = L->d_slice_len; L->d_slice_len = nullptr;
    V.s_perm = L->d_perm; L->d_perm = nullptr;
    V.s_col = L->d_col; L->d_col = nullptr;
    FGPU_CUDA_CHECK(ctx, cudaMalloc(&V.s_val, std::max<int64_t>(L->nstored, 1) * sizeof(float)));
    FGPU_CUDA_CHECK(ctx, cudaMalloc(&V.dinv, std::max<int64_t>(V.n, 1) * sizeof(float)));
    const int g = (int)std::max<int64_t>(1, std::min<int64_t>((L->nstored + 255) / 256, 152 * 32));
    amg_sell_values_kernel<<<g, 256, 0, ctx->stream>>>(L->nstored, L->d_src, (const double*)A->d_val, V.s_val);
    const int gd = (int)std::max<int64_t>(1, std::min<int64_t>((V.n + 255) / 256, 152 * 16));
    amg_dinv_kernel<<<gd, 256, 0, ctx->stream>>>(V.n, A->d_ia, A->d_ja, (const double*)A->d_val, V.dinv);
    ctx->launches += 2;
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    FGPU_CUDA_CHECK(ctx, cudaStreamSynchronize(ctx->stream));   // the layout's d_src is freed on return
    return FGPU_OK;
}

cudaError_t upload_f32(float** dst, const std::vector<double>& v) {
    std::vector<float> f(v.size());
    for (size_t i = 0; i < v.size(); ++i) f[i] = (float)v[i];
    return upload(dst, f.data(), f.size());
}

}  // namespace

// binary32 copy of device FP64 values
static __global__ void amg_f32_kernel(int64_t n, const double* __restrict__ a, float* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) out[i] = (float)a[i];
}

// prolongator / restriction of a device-built level: the CSR index arrays are taken over, the values
// rounded to binary32 (the host path's (float)a)
static int take_transfer(fgpu_ctx* ctx, AmgDevCsr& D, int64_t** ia, int32_t** ja, float** a) {
    FGPU_CUDA_CHECK(ctx, cudaMalloc(a, std::max<int64_t>(D.nnz, 1) * sizeof(float)));
    const int g = (int)std::max<int64_t>(1, std::min<int64_t>((D.nnz + 255) / 256, 152 * 16));
    amg_f32_kernel<<<g, 256, 0, ctx->stream>>>(D.nnz, D.a, *a);
    ctx->launches++;
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    *ia = D.ia;
    *ja = D.ja;
    D.ia = nullptr;
    D.ja = nullptr;
    return FGPU_OK;
}

int amg_setup(fgpu_ctx* ctx, const fgpu_matrix* A, const fgpu_amg_cfg* cfg, fgpu_amg* M) {
    const auto t0 = std::chrono::steady_clock::now();
    const int64_t n = A->nrows, nnz = A->nnz;
    if (cfg && cfg->smoother_degree >= 2) M->degree = cfg->smoother_degree;
    const AmgHostCfg hc = amg_host_cfg(cfg, ctx->host_threads);
    // levels 0 .. ndev-1 built on the device (D), the rest on the host (H)
    AmgDevHierarchy D;
    AmgHierarchy& H = D.tail;
    const AmgNns* nns = M->nns.m > 0 ? &M->nns : nullptr;
    if (!cfg || !cfg->setup_on_host) {
        const int rc = amg_build_device(ctx, A, hc, D, nns);
        if (rc) return rc;
    } else {
        HostCsr H0;
        H0.nrows = H0.ncols = n;
        H0.ia.resize(n + 1);
        H0.ja.resize(nnz);
        H0.a.resize(nnz);
        FGPU_CUDA_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
        FGPU_CUDA_CHECK(ctx, cudaMemcpy(H0.ia.data(), A->d_ia, (n + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost));
        FGPU_CUDA_CHECK(ctx, cudaMemcpy(H0.ja.data(), A->d_ja, nnz * sizeof(int32_t), cudaMemcpyDeviceToHost));
        FGPU_CUDA_CHECK(ctx, cudaMemcpy(H0.a.data(), A->d_val, nnz * sizeof(double), cudaMemcpyDeviceToHost));
        std::string err;
        if (!amg_build_host(std::move(H0), hc, H, err, nns)) { ctx->err = err; return FGPU_ERR_INVALID; }
    }
    const auto t_layout = std::chrono::steady_clock::now();
    const int ndev = (int)D.levels.size();
    const int nlev = ndev + (int)H.levels.size();
    M->L.assign(nlev, fgpu_amg::Level());
    int nl = 0;
    for (int l = 0; l < nlev; ++l) {
        fgpu_amg::Level& V = M->L[l];
        const bool coarsest = l == nlev - 1;
        const bool dev = l < ndev;
        AmgHostLevel* hl = dev ? nullptr : &H.levels[l - ndev];
        V.n = dev ? D.levels[l].A.nrows : hl->A.nrows;
        V.nnz = dev ? D.levels[l].A.nnz : (int64_t)hl->A.ja.size();
        V.lmax = dev ? D.levels[l].lmax : hl->lmax;
        cheb_coefs(V, coarsest ? M->coarse_degree : M->degree);
        if (l == 0 && A->nnz < ((int64_t)1 << 31)) {
            const int rc0 = upload_level0_device(ctx, A, V);
            if (rc0) return rc0;
        } else if (dev && V.nnz < ((int64_t)1 << 31)) {
            fgpu_matrix view;                       // the level operator's device arrays (not owned)
            view.ctx = ctx;
            view.nrows = V.n;
            view.nnz = V.nnz;
            view.d_ia = D.levels[l].A.ia;
            view.d_ja = D.levels[l].A.ja;
            view.d_val = D.levels[l].A.a;
            const int rc0 = upload_level0_device(ctx, &view, V);
            if (rc0) return rc0;
        } else {
            HostCsr copy;
            if (dev) {
                const int rc0 = amg_copy_to_host(ctx, D.levels[l].A, copy);
                if (rc0) return rc0;
            }
            const HostCsr& HA = dev ? copy : hl->A;
            std::vector<double> dinv(V.n, 0.0);
            for (int64_t i = 0; i < V.n; ++i)
                for (int64_t p = HA.ia[i]; p < HA.ia[i + 1]; ++p)
                    if (HA.ja[p] == i) dinv[i] = 1.0 / HA.a[p];
            FGPU_CUDA_CHECK(ctx, upload_f32(&V.dinv, dinv));
            FGPU_CUDA_CHECK(ctx, upload_sell(V, HA));
        }
        if (!coarsest && dev) {
            AmgDevLevel& dl = D.levels[l];
            V.p_nnz = dl.P.nnz;
            V.r_nnz = dl.R.nnz;
            V.pG = lanes_for(dl.P.nrows, V.p_nnz);
            V.rG = lanes_for(dl.R.nrows, V.r_nnz);
            int rc0 = take_transfer(ctx, dl.P, &V.p_ia, &V.p_ja, &V.p_a);
            if (!rc0) rc0 = take_transfer(ctx, dl.R, &V.r_ia, &V.r_ja, &V.r_a);
            if (rc0) return rc0;
        } else if (!coarsest) {
            V.p_nnz = (int64_t)hl->P.ja.size();
            V.r_nnz = (int64_t)hl->R.ja.size();
            V.pG = lanes_for(hl->P.nrows, V.p_nnz);
            V.rG = lanes_for(hl->R.nrows, V.r_nnz);
            FGPU_CUDA_CHECK(ctx, upload(&V.p_ia, hl->P.ia.data(), hl->P.ia.size()));
            FGPU_CUDA_CHECK(ctx, upload(&V.p_ja, hl->P.ja.data(), hl->P.ja.size()));
            FGPU_CUDA_CHECK(ctx, upload_f32(&V.p_a, hl->P.a));
            FGPU_CUDA_CHECK(ctx, upload(&V.r_ia, hl->R.ia.data(), hl->R.ia.size()));
            FGPU_CUDA_CHECK(ctx, upload(&V.r_ja, hl->R.ja.data(), hl->R.ja.size()));
            FGPU_CUDA_CHECK(ctx, upload_f32(&V.r_a, hl->R.a));
        }
        float** vecs[6] = {&V.x, &V.b, &V.w, &V.d0, &V.d1, &V.e};
        for (float** v : vecs) FGPU_CUDA_CHECK(ctx, cudaMalloc(v, std::max<int64_t>(V.n, 1) * sizeof(float)));
        if (coarsest && !H.coarse_inv.empty()) {
            FGPU_CUDA_CHECK(ctx, upload_f32(&M->coarse_inv, H.coarse_inv));
            nl += l == 0 ? 2 : 1;
        } else if (coarsest) {
            nl += M->coarse_degree;               // start + coarse_degree - 1 steps
        } else {
            nl += 1 + (M->degree - 1) + 2 + 2 + (M->degree - 1) + 0;   // start, steps, resid, restrict | prolong, resid-start, steps
        }
    }
    M->launches_per_cycle = nl;
    FGPU_CUDA_CHECK(ctx, cudaStreamSynchronize(ctx->stream));   // the device levels' FP64 values are freed on return
    M->device_levels = ndev;
    M->setup_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    M->times = D.times;
    M->times.layout = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_layout).count();
    if (cfg && cfg->setup_on_host) M->times.tail = M->setup_ms - M->times.layout;
    M->times.total = M->setup_ms;
    return FGPU_OK;
}

}  // namespace fgpu

using namespace fgpu;

extern "C" int fgpu_amg_create(fgpu_ctx* ctx, const fgpu_matrix* A, const fgpu_amg_cfg* cfg, fgpu_amg** out) {
    if (!ctx || !A || !out) return FGPU_ERR_INVALID;
    if (ctx->capturing) { ctx->err = "gamg: set-up is not capturable"; return FGPU_ERR_INVALID; }
    if (A->precision != FGPU_F64) { ctx->err = "gamg: FP64 matrices only"; return FGPU_ERR_INVALID; }
    *out = nullptr;
    fgpu_amg* M = new fgpu_amg();
    M->ctx = ctx;
    M->A = A;
    if (cfg) M->cfg = *cfg;
    bool has_nns = false;
    int rc = amg_nns_from_cfg(ctx, cfg, A->nrows, M->nns, &has_nns);
    if (rc) {
        delete M;
        return rc;
    }
    M->cfg.nns = nullptr;
    M->cfg.nns_host = nullptr;
    rc = amg_setup(ctx, A, &M->cfg, M);
    if (rc) {
        for (auto& V : M->L) free_level(V);
        cudaFree(M->coarse_inv);
        delete M;
        return rc;
    }
    *out = M;
    return FGPU_OK;
}

extern "C" int fgpu_amg_update(fgpu_amg* M) {
    if (!M) return FGPU_ERR_INVALID;
    fgpu_ctx* ctx = M->ctx;
    if (ctx->capturing) { ctx->err = "gamg: set-up is not capturable"; return FGPU_ERR_INVALID; }
    for (auto& V : M->L) free_level(V);
    cudaFree(M->coarse_inv);
    M->coarse_inv = nullptr;
    return amg_setup(ctx, M->A, &M->cfg, M);
}

extern "C" int fgpu_amg_info(const fgpu_amg* M, int* nlevels, int64_t* rows, int64_t* nnz, double* setup_ms) {
    if (!M) return FGPU_ERR_INVALID;
    if (nlevels) *nlevels = (int)M->L.size();
    for (size_t l = 0; l < M->L.size() && l < 16; ++l) {
        if (rows) rows[l] = M->L[l].n;
        if (nnz) nnz[l] = M->L[l].nnz;
    }
    if (setup_ms) *setup_ms = M->setup_ms;
    return FGPU_OK;
}

extern "C" int fgpu_amg_setup_info(const fgpu_amg* M, int* device_levels, double* phases_ms) {
    if (!M) return FGPU_ERR_INVALID;
    if (device_levels) *device_levels = M->device_levels;
    if (phases_ms) {
        const AmgSetupTimes& t = M->times;
        const double v[9] = {t.graph, t.aggregate, t.lanczos, t.prolong, t.galerkin, t.tail, t.layout, t.total, (double)t.handoff};
        for (int k = 0; k < 9; ++k) phases_ms[k] = v[k];
    }
    return FGPU_OK;
}

extern "C" int fgpu_amg_destroy(fgpu_amg* M) {
    if (!M) return FGPU_OK;
    for (auto& V : M->L) free_level(V);
    cudaFree(M->coarse_inv);
    cudaFree(M->xacc);
    cudaFree(M->tres);
    delete M;
    return FGPU_OK;
}
