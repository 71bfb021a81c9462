// Device set-up of the smoothed-aggregation hierarchy (the default of fgpu_amg_create).
//
// The construction of the host set-up (amg_setup.cpp: Vanek, Mandel, Brezina 1996; PETSc PCGAMG "agg"
// options of the reference, feelpp/feel/feelalg/preconditionerpetsc.cpp:2229-2330), every step on the
// device (but the QR of a near null space's aggregates), and every floating-point result formed in the
// host set-up's order with the same roundings, so that the device levels equal the host levels bit for bit:
//   * diagonal and strength graph: a row kernel marks |a_ij| > theta sqrt(|a_ii a_jj|) (j != i,
//     a_ij != 0); its transpose is built by counting, a scan and a fill, each row sorted, and the two
//     sorted lists merged per row (the symmetrised graph);
//   * aggregation: the host set-up's rounds of a distance-2 independent set (roots), then roots'
//     neighbours, then the rest by their first aggregated neighbour, each step a kernel over the nodes;
//   * lambda_max(D^-1 A): 12 Lanczos steps on D^-1/2 A D^-1/2 from the host set-up's start vector, the
//     products one thread per row in column order, the dot products as sequential sums over chunks of
//     1024 rows combined in chunk order (the host's partition), the tridiagonal's largest eigenvalue
//     by the host's Sturm bisection;
//   * P0(i, agg(i)) = 1/sqrt(|agg|), A P0, and P = P0 - omega D^-1 (A P0) merged row by row;
//   * R = P^T by counting, a scan, a fill and a per-row sort;
//   * sparse products A P0, A P and R (A P): one warp per row of the left factor. The row's products
//     are enumerated in (left column, right column) order 32 at a time; lanes holding the same output
//     column form a group whose lowest lane inserts the column into a shared-memory hash table and adds
//     the group's products to its running sum one by one in lane order, so every output entry is the
//     host's sequential sum. Rows with more distinct columns than the small table holds are listed and
//     redone with a larger table; the row is then sorted by column in shared memory (bitonic sort of
//     the table's slot list) and written out.
// Levels of at most 2048 rows, and any level with a row beyond the kernels' staging capacity, go to
// the host set-up for the rest of the hierarchy (the results are the same either way).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "fgpu_core.h"
#include "scan.cuh"

namespace fgpu {

AmgDevCsr::AmgDevCsr(AmgDevCsr&& o) noexcept { *this = std::move(o); }
AmgDevCsr& AmgDevCsr::operator=(AmgDevCsr&& o) noexcept {
    if (this != &o) {
        std::swap(nrows, o.nrows); std::swap(ncols, o.ncols); std::swap(nnz, o.nnz);
        std::swap(ia, o.ia); std::swap(ja, o.ja); std::swap(a, o.a); std::swap(own, o.own);
    }
    return *this;
}
AmgDevCsr::~AmgDevCsr() {
    if (own) { cudaFree(ia); cudaFree(ja); cudaFree(a); }
}

namespace {

constexpr int kStOverflow = 1;               // a row beyond a kernel's staging capacity
constexpr int kStDiag = 2;                   // a non-positive diagonal entry
constexpr int64_t kLanczosChunk = 1024;      // rows per partial sum (the host set-up's partition)
constexpr int kLanczosSteps = 12;
constexpr int64_t kHandoffRows = 2048;       // levels this small continue on the host (P2 48^3: an 11 K-row
                                              // level 1 built on the host took 21 ms of a 50 ms set-up, 1 ms on the device)
constexpr int kSortMax = 16384;              // longest row sorted by seg_sort_kernel
constexpr int kNumBins = 4;
constexpr int kBins[kNumBins] = {256, 1024, 2048, 8192};  // hash table sizes (at most half full)
constexpr int kBinLog[kNumBins] = {8, 10, 11, 13};

int grid_rows(int64_t n, int per_block, int cap = 152 * 16) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + per_block - 1) / per_block, cap));
}

struct Work {                                // device scratch freed at scope exit
    std::vector<void*> ptrs;
    Work() = default;
    Work(const Work&) = delete;
    Work& operator=(const Work&) = delete;
    ~Work() { for (void* p : ptrs) cudaFree(p); }
    template <typename T>
    T* get(int64_t n) {
        void* p = nullptr;
        if (cudaMalloc(&p, std::max<int64_t>(n, 1) * sizeof(T)) != cudaSuccess) { cudaGetLastError(); return nullptr; }
        ptrs.push_back(p);
        return static_cast<T*>(p);
    }
};

#define DEV_TRY(call)                                                                                         \
    do {                                                                                                      \
        const cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess) { ctx->err = std::string("gamg device set-up: ") + cudaGetErrorString(e_); return FGPU_ERR_CUDA; } \
    } while (0)
#define DEV_ALLOC(ok)                                                                                         \
    do {                                                                                                      \
        if (!(ok)) { ctx->err = "gamg device set-up: device allocation failed"; return FGPU_ERR_ALLOC; }    \
    } while (0)

int alloc_csr(fgpu_ctx* ctx, AmgDevCsr& C, int64_t nrows, int64_t ncols, int64_t nnz) {
    C = AmgDevCsr();
    C.nrows = nrows;
    C.ncols = ncols;
    C.nnz = nnz;
    DEV_TRY(cudaMalloc(&C.ia, (nrows + 1) * sizeof(int64_t)));
    DEV_TRY(cudaMalloc(&C.ja, std::max<int64_t>(nnz, 1) * sizeof(int32_t)));
    DEV_TRY(cudaMalloc(&C.a, std::max<int64_t>(nnz, 1) * sizeof(double)));
    return FGPU_OK;
}

int read_status(fgpu_ctx* ctx, const int* d_status, int* h) {
    DEV_TRY(cudaMemcpyAsync(h, d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    DEV_TRY(cudaStreamSynchronize(ctx->stream));
    return FGPU_OK;
}

// ---------------------------------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------------------------------

// diagonal (the last stored (i, i) entry, as the host's `diagonal`); flags a non-positive one
__global__ void diag_kernel(int64_t n, const int64_t* __restrict__ ia, const int32_t* __restrict__ ja, const double* __restrict__ a,
                            double* __restrict__ d, int* __restrict__ status) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double v = 0.0;
        for (int64_t p = ia[i]; p < ia[i + 1]; ++p)
            if (ja[p] == i) v = a[p];
        d[i] = v;
        if (!(v > 0.0)) atomicOr(status, kStDiag);
    }
}

// strong couplings of each row: counts (out == nullptr) or columns in row order at off[i]
__global__ void strong_kernel(int64_t n, const int64_t* __restrict__ ia, const int32_t* __restrict__ ja, const double* __restrict__ a,
                              const double* __restrict__ d, double theta, uint32_t* __restrict__ cnt, const uint32_t* __restrict__ off,
                              int32_t* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint32_t k = 0;
        for (int64_t p = ia[i]; p < ia[i + 1]; ++p) {
            const int32_t j = ja[p];
            const double v = a[p];
            if (j == i || v == 0.0) continue;
            // theta = 0 (the default): every nonzero coupling is strong (0 * sqrt of the positive, finite
            // diagonal product is 0), without the diagonal loads and the square root
            if (theta == 0.0 || fabs(v) > theta * sqrt(fabs(__dmul_rn(d[i], d[j])))) {
                if (out) out[off[i] + k] = j;
                ++k;
            }
        }
        if (cnt) cnt[i] = k;
    }
}

// column counts of a list of column indices
__global__ void col_count_kernel(int64_t nnz, const int32_t* __restrict__ col, uint32_t* __restrict__ cnt) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nnz; q += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(cnt + col[q], 1u);
}

// transpose fill: entry (i, col[q]) goes to row col[q] of the transpose (positions by cursors; the
// rows are sorted afterwards). Row pointers of the source in 32-bit (off32) or 64-bit (off64) form.
__global__ void transpose_fill_kernel(int64_t n, const uint32_t* __restrict__ off32, const int64_t* __restrict__ off64,
                                      const int32_t* __restrict__ col, const double* __restrict__ val, uint32_t* __restrict__ cursor,
                                      int32_t* __restrict__ oj, double* __restrict__ oa) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = off64 ? off64[i] : off32[i], e = off64 ? off64[i + 1] : off32[i + 1];
        for (int64_t q = b; q < e; ++q) {
            const uint32_t t = atomicAdd(cursor + col[q], 1u);
            oj[t] = (int32_t)i;
            if (val) oa[t] = val[q];
        }
    }
}

// each row's keys (and values) sorted by key: one warp per row, bitonic sort in shared memory (cap
// entries per warp)
__global__ void __launch_bounds__(128) seg_sort_kernel(int64_t n, const uint32_t* __restrict__ off32, const int64_t* __restrict__ off64,
                                                       int cap, int32_t* __restrict__ key, double* __restrict__ val,
                                                       int* __restrict__ status) {
    extern __shared__ __align__(16) unsigned char ss_smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, warps = blockDim.x >> 5;
    double* sv = reinterpret_cast<double*>(ss_smem) + (size_t)warp * cap;
    int32_t* sk = reinterpret_cast<int32_t*>(ss_smem + (val ? (size_t)warps * cap * 8 : 0)) + (size_t)warp * cap;
    for (int64_t r = (int64_t)blockIdx.x * warps + warp; r < n; r += (int64_t)gridDim.x * warps) {
        const int64_t b = off64 ? off64[r] : off32[r], e = off64 ? off64[r + 1] : off32[r + 1];
        const int len = (int)(e - b);
        if (len <= 1) continue;
        if (len > cap) {
            if (lane == 0) atomicOr(status, kStOverflow);
            continue;
        }
        int P = 1;
        while (P < len) P <<= 1;
        for (int k = lane; k < P; k += 32) {
            sk[k] = k < len ? key[b + k] : INT32_MAX;
            if (val) sv[k] = k < len ? val[b + k] : 0.0;
        }
        __syncwarp();
        for (int size = 2; size <= P; size <<= 1)
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                for (int k = lane; k < P; k += 32) {
                    const int l = k ^ stride;
                    if (l > k) {
                        const bool up = (k & size) == 0;
                        const int32_t x = sk[k], y = sk[l];
                        if ((x > y) == up) {
                            sk[k] = y;
                            sk[l] = x;
                            if (val) {
                                const double t = sv[k];
                                sv[k] = sv[l];
                                sv[l] = t;
                            }
                        }
                    }
                }
                __syncwarp();
            }
        for (int k = lane; k < len; k += 32) {
            key[b + k] = sk[k];
            if (val) val[b + k] = sv[k];
        }
        __syncwarp();
    }
}

// longest row of a CSR offset array (32- or 64-bit)
__global__ void max_row_kernel(int64_t n, const uint32_t* __restrict__ off32, const int64_t* __restrict__ off64,
                               unsigned long long* __restrict__ out) {
    unsigned long long m = 0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        m = max(m, (unsigned long long)(off64 ? off64[r + 1] - off64[r] : off32[r + 1] - off32[r]));
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// union of two sorted rows (count when out == nullptr)
__global__ void merge_kernel(int64_t n, const uint32_t* __restrict__ pa, const int32_t* __restrict__ ja_, const uint32_t* __restrict__ pb,
                             const int32_t* __restrict__ jb, uint32_t* __restrict__ cnt, const uint32_t* __restrict__ off,
                             int32_t* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint32_t a = pa[i], b = pb[i], k = 0;
        const uint32_t ae = pa[i + 1], be = pb[i + 1];
        while (a < ae || b < be) {
            int32_t v;
            if (b >= be || (a < ae && ja_[a] < jb[b])) v = ja_[a++];
            else if (a >= ae || jb[b] < ja_[a]) v = jb[b++];
            else { v = ja_[a++]; ++b; }
            if (out) out[off[i] + k] = v;
            ++k;
        }
        if (cnt) cnt[i] = k;
    }
}

// Lanczos: w_i = s_i sum_p (a_p s_j) v_j, the row summed in column order (one thread per row)
__global__ void lanczos_spmv_kernel(int64_t n, const int64_t* __restrict__ ia, const int32_t* __restrict__ ja, const double* __restrict__ a,
                                    const double* __restrict__ s, const double* __restrict__ v, double* __restrict__ w) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int64_t p = ia[i]; p < ia[i + 1]; ++p) {
            const int32_t j = ja[p];
            acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(a[p], s[j]), v[j]));
        }
        w[i] = __dmul_rn(s[i], acc);
    }
}
// partial[c] = sum over the rows of chunk c of x_i y_i, in row order: one block per chunk; the block
// forms a tile's products in shared memory, one thread adds them in order
constexpr int kDotTile = 1024;
__global__ void __launch_bounds__(128) chunk_dot_kernel(int64_t n, const double* __restrict__ x, const double* __restrict__ y,
                                                        double* __restrict__ partial) {
    __shared__ double buf[kDotTile];
    const int64_t c = blockIdx.x;
    const int64_t r0 = c * kLanczosChunk, r1 = min(n, r0 + kLanczosChunk);
    double t = 0.0;
    for (int64_t b = r0; b < r1; b += kDotTile) {
        const int m = (int)min((int64_t)kDotTile, r1 - b);
        for (int k = threadIdx.x; k < m; k += blockDim.x) buf[k] = __dmul_rn(x[b + k], y[b + k]);
        __syncthreads();
        if (threadIdx.x == 0)
            for (int k = 0; k < m; ++k) t = __dadd_rn(t, buf[k]);
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[c] = t;
}
// w_i -= a v_i + b vold_i
__global__ void lanczos_update_kernel(int64_t n, double a, double b, const double* __restrict__ v, const double* __restrict__ vold,
                                      double* __restrict__ w) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        w[i] = __dsub_rn(w[i], __dadd_rn(__dmul_rn(a, v[i]), __dmul_rn(b, vold[i])));
}
// vold = v; v = w / b
__global__ void lanczos_next_kernel(int64_t n, double b, const double* __restrict__ w, double* __restrict__ v, double* __restrict__ vold) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        vold[i] = v[i];
        v[i] = __ddiv_rn(w[i], b);
    }
}
__global__ void inv_sqrt_kernel(int64_t n, const double* __restrict__ d, double* __restrict__ s) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s[i] = d[i] > 0.0 ? __ddiv_rn(1.0, __dsqrt_rn(d[i])) : 0.0;
}

// tentative prolongator rows: one entry (agg_i, s0[agg_i]) where agg_i >= 0
__global__ void p0_count_kernel(int64_t n, const int32_t* __restrict__ agg, uint32_t* __restrict__ cnt) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        cnt[i] = agg[i] >= 0 ? 1u : 0u;
}
__global__ void p0_fill_kernel(int64_t n, const int32_t* __restrict__ agg, const double* __restrict__ s0, const uint32_t* __restrict__ off,
                               int64_t* __restrict__ ia, int32_t* __restrict__ ja, double* __restrict__ a) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i <= n; i += (int64_t)gridDim.x * blockDim.x) {
        ia[i] = off[i];
        if (i < n && agg[i] >= 0) {
            ja[off[i]] = agg[i];
            a[off[i]] = s0[agg[i]];
        }
    }
}

// P = P0 - omega D^-1 (A P0), the two sorted rows merged (count when oj == nullptr)
__global__ void prolong_merge_kernel(int64_t n, const int64_t* __restrict__ p0i, const int32_t* __restrict__ p0j,
                                     const double* __restrict__ p0a, const int64_t* __restrict__ qi, const int32_t* __restrict__ qj,
                                     const double* __restrict__ qa, const double* __restrict__ d, double omega, uint32_t* __restrict__ cnt,
                                     const uint32_t* __restrict__ off, int32_t* __restrict__ oj, double* __restrict__ oa) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double f = d[i] != 0.0 ? __ddiv_rn(omega, d[i]) : 0.0;
        int64_t p = p0i[i];
        const int64_t pe = p0i[i + 1];
        uint32_t k = 0;
        const int64_t o = oj ? (int64_t)off[i] : 0;
        for (int64_t q = qi[i]; q < qi[i + 1]; ++q) {
            const int32_t c = qj[q];
            for (; p < pe && p0j[p] < c; ++p, ++k)
                if (oj) { oj[o + k] = p0j[p]; oa[o + k] = p0a[p]; }
            double v = __dmul_rn(-f, qa[q]);
            if (p < pe && p0j[p] == c) { v = __dadd_rn(v, p0a[p]); ++p; }
            if (oj) { oj[o + k] = c; oa[o + k] = v; }
            ++k;
        }
        for (; p < pe; ++p, ++k)
            if (oj) { oj[o + k] = p0j[p]; oa[o + k] = p0a[p]; }
        if (cnt) cnt[i] = k;
    }
}

__global__ void u32_to_i64_kernel(int64_t n1, const uint32_t* __restrict__ a, int64_t* __restrict__ b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n1; i += (int64_t)gridDim.x * blockDim.x) b[i] = a[i];
}

// longest row and largest product count of a sparse product's rows (left factor A, right factor B)
__global__ void row_stats_kernel(int64_t n, const int64_t* __restrict__ ia, const int32_t* __restrict__ ja, const int64_t* __restrict__ ib,
                                 unsigned long long* __restrict__ out) {
    unsigned long long mlen = 0, mprod = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        unsigned long long pr = 0;
        for (int64_t p = ia[i]; p < ia[i + 1]; ++p) pr += (unsigned long long)(ib[ja[p] + 1] - ib[ja[p]]);
        mlen = max(mlen, (unsigned long long)(ia[i + 1] - ia[i]));
        mprod = max(mprod, pr);
    }
    for (int o = 16; o > 0; o >>= 1) {
        mlen = max(mlen, __shfl_xor_sync(0xffffffffu, mlen, o));
        mprod = max(mprod, __shfl_xor_sync(0xffffffffu, mprod, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(out, mlen);
        atomicMax(out + 1, mprod);
    }
}

// node of each dof (near null space levels: nodes are consecutive dof ranges)
__global__ void node_of_kernel(int64_t nn, const int64_t* __restrict__ node_ptr, int32_t* __restrict__ node_of) {
    for (int64_t I = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; I < nn; I += (int64_t)gridDim.x * blockDim.x)
        for (int64_t i = node_ptr[I]; i < node_ptr[I + 1]; ++i) node_of[i] = (int32_t)I;
}

// node graph of the dof graph (sp, sj): one warp per node, the nodes of its dofs' neighbours gathered in
// shared memory (cap entries per warp), sorted (bitonic), duplicates and the node itself removed; count
// (out == nullptr) or fill
constexpr int kCollapseMax = 16384;
__global__ void __launch_bounds__(128) collapse_kernel(int64_t nn, const int64_t* __restrict__ node_ptr, const uint32_t* __restrict__ sp,
                                                       const int32_t* __restrict__ sj, const int32_t* __restrict__ node_of, int cap,
                                                       uint32_t* __restrict__ cnt, const uint32_t* __restrict__ off,
                                                       int32_t* __restrict__ out, int* __restrict__ status) {
    extern __shared__ __align__(16) int32_t cbuf[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, warps = blockDim.x >> 5;
    int32_t* b = cbuf + (size_t)warp * cap;
    for (int64_t I = (int64_t)blockIdx.x * warps + warp; I < nn; I += (int64_t)gridDim.x * warps) {
        const uint32_t q0 = sp[node_ptr[I]], q1 = sp[node_ptr[I + 1]];
        const int len = (int)(q1 - q0);
        if (len > cap) {
            if (lane == 0) {
                atomicOr(status, kStOverflow);
                if (cnt) cnt[I] = 0;
            }
            continue;
        }
        int P = 1;
        while (P < len) P <<= 1;
        for (int k = lane; k < P; k += 32) {
            const int32_t J = k < len ? node_of[sj[q0 + k]] : INT32_MAX;
            b[k] = (J == (int32_t)I) ? INT32_MAX : J;
        }
        __syncwarp();
        for (int size = 2; size <= P; size <<= 1)
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                for (int k = lane; k < P; k += 32) {
                    const int l = k ^ stride;
                    if (l > k) {
                        const bool up = (k & size) == 0;
                        const int32_t x = b[k], y = b[l];
                        if ((x > y) == up) { b[k] = y; b[l] = x; }
                    }
                }
                __syncwarp();
            }
        // distinct values: a position k counts when b[k] is real and differs from b[k - 1]
        uint32_t run = 0;
        for (int k0 = 0; k0 < P; k0 += 32) {
            const int k = k0 + lane;
            const bool keep = k < P && b[k] != INT32_MAX && (k == 0 || b[k] != b[k - 1]);
            const unsigned m = __ballot_sync(0xffffffffu, keep);
            if (keep && out) out[off[I] + run + __popc(m & ((1u << lane) - 1u))] = b[k];
            run += __popc(m);
        }
        if (cnt && lane == 0) cnt[I] = run;
        __syncwarp();
    }
}

// longest gathered list of collapse_kernel: max over nodes of the node's dof rows' total length
__global__ void node_len_kernel(int64_t nn, const int64_t* __restrict__ node_ptr, const uint32_t* __restrict__ sp,
                                unsigned long long* __restrict__ out) {
    unsigned long long m = 0;
    for (int64_t I = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; I < nn; I += (int64_t)gridDim.x * blockDim.x)
        m = max(m, (unsigned long long)(sp[node_ptr[I + 1]] - sp[node_ptr[I]]));
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// rigid body modes at the dof nodes: node coordinates from the first incident element's affine map
// (barycentric weights of the local node), then the six modes about the centroid c
__global__ void node_coords_kernel(int64_t nnodes, int n, const int64_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                                   const int32_t* __restrict__ tets, const double* __restrict__ xyz, const double* __restrict__ lam,
                                   double* __restrict__ out) {
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < nnodes; m += (int64_t)gridDim.x * blockDim.x) {
        double x[3] = {0.0, 0.0, 0.0};
        if (inc_ptr[m + 1] > inc_ptr[m]) {
            const int32_t code = inc[inc_ptr[m]];
            const int64_t e = code >> 5;
            const int a = code & 31;
            for (int v = 0; v < 4; ++v) {
                const double w = lam[a * 4 + v];
                const int64_t g = tets[e * 4 + v];
                for (int d = 0; d < 3; ++d) x[d] = fma(w, xyz[g * 3 + d], x[d]);
            }
        }
        for (int d = 0; d < 3; ++d) out[m * 3 + d] = x[d];
    }
}
__global__ void rbm_kernel(int64_t nnodes, const double* __restrict__ xn, double cx, double cy, double cz, double* __restrict__ m0,
                           double* __restrict__ m1, double* __restrict__ m2, double* __restrict__ m3, double* __restrict__ m4,
                           double* __restrict__ m5) {
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < nnodes; m += (int64_t)gridDim.x * blockDim.x) {
        const double x = xn[m * 3] - cx, y = xn[m * 3 + 1] - cy, z = xn[m * 3 + 2] - cz;
        const int64_t r = m * 3;
        m0[r] = 1.0; m0[r + 1] = 0.0; m0[r + 2] = 0.0;
        m1[r] = 0.0; m1[r + 1] = 1.0; m1[r + 2] = 0.0;
        m2[r] = 0.0; m2[r + 1] = 0.0; m2[r + 2] = 1.0;
        m3[r] = -y; m3[r + 1] = x; m3[r + 2] = 0.0;
        m4[r] = 0.0; m4[r + 1] = -z; m4[r + 2] = y;
        m5[r] = z; m5[r + 1] = 0.0; m5[r + 2] = -x;
    }
}

// Aggregation rounds (the host set-up's aggregate_mis2, amg_setup.cpp): states 0 undecided, 1 root,
// 2 out, 3 no strong neighbours; each kernel reads the previous step's arrays only.
__global__ void mis_init_kernel(int64_t n, const uint32_t* __restrict__ sp, int8_t* __restrict__ state) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        state[i] = sp[i + 1] > sp[i] ? 0 : 3;
}
// largest undecided key and any root in the closed neighbourhood (8 lanes per node, reductions by
// shuffles: max and or do not depend on the order)
constexpr int kMisLanes = 8;
__global__ void __launch_bounds__(256) mis_pass1_kernel(int64_t n, const uint32_t* __restrict__ sp, const int32_t* __restrict__ sj,
                                                        const int8_t* __restrict__ state, uint64_t* __restrict__ m1,
                                                        uint8_t* __restrict__ r1) {
    const int sub = threadIdx.x & (kMisLanes - 1);
    const int64_t groups = (int64_t)gridDim.x * (blockDim.x / kMisLanes);
    for (int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kMisLanes;; i += groups) {
        const bool live = i < n;
        uint64_t m = 0;
        unsigned r = 0;
        if (live) {
            if (sub == 0) {
                m = state[i] == 0 ? amg_mis_key(i) : 0;
                r = state[i] == 1;
            }
            for (uint32_t q = sp[i] + sub; q < sp[i + 1]; q += kMisLanes) {
                const int32_t j = sj[q];
                const int8_t sjs = state[j];
                if (sjs == 0) m = max(m, amg_mis_key(j));
                r |= sjs == 1;
            }
        }
        for (int o = kMisLanes / 2; o > 0; o >>= 1) {
            m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
            r |= __shfl_xor_sync(0xffffffffu, r, o);
        }
        if (live && sub == 0) {
            m1[i] = m;
            r1[i] = (uint8_t)r;
        }
        // all lanes of the warp leave together (the shuffles above need them)
        if (__all_sync(0xffffffffu, i >= n)) break;
    }
}
// the same over distance 2, and the new state; counts the nodes left undecided
__global__ void __launch_bounds__(256) mis_pass2_kernel(int64_t n, const uint32_t* __restrict__ sp, const int32_t* __restrict__ sj,
                                                        const int8_t* __restrict__ state, const uint64_t* __restrict__ m1,
                                                        const uint8_t* __restrict__ r1, int8_t* __restrict__ nstate,
                                                        unsigned long long* __restrict__ undecided) {
    const int sub = threadIdx.x & (kMisLanes - 1);
    const int64_t groups = (int64_t)gridDim.x * (blockDim.x / kMisLanes);
    unsigned long long c = 0;
    for (int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kMisLanes;; i += groups) {
        const bool live = i < n;
        const int8_t s0 = live ? state[i] : (int8_t)3;
        uint64_t m = 0;
        unsigned r = 0;
        if (live && s0 == 0) {
            if (sub == 0) {
                m = m1[i];
                r = r1[i];
            }
            for (uint32_t q = sp[i] + sub; q < sp[i + 1]; q += kMisLanes) {
                m = max(m, m1[sj[q]]);
                r |= r1[sj[q]];
            }
        }
        for (int o = kMisLanes / 2; o > 0; o >>= 1) {
            m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
            r |= __shfl_xor_sync(0xffffffffu, r, o);
        }
        if (live && sub == 0) {
            int8_t ns = s0;
            if (s0 == 0) {
                if (r) ns = 2;
                else if (m == amg_mis_key(i)) ns = 1;
                else ++c;
            }
            nstate[i] = ns;
        }
        // all lanes of the warp leave together (the shuffles above need them)
        if (__all_sync(0xffffffffu, i >= n)) break;
    }
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(undecided, c);
}
__global__ void mis_root_flag_kernel(int64_t n, const int8_t* __restrict__ state, uint32_t* __restrict__ flag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        flag[i] = state[i] == 1 ? 1u : 0u;
}
// roots and their neighbours (a node has at most one root neighbour)
__global__ void mis_assign1_kernel(int64_t n, const uint32_t* __restrict__ sp, const int32_t* __restrict__ sj,
                                   const int8_t* __restrict__ state, const uint32_t* __restrict__ rank, int32_t* __restrict__ a1) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int32_t a = -1;
        if (state[i] == 1) {
            a = (int32_t)rank[i];
        } else {
            for (uint32_t q = sp[i]; q < sp[i + 1]; ++q)
                if (state[sj[q]] == 1) { a = (int32_t)rank[sj[q]]; break; }
        }
        a1[i] = a;
    }
}
// the other coupled nodes join the aggregate of their first neighbour (column order) aggregated above
__global__ void mis_assign2_kernel(int64_t n, const uint32_t* __restrict__ sp, const int32_t* __restrict__ sj,
                                   const int8_t* __restrict__ state, const int32_t* __restrict__ a1, int32_t* __restrict__ agg) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int32_t a = a1[i];
        if (a < 0 && state[i] != 3)
            for (uint32_t q = sp[i]; q < sp[i + 1]; ++q)
                if (a1[sj[q]] >= 0) { a = a1[sj[q]]; break; }
        agg[i] = a;
    }
}
// tentative scaling of the constant vector: aggregate sizes, then 1/sqrt(size)
__global__ void agg_size_kernel(int64_t n, const int32_t* __restrict__ agg, unsigned int* __restrict__ sz) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (agg[i] >= 0) atomicAdd(sz + agg[i], 1u);
}
__global__ void agg_scale_kernel(int64_t nagg, const unsigned int* __restrict__ sz, double* __restrict__ s0) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nagg; c += (int64_t)gridDim.x * blockDim.x)
        s0[c] = __ddiv_rn(1.0, __dsqrt_rn((double)sz[c]));
}

// Sparse product C = A B, one warp per row of A (see the file comment). Count pass (oj == nullptr):
// cnt[i] = distinct columns of row i, or row i appended to `ovf` when it holds more than tsize / 2
// (status overflow when ovf is null). Fill pass: rows whose count exceeds tsize / 2 are left to a
// larger table; the others are written sorted at off[i].
struct SpgemmArgs {
    int64_t nrows = 0;
    const int32_t* rows = nullptr;   // row list (null: rows 0..nrows-1)
    const int64_t* ia = nullptr;
    const int32_t* ja = nullptr;
    const double* a = nullptr;
    const int64_t* ib = nullptr;
    const int32_t* jb = nullptr;
    const double* b = nullptr;
    int tsize = 256;                 // hash slots per warp (power of two, >= 64)
    int tshift = 24;                 // 32 - log2(tsize)
    int warps = 8;                   // warps per block
    int wbytes = 0;                  // shared memory per warp
    uint32_t* cnt = nullptr;
    int32_t* ovf = nullptr;
    uint32_t* novf = nullptr;
    const int64_t* off = nullptr;
    int32_t* oj = nullptr;
    double* oa = nullptr;
    int* status = nullptr;
};

int spgemm_warp_bytes(int tsize) {
    const int b = tsize * 8 + 32 * 8 + tsize * 4 + (tsize / 2) * 4;
    return (b + 15) & ~15;
}

__global__ void __launch_bounds__(256) spgemm_kernel(SpgemmArgs g) {
    extern __shared__ __align__(16) unsigned char sg_smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* base = sg_smem + (size_t)warp * g.wbytes;
    double* hv = reinterpret_cast<double*>(base);                               // tsize values
    double* stage = hv + g.tsize;                                               // 32 products
    int32_t* hk = reinterpret_cast<int32_t*>(stage + 32);                       // tsize keys (-1: empty)
    int32_t* list = hk + g.tsize;                                               // tsize / 2 used slots
    const int T = g.tsize, half = g.tsize / 2;
    const bool fill = g.oj != nullptr;
    for (int k = lane; k < T; k += 32) hk[k] = -1;
    __syncwarp();
    for (int64_t r = (int64_t)blockIdx.x * g.warps + warp; r < g.nrows; r += (int64_t)gridDim.x * g.warps) {
        const int64_t i = g.rows ? (int64_t)g.rows[r] : r;
        if (fill && g.off[i + 1] - g.off[i] > half) continue;        // a larger table's row
        const int64_t a0 = g.ia[i];
        const int na = (int)(g.ia[i + 1] - a0);
        int nuniq = 0;
        bool over = false;
        // the row of A in chunks of 32 entries (one per lane: its B row's start, length and the A value);
        // the chunk's products in (A column, B column) order, 32 at a time
        for (int c0 = 0; c0 < na && !over; c0 += 32) {
            const int cn = min(32, na - c0);
            int len = 0;
            int64_t bstart = 0;
            double av = 0.0;
            if (lane < cn) {
                const int32_t c = g.ja[a0 + c0 + lane];
                bstart = g.ib[c];
                len = (int)(g.ib[c + 1] - bstart);
                if (fill) av = g.a[a0 + c0 + lane];
            }
            int x = len;
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            const int excl = x - len;
            const int ctot = __shfl_sync(0xffffffffu, x, 31);
            for (int s0 = 0; s0 < ctot; s0 += 32) {
                const int pidx = s0 + lane;
                const bool act = pidx < ctot;
                // the chunk entry of product pidx: the last lane e < cn with excl_e <= pidx (fixed 5 steps)
                int lo = 0;
                for (int step = 16; step > 0; step >>= 1) {
                    const int cand = lo + step;
                    const int ec = __shfl_sync(0xffffffffu, excl, cand & 31);
                    if (cand < cn && ec <= pidx) lo = cand;
                }
                const int e_excl = __shfl_sync(0xffffffffu, excl, lo);
                const int64_t e_start = __shfl_sync(0xffffffffu, bstart, lo);
                const double e_a = __shfl_sync(0xffffffffu, av, lo);
                int32_t col = -1;
                double val = 0.0;
                if (act) {
                    const int64_t q = e_start + (pidx - e_excl);
                    col = g.jb[q];
                    if (fill) val = __dmul_rn(e_a, g.b[q]);
                }
                const unsigned grp = __match_any_sync(0xffffffffu, col);
                const bool leader = act && lane == __ffs(grp) - 1;
                int slot = -1;
                bool newkey = false;
                if (leader) {
                    uint32_t h = ((uint32_t)col * 2654435761u) >> g.tshift;
                    for (int probe = 0; probe < T; ++probe) {
                        const int32_t old = atomicCAS(hk + h, -1, col);
                        if (old == -1) { newkey = true; slot = (int)h; break; }
                        if (old == col) { slot = (int)h; break; }
                        h = (h + 1) & (uint32_t)(T - 1);
                    }
                    if (slot < 0) over = true;
                }
                const unsigned nb = __ballot_sync(0xffffffffu, newkey);
                if (newkey) {
                    const int pos = nuniq + __popc(nb & ((1u << lane) - 1u));
                    if (pos < half) list[pos] = slot;
                }
                nuniq += __popc(nb);
                if (fill) {
                    stage[lane] = val;
                    __syncwarp();
                    if (leader && slot >= 0) {
                        double v = newkey ? 0.0 : hv[slot];
                        for (unsigned m = grp; m; m &= m - 1u) v = __dadd_rn(v, stage[__ffs(m) - 1]);
                        hv[slot] = v;
                    }
                }
                __syncwarp();
                if (__any_sync(0xffffffffu, over) || nuniq > half) { over = true; break; }
            }
        }
        if (over) {
            for (int k = lane; k < T; k += 32) hk[k] = -1;
            __syncwarp();
            if (lane == 0) {
                if (!fill && g.ovf) {
                    g.ovf[atomicAdd(g.novf, 1u)] = (int32_t)i;
                    g.cnt[i] = 0;
                } else {
                    atomicOr(g.status, kStOverflow);
                    if (!fill) g.cnt[i] = 0;
                }
            }
            continue;
        }
        if (!fill) {
            if (lane == 0) g.cnt[i] = (uint32_t)nuniq;
        } else {
            // sort the used slots by key (padding slots -1 sort last), then write the row
            int P = 1;
            while (P < nuniq) P <<= 1;
            for (int k = nuniq + lane; k < P; k += 32) list[k] = -1;
            __syncwarp();
            for (int size = 2; size <= P; size <<= 1)
                for (int stride = size >> 1; stride > 0; stride >>= 1) {
                    for (int k = lane; k < P; k += 32) {
                        const int l = k ^ stride;
                        if (l > k) {
                            const bool up = (k & size) == 0;
                            const int32_t sa = list[k], sb = list[l];
                            const int32_t ka = sa < 0 ? INT32_MAX : hk[sa], kb = sb < 0 ? INT32_MAX : hk[sb];
                            if ((ka > kb) == up) {
                                list[k] = sb;
                                list[l] = sa;
                            }
                        }
                    }
                    __syncwarp();
                }
            const int64_t ob = g.off[i];
            for (int k = lane; k < nuniq; k += 32) {
                const int32_t s = list[k];
                g.oj[ob + k] = hk[s];
                g.oa[ob + k] = hv[s];
            }
        }
        __syncwarp();
        for (int k = lane; k < nuniq; k += 32) hk[list[k]] = -1;
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------------------------------
// host drivers
// ---------------------------------------------------------------------------------------------------

int launch_spgemm(fgpu_ctx* ctx, SpgemmArgs g, int bin) {
    g.tsize = kBins[bin];
    g.tshift = 32 - kBinLog[bin];
    g.wbytes = spgemm_warp_bytes(g.tsize);
    g.warps = std::max(1, std::min(8, (110 * 1024) / g.wbytes));
    const int smem = g.warps * g.wbytes;
    DEV_TRY(cudaFuncSetAttribute(spgemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    const int per_sm = std::max(1, std::min(2048 / (32 * g.warps), (228 * 1024) / (smem + 1024)));
    const int blocks = grid_rows(g.nrows, g.warps, 152 * per_sm);
    spgemm_kernel<<<blocks, 32 * g.warps, smem, ctx->stream>>>(g);
    ctx->launches++;
    DEV_TRY(cudaGetLastError());
    return FGPU_OK;
}

// C = A B (rows sorted by column). *overflow: a row with more distinct columns than the largest table.
int spgemm_dev(fgpu_ctx* ctx, const AmgDevCsr& A, const AmgDevCsr& B, AmgDevCsr& C, int* d_status, bool* overflow) {
    *overflow = false;
    const int64_t n = A.nrows;
    Work w;
    unsigned long long* stats = w.get<unsigned long long>(2);
    uint32_t* cnt = w.get<uint32_t>(n + 1);
    uint32_t* off32 = w.get<uint32_t>(n + 1);
    int32_t* ovf[kNumBins] = {nullptr, w.get<int32_t>(n), w.get<int32_t>(n), w.get<int32_t>(n)};
    uint32_t* novf = w.get<uint32_t>(kNumBins);
    DEV_ALLOC(stats && cnt && off32 && ovf[1] && ovf[2] && ovf[3] && novf);
    DEV_TRY(cudaMemsetAsync(stats, 0, 2 * sizeof(unsigned long long), ctx->stream));
    DEV_TRY(cudaMemsetAsync(novf, 0, kNumBins * sizeof(uint32_t), ctx->stream));
    row_stats_kernel<<<grid_rows(n, 256), 256, 0, ctx->stream>>>(n, A.ia, A.ja, B.ia, stats);
    ctx->launches++;
    unsigned long long hs[2] = {0, 0};
    DEV_TRY(cudaMemcpyAsync(hs, stats, sizeof(hs), cudaMemcpyDeviceToHost, ctx->stream));
    DEV_TRY(cudaStreamSynchronize(ctx->stream));
    if (hs[1] > 0x7fffffffull) { *overflow = true; return FGPU_OK; }
    SpgemmArgs g;
    g.ia = A.ia; g.ja = A.ja; g.a = A.a;
    g.ib = B.ia; g.jb = B.ja; g.b = B.a;
    g.status = d_status;
    // count: all rows with the smallest table, the rows it cannot hold with the next ones in turn
    int64_t rows_in[kNumBins] = {n, 0, 0, 0};
    {
        for (int bin = 0; bin < kNumBins; ++bin) {
            if (bin > 0 && rows_in[bin] == 0) break;
            SpgemmArgs c = g;
            c.nrows = rows_in[bin];
            c.rows = ovf[bin];
            c.cnt = cnt;
            c.ovf = bin + 1 < kNumBins ? ovf[bin + 1] : nullptr;
            c.novf = bin + 1 < kNumBins ? novf + bin + 1 : nullptr;
            int rc = launch_spgemm(ctx, c, bin);
            if (rc) return rc;
            if (bin + 1 < kNumBins) {
                uint32_t hn = 0;
                DEV_TRY(cudaMemcpyAsync(&hn, novf + bin + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
                DEV_TRY(cudaStreamSynchronize(ctx->stream));
                rows_in[bin + 1] = hn;
            }
        }
    }
    int st = 0;
    int rc = read_status(ctx, d_status, &st);
    if (rc) return rc;
    if (st & kStOverflow) { *overflow = true; return FGPU_OK; }
    uint64_t total = 0;
    rc = scan_u32(ctx, cnt, off32, n, &total);
    if (rc) return rc;
    rc = alloc_csr(ctx, C, n, B.ncols, (int64_t)total);
    if (rc) return rc;
    u32_to_i64_kernel<<<grid_rows(n + 1, 256), 256, 0, ctx->stream>>>(n + 1, off32, C.ia);
    ctx->launches++;
    g.off = C.ia; g.oj = C.ja; g.oa = C.a;
    for (int bin = 0; bin < kNumBins; ++bin) {
        if (rows_in[bin] == 0) continue;
        SpgemmArgs f = g;
        f.nrows = rows_in[bin];
        f.rows = ovf[bin];
        rc = launch_spgemm(ctx, f, bin);
        if (rc) return rc;
    }
    rc = read_status(ctx, d_status, &st);
    if (rc) return rc;
    *overflow = (st & kStOverflow) != 0;
    return FGPU_OK;
}

int seg_sort(fgpu_ctx* ctx, int64_t n, const uint32_t* off32, const int64_t* off64, int32_t* key, double* val, int* d_status) {
    unsigned long long* dmax = nullptr;
    DEV_TRY(cudaMalloc(&dmax, sizeof(unsigned long long)));
    struct Free { unsigned long long* p; ~Free() { cudaFree(p); } } fr{dmax};
    DEV_TRY(cudaMemsetAsync(dmax, 0, sizeof(unsigned long long), ctx->stream));
    max_row_kernel<<<grid_rows(n, 256), 256, 0, ctx->stream>>>(n, off32, off64, dmax);
    unsigned long long hmax = 0;
    DEV_TRY(cudaMemcpyAsync(&hmax, dmax, sizeof(hmax), cudaMemcpyDeviceToHost, ctx->stream));
    DEV_TRY(cudaStreamSynchronize(ctx->stream));
    ctx->launches++;
    if (hmax <= 1) return FGPU_OK;
    int cap = 32;
    while (cap < (int)std::min<unsigned long long>(hmax, (unsigned long long)kSortMax + 1)) cap <<= 1;
    cap = std::min(cap, kSortMax);              // longer rows raise the overflow status
    const int bytes = val ? 12 : 4;
    const int warps = std::max(1, std::min(4, (96 * 1024) / (cap * bytes)));
    const int smem = warps * cap * bytes;
    DEV_TRY(cudaFuncSetAttribute(seg_sort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    seg_sort_kernel<<<grid_rows(n, warps, 152 * 8), warps * 32, smem, ctx->stream>>>(n, off32, off64, cap, key, val, d_status);
    ctx->launches++;
    DEV_TRY(cudaGetLastError());
    return FGPU_OK;
}

// T = M^T of an n x m device CSR (rows of T sorted by column of M)
int transpose_dev(fgpu_ctx* ctx, const AmgDevCsr& M, AmgDevCsr& T, int* d_status) {
    const int64_t m = M.ncols;
    Work w;
    uint32_t* tcnt = w.get<uint32_t>(m + 1);
    uint32_t* toff = w.get<uint32_t>(m + 1);
    uint32_t* cur = w.get<uint32_t>(m + 1);
    DEV_ALLOC(tcnt && toff && cur);
    DEV_TRY(cudaMemsetAsync(tcnt, 0, (m + 1) * sizeof(uint32_t), ctx->stream));
    col_count_kernel<<<grid_rows(M.nnz, 256), 256, 0, ctx->stream>>>(M.nnz, M.ja, tcnt);
    ctx->launches++;
    int rc = scan_u32(ctx, tcnt, toff, m, nullptr);
    if (rc) return rc;
    rc = alloc_csr(ctx, T, m, M.nrows, M.nnz);
    if (rc) return rc;
    DEV_TRY(cudaMemcpyAsync(cur, toff, (m + 1) * sizeof(uint32_t), cudaMemcpyDeviceToDevice, ctx->stream));
    transpose_fill_kernel<<<grid_rows(M.nrows, 256), 256, 0, ctx->stream>>>(M.nrows, nullptr, M.ia, M.ja, M.a, cur, T.ja, T.a);
    u32_to_i64_kernel<<<grid_rows(m + 1, 256), 256, 0, ctx->stream>>>(m + 1, toff, T.ia);
    ctx->launches += 2;
    rc = seg_sort(ctx, m, nullptr, T.ia, T.ja, T.a, d_status);
    if (rc) return rc;
    DEV_TRY(cudaStreamSynchronize(ctx->stream));     // the scratch above is freed on return
    return FGPU_OK;
}

// lambda_max(D^-1 A) by Lanczos on its own stream, driven by its own host thread (it runs while the
// host aggregates); the same arithmetic as the host set-up's estimate
struct LanczosJob {
    int64_t n = 0;
    const int64_t* ia = nullptr;
    const int32_t* ja = nullptr;
    const double* a = nullptr;
    const double* d = nullptr;
    double *s = nullptr, *v = nullptr, *vold = nullptr, *wv = nullptr, *part = nullptr;
    cudaStream_t st = nullptr;
    double lmax = 0;
    int launches = 0;
    cudaError_t err = cudaSuccess;

    bool ok(cudaError_t e) {
        if (e != cudaSuccess && err == cudaSuccess) err = e;
        return e == cudaSuccess;
    }
    int device = 0;
    void run() {
        if (!ok(cudaSetDevice(device))) return;
        std::vector<double> hv0;
        amg_lanczos_start(n, hv0);
        const int64_t nch = (n + kLanczosChunk - 1) / kLanczosChunk;
        if (!ok(cudaMemcpyAsync(v, hv0.data(), n * sizeof(double), cudaMemcpyHostToDevice, st))) return;
        if (!ok(cudaMemsetAsync(vold, 0, n * sizeof(double), st))) return;
        inv_sqrt_kernel<<<grid_rows(n, 256), 256, 0, st>>>(n, d, s);
        ++launches;
        std::vector<double> al, be, hp(nch);
        double bprev = 0.0;
        auto dot = [&](const double* x, const double* y, double* out) {
            chunk_dot_kernel<<<(int)nch, 128, 0, st>>>(n, x, y, part);
            ++launches;
            if (!ok(cudaMemcpyAsync(hp.data(), part, nch * sizeof(double), cudaMemcpyDeviceToHost, st)) || !ok(cudaStreamSynchronize(st)))
                return false;
            double t = 0.0;
            for (int64_t c = 0; c < nch; ++c) t += hp[c];
            *out = t;
            return true;
        };
        for (int k = 0; k < kLanczosSteps; ++k) {
            lanczos_spmv_kernel<<<grid_rows(n, 256), 256, 0, st>>>(n, ia, ja, a, s, v, wv);
            ++launches;
            double al_k = 0.0, b2 = 0.0;
            if (!dot(wv, v, &al_k)) return;
            lanczos_update_kernel<<<grid_rows(n, 256), 256, 0, st>>>(n, al_k, bprev, v, vold, wv);
            ++launches;
            if (!dot(wv, wv, &b2)) return;
            const double b = std::sqrt(b2);
            al.push_back(al_k);
            if (b < 1e-14 * std::fabs(al_k) || k + 1 == kLanczosSteps) break;
            be.push_back(b);
            lanczos_next_kernel<<<grid_rows(n, 256), 256, 0, st>>>(n, b, wv, v, vold);
            ++launches;
            bprev = b;
        }
        ok(cudaGetLastError());
        lmax = amg_tridiag_lmax(al, be);
    }
};

// One level on the device: lambda_max, strength graph, aggregation (host), P, R, A_c = R (A P).
// *handoff: the level goes to the host set-up instead (a row beyond a kernel's capacity, or nothing
// to coarsen); *last: the coarsening stagnates and A_c is the coarsest operator.
int level_dev(fgpu_ctx* ctx, AmgDevLevel& L, const AmgHostCfg& cfg, const AmgNns* nns, AmgNns* next, int* d_status, AmgDevCsr& Ac,
              bool* handoff, bool* last, AmgSetupTimes& tm) {
    using clock = std::chrono::steady_clock;
    auto ms_since = [](clock::time_point t) { return std::chrono::duration<double, std::milli>(clock::now() - t).count(); };
    auto tphase = clock::now();
    *handoff = false;
    *last = false;
    const AmgDevCsr& A = L.A;
    const int64_t n = A.nrows;
    const int64_t nch = (n + kLanczosChunk - 1) / kLanczosChunk;
    Work w;
    double* d = w.get<double>(n);
    uint32_t* cnt = w.get<uint32_t>(n + 1);
    uint32_t* tp = w.get<uint32_t>(n + 1);
    LanczosJob lz;
    lz.n = n; lz.ia = A.ia; lz.ja = A.ja; lz.a = A.a; lz.d = d; lz.device = ctx->device;
    lz.s = w.get<double>(n);
    lz.v = w.get<double>(n);
    lz.vold = w.get<double>(n);
    lz.wv = w.get<double>(n);
    lz.part = w.get<double>(nch);
    DEV_ALLOC(d && cnt && tp && lz.s && lz.v && lz.vold && lz.wv && lz.part);
    diag_kernel<<<grid_rows(n, 256), 256, 0, ctx->stream>>>(n, A.ia, A.ja, A.a, d, d_status);
    ctx->launches++;
    // the Lanczos thread and stream: started once the diagonal is formed, joined before any return
    std::thread lanczos;
    cudaEvent_t d_ready = nullptr;
    struct LanczosGuard {
        std::thread& t;
        LanczosJob& job;
        cudaEvent_t& ev;
        ~LanczosGuard() {
            if (t.joinable()) t.join();
            if (job.st) cudaStreamDestroy(job.st);
            if (ev) cudaEventDestroy(ev);
        }
    } lanczos_guard{lanczos, lz, d_ready};
    DEV_TRY(cudaEventCreateWithFlags(&d_ready, cudaEventDisableTiming));
    DEV_TRY(cudaEventRecord(d_ready, ctx->stream));
    DEV_TRY(cudaStreamCreateWithFlags(&lz.st, cudaStreamNonBlocking));
    DEV_TRY(cudaStreamWaitEvent(lz.st, d_ready, 0));
    lanczos = std::thread([&lz] { lz.run(); });
    strong_kernel<<<grid_rows(n, 256), 256, 0, ctx->stream>>>(n, A.ia, A.ja, A.a, d, cfg.threshold, cnt, nullptr, nullptr);
    ctx->launches++;
    uint64_t ns = 0;
    int rc = scan_u32(ctx, cnt, tp, n, &ns);
    if (rc) return rc;
    int st = 0;
    rc = read_status(ctx, d_status, &st);
    if (rc) return rc;
    if (st & kStDiag) { ctx->err = "gamg: the diagonal must be positive (SPD matrix)"; return FGPU_ERR_INVALID; }
    // strength graph S, its rows in column order
    int32_t* tmpj = w.get<int32_t>((int64_t)ns);
    DEV_ALLOC(tmpj);
    strong_kernel<<<grid_rows(n, 256), 256, 0, ctx->stream>>>(n, A.ia, A.ja, A.a, d, cfg.threshold, nullptr, tp, tmpj);
    ctx->launches++;
    // the graph to aggregate: the symmetrised dof graph S + S^T, or (near null space) its node graph,
    // formed as N(S) + N(S)^T (the same sorted rows as N(S + S^T): a node pair is coupled when any of
    // their dofs are, in either direction), which symmetrises the node graph instead of the nine-times
    // larger dof graph of a 3-component operator (vector P2 48^3 beam, the set-up run alone: graph phase
    // 113 -> 54 ms, set-up 750 -> 705 ms, the Lanczos estimate on its own stream now overlapping the
    // aggregation; after the other solves of the elasticity workload 742 ms)
    int64_t ng = n;
    const uint32_t* gp = tp;
    const int32_t* gjs = tmpj;
    if (nns) {
        ng = (int64_t)nns->node_ptr.size() - 1;
        int64_t* dnp = w.get<int64_t>(ng + 1);
        int32_t* node_of = w.get<int32_t>(n);
        uint32_t* ncnt = w.get<uint32_t>(ng + 1);
        uint32_t* np32 = w.get<uint32_t>(ng + 1);
        DEV_ALLOC(dnp && node_of && ncnt && np32);
        unsigned long long* dmax = w.get<unsigned long long>(1);
        DEV_ALLOC(dmax);
        DEV_TRY(cudaMemcpyAsync(dnp, nns->node_ptr.data(), (ng + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
        DEV_TRY(cudaMemsetAsync(dmax, 0, sizeof(unsigned long long), ctx->stream));
        node_of_kernel<<<grid_rows(ng, 256), 256, 0, ctx->stream>>>(ng, dnp, node_of);
        node_len_kernel<<<grid_rows(ng, 256), 256, 0, ctx->stream>>>(ng, dnp, tp, dmax);
        unsigned long long hmax = 0;
        DEV_TRY(cudaMemcpyAsync(&hmax, dmax, sizeof(hmax), cudaMemcpyDeviceToHost, ctx->stream));
        DEV_TRY(cudaStreamSynchronize(ctx->stream));
        if (hmax > (unsigned long long)kCollapseMax) { *handoff = true; tm.handoff = 2; return FGPU_OK; }
        int cap = 32;
        while (cap < (int)hmax) cap <<= 1;
        const int cwarps = std::max(1, std::min(4, (96 * 1024) / (cap * 4)));
        const int csmem = cwarps * cap * 4;
        DEV_TRY(cudaFuncSetAttribute(collapse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, csmem));
        collapse_kernel<<<grid_rows(ng, cwarps, 152 * 8), cwarps * 32, csmem, ctx->stream>>>(ng, dnp, tp, tmpj, node_of, cap, ncnt, nullptr,
                                                                                            nullptr, d_status);
        ctx->launches += 3;
        uint64_t nnj = 0;
        rc = scan_u32(ctx, ncnt, np32, ng, &nnj);
        if (rc) return rc;
        int32_t* nj = w.get<int32_t>((int64_t)nnj);
        DEV_ALLOC(nj);
        collapse_kernel<<<grid_rows(ng, cwarps, 152 * 8), cwarps * 32, csmem, ctx->stream>>>(ng, dnp, tp, tmpj, node_of, cap, nullptr, np32,
                                                                                            nj, d_status);
        ctx->launches++;
        gp = np32;
        gjs = nj;
        ns = nnj;
    }
    // symmetrise: the transpose by column counts and cursors, its rows sorted, merged row by row
    uint32_t* tcnt = w.get<uint32_t>(ng + 1);
    uint32_t* tc = w.get<uint32_t>(ng + 1);
    uint32_t* cur = w.get<uint32_t>(ng + 1);
    int32_t* tj = w.get<int32_t>((int64_t)ns);
    uint32_t* sp32 = w.get<uint32_t>(ng + 1);
    DEV_ALLOC(tcnt && tc && cur && tj && sp32);
    DEV_TRY(cudaMemsetAsync(tcnt, 0, (ng + 1) * sizeof(uint32_t), ctx->stream));
    col_count_kernel<<<grid_rows((int64_t)ns, 256), 256, 0, ctx->stream>>>((int64_t)ns, gjs, tcnt);
    ctx->launches++;
    rc = scan_u32(ctx, tcnt, tc, ng, nullptr);
    if (rc) return rc;
    DEV_TRY(cudaMemcpyAsync(cur, tc, (ng + 1) * sizeof(uint32_t), cudaMemcpyDeviceToDevice, ctx->stream));
    transpose_fill_kernel<<<grid_rows(ng, 256), 256, 0, ctx->stream>>>(ng, gp, nullptr, gjs, nullptr, cur, tj, nullptr);
    ctx->launches++;
    rc = seg_sort(ctx, ng, tc, nullptr, tj, nullptr, d_status);
    if (rc) return rc;
    merge_kernel<<<grid_rows(ng, 256), 256, 0, ctx->stream>>>(ng, gp, gjs, tc, tj, cnt, nullptr, nullptr);
    ctx->launches++;
    uint64_t nsg = 0;
    rc = scan_u32(ctx, cnt, sp32, ng, &nsg);
    if (rc) return rc;
    int32_t* sj = w.get<int32_t>((int64_t)nsg);
    DEV_ALLOC(sj);
    merge_kernel<<<grid_rows(ng, 256), 256, 0, ctx->stream>>>(ng, gp, gjs, tc, tj, nullptr, sp32, sj);
    ctx->launches++;
    const uint32_t* gp32 = sp32;
    const int32_t* gj = sj;
    rc = read_status(ctx, d_status, &st);
    if (rc) return rc;
    if (st & kStOverflow) { *handoff = true; tm.handoff = nns ? 2 : 1; return FGPU_OK; }
    tm.graph += ms_since(tphase);
    tphase = clock::now();
    // aggregation: rounds of the distance-2 independent set, then the two assignment steps
    int8_t* mstate = w.get<int8_t>(ng);
    int8_t* mnext = w.get<int8_t>(ng);
    uint64_t* m1 = w.get<uint64_t>(ng);
    uint8_t* r1 = w.get<uint8_t>(ng);
    unsigned long long* dund = w.get<unsigned long long>(1);
    uint32_t* rflag = w.get<uint32_t>(ng + 1);
    uint32_t* rank = w.get<uint32_t>(ng + 1);
    int32_t* a1 = w.get<int32_t>(ng);
    int32_t* dagg_node = w.get<int32_t>(ng);
    DEV_ALLOC(mstate && mnext && m1 && r1 && dund && rflag && rank && a1 && dagg_node);
    const int gg = grid_rows(ng, 256);
    const int gm = grid_rows(ng, 256 / kMisLanes, 152 * 16);
    mis_init_kernel<<<gg, 256, 0, ctx->stream>>>(ng, gp32, mstate);
    ctx->launches++;
    for (int round = 0;; ++round) {
        if (round > 1000) { ctx->err = "gamg device set-up: aggregation did not converge"; return FGPU_ERR_INVALID; }
        DEV_TRY(cudaMemsetAsync(dund, 0, sizeof(unsigned long long), ctx->stream));
        mis_pass1_kernel<<<gm, 256, 0, ctx->stream>>>(ng, gp32, gj, mstate, m1, r1);
        mis_pass2_kernel<<<gm, 256, 0, ctx->stream>>>(ng, gp32, gj, mstate, m1, r1, mnext, dund);
        ctx->launches += 2;
        std::swap(mstate, mnext);
        unsigned long long hund = 0;
        DEV_TRY(cudaMemcpyAsync(&hund, dund, sizeof(hund), cudaMemcpyDeviceToHost, ctx->stream));
        DEV_TRY(cudaStreamSynchronize(ctx->stream));
        if (hund == 0) break;
    }
    mis_root_flag_kernel<<<gg, 256, 0, ctx->stream>>>(ng, mstate, rflag);
    ctx->launches++;
    uint64_t nroots = 0;
    rc = scan_u32(ctx, rflag, rank, ng, &nroots);
    if (rc) return rc;
    mis_assign1_kernel<<<gg, 256, 0, ctx->stream>>>(ng, gp32, gj, mstate, rank, a1);
    mis_assign2_kernel<<<gg, 256, 0, ctx->stream>>>(ng, gp32, gj, mstate, a1, dagg_node);
    ctx->launches += 2;
    const int64_t nagg = (int64_t)nroots;
    std::vector<int32_t> agg_node;
    std::vector<int32_t>& hagg = nns ? agg_node : L.agg;
    hagg.resize(ng);
    DEV_TRY(cudaMemcpyAsync(hagg.data(), dagg_node, ng * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    DEV_TRY(cudaStreamSynchronize(ctx->stream));
    tm.aggregate += ms_since(tphase);
    tphase = clock::now();
    if (nagg == 0 || nagg >= ng) { *handoff = true; tm.handoff = 3; return FGPU_OK; }
    AmgDevCsr P0;
    int64_t ncoarse = nagg;
    if (nns) {
        // tentative prolongator from the near null space (host QR per aggregate, the host set-up's code)
        HostCsr hP0;
        if (amg_tentative_nns(*nns, agg_node, nagg, cfg.nthreads > 0 ? cfg.nthreads : 1, hP0, *next)) {
            ctx->err = "gamg: coarse level too large";
            return FGPU_ERR_INVALID;
        }
        if (hP0.ncols == 0 || hP0.ncols >= n) { *handoff = true; tm.handoff = 3; return FGPU_OK; }
        ncoarse = hP0.ncols;
        L.agg.assign(n, -1);
        for (int64_t I = 0; I < ng; ++I)
            for (int64_t i = nns->node_ptr[I]; i < nns->node_ptr[I + 1]; ++i) L.agg[i] = agg_node[I];
        rc = alloc_csr(ctx, P0, n, hP0.ncols, (int64_t)hP0.ja.size());
        if (rc) return rc;
        DEV_TRY(cudaMemcpyAsync(P0.ia, hP0.ia.data(), (n + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
        if (!hP0.ja.empty()) {
            DEV_TRY(cudaMemcpyAsync(P0.ja, hP0.ja.data(), hP0.ja.size() * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
            DEV_TRY(cudaMemcpyAsync(P0.a, hP0.a.data(), hP0.a.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
        }
        DEV_TRY(cudaStreamSynchronize(ctx->stream));            // hP0 is freed on leaving this block
    } else {
    // tentative prolongator (1/sqrt(|agg|), the host's 1.0 / std::sqrt of the exact size) and A P0
    const int32_t* dagg = dagg_node;
    unsigned int* dsz = w.get<unsigned int>(nagg);
    double* ds0 = w.get<double>(nagg);
    DEV_ALLOC(dsz && ds0);
    DEV_TRY(cudaMemsetAsync(dsz, 0, nagg * sizeof(unsigned int), ctx->stream));
    agg_size_kernel<<<grid_rows(n, 256), 256, 0, ctx->stream>>>(n, dagg, dsz);
    agg_scale_kernel<<<grid_rows(nagg, 256), 256, 0, ctx->stream>>>(nagg, dsz, ds0);
    p0_count_kernel<<<grid_rows(n, 256), 256, 0, ctx->stream>>>(n, dagg, cnt);
    ctx->launches += 3;
    uint64_t n0 = 0;
    rc = scan_u32(ctx, cnt, tp, n, &n0);
    if (rc) return rc;
    rc = alloc_csr(ctx, P0, n, nagg, (int64_t)n0);
    if (rc) return rc;
    p0_fill_kernel<<<grid_rows(n + 1, 256), 256, 0, ctx->stream>>>(n, dagg, ds0, tp, P0.ia, P0.ja, P0.a);
    ctx->launches++;
    }
    bool ovf = false;
    // lambda_max: wait for the Lanczos thread (A P0 does not need it)
    auto join_lanczos = [&]() -> int {
        const auto tw = clock::now();
        if (lanczos.joinable()) lanczos.join();
        ctx->launches += lz.launches;
        lz.launches = 0;
        tm.lanczos += ms_since(tw);
        if (lz.err != cudaSuccess) { ctx->err = std::string("gamg device set-up: lambda_max: ") + cudaGetErrorString(lz.err); return FGPU_ERR_CUDA; }
        L.lmax = lz.lmax;
        return FGPU_OK;
    };
    if (cfg.agg_smooths <= 0) {
        L.P = std::move(P0);
        rc = join_lanczos();
        if (rc) return rc;
    } else {
        AmgDevCsr AP0;
        rc = spgemm_dev(ctx, A, P0, AP0, d_status, &ovf);
        if (rc) return rc;
        if (ovf) { *handoff = true; tm.handoff = 4; return FGPU_OK; }
        rc = join_lanczos();
        if (rc) return rc;
        const double omega = 4.0 / (3.0 * L.lmax);
        prolong_merge_kernel<<<grid_rows(n, 256), 256, 0, ctx->stream>>>(n, P0.ia, P0.ja, P0.a, AP0.ia, AP0.ja, AP0.a, d, omega, cnt,
                                                                        nullptr, nullptr, nullptr);
        ctx->launches++;
        uint64_t pn = 0;
        rc = scan_u32(ctx, cnt, tp, n, &pn);
        if (rc) return rc;
        rc = alloc_csr(ctx, L.P, n, ncoarse, (int64_t)pn);
        if (rc) return rc;
        prolong_merge_kernel<<<grid_rows(n, 256), 256, 0, ctx->stream>>>(n, P0.ia, P0.ja, P0.a, AP0.ia, AP0.ja, AP0.a, d, omega, nullptr,
                                                                        tp, L.P.ja, L.P.a);
        u32_to_i64_kernel<<<grid_rows(n + 1, 256), 256, 0, ctx->stream>>>(n + 1, tp, L.P.ia);
        ctx->launches += 2;
        DEV_TRY(cudaStreamSynchronize(ctx->stream));         // P0 and A P0 are freed on leaving this block
    }
    rc = transpose_dev(ctx, L.P, L.R, d_status);
    if (rc) return rc;
    rc = read_status(ctx, d_status, &st);
    if (rc) return rc;
    if (st & kStOverflow) { *handoff = true; tm.handoff = 5; return FGPU_OK; }
    tm.prolong += ms_since(tphase);
    tphase = clock::now();
    // Galerkin product A_c = R (A P)
    AmgDevCsr AP;
    rc = spgemm_dev(ctx, A, L.P, AP, d_status, &ovf);
    if (rc) return rc;
    if (ovf) { *handoff = true; tm.handoff = 6; return FGPU_OK; }
    rc = spgemm_dev(ctx, L.R, AP, Ac, d_status, &ovf);
    if (rc) return rc;
    if (ovf) { *handoff = true; tm.handoff = 7; return FGPU_OK; }
    DEV_TRY(cudaStreamSynchronize(ctx->stream));             // the scratch of this level is freed on return
    tm.galerkin += ms_since(tphase);
    if ((double)ncoarse > 0.9 * (double)n) *last = true;
    return FGPU_OK;
}

}  // namespace

int amg_copy_to_host(fgpu_ctx* ctx, const AmgDevCsr& D, HostCsr& H) {
    H.nrows = D.nrows;
    H.ncols = D.ncols;
    H.ia.assign(D.nrows + 1, 0);
    H.ja.resize(D.nnz);
    H.a.resize(D.nnz);
    if (!D.ia) return FGPU_OK;
    DEV_TRY(cudaMemcpyAsync(H.ia.data(), D.ia, (D.nrows + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    if (D.nnz) {
        DEV_TRY(cudaMemcpyAsync(H.ja.data(), D.ja, D.nnz * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
        DEV_TRY(cudaMemcpyAsync(H.a.data(), D.a, D.nnz * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    }
    DEV_TRY(cudaStreamSynchronize(ctx->stream));
    return FGPU_OK;
}

int amg_build_device(fgpu_ctx* ctx, const fgpu_matrix* Am, const AmgHostCfg& cfg, AmgDevHierarchy& H, const AmgNns* nns) {
    const auto t0 = std::chrono::steady_clock::now();
    const int max_levels = cfg.max_levels > 0 ? cfg.max_levels : 10;
    const int64_t coarse_lim = cfg.coarse_eq_lim > 0 ? cfg.coarse_eq_lim : 800;
    H.levels.clear();
    H.tail = AmgHierarchy();
    int* d_status = nullptr;
    DEV_TRY(cudaMalloc(&d_status, sizeof(int)));
    struct StatusFree {
        int* p;
        ~StatusFree() { cudaFree(p); }
    } status_free{d_status};
    DEV_TRY(cudaMemsetAsync(d_status, 0, sizeof(int), ctx->stream));
    H.levels.emplace_back();
    {
        AmgDevCsr& A0 = H.levels[0].A;               // a view of the matrix's own arrays
        A0.own = false;
        A0.nrows = A0.ncols = Am->nrows;
        A0.nnz = Am->nnz;
        A0.ia = Am->d_ia;
        A0.ja = Am->d_ja;
        A0.a = static_cast<double*>(Am->d_val);
    }
    H.times = AmgSetupTimes();
    AmgNns cur;
    if (nns) cur = *nns;
    bool last = false;
    int l = 0;
    for (; l + 1 < max_levels && !last; ++l) {
        AmgDevLevel& L = H.levels[l];
        if (L.A.nrows <= coarse_lim || L.A.nrows <= kHandoffRows || L.A.nnz >= ((int64_t)1 << 32)) break;
        AmgDevCsr Ac;
        AmgNns next;
        bool handoff = false;
        const int rc = level_dev(ctx, L, cfg, nns ? &cur : nullptr, &next, d_status, Ac, &handoff, &last, H.times);
        if (rc) return rc;
        if (handoff) {
            DEV_TRY(cudaStreamSynchronize(ctx->stream));
            L.P = AmgDevCsr();
            L.R = AmgDevCsr();
            L.agg.clear();
            L.lmax = 0;
            DEV_TRY(cudaMemsetAsync(d_status, 0, sizeof(int), ctx->stream));
            last = false;
            break;
        }
        H.levels.emplace_back();
        H.levels.back().A = std::move(Ac);
        if (nns) cur = std::move(next);
    }
    // the rest on the host, from level l (its operator copied)
    const auto t1 = std::chrono::steady_clock::now();
    HostCsr Al;
    int rc = amg_copy_to_host(ctx, H.levels[l].A, Al);
    if (rc) return rc;
    AmgHostCfg tc = cfg;
    tc.max_levels = last ? 1 : max_levels - l;
    std::string err;
    if (!amg_build_host(std::move(Al), tc, H.tail, err, nns ? &cur : nullptr)) { ctx->err = err; return FGPU_ERR_INVALID; }
    H.levels.resize(l);
    const auto t2 = std::chrono::steady_clock::now();
    H.times.total = std::chrono::duration<double, std::milli>(t2 - t0).count();
    H.times.tail = std::chrono::duration<double, std::milli>(t2 - t1).count();
    return FGPU_OK;
}

}  // namespace fgpu

namespace fgpu {

int amg_nns_from_cfg(fgpu_ctx* ctx, const fgpu_amg_cfg* cfg, int64_t n, AmgNns& nns, bool* has) {
    *has = false;
    if (!cfg || cfg->nns_count <= 0) return FGPU_OK;
    if (!cfg->nns || amg_nns_layout(cfg, n, nns)) { ctx->err = "gamg: invalid near null space (count, block size or vectors)"; return FGPU_ERR_INVALID; }
    std::vector<double> col(n);
    for (int j = 0; j < nns.m; ++j) {
        const fgpu_vector* v = cfg->nns[j];
        if (!v || v->n != n) { ctx->err = "gamg: a near null space vector does not match the matrix"; return FGPU_ERR_INVALID; }
        DEV_TRY(cudaMemcpyAsync(col.data(), v->d, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        DEV_TRY(cudaStreamSynchronize(ctx->stream));
        for (int64_t i = 0; i < n; ++i) nns.B[(size_t)i * nns.m + j] = col[i];
    }
    *has = true;
    return FGPU_OK;
}

}  // namespace fgpu

extern "C" int fgpu_space_rigid_body_modes(const fgpu_space* V, fgpu_vector* const* out) {
    using namespace fgpu;
    if (!V || !out) return FGPU_ERR_INVALID;
    fgpu_ctx* ctx = V->ctx;
    if (V->ncomp != 3 || V->mesh->cv != 4) { ctx->err = "rigid body modes: Pchv spaces on tetrahedral meshes only"; return FGPU_ERR_INVALID; }
    const int64_t nn = V->ndof / 3;
    for (int k = 0; k < 6; ++k)
        if (!out[k] || out[k]->n != V->ndof) { ctx->err = "rigid body modes: six vectors of the space's size"; return FGPU_ERR_INVALID; }
    std::vector<double> ref;
    if (!lagrange_nodes(V->order, ref) || (int)ref.size() != 3 * V->n) { ctx->err = "rigid body modes: orders 1-3"; return FGPU_ERR_INVALID; }
    std::vector<double> lam((size_t)V->n * 4);
    for (int a = 0; a < V->n; ++a) {                // barycentrics of the reference nodes ([-1, 1] reference tetrahedron)
        const double l1 = 0.5 * (1.0 + ref[a * 3]), l2 = 0.5 * (1.0 + ref[a * 3 + 1]), l3 = 0.5 * (1.0 + ref[a * 3 + 2]);
        lam[a * 4] = 1.0 - l1 - l2 - l3;
        lam[a * 4 + 1] = l1;
        lam[a * 4 + 2] = l2;
        lam[a * 4 + 3] = l3;
    }
    fgpu_mesh* M = V->mesh;
    if (M->h_xyz_stale) {
        DEV_TRY(cudaMemcpyAsync(M->h_xyz.data(), M->d_xyz, M->h_xyz.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        DEV_TRY(cudaStreamSynchronize(ctx->stream));
        M->h_xyz_stale = false;
    }
    double c[3] = {0.0, 0.0, 0.0};
    for (int64_t v = 0; v < M->nv; ++v)
        for (int d = 0; d < 3; ++d) c[d] += M->h_xyz[v * 3 + d];
    for (int d = 0; d < 3; ++d) c[d] /= (double)std::max<int64_t>(M->nv, 1);
    double *dlam = nullptr, *xn = nullptr;
    DEV_TRY(cudaMalloc(&dlam, lam.size() * sizeof(double)));
    struct Free { double*& a; double*& b; ~Free() { cudaFree(a); cudaFree(b); } } fr{dlam, xn};
    DEV_TRY(cudaMalloc(&xn, std::max<int64_t>(nn, 1) * 3 * sizeof(double)));
    DEV_TRY(cudaMemcpyAsync(dlam, lam.data(), lam.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    node_coords_kernel<<<grid_rows(nn, 256), 256, 0, ctx->stream>>>(nn, V->n, V->d_inc_ptr, V->d_inc, M->d_tets, M->d_xyz, dlam, xn);
    rbm_kernel<<<grid_rows(nn, 256), 256, 0, ctx->stream>>>(nn, xn, c[0], c[1], c[2], out[0]->d, out[1]->d, out[2]->d, out[3]->d,
                                                           out[4]->d, out[5]->d);
    ctx->launches += 2;
    DEV_TRY(cudaGetLastError());
    DEV_TRY(cudaStreamSynchronize(ctx->stream));
    return FGPU_OK;
}

// ---------------------------------------------------------------------------------------------------
// The device-built hierarchy copied into the host set-up's inspection object (fgpu_amg_host_*), so
// that it can be compared with fgpu_amg_host_build's level by level.
// ---------------------------------------------------------------------------------------------------
extern "C" int fgpu_amg_device_build(fgpu_ctx* ctx, const fgpu_matrix* A, const fgpu_amg_cfg* cfg, fgpu_amg_host** out) {
    using namespace fgpu;
    if (!ctx || !A || !out) return FGPU_ERR_INVALID;
    *out = nullptr;
    if (A->precision != FGPU_F64) { ctx->err = "gamg: FP64 matrices only"; return FGPU_ERR_INVALID; }
    if (ctx->capturing) { ctx->err = "gamg: set-up is not capturable"; return FGPU_ERR_INVALID; }
    const AmgHostCfg hc = amg_host_cfg(cfg, ctx->host_threads);
    AmgNns nns;
    bool has_nns = false;
    int rc = amg_nns_from_cfg(ctx, cfg, A->nrows, nns, &has_nns);
    if (rc) return rc;
    AmgDevHierarchy D;
    rc = amg_build_device(ctx, A, hc, D, has_nns ? &nns : nullptr);
    if (rc) return rc;
    fgpu_amg_host* h = new fgpu_amg_host();
    for (auto& dl : D.levels) {
        h->H.levels.emplace_back();
        AmgHostLevel& hl = h->H.levels.back();
        if ((rc = amg_copy_to_host(ctx, dl.A, hl.A)) || (rc = amg_copy_to_host(ctx, dl.P, hl.P)) ||
            (rc = amg_copy_to_host(ctx, dl.R, hl.R))) {
            delete h;
            return rc;
        }
        hl.agg = dl.agg;
        hl.lmax = dl.lmax;
    }
    for (auto& tl : D.tail.levels) h->H.levels.push_back(std::move(tl));
    h->H.coarse_inv.swap(D.tail.coarse_inv);
    h->device_levels = (int)D.levels.size();
    *out = h;
    return FGPU_OK;
}
