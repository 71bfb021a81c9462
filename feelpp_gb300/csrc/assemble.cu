// Device assembly kernels: per-element geometry, row-owner gather assembly of
// the CSR values (scalar Laplacian/mass and vector elasticity), load vector,
// strong Dirichlet rows.
//
// Formulation. On an affine tetrahedron the geometric map is constant, so the
// quadrature sum the reference evaluates per entry,
//     K_e(i,j) = sum_q w_q J (kappa (B ghat_j(q)).(B ghat_i(q)) + mass phi_j(q) phi_i(q))
// (feelpp/feel/feelvf/bilinearformcontext.hpp:552-590, pointsetquadrature.hpp:403-416),
// factors into 7 element coefficients times 7 reference tensors computed once
// with the same quadrature rule:
//     K_e = sum_k c_k T_k,  c = kappa J (G00, G11, G22, G01, G02, G12) (G = B^T B), c_6 = mass J.
// The result equals the quadrature form up to rounding.
//
// Scatter. Instead of adding element blocks into the CSR (MatSetValues
// ADD_VALUES, matrixpetsc.cpp:919-935), each CSR row is owned by one group of
// lanes which walks the elements containing the row's dof in increasing
// element order and sums the row of each element matrix into a shared-memory
// copy of the row; the row is then written once, coalesced. Every entry is
// summed in element insertion order, the order the reference adds into PETSc;
// no float atomics, deterministic.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "df64.h"
#include "fgpu_core.h"
#include "scan.cuh"
#include "asm_device.cuh"

namespace fgpu {

// ---------------------------------------------------------------------------
// Reference tables resident on the device, one copy per (device, order, degree).
// ---------------------------------------------------------------------------
static std::mutex g_tab_mutex;
static std::map<std::tuple<int, int, int>, DevTables*> g_tabs;

template <typename T>
static cudaError_t upload(const std::vector<T>& h, T** d) {
    cudaError_t e = cudaMalloc((void**)d, h.size() * sizeof(T));
    if (e != cudaSuccess) return e;
    return cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
}

DevTables* get_dev_tables(int order, int qdeg, std::string& err) {
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lock(g_tab_mutex);
    auto key = std::make_tuple(dev, order, qdeg);
    auto it = g_tabs.find(key);
    if (it != g_tabs.end()) return it->second;
    RefTables R;
    if (!build_ref_tables(order, qdeg, R, err)) return nullptr;
    DevTables* D = new DevTables();
    D->order = order; D->n = R.n; D->Q = R.Q; D->qdeg = qdeg;
    std::vector<float> T7f(R.T7.begin(), R.T7.end()), Sf(R.S.begin(), R.S.end());
    std::vector<float> T7h(R.T7.size()), T7l(R.T7.size());
    for (size_t k = 0; k < R.T7.size(); ++k) {
        T7h[k] = (float)R.T7[k];
        T7l[k] = (float)(R.T7[k] - (double)T7h[k]);
    }
    const int n = R.n, ntri = n * (n + 1) / 2;
    std::vector<float> T7th((size_t)7 * ntri), T7tl((size_t)7 * ntri);
    std::vector<uint16_t> tri((size_t)n * n);
    for (int i = 0, t = 0; i < n; ++i)
        for (int j = i; j < n; ++j, ++t) {
            tri[(size_t)i * n + j] = tri[(size_t)j * n + i] = (uint16_t)t;
            for (int k = 0; k < 7; ++k) {
                T7th[(size_t)k * ntri + t] = T7h[((size_t)k * n + i) * n + j];
                T7tl[(size_t)k * ntri + t] = T7l[((size_t)k * n + i) * n + j];
            }
        }
    std::vector<float> Sth((size_t)9 * ntri), Stl((size_t)9 * ntri);
    for (int i = 0, t = 0; i < n; ++i)
        for (int j = i; j < n; ++j, ++t)
            for (int ab = 0; ab < 9; ++ab) {
                const double v = R.S[((size_t)ab * n + i) * n + j];
                Sth[(size_t)ab * ntri + t] = (float)v;
                Stl[(size_t)ab * ntri + t] = (float)(v - (double)(float)v);
            }
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = upload(Sth, &D->d_Sth);
    if (e == cudaSuccess) e = upload(Stl, &D->d_Stl);
    if (e == cudaSuccess) e = upload(T7th, &D->d_T7th);
    if (e == cudaSuccess) e = upload(T7tl, &D->d_T7tl);
    if (e == cudaSuccess) e = upload(tri, &D->d_tri);
    if (e == cudaSuccess) e = upload(T7h, &D->d_T7h);
    if (e == cudaSuccess) e = upload(T7l, &D->d_T7l);
    if (e == cudaSuccess) e = upload(R.T7, &D->d_T7);
    if (e == cudaSuccess) e = upload(R.S, &D->d_S);
    if (e == cudaSuccess) e = upload(T7f, &D->d_T7f);
    if (e == cudaSuccess) e = upload(Sf, &D->d_Sf);
    if (e == cudaSuccess) e = upload(R.phi, &D->d_phi);
    if (e == cudaSuccess) e = upload(R.dphi, &D->d_dphi);
    if (e == cudaSuccess) e = upload(R.qx, &D->d_qx);
    if (e == cudaSuccess) e = upload(R.qw, &D->d_qw);
    if (e != cudaSuccess) {
        err = std::string("reference table upload: ") + cudaGetErrorString(e);
        delete D;
        return nullptr;
    }
    g_tabs[key] = D;
    return D;
}

// ---------------------------------------------------------------------------
// Profiling with CUDA events on the launch stream.
// ---------------------------------------------------------------------------
void prof_begin(fgpu_ctx* ctx, const char* name, PendingEvent& ev) {
    ++ctx->launches;
    if (!ctx->profile || ctx->capturing) return;
    ev.name = name;
    if (ctx->event_pool.size() >= 2) {
        ev.start = ctx->event_pool.back(); ctx->event_pool.pop_back();
        ev.stop = ctx->event_pool.back(); ctx->event_pool.pop_back();
    } else {
        cudaEventCreate(&ev.start);
        cudaEventCreate(&ev.stop);
    }
    cudaEventRecord(ev.start, ctx->stream);
}

void prof_end(fgpu_ctx* ctx, PendingEvent& ev) {
    if (!ctx->profile || ctx->capturing) return;
    cudaEventRecord(ev.stop, ctx->stream);
    ctx->pending.push_back(ev);
}

// ---------------------------------------------------------------------------
// Geometry: one thread per element (geomap.hpp:2310-2350, :1971-1991).
// Record layout (8 doubles) for the Laplacian/mass form:
//   [kappa J G00, kappa J G11, kappa J G22, kappa J G01, kappa J G02, kappa J G12, mass J, J]
// Record layout (16 doubles) for elasticity:
//   [B (9, row-major), G00, G11, G22, G01, G02, G12, J]
// ---------------------------------------------------------------------------
__global__ void geometry_kernel(int64_t nt, const double* __restrict__ xyz, const int32_t* __restrict__ tets, int kind,
                                const double* __restrict__ kappa, double kappa_c, double mass, double* __restrict__ coef,
                                int* __restrict__ status) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nt; e += (int64_t)gridDim.x * blockDim.x) {
        int4 t = *reinterpret_cast<const int4*>(tets + 4 * e);
        double x0 = xyz[3 * (int64_t)t.x], y0 = xyz[3 * (int64_t)t.x + 1], z0 = xyz[3 * (int64_t)t.x + 2];
        // K(r, c) = (X_{c+1} - X_0)[r] / 2
        double K[9];
        const int vv[3] = {t.y, t.z, t.w};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double* X = xyz + 3 * (int64_t)vv[c];
            K[0 * 3 + c] = 0.5 * X[0] - 0.5 * x0;
            K[1 * 3 + c] = 0.5 * X[1] - 0.5 * y0;
            K[2 * 3 + c] = 0.5 * X[2] - 0.5 * z0;
        }
        double c00 = K[4] * K[8] - K[5] * K[7];
        double c01 = K[5] * K[6] - K[3] * K[8];
        double c02 = K[3] * K[7] - K[4] * K[6];
        double det = K[0] * c00 + K[1] * c01 + K[2] * c02;
        double J = fabs(det);
        if (!(J > 0.0) || !isfinite(J)) atomicOr(status, kStatusBadElement);
        double cof[9] = {c00, c01, c02,
                         K[2] * K[7] - K[1] * K[8], K[0] * K[8] - K[2] * K[6], K[1] * K[6] - K[0] * K[7],
                         K[1] * K[5] - K[2] * K[4], K[2] * K[3] - K[0] * K[5], K[0] * K[4] - K[1] * K[3]};
        double B[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) B[i] = cof[i] / det;
        // G = B^T B
        double G[6];
        const int pa[6] = {0, 1, 2, 0, 0, 1}, pb[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
        for (int k = 0; k < 6; ++k)
            G[k] = B[0 * 3 + pa[k]] * B[0 * 3 + pb[k]] + B[1 * 3 + pa[k]] * B[1 * 3 + pb[k]] + B[2 * 3 + pa[k]] * B[2 * 3 + pb[k]];
        if (kind == FGPU_FORM_LAPLACE_MASS) {
            double kJ = (kappa ? kappa[e] : kappa_c) * J;
            double* o = coef + 8 * e;
            double2* o2 = reinterpret_cast<double2*>(o);
            o2[0] = make_double2(kJ * G[0], kJ * G[1]);
            o2[1] = make_double2(kJ * G[2], kJ * G[3]);
            o2[2] = make_double2(kJ * G[4], kJ * G[5]);
            o2[3] = make_double2(mass * J, J);
        } else {
            double* o = coef + 16 * e;
#pragma unroll
            for (int i = 0; i < 9; ++i) o[i] = B[i];
#pragma unroll
            for (int k = 0; k < 6; ++k) o[9 + k] = G[k];
            o[15] = J;
        }
    }
}

int launch_geometry(fgpu_ctx* ctx, const fgpu_mesh* mesh, int kind, const double* d_kappa, double kappa,
                    double mass, double lam, double mu, double* d_coef) {
    (void)lam; (void)mu;
    if (mesh->cv != 4) { ctx->err = "this operation takes tetrahedral meshes"; return FGPU_ERR_INVALID; }
    int threads = 256;
    int64_t blocks = (mesh->nt + threads - 1) / threads;
    if (blocks > 152 * 64) blocks = 152 * 64;
    if (blocks < 1) blocks = 1;
    PendingEvent ev;
    prof_begin(ctx, "geometry", ev);
    geometry_kernel<<<(int)blocks, threads, 0, ctx->stream>>>(mesh->nt, mesh->d_xyz, mesh->d_tets, kind, d_kappa, kappa,
                                                            mass, d_coef, ctx->d_status);
    prof_end(ctx, ev);
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

// ---------------------------------------------------------------------------
// Row-owner gather assembly, scalar forms.
// One group of G lanes owns one row (dof node) at a time. Shared memory holds
// the reference tensors (7 n n, compute type CT) and, per group, the row's
// column ids and accumulators.
// ---------------------------------------------------------------------------
template <int G>
__device__ __forceinline__ unsigned group_mask() {
    if (G >= 32) return 0xffffffffu;
    unsigned lane = threadIdx.x & 31u;
    return ((1u << (G & 31)) - 1u) << (lane / G * G);
}

__device__ __forceinline__ int lower_bound_s(const int32_t* a, int len, int32_t key) {
    int lo = 0, hi = len;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

template <typename CT>
__device__ __forceinline__ CT to_ct(double v) { return (CT)v; }

template <typename VT, typename CT, int N, int G>
__global__ void __launch_bounds__(256) gather_scalar_kernel(
    int64_t nrows, const int64_t* __restrict__ sia, const int32_t* __restrict__ sja,
    const int64_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc, const int32_t* __restrict__ l2n,
    const double* __restrict__ coef, const CT* __restrict__ T7g, int maxrow, VT* __restrict__ val, int accumulate,
    int* __restrict__ status) {
    extern __shared__ __align__(16) unsigned char smem[];
    CT* T7 = reinterpret_cast<CT*>(smem);
    constexpr int NT = 7 * N * N;
    for (int k = threadIdx.x; k < NT; k += blockDim.x) T7[k] = T7g[k];
    const int gpb = blockDim.x / G;
    const int g = threadIdx.x / G, lane = threadIdx.x % G;
    size_t t7bytes = ((size_t)NT * sizeof(CT) + 15) & ~(size_t)15;
    CT* acc = reinterpret_cast<CT*>(smem + t7bytes) + (size_t)g * maxrow;
    int32_t* cols = reinterpret_cast<int32_t*>(smem + t7bytes + (size_t)gpb * maxrow * sizeof(CT)) + (size_t)g * maxrow;
    __syncthreads();
    const unsigned mask = group_mask<G>();
    for (int64_t r = (int64_t)blockIdx.x * gpb + g; r < nrows; r += (int64_t)gridDim.x * gpb) {
        const int64_t start = sia[r];
        const int len = (int)(sia[r + 1] - start);
        if (len > maxrow) {
            if (lane == 0) atomicOr(status, kStatusRowOverflow);
            continue;
        }
        for (int k = lane; k < len; k += G) {
            cols[k] = sja[start + k];
            acc[k] = accumulate ? (CT)val[start + k] : (CT)0;
        }
        __syncwarp(mask);
        const int64_t tb = inc_ptr[r], te = inc_ptr[r + 1];
        for (int64_t t = tb; t < te; ++t) {
            const int32_t code = inc[t];
            const int64_t e = code >> 5;
            const int li = code & 31;
            if (lane < N) {
                const double2* cp = reinterpret_cast<const double2*>(coef + 8 * e);
                const double2 ca = __ldg(cp), cb = __ldg(cp + 1), cc = __ldg(cp + 2), cd = __ldg(cp + 3);
                const int32_t col = l2n[e * N + lane];
                const CT* tk = T7 + li * N + lane;
                CT v = to_ct<CT>(ca.x) * tk[0 * N * N];
                v += to_ct<CT>(ca.y) * tk[1 * N * N];
                v += to_ct<CT>(cb.x) * tk[2 * N * N];
                v += to_ct<CT>(cb.y) * tk[3 * N * N];
                v += to_ct<CT>(cc.x) * tk[4 * N * N];
                v += to_ct<CT>(cc.y) * tk[5 * N * N];
                v += to_ct<CT>(cd.x) * tk[6 * N * N];
                const int pos = lower_bound_s(cols, len, col);
                if (pos < len && cols[pos] == col) acc[pos] += v;
                else atomicOr(status, kStatusMissingEntry);
            }
            __syncwarp(mask);
        }
        for (int k = lane; k < len; k += G) val[start + k] = (VT)acc[k];
        __syncwarp(mask);
    }
}

// Vector elasticity (Pchv, ncomp = 3). A group owns the 3 component rows of a
// dof node. For element e (local index li of the node) and lane j, the 3x3
// block K[(c,li),(d,j)] = J (lambda Y_cd + mu Y_dc + mu delta_cd tr(G X)),
// X_ab = S_ab(li, j), Y = B X B^T, is the quadrature sum of
// lambda div u div v + 2 mu eps(u):eps(v) (qs_elasticity.cpp:46-63) written
// with the reference tensors S_ab = sum_q w_q d_a phi_i d_b phi_j.
template <typename VT, typename CT, int N, int G>
__global__ void __launch_bounds__(256) gather_elasticity_kernel(
    int64_t nnodes, const int64_t* __restrict__ sia, const int32_t* __restrict__ sja,
    const int64_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc, const int32_t* __restrict__ l2n,
    const double* __restrict__ coef, const CT* __restrict__ Sg, double lam, double mu, int maxrow,
    VT* __restrict__ val, int accumulate, int* __restrict__ status) {
    extern __shared__ __align__(16) unsigned char smem[];
    CT* S = reinterpret_cast<CT*>(smem);
    constexpr int NS = 9 * N * N;
    for (int k = threadIdx.x; k < NS; k += blockDim.x) S[k] = Sg[k];
    const int gpb = blockDim.x / G;
    const int g = threadIdx.x / G, lane = threadIdx.x % G;
    size_t sbytes = ((size_t)NS * sizeof(CT) + 15) & ~(size_t)15;
    CT* acc = reinterpret_cast<CT*>(smem + sbytes) + (size_t)g * 9 * maxrow;   // [3][3*maxrow]
    int32_t* cols = reinterpret_cast<int32_t*>(smem + sbytes + (size_t)gpb * 9 * maxrow * sizeof(CT)) + (size_t)g * maxrow;
    __syncthreads();
    const unsigned mask = group_mask<G>();
    for (int64_t m = (int64_t)blockIdx.x * gpb + g; m < nnodes; m += (int64_t)gridDim.x * gpb) {
        const int64_t sstart = sia[m];
        const int len = (int)(sia[m + 1] - sstart);
        if (len > maxrow) {
            if (lane == 0) atomicOr(status, kStatusRowOverflow);
            continue;
        }
        const int64_t row0 = 9 * sstart;  // start of row 3m: 9 * sia[m]; row 3m+c starts at row0 + c*3*len
        for (int k = lane; k < len; k += G) cols[k] = sja[sstart + k];
        for (int k = lane; k < 9 * len; k += G) acc[k] = accumulate ? (CT)val[row0 + k] : (CT)0;
        __syncwarp(mask);
        for (int64_t t = inc_ptr[m]; t < inc_ptr[m + 1]; ++t) {
            const int32_t code = inc[t];
            const int64_t e = code >> 5;
            const int li = code & 31;
            if (lane < N) {
                const double* cr = coef + 16 * e;
                CT B[9], Gm[6];
#pragma unroll
                for (int i = 0; i < 9; ++i) B[i] = (CT)__ldg(cr + i);
#pragma unroll
                for (int i = 0; i < 6; ++i) Gm[i] = (CT)__ldg(cr + 9 + i);
                const CT J = (CT)__ldg(cr + 15);
                CT X[9];
#pragma unroll
                for (int ab = 0; ab < 9; ++ab) X[ab] = S[(ab * N + li) * N + lane];
                // Z = X B^T : Z_ad = sum_b X_ab B_db ; Y = B Z : Y_cd = sum_a B_ca Z_ad
                CT Z[9], Y[9];
#pragma unroll
                for (int a = 0; a < 3; ++a)
#pragma unroll
                    for (int d = 0; d < 3; ++d) Z[a * 3 + d] = X[a * 3 + 0] * B[d * 3 + 0] + X[a * 3 + 1] * B[d * 3 + 1] + X[a * 3 + 2] * B[d * 3 + 2];
#pragma unroll
                for (int c = 0; c < 3; ++c)
#pragma unroll
                    for (int d = 0; d < 3; ++d) Y[c * 3 + d] = B[c * 3 + 0] * Z[0 * 3 + d] + B[c * 3 + 1] * Z[1 * 3 + d] + B[c * 3 + 2] * Z[2 * 3 + d];
                CT tr = Gm[0] * X[0] + Gm[1] * X[4] + Gm[2] * X[8] + Gm[3] * (X[1] + X[3]) + Gm[4] * (X[2] + X[6]) + Gm[5] * (X[5] + X[7]);
                const CT lJ = (CT)lam * J, mJ = (CT)mu * J;
                const int32_t col = l2n[e * N + lane];
                const int pos = lower_bound_s(cols, len, col);
                if (pos < len && cols[pos] == col) {
#pragma unroll
                    for (int c = 0; c < 3; ++c)
#pragma unroll
                        for (int d = 0; d < 3; ++d) {
                            CT v = lJ * Y[c * 3 + d] + mJ * Y[d * 3 + c];
                            if (c == d) v += mJ * tr;
                            acc[c * 3 * len + 3 * pos + d] += v;
                        }
                } else {
                    atomicOr(status, kStatusMissingEntry);
                }
            }
            __syncwarp(mask);
        }
        for (int k = lane; k < 9 * len; k += G) val[row0 + k] = (VT)acc[k];
        __syncwarp(mask);
    }
}

template <typename VT, typename CT, int N, int G>
static int run_gather_scalar(fgpu_ctx* ctx, fgpu_matrix* A, const CT* T7, const double* d_coef, int accumulate) {
    const DevPattern& P = *A->pattern;
    const fgpu_space* V = A->space;
    const int threads = 256, gpb = threads / G;
    size_t t7bytes = ((size_t)7 * N * N * sizeof(CT) + 15) & ~(size_t)15;
    size_t smem = t7bytes + (size_t)gpb * P.max_row * (sizeof(CT) + sizeof(int32_t));
    auto kern = gather_scalar_kernel<VT, CT, N, G>;
    if (smem > 48 * 1024) FGPU_CUDA_CHECK(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (smem > 227 * 1024) { ctx->err = "pattern rows too long for the gather kernel"; return FGPU_ERR_INVALID; }
    int per_sm = 0;
    FGPU_CUDA_CHECK(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem));
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    int64_t need = (P.nrows + gpb - 1) / gpb;
    int64_t blocks = std::min<int64_t>(need, (int64_t)std::max(per_sm, 1) * sms);
    if (blocks < 1) blocks = 1;
    PendingEvent ev;
    prof_begin(ctx, "assemble_gather", ev);
    kern<<<(int)blocks, threads, smem, ctx->stream>>>(P.nrows, P.d_ia, P.d_ja, V->d_inc_ptr, V->d_inc, V->d_l2n, d_coef,
                                                      T7, P.max_row, reinterpret_cast<VT*>(A->d_val), accumulate,
                                                      ctx->d_status);
    prof_end(ctx, ev);
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

template <typename VT, typename CT, int N, int G>
static int run_gather_elasticity(fgpu_ctx* ctx, fgpu_matrix* A, const CT* S, const double* d_coef, double lam,
                                 double mu, int accumulate) {
    const DevPattern& P = *A->pattern;
    const fgpu_space* V = A->space;
    const int threads = 256, gpb = threads / G;
    size_t sbytes = ((size_t)9 * N * N * sizeof(CT) + 15) & ~(size_t)15;
    size_t smem = sbytes + (size_t)gpb * P.max_row * (9 * sizeof(CT) + sizeof(int32_t));
    auto kern = gather_elasticity_kernel<VT, CT, N, G>;
    if (smem > 227 * 1024) { ctx->err = "pattern rows too long for the elasticity gather kernel"; return FGPU_ERR_INVALID; }
    if (smem > 48 * 1024) FGPU_CUDA_CHECK(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    FGPU_CUDA_CHECK(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem));
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    int64_t need = (P.nrows + gpb - 1) / gpb;
    int64_t blocks = std::min<int64_t>(need, (int64_t)std::max(per_sm, 1) * sms);
    if (blocks < 1) blocks = 1;
    PendingEvent ev;
    prof_begin(ctx, "assemble_gather_elasticity", ev);
    kern<<<(int)blocks, threads, smem, ctx->stream>>>(P.nrows, P.d_ia, P.d_ja, V->d_inc_ptr, V->d_inc, V->d_l2n, d_coef, S,
                                                      lam, mu, P.max_row, reinterpret_cast<VT*>(A->d_val), accumulate,
                                                      ctx->d_status);
    prof_end(ctx, ev);
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

int launch_assemble_gather(fgpu_ctx* ctx, fgpu_matrix* A, const DevTables* tab, int kind, const double* d_coef,
                           int accumulate) {
    const int order = A->space->order;
    const bool f32 = A->precision == FGPU_F32;
    if (kind == FGPU_FORM_LAPLACE_MASS) {
        if (A->ncomp != 1) { ctx->err = "Laplace/mass form needs a scalar space"; return FGPU_ERR_INVALID; }
        if (order == 1) return f32 ? run_gather_scalar<float, float, 4, 8>(ctx, A, tab->d_T7f, d_coef, accumulate)
                                   : run_gather_scalar<double, double, 4, 8>(ctx, A, tab->d_T7, d_coef, accumulate);
        if (order == 2) return f32 ? run_gather_scalar<float, float, 10, 16>(ctx, A, tab->d_T7f, d_coef, accumulate)
                                   : run_gather_scalar<double, double, 10, 16>(ctx, A, tab->d_T7, d_coef, accumulate);
        if (order == 3) return f32 ? run_gather_scalar<float, float, 20, 32>(ctx, A, tab->d_T7f, d_coef, accumulate)
                                   : run_gather_scalar<double, double, 20, 32>(ctx, A, tab->d_T7, d_coef, accumulate);
    }
    ctx->err = "unsupported form/order";
    return FGPU_ERR_INVALID;
}

int launch_assemble_elasticity(fgpu_ctx* ctx, fgpu_matrix* A, const DevTables* tab, const double* d_coef, double lam,
                               double mu, int accumulate) {
    const int order = A->space->order;
    const bool f32 = A->precision == FGPU_F32;
    if (A->ncomp != 3) { ctx->err = "elasticity needs a 3-component space"; return FGPU_ERR_INVALID; }
    if (order == 1) return f32 ? run_gather_elasticity<float, float, 4, 8>(ctx, A, tab->d_Sf, d_coef, lam, mu, accumulate)
                               : run_gather_elasticity<double, double, 4, 8>(ctx, A, tab->d_S, d_coef, lam, mu, accumulate);
    if (order == 2) return f32 ? run_gather_elasticity<float, float, 10, 16>(ctx, A, tab->d_Sf, d_coef, lam, mu, accumulate)
                               : run_gather_elasticity<double, double, 10, 16>(ctx, A, tab->d_S, d_coef, lam, mu, accumulate);
    ctx->err = "elasticity supports P1 and P2";
    return FGPU_ERR_INVALID;
}

// ---------------------------------------------------------------------------
// Load vector (linearformcontext.hpp:305, 395-410): element values into a
// work buffer, then a per-node gather in element order (no float atomics).
// ---------------------------------------------------------------------------
template <int N>
__global__ void rhs_element_kernel(int64_t nt, const double* __restrict__ xyz, const int32_t* __restrict__ tets, int ncomp,
                                   int Q, const double* __restrict__ qx, const double* __restrict__ qw,
                                   const double* __restrict__ phi, int fkind, double f0, double f1, double f2,
                                   double* __restrict__ work) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nt; e += (int64_t)gridDim.x * blockDim.x) {
        int4 t = *reinterpret_cast<const int4*>(tets + 4 * e);
        double X[4][3];
        const int vv[4] = {t.x, t.y, t.z, t.w};
#pragma unroll
        for (int v = 0; v < 4; ++v)
#pragma unroll
            for (int d = 0; d < 3; ++d) X[v][d] = xyz[3 * (int64_t)vv[v] + d];
        double K[9];
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int r = 0; r < 3; ++r) K[r * 3 + c] = 0.5 * X[c + 1][r] - 0.5 * X[0][r];
        double det = K[0] * (K[4] * K[8] - K[5] * K[7]) + K[1] * (K[5] * K[6] - K[3] * K[8]) + K[2] * (K[3] * K[7] - K[4] * K[6]);
        double J = fabs(det);
        double F[3][N];
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int i = 0; i < N; ++i) F[c][i] = 0.0;
        for (int q = 0; q < Q; ++q) {
            double xh = qx[3 * q], yh = qx[3 * q + 1], zh = qx[3 * q + 2];
            double g0 = -0.5 * (1 + xh + yh + zh), g1 = 0.5 * (1 + xh), g2 = 0.5 * (1 + yh), g3 = 0.5 * (1 + zh);
            double p[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) p[d] = X[0][d] * g0 + X[1][d] * g1 + X[2][d] * g2 + X[3][d] * g3;
            double wJ = qw[q] * J;
            double fv[3];
            if (fkind == FGPU_RHS_SINE) {
                const double pi = 3.141592653589793;
                fv[0] = 3.0 * pi * pi * sin(pi * p[0]) * sin(pi * p[1]) * sin(pi * p[2]);
                fv[1] = fv[2] = 0.0;
            } else if (fkind == FGPU_RHS_CONST_VEC) {
                fv[0] = f0; fv[1] = f1; fv[2] = f2;
            } else {
                fv[0] = f0; fv[1] = fv[2] = 0.0;
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                if (c >= ncomp) break;
                double s = wJ * fv[c];
#pragma unroll
                for (int i = 0; i < N; ++i) F[c][i] += s * phi[q * N + i];
            }
        }
        for (int c = 0; c < ncomp; ++c)
#pragma unroll
            for (int i = 0; i < N; ++i) work[(e * ncomp + c) * N + i] = F[c][i];
    }
}

__global__ void rhs_gather_kernel(int64_t nnodes, int N, int ncomp, const int64_t* __restrict__ inc_ptr,
                                  const int32_t* __restrict__ inc, const double* __restrict__ work,
                                  double* __restrict__ out, int accumulate) {
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < nnodes; m += (int64_t)gridDim.x * blockDim.x) {
        for (int c = 0; c < ncomp; ++c) {
            double s = accumulate ? out[m * ncomp + c] : 0.0;
            for (int64_t t = inc_ptr[m]; t < inc_ptr[m + 1]; ++t) {
                int32_t code = inc[t];
                int64_t e = code >> 5;
                int li = code & 31;
                s += work[(e * ncomp + c) * N + li];
            }
            out[m * ncomp + c] = s;
        }
    }
}

int launch_rhs(fgpu_ctx* ctx, const fgpu_space* V, const DevTables* tab, int fkind, const double* fc, double* d_out,
               int accumulate, double* d_work) {
    const fgpu_mesh* M = V->mesh;
    int threads = 128;
    int64_t blocks = std::min<int64_t>((M->nt + threads - 1) / threads, 152 * 32);
    if (blocks < 1) blocks = 1;
    PendingEvent ev;
    prof_begin(ctx, "rhs_element", ev);
    switch (V->n) {
        case 4: rhs_element_kernel<4><<<(int)blocks, threads, 0, ctx->stream>>>(M->nt, M->d_xyz, M->d_tets, V->ncomp, tab->Q, tab->d_qx, tab->d_qw, tab->d_phi, fkind, fc[0], fc[1], fc[2], d_work); break;
        case 10: rhs_element_kernel<10><<<(int)blocks, threads, 0, ctx->stream>>>(M->nt, M->d_xyz, M->d_tets, V->ncomp, tab->Q, tab->d_qx, tab->d_qw, tab->d_phi, fkind, fc[0], fc[1], fc[2], d_work); break;
        case 20: rhs_element_kernel<20><<<(int)blocks, threads, 0, ctx->stream>>>(M->nt, M->d_xyz, M->d_tets, V->ncomp, tab->Q, tab->d_qx, tab->d_qw, tab->d_phi, fkind, fc[0], fc[1], fc[2], d_work); break;
        default: ctx->err = "unsupported order"; return FGPU_ERR_INVALID;
    }
    prof_end(ctx, ev);
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    int64_t nn = V->topo.nnodes;
    int64_t gb = std::min<int64_t>((nn + 255) / 256, 152 * 16);
    if (gb < 1) gb = 1;
    PendingEvent ev2;
    prof_begin(ctx, "rhs_gather", ev2);
    rhs_gather_kernel<<<(int)gb, 256, 0, ctx->stream>>>(nn, V->n, V->ncomp, V->d_inc_ptr, V->d_inc, d_work, d_out, accumulate);
    prof_end(ctx, ev2);
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

// Same two load-vector kernels launched on an explicit stream with caller-given
// tables and work buffer (used by the allocation-free entry point). Tetrahedral
// P1-P3 spaces only; on failure `err` says why (the CUDA error of the launch, or
// the unsupported local size).
int launch_rhs_raw(cudaStream_t stream, const fgpu_space* V, int Q, const double* qx, const double* qw,
                   const double* phi, int fkind, const double* fc, double* d_out, int accumulate, double* d_work,
                   std::string& err) {
    const fgpu_mesh* M = V->mesh;
    int threads = 128;
    int64_t blocks = std::min<int64_t>((M->nt + threads - 1) / threads, 152 * 32);
    if (blocks < 1) blocks = 1;
    switch (V->n) {
        case 4: rhs_element_kernel<4><<<(int)blocks, threads, 0, stream>>>(M->nt, M->d_xyz, M->d_tets, V->ncomp, Q, qx, qw, phi, fkind, fc[0], fc[1], fc[2], d_work); break;
        case 10: rhs_element_kernel<10><<<(int)blocks, threads, 0, stream>>>(M->nt, M->d_xyz, M->d_tets, V->ncomp, Q, qx, qw, phi, fkind, fc[0], fc[1], fc[2], d_work); break;
        case 20: rhs_element_kernel<20><<<(int)blocks, threads, 0, stream>>>(M->nt, M->d_xyz, M->d_tets, V->ncomp, Q, qx, qw, phi, fkind, fc[0], fc[1], fc[2], d_work); break;
        default:
            err = "load vector: " + std::to_string(V->n) + " local dofs per component (P1-P3 tetrahedra have 4, 10 or 20)";
            return FGPU_ERR_INVALID;
    }
    cudaError_t ce = cudaGetLastError();
    if (ce != cudaSuccess) { err = std::string("load-vector element kernel: ") + cudaGetErrorString(ce); return FGPU_ERR_CUDA; }
    int64_t nn = V->topo.nnodes;
    int64_t gb = std::min<int64_t>((nn + 255) / 256, 152 * 16);
    if (gb < 1) gb = 1;
    rhs_gather_kernel<<<(int)gb, 256, 0, stream>>>(nn, V->n, V->ncomp, V->d_inc_ptr, V->d_inc, d_work, d_out, accumulate);
    ce = cudaGetLastError();
    if (ce != cudaSuccess) { err = std::string("load-vector gather kernel: ") + cudaGetErrorString(ce); return FGPU_ERR_CUDA; }
    return FGPU_OK;
}

// ---------------------------------------------------------------------------
// Strong Dirichlet (MatrixPetsc::zeroRows, matrixpetsc.cpp:1762-1860); the
// pattern is kept (MAT_KEEP_NONZERO_PATTERN). One warp per group of 32
// consecutive rows; its lanes sweep the group's entries flat, U chunks of 32
// at a time, with the column reads of the next U chunks in flight while the
// mask reads, row lookups and value reads of these are made. Each entry's row
// comes from a binary search over the row starts held one per lane (the U
// searches interleaved). In the symmetric mode a kept row subtracts the
// A_ij g_j of its eliminated columns from its right-hand side in column order,
// the lane that owns the row reading them from a per-warp shared buffer one
// after another, as a single thread walking the row would. Measured at P2 64^3
// (symmetric mode, boundary rows): 0.21 ms with U = 3 (U = 2: 0.33, U = 4: 0.22,
// U = 8: 0.25 ms, 122 registers); a thread per row walking its own row took
// 0.69 ms, a warp per row 0.67 ms, this sweep without the prefetch, with one
// row search and one value read per chunk and the subtractions shuffled one
// lane at a time, 0.48 ms.
// ---------------------------------------------------------------------------
template <typename VT, int U = 3>
__global__ void __launch_bounds__(256) dirichlet_kernel(int64_t nrows, const int64_t* __restrict__ ia,
                                                        const int32_t* __restrict__ ja, VT* __restrict__ val,
                                                        double* __restrict__ rhs, const uint8_t* __restrict__ mask,
                                                        const double* __restrict__ g, int mode, double diag) {
    constexpr unsigned kAll = 0xffffffffu;
    __shared__ double2 hitbuf[8][32];                   // per warp: (A_ij, g_j) of one chunk's eliminated columns
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const bool sym = mode == FGPU_ON_ELIMINATION_SYMMETRIC, keep = mode == FGPU_ON_ELIMINATION_KEEP_DIAGONAL;
    const int64_t ngroups = (nrows + 31) >> 5;
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t grp = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib; grp < ngroups; grp += nw) {
        const int64_t r0 = grp << 5;
        const int cnt = (int)(nrows - r0 < 32 ? nrows - r0 : 32);
        const bool own = lane < cnt;                     // lane owns row r0 + lane
        const int64_t base = ia[r0], end = ia[r0 + cnt];
        const int off = own ? (int)(ia[r0 + lane] - base) : INT_MAX;       // the row's entries: [off, offn)
        const int offn = own ? (int)(ia[r0 + lane + 1] - base) : INT_MAX;
        const bool mrow = own && mask[r0 + lane] != 0;
        double s = (sym && own && rhs) ? rhs[r0 + lane] : 0.0;
        const unsigned mrows = __ballot_sync(kAll, mrow);
        if (!mrows && !sym) continue;                    // no eliminated row, nothing else to do
        const int len = (int)(end - base);
        bool touched = false;
        unsigned mydiag = 0;                             // rows whose diagonal entry this lane wrote
        int32_t cn[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int q = 32 * u + lane;
            cn[u] = q < len ? ja[base + q] : -1;
        }
        for (int q0 = 0; q0 < len; q0 += 32 * U) {
            int32_t c[U];
#pragma unroll
            for (int u = 0; u < U; ++u) c[u] = cn[u];
            const int q1 = q0 + 32 * U;
            if (q1 < len) {
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int q = q1 + 32 * u + lane;
                    cn[u] = q < len ? ja[base + q] : -1;
                }
            }
            unsigned hm = 0;                             // chunks whose entry is in an eliminated column
            if (sym) {
#pragma unroll
                for (int u = 0; u < U; ++u)
                    if (c[u] >= 0 && mask[c[u]]) hm |= 1u << u;
            }
            const bool ov = mrow && off < q1 && offn > q0;
            if (!__any_sync(kAll, ov || hm != 0)) continue;
            int k[U];                                    // each entry's row: the last row start <= q
#pragma unroll
            for (int u = 0; u < U; ++u) k[u] = 0;
#pragma unroll
            for (int st = 16; st; st >>= 1) {
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int t = __shfl_sync(kAll, off, k[u] + st);
                    if (t <= q0 + 32 * u + lane) k[u] += st;
                }
            }
            unsigned inm = 0, dgm = 0, hh = 0;
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const bool in = c[u] >= 0 && ((mrows >> k[u]) & 1u);
                if (in) inm |= 1u << u;
                if (in && c[u] == r0 + k[u]) dgm |= 1u << u;
                if (((hm >> u) & 1u) && !in) hh |= 1u << u;
            }
            const unsigned rd = hh | (keep ? dgm : 0u);
            double v[U], gc[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int64_t p = base + q0 + 32 * u + lane;
                v[u] = ((rd >> u) & 1u) ? (double)val[p] : 0.0;
                gc[u] = (((hh >> u) & 1u) && g) ? g[c[u]] : 0.0;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (!((inm >> u) & 1u)) continue;
                const int64_t p = base + q0 + 32 * u + lane, r = r0 + k[u];
                const bool dg = (dgm >> u) & 1u;
                if (keep) {
                    if (!dg) val[p] = (VT)0;
                    else if (rhs) rhs[r] = v[u] * (g ? g[r] : 0.0);
                } else {
                    val[p] = dg ? (VT)diag : (VT)0;
                    if (dg && rhs) rhs[r] = diag * (g ? g[r] : 0.0);
                }
                if (dg) mydiag |= 1u << k[u];
            }
            if (!__any_sync(kAll, hh != 0)) continue;
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const unsigned bal = __ballot_sync(kAll, (hh >> u) & 1u);
                if (!bal) continue;
                if ((hh >> u) & 1u) {
                    hitbuf[wib][lane] = make_double2(v[u], gc[u]);
                    val[base + q0 + 32 * u + lane] = (VT)0;
                }
                __syncwarp();
                if (own && !mrow) {                      // this chunk's eliminated columns of the lane's row
                    const int qs = q0 + 32 * u;
                    const int lo = off - qs > 0 ? off - qs : 0, hi = offn - qs < 32 ? offn - qs : 32;
                    if (lo < hi) {
                        unsigned mine = bal & (hi == 32 ? kAll : (1u << hi) - 1u) & ~((1u << lo) - 1u);
                        while (mine) {
                            const int j = __ffs(mine) - 1;
                            mine &= mine - 1;
                            const double2 e = hitbuf[wib][j];
                            s -= e.x * e.y;
                            touched = true;
                        }
                    }
                }
                __syncwarp();
            }
        }
        if (rhs && touched) rhs[r0 + lane] = s;
        const unsigned diagrows = __reduce_or_sync(kAll, mydiag);
        if (rhs && mrow && !((diagrows >> lane) & 1u))  // an eliminated row without a diagonal entry
            rhs[r0 + lane] = (keep ? 0.0 : diag) * (g ? g[r0 + lane] : 0.0);
    }
}

int launch_dirichlet(fgpu_ctx* ctx, fgpu_matrix* A, double* d_rhs, const uint8_t* d_mask, const double* d_g, int mode,
                     double diag) {
    int64_t blocks = std::min<int64_t>((A->nrows + 255) / 256, 152 * 16);   // 8 groups of 32 rows per block
    if (blocks < 1) blocks = 1;
    PendingEvent ev;
    prof_begin(ctx, "dirichlet", ev);
    if (A->precision == FGPU_F32)
        dirichlet_kernel<float><<<(int)blocks, 256, 0, ctx->stream>>>(A->nrows, A->d_ia, A->d_ja, (float*)A->d_val, d_rhs,
                                                                      d_mask, d_g, mode, diag);
    else
        dirichlet_kernel<double><<<(int)blocks, 256, 0, ctx->stream>>>(A->nrows, A->d_ia, A->d_ja, (double*)A->d_val, d_rhs,
                                                                       d_mask, d_g, mode, diag);
    prof_end(ctx, ev);
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

// ---------------------------------------------------------------------------
// Expanded (component) CSR of a vector space from its node pattern: row 3m+c
// holds columns 3n+d for the neighbours n of m (ascending), d = 0..2.
// ---------------------------------------------------------------------------
__global__ void expand_ia_kernel(int64_t nnodes, int nc, const int64_t* __restrict__ sia, int64_t* __restrict__ ia) {
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m <= nnodes; m += (int64_t)gridDim.x * blockDim.x) {
        if (m == nnodes) { ia[nnodes * nc] = (int64_t)nc * nc * sia[nnodes]; continue; }
        int64_t len = sia[m + 1] - sia[m];
        for (int c = 0; c < nc; ++c) ia[m * nc + c] = (int64_t)nc * nc * sia[m] + c * nc * len;
    }
}
__global__ void expand_ja_kernel(int64_t nnodes, int nc, const int64_t* __restrict__ sia, const int32_t* __restrict__ sja,
                                 int32_t* __restrict__ ja) {
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < nnodes; m += (int64_t)gridDim.x * blockDim.x) {
        int64_t b = sia[m], len = sia[m + 1] - b;
        for (int c = 0; c < nc; ++c) {
            int64_t o = (int64_t)nc * nc * b + c * nc * len;
            for (int64_t k = 0; k < len; ++k)
                for (int d = 0; d < nc; ++d) ja[o + k * nc + d] = sja[b + k] * nc + d;
        }
    }
}

int launch_expand_pattern(fgpu_ctx* ctx, const DevPattern& P, int nc, int64_t* d_ia, int32_t* d_ja) {
    int64_t blocks = std::min<int64_t>((P.nrows + 256) / 256, 152 * 16);
    expand_ia_kernel<<<(int)blocks, 256, 0, ctx->stream>>>(P.nrows, nc, P.d_ia, d_ia);
    expand_ja_kernel<<<(int)blocks, 256, 0, ctx->stream>>>(P.nrows, nc, P.d_ia, P.d_ja, d_ja);
    ctx->launches += 2;
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

template <typename A, typename B>
__global__ void convert_kernel(int64_t n, const A* __restrict__ a, B* __restrict__ b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (B)a[i];
}

int launch_convert_values(fgpu_ctx* ctx, const fgpu_matrix* src, fgpu_matrix* dst) {
    int64_t n = src->nnz;
    int64_t blocks = std::min<int64_t>((n + 255) / 256, 152 * 32);
    if (blocks < 1) blocks = 1;
    PendingEvent ev;
    prof_begin(ctx, "convert_values", ev);
    if (src->precision == FGPU_F64 && dst->precision == FGPU_F32)
        convert_kernel<double, float><<<(int)blocks, 256, 0, ctx->stream>>>(n, (const double*)src->d_val, (float*)dst->d_val);
    else if (src->precision == FGPU_F32 && dst->precision == FGPU_F64)
        convert_kernel<float, double><<<(int)blocks, 256, 0, ctx->stream>>>(n, (const float*)src->d_val, (double*)dst->d_val);
    else
        FGPU_CUDA_CHECK(ctx, cudaMemcpyAsync(dst->d_val, src->d_val, n * (src->precision == FGPU_F32 ? 4 : 8),
                                             cudaMemcpyDeviceToDevice, ctx->stream));
    prof_end(ctx, ev);
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

}  // namespace fgpu

// ===========================================================================
// FP64-accurate assembly on the FP32 pipes (df64) and the pure FP32 path.
// ===========================================================================
namespace fgpu {

// Element e's coefficient record into rec + 4 e (geometry_df_record, asm_device.cuh).
__device__ __forceinline__ void geometry_df_element(int64_t e, const double* __restrict__ xyz, const int32_t* __restrict__ tets,
                                                    const double* __restrict__ kappa, df kc, df mc, df ksc,
                                                    float4* __restrict__ rec, int* __restrict__ status) {
    geometry_df_record(e, xyz, tets, kappa, kc, mc, ksc, rec + 4 * e, status);
}

// kscale (device scalar or null): time-dependent factor of the stiffness
// coefficient, read at run time so that captured graphs see its new value.
__global__ void geometry_df_kernel(int64_t nt, const double* __restrict__ xyz, const int32_t* __restrict__ tets,
                                   const double* __restrict__ kappa, double kappa_c, double mass, const double* __restrict__ kscale,
                                   float4* __restrict__ rec, int* __restrict__ status) {
    const df kc = d2df(kappa_c), mc = d2df(mass);
    const df ksc = kscale ? d2df(*kscale) : df{1.0f, 0.0f};
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nt; e += (int64_t)gridDim.x * blockDim.x)
        geometry_df_element(e, xyz, tets, kappa, kc, mc, ksc, rec, status);
}

int launch_geometry_df(fgpu_ctx* ctx, const fgpu_mesh* mesh, const double* d_kappa, double kappa, double mass,
                       float4* d_rec, const double* d_kscale) {
    if (mesh->cv != 4) { ctx->err = "this operation takes tetrahedral meshes"; return FGPU_ERR_INVALID; }
    int threads = 256;
    int64_t blocks = std::min<int64_t>((mesh->nt + threads - 1) / threads, 152 * 16);
    if (blocks < 1) blocks = 1;
    PendingEvent ev;
    prof_begin(ctx, "geometry", ev);
    geometry_df_kernel<<<(int)blocks, threads, 0, ctx->stream>>>(mesh->nt, mesh->d_xyz, mesh->d_tets, d_kappa, kappa, mass,
                                                               d_kscale, d_rec, ctx->d_status);
    prof_end(ctx, ev);
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

// Position table: pos[(e n + i) n + j] = offset of node l2n[e][j] inside the
// pattern row of node l2n[e][i] (rows are at most 255 long). Built once per pattern.
__global__ void positions_kernel(int64_t nt, int n, const int32_t* __restrict__ l2n, const int64_t* __restrict__ ia,
                                 const int32_t* __restrict__ ja, uint8_t* __restrict__ pos, int* __restrict__ status) {
    const int64_t total = nt * n * n;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = t / (n * n);
        const int ij = (int)(t - e * n * n);
        const int i = ij / n, j = ij - i * n;
        const int32_t row = l2n[e * n + i], col = l2n[e * n + j];
        const int64_t b = ia[row];
        int lo = 0, hi = (int)(ia[row + 1] - b);
        while (lo < hi) {
            int mid = (lo + hi) >> 1;
            if (ja[b + mid] < col) lo = mid + 1; else hi = mid;
        }
        if (lo >= (int)(ia[row + 1] - b) || ja[b + lo] != col || lo > 255) {
            atomicOr(status, kStatusMissingEntry);
            lo = 0;
        }
        pos[t] = (uint8_t)lo;
    }
}

int launch_build_positions(fgpu_ctx* ctx, fgpu_space* V) {
    if (V->d_pos) return FGPU_OK;
    const int64_t total = V->mesh->nt * (int64_t)V->n * V->n;
    // 64 bytes of padding: the streamed assembly copies the table in aligned 4-byte words that
    // may run up to 12 bytes past an element's last row
    cudaError_t e = cudaMalloc(&V->d_pos, total + 64);
    if (e != cudaSuccess) { ctx->err = "position table allocation failed"; V->d_pos = nullptr; return FGPU_ERR_ALLOC; }
    int64_t blocks = std::min<int64_t>((total + 255) / 256, 152 * 64);
    PendingEvent ev;
    prof_begin(ctx, "positions", ev);
    positions_kernel<<<(int)std::max<int64_t>(blocks, 1), 256, 0, ctx->stream>>>(V->mesh->nt, V->n, V->d_l2n, V->pattern->d_ia,
                                                                              V->pattern->d_ja, V->d_pos, ctx->d_status);
    prof_end(ctx, ev);
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

// Warp-per-row gather. A warp owns one CSR row (dof node) at a time; each pass
// evaluates the rows of EPB incident elements at once (lane = slot * N + column).
// Each slot adds into its own shared-memory copy of the row (no two lanes of a
// slot share a column), and the EPB copies are summed in slot order when the row
// is written: the summation order is fixed, hence reproducible, without float
// atomics.
//   DF64: value = sum_k c_k T_k[li][j] as a compensated dot product (TwoProduct +
//         TwoSum on binary32), accumulation in df64, output converted to binary64
//         with integer operations.
//   F32 : binary32 coefficients, tables and accumulation.
__device__ __forceinline__ df record_entry_df(const float4* __restrict__ rp, const float* __restrict__ Th,
                                              const float* __restrict__ Tl, int stride, int tix) {
    float ch[7], cl[7];
    load_record(rp, ch, cl, true);
    return coef_entry_df(ch, cl, Th, Tl, stride, tix);
}
__device__ __forceinline__ float record_entry_f(const float4* __restrict__ rp, const float* __restrict__ Th, int stride, int tix) {
    float ch[7], cl[7];
    load_record(rp, ch, cl, false);
    return coef_entry_f(ch, Th, stride, tix);
}

template <int N>
struct RecordSource {
    const float4* __restrict__ rec;
    const float* __restrict__ Th;     // 7 N N (shared memory)
    const float* __restrict__ Tl;
    __device__ __forceinline__ df value_df(int64_t e, int li, int j) const {
        return record_entry_df(rec + 4 * e, Th, Tl, N * N, li * N + j);
    }
    __device__ __forceinline__ float value_f(int64_t e, int li, int j) const {
        return record_entry_f(rec + 4 * e, Th, N * N, li * N + j);
    }
};

// One pattern row r assembled by one warp: the row's incident elements are
// taken EPB at a time (lane = slot * N + j evaluates entry (li, j) of element
// slot), each slot accumulates into its own copy of the row in shared memory
// (acc: EPB copies with stride maxrow), and the copies are summed in slot order
// at the end, so the result does not depend on scheduling. acc is all zero on
// entry and on exit.
template <int MODE, int N, int EPB, class Src>
__device__ __forceinline__ void gather_row(int64_t r, const int64_t* __restrict__ sia, const int64_t* __restrict__ inc_ptr,
                                           const int32_t* __restrict__ inc, const uint8_t* __restrict__ posg, const Src& src,
                                           int maxrow, void* __restrict__ valv, int accumulate, int* __restrict__ status,
                                           float* __restrict__ acc, int lane) {
    constexpr int ACCW = MODE == kModeDF64 ? 2 : 1;   // floats per accumulator entry
    const int slot = lane / N, j = lane - slot * N;
    const bool lane_used = lane < EPB * N;
    float* myacc = acc + (size_t)(slot < EPB ? slot : 0) * maxrow * ACCW;
    const int64_t start = sia[r];
    const int len = (int)(sia[r + 1] - start);
    const int64_t tb = inc_ptr[r], te = inc_ptr[r + 1];
    if (len > maxrow) {
        if (lane == 0) atomicOr(status, kStatusRowOverflow);
        return;
    }
    for (int64_t c0 = tb; c0 < te; c0 += 32) {
        const int nin = (int)min((int64_t)32, te - c0);
        const int32_t mycode = lane < nin ? inc[c0 + lane] : 0;
        for (int b = 0; b < nin; b += EPB) {
            const int idx = b + slot;
            const int32_t code = __shfl_sync(0xffffffffu, mycode, idx < 32 ? idx : 31);
            if (lane_used && idx < nin) {
                const int64_t e = code >> 5;
                const int li = code & 31;
                const int pos = posg[e * (N * N) + li * N + j];
                if (MODE == kModeDF64) {
                    df a = df_add(df{myacc[2 * pos], myacc[2 * pos + 1]}, src.value_df(e, li, j));
                    myacc[2 * pos] = a.hi;
                    myacc[2 * pos + 1] = a.lo;
                } else {
                    myacc[pos] = f_add(myacc[pos], src.value_f(e, li, j));
                }
            }
            __syncwarp();
        }
    }
    // write the row: sum the slot copies in slot order (+ the old value for '+='), reset them
    for (int k = lane; k < len; k += 32) {
        if (MODE == kModeDF64) {
            df a{acc[2 * k], acc[2 * k + 1]};
            acc[2 * k] = 0.0f;
            acc[2 * k + 1] = 0.0f;
#pragma unroll
            for (int s = 1; s < EPB; ++s) {
                float* q = acc + (size_t)s * maxrow * 2 + 2 * k;
                a = df_add(a, df{q[0], q[1]});
                q[0] = 0.0f;
                q[1] = 0.0f;
            }
            double* out = reinterpret_cast<double*>(valv) + start + k;
            if (accumulate) a = df_add(d2df(*out), a);
            *out = df2d(a);
        } else {
            float a = acc[k];
            acc[k] = 0.0f;
#pragma unroll
            for (int s = 1; s < EPB; ++s) {
                a = f_add(a, acc[(size_t)s * maxrow + k]);
                acc[(size_t)s * maxrow + k] = 0.0f;
            }
            float* out = reinterpret_cast<float*>(valv) + start + k;
            *out = accumulate ? f_add(*out, a) : a;
        }
    }
    __syncwarp();
}

template <int MODE, int N, int EPB>
__global__ void __launch_bounds__(256) gather_row_kernel(
    int64_t nrows, const int64_t* __restrict__ sia, const int64_t* __restrict__ inc_ptr,
    const int32_t* __restrict__ inc, const uint8_t* __restrict__ posg, const float4* __restrict__ rec,
    const float* __restrict__ Thg, const float* __restrict__ Tlg, int maxrow, void* __restrict__ valv,
    int accumulate, int* __restrict__ status) {
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int NT = 7 * N * N;
    float* Th = reinterpret_cast<float*>(smem);
    float* Tl = Th + NT;
    for (int k = threadIdx.x; k < NT; k += blockDim.x) {
        Th[k] = Thg[k];
        if (MODE == kModeDF64) Tl[k] = Tlg[k];
    }
    const int tbytes = ((MODE == kModeDF64 ? 2 : 1) * NT * 4 + 15) & ~15;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    constexpr int ACCW = MODE == kModeDF64 ? 2 : 1;
    float* acc = reinterpret_cast<float*>(smem + tbytes) + (size_t)warp * EPB * maxrow * ACCW;
    __syncthreads();
    // accumulators start at zero once; each row resets what it used
    for (int k = lane; k < EPB * maxrow * ACCW; k += 32) acc[k] = 0.0f;
    __syncwarp();
    for (int64_t r = (int64_t)blockIdx.x * wpb + warp; r < nrows; r += (int64_t)gridDim.x * wpb)
        gather_row<MODE, N, EPB>(r, sia, inc_ptr, inc, posg, RecordSource<N>{rec, Th, Tl}, maxrow, valv, accumulate, status, acc,
                                 lane);
}

template <int MODE, int N, int EPB>
static int run_gather_row(fgpu_ctx* ctx, fgpu_matrix* A, const DevTables* tab, const float4* rec, int accumulate) {
    const DevPattern& P = *A->pattern;
    const fgpu_space* V = A->space;
    const int threads = 256, wpb = threads / 32;
    const int NT = 7 * N * N;
    size_t tbytes = ((MODE == kModeDF64 ? 2 : 1) * NT * 4 + 15) & ~15;
    size_t smem = tbytes + (size_t)wpb * EPB * P.max_row * (MODE == kModeDF64 ? 8 : 4);
    auto kern = gather_row_kernel<MODE, N, EPB>;
    if (P.max_row > 256) { ctx->err = "pattern rows longer than 256 entries"; return FGPU_ERR_INVALID; }
    if (smem > 227 * 1024) { ctx->err = "pattern rows too long for the gather kernel"; return FGPU_ERR_INVALID; }
    if (smem > 48 * 1024) FGPU_CUDA_CHECK(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    FGPU_CUDA_CHECK(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem));
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    int64_t need = (P.nrows + wpb - 1) / wpb;
    int64_t blocks = std::min<int64_t>(need, (int64_t)std::max(per_sm, 1) * sms);
    if (blocks < 1) blocks = 1;
    PendingEvent ev;
    prof_begin(ctx, "assemble_gather", ev);
    kern<<<(int)blocks, threads, smem, ctx->stream>>>(P.nrows, P.d_ia, V->d_inc_ptr, V->d_inc, V->d_pos, rec,
                                                      MODE == kModeDF64 ? tab->d_T7h : tab->d_T7f, tab->d_T7l, P.max_row,
                                                      A->d_val, accumulate, ctx->d_status);
    prof_end(ctx, ev);
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

__global__ void axpby_kernel(int64_t n, double a, const double* __restrict__ x, double b, double* __restrict__ y) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = a * x[i] + b * y[i];
}

int launch_axpby(fgpu_ctx* ctx, int64_t n, double a, const double* x, double b, double* y) {
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 8));
    axpby_kernel<<<(int)blocks, 256, 0, ctx->stream>>>(n, a, x, b, y);
    ++ctx->launches;
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

// ---------------------------------------------------------------------------
// Batched assembly: many independent problems (meshes, orders, kappas) in one
// geometry launch and one persistent gather launch. Rows of all problems form
// one global index space; warps take chunks of rows from a device work queue
// (atomic counter), find the row's problem by binary search over the row
// offsets, and run the same per-row body as the single-problem kernel, so a
// batched matrix is bit-identical to the one assembled alone.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int batch_find(const int64_t* __restrict__ off, int nprob, int64_t g) {
    int lo = 0, hi = nprob - 1;        // largest p with off[p] <= g
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(off + mid) <= g) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__global__ void batch_geometry_kernel(int nprob, const BatchProblem* __restrict__ probs, const int64_t* __restrict__ elem_off,
                                      int64_t total, int* __restrict__ status) {
    int p = -1;
    int64_t pe0 = 0, pe1 = 0;
    df kc{0.0f, 0.0f}, mc{0.0f, 0.0f};
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x) {
        if (g < pe0 || g >= pe1) {
            p = batch_find(elem_off, nprob, g);
            pe0 = elem_off[p];
            pe1 = elem_off[p + 1];
            kc = d2df(probs[p].kappa_c);
            mc = d2df(probs[p].mass);
        }
        const BatchProblem& P = probs[p];
        geometry_df_element(g - pe0, P.xyz, P.tets, P.kappa, kc, mc, df{1.0f, 0.0f}, P.rec, status);
    }
}

// table offsets (floats) of orders 1..3 inside the shared table block: 7 n^2 each
__host__ __device__ constexpr int batch_tab_off(int order) { return order == 1 ? 0 : order == 2 ? 7 * 16 : 7 * 16 + 7 * 100; }
constexpr int kBatchTabFloats = 7 * 16 + 7 * 100 + 7 * 400;

template <int MODE>
__global__ void __launch_bounds__(256) batch_gather_kernel(int nprob, const BatchProblem* __restrict__ probs,
                                                           const int64_t* __restrict__ row_off, int64_t total,
                                                           const float* __restrict__ Thg, const float* __restrict__ Tlg,
                                                           int acc_floats, unsigned long long* __restrict__ counter, int chunk,
                                                           int accumulate, int* __restrict__ status) {
    extern __shared__ __align__(16) unsigned char smem[];
    float* Th = reinterpret_cast<float*>(smem);
    float* Tl = Th + kBatchTabFloats;
    for (int k = threadIdx.x; k < kBatchTabFloats; k += blockDim.x) {
        Th[k] = Thg[k];
        if (MODE == kModeDF64) Tl[k] = Tlg[k];
    }
    const int tfloats = ((MODE == kModeDF64 ? 2 : 1) * kBatchTabFloats + 3) & ~3;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float* acc = reinterpret_cast<float*>(smem) + tfloats + (size_t)warp * acc_floats;
    __syncthreads();
    for (int k = lane; k < acc_floats; k += 32) acc[k] = 0.0f;
    __syncwarp();
    int p = -1;
    int64_t pr0 = 0, pr1 = 0;
    while (true) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(counter, (unsigned long long)chunk);
        base = __shfl_sync(0xffffffffu, base, 0);
        if ((int64_t)base >= total) break;
        const int64_t end = min((int64_t)base + chunk, total);
        for (int64_t g = (int64_t)base; g < end; ++g) {
            if (g < pr0 || g >= pr1) {
                p = batch_find(row_off, nprob, g);
                pr0 = row_off[p];
                pr1 = row_off[p + 1];
            }
            const BatchProblem& P = probs[p];
            const int64_t r = g - pr0;
            switch (P.order) {
                case 1:
                    gather_row<MODE, 4, 8>(r, P.sia, P.inc_ptr, P.inc, P.pos,
                                           RecordSource<4>{P.rec, Th + batch_tab_off(1), Tl + batch_tab_off(1)},
                                           P.maxrow, P.val, accumulate, status, acc, lane);
                    break;
                case 2:
                    gather_row<MODE, 10, 3>(r, P.sia, P.inc_ptr, P.inc, P.pos,
                                           RecordSource<10>{P.rec, Th + batch_tab_off(2), Tl + batch_tab_off(2)},
                                            P.maxrow, P.val, accumulate, status, acc, lane);
                    break;
                default:
                    gather_row<MODE, 20, 1>(r, P.sia, P.inc_ptr, P.inc, P.pos,
                                           RecordSource<20>{P.rec, Th + batch_tab_off(3), Tl + batch_tab_off(3)},
                                            P.maxrow, P.val, accumulate, status, acc, lane);
                    break;
            }
        }
    }
}

int launch_batch_geometry(fgpu_ctx* ctx, int nprob, const BatchProblem* d_probs, const int64_t* d_elem_off, int64_t total_elems) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((total_elems + 255) / 256, (int64_t)sms * 16));
    PendingEvent ev;
    prof_begin(ctx, "batch_geometry", ev);
    batch_geometry_kernel<<<(int)blocks, 256, 0, ctx->stream>>>(nprob, d_probs, d_elem_off, total_elems, ctx->d_status);
    prof_end(ctx, ev);
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

// shared tables of orders 1..3 (hi, lo) for the batch kernel, per device
static std::mutex g_btab_mutex;
static std::map<int, std::pair<float*, float*>> g_btabs;
static int batch_tables(fgpu_ctx* ctx, float** h, float** l) {
    std::lock_guard<std::mutex> lock(g_btab_mutex);
    auto it = g_btabs.find(ctx->device);
    if (it != g_btabs.end()) { *h = it->second.first; *l = it->second.second; return FGPU_OK; }
    float *dh = nullptr, *dl = nullptr;
    FGPU_CUDA_CHECK(ctx, cudaMalloc(&dh, kBatchTabFloats * sizeof(float)));
    FGPU_CUDA_CHECK(ctx, cudaMalloc(&dl, kBatchTabFloats * sizeof(float)));
    for (int order = 1; order <= 3; ++order) {
        std::string err;
        DevTables* t = get_dev_tables(order, 2 * order, err);
        if (!t) { ctx->err = err; return FGPU_ERR_INVALID; }
        const size_t nb = (size_t)7 * t->n * t->n * sizeof(float);
        FGPU_CUDA_CHECK(ctx, cudaMemcpy(dh + batch_tab_off(order), t->d_T7h, nb, cudaMemcpyDeviceToDevice));
        FGPU_CUDA_CHECK(ctx, cudaMemcpy(dl + batch_tab_off(order), t->d_T7l, nb, cudaMemcpyDeviceToDevice));
    }
    g_btabs[ctx->device] = {dh, dl};
    *h = dh;
    *l = dl;
    return FGPU_OK;
}

// The two-phase element phase works on groups of 32 consecutive elements: each warp forms the
// coefficient records of a group, one per lane (geometry_df_record, the same arithmetic as
// geometry_df_kernel), into shared memory, then the group's element matrices. With NTRI <= 64 each lane
// holds the table values of its (at most two) entries in registers (tri_lane_tables); with more entries
// (P3) two elements share each table value read from shared memory.
template <int MODE, int N>
__device__ __forceinline__ void tri_lane_tables(const float* Th, const float* Tl, int lane, float* th0, float* tl0, float* th1,
                                                float* tl1) {
    constexpr int NTRI = N * (N + 1) / 2;
    constexpr int EPW = NTRI >= 32 ? 1 : 32 / NTRI;
    const int sub = lane / NTRI < EPW ? lane / NTRI : EPW;
    const int t0 = EPW > 1 ? lane - sub * NTRI : lane;
    const int t1 = t0 + (EPW > 1 ? NTRI : 32);
#pragma unroll
    for (int k = 0; k < 7; ++k) {
        const bool ok0 = sub < EPW && t0 < NTRI, ok1 = sub < EPW && t1 < NTRI;
        th0[k] = ok0 ? Th[k * NTRI + t0] : 0.0f;
        th1[k] = ok1 ? Th[k * NTRI + t1] : 0.0f;
        tl0[k] = (MODE == kModeDF64 && ok0) ? Tl[k * NTRI + t0] : 0.0f;
        tl1[k] = (MODE == kModeDF64 && ok1) ? Tl[k * NTRI + t1] : 0.0f;
    }
}

// the upper triangles of elements e0 .. e0 + cnt - 1 from their records in wrec (shared memory)
template <int MODE, int N>
__device__ __forceinline__ void tri_group_entries(void* __restrict__ kbuf, int64_t e0, int cnt, const float4* wrec, const float* Th,
                                                  const float* Tl, int lane, const float* th0, const float* tl0, const float* th1,
                                                  const float* tl1) {
    constexpr int NTRI = N * (N + 1) / 2;
    constexpr int EPW = NTRI >= 32 ? 1 : 32 / NTRI;      // elements per warp pass (P1: 3)
    constexpr bool DF = MODE == kModeDF64;
    if (NTRI <= 64) {
        const int sub = lane / NTRI < EPW ? lane / NTRI : EPW;
        const int t0 = EPW > 1 ? lane - sub * NTRI : lane;
        const int t1 = t0 + (EPW > 1 ? NTRI : 32);
        for (int j0 = 0; j0 < cnt; j0 += EPW) {
            const int j = j0 + sub;
            if (sub >= EPW || j >= cnt) continue;
            float ch[7], cl[7];
            load_record_shared(wrec + 4 * j, ch, cl, DF);
            const int64_t e = e0 + j;
            if (DF) {
                float2* kb = reinterpret_cast<float2*>(kbuf) + e * NTRI;
                if (t0 < NTRI) {
                    const df v = coef_entry_df_reg(ch, cl, th0, tl0);
                    kb[t0] = make_float2(v.hi, v.lo);
                }
                if (t1 < NTRI) {
                    const df v = coef_entry_df_reg(ch, cl, th1, tl1);
                    kb[t1] = make_float2(v.hi, v.lo);
                }
            } else {
                float* kb = reinterpret_cast<float*>(kbuf) + e * NTRI;
                if (t0 < NTRI) {
                    float v = 0.0f;
#pragma unroll
                    for (int k = 0; k < 7; ++k) v = fmaf(ch[k], th0[k], v);
                    kb[t0] = v;
                }
                if (t1 < NTRI) {
                    float v = 0.0f;
#pragma unroll
                    for (int k = 0; k < 7; ++k) v = fmaf(ch[k], th1[k], v);
                    kb[t1] = v;
                }
            }
        }
    } else {
        for (int j = 0; j < cnt; j += 2) {
            const bool two = j + 1 < cnt;
            float ch0[7], cl0[7], ch1[7], cl1[7];
            load_record_shared(wrec + 4 * j, ch0, cl0, DF);
            load_record_shared(wrec + 4 * (two ? j + 1 : j), ch1, cl1, DF);
            const int64_t e = e0 + j;
            for (int t = lane; t < NTRI; t += 32) {
                float th[7], tl[7];
#pragma unroll
                for (int k = 0; k < 7; ++k) {
                    th[k] = Th[k * NTRI + t];
                    tl[k] = DF ? Tl[k * NTRI + t] : 0.0f;
                }
                if (DF) {
                    float2* kb = reinterpret_cast<float2*>(kbuf);
                    const df v0 = coef_entry_df_reg(ch0, cl0, th, tl);
                    kb[e * NTRI + t] = make_float2(v0.hi, v0.lo);
                    if (two) {
                        const df v1 = coef_entry_df_reg(ch1, cl1, th, tl);
                        kb[(e + 1) * NTRI + t] = make_float2(v1.hi, v1.lo);
                    }
                } else {
                    float* kb = reinterpret_cast<float*>(kbuf);
                    float v0 = 0.0f, v1 = 0.0f;
#pragma unroll
                    for (int k = 0; k < 7; ++k) {
                        v0 = fmaf(ch0[k], th[k], v0);
                        v1 = fmaf(ch1[k], th[k], v1);
                    }
                    kb[e * NTRI + t] = v0;
                    if (two) kb[(e + 1) * NTRI + t] = v1;
                }
            }
        }
    }
}

// ---- two-phase batches: the element kernel and the gather-map kernel of the
// single-problem path over all problems (same per-entry arithmetic and order,
// so each matrix gets the bits FGPU_ALGO_TWO_PHASE gives it alone) ----
// upper-triangle tables of orders 1..3 in one block: 7 n(n+1)/2 each
__host__ __device__ constexpr int batch_tri_off(int order) { return order == 1 ? 0 : order == 2 ? 7 * 10 : 7 * 10 + 7 * 55; }
constexpr int kBatchTriFloats = 7 * 10 + 7 * 55 + 7 * 210;

template <int MODE>
__global__ void __launch_bounds__(256) batch_element_kernel(int nprob, const BatchProblem* __restrict__ probs,
                                                            const int64_t* __restrict__ grp_off, int64_t total_groups,
                                                            const float* __restrict__ Thg, const float* __restrict__ Tlg,
                                                            int* __restrict__ status) {
    __shared__ float Th[kBatchTriFloats];
    __shared__ float Tl[MODE == kModeDF64 ? kBatchTriFloats : 1];
    __shared__ float4 srec[8 * 32 * 4];                  // per warp: the records of 32 elements
    for (int k = threadIdx.x; k < kBatchTriFloats; k += blockDim.x) {
        Th[k] = Thg[k];
        if (MODE == kModeDF64) Tl[k] = Tlg[k];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    float4* wrec = srec + (threadIdx.x >> 5) * 32 * 4;
    int p = -1;
    int64_t pg0 = 0, pg1 = 0;
    // one warp per group of 32 consecutive elements of one problem (the single-problem kernel's groups)
    for (int64_t g = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); g < total_groups; g += nw) {
        if (g < pg0 || g >= pg1) {
            p = batch_find(grp_off, nprob, g);
            pg0 = grp_off[p];
            pg1 = grp_off[p + 1];
        }
        const BatchProblem& P = probs[p];
        const int64_t e0 = (g - pg0) * 32;
        const int cnt = (int)(P.nt - e0 < 32 ? P.nt - e0 : 32);
        if (lane < cnt)
            geometry_df_record(e0 + lane, P.xyz, P.tets, P.kappa, d2df(P.kappa_c), d2df(P.mass), df{1.0f, 0.0f}, wrec + 4 * lane,
                               status);
        __syncwarp();
        float th0[7], tl0[7], th1[7], tl1[7];
        const int to = batch_tri_off(P.order);
        if (P.order == 1) {
            tri_lane_tables<MODE, 4>(Th + to, Tl + to, lane, th0, tl0, th1, tl1);
            tri_group_entries<MODE, 4>(P.kbuf, e0, cnt, wrec, Th + to, Tl + to, lane, th0, tl0, th1, tl1);
        } else if (P.order == 2) {
            tri_lane_tables<MODE, 10>(Th + to, Tl + to, lane, th0, tl0, th1, tl1);
            tri_group_entries<MODE, 10>(P.kbuf, e0, cnt, wrec, Th + to, Tl + to, lane, th0, tl0, th1, tl1);
        } else {
            tri_group_entries<MODE, 20>(P.kbuf, e0, cnt, wrec, Th + to, Tl + to, lane, th0, tl0, th1, tl1);
        }
        __syncwarp();
    }
}

template <int MODE>
__global__ void __launch_bounds__(256) batch_gather_map_kernel(int nprob, const BatchProblem* __restrict__ probs,
                                                               const int64_t* __restrict__ nz_off, int64_t total, int accumulate) {
    int p = -1;
    int64_t pz0 = 0, pz1 = 0;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x) {
        if (g < pz0 || g >= pz1) {
            p = batch_find(nz_off, nprob, g);
            pz0 = nz_off[p];
            pz1 = nz_off[p + 1];
        }
        const BatchProblem& P = probs[p];
        const int64_t k = g - pz0;
        const uint32_t p0 = __ldg(P.gptr + k), p1 = __ldg(P.gptr + k + 1);
        if (MODE == kModeDF64) {
            // the single-matrix gather's compensated sum (same bits)
            const float2* kb = reinterpret_cast<const float2*>(P.kbuf);
            float sh = 0.0f, sl = 0.0f;
            for (uint32_t q = p0; q < p1; q += 4) {
                uint32_t ix[4];
                float2 v[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) ix[u] = q + u < p1 ? __ldg(P.gidx + q + u) : 0u;
#pragma unroll
                for (int u = 0; u < 4; ++u) v[u] = q + u < p1 ? __ldg(kb + (ix[u] & 0x7FFFFFFFu)) : make_float2(0.0f, 0.0f);
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (q + u < p1) {
                        const df t = two_sum(sh, v[u].x);
                        sh = t.hi;
                        sl = f_add(sl, f_add(t.lo, v[u].y));
                    }
            }
            df s = two_sum(sh, sl);
            double* out = reinterpret_cast<double*>(P.val) + k;
            if (accumulate) s = df_add(d2df(*out), s);
            *out = df2d(s);
        } else {
            const float* kb = reinterpret_cast<const float*>(P.kbuf);
            float s = 0.0f;
            for (uint32_t q = p0; q < p1; q += 4) {
                uint32_t ix[4];
                float v[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) ix[u] = q + u < p1 ? __ldg(P.gidx + q + u) : 0u;
#pragma unroll
                for (int u = 0; u < 4; ++u) v[u] = q + u < p1 ? __ldg(kb + (ix[u] & 0x7FFFFFFFu)) : 0.0f;
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (q + u < p1) s = (q + u == p0) ? v[u] : f_add(s, v[u]);
            }
            float* out = reinterpret_cast<float*>(P.val) + k;
            *out = accumulate ? f_add(*out, s) : s;
        }
    }
}

static std::map<int, std::pair<float*, float*>> g_btri;
static int batch_tri_tables(fgpu_ctx* ctx, float** h, float** l) {
    std::lock_guard<std::mutex> lock(g_btab_mutex);
    auto it = g_btri.find(ctx->device);
    if (it != g_btri.end()) { *h = it->second.first; *l = it->second.second; return FGPU_OK; }
    float *dh = nullptr, *dl = nullptr;
    FGPU_CUDA_CHECK(ctx, cudaMalloc(&dh, kBatchTriFloats * sizeof(float)));
    FGPU_CUDA_CHECK(ctx, cudaMalloc(&dl, kBatchTriFloats * sizeof(float)));
    for (int order = 1; order <= 3; ++order) {
        std::string err;
        DevTables* t = get_dev_tables(order, 2 * order, err);
        if (!t) { ctx->err = err; return FGPU_ERR_INVALID; }
        const size_t nb = (size_t)7 * (t->n * (t->n + 1) / 2) * sizeof(float);
        FGPU_CUDA_CHECK(ctx, cudaMemcpy(dh + batch_tri_off(order), t->d_T7th, nb, cudaMemcpyDeviceToDevice));
        FGPU_CUDA_CHECK(ctx, cudaMemcpy(dl + batch_tri_off(order), t->d_T7tl, nb, cudaMemcpyDeviceToDevice));
    }
    g_btri[ctx->device] = {dh, dl};
    *h = dh;
    *l = dl;
    return FGPU_OK;
}

int launch_batch_two_phase(fgpu_ctx* ctx, int nprob, const BatchProblem* d_probs, const int64_t* d_grp_off,
                           int64_t total_groups, const int64_t* d_nz_off, int64_t total_nnz, int f32, int threads,
                           int accumulate) {
    float *Th = nullptr, *Tl = nullptr;
    int rc = batch_tri_tables(ctx, &Th, &Tl);
    if (rc) return rc;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    {
        const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((total_groups + 7) / 8, (int64_t)sms * 16));
        PendingEvent ev;
        prof_begin(ctx, "batch_elements", ev);
        if (f32)
            batch_element_kernel<kModeF32><<<(int)blocks, 256, 0, ctx->stream>>>(nprob, d_probs, d_grp_off, total_groups, Th, Tl,
                                                                                 ctx->d_status);
        else
            batch_element_kernel<kModeDF64><<<(int)blocks, 256, 0, ctx->stream>>>(nprob, d_probs, d_grp_off, total_groups, Th, Tl,
                                                                                  ctx->d_status);
        prof_end(ctx, ev);
        FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    }
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((total_nnz + threads - 1) / threads, (int64_t)sms * (2048 / threads) * 4));
    PendingEvent ev;
    prof_begin(ctx, "batch_gather", ev);
    if (f32) batch_gather_map_kernel<kModeF32><<<(int)blocks, threads, 0, ctx->stream>>>(nprob, d_probs, d_nz_off, total_nnz, accumulate);
    else batch_gather_map_kernel<kModeDF64><<<(int)blocks, threads, 0, ctx->stream>>>(nprob, d_probs, d_nz_off, total_nnz, accumulate);
    prof_end(ctx, ev);
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

int launch_batch_gather(fgpu_ctx* ctx, int nprob, const BatchProblem* d_probs, const int64_t* d_row_off, int64_t total_rows,
                        int f32, int acc_floats, unsigned long long* d_counter, const BatchLaunch& cfg, int accumulate) {
    float *Th = nullptr, *Tl = nullptr;
    int rc = batch_tables(ctx, &Th, &Tl);
    if (rc) return rc;
    const int threads = cfg.threads, wpb = threads / 32;
    const size_t tfloats = ((f32 ? 1 : 2) * kBatchTabFloats + 3) & ~3;
    const size_t smem = (tfloats + (size_t)wpb * acc_floats) * sizeof(float);
    auto kern = f32 ? batch_gather_kernel<kModeF32> : batch_gather_kernel<kModeDF64>;
    if (smem > 227 * 1024) { ctx->err = "batch: staging buffers exceed shared memory"; return FGPU_ERR_INVALID; }
    FGPU_CUDA_CHECK(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    FGPU_CUDA_CHECK(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem));
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int blocks = std::max(1, std::max(per_sm, 1) * sms);
    FGPU_CUDA_CHECK(ctx, cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), ctx->stream));
    PendingEvent ev;
    prof_begin(ctx, "batch_gather", ev);
    kern<<<blocks, threads, smem, ctx->stream>>>(nprob, d_probs, d_row_off, total_rows, Th, Tl, acc_floats, d_counter, cfg.chunk,
                                                 accumulate, ctx->d_status);
    prof_end(ctx, ev);
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

// ---------------------------------------------------------------------------
// Two-phase assembly.
//   Phase 1 (element_tri_kernel): each element matrix is computed once, as its
//   upper triangle (NTRI = n (n + 1) / 2 entries; the reference tensors are
//   exactly symmetric), into a device buffer; each warp forms the coefficient
//   records of 32 elements (one per lane, in shared memory), then their
//   matrices with lanes over entries, contiguous writes.
//   Phase 2 (gather_map_kernel): one thread per CSR entry sums its
//   contributions in element order through a gather map built once per space
//   (gptr: nnz + 1 offsets, gidx: buffer index of each contribution), which is
//   the order in which the reference's element loop adds element blocks into
//   the matrix (bilinearformcontext.hpp:784-847 -> MatSetValues ADD_VALUES).
//   No float atomics; the gather is a streaming pass over gptr, gidx and the
//   CSR values.
// ---------------------------------------------------------------------------
template <int MODE, int N>
__global__ void __launch_bounds__(256) element_tri_kernel(int64_t nt, GeoIn geo, const float* __restrict__ Thg,
                                                          const float* __restrict__ Tlg, void* __restrict__ kbuf,
                                                          int* __restrict__ status) {
    constexpr int NTRI = N * (N + 1) / 2;
    constexpr bool DF = MODE == kModeDF64;
    __shared__ float Th[7 * NTRI];
    __shared__ float Tl[DF ? 7 * NTRI : 1];
    __shared__ float4 srec[8 * 32 * 4];                  // per warp: the records of 32 elements
    for (int k = threadIdx.x; k < 7 * NTRI; k += blockDim.x) {
        Th[k] = Thg[k];
        if (DF) Tl[k] = Tlg[k];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t wid = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    float th0[7], tl0[7], th1[7], tl1[7];
    if (NTRI <= 64) tri_lane_tables<MODE, N>(Th, Tl, lane, th0, tl0, th1, tl1);   // the same for every element
    const df kc = d2df(geo.kc), mc = d2df(geo.mc);
    const df ksc = geo.kscale ? d2df(*geo.kscale) : df{1.0f, 0.0f};
    float4* wrec = srec + (threadIdx.x >> 5) * 32 * 4;
    for (int64_t g0 = wid * 32; g0 < nt; g0 += nw * 32) {
        if (g0 + lane < nt) geometry_df_record(g0 + lane, geo.xyz, geo.tets, geo.kappa, kc, mc, ksc, wrec + 4 * lane, status);
        __syncwarp();
        const int cnt = (int)(nt - g0 < 32 ? nt - g0 : 32);
        tri_group_entries<MODE, N>(kbuf, g0, cnt, wrec, Th, Tl, lane, th0, tl0, th1, tl1);
        __syncwarp();
    }
}

// One thread per CSR entry, its contributions in batches of B (the index and
// value loads of a batch are issued together; the sum stays in element
// order, so B, like the launch shape, does not change the result; the tuner
// picks it). Measured against three alternatives at P2 48^3 (this: 0.32 ms):
// entries sorted by contribution count within 256-entry windows (0.50 ms: the
// permuted writes lose their coalescing); a warp-flat load of the 32 entries'
// contributions staged in shared memory (0.39 ms: fewer loads in flight per
// warp); a split into entries with at most 2 contributions (one unrolled step,
// 0.21 ms, 70 % of DRAM peak) and the others taken from a list sorted by count
// (0.30 ms: the sorted list scatters the reads of the element buffer, 1.75 GB
// of DRAM reads for 5.4 M entries). At P2 64^3 two entries per thread (k and
// k + stride, loads issued together) took 0.90 ms against 0.655 ms. A symmetric
// map (entries j >= i only, each thread also storing its value at the transpose's
// position) halves the map and the buffer reads on paper but took 0.785 ms
// against 0.64 ms: at 48^3 its DRAM reads stayed at 888 MB (the transposes'
// second reads of the buffer hit L2 here), with more warp instructions (half the
// lanes idle) and scattered stores. One batch of 6 per entry with the entries of
// more than 6 contributions (the vertex-row diagonals, 0.5 % of the entries) left
// to a second kernel over their list: timed by the tuner against B = 2, 4, 8 and
// never picked at P2 or P3 64^3 (the warps' longest entries are not what bounds
// the kernel). L2 eviction hints (map and values evict-first, element buffer
// evict-last) raised the DRAM reads at P2 48^3 from 900 to 1010 MB and the time
// from 0.275 to 0.295 ms. The grid matters for the reads: with more blocks than
// fit at once, each wave of resident blocks strides over the whole matrix and an
// entry and its transpose are read in different waves (900 MB); one entry per
// thread sweeps the entries in order and reads exactly the design bytes (660 MB)
// but took 0.30 ms: the kernel is bound by issue and by the latency of its three
// dependent loads, not by DRAM.
template <int MODE, int B = 4>
__global__ void __launch_bounds__(256) gather_map_kernel(int64_t nnz, const uint32_t* __restrict__ gptr,
                                                         const uint32_t* __restrict__ gidx, const void* __restrict__ kbuf,
                                                         void* __restrict__ valv, int accumulate, double* __restrict__ hout) {
    // hout (binary64 results only): a mapped page-locked host buffer that receives a copy of each value
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t p0 = __ldg(gptr + k), p1 = __ldg(gptr + k + 1);
        if (MODE == kModeDF64) {
            // compensated sum in element order: the high parts through TwoSum, their rounding errors and
            // the low parts in one binary32 accumulator, normalised once (error ~ (count) u^2 |sum|)
            const float2* kb = reinterpret_cast<const float2*>(kbuf);
            float sh = 0.0f, sl = 0.0f;
            for (uint32_t p = p0; p < p1; p += B) {
                uint32_t ix[B];
                float2 v[B];
#pragma unroll
                for (int u = 0; u < B; ++u) ix[u] = p + u < p1 ? __ldg(gidx + p + u) : 0u;
#pragma unroll
                for (int u = 0; u < B; ++u) v[u] = p + u < p1 ? __ldg(kb + (ix[u] & 0x7FFFFFFFu)) : make_float2(0.0f, 0.0f);
#pragma unroll
                for (int u = 0; u < B; ++u)
                    if (p + u < p1) {
                        const df t = two_sum(sh, v[u].x);
                        sh = t.hi;
                        sl = f_add(sl, f_add(t.lo, v[u].y));
                    }
            }
            df s = two_sum(sh, sl);
            double* out = reinterpret_cast<double*>(valv) + k;
            if (accumulate) s = df_add(d2df(*out), s);
            const double r = df2d(s);
            *out = r;
            if (hout) hout[k] = r;
        } else {
            const float* kb = reinterpret_cast<const float*>(kbuf);
            float s = 0.0f;
            for (uint32_t p = p0; p < p1; p += B) {
                uint32_t ix[B];
                float v[B];
#pragma unroll
                for (int u = 0; u < B; ++u) ix[u] = p + u < p1 ? __ldg(gidx + p + u) : 0u;
#pragma unroll
                for (int u = 0; u < B; ++u) v[u] = p + u < p1 ? __ldg(kb + (ix[u] & 0x7FFFFFFFu)) : 0.0f;
#pragma unroll
                for (int u = 0; u < B; ++u)
                    if (p + u < p1) s = (p + u == p0) ? v[u] : f_add(s, v[u]);
            }
            float* out = reinterpret_cast<float*>(valv) + k;
            *out = accumulate ? f_add(*out, s) : s;
        }
    }
}

// The same gather software-pipelined over a thread's grid-stride entries. One entry costs three
// dependent loads (its gptr range, then its gidx indices, then the element-buffer values), so the
// plain kernel keeps one round trip of DRAM latency per load level in flight per thread. Here
// iteration i issues the element-buffer loads of entry k (indices already in registers), the gidx
// loads of entry k + S and the gptr loads of entry k + 2S together, then sums entry k: one latency
// per entry instead of three. Entries with more than B contributions load their further batches
// in place. The sum of every entry is the same sequence of operations as in gather_map_kernel, so
// the values are the same bits. Measured at 64^3 (tuned shapes): binary32 P3 1.87 against 2.12 ms,
// P2 0.43 against 0.46 ms; df64 P2 0.66 against 0.64 ms (more registers, and the three entries in
// flight widen the window of element-buffer lines: 880 against 803 MB of DRAM reads at 48^3). The
// tuner times both.
template <int MODE, int B = 4>
__global__ void __launch_bounds__(256) gather_map_pipe_kernel(int64_t nnz, const uint32_t* __restrict__ gptr,
                                                              const uint32_t* __restrict__ gidx, const void* __restrict__ kbuf,
                                                              void* __restrict__ valv, int accumulate, double* __restrict__ hout) {
    const int64_t S = (int64_t)gridDim.x * blockDim.x;
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= nnz) return;
    uint32_t a0 = __ldg(gptr + k), a1 = __ldg(gptr + k + 1);          // entry k
    int64_t kn = k + S;
    uint32_t b0 = 0, b1 = 0;                                            // entry k + S
    if (kn < nnz) {
        b0 = __ldg(gptr + kn);
        b1 = __ldg(gptr + kn + 1);
    }
    uint32_t ix[B];
#pragma unroll
    for (int u = 0; u < B; ++u) ix[u] = a0 + u < a1 ? __ldg(gidx + a0 + u) : 0u;
    for (;;) {
        // loads of three entries in flight together
        uint32_t nx[B];
        uint32_t c0 = 0, c1 = 0;
        const int64_t knn = kn + S;
        if (MODE == kModeDF64) {
            const float2* kb = reinterpret_cast<const float2*>(kbuf);
            float2 v[B];
#pragma unroll
            for (int u = 0; u < B; ++u) v[u] = a0 + u < a1 ? __ldg(kb + (ix[u] & 0x7FFFFFFFu)) : make_float2(0.0f, 0.0f);
#pragma unroll
            for (int u = 0; u < B; ++u) nx[u] = b0 + u < b1 ? __ldg(gidx + b0 + u) : 0u;
            if (knn < nnz) {
                c0 = __ldg(gptr + knn);
                c1 = __ldg(gptr + knn + 1);
            }
            float sh = 0.0f, sl = 0.0f;
#pragma unroll
            for (int u = 0; u < B; ++u)
                if (a0 + u < a1) {
                    const df t = two_sum(sh, v[u].x);
                    sh = t.hi;
                    sl = f_add(sl, f_add(t.lo, v[u].y));
                }
            for (uint32_t p = a0 + B; p < a1; p += B) {
                uint32_t jx[B];
                float2 w[B];
#pragma unroll
                for (int u = 0; u < B; ++u) jx[u] = p + u < a1 ? __ldg(gidx + p + u) : 0u;
#pragma unroll
                for (int u = 0; u < B; ++u) w[u] = p + u < a1 ? __ldg(kb + (jx[u] & 0x7FFFFFFFu)) : make_float2(0.0f, 0.0f);
#pragma unroll
                for (int u = 0; u < B; ++u)
                    if (p + u < a1) {
                        const df t = two_sum(sh, w[u].x);
                        sh = t.hi;
                        sl = f_add(sl, f_add(t.lo, w[u].y));
                    }
            }
            df sum = two_sum(sh, sl);
            double* out = reinterpret_cast<double*>(valv) + k;
            if (accumulate) sum = df_add(d2df(*out), sum);
            const double r = df2d(sum);
            *out = r;
            if (hout) hout[k] = r;
        } else {
            const float* kb = reinterpret_cast<const float*>(kbuf);
            float v[B];
#pragma unroll
            for (int u = 0; u < B; ++u) v[u] = a0 + u < a1 ? __ldg(kb + (ix[u] & 0x7FFFFFFFu)) : 0.0f;
#pragma unroll
            for (int u = 0; u < B; ++u) nx[u] = b0 + u < b1 ? __ldg(gidx + b0 + u) : 0u;
            if (knn < nnz) {
                c0 = __ldg(gptr + knn);
                c1 = __ldg(gptr + knn + 1);
            }
            float sum = 0.0f;
#pragma unroll
            for (int u = 0; u < B; ++u)
                if (a0 + u < a1) sum = (u == 0) ? v[u] : f_add(sum, v[u]);
            for (uint32_t p = a0 + B; p < a1; p += B) {
                uint32_t jx[B];
                float w[B];
#pragma unroll
                for (int u = 0; u < B; ++u) jx[u] = p + u < a1 ? __ldg(gidx + p + u) : 0u;
#pragma unroll
                for (int u = 0; u < B; ++u) w[u] = p + u < a1 ? __ldg(kb + (jx[u] & 0x7FFFFFFFu)) : 0.0f;
#pragma unroll
                for (int u = 0; u < B; ++u)
                    if (p + u < a1) sum = f_add(sum, w[u]);
            }
            float* out = reinterpret_cast<float*>(valv) + k;
            *out = accumulate ? f_add(*out, sum) : sum;
        }
        if (kn >= nnz) break;
        k = kn;
        kn = knn;
        a0 = b0;
        a1 = b1;
        b0 = c0;
        b1 = c1;
#pragma unroll
        for (int u = 0; u < B; ++u) ix[u] = nx[u];
    }
}

// ---- gather map construction (once per space) ----
// contributions per CSR entry (integer atomics: the counts do not depend on order)
__global__ void map_count_kernel(int64_t nt, int n, const int32_t* __restrict__ l2n, const int64_t* __restrict__ ia,
                                 const uint8_t* __restrict__ pos, uint32_t* __restrict__ cnt) {
    const int64_t total = nt * n * n;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = t / (n * n);
        const int i = (int)((t - e * n * n) / n);
        atomicAdd(cnt + ia[l2n[e * n + i]] + pos[t], 1u);
    }
}

// fill: one warp per row, incident elements in element order, lanes over the
// element row's columns (distinct entries), a per-entry cursor in shared memory
__global__ void __launch_bounds__(256) map_fill_kernel(int64_t nrows, int n, int ntri, const int64_t* __restrict__ ia,
                                                       const int64_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                                                       const uint8_t* __restrict__ pos, const uint16_t* __restrict__ trig,
                                                       const uint32_t* __restrict__ gptr, uint32_t* __restrict__ gidx,
                                                       int* __restrict__ status) {
    __shared__ uint32_t cur[8][256];
    __shared__ uint16_t tri[32 * 32];   // n <= 32 (checked by the launcher)
    for (int k = threadIdx.x; k < n * n; k += blockDim.x) tri[k] = trig[k];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int64_t r = (int64_t)blockIdx.x * 8 + warp; r < nrows; r += (int64_t)gridDim.x * 8) {
        const int64_t start = ia[r];
        const int len = (int)(ia[r + 1] - start);
        if (len > 256) {
            if (lane == 0) atomicOr(status, kStatusRowOverflow);
            continue;
        }
        for (int k = lane; k < len; k += 32) cur[warp][k] = gptr[start + k];
        __syncwarp();
        for (int64_t t = inc_ptr[r]; t < inc_ptr[r + 1]; ++t) {
            const int32_t code = inc[t];
            const int64_t e = code >> 5;
            const int li = code & 31;
            if (lane < n) {
                const int p = pos[(e * n + li) * n + lane];
                const uint32_t slot = cur[warp][p];
                cur[warp][p] = slot + 1;
                // bit 31: the contribution is K_e(li, lj) with li > lj, stored as (lj, li)
                gidx[slot] = (uint32_t)(e * ntri + tri[li * n + lane]) | (li > lane ? 0x80000000u : 0u);
            }
            __syncwarp();
        }
    }
}

int launch_build_gather_map(fgpu_ctx* ctx, fgpu_space* V) {
    if (V->d_gptr) return FGPU_OK;
    const DevPattern& P = *V->pattern;
    const int n = V->n;
    const int64_t nt = V->mesh->nt, nnz = P.nnz;
    const int64_t contrib = nt * n * n;
    if (contrib >= (int64_t)UINT32_MAX || nt * (int64_t)(n * (n + 1) / 2) >= ((int64_t)1 << 31)) {
        ctx->err = "gather map: more than 2^32 contributions or 2^31 buffered entries";
        return FGPU_ERR_INVALID;
    }
    if (!V->d_pos) { ctx->err = "gather map: no position table"; return FGPU_ERR_INVALID; }
    if (n > 32) { ctx->err = "gather map: more than 32 local dofs"; return FGPU_ERR_INVALID; }
    // upper-triangle index of (min(i,j), max(i,j)) in the element buffer's row-major (i <= j) order
    std::vector<uint16_t> htri((size_t)n * n);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            const int a = std::min(i, j), b = std::max(i, j);
            htri[(size_t)i * n + j] = (uint16_t)(a * n - a * (a - 1) / 2 + (b - a));
        }
    uint16_t* d_tri = nullptr;
    uint32_t *cnt = nullptr, *gptr = nullptr, *gidx = nullptr;
    cudaError_t e = cudaMalloc(&d_tri, htri.size() * sizeof(uint16_t));
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_tri, htri.data(), htri.size() * sizeof(uint16_t), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMalloc(&cnt, nnz * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&gptr, (nnz + 1) * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&gidx, contrib * sizeof(uint32_t));
    if (e != cudaSuccess) {
        cudaGetLastError();
        cudaFree(d_tri); cudaFree(cnt); cudaFree(gptr); cudaFree(gidx);
        ctx->err = "gather map: allocation failed";
        return FGPU_ERR_ALLOC;
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    cudaMemsetAsync(cnt, 0, nnz * sizeof(uint32_t), ctx->stream);
    map_count_kernel<<<sms * 16, 256, 0, ctx->stream>>>(nt, n, V->d_l2n, P.d_ia, V->d_pos, cnt);
    uint64_t total = 0;
    int rcs = scan_u32(ctx, cnt, gptr, nnz, &total);
    if (rcs) { cudaFree(d_tri); cudaFree(cnt); cudaFree(gptr); cudaFree(gidx); return rcs; }
    map_fill_kernel<<<sms * 8, 256, 0, ctx->stream>>>(P.nrows, n, n * (n + 1) / 2, P.d_ia, V->d_inc_ptr, V->d_inc, V->d_pos,
                                                      d_tri, gptr, gidx, ctx->d_status);
    ctx->launches += 2;
    e = cudaGetLastError();
    cudaStreamSynchronize(ctx->stream);
    cudaFree(cnt);
    cudaFree(d_tri);
    if (e != cudaSuccess) {
        cudaFree(gptr); cudaFree(gidx);
        ctx->err = std::string("gather map: ") + cudaGetErrorString(e);
        return FGPU_ERR_CUDA;
    }
    V->d_gptr = gptr;
    V->d_gidx = gidx;
    return FGPU_OK;
}

// Launch shape of the two-phase kernels: threads per block and blocks per SM of the element kernel
// and of the gather, and the gather's contributions per load batch. None changes the values.
struct TwoPhaseShape {
    int el_threads = 256, el_bpsm = 16, g_threads = 256, g_bpsm = 32, g_batch = 4, g_pipe = 0;
};

template <int MODE, int N>
static void launch_element_tri(fgpu_ctx* ctx, fgpu_matrix* A, const DevTables* tab, const GeoIn* geo, int sms,
                               const TwoPhaseShape& sh) {
    const int64_t nt = A->space->mesh->nt;
    const int64_t warps = (nt + 31) / 32, wpb = sh.el_threads / 32;       // 32 elements per warp
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((warps + wpb - 1) / wpb, (int64_t)sms * sh.el_bpsm));
    element_tri_kernel<MODE, N><<<(int)blocks, sh.el_threads, 0, ctx->stream>>>(nt, *geo, tab->d_T7th, tab->d_T7tl, A->d_kbuf,
                                                                             ctx->d_status);
}

template <int MODE>
static void launch_gather_map(fgpu_ctx* ctx, fgpu_matrix* A, int sms, const TwoPhaseShape& sh, int accumulate, double* hout) {
    const fgpu_space* V = A->space;
    const int64_t nnz = A->pattern->nnz;
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((nnz + sh.g_threads - 1) / sh.g_threads, (int64_t)sms * sh.g_bpsm));
    if (sh.g_pipe) {
        switch (sh.g_batch) {
            case 2: gather_map_pipe_kernel<MODE, 2><<<(int)blocks, sh.g_threads, 0, ctx->stream>>>(nnz, V->d_gptr, V->d_gidx, A->d_kbuf, A->d_val, accumulate, hout); break;
            case 8: gather_map_pipe_kernel<MODE, 8><<<(int)blocks, sh.g_threads, 0, ctx->stream>>>(nnz, V->d_gptr, V->d_gidx, A->d_kbuf, A->d_val, accumulate, hout); break;
            default: gather_map_pipe_kernel<MODE, 4><<<(int)blocks, sh.g_threads, 0, ctx->stream>>>(nnz, V->d_gptr, V->d_gidx, A->d_kbuf, A->d_val, accumulate, hout); break;
        }
        return;
    }
    switch (sh.g_batch) {
        case 2: gather_map_kernel<MODE, 2><<<(int)blocks, sh.g_threads, 0, ctx->stream>>>(nnz, V->d_gptr, V->d_gidx, A->d_kbuf, A->d_val, accumulate, hout); break;
        case 8: gather_map_kernel<MODE, 8><<<(int)blocks, sh.g_threads, 0, ctx->stream>>>(nnz, V->d_gptr, V->d_gidx, A->d_kbuf, A->d_val, accumulate, hout); break;
        default: gather_map_kernel<MODE, 4><<<(int)blocks, sh.g_threads, 0, ctx->stream>>>(nnz, V->d_gptr, V->d_gidx, A->d_kbuf, A->d_val, accumulate, hout); break;
    }
}

// median of 5 timed launches (after one warm-up) of fn on the context's stream, in ms
template <class F>
static float median_ms(fgpu_ctx* ctx, F&& fn) {
    cudaEvent_t ev[6];
    for (auto& e : ev) cudaEventCreate(&e);
    fn();
    for (int r = 0; r < 5; ++r) {
        cudaEventRecord(ev[r], ctx->stream);
        fn();
    }
    cudaEventRecord(ev[5], ctx->stream);
    cudaEventSynchronize(ev[5]);
    float t[5];
    for (int r = 0; r < 5; ++r) cudaEventElapsedTime(&t[r], ev[r], ev[r + 1]);
    for (auto& e : ev) cudaEventDestroy(e);
    std::sort(t, t + 5);
    ctx->launches += 6;
    return t[2];
}

// Time the candidate shapes on the real inputs (the element buffer and the values are written by the
// candidates; the assembly that follows overwrites both).
template <int MODE, int N>
static int tune_two_phase(fgpu_ctx* ctx, fgpu_matrix* A, const DevTables* tab, const GeoIn* geo, bool elements, int sms,
                          TwoPhaseShape& best) {
    float best_ms = 1e30f;
    TwoPhaseShape s = best;
    for (int th : {128, 256})
        for (int bp : {4, 8, 16, 32}) {
            if (!elements) break;                  // the tensor-core element kernel has its own shape
            s.el_threads = th;
            s.el_bpsm = bp;
            const float ms = median_ms(ctx, [&] { launch_element_tri<MODE, N>(ctx, A, tab, geo, sms, s); });
            if (ms < best_ms) { best_ms = ms; best.el_threads = th; best.el_bpsm = bp; }
        }
    best_ms = 1e30f;
    for (int th : {128, 256})
        for (int bp : {8, 16, 32, 64})
            for (int b : {2, 4, 8}) {
                s.g_threads = th;
                s.g_bpsm = bp;
                s.g_batch = b;
                const float ms = median_ms(ctx, [&] { launch_gather_map<MODE>(ctx, A, sms, s, 0, nullptr); });
                if (ms < best_ms) { best_ms = ms; best.g_threads = th; best.g_bpsm = bp; best.g_batch = b; }
            }
    // the software-pipelined gather, its grid at most the resident blocks (a sweep over the entries)
    for (int th : {128, 256})
        for (int bp : {2, 4, 6, 8})
            for (int b : {2, 4}) {
                s.g_threads = th;
                s.g_bpsm = bp * (256 / th);
                s.g_batch = b;
                s.g_pipe = 1;
                const float ms = median_ms(ctx, [&] { launch_gather_map<MODE>(ctx, A, sms, s, 0, nullptr); });
                if (ms < best_ms) { best_ms = ms; best.g_threads = th; best.g_bpsm = s.g_bpsm; best.g_batch = b; best.g_pipe = 1; }
            }
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

template <int MODE, int N>
static int run_two_phase(fgpu_ctx* ctx, fgpu_matrix* A, const DevTables* tab, const float4* rec, const GeoIn* geo,
                         int accumulate, double* host = nullptr) {
    fgpu_space* V = A->space;
    const int64_t nt = V->mesh->nt;
    constexpr int NTRI = N * (N + 1) / 2;
    const bool tc = MODE == kModeDF64 && (ctx->tensor_cores & FGPU_TC_DF64);
    if (!rec && tc) {
        // the tensor-core element kernel reads the coefficient records from device memory
        const int rc = launch_geometry_df(ctx, V->mesh, geo->kappa, geo->kc, geo->mc, reinterpret_cast<float4*>(A->d_coef), geo->kscale);
        if (rc) return rc;
        rec = reinterpret_cast<const float4*>(A->d_coef);
    }
    if (!V->d_gptr) {
        if (ctx->capturing) { ctx->err = "two-phase assembly: assemble once before capturing (gather map)"; return FGPU_ERR_INVALID; }
        int rc = launch_build_gather_map(ctx, V);
        if (rc) return rc;
    }
    const size_t need = (size_t)nt * NTRI * (MODE == kModeDF64 ? 8 : 4);
    if (A->kbuf_bytes < need) {
        if (ctx->capturing) { ctx->err = "two-phase assembly: assemble once before capturing (element buffer)"; return FGPU_ERR_INVALID; }
        cudaFree(A->d_kbuf);
        A->d_kbuf = nullptr;
        A->kbuf_bytes = 0;
        if (cudaMalloc(&A->d_kbuf, need) != cudaSuccess) { cudaGetLastError(); ctx->err = "two-phase assembly: element buffer allocation failed"; return FGPU_ERR_ALLOC; }
        A->kbuf_bytes = need;
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int64_t nnz = A->pattern->nnz;
    TwoPhaseShape shape;
    const std::string key = "two_phase|" + tune_device_key(ctx->device) + "|P" + std::to_string(V->order) + "|" +
                            (MODE == kModeDF64 ? "f64" : "f32") + "|n2^" + std::to_string(tune_size_class(nnz));
    std::vector<int> tv;
    if (ctx->tune == 0 && tune_lookup(ctx->tune_file, key, tv) && (tv.size() == 5 || tv.size() == 6)) {
        shape = TwoPhaseShape{tv[0], tv[1], tv[2], tv[3], tv[4], tv.size() == 6 ? tv[5] : 0};
    } else if (ctx->tune == 0 && !ctx->capturing && accumulate == 0 && !host) {
        int rc = tune_two_phase<MODE, N>(ctx, A, tab, geo, !tc, sms, shape);
        if (rc) return rc;
        tune_record(ctx->tune_file, key, {shape.el_threads, shape.el_bpsm, shape.g_threads, shape.g_bpsm, shape.g_batch, shape.g_pipe});
    }
    {
        PendingEvent ev;
        prof_begin(ctx, "assemble_elements", ev);
        if (tc) {
            // the df64 element matrices on the tensor cores (bf16 slices, exact level sums)
            const int rc = launch_element_tri_tc(ctx, V->order, nt, rec, tab->d_T7th, tab->d_T7tl, A->d_kbuf);
            if (rc) return rc;
        } else {
            launch_element_tri<MODE, N>(ctx, A, tab, geo, sms, shape);
        }
        prof_end(ctx, ev);
        FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    }
    if (host) return launch_gather_phase_to_host(ctx, A, host, 4);
    PendingEvent ev;
    prof_begin(ctx, "assemble_gather", ev);
    launch_gather_map<MODE>(ctx, A, sms, shape, accumulate, nullptr);
    prof_end(ctx, ev);
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

// Two-phase helpers for element kernels defined elsewhere (curved elements): the gather map and an
// element buffer of at least `need` bytes, then phase 2 for the matrix's precision.
int ensure_two_phase(fgpu_ctx* ctx, fgpu_matrix* A, size_t need) {
    fgpu_space* V = A->space;
    if (!V->d_gptr) {
        if (ctx->capturing) { ctx->err = "two-phase assembly: assemble once before capturing (gather map)"; return FGPU_ERR_INVALID; }
        int rc = launch_build_gather_map(ctx, V);
        if (rc) return rc;
    }
    if (A->kbuf_bytes < need) {
        if (ctx->capturing) { ctx->err = "two-phase assembly: assemble once before capturing (element buffer)"; return FGPU_ERR_INVALID; }
        cudaFree(A->d_kbuf);
        A->d_kbuf = nullptr;
        A->kbuf_bytes = 0;
        if (cudaMalloc(&A->d_kbuf, need) != cudaSuccess) { cudaGetLastError(); ctx->err = "two-phase assembly: element buffer allocation failed"; return FGPU_ERR_ALLOC; }
        A->kbuf_bytes = need;
    }
    return FGPU_OK;
}

int launch_gather_phase(fgpu_ctx* ctx, fgpu_matrix* A, int accumulate) {
    fgpu_space* V = A->space;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int64_t nnz = A->pattern->nnz;
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((nnz + 255) / 256, (int64_t)sms * 32));
    PendingEvent ev;
    prof_begin(ctx, "assemble_gather", ev);
    if (A->precision == FGPU_F32)
        gather_map_kernel<kModeF32><<<(int)blocks, 256, 0, ctx->stream>>>(nnz, V->d_gptr, V->d_gidx, A->d_kbuf, A->d_val, accumulate, nullptr);
    else
        gather_map_kernel<kModeDF64><<<(int)blocks, 256, 0, ctx->stream>>>(nnz, V->d_gptr, V->d_gidx, A->d_kbuf, A->d_val, accumulate, nullptr);
    prof_end(ctx, ev);
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

// Phase 2 in nchunks ranges of CSR entries, each range copied to host memory (pinned for overlap) on
// its own copy stream as soon as its gather ends: the copies of earlier ranges overlap the gathers of
// later ones. FP64 matrices.
int launch_gather_phase_to_host(fgpu_ctx* ctx, fgpu_matrix* A, double* host, int nchunks) {
    fgpu_space* V = A->space;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int64_t nnz = A->pattern->nnz;
    nchunks = std::max(1, std::min(nchunks, 4));
    if (!ctx->copy_streams[0]) {
        for (int i = 0; i < 4; ++i) FGPU_CUDA_CHECK(ctx, cudaStreamCreateWithFlags(&ctx->copy_streams[i], cudaStreamNonBlocking));
        for (int i = 0; i < 5; ++i) FGPU_CUDA_CHECK(ctx, cudaEventCreateWithFlags(&ctx->copy_events[i], cudaEventDisableTiming));
    }
    // direct stores: the gather writes every value to device memory and to the mapped host buffer.
    // (Element kernel and gather in eight ranges each, a range of entries gathered on a side stream
    // once the element ranges it reads were done, measured slower: 16.4 against 19.2 Gnnz/s end to
    // end at P2 64^3; so was a variant with the elements ordered by the first of four row chunks that
    // reads them: 16.8-16.9 against 19.7 Gnnz/s, with a gather grid of 4 or 32 blocks per SM.)
    double* hdev = nullptr;
    if (ctx->host_transfer != FGPU_HOST_TRANSFER_COPY) {
        cudaPointerAttributes pa{};
        if (cudaPointerGetAttributes(&pa, host) == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer)
            hdev = static_cast<double*>(pa.devicePointer);
        else
            cudaGetLastError();
        if (!hdev && ctx->host_transfer == FGPU_HOST_TRANSFER_DIRECT) {
            ctx->err = "direct host transfer: the host buffer is not page-locked and mapped";
            return FGPU_ERR_INVALID;
        }
    }
    if (hdev) {
        const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((nnz + 255) / 256, (int64_t)sms * 32));
        PendingEvent ev;
        prof_begin(ctx, "assemble_gather", ev);
        gather_map_kernel<kModeDF64><<<(int)blocks, 256, 0, ctx->stream>>>(nnz, V->d_gptr, V->d_gidx, A->d_kbuf, A->d_val, 0, hdev);
        prof_end(ctx, ev);
        ctx->launches++;
        FGPU_CUDA_CHECK(ctx, cudaGetLastError());
        FGPU_CUDA_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
        return FGPU_OK;
    }
    const int64_t chunk = ((nnz + nchunks - 1) / nchunks + 255) & ~(int64_t)255;
    PendingEvent ev;
    prof_begin(ctx, "assemble_gather", ev);
    for (int c = 0; c < nchunks; ++c) {
        const int64_t k0 = (int64_t)c * chunk;
        if (k0 >= nnz) break;
        const int64_t k1 = std::min(nnz, k0 + chunk);
        const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((k1 - k0 + 255) / 256, (int64_t)sms * 32));
        gather_map_kernel<kModeDF64><<<(int)blocks, 256, 0, ctx->stream>>>(k1 - k0, V->d_gptr + k0, V->d_gidx, A->d_kbuf,
                                                                         (double*)A->d_val + k0, 0, nullptr);
        ctx->launches++;
        FGPU_CUDA_CHECK(ctx, cudaGetLastError());
        FGPU_CUDA_CHECK(ctx, cudaEventRecord(ctx->copy_events[c], ctx->stream));
        FGPU_CUDA_CHECK(ctx, cudaStreamWaitEvent(ctx->copy_streams[c], ctx->copy_events[c], 0));
        FGPU_CUDA_CHECK(ctx, cudaMemcpyAsync(host + k0, (const double*)A->d_val + k0, (k1 - k0) * sizeof(double),
                                             cudaMemcpyDeviceToHost, ctx->copy_streams[c]));
    }
    prof_end(ctx, ev);
    for (int c = 0; c < nchunks; ++c) FGPU_CUDA_CHECK(ctx, cudaStreamSynchronize(ctx->copy_streams[c]));
    return FGPU_OK;
}

int launch_rhs_gather(fgpu_ctx* ctx, const fgpu_space* V, const double* d_work, double* d_out, int accumulate) {
    const int64_t nn = V->topo.nnodes;
    const int64_t gb = std::max<int64_t>(1, std::min<int64_t>((nn + 255) / 256, 152 * 16));
    PendingEvent ev;
    prof_begin(ctx, "rhs_gather", ev);
    rhs_gather_kernel<<<(int)gb, 256, 0, ctx->stream>>>(nn, V->n, V->ncomp, V->d_inc_ptr, V->d_inc, d_work, d_out, accumulate);
    prof_end(ctx, ev);
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

int launch_assemble_two_phase_host(fgpu_ctx* ctx, fgpu_matrix* A, const DevTables* tab, const float4* rec, const GeoIn* geo,
                                   double* host) {
    if (A->ncomp != 1 || A->precision != FGPU_F64) { ctx->err = "assemble to host: scalar FP64 matrices"; return FGPU_ERR_INVALID; }
    switch (A->space->order) {
        case 1: return run_two_phase<kModeDF64, 4>(ctx, A, tab, rec, geo, 0, host);
        case 2: return run_two_phase<kModeDF64, 10>(ctx, A, tab, rec, geo, 0, host);
        case 3: return run_two_phase<kModeDF64, 20>(ctx, A, tab, rec, geo, 0, host);
        default: ctx->err = "unsupported order"; return FGPU_ERR_INVALID;
    }
}

int launch_assemble_two_phase(fgpu_ctx* ctx, fgpu_matrix* A, const DevTables* tab, const float4* rec, const GeoIn* geo, int accumulate) {
    const int order = A->space->order;
    const bool f32 = A->precision == FGPU_F32;
    if (A->ncomp != 1) { ctx->err = "Laplace/mass form needs a scalar space"; return FGPU_ERR_INVALID; }
    if (order == 1) return f32 ? run_two_phase<kModeF32, 4>(ctx, A, tab, rec, geo, accumulate)
                               : run_two_phase<kModeDF64, 4>(ctx, A, tab, rec, geo, accumulate);
    if (order == 2) return f32 ? run_two_phase<kModeF32, 10>(ctx, A, tab, rec, geo, accumulate)
                               : run_two_phase<kModeDF64, 10>(ctx, A, tab, rec, geo, accumulate);
    if (order == 3) return f32 ? run_two_phase<kModeF32, 20>(ctx, A, tab, rec, geo, accumulate)
                               : run_two_phase<kModeDF64, 20>(ctx, A, tab, rec, geo, accumulate);
    ctx->err = "unsupported order";
    return FGPU_ERR_INVALID;
}

// ---------------------------------------------------------------------------
// Two-phase vector P1/P2 linear elasticity in df64 (or binary32).
// lambda div u div v + 2 mu eps(u):eps(v) (qs_elasticity.cpp:46-63): for the
// scalar pair (i, j) with X_ab = S_ab(i, j) (reference tensors) and
// Y = B X B^T (B = K^-T), the 3x3 block of K_e at rows (c, i), columns (d, j) is
//   lambda J Y_cd + mu J Y_dc + delta_cd mu J tr(Y).
// Records: 24 floats per element: hi parts of (B_00..B_22, lambda J, mu J, 0), then lo parts.
// Phase 1 stores the blocks of the pairs i <= j (n(n+1)/2 x 9 values per element);
// phase 2, one warp per scalar pattern row, lanes over its entries, sums the 9
// entries of each node pair over the contributions of the gather map in element
// order (a contribution with li > lj reads its block transposed) and writes them
// into the expanded CSR (row 3m+c, columns 3n'+d).
// ---------------------------------------------------------------------------
__global__ void geometry_el_df_kernel(int64_t nt, const double* __restrict__ xyz, const int32_t* __restrict__ tets, double lam,
                                      double mu, float4* __restrict__ rec, int* __restrict__ status) {
    const df lamd = d2df(lam), mud = d2df(mu);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nt; e += (int64_t)gridDim.x * blockDim.x) {
        const int4 t = *reinterpret_cast<const int4*>(tets + 4 * e);
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
        const df det = df_add(df_add(df_mul(K[0], C[0]), df_mul(K[1], C[1])), df_mul(K[2], C[2]));
        const df J = det.hi < 0.0f ? df_neg(det) : det;
        if (!(J.hi > 0.0f) || !isfinite(J.hi)) atomicOr(status, kStatusBadElement);
        const df inv = df_recip(det);
        df v[12];
#pragma unroll
        for (int i = 0; i < 9; ++i) v[i] = df_mul(C[i], inv);      // B = C / det = K^-T
        v[9] = df_mul(lamd, J);
        v[10] = df_mul(mud, J);
        v[11] = df{0.0f, 0.0f};
        float4* o = rec + 6 * e;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            o[q] = make_float4(v[4 * q].hi, v[4 * q + 1].hi, v[4 * q + 2].hi, v[4 * q + 3].hi);
            o[3 + q] = make_float4(v[4 * q].lo, v[4 * q + 1].lo, v[4 * q + 2].lo, v[4 * q + 3].lo);
        }
    }
}

int launch_geometry_el_df(fgpu_ctx* ctx, const fgpu_mesh* mesh, double lam, double mu, float4* d_rec) {
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((mesh->nt + 255) / 256, 152 * 16));
    PendingEvent ev;
    prof_begin(ctx, "geometry", ev);
    geometry_el_df_kernel<<<(int)blocks, 256, 0, ctx->stream>>>(mesh->nt, mesh->d_xyz, mesh->d_tets, lam, mu, d_rec, ctx->d_status);
    prof_end(ctx, ev);
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

// one 3x3 block from the pair's reference tensors (Xh/Xl: S_ab hi/lo) and the
// element's B, lambda J, mu J; df64 or binary32 (MODE)
template <int MODE>
__device__ __forceinline__ void el_block(const float* Xh, const float* Xl, const df* B, df lJ, df mJ, df* out) {
    if (MODE == kModeDF64) {
        df X[9], Z[9], Y[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) X[k] = quick_two_sum(Xh[k], Xl[k]);
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int d = 0; d < 3; ++d)
                Z[a * 3 + d] = df_add(df_add(df_mul(X[a * 3 + 0], B[d * 3 + 0]), df_mul(X[a * 3 + 1], B[d * 3 + 1])),
                                      df_mul(X[a * 3 + 2], B[d * 3 + 2]));
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int d = 0; d < 3; ++d)
                Y[c * 3 + d] = df_add(df_add(df_mul(B[c * 3 + 0], Z[0 * 3 + d]), df_mul(B[c * 3 + 1], Z[1 * 3 + d])),
                                      df_mul(B[c * 3 + 2], Z[2 * 3 + d]));
        const df tr = df_add(df_add(Y[0], Y[4]), Y[8]);
        const df mtr = df_mul(mJ, tr);
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                df v = df_add(df_mul(lJ, Y[c * 3 + d]), df_mul(mJ, Y[d * 3 + c]));
                if (c == d) v = df_add(v, mtr);
                out[c * 3 + d] = v;
            }
    } else {
        float Bf[9], Z[9], Y[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) Bf[k] = B[k].hi;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int d = 0; d < 3; ++d)
                Z[a * 3 + d] = fmaf(Xh[a * 3 + 0], Bf[d * 3 + 0], fmaf(Xh[a * 3 + 1], Bf[d * 3 + 1], Xh[a * 3 + 2] * Bf[d * 3 + 2]));
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int d = 0; d < 3; ++d)
                Y[c * 3 + d] = fmaf(Bf[c * 3 + 0], Z[0 * 3 + d], fmaf(Bf[c * 3 + 1], Z[1 * 3 + d], Bf[c * 3 + 2] * Z[2 * 3 + d]));
        const float tr = Y[0] + Y[4] + Y[8];
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                float v = fmaf(lJ.hi, Y[c * 3 + d], mJ.hi * Y[d * 3 + c]);
                if (c == d) v = fmaf(mJ.hi, tr, v);
                out[c * 3 + d] = df{v, 0.0f};
            }
    }
}

template <int MODE, int N>
__global__ void __launch_bounds__(128) element_el_kernel(int64_t nt, const float4* __restrict__ rec, const float* __restrict__ Shg,
                                                         const float* __restrict__ Slg, void* __restrict__ kbuf) {
    constexpr int NTRI = N * (N + 1) / 2;
    __shared__ float Sh[9 * NTRI];
    __shared__ float Sl[9 * NTRI];
    for (int k = threadIdx.x; k < 9 * NTRI; k += blockDim.x) {
        Sh[k] = Shg[k];
        Sl[k] = Slg[k];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t e = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); e < nt; e += nw) {   // one warp per element
        const float4* rp = rec + 6 * e;
        df B[9], lJ, mJ;
        {
            float h[12], l[12];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                const float4 a = __ldg(rp + q), b = __ldg(rp + 3 + q);
                h[4 * q] = a.x; h[4 * q + 1] = a.y; h[4 * q + 2] = a.z; h[4 * q + 3] = a.w;
                l[4 * q] = b.x; l[4 * q + 1] = b.y; l[4 * q + 2] = b.z; l[4 * q + 3] = b.w;
            }
#pragma unroll
            for (int k = 0; k < 9; ++k) B[k] = df{h[k], l[k]};
            lJ = df{h[9], l[9]};
            mJ = df{h[10], l[10]};
        }
        for (int t = lane; t < NTRI; t += 32) {
            float Xh[9], Xl[9];
#pragma unroll
            for (int ab = 0; ab < 9; ++ab) {
                Xh[ab] = Sh[ab * NTRI + t];
                Xl[ab] = Sl[ab * NTRI + t];
            }
            df blk[9];
            el_block<MODE>(Xh, Xl, B, lJ, mJ, blk);
            const int64_t o = (e * NTRI + t) * 9;
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                if (MODE == kModeDF64) reinterpret_cast<float2*>(kbuf)[o + k] = make_float2(blk[k].hi, blk[k].lo);
                else reinterpret_cast<float*>(kbuf)[o + k] = blk[k].hi;
            }
        }
    }
}

template <int MODE>
__global__ void __launch_bounds__(256) gather_el_kernel(int64_t nrows, const int64_t* __restrict__ sia, const uint32_t* __restrict__ gptr,
                                                        const uint32_t* __restrict__ gidx, const void* __restrict__ kbuf,
                                                        void* __restrict__ valv, int accumulate) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t m = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp; m < nrows; m += nw) {
        const int64_t s0 = sia[m];
        const int len = (int)(sia[m + 1] - s0);
        for (int pos = lane; pos < len; pos += 32) {
            const int64_t ks = s0 + pos;
            const uint32_t p0 = __ldg(gptr + ks), p1 = __ldg(gptr + ks + 1);
            // (a compensated sum per component, as in gather_map_kernel, took 4.71 against 4.25 ms for the
            // P2 48^3 elasticity assembly: the nine components' two accumulators)
            df acc[9];
            float accf[9];
#pragma unroll
            for (int k = 0; k < 9; ++k) { acc[k] = df{0.0f, 0.0f}; accf[k] = 0.0f; }
            for (uint32_t p = p0; p < p1; ++p) {
                const uint32_t g = __ldg(gidx + p);
                const bool tr = (g & 0x80000000u) != 0;
                const int64_t base = (int64_t)(g & 0x7FFFFFFFu) * 9;
#pragma unroll
                for (int c = 0; c < 3; ++c)
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        const int k = tr ? d * 3 + c : c * 3 + d;
                        if (MODE == kModeDF64) {
                            const float2 v = __ldg(reinterpret_cast<const float2*>(kbuf) + base + k);
                            acc[c * 3 + d] = p == p0 ? df{v.x, v.y} : df_add(acc[c * 3 + d], df{v.x, v.y});
                        } else {
                            const float v = __ldg(reinterpret_cast<const float*>(kbuf) + base + k);
                            accf[c * 3 + d] = p == p0 ? v : f_add(accf[c * 3 + d], v);
                        }
                    }
            }
#pragma unroll
            for (int c = 0; c < 3; ++c)
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    const int64_t o = 9 * s0 + (int64_t)c * 3 * len + 3 * pos + d;
                    if (MODE == kModeDF64) {
                        double* out = reinterpret_cast<double*>(valv) + o;
                        df a = acc[c * 3 + d];
                        if (accumulate) a = df_add(d2df(*out), a);
                        *out = df2d(a);
                    } else {
                        float* out = reinterpret_cast<float*>(valv) + o;
                        *out = accumulate ? f_add(*out, accf[c * 3 + d]) : accf[c * 3 + d];
                    }
                }
        }
    }
}

template <int MODE, int N>
static int run_el_two_phase(fgpu_ctx* ctx, fgpu_matrix* A, const DevTables* tab, const float4* rec, int accumulate) {
    fgpu_space* V = A->space;
    const int64_t nt = V->mesh->nt;
    constexpr int NTRI = N * (N + 1) / 2;
    if (!V->d_gptr) {
        if (ctx->capturing) { ctx->err = "two-phase assembly: assemble once before capturing (gather map)"; return FGPU_ERR_INVALID; }
        int rc = launch_build_gather_map(ctx, V);
        if (rc) return rc;
    }
    const size_t need = (size_t)nt * NTRI * 9 * (MODE == kModeDF64 ? 8 : 4);
    if (A->kbuf_bytes < need) {
        if (ctx->capturing) { ctx->err = "two-phase assembly: assemble once before capturing (element buffer)"; return FGPU_ERR_INVALID; }
        cudaFree(A->d_kbuf);
        A->d_kbuf = nullptr;
        A->kbuf_bytes = 0;
        if (cudaMalloc(&A->d_kbuf, need) != cudaSuccess) { cudaGetLastError(); ctx->err = "two-phase assembly: element buffer allocation failed"; return FGPU_ERR_ALLOC; }
        A->kbuf_bytes = need;
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    {
        const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((nt + 3) / 4, (int64_t)sms * 16));
        PendingEvent ev;
        prof_begin(ctx, "assemble_elements", ev);
        element_el_kernel<MODE, N><<<(int)blocks, 128, 0, ctx->stream>>>(nt, rec, tab->d_Sth, tab->d_Stl, A->d_kbuf);
        prof_end(ctx, ev);
        FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    }
    const DevPattern& P = *A->pattern;
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((P.nrows + 7) / 8, (int64_t)sms * 16));
    PendingEvent ev;
    prof_begin(ctx, "assemble_gather_elasticity", ev);
    gather_el_kernel<MODE><<<(int)blocks, 256, 0, ctx->stream>>>(P.nrows, P.d_ia, V->d_gptr, V->d_gidx, A->d_kbuf, A->d_val, accumulate);
    prof_end(ctx, ev);
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

int launch_assemble_elasticity_two_phase(fgpu_ctx* ctx, fgpu_matrix* A, const DevTables* tab, const float4* rec, int accumulate) {
    const int order = A->space->order;
    const bool f32 = A->precision == FGPU_F32;
    if (A->ncomp != 3) { ctx->err = "elasticity needs a 3-component space"; return FGPU_ERR_INVALID; }
    if (order == 1) return f32 ? run_el_two_phase<kModeF32, 4>(ctx, A, tab, rec, accumulate)
                               : run_el_two_phase<kModeDF64, 4>(ctx, A, tab, rec, accumulate);
    if (order == 2) return f32 ? run_el_two_phase<kModeF32, 10>(ctx, A, tab, rec, accumulate)
                               : run_el_two_phase<kModeDF64, 10>(ctx, A, tab, rec, accumulate);
    ctx->err = "elasticity supports P1 and P2";
    return FGPU_ERR_INVALID;
}

int launch_assemble_gather_df(fgpu_ctx* ctx, fgpu_matrix* A, const DevTables* tab, const float4* rec, int accumulate) {
    const int order = A->space->order;
    const bool f32 = A->precision == FGPU_F32;
    if (A->ncomp != 1) { ctx->err = "Laplace/mass form needs a scalar space"; return FGPU_ERR_INVALID; }
    if (order == 1) return f32 ? run_gather_row<kModeF32, 4, 8>(ctx, A, tab, rec, accumulate)
                               : run_gather_row<kModeDF64, 4, 8>(ctx, A, tab, rec, accumulate);
    if (order == 2) return f32 ? run_gather_row<kModeF32, 10, 3>(ctx, A, tab, rec, accumulate)
                               : run_gather_row<kModeDF64, 10, 3>(ctx, A, tab, rec, accumulate);
    if (order == 3) return f32 ? run_gather_row<kModeF32, 20, 1>(ctx, A, tab, rec, accumulate)
                               : run_gather_row<kModeDF64, 20, 1>(ctx, A, tab, rec, accumulate);
    ctx->err = "unsupported order";
    return FGPU_ERR_INVALID;
}

}  // namespace fgpu

// ===========================================================================
// Error norms against u = sin(pi x) sin(pi y) sin(pi z): normL2 / normH1
// (feelpp/feel/feelvf/norml2.hpp:37, normh1.hpp = integrate(elements, (u_h - u)^2)).
// One thread per element in binary64; per-block partial sums, summed on the host.
// ===========================================================================
namespace fgpu {

template <int N>
__global__ void norms_sine_kernel(int64_t nt, const double* __restrict__ xyz, const int32_t* __restrict__ tets,
                                  const int32_t* __restrict__ l2n, const double* __restrict__ u, int Q,
                                  const double* __restrict__ qx, const double* __restrict__ qw, const double* __restrict__ phi,
                                  const double* __restrict__ dphi, double* __restrict__ partial) {
    __shared__ double s0[256], s1[256];
    double a0 = 0.0, a1 = 0.0;
    const double pi = 3.141592653589793;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nt; e += (int64_t)gridDim.x * blockDim.x) {
        const int4 t = *reinterpret_cast<const int4*>(tets + 4 * e);
        const int vv[4] = {t.x, t.y, t.z, t.w};
        double X[4][3];
#pragma unroll
        for (int v = 0; v < 4; ++v)
#pragma unroll
            for (int d = 0; d < 3; ++d) X[v][d] = xyz[3 * (int64_t)vv[v] + d];
        double K[9];
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int r = 0; r < 3; ++r) K[r * 3 + c] = 0.5 * X[c + 1][r] - 0.5 * X[0][r];
        const double c00 = K[4] * K[8] - K[5] * K[7], c01 = K[5] * K[6] - K[3] * K[8], c02 = K[3] * K[7] - K[4] * K[6];
        const double det = K[0] * c00 + K[1] * c01 + K[2] * c02;
        const double cof[9] = {c00, c01, c02,
                               K[2] * K[7] - K[1] * K[8], K[0] * K[8] - K[2] * K[6], K[1] * K[6] - K[0] * K[7],
                               K[1] * K[5] - K[2] * K[4], K[2] * K[3] - K[0] * K[5], K[0] * K[4] - K[1] * K[3]};
        const double J = fabs(det);
        double ue[N];
#pragma unroll
        for (int i = 0; i < N; ++i) ue[i] = u[l2n[e * N + i]];
        for (int q = 0; q < Q; ++q) {
            const double xh = qx[3 * q], yh = qx[3 * q + 1], zh = qx[3 * q + 2];
            const double g[4] = {-0.5 * (1 + xh + yh + zh), 0.5 * (1 + xh), 0.5 * (1 + yh), 0.5 * (1 + zh)};
            double p[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) p[d] = X[0][d] * g[0] + X[1][d] * g[1] + X[2][d] * g[2] + X[3][d] * g[3];
            double uh = 0.0, gh[3] = {0.0, 0.0, 0.0};
#pragma unroll
            for (int i = 0; i < N; ++i) {
                uh += ue[i] * phi[q * N + i];
#pragma unroll
                for (int a = 0; a < 3; ++a) gh[a] += ue[i] * dphi[(q * N + i) * 3 + a];
            }
            // physical gradient B ghat, B = cof / det
            double gp[3];
#pragma unroll
            for (int r = 0; r < 3; ++r) gp[r] = (cof[3 * r] * gh[0] + cof[3 * r + 1] * gh[1] + cof[3 * r + 2] * gh[2]) / det;
            const double sx = sin(pi * p[0]), sy = sin(pi * p[1]), sz = sin(pi * p[2]);
            const double cx = cos(pi * p[0]), cy = cos(pi * p[1]), cz = cos(pi * p[2]);
            const double ex = uh - sx * sy * sz;
            const double g0 = gp[0] - pi * cx * sy * sz, g1 = gp[1] - pi * sx * cy * sz, g2 = gp[2] - pi * sx * sy * cz;
            const double wJ = qw[q] * J;
            a0 += wJ * ex * ex;
            a1 += wJ * (g0 * g0 + g1 * g1 + g2 * g2);
        }
    }
    s0[threadIdx.x] = a0;
    s1[threadIdx.x] = a1;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            s0[threadIdx.x] += s0[threadIdx.x + o];
            s1[threadIdx.x] += s1[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[2 * blockIdx.x] = s0[0];
        partial[2 * blockIdx.x + 1] = s1[0];
    }
}

int launch_norms_sine(fgpu_ctx* ctx, const fgpu_space* V, const DevTables* tab, const double* d_u, double* l2, double* h1) {
    const fgpu_mesh* M = V->mesh;
    const int threads = 256;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((M->nt + threads - 1) / threads, 152 * 8));
    double* partial = nullptr;
    FGPU_CUDA_CHECK(ctx, cudaMalloc(&partial, 2 * blocks * sizeof(double)));
    switch (V->n) {
        case 4: norms_sine_kernel<4><<<blocks, threads, 0, ctx->stream>>>(M->nt, M->d_xyz, M->d_tets, V->d_l2n, d_u, tab->Q, tab->d_qx, tab->d_qw, tab->d_phi, tab->d_dphi, partial); break;
        case 10: norms_sine_kernel<10><<<blocks, threads, 0, ctx->stream>>>(M->nt, M->d_xyz, M->d_tets, V->d_l2n, d_u, tab->Q, tab->d_qx, tab->d_qw, tab->d_phi, tab->d_dphi, partial); break;
        case 20: norms_sine_kernel<20><<<blocks, threads, 0, ctx->stream>>>(M->nt, M->d_xyz, M->d_tets, V->d_l2n, d_u, tab->Q, tab->d_qx, tab->d_qw, tab->d_phi, tab->d_dphi, partial); break;
        default: cudaFree(partial); ctx->err = "unsupported order"; return FGPU_ERR_INVALID;
    }
    ctx->launches++;
    std::vector<double> h(2 * blocks);
    cudaError_t e = cudaMemcpyAsync(h.data(), partial, h.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(partial);
    if (e != cudaSuccess) { ctx->err = cudaGetErrorString(e); return FGPU_ERR_CUDA; }
    double s0 = 0, s1 = 0;
    for (int b = 0; b < blocks; ++b) { s0 += h[2 * b]; s1 += h[2 * b + 1]; }
    *l2 = std::sqrt(s0);
    *h1 = std::sqrt(s1);
    return FGPU_OK;
}

}  // namespace fgpu
