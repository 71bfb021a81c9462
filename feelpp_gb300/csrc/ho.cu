// Curved (P2-geometry) tetrahedra: the GEOMAP_HO path of the reference
// (feelpp/feel/feelpoly/geomap.hpp: for a non-linear map the context
// recomputes K = G grad(psi)^T, J and B = K^-T at every quadrature point,
// :1014-1042, :2310-2350) for the scalar Laplace/mass form and the load vector.
//
// The map is x(xh) = sum_g X_g psi_g(xh) with the 10 P2 Lagrange functions
// (vertices, then the edge nodes in e2p order). Element matrices by quadrature:
//   K_e(i, j) = sum_q dphi_i(q)^T G_q dphi_j(q) + m_q phi_i(q) phi_j(q),
//   G_q = w_q |det K_q| kappa B_q^T B_q,  m_q = w_q |det K_q| mass,
// where dphi are reference gradients. One warp per element: the lanes first
// take one quadrature point each and form G_q, m_q (the map, its cofactors,
// determinant and inverse) in double-float on the FP32 pipes (binary64 runs at
// 1/71 of the binary32 rate here; binary32 for FP32 matrices), stored in shared
// memory; then for every
// q the lanes form W_q = G_q dphi_j(q) for one local dof each, and each lane
// adds dphi_i . W_j + m_q phi_i phi_j into the upper-triangle entries it owns
// (double-float on the FP32 pipes for FP64 matrices, binary32 for FP32). The
// element matrices go to the two-phase element buffer and the gather map sums
// them per CSR entry in element order, as for affine elements.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "df64.h"
#include "fgpu_core.h"
#include "tc_ptx.cuh"

namespace fgpu {

namespace {

enum HoMode { kHoF32 = 0, kHoDF64 = 1 };

// G geometric nodes per element: 10 (P2-geometry tetrahedra) or 8 (Q1 hexahedra)
template <int N, int G>
struct HoLimits {
    // tetrahedra: quadrature degree <= 5 / 7 / 8; hexahedra: m^3 Gauss points, m <= 4 (Q1) / 3 (Q2)
    static constexpr int QMAX = G == 8 ? (N == 8 ? 64 : 27) : N == 4 ? 14 : N == 10 ? 31 : 43;
};

struct HoTables {
    int n = 0, Q = 0, ntri = 0;
    float* d_dh = nullptr;     // Q n 3: reference gradients of the space's basis (df64 hi)
    float* d_dl = nullptr;     //        (df64 lo)
    float* d_ph = nullptr;     // Q n: basis values (df64 hi)
    float* d_pl = nullptr;     //      (df64 lo)
    double* d_phi = nullptr;   // Q n (binary64, load vector)
    int G = 10;                // geometric nodes per element
    double* d_gd = nullptr;    // Q G 3: reference gradients of the geometric basis (P2 tet / Q1 hex)
    double* d_gp = nullptr;    // Q G: geometric basis values
    double* d_qw = nullptr;    // Q
    float* d_gdh = nullptr;    // Q 10 3: d_gd as double-float (hi)
    float* d_gdl = nullptr;    //                               (lo)
    float* d_qwh = nullptr;    // Q: weights as double-float (hi)
    float* d_qwl = nullptr;    //                            (lo)
    uint8_t* d_ti = nullptr;   // ntri: row of each upper-triangle entry
    uint8_t* d_tj = nullptr;   // ntri: column
    float* d_tcB = nullptr;    // tensor-core B operand: per chunk of points, per accumulator, tf32 hi / lo
    std::vector<double> dphi, phi;   // Q n 3, Q n (host copies for building d_tcB)
};

std::mutex g_ho_mutex;
std::map<std::tuple<int, int, int>, HoTables*> g_ho_tabs;

template <typename T>
cudaError_t up(T** dst, const std::vector<T>& v) {
    cudaError_t e = cudaMalloc(dst, std::max<size_t>(v.size(), 1) * sizeof(T));
    if (e == cudaSuccess && !v.empty()) e = cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    return e;
}

// hex: Q1/Q2 hexahedra (geometry Q1), else P-order tetrahedra with P2 geometry
HoTables* get_ho_tables(fgpu_ctx* ctx, int order, int qdeg, bool hex = false) {
    std::lock_guard<std::mutex> lock(g_ho_mutex);
    const auto key = std::make_tuple(ctx->device, order + (hex ? 100 : 0), qdeg);
    auto it = g_ho_tabs.find(key);
    if (it != g_ho_tabs.end()) return it->second;
    RefTables R, G;
    std::string err;
    const bool ok = hex ? build_hex_ref_tables(order, qdeg, R, err) && build_hex_ref_tables(1, qdeg, G, err)
                        : build_ref_tables(order, qdeg, R, err) && build_ref_tables(2, qdeg, G, err);
    if (!ok) { ctx->err = err; return nullptr; }
    HoTables* T = new HoTables();
    T->G = G.n;
    T->n = R.n;
    T->Q = R.Q;
    T->ntri = R.n * (R.n + 1) / 2;
    std::vector<float> dh(R.dphi.size()), dl(R.dphi.size()), ph(R.phi.size()), pl(R.phi.size());
    for (size_t k = 0; k < R.dphi.size(); ++k) {
        dh[k] = (float)R.dphi[k];
        dl[k] = (float)(R.dphi[k] - (double)dh[k]);
    }
    for (size_t k = 0; k < R.phi.size(); ++k) {
        ph[k] = (float)R.phi[k];
        pl[k] = (float)(R.phi[k] - (double)ph[k]);
    }
    std::vector<float> gdh(G.dphi.size()), gdl(G.dphi.size()), qwh(R.qw.size()), qwl(R.qw.size());
    for (size_t k = 0; k < G.dphi.size(); ++k) {
        gdh[k] = (float)G.dphi[k];
        gdl[k] = (float)(G.dphi[k] - (double)gdh[k]);
    }
    for (size_t k = 0; k < R.qw.size(); ++k) {
        qwh[k] = (float)R.qw[k];
        qwl[k] = (float)(R.qw[k] - (double)qwh[k]);
    }
    std::vector<uint8_t> ti, tj;
    for (int i = 0; i < R.n; ++i)
        for (int j = i; j < R.n; ++j) {
            ti.push_back((uint8_t)i);
            tj.push_back((uint8_t)j);
        }
    cudaError_t e = up(&T->d_dh, dh);
    if (e == cudaSuccess) e = up(&T->d_dl, dl);
    if (e == cudaSuccess) e = up(&T->d_ph, ph);
    if (e == cudaSuccess) e = up(&T->d_pl, pl);
    if (e == cudaSuccess) e = up(&T->d_phi, R.phi);
    if (e == cudaSuccess) e = up(&T->d_gd, G.dphi);
    if (e == cudaSuccess) e = up(&T->d_gp, G.phi);
    if (e == cudaSuccess) e = up(&T->d_qw, R.qw);
    if (e == cudaSuccess) e = up(&T->d_gdh, gdh);
    if (e == cudaSuccess) e = up(&T->d_gdl, gdl);
    if (e == cudaSuccess) e = up(&T->d_qwh, qwh);
    if (e == cudaSuccess) e = up(&T->d_qwl, qwl);
    if (e == cudaSuccess) e = up(&T->d_ti, ti);
    if (e == cudaSuccess) e = up(&T->d_tj, tj);
    if (e != cudaSuccess) {
        cudaGetLastError();
        ctx->err = std::string("curved-element tables: ") + cudaGetErrorString(e);
        delete T;
        return nullptr;
    }
    T->dphi = R.dphi;
    T->phi = R.phi;
    g_ho_tabs[key] = T;
    return T;
}

// K = sum_g X_g grad(psi_g)^T at one point, then |det K| and B = K^-T (cofactors / det)
template <int GN>
__device__ __forceinline__ double ho_map(const double* X /* GN x 3 */, const double* gd /* GN x 3 */, double B[9]) {
    double K[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) K[k] = 0.0;
    for (int g = 0; g < GN; ++g)
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) K[3 * r + c] = fma(X[3 * g + r], gd[3 * g + c], K[3 * r + c]);
    const double c00 = K[4] * K[8] - K[5] * K[7], c01 = K[5] * K[6] - K[3] * K[8], c02 = K[3] * K[7] - K[4] * K[6];
    const double det = K[0] * c00 + K[1] * c01 + K[2] * c02;
    const double cof[9] = {c00, c01, c02,
                           K[2] * K[7] - K[1] * K[8], K[0] * K[8] - K[2] * K[6], K[1] * K[6] - K[0] * K[7],
                           K[1] * K[5] - K[2] * K[4], K[2] * K[3] - K[0] * K[5], K[0] * K[4] - K[1] * K[3]};
#pragma unroll
    for (int k = 0; k < 9; ++k) B[k] = cof[k] / det;
    return det;
}

__device__ __forceinline__ df ldf(const float* h, const float* l, int k) { return df{h[k], l[k]}; }
// s + e += a b: the exact product of the high parts (FMA) split into its rounded value, added to s by
// TwoSum, and its error; the cross terms a.hi b.lo + a.lo b.hi and the TwoSum error go to e
__device__ __forceinline__ void ho_dot_term(df a, df b, float& s, float& e) {
    const float p = f_mul(a.hi, b.hi);
    e = f_fma(a.hi, b.lo, e);
    e = f_fma(a.lo, b.hi, e);
    e = f_add(e, f_fma(a.hi, b.hi, -p));
    const df t = two_sum(s, p);
    s = t.hi;
    e = f_add(e, t.lo);
}
__device__ __forceinline__ df dfun(float2 v) { return df{v.x, v.y}; }
__device__ __forceinline__ float2 dfpack(df v) { return make_float2(v.hi, v.lo); }

// LPG lanes per element (32: one element per warp; 8: four elements per warp, for at most 8 points)
template <int MODE, int N, int GN, int LPG = 32>
__global__ void __launch_bounds__(128) ho_element_kernel(int64_t nt, const double* __restrict__ xyz, const int32_t* __restrict__ tets,
                                                         const double* __restrict__ ho, int Q, const float* __restrict__ Dhg,
                                                         const float* __restrict__ Dlg, const float* __restrict__ Phg,
                                                         const float* __restrict__ Plg, const float* __restrict__ gdh,
                                                         const float* __restrict__ gdl, const float* __restrict__ qwh,
                                                         const float* __restrict__ qwl, const uint8_t* __restrict__ tig,
                                                         const uint8_t* __restrict__ tjg, const double* __restrict__ d_kappa,
                                                         double kappa, double mass, const double* __restrict__ kscale,
                                                         void* __restrict__ kbuf, int* __restrict__ status) {
    constexpr int NTRI = N * (N + 1) / 2;
    constexpr int EPW = 32 / LPG;                  // elements per warp
    constexpr int QM = LPG == 32 ? HoLimits<N, GN>::QMAX : LPG;
    constexpr int PER = (NTRI + LPG - 1) / LPG;    // entries per lane
    __shared__ float Dh[QM * N * 3], Dl[QM * N * 3], Ph[QM * N], Pl[QM * N];
    __shared__ uint8_t ti[NTRI], tj[NTRI];
    __shared__ float2 Gs[4][EPW][QM * 7];          // per element: G_q (00, 11, 22, 01, 02, 12) and m_q
    __shared__ float2 Ws[4][EPW][3 * N];           // per element: W_q = G_q dphi_j
    __shared__ float2 Xs[4][EPW][3 * GN];          // per element: its geometric nodes (double-float)
    for (int k = threadIdx.x; k < Q * N * 3; k += blockDim.x) { Dh[k] = Dhg[k]; Dl[k] = Dlg[k]; }
    for (int k = threadIdx.x; k < Q * N; k += blockDim.x) { Ph[k] = Phg[k]; Pl[k] = Plg[k]; }
    for (int k = threadIdx.x; k < NTRI; k += blockDim.x) { ti[k] = tig[k]; tj[k] = tjg[k]; }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int grp = lane / LPG, gl = lane % LPG;
    float2* XsG = Xs[warp][grp];
    float2* GsG = Gs[warp][grp];
    float2* WsG = Ws[warp][grp];
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    const df ksd = d2df(kscale ? *kscale : 1.0), massd = d2df(mass);
    for (int64_t e0 = ((int64_t)blockIdx.x * (blockDim.x >> 5) + warp) * EPW; e0 < nt; e0 += nw * EPW) {
        const int64_t e = e0 + grp;
        const bool live = e < nt;                  // the warp's loops stay uniform; a dead slot writes nothing
        // the element's nodes: tetrahedra 4 vertices and 6 edge nodes, hexahedra 8 vertices
        for (int k = gl; k < 3 * GN && live; k += LPG) {
            if (GN == 8) XsG[k] = dfpack(d2df(xyz[3 * (int64_t)tets[8 * e + k / 3] + k % 3]));
            else if (k < 12) XsG[k] = dfpack(d2df(xyz[3 * (int64_t)tets[4 * e + k / 3] + k % 3]));
            else XsG[k] = dfpack(d2df(ho[18 * e + (k - 12)]));
        }
        __syncwarp();
        const df kap = live ? df_mul(d2df(d_kappa ? d_kappa[e] : kappa), ksd) : df{0.0f, 0.0f};
        // geometry: one quadrature point per lane; double-float on the FP32 pipes (binary32 for FP32
        // matrices): K = sum_g X_g grad(psi_g)^T, cofactors, det, B = cof / det, G = w J kappa B^T B
        for (int q = gl; q < Q; q += LPG) {
            const float* gh = gdh + (size_t)q * 3 * GN;
            const float* gl = gdl + (size_t)q * 3 * GN;
            float2 g[7];
            if (MODE == kHoDF64) {
                // (the map's entries keep double-float multiply-adds: sum_g X_g grad(psi_g) cancels heavily,
                // since the gradients sum to zero, and a compensated dot product with one binary32 error
                // term missed the 1e-12 parity on curved P2 elements)
                df K[9];
#pragma unroll
                for (int k = 0; k < 9; ++k) K[k] = df{0.0f, 0.0f};
                for (int gg = 0; gg < GN; ++gg) {
                    const df d0 = df{__ldg(gh + 3 * gg), __ldg(gl + 3 * gg)};
                    const df d1 = df{__ldg(gh + 3 * gg + 1), __ldg(gl + 3 * gg + 1)};
                    const df d2 = df{__ldg(gh + 3 * gg + 2), __ldg(gl + 3 * gg + 2)};
#pragma unroll
                    for (int r = 0; r < 3; ++r) {
                        const df x = live ? dfun(XsG[3 * gg + r]) : df{(float)(gg == r + 1), 0.0f};
                        K[3 * r] = df_add(K[3 * r], df_mul(x, d0));
                        K[3 * r + 1] = df_add(K[3 * r + 1], df_mul(x, d1));
                        K[3 * r + 2] = df_add(K[3 * r + 2], df_mul(x, d2));
                    }
                }
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
                if (live && (!(J.hi > 0.0f) || !isfinite(J.hi))) atomicOr(status, kStatusBadElement);
                const df inv = df_recip(det);
                df B[9];
#pragma unroll
                for (int k = 0; k < 9; ++k) B[k] = df_mul(C[k], inv);
                const df wJ = df_mul(df{qwh[q], qwl[q]}, J), sc = df_mul(wJ, kap);
                const int pa[6] = {0, 1, 2, 0, 0, 1}, pb[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
                for (int k = 0; k < 6; ++k) {
                    df t = df_mul(B[pa[k]], B[pb[k]]);
                    t = df_add(t, df_mul(B[3 + pa[k]], B[3 + pb[k]]));
                    t = df_add(t, df_mul(B[6 + pa[k]], B[6 + pb[k]]));
                    g[k] = dfpack(df_mul(sc, t));
                }
                g[6] = dfpack(df_mul(wJ, massd));
            } else {
                float K[9];
#pragma unroll
                for (int k = 0; k < 9; ++k) K[k] = 0.0f;
                for (int gg = 0; gg < GN; ++gg)
#pragma unroll
                    for (int r = 0; r < 3; ++r) {
                        const float x = live ? XsG[3 * gg + r].x + XsG[3 * gg + r].y : (float)(gg == r + 1);
#pragma unroll
                        for (int c = 0; c < 3; ++c) K[3 * r + c] = fmaf(x, __ldg(gh + 3 * gg + c), K[3 * r + c]);
                    }
                const float C[9] = {K[4] * K[8] - K[5] * K[7], K[5] * K[6] - K[3] * K[8], K[3] * K[7] - K[4] * K[6],
                                    K[2] * K[7] - K[1] * K[8], K[0] * K[8] - K[2] * K[6], K[1] * K[6] - K[0] * K[7],
                                    K[1] * K[5] - K[2] * K[4], K[2] * K[3] - K[0] * K[5], K[0] * K[4] - K[1] * K[3]};
                const float det = K[0] * C[0] + K[1] * C[1] + K[2] * C[2];
                const float J = fabsf(det);
                if (live && (!(J > 0.0f) || !isfinite(J))) atomicOr(status, kStatusBadElement);
                float B[9];
#pragma unroll
                for (int k = 0; k < 9; ++k) B[k] = C[k] / det;
                const float wJ = qwh[q] * J, sc = wJ * (kap.hi + kap.lo);
                const int pa[6] = {0, 1, 2, 0, 0, 1}, pb[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
                for (int k = 0; k < 6; ++k)
                    g[k] = make_float2(sc * (B[pa[k]] * B[pb[k]] + B[3 + pa[k]] * B[3 + pb[k]] + B[6 + pa[k]] * B[6 + pb[k]]), 0.0f);
                g[6] = make_float2(wJ * (massd.hi + massd.lo), 0.0f);
            }
#pragma unroll
            for (int k = 0; k < 7; ++k) GsG[q * 7 + k] = g[k];
        }
        __syncwarp();
        // double-float entries as a compensated dot product over the points: the high parts of the exact
        // products through TwoSum, their errors, the cross terms and the low parts in a binary32
        // accumulator (the arithmetic of the affine kernel's coef_entry_df); binary32: plain sums
        float acs[PER], ace[PER];
#pragma unroll
        for (int u = 0; u < PER; ++u) { acs[u] = 0.0f; ace[u] = 0.0f; }
        for (int q = 0; q < Q; ++q) {
            const float2* G = &GsG[q * 7];
            for (int jl = gl; jl < N; jl += LPG) {
                const int b0 = (q * N + jl) * 3;
                if (MODE == kHoDF64) {
                    const df d0 = ldf(Dh, Dl, b0), d1 = ldf(Dh, Dl, b0 + 1), d2 = ldf(Dh, Dl, b0 + 2);
                    const df g00 = dfun(G[0]), g11 = dfun(G[1]), g22 = dfun(G[2]), g01 = dfun(G[3]), g02 = dfun(G[4]), g12 = dfun(G[5]);
                    const df w0 = df_add(df_add(df_mul(g00, d0), df_mul(g01, d1)), df_mul(g02, d2));
                    const df w1 = df_add(df_add(df_mul(g01, d0), df_mul(g11, d1)), df_mul(g12, d2));
                    const df w2 = df_add(df_add(df_mul(g02, d0), df_mul(g12, d1)), df_mul(g22, d2));
                    WsG[jl] = dfpack(w0);
                    WsG[N + jl] = dfpack(w1);
                    WsG[2 * N + jl] = dfpack(w2);
                } else {
                    const float d0 = Dh[b0], d1 = Dh[b0 + 1], d2 = Dh[b0 + 2];
                    WsG[jl] = make_float2(fmaf(G[0].x, d0, fmaf(G[3].x, d1, G[4].x * d2)), 0.0f);
                    WsG[N + jl] = make_float2(fmaf(G[3].x, d0, fmaf(G[1].x, d1, G[5].x * d2)), 0.0f);
                    WsG[2 * N + jl] = make_float2(fmaf(G[4].x, d0, fmaf(G[5].x, d1, G[2].x * d2)), 0.0f);
                }
            }
            __syncwarp();
#pragma unroll
            for (int u = 0; u < PER; ++u) {
                const int t = gl + LPG * u;
                if (t >= NTRI) break;
                const int i = ti[t], j = tj[t];
                const int bi = (q * N + i) * 3;
                if (MODE == kHoDF64) {
                    ho_dot_term(ldf(Dh, Dl, bi), dfun(WsG[j]), acs[u], ace[u]);
                    ho_dot_term(ldf(Dh, Dl, bi + 1), dfun(WsG[N + j]), acs[u], ace[u]);
                    ho_dot_term(ldf(Dh, Dl, bi + 2), dfun(WsG[2 * N + j]), acs[u], ace[u]);
                    ho_dot_term(dfun(G[6]), df_mul(ldf(Ph, Pl, q * N + i), ldf(Ph, Pl, q * N + j)), acs[u], ace[u]);
                } else {
                    float v = Dh[bi] * WsG[j].x;
                    v = fmaf(Dh[bi + 1], WsG[N + j].x, v);
                    v = fmaf(Dh[bi + 2], WsG[2 * N + j].x, v);
                    v = fmaf(G[6].x, Ph[q * N + i] * Ph[q * N + j], v);
                    acs[u] += v;
                }
            }
            __syncwarp();
        }
#pragma unroll
        for (int u = 0; u < PER && live; ++u) {
            const int t = gl + LPG * u;
            if (t >= NTRI) break;
            if (MODE == kHoDF64) reinterpret_cast<float2*>(kbuf)[e * NTRI + t] = dfpack(two_sum(acs[u], ace[u]));
            else reinterpret_cast<float*>(kbuf)[e * NTRI + t] = acs[u];
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Binary32 element matrices on the tensor cores (tcgen05, kind::tf32).
//
// With the per-point coefficients g_q = (G00, G11, G22, G01, G02, G12, m, 0) of an
// element (G_q = w_q |det K_q| kappa B_q^T B_q, m = w_q |det K_q| mass) the
// upper triangle of its matrix is one row of a dense product:
//     K_e(t) = sum_q sum_r g_{q,r}(e) T_{q,r}(t),   t = (i, j), i <= j,
//     T_{q,0..2}(t) = d_a,i d_a,j,  T_{q,3}(t) = d0_i d1_j + d1_i d0_j,  (02, 12 likewise),
//     T_{q,6}(t) = phi_i phi_j,  T_{q,7} = 0  (d: reference gradients at point q),
// i.e. for a tile of 128 elements D (128 x NTRI) = A (128 x 8Q) * B^T (8Q x NTRI),
// with K = 8 per quadrature point: one tf32 MMA k-step per point. B is the same for
// every element (built once on the host, split into tf32 high and low parts in the
// shared-memory core-matrix layout of each chunk of QC points) and is staged per
// chunk with a bulk asynchronous copy (cp.async.bulk, completion counted on an
// mbarrier); A is formed by the CTA's 128 threads (one element each: the map, its
// cofactors, determinant and B = K^-T at the chunk's points, in binary32) into one
// of two stages while the tensor cores run the previous chunk's 3xTF32 products
// (hi*hi + hi*lo + lo*hi into the FP32 accumulator in tensor memory). The
// epilogue reads each element's row back with tcgen05.ld and stores it into the
// two-phase element buffer. NACC accumulators of NP columns cover NTRI (two for
// Q2 hexahedra, 378 entries). Every mbarrier wait is bounded: a timeout sets a
// status bit and a shared flag, every thread leaves at the next barrier, and the
// tensor memory is freed.
// ---------------------------------------------------------------------------
constexpr int kHoTcThreads = 128;
constexpr int kHoTcQC = 1;                       // quadrature points per chunk (K = 8: one MMA k-step)
constexpr int kHoTcBStages = 4;                  // table stages; the copy for chunk c + 2 starts at chunk c
constexpr int kStatusHoTcTimeout = 512;

template <int N, int GN>
struct HoTcDims {
    static constexpr int NTRI = N * (N + 1) / 2;
    static constexpr int NACC = NTRI > 256 ? 2 : 1;
    static constexpr int NP = ((NTRI + NACC - 1) / NACC + 15) / 16 * 16;     // MMA N per accumulator
    static constexpr int ACC_STRIDE = NACC == 2 ? 256 : NP;                   // tensor-memory columns between accumulators
    static constexpr int NCOLS_USED = (NACC - 1) * ACC_STRIDE + NP;
    static constexpr int NCOLS = NCOLS_USED <= 32 ? 32 : NCOLS_USED <= 64 ? 64 : NCOLS_USED <= 128 ? 128
                                 : NCOLS_USED <= 256 ? 256 : 512;            // tensor-memory allocation
    static constexpr int KC = 8 * kHoTcQC;
    static constexpr int ABYTES = kTcTile * KC * 4;                           // one part (hi or lo) of A
    static constexpr int BPART = NP * KC * 4;                                 // one part of one accumulator's B
    static constexpr int BSTAGE = NACC * 2 * BPART;
    static constexpr int QM = HoLimits<N, GN>::QMAX;
    static constexpr int SMEM_USED = 1024 + kHoTcBStages * BSTAGE + 2 * 2 * ABYTES + QM * GN * 3 * 4 + QM * 4 + 16 + 256;
    // at most 512 / NCOLS blocks per SM, so that their tensor-memory allocations always fit
    static constexpr int MAXCTA = 512 / NCOLS;
    static constexpr int SMEM_MIN = 228 * 1024 / (MAXCTA + 1) + 1024;
    static constexpr int SMEM = SMEM_USED > SMEM_MIN ? SMEM_USED : SMEM_MIN;
};

struct HoTcShared {
    uint64_t bfull[kHoTcBStages], mma[kHoTcBStages];
    uint32_t tmem;
    int bad;
};

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, void* mbar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(mbar))
                 : "memory");
}

template <int N, int GN>
__global__ void __launch_bounds__(kHoTcThreads) ho_element_tc_kernel(int64_t nt, const double* __restrict__ xyz,
                                                                    const int32_t* __restrict__ tets, const double* __restrict__ ho,
                                                                    int Q, const float* __restrict__ Bg, const float* __restrict__ gdh,
                                                                    const float* __restrict__ qwh, const double* __restrict__ d_kappa,
                                                                    double kappa, double mass, const double* __restrict__ kscale,
                                                                    float* __restrict__ kbuf, int* __restrict__ status, int budget) {
    typedef HoTcDims<N, GN> D;
    constexpr int NB = kHoTcBStages;
    extern __shared__ __align__(1024) unsigned char ho_smem[];
    unsigned char* base = (unsigned char*)(((uintptr_t)ho_smem + 1023) & ~(uintptr_t)1023);
    unsigned char* Bs = base;                                   // NB stages of B
    unsigned char* As = Bs + NB * D::BSTAGE;                    // 2 stages of (A hi, A lo)
    float* gds = reinterpret_cast<float*>(As + 4 * D::ABYTES);  // Q GN 3 geometric reference gradients
    float* qws = gds + D::QM * GN * 3;
    HoTcShared* sh = reinterpret_cast<HoTcShared*>(((uintptr_t)(qws + D::QM) + 15) & ~(uintptr_t)15);   // mbarriers: 8-byte aligned
    const int t = threadIdx.x;
    for (int k = t; k < Q * GN * 3; k += kHoTcThreads) gds[k] = gdh[k];
    for (int k = t; k < Q; k += kHoTcThreads) qws[k] = qwh[k];
    const int64_t ntiles = (nt + kTcTile - 1) / kTcTile;
    const int nchunks = (Q + kHoTcQC - 1) / kHoTcQC;
    const int64_t mytiles = blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const uint32_t total = (uint32_t)(mytiles * nchunks);       // chunks this block runs
    // table chunk of chunk c (every tile runs the same sequence of chunks)
    auto copy_chunk = [&](uint32_t c) {
        bulk_g2s(Bs + (c % NB) * D::BSTAGE, Bg + (size_t)(c % (uint32_t)nchunks) * (D::BSTAGE / 4), D::BSTAGE, &sh->bfull[c % NB]);
    };
    if (t == 0) {
        for (int s = 0; s < NB; ++s) {
            mbar_init(&sh->bfull[s], 1);
            mbar_init(&sh->mma[s], 1);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        sh->bad = 0;
        for (uint32_t c = 0; c < 2 && c < total; ++c) copy_chunk(c);
    }
    if ((t >> 5) == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sh->tmem)),
                     "r"(D::NCOLS) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = sh->tmem;
    const uint32_t lane_addr = tmem + ((uint32_t)((t >> 5) * 32) << 16);
    const float ksc = kscale ? (float)*kscale : 1.0f;
    constexpr uint32_t idesc = make_idesc_tf32(D::NP);
    constexpr uint32_t lbo = 128, sbo = (D::KC / 4) * 128;
    uint32_t c = 0;                                             // chunk counter over all tiles
    bool quit = false;
    for (int64_t tile = blockIdx.x; tile < ntiles && !quit; tile += gridDim.x) {
        const int64_t e = tile * kTcTile + t;
        const bool live = e < nt;
        float X[3 * GN];
        float kap = 0.0f;
        if (live) {
#pragma unroll
            for (int k = 0; k < 3 * GN; ++k) {
                if (GN == 8) X[k] = (float)xyz[3 * (int64_t)tets[8 * e + k / 3] + k % 3];
                else if (k < 12) X[k] = (float)xyz[3 * (int64_t)tets[4 * e + k / 3] + k % 3];
                else X[k] = (float)ho[18 * e + (k - 12)];
            }
            kap = (float)(d_kappa ? d_kappa[e] : kappa) * ksc;
        }
        for (int ch = 0; ch < nchunks; ++ch, ++c) {
            unsigned char* Ah = As + 2 * (c & 1u) * D::ABYTES;
            unsigned char* Al = Ah + D::ABYTES;
            // chunk c - 2 done: its A stage and its table stage are free
            if (c >= 2 && !mbar_wait(&sh->mma[(c - 2) % NB], ((c - 2) / NB) & 1u, budget)) sh->bad = 1;
            if (t == 0 && c + 2 < total && !sh->bad) copy_chunk(c + 2);
            // this element's coefficients at the chunk's points (zero past the last point or element)
#pragma unroll
            for (int ql = 0; ql < kHoTcQC; ++ql) {
                const int q = ch * kHoTcQC + ql;
                float g[8];
#pragma unroll
                for (int r = 0; r < 8; ++r) g[r] = 0.0f;
                if (live && q < Q) {
                    const float* gq = gds + q * GN * 3;
                    float K[9];
#pragma unroll
                    for (int k = 0; k < 9; ++k) K[k] = 0.0f;
#pragma unroll
                    for (int gg = 0; gg < GN; ++gg)
#pragma unroll
                        for (int r = 0; r < 3; ++r)
#pragma unroll
                            for (int cc = 0; cc < 3; ++cc) K[3 * r + cc] = fmaf(X[3 * gg + r], gq[3 * gg + cc], K[3 * r + cc]);
                    const float C[9] = {K[4] * K[8] - K[5] * K[7], K[5] * K[6] - K[3] * K[8], K[3] * K[7] - K[4] * K[6],
                                        K[2] * K[7] - K[1] * K[8], K[0] * K[8] - K[2] * K[6], K[1] * K[6] - K[0] * K[7],
                                        K[1] * K[5] - K[2] * K[4], K[2] * K[3] - K[0] * K[5], K[0] * K[4] - K[1] * K[3]};
                    const float det = K[0] * C[0] + K[1] * C[1] + K[2] * C[2];
                    const float J = fabsf(det);
                    if (!(J > 0.0f) || !isfinite(J)) atomicOr(status, kStatusBadElement);
                    const float id = 1.0f / det;
                    float B[9];
#pragma unroll
                    for (int k = 0; k < 9; ++k) B[k] = C[k] * id;
                    const float wJ = qws[q] * J, sc = wJ * kap;
                    const int pa[6] = {0, 1, 2, 0, 0, 1}, pb[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
                    for (int k = 0; k < 6; ++k)
                        g[k] = sc * (B[pa[k]] * B[pb[k]] + B[3 + pa[k]] * B[3 + pb[k]] + B[6 + pa[k]] * B[6 + pb[k]]);
                    g[6] = wJ * (float)mass;
                }
#pragma unroll
                for (int r = 0; r < 8; ++r) {
                    const float h = tf32_hi(g[r]);
                    *reinterpret_cast<float*>(Ah + core_off(t, 8 * ql + r, D::KC)) = h;
                    *reinterpret_cast<float*>(Al + core_off(t, 8 * ql + r, D::KC)) = g[r] - h;
                }
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncthreads();
            if (sh->bad) { quit = true; break; }
            if (t == 0) {
                if (!mbar_wait(&sh->bfull[c % NB], (c / NB) & 1u, budget)) {
                    sh->bad = 1;
                    atomicOr(status, kStatusHoTcTimeout);
                } else {
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const unsigned char* Bst = Bs + (c % NB) * D::BSTAGE;
#pragma unroll
                    for (int a = 0; a < D::NACC; ++a) {
                        const unsigned char* Bh = Bst + (2 * a) * D::BPART;
                        const unsigned char* Bl = Bh + D::BPART;
#pragma unroll
                        for (int ks = 0; ks < kHoTcQC; ++ks) {
                            const uint64_t ah = make_sdesc(smem_u32(Ah) + ks * 256, lbo, sbo);
                            const uint64_t al = make_sdesc(smem_u32(Al) + ks * 256, lbo, sbo);
                            const uint64_t bh = make_sdesc(smem_u32(Bh) + ks * 256, lbo, sbo);
                            const uint64_t bl = make_sdesc(smem_u32(Bl) + ks * 256, lbo, sbo);
                            const uint32_t dst = tmem + (uint32_t)(a * D::ACC_STRIDE);
                            tc_mma(dst, ah, bh, idesc, (ch > 0 || ks > 0) ? 1u : 0u);
                            tc_mma(dst, ah, bl, idesc, 1u);
                            tc_mma(dst, al, bh, idesc, 1u);
                        }
                    }
                    tc_commit(&sh->mma[c % NB]);
                }
            }
        }
        if (quit) break;
        // epilogue: the last chunk's commit completes the accumulator
        const uint32_t cl = c - 1;
        if (!mbar_wait(&sh->mma[cl % NB], (cl / NB) & 1u, budget)) {
            sh->bad = 1;
            atomicOr(status, kStatusHoTcTimeout);
        }
        __syncthreads();
        if (sh->bad) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll 1
        for (int a = 0; a < D::NACC; ++a)
            for (int col = 0; col < D::NP; col += 16) {
                uint32_t r[16];
                tmem_ld16_nowait(lane_addr + (uint32_t)(a * D::ACC_STRIDE + col), r);
                tmem_wait_ld();
                if (live) {
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        const int tt = a * D::NP + col + i;   // accumulator a holds entries a NP .. a NP + NP - 1
                        if (tt < D::NTRI) kbuf[e * D::NTRI + tt] = __uint_as_float(r[i]);
                    }
                }
            }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
    }
    // after a failure, wait (bounded) for the products and copies this block issued before the tensor
    // memory and the shared memory go away
    if (t == 0 && sh->bad) {
        for (uint32_t k = (c > 2 ? c - 2 : 0); k < c; ++k) mbar_wait(&sh->mma[k % NB], (k / NB) & 1u, budget);
        for (uint32_t k = (c > 2 ? c - 2 : 0); k < c + 2 && k < total; ++k) mbar_wait(&sh->bfull[k % NB], (k / NB) & 1u, budget);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if ((t >> 5) == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(D::NCOLS) : "memory");
}

// load vector on curved elements: thread per element, per point the map, J and the physical point
template <int N, int GN>
__global__ void ho_rhs_kernel(int64_t nt, const double* __restrict__ xyz, const int32_t* __restrict__ tets,
                              const double* __restrict__ ho, int Q, const double* __restrict__ qw, const double* __restrict__ phi,
                              const double* __restrict__ gd, const double* __restrict__ gp, int fkind, double f0,
                              double* __restrict__ work, int* __restrict__ status) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nt; e += (int64_t)gridDim.x * blockDim.x) {
        double X[3 * GN];
        if (GN == 8) {
#pragma unroll
            for (int v = 0; v < 8; ++v)
#pragma unroll
                for (int r = 0; r < 3; ++r) X[3 * v + r] = xyz[3 * (int64_t)tets[8 * e + v] + r];
        } else {
#pragma unroll
            for (int v = 0; v < 4; ++v)
#pragma unroll
                for (int r = 0; r < 3; ++r) X[3 * v + r] = xyz[3 * (int64_t)tets[4 * e + v] + r];
#pragma unroll
            for (int k = 0; k < 3 * GN - 12; ++k) X[12 + k] = ho[18 * e + k];
        }
        double F[N];
#pragma unroll
        for (int i = 0; i < N; ++i) F[i] = 0.0;
        for (int q = 0; q < Q; ++q) {
            double B[9];
            const double J = fabs(ho_map<GN>(X, gd + (size_t)q * 3 * GN, B));
            if (!(J > 0.0) || !isfinite(J)) atomicOr(status, kStatusBadElement);
            double f = f0;
            if (fkind == FGPU_RHS_SINE) {
                double p[3] = {0.0, 0.0, 0.0};
                for (int g = 0; g < GN; ++g)
#pragma unroll
                    for (int r = 0; r < 3; ++r) p[r] = fma(X[3 * g + r], gp[q * GN + g], p[r]);
                const double pi = 3.141592653589793;
                f = 3.0 * pi * pi * sin(pi * p[0]) * sin(pi * p[1]) * sin(pi * p[2]);
            }
            const double s = qw[q] * J * f;
#pragma unroll
            for (int i = 0; i < N; ++i) F[i] = fma(s, phi[q * N + i], F[i]);
        }
#pragma unroll
        for (int i = 0; i < N; ++i) work[e * N + i] = F[i];
    }
}


// ---- host side of the tensor-core element kernel ----
// B operand of HoTcDims<N, GN> from the reference tables: per chunk of kHoTcQC points, per accumulator,
// the tf32 high then low parts of T_{q,r}(t) in the shared-memory core-matrix layout (row = entry,
// K index = 8 (point in chunk) + r).
template <int N, int GN>
static int ho_tc_tables(fgpu_ctx* ctx, HoTables* T) {
    typedef HoTcDims<N, GN> D;
    std::lock_guard<std::mutex> lock(g_ho_mutex);
    if (T->d_tcB) return FGPU_OK;
    const int Q = T->Q, nch = (Q + kHoTcQC - 1) / kHoTcQC;
    std::vector<float> B((size_t)nch * (D::BSTAGE / 4), 0.0f);
    std::vector<int> ti, tj;
    for (int i = 0; i < N; ++i)
        for (int j = i; j < N; ++j) {
            ti.push_back(i);
            tj.push_back(j);
        }
    auto tf32_hi_host = [](float x) {
        uint32_t u;
        std::memcpy(&u, &x, 4);
        u = (u + 0x1000u) & 0xFFFFE000u;
        float h;
        std::memcpy(&h, &u, 4);
        return h;
    };
    auto off = [](int row, int k) { return (size_t)((row >> 3) * (D::KC / 4) * 128 + (k >> 2) * 128 + (row & 7) * 16 + (k & 3) * 4) / 4; };
    for (int ch = 0; ch < nch; ++ch)
        for (int a = 0; a < D::NACC; ++a)
            for (int n = 0; n < D::NP; ++n) {
                const int t = a * D::NP + n;
                for (int ql = 0; ql < kHoTcQC; ++ql) {
                    const int q = ch * kHoTcQC + ql;
                    for (int r = 0; r < 8; ++r) {
                        double v = 0.0;
                        if (t < D::NTRI && q < Q && r < 7) {
                            const int i = ti[t], j = tj[t];
                            const double* di = &T->dphi[((size_t)q * N + i) * 3];
                            const double* dj = &T->dphi[((size_t)q * N + j) * 3];
                            switch (r) {
                                case 0: v = di[0] * dj[0]; break;
                                case 1: v = di[1] * dj[1]; break;
                                case 2: v = di[2] * dj[2]; break;
                                case 3: v = di[0] * dj[1] + di[1] * dj[0]; break;
                                case 4: v = di[0] * dj[2] + di[2] * dj[0]; break;
                                case 5: v = di[1] * dj[2] + di[2] * dj[1]; break;
                                default: v = T->phi[(size_t)q * N + i] * T->phi[(size_t)q * N + j]; break;
                            }
                        }
                        const float h = tf32_hi_host((float)v);
                        const size_t base = (size_t)ch * (D::BSTAGE / 4) + (size_t)(2 * a) * (D::BPART / 4);
                        B[base + off(n, 8 * ql + r)] = h;
                        B[base + D::BPART / 4 + off(n, 8 * ql + r)] = (float)(v - (double)h);
                    }
                }
            }
    cudaError_t e = up(&T->d_tcB, B);
    if (e != cudaSuccess) { cudaGetLastError(); ctx->err = "tensor-core element tables: upload failed"; return FGPU_ERR_CUDA; }
    return FGPU_OK;
}

constexpr int kHoTcWaitBudget = 1 << 22;

template <int N, int GN>
static int launch_ho_tc(fgpu_ctx* ctx, fgpu_matrix* A, HoTables* T, const double* d_kappa, const fgpu_form_desc* f) {
    typedef HoTcDims<N, GN> D;
    const fgpu_mesh* M = A->space->mesh;
    if (T->Q > D::QM) { ctx->err = "tensor-core element kernel: too many quadrature points"; return FGPU_ERR_INVALID; }
    int rc = ho_tc_tables<N, GN>(ctx, T);
    if (rc) return rc;
    auto kern = ho_element_tc_kernel<N, GN>;
    FGPU_CUDA_CHECK(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, D::SMEM));
    // resident blocks per SM from the registers and the shared memory (the occupancy calculator gives 1
    // for kernels that allocate tensor memory; the blocks here never wait for one another, so more blocks
    // than fit only queue), and at most 512 / NCOLS so that their tensor-memory allocations fit
    cudaFuncAttributes fa{};
    FGPU_CUDA_CHECK(ctx, cudaFuncGetAttributes(&fa, kern));
    int sms = 0, smem_sm = 0, regs_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, ctx->device);
    cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, ctx->device);
    const int by_smem = smem_sm / (D::SMEM + 1024);
    const int by_regs = regs_sm / (((fa.numRegs + 7) & ~7) * kHoTcThreads);
    const int per_sm = std::max(1, std::min(std::min(by_smem, by_regs), D::MAXCTA));
    const int64_t ntiles = (M->nt + kTcTile - 1) / kTcTile;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(ntiles, (int64_t)per_sm * sms));
    kern<<<blocks, kHoTcThreads, D::SMEM, ctx->stream>>>(M->nt, M->d_xyz, M->d_tets, M->d_ho, T->Q, T->d_tcB, T->d_gdh, T->d_qwh,
                                                         d_kappa, f->kappa, f->mass, f->kappa_scale, (float*)A->d_kbuf,
                                                         ctx->d_status, kHoTcWaitBudget);
    return FGPU_OK;
}

int ho_qdeg_ok(fgpu_ctx* ctx, int order, int qdeg) {
    const int lim = order == 1 ? 5 : order == 2 ? 7 : 8;
    if (qdeg > lim) {
        ctx->err = "curved elements: quadrature degree above " + std::to_string(lim) + " for this order";
        return FGPU_ERR_INVALID;
    }
    return FGPU_OK;
}

int hex_qdeg_ok(fgpu_ctx* ctx, int order, int qdeg) {
    const int lim = order == 1 ? 6 : 4;   // 4^3 / 3^3 Gauss points
    if (qdeg > lim) {
        ctx->err = "hexahedra: quadrature degree above " + std::to_string(lim) + " for this order";
        return FGPU_ERR_INVALID;
    }
    return FGPU_OK;
}

}  // namespace

// Q1/Q2 hexahedra: the curved-element kernels with the trilinear (Q1) map and tensor Gauss rules
int launch_assemble_hex(fgpu_ctx* ctx, fgpu_matrix* A, const fgpu_form_desc* f, const double* d_kappa, int accumulate) {
    fgpu_space* V = A->space;
    const fgpu_mesh* M = V->mesh;
    if (f->kind != FGPU_FORM_LAPLACE_MASS || V->ncomp != 1 || f->range != FGPU_RANGE_ELEMENTS || f->mass_h != 0.0 ||
        f->dn_trial != 0.0 || f->dn_test != 0.0) {
        ctx->err = "hexahedra: scalar Laplace/mass forms over elements(mesh) only";
        return FGPU_ERR_INVALID;
    }
    const int qdeg = f->quad_degree > 0 ? f->quad_degree : 2 * V->order;
    int rc = hex_qdeg_ok(ctx, V->order, qdeg);
    if (rc) return rc;
    HoTables* T = get_ho_tables(ctx, V->order, qdeg, true);
    if (!T) return FGPU_ERR_INVALID;
    const bool f32 = A->precision == FGPU_F32;
    rc = ensure_two_phase(ctx, A, (size_t)M->nt * T->ntri * (f32 ? 4 : 8));
    if (rc) return rc;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((M->nt + 3) / 4, 152 * 32));
    PendingEvent ev;
    prof_begin(ctx, "assemble_elements_hex", ev);
#define HEX_LAUNCH(MODE, NN, LPG, NB)                                                                                         \
    ho_element_kernel<MODE, NN, 8, LPG><<<NB, 128, 0, ctx->stream>>>(M->nt, M->d_xyz, M->d_tets, nullptr, T->Q, T->d_dh,      \
                                                                    T->d_dl, T->d_ph, T->d_pl, T->d_gdh, T->d_gdl, T->d_qwh,   \
                                                                    T->d_qwl, T->d_ti, T->d_tj, d_kappa, f->kappa, f->mass,    \
                                                                    f->kappa_scale, A->d_kbuf, ctx->d_status)
    if (f32 && (ctx->tensor_cores & FGPU_TC_F32)) {
        rc = V->n == 8 ? launch_ho_tc<8, 8>(ctx, A, T, d_kappa, f) : launch_ho_tc<27, 8>(ctx, A, T, d_kappa, f);
        if (rc) return rc;
    } else if (V->n == 8 && T->Q <= 8) {
        // Q1 with the 2^3 rule: four elements per warp, one point and one dof per lane
        const int nb4 = (int)std::max<int64_t>(1, std::min<int64_t>((M->nt + 15) / 16, 152 * 32));
        if (f32) HEX_LAUNCH(kHoF32, 8, 8, nb4); else HEX_LAUNCH(kHoDF64, 8, 8, nb4);
    } else if (V->n == 8) {
        if (f32) HEX_LAUNCH(kHoF32, 8, 32, blocks); else HEX_LAUNCH(kHoDF64, 8, 32, blocks);
    } else {
        if (f32) HEX_LAUNCH(kHoF32, 27, 32, blocks); else HEX_LAUNCH(kHoDF64, 27, 32, blocks);
    }
#undef HEX_LAUNCH
    prof_end(ctx, ev);
    ctx->launches++;
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    rc = launch_gather_phase(ctx, A, accumulate);
    ctx->launches++;
    return rc;
}

int launch_rhs_hex(fgpu_ctx* ctx, const fgpu_space* V, const fgpu_rhs_desc* rhs, double* d_out, int accumulate) {
    const fgpu_mesh* M = V->mesh;
    if (V->ncomp != 1 || (rhs->kind != FGPU_RHS_SINE && rhs->kind != FGPU_RHS_CONST)) {
        ctx->err = "hexahedra: scalar sine or constant sources only";
        return FGPU_ERR_INVALID;
    }
    const int qdeg = rhs->quad_degree > 0 ? rhs->quad_degree : 2 * V->order;
    int rc = hex_qdeg_ok(ctx, V->order, qdeg);
    if (rc) return rc;
    HoTables* T = get_ho_tables(ctx, V->order, qdeg, true);
    if (!T) return FGPU_ERR_INVALID;
    double* work = nullptr;
    FGPU_CUDA_CHECK(ctx, cudaMalloc(&work, std::max<int64_t>(M->nt * V->n, 1) * sizeof(double)));
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((M->nt + 127) / 128, 152 * 32));
    PendingEvent ev;
    prof_begin(ctx, "rhs_element_hex", ev);
    if (V->n == 8)
        ho_rhs_kernel<8, 8><<<blocks, 128, 0, ctx->stream>>>(M->nt, M->d_xyz, M->d_tets, nullptr, T->Q, T->d_qw, T->d_phi, T->d_gd, T->d_gp, rhs->kind, rhs->c[0], work, ctx->d_status);
    else
        ho_rhs_kernel<27, 8><<<blocks, 128, 0, ctx->stream>>>(M->nt, M->d_xyz, M->d_tets, nullptr, T->Q, T->d_qw, T->d_phi, T->d_gd, T->d_gp, rhs->kind, rhs->c[0], work, ctx->d_status);
    prof_end(ctx, ev);
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) rc = launch_rhs_gather(ctx, V, work, d_out, accumulate);
    ctx->launches++;
    cudaStreamSynchronize(ctx->stream);
    cudaFree(work);
    if (e != cudaSuccess) { ctx->err = std::string("hexahedral load vector: ") + cudaGetErrorString(e); return FGPU_ERR_CUDA; }
    return rc;
}

int launch_assemble_ho(fgpu_ctx* ctx, fgpu_matrix* A, const fgpu_form_desc* f, const double* d_kappa, int accumulate) {
    fgpu_space* V = A->space;
    const fgpu_mesh* M = V->mesh;
    if (f->kind != FGPU_FORM_LAPLACE_MASS || V->ncomp != 1) {
        ctx->err = "curved elements: scalar Laplace/mass forms only";
        return FGPU_ERR_INVALID;
    }
    const int qdeg = f->quad_degree > 0 ? f->quad_degree : std::min(2 * V->order + 2, 8);
    int rc = ho_qdeg_ok(ctx, V->order, qdeg);
    if (rc) return rc;
    HoTables* T = get_ho_tables(ctx, V->order, qdeg);
    if (!T) return FGPU_ERR_INVALID;
    const bool f32 = A->precision == FGPU_F32;
    rc = ensure_two_phase(ctx, A, (size_t)M->nt * T->ntri * (f32 ? 4 : 8));
    if (rc) return rc;
    const int64_t warps = M->nt;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((warps + 3) / 4, 152 * 32));
    PendingEvent ev;
    prof_begin(ctx, "assemble_elements_ho", ev);
#define HO_LAUNCH(MODE, NN)                                                                                                   \
    ho_element_kernel<MODE, NN, 10><<<blocks, 128, 0, ctx->stream>>>(M->nt, M->d_xyz, M->d_tets, M->d_ho, T->Q, T->d_dh, T->d_dl,  \
                                                                T->d_ph, T->d_pl, T->d_gdh, T->d_gdl, T->d_qwh, T->d_qwl,      \
                                                                T->d_ti, T->d_tj, d_kappa,                                     \
                                                                f->kappa, f->mass, f->kappa_scale, A->d_kbuf, ctx->d_status)
    if (f32 && (ctx->tensor_cores & FGPU_TC_F32)) {
        rc = V->n == 4 ? launch_ho_tc<4, 10>(ctx, A, T, d_kappa, f)
             : V->n == 10 ? launch_ho_tc<10, 10>(ctx, A, T, d_kappa, f) : launch_ho_tc<20, 10>(ctx, A, T, d_kappa, f);
        if (rc) return rc;
    } else {
        switch (V->n) {
            case 4: if (f32) HO_LAUNCH(kHoF32, 4); else HO_LAUNCH(kHoDF64, 4); break;
            case 10: if (f32) HO_LAUNCH(kHoF32, 10); else HO_LAUNCH(kHoDF64, 10); break;
            default: if (f32) HO_LAUNCH(kHoF32, 20); else HO_LAUNCH(kHoDF64, 20); break;
        }
    }
#undef HO_LAUNCH
    prof_end(ctx, ev);
    ctx->launches++;
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    rc = launch_gather_phase(ctx, A, accumulate);
    ctx->launches++;
    return rc;
}

int launch_rhs_ho(fgpu_ctx* ctx, const fgpu_space* V, const fgpu_rhs_desc* rhs, double* d_out, int accumulate) {
    const fgpu_mesh* M = V->mesh;
    if (V->ncomp != 1 || (rhs->kind != FGPU_RHS_SINE && rhs->kind != FGPU_RHS_CONST)) {
        ctx->err = "curved elements: scalar sine or constant sources only";
        return FGPU_ERR_INVALID;
    }
    const int qdeg = rhs->quad_degree > 0 ? rhs->quad_degree : std::min(2 * V->order + 2, 8);
    int rc = ho_qdeg_ok(ctx, V->order, qdeg);
    if (rc) return rc;
    HoTables* T = get_ho_tables(ctx, V->order, qdeg);
    if (!T) return FGPU_ERR_INVALID;
    double* work = nullptr;
    FGPU_CUDA_CHECK(ctx, cudaMalloc(&work, std::max<int64_t>(M->nt * V->n, 1) * sizeof(double)));
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((M->nt + 127) / 128, 152 * 32));
    PendingEvent ev;
    prof_begin(ctx, "rhs_element_ho", ev);
    switch (V->n) {
        case 4: ho_rhs_kernel<4, 10><<<blocks, 128, 0, ctx->stream>>>(M->nt, M->d_xyz, M->d_tets, M->d_ho, T->Q, T->d_qw, T->d_phi, T->d_gd, T->d_gp, rhs->kind, rhs->c[0], work, ctx->d_status); break;
        case 10: ho_rhs_kernel<10, 10><<<blocks, 128, 0, ctx->stream>>>(M->nt, M->d_xyz, M->d_tets, M->d_ho, T->Q, T->d_qw, T->d_phi, T->d_gd, T->d_gp, rhs->kind, rhs->c[0], work, ctx->d_status); break;
        default: ho_rhs_kernel<20, 10><<<blocks, 128, 0, ctx->stream>>>(M->nt, M->d_xyz, M->d_tets, M->d_ho, T->Q, T->d_qw, T->d_phi, T->d_gd, T->d_gp, rhs->kind, rhs->c[0], work, ctx->d_status); break;
    }
    prof_end(ctx, ev);
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) rc = launch_rhs_gather(ctx, V, work, d_out, accumulate);
    ctx->launches++;
    cudaStreamSynchronize(ctx->stream);
    cudaFree(work);
    if (e != cudaSuccess) { ctx->err = std::string("curved load vector: ") + cudaGetErrorString(e); return FGPU_ERR_CUDA; }
    return rc;
}

}  // namespace fgpu

using namespace fgpu;

extern "C" int fgpu_mesh_set_ho_nodes(fgpu_mesh* M, const double* ho) {
    if (!M) return FGPU_ERR_INVALID;
    fgpu_ctx* ctx = M->ctx;
    if (ctx->capturing) { ctx->err = "mesh_set_ho_nodes: not capturable"; return FGPU_ERR_INVALID; }
    if (M->cv != 4) { ctx->err = "mesh_set_ho_nodes: tetrahedral meshes only"; return FGPU_ERR_INVALID; }
    if (!ho) {
        cudaFree(M->d_ho);
        M->d_ho = nullptr;
        return FGPU_OK;
    }
    const size_t bytes = (size_t)M->nt * 18 * sizeof(double);
    if (!M->d_ho) FGPU_CUDA_CHECK(ctx, cudaMalloc(&M->d_ho, std::max<size_t>(bytes, 8)));
    FGPU_CUDA_CHECK(ctx, cudaMemcpyAsync(M->d_ho, ho, bytes, cudaMemcpyHostToDevice, ctx->stream));
    FGPU_CUDA_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
    return FGPU_OK;
}
