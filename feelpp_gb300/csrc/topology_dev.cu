// Device construction of the dof table, the node -> element incidence and the
// scalar node pattern (the set-up that Feel++ runs on the host in DofTable::build
// and Stencil::computeGraph), giving the same arrays as topology.cpp bit for bit.
//
// Dof numbering. Feel++ numbers entity dofs by first encounter over the elements
// in insertion order, inside an element vertices 0..3, edges 0..5, faces 0..3
// (feelpp/feel/feeldiscr/doftable.hpp:1213-1250, 2364-2455; doffromelement.hpp:505-530).
// Equivalently: give each entity the key min over its occurrences of
// (element * 14 + local entity position), vertices at positions 0..3, edges 4..9,
// faces 10..13; an entity's first dof is the number of dofs of all entities with
// a smaller key. That is an exclusive scan over the key space weighted by the
// entities' dof counts, with no sort. An edge's two P3 dofs take their order from
// the orientation of the edge in its first element (REVERSE when
// id(e2p[j][0]) > id(e2p[j][1]), mesh3d.hpp:750-782, doffromelement.hpp:282-333).
//
// Edges and faces are identified through an open-addressing hash table of
// their sorted vertex ids (64-bit keys: faces pack three 21-bit ids, so meshes of
// up to 2^21 vertices; larger meshes use the host path). Entity ids in the table
// depend on the insertion order, the dof numbers do not.
//
// Incidence lists are filled with atomic cursors, then each list is sorted by
// element (a fixed result). Pattern rows are the sorted unique nodes of a row's
// elements (Stencil::computeGraph, stencil.hpp:1500-1692, COUPLED pattern), one
// warp per row with a shared-memory bitonic sort.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "fgpu_core.h"
#include "scan.cuh"

namespace fgpu {

namespace {

__constant__ int c_edge_verts[6][2];
__constant__ int c_face_verts[4][3];

constexpr unsigned long long kEmpty = ~0ull;
constexpr int kStatusTableFull = 32;     // hash table probe limit reached
constexpr int kStatusSortOverflow = 64;  // an incidence list or pattern row longer than the sort buffer

__device__ __forceinline__ uint32_t hash_insert(unsigned long long* tab, uint32_t mask, unsigned long long key, int* status) {
    uint32_t h = (uint32_t)((key * 0x9E3779B97F4A7C15ull) >> 32) & mask;
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        const unsigned long long prev = atomicCAS(tab + h, kEmpty, key);
        if (prev == kEmpty || prev == key) return h;
        h = (h + 1) & mask;
    }
    atomicOr(status, kStatusTableFull);
    return 0;
}

__global__ void entity_keys_kernel(int64_t nt, const int32_t* __restrict__ tets, int ndpe, int ndpf, uint32_t* __restrict__ kv,
                                   unsigned long long* __restrict__ etab, uint32_t emask, uint32_t* __restrict__ ke,
                                   unsigned long long* __restrict__ ftab, uint32_t fmask, uint32_t* __restrict__ kf,
                                   uint32_t* __restrict__ occ_e, uint32_t* __restrict__ occ_f, int* __restrict__ status) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nt; e += (int64_t)gridDim.x * blockDim.x) {
        const int4 t4 = *reinterpret_cast<const int4*>(tets + 4 * e);
        const int v[4] = {t4.x, t4.y, t4.z, t4.w};
        const uint32_t base = (uint32_t)(e * 14);
#pragma unroll
        for (int i = 0; i < 4; ++i) atomicMin(kv + v[i], base + i);
        if (ndpe > 0) {
#pragma unroll
            for (int j = 0; j < 6; ++j) {
                const int a = v[c_edge_verts[j][0]], b = v[c_edge_verts[j][1]];
                const unsigned long long key = ((unsigned long long)(uint32_t)min(a, b) << 32) | (uint32_t)max(a, b);
                const uint32_t s = hash_insert(etab, emask, key, status);
                occ_e[e * 6 + j] = s;
                atomicMin(ke + s, base + 4 + j);
            }
        }
        if (ndpf > 0) {
#pragma unroll
            for (int f = 0; f < 4; ++f) {
                int a = v[c_face_verts[f][0]], b = v[c_face_verts[f][1]], c = v[c_face_verts[f][2]];
                if (a > b) { const int x = a; a = b; b = x; }
                if (b > c) { const int x = b; b = c; c = x; }
                if (a > b) { const int x = a; a = b; b = x; }
                const unsigned long long key = ((unsigned long long)a << 42) | ((unsigned long long)b << 21) | (unsigned long long)c;
                const uint32_t s = hash_insert(ftab, fmask, key, status);
                occ_f[e * 4 + f] = s;
                atomicMin(kf + s, base + 10 + f);
            }
        }
    }
}

// dof counts at the first-encounter keys of the entities
__global__ void entity_weights_kernel(int64_t nv, const uint32_t* __restrict__ kv, int64_t ecap,
                                      const unsigned long long* __restrict__ etab, const uint32_t* __restrict__ ke, int ndpe,
                                      int64_t fcap, const unsigned long long* __restrict__ ftab, const uint32_t* __restrict__ kf,
                                      int ndpf, uint32_t* __restrict__ w) {
    const int64_t total = nv + ecap + fcap;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        if (i < nv) {
            if (kv[i] != 0xFFFFFFFFu) w[kv[i]] = 1;
        } else if (i < nv + ecap) {
            const int64_t s = i - nv;
            if (etab[s] != kEmpty) w[ke[s]] = (uint32_t)ndpe;
        } else {
            const int64_t s = i - nv - ecap;
            if (ftab[s] != kEmpty) w[kf[s]] = (uint32_t)ndpf;
        }
    }
}

__global__ void l2n_kernel(int64_t nt, const int32_t* __restrict__ tets, int n, int ndpe, int ndpf, const uint32_t* __restrict__ kv,
                           const uint32_t* __restrict__ ke, const uint32_t* __restrict__ kf, const uint32_t* __restrict__ occ_e,
                           const uint32_t* __restrict__ occ_f, const uint32_t* __restrict__ off, int32_t* __restrict__ l2n) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nt; e += (int64_t)gridDim.x * blockDim.x) {
        const int4 t4 = *reinterpret_cast<const int4*>(tets + 4 * e);
        const int v[4] = {t4.x, t4.y, t4.z, t4.w};
        int32_t* out = l2n + e * n;
        int lc = 0;
        for (int i = 0; i < 4; ++i) out[lc++] = (int32_t)off[kv[v[i]]];
        for (int j = 0; j < 6 && ndpe > 0; ++j) {
            const uint32_t key1 = ke[occ_e[e * 6 + j]];
            const int64_t e1 = key1 / 14;
            const int j1 = (int)(key1 - e1 * 14) - 4;
            const int4 u4 = *reinterpret_cast<const int4*>(tets + 4 * e1);
            const int u[4] = {u4.x, u4.y, u4.z, u4.w};
            const bool rev1 = u[c_edge_verts[j1][0]] > u[c_edge_verts[j1][1]];
            const bool rev = v[c_edge_verts[j][0]] > v[c_edge_verts[j][1]];
            const uint32_t base = off[key1];
            for (int l = 0; l < ndpe; ++l) {
                const int s = rev ? ndpe - 1 - l : l;                 // edge slot of this local dof
                out[lc++] = (int32_t)(base + (rev1 ? ndpe - 1 - s : s));  // slots numbered in the first element's order
            }
        }
        for (int f = 0; f < 4 && ndpf > 0; ++f) {
            const uint32_t base = off[kf[occ_f[e * 4 + f]]];
            for (int l = 0; l < ndpf; ++l) out[lc++] = (int32_t)(base + l);
        }
    }
}

__global__ void count_nodes_kernel(int64_t total, const int32_t* __restrict__ l2n, uint32_t* __restrict__ cnt) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total; k += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(cnt + l2n[k], 1u);
}

__global__ void u32_to_i64_kernel(int64_t n, const uint32_t* __restrict__ in, int64_t* __restrict__ out) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) out[k] = in[k];
}

__global__ void fill_incidence_kernel(int64_t nt, int n, const int32_t* __restrict__ l2n, uint32_t* __restrict__ cursor,
                                      int32_t* __restrict__ inc) {
    const int64_t total = nt * n;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = k / n;
        const int l = (int)(k - e * n);
        const uint32_t p = atomicAdd(cursor + l2n[k], 1u);
        inc[p] = (int32_t)((e << 5) | l);
    }
}

// Bitonic sort of buf[0, S) (S a power of two, padded with INT_MAX) by one warp.
__device__ void warp_bitonic_sort(int32_t* buf, int S, int lane) {
    for (int k = 2; k <= S; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < S; i += 32) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const int32_t a = buf[i], b = buf[ixj];
                    const bool up = (i & k) == 0;
                    if ((a > b) == up) { buf[i] = b; buf[ixj] = a; }
                }
            }
            __syncwarp();
        }
    }
}

// Sort each node's incidence list by element (warp per node).
__global__ void sort_incidence_kernel(int64_t nnodes, const int64_t* __restrict__ ptr, int32_t* __restrict__ inc, int S,
                                      int* __restrict__ status) {
    extern __shared__ int32_t sbuf[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int32_t* buf = sbuf + (size_t)warp * S;
    for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp; r < nnodes; r += (int64_t)gridDim.x * (blockDim.x >> 5)) {
        const int64_t b = ptr[r];
        const int len = (int)(ptr[r + 1] - b);
        if (len > S) {
            if (lane == 0) atomicOr(status, kStatusSortOverflow);
            continue;
        }
        int P = 1;
        while (P < len) P <<= 1;
        for (int i = lane; i < P; i += 32) buf[i] = i < len ? inc[b + i] : 0x7FFFFFFF;
        __syncwarp();
        warp_bitonic_sort(buf, P, lane);
        for (int i = lane; i < len; i += 32) inc[b + i] = buf[i];
        __syncwarp();
    }
}

// Pattern rows: sorted unique nodes of the elements of each row. pass 0 counts
// (cnt[r]), pass 1 writes ja[ia[r] ...]; max_row by atomicMax.
__global__ void pattern_rows_kernel(int64_t nrows, int n, const int64_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                                    const int32_t* __restrict__ l2n, int S, int pass, uint32_t* __restrict__ cnt,
                                    const int64_t* __restrict__ ia, int32_t* __restrict__ ja, int* __restrict__ max_row,
                                    int* __restrict__ status) {
    extern __shared__ int32_t sbuf[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int32_t* buf = sbuf + (size_t)warp * S;
    for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp; r < nrows; r += (int64_t)gridDim.x * (blockDim.x >> 5)) {
        const int64_t b = inc_ptr[r];
        const int m = (int)(inc_ptr[r + 1] - b);
        const int C = m * n;
        if (C > S) {
            if (lane == 0) atomicOr(status, kStatusSortOverflow);
            continue;
        }
        int P = 1;
        while (P < C) P <<= 1;
        for (int i = lane; i < P; i += 32) {
            int32_t x = 0x7FFFFFFF;
            if (i < C) {
                const int k = i / n, j = i - k * n;
                x = l2n[(int64_t)(inc[b + k] >> 5) * n + j];
            }
            buf[i] = x;
        }
        __syncwarp();
        warp_bitonic_sort(buf, P, lane);
        // unique entries in order: position = number of distinct values before
        int run = 0;
        for (int i0 = 0; i0 < C; i0 += 32) {
            const int i = i0 + lane;
            const bool first = i < C && (i == 0 || buf[i] != buf[i - 1]);
            const unsigned bal = __ballot_sync(0xffffffffu, first);
            if (pass == 1 && first) ja[ia[r] + run + __popc(bal & ((1u << lane) - 1u))] = buf[i];
            run += __popc(bal);
        }
        if (pass == 0 && lane == 0) {
            cnt[r] = (uint32_t)run;
            atomicMax(max_row, run);
        }
        __syncwarp();
    }
}

int sort_buffer_size(int64_t need) {
    int S = 32;
    while (S < need) S <<= 1;
    return S;
}

}  // namespace

// Builds V->d_l2n, d_inc_ptr, d_inc and the host copies topo.l2n / nnodes
// (used by the host queries). Returns FGPU_ERR_INVALID with an empty message
// when the mesh is outside this path's limits (the caller then uses the host path).
// reference-element tables in constant memory, once per device
static int ensure_tables(fgpu_ctx* ctx) {
    static std::mutex mu;
    static std::vector<char> done(256, 0);
    std::lock_guard<std::mutex> lock(mu);
    if (ctx->device < 0 || ctx->device >= 256) return FGPU_ERR_INVALID;
    if (!done[ctx->device]) {
        FGPU_CUDA_CHECK(ctx, cudaMemcpyToSymbol(c_edge_verts, kEdgeVerts, sizeof(int) * 12));
        FGPU_CUDA_CHECK(ctx, cudaMemcpyToSymbol(c_face_verts, kFaceVerts, sizeof(int) * 12));
        done[ctx->device] = 1;
    }
    return FGPU_OK;
}

int build_space_device(fgpu_ctx* ctx, fgpu_space* V) {
    const fgpu_mesh* M = V->mesh;
    const int64_t nt = M->nt, nv = M->nv;
    const int order = V->order, n = V->n, ndpe = dofs_per_edge(order), ndpf = dofs_per_face(order);
    if (M->cv != 4) return FGPU_ERR_INVALID;
    if (nv >= ((int64_t)1 << 21) || nt * 14 >= (int64_t)0xFFFFFFFF || nt >= ((int64_t)1 << 26)) return FGPU_ERR_INVALID;
    {
        const int rc = ensure_tables(ctx);
        if (rc) return rc;
    }
    // the host path's input checks: vertex range and repeated vertices
    for (int64_t k = 0; k < nt; ++k) {
        const int32_t* t = M->h_tets.data() + 4 * k;
        for (int i = 0; i < 4; ++i)
            if (t[i] < 0 || t[i] >= nv) { ctx->err = "tetrahedron vertex index out of range"; return FGPU_ERR_OUT_OF_RANGE; }
        if (t[0] == t[1] || t[0] == t[2] || t[0] == t[3] || t[1] == t[2] || t[1] == t[3] || t[2] == t[3]) {
            ctx->err = "tetrahedron with a repeated vertex";
            return FGPU_ERR_OUT_OF_RANGE;
        }
    }
    uint32_t ecap = 1, fcap = 1;
    while (ecap < (uint64_t)nt * 6 / 2 + 1024) ecap <<= 1;     // > 2x the number of edges (about 1.2 T)
    while (fcap < (uint64_t)nt * 4 + 1024) fcap <<= 1;         // > 2x the number of faces (about 2 T)
    if (ndpe == 0) ecap = 1;
    if (ndpf == 0) fcap = 1;
    uint32_t *kv = nullptr, *ke = nullptr, *kf = nullptr, *occ_e = nullptr, *occ_f = nullptr, *w = nullptr, *off = nullptr;
    unsigned long long *etab = nullptr, *ftab = nullptr;
    uint32_t* cnt = nullptr;
    auto cleanup = [&]() {
        cudaFree(kv); cudaFree(ke); cudaFree(kf); cudaFree(occ_e); cudaFree(occ_f); cudaFree(w); cudaFree(off);
        cudaFree(etab); cudaFree(ftab); cudaFree(cnt);
    };
    cudaError_t e = cudaMalloc(&kv, nv * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&ke, (size_t)ecap * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&kf, (size_t)fcap * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&etab, (size_t)ecap * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&ftab, (size_t)fcap * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&occ_e, (size_t)(ndpe ? nt * 6 : 1) * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&occ_f, (size_t)(ndpf ? nt * 4 : 1) * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&w, (size_t)nt * 14 * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&off, ((size_t)nt * 14 + 1) * sizeof(uint32_t));
    if (e != cudaSuccess) { cudaGetLastError(); cleanup(); ctx->err = "device dof table: allocation failed"; return FGPU_ERR_ALLOC; }
    cudaStream_t s = ctx->stream;
    cudaMemsetAsync(kv, 0xFF, nv * sizeof(uint32_t), s);
    cudaMemsetAsync(ke, 0xFF, (size_t)ecap * sizeof(uint32_t), s);
    cudaMemsetAsync(kf, 0xFF, (size_t)fcap * sizeof(uint32_t), s);
    cudaMemsetAsync(etab, 0xFF, (size_t)ecap * sizeof(unsigned long long), s);
    cudaMemsetAsync(ftab, 0xFF, (size_t)fcap * sizeof(unsigned long long), s);
    cudaMemsetAsync(w, 0, (size_t)nt * 14 * sizeof(uint32_t), s);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int eb = (int)std::max<int64_t>(1, std::min<int64_t>((nt + 255) / 256, (int64_t)sms * 16));
    entity_keys_kernel<<<eb, 256, 0, s>>>(nt, M->d_tets, ndpe, ndpf, kv, etab, ecap - 1, ke, ftab, fcap - 1, kf, occ_e, occ_f,
                                          ctx->d_status);
    entity_weights_kernel<<<sms * 16, 256, 0, s>>>(nv, kv, ndpe ? ecap : 0, etab, ke, ndpe, ndpf ? fcap : 0, ftab, kf, ndpf, w);
    ctx->launches += 2;
    uint64_t ndof_nodes = 0;
    int rc = scan_u32(ctx, w, off, nt * 14, &ndof_nodes);
    if (rc) { cleanup(); return rc; }
    int hst = 0;
    cudaMemcpy(&hst, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost);
    if (hst & kStatusTableFull) { cudaMemset(ctx->d_status, 0, sizeof(int)); cleanup(); ctx->err = "device dof table: hash table full"; return FGPU_ERR_INVALID; }
    if (ndof_nodes >= ((uint64_t)1 << 31)) { cleanup(); ctx->err = "too many dofs for 32-bit indices"; return FGPU_ERR_INVALID; }
    const int64_t N = (int64_t)ndof_nodes;
    e = cudaMalloc(&V->d_l2n, (size_t)nt * n * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&V->d_inc_ptr, (size_t)(N + 1) * sizeof(int64_t));
    if (e == cudaSuccess) e = cudaMalloc(&V->d_inc, (size_t)nt * n * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&cnt, (size_t)(N + 1) * sizeof(uint32_t));
    if (e != cudaSuccess) { cudaGetLastError(); cleanup(); ctx->err = "device dof table: allocation failed"; return FGPU_ERR_ALLOC; }
    l2n_kernel<<<eb, 256, 0, s>>>(nt, M->d_tets, n, ndpe, ndpf, kv, ke, kf, occ_e, occ_f, off, V->d_l2n);
    ctx->launches++;
    // incidence
    // the list offsets reuse `off` (14 T + 1 entries); very small meshes (a P3 element alone carries 20
    // nodes) get their own buffer
    uint32_t* cptr = off;
    if (N > nt * 14) {
        cudaStreamSynchronize(s);         // l2n_kernel has read the entity offsets
        cudaFree(off);
        off = nullptr;
        if (cudaMalloc(&off, (size_t)(N + 1) * sizeof(uint32_t)) != cudaSuccess) {
            cudaGetLastError(); cleanup(); ctx->err = "device dof table: allocation failed"; return FGPU_ERR_ALLOC;
        }
        cptr = off;
    }
    cudaMemsetAsync(cnt, 0, (size_t)(N + 1) * sizeof(uint32_t), s);
    const int64_t tn = nt * n;
    const int cb = (int)std::max<int64_t>(1, std::min<int64_t>((tn + 255) / 256, (int64_t)sms * 16));
    count_nodes_kernel<<<cb, 256, 0, s>>>(tn, V->d_l2n, cnt);
    ctx->launches++;
    uint64_t tot = 0;
    rc = scan_u32(ctx, cnt, cptr, N, &tot);
    if (rc) { cleanup(); return rc; }
    u32_to_i64_kernel<<<sms * 8, 256, 0, s>>>(N + 1, cptr, V->d_inc_ptr);
    fill_incidence_kernel<<<cb, 256, 0, s>>>(nt, n, V->d_l2n, cptr, V->d_inc);   // cptr advances to the list ends
    ctx->launches += 2;
    // longest incidence list (host: from the counts)
    std::vector<int64_t> hptr(N + 1);
    cudaMemcpyAsync(hptr.data(), V->d_inc_ptr, (N + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    int64_t maxinc = 0;
    for (int64_t r = 0; r < N; ++r) maxinc = std::max(maxinc, hptr[r + 1] - hptr[r]);
    const int Si = sort_buffer_size(maxinc);
    const int wpb = std::max(1, std::min(8, (int)(32768 / (Si * 4))));
    sort_incidence_kernel<<<sms * 8, wpb * 32, (size_t)wpb * Si * 4, s>>>(N, V->d_inc_ptr, V->d_inc, Si, ctx->d_status);
    ctx->launches++;
    e = cudaGetLastError();
    // host copies for the host-side queries (l2g, boundary dofs)
    V->topo.order = order;
    V->topo.n = n;
    V->topo.nnodes = N;
    V->topo.l2n.resize((size_t)nt * n);
    V->topo.inc_ptr.swap(hptr);
    if (e == cudaSuccess) e = cudaMemcpyAsync(V->topo.l2n.data(), V->d_l2n, (size_t)nt * n * sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cleanup();
    if (e != cudaSuccess) { ctx->err = std::string("device dof table: ") + cudaGetErrorString(e); return FGPU_ERR_CUDA; }
    V->dev_topology = true;
    V->max_incidence = (int)maxinc;
    return FGPU_OK;
}

// Scalar node pattern on the device from the incidence lists (after build_space_device
// or the host topology upload). Fills P (device ia/ja, nnz, max_row) and the host ia.
namespace {

// boundary faces: every local face is inserted in a face hash with an occurrence count
__global__ void face_count_kernel(int64_t nt, const int32_t* __restrict__ tets, unsigned long long* __restrict__ ftab, uint32_t fmask,
                                  uint32_t* __restrict__ occ, uint32_t* __restrict__ cnt, int* __restrict__ status) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt * 4; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = t >> 2;
        const int f = (int)(t & 3);
        int a = tets[4 * e + c_face_verts[f][0]], b = tets[4 * e + c_face_verts[f][1]], c = tets[4 * e + c_face_verts[f][2]];
        if (a > b) { const int x = a; a = b; b = x; }
        if (b > c) { const int x = b; b = c; c = x; }
        if (a > b) { const int x = a; a = b; b = x; }
        const unsigned long long key = ((unsigned long long)a << 42) | ((unsigned long long)b << 21) | (unsigned long long)c;
        const uint32_t sl = hash_insert(ftab, fmask, key, status);
        occ[t] = sl;
        atomicAdd(cnt + sl, 1u);
    }
}

// the nodes carried by faces of one element (with xmax_on: whose vertices all have x <= xmax)
__global__ void boundary_mark_kernel(int64_t nt, const int32_t* __restrict__ tets, const double* __restrict__ xyz, int n,
                                     const int32_t* __restrict__ l2n, const uint32_t* __restrict__ occ, const uint32_t* __restrict__ cnt,
                                     const int* __restrict__ fl, int nfl, int xmax_on, double xmax, uint8_t* __restrict__ mark) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt * 4; t += (int64_t)gridDim.x * blockDim.x) {
        if (cnt[occ[t]] != 1) continue;
        const int64_t e = t >> 2;
        const int f = (int)(t & 3);
        if (xmax_on) {
            bool ok = true;
            for (int v = 0; v < 3; ++v) ok = ok && xyz[3 * (int64_t)tets[4 * e + c_face_verts[f][v]]] <= xmax + 1e-12;
            if (!ok) continue;
        }
        for (int k = 0; k < nfl; ++k) mark[l2n[e * n + fl[f * nfl + k]]] = 1;
    }
}

}  // namespace

// Boundary dof nodes on the device (the host restatement is topology.cpp boundary_nodes): FGPU_OK, or
// FGPU_ERR_INVALID when the mesh is too large for the packed face keys (the caller then uses the host).
int boundary_nodes_device(fgpu_ctx* ctx, const fgpu_space* V, int xmax_on, double xmax, std::vector<int32_t>& nodes) {
    const fgpu_mesh* M = V->mesh;
    const int64_t nt = M->nt;
    if (M->cv != 4 || M->nv >= ((int64_t)1 << 21) || nt == 0) return FGPU_ERR_INVALID;
    if (ensure_tables(ctx) != FGPU_OK) return FGPU_ERR_INVALID;
    const int ndpe = dofs_per_edge(V->order), ndpf = dofs_per_face(V->order);
    std::vector<int> fl;
    int nfl = 0;
    for (int f = 0; f < 4; ++f) {
        std::vector<int> d;
        for (int v = 0; v < 3; ++v) d.push_back(kFaceVerts[f][v]);
        for (int j = 0; j < 6; ++j) {
            const int a = kEdgeVerts[j][0], b = kEdgeVerts[j][1];
            bool ina = false, inb = false;
            for (int v = 0; v < 3; ++v) {
                ina |= kFaceVerts[f][v] == a;
                inb |= kFaceVerts[f][v] == b;
            }
            if (ina && inb)
                for (int l = 0; l < ndpe; ++l) d.push_back(4 + j * ndpe + l);
        }
        for (int l = 0; l < ndpf; ++l) d.push_back(4 + 6 * ndpe + f * ndpf + l);
        nfl = (int)d.size();
        fl.insert(fl.end(), d.begin(), d.end());
    }
    uint32_t cap = 1;
    while (cap < (uint32_t)std::min<int64_t>(4 * nt, (int64_t)1 << 31)) cap <<= 1;
    const int64_t nnodes = V->topo.nnodes;
    unsigned long long* ftab = nullptr;
    uint32_t *occ = nullptr, *cnt = nullptr;
    int* dfl = nullptr;
    uint8_t* mark = nullptr;
    auto cleanup = [&]() { cudaFree(ftab); cudaFree(occ); cudaFree(cnt); cudaFree(dfl); cudaFree(mark); };
    cudaError_t e = cudaMalloc(&ftab, (size_t)cap * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&cnt, (size_t)cap * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&occ, (size_t)nt * 4 * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&dfl, fl.size() * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&mark, std::max<int64_t>(nnodes, 1));
    if (e == cudaSuccess) e = cudaMemsetAsync(ftab, 0xFF, (size_t)cap * sizeof(unsigned long long), ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(cnt, 0, (size_t)cap * sizeof(uint32_t), ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(mark, 0, std::max<int64_t>(nnodes, 1), ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dfl, fl.data(), fl.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream);
    if (e != cudaSuccess) { cudaGetLastError(); cleanup(); return FGPU_ERR_INVALID; }
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((nt * 4 + 255) / 256, 152 * 32));
    face_count_kernel<<<blocks, 256, 0, ctx->stream>>>(nt, M->d_tets, ftab, cap - 1, occ, cnt, ctx->d_status);
    boundary_mark_kernel<<<blocks, 256, 0, ctx->stream>>>(nt, M->d_tets, M->d_xyz, V->n, V->d_l2n, occ, cnt, dfl, nfl, xmax_on, xmax,
                                                          mark);
    ctx->launches += 2;
    int st = 0;
    std::vector<uint8_t> hm(nnodes);
    e = cudaMemcpyAsync(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hm.data(), mark, nnodes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cleanup();
    if (e != cudaSuccess) { ctx->err = std::string("boundary dofs: ") + cudaGetErrorString(e); return FGPU_ERR_CUDA; }
    if (st & kStatusTableFull) {
        cudaMemset(ctx->d_status, 0, sizeof(int));
        return FGPU_ERR_INVALID;
    }
    nodes.clear();
    for (int64_t r = 0; r < nnodes; ++r)
        if (hm[r]) nodes.push_back((int32_t)r);
    return FGPU_OK;
}

int build_pattern_device(fgpu_ctx* ctx, fgpu_space* V, DevPattern& P, std::vector<int64_t>& h_ia) {
    const int64_t N = V->topo.nnodes;
    const int n = V->n;
    int maxinc = V->max_incidence;
    if (maxinc <= 0) {
        for (int64_t r = 0; r < N; ++r) maxinc = std::max<int64_t>(maxinc, V->topo.inc_ptr[r + 1] - V->topo.inc_ptr[r]);
    }
    const int S = sort_buffer_size((int64_t)maxinc * n);
    if (S > 4096) { ctx->err = "device pattern: rows too long for the sort buffer"; return FGPU_ERR_INVALID; }
    const int wpb = std::max(1, std::min(8, (int)(32768 / (S * 4))));
    uint32_t *cnt = nullptr, *ptr32 = nullptr;
    int* dmax = nullptr;
    cudaError_t e = cudaMalloc(&cnt, (size_t)(N + 1) * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&ptr32, (size_t)(N + 1) * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&dmax, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&P.d_ia, (size_t)(N + 1) * sizeof(int64_t));
    auto cleanup = [&]() { cudaFree(cnt); cudaFree(ptr32); cudaFree(dmax); };
    if (e != cudaSuccess) { cudaGetLastError(); cleanup(); ctx->err = "device pattern: allocation failed"; return FGPU_ERR_ALLOC; }
    cudaStream_t s = ctx->stream;
    cudaMemsetAsync(dmax, 0, sizeof(int), s);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const size_t smem = (size_t)wpb * S * 4;
    pattern_rows_kernel<<<sms * 8, wpb * 32, smem, s>>>(N, n, V->d_inc_ptr, V->d_inc, V->d_l2n, S, 0, cnt, nullptr, nullptr, dmax,
                                                       ctx->d_status);
    ctx->launches++;
    uint64_t nnz = 0;
    int rc = scan_u32(ctx, cnt, ptr32, N, &nnz);
    if (rc) { cleanup(); return rc; }
    u32_to_i64_kernel<<<sms * 8, 256, 0, s>>>(N + 1, ptr32, P.d_ia);
    e = cudaMalloc(&P.d_ja, (size_t)std::max<uint64_t>(nnz, 1) * sizeof(int32_t));
    if (e != cudaSuccess) { cudaGetLastError(); cleanup(); ctx->err = "device pattern: allocation failed"; return FGPU_ERR_ALLOC; }
    pattern_rows_kernel<<<sms * 8, wpb * 32, smem, s>>>(N, n, V->d_inc_ptr, V->d_inc, V->d_l2n, S, 1, nullptr, P.d_ia, P.d_ja, dmax,
                                                       ctx->d_status);
    ctx->launches += 2;
    int mx = 0, hst = 0;
    cudaMemcpyAsync(&mx, dmax, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&hst, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, s);
    h_ia.resize(N + 1);
    cudaMemcpyAsync(h_ia.data(), P.d_ia, (N + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, s);
    e = cudaStreamSynchronize(s);
    cleanup();
    if (e != cudaSuccess) { ctx->err = std::string("device pattern: ") + cudaGetErrorString(e); return FGPU_ERR_CUDA; }
    if (hst & kStatusSortOverflow) {
        cudaMemset(ctx->d_status, 0, sizeof(int));
        ctx->err = "device pattern: sort buffer overflow";
        return FGPU_ERR_INVALID;
    }
    P.nrows = N;
    P.nnz = (int64_t)nnz;
    P.max_row = mx;
    return FGPU_OK;
}

}  // namespace fgpu
