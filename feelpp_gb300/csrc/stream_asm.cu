// Streamed two-phase assembly of the affine Laplace/mass form (FGPU_ALGO_STREAMED).
//
// The two-phase assembly (assemble.cu) computes every element matrix once into
// a T x n(n+1)/2 element buffer in device memory, then sums each CSR entry's
// contributions in element order through a gather map of T n^2 indices. Both
// buffers make it move about three times the algorithmic bytes of an assembly
// (CSR values written once, pattern and element data read once).
//
// This kernel does the same arithmetic in the same order, so its values are
// bit-identical to the two-phase path, without either buffer:
//  * element tasks (EC consecutive elements) form the df64 coefficient record
//    of each element from the vertex coordinates in shared memory and write the
//    element's upper triangle into a ring of R element slots (R a power of two,
//    a few tens of MB: it stays in L2, stored with an evict-last policy);
//  * gather tasks (RG consecutive pattern rows) walk each row's incident
//    elements in element order (the reference's element loop order,
//    bilinearformcontext.hpp:784-847 -> MatSetValues ADD_VALUES) with one lane
//    per element column, read the entry from the ring and its offset in the row
//    from the position table, accumulate in shared memory and write the row's
//    CSR values once.
// One persistent launch runs both kinds of task. Tasks are handed out by a
// ticket counter in an order built once per space on the host: a gather task
// comes after the element tasks that produce its rows' elements, and an element
// task comes after the gather tasks that still read the ring slots it
// overwrites. A task waits only for tasks with smaller tickets, which are held
// by blocks already running, so the waits always end; each wait is bounded
// anyway (a timeout sets a status bit and every block returns).
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "asm_device.cuh"
#include "df64.h"
#include "fgpu_core.h"

namespace fgpu {

void prof_begin(fgpu_ctx* ctx, const char* name, PendingEvent& ev);
void prof_end(fgpu_ctx* ctx, PendingEvent& ev);

namespace {

constexpr int kEC = 256;                 // elements per element task (one thread per element for the geometry)
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr long long kMaxSpins = 1LL << 23;   // x ~200 ns sleeps: a wait gives up after a few seconds

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(uint32_t* p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint64_t evict_last_policy() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ void st_keep(float2* p, float2 v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(p), "f"(v.x), "f"(v.y), "l"(pol) : "memory");
}
__device__ __forceinline__ void st_keep(float* p, float v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(p), "f"(v), "l"(pol) : "memory");
}

// Control block, zeroed before each launch: [0] ticket counter, [1] element-task
// watermark (element tasks 0..w-1 done), [2] gather watermark, [3] abort flag,
// then one done flag per element task and per gather task.
struct StreamArgs {
    int64_t nt, nrows, ntickets;
    const double* xyz;
    const int32_t* tets;
    const double* kappa;
    double kappa_c, mass;
    const double* kscale;
    const int64_t* ia;
    const int64_t* inc_ptr;
    const int32_t* inc;
    const uint8_t* pos;
    const float* Th;                      // 7 x NTRI reference tensors (upper triangle), df64 hi / lo
    const float* Tl;
    const uint16_t* tri;                  // n x n -> upper-triangle index of (min, max)
    void* ring;
    int64_t ring_mask;                    // ring slots - 1
    void* val;
    double* hout;                         // mapped page-locked host copy of the values (FP64) or null
    int accumulate;
    const int32_t* ticket;                // >= 0: element task k; < 0: gather task -(s + 1)
    const int32_t* e_need_g;              // per element task: gather watermark to wait for
    const int32_t* g_need_e;              // per gather task: element watermark to wait for
    const int32_t* g_rows;                // per gather task: first row (rows g_rows[s] .. g_rows[s] + rg - 1)
    uint32_t* ctl;
    int ne, ng, rg, maxrow;
    int* status;
};

// Wait (one thread) until watermark >= need, advancing the shared watermark over
// the done flags. Returns false when the launch was aborted or the wait gave up.
__device__ __forceinline__ bool wait_mark(uint32_t* mark, const uint32_t* done, uint32_t need, uint32_t* abort, int* status) {
    uint32_t w = ld_acquire(mark);
    long long spins = 0;
    while (w < need) {
        const uint32_t w0 = w;
        while (w < need && ld_acquire(done + w)) ++w;
        if (w > w0) {
            __threadfence();
            atomicMax(mark, w);
        }
        if (w >= need) break;
        if (ld_acquire(abort)) return false;
        if (++spins > kMaxSpins) {
            atomicExch(abort, 1u);
            atomicOr(status, kStatusStreamTimeout);
            return false;
        }
        __nanosleep(200);
        const uint32_t m = ld_acquire(mark);
        if (m > w) w = m;
    }
    return true;
}

template <int MODE, int N>
__global__ void __launch_bounds__(kThreads) stream_assemble_kernel(StreamArgs a) {
    constexpr int NTRI = N * (N + 1) / 2;
    constexpr int EPW = NTRI >= 32 ? 1 : 32 / NTRI;         // elements per warp pass (element tasks)
    constexpr int RPW = 32 / N;                             // rows per warp pass (gather tasks)
    constexpr int ACCW = MODE == kModeDF64 ? 2 : 1;
    constexpr int kRecOff = (14 * NTRI + 3) & ~3;           // floats before the records
    extern __shared__ __align__(16) unsigned char smem[];
    float* Th = reinterpret_cast<float*>(smem);
    float* Tl = Th + 7 * NTRI;
    float* rec = Th + kRecOff;                              // kEC x 16, 16-byte aligned
    uint16_t* tri = reinterpret_cast<uint16_t*>(rec + kEC * 16);
    float* accb = reinterpret_cast<float*>(tri + ((N * N + 7) & ~7));
    __shared__ int s_ticket, s_ok;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int k = tid; k < 7 * NTRI; k += kThreads) {
        Th[k] = a.Th[k];
        if (MODE == kModeDF64) Tl[k] = a.Tl[k];
    }
    for (int k = tid; k < N * N; k += kThreads) tri[k] = a.tri[k];
    float* acc = accb + (size_t)warp * RPW * a.maxrow * ACCW;
    for (int k = lane; k < RPW * a.maxrow * ACCW; k += 32) acc[k] = MODE == kModeDF64 ? 0.0f : -0.0f;
    const uint64_t keep = evict_last_policy();
    const df kc = d2df(a.kappa_c), mc = d2df(a.mass);
    const df ksc = a.kscale ? d2df(*a.kscale) : df{1.0f, 0.0f};
    uint32_t* abort = a.ctl + 3;
    uint32_t* e_done = a.ctl + 4;
    uint32_t* g_done = e_done + a.ne;
    __syncthreads();

    for (;;) {
        if (tid == 0) s_ticket = (int)atomicAdd(a.ctl, 1u);
        __syncthreads();
        const int64_t t = s_ticket;
        if (t >= a.ntickets) break;
        const int code = a.ticket[t];
        if (code >= 0) {
            // ---- element task: elements e0 .. e0 + cnt - 1 into ring slots (e0 & mask) ..
            const int64_t e0 = (int64_t)code * kEC;
            const int cnt = (int)min((int64_t)kEC, a.nt - e0);
            if (tid == 0) s_ok = a.e_need_g[code] > 0
                                     ? wait_mark(a.ctl + 2, g_done, (uint32_t)a.e_need_g[code], abort, a.status)
                                     : !ld_acquire(abort);
            if (tid < cnt)
                geometry_df_record(e0 + tid, a.xyz, a.tets, a.kappa, kc, mc, ksc, reinterpret_cast<float4*>(rec + 16 * tid),
                                   a.status);
            __syncthreads();
            if (!s_ok) break;
            const int sub = lane / NTRI < EPW ? lane / NTRI : EPW;
            const int t0 = EPW > 1 ? lane - sub * NTRI : lane;
            const int64_t slot0 = e0 & a.ring_mask;
            for (int le = warp * EPW + sub; sub < EPW && le < cnt; le += kWarps * EPW) {
                float ch[7], cl[7];
                const float* r = rec + 16 * le;
#pragma unroll
                for (int k = 0; k < 7; ++k) {
                    ch[k] = r[k];
                    cl[k] = r[8 + k];
                }
                for (int tt = t0; tt < NTRI; tt += (EPW > 1 ? NTRI : 32)) {
                    if (MODE == kModeDF64) {
                        const df v = coef_entry_df(ch, cl, Th, Tl, NTRI, tt);
                        st_keep(reinterpret_cast<float2*>(a.ring) + (slot0 + le) * NTRI + tt, make_float2(v.hi, v.lo), keep);
                    } else {
                        st_keep(reinterpret_cast<float*>(a.ring) + (slot0 + le) * NTRI + tt, coef_entry_f(ch, Th, NTRI, tt), keep);
                    }
                }
            }
            __syncthreads();
            if (tid == 0) {
                __threadfence();
                st_release(e_done + code, 1u);
            }
        } else {
            // ---- gather task: rows r0 .. r0 + rg - 1, each summed in element order
            const int s = -code - 1;
            const int64_t r0 = a.g_rows[s];
            const int64_t r1 = min(a.nrows, r0 + a.rg);
            if (tid == 0) s_ok = wait_mark(a.ctl + 1, e_done, (uint32_t)a.g_need_e[s], abort, a.status);
            __syncthreads();
            if (!s_ok) break;
            const int sub = lane / N, j = lane - sub * N;
            float* myacc = acc + (size_t)(sub < RPW ? sub : 0) * a.maxrow * ACCW;
            for (int64_t rb = r0 + (int64_t)warp * RPW; rb < r1; rb += (int64_t)kWarps * RPW) {
                const int64_t r = rb + sub;
                if (sub < RPW && r < r1) {
                    const int64_t tb = a.inc_ptr[r], te = a.inc_ptr[r + 1];
                    for (int64_t c = tb; c < te; ++c) {
                        const int32_t code2 = __ldg(a.inc + c);
                        const int64_t e = code2 >> 5;
                        const int li = code2 & 31;
                        const int p = __ldcs(a.pos + (e * N + li) * N + j);
                        const int64_t src = (e & a.ring_mask) * NTRI + tri[li * N + j];
                        if (MODE == kModeDF64) {
                            const float2 v = __ldcg(reinterpret_cast<const float2*>(a.ring) + src);
                            const df tw = two_sum(myacc[2 * p], v.x);
                            myacc[2 * p] = tw.hi;
                            myacc[2 * p + 1] = f_add(myacc[2 * p + 1], f_add(tw.lo, v.y));
                        } else {
                            const float v = __ldcg(reinterpret_cast<const float*>(a.ring) + src);
                            myacc[p] = f_add(myacc[p], v);
                        }
                    }
                }
                __syncwarp();
                // write the rows of this pass: all 32 lanes over each row's entries
#pragma unroll 1
                for (int q = 0; q < RPW; ++q) {
                    const int64_t rq = rb + q;
                    if (rq >= r1) break;
                    const int64_t start = a.ia[rq];
                    const int len = (int)(a.ia[rq + 1] - start);
                    float* qa = acc + (size_t)q * a.maxrow * ACCW;
                    for (int k = lane; k < len; k += 32) {
                        if (MODE == kModeDF64) {
                            df sv = two_sum(qa[2 * k], qa[2 * k + 1]);
                            qa[2 * k] = 0.0f;
                            qa[2 * k + 1] = 0.0f;
                            double* out = reinterpret_cast<double*>(a.val) + start + k;
                            if (a.accumulate) sv = df_add(d2df(*out), sv);
                            const double rv = df2d(sv);
                            __stcs(out, rv);
                            if (a.hout) a.hout[start + k] = rv;
                        } else {
                            const float sv = qa[k];
                            qa[k] = -0.0f;
                            float* out = reinterpret_cast<float*>(a.val) + start + k;
                            __stcs(out, a.accumulate ? f_add(*out, sv) : sv);
                        }
                    }
                }
                __syncwarp();
            }
            __syncthreads();
            if (tid == 0) {
                __threadfence();
                st_release(g_done + s, 1u);
            }
        }
        __syncthreads();
    }
}

// last incident element of each pattern row (incidence lists are sorted by element)
__global__ void row_last_elem_kernel(int64_t nrows, const int64_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                                     int32_t* __restrict__ last) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x)
        last[r] = inc[inc_ptr[r + 1] - 1] >> 5;
}

// per element task: the largest gather sequence index among the tasks that read its elements' rows
__global__ void etask_gmax_kernel(int64_t nt, int n, const int32_t* __restrict__ l2n, const int32_t* __restrict__ gseq,
                                  int rg, int32_t* __restrict__ out) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nt; e += (int64_t)gridDim.x * blockDim.x) {
        int m = 0;
        for (int j = 0; j < n; ++j) m = max(m, gseq[l2n[e * n + j] / rg]);
        atomicMax(out + e / kEC, m);
    }
}

template <int MODE, int N>
size_t stream_smem_bytes(int maxrow) {
    constexpr int NTRI = N * (N + 1) / 2;
    const size_t f = (size_t)((14 * NTRI + 3) & ~3) + (size_t)kEC * 16;
    return f * 4 + ((N * N + 7) & ~7) * 2 + (size_t)kWarps * (32 / N) * maxrow * (MODE == kModeDF64 ? 8 : 4);
}

}  // namespace

// Per-space schedule of the streamed assembly (built once, on first use).
struct StreamPlan {
    int rg = 0, ne = 0, ng = 0;
    int64_t ring = 0;                 // ring slots (elements), a power of two
    int64_t ntickets = 0;
    int32_t* d_ticket = nullptr;
    int32_t* d_e_need_g = nullptr;
    int32_t* d_g_need_e = nullptr;
    int32_t* d_g_rows = nullptr;
    uint32_t* d_ctl = nullptr;
    size_t ctl_bytes = 0;
    ~StreamPlan() {
        cudaFree(d_ticket);
        cudaFree(d_e_need_g);
        cudaFree(d_g_need_e);
        cudaFree(d_g_rows);
        cudaFree(d_ctl);
    }
};

void stream_plan_free(StreamPlan* p) { delete p; }

int64_t stream_plan_ring(const StreamPlan* p) { return p ? p->ring : 0; }

static int build_stream_plan(fgpu_ctx* ctx, fgpu_space* V, StreamPlan*& out) {
    const DevPattern& P = *V->pattern;
    const int n = V->n;
    const int64_t nt = V->mesh->nt, nrows = P.nrows;
    const int rpw = 32 / n;
    auto plan = std::make_unique<StreamPlan>();
    plan->rg = kWarps * rpw * 4;
    const int64_t ne = (nt + kEC - 1) / kEC, ng = (nrows + plan->rg - 1) / plan->rg;
    if (ne >= (1 << 30) || ng >= (1 << 30)) { ctx->err = "streamed assembly: too many tasks"; return FGPU_ERR_INVALID; }
    plan->ne = (int)ne;
    plan->ng = (int)ng;
    int32_t *d_last = nullptr, *d_gseq = nullptr, *d_gmax = nullptr;
    auto cleanup = [&] { cudaFree(d_last); cudaFree(d_gseq); cudaFree(d_gmax); };
    cudaError_t e = cudaMalloc(&d_last, nrows * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&d_gseq, ng * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&d_gmax, ne * sizeof(int32_t));
    if (e != cudaSuccess) { cudaGetLastError(); cleanup(); ctx->err = "streamed assembly: plan allocation failed"; return FGPU_ERR_ALLOC; }
    row_last_elem_kernel<<<152 * 8, 256, 0, ctx->stream>>>(nrows, V->d_inc_ptr, V->d_inc, d_last);
    std::vector<int32_t> last(nrows);
    e = cudaMemcpyAsync(last.data(), d_last, nrows * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { cleanup(); ctx->err = std::string("streamed assembly plan: ") + cudaGetErrorString(e); return FGPU_ERR_CUDA; }
    // gather tasks sorted (stably) by the number of element tasks they need
    std::vector<int32_t> need_task(ng), order(ng), gseq(ng), need_seq(ng);
    for (int64_t j = 0; j < ng; ++j) {
        int32_t m = 0;
        const int64_t r1 = std::min<int64_t>(nrows, (j + 1) * plan->rg);
        for (int64_t r = j * plan->rg; r < r1; ++r) m = std::max(m, last[r]);
        need_task[j] = m / kEC + 1;
        order[j] = (int32_t)j;
    }
    std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) { return need_task[x] < need_task[y]; });
    for (int64_t s = 0; s < ng; ++s) {
        gseq[order[s]] = (int32_t)s;
        need_seq[s] = need_task[order[s]];
    }
    e = cudaMemcpyAsync(d_gseq, gseq.data(), ng * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_gmax, 0, ne * sizeof(int32_t), ctx->stream);
    if (e != cudaSuccess) { cleanup(); ctx->err = std::string("streamed assembly plan: ") + cudaGetErrorString(e); return FGPU_ERR_CUDA; }
    etask_gmax_kernel<<<152 * 8, 256, 0, ctx->stream>>>(nt, n, V->d_l2n, d_gseq, plan->rg, d_gmax);
    std::vector<int32_t> gmax(ne);
    e = cudaMemcpyAsync(gmax.data(), d_gmax, ne * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cleanup();
    if (e != cudaSuccess) { ctx->err = std::string("streamed assembly plan: ") + cudaGetErrorString(e); return FGPU_ERR_CUDA; }
    // smallest power-of-two ring such that every gather task an element task must wait for
    // is handed out before it (need_seq is non-decreasing, so the last one decides)
    int64_t ntp = kEC;
    while (ntp < nt) ntp *= 2;
    int64_t ring = 2 * kEC;
    std::vector<int32_t> e_need_g(ne, 0);
    for (;; ring *= 2) {
        std::fill(e_need_g.begin(), e_need_g.end(), 0);
        if (ring >= ntp) { ring = ntp; break; }
        const int64_t lag = ring / kEC;
        bool ok = true;
        for (int64_t k = lag; k < ne && ok; ++k) {
            const int32_t g = gmax[k - lag];            // gather tasks up to g read the slots E_k overwrites
            e_need_g[k] = g + 1;
            ok = need_seq[g] <= k;
        }
        if (ok) break;
    }
    plan->ring = ring;
    // tickets: E_0, gathers that need only E_0, E_1, gathers that need E_0..E_1, ...
    std::vector<int32_t> tickets;
    tickets.reserve(ne + ng);
    int64_t p = 0;
    for (int64_t k = 0; k < ne; ++k) {
        tickets.push_back((int32_t)k);
        while (p < ng && need_seq[p] <= k + 1) {
            tickets.push_back((int32_t)(-(p + 1)));
            ++p;
        }
    }
    std::vector<int32_t> g_rows(ng);
    for (int64_t s = 0; s < ng; ++s) g_rows[s] = (int32_t)((int64_t)order[s] * plan->rg);
    if (nrows >= ((int64_t)1 << 31)) { ctx->err = "streamed assembly: more than 2^31 rows"; return FGPU_ERR_INVALID; }
    plan->ntickets = (int64_t)tickets.size();
    plan->ctl_bytes = (4 + ne + ng) * sizeof(uint32_t);
    e = cudaMalloc(&plan->d_ticket, tickets.size() * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&plan->d_e_need_g, ne * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&plan->d_g_need_e, ng * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&plan->d_g_rows, ng * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&plan->d_ctl, plan->ctl_bytes);
    if (e != cudaSuccess) { cudaGetLastError(); ctx->err = "streamed assembly: plan allocation failed"; return FGPU_ERR_ALLOC; }
    e = cudaMemcpyAsync(plan->d_ticket, tickets.data(), tickets.size() * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(plan->d_e_need_g, e_need_g.data(), ne * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(plan->d_g_need_e, need_seq.data(), ng * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(plan->d_g_rows, g_rows.data(), ng * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { ctx->err = std::string("streamed assembly plan: ") + cudaGetErrorString(e); return FGPU_ERR_CUDA; }
    out = plan.release();
    return FGPU_OK;
}

template <int MODE, int N>
static int run_streamed(fgpu_ctx* ctx, fgpu_matrix* A, const DevTables* tab, const double* d_kappa, double kappa,
                        double mass, const double* kscale, int accumulate, double* hout) {
    fgpu_space* V = A->space;
    constexpr int NTRI = N * (N + 1) / 2;
    if (!V->stream_plan) {
        if (ctx->capturing) { ctx->err = "streamed assembly: assemble once before capturing (schedule)"; return FGPU_ERR_INVALID; }
        int rc = build_stream_plan(ctx, V, V->stream_plan);
        if (rc) return rc;
    }
    const StreamPlan& plan = *V->stream_plan;
    const size_t need = (size_t)plan.ring * NTRI * (MODE == kModeDF64 ? 8 : 4);
    if (A->kbuf_bytes < need) {
        if (ctx->capturing) { ctx->err = "streamed assembly: assemble once before capturing (element ring)"; return FGPU_ERR_INVALID; }
        cudaFree(A->d_kbuf);
        A->d_kbuf = nullptr;
        A->kbuf_bytes = 0;
        if (cudaMalloc(&A->d_kbuf, need) != cudaSuccess) { cudaGetLastError(); ctx->err = "streamed assembly: element ring allocation failed"; return FGPU_ERR_ALLOC; }
        A->kbuf_bytes = need;
    }
    const int maxrow = A->pattern->max_row;
    const size_t smem = stream_smem_bytes<MODE, N>(maxrow);
    auto kern = stream_assemble_kernel<MODE, N>;
    if (smem > 227 * 1024) { ctx->err = "streamed assembly: pattern rows too long"; return FGPU_ERR_INVALID; }
    FGPU_CUDA_CHECK(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0, sms = 0;
    FGPU_CUDA_CHECK(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem));
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((int64_t)std::max(per_sm, 1) * sms, plan.ntickets));
    StreamArgs args{};
    args.nt = V->mesh->nt;
    args.nrows = A->pattern->nrows;
    args.ntickets = plan.ntickets;
    args.xyz = V->mesh->d_xyz;
    args.tets = V->mesh->d_tets;
    args.kappa = d_kappa;
    args.kappa_c = kappa;
    args.mass = mass;
    args.kscale = kscale;
    args.ia = A->pattern->d_ia;
    args.inc_ptr = V->d_inc_ptr;
    args.inc = V->d_inc;
    args.pos = V->d_pos;
    args.Th = tab->d_T7th;                  // binary32 matrices use the high parts (fl32 of the tensors)
    args.Tl = tab->d_T7tl;
    args.tri = tab->d_tri;
    args.ring = A->d_kbuf;
    args.ring_mask = plan.ring - 1;
    args.val = A->d_val;
    args.hout = hout;
    args.accumulate = accumulate;
    args.ticket = plan.d_ticket;
    args.e_need_g = plan.d_e_need_g;
    args.g_need_e = plan.d_g_need_e;
    args.g_rows = plan.d_g_rows;
    args.ctl = plan.d_ctl;
    args.ne = plan.ne;
    args.ng = plan.ng;
    args.rg = plan.rg;
    args.maxrow = maxrow;
    args.status = ctx->d_status;
    FGPU_CUDA_CHECK(ctx, cudaMemsetAsync(plan.d_ctl, 0, plan.ctl_bytes, ctx->stream));
    PendingEvent ev;
    prof_begin(ctx, "assemble_streamed", ev);
    kern<<<(int)blocks, kThreads, smem, ctx->stream>>>(args);
    prof_end(ctx, ev);
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    return FGPU_OK;
}

// Streamed assembly of kappa*inner(gradt(u),grad(v)) + mass*idt(u)*id(v) on affine tetrahedra
// (scalar P1-P3): FP64 matrices in df64 arithmetic, FP32 matrices in binary32; hout (FP64
// only): a device-mapped page-locked host buffer that receives a copy of every value.
int launch_assemble_streamed(fgpu_ctx* ctx, fgpu_matrix* A, const DevTables* tab, const double* d_kappa, double kappa,
                             double mass, const double* kscale, int accumulate, double* hout) {
    fgpu_space* V = A->space;
    if (A->ncomp != 1 || V->mesh->cv != 4 || V->mesh->d_ho) { ctx->err = "streamed assembly: scalar spaces on affine tetrahedra"; return FGPU_ERR_INVALID; }
    if (!V->d_pos) { ctx->err = "streamed assembly: no position table (pattern rows longer than 256)"; return FGPU_ERR_INVALID; }
    if (hout && A->precision != FGPU_F64) { ctx->err = "streamed assembly: host copies of FP64 matrices only"; return FGPU_ERR_INVALID; }
    const bool f32 = A->precision == FGPU_F32;
    switch (V->order) {
        case 1: return f32 ? run_streamed<kModeF32, 4>(ctx, A, tab, d_kappa, kappa, mass, kscale, accumulate, hout)
                           : run_streamed<kModeDF64, 4>(ctx, A, tab, d_kappa, kappa, mass, kscale, accumulate, hout);
        case 2: return f32 ? run_streamed<kModeF32, 10>(ctx, A, tab, d_kappa, kappa, mass, kscale, accumulate, hout)
                           : run_streamed<kModeDF64, 10>(ctx, A, tab, d_kappa, kappa, mass, kscale, accumulate, hout);
        case 3: return f32 ? run_streamed<kModeF32, 20>(ctx, A, tab, d_kappa, kappa, mass, kscale, accumulate, hout)
                           : run_streamed<kModeDF64, 20>(ctx, A, tab, d_kappa, kappa, mass, kscale, accumulate, hout);
        default: ctx->err = "unsupported order"; return FGPU_ERR_INVALID;
    }
}

}  // namespace fgpu
