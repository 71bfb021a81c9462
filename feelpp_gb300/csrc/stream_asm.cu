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
#include <type_traits>
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
constexpr long long kMaxSpins = 1LL << 24;   // x ~100 ns sleeps (plus a flag scan): a wait gives up after a few seconds
constexpr int kMaxRowsPerTask = 256;

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
    const int32_t* g_rows;                // per gather task: first row
    const int32_t* g_cnt;                 // per gather task: number of rows
    const uint8_t* g_order;               // per row: the task-local row processed in its place
    uint32_t* ctl;
    int ne, ng, maxrow;
    int* status;
};

// asynchronous global -> shared copies (completed by cp_async_wait_all)
__device__ __forceinline__ void cp_async(void* dst, const void* src, int bytes) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    if (bytes == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;" ::: "memory");
}

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// A finished task publishes its done flag (after the block's barrier, so every thread's
// writes are ordered before it).
__device__ __forceinline__ void finish_task(uint32_t* done, uint32_t k) {
    __threadfence();
    st_release(done + k, 1u);
}

// Watermarks: mark <= number of leading tasks (in task index order) that are done. One warp
// waits until mark >= need, moving the shared mark over the done flags 32 at a time (a
// ballot finds the leading run of set flags), so waiters share the scan. Returns false when
// the launch was aborted or the wait gave up (the abort flag and a status bit are then set).
__device__ __forceinline__ bool wait_mark(uint32_t* mark, const uint32_t* done, uint32_t need, uint32_t* abort, int* status,
                                          int lane) {
    uint32_t w = __shfl_sync(0xffffffffu, ld_acquire(mark), 0);   // one value for the whole warp
    long long spins = 0;
    while (w < need) {
        const uint32_t idx = w + lane;
        const bool f = idx >= need || ld_relaxed(done + idx) != 0u;
        const unsigned b = __ballot_sync(0xffffffffu, f);
        const uint32_t run = b == 0xffffffffu ? 32u : (uint32_t)(__ffs(~b) - 1);
        if (run > 0) {
            w = min(w + run, need);
            __threadfence();
            if (lane == 0) atomicMax(mark, w);
            if (w >= need) break;
        }
        if (run < 32) {
            if (__shfl_sync(0xffffffffu, ld_acquire(abort), 0)) return false;
            if (++spins > kMaxSpins) {
                if (lane == 0) {
                    atomicExch(abort, 1u);
                    atomicOr(status, kStatusStreamTimeout);
                }
                return false;
            }
            __nanosleep(100);
            const uint32_t m = __shfl_sync(0xffffffffu, ld_acquire(mark), 0);
            if (m > w) w = m;
        }
    }
    __threadfence();
    return true;
}

// One contribution into a row accumulator, as the two-phase gather sums it: df64 entries
// keep the TwoSum of the high parts and one binary32 sum of the low parts and errors.
__device__ __forceinline__ void accumulate_entry(float* acc, int p, float2 v) {
    const df tw = two_sum(acc[2 * p], v.x);
    acc[2 * p] = tw.hi;
    acc[2 * p + 1] = f_add(acc[2 * p + 1], f_add(tw.lo, v.y));
}
__device__ __forceinline__ void accumulate_entry(float* acc, int p, float v) { acc[p] = f_add(acc[p], v); }

// Shared-memory layout of the kernel (floats unless noted): the reference tensors (hi, lo),
// the n x n triangle-index table (u16), the row accumulators of the gather tasks, then one
// region used by an element task for its coefficient records and by a gather task for its
// staged contributions (values, incidence codes, positions).
template <int MODE, int N>
struct StreamSmem {
    static constexpr int NTRI = N * (N + 1) / 2;
    static constexpr int RPW = 32 / N;                                  // gather rows per warp pass
    static constexpr int VB = MODE == kModeDF64 ? 8 : 4;                // bytes of a staged value
    static constexpr int PW = (N + 3 + 3) / 4;                          // 4-byte words covering an element row of positions
    static constexpr int PER_INC = 4 + N * VB + 4 * PW;                 // staged bytes per incidence
    static constexpr int CAP = (49152 / PER_INC) & ~31;                 // incidences staged per gather task
    static constexpr size_t tab_bytes = (size_t)((14 * NTRI + 3) & ~3) * 4;
    static constexpr size_t tri_bytes = (size_t)((N * N + 7) & ~7) * 2;
    __host__ __device__ static size_t acc_bytes(int maxrow) { return ((size_t)kWarps * RPW * maxrow * VB + 15) & ~(size_t)15; }
    static constexpr size_t region_bytes() {
        return (size_t)kEC * 64 > (size_t)CAP * PER_INC ? (size_t)kEC * 64 : (size_t)CAP * PER_INC;
    }
    static size_t bytes(int maxrow) { return tab_bytes + tri_bytes + acc_bytes(maxrow) + region_bytes(); }
};

template <int MODE, int N>
__global__ void __launch_bounds__(kThreads, 3) stream_assemble_kernel(StreamArgs a) {
    using SM = StreamSmem<MODE, N>;
    constexpr int NTRI = SM::NTRI;
    constexpr int EPW = NTRI >= 32 ? 1 : 32 / NTRI;         // elements per warp pass (element tasks)
    constexpr int RPW = SM::RPW;
    constexpr int ACCW = MODE == kModeDF64 ? 2 : 1;
    constexpr int CAP = SM::CAP;
    using VT = typename std::conditional<MODE == kModeDF64, float2, float>::type;
    extern __shared__ __align__(16) unsigned char smem[];
    float* Th = reinterpret_cast<float*>(smem);
    float* Tl = Th + 7 * NTRI;
    uint16_t* tri = reinterpret_cast<uint16_t*>(smem + SM::tab_bytes);
    float* accb = reinterpret_cast<float*>(smem + SM::tab_bytes + SM::tri_bytes);
    unsigned char* region = smem + SM::tab_bytes + SM::tri_bytes + SM::acc_bytes(a.maxrow);
    float* rec = reinterpret_cast<float*>(region);                       // element task: kEC x 16
    constexpr int PW = SM::PW;
    VT* s_val = reinterpret_cast<VT*>(region);                           // gather task: CAP x N values
    uint32_t* s_posw = reinterpret_cast<uint32_t*>(region + (size_t)CAP * N * sizeof(VT));   // CAP x PW words
    int32_t* s_code = reinterpret_cast<int32_t*>(s_posw + CAP * PW);
    const uint8_t* s_posb = reinterpret_cast<const uint8_t*>(s_posw);
    const uint32_t* posw = reinterpret_cast<const uint32_t*>(a.pos);
    __shared__ int s_ticket, s_ok;
    __shared__ int64_t s_incp[kMaxRowsPerTask + 1], s_ia[kMaxRowsPerTask + 1];
    __shared__ uint8_t s_order[kMaxRowsPerTask];

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
    const int sub = lane / N, jc = lane - sub * N;          // gather: row slot of the lane, element column
    const unsigned submask = sub < RPW ? (((1u << N) - 1u) << (sub * N)) : 0u;
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
            if (warp == 0) {
                const bool ok = a.e_need_g[code] > 0
                                    ? wait_mark(a.ctl + 2, g_done, (uint32_t)a.e_need_g[code], abort, a.status, lane)
                                    : !ld_acquire(abort);
                if (lane == 0) s_ok = ok;
            }
            if (tid < cnt)
                geometry_df_record(e0 + tid, a.xyz, a.tets, a.kappa, kc, mc, ksc, reinterpret_cast<float4*>(rec + 16 * tid),
                                   a.status);
            __syncthreads();
            if (!s_ok) break;
            const int esub = lane / NTRI < EPW ? lane / NTRI : EPW;
            const int t0 = EPW > 1 ? lane - esub * NTRI : lane;
            const int64_t slot0 = e0 & a.ring_mask;
            for (int le = warp * EPW + esub; esub < EPW && le < cnt; le += kWarps * EPW) {
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
            if (tid == 0) finish_task(e_done, (uint32_t)code);
        } else {
            // ---- gather task: rows r0 .. r0 + nr - 1, each summed in element order
            const int s = -code - 1;
            const int64_t r0 = a.g_rows[s];
            const int nr = a.g_cnt[s];
            if (warp == 0) {
                const bool ok = wait_mark(a.ctl + 1, e_done, (uint32_t)a.g_need_e[s], abort, a.status, lane);
                if (lane == 0) s_ok = ok;
            }
            for (int k = tid; k <= nr; k += kThreads) {     // row bounds of the task, one coalesced load
                s_incp[k] = __ldcs(a.inc_ptr + r0 + k);
                s_ia[k] = __ldcs(a.ia + r0 + k);
                if (k < nr) s_order[k] = a.g_order[r0 + k];
            }
            __syncthreads();
            if (!s_ok) break;
            // stage the incidence codes of all rows (one contiguous range), then every
            // (incidence, column) pair's offset in its row and element-matrix entry
            const int64_t c0 = s_incp[0];
            const int ninc = (int)(s_incp[nr] - c0);        // <= CAP (the schedule sizes the tasks)
            for (int k = tid; k < ninc; k += kThreads) s_code[k] = __ldcs(a.inc + c0 + k);
            __syncthreads();
            // asynchronous copies into shared memory: each (incidence, column) pair's element-matrix
            // entry from the ring, and each incidence's row of the position table as aligned words
            const int nq = ninc * N;
            for (int q = tid; q < nq; q += kThreads) {
                const int idx = q / N, j = q - idx * N;
                const int32_t cd = s_code[idx];
                const int64_t e = cd >> 5;
                const int li = cd & 31;
                cp_async(s_val + q, reinterpret_cast<const VT*>(a.ring) + (e & a.ring_mask) * NTRI + tri[li * N + j], (int)sizeof(VT));
            }
            for (int q = tid; q < ninc * PW; q += kThreads) {
                const int idx = q / PW, w = q - idx * PW;
                const int32_t cd = s_code[idx];
                const int64_t base = ((int64_t)(cd >> 5) * N + (cd & 31)) * N;
                cp_async(s_posw + q, posw + (base >> 2) + w, 4);
            }
            cp_async_wait_all();
            __syncthreads();
            // rows: N lanes per row (one element column each), RPW rows per warp pass
            float* myacc = acc + (size_t)(sub < RPW ? sub : 0) * a.maxrow * ACCW;
            // rows are taken longest first (the schedule's order within the task), so that the
            // rows of one warp pass have similar numbers of incident elements
            for (int lb = warp * RPW; lb < nr; lb += kWarps * RPW) {
                if (sub < RPW && lb + sub < nr) {
                    const int lr = s_order[lb + sub];
                    const int ib = (int)(s_incp[lr] - c0), ie = (int)(s_incp[lr + 1] - c0);
                    // the next incidence's position and value are read while this one is added
                    // ((e N + li) N = li N mod 4, since N is even: the byte offset in the staged words)
                    int pn = 0;
                    VT vn{};
                    if (ib < ie) {
                        pn = s_posb[ib * PW * 4 + ((s_code[ib] & 31) * N & 3) + jc];
                        vn = s_val[ib * N + jc];
                    }
                    for (int idx = ib; idx < ie; ++idx) {
                        const int pc = pn;
                        const VT vc = vn;
                        if (idx + 1 < ie) {
                            pn = s_posb[(idx + 1) * PW * 4 + ((s_code[idx + 1] & 31) * N & 3) + jc];
                            vn = s_val[(idx + 1) * N + jc];
                        }
                        accumulate_entry(myacc, pc, vc);
                        __syncwarp(submask);
                    }
                    const int64_t start = s_ia[lr];
                    const int len = (int)(s_ia[lr + 1] - start);
                    for (int k = jc; k < len; k += N) {
                        if (MODE == kModeDF64) {
                            df sv = two_sum(myacc[2 * k], myacc[2 * k + 1]);
                            myacc[2 * k] = 0.0f;
                            myacc[2 * k + 1] = 0.0f;
                            double* out = reinterpret_cast<double*>(a.val) + start + k;
                            if (a.accumulate) sv = df_add(d2df(*out), sv);
                            const double rv = df2d(sv);
                            __stcs(out, rv);
                            if (a.hout) a.hout[start + k] = rv;
                        } else {
                            const float sv = myacc[k];
                            myacc[k] = -0.0f;
                            float* out = reinterpret_cast<float*>(a.val) + start + k;
                            __stcs(out, a.accumulate ? f_add(*out, sv) : sv);
                        }
                    }
                    __syncwarp(submask);
                }
            }
            __syncthreads();
            if (tid == 0) finish_task(g_done, (uint32_t)s);
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
__global__ void etask_gmax_kernel(int64_t nt, int n, const int32_t* __restrict__ l2n, const int32_t* __restrict__ gseq_of_row,
                                  int32_t* __restrict__ out) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nt; e += (int64_t)gridDim.x * blockDim.x) {
        int m = 0;
        for (int j = 0; j < n; ++j) m = max(m, gseq_of_row[l2n[e * n + j]]);
        atomicMax(out + e / kEC, m);
    }
}

}  // namespace

// Per-space schedule of the streamed assembly (built once, on first use).
struct StreamPlan {
    int ne = 0, ng = 0, delay = 0, ctas = 0, cap = 0;
    bool unsupported = false;         // an incidence list longer than a gather task can stage
    int64_t ring = 0;                 // ring slots (elements), a power of two
    int64_t ntickets = 0;
    int32_t* d_ticket = nullptr;
    int32_t* d_e_need_g = nullptr;
    int32_t* d_g_need_e = nullptr;
    int32_t* d_g_rows = nullptr;
    int32_t* d_g_cnt = nullptr;
    uint8_t* d_g_order = nullptr;     // per row: task-local rows by decreasing incidence count
    uint32_t* d_ctl = nullptr;
    size_t ctl_bytes = 0;
    ~StreamPlan() {
        cudaFree(d_ticket);
        cudaFree(d_e_need_g);
        cudaFree(d_g_need_e);
        cudaFree(d_g_rows);
        cudaFree(d_g_cnt);
        cudaFree(d_g_order);
        cudaFree(d_ctl);
    }
};

void stream_plan_free(StreamPlan* p) { delete p; }

int64_t stream_plan_ring(const StreamPlan* p) { return p ? p->ring : 0; }

// cap: incidences a gather task can stage; ctas: blocks of the persistent launch.
static int build_stream_plan(fgpu_ctx* ctx, fgpu_space* V, int cap, int ctas, StreamPlan*& out) {
    const DevPattern& P = *V->pattern;
    const int n = V->n;
    const int64_t nt = V->mesh->nt, nrows = P.nrows;
    auto plan = std::make_unique<StreamPlan>();
    plan->cap = cap;
    plan->ctas = ctas;
    if (nrows >= ((int64_t)1 << 31)) { ctx->err = "streamed assembly: more than 2^31 rows"; return FGPU_ERR_INVALID; }
    const int64_t ne = (nt + kEC - 1) / kEC;
    int32_t *d_last = nullptr, *d_gseq = nullptr, *d_gmax = nullptr;
    auto cleanup = [&] { cudaFree(d_last); cudaFree(d_gseq); cudaFree(d_gmax); };
    cudaError_t e = cudaMalloc(&d_last, nrows * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&d_gseq, nrows * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&d_gmax, ne * sizeof(int32_t));
    if (e != cudaSuccess) { cudaGetLastError(); cleanup(); ctx->err = "streamed assembly: plan allocation failed"; return FGPU_ERR_ALLOC; }
    row_last_elem_kernel<<<152 * 8, 256, 0, ctx->stream>>>(nrows, V->d_inc_ptr, V->d_inc, d_last);
    std::vector<int32_t> last(nrows);
    std::vector<int64_t> incp(nrows + 1);
    e = cudaMemcpyAsync(last.data(), d_last, nrows * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(incp.data(), V->d_inc_ptr, (nrows + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { cleanup(); ctx->err = std::string("streamed assembly plan: ") + cudaGetErrorString(e); return FGPU_ERR_CUDA; }
    // gather tasks: runs of consecutive rows holding at most `cap` incidences and kMaxRowsPerTask rows
    std::vector<int32_t> g_start, g_cnt, need_task;
    for (int64_t r = 0; r < nrows;) {
        if (incp[r + 1] - incp[r] > cap) { cleanup(); plan->unsupported = true; out = plan.release(); return FGPU_OK; }
        int64_t r1 = r;
        int32_t m = 0;
        while (r1 < nrows && r1 - r < kMaxRowsPerTask && incp[r1 + 1] - incp[r] <= cap) m = std::max(m, last[r1++]);
        g_start.push_back((int32_t)r);
        g_cnt.push_back((int32_t)(r1 - r));
        need_task.push_back(m / kEC + 1);
        r = r1;
    }
    const int64_t ng = (int64_t)g_start.size();
    if (ng >= (1 << 30)) { cleanup(); ctx->err = "streamed assembly: too many tasks"; return FGPU_ERR_INVALID; }
    plan->ne = (int)ne;
    plan->ng = (int)ng;
    // gather tasks sorted (stably) by the number of element tasks they need
    std::vector<int32_t> order(ng), need_seq(ng), gseq_of_row(nrows);
    for (int64_t j = 0; j < ng; ++j) order[j] = (int32_t)j;
    std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) { return need_task[x] < need_task[y]; });
    std::vector<int32_t> rows_seq(ng), cnt_seq(ng);
    for (int64_t sq = 0; sq < ng; ++sq) {
        const int32_t j = order[sq];
        need_seq[sq] = need_task[j];
        rows_seq[sq] = g_start[j];
        cnt_seq[sq] = g_cnt[j];
        for (int32_t r = g_start[j]; r < g_start[j] + g_cnt[j]; ++r) gseq_of_row[r] = (int32_t)sq;
    }
    e = cudaMemcpyAsync(d_gseq, gseq_of_row.data(), nrows * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_gmax, 0, ne * sizeof(int32_t), ctx->stream);
    if (e != cudaSuccess) { cleanup(); ctx->err = std::string("streamed assembly plan: ") + cudaGetErrorString(e); return FGPU_ERR_CUDA; }
    etask_gmax_kernel<<<152 * 8, 256, 0, ctx->stream>>>(nt, n, V->d_l2n, d_gseq, d_gmax);
    std::vector<int32_t> gmax(ne);
    e = cudaMemcpyAsync(gmax.data(), d_gmax, ne * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cleanup();
    if (e != cudaSuccess) { ctx->err = std::string("streamed assembly plan: ") + cudaGetErrorString(e); return FGPU_ERR_CUDA; }
    // Gather task s is handed out `delay` element tasks after the last element task it needs, and
    // an element task `delay` further than the gather tasks that read the slots it overwrites, so
    // that with `ctas` blocks taking tickets in order a task seldom finds its inputs unfinished.
    // The ring is the smallest power of two that keeps the second distance (need_seq is
    // non-decreasing, so the last gather task an element task waits for decides).
    const int64_t delay = std::max<int64_t>(1, (int64_t)ctas * ne / (ne + ng) + 1);
    auto placed = [&](int64_t g) { return std::min<int64_t>(need_seq[g] - 1 + delay, ne - 1); };
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
            ok = placed(g) + delay < k;
        }
        if (ok) break;
    }
    plan->ring = ring;
    plan->delay = (int)delay;
    // tickets: E_0, E_1, ..., each followed by the gather tasks placed after it
    std::vector<int32_t> tickets;
    tickets.reserve(ne + ng);
    int64_t p = 0;
    for (int64_t k = 0; k < ne; ++k) {
        tickets.push_back((int32_t)k);
        while (p < ng && placed(p) <= k) {
            tickets.push_back((int32_t)(-(p + 1)));
            ++p;
        }
    }
    // within each gather task, rows by decreasing number of incident elements (stable)
    std::vector<uint8_t> g_order(nrows);
    {
        std::vector<int32_t> loc;
        for (int64_t j = 0; j < ng; ++j) {
            const int32_t r0 = g_start[j], cnt = g_cnt[j];
            loc.resize(cnt);
            for (int32_t k = 0; k < cnt; ++k) loc[k] = k;
            std::stable_sort(loc.begin(), loc.end(), [&](int32_t x, int32_t y) {
                return incp[r0 + x + 1] - incp[r0 + x] > incp[r0 + y + 1] - incp[r0 + y];
            });
            for (int32_t k = 0; k < cnt; ++k) g_order[r0 + k] = (uint8_t)loc[k];
        }
    }
    plan->ntickets = (int64_t)tickets.size();
    plan->ctl_bytes = (4 + ne + ng) * sizeof(uint32_t);
    e = cudaMalloc(&plan->d_ticket, tickets.size() * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&plan->d_e_need_g, ne * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&plan->d_g_need_e, ng * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&plan->d_g_rows, ng * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&plan->d_g_cnt, ng * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&plan->d_g_order, nrows);
    if (e == cudaSuccess) e = cudaMalloc(&plan->d_ctl, plan->ctl_bytes);
    if (e != cudaSuccess) { cudaGetLastError(); ctx->err = "streamed assembly: plan allocation failed"; return FGPU_ERR_ALLOC; }
    e = cudaMemcpyAsync(plan->d_ticket, tickets.data(), tickets.size() * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(plan->d_e_need_g, e_need_g.data(), ne * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(plan->d_g_need_e, need_seq.data(), ng * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(plan->d_g_rows, rows_seq.data(), ng * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(plan->d_g_cnt, cnt_seq.data(), ng * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(plan->d_g_order, g_order.data(), nrows, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { ctx->err = std::string("streamed assembly plan: ") + cudaGetErrorString(e); return FGPU_ERR_CUDA; }
    out = plan.release();
    return FGPU_OK;
}

template <int MODE, int N>
static int run_streamed(fgpu_ctx* ctx, fgpu_matrix* A, const DevTables* tab, const double* d_kappa, double kappa,
                        double mass, const double* kscale, int accumulate, double* hout) {
    fgpu_space* V = A->space;
    using SM = StreamSmem<MODE, N>;
    constexpr int NTRI = SM::NTRI;
    const int maxrow = A->pattern->max_row;
    const size_t smem = SM::bytes(maxrow);
    auto kern = stream_assemble_kernel<MODE, N>;
    if (smem > 227 * 1024) { ctx->err = "streamed assembly: pattern rows too long"; return FGPU_ERR_INVALID; }
    FGPU_CUDA_CHECK(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0, sms = 0;
    FGPU_CUDA_CHECK(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem));
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int ctas = std::max(per_sm, 1) * sms;
    if (!V->stream_plan || V->stream_plan->ctas != ctas || V->stream_plan->cap != SM::CAP) {
        if (ctx->capturing) { ctx->err = "streamed assembly: assemble once before capturing (schedule)"; return FGPU_ERR_INVALID; }
        stream_plan_free(V->stream_plan);
        V->stream_plan = nullptr;
        int rc = build_stream_plan(ctx, V, SM::CAP, ctas, V->stream_plan);
        if (rc) return rc;
    }
    if (V->stream_plan->unsupported) return kStreamedUnsupported;
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
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(ctas, plan.ntickets));
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
    args.g_cnt = plan.d_g_cnt;
    args.g_order = plan.d_g_order;
    args.ctl = plan.d_ctl;
    args.ne = plan.ne;
    args.ng = plan.ng;
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
// Returns kStreamedUnsupported (nothing launched) when a dof belongs to more elements than a
// gather task can stage; the two-phase assembly gives the same values.
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
