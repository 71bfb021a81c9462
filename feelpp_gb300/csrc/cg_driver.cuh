// Preconditioned conjugate gradients driver shared by the assembled (CSR)
// solver (solve.cu) and the matrix-free solver (matfree.cu).
//
// The method is KSPCG with PCJACOBI of the PETSc backend the reference solves
// with (feelpp/feel/feelalg/solverlinearpetsc.cpp:490-570, ksp-type=cg,
// pc-type=jacobi), stopped on the unpreconditioned residual
// ||r|| <= rtol ||b||. Additions:
//   * Chebyshev-Jacobi: the preconditioner is the degree-K Chebyshev
//     polynomial in D^-1 A over [lmin, lmax] applied to D^-1 r (K - 1 extra
//     operator applications per iteration). lmax comes from a short Lanczos
//     run (Jacobi-CG coefficients on b), lmax_used = 1.1 lmax_est as in
//     PETSc's Chebyshev eigenvalue transform (-ksp_chebyshev_esteig 0,0.1,0,1.1
//     gives the emax factor), lmin = ratio * lmax_used.
//   * check_every iterations run from one captured CUDA graph; the host polls
//     the device scalars between replays (every kernel returns at once once
//     the device stop flag is set).
//   * reliable updates for the mixed-precision solve (see RefreshFn).
#pragma once
#include <algorithm>
#include <cmath>
#include <functional>
#include <string>
#include <vector>

#include "cg_kernels.cuh"

namespace fgpu {

template <class PL>
struct CgOperator {
    // y = A x. When `partial` is set, per-block partial sums of x.y go to
    // partial[0, npq). Every kernel returns at once when sc && sc->done.
    std::function<void(const typename PL::S* x, typename PL::S* y, typename PL::D* partial, const CGScalars<PL>* sc)> apply;
    int npq = 0;              // blocks writing x.y partials
    int launches = 1;         // kernels per application (launch accounting)
    bool graph = true;        // the iterations may be captured into a CUDA graph
};

struct CgOptions {
    double rtol = 1e-10;
    int maxit = 1000;
    int check_every = 16;
    int cheb_degree = 0;      // < 2: Jacobi; K >= 2: Chebyshev-Jacobi of degree K
    double cheb_ratio = 0.03; // lmin / lmax of the Chebyshev interval
    int est_iters = 16;       // Lanczos steps of the lmax estimate
    double delta = 0.1;       // reliable updates: recurrence reduction between replacements
};

struct CgResult {
    int iters = 0, fail = 0, nrefresh = 0;
    bool true_conv = false;
    double rr = 0, bb = 0, lmax = 0, lmin = 0;
};

// Reliable updates (mixed precision): at a poll point where the recurrence
// residual has dropped by delta since the last update, or claims convergence,
// the callback folds x into the binary64 solution, zeroes x and replaces r by
// the binary64 residual (scaled like the binary32 system); the search
// direction is kept, except after a converged recurrence (its last iteration
// left p without the beta update), where p restarts from the new z.
// The callback returns FGPU_OK, an FGPU_ERR_* code, or kRefreshStagnated when
// the binary64 residual stopped decreasing (the binary32 system is too far
// from the binary64 one at this conditioning): the run then ends with fail = 3.
template <class PL>
using RefreshFn = std::function<int(typename PL::S* x, typename PL::S* r, bool* converged)>;
static constexpr int kRefreshStagnated = 1000;

// An external preconditioner (AMG V-cycle): z = M r, per-block partial sums of
// r.z into rz_partial (vec_blocks(n) blocks of kVecThreads, the layout the CG
// kernels read) and, when p_out is set, p = z. Every kernel returns at once
// when gate && gate->done. `launches` = kernels per application.
template <class PL>
struct PcHook {
    std::function<void(const typename PL::S* r, typename PL::S* z, typename PL::D* rz_partial, typename PL::S* p_out,
                       const CGScalars<PL>* gate)>
        apply;
    int launches = 0;
};

// dst = scale * src
template <class PL>
__global__ void scale_vec_kernel(int64_t n, const typename PL::S* __restrict__ src, typename PL::S* __restrict__ dst,
                                 typename PL::D scale) {
    const typename PL::A a = PL::from_d(scale);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = PL::st(PL::mul(a, PL::ld(src[i])));
}

// One step k >= 1 of the Chebyshev iteration for A z = r from z = 0 with the
// Jacobi diagonal (three-term form, Saad, Iterative Methods for Sparse Linear
// Systems, 2nd ed., Algorithm 12.1):
//   w_k = w_{k-1} - A d_{k-1}            (w_0 = r)
//   d_k = c1_k d_{k-1} + c2_k D^-1 w_k   (d_0 = D^-1 r / theta = z_1)
//   z_{k+1} = z_k + d_k
// q holds A d_{k-1}. The first step reads w_0 = r and d_0 = z. The last step
// writes per-block partial sums of r.z to partial_rz and, when p_out is set,
// p = z.
template <class PL>
__global__ void cheb_step_kernel(int64_t n, const typename PL::S* __restrict__ r, typename PL::S* __restrict__ w,
                                 typename PL::S* __restrict__ d, typename PL::S* __restrict__ z,
                                 const typename PL::S* __restrict__ dinv, const typename PL::S* __restrict__ q,
                                 typename PL::D c1, typename PL::D c2, int first, int last,
                                 typename PL::D* __restrict__ partial_rz, typename PL::S* __restrict__ p_out,
                                 const CGScalars<PL>* __restrict__ sc) {
    if (sc && sc->done) return;
    __shared__ typename PL::D sh[32];
    const typename PL::A a1 = PL::from_d(c1), a2 = PL::from_d(c2);
    typename PL::D rz = PL::dzero();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const typename PL::A wi = PL::sub(PL::ld(first ? r[i] : w[i]), PL::ld(q[i]));
        if (!last) w[i] = PL::st(wi);
        const typename PL::A zi0 = PL::ld(z[i]);
        const typename PL::A dprev = first ? zi0 : PL::ld(d[i]);
        const typename PL::A dn = PL::madd(PL::mul(a1, dprev), a2, PL::mul(PL::ld(dinv[i]), wi));
        if (!last) d[i] = PL::st(dn);
        const typename PL::S zs = PL::st(PL::add(zi0, dn));
        z[i] = zs;
        if (last) {
            if (p_out) p_out[i] = zs;
            rz = PL::dmadd(rz, PL::ld(r[i]), PL::ld(zs));
        }
    }
    if (last) {
        const typename PL::D t = block_sum<PL>(rz, sh);
        if (threadIdx.x == 0) partial_rz[blockIdx.x] = t;
    }
}

// Largest eigenvalue of the symmetric tridiagonal matrix (diag, off) by Sturm
// bisection.
static inline double tridiag_max_eig(const std::vector<double>& dg, const std::vector<double>& off) {
    const int m = (int)dg.size();
    if (m == 0) return 0.0;
    double hi = 0.0;
    for (int j = 0; j < m; ++j) {
        double g = std::fabs(dg[j]);
        if (j > 0) g += std::fabs(off[j - 1]);
        if (j + 1 < m) g += std::fabs(off[j]);
        hi = std::max(hi, g);
    }
    auto below = [&](double x) {   // number of eigenvalues < x
        int c = 0;
        double qv = 1.0;
        for (int j = 0; j < m; ++j) {
            const double o2 = j > 0 ? off[j - 1] * off[j - 1] : 0.0;
            qv = dg[j] - x - (j > 0 ? o2 / qv : 0.0);
            if (qv == 0.0) qv = -1e-300;
            if (qv < 0) ++c;
        }
        return c;
    };
    double lo = 0.0;
    for (int it = 0; it < 200 && hi - lo > 1e-12 * hi; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (below(mid) == m) hi = mid;
        else lo = mid;
    }
    return hi;
}

static inline CgOptions cg_options(const fgpu_solver_cfg* cfg) {
    CgOptions o;
    o.rtol = cfg->rtol;
    o.maxit = cfg->maxit;
    o.check_every = cfg->check_every > 0 ? cfg->check_every : 16;
    o.cheb_degree = cfg->pc == FGPU_PC_CHEB_JACOBI ? (cfg->cheb_degree > 0 ? cfg->cheb_degree : 3) : 0;
    o.cheb_ratio = cfg->cheb_ratio > 0 ? cfg->cheb_ratio : 0.03;
    o.delta = cfg->inner_rtol > 0 ? cfg->inner_rtol : 0.1;
    return o;
}

template <class PL>
static int cg_run(fgpu_ctx* ctx, int64_t n, const CgOperator<PL>& A, const typename PL::S* dinv,
                  const typename PL::S* b, typename PL::S* x, const CgOptions& o, CgResult* res,
                  const RefreshFn<PL>* refresh = nullptr, const PcHook<PL>* pch = nullptr) {
    typedef typename PL::S S;
    typedef typename PL::D D;
    cudaStream_t s = ctx->stream;
    const int vb = vec_blocks(n);
    const int nbp = std::max(A.npq, vb);
    const bool cheb = !pch && o.cheb_degree >= 2;
    const int K = cheb ? o.cheb_degree : 0;
    int check_every = std::max(o.check_every, 1);
    if (check_every & 1) ++check_every;   // parity of the scalar double buffer repeats per replay
    S *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *d = nullptr, *w = nullptr, *dinv0 = nullptr, *xe = nullptr;
    D *partial = nullptr, *pq_partial = nullptr;
    CGScalars<PL>* sc = nullptr;
    CGScalars<PL>* hsc = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    auto cleanup = [&]() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        cudaFree(r); cudaFree(z); cudaFree(p); cudaFree(q); cudaFree(d); cudaFree(w); cudaFree(dinv0); cudaFree(xe);
        cudaFree(partial); cudaFree(pq_partial); cudaFree(sc);
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
    CK(cudaMalloc(&r, n * sizeof(S)));
    CK(cudaMalloc(&z, n * sizeof(S)));
    CK(cudaMalloc(&p, n * sizeof(S)));
    CK(cudaMalloc(&q, n * sizeof(S)));
    CK(cudaMalloc(&partial, 3 * nbp * sizeof(D)));
    CK(cudaMalloc(&pq_partial, nbp * sizeof(D)));
    CK(cudaMalloc(&sc, sizeof(CGScalars<PL>)));
    CK(cudaMallocHost(&hsc, sizeof(CGScalars<PL>)));
    auto poll = [&]() -> cudaError_t {
        cudaError_t e = cudaMemcpyAsync(hsc, sc, sizeof(CGScalars<PL>), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        return e;
    };
    std::vector<D> c1, c2;
    const S* dz = dinv;                   // diagonal the update kernels apply (D^-1, or D^-1 / theta)
    if (cheb) {
        CK(cudaMalloc(&d, n * sizeof(S)));
        CK(cudaMalloc(&w, n * sizeof(S)));
        CK(cudaMalloc(&dinv0, n * sizeof(S)));
        CK(cudaMalloc(&xe, n * sizeof(S)));
        // lmax(D^-1 A): Lanczos tridiagonal from the coefficients of a short
        // Jacobi-CG run on b from x = 0 (in scratch vectors)
        CK(cudaMemsetAsync(xe, 0, n * sizeof(S), s));
        CK(cudaMemcpyAsync(r, b, n * sizeof(S), cudaMemcpyDeviceToDevice, s));
        cg_init_kernel<PL><<<vb, kVecThreads, 0, s>>>(n, b, r, dinv, z, p, partial);
        cg_init_scalars<PL><<<1, 256, 0, s>>>(partial, vb, PL::host_from_double(0.0), sc);
        ctx->launches += 2;
        CK(cudaGetLastError());
        CK(poll());
        std::vector<double> alpha, beta;
        double rz_old = PL::host_to_double(hsc->rz[0]);
        for (int k = 0; k < o.est_iters && !hsc->done; ++k) {
            const int parity = k & 1;
            A.apply(p, q, pq_partial, sc);
            cg_update_kernel<PL><<<vb, kVecThreads, 0, s>>>(n, xe, r, z, p, q, dinv, pq_partial, A.npq, partial, sc, parity);
            cg_p_kernel<PL><<<vb, kVecThreads, 0, s>>>(n, p, z, partial, vb, 1 << 30, sc, parity);
            ctx->launches += A.launches + 2;
            CK(cudaGetLastError());
            CK(poll());
            if (hsc->fail) break;
            const double pq = PL::host_to_double(hsc->pq);
            const double rz_new = PL::host_to_double(hsc->rz[parity ^ 1]);
            if (!(pq > 0) || !(rz_old > 0)) break;
            alpha.push_back(rz_old / pq);
            beta.push_back(rz_new / rz_old);
            rz_old = rz_new;
        }
        const int m = (int)alpha.size();
        std::vector<double> dg(m), off(m > 0 ? m - 1 : 0);
        for (int j = 0; j < m; ++j) {
            dg[j] = 1.0 / alpha[j] + (j > 0 ? beta[j - 1] / alpha[j - 1] : 0.0);
            if (j + 1 < m) off[j] = std::sqrt(std::max(beta[j], 0.0)) / alpha[j];
        }
        double lmax = m > 0 ? tridiag_max_eig(dg, off) : 2.0;
        if (!(lmax > 0) || !std::isfinite(lmax)) lmax = 2.0;
        const double emax = 1.1 * lmax, emin = o.cheb_ratio * emax;
        const double theta = 0.5 * (emax + emin), delta = 0.5 * (emax - emin), sigma = theta / delta;
        double rho = 1.0 / sigma;
        for (int k = 1; k < K; ++k) {
            const double rn = 1.0 / (2.0 * sigma - rho);
            c1.push_back(PL::host_from_double(rn * rho));
            c2.push_back(PL::host_from_double(2.0 * rn / delta));
            rho = rn;
        }
        scale_vec_kernel<PL><<<vb, 256, 0, s>>>(n, dinv, dinv0, PL::host_from_double(1.0 / theta));
        ctx->launches++;
        dz = dinv0;
        if (res) { res->lmax = emax; res->lmin = emin; }
    }
    // z = P r from z_1 = dz r (already in z): K - 1 Chebyshev steps; the last
    // one rewrites the r.z partials (partial + vb) and optionally p
    auto precond = [&](S* p_out, const CGScalars<PL>* gate) {
        for (int k = 1; k < K; ++k) {
            A.apply(k == 1 ? z : d, q, nullptr, gate);
            cheb_step_kernel<PL><<<vb, kVecThreads, 0, s>>>(n, r, w, d, z, dinv, q, c1[k - 1], c2[k - 1], k == 1, k == K - 1,
                                                            partial + vb, p_out, gate);
            ctx->launches += A.launches + 1;
        }
    };
    // initial residual r = b - A x and the first direction
    A.apply(x, q, nullptr, nullptr);
    residual_from_q_kernel<PL><<<vb, 256, 0, s>>>(n, b, q, r);
    cg_init_kernel<PL><<<vb, kVecThreads, 0, s>>>(n, b, r, dz, z, p, partial);
    ctx->launches += A.launches + 2;
    if (cheb) precond(p, nullptr);
    if (pch) pch->apply(r, z, partial + vb, p, nullptr);
    cg_init_scalars<PL><<<1, 256, 0, s>>>(partial, vb, PL::host_from_double(o.rtol * o.rtol), sc);
    ctx->launches++;
    CK(cudaGetLastError());
    auto iteration = [&](int parity) {
        A.apply(p, q, pq_partial, sc);
        cg_update_kernel<PL><<<vb, kVecThreads, 0, s>>>(n, x, r, z, p, q, dz, pq_partial, A.npq, partial, sc, parity);
        ctx->launches += A.launches + 1;
        if (cheb) precond(nullptr, sc);
        if (pch) pch->apply(r, z, partial + vb, nullptr, sc);
        cg_p_kernel<PL><<<vb, kVecThreads, 0, s>>>(n, p, z, partial, vb, o.maxit, sc, parity);
        ctx->launches++;
    };
    if (A.graph) {
        const int64_t l0 = ctx->launches;
        CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < check_every; ++k) iteration(k & 1);
        cudaError_t e = cudaStreamEndCapture(s, &graph);
        if (e != cudaSuccess) { ctx->err = std::string("graph capture: ") + cudaGetErrorString(e); cleanup(); return FGPU_ERR_CUDA; }
        ctx->launches = l0;
        CK(cudaGraphInstantiate(&exec, graph, 0));
    }
    const int64_t per_replay =
        (int64_t)check_every * (A.launches + 2 + (cheb ? (K - 1) * (A.launches + 1) : 0) + (pch ? pch->launches : 0));
    CK(poll());
    int guard = 0, parity = 0, nref = 0, nbreak = 0;
    double rr_ref = PL::host_to_double(hsc->rr);
    while (true) {
        bool want = false;
        if (hsc->done) {
            if (!refresh || hsc->fail == 2) break;
            // recurrence converged: verify in binary64; binary32 breakdown
            // (p.Ap <= 0 from rounding): replace the residual and restart p
            if (hsc->fail == 1 && ++nbreak > 3) break;
            want = true;
        } else if (refresh && PL::host_to_double(hsc->rr) <= o.delta * o.delta * rr_ref) {
            want = true;
        }
        if (want) {
            bool conv = false;
            const int rc2 = (*refresh)(x, r, &conv);
            if (rc2 == kRefreshStagnated) { hsc->fail = 3; break; }
            if (rc2) { cleanup(); return rc2; }
            ++nref;
            if (conv) { if (res) res->true_conv = true; break; }
            if (hsc->it >= o.maxit) { hsc->fail = 2; break; }
            S* p_restart = hsc->done ? p : nullptr;
            cg_refresh_kernel<PL><<<vb, kVecThreads, 0, s>>>(n, r, dz, z, partial, p_restart);
            ctx->launches++;
            if (cheb) precond(p_restart, nullptr);
            if (pch) pch->apply(r, z, partial + vb, p_restart, nullptr);
            cg_refresh_scalars<PL><<<1, 256, 0, s>>>(partial, vb, sc);
            ctx->launches++;
            CK(cudaGetLastError());
            CK(poll());
            rr_ref = PL::host_to_double(hsc->rr);
            continue;
        }
        if (A.graph) {
            CK(cudaGraphLaunch(exec, s));
            ctx->launches += per_replay;
            guard += check_every;
        } else {
            iteration(parity);
            parity ^= 1;
            ++guard;
        }
        CK(poll());
        if (guard > o.maxit + 2 * check_every) break;
    }
    if (res) {
        res->nrefresh = nref;
        res->iters = hsc->it;
        res->fail = hsc->fail;
        res->rr = PL::host_to_double(hsc->rr);
        res->bb = PL::host_to_double(hsc->bb);
    }
    cleanup();
#undef CK
    return FGPU_OK;
}

// the AMG V-cycle as a CG preconditioner (amg.cu)
template <class PL>
PcHook<PL> amg_pc_hook(fgpu_amg* M);

// the p-multigrid V-cycle of a matrix-free operator as a CG preconditioner (pmg.cu)
template <class PL>
PcHook<PL> pmg_pc_hook(fgpu_pmg* P);

}  // namespace fgpu
