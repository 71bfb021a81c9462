// Restarted GMRES(m), the reference's default Krylov method (ksp-type gmres, restart 30:
// feelpp/feel/feelalg/backend.cpp:56, 733; PETSc KSPGMRES), for the matrices that CG cannot take:
// non-symmetric ones such as the default elimination of on() (rows zeroed, columns kept,
// matrixpetsc.cpp:1834-1840) or non-symmetric Nitsche terms.
//
// Right preconditioning (A M^-1 y = b, x = M^-1 y) so that the Arnoldi residual is the true
// residual ||b - A x||_2 and the stopping test is the CG one (rtol ||b||_2); PETSc's default is left
// preconditioning with the preconditioned norm, so iteration counts differ while the solutions agree
// to the tolerance. M: none, Jacobi, or the smoothed-aggregation AMG V-cycle (binary32).
//
// Orthogonalisation: classical Gram-Schmidt twice (CGS2), each pass one multi-dot kernel over the
// basis and one update kernel, so an iteration costs two passes over the basis instead of j + 1
// sequential dot products; one small device-to-host read per iteration (the new Hessenberg column)
// feeds the Givens rotations on the host. All reductions are fixed-order block sums: repeated solves
// give the same bits.
#include <algorithm>
#include <cmath>
#include <vector>

#include "fgpu_core.h"

namespace fgpu {
int launch_spmv(fgpu_ctx* ctx, const fgpu_matrix* A, const double* x, double* y, double alpha_b, const double* b);

namespace {

constexpr int kGmBlocks = 304;        // two blocks per SM for the multi-dot partials

__global__ void gm_diag_inv_kernel(int64_t n, const int64_t* __restrict__ ia, const int32_t* __restrict__ ja,
                                   const double* __restrict__ val, double* __restrict__ dinv) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        int64_t lo = ia[r], hi = ia[r + 1];
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (ja[mid] < r) lo = mid + 1; else hi = mid;
        }
        const double d = (lo < ia[r + 1] && ja[lo] == r) ? val[lo] : 0.0;
        dinv[r] = d != 0.0 ? 1.0 / d : 1.0;
    }
}

__device__ __forceinline__ double gm_block_sum(double v, double* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    v = 0.0;
    if (w == 0) {
        v = l < (int)(blockDim.x >> 5) ? sh[l] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    return v;
}

// partial[i * gridDim.x + b] = block b's part of V_i . w, i < k (blockIdx.y = i)
__global__ void __launch_bounds__(256) gm_multidot_kernel(int64_t n, const double* __restrict__ V, int64_t ldv,
                                                          const double* __restrict__ w, double* __restrict__ partial) {
    __shared__ double sh[32];
    const double* v = V + (int64_t)blockIdx.y * ldv;
    double s = 0.0;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) s = fma(v[t], w[t], s);
    s = gm_block_sum(s, sh);
    if (threadIdx.x == 0) partial[(int64_t)blockIdx.y * gridDim.x + blockIdx.x] = s;
}

// out[i] = sum of partial[i * nb ...] in block order (one block per i); acc: out[i] += (the sum)
__global__ void gm_reduce_kernel(int nb, const double* __restrict__ partial, double* __restrict__ out, int acc) {
    __shared__ double sh[32];
    double s = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) s += partial[(int64_t)blockIdx.x * nb + b];
    s = gm_block_sum(s, sh);
    if (threadIdx.x == 0) out[blockIdx.x] = acc ? out[blockIdx.x] + s : s;
}

// w -= sum_i h[i] V_i (i < k)
__global__ void gm_update_kernel(int64_t n, int k, const double* __restrict__ V, int64_t ldv, const double* __restrict__ h,
                                 double* __restrict__ w) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        double s = w[t];
        for (int i = 0; i < k; ++i) s = fma(-h[i], V[(int64_t)i * ldv + t], s);
        w[t] = s;
    }
}

// out = w / sqrt(ww) (out = w when ww is 0)
__global__ void gm_normalise_kernel(int64_t n, const double* __restrict__ w, const double* __restrict__ ww, double* __restrict__ out) {
    const double nrm = sqrt(*ww);
    const double inv = nrm > 0.0 ? 1.0 / nrm : 1.0;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) out[t] = w[t] * inv;
}

__global__ void gm_scale_kernel(int64_t n, double a, double* __restrict__ v) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) v[t] *= a;
}

// out = sum_i y[i] V_i (i < k)
__global__ void gm_combine_kernel(int64_t n, int k, const double* __restrict__ V, int64_t ldv, const double* __restrict__ y,
                                  double* __restrict__ out) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int i = 0; i < k; ++i) s = fma(y[i], V[(int64_t)i * ldv + t], s);
        out[t] = s;
    }
}

// r = b - Ax (Ax in r on entry)
__global__ void gm_residual_kernel(int64_t n, const double* __restrict__ b, double* __restrict__ r) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) r[t] = b[t] - r[t];
}

__global__ void gm_jacobi_kernel(int64_t n, const double* __restrict__ dinv, const double* __restrict__ v, double* __restrict__ z) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) z[t] = dinv[t] * v[t];
}

__global__ void gm_to_f32_kernel(int64_t n, const double* __restrict__ v, float* __restrict__ f) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) f[t] = (float)v[t];
}

__global__ void gm_from_f32_kernel(int64_t n, const float* __restrict__ f, double* __restrict__ z) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) z[t] = (double)f[t];
}

__global__ void gm_axpy_kernel(int64_t n, const double* __restrict__ z, double* __restrict__ x) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) x[t] += z[t];
}

struct GmWork {
    double *V = nullptr, *w = nullptr, *z = nullptr, *dinv = nullptr, *partial = nullptr, *small = nullptr;
    float *f_in = nullptr;
    ~GmWork() {
        cudaFree(V); cudaFree(w); cudaFree(z); cudaFree(dinv); cudaFree(partial); cudaFree(small); cudaFree(f_in);
    }
};

// Timing events and the launch count of one solve: released and booked on every
// exit of solve_gmres, the early error returns included.
struct GmScope {
    fgpu_ctx* ctx;
    const int64_t* launches;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    GmScope(fgpu_ctx* c, const int64_t* l) : ctx(c), launches(l) {
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
    }
    ~GmScope() {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        ctx->launches += *launches;
    }
};

}  // namespace

int solve_gmres(fgpu_ctx* ctx, const fgpu_matrix* A, fgpu_amg* amg, const double* b, double* x, const fgpu_solver_cfg* cfg,
                int restart, fgpu_solve_stats* st) {
    const int64_t n = A->nrows;
    const int m = restart > 0 ? std::min(restart, 200) : 30;
    const int pc = cfg->pc;
    if (pc != FGPU_PC_NONE && pc != FGPU_PC_JACOBI && pc != FGPU_PC_GAMG) {
        ctx->err = "gmres: preconditioners none, jacobi or gamg";
        return FGPU_ERR_INVALID;
    }
    if (pc == FGPU_PC_GAMG && (!amg || amg_rows(amg) != n || amg_context(amg) != ctx)) {
        ctx->err = "gmres: pc gamg needs an AMG of this matrix on this context";
        return FGPU_ERR_INVALID;
    }
    if (A->precision != FGPU_F64) { ctx->err = "gmres: FP64 matrices"; return FGPU_ERR_INVALID; }
    cudaStream_t s = ctx->stream;
    const int vb = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 8));
    GmWork W;
    const int64_t ldv = (n + 31) / 32 * 32;
    cudaError_t e = cudaMalloc(&W.V, (size_t)(m + 1) * ldv * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&W.w, n * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&W.z, n * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&W.partial, (size_t)(m + 1) * kGmBlocks * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&W.small, (size_t)(2 * m + 8) * sizeof(double));
    if (e == cudaSuccess && pc == FGPU_PC_JACOBI) e = cudaMalloc(&W.dinv, n * sizeof(double));
    if (e == cudaSuccess && pc == FGPU_PC_GAMG) e = cudaMalloc(&W.f_in, n * sizeof(float));
    if (e != cudaSuccess) { cudaGetLastError(); ctx->err = "gmres: allocation failed"; return FGPU_ERR_ALLOC; }
    double* h1 = W.small;                 // m + 1: first CGS pass
    double* h2 = W.small + (m + 1);       // m + 1: second pass; h2[m + 1] .. holds w.w (see below)
    double* ww = W.small + 2 * m + 4;     // w.w
    double* ydev = W.small;               // reused for the least-squares solution at the end of a cycle
    int64_t launches = 0;
    if (pc == FGPU_PC_JACOBI) {
        gm_diag_inv_kernel<<<vb, 256, 0, s>>>(n, A->pattern->d_ia, A->pattern->d_ja, (const double*)A->d_val, W.dinv);
        ++launches;
    }
    auto dots = [&](int k, const double* V, const double* w, double* out, int acc) {
        gm_multidot_kernel<<<dim3(kGmBlocks, k), 256, 0, s>>>(n, V, ldv, w, W.partial);
        gm_reduce_kernel<<<k, 256, 0, s>>>(kGmBlocks, W.partial, out, acc);
        launches += 2;
    };
    auto precond = [&](const double* v, double* z) -> int {
        if (pc == FGPU_PC_NONE) {
            cudaMemcpyAsync(z, v, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
        } else if (pc == FGPU_PC_JACOBI) {
            gm_jacobi_kernel<<<vb, 256, 0, s>>>(n, W.dinv, v, z);
            ++launches;
        } else {
            gm_to_f32_kernel<<<vb, 256, 0, s>>>(n, v, W.f_in);
            const float* xa = nullptr;
            launches += 2 + amg_vcycle_f32(amg, W.f_in, nullptr, &xa, 1);
            gm_from_f32_kernel<<<vb, 256, 0, s>>>(n, xa, z);
        }
        return FGPU_OK;
    };
    auto residual_into = [&](double* r) -> int {     // r = b - A x
        int rc = launch_spmv(ctx, A, x, r, 0.0, nullptr);
        if (rc) return rc;
        gm_residual_kernel<<<vb, 256, 0, s>>>(n, b, r);
        launches += 2;
        return FGPU_OK;
    };
    auto read = [&](double* host, const double* dev, int cnt) -> int {
        FGPU_CUDA_CHECK(ctx, cudaMemcpyAsync(host, dev, cnt * sizeof(double), cudaMemcpyDeviceToHost, s));
        FGPU_CUDA_CHECK(ctx, cudaStreamSynchronize(s));
        return FGPU_OK;
    };
    GmScope scope(ctx, &launches);
    cudaEvent_t e0 = scope.e0, e1 = scope.e1;
    cudaEventRecord(e0, s);
    double bb = 0.0;
    dots(1, b, b, ww, 0);
    int rc = read(&bb, ww, 1);
    if (rc) return rc;
    const double bnorm = std::sqrt(bb);
    const double tol = cfg->rtol * bnorm;
    const int maxit = cfg->maxit > 0 ? cfg->maxit : 10000;
    std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), y(m);
    int it = 0, status = FGPU_OK;
    double res = bnorm;
    bool converged = bnorm == 0.0;
    if (converged) FGPU_CUDA_CHECK(ctx, cudaMemsetAsync(x, 0, n * sizeof(double), s));
    while (!converged && it < maxit) {
        // r0 = b - A x, v_0 = r0 / beta
        rc = residual_into(W.V);
        if (rc) return rc;
        dots(1, W.V, W.V, ww, 0);
        double beta2 = 0.0;
        rc = read(&beta2, ww, 1);
        if (rc) return rc;
        const double beta = std::sqrt(beta2);
        res = beta;
        if (!(beta > tol)) { converged = true; break; }
        gm_scale_kernel<<<vb, 256, 0, s>>>(n, 1.0 / beta, W.V);
        ++launches;
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int k = 0;
        for (int j = 0; j < m && it < maxit; ++j) {
            double* vj = W.V + (int64_t)j * ldv;
            precond(vj, W.z);
            rc = launch_spmv(ctx, A, W.z, W.w, 0.0, nullptr);
            if (rc) return rc;
            ++launches;
            // CGS2 against v_0 .. v_j
            dots(j + 1, W.V, W.w, h1, 0);
            gm_update_kernel<<<vb, 256, 0, s>>>(n, j + 1, W.V, ldv, h1, W.w);
            dots(j + 1, W.V, W.w, h2, 0);
            gm_update_kernel<<<vb, 256, 0, s>>>(n, j + 1, W.V, ldv, h2, W.w);
            dots(1, W.w, W.w, ww, 0);
            gm_normalise_kernel<<<vb, 256, 0, s>>>(n, W.w, ww, W.V + (int64_t)(j + 1) * ldv);
            launches += 3;
            std::vector<double> hc(2 * (m + 1) + 8);
            rc = read(hc.data(), W.small, 2 * m + 8);
            if (rc) return rc;
            for (int i = 0; i <= j; ++i) H[(size_t)i * m + j] = hc[i] + hc[(m + 1) + i];
            const double hn = std::sqrt(hc[2 * m + 4]);
            H[(size_t)(j + 1) * m + j] = hn;
            for (int i = 0; i < j; ++i) {     // earlier rotations
                const double a = H[(size_t)i * m + j], c = H[(size_t)(i + 1) * m + j];
                H[(size_t)i * m + j] = cs[i] * a + sn[i] * c;
                H[(size_t)(i + 1) * m + j] = -sn[i] * a + cs[i] * c;
            }
            const double a = H[(size_t)j * m + j], c = H[(size_t)(j + 1) * m + j];
            const double rr = std::hypot(a, c);
            cs[j] = rr > 0.0 ? a / rr : 1.0;
            sn[j] = rr > 0.0 ? c / rr : 0.0;
            H[(size_t)j * m + j] = rr;
            H[(size_t)(j + 1) * m + j] = 0.0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            ++it;
            k = j + 1;
            res = std::fabs(g[j + 1]);
            if (!(res > tol) || !(hn > 0.0)) break;
        }
        // y = H^-1 g (upper triangular k x k), x += M^-1 (V y)
        for (int i = k - 1; i >= 0; --i) {
            double sum = g[i];
            for (int l = i + 1; l < k; ++l) sum -= H[(size_t)i * m + l] * y[l];
            const double d = H[(size_t)i * m + i];
            if (d == 0.0) { status = FGPU_ERR_BREAKDOWN; y[i] = 0.0; } else y[i] = sum / d;
        }
        if (status) break;
        FGPU_CUDA_CHECK(ctx, cudaMemcpyAsync(ydev, y.data(), k * sizeof(double), cudaMemcpyHostToDevice, s));
        gm_combine_kernel<<<vb, 256, 0, s>>>(n, k, W.V, ldv, ydev, W.w);
        precond(W.w, W.z);
        gm_axpy_kernel<<<vb, 256, 0, s>>>(n, W.z, x);
        launches += 2;
        FGPU_CUDA_CHECK(ctx, cudaStreamSynchronize(s));   // ydev is overwritten by the next cycle's dots
    }
    // final binary64 residual
    double rfin = 0.0;
    if (bnorm > 0.0) {
        rc = residual_into(W.w);
        if (rc) return rc;
        dots(1, W.w, W.w, ww, 0);
        rc = read(&rfin, ww, 1);
        if (rc) return rc;
        rfin = std::sqrt(rfin);
    }
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    FGPU_CUDA_CHECK(ctx, cudaGetLastError());
    if (st) {
        *st = fgpu_solve_stats{};
        st->iterations = it;
        st->outer = (it + m - 1) / m;
        st->rel_residual = bnorm > 0.0 ? rfin / bnorm : 0.0;
        st->time_ms = ms;
    }
    if (status) { ctx->err = "gmres: breakdown (singular Hessenberg)"; return status; }
    if (bnorm > 0.0 && !(rfin <= cfg->rtol * bnorm * 1.0000001)) {
        ctx->err = "gmres: not converged";
        return FGPU_ERR_NOT_CONVERGED;
    }
    return FGPU_OK;
}

}  // namespace fgpu
