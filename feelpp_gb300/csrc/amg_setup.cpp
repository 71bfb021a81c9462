// Smoothed-aggregation AMG hierarchy (host set-up), the preconditioner the
// reference's users select with pc-type=gamg (PETSc PCGAMG, type "agg";
// feelpp/feel/feelalg/preconditionerpetsc.cpp:2229-2330, defaults
// feelpp/feel/feelalg/backend.cpp:813-818: threshold 0, coarse-eq-lim 800,
// nsmooths 1, 10 levels).
//
// Per level (Vanek, Mandel, Brezina, "Algebraic multigrid by smoothed
// aggregation for second and fourth order elliptic problems", Computing 56,
// 1996):
//   1. strength graph: j is a strong neighbour of i when
//      |a_ij| > theta sqrt(|a_ii a_jj|) (theta = 0: every stored coupling),
//      symmetrised;
//   2. aggregation: roots form a maximal distance-2 independent set (rounds
//      with hashed priorities, order-independent), their neighbours join them,
//      the other nodes join a neighbouring aggregate; nodes without strong
//      neighbours (rows eliminated by on(), decoupled) are left out: their
//      prolongator rows are zero and the smoother solves them exactly;
//   3. tentative prolongator: P0(i, agg(i)) = 1/sqrt(|agg|) (the constant near
//      null space, orthonormal columns);
//   4. prolongator smoothing: P = (I - omega D^-1 A) P0, omega = 4 / (3 lmax),
//      lmax = lmax(D^-1 A) from a Lanczos estimate;
//   5. Galerkin coarse operator A_c = P^T A P (R = P^T stored explicitly),
//      by row-wise sparse products with a dense accumulator per thread;
// until the level has at most coarse_eq_lim rows or max_levels is reached;
// the coarsest operator is inverted densely (Cholesky) when small enough.
//
// Everything is deterministic: the row loops are split among threads, but
// each output entry is accumulated in a fixed order and rows keep sorted
// columns, so the hierarchy does not depend on the thread count.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <functional>
#include <string>
#include <thread>
#include <vector>

#include "fgpu_core.h"

namespace fgpu {

namespace {

void parallel_rows(int nthreads, int64_t n, const std::function<void(int, int64_t, int64_t)>& fn) {
    const int T = (int)std::max<int64_t>(1, std::min<int64_t>(nthreads, (n + 4095) / 4096));
    if (T == 1) { fn(0, 0, n); return; }
    std::vector<std::thread> th;
    for (int t = 0; t < T; ++t) {
        const int64_t b = n * t / T, e = n * (t + 1) / T;
        th.emplace_back(fn, t, b, e);
    }
    for (auto& x : th) x.join();
}

// fn(chunk, r0, r1) over fixed chunks of `chunk` rows, the chunks spread over the threads: per-chunk
// partial sums combined in chunk order do not depend on the thread count
void parallel_chunks(int nthreads, int64_t n, int64_t chunk, const std::function<void(int64_t, int64_t, int64_t)>& fn) {
    const int64_t nc = (n + chunk - 1) / chunk;
    parallel_rows(nthreads, nc * 4096, [&](int, int64_t c0, int64_t c1) {
        for (int64_t c = c0 / 4096; c < c1 / 4096; ++c) fn(c, c * chunk, std::min(n, (c + 1) * chunk));
    });
}

// C = A * B (rows of A times B), Gustavson with a dense accumulator; columns
// of every row sorted. Each entry sums its products in (A column, B column) order.
void spgemm(const HostCsr& A, const HostCsr& B, HostCsr& C, int nthreads) {
    C.nrows = A.nrows;
    C.ncols = B.ncols;
    const int T = (int)std::max<int64_t>(1, std::min<int64_t>(nthreads, (A.nrows + 4095) / 4096));
    std::vector<std::vector<int32_t>> tj(T);
    std::vector<std::vector<double>> ta(T);
    std::vector<int64_t> len(A.nrows, 0);
    parallel_rows(T, A.nrows, [&](int t, int64_t r0, int64_t r1) {
        std::vector<double> acc(B.ncols, 0.0);
        std::vector<int32_t> mark(B.ncols, -1), cols;
        auto& J = tj[t];
        auto& V = ta[t];
        for (int64_t i = r0; i < r1; ++i) {
            cols.clear();
            for (int64_t p = A.ia[i]; p < A.ia[i + 1]; ++p) {
                const int32_t k = A.ja[p];
                const double a = A.a[p];
                for (int64_t q = B.ia[k]; q < B.ia[k + 1]; ++q) {
                    const int32_t j = B.ja[q];
                    if (mark[j] != (int32_t)(i & 0x7fffffff)) {
                        mark[j] = (int32_t)(i & 0x7fffffff);
                        acc[j] = 0.0;
                        cols.push_back(j);
                    }
                    acc[j] += a * B.a[q];
                }
            }
            std::sort(cols.begin(), cols.end());
            for (int32_t j : cols) {
                J.push_back(j);
                V.push_back(acc[j]);
            }
            len[i] = (int64_t)cols.size();
        }
    });
    C.ia.assign(A.nrows + 1, 0);
    for (int64_t i = 0; i < A.nrows; ++i) C.ia[i + 1] = C.ia[i] + len[i];
    C.ja.resize(C.ia[A.nrows]);
    C.a.resize(C.ia[A.nrows]);
    int64_t off = 0;
    for (int t = 0; t < T; ++t) {
        std::copy(tj[t].begin(), tj[t].end(), C.ja.begin() + off);
        std::copy(ta[t].begin(), ta[t].end(), C.a.begin() + off);
        off += (int64_t)tj[t].size();
    }
}

void transpose(const HostCsr& A, HostCsr& T) {
    T.nrows = A.ncols;
    T.ncols = A.nrows;
    T.ia.assign(A.ncols + 1, 0);
    for (int64_t p = 0; p < A.ia[A.nrows]; ++p) T.ia[A.ja[p] + 1]++;
    for (int64_t j = 0; j < A.ncols; ++j) T.ia[j + 1] += T.ia[j];
    T.ja.resize(A.ia[A.nrows]);
    T.a.resize(A.ia[A.nrows]);
    std::vector<int64_t> fill(T.ia.begin(), T.ia.end() - 1);
    for (int64_t i = 0; i < A.nrows; ++i)
        for (int64_t p = A.ia[i]; p < A.ia[i + 1]; ++p) {
            const int64_t q = fill[A.ja[p]]++;
            T.ja[q] = (int32_t)i;
            T.a[q] = A.a[p];
        }
}

std::vector<double> diagonal(const HostCsr& A) {
    std::vector<double> d(A.nrows, 0.0);
    for (int64_t i = 0; i < A.nrows; ++i)
        for (int64_t p = A.ia[i]; p < A.ia[i + 1]; ++p)
            if (A.ja[p] == i) d[i] = A.a[p];
    return d;
}

// lmax(D^-1 A) of a symmetric positive definite A: Lanczos on D^-1/2 A D^-1/2
// (m steps from a fixed pseudo-random start), largest Ritz value by bisection
double lmax_estimate(const HostCsr& A, const std::vector<double>& d, int m, int nthreads) {
    const int64_t n = A.nrows;
    if (n == 0) return 1.0;
    std::vector<double> s(n), v, vold(n, 0.0), w(n);
    for (int64_t i = 0; i < n; ++i) s[i] = d[i] > 0 ? 1.0 / std::sqrt(d[i]) : 0.0;
    amg_lanczos_start(n, v);
    std::vector<double> al, be;
    double bprev = 0;
    const int T = (int)std::max<int64_t>(1, std::min<int64_t>(nthreads, (n + 4095) / 4096));
    constexpr int64_t kChunk = 1024;
    const int64_t nch = (n + kChunk - 1) / kChunk;
    std::vector<double> pa(nch), pb(nch);
    for (int k = 0; k < m; ++k) {
        parallel_chunks(T, n, kChunk, [&](int64_t c, int64_t r0, int64_t r1) {
            double sa = 0;
            for (int64_t i = r0; i < r1; ++i) {
                double acc = 0;
                for (int64_t p = A.ia[i]; p < A.ia[i + 1]; ++p) acc += A.a[p] * s[A.ja[p]] * v[A.ja[p]];
                w[i] = s[i] * acc;
                sa += w[i] * v[i];
            }
            pa[c] = sa;
        });
        double a = 0;
        for (int64_t c = 0; c < nch; ++c) a += pa[c];
        parallel_chunks(T, n, kChunk, [&](int64_t c, int64_t r0, int64_t r1) {
            double sb = 0;
            for (int64_t i = r0; i < r1; ++i) {
                w[i] -= a * v[i] + bprev * vold[i];
                sb += w[i] * w[i];
            }
            pb[c] = sb;
        });
        double b = 0;
        for (int64_t c = 0; c < nch; ++c) b += pb[c];
        b = std::sqrt(b);
        al.push_back(a);
        if (b < 1e-14 * std::fabs(a) || k + 1 == m) break;
        be.push_back(b);
        parallel_rows(T, n, [&](int, int64_t r0, int64_t r1) {
            for (int64_t i = r0; i < r1; ++i) {
                vold[i] = v[i];
                v[i] = w[i] / b;
            }
        });
        bprev = b;
    }
    return amg_tridiag_lmax(al, be);
}

// strong neighbours (symmetrised, without the diagonal) as a CSR graph
void strength(const HostCsr& A, const std::vector<double>& d, double theta, std::vector<int64_t>& sp, std::vector<int32_t>& sj,
              int nthreads) {
    const int64_t n = A.nrows;
    std::vector<int64_t> cnt(n + 1, 0);
    auto strong = [&](int64_t i, int64_t p) {
        const int32_t j = A.ja[p];
        if (j == i || A.a[p] == 0.0) return false;
        return std::fabs(A.a[p]) > theta * std::sqrt(std::fabs(d[i] * d[j]));
    };
    parallel_rows(nthreads, n, [&](int, int64_t r0, int64_t r1) {
        for (int64_t i = r0; i < r1; ++i)
            for (int64_t p = A.ia[i]; p < A.ia[i + 1]; ++p)
                if (strong(i, p)) cnt[i + 1]++;
    });
    // symmetrise: a coupling counts when either direction is strong
    sp.assign(n + 1, 0);
    std::vector<int32_t> tmpj;
    std::vector<int64_t> tp(n + 1, 0);
    for (int64_t i = 0; i < n; ++i) tp[i + 1] = tp[i] + cnt[i + 1];
    tmpj.resize(tp[n]);
    parallel_rows(nthreads, n, [&](int, int64_t r0, int64_t r1) {
        for (int64_t i = r0; i < r1; ++i) {
            int64_t q = tp[i];
            for (int64_t p = A.ia[i]; p < A.ia[i + 1]; ++p)
                if (strong(i, p)) tmpj[q++] = A.ja[p];
        }
    });
    // transpose of the strong graph, merged with it (sorted, unique)
    std::vector<int64_t> tc(n + 1, 0);
    for (int64_t q = 0; q < tp[n]; ++q) tc[tmpj[q] + 1]++;
    for (int64_t i = 0; i < n; ++i) tc[i + 1] += tc[i];
    std::vector<int32_t> tj(tp[n]);
    {
        std::vector<int64_t> f(tc.begin(), tc.end() - 1);
        for (int64_t i = 0; i < n; ++i)
            for (int64_t q = tp[i]; q < tp[i + 1]; ++q) tj[f[tmpj[q]]++] = (int32_t)i;
    }
    // merge of the two sorted lists per row: count, offsets, fill (rows in parallel)
    auto merge_row = [&](int64_t i, int32_t* out) {
        int64_t a = tp[i], b = tc[i], k = 0;
        const int64_t ae = tp[i + 1], bend = tc[i + 1];
        while (a < ae || b < bend) {
            int32_t v;
            if (b >= bend || (a < ae && tmpj[a] < tj[b])) v = tmpj[a++];
            else if (a >= ae || tj[b] < tmpj[a]) v = tj[b++];
            else { v = tmpj[a++]; ++b; }
            if (out) out[k] = v;
            ++k;
        }
        return k;
    };
    std::vector<int64_t> len(n + 1, 0);
    parallel_rows(nthreads, n, [&](int, int64_t r0, int64_t r1) {
        for (int64_t i = r0; i < r1; ++i) len[i + 1] = merge_row(i, nullptr);
    });
    for (int64_t i = 0; i < n; ++i) sp[i + 1] = sp[i] + len[i + 1];
    sj.assign(sp[n], 0);
    parallel_rows(nthreads, n, [&](int, int64_t r0, int64_t r1) {
        for (int64_t i = r0; i < r1; ++i) merge_row(i, sj.data() + sp[i]);
    });
}

// Aggregation (returns the number of aggregates; agg[i] = -1 for nodes without strong neighbours):
//   1. roots: a maximal distance-2 independent set (no two roots within two edges), found in rounds: an
//      undecided node becomes a root when its key is the largest among the undecided nodes within
//      distance 2 and no root lies within distance 2 of it; a node with a root within distance 2 is
//      out. Keys: a hash of the node index in the high 32 bits, the index in the low ones (distinct);
//   2. a root's neighbours join its aggregate (a node has at most one root neighbour);
//   3. every other coupled node (within distance 2 of a root, as the set is maximal) joins the
//      aggregate of its first neighbour, in column order, that step 2 aggregated.
// Aggregates are numbered by root index. Every step reads the previous step's arrays only, so the
// result does not depend on the order in which nodes are visited: the device set-up runs the same
// rounds as kernels and gets the same aggregates.
void aggregate_mis2(int64_t n, const int64_t* sp, const int32_t* sj, std::vector<int32_t>& agg, int nthreads) {
    std::vector<int8_t> state(n), nstate(n);     // 0 undecided, 1 root, 2 out, 3 no strong neighbours
    std::vector<uint64_t> m1(n);
    std::vector<uint8_t> r1(n);
    int64_t undecided = 0;
    for (int64_t i = 0; i < n; ++i) {
        state[i] = sp[i + 1] > sp[i] ? 0 : 3;
        undecided += state[i] == 0;
    }
    while (undecided > 0) {
        parallel_rows(nthreads, n, [&](int, int64_t r0, int64_t r1_) {
            for (int64_t i = r0; i < r1_; ++i) {
                uint64_t m = state[i] == 0 ? amg_mis_key(i) : 0;
                uint8_t r = state[i] == 1;
                for (int64_t q = sp[i]; q < sp[i + 1]; ++q) {
                    const int32_t j = sj[q];
                    if (state[j] == 0) m = std::max(m, amg_mis_key(j));
                    r |= state[j] == 1;
                }
                m1[i] = m;
                r1[i] = r;
            }
        });
        std::vector<int64_t> cnt(std::max(1, nthreads), 0);
        parallel_rows(nthreads, n, [&](int t, int64_t r0, int64_t r1_) {
            int64_t c = 0;
            for (int64_t i = r0; i < r1_; ++i) {
                nstate[i] = state[i];
                if (state[i] != 0) continue;
                uint64_t m = m1[i];
                uint8_t r = r1[i];
                for (int64_t q = sp[i]; q < sp[i + 1]; ++q) {
                    m = std::max(m, m1[sj[q]]);
                    r |= r1[sj[q]];
                }
                if (r) nstate[i] = 2;
                else if (m == amg_mis_key(i)) nstate[i] = 1;
                else ++c;
            }
            cnt[t] += c;
        });
        state.swap(nstate);
        undecided = 0;
        for (int64_t c : cnt) undecided += c;
    }
    std::vector<int32_t> rank(n, -1);
    int32_t nroots = 0;
    for (int64_t i = 0; i < n; ++i)
        if (state[i] == 1) rank[i] = nroots++;
    std::vector<int32_t> a1(n, -1);
    parallel_rows(nthreads, n, [&](int, int64_t r0, int64_t r1_) {
        for (int64_t i = r0; i < r1_; ++i) {
            if (state[i] == 1) { a1[i] = rank[i]; continue; }
            for (int64_t q = sp[i]; q < sp[i + 1]; ++q)
                if (state[sj[q]] == 1) { a1[i] = rank[sj[q]]; break; }
        }
    });
    agg.assign(n, -1);
    parallel_rows(nthreads, n, [&](int, int64_t r0, int64_t r1_) {
        for (int64_t i = r0; i < r1_; ++i) {
            if (a1[i] >= 0 || state[i] == 3) { agg[i] = a1[i]; continue; }
            for (int64_t q = sp[i]; q < sp[i + 1]; ++q)
                if (a1[sj[q]] >= 0) { agg[i] = a1[sj[q]]; break; }
        }
    });
}

int64_t aggregate(int64_t n, const std::vector<int64_t>& sp, const std::vector<int32_t>& sj, std::vector<int32_t>& agg, int nthreads) {
    aggregate_mis2(n, sp.data(), sj.data(), agg, nthreads);
    int64_t nagg = 0;
    for (int64_t i = 0; i < n; ++i) nagg = std::max<int64_t>(nagg, agg[i] + 1);
    return nagg;
}

// P0(i, agg(i)) = 1/sqrt(|agg|): the constant near null space
void tentative_constant(int64_t n, const std::vector<int32_t>& agg, int64_t nagg, HostCsr& P0) {
    std::vector<double> sz(nagg, 0.0);
    for (int64_t i = 0; i < n; ++i)
        if (agg[i] >= 0) sz[agg[i]] += 1.0;
    std::vector<double> s0(nagg);
    for (int64_t c = 0; c < nagg; ++c) s0[c] = 1.0 / std::sqrt(sz[c]);
    P0.nrows = n;
    P0.ncols = nagg;
    P0.ia.assign(n + 1, 0);
    for (int64_t i = 0; i < n; ++i) P0.ia[i + 1] = P0.ia[i] + (agg[i] >= 0 ? 1 : 0);
    P0.ja.resize(P0.ia[n]);
    P0.a.resize(P0.ia[n]);
    for (int64_t i = 0; i < n; ++i)
        if (agg[i] >= 0) {
            P0.ja[P0.ia[i]] = agg[i];
            P0.a[P0.ia[i]] = s0[agg[i]];
        }
}

// P = (I - omega D^-1 A) P0 (nsmooth > 0) or P0
void smooth_prolongator(const HostCsr& A, const std::vector<double>& d, HostCsr&& P0, double omega, int nsmooth, HostCsr& P,
                        int nthreads) {
    if (nsmooth <= 0) { P = std::move(P0); return; }
    HostCsr AP;
    spgemm(A, P0, AP, nthreads);
    // P = P0 - omega D^-1 (A P0): merge the sorted rows (count, offsets, fill; rows in parallel)
    P.nrows = A.nrows;
    P.ncols = P0.ncols;
    P.ia.assign(A.nrows + 1, 0);
    auto merge_row = [&](int64_t i, int32_t* oj, double* oa) {
        const double f = d[i] != 0.0 ? omega / d[i] : 0.0;
        int64_t p = P0.ia[i], k = 0;
        const int64_t pe = P0.ia[i + 1];
        auto put = [&](int32_t j, double v) {
            if (oj) { oj[k] = j; oa[k] = v; }
            ++k;
        };
        for (int64_t q = AP.ia[i]; q < AP.ia[i + 1]; ++q) {
            while (p < pe && P0.ja[p] < AP.ja[q]) { put(P0.ja[p], P0.a[p]); ++p; }
            double v = -f * AP.a[q];
            if (p < pe && P0.ja[p] == AP.ja[q]) { v += P0.a[p]; ++p; }
            put(AP.ja[q], v);
        }
        while (p < pe) { put(P0.ja[p], P0.a[p]); ++p; }
        return k;
    };
    std::vector<int64_t> len(A.nrows + 1, 0);
    parallel_rows(nthreads, A.nrows, [&](int, int64_t r0, int64_t r1) {
        for (int64_t i = r0; i < r1; ++i) len[i + 1] = merge_row(i, nullptr, nullptr);
    });
    for (int64_t i = 0; i < A.nrows; ++i) P.ia[i + 1] = P.ia[i] + len[i + 1];
    P.ja.assign(P.ia[A.nrows], 0);
    P.a.assign(P.ia[A.nrows], 0.0);
    parallel_rows(nthreads, A.nrows, [&](int, int64_t r0, int64_t r1) {
        for (int64_t i = r0; i < r1; ++i) merge_row(i, P.ja.data() + P.ia[i], P.a.data() + P.ia[i]);
    });
}

// dense inverse of a symmetric positive definite matrix (Cholesky); false when not SPD. The columns of
// the inverse are independent solves, split among the threads.
bool spd_inverse(int64_t n, std::vector<double>& M, int nthreads) {
    std::vector<double> L(M);
    for (int64_t j = 0; j < n; ++j) {
        double s = L[j * n + j];
        for (int64_t k = 0; k < j; ++k) s -= L[j * n + k] * L[j * n + k];
        if (!(s > 0)) return false;
        const double ljj = std::sqrt(s);
        L[j * n + j] = ljj;
        for (int64_t i = j + 1; i < n; ++i) {
            double t = L[i * n + j];
            for (int64_t k = 0; k < j; ++k) t -= L[i * n + k] * L[j * n + k];
            L[i * n + j] = t / ljj;
        }
    }
    // columns of the inverse: solve L L^T x = e_c
    std::vector<double> inv((size_t)n * n);
    const int T = (int)std::max<int64_t>(1, std::min<int64_t>(nthreads, n / 16));
    parallel_rows(T, n * 4096, [&](int, int64_t c0, int64_t c1) {
        std::vector<double> y(n);
        for (int64_t c = (c0 + 4095) / 4096; c < (c1 + 4095) / 4096; ++c) {
            for (int64_t i = 0; i < n; ++i) {
                double t = i == c ? 1.0 : 0.0;
                for (int64_t k = 0; k < i; ++k) t -= L[i * n + k] * y[k];
                y[i] = t / L[i * n + i];
            }
            for (int64_t i = n - 1; i >= 0; --i) {
                double t = y[i];
                for (int64_t k = i + 1; k < n; ++k) t -= L[k * n + i] * inv[k * n + c];
                inv[i * n + c] = t / L[i * n + i];
            }
        }
    });
    M.swap(inv);
    return true;
}

}  // namespace

// fixed pseudo-random start of the Lanczos estimate, normalised
void amg_lanczos_start(int64_t n, std::vector<double>& v) {
    v.assign(n, 0.0);
    uint64_t h = 0x9E3779B97F4A7C15ull;
    double nv = 0;
    for (int64_t i = 0; i < n; ++i) {
        h ^= h >> 33; h *= 0xff51afd7ed558ccdull; h ^= h >> 33;
        v[i] = (double)(h >> 11) * (1.0 / 9007199254740992.0) - 0.5;
        nv += v[i] * v[i];
    }
    nv = std::sqrt(nv);
    for (auto& x : v) x /= nv;
}

// largest eigenvalue of the symmetric tridiagonal (al, be) by Sturm bisection
double amg_tridiag_lmax(const std::vector<double>& al, const std::vector<double>& be) {
    const int mm = (int)al.size();
    double hi = 0;
    for (int j = 0; j < mm; ++j) {
        double g = std::fabs(al[j]);
        if (j > 0) g += std::fabs(be[j - 1]);
        if (j + 1 < mm) g += std::fabs(be[j]);
        hi = std::max(hi, g);
    }
    double lo = 0;
    auto below = [&](double x) {
        int c = 0;
        double q = 1.0;
        for (int j = 0; j < mm; ++j) {
            q = al[j] - x - (j > 0 ? be[j - 1] * be[j - 1] / q : 0.0);
            if (q == 0.0) q = -1e-300;
            if (q < 0) ++c;
        }
        return c;
    };
    for (int it = 0; it < 200 && hi - lo > 1e-10 * hi; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (below(mid) == mm) hi = mid;
        else lo = mid;
    }
    return hi > 0 ? hi : 1.0;
}


// node layout and storage of a near null space (values filled by the caller); nonzero when invalid
int amg_nns_layout(const fgpu_amg_cfg* cfg, int64_t n, AmgNns& nns) {
    const int bs = cfg->block_size > 0 ? cfg->block_size : 1;
    if (cfg->nns_count <= 0 || cfg->nns_count > 64 || n % bs != 0) return FGPU_ERR_INVALID;
    nns.m = cfg->nns_count;
    nns.node_ptr.resize(n / bs + 1);
    for (int64_t I = 0; I <= n / bs; ++I) nns.node_ptr[I] = I * bs;
    nns.B.assign((size_t)n * nns.m, 0.0);
    return FGPU_OK;
}

AmgHostCfg amg_host_cfg(const fgpu_amg_cfg* cfg, int nthreads) {
    AmgHostCfg hc;
    if (cfg) {
        hc.threshold = cfg->threshold;
        if (cfg->max_levels > 0) hc.max_levels = cfg->max_levels;
        if (cfg->coarse_eq_lim > 0) hc.coarse_eq_lim = cfg->coarse_eq_lim;
        hc.agg_smooths = cfg->agg_smooths == 0 ? 1 : cfg->agg_smooths < 0 ? 0 : cfg->agg_smooths;
    }
    hc.nthreads = nthreads;
    return hc;
}

void amg_collapse_graph(const std::vector<int64_t>& node_ptr, const std::vector<int64_t>& sp, const int32_t* sj, int nthreads,
                        std::vector<int64_t>& np, std::vector<int32_t>& nj) {
    const int64_t nn = (int64_t)node_ptr.size() - 1;
    const int64_t nd = node_ptr[nn];
    std::vector<int32_t> node_of(nd);
    for (int64_t I = 0; I < nn; ++I)
        for (int64_t i = node_ptr[I]; i < node_ptr[I + 1]; ++i) node_of[i] = (int32_t)I;
    auto row = [&](int64_t I, std::vector<int32_t>& tmp) {
        tmp.clear();
        for (int64_t i = node_ptr[I]; i < node_ptr[I + 1]; ++i)
            for (int64_t q = sp[i]; q < sp[i + 1]; ++q) {
                const int32_t J = node_of[sj[q]];
                if (J != I) tmp.push_back(J);
            }
        std::sort(tmp.begin(), tmp.end());
        tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
    };
    std::vector<int64_t> len(nn + 1, 0);
    parallel_rows(nthreads, nn, [&](int, int64_t r0, int64_t r1) {
        std::vector<int32_t> tmp;
        for (int64_t I = r0; I < r1; ++I) { row(I, tmp); len[I + 1] = (int64_t)tmp.size(); }
    });
    np.assign(nn + 1, 0);
    for (int64_t I = 0; I < nn; ++I) np[I + 1] = np[I] + len[I + 1];
    nj.assign(np[nn], 0);
    parallel_rows(nthreads, nn, [&](int, int64_t r0, int64_t r1) {
        std::vector<int32_t> tmp;
        for (int64_t I = r0; I < r1; ++I) {
            row(I, tmp);
            std::copy(tmp.begin(), tmp.end(), nj.begin() + np[I]);
        }
    });
}

// Per aggregate (its nodes in increasing order, their dofs in increasing order): B restricted to the
// aggregate's k dofs (k x m) = Q R by modified Gram-Schmidt; a column whose orthogonal part is below
// 1e-12 of its norm is dropped, so the aggregate gets r <= m coarse dofs. P0 holds Q (rows: the dofs,
// columns: the aggregate's coarse dofs); the coarse level's vectors are the rows of R.
int amg_tentative_nns(const AmgNns& nns, const std::vector<int32_t>& agg_node, int64_t nagg, int nthreads, HostCsr& P0,
                      AmgNns& coarse) {
    const int m = nns.m;
    const int64_t nn = (int64_t)nns.node_ptr.size() - 1;
    const int64_t nd = nns.node_ptr[nn];
    // nodes of each aggregate (counting sort, increasing node order)
    std::vector<int64_t> aptr(nagg + 1, 0);
    for (int64_t I = 0; I < nn; ++I)
        if (agg_node[I] >= 0) aptr[agg_node[I] + 1]++;
    for (int64_t c = 0; c < nagg; ++c) aptr[c + 1] += aptr[c];
    std::vector<int32_t> anodes(aptr[nagg]);
    {
        std::vector<int64_t> f(aptr.begin(), aptr.end() - 1);
        for (int64_t I = 0; I < nn; ++I)
            if (agg_node[I] >= 0) anodes[f[agg_node[I]]++] = (int32_t)I;
    }
    // QR of each aggregate
    std::vector<std::vector<double>> Q(nagg), R(nagg);
    std::vector<int> rank(nagg, 0);
    parallel_rows(nthreads, nagg, [&](int, int64_t c0, int64_t c1) {
        for (int64_t c = c0; c < c1; ++c) {
            std::vector<int64_t> dofs;
            for (int64_t t = aptr[c]; t < aptr[c + 1]; ++t)
                for (int64_t i = nns.node_ptr[anodes[t]]; i < nns.node_ptr[anodes[t] + 1]; ++i) dofs.push_back(i);
            const int64_t k = (int64_t)dofs.size();
            std::vector<double>& q = Q[c];               // k x m, column-major (kept columns first)
            std::vector<double>& r = R[c];               // m x m, row-major (rows: kept columns)
            q.assign((size_t)k * m, 0.0);
            r.assign((size_t)m * m, 0.0);
            int kept = 0;
            std::vector<double> v(k);
            for (int j = 0; j < m; ++j) {
                double n0 = 0.0;
                for (int64_t t = 0; t < k; ++t) {
                    v[t] = nns.B[(size_t)dofs[t] * m + j];
                    n0 += v[t] * v[t];
                }
                n0 = std::sqrt(n0);
                for (int l = 0; l < kept; ++l) {
                    double dot = 0.0;
                    for (int64_t t = 0; t < k; ++t) dot += q[(size_t)l * k + t] * v[t];
                    r[(size_t)l * m + j] = dot;
                    for (int64_t t = 0; t < k; ++t) v[t] -= dot * q[(size_t)l * k + t];
                }
                double nv = 0.0;
                for (int64_t t = 0; t < k; ++t) nv += v[t] * v[t];
                nv = std::sqrt(nv);
                if (nv > 1e-12 * n0 && nv > 1e-300) {
                    for (int64_t t = 0; t < k; ++t) q[(size_t)kept * k + t] = v[t] / nv;
                    r[(size_t)kept * m + j] = nv;
                    ++kept;
                }
            }
            rank[c] = kept;
        }
    });
    std::vector<int64_t> cptr(nagg + 1, 0);
    for (int64_t c = 0; c < nagg; ++c) cptr[c + 1] = cptr[c] + rank[c];
    if (cptr[nagg] >= ((int64_t)1 << 31)) return FGPU_ERR_INVALID;
    // P0 rows: a dof of aggregate c holds the c's Q row at columns cptr[c] ..
    std::vector<int32_t> agg_dof(nd, -1);
    std::vector<int64_t> pos_in_agg(nd, 0);
    for (int64_t c = 0; c < nagg; ++c) {
        int64_t t = 0;
        for (int64_t a = aptr[c]; a < aptr[c + 1]; ++a)
            for (int64_t i = nns.node_ptr[anodes[a]]; i < nns.node_ptr[anodes[a] + 1]; ++i) {
                agg_dof[i] = (int32_t)c;
                pos_in_agg[i] = t++;
            }
    }
    P0.nrows = nd;
    P0.ncols = cptr[nagg];
    P0.ia.assign(nd + 1, 0);
    for (int64_t i = 0; i < nd; ++i) P0.ia[i + 1] = P0.ia[i] + (agg_dof[i] >= 0 ? rank[agg_dof[i]] : 0);
    P0.ja.resize(P0.ia[nd]);
    P0.a.resize(P0.ia[nd]);
    for (int64_t i = 0; i < nd; ++i) {
        const int32_t c = agg_dof[i];
        if (c < 0) continue;
        const int64_t k = (int64_t)Q[c].size() / m;
        for (int l = 0; l < rank[c]; ++l) {
            P0.ja[P0.ia[i] + l] = (int32_t)(cptr[c] + l);
            P0.a[P0.ia[i] + l] = Q[c][(size_t)l * k + pos_in_agg[i]];
        }
    }
    // next level: node c = aggregate c, its dofs the rank[c] coarse dofs, its vectors the rows of R
    coarse.m = m;
    coarse.node_ptr = cptr;
    coarse.B.assign((size_t)cptr[nagg] * m, 0.0);
    for (int64_t c = 0; c < nagg; ++c)
        for (int l = 0; l < rank[c]; ++l)
            for (int j = 0; j < m; ++j) coarse.B[(size_t)(cptr[c] + l) * m + j] = R[c][(size_t)l * m + j];
    return FGPU_OK;
}

bool amg_build_host(HostCsr&& A0, const AmgHostCfg& cfg, AmgHierarchy& H, std::string& err, const AmgNns* nns) {
    const int nthreads = cfg.nthreads > 0 ? cfg.nthreads : (int)std::max(1u, std::thread::hardware_concurrency());
    const int max_levels = cfg.max_levels > 0 ? cfg.max_levels : 10;
    const int64_t coarse_lim = cfg.coarse_eq_lim > 0 ? cfg.coarse_eq_lim : 800;
    H.levels.clear();
    H.coarse_inv.clear();
    H.levels.emplace_back();
    H.levels[0].A = std::move(A0);
    AmgNns cur;
    if (nns) {
        cur = *nns;
        if (cur.m <= 0 || cur.node_ptr.empty() || cur.node_ptr.back() != H.levels[0].A.nrows ||
            (int64_t)cur.B.size() != H.levels[0].A.nrows * cur.m) {
            err = "gamg: near null space does not match the matrix";
            return false;
        }
    }
    for (int l = 0; l + 1 < max_levels; ++l) {
        AmgHostLevel& L = H.levels[l];
        const HostCsr& A = L.A;
        if (A.nrows <= coarse_lim) break;
        const std::vector<double> d = diagonal(A);
        for (int64_t i = 0; i < A.nrows; ++i)
            if (!(d[i] > 0)) { err = "gamg: the diagonal must be positive (SPD matrix)"; return false; }
        L.lmax = lmax_estimate(A, d, 12, nthreads);
        std::vector<int64_t> sp;
        std::vector<int32_t> sj;
        strength(A, d, cfg.threshold, sp, sj, nthreads);
        HostCsr P0;
        AmgNns next;
        int64_t nagg = 0;
        if (!nns) {
            nagg = aggregate(A.nrows, sp, sj, L.agg, nthreads);
            if (nagg == 0 || nagg >= A.nrows) break;          // nothing to coarsen
            tentative_constant(A.nrows, L.agg, nagg, P0);
        } else {
            std::vector<int64_t> np;
            std::vector<int32_t> nj, agg_node;
            amg_collapse_graph(cur.node_ptr, sp, sj.data(), nthreads, np, nj);
            const int64_t nn = (int64_t)cur.node_ptr.size() - 1;
            nagg = aggregate(nn, np, nj, agg_node, nthreads);
            if (nagg == 0 || nagg >= nn) break;
            if (amg_tentative_nns(cur, agg_node, nagg, nthreads, P0, next)) { err = "gamg: coarse level too large"; return false; }
            if (P0.ncols == 0 || P0.ncols >= A.nrows) break;
            L.agg.assign(A.nrows, -1);
            for (int64_t I = 0; I < nn; ++I)
                for (int64_t i = cur.node_ptr[I]; i < cur.node_ptr[I + 1]; ++i) L.agg[i] = agg_node[I];
        }
        const double omega = 4.0 / (3.0 * L.lmax);
        smooth_prolongator(A, d, std::move(P0), omega, cfg.agg_smooths, L.P, nthreads);
        transpose(L.P, L.R);
        HostCsr AP, Ac;
        spgemm(A, L.P, AP, nthreads);
        spgemm(L.R, AP, Ac, nthreads);
        const int64_t nc = Ac.nrows;
        H.levels.emplace_back();
        H.levels.back().A = std::move(Ac);
        if (nns) cur = std::move(next);
        if ((double)nc > 0.9 * (double)H.levels[l].A.nrows) break;   // stagnating coarsening
    }
    AmgHostLevel& C = H.levels.back();
    {
        const std::vector<double> d = diagonal(C.A);
        for (int64_t i = 0; i < C.A.nrows; ++i)
            if (!(d[i] > 0)) { err = "gamg: coarse diagonal not positive (matrix not SPD)"; return false; }
        C.lmax = lmax_estimate(C.A, d, 12, nthreads);
    }
    if (C.A.nrows <= kAmgDenseCoarse) {
        const int64_t n = C.A.nrows;
        std::vector<double> M((size_t)n * n, 0.0);
        for (int64_t i = 0; i < n; ++i)
            for (int64_t p = C.A.ia[i]; p < C.A.ia[i + 1]; ++p) M[i * n + C.A.ja[p]] = C.A.a[p];
        if (spd_inverse(n, M, nthreads)) H.coarse_inv.swap(M);
    }
    return true;
}

}  // namespace fgpu

// ---------------------------------------------------------------------------
// Host-only entry points: build and inspect a hierarchy from a host CSR (no
// device needed), for checking the set-up against its definition.
// ---------------------------------------------------------------------------

extern "C" int fgpu_amg_host_build(int64_t n, const int64_t* ia, const int32_t* ja, const double* a, const fgpu_amg_cfg* cfg,
                                   int nthreads, fgpu_amg_host** out) {
    if (!out || n < 0 || (n > 0 && (!ia || !ja || !a))) return FGPU_ERR_INVALID;
    *out = nullptr;
    fgpu::HostCsr A;
    A.nrows = A.ncols = n;
    A.ia.assign(ia, ia + n + 1);
    A.ja.assign(ja, ja + ia[n]);
    A.a.assign(a, a + ia[n]);
    const fgpu::AmgHostCfg hc = fgpu::amg_host_cfg(cfg, nthreads);
    fgpu::AmgNns nns;
    if (cfg && cfg->nns_count > 0) {
        if (!cfg->nns_host || fgpu::amg_nns_layout(cfg, n, nns)) return FGPU_ERR_INVALID;
        for (int64_t i = 0; i < n; ++i)
            for (int j = 0; j < nns.m; ++j) nns.B[(size_t)i * nns.m + j] = cfg->nns_host[(size_t)j * n + i];
    }
    fgpu_amg_host* h = new fgpu_amg_host();
    std::string err;
    if (!fgpu::amg_build_host(std::move(A), hc, h->H, err, nns.m ? &nns : nullptr)) {
        delete h;
        return FGPU_ERR_INVALID;
    }
    *out = h;
    return FGPU_OK;
}

extern "C" int fgpu_amg_host_levels(const fgpu_amg_host* h) { return h ? (int)h->H.levels.size() : 0; }

extern "C" int fgpu_amg_host_device_levels(const fgpu_amg_host* h) { return h ? h->device_levels : 0; }

extern "C" int fgpu_amg_host_level(const fgpu_amg_host* h, int l, int64_t* n, int64_t* nnz, int64_t* p_nnz, int64_t* p_cols,
                                   double* lmax) {
    if (!h || l < 0 || l >= (int)h->H.levels.size()) return FGPU_ERR_INVALID;
    const fgpu::AmgHostLevel& L = h->H.levels[l];
    if (n) *n = L.A.nrows;
    if (nnz) *nnz = (int64_t)L.A.ja.size();
    if (p_nnz) *p_nnz = (int64_t)L.P.ja.size();
    if (p_cols) *p_cols = L.P.ncols;
    if (lmax) *lmax = L.lmax;
    return FGPU_OK;
}

extern "C" int fgpu_amg_host_export(const fgpu_amg_host* h, int l, int64_t* ia, int32_t* ja, double* a, int64_t* pia, int32_t* pja,
                                    double* pa, int32_t* agg) {
    if (!h || l < 0 || l >= (int)h->H.levels.size()) return FGPU_ERR_INVALID;
    const fgpu::AmgHostLevel& L = h->H.levels[l];
    if (ia) std::copy(L.A.ia.begin(), L.A.ia.end(), ia);
    if (ja) std::copy(L.A.ja.begin(), L.A.ja.end(), ja);
    if (a) std::copy(L.A.a.begin(), L.A.a.end(), a);
    if (pia) std::copy(L.P.ia.begin(), L.P.ia.end(), pia);
    if (pja) std::copy(L.P.ja.begin(), L.P.ja.end(), pja);
    if (pa) std::copy(L.P.a.begin(), L.P.a.end(), pa);
    if (agg) std::copy(L.agg.begin(), L.agg.end(), agg);
    return FGPU_OK;
}

extern "C" int fgpu_amg_host_coarse_inverse(const fgpu_amg_host* h, double* out) {
    if (!h) return FGPU_ERR_INVALID;
    if (h->H.coarse_inv.empty()) return 0;
    if (out) std::copy(h->H.coarse_inv.begin(), h->H.coarse_inv.end(), out);
    return 1;
}

extern "C" int fgpu_amg_host_destroy(fgpu_amg_host* h) {
    delete h;
    return FGPU_OK;
}
