// ============================================================================
// ORACLE — test infrastructure only.
//
// A plain C++ CPU restatement of the Feel++ assembly path (form2/form1 over
// elements(mesh), on(), backend()->solve with CG+Jacobi) for Lagrange Pch/Pchv
// P1..P3 on affine tetrahedra. Only tests/, __graft_entry__.smoke() and the
// CPU-baseline leg of bench.py may load this library, and only as the checker
// or the timed CPU baseline. The product (feelpp_gb300) never links it.
//
// The reference itself cannot be built here (no PETSc/Boost/Eigen/MPI/GiNaC),
// so each function below restates the reference algorithm and cites the file
// and lines it follows (paths relative to the Feel++ source tree).
//
// Parity status: per-entry values are pinned by the restated algorithm plus
// the reference's own property tests (quadrature exactness, Lagrange
// Kronecker property, form energies); the Eigen 3x3 inverse and the PETSc
// MatSetValues/MatZeroRows/KSPCG boundaries are restated from their published
// semantics.
// ============================================================================
#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <map>
#include <set>
#include <tuple>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "quad_tables.h"

namespace {

using std::vector;
typedef std::complex<double> cplx;

// ---------------------------------------------------------------------------
// Reference tetrahedron and its entity tables
// feelpp/feel/feelmesh/refsimplex.hpp:151-165 (vertices),
// feelpp/feel/feelmesh/simplexordering.hpp:284-293 (e2p), :341-347 (f2p).
// ---------------------------------------------------------------------------
const double kRefV[4][3] = {{-1, -1, -1}, {1, -1, -1}, {-1, 1, -1}, {-1, -1, 1}};
const int kE2P[6][2] = {{1, 2}, {2, 0}, {0, 1}, {0, 3}, {1, 3}, {2, 3}};
const int kF2P[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};

int nloc_of(int order) { return (order + 1) * (order + 2) * (order + 3) / 6; }
int ndpe_of(int order) { return order - 1; }                                  // dofs per edge
int ndpf_of(int order) { return order >= 3 ? (order - 1) * (order - 2) / 2 : 0; }  // dofs per face
int ndpv_of(int order) { return order >= 4 ? (order - 1) * (order - 2) * (order - 3) / 6 : 0; }

// ---------------------------------------------------------------------------
// Small dense helpers (row-major).
// ---------------------------------------------------------------------------
struct Mat {
    int r = 0, c = 0;
    vector<double> a;
    Mat() {}
    Mat(int r_, int c_, double v = 0) : r(r_), c(c_), a((size_t)r_ * c_, v) {}
    double& operator()(int i, int j) { return a[(size_t)i * c + j]; }
    double operator()(int i, int j) const { return a[(size_t)i * c + j]; }
};

Mat matmul(const Mat& A, const Mat& B) {
    Mat C(A.r, B.c);
    for (int i = 0; i < A.r; ++i)
        for (int k = 0; k < A.c; ++k)
            for (int j = 0; j < B.c; ++j) C(i, j) += A(i, k) * B(k, j);
    return C;
}

// Gaussian elimination with partial pivoting: solves A X = B in place (B gets X).
// Restates the LU solve used by feelpp/feel/feelalg/lu.hpp (Doolittle + pivoting).
bool lu_solve(Mat A, Mat& B) {
    int n = A.r;
    for (int k = 0; k < n; ++k) {
        int p = k;
        for (int i = k + 1; i < n; ++i)
            if (std::fabs(A(i, k)) > std::fabs(A(p, k))) p = i;
        if (A(p, k) == 0.0) return false;
        if (p != k) {
            for (int j = 0; j < n; ++j) std::swap(A(k, j), A(p, j));
            for (int j = 0; j < B.c; ++j) std::swap(B(k, j), B(p, j));
        }
        for (int i = k + 1; i < n; ++i) {
            double f = A(i, k) / A(k, k);
            for (int j = k; j < n; ++j) A(i, j) -= f * A(k, j);
            for (int j = 0; j < B.c; ++j) B(i, j) -= f * B(k, j);
        }
    }
    for (int k = n - 1; k >= 0; --k)
        for (int j = 0; j < B.c; ++j) {
            double s = B(k, j);
            for (int i = k + 1; i < n; ++i) s -= A(k, i) * B(i, j);
            B(k, j) = s / A(k, k);
        }
    return true;
}

// ---------------------------------------------------------------------------
// Jacobi polynomials, Gauss-Lobatto points.
// feelpp/feel/feelpoly/jacobi.hpp:657-690 (dyna::JacobiBatchEvaluation, the
// three-term recurrence), :700-760 (roots: Newton from Chebyshev guesses with
// deflation), :905-960 (dyna::gausslobattojacobi).
// ---------------------------------------------------------------------------
template <typename S>
void jacobi_all(int N, double a, double b, S x, S* out) {
    out[0] = S(1.0);
    if (N == 0) return;
    out[1] = 0.5 * (S(a - b) + (a + b + 2.0) * x);
    double apb = a + b;
    for (int k = 2; k <= N; ++k) {
        double kv = k;
        double a1 = 2.0 * kv * (kv + apb) * (2.0 * kv + apb - 2.0);
        double a2 = (2.0 * kv + apb - 1.0) * (a * a - b * b);
        double a3 = (2.0 * kv + apb - 2.0) * (2.0 * kv + apb - 1.0) * (2.0 * kv + apb);
        double a4 = 2.0 * (kv + a - 1.0) * (kv + b - 1.0) * (2.0 * kv + apb);
        a2 /= a1; a3 /= a1; a4 /= a1;
        out[k] = a2 * out[k - 1] + a3 * x * out[k - 1] - a4 * out[k - 2];
    }
}
double jacobi_val(int N, double a, double b, double x) {
    double t[32];
    jacobi_all<double>(N, a, b, x, t);
    return t[N];
}
double jacobi_der(int N, double a, double b, double x) {
    // d/dx P_N^{a,b} = 0.5 (a+b+N+1) P_{N-1}^{a+1,b+1}   (jacobi.hpp:575-590)
    if (N == 0) return 0.0;
    return 0.5 * (a + b + N + 1.0) * jacobi_val(N - 1, a + 1.0, b + 1.0, x);
}

// Gauss-Lobatto nodes (ascending), N points.
vector<double> gll_nodes(int N) {
    vector<double> xr(N);
    xr[0] = -1.0;
    xr[N - 1] = 1.0;
    int m = N - 2;  // interior: roots of P_{N-2}^{1,1}
    vector<double> r(m);
    const double eps = 2.220446049250313e-16;
    for (int k = 0; k < m; ++k) {
        double pi = 4.0 * std::atan(1.0);
        double x = -std::cos((2.0 * k + 1.0) * pi / (2.0 * m));
        if (k > 0) x = 0.5 * (x + r[k - 1]);
        for (int it = 0; it < 30; ++it) {
            double s = 0;
            for (int i = 0; i < k; ++i) s += 1.0 / (x - r[i]);
            double jf = jacobi_val(m, 1.0, 1.0, x);
            double jdf = jacobi_der(m, 1.0, 1.0, x);
            double delta = jf / (jdf - jf * s);
            x -= delta;
            if (std::fabs(delta) <= eps) break;
        }
        r[k] = x;
    }
    for (int i = 0; i < m; ++i) xr[i + 1] = r[i];
    return xr;
}

// ---------------------------------------------------------------------------
// Lagrange node set on the reference tetrahedron.
// Equispaced construction: feelpp/feel/feelpoly/equispaced.hpp:118-145
// (vertices, then edges 0..5, faces 0..3, interior), :480-560 (lattices),
// :700-730 (pt_to_edge / pt_to_face maps).
// 3D warp & blend (PointSetFekete -> PointSetWarpBlend for 3D simplices,
// feelpp/feel/feelpoly/fekete.hpp:1251-1262): feelpp/feel/feelpoly/
// warpblend.hpp:70-135 (only edge points are warped for Order 3, faces too
// for Order >= 4), :146-206, :218-300, :304-348, :351-440.
// ---------------------------------------------------------------------------
typedef vector<std::array<double, 3>> Pts;

Pts equispaced_nodes(int order) {
    Pts P;
    for (int v = 0; v < 4; ++v) P.push_back({kRefV[v][0], kRefV[v][1], kRefV[v][2]});
    if (order == 1) return P;
    for (int e = 0; e < 6; ++e) {
        const double* u = kRefV[kE2P[e][0]];
        const double* w = kRefV[kE2P[e][1]];
        for (int i = 1; i < order; ++i) {
            double x = -1.0 + 2.0 * i / order;  // line lattice on [-1,1]
            double t = 0.5 * (x + 1.0);
            P.push_back({u[0] + t * (w[0] - u[0]), u[1] + t * (w[1] - u[1]), u[2] + t * (w[2] - u[2])});
        }
    }
    for (int f = 0; f < 4; ++f) {
        const double* u = kRefV[kF2P[f][0]];
        const double* v = kRefV[kF2P[f][1]];
        const double* w = kRefV[kF2P[f][2]];
        // interior points of the triangle lattice: i over h1 (v2-v0), j over h0 (v1-v0)
        for (int i = 1; i < order; ++i)
            for (int j = 1; j < order - i; ++j) {
                double X = -1.0 + 2.0 * j / order, Y = -1.0 + 2.0 * i / order;
                double s = 0.5 * (X + 1.0), t = 0.5 * (Y + 1.0);
                P.push_back({u[0] + s * (v[0] - u[0]) + t * (w[0] - u[0]),
                             u[1] + s * (v[1] - u[1]) + t * (w[1] - u[1]),
                             u[2] + s * (v[2] - u[2]) + t * (w[2] - u[2])});
            }
    }
    // interior (tetrahedron lattice, interior == 1)
    for (int i = 1; i < order; ++i)
        for (int j = 1; j < order - i; ++j)
            for (int k = 1; k < order - i - j; ++k) {
                double a = double(i) / order, b = double(j) / order, c = double(k) / order;
                P.push_back({-1 + 2 * c, -1 + 2 * b, -1 + 2 * a});
            }
    return P;
}

struct WarpBlend3D {
    int order;
    Mat Vref, Veq;  // 3x4 vertex matrices (columns = vertices)
    std::map<int, std::pair<std::array<double, 3>, std::array<double, 3>>> axis;

    explicit WarpBlend3D(int o) : order(o), Vref(3, 4), Veq(3, 4) {
        for (int v = 0; v < 4; ++v)
            for (int d = 0; d < 3; ++d) Vref(d, v) = kRefV[v][d];
        // equiVertices (warpblend.hpp:146-168)
        const double pi = M_PI;
        for (int i = 0; i < 3; ++i) {
            double angle = pi * (7.0 + 4.0 * i) / 6.0;
            Veq(0, i) = std::cos(angle);
            Veq(1, i) = std::sin(angle);
            Veq(2, i) = -std::sqrt(2.0) / 4.0;
        }
        for (int i = 0; i < 3; ++i)
            for (int v = 0; v < 4; ++v) Veq(i, v) *= 2.0 / std::sqrt(3.0);
        Veq(2, 3) = std::sqrt(6.0) / 2.0;
        blend_axis();
    }
    std::array<double, 3> vtx(int which, int i) const {
        const Mat& M = which == 0 ? Vref : Veq;
        return {M(0, i), M(1, i), M(2, i)};
    }
    // blendAxis (warpblend.hpp:170-190)
    void blend_axis() {
        for (int i = 0; i < 4; ++i) {
            vector<int> idx;
            for (int j = 0; j < 4; ++j)
                if (j != (18 + i * (-6 + (i - 1) * (-3 + 4 * (i - 2)))) / 6) idx.push_back(j);
            auto v0 = vtx(1, idx[0]), v1 = vtx(1, idx[1]), v2 = vtx(1, idx[2]);
            std::array<double, 3> f, s;
            for (int d = 0; d < 3; ++d) {
                f[d] = v1[d] - v0[d];
                s[d] = v2[d] - (v1[d] + v0[d]) / 2.0;
            }
            double nf = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
            double ns = std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
            for (int d = 0; d < 3; ++d) { f[d] /= nf; s[d] /= ns; }
            axis[i] = {f, s};
        }
    }
    // entityMap (warpblend.hpp:193-210)
    static int entity_map(int top_dim, int id) {
        if (top_dim == 2) return (12 + id * (6 + (id - 1) * (-9 + 4 * (id - 2)))) / 6;
        if (id == 5) return 2;
        if (id > 2) return 1;
        return 0;
    }
    // toEquilateral (warpblend.hpp:222-262): affine map reference <-> equilateral
    Mat to_equilateral(Mat pts, bool to_equi) const {
        Mat Cr(3, 3), Ce(3, 3);
        for (int i = 0; i < 3; ++i)
            for (int d = 0; d < 3; ++d) {
                Cr(d, i) = Vref(d, 3) - Vref(d, i);
                Ce(d, i) = Veq(d, 3) - Veq(d, i);
            }
        Mat Crinv(3, 3);
        for (int i = 0; i < 3; ++i) Crinv(i, i) = 1.0;
        lu_solve(Cr, Crinv);
        Mat A = matmul(Ce, Crinv);
        std::array<double, 3> b;
        for (int d = 0; d < 3; ++d) {
            double s = 0;
            for (int k = 0; k < 3; ++k) s += A(d, k) * Vref(k, 0);
            b[d] = Veq(d, 0) - s;
        }
        if (to_equi) {
            Mat R = matmul(A, pts);
            for (int j = 0; j < R.c; ++j)
                for (int d = 0; d < 3; ++d) R(d, j) += b[d];
            return R;
        }
        for (int j = 0; j < pts.c; ++j)
            for (int d = 0; d < 3; ++d) pts(d, j) -= b[d];
        lu_solve(A, pts);
        return pts;
    }
    // toBarycentric (warpblend.hpp:264-292): returns a 4 x npts matrix
    Mat to_barycentric(Mat pts) const {
        Mat C(3, 3);
        for (int i = 0; i < 3; ++i) {
            int k = (3 - 3 % 2 + i) % 3;
            for (int d = 0; d < 3; ++d) C(d, i) = Veq(d, k) - Veq(d, 3);
        }
        for (int j = 0; j < pts.c; ++j)
            for (int d = 0; d < 3; ++d) pts(d, j) -= Veq(d, 3);
        lu_solve(C, pts);
        Mat R(4, pts.c);
        for (int j = 0; j < pts.c; ++j) {
            R(0, j) = 1.0;
            for (int i = 1; i < 4; ++i) {
                R(i, j) = pts(i - 1, j);
                R(0, j) -= R(i, j);
            }
        }
        return R;
    }
    double alpha(int d) const {
        static const double a2[16] = {0, 0, 0, 1.4152, 0.1001, 0.2751, 0.9808, 1.0999,
                                      1.2832, 1.3648, 1.4773, 1.4959, 1.5743, 1.5770, 1.6223, 1.6258};
        static const double a3[16] = {0, 0, 0, 0, 0.1002, 1.1332, 1.5608, 1.3413,
                                      1.2577, 1.1603, 1.0153, 0.6080, 0.4523, 0.8856, 0.8717, 0.9655};
        if (d == 2) return order <= 15 ? a2[order] : 5.0 / 3.0;
        return order <= 15 ? a3[order] : 1.0;
    }
    // warpFactor (warpblend.hpp:330-356)
    vector<double> warp_factor(const vector<double>& x, const vector<double>& xout) const {
        int n1 = order + 1;
        vector<double> warp(xout.size(), 0.0), xeq(n1);
        for (int i = 0; i < n1; ++i) xeq[i] = -1.0 + 2.0 * i / order;
        for (int i = 0; i < n1; ++i) {
            vector<double> d(xout.size(), x[i] - xeq[i]);
            for (int j = 1; j < n1 - 1; ++j)
                if (i != j)
                    for (size_t l = 0; l < d.size(); ++l) d[l] = (d[l] * xout[l] - d[l] * xeq[j]) / (xeq[i] - xeq[j]);
            if (i != 0)
                for (auto& v : d) v *= -1.0 / (xeq[i] - xeq[0]);
            if (i != n1 - 1)
                for (auto& v : d) v *= 1.0 / (xeq[i] - xeq[n1 - 1]);
            for (size_t l = 0; l < d.size(); ++l) warp[l] += d[l];
        }
        return warp;
    }
    // getCoordinates (warpblend.hpp:359-382)
    static Mat get_coordinates(const Mat& pts, int face_id) {
        std::map<int, vector<int>> faces;
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j)
                if (j != i) faces[i].push_back(j);
        for (int i = 2; i < 4; ++i) {
            faces[i][1] = faces[i][2];
            faces[i][2] = 1;
        }
        Mat c(3, pts.c);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < pts.c; ++j) c(i, j) = pts(faces[face_id][i], j);
        return c;
    }
    // 2D face deformation (warpblend.hpp:384-415)
    Mat face_deformation_2d(const Mat& cb) const {
        int n = cb.c;
        Mat blend(3, n), wf(3, n), warp(3, n), def(2, n);
        vector<double> g = gll_nodes(order + 1);
        for (int i = 0; i < 3; ++i) {
            vector<double> r(n);
            for (int j = 0; j < n; ++j) {
                blend(i, j) = 4.0 * cb((i + 1) % 3, j) * cb((i + 2) % 3, j);
                r[j] = cb((i + 2) % 3, j) - cb((i + 1) % 3, j);
            }
            vector<double> w = warp_factor(g, r);
            for (int j = 0; j < n; ++j) wf(i, j) = w[j];
        }
        double a = alpha(2);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < n; ++j) warp(i, j) = blend(i, j) * wf(i, j) * (1.0 + a * a * cb(i, j) * cb(i, j));
        for (int i = 0; i < 3; ++i) {
            double angle = 2.0 * i * M_PI / 3.0;
            for (int j = 0; j < n; ++j) {
                def(0, j) += std::cos(angle) * warp(i, j);
                def(1, j) += std::sin(angle) * warp(i, j);
            }
        }
        return def;
    }
    // face deformation mapped into 3D (warpblend.hpp:418-432)
    Mat face_deformation_3d(const Mat& bary, int face_id) const {
        Mat cb = get_coordinates(bary, face_id);
        Mat def = face_deformation_2d(cb);
        Mat w(3, bary.c);
        const auto& ax = axis.at(face_id);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < bary.c; ++j) w(i, j) = ax.first[i] * def(0, j) + ax.second[i] * def(1, j);
        return w;
    }
    Pts nodes() const {
        Pts P = equispaced_nodes(order);
        if (order <= 2) return P;
        // Order 3: max_entity_dim = 1 (edges); Order >= 4 would also warp faces
        // and the interior, which this path does not use.
        int ne = order - 1;
        for (int e = 0; e < 6; ++e) {
            Mat pts(3, ne);
            for (int l = 0; l < ne; ++l)
                for (int d = 0; d < 3; ++d) pts(d, l) = P[4 + e * ne + l][d];
            Mat eq = to_equilateral(pts, true);
            Mat bary = to_barycentric(eq);
            Mat w = face_deformation_3d(bary, entity_map(1, e));
            for (int j = 0; j < eq.c; ++j)
                for (int d = 0; d < 3; ++d) eq(d, j) += w(d, j);
            Mat back = to_equilateral(eq, false);
            for (int l = 0; l < ne; ++l)
                for (int d = 0; d < 3; ++d) P[4 + e * ne + l][d] = back(d, l);
        }
        return P;
    }
};

Pts lagrange_nodes(int order) {
    if (order <= 2) return equispaced_nodes(order);
    return WarpBlend3D(order).nodes();
}

// ---------------------------------------------------------------------------
// Orthonormal Dubiner basis on the reference tetrahedron.
// feelpp/feel/feelpoly/dubiner.hpp:673-735 (evaluate<3>: collapsed coordinates,
// Jacobi products, scalings and the sqrt((i+1/2)(i+j+1)(i+j+k+3/2)) norm).
// Templated on the scalar so that gradients can be taken by complex-step
// differentiation (exact to rounding, no subtractive cancellation).
// ---------------------------------------------------------------------------
template <typename S>
void dubiner_eval(int N, S x, S y, S z, vector<S>& out) {
    // collapsed coordinates (feelpp/feel/feelpoly/expansiontypes? details::etas):
    // eta1 = 2(1+x)/(-y-z) - 1, eta2 = 2(1+y)/(1-z) - 1, eta3 = z,
    // with the removable singularities set to -1.
    S e1, e2, e3 = z;
    S d1 = -y - z, d2 = 1.0 - z;
    if (std::abs(d1) < 1e-300) e1 = S(-1.0); else e1 = 2.0 * (1.0 + x) / d1 - 1.0;
    if (std::abs(d2) < 1e-300) e2 = S(-1.0); else e2 = 2.0 * (1.0 + y) / d2 - 1.0;
    S s2 = 0.5 * (1.0 - e2), s3 = 0.5 * (1.0 - e3);
    vector<S> as(N + 1);
    jacobi_all<S>(N, 0.0, 0.0, e1, as.data());
    out.clear();
    for (int k = 0; k <= N; ++k)
        for (int i = 0; i <= k; ++i)
            for (int j = 0; j <= k - i; ++j) {
                int ii = k - i - j, jj = j, kk = i;
                vector<S> bs(N + 2), cs(N + 2);
                jacobi_all<S>(N - ii, 2.0 * ii + 1.0, 0.0, e2, bs.data());
                jacobi_all<S>(N - ii - jj, 2.0 * (ii + jj + 1), 0.0, e3, cs.data());
                S p2 = S(1.0), p3 = S(1.0);
                for (int t = 0; t < ii; ++t) p2 *= s2;
                for (int t = 0; t < ii + jj; ++t) p3 *= s3;
                double nrm = std::sqrt((ii + 0.5) * (ii + jj + 1.0) * (ii + jj + kk + 1.5));
                out.push_back(nrm * as[ii] * p2 * bs[jj] * p3 * cs[kk]);
            }
}

// Lagrange basis: the dual basis of point evaluations at the node set gives
// coefficients A = (V^T)^{-1}, V_kj = P_j(x_k)  (feelpp/feel/feelpoly/
// lagrange.hpp:303-330 and dualbasis.hpp; polynomialset.hpp:776-1080 for the
// tabulation at quadrature points, PreCompute).
struct LagrangeBasis {
    int order, n;
    Mat A;  // n x n : phi_i = sum_j A(i,j) P_j
    explicit LagrangeBasis(int o) : order(o), n(nloc_of(o)) {
        Pts P = lagrange_nodes(o);
        Mat VT(n, n);  // VT(j,k) = P_j(x_k)
        vector<double> vals;
        for (int k = 0; k < n; ++k) {
            dubiner_eval<double>(o, P[k][0], P[k][1], P[k][2], vals);
            for (int j = 0; j < n; ++j) VT(j, k) = vals[j];
        }
        // A VT = I  <=>  VT^T A^T = I
        Mat VTt(n, n), I(n, n);
        for (int i = 0; i < n; ++i) {
            I(i, i) = 1.0;
            for (int j = 0; j < n; ++j) VTt(i, j) = VT(j, i);
        }
        lu_solve(VTt, I);  // I now = A^T
        A = Mat(n, n);
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) A(i, j) = I(j, i);
    }
    void eval(const double* x, double* phi, double* dphi /* n x 3 or null */) const {
        vector<double> v;
        dubiner_eval<double>(order, x[0], x[1], x[2], v);
        for (int i = 0; i < n; ++i) {
            double s = 0;
            for (int j = 0; j < n; ++j) s += A(i, j) * v[j];
            phi[i] = s;
        }
        if (!dphi) return;
        const double h = 1e-30;
        for (int d = 0; d < 3; ++d) {
            cplx X(x[0]), Y(x[1]), Z(x[2]);
            if (d == 0) X += cplx(0, h);
            if (d == 1) Y += cplx(0, h);
            if (d == 2) Z += cplx(0, h);
            vector<cplx> vc;
            dubiner_eval<cplx>(order, X, Y, Z, vc);
            for (int i = 0; i < n; ++i) {
                double s = 0;
                for (int j = 0; j < n; ++j) s += A(i, j) * vc[j].imag() / h;
                dphi[i * 3 + d] = s;
            }
        }
    }
};

// Tabulation of a Lagrange basis at a quadrature rule (PreCompute).
struct Tab {
    int order, n, Q;
    vector<double> w, pts;   // Q, Q*3
    vector<double> phi;      // Q*n
    vector<double> dphi;     // Q*n*3
    vector<double> gphi;     // Q*4 (P1 geometric basis)
};

bool make_tab(int order, int qdeg, Tab& t) {
    if (qdeg < 1 || qdeg > 8) return false;
    t.order = order;
    LagrangeBasis L(order);
    t.n = L.n;
    t.Q = orc_quad_npts[qdeg];
    const double* q = orc_quad_tab[qdeg];
    t.w.resize(t.Q); t.pts.resize(t.Q * 3); t.phi.resize(t.Q * t.n); t.dphi.resize(t.Q * t.n * 3); t.gphi.resize(t.Q * 4);
    for (int k = 0; k < t.Q; ++k) {
        t.pts[3 * k] = q[4 * k]; t.pts[3 * k + 1] = q[4 * k + 1]; t.pts[3 * k + 2] = q[4 * k + 2];
        t.w[k] = q[4 * k + 3];
        L.eval(&t.pts[3 * k], &t.phi[k * t.n], &t.dphi[k * t.n * 3]);
        double x = t.pts[3 * k], y = t.pts[3 * k + 1], z = t.pts[3 * k + 2];
        t.gphi[4 * k + 0] = -0.5 * (1 + x + y + z);
        t.gphi[4 * k + 1] = 0.5 * (1 + x);
        t.gphi[4 * k + 2] = 0.5 * (1 + y);
        t.gphi[4 * k + 3] = 0.5 * (1 + z);
    }
    return true;
}

// ---------------------------------------------------------------------------
// Geometric map of an affine tetrahedron.
// feelpp/feel/feelpoly/geomap.hpp:2310-2350 (K = G * grad(phi_geo)),
// :1971-1991 (J = |det K|, B = (K^{-1})^T). The P1 geometric basis gradients on
// the reference element are (-1/2,-1/2,-1/2), (1/2,0,0), (0,1/2,0), (0,0,1/2).
// The 3x3 inverse is the cofactor formula (Eigen's compute_inverse<3x3>).
// ---------------------------------------------------------------------------
static void geomap_finish(const double K[9], double& J, double B[9], double& detK);

void geomap(const double* xyz, const int32_t* tet, double K[9], double& J, double B[9], double& detK) {
    const double g[4][3] = {{-0.5, -0.5, -0.5}, {0.5, 0, 0}, {0, 0.5, 0}, {0, 0, 0.5}};
    for (int i = 0; i < 9; ++i) K[i] = 0;
    for (int v = 0; v < 4; ++v) {
        const double* X = xyz + 3 * (int64_t)tet[v];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) K[3 * r + c] += X[r] * g[v][c];
    }
    geomap_finish(K, J, B, detK);
}

// Curved (P2) tetrahedra: x(xh) = sum_g X_g psi_g(xh) over the 10 P2 Lagrange
// functions (vertices, then edge midpoints in e2p order); at each quadrature
// point K = sum_g X_g (grad psi_g)^T, then J and B as for the affine map
// (feelpp/feel/feelpoly/geomap.hpp:2310-2350; the context recomputes K at every
// point when the map is not linear, :1014-1042).
static void geomap_ho(const double X[10][3], const double* dpsi /* 10 x 3 */, double K[9], double& J, double B[9],
                      double& detK) {
    for (int i = 0; i < 9; ++i) K[i] = 0;
    for (int g = 0; g < 10; ++g)
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) K[3 * r + c] += X[g][r] * dpsi[3 * g + c];
    geomap_finish(K, J, B, detK);
}

static void geomap_finish(const double K[9], double& J, double B[9], double& detK) {
    double c00 = K[4] * K[8] - K[5] * K[7];
    double c01 = K[5] * K[6] - K[3] * K[8];
    double c02 = K[3] * K[7] - K[4] * K[6];
    detK = K[0] * c00 + K[1] * c01 + K[2] * c02;
    J = std::fabs(detK);
    // Kinv(i,j) = cof(j,i)/det ; B = Kinv^T -> B(i,j) = cof(i,j)/det
    double cof[9] = {c00, c01, c02,
                     K[2] * K[7] - K[1] * K[8], K[0] * K[8] - K[2] * K[6], K[1] * K[6] - K[0] * K[7],
                     K[1] * K[5] - K[2] * K[4], K[2] * K[3] - K[0] * K[5], K[0] * K[4] - K[1] * K[3]};
    for (int i = 0; i < 9; ++i) B[i] = cof[i] / detK;
}

// ---------------------------------------------------------------------------
// Mesh entities and DOF table.
// Edges: feelpp/feel/feelmesh/mesh3d.hpp:700-782 (key = sorted point ids; the
// element's edge j is REVERSE-permuted when id(e2p[j][0]) > id(e2p[j][1])).
// Faces: mesh3d.hpp (updateEntitiesCoDimensionOne), key = sorted point ids.
// Numbering: feelpp/feel/feeldiscr/doftable.hpp:2364-2455 (element loop in
// insertion order), doffromelement.hpp:505-530 (vertex -> edge -> face ->
// volume), :163-336 (per-entity keys, reversed edge slots),
// doftable.hpp:1213-1250 (insertDof: first encounter gets next_free_dof,
// which then advances by nComponents), :1286-1300 (component c of a node
// is global dof base + c, local index nLocalDof*c + l).
// ---------------------------------------------------------------------------
struct VecHash {
    size_t operator()(const std::vector<int64_t>& v) const {
        size_t h = 1469598103934665603ull;
        for (auto x : v) { h ^= (size_t)x + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2); }
        return h;
    }
};

int64_t build_dof_table(int64_t T, const int32_t* tets, int order, int ncomp, int32_t* l2g) {
    const int nl = nloc_of(order);
    const int ndpe = ndpe_of(order), ndpf = ndpf_of(order), ndpv = ndpv_of(order);
    std::unordered_map<std::vector<int64_t>, int64_t, VecHash> edges, faces;
    // map_gdof: key (entity dim, entity-local gdof key) -> dof base
    std::map<std::tuple<int, int64_t>, int64_t> map_gdof;
    int64_t next_free = 0, next_edge = 0, next_face = 0;
    for (int64_t e = 0; e < T; ++e) {
        const int32_t* t = tets + 4 * e;
        int lc = 0;
        auto insert = [&](int dim, int64_t key) {
            auto it = map_gdof.find({dim, key});
            int64_t base;
            if (it == map_gdof.end()) {
                base = next_free;
                map_gdof.emplace(std::make_tuple(dim, key), base);
                next_free += ncomp;
            } else {
                base = it->second;
            }
            for (int c = 0; c < ncomp; ++c) l2g[e * (int64_t)nl * ncomp + (int64_t)nl * c + lc] = (int32_t)(base + c);
            ++lc;
        };
        // vertices
        for (int i = 0; i < 4; ++i) insert(0, (int64_t)t[i]);
        // edges
        for (int j = 0; j < 6; ++j) {
            int64_t i1 = t[kE2P[j][0]], i2 = t[kE2P[j][1]];
            std::vector<int64_t> key = {std::min(i1, i2), std::max(i1, i2)};
            auto it = edges.find(key);
            int64_t eid;
            if (it == edges.end()) { eid = next_edge++; edges.emplace(key, eid); }
            else eid = it->second;
            bool reverse = i1 > i2;
            for (int l = 0; l < ndpe; ++l) {
                int64_t g = eid * ndpe + (reverse ? ndpe - 1 - l : l);
                insert(1, g);
            }
        }
        // faces (1 dof per face for P3; the permutation does not matter then)
        for (int f = 0; f < 4; ++f) {
            std::vector<int64_t> key = {t[kF2P[f][0]], t[kF2P[f][1]], t[kF2P[f][2]]};
            std::sort(key.begin(), key.end());
            auto it = faces.find(key);
            int64_t fid;
            if (it == faces.end()) { fid = next_face++; faces.emplace(key, fid); }
            else fid = it->second;
            for (int l = 0; l < ndpf; ++l) insert(2, fid * ndpf + l);
        }
        for (int l = 0; l < ndpv; ++l) insert(3, e * ndpv + l);
    }
    return next_free;
}

}  // namespace

extern "C" {

int orc_version() { return 1; }

// Quadrature rule of degree `deg`; writes npts*(x,y,z,w) if out != null, returns npts.
int orc_quad(int deg, double* out) {
    if (deg < 1 || deg > 8) return -1;
    int n = orc_quad_npts[deg];
    if (out) std::memcpy(out, orc_quad_tab[deg], sizeof(double) * 4 * n);
    return n;
}

// Lagrange node set (reference coordinates), nloc x 3; returns nloc.
int orc_nodes(int order, double* out) {
    if (order < 1 || order > 3) return -1;
    Pts P = lagrange_nodes(order);
    for (size_t i = 0; i < P.size(); ++i)
        for (int d = 0; d < 3; ++d) out[3 * i + d] = P[i][d];
    return (int)P.size();
}

// Gauss-Lobatto points (ascending) for n points.
int orc_gll(int n, double* out) {
    if (n < 2 || n > 20) return -1;
    auto g = gll_nodes(n);
    for (int i = 0; i < n; ++i) out[i] = g[i];
    return n;
}

// Lagrange basis values (npts x nloc) and reference gradients (npts x nloc x 3).
int orc_tabulate(int order, int npts, const double* pts, double* phi, double* dphi) {
    if (order < 1 || order > 3) return -1;
    LagrangeBasis L(order);
    for (int k = 0; k < npts; ++k) L.eval(pts + 3 * k, phi + (size_t)k * L.n, dphi ? dphi + (size_t)k * L.n * 3 : nullptr);
    return L.n;
}

// DOF table: l2g (T x nloc*ncomp, local index nloc*c + l). Returns N or -1.
int64_t orc_dof_table(int64_t T, const int32_t* tets, int order, int ncomp, int32_t* l2g) {
    if (order < 1 || order > 3 || ncomp < 1) return -1;
    return build_dof_table(T, tets, order, ncomp, l2g);
}

// Sparsity pattern (COUPLED, diag_is_nonzero): feelpp/feel/feeldiscr/
// stencil.hpp:1500-1692 (row(ig).insert(sorted element dofs) as std::set),
// feelpp/feel/feelalg/graphcsr.cpp:634-660 (addMissingZeroEntriesDiagonal),
// :990-1020 (close: ia running counts, ja = concatenated sorted sets).
// Two calls: ja == null fills ia (N+1) only; then ja (ia[N]) is filled.
int orc_pattern(int64_t N, int64_t T, int nle, const int32_t* l2g, int64_t* ia, int32_t* ja) {
    vector<std::set<int32_t>> rows(N);
    for (int64_t e = 0; e < T; ++e) {
        vector<int32_t> d(l2g + e * nle, l2g + (e + 1) * nle);
        std::sort(d.begin(), d.end());
        for (int i = 0; i < nle; ++i) rows[l2g[e * nle + i]].insert(d.begin(), d.end());
    }
    for (int64_t r = 0; r < N; ++r) rows[r].insert((int32_t)r);
    ia[0] = 0;
    for (int64_t r = 0; r < N; ++r) ia[r + 1] = ia[r] + (int64_t)rows[r].size();
    if (ja)
        for (int64_t r = 0; r < N; ++r) {
            int64_t p = ia[r];
            for (auto c : rows[r]) ja[p++] = c;
        }
    return 0;
}

// Per-element J = |det K| and B = K^{-T} (row-major 3x3).
int orc_geometry(const double* xyz, int64_t T, const int32_t* tets, double* J, double* B, double* detK) {
    for (int64_t e = 0; e < T; ++e) {
        double K[9], Bl[9], j, d;
        geomap(xyz, tets + 4 * e, K, j, Bl, d);
        if (J) J[e] = j;
        if (detK) detK[e] = d;
        if (B) std::memcpy(B + 9 * e, Bl, sizeof(Bl));
    }
    return 0;
}

// Element-colouring used by the multi-threaded CPU baseline: greedy, elements
// sharing a vertex get different colours (the reference's TBB path instead
// serialises the scatter with a mutex, feelpp/feel/feelvf/integrator.hpp:605-621).
static int colour_elements(int64_t V, int64_t T, const int32_t* tets, vector<int>& col) {
    vector<uint64_t> used(V, 0);
    col.assign(T, 0);
    int nc = 0;
    for (int64_t e = 0; e < T; ++e) {
        uint64_t m = 0;
        for (int i = 0; i < 4; ++i) m |= used[tets[4 * e + i]];
        int c = 0;
        while (c < 64 && (m >> c & 1)) ++c;
        if (c == 64) return -1;
        col[e] = c;
        nc = std::max(nc, c + 1);
        for (int i = 0; i < 4; ++i) used[tets[4 * e + i]] |= (1ull << c);
    }
    return nc;
}

// Bilinear form assembly into a CSR with a fixed pattern.
// kind 0: kappa * inner(gradt(u), grad(v)) + mass * idt(u) * id(v)   (scalar)
// kind 1: inner(sigma(u), grad(v)), sigma = lambda tr(eps) I + 2 mu eps  (vector, ncomp 3)
// Element loop: feelpp/feel/feelvf/integrator.hpp:975-1238; local matrix
// K_e(i,j) = sum_q w_q J * evalijq(i,j,q): bilinearformcontext.hpp:552-590 and
// pointsetquadrature.hpp:403-416 (M_prod[q] = w_q J, pointsetquadrature.hpp:481-495);
// physical gradients grad phi_i(q) = B * ghat phi_i(q): polynomialset_impl.hpp:278-305;
// scatter: bilinearformcontext.hpp:784-847 -> MatrixPetsc::addMatrix
// (matrixpetsc.cpp:919-935, MatSetValues ADD_VALUES, row-major block, each
// column found by a search of the sorted row).
// kappa: per-element array (T) or null -> kappa_const. nthreads > 1 runs the
// element colours in parallel (timing only; the sequential order is the
// reference's summation order).
int orc_assemble(int order, int ncomp, int qdeg, const double* xyz, int64_t T, const int32_t* tets,
                 const int32_t* l2g, int kind, const double* kappa, double kappa_const, double mass,
                 double lam, double mu, int64_t N, const int64_t* ia, const int32_t* ja, double* val,
                 int nthreads, int64_t V) {
    Tab tab;
    if (!make_tab(order, qdeg, tab)) return -1;
    const int n = tab.n, Q = tab.Q, nle = n * ncomp;
    if (kind == 1 && ncomp != 3) return -2;
    auto element = [&](int64_t e, vector<double>& Ke, vector<double>& gp) {
        double K[9], B[9], J, d;
        geomap(xyz, tets + 4 * e, K, J, B, d);
        double kap = kappa ? kappa[e] : kappa_const;
        std::fill(Ke.begin(), Ke.end(), 0.0);
        for (int q = 0; q < Q; ++q) {
            double wJ = tab.w[q] * J;
            for (int i = 0; i < n; ++i) {
                const double* gh = &tab.dphi[(size_t)(q * n + i) * 3];
                for (int r = 0; r < 3; ++r) gp[i * 3 + r] = B[3 * r] * gh[0] + B[3 * r + 1] * gh[1] + B[3 * r + 2] * gh[2];
            }
            const double* ph = &tab.phi[(size_t)q * n];
            if (kind == 0) {
                for (int i = 0; i < n; ++i)
                    for (int j = 0; j < n; ++j) {
                        double g = gp[j * 3] * gp[i * 3] + gp[j * 3 + 1] * gp[i * 3 + 1] + gp[j * 3 + 2] * gp[i * 3 + 2];
                        Ke[(size_t)i * nle + j] += wJ * (kap * g + mass * ph[j] * ph[i]);
                    }
            } else {
                for (int c = 0; c < 3; ++c)
                    for (int i = 0; i < n; ++i)
                        for (int dd = 0; dd < 3; ++dd)
                            for (int j = 0; j < n; ++j) {
                                const double* gi = &gp[i * 3];
                                const double* gj = &gp[j * 3];
                                double v = lam * gj[dd] * gi[c] + mu * gj[c] * gi[dd];
                                if (c == dd) v += mu * (gj[0] * gi[0] + gj[1] * gi[1] + gj[2] * gi[2]);
                                Ke[(size_t)(n * c + i) * nle + (n * dd + j)] += wJ * v;
                            }
            }
        }
    };
    auto scatter = [&](int64_t e, const vector<double>& Ke) {
        const int32_t* rows = l2g + e * nle;
        for (int i = 0; i < nle; ++i) {
            int64_t r = rows[i];
            const int32_t* b = ja + ia[r];
            const int32_t* en = ja + ia[r + 1];
            for (int j = 0; j < nle; ++j) {
                const int32_t* p = std::lower_bound(b, en, rows[j]);
                val[p - ja] += Ke[(size_t)i * nle + j];
            }
        }
    };
    if (nthreads <= 1) {
        vector<double> Ke((size_t)nle * nle), gp(n * 3);
        for (int64_t e = 0; e < T; ++e) {
            element(e, Ke, gp);
            scatter(e, Ke);
        }
        return 0;
    }
#ifdef _OPENMP
    vector<int> col;
    int nc = colour_elements(V, T, tets, col);
    if (nc < 0) return -3;
    vector<vector<int64_t>> bycol(nc);
    for (int64_t e = 0; e < T; ++e) bycol[col[e]].push_back(e);
#pragma omp parallel num_threads(nthreads)
    {
        vector<double> Ke((size_t)nle * nle), gp(n * 3);
        for (int c = 0; c < nc; ++c) {
            const auto& L = bycol[c];
#pragma omp for schedule(static)
            for (int64_t k = 0; k < (int64_t)L.size(); ++k) {
                element(L[k], Ke, gp);
                scatter(L[k], Ke);
            }
        }
    }
    return 0;
#else
    return -4;
#endif
}

// Load vector: F_e(i) = sum_q w_q J f(x_q) phi_i(q); linearformcontext.hpp:305,
// scatter linearformcontext.hpp:395-410 -> VecSetValues ADD_VALUES
// (vectorpetsc.cpp:179-189). x_q = sum_v x_v phi_geo_v(q) (geomap.hpp:1965-1969).
// fkind 0: f = 3 pi^2 sin(pi x) sin(pi y) sin(pi z) (scalar);
// fkind 1: constant vector (fc[0], fc[1], fc[2]) (ncomp = 3);
// fkind 2: constant scalar fc[0].
int orc_rhs(int order, int ncomp, int qdeg, const double* xyz, int64_t T, const int32_t* tets,
            const int32_t* l2g, int fkind, const double* fc, double* F) {
    Tab tab;
    if (!make_tab(order, qdeg, tab)) return -1;
    const int n = tab.n, Q = tab.Q, nle = n * ncomp;
    vector<double> Fe(nle);
    for (int64_t e = 0; e < T; ++e) {
        double K[9], B[9], J, d;
        geomap(xyz, tets + 4 * e, K, J, B, d);
        std::fill(Fe.begin(), Fe.end(), 0.0);
        for (int q = 0; q < Q; ++q) {
            double X[3] = {0, 0, 0};
            for (int v = 0; v < 4; ++v)
                for (int r = 0; r < 3; ++r) X[r] += xyz[3 * (int64_t)tets[4 * e + v] + r] * tab.gphi[4 * q + v];
            double wJ = tab.w[q] * J;
            const double* ph = &tab.phi[(size_t)q * n];
            for (int c = 0; c < ncomp; ++c) {
                double f;
                if (fkind == 0) f = 3.0 * M_PI * M_PI * std::sin(M_PI * X[0]) * std::sin(M_PI * X[1]) * std::sin(M_PI * X[2]);
                else if (fkind == 1) f = fc[c];
                else f = fc[0];
                for (int i = 0; i < n; ++i) Fe[n * c + i] += wJ * f * ph[i];
            }
        }
        for (int i = 0; i < nle; ++i) F[l2g[e * nle + i]] += Fe[i];
    }
    return 0;
}

// Scalar Laplace/mass matrix and load vector on curved (P2-geometry) tetrahedra:
// ho = T x 6 x 3 coordinates of the edge nodes (e2p order). Same quadrature sums
// as orc_assemble / orc_rhs with the map evaluated per point.
static void element_nodes(const double* xyz, const int32_t* tet, const double* ho, double X[10][3]) {
    for (int v = 0; v < 4; ++v)
        for (int r = 0; r < 3; ++r) X[v][r] = xyz[3 * (int64_t)tet[v] + r];
    for (int j = 0; j < 6; ++j)
        for (int r = 0; r < 3; ++r) X[4 + j][r] = ho[3 * j + r];
}

int orc_assemble_ho(int order, int qdeg, const double* xyz, int64_t T, const int32_t* tets, const double* ho,
                    const int32_t* l2g, const double* kappa, double kappa_const, double mass, const int64_t* ia,
                    const int32_t* ja, double* val) {
    Tab tab, geo;
    if (!make_tab(order, qdeg, tab) || !make_tab(2, qdeg, geo)) return -1;
    const int n = tab.n, Q = tab.Q;
    vector<double> Ke((size_t)n * n), gp(n * 3);
    for (int64_t e = 0; e < T; ++e) {
        double X[10][3];
        element_nodes(xyz, tets + 4 * e, ho + 18 * e, X);
        const double kap = kappa ? kappa[e] : kappa_const;
        std::fill(Ke.begin(), Ke.end(), 0.0);
        for (int q = 0; q < Q; ++q) {
            double K[9], B[9], J, d;
            geomap_ho(X, &geo.dphi[(size_t)q * 10 * 3], K, J, B, d);
            const double wJ = tab.w[q] * J;
            for (int i = 0; i < n; ++i) {
                const double* gh = &tab.dphi[(size_t)(q * n + i) * 3];
                for (int r = 0; r < 3; ++r) gp[i * 3 + r] = B[3 * r] * gh[0] + B[3 * r + 1] * gh[1] + B[3 * r + 2] * gh[2];
            }
            const double* ph = &tab.phi[(size_t)q * n];
            for (int i = 0; i < n; ++i)
                for (int j = 0; j < n; ++j) {
                    double g = gp[j * 3] * gp[i * 3] + gp[j * 3 + 1] * gp[i * 3 + 1] + gp[j * 3 + 2] * gp[i * 3 + 2];
                    Ke[(size_t)i * n + j] += wJ * (kap * g + mass * ph[j] * ph[i]);
                }
        }
        const int32_t* rows = l2g + e * n;
        for (int i = 0; i < n; ++i) {
            const int32_t* b = ja + ia[rows[i]];
            const int32_t* en = ja + ia[rows[i] + 1];
            for (int j = 0; j < n; ++j) val[std::lower_bound(b, en, rows[j]) - ja] += Ke[(size_t)i * n + j];
        }
    }
    return 0;
}

int orc_rhs_ho(int order, int qdeg, const double* xyz, int64_t T, const int32_t* tets, const double* ho, const int32_t* l2g,
               int fkind, const double* fc, double* F) {
    Tab tab, geo;
    if (!make_tab(order, qdeg, tab) || !make_tab(2, qdeg, geo)) return -1;
    const int n = tab.n, Q = tab.Q;
    vector<double> Fe(n);
    for (int64_t e = 0; e < T; ++e) {
        double X[10][3];
        element_nodes(xyz, tets + 4 * e, ho + 18 * e, X);
        std::fill(Fe.begin(), Fe.end(), 0.0);
        for (int q = 0; q < Q; ++q) {
            double K[9], B[9], J, d;
            geomap_ho(X, &geo.dphi[(size_t)q * 10 * 3], K, J, B, d);
            double P[3] = {0, 0, 0};
            for (int g = 0; g < 10; ++g)
                for (int r = 0; r < 3; ++r) P[r] += X[g][r] * geo.phi[(size_t)q * 10 + g];
            const double f = fkind == 0 ? 3.0 * M_PI * M_PI * std::sin(M_PI * P[0]) * std::sin(M_PI * P[1]) * std::sin(M_PI * P[2])
                                        : fc[0];
            const double wJ = tab.w[q] * J;
            for (int i = 0; i < n; ++i) Fe[i] += wJ * f * tab.phi[(size_t)q * n + i];
        }
        for (int i = 0; i < n; ++i) F[l2g[e * n + i]] += Fe[i];
    }
    return 0;
}

// Boundary dofs: dofs carried by the boundary faces (faces owned by exactly
// one element), feelpp/feel/feelvf/on.hpp:457-701 (onFaces collects the face
// dofs: its vertices, edges and face interior). If `xplane_on` is set only
// faces whose three vertices have x <= xplane + 1e-12 are used (a marked
// "Dirichlet" face range). Writes a 0/1 mask of size N.
int orc_boundary_mask(int order, int ncomp, const double* xyz, int64_t T, const int32_t* tets,
                      const int32_t* l2g, int xplane_on, double xplane, int64_t N, uint8_t* mask) {
    const int n = nloc_of(order), nle = n * ncomp;
    std::map<std::array<int32_t, 3>, int> cnt;
    for (int64_t e = 0; e < T; ++e)
        for (int f = 0; f < 4; ++f) {
            std::array<int32_t, 3> k = {tets[4 * e + kF2P[f][0]], tets[4 * e + kF2P[f][1]], tets[4 * e + kF2P[f][2]]};
            std::sort(k.begin(), k.end());
            cnt[k]++;
        }
    const int ndpe = ndpe_of(order), ndpf = ndpf_of(order);
    std::memset(mask, 0, N);
    for (int64_t e = 0; e < T; ++e)
        for (int f = 0; f < 4; ++f) {
            std::array<int32_t, 3> k = {tets[4 * e + kF2P[f][0]], tets[4 * e + kF2P[f][1]], tets[4 * e + kF2P[f][2]]};
            std::sort(k.begin(), k.end());
            if (cnt[k] != 1) continue;
            if (xplane_on) {
                bool ok = true;
                for (int v = 0; v < 3; ++v) ok = ok && xyz[3 * (int64_t)k[v]] <= xplane + 1e-12;
                if (!ok) continue;
            }
            // local dofs on face f: its 3 vertices, the dofs of its 3 edges, its face dofs
            vector<int> loc;
            for (int v = 0; v < 3; ++v) loc.push_back(kF2P[f][v]);
            for (int j = 0; j < 6; ++j) {
                bool on = false;
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b)
                        if (kE2P[j][0] == kF2P[f][a] && kE2P[j][1] == kF2P[f][b]) on = true;
                if (on)
                    for (int l = 0; l < ndpe; ++l) loc.push_back(4 + j * ndpe + l);
            }
            for (int l = 0; l < ndpf; ++l) loc.push_back(4 + 6 * ndpe + f * ndpf + l);
            for (int li : loc)
                for (int c = 0; c < ncomp; ++c) mask[l2g[e * nle + n * c + li]] = 1;
        }
    return 0;
}

// Strong Dirichlet on the assembled system, MatrixPetsc::zeroRows
// (feelpp/feel/feelalg/matrixpetsc.cpp:1762-1860) with the PETSc semantics of
//  mode 0: MatZeroRows(rows, diag, x=g, b): rows zeroed (pattern kept), A_ii = diag, b_i = diag*g_i
//  mode 1: MatZeroRowsColumns: additionally b_j -= A_ji g_i for the other rows, then columns zeroed
//  mode 2: elimination keeping the diagonal (KEEP_DIAGONAL): A_ii kept, b_i = A_ii g_i
int orc_dirichlet(int64_t N, const int64_t* ia, const int32_t* ja, double* val, double* b,
                  const uint8_t* mask, const double* g, int mode, double diag) {
    if (mode == 1) {
        for (int64_t r = 0; r < N; ++r) {
            if (mask[r]) continue;
            for (int64_t p = ia[r]; p < ia[r + 1]; ++p)
                if (mask[ja[p]]) {
                    b[r] -= val[p] * (g ? g[ja[p]] : 0.0);
                    val[p] = 0.0;
                }
        }
    }
    for (int64_t r = 0; r < N; ++r) {
        if (!mask[r]) continue;
        double dkeep = 0;
        for (int64_t p = ia[r]; p < ia[r + 1]; ++p) {
            if (ja[p] == r) dkeep = val[p];
            val[p] = 0.0;
        }
        double dd = mode == 2 ? dkeep : diag;
        for (int64_t p = ia[r]; p < ia[r + 1]; ++p)
            if (ja[p] == r) val[p] = dd;
        b[r] = dd * (g ? g[r] : 0.0);
    }
    return 0;
}

// y = A x
int orc_spmv(int64_t N, const int64_t* ia, const int32_t* ja, const double* val, const double* x, double* y) {
    for (int64_t r = 0; r < N; ++r) {
        double s = 0;
        for (int64_t p = ia[r]; p < ia[r + 1]; ++p) s += val[p] * x[ja[p]];
        y[r] = s;
    }
    return 0;
}

// Preconditioned CG with a Jacobi preconditioner, x0 = 0, stop when
// ||r||_2 <= rtol ||b||_2 (unpreconditioned residual; PETSc KSPCG + PCJACOBI
// with KSP_NORM_UNPRECONDITIONED and the initial-residual convergence test of
// feelpp/feel/feelalg/solverlinearpetsc.cpp:548-555). Returns iterations or
// -1 on breakdown / -2 on maxit; `res` gets the final relative residual.
int orc_pcg(int64_t N, const int64_t* ia, const int32_t* ja, const double* val, const double* b,
            double* x, double rtol, int maxit, double* res, int nthreads) {
    vector<double> r(N), z(N), p(N), q(N), dinv(N);
    for (int64_t i = 0; i < N; ++i) {
        double d = 0;
        for (int64_t k = ia[i]; k < ia[i + 1]; ++k)
            if (ja[k] == i) d = val[k];
        dinv[i] = d != 0.0 ? 1.0 / d : 1.0;
        x[i] = 0.0;
        r[i] = b[i];
    }
    auto dot = [&](const vector<double>& a, const vector<double>& c) {
        double s = 0;
#pragma omp parallel for reduction(+ : s) num_threads(nthreads) if (nthreads > 1)
        for (int64_t i = 0; i < N; ++i) s += a[i] * c[i];
        return s;
    };
    double bn = std::sqrt(dot(r, r));
    if (bn == 0.0) { if (res) *res = 0; return 0; }
    for (int64_t i = 0; i < N; ++i) { z[i] = dinv[i] * r[i]; p[i] = z[i]; }
    double rz = dot(r, z);
    for (int it = 1; it <= maxit; ++it) {
#pragma omp parallel for num_threads(nthreads) if (nthreads > 1) schedule(static)
        for (int64_t i = 0; i < N; ++i) {
            double s = 0;
            for (int64_t k = ia[i]; k < ia[i + 1]; ++k) s += val[k] * p[ja[k]];
            q[i] = s;
        }
        double pq = dot(p, q);
        if (pq <= 0.0) { if (res) *res = std::sqrt(dot(r, r)) / bn; return -1; }
        double alpha = rz / pq;
        for (int64_t i = 0; i < N; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
        double rn = std::sqrt(dot(r, r));
        if (rn <= rtol * bn) { if (res) *res = rn / bn; return it; }
        for (int64_t i = 0; i < N; ++i) z[i] = dinv[i] * r[i];
        double rz2 = dot(r, z);
        double beta = rz2 / rz;
        rz = rz2;
        for (int64_t i = 0; i < N; ++i) p[i] = z[i] + beta * p[i];
    }
    if (res) *res = std::sqrt(dot(r, r)) / bn;
    return -2;
}

// L2 and H1-seminorm errors of a scalar field u_h against
// u = sin(pi x) sin(pi y) sin(pi z): normL2 / normH1
// (feelpp/feel/feelvf/norml2.hpp:37, normh1.hpp), i.e. integrate(elements,
// (u_h - u)^2).evaluate() with the given quadrature degree.
int orc_errors(int order, int qdeg, const double* xyz, int64_t T, const int32_t* tets, const int32_t* l2g,
               const double* u, double* l2, double* h1) {
    Tab tab;
    if (!make_tab(order, qdeg, tab)) return -1;
    const int n = tab.n, Q = tab.Q;
    double s0 = 0, s1 = 0;
    vector<double> gp(n * 3);
    for (int64_t e = 0; e < T; ++e) {
        double K[9], B[9], J, d;
        geomap(xyz, tets + 4 * e, K, J, B, d);
        for (int q = 0; q < Q; ++q) {
            double X[3] = {0, 0, 0};
            for (int v = 0; v < 4; ++v)
                for (int r = 0; r < 3; ++r) X[r] += xyz[3 * (int64_t)tets[4 * e + v] + r] * tab.gphi[4 * q + v];
            double uh = 0, g[3] = {0, 0, 0};
            for (int i = 0; i < n; ++i) {
                double ui = u[l2g[e * n + i]];
                uh += ui * tab.phi[q * n + i];
                const double* gh = &tab.dphi[(size_t)(q * n + i) * 3];
                for (int r = 0; r < 3; ++r) g[r] += ui * (B[3 * r] * gh[0] + B[3 * r + 1] * gh[1] + B[3 * r + 2] * gh[2]);
            }
            double sx = std::sin(M_PI * X[0]), sy = std::sin(M_PI * X[1]), sz = std::sin(M_PI * X[2]);
            double cx = std::cos(M_PI * X[0]), cy = std::cos(M_PI * X[1]), cz = std::cos(M_PI * X[2]);
            double ue = sx * sy * sz;
            double ge[3] = {M_PI * cx * sy * sz, M_PI * sx * cy * sz, M_PI * sx * sy * cz};
            double wJ = tab.w[q] * J;
            s0 += wJ * (uh - ue) * (uh - ue);
            for (int r = 0; r < 3; ++r) s1 += wJ * (g[r] - ge[r]) * (g[r] - ge[r]);
        }
    }
    *l2 = std::sqrt(s0);
    *h1 = std::sqrt(s1);
    return 0;
}

int orc_num_threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
