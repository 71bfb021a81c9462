// A Feel++-style application written against include/fgpu_feel.hpp (the C++ shim over the
// C-ABI): the P2 Laplacian + mass with a piecewise-constant kappa, the sine load, on() with a
// homogeneous value on the boundary faces, and a.solve(). It reads the mesh (vertices,
// tetrahedra, kappa) from a binary file and writes the assembled CSR (32-bit offsets), the
// load vector, the solution and the solver statistics, so that a test can compare them with the
// Python front end and the oracle.
//
//   shim_poisson in.bin out.bin [--ksp-type cg --pc-type jacobi --on.type elimination_symmetric ...]
//
// in.bin : int64 nv, int64 nt, double xyz[nv*3], int32 tets[nt*4], double kappa[nt]
// out.bin: int64 nrows, int64 nnz, int32 ia[nrows+1], int32 ja[nnz], double val[nnz],
//          double load[nrows], double u[nrows], int64 iterations, double rel_residual, double l2, double h1
#include <cstdio>
#include <fstream>
#include <iostream>

#include "fgpu_feel.hpp"

using namespace fgpu_feel;

int main(int argc, char** argv) {
    if (argc < 3) {
        std::cerr << "usage: shim_poisson in.bin out.bin [options]\n";
        return 2;
    }
    std::ifstream in(argv[1], std::ios::binary);
    int64_t nv = 0, nt = 0;
    in.read(reinterpret_cast<char*>(&nv), 8);
    in.read(reinterpret_cast<char*>(&nt), 8);
    std::vector<double> xyz((size_t)nv * 3), kappa((size_t)nt);
    std::vector<int32_t> tets((size_t)nt * 4);
    in.read(reinterpret_cast<char*>(xyz.data()), (std::streamsize)(xyz.size() * 8));
    in.read(reinterpret_cast<char*>(tets.data()), (std::streamsize)(tets.size() * 4));
    in.read(reinterpret_cast<char*>(kappa.data()), (std::streamsize)(kappa.size() * 8));
    if (!in) {
        std::cerr << "cannot read " << argv[1] << "\n";
        return 2;
    }
    try {
        Backend be(argc - 2, argv + 2);
        auto mesh = Mesh::fromArrays(be, xyz, tets);
        auto Xh = Pch<2>(mesh);
        auto u = Xh->element();
        auto v = Xh->element();
        auto k = Xh->p0(kappa);

        auto a = form2(_test = Xh, _trial = Xh);
        a = integrate(_range = elements(mesh), _expr = idv(k) * inner(gradt(u), grad(v)) + idt(u) * id(v));
        std::vector<int32_t> ia, ja;
        std::vector<double> val;
        a.csr32(ia, ja, val);

        auto l = form1(_test = Xh);
        l = integrate(_range = elements(mesh), _expr = expr("3*pi*pi*sin(pi*x)*sin(pi*y)*sin(pi*z)") * id(v));
        const std::vector<double> load = l.vector().toHost();

        a += on(_range = boundaryfaces(mesh), _rhs = l, _element = u, _expr = cst(0.));
        const SolveStats st = a.solve(_rhs = l, _solution = u);
        const std::vector<double> sol = u.toHost();
        const auto err = errorsSine(u);

        std::ofstream out(argv[2], std::ios::binary);
        const int64_t nrows = (int64_t)ia.size() - 1, nnz = (int64_t)ja.size(), it = st.iterations;
        out.write(reinterpret_cast<const char*>(&nrows), 8);
        out.write(reinterpret_cast<const char*>(&nnz), 8);
        out.write(reinterpret_cast<const char*>(ia.data()), (std::streamsize)(ia.size() * 4));
        out.write(reinterpret_cast<const char*>(ja.data()), (std::streamsize)(ja.size() * 4));
        out.write(reinterpret_cast<const char*>(val.data()), (std::streamsize)(val.size() * 8));
        out.write(reinterpret_cast<const char*>(load.data()), (std::streamsize)(load.size() * 8));
        out.write(reinterpret_cast<const char*>(sol.data()), (std::streamsize)(sol.size() * 8));
        out.write(reinterpret_cast<const char*>(&it), 8);
        out.write(reinterpret_cast<const char*>(&st.rel_residual), 8);
        out.write(reinterpret_cast<const char*>(&err.first), 8);
        out.write(reinterpret_cast<const char*>(&err.second), 8);
        std::printf("shim_poisson: nrows %lld nnz %lld iterations %lld rel_residual %.3e L2 %.6e\n", (long long)nrows,
                    (long long)nnz, (long long)it, st.rel_residual, err.first);
    } catch (const Error& e) {
        std::cerr << "fgpu_feel error " << e.code << ": " << e.what() << "\n";
        return 1;
    }
    return 0;
}
