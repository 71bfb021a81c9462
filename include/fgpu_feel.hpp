// fgpu_feel.hpp — a Feel++-shaped C++ front end over the C-ABI of fgpu.h.
//
// This is the binding a Feel++ maintainer would compile into Feel++ to send the
// supported integrands of `form2 = integrate(elements(mesh), expr)` to the GB300
// backend. Here it is self-contained (minimal Mesh / FunctionSpace / Element types
// instead of Feel++'s), so that user code reads like a Feel++ application:
//
//   fgpu_feel::Backend be(argc, argv);                       // --ksp-type, --pc-type, --on.type, --ksp-rtol
//   auto mesh = fgpu_feel::Mesh::fromArrays(be, xyz, tets);  // insertion order (elements.hpp:780-809)
//   auto Xh = fgpu_feel::Pch<2>(mesh);
//   auto u = Xh->element(), v = Xh->element();
//   auto k = Xh->p0(kappa);                                  // piecewise-constant coefficient
//   auto a = form2(_test = Xh, _trial = Xh);
//   a = integrate(_range = elements(mesh), _expr = idv(k) * inner(gradt(u), grad(v)) + idt(u) * id(v));
//   auto l = form1(_test = Xh);
//   l = integrate(_range = elements(mesh), _expr = expr("3*pi*pi*sin(pi*x)*sin(pi*y)*sin(pi*z)") * id(v));
//   a += on(_range = boundaryfaces(mesh), _rhs = l, _element = u, _expr = cst(0.));
//   a.solve(_rhs = l, _solution = u);
//
// Each call maps to one C-ABI entry point (the Feel++ interfaces they replace are
// cited in fgpu.h): integrate(...) on a bilinear form -> fgpu_assemble_matrix, on a
// linear form -> fgpu_assemble_vector, on(...) -> fgpu_space_boundary_dofs +
// fgpu_dirichlet, solve -> fgpu_solve_cg / fgpu_solve_gmres / fgpu_solve_cg_amg with the
// ksp/pc options of the backend (Feel++ defaults: --ksp-type=gmres, --on.type=elimination).
// Integrands outside the supported patterns throw fgpu_feel::Error: inside Feel++ the
// shim would leave those to the CPU Integrator; here there is no CPU path. Failures of
// the library become exceptions carrying fgpu_last_error (Feel++ aborts through
// LOG(FATAL) / CHKERRABORT instead).
#pragma once

#include <algorithm>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "fgpu.h"

namespace fgpu_feel {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& msg) : std::runtime_error(msg), code(c) {}
};

inline void check(int rc, const fgpu_ctx* ctx, const char* what) {
    if (rc != FGPU_OK)
        throw Error(rc, std::string(what) + ": " + (ctx ? fgpu_last_error(ctx) : "backend creation failed"));
}

// ---- Backend<double>::build("gb300") with the option database of a Feel++ run -------------
class Backend {
public:
    std::string ksp_type = "gmres";          // Feel++ default ksp-type (backend.cpp:56)
    std::string pc_type = "jacobi";          // LU is not provided by the GPU backend
    std::string on_type = "elimination";     // Feel++ default on.type (options.cpp:338-340)
    double ksp_rtol = 1e-10;
    int ksp_maxit = 100000;
    int gmres_restart = 30;

    explicit Backend(int argc = 0, char** argv = nullptr, int device = 0) {
        for (int i = 1; i + 1 < argc; ++i) {
            const std::string k = argv[i], v = argv[i + 1];
            if (k == "--ksp-type") ksp_type = v, ++i;
            else if (k == "--pc-type") pc_type = v, ++i;
            else if (k == "--on.type") on_type = v, ++i;
            else if (k == "--ksp-rtol") ksp_rtol = std::stod(v), ++i;
            else if (k == "--ksp-maxit") ksp_maxit = std::stoi(v), ++i;
            else if (k == "--ksp-gmres-restart") gmres_restart = std::stoi(v), ++i;
        }
        fgpu_config cfg{};
        cfg.device = device;
        check(fgpu_create(&cfg, &ctx_), ctx_, "fgpu_create");
    }
    ~Backend() { fgpu_destroy(ctx_); }
    Backend(const Backend&) = delete;
    Backend& operator=(const Backend&) = delete;
    fgpu_ctx* ctx() const { return ctx_; }

private:
    fgpu_ctx* ctx_ = nullptr;
};

// ---- mesh (tetrahedra, vertex ids in insertion order) -------------------------------------
class Mesh {
public:
    static std::shared_ptr<Mesh> fromArrays(Backend& be, const std::vector<double>& xyz, const std::vector<int32_t>& tets) {
        auto m = std::shared_ptr<Mesh>(new Mesh(be));
        check(fgpu_mesh_upload(be.ctx(), (int64_t)xyz.size() / 3, xyz.data(), (int64_t)tets.size() / 4, tets.data(), &m->h_),
              be.ctx(), "fgpu_mesh_upload");
        m->nt_ = (int64_t)tets.size() / 4;
        return m;
    }
    ~Mesh() { fgpu_mesh_destroy(h_); }
    fgpu_mesh* handle() const { return h_; }
    Backend& backend() const { return be_; }
    int64_t numElements() const { return nt_; }

private:
    explicit Mesh(Backend& be) : be_(be) {}
    Backend& be_;
    fgpu_mesh* h_ = nullptr;
    int64_t nt_ = 0;
};

struct ElementsRange { std::shared_ptr<Mesh> mesh; };
struct BoundaryFacesRange { std::shared_ptr<Mesh> mesh; };
inline ElementsRange elements(const std::shared_ptr<Mesh>& m) { return {m}; }
inline BoundaryFacesRange boundaryfaces(const std::shared_ptr<Mesh>& m) { return {m}; }

class FunctionSpace;

// ---- an element of a space: its coefficient vector lives on the device --------------------
class Element {
public:
    Element(std::shared_ptr<FunctionSpace> V, int64_t n);
    ~Element() { fgpu_vector_destroy(h_); }
    Element(const Element&) = delete;
    Element& operator=(const Element&) = delete;
    Element(Element&& o) noexcept : V_(std::move(o.V_)), h_(o.h_), n_(o.n_) { o.h_ = nullptr; }
    fgpu_vector* handle() const { return h_; }
    const std::shared_ptr<FunctionSpace>& functionSpace() const { return V_; }
    std::vector<double> toHost() const;

private:
    std::shared_ptr<FunctionSpace> V_;
    fgpu_vector* h_ = nullptr;
    int64_t n_ = 0;
};

// ---- Pch<Order> on tetrahedra (DofTable numbering of the reference) -----------------------
class FunctionSpace : public std::enable_shared_from_this<FunctionSpace> {
public:
    FunctionSpace(std::shared_ptr<Mesh> m, int order) : mesh_(std::move(m)), order_(order) {
        fgpu_ctx* c = mesh_->backend().ctx();
        check(fgpu_space_create(c, mesh_->handle(), order, 1, &h_), c, "fgpu_space_create");
        int nloc = 0;
        check(fgpu_space_ndof(h_, &ndof_, &nloc), c, "fgpu_space_ndof");
    }
    ~FunctionSpace() { fgpu_space_destroy(h_); }
    Element element() { return Element(shared_from_this(), ndof_); }
    // a P0 (one value per element) coefficient, as `idv(k)` of a Pdh<0> element in Feel++
    std::vector<double> p0(const std::vector<double>& values) const {
        if ((int64_t)values.size() != mesh_->numElements()) throw Error(FGPU_ERR_INVALID, "p0: one value per element");
        return values;
    }
    fgpu_space* handle() const { return h_; }
    const std::shared_ptr<Mesh>& mesh() const { return mesh_; }
    int64_t nDof() const { return ndof_; }
    int order() const { return order_; }

private:
    std::shared_ptr<Mesh> mesh_;
    int order_;
    fgpu_space* h_ = nullptr;
    int64_t ndof_ = 0;
};

template <int Order>
std::shared_ptr<FunctionSpace> Pch(const std::shared_ptr<Mesh>& m) {
    static_assert(Order >= 1 && Order <= 3, "Pch<1..3>");
    return std::make_shared<FunctionSpace>(m, Order);
}

inline Element::Element(std::shared_ptr<FunctionSpace> V, int64_t n) : V_(std::move(V)), n_(n) {
    fgpu_ctx* c = V_->mesh()->backend().ctx();
    check(fgpu_vector_create(c, n, &h_), c, "fgpu_vector_create");
}
inline std::vector<double> Element::toHost() const {
    std::vector<double> out((size_t)n_);
    check(fgpu_vector_download(h_, out.data()), V_->mesh()->backend().ctx(), "fgpu_vector_download");
    return out;
}

// ---- expression nodes of the supported integrands ---------------------------------------
struct GradT {};
struct Grad {};
struct IdT {};
struct Id {};
inline GradT gradt(const Element&) { return {}; }
inline Grad grad(const Element&) { return {}; }
inline IdT idt(const Element&) { return {}; }
inline Id id(const Element&) { return {}; }

struct Cst { double c; };
inline Cst cst(double c) { return {c}; }
struct P0Field { const std::vector<double>* v; };
inline P0Field idv(const std::vector<double>& k) { return {&k}; }

// kappa * inner(gradt(u), grad(v)) + mass * idt(u) * id(v)
struct Form2Expr {
    double kappa = 0.0;
    const std::vector<double>* kappa_elem = nullptr;
    double mass = 0.0;
};
inline Form2Expr inner(GradT, Grad) { return Form2Expr{1.0, nullptr, 0.0}; }
inline Form2Expr operator*(IdT, Id) { return Form2Expr{0.0, nullptr, 1.0}; }
inline Form2Expr operator*(double c, Form2Expr e) { e.kappa *= c; e.mass *= c; return e; }
inline Form2Expr operator*(Cst c, Form2Expr e) { return c.c * e; }
inline Form2Expr operator*(P0Field k, Form2Expr e) {
    if (e.mass != 0.0 || e.kappa_elem) throw Error(FGPU_ERR_INVALID, "idv(k) scales the stiffness term only");
    e.kappa_elem = k.v;
    return e;
}
inline Form2Expr operator+(Form2Expr a, const Form2Expr& b) {
    if (a.kappa_elem && (b.kappa_elem || b.kappa != 0.0)) throw Error(FGPU_ERR_INVALID, "one stiffness coefficient");
    if (b.kappa_elem && a.kappa != 0.0) throw Error(FGPU_ERR_INVALID, "one stiffness coefficient");
    if (b.kappa_elem) a.kappa_elem = b.kappa_elem;
    a.kappa += b.kappa;
    a.mass += b.mass;
    return a;
}

// f * id(v): the manufactured source 3 pi^2 sin(pi x) sin(pi y) sin(pi z) or a constant
struct Source { int kind; double c; };
inline Source expr(const std::string& s) {
    std::string t;
    for (char ch : s)
        if (ch != ' ') t += ch;
    if (t == "3*pi*pi*sin(pi*x)*sin(pi*y)*sin(pi*z)" || t == "3*pi^2*sin(pi*x)*sin(pi*y)*sin(pi*z)")
        return {FGPU_RHS_SINE, 0.0};
    throw Error(FGPU_ERR_INVALID, "expr(\"" + s + "\"): not an integrand of the GPU backend");
}
struct Form1Expr { int kind; double c; };
inline Form1Expr operator*(Source f, Id) { return {f.kind, f.c}; }
inline Form1Expr operator*(Cst c, Id) { return {FGPU_RHS_CONST, c.c}; }

// ---- named arguments (_range = ..., _expr = ..., as Feel++'s boost::parameter keywords) ---
template <class Tag, class T>
struct Named { T v; };
#define FGPU_FEEL_KEYWORD(name)                                                   \
    struct name##_tag {};                                                         \
    struct name##_kw {                                                            \
        template <class T>                                                        \
        Named<name##_tag, T> operator=(T v) const { return {std::move(v)}; }      \
    };                                                                            \
    inline constexpr name##_kw _##name {};
FGPU_FEEL_KEYWORD(range)
FGPU_FEEL_KEYWORD(expr)
FGPU_FEEL_KEYWORD(test)
FGPU_FEEL_KEYWORD(trial)
#undef FGPU_FEEL_KEYWORD
struct rhs_tag {};
struct element_tag {};
struct solution_tag {};
class LinearForm;
struct rhs_kw { Named<rhs_tag, LinearForm*> operator=(LinearForm& l) const { return {&l}; } };
struct element_kw { Named<element_tag, Element*> operator=(Element& u) const { return {&u}; } };
struct solution_kw { Named<solution_tag, Element*> operator=(Element& u) const { return {&u}; } };
inline constexpr rhs_kw _rhs{};
inline constexpr element_kw _element{};
inline constexpr solution_kw _solution{};

template <class R, class E>
struct Integral { R range; E expr; };
template <class R, class E>
Integral<R, E> integrate(Named<range_tag, R> r, Named<expr_tag, E> e) { return {r.v, e.v}; }

struct OnExpr {
    BoundaryFacesRange range;
    LinearForm* rhs;
    Element* element;
    double g;
};
inline OnExpr on(Named<range_tag, BoundaryFacesRange> r, Named<rhs_tag, LinearForm*> l, Named<element_tag, Element*> u,
                 Named<expr_tag, Cst> g) {
    return {r.v, l.v, u.v, g.v.c};
}

// ---- form1(_test = Xh): a device vector filled by integrate(...) --------------------------
class LinearForm {
public:
    explicit LinearForm(std::shared_ptr<FunctionSpace> V) : V_(std::move(V)), vec_(V_->element()) {}
    LinearForm& operator=(const Integral<ElementsRange, Form1Expr>& I) { assemble(I, 0); return *this; }
    LinearForm& operator+=(const Integral<ElementsRange, Form1Expr>& I) { assemble(I, 1); return *this; }
    Element& vector() { return vec_; }
    const std::shared_ptr<FunctionSpace>& functionSpace() const { return V_; }

private:
    void assemble(const Integral<ElementsRange, Form1Expr>& I, int acc) {
        fgpu_rhs_desc d{};
        d.kind = I.expr.kind;
        d.c[0] = I.expr.c;
        d.range = FGPU_RANGE_ELEMENTS;
        fgpu_ctx* c = V_->mesh()->backend().ctx();
        check(fgpu_assemble_vector(c, V_->handle(), &d, vec_.handle(), acc), c, "fgpu_assemble_vector");
    }
    std::shared_ptr<FunctionSpace> V_;
    Element vec_;
};

struct SolveStats {
    int iterations = 0;
    double rel_residual = 0.0;
    double time_ms = 0.0;
};

// ---- form2(_test = Xh, _trial = Xh): the device CSR matrix with the GraphCSR pattern ------
class BilinearForm {
public:
    explicit BilinearForm(std::shared_ptr<FunctionSpace> V) : V_(std::move(V)) {
        fgpu_ctx* c = ctx();
        check(fgpu_matrix_create(c, V_->handle(), V_->handle(), FGPU_F64, &A_), c, "fgpu_matrix_create");
    }
    ~BilinearForm() {
        if (amg_) fgpu_amg_destroy(amg_);
        fgpu_matrix_destroy(A_);
    }
    BilinearForm(const BilinearForm&) = delete;
    BilinearForm& operator=(const BilinearForm&) = delete;
    BilinearForm(BilinearForm&& o) noexcept : V_(std::move(o.V_)), A_(o.A_), amg_(o.amg_) { o.A_ = nullptr; o.amg_ = nullptr; }

    BilinearForm& operator=(const Integral<ElementsRange, Form2Expr>& I) { assemble(I.expr, 0); return *this; }
    BilinearForm& operator+=(const Integral<ElementsRange, Form2Expr>& I) { assemble(I.expr, 1); return *this; }
    BilinearForm& operator+=(const OnExpr& o) {
        fgpu_ctx* c = ctx();
        int64_t cnt = 0;
        check(fgpu_space_boundary_dofs(V_->handle(), 0, 0.0, &cnt, nullptr), c, "fgpu_space_boundary_dofs");
        std::vector<int32_t> dofs((size_t)cnt);
        check(fgpu_space_boundary_dofs(V_->handle(), 0, 0.0, &cnt, dofs.data()), c, "fgpu_space_boundary_dofs");
        std::vector<double> g((size_t)cnt, o.g);
        const std::string& t = V_->mesh()->backend().on_type;
        const int mode = t == "elimination_symmetric" ? FGPU_ON_ELIMINATION_SYMMETRIC
                         : t == "elimination_keep_diagonal" ? FGPU_ON_ELIMINATION_KEEP_DIAGONAL : FGPU_ON_ELIMINATION;
        check(fgpu_dirichlet(c, A_, o.rhs->vector().handle(), cnt, dofs.data(), o.g != 0.0 ? g.data() : nullptr, mode, 1.0), c,
              "fgpu_dirichlet");
        return *this;
    }

    // a.solve(_rhs = l, _solution = u) with the backend's ksp / pc options
    SolveStats solve(Named<rhs_tag, LinearForm*> l, Named<solution_tag, Element*> u) {
        const Backend& be = V_->mesh()->backend();
        fgpu_ctx* c = ctx();
        fgpu_solver_cfg sc{};
        sc.rtol = be.ksp_rtol;
        sc.maxit = be.ksp_maxit;
        sc.pc = be.pc_type == "gamg" ? FGPU_PC_GAMG : be.pc_type == "none" ? FGPU_PC_NONE : FGPU_PC_JACOBI;
        if (be.pc_type == "lu") throw Error(FGPU_ERR_INVALID, "--pc-type=lu: no direct solver on the GPU backend");
        fgpu_solve_stats st{};
        if (sc.pc == FGPU_PC_GAMG && !amg_) check(fgpu_amg_create(c, A_, nullptr, &amg_), c, "fgpu_amg_create");
        const fgpu_vector* b = l.v->vector().handle();
        fgpu_vector* x = u.v->handle();
        if (be.ksp_type == "gmres")
            check(fgpu_solve_gmres(c, A_, amg_, b, x, &sc, be.gmres_restart, &st), c, "fgpu_solve_gmres");
        else if (be.ksp_type == "cg" && sc.pc == FGPU_PC_GAMG)
            check(fgpu_solve_cg_amg(c, A_, amg_, b, x, &sc, &st), c, "fgpu_solve_cg_amg");
        else if (be.ksp_type == "cg")
            check(fgpu_solve_cg(c, A_, nullptr, b, x, &sc, &st), c, "fgpu_solve_cg");
        else
            throw Error(FGPU_ERR_INVALID, "--ksp-type=" + be.ksp_type + ": cg or gmres");
        return {st.iterations, st.rel_residual, st.time_ms};
    }

    fgpu_matrix* handle() const { return A_; }
    // CSR arrays with 32-bit offsets, as MatSeqAIJSetPreallocationCSR takes them
    void csr32(std::vector<int32_t>& ia, std::vector<int32_t>& ja, std::vector<double>& val) const {
        int64_t nr = 0, nnz = 0;
        int prec = 0;
        check(fgpu_matrix_info(A_, &nr, &nnz, &prec), ctx(), "fgpu_matrix_info");
        ia.resize((size_t)nr + 1);
        ja.resize((size_t)nnz);
        val.resize((size_t)nnz);
        check(fgpu_matrix_get_csr32(A_, ia.data(), ja.data(), val.data()), ctx(), "fgpu_matrix_get_csr32");
    }

private:
    fgpu_ctx* ctx() const { return V_->mesh()->backend().ctx(); }
    void assemble(const Form2Expr& e, int acc) {
        fgpu_form_desc d{};
        d.kind = FGPU_FORM_LAPLACE_MASS;
        d.kappa = e.kappa_elem ? 0.0 : e.kappa;
        d.kappa_elem = e.kappa_elem ? e.kappa_elem->data() : nullptr;
        d.mass = e.mass;
        d.algo = FGPU_ALGO_AUTO;
        d.range = FGPU_RANGE_ELEMENTS;
        check(fgpu_assemble_matrix(ctx(), A_, &d, acc), ctx(), "fgpu_assemble_matrix");
    }
    std::shared_ptr<FunctionSpace> V_;
    fgpu_matrix* A_ = nullptr;
    fgpu_amg* amg_ = nullptr;
};

inline BilinearForm form2(Named<test_tag, std::shared_ptr<FunctionSpace>> test, Named<trial_tag, std::shared_ptr<FunctionSpace>> trial) {
    if (test.v != trial.v) throw Error(FGPU_ERR_INVALID, "form2: test and trial spaces must be the same");
    return BilinearForm(test.v);
}
inline LinearForm form1(Named<test_tag, std::shared_ptr<FunctionSpace>> test) { return LinearForm(test.v); }

// normL2 / normH1 (seminorm) of u - sin(pi x) sin(pi y) sin(pi z) (feelvf/norml2.hpp:37, normh1.hpp)
inline std::pair<double, double> errorsSine(const Element& u) {
    fgpu_ctx* c = u.functionSpace()->mesh()->backend().ctx();
    double l2 = 0, h1 = 0;
    check(fgpu_norms_sine(c, u.functionSpace()->handle(), u.handle(), 0, &l2, &h1), c, "fgpu_norms_sine");
    return {l2, h1};
}

}  // namespace fgpu_feel
