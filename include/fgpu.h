/*
 * fgpu.h — C-ABI of the GB300-native assembly + solve backend for the Feel++
 * variational-form hot path:
 *
 *   auto a = form2(_test=Xh,_trial=Xh);
 *   a  = integrate(_range=elements(mesh), _expr=kappa*inner(gradt(u),grad(v)) + idt(u)*id(v));
 *   auto l = form1(_test=Xh);
 *   l  = integrate(_range=elements(mesh), _expr=f*id(v));
 *   a += on(_range=boundaryfaces(mesh), _rhs=l, _element=u, _expr=cst(0.));
 *   a.solve(_rhs=l, _solution=u);
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, returns
 * an int status (FGPU_OK == 0) and never aborts or throws; the message of the
 * last failure is available from fgpu_last_error(). Objects are opaque
 * handles owned by the library; host arrays passed in are copied.
 *
 * Each declaration names the Feel++ interface it replaces (paths relative to
 * the Feel++ source tree).
 */
#ifndef FGPU_H
#define FGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the reference aborts via CHKERRABORT / LOG(FATAL)) ---- */
#define FGPU_OK 0
#define FGPU_ERR_INVALID 1        /* bad argument / unsupported combination */
#define FGPU_ERR_CUDA 2           /* CUDA runtime error */
#define FGPU_ERR_BAD_ELEMENT 3    /* degenerate element: |det K| <= 0 or non-finite */
#define FGPU_ERR_OUT_OF_RANGE 4   /* vertex / dof index out of range */
#define FGPU_ERR_NOT_CONVERGED 5  /* solver reached maxit */
#define FGPU_ERR_BREAKDOWN 6      /* CG breakdown (p.Ap <= 0: matrix not SPD) */
#define FGPU_ERR_PATTERN 7        /* assembly met a column absent from the pattern */
#define FGPU_ERR_ALLOC 8          /* device allocation failed */

/* ---- precision / form kinds / options ---- */
#define FGPU_F64 0
#define FGPU_F32 1
#define FGPU_DF64 2               /* matrix-free operators: double-float arithmetic (~48 bits), binary64 interface */

#define FGPU_FORM_LAPLACE_MASS 0  /* kappa*inner(gradt(u),grad(v)) + mass*idt(u)*id(v)          */
#define FGPU_FORM_ELASTICITY 1    /* inner(lambda tr(eps(u)) I + 2 mu eps(u), grad(v)), Pchv    */

#define FGPU_ALGO_AUTO 0          /* best available algorithm for the form */
#define FGPU_ALGO_GATHER 1        /* row-owner gather: each CSR row summed by one warp, element order */
#define FGPU_ALGO_COLOUR 2        /* element-coloured scatter-add (matrix-free binary32 operators,
                                     fgpu_operator_set_algo); assembly runs FGPU_ALGO_GATHER */
#define FGPU_ALGO_GATHER_NATIVE_F64 3 /* row-owner gather in native FP64 arithmetic (FP64 matrices; the
                                     default FP64 path computes in double-float on the FP32 pipes) */
#define FGPU_ALGO_TWO_PHASE 4     /* element matrices (upper triangles; 3x3 blocks for elasticity) into
                                     a device buffer in df64 (FP64 matrices) or binary32, then each CSR
                                     entry sums its contributions in element order through a gather map
                                     built once per space */
#define FGPU_ALGO_STREAMED 5      /* scalar Laplace/mass forms on affine tetrahedra: the arithmetic and
                                     summation order of FGPU_ALGO_TWO_PHASE (bit-identical values) in one
                                     persistent launch, element matrices through a ring of element slots
                                     that stays in L2, each pattern row summed once its elements are done;
                                     no element buffer, no gather map.
   FGPU_ALGO_AUTO picks by the form and the mesh only, never by free memory or capture state, so its
   values do not depend on other users of the device: TWO_PHASE when the pattern rows have at most
   256 entries, GATHER otherwise. A buffer it cannot allocate is an error (FGPU_ERR_ALLOC). */

/* how fgpu_assemble_matrix_host moves the values to host memory */
#define FGPU_HOST_TRANSFER_AUTO 0   /* DIRECT when the host buffer is page-locked and mapped, else COPY */
#define FGPU_HOST_TRANSFER_COPY 1   /* copy-engine transfers of ranges of entries, overlapping the gather */
#define FGPU_HOST_TRANSFER_DIRECT 2 /* the gather kernel stores each value to device and host memory
                                       (page-locked buffers only; over NVLink-C2C on Grace hosts) */

#define FGPU_RANGE_ELEMENTS 0       /* _range=elements(mesh) */
#define FGPU_RANGE_BOUNDARY_FACES 1 /* _range=boundaryfaces(mesh): faces of one element */
#define FGPU_RANGE_MARKED_FACES 2   /* boundary faces whose vertices all have x <= range_xmax
                                       (markedfaces of a plane), e.g. a clamped or loaded end */

#define FGPU_RHS_SINE 0           /* f = 3 pi^2 sin(pi x) sin(pi y) sin(pi z) */
#define FGPU_RHS_CONST_VEC 1      /* f = (c0, c1, c2) (Pchv) */
#define FGPU_RHS_CONST 2          /* f = c0 */
#define FGPU_RHS_FACE 3           /* face ranges only: c0*id(v) + c1*id(v)/hFace() + c2*inner(grad(v),N()),
                                     e.g. the Nitsche load -inner(k*grad(v)*N(),g) + gamma*k*g*id(v)/hFace() */

#define FGPU_ON_ELIMINATION 0     /* MatZeroRows: row zeroed, diag set, b_i = diag*g_i (default) */
#define FGPU_ON_ELIMINATION_SYMMETRIC 1 /* MatZeroRowsColumns: also b_j -= A_ji g_i, column zeroed */
#define FGPU_ON_ELIMINATION_KEEP_DIAGONAL 2 /* row zeroed except the diagonal, b_i = A_ii g_i */

#define FGPU_PC_NONE 0
#define FGPU_PC_JACOBI 1
#define FGPU_PC_CHEB_JACOBI 2     /* degree-K Chebyshev polynomial in D^-1 A (Jacobi-scaled), PETSc
                                     KSPCHEBYSHEV+PCJACOBI used as a fixed preconditioner */
#define FGPU_PC_PMG 4             /* p-multigrid V-cycle of a matrix-free operator (fgpu_pmg_create): binary32
                                     Chebyshev smoothing on the order-p operator, the assembled P1 operator
                                     on the same mesh as coarse level, solved by one AMG V-cycle */
#define FGPU_PC_GAMG 3            /* smoothed-aggregation AMG V-cycle (pc-type=gamg): fgpu_amg_create,
                                     then fgpu_solve_cg_amg */

#define FGPU_ARITH_F64 0          /* solver arithmetic: native FP64 (default) */
#define FGPU_ARITH_DF64 1         /* double-float on the FP32 pipes (~48 bits; moderately conditioned systems) */

typedef struct fgpu_ctx fgpu_ctx;
typedef struct fgpu_graph fgpu_graph;
typedef struct fgpu_bc fgpu_bc;
typedef struct fgpu_batch fgpu_batch;
typedef struct fgpu_amg fgpu_amg;
typedef struct fgpu_pmg fgpu_pmg;
typedef struct fgpu_operator fgpu_operator;
typedef struct fgpu_mesh fgpu_mesh;
typedef struct fgpu_space fgpu_space;
typedef struct fgpu_matrix fgpu_matrix;
typedef struct fgpu_vector fgpu_vector;

typedef struct {
    int device;        /* CUDA device ordinal */
    void* stream;      /* cudaStream_t to launch on, or NULL for a library-owned stream */
    int profile;       /* 1: time every kernel launch with CUDA events (fgpu_prof_get) */
    int host_threads;  /* host threads for setup work (pattern build); 0 = all cores */
    int host_setup;    /* 1: build dof tables, incidence and patterns on the host (topology.cpp);
                          0 (default): on the device (topology_dev.cu; same arrays), with the host
                          path used automatically for meshes of 2^21 vertices or more */
    int tune;          /* 0 (default): launch shapes that do not change results (threads per block,
                          blocks per SM, loads per batch of the two-phase assembly kernels; the CG's
                          SpMV layout) are timed on the first use of a (device, kernel, order, precision,
                          size class) key and the fastest kept; -1: fixed default shapes */
    const char* tune_cache; /* file the picks are appended to and read from at creation (NULL: none) */
} fgpu_config;

typedef struct {
    int kind;                 /* FGPU_FORM_* */
    double kappa;             /* constant diffusion coefficient when kappa_elem == NULL */
    const double* kappa_elem; /* per-element coefficient (host array, T values) or NULL */
    double mass;              /* coefficient of idt(u)*id(v) (0: pure Laplacian) */
    double lambda, mu;        /* Lame coefficients (FGPU_FORM_ELASTICITY) */
    int quad_degree;          /* exact quadrature degree; 0 = 2*order (feelvf default im(2p)) */
    int algo;                 /* FGPU_ALGO_* */
    const double* kappa_scale;/* device scalar multiplying kappa, read when the kernels run, so a
                                 captured graph sees its current value (a time-dependent
                                 coefficient kappa(t)); NULL = 1. Laplace/mass forms only. */
    int range;                /* FGPU_RANGE_*; on faces (scalar spaces, kappa = 0):
                                 int_f mass*u*v + mass_h*u*v/hFace + dn_trial*(grad u.N)*v
                                       + dn_test*(grad v.N)*u
                                 (Robin: mass; symmetric Nitsche: dn_trial = dn_test = -k,
                                 mass_h = gamma*k), N the unit outward normal, hFace the
                                 longest edge of the face */
    double range_xmax;        /* FGPU_RANGE_MARKED_FACES */
    double mass_h;            /* faces only: coefficient of idt(u)*id(v)/hFace() */
    double dn_trial;          /* faces only: coefficient of inner(gradt(u)*N(), id(v)) */
    double dn_test;           /* faces only: coefficient of inner(grad(v)*N(), idt(u)) */
} fgpu_form_desc;

typedef struct {
    int kind;                 /* FGPU_RHS_* */
    double c[3];
    int quad_degree;          /* 0 = 2*order */
    int range;                /* FGPU_RANGE_*; on faces: FGPU_RHS_CONST (int_f c0 v, Neumann) or
                                 FGPU_RHS_FACE */
    double range_xmax;        /* FGPU_RANGE_MARKED_FACES */
} fgpu_rhs_desc;

typedef struct {
    double rtol;              /* stop when ||b - A x||_2 <= rtol ||b||_2 (ksp-rtol) */
    int maxit;                /* ksp-max-it */
    int pc;                   /* FGPU_PC_* (pc-type) */
    int mixed;                /* 1: binary32 CG with binary64 reliable updates (residual replacement) */
    double inner_rtol;        /* mixed: reduction of the binary32 recurrence residual between two
                                 binary64 residual replacements (0 = 0.1) */
    int check_every;          /* iterations per convergence poll (0 = 16) */
    int arith;                /* FGPU_ARITH_* of the non-mixed solve */
    int cheb_degree;          /* FGPU_PC_CHEB_JACOBI: polynomial degree K (0 = 3); K - 1 extra
                                 operator applications per iteration */
    double cheb_ratio;        /* FGPU_PC_CHEB_JACOBI: lambda_min / lambda_max of the interval (0 = 0.03);
                                 lambda_max = 1.1 x a Lanczos estimate (ksp_chebyshev_esteig 0,0.1,0,1.1) */
} fgpu_solver_cfg;

typedef struct {              /* smoothed-aggregation AMG (PETSc PCGAMG "agg" options of the reference) */
    double threshold;         /* pc-gamg-threshold: drop couplings |a_ij| <= threshold sqrt(a_ii a_jj) (0) */
    int max_levels;           /* pc-mg-levels (0 = 10) */
    int coarse_eq_lim;        /* pc-gamg-coarse-eq-lim (0 = 800) */
    int agg_smooths;          /* pc-gamg-nsmooths: 0 = default 1 (smoothed aggregation); -1 = none */
    int smoother_degree;      /* Chebyshev degree of the level smoothers (0 = 3, i.e. 2 operator sweeps) */
    int setup_on_host;        /* 0: hierarchy built on the device (levels of at most 16384 rows on the host);
                                 1: built on the host. Both give the same hierarchy bit for bit. */
    /* near null space (PETSc MatSetNearNullSpace, which the reference attaches on solve:
     * feelpp/feel/feelalg/backend.hpp:1074-1088; e.g. the six rigid body modes of an elasticity space,
     * fgpu_space_rigid_body_modes). nns_count = 0: the constant vector per aggregate. Otherwise the
     * aggregation runs on nodes of block_size consecutive rows and each aggregate's tentative
     * prolongator is the Q of the QR factorisation of the vectors restricted to its rows. */
    int block_size;           /* rows per node (0 = 1) */
    int nns_count;            /* number of vectors */
    const fgpu_vector* const* nns;   /* fgpu_amg_create / fgpu_amg_device_build: device vectors of the matrix's size */
    const double* nns_host;   /* fgpu_amg_host_build: nns_count x n values, vector after vector */
} fgpu_amg_cfg;

typedef struct {
    int iterations;           /* total (inner) CG iterations */
    int outer;                /* binary64 residual replacements (mixed) */
    double rel_residual;      /* final ||b - A x||_2 / ||b||_2 recomputed in FP64 */
    double time_ms;           /* solve wall time on the device stream */
    double eig_max;           /* FGPU_PC_CHEB_JACOBI: lambda_max used for D^-1 A (0 otherwise) */
    int fallback;             /* mixed: 1 when the binary32 iteration broke down (p.Ap <= 0 in
                                 binary32, an ill-conditioned system) and the solve finished in FP64 */
    int fallback_iterations;  /* FP64 iterations after the fallback */
} fgpu_solve_stats;

/* ---- context (replaces Feel::Environment + Backend<double>::build(kind),
 *      feelpp/feel/feelalg/backend.cpp:218-250) ---- */
int fgpu_create(const fgpu_config* cfg, fgpu_ctx** out);
int fgpu_destroy(fgpu_ctx* ctx);
const char* fgpu_last_error(const fgpu_ctx* ctx);
int fgpu_sync(fgpu_ctx* ctx);
/* number of kernels this context has launched so far */
int64_t fgpu_launch_count(const fgpu_ctx* ctx);

/* ---- mesh (replaces Mesh<Simplex<3>> element storage, feelpp/feel/feelmesh/
 *      elements.hpp:780-809; vertex coordinates and tetrahedra in insertion order) ---- */
int fgpu_mesh_upload(fgpu_ctx* ctx, int64_t nv, const double* xyz, int64_t nt, const int32_t* tets,
                     fgpu_mesh** out);
/* replace the vertex coordinates (host array, nv x 3): a moved mesh keeps its topology */
int fgpu_mesh_set_coords(fgpu_mesh* mesh, const double* xyz);
/* Hexahedral mesh (Mesh<Hypercube<3,1>>, e.g. from MeshStructured, feelpp/feel/feeldiscr/meshstructured.hpp):
 * nh x 8 vertex ids in the reference hexahedron's order (feelpp/feel/feelmesh/refhypercube.hpp:148-183:
 * the z = -1 face counter-clockwise from (-1,-1,-1), then the z = +1 face). Spaces: scalar Q1/Q2
 * (fgpu_space_create order 1 or 2); forms: Laplace/mass over elements(mesh) with the trilinear map at
 * every point of the tensor Gauss rule of feelpp/feel/feelpoly/gausshypercube.cpp; load vectors; on()
 * through fgpu_space_boundary_dofs; CG/AMG on the assembled matrix; EnSight export. */
int fgpu_mesh_upload_hex(fgpu_ctx* ctx, int64_t nv, const double* xyz, int64_t nh, const int32_t* hexes, fgpu_mesh** out);
int fgpu_mesh_cell_vertices(const fgpu_mesh* mesh, int* nverts);   /* 4 or 8 */
/* curved (P2-geometry, GEOMAP_HO) elements: ho = T x 6 x 3 coordinates of each element's edge nodes in
 * the local edge order (1,2) (2,0) (0,1) (0,3) (1,3) (2,3) (host array, copied); NULL makes the mesh
 * affine again. On a curved mesh the scalar Laplace/mass form and the sine / constant load vector are
 * integrated with per-point maps (quadrature degree <= 5 / 7 / 8 for P1 / P2 / P3, default 2p + 2);
 * face integrals, elasticity, matrix-free operators, batches and error norms refuse. */
int fgpu_mesh_set_ho_nodes(fgpu_mesh* mesh, const double* ho);
int fgpu_mesh_destroy(fgpu_mesh* mesh);

/* ---- function space Pch<order> (ncomp = 1) / Pchv<order> (ncomp = 3)
 *      (replaces FunctionSpace::init + DofTable::build, feelpp/feel/feeldiscr/
 *      functionspace.hpp:1314-1440, doftable.hpp:1802-1970, 2364-2455) ---- */
int fgpu_space_create(fgpu_ctx* ctx, fgpu_mesh* mesh, int order, int ncomp, fgpu_space** out);
int fgpu_space_ndof(const fgpu_space* V, int64_t* ndof, int* nloc);
/* local-to-global table, T x (nloc*ncomp), local index nloc*c + l
 * (DofTable::localToGlobalIndices, feelpp/feel/feeldiscr/doftable.hpp:742) */
int fgpu_space_l2g(const fgpu_space* V, int32_t* out);
/* dofs of the faces owned by one element (boundaryfaces(mesh)); with xmax_on only
 * faces whose vertices all have x <= xmax (a marked face range). Call with dofs
 * == NULL to get the count. (IntegratorOnExpr::onFaces, feelpp/feel/feelvf/on.hpp:457-701) */
int fgpu_space_boundary_dofs(const fgpu_space* V, int xmax_on, double xmax, int64_t* count, int32_t* dofs);
int fgpu_space_destroy(fgpu_space* V);

/* ---- matrix (replaces Backend::newMatrix -> stencil() -> GraphCSR::close ->
 *      MatrixPetsc::init, feelpp/feel/feelalg/backend.hpp:349-452,
 *      feelpp/feel/feeldiscr/stencil.hpp:1500-1692, feelpp/feel/feelalg/graphcsr.cpp:634-660,
 *      990-1020, matrixpetsc.cpp:316-415). The pattern is COUPLED with a nonzero diagonal. ---- */
int fgpu_matrix_create(fgpu_ctx* ctx, fgpu_space* test, fgpu_space* trial, int precision, fgpu_matrix** out);
/* a matrix with the same pattern and another value precision (values not copied) */
int fgpu_matrix_create_like(const fgpu_matrix* A, int precision, fgpu_matrix** out);
int fgpu_matrix_info(const fgpu_matrix* A, int64_t* nrows, int64_t* nnz, int* precision);
/* host copies of the CSR arrays; any pointer may be NULL (values as double) */
int fgpu_matrix_get_csr(const fgpu_matrix* A, int64_t* ia, int32_t* ja, double* val);
/* the same with 32-bit row offsets, the PetscInt width of a default PETSc build that
 * MatSeqAIJSetPreallocationCSR takes (MatrixPetsc::init, feelpp/feel/feelalg/matrixpetsc.hpp:625,
 * matrixpetsc.cpp:405-413); FGPU_ERR_INVALID when nnz does not fit in int32 */
int fgpu_matrix_get_csr32(const fgpu_matrix* A, int32_t* ia, int32_t* ja, double* val);
/* device pointer of the value array (double or float per precision) */
int fgpu_matrix_values_device(const fgpu_matrix* A, void** dptr);
/* MatrixPetsc::zero (MatZeroEntries, matrixpetsc.cpp:617-627) */
int fgpu_matrix_zero(fgpu_matrix* A);
/* dst = (precision of dst) src values, same pattern */
int fgpu_matrix_convert(const fgpu_matrix* src, fgpu_matrix* dst);
int fgpu_matrix_destroy(fgpu_matrix* A);

/* ---- a = integrate(elements(mesh), expr) / a += ... (BilinearForm::operator= / +=
 *      -> Integrator::assemble -> BilinearForm::Context::integrate/assemble ->
 *      MatrixPetsc::addMatrix; feelpp/feel/feelvf/bilinearform.hpp:1440-1456,
 *      integrator.hpp:975-1238, bilinearformcontext.hpp:458-628, 784-847,
 *      feelpp/feel/feelalg/matrixpetsc.cpp:919-935). accumulate = 0 for '=', 1 for '+='. ---- */
int fgpu_assemble_matrix(fgpu_ctx* ctx, fgpu_matrix* A, const fgpu_form_desc* form, int accumulate);
/* same, with the per-element coefficient already on the device (T doubles) */
/* assemble (accumulate = 0) and write the values to host memory (nnz doubles, CSR order): for the
 * two-phase FP64 Laplace/mass path the gather runs in four ranges of entries and each range is copied
 * to the host while the next is gathered (pin host_val for the overlap); other forms assemble, then
 * copy. The device values are the same as after fgpu_assemble_matrix. */
int fgpu_assemble_matrix_host(fgpu_ctx* ctx, fgpu_matrix* A, const fgpu_form_desc* form, double* host_val);
/* element matrices on the tensor cores, a mask of
 *   FGPU_TC_F32 (default on): binary32 element matrices of the quadrature form (curved tetrahedra,
 *     hexahedra: the per-point contraction K_e = sum_q dphi^T G_q dphi + m_q phi phi^T of
 *     BilinearForm::Context::integrate, feelpp/feel/feelvf/bilinearformcontext.hpp:585-589) with
 *     tcgen05 kind::tf32, 3xTF32 products, FP32 accumulation in tensor memory;
 *   FGPU_TC_DF64 (default off): FP64-accurate element matrices of the affine Laplace/mass form in the
 *     two-phase assembly with tcgen05 kind::f16 on exact bf16 slices of the coefficients and the
 *     reference tensors (levels of slice products summed exactly in FP32); values within ~3e-14 of
 *     sum_k |c_k T_k| of the CUDA-core df64 kernel's, not the same bits, and slower than it on GB300
 *     (0.42 against 0.33 ms for the P2 64^3 element phase).
 * 0 keeps every element kernel on the CUDA cores. */
#define FGPU_TC_F32 1
#define FGPU_TC_DF64 2
int fgpu_set_tensor_cores(fgpu_ctx* ctx, int mask);
/* FGPU_HOST_TRANSFER_* for later fgpu_assemble_matrix_host calls (default AUTO) */
int fgpu_set_host_transfer(fgpu_ctx* ctx, int mode);
int fgpu_assemble_matrix_dev(fgpu_ctx* ctx, fgpu_matrix* A, const fgpu_form_desc* form, const double* d_kappa,
                             int accumulate);

/* ---- vectors (replaces VectorPetsc, feelpp/feel/feelalg/vectorpetsc.cpp) ---- */
int fgpu_vector_create(fgpu_ctx* ctx, int64_t n, fgpu_vector** out);
int fgpu_vector_upload(fgpu_vector* v, const double* host);
int fgpu_vector_download(const fgpu_vector* v, double* host);
int fgpu_vector_zero(fgpu_vector* v);
int fgpu_vector_device(const fgpu_vector* v, double** dptr);
int fgpu_vector_destroy(fgpu_vector* v);

/* ---- l = integrate(elements(mesh), f*id(v)) (LinearForm::operator= / +=,
 *      feelpp/feel/feelvf/linearform.hpp:1209-1230, linearformcontext.hpp:305, 395-410) ---- */
int fgpu_assemble_vector(fgpu_ctx* ctx, const fgpu_space* V, const fgpu_rhs_desc* rhs, fgpu_vector* out,
                         int accumulate);

/* ---- a += on(range, rhs=l, element=u, expr=g) (feelpp/feel/feelvf/on.hpp:1140-1190 ->
 *      MatrixPetsc::zeroRows, feelpp/feel/feelalg/matrixpetsc.cpp:1762-1860).
 *      dofs: host array of ndofs global dof indices; values: g at those dofs (NULL = 0). ---- */
int fgpu_dirichlet(fgpu_ctx* ctx, fgpu_matrix* A, fgpu_vector* rhs, int64_t ndofs, const int32_t* dofs,
                   const double* values, int mode, double diag);

/* ---- y = A x (MatrixSparse::multVector / MatMult) ---- */
int fgpu_matrix_mult(fgpu_ctx* ctx, const fgpu_matrix* A, const fgpu_vector* x, fgpu_vector* y);

/* ---- a.solve(_rhs=l, _solution=u) with --ksp-type=cg --pc-type=jacobi
 *      (BilinearFormBase::solve -> Backend::solve -> SolverLinearPetsc::solve,
 *      feelpp/feel/feelvf/bilinearformbase.hpp:447-466, feelpp/feel/feelalg/
 *      solverlinearpetsc.cpp:490-570). A32 is used by the mixed solver (may be
 *      NULL: then it is made from A). x is the initial guess and the solution. ---- */
/* ---- KSPGMRES, the reference's default ksp-type (feelpp/feel/feelalg/backend.cpp:56, 733 -> PETSc
 *      KSPSolve, solverlinearpetsc.cpp:490-570): restarted GMRES(restart; 0 = 30) with right
 *      preconditioning (pc NONE, JACOBI, or GAMG with `amg` from fgpu_amg_create on A), stopping when
 *      ||b - A x||_2 <= rtol ||b||_2; for non-symmetric matrices (elimination without symmetric
 *      column zeroing, non-symmetric Nitsche terms). x holds the initial guess. ---- */
int fgpu_solve_gmres(fgpu_ctx* ctx, const fgpu_matrix* A, fgpu_amg* amg, const fgpu_vector* b, fgpu_vector* x,
                     const fgpu_solver_cfg* cfg, int restart, fgpu_solve_stats* stats);
int fgpu_solve_cg(fgpu_ctx* ctx, const fgpu_matrix* A, const fgpu_matrix* A32, const fgpu_vector* b, fgpu_vector* x,
                  const fgpu_solver_cfg* cfg, fgpu_solve_stats* stats);
/* ---- the same solve to tolerances below the binary64 floor of stiff systems (the reference's
 *      KSPSolve with rtol 1e-10 on the clamped elasticity beam): iterative refinement whose solution is
 *      the unevaluated double-double sum x + x_lo and whose outer residual b - A (x + x_lo) is formed in
 *      double-double arithmetic; each outer step solves for the correction with the solver of cfg
 *      (pc JACOBI / CHEB_JACOBI / NONE, or GAMG with `amg` of A; mixed allowed without GAMG) to a
 *      relative reduction inner_reduction (0 = 1e-6). Stops when the double-double residual reaches
 *      cfg->rtol ||b||; stats->rel_residual is that residual, stats->outer the outer steps, stats->iterations
 *      the inner iterations. x holds the initial guess; x_lo (may be NULL) receives the low part. ---- */
int fgpu_solve_cg_refine_dd(fgpu_ctx* ctx, const fgpu_matrix* A, fgpu_amg* amg, const fgpu_vector* b, fgpu_vector* x,
                            fgpu_vector* x_lo, const fgpu_solver_cfg* cfg, double inner_reduction, fgpu_solve_stats* stats);

/* ---- --pc-type=gamg (PCGAMG smoothed aggregation, feelpp/feel/feelalg/preconditionerpetsc.cpp:2229-2330):
 *      fgpu_amg_create builds the hierarchy from the FP64 matrix A as it is now (host set-up: strength
 *      graph, aggregation, smoothed prolongators, Galerkin products; levels then kept on the device in
 *      binary32); fgpu_amg_update rebuilds it from A's current values; fgpu_solve_cg_amg runs CG in the
 *      arithmetic of cfg->arith (FP64 or df64; cfg->mixed must be 0) preconditioned by one V-cycle per
 *      iteration (Chebyshev level smoothers, dense coarsest solve). A must outlive the hierarchy. ---- */
int fgpu_amg_create(fgpu_ctx* ctx, const fgpu_matrix* A, const fgpu_amg_cfg* cfg, fgpu_amg** out);
int fgpu_amg_update(fgpu_amg* amg);
/* levels, rows[level], nnz[level] (arrays of at least 16 entries or NULL), set-up time in ms */
int fgpu_amg_info(const fgpu_amg* amg, int* nlevels, int64_t* rows, int64_t* nnz, double* setup_ms);
/* levels whose set-up ran on the device, and the set-up's phases in ms (9 entries or NULL): strength
 * graph, greedy aggregation (host), lambda_max, prolongator and restriction, Galerkin products, host
 * set-up of the levels below the device ones (all levels with setup_on_host), level layouts and
 * uploads, total; then the code of the step that handed a level of more than 16384 rows to the host
 * (0 none, 1 strength graph, 2 node graph, 3 nothing to coarsen, 4 A P0, 5 R = P^T, 6 A P, 7 R (A P)) */
int fgpu_amg_setup_info(const fgpu_amg* amg, int* device_levels, double* phases_ms);
int fgpu_amg_destroy(fgpu_amg* amg);
int fgpu_solve_cg_amg(fgpu_ctx* ctx, const fgpu_matrix* A, fgpu_amg* amg, const fgpu_vector* b, fgpu_vector* x,
                      const fgpu_solver_cfg* cfg, fgpu_solve_stats* stats);

/* ---- p-multigrid for matrix-free operators (FGPU_PC_PMG): op32 = the binary32 order-p operator (its
 *      Dirichlet dofs set), A1 = the assembled FP64 P1 form on the same mesh with the same coefficients and
 *      Dirichlet rows eliminated, amg = fgpu_amg_create(A1). One V-cycle: Chebyshev smoothing of degree
 *      smoother_degree on op32, restriction to P1 by the transpose of the P1 -> Pp interpolation, one
 *      AMG V-cycle, prolongation, post-smoothing. fgpu_solve_cg_operator_pmg runs the matrix-free solve of
 *      fgpu_solve_cg_operator (plain binary64 or mixed) with it as preconditioner. ---- */
typedef struct {
    int smoother_degree;      /* Chebyshev degree of the order-p smoothing (0 = 3: two operator sweeps) */
    int coarse_cycles;        /* AMG V-cycles per coarse solve (0 = 4, at most 4) */
} fgpu_pmg_cfg;
int fgpu_pmg_create(fgpu_ctx* ctx, fgpu_operator* op32, const fgpu_matrix* A1, fgpu_amg* amg, const fgpu_pmg_cfg* cfg,
                    fgpu_pmg** out);
/* lambda_max(D^-1 A_p) estimate, coarse rows, set-up time */
int fgpu_pmg_info(const fgpu_pmg* pmg, double* lmax, int64_t* coarse_rows, double* setup_ms);
int fgpu_pmg_destroy(fgpu_pmg* pmg);

/* host-only hierarchy (no device): the same set-up from a host CSR, for inspection and tests.
 * fgpu_amg_host_level: rows, nnz of A_l, nnz and columns of P_l (0 on the coarsest), lmax(D^-1 A_l);
 * fgpu_amg_host_export: copies A_l (ia n+1, ja, a), P_l (ia n+1, ja, a) and the aggregate of each
 * row (-1: left out) into caller arrays (NULL skips); fgpu_amg_host_coarse_inverse: 1 and the dense
 * inverse of the coarsest operator (row-major) when one was formed, else 0. */
typedef struct fgpu_amg_host fgpu_amg_host;
int fgpu_amg_host_build(int64_t n, const int64_t* ia, const int32_t* ja, const double* a, const fgpu_amg_cfg* cfg, int nthreads,
                        fgpu_amg_host** out);
int fgpu_amg_host_levels(const fgpu_amg_host* h);
int fgpu_amg_host_level(const fgpu_amg_host* h, int level, int64_t* n, int64_t* nnz, int64_t* p_nnz, int64_t* p_cols, double* lmax);
int fgpu_amg_host_export(const fgpu_amg_host* h, int level, int64_t* ia, int32_t* ja, double* a, int64_t* pia, int32_t* pja,
                         double* pa, int32_t* agg);
int fgpu_amg_host_coarse_inverse(const fgpu_amg_host* h, double* out);
int fgpu_amg_host_destroy(fgpu_amg_host* h);
/* the device set-up's hierarchy of an assembled FP64 matrix, copied into a host inspection object
 * (replaces the host set-up of fgpu_amg_create; amg_setup.cpp's construction, same bits);
 * fgpu_amg_host_device_levels: how many of its levels the device built (0 for fgpu_amg_host_build) */
int fgpu_amg_device_build(fgpu_ctx* ctx, const fgpu_matrix* A, const fgpu_amg_cfg* cfg, fgpu_amg_host** out);
/* the six rigid body modes of a Pchv (ncomp = 3) space at its dof nodes (affine element maps): the
 * translations along x, y, z and the rotations (-y, x, 0), (0, -z, y), (z, 0, -x) about the centroid
 * of the mesh vertices; out: six vectors of the space's size (created by the caller) */
int fgpu_space_rigid_body_modes(const fgpu_space* V, fgpu_vector* const* out);
int fgpu_amg_host_device_levels(const fgpu_amg_host* h);

/* ---- EnSight Gold export (the reference's default exporter, feelpp/feel/feelfilters/exporterensightgold.hpp):
 *      writes prefix.case, prefix.geo (C Binary, one part of tetra4, vertex coordinates) and
 *      prefix.<name>.scl per field (values at the vertices: the vertex dofs of the scalar space V).
 *      Field names: 1-19 characters among letters, digits and '_'. ---- */
int fgpu_export_ensight(const fgpu_space* V, const char* prefix, int nfields, const char* const* names,
                        const fgpu_vector* const* fields);

/* ---- error norms of a scalar field against u = sin(pi x) sin(pi y) sin(pi z):
 *      normL2(u_h - u) and the H1 seminorm (feelpp/feel/feelvf/norml2.hpp:37, normh1.hpp) ---- */
int fgpu_norms_sine(fgpu_ctx* ctx, const fgpu_space* V, const fgpu_vector* u, int quad_degree, double* l2, double* h1);

/* ---- matrix-free operator of a form (the reference applies form-level operators with
 *      MatrixShell::multVector, feelpp/feel/feelalg/matrixshell.hpp:49,120 and
 *      OperatorLinearFree::apply, feelpp/feel/feeldiscr/operatorlinearfree.hpp:116-170;
 *      there is no element-level one). precision: FGPU_F32, FGPU_F64 (native) or FGPU_DF64.
 *      Dirichlet dofs are eliminated symmetrically (the operator then equals the assembled
 *      matrix after on(..., elimination_symmetric)). ---- */
int fgpu_operator_create(fgpu_ctx* ctx, fgpu_space* V, const fgpu_form_desc* form, int precision, fgpu_operator** out);
int fgpu_operator_set_dirichlet(fgpu_operator* op, int64_t ndofs, const int32_t* dofs);
int fgpu_operator_apply(fgpu_ctx* ctx, fgpu_operator* op, const fgpu_vector* x, fgpu_vector* y);
int fgpu_operator_destroy(fgpu_operator* op);
/* run the binary32 element phase on the tensor cores (tcgen05.mma kind::tf32, 3xTF32 split,
 * accumulator in tensor memory); P2 / P3 binary32 operators (default: on for P3, off for P2, the
 * faster of the two for each order) */
int fgpu_operator_set_tensor_cores(fgpu_operator* op, int on);
/* binary32 operators: FGPU_ALGO_GATHER (element buffer, then one node-ordered gather; default) or
 * FGPU_ALGO_COLOUR (elements coloured so that a colour shares no vertex, one launch per colour
 * adds y_e into y: no element buffer, no node phase; sums in colour order) */
int fgpu_operator_set_algo(fgpu_operator* op, int algo);
/* tensor-core self-check: D = A B^T with A 128 x 24 and B 144 x 24 (row-major binary32, host
 * arrays) through the same staging / descriptors / MMA / read-back as the operator */
int fgpu_tc_selftest(fgpu_ctx* ctx, const float* A, const float* B, float* D);
/* matrix-free PCG (Jacobi from the operator diagonal): plain with a binary64 operator, or
 * mixed (cfg->mixed) with a binary32 inner operator op32 refined by op's residual */
int fgpu_solve_cg_operator(fgpu_ctx* ctx, fgpu_operator* op, fgpu_operator* op32, const fgpu_vector* b, fgpu_vector* x,
                           const fgpu_solver_cfg* cfg, fgpu_solve_stats* stats);
/* the same with the p-multigrid preconditioner pmg (cfg->pc = FGPU_PC_PMG; see fgpu_pmg_create) */
int fgpu_solve_cg_operator_pmg(fgpu_ctx* ctx, fgpu_operator* op, fgpu_operator* op32, fgpu_pmg* pmg, const fgpu_vector* b,
                               fgpu_vector* x, const fgpu_solver_cfg* cfg, fgpu_solve_stats* stats);

/* ---- host-only queries (no device needed): the dof numbering, the sparsity
 *      pattern and the reference tables the device kernels use ---- */
/* dof table of Pch/Pchv<order> on a mesh: l2g (T x nloc*ncomp) as fgpu_space_l2g;
 * returns the number of dofs in *ndof (DofTable::build, doftable.hpp:1802-1970) */
int fgpu_host_dof_table(int64_t nv, int64_t nt, const int32_t* tets, int order, int ncomp, int32_t* l2g,
                        int64_t* ndof);
/* CSR pattern of Pch/Pchv<order> (Stencil::computeGraph + GraphCSR::close). Call with
 * ja == NULL to fill ia (ndof + 1) and get *nnz, then again with ja (nnz). */
int fgpu_host_pattern(int64_t nv, int64_t nt, const int32_t* tets, int order, int ncomp, int64_t* ia, int32_t* ja,
                      int64_t* nnz);
/* Q1/Q2 on hexahedra: first-encounter dof table (nh x 8 or nh x 27) and the reference tables (local dof
 * points n x 3, Gauss points Q x 3 and weights, basis values Q x n and reference gradients Q x n x 3;
 * call with NULL arrays to get Q) */
int fgpu_host_hex_dof_table(int64_t nv, int64_t nh, const int32_t* hexes, int order, int32_t* l2g, int64_t* ndof);
int fgpu_host_hex_ref_tables(int order, int qdeg, double* nodes, double* qx, double* qw, double* phi, double* dphi, int* nq);
/* Lagrange node set (nloc x 3), basis values (Q x nloc) and reference gradients
 * (Q x nloc x 3) at the degree-qdeg rule, and the reference tensors
 * S (9 x nloc x nloc) and M (nloc x nloc); any output may be NULL. Returns Q in *npts. */
int fgpu_host_ref_tables(int order, int qdeg, double* nodes, double* phi, double* dphi, double* S, double* M,
                         int* npts);

/* ---- load vector without device allocation (no counterpart in the reference).
 *      For callers that cannot call cudaMalloc when they assemble: the device memory
 *      belongs to the host application's pool allocator, or allocation is forbidden
 *      after set-up (fixed-latency stepping, code later captured into graphs).
 *      Same result as fgpu_assemble_vector; the per-element scratch lives in a
 *      static device array of FGPU_NOALLOC_MAX_ELEMENT_VALUES doubles (16 MiB, held
 *      by every GPU that loads the library until exit), so T*nloc*ncomp must not
 *      exceed it (else FGPU_ERR_INVALID). The first call on a device sets it up
 *      (symbol lookup + table copy) and must come before any stream capture. All
 *      calls share the scratch: calls that overlap on the GPU race. d_out is a
 *      device array of ndof doubles; stream is a cudaStream_t (NULL = default),
 *      which the caller orders after the context's stream (the space's arrays are
 *      uploaded there). Tetrahedral P1-P3 spaces and the element sources SINE,
 *      CONST and CONST_VEC only; anything else is refused with a message. ---- */
#define FGPU_NOALLOC_MAX_ELEMENT_VALUES (1 << 21)
int fgpu_assemble_vector_noalloc(const fgpu_space* V, const fgpu_rhs_desc* rhs, double* d_out, int accumulate,
                                 void* stream);

/* ---- Dirichlet rows as a device object, for repeated application (each time
 *      step's reassembled matrix) and for graph capture. Same semantics as
 *      fgpu_dirichlet (on(), feelpp/feel/feelvf/on.hpp:1140-1190 ->
 *      MatrixPetsc::zeroRows, matrixpetsc.cpp:1762-1860); n = rows of the
 *      matrices it is applied to. ---- */
int fgpu_bc_create(fgpu_ctx* ctx, int64_t n, int64_t ndofs, const int32_t* dofs, const double* values, fgpu_bc** out);
int fgpu_bc_apply(fgpu_ctx* ctx, const fgpu_bc* bc, fgpu_matrix* A, fgpu_vector* rhs, int mode, double diag);
int fgpu_bc_destroy(fgpu_bc* bc);

/* ---- vector updates (VectorPetsc::add / scale, feelpp/feel/feelalg/vectorpetsc.cpp):
 *      y = a x + b y; dst = src ---- */
int fgpu_vector_axpby(fgpu_ctx* ctx, double a, const fgpu_vector* x, double b, fgpu_vector* y);
int fgpu_vector_copy(fgpu_ctx* ctx, const fgpu_vector* src, fgpu_vector* dst);

/* ---- CUDA graphs of library calls (no reference counterpart: Feel++ re-runs
 *      its host loops every time step). Between fgpu_graph_begin and
 *      fgpu_graph_end the context's stream is captured; these calls may be
 *      captured: fgpu_assemble_matrix_dev, fgpu_assemble_matrix without host
 *      kappa (kappa_elem NULL), fgpu_batch_assemble, fgpu_bc_apply,
 *      fgpu_matrix_mult, fgpu_vector_axpby, fgpu_vector_copy, fgpu_vector_zero,
 *      fgpu_vector_upload (from pinned host memory: the copy reads the host
 *      buffer when the graph runs), fgpu_assemble_vector_noalloc on the
 *      context's stream. Every captured call must have run once before the
 *      capture (first calls allocate and upload tables); other calls return
 *      FGPU_ERR_INVALID while capturing. Status words of captured kernels are
 *      checked by fgpu_graph_launch, which replays the graph `count` times and
 *      then synchronizes. ---- */
int fgpu_graph_begin(fgpu_ctx* ctx);
int fgpu_graph_end(fgpu_ctx* ctx, fgpu_graph** out);
int fgpu_graph_launch(fgpu_ctx* ctx, fgpu_graph* g, int count);
int fgpu_graph_destroy(fgpu_graph* g);

/* ---- batches of independent problems (no reference counterpart as one call:
 *      replaces a loop of form2 assemblies over independent meshes,
 *      feelpp/feel/feelvf/integrator.hpp:975-1238 per mesh). mats: nprob
 *      matrices of scalar spaces (orders 1-3, one precision) created with
 *      fgpu_matrix_create; descs: their Laplace/mass forms (default quadrature);
 *      d_kappa: nprob device arrays of per-element kappa (or NULL / NULL
 *      entries). fgpu_batch_assemble runs all problems in three launches
 *      (geometry, element matrices, gather map: the bits of FGPU_ALGO_TWO_PHASE)
 *      when their buffers fit in device memory, else two (geometry, persistent
 *      fused gather with a device work queue: the bits of FGPU_ALGO_GATHER); the
 *      launch shape is tuned on the first '=' call; fgpu_batch_get_launch
 *      reports it, chunk = 0 for a two-phase batch. ---- */
int fgpu_batch_create(fgpu_ctx* ctx, int nprob, fgpu_matrix* const* mats, const fgpu_form_desc* descs,
                      const double* const* d_kappa, fgpu_batch** out);
int fgpu_batch_assemble(fgpu_ctx* ctx, fgpu_batch* b, int accumulate);
int fgpu_batch_set_launch(fgpu_batch* b, int threads, int chunk);
int fgpu_batch_set_algo(fgpu_batch* b, int algo);   /* FGPU_ALGO_GATHER, _TWO_PHASE or _AUTO; re-tunes */
int fgpu_batch_get_launch(const fgpu_batch* b, int* threads, int* chunk, int* tuned);
int fgpu_batch_destroy(fgpu_batch* b);

/* df64 (double-float) arithmetic self-check on the host: op 0 round trip double->df64->double,
 * 1 a+b, 2 a*b, 3 1/a, 4 a-b, all through df64; writes n results */
int fgpu_host_df64_ops(int op, int64_t n, const double* a, const double* b, double* out);

/* ---- per-kernel device timings (CUDA events), enabled by fgpu_config.profile ---- */
int fgpu_prof_reset(fgpu_ctx* ctx);
/* total device time and launch count of the kernels tagged `name` */
int fgpu_prof_get(fgpu_ctx* ctx, const char* name, int64_t* count, double* total_ms);

#ifdef __cplusplus
}
#endif
#endif /* FGPU_H */
