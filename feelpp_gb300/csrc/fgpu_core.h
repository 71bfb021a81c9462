// Internal declarations of the GB300 assembly backend (not part of the C-ABI).
#pragma once
#include <atomic>
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/fgpu.h"

namespace fgpu {

struct StreamPlan;                   // schedule of the streamed assembly (stream_asm.cu)
void stream_plan_free(StreamPlan* p);

// ---------------------------------------------------------------------------
// Reference tetrahedron conventions (Feel++: feelpp/feel/feelmesh/refsimplex.hpp:151-165,
// feelpp/feel/feelmesh/simplexordering.hpp:284-293 edges, :341-347 faces).
// ---------------------------------------------------------------------------
extern const int kEdgeVerts[6][2];
extern const int kFaceVerts[4][3];

inline int nloc_of(int order) { return (order + 1) * (order + 2) * (order + 3) / 6; }
inline int dofs_per_edge(int order) { return order - 1; }
inline int dofs_per_face(int order) { return order >= 3 ? (order - 1) * (order - 2) / 2 : 0; }

// Tabulated Lagrange basis of order p on a quadrature rule, and the reference
// tensors of the affine Laplacian / mass / elasticity forms.
struct RefTables {
    int order = 0, n = 0, qdeg = 0, Q = 0;
    std::vector<double> nodes;  // n x 3
    std::vector<double> qx, qw; // Q x 3, Q
    std::vector<double> phi;    // Q x n
    std::vector<double> dphi;   // Q x n x 3 (reference gradients)
    std::vector<double> S;      // 9 x n x n : S[ab][i][j] = sum_q w_q d_a phi_i d_b phi_j
    std::vector<double> M;      // n x n     : sum_q w_q phi_i phi_j
    std::vector<double> T7;     // 7 x n x n : symmetric Laplacian/mass tensors (S00,S11,S22,S01+S10,S02+S20,S12+S21,M)
};
bool lagrange_nodes(int order, std::vector<double>& xyz);
bool build_ref_tables(int order, int qdeg, RefTables& out, std::string& err);

struct FaceTables {                  // boundary-face integrals per unit face area
    int order = 0, n = 0;
    std::vector<double> Mf;          // 4 x n x n : (1/|f|) int_f phi_i phi_j
    std::vector<double> Lf;          // 4 x n     : (1/|f|) int_f phi_i
    std::vector<double> Gf;          // 4 x 3 x n x n : (1/|f|) int_f phi_i dphi_j/dxhat_a
    std::vector<double> Df;          // 4 x 3 x n : (1/|f|) int_f dphi_i/dxhat_a
};
bool build_face_tables(int order, FaceTables& out, std::string& err);

// ---------------------------------------------------------------------------
// Host topology: entities, DOF numbering, colouring, sparsity pattern.
// ---------------------------------------------------------------------------
struct Topology {
    int order = 0;
    int n = 0;                       // scalar local dofs per element
    int64_t nnodes = 0;              // scalar dof nodes
    std::vector<int32_t> l2n;        // T x n : element -> dof node (first-encounter numbering)
    std::vector<int64_t> inc_ptr;    // nnodes + 1
    std::vector<int32_t> inc;        // (element << 5) | local index, sorted by element per node
    std::vector<uint8_t> edge_rev;   // T x 6 (1 when the element's edge is REVERSE-permuted)
};
bool build_topology(int64_t nv, int64_t nt, const int32_t* tets, int order, Topology& topo, std::string& err);

// hexahedral meshes (Q1 geometry; Q1/Q2 spaces)
extern const int kHexEdgeVerts[12][2];
extern const int kHexFaceVerts[6][4];
int hex_nloc(int order);
void hex_dof_points(int order, std::vector<double>& pts);
bool build_hex_ref_tables(int order, int qdeg, RefTables& out, std::string& err);
bool build_hex_topology(int64_t nv, int64_t nh, const int32_t* hexes, int order, Topology& topo, std::string& err);
bool hex_boundary_nodes(int64_t nh, const int32_t* hexes, const double* xyz, const Topology& topo, int xmax_on, double xmax,
                        std::vector<int32_t>& nodes);

struct NodePattern {                 // scalar node-to-node pattern (COUPLED + diagonal)
    int64_t nrows = 0, nnz = 0;
    int max_row = 0;
    std::vector<int64_t> ia;
    std::vector<int32_t> ja;
};
bool build_node_pattern(const Topology& topo, int64_t nt, NodePattern& pat, int nthreads, std::string& err);

int colour_elements(int64_t nv, int64_t nt, const int32_t* tets, std::vector<int32_t>& perm,
                    std::vector<int64_t>& colour_ptr);
int boundary_faces_coloured(int64_t nt, const int32_t* tets, const double* xyz, int xmax_on, double xmax, int whole_element,
                            std::vector<int32_t>& faces, std::vector<int64_t>& colour_ptr);

// Smoothed-aggregation AMG hierarchy built on the host (amg_setup.cpp).
struct HostCsr {
    int64_t nrows = 0, ncols = 0;
    std::vector<int64_t> ia;
    std::vector<int32_t> ja;
    std::vector<double> a;
};
struct AmgHostLevel {
    HostCsr A;                       // level operator
    HostCsr P, R;                    // prolongator from the next coarser level, R = P^T (empty on the coarsest)
    std::vector<int32_t> agg;        // aggregate of each row (-1: left out)
    double lmax = 0;                 // lmax(D^-1 A) estimate (Lanczos)
};
struct AmgHostCfg {
    double threshold = 0.0;          // strength threshold (pc-gamg-threshold)
    int max_levels = 10;             // pc-mg-levels
    int coarse_eq_lim = 800;         // pc-gamg-coarse-eq-lim
    int agg_smooths = 1;             // pc-gamg-nsmooths (0: unsmoothed aggregation)
    int nthreads = 0;                // host threads (0: all)
};
struct AmgHierarchy {
    std::vector<AmgHostLevel> levels;
    std::vector<double> coarse_inv;  // dense inverse of the coarsest operator (row-major), or empty
};
constexpr int64_t kAmgDenseCoarse = 2048;   // largest coarsest level inverted densely
// Near null space of a level (PETSc's MatNullSpace given to GAMG, e.g. the rigid body modes of an
// elasticity space): m vectors on the level's dofs, the dofs grouped in nodes (consecutive ranges).
// Aggregation then runs on the nodes and each aggregate's tentative prolongator is the Q of the QR
// factorisation of the vectors restricted to its dofs; R gives the next level's vectors.
struct AmgNns {
    int m = 0;
    std::vector<int64_t> node_ptr;   // nodes + 1 dof offsets
    std::vector<double> B;           // ndof x m, row-major
};
bool amg_build_host(HostCsr&& A0, const AmgHostCfg& cfg, AmgHierarchy& H, std::string& err, const AmgNns* nns = nullptr);
// node graph of a dof graph: nodes I, J coupled when a dof of I and a dof of J are (no self loops)
void amg_collapse_graph(const std::vector<int64_t>& node_ptr, const std::vector<int64_t>& sp, const int32_t* sj, int nthreads,
                        std::vector<int64_t>& np, std::vector<int32_t>& nj);
// tentative prolongator of node aggregates from the near null space; `coarse` receives the next level's
int amg_tentative_nns(const AmgNns& nns, const std::vector<int32_t>& agg_node, int64_t nagg, int nthreads, HostCsr& P0,
                      AmgNns& coarse);
AmgHostCfg amg_host_cfg(const fgpu_amg_cfg* cfg, int nthreads);
int amg_nns_layout(const fgpu_amg_cfg* cfg, int64_t n, AmgNns& nns);
// pieces of the host set-up shared with the device set-up (amg_dev.cu)
// key of a node in the aggregation's independent-set rounds: a hash of the index above the index
__host__ __device__ inline uint64_t amg_mis_key(int64_t i) {
    uint64_t z = (uint64_t)i + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return ((z >> 32) << 32) | (uint64_t)(uint32_t)i;
}
void amg_lanczos_start(int64_t n, std::vector<double>& v);
double amg_tridiag_lmax(const std::vector<double>& al, const std::vector<double>& be);

// The hierarchy built on the device (amg_dev.cu): device CSR levels down to the first level handed to
// the host set-up; `tail` holds that level and the ones below it.
struct AmgDevCsr {
    int64_t nrows = 0, ncols = 0, nnz = 0;
    int64_t* ia = nullptr;
    int32_t* ja = nullptr;
    double* a = nullptr;
    bool own = true;                 // false: a view of arrays owned elsewhere
    AmgDevCsr() = default;
    AmgDevCsr(const AmgDevCsr&) = delete;
    AmgDevCsr& operator=(const AmgDevCsr&) = delete;
    AmgDevCsr(AmgDevCsr&& o) noexcept;
    AmgDevCsr& operator=(AmgDevCsr&& o) noexcept;
    ~AmgDevCsr();
};
struct AmgDevLevel {
    AmgDevCsr A, P, R;               // level operator (level 0: a view of the matrix), prolongator, R = P^T
    std::vector<int32_t> agg;
    double lmax = 0;
};
struct AmgSetupTimes {                // wall times of the set-up phases (ms), summed over the levels
    double graph = 0;                // diagonal, strength graph and its copy to the host
    double aggregate = 0;            // aggregation
    double lanczos = 0;              // lambda_max estimate
    double prolong = 0;              // P0, A P0, P, R = P^T
    double galerkin = 0;             // A P and R (A P)
    double tail = 0;                 // host set-up of the levels below the device ones
    double layout = 0;               // level layouts (SELL-C-sigma, binary32 copies) and uploads
    double total = 0;
    int handoff = 0;                 // why the device set-up handed a level of more than 16384 rows to the host:
                                     // 0 none, 1 strength graph, 2 node graph, 3 nothing to coarsen, 4 A P0,
                                     // 5 R = P^T, 6 A P, 7 R (A P) (a row beyond the kernels' staging)
};
struct AmgDevHierarchy {
    std::vector<AmgDevLevel> levels;
    AmgHierarchy tail;
    AmgSetupTimes times;
};
int amg_build_device(fgpu_ctx* ctx, const fgpu_matrix* A, const AmgHostCfg& cfg, AmgDevHierarchy& H, const AmgNns* nns = nullptr);
// the near null space of fgpu_amg_cfg (device vectors) for a matrix of n rows; *has = false without one
int amg_nns_from_cfg(fgpu_ctx* ctx, const fgpu_amg_cfg* cfg, int64_t n, AmgNns& nns, bool* has);
int amg_copy_to_host(fgpu_ctx* ctx, const AmgDevCsr& D, HostCsr& H);

// Boundary dof nodes: the nodes carried by faces owned by one element; when
// `xmax_on` only the faces whose three vertices satisfy x <= xmax (+1e-12).
bool boundary_nodes(int64_t nt, const int32_t* tets, const double* xyz, const Topology& topo, int xmax_on,
                    double xmax, std::vector<int32_t>& nodes);

}  // namespace fgpu

// ---------------------------------------------------------------------------
// Opaque handle definitions.
// ---------------------------------------------------------------------------
struct ProfAcc {
    int64_t count = 0;
    double total_ms = 0;
};
struct PendingEvent {
    std::string name;
    cudaEvent_t start, stop;
};

struct fgpu_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;
    int profile = 0;
    std::map<std::string, ProfAcc> prof;
    std::vector<PendingEvent> pending;
    std::vector<cudaEvent_t> event_pool;
    int* d_status = nullptr;       // device status word written by kernels (bit flags)
    int64_t launches = 0;          // kernels launched by this context
    int host_threads = 1;
    int host_setup = 0;            // 1: dof tables and patterns built on the host (default: device)
    int capturing = 0;             // the stream is being captured into a graph
    int64_t capture_launches0 = 0;
    cudaStream_t copy_streams[4] = {nullptr, nullptr, nullptr, nullptr};   // large host<->device copies in chunks
    cudaEvent_t copy_events[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    int host_transfer = 0;         // FGPU_HOST_TRANSFER_*: how results reach host buffers
    int tune = 0;                  // 0: time launch shapes on first use; -1: fixed default shapes
    std::string tune_file;         // cache file of the picks ("" = none)
    int tensor_cores = FGPU_TC_F32; // element kernels on tcgen05 (fgpu_set_tensor_cores mask)
};

struct fgpu_graph {
    fgpu_ctx* ctx = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t launches = 0;          // kernels per replay
};

struct fgpu_bc {
    fgpu_ctx* ctx = nullptr;
    int64_t n = 0;
    uint8_t* d_mask = nullptr;
    double* d_g = nullptr;         // null: homogeneous
};

struct fgpu_mesh {
    fgpu_ctx* ctx = nullptr;
    int64_t nv = 0, nt = 0;
    std::vector<double> h_xyz;       // host copy (refreshed from the device when stale)
    bool h_xyz_stale = false;
    uint64_t coords_version = 0;     // incremented whenever the coordinates change
    int cv = 4;                      // vertices per element: 4 (tetrahedra) or 8 (hexahedra)
    std::vector<int32_t> h_tets;     // T x cv element vertices
    double* d_xyz = nullptr;
    int32_t* d_tets = nullptr;
    double* d_ho = nullptr;          // curved (P2-geometry) elements: T x 6 x 3 edge nodes (e2p order), or null
    // element colouring (lazily built): elements sorted by colour
    int ncolours = 0;
    std::vector<int64_t> colour_ptr;
    int32_t* d_colour_perm = nullptr;
};

struct DevPattern {                  // device copy of a scalar node pattern
    int64_t nrows = 0, nnz = 0;
    int max_row = 0;
    int64_t* d_ia = nullptr;
    int32_t* d_ja = nullptr;
    ~DevPattern();
};

struct fgpu_space {
    fgpu_ctx* ctx = nullptr;
    fgpu_mesh* mesh = nullptr;
    int order = 0, ncomp = 1, n = 0;
    int64_t ndof = 0;
    fgpu::Topology topo;
    int32_t* d_l2n = nullptr;        // T x n
    int64_t* d_inc_ptr = nullptr;
    int32_t* d_inc = nullptr;
    std::shared_ptr<DevPattern> pattern;   // scalar node pattern, built on demand
    fgpu::NodePattern h_pattern;
    uint8_t* d_pos = nullptr;        // T x n x n: position of node l2n[e][j] in row l2n[e][i] (rows <= 255)
    bool dev_topology = false;       // dof table / incidence built on the device
    int max_incidence = 0;           // longest node -> element list (device build)
    struct FaceSet {                 // boundary faces of a range, coloured (scatter without conflicts)
        int xmax_on = 0;
        double xmax = 0;
        int whole = 0;               // coloured over whole elements (normal-derivative terms)
        int32_t* d_faces = nullptr;  // e * 4 + f, sorted by colour
        std::vector<int64_t> colour_ptr;
    };
    std::vector<FaceSet> face_sets;
    std::vector<int32_t> bnd_nodes;  // last boundary-dof query (range, xmax, coordinates version)
    bool bnd_valid = false;
    int bnd_xmax_on = 0;
    double bnd_xmax = 0;
    uint64_t bnd_coords = 0;
    uint32_t* d_gptr = nullptr;      // two-phase gather map: nnz + 1 offsets into d_gidx
    uint32_t* d_gidx = nullptr;      // T n n element-buffer indices, per CSR entry in element order
    fgpu::StreamPlan* stream_plan = nullptr;   // streamed assembly: task order and waits (built on first use)
};

struct SellLayout {                  // SELL-C-sigma (C = 32, sigma = 256) copy of a CSR pattern
    int64_t nrows = 0, nslices = 0, nstored = 0;
    int32_t* d_perm = nullptr;       // sorted position -> row
    int64_t* d_slice_ptr = nullptr;  // nslices + 1, start of each slice (in entries)
    int32_t* d_slice_len = nullptr;  // max row length in the slice
    int32_t* d_col = nullptr;        // nstored column ids (padding: the row itself)
    int32_t* d_src = nullptr;        // nstored CSR positions of the entries (-1: padding)
    ~SellLayout();
};

struct fgpu_matrix {
    fgpu_ctx* ctx = nullptr;
    fgpu_space* space = nullptr;     // test == trial space
    int precision = FGPU_F64;
    int ncomp = 1;
    int64_t nrows = 0, nnz = 0;
    std::shared_ptr<DevPattern> pattern;   // scalar node pattern
    int64_t* d_ia = nullptr;         // expanded (component) CSR row pointers
    int32_t* d_ja = nullptr;         // expanded column indices (== pattern->d_ja when ncomp == 1)
    bool own_ia_ja = false;
    void* d_val = nullptr;           // nnz values (double or float)
    double* d_coef = nullptr;        // per-element coefficient records of the last assembly
    int64_t coef_cap = 0;
    double* d_kappa_stage = nullptr; // staging copy of a host per-element kappa (T doubles)
    void* d_kbuf = nullptr;          // two-phase assembly: element matrices (upper triangles)
    size_t kbuf_bytes = 0;
    mutable std::shared_ptr<SellLayout> sell; // solver layout, built on first solve
};

struct fgpu_vector {
    fgpu_ctx* ctx = nullptr;
    int64_t n = 0;
    double* d = nullptr;
};

// ---------------------------------------------------------------------------
// Kernel launchers (assemble.cu / solve.cu)
// ---------------------------------------------------------------------------
namespace fgpu {

enum StatusBits : int {
    kStatusBadElement = 1,     // |det K| <= 0 or non-finite
    kStatusRowOverflow = 2,    // a pattern row longer than the kernel's staging buffer
    kStatusMissingEntry = 4,   // an element column absent from its row (pattern mismatch)
    kStatusBreakdown = 8,      // CG breakdown (p.Ap <= 0)
    kStatusStreamTimeout = 256,// streamed assembly: a wait for another task gave up
    kStatusOzTimeout = 1024,   // tensor-core df64 element kernel: a wait for its products gave up
};

// element_tc.cu: df64 element buffer of the affine Laplace/mass form on the tensor cores (orders 1-3)
int launch_element_tri_tc(fgpu_ctx* ctx, int order, int64_t nt, const float4* rec, const float* Th, const float* Tl, void* kbuf);

struct DevTables {                     // device copies of the reference tables
    int order = 0, n = 0, Q = 0, qdeg = 0;
    double* d_T7 = nullptr;            // 7 n n
    double* d_S = nullptr;             // 9 n n
    float* d_T7f = nullptr;
    float* d_Sf = nullptr;
    float* d_T7h = nullptr;            // df64 split of T7: hi = fl32(T), lo = fl32(T - hi)
    float* d_T7l = nullptr;
    float* d_T7th = nullptr;           // the same split in upper-triangle order: 7 x n(n+1)/2
    float* d_T7tl = nullptr;
    uint16_t* d_tri = nullptr;         // n x n: (i, j) -> upper-triangle index of (min, max)
    float* d_Sth = nullptr;            // elasticity tensors S_ab(i, j), i <= j, df64 split: 9 x n(n+1)/2
    float* d_Stl = nullptr;
    double* d_phi = nullptr;           // Q n
    double* d_dphi = nullptr;          // Q n 3
    double* d_qx = nullptr;            // Q 3
    double* d_qw = nullptr;            // Q
};
DevTables* get_dev_tables(int order, int qdeg, std::string& err);

void prof_begin(fgpu_ctx* ctx, const char* name, PendingEvent& ev);
void prof_end(fgpu_ctx* ctx, PendingEvent& ev);

int launch_geometry(fgpu_ctx* ctx, const fgpu_mesh* mesh, int kind, const double* d_kappa, double kappa,
                    double mass, double lam, double mu, double* d_coef);
int launch_assemble_gather(fgpu_ctx* ctx, fgpu_matrix* A, const DevTables* tab, int kind, const double* d_coef,
                           int accumulate);
int launch_assemble_colour(fgpu_ctx* ctx, fgpu_matrix* A, const DevTables* tab, int kind, const double* d_coef,
                           int accumulate);
int launch_geometry_df(fgpu_ctx* ctx, const fgpu_mesh* mesh, const double* d_kappa, double kappa, double mass,
                       float4* d_rec, const double* d_kscale = nullptr);
int launch_assemble_gather_df(fgpu_ctx* ctx, fgpu_matrix* A, const DevTables* tab, const float4* rec, int accumulate);
// inputs of the element coefficient records when the geometry runs inside the element kernel
struct GeoIn {
    const double* xyz = nullptr;
    const int32_t* tets = nullptr;
    const double* kappa = nullptr;     // per element, or null: kc
    double kc = 0.0, mc = 0.0;
    const double* kscale = nullptr;    // device factor of kappa, or null
};
// two-phase Laplace/mass assembly from coefficient records (rec) or with the geometry fused into the
// element kernel (rec null, geo given)
int launch_assemble_two_phase(fgpu_ctx* ctx, fgpu_matrix* A, const DevTables* tab, const float4* rec, const GeoIn* geo, int accumulate);
constexpr int kStreamedUnsupported = -1;   // launch_assemble_streamed: use the two-phase path
int launch_assemble_streamed(fgpu_ctx* ctx, fgpu_matrix* A, const DevTables* tab, const double* d_kappa, double kappa,
                             double mass, const double* kscale, int accumulate, double* hout);
int launch_geometry_el_df(fgpu_ctx* ctx, const fgpu_mesh* mesh, double lam, double mu, float4* d_rec);
int launch_assemble_elasticity_two_phase(fgpu_ctx* ctx, fgpu_matrix* A, const DevTables* tab, const float4* rec, int accumulate);
int launch_build_gather_map(fgpu_ctx* ctx, fgpu_space* V);
int mf_apply_f32_gated(fgpu_ctx* ctx, fgpu_operator* op, const float* x, float* y, const int* stop);
int64_t operator_nnodes(const fgpu_operator* op);
int operator_precision(const fgpu_operator* op);
const fgpu_space* operator_space(const fgpu_operator* op);
const uint8_t* operator_mask(const fgpu_operator* op);
const float* operator_diag_f32(fgpu_ctx* ctx, fgpu_operator* op);
int amg_vcycle_f32(fgpu_amg* M, const float* r, const int* stop, const float** x, int cycles);
int64_t amg_rows(const fgpu_amg* M);
const fgpu_ctx* amg_context(const fgpu_amg* M);
int build_sell(fgpu_ctx* ctx, const fgpu_matrix* A, std::shared_ptr<SellLayout>& out);
int solve_gmres(fgpu_ctx* ctx, const fgpu_matrix* A, fgpu_amg* amg, const double* b, double* x, const fgpu_solver_cfg* cfg,
                int restart, fgpu_solve_stats* st);
int ensure_two_phase(fgpu_ctx* ctx, fgpu_matrix* A, size_t need);
int launch_assemble_two_phase_host(fgpu_ctx* ctx, fgpu_matrix* A, const DevTables* tab, const float4* rec, const GeoIn* geo,
                                   double* host);
int launch_gather_phase_to_host(fgpu_ctx* ctx, fgpu_matrix* A, double* host, int nchunks);
int launch_gather_phase(fgpu_ctx* ctx, fgpu_matrix* A, int accumulate);
int launch_rhs_gather(fgpu_ctx* ctx, const fgpu_space* V, const double* d_work, double* d_out, int accumulate);
int launch_assemble_ho(fgpu_ctx* ctx, fgpu_matrix* A, const fgpu_form_desc* f, const double* d_kappa, int accumulate);
int launch_rhs_ho(fgpu_ctx* ctx, const fgpu_space* V, const fgpu_rhs_desc* rhs, double* d_out, int accumulate);
int launch_assemble_hex(fgpu_ctx* ctx, fgpu_matrix* A, const fgpu_form_desc* f, const double* d_kappa, int accumulate);
int launch_rhs_hex(fgpu_ctx* ctx, const fgpu_space* V, const fgpu_rhs_desc* rhs, double* d_out, int accumulate);
int boundary_nodes_device(fgpu_ctx* ctx, const fgpu_space* V, int xmax_on, double xmax, std::vector<int32_t>& nodes);
int launch_face_matrix(fgpu_ctx* ctx, fgpu_matrix* A, int range, double xmax, double mass, double mass_h, double dn_trial,
                       double dn_test, int accumulate);
int launch_face_load(fgpu_ctx* ctx, const fgpu_space* V, int range, double xmax, double g, double g_h, double g_dn,
                     double* d_rhs, int accumulate);
int build_space_device(fgpu_ctx* ctx, fgpu_space* V);
int build_pattern_device(fgpu_ctx* ctx, fgpu_space* V, DevPattern& P, std::vector<int64_t>& h_ia);
int launch_build_positions(fgpu_ctx* ctx, fgpu_space* V);

// One problem of a batch (device-side descriptor, built by batch.cu).
struct BatchProblem {
    int order, n, maxrow, pad;
    int64_t row0, nrows;             // global row range
    int64_t elem0, nt;               // global element range
    const int64_t* sia;              // scalar pattern rows
    const int64_t* inc_ptr;
    const int32_t* inc;
    const uint8_t* pos;
    const double* xyz;
    const int32_t* tets;
    const double* kappa;             // per-element kappa (device) or null
    double kappa_c, mass;
    float4* rec;                     // coefficient records (the matrix's d_coef)
    void* val;                       // matrix values
    // two-phase batches
    int64_t nz0, nnz;                // global CSR entry range
    const uint32_t* gptr;            // the space's gather map
    const uint32_t* gidx;
    void* kbuf;                      // the matrix's element buffer
};
struct BatchLaunch {                 // launch configuration picked by the batch tuner
    int threads = 256;
    int chunk = 16;                  // rows taken per work-queue grab
};
int launch_batch_geometry(fgpu_ctx* ctx, int nprob, const BatchProblem* d_probs, const int64_t* d_elem_off,
                          int64_t total_elems);
int launch_batch_two_phase(fgpu_ctx* ctx, int nprob, const BatchProblem* d_probs, const int64_t* d_grp_off,
                           int64_t total_groups, const int64_t* d_nz_off, int64_t total_nnz, int f32, int threads,
                           int accumulate);
int launch_batch_gather(fgpu_ctx* ctx, int nprob, const BatchProblem* d_probs, const int64_t* d_row_off,
                        int64_t total_rows, int f32, int acc_floats, unsigned long long* d_counter,
                        const BatchLaunch& cfg, int accumulate);
int launch_rhs(fgpu_ctx* ctx, const fgpu_space* V, const DevTables* tab, int fkind, const double* fc,
               double* d_out, int accumulate, double* d_work);
int launch_dirichlet(fgpu_ctx* ctx, fgpu_matrix* A, double* d_rhs, const uint8_t* d_mask, const double* d_g,
                     int mode, double diag);
int launch_axpby(fgpu_ctx* ctx, int64_t n, double a, const double* x, double b, double* y);
int launch_spmv(fgpu_ctx* ctx, const fgpu_matrix* A, const double* x, double* y, double alpha_b, const double* b);
int launch_convert_values(fgpu_ctx* ctx, const fgpu_matrix* src, fgpu_matrix* dst);

int solve_pcg(fgpu_ctx* ctx, const fgpu_matrix* A, const double* d_b, double* d_x, const fgpu_solver_cfg* cfg,
              fgpu_solve_stats* st, fgpu_amg* amg = nullptr);
int solve_pcg_mixed(fgpu_ctx* ctx, const fgpu_matrix* A64, const fgpu_matrix* A32, const double* d_b, double* d_x,
                    const fgpu_solver_cfg* cfg, fgpu_solve_stats* st);
// launch-shape autotuner store (tune.cpp)
void tune_load_cache_file(const std::string& path);
bool tune_lookup(const std::string& file, const std::string& key, std::vector<int>& vals);
void tune_record(const std::string& file, const std::string& key, const std::vector<int>& vals);
std::string tune_device_key(int device);
int tune_size_class(int64_t n);

int solve_refine_dd(fgpu_ctx* ctx, const fgpu_matrix* A, const fgpu_matrix* A32, fgpu_amg* amg, const double* b, double* xh,
                    double* xl_out, const fgpu_solver_cfg* cfg, double inner_reduction, fgpu_solve_stats* st);

}  // namespace fgpu

#define FGPU_CUDA_CHECK(ctx, call)                                                        \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            (ctx)->err = std::string(#call) + ": " + cudaGetErrorString(e_);              \
            return FGPU_ERR_CUDA;                                                         \
        }                                                                                 \
    } while (0)

// A hierarchy held for inspection (fgpu_amg_host_*): built on the host, or on the device and copied
// (device_levels = the levels the device set-up built).
struct fgpu_amg_host {
    fgpu::AmgHierarchy H;
    int device_levels = 0;
};
