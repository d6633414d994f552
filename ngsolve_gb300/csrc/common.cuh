// common.cuh -- internal structures and helpers of libgh1 (not part of the ABI).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>
#include <array>
#include <stdexcept>
#include <cstdio>
#include "../../include/gh1.h"

namespace gh1 {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define GH1_CUDA(call)                                                                  \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      throw ::gh1::Error(e_ == cudaErrorMemoryAllocation ? GH1_ERR_NOMEM : GH1_ERR_CUDA, \
                         std::string(#call) + ": " + cudaGetErrorString(e_));          \
  } while (0)
#define GH1_CHECK(cond, code, msg) \
  do { if (!(cond)) throw ::gh1::Error(code, msg); } while (0)
#define GH1_LAUNCH_CHECK() GH1_CUDA(cudaGetLastError())

constexpr int MAX_HEX_ORDER = 8;   // n = p+1 <= 9 per direction
constexpr int MAX_TET_ORDER = 8;
constexpr int N_TET_CLASSES = 24;  // permutations of 4 vertex ranks
constexpr int TET_NQ_MAX = 24;     // symmetric rules of degree <= 6 (order p <= 4)

// device buffer with RAII
template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  explicit DBuf(size_t count) { alloc(count); }
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  ~DBuf() { release(); }
  void alloc(size_t count) {
    release();
    if (count) GH1_CUDA(cudaMalloc((void**)&p, count * sizeof(T)));
    n = count;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr; n = 0;
  }
  void upload(const T* h, size_t count, cudaStream_t s) {
    if (n != count) alloc(count);
    if (count) GH1_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
  }
  void upload(const std::vector<T>& h, cudaStream_t s) { upload(h.data(), h.size(), s); }
  void zero(cudaStream_t s) { if (n) GH1_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s)); }
  size_t bytes() const { return n * sizeof(T); }
};

}  // namespace gh1

struct gh1_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  int nsm = 0;
  int cc_major = 0, cc_minor = 0;
  // scratch for reductions
  gh1::DBuf<double> red;        // partial sums
  gh1::DBuf<unsigned int> cnt;  // completion counters
  double* h_pinned = nullptr;   // small pinned host staging
};

struct gh1_mesh {
  gh1_ctx* ctx = nullptr;
  int nv = 0, ne = 0, et = 0;
  std::vector<double> X;
  std::vector<int32_t> el;
  gh1::DBuf<double> d_X;
  gh1::DBuf<int32_t> d_el;
  // deformation field (gh1_mesh_set_deformation): [3][ndof] in the H1 space
  // def_space (borrowed) of this mesh; operators made while it is set see the
  // deformed, curved elements
  gh1_space* def_space = nullptr;
  gh1::DBuf<double> d_def;
};

struct gh1_space {
  gh1_ctx* ctx = nullptr;
  gh1_mesh* mesh = nullptr;
  int et = 8, p = 1, nloc = 0, n1 = 2;  // n1 = p+1 (hex DOFs per direction)
  int nvert = 8, nedge = 12, nface = 6;
  int64_t ndof = 0, nfree = 0;
  int ned = 0, nfa = 0;
  int n_edge_dofs = 0, n_face_dofs = 0, n_cell_dofs = 0;
  int64_t first_edge = 0, first_face = 0, first_cell = 0;
  std::vector<int32_t> el_dofs;   // ne*nloc, reference local order
  std::vector<uint8_t> freedof;   // ndof
  // Dirichlet on the caller's boundary faces only (sorted vertex numbers,
  // padded with INT32_MAX); read by the space construction, then released
  bool dir_select = false;
  std::vector<std::array<int32_t, 4>> dir_faces;
  gh1::DBuf<int32_t> d_eldofs;    // ne*nloc (reference local order)
  gh1::DBuf<uint8_t> d_free;      // ndof
  // hex: tensor-ordered signed DOF table  tdof[e*tstride + (a*n+b)*n+c] = dof | (sign<0 ? 1<<31 : 0);
  // the per-element stride is padded to 16 bytes so rows can be bulk-copied
  gh1::DBuf<int32_t> d_tdof;
  int tstride = 0;
  // hex: integration rule (Gauss, q = p+1 points) and 1D tables B[q][n], D[q][n]
  int nq1 = 0;                    // points per direction
  std::vector<double> gx, gw;     // Gauss points / weights on [0,1]
  gh1::DBuf<double> d_gx, d_gw;
  gh1::DBuf<double> d_B64, d_D64;
  gh1::DBuf<float> d_B32, d_D32;
  // tet: orientation class per element, rule, per-class tables
  gh1::DBuf<uint8_t> d_class;     // ne
  int tet_nq = 0, tet_nq_mass = 0;
  gh1::DBuf<double> d_tq, d_tqm;  // rules: (x,y,z,w) * nq
  gh1::DBuf<double> d_tab64;      // [class][q][i][4]  (value, dx, dy, dz) at stiffness rule
  gh1::DBuf<float> d_tab32;
  gh1::DBuf<double> d_tabm64;     // [class][q][i] values at mass/rhs rule
  gh1::DBuf<double> d_S;          // [class][7][nloc][nloc] reference stiffness/mass blocks
  // CSR pattern (built lazily)
  bool have_graph = false;
  int64_t nnz = 0;
  gh1::DBuf<int64_t> d_rowptr;
  gh1::DBuf<int32_t> d_colind;
  gh1_mesh* def_of = nullptr;     // the mesh whose deformation field lives in this space
};

// G = s * Ji K Ji^T for the symmetric tensor K = (xx yy zz xy xz yz), written
// as the metric components (xx yy zz xy xz yz); Ji is the inverse Jacobian,
// row-major, so that the mapped gradient is Ji^T times the reference gradient.
__device__ __forceinline__ void tensor_metric(const double* Ji, const double* K, double s, double* g) {
  const double Km[9] = {K[0], K[3], K[4], K[3], K[1], K[5], K[4], K[5], K[2]};
  double T[9];  // Ji K
  for (int a = 0; a < 3; a++)
    for (int l = 0; l < 3; l++) T[3 * a + l] = Ji[3 * a] * Km[l] + Ji[3 * a + 1] * Km[3 + l] + Ji[3 * a + 2] * Km[6 + l];
  const int ia[6] = {0, 1, 2, 0, 0, 1}, ib[6] = {0, 1, 2, 1, 2, 2};
  for (int c = 0; c < 6; c++) {
    const int a = ia[c], b = ib[c];
    g[c] = s * (T[3 * a] * Ji[3 * b] + T[3 * a + 1] * Ji[3 * b + 1] + T[3 * a + 2] * Ji[3 * b + 2]);
  }
}

struct gh1_form {
  gh1_space* sp = nullptr;
  gh1::DBuf<double> d_kappa;  // ne
  gh1::DBuf<double> d_mu;     // ne (empty: mu = 0)
  bool has_mu = false;
  gh1::DBuf<double> d_K6;     // ne x 6 symmetric diffusion tensors (xx yy zz xy xz yz); empty: kappa I
  bool has_K6 = false;
  // generic B^T D B form (gh1_form_set_bdb): D in physical coordinates, row =
  // test component (v, dv/dx, dv/dy, dv/dz), column = trial component; [ne][4][4]
  // (bdb_mode 1) or [ne][nq][4][4] at the points of the space's rule (bdb_mode 2).
  // While set it replaces kappa / mu / K6.
  gh1::DBuf<double> d_bdb;
  int bdb_mode = 0;
  int version = 0;            // bumped on coefficient change
  // references: the caller's (dropped by gh1_form_free) plus one per operator
  // made from the form (dropped when the operator is freed); the form is
  // destroyed when the last one goes
  int refs = 1;
  // gh1_adjoint_grad cache: this form's operator (FP64 + FP32 data; its metrics
  // follow coefficient changes) and the unit-mass operator for J and the adjoint
  // right-hand side; released with the form
  gh1_op* adj_A = nullptr;
  gh1_form* adj_mass = nullptr;
  gh1_op* adj_M = nullptr;
  gh1_form() = default;
  gh1_form(const gh1_form&) = delete;
  gh1_form& operator=(const gh1_form&) = delete;
  ~gh1_form();  // api.cu
};

struct gh1_op {
  gh1_ctx* ctx = nullptr;
  int kind = GH1_OP_CSR;
  gh1_form* form = nullptr;   // NULL for imported CSR
  bool form_ref = false;      // this operator holds a reference on form (released with it)
  gh1_space* sp = nullptr;
  int64_t nrows = 0;
  gh1_op* inner = nullptr;    // GH1_OP_BLOCK: the repeated operator (borrowed)
  int nblocks = 0;            // GH1_OP_BLOCK: copies of inner on consecutive slices
  // CSR data
  int64_t nnz = 0;
  gh1::DBuf<int64_t> d_rowptr_own;
  gh1::DBuf<int32_t> d_colind_own;
  const int64_t* rowptr = nullptr;
  const int32_t* colind = nullptr;
  gh1::DBuf<double> d_vals;
  gh1::DBuf<float> d_vals32;
  // matrix-free data
  int prec_mask = 1;
  int form_version = -1;
  // hex: G[e*gstride + c*nq + q], c = xx yy zz xy xz yz (+ mass coefficient as c = 6);
  //      gstride padded to a multiple of 16 bytes (bulk-copy rows)
  // tet: G[e*6 + c] and M[e]
  gh1::DBuf<double> d_G64;
  gh1::DBuf<float> d_G32;
  int ncomp = 6, gstride64 = 0, gstride32 = 0;
  gh1::DBuf<double> d_M64;    // tet mass coefficient [e]
  gh1::DBuf<float> d_M32;
  // generic B^T D B operator: 0 = none; 1 = reference-coordinate matrices
  // Mh = w |det J| T^T D T per rule point in G (hex [e][16][nq] with gstride,
  // tet [e][nq][16]); 2 = per-element Mh without the rule weight, [e][16] (affine
  // elements with D per element), weighted in the kernel.  T = diag(1, J^{-T}).
  int bdb = 0;
  int bdb_per_sm[2] = {0, 0};                // hex: resident blocks of the B^T D B apply [FP64/FP32]
  bool bdb_pair = false;                     // hex: the FP32 apply on the paired kernel (G mode 3 of
                                             // hexpair.cu with records per element, 4 per point), timed
                                             // against the one-element kernel
  bool bdb_points_only = false;              // hex: per-point records even for affine elements (assembly)
  // a generic form of Laplace type on hexes (D = diag(mu, K), K symmetric) runs on
  // the standard kernels: per element through these coefficient arrays, per point
  // through lap_pp (the form's D, read by the metric kernel)
  bool lap_ov = false;
  gh1::DBuf<double> d_ovK6, d_ovmu;
  const double* lap_pp = nullptr;
  int tet_ncb = 0;                           // tet: 16-point chunks of the degree-2p rule
  gh1::DBuf<double> d_tetB64, d_tetBw64;     // tet: [class][chunk][nlocp][64] value and reference-gradient
  gh1::DBuf<float> d_tetB32, d_tetBw32;      //      rows (component*16 + point), weights [chunk*16]
  gh1::DBuf<int> d_err;       // device error flag of the pipelined apply (bounded waits)
  int hex_per_sm[2][2] = {{0, 0}, {0, 0}};  // resident blocks per SM of the hex apply [FP64/FP32][G mode]
  int hex_gmode[2] = {0, 0};                 // autotuned hex apply variant per precision: 0/1 = G tile by TMA /
                                             // direct loads; FP32 also 2/3 = the same with two elements per lane,
                                             // 4 = two elements per lane with per-element (affine) metrics,
                                             // 5 = slice / pencil form of 4 (hexpair.cu),
                                             // 6 = 1D contractions on the tensor cores (hextc.cu)
  int pair_per_sm[5] = {0, 0, 0, 0, 0};      // resident blocks per SM of the paired FP32 apply [G mode]
  int slice_per_sm = 0;                      // ... of the slice-form FP32 apply (0: not available)
  int tc_per_sm = 0;                         // ... of the tensor-core FP32 apply (0: not available)
  bool all_affine = false;                   // hex: every element map affine (G mode 2 available)
  gh1::DBuf<float> d_Ga32;                   // hex, all affine: per-element metric records [ne][8]
  int multi_per_sm[2] = {0, 0};              // resident blocks per SM of the multi-rhs apply
  int multi_pair_per_sm = 0;                 // ... of the FP32 multi-rhs apply with two rhs per lane
  int multi_pair = -1;                       // FP32 multi-rhs apply: 1 = two rhs per lane, 0 = one
                                             // (timed per problem by gh1_batch_create; -1: not timed, two)
  int spmv_L[2] = {0, 0};                    // autotuned SpMV sub-warp width (FP64, FP32)
  bool has_mass = false;
  // tet tiled apply (tetapply.cu): elements sorted by orientation class, tiles of
  // up to 32 same-class elements, per-class GEMM tables
  gh1::DBuf<int> d_tet_perm;                 // class-sorted element order
  gh1::DBuf<int> d_tet_tiles;                // [ntiles][4] = class, first position, count, 0
  gh1::DBuf<int> d_tet_tdofs;                // [ntiles][nlocp][TET_TE]: DOF of local DOF i of tile
                                             // element e (-1 past the tile's count or nloc)
  int tet_ntiles = 0, tet_R = 0, tet_Rp = 0, tet_Rs = 0;
  gh1::DBuf<double> d_tetD64, d_tetw64;      // [class][nloc][Rs] table rows, per-row weights [Rp]
  gh1::DBuf<float> d_tetD32, d_tetw32;
  int tet_tiles_per_sm[2] = {0, 0};          // [FP64/FP32] resident blocks; 0: does not fit, element-wise kernel
  bool tet_chunked = false;                  // tables streamed in 16-point chunks (orders with large rules)
  int tet_tc_per_sm = 0;                     // resident CTAs of the tensor-core FP32 tet apply (0: not available)
  int tet_tc_ntiles = 0;                     // its tiles of up to 128 same-class elements
  gh1::DBuf<int> d_tet_tc_tiles;             // [ntiles][4] = class, first position, count, 0
  gh1::DBuf<float> d_tet_tc_tab;             // per class: both B operands, TF32 hi / lo parts, in the
                                             // kernel's shared-memory layout (copied as is)
  gh1::DBuf<int> d_tet_tc_dofs;              // [tile][nloc][128]: DOF of local DOF i of tile row m
                                             // (0 past the tile's count), coalesced per i
  gh1::DBuf<float> d_tet_tc_G;               // [tile][6][128]: the FP32 metric of tile row m (rebuilt
                                             // with the metric)
  bool tet_use_tc = false;                   // FP32 tet apply on the tensor cores (timed at setup)
  bool tet_bdb_tc = false;                   // FP32 tet B^T D B (records per element) on the tensor cores
  int tet_bdb_tc_per_sm = 0;                 // its resident CTAs (0: not available)
  gh1::DBuf<float> d_tet_bdb_tab;            // its class operands (TF32 hi / lo, shared-memory layout)
  gh1::DBuf<float> d_tet_bdb_M;              // its element records tile-major [tile][16][128]
  int tet_ncg = 0, tet_ncm = 0;              // gradient / mass-rule chunks
  gh1::DBuf<double> d_tetDm64, d_tetwm64;    // chunked mass-rule tables and weights
  gh1::DBuf<float> d_tetDm32, d_tetwm32;
  gh1::DBuf<double> d_diag;   // operator diagonal (FP64)
  bool have_diag = false;
  // scratch vectors for accumulate / scaling
  gh1::DBuf<double> d_tmp64;
  gh1::DBuf<float> d_tmp32;
  gh1_op() = default;
  gh1_op(const gh1_op&) = delete;
  gh1_op& operator=(const gh1_op&) = delete;
  ~gh1_op();  // api.cu: drops the form reference
};

struct gh1_pre {
  gh1_op* op = nullptr;        // Jacobi: the operator of the diagonal (NULL otherwise)
  gh1_ctx* ctx = nullptr;
  int64_t n = 0;
  int kind = 0;                // 0 Jacobi, 1 block Jacobi, 2 exact low-order solve, 3 sum a + b
  gh1::DBuf<double> d_inv64;   // Jacobi: 1/A_ii on free DOFs, 0 elsewhere
  gh1::DBuf<float> d_inv32;
  gh1::DBuf<uint8_t> d_free;   // free-DOF mask (the true-residual norm of CG)
  // block Jacobi: block b holds bdofs[boff[b] .. boff[b+1]), its inverse (row-major) at binv[moff[b]]
  int64_t nblocks = 0;
  int smax = 0;
  gh1::DBuf<int64_t> d_boff, d_moff;
  gh1::DBuf<int32_t> d_bdofs;
  gh1::DBuf<double> d_binv64;
  gh1::DBuf<float> d_binv32;
  // low-order solve: dense inverse of the coarse matrix on its nc free DOFs, cfine[a] = fine DOF of coarse DOF a
  int nc = 0;
  gh1::DBuf<int32_t> d_cfine;
  gh1::DBuf<double> d_cinv64;
  gh1::DBuf<float> d_cinv32;
  gh1_pre* a = nullptr;        // sum: the two parts (borrowed)
  gh1_pre* b = nullptr;
};

namespace gh1 {
// *p += v as a reduction (red.global: nothing is returned, the add completes in
// L2 without a round trip to the SM): the scatter of every apply, assembly and
// diagonal kernel.  atomicAdd with its result unused measured slower here.
__device__ __forceinline__ void red_add(float* p, float v) {
  asm volatile("red.global.add.f32 [%0], %1;" ::"l"(p), "f"(v) : "memory");
}
__device__ __forceinline__ void red_add(double* p, double v) {
  asm volatile("red.global.add.f64 [%0], %1;" ::"l"(p), "d"(v) : "memory");
}
// form references held by operators (api.cu)
void form_retain(gh1_form* f);
void form_release(gh1_form* f);
// host helpers implemented in api.cu
int grid_for(gh1_ctx* ctx, int64_t work, int block, int per_sm = 8);
void check_kernel(gh1_ctx* ctx, const char* what);

// kernels / drivers (implemented in the .cu files)
void build_tables(gh1_space* sp);                                   // tables.cu
// values and reference gradients [class][q][i][4] at the degree-2p tet rule (tables.cu)
void tet_mass_rule_tables(gh1_space* sp, gh1::DBuf<double>& t64, gh1::DBuf<float>& t32);
int space_rule_size(const gh1_space* sp);                           // points of the B^T D B rule
void space_qpoints(gh1_space* sp, double* ref /* nq x 4 or NULL */, double* xyz /* device, ne x nq x 3 or NULL */);
void bdb_setup(gh1_op* op);                                         // bdb.cu
bool bdb_laplace_route(gh1_op* op);                                 // bdb.cu: hex generic form of Laplace type?
void bdb_apply(gh1_op* op, const void* x, void* y, int prec, double* partial, unsigned int* counter, double* energy,
               const int* skip);                                    // bdb.cu
void bdb_diag(gh1_op* op, double* diag);                            // bdb.cu
void tet_bdb_setup(gh1_op* op);                                     // tetapply.cu
void tet_bdb_apply(gh1_op* op, int prec, const void* x, void* y, double* partial, unsigned int* counter,
                   double* energy, const int* skip);                // tetapply.cu
void tet_bdb_diag(gh1_op* op, double* diag);                        // tetapply.cu
void tet_bdb_assemble(gh1_op* op, const int64_t* rowptr, const int32_t* colind, double* vals, int* bad);  // tetapply.cu
void build_graph(gh1_space* sp);                                    // assemble.cu (host)
bool build_graph_gpu(gh1_space* sp);                                // graph.cu
void assemble_csr(gh1_form* f, double* vals);                       // assemble.cu
void rhs_elementwise(gh1_space* sp, const double* f, double* b);    // assemble.cu
void matfree_setup(gh1_op* op);                                     // matfree.cu
void matfree_apply(gh1_op* op, const void* x, void* y, int prec, double* energy_partials, unsigned int* counter,
                   double* energy_out);                              // matfree.cu
void matfree_diag(gh1_op* op, double* diag);                        // matfree.cu
void elem_grad_dot(gh1_space* sp, const double* u, const double* w, double* out);  // matfree.cu
void elem_grad_dot_with(gh1_op* op, const double* u, const double* w, double* out);  // matfree.cu
int matfree_apply_multi(gh1_op* op, int R, const int* phase, int want, const void* x, void* y, int prec, double* partial,
                        unsigned int* counter, double* energy, bool prepare_only);  // matfree.cu
void matfree_apply_ex(gh1_op* op, const void* x, void* y, int prec, double* partial, unsigned int* counter,
                      double* energy, const int* skip);  // matfree.cu
void mass_apply(gh1_op* op, const double* x, double* y);            // matfree.cu
void spmv(gh1_op* op, const void* x, void* y, int prec);            // spmv.cu
// tiled tet apply (tetapply.cu): setup after the tet geometry; apply returns false
// when the tiled kernel does not fit (the caller then runs the element-wise kernel)
void tet_tiles_setup(gh1_op* op);
bool tet_tiles_apply(gh1_op* op, int prec, const void* x, void* y, double* partial, unsigned int* counter,
                     double* energy, const int* skip);
// paired FP32 hex apply (hexpair.cu): two elements per lane, packed f32x2 arithmetic
bool hex_pair_supported(int N);
void set_first_wait_polls();  // hexpair.cu: GH1_FIRST_WAIT_POLLS (timeout-path tests)
void upload_pair_tables(gh1_space* sp);
int hex_pair_occupancy(gh1_op* op, int gmode);
void hex_affine_setup(gh1_op* op);
int hex_multi_pair_launch(gh1_op* op, int R, const int* phase, int want, const float* x, float* y, double* partial,
                          unsigned int* counter, double* energy, bool prepare_only);
void hex_pair_apply(gh1_op* op, int gmode, const float* x, float* y, double* partial, unsigned int* counter,
                    double* energy, const int* skip);
// slice / pencil form of the paired apply for all-affine meshes (hexpair.cu)
bool hex_slice_supported(int N);
void hex_slice_setup(gh1_op* op);
void hex_slice_apply(gh1_op* op, const float* x, float* y, double* partial, unsigned int* counter, double* energy,
                     const int* skip);
// FP32 tet apply with both tile products on the tensor cores (tettc.cu)
bool tet_tc_supported(int p);
void tet_tc_setup(gh1_op* op);
// tensor-core tet B^T D B (tettc.cu): setup from the degree-2p tables [class][q][i][4]
// (t64, FP64), after the class tiles and the element records; apply
void tet_bdb_tc_setup(gh1_op* op, const double* t64);
// the same kernel for standard FP32 tet forms with a mass term (records from
// kappa / K and mu, bdb.cu tet_standard_records), kept when faster than the tiles
void tet_mass_tc_setup(gh1_op* op);
void tet_standard_records(gh1_op* op, float* M32);  // bdb.cu
void tet_mass_rule_tables(gh1_space* sp, gh1::DBuf<double>& t64, gh1::DBuf<float>& t32);  // tables.cu
void tet_bdb_tc_apply(gh1_op* op, const float* x, float* y, double* partial, unsigned int* counter, double* energy,
                      const int* skip);
void tet_tc_apply(gh1_op* op, const float* x, float* y, double* partial, unsigned int* counter, double* energy,
                  const int* skip);
// FP32 hex apply with the 1D contractions on the tensor cores (hextc.cu)
bool hex_tc_supported(int N);
int hex_tc_occupancy(gh1_op* op);
void hex_tc_apply(gh1_op* op, const float* x, float* y, double* partial, unsigned int* counter, double* energy,
                  const int* skip);
void spmv_prepare(gh1_op* op, int prec);                            // spmv.cu (call before capture)
// preconditioners (precond.cu): block Jacobi, exact low-order solve, their sum;
// pre_apply_any launches kernels only (capturable), pre_prepare before capture
void block_jacobi_setup(gh1_pre* pr, gh1_op* csr, int64_t nblocks, const std::vector<int64_t>& off,
                        const std::vector<int32_t>& dofs);
void coarse_setup(gh1_pre* pr, gh1_op* csr, int64_t nfine, const std::vector<int32_t>& embed,
                  const std::vector<uint8_t>& cfreemask);
void pre_apply_any(gh1_pre* pr, double s, const void* x, void* y, int prec, int accumulate);
void pre_prepare(gh1_pre* pr);
void smoothing_blocks(gh1_space* sp, int blocktype, std::vector<int64_t>& off, std::vector<int32_t>& dofs);
// any operator kind (api.cu): y = A x into a y the call zeroes first where the kind
// needs it; skip as for the CG graph kernels; prepare / refresh before capture
void op_apply_any(gh1_op* op, const void* x, void* y, int prec, const int* skip);
void op_prepare_any(gh1_op* op, int prec);
void op_refresh_any(gh1_op* op);
void op_check_err(gh1_op* op);  // throws GH1_ERR_CUDA if a bounded wait of the apply ran out
void spmv_skip(gh1_op* op, const void* x, void* y, int prec, const int* skip);  // spmv.cu
void csr_diag(gh1_op* op, double* diag);                            // spmv.cu
int cg_solve(gh1_op* op, gh1_pre* pre, const double* b, double* x, const gh1_cg_opts* o, gh1_cg_result* r);  // cg.cu
void vec_axpby(gh1_ctx* ctx, int64_t n, double a, const void* x, double b, void* y, int prec);  // cg.cu
void jacobi_invert(gh1_ctx* ctx, int64_t n, const double* diag, const uint8_t* freedof, double* inv64, float* inv32);  // cg.cu
void jacobi_apply(gh1_ctx* ctx, int64_t n, double s, const double* inv64, const float* inv32, const void* x, void* y,
                  int prec, int accumulate);  // cg.cu
void shape_eval_gpu(gh1_ctx* ctx, int et, int p, const int32_t* vnums, int npts, const double* pts, double* val,
                    double* grad);  // tables.cu
}  // namespace gh1
