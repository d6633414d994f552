/* gh1.h -- C ABI of the GB300-native high-order H1 operator library.
 *
 * This library replaces, on one GPU, the hot path of NGSolve's H1 Poisson
 * stack: shape/gradient evaluation at integration points, element-matrix
 * assembly into a CSR SparseMatrix, sum-factorized matrix-free Apply on hexes
 * (element-wise B^T D B on tets), CSR SpMV, Jacobi-preconditioned CG (FP64 and
 * FP32-inner/FP64-refined), the adjoint dJ/dkappa contraction and batched solves.
 *
 * Conventions
 *  - Every entry point returns an int status (GH1_OK = 0) and never throws;
 *    gh1_last_error(ctx) gives the message of the last failure on a context.
 *  - Vectors passed to apply / solve calls are DEVICE pointers of the
 *    precision named in the call (double* for GH1_F64, float* for GH1_F32).
 *    Setup arrays (coordinates, connectivity, coefficients) are HOST pointers
 *    unless a `mem` argument says GH1_MEM_DEVICE.
 *  - All device work is ordered on the context's stream (gh1_set_stream).
 *    A context is not thread safe: use one per host thread.
 *  - Element types: 4 = tetrahedron, 8 = hexahedron, vertex order as in
 *    NGSolve's ET_trait<ET_TET>/<ET_HEX> (fem/elementtopology.cpp:74-119).
 *  - DOF numbering follows H1HighOrderFESpace::UpdateDofTables/GetDofNrs
 *    (comp/h1hofespace.cpp:823-950, :1389-1420): vertices, then edges, faces,
 *    cells; edges and faces are numbered by their sorted global vertex tuples.
 */
#ifndef GH1_H
#define GH1_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  GH1_OK = 0,
  GH1_ERR_ARG = 1,          /* invalid argument (the message says which)       */
  GH1_ERR_CUDA = 2,         /* a CUDA runtime call failed                       */
  GH1_ERR_NOMEM = 3,        /* device allocation failed                         */
  GH1_ERR_UNSUPPORTED = 4,  /* element type / order / precision not provided    */
  GH1_ERR_ILLEGAL_DNUMS = 5,/* scatter met a column missing from the pattern    */
  GH1_MAXITER = 6,          /* solver stopped at maxit without reaching tol     */
  GH1_BREAKDOWN = 7         /* CG breakdown: s^T A s <= 0 or a NaN appeared     */
};
enum { GH1_F64 = 0, GH1_F32 = 1 };
enum { GH1_MEM_HOST = 0, GH1_MEM_DEVICE = 1 };
enum { GH1_OP_CSR = 0, GH1_OP_MATFREE = 1, GH1_OP_BLOCK = 2 };

typedef struct gh1_ctx gh1_ctx;
typedef struct gh1_mesh gh1_mesh;
typedef struct gh1_space gh1_space;
typedef struct gh1_form gh1_form;
typedef struct gh1_op gh1_op;
typedef struct gh1_pre gh1_pre;

/* ---- lifetime ---------------------------------------------------------- */
int gh1_create(gh1_ctx** ctx, int device);
int gh1_destroy(gh1_ctx* ctx);
/* stream: a cudaStream_t (NULL = legacy default stream) */
int gh1_set_stream(gh1_ctx* ctx, void* stream);
const char* gh1_last_error(gh1_ctx* ctx);
int gh1_version(void);

/* ---- mesh and space -----------------------------------------------------
 * Replaces MeshAccess + H1HighOrderFESpace construction
 * (comp/meshaccess.cpp:1670, comp/h1hofespace.cpp:564-950).            */
int gh1_mesh_upload(gh1_ctx* ctx, int nv, const double* coords /*nv*3*/, int ne, int et,
                    const int32_t* elem_vertices /*ne*et*/, gh1_mesh** mesh);
int gh1_mesh_free(gh1_mesh* mesh);
/* dirichlet: 1 = all boundary DOFs are Dirichlet (dirichlet=".*"), 0 = none */
int gh1_space_h1(gh1_mesh* mesh, int order, int dirichlet, gh1_space** space);
/* H1 space with Dirichlet conditions on the listed boundary faces only: the
 * FESpace "dirichlet" regular expression resolved to the boundary elements
 * whose condition name it matches (comp/fespace.cpp:440-516, 765-830); the
 * DOFs of those faces, of their edges and of their vertices are not free.
 * faces: host int32[nbf*3] (tets) or [nbf*4] (hexes), vertex numbers in any
 * order.  A face that is not a face of the mesh, or an interior face, is
 * GH1_ERR_ARG; nbf = 0 leaves every DOF free.                                */
int gh1_space_h1_bnd(gh1_mesh* mesh, int order, int64_t nbf, const int32_t* faces, gh1_space** space);
int gh1_space_free(gh1_space* space);
/* info[0..5] = ndof, nloc, nedges, nfaces, nfree, ne */
int gh1_space_info(gh1_space* space, int64_t* info);
/* element DOF numbers in NGSolve's local order (GetDofNrs), host ne*nloc */
int gh1_space_get_dofs(gh1_space* space, int32_t* elem_dofs);
/* FreeDofs() as one byte per DOF, host ndof */
int gh1_space_get_freedofs(gh1_space* space, uint8_t* freedofs);
/* shape values and reference gradients at points, evaluated on the GPU with the
 * element's vertex numbers (H1HighOrderFE::CalcShape/CalcDShape,
 * fem/tscalarfe_impl.hpp:24-56); host out: val[npts*nloc], grad[npts*nloc*3] */
int gh1_shape_eval(gh1_ctx* ctx, int et, int order, const int32_t* vnums, int npts,
                   const double* pts, double* val, double* grad);

/* ---- bilinear form  kappa_e grad u.grad v + mu_e u v --------------------
 * Replaces BilinearForm + SymbolicBFI for the Laplace/mass slice
 * (comp/bilinearform.cpp:832, fem/symbolicintegrator.cpp:1548-1830).
 * kappa / mu: per-element coefficients (NULL: kappa = 1, mu = 0).        */
int gh1_form_create(gh1_space* space, const double* kappa, const double* mu, int mem, gh1_form** form);
int gh1_form_set_coefs(gh1_form* form, const double* kappa, const double* mu, int mem);
/* Anisotropic diffusion (K grad u).grad v with one symmetric tensor per element,
 * NGSolve's InnerProduct(K*grad(u), grad(v)) with a matrix-valued
 * CoefficientFunction: the D matrix of B^T D B (fem/symbolicintegrator.cpp:
 * 1548-1830) becomes w|det J| K in place of w|det J| kappa I.
 * K6: ne*6 doubles per element (xx yy zz xy xz yz), host or device per mem;
 * NULL returns the form to the scalar kappa.  While a tensor is set, kappa is
 * ignored (fold a scalar term in as kappa I), and gh1_adjoint_grad rejects the
 * form (dJ/dkappa needs the scalar coefficient).  Operators made from the form
 * afterwards, and matrix-free operators at their next apply, use the tensor. */
int gh1_form_set_tensor(gh1_form* form, const double* K6, int mem);
/* Generic B^T D B form (the reference's fused symbolic operator for arbitrary
 * bilinear integrands, comp/matrixfree.cpp:1090-1330 AssembleBDBFused, applied on
 * the device by ngscuda/cuda_matrix_free_btdtb.cpp:60-310):
 *   a(u, v) = sum_e int_e (B v)^T D (B u) dx,  B w = (w, dw/dx, dw/dy, dw/dz),
 * D in physical coordinates, row = test component, column = trial component
 * (row-major 4x4).  Diffusion K grad u . grad v is D[1+k][1+l] = K_kl, reaction
 * c u v is D[0][0] = c, convection (b . grad u) v is D[0][1+l] = b_l, and
 * u (b . grad v) is D[1+k][0] = b_k; D need not be symmetric.
 * per_point = 0: D[ne][16], one matrix per element (as the reference evaluates
 * it); per_point = 1: D[ne][nq][16] at the points of the space's rule
 * (gh1_space_qpoints: hex tensor Gauss with p+1 points per direction, tet the
 * degree-2p rule).  Host or device per mem; NULL returns the form to kappa / mu /
 * K6, which a set D replaces.  Such a form gives matrix-free operators
 * (gh1_matfree_create, FP64 and FP32, with their diagonal for Jacobi) and CSR
 * matrices (gh1_assemble_csr, not symmetric when D is not);
 * gh1_adjoint_grad and gh1_batch_create reject it. */
int gh1_form_set_bdb(gh1_form* form, const double* D, int per_point, int mem);
/* The rule the generic form integrates with: *nq points per element; ref (host,
 * may be NULL): nq x 4 reference coordinates and weight; xyz (may be NULL):
 * ne x nq x 3 physical coordinates, host or device per mem.  A point-wise D of
 * gh1_form_set_bdb follows this point order. */
int gh1_space_qpoints(gh1_space* space, double* ref, double* xyz, int mem, int* nq);
/* Curved elements: MeshAccess::SetDeformation (comp/meshaccess.cpp:1573-1580,
 * ALE_ElementTransformation :240-340).  d: 3 * ndof(space) values, the x, y and z
 * components of a displacement field in the H1 space `space` of this mesh one
 * after the other (VectorH1 numbering), host or device per mem.  Element maps
 * become x(xi) + d(xi), Jacobians J(xi) + grad d(xi), at every rule point.
 * Forms, operators, load vectors and rule points made while it is set use the
 * deformed elements (made before: the mesh as it was); on tets the operators
 * then take the per-point B^T D B path, and the element contraction of
 * gh1_adjoint_grad is not available.  d = NULL removes the deformation; freeing
 * `space` removes it too. */
int gh1_mesh_set_deformation(gh1_mesh* mesh, gh1_space* space, const double* d, int mem);
/* Releases the caller's handle.  Operators made from the form (gh1_assemble_csr,
 * gh1_matfree_create, gh1_batch_create) keep it alive, as the reference's
 * BilinearFormApplication holds its BilinearForm: its memory goes when the last
 * of them is freed.  The space must outlive the form and its operators.     */
int gh1_form_free(gh1_form* form);

/* BilinearForm.Assemble() -> SparseMatrix (comp/bilinearform.cpp:832-1000,
 * linalg/sparsematrix_impl.hpp:148-190): GPU element matrices scattered into
 * the MatrixGraph pattern (full storage, sorted columns).               */
int gh1_assemble_csr(gh1_form* form, gh1_op** csr);
/* info[0..1] = nrows, nnz */
int gh1_csr_info(gh1_op* csr, int64_t* info);
int gh1_csr_export(gh1_op* csr, int64_t* rowptr, int32_t* colind, double* vals, int mem);
/* Upload an externally built CSR matrix (e.g. NGSolve's own SparseMatrix) */
int gh1_csr_import(gh1_ctx* ctx, int64_t nrows, int64_t nnz, const int64_t* rowptr, const int32_t* colind,
                   const double* vals, int mem, gh1_op** csr);

/* BilinearForm(nonassemble=True).mat -> BilinearFormApplication
 * (comp/bilinearform.cpp:7549-7607): sum-factorized on hexes, element-wise
 * B^T D B on tets.  precision_mask: bit0 = FP64 data, bit1 = FP32 data.  */
int gh1_matfree_create(gh1_form* form, int precision_mask, gh1_op** op);

/* BaseMatrix::Mult / MultAdd (linalg/basematrix.hpp:117-126):
 * y = s*A*x (accumulate=0) or y += s*A*x (accumulate=1); device pointers. */
int gh1_op_apply(gh1_op* op, double s, const void* x, void* y, int precision, int accumulate);
/* info[0..5] = kind (GH1_OP_*), nrows, ne, order, and for a hex matrix-free
 * operator the autotuned apply variant in FP64 and FP32 (0 / 1: one element per
 * lane with the G tile staged by bulk copy / loaded directly; 2 / 3: the same
 * with two elements per lane, FP32 only; 4: two elements per lane with one metric
 * per element, FP32, chosen only when every element map is affine; 5: the slice /
 * pencil form of 4, orders 1-4; 6: the 1D contractions on the tensor cores
 * (tcgen05), FP32, orders 4-7; -1: not applicable).  A generic B^T D B operator
 * (gh1_form_set_bdb, hex or tet) reports 7 in both: metric records per rule
 * point, or 8: one record per element (affine elements, D per element); in FP32
 * a hex one reports 9 / 11 when the two-elements-per-lane kernel runs it (records
 * per element / per point), a tet one 10 when both tile products run on the
 * tensor cores (records per element, orders 2-4), each kept only when faster.
 * For a tet matrix-free operator info[5] is 6 when its FP32 apply runs both tile
 * products on the tensor cores (orders 2-4 without a mass term), 10 with a mass
 * term (the B^T D B tensor-core kernel), kept when faster, else -1.  For a CSR operator info[4..5]
 * are the autotuned SpMV configuration in FP64 and FP32: lanes per row L, plus
 * 100 when each lane keeps 8 instead of 4 nonzeros in flight (0: not tuned yet). */
int gh1_op_info(gh1_op* op, int64_t* info);
/* Waits for the context's stream and reports whether a matrix-free apply of op
 * since the last check met a device wait that ran out of its bound (GH1_ERR_CUDA:
 * the kernel drained its copies and returned, the context stays usable, the
 * result is invalid); GH1_OK otherwise.  gh1_op_apply is asynchronous and does
 * not wait; gh1_cg, gh1_batch_solve and gh1_adjoint_grad run this check before
 * they return.  The counterpart of the reference's synchronizing apply
 * (the `synckernels` device synchronize in ngscuda/cuda_linalg.cpp:370-412). */
int gh1_op_check(gh1_op* op);
int gh1_op_free(gh1_op* op);

/* Block-diagonal operator diag(A, ..., A) with nblocks copies of op on
 * consecutive slices of length nrows(op): the bilinear forms
 * InnerProduct(grad(u), grad(v)) and InnerProduct(u, v) on VectorH1, whose DOFs
 * are the component spaces' DOFs one after the other (CompoundFESpace,
 * comp/h1hofespace.cpp:2482-2560, VectorH1FESpace with interleaved = false).
 * The block operator works with gh1_op_apply, gh1_jacobi_create (freedofs of
 * length nblocks * nrows, or the inner space's repeated), gh1_cg and
 * gh1_op_info (kind GH1_OP_BLOCK).  op is borrowed: it must outlive the block
 * operator. */
int gh1_op_block_create(gh1_op* op, int nblocks, gh1_op** block);

/* ---- preconditioner -----------------------------------------------------
 * a.mat.CreateSmoother(freedofs) / Preconditioner(a,"local")
 * (linalg/jacobi.cpp:40-110): invdiag = 1/A_ii on free DOFs, 0 elsewhere.
 * freedofs: NULL = the space's free DOFs.                                */
int gh1_jacobi_create(gh1_op* op, const uint8_t* freedofs, int mem, gh1_pre** pre);
/* y = s*C*x (accumulate=0) or y += s*C*x for any preconditioner below. */
int gh1_pre_apply(gh1_pre* pre, double s, const void* x, void* y, int precision, int accumulate);
int gh1_pre_free(gh1_pre* pre);

/* Additive Schwarz: block Jacobi plus an exact low-order solve, the reference's
 * tutorial preconditioner jac + loemb @ loinv @ loemb.T
 * (docs/i-tutorials/unit-5.5-cuda/poisson_cuda.ipynb cells 9-13).
 * Smoothing blocks of H1HighOrderFESpace::CreateSmoothingBlocks
 * (comp/h1hofespace.cpp:1477-1600), only free DOFs, empty blocks dropped:
 * blocktype 4 = VE + F + I (each vertex with the DOFs of the edges at it, each
 * face, each element's interior), 3 = V + E + F + I.  First call with offsets /
 * dofs NULL for the sizes; then offsets[nblocks+1] and dofs[nentries] (host). */
int gh1_space_smoothing_blocks(gh1_space* space, int blocktype, int64_t* nblocks, int64_t* nentries, int64_t* offsets,
                               int32_t* dofs);
/* BlockJacobiPrecond (linalg/blockjacobi.cpp; device apply DevBlockJacobiMatrix,
 * ngscuda/dev_blockjacobi.cpp:49-137): the dense diagonal blocks of an assembled
 * SPD matrix (gh1_assemble_csr / gh1_csr_import), inverted on the GPU;
 * y = s sum_b E_b A_b^{-1} E_b^T x.  Blocks: offsets[nblocks+1] into dofs,
 * host or device per mem; up to 4096 DOFs a block. */
int gh1_blockjacobi_create(gh1_op* csr, int64_t nblocks, const int64_t* offsets, const int32_t* dofs, int mem,
                           gh1_pre** pre);
/* Exact low-order solve P A_c^{-1} P^T: csr is the low-order matrix (the p = 1
 * form, a.loform; in the hierarchical basis its DOFs are the first DOFs of the
 * high-order space, embed = NULL), embed[i] the fine DOF of coarse DOF i,
 * freedofs the coarse free DOFs (NULL: all); the matrix on the free coarse DOFs
 * is inverted on the GPU (the reference factorizes it with its sparse Cholesky,
 * ngscuda/dev_sparsecholesky.cpp); up to 8192 free coarse DOFs. */
int gh1_coarse_create(gh1_op* csr, int64_t nfine, const int32_t* embed, const uint8_t* freedofs, int mem,
                      gh1_pre** pre);
/* y = s (A + B) x (SumMatrix); a and b are borrowed and must outlive the sum.
 * gh1_cg takes any of these preconditioners; other than Jacobi they run as
 * their own kernels inside the device-side CG loop. */
int gh1_pre_sum(gh1_pre* a, gh1_pre* b, gh1_pre** sum);

/* ---- projector ----------------------------------------------------------------
 * Projector(mask, range) (linalg/diagonalmatrix.cpp:13-110; the reference's GPU
 * DevProjector, ngscuda/linalg_kernels.cu:304-376): keeps the entries whose mask
 * byte is nonzero (range = 1) or zero (range = 0) and zeroes the others.
 * mask: one byte per entry (the gh1_space_get_freedofs layout), host or device.
 * apply: y = s*P*x (accumulate = 0) or y += s*P*x; project: x = P*x in place.  */
typedef struct gh1_proj gh1_proj;
int gh1_projector_create(gh1_ctx* ctx, int64_t n, const uint8_t* mask, int range, int mem, gh1_proj** proj);
int gh1_projector_apply(gh1_proj* proj, double s, const void* x, void* y, int precision, int accumulate);
int gh1_projector_project(gh1_proj* proj, void* x, int precision);
int gh1_projector_free(gh1_proj* proj);

/* ---- right-hand side ------------------------------------------------------
 * LinearForm(f*v*dx) with f piecewise constant per element, integration
 * order 2p (fem/symbolicintegrator.cpp:1109).  b: device double[ndof].    */
int gh1_rhs_elementwise(gh1_space* space, const double* f_elem, int mem, double* b);

/* ---- CG --------------------------------------------------------------------
 * solvers.CG / CGSolver._SolveImpl (python/krylovspace.py:263-337).
 * mode GH1_CG_FP64: the reference algorithm on the GPU in FP64.
 * mode GH1_CG_MIXED: FP32 inner Jacobi-PCG inside FP64 iterative refinement
 *   (outer residual b - A x, dot products and updates in FP64).
 * stop_rule GH1_STOP_PRECOND: sqrt|w.d| <= tol * first (the reference rule);
 * GH1_STOP_TRUE: ||b - A x||_free <= tol * ||b||_free.                     */
enum { GH1_CG_FP64 = 0, GH1_CG_MIXED = 1 };
enum { GH1_STOP_PRECOND = 0, GH1_STOP_TRUE = 1 };
typedef struct {
  double tol;          /* relative tolerance                                   */
  int maxit;           /* maximal iterations (inner iterations for MIXED)      */
  int mode;            /* GH1_CG_FP64 / GH1_CG_MIXED                           */
  int stop_rule;       /* GH1_STOP_PRECOND / GH1_STOP_TRUE                     */
  int initialize;      /* 1: start from x = 0, 0: use x as initial guess       */
  double inner_tol;    /* MIXED: relative reduction per inner solve (0=default)*/
  int max_outer;       /* MIXED: maximal refinement steps (0 = default 30)      */
  int check_every;     /* iterations per body of the device-side WHILE loop (0=auto) */
  double* res_hist;    /* optional host buffer [maxit+1] of residuals (may be NULL) */
} gh1_cg_opts;
typedef struct {
  int status;          /* GH1_OK, GH1_MAXITER or GH1_BREAKDOWN                  */
  int iterations;      /* CheckResidual calls (FP64) / total inner iterations   */
  int outer;           /* MIXED: refinement steps taken                         */
  int applies64;       /* FP64 operator applications                            */
  int applies32;       /* FP32 operator applications                            */
  double first_res;    /* first residual of the stop rule                       */
  double final_res;    /* last residual of the stop rule                        */
  double true_relres;  /* ||b-Ax||_free/||b||_free at exit (FP64)               */
} gh1_cg_result;
/* b, x: device double[ndof].  pre may be NULL only for GH1_CG_FP64 (then no
 * preconditioning and no Dirichlet projection).                            */
int gh1_cg(gh1_op* op, gh1_pre* pre, const double* b, double* x, const gh1_cg_opts* opts, gh1_cg_result* res);

/* ---- adjoint ---------------------------------------------------------------
 * Element-wise integral of grad u . grad w (Integrate(..., element_wise=True),
 * comp/python_comp.cpp:3703-3948): out[e] = int_e grad u.grad w (device ptrs). */
int gh1_elem_grad_dot(gh1_space* space, const double* u, const double* w, double* out);
/* J(kappa) = 1/2 int (u - u_target)^2 with A(kappa) u = f (zero Dirichlet);
 * dJ/dkappa_e = -int_e grad u . grad lambda,  A lambda = M (u - u_target).
 * f, u_target: device double[ndof] (f already assembled); kappa: the form's.
 * Both solves run the mixed-precision CG (FP32 inner, FP64 refinement) to the
 * true relative residual tol.  The form keeps its operator between calls
 * (released by gh1_form_free); only the Jacobi diagonal is rebuilt per call.
 * Outputs (device): u[ndof], lambda[ndof], dJdkappa[ne]; J on the host.   */
int gh1_adjoint_grad(gh1_form* form, const double* f, const double* u_target, double tol,
                     double* u, double* lambda, double* dJdkappa, double* J);

/* ---- batched solves ----------------------------------------------------------
 * Many independent hex problems (forms), 1..16 right-hand sides each (config
 * "256 problems x 16 rhs"), solved by the mixed-precision method of gh1_cg:
 * every (problem, rhs) pair is a device-side state machine (FP64 residual ->
 * FP32 inner Jacobi-PCG -> FP64 correction) and all problems advance together
 * in ONE launch of one CUDA graph: a conditional WHILE node whose body is one
 * round of every problem (one branch per problem) repeats on the device until
 * all pairs converged.  The multi-rhs apply reads each element's G tile once
 * for all right-hand sides; gh1_batch_create times its two FP32 forms (one or
 * two right-hand sides per lane) on each problem and keeps the faster.  No
 * counterpart in the reference, which solves one system per CGSolver call
 * (python/krylovspace.py:263-291).
 * rhs[p], x[p]: device double[nrhs[p]*ndof_p], right-hand side r at offset
 * r*ndof_p.  opts: tol, maxit (per inner solve), inner_tol, max_outer,
 * check_every (inner iterations per round), initialize.
 * res: sum(nrhs) results, problem-major.                                      */
typedef struct gh1_batch gh1_batch;
int gh1_batch_create(gh1_ctx* ctx, int nprob, gh1_form* const* forms, const int* nrhs, gh1_batch** batch);
int gh1_batch_solve(gh1_batch* batch, const double* const* rhs, double* const* x, const gh1_cg_opts* opts,
                    gh1_cg_result* res);
int gh1_batch_free(gh1_batch* batch);

/* ---- shape evaluation without device allocation ------------------------------
 * No counterpart in the reference.  gh1_shape_eval allocates device buffers on
 * every call (copies of the points and outputs, and per-point scratch); some
 * callers cannot let a library allocate at that point: hosts that hand all
 * device memory out of their own fixed pool or budget, and loops that must not
 * stall on cudaMalloc/cudaFree (which can synchronise the device).  This
 * variant computes the same values with the same kernel, from DEVICE inputs
 * into DEVICE outputs, and takes its scratch from one fixed array compiled into
 * the library (GH1_SHAPE_NOALLOC_MAX_ENTRIES entries of 32 bytes = 8 MiB),
 * which every GPU that loads the library holds until the process exits.
 *  - npts * nloc must not exceed GH1_SHAPE_NOALLOC_MAX_ENTRIES
 *    (nloc = (p+1)(p+2)(p+3)/6 on tets, (p+1)^3 on hexes); larger requests are
 *    rejected with GH1_ERR_ARG before any device work.
 *  - vnums: host int32[et]; pts: device double[npts*3]; val: device
 *    double[npts*nloc]; grad: device double[npts*nloc*3] (device or managed
 *    memory of the context's device).
 *  - Asynchronous: the work is queued on the context's stream and the call
 *    returns without waiting for it.
 *  - The first call on each device looks up the scratch array's device address
 *    (cudaGetSymbolAddress) with that device current; make that first call
 *    before any stream capture.
 *  - All calls share the one scratch array, which keeps the last call's
 *    contents (nothing in it has to start at zero: every entry a thread reads
 *    it has written first in the same call).  Calls whose work overlaps on the
 *    GPU (two streams, or two contexts on one device) race on it.            */
#define GH1_SHAPE_NOALLOC_MAX_ENTRIES 262144
int gh1_shape_eval_noalloc(gh1_ctx* ctx, int et, int order, const int32_t* vnums, int npts,
                           const double* pts, double* val, double* grad);

#ifdef __cplusplus
}
#endif
#endif /* GH1_H */
