// api.cu -- C ABI entry points of libgh1 and the host-side space setup.
//
// Host work here is mesh bookkeeping that netgen/NGSolve also do on the CPU:
// edge/face enumeration (netgen MeshTopology; numbering rule: sorted by the
// sorted global vertex tuple), the DOF tables of H1HighOrderFESpace
// (comp/h1hofespace.cpp:823-950, GetDofNrs :1389-1420) and the Dirichlet
// DOF set (comp/fespace.cpp:440-516, :765-830).  All numerics run on the GPU.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <numeric>
#include <thread>
#include <cstdlib>
#include "common.cuh"
#include "basis.cuh"

using namespace gh1;

namespace {

template <class F>
int guard(gh1_ctx* ctx, F&& f) {
  try {
    f();
    return GH1_OK;
  } catch (const Error& e) {
    if (ctx) ctx->err = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    if (ctx) ctx->err = "host allocation failed";
    return GH1_ERR_NOMEM;
  } catch (const std::exception& e) {
    if (ctx) ctx->err = e.what();
    return GH1_ERR_ARG;
  }
}

// parallel for over [0,n) with std::thread (host setup only)
template <class F>
void host_parallel(int64_t n, F&& f) {
  int nt = (int)std::min<int64_t>(std::max(1u, std::thread::hardware_concurrency()), 64);
  if (n < 4096 || nt <= 1) { for (int64_t i = 0; i < n; i++) f(i); return; }
  std::vector<std::thread> th;
  int64_t chunk = (n + nt - 1) / nt;
  for (int t = 0; t < nt; t++) {
    int64_t a = t * chunk, b = std::min(n, a + chunk);
    if (a >= b) break;
    th.emplace_back([=, &f]() { for (int64_t i = a; i < b; i++) f(i); });
  }
  for (auto& t : th) t.join();
}

// sorted-unique numbering of keys; returns id per input key
template <class K>
std::vector<int32_t> number_keys(const std::vector<K>& keys, int& nunique) {
  std::vector<int64_t> idx(keys.size());
  std::iota(idx.begin(), idx.end(), 0);
  std::sort(idx.begin(), idx.end(), [&](int64_t a, int64_t b) { return keys[a] < keys[b]; });
  std::vector<int32_t> id(keys.size());
  int cur = -1;
  for (size_t k = 0; k < idx.size(); k++) {
    if (k == 0 || keys[idx[k]] != keys[idx[k - 1]]) cur++;
    id[idx[k]] = cur;
  }
  nunique = cur + 1;
  return id;
}

int tet_class_of(const int* vn) {
  // class = lexicographic index of the rank permutation (r0,r1,r2,r3)
  int r[4];
  for (int i = 0; i < 4; i++) { r[i] = 0; for (int j = 0; j < 4; j++) if (vn[j] < vn[i]) r[i]++; }
  int used[4] = {0, 0, 0, 0}, code = 0;
  const int fact[4] = {6, 2, 1, 1};
  for (int i = 0; i < 4; i++) {
    int smaller = 0;
    for (int v = 0; v < r[i]; v++) if (!used[v]) smaller++;
    code += smaller * fact[i];
    used[r[i]] = 1;
  }
  return code;
}

void build_space(gh1_space* sp) {
  gh1_mesh* m = sp->mesh;
  const bool tet = m->et == 4;
  sp->et = m->et;
  sp->nvert = tet ? 4 : 8;
  sp->nedge = tet ? 6 : 12;
  sp->nface = tet ? 4 : 6;
  const int p = sp->p, ne = m->ne, nv = m->nv;
  const int fv = tet ? 3 : 4;
  auto ev = [&](int e, int i) { return m->el[(size_t)e * sp->nvert + i]; };
  auto ledge = [&](int i, int j) { return tet ? TetTopo::edge(i, j) : HexTopo::edge(i, j); };
  auto lface = [&](int i, int j) { return tet ? TetTopo::face(i, j) : HexTopo::face(i, j); };

  std::vector<uint64_t> ekeys((size_t)ne * sp->nedge);
  host_parallel(ne, [&](int64_t e) {
    for (int i = 0; i < sp->nedge; i++) {
      uint32_t a = ev(e, ledge(i, 0)), b = ev(e, ledge(i, 1));
      if (a > b) std::swap(a, b);
      ekeys[e * sp->nedge + i] = ((uint64_t)a << 32) | b;
    }
  });
  std::vector<int32_t> el_edges = number_keys(ekeys, sp->ned);
  std::vector<std::array<int32_t, 4>> fkeys((size_t)ne * sp->nface);
  host_parallel(ne, [&](int64_t e) {
    for (int i = 0; i < sp->nface; i++) {
      std::array<int32_t, 4> t{INT32_MAX, INT32_MAX, INT32_MAX, INT32_MAX};
      for (int j = 0; j < fv; j++) t[j] = ev(e, lface(i, j));
      for (int j = 1; j < fv; j++)  // insertion sort of the face's 3 or 4 vertex numbers
        for (int k = j; k > 0 && t[k - 1] > t[k]; k--) std::swap(t[k - 1], t[k]);
      fkeys[e * sp->nface + i] = t;
    }
  });
  std::vector<int32_t> el_faces = number_keys(fkeys, sp->nfa);

  sp->n_edge_dofs = p > 1 ? p - 1 : 0;
  sp->n_face_dofs = tet ? (p > 2 ? (p - 1) * (p - 2) / 2 : 0) : (p > 1 ? (p - 1) * (p - 1) : 0);
  sp->n_cell_dofs = tet ? (p > 3 ? (p - 1) * (p - 2) * (p - 3) / 6 : 0) : (p > 1 ? (p - 1) * (p - 1) * (p - 1) : 0);
  sp->first_edge = nv;
  sp->first_face = sp->first_edge + (int64_t)sp->ned * sp->n_edge_dofs;
  sp->first_cell = sp->first_face + (int64_t)sp->nfa * sp->n_face_dofs;
  sp->ndof = sp->first_cell + (int64_t)ne * sp->n_cell_dofs;
  GH1_CHECK(sp->ndof < INT32_MAX, GH1_ERR_UNSUPPORTED, "more than 2^31-1 DOFs");
  sp->nloc = tet ? (p + 1) * (p + 2) * (p + 3) / 6 : (p + 1) * (p + 1) * (p + 1);
  sp->n1 = p + 1;
  const int nloc = sp->nloc;

  // element DOFs in NGSolve's local order
  sp->el_dofs.assign((size_t)ne * nloc, 0);
  host_parallel(ne, [&](int64_t e) {
    int32_t* d = &sp->el_dofs[(size_t)e * nloc];
    int ii = 0;
    for (int i = 0; i < sp->nvert; i++) d[ii++] = ev(e, i);
    for (int i = 0; i < sp->nedge; i++)
      for (int k = 0; k < sp->n_edge_dofs; k++) d[ii++] = (int32_t)(sp->first_edge + (int64_t)el_edges[e * sp->nedge + i] * sp->n_edge_dofs + k);
    for (int i = 0; i < sp->nface; i++)
      for (int k = 0; k < sp->n_face_dofs; k++) d[ii++] = (int32_t)(sp->first_face + (int64_t)el_faces[e * sp->nface + i] * sp->n_face_dofs + k);
    for (int k = 0; k < sp->n_cell_dofs; k++) d[ii++] = (int32_t)(sp->first_cell + e * sp->n_cell_dofs + k);
  });

  // Dirichlet faces: every boundary face (one adjacent element), or the
  // caller's selection of boundary faces -> their closure's DOFs are not free
  std::vector<int32_t> fcount(sp->nfa, 0);
  for (size_t k = 0; k < el_faces.size(); k++) fcount[el_faces[k]]++;
  std::vector<uint8_t> fdir(sp->nfa, 0);
  if (sp->dir_select) {
    std::vector<std::array<int32_t, 4>> sel = sp->dir_faces;
    std::sort(sel.begin(), sel.end());
    sel.erase(std::unique(sel.begin(), sel.end()), sel.end());
    std::vector<uint8_t> found(sel.size(), 0);
    for (size_t k = 0; k < fkeys.size(); k++) {
      auto it = std::lower_bound(sel.begin(), sel.end(), fkeys[k]);
      if (it == sel.end() || *it != fkeys[k]) continue;
      GH1_CHECK(fcount[el_faces[k]] == 1, GH1_ERR_ARG, "a Dirichlet face is an interior face");
      fdir[el_faces[k]] = 1;
      found[it - sel.begin()] = 1;
    }
    for (auto v : found) GH1_CHECK(v, GH1_ERR_ARG, "a Dirichlet face is not a face of the mesh");
  } else {
    for (int f = 0; f < sp->nfa; f++) fdir[f] = fcount[f] == 1;
  }
  sp->freedof.assign(sp->ndof, 1);
  if (sp->mesh && sp->freedof.size()) {
    for (int e = 0; e < ne; e++)
      for (int i = 0; i < sp->nface; i++) {
        int f = el_faces[(size_t)e * sp->nface + i];
        if (!fdir[f]) continue;
        for (int k = 0; k < sp->n_face_dofs; k++) sp->freedof[sp->first_face + (int64_t)f * sp->n_face_dofs + k] = 0;
        for (int j = 0; j < fv; j++) sp->freedof[ev(e, lface(i, j))] = 0;
        for (int j = 0; j < fv; j++) {
          int a = ev(e, lface(i, j)), b = ev(e, lface(i, (j + 1) % fv));
          for (int ie = 0; ie < sp->nedge; ie++) {
            int ea = ev(e, ledge(ie, 0)), eb = ev(e, ledge(ie, 1));
            if ((ea == a && eb == b) || (ea == b && eb == a)) {
              int ge = el_edges[(size_t)e * sp->nedge + ie];
              for (int k = 0; k < sp->n_edge_dofs; k++) sp->freedof[sp->first_edge + (int64_t)ge * sp->n_edge_dofs + k] = 0;
            }
          }
        }
      }
  }

  cudaStream_t s = sp->ctx->stream;
  sp->d_eldofs.upload(sp->el_dofs, s);

  if (!tet) {
    // tensor-ordered signed DOF table: every hex shape is sign * psi_a psi_b psi_c
    const int n = p + 1, n3 = n * n * n;
    sp->tstride = (n3 + 3) / 4 * 4;
    const int ts = sp->tstride;
    std::vector<int32_t> tdof((size_t)ne * ts, 0);
    for (int64_t e = 0; e < ne; e++)
      for (int t = 0; t < n3; t++) tdof[(size_t)e * ts + t] = -1;
    host_parallel(ne, [&](int64_t e) {
      int32_t* T = &tdof[(size_t)e * ts];
      int vn[8];
      for (int i = 0; i < 8; i++) vn[i] = ev(e, i);
      auto put = [&](int a, int b, int c, int64_t dof, int sign) {
        T[(a * n + b) * n + c] = (int32_t)dof | (sign < 0 ? (int32_t)0x80000000u : 0);
      };
      for (int v = 0; v < 8; v++) put(HexTopo::coord(v, 0), HexTopo::coord(v, 1), HexTopo::coord(v, 2), vn[v], 1);
      for (int i = 0; i < 12 && p >= 2; i++) {
        int e0 = HexTopo::edge(i, 0), e1 = HexTopo::edge(i, 1);
        if (vn[e0] > vn[e1]) std::swap(e0, e1);
        int d = 0;
        while (HexTopo::coord(e0, d) == HexTopo::coord(e1, d)) d++;
        int flip = HexTopo::coord(e0, d) == 1;  // xi = 1-2t  ->  P_k(xi) = (-1)^k P_k(2t-1)
        int64_t base = sp->first_edge + (int64_t)el_edges[e * 12 + i] * sp->n_edge_dofs;
        for (int k = 0; k < p - 1; k++) {
          int idx[3] = {HexTopo::coord(e0, 0), HexTopo::coord(e0, 1), HexTopo::coord(e0, 2)};
          idx[d] = k + 2;
          put(idx[0], idx[1], idx[2], base + k, (flip && (k & 1)) ? -1 : 1);
        }
      }
      for (int i = 0; i < 6 && p >= 2; i++) {
        int f[4] = {HexTopo::face(i, 0), HexTopo::face(i, 1), HexTopo::face(i, 2), HexTopo::face(i, 3)};
        int fmin = 0;
        for (int j = 1; j < 4; j++) if (vn[f[j]] < vn[f[fmin]]) fmin = j;
        int j1 = (fmin + 3) % 4, j2 = (fmin + 1) % 4;
        if (vn[f[j2]] < vn[f[j1]]) std::swap(j1, j2);
        int g0 = f[fmin], g1 = f[j1], g3 = f[j2];
        int d1 = 0, d2 = 0;
        while (HexTopo::coord(g0, d1) == HexTopo::coord(g1, d1)) d1++;
        while (HexTopo::coord(g0, d2) == HexTopo::coord(g3, d2)) d2++;
        int s1 = HexTopo::coord(g0, d1) == 0 ? -1 : 1;  // xi = sigma[g0]-sigma[g1]
        int s2 = HexTopo::coord(g0, d2) == 0 ? -1 : 1;
        int64_t base = sp->first_face + (int64_t)el_faces[e * 6 + i] * sp->n_face_dofs;
        for (int k = 0; k < p - 1; k++)
          for (int j = 0; j < p - 1; j++) {
            int idx[3] = {HexTopo::coord(g0, 0), HexTopo::coord(g0, 1), HexTopo::coord(g0, 2)};
            idx[d1] = k + 2;
            idx[d2] = j + 2;
            int sg = ((s1 < 0 && (k & 1)) ? -1 : 1) * ((s2 < 0 && (j & 1)) ? -1 : 1);
            put(idx[0], idx[1], idx[2], base + k * (p - 1) + j, sg);
          }
      }
      if (p >= 2) {
        int64_t base = sp->first_cell + (int64_t)e * sp->n_cell_dofs;
        for (int i = 0; i < p - 1; i++)
          for (int j = 0; j < p - 1; j++)
            for (int k = 0; k < p - 1; k++) put(i + 2, j + 2, k + 2, base + (i * (p - 1) + j) * (p - 1) + k, 1);
      }
    });
    for (size_t k = 0; k < tdof.size(); k++) GH1_CHECK(tdof[k] != -1, GH1_ERR_ARG, "hex tensor map incomplete");
    sp->d_tdof.upload(tdof, s);
  } else {
    std::vector<uint8_t> cls(ne);
    host_parallel(ne, [&](int64_t e) {
      int vn[4] = {ev(e, 0), ev(e, 1), ev(e, 2), ev(e, 3)};
      cls[e] = (uint8_t)tet_class_of(vn);
    });
    sp->d_class.upload(cls, s);
  }
  int64_t nfree = 0;
  for (auto v : sp->freedof) nfree += v;
  sp->nfree = nfree;
  sp->d_free.upload(sp->freedof, s);
  build_tables(sp);
  GH1_CUDA(cudaStreamSynchronize(s));
}

}  // namespace

namespace gh1 {
int grid_for(gh1_ctx* ctx, int64_t work, int block, int per_sm) {
  int64_t need = (work + block - 1) / block;
  int64_t cap = (int64_t)ctx->nsm * per_sm;
  return (int)std::max<int64_t>(1, std::min(need, cap));
}
void check_kernel(gh1_ctx* ctx, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) throw Error(GH1_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
}  // namespace gh1

gh1_form::~gh1_form() {
  delete adj_M;  // before the mass form it refers to
  delete adj_A;
  delete adj_mass;
}

namespace gh1 {
void form_retain(gh1_form* f) { f->refs++; }
void form_release(gh1_form* f) {
  if (--f->refs == 0) delete f;
}
}  // namespace gh1

gh1_op::~gh1_op() {
  if (form_ref && form) gh1::form_release(form);
}

// =============================================================================
namespace gh1 {

// y = A x for every operator kind.  CSR writes y; the matrix-free apply adds into
// a y that is zero on entry; a block operator applies its inner operator slice by
// slice.  skip: as for the CG graph kernels (NULL outside graphs).
void op_apply_any(gh1_op* op, const void* x, void* y, int prec, const int* skip) {
  if (op->kind == GH1_OP_CSR) {
    spmv_skip(op, x, y, prec, skip);
  } else if (op->kind == GH1_OP_MATFREE) {
    matfree_apply_ex(op, x, y, prec, nullptr, nullptr, nullptr, skip);
  } else {
    const size_t bytes = (size_t)op->inner->nrows * (prec == GH1_F64 ? 8 : 4);
    for (int b = 0; b < op->nblocks; b++)
      op_apply_any(op->inner, (const char*)x + b * bytes, (char*)y + b * bytes, prec, skip);
  }
}

// per-operator setup that must not run inside a stream capture (SpMV autotuning)
void op_prepare_any(gh1_op* op, int prec) {
  if (op->kind == GH1_OP_CSR) spmv_prepare(op, prec);
  else if (op->kind == GH1_OP_BLOCK) op_prepare_any(op->inner, prec);
}

// matrix-free data of a form whose coefficients changed since the setup
void op_refresh_any(gh1_op* op) {
  if (op->kind == GH1_OP_MATFREE && op->form && op->form_version != op->form->version) matfree_setup(op);
  else if (op->kind == GH1_OP_BLOCK) op_refresh_any(op->inner);
}

// A bounded device wait of a matrix-free apply that ran out sets the operator's
// error flag (the kernel drained its copies and returned, so the context is
// usable and the result is not).  Report it, once, after the stream is synchronized.
void op_check_err(gh1_op* op) {
  if (op->kind == GH1_OP_BLOCK) {
    op_check_err(op->inner);
    return;
  }
  if (op->kind != GH1_OP_MATFREE || op->d_err.n == 0) return;
  int h = 0;
  GH1_CUDA(cudaMemcpy(&h, op->d_err.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (h != 0) {
    GH1_CUDA(cudaMemset(op->d_err.p, 0, sizeof(int)));
    throw Error(GH1_ERR_CUDA, "a bounded wait in the matrix-free apply timed out; its results are invalid");
  }
}

// operator diagonal (FP64, device)
static void op_diag_any(gh1_op* op, double* diag) {
  if (op->kind == GH1_OP_CSR) {
    csr_diag(op, diag);
  } else if (op->kind == GH1_OP_MATFREE) {
    matfree_diag(op, diag);
  } else {
    const int64_t n = op->inner->nrows;
    op_diag_any(op->inner, diag);
    for (int b = 1; b < op->nblocks; b++)
      GH1_CUDA(cudaMemcpyAsync(diag + b * n, diag, n * sizeof(double), cudaMemcpyDeviceToDevice, op->ctx->stream));
  }
}

}  // namespace gh1

extern "C" {

int gh1_version(void) { return 1; }

int gh1_create(gh1_ctx** out, int device) {
  if (!out) return GH1_ERR_ARG;
  gh1_ctx* c = new gh1_ctx();
  int rc = guard(c, [&] {
    int n = 0;
    GH1_CUDA(cudaGetDeviceCount(&n));
    GH1_CHECK(device >= 0 && device < n, GH1_ERR_ARG, "no such CUDA device");
    GH1_CUDA(cudaSetDevice(device));
    c->device = device;
    cudaDeviceProp prop;
    GH1_CUDA(cudaGetDeviceProperties(&prop, device));
    c->nsm = prop.multiProcessorCount;
    c->cc_major = prop.major;
    c->cc_minor = prop.minor;
    c->red.alloc(1 << 16);
    c->cnt.alloc(64);
    c->cnt.zero(nullptr);
    GH1_CUDA(cudaMallocHost((void**)&c->h_pinned, 4096));
    GH1_CUDA(cudaDeviceSynchronize());
  });
  if (rc != GH1_OK) {
    // keep the message reachable: return the context with the error set
    *out = c;
    return rc;
  }
  *out = c;
  return GH1_OK;
}

int gh1_destroy(gh1_ctx* ctx) {
  if (!ctx) return GH1_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
  delete ctx;
  return GH1_OK;
}

int gh1_set_stream(gh1_ctx* ctx, void* stream) {
  if (!ctx) return GH1_ERR_ARG;
  ctx->stream = (cudaStream_t)stream;
  return GH1_OK;
}

const char* gh1_last_error(gh1_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int gh1_mesh_upload(gh1_ctx* ctx, int nv, const double* coords, int ne, int et, const int32_t* ev, gh1_mesh** out) {
  if (!ctx || !out) return GH1_ERR_ARG;
  return guard(ctx, [&] {
    GH1_CHECK(et == 4 || et == 8, GH1_ERR_UNSUPPORTED, "element type must be 4 (tet) or 8 (hex)");
    GH1_CHECK(nv > 0 && ne > 0 && coords && ev, GH1_ERR_ARG, "empty mesh");
    for (int64_t k = 0; k < (int64_t)ne * et; k++)
      GH1_CHECK(ev[k] >= 0 && ev[k] < nv, GH1_ERR_ARG, "element vertex index out of range");
    GH1_CUDA(cudaSetDevice(ctx->device));
    gh1_mesh* m = new gh1_mesh();
    m->ctx = ctx; m->nv = nv; m->ne = ne; m->et = et;
    m->X.assign(coords, coords + 3 * (size_t)nv);
    m->el.assign(ev, ev + (size_t)ne * et);
    m->d_X.upload(m->X, ctx->stream);
    m->d_el.upload(m->el, ctx->stream);
    GH1_CUDA(cudaStreamSynchronize(ctx->stream));
    *out = m;
  });
}

int gh1_mesh_free(gh1_mesh* m) {
  if (m && m->def_space) m->def_space->def_of = nullptr;  // the two may be freed in either order
  delete m;
  return GH1_OK;
}

static void upload_coef(gh1_ctx* ctx, DBuf<double>& dst, const double* src, int mem, int64_t n, double dflt);
int gh1_mesh_set_deformation(gh1_mesh* m, gh1_space* sp, const double* d, int mem) {
  if (!m) return GH1_ERR_ARG;
  return guard(m->ctx, [&] {
    GH1_CHECK(mem == GH1_MEM_HOST || mem == GH1_MEM_DEVICE, GH1_ERR_ARG, "mem must be GH1_MEM_HOST or GH1_MEM_DEVICE");
    if (m->def_space) m->def_space->def_of = nullptr;
    m->def_space = nullptr;
    m->d_def.release();
    if (!d) return;
    GH1_CHECK(sp && sp->mesh == m, GH1_ERR_ARG, "the deformation lives in an H1 space of this mesh");
    GH1_CHECK(m->et == 8 || sp->p <= MAX_TET_ORDER, GH1_ERR_UNSUPPORTED, "deformation order out of range");
    upload_coef(m->ctx, m->d_def, d, mem, 3 * sp->ndof, 0.0);
    m->def_space = sp;
    sp->def_of = m;
    GH1_CUDA(cudaStreamSynchronize(m->ctx->stream));
  });
}

int gh1_space_h1(gh1_mesh* m, int order, int dirichlet, gh1_space** out) {
  if (!m || !out) return GH1_ERR_ARG;
  return guard(m->ctx, [&] {
    int maxp = m->et == 4 ? MAX_TET_ORDER : MAX_HEX_ORDER;
    GH1_CHECK(order >= 1 && order <= maxp, GH1_ERR_UNSUPPORTED, "order out of the supported range");
    GH1_CUDA(cudaSetDevice(m->ctx->device));
    gh1_space* sp = new gh1_space();
    sp->ctx = m->ctx; sp->mesh = m; sp->p = order;
    try {
      build_space(sp);
      if (!dirichlet) {
        std::fill(sp->freedof.begin(), sp->freedof.end(), 1);
        sp->nfree = sp->ndof;
        sp->d_free.upload(sp->freedof, sp->ctx->stream);
        GH1_CUDA(cudaStreamSynchronize(sp->ctx->stream));
      }
    } catch (...) { delete sp; throw; }
    *out = sp;
  });
}

int gh1_space_h1_bnd(gh1_mesh* m, int order, int64_t nbf, const int32_t* faces, gh1_space** out) {
  if (!m || !out || nbf < 0 || (nbf > 0 && !faces)) return GH1_ERR_ARG;
  return guard(m->ctx, [&] {
    int maxp = m->et == 4 ? MAX_TET_ORDER : MAX_HEX_ORDER;
    GH1_CHECK(order >= 1 && order <= maxp, GH1_ERR_UNSUPPORTED, "order out of the supported range");
    GH1_CUDA(cudaSetDevice(m->ctx->device));
    gh1_space* sp = new gh1_space();
    sp->ctx = m->ctx; sp->mesh = m; sp->p = order;
    try {
      const int fv = m->et == 4 ? 3 : 4;
      sp->dir_select = true;
      sp->dir_faces.resize(nbf);
      for (int64_t k = 0; k < nbf; k++) {
        std::array<int32_t, 4> t{INT32_MAX, INT32_MAX, INT32_MAX, INT32_MAX};
        for (int j = 0; j < fv; j++) {
          t[j] = faces[k * fv + j];
          GH1_CHECK(t[j] >= 0 && t[j] < m->nv, GH1_ERR_ARG, "Dirichlet face vertex out of range");
        }
        std::sort(t.begin(), t.begin() + fv);
        sp->dir_faces[k] = t;
      }
      build_space(sp);
      sp->dir_faces = {};
    } catch (...) { delete sp; throw; }
    *out = sp;
  });
}

int gh1_space_free(gh1_space* sp) {
  if (sp && sp->def_of) {  // the mesh's deformation lived in this space
    sp->def_of->def_space = nullptr;
    sp->def_of->d_def.release();
  }
  delete sp;
  return GH1_OK;
}

int gh1_space_info(gh1_space* sp, int64_t* info) {
  if (!sp || !info) return GH1_ERR_ARG;
  info[0] = sp->ndof; info[1] = sp->nloc; info[2] = sp->ned; info[3] = sp->nfa; info[4] = sp->nfree; info[5] = sp->mesh->ne;
  return GH1_OK;
}

int gh1_space_get_dofs(gh1_space* sp, int32_t* out) {
  if (!sp || !out) return GH1_ERR_ARG;
  std::memcpy(out, sp->el_dofs.data(), sp->el_dofs.size() * sizeof(int32_t));
  return GH1_OK;
}

int gh1_space_get_freedofs(gh1_space* sp, uint8_t* out) {
  if (!sp || !out) return GH1_ERR_ARG;
  std::memcpy(out, sp->freedof.data(), sp->freedof.size());
  return GH1_OK;
}

static void upload_coef(gh1_ctx* ctx, DBuf<double>& dst, const double* src, int mem, int64_t n, double dflt) {
  dst.alloc(n);
  if (!src) {
    std::vector<double> h(n, dflt);
    dst.upload(h, ctx->stream);
  } else if (mem == GH1_MEM_DEVICE) {
    GH1_CUDA(cudaMemcpyAsync(dst.p, src, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  } else {
    dst.upload(src, n, ctx->stream);
  }
}

int gh1_form_create(gh1_space* sp, const double* kappa, const double* mu, int mem, gh1_form** out) {
  if (!sp || !out) return GH1_ERR_ARG;
  return guard(sp->ctx, [&] {
    GH1_CUDA(cudaSetDevice(sp->ctx->device));
    gh1_form* f = new gh1_form();
    f->sp = sp;
    upload_coef(sp->ctx, f->d_kappa, kappa, mem, sp->mesh->ne, 1.0);
    f->has_mu = mu != nullptr;
    if (mu) upload_coef(sp->ctx, f->d_mu, mu, mem, sp->mesh->ne, 0.0);
    GH1_CUDA(cudaStreamSynchronize(sp->ctx->stream));
    *out = f;
  });
}

int gh1_form_set_coefs(gh1_form* f, const double* kappa, const double* mu, int mem) {
  if (!f) return GH1_ERR_ARG;
  return guard(f->sp->ctx, [&] {
    upload_coef(f->sp->ctx, f->d_kappa, kappa, mem, f->sp->mesh->ne, 1.0);
    f->has_mu = mu != nullptr;
    if (mu) upload_coef(f->sp->ctx, f->d_mu, mu, mem, f->sp->mesh->ne, 0.0);
    else f->d_mu.release();
    f->version++;
    GH1_CUDA(cudaStreamSynchronize(f->sp->ctx->stream));
  });
}

int gh1_form_set_tensor(gh1_form* f, const double* K6, int mem) {
  if (!f) return GH1_ERR_ARG;
  return guard(f->sp->ctx, [&] {
    GH1_CHECK(mem == GH1_MEM_HOST || mem == GH1_MEM_DEVICE, GH1_ERR_ARG, "mem must be GH1_MEM_HOST or GH1_MEM_DEVICE");
    if (K6) {
      upload_coef(f->sp->ctx, f->d_K6, K6, mem, (size_t)6 * f->sp->mesh->ne, 0.0);
      f->has_K6 = true;
    } else {
      f->d_K6.release();
      f->has_K6 = false;
    }
    f->version++;
    GH1_CUDA(cudaStreamSynchronize(f->sp->ctx->stream));
  });
}

// The caller's reference; operators made from the form keep it alive until the
// last of them is freed (the operators read its coefficients when they refresh).
int gh1_form_free(gh1_form* f) {
  if (f) gh1::form_release(f);
  return GH1_OK;
}

int gh1_form_set_bdb(gh1_form* f, const double* D, int per_point, int mem) {
  if (!f) return GH1_ERR_ARG;
  return guard(f->sp->ctx, [&] {
    GH1_CHECK(mem == GH1_MEM_HOST || mem == GH1_MEM_DEVICE, GH1_ERR_ARG, "mem must be GH1_MEM_HOST or GH1_MEM_DEVICE");
    GH1_CHECK(per_point == 0 || per_point == 1, GH1_ERR_ARG, "per_point is 0 (D per element) or 1 (D per rule point)");
    if (D) {
      const int64_t n = (int64_t)f->sp->mesh->ne * (per_point ? space_rule_size(f->sp) : 1) * 16;
      upload_coef(f->sp->ctx, f->d_bdb, D, mem, n, 0.0);
      f->bdb_mode = per_point ? 2 : 1;
    } else {
      f->d_bdb.release();
      f->bdb_mode = 0;
    }
    f->version++;
    GH1_CUDA(cudaStreamSynchronize(f->sp->ctx->stream));
  });
}
int gh1_space_qpoints(gh1_space* sp, double* ref, double* xyz, int mem, int* nq) {
  if (!sp) return GH1_ERR_ARG;
  return guard(sp->ctx, [&] {
    GH1_CHECK(mem == GH1_MEM_HOST || mem == GH1_MEM_DEVICE, GH1_ERR_ARG, "mem must be GH1_MEM_HOST or GH1_MEM_DEVICE");
    GH1_CUDA(cudaSetDevice(sp->ctx->device));
    const int n = space_rule_size(sp);
    if (nq) *nq = n;
    if (ref) space_qpoints(sp, ref, nullptr);
    if (xyz) {
      if (mem == GH1_MEM_DEVICE) {
        space_qpoints(sp, nullptr, xyz);
      } else {
        DBuf<double> d((size_t)sp->mesh->ne * n * 3);
        space_qpoints(sp, nullptr, d.p);
        GH1_CUDA(cudaMemcpyAsync(xyz, d.p, d.bytes(), cudaMemcpyDeviceToHost, sp->ctx->stream));
      }
    }
    GH1_CUDA(cudaStreamSynchronize(sp->ctx->stream));
  });
}
int gh1_assemble_csr(gh1_form* f, gh1_op** out) {
  if (!f || !out) return GH1_ERR_ARG;
  return guard(f->sp->ctx, [&] {
    gh1_space* sp = f->sp;
    GH1_CUDA(cudaSetDevice(sp->ctx->device));
    if (!sp->have_graph) {
      // GPU pattern build; the host one for very high orders or GH1_GRAPH=host
      const char* g = getenv("GH1_GRAPH");
      const bool host = g && std::string(g) == "host";
      if (host || !build_graph_gpu(sp)) build_graph(sp);
    }
    gh1_op* op = new gh1_op();
    op->ctx = sp->ctx; op->kind = GH1_OP_CSR; op->form = f; op->sp = sp;
    form_retain(f);
    op->form_ref = true;
    op->nrows = sp->ndof; op->nnz = sp->nnz;
    op->rowptr = sp->d_rowptr.p; op->colind = sp->d_colind.p;
    try {
      op->d_vals.alloc(sp->nnz);
      assemble_csr(f, op->d_vals.p);
    } catch (...) { delete op; throw; }
    *out = op;
  });
}

int gh1_csr_info(gh1_op* op, int64_t* info) {
  if (!op || !info || op->kind != GH1_OP_CSR) return GH1_ERR_ARG;
  info[0] = op->nrows; info[1] = op->nnz;
  return GH1_OK;
}

int gh1_csr_export(gh1_op* op, int64_t* rowptr, int32_t* colind, double* vals, int mem) {
  if (!op || op->kind != GH1_OP_CSR) return GH1_ERR_ARG;
  return guard(op->ctx, [&] {
    cudaMemcpyKind k = mem == GH1_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    cudaStream_t s = op->ctx->stream;
    if (rowptr) GH1_CUDA(cudaMemcpyAsync(rowptr, op->rowptr, (op->nrows + 1) * sizeof(int64_t), k, s));
    if (colind) GH1_CUDA(cudaMemcpyAsync(colind, op->colind, op->nnz * sizeof(int32_t), k, s));
    if (vals) GH1_CUDA(cudaMemcpyAsync(vals, op->d_vals.p, op->nnz * sizeof(double), k, s));
    GH1_CUDA(cudaStreamSynchronize(s));
  });
}

int gh1_csr_import(gh1_ctx* ctx, int64_t nrows, int64_t nnz, const int64_t* rowptr, const int32_t* colind,
                   const double* vals, int mem, gh1_op** out) {
  if (!ctx || !out || !rowptr || !colind || !vals || nrows <= 0) return GH1_ERR_ARG;
  return guard(ctx, [&] {
    GH1_CUDA(cudaSetDevice(ctx->device));
    gh1_op* op = new gh1_op();
    op->ctx = ctx; op->kind = GH1_OP_CSR; op->nrows = nrows; op->nnz = nnz;
    cudaMemcpyKind k = mem == GH1_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    try {
      op->d_rowptr_own.alloc(nrows + 1);
      op->d_colind_own.alloc(nnz);
      op->d_vals.alloc(nnz);
      GH1_CUDA(cudaMemcpyAsync(op->d_rowptr_own.p, rowptr, (nrows + 1) * sizeof(int64_t), k, ctx->stream));
      GH1_CUDA(cudaMemcpyAsync(op->d_colind_own.p, colind, nnz * sizeof(int32_t), k, ctx->stream));
      GH1_CUDA(cudaMemcpyAsync(op->d_vals.p, vals, nnz * sizeof(double), k, ctx->stream));
      GH1_CUDA(cudaStreamSynchronize(ctx->stream));
    } catch (...) { delete op; throw; }
    op->rowptr = op->d_rowptr_own.p;
    op->colind = op->d_colind_own.p;
    *out = op;
  });
}

int gh1_matfree_create(gh1_form* f, int prec_mask, gh1_op** out) {
  if (!f || !out) return GH1_ERR_ARG;
  return guard(f->sp->ctx, [&] {
    GH1_CHECK((prec_mask & 3) != 0, GH1_ERR_ARG, "precision mask must include FP64 (1) and/or FP32 (2)");
    GH1_CUDA(cudaSetDevice(f->sp->ctx->device));
    gh1_op* op = new gh1_op();
    op->ctx = f->sp->ctx; op->kind = GH1_OP_MATFREE; op->form = f; op->sp = f->sp;
    op->nrows = f->sp->ndof; op->prec_mask = prec_mask & 3;
    form_retain(f);
    op->form_ref = true;
    try {
      matfree_setup(op);
    } catch (...) { delete op; throw; }
    *out = op;
  });
}

int gh1_op_info(gh1_op* op, int64_t* info) {
  if (!op || !info) return GH1_ERR_ARG;
  if (op->kind == GH1_OP_BLOCK) {  // the inner operator's description, with the block kind and size
    const int rc = gh1_op_info(op->inner, info);
    info[0] = GH1_OP_BLOCK;
    info[1] = op->nrows;
    return rc;
  }
  info[0] = op->kind; info[1] = op->nrows;
  info[2] = op->sp ? op->sp->mesh->ne : 0;
  info[3] = op->sp ? op->sp->p : 0;
  const bool hexmf = op->kind == GH1_OP_MATFREE && op->sp && op->sp->et == 8;
  info[4] = hexmf ? op->hex_gmode[0] : -1;
  info[5] = hexmf && (op->prec_mask & 2) ? op->hex_gmode[1] : -1;
  if (op->kind == GH1_OP_MATFREE && op->sp && op->sp->et == 4 && op->tet_use_tc) info[5] = 6;
  if (op->kind == GH1_OP_MATFREE && op->sp && op->sp->et == 4 && !op->bdb && op->tet_bdb_tc) info[5] = 10;
  if (op->kind == GH1_OP_MATFREE && op->bdb) {  // generic B^T D B: records per point (7) or per element (8;
    info[4] = 6 + op->bdb;                       // FP32 9 / 11: hex paired kernel, per element / per
                                                 // point; 10: tet tensor cores)
    info[5] = (op->prec_mask & 2) ? (op->bdb_pair ? (op->bdb == 2 ? 9 : 11) : op->tet_bdb_tc ? 10 : 6 + op->bdb)
                                  : -1;
  }
  if (op->kind == GH1_OP_CSR) {  // autotuned SpMV configuration (0 until the first SpMV)
    info[4] = op->spmv_L[0];
    info[5] = op->spmv_L[1];
  }
  return GH1_OK;
}


int gh1_op_block_create(gh1_op* op, int nblocks, gh1_op** out) {
  if (!op || !out) return GH1_ERR_ARG;
  return guard(op->ctx, [&] {
    GH1_CHECK(nblocks >= 1, GH1_ERR_ARG, "nblocks must be positive");
    GH1_CHECK(op->kind != GH1_OP_BLOCK, GH1_ERR_ARG, "the inner operator of a block operator is a scalar operator");
    auto* b = new gh1_op();
    b->ctx = op->ctx;
    b->kind = GH1_OP_BLOCK;
    b->inner = op;
    b->nblocks = nblocks;
    b->nrows = (int64_t)nblocks * op->nrows;
    b->sp = op->sp;  // for gh1_op_info (elements, order); the DOFs are nblocks * sp->ndof
    b->prec_mask = op->kind == GH1_OP_CSR ? 3 : op->prec_mask;
    *out = b;
  });
}

int gh1_op_apply(gh1_op* op, double s, const void* x, void* y, int prec, int accumulate) {
  if (!op || !x || !y) return op ? (op->ctx->err = "null vector", GH1_ERR_ARG) : GH1_ERR_ARG;
  return guard(op->ctx, [&] {
    GH1_CHECK(prec == GH1_F64 || prec == GH1_F32, GH1_ERR_ARG, "precision must be GH1_F64 or GH1_F32");
    GH1_CHECK(x != y, GH1_ERR_ARG, "x and y must not alias");
    cudaStream_t st = op->ctx->stream;
    const size_t es = prec == GH1_F64 ? 8 : 4;
    bool plain = (s == 1.0 && !accumulate);
    void* target = y;
    if (!plain) {
      if (prec == GH1_F64) { if (op->d_tmp64.n < (size_t)op->nrows) op->d_tmp64.alloc(op->nrows); target = op->d_tmp64.p; }
      else { if (op->d_tmp32.n < (size_t)op->nrows) op->d_tmp32.alloc(op->nrows); target = op->d_tmp32.p; }
    }
    if (op->kind == GH1_OP_CSR) {
      spmv(op, x, target, prec);
    } else {
      GH1_CHECK(prec == GH1_F64 ? (op->prec_mask & 1) : (op->prec_mask & 2), GH1_ERR_UNSUPPORTED,
                "operator was not set up for this precision");
      op_refresh_any(op);
      op_prepare_any(op, prec);
      GH1_CUDA(cudaMemsetAsync(target, 0, op->nrows * es, st));
      op_apply_any(op, x, target, prec, nullptr);
    }
    if (!plain) vec_axpby(op->ctx, op->nrows, s, target, accumulate ? 1.0 : 0.0, y, prec);
  });
}

int gh1_op_check(gh1_op* op) {
  if (!op) return GH1_ERR_ARG;
  return guard(op->ctx, [&] {
    GH1_CUDA(cudaStreamSynchronize(op->ctx->stream));
    op_check_err(op);
  });
}

int gh1_op_free(gh1_op* op) { delete op; return GH1_OK; }

int gh1_jacobi_create(gh1_op* op, const uint8_t* freedofs, int mem, gh1_pre** out) {
  if (!op || !out) return GH1_ERR_ARG;
  return guard(op->ctx, [&] {
    GH1_CUDA(cudaSetDevice(op->ctx->device));
    cudaStream_t st = op->ctx->stream;
    gh1_pre* pr = new gh1_pre();
    pr->op = op; pr->ctx = op->ctx; pr->n = op->nrows;
    try {
      pr->d_free.alloc(op->nrows);
      if (freedofs) {
        GH1_CUDA(cudaMemcpyAsync(pr->d_free.p, freedofs, op->nrows,
                                 mem == GH1_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
      } else if (op->sp) {  // the space's free DOFs, once per block of a block operator
        const int64_t n = op->sp->ndof;
        for (int64_t o = 0; o < op->nrows; o += n)
          GH1_CUDA(cudaMemcpyAsync(pr->d_free.p + o, op->sp->d_free.p, n, cudaMemcpyDeviceToDevice, st));
      } else {
        GH1_CUDA(cudaMemsetAsync(pr->d_free.p, 1, op->nrows, st));
      }
      DBuf<double> diag(op->nrows);
      op_diag_any(op, diag.p);
      pr->d_inv64.alloc(op->nrows);
      pr->d_inv32.alloc(op->nrows);
      jacobi_invert(op->ctx, op->nrows, diag.p, pr->d_free.p, pr->d_inv64.p, pr->d_inv32.p);
      GH1_CUDA(cudaStreamSynchronize(st));
    } catch (...) { delete pr; throw; }
    *out = pr;
  });
}

int gh1_pre_apply(gh1_pre* pr, double s, const void* x, void* y, int prec, int accumulate) {
  if (!pr || !x || !y) return GH1_ERR_ARG;
  return guard(pr->ctx, [&] {
    GH1_CHECK(prec == GH1_F64 || prec == GH1_F32, GH1_ERR_ARG, "precision must be GH1_F64 or GH1_F32");
    pre_prepare(pr);
    pre_apply_any(pr, s, x, y, prec, accumulate);
  });
}

int gh1_pre_free(gh1_pre* pr) { delete pr; return GH1_OK; }


int gh1_space_smoothing_blocks(gh1_space* sp, int blocktype, int64_t* nblocks, int64_t* nentries, int64_t* offsets,
                               int32_t* dofs) {
  if (!sp || !nblocks || !nentries) return GH1_ERR_ARG;
  return guard(sp->ctx, [&] {
    std::vector<int64_t> off;
    std::vector<int32_t> d;
    smoothing_blocks(sp, blocktype, off, d);
    *nblocks = (int64_t)off.size() - 1;
    *nentries = (int64_t)d.size();
    if (offsets) std::copy(off.begin(), off.end(), offsets);
    if (dofs) std::copy(d.begin(), d.end(), dofs);
  });
}

int gh1_blockjacobi_create(gh1_op* csr, int64_t nblocks, const int64_t* offsets, const int32_t* dofs, int mem,
                           gh1_pre** out) {
  if (!csr || !out || nblocks < 0 || (nblocks > 0 && (!offsets || !dofs))) return GH1_ERR_ARG;
  return guard(csr->ctx, [&] {
    GH1_CHECK(mem == GH1_MEM_HOST || mem == GH1_MEM_DEVICE, GH1_ERR_ARG, "mem must be GH1_MEM_HOST or GH1_MEM_DEVICE");
    GH1_CUDA(cudaSetDevice(csr->ctx->device));
    cudaStream_t st = csr->ctx->stream;
    const auto kind = mem == GH1_MEM_DEVICE ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost;
    std::vector<int64_t> off(nblocks + 1, 0);
    if (nblocks > 0) GH1_CUDA(cudaMemcpy(off.data(), offsets, (nblocks + 1) * sizeof(int64_t), kind));
    GH1_CHECK(off[0] == 0, GH1_ERR_ARG, "offsets[0] must be 0");
    for (int64_t b = 0; b < nblocks; b++) GH1_CHECK(off[b + 1] >= off[b], GH1_ERR_ARG, "offsets must not decrease");
    std::vector<int32_t> d(off[nblocks]);
    if (!d.empty()) GH1_CUDA(cudaMemcpy(d.data(), dofs, d.size() * sizeof(int32_t), kind));
    gh1_pre* pr = new gh1_pre();
    pr->ctx = csr->ctx;
    pr->n = csr->nrows;
    try {
      block_jacobi_setup(pr, csr, nblocks, off, d);
      // free mask: the DOFs some block covers
      std::vector<uint8_t> mask(csr->nrows, 0);
      for (int32_t x : d) mask[x] = 1;
      pr->d_free.upload(mask, st);
      GH1_CUDA(cudaStreamSynchronize(st));
    } catch (...) { delete pr; throw; }
    *out = pr;
  });
}

int gh1_coarse_create(gh1_op* csr, int64_t nfine, const int32_t* embed, const uint8_t* freedofs, int mem,
                      gh1_pre** out) {
  if (!csr || !out || nfine <= 0) return GH1_ERR_ARG;
  return guard(csr->ctx, [&] {
    GH1_CHECK(mem == GH1_MEM_HOST || mem == GH1_MEM_DEVICE, GH1_ERR_ARG, "mem must be GH1_MEM_HOST or GH1_MEM_DEVICE");
    GH1_CUDA(cudaSetDevice(csr->ctx->device));
    cudaStream_t st = csr->ctx->stream;
    const auto kind = mem == GH1_MEM_DEVICE ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost;
    const int64_t nco = csr->nrows;
    GH1_CHECK(embed || nco <= nfine, GH1_ERR_ARG, "the identity embedding needs nfine >= the coarse size");
    std::vector<int32_t> emb(nco);
    if (embed) GH1_CUDA(cudaMemcpy(emb.data(), embed, nco * sizeof(int32_t), kind));
    else for (int64_t i = 0; i < nco; i++) emb[i] = (int32_t)i;
    std::vector<uint8_t> cf(nco, 1);
    if (freedofs) GH1_CUDA(cudaMemcpy(cf.data(), freedofs, nco, kind));
    gh1_pre* pr = new gh1_pre();
    pr->ctx = csr->ctx;
    pr->n = nfine;
    try {
      coarse_setup(pr, csr, nfine, emb, cf);
      std::vector<uint8_t> mask(nfine, 0);
      for (int64_t i = 0; i < nco; i++)
        if (cf[i]) mask[emb[i]] = 1;
      pr->d_free.upload(mask, st);
      GH1_CUDA(cudaStreamSynchronize(st));
    } catch (...) { delete pr; throw; }
    *out = pr;
  });
}

int gh1_pre_sum(gh1_pre* a, gh1_pre* b, gh1_pre** out) {
  if (!a || !b || !out) return GH1_ERR_ARG;
  return guard(a->ctx, [&] {
    GH1_CHECK(a->n == b->n && a->ctx == b->ctx, GH1_ERR_ARG, "the two preconditioners differ in size or context");
    gh1_pre* pr = new gh1_pre();
    pr->ctx = a->ctx;
    pr->n = a->n;
    pr->kind = 3;
    pr->a = a;
    pr->b = b;
    try {
      // free mask: the union of the parts'
      pr->d_free.alloc(pr->n);
      std::vector<uint8_t> ma(pr->n), mb(pr->n);
      GH1_CUDA(cudaMemcpy(ma.data(), a->d_free.p, pr->n, cudaMemcpyDeviceToHost));
      GH1_CUDA(cudaMemcpy(mb.data(), b->d_free.p, pr->n, cudaMemcpyDeviceToHost));
      for (int64_t i = 0; i < pr->n; i++) ma[i] |= mb[i];
      pr->d_free.upload(ma, a->ctx->stream);
      GH1_CUDA(cudaStreamSynchronize(a->ctx->stream));
    } catch (...) { delete pr; throw; }
    *out = pr;
  });
}

int gh1_rhs_elementwise(gh1_space* sp, const double* f, int mem, double* b) {
  if (!sp || !f || !b) return GH1_ERR_ARG;
  return guard(sp->ctx, [&] {
    DBuf<double> df;
    upload_coef(sp->ctx, df, f, mem, sp->mesh->ne, 0.0);
    rhs_elementwise(sp, df.p, b);
    GH1_CUDA(cudaStreamSynchronize(sp->ctx->stream));
  });
}

int gh1_cg(gh1_op* op, gh1_pre* pre, const double* b, double* x, const gh1_cg_opts* o, gh1_cg_result* r) {
  if (!op || !b || !x || !o || !r) return op ? (op->ctx->err = "null argument", GH1_ERR_ARG) : GH1_ERR_ARG;
  int status = GH1_OK;
  int rc = guard(op->ctx, [&] {
    GH1_CHECK(o->mode == GH1_CG_FP64 || o->mode == GH1_CG_MIXED, GH1_ERR_ARG, "unknown CG mode");
    GH1_CHECK(o->mode == GH1_CG_FP64 || pre, GH1_ERR_ARG, "mixed-precision CG needs a preconditioner");
    GH1_CHECK(o->maxit > 0 && o->tol >= 0, GH1_ERR_ARG, "maxit must be positive and tol non-negative");
    op_refresh_any(op);
    status = cg_solve(op, pre, b, x, o, r);
  });
  return rc != GH1_OK ? rc : status;
}

int gh1_elem_grad_dot(gh1_space* sp, const double* u, const double* w, double* out) {
  if (!sp || !u || !w || !out) return GH1_ERR_ARG;
  return guard(sp->ctx, [&] { elem_grad_dot(sp, u, w, out); });
}

int gh1_shape_eval(gh1_ctx* ctx, int et, int order, const int32_t* vnums, int npts, const double* pts,
                   double* val, double* grad) {
  if (!ctx || !vnums || !pts || !val || !grad || npts <= 0) return GH1_ERR_ARG;
  return guard(ctx, [&] {
    GH1_CHECK(et == 4 || et == 8, GH1_ERR_UNSUPPORTED, "element type must be 4 or 8");
    GH1_CHECK(order >= 1 && order <= (et == 4 ? MAX_TET_ORDER : MAX_HEX_ORDER), GH1_ERR_UNSUPPORTED, "order out of range");
    shape_eval_gpu(ctx, et, order, vnums, npts, pts, val, grad);
  });
}

}  // extern "C"
