// bdb.cu -- generic B^T D B operator: y = A x for
//   a(u, v) = sum_e int_e (B v)^T D (B u) dx,   B w = (w, dw/dx, dw/dy, dw/dz),
// with D a 4x4 matrix per element or per rule point: any bilinear integrand in
// u, grad u, v, grad v (full diffusion tensors, convection b.grad(u) v and its
// transpose u c.grad(v), reaction, non-symmetric combinations).
//
// Replaces the reference's fused symbolic B^T D B operator: AssembleBDBFused
// (comp/matrixfree.cpp:1090-1330) evaluates D per element from the integrand,
// one entry per (trial component, test component) pair, and keeps the
// Jacobians per element (per point on curved elements); MatrixFreeBTDTB
// (ngscuda/cuda_matrix_free_btdtb.cpp:60-310) applies B^T (J-transformed D) B
// on the device.  Here setup folds the geometry into reference-coordinate
// matrices
//   Mh = s T^T D T,   T = diag(1, J^{-T}),   s = w |det J|,
// so the kernels need no Jacobian:
//  - hex: the sum-factorized one-element apply of hexsf.cuh with the point
//    transform (vm, vx, vy, vz) = Mh (u, du/dxi, du/deta, du/dzeta); G mode 2
//    streams Mh per point, G mode 3 (affine hexes, D per element) reads one
//    16-value record per element and applies the rule weight in the kernel;
//  - tet: tetapply.cu (same-class tiles, 16-point chunks of the degree-2p rule).
// The rule is the one of the space: tensor Gauss with p+1 points per direction
// on hexes, degree 2p on tets (the reference's BDB rule has order 2p as well).
#include <cstdlib>
#include <string>
#include <vector>
#include "common.cuh"
#include "hexcore.cuh"
#include "hexsf.cuh"
#include "deform.cuh"

namespace gh1 {

// Mh[r][c] = s sum_{a,b} T[a][r] D[a][b] T[b][c] with T = diag(1, J^{-T}): the
// physical gradient component k of a shape is sum_j Ji[3j+k] times its reference
// component j (Ji = J^{-1}, row-major).  D and Mh are row = test, column = trial.
__device__ __forceinline__ void bdb_transform(const double* Ji, const double* D, double s, double* M) {
  double T[4][4];
  for (int a = 0; a < 4; a++)
    for (int c = 0; c < 4; c++) T[a][c] = 0;
  T[0][0] = 1;
  for (int k = 0; k < 3; k++)
    for (int j = 0; j < 3; j++) T[1 + k][1 + j] = Ji[3 * j + k];
  double DT[4][4];
  for (int a = 0; a < 4; a++)
    for (int c = 0; c < 4; c++) {
      double v = 0;
      for (int b = 0; b < 4; b++) v += D[4 * a + b] * T[b][c];
      DT[a][c] = v;
    }
  for (int r = 0; r < 4; r++)
    for (int c = 0; c < 4; c++) {
      double v = 0;
      for (int a = 0; a < 4; a++) v += T[a][r] * DT[a][c];
      M[4 * r + c] = s * v;
    }
}

// hex, per rule point: G[e*gs + m*nq + q] = Mh_m (m = 4 r + c), D per element
// ([e][16]) or per point ([e][q][16])
__global__ void hex_bdb_point_kernel(int ne, int nq1, const double* __restrict__ X, const int* __restrict__ el,
                                     const double* __restrict__ gx, const double* __restrict__ gw,
                                     const double* __restrict__ D, int per_point, double* G64, int gs64, float* G32,
                                     int gs32, DeformView dv) {
  const int nq = nq1 * nq1 * nq1;
  const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= (int64_t)ne * nq) return;
  const int e = (int)(id / nq), q = (int)(id % nq);
  const int i = q / (nq1 * nq1), j = (q / nq1) % nq1, k = q % nq1;
  int v[8];
  for (int a = 0; a < 8; a++) v[a] = el[(size_t)e * 8 + a];
  double J[9], Ji[9], det;
  hex_jacobian(X, v, gx[i], gx[j], gx[k], J);
  deform_add(dv, e, gx[i], gx[j], gx[k], J, nullptr);
  inv3(J, Ji, det);
  const double* De = per_point ? D + ((size_t)e * nq + q) * 16 : D + (size_t)e * 16;
  double M[16];
  bdb_transform(Ji, De, gw[i] * gw[j] * gw[k] * fabs(det), M);
  for (int m = 0; m < 16; m++) {
    if (G64) G64[(size_t)e * gs64 + (size_t)m * nq + q] = M[m];
    if (G32) G32[(size_t)e * gs32 + (size_t)m * nq + q] = (float)M[m];
  }
}

// hex, one record per element (D per element): Mh without the rule weight from
// the Jacobian at the center.  *flag = 1 when the Jacobian at a vertex of the
// reference cube differs from the center one: that element map is not affine
// and the caller switches to per-point records.
__global__ void hex_bdb_elem_kernel(int ne, const double* __restrict__ X, const int* __restrict__ el,
                                    const double* __restrict__ D, double* G64, float* G32, int* flag) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  int v[8];
  for (int a = 0; a < 8; a++) v[a] = el[(size_t)e * 8 + a];
  double J0[9], J[9], Ji[9], det, scale = 0, dev = 0;
  hex_jacobian(X, v, 0.5, 0.5, 0.5, J0);
  for (int c = 0; c < 9; c++) scale = fmax(scale, fabs(J0[c]));
  for (int corner = 0; corner < 8; corner++) {
    hex_jacobian(X, v, corner & 1, (corner >> 1) & 1, (corner >> 2) & 1, J);
    for (int c = 0; c < 9; c++) dev = fmax(dev, fabs(J[c] - J0[c]));
  }
  if (dev > 1e-12 * scale) atomicExch(flag, 1);
  inv3(J0, Ji, det);
  double M[16];
  bdb_transform(Ji, D + (size_t)e * 16, fabs(det), M);
  for (int m = 0; m < 16; m++) {
    if (G64) G64[(size_t)e * 16 + m] = M[m];
    if (G32) G32[(size_t)e * 16 + m] = (float)M[m];
  }
}

// tet, map x = v3 + sum_j (v_j - v3) xi_j (+ the deformation): one record
// [e][16] without the rule weight (out_pp = 0: affine element, D per element), or
// [e][q][16] with it (out_pp = 1); D per element or per point (d_pp)
__global__ void tet_bdb_geom_kernel(int ne, int nq, const double* __restrict__ X, const int* __restrict__ el,
                                    const double* __restrict__ rule, const double* __restrict__ D, int d_pp, int out_pp,
                                    double* M64, float* M32, DeformView dv) {
  const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int nper = out_pp ? nq : 1;
  if (id >= (int64_t)ne * nper) return;
  const int e = (int)(id / nper), q = (int)(id % nper);
  const int* v = el + (size_t)e * 4;
  const double* p3 = X + 3 * (size_t)v[3];
  double J[9], Ji[9], det;
  for (int j = 0; j < 3; j++) {
    const double* pj = X + 3 * (size_t)v[j];
    for (int k = 0; k < 3; k++) J[3 * k + j] = pj[k] - p3[k];
  }
  if (out_pp) deform_add(dv, e, rule[4 * q], rule[4 * q + 1], rule[4 * q + 2], J, nullptr);
  inv3(J, Ji, det);
  const double s = out_pp ? rule[4 * q + 3] * fabs(det) : fabs(det);
  double M[16];
  bdb_transform(Ji, D + (d_pp ? (size_t)id : (size_t)e) * 16, s, M);
  for (int m = 0; m < 16; m++) {
    if (M64) M64[(size_t)id * 16 + m] = M[m];
    if (M32) M32[(size_t)id * 16 + m] = (float)M[m];
  }
}

// Diagonal of the hex operator, sum-factorized as for Laplace + mass: each of
// the 10 symmetric component pairs (r <= s) of Mh + Mh^T is a product of 1D
// factor pairs, BB, DD or BD per direction (D where the pair differentiates in
// that direction), contracted direction by direction.
__global__ void __launch_bounds__(256) hex_bdb_diag_kernel(int ne, int N, const int* __restrict__ tdof, int tstride,
                                                            const double* __restrict__ G, int gstride, int per_elem,
                                                            const double* __restrict__ gw, const double* __restrict__ B,
                                                            const double* __restrict__ D, double* diag) {
  extern __shared__ double dsm[];
  const int N2 = N * N, N3 = N2 * N;
  double* g = dsm;
  double* h = dsm + 10 * N3;
  const int pr[10] = {0, 1, 2, 3, 0, 0, 0, 1, 1, 2}, ps[10] = {0, 1, 2, 3, 1, 2, 3, 2, 3, 3};
  // factor selector of pair m in direction d (1 = x, 2 = y, 3 = z): 0 = B*B, 1 = D*D, 2 = B*D
  auto sel = [&](int m, int d) {
    const int c = (pr[m] == d) + (ps[m] == d);
    return c == 0 ? 0 : (c == 2 ? 1 : 2);
  };
  auto fac = [&](int s, int q, int a) {
    const double b = B[q * N + a], d = D[q * N + a];
    return s == 0 ? b * b : (s == 1 ? d * d : b * d);
  };
  for (int e = blockIdx.x; e < ne; e += gridDim.x) {
    const double* Ge = G + (size_t)e * gstride;
    for (int t = threadIdx.x; t < 10 * N3; t += blockDim.x) {
      const int m = t / N3, q = t % N3, r = pr[m], s = ps[m];
      double v;
      if (per_elem) {
        const double w = gw[q / N2] * gw[(q / N) % N] * gw[q % N];
        v = w * (Ge[4 * r + s] + (r != s ? Ge[4 * s + r] : 0.0));
      } else {
        v = Ge[(size_t)(4 * r + s) * N3 + q] + (r != s ? Ge[(size_t)(4 * s + r) * N3 + q] : 0.0);
      }
      g[t] = v;
    }
    __syncthreads();
    // z: h[m][i][j][c] = sum_k f(k,c) g[m][i][j][k]
    for (int t = threadIdx.x; t < 10 * N3; t += blockDim.x) {
      const int m = t / N3, r = t % N3, ij = r / N, c = r % N, f = sel(m, 3);
      double v = 0;
      for (int k = 0; k < N; k++) v += fac(f, k, c) * g[m * N3 + ij * N + k];
      h[t] = v;
    }
    __syncthreads();
    // y: g[m][i][b][c] = sum_j f(j,b) h[m][i][j][c]
    for (int t = threadIdx.x; t < 10 * N3; t += blockDim.x) {
      const int m = t / N3, r = t % N3, i = r / N2, b = (r / N) % N, c = r % N, f = sel(m, 2);
      double v = 0;
      for (int j = 0; j < N; j++) v += fac(f, j, b) * h[m * N3 + (i * N + j) * N + c];
      g[t] = v;
    }
    __syncthreads();
    // x, and the sum over the pairs
    for (int t = threadIdx.x; t < N3; t += blockDim.x) {
      const int a = t / N2, bc = t % N2;
      double v = 0;
      for (int m = 0; m < 10; m++) {
        const int f = sel(m, 1);
        for (int i = 0; i < N; i++) v += fac(f, i, a) * g[m * N3 + i * N2 + bc];
      }
      red_add(diag + (tdof[(size_t)e * tstride + t] & 0x7fffffff), v);
    }
    __syncthreads();
  }
}

// D per element of the form kappa grad.grad + mu u v (or K grad.grad + mu u v):
// the B^T D B path of curved tets takes the standard forms this way
__global__ void coef_bdb_kernel(int ne, const double* __restrict__ kappa, const double* __restrict__ K6,
                                const double* __restrict__ mu, double* D) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  double* d = D + (size_t)e * 16;
  for (int c = 0; c < 16; c++) d[c] = 0;
  d[0] = mu ? mu[e] : 0.0;
  if (K6) {
    const double* k = K6 + (size_t)e * 6;
    d[5] = k[0]; d[10] = k[1]; d[15] = k[2];
    d[6] = d[9] = k[3];
    d[7] = d[13] = k[4];
    d[11] = d[14] = k[5];
  } else {
    d[5] = d[10] = d[15] = kappa[e];
  }
}

// structure of D records: flags[0] = a value-gradient coupling is non-zero,
// flags[1] = the gradient block is not symmetric, flags[2] = the value entry is
// non-zero somewhere
__global__ void bdb_structure_kernel(int64_t nrec, const double* __restrict__ D, int* flags) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrec; r += (int64_t)gridDim.x * blockDim.x) {
    const double* d = D + r * 16;
    if (d[1] != 0.0 || d[2] != 0.0 || d[3] != 0.0 || d[4] != 0.0 || d[8] != 0.0 || d[12] != 0.0) atomicOr(flags, 1);
    double sc = 0;
    for (int c = 5; c < 16; c++) sc = fmax(sc, fabs(d[c]));
    const double tol = 1e-14 * sc;
    if (fabs(d[6] - d[9]) > tol || fabs(d[7] - d[13]) > tol || fabs(d[11] - d[14]) > tol) atomicOr(flags + 1, 1);
    if (d[0] != 0.0) atomicOr(flags + 2, 1);
  }
}

// per-element D of Laplace type -> K6 (xx yy zz xy xz yz) and mu
__global__ void bdb_to_k6_kernel(int ne, const double* __restrict__ D, double* K6, double* mu) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const double* d = D + (size_t)e * 16;
  double* k = K6 + (size_t)e * 6;
  k[0] = d[5]; k[1] = d[10]; k[2] = d[15];
  k[3] = 0.5 * (d[6] + d[9]); k[4] = 0.5 * (d[7] + d[13]); k[5] = 0.5 * (d[11] + d[14]);
  if (mu) mu[e] = d[0];
}

// A generic form on hexes whose D is diag(mu, K) with K symmetric (diffusion
// with any tensor, reaction; no convection) is the standard operator with
// per-element or per-point coefficients: it takes the standard kernels (all
// autotuned variants, the per-element metric on affine meshes) instead of the
// 16-coefficient B^T D B kernel.  GH1_BDB_STANDARD=0 keeps the B^T D B kernel.
bool bdb_laplace_route(gh1_op* op) {
  gh1_space* sp = op->sp;
  gh1_form* f = op->form;
  op->lap_ov = false;
  op->lap_pp = nullptr;
  op->d_ovK6.release();
  op->d_ovmu.release();
  const char* env = getenv("GH1_BDB_STANDARD");
  if (sp->et != 8 || !f->bdb_mode || (env && std::string(env) == "0")) return false;
  cudaStream_t s = sp->ctx->stream;
  const int ne = sp->mesh->ne, nq = sp->nq1 * sp->nq1 * sp->nq1;
  const int64_t nrec = (int64_t)ne * (f->bdb_mode == 2 ? nq : 1);
  DBuf<int> flags(3);
  flags.zero(s);
  if (nrec > 0) {
    bdb_structure_kernel<<<grid_for(sp->ctx, nrec, 256), 256, 0, s>>>(nrec, f->d_bdb.p, flags.p);
    check_kernel(sp->ctx, "bdb_structure_kernel");
  }
  int h[3] = {0, 0, 0};
  GH1_CUDA(cudaMemcpyAsync(h, flags.p, sizeof(h), cudaMemcpyDeviceToHost, s));
  GH1_CUDA(cudaStreamSynchronize(s));
  if (h[0] || h[1]) return false;
  op->lap_ov = true;
  op->has_mass = h[2] != 0;
  if (f->bdb_mode == 2) {
    op->lap_pp = f->d_bdb.p;
  } else {
    op->d_ovK6.alloc((size_t)std::max(ne, 1) * 6);
    if (op->has_mass) op->d_ovmu.alloc(std::max(ne, 1));
    if (ne > 0) {
      bdb_to_k6_kernel<<<(ne + 127) / 128, 128, 0, s>>>(ne, f->d_bdb.p, op->d_ovK6.p, op->has_mass ? op->d_ovmu.p : nullptr);
      check_kernel(sp->ctx, "bdb_to_k6_kernel");
    }
    GH1_CUDA(cudaStreamSynchronize(s));
  }
  return true;
}

#define GH1_BDB_SWITCH(N, CASE)                                                                        \
  switch (N) {                                                                                         \
    CASE(2) CASE(3) CASE(4) CASE(5) CASE(6) CASE(7) CASE(8) CASE(9)                                   \
    default: throw Error(GH1_ERR_UNSUPPORTED, "hex order out of range");                              \
  }

template <class T>
static int hex_bdb_occupancy(gh1_op* op, int gstride) {
  const int tstride = op->sp->tstride;
  int v = 0;
#define GH1_BOCC_CASE(NN)                                                                                   \
  case NN:                                                                                                  \
    v = op->bdb == 2 ? hex_apply_occupancy<NN, T, true, 3>(HexSmem<NN, T>::total(gstride, tstride, 3))     \
                     : hex_apply_occupancy<NN, T, true, 2>(HexSmem<NN, T>::total(gstride, tstride, 2));    \
    break;
  GH1_BDB_SWITCH(op->sp->p + 1, GH1_BOCC_CASE)
#undef GH1_BOCC_CASE
  return v;
}

template <class T>
static void hex_bdb_launch(gh1_op* op, const T* x, T* y, const T* G, int gstride, double* partial,
                           unsigned int* counter, double* energy, const int* skip) {
#define GH1_BAPP_CASE(NN)                                                                                  \
  case NN:                                                                                                 \
    if (op->bdb == 2) launch_hex_apply<NN, T, true, 3>(op, x, y, G, gstride, partial, counter, energy, skip); \
    else launch_hex_apply<NN, T, true, 2>(op, x, y, G, gstride, partial, counter, energy, skip);          \
    break;
  GH1_BDB_SWITCH(op->sp->p + 1, GH1_BAPP_CASE)
#undef GH1_BAPP_CASE
}

// FP32 records Mh = |det J| T^T D T per element (reference coordinates, no rule
// weight) of a standard tet form, D = diag(mu, kappa I or K): the input of the
// tensor-core B^T D B kernel for stiffness + mass forms
void tet_standard_records(gh1_op* op, float* M32) {
  gh1_space* sp = op->sp;
  gh1_form* f = op->form;
  const int ne = sp->mesh->ne;
  if (ne == 0) return;
  cudaStream_t s = sp->ctx->stream;
  DBuf<double> D((size_t)ne * 16), M64((size_t)ne * 16);
  coef_bdb_kernel<<<(ne + 127) / 128, 128, 0, s>>>(ne, f->d_kappa.p, f->has_K6 ? f->d_K6.p : nullptr,
                                                  op->has_mass ? f->d_mu.p : nullptr, D.p);
  check_kernel(sp->ctx, "coef_bdb_kernel");
  tet_bdb_geom_kernel<<<(ne + 127) / 128, 128, 0, s>>>(ne, sp->tet_nq_mass, sp->mesh->d_X.p, sp->mesh->d_el.p,
                                                       sp->d_tqm.p, D.p, 0, 0, M64.p, M32, deform_view(sp->mesh));
  check_kernel(sp->ctx, "tet_bdb_geom_kernel");
  GH1_CUDA(cudaStreamSynchronize(s));  // D and M64 go out of scope
}

// FP32: the paired kernel (two elements per lane; G mode 3 of hexpair.cu with one
// record per affine element, 4 with records per point) or the one-element
// kernel, whichever is faster on this operator's mesh (GH1_BDB_PAIR=0/1 forces one)
static int bdb_pair_mode(const gh1_op* op) { return op->bdb == 2 ? 3 : 4; }

static bool bdb_pair_choice(gh1_op* op) {
  gh1_space* sp = op->sp;
  op->bdb_pair = false;
  op->pair_per_sm[3] = op->pair_per_sm[4] = 0;
  if (!(op->prec_mask & 2) || !op->bdb || !hex_pair_supported(sp->p + 1)) return false;
  set_first_wait_polls();
  upload_pair_tables(sp);
  const int gm = bdb_pair_mode(op);
  op->pair_per_sm[gm] = hex_pair_occupancy(op, gm);
  if (op->pair_per_sm[gm] <= 0) return false;
  const char* env = getenv("GH1_BDB_PAIR");
  if (env) return env[0] == '1';
  if (sp->mesh->ne < 4096) return false;
  cudaStream_t s = sp->ctx->stream;
  DBuf<float> xs(op->nrows), ys(op->nrows);
  xs.zero(s);
  cudaEvent_t a, b;
  GH1_CUDA(cudaEventCreate(&a));
  GH1_CUDA(cudaEventCreate(&b));
  float ms[2];
  for (int v = 0; v < 2; v++) {
    for (int r = 0; r < 5; r++) {
      if (r == 2) GH1_CUDA(cudaEventRecord(a, s));
      if (v == 0) hex_bdb_launch<float>(op, xs.p, ys.p, op->d_G32.p, op->gstride32, nullptr, nullptr, nullptr, nullptr);
      else hex_pair_apply(op, gm, xs.p, ys.p, nullptr, nullptr, nullptr, nullptr);
    }
    GH1_CUDA(cudaEventRecord(b, s));
    GH1_CUDA(cudaEventSynchronize(b));
    GH1_CUDA(cudaEventElapsedTime(&ms[v], a, b));
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms[1] < ms[0];
}

void bdb_setup(gh1_op* op) {
  gh1_space* sp = op->sp;
  gh1_form* f = op->form;
  cudaStream_t s = sp->ctx->stream;
  const int ne = sp->mesh->ne;
  const bool want32 = (op->prec_mask & 2) != 0;
  const bool deformed = sp->mesh->def_space != nullptr;
  const DeformView dv = deform_view(sp->mesh);
  // D: the form's generic matrices, or (a standard form on a curved tet mesh)
  // diag(mu, kappa I or K) per element
  int dmode = f->bdb_mode;
  const double* Dsrc = f->d_bdb.p;
  DBuf<double> Dcoef;
  if (dmode == 0) {
    Dcoef.alloc((size_t)std::max(ne, 1) * 16);
    if (ne > 0) {
      coef_bdb_kernel<<<(ne + 127) / 128, 128, 0, s>>>(ne, f->d_kappa.p, f->has_K6 ? f->d_K6.p : nullptr,
                                                      f->has_mu ? f->d_mu.p : nullptr, Dcoef.p);
      check_kernel(sp->ctx, "coef_bdb_kernel");
    }
    Dsrc = Dcoef.p;
    dmode = 1;
  }
  op->has_mass = true;  // the value component is always interpolated
  op->d_M64.release();
  op->d_M32.release();
  if (sp->et == 8) {
    const int nq = sp->nq1 * sp->nq1 * sp->nq1;
    // one record per element when D is per element and every element map is
    // affine (GH1_BDB_AFFINE=0 keeps the per-point records)
    const char* env = getenv("GH1_BDB_AFFINE");
    bool elem = dmode == 1 && !(env && std::string(env) == "0") && ne > 0 && !op->bdb_points_only && !deformed;
    if (elem) {
      op->d_G64.alloc((size_t)ne * 16);
      if (want32) op->d_G32.alloc((size_t)ne * 16); else op->d_G32.release();
      DBuf<int> flag(1);
      flag.zero(s);
      hex_bdb_elem_kernel<<<(ne + 127) / 128, 128, 0, s>>>(ne, sp->mesh->d_X.p, sp->mesh->d_el.p, Dsrc, op->d_G64.p,
                                                           want32 ? op->d_G32.p : nullptr, flag.p);
      check_kernel(sp->ctx, "hex_bdb_elem_kernel");
      int h = 0;
      GH1_CUDA(cudaMemcpyAsync(&h, flag.p, sizeof(int), cudaMemcpyDeviceToHost, s));
      GH1_CUDA(cudaStreamSynchronize(s));
      elem = h == 0;
      op->gstride64 = op->gstride32 = 16;
    }
    if (!elem) {
      op->gstride64 = (int)(round16((size_t)16 * nq * sizeof(double)) / sizeof(double));
      op->gstride32 = (int)(round16((size_t)16 * nq * sizeof(float)) / sizeof(float));
      op->d_G64.alloc((size_t)ne * op->gstride64);
      if (want32) op->d_G32.alloc((size_t)ne * op->gstride32); else op->d_G32.release();
      const int64_t tot = (int64_t)ne * nq;
      if (tot > 0) {
        hex_bdb_point_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(
            ne, sp->nq1, sp->mesh->d_X.p, sp->mesh->d_el.p, sp->d_gx.p, sp->d_gw.p, Dsrc, dmode == 2 ? 1 : 0,
            op->d_G64.p, op->gstride64, want32 ? op->d_G32.p : nullptr, op->gstride32, dv);
        check_kernel(sp->ctx, "hex_bdb_point_kernel");
      }
    }
    op->ncomp = 16;
    op->bdb = elem ? 2 : 1;
    upload_const_tables(sp);
    op->bdb_per_sm[0] = hex_bdb_occupancy<double>(op, op->gstride64);
    op->bdb_per_sm[1] = want32 ? hex_bdb_occupancy<float>(op, op->gstride32) : 0;
    op->bdb_pair = bdb_pair_choice(op);
  } else {
    const int nq = sp->tet_nq_mass, d_pp = dmode == 2 ? 1 : 0, per_point = (d_pp || deformed) ? 1 : 0;
    const size_t nrec = (size_t)ne * (per_point ? nq : 1) * 16;
    op->d_G64.alloc(nrec);
    if (want32) op->d_G32.alloc(nrec); else op->d_G32.release();
    const int64_t tot = (int64_t)ne * (per_point ? nq : 1);
    if (tot > 0) {
      tet_bdb_geom_kernel<<<(unsigned)((tot + 127) / 128), 128, 0, s>>>(ne, nq, sp->mesh->d_X.p, sp->mesh->d_el.p,
                                                                        sp->d_tqm.p, Dsrc, d_pp, per_point, op->d_G64.p,
                                                                        want32 ? op->d_G32.p : nullptr, dv);
      check_kernel(sp->ctx, "tet_bdb_geom_kernel");
    }
    op->bdb = per_point ? 1 : 2;
    tet_bdb_setup(op);
  }
  GH1_CUDA(cudaStreamSynchronize(s));
  op->form_version = f->version;
  op->have_diag = false;
}

void bdb_apply(gh1_op* op, const void* x, void* y, int prec, double* partial, unsigned int* counter, double* energy,
               const int* skip) {
  if (op->sp->et != 8) {
    tet_bdb_apply(op, prec, x, y, partial, counter, energy, skip);
    return;
  }
  if (prec == GH1_F64)
    hex_bdb_launch<double>(op, (const double*)x, (double*)y, op->d_G64.p, op->gstride64, partial, counter, energy, skip);
  else if (op->bdb_pair)
    hex_pair_apply(op, bdb_pair_mode(op), (const float*)x, (float*)y, partial, counter, energy, skip);
  else
    hex_bdb_launch<float>(op, (const float*)x, (float*)y, op->d_G32.p, op->gstride32, partial, counter, energy, skip);
}

void bdb_diag(gh1_op* op, double* diag) {
  gh1_space* sp = op->sp;
  if (sp->et != 8) {
    tet_bdb_diag(op, diag);
    return;
  }
  const int ne = sp->mesh->ne, N = sp->p + 1;
  if (ne == 0) return;
  const size_t smem = (size_t)20 * N * N * N * sizeof(double);
  if (smem > 48 * 1024)
    GH1_CUDA(cudaFuncSetAttribute(hex_bdb_diag_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int grid = std::min(ne, sp->ctx->nsm * 8);
  hex_bdb_diag_kernel<<<grid, 256, smem, sp->ctx->stream>>>(ne, N, sp->d_tdof.p, sp->tstride, op->d_G64.p, op->gstride64,
                                                           op->bdb == 2 ? 1 : 0, sp->d_gw.p, sp->d_B64.p, sp->d_D64.p,
                                                           diag);
  check_kernel(sp->ctx, "hex_bdb_diag_kernel");
}

}  // namespace gh1
