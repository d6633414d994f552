// assemble.cu -- BilinearForm::Assemble on the GPU: CSR pattern, element
// matrices, scatter; and the element-wise right-hand side.
//
// Pattern: MatrixGraph (linalg/sparsematrix.cpp:450-900) -- row r holds the
// sorted union of the DOFs of all elements containing DOF r, diagonal included,
// full storage.  build_graph here is the host build (threads, marker arrays),
// used when graph.cu's GPU build does not apply (rows over its candidate cap).
// Element matrices: kappa grad.grad + mu u v (T_CalcElementMatrixAdd,
// fem/symbolicintegrator.cpp:1548-1830).
//   tet: K_e = sum_blk Gbar_blk S^c_blk + M_e S^c_mass with the per-class
//        reference blocks of tables.cu (exact for the affine map);
//   hex: K_tt' = sum_q (grad phi_t)^T G_q (grad phi_t') + M_q phi_t phi_t' with
//        the tensor factors of the 1D tables.
// Scatter: AddElementMatrix (linalg/sparsematrix_impl.hpp:148-190) as a binary
// search of the column in the sorted CSR row and an FP64 atomic add (the
// reference's use_atomic variant); a missing column raises the reference's
// "illegal dnums" error as GH1_ERR_ILLEGAL_DNUMS.
#include <algorithm>
#include <cstdlib>
#include <thread>
#include <vector>
#include "common.cuh"
#include "deform.cuh"

namespace gh1 {

void build_graph(gh1_space* sp) {
  const int64_t ndof = sp->ndof;
  const int ne = sp->mesh->ne, nloc = sp->nloc;
  const std::vector<int32_t>& ed = sp->el_dofs;
  std::vector<int64_t> cnt(ndof + 1, 0);
  for (size_t k = 0; k < ed.size(); k++) cnt[ed[k] + 1]++;
  for (int64_t i = 0; i < ndof; i++) cnt[i + 1] += cnt[i];
  std::vector<int32_t> dof2el(cnt[ndof]);
  {
    std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
    for (int e = 0; e < ne; e++)
      for (int i = 0; i < nloc; i++) dof2el[fill[ed[(size_t)e * nloc + i]]++] = e;
  }
  int nt = (int)std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
  std::vector<int64_t> rowlen(ndof, 0);
  // pass 1: row lengths (marker array per thread for de-duplication)
  auto pass = [&](int t, bool write, std::vector<int32_t>* colind, const std::vector<int64_t>* rowptr) {
    std::vector<int64_t> mark(ndof, -1);
    std::vector<int32_t> buf;
    int64_t chunk = (ndof + nt - 1) / nt, a = t * chunk, b = std::min(ndof, a + chunk);
    for (int64_t r = a; r < b; r++) {
      buf.clear();
      for (int64_t k = cnt[r]; k < cnt[r + 1]; k++) {
        const int32_t* d = &ed[(size_t)dof2el[k] * nloc];
        for (int i = 0; i < nloc; i++)
          if (mark[d[i]] != r) { mark[d[i]] = r; buf.push_back(d[i]); }
      }
      if (!write) { rowlen[r] = (int64_t)buf.size(); continue; }
      std::sort(buf.begin(), buf.end());
      std::copy(buf.begin(), buf.end(), colind->begin() + (*rowptr)[r]);
    }
  };
  {
    std::vector<std::thread> th;
    for (int t = 0; t < nt; t++) th.emplace_back(pass, t, false, nullptr, nullptr);
    for (auto& x : th) x.join();
  }
  std::vector<int64_t> rowptr(ndof + 1, 0);
  for (int64_t r = 0; r < ndof; r++) rowptr[r + 1] = rowptr[r] + rowlen[r];
  std::vector<int32_t> colind(rowptr[ndof]);
  {
    std::vector<std::thread> th;
    for (int t = 0; t < nt; t++) th.emplace_back(pass, t, true, &colind, &rowptr);
    for (auto& x : th) x.join();
  }
  sp->nnz = rowptr[ndof];
  sp->d_rowptr.upload(rowptr, sp->ctx->stream);
  sp->d_colind.upload(colind, sp->ctx->stream);
  GH1_CUDA(cudaStreamSynchronize(sp->ctx->stream));
  sp->have_graph = true;
}

__device__ __forceinline__ int64_t find_col(const int64_t* rowptr, const int32_t* colind, int row, int col) {
  int64_t lo = rowptr[row], hi = rowptr[row + 1] - 1;
  while (lo <= hi) {
    int64_t mid = (lo + hi) >> 1;
    int c = colind[mid];
    if (c == col) return mid;
    if (c < col) lo = mid + 1; else hi = mid - 1;
  }
  return -1;
}

// tet: one thread per (element, i, j)
__global__ void tet_assemble_kernel(int ne, int nloc, const int* __restrict__ eldofs, const uint8_t* __restrict__ cls,
                                    const double* __restrict__ Ge, const double* __restrict__ Me, const double* __restrict__ S,
                                    const int64_t* __restrict__ rowptr, const int32_t* __restrict__ colind, double* vals,
                                    int* bad) {
  const int64_t per = (int64_t)nloc * nloc;
  for (int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; id < (int64_t)ne * per;
       id += (int64_t)gridDim.x * blockDim.x) {
    int e = (int)(id / per), ij = (int)(id % per), i = ij / nloc, j = ij % nloc;
    const double* Sc = S + (size_t)cls[e] * 7 * per + ij;
    const double* g = Ge + (size_t)e * 6;
    double k = g[0] * Sc[0] + g[1] * Sc[per] + g[2] * Sc[2 * per] + g[3] * Sc[3 * per] + g[4] * Sc[4 * per] + g[5] * Sc[5 * per];
    if (Me) k += Me[e] * Sc[6 * per];
    int row = eldofs[(size_t)e * nloc + i], col = eldofs[(size_t)e * nloc + j];
    int64_t pos = find_col(rowptr, colind, row, col);
    if (pos < 0) { atomicExch(bad, 1); continue; }
    red_add(vals + pos, k);
  }
}

// hex: one thread per (element, t, t'), tensor indices with signs
// bdb != 0: the generic B^T D B form, Gq = [16][N3] reference-coordinate
// matrices per point (row = test component, column = trial component)
__global__ void hex_assemble_kernel(int ne, int N, const int* __restrict__ tdof, int tstride, const double* __restrict__ Gq,
                                    int gstride, int mass, int bdb, const double* __restrict__ B, const double* __restrict__ D,
                                    const int64_t* __restrict__ rowptr, const int32_t* __restrict__ colind, double* vals,
                                    int* bad) {
  const int N3 = N * N * N;
  const int64_t per = (int64_t)N3 * N3;
  for (int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; id < (int64_t)ne * per;
       id += (int64_t)gridDim.x * blockDim.x) {
    int e = (int)(id / per), tt = (int)(id % per), t = tt / N3, u = tt % N3;
    int a = t / (N * N), b = (t / N) % N, c = t % N;
    int a2 = u / (N * N), b2 = (u / N) % N, c2 = u % N;
    const double* Ge = Gq + (size_t)e * gstride;
    double s = 0;
    for (int i = 0; i < N; i++) {
      double Ba = B[i * N + a], Da = D[i * N + a], Ba2 = B[i * N + a2], Da2 = D[i * N + a2];
      for (int j = 0; j < N; j++) {
        double Bb = B[j * N + b], Db = D[j * N + b], Bb2 = B[j * N + b2], Db2 = D[j * N + b2];
        for (int k = 0; k < N; k++) {
          double Bc = B[k * N + c], Dc = D[k * N + c], Bc2 = B[k * N + c2], Dc2 = D[k * N + c2];
          int q = (i * N + j) * N + k;
          double x1 = Da * Bb * Bc, y1 = Ba * Db * Bc, z1 = Ba * Bb * Dc;
          double x2 = Da2 * Bb2 * Bc2, y2 = Ba2 * Db2 * Bc2, z2 = Ba2 * Bb2 * Dc2;
          if (bdb) {
            const double b1[4] = {Ba * Bb * Bc, x1, y1, z1}, b2[4] = {Ba2 * Bb2 * Bc2, x2, y2, z2};
            for (int r = 0; r < 4; r++)
              for (int cc = 0; cc < 4; cc++) s += b1[r] * Ge[(4 * r + cc) * N3 + q] * b2[cc];
            continue;
          }
          double gxx = Ge[q], gyy = Ge[N3 + q], gzz = Ge[2 * N3 + q], gxy = Ge[3 * N3 + q], gxz = Ge[4 * N3 + q],
                 gyz = Ge[5 * N3 + q];
          s += x1 * (gxx * x2 + gxy * y2 + gxz * z2) + y1 * (gxy * x2 + gyy * y2 + gyz * z2) + z1 * (gxz * x2 + gyz * y2 + gzz * z2);
          if (mass) s += Ge[6 * N3 + q] * (Ba * Bb * Bc) * (Ba2 * Bb2 * Bc2);
        }
      }
    }
    int dt = tdof[(size_t)e * tstride + t], du = tdof[(size_t)e * tstride + u];
    if ((dt < 0) != (du < 0)) s = -s;
    int64_t pos = find_col(rowptr, colind, dt & 0x7fffffff, du & 0x7fffffff);
    if (pos < 0) { atomicExch(bad, 1); continue; }
    red_add(vals + pos, s);
  }
}

// hex, sum-factorized element matrices (N = p+1 <= 5), one block per element.
// With X^m = D if m = x else B (likewise Y, Z), the stiffness entry is
//   K[(a,b,c),(a',b',c')] = sum_{m,n} sum_{i,j,k} G_mn(i,j,k) X^m_a(i) X^n_a'(i) Y^m_b(j) Y^n_b'(j) Z^m_c(k) Z^n_c'(k)
// (+ the mass term with all factors B and weight G_6).  Per term (m,n):
//   A[i][j][cc']  = sum_k Z^m_c(k) Z^n_c'(k) G_mn(i,j,k)            N^5 FMAs
//   C_v[i][bb'][cc'] += sum_j Y^m_b(j) Y^n_b'(j) A[i][j][cc']        N^6 FMAs
// where v = (m == x, n == x) selects one of four x-variants; then
//   K[aa'][bb'][cc'] = sum_v sum_i X^v_a(i) X^v_a'(i) C_v[i][bb'][cc']  4 N^7 FMAs
// (N = 4: ~1.2e5 FMAs per element instead of ~5e6 for the entry-by-entry sum).
__global__ void __launch_bounds__(256) hex_assemble_sf_kernel(int ne, int N, const int* __restrict__ tdof, int tstride,
                                                              const double* __restrict__ Gq, int gstride, int mass, int bdb,
                                                              const double* __restrict__ Btab,
                                                              const double* __restrict__ Dtab,
                                                              const int64_t* __restrict__ rowptr,
                                                              const int32_t* __restrict__ colind, double* vals, int* bad) {
  extern __shared__ double sfm[];
  const int N2 = N * N, N3 = N2 * N, N4 = N2 * N2, N5 = N4 * N, N6 = N3 * N3;
  double* sB = sfm;             // [q][a]
  double* sD = sB + N2;         // [q][a]
  double* sG = sD + N2;         // [7][N3] (B^T D B: [16][N3])
  double* sA = sG + (bdb ? 16 : 7) * N3;  // [i][j][c][c']
  double* sC = sA + N4;         // [4][i][b][b'][c][c']
  int* sT = (int*)(sC + 4 * N5);  // DOF row of the element
  for (int k = threadIdx.x; k < N2; k += blockDim.x) { sB[k] = Btab[k]; sD[k] = Dtab[k]; }
  for (int e = blockIdx.x; e < ne; e += gridDim.x) {
    __syncthreads();
    const double* Ge = Gq + (size_t)e * gstride;
    for (int k = threadIdx.x; k < (bdb ? 16 : (mass ? 7 : 6)) * N3; k += blockDim.x) sG[k] = Ge[k];
    for (int k = threadIdx.x; k < N3; k += blockDim.x) sT[k] = tdof[(size_t)e * tstride + k];
    for (int k = threadIdx.x; k < 4 * N5; k += blockDim.x) sC[k] = 0;
    const int nterm = bdb ? 16 : (mass ? 10 : 9);
    for (int term = 0; term < nterm; term++) {
      // term < 9: (m, n) = (term / 3, term % 3); term 9: mass.  B^T D B: (m, n) =
      // (term / 4 - 1, term % 4 - 1) with -1 the value (all factors B), weight G_term
      int m, n, gc;
      if (bdb) {
        m = term / 4 - 1;
        n = term % 4 - 1;
        gc = term;
      } else {
        m = term < 9 ? term / 3 : -1;
        n = term < 9 ? term % 3 : -1;
        gc = term == 9 ? 6 : (m == n ? m : 3 + m + n - 1);  // xy -> 3, xz -> 4, yz -> 5
      }
      const double* Zm = m == 2 ? sD : sB;
      const double* Zn = n == 2 ? sD : sB;
      const double* Ym = m == 1 ? sD : sB;
      const double* Yn = n == 1 ? sD : sB;
      const int v = (m == 0 ? 2 : 0) + (n == 0 ? 1 : 0);
      __syncthreads();  // sG / sC ready, previous term done with sA
      for (int o = threadIdx.x; o < N4; o += blockDim.x) {
        const int i = o / N3, j = (o / N2) % N, c = (o / N) % N, c2 = o % N;
        const double* g = sG + gc * N3 + (i * N + j) * N;
        double s = 0;
        for (int k = 0; k < N; k++) s += Zm[k * N + c] * Zn[k * N + c2] * g[k];
        sA[o] = s;
      }
      __syncthreads();
      double* Cv = sC + v * N5;
      for (int o = threadIdx.x; o < N5; o += blockDim.x) {
        const int i = o / N4, b = (o / N3) % N, b2 = (o / N2) % N, cc = o % N2;
        double s = 0;
        for (int j = 0; j < N; j++) s += Ym[j * N + b] * Yn[j * N + b2] * sA[(i * N + j) * N2 + cc];
        Cv[o] += s;
      }
    }
    __syncthreads();
    for (int o = threadIdx.x; o < N6; o += blockDim.x) {
      const int a = o / N5, a2 = (o / N4) % N, r = o % N4;  // r = (b, b', c, c')
      const int b = r / N3, b2 = (r / N2) % N, c = (r / N) % N, c2 = r % N;
      double s = 0;
      for (int i = 0; i < N; i++) {
        const double Ba = sB[i * N + a], Da = sD[i * N + a], Ba2 = sB[i * N + a2], Da2 = sD[i * N + a2];
        const int ci = i * N4 + r;
        s += Ba * Ba2 * sC[ci] + Ba * Da2 * sC[N5 + ci] + Da * Ba2 * sC[2 * N5 + ci] + Da * Da2 * sC[3 * N5 + ci];
      }
      const int t = (a * N + b) * N + c, u = (a2 * N + b2) * N + c2;
      const int dt = sT[t], du = sT[u];
      if ((dt < 0) != (du < 0)) s = -s;
      const int64_t pos = find_col(rowptr, colind, dt & 0x7fffffff, du & 0x7fffffff);
      if (pos < 0) { atomicExch(bad, 1); continue; }
      red_add(vals + pos, s);
    }
  }
}

static size_t hex_assemble_sf_smem(int N, bool bdb) {
  const size_t N2 = N * N, N3 = N2 * N, N4 = N2 * N2, N5 = N4 * N;
  return (2 * N2 + (bdb ? 16 : 7) * N3 + N4 + 4 * N5) * sizeof(double) + N3 * sizeof(int);
}

void assemble_csr(gh1_form* f, double* vals) {
  gh1_space* sp = f->sp;
  gh1_ctx* ctx = sp->ctx;
  cudaStream_t s = ctx->stream;
  // geometry (G, M) in FP64 through a temporary matrix-free operator
  gh1_op geo;
  geo.ctx = ctx; geo.kind = GH1_OP_MATFREE; geo.form = f; geo.sp = sp; geo.nrows = sp->ndof; geo.prec_mask = 1;
  geo.bdb_points_only = true;  // B^T D B on hexes: matrices per point, the layout the kernels read
  matfree_setup(&geo);
  const int bdb = geo.bdb ? 1 : 0;
  GH1_CUDA(cudaMemsetAsync(vals, 0, sp->nnz * sizeof(double), s));
  DBuf<int> bad(1);
  bad.zero(s);
  const int ne = sp->mesh->ne;
  if (sp->et == 4 && bdb) {
    tet_bdb_assemble(&geo, sp->d_rowptr.p, sp->d_colind.p, vals, bad.p);
  } else if (sp->et == 4) {
    int64_t tot = (int64_t)ne * sp->nloc * sp->nloc;
    int grid = (int)std::min<int64_t>((tot + 255) / 256, (int64_t)ctx->nsm * 32);
    tet_assemble_kernel<<<grid, 256, 0, s>>>(ne, sp->nloc, sp->d_eldofs.p, sp->d_class.p, geo.d_G64.p,
                                             geo.has_mass ? geo.d_M64.p : nullptr, sp->d_S.p, sp->d_rowptr.p,
                                             sp->d_colind.p, vals, bad.p);
    check_kernel(ctx, "tet_assemble_kernel");
  } else if (sp->p + 1 <= 5 && !getenv("GH1_HEX_ASSEMBLE_ENTRYWISE")) {
    const int N = sp->p + 1;
    const size_t smem = hex_assemble_sf_smem(N, bdb);
    static bool attr = false;
    if (!attr) {
      GH1_CUDA(cudaFuncSetAttribute(hex_assemble_sf_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024));
      attr = true;
    }
    const int grid = std::max(1, std::min(ne, ctx->nsm * 8));
    hex_assemble_sf_kernel<<<grid, 256, smem, s>>>(ne, N, sp->d_tdof.p, sp->tstride, geo.d_G64.p, geo.gstride64,
                                                   geo.has_mass ? 1 : 0, bdb, sp->d_B64.p, sp->d_D64.p, sp->d_rowptr.p,
                                                   sp->d_colind.p, vals, bad.p);
    check_kernel(ctx, "hex_assemble_sf_kernel");
  } else {
    const int N = sp->p + 1;
    int64_t tot = (int64_t)ne * N * N * N * N * N * N;
    int grid = (int)std::min<int64_t>((tot + 255) / 256, (int64_t)ctx->nsm * 32);
    hex_assemble_kernel<<<grid, 256, 0, s>>>(ne, N, sp->d_tdof.p, sp->tstride, geo.d_G64.p, geo.gstride64,
                                             geo.has_mass ? 1 : 0, bdb, sp->d_B64.p, sp->d_D64.p, sp->d_rowptr.p, sp->d_colind.p,
                                             vals, bad.p);
    check_kernel(ctx, "hex_assemble_kernel");
  }
  int hbad = 0;
  GH1_CUDA(cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  GH1_CUDA(cudaStreamSynchronize(s));
  GH1_CHECK(!hbad, GH1_ERR_ILLEGAL_DNUMS, "SparseMatrix AddElementMatrix: illegal dnums");
}

// ---- LinearForm f*v, f piecewise constant ---------------------------------------
__global__ void hex_wdet_kernel(int ne, int nq1, const double* __restrict__ X, const int* __restrict__ el,
                                const double* __restrict__ gx, const double* __restrict__ gw, double* wdet,
                                DeformView dv) {
  const int nq = nq1 * nq1 * nq1;
  int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= (int64_t)ne * nq) return;
  int e = (int)(id / nq), q = (int)(id % nq);
  int i = q / (nq1 * nq1), j = (q / nq1) % nq1, k = q % nq1;
  double x = gx[i], y = gx[j], z = gx[k];
  const double dl[8][3] = {
      {-(1 - y) * (1 - z), -(1 - x) * (1 - z), -(1 - x) * (1 - y)}, {(1 - y) * (1 - z), -x * (1 - z), -x * (1 - y)},
      {y * (1 - z), x * (1 - z), -x * y},                           {-y * (1 - z), (1 - x) * (1 - z), -(1 - x) * y},
      {-(1 - y) * z, -(1 - x) * z, (1 - x) * (1 - y)},             {(1 - y) * z, -x * z, x * (1 - y)},
      {y * z, x * z, x * y},                                        {-y * z, (1 - x) * z, (1 - x) * y}};
  double J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int a = 0; a < 8; a++) {
    const double* pa = X + 3 * (size_t)el[(size_t)e * 8 + a];
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 3; c++) J[3 * r + c] += pa[r] * dl[a][c];
  }
  deform_add(dv, e, x, y, z, J, nullptr);
  double det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) + J[2] * (J[3] * J[7] - J[4] * J[6]);
  wdet[id] = gw[i] * gw[j] * gw[k] * fabs(det);
}

// b(a,b,c) += f_e sum_i B(i,a) sum_j B(j,b) sum_k B(k,c) wdet(i,j,k): one block per element
__global__ void __launch_bounds__(128) hex_rhs_kernel(int ne, int N, const int* __restrict__ tdof, int tstride,
                                                       const double* __restrict__ wdet, const double* __restrict__ B,
                                                       const double* __restrict__ f, double* b) {
  extern __shared__ double rsm[];
  const int N2 = N * N, N3 = N2 * N;
  double* u = rsm;
  double* v = rsm + N3;
  for (int e = blockIdx.x; e < ne; e += gridDim.x) {
    for (int t = threadIdx.x; t < N3; t += blockDim.x) u[t] = wdet[(size_t)e * N3 + t];
    __syncthreads();
    for (int t = threadIdx.x; t < N3; t += blockDim.x) {  // contract k -> c
      const int ij = t / N, c = t % N;
      double s = 0;
      for (int k = 0; k < N; k++) s += B[k * N + c] * u[ij * N + k];
      v[t] = s;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < N3; t += blockDim.x) {  // contract j -> b
      const int i = t / N2, bb = (t / N) % N, c = t % N;
      double s = 0;
      for (int j = 0; j < N; j++) s += B[j * N + bb] * v[(i * N + j) * N + c];
      u[t] = s;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < N3; t += blockDim.x) {  // contract i -> a
      const int a = t / N2, bc = t % N2;
      double s = 0;
      for (int i = 0; i < N; i++) s += B[i * N + a] * u[i * N2 + bc];
      s *= f[e];
      const int d = tdof[(size_t)e * tstride + t];
      red_add(b + (d & 0x7fffffff), d < 0 ? -s : s);
    }
    __syncthreads();
  }
}

// deformed meshes: |det J| per rule point (the Jacobian gains the field's gradient)
__global__ void tet_rhs_kernel(int ne, int nloc, int nqm, const int* __restrict__ eldofs, const uint8_t* __restrict__ cls,
                               const double* __restrict__ X, const int* __restrict__ el, const double* __restrict__ tabm,
                               const double* __restrict__ rulem, const double* __restrict__ f, double* b,
                               DeformView dv) {
  int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= (int64_t)ne * nloc) return;
  int e = (int)(id / nloc), i = (int)(id % nloc);
  const int* v = el + (size_t)e * 4;
  const double* p3 = X + 3 * (size_t)v[3];
  double J[9];
  for (int j = 0; j < 3; j++)
    for (int k = 0; k < 3; k++) J[3 * k + j] = X[3 * (size_t)v[j] + k] - p3[k];
  double det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) + J[2] * (J[3] * J[7] - J[4] * J[6]);
  const double* tc = tabm + (size_t)cls[e] * nqm * nloc;
  double s = 0;
  if (dv.d) {
    for (int q = 0; q < nqm; q++) {
      double Jq[9];
      for (int c = 0; c < 9; c++) Jq[c] = J[c];
      deform_add(dv, e, rulem[4 * q], rulem[4 * q + 1], rulem[4 * q + 2], Jq, nullptr);
      const double dq = Jq[0] * (Jq[4] * Jq[8] - Jq[5] * Jq[7]) - Jq[1] * (Jq[3] * Jq[8] - Jq[5] * Jq[6]) +
                        Jq[2] * (Jq[3] * Jq[7] - Jq[4] * Jq[6]);
      s += rulem[4 * q + 3] * fabs(dq) * tc[(size_t)q * nloc + i];
    }
    red_add(b + eldofs[id], f[e] * s);
    return;
  }
  for (int q = 0; q < nqm; q++) s += rulem[4 * q + 3] * tc[(size_t)q * nloc + i];
  red_add(b + eldofs[id], f[e] * fabs(det) * s);
}

void rhs_elementwise(gh1_space* sp, const double* f, double* b) {
  gh1_ctx* ctx = sp->ctx;
  cudaStream_t s = ctx->stream;
  const int ne = sp->mesh->ne;
  GH1_CUDA(cudaMemsetAsync(b, 0, sp->ndof * sizeof(double), s));
  if (sp->et == 8) {
    const int N = sp->p + 1, nq = sp->nq1 * sp->nq1 * sp->nq1;
    DBuf<double> wdet((size_t)ne * nq);
    int64_t tot = (int64_t)ne * nq;
    hex_wdet_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(ne, sp->nq1, sp->mesh->d_X.p, sp->mesh->d_el.p, sp->d_gx.p,
                                                                   sp->d_gw.p, wdet.p, deform_view(sp->mesh));
    check_kernel(ctx, "hex_wdet_kernel");
    hex_rhs_kernel<<<std::min(ne, ctx->nsm * 16), 128, 2 * (size_t)N * N * N * sizeof(double), s>>>(
        ne, N, sp->d_tdof.p, sp->tstride, wdet.p, sp->d_B64.p, f, b);
    check_kernel(ctx, "hex_rhs_kernel");
    GH1_CUDA(cudaStreamSynchronize(s));
  } else {
    int64_t tot = (int64_t)ne * sp->nloc;
    tet_rhs_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(ne, sp->nloc, sp->tet_nq_mass, sp->d_eldofs.p, sp->d_class.p,
                                                                  sp->mesh->d_X.p, sp->mesh->d_el.p, sp->d_tabm64.p,
                                                                  sp->d_tqm.p, f, b, deform_view(sp->mesh));
    check_kernel(ctx, "tet_rhs_kernel");
  }
}

}  // namespace gh1
