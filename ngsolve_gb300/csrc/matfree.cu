// matfree.cu -- matrix-free operator  y = A x  for kappa grad.grad + mu u v.
//
// Replaces BilinearFormApplication / S_BilinearForm::AddMatrix1
// (comp/bilinearform.cpp:4668-4760, :7549-7607) with per-element
// SymbolicBFI::ApplyElementMatrix (fem/symbolicintegrator.cpp:2959-3040).
//
// Hexes: sum factorization.  Every hex shape is sign * psi_a(x) psi_b(y) psi_c(z)
// (derivation in basis.cuh), so the element gradient at the tensor Gauss points
// is three 1D contractions per component.  One thread group per element
// (N*N threads, N = p+1), lane (a,b) owning a pencil along the third index:
//   gather (signed, by the tensor DOF table) -> contract c -> transpose ->
//   contract b -> transpose -> contract a -> qp:  v = G_q grad u -> transposed
//   chain -> signed atomic scatter.
// G_q = kappa_e w_q |det J_q| J_q^{-1} J_q^{-T} (6 values per point) is built
// once in FP64 from the trilinear element map and stored in the inner
// precision (FP32 or FP64): it is the per-element coefficient tile the apply
// streams from HBM.
//
// Tets: element-wise B^T D B with per-orientation-class reference gradient
// tables (the role of the reference's JIT MatrixFreeBTDTB kernel,
// ngscuda/cuda_matrix_free_btdtb.cpp:60-310) and a per-element constant
// G_e = kappa_e |det J| J^{-1} J^{-T} (affine map, comp/meshaccess.cpp:541-552).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdlib>
#include <type_traits>
#include <vector>
#include "common.cuh"
#include "basis.cuh"
#include "hexcore.cuh"
#include "hexsf.cuh"
#include "deform.cuh"

namespace gh1 {

// ---------------------------------------------------------------------------
// geometry
// G[e*gs + c*nq + q] (c: xx yy zz xy xz yz, and mu w |det J| as c = 6 when mu
// is given) for hex elements; FP64 arithmetic, stored in FP64 and/or FP32
__global__ void hex_geom_kernel(int ne, int nq1, const double* __restrict__ X, const int* __restrict__ el,
                                const double* __restrict__ gx, const double* __restrict__ gw,
                                const double* __restrict__ kappa, const double* __restrict__ K6,
                                const double* __restrict__ mu, double* G64, int gs64, float* G32, int gs32,
                                DeformView dv, const double* __restrict__ Dpp) {
  const int nq = nq1 * nq1 * nq1;
  int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= (int64_t)ne * nq) return;
  int e = (int)(id / nq), q = (int)(id % nq);
  int i = q / (nq1 * nq1), j = (q / nq1) % nq1, k = q % nq1;
  int v[8];
  for (int a = 0; a < 8; a++) v[a] = el[(size_t)e * 8 + a];
  double J[9], Ji[9], det;
  hex_jacobian(X, v, gx[i], gx[j], gx[k], J);
  deform_add(dv, e, gx[i], gx[j], gx[k], J, nullptr);
  inv3(J, Ji, det);
  double wdet = gw[i] * gw[j] * gw[k] * fabs(det);
  double g[7];
  if (Dpp) {  // a generic form of Laplace type with D per point: K = the gradient block, mu = the value entry
    const double* d = Dpp + ((size_t)e * nq + q) * 16;
    const double K[6] = {d[5], d[10], d[15], 0.5 * (d[6] + d[9]), 0.5 * (d[7] + d[13]), 0.5 * (d[11] + d[14])};
    tensor_metric(Ji, K, wdet, g);
    g[6] = d[0] * wdet;
    const int nc = mu ? 7 : 6;
    for (int c = 0; c < nc; c++) {
      if (G64) G64[(size_t)e * gs64 + c * nq + q] = g[c];
      if (G32) G32[(size_t)e * gs32 + c * nq + q] = (float)g[c];
    }
    return;
  }
  if (K6) {
    tensor_metric(Ji, K6 + 6 * (size_t)e, wdet, g);
  } else {
    double f = kappa[e] * wdet;
    g[0] = f * (Ji[0] * Ji[0] + Ji[1] * Ji[1] + Ji[2] * Ji[2]);
    g[1] = f * (Ji[3] * Ji[3] + Ji[4] * Ji[4] + Ji[5] * Ji[5]);
    g[2] = f * (Ji[6] * Ji[6] + Ji[7] * Ji[7] + Ji[8] * Ji[8]);
    g[3] = f * (Ji[0] * Ji[3] + Ji[1] * Ji[4] + Ji[2] * Ji[5]);
    g[4] = f * (Ji[0] * Ji[6] + Ji[1] * Ji[7] + Ji[2] * Ji[8]);
    g[5] = f * (Ji[3] * Ji[6] + Ji[4] * Ji[7] + Ji[5] * Ji[8]);
  }
  const int nc = mu ? 7 : 6;
  if (mu) g[6] = mu[e] * wdet;
  for (int c = 0; c < nc; c++) {
    if (G64) G64[(size_t)e * gs64 + c * nq + q] = g[c];
    if (G32) G32[(size_t)e * gs32 + c * nq + q] = (float)g[c];
  }
}

// tet: G[e][6] = kappa |det| J^{-1} J^{-T}, M[e] = mu |det|
__global__ void tet_geom_kernel(int ne, const double* __restrict__ X, const int* __restrict__ el,
                                const double* __restrict__ kappa, const double* __restrict__ K6,
                                const double* __restrict__ mu, double* G64, float* G32, double* M64, float* M32) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int* v = el + (size_t)e * 4;
  const double* p3 = X + 3 * (size_t)v[3];
  double J[9], Ji[9], det;
  for (int j = 0; j < 3; j++) {
    const double* pj = X + 3 * (size_t)v[j];
    for (int k = 0; k < 3; k++) J[3 * k + j] = pj[k] - p3[k];
  }
  inv3(J, Ji, det);
  double g[6];
  if (K6) {
    tensor_metric(Ji, K6 + 6 * (size_t)e, fabs(det), g);
  } else {
    double f = kappa[e] * fabs(det);
    g[0] = f * (Ji[0] * Ji[0] + Ji[1] * Ji[1] + Ji[2] * Ji[2]);
    g[1] = f * (Ji[3] * Ji[3] + Ji[4] * Ji[4] + Ji[5] * Ji[5]);
    g[2] = f * (Ji[6] * Ji[6] + Ji[7] * Ji[7] + Ji[8] * Ji[8]);
    g[3] = f * (Ji[0] * Ji[3] + Ji[1] * Ji[4] + Ji[2] * Ji[5]);
    g[4] = f * (Ji[0] * Ji[6] + Ji[1] * Ji[7] + Ji[2] * Ji[8]);
    g[5] = f * (Ji[3] * Ji[6] + Ji[4] * Ji[7] + Ji[5] * Ji[8]);
  }
  for (int c = 0; c < 6; c++) {
    if (G64) G64[(size_t)e * 6 + c] = g[c];
    if (G32) G32[(size_t)e * 6 + c] = (float)g[c];
  }
  if (mu) {
    double m = mu[e] * fabs(det);
    if (M64) M64[e] = m;
    if (M32) M32[e] = (float)m;
  }
}

// Multi-right-hand-side apply for batched solves: Y_r += A X_r for the right-hand
// sides r < R with phase[r] == want (vectors stored rhs-major, stride n).
// The G tiles and DOF rows of a chunk are bulk-copied once (TMA, mbarriers) and
// reused for every active right-hand side, so the dominant G stream is read once
// per R applications.  Per-rhs energies x_r^T A x_r go to energy[r].
template <int N, class T, bool MASS>
__global__ void __launch_bounds__(HexCfg<N>::BLOCK)
hex_apply_multi_kernel(int ne, int64_t n, int R, const int* __restrict__ phase, int want, const int* __restrict__ tdof,
                       int tstride,
                       const T* __restrict__ Gq, int gstride, const T* __restrict__ x, T* __restrict__ y, int first_cell,
                       double* partial, unsigned int* counter, double* energy, int* err) {
  using C = HexCfg<N>;
  using SM = HexSmem<N, T>;
  constexpr int N2 = C::N2, N3 = C::N3, G = C::G, EPW = C::EPW, CN3 = EPW * N3;
  constexpr int RMAX = 16;
  __shared__ float sacc[C::EPB][RMAX];
  __shared__ int sact[RMAX];
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int gid = threadIdx.x / G, lane = threadIdx.x % G;
  const int slot = lane / N2, pl = lane % N2;
  const size_t rowg = round16((size_t)gstride * sizeof(T)), rowt = round16((size_t)tstride * sizeof(int));
  const size_t gb = SM::gbytes(gstride), tb = SM::tbytes(tstride);
  unsigned char* gp = smem_raw + SM::tables + (size_t)gid * SM::group(gstride, tstride, 0);
  T* gbuf = (T*)gp;
  auto tbuf = [&](int b) { return (int*)(gp + gb + b * tb); };
  T* work = (T*)(gp + gb + 2 * tb);
  const int so = slot < EPW ? slot * N3 : 0;
  T *su = work + so, *s1 = work + CN3 + so, *s2 = work + 2 * CN3 + so, *t2 = work + 3 * CN3 + so,
    *t3 = work + 4 * CN3 + so;
  uint64_t* mbar = (uint64_t*)(gp + gb + 2 * tb + SM::work);
  for (int r = threadIdx.x; r < RMAX; r += blockDim.x) sact[r] = (r < R) ? (phase[r] == want) : 0;
  for (int t = threadIdx.x; t < C::EPB * RMAX; t += blockDim.x) (&sacc[0][0])[t] = 0.f;
  if (lane == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    mbar_init(&mbar[2], 1);
    fence_mbar_init();
  }
  __syncthreads();
  int any = 0;
  for (int r = 0; r < R; r++) any |= sact[r];
  const int nch = (ne + EPW - 1) / EPW;
  const int stride = gridDim.x * C::EPB;
  int ch = blockIdx.x * C::EPB + gid;
  auto rows_of = [&](int c) { return min(EPW, ne - c * EPW); };
  auto issue = [&](int c, int b) {
    const uint32_t bt = (uint32_t)(rows_of(c) * rowt), bg = (uint32_t)(rows_of(c) * rowg);
    mbar_expect_tx(&mbar[b], bt);
    bulk_g2s(tbuf(b), tdof + (size_t)c * EPW * tstride, bt, &mbar[b]);
    mbar_expect_tx(&mbar[2], bg);
    bulk_g2s(gbuf, Gq + (size_t)c * EPW * gstride, bg, &mbar[2]);
  };
  int issued = 0, waited = 0;
  bool ok = true;
  if (any && ch < nch && lane == 0) issue(ch, 0);
  if (any && ch < nch) issued = 1;
  for (int k = 0; any && ok && ch < nch; ch += stride, k++) {
    const int b = k & 1;
    ok = group_all<G>(gid, mbar_wait_bounded(&mbar[b], (k >> 1) & 1) && mbar_wait_bounded(&mbar[2], k & 1));
    waited++;
    if (!ok) break;
    const int* td = tbuf(b);
    const int nrow = rows_of(ch);
    const bool act_el = slot < EPW && ch * EPW + slot < ne;
    const T* Ge = (const T*)((const unsigned char*)gbuf + (slot < EPW ? slot : 0) * rowg);
    for (int r = 0; r < R; r++) {
      if (!sact[r]) continue;
      const T* xr = x + (size_t)r * n;
      T* yr = y + (size_t)r * n;
      for (int t = lane; t < CN3; t += G) {
        T v = 0;
        if (t / N3 < nrow) {
          const int d = td[(t / N3) * (int)(rowt / sizeof(int)) + t % N3];
          v = __ldg(xr + (d & 0x7fffffff));
          if (d < 0) v = -v;
        }
        work[t] = v;
      }
      group_sync<G>(gid);
      T gx[N], gy[N], gz[N], uq[N];
      hex_forward<N, T, MASS>(pl, act_el, gid, su, s1, s2, t2, t3, gx, gy, gz, uq);
      T vx[N], vy[N], vz[N], vm[N];
      T en = 0;
      if (act_el) {
#pragma unroll
        for (int i = 0; i < N; i++) {
          const int o = i * N2 + pl;
          T gxx = Ge[o], gyy = Ge[N3 + o], gzz = Ge[2 * N3 + o], gxy = Ge[3 * N3 + o], gxz = Ge[4 * N3 + o],
            gyz = Ge[5 * N3 + o];
          vx[i] = gxx * gx[i] + gxy * gy[i] + gxz * gz[i];
          vy[i] = gxy * gx[i] + gyy * gy[i] + gyz * gz[i];
          vz[i] = gxz * gx[i] + gyz * gy[i] + gzz * gz[i];
          en += gx[i] * vx[i] + gy[i] * vy[i] + gz[i] * vz[i];
          if (MASS) {
            vm[i] = Ge[6 * N3 + o] * uq[i];
            en += uq[i] * vm[i];
          }
        }
      }
      // per-rhs energy: warp sum, one shared-memory add per warp
      float ef = (float)en;
      for (int o = 16; o > 0; o >>= 1) ef += __shfl_xor_sync(0xffffffffu, ef, o);
      if ((lane & 31) == 0) atomicAdd(&sacc[gid][r], ef);
      hex_backward<N, T, MASS>(pl, act_el, gid, su, s1, s2, t2, t3, vx, vy, vz, vm);
      for (int t = lane; t < CN3; t += G) {
        if (t / N3 >= nrow) continue;
        const int d = td[(t / N3) * (int)(rowt / sizeof(int)) + t % N3];
        const int dof = d & 0x7fffffff;
        const T v = d < 0 ? -work[t] : work[t];
        if (dof >= first_cell) yr[dof] = v;
        else atomic_add_t(yr + dof, v);
      }
      group_sync<G>(gid);
    }
    // all right-hand sides of this chunk are done: refill both buffers for the next chunk
    group_sync<G>(gid);
    if (lane == 0 && ch + stride < nch) {
      fence_proxy_async();
      issue(ch + stride, b ^ 1);
    }
    if (ch + stride < nch) issued++;
  }
  if (!ok) {
    if (lane == 0) {
      atomicExch(err, 1);
      for (int j = waited; j < issued; j++) {
        mbar_wait_bounded(&mbar[j & 1], (j >> 1) & 1);
        mbar_wait_bounded(&mbar[2], j & 1);
      }
    }
    group_sync<G>(gid);
  }
  // block sums per rhs -> partial[r][block]; the last block totals into energy[r]
  __syncthreads();
  __shared__ bool last;
  if (threadIdx.x < RMAX) {
    float s = 0;
    for (int g = 0; g < C::EPB; g++) s += sacc[g][threadIdx.x];
    if (threadIdx.x < R) partial[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = (double)s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last) {
    __threadfence();
    if (threadIdx.x < R && sact[threadIdx.x]) {
      double s = 0;
      for (int i = 0; i < (int)gridDim.x; i++) s += ((volatile double*)partial)[(size_t)threadIdx.x * gridDim.x + i];
      energy[threadIdx.x] = s;
    }
    if (threadIdx.x == 0) *counter = 0u;
  }
}

// element-wise  int_e grad u . grad w  (geometry from G / kappa_e)
template <int N>
__global__ void __launch_bounds__(HexCfg<N>::BLOCK)
hex_graddot_kernel(int ne, const int* __restrict__ tdof, int tstride, const double* __restrict__ Gq, int gstride,
                   const double* __restrict__ kappa, const double* __restrict__ u, const double* __restrict__ w, double* out) {
  using C = HexCfg<N>;
  using T = double;
  constexpr int N2 = C::N2, N3 = C::N3, G = C::G;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int gid = threadIdx.x / G, lane = threadIdx.x % G;
  T* base = (T*)(smem_raw + HexSmem<N, T>::tables) + (size_t)gid * 5 * N3;
  T *su = base, *s1 = base + N3, *s2 = base + 2 * N3, *t2 = base + 3 * N3, *t3 = base + 4 * N3;
  __shared__ double red[C::EPB][(C::G + 31) / 32];
  for (int e0 = blockIdx.x * C::EPB; e0 < ne; e0 += gridDim.x * C::EPB) {
    int e = e0 + gid;
    bool valid = e < ne;
    T ux[N], uy[N], uz[N], wx[N], wy[N], wz[N], dummy[N];
    for (int t = lane; t < N3; t += G) {
      int d = valid ? tdof[(size_t)e * tstride + t] : 0;
      T v = valid ? u[d & 0x7fffffff] : 0.0;
      su[t] = d < 0 ? -v : v;
    }
    group_sync<G>(gid);
    hex_forward<N, T, false>(lane, lane < N2, gid, su, s1, s2, t2, t3, ux, uy, uz, dummy);
    for (int t = lane; t < N3; t += G) {
      int d = valid ? tdof[(size_t)e * tstride + t] : 0;
      T v = valid ? w[d & 0x7fffffff] : 0.0;
      su[t] = d < 0 ? -v : v;
    }
    group_sync<G>(gid);
    hex_forward<N, T, false>(lane, lane < N2, gid, su, s1, s2, t2, t3, wx, wy, wz, dummy);
    double acc = 0;
    if (lane < N2 && valid) {
      const T* Ge = Gq + (size_t)e * gstride + lane;
      double ik = 1.0 / kappa[e];
      for (int i = 0; i < N; i++) {
        const int o = i * N2;
        T gxx = Ge[o], gyy = Ge[N3 + o], gzz = Ge[2 * N3 + o], gxy = Ge[3 * N3 + o], gxz = Ge[4 * N3 + o], gyz = Ge[5 * N3 + o];
        acc += ik * (ux[i] * (gxx * wx[i] + gxy * wy[i] + gxz * wz[i]) + uy[i] * (gxy * wx[i] + gyy * wy[i] + gyz * wz[i]) +
                     uz[i] * (gxz * wx[i] + gyz * wy[i] + gzz * wz[i]));
      }
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((lane & 31) == 0) red[gid][lane >> 5] = acc;
    group_sync<G>(gid);
    if (lane == 0 && valid) {
      double s = 0;
      for (int i = 0; i < G / 32; i++) s += red[gid][i];
      out[e] = s;
    }
    group_sync<G>(gid);
  }
}

// diagonal of the hex operator, sum-factorized: one block per element,
//   d(a,b,c) = sum_m sum_i h_m(i,a) sum_j g_m(j,b) sum_k f_m(k,c) G_m(i,j,k)
// with the per-component factor pairs (D D, B B, ...) of grad phi_t . G grad phi_t.
__global__ void __launch_bounds__(256) hex_diag_kernel(int ne, int N, const int* __restrict__ tdof, int tstride,
                                                        const double* __restrict__ Gq, int gstride, int mass,
                                                        const double* __restrict__ B, const double* __restrict__ D,
                                                        double* diag) {
  extern __shared__ double dsm[];
  const int N2 = N * N, N3 = N2 * N, nc = mass ? 7 : 6;
  double* g = dsm;             // nc * N3: G, then H, then K (in place per stage via ping-pong)
  double* h = dsm + 7 * N3;    // nc * N3
  // factor selectors per component m: 0 = B*B, 1 = D*D, 2 = B*D ; weights of the i-stage
  // m:        xx   yy   zz   xy   xz   yz   mass
  const int fk[7] = {0, 0, 1, 0, 2, 2, 0};  // k-factor (c index)
  const int fj[7] = {0, 1, 0, 2, 0, 2, 0};  // j-factor (b index)
  const int fi[7] = {1, 0, 0, 2, 2, 0, 0};  // i-factor (a index)
  const double wi[7] = {1, 1, 1, 2, 2, 2, 1};
  auto fac = [&](int sel, int q, int a) {
    const double b = B[q * N + a], d = D[q * N + a];
    return sel == 0 ? b * b : (sel == 1 ? d * d : b * d);
  };
  for (int e = blockIdx.x; e < ne; e += gridDim.x) {
    const double* Ge = Gq + (size_t)e * gstride;
    for (int t = threadIdx.x; t < nc * N3; t += blockDim.x) g[t] = Ge[t];
    __syncthreads();
    // contract k: h[m][i][j][c] = sum_k f_m(k,c) g[m][i][j][k]
    for (int t = threadIdx.x; t < nc * N3; t += blockDim.x) {
      const int m = t / N3, r = t % N3, ij = r / N, c = r % N;
      double v = 0;
      for (int k = 0; k < N; k++) v += fac(fk[m], k, c) * g[m * N3 + ij * N + k];
      h[t] = v;
    }
    __syncthreads();
    // contract j: g[m][i][b][c] = sum_j g_m(j,b) h[m][i][j][c]
    for (int t = threadIdx.x; t < nc * N3; t += blockDim.x) {
      const int m = t / N3, r = t % N3, i = r / N2, b = (r / N) % N, c = r % N;
      double v = 0;
      for (int j = 0; j < N; j++) v += fac(fj[m], j, b) * h[m * N3 + (i * N + j) * N + c];
      g[t] = v;
    }
    __syncthreads();
    // contract i and sum the components
    for (int t = threadIdx.x; t < N3; t += blockDim.x) {
      const int a = t / N2, bc = t % N2;
      double v = 0;
      for (int m = 0; m < nc; m++)
        for (int i = 0; i < N; i++) v += wi[m] * fac(fi[m], i, a) * g[m * N3 + i * N2 + bc];
      red_add(diag + (tdof[(size_t)e * tstride + t] & 0x7fffffff), v);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// tets: one warp per element
template <class T, bool MASS>
__global__ void __launch_bounds__(256)
tet_apply_kernel(int ne, int nloc, int nq, int nqm, const int* __restrict__ eldofs, const uint8_t* __restrict__ cls,
                 const T* __restrict__ Ge, const T* __restrict__ Me, const T* __restrict__ tab, const double* __restrict__ rule,
                 const double* __restrict__ tabm, const double* __restrict__ rulem, const T* __restrict__ x,
                 T* __restrict__ y, double* partial, unsigned int* counter, double* energy, const int* skip) {
  if (skip && *(volatile const int*)skip) return;
  constexpr int WPB = 8;
  __shared__ T sx[WPB][96];
  __shared__ T sv[WPB][4 * 128];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T acc = 0;
  for (int e = blockIdx.x * WPB + w; e < ne; e += gridDim.x * WPB) {
    const int* dn = eldofs + (size_t)e * nloc;
    for (int i = lane; i < nloc; i += 32) sx[w][i] = x[dn[i]];
    __syncwarp();
    const int c = cls[e];
    const T* tc = tab + (size_t)c * nq * nloc * 4;
    T g0 = Ge[(size_t)e * 6 + 0], g1 = Ge[(size_t)e * 6 + 1], g2 = Ge[(size_t)e * 6 + 2];
    T g3 = Ge[(size_t)e * 6 + 3], g4 = Ge[(size_t)e * 6 + 4], g5 = Ge[(size_t)e * 6 + 5];
    for (int q = lane; q < nq; q += 32) {
      T ux = 0, uy = 0, uz = 0;
      const T* tq = tc + (size_t)q * nloc * 4;
      for (int i = 0; i < nloc; i++) {
        T xi = sx[w][i];
        ux += tq[4 * i + 1] * xi; uy += tq[4 * i + 2] * xi; uz += tq[4 * i + 3] * xi;
      }
      T wq = (T)rule[4 * q + 3];
      T vx = wq * (g0 * ux + g3 * uy + g4 * uz);
      T vy = wq * (g3 * ux + g1 * uy + g5 * uz);
      T vz = wq * (g4 * ux + g5 * uy + g2 * uz);
      acc += ux * vx + uy * vy + uz * vz;
      sv[w][4 * q + 0] = vx; sv[w][4 * q + 1] = vy; sv[w][4 * q + 2] = vz;
    }
    if (MASS) {
      // mass at the order-2p rule, FP64 values table (small element counts only)
      const double* tm = tabm + (size_t)c * nqm * nloc;
      T m = Me[e];
      for (int q = lane; q < nqm && q < 128; q += 32) {
        double u = 0;
        for (int i = 0; i < nloc; i++) u += tm[(size_t)q * nloc + i] * (double)sx[w][i];
        double vm = (double)m * rulem[4 * q + 3] * u;
        acc += (T)(u * vm);
        sv[w][4 * q + 3] = (T)vm;
      }
    }
    __syncwarp();
    for (int i = lane; i < nloc; i += 32) {
      T r = 0;
      for (int q = 0; q < nq; q++) {
        const T* t = tc + ((size_t)q * nloc + i) * 4;
        r += t[1] * sv[w][4 * q] + t[2] * sv[w][4 * q + 1] + t[3] * sv[w][4 * q + 2];
      }
      if (MASS) {
        const double* tm = tabm + (size_t)c * nqm * nloc;
        for (int q = 0; q < nqm && q < 128; q++) r += (T)(tm[(size_t)q * nloc + i] * (double)sv[w][4 * q + 3]);
      }
      red_add(y + dn[i], r);
    }
    __syncwarp();
  }
  double accd = (double)acc;
  for (int o = 16; o > 0; o >>= 1) accd += __shfl_xor_sync(0xffffffffu, accd, o);
  if (partial) block_reduce_finish(lane == 0 ? accd : 0.0, partial, counter, energy);
}

__global__ void tet_diag_kernel(int ne, int nloc, const int* __restrict__ eldofs, const uint8_t* __restrict__ cls,
                                const double* __restrict__ Ge, const double* __restrict__ Me, const double* __restrict__ S,
                                double* diag) {
  int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= (int64_t)ne * nloc) return;
  int e = (int)(id / nloc), i = (int)(id % nloc);
  const double* Sc = S + (size_t)cls[e] * 7 * nloc * nloc;
  double s = 0;
  for (int b = 0; b < 6; b++) s += Ge[(size_t)e * 6 + b] * Sc[((size_t)b * nloc + i) * nloc + i];
  if (Me) s += Me[e] * Sc[((size_t)6 * nloc + i) * nloc + i];
  red_add(diag + eldofs[id], s);
}

__global__ void tet_graddot_kernel(int ne, int nloc, int nq, const int* __restrict__ eldofs, const uint8_t* __restrict__ cls,
                                   const double* __restrict__ Ge, const double* __restrict__ kappa,
                                   const double* __restrict__ tab, const double* __restrict__ rule,
                                   const double* __restrict__ u, const double* __restrict__ w, double* out) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int* dn = eldofs + (size_t)e * nloc;
  const double* tc = tab + (size_t)cls[e] * nq * nloc * 4;
  const double* g = Ge + (size_t)e * 6;
  double acc = 0;
  for (int q = 0; q < nq; q++) {
    double a[3] = {0, 0, 0}, b[3] = {0, 0, 0};
    for (int i = 0; i < nloc; i++) {
      const double* t = tc + ((size_t)q * nloc + i) * 4;
      double ui = u[dn[i]], wi = w[dn[i]];
      for (int k = 0; k < 3; k++) { a[k] += t[1 + k] * ui; b[k] += t[1 + k] * wi; }
    }
    acc += rule[4 * q + 3] * (a[0] * (g[0] * b[0] + g[3] * b[1] + g[4] * b[2]) + a[1] * (g[3] * b[0] + g[1] * b[1] + g[5] * b[2]) +
                              a[2] * (g[4] * b[0] + g[5] * b[1] + g[2] * b[2]));
  }
  out[e] = acc / kappa[e];
}

#define GH1_HEX_SWITCH(N, CASE)                                                                        \
  switch (N) {                                                                                         \
    CASE(2) CASE(3) CASE(4) CASE(5) CASE(6) CASE(7) CASE(8) CASE(9)                                   \
    default: throw Error(GH1_ERR_UNSUPPORTED, "hex order out of range");                              \
  }

template <class T, int GM>
void hex_apply_dispatch_gm(gh1_op* op, const T* x, T* y, const T* G, int gstride, double* partial,
                           unsigned int* counter, double* energy, const int* skip) {
  const bool mass = op->has_mass;
#define GH1_HEX_CASE(NN)                                                                                      \
  case NN:                                                                                                    \
    if (mass) launch_hex_apply<NN, T, true, GM>(op, x, y, G, gstride, partial, counter, energy, skip);       \
    else launch_hex_apply<NN, T, false, GM>(op, x, y, G, gstride, partial, counter, energy, skip);           \
    break;
  GH1_HEX_SWITCH(op->sp->p + 1, GH1_HEX_CASE)
#undef GH1_HEX_CASE
}

template <class T>
void hex_apply_dispatch(gh1_op* op, const T* x, T* y, const T* G, int gstride, double* partial, unsigned int* counter,
                        double* energy, const int* skip) {
  const int pi = std::is_same<T, float>::value ? 1 : 0;
  const int gm = op->hex_gmode[pi];
  if constexpr (std::is_same<T, float>::value) {
    if (gm == 6) {
      hex_tc_apply(op, x, y, partial, counter, energy, skip);
      return;
    }
    if (gm == 5) {
      hex_slice_apply(op, x, y, partial, counter, energy, skip);
      return;
    }
    if (gm >= 2) {
      hex_pair_apply(op, gm - 2, x, y, partial, counter, energy, skip);
      return;
    }
  }
  if (gm == 0) hex_apply_dispatch_gm<T, 0>(op, x, y, G, gstride, partial, counter, energy, skip);
  else hex_apply_dispatch_gm<T, 1>(op, x, y, G, gstride, partial, counter, energy, skip);
}

template <class T, int GM>
int hex_occupancy_dispatch(gh1_op* op, int gstride) {
  const bool mass = op->has_mass;
  const int tstride = op->sp->tstride;
  int v = 0;
#define GH1_OCC_CASE(NN)                                                                                        \
  case NN:                                                                                                      \
    v = mass ? hex_apply_occupancy<NN, T, true, GM>(HexSmem<NN, T>::total(gstride, tstride, GM))               \
             : hex_apply_occupancy<NN, T, false, GM>(HexSmem<NN, T>::total(gstride, tstride, GM));             \
    break;
  GH1_HEX_SWITCH(op->sp->p + 1, GH1_OCC_CASE)
#undef GH1_OCC_CASE
  return v;
}

// Autotuner: times each variant -- G tile staged in shared memory by TMA vs
// direct coalesced loads, for FP32 each of those with two elements per lane, the
// per-element-metric and slice forms on affine meshes, and the tensor-core form
// -- on this operator's own mesh and keeps the fastest.  The choice is cached per
// (order, precision, element-count bucket, affine mesh) for the process.
// GH1_HEX_GMODE=0..6 forces a variant (FP64 takes it modulo 2; a variant this
// operator does not provide falls back to its number modulo 2).
template <class T>
void hex_autotune(gh1_op* op, const T* G, int gstride) {
  const int pi = std::is_same<T, float>::value ? 1 : 0;
  std::vector<int> modes = {0, 1};
  if (pi == 1) {
    if (op->pair_per_sm[0] > 0 && op->pair_per_sm[1] > 0) {
      modes.push_back(2);
      modes.push_back(3);
      if (op->pair_per_sm[2] > 0) modes.push_back(4);
      if (op->pair_per_sm[2] > 0 && op->slice_per_sm > 0) modes.push_back(5);
    }
    if (op->tc_per_sm > 0) modes.push_back(6);
  }
  const char* env = getenv("GH1_HEX_GMODE");
  if (env && env[0] >= '0' && env[0] <= '6') {
    const int m = env[0] - '0';
    op->hex_gmode[pi] = std::find(modes.begin(), modes.end(), m) != modes.end() ? m : m % 2;
    return;
  }
  static std::vector<std::array<int, 4>> cache;  // N, precision, log2(ne), choice
  const int N = op->sp->p + 1, ne = op->sp->mesh->ne;
  int lb = 0;
  while ((1 << (lb + 1)) <= ne) lb++;
  const int key = lb + (op->has_mass ? 100 : 0) + (op->all_affine ? 1000 : 0);  // mesh-size bucket, mass, affine
  for (auto& c : cache)
    if (c[0] == N && c[1] == pi && c[2] == key && std::find(modes.begin(), modes.end(), c[3]) != modes.end()) {
      op->hex_gmode[pi] = c[3];
      return;
    }
  if (ne < 4096) {  // small meshes: no measurable difference, skip the timing
    op->hex_gmode[pi] = 0;
    return;
  }
  cudaStream_t s = op->sp->ctx->stream;
  DBuf<T> xs(op->nrows), ys(op->nrows);
  xs.zero(s);
  cudaEvent_t a, b;
  GH1_CUDA(cudaEventCreate(&a));
  GH1_CUDA(cudaEventCreate(&b));
  float best = 1e30f;
  int choice = 0;
  for (int gm : modes) {
    op->hex_gmode[pi] = gm;
    for (int r = 0; r < 2; r++) hex_apply_dispatch<T>(op, xs.p, ys.p, G, gstride, nullptr, nullptr, nullptr, nullptr);
    GH1_CUDA(cudaEventRecord(a, s));
    for (int r = 0; r < 3; r++) hex_apply_dispatch<T>(op, xs.p, ys.p, G, gstride, nullptr, nullptr, nullptr, nullptr);
    GH1_CUDA(cudaEventRecord(b, s));
    GH1_CUDA(cudaEventSynchronize(b));
    float ms = 0;
    GH1_CUDA(cudaEventElapsedTime(&ms, a, b));
    if (ms < best) { best = ms; choice = gm; }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  op->hex_gmode[pi] = choice;
  cache.push_back({N, pi, key, choice});
}

// ---- multi-right-hand-side apply (batched solves) ----------------------------
template <int N, class T, bool MASS>
int hex_multi_occupancy(size_t smem) {
  static bool attr = false;
  auto kern = hex_apply_multi_kernel<N, T, MASS>;
  if (!attr) {
    int dev = 0, optin = 0;
    GH1_CUDA(cudaGetDevice(&dev));
    GH1_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    cudaFuncAttributes fa;
    GH1_CUDA(cudaFuncGetAttributes(&fa, kern));
    GH1_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes));
    attr = true;
  }
  int v = 0;
  GH1_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kern, HexCfg<N>::BLOCK, smem));
  GH1_CHECK(v >= 1, GH1_ERR_UNSUPPORTED, "multi-rhs hex apply does not fit on an SM");
  return v;
}

template <int N, class T, bool MASS>
int hex_multi_launch(gh1_op* op, int R, const int* phase, int want, const T* x, T* y, double* partial,
                     unsigned int* counter, double* energy, bool prepare_only) {
  using C = HexCfg<N>;
  gh1_space* sp = op->sp;
  if constexpr (std::is_same<T, float>::value) {
    // FP32: two right-hand sides per lane or one, as timed for this operator
    // (GH1_MULTI_PAIR=0 / 1 forces one / two per lane)
    const char* env = getenv("GH1_MULTI_PAIR");
    const bool paired = env && (env[0] == '0' || env[0] == '1') ? env[0] == '1' : op->multi_pair != 0;
    if (paired && hex_pair_supported(N))
      return hex_multi_pair_launch(op, R, phase, want, x, y, partial, counter, energy, prepare_only);
  }
  const int gs = std::is_same<T, float>::value ? op->gstride32 : op->gstride64;
  const T* G = std::is_same<T, float>::value ? (const T*)op->d_G32.p : (const T*)op->d_G64.p;
  const size_t smem = HexSmem<N, T>::total(gs, sp->tstride, 0);
  const int pi = std::is_same<T, float>::value ? 1 : 0;
  if (prepare_only || op->multi_per_sm[pi] <= 0) op->multi_per_sm[pi] = hex_multi_occupancy<N, T, MASS>(smem);
  const int ne = sp->mesh->ne, nch = (ne + C::EPW - 1) / C::EPW;
  const int grid = std::min((nch + C::EPB - 1) / C::EPB, sp->ctx->nsm * op->multi_per_sm[pi]);
  if (prepare_only) return grid;
  hex_apply_multi_kernel<N, T, MASS><<<grid, C::BLOCK, smem, sp->ctx->stream>>>(
      ne, op->nrows, R, phase, want, sp->d_tdof.p, sp->tstride, G, gs, x, y, (int)sp->first_cell, partial, counter, energy,
      op->d_err.p);
  check_kernel(sp->ctx, "hex_apply_multi_kernel");
  return grid;
}

// y_r += A x_r for rhs with phase[r] == want; energies into energy[r].  Returns the
// grid size (partial must hold R * grid doubles).  prepare_only: set up occupancy
// (call before any stream capture) and return the grid without launching.
int matfree_apply_multi(gh1_op* op, int R, const int* phase, int want, const void* x, void* y, int prec, double* partial,
                        unsigned int* counter, double* energy, bool prepare_only) {
  GH1_CHECK(op->sp->et == 8, GH1_ERR_UNSUPPORTED, "batched solves need hex meshes");
  GH1_CHECK(R >= 1 && R <= 16, GH1_ERR_UNSUPPORTED, "batched solves take 1..16 right-hand sides per problem");
  const bool mass = op->has_mass;
  int g = 0;
#define GH1_MULTI_CASE(NN)                                                                                          \
  case NN:                                                                                                          \
    if (prec == GH1_F64)                                                                                            \
      g = mass ? hex_multi_launch<NN, double, true>(op, R, phase, want, (const double*)x, (double*)y, partial,      \
                                                    counter, energy, prepare_only)                                  \
               : hex_multi_launch<NN, double, false>(op, R, phase, want, (const double*)x, (double*)y, partial,     \
                                                     counter, energy, prepare_only);                                \
    else                                                                                                            \
      g = mass ? hex_multi_launch<NN, float, true>(op, R, phase, want, (const float*)x, (float*)y, partial, counter, \
                                                   energy, prepare_only)                                            \
               : hex_multi_launch<NN, float, false>(op, R, phase, want, (const float*)x, (float*)y, partial, counter, \
                                                    energy, prepare_only);                                          \
    break;
  GH1_HEX_SWITCH(op->sp->p + 1, GH1_MULTI_CASE)
#undef GH1_MULTI_CASE
  return g;
}

static int pad16(int count, int elem_bytes) {
  const int per = 16 / elem_bytes;
  return (count + per - 1) / per * per;
}

void matfree_setup(gh1_op* op) {
  gh1_space* sp = op->sp;
  gh1_form* f = op->form;
  cudaStream_t s = sp->ctx->stream;
  const int ne = sp->mesh->ne;
  const bool want32 = (op->prec_mask & 2) != 0;  // FP64 data always exists: diagonal, adjoint, refinement
  if (op->d_err.n == 0) {
    op->d_err.alloc(1);
    op->d_err.zero(s);
  }
  op->bdb = 0;
  // generic B^T D B form (bdb.cu); on a deformed tet mesh every form goes this
  // way, its metrics per rule point (the tet kernels assume affine elements)
  // (a hex form of Laplace type takes the standard kernels with its coefficients)
  const bool lap = bdb_laplace_route(op);
  if ((f->bdb_mode && !lap) || (sp->et == 4 && sp->mesh->def_space)) {
    bdb_setup(op);
    return;
  }
  if (!lap) op->has_mass = f->has_mu;
  if (sp->et == 8) {
    // coefficients: the form's, or those of a generic form of Laplace type
    const double* kap = f->d_kappa.p;
    const double* K6 = lap ? op->d_ovK6.p : (f->has_K6 ? f->d_K6.p : nullptr);
    const double* mu = !op->has_mass ? nullptr : (lap ? op->d_ovmu.p : f->d_mu.p);
    const int nq = sp->nq1 * sp->nq1 * sp->nq1;
    op->ncomp = op->has_mass ? 7 : 6;
    op->gstride64 = pad16(op->ncomp * nq, 8);
    op->gstride32 = pad16(op->ncomp * nq, 4);
    op->d_G64.alloc((size_t)ne * op->gstride64);
    if (want32) op->d_G32.alloc((size_t)ne * op->gstride32); else op->d_G32.release();
    int64_t tot = (int64_t)ne * nq;
    hex_geom_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(
        ne, sp->nq1, sp->mesh->d_X.p, sp->mesh->d_el.p, sp->d_gx.p, sp->d_gw.p, kap, K6,
        op->lap_pp ? (op->has_mass ? op->lap_pp : nullptr) : mu, op->d_G64.p, op->gstride64,
        want32 ? op->d_G32.p : nullptr, op->gstride32, deform_view(sp->mesh), op->lap_pp);
    check_kernel(sp->ctx, "hex_geom_kernel");
    upload_const_tables(sp);
    op->hex_per_sm[0][0] = hex_occupancy_dispatch<double, 0>(op, op->gstride64);
    op->hex_per_sm[0][1] = hex_occupancy_dispatch<double, 1>(op, op->gstride64);
    if (want32) {
      op->hex_per_sm[1][0] = hex_occupancy_dispatch<float, 0>(op, op->gstride32);
      op->hex_per_sm[1][1] = hex_occupancy_dispatch<float, 1>(op, op->gstride32);
      if (hex_pair_supported(sp->p + 1)) {
        set_first_wait_polls();
        upload_pair_tables(sp);
        op->pair_per_sm[0] = hex_pair_occupancy(op, 0);
        op->pair_per_sm[1] = hex_pair_occupancy(op, 1);
        hex_affine_setup(op);
        op->pair_per_sm[2] = op->all_affine ? hex_pair_occupancy(op, 2) : 0;
        hex_slice_setup(op);
      }
      op->tc_per_sm = hex_tc_occupancy(op);
    }
    hex_autotune<double>(op, op->d_G64.p, op->gstride64);
    if (want32) hex_autotune<float>(op, op->d_G32.p, op->gstride32);
  } else {
    op->d_G64.alloc((size_t)ne * 6);
    if (want32) op->d_G32.alloc((size_t)ne * 6); else op->d_G32.release();
    if (op->has_mass) {
      op->d_M64.alloc(ne);
      if (want32) op->d_M32.alloc(ne);
    }
    tet_geom_kernel<<<(ne + 255) / 256, 256, 0, s>>>(ne, sp->mesh->d_X.p, sp->mesh->d_el.p, f->d_kappa.p,
                                                      f->has_K6 ? f->d_K6.p : nullptr, op->has_mass ? f->d_mu.p : nullptr, op->d_G64.p,
                                                      want32 ? op->d_G32.p : nullptr, op->has_mass ? op->d_M64.p : nullptr,
                                                      (op->has_mass && want32) ? op->d_M32.p : nullptr);
    check_kernel(sp->ctx, "tet_geom_kernel");
    tet_tiles_setup(op);
  }
  op->form_version = f->version;
  op->have_diag = false;
}

template <class T>
void tet_apply_launch(gh1_op* op, const T* x, T* y, const T* G, const T* M, const T* tab, double* partial,
                      unsigned int* counter, double* energy, const int* skip) {
  gh1_space* sp = op->sp;
  const int ne = sp->mesh->ne;
  GH1_CHECK(sp->nloc <= 96 && sp->tet_nq <= 128, GH1_ERR_UNSUPPORTED, "tet order too high for the matrix-free kernel");
  int grid = std::max(1, std::min((ne + 7) / 8, sp->ctx->nsm * 8));
  if (M)
    tet_apply_kernel<T, true><<<grid, 256, 0, sp->ctx->stream>>>(ne, sp->nloc, sp->tet_nq, sp->tet_nq_mass, sp->d_eldofs.p,
                                                                 sp->d_class.p, G, M, tab, sp->d_tq.p, sp->d_tabm64.p,
                                                                 sp->d_tqm.p, x, y, partial, counter, energy, skip);
  else
    tet_apply_kernel<T, false><<<grid, 256, 0, sp->ctx->stream>>>(ne, sp->nloc, sp->tet_nq, sp->tet_nq_mass, sp->d_eldofs.p,
                                                                  sp->d_class.p, G, M, tab, sp->d_tq.p, sp->d_tabm64.p,
                                                                  sp->d_tqm.p, x, y, partial, counter, energy, skip);
  check_kernel(sp->ctx, "tet_apply_kernel");
}

void matfree_apply_ex(gh1_op* op, const void* x, void* y, int prec, double* partial, unsigned int* counter,
                      double* energy, const int* skip) {
  gh1_space* sp = op->sp;
  if (op->bdb) {
    bdb_apply(op, x, y, prec, partial, counter, energy, skip);
    return;
  }
  if (sp->et == 8) {
    if (prec == GH1_F64)
      hex_apply_dispatch<double>(op, (const double*)x, (double*)y, op->d_G64.p, op->gstride64, partial, counter, energy,
                                 skip);
    else
      hex_apply_dispatch<float>(op, (const float*)x, (float*)y, op->d_G32.p, op->gstride32, partial, counter, energy,
                                skip);
  } else {
    if (tet_tiles_apply(op, prec, x, y, partial, counter, energy, skip)) return;
    GH1_CHECK(sp->tet_nq_mass <= 128 || !op->has_mass, GH1_ERR_UNSUPPORTED, "tet mass rule too large");
    if (prec == GH1_F64)
      tet_apply_launch<double>(op, (const double*)x, (double*)y, op->d_G64.p, op->has_mass ? op->d_M64.p : nullptr,
                               sp->d_tab64.p, partial, counter, energy, skip);
    else
      tet_apply_launch<float>(op, (const float*)x, (float*)y, op->d_G32.p, op->has_mass ? op->d_M32.p : nullptr,
                              sp->d_tab32.p, partial, counter, energy, skip);
  }
}

void matfree_apply(gh1_op* op, const void* x, void* y, int prec, double* partial, unsigned int* counter, double* energy) {
  matfree_apply_ex(op, x, y, prec, partial, counter, energy, nullptr);
}

void matfree_diag(gh1_op* op, double* diag) {
  gh1_space* sp = op->sp;
  cudaStream_t s = sp->ctx->stream;
  GH1_CUDA(cudaMemsetAsync(diag, 0, sp->ndof * sizeof(double), s));
  if (op->bdb) {
    bdb_diag(op, diag);
    return;
  }
  const int ne = sp->mesh->ne;
  if (sp->et == 8) {
    const int N = sp->p + 1;
    const size_t smem = (size_t)14 * N * N * N * sizeof(double);
    if (smem > 48 * 1024)
      GH1_CUDA(cudaFuncSetAttribute(hex_diag_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int grid = std::min(ne, sp->ctx->nsm * 8);
    hex_diag_kernel<<<grid, 256, smem, s>>>(ne, N, sp->d_tdof.p, sp->tstride, op->d_G64.p, op->gstride64,
                                            op->has_mass ? 1 : 0, sp->d_B64.p, sp->d_D64.p, diag);
    check_kernel(sp->ctx, "hex_diag_kernel");
  } else {
    int64_t tot = (int64_t)ne * sp->nloc;
    tet_diag_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(ne, sp->nloc, sp->d_eldofs.p, sp->d_class.p, op->d_G64.p,
                                                                   op->has_mass ? op->d_M64.p : nullptr, sp->d_S.p, diag);
    check_kernel(sp->ctx, "tet_diag_kernel");
  }
}

template <int N>
void launch_hex_graddot(gh1_op* op, const double* u, const double* w, double* out) {
  using C = HexCfg<N>;
  gh1_space* sp = op->sp;
  const size_t smem = HexSmem<N, double>::tables + (size_t)C::EPB * HexSmem<N, double>::work;
  static bool attr_set = false;
  if (!attr_set) {
    GH1_CUDA(cudaFuncSetAttribute(hex_graddot_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set = true;
  }
  int ne = sp->mesh->ne;
  int grid = std::max(1, std::min((ne + C::EPB - 1) / C::EPB, sp->ctx->nsm * 16));
  hex_graddot_kernel<N><<<grid, C::BLOCK, smem, sp->ctx->stream>>>(ne, sp->d_tdof.p, sp->tstride, op->d_G64.p,
                                                                    op->gstride64, op->form->d_kappa.p, u, w, out);
  check_kernel(sp->ctx, "hex_graddot_kernel");
}

void elem_grad_dot(gh1_space* sp, const double* u, const double* w, double* out) {
  // geometry of a unit-coefficient form
  gh1_form f;
  f.sp = sp;
  std::vector<double> ones(sp->mesh->ne, 1.0);
  f.d_kappa.upload(ones, sp->ctx->stream);
  gh1_op op;
  op.ctx = sp->ctx; op.kind = GH1_OP_MATFREE; op.form = &f; op.sp = sp; op.nrows = sp->ndof; op.prec_mask = 1;
  matfree_setup(&op);
  elem_grad_dot_with(&op, u, w, out);
  GH1_CUDA(cudaStreamSynchronize(sp->ctx->stream));
}

void elem_grad_dot_with(gh1_op* op, const double* u, const double* w, double* out) {
  gh1_space* sp = op->sp;
  GH1_CHECK(!(sp->et == 4 && sp->mesh->def_space), GH1_ERR_UNSUPPORTED,
            "the element contraction on tets needs affine elements (the mesh is deformed)");
  const double* kappa = op->form->d_kappa.p;
  if (sp->et == 8) {
#define GH1_GD_CASE(NN) \
  case NN:              \
    launch_hex_graddot<NN>(op, u, w, out); \
    break;
    GH1_HEX_SWITCH(sp->p + 1, GH1_GD_CASE)
#undef GH1_GD_CASE
  } else {
    int ne = sp->mesh->ne;
    tet_graddot_kernel<<<(ne + 127) / 128, 128, 0, sp->ctx->stream>>>(ne, sp->nloc, sp->tet_nq, sp->d_eldofs.p,
                                                                       sp->d_class.p, op->d_G64.p, kappa, sp->d_tab64.p,
                                                                       sp->d_tq.p, u, w, out);
    check_kernel(sp->ctx, "tet_graddot_kernel");
  }
}

}  // namespace gh1
