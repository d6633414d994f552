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
#include <cmath>
#include <type_traits>
#include "common.cuh"
#include "basis.cuh"

namespace gh1 {

// ---------------------------------------------------------------------------
// geometry
__device__ __forceinline__ void inv3(const double* J, double* Ji, double& det) {
  det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) + J[2] * (J[3] * J[7] - J[4] * J[6]);
  double id = 1.0 / det;
  Ji[0] = (J[4] * J[8] - J[5] * J[7]) * id; Ji[1] = (J[2] * J[7] - J[1] * J[8]) * id; Ji[2] = (J[1] * J[5] - J[2] * J[4]) * id;
  Ji[3] = (J[5] * J[6] - J[3] * J[8]) * id; Ji[4] = (J[0] * J[8] - J[2] * J[6]) * id; Ji[5] = (J[2] * J[3] - J[0] * J[5]) * id;
  Ji[6] = (J[3] * J[7] - J[4] * J[6]) * id; Ji[7] = (J[1] * J[6] - J[0] * J[7]) * id; Ji[8] = (J[0] * J[4] - J[1] * J[3]) * id;
}

// J[3k+j] = d x_k / d xi_j of the trilinear hex map at (x,y,z)
__device__ __forceinline__ void hex_jacobian(const double* X, const int* v, double x, double y, double z, double* J) {
  const double dl[8][3] = {
      {-(1 - y) * (1 - z), -(1 - x) * (1 - z), -(1 - x) * (1 - y)}, {(1 - y) * (1 - z), -x * (1 - z), -x * (1 - y)},
      {y * (1 - z), x * (1 - z), -x * y},                           {-y * (1 - z), (1 - x) * (1 - z), -(1 - x) * y},
      {-(1 - y) * z, -(1 - x) * z, (1 - x) * (1 - y)},             {(1 - y) * z, -x * z, x * (1 - y)},
      {y * z, x * z, x * y},                                        {-y * z, (1 - x) * z, (1 - x) * y}};
  for (int i = 0; i < 9; i++) J[i] = 0;
  for (int a = 0; a < 8; a++) {
    const double* pa = X + 3 * (size_t)v[a];
    for (int k = 0; k < 3; k++)
      for (int j = 0; j < 3; j++) J[3 * k + j] += pa[k] * dl[a][j];
  }
}

// G[e][c][q] (c: xx yy zz xy xz yz) and M[e][q] for hex elements, FP64 math
__global__ void hex_geom_kernel(int ne, int nq1, const double* __restrict__ X, const int* __restrict__ el,
                                const double* __restrict__ gx, const double* __restrict__ gw,
                                const double* __restrict__ kappa, const double* __restrict__ mu, double* G64,
                                float* G32, double* M64, float* M32) {
  const int nq = nq1 * nq1 * nq1;
  int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= (int64_t)ne * nq) return;
  int e = (int)(id / nq), q = (int)(id % nq);
  int i = q / (nq1 * nq1), j = (q / nq1) % nq1, k = q % nq1;
  int v[8];
  for (int a = 0; a < 8; a++) v[a] = el[(size_t)e * 8 + a];
  double J[9], Ji[9], det;
  hex_jacobian(X, v, gx[i], gx[j], gx[k], J);
  inv3(J, Ji, det);
  double wdet = gw[i] * gw[j] * gw[k] * fabs(det);
  double f = kappa[e] * wdet;
  double g[6];
  g[0] = f * (Ji[0] * Ji[0] + Ji[1] * Ji[1] + Ji[2] * Ji[2]);
  g[1] = f * (Ji[3] * Ji[3] + Ji[4] * Ji[4] + Ji[5] * Ji[5]);
  g[2] = f * (Ji[6] * Ji[6] + Ji[7] * Ji[7] + Ji[8] * Ji[8]);
  g[3] = f * (Ji[0] * Ji[3] + Ji[1] * Ji[4] + Ji[2] * Ji[5]);
  g[4] = f * (Ji[0] * Ji[6] + Ji[1] * Ji[7] + Ji[2] * Ji[8]);
  g[5] = f * (Ji[3] * Ji[6] + Ji[4] * Ji[7] + Ji[5] * Ji[8]);
  for (int c = 0; c < 6; c++) {
    size_t o = ((size_t)e * 6 + c) * nq + q;
    if (G64) G64[o] = g[c];
    if (G32) G32[o] = (float)g[c];
  }
  if (mu) {
    double m = mu[e] * wdet;
    if (M64) M64[(size_t)e * nq + q] = m;
    if (M32) M32[(size_t)e * nq + q] = (float)m;
  }
}

// tet: G[e][6] = kappa |det| J^{-1} J^{-T}, M[e] = mu |det|
__global__ void tet_geom_kernel(int ne, const double* __restrict__ X, const int* __restrict__ el,
                                const double* __restrict__ kappa, const double* __restrict__ mu, double* G64,
                                float* G32, double* M64, float* M32) {
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
  double f = kappa[e] * fabs(det);
  double g[6];
  g[0] = f * (Ji[0] * Ji[0] + Ji[1] * Ji[1] + Ji[2] * Ji[2]);
  g[1] = f * (Ji[3] * Ji[3] + Ji[4] * Ji[4] + Ji[5] * Ji[5]);
  g[2] = f * (Ji[6] * Ji[6] + Ji[7] * Ji[7] + Ji[8] * Ji[8]);
  g[3] = f * (Ji[0] * Ji[3] + Ji[1] * Ji[4] + Ji[2] * Ji[5]);
  g[4] = f * (Ji[0] * Ji[6] + Ji[1] * Ji[7] + Ji[2] * Ji[8]);
  g[5] = f * (Ji[3] * Ji[6] + Ji[4] * Ji[7] + Ji[5] * Ji[8]);
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

// ---------------------------------------------------------------------------
// thread-group helpers
template <int G>
__device__ __forceinline__ void group_sync(int gid) {
  if (G == 32) __syncwarp();
  else asm volatile("bar.sync %0, %1;" ::"r"(gid + 1), "r"(G) : "memory");
}

template <class T>
__device__ __forceinline__ void atomic_add_t(T* p, T v) { atomicAdd(p, v); }

// End-of-kernel reduction of one double per thread into partial[blockIdx.x];
// the last block to finish sums all partials into *out and resets the counter.
// (threadfence reduction: no block waits on another.)
__device__ void block_reduce_finish(double v, double* partial, unsigned int* counter, double* out) {
  __shared__ double red[32];
  __shared__ bool last;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0;
    for (int i = 0; i < (int)(blockDim.x + 31) / 32; i++) s += red[i];
    partial[blockIdx.x] = s;
    __threadfence();
    unsigned int t = atomicAdd(counter, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {
    __threadfence();
    double s = 0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) s += ((volatile double*)partial)[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (l == 0) red[w] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double tot = 0;
      for (int i = 0; i < (int)(blockDim.x + 31) / 32; i++) tot += red[i];
      *out = tot;
      *counter = 0u;
    }
  }
}

template <int N>
struct HexCfg {
  static constexpr int N2 = N * N, N3 = N * N * N;
  static constexpr int G = ((N2 + 31) / 32) * 32;  // threads per element
  static constexpr int EPB = G == 32 ? 8 : (G == 64 ? 4 : 2);  // elements per block
  static constexpr int BLOCK = G * EPB;
};

template <int N, class T>
constexpr size_t hex_smem_bytes() {
  return (size_t)HexCfg<N>::EPB * (5 * HexCfg<N>::N3 * sizeof(T) + HexCfg<N>::N3 * sizeof(int)) + 2 * N * N * sizeof(T);
}

// Forward chain: gathered coefficients in su[(a*N+b)*N+c] -> reference gradient
// components at the qp of lane (j,k) for all i (registers gx[i], gy[i], gz[i]),
// plus the interpolated value uq[i] when WANT_U.
template <int N, class T, bool WANT_U>
__device__ __forceinline__ void hex_forward(int lane, int gid, const T* sB, const T* sD, T* su, T* s1, T* s2, T* t2,
                                            T* t3, T* gx, T* gy, T* gz, T* uq) {
  constexpr int N2 = N * N, G = HexCfg<N>::G;
  T* t1 = su;  // alias: u is consumed by stage 1 before t1 is written
  if (lane < N2) {
    const int a = lane / N, b = lane % N;
    T u[N];
#pragma unroll
    for (int c = 0; c < N; c++) u[c] = su[(a * N + b) * N + c];
#pragma unroll
    for (int k = 0; k < N; k++) {
      T ub = 0, ud = 0;
#pragma unroll
      for (int c = 0; c < N; c++) { ub += sB[k * N + c] * u[c]; ud += sD[k * N + c] * u[c]; }
      s1[(a * N + b) * N + k] = ub;
      s2[(a * N + b) * N + k] = ud;
    }
  }
  group_sync<G>(gid);
  if (lane < N2) {
    const int a = lane / N, k = lane % N;
    T v1[N], v2[N];
#pragma unroll
    for (int b = 0; b < N; b++) { v1[b] = s1[(a * N + b) * N + k]; v2[b] = s2[(a * N + b) * N + k]; }
#pragma unroll
    for (int j = 0; j < N; j++) {
      T bb = 0, db = 0, bd = 0;
#pragma unroll
      for (int b = 0; b < N; b++) {
        bb += sB[j * N + b] * v1[b];
        db += sD[j * N + b] * v1[b];
        bd += sB[j * N + b] * v2[b];
      }
      t1[(a * N + j) * N + k] = bb;
      t2[(a * N + j) * N + k] = db;
      t3[(a * N + j) * N + k] = bd;
    }
  }
  group_sync<G>(gid);
  if (lane < N2) {
    const int j = lane / N, k = lane % N;
    T w1[N], w2[N], w3[N];
#pragma unroll
    for (int a = 0; a < N; a++) {
      w1[a] = t1[(a * N + j) * N + k];
      w2[a] = t2[(a * N + j) * N + k];
      w3[a] = t3[(a * N + j) * N + k];
    }
#pragma unroll
    for (int i = 0; i < N; i++) {
      T x = 0, y = 0, z = 0, uu = 0;
#pragma unroll
      for (int a = 0; a < N; a++) {
        x += sD[i * N + a] * w1[a];
        y += sB[i * N + a] * w2[a];
        z += sB[i * N + a] * w3[a];
        if (WANT_U) uu += sB[i * N + a] * w1[a];
      }
      gx[i] = x; gy[i] = y; gz[i] = z;
      if (WANT_U) uq[i] = uu;
    }
  }
  group_sync<G>(gid);
}

// Transposed chain: lane (j,k) holds vx,vy,vz (and vm) at its qp column ->
// element residual in su[(a*N+b)*N+c].
template <int N, class T, bool WANT_M>
__device__ __forceinline__ void hex_backward(int lane, int gid, const T* sB, const T* sD, T* su, T* s1, T* s2, T* t2,
                                             T* t3, const T* vx, const T* vy, const T* vz, const T* vm) {
  constexpr int N2 = N * N, G = HexCfg<N>::G;
  T* t1 = su;
  if (lane < N2) {
    const int j = lane / N, k = lane % N;
#pragma unroll
    for (int a = 0; a < N; a++) {
      T w1 = 0, w2 = 0, w3 = 0;
#pragma unroll
      for (int i = 0; i < N; i++) {
        w1 += sD[i * N + a] * vx[i];
        if (WANT_M) w1 += sB[i * N + a] * vm[i];
        w2 += sB[i * N + a] * vy[i];
        w3 += sB[i * N + a] * vz[i];
      }
      t1[(a * N + j) * N + k] = w1;
      t2[(a * N + j) * N + k] = w2;
      t3[(a * N + j) * N + k] = w3;
    }
  }
  group_sync<G>(gid);
  if (lane < N2) {
    const int a = lane / N, k = lane % N;
    T r1[N], r2[N], r3[N];
#pragma unroll
    for (int j = 0; j < N; j++) {
      r1[j] = t1[(a * N + j) * N + k];
      r2[j] = t2[(a * N + j) * N + k];
      r3[j] = t3[(a * N + j) * N + k];
    }
#pragma unroll
    for (int b = 0; b < N; b++) {
      T v1 = 0, v2 = 0;
#pragma unroll
      for (int j = 0; j < N; j++) {
        v1 += sB[j * N + b] * r1[j] + sD[j * N + b] * r2[j];
        v2 += sB[j * N + b] * r3[j];
      }
      s1[(a * N + b) * N + k] = v1;
      s2[(a * N + b) * N + k] = v2;
    }
  }
  group_sync<G>(gid);
  if (lane < N2) {
    const int a = lane / N, b = lane % N;
    T r1[N], r2[N];
#pragma unroll
    for (int k = 0; k < N; k++) { r1[k] = s1[(a * N + b) * N + k]; r2[k] = s2[(a * N + b) * N + k]; }
#pragma unroll
    for (int c = 0; c < N; c++) {
      T v = 0;
#pragma unroll
      for (int k = 0; k < N; k++) v += sB[k * N + c] * r1[k] + sD[k * N + c] * r2[k];
      su[(a * N + b) * N + c] = v;
    }
  }
  group_sync<G>(gid);
}

// y += A x over all hex elements; optional energy sum_e x_e^T A_e x_e.
// skip != NULL: the kernel returns immediately when *skip != 0 (CG finished).
template <int N, class T, bool MASS>
__global__ void __launch_bounds__(HexCfg<N>::BLOCK)
hex_apply_kernel(int ne, const int* __restrict__ tdof, const T* __restrict__ Gq, const T* __restrict__ Mq,
                 const T* __restrict__ x, T* __restrict__ y, const T* __restrict__ Bg, const T* __restrict__ Dg,
                 double* partial, unsigned int* counter, double* energy, const int* skip) {
  using C = HexCfg<N>;
  constexpr int N2 = C::N2, N3 = C::N3, G = C::G;
  if (skip && *(volatile const int*)skip) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sB = (T*)smem_raw;
  T* sD = sB + N2;
  const int gid = threadIdx.x / G, lane = threadIdx.x % G;
  T* base = sD + N2 + (size_t)gid * 5 * N3;
  T *su = base, *s1 = base + N3, *s2 = base + 2 * N3, *t2 = base + 3 * N3, *t3 = base + 4 * N3;
  int* sidx = (int*)(sD + N2 + (size_t)C::EPB * 5 * N3) + gid * N3;
  for (int t = threadIdx.x; t < N2; t += blockDim.x) { sB[t] = Bg[t]; sD[t] = Dg[t]; }
  __syncthreads();
  T acc = 0;  // per-lane energy in the working precision (FP64 throughput is scarce)
  for (int e = blockIdx.x * C::EPB + gid; e < ne; e += gridDim.x * C::EPB) {
    const int* td = tdof + (size_t)e * N3;
    for (int t = lane; t < N3; t += G) {
      int d = __ldg(td + t);
      sidx[t] = d;
      T v = __ldg(x + (d & 0x7fffffff));
      su[t] = d < 0 ? -v : v;
    }
    group_sync<G>(gid);
    T gx[N], gy[N], gz[N], uq[N];
    hex_forward<N, T, MASS>(lane, gid, sB, sD, su, s1, s2, t2, t3, gx, gy, gz, uq);
    T vx[N], vy[N], vz[N], vm[N];
    if (lane < N2) {
      const T* Ge = Gq + (size_t)e * 6 * N3 + lane;
#pragma unroll
      for (int i = 0; i < N; i++) {
        const int o = i * N2;
        T gxx = __ldg(Ge + o), gyy = __ldg(Ge + N3 + o), gzz = __ldg(Ge + 2 * N3 + o);
        T gxy = __ldg(Ge + 3 * N3 + o), gxz = __ldg(Ge + 4 * N3 + o), gyz = __ldg(Ge + 5 * N3 + o);
        vx[i] = gxx * gx[i] + gxy * gy[i] + gxz * gz[i];
        vy[i] = gxy * gx[i] + gyy * gy[i] + gyz * gz[i];
        vz[i] = gxz * gx[i] + gyz * gy[i] + gzz * gz[i];
        T en = gx[i] * vx[i] + gy[i] * vy[i] + gz[i] * vz[i];
        if (MASS) {
          vm[i] = __ldg(Mq + (size_t)e * N3 + o + lane) * uq[i];
          en += uq[i] * vm[i];
        }
        acc += en;
      }
    }
    hex_backward<N, T, MASS>(lane, gid, sB, sD, su, s1, s2, t2, t3, vx, vy, vz, vm);
    for (int t = lane; t < N3; t += G) {
      int d = sidx[t];
      T v = su[t];
      atomic_add_t(y + (d & 0x7fffffff), d < 0 ? -v : v);
    }
    group_sync<G>(gid);
  }
  if (partial) block_reduce_finish((double)acc, partial, counter, energy);
}

// element-wise  int_e grad u . grad w  (geometry from G / kappa_e)
template <int N>
__global__ void __launch_bounds__(HexCfg<N>::BLOCK)
hex_graddot_kernel(int ne, const int* __restrict__ tdof, const double* __restrict__ Gq, const double* __restrict__ kappa,
                   const double* __restrict__ u, const double* __restrict__ w, const double* __restrict__ Bg,
                   const double* __restrict__ Dg, double* out) {
  using C = HexCfg<N>;
  using T = double;
  constexpr int N2 = C::N2, N3 = C::N3, G = C::G;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sB = (T*)smem_raw;
  T* sD = sB + N2;
  const int gid = threadIdx.x / G, lane = threadIdx.x % G;
  T* base = sD + N2 + (size_t)gid * 5 * N3;
  T *su = base, *s1 = base + N3, *s2 = base + 2 * N3, *t2 = base + 3 * N3, *t3 = base + 4 * N3;
  __shared__ double red[C::EPB][(C::G + 31) / 32];
  for (int t = threadIdx.x; t < N2; t += blockDim.x) { sB[t] = Bg[t]; sD[t] = Dg[t]; }
  __syncthreads();
  for (int e0 = blockIdx.x * C::EPB; e0 < ne; e0 += gridDim.x * C::EPB) {
    int e = e0 + gid;
    bool valid = e < ne;
    T ux[N], uy[N], uz[N], wx[N], wy[N], wz[N], dummy[N];
    for (int t = lane; t < N3; t += G) {
      int d = valid ? tdof[(size_t)e * N3 + t] : 0;
      T v = valid ? u[d & 0x7fffffff] : 0.0;
      su[t] = d < 0 ? -v : v;
    }
    group_sync<G>(gid);
    hex_forward<N, T, false>(lane, gid, sB, sD, su, s1, s2, t2, t3, ux, uy, uz, dummy);
    for (int t = lane; t < N3; t += G) {
      int d = valid ? tdof[(size_t)e * N3 + t] : 0;
      T v = valid ? w[d & 0x7fffffff] : 0.0;
      su[t] = d < 0 ? -v : v;
    }
    group_sync<G>(gid);
    hex_forward<N, T, false>(lane, gid, sB, sD, su, s1, s2, t2, t3, wx, wy, wz, dummy);
    double acc = 0;
    if (lane < N2 && valid) {
      const T* Ge = Gq + (size_t)e * 6 * N3 + lane;
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

// diagonal of the hex operator: one thread per (element, tensor index)
__global__ void hex_diag_kernel(int ne, int N, const int* __restrict__ tdof, const double* __restrict__ Gq,
                                const double* __restrict__ Mq, const double* __restrict__ B, const double* __restrict__ D,
                                double* diag) {
  const int N3 = N * N * N;
  int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= (int64_t)ne * N3) return;
  int e = (int)(id / N3), t = (int)(id % N3);
  int a = t / (N * N), b = (t / N) % N, c = t % N;
  const double* Ge = Gq + (size_t)e * 6 * N3;
  double s = 0;
  for (int i = 0; i < N; i++) {
    double Ba = B[i * N + a], Da = D[i * N + a];
    for (int j = 0; j < N; j++) {
      double Bb = B[j * N + b], Db = D[j * N + b];
      for (int k = 0; k < N; k++) {
        double Bc = B[k * N + c], Dc = D[k * N + c];
        int q = (i * N + j) * N + k;
        double gx = Da * Bb * Bc, gy = Ba * Db * Bc, gz = Ba * Bb * Dc;
        s += Ge[q] * gx * gx + Ge[N3 + q] * gy * gy + Ge[2 * N3 + q] * gz * gz +
             2 * (Ge[3 * N3 + q] * gx * gy + Ge[4 * N3 + q] * gx * gz + Ge[5 * N3 + q] * gy * gz);
        if (Mq) { double v = Ba * Bb * Bc; s += Mq[(size_t)e * N3 + q] * v * v; }
      }
    }
  }
  atomicAdd(diag + (tdof[id] & 0x7fffffff), s);
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
      atomicAdd(y + dn[i], r);
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
  atomicAdd(diag + eldofs[id], s);
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

// ---------------------------------------------------------------------------
// host drivers
// sets the dynamic shared-memory limit and returns resident blocks per SM;
// done once per instantiation, outside any stream capture (called at setup)
template <int N, class T, bool MASS>
int hex_apply_prepare() {
  static int per_sm = -1;
  if (per_sm < 0) {
    size_t smem = hex_smem_bytes<N, T>();
    GH1_CUDA(cudaFuncSetAttribute(hex_apply_kernel<N, T, MASS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int v = 0;
    GH1_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, hex_apply_kernel<N, T, MASS>, HexCfg<N>::BLOCK, smem));
    per_sm = v < 1 ? 1 : v;
  }
  return per_sm;
}

void hex_prepare_all(int N) {
#define GH1_PREP(NN)                                                                              \
  case NN:                                                                                        \
    hex_apply_prepare<NN, float, false>(); hex_apply_prepare<NN, float, true>();                  \
    hex_apply_prepare<NN, double, false>(); hex_apply_prepare<NN, double, true>();                \
    break;
  switch (N) {
    GH1_PREP(2) GH1_PREP(3) GH1_PREP(4) GH1_PREP(5) GH1_PREP(6) GH1_PREP(7) GH1_PREP(8) GH1_PREP(9)
    default: break;
  }
#undef GH1_PREP
}

template <int N, class T, bool MASS>
void launch_hex_apply(gh1_op* op, const T* x, T* y, const T* G, const T* M, double* partial, unsigned int* counter,
                      double* energy, const int* skip, int nblocks_override = 0) {
  using C = HexCfg<N>;
  gh1_space* sp = op->sp;
  size_t smem = hex_smem_bytes<N, T>();
  const int per_sm = hex_apply_prepare<N, T, MASS>();
  int ne = sp->mesh->ne;
  int blocks_needed = (ne + C::EPB - 1) / C::EPB;
  int grid = std::min(blocks_needed, sp->ctx->nsm * per_sm);
  if (nblocks_override > 0) grid = std::min(blocks_needed, nblocks_override);
  const T* Bt = std::is_same<T, float>::value ? (const T*)sp->d_B32.p : (const T*)sp->d_B64.p;
  const T* Dt = std::is_same<T, float>::value ? (const T*)sp->d_D32.p : (const T*)sp->d_D64.p;
  hex_apply_kernel<N, T, MASS><<<grid, C::BLOCK, smem, sp->ctx->stream>>>(ne, sp->d_tdof.p, G, M, x, y, Bt, Dt, partial,
                                                                           counter, energy, skip);
  check_kernel(sp->ctx, "hex_apply_kernel");
}

template <class T>
void hex_apply_dispatch(gh1_op* op, const T* x, T* y, const T* G, const T* M, double* partial, unsigned int* counter,
                        double* energy, const int* skip) {
  const int N = op->sp->p + 1;
  bool mass = M != nullptr;
#define GH1_HEX_CASE(NN)                                                                                  \
  case NN:                                                                                                \
    if (mass) launch_hex_apply<NN, T, true>(op, x, y, G, M, partial, counter, energy, skip);             \
    else launch_hex_apply<NN, T, false>(op, x, y, G, M, partial, counter, energy, skip);                 \
    break;
  switch (N) {
    GH1_HEX_CASE(2) GH1_HEX_CASE(3) GH1_HEX_CASE(4) GH1_HEX_CASE(5) GH1_HEX_CASE(6) GH1_HEX_CASE(7)
    GH1_HEX_CASE(8) GH1_HEX_CASE(9)
    default: throw Error(GH1_ERR_UNSUPPORTED, "hex order out of range");
  }
#undef GH1_HEX_CASE
}

int matfree_grid_blocks(gh1_op* op) {
  // number of blocks the apply launches (sizes the partial-sum buffer)
  gh1_space* sp = op->sp;
  int ne = sp->mesh->ne;
  if (sp->et == 4) return std::max(1, std::min((ne + 7) / 8, sp->ctx->nsm * 8));
  return std::max(1, std::min(ne, sp->ctx->nsm * 32));
}

void matfree_setup(gh1_op* op) {
  gh1_space* sp = op->sp;
  gh1_form* f = op->form;
  cudaStream_t s = sp->ctx->stream;
  const int ne = sp->mesh->ne;
  const bool want64 = true;  // the FP64 copy also serves the diagonal and the adjoint contraction
  const bool want32 = (op->prec_mask & 2) != 0;
  op->has_mass = f->has_mu;
  if (sp->et == 8) {
    const int nq = sp->nq1 * sp->nq1 * sp->nq1;
    op->d_G64.alloc((size_t)ne * 6 * nq);
    if (want32) op->d_G32.alloc((size_t)ne * 6 * nq); else op->d_G32.release();
    if (op->has_mass) {
      op->d_M64.alloc((size_t)ne * nq);
      if (want32) op->d_M32.alloc((size_t)ne * nq);
    }
    int64_t tot = (int64_t)ne * nq;
    hex_geom_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(
        ne, sp->nq1, sp->mesh->d_X.p, sp->mesh->d_el.p, sp->d_gx.p, sp->d_gw.p, f->d_kappa.p,
        op->has_mass ? f->d_mu.p : nullptr, want64 ? op->d_G64.p : nullptr, want32 ? op->d_G32.p : nullptr,
        op->has_mass ? op->d_M64.p : nullptr, (op->has_mass && want32) ? op->d_M32.p : nullptr);
    check_kernel(sp->ctx, "hex_geom_kernel");
    hex_prepare_all(sp->p + 1);
  } else {
    op->d_G64.alloc((size_t)ne * 6);
    if (want32) op->d_G32.alloc((size_t)ne * 6); else op->d_G32.release();
    if (op->has_mass) {
      op->d_M64.alloc(ne);
      if (want32) op->d_M32.alloc(ne);
    }
    tet_geom_kernel<<<(ne + 255) / 256, 256, 0, s>>>(ne, sp->mesh->d_X.p, sp->mesh->d_el.p, f->d_kappa.p,
                                                      op->has_mass ? f->d_mu.p : nullptr, op->d_G64.p,
                                                      want32 ? op->d_G32.p : nullptr, op->has_mass ? op->d_M64.p : nullptr,
                                                      (op->has_mass && want32) ? op->d_M32.p : nullptr);
    check_kernel(sp->ctx, "tet_geom_kernel");
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
  if (sp->et == 8) {
    if (prec == GH1_F64)
      hex_apply_dispatch<double>(op, (const double*)x, (double*)y, op->d_G64.p, op->has_mass ? op->d_M64.p : nullptr,
                                 partial, counter, energy, skip);
    else
      hex_apply_dispatch<float>(op, (const float*)x, (float*)y, op->d_G32.p, op->has_mass ? op->d_M32.p : nullptr,
                                partial, counter, energy, skip);
  } else {
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
  const int ne = sp->mesh->ne;
  if (sp->et == 8) {
    const int N = sp->p + 1;
    int64_t tot = (int64_t)ne * N * N * N;
    hex_diag_kernel<<<(unsigned)((tot + 127) / 128), 128, 0, s>>>(ne, N, sp->d_tdof.p, op->d_G64.p,
                                                                   op->has_mass ? op->d_M64.p : nullptr, sp->d_B64.p,
                                                                   sp->d_D64.p, diag);
    check_kernel(sp->ctx, "hex_diag_kernel");
  } else {
    int64_t tot = (int64_t)ne * sp->nloc;
    tet_diag_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(ne, sp->nloc, sp->d_eldofs.p, sp->d_class.p, op->d_G64.p,
                                                                   op->has_mass ? op->d_M64.p : nullptr, sp->d_S.p, diag);
    check_kernel(sp->ctx, "tet_diag_kernel");
  }
}

template <int N>
void launch_hex_graddot(gh1_space* sp, const double* G, const double* kappa, const double* u, const double* w, double* out) {
  using C = HexCfg<N>;
  size_t smem = hex_smem_bytes<N, double>();
  static bool attr_set = false;
  if (!attr_set) {
    GH1_CUDA(cudaFuncSetAttribute(hex_graddot_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set = true;
  }
  int ne = sp->mesh->ne;
  int grid = std::max(1, std::min((ne + C::EPB - 1) / C::EPB, sp->ctx->nsm * 16));
  hex_graddot_kernel<N><<<grid, C::BLOCK, smem, sp->ctx->stream>>>(ne, sp->d_tdof.p, G, kappa, u, w, sp->d_B64.p,
                                                                    sp->d_D64.p, out);
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
  const double* kappa = op->form->d_kappa.p;
  if (sp->et == 8) {
    switch (sp->p + 1) {
      case 2: launch_hex_graddot<2>(sp, op->d_G64.p, kappa, u, w, out); break;
      case 3: launch_hex_graddot<3>(sp, op->d_G64.p, kappa, u, w, out); break;
      case 4: launch_hex_graddot<4>(sp, op->d_G64.p, kappa, u, w, out); break;
      case 5: launch_hex_graddot<5>(sp, op->d_G64.p, kappa, u, w, out); break;
      case 6: launch_hex_graddot<6>(sp, op->d_G64.p, kappa, u, w, out); break;
      case 7: launch_hex_graddot<7>(sp, op->d_G64.p, kappa, u, w, out); break;
      case 8: launch_hex_graddot<8>(sp, op->d_G64.p, kappa, u, w, out); break;
      case 9: launch_hex_graddot<9>(sp, op->d_G64.p, kappa, u, w, out); break;
      default: throw Error(GH1_ERR_UNSUPPORTED, "hex order out of range");
    }
  } else {
    int ne = sp->mesh->ne;
    tet_graddot_kernel<<<(ne + 127) / 128, 128, 0, sp->ctx->stream>>>(ne, sp->nloc, sp->tet_nq, sp->d_eldofs.p,
                                                                       sp->d_class.p, op->d_G64.p, kappa, sp->d_tab64.p,
                                                                       sp->d_tq.p, u, w, out);
    check_kernel(sp->ctx, "tet_graddot_kernel");
  }
}

}  // namespace gh1
