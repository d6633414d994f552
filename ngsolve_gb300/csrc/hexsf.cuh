// hexsf.cuh -- the sum-factorization core of the one-element hex apply, shared
// by the translation units that instantiate it (matfree.cu: Laplace / mass
// kernels, bdb.cu: generic B^T D B kernels).  The 1D factor tables live in
// constant memory with internal linkage: every including translation unit has
// its own copy and fills it with upload_const_tables before its first launch.
#pragma once
#include <algorithm>
#include <cmath>
#include <vector>
#include "common.cuh"
#include "hexcore.cuh"

namespace gh1 {

// ---------------------------------------------------------------------------
// 1D hex factor tables B[q][a] = psi_a(x_q), D[q][a] = psi_a'(x_q) of every order
// in constant memory: with the contraction loops unrolled the FMAs take their
// table operand straight from the constant bank (no shared-memory load per FMA).
static __constant__ float c_B32[TAB_TOTAL], c_D32[TAB_TOTAL];
static __constant__ double c_B64[TAB_TOTAL], c_D64[TAB_TOTAL];
// Even-odd (reflection) form of the 1D contractions.  The Gauss points are
// symmetric about 1/2, psi_0 and psi_1 swap under x -> 1-x and psi_c picks up
// (-1)^c for c >= 2, so with q' = N-1-q:
//   B[q'][0] = B[q][1], B[q'][1] = B[q][0], B[q'][c] = (-1)^c B[q][c];
//   D[q'][0] = -D[q][1], D[q'][1] = -D[q][0], D[q'][c] = -(-1)^c D[q][c].
// A contraction then splits into an even part (inputs u0+u1 and the even c) and
// an odd part (u0-u1 and the odd c) evaluated for q < N/2 only, ~25 % fewer FMAs.
// c_EO*[0..3][W(N) + q] hold (B[q][0] +- B[q][1]) / 2 and (D[q][0] +- D[q][1]) / 2.
static __constant__ float c_EO32[4][64];
static __constant__ double c_EO64[4][64];
// 1D Gauss weights of every order at offset eo_off(N) (the per-element metric
// records of the generic B^T D B apply are weighted per point in the kernel)
static __constant__ float c_W32[64];
static __constant__ double c_W64[64];
template <class T> struct CTab;
template <> struct CTab<float> {
  static __device__ __forceinline__ float B(int i) { return c_B32[i]; }
  static __device__ __forceinline__ float D(int i) { return c_D32[i]; }
  static __device__ __forceinline__ float EO(int k, int i) { return c_EO32[k][i]; }
  static __device__ __forceinline__ float W(int i) { return c_W32[i]; }
};
template <> struct CTab<double> {
  static __device__ __forceinline__ double B(int i) { return c_B64[i]; }
  static __device__ __forceinline__ double D(int i) { return c_D64[i]; }
  static __device__ __forceinline__ double EO(int k, int i) { return c_EO64[k][i]; }
  static __device__ __forceinline__ double W(int i) { return c_W64[i]; }
};

static void upload_const_tables(gh1_space* sp) {
  const int N = sp->p + 1, off = tab_off(N);
  cudaStream_t s = sp->ctx->stream;
  GH1_CUDA(cudaMemcpyToSymbolAsync(c_B32, sp->d_B32.p, N * N * sizeof(float), off * sizeof(float), cudaMemcpyDeviceToDevice, s));
  GH1_CUDA(cudaMemcpyToSymbolAsync(c_D32, sp->d_D32.p, N * N * sizeof(float), off * sizeof(float), cudaMemcpyDeviceToDevice, s));
  GH1_CUDA(cudaMemcpyToSymbolAsync(c_B64, sp->d_B64.p, N * N * sizeof(double), off * sizeof(double), cudaMemcpyDeviceToDevice, s));
  GH1_CUDA(cudaMemcpyToSymbolAsync(c_D64, sp->d_D64.p, N * N * sizeof(double), off * sizeof(double), cudaMemcpyDeviceToDevice, s));
  // even-odd coefficients, after checking the reflection symmetry they rely on
  std::vector<double> B(N * N), D(N * N);
  GH1_CUDA(cudaMemcpyAsync(B.data(), sp->d_B64.p, N * N * sizeof(double), cudaMemcpyDeviceToHost, s));
  GH1_CUDA(cudaMemcpyAsync(D.data(), sp->d_D64.p, N * N * sizeof(double), cudaMemcpyDeviceToHost, s));
  GH1_CUDA(cudaStreamSynchronize(s));
  double eo[4][16];
  GH1_CHECK(hex_eo_coefficients(B.data(), D.data(), N, eo) <= 1e-12, GH1_ERR_ARG,
            "internal: 1D hex tables lack the reflection symmetry");
  float eo32[4][16];
  for (int k = 0; k < 4; k++)
    for (int q = 0; q < 16; q++) eo32[k][q] = (float)eo[k][q];
  for (int k = 0; k < 4; k++) {
    GH1_CUDA(cudaMemcpyToSymbol(c_EO64, eo[k], N * sizeof(double), (k * 64 + eo_off(N)) * sizeof(double)));
    GH1_CUDA(cudaMemcpyToSymbol(c_EO32, eo32[k], N * sizeof(float), (k * 64 + eo_off(N)) * sizeof(float)));
  }
  GH1_CHECK((int)sp->gw.size() == N, GH1_ERR_ARG, "internal: hex rule size");
  std::vector<float> w32(sp->gw.begin(), sp->gw.end());
  GH1_CUDA(cudaMemcpyToSymbol(c_W64, sp->gw.data(), N * sizeof(double), eo_off(N) * sizeof(double)));
  GH1_CUDA(cudaMemcpyToSymbol(c_W32, w32.data(), N * sizeof(float), eo_off(N) * sizeof(float)));
}

// out_b[q] = sum_c B[q][c] u[c] and out_d[q] = sum_c D[q][c] u[c] (either may be
// skipped): the forward contraction in even-odd form
template <int N, class T, bool WB, bool WD>
__device__ __forceinline__ void eo_fwd(const T* u, T* ob, T* od) {
  constexpr int O = tab_off(N), W = eo_off(N), M = N / 2;
  using TB = CTab<T>;
  const T s = u[0] + u[1], d = u[0] - u[1];
#pragma unroll
  for (int q = 0; q < M; q++) {
    T eb = 0, obb = 0, ed = 0, odd = 0;
    if (WB) { eb = TB::EO(0, W + q) * s; obb = TB::EO(1, W + q) * d; }
    if (WD) { ed = TB::EO(2, W + q) * s; odd = TB::EO(3, W + q) * d; }
#pragma unroll
    for (int c = 2; c < N; c++) {
      if (c % 2 == 0) {
        if (WB) eb += TB::B(O + q * N + c) * u[c];
        if (WD) ed += TB::D(O + q * N + c) * u[c];
      } else {
        if (WB) obb += TB::B(O + q * N + c) * u[c];
        if (WD) odd += TB::D(O + q * N + c) * u[c];
      }
    }
    if (WB) { ob[q] = eb + obb; ob[N - 1 - q] = eb - obb; }
    if (WD) { od[q] = ed + odd; od[N - 1 - q] = odd - ed; }
  }
  if (N % 2 == 1) {  // middle point: B keeps its even part, D its odd part
    constexpr int q = M;
    T eb = 0, odd = 0;
    if (WB) eb = TB::EO(0, W + q) * s;
    if (WD) odd = TB::EO(3, W + q) * d;
#pragma unroll
    for (int c = 2; c < N; c++) {
      if (c % 2 == 0) { if (WB) eb += TB::B(O + q * N + c) * u[c]; }
      else { if (WD) odd += TB::D(O + q * N + c) * u[c]; }
    }
    if (WB) ob[q] = eb;
    if (WD) od[q] = odd;
  }
}

// out[a] (+)= sum_q B[q][a] v[q] (WANT_D = false) or sum_q D[q][a] v[q]: the
// transposed contraction in even-odd form; ACC adds into out
template <int N, class T, bool WANT_D, bool ACC>
__device__ __forceinline__ void eo_bwd(const T* v, T* out) {
  constexpr int O = tab_off(N), W = eo_off(N), M = N / 2;
  using TB = CTab<T>;
  T vs[M > 0 ? M : 1], vd[M > 0 ? M : 1];
#pragma unroll
  for (int k = 0; k < M; k++) { vs[k] = v[k] + v[N - 1 - k]; vd[k] = v[k] - v[N - 1 - k]; }
  // a = 0, 1
  T P = 0, Q = 0;
#pragma unroll
  for (int k = 0; k < M; k++) {
    if (!WANT_D) { P += TB::EO(0, W + k) * vs[k]; Q += TB::EO(1, W + k) * vd[k]; }
    else { P += TB::EO(2, W + k) * vd[k]; Q += TB::EO(3, W + k) * vs[k]; }
  }
  if (N % 2 == 1) {
    if (!WANT_D) P += TB::B(O + M * N) * v[M];
    else Q += TB::D(O + M * N) * v[M];
  }
  T r[N];
  r[0] = P + Q;
  r[1] = P - Q;
#pragma unroll
  for (int a = 2; a < N; a++) {
    // B: even a uses vs (+ the middle point), odd a uses vd; D: the reverse
    const bool sym = WANT_D ? (a % 2 == 1) : (a % 2 == 0);
    T t = 0;
#pragma unroll
    for (int k = 0; k < M; k++) t += (WANT_D ? TB::D(O + k * N + a) : TB::B(O + k * N + a)) * (sym ? vs[k] : vd[k]);
    if (N % 2 == 1 && sym) t += (WANT_D ? TB::D(O + M * N + a) : TB::B(O + M * N + a)) * v[M];
    r[a] = t;
  }
#pragma unroll
  for (int a = 0; a < N; a++) out[a] = ACC ? out[a] + r[a] : r[a];
}

// shared memory of the pipelined apply, per element group:
//   [G tile (G mode 0 only)] | DOF-table tile x2 | 5 work arrays | 3 mbarriers
template <int N, class T>
struct HexSmem {
  static constexpr int W = HexCfg<N>::EPW;
  static constexpr size_t tables = 0;
  static __host__ __device__ size_t gbytes(int gstride) { return W * round16((size_t)gstride * sizeof(T)); }
  static __host__ __device__ size_t tbytes(int tstride) { return W * round16((size_t)tstride * sizeof(int)); }
  static constexpr size_t work = round16(5 * (size_t)W * N * N * N * sizeof(T));
  static __host__ __device__ size_t group(int gstride, int tstride, int gmode) {
    return (gmode == 0 ? gbytes(gstride) : 0) + 2 * tbytes(tstride) + work + 32;
  }
  static __host__ __device__ size_t total(int gstride, int tstride, int gmode) {
    return tables + (size_t)HexCfg<N>::EPB * group(gstride, tstride, gmode);
  }
};


// Forward chain: gathered coefficients in su[(a*N+b)*N+c] -> reference gradient
// components at the qp of lane (j,k) for all i (registers gx[i], gy[i], gz[i]),
// plus the interpolated value uq[i] when WANT_U.
template <int N, class T, bool WANT_U>
__device__ __forceinline__ void hex_forward(int pl, bool active, int gid, T* su, T* s1, T* s2, T* t2, T* t3, T* gx, T* gy,
                                            T* gz, T* uq) {
  constexpr int G = HexCfg<N>::G;
  using TB = CTab<T>;
  T* t1 = su;  // alias: u is consumed by stage 1 before t1 is written
  if (active) {
    const int a = pl / N, b = pl % N;
    T u[N], ub[N], ud[N];
#pragma unroll
    for (int c = 0; c < N; c++) u[c] = su[(a * N + b) * N + c];
    eo_fwd<N, T, true, true>(u, ub, ud);
#pragma unroll
    for (int k = 0; k < N; k++) {
      s1[(a * N + b) * N + k] = ub[k];
      s2[(a * N + b) * N + k] = ud[k];
    }
  }
  group_sync<G>(gid);
  if (active) {
    const int a = pl / N, k = pl % N;
    T v1[N], v2[N], bb[N], db[N], bd[N];
#pragma unroll
    for (int b = 0; b < N; b++) { v1[b] = s1[(a * N + b) * N + k]; v2[b] = s2[(a * N + b) * N + k]; }
    eo_fwd<N, T, true, true>(v1, bb, db);
    eo_fwd<N, T, true, false>(v2, bd, nullptr);
#pragma unroll
    for (int j = 0; j < N; j++) {
      t1[(a * N + j) * N + k] = bb[j];
      t2[(a * N + j) * N + k] = db[j];
      t3[(a * N + j) * N + k] = bd[j];
    }
  }
  group_sync<G>(gid);
  if (active) {
    const int j = pl / N, k = pl % N;
    T w1[N], w2[N], w3[N];
#pragma unroll
    for (int a = 0; a < N; a++) {
      w1[a] = t1[(a * N + j) * N + k];
      w2[a] = t2[(a * N + j) * N + k];
      w3[a] = t3[(a * N + j) * N + k];
    }
    eo_fwd<N, T, WANT_U, true>(w1, uq, gx);
    eo_fwd<N, T, true, false>(w2, gy, nullptr);
    eo_fwd<N, T, true, false>(w3, gz, nullptr);
  }
  group_sync<G>(gid);
}

// Transposed chain: lane (j,k) holds vx,vy,vz (and vm) at its qp column ->
// element residual in su[(a*N+b)*N+c].
template <int N, class T, bool WANT_M>
__device__ __forceinline__ void hex_backward(int pl, bool active, int gid, T* su, T* s1, T* s2, T* t2, T* t3,
                                             const T* vx, const T* vy, const T* vz, const T* vm) {
  constexpr int G = HexCfg<N>::G;
  using TB = CTab<T>;
  T* t1 = su;
  if (active) {
    const int j = pl / N, k = pl % N;
    T w1[N], w2[N], w3[N];
    eo_bwd<N, T, true, false>(vx, w1);
    if (WANT_M) eo_bwd<N, T, false, true>(vm, w1);
    eo_bwd<N, T, false, false>(vy, w2);
    eo_bwd<N, T, false, false>(vz, w3);
#pragma unroll
    for (int a = 0; a < N; a++) {
      t1[(a * N + j) * N + k] = w1[a];
      t2[(a * N + j) * N + k] = w2[a];
      t3[(a * N + j) * N + k] = w3[a];
    }
  }
  group_sync<G>(gid);
  if (active) {
    const int a = pl / N, k = pl % N;
    T r1[N], r2[N], r3[N];
#pragma unroll
    for (int j = 0; j < N; j++) {
      r1[j] = t1[(a * N + j) * N + k];
      r2[j] = t2[(a * N + j) * N + k];
      r3[j] = t3[(a * N + j) * N + k];
    }
    T v1[N], v2[N];
    eo_bwd<N, T, false, false>(r1, v1);
    eo_bwd<N, T, true, true>(r2, v1);
    eo_bwd<N, T, false, false>(r3, v2);
#pragma unroll
    for (int b = 0; b < N; b++) {
      s1[(a * N + b) * N + k] = v1[b];
      s2[(a * N + b) * N + k] = v2[b];
    }
  }
  group_sync<G>(gid);
  if (active) {
    const int a = pl / N, b = pl % N;
    T r1[N], r2[N];
#pragma unroll
    for (int k = 0; k < N; k++) { r1[k] = s1[(a * N + b) * N + k]; r2[k] = s2[(a * N + b) * N + k]; }
    T v[N];
    eo_bwd<N, T, false, false>(r1, v);
    eo_bwd<N, T, true, true>(r2, v);
#pragma unroll
    for (int c = 0; c < N; c++) su[(a * N + b) * N + c] = v[c];
  }
  group_sync<G>(gid);
}

// y += A x over all hex elements; optional energy sum_e x_e^T A_e x_e.
// Persistent element groups.  A group works on a chunk of EPW consecutive
// elements at a time (EPW = 1 for p >= 4; low orders pack several elements into
// one warp, N*N lanes each).  Per chunk (DOF-row buffer b):
//   lane 0 bulk-copies (TMA) the DOF-table rows of the NEXT chunk into buffer
//   b^1 (mbarrier T[b^1]);
//   forward contractions;
//   wait for T[b^1] and issue the x gather of the next chunk into registers
//   (the loads complete under the remaining work);
//   [G mode 0: wait for the G tiles of this chunk (mbarrier Gb)] quadrature-
//   point transform, then lane 0 bulk-copies the next chunk's G tiles;
//   transposed contractions and scatter (DOFs >= first_cell belong to one
//   element alone: plain stores, the rest atomic adds).
// skip != NULL: the kernel returns immediately when *skip != 0 (CG finished).
// G modes: 0 = per-point metric tiles bulk-copied to shared memory, 1 = the same
// read directly (coalesced); 2 / 3 = generic B^T D B (bdb.cu, MASS = true): 16
// reference-coordinate coefficients per point, or one record per affine element.
template <int N, class T, bool MASS, int GM>
__global__ void __launch_bounds__(HexCfg<N>::BLOCK)
hex_apply_kernel(int ne, const int* __restrict__ tdof, int tstride, const T* __restrict__ Gq, int gstride,
                 const T* __restrict__ x, T* __restrict__ y, int first_cell, double* partial, unsigned int* counter,
                 double* energy, const int* skip, int* err) {
  using C = HexCfg<N>;
  using SM = HexSmem<N, T>;
  constexpr int N2 = C::N2, N3 = C::N3, G = C::G, EPW = C::EPW, CN3 = EPW * N3;
  constexpr int NG = (CN3 + G - 1) / G;  // gathered values per lane
  if (skip && *(volatile const int*)skip) return;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int gid = threadIdx.x / G, lane = threadIdx.x % G;
  const int slot = lane / N2, pl = lane % N2;  // element slot of this lane and its pencil
  const size_t rowg = round16((size_t)gstride * sizeof(T)), rowt = round16((size_t)tstride * sizeof(int));
  const size_t gb = GM == 0 ? SM::gbytes(gstride) : 0, tb = SM::tbytes(tstride);
  unsigned char* gp = smem_raw + SM::tables + (size_t)gid * SM::group(gstride, tstride, GM);
  T* gbuf = (T*)gp;
  auto tbuf = [&](int b) { return (int*)(gp + gb + b * tb); };  // arithmetic keeps them out of local memory
  T* work = (T*)(gp + gb + 2 * tb);
  const int so = slot < EPW ? slot * N3 : 0;  // this lane's slot offset in the work arrays
  T *su = work + so, *s1 = work + CN3 + so, *s2 = work + 2 * CN3 + so, *t2 = work + 3 * CN3 + so,
    *t3 = work + 4 * CN3 + so;
  uint64_t* mbar = (uint64_t*)(gp + gb + 2 * tb + SM::work);  // [0],[1]: DOF rows, [2]: G tiles
  if (lane == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    mbar_init(&mbar[2], 1);
    fence_mbar_init();
  }
  __syncthreads();
  const int nch = (ne + EPW - 1) / EPW;
  const int stride = gridDim.x * C::EPB;
  int ch = blockIdx.x * C::EPB + gid;
  auto rows_of = [&](int c) { return min(EPW, ne - c * EPW); };
  auto issue_t = [&](int c, int b) {
    const uint32_t bytes = (uint32_t)(rows_of(c) * rowt);
    mbar_expect_tx(&mbar[b], bytes);
    bulk_g2s(tbuf(b), tdof + (size_t)c * EPW * tstride, bytes, &mbar[b]);
  };
  auto issue_g = [&](int c) {
    const uint32_t bytes = (uint32_t)(rows_of(c) * rowg);
    mbar_expect_tx(&mbar[2], bytes);
    bulk_g2s(gbuf, Gq + (size_t)c * EPW * gstride, bytes, &mbar[2]);
  };
  auto gather = [&](int c, const int* tn, T* xr) {
    const int nrow = rows_of(c);
#pragma unroll
    for (int j = 0; j < NG; j++) {
      const int t = lane + j * G;
      xr[j] = 0;
      if (t < CN3 && t / N3 < nrow) {
        const int d = tn[(t / N3) * (int)(rowt / sizeof(int)) + t % N3];
        const T v = __ldg(x + (d & 0x7fffffff));
        xr[j] = d < 0 ? -v : v;
      }
    }
  };
  T xr[NG];   // gathered (signed) coefficients of the chunk about to be computed
  T acc = 0;  // per-lane energy in the working precision (FP64 throughput is scarce)
  int t_issued = 0, t_waited = 0, g_issued = 0, g_waited = 0;
  bool ok = true;
  if (ch < nch) {
    if (lane == 0) {
      issue_t(ch, 0);
      if (GM == 0) issue_g(ch);
    }
    t_issued = 1;
    g_issued = GM == 0 ? 1 : 0;
    ok = group_all<G>(gid, mbar_wait_bounded(&mbar[0], 0));
    if (ok) {
      t_waited = 1;  // a wait counts only once it succeeded: the drain covers the rest
      gather(ch, tbuf(0), xr);
    }
  }
  for (int k = 0; ok && ch < nch; ch += stride, k++) {
    const int b = k & 1;
    const bool has_next = ch + stride < nch;
    const bool active = slot < EPW && ch * EPW + slot < ne;
#pragma unroll
    for (int j = 0; j < NG; j++) {
      const int t = lane + j * G;
      if (t < CN3) work[t] = xr[j];  // su of every slot
    }
    if (lane == 0 && has_next) {
      fence_proxy_async();  // DOF-row buffer b^1 was last read through the generic proxy
      issue_t(ch + stride, b ^ 1);
    }
    if (has_next) t_issued++;
    group_sync<G>(gid);
    T gx[N], gy[N], gz[N], uq[N];
    hex_forward<N, T, MASS>(pl, active, gid, su, s1, s2, t2, t3, gx, gy, gz, uq);
    if (has_next) {
      ok = group_all<G>(gid, mbar_wait_bounded(&mbar[b ^ 1], ((k + 1) >> 1) & 1));
      if (!ok) break;
      t_waited++;
      gather(ch + stride, tbuf(b ^ 1), xr);
    }
    if (GM == 0) {
      ok = group_all<G>(gid, mbar_wait_bounded(&mbar[2], k & 1));
      if (!ok) break;
      g_waited++;
    }
    // G mode 0: the tiles are in shared memory; mode 1: coalesced loads from HBM
    const T* Gsrc = GM == 0 ? (const T*)((const unsigned char*)gbuf + (slot < EPW ? slot : 0) * rowg)
                            : Gq + ((size_t)ch * EPW + (slot < EPW ? slot : 0)) * gstride;
    T vx[N], vy[N], vz[N], vm[N];
    if (active && GM >= 2) {
      // generic B^T D B: (vm, vx, vy, vz) = Mh (uq, gx, gy, gz) at every point;
      // GM 2 streams Mh per point, GM 3 reads one record per element and weights it
      T me[16], wjk = 0;
      if (GM == 3) {
#pragma unroll
        for (int c = 0; c < 16; c++) me[c] = __ldg(Gsrc + c);
        wjk = CTab<T>::W(eo_off(N) + pl / N) * CTab<T>::W(eo_off(N) + pl % N);
      }
#pragma unroll
      for (int i = 0; i < N; i++) {
        const int o = i * N2 + pl;
        T m[16];
        if (GM == 2) {
#pragma unroll
          for (int c = 0; c < 16; c++) m[c] = __ldcs(Gsrc + c * N3 + o);
        } else {
          const T w = CTab<T>::W(eo_off(N) + i) * wjk;
#pragma unroll
          for (int c = 0; c < 16; c++) m[c] = w * me[c];
        }
        const T a0 = uq[i], a1 = gx[i], a2 = gy[i], a3 = gz[i];
        vm[i] = m[0] * a0 + m[1] * a1 + m[2] * a2 + m[3] * a3;
        vx[i] = m[4] * a0 + m[5] * a1 + m[6] * a2 + m[7] * a3;
        vy[i] = m[8] * a0 + m[9] * a1 + m[10] * a2 + m[11] * a3;
        vz[i] = m[12] * a0 + m[13] * a1 + m[14] * a2 + m[15] * a3;
        if (partial) acc += a0 * vm[i] + a1 * vx[i] + a2 * vy[i] + a3 * vz[i];
      }
    } else if (active) {
#pragma unroll
      for (int i = 0; i < N; i++) {
        const int o = i * N2 + pl;
        T gxx, gyy, gzz, gxy, gxz, gyz;
        if (GM == 0) {
          gxx = Gsrc[o]; gyy = Gsrc[N3 + o]; gzz = Gsrc[2 * N3 + o];
          gxy = Gsrc[3 * N3 + o]; gxz = Gsrc[4 * N3 + o]; gyz = Gsrc[5 * N3 + o];
        } else {
          gxx = __ldcs(Gsrc + o); gyy = __ldcs(Gsrc + N3 + o); gzz = __ldcs(Gsrc + 2 * N3 + o);
          gxy = __ldcs(Gsrc + 3 * N3 + o); gxz = __ldcs(Gsrc + 4 * N3 + o); gyz = __ldcs(Gsrc + 5 * N3 + o);
        }
        vx[i] = gxx * gx[i] + gxy * gy[i] + gxz * gz[i];
        vy[i] = gxy * gx[i] + gyy * gy[i] + gyz * gz[i];
        vz[i] = gxz * gx[i] + gyz * gy[i] + gzz * gz[i];
        if (MASS) vm[i] = (GM == 0 ? Gsrc[6 * N3 + o] : __ldcs(Gsrc + 6 * N3 + o)) * uq[i];
        if (partial) {  // x^T A x only when the caller asks for it (CG)
          T en = gx[i] * vx[i] + gy[i] * vy[i] + gz[i] * vz[i];
          if (MASS) en += uq[i] * vm[i];
          acc += en;
        }
      }
    }
    if (GM == 0) {
      group_sync<G>(gid);  // everyone is done with the G tiles
      if (lane == 0 && has_next) {
        fence_proxy_async();
        issue_g(ch + stride);
      }
      if (has_next) g_issued++;
    }
    hex_backward<N, T, MASS>(pl, active, gid, su, s1, s2, t2, t3, vx, vy, vz, vm);
    const int* td = tbuf(b);
    const int nrow = rows_of(ch);
    for (int t = lane; t < CN3; t += G) {
      if (t / N3 >= nrow) continue;
      const int d = td[(t / N3) * (int)(rowt / sizeof(int)) + t % N3];
      const int dof = d & 0x7fffffff;
      const T v = d < 0 ? -work[t] : work[t];
      if (dof >= first_cell) y[dof] = v;  // element-interior DOF: single writer
      else atomic_add_t(y + dof, v);
    }
    group_sync<G>(gid);
  }
  if (!ok) {
    // record the failure, then give the copies still in flight a bounded chance
    // to land before the block (and its shared memory) retires
    if (lane == 0) {
      atomicExch(err, 1);
      for (int j = t_waited; j < t_issued; j++) mbar_wait_bounded(&mbar[j & 1], (j >> 1) & 1);
      for (int j = g_waited; j < g_issued; j++) mbar_wait_bounded(&mbar[2], j & 1);
    }
    group_sync<G>(gid);
  }
  if (partial) block_reduce_finish((double)acc, partial, counter, energy);
}

// ---------------------------------------------------------------------------
// host drivers
// raises the dynamic shared-memory limit of one instantiation (once) and
// returns its resident blocks per SM for a given shared-memory size; called at
// setup, outside any stream capture, and cached in the operator
template <int N, class T, bool MASS, int GM>
int hex_apply_occupancy(size_t smem) {
  static bool attr = false;
  auto kern = hex_apply_kernel<N, T, MASS, GM>;
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
  GH1_CHECK(v >= 1, GH1_ERR_UNSUPPORTED, "hex apply does not fit on an SM (shared memory)");
  return v;
}

template <int N, class T, bool MASS, int GM>
void launch_hex_apply(gh1_op* op, const T* x, T* y, const T* G, int gstride, double* partial, unsigned int* counter,
                      double* energy, const int* skip) {
  using C = HexCfg<N>;
  gh1_space* sp = op->sp;
  const size_t smem = HexSmem<N, T>::total(gstride, sp->tstride, GM);
  const int pi = std::is_same<T, float>::value ? 1 : 0;
  const int per_sm = GM >= 2 ? op->bdb_per_sm[pi] : op->hex_per_sm[pi][GM];
  GH1_CHECK(per_sm > 0, GH1_ERR_ARG, "internal: hex apply occupancy not prepared");
  const int ne = sp->mesh->ne;
  const int nch = (ne + C::EPW - 1) / C::EPW;
  const int blocks_needed = (nch + C::EPB - 1) / C::EPB;
  const int grid = std::min(blocks_needed, sp->ctx->nsm * per_sm);
  hex_apply_kernel<N, T, MASS, GM><<<grid, C::BLOCK, smem, sp->ctx->stream>>>(
      ne, sp->d_tdof.p, sp->tstride, G, gstride, x, y, (int)sp->first_cell, partial, counter, energy, skip, op->d_err.p);
  check_kernel(sp->ctx, "hex_apply_kernel");
}

}  // namespace gh1
