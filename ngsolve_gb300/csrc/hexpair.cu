// hexpair.cu -- FP32 hex apply y += A x with two elements per lane.
//
// Same operator and algorithm as hex_apply_kernel (matfree.cu: sum-factorized
// SymbolicBFI::ApplyElementMatrix, fem/symbolicintegrator.cpp:2959-3040, with the
// per-point coefficient tile G_q = kappa w |det J| J^{-1} J^{-T}), restructured
// for the packed FP32 pipe of sm_103a: a lane owns the same pencil of TWO
// consecutive elements and keeps both values in one 64-bit register, so every
// contraction step is one fma.rn.f32x2 for two elements, every work-array access
// one 8-byte shared-memory access for two elements, and the loop / address /
// barrier overhead of the element loop is paid once per pair.  The FP32 apply is
// instruction-issue bound in the one-element form; this halves the arithmetic
// and shared-memory instruction count per element.
//
// Layout per element group (G threads, S = HexCfg::EPW pencil slots, E = 2 S
// elements per chunk, element 2s+h of a chunk in slot s, half h):
//   [G tiles of the E elements (G mode 0)] | DOF-table rows x2 buffers |
//   6 packed work arrays of float2 (u dense, s and t padded, see PairLayout) |
//   3 mbarriers
// Pipelining as in the one-element kernel: the DOF rows of the next chunk are
// bulk-copied (TMA) during the forward contractions, the next chunk's x gather
// is issued before the quadrature-point transform, and in G mode 0 the G tiles
// of the next chunk are bulk-copied during the transposed contractions.
// Every mbarrier wait is bounded; a timeout sets *err and the kernel drains its
// copies in flight and returns.
#include <algorithm>
#include <cstdlib>
#include <vector>
#include "common.cuh"
#include "hexcore.cuh"

namespace gh1 {

typedef unsigned long long f2;  // packed pair: low half element 2s, high half element 2s+1

__device__ __forceinline__ f2 pack2(float lo, float hi) {
  f2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void unpack2(f2 v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
  f2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
  f2 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2 add2(f2 a, f2 b) {
  f2 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}

// Poll limit of the paired apply's first mbarrier wait.  The default is the
// bound of every other wait (2^22 polls); GH1_FIRST_WAIT_POLLS read at operator
// setup lowers it so that a test can make that wait run out on purpose: the
// kernel then sets the operator's error flag, drains its copies in flight with
// the full bound and returns, and the host reports GH1_ERR_CUDA.
__device__ int g_first_wait_polls = 1 << 22;

void set_first_wait_polls() {
  const char* env = getenv("GH1_FIRST_WAIT_POLLS");
  const int v = env ? std::max(0, atoi(env)) : (1 << 22);
  GH1_CUDA(cudaMemcpyToSymbol(g_first_wait_polls, &v, sizeof(int)));
}

// 1D factor tables (32-bit); a coefficient enters the packed FMA broadcast to
// both halves, which the packed pipe takes from the constant bank at no extra
// instruction (a table of pre-duplicated 64-bit pairs costs a move per FMA)
__constant__ float c_Bp[TAB_TOTAL], c_Dp[TAB_TOTAL];
// 1D Gauss weights of every order: N weights at offset N(N-1)/2 - 1
__constant__ float c_Wp[64];
__device__ __forceinline__ f2 bcast(float t) {
  f2 r;
  asm("mov.b64 %0, {%1, %1};" : "=l"(r) : "f"(t));
  return r;
}
__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
  f2 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
// t (+)= c x: the first term of an unrolled sum starts it with a multiply
__device__ __forceinline__ f2 mac2(bool first, float c, f2 x, f2 t) { return first ? mul2(bcast(c), x) : fma2(bcast(c), x, t); }

// Even-odd coefficients of the vertex pair, (B[q][0] +- B[q][1]) / 2 and
// (D[q][0] +- D[q][1]) / 2 at offset eo_off(N): the packed contractions below use
// the reflection symmetry of the 1D tables on the Gauss points (psi_0 <-> psi_1,
// psi_c -> (-1)^c psi_c under x -> 1-x; checked when the tables are uploaded), so
// B u at the points q and N-1-q is (even part) +- (odd part) and every 1D
// contraction takes about a third fewer packed FMAs at N = 5.
__constant__ float c_EOp[4][64];

// ob[q] = sum_c B[q][c] u[c], od[q] = sum_c D[q][c] u[c] (either may be skipped)
template <int N, bool WB, bool WD>
__device__ __forceinline__ void eo2_fwd(const f2* u, f2* ob, f2* od) {
  constexpr int O = tab_off(N), W = eo_off(N), M = N / 2;
  const f2 s = add2(u[0], u[1]), d = sub2(u[0], u[1]);
#pragma unroll
  for (int q = 0; q < M; q++) {
    f2 eb = 0, obb = 0, ed = 0, odd = 0;
    if (WB) { eb = mul2(bcast(c_EOp[0][W + q]), s); obb = mul2(bcast(c_EOp[1][W + q]), d); }
    if (WD) { ed = mul2(bcast(c_EOp[2][W + q]), s); odd = mul2(bcast(c_EOp[3][W + q]), d); }
#pragma unroll
    for (int c = 2; c < N; c++) {
      if (c % 2 == 0) {
        if (WB) eb = fma2(bcast(c_Bp[O + q * N + c]), u[c], eb);
        if (WD) ed = fma2(bcast(c_Dp[O + q * N + c]), u[c], ed);
      } else {
        if (WB) obb = fma2(bcast(c_Bp[O + q * N + c]), u[c], obb);
        if (WD) odd = fma2(bcast(c_Dp[O + q * N + c]), u[c], odd);
      }
    }
    if (WB) { ob[q] = add2(eb, obb); ob[N - 1 - q] = sub2(eb, obb); }
    if (WD) { od[q] = add2(ed, odd); od[N - 1 - q] = sub2(odd, ed); }
  }
  if (N % 2 == 1) {  // middle point: B keeps its even part, D its odd part
    constexpr int q = M;
    f2 eb = 0, odd = 0;
    if (WB) eb = mul2(bcast(c_EOp[0][W + q]), s);
    if (WD) odd = mul2(bcast(c_EOp[3][W + q]), d);
#pragma unroll
    for (int c = 2; c < N; c++) {
      if (c % 2 == 0) { if (WB) eb = fma2(bcast(c_Bp[O + q * N + c]), u[c], eb); }
      else { if (WD) odd = fma2(bcast(c_Dp[O + q * N + c]), u[c], odd); }
    }
    if (WB) ob[q] = eb;
    if (WD) od[q] = odd;
  }
}

// out[a] (+)= sum_q B[q][a] v[q] (WANT_D false) or sum_q D[q][a] v[q] (WANT_D true)
template <int N, bool WANT_D, bool ACC>
__device__ __forceinline__ void eo2_bwd(const f2* v, f2* out) {
  constexpr int O = tab_off(N), W = eo_off(N), M = N / 2;
  f2 vs[M > 0 ? M : 1], vd[M > 0 ? M : 1];
#pragma unroll
  for (int k = 0; k < M; k++) { vs[k] = add2(v[k], v[N - 1 - k]); vd[k] = sub2(v[k], v[N - 1 - k]); }
  // a = 0, 1: out[0] = P + Q, out[1] = P - Q
  f2 P = 0, Q = 0;
#pragma unroll
  for (int k = 0; k < M; k++) {
    if (!WANT_D) { P = mac2(k == 0, c_EOp[0][W + k], vs[k], P); Q = mac2(k == 0, c_EOp[1][W + k], vd[k], Q); }
    else { P = mac2(k == 0, c_EOp[2][W + k], vd[k], P); Q = mac2(k == 0, c_EOp[3][W + k], vs[k], Q); }
  }
  if (N % 2 == 1) {
    if (!WANT_D) P = mac2(M == 0, c_Bp[O + M * N], v[M], P);
    else Q = mac2(M == 0, c_Dp[O + M * N], v[M], Q);
  }
  out[0] = ACC ? add2(out[0], add2(P, Q)) : add2(P, Q);
  out[1] = ACC ? add2(out[1], sub2(P, Q)) : sub2(P, Q);
#pragma unroll
  for (int a = 2; a < N; a++) {
    // B: even a takes vs (and the middle point), odd a takes vd; D: the reverse
    const bool sym = WANT_D ? (a % 2 == 1) : (a % 2 == 0);
    f2 t = ACC ? out[a] : (f2)0;
#pragma unroll
    for (int k = 0; k < M; k++)
      t = mac2(!ACC && k == 0, WANT_D ? c_Dp[O + k * N + a] : c_Bp[O + k * N + a], sym ? vs[k] : vd[k], t);
    if (N % 2 == 1 && sym) t = mac2(!ACC && M == 0, WANT_D ? c_Dp[O + M * N + a] : c_Bp[O + M * N + a], v[M], t);
    out[a] = t;
  }
}

// resident blocks per SM the register allocation must allow, measured per
// variant (p=4: 4 blocks = 128 registers with the G tile in shared memory or a
// metric per element, 5 blocks = 96 with direct G loads; p=6: 3 blocks = 168)
constexpr int pair_min_blocks(int N, bool mass, int gm) {
  return gm == 4 ? (N <= 5 ? 4 : 2) : gm == 3 ? (N <= 4 ? 4 : N == 5 ? 3 : 2)  // B^T D B records: 16 packed coefficients in registers
         : N == 2 ? 6
         : N == 3 ? (mass ? (gm ? 5 : 4) : (gm ? 6 : 5))
         : N == 4 ? (mass ? (gm ? 5 : 4) : 5)
         : N == 5 ? (mass ? (gm ? 4 : 3) : (gm == 1 ? 5 : 4))
         : N == 6 ? 2
                  : (mass && gm == 0 ? 2 : 3);
}

// Even-odd (reflection) form of the 1D contractions, per order and metric mode,
// as measured on the 1-16 M DOF operators: it takes about a third fewer packed
// FMAs and pays where the kernel is issue-bound (p=4 with a metric per element
// or a staged G tile, p >= 5); the per-point metric loaded directly at p <= 4 runs
// faster with the plain form.
constexpr bool pair_eo(int N, int GM) {
  return N == 3 ? GM == 0 : N == 4 ? GM != 2 : N == 5 ? GM != 1 : true;
}

// Work-array layouts.  Element index (a,b,c) sits at a*SA + b*SB + c in the s
// arrays (stage-1 outputs) and at a*TA + b*TB + c in the t arrays (stage-2
// outputs); the coefficient array u is dense.  Each stage reads and writes
// 8-byte words with one of three lane patterns (lanes over (a,b), (a,c) or
// (b,c)).  At N = 5 no single padding serves all three conflict-free, but
// per-array paddings do: SA, SB = 35, 7 and TA, TB = 27, 5 with the stage-2 lanes
// permuted by c_p2 leave every access at the minimum of two wavefronts per warp
// (dense layout: three for the stage-2 pattern).  Other orders stay dense.
template <int N>
struct PairLayout {
  static constexpr int SA = N == 5 ? 35 : N * N, SB = N == 5 ? 7 : N;
  static constexpr int TA = N == 5 ? 27 : N * N, TB = N;
  static constexpr int SW = (N - 1) * (SA + SB) + N, TW = (N - 1) * (TA + TB) + N;  // words per array
};
// stage-2 lane -> (a, c) = (v / 5, v % 5) at N = 5: lanes 0-15 and 16-24 each hit
// 16 (9) distinct bank pairs in both the s and the t layout
__constant__ unsigned char c_p2[25] = {0, 1, 2, 4, 5, 7, 10, 11, 12, 13, 14, 17, 19, 20, 22, 23,
                                       3, 6, 8, 9, 15, 16, 18, 21, 24};

template <int N>
struct PairCfg {
  static constexpr int N2 = N * N, N3 = N * N * N;
  static constexpr int G = HexCfg<N>::G;      // threads per element group
  static constexpr int S = HexCfg<N>::EPW;    // pencil slots per group
  static constexpr int E = 2 * S;             // elements per chunk
  static constexpr int EPB = HexCfg<N>::EPB;  // groups per block
  static constexpr int BLOCK = G * EPB;
  static constexpr int NG = (S * N3 + G - 1) / G;  // (slot, local DOF) positions per lane
  static __host__ __device__ size_t gbytes(int gstride) { return E * round16((size_t)gstride * sizeof(float)); }
  static __host__ __device__ size_t tbytes(int tstride) { return E * round16((size_t)tstride * sizeof(int)); }
  // u (dense), s1, s2 (layout S), t1, t2, t3 (layout T), per slot; 16-byte rounded
  static constexpr size_t work =
      round16((size_t)S * (N3 + 2 * PairLayout<N>::SW + 3 * PairLayout<N>::TW) * sizeof(f2));
  static __host__ __device__ size_t group(int gstride, int tstride, int gmode) {
    return (gmode == 0 ? gbytes(gstride) : 0) + 2 * tbytes(tstride) + work + 32;
  }
  static __host__ __device__ size_t total(int gstride, int tstride, int gmode) {
    return (size_t)EPB * group(gstride, tstride, gmode);
  }
};

// forward chain on packed pairs (see hex_forward in matfree.cu): coefficients in
// su[(a*N+b)*N+c] -> reference gradient at the points of lane (j,k).  (pa, pk):
// this lane's stage-2 pair.  EO: the 1D contractions in even-odd form.
template <int N, bool WANT_U, bool EO>
__device__ __forceinline__ void pair_forward(int pl, int pa, int pk, bool active, int gid, const f2* su, f2* s1, f2* s2,
                                             f2* t1, f2* t2, f2* t3, f2* gx, f2* gy, f2* gz, f2* uq) {
  constexpr int G = HexCfg<N>::G, O = tab_off(N);
  using L = PairLayout<N>;
  if (active) {
    const int a = pl / N, b = pl % N;
    f2 u[N];
#pragma unroll
    for (int c = 0; c < N; c++) u[c] = su[(a * N + b) * N + c];
    if constexpr (EO) {
      f2 ub[N], ud[N];
      eo2_fwd<N, true, true>(u, ub, ud);
#pragma unroll
      for (int k = 0; k < N; k++) {
        s1[a * L::SA + b * L::SB + k] = ub[k];
        s2[a * L::SA + b * L::SB + k] = ud[k];
      }
    } else {
#pragma unroll
      for (int k = 0; k < N; k++) {
        f2 ub = mul2(bcast(c_Bp[O + k * N]), u[0]), ud = mul2(bcast(c_Dp[O + k * N]), u[0]);
#pragma unroll
        for (int c = 1; c < N; c++) {
          ub = fma2(bcast(c_Bp[O + k * N + c]), u[c], ub);
          ud = fma2(bcast(c_Dp[O + k * N + c]), u[c], ud);
        }
        s1[a * L::SA + b * L::SB + k] = ub;
        s2[a * L::SA + b * L::SB + k] = ud;
      }
    }
  }
  group_sync<G>(gid);
  if (active) {
    const int a = pa, k = pk;
    f2 v1[N], v2[N];
#pragma unroll
    for (int b = 0; b < N; b++) { v1[b] = s1[a * L::SA + b * L::SB + k]; v2[b] = s2[a * L::SA + b * L::SB + k]; }
    if constexpr (EO) {
      f2 bb[N], db[N], bd[N];
      eo2_fwd<N, true, true>(v1, bb, db);
      eo2_fwd<N, true, false>(v2, bd, nullptr);
#pragma unroll
      for (int j = 0; j < N; j++) {
        t1[a * L::TA + j * L::TB + k] = bb[j];
        t2[a * L::TA + j * L::TB + k] = db[j];
        t3[a * L::TA + j * L::TB + k] = bd[j];
      }
    } else {
#pragma unroll
      for (int j = 0; j < N; j++) {
        f2 bb = mul2(bcast(c_Bp[O + j * N]), v1[0]), db = mul2(bcast(c_Dp[O + j * N]), v1[0]), bd = mul2(bcast(c_Bp[O + j * N]), v2[0]);
#pragma unroll
        for (int b = 1; b < N; b++) {
          bb = fma2(bcast(c_Bp[O + j * N + b]), v1[b], bb);
          db = fma2(bcast(c_Dp[O + j * N + b]), v1[b], db);
          bd = fma2(bcast(c_Bp[O + j * N + b]), v2[b], bd);
        }
        t1[a * L::TA + j * L::TB + k] = bb;
        t2[a * L::TA + j * L::TB + k] = db;
        t3[a * L::TA + j * L::TB + k] = bd;
      }
    }
  }
  group_sync<G>(gid);
  if (active) {
    const int j = pl / N, k = pl % N;
    f2 w1[N], w2[N], w3[N];
#pragma unroll
    for (int a = 0; a < N; a++) {
      w1[a] = t1[a * L::TA + j * L::TB + k];
      w2[a] = t2[a * L::TA + j * L::TB + k];
      w3[a] = t3[a * L::TA + j * L::TB + k];
    }
    if constexpr (EO) {
      eo2_fwd<N, WANT_U, true>(w1, uq, gx);
      eo2_fwd<N, true, false>(w2, gy, nullptr);
      eo2_fwd<N, true, false>(w3, gz, nullptr);
    } else {
#pragma unroll
      for (int i = 0; i < N; i++) {
        f2 x = mul2(bcast(c_Dp[O + i * N]), w1[0]), y = mul2(bcast(c_Bp[O + i * N]), w2[0]), z = mul2(bcast(c_Bp[O + i * N]), w3[0]);
        f2 uu = 0;
        if (WANT_U) uu = mul2(bcast(c_Bp[O + i * N]), w1[0]);
#pragma unroll
        for (int a = 1; a < N; a++) {
          x = fma2(bcast(c_Dp[O + i * N + a]), w1[a], x);
          y = fma2(bcast(c_Bp[O + i * N + a]), w2[a], y);
          z = fma2(bcast(c_Bp[O + i * N + a]), w3[a], z);
          if (WANT_U) uu = fma2(bcast(c_Bp[O + i * N + a]), w1[a], uu);
        }
        gx[i] = x; gy[i] = y; gz[i] = z;
        if (WANT_U) uq[i] = uu;
      }
    }
  }
  group_sync<G>(gid);
}

// transposed chain on packed pairs (see hex_backward in matfree.cu)
template <int N, bool WANT_M, bool EO>
__device__ __forceinline__ void pair_backward(int pl, int pa, int pk, bool active, int gid, f2* su, f2* s1, f2* s2,
                                              f2* t1, f2* t2, f2* t3, const f2* vx, const f2* vy, const f2* vz,
                                              const f2* vm) {
  constexpr int G = HexCfg<N>::G, O = tab_off(N);
  using L = PairLayout<N>;
  if (active) {
    const int j = pl / N, k = pl % N;
    if constexpr (EO) {
      f2 w[N];
      eo2_bwd<N, true, false>(vx, w);
      if (WANT_M) eo2_bwd<N, false, true>(vm, w);
#pragma unroll
      for (int a = 0; a < N; a++) t1[a * L::TA + j * L::TB + k] = w[a];
      eo2_bwd<N, false, false>(vy, w);
#pragma unroll
      for (int a = 0; a < N; a++) t2[a * L::TA + j * L::TB + k] = w[a];
      eo2_bwd<N, false, false>(vz, w);
#pragma unroll
      for (int a = 0; a < N; a++) t3[a * L::TA + j * L::TB + k] = w[a];
    } else {
#pragma unroll
      for (int a = 0; a < N; a++) {
        f2 w1 = mul2(bcast(c_Dp[O + a]), vx[0]), w2 = mul2(bcast(c_Bp[O + a]), vy[0]), w3 = mul2(bcast(c_Bp[O + a]), vz[0]);
        if (WANT_M) w1 = fma2(bcast(c_Bp[O + a]), vm[0], w1);
#pragma unroll
        for (int i = 1; i < N; i++) {
          w1 = fma2(bcast(c_Dp[O + i * N + a]), vx[i], w1);
          if (WANT_M) w1 = fma2(bcast(c_Bp[O + i * N + a]), vm[i], w1);
          w2 = fma2(bcast(c_Bp[O + i * N + a]), vy[i], w2);
          w3 = fma2(bcast(c_Bp[O + i * N + a]), vz[i], w3);
        }
        t1[a * L::TA + j * L::TB + k] = w1;
        t2[a * L::TA + j * L::TB + k] = w2;
        t3[a * L::TA + j * L::TB + k] = w3;
      }
    }
  }
  group_sync<G>(gid);
  if (active) {
    const int a = pa, k = pk;
    f2 r1[N], r2[N], r3[N];
#pragma unroll
    for (int j = 0; j < N; j++) {
      r1[j] = t1[a * L::TA + j * L::TB + k];
      r2[j] = t2[a * L::TA + j * L::TB + k];
      r3[j] = t3[a * L::TA + j * L::TB + k];
    }
    if constexpr (EO) {
      f2 v[N];
      eo2_bwd<N, false, false>(r1, v);
      eo2_bwd<N, true, true>(r2, v);
#pragma unroll
      for (int b = 0; b < N; b++) s1[a * L::SA + b * L::SB + k] = v[b];
      eo2_bwd<N, false, false>(r3, v);
#pragma unroll
      for (int b = 0; b < N; b++) s2[a * L::SA + b * L::SB + k] = v[b];
    } else {
#pragma unroll
      for (int b = 0; b < N; b++) {
        f2 v1 = mul2(bcast(c_Bp[O + b]), r1[0]), v2 = mul2(bcast(c_Bp[O + b]), r3[0]);
        v1 = fma2(bcast(c_Dp[O + b]), r2[0], v1);
#pragma unroll
        for (int j = 1; j < N; j++) {
          v1 = fma2(bcast(c_Bp[O + j * N + b]), r1[j], v1);
          v1 = fma2(bcast(c_Dp[O + j * N + b]), r2[j], v1);
          v2 = fma2(bcast(c_Bp[O + j * N + b]), r3[j], v2);
        }
        s1[a * L::SA + b * L::SB + k] = v1;
        s2[a * L::SA + b * L::SB + k] = v2;
      }
    }
  }
  group_sync<G>(gid);
  if (active) {
    const int a = pl / N, b = pl % N;
    f2 r1[N], r2[N];
#pragma unroll
    for (int k = 0; k < N; k++) { r1[k] = s1[a * L::SA + b * L::SB + k]; r2[k] = s2[a * L::SA + b * L::SB + k]; }
    if constexpr (EO) {
      f2 v[N];
      eo2_bwd<N, false, false>(r1, v);
      eo2_bwd<N, true, true>(r2, v);
#pragma unroll
      for (int c = 0; c < N; c++) su[(a * N + b) * N + c] = v[c];
    } else {
#pragma unroll
      for (int c = 0; c < N; c++) {
        f2 v = mul2(bcast(c_Bp[O + c]), r1[0]);
        v = fma2(bcast(c_Dp[O + c]), r2[0], v);
#pragma unroll
        for (int k = 1; k < N; k++) {
          v = fma2(bcast(c_Bp[O + k * N + c]), r1[k], v);
          v = fma2(bcast(c_Dp[O + k * N + c]), r2[k], v);
        }
        su[(a * N + b) * N + c] = v;
      }
    }
  }
  group_sync<G>(gid);
}

// GM: 0 = per-point G tile bulk-copied into shared memory, 1 = per-point G rows
// loaded directly (after a bulk L2 prefetch), 2 = one metric record per affine
// element (8 floats: G and the mass coefficient), 3 = the generic B^T D B form
// with one 16-float record per affine element (the reference-coordinate 4x4
// matrix Mh of bdb.cu, row = test component (v, d/dxi, d/deta, d/dzeta), column =
// trial component; MASS = true), the rule weight applied in the kernel; 4 = the
// generic form with a 16-float record per rule point (weights included; rows of
// N^3 values per element, loaded directly after a bulk L2 prefetch).
template <int N, bool MASS, int GM>
__global__ void __launch_bounds__(PairCfg<N>::BLOCK, pair_min_blocks(N, MASS, GM))
hex_apply_pair_kernel(int ne, const int* __restrict__ tdof, int tstride, const float* __restrict__ Gq, int gstride,
                      const float* __restrict__ x, float* __restrict__ y, int first_cell, double* partial,
                      unsigned int* counter, double* energy, const int* skip, int* err) {
  using C = PairCfg<N>;
  constexpr int N2 = C::N2, N3 = C::N3, G = C::G, S = C::S, E = C::E, SN3 = S * N3, NG = C::NG;
  if (skip && *(volatile const int*)skip) return;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int gid = threadIdx.x / G, lane = threadIdx.x % G;
  const int slot = lane / N2, pl = lane % N2;
  const int rowg = (int)(round16((size_t)gstride * sizeof(float)) / sizeof(float));  // floats per G row
  const int rowt = (int)(round16((size_t)tstride * sizeof(int)) / sizeof(int));       // ints per DOF row
  const size_t gb = GM == 0 ? C::gbytes(gstride) : 0, tb = C::tbytes(tstride);
  unsigned char* gp = smem_raw + (size_t)gid * C::group(gstride, tstride, GM);
  float* gbuf = (float*)gp;
  auto tbuf = [&](int b) { return (int*)(gp + gb + b * tb); };
  f2* work = (f2*)(gp + gb + 2 * tb);
  using LY = PairLayout<N>;
  const int sl = slot < S ? slot : 0;  // this lane's slot (inactive lanes alias slot 0)
  f2* su = work + sl * N3;             // gathered x on entry, local residual on exit
  f2* s1 = work + S * N3 + sl * LY::SW;
  f2* s2 = s1 + S * LY::SW;
  f2* t1 = work + S * N3 + 2 * S * LY::SW + sl * LY::TW;
  f2* t2 = t1 + S * LY::TW;
  f2* t3 = t2 + S * LY::TW;
  int pa = pl / N, pk = pl % N;  // stage-2 lane pair
  if (N == 5) {
    const int v = c_p2[pl];
    pa = v / 5;
    pk = v % 5;
  }
  uint64_t* mbar = (uint64_t*)(gp + gb + 2 * tb + C::work);  // [0],[1]: DOF rows, [2]: G tiles
  if (lane == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    mbar_init(&mbar[2], 1);
    fence_mbar_init();
  }
  __syncthreads();
  const int nch = (ne + E - 1) / E;
  const int stride = gridDim.x * C::EPB;
  int ch = blockIdx.x * C::EPB + gid;
  auto rows_of = [&](int c) { return min(E, ne - c * E); };
  auto issue_t = [&](int c, int b) {
    const uint32_t bytes = (uint32_t)(rows_of(c) * rowt * sizeof(int));
    mbar_expect_tx(&mbar[b], bytes);
    bulk_g2s(tbuf(b), tdof + (size_t)c * E * tstride, bytes, &mbar[b]);
  };
  auto issue_g = [&](int c) {
    const uint32_t bytes = (uint32_t)(rows_of(c) * rowg * sizeof(float));
    mbar_expect_tx(&mbar[2], bytes);
    bulk_g2s(gbuf, Gq + (size_t)c * E * gstride, bytes, &mbar[2]);
  };
  // gathered pairs of the chunk: position t = s*N3 + l -> (element 2s, 2s+1; local DOF l).
  // Plain loads only: nothing consumes them until the chunk starts (put_x), so the
  // gather latency overlaps the rest of the current chunk.  The shape signs (bit 31
  // of the DOF rows) go to sg: bits 2j and 2j+1 for the two halves of position j.
  auto gather = [&](int c, const int* tn, f2* xr, unsigned& sg) {
    const int nrow = rows_of(c);
    sg = 0u;
#pragma unroll
    for (int j = 0; j < NG; j++) {
      const int t = lane + j * G;
      float v0 = 0.f, v1 = 0.f;
      if (t < SN3) {
        const int s = t / N3, l = t % N3;
        if (2 * s < nrow) {
          const unsigned d = (unsigned)tn[(2 * s) * rowt + l];
          v0 = __ldg(x + (d & 0x7fffffffu));
          sg |= (d >> 31) << (2 * j);
        }
        if (2 * s + 1 < nrow) {
          const unsigned d = (unsigned)tn[(2 * s + 1) * rowt + l];
          v1 = __ldg(x + (d & 0x7fffffffu));
          sg |= (d >> 31) << (2 * j + 1);
        }
      }
      xr[j] = pack2(v0, v1);
    }
  };
  // signed coefficients into the work array
  auto put_x = [&](const f2* xr, unsigned sg) {
#pragma unroll
    for (int j = 0; j < NG; j++) {
      const int t = lane + j * G;
      if (t < SN3)
        work[t] = xr[j] ^ (((f2)((sg >> (2 * j + 1)) & 1u) << 63) | ((f2)((sg >> (2 * j)) & 1u) << 31));
    }
  };
  f2 xr[NG];
  unsigned xs = 0u;
  f2 acc = 0;  // per-lane energy of both elements (working precision)
  const bool want_e = partial != nullptr;
  int t_issued = 0, t_waited = 0, g_issued = 0, g_waited = 0;
  bool ok = true;
  if (ch < nch) {
    if (lane == 0) {
      issue_t(ch, 0);
      if (GM == 0) issue_g(ch);
      else if (GM == 1 || GM == 4) bulk_prefetch_l2(Gq + (size_t)ch * E * gstride, (uint32_t)(rows_of(ch) * rowg * sizeof(float)));
    }
    t_issued = 1;
    g_issued = GM == 0 ? 1 : 0;
    // the first wait may be shortened (GH1_FIRST_WAIT_POLLS) to test the timeout path
    ok = group_all<G>(gid, mbar_wait_polls(&mbar[0], 0, g_first_wait_polls));
    if (ok) {
      t_waited = 1;  // a wait counts only once it succeeded: the drain covers the rest
      gather(ch, tbuf(0), xr, xs);
    }
  }
  for (int k = 0; ok && ch < nch; ch += stride, k++) {
    const int b = k & 1;
    const bool has_next = ch + stride < nch;
    const int e0 = ch * E + 2 * slot;  // first element of this lane's pair
    const bool active = slot < S && e0 < ne;
    const bool second = active && e0 + 1 < ne;
    put_x(xr, xs);
    if (lane == 0 && has_next) {
      fence_proxy_async();
      issue_t(ch + stride, b ^ 1);
      // G mode 1 reads the next chunk's G rows with plain loads: stage them in L2 now
      if (GM == 1 || GM == 4) bulk_prefetch_l2(Gq + (size_t)(ch + stride) * E * gstride, (uint32_t)(rows_of(ch + stride) * rowg * sizeof(float)));
    }
    if (has_next) t_issued++;
    group_sync<G>(gid);
    f2 gx[N], gy[N], gz[N], uq[N];
    pair_forward<N, MASS, pair_eo(N, GM)>(pl, pa, pk, active, gid, su, s1, s2, t1, t2, t3, gx, gy, gz, uq);
    if (has_next) {
      ok = group_all<G>(gid, mbar_wait_bounded(&mbar[b ^ 1], ((k + 1) >> 1) & 1));
      if (!ok) break;
      t_waited++;
      gather(ch + stride, tbuf(b ^ 1), xr, xs);
    }
    if (GM == 0) {
      ok = group_all<G>(gid, mbar_wait_bounded(&mbar[2], k & 1));
      if (!ok) break;
      g_waited++;
    }
    // G rows of the pair; a missing second element reuses the first row (its
    // gathered coefficients are zero, so its half stays zero and finite)
    const int r0 = active ? 2 * slot : 0, r1 = second ? r0 + 1 : r0;
    const float* Ga = GM == 0 ? gbuf + (size_t)r0 * rowg : Gq + ((size_t)ch * E + r0) * gstride;
    const float* Gb = GM == 0 ? gbuf + (size_t)r1 * rowg : Gq + ((size_t)ch * E + r1) * gstride;
    f2 vx[N], vy[N], vz[N], vm[N];
    if (GM == 4 && active) {
      // (vm, vx, vy, vz) = Mh_q (uq, gx, gy, gz) with a record per point (weights
      // included): 16 rows of N^3 values per element, loaded directly
#pragma unroll
      for (int i = 0; i < N; i++) {
        const int o = i * N2 + pl;
        f2 mq[16];
#pragma unroll
        for (int c = 0; c < 16; c++) mq[c] = pack2(__ldcs(Ga + c * N3 + o), __ldcs(Gb + c * N3 + o));
        const f2 a0 = uq[i], a1 = gx[i], a2 = gy[i], a3 = gz[i];
        vm[i] = fma2(mq[3], a3, fma2(mq[2], a2, fma2(mq[1], a1, mul2(mq[0], a0))));
        vx[i] = fma2(mq[7], a3, fma2(mq[6], a2, fma2(mq[5], a1, mul2(mq[4], a0))));
        vy[i] = fma2(mq[11], a3, fma2(mq[10], a2, fma2(mq[9], a1, mul2(mq[8], a0))));
        vz[i] = fma2(mq[15], a3, fma2(mq[14], a2, fma2(mq[13], a1, mul2(mq[12], a0))));
        if (want_e) acc = add2(acc, fma2(a0, vm[i], fma2(a3, vz[i], fma2(a2, vy[i], mul2(a1, vx[i])))));
      }
    } else if (GM == 3 && active) {
      // (vm, vx, vy, vz) = w_i w_j w_k Mh (uq, gx, gy, gz) with one Mh per element
      constexpr int WO = N * (N - 1) / 2 - 1;
      f2 em[16];
      const float4* Ea = (const float4*)(Gq + ((size_t)ch * E + r0) * 16);
      const float4* Eb = (const float4*)(Gq + ((size_t)ch * E + r1) * 16);
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const float4 a = __ldg(Ea + q), b = __ldg(Eb + q);
        em[4 * q] = pack2(a.x, b.x); em[4 * q + 1] = pack2(a.y, b.y);
        em[4 * q + 2] = pack2(a.z, b.z); em[4 * q + 3] = pack2(a.w, b.w);
      }
      const float wjk = c_Wp[WO + pl / N] * c_Wp[WO + pl % N];
#pragma unroll
      for (int i = 0; i < N; i++) {
        const f2 w = bcast(c_Wp[WO + i] * wjk);
        const f2 a0 = mul2(w, uq[i]), a1 = mul2(w, gx[i]), a2 = mul2(w, gy[i]), a3 = mul2(w, gz[i]);
        vm[i] = fma2(em[3], a3, fma2(em[2], a2, fma2(em[1], a1, mul2(em[0], a0))));
        vx[i] = fma2(em[7], a3, fma2(em[6], a2, fma2(em[5], a1, mul2(em[4], a0))));
        vy[i] = fma2(em[11], a3, fma2(em[10], a2, fma2(em[9], a1, mul2(em[8], a0))));
        vz[i] = fma2(em[15], a3, fma2(em[14], a2, fma2(em[13], a1, mul2(em[12], a0))));
        if (want_e) acc = add2(acc, fma2(uq[i], vm[i], fma2(gz[i], vz[i], fma2(gy[i], vy[i], mul2(gx[i], vx[i])))));
      }
    } else if (active) {
      // G mode 2 (every element affine): one metric per element, records of 8
      // floats (xx yy zz xy xz yz, mass, pad), times the rule weight w_i w_j w_k
      constexpr int WO = N * (N - 1) / 2 - 1;
      f2 ea[7];
      float wjk = 0.f;
      if (GM == 2) {
        // the two 32-byte records as 16-byte loads (4 load instructions per pair
        // instead of 12-14 scalar ones: every lane reads the same address)
        const float4* Ea = (const float4*)(Gq + ((size_t)ch * E + r0) * 8);
        const float4* Eb = (const float4*)(Gq + ((size_t)ch * E + r1) * 8);
        const float4 a0 = __ldg(Ea), a1 = __ldg(Ea + 1), b0 = __ldg(Eb), b1 = __ldg(Eb + 1);
        ea[0] = pack2(a0.x, b0.x); ea[1] = pack2(a0.y, b0.y); ea[2] = pack2(a0.z, b0.z);
        ea[3] = pack2(a0.w, b0.w); ea[4] = pack2(a1.x, b1.x); ea[5] = pack2(a1.y, b1.y);
        ea[6] = pack2(a1.z, b1.z);
        wjk = c_Wp[WO + pl / N] * c_Wp[WO + pl % N];
      }
#pragma unroll
      for (int i = 0; i < N; i++) {
        const int o = i * N2 + pl;
        auto ld = [&](int comp) {
          if (GM == 0) return pack2(Ga[comp * N3 + o], Gb[comp * N3 + o]);
          return pack2(__ldcs(Ga + comp * N3 + o), __ldcs(Gb + comp * N3 + o));
        };
        if (GM == 2) {
          const f2 w = bcast(c_Wp[WO + i] * wjk);
          const f2 sx = mul2(w, gx[i]), sy = mul2(w, gy[i]), sz = mul2(w, gz[i]);
          vx[i] = fma2(ea[4], sz, fma2(ea[3], sy, mul2(ea[0], sx)));
          vy[i] = fma2(ea[5], sz, fma2(ea[1], sy, mul2(ea[3], sx)));
          vz[i] = fma2(ea[2], sz, fma2(ea[5], sy, mul2(ea[4], sx)));
        } else {
          const f2 gxx = ld(0), gyy = ld(1), gzz = ld(2), gxy = ld(3), gxz = ld(4), gyz = ld(5);
          vx[i] = fma2(gxz, gz[i], fma2(gxy, gy[i], mul2(gxx, gx[i])));
          vy[i] = fma2(gyz, gz[i], fma2(gyy, gy[i], mul2(gxy, gx[i])));
          vz[i] = fma2(gzz, gz[i], fma2(gyz, gy[i], mul2(gxz, gx[i])));
        }
        if (MASS) {
          if (GM == 2) vm[i] = mul2(mul2(bcast(c_Wp[WO + i] * wjk), ea[6]), uq[i]);
          else vm[i] = mul2(ld(6), uq[i]);
        }
        if (want_e) {  // x^T A x only for a caller that asks for it (CG)
          f2 en = fma2(gz[i], vz[i], fma2(gy[i], vy[i], mul2(gx[i], vx[i])));
          if (MASS) en = fma2(uq[i], vm[i], en);
          acc = add2(acc, en);
        }
      }
    }
    if (GM == 0) {
      group_sync<G>(gid);
      if (lane == 0 && has_next) {
        fence_proxy_async();
        issue_g(ch + stride);
      }
      if (has_next) g_issued++;
    }
    pair_backward<N, MASS, pair_eo(N, GM)>(pl, pa, pk, active, gid, su, s1, s2, t1, t2, t3, vx, vy, vz, vm);
    const int* td = tbuf(b);
    const int nrow = rows_of(ch);
#pragma unroll
    for (int j = 0; j < NG; j++) {
      const int t = lane + j * G;
      if (t < SN3) {
        const int s = t / N3, l = t % N3;
        float v0, v1;
        unpack2(work[t], v0, v1);
#pragma unroll
        for (int h = 0; h < 2; h++) {
          if (2 * s + h < nrow) {
            const int d = td[(2 * s + h) * rowt + l];
            const int dof = d & 0x7fffffff;
            const float v = __int_as_float(__float_as_int(h ? v1 : v0) ^ (d & (int)0x80000000));
            if (dof >= first_cell) y[dof] = v;  // element-interior DOF: single writer
            else red_add(y + dof, v);
          }
        }
      }
    }
    group_sync<G>(gid);
  }
  if (!ok) {
    if (lane == 0) {
      atomicExch(err, 1);
      for (int j = t_waited; j < t_issued; j++) mbar_wait_bounded(&mbar[j & 1], (j >> 1) & 1);
      for (int j = g_waited; j < g_issued; j++) mbar_wait_bounded(&mbar[2], j & 1);
    }
    group_sync<G>(gid);
  }
  if (partial) {
    float a0, a1;
    unpack2(acc, a0, a1);
    block_reduce_finish((double)a0 + (double)a1, partial, counter, energy);
  }
}

// ---- multi-right-hand-side apply, two right-hand sides per lane -------------------
// Y_r += A X_r for the rhs r < R with phase[r] == want (batched solves; vectors
// rhs-major with stride n), FP32.  Same chunk pipeline as hex_apply_multi_kernel
// (matfree.cu): the G tile and DOF rows of a chunk of EPW elements are bulk-copied
// once and reused for every rhs.  The active rhs are processed in pairs: a lane
// holds its pencil for rhs (ra, rb) in one packed register, so the gather indices,
// signs and G values are shared and every contraction step serves two rhs (an odd
// count leaves the second half zero).  Per-rhs energies x_r^T A x_r go to energy[r].
template <int N, bool MASS>
__global__ void __launch_bounds__(HexCfg<N>::BLOCK)
hex_apply_multi_pair_kernel(int ne, int64_t n, int R, const int* __restrict__ phase, int want,
                            const int* __restrict__ tdof, int tstride, const float* __restrict__ Gq, int gstride,
                            const float* __restrict__ x, float* __restrict__ y, int first_cell, double* partial,
                            unsigned int* counter, double* energy, int* err) {
  using C = HexCfg<N>;
  using LY = PairLayout<N>;
  constexpr int N2 = C::N2, N3 = C::N3, G = C::G, S = C::EPW, SN3 = S * N3, RMAX = 16;
  __shared__ float sacc[C::EPB][RMAX];
  __shared__ int slist[RMAX], scount;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int gid = threadIdx.x / G, lane = threadIdx.x % G;
  const int slot = lane / N2, pl = lane % N2;
  const int rowg = (int)(round16((size_t)gstride * sizeof(float)) / sizeof(float));
  const int rowt = (int)(round16((size_t)tstride * sizeof(int)) / sizeof(int));
  const size_t gb = (size_t)S * rowg * sizeof(float), tb = (size_t)S * rowt * sizeof(int);
  const size_t work_bytes = round16((size_t)S * (N3 + 2 * LY::SW + 3 * LY::TW) * sizeof(f2));
  unsigned char* gp = smem_raw + (size_t)gid * (gb + 2 * tb + work_bytes + 32);
  float* gbuf = (float*)gp;
  auto tbuf = [&](int b) { return (int*)(gp + gb + b * tb); };
  f2* work = (f2*)(gp + gb + 2 * tb);
  const int sl = slot < S ? slot : 0;
  f2* su = work + sl * N3;
  f2* s1 = work + SN3 + sl * LY::SW;
  f2* s2 = s1 + S * LY::SW;
  f2* t1 = work + SN3 + 2 * S * LY::SW + sl * LY::TW;
  f2* t2 = t1 + S * LY::TW;
  f2* t3 = t2 + S * LY::TW;
  int pa = pl / N, pk = pl % N;
  if (N == 5) {
    const int v = c_p2[pl];
    pa = v / 5;
    pk = v % 5;
  }
  uint64_t* mbar = (uint64_t*)(gp + gb + 2 * tb + work_bytes);
  if (threadIdx.x == 0) {  // active rhs in ascending order
    int c = 0;
    for (int r = 0; r < R && r < RMAX; r++)
      if (phase[r] == want) slist[c++] = r;
    scount = c;
  }
  for (int t = threadIdx.x; t < C::EPB * RMAX; t += blockDim.x) (&sacc[0][0])[t] = 0.f;
  if (lane == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    mbar_init(&mbar[2], 1);
    fence_mbar_init();
  }
  __syncthreads();
  const int nact = scount;
  const int nch = (ne + S - 1) / S;
  const int stride = gridDim.x * C::EPB;
  int ch = blockIdx.x * C::EPB + gid;
  auto rows_of = [&](int c) { return min(S, ne - c * S); };
  auto issue = [&](int c, int b) {
    const uint32_t bt = (uint32_t)(rows_of(c) * rowt * sizeof(int)), bg = (uint32_t)(rows_of(c) * rowg * sizeof(float));
    mbar_expect_tx(&mbar[b], bt);
    bulk_g2s(tbuf(b), tdof + (size_t)c * S * tstride, bt, &mbar[b]);
    mbar_expect_tx(&mbar[2], bg);
    bulk_g2s(gbuf, Gq + (size_t)c * S * gstride, bg, &mbar[2]);
  };
  int issued = 0, waited = 0;
  bool ok = true;
  if (nact > 0 && ch < nch && lane == 0) issue(ch, 0);
  if (nact > 0 && ch < nch) issued = 1;
  for (int k = 0; nact > 0 && ok && ch < nch; ch += stride, k++) {
    const int b = k & 1;
    ok = group_all<G>(gid, mbar_wait_bounded(&mbar[b], (k >> 1) & 1) && mbar_wait_bounded(&mbar[2], k & 1));
    waited++;
    if (!ok) break;
    const int* td = tbuf(b);
    const int nrow = rows_of(ch);
    const bool act_el = slot < S && ch * S + slot < ne;
    const float* Ge = gbuf + (size_t)sl * rowg;
    for (int q = 0; q < nact; q += 2) {
      const int ra = slist[q], rb = q + 1 < nact ? slist[q + 1] : -1;
      const float* xa = x + (size_t)ra * n;
      const float* xb = x + (size_t)(rb >= 0 ? rb : ra) * n;
      for (int t = lane; t < SN3; t += G) {
        float va = 0.f, vb = 0.f;
        unsigned sg = 0u;
        if (t / N3 < nrow) {
          const int d = td[(t / N3) * rowt + t % N3];
          const int dof = d & 0x7fffffff;
          va = __ldg(xa + dof);
          if (rb >= 0) vb = __ldg(xb + dof);
          sg = (unsigned)d & 0x80000000u;
        }
        work[t] = pack2(va, vb) ^ (((f2)sg << 32) | (f2)sg);
      }
      group_sync<G>(gid);
      f2 gx[N], gy[N], gz[N], uq[N];
      pair_forward<N, MASS, true>(pl, pa, pk, act_el, gid, su, s1, s2, t1, t2, t3, gx, gy, gz, uq);
      f2 vx[N], vy[N], vz[N], vm[N];
      f2 en = 0;
      if (act_el) {
#pragma unroll
        for (int i = 0; i < N; i++) {
          const int o = i * N2 + pl;
          const f2 gxx = bcast(Ge[o]), gyy = bcast(Ge[N3 + o]), gzz = bcast(Ge[2 * N3 + o]);
          const f2 gxy = bcast(Ge[3 * N3 + o]), gxz = bcast(Ge[4 * N3 + o]), gyz = bcast(Ge[5 * N3 + o]);
          vx[i] = fma2(gxz, gz[i], fma2(gxy, gy[i], mul2(gxx, gx[i])));
          vy[i] = fma2(gyz, gz[i], fma2(gyy, gy[i], mul2(gxy, gx[i])));
          vz[i] = fma2(gzz, gz[i], fma2(gyz, gy[i], mul2(gxz, gx[i])));
          en = fma2(gz[i], vz[i], fma2(gy[i], vy[i], fma2(gx[i], vx[i], en)));
          if (MASS) {
            vm[i] = mul2(bcast(Ge[6 * N3 + o]), uq[i]);
            en = fma2(uq[i], vm[i], en);
          }
        }
      }
      float ea, eb;
      unpack2(en, ea, eb);
      for (int o = 16; o > 0; o >>= 1) {
        ea += __shfl_xor_sync(0xffffffffu, ea, o);
        eb += __shfl_xor_sync(0xffffffffu, eb, o);
      }
      if ((lane & 31) == 0) {
        atomicAdd(&sacc[gid][ra], ea);
        if (rb >= 0) atomicAdd(&sacc[gid][rb], eb);
      }
      pair_backward<N, MASS, true>(pl, pa, pk, act_el, gid, su, s1, s2, t1, t2, t3, vx, vy, vz, vm);
      float* ya = y + (size_t)ra * n;
      float* yb = y + (size_t)(rb >= 0 ? rb : ra) * n;
      for (int t = lane; t < SN3; t += G) {
        if (t / N3 >= nrow) continue;
        const int d = td[(t / N3) * rowt + t % N3];
        const int dof = d & 0x7fffffff;
        const unsigned sg = (unsigned)d & 0x80000000u;
        float wa, wb;
        unpack2(work[t] ^ (((f2)sg << 32) | (f2)sg), wa, wb);
        if (dof >= first_cell) {  // element-interior DOF: single writer
          ya[dof] = wa;
          if (rb >= 0) yb[dof] = wb;
        } else {
          red_add(ya + dof, wa);
          if (rb >= 0) red_add(yb + dof, wb);
        }
      }
      group_sync<G>(gid);
    }
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
    float sum = 0;
    for (int g = 0; g < C::EPB; g++) sum += sacc[g][threadIdx.x];
    if (threadIdx.x < R) partial[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = (double)sum;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last) {
    __threadfence();
    if (threadIdx.x < R && phase[threadIdx.x] == want) {
      double sum = 0;
      for (int i = 0; i < (int)gridDim.x; i++) sum += ((volatile double*)partial)[(size_t)threadIdx.x * gridDim.x + i];
      energy[threadIdx.x] = sum;
    }
    if (threadIdx.x == 0) *counter = 0u;
  }
}

// ---- slice / pencil form (affine meshes) ------------------------------------------
// Same operator as hex_apply_pair_kernel in G mode 2, with a different split of
// the contractions between the threads of a warp.  A warp owns P = 32/N element
// pairs (two elements per lane, packed as above).  Lane (t, p) = (lane / P, lane % P).
// The lane's N x N slice u[a = t][.][.] of both elements sits in registers (N = 2,
// 4) or is read again from the staging array per plane (N = 3, 5), its result
// slice is in registers, and the chunk runs one quadrature plane k at a time:
//   slice phase:  lane (a = t) contracts its slice along z (c -> k) and y
//                 (b -> j) and writes bb, db, bd at (a, j) of plane k;
//   pencil phase: lane (j = t) reads the N values along a of the three arrays,
//                 forms the gradient at the N points (i, j, k), applies the
//                 metric, contracts back along a and writes in place;
//   slice phase:  lane (a = t) reads its row of the plane, contracts back along
//                 y and accumulates the transposed z contraction of plane k into
//                 its result slice (registers).
// Per plane the exchange array X[array][j][a][p] (unit stride in p, stride P in
// a, j stride SJ = P mod 16) moves 3 N^2 words per pair each way at the two-
// wavefront minimum of an 8-byte warp access: 3 N^3 per element pair in all,
// against 5 N^3 in the pencil-per-lane form (plus N^3 re-reads of the slice).
// Only one plane is resident, so the warp needs 4.4 KB of exchange space at
// N = 5, and with the slice re-read per plane 12 warps per SM fit in registers.
// The x gather and the scatter run in DOF order (consecutive lanes on
// consecutive local DOFs of one element: coalesced index and x loads, atomics
// that share sectors) through the staging array su[p][a][m] (m = b N + c, a
// stride SUA = P and pair stride SPU = 1 mod 16: conflict-free slice reads and
// writes); every index load of a chunk is issued before its first x load, and
// every x load before the first store, so a chunk waits for two load latencies.
// All exchanges stay inside one warp (__syncwarp; no block barriers, no waits).
template <int N>
struct SliceCfg {
  static constexpr int P = 32 / N;                                      // element pairs per warp
  static constexpr int NP = N * P;                                      // active lanes
  static constexpr int N2 = N * N, N3 = N * N * N;
  static constexpr int SJ = NP + ((P - NP) % 16 + 16) % 16;             // >= NP, == P (mod 16)
  static constexpr int PL = (N - 1) * SJ + NP;                          // words per array of one plane
  static constexpr int XW = 3 * PL;                                     // exchange words per warp (one plane)
  static constexpr int SUA = N2 + ((P - N2) % 16 + 16) % 16;            // >= N^2, == P (mod 16)
  static constexpr int SPU0 = (N - 1) * SUA + N2;
  static constexpr int SPU = SPU0 + ((1 - SPU0) % 16 + 16) % 16;        // >= SPU0, == 1 (mod 16)
  static constexpr int SUW = P * SPU;                                   // staging words per warp
  static constexpr int W = XW + SUW;                                    // words per warp
  static constexpr int NT = P * N3, NI = (NT + 31) / 32;                // DOF-order items per warp / lane
  static constexpr int WARPS = 2, BLOCK = 32 * WARPS;
  static constexpr size_t smem = (size_t)WARPS * W * sizeof(f2);
};
// resident 64-thread blocks per SM the register allocation must allow: 12 warps
// (168 registers) at N = 4 and 5, where the result slice and the plane
// temporaries are live together; more warps at lower orders
constexpr int slice_min_blocks(int N) { return N <= 3 ? 8 : 6; }

template <int N, bool MASS>
__global__ void __launch_bounds__(SliceCfg<N>::BLOCK, slice_min_blocks(N))
hex_apply_slice_kernel(int ne, const int* __restrict__ tdof, int tstride, const float* __restrict__ Ga,
                       const float* __restrict__ x, float* __restrict__ y, int first_cell, double* partial,
                       unsigned int* counter, double* energy, const int* skip) {
  using C = SliceCfg<N>;
  constexpr int P = C::P, NP = C::NP, SJ = C::SJ, PL = C::PL, N2 = C::N2, N3 = C::N3, O = tab_off(N);
  constexpr int SUA = C::SUA, SPU = C::SPU, NT = C::NT, NI = C::NI;
  constexpr int WO = N * (N - 1) / 2 - 1;   // offset of this order's Gauss weights
  if (skip && *(volatile const int*)skip) return;
  extern __shared__ __align__(16) unsigned char slice_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  f2* X = (f2*)slice_raw + (size_t)warp * C::W;  // one plane: [array][j][a][p]
  f2* su = X + C::XW;                            // gather / scatter staging [p][a][m]
  const bool act = lane < NP;
  const int t = act ? lane / P : 0, p = lane % P;
  const int ps = t * SJ + p;                // pencil-phase word offset of this lane (j = t)
  const int ss = p * SPU + t * SUA;         // slice-phase staging offset of this lane (a = t)
  const int nch = (ne + 2 * P - 1) / (2 * P);
  f2 acc = 0;
  const bool want_e = partial != nullptr;
  for (int ch = blockIdx.x * C::WARPS + warp; ch < nch; ch += gridDim.x * C::WARPS) {
    const int eb = ch * 2 * P, nrow = min(2 * P, ne - eb);
    const int e0 = eb + 2 * p;
    const bool v0 = act && e0 < ne, v1 = act && e0 + 1 < ne;
    // gather in DOF order: item q = (pair, local DOF l), both elements of the pair;
    // all index loads, then all x loads, then the stores
    {
      int d0[NI], d1[NI];
#pragma unroll
      for (int j = 0; j < NI; j++) {
        const int q = lane + 32 * j;
        const int pp = q / N3, l = q % N3;
        d0[j] = (q < NT && 2 * pp < nrow) ? __ldg(tdof + (size_t)(eb + 2 * pp) * tstride + l) : -1;
        d1[j] = (q < NT && 2 * pp + 1 < nrow) ? __ldg(tdof + (size_t)(eb + 2 * pp + 1) * tstride + l) : -1;
      }
      float g0[NI], g1[NI];
#pragma unroll
      for (int j = 0; j < NI; j++) {
        g0[j] = d0[j] != -1 ? __ldg(x + (d0[j] & 0x7fffffff)) : 0.f;
        g1[j] = d1[j] != -1 ? __ldg(x + (d1[j] & 0x7fffffff)) : 0.f;
      }
      __syncwarp();  // the previous chunk's scatter has read su
#pragma unroll
      for (int j = 0; j < NI; j++) {
        const int q = lane + 32 * j;
        if (q < NT) {
          const int pp = q / N3, l = q % N3;
          const float a0 = __int_as_float(__float_as_int(g0[j]) ^ (d0[j] != -1 ? (d0[j] & (int)0x80000000) : 0));
          const float a1 = __int_as_float(__float_as_int(g1[j]) ^ (d1[j] != -1 ? (d1[j] & (int)0x80000000) : 0));
          su[pp * SPU + (l / N2) * SUA + l % N2] = pack2(a0, a1);
        }
      }
    }
    __syncwarp();
    // KEEP_U: the slice stays in registers for the whole chunk (N = 2 and 4, where
    // it fits the register budget without spills); otherwise each plane reads
    // it again from the staging array
    constexpr bool KEEP_U = N == 2 || N == 4;
    f2 out[N2], uk[KEEP_U ? N2 : 1];
#pragma unroll
    for (int m = 0; m < N2; m++) out[m] = 0;
    if constexpr (KEEP_U) {
#pragma unroll
      for (int m = 0; m < N2; m++) uk[m] = act ? su[ss + m] : (f2)0;
    }
    // metric of the pencil lane's two elements (a missing element reuses a valid one)
    f2 ea[7];
    {
      const int r0 = v0 ? e0 : eb, r1 = v1 ? e0 + 1 : r0;
#pragma unroll
      for (int c = 0; c < (MASS ? 7 : 6); c++) ea[c] = pack2(__ldg(Ga + (size_t)r0 * 8 + c), __ldg(Ga + (size_t)r1 * 8 + c));
    }
    const float wj = c_Wp[WO + t];
#pragma unroll 1
    for (int k = 0; k < N; k++) {
      // slice phase: stages 1 (c -> k) and 2 (b -> j) for plane k; the slice is
      // read again from the staging array row by row (registers hold the result
      // slice across the planes)
      f2 ub[N], ud[N];
#pragma unroll
      for (int b = 0; b < N; b++) {
        f2 u[N];
        if constexpr (KEEP_U) {
#pragma unroll
          for (int c = 0; c < N; c++) u[c] = uk[b * N + c];
        } else {
#pragma unroll
          for (int c = 0; c < N; c++) u[c] = act ? su[ss + b * N + c] : (f2)0;
        }
        f2 sb = mul2(bcast(c_Bp[O + k * N]), u[0]), sd = mul2(bcast(c_Dp[O + k * N]), u[0]);
#pragma unroll
        for (int c = 1; c < N; c++) {
          sb = fma2(bcast(c_Bp[O + k * N + c]), u[c], sb);
          sd = fma2(bcast(c_Dp[O + k * N + c]), u[c], sd);
        }
        ub[b] = sb;
        ud[b] = sd;
      }
      __syncwarp();  // the previous plane's readers of X are done
#pragma unroll
      for (int j = 0; j < N; j++) {
        f2 bb = mul2(bcast(c_Bp[O + j * N]), ub[0]), db = mul2(bcast(c_Dp[O + j * N]), ub[0]),
           bd = mul2(bcast(c_Bp[O + j * N]), ud[0]);
#pragma unroll
        for (int b = 1; b < N; b++) {
          bb = fma2(bcast(c_Bp[O + j * N + b]), ub[b], bb);
          db = fma2(bcast(c_Dp[O + j * N + b]), ub[b], db);
          bd = fma2(bcast(c_Bp[O + j * N + b]), ud[b], bd);
        }
        if (act) {
          f2* w = X + j * SJ + lane;
          w[0] = bb;
          w[PL] = db;
          w[2 * PL] = bd;
        }
      }
      __syncwarp();
      // pencil phase: lane (j = t, p), points (i, j, k)
      if (act) {
        f2* w = X + ps;
        f2 w1[N], w2[N], w3[N];
#pragma unroll
        for (int a = 0; a < N; a++) {
          w1[a] = w[a * P];
          w2[a] = w[PL + a * P];
          w3[a] = w[2 * PL + a * P];
        }
        const float wjk = wj * c_Wp[WO + k];
        f2 vx[N], vy[N], vz[N], vm[N];
#pragma unroll
        for (int i = 0; i < N; i++) {
          f2 gx = mul2(bcast(c_Dp[O + i * N]), w1[0]), gy = mul2(bcast(c_Bp[O + i * N]), w2[0]),
             gz = mul2(bcast(c_Bp[O + i * N]), w3[0]);
          f2 uq = 0;
          if (MASS) uq = mul2(bcast(c_Bp[O + i * N]), w1[0]);
#pragma unroll
          for (int a = 1; a < N; a++) {
            gx = fma2(bcast(c_Dp[O + i * N + a]), w1[a], gx);
            gy = fma2(bcast(c_Bp[O + i * N + a]), w2[a], gy);
            gz = fma2(bcast(c_Bp[O + i * N + a]), w3[a], gz);
            if (MASS) uq = fma2(bcast(c_Bp[O + i * N + a]), w1[a], uq);
          }
          const f2 wq = bcast(c_Wp[WO + i] * wjk);
          const f2 sx = mul2(wq, gx), sy = mul2(wq, gy), sz = mul2(wq, gz);
          vx[i] = fma2(ea[4], sz, fma2(ea[3], sy, mul2(ea[0], sx)));
          vy[i] = fma2(ea[5], sz, fma2(ea[1], sy, mul2(ea[3], sx)));
          vz[i] = fma2(ea[2], sz, fma2(ea[5], sy, mul2(ea[4], sx)));
          if (MASS) vm[i] = mul2(mul2(wq, ea[6]), uq);
          if (want_e) {  // x^T A x only for a caller that asks for it (CG)
            f2 en = fma2(gz, vz[i], fma2(gy, vy[i], mul2(gx, vx[i])));
            if (MASS) en = fma2(uq, vm[i], en);
            acc = add2(acc, en);
          }
        }
#pragma unroll
        for (int a = 0; a < N; a++) {
          f2 q1 = mul2(bcast(c_Dp[O + a]), vx[0]), q2 = mul2(bcast(c_Bp[O + a]), vy[0]),
             q3 = mul2(bcast(c_Bp[O + a]), vz[0]);
          if (MASS) q1 = fma2(bcast(c_Bp[O + a]), vm[0], q1);
#pragma unroll
          for (int i = 1; i < N; i++) {
            q1 = fma2(bcast(c_Dp[O + i * N + a]), vx[i], q1);
            if (MASS) q1 = fma2(bcast(c_Bp[O + i * N + a]), vm[i], q1);
            q2 = fma2(bcast(c_Bp[O + i * N + a]), vy[i], q2);
            q3 = fma2(bcast(c_Bp[O + i * N + a]), vz[i], q3);
          }
          w[a * P] = q1;
          w[PL + a * P] = q2;
          w[2 * PL + a * P] = q3;
        }
      }
      __syncwarp();
      // slice phase, transposed: stage 2 (j -> b) on plane k, then this plane's
      // share of stage 1 (k -> c) into the result slice
      if (act) {
        f2 r1[N], r2[N], r3[N];
        const f2* w = X + lane;
#pragma unroll
        for (int j = 0; j < N; j++) {
          r1[j] = w[j * SJ];
          r2[j] = w[PL + j * SJ];
          r3[j] = w[2 * PL + j * SJ];
        }
#pragma unroll
        for (int b = 0; b < N; b++) {
          f2 vb = mul2(bcast(c_Bp[O + b]), r1[0]), vd = mul2(bcast(c_Bp[O + b]), r3[0]);
          vb = fma2(bcast(c_Dp[O + b]), r2[0], vb);
#pragma unroll
          for (int j = 1; j < N; j++) {
            vb = fma2(bcast(c_Bp[O + j * N + b]), r1[j], vb);
            vb = fma2(bcast(c_Dp[O + j * N + b]), r2[j], vb);
            vd = fma2(bcast(c_Bp[O + j * N + b]), r3[j], vd);
          }
#pragma unroll
          for (int c = 0; c < N; c++)
            out[b * N + c] = fma2(bcast(c_Dp[O + k * N + c]), vd, fma2(bcast(c_Bp[O + k * N + c]), vb, out[b * N + c]));
        }
      }
    }
    // result slice -> staging (this lane's own words), then the scatter in DOF order
    if (act) {
#pragma unroll
      for (int m = 0; m < N2; m++) su[ss + m] = out[m];
    }
    __syncwarp();
    {
      int d0[NI], d1[NI];
#pragma unroll
      for (int j = 0; j < NI; j++) {
        const int q = lane + 32 * j;
        const int pp = q / N3, l = q % N3;
        d0[j] = (q < NT && 2 * pp < nrow) ? __ldg(tdof + (size_t)(eb + 2 * pp) * tstride + l) : -1;
        d1[j] = (q < NT && 2 * pp + 1 < nrow) ? __ldg(tdof + (size_t)(eb + 2 * pp + 1) * tstride + l) : -1;
      }
#pragma unroll
      for (int j = 0; j < NI; j++) {
        const int q = lane + 32 * j;
        if (q < NT) {
          const int pp = q / N3, l = q % N3;
          float o0, o1;
          unpack2(su[pp * SPU + (l / N2) * SUA + l % N2], o0, o1);
          if (d0[j] != -1) {
            const int dof = d0[j] & 0x7fffffff;
            const float v = __int_as_float(__float_as_int(o0) ^ (d0[j] & (int)0x80000000));
            if (dof >= first_cell) y[dof] = v;
            else red_add(y + dof, v);
          }
          if (d1[j] != -1) {
            const int dof = d1[j] & 0x7fffffff;
            const float v = __int_as_float(__float_as_int(o1) ^ (d1[j] & (int)0x80000000));
            if (dof >= first_cell) y[dof] = v;
            else red_add(y + dof, v);
          }
        }
      }
    }
  }
  if (partial) {
    float a0, a1;
    unpack2(acc, a0, a1);
    block_reduce_finish((double)a0 + (double)a1, partial, counter, energy);
  }
}

// ---- host side ------------------------------------------------------------------
bool hex_pair_supported(int N) { return N >= 2 && N <= 7; }
bool hex_slice_supported(int N) { return N >= 2 && N <= 5; }

void upload_pair_tables(gh1_space* sp) {
  const int N = sp->p + 1;
  if (!hex_pair_supported(N)) return;
  const size_t off = tab_off(N) * sizeof(float);
  cudaStream_t s = sp->ctx->stream;
  GH1_CUDA(cudaMemcpyToSymbolAsync(c_Bp, sp->d_B32.p, N * N * sizeof(float), off, cudaMemcpyDeviceToDevice, s));
  GH1_CUDA(cudaMemcpyToSymbolAsync(c_Dp, sp->d_D32.p, N * N * sizeof(float), off, cudaMemcpyDeviceToDevice, s));
  std::vector<float> w(sp->gw.begin(), sp->gw.end());
  GH1_CUDA(cudaMemcpyToSymbolAsync(c_Wp, w.data(), N * sizeof(float), (N * (N - 1) / 2 - 1) * sizeof(float),
                                   cudaMemcpyHostToDevice, s));
  std::vector<double> B(N * N), D(N * N);
  GH1_CUDA(cudaMemcpyAsync(B.data(), sp->d_B64.p, N * N * sizeof(double), cudaMemcpyDeviceToHost, s));
  GH1_CUDA(cudaMemcpyAsync(D.data(), sp->d_D64.p, N * N * sizeof(double), cudaMemcpyDeviceToHost, s));
  GH1_CUDA(cudaStreamSynchronize(s));  // the host staging vectors go out of scope
  double eo[4][16];
  GH1_CHECK(hex_eo_coefficients(B.data(), D.data(), N, eo) <= 1e-12, GH1_ERR_ARG,
            "internal: 1D hex tables lack the reflection symmetry");
  for (int k = 0; k < 4; k++) {
    float e32[16];
    for (int q = 0; q < 16; q++) e32[q] = (float)eo[k][q];
    GH1_CUDA(cudaMemcpyToSymbol(c_EOp, e32, N * sizeof(float), (k * 64 + eo_off(N)) * sizeof(float)));
  }
}

// Per-element metric of an affine hex (x = P0 + J xi: J[3k+j] = d x_k / d xi_j
// with the columns P1-P0, P3-P0, P4-P0 in the reference vertex order), and a
// flag if any element's trilinear map has a bilinear or trilinear part (its
// coefficients P0-P1+P2-P3, P0-P1-P4+P5, P0-P3-P4+P7, -P0+P1-P2+P3+P4-P5+P6-P7)
// above 1e-12 of the element's edge vectors.
__global__ void hex_affine_kernel(int ne, const double* __restrict__ X, const int* __restrict__ el,
                                  const double* __restrict__ kappa, const double* __restrict__ K6,
                                  const double* __restrict__ mu, float* Ga, int* nonaffine) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  double P[8][3];
  for (int a = 0; a < 8; a++)
    for (int k = 0; k < 3; k++) P[a][k] = X[3 * (size_t)el[(size_t)e * 8 + a] + k];
  double J[9], scale = 0, dev = 0;
  for (int k = 0; k < 3; k++) {
    J[3 * k + 0] = P[1][k] - P[0][k];
    J[3 * k + 1] = P[3][k] - P[0][k];
    J[3 * k + 2] = P[4][k] - P[0][k];
    scale = fmax(scale, fmax(fabs(J[3 * k]), fmax(fabs(J[3 * k + 1]), fabs(J[3 * k + 2]))));
    dev = fmax(dev, fabs(P[0][k] - P[1][k] + P[2][k] - P[3][k]));
    dev = fmax(dev, fabs(P[0][k] - P[1][k] - P[4][k] + P[5][k]));
    dev = fmax(dev, fabs(P[0][k] - P[3][k] - P[4][k] + P[7][k]));
    dev = fmax(dev, fabs(-P[0][k] + P[1][k] - P[2][k] + P[3][k] + P[4][k] - P[5][k] + P[6][k] - P[7][k]));
  }
  if (dev > 1e-12 * scale) atomicExch(nonaffine, 1);
  const double det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
                     J[2] * (J[3] * J[7] - J[4] * J[6]);
  const double id = 1.0 / det;
  const double Ji[9] = {(J[4] * J[8] - J[5] * J[7]) * id, (J[2] * J[7] - J[1] * J[8]) * id,
                        (J[1] * J[5] - J[2] * J[4]) * id, (J[5] * J[6] - J[3] * J[8]) * id,
                        (J[0] * J[8] - J[2] * J[6]) * id, (J[2] * J[3] - J[0] * J[5]) * id,
                        (J[3] * J[7] - J[4] * J[6]) * id, (J[1] * J[6] - J[0] * J[7]) * id,
                        (J[0] * J[4] - J[1] * J[3]) * id};
  float* g = Ga + (size_t)e * 8;
  if (K6) {
    double t[6];
    tensor_metric(Ji, K6 + 6 * (size_t)e, fabs(det), t);
    for (int c = 0; c < 6; c++) g[c] = (float)t[c];
  } else {
    const double f = kappa[e] * fabs(det);
    g[0] = (float)(f * (Ji[0] * Ji[0] + Ji[1] * Ji[1] + Ji[2] * Ji[2]));
    g[1] = (float)(f * (Ji[3] * Ji[3] + Ji[4] * Ji[4] + Ji[5] * Ji[5]));
    g[2] = (float)(f * (Ji[6] * Ji[6] + Ji[7] * Ji[7] + Ji[8] * Ji[8]));
    g[3] = (float)(f * (Ji[0] * Ji[3] + Ji[1] * Ji[4] + Ji[2] * Ji[5]));
    g[4] = (float)(f * (Ji[0] * Ji[6] + Ji[1] * Ji[7] + Ji[2] * Ji[8]));
    g[5] = (float)(f * (Ji[3] * Ji[6] + Ji[4] * Ji[7] + Ji[5] * Ji[8]));
  }
  g[6] = mu ? (float)(mu[e] * fabs(det)) : 0.f;
  g[7] = 0.f;
}

// Detects an all-affine hex mesh and builds the per-element metric records for
// G mode 2 (GH1_HEX_AFFINE=0 keeps the per-point metric only).
void hex_affine_setup(gh1_op* op) {
  gh1_space* sp = op->sp;
  op->all_affine = false;
  op->d_Ga32.release();
  const char* env = getenv("GH1_HEX_AFFINE");
  // curved elements or coefficients per point: per-point metrics only
  if ((env && env[0] == '0') || !hex_pair_supported(sp->p + 1) || sp->mesh->def_space || op->lap_pp) return;
  const int ne = sp->mesh->ne;
  cudaStream_t s = sp->ctx->stream;
  op->d_Ga32.alloc((size_t)ne * 8);
  DBuf<int> flag(1);
  flag.zero(s);
  const gh1_form* f = op->form;
  const double* K6 = op->lap_ov ? op->d_ovK6.p : (f->has_K6 ? f->d_K6.p : nullptr);
  const double* mu = !op->has_mass ? nullptr : (op->lap_ov ? op->d_ovmu.p : f->d_mu.p);
  hex_affine_kernel<<<(ne + 127) / 128, 128, 0, s>>>(ne, sp->mesh->d_X.p, sp->mesh->d_el.p, f->d_kappa.p, K6, mu,
                                                     op->d_Ga32.p, flag.p);
  check_kernel(sp->ctx, "hex_affine_kernel");
  int h = 1;
  GH1_CUDA(cudaMemcpyAsync(&h, flag.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  GH1_CUDA(cudaStreamSynchronize(s));
  op->all_affine = (h == 0);
  if (!op->all_affine) op->d_Ga32.release();
}

template <int N, bool MASS, int GM>
static int pair_occupancy(size_t smem) {
  static bool attr = false;
  auto kern = hex_apply_pair_kernel<N, MASS, GM>;
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
  GH1_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kern, PairCfg<N>::BLOCK, smem));
  return v;
}

template <int N, bool MASS, int GM>
static void pair_launch(gh1_op* op, const float* x, float* y, double* partial, unsigned int* counter, double* energy,
                        const int* skip) {
  using C = PairCfg<N>;
  gh1_space* sp = op->sp;
  const size_t smem = C::total(GM == 2 ? 8 : op->gstride32, sp->tstride, GM);
  const int per_sm = op->pair_per_sm[GM];
  GH1_CHECK(per_sm > 0, GH1_ERR_ARG, "internal: paired hex apply occupancy not prepared");
  const int ne = sp->mesh->ne;
  const int nch = (ne + C::E - 1) / C::E;
  const int blocks_needed = (nch + C::EPB - 1) / C::EPB;
  const int grid = std::min(blocks_needed, sp->ctx->nsm * per_sm);
  const float* G = GM == 2 ? op->d_Ga32.p : op->d_G32.p;
  const int gs = GM == 2 ? 8 : op->gstride32;
  hex_apply_pair_kernel<N, MASS, GM><<<grid, C::BLOCK, smem, sp->ctx->stream>>>(
      ne, sp->d_tdof.p, sp->tstride, G, gs, x, y, (int)sp->first_cell, partial, counter, energy, skip, op->d_err.p);
  check_kernel(sp->ctx, "hex_apply_pair_kernel");
}

#define GH1_PAIR_SWITCH(N, CASE)                                                     \
  switch (N) {                                                                       \
    CASE(2) CASE(3) CASE(4) CASE(5) CASE(6) CASE(7)                                  \
    default: throw Error(GH1_ERR_UNSUPPORTED, "paired hex apply: order out of range"); \
  }

int hex_pair_occupancy(gh1_op* op, int gm) {
  const bool mass = op->has_mass;
  const int ts = op->sp->tstride, gs = op->gstride32;
  int v = 0;
#define GH1_PAIR_OCC(NN)                                                                                       \
  case NN:                                                                                                     \
    if (gm == 0) v = mass ? pair_occupancy<NN, true, 0>(PairCfg<NN>::total(gs, ts, 0))                        \
                          : pair_occupancy<NN, false, 0>(PairCfg<NN>::total(gs, ts, 0));                      \
    else if (gm == 1) v = mass ? pair_occupancy<NN, true, 1>(PairCfg<NN>::total(gs, ts, 1))                   \
                               : pair_occupancy<NN, false, 1>(PairCfg<NN>::total(gs, ts, 1));                 \
    else if (gm == 2) v = mass ? pair_occupancy<NN, true, 2>(PairCfg<NN>::total(8, ts, 2))                    \
                               : pair_occupancy<NN, false, 2>(PairCfg<NN>::total(8, ts, 2));                  \
    else if (gm == 3) v = pair_occupancy<NN, true, 3>(PairCfg<NN>::total(16, ts, 3));                         \
    else v = pair_occupancy<NN, true, 4>(PairCfg<NN>::total(gs, ts, 4));                                      \
    break;
  GH1_PAIR_SWITCH(op->sp->p + 1, GH1_PAIR_OCC)
#undef GH1_PAIR_OCC
  return v;
}

void hex_pair_apply(gh1_op* op, int gm, const float* x, float* y, double* partial, unsigned int* counter,
                    double* energy, const int* skip) {
  const bool mass = op->has_mass;
#define GH1_PAIR_CASE(NN)                                                                       \
  case NN:                                                                                      \
    if (gm == 0) {                                                                              \
      if (mass) pair_launch<NN, true, 0>(op, x, y, partial, counter, energy, skip);             \
      else pair_launch<NN, false, 0>(op, x, y, partial, counter, energy, skip);                 \
    } else if (gm == 1) {                                                                       \
      if (mass) pair_launch<NN, true, 1>(op, x, y, partial, counter, energy, skip);             \
      else pair_launch<NN, false, 1>(op, x, y, partial, counter, energy, skip);                 \
    } else if (gm == 2) {                                                                       \
      if (mass) pair_launch<NN, true, 2>(op, x, y, partial, counter, energy, skip);             \
      else pair_launch<NN, false, 2>(op, x, y, partial, counter, energy, skip);                 \
    } else if (gm == 3) {                                                                       \
      pair_launch<NN, true, 3>(op, x, y, partial, counter, energy, skip);                       \
    } else {                                                                                    \
      pair_launch<NN, true, 4>(op, x, y, partial, counter, energy, skip);                       \
    }                                                                                           \
    break;
  GH1_PAIR_SWITCH(op->sp->p + 1, GH1_PAIR_CASE)
#undef GH1_PAIR_CASE
}

// slice-form apply (all-affine meshes): DOF table copy, occupancy, launch
template <int N, bool MASS>
static int slice_occupancy() {
  using C = SliceCfg<N>;
  auto kern = hex_apply_slice_kernel<N, MASS>;
  GH1_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::smem));
  int v = 0;
  GH1_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kern, C::BLOCK, C::smem));
  return v;
}

// Occupancy of the slice-form apply when the mesh is all affine and the order is
// supported (GH1_HEX_SLICE=0 turns the variant off); op->slice_per_sm = 0 otherwise.
void hex_slice_setup(gh1_op* op) {
  op->slice_per_sm = 0;
  const int N = op->sp->p + 1;
  const char* env = getenv("GH1_HEX_SLICE");
  if (!op->all_affine || !hex_slice_supported(N) || (env && env[0] == '0')) return;
  const bool m = op->has_mass;
  int v = 0;
  switch (N) {
    case 2: v = m ? slice_occupancy<2, true>() : slice_occupancy<2, false>(); break;
    case 3: v = m ? slice_occupancy<3, true>() : slice_occupancy<3, false>(); break;
    case 4: v = m ? slice_occupancy<4, true>() : slice_occupancy<4, false>(); break;
    case 5: v = m ? slice_occupancy<5, true>() : slice_occupancy<5, false>(); break;
    default: break;
  }
  op->slice_per_sm = std::max(v, 0);
}

template <int N, bool MASS>
static void slice_launch(gh1_op* op, const float* x, float* y, double* partial, unsigned int* counter, double* energy,
                         const int* skip) {
  using C = SliceCfg<N>;
  gh1_space* sp = op->sp;
  GH1_CHECK(op->slice_per_sm > 0, GH1_ERR_ARG, "internal: slice hex apply not prepared");
  const int ne = sp->mesh->ne, nch = (ne + 2 * C::P - 1) / (2 * C::P);
  const int grid = std::max(1, std::min((nch + C::WARPS - 1) / C::WARPS, sp->ctx->nsm * op->slice_per_sm));
  hex_apply_slice_kernel<N, MASS><<<grid, C::BLOCK, C::smem, sp->ctx->stream>>>(
      ne, sp->d_tdof.p, sp->tstride, op->d_Ga32.p, x, y, (int)sp->first_cell, partial, counter, energy, skip);
  check_kernel(sp->ctx, "hex_apply_slice_kernel");
}

void hex_slice_apply(gh1_op* op, const float* x, float* y, double* partial, unsigned int* counter, double* energy,
                     const int* skip) {
  const bool m = op->has_mass;
  switch (op->sp->p + 1) {
    case 2: m ? slice_launch<2, true>(op, x, y, partial, counter, energy, skip) : slice_launch<2, false>(op, x, y, partial, counter, energy, skip); break;
    case 3: m ? slice_launch<3, true>(op, x, y, partial, counter, energy, skip) : slice_launch<3, false>(op, x, y, partial, counter, energy, skip); break;
    case 4: m ? slice_launch<4, true>(op, x, y, partial, counter, energy, skip) : slice_launch<4, false>(op, x, y, partial, counter, energy, skip); break;
    case 5: m ? slice_launch<5, true>(op, x, y, partial, counter, energy, skip) : slice_launch<5, false>(op, x, y, partial, counter, energy, skip); break;
    default: throw Error(GH1_ERR_UNSUPPORTED, "slice hex apply: order out of range");
  }
}

// paired multi-rhs apply: occupancy (prepare_only, outside stream capture) and launch
template <int N, bool MASS>
static int multi_pair_launch_n(gh1_op* op, int R, const int* phase, int want, const float* x, float* y,
                               double* partial, unsigned int* counter, double* energy, bool prepare_only) {
  using C = HexCfg<N>;
  using LY = PairLayout<N>;
  gh1_space* sp = op->sp;
  const size_t gb = (size_t)C::EPW * round16((size_t)op->gstride32 * sizeof(float));
  const size_t tb = (size_t)C::EPW * round16((size_t)sp->tstride * sizeof(int));
  const size_t work = round16((size_t)C::EPW * (C::N3 + 2 * LY::SW + 3 * LY::TW) * sizeof(f2));
  const size_t smem = (size_t)C::EPB * (gb + 2 * tb + work + 32);
  auto kern = hex_apply_multi_pair_kernel<N, MASS>;
  if (prepare_only || op->multi_pair_per_sm <= 0) {
    int dev = 0, optin = 0;
    GH1_CUDA(cudaGetDevice(&dev));
    GH1_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    cudaFuncAttributes fa;
    GH1_CUDA(cudaFuncGetAttributes(&fa, kern));
    GH1_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes));
    int v = 0;
    GH1_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kern, C::BLOCK, smem));
    GH1_CHECK(v >= 1, GH1_ERR_UNSUPPORTED, "paired multi-rhs hex apply does not fit on an SM");
    op->multi_pair_per_sm = v;
  }
  const int ne = sp->mesh->ne, nch = (ne + C::EPW - 1) / C::EPW;
  const int grid = std::min((nch + C::EPB - 1) / C::EPB, sp->ctx->nsm * op->multi_pair_per_sm);
  if (prepare_only) return grid;
  kern<<<grid, C::BLOCK, smem, sp->ctx->stream>>>(ne, op->nrows, R, phase, want, sp->d_tdof.p, sp->tstride, op->d_G32.p,
                                                  op->gstride32, x, y, (int)sp->first_cell, partial, counter, energy,
                                                  op->d_err.p);
  check_kernel(sp->ctx, "hex_apply_multi_pair_kernel");
  return grid;
}

int hex_multi_pair_launch(gh1_op* op, int R, const int* phase, int want, const float* x, float* y, double* partial,
                          unsigned int* counter, double* energy, bool prepare_only) {
  const bool mass = op->has_mass;
  int g = 0;
#define GH1_MPAIR_CASE(NN)                                                                                         \
  case NN:                                                                                                         \
    g = mass ? multi_pair_launch_n<NN, true>(op, R, phase, want, x, y, partial, counter, energy, prepare_only)      \
             : multi_pair_launch_n<NN, false>(op, R, phase, want, x, y, partial, counter, energy, prepare_only);    \
    break;
  GH1_PAIR_SWITCH(op->sp->p + 1, GH1_MPAIR_CASE)
#undef GH1_MPAIR_CASE
  return g;
}

}  // namespace gh1
