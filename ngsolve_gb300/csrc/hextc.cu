// hextc.cu -- FP32 hex apply y += A x with the 1D contractions of the sum
// factorization on the 5th-generation tensor cores (tcgen05.mma, kind::tf32).
//
// Same operator as hex_apply_kernel (matfree.cu: sum-factorized
// SymbolicBFI::ApplyElementMatrix, fem/symbolicintegrator.cpp:2959-3040).  Each
// of the six 1D contraction stages (three forward, three transposed) is a GEMM
// D[M x 16] = A[M x 8] * T[16 x 8]^T:
//   - M = 128 rows = the pencils of EPT = floor(128 / N^2) elements of a tile
//     (row = e*N^2 + (first free index)*N + (second free index), padding rows
//     are zero), one row per thread of the 128-thread CTA;
//   - K = the contracted index (N <= 8, zero-padded to 8);
//   - the 16 columns = the outputs of one or two 1D tables (B and D stacked,
//     n < N and N <= n < 2N), the shared, reused operand.
// A and T live in shared memory (K-major, no swizzle: 8-row x 16-byte core
// matrices, LBO = 128 B between the two K halves, SBO = 256 B between 8-row
// groups); D lives in tensor memory (64 columns per CTA).  After each stage a
// thread reads its own row back (tcgen05.ld 32x32b) and writes the values into
// the next stage's A operand with the contraction index changed (the
// transpose of the sum factorization goes through shared memory).
// Accuracy: FP32 data and tables are split into TF32 high and low parts and
// every product is formed as hi*hi + lo*hi + hi*lo (3xTF32, accumulated in
// FP32 in tensor memory), which keeps the apply at FP32 accuracy.
// One thread issues the MMAs of a stage and commits them to an mbarrier; the
// CTA waits on it with a bounded wait (timeout: error flag, drain, return).
#include <algorithm>
#include <cstdlib>
#include "common.cuh"
#include "hexcore.cuh"

namespace gh1 {

template <int N>
struct TcCfg {
  static constexpr int N2 = N * N, N3 = N * N * N;
  static constexpr int EPT = 128 / N2;        // elements per tile
  static constexpr int ROWS = EPT * N2;       // valid rows of the M = 128 tile
  static constexpr int TV = EPT * N3;         // DOF slots per tile
  static constexpr int AF = 128 * 8;          // floats per A operand (hi or lo)
  static constexpr int TF = 16 * 8;           // floats per table operand
  static constexpr int NA = 4;                // A operands alive at once
  static constexpr int NT = 5;                // tables: BD, DB, B, B^T, D^T
  // float offsets in dynamic shared memory
  static constexpr int A_OFF = 0;                              // [NA][hi, lo][AF]
  static constexpr int T_OFF = A_OFF + NA * 2 * AF;            // [NT][hi, lo][TF]
  static constexpr int IDX_OFF = T_OFF + NT * 2 * TF;          // int[TV]
  static constexpr int OUT_OFF = IDX_OFF + ((TV + 3) / 4) * 4;  // float[TV]
  static constexpr int W_OFF = OUT_OFF + ((TV + 3) / 4) * 4;   // 1D weights [8]
  static constexpr int BAR_OFF = W_OFF + 8;                    // mbarrier (8 B) + TMEM base (4 B)
  static constexpr size_t smem = (size_t)(BAR_OFF + 4) * sizeof(float);
};

enum { TC_BD = 0, TC_DB = 1, TC_B = 2, TC_BT = 3, TC_DT = 4 };

__device__ __forceinline__ int tc_off(int r, int k) { return (r >> 3) * 64 + (k >> 2) * 32 + (r & 7) * 4 + (k & 3); }
__device__ __forceinline__ float tf32_hi(float v) { return __uint_as_float(__float_as_uint(v) & 0xffffe000u); }
// value into an A operand: TF32 high part and the FP32 remainder
__device__ __forceinline__ void tc_put(float* A, int r, int k, float v) {
  const float h = tf32_hi(v);
  A[tc_off(r, k)] = h;
  A[128 * 8 + tc_off(r, k)] = v - h;
}
__device__ __forceinline__ uint64_t tc_desc(const float* p) {
  return (uint64_t)((smem_u32(p) & 0x3FFFF) >> 4) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(256 >> 4) << 32) |
         (1ull << 46);
}
// kind::tf32, D = F32, A = B = TF32, both K-major, N = 16, M = 128
constexpr uint32_t TC_IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((16u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
               "l"(a), "l"(b), "r"(TC_IDESC), "r"(acc)
               : "memory");
}
// D (+)= A * T with the 3xTF32 split: hi*hi + lo*hi + hi*lo
__device__ __forceinline__ void tc_term(uint32_t d, const float* A, const float* T, bool first) {
  const uint64_t ah = tc_desc(A), al = tc_desc(A + 128 * 8), th = tc_desc(T), tl = tc_desc(T + 16 * 8);
  tc_mma(d, ah, th, first ? 0u : 1u);
  tc_mma(d, al, th, 1u);
  tc_mma(d, ah, tl, 1u);
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
// 16 consecutive TMEM columns of this thread's lane
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Stage hand-off: the A operands written by the threads become visible to the
// tensor core (async proxy), TMEM reads of the previous stage are ordered
// before the new MMAs, and thread 0 issues `issue()` and commits.
template <class F>
__device__ __forceinline__ void tc_stage(uint64_t* bar, F&& issue) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 0) {
    tc_fence_after();
    issue();
    tc_commit(bar);
  }
}

template <int N, bool MASS, bool AFF>
__global__ void __launch_bounds__(128)
hex_apply_tc_kernel(int ne, const int* __restrict__ tdof, int tstride, const float* __restrict__ Gq, int gstride,
                    const double* __restrict__ B64, const double* __restrict__ D64, const double* __restrict__ gw,
                    const float* __restrict__ x, float* __restrict__ y, int first_cell, double* partial,
                    unsigned int* counter, double* energy, const int* skip, int* err) {
  using C = TcCfg<N>;
  constexpr int N2 = C::N2, N3 = C::N3, EPT = C::EPT, ROWS = C::ROWS, TV = C::TV;
  if (skip && *(volatile const int*)skip) return;
  extern __shared__ __align__(1024) float tsm[];
  float* A = tsm + C::A_OFF;  // A operand k: A + k * 2 * AF (hi), + AF (lo)
  float* T = tsm + C::T_OFF;  // table k: T + k * 2 * TF (hi), + TF (lo)
  int* idx = (int*)(tsm + C::IDX_OFF);
  float* obuf = tsm + C::OUT_OFF;
  float* wq = tsm + C::W_OFF;
  uint64_t* bar = (uint64_t*)(tsm + C::BAR_OFF);
  uint32_t* tslot = (uint32_t*)(tsm + C::BAR_OFF + 2);
  const int t = threadIdx.x, warp = t >> 5;
  auto Aop = [&](int k) { return A + k * 2 * C::AF; };
  auto Top = [&](int k) { return T + k * 2 * C::TF; };

  // operands start at zero: padding rows and the K columns >= N stay zero
  for (int i = t; i < C::NA * 2 * C::AF; i += 128) A[i] = 0.f;
  // the five tables, split hi / lo from FP64: row n = output, column k = input
  for (int i = t; i < C::NT * 16 * 8; i += 128) {
    const int tb = i / 128, n = (i / 8) % 16, k = i % 8;
    double v = 0.0;
    if (k < N) {
      if (tb == TC_BD) v = n < N ? B64[n * N + k] : (n < 2 * N ? D64[(n - N) * N + k] : 0.0);
      else if (tb == TC_DB) v = n < N ? D64[n * N + k] : (n < 2 * N ? B64[(n - N) * N + k] : 0.0);
      else if (tb == TC_B) v = n < N ? B64[n * N + k] : 0.0;
      else if (tb == TC_BT) v = n < N ? B64[k * N + n] : 0.0;
      else v = n < N ? D64[k * N + n] : 0.0;
    }
    const float h = tf32_hi((float)v);
    float* Tb = Top(tb);
    Tb[tc_off(n, k)] = h;
    Tb[C::TF + tc_off(n, k)] = (float)(v - (double)h);
  }
  if (t < N) wq[t] = (float)gw[t];
  if (t == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" ::"r"(smem_u32(tslot)) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);  // this thread's lane, column 0
  const int ntiles = (ne + EPT - 1) / EPT;
  uint32_t ph = 0;
  bool ok = true;
  float acc = 0.f;
  float v[16], w2[16], w3[16];
  // row decomposition: r = e*N^2 + p*N + q (two free indices of the stage)
  const bool act = t < ROWS;
  const int re = t / N2, rp = (t / N) % N, rq = t % N;

  auto wait = [&]() {
    const bool got = mbar_wait_bounded(bar, ph);
    ph ^= 1u;
    tc_fence_after();
    return __syncthreads_and(got) != 0;
  };

  for (int tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x) {
    const int e0 = tile * EPT;
    // ---- DOF rows and the signed gather into A0[row (e,a,b)][c] ---------------
    for (int i = t; i < TV; i += 128) {
      const int e = i / N3, l = i % N3;
      idx[i] = e0 + e < ne ? tdof[(size_t)(e0 + e) * tstride + l] : -1;
    }
    __syncthreads();
    for (int i = t; i < TV; i += 128) {
      const int d = idx[i];
      float u = 0.f;
      if (d != -1) {
        u = __ldg(x + (d & 0x7fffffff));
        if (d < 0) u = -u;
      }
      const int e = i / N3, l = i % N3;
      tc_put(Aop(0), e * N2 + l / N, l % N, u);
    }
    // ---- forward 1: contract c: s1 = B u, s2 = D u (cols 0..2N) ---------------
    tc_stage(bar, [&] { tc_term(tmem, Aop(0), Top(TC_BD), true); });
    if (!(ok = wait())) break;
    tc_ld16(tl, v);
    if (act) {  // row (e,a,b) -> rows (e,a,k), column b
#pragma unroll
      for (int k = 0; k < N; k++) {
        tc_put(Aop(1), re * N2 + rp * N + k, rq, v[k]);
        tc_put(Aop(2), re * N2 + rp * N + k, rq, v[N + k]);
      }
    }
    // ---- forward 2: contract b: t1 = B s1, t2 = D s1 (cols 0..), t3 = B s2 (16..)
    tc_stage(bar, [&] {
      tc_term(tmem, Aop(1), Top(TC_BD), true);
      tc_term(tmem + 16, Aop(2), Top(TC_B), true);
    });
    if (!(ok = wait())) break;
    tc_ld16(tl, v);
    tc_ld16(tl + 16, w3);
    if (act) {  // row (e,a,k) -> rows (e,j,k), column a
#pragma unroll
      for (int j = 0; j < N; j++) {
        tc_put(Aop(1), re * N2 + j * N + rq, rp, v[j]);
        tc_put(Aop(2), re * N2 + j * N + rq, rp, v[N + j]);
        tc_put(Aop(3), re * N2 + j * N + rq, rp, w3[j]);
      }
    }
    // ---- forward 3: contract a: gx = D t1, uq = B t1 (0..), gy = B t2 (16..),
    // gz = B t3 (32..)
    tc_stage(bar, [&] {
      tc_term(tmem, Aop(1), Top(TC_DB), true);
      tc_term(tmem + 16, Aop(2), Top(TC_B), true);
      tc_term(tmem + 32, Aop(3), Top(TC_B), true);
    });
    if (!(ok = wait())) break;
    tc_ld16(tl, v);
    tc_ld16(tl + 16, w2);
    tc_ld16(tl + 32, w3);
    // ---- metric at the points (i, j, k) of row (e,j,k): own row, column i ------
    if (act) {
      const int e = e0 + re;
      const bool valid = e < ne;
      float ea[7];
      if (AFF) {
#pragma unroll
        for (int c = 0; c < 7; c++) ea[c] = valid && (c < 6 || MASS) ? __ldg(Gq + (size_t)e * 8 + c) : 0.f;
      }
      const float wjk = wq[rp] * wq[rq];
#pragma unroll
      for (int i = 0; i < N; i++) {
        const float gx = v[i], uq = v[N + i], gy = w2[i], gz = w3[i];
        float gxx, gyy, gzz, gxy, gxz, gyz, gm = 0.f;
        if (AFF) {
          const float wt = wq[i] * wjk;
          gxx = wt * ea[0]; gyy = wt * ea[1]; gzz = wt * ea[2];
          gxy = wt * ea[3]; gxz = wt * ea[4]; gyz = wt * ea[5];
          if (MASS) gm = wt * ea[6];
        } else {
          const float* Ge = Gq + (size_t)(valid ? e : 0) * gstride + i * N2 + rp * N + rq;
          gxx = valid ? __ldcs(Ge) : 0.f; gyy = valid ? __ldcs(Ge + N3) : 0.f; gzz = valid ? __ldcs(Ge + 2 * N3) : 0.f;
          gxy = valid ? __ldcs(Ge + 3 * N3) : 0.f; gxz = valid ? __ldcs(Ge + 4 * N3) : 0.f;
          gyz = valid ? __ldcs(Ge + 5 * N3) : 0.f;
          if (MASS) gm = valid ? __ldcs(Ge + 6 * N3) : 0.f;
        }
        const float vx = gxx * gx + gxy * gy + gxz * gz;
        const float vy = gxy * gx + gyy * gy + gyz * gz;
        const float vz = gxz * gx + gyz * gy + gzz * gz;
        acc += gx * vx + gy * vy + gz * vz;
        tc_put(Aop(0), t, i, vx);
        tc_put(Aop(1), t, i, vy);
        tc_put(Aop(2), t, i, vz);
        if (MASS) {
          const float vm = gm * uq;
          acc += uq * vm;
          tc_put(Aop(3), t, i, vm);
        }
      }
    }
    // ---- backward 1: contract i: w1 = D^T vx (+ B^T vm), w2 = B^T vy, w3 = B^T vz
    tc_stage(bar, [&] {
      tc_term(tmem, Aop(0), Top(TC_DT), true);
      if (MASS) tc_term(tmem, Aop(3), Top(TC_BT), false);
      tc_term(tmem + 16, Aop(1), Top(TC_BT), true);
      tc_term(tmem + 32, Aop(2), Top(TC_BT), true);
    });
    if (!(ok = wait())) break;
    tc_ld16(tl, v);
    tc_ld16(tl + 16, w2);
    tc_ld16(tl + 32, w3);
    if (act) {  // row (e,j,k) -> rows (e,a,k), column j
#pragma unroll
      for (int a = 0; a < N; a++) {
        tc_put(Aop(0), re * N2 + a * N + rq, rp, v[a]);
        tc_put(Aop(1), re * N2 + a * N + rq, rp, w2[a]);
        tc_put(Aop(2), re * N2 + a * N + rq, rp, w3[a]);
      }
    }
    // ---- backward 2: contract j: v1 = B^T w1 + D^T w2 (0..), v2 = B^T w3 (16..)
    tc_stage(bar, [&] {
      tc_term(tmem, Aop(0), Top(TC_BT), true);
      tc_term(tmem, Aop(1), Top(TC_DT), false);
      tc_term(tmem + 16, Aop(2), Top(TC_BT), true);
    });
    if (!(ok = wait())) break;
    tc_ld16(tl, v);
    tc_ld16(tl + 16, w2);
    if (act) {  // row (e,a,k) -> rows (e,a,b), column k
#pragma unroll
      for (int b = 0; b < N; b++) {
        tc_put(Aop(0), re * N2 + rp * N + b, rq, v[b]);
        tc_put(Aop(1), re * N2 + rp * N + b, rq, w2[b]);
      }
    }
    // ---- backward 3: contract k: out = B^T v1 + D^T v2 -------------------------
    tc_stage(bar, [&] {
      tc_term(tmem, Aop(0), Top(TC_BT), true);
      tc_term(tmem, Aop(1), Top(TC_DT), false);
    });
    if (!(ok = wait())) break;
    tc_ld16(tl, v);
    if (act) {  // row (e,a,b): out[c] at tile slot e*N^3 + (a*N+b)*N + c
#pragma unroll
      for (int c = 0; c < N; c++) obuf[re * N3 + (rp * N + rq) * N + c] = v[c];
    }
    __syncthreads();
    // ---- signed scatter in DOF order: element-interior DOFs have one writer ---
    for (int i = t; i < TV; i += 128) {
      const int d = idx[i];
      if (d == -1) continue;
      const int dof = d & 0x7fffffff;
      const float val = d < 0 ? -obuf[i] : obuf[i];
      if (dof >= first_cell) y[dof] = val;
      else red_add(y + dof, val);
    }
    __syncthreads();  // idx / obuf / A0 are rewritten by the next tile
  }
  if (!ok) {
    // a commit is outstanding only if the failed wait was its first: give it a
    // bounded chance to land before TMEM is released
    if (t == 0) {
      atomicExch(err, 1);
      mbar_wait_bounded(bar, ph ^ 1u);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" ::"r"(tmem) : "memory");
  if (partial) block_reduce_finish((double)acc, partial, counter, energy);
}

// ---- host side -----------------------------------------------------------------
bool hex_tc_supported(int N) { return N >= 5 && N <= 8; }

template <int N, bool MASS, bool AFF>
static int tc_occupancy() {
  auto kern = hex_apply_tc_kernel<N, MASS, AFF>;
  GH1_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TcCfg<N>::smem));
  // the largest shared-memory carveout: several CTAs per SM hide each other's
  // MMA round trips (without it the occupancy query assumed one CTA per SM)
  GH1_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared));
  int v = 0;
  GH1_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kern, 128, TcCfg<N>::smem));
  // The query reports one CTA per SM for this kernel; the shared memory and
  // registers allow more (ncu's limits for the launch agree), and the persistent
  // tile loop is correct for any grid, so size the grid by those limits.
  int dev = 0, smem_sm = 0, regs_sm = 0;
  GH1_CUDA(cudaGetDevice(&dev));
  GH1_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
  GH1_CUDA(cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev));
  cudaFuncAttributes fa;
  GH1_CUDA(cudaFuncGetAttributes(&fa, kern));
  const int by_smem = smem_sm / (int)(TcCfg<N>::smem + fa.sharedSizeBytes + 1024);
  const int by_regs = regs_sm / (128 * ((fa.numRegs + 7) / 8 * 8));
  v = std::max(v, std::min(by_smem, by_regs));
  // 64 TMEM columns per CTA: at most 8 resident CTAs share the SM's 512 columns
  return std::min(v, 8);
}

#define GH1_TC_SWITCH(N, CASE)                                                            \
  switch (N) {                                                                            \
    CASE(5) CASE(6) CASE(7) CASE(8)                                                       \
    default: throw Error(GH1_ERR_UNSUPPORTED, "tensor-core hex apply: order out of range"); \
  }

// resident CTAs per SM of the tensor-core apply for this operator (0: not available)
int hex_tc_occupancy(gh1_op* op) {
  const int N = op->sp->p + 1;
  const char* env = getenv("GH1_HEX_TC");
  if (!hex_tc_supported(N) || (env && env[0] == '0')) return 0;
  const bool m = op->has_mass, aff = op->all_affine;
  int v = 0;
#define GH1_TC_OCC(NN)                                                                                 \
  case NN:                                                                                             \
    v = m ? (aff ? tc_occupancy<NN, true, true>() : tc_occupancy<NN, true, false>())                  \
          : (aff ? tc_occupancy<NN, false, true>() : tc_occupancy<NN, false, false>());               \
    break;
  GH1_TC_SWITCH(N, GH1_TC_OCC)
#undef GH1_TC_OCC
  return v;
}

template <int N, bool MASS, bool AFF>
static void tc_launch(gh1_op* op, const float* x, float* y, double* partial, unsigned int* counter, double* energy,
                      const int* skip) {
  gh1_space* sp = op->sp;
  GH1_CHECK(op->tc_per_sm > 0, GH1_ERR_ARG, "internal: tensor-core hex apply occupancy not prepared");
  const int ne = sp->mesh->ne;
  const int ntiles = (ne + TcCfg<N>::EPT - 1) / TcCfg<N>::EPT;
  const int grid = std::max(1, std::min(ntiles, sp->ctx->nsm * op->tc_per_sm));
  const float* G = AFF ? op->d_Ga32.p : op->d_G32.p;
  hex_apply_tc_kernel<N, MASS, AFF><<<grid, 128, TcCfg<N>::smem, sp->ctx->stream>>>(
      ne, sp->d_tdof.p, sp->tstride, G, AFF ? 8 : op->gstride32, sp->d_B64.p, sp->d_D64.p, sp->d_gw.p, x, y,
      (int)sp->first_cell, partial, counter, energy, skip, op->d_err.p);
  check_kernel(sp->ctx, "hex_apply_tc_kernel");
}

void hex_tc_apply(gh1_op* op, const float* x, float* y, double* partial, unsigned int* counter, double* energy,
                  const int* skip) {
  const bool m = op->has_mass, aff = op->all_affine;
#define GH1_TC_CASE(NN)                                                                                        \
  case NN:                                                                                                     \
    if (m) { if (aff) tc_launch<NN, true, true>(op, x, y, partial, counter, energy, skip);                    \
             else tc_launch<NN, true, false>(op, x, y, partial, counter, energy, skip); }                      \
    else { if (aff) tc_launch<NN, false, true>(op, x, y, partial, counter, energy, skip);                     \
           else tc_launch<NN, false, false>(op, x, y, partial, counter, energy, skip); }                       \
    break;
  GH1_TC_SWITCH(op->sp->p + 1, GH1_TC_CASE)
#undef GH1_TC_CASE
}

}  // namespace gh1
