// tettc.cu -- FP32 tet apply y += A x with both products of a tile on the
// 5th-generation tensor cores (tcgen05.mma, kind::tf32).
//
// Same operator as tet_tile_kernel (tetapply.cu) and the reference's element-wise
// ApplyElementMatrix (fem/symbolicintegrator.cpp:2959-3040) on affine tets:
// y_e = B^T diag(w_q kappa_e |det J| J^{-1} J^{-T}) B x_e.  All elements of one
// orientation class share one table D_c[i][r] of reference gradients at the rule
// points (r = component * nq + point), so a tile of up to 128 same-class
// elements is two GEMMs with the table as the shared, reused operand:
//   P[m][r] = sum_i X[m][i] D_c[i][r]     (M = 128 elements, K = nloc, N = 3 nq)
//   V[m][r] = w_q G_m (P[m][.] at point q)   (per element and point, registers)
//   Y[m][i] = sum_r V[m][r] D_c[i][r]     (M = 128 elements, K = 3 nq, N = nloc)
// Two threads own one element (one row of X, P, V, Y; the second warpgroup
// reads the same tensor-memory lanes as the first): each gathers half of its
// DOFs, writes half of its operand row, reads the accumulator row back from
// tensor memory (tcgen05.ld 32x32b), applies the metric to half of the columns
// and scatters half of the result with atomics.  No transposes between the
// products.  Operands are K-major without swizzle
// (8-row x 16-byte core matrices, LBO = 128 B along K, SBO = K/4 x 128 B per
// 8-row group); FP32 values are split into TF32 high and low parts and every
// product is hi*hi + lo*hi + hi*lo (3xTF32), accumulated in FP32 in tensor memory.
#include <algorithm>
#include <cstdlib>
#include <type_traits>
#include <vector>
#include "common.cuh"
#include "hexcore.cuh"

namespace gh1 {

template <int P>
struct TetTcCfg {
  static constexpr int NLOC = (P + 1) * (P + 2) * (P + 3) / 6;
  static constexpr int NQ = P == 2 ? 4 : P == 3 ? 14 : 24;  // stiffness rule points (tables.cu tet_rule)
  static constexpr int R = 3 * NQ;
  static constexpr int K1 = (NLOC + 7) / 8 * 8;    // forward K (local DOFs)
  static constexpr int N1 = (R + 15) / 16 * 16;    // forward N (gradient rows)
  static constexpr int K2 = (R + 7) / 8 * 8;       // backward K
  static constexpr int N2 = (NLOC + 15) / 16 * 16; // backward N
  static constexpr int C2 = N1;                     // TMEM column of the backward accumulator
  static constexpr int TCOLS = (N1 + N2) <= 32 ? 32 : (N1 + N2) <= 64 ? 64 : (N1 + N2) <= 128 ? 128 : 256;
  // the backward product runs in two K chunks of V (columns [0, KA) and
  // [KA, K2)), so its operand needs no more room than the forward one: two
  // CTAs fit on an SM and one's products overlap the other's gather / scatter
  static constexpr int KA = K2 <= K1 ? K2 : K1;     // first chunk (a multiple of 8)
  static constexpr int KB = K2 - KA;                // second chunk (0: one chunk)
  // float offsets in dynamic shared memory; A1 and the A2 chunks share their
  // space (each is read by its product, which completes before the next is written)
  static constexpr int A1 = 0;                      // [hi, lo][128][K1]
  static constexpr int A2 = 0;                      // [hi, lo][128][KA] and then [hi, lo][128][KB]
  static constexpr int AW = 2 * 128 * (K1 > KA ? K1 : KA);
  static constexpr int T1 = AW;                     // [hi, lo][N1][K1]
  static constexpr int T2 = T1 + 2 * N1 * K1;       // [hi, lo][N2][K2]
  static constexpr int W = T2 + 2 * N2 * K2;        // weights [R] (padded to 4)
  static constexpr int BAR = W + (R + 3) / 4 * 4;   // mbarrier (8 B) + TMEM base (4 B)
  static constexpr size_t smem = (size_t)(BAR + 4) * sizeof(float);
  static constexpr int TAB = 2 * N1 * K1 + 2 * N2 * K2;  // floats of one class's operands (T1, T2)
};

// element (row r, column k) of a K-major operand with K columns
template <int K>
__device__ __forceinline__ int tt_off(int r, int k) { return (r >> 3) * (K * 8) + (k >> 2) * 32 + (r & 7) * 4 + (k & 3); }

__device__ __forceinline__ float tt_hi(float v) { return __uint_as_float(__float_as_uint(v) & 0xffffe000u); }

template <int K>
__device__ __forceinline__ uint64_t tt_desc(const float* p) {
  return (uint64_t)((smem_u32(p) & 0x3FFFF) >> 4) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)((K * 32) >> 4) << 32) |
         (1ull << 46);
}
// kind::tf32, D = F32, A = B = TF32, both K-major, M = 128
template <int N>
__device__ __forceinline__ uint32_t tt_idesc() {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((128u >> 4) << 24);
}
__device__ __forceinline__ void tt_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
               "l"(a), "l"(b), "r"(idesc), "r"(acc)
               : "memory");
}
// D (+)= A * T^T over the K columns [K0, K0 + KC) of T (KC/8 steps of 8),
// 3xTF32: A is [hi][128][KC] then [lo], T is [hi][ROWS_T][KT] then [lo];
// ACC: add to D from the first step on
template <int KC, int KT, int K0, int N, int ROWS_T, bool ACC>
__device__ __forceinline__ void tt_gemm(uint32_t d, const float* A, const float* T) {
  const uint32_t idesc = tt_idesc<N>();
  const float* Al = A + 128 * KC;
  const float* Tl = T + ROWS_T * KT;
#pragma unroll
  for (int s = 0; s < KC / 8; s++) {
    const int o = s * 64, ot = (K0 / 8 + s) * 64;  // two core matrices (2 x 32 floats) per K step of 8
    tt_mma(d, tt_desc<KC>(A + o), tt_desc<KT>(T + ot), idesc, (ACC || s > 0) ? 1u : 0u);
    tt_mma(d, tt_desc<KC>(Al + o), tt_desc<KT>(T + ot), idesc, 1u);
    tt_mma(d, tt_desc<KC>(A + o), tt_desc<KT>(Tl + ot), idesc, 1u);
  }
}
__device__ __forceinline__ void tt_ld16(uint32_t taddr, float* v) {
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
// one row of four consecutive K values (hi and lo parts), 16-byte stores
template <int K>
__device__ __forceinline__ void tt_put4(float* A, int r, int k, const float* v) {
  float h[4], l[4];
#pragma unroll
  for (int j = 0; j < 4; j++) { h[j] = tt_hi(v[j]); l[j] = v[j] - h[j]; }
  *(float4*)(A + tt_off<K>(r, k)) = make_float4(h[0], h[1], h[2], h[3]);
  *(float4*)(A + 128 * K + tt_off<K>(r, k)) = make_float4(l[0], l[1], l[2], l[3]);
}

// tiles: [ntiles][4] = class, first position in perm, element count (<= 128), 0
constexpr int TT_THREADS = 256;

// resident CTAs the register allocation must allow: 3 at p = 3 (shared memory
// and TMEM hold 4), 2 at p = 4 (shared memory holds 2); p = 2 fits 4 as compiled
template <int P>
__global__ void __launch_bounds__(TT_THREADS, P == 3 ? 3 : 2)
tet_tc_kernel(int ntiles, const int* __restrict__ tiles, const int* __restrict__ tdofs, const float* __restrict__ Gt,
              const float* __restrict__ tab, const double* __restrict__ W64,
              const float* __restrict__ x, float* __restrict__ y, double* partial, unsigned int* counter,
              double* energy, const int* skip, int* err) {
  using C = TetTcCfg<P>;
  constexpr int NLOC = C::NLOC, NQ = C::NQ, R = C::R, K1 = C::K1, N1 = C::N1, K2 = C::K2, N2 = C::N2;
  if (skip && *(volatile const int*)skip) return;
  extern __shared__ __align__(1024) float ts[];
  float* sA1 = ts + C::A1;
  float* sA2 = ts + C::A2;
  float* sT1 = ts + C::T1;
  float* sT2 = ts + C::T2;
  float* sW = ts + C::W;
  uint64_t* bar = (uint64_t*)(ts + C::BAR);
  uint32_t* tslot = (uint32_t*)(ts + C::BAR + 2);
  const int t = threadIdx.x, warp = t >> 5, m = t & 127, half = t >> 7;  // element row m, half of its work
  // zero operands: padding columns (K >= nloc, K >= R) stay zero
  for (int i = t; i < C::AW; i += TT_THREADS) ts[i] = 0.f;
  for (int i = t; i < R; i += TT_THREADS) sW[i] = (float)W64[i];
  if (t == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)), "r"(C::TCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  const uint32_t tl = tmem + ((uint32_t)((warp & 3) * 32) << 16);  // lanes of row m
  uint32_t ph = 0;
  bool ok = true;
  double acc = 0.0;
  int loaded = -1;
  auto issue_stage = [&](auto&& issue) {  // operands visible to the tensor core, issue, commit
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (t == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      issue();
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                   : "memory");
    }
  };
  auto wait_stage = [&]() {
    const bool got = mbar_wait_bounded(bar, ph);
    ph ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    return __syncthreads_and(got) != 0;
  };
  // this thread's half of an element's DOF values: loaded for the next tile
  // while the current tile's second product runs
  constexpr int H1 = K1 / 2;  // a multiple of 4
  float xv[H1];
  // DOF of local DOF i of this thread's row in tile tl_ (tile-major table: the
  // 32 rows of a warp read 128 consecutive bytes)
  auto dof_of = [&](int tl_, int i) { return __ldg(tdofs + ((size_t)tl_ * NLOC + i) * 128 + m); };
  auto gather = [&](int tl_) {
    const bool a = m < tiles[4 * tl_ + 2];
#pragma unroll
    for (int j = 0; j < H1; j++) {
      const int i = half * H1 + j;
      xv[j] = (a && i < NLOC) ? __ldg(x + dof_of(tl_, i)) : 0.f;
    }
  };
  // a contiguous range of the class-sorted tiles per CTA: consecutive tiles
  // share their class, so the class operands are copied only where it changes
  const int t0 = (int)((long long)ntiles * blockIdx.x / gridDim.x);
  const int t1 = (int)((long long)ntiles * (blockIdx.x + 1) / gridDim.x);
  if (t0 < t1) gather(t0);
  for (int tile = t0; ok && tile < t1; tile++) {
    const int cls = tiles[4 * tile], cnt = tiles[4 * tile + 2];
    if (cls != loaded) {  // both B operands of the class (TF32 hi / lo, final layout)
      __syncthreads();    // the previous tile's products have completed (its last wait)
      const float4* src = (const float4*)(tab + (size_t)cls * C::TAB);
      float4* dst = (float4*)sT1;
      for (int k = t; k < C::TAB / 4; k += TT_THREADS) dst[k] = __ldg(src + k);
      loaded = cls;
    }
    // ---- the gathered half of this row's element into A1 ---------------------------
    const bool act = m < cnt;
#pragma unroll
    for (int j = 0; j < H1; j += 4) tt_put4<K1>(sA1, m, half * H1 + j, xv + j);
    // ---- P = X D_c ------------------------------------------------------------------
    issue_stage([&] { tt_gemm<K1, K1, 0, N1, N1, false>(tmem, sA1, sT1); });
    if (!(ok = wait_stage())) break;
    float pv[N1];
#pragma unroll
    for (int c = 0; c < N1; c += 16) tt_ld16(tl + c, pv + c);
    // ---- metric at the points, into row m of the A2 chunk: this half writes the
    // column groups [4j, 4j+4) with j = half (mod 2); column r = component * nq + point
    float g[6];
#pragma unroll
    for (int c = 0; c < 6; c++) g[c] = act ? __ldg(Gt + ((size_t)tile * 6 + c) * 128 + m) : 0.f;
    float en = 0.f;
    auto transform = [&](auto k0c, auto kcc) {  // columns [K0, K0 + KC) into an operand with KC columns
      constexpr int K0 = decltype(k0c)::value, KC = decltype(kcc)::value;
#pragma unroll
      for (int j = 0; j < KC / 4; j++) {
        if (((K0 / 4 + j) & 1) != half) continue;
        float vv[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
          const int r = K0 + 4 * j + k;
          float v = 0.f;
          if (r < R) {
            const int q = r % NQ, c = r / NQ;
            const float ux = pv[q], uy = pv[NQ + q], uz = pv[2 * NQ + q];
            const float gx = c == 0 ? g[0] : c == 1 ? g[3] : g[4];
            const float gy = c == 0 ? g[3] : c == 1 ? g[1] : g[5];
            const float gz = c == 0 ? g[4] : c == 1 ? g[5] : g[2];
            v = sW[q] * (gx * ux + gy * uy + gz * uz);
            if (partial) en += pv[r] * v;
          }
          vv[k] = v;
        }
        tt_put4<KC>(sA2, m, 4 * j, vv);
      }
    };
    // ---- Y = V D_c^T in its K chunks (the next tile's gather overlaps the last),
    // then the scatter ----------------------------------------------------------------
    transform(std::integral_constant<int, 0>(), std::integral_constant<int, C::KA>());
    issue_stage([&] { tt_gemm<C::KA, K2, 0, N2, N2, false>(tmem + C::C2, sA2, sT2); });
    if constexpr (C::KB > 0) {
      if (!(ok = wait_stage())) break;
      transform(std::integral_constant<int, C::KA>(), std::integral_constant<int, C::KB>());
      issue_stage([&] { tt_gemm<C::KB, K2, C::KA, N2, N2, true>(tmem + C::C2, sA2, sT2); });
    }
    if (partial) acc += (double)en;
    if (tile + 1 < t1) gather(tile + 1);
    if (!(ok = wait_stage())) break;
    float yv[N2];
#pragma unroll
    for (int c = 0; c < N2; c += 16) tt_ld16(tl + C::C2 + c, yv + c);
    if (act) {  // compile-time register indices in both halves
      constexpr int HS = (NLOC + 1) / 2;
      if (half == 0) {
#pragma unroll
        for (int i = 0; i < HS; i++) red_add(y + dof_of(tile, i), yv[i]);
      } else {
#pragma unroll
        for (int i = HS; i < NLOC; i++) red_add(y + dof_of(tile, i), yv[i]);
      }
    }
  }
  if (!ok && t == 0) {
    atomicExch(err, 1);
    mbar_wait_bounded(bar, ph ^ 1u);  // the commit the failed wait gave up on
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(C::TCOLS) : "memory");
  if (partial) block_reduce_finish(acc, partial, counter, energy);
}

// ---- host side -------------------------------------------------------------------
bool tet_tc_supported(int p) { return p >= 2 && p <= 4; }

template <int P>
static int tet_tc_occupancy_p() {
  auto kern = tet_tc_kernel<P>;
  GH1_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TetTcCfg<P>::smem));
  // resident CTAs by shared memory and by registers (a grid above both would run
  // a second, partly empty wave: p = 2 holds 4 CTAs by registers, 10 by shared
  // memory), and by TMEM: at most 512 columns per SM
  int dev = 0, smem_sm = 0, regs_sm = 0;
  GH1_CUDA(cudaGetDevice(&dev));
  GH1_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
  GH1_CUDA(cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev));
  cudaFuncAttributes fa;
  GH1_CUDA(cudaFuncGetAttributes(&fa, kern));
  const int by_smem = smem_sm / (int)(TetTcCfg<P>::smem + fa.sharedSizeBytes + 1024);
  const int by_regs = regs_sm / (TT_THREADS * ((fa.numRegs + 7) / 8 * 8));
  return std::min(std::min(by_smem, by_regs), 512 / TetTcCfg<P>::TCOLS);
}

// per class: the table D_c as the B operand of both products, split into TF32
// high and low parts from FP64, in the kernel's shared-memory layout
// ([hi, lo][N1][K1] then [hi, lo][N2][K2]; zero padding)
template <int P>
__global__ void tet_tc_table_kernel(int ncls, const double* __restrict__ D64, int nlocp, int Rs, float* __restrict__ tab) {
  using C = TetTcCfg<P>;
  constexpr int NLOC = C::NLOC, R = C::R, K1 = C::K1, N1 = C::N1, K2 = C::K2, N2 = C::N2;
  const int64_t tot = (int64_t)ncls * (N1 * K1 + N2 * K2);
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < tot; k += (int64_t)gridDim.x * blockDim.x) {
    const int cls = (int)(k / (N1 * K1 + N2 * K2)), j = (int)(k % (N1 * K1 + N2 * K2));
    const double* Dc = D64 + (size_t)cls * nlocp * Rs;
    float* T1 = tab + (size_t)cls * C::TAB;
    float* T2 = T1 + 2 * N1 * K1;
    if (j < N1 * K1) {
      const int n = j / K1, i = j % K1;
      const double v = (n < R && i < NLOC) ? Dc[(size_t)i * Rs + n] : 0.0;
      const float h = tt_hi((float)v);
      T1[tt_off<K1>(n, i)] = h;
      T1[N1 * K1 + tt_off<K1>(n, i)] = (float)(v - (double)h);
    } else {
      const int jj = j - N1 * K1, i = jj / K2, r = jj % K2;
      const double v = (i < NLOC && r < R) ? Dc[(size_t)i * Rs + r] : 0.0;
      const float h = tt_hi((float)v);
      T2[tt_off<K2>(i, r)] = h;
      T2[N2 * K2 + tt_off<K2>(i, r)] = (float)(v - (double)h);
    }
  }
}

template <int P>
static void tet_tc_table_p(gh1_op* op) {
  using C = TetTcCfg<P>;
  gh1_space* sp = op->sp;
  op->d_tet_tc_tab.alloc((size_t)N_TET_CLASSES * C::TAB);
  const int64_t tot = (int64_t)N_TET_CLASSES * (C::N1 * C::K1 + C::N2 * C::K2);
  tet_tc_table_kernel<P><<<(unsigned)((tot + 255) / 256), 256, 0, sp->ctx->stream>>>(
      N_TET_CLASSES, op->d_tetD64.p, (sp->nloc + 15) / 16 * 16, op->tet_Rs, op->d_tet_tc_tab.p);
  check_kernel(sp->ctx, "tet_tc_table_kernel");
}

// tile-major DOF table: tdofs[(t * nloc + i) * 128 + m] = DOF i of the element in
// row m of tile t (0 past the tile's count)
__global__ void tet_tc_dofs_kernel(int ntiles, int nloc, const int* __restrict__ tiles, const int* __restrict__ perm,
                                   const int* __restrict__ eldofs, int* __restrict__ tdofs) {
  const int64_t tot = (int64_t)ntiles * nloc * 128;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < tot; k += (int64_t)gridDim.x * blockDim.x) {
    const int m = (int)(k % 128), i = (int)((k / 128) % nloc), t = (int)(k / (128 * (int64_t)nloc));
    const int st = tiles[4 * t + 1], cnt = tiles[4 * t + 2];
    tdofs[k] = m < cnt ? eldofs[(size_t)perm[st + m] * nloc + i] : 0;
  }
}

// tile-major metric: Gt[(t * 6 + c) * 128 + m] = component c of the FP32 metric
// of the element in row m of tile t (0 past the tile's count)
__global__ void tet_tc_g_kernel(int ntiles, const int* __restrict__ tiles, const int* __restrict__ perm,
                                const float* __restrict__ G, float* __restrict__ Gt) {
  const int64_t tot = (int64_t)ntiles * 6 * 128;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < tot; k += (int64_t)gridDim.x * blockDim.x) {
    const int m = (int)(k % 128), c = (int)((k / 128) % 6), t = (int)(k / (128 * 6));
    const int st = tiles[4 * t + 1], cnt = tiles[4 * t + 2];
    Gt[k] = m < cnt ? G[(size_t)perm[st + m] * 6 + c] : 0.f;
  }
}

// tiles of up to 128 same-class elements (consecutive 32-element tiles of the
// class-sorted order merged) and their tile-major DOF table
static void tet_tc_build_tiles(gh1_op* op) {
  gh1_space* sp = op->sp;
  cudaStream_t s = sp->ctx->stream;
  std::vector<int> small(4 * (size_t)op->tet_ntiles);
  GH1_CUDA(cudaMemcpyAsync(small.data(), op->d_tet_tiles.p, small.size() * sizeof(int), cudaMemcpyDeviceToHost, s));
  GH1_CUDA(cudaStreamSynchronize(s));
  std::vector<int> tiles;
  for (int k = 0; k < op->tet_ntiles; k++) {
    const int c = small[4 * k], a = small[4 * k + 1], n = small[4 * k + 2];
    const size_t m = tiles.size();
    if (m && tiles[m - 4] == c && tiles[m - 3] + tiles[m - 2] == a && tiles[m - 2] + n <= 128) {
      tiles[m - 2] += n;
    } else {
      tiles.insert(tiles.end(), {c, a, n, 0});
    }
  }
  op->d_tet_tc_tiles.upload(tiles, s);
  op->tet_tc_ntiles = (int)tiles.size() / 4;
  op->d_tet_tc_dofs.alloc((size_t)op->tet_tc_ntiles * sp->nloc * 128);
  const int64_t tot = (int64_t)op->tet_tc_ntiles * sp->nloc * 128;
  tet_tc_dofs_kernel<<<(unsigned)std::min<int64_t>((tot + 255) / 256, 65535), 256, 0, s>>>(
      op->tet_tc_ntiles, sp->nloc, op->d_tet_tc_tiles.p, op->d_tet_perm.p, sp->d_eldofs.p, op->d_tet_tc_dofs.p);
  check_kernel(sp->ctx, "tet_tc_dofs_kernel");
  GH1_CUDA(cudaStreamSynchronize(s));  // host staging goes out of scope
}

// tiles of up to 128 same-class elements over the class-sorted order of the
// tiled apply, and the CTAs per SM (0: not available: order, mass term,
// GH1_TET_TC=0)
void tet_tc_setup(gh1_op* op) {
  gh1_space* sp = op->sp;
  op->tet_tc_per_sm = 0;
  const char* env = getenv("GH1_TET_TC");
  if (!tet_tc_supported(sp->p) || op->has_mass || !(op->prec_mask & 2) || op->tet_ntiles == 0 || op->tet_chunked ||
      (env && env[0] == '0'))
    return;
  cudaStream_t s = sp->ctx->stream;
  tet_tc_build_tiles(op);
  {
    op->d_tet_tc_G.alloc((size_t)op->tet_tc_ntiles * 6 * 128);
    const int64_t tg = (int64_t)op->tet_tc_ntiles * 6 * 128;
    tet_tc_g_kernel<<<(unsigned)std::min<int64_t>((tg + 255) / 256, 65535), 256, 0, s>>>(
        op->tet_tc_ntiles, op->d_tet_tc_tiles.p, op->d_tet_perm.p, op->d_G32.p, op->d_tet_tc_G.p);
    check_kernel(sp->ctx, "tet_tc_g_kernel");
  }
  switch (sp->p) {
    case 2: op->tet_tc_per_sm = tet_tc_occupancy_p<2>(); tet_tc_table_p<2>(op); break;
    case 3: op->tet_tc_per_sm = tet_tc_occupancy_p<3>(); tet_tc_table_p<3>(op); break;
    case 4: op->tet_tc_per_sm = tet_tc_occupancy_p<4>(); tet_tc_table_p<4>(op); break;
    default: break;
  }
  GH1_CUDA(cudaStreamSynchronize(s));
}

template <int P>
static void tet_tc_launch_p(gh1_op* op, const float* x, float* y, double* partial, unsigned int* counter,
                            double* energy, const int* skip) {
  gh1_space* sp = op->sp;
  const int grid = std::max(1, std::min(op->tet_tc_ntiles, sp->ctx->nsm * op->tet_tc_per_sm));
  tet_tc_kernel<P><<<grid, TT_THREADS, TetTcCfg<P>::smem, sp->ctx->stream>>>(
      op->tet_tc_ntiles, op->d_tet_tc_tiles.p, op->d_tet_tc_dofs.p, op->d_tet_tc_G.p, op->d_tet_tc_tab.p,
      op->d_tetw64.p, x, y, partial, counter, energy, skip, op->d_err.p);
  check_kernel(sp->ctx, "tet_tc_kernel");
}

void tet_tc_apply(gh1_op* op, const float* x, float* y, double* partial, unsigned int* counter, double* energy,
                  const int* skip) {
  GH1_CHECK(op->tet_tc_per_sm > 0, GH1_ERR_ARG, "internal: tensor-core tet apply not prepared");
  switch (op->sp->p) {
    case 2: tet_tc_launch_p<2>(op, x, y, partial, counter, energy, skip); break;
    case 3: tet_tc_launch_p<3>(op, x, y, partial, counter, energy, skip); break;
    case 4: tet_tc_launch_p<4>(op, x, y, partial, counter, energy, skip); break;
    default: throw Error(GH1_ERR_UNSUPPORTED, "tensor-core tet apply: order out of range");
  }
}


// ---- generic B^T D B on the tensor cores (records per element) -------------------
// The same machinery for a(u, v) = sum_e int_e (B v)^T D_e (B u), B w = (w, grad w),
// on affine tets with one reference-coordinate record Mh_e per element (bdb.cu):
//   P[m][r] = sum_i X[m][i] T_c[i][r]     r = 4 q + comp: value and the three
//                                         reference derivatives at point q of the
//                                         degree-2p rule (point-major columns)
//   V[m][4q + .] = w_q Mh_m P[m][4q + .]  (per element and point, registers)
//   Y[m][i] = sum_r V[m][r] T_c[i][r]
// Point-major columns make every chunk of KC = 40 columns (10 points) of V
// self-contained, so the second product runs in chunks through two
// shared-memory buffers: the transform of chunk j fills one while the product of
// chunk j-1 reads the other (two mbarriers, one product in flight on each).
template <int P>
struct TetBdbTcCfg {
  static constexpr int NLOC = (P + 1) * (P + 2) * (P + 3) / 6;
  static constexpr int NQ = P == 2 ? 14 : P == 3 ? 24 : 46;  // degree-2p rule points (tables.cu tet_rule)
  static constexpr int R = 4 * NQ;
  static constexpr int K1 = (NLOC + 7) / 8 * 8;    // forward K (local DOFs)
  static constexpr int N1 = (R + 15) / 16 * 16;    // forward N = backward K
  static constexpr int N2 = (NLOC + 15) / 16 * 16; // backward N
  static constexpr int KC = 40;                     // chunk of V columns (10 points; a multiple of 8)
  static constexpr int NCH = (N1 + KC - 1) / KC;
  static constexpr int LW = N1 - (NCH - 1) * KC;    // width of the last chunk (a multiple of 8)
  static constexpr int C2 = N1;                     // TMEM column of the backward accumulator
  static constexpr int TCOLS = (N1 + N2) <= 128 ? 128 : 256;
  static constexpr int ABUF = 2 * 128 * KC;         // floats of one operand buffer (hi, lo)
  static constexpr int T1 = 2 * ABUF;               // [hi, lo][N1][K1]
  static constexpr int T2 = T1 + 2 * N1 * K1;       // [hi, lo][N2][N1]
  static constexpr int W = T2 + 2 * N2 * N1;        // rule weights [NQ] (padded to 4)
  static constexpr int BAR = W + (NQ + 3) / 4 * 4;  // two mbarriers (16 B) + TMEM base (4 B)
  static constexpr size_t smem = (size_t)(BAR + 6) * sizeof(float);
  static constexpr int TAB = 2 * N1 * K1 + 2 * N2 * N1;  // floats of one class's operands
  static_assert(K1 <= KC && LW % 8 == 0 && (LW / 2) % 4 == 0, "chunk layout");
  static_assert(N1 + N2 <= 256, "tensor memory columns");
};

// W consecutive accumulator columns of this thread's row (W = 4, 8, 12, 16, 20)
template <int W>
__device__ __forceinline__ void tt_ldw(uint32_t taddr, float* v) {
  uint32_t r[20];
  if constexpr (W >= 16) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
  }
  constexpr int O8 = W >= 16 ? 16 : 0;
  if constexpr ((W - O8) >= 8) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[O8]), "=r"(r[O8 + 1]), "=r"(r[O8 + 2]), "=r"(r[O8 + 3]), "=r"(r[O8 + 4]), "=r"(r[O8 + 5]),
                   "=r"(r[O8 + 6]), "=r"(r[O8 + 7])
                 : "r"(taddr + O8));
  }
  constexpr int O4 = O8 + ((W - O8) >= 8 ? 8 : 0);
  if constexpr ((W - O4) >= 4) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[O4]), "=r"(r[O4 + 1]), "=r"(r[O4 + 2]), "=r"(r[O4 + 3])
                 : "r"(taddr + O4));
  }
  static_assert(W % 4 == 0 && W <= 20, "column count");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < W; i++) v[i] = __uint_as_float(r[i]);
}

template <int P>
__global__ void __launch_bounds__(TT_THREADS, 1)
tet_bdb_tc_kernel(int ntiles, const int* __restrict__ tiles, const int* __restrict__ tdofs, const float* __restrict__ Mt,
                  const float* __restrict__ tab, const double* __restrict__ W64, const float* __restrict__ x,
                  float* __restrict__ y, double* partial, unsigned int* counter, double* energy, const int* skip,
                  int* err) {
  using C = TetBdbTcCfg<P>;
  constexpr int NLOC = C::NLOC, NQ = C::NQ, K1 = C::K1, N1 = C::N1, N2 = C::N2, KC = C::KC, NCH = C::NCH;
  if (skip && *(volatile const int*)skip) return;
  extern __shared__ __align__(1024) float ts[];
  float* sA = ts;  // buffer 0: X (K = K1), then V chunks alternate between buffers 0 and 1
  float* sT1 = ts + C::T1;
  float* sT2 = ts + C::T2;
  float* sW = ts + C::W;
  uint64_t* bar = (uint64_t*)(ts + C::BAR);  // [0], [1]
  uint32_t* tslot = (uint32_t*)(ts + C::BAR + 4);
  const int t = threadIdx.x, warp = t >> 5, m = t & 127, half = t >> 7;
  for (int i = t; i < 2 * C::ABUF; i += TT_THREADS) ts[i] = 0.f;
  for (int i = t; i < NQ; i += TT_THREADS) sW[i] = (float)W64[i];
  if (t == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)), "r"(C::TCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  const uint32_t tl = tmem + ((uint32_t)((warp & 3) * 32) << 16);  // lanes of row m
  uint32_t ph[2] = {0u, 0u};
  int pend[2] = {0, 0};  // commits issued on each barrier and not yet waited for (0 or 1)
  bool ok = true;
  double acc = 0.0;
  int loaded = -1;
  auto issue_on = [&](int b, auto&& issue) {  // operands visible to the tensor core, issue, commit to bar[b]
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (t == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      issue();
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(&bar[b]))
                   : "memory");
    }
    pend[b] = 1;
  };
  auto wait_on = [&](int b) {
    const bool got = mbar_wait_bounded(&bar[b], ph[b]);
    if (got) {
      ph[b] ^= 1u;
      pend[b] = 0;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    return __syncthreads_and(got) != 0;
  };
  constexpr int H1 = K1 / 2;
  float xv[H1];
  auto dof_of = [&](int tl_, int i) { return __ldg(tdofs + ((size_t)tl_ * NLOC + i) * 128 + m); };
  auto gather = [&](int tl_) {
    const bool a = m < tiles[4 * tl_ + 2];
#pragma unroll
    for (int j = 0; j < H1; j++) {
      const int i = half * H1 + j;
      xv[j] = (a && i < NLOC) ? __ldg(x + dof_of(tl_, i)) : 0.f;
    }
  };
  const int t0 = (int)((long long)ntiles * blockIdx.x / gridDim.x);
  const int t1 = (int)((long long)ntiles * (blockIdx.x + 1) / gridDim.x);
  if (t0 < t1) gather(t0);
  for (int tile = t0; ok && tile < t1; tile++) {
    const int cls = tiles[4 * tile], cnt = tiles[4 * tile + 2];
    if (cls != loaded) {  // both B operands of the class (TF32 hi / lo, final layout)
      __syncthreads();
      const float4* src = (const float4*)(tab + (size_t)cls * C::TAB);
      float4* dst = (float4*)sT1;
      for (int k = t; k < C::TAB / 4; k += TT_THREADS) dst[k] = __ldg(src + k);
      loaded = cls;
    }
    const bool act = m < cnt;
#pragma unroll
    for (int j = 0; j < H1; j += 4) tt_put4<K1>(sA, m, half * H1 + j, xv + j);
    float mh[16];
#pragma unroll
    for (int c = 0; c < 16; c++) mh[c] = act ? __ldg(Mt + ((size_t)tile * 16 + c) * 128 + m) : 0.f;
    // ---- P = X T_c ------------------------------------------------------------------
    issue_on(1, [&] { tt_gemm<K1, K1, 0, N1, N1, false>(tmem, sA, sT1); });
    if (!(ok = wait_on(1))) break;
    // ---- V chunk by chunk, Y += V_j T_c[:, chunk j]^T -----------------------------------
    float en = 0.f;
    auto chunk = [&](auto jc) {
      constexpr int J = decltype(jc)::value;
      constexpr int KCJ = J < NCH - 1 ? KC : C::LW, K0 = J * KC, HW = KCJ / 2;
      float* buf = sA + (J & 1) * C::ABUF;
      if (J >= 2 && ok) ok = wait_on(J & 1);  // the product of chunk J-2 has read this buffer
      if (!ok) return;
      float pv[HW];
      tt_ldw<HW>(tl + K0 + half * HW, pv);
#pragma unroll
      for (int pt = 0; pt < HW / 4; pt++) {
        const int q = (K0 + half * HW) / 4 + pt;
        float o[4];
        const float w = q < NQ ? sW[q < NQ ? q : 0] : 0.f;
#pragma unroll
        for (int r = 0; r < 4; r++) {
          o[r] = w * (mh[4 * r] * pv[4 * pt] + mh[4 * r + 1] * pv[4 * pt + 1] + mh[4 * r + 2] * pv[4 * pt + 2] +
                      mh[4 * r + 3] * pv[4 * pt + 3]);
          if (partial) en += pv[4 * pt + r] * o[r];
        }
        tt_put4<KCJ>(buf, m, half * HW + 4 * pt, o);
      }
      issue_on(J & 1, [&] { tt_gemm<KCJ, N1, K0, N2, N2, (J > 0)>(tmem + C::C2, buf, sT2); });
    };
    static_assert(NCH <= 5, "chunk count");
    chunk(std::integral_constant<int, 0>());
    if constexpr (NCH > 1) chunk(std::integral_constant<int, 1>());
    if constexpr (NCH > 2) chunk(std::integral_constant<int, 2>());
    if constexpr (NCH > 3) chunk(std::integral_constant<int, 3>());
    if constexpr (NCH > 4) chunk(std::integral_constant<int, 4>());
    if (!ok) break;
    if (partial) acc += (double)en;
    if (tile + 1 < t1) gather(tile + 1);
    // the last two products (each barrier has at most one in flight)
    if (NCH >= 2 && pend[(NCH - 2) & 1]) {
      if (!(ok = wait_on((NCH - 2) & 1))) break;
    }
    if (!(ok = wait_on((NCH - 1) & 1))) break;
    float yv[N2];
#pragma unroll
    for (int c = 0; c < N2; c += 16) tt_ld16(tl + C::C2 + c, yv + c);
    if (act) {
      constexpr int HS = (NLOC + 1) / 2;
      if (half == 0) {
#pragma unroll
        for (int i = 0; i < HS; i++) red_add(y + dof_of(tile, i), yv[i]);
      } else {
#pragma unroll
        for (int i = HS; i < NLOC; i++) red_add(y + dof_of(tile, i), yv[i]);
      }
    }
  }
  if (!ok && t == 0) {
    atomicExch(err, 1);
    for (int b = 0; b < 2; b++)
      if (pend[b]) mbar_wait_bounded(&bar[b], ph[b]);  // the commits still in flight
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(C::TCOLS) : "memory");
  if (partial) block_reduce_finish(acc, partial, counter, energy);
}

// per class: T_c as the B operand of both products (TF32 hi / lo from FP64), from
// the degree-2p tables t64[class][q][i][4]: T1[r][i] and T2[i][r] with r = 4q + comp
template <int P>
__global__ void tet_bdb_tc_table_kernel(int ncls, const double* __restrict__ t64, float* __restrict__ tab) {
  using C = TetBdbTcCfg<P>;
  constexpr int NLOC = C::NLOC, NQ = C::NQ, R = C::R, K1 = C::K1, N1 = C::N1, N2 = C::N2;
  const int64_t per = (int64_t)N1 * K1 + (int64_t)N2 * N1, tot = (int64_t)ncls * per;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < tot; k += (int64_t)gridDim.x * blockDim.x) {
    const int cls = (int)(k / per);
    const int64_t j = k % per;
    float* T1 = tab + (size_t)cls * C::TAB;
    float* T2 = T1 + 2 * N1 * K1;
    int r, i;
    if (j < (int64_t)N1 * K1) { r = (int)(j / K1); i = (int)(j % K1); }
    else { i = (int)((j - (int64_t)N1 * K1) / N1); r = (int)((j - (int64_t)N1 * K1) % N1); }
    const int q = r / 4, comp = r % 4;
    const double v = (r < R && i < NLOC && q < NQ) ? t64[(((size_t)cls * NQ + q) * NLOC + i) * 4 + comp] : 0.0;
    const float h = tt_hi((float)v);
    if (j < (int64_t)N1 * K1) {
      T1[tt_off<K1>(r, i)] = h;
      T1[N1 * K1 + tt_off<K1>(r, i)] = (float)(v - (double)h);
    } else {
      T2[tt_off<N1>(i, r)] = h;
      T2[N2 * N1 + tt_off<N1>(i, r)] = (float)(v - (double)h);
    }
  }
}

// tile-major element records: Mt[(t * 16 + c) * 128 + m] (0 past the tile's count)
__global__ void tet_bdb_tc_rec_kernel(int ntiles, const int* __restrict__ tiles, const int* __restrict__ perm,
                                      const float* __restrict__ M, float* __restrict__ Mt) {
  const int64_t tot = (int64_t)ntiles * 16 * 128;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < tot; k += (int64_t)gridDim.x * blockDim.x) {
    const int m = (int)(k % 128), c = (int)((k / 128) % 16), t = (int)(k / (128 * 16));
    const int st = tiles[4 * t + 1], cnt = tiles[4 * t + 2];
    Mt[k] = m < cnt ? M[(size_t)perm[st + m] * 16 + c] : 0.f;
  }
}

template <int P>
static int tet_bdb_tc_prepare_p(gh1_op* op, const double* t64) {
  using C = TetBdbTcCfg<P>;
  gh1_space* sp = op->sp;
  GH1_CHECK(sp->tet_nq_mass == C::NQ, GH1_ERR_ARG, "internal: tet B^T D B rule size");
  auto kern = tet_bdb_tc_kernel<P>;
  int dev = 0, optin = 0;
  GH1_CUDA(cudaGetDevice(&dev));
  GH1_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  cudaFuncAttributes fa;
  GH1_CUDA(cudaFuncGetAttributes(&fa, kern));
  if ((size_t)optin < C::smem + fa.sharedSizeBytes) return 0;
  GH1_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::smem));
  // resident CTAs by shared memory and by registers (TMEM below)
  int smem_sm = 0, regs_sm = 0;
  GH1_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
  GH1_CUDA(cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev));
  const int v = std::min(smem_sm / (int)(C::smem + fa.sharedSizeBytes + 1024),
                         regs_sm / (TT_THREADS * ((fa.numRegs + 7) / 8 * 8)));
  if (v <= 0) return 0;
  op->d_tet_bdb_tab.alloc((size_t)N_TET_CLASSES * C::TAB);
  const int64_t tot = (int64_t)N_TET_CLASSES * ((int64_t)C::N1 * C::K1 + (int64_t)C::N2 * C::N1);
  tet_bdb_tc_table_kernel<P><<<(unsigned)std::min<int64_t>((tot + 255) / 256, 65535), 256, 0, sp->ctx->stream>>>(
      N_TET_CLASSES, t64, op->d_tet_bdb_tab.p);
  check_kernel(sp->ctx, "tet_bdb_tc_table_kernel");
  return std::min(v, 512 / C::TCOLS);
}

template <int P>
static void tet_bdb_tc_launch_p(gh1_op* op, const float* x, float* y, double* partial, unsigned int* counter,
                                double* energy, const int* skip) {
  gh1_space* sp = op->sp;
  const int grid = std::max(1, std::min(op->tet_tc_ntiles, sp->ctx->nsm * op->tet_bdb_tc_per_sm));
  tet_bdb_tc_kernel<P><<<grid, TT_THREADS, TetBdbTcCfg<P>::smem, sp->ctx->stream>>>(
      op->tet_tc_ntiles, op->d_tet_tc_tiles.p, op->d_tet_tc_dofs.p, op->d_tet_bdb_M.p, op->d_tet_bdb_tab.p,
      op->d_tetBw64.p, x, y, partial, counter, energy, skip, op->d_err.p);
  check_kernel(sp->ctx, "tet_bdb_tc_kernel");
}

void tet_bdb_tc_apply(gh1_op* op, const float* x, float* y, double* partial, unsigned int* counter, double* energy,
                      const int* skip) {
  GH1_CHECK(op->tet_bdb_tc_per_sm > 0, GH1_ERR_ARG, "internal: tensor-core tet B^T D B apply not prepared");
  switch (op->sp->p) {
    case 2: tet_bdb_tc_launch_p<2>(op, x, y, partial, counter, energy, skip); break;
    case 3: tet_bdb_tc_launch_p<3>(op, x, y, partial, counter, energy, skip); break;
    case 4: tet_bdb_tc_launch_p<4>(op, x, y, partial, counter, energy, skip); break;
    default: throw Error(GH1_ERR_UNSUPPORTED, "tensor-core tet B^T D B apply: order out of range");
  }
}

// FP32, records per element, p = 2..4: the tensor-core form, kept when the setup's
// timing finds it faster than the class-tiled kernel (GH1_TET_BDB_TC=0/1 forces)
static void tet_bdb_tc_prepare(gh1_op* op, const double* t64, const float* rec32, const char* env);

void tet_bdb_tc_setup(gh1_op* op, const double* t64) {
  gh1_space* sp = op->sp;
  op->tet_bdb_tc = false;
  op->tet_bdb_tc_per_sm = 0;
  const char* env = getenv("GH1_TET_BDB_TC");
  if (!(op->prec_mask & 2) || op->bdb != 2 || sp->p < 2 || sp->p > 4 || op->tet_ntiles == 0 ||
      (env && env[0] == '0'))
    return;
  tet_bdb_tc_prepare(op, t64, op->d_G32.p, env);
}

// FP32 stiffness + mass tet forms (p = 2..4, affine): the tensor-core B^T D B
// kernel on the records of D = diag(mu, kappa I or K) and the degree-2p rule,
// which integrates both terms exactly; GH1_TET_BDB_TC=0/1 forces as for the
// generic forms
void tet_mass_tc_setup(gh1_op* op) {
  gh1_space* sp = op->sp;
  op->tet_bdb_tc = false;
  op->tet_bdb_tc_per_sm = 0;
  const char* env = getenv("GH1_TET_BDB_TC");
  if (!(op->prec_mask & 2) || op->bdb || !op->has_mass || sp->p < 2 || sp->p > 4 || op->tet_ntiles == 0 ||
      op->tet_chunked || sp->mesh->def_space || (env && env[0] == '0'))
    return;
  cudaStream_t s = sp->ctx->stream;
  DBuf<double> t64;
  DBuf<float> t32;
  tet_mass_rule_tables(sp, t64, t32);
  DBuf<float> rec((size_t)std::max(sp->mesh->ne, 1) * 16);
  tet_standard_records(op, rec.p);
  // rule weights of the degree-2p rule
  std::vector<double> rule(4 * (size_t)sp->tet_nq_mass), w((size_t)sp->tet_nq_mass);
  GH1_CUDA(cudaMemcpyAsync(rule.data(), sp->d_tqm.p, rule.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  GH1_CUDA(cudaStreamSynchronize(s));
  for (int q = 0; q < sp->tet_nq_mass; q++) w[q] = rule[4 * q + 3];
  op->d_tetBw64.upload(w, s);
  tet_bdb_tc_prepare(op, t64.p, rec.p, env);
  GH1_CUDA(cudaStreamSynchronize(s));  // tables and records go out of scope
}

static void tet_bdb_tc_prepare(gh1_op* op, const double* t64, const float* rec32, const char* env) {
  gh1_space* sp = op->sp;
  cudaStream_t s = sp->ctx->stream;
  switch (sp->p) {
    case 2: op->tet_bdb_tc_per_sm = tet_bdb_tc_prepare_p<2>(op, t64); break;
    case 3: op->tet_bdb_tc_per_sm = tet_bdb_tc_prepare_p<3>(op, t64); break;
    default: op->tet_bdb_tc_per_sm = tet_bdb_tc_prepare_p<4>(op, t64); break;
  }
  if (op->tet_bdb_tc_per_sm <= 0) return;
  tet_tc_build_tiles(op);
  op->d_tet_bdb_M.alloc((size_t)op->tet_tc_ntiles * 16 * 128);
  const int64_t tm = (int64_t)op->tet_tc_ntiles * 16 * 128;
  tet_bdb_tc_rec_kernel<<<(unsigned)std::min<int64_t>((tm + 255) / 256, 65535), 256, 0, s>>>(
      op->tet_tc_ntiles, op->d_tet_tc_tiles.p, op->d_tet_perm.p, rec32, op->d_tet_bdb_M.p);
  check_kernel(sp->ctx, "tet_bdb_tc_rec_kernel");
  GH1_CUDA(cudaStreamSynchronize(s));
  if (env && env[0] == '1') {
    op->tet_bdb_tc = true;
    return;
  }
  if (sp->mesh->ne < 4096) return;
  DBuf<float> xs(op->nrows), ys(op->nrows);
  xs.zero(s);
  cudaEvent_t a, b;
  GH1_CUDA(cudaEventCreate(&a));
  GH1_CUDA(cudaEventCreate(&b));
  float ms[2];
  for (int v = 0; v < 2; v++) {
    op->tet_bdb_tc = v == 1;
    for (int r = 0; r < 5; r++) {
      if (r == 2) GH1_CUDA(cudaEventRecord(a, s));
      if (op->bdb) tet_bdb_apply(op, GH1_F32, xs.p, ys.p, nullptr, nullptr, nullptr, nullptr);
      else tet_tiles_apply(op, GH1_F32, xs.p, ys.p, nullptr, nullptr, nullptr, nullptr);
    }
    GH1_CUDA(cudaEventRecord(b, s));
    GH1_CUDA(cudaEventSynchronize(b));
    GH1_CUDA(cudaEventElapsedTime(&ms[v], a, b));
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  op->tet_bdb_tc = ms[1] < ms[0];
}

}  // namespace gh1
