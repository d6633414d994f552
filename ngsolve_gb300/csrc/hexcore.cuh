// hexcore.cuh -- pieces shared by the hex sum-factorization kernels: the layout
// of the 1D factor tables in constant memory, the thread-group configuration,
// group barriers and votes, the end-of-kernel energy reduction, and the bulk-copy
// (TMA) / mbarrier helpers of the pipelined element loops.
#pragma once
#include <algorithm>
#include <cmath>
#include "common.cuh"

namespace gh1 {

// offset of the N x N factor table of order p = N-1 inside the concatenated
// tables of every order
constexpr int tab_off(int N) { return N <= 2 ? 0 : tab_off(N - 1) + (N - 1) * (N - 1); }
constexpr int TAB_TOTAL = tab_off(MAX_HEX_ORDER + 2);
// offset of the N per-point entries of order p = N-1 in the tables of every order
// that hold one value per 1D point (rule weights, even-odd coefficients)
constexpr int eo_off(int N) { return N * (N - 1) / 2 - 1; }

// Even-odd coefficients of the vertex pair of the N x N tables B = psi_a(x_q),
// D = psi_a'(x_q): eo[0..3][q] = (B[q][0] + B[q][1]) / 2, (B[q][0] - B[q][1]) / 2,
// (D[q][0] + D[q][1]) / 2, (D[q][0] - D[q][1]) / 2.  Returns the largest
// deviation from the reflection symmetry the even-odd contractions rely on
// (psi_0 <-> psi_1 and psi_c -> (-1)^c psi_c under x -> 1-x), relative to the
// tables' scale.
inline double hex_eo_coefficients(const double* B, const double* D, int N, double eo[4][16]) {
  double scale = 0, dev = 0;
  for (int q = 0; q < N; q++)
    for (int c = 0; c < N; c++) {
      const int qr = N - 1 - q, cr = c < 2 ? 1 - c : c;
      const double sg = c < 2 ? 1.0 : ((c % 2) ? -1.0 : 1.0);
      scale = std::max(scale, std::max(std::fabs(B[q * N + c]), std::fabs(D[q * N + c])));
      dev = std::max(dev, std::fabs(B[qr * N + c] - sg * B[q * N + cr]));
      dev = std::max(dev, std::fabs(D[qr * N + c] + sg * D[q * N + cr]));
    }
  for (int k = 0; k < 4; k++)
    for (int q = 0; q < 16; q++) eo[k][q] = 0.0;
  for (int q = 0; q < N; q++) {
    eo[0][q] = 0.5 * (B[q * N] + B[q * N + 1]);
    eo[1][q] = 0.5 * (B[q * N] - B[q * N + 1]);
    eo[2][q] = 0.5 * (D[q * N] + D[q * N + 1]);
    eo[3][q] = 0.5 * (D[q * N] - D[q * N + 1]);
  }
  return scale > 0 ? dev / scale : dev;
}

// ---------------------------------------------------------------------------
// element geometry (FP64)
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

// ---------------------------------------------------------------------------
// thread-group helpers
template <int G>
__device__ __forceinline__ void group_sync(int gid) {
  if (G == 32) __syncwarp();
  else asm volatile("bar.sync %0, %1;" ::"r"(gid + 1), "r"(G) : "memory");
}

template <class T>
__device__ __forceinline__ void atomic_add_t(T* p, T v) { red_add(p, v); }

// End-of-kernel reduction of one double per thread into partial[blockIdx.x];
// the last block to finish sums all partials into *out and resets the counter.
// (threadfence reduction: no block waits on another.)
static __device__ void block_reduce_finish(double v, double* partial, unsigned int* counter, double* out) {
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

// Element groups: EPW element slots of N^2 pencils each on G threads.  Low
// orders share a warp; at N = 6 two slots share 96 threads (75 % of the lanes
// busy, against 56 % for one 36-pencil element on 64 threads).
template <int N>
struct HexCfg {
  static constexpr int N2 = N * N, N3 = N * N * N;
  static constexpr int EPW = N2 <= 32 ? 32 / N2 : (N == 6 ? 2 : 1);  // elements per group
  static constexpr int G = ((EPW * N2 + 31) / 32) * 32;              // threads per element group
  static constexpr int EPB = G == 32 ? 4 : 2;                        // element groups per block
  static constexpr int BLOCK = G * EPB;
};

__host__ __device__ constexpr size_t round16(size_t b) { return (b + 15) / 16 * 16; }

// ---- bulk-copy (TMA) and mbarrier helpers ------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
// global -> shared bulk copy (size and both addresses multiples of 16 bytes)
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
// bulk prefetch of a contiguous global range into L2 (16-byte aligned, size a
// multiple of 16): the later loads of the range hit L2 instead of HBM
__device__ __forceinline__ void bulk_prefetch_l2(const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
               : "=r"(ok)
               : "r"(smem_u32(bar)), "r"(parity)
               : "memory");
  return ok != 0;
}
// bounded wait: false after ~2^22 polls (an error, never expected)
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  for (int i = 0; i < (1 << 22); i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
// the same with a given poll limit (0: report a timeout without polling)
__device__ __forceinline__ bool mbar_wait_polls(uint64_t* bar, uint32_t parity, int polls) {
  for (int i = 0; i < polls; i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
// all threads of the element group agree on a predicate
template <int G>
__device__ __forceinline__ bool group_all(int gid, bool v) {
  if (G == 32) return __all_sync(0xffffffffu, v);
  uint32_t r;
  asm volatile("{\n .reg .pred p, q;\n setp.ne.u32 q, %1, 0;\n bar.red.and.pred p, %2, %3, q;\n selp.u32 %0, 1, 0, p;\n}"
               : "=r"(r)
               : "r"((uint32_t)v), "r"(gid + 1), "r"(G)
               : "memory");
  return r != 0;
}

}  // namespace gh1
