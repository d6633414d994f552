// reduce.cuh -- grid-wide reductions without inter-block waiting (threadfence
// pattern: every block writes a partial sum, the last block to finish totals).
#pragma once
#include <cuda_runtime.h>

namespace gh1 {

// grid-wide reduction of K doubles per thread; returns true in the last block,
// where tot[] holds the totals (all threads).  No block waits for another.
template <int K>
__device__ bool grid_reduce(double (&v)[K], double* partial, unsigned int* counter, double (&tot)[K]) {
  __shared__ double red[K][32];
  __shared__ bool last;
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < K; k++) {
    double x = v[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (l == 0) red[k][w] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < K; k++) {
      double s = 0;
      for (int i = 0; i < nw; i++) s += red[k][i];
      partial[(size_t)k * gridDim.x + blockIdx.x] = s;
    }
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
#pragma unroll
  for (int k = 0; k < K; k++) {
    double s = 0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) s += ((volatile double*)partial)[(size_t)k * gridDim.x + i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __syncthreads();
    if (l == 0) red[k][w] = s;
    __syncthreads();
    double t = 0;
    for (int i = 0; i < nw; i++) t += red[k][i];
    tot[k] = t;
  }
  if (threadIdx.x == 0) *counter = 0u;
  return true;
}

}  // namespace gh1
