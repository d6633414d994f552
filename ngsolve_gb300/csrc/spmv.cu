// spmv.cu -- CSR SpMV y = A x (SparseMatrix::MultAdd, linalg/sparsematrix_impl.hpp:
// 264-290 with RowTimesVector, linalg/sparsematrix.hpp:625-672).  The reference
// GPU path calls cusparseSpMV (ngscuda/cuda_linalg.cpp:244-275); this kernel
// replaces it.  HBM-bound: per nonzero 8 B (FP64 value) + 4 B (column) streamed
// once; x is gathered through L2/L1.
//
// Mapping: a sub-warp of L lanes per row; each lane walks the row in strides of
// L with a U-way unrolled body (U = 4 or 8) so that 2U streaming loads and U
// gathers are in flight per lane; shuffle reduction.  L and U are autotuned per
// matrix (L = 4..32).
#include <algorithm>
#include <cstdlib>
#include <iterator>
#include "common.cuh"

namespace gh1 {

template <class TV, class TX, int L, int U>
__global__ void __launch_bounds__(256) csr_spmv_kernel(int64_t nrows, const int64_t* __restrict__ rowptr,
                                                       const int32_t* __restrict__ colind, const TV* __restrict__ vals,
                                                       const TX* __restrict__ x, TX* __restrict__ y, const int* skip) {
  if (skip && *(volatile const int*)skip) return;
  // all lanes of a warp iterate together (the shuffle needs the full warp)
  constexpr int RPW = 32 / L;  // rows per warp
  const int sub = threadIdx.x % L;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) / 32;
  const int slot = (threadIdx.x % 32) / L;
  for (int64_t r0 = warp * RPW; r0 < nrows; r0 += nwarps * RPW) {
    const int64_t row = r0 + slot;
    TX acc = 0;
    if (row < nrows) {
      const int64_t beg = __ldg(rowptr + row), end = __ldg(rowptr + row + 1);
      int64_t k = beg + sub;
      if (U == 8) {
        for (; k + 7 * L < end; k += 8 * L) {
          int c[8];
          TV v[8];
#pragma unroll
          for (int j = 0; j < 8; j++) {
            c[j] = __ldcs(colind + k + j * L);
            v[j] = __ldcs(vals + k + j * L);
          }
          TX t = 0;
#pragma unroll
          for (int j = 0; j < 8; j++) t += (TX)v[j] * __ldg(x + c[j]);
          acc += t;
        }
      }
      for (; k + 3 * L < end; k += 4 * L) {
        const int c0 = __ldcs(colind + k), c1 = __ldcs(colind + k + L), c2 = __ldcs(colind + k + 2 * L),
                  c3 = __ldcs(colind + k + 3 * L);
        const TV v0 = __ldcs(vals + k), v1 = __ldcs(vals + k + L), v2 = __ldcs(vals + k + 2 * L),
                 v3 = __ldcs(vals + k + 3 * L);
        acc += (TX)v0 * __ldg(x + c0) + (TX)v1 * __ldg(x + c1) + (TX)v2 * __ldg(x + c2) + (TX)v3 * __ldg(x + c3);
      }
      for (; k < end; k += L) acc += (TX)__ldcs(vals + k) * __ldg(x + __ldcs(colind + k));
    }
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, L);
    if (sub == 0 && row < nrows) y[row] = acc;
  }
}

template <class TV, class TX, int L, int U>
void launch_spmv_L(gh1_ctx* ctx, cudaStream_t s, int64_t nrows, const int64_t* rowptr, const int32_t* colind,
                   const TV* vals, const TX* x, TX* y, const int* skip) {
  const int block = 256;
  const int64_t rows_per_block = block / L;
  const int64_t need = (nrows + rows_per_block - 1) / rows_per_block;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)ctx->nsm * 16));
  csr_spmv_kernel<TV, TX, L, U><<<grid, block, 0, s>>>(nrows, rowptr, colind, vals, x, y, skip);
  check_kernel(ctx, "csr_spmv_kernel");
}

template <class TV, class TX>
void launch_spmv(gh1_ctx* ctx, cudaStream_t s, int L, int64_t nrows, const int64_t* rowptr, const int32_t* colind,
                 const TV* vals, const TX* x, TX* y, const int* skip) {
  // L encodes the unroll too: L + 100 selects U = 8
  switch (L) {
    case 4: launch_spmv_L<TV, TX, 4, 4>(ctx, s, nrows, rowptr, colind, vals, x, y, skip); break;
    case 8: launch_spmv_L<TV, TX, 8, 4>(ctx, s, nrows, rowptr, colind, vals, x, y, skip); break;
    case 16: launch_spmv_L<TV, TX, 16, 4>(ctx, s, nrows, rowptr, colind, vals, x, y, skip); break;
    case 104: launch_spmv_L<TV, TX, 4, 8>(ctx, s, nrows, rowptr, colind, vals, x, y, skip); break;
    case 108: launch_spmv_L<TV, TX, 8, 8>(ctx, s, nrows, rowptr, colind, vals, x, y, skip); break;
    case 116: launch_spmv_L<TV, TX, 16, 8>(ctx, s, nrows, rowptr, colind, vals, x, y, skip); break;
    case 132: launch_spmv_L<TV, TX, 32, 8>(ctx, s, nrows, rowptr, colind, vals, x, y, skip); break;
    default: launch_spmv_L<TV, TX, 32, 4>(ctx, s, nrows, rowptr, colind, vals, x, y, skip); break;
  }
}

__global__ void f64_to_f32_kernel(int64_t n, const double* a, float* b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) b[i] = (float)a[i];
}

// picks the sub-warp width by timing the candidates once on this matrix
// (never inside a stream capture: callers prepare before capturing)
static int spmv_tune(gh1_op* op, int prec) {
  int& L = op->spmv_L[prec == GH1_F64 ? 0 : 1];
  if (L > 0) return L;
  gh1_ctx* ctx = op->ctx;
  cudaStream_t s = ctx->stream;
  const int64_t n = op->nrows;
  const size_t es = prec == GH1_F64 ? 8 : 4;
  DBuf<char> xs(n * es), ys(n * es);
  xs.zero(s);
  cudaEvent_t a, b;
  GH1_CUDA(cudaEventCreate(&a));
  GH1_CUDA(cudaEventCreate(&b));
  float best = 1e30f;
  int bestL = 32;
  // GH1_SPMV_L forces one of the candidates (tests run every form this way)
  const char* env = getenv("GH1_SPMV_L");
  const int cands[] = {4, 8, 16, 32, 104, 108, 116, 132};
  if (env && std::find(std::begin(cands), std::end(cands), atoi(env)) != std::end(cands)) {
    L = atoi(env);
    return L;
  }
  for (int cand : cands) {
    for (int rep = 0; rep < 2; rep++) {  // 3 warm-up launches, then 5 timed
      if (rep == 1) GH1_CUDA(cudaEventRecord(a, s));
      for (int k = 0; k < 3 + 2 * rep; k++) {
        if (prec == GH1_F64)
          launch_spmv<double, double>(ctx, s, cand, n, op->rowptr, op->colind, op->d_vals.p, (const double*)xs.p,
                                      (double*)ys.p, nullptr);
        else
          launch_spmv<float, float>(ctx, s, cand, n, op->rowptr, op->colind, op->d_vals32.p, (const float*)xs.p,
                                    (float*)ys.p, nullptr);
      }
    }
    GH1_CUDA(cudaEventRecord(b, s));
    GH1_CUDA(cudaEventSynchronize(b));
    float ms = 0;
    GH1_CUDA(cudaEventElapsedTime(&ms, a, b));
    if (ms < best) { best = ms; bestL = cand; }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  L = bestL;
  return L;
}

void spmv_prepare(gh1_op* op, int prec) {
  if (prec != GH1_F64 && op->d_vals32.n != (size_t)op->nnz) {
    op->d_vals32.alloc(op->nnz);
    f64_to_f32_kernel<<<op->ctx->nsm * 8, 256, 0, op->ctx->stream>>>(op->nnz, op->d_vals.p, op->d_vals32.p);
    check_kernel(op->ctx, "f64_to_f32_kernel");
  }
  spmv_tune(op, prec);
}

void spmv_skip(gh1_op* op, const void* x, void* y, int prec, const int* skip) {
  gh1_ctx* ctx = op->ctx;
  const int L = op->spmv_L[prec == GH1_F64 ? 0 : 1];
  GH1_CHECK(L > 0, GH1_ERR_ARG, "internal: SpMV not prepared");
  if (prec == GH1_F64)
    launch_spmv<double, double>(ctx, ctx->stream, L, op->nrows, op->rowptr, op->colind, op->d_vals.p, (const double*)x,
                                (double*)y, skip);
  else
    launch_spmv<float, float>(ctx, ctx->stream, L, op->nrows, op->rowptr, op->colind, op->d_vals32.p, (const float*)x,
                              (float*)y, skip);
}

void spmv(gh1_op* op, const void* x, void* y, int prec) {
  spmv_prepare(op, prec);
  spmv_skip(op, x, y, prec, nullptr);
}

__global__ void csr_diag_kernel(int64_t nrows, const int64_t* rowptr, const int32_t* colind, const double* vals, double* diag) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
    int64_t lo = rowptr[r], hi = rowptr[r + 1] - 1;
    double d = 0;
    while (lo <= hi) {
      int64_t mid = (lo + hi) >> 1;
      int c = colind[mid];
      if (c == r) { d = vals[mid]; break; }
      if (c < r) lo = mid + 1; else hi = mid - 1;
    }
    diag[r] = d;
  }
}

void csr_diag(gh1_op* op, double* diag) {
  csr_diag_kernel<<<op->ctx->nsm * 8, 256, 0, op->ctx->stream>>>(op->nrows, op->rowptr, op->colind, op->d_vals.p, diag);
  check_kernel(op->ctx, "csr_diag_kernel");
}

}  // namespace gh1
