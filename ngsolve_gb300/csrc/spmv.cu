// spmv.cu -- CSR SpMV y = A x (SparseMatrix::MultAdd, linalg/sparsematrix_impl.hpp:
// 264-290 with RowTimesVector, linalg/sparsematrix.hpp:625-672).  The reference
// GPU path calls cusparseSpMV (ngscuda/cuda_linalg.cpp:244-275); this kernel
// replaces it.  HBM-bound: per nonzero 8 B (FP64 value) + 4 B (column) streamed
// once; x is gathered through L2/L1.
//
// Mapping: a sub-warp of L lanes per row (L = 32 for rows of ~100 entries, 16/8
// for shorter rows), lanes stride the row in order, then a shuffle reduction.
#include <algorithm>
#include "common.cuh"

namespace gh1 {

template <class TV, class TX, int L>
__global__ void __launch_bounds__(256) csr_spmv_kernel(int64_t nrows, const int64_t* __restrict__ rowptr,
                                                       const int32_t* __restrict__ colind, const TV* __restrict__ vals,
                                                       const TX* __restrict__ x, TX* __restrict__ y) {
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
      for (int64_t k = beg + sub; k < end; k += L) acc += (TX)__ldcs(vals + k) * __ldg(x + __ldcs(colind + k));
    }
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, L);
    if (sub == 0 && row < nrows) y[row] = acc;
  }
}

template <class TV, class TX>
void launch_spmv(gh1_ctx* ctx, int64_t nrows, int64_t nnz, const int64_t* rowptr, const int32_t* colind, const TV* vals,
                 const TX* x, TX* y) {
  double avg = nrows ? (double)nnz / nrows : 0;
  const int block = 256;
  auto grid_of = [&](int L) {
    int64_t rows_per_block = block / L;
    int64_t need = (nrows + rows_per_block - 1) / rows_per_block;
    return (int)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)ctx->nsm * 16));
  };
  if (avg >= 48)
    csr_spmv_kernel<TV, TX, 32><<<grid_of(32), block, 0, ctx->stream>>>(nrows, rowptr, colind, vals, x, y);
  else if (avg >= 12)
    csr_spmv_kernel<TV, TX, 16><<<grid_of(16), block, 0, ctx->stream>>>(nrows, rowptr, colind, vals, x, y);
  else
    csr_spmv_kernel<TV, TX, 4><<<grid_of(4), block, 0, ctx->stream>>>(nrows, rowptr, colind, vals, x, y);
  check_kernel(ctx, "csr_spmv_kernel");
}

__global__ void f64_to_f32_kernel(int64_t n, const double* a, float* b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) b[i] = (float)a[i];
}

void spmv(gh1_op* op, const void* x, void* y, int prec) {
  if (prec == GH1_F64) {
    launch_spmv<double, double>(op->ctx, op->nrows, op->nnz, op->rowptr, op->colind, op->d_vals.p, (const double*)x,
                                (double*)y);
  } else {
    if (op->d_vals32.n != (size_t)op->nnz) {
      op->d_vals32.alloc(op->nnz);
      f64_to_f32_kernel<<<op->ctx->nsm * 8, 256, 0, op->ctx->stream>>>(op->nnz, op->d_vals.p, op->d_vals32.p);
      check_kernel(op->ctx, "f64_to_f32_kernel");
    }
    launch_spmv<float, float>(op->ctx, op->nrows, op->nnz, op->rowptr, op->colind, op->d_vals32.p, (const float*)x,
                              (float*)y);
  }
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
