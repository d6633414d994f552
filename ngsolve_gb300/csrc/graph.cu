// graph.cu -- the CSR pattern of BilinearForm::Assemble built on the GPU.
//
// Same result as build_graph (assemble.cu, the MatrixGraph of
// linalg/sparsematrix.cpp:450-900): row r holds the sorted union of the DOFs of
// all elements containing DOF r (diagonal included, full storage).
//   1. DOF -> element incidence: counts, exclusive scan, fill;
//   2. per row, one warp gathers the DOF lists of the row's elements into shared
//      memory (deg(r) * nloc candidates), sorts them (bitonic, padded to the next
//      power of two) and counts / writes the distinct values;
//   3. row pointers = exclusive scan of the counts; a second pass writes colind.
// Rows with more than GRAPH_CAP candidates (very high orders) make the caller
// fall back to the host build.
#include <algorithm>
#include <climits>
#include <vector>
#include "common.cuh"

namespace gh1 {

constexpr int GRAPH_CAP = 4096;     // candidates per row handled in shared memory
constexpr int GRAPH_WARPS = 4;      // rows in flight per block
constexpr int SCAN_CHUNK = 1024;    // elements per block of the scan

__global__ void graph_count_kernel(int64_t n, const int* __restrict__ eldofs, int* deg) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(deg + eldofs[k], 1);
}

__global__ void graph_fill_kernel(int64_t n, int nloc, const int* __restrict__ eldofs, const int64_t* __restrict__ start,
                                  int* cursor, int* dof2el) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const int d = eldofs[k];
    const int pos = atomicAdd(cursor + d, 1);
    dof2el[start[d] + pos] = (int)(k / nloc);
  }
}

// exclusive scan, pass 1: per chunk local exclusive sums and the chunk total
template <class TI>
__global__ void scan_local_kernel(int64_t n, const TI* __restrict__ in, int64_t* out, int64_t* sums) {
  __shared__ int64_t s[SCAN_CHUNK];
  const int64_t base = (int64_t)blockIdx.x * SCAN_CHUNK;
  for (int i = threadIdx.x; i < SCAN_CHUNK; i += blockDim.x) s[i] = base + i < n ? (int64_t)in[base + i] : 0;
  __syncthreads();
  if (threadIdx.x == 0) {  // 1024 adds per chunk: negligible at setup
    int64_t run = 0;
    for (int i = 0; i < SCAN_CHUNK; i++) {
      const int64_t v = s[i];
      s[i] = run;
      run += v;
    }
    sums[blockIdx.x] = run;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < SCAN_CHUNK; i += blockDim.x)
    if (base + i < n) out[base + i] = s[i];
}

__global__ void scan_add_kernel(int64_t n, const int64_t* __restrict__ offs, int64_t* out) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    out[k] += offs[k / SCAN_CHUNK];
}

// out[0..n] = exclusive scan of in[0..n) (out[n] = total); returns the total
template <class TI>
static int64_t exclusive_scan(gh1_ctx* ctx, int64_t n, const TI* in, int64_t* out) {
  cudaStream_t s = ctx->stream;
  const int64_t nb = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
  DBuf<int64_t> sums(std::max<int64_t>(nb, 1));
  if (nb > 0) {
    scan_local_kernel<TI><<<(unsigned)nb, 256, 0, s>>>(n, in, out, sums.p);
    check_kernel(ctx, "scan_local_kernel");
  }
  std::vector<int64_t> h(nb);
  if (nb) GH1_CUDA(cudaMemcpyAsync(h.data(), sums.p, nb * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  GH1_CUDA(cudaStreamSynchronize(s));
  int64_t run = 0;
  for (int64_t b = 0; b < nb; b++) {
    const int64_t v = h[b];
    h[b] = run;
    run += v;
  }
  if (nb) {
    sums.upload(h.data(), nb, s);
    scan_add_kernel<<<(unsigned)std::min<int64_t>((n + 255) / 256, (int64_t)ctx->nsm * 16), 256, 0, s>>>(n, sums.p, out);
    check_kernel(ctx, "scan_add_kernel");
  }
  GH1_CUDA(cudaMemcpyAsync(out + n, &run, sizeof(int64_t), cudaMemcpyHostToDevice, s));
  GH1_CUDA(cudaStreamSynchronize(s));  // `run` and the staging vector go out of scope
  return run;
}

__global__ void graph_max_kernel(int64_t n, const int* __restrict__ v, int* mx) {
  int m = 0;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    m = max(m, v[k]);
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(mx, m);
}

// One warp per row: candidates -> bitonic sort in shared memory (padded with
// INT_MAX to the next power of two) -> distinct values counted (FILL = false) or
// written to colind[rowptr[r]...] in ascending order (FILL = true).
template <bool FILL>
__global__ void __launch_bounds__(32 * GRAPH_WARPS)
graph_rows_kernel(int64_t ndof, int nloc, int pmax, const int64_t* __restrict__ start, const int* __restrict__ dof2el,
                  const int* __restrict__ eldofs, int* rowlen, const int64_t* __restrict__ rowptr, int* colind) {
  extern __shared__ int gbuf_rows[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int* b = gbuf_rows + (size_t)w * pmax;
  const int64_t nw = (int64_t)gridDim.x * GRAPH_WARPS;
  for (int64_t r = (int64_t)blockIdx.x * GRAPH_WARPS + w; r < ndof; r += nw) {
    const int64_t s0 = start[r];
    const int m = (int)(start[r + 1] - s0) * nloc;  // <= pmax (checked by the caller)
    int P = 1;
    while (P < m) P <<= 1;
    for (int i = lane; i < P; i += 32) b[i] = i < m ? eldofs[(size_t)dof2el[s0 + i / nloc] * nloc + i % nloc] : INT_MAX;
    __syncwarp();
    for (int k = 2; k <= P; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int i = lane; i < P; i += 32) {  // the pairs (i, i^j) partition [0, P)
          const int ixj = i ^ j;
          if (ixj > i) {
            const int x = b[i], y = b[ixj];
            if ((x > y) == ((i & k) == 0)) {
              b[i] = y;
              b[ixj] = x;
            }
          }
        }
        __syncwarp();
      }
    int count = 0;
    const int64_t out0 = FILL ? rowptr[r] : 0;
    for (int i0 = 0; i0 < m; i0 += 32) {
      const int i = i0 + lane;
      const bool head = i < m && (i == 0 || b[i] != b[i - 1]);
      const unsigned bal = __ballot_sync(0xffffffffu, head);
      if (FILL && head) colind[out0 + count + __popc(bal & ((1u << lane) - 1u))] = b[i];
      count += __popc(bal);
    }
    if (!FILL && lane == 0) rowlen[r] = count;
    __syncwarp();
  }
}

// Builds sp->d_rowptr / d_colind / nnz on the GPU; false (nothing changed) when a
// row has more candidates than GRAPH_CAP.
bool build_graph_gpu(gh1_space* sp) {
  gh1_ctx* ctx = sp->ctx;
  cudaStream_t s = ctx->stream;
  const int64_t ndof = sp->ndof, n = (int64_t)sp->mesh->ne * sp->nloc;
  const int nloc = sp->nloc;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->nsm * 16));
  DBuf<int> deg(ndof), mx(1);
  deg.zero(s);
  mx.zero(s);
  graph_count_kernel<<<grid, 256, 0, s>>>(n, sp->d_eldofs.p, deg.p);
  check_kernel(ctx, "graph_count_kernel");
  graph_max_kernel<<<grid, 256, 0, s>>>(ndof, deg.p, mx.p);
  check_kernel(ctx, "graph_max_kernel");
  int hmx = 0;
  GH1_CUDA(cudaMemcpyAsync(&hmx, mx.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  GH1_CUDA(cudaStreamSynchronize(s));
  if ((int64_t)hmx * nloc > GRAPH_CAP) return false;
  int pmax = 1;
  while (pmax < hmx * nloc) pmax <<= 1;
  DBuf<int64_t> start(ndof + 1);
  exclusive_scan(ctx, ndof, deg.p, start.p);
  DBuf<int> cursor(ndof), dof2el(n);
  cursor.zero(s);
  graph_fill_kernel<<<grid, 256, 0, s>>>(n, nloc, sp->d_eldofs.p, start.p, cursor.p, dof2el.p);
  check_kernel(ctx, "graph_fill_kernel");
  const size_t smem = (size_t)GRAPH_WARPS * pmax * sizeof(int);
  static bool attr = false;
  if (!attr) {
    GH1_CUDA(cudaFuncSetAttribute(graph_rows_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  GRAPH_WARPS * GRAPH_CAP * (int)sizeof(int)));
    GH1_CUDA(cudaFuncSetAttribute(graph_rows_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  GRAPH_WARPS * GRAPH_CAP * (int)sizeof(int)));
    attr = true;
  }
  const int rgrid = (int)std::max<int64_t>(1, std::min<int64_t>((ndof + GRAPH_WARPS - 1) / GRAPH_WARPS, (int64_t)ctx->nsm * 32));
  DBuf<int> rowlen(ndof);
  graph_rows_kernel<false><<<rgrid, 32 * GRAPH_WARPS, smem, s>>>(ndof, nloc, pmax, start.p, dof2el.p, sp->d_eldofs.p,
                                                                  rowlen.p, nullptr, nullptr);
  check_kernel(ctx, "graph_rows_kernel");
  sp->d_rowptr.alloc(ndof + 1);
  const int64_t nnz = exclusive_scan(ctx, ndof, rowlen.p, sp->d_rowptr.p);
  sp->d_colind.alloc(nnz);
  graph_rows_kernel<true><<<rgrid, 32 * GRAPH_WARPS, smem, s>>>(ndof, nloc, pmax, start.p, dof2el.p, sp->d_eldofs.p,
                                                                 nullptr, sp->d_rowptr.p, sp->d_colind.p);
  check_kernel(ctx, "graph_rows_kernel");
  GH1_CUDA(cudaStreamSynchronize(s));  // the temporaries are freed at scope exit
  sp->nnz = nnz;
  sp->have_graph = true;
  return true;
}

}  // namespace gh1
