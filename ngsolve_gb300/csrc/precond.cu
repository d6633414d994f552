// precond.cu -- smoothing blocks, block-Jacobi smoother and exact low-order solve.
//
// Replaces the reference's additive Schwarz preconditioner of its CUDA tutorial
// (docs/i-tutorials/unit-5.5-cuda/poisson_cuda.ipynb, cells 9-13):
//   C^{-1} = P A_cc^{-1} P^T + sum_i E_i A_i^{-1} E_i^T
// with
//  - the blocks of H1HighOrderFESpace::CreateSmoothingBlocks
//    (comp/h1hofespace.cpp:1477-1600; built on the host in api.cu),
//  - BlockJacobiPrecond (linalg/blockjacobi.cpp): inverses of the dense diagonal
//    blocks A_i = A[block i, block i] of the assembled matrix; the device apply
//    of DevBlockJacobiMatrix (ngscuda/dev_blockjacobi.cpp:49-137), one warp per
//    block here, the block's inverse read column by column (coalesced),
//  - the low-order solve loemb @ loinv @ loemb.T: the low-order matrix on the
//    free coarse DOFs, inverted exactly (the reference factorizes it with its
//    sparse Cholesky, DevSparseCholesky in ngscuda/dev_sparsecholesky.cpp; here a
//    dense Gauss-Jordan inverse on the GPU, for coarse spaces up to 8192 free
//    DOFs) and applied as one dense matrix-vector product,
//  - the sum of the two (SumMatrix).
// Every apply is kernels only (no host synchronization), so the device-side CG
// loop captures it into its graph.
#include <algorithm>
#include <vector>
#include "common.cuh"
#include "basis.cuh"

namespace gh1 {

// H1HighOrderFESpace::CreateSmoothingBlocks (comp/h1hofespace.cpp:1477-1600),
// filtered by the free DOFs (FilteredTableCreator): blocktype 4 = VE + F + I
// (each vertex with the DOFs of the edges at it, each face, each element's
// interior), 3 = V + E + F + I.  Empty blocks are dropped.
void smoothing_blocks(gh1_space* sp, int blocktype, std::vector<int64_t>& off, std::vector<int32_t>& dofs) {
  GH1_CHECK(blocktype == 3 || blocktype == 4, GH1_ERR_UNSUPPORTED, "blocktype 3 (V+E+F+I) or 4 (VE+F+I)");
  gh1_mesh* m = sp->mesh;
  const int ne = m->ne, nv = m->nv, nloc = sp->nloc, nvert = sp->nvert, ned = sp->n_edge_dofs;
  const bool tet = sp->et == 4;
  const std::vector<uint8_t>& fr = sp->freedof;
  off.assign(1, 0);
  dofs.clear();
  auto add_block = [&](const std::vector<int32_t>& b) {
    size_t before = dofs.size();
    for (int32_t d : b)
      if (fr[d]) dofs.push_back(d);
    if (dofs.size() > before) off.push_back((int64_t)dofs.size());
  };
  std::vector<int32_t> tmp;
  if (blocktype == 4) {
    std::vector<std::vector<int32_t>> vb(nv);
    for (int v = 0; v < nv; v++) vb[v].push_back(v);
    if (ned > 0)
      for (int e = 0; e < ne; e++) {
        const int32_t* d = &sp->el_dofs[(size_t)e * nloc];
        for (int i = 0; i < sp->nedge; i++) {
          const int a = m->el[(size_t)e * nvert + (tet ? TetTopo::edge(i, 0) : HexTopo::edge(i, 0))];
          const int b = m->el[(size_t)e * nvert + (tet ? TetTopo::edge(i, 1) : HexTopo::edge(i, 1))];
          for (int k = 0; k < ned; k++) {
            vb[a].push_back(d[nvert + i * ned + k]);
            vb[b].push_back(d[nvert + i * ned + k]);
          }
        }
      }
    for (int v = 0; v < nv; v++) {
      std::sort(vb[v].begin() + 1, vb[v].end());
      vb[v].erase(std::unique(vb[v].begin() + 1, vb[v].end()), vb[v].end());
      add_block(vb[v]);
    }
  } else {
    for (int v = 0; v < nv; v++) add_block({v});
    for (int g = 0; g < sp->ned; g++) {
      tmp.clear();
      for (int k = 0; k < ned; k++) tmp.push_back((int32_t)(sp->first_edge + (int64_t)g * ned + k));
      add_block(tmp);
    }
  }
  for (int f = 0; f < sp->nfa; f++) {
    tmp.clear();
    for (int k = 0; k < sp->n_face_dofs; k++) tmp.push_back((int32_t)(sp->first_face + (int64_t)f * sp->n_face_dofs + k));
    add_block(tmp);
  }
  for (int e = 0; e < ne; e++) {
    tmp.clear();
    for (int k = 0; k < sp->n_cell_dofs; k++) tmp.push_back((int32_t)(sp->first_cell + (int64_t)e * sp->n_cell_dofs + k));
    add_block(tmp);
  }
}


__device__ __forceinline__ double csr_entry(const int64_t* rowptr, const int32_t* colind, const double* vals, int row,
                                            int col) {
  int64_t lo = rowptr[row], hi = rowptr[row + 1] - 1;
  while (lo <= hi) {
    const int64_t mid = (lo + hi) >> 1;
    const int c = colind[mid];
    if (c == col) return vals[mid];
    if (c < col) lo = mid + 1; else hi = mid - 1;
  }
  return 0.0;  // not in the pattern: the two DOFs share no element
}

// One block per CTA: M = A[dofs, dofs] (row-major, s x s), then the in-place
// Gauss-Jordan inverse without pivoting (the blocks of an SPD matrix are SPD:
// every pivot is a Schur complement's diagonal, positive).  A pivot that is
// not positive sets *bad.
__global__ void __launch_bounds__(256) block_invert_kernel(int64_t nblocks, const int64_t* __restrict__ boff,
                                                           const int64_t* __restrict__ moff, const int32_t* __restrict__ dofs,
                                                           const int64_t* __restrict__ rowptr,
                                                           const int32_t* __restrict__ colind,
                                                           const double* __restrict__ vals, double* inv, int* bad) {
  for (int64_t b = blockIdx.x; b < nblocks; b += gridDim.x) {
    const int64_t o = boff[b];
    const int s = (int)(boff[b + 1] - o);
    double* M = inv + moff[b];
    for (int t = threadIdx.x; t < s * s; t += blockDim.x) M[t] = csr_entry(rowptr, colind, vals, dofs[o + t / s], dofs[o + t % s]);
    __syncthreads();
    for (int k = 0; k < s; k++) {
      const double akk = M[k * s + k];
      if (!(akk > 0.0)) {
        if (threadIdx.x == 0) atomicExch(bad, 1);
        break;  // uniform: every thread read the same pivot
      }
      const double piv = 1.0 / akk;
      __syncthreads();
      // row k scaled; the diagonal becomes 1/a_kk
      for (int j = threadIdx.x; j < s; j += blockDim.x) M[k * s + j] = j == k ? piv : M[k * s + j] * piv;
      __syncthreads();
      // a_ij -= a_ik a_kj (new row k) for i, j != k
      for (int t = threadIdx.x; t < s * s; t += blockDim.x) {
        const int i = t / s, j = t % s;
        if (i != k && j != k) M[t] -= M[i * s + k] * M[k * s + j];
      }
      __syncthreads();
      for (int i = threadIdx.x; i < s; i += blockDim.x)
        if (i != k) M[i * s + k] *= -piv;
      __syncthreads();
    }
    __syncthreads();
  }
}

template <class T>
__global__ void to_f32_kernel(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

// y[dof_r] += s sum_c Ainv_b[r][c] x[dof_c], one warp per block: the block's x
// values go to shared memory, lane r owns rows r, r+32, ...; Ainv is symmetric,
// so column c of the stored row-major inverse is read with consecutive lanes on
// consecutive rows (coalesced).
template <class T>
__global__ void __launch_bounds__(256) block_apply_kernel(int64_t nblocks, int smax, const int64_t* __restrict__ boff,
                                                          const int64_t* __restrict__ moff, const int32_t* __restrict__ dofs,
                                                          const T* __restrict__ inv, T s, const T* __restrict__ x,
                                                          T* __restrict__ y) {
  extern __shared__ __align__(16) unsigned char bsm[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  T* xs = (T*)bsm + (size_t)w * smax;
  for (int64_t b = (int64_t)blockIdx.x * nw + w; b < nblocks; b += (int64_t)gridDim.x * nw) {
    const int64_t o = boff[b];
    const int n = (int)(boff[b + 1] - o);
    const T* M = inv + moff[b];
    for (int c = lane; c < n; c += 32) xs[c] = x[dofs[o + c]];
    __syncwarp();
    for (int r0 = 0; r0 < n; r0 += 32) {
      const int r = r0 + lane;
      T acc = 0;
      if (r < n)
        for (int c = 0; c < n; c++) acc += M[(size_t)c * n + r] * xs[c];
      if (r < n) red_add(y + dofs[o + r], s * acc);
    }
    __syncwarp();
  }
}

// dense Gauss-Jordan inverse of an n x n matrix, one pivot step per two
// launches: the pivot row and column are copied first, so the rank-1 update
// reads no entry another thread of the same launch writes
__global__ void gj_copy_kernel(int n, int k, const double* __restrict__ M, double* __restrict__ row,
                               double* __restrict__ col) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    row[i] = M[(size_t)k * n + i];
    col[i] = M[(size_t)i * n + k];
  }
}
__global__ void gj_update_kernel(int n, int k, double* __restrict__ M, const double* __restrict__ row,
                                 const double* __restrict__ col, int* bad) {
  const double akk = row[k];
  if (!(akk > 0.0)) {
    if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) atomicExch(bad, 1);
    return;
  }
  const double piv = 1.0 / akk;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  for (int i = blockIdx.y; i < n; i += gridDim.y) {
    double v;
    if (i == k) v = j == k ? piv : row[j] * piv;
    else if (j == k) v = -col[i] * piv;
    else v = M[(size_t)i * n + j] - col[i] * row[j] * piv;
    M[(size_t)i * n + j] = v;
  }
}

// the coarse matrix on the free coarse DOFs: Mc[a][b] = A[cfree[a], cfree[b]]
__global__ void coarse_extract_kernel(int nc, const int32_t* __restrict__ cfree, const int32_t* __restrict__ cmap,
                                      const int64_t* __restrict__ rowptr, const int32_t* __restrict__ colind,
                                      const double* __restrict__ vals, double* Mc) {
  const int a = blockIdx.x;
  if (a >= nc) return;
  const int r = cfree[a];
  for (int64_t k = rowptr[r] + threadIdx.x; k < rowptr[r + 1]; k += blockDim.x) {
    const int b = cmap[colind[k]];
    if (b >= 0) Mc[(size_t)a * nc + b] = vals[k];
  }
}

// y[fine[a]] += s sum_b Minv[a][b] x[fine[b]]: one warp per row a (the inverse
// is symmetric; the row is read coalesced), x gathered through the cache
template <class T>
__global__ void __launch_bounds__(256) coarse_apply_kernel(int nc, const int32_t* __restrict__ fine,
                                                           const T* __restrict__ Minv, T s, const T* __restrict__ x,
                                                           T* __restrict__ y) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int nwt = (gridDim.x * blockDim.x) >> 5;
  for (int a = w; a < nc; a += nwt) {
    const T* row = Minv + (size_t)a * nc;
    T acc = 0;
    for (int b = lane; b < nc; b += 32) acc += row[b] * __ldg(x + fine[b]);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) y[fine[a]] += s * acc;
  }
}

// ---------------------------------------------------------------------------
void block_jacobi_setup(gh1_pre* pr, gh1_op* csr, int64_t nblocks, const std::vector<int64_t>& off,
                        const std::vector<int32_t>& dofs) {
  gh1_ctx* ctx = csr->ctx;
  cudaStream_t st = ctx->stream;
  GH1_CHECK(csr->kind == GH1_OP_CSR && csr->rowptr && csr->d_vals.p, GH1_ERR_ARG,
            "the block smoother needs an assembled (CSR) matrix");
  std::vector<int64_t> moff(nblocks + 1, 0);
  int smax = 0;
  for (int64_t b = 0; b < nblocks; b++) {
    const int64_t s = off[b + 1] - off[b];
    GH1_CHECK(s >= 0 && s <= 4096, GH1_ERR_ARG, "smoothing blocks hold 0..4096 DOFs");
    smax = std::max(smax, (int)s);
    moff[b + 1] = moff[b] + s * s;
  }
  for (auto d : dofs) GH1_CHECK(d >= 0 && d < csr->nrows, GH1_ERR_ARG, "block DOF out of range");
  pr->kind = 1;
  pr->nblocks = nblocks;
  pr->smax = std::max(smax, 1);
  pr->d_boff.upload(off, st);
  pr->d_moff.upload(moff, st);
  pr->d_bdofs.upload(dofs, st);
  pr->d_binv64.alloc(std::max<int64_t>(moff[nblocks], 1));
  DBuf<int> bad(1);
  bad.zero(st);
  if (nblocks > 0) {
    const int grid = (int)std::min<int64_t>(nblocks, (int64_t)ctx->nsm * 8);
    block_invert_kernel<<<grid, 256, 0, st>>>(nblocks, pr->d_boff.p, pr->d_moff.p, pr->d_bdofs.p, csr->rowptr,
                                             csr->colind, csr->d_vals.p, pr->d_binv64.p, bad.p);
    check_kernel(ctx, "block_invert_kernel");
  }
  pr->d_binv32.alloc(std::max<int64_t>(moff[nblocks], 1));
  to_f32_kernel<float><<<grid_for(ctx, moff[nblocks], 256), 256, 0, st>>>(moff[nblocks], pr->d_binv64.p, pr->d_binv32.p);
  check_kernel(ctx, "to_f32_kernel");
  int h = 0;
  GH1_CUDA(cudaMemcpyAsync(&h, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  GH1_CUDA(cudaStreamSynchronize(st));
  GH1_CHECK(h == 0, GH1_ERR_ARG, "a smoothing block of the matrix is not positive definite");
}

void coarse_setup(gh1_pre* pr, gh1_op* csr, int64_t nfine, const std::vector<int32_t>& embed,
                  const std::vector<uint8_t>& cfreemask) {
  gh1_ctx* ctx = csr->ctx;
  cudaStream_t st = ctx->stream;
  GH1_CHECK(csr->kind == GH1_OP_CSR && csr->rowptr && csr->d_vals.p, GH1_ERR_ARG,
            "the low-order solve needs an assembled (CSR) low-order matrix");
  const int64_t ncoarse = csr->nrows;
  std::vector<int32_t> cfree, fine, cmap(ncoarse, -1);
  for (int64_t i = 0; i < ncoarse; i++)
    if (cfreemask[i]) {
      cmap[i] = (int32_t)cfree.size();
      cfree.push_back((int32_t)i);
      GH1_CHECK(embed[i] >= 0 && embed[i] < nfine, GH1_ERR_ARG, "embedding target out of range");
      fine.push_back(embed[i]);
    }
  const int nc = (int)cfree.size();
  GH1_CHECK(nc <= 8192, GH1_ERR_UNSUPPORTED, "the exact low-order solve takes up to 8192 free coarse DOFs");
  pr->kind = 2;
  pr->nc = nc;
  pr->d_cfine.upload(fine, st);
  pr->d_cinv64.alloc(std::max<int64_t>((int64_t)nc * nc, 1));
  GH1_CUDA(cudaMemsetAsync(pr->d_cinv64.p, 0, (size_t)nc * nc * sizeof(double), st));
  if (nc > 0) {
    DBuf<int32_t> dcf, dcm;
    dcf.upload(cfree, st);
    dcm.upload(cmap, st);
    coarse_extract_kernel<<<nc, 128, 0, st>>>(nc, dcf.p, dcm.p, csr->rowptr, csr->colind, csr->d_vals.p, pr->d_cinv64.p);
    check_kernel(ctx, "coarse_extract_kernel");
    DBuf<double> row(nc), col(nc);
    DBuf<int> bad(1);
    bad.zero(st);
    const dim3 g((nc + 127) / 128, std::min(nc, 1024));
    for (int k = 0; k < nc; k++) {
      gj_copy_kernel<<<(nc + 255) / 256, 256, 0, st>>>(nc, k, pr->d_cinv64.p, row.p, col.p);
      gj_update_kernel<<<g, 128, 0, st>>>(nc, k, pr->d_cinv64.p, row.p, col.p, bad.p);
    }
    check_kernel(ctx, "gj_update_kernel");
    int h = 0;
    GH1_CUDA(cudaMemcpyAsync(&h, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    GH1_CUDA(cudaStreamSynchronize(st));
    GH1_CHECK(h == 0, GH1_ERR_ARG, "the low-order matrix on the free DOFs is not positive definite");
  }
  pr->d_cinv32.alloc(std::max<int64_t>((int64_t)nc * nc, 1));
  to_f32_kernel<float><<<grid_for(ctx, (int64_t)nc * nc, 256), 256, 0, st>>>((int64_t)nc * nc, pr->d_cinv64.p,
                                                                             pr->d_cinv32.p);
  check_kernel(ctx, "to_f32_kernel");
  GH1_CUDA(cudaStreamSynchronize(st));
}

// y = s C x (accumulate = 0) or y += s C x; kernels only
void pre_apply_any(gh1_pre* pr, double s, const void* x, void* y, int prec, int accumulate) {
  gh1_ctx* ctx = pr->ctx;
  cudaStream_t st = ctx->stream;
  const size_t es = prec == GH1_F64 ? sizeof(double) : sizeof(float);
  switch (pr->kind) {
    case 0:
      jacobi_apply(ctx, pr->n, s, pr->d_inv64.p, pr->d_inv32.p, x, y, prec, accumulate);
      return;
    case 3:
      pre_apply_any(pr->a, s, x, y, prec, accumulate);
      pre_apply_any(pr->b, s, x, y, prec, 1);
      return;
    default:
      break;
  }
  if (!accumulate) GH1_CUDA(cudaMemsetAsync(y, 0, pr->n * es, st));
  if (pr->kind == 1) {
    if (pr->nblocks == 0) return;
    const int grid = (int)std::min<int64_t>((pr->nblocks + 7) / 8, (int64_t)ctx->nsm * 8);
    const size_t smem = (size_t)8 * pr->smax * es;
    if (prec == GH1_F64)
      block_apply_kernel<double><<<grid, 256, smem, st>>>(pr->nblocks, pr->smax, pr->d_boff.p, pr->d_moff.p,
                                                          pr->d_bdofs.p, pr->d_binv64.p, s, (const double*)x, (double*)y);
    else
      block_apply_kernel<float><<<grid, 256, smem, st>>>(pr->nblocks, pr->smax, pr->d_boff.p, pr->d_moff.p,
                                                         pr->d_bdofs.p, pr->d_binv32.p, (float)s, (const float*)x, (float*)y);
    check_kernel(ctx, "block_apply_kernel");
  } else {
    if (pr->nc == 0) return;
    const int grid = std::min((pr->nc + 7) / 8, ctx->nsm * 8);
    if (prec == GH1_F64)
      coarse_apply_kernel<double><<<grid, 256, 0, st>>>(pr->nc, pr->d_cfine.p, pr->d_cinv64.p, s, (const double*)x,
                                                         (double*)y);
    else
      coarse_apply_kernel<float><<<grid, 256, 0, st>>>(pr->nc, pr->d_cfine.p, pr->d_cinv32.p, (float)s, (const float*)x,
                                                        (float*)y);
    check_kernel(ctx, "coarse_apply_kernel");
  }
}

// the largest dynamic shared memory a block apply asks for, allowed once
// outside any stream capture
void pre_prepare(gh1_pre* pr) {
  if (pr->kind == 3) {
    pre_prepare(pr->a);
    pre_prepare(pr->b);
  } else if (pr->kind == 1) {
    const size_t smem = (size_t)8 * pr->smax * sizeof(double);
    GH1_CHECK(smem <= 200 * 1024, GH1_ERR_UNSUPPORTED, "smoothing blocks too large for the block apply");
    if (smem > 48 * 1024) {
      GH1_CUDA(cudaFuncSetAttribute(block_apply_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      GH1_CUDA(cudaFuncSetAttribute(block_apply_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
  }
}

}  // namespace gh1
