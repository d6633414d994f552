// tetapply.cu -- matrix-free tet apply y += A x as two small GEMMs per tile of
// same-class elements.
//
// Same operator as tet_apply_kernel (matfree.cu) and as the reference's
// element-wise ApplyElementMatrix (fem/symbolicintegrator.cpp:2959-3040) on affine
// tets: y_e = B^T diag(kappa_e w_q |det J| J^{-1} J^{-T}) B x_e (+ mass).  The
// reference shapes depend on the element's vertex numbers only through their
// ranks (orientation class, 24 permutations), so all elements of one class share
// one table D_c of reference gradients (and values) at the rule points.  Elements
// are sorted by class once; a tile is up to 32 elements of one class, and per tile
//   P = D_c^T X           (rows: d/dx, d/dy, d/dz at nq points [+ values at the
//                          mass rule], columns: elements)
//   V = per-point 3x3 metric transform of P (per element constant, rule weight)
//   Y = D_c V             (local residuals), scattered with atomics.
// Both products are register-tiled FP32/FP64 FMA loops over shared memory
// (8 column groups of 4 elements x 16 row groups per 128-thread block).  The
// per-class table stays in shared memory while a block's tiles keep its class.
#include <algorithm>
#include <string>
#include <vector>
#include "common.cuh"
#include "hexcore.cuh"

namespace gh1 {

constexpr int TET_TT = 128;  // threads per block
constexpr int TET_TE = 32;   // elements per tile
constexpr int TET_RB = 8;    // row-tile depth of the first product (rows per thread per pass)
constexpr int TET_TI = 12;   // maximum row-tile depth of the second product (nloc <= 192, p <= 8)
// row-tile depth a chunked kernel is compiled for: 6 up to p = 6, else 12
inline int tet_ti_of(int nlocp) { return nlocp / 16 <= 6 ? 6 : 12; }

__host__ __device__ inline size_t tet_r16(size_t b) { return (b + 15) / 16 * 16; }

// sizes per order: local DOFs, points of the stiffness rule (degree 2p-2) and of
// the mass rule (degree 2p) -- the rules of tet_rule in tables.cu
template <int P>
struct TetDims {
  static constexpr int NLOC = (P + 1) * (P + 2) * (P + 3) / 6;
  static constexpr int NQ = P == 1 ? 1 : P == 2 ? 4 : P == 3 ? 14 : 24;
  static constexpr int NQM = P == 1 ? 4 : P == 2 ? 14 : P == 3 ? 24 : 46;
  static constexpr int NLOCP = (NLOC + 15) / 16 * 16;
  template <bool MASS>
  static constexpr int R() { return 3 * NQ + (MASS ? NQM : 0); }
  template <bool MASS>
  static constexpr int RP() { return (R<MASS>() + 15) / 16 * 16; }
};

// shared-memory carve-up of one block
template <class T>
struct TetSmem {
  int nlocp, Rp, Rs;
  __host__ __device__ size_t d() const { return tet_r16((size_t)nlocp * Rs * sizeof(T)); }
  __host__ __device__ size_t x() const { return tet_r16((size_t)nlocp * TET_TE * sizeof(T)); }
  __host__ __device__ size_t p() const { return tet_r16((size_t)Rp * TET_TE * sizeof(T)); }
  __host__ __device__ size_t w() const { return tet_r16((size_t)Rp * sizeof(T)); }
  __host__ __device__ size_t g() const { return tet_r16((size_t)TET_TE * 7 * sizeof(T)); }
  __host__ __device__ size_t dof() const { return tet_r16((size_t)TET_TE * nlocp * sizeof(int)); }
  __host__ __device__ size_t total() const { return d() + x() + p() + w() + g() + dof(); }
};

// four consecutive values from shared memory (16-byte aligned)
__device__ __forceinline__ void ld4(const float* p, float* v) {
  const float4 a = *(const float4*)p;
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
}
__device__ __forceinline__ void ld4(const double* p, double* v) {
  const double2 a = *(const double2*)p, b = *(const double2*)(p + 2);
  v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}

__device__ __forceinline__ void st4(float* p, const float* v) { *(float4*)p = make_float4(v[0], v[1], v[2], v[3]); }
__device__ __forceinline__ void st4(double* p, const double* v) {
  *(double2*)p = make_double2(v[0], v[1]);
  *(double2*)(p + 2) = make_double2(v[2], v[3]);
}

// tiles: [ntiles][4] = class, first position in perm, element count, 0.  Block b
// takes the contiguous tile range [b*ntiles/grid, (b+1)*ntiles/grid), which keeps
// its class (and the table in shared memory) for most consecutive tiles.
// D: [class][nlocp][Rs] with rows i >= nloc and columns r >= R zero; W: [Rp].
// Shared X and DOF rows are [i][element], P is [row][element].
template <class T, bool MASS, int P>
__global__ void __launch_bounds__(TET_TT)
tet_tile_kernel(int ntiles, const int* __restrict__ tiles, const int* __restrict__ perm, const int* __restrict__ tdofs,
                const T* __restrict__ Ge, const T* __restrict__ Me, const T* __restrict__ D, const T* __restrict__ W,
                const T* __restrict__ x, T* __restrict__ y, double* partial, unsigned int* counter, double* energy,
                const int* skip) {
  using Dm = TetDims<P>;
  constexpr int nloc = Dm::NLOC, nlocp = Dm::NLOCP, nq = Dm::NQ, nqm = Dm::NQM;
  constexpr int Rp = Dm::template RP<MASS>(), Rs = Rp + 1, ni = nlocp / 16;
  if (skip && *(volatile const int*)skip) return;
  extern __shared__ __align__(16) unsigned char smem[];
  const TetSmem<T> L{nlocp, Rp, Rs};
  T* sD = (T*)smem;
  T* sX = (T*)(smem + L.d());
  T* sP = (T*)(smem + L.d() + L.x());
  T* sW = (T*)(smem + L.d() + L.x() + L.p());
  T* sG = (T*)(smem + L.d() + L.x() + L.p() + L.w());
  int* sDof = (int*)(smem + L.d() + L.x() + L.p() + L.w() + L.g());
  const int tid = threadIdx.x, cg = tid & 7, rg = tid >> 3;  // 4 elements x (rows rg + 16 t)
  const int t0 = (int)((long long)ntiles * blockIdx.x / gridDim.x);
  const int t1 = (int)((long long)ntiles * (blockIdx.x + 1) / gridDim.x);
  const size_t dsize = (size_t)nlocp * Rs;
  for (int r = tid; r < Rp; r += TET_TT) sW[r] = W[r];
  int loaded = -1;
  T acc = 0;  // energy x^T A x of this thread's quadrature terms (working precision: FP64 is scarce)
  for (int t = t0; t < t1; t++) {
    const int cls = tiles[4 * t], start = tiles[4 * t + 1], cnt = tiles[4 * t + 2];
    __syncthreads();  // the previous tile is done with the shared arrays
    if (cls != loaded) {
      const T* src = D + (size_t)cls * dsize;
      for (size_t k = tid; k < dsize; k += TET_TT) sD[k] = src[k];
      loaded = cls;
    }
    // the tile's DOFs in tile-major order (element index fastest): entry
    // k = i * TET_TE + e is read coalesced and stored conflict-free
    for (int k = tid; k < TET_TE * nlocp; k += TET_TT) {
      const int d = tdofs[(size_t)t * TET_TE * nlocp + k];
      sDof[k] = d < 0 ? 0 : d;
      sX[k] = d < 0 ? T(0) : x[d];
    }
    for (int k = tid; k < TET_TE * 7; k += TET_TT) {
      const int e = k / 7, c = k % 7;
      T v = 0;
      if (e < cnt) v = c < 6 ? Ge[(size_t)perm[start + e] * 6 + c] : (MASS ? Me[perm[start + e]] : T(0));
      sG[k] = v;
    }
    __syncthreads();
    // P[r][e] = sum_i D[i][r] X[i][e]
    // unrolled (nt compile-time) unless the mass rule makes the table long (p = 4 with mass)
#pragma unroll(Rp <= 16 * TET_RB ? 1 : (Rp <= 256 ? 2 : 1))
    for (int r0 = 0; r0 < Rp; r0 += 16 * TET_RB) {
      const int nt = min(TET_RB, (Rp - r0) / 16);
      T a[TET_RB][4];
#pragma unroll
      for (int u = 0; u < TET_RB; u++) a[u][0] = a[u][1] = a[u][2] = a[u][3] = 0;
#pragma unroll
      for (int i = 0; i < nloc; i++) {
        T xv[4];
        ld4(sX + i * TET_TE + 4 * cg, xv);
        const T* drow = sD + (size_t)i * Rs + r0 + rg;
#pragma unroll
        for (int u = 0; u < TET_RB; u++)
          if (u < nt) {
            const T dv = drow[16 * u];
            a[u][0] += dv * xv[0]; a[u][1] += dv * xv[1]; a[u][2] += dv * xv[2]; a[u][3] += dv * xv[3];
          }
      }
#pragma unroll
      for (int u = 0; u < TET_RB; u++)
        if (u < nt) {
          st4(sP + (size_t)(r0 + rg + 16 * u) * TET_TE + 4 * cg, a[u]);
        }
    }
    __syncthreads();
    // per-point transform v = w_q G_e grad u (and the mass term), in place
    for (int k = tid; k < nq * TET_TE; k += TET_TT) {
      const int q = k / TET_TE, e = k % TET_TE;
      const T* g = sG + e * 7;
      T* px = sP + (size_t)q * TET_TE + e;
      T* py = px + (size_t)nq * TET_TE;
      T* pz = py + (size_t)nq * TET_TE;
      const T ux = *px, uy = *py, uz = *pz, w = sW[q];
      const T vx = w * (g[0] * ux + g[3] * uy + g[4] * uz);
      const T vy = w * (g[3] * ux + g[1] * uy + g[5] * uz);
      const T vz = w * (g[4] * ux + g[5] * uy + g[2] * uz);
      if (partial) acc += ux * vx + uy * vy + uz * vz;
      *px = vx; *py = vy; *pz = vz;
    }
    if (MASS) {
      for (int k = tid; k < nqm * TET_TE; k += TET_TT) {
        const int q = k / TET_TE, e = k % TET_TE;
        T* pm = sP + (size_t)(3 * nq + q) * TET_TE + e;
        const T u = *pm, vm = sW[3 * nq + q] * sG[e * 7 + 6] * u;
        if (partial) acc += u * vm;
        *pm = vm;
      }
    }
    __syncthreads();
    // Y[i][e] = sum_r D[i][r] V[r][e], rows i = rg + 16 t; scatter
    T b[ni][4];
#pragma unroll
    for (int u = 0; u < ni; u++) b[u][0] = b[u][1] = b[u][2] = b[u][3] = 0;
#pragma unroll 16
    for (int r = 0; r < Rp; r++) {
      T pv[4];
      ld4(sP + (size_t)r * TET_TE + 4 * cg, pv);
#pragma unroll
      for (int u = 0; u < ni; u++)
        if (u < ni) {
          const T dv = sD[(size_t)(rg + 16 * u) * Rs + r];
          b[u][0] += dv * pv[0]; b[u][1] += dv * pv[1]; b[u][2] += dv * pv[2]; b[u][3] += dv * pv[3];
        }
    }
#pragma unroll
    for (int u = 0; u < ni; u++) {
      const int i = rg + 16 * u;
      if (u < ni && i < nloc) {
#pragma unroll
        for (int c = 0; c < 4; c++) {
          const int e = 4 * cg + c;
          if (e < cnt) red_add(y + sDof[i * TET_TE + e], b[u][c]);
        }
      }
    }
  }
  if (partial) block_reduce_finish((double)acc, partial, counter, energy);
}

// ---- chunked variant (orders whose whole class table does not fit in shared memory)
// The rule points go through shared memory 16 at a time: per chunk the table
// slice (48 gradient rows, or 16 value rows of the mass rule) is loaded, the two
// products run on it and Y accumulates in registers across chunks.
//   Dg: [class][gradient chunk][nlocp][48] (rows: d/dx, d/dy, d/dz of 16 points)
//   Dm: [class][mass chunk][nlocp][16];  Wg, Wm: rule weights, zero-padded
constexpr int TET_QC = 16;

template <class T, bool MASS, int TI>
__global__ void __launch_bounds__(TET_TT)
tet_tile_chunk_kernel(int ntiles, const int* __restrict__ tiles, const int* __restrict__ perm, int nloc, int nlocp, int ncg,
                      int ncm, const int* __restrict__ tdofs, const T* __restrict__ Ge, const T* __restrict__ Me,
                      const T* __restrict__ Dg, const T* __restrict__ Dm, const T* __restrict__ Wg,
                      const T* __restrict__ Wm, const T* __restrict__ x, T* __restrict__ y, double* partial,
                      unsigned int* counter, double* energy, const int* skip) {
  if (skip && *(volatile const int*)skip) return;
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int RS = 3 * TET_QC + 1;  // row stride of the table slice (odd: conflict-free column reads)
  T* sD = (T*)smem;                                                   // [nlocp][RS]
  T* sX = (T*)(smem + tet_r16((size_t)nlocp * RS * sizeof(T)));       // [nlocp][TE]
  T* sP = sX + (size_t)nlocp * TET_TE;                                // [48][TE]
  T* sG = sP + (size_t)3 * TET_QC * TET_TE;                           // [TE][7]
  int* sDof = (int*)(sG + TET_TE * 7);                                // [nlocp][TE]
  const int tid = threadIdx.x, cg = tid & 7, rg = tid >> 3;
  const int t0 = (int)((long long)ntiles * blockIdx.x / gridDim.x);
  const int t1 = (int)((long long)ntiles * (blockIdx.x + 1) / gridDim.x);
  const int ni = nlocp / 16;  // block-uniform
  T acc = 0;  // energy of this thread's quadrature terms, in the working precision
  for (int t = t0; t < t1; t++) {
    const int cls = tiles[4 * t], start = tiles[4 * t + 1], cnt = tiles[4 * t + 2];
    __syncthreads();
    // the tile's DOFs in tile-major order: entry k = i * TET_TE + e is read coalesced
    for (int k = tid; k < TET_TE * nlocp; k += TET_TT) {
      const int d = tdofs[(size_t)t * TET_TE * nlocp + k];
      sDof[k] = d < 0 ? 0 : d;
      sX[k] = d < 0 ? T(0) : x[d];
    }
    for (int k = tid; k < TET_TE * 7; k += TET_TT) {
      const int e = k / 7, c = k % 7;
      T v = 0;
      if (e < cnt) v = c < 6 ? Ge[(size_t)perm[start + e] * 6 + c] : (MASS ? Me[perm[start + e]] : T(0));
      sG[k] = v;
    }
    T b[TI][4];
#pragma unroll
    for (int u = 0; u < TI; u++) b[u][0] = b[u][1] = b[u][2] = b[u][3] = 0;
    const int nchunk = ncg + (MASS ? ncm : 0);
    for (int cc = 0; cc < nchunk; cc++) {
      const bool grad = cc < ncg;
      const int RC = grad ? 3 * TET_QC : TET_QC;  // rows of this slice
      const T* src = grad ? Dg + ((size_t)cls * ncg + cc) * nlocp * (3 * TET_QC)
                          : Dm + ((size_t)cls * ncm + (cc - ncg)) * nlocp * TET_QC;
      __syncthreads();  // X, G, DOFs ready; the previous slice is consumed
      for (int k = tid; k < nlocp * RC; k += TET_TT) sD[(k / RC) * RS + k % RC] = src[k];
      __syncthreads();
      // P[r][e] = sum_i D[i][r] X[i][e], rows r = rg + 16 u
      {
        T a[3][4];
#pragma unroll
        for (int u = 0; u < 3; u++) a[u][0] = a[u][1] = a[u][2] = a[u][3] = 0;
        const int nt = RC / 16;
        for (int i = 0; i < nloc; i++) {
          T xv[4];
          ld4(sX + i * TET_TE + 4 * cg, xv);
#pragma unroll
          for (int u = 0; u < 3; u++)
            if (u < nt) {
              const T dv = sD[i * RS + rg + 16 * u];
              a[u][0] += dv * xv[0]; a[u][1] += dv * xv[1]; a[u][2] += dv * xv[2]; a[u][3] += dv * xv[3];
            }
        }
#pragma unroll
        for (int u = 0; u < 3; u++)
          if (u < nt) st4(sP + (size_t)(rg + 16 * u) * TET_TE + 4 * cg, a[u]);
      }
      __syncthreads();
      if (grad) {
        for (int k = tid; k < TET_QC * TET_TE; k += TET_TT) {
          const int q = k / TET_TE, e = k % TET_TE;
          const T* g = sG + e * 7;
          T* px = sP + (size_t)q * TET_TE + e;
          T* py = px + (size_t)TET_QC * TET_TE;
          T* pz = py + (size_t)TET_QC * TET_TE;
          const T ux = *px, uy = *py, uz = *pz, w = Wg[cc * TET_QC + q];
          const T vx = w * (g[0] * ux + g[3] * uy + g[4] * uz);
          const T vy = w * (g[3] * ux + g[1] * uy + g[5] * uz);
          const T vz = w * (g[4] * ux + g[5] * uy + g[2] * uz);
          if (partial) acc += ux * vx + uy * vy + uz * vz;
          *px = vx; *py = vy; *pz = vz;
        }
      } else {
        for (int k = tid; k < TET_QC * TET_TE; k += TET_TT) {
          const int q = k / TET_TE, e = k % TET_TE;
          T* pm = sP + (size_t)q * TET_TE + e;
          const T u = *pm, vm = Wm[(cc - ncg) * TET_QC + q] * sG[e * 7 + 6] * u;
          if (partial) acc += u * vm;
          *pm = vm;
        }
      }
      __syncthreads();
      // Y[i][e] += sum_r D[i][r] V[r][e], rows i = rg + 16 u
      for (int r = 0; r < RC; r++) {
        T pv[4];
        ld4(sP + (size_t)r * TET_TE + 4 * cg, pv);
#pragma unroll
        for (int u = 0; u < TI; u++)
          if (u < ni) {
            const T dv = sD[(rg + 16 * u) * RS + r];
            b[u][0] += dv * pv[0]; b[u][1] += dv * pv[1]; b[u][2] += dv * pv[2]; b[u][3] += dv * pv[3];
          }
      }
    }
#pragma unroll
    for (int u = 0; u < TI; u++) {
      const int i = rg + 16 * u;
      if (u < ni && i < nloc) {
#pragma unroll
        for (int c = 0; c < 4; c++) {
          const int e = 4 * cg + c;
          if (e < cnt) red_add(y + sDof[i * TET_TE + e], b[u][c]);
        }
      }
    }
  }
  if (partial) block_reduce_finish((double)acc, partial, counter, energy);
}

template <class T>
__host__ __device__ inline size_t tet_chunk_smem(int nlocp) {
  return tet_r16((size_t)nlocp * (3 * TET_QC + 1) * sizeof(T)) +
         tet_r16(((size_t)nlocp * TET_TE + 3 * TET_QC * TET_TE + TET_TE * 7) * sizeof(T) +
                 (size_t)nlocp * TET_TE * sizeof(int));
}

// D[c][i][r] from the per-class tables: rows r < 3 nq are d/dx, d/dy, d/dz of
// shape i at the stiffness-rule points (tab[c][q][i][1..3]); the next nqm rows the
// values at the mass-rule points (tabm[c][q][i]); everything else zero
template <class T>
__global__ void tet_tile_table_kernel(int ncls, int nloc, int nlocp, int nq, int nqm, int R, int Rs,
                                      const T* __restrict__ tab, const double* __restrict__ tabm, T* D) {
  const int64_t tot = (int64_t)ncls * nlocp * Rs;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < tot; k += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(k % Rs), i = (int)((k / Rs) % nlocp), c = (int)(k / ((int64_t)Rs * nlocp));
    T v = 0;
    if (i < nloc && r < R) {
      if (r < 3 * nq) v = tab[(((size_t)c * nq + r % nq) * nloc + i) * 4 + 1 + r / nq];
      else v = (T)tabm[((size_t)c * nqm + (r - 3 * nq)) * nloc + i];
    }
    D[k] = v;
  }
}

template <class T, bool MASS, int P>
static int tet_tile_occupancy_p() {
  auto kern = tet_tile_kernel<T, MASS, P>;
  using Dm = TetDims<P>;
  const TetSmem<T> L{Dm::NLOCP, Dm::template RP<MASS>(), Dm::template RP<MASS>() + 1};
  const size_t smem = L.total();
  int dev = 0, optin = 0;
  GH1_CUDA(cudaGetDevice(&dev));
  GH1_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  cudaFuncAttributes fa;
  GH1_CUDA(cudaFuncGetAttributes(&fa, kern));
  const int avail = optin - (int)fa.sharedSizeBytes;
  if ((long long)smem > avail) return 0;
  GH1_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, avail));
  int v = 0;
  GH1_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kern, TET_TT, smem));
  return v;
}

#define GH1_TET_P_SWITCH(P, CASE)                                                  \
  switch (P) {                                                                     \
    CASE(1) CASE(2) CASE(3) CASE(4)                                                \
    default: throw Error(GH1_ERR_UNSUPPORTED, "tiled tet apply: order out of range"); \
  }

template <class T>
static int tet_tile_occupancy(int p, bool mass) {
  int v = 0;
#define GH1_TET_OCC(PP)                                                                            \
  case PP:                                                                                         \
    v = mass ? tet_tile_occupancy_p<T, true, PP>() : tet_tile_occupancy_p<T, false, PP>();         \
    break;
  GH1_TET_P_SWITCH(p, GH1_TET_OCC)
#undef GH1_TET_OCC
  return v;
}

// the space's rules are the ones the compiled sizes assume
static bool tet_dims_match(int p, int nq, int nqm) {
  switch (p) {
    case 1: return nq == TetDims<1>::NQ && nqm == TetDims<1>::NQM;
    case 2: return nq == TetDims<2>::NQ && nqm == TetDims<2>::NQM;
    case 3: return nq == TetDims<3>::NQ && nqm == TetDims<3>::NQM;
    case 4: return nq == TetDims<4>::NQ && nqm == TetDims<4>::NQM;
    default: return false;
  }
}

// chunked tables: Dg[c][cc][i][r] (r < 48: component r / 16 of point cc*16 + r % 16)
// and Dm[c][cm][i][r] (value at mass point cm*16 + r); zero beyond the rules
template <class T>
__global__ void tet_chunk_table_kernel(int ncls, int nloc, int nlocp, int nq, int nqm, int ncg, int ncm,
                                       const T* __restrict__ tab, const double* __restrict__ tabm, T* Dg, T* Dm) {
  const int64_t tg = (int64_t)ncls * ncg * nlocp * 3 * TET_QC, tm = (int64_t)ncls * ncm * nlocp * TET_QC;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < tg + tm; k += (int64_t)gridDim.x * blockDim.x) {
    if (k < tg) {
      const int r = (int)(k % (3 * TET_QC)), i = (int)((k / (3 * TET_QC)) % nlocp);
      const int64_t ccc = k / ((int64_t)3 * TET_QC * nlocp);
      const int cc = (int)(ccc % ncg), c = (int)(ccc / ncg);
      const int q = cc * TET_QC + r % TET_QC, comp = r / TET_QC;
      Dg[k] = (i < nloc && q < nq) ? tab[(((size_t)c * nq + q) * nloc + i) * 4 + 1 + comp] : T(0);
    } else {
      const int64_t km = k - tg;
      const int r = (int)(km % TET_QC), i = (int)((km / TET_QC) % nlocp);
      const int64_t ccc = km / ((int64_t)TET_QC * nlocp);
      const int cm = (int)(ccc % ncm), c = (int)(ccc / ncm);
      const int q = cm * TET_QC + r;
      Dm[km] = (i < nloc && q < nqm) ? (T)tabm[((size_t)c * nqm + q) * nloc + i] : T(0);
    }
  }
}

template <class T, bool MASS, int TI>
static int tet_chunk_occupancy_ti(int nlocp) {
  auto kern = tet_tile_chunk_kernel<T, MASS, TI>;
  const size_t smem = tet_chunk_smem<T>(nlocp);
  int dev = 0, optin = 0;
  GH1_CUDA(cudaGetDevice(&dev));
  GH1_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  cudaFuncAttributes fa;
  GH1_CUDA(cudaFuncGetAttributes(&fa, kern));
  const int avail = optin - (int)fa.sharedSizeBytes;
  if ((long long)smem > avail) return 0;
  GH1_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, avail));
  int v = 0;
  GH1_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kern, TET_TT, smem));
  return v;
}

template <class T, bool MASS>
static int tet_chunk_occupancy(int nlocp) {
  return tet_ti_of(nlocp) == 6 ? tet_chunk_occupancy_ti<T, MASS, 6>(nlocp) : tet_chunk_occupancy_ti<T, MASS, 12>(nlocp);
}

// chunked tables and weights for all precisions the operator carries
static void tet_chunk_setup(gh1_op* op, const std::vector<double>& rule, const std::vector<double>& rulem) {
  gh1_space* sp = op->sp;
  cudaStream_t s = sp->ctx->stream;
  const int nloc = sp->nloc, nq = sp->tet_nq, nqm = sp->tet_nq_mass, nlocp = (nloc + 15) / 16 * 16;
  const int ncg = (nq + TET_QC - 1) / TET_QC, ncm = (nqm + TET_QC - 1) / TET_QC, ncls = N_TET_CLASSES;
  op->tet_chunked = true;
  op->tet_ncg = ncg;
  op->tet_ncm = ncm;
  const int64_t ng = (int64_t)ncls * ncg * nlocp * 3 * TET_QC, nm = (int64_t)ncls * ncm * nlocp * TET_QC;
  std::vector<double> wg((size_t)ncg * TET_QC, 0.0), wm((size_t)ncm * TET_QC, 0.0);
  for (int q = 0; q < nq; q++) wg[q] = rule[4 * q + 3];
  for (int q = 0; q < nqm; q++) wm[q] = rulem[4 * q + 3];
  const int tgrid = (int)std::min<int64_t>((ng + nm + 255) / 256, 4096);
  op->d_tetD64.alloc(ng);
  op->d_tetDm64.alloc(nm);
  tet_chunk_table_kernel<double><<<tgrid, 256, 0, s>>>(ncls, nloc, nlocp, nq, nqm, ncg, ncm, sp->d_tab64.p,
                                                       sp->d_tabm64.p, op->d_tetD64.p, op->d_tetDm64.p);
  check_kernel(sp->ctx, "tet_chunk_table_kernel");
  op->d_tetw64.upload(wg, s);
  op->d_tetwm64.upload(wm, s);
  op->tet_tiles_per_sm[0] = op->has_mass ? tet_chunk_occupancy<double, true>(nlocp) : tet_chunk_occupancy<double, false>(nlocp);
  if (op->prec_mask & 2) {
    op->d_tetD32.alloc(ng);
    op->d_tetDm32.alloc(nm);
    tet_chunk_table_kernel<float><<<tgrid, 256, 0, s>>>(ncls, nloc, nlocp, nq, nqm, ncg, ncm, sp->d_tab32.p,
                                                        sp->d_tabm64.p, op->d_tetD32.p, op->d_tetDm32.p);
    check_kernel(sp->ctx, "tet_chunk_table_kernel");
    std::vector<float> wg32(wg.begin(), wg.end()), wm32(wm.begin(), wm.end());
    op->d_tetw32.upload(wg32, s);
    op->d_tetwm32.upload(wm32, s);
    op->tet_tiles_per_sm[1] = op->has_mass ? tet_chunk_occupancy<float, true>(nlocp) : tet_chunk_occupancy<float, false>(nlocp);
  }
  GH1_CUDA(cudaStreamSynchronize(s));  // host staging vectors go out of scope
}

// tile-major DOF table of the 32-element tiles: tdofs[(t * nlocp + i) * TET_TE + e]
// = DOF i of element e of tile t, -1 past the tile's count or nloc
__global__ void tet_tile_dofs_kernel(int ntiles, int nloc, int nlocp, const int* __restrict__ tiles,
                                     const int* __restrict__ perm, const int* __restrict__ eldofs, int* __restrict__ tdofs) {
  const int64_t tot = (int64_t)ntiles * nlocp * TET_TE;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < tot; k += (int64_t)gridDim.x * blockDim.x) {
    const int e = (int)(k % TET_TE), i = (int)((k / TET_TE) % nlocp), t = (int)(k / ((int64_t)TET_TE * nlocp));
    const int st = tiles[4 * t + 1], cnt = tiles[4 * t + 2];
    tdofs[k] = (e < cnt && i < nloc) ? eldofs[(size_t)perm[st + e] * nloc + i] : -1;
  }
}

// counting sort of the elements by orientation class; tiles of up to TET_TE
// elements of one class ([ntiles][4] = class, first position, count, 0)
static void tet_class_tiles(gh1_op* op) {
  gh1_space* sp = op->sp;
  cudaStream_t s = sp->ctx->stream;
  const int ne = sp->mesh->ne, ncls = N_TET_CLASSES;
  std::vector<uint8_t> cls(ne);
  GH1_CUDA(cudaMemcpyAsync(cls.data(), sp->d_class.p, ne, cudaMemcpyDeviceToHost, s));
  GH1_CUDA(cudaStreamSynchronize(s));
  std::vector<int> count(ncls + 1, 0), perm(ne), tiles;
  for (int e = 0; e < ne; e++) count[cls[e] + 1]++;
  for (int c = 0; c < ncls; c++) count[c + 1] += count[c];
  std::vector<int> pos(count.begin(), count.end() - 1);
  for (int e = 0; e < ne; e++) perm[pos[cls[e]]++] = e;
  for (int c = 0; c < ncls; c++)
    for (int a = count[c]; a < count[c + 1]; a += TET_TE) {
      tiles.push_back(c);
      tiles.push_back(a);
      tiles.push_back(std::min(TET_TE, count[c + 1] - a));
      tiles.push_back(0);
    }
  op->d_tet_perm.upload(perm, s);
  op->d_tet_tiles.upload(tiles, s);
  op->tet_ntiles = (int)tiles.size() / 4;
  const int nloc = sp->nloc, nlocp = (nloc + 15) / 16 * 16;
  op->d_tet_tdofs.alloc((size_t)op->tet_ntiles * nlocp * TET_TE);
  const int64_t tot = (int64_t)op->tet_ntiles * nlocp * TET_TE;
  tet_tile_dofs_kernel<<<(unsigned)std::min<int64_t>((tot + 255) / 256, 65535), 256, 0, s>>>(
      op->tet_ntiles, nloc, nlocp, op->d_tet_tiles.p, op->d_tet_perm.p, sp->d_eldofs.p, op->d_tet_tdofs.p);
  check_kernel(sp->ctx, "tet_tile_dofs_kernel");
  GH1_CUDA(cudaStreamSynchronize(s));  // host staging vectors go out of scope
}

// Class-sorted element order, tiles, tables and occupancy.  GH1_TET_KERNEL=elementwise
// keeps the element-wise kernel (for comparisons).
void tet_tiles_setup(gh1_op* op) {
  gh1_space* sp = op->sp;
  op->tet_tiles_per_sm[0] = op->tet_tiles_per_sm[1] = 0;
  const char* env = getenv("GH1_TET_KERNEL");
  if (env && std::string(env) == "elementwise") return;
  const int ne = sp->mesh->ne, nloc = sp->nloc, nq = sp->tet_nq, nqm = sp->tet_nq_mass;
  const int nlocp = (nloc + 15) / 16 * 16;
  op->tet_chunked = false;
  if (nlocp / 16 > TET_TI || ne == 0) return;
  const int R = 3 * nq + (op->has_mass ? nqm : 0), Rp = (R + 15) / 16 * 16, Rs = Rp + 1;
  const int ncls = N_TET_CLASSES;
  cudaStream_t s = sp->ctx->stream;
  tet_class_tiles(op);
  std::vector<double> rule(4 * (size_t)nq), rulem(4 * (size_t)nqm);
  GH1_CUDA(cudaMemcpyAsync(rule.data(), sp->d_tq.p, rule.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  if (nqm) GH1_CUDA(cudaMemcpyAsync(rulem.data(), sp->d_tqm.p, rulem.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  GH1_CUDA(cudaStreamSynchronize(s));
  const bool mass = op->has_mass;
  // the whole class table in shared memory (compiled orders), else 16-point chunks
  const TetSmem<double> full{nlocp, Rp, Rs};
  if (!tet_dims_match(sp->p, nq, nqm) || full.total() > (size_t)200 * 1024) {
    tet_chunk_setup(op, rule, rulem);
    return;
  }
  std::vector<double> w(Rp, 0.0);
  for (int r = 0; r < 3 * nq; r++) w[r] = rule[4 * (r % nq) + 3];
  if (op->has_mass)
    for (int q = 0; q < nqm; q++) w[3 * nq + q] = rulem[4 * q + 3];
  op->tet_R = R; op->tet_Rp = Rp; op->tet_Rs = Rs;
  const int64_t tot = (int64_t)ncls * nlocp * Rs;
  const int tgrid = (int)std::min<int64_t>((tot + 255) / 256, 4096);
  op->d_tetD64.alloc(tot);
  tet_tile_table_kernel<double><<<tgrid, 256, 0, s>>>(ncls, nloc, nlocp, nq, nqm, R, Rs, sp->d_tab64.p, sp->d_tabm64.p,
                                                      op->d_tetD64.p);
  check_kernel(sp->ctx, "tet_tile_table_kernel");
  op->d_tetw64.upload(w, s);
  op->tet_tiles_per_sm[0] = tet_tile_occupancy<double>(sp->p, mass);
  if (op->prec_mask & 2) {
    op->d_tetD32.alloc(tot);
    tet_tile_table_kernel<float><<<tgrid, 256, 0, s>>>(ncls, nloc, nlocp, nq, nqm, R, Rs, sp->d_tab32.p, sp->d_tabm64.p,
                                                       op->d_tetD32.p);
    check_kernel(sp->ctx, "tet_tile_table_kernel");
    std::vector<float> w32(w.begin(), w.end());
    op->d_tetw32.upload(w32, s);
    op->tet_tiles_per_sm[1] = tet_tile_occupancy<float>(sp->p, mass);
  }
  GH1_CUDA(cudaStreamSynchronize(s));  // host staging vectors go out of scope
  // FP32: the same products on the tensor cores, kept when faster on this mesh
  // (GH1_TET_KERNEL=tc / tile forces one)
  tet_tc_setup(op);
  op->tet_use_tc = false;
  if (op->tet_tc_per_sm > 0) {
    const char* force = getenv("GH1_TET_KERNEL");
    if (force && std::string(force) == "tc") {
      op->tet_use_tc = true;
    } else if (!(force && std::string(force) == "tile") && ne >= 4096) {
      DBuf<float> xs(op->nrows), ys(op->nrows);
      xs.zero(s);
      cudaEvent_t a, b;
      GH1_CUDA(cudaEventCreate(&a));
      GH1_CUDA(cudaEventCreate(&b));
      float ms[2];
      for (int v = 0; v < 2; v++) {
        op->tet_use_tc = v == 1;
        for (int r = 0; r < 5; r++) {
          if (r == 2) GH1_CUDA(cudaEventRecord(a, s));
          tet_tiles_apply(op, GH1_F32, xs.p, ys.p, nullptr, nullptr, nullptr, nullptr);
        }
        GH1_CUDA(cudaEventRecord(b, s));
        GH1_CUDA(cudaEventSynchronize(b));
        GH1_CUDA(cudaEventElapsedTime(&ms[v], a, b));
      }
      cudaEventDestroy(a);
      cudaEventDestroy(b);
      op->tet_use_tc = ms[1] < ms[0];
    }
  }
  tet_mass_tc_setup(op);  // FP32 with a mass term: the tensor-core B^T D B kernel where faster
}

template <class T, bool MASS, int P>
static void tet_tile_launch_p(gh1_op* op, int grid, const T* D, const T* W, const T* G, const T* M, const T* x, T* y,
                              double* partial, unsigned int* counter, double* energy, const int* skip) {
  using Dm = TetDims<P>;
  const TetSmem<T> L{Dm::NLOCP, Dm::template RP<MASS>(), Dm::template RP<MASS>() + 1};
  gh1_space* sp = op->sp;
  tet_tile_kernel<T, MASS, P><<<grid, TET_TT, L.total(), sp->ctx->stream>>>(
      op->tet_ntiles, op->d_tet_tiles.p, op->d_tet_perm.p, op->d_tet_tdofs.p, G, M, D, W, x, y, partial, counter, energy,
      skip);
  check_kernel(sp->ctx, "tet_tile_kernel");
}

template <class T>
static void tet_tile_launch(gh1_op* op, int per_sm, const T* D, const T* W, const T* G, const T* M, const T* x, T* y,
                            double* partial, unsigned int* counter, double* energy, const int* skip) {
  gh1_space* sp = op->sp;
  const int grid = std::max(1, std::min(op->tet_ntiles, sp->ctx->nsm * per_sm));
  const bool mass = op->has_mass;
#define GH1_TET_LAUNCH(PP)                                                                                   \
  case PP:                                                                                                   \
    if (mass) tet_tile_launch_p<T, true, PP>(op, grid, D, W, G, M, x, y, partial, counter, energy, skip);   \
    else tet_tile_launch_p<T, false, PP>(op, grid, D, W, G, M, x, y, partial, counter, energy, skip);       \
    break;
  GH1_TET_P_SWITCH(sp->p, GH1_TET_LAUNCH)
#undef GH1_TET_LAUNCH
}

template <class T>
static void tet_chunk_launch(gh1_op* op, int per_sm, const T* Dg, const T* Dm, const T* Wg, const T* Wm, const T* G,
                             const T* M, const T* x, T* y, double* partial, unsigned int* counter, double* energy,
                             const int* skip) {
  gh1_space* sp = op->sp;
  const int nlocp = (sp->nloc + 15) / 16 * 16;
  const int grid = std::max(1, std::min(op->tet_ntiles, sp->ctx->nsm * per_sm));
  const size_t smem = tet_chunk_smem<T>(nlocp);
#define GH1_CHUNK_LAUNCH(MASS, TI)                                                                       \
  tet_tile_chunk_kernel<T, MASS, TI><<<grid, TET_TT, smem, sp->ctx->stream>>>(                            \
      op->tet_ntiles, op->d_tet_tiles.p, op->d_tet_perm.p, sp->nloc, nlocp, op->tet_ncg, op->tet_ncm,      \
      op->d_tet_tdofs.p, G, M, Dg, Dm, Wg, Wm, x, y, partial, counter, energy, skip)
  const bool ti6 = tet_ti_of(nlocp) == 6;
  if (op->has_mass) {
    if (ti6) GH1_CHUNK_LAUNCH(true, 6); else GH1_CHUNK_LAUNCH(true, 12);
  } else {
    if (ti6) GH1_CHUNK_LAUNCH(false, 6); else GH1_CHUNK_LAUNCH(false, 12);
  }
#undef GH1_CHUNK_LAUNCH
  check_kernel(sp->ctx, "tet_tile_chunk_kernel");
}

bool tet_tiles_apply(gh1_op* op, int prec, const void* x, void* y, double* partial, unsigned int* counter,
                     double* energy, const int* skip) {
  const int pi = prec == GH1_F64 ? 0 : 1;
  const int per_sm = op->tet_tiles_per_sm[pi];
  if (per_sm <= 0) return false;
  if (op->tet_chunked) {
    if (prec == GH1_F64)
      tet_chunk_launch<double>(op, per_sm, op->d_tetD64.p, op->d_tetDm64.p, op->d_tetw64.p, op->d_tetwm64.p,
                               op->d_G64.p, op->has_mass ? op->d_M64.p : nullptr, (const double*)x, (double*)y,
                               partial, counter, energy, skip);
    else
      tet_chunk_launch<float>(op, per_sm, op->d_tetD32.p, op->d_tetDm32.p, op->d_tetw32.p, op->d_tetwm32.p,
                              op->d_G32.p, op->has_mass ? op->d_M32.p : nullptr, (const float*)x, (float*)y,
                              partial, counter, energy, skip);
    return true;
  }
  if (prec == GH1_F32 && op->tet_use_tc) {
    tet_tc_apply(op, (const float*)x, (float*)y, partial, counter, energy, skip);
    return true;
  }
  if (prec == GH1_F32 && op->tet_bdb_tc) {  // stiffness + mass on the tensor cores
    tet_bdb_tc_apply(op, (const float*)x, (float*)y, partial, counter, energy, skip);
    return true;
  }
  if (prec == GH1_F64)
    tet_tile_launch<double>(op, per_sm, op->d_tetD64.p, op->d_tetw64.p, op->d_G64.p,
                            op->has_mass ? op->d_M64.p : nullptr, (const double*)x, (double*)y, partial, counter,
                            energy, skip);
  else
    tet_tile_launch<float>(op, per_sm, op->d_tetD32.p, op->d_tetw32.p, op->d_G32.p,
                           op->has_mass ? op->d_M32.p : nullptr, (const float*)x, (float*)y, partial, counter,
                           energy, skip);
  return true;
}

// ---- generic B^T D B on same-class tiles (bdb.cu sets up the element records) ----
// The degree-2p rule goes through shared memory 16 points at a time.  Per chunk
// the table slice holds 64 rows: value, d/dxi, d/deta, d/dzeta (row comp*16 + point)
// of every local shape; the tile products are those of the chunked kernel and the
// point transform is the 4x4 reference-coordinate matrix Mh of the element (times
// the rule weight; PP: one matrix per point, weight included).
//   Tb: [class][chunk][nlocp][64];  Wb: [chunk*16] weights, zero beyond the rule
template <class T>
__host__ __device__ inline size_t tet_bdb_smem(int nlocp) {
  return tet_r16((size_t)nlocp * (4 * TET_QC + 1) * sizeof(T)) +
         ((size_t)nlocp * TET_TE + 4 * TET_QC * TET_TE + TET_TE * 17) * sizeof(T) + (size_t)nlocp * TET_TE * sizeof(int);
}

template <class T, bool PP, int TI>
__global__ void __launch_bounds__(TET_TT)
tet_bdb_kernel(int ntiles, const int* __restrict__ tiles, const int* __restrict__ perm, int nloc, int nlocp, int ncb,
               int nq, const int* __restrict__ tdofs, const T* __restrict__ Mh, const T* __restrict__ Tb,
               const T* __restrict__ Wb, const T* __restrict__ x, T* __restrict__ y, double* partial,
               unsigned int* counter, double* energy, const int* skip) {
  if (skip && *(volatile const int*)skip) return;
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int RC = 4 * TET_QC, RS = RC + 1;  // rows per chunk; odd stride: conflict-free column reads
  T* sD = (T*)smem;                                                // [nlocp][RS]
  T* sX = (T*)(smem + tet_r16((size_t)nlocp * RS * sizeof(T)));    // [nlocp][TE]
  T* sP = sX + (size_t)nlocp * TET_TE;                             // [64][TE]
  T* sM = sP + (size_t)RC * TET_TE;                                // [TE][17] element records
  int* sDof = (int*)(sM + TET_TE * 17);                            // [nlocp][TE]
  const int tid = threadIdx.x, cg = tid & 7, rg = tid >> 3;
  const int t0 = (int)((long long)ntiles * blockIdx.x / gridDim.x);
  const int t1 = (int)((long long)ntiles * (blockIdx.x + 1) / gridDim.x);
  const int ni = nlocp / 16;  // block-uniform
  T acc = 0;  // energy of this thread's quadrature terms, in the working precision
  for (int t = t0; t < t1; t++) {
    const int cls = tiles[4 * t], start = tiles[4 * t + 1], cnt = tiles[4 * t + 2];
    __syncthreads();
    // the tile's DOFs in tile-major order: entry k = i * TET_TE + e is read coalesced
    for (int k = tid; k < TET_TE * nlocp; k += TET_TT) {
      const int d = tdofs[(size_t)t * TET_TE * nlocp + k];
      sDof[k] = d < 0 ? 0 : d;
      sX[k] = d < 0 ? T(0) : x[d];
    }
    if (!PP)
      for (int k = tid; k < TET_TE * 16; k += TET_TT) {
        const int e = k / 16, c = k % 16;
        sM[e * 17 + c] = e < cnt ? Mh[(size_t)perm[start + e] * 16 + c] : T(0);
      }
    T b[TI][4];
#pragma unroll
    for (int u = 0; u < TI; u++) b[u][0] = b[u][1] = b[u][2] = b[u][3] = 0;
    for (int cc = 0; cc < ncb; cc++) {
      const T* src = Tb + ((size_t)cls * ncb + cc) * nlocp * RC;
      __syncthreads();  // X, records, DOFs ready; the previous slice is consumed
      for (int k = tid; k < nlocp * RC; k += TET_TT) sD[(k / RC) * RS + k % RC] = src[k];
      __syncthreads();
      // P[r][e] = sum_i D[i][r] X[i][e], rows r = rg + 16 u
      {
        T a[4][4];
#pragma unroll
        for (int u = 0; u < 4; u++) a[u][0] = a[u][1] = a[u][2] = a[u][3] = 0;
        for (int i = 0; i < nloc; i++) {
          T xv[4];
          ld4(sX + i * TET_TE + 4 * cg, xv);
#pragma unroll
          for (int u = 0; u < 4; u++) {
            const T dv = sD[i * RS + rg + 16 * u];
            a[u][0] += dv * xv[0]; a[u][1] += dv * xv[1]; a[u][2] += dv * xv[2]; a[u][3] += dv * xv[3];
          }
        }
#pragma unroll
        for (int u = 0; u < 4; u++) st4(sP + (size_t)(rg + 16 * u) * TET_TE + 4 * cg, a[u]);
      }
      __syncthreads();
      // point transform (v, v_x, v_y, v_z) = Mh (u, u_x, u_y, u_z), in place
      for (int k = tid; k < TET_QC * TET_TE; k += TET_TT) {
        const int q = k / TET_TE, e = k % TET_TE, qg = cc * TET_QC + q;
        T in[4], m[16];
#pragma unroll
        for (int c = 0; c < 4; c++) in[c] = sP[(size_t)(c * TET_QC + q) * TET_TE + e];
        if (PP) {
          const bool ok = e < cnt && qg < nq;
          const T* mp = Mh + ((size_t)(ok ? perm[start + e] : 0) * nq + (ok ? qg : 0)) * 16;
#pragma unroll
          for (int c = 0; c < 16; c++) m[c] = ok ? mp[c] : T(0);
        } else {
          const T w = Wb[qg];
#pragma unroll
          for (int c = 0; c < 16; c++) m[c] = w * sM[e * 17 + c];
        }
#pragma unroll
        for (int r = 0; r < 4; r++) {
          const T o = m[4 * r] * in[0] + m[4 * r + 1] * in[1] + m[4 * r + 2] * in[2] + m[4 * r + 3] * in[3];
          if (partial) acc += in[r] * o;
          sP[(size_t)(r * TET_QC + q) * TET_TE + e] = o;
        }
      }
      __syncthreads();
      // Y[i][e] += sum_r D[i][r] V[r][e], rows i = rg + 16 u
      for (int r = 0; r < RC; r++) {
        T pv[4];
        ld4(sP + (size_t)r * TET_TE + 4 * cg, pv);
#pragma unroll
        for (int u = 0; u < TI; u++)
          if (u < ni) {
            const T dv = sD[(rg + 16 * u) * RS + r];
            b[u][0] += dv * pv[0]; b[u][1] += dv * pv[1]; b[u][2] += dv * pv[2]; b[u][3] += dv * pv[3];
          }
      }
    }
#pragma unroll
    for (int u = 0; u < TI; u++) {
      const int i = rg + 16 * u;
      if (u < ni && i < nloc) {
#pragma unroll
        for (int c = 0; c < 4; c++) {
          const int e = 4 * cg + c;
          if (e < cnt) red_add(y + sDof[i * TET_TE + e], b[u][c]);
        }
      }
    }
  }
  if (partial) block_reduce_finish((double)acc, partial, counter, energy);
}

// Tb[c][cc][i][r] from the values and reference gradients at the degree-2p rule
// (t: [class][q][i][4]); zero for i >= nloc and points beyond the rule
template <class T>
__global__ void tet_bdb_table_kernel(int ncls, int nloc, int nlocp, int nq, int ncb, const T* __restrict__ t, T* Tb) {
  const int64_t tot = (int64_t)ncls * ncb * nlocp * 4 * TET_QC;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < tot; k += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(k % (4 * TET_QC)), i = (int)((k / (4 * TET_QC)) % nlocp);
    const int64_t ccc = k / ((int64_t)4 * TET_QC * nlocp);
    const int cc = (int)(ccc % ncb), c = (int)(ccc / ncb);
    const int q = cc * TET_QC + r % TET_QC, comp = r / TET_QC;
    Tb[k] = (i < nloc && q < nq) ? t[(((size_t)c * nq + q) * nloc + i) * 4 + comp] : T(0);
  }
}

template <class T, bool PP, int TI>
static int tet_bdb_occupancy_ti(int nlocp) {
  auto kern = tet_bdb_kernel<T, PP, TI>;
  const size_t smem = tet_bdb_smem<T>(nlocp);
  int dev = 0, optin = 0;
  GH1_CUDA(cudaGetDevice(&dev));
  GH1_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  cudaFuncAttributes fa;
  GH1_CUDA(cudaFuncGetAttributes(&fa, kern));
  const int avail = optin - (int)fa.sharedSizeBytes;
  GH1_CHECK((long long)smem <= avail, GH1_ERR_UNSUPPORTED, "tet B^T D B apply does not fit in shared memory");
  GH1_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, avail));
  int v = 0;
  GH1_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kern, TET_TT, smem));
  GH1_CHECK(v >= 1, GH1_ERR_UNSUPPORTED, "tet B^T D B apply does not fit on an SM");
  return v;
}

template <class T, bool PP>
static int tet_bdb_occupancy(int nlocp) {
  return tet_ti_of(nlocp) == 6 ? tet_bdb_occupancy_ti<T, PP, 6>(nlocp) : tet_bdb_occupancy_ti<T, PP, 12>(nlocp);
}

void tet_bdb_setup(gh1_op* op) {
  gh1_space* sp = op->sp;
  cudaStream_t s = sp->ctx->stream;
  const int nloc = sp->nloc, nq = sp->tet_nq_mass, nlocp = (nloc + 15) / 16 * 16, ncls = N_TET_CLASSES;
  GH1_CHECK(nlocp / 16 <= TET_TI, GH1_ERR_UNSUPPORTED, "tet order too high for the B^T D B apply");
  const int ncb = (nq + TET_QC - 1) / TET_QC;
  op->tet_ncb = ncb;
  tet_class_tiles(op);
  DBuf<double> t64;
  DBuf<float> t32;
  tet_mass_rule_tables(sp, t64, t32);
  const int64_t nt = (int64_t)ncls * ncb * nlocp * 4 * TET_QC;
  const int tgrid = (int)std::min<int64_t>((nt + 255) / 256, 4096);
  op->d_tetB64.alloc(nt);
  tet_bdb_table_kernel<double><<<tgrid, 256, 0, s>>>(ncls, nloc, nlocp, nq, ncb, t64.p, op->d_tetB64.p);
  check_kernel(sp->ctx, "tet_bdb_table_kernel");
  std::vector<double> rule(4 * (size_t)nq), w((size_t)ncb * TET_QC, 0.0);
  GH1_CUDA(cudaMemcpyAsync(rule.data(), sp->d_tqm.p, rule.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  GH1_CUDA(cudaStreamSynchronize(s));
  for (int q = 0; q < nq; q++) w[q] = rule[4 * q + 3];
  op->d_tetBw64.upload(w, s);
  const bool pp = op->bdb == 1;
  op->bdb_per_sm[0] = pp ? tet_bdb_occupancy<double, true>(nlocp) : tet_bdb_occupancy<double, false>(nlocp);
  op->bdb_per_sm[1] = 0;
  if (op->prec_mask & 2) {
    op->d_tetB32.alloc(nt);
    tet_bdb_table_kernel<float><<<tgrid, 256, 0, s>>>(ncls, nloc, nlocp, nq, ncb, t32.p, op->d_tetB32.p);
    check_kernel(sp->ctx, "tet_bdb_table_kernel");
    std::vector<float> w32(w.begin(), w.end());
    op->d_tetBw32.upload(w32, s);
    op->bdb_per_sm[1] = pp ? tet_bdb_occupancy<float, true>(nlocp) : tet_bdb_occupancy<float, false>(nlocp);
  }
  GH1_CUDA(cudaStreamSynchronize(s));
  tet_bdb_tc_setup(op, t64.p);         // FP32, records per element: the tensor-core form where faster
  GH1_CUDA(cudaStreamSynchronize(s));  // tables and host staging go out of scope
}

template <class T>
static void tet_bdb_launch(gh1_op* op, int per_sm, const T* Mh, const T* Tb, const T* Wb, const T* x, T* y,
                           double* partial, unsigned int* counter, double* energy, const int* skip) {
  gh1_space* sp = op->sp;
  const int nlocp = (sp->nloc + 15) / 16 * 16;
  const int grid = std::max(1, std::min(op->tet_ntiles, sp->ctx->nsm * per_sm));
  const size_t smem = tet_bdb_smem<T>(nlocp);
#define GH1_BDB_LAUNCH(PP, TI)                                                                            \
  tet_bdb_kernel<T, PP, TI><<<grid, TET_TT, smem, sp->ctx->stream>>>(                                     \
      op->tet_ntiles, op->d_tet_tiles.p, op->d_tet_perm.p, sp->nloc, nlocp, op->tet_ncb, sp->tet_nq_mass,  \
      op->d_tet_tdofs.p, Mh, Tb, Wb, x, y, partial, counter, energy, skip)
  const bool ti6 = tet_ti_of(nlocp) == 6;
  if (op->bdb == 1) {
    if (ti6) GH1_BDB_LAUNCH(true, 6); else GH1_BDB_LAUNCH(true, 12);
  } else {
    if (ti6) GH1_BDB_LAUNCH(false, 6); else GH1_BDB_LAUNCH(false, 12);
  }
#undef GH1_BDB_LAUNCH
  check_kernel(sp->ctx, "tet_bdb_kernel");
}

void tet_bdb_apply(gh1_op* op, int prec, const void* x, void* y, double* partial, unsigned int* counter,
                   double* energy, const int* skip) {
  if (op->tet_ntiles == 0) return;
  if (prec == GH1_F64)
    tet_bdb_launch<double>(op, op->bdb_per_sm[0], op->d_G64.p, op->d_tetB64.p, op->d_tetBw64.p, (const double*)x,
                           (double*)y, partial, counter, energy, skip);
  else if (op->tet_bdb_tc) {
    tet_bdb_tc_apply(op, (const float*)x, (float*)y, partial, counter, energy, skip);
  } else {
    GH1_CHECK(op->bdb_per_sm[1] > 0, GH1_ERR_ARG, "operator has no FP32 data (precision_mask)");
    tet_bdb_launch<float>(op, op->bdb_per_sm[1], op->d_G32.p, op->d_tetB32.p, op->d_tetBw32.p, (const float*)x,
                          (float*)y, partial, counter, energy, skip);
  }
}

// diagonal: per (element, local shape) the sum over the rule points of B^T Mh B
__global__ void tet_bdb_diag_kernel(int ne, int nloc, int nlocp, int ncb, int nq, const int* __restrict__ eldofs,
                                    const uint8_t* __restrict__ cls, const double* __restrict__ Mh, int per_point,
                                    const double* __restrict__ Tb, const double* __restrict__ Wb, double* diag) {
  const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= (int64_t)ne * nloc) return;
  const int e = (int)(id / nloc), i = (int)(id % nloc), c = cls[e];
  double s = 0;
  for (int q = 0; q < nq; q++) {
    const double* row = Tb + (((size_t)c * ncb + q / TET_QC) * nlocp + i) * 4 * TET_QC + q % TET_QC;
    const double bv[4] = {row[0], row[TET_QC], row[2 * TET_QC], row[3 * TET_QC]};
    const double* m = per_point ? Mh + ((size_t)e * nq + q) * 16 : Mh + (size_t)e * 16;
    const double w = per_point ? 1.0 : Wb[q];
    double t = 0;
    for (int r = 0; r < 4; r++)
      for (int k = 0; k < 4; k++) t += bv[r] * m[4 * r + k] * bv[k];
    s += w * t;
  }
  red_add(diag + eldofs[id], s);
}

void tet_bdb_diag(gh1_op* op, double* diag) {
  gh1_space* sp = op->sp;
  const int ne = sp->mesh->ne, nloc = sp->nloc, nlocp = (nloc + 15) / 16 * 16;
  const int64_t tot = (int64_t)ne * nloc;
  if (tot == 0) return;
  tet_bdb_diag_kernel<<<(unsigned)((tot + 127) / 128), 128, 0, sp->ctx->stream>>>(
      ne, nloc, nlocp, op->tet_ncb, sp->tet_nq_mass, sp->d_eldofs.p, sp->d_class.p, op->d_G64.p, op->bdb == 1 ? 1 : 0,
      op->d_tetB64.p, op->d_tetBw64.p, diag);
  check_kernel(sp->ctx, "tet_bdb_diag_kernel");
}

// element matrices of the generic form on tets, one thread per (element, i, j):
// K_ij = sum_q sum_rc B_r(i,q) Mh_rc(q) B_c(j,q) (B from the chunked value /
// reference-gradient table, Mh per point or w_q times the element's record),
// scattered into the CSR pattern as the other assemblies do
__global__ void tet_bdb_assemble_kernel(int ne, int nloc, int nlocp, int ncb, int nq, const int* __restrict__ eldofs,
                                        const uint8_t* __restrict__ cls, const double* __restrict__ Mh, int per_point,
                                        const double* __restrict__ Tb, const double* __restrict__ Wb,
                                        const int64_t* __restrict__ rowptr, const int32_t* __restrict__ colind,
                                        double* vals, int* bad) {
  const int64_t per = (int64_t)nloc * nloc;
  for (int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; id < (int64_t)ne * per;
       id += (int64_t)gridDim.x * blockDim.x) {
    const int e = (int)(id / per), ij = (int)(id % per), i = ij / nloc, j = ij % nloc, c = cls[e];
    double k = 0;
    for (int q = 0; q < nq; q++) {
      const double* ri = Tb + (((size_t)c * ncb + q / TET_QC) * nlocp + i) * 4 * TET_QC + q % TET_QC;
      const double* rj = Tb + (((size_t)c * ncb + q / TET_QC) * nlocp + j) * 4 * TET_QC + q % TET_QC;
      const double bi[4] = {ri[0], ri[TET_QC], ri[2 * TET_QC], ri[3 * TET_QC]};
      const double bj[4] = {rj[0], rj[TET_QC], rj[2 * TET_QC], rj[3 * TET_QC]};
      const double* m = per_point ? Mh + ((size_t)e * nq + q) * 16 : Mh + (size_t)e * 16;
      double t = 0;
      for (int r = 0; r < 4; r++)
        for (int cc = 0; cc < 4; cc++) t += bi[r] * m[4 * r + cc] * bj[cc];
      k += (per_point ? 1.0 : Wb[q]) * t;
    }
    const int row = eldofs[(size_t)e * nloc + i], col = eldofs[(size_t)e * nloc + j];
    int64_t lo = rowptr[row], hi = rowptr[row + 1] - 1, pos = -1;
    while (lo <= hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (colind[mid] == col) { pos = mid; break; }
      if (colind[mid] < col) lo = mid + 1; else hi = mid - 1;
    }
    if (pos < 0) { atomicExch(bad, 1); continue; }
    red_add(vals + pos, k);
  }
}

void tet_bdb_assemble(gh1_op* op, const int64_t* rowptr, const int32_t* colind, double* vals, int* bad) {
  gh1_space* sp = op->sp;
  const int ne = sp->mesh->ne, nloc = sp->nloc, nlocp = (nloc + 15) / 16 * 16;
  const int64_t tot = (int64_t)ne * nloc * nloc;
  if (tot == 0) return;
  const int grid = (int)std::min<int64_t>((tot + 255) / 256, (int64_t)sp->ctx->nsm * 32);
  tet_bdb_assemble_kernel<<<grid, 256, 0, sp->ctx->stream>>>(ne, nloc, nlocp, op->tet_ncb, sp->tet_nq_mass, sp->d_eldofs.p,
                                                             sp->d_class.p, op->d_G64.p, op->bdb == 1 ? 1 : 0,
                                                             op->d_tetB64.p, op->d_tetBw64.p, rowptr, colind, vals, bad);
  check_kernel(sp->ctx, "tet_bdb_assemble_kernel");
}

}  // namespace gh1
