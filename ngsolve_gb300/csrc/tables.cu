// tables.cu -- integration rules and GPU evaluation of shapes / reference
// gradients at the integration points.
//
// Replaces the per-element shape recomputation of T_CalcElementMatrixAdd /
// ApplyElementMatrix (fem/symbolicintegrator.cpp:1548-1830, :2959-3040, via
// CalcMappedDShape fem/tscalarfe_impl.hpp:759-890) by tables computed once:
//  - hex: the 1D factor tables B[q][a] = psi_a(x_q), D[q][a] = psi_a'(x_q)
//    at the Gauss points of SelectIntegrationRule(ET_HEX, 2p)
//    (fem/intrule.cpp:3118-3132, :3234-3263): q = p+1 points per direction;
//  - tet: shape values and reference gradients per orientation class (the
//    24 rank permutations of the element's vertex numbers; the shapes depend
//    on vertex numbers only through comparisons, fem/elementtopology.hpp:
//    1208-1236) at the rule of order 2p-2 (bilinear, :1433-1455) and of
//    order 2p (mass / linear form, :1109), plus the six reference stiffness
//    blocks S_ab = sum_q w_q d_a phi_i d_b phi_j and the reference mass block.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>
#include "common.cuh"
#include "basis.cuh"
#include "tet_rules.inc"
#include "deform.cuh"

namespace gh1 {

// Gauss-Legendre on (0,1), Newton on P_n (ComputeGaussRule, fem/intrule.cpp:700-740)
void gauss01(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0);
  w.assign(n, 0);
  int m = (n + 1) / 2;
  for (int i = 1; i <= m; i++) {
    double z = std::cos(M_PI * (i - 0.25) / (n + 0.5)), z1, pp = 1, p1, p2, p3;
    for (int it = 0; it < 100; it++) {
      p1 = 1; p2 = 0;
      for (int j = 1; j <= n; j++) { p3 = p2; p2 = p1; p1 = ((2 * j - 1) * z * p2 - (j - 1) * p3) / j; }
      pp = n * (z * p1 - p2) / (z * z - 1);
      z1 = z;
      z = z1 - p1 / pp;
      if (std::fabs(z - z1) < 1e-15) break;
    }
    p1 = 1; p2 = 0;
    for (int j = 1; j <= n; j++) { p3 = p2; p2 = p1; p1 = ((2 * j - 1) * z * p2 - (j - 1) * p3) / j; }
    pp = n * (z * p1 - p2) / (z * z - 1);
    x[i - 1] = 0.5 * (1 - z);
    x[n - i] = 0.5 * (1 + z);
    w[i - 1] = w[n - i] = 1.0 / ((1 - z * z) * pp * pp);
  }
}

// tet rule of a given order: tabulated symmetric rules up to degree 6 (the point
// counts of fem/intrule.cpp:2596-2812), a 46-point symmetric rule for degrees 7
// and 8 (gen_tet_rules.py; the reference's collapsed rule there has 216 points),
// collapsed tensor Gauss rule above.
void tet_rule(int order, std::vector<double>& r /* x,y,z,w per point */) {
  r.clear();
  auto add = [&](const double (*t)[4], int n) { for (int i = 0; i < n; i++) for (int k = 0; k < 4; k++) r.push_back(t[i][k]); };
  if (order <= 1) add(TET_RULE_D1, 1);
  else if (order == 2) add(TET_RULE_D2, 4);
  else if (order <= 5) add(TET_RULE_D5, 14);
  else if (order == 6) add(TET_RULE_D6, 24);
  else if (order <= 8) add(TET_RULE_D8, 46);
  else {
    int n = order / 2 + 2;
    std::vector<double> g, gw;
    gauss01(n, g, gw);
    for (int k = 0; k < n; k++)
      for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
          double xx = g[i], yy = g[j], zz = g[k];
          r.push_back(xx);
          r.push_back(yy * (1 - xx));
          r.push_back(zz * (1 - xx) * (1 - yy));
          r.push_back(gw[i] * gw[j] * gw[k] * (1 - xx) * (1 - xx) * (1 - yy));
        }
  }
}

__device__ void class_ranks(int c, int* vn) {
  // inverse of the lexicographic permutation index used on the host
  int avail[4] = {0, 1, 2, 3}, navail = 4;
  const int fact[4] = {6, 2, 1, 1};
  for (int i = 0; i < 4; i++) {
    int k = c / fact[i];
    c %= fact[i];
    vn[i] = avail[k];
    for (int j = k; j < navail - 1; j++) avail[j] = avail[j + 1];
    navail--;
  }
}

__global__ void hex_1d_tables(int p, int nq, const double* gx, double* B64, double* D64, float* B32, float* D32) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  const int n = p + 1;
  Dual3 psi[MAX_HEX_ORDER + 1];
  hex_psi<Dual3>(p, Dual3(gx[q], 1.0, 0.0, 0.0), psi);
  for (int a = 0; a < n; a++) {
    B64[q * n + a] = psi[a].v;
    D64[q * n + a] = psi[a].dx;
    B32[q * n + a] = (float)psi[a].v;
    D32[q * n + a] = (float)psi[a].dx;
  }
}

// one thread per (class, point): values + reference gradients
__global__ void tet_class_tables(int p, int nloc, int nq, const double* rule, double* tab64, float* tab32,
                                 int values_only, Dual3* scratch) {
  int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= N_TET_CLASSES * nq) return;
  int c = id / nq, q = id % nq;
  int vn[4];
  class_ranks(c, vn);
  Dual3* sh = scratch + (size_t)id * nloc;  // global scratch keeps local memory small
  tet_shapes<Dual3>(p, vn, Dual3(rule[4 * q], 1, 0, 0), Dual3(rule[4 * q + 1], 0, 1, 0), Dual3(rule[4 * q + 2], 0, 0, 1), sh);
  for (int i = 0; i < nloc; i++) {
    size_t o = ((size_t)c * nq + q) * nloc + i;
    if (values_only) {
      tab64[o] = sh[i].v;
    } else {
      tab64[4 * o + 0] = sh[i].v;
      tab64[4 * o + 1] = sh[i].dx;
      tab64[4 * o + 2] = sh[i].dy;
      tab64[4 * o + 3] = sh[i].dz;
      if (tab32) {
        tab32[4 * o + 0] = (float)sh[i].v;
        tab32[4 * o + 1] = (float)sh[i].dx;
        tab32[4 * o + 2] = (float)sh[i].dy;
        tab32[4 * o + 3] = (float)sh[i].dz;
      }
    }
  }
}

// S[c][blk][i][j]: blk 0..2 = S_aa, 3 = S_01+S_10, 4 = S_02+S_20, 5 = S_12+S_21, 6 = mass
__global__ void tet_ref_blocks(int nloc, int nq, const double* rule, const double* tab, int nqm, const double* rulem,
                               const double* tabm, double* S) {
  int c = blockIdx.y, blk = blockIdx.z;
  for (int ij = blockIdx.x * blockDim.x + threadIdx.x; ij < nloc * nloc; ij += gridDim.x * blockDim.x) {
    int i = ij / nloc, j = ij % nloc;
    double s = 0;
    if (blk < 6) {
      const int A[6] = {0, 1, 2, 0, 0, 1}, Bc[6] = {0, 1, 2, 1, 2, 2};
      int a = A[blk] + 1, b = Bc[blk] + 1;
      for (int q = 0; q < nq; q++) {
        const double* ti = tab + 4 * (((size_t)c * nq + q) * nloc + i);
        const double* tj = tab + 4 * (((size_t)c * nq + q) * nloc + j);
        double v = ti[a] * tj[b];
        if (blk >= 3) v += ti[b] * tj[a];
        s += rule[4 * q + 3] * v;
      }
    } else {
      for (int q = 0; q < nqm; q++)
        s += rulem[4 * q + 3] * tabm[((size_t)c * nqm + q) * nloc + i] * tabm[((size_t)c * nqm + q) * nloc + j];
    }
    S[(((size_t)c * 7 + blk) * nloc + i) * nloc + j] = s;
  }
}

void build_tables(gh1_space* sp) {
  cudaStream_t s = sp->ctx->stream;
  const int p = sp->p;
  if (sp->et == 8) {
    sp->nq1 = (2 * p) / 2 + 1;
    gauss01(sp->nq1, sp->gx, sp->gw);
    sp->d_gx.upload(sp->gx, s);
    sp->d_gw.upload(sp->gw, s);
    const int n = p + 1, nq = sp->nq1;
    sp->d_B64.alloc(nq * n); sp->d_D64.alloc(nq * n);
    sp->d_B32.alloc(nq * n); sp->d_D32.alloc(nq * n);
    hex_1d_tables<<<1, 32, 0, s>>>(p, nq, sp->d_gx.p, sp->d_B64.p, sp->d_D64.p, sp->d_B32.p, sp->d_D32.p);
    check_kernel(sp->ctx, "hex_1d_tables");
  } else {
    std::vector<double> r, rm;
    tet_rule(2 * p - 2 > 0 ? 2 * p - 2 : 0, r);
    tet_rule(2 * p, rm);
    sp->tet_nq = (int)r.size() / 4;
    sp->tet_nq_mass = (int)rm.size() / 4;
    sp->d_tq.upload(r, s);
    sp->d_tqm.upload(rm, s);
    const int nloc = sp->nloc, nq = sp->tet_nq, nqm = sp->tet_nq_mass;
    sp->d_tab64.alloc((size_t)N_TET_CLASSES * nq * nloc * 4);
    sp->d_tab32.alloc((size_t)N_TET_CLASSES * nq * nloc * 4);
    sp->d_tabm64.alloc((size_t)N_TET_CLASSES * nqm * nloc);
    int tot = N_TET_CLASSES * nq;
    int totm = N_TET_CLASSES * nqm;
    DBuf<Dual3> scratch((size_t)std::max(tot, totm) * nloc);
    tet_class_tables<<<(tot + 63) / 64, 64, 0, s>>>(p, nloc, nq, sp->d_tq.p, sp->d_tab64.p, sp->d_tab32.p, 0, scratch.p);
    check_kernel(sp->ctx, "tet_class_tables");
    tet_class_tables<<<(totm + 63) / 64, 64, 0, s>>>(p, nloc, nqm, sp->d_tqm.p, sp->d_tabm64.p, nullptr, 1, scratch.p);
    check_kernel(sp->ctx, "tet_class_tables(mass)");
    sp->d_S.alloc((size_t)N_TET_CLASSES * 7 * nloc * nloc);
    dim3 g((nloc * nloc + 127) / 128, N_TET_CLASSES, 7);
    tet_ref_blocks<<<g, 128, 0, s>>>(nloc, nq, sp->d_tq.p, sp->d_tab64.p, nqm, sp->d_tqm.p, sp->d_tabm64.p, sp->d_S.p);
    check_kernel(sp->ctx, "tet_ref_blocks");
    GH1_CUDA(cudaStreamSynchronize(s));  // scratch is released on return
  }
}

// values and reference gradients at the degree-2p rule (the generic B^T D B
// rule of tets; the mass table holds values only)
void tet_mass_rule_tables(gh1_space* sp, DBuf<double>& t64, DBuf<float>& t32) {
  cudaStream_t s = sp->ctx->stream;
  const int nloc = sp->nloc, nqm = sp->tet_nq_mass, tot = N_TET_CLASSES * nqm;
  t64.alloc((size_t)tot * nloc * 4);
  t32.alloc((size_t)tot * nloc * 4);
  DBuf<Dual3> scratch((size_t)tot * nloc);
  tet_class_tables<<<(tot + 63) / 64, 64, 0, s>>>(sp->p, nloc, nqm, sp->d_tqm.p, t64.p, t32.p, 0, scratch.p);
  check_kernel(sp->ctx, "tet_class_tables(2p)");
  GH1_CUDA(cudaStreamSynchronize(s));  // scratch is released on return
}

// the rule of the generic B^T D B form: hex tensor Gauss with p+1 points per
// direction (point q = (i*n + j)*n + k at (x_i, x_j, x_k)), tet the degree-2p rule
int space_rule_size(const gh1_space* sp) { return sp->et == 8 ? sp->nq1 * sp->nq1 * sp->nq1 : sp->tet_nq_mass; }

// physical coordinates of the rule points: hex trilinear map, tet affine map
// x = v3 + sum_j (v_j - v3) xi_j
__global__ void qpoints_kernel(int et, int ne, int nq, int nq1, const double* __restrict__ X, const int* __restrict__ el,
                               const double* __restrict__ gx, const double* __restrict__ tqm, double* xyz, DeformView dv) {
  const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= (int64_t)ne * nq) return;
  const int e = (int)(id / nq), q = (int)(id % nq);
  double out[3] = {0, 0, 0}, Jd[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (et == 8) {
    const double x = gx[q / (nq1 * nq1)], y = gx[(q / nq1) % nq1], z = gx[q % nq1];
    deform_add(dv, e, x, y, z, Jd, out);  // the displacement (Jd unused)
    const double lam[8] = {(1 - x) * (1 - y) * (1 - z), x * (1 - y) * (1 - z), x * y * (1 - z), (1 - x) * y * (1 - z),
                           (1 - x) * (1 - y) * z,       x * (1 - y) * z,       x * y * z,       (1 - x) * y * z};
    for (int a = 0; a < 8; a++) {
      const double* pa = X + 3 * (size_t)el[(size_t)e * 8 + a];
      for (int k = 0; k < 3; k++) out[k] += lam[a] * pa[k];
    }
  } else {
    const double* p3 = X + 3 * (size_t)el[(size_t)e * 4 + 3];
    deform_add(dv, e, tqm[4 * q], tqm[4 * q + 1], tqm[4 * q + 2], Jd, out);
    for (int k = 0; k < 3; k++) out[k] += p3[k];
    for (int j = 0; j < 3; j++) {
      const double* pj = X + 3 * (size_t)el[(size_t)e * 4 + j];
      for (int k = 0; k < 3; k++) out[k] += (pj[k] - p3[k]) * tqm[4 * q + j];
    }
  }
  for (int k = 0; k < 3; k++) xyz[id * 3 + k] = out[k];
}

void space_qpoints(gh1_space* sp, double* ref, double* xyz) {
  cudaStream_t s = sp->ctx->stream;
  const int nq = space_rule_size(sp), ne = sp->mesh->ne;
  if (ref) {
    if (sp->et == 8) {
      const int n = sp->nq1;
      for (int q = 0; q < nq; q++) {
        const int i = q / (n * n), j = (q / n) % n, k = q % n;
        ref[4 * q] = sp->gx[i];
        ref[4 * q + 1] = sp->gx[j];
        ref[4 * q + 2] = sp->gx[k];
        ref[4 * q + 3] = sp->gw[i] * sp->gw[j] * sp->gw[k];
      }
    } else {
      GH1_CUDA(cudaMemcpyAsync(ref, sp->d_tqm.p, (size_t)nq * 4 * sizeof(double), cudaMemcpyDeviceToHost, s));
      GH1_CUDA(cudaStreamSynchronize(s));
    }
  }
  if (xyz && ne > 0) {
    const int64_t tot = (int64_t)ne * nq;
    qpoints_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(sp->et, ne, nq, sp->nq1, sp->mesh->d_X.p, sp->mesh->d_el.p,
                                                                 sp->d_gx.p, sp->d_tqm.p, xyz, deform_view(sp->mesh));
    check_kernel(sp->ctx, "qpoints_kernel");
  }
}

// ---- shape evaluation at arbitrary points (gh1_shape_eval) -------------------
__global__ void shape_eval_kernel(int et, int p, int nloc, int v0, int v1, int v2, int v3, int v4, int v5, int v6, int v7,
                                  int npts, const double* pts, double* val, double* grad, Dual3* scratch) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= npts) return;
  int vn[8] = {v0, v1, v2, v3, v4, v5, v6, v7};
  Dual3* sh = scratch + (size_t)q * nloc;
  Dual3 X(pts[3 * q], 1, 0, 0), Y(pts[3 * q + 1], 0, 1, 0), Z(pts[3 * q + 2], 0, 0, 1);
  if (et == 4) tet_shapes<Dual3>(p, vn, X, Y, Z, sh);
  else hex_shapes<Dual3>(p, vn, X, Y, Z, sh);
  for (int i = 0; i < nloc; i++) {
    val[(size_t)q * nloc + i] = sh[i].v;
    grad[((size_t)q * nloc + i) * 3 + 0] = sh[i].dx;
    grad[((size_t)q * nloc + i) * 3 + 1] = sh[i].dy;
    grad[((size_t)q * nloc + i) * 3 + 2] = sh[i].dz;
  }
}

void shape_eval_gpu(gh1_ctx* ctx, int et, int p, const int32_t* vnums, int npts, const double* pts, double* val,
                    double* grad) {
  int nloc = et == 4 ? (p + 1) * (p + 2) * (p + 3) / 6 : (p + 1) * (p + 1) * (p + 1);
  int v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = 0; i < et; i++) v[i] = vnums[i];
  cudaStream_t s = ctx->stream;
  DBuf<double> dp(3 * (size_t)npts), dv((size_t)npts * nloc), dg((size_t)npts * nloc * 3);
  DBuf<Dual3> scratch((size_t)npts * nloc);
  dp.upload(pts, 3 * (size_t)npts, s);
  shape_eval_kernel<<<(npts + 31) / 32, 32, 0, s>>>(et, p, nloc, v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], npts,
                                                     dp.p, dv.p, dg.p, scratch.p);
  check_kernel(ctx, "shape_eval_kernel");
  GH1_CUDA(cudaMemcpyAsync(val, dv.p, dv.bytes(), cudaMemcpyDeviceToHost, s));
  GH1_CUDA(cudaMemcpyAsync(grad, dg.p, dg.bytes(), cudaMemcpyDeviceToHost, s));
  GH1_CUDA(cudaStreamSynchronize(s));
}

// ---- shape evaluation into caller-owned device memory, no allocation -----------
// For callers that cannot let the library allocate device memory (their own
// fixed pool, or a loop that must not stall on cudaMalloc / cudaFree): the
// per-(point, shape) scratch of shape_eval_kernel lives in this fixed module
// array, GH1_SHAPE_NOALLOC_MAX_ENTRIES Dual3 values (8 MiB), which every device
// that loads the library holds until the process exits.  The array name is only
// a host-side handle; kernels get its device address from cudaGetSymbolAddress.
static __device__ __align__(256) double shape_noalloc_scratch[4 * (size_t)GH1_SHAPE_NOALLOC_MAX_ENTRIES];
static_assert(sizeof(Dual3) == 4 * sizeof(double), "scratch entry is one Dual3");

constexpr int kNoallocMaxDevices = 64;
static std::mutex shape_noalloc_mu;
static void* shape_noalloc_addr[kNoallocMaxDevices] = {};

// the scratch array's address on `device` (current), looked up on first use
static Dual3* shape_noalloc_scratch_on(int device) {
  GH1_CHECK(device >= 0 && device < kNoallocMaxDevices, GH1_ERR_UNSUPPORTED,
            "gh1_shape_eval_noalloc: device index beyond the supported 64");
  std::lock_guard<std::mutex> lock(shape_noalloc_mu);
  if (!shape_noalloc_addr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, shape_noalloc_scratch);
    if (e != cudaSuccess)
      throw Error(GH1_ERR_CUDA, std::string("gh1_shape_eval_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    shape_noalloc_addr[device] = p;
  }
  return (Dual3*)shape_noalloc_addr[device];
}

// true if the device can address p as memory of `device` (device or managed)
static bool device_pointer_on(const void* p, int device) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeManaged) return true;
  return a.type == cudaMemoryTypeDevice && a.device == device;
}

static void shape_eval_noalloc(gh1_ctx* ctx, int et, int p, const int32_t* vnums, int npts, const double* pts,
                               double* val, double* grad) {
  GH1_CHECK(et == 4 || et == 8, GH1_ERR_UNSUPPORTED, "element type must be 4 or 8");
  GH1_CHECK(p >= 1 && p <= (et == 4 ? MAX_TET_ORDER : MAX_HEX_ORDER), GH1_ERR_UNSUPPORTED, "order out of range");
  const int nloc = et == 4 ? (p + 1) * (p + 2) * (p + 3) / 6 : (p + 1) * (p + 1) * (p + 1);
  const int64_t entries = (int64_t)npts * nloc;
  GH1_CHECK(entries <= GH1_SHAPE_NOALLOC_MAX_ENTRIES, GH1_ERR_ARG,
            "gh1_shape_eval_noalloc: npts * nloc = " + std::to_string(entries) + " exceeds the fixed scratch of " +
                std::to_string(GH1_SHAPE_NOALLOC_MAX_ENTRIES) + " entries; split the points into smaller calls");
  // the scratch lookup needs the context's device current; restore the caller's
  int prev = -1;
  GH1_CUDA(cudaGetDevice(&prev));
  if (prev != ctx->device) GH1_CUDA(cudaSetDevice(ctx->device));
  struct Restore {
    int dev, prev;
    ~Restore() {
      if (prev >= 0 && prev != dev) cudaSetDevice(prev);
    }
  } restore{ctx->device, prev};
  GH1_CHECK(device_pointer_on(pts, ctx->device) && device_pointer_on(val, ctx->device) &&
                device_pointer_on(grad, ctx->device),
            GH1_ERR_ARG, "gh1_shape_eval_noalloc: pts, val and grad must be device memory of the context's device");
  Dual3* scratch = shape_noalloc_scratch_on(ctx->device);
  int v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = 0; i < et; i++) v[i] = vnums[i];
  shape_eval_kernel<<<(npts + 31) / 32, 32, 0, ctx->stream>>>(et, p, nloc, v[0], v[1], v[2], v[3], v[4], v[5], v[6],
                                                               v[7], npts, pts, val, grad, scratch);
  check_kernel(ctx, "shape_eval_kernel (no-allocation entry)");
}

}  // namespace gh1

extern "C" int gh1_shape_eval_noalloc(gh1_ctx* ctx, int et, int order, const int32_t* vnums, int npts,
                                      const double* pts, double* val, double* grad) {
  if (!ctx) return GH1_ERR_ARG;
  if (!vnums || !pts || !val || !grad || npts <= 0) {
    ctx->err = "gh1_shape_eval_noalloc: null pointer or npts <= 0";
    return GH1_ERR_ARG;
  }
  try {
    gh1::shape_eval_noalloc(ctx, et, order, vnums, npts, pts, val, grad);
    return GH1_OK;
  } catch (const gh1::Error& e) {
    ctx->err = e.what();
    return e.code;
  } catch (const std::exception& e) {
    ctx->err = e.what();
    return GH1_ERR_ARG;
  }
}
