// cg.cu -- Jacobi preconditioner, preconditioned CG (FP64 and FP32-inner with
// FP64 iterative refinement) and the adjoint gradient entry point.
//
// CG follows CGSolver._SolveImpl (python/krylovspace.py:263-291) step by step:
//   d = b - A x; w = P d; s = w; wdn = w.d; check sqrt|wdn|
//   loop: w = A s; wd = wdn; as_s = s.w; (as_s == 0 or wd == 0 -> stop)
//         alpha = wd/as_s; x += alpha s; d -= alpha w; w = P d; wdn = w.d;
//         check; beta = wdn/wd; s = w + beta s
// with CheckResidual (:129-219): iterations counts checks, converged when
// iterations >= maxiter or residual <= tol * first residual.
// GPU layout of one iteration: [apply: y = A s, s.y as the sum of element
// energies s_e^T A_e s_e] -> [update: alpha, d, w = P d, y = 0, w.d, |d|^2;
// the last block forms beta and the convergence flag] -> [direction: x +=
// alpha s, then s = w + beta s; the step the solve stops at adds its alpha s
// after the loop].  All scalars stay on the device.  One inner solve is ONE graph
// launch: a conditional WHILE node (the reference's device CG loop,
// ngscuda/cuda_krylov.cpp:19-203 with ngscuda/cuda_core.hpp:170-250) whose body
// holds `chunk` iterations and a one-thread kernel that sets the loop condition
// from the device-side convergence flag; the host synchronizes once per solve.
// Every device loop is bounded by maxit (the body count is capped as well);
// kernels after convergence return at their first instruction.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <vector>
#include "common.cuh"
#include "reduce.cuh"

namespace gh1 {

struct CGState {
  double wd, wdn, energy, alpha, beta, res0, stop, res, dd, bb;
  int it, maxit, done, status, rule;
  int xpend;  // the last step's x += alpha s is still due (the solve stopped before the direction kernel)
};

constexpr int RED_BLOCK = 256;

// 16-byte vector access for the bandwidth-bound CG updates
template <class T> struct V16;
template <> struct V16<float> {
  using type = float4;
  static constexpr int W = 4;
  static __device__ __forceinline__ void get(const type& v, float* o) { o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w; }
  static __device__ __forceinline__ type make(const float* o) { return make_float4(o[0], o[1], o[2], o[3]); }
};
template <> struct V16<double> {
  using type = double2;
  static constexpr int W = 2;
  static __device__ __forceinline__ void get(const type& v, double* o) { o[0] = v.x; o[1] = v.y; }
  static __device__ __forceinline__ type make(const double* o) { return make_double2(o[0], o[1]); }
};

template <class T>
__global__ void __launch_bounds__(RED_BLOCK) cg_init_kernel(int64_t n, const T* __restrict__ inv, T* __restrict__ d,
                                                            T* __restrict__ w, T* __restrict__ s, CGState* st, double tol,
                                                            double* hist, double* partial, unsigned int* counter) {
  T a0 = 0, a1 = 0;  // thread-local sums in the working precision
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    T di = d[i], iv = inv[i];
    T wi = iv * di;
    w[i] = wi;
    s[i] = wi;
    a0 += wi * di;
    if (iv != (T)0) a1 += di * di;
  }
  double v[2] = {(double)a0, (double)a1}, tot[2];
  if (grid_reduce<2>(v, partial, counter, tot) && threadIdx.x == 0) {
    st->wdn = tot[0];
    st->wd = tot[0];
    st->dd = tot[1];
    double r = st->rule == GH1_STOP_TRUE ? sqrt(tot[1]) : sqrt(fabs(tot[0]));
    st->res0 = r;
    st->res = r;
    st->stop = st->rule == GH1_STOP_TRUE ? tol * sqrt(st->bb) : tol * r;
    st->it = 1;
    if (hist) hist[0] = r;
    st->status = GH1_OK;
    st->done = (r <= st->stop || st->maxit <= 1 || tot[0] == 0.0) ? 1 : 0;
    if (st->done && !(r <= st->stop) && tot[0] != 0.0) st->status = GH1_MAXITER;
  }
}

// d -= alpha y; w = P d; y = 0 on [0, zero_end); partial sums of w.d and |d_free|^2.
// x += alpha s is left to cg_dir_kernel, which reads s anyway (one vector pass
// less per iteration); the entries of y from zero_end on are written, not
// accumulated, by the next apply (element-interior DOFs of a hex operator), so
// they need no clearing.
template <class T>
__global__ void __launch_bounds__(RED_BLOCK) cg_update_kernel(int64_t n, int64_t zero_end, const T* __restrict__ inv,
                                                              T* __restrict__ d, T* __restrict__ w, T* __restrict__ y,
                                                              CGState* st, double* hist, double* partial,
                                                              unsigned int* counter) {
  if (*(volatile int*)&st->done) return;
  const double wd = st->wd, en = st->energy;
  if (!(en > 0.0) || wd == 0.0 || !isfinite(en)) {
    // as_s == 0 or wd == 0 (krylovspace.py:276): stop; non-positive or NaN energy: breakdown
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      st->done = 1;
      st->status = (en == 0.0 || wd == 0.0) ? GH1_OK : GH1_BREAKDOWN;
    }
    return;
  }
  using VT = V16<T>;
  using V = typename VT::type;
  constexpr int W = VT::W;
  const T alpha = (T)(wd / en);
  T a0 = 0, a1 = 0;
  const int64_t nv = n / W, tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, nth = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = tid; i < nv; i += nth) {
    T yv[W], iv[W], dv[W], wv[W];
    VT::get(((const V*)y)[i], yv);
    VT::get(((const V*)inv)[i], iv);
    VT::get(((const V*)d)[i], dv);
#pragma unroll
    for (int c = 0; c < W; c++) {
      dv[c] -= alpha * yv[c];
      wv[c] = iv[c] * dv[c];
      a0 += wv[c] * dv[c];
      if (iv[c] != (T)0) a1 += dv[c] * dv[c];
    }
    ((V*)d)[i] = VT::make(dv);
    ((V*)w)[i] = VT::make(wv);
    if (i * W < zero_end) {
      const T z[W] = {};
      ((V*)y)[i] = VT::make(z);
    }
  }
  for (int64_t i = nv * W + tid; i < n; i += nth) {
    T yi = y[i], iv = inv[i];
    T di = d[i] - alpha * yi;
    d[i] = di;
    T wi = iv * di;
    w[i] = wi;
    if (i < zero_end) y[i] = (T)0;
    a0 += wi * di;
    if (iv != (T)0) a1 += di * di;
  }
  double v[2] = {(double)a0, (double)a1}, tot[2];
  if (grid_reduce<2>(v, partial, counter, tot) && threadIdx.x == 0) {
    double wdn = tot[0];
    double r = st->rule == GH1_STOP_TRUE ? sqrt(tot[1]) : sqrt(fabs(wdn));
    st->alpha = wd / en;
    st->dd = tot[1];
    st->res = r;
    if (hist) hist[st->it] = r;
    st->it += 1;
    st->beta = wdn / wd;
    st->wdn = wdn;
    st->wd = wdn;
    if (!isfinite(r)) { st->done = 1; st->status = GH1_BREAKDOWN; }
    else if (r <= st->stop) { st->done = 1; st->status = GH1_OK; }
    else if (st->it >= st->maxit) { st->done = 1; st->status = GH1_MAXITER; }
    st->xpend = st->done;  // stopped here: cg_dir_kernel will not run, cg_xfix_kernel adds alpha s
  }
}

// A preconditioner other than Jacobi (block Jacobi, low-order solve, their sum)
// runs as its own kernels between these: the state starts from w = C d and d,
// the update leaves w.d to cg_wd_kernel, which runs after w = C d.
template <class T>
__global__ void __launch_bounds__(RED_BLOCK) cg_init_gen_kernel(int64_t n, const uint8_t* __restrict__ fr,
                                                                const T* __restrict__ d, const T* __restrict__ w,
                                                                T* __restrict__ s, CGState* st, double tol, double* hist,
                                                                double* partial, unsigned int* counter) {
  T a0 = 0, a1 = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T di = d[i], wi = w[i];
    s[i] = wi;
    a0 += wi * di;
    if (fr[i]) a1 += di * di;
  }
  double v[2] = {(double)a0, (double)a1}, tot[2];
  if (grid_reduce<2>(v, partial, counter, tot) && threadIdx.x == 0) {
    st->wdn = tot[0];
    st->wd = tot[0];
    st->dd = tot[1];
    double r = st->rule == GH1_STOP_TRUE ? sqrt(tot[1]) : sqrt(fabs(tot[0]));
    st->res0 = r;
    st->res = r;
    st->stop = st->rule == GH1_STOP_TRUE ? tol * sqrt(st->bb) : tol * r;
    st->it = 1;
    if (hist) hist[0] = r;
    st->status = GH1_OK;
    st->done = (r <= st->stop || st->maxit <= 1 || tot[0] == 0.0) ? 1 : 0;
    if (st->done && !(r <= st->stop) && tot[0] != 0.0) st->status = GH1_MAXITER;
  }
}

// d -= alpha y; y = 0 on [0, zero_end); |d_free|^2 into st->dd
template <class T>
__global__ void __launch_bounds__(RED_BLOCK) cg_update_gen_kernel(int64_t n, int64_t zero_end, const uint8_t* __restrict__ fr,
                                                                  T* __restrict__ d, T* __restrict__ y, CGState* st,
                                                                  double* partial, unsigned int* counter) {
  if (*(volatile int*)&st->done) return;
  const double wd = st->wd, en = st->energy;
  if (!(en > 0.0) || wd == 0.0 || !isfinite(en)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      st->done = 1;
      st->status = (en == 0.0 || wd == 0.0) ? GH1_OK : GH1_BREAKDOWN;
    }
    return;
  }
  const T alpha = (T)(wd / en);
  T a1 = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T di = d[i] - alpha * y[i];
    d[i] = di;
    if (i < zero_end) y[i] = (T)0;
    if (fr[i]) a1 += di * di;
  }
  double v[1] = {(double)a1}, tot[1];
  if (grid_reduce<1>(v, partial, counter, tot) && threadIdx.x == 0) {
    st->alpha = wd / en;
    st->dd = tot[0];
  }
}

// w.d for the new w = C d, then the step's state as cg_update_kernel ends it
template <class T>
__global__ void __launch_bounds__(RED_BLOCK) cg_wd_kernel(int64_t n, const T* __restrict__ d, const T* __restrict__ w,
                                                          CGState* st, double* hist, double* partial,
                                                          unsigned int* counter) {
  if (*(volatile int*)&st->done) return;
  T a0 = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a0 += w[i] * d[i];
  double v[1] = {(double)a0}, tot[1];
  if (grid_reduce<1>(v, partial, counter, tot) && threadIdx.x == 0) {
    const double wdn = tot[0], wd = st->wd;
    const double r = st->rule == GH1_STOP_TRUE ? sqrt(st->dd) : sqrt(fabs(wdn));
    st->res = r;
    if (hist) hist[st->it] = r;
    st->it += 1;
    st->beta = wdn / wd;
    st->wdn = wdn;
    st->wd = wdn;
    if (!isfinite(r)) { st->done = 1; st->status = GH1_BREAKDOWN; }
    else if (r <= st->stop) { st->done = 1; st->status = GH1_OK; }
    else if (st->it >= st->maxit) { st->done = 1; st->status = GH1_MAXITER; }
    st->xpend = st->done;
  }
}

// tail of the WHILE body: count the body launches and keep looping while the
// solve is not done and the launch bound ctl[1] is not reached
__global__ void cg_loop_kernel(const CGState* st, int* ctl, cudaGraphConditionalHandle h) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    const int launches = ++ctl[0];
    cudaGraphSetConditional(h, (!*(volatile const int*)&st->done && launches < ctl[1]) ? 1u : 0u);
  }
}

// x += alpha s (the update step's x correction), then s = w + beta s.  With
// x == nullptr (a fresh start of a continued solve) only the direction update.
template <class T>
__global__ void __launch_bounds__(RED_BLOCK) cg_dir_kernel(int64_t n, const T* __restrict__ w, T* __restrict__ s,
                                                           T* __restrict__ x, const CGState* st) {
  if (*(volatile const int*)&st->done) return;
  using VT = V16<T>;
  using V = typename VT::type;
  constexpr int W = VT::W;
  const T beta = (T)st->beta, alpha = (T)st->alpha;
  const int64_t nv = n / W, tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, nth = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = tid; i < nv; i += nth) {
    T wv[W], sv[W];
    VT::get(((const V*)w)[i], wv);
    VT::get(((const V*)s)[i], sv);
    if (x) {
      T xv[W];
      VT::get(((const V*)x)[i], xv);
#pragma unroll
      for (int c = 0; c < W; c++) xv[c] += alpha * sv[c];
      ((V*)x)[i] = VT::make(xv);
    }
#pragma unroll
    for (int c = 0; c < W; c++) sv[c] = wv[c] + beta * sv[c];
    ((V*)s)[i] = VT::make(sv);
  }
  for (int64_t i = nv * W + tid; i < n; i += nth) {
    if (x) x[i] += alpha * s[i];
    s[i] = w[i] + beta * s[i];
  }
}

// after the loop: the x correction of the step the solve stopped at
template <class T>
__global__ void __launch_bounds__(RED_BLOCK) cg_xfix_kernel(int64_t n, const T* __restrict__ s, T* __restrict__ x,
                                                            const CGState* st) {
  if (!*(volatile const int*)&st->xpend) return;
  const T alpha = (T)st->alpha;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] += alpha * s[i];
}

// r = b - y (FP64), |r_free|^2 and |b_free|^2 ; free = mask
__global__ void __launch_bounds__(RED_BLOCK) residual_kernel(int64_t n, const double* __restrict__ b, const double* __restrict__ y,
                                                             const uint8_t* __restrict__ freedof, double* __restrict__ r,
                                                             double* out2, double* partial, unsigned int* counter) {
  double v[2] = {0, 0}, tot[2];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double ri = b[i] - y[i];
    if (r) r[i] = ri;
    if (freedof[i]) { v[0] += ri * ri; v[1] += b[i] * b[i]; }
  }
  if (grid_reduce<2>(v, partial, counter, tot) && threadIdx.x == 0) { out2[0] = tot[0]; out2[1] = tot[1]; }
}

template <class TA, class TB>
__global__ void axpby_kernel(int64_t n, double a, const TA* x, double b, TB* y) {  // x may alias y
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (TB)(a * (double)x[i] + (b == 0.0 ? 0.0 : b * (double)y[i]));
}

__global__ void scale_to_f32_kernel(int64_t n, const double* __restrict__ r, const double* __restrict__ norm2,
                                    float* __restrict__ d32) {
  const double sc = norm2[0] > 0 ? 1.0 / sqrt(norm2[0]) : 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    d32[i] = (float)(r[i] * sc);
}

__global__ void correct_kernel(int64_t n, const float* __restrict__ c32, const double* __restrict__ norm2, double* __restrict__ x) {
  const double sc = sqrt(norm2[0]);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] += sc * (double)c32[i];
}

__global__ void jacobi_invert_kernel(int64_t n, const double* diag, const uint8_t* freedof, double* inv64, float* inv32) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double v = (freedof[i] && diag[i] != 0.0) ? 1.0 / diag[i] : 0.0;
    inv64[i] = v;
    inv32[i] = (float)v;
  }
}

template <class T>
__global__ void jacobi_apply_kernel(int64_t n, double s, const T* __restrict__ inv, const T* __restrict__ x, T* __restrict__ y,
                                    int acc) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    T v = (T)s * inv[i] * x[i];
    y[i] = acc ? y[i] + v : v;
  }
}

void jacobi_invert(gh1_ctx* ctx, int64_t n, const double* diag, const uint8_t* freedof, double* inv64, float* inv32) {
  jacobi_invert_kernel<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(n, diag, freedof, inv64, inv32);
  check_kernel(ctx, "jacobi_invert_kernel");
}

void jacobi_apply(gh1_ctx* ctx, int64_t n, double s, const double* inv64, const float* inv32, const void* x, void* y, int prec,
                  int acc) {
  if (prec == GH1_F64)
    jacobi_apply_kernel<double><<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(n, s, inv64, (const double*)x, (double*)y, acc);
  else
    jacobi_apply_kernel<float><<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(n, s, inv32, (const float*)x, (float*)y, acc);
  check_kernel(ctx, "jacobi_apply_kernel");
}

void vec_axpby(gh1_ctx* ctx, int64_t n, double a, const void* x, double b, void* y, int prec) {
  if (prec == GH1_F64)
    axpby_kernel<double, double><<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(n, a, (const double*)x, b, (double*)y);
  else
    axpby_kernel<float, float><<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(n, a, (const float*)x, b, (float*)y);
  check_kernel(ctx, "axpby_kernel");
}

// ---------------------------------------------------------------------------
namespace {

struct Scratch {
  // reduction scratch: partial sums [2 * grid] per reduction site + counters
  DBuf<double> partial;
  DBuf<unsigned int> counters;
  DBuf<CGState> state;
  DBuf<double> hist;
  DBuf<double> norm2;  // [2]
};

int red_grid(gh1_ctx* ctx, int64_t n) { return grid_for(ctx, n, RED_BLOCK, 8); }

// operator apply with the device energy sink (y must be zero on entry)
void op_apply_energy(gh1_op* op, const void* x, void* y, int prec, double* partial, unsigned int* counter, double* energy,
                     const int* skip) {
  if (op->kind == GH1_OP_MATFREE) {
    matfree_apply_ex(op, x, y, prec, partial, counter, energy, skip);
  } else {
    throw Error(GH1_ERR_UNSUPPORTED, "internal: CSR energy path");
  }
}

// s^T y for CSR operators (the apply has no element energies)
template <class T>
__global__ void __launch_bounds__(RED_BLOCK) dot_energy_kernel(int64_t n, const T* __restrict__ a, const T* __restrict__ b,
                                                               double* out, double* partial, unsigned int* counter,
                                                               const int* skip) {
  if (*(volatile const int*)skip) return;
  double v[1] = {0}, tot[1];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v[0] += (double)a[i] * (double)b[i];
  if (grid_reduce<1>(v, partial, counter, tot) && threadIdx.x == 0) *out = tot[0];
}

// One PCG solve in precision T on vectors already on the device.
// d holds the initial residual on entry; x the initial guess.
template <class T>
struct PCG {
  gh1_op* op;
  gh1_ctx* ctx;
  int64_t n;
  const T* inv;
  T *x, *d, *w, *s, *y;
  int prec;
  CGState* st;
  double* partial;       // [4 * grid_max]
  unsigned int* counters;  // [4]
  double* hist;
  int chunk;
  int* ctl;              // [2]: body launches so far, bound on body launches
  int64_t zero_end;      // the apply writes (does not accumulate) y from here on
  gh1_pre* gpre = nullptr;       // a preconditioner other than Jacobi (inv unused then)
  const uint8_t* fr = nullptr;   // its free-DOF mask
  int applies = 0;

  void launch_iteration(cudaStream_t cs) {
    int g = red_grid(ctx, n);
    if (op->kind == GH1_OP_MATFREE) {
      op_apply_energy(op, s, y, prec, partial + 2 * ctx->nsm * 64, counters + 1, &st->energy, &st->done);
    } else {  // CSR or block operator: s^T A s by a separate reduction
      op_apply_any(op, s, y, prec, &st->done);
      dot_energy_kernel<T><<<g, RED_BLOCK, 0, cs>>>(n, s, y, &st->energy, partial + 2 * ctx->nsm * 64, counters + 1, &st->done);
      check_kernel(ctx, "dot_energy_kernel");
    }
    if (gpre) {
      cg_update_gen_kernel<T><<<g, RED_BLOCK, 0, cs>>>(n, zero_end, fr, d, y, st, partial, counters + 2);
      check_kernel(ctx, "cg_update_gen_kernel");
      pre_apply_any(gpre, 1.0, d, w, prec, 0);
      cg_wd_kernel<T><<<g, RED_BLOCK, 0, cs>>>(n, d, w, st, hist, partial, counters + 4);
      check_kernel(ctx, "cg_wd_kernel");
    } else {
      cg_update_kernel<T><<<g, RED_BLOCK, 0, cs>>>(n, zero_end, inv, d, w, y, st, hist, partial, counters + 2);
      check_kernel(ctx, "cg_update_kernel");
    }
    cg_dir_kernel<T><<<g, RED_BLOCK, 0, cs>>>(n, w, s, x, st);
    check_kernel(ctx, "cg_dir_kernel");
  }

  // returns iterations (checks) and fills host state
  CGState run(double tol, int maxit, int rule, double bb, cudaStream_t cs, cudaGraphExec_t* cache_exec, int* cache_chunk) {
    CGState h{};
    h.maxit = maxit;
    h.rule = rule;
    h.bb = bb;
    GH1_CUDA(cudaMemcpyAsync(st, &h, sizeof(CGState), cudaMemcpyHostToDevice, cs));
    GH1_CUDA(cudaMemsetAsync(y, 0, n * sizeof(T), cs));
    int g = red_grid(ctx, n);
    if (gpre) {
      pre_prepare(gpre);
      pre_apply_any(gpre, 1.0, d, w, prec, 0);
      cg_init_gen_kernel<T><<<g, RED_BLOCK, 0, cs>>>(n, fr, d, w, s, st, tol, hist, partial, counters + 0);
      check_kernel(ctx, "cg_init_gen_kernel");
    } else {
      cg_init_kernel<T><<<g, RED_BLOCK, 0, cs>>>(n, inv, d, w, s, st, tol, hist, partial, counters + 0);
      check_kernel(ctx, "cg_init_kernel");
    }
    CGState* hs = (CGState*)ctx->h_pinned;
    // one WHILE node whose body is `chunk` iterations plus the loop condition,
    // built once per solve shape
    cudaGraphExec_t exec = *cache_exec;
    if (!exec || *cache_chunk != chunk) {
      if (exec) cudaGraphExecDestroy(exec);
      *cache_exec = nullptr;
      op_prepare_any(op, prec);
      cudaGraph_t graph;
      GH1_CUDA(cudaGraphCreate(&graph, 0));
      try {
        cudaGraphConditionalHandle handle;
        GH1_CUDA(cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault));
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = handle;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t loop;
        GH1_CUDA(cudaGraphAddNode(&loop, graph, nullptr, nullptr, 0, &cp));
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        GH1_CUDA(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        try {
          for (int k = 0; k < chunk; k++) launch_iteration(cs);
          cg_loop_kernel<<<1, 32, 0, cs>>>(st, ctl, handle);
          check_kernel(ctx, "cg_loop_kernel");
        } catch (...) {
          cudaGraph_t dummy;
          cudaStreamEndCapture(cs, &dummy);
          throw;
        }
        GH1_CUDA(cudaStreamEndCapture(cs, &body));
        GH1_CUDA(cudaGraphInstantiate(&exec, graph, 0));
      } catch (...) {
        cudaGraphDestroy(graph);
        throw;
      }
      cudaGraphDestroy(graph);
      *cache_exec = exec;
      *cache_chunk = chunk;
    }
    const int hctl[2] = {0, (maxit + chunk - 1) / chunk + 2};
    GH1_CUDA(cudaMemcpyAsync(ctl, hctl, sizeof(hctl), cudaMemcpyHostToDevice, cs));
    GH1_CUDA(cudaGraphLaunch(exec, cs));
    cg_xfix_kernel<T><<<red_grid(ctx, n), RED_BLOCK, 0, cs>>>(n, s, x, st);
    check_kernel(ctx, "cg_xfix_kernel");
    GH1_CUDA(cudaMemcpyAsync(hs, st, sizeof(CGState), cudaMemcpyDeviceToHost, cs));
    GH1_CUDA(cudaStreamSynchronize(cs));
    CGState out = *hs;
    applies = out.it - 1;
    return out;
  }
};

struct Work {
  DBuf<double> d64, w64, s64, y64, r64;
  DBuf<float> x32, d32, w32, s32, y32;
};

}  // namespace

// per-operator cached graphs would outlive changes of pointers; graphs are
// rebuilt per solve (capture + instantiate cost a few hundred microseconds).
int cg_solve(gh1_op* op, gh1_pre* pre, const double* b, double* x, const gh1_cg_opts* o, gh1_cg_result* r) {
  gh1_ctx* ctx = op->ctx;
  const int64_t n = op->nrows;
  cudaStream_t user = ctx->stream;
  cudaStream_t cs;
  GH1_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaEvent_t ev;
  GH1_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  GH1_CUDA(cudaEventRecord(ev, user));
  GH1_CUDA(cudaStreamWaitEvent(cs, ev, 0));
  ctx->stream = cs;  // kernels launched by the operator go to the solver stream
  int status = GH1_OK;
  std::vector<cudaGraphExec_t> execs;
  try {
    std::memset(r, 0, sizeof(*r));
    const int grid_max = ctx->nsm * 64;
    DBuf<double> partial((size_t)4 * grid_max + 8);
    DBuf<unsigned int> counters(8);
    counters.zero(cs);
    DBuf<CGState> st(1);
    DBuf<double> hist((size_t)o->maxit + 2);
    DBuf<double> norm2(2);
    DBuf<int> ctl(2);
    DBuf<uint8_t> ones;
    const uint8_t* freemask = pre ? pre->d_free.p : nullptr;
    if (!freemask) {
      ones.alloc(n);
      GH1_CUDA(cudaMemsetAsync(ones.p, 1, n, cs));
      freemask = ones.p;
    }
    DBuf<double> inv_ident;
    gh1_pre* gpre = (pre && pre->kind != 0) ? pre : nullptr;  // a preconditioner run as its own kernels
    GH1_CHECK(!pre || pre->n == n, GH1_ERR_ARG, "the preconditioner's size differs from the operator's");
    const double* inv64 = (pre && !gpre) ? pre->d_inv64.p : nullptr;
    if (!inv64) {
      std::vector<double> one(n, 1.0);
      inv_ident.upload(one, cs);
      inv64 = inv_ident.p;
    }
    int chunk = o->check_every > 0 ? o->check_every : 8;
    // every hex matrix-free apply writes the element-interior DOFs (from
    // first_cell on) instead of adding to them, so the CG update clears y below it only
    const int64_t zero_end = (op->kind == GH1_OP_MATFREE && op->sp && op->sp->et == 8) ? op->sp->first_cell : n;
    auto bnorm2 = [&](const double* y, double* rr) {  // |b - y|^2, |b|^2 on free DOFs
      int g = red_grid(ctx, n);
      residual_kernel<<<g, RED_BLOCK, 0, cs>>>(n, b, y, freemask, rr, norm2.p, partial.p, counters.p + 3);
      check_kernel(ctx, "residual_kernel");
      double h[2];
      GH1_CUDA(cudaMemcpyAsync(h, norm2.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, cs));
      GH1_CUDA(cudaStreamSynchronize(cs));
      return std::pair<double, double>(h[0], h[1]);
    };
    Work W;
    W.d64.alloc(n); W.w64.alloc(n); W.s64.alloc(n); W.y64.alloc(n);
    auto apply64 = [&](const double* in, double* out) {
      GH1_CUDA(cudaMemsetAsync(out, 0, n * sizeof(double), cs));
      op_prepare_any(op, GH1_F64);
      op_apply_any(op, in, out, GH1_F64, nullptr);
      r->applies64++;
    };
    if (o->initialize) GH1_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), cs));
    // d = b - A x  (|b_free| as the reference scale of the true-residual rule)
    std::pair<double, double> rb;
    if (o->initialize) {
      GH1_CUDA(cudaMemcpyAsync(W.d64.p, b, n * sizeof(double), cudaMemcpyDeviceToDevice, cs));
      GH1_CUDA(cudaMemsetAsync(W.y64.p, 0, n * sizeof(double), cs));
      rb = bnorm2(W.y64.p, nullptr);
    } else {
      apply64(x, W.y64.p);
      rb = bnorm2(W.y64.p, W.d64.p);
    }
    const double bb = rb.second;
    cudaGraphExec_t exec64 = nullptr, exec32 = nullptr;
    int ch64 = 0, ch32 = 0;
    double final_rr = 0.0;  // |b - A x|^2 on free DOFs for the returned x
    if (o->mode == GH1_CG_FP64) {
      PCG<double> P{op, ctx, n, inv64, x, W.d64.p, W.w64.p, W.s64.p, W.y64.p, GH1_F64, st.p, partial.p, counters.p, hist.p, chunk,
                    ctl.p, zero_end, gpre, freemask};
      GH1_CUDA(cudaMemsetAsync(W.y64.p, 0, n * sizeof(double), cs));
      CGState res = P.run(o->tol, o->maxit, o->stop_rule, bb, cs, &exec64, &ch64);
      execs.push_back(exec64);
      r->iterations = res.it;
      r->applies64 += P.applies;
      r->first_res = res.res0;
      r->final_res = res.res;
      status = res.status;
      if (o->res_hist && res.it > 0)
        GH1_CUDA(cudaMemcpyAsync(o->res_hist, hist.p, sizeof(double) * std::min(res.it, o->maxit + 1), cudaMemcpyDeviceToHost, cs));
    } else {
      // FP32 inner PCG inside FP64 iterative refinement
      W.x32.alloc(n); W.d32.alloc(n); W.w32.alloc(n); W.s32.alloc(n); W.y32.alloc(n); W.r64.alloc(n);
      GH1_CHECK(op->kind == GH1_OP_CSR || (op->prec_mask & 2), GH1_ERR_UNSUPPORTED,
                "mixed precision needs an operator set up with FP32 data (precision mask bit 1)");
      op_prepare_any(op, GH1_F32);
      const double inner_tol = o->inner_tol > 0 ? o->inner_tol : 1e-4;
      const int max_outer = o->max_outer > 0 ? o->max_outer : 30;
      const double target = o->tol * std::sqrt(bb);
      double rr = o->initialize ? bb : rb.first;
      std::vector<double> hh;
      int total_inner = 0;
      status = GH1_MAXITER;
      r->first_res = std::sqrt(rr);
      for (int outer = 0; outer <= max_outer; outer++) {
        if (outer > 0) {
          apply64(x, W.y64.p);
          auto q = bnorm2(W.y64.p, W.r64.p);
          rr = q.first;
        } else if (o->initialize) {
          GH1_CUDA(cudaMemcpyAsync(W.r64.p, b, n * sizeof(double), cudaMemcpyDeviceToDevice, cs));
          double h2[2] = {rr, bb};
          GH1_CUDA(cudaMemcpyAsync(norm2.p, h2, sizeof(h2), cudaMemcpyHostToDevice, cs));
        } else {
          GH1_CUDA(cudaMemcpyAsync(W.r64.p, W.d64.p, n * sizeof(double), cudaMemcpyDeviceToDevice, cs));
          double h2[2] = {rr, bb};
          GH1_CUDA(cudaMemcpyAsync(norm2.p, h2, sizeof(h2), cudaMemcpyHostToDevice, cs));
        }
        hh.push_back(std::sqrt(rr));
        final_rr = rr;
        r->final_res = std::sqrt(rr);
        r->outer = outer;
        if (std::sqrt(rr) <= target) { status = GH1_OK; break; }
        if (outer == max_outer || total_inner >= o->maxit) break;
        // inner: A c = r / |r|  in FP32, c0 = 0.  The last refinement step only
        // needs the reduction that is still missing; it aims two decades below
        // the target, because with the hierarchical basis at p >= 3 (cond(A) up
        // to ~1e9) the error of x is a few hundred times the relative residual:
        // the returned x then carries the error of a residual ~tol/100, not tol.
        const double missing = target / std::sqrt(rr);
        const double tol_k = std::min(0.5, std::max(inner_tol, 0.01 * missing));
        scale_to_f32_kernel<<<grid_for(ctx, n, 256), 256, 0, cs>>>(n, W.r64.p, norm2.p, W.d32.p);
        check_kernel(ctx, "scale_to_f32_kernel");
        GH1_CUDA(cudaMemsetAsync(W.x32.p, 0, n * sizeof(float), cs));
        PCG<float> P{op, ctx, n, gpre ? nullptr : pre->d_inv32.p, W.x32.p, W.d32.p, W.w32.p, W.s32.p, W.y32.p, GH1_F32,
                     st.p, partial.p, counters.p, nullptr, chunk, ctl.p, zero_end, gpre, freemask};
        CGState res = P.run(tol_k, std::max(2, o->maxit - total_inner), GH1_STOP_PRECOND, 0.0, cs, &exec32, &ch32);
        total_inner += res.it;
        r->applies32 += P.applies;
        if (res.status == GH1_BREAKDOWN) { status = GH1_BREAKDOWN; break; }
        correct_kernel<<<grid_for(ctx, n, 256), 256, 0, cs>>>(n, W.x32.p, norm2.p, x);
        check_kernel(ctx, "correct_kernel");
      }
      execs.push_back(exec32);
      r->iterations = total_inner;
      if (o->res_hist) for (size_t k = 0; k < hh.size() && (int)k <= o->maxit; k++) o->res_hist[k] = hh[k];
    }
    // true relative residual at exit.  The mixed loop leaves only through its
    // check of |b - A x|^2 for the current x (x changes only in correct_kernel,
    // which the next check always follows), so that residual is reused there.
    if (o->mode == GH1_CG_FP64) {
      apply64(x, W.y64.p);
      final_rr = bnorm2(W.y64.p, nullptr).first;
    }
    r->true_relres = bb > 0 ? std::sqrt(final_rr / bb) : std::sqrt(final_rr);
    r->status = status;
    GH1_CUDA(cudaStreamSynchronize(cs));
    op_check_err(op);
  } catch (...) {
    for (auto e : execs) if (e) cudaGraphExecDestroy(e);
    cudaStreamSynchronize(cs);
    ctx->stream = user;
    cudaEventDestroy(ev);
    cudaStreamDestroy(cs);
    throw;
  }
  for (auto e : execs) if (e) cudaGraphExecDestroy(e);
  ctx->stream = user;
  GH1_CUDA(cudaEventRecord(ev, cs));
  GH1_CUDA(cudaStreamWaitEvent(user, ev, 0));
  cudaEventDestroy(ev);
  cudaStreamDestroy(cs);
  return status;
}

}  // namespace gh1

// ---------------------------------------------------------------------------
// adjoint gradient
extern "C" int gh1_adjoint_grad(gh1_form* form, const double* f, const double* u_target, double tol, double* u, double* lam,
                                double* dJdkappa, double* J) {
  if (!form || !f || !u_target || !u || !lam || !dJdkappa || !J) return GH1_ERR_ARG;
  gh1_ctx* ctx = form->sp->ctx;
  try {
    using namespace gh1;
    gh1_space* sp = form->sp;
    GH1_CHECK(!form->has_K6, GH1_ERR_UNSUPPORTED, "gh1_adjoint_grad: dJ/dkappa needs a scalar kappa (a tensor is set)");
    GH1_CHECK(form->bdb_mode == 0, GH1_ERR_UNSUPPORTED, "gh1_adjoint_grad: dJ/dkappa needs a scalar kappa (a B^T D B form is set)");
    const int64_t n = sp->ndof;
    cudaStream_t s = ctx->stream;
    // the operator with FP64 and FP32 data, kept on the form between calls; the
    // metrics follow the current kappa, the Jacobi diagonal is rebuilt per call
    int rc = GH1_OK;
    if (!form->adj_A) {
      rc = gh1_matfree_create(form, 3, &form->adj_A);
      if (rc) return rc;
      // the form owns this operator (it is deleted with the form), so the
      // operator must not keep the form alive in turn
      form->adj_A->form_ref = false;
      form->refs--;
    }
    gh1_op* A = form->adj_A;
    if (A->form_version != form->version) matfree_setup(A);
    gh1_pre* P = nullptr;
    rc = gh1_jacobi_create(A, nullptr, 0, &P);
    if (rc) return rc;
    // forward and adjoint solves: FP32 inner CG inside FP64 refinement, FP64 true residual
    gh1_cg_opts o{};
    o.tol = tol; o.maxit = 100000; o.mode = GH1_CG_MIXED; o.stop_rule = GH1_STOP_TRUE; o.initialize = 1;
    gh1_cg_result res{};
    rc = gh1_cg(A, P, f, u, &o, &res);
    if (rc != GH1_OK) { gh1_pre_free(P); return rc; }
    // unit-mass operator for J and the adjoint right-hand side (built once)
    if (!form->adj_M) {
      gh1_form* mf = new gh1_form();
      form->adj_mass = mf;
      mf->sp = sp;
      std::vector<double> zeros(sp->mesh->ne, 0.0), ones(sp->mesh->ne, 1.0);
      mf->d_kappa.upload(zeros, s);
      mf->d_mu.upload(ones, s);
      mf->has_mu = true;
      gh1_op* M = new gh1_op();
      form->adj_M = M;
      M->ctx = ctx; M->kind = GH1_OP_MATFREE; M->form = mf; M->sp = sp; M->nrows = n; M->prec_mask = 1;
      matfree_setup(M);
      GH1_CUDA(cudaStreamSynchronize(s));  // the host staging vectors go out of scope
    }
    gh1_op* Mop = form->adj_M;
    DBuf<double> e(n), Me(n), tmp(1);
    axpby_kernel<double, double><<<grid_for(ctx, n, 256), 256, 0, s>>>(n, 1.0, u, 0.0, e.p);
    axpby_kernel<double, double><<<grid_for(ctx, n, 256), 256, 0, s>>>(n, -1.0, u_target, 1.0, e.p);
    GH1_CUDA(cudaMemsetAsync(Me.p, 0, n * sizeof(double), s));
    DBuf<double> partial((size_t)ctx->nsm * 64 + 8);
    DBuf<unsigned int> cnt(1);
    cnt.zero(s);
    DBuf<double> en(1);
    matfree_apply_ex(Mop, e.p, Me.p, GH1_F64, partial.p, cnt.p, en.p, nullptr);
    double hJ = 0;
    GH1_CUDA(cudaMemcpyAsync(&hJ, en.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    GH1_CUDA(cudaStreamSynchronize(s));
    *J = 0.5 * hJ;
    rc = gh1_cg(A, P, Me.p, lam, &o, &res);
    if (rc != GH1_OK) { gh1_pre_free(P); return rc; }
    elem_grad_dot_with(A, u, lam, dJdkappa);
    axpby_kernel<double, double><<<grid_for(ctx, sp->mesh->ne, 256), 256, 0, s>>>(sp->mesh->ne, -1.0, dJdkappa, 0.0, dJdkappa);
    GH1_CUDA(cudaStreamSynchronize(s));
    gh1_pre_free(P);
    return GH1_OK;
  } catch (const gh1::Error& e) {
    ctx->err = e.what();
    return e.code;
  } catch (const std::exception& e) {
    ctx->err = e.what();
    return GH1_ERR_ARG;
  }
}
