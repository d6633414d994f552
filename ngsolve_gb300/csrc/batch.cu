// batch.cu -- batched solves: many independent problems, up to 16 right-hand
// sides each, advanced together by ONE launch of one CUDA graph.
//
// Every (problem, rhs) pair runs the mixed-precision solver of cg.cu as a small
// state machine in device memory:
//   NEED    : FP64 residual r = b - A x (multi-rhs FP64 apply), converged? ->
//             DONE, else start an inner solve on r/|r|
//   INNER   : FP32 Jacobi-PCG iterations (CGSolver._SolveImpl steps,
//             python/krylovspace.py:263-291) on the multi-rhs FP32 apply
//   CORRECT : x += |r| c, back to NEED
// One graph round per problem = [FP64 apply, residual, begin] + K x [FP32 apply,
// update, direction] + [correct]; problems are independent graph branches.
// Kernels whose rhs is in another phase return at once, so the round is the
// body of a conditional WHILE node that repeats on the device until every pair
// is DONE (a one-thread kernel at the end of the body sets the condition from a
// device counter; the host waits once, after the launch).
// The multi-rhs apply stages each element's G tile once for all active rhs; its
// FP32 form (two right-hand sides per lane or one) is timed per problem at
// gh1_batch_create.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#include "common.cuh"
#include "reduce.cuh"

namespace gh1 {

enum { PH_NEED = 0, PH_INNER = 1, PH_CORRECT = 2, PH_DONE = 3 };

struct RState {
  double wd, beta, res0, stop, rnorm, bnorm2, inner_tol_k;
  int it, total, outer, status;
};

constexpr int BB = 256;

// phase NEED: y64 <- b - y64 ; |r_free|^2, |b_free|^2 ; decide DONE or start
__global__ void __launch_bounds__(BB) b_residual(int64_t n, const double* __restrict__ b, double* __restrict__ y64,
                                                 const uint8_t* __restrict__ freedof, int* phase, RState* st, double tol,
                                                 double inner_tol, int max_outer, double* partial, unsigned int* cnt,
                                                 int* done_total) {
  const int r = blockIdx.y;
  if (phase[r] != PH_NEED) return;
  const double* br = b + (size_t)r * n;
  double* yr = y64 + (size_t)r * n;
  double v[2] = {0, 0}, tot[2];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double ri = br[i] - yr[i];
    yr[i] = ri;
    if (freedof[i]) { v[0] += ri * ri; v[1] += br[i] * br[i]; }
  }
  if (grid_reduce<2>(v, partial + (size_t)r * 2 * gridDim.x, cnt + r, tot) && threadIdx.x == 0) {
    RState& s = st[r];
    if (s.outer == 0) s.bnorm2 = tot[1];
    const double target = tol * sqrt(s.bnorm2), rn = sqrt(tot[0]);
    s.rnorm = rn;
    if (rn <= target || s.outer >= max_outer || !isfinite(rn)) {
      s.status = rn <= target ? GH1_OK : (isfinite(rn) ? GH1_MAXITER : GH1_BREAKDOWN);
      phase[r] = PH_DONE;
      atomicAdd(done_total, 1);
    } else {
      s.inner_tol_k = fmin(0.5, fmax(inner_tol, 0.1 * target / rn));
    }
  }
}

// phase NEED (not done): d = r/|r|, c = 0, y32 = 0, w = P d, s = w ; start the inner CG
__global__ void __launch_bounds__(BB) b_begin(int64_t n, const double* __restrict__ y64, const float* __restrict__ inv,
                                              float* __restrict__ x32, float* __restrict__ d32, float* __restrict__ w32,
                                              float* __restrict__ s32, float* __restrict__ y32, int* phase, RState* st,
                                              double* partial, unsigned int* cnt) {
  const int r = blockIdx.y;
  if (phase[r] != PH_NEED) return;
  const size_t o = (size_t)r * n;
  const double sc = 1.0 / st[r].rnorm;
  float a0 = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float di = (float)(y64[o + i] * sc), iv = inv[i];
    const float wi = iv * di;
    d32[o + i] = di;
    w32[o + i] = wi;
    s32[o + i] = wi;
    x32[o + i] = 0.f;
    y32[o + i] = 0.f;
    a0 += wi * di;
  }
  double v[1] = {(double)a0}, tot[1];
  if (grid_reduce<1>(v, partial + (size_t)r * 2 * gridDim.x, cnt + r, tot) && threadIdx.x == 0) {
    RState& s = st[r];
    s.wd = tot[0];
    s.res0 = sqrt(fabs(tot[0]));
    s.stop = s.inner_tol_k * s.res0;
    s.it = 1;
    phase[r] = tot[0] > 0 ? PH_INNER : PH_CORRECT;
  }
}

// phase INNER: alpha = wd / s^T A s ; c += alpha s ; d -= alpha y ; w = P d ; y = 0
__global__ void __launch_bounds__(BB) b_update(int64_t n, const float* __restrict__ inv, float* __restrict__ x32,
                                               float* __restrict__ d32, float* __restrict__ w32, const float* __restrict__ s32,
                                               float* __restrict__ y32, int* phase, RState* st, const double* energy,
                                               int inner_maxit, double* partial, unsigned int* cnt) {
  const int r = blockIdx.y;
  if (phase[r] != PH_INNER) return;
  const double wd = st[r].wd, en = energy[r];
  if (!(en > 0.0) || !isfinite(en)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) phase[r] = PH_CORRECT;
    return;
  }
  const size_t o = (size_t)r * n;
  const float alpha = (float)(wd / en);
  float a0 = 0;
  const int64_t nv = n / 4;
  const bool aligned = (o % 4) == 0;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, nth = (int64_t)gridDim.x * blockDim.x;
  int64_t i0 = 0;
  if (aligned) {
    for (int64_t i = tid; i < nv; i += nth) {
      float4 s = ((const float4*)(s32 + o))[i], y = ((const float4*)(y32 + o))[i], iv = ((const float4*)inv)[i];
      float4 x = ((float4*)(x32 + o))[i], d = ((float4*)(d32 + o))[i], w;
      x.x += alpha * s.x; x.y += alpha * s.y; x.z += alpha * s.z; x.w += alpha * s.w;
      d.x -= alpha * y.x; d.y -= alpha * y.y; d.z -= alpha * y.z; d.w -= alpha * y.w;
      w.x = iv.x * d.x; w.y = iv.y * d.y; w.z = iv.z * d.z; w.w = iv.w * d.w;
      a0 += w.x * d.x + w.y * d.y + w.z * d.z + w.w * d.w;
      ((float4*)(x32 + o))[i] = x;
      ((float4*)(d32 + o))[i] = d;
      ((float4*)(w32 + o))[i] = w;
      ((float4*)(y32 + o))[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    i0 = nv * 4;
  }
  for (int64_t i = i0 + tid; i < n; i += nth) {
    x32[o + i] += alpha * s32[o + i];
    const float di = d32[o + i] - alpha * y32[o + i];
    d32[o + i] = di;
    const float wi = inv[i] * di;
    w32[o + i] = wi;
    y32[o + i] = 0.f;
    a0 += wi * di;
  }
  double v[1] = {(double)a0}, tot[1];
  if (grid_reduce<1>(v, partial + (size_t)r * 2 * gridDim.x, cnt + r, tot) && threadIdx.x == 0) {
    RState& s = st[r];
    const double wdn = tot[0], res = sqrt(fabs(wdn));
    s.beta = wdn / wd;
    s.wd = wdn;
    s.it += 1;
    s.total += 1;
    if (!(res > s.stop) || s.it >= inner_maxit || !isfinite(res)) phase[r] = PH_CORRECT;
  }
}

// phase INNER: s = w + beta s
__global__ void __launch_bounds__(BB) b_dir(int64_t n, const float* __restrict__ w32, float* __restrict__ s32,
                                            const int* phase, const RState* st) {
  const int r = blockIdx.y;
  if (phase[r] != PH_INNER) return;
  const size_t o = (size_t)r * n;
  const float beta = (float)st[r].beta;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s32[o + i] = w32[o + i] + beta * s32[o + i];
}

// tail of the WHILE body: count the rounds and loop while a (problem, rhs)
// pair is not done and the round bound ctl[1] is not reached
__global__ void b_loop_kernel(const int* done_total, int total, int* ctl, cudaGraphConditionalHandle h) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    const int rounds = ++ctl[0];
    cudaGraphSetConditional(h, (*(volatile const int*)done_total < total && rounds < ctl[1]) ? 1u : 0u);
  }
}

// phase CORRECT: x += |r| c ; y64 = 0 ; then back to NEED (last block)
__global__ void __launch_bounds__(BB) b_correct(int64_t n, const float* __restrict__ x32, double* __restrict__ x,
                                                double* __restrict__ y64, int* phase, RState* st, double* partial,
                                                unsigned int* cnt) {
  const int r = blockIdx.y;
  if (phase[r] != PH_CORRECT) return;
  const size_t o = (size_t)r * n;
  const double sc = st[r].rnorm;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[o + i] += sc * (double)x32[o + i];
    y64[o + i] = 0.0;
  }
  double v[1] = {0}, tot[1];
  if (grid_reduce<1>(v, partial + (size_t)r * 2 * gridDim.x, cnt + r, tot) && threadIdx.x == 0) {
    st[r].outer += 1;
    phase[r] = PH_NEED;
  }
}

}  // namespace gh1

using namespace gh1;

struct gh1_batch {
  gh1_ctx* ctx = nullptr;
  struct Prob {
    gh1_form* form = nullptr;
    gh1_op* op = nullptr;
    gh1_pre* pre = nullptr;
    int R = 0;
    int64_t n = 0;
    DBuf<float> x32, d32, w32, s32, y32;
    DBuf<double> y64, energy, partial;
    DBuf<RState> st;
    DBuf<int> phase;
    DBuf<unsigned int> cnt;  // [6][R]: residual, begin, update, correct, apply
    int gx = 1, gapply = 1;
  };
  std::vector<Prob*> probs;
  DBuf<int> done_total;
  DBuf<int> ctl;  // [2]: rounds so far, bound on rounds
  ~gh1_batch() {
    for (auto* p : probs) {
      if (p->pre) gh1_pre_free(p->pre);
      if (p->op) gh1_op_free(p->op);
      delete p;
    }
  }
};

namespace {
// The FP32 multi-rhs apply of one problem, two right-hand sides per lane or
// one, timed on the problem's own operator with all its rhs active; the faster
// form is kept on the operator (the batched solves' tile choice).
void tune_multi_pair(gh1_ctx* ctx, gh1_batch::Prob* P) {
  gh1_op* op = P->op;
  cudaStream_t s = ctx->stream;
  const int R = P->R;
  std::vector<int> inner(R, PH_INNER);
  GH1_CUDA(cudaMemcpyAsync(P->phase.p, inner.data(), R * sizeof(int), cudaMemcpyHostToDevice, s));
  P->s32.zero(s);
  P->y32.zero(s);
  cudaEvent_t a, b;
  GH1_CUDA(cudaEventCreate(&a));
  GH1_CUDA(cudaEventCreate(&b));
  float best = 1e30f;
  int choice = 1;
  for (int pr = 1; pr >= 0; pr--) {
    op->multi_pair = pr;
    unsigned int* c = P->cnt.p + 4 * R;
    matfree_apply_multi(op, R, P->phase.p, PH_INNER, P->s32.p, P->y32.p, GH1_F32, P->partial.p, c, P->energy.p, false);
    GH1_CUDA(cudaEventRecord(a, s));
    for (int k = 0; k < 3; k++)
      matfree_apply_multi(op, R, P->phase.p, PH_INNER, P->s32.p, P->y32.p, GH1_F32, P->partial.p, c, P->energy.p, false);
    GH1_CUDA(cudaEventRecord(b, s));
    GH1_CUDA(cudaEventSynchronize(b));
    float ms = 0;
    GH1_CUDA(cudaEventElapsedTime(&ms, a, b));
    if (ms < best) { best = ms; choice = pr; }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  op->multi_pair = choice;
  GH1_CUDA(cudaMemsetAsync(P->phase.p, 0, R * sizeof(int), s));  // PH_NEED
}

template <class F>
int bguard(gh1_ctx* ctx, F&& f) {
  try {
    f();
    return GH1_OK;
  } catch (const Error& e) {
    ctx->err = e.what();
    return e.code;
  } catch (const std::exception& e) {
    ctx->err = e.what();
    return GH1_ERR_ARG;
  }
}
}  // namespace

extern "C" int gh1_batch_create(gh1_ctx* ctx, int nprob, gh1_form* const* forms, const int* nrhs, gh1_batch** out) {
  if (!ctx || !forms || !nrhs || !out || nprob <= 0) return GH1_ERR_ARG;
  return bguard(ctx, [&] {
    gh1_batch* B = new gh1_batch();
    B->ctx = ctx;
    try {
      for (int i = 0; i < nprob; i++) {
        GH1_CHECK(forms[i] && forms[i]->sp->ctx == ctx, GH1_ERR_ARG, "batch: form of another context");
        GH1_CHECK(forms[i]->sp->et == 8, GH1_ERR_UNSUPPORTED, "batch: hex meshes only");
        GH1_CHECK(forms[i]->bdb_mode == 0, GH1_ERR_UNSUPPORTED, "batch: Laplace / mass forms only (a B^T D B form is set)");
        GH1_CHECK(nrhs[i] >= 1 && nrhs[i] <= 16, GH1_ERR_UNSUPPORTED, "batch: 1..16 right-hand sides per problem");
        auto* P = new gh1_batch::Prob();
        B->probs.push_back(P);
        P->form = forms[i];
        P->R = nrhs[i];
        int rc = gh1_matfree_create(forms[i], 3, &P->op);
        if (rc) throw Error(rc, ctx->err);
        rc = gh1_jacobi_create(P->op, nullptr, GH1_MEM_HOST, &P->pre);
        if (rc) throw Error(rc, ctx->err);
        const int64_t n = P->op->nrows, R = P->R;
        P->n = n;
        P->x32.alloc(R * n); P->d32.alloc(R * n); P->w32.alloc(R * n); P->s32.alloc(R * n); P->y32.alloc(R * n);
        P->y64.alloc(R * n);
        P->energy.alloc(16);
        P->st.alloc(R);
        P->phase.alloc(R);
        P->cnt.alloc(6 * R);
        P->cnt.zero(ctx->stream);
        P->gx = (int)std::max<int64_t>(1, std::min<int64_t>((n + BB - 1) / BB, std::max<int64_t>(1, ctx->nsm * 16 / R)));
        // grids of the FP64 apply and of both FP32 forms (one or two rhs per lane)
        int g32[2];
        for (int pr = 0; pr < 2; pr++) {
          P->op->multi_pair = pr;
          g32[pr] = matfree_apply_multi(P->op, P->R, P->phase.p, PH_INNER, nullptr, nullptr, GH1_F32, nullptr, nullptr,
                                        nullptr, true);
        }
        P->gapply = std::max({matfree_apply_multi(P->op, P->R, P->phase.p, PH_NEED, nullptr, nullptr, GH1_F64, nullptr,
                                                  nullptr, nullptr, true),
                              g32[0], g32[1]});
        P->partial.alloc((size_t)R * std::max(2 * P->gx, P->gapply) + 8);
        tune_multi_pair(ctx, P);
      }
      B->done_total.alloc(1);
      B->ctl.alloc(2);
      GH1_CUDA(cudaStreamSynchronize(ctx->stream));
    } catch (...) {
      delete B;
      throw;
    }
    *out = B;
  });
}

extern "C" int gh1_batch_free(gh1_batch* B) {
  delete B;
  return GH1_OK;
}

extern "C" int gh1_batch_solve(gh1_batch* B, const double* const* rhs, double* const* x, const gh1_cg_opts* o,
                               gh1_cg_result* res) {
  if (!B || !rhs || !x || !o || !res) return GH1_ERR_ARG;
  gh1_ctx* ctx = B->ctx;
  int status = GH1_OK;
  int rc = bguard(ctx, [&] {
    const int np = (int)B->probs.size();
    const double inner_tol = o->inner_tol > 0 ? o->inner_tol : 1e-4;
    const int max_outer = o->max_outer > 0 ? o->max_outer : 30;
    const int K = o->check_every > 0 ? o->check_every : 16;
    const int inner_maxit = std::max(2, o->maxit);
    cudaStream_t user = ctx->stream;
    cudaStream_t cs;
    GH1_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    const int ns = std::min(np, 16);
    std::vector<cudaStream_t> pool(ns);
    std::vector<cudaEvent_t> ev(ns + 1);
    for (int i = 0; i < ns; i++) GH1_CUDA(cudaStreamCreateWithFlags(&pool[i], cudaStreamNonBlocking));
    for (auto& e : ev) GH1_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool capturing = false;
    auto cleanup = [&] {
      if (capturing) {  // a failure inside the capture: end it before the stream goes
        cudaGraph_t dummy;
        cudaStreamEndCapture(cs, &dummy);
      }
      ctx->stream = user;
      if (exec) cudaGraphExecDestroy(exec);
      if (graph) cudaGraphDestroy(graph);
      for (auto& e : ev) cudaEventDestroy(e);
      for (auto& s : pool) cudaStreamDestroy(s);
      cudaStreamDestroy(cs);
    };
    try {
      GH1_CUDA(cudaEventRecord(ev[ns], user));
      GH1_CUDA(cudaStreamWaitEvent(cs, ev[ns], 0));
      int total = 0;
      for (int i = 0; i < np; i++) {
        auto* P = B->probs[i];
        total += P->R;
        std::vector<RState> h(P->R);
        std::memset(h.data(), 0, h.size() * sizeof(RState));
        GH1_CUDA(cudaMemcpyAsync(P->st.p, h.data(), h.size() * sizeof(RState), cudaMemcpyHostToDevice, cs));
        GH1_CUDA(cudaMemsetAsync(P->phase.p, 0, P->R * sizeof(int), cs));  // PH_NEED
        GH1_CUDA(cudaMemsetAsync(P->y64.p, 0, P->y64.bytes(), cs));
        if (o->initialize) GH1_CUDA(cudaMemsetAsync(x[i], 0, (size_t)P->R * P->n * sizeof(double), cs));
      }
      GH1_CUDA(cudaMemsetAsync(B->done_total.p, 0, sizeof(int), cs));
      const int max_rounds = (inner_maxit + K - 1) / K * (max_outer + 1) + max_outer + 4;
      // ---- one WHILE node; its body is one round of every problem, as parallel
      // branches, and the loop condition -------------------------------------
      GH1_CUDA(cudaGraphCreate(&graph, 0));
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
      capturing = true;
      GH1_CUDA(cudaEventRecord(ev[ns], cs));
      for (int s = 0; s < ns; s++) GH1_CUDA(cudaStreamWaitEvent(pool[s], ev[ns], 0));
      for (int i = 0; i < np; i++) {
        auto* P = B->probs[i];
        cudaStream_t st = pool[i % ns];
        ctx->stream = st;
        const int64_t n = P->n;
        const int R = P->R;
        dim3 gv(P->gx, R);
        unsigned int* c = P->cnt.p;
        matfree_apply_multi(P->op, R, P->phase.p, PH_NEED, x[i], P->y64.p, GH1_F64, P->partial.p, c + 4 * R,
                            P->energy.p, false);
        b_residual<<<gv, BB, 0, st>>>(n, rhs[i], P->y64.p, P->pre->d_free.p, P->phase.p, P->st.p, o->tol, inner_tol,
                                      max_outer, P->partial.p, c, B->done_total.p);
        check_kernel(ctx, "b_residual");
        b_begin<<<gv, BB, 0, st>>>(n, P->y64.p, P->pre->d_inv32.p, P->x32.p, P->d32.p, P->w32.p, P->s32.p, P->y32.p,
                                   P->phase.p, P->st.p, P->partial.p, c + R);
        check_kernel(ctx, "b_begin");
        for (int k = 0; k < K; k++) {
          matfree_apply_multi(P->op, R, P->phase.p, PH_INNER, P->s32.p, P->y32.p, GH1_F32, P->partial.p, c + 4 * R,
                              P->energy.p, false);
          b_update<<<gv, BB, 0, st>>>(n, P->pre->d_inv32.p, P->x32.p, P->d32.p, P->w32.p, P->s32.p, P->y32.p, P->phase.p,
                                      P->st.p, P->energy.p, inner_maxit, P->partial.p, c + 2 * R);
          check_kernel(ctx, "b_update");
          b_dir<<<gv, BB, 0, st>>>(n, P->w32.p, P->s32.p, P->phase.p, P->st.p);
          check_kernel(ctx, "b_dir");
        }
        b_correct<<<gv, BB, 0, st>>>(n, P->x32.p, x[i], P->y64.p, P->phase.p, P->st.p, P->partial.p, c + 3 * R);
        check_kernel(ctx, "b_correct");
      }
      for (int s = 0; s < ns; s++) {
        GH1_CUDA(cudaEventRecord(ev[s], pool[s]));
        GH1_CUDA(cudaStreamWaitEvent(cs, ev[s], 0));
      }
      ctx->stream = cs;
      b_loop_kernel<<<1, 32, 0, cs>>>(B->done_total.p, total, B->ctl.p, handle);
      check_kernel(ctx, "b_loop_kernel");
      capturing = false;
      GH1_CUDA(cudaStreamEndCapture(cs, &body));
      GH1_CUDA(cudaGraphInstantiate(&exec, graph, 0));
      // ---- one launch: rounds run on the device until every (problem, rhs) is
      // done or the round bound is reached --------------------------------------
      const int hctl[2] = {0, max_rounds};
      GH1_CUDA(cudaMemcpyAsync(B->ctl.p, hctl, sizeof(hctl), cudaMemcpyHostToDevice, cs));
      GH1_CUDA(cudaGraphLaunch(exec, cs));
      GH1_CUDA(cudaStreamSynchronize(cs));
      // ---- results -------------------------------------------------------------
      int k = 0;
      for (int i = 0; i < np; i++) {
        auto* P = B->probs[i];
        std::vector<RState> h(P->R);
        std::vector<int> ph(P->R);
        GH1_CUDA(cudaMemcpyAsync(h.data(), P->st.p, h.size() * sizeof(RState), cudaMemcpyDeviceToHost, cs));
        GH1_CUDA(cudaMemcpyAsync(ph.data(), P->phase.p, ph.size() * sizeof(int), cudaMemcpyDeviceToHost, cs));
        GH1_CUDA(cudaStreamSynchronize(cs));
        for (int r = 0; r < P->R; r++, k++) {
          gh1_cg_result& q = res[k];
          std::memset(&q, 0, sizeof(q));
          q.iterations = h[r].total;
          q.outer = h[r].outer;
          q.applies32 = h[r].total;
          q.applies64 = h[r].outer + 1;
          q.first_res = std::sqrt(h[r].bnorm2);
          q.final_res = h[r].rnorm;
          q.true_relres = h[r].bnorm2 > 0 ? h[r].rnorm / std::sqrt(h[r].bnorm2) : h[r].rnorm;
          q.status = ph[r] == PH_DONE ? h[r].status : GH1_MAXITER;
          if (q.status != GH1_OK && status == GH1_OK) status = q.status;
        }
        int herr = 0;
        GH1_CUDA(cudaMemcpy(&herr, P->op->d_err.p, sizeof(int), cudaMemcpyDeviceToHost));
        GH1_CHECK(herr == 0, GH1_ERR_CUDA, "batch: a bounded wait in the multi-rhs apply timed out");
      }
      GH1_CUDA(cudaEventRecord(ev[0], cs));
      GH1_CUDA(cudaStreamWaitEvent(user, ev[0], 0));
      GH1_CUDA(cudaStreamSynchronize(cs));
    } catch (...) {
      cleanup();
      throw;
    }
    cleanup();
  });
  return rc != GH1_OK ? rc : status;
}
