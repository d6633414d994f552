// proj.cu -- Projector(mask, range): the diagonal 0/1 operator that keeps the
// entries whose mask bit equals `range` (linalg/diagonalmatrix.cpp:13-110; the
// reference's GPU version is DevProjector, ngscuda/linalg_kernels.cu:304-376).
//   Mult:     y = P x
//   MultAdd:  y += s P x
//   Project:  x = P x in place
// The mask is one byte per DOF (the FreeDofs() layout of gh1_space_get_freedofs).
#include <algorithm>
#include "common.cuh"

struct gh1_proj {
  gh1_ctx* ctx = nullptr;
  int64_t n = 0;
  bool keep = true;                 // range: keep entries whose mask byte is nonzero
  gh1::DBuf<uint8_t> d_mask;
};

namespace gh1 {

template <class T>
__global__ void proj_apply_kernel(int64_t n, const uint8_t* __restrict__ mask, bool keep, T s, const T* __restrict__ x,
                                  T* __restrict__ y, bool accumulate) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const bool on = (mask[i] != 0) == keep;
    if (accumulate) {
      if (on) y[i] += s * x[i];
    } else {
      y[i] = on ? s * x[i] : T(0);
    }
  }
}

template <class T>
__global__ void proj_project_kernel(int64_t n, const uint8_t* __restrict__ mask, bool keep, T* __restrict__ x) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if ((mask[i] != 0) != keep) x[i] = T(0);
}

template <class F>
static int proj_guard(gh1_ctx* ctx, F&& f) {
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

}  // namespace gh1

extern "C" {

int gh1_projector_create(gh1_ctx* ctx, int64_t n, const uint8_t* mask, int range, int mem, gh1_proj** out) {
  if (!ctx || !out || (n > 0 && !mask) || n < 0) return GH1_ERR_ARG;
  return gh1::proj_guard(ctx, [&] {
    auto* p = new gh1_proj();
    p->ctx = ctx;
    p->n = n;
    p->keep = range != 0;
    p->d_mask.alloc(n);
    if (n)
      GH1_CUDA(cudaMemcpyAsync(p->d_mask.p, mask, n, mem == GH1_MEM_DEVICE ? cudaMemcpyDeviceToDevice
                                                                         : cudaMemcpyHostToDevice, ctx->stream));
    GH1_CUDA(cudaStreamSynchronize(ctx->stream));
    *out = p;
  });
}

int gh1_projector_apply(gh1_proj* p, double s, const void* x, void* y, int precision, int accumulate) {
  if (!p || !x || !y) return p ? (p->ctx->err = "null vector", GH1_ERR_ARG) : GH1_ERR_ARG;
  return gh1::proj_guard(p->ctx, [&] {
    GH1_CHECK(precision == GH1_F64 || precision == GH1_F32, GH1_ERR_ARG, "precision must be GH1_F64 or GH1_F32");
    GH1_CHECK(accumulate || x != y, GH1_ERR_ARG, "x and y must not alias (use gh1_projector_project)");
    const int grid = gh1::grid_for(p->ctx, p->n, 256);
    if (precision == GH1_F64)
      gh1::proj_apply_kernel<double><<<grid, 256, 0, p->ctx->stream>>>(p->n, p->d_mask.p, p->keep, s, (const double*)x,
                                                                       (double*)y, accumulate != 0);
    else
      gh1::proj_apply_kernel<float><<<grid, 256, 0, p->ctx->stream>>>(p->n, p->d_mask.p, p->keep, (float)s,
                                                                      (const float*)x, (float*)y, accumulate != 0);
    gh1::check_kernel(p->ctx, "proj_apply_kernel");
  });
}

int gh1_projector_project(gh1_proj* p, void* x, int precision) {
  if (!p || !x) return p ? (p->ctx->err = "null vector", GH1_ERR_ARG) : GH1_ERR_ARG;
  return gh1::proj_guard(p->ctx, [&] {
    GH1_CHECK(precision == GH1_F64 || precision == GH1_F32, GH1_ERR_ARG, "precision must be GH1_F64 or GH1_F32");
    const int grid = gh1::grid_for(p->ctx, p->n, 256);
    if (precision == GH1_F64)
      gh1::proj_project_kernel<double><<<grid, 256, 0, p->ctx->stream>>>(p->n, p->d_mask.p, p->keep, (double*)x);
    else
      gh1::proj_project_kernel<float><<<grid, 256, 0, p->ctx->stream>>>(p->n, p->d_mask.p, p->keep, (float*)x);
    gh1::check_kernel(p->ctx, "proj_project_kernel");
  });
}

int gh1_projector_free(gh1_proj* p) {
  delete p;
  return GH1_OK;
}

}  // extern "C"
