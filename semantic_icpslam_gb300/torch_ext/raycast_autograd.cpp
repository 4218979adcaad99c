// libtorch C++ form of the differentiable raycast: a torch::autograd::Function
// whose forward renders the vertex and normal maps at exp(xi) P through the
// library's visibility, z-range and raycast entry points, and whose backward
// is sf_RaycastAdjoint (the gradient with respect to the left se(3)
// perturbation xi = (rho, omega), exact at xi = 0, and to the map's TSDF
// values, one float per voxel index).  The kernels are the library's CUDA
// kernels; this file is plumbing over include/sfusion.h.
#include <torch/extension.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "sfusion.h"

namespace {

using torch::Tensor;
using torch::autograd::AutogradContext;
using torch::autograd::variable_list;

void check(int st, const char *what) { TORCH_CHECK(st == SF_OK, what, " returned status ", st); }

// A renderer: the context and map handles, the image size, intrinsics and
// depth range, and the rendering-block buffer CreateRenderingBlocks needs.
struct Renderer {
  sf_context *ctx;
  sf_map *map;
  int cols, rows;
  float fx, fy, cx, cy, dmin, dmax;
  Tensor blocks, nblk;
};

sf_image image_of(const Tensor &t) {
  sf_image im;
  im.data = t.data_ptr();
  im.step = (size_t)t.stride(0) * t.element_size();
  im.cols = (int)t.size(1);
  im.rows = (int)t.size(0);
  return im;
}

// exp(xi) P for the twist xi = (rho, omega) (Rodrigues rotation, left
// Jacobian translation), P a 4x4 row-major double camera -> world pose.
void exp_times(const double xi[6], const double *P, double out[16]) {
  const double *r = xi, *w = xi + 3;
  const double th = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
  const double W[9] = {0, -w[2], w[1], w[2], 0, -w[0], -w[1], w[0], 0};
  double W2[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) W2[i * 3 + j] = W[i * 3 + 0] * W[0 * 3 + j] + W[i * 3 + 1] * W[1 * 3 + j] + W[i * 3 + 2] * W[2 * 3 + j];
  double a, b, c;
  if (th < 1e-10) {
    a = 1.0; b = 0.5; c = 1.0 / 6.0;
  } else {
    a = std::sin(th) / th;
    b = (1 - std::cos(th)) / (th * th);
    c = (th - std::sin(th)) / (th * th * th);
  }
  double T[16] = {0};
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) T[i * 4 + j] = (i == j) + a * W[i * 3 + j] + b * W2[i * 3 + j];
    double t = 0;
    for (int j = 0; j < 3; ++j) t += ((i == j) + b * W[i * 3 + j] + c * W2[i * 3 + j]) * r[j];
    T[i * 4 + 3] = t;
  }
  T[15] = 1;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      double v = 0;
      for (int k = 0; k < 4; ++k) v += T[i * 4 + k] * P[k * 4 + j];
      out[i * 4 + j] = v;
    }
}

// Frame::GpuRotation / GpuInvRotation / GpuTranslation (Core/Frame.cc:626-645)
void pose_to_gpu(const double *P, sf_mat3 &R, sf_mat3 &RI, sf_float3 &t) {
  float *r = &R.rowx.x, *ri = &RI.rowx.x;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      r[i * 3 + j] = (float)P[i * 4 + j];
      ri[j * 3 + i] = (float)P[i * 4 + j];
    }
  t.x = (float)P[3]; t.y = (float)P[7]; t.z = (float)P[11];
}

float inv_f(float f) { return (float)(1.0 / (double)f); }

struct RaycastFunction : public torch::autograd::Function<RaycastFunction> {
  static variable_list forward(AutogradContext *actx, Tensor xi, Tensor sdf, int64_t handle, Tensor P) {
    Renderer &r = *reinterpret_cast<Renderer *>(handle);
    TORCH_CHECK(xi.numel() == 6, "xi must have 6 elements");
    auto xih = xi.detach().to(torch::kCPU, torch::kFloat64).contiguous();
    auto Ph = P.detach().to(torch::kCPU, torch::kFloat64).contiguous();
    TORCH_CHECK(Ph.numel() == 16, "P must be 4x4");
    auto Pe = torch::empty({4, 4}, torch::kFloat64);
    exp_times(xih.data_ptr<double>(), Ph.data_ptr<double>(), Pe.data_ptr<double>());
    sf_mat3 R, RI;
    sf_float3 t;
    pose_to_gpu(Pe.data_ptr<double>(), R, RI, t);
    uint32_t nvis = 0;
    check(sf_CheckBlockVisibility(r.ctx, r.map, R, RI, t, r.cols, r.rows, r.fx, r.fy, r.cx, r.cy, r.dmax, r.dmin,
                                  &nvis),
          "sf_CheckBlockVisibility");
    auto opt = torch::TensorOptions().dtype(torch::kFloat32).device(torch::kCUDA);
    auto zmin = torch::empty({(r.rows + 7) / 8, (r.cols + 7) / 8}, opt), zmax = torch::empty_like(zmin);
    int ok = 0;
    check(sf_CreateRenderingBlocks(r.ctx, r.map, image_of(zmin), image_of(zmax), r.dmax, r.dmin,
                                   static_cast<sf_rendering_block *>(r.blocks.data_ptr()),
                                   static_cast<uint32_t *>(r.nblk.data_ptr()), RI, t, nvis, r.fx, r.fy, r.cx, r.cy,
                                   &ok),
          "sf_CreateRenderingBlocks");
    auto vm = torch::empty({r.rows, r.cols, 4}, opt), nm = torch::empty_like(vm);
    check(sf_Raycast(r.ctx, r.map, image_of(vm), image_of(nm), image_of(zmin), image_of(zmax), R, RI, t,
                     inv_f(r.fx), inv_f(r.fy), r.cx, r.cy),
          "sf_Raycast");
    actx->save_for_backward({zmin, zmax, Pe});
    actx->saved_data["handle"] = handle;
    actx->saved_data["n"] = sdf.size(0);
    actx->saved_data["xi_dtype"] = xi.scalar_type();
    actx->saved_data["xi_device"] = xi.device();
    return {vm, nm};
  }

  static variable_list backward(AutogradContext *actx, variable_list grads) {
    auto saved = actx->get_saved_variables();
    Renderer &r = *reinterpret_cast<Renderer *>(actx->saved_data["handle"].toInt());
    const Tensor &zmin = saved[0], &zmax = saved[1], &Pe = saved[2];
    sf_mat3 R, RI;
    sf_float3 t;
    pose_to_gpu(Pe.data_ptr<double>(), R, RI, t);
    auto gv = grads[0].defined() ? grads[0].contiguous().to(torch::kFloat32) : Tensor();
    auto gn = grads[1].defined() ? grads[1].contiguous().to(torch::kFloat32) : Tensor();
    if (!gv.defined()) gv = torch::zeros({r.rows, r.cols, 4}, zmin.options());
    auto gsdf = torch::zeros({actx->saved_data["n"].toInt()}, zmin.options());
    double gpose[6];
    sf_image gni;
    std::memset(&gni, 0, sizeof(gni));
    if (gn.defined()) gni = image_of(gn);
    check(sf_RaycastAdjoint(r.ctx, r.map, image_of(zmin), image_of(zmax), R, RI, t, inv_f(r.fx), inv_f(r.fy), r.cx,
                            r.cy, image_of(gv), gni, gsdf.data_ptr<float>(), gpose),
          "sf_RaycastAdjoint");
    auto gxi = torch::from_blob(gpose, {6}, torch::kFloat64)
                   .clone()
                   .to(actx->saved_data["xi_device"].toDevice(), actx->saved_data["xi_dtype"].toScalarType());
    return {gxi, gsdf, Tensor(), Tensor()};
  }
};

int64_t renderer_create(int64_t ctx, int64_t map, int64_t cols, int64_t rows, double fx, double fy, double cx, double cy,
                        double dmin, double dmax, int64_t max_blocks) {
  auto *r = new Renderer;
  r->ctx = reinterpret_cast<sf_context *>(ctx);
  r->map = reinterpret_cast<sf_map *>(map);
  r->cols = (int)cols;
  r->rows = (int)rows;
  r->fx = (float)fx; r->fy = (float)fy; r->cx = (float)cx; r->cy = (float)cy;
  r->dmin = (float)dmin; r->dmax = (float)dmax;
  auto u8 = torch::TensorOptions().dtype(torch::kUInt8).device(torch::kCUDA);
  r->blocks = torch::empty({max_blocks, 16}, u8);
  r->nblk = torch::empty({1}, u8.dtype(torch::kInt32));
  return reinterpret_cast<int64_t>(r);
}

void renderer_destroy(int64_t handle) { delete reinterpret_cast<Renderer *>(handle); }

variable_list raycast(Tensor xi, Tensor sdf, int64_t handle, Tensor P) {
  return RaycastFunction::apply(xi, sdf, handle, P);
}

}  // namespace

PYBIND11_MODULE(TORCH_EXTENSION_NAME, m) {
  m.doc() = "libtorch C++ autograd form of the differentiable raycast";
  m.def("renderer_create", &renderer_create);
  m.def("renderer_destroy", &renderer_destroy);
  m.def("raycast", &raycast, "vertex and normal maps at exp(xi) P; differentiable in xi and sdf");
}
