"""torch.autograd form of the raycast and its adjoint, and the keyframe map
refinement they drive (outside the drop-in loop).

* TorchMap: a voxel-block map whose arrays are torch tensors handed to
  sf_map_wrap, so the TSDF values are a (strided) torch view of the voxels
  the kernels read.
* Renderer: visibility, z-range and raycast for a pose (sf_CheckBlockVisibility,
  sf_CreateRenderingBlocks, sf_Raycast; Mapping::RayTrace's order) and the
  adjoint (sf_RaycastAdjoint).
* raycast(xi, sdf, renderer, P): an autograd function rendering vertex and
  normal maps at exp(xi) P.  Its backward gives dL/dxi (the left se(3)
  perturbation, exact at xi = 0) and dL/dsdf (one value per voxel index).
* refine_tsdf: Adam on the observed voxels' TSDF values against keyframes'
  depth, the gradient summed over keyframes by the adjoint.

The autograd layer is plumbing over the C ABI; the forward and backward
passes are the library's CUDA kernels.
"""
import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import Image, Intrinsics, MapConfig, call

__all__ = ["TorchMap", "Renderer", "raycast", "raycast_cpp", "refine_tsdf", "se3_exp"]


def se3_exp(xi):
    """exp of the twist xi = (rho, omega), translation first, as a 4x4 float64
    matrix (Rodrigues rotation, left-Jacobian translation)."""
    xi = np.asarray(xi, np.float64)
    rho, w = xi[:3], xi[3:]
    th = np.linalg.norm(w)
    W = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
    if th < 1e-10:
        R, V = np.eye(3) + W, np.eye(3) + 0.5 * W
    else:
        a, b, c = np.sin(th) / th, (1 - np.cos(th)) / th ** 2, (th - np.sin(th)) / th ** 3
        R = np.eye(3) + a * W + b * W @ W
        V = np.eye(3) + b * W + c * W @ W
    T = np.eye(4)
    T[:3, :3], T[:3, 3] = R, V @ rho
    return T


def _img(t):
    t = t.contiguous() if not t.is_contiguous() else t
    return Image(t.data_ptr(), t.stride(0) * t.element_size(), t.shape[1], t.shape[0])


def _pose(P):
    from . import pose_to_gpu
    return pose_to_gpu(np.asarray(P, np.float64))


class TorchMap:
    """Voxel-block map (Mapping/DeviceMap.h layout) in torch tensors."""

    def __init__(self, ctx, voxel_size, trunc_dist, num_buckets, num_excess, num_sdf_blocks, depth_min=0.1,
                 depth_max=3.0, max_rendering_blocks=260000):
        dev = "cuda"
        ne = num_buckets + num_excess
        i32 = torch.int32
        self.cfg = MapConfig(voxel_size, trunc_dist, depth_min, depth_max, num_buckets, num_excess, num_sdf_blocks,
                             max_rendering_blocks)
        self.heap_mem = torch.empty(num_sdf_blocks, dtype=i32, device=dev)
        self.entry_ptr = torch.empty(1, dtype=i32, device=dev)
        self.heap_counter = torch.empty(1, dtype=i32, device=dev)
        self.bucket_mutex = torch.empty(num_buckets, dtype=i32, device=dev)
        self.voxels = torch.empty(num_sdf_blocks * 512 * 4, dtype=torch.float32, device=dev)  # 16 B per voxel
        self.no_visible = torch.empty(1, dtype=i32, device=dev)
        self.entries = torch.full((ne * 8,), -1, dtype=i32, device=dev)  # 32 B per entry, ptr = -1
        self.visible = torch.full((ne * 8,), -1, dtype=i32, device=dev)
        a = _lib.DeviceMap(self.heap_mem.data_ptr(), self.entry_ptr.data_ptr(), self.heap_counter.data_ptr(),
                           self.bucket_mutex.data_ptr(), self.voxels.data_ptr(), self.no_visible.data_ptr(),
                           self.entries.data_ptr(), self.visible.data_ptr())
        self.h = C.c_void_p()
        call("sf_map_wrap", C.byref(self.cfg), C.byref(a), C.byref(self.h))
        call("sf_ResetMap", ctx.h, self.h)
        ctx.sync()
        self.num_voxels = num_sdf_blocks * 512

    def sdf(self):
        """TSDF values, one per voxel index: a strided view of the voxels."""
        return self.voxels.view(-1, 4)[:, 0]

    def weight(self):
        """Integration weights (uint8 byte 4 of each voxel) as int32."""
        return self.voxels.view(torch.uint8).view(-1, 16)[:, 4].to(torch.int32)

    def close(self):
        if self.h:
            call("sf_map_destroy", self.h)
            self.h = None


class Renderer:
    """Raycast of a TorchMap (or any sf_map handle) and its adjoint."""

    def __init__(self, ctx, tmap, cols, rows, K, depth_max=3.0, depth_min=0.1):
        self.ctx, self.map, self.cols, self.rows = ctx, tmap, cols, rows
        self.K = tuple(float(k) for k in K)
        self.dmax, self.dmin = depth_max, depth_min
        self.invfx = float(np.float32(1.0 / np.float64(np.float32(K[0]))))
        self.invfy = float(np.float32(1.0 / np.float64(np.float32(K[1]))))
        self.zc, self.zr = (cols + 7) // 8, (rows + 7) // 8
        cap = tmap.cfg.max_rendering_blocks
        self.blocks = torch.empty((cap, 16), dtype=torch.uint8, device="cuda")
        self.nblk = torch.empty(1, dtype=torch.int32, device="cuda")

    def render(self, P):
        """(vmap, nmap, zmin, zmax) at camera -> world pose P (4x4)."""
        R, RI, t = _pose(P)
        nvis = C.c_uint32()
        call("sf_CheckBlockVisibility", self.ctx.h, self.map.h, R, RI, t, self.cols, self.rows, *self.K, self.dmax,
             self.dmin, C.byref(nvis))
        zmin = torch.empty((self.zr, self.zc), dtype=torch.float32, device="cuda")
        zmax = torch.empty_like(zmin)
        ok = C.c_int()
        call("sf_CreateRenderingBlocks", self.ctx.h, self.map.h, _img(zmin), _img(zmax), self.dmax, self.dmin,
             self.blocks.data_ptr(), self.nblk.data_ptr(), RI, t, nvis.value, *self.K, C.byref(ok))
        vm = torch.empty((self.rows, self.cols, 4), dtype=torch.float32, device="cuda")
        nm = torch.empty_like(vm)
        call("sf_Raycast", self.ctx.h, self.map.h, _img(vm), _img(nm), _img(zmin), _img(zmax), R, RI, t,
             self.invfx, self.invfy, self.K[2], self.K[3])
        return vm, nm, zmin, zmax

    def adjoint(self, P, zmin, zmax, grad_vmap, grad_nmap=None, grad_sdf=None):
        """dL/dxi (6 doubles) of the render at P; dL/dsdf added into grad_sdf."""
        R, RI, t = _pose(P)
        g = (C.c_double * 6)()
        gv = grad_vmap.contiguous().float()
        gn = grad_nmap.contiguous().float() if grad_nmap is not None else None
        call("sf_RaycastAdjoint", self.ctx.h, self.map.h, _img(zmin), _img(zmax), R, RI, t, self.invfx, self.invfy,
             self.K[2], self.K[3], _img(gv), _img(gn) if gn is not None else Image(),
             grad_sdf.data_ptr() if grad_sdf is not None else None, g)
        return np.array(g[:])


class _RaycastFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx_, xi, sdf, renderer, P):
        Pe = se3_exp(xi.detach().double().cpu().numpy()) @ np.asarray(P, np.float64)
        vm, nm, zmin, zmax = renderer.render(Pe)
        ctx_.renderer, ctx_.P, ctx_.n = renderer, Pe, sdf.shape[0]
        ctx_.save_for_backward(zmin, zmax)
        ctx_.xi_dtype, ctx_.xi_device = xi.dtype, xi.device
        return vm, nm

    @staticmethod
    def backward(ctx_, gvm, gnm):
        zmin, zmax = ctx_.saved_tensors
        gsdf = torch.zeros(ctx_.n, dtype=torch.float32, device="cuda")
        gx = ctx_.renderer.adjoint(ctx_.P, zmin, zmax, gvm, gnm, gsdf)
        return torch.tensor(gx, dtype=ctx_.xi_dtype, device=ctx_.xi_device), gsdf, None, None


def raycast(xi, sdf, renderer, P):
    """Vertex and normal maps rendered at exp(xi) P, differentiable in xi and
    in sdf (the map's TSDF values, e.g. TorchMap.sdf())."""
    return _RaycastFn.apply(xi, sdf, renderer, P)


def _torch_ext():
    """The libtorch C++ extension (torch_ext/raycast_autograd.cpp, built next
    to the library as sf_torch.so)."""
    from . import sf_torch
    return sf_torch


def raycast_cpp(xi, sdf, renderer, P):
    """raycast() through the libtorch C++ torch::autograd::Function: the same
    forward and backward (sf_Raycast / sf_RaycastAdjoint), with the autograd
    node implemented in C++."""
    ext = _torch_ext()
    if getattr(renderer, "_cpp", None) is None:
        r = renderer
        renderer._cpp = ext.renderer_create(r.ctx.h.value, r.map.h.value, r.cols, r.rows, *r.K, r.dmin, r.dmax,
                                            r.blocks.shape[0])
    Pt = torch.as_tensor(np.asarray(P, np.float64))
    vm, nm = ext.raycast(xi, sdf, renderer._cpp, Pt)
    return vm, nm


def refine_tsdf(renderer, tmap, keyframes, steps=50, lr=0.01, betas=(0.9, 0.999), eps=1e-8):
    """Adam on the observed voxels' TSDF values against keyframe depth.

    keyframes: [(P, depth)] with P the 4x4 camera -> world pose and depth a
    (rows, cols) float tensor in metres (NaN or 0 where unobserved).  The
    loss is the sum over keyframes and pixels of (rendered z - depth)^2;
    its gradient comes from the raycast adjoint.  Values are clamped to the
    normalised range [-1, 1].  Returns the loss before each step."""
    sdf = tmap.sdf()
    observed = tmap.weight() > 0
    m = torch.zeros(tmap.num_voxels, dtype=torch.float32, device="cuda")
    v = torch.zeros_like(m)
    b1, b2 = betas
    losses = []
    for it in range(1, steps + 1):
        grad = torch.zeros_like(m)
        total = 0.0
        for P, d in keyframes:
            vm, nm, zmin, zmax = renderer.render(P)
            z = vm[..., 2]
            ok = torch.isfinite(z) & torch.isfinite(d) & (d > 0)
            r = torch.where(ok, z - d, torch.zeros_like(z))
            total += float((r * r).sum())
            gv = torch.zeros_like(vm)
            gv[..., 2] = 2.0 * r
            renderer.adjoint(P, zmin, zmax, gv, None, grad)
        losses.append(total)
        grad = torch.where(observed, grad, torch.zeros_like(grad))
        m.mul_(b1).add_(grad, alpha=1 - b1)
        v.mul_(b2).addcmul_(grad, grad, value=1 - b2)
        step = lr * (m / (1 - b1 ** it)) / ((v / (1 - b2 ** it)).sqrt() + eps)
        new = torch.where(observed, (sdf - step).clamp(-1.0, 1.0), sdf)
        sdf.copy_(new)
    return losses
