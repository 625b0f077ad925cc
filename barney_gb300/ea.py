"""Differentiable fixed-step emission-absorption rendering.

EAProblem holds a density grid (the structured field, FP32, x-fastest), a
transfer function and a set of views on the GPU; render/backward call the
native march (gbv_ea_render) and its path-replay adjoint (gbv_ea_backward).
ea_render_autograd wraps both as a torch.autograd.Function so that
d(loss)/d(voxels) and d(loss)/d(TF entries) come from the hand-written
adjoint kernel.
"""
from __future__ import annotations

import ctypes as C
import copy

import numpy as np

from . import _native as N
from .device import _ptr, _stream, ea_views
from .scenes import Scene


class EAProblem:
    """store: optional GpuScene whose brick-corner store (any format and brick
    shape) the forward march reads instead of the FP32 linear field; the
    adjoint and the FP64 march always read the FP32 linear field."""

    def __init__(self, scene: Scene, views, step: float, scalars=None, tf=None, store=None):
        import torch
        self.s = scene
        self.store = store
        self.views = list(views)
        self.step = float(step)
        self._views_c = ea_views(self.views)
        self.npx = sum(v["width"] * v["height"] for v in self.views)
        self.scalars = (scalars if scalars is not None else
                        torch.from_numpy(np.ascontiguousarray(scene.scalars).reshape(-1)).cuda())
        self.tf = tf if tf is not None else torch.from_numpy(np.ascontiguousarray(scene.tf, np.float32)).cuda()

    def record(self, scalars=None, tf=None) -> N.GbvScene:
        s = self.s
        r = N.GbvScene()
        r.d_voxels = (self.scalars if scalars is None else scalars).data_ptr()
        r.format, r.layout = N.GBV_VOXEL_F32, N.GBV_LAYOUT_LINEAR
        r.dims[:] = list(s.dims)
        origin, spacing = s.geometry()
        r.origin[:] = list(origin)
        r.spacing[:] = list(spacing)
        t = self.tf if tf is None else tf
        r.d_tf = t.data_ptr()
        r.tf_n = t.shape[0]
        r.domain[:] = list(s.domain)
        r.base_density = s.base_density
        return r

    def render(self, scalars=None, tf=None):
        """FP32 images, (num pixels over all views, 4)."""
        import torch
        out = torch.empty((self.npx, 4), dtype=torch.float32, device="cuda")
        rec = self.record(scalars, tf)
        if self.store is not None and scalars is None:
            g = self.store
            rec.d_voxels = g.voxels.data_ptr()
            rec.d_scale_offset = g.scale_offset.data_ptr() if g.scale_offset is not None else None
            rec.format, rec.layout = g.fmt, g.layout
            rec.brick_log2[:] = list(g.brick)
        N.check(N.lib().gbv_ea_render(C.byref(rec), self._views_c, len(self.views), self.step, _ptr(out),
                                      _stream()), "gbv_ea_render")
        return out

    def render_f64(self, scalars=None, tf=None):
        """FP64 images (finite-difference check mode)."""
        import torch
        out = torch.empty((self.npx, 4), dtype=torch.float64, device="cuda")
        rec = self.record(scalars, tf)
        N.check(N.lib().gbv_ea_render_f64(C.byref(rec), self._views_c, len(self.views), self.step, _ptr(out),
                                          _stream()), "gbv_ea_render_f64")
        return out

    def backward(self, images, grad_images, scalars=None, tf=None):
        """(dL/dvoxels, dL/dTF) for dL/dimages = grad_images."""
        import torch
        gv = torch.zeros(self.scalars.numel(), dtype=torch.float32, device="cuda")
        gt = torch.zeros(self.tf.numel(), dtype=torch.float32, device="cuda")
        rec = self.record(scalars, tf)
        images = images.contiguous().float()
        grad_images = grad_images.contiguous().float()
        N.check(N.lib().gbv_ea_backward(C.byref(rec), self._views_c, len(self.views), self.step, _ptr(images),
                                        _ptr(grad_images), _ptr(gv), _ptr(gt), _stream()), "gbv_ea_backward")
        return gv, gt.reshape(self.tf.shape)

    # finite-difference helpers (the FP32 values actually stored are returned)
    def with_voxel(self, index: int, value: float) -> "EAProblem":
        q = copy.copy(self)
        q.scalars = self.scalars.clone()
        q.scalars[index] = value
        return q

    def with_tf_entry(self, index: int, value: float) -> "EAProblem":
        q = copy.copy(self)
        q.tf = self.tf.clone()
        q.tf.view(-1)[index] = value
        return q


def _autograd():
    import torch

    class EARender(torch.autograd.Function):
        @staticmethod
        def forward(ctx, scalars, tf, problem):
            scalars = scalars.contiguous()
            tf = tf.contiguous()
            img = problem.render(scalars, tf)
            ctx.problem = problem
            ctx.save_for_backward(scalars, tf, img)
            return img

        @staticmethod
        def backward(ctx, grad_img):
            scalars, tf, img = ctx.saved_tensors
            gv, gt = ctx.problem.backward(img, grad_img, scalars, tf)
            return gv.reshape(scalars.shape), gt.reshape(tf.shape), None

    return EARender


_EARender = None


def ea_render_autograd(scalars, tf, problem: EAProblem):
    """Differentiable EA render of `problem`'s views with the given voxels and TF."""
    global _EARender
    if _EARender is None:
        _EARender = _autograd()
    return _EARender.apply(scalars, tf, problem)
