"""Differentiable sequential lens: RMS spot radius and its gradient on the GPU.

A stack of even aspheres (raypier's AsphericFace with a circular aperture,
refracting as DielectricMaterial) traced in order onto an image plane.  The
forward is the plain FP64 path's arithmetic (the same image points as
``tracer.trace_rays`` on ``workloads.config4_spec(params)``); the gradient is
the library's hand-written adjoint (``rp_lens_backward``), which re-traces
every ray from its input up to each surface in turn instead of keeping the
forward's ray states.  PyTorch is used only for the
``torch.autograd.Function`` wrapper.

Parameters (``5 * n_surfaces`` doubles): curvature (raypier sign, R =
-curvature), conic constant, A4, A6 and thickness (vertex to next vertex; the
last one from the last vertex to the image plane) of every surface.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native, runtime


class Lens:
    """A device lens (rp_lens) and the input rays it traces."""

    def __init__(self, semi_diameter, n_index, rays, z0=0.0, max_length=1000.0, atol=1e-8, tolerance=1e-4,
                 ctx: runtime.Context | None = None):
        self.ctx = ctx or runtime.get_context()
        self.lib = self.ctx.lib
        self.n_surfaces = len(semi_diameter)
        if len(n_index) != self.n_surfaces + 1:
            raise ValueError("n_index needs one entry per medium: n_surfaces + 1")
        self._semi = np.ascontiguousarray(semi_diameter, dtype=np.double)
        self._nidx = np.ascontiguousarray(n_index, dtype=np.double)
        desc = _native.LensDesc(self.n_surfaces, 0, z0, max_length, atol, tolerance,
                                self._semi.ctypes.data, self._nidx.ctypes.data)
        rays = np.ascontiguousarray(rays)
        self.n_rays = rays.shape[0]
        self.rays = runtime.DeviceRays(self.ctx, max(self.n_rays, 1))
        self.rays.upload(rays)
        h = ctypes.c_void_p()
        _native.check(self.lib.rp_lens_create(self.ctx.handle, ctypes.byref(desc), self.n_rays, ctypes.byref(h)),
                      "rp_lens_create")
        self.handle = h
        self.ctx.attach()
        self.n_params = 5 * self.n_surfaces

    def forward(self, params) -> tuple[float, int]:
        """RMS spot radius (mm) and the number of rays that reached the image."""
        p = np.ascontiguousarray(params, dtype=np.double)
        if p.shape != (self.n_params,):
            raise ValueError(f"expected {self.n_params} parameters")
        loss = ctypes.c_double()
        nv = ctypes.c_uint64()
        _native.check(self.lib.rp_lens_forward(self.handle, p.ctypes.data, self.rays.handle, ctypes.byref(loss),
                                               ctypes.byref(nv)), "rp_lens_forward")
        return loss.value, nv.value

    def backward(self) -> np.ndarray:
        """d loss / d params of the last forward."""
        g = np.zeros(self.n_params, dtype=np.double)
        _native.check(self.lib.rp_lens_backward(self.handle, g.ctypes.data), "rp_lens_backward")
        return g

    def image(self, n=None):
        """Image-plane (x, y) and reached flags of the last forward."""
        n = self.n_rays if n is None else n
        xy = np.zeros((n, 2), dtype=np.double)
        valid = np.zeros(n, dtype=np.uint8)
        _native.check(self.lib.rp_lens_image(self.handle, xy.ctypes.data, valid.ctypes.data, n), "rp_lens_image")
        return xy, valid.astype(bool)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.rp_lens_destroy(self.handle)
            self.handle = None
            self.ctx.detach()
        if getattr(self, "rays", None) is not None:
            self.rays.free()
            self.rays = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def spot_rms(lens: Lens, params):
    """RMS spot radius as a differentiable function of a float64 torch tensor."""
    import torch

    class SpotRMS(torch.autograd.Function):
        @staticmethod
        def forward(ctx, p):
            loss, _ = lens.forward(p.detach().cpu().numpy())
            return torch.tensor(loss, dtype=torch.float64)

        @staticmethod
        def backward(ctx, grad_out):
            g = torch.from_numpy(lens.backward())
            return grad_out * g

    return SpotRMS.apply(params)


def config4_lens(n_rays=None, ctx=None) -> Lens:
    """The 262,144-ray, eight-surface configuration of workloads.CONFIG4."""
    from . import workloads as W
    from .ctracer import ray_dtype
    rays, _ = W.config4_rays(ray_dtype, n_rays)
    C = W.CONFIG4
    return Lens(W.LENS4_SEMI, W.LENS4_INDEX, rays, z0=0.0, max_length=C["max_length"], atol=C["atol"],
                tolerance=C["tolerance"], ctx=ctx)


def central_differences(lens: Lens, params, rel_step=1e-6, index=None):
    """Central finite differences of the loss, step rel_step * |p| per parameter."""
    p0 = np.asarray(params, dtype=np.double)
    idx = range(p0.shape[0]) if index is None else index
    out = {}
    for j in idx:
        h = rel_step * abs(p0[j]) if p0[j] != 0.0 else rel_step
        pp, pm = p0.copy(), p0.copy()
        pp[j] += h
        pm[j] -= h
        out[j] = (lens.forward(pp)[0] - lens.forward(pm)[0]) / (pp[j] - pm[j])
    lens.forward(p0)  # leave the lens at p0 for a following backward
    return out
