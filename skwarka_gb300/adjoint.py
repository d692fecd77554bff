"""torch.autograd harness over the C ABI's direct-lighting adjoint.

This is a test harness: the forward is skw_render_direct and the backward is
skw_render_direct_adjoint (a hand-written CUDA adjoint that replays the
forward's rays from the same seed); torch only carries the tensors.

Parameters: per-triangle RGB albedo (n_triangles, 3) and one scale of every
area light's radiance.  Geometry and visibility are fixed."""
from __future__ import annotations

import ctypes as C

from . import _lib
from .render import Camera, RenderScene, c_camera, skw_render_params


def _set_params(scene: RenderScene, albedo, emission_scale) -> None:
    import torch
    lib = _lib.load()
    a = albedo.detach().to(torch.float32).contiguous()
    if a.shape != (scene.n_triangles, 3) or not a.is_cuda:
        raise ValueError(f"albedo must be a CUDA tensor of shape ({scene.n_triangles}, 3)")
    s = torch.cuda.current_stream().cuda_stream
    _lib.check(lib.skw_scene_set_triangle_albedo(scene.handle, a.data_ptr(), s), scene.ctx.handle)
    _lib.check(lib.skw_scene_set_emission_scale(scene.handle, float(emission_scale)), scene.ctx.handle)
    scene._albedo_keepalive = a  # the copy is stream-ordered


class DirectLighting:
    """render(albedo, emission_scale) -> (H, W, 3) image, differentiable in
    both arguments through the CUDA adjoint."""

    def __init__(self, scene: RenderScene, camera: Camera, spp_x: int = 4, spp_y: int = 4, light_samples: int = 1,
                 seed: int = 0, sampler: int = 0):
        self.scene, self.camera = scene, camera
        self.params = skw_render_params(spp_x, spp_y, light_samples, seed, sampler)
        scene.n_triangles = int(_lib.load().skw_scene_n_triangles(scene.handle))

    def forward_image(self, albedo, emission_scale):
        import torch
        _set_params(self.scene, albedo, emission_scale)
        out = torch.empty((self.camera.height, self.camera.width, 3), dtype=torch.float32, device="cuda")
        cam = c_camera(self.camera)
        _lib.check(_lib.load().skw_render_direct(self.scene.handle, C.byref(cam), C.byref(self.params), out.data_ptr(),
                                                 torch.cuda.current_stream().cuda_stream), self.scene.ctx.handle)
        return out

    def adjoint(self, albedo, emission_scale, d_image):
        """(dL/d albedo (n_triangles, 3), dL/d emission_scale) for dL/dI = d_image."""
        import torch
        _set_params(self.scene, albedo, emission_scale)
        g_alb = torch.zeros((self.scene.n_triangles, 3), dtype=torch.float32, device="cuda")
        g_em = torch.zeros(1, dtype=torch.float64, device="cuda")
        d = d_image.detach().to(torch.float32).contiguous()
        cam = c_camera(self.camera)
        _lib.check(_lib.load().skw_render_direct_adjoint(self.scene.handle, C.byref(cam), C.byref(self.params),
                                                         d.data_ptr(), g_alb.data_ptr(), g_em.data_ptr(),
                                                         torch.cuda.current_stream().cuda_stream),
                   self.scene.ctx.handle)
        return g_alb, g_em

    def __call__(self, albedo, emission_scale):
        return _Fn.apply(albedo, emission_scale, self)


def _make_fn():
    import torch

    class Fn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, albedo, emission_scale, renderer):
            ctx.renderer = renderer
            ctx.save_for_backward(albedo, emission_scale)
            return renderer.forward_image(albedo, float(emission_scale))

        @staticmethod
        def backward(ctx, grad_out):
            albedo, emission_scale = ctx.saved_tensors
            g_alb, g_em = ctx.renderer.adjoint(albedo, float(emission_scale), grad_out)
            return g_alb.to(albedo.dtype), g_em.to(emission_scale.dtype).reshape(emission_scale.shape), None

    return Fn


class _LazyFn:
    _fn = None

    def apply(self, *a):
        if _LazyFn._fn is None:
            _LazyFn._fn = _make_fn()
        return _LazyFn._fn.apply(*a)


_Fn = _LazyFn()
