"""torch.autograd.Function over the forward/adjoint C-ABI pair.

    render = DiffRender(gpu_scene, camera, spp=32, max_depth=6)
    image = render(albedo, emission)        # (H, W, 3) CUDA tensor
    loss = ((image - target) ** 2).sum()
    loss.backward()                         # albedo.grad, emission.grad via the path-replay adjoint

forward = mcrt_render, backward = mcrt_render_adjoint with the same seed, so the
gradient is the exact derivative of the Monte Carlo estimate that forward returned
(common random numbers).  Parameters: albedo (num_albedo_params, 3) for the Lambert
materials whose albedo_param is set, emission (num_emission_params, 3) for the emitters
whose emission_param is set.
"""
from __future__ import annotations

import numpy as np
import torch

from .scene import CameraDesc, GpuScene


class _RenderFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, albedo, emission, owner):
        params = (albedo.detach().clone(), emission.detach().clone())
        owner._apply(*params)
        img = torch.empty((owner.camera.height, owner.camera.width, 3), dtype=torch.float32, device=albedo.device)
        owner.scene.render(owner.camera, out=img, **owner.kw)
        ctx.owner = owner
        # the parameters this image was rendered with: the scene may hold others by the
        # time backward runs (a second forward, an optimiser step), and the path-replay
        # derivative depends on them (it divides by the albedo at each vertex)
        ctx.params = params
        return img

    @staticmethod
    def backward(ctx, grad_img):
        o = ctx.owner
        current = o.applied
        o._apply(*ctx.params)
        try:
            ga, ge, _ = o.scene.render_adjoint(o.camera, o.kw["spp"], o.kw["max_depth"], grad_img.contiguous(),
                                               o.n_albedo, o.n_emission, rr_depth=o.kw["rr_depth"],
                                               seed=o.kw["seed"], traverse=o.kw["traverse"])
        finally:
            if current is not None and current[0] is not ctx.params[0]:
                o._apply(*current)  # the scene keeps the latest forward's parameters
        return ga.clone(), ge.clone(), None


class DiffRender:
    def __init__(self, scene: GpuScene, camera: CameraDesc, spp: int, max_depth: int, rr_depth: int = -1,
                 seed: int = 0, traverse: int = 0):
        self.scene = scene
        self.camera = camera
        self.kw = dict(spp=spp, max_depth=max_depth, rr_depth=rr_depth, seed=seed, traverse=traverse)
        mats = scene.desc.materials
        self.alb_mats = np.array([i for i, m in enumerate(mats) if m.albedo_param >= 0], np.int64)
        self.alb_idx = np.array([mats[i].albedo_param for i in self.alb_mats], np.int64)
        self.em_mats = np.array([i for i, m in enumerate(mats) if m.emission_param >= 0], np.int64)
        self.em_idx = np.array([mats[i].emission_param for i in self.em_mats], np.int64)
        self.n_albedo = int(self.alb_idx.max() + 1) if self.alb_idx.size else 0
        self.n_emission = int(self.em_idx.max() + 1) if self.em_idx.size else 0
        self.applied = None  # the (albedo, emission) pair the scene's materials hold

    def _apply(self, albedo: torch.Tensor, emission: torch.Tensor):
        a = albedo.detach().float().cpu().numpy()
        e = emission.detach().float().cpu().numpy()
        mats = list(self.scene.desc.materials)
        for mi, k in zip(self.alb_mats, self.alb_idx):
            mats[mi].color = tuple(float(x) for x in a[k])
        for mi, k in zip(self.em_mats, self.em_idx):
            mats[mi].color = tuple(float(x) for x in e[k])
        self.scene.set_materials(mats)
        self.applied = (albedo, emission)

    def __call__(self, albedo: torch.Tensor, emission: torch.Tensor) -> torch.Tensor:
        return _RenderFn.apply(albedo, emission, self)
