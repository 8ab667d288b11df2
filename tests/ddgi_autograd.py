"""Thin torch.autograd.Function over ddgi_forward_record / ddgi_backward
(test harness only).

    atlas = AtlasFunction.apply(albedo, sun, sky, runner)

runs K probe updates from a zero atlas with the given per-material albedo
(M x 3), sun radiance (3) and sky radiance (3), and returns the final colour
atlas (H x W x 4, float32); its backward returns the gradients of those three
parameters with the hit set held fixed.
"""
import numpy as np
import torch

from vulkanexp_gb300 import abi
from vulkanexp_gb300.ddgi import Context


class Runner:
    def __init__(self, workload, orientations, checkpoint_every=2):
        self.w = workload
        self.orient = np.ascontiguousarray(orientations, np.float32).reshape(-1, 9)
        self.C = checkpoint_every
        self.ctx = Context(workload.grid)
        self.ctx.build_scene(workload.scene)
        self.materials = workload.scene.materials.copy()

    def forward(self, albedo, sun, sky):
        m = self.materials.copy()
        m["base_color"] = albedo
        self.ctx.set_materials(m)
        L = self.w.light
        self.ctx.set_light(abi.make_light(L.direction[:3], sun, sky))
        for kind in (abi.ATLAS_COLOR, abi.ATLAS_DEPTH):
            self.ctx.set_atlas(kind, np.zeros(self.ctx.atlas_shape(kind), np.float32))
        self.ctx.set_probe_states(np.ones(self.w.grid.probe_count(), np.uint32))
        self.ctx.forward_record(self.orient, self.C)
        return self.ctx.get_atlas(abi.ATLAS_COLOR)

    def backward(self, grad_color):
        return self.ctx.backward(grad_color, len(self.materials))

    def close(self):
        self.ctx.close()


class AtlasFunction(torch.autograd.Function):
    @staticmethod
    def forward(fctx, albedo, sun, sky, runner):
        fctx.runner = runner
        atlas = runner.forward(albedo.detach().cpu().numpy(), sun.detach().cpu().numpy(), sky.detach().cpu().numpy())
        return torch.from_numpy(atlas)

    @staticmethod
    def backward(fctx, grad):
        ga, gs, gk = fctx.runner.backward(grad.detach().contiguous().cpu().numpy().astype(np.float32))
        return torch.from_numpy(ga).double(), torch.from_numpy(gs).double(), torch.from_numpy(gk).double(), None
