"""Gradient test harness: the GGX Cornell box's material parameters as torch
tensors, rendered through mcrt_render and differentiated through mcrt_adjoint
(path-replay backpropagation) inside a torch.autograd.Function.  Test code only:
the library itself has no torch dependency on this path."""
import numpy as np
import torch

import mcrt_gb300 as M
from mcrt_gb300 import scenes

SLOTS = list(scenes.GGX_SLOTS)
LIGHT = scenes.LIGHT_SLOT


class CornellRenderer:
    """The differentiable scene on one context: set parameters, render, adjoint."""

    def __init__(self, ctx, seed=1234, width=256, height=256, max_depth=8, nee=True):
        self.ctx = ctx
        self.sc = scenes.cornell_box_ggx(seed)
        c = self.sc["camera"]
        self.w, self.h, self.depth, self.nee = width, height, max_depth, nee
        self.cam = M.compute_camera(width, height, c["look_from"], c["look_at"], c["vfov"], 0.0)
        ctx.upload_scene(vertices=self.sc["vertices"], triangles=self.sc["triangles"],
                         materials=self.sc["materials"], env=M.gradient_env_map())

    def set_params(self, albedo, roughness, radiance):
        md = scenes.ggx_materials(np.asarray(albedo, np.float32), np.asarray(roughness, np.float32),
                                  np.asarray(radiance, np.float32))
        self.ctx.update_materials(md)

    def image(self, spp, first_frame):
        """Mean of the samples of frames first_frame .. first_frame+spp-1, float64 (h, w, 3)."""
        r = self.ctx.render(self.cam, self.w, self.h, spp, first_frame=first_frame, max_depth=self.depth,
                            nee=self.nee, outputs=("sum",))
        return r["sum"] / spp

    def adjoint(self, d_image, spp, first_frame):
        return self.ctx.adjoint(self.cam, self.w, self.h, spp, d_image, first_frame=first_frame,
                                max_depth=self.depth, nee=self.nee)


class RenderImage(torch.autograd.Function):
    """image = render(albedo (5, 3), roughness (5), radiance (3)); backward replays
    `adj_spp` paths from frame `adj_frame` with the incoming image gradient."""

    @staticmethod
    def forward(ctx, albedo, roughness, radiance, renderer, spp, frame, adj_spp, adj_frame):
        renderer.set_params(albedo.detach().numpy(), roughness.detach().numpy(), radiance.detach().numpy())
        ctx.renderer, ctx.adj_spp, ctx.adj_frame = renderer, adj_spp, adj_frame
        return torch.from_numpy(renderer.image(spp, frame))

    @staticmethod
    def backward(ctx, grad_image):
        g = ctx.renderer.adjoint(grad_image.detach().numpy().astype(np.float32), ctx.adj_spp, ctx.adj_frame)
        g = torch.from_numpy(g)
        return g[SLOTS, :3], g[SLOTS, 3], g[LIGHT, :3], None, None, None, None, None


def l2_loss(image, target):
    return ((image - target) ** 2).mean()
