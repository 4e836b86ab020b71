"""nr_adjoint inside torch autograd, for the tests (test harness only: the
product exposes the adjoint through the C ABI and needs no torch).

RenderImage.apply(theta, scene, mats, params) renders the image of the
material parameters theta, a (num_mats, 7) float64 tensor in nr_adjoint's
columns (albedo r g b, roughness, emission r g b; inverse.param_table),
with nr_render; its backward calls nr_adjoint with the incoming
d loss / d image on the same samples (same params, so the same Philox seed)
and returns d loss / d theta, zero where a material has no such parameter.
"""
import numpy as np
import torch


class RenderImage(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, scene, mats, params):
        from nuray_gb300 import inverse
        P = theta.detach().cpu().numpy().astype(np.float64)
        _, mask = inverse.param_table(mats)
        cur = inverse.apply(mats, P)
        scene.set_materials(cur)
        img = scene.render(params)
        ctx.scene, ctx.cur, ctx.params = scene, cur, params
        ctx.mask = torch.from_numpy(mask)
        return torch.from_numpy(img.astype(np.float64))

    @staticmethod
    def backward(ctx, grad_img):
        ctx.scene.set_materials(ctx.cur)
        g = ctx.scene.adjoint(ctx.params, grad_img.detach().cpu().numpy().astype(np.float32))
        g = torch.from_numpy(g.astype(np.float64)) * ctx.mask
        return g, None, None, None
