"""torch.autograd binding of the path-replay adjoint (gkrt_adjoint_forward / _backward).

    img = render_materials(renderer, fc, spp, albedo, roughness)   # (H, W, 3)
    loss = ((img - target) ** 2).mean(); loss.backward()           # grads on albedo, roughness

albedo: (n, 3) float32 CUDA tensor, roughness: (n,) float32 CUDA tensor, for materials
[first, first + n). The forward call writes them into the scene's materials; the backward
call replays the same paths. torch is only imported by this module.
"""
from __future__ import annotations

import torch


class MaterialRender(torch.autograd.Function):
    @staticmethod
    def forward(ctx, albedo, roughness, renderer, fc, spp, first, sample_roughness):
        a = albedo.detach().contiguous()
        r = roughness.detach().contiguous()
        stream = torch.cuda.current_stream().cuda_stream
        renderer.set_material_params(a.data_ptr(), r.data_ptr(), first, a.shape[0], stream)
        v = renderer.image_view(0)
        img = torch.empty((v.height, v.width, 4), dtype=torch.float32, device=albedo.device)
        sr = sample_roughness.contiguous() if sample_roughness is not None else None
        renderer.adjoint_forward(fc, spp, img.data_ptr(), sr.data_ptr() if sr is not None else None, stream)
        ctx.renderer, ctx.fc, ctx.spp, ctx.first, ctx.n = renderer, fc, spp, first, a.shape[0]
        ctx.sr = sr
        ctx.nmat = renderer.material_count
        return img[..., :3]

    @staticmethod
    def backward(ctx, grad):
        r = ctx.renderer
        H, W = grad.shape[0], grad.shape[1]
        g = torch.zeros((H, W, 4), dtype=torch.float32, device=grad.device)
        g[..., :3] = grad
        ga = torch.zeros((ctx.nmat, 3), dtype=torch.float64, device=grad.device)
        gr = torch.zeros((ctx.nmat,), dtype=torch.float64, device=grad.device)
        stream = torch.cuda.current_stream().cuda_stream
        r.adjoint_backward(ctx.fc, ctx.spp, g.data_ptr(), ga.data_ptr(), gr.data_ptr(),
                           ctx.sr.data_ptr() if ctx.sr is not None else None, stream)
        s = slice(ctx.first, ctx.first + ctx.n)
        return ga[s].float(), gr[s].float(), None, None, None, None, None


def render_materials(renderer, fc, spp, albedo, roughness, first=0, sample_roughness=None):
    return MaterialRender.apply(albedo, roughness, renderer, fc, spp, first, sample_roughness)
