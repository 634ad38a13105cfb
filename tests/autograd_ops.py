"""Thin torch.autograd.Function wrappers over the engine's forward/backward C-ABI op pairs.

Test harness only: the engine itself has no torch dependency.  Each wrapper runs the engine on
torch's current stream so autograd's ordering holds."""
import torch

import omega2d_gb300 as og


class ProbeVelocity(torch.autograd.Function):
    """u_p = (1/2 pi) sum_j s_j K(|p - x_j|^2; r_j) J(p - x_j) at field points p (finalized,
    zero freestream); differentiable in the source positions and strengths."""

    @staticmethod
    def forward(ctx, sx, sy, sr, ss, px, py, engine, core, accum):
        engine.set_stream(torch.cuda.current_stream().cuda_stream)
        u = torch.zeros_like(px)
        v = torch.zeros_like(py)
        og.points_affect_points_dev(engine, core, og.VELONLY, accum, sx, sy, sr, ss, px, py, None, u, v,
                                    finalize=True)
        ctx.save_for_backward(sx, sy, sr, ss, px, py)
        ctx.engine, ctx.core, ctx.accum = engine, core, accum
        return u, v

    @staticmethod
    def backward(ctx, gu, gv):
        sx, sy, sr, ss, px, py = ctx.saved_tensors
        gsx, gsy, gss = (torch.zeros_like(sx) for _ in range(3))
        ctx.engine.set_stream(torch.cuda.current_stream().cuda_stream)
        og.points_affect_points_vjp_dev(ctx.engine, ctx.core, ctx.accum, sx, sy, sr, ss, px, py, None,
                                        gu.contiguous(), gv.contiguous(), gsx, gsy, gss)
        return gsx, gsy, None, gss, None, None, None, None, None


class PanelVelocity(torch.autograd.Function):
    """Finalized velocity of the panels' vortex and source sheets at points (zero freestream),
    differentiable in the panel strengths."""

    @staticmethod
    def forward(ctx, vs, ss, nx, ny, idx, px, py, engine, accum):
        engine.set_stream(torch.cuda.current_stream().cuda_stream)
        u = torch.zeros_like(px)
        v = torch.zeros_like(py)
        og.panels_affect_points_dev(engine, accum, nx, ny, idx, vs, ss, px, py, u, v, finalize=True)
        ctx.save_for_backward(nx, ny, idx, px, py)
        ctx.engine, ctx.accum, ctx.npan = engine, accum, vs.numel()
        return u, v

    @staticmethod
    def backward(ctx, gu, gv):
        nx, ny, idx, px, py = ctx.saved_tensors
        gvs = torch.zeros(ctx.npan, device=px.device)
        gss = torch.zeros(ctx.npan, device=px.device)
        ctx.engine.set_stream(torch.cuda.current_stream().cuda_stream)
        og.panels_affect_points_vjp_dev(ctx.engine, ctx.accum, nx, ny, idx, px, py, gu.contiguous(), gv.contiguous(),
                                        gvs, gss)
        return gvs, gss, None, None, None, None, None, None, None
