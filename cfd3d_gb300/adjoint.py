"""Gradient-check harness of the discrete adjoint: the FP64 residual as a
torch.autograd.Function whose backward is cfd3d_residual_vjp.

The function differentiated is R(pv): the residual of cfd3d_residual on an engine whose
interior pv is the argument, each interior cell's dv and tv(1:2) its EOS and the eddy
viscosity tv(3) and the dual-time history held at the engine's stored values.  State
setting goes through the public C ABI only: cfd3d_eos_eval for the EOS of the new state,
cfd3d_upload_state for the fields.  This module serves gradient checks; the solver's hot
path does not use it.
"""
import numpy as np

from . import native


class StateSetter:
    """Sets an engine's interior pv with EOS-consistent dv / tv(1:2), keeping everything
    else (ghost values before the boundary program, tv(3), qq) as captured at creation."""

    def __init__(self, engine):
        self.e = engine
        self.base = [engine.download(n) for n in range(len(engine.case["blocks"]))]
        self.fluid = int(engine.case["cfg"].get("fluid", 2))
        self.prop = int(engine.case["cfg"].get("iturb", 0)) != -3

    def interior(self, n):
        return self.base[n]["pv"][3:-3, 3:-3, 3:-3, :].copy()

    def fields(self, n, pv_int):
        """Padded pv, dv, tv for block n with interior pv = pv_int."""
        b = self.base[n]
        pv = b["pv"].copy()
        dv = b["dv"].copy()
        tv = b["tv"].copy() if self.e.ntv else None
        pv[3:-3, 3:-3, 3:-3, :] = pv_int
        pref = float(self.e.case["cfg"]["pref"])
        flat = pv_int.reshape(-1, pv_int.shape[-1])
        d, t = native.eos_eval(flat[:, 0] + pref, flat[:, 4], flat[:, 5], flat[:, 6], fluid=self.fluid,
                               prop=self.prop)
        dv[3:-3, 3:-3, 3:-3, :] = d.reshape(pv_int.shape[:-1] + (18,))
        if tv is not None and self.prop:
            tv[3:-3, 3:-3, 3:-3, :2] = t.reshape(pv_int.shape[:-1] + (2,))
        return pv, dv, tv

    def apply(self, pv_blocks):
        for n, p in enumerate(pv_blocks):
            pv, dv, tv = self.fields(n, p)
            self.e.upload(n, pv=pv, dv=dv, tv=tv)

    def residual(self, pv_blocks):
        self.apply(pv_blocks)
        return [self.e.residual(n)["res"] for n in range(len(pv_blocks))]


def residual_function():
    """torch.autograd.Function R(pv) over one engine (imported lazily: torch is needed only
    by the gradient-check harness)."""
    import torch

    class Residual(torch.autograd.Function):
        @staticmethod
        def forward(ctx, pv, setter):
            shapes = [setter.interior(n).shape for n in range(len(setter.base))]
            blocks, off = [], 0
            flat = pv.detach().cpu().numpy()
            for s in shapes:
                m = int(np.prod(s))
                blocks.append(flat[off:off + m].reshape(s))
                off += m
            res = setter.residual(blocks)
            ctx.setter = setter
            ctx.blocks = blocks
            return torch.from_numpy(np.concatenate([r.reshape(-1) for r in res]))

        @staticmethod
        def backward(ctx, gres):
            setter = ctx.setter
            setter.apply(ctx.blocks)
            g = gres.detach().cpu().numpy()
            cot, off = [], 0
            for p in ctx.blocks:
                m = p.size
                cot.append(g[off:off + m].reshape(p.shape))
                off += m
            gs, _ = setter.e.residual_vjp(cot)
            return torch.from_numpy(np.concatenate([x.reshape(-1) for x in gs])), None

    return Residual
