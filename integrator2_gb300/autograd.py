"""Pair integrals as differentiable functions of the vertex coordinates (torch.autograd).

`pair_integrals(V, C, pairs, ...)` returns, for every pair class, J (n, 3) and P (n,) computed
by the CUDA path through the C-ABI; their gradient with respect to V is the library's adjoint
kernel (i2_evaluator_backward_class), which recomputes the refined sub-cells of the forward pass
on dual numbers instead of storing them.  The refinement chosen by the forward pass is frozen in
the backward pass.  torch is used for device buffers and the autograd graph only.
"""
from __future__ import annotations

import numpy as np
import torch

from . import api

CLASSES = (api.SIMPLE_NEIGHBORS, api.ATTACHED_NEIGHBORS, api.NOT_NEIGHBORS, api.SELF)


class _Settings:
    def __init__(self, mode="fixed", level=0, tol=1e-6, max_level=5, precision=api.PRECISION_FP64, hard_tol=1e-8,
                 self_sign=0, rule=(10, 8, 3, 24)):
        self.mode, self.level, self.tol, self.max_level = mode, level, tol, max_level
        self.precision, self.hard_tol, self.self_sign, self.rule = precision, hard_tol, self_sign, rule

    def integrator(self, mesh):
        it = api.NumericalIntegrator3D(mesh, api.qf3D13)
        if self.mode == "fixed":
            it.setFixedRefinementLevel(self.level)
        elif self.mode == "compat":
            it.setErrorControl(api.AUTOMATIC_ERROR_CONTROL, 1e-6, self.max_level)
        else:
            it.setErrorControl(api.RELATIVE_ERROR_CONTROL, self.tol, self.max_level)
        it.setPrecision(self.precision)
        it.setHardPairTolerance(self.hard_tol)
        it.setSelfConvention(self.self_sign)
        it.setPotentialRule(*self.rule)
        return it


class PairIntegrals(torch.autograd.Function):
    @staticmethod
    def forward(ctx, V, C, pairs, settings):
        dev = torch.device("cuda", torch.cuda.current_device())
        mesh = api.Mesh3D()
        mesh.setGeometry(V.detach().to("cpu", torch.float64).numpy(), np.ascontiguousarray(C.cpu().numpy(), np.int32))
        mesh.prepareMesh(3.0)  # the class lists come from the caller; the cutoff keeps set-up O(N)
        it = settings.integrator(mesh)
        ev = api.EvaluatorJ3DK(mesh, it)
        ev.setStream(torch.cuda.current_stream(dev).cuda_stream)
        outs, dpairs = [], []
        for cls, pr in zip(CLASSES, pairs):
            p = pr.to(dev, torch.int32).contiguous()
            n = p.shape[0]
            J = torch.empty((n, 3), dtype=torch.float64, device=dev)
            P = torch.empty((n,), dtype=torch.float64, device=dev)
            if n:
                ev.runClassDevice(cls, p.data_ptr(), n, 0, J.data_ptr(), P.data_ptr())
            outs += [J, P]
            dpairs.append(p)
        ctx.keep = (mesh, it, ev, dpairs)
        ctx.v_meta = (V.shape, V.dtype, V.device)
        return tuple(outs)

    @staticmethod
    def backward(ctx, *grads):
        mesh, it, ev, dpairs = ctx.keep
        shape, dtype, device = ctx.v_meta
        dev = dpairs[0].device
        gradV = torch.zeros(shape, dtype=torch.float64, device=dev)
        for k, (cls, p) in enumerate(zip(CLASSES, dpairs)):
            gJ, gP = grads[2 * k], grads[2 * k + 1]
            n = p.shape[0]
            if n == 0 or (gJ is None and gP is None):
                continue
            gJ = None if gJ is None else gJ.to(dev, torch.float64).contiguous()
            gP = None if gP is None else gP.to(dev, torch.float64).contiguous()
            ev.backwardClass(cls, p.data_ptr(), n, 0 if gJ is None else gJ.data_ptr(), 0 if gP is None else gP.data_ptr(),
                             gradV.data_ptr())
        return gradV.to(device, dtype), None, None, None


def pair_integrals(V: torch.Tensor, C, pairs, **settings):
    """V (nv, 3) vertex coordinates (requires_grad for the adjoint), C (nc, 3) cells, pairs: four
    (n, 2) index tensors (common vertex, common edge, disjoint, self).  Settings: mode ("fixed",
    "compat" or "relative"), level, tol, max_level, precision (api.PRECISION_FP64 / _MIXED),
    hard_tol, self_sign, rule.  Returns [(J, P)] per class."""
    C = torch.as_tensor(np.asarray(C, np.int32))
    pairs = [torch.as_tensor(np.ascontiguousarray(np.asarray(p, np.int32).reshape(-1, 2))) for p in pairs]
    out = PairIntegrals.apply(V, C, pairs, _Settings(**settings))
    return [(out[2 * k], out[2 * k + 1]) for k in range(4)]
