"""torch.autograd.Function over the adjoint C ABI (test harness only).

LbmObjective.apply(fx, tau, alpha) runs the forward model through lbm_adj_forward and returns J;
backward() calls lbm_adj_backward and scales the gradients by the incoming grad_output. The
tensors are CPU float64 scalars / vectors; the model itself runs on the GPU.
"""
from __future__ import annotations

import numpy as np
import torch


class LbmObjective(torch.autograd.Function):
    @staticmethod
    def forward(ctx, fx, tau, alpha, adj, steps, window):
        adj.set_params(float(tau), float(fx), 0.0)
        adj.set_alpha(alpha.detach().cpu().numpy())
        J = adj.forward(steps, window)
        ctx.adj = adj
        return torch.tensor(J[0], dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad_out):
        g = ctx.adj.backward(want_alpha=True)
        s = float(grad_out)
        return (torch.tensor(g["fx"][0] * s, dtype=torch.float64),
                torch.tensor(g["tau"][0] * s, dtype=torch.float64),
                torch.from_numpy(np.ascontiguousarray(g["alpha"][0] * s)),
                None, None, None)
