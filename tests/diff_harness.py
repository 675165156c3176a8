"""Thin test harness: the weighted-ray image as a torch.autograd.Function
whose backward is the engine's hand-written adjoint (mx_diff_adjoint)."""
import numpy as np
import torch

from marx_gb300.diff import RECORD


class WeightedImage(torch.autograd.Function):
    """image = WeightedImage.apply(theta, diff): theta a float64 tensor of
    18 parameters, diff a marx_gb300.diff.DiffImage.  The forward records the
    rays' decisions; the backward differentiates through them."""

    @staticmethod
    def forward(ctx, theta, diff):
        t = theta.detach().cpu().numpy().astype(np.float64)
        img = diff.forward(t, RECORD)
        ctx.diff = diff
        ctx.theta = t
        ctx.device = theta.device
        return img

    @staticmethod
    def backward(ctx, grad_image):
        g = ctx.diff.adjoint(ctx.theta, grad_image.contiguous())
        return torch.as_tensor(g, dtype=torch.float64, device=ctx.device), None
