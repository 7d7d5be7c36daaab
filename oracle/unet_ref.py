"""CPU reference of the U-Net warm-start network (natrix_gb300/core/warmstart.py)
in float64 with torch autograd — TEST INFRASTRUCTURE ONLY (the network has
no counterpart in the reference; this is the checker of its kernels).

The same layers and wiring; weights are rounded to bf16 as the GPU packs them.
`forward` keeps activations in float64; `forward_mirrored` rounds every tensor
the GPU stores in bf16 at the same point -- activations on the way forward and
activation gradients on the way back -- so the remaining difference is FP32
versus FP64 accumulation."""
from __future__ import annotations

import torch
import torch.nn.functional as F


def bf16_round(t: torch.Tensor) -> torch.Tensor:
    return t.to(torch.bfloat16).to(t.dtype)


class _Round(torch.autograd.Function):
    """bf16 rounding of a stored tensor: forward value and incoming gradient."""

    @staticmethod
    def forward(ctx, t):
        return bf16_round(t)

    @staticmethod
    def backward(ctx, g):
        return bf16_round(g)


def forward_mirrored(params: dict, x: torch.Tensor) -> torch.Tensor:
    """The GPU's rounding points: every ReLU output, pooled and upsampled
    tensor is stored in bf16 (and so is the gradient flowing into it); the
    two uses of e1 / e2 (pooling and the skip) each store their gradient in
    bf16 before the sum, which is stored again."""
    R = _Round.apply

    def conv(name, inp):
        w, b = params[name]
        return F.relu(F.conv2d(inp, w, b, padding=1))

    x = bf16_round(x)
    a11 = R(conv("c11", x))
    e1 = R(conv("c12", a11))
    q1 = R(F.avg_pool2d(R(e1), 2))
    a21 = R(conv("c21", q1))
    e2 = R(conv("c22", a21))
    q2 = R(F.avg_pool2d(R(e2), 2))
    a31 = R(conv("c31", q2))
    e3 = R(conv("c32", a31))
    u3 = R(F.interpolate(e3, scale_factor=2, mode="nearest"))
    a41 = R(conv("c41", torch.cat([u3, R(e2)], 1)))
    d2 = R(conv("c42", a41))
    u2 = R(F.interpolate(d2, scale_factor=2, mode="nearest"))
    a51 = R(conv("c51", torch.cat([u2, R(e1)], 1)))
    w, b = params["c52"]
    d1f = F.relu(F.conv2d(a51, w, b, padding=1))
    hw, hb = params["head"]
    # the head reads the FP32 ReLU output; the stored d1 (bf16) feeds its gradient
    d1 = d1f + (R(d1f) - d1f).detach()
    return (d1f * hw.view(1, -1, 1, 1)).sum(1) + hb + 0 * d1.sum()


def forward(params: dict, x: torch.Tensor) -> torch.Tensor:
    """params: name -> (w [cout][cin][3][3], b [cout]) float64 (weights already
    bf16-rounded), plus 'head' -> (w [16], b [1]); x: (B, 2, H, W)."""
    def conv(name, inp):
        w, b = params[name]
        return F.relu(F.conv2d(inp, w, b, padding=1))

    a11 = conv("c11", x)
    e1 = conv("c12", a11)
    a21 = conv("c21", F.avg_pool2d(e1, 2))
    e2 = conv("c22", a21)
    a31 = conv("c31", F.avg_pool2d(e2, 2))
    e3 = conv("c32", a31)
    u3 = F.interpolate(e3, scale_factor=2, mode="nearest")
    a41 = conv("c41", torch.cat([u3, e2], 1))
    d2 = conv("c42", a41)
    u2 = F.interpolate(d2, scale_factor=2, mode="nearest")
    a51 = conv("c51", torch.cat([u2, e1], 1))
    d1 = conv("c52", a51)
    hw, hb = params["head"]
    return (d1 * hw.view(1, -1, 1, 1)).sum(1) + hb


def apply_operator(p: torch.Tensor, mask: torch.Tensor) -> torch.Tensor:
    """(A p) with the sweep's neighbour rule (shader.Poisson.comp:17-38):
    wall or obstacle neighbour -> centre value.  p: (B, H, W), mask bool."""
    B, H, W = p.shape
    obs = mask.bool()

    def nb(shift_y, shift_x):
        pp = torch.roll(p, shifts=(-shift_y, -shift_x), dims=(1, 2))
        oo = torch.roll(obs, shifts=(-shift_y, -shift_x), dims=(1, 2))
        wall = torch.zeros_like(obs)
        if shift_x == -1:
            wall[:, :, 0] = True
        if shift_x == 1:
            wall[:, :, W - 1] = True
        if shift_y == -1:
            wall[:, 0, :] = True
        if shift_y == 1:
            wall[:, H - 1, :] = True
        return torch.where(wall | oo, p, pp)

    return nb(0, -1) + nb(0, 1) + nb(-1, 0) + nb(1, 0) - 4 * p


def loss(p: torch.Tensor, target: torch.Tensor, b: torch.Tensor, mask: torch.Tensor,
         lam: float) -> torch.Tensor:
    """Same definition as natrix_nn_loss, batch-mean."""
    fluid = (~mask.bool()).to(p.dtype)
    n = fluid.sum((1, 2)).clamp(min=1)
    e = (p - target) * fluid
    mean_e = e.sum((1, 2)) / n
    lp = (((e - mean_e.view(-1, 1, 1)) * fluid) ** 2).sum((1, 2)) / n
    r = (b - apply_operator(p, mask)) * fluid
    lr = (r ** 2).sum((1, 2)) / ((b * fluid) ** 2).sum((1, 2)).clamp(min=1e-300)
    return (lp + lam * lr).mean()
