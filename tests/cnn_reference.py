"""Float64 CPU reference of the warm-start CNN and its layers (torch autograd on the CPU).

Test infrastructure only: the GPU kernels (iane_gb_cnn_*) are checked against these.
Layouts follow the kernels: volumes [channel][z][y][x]; weights [co][ci][27] with tap
t = tx + 3 ty + 9 tz reading x(v + (t - 1)) -- torch's conv3d (a cross-correlation) with
weight [co][ci][kz][ky][kx] and padding 1 is the same operation.
"""
from __future__ import annotations

import torch
import torch.nn.functional as F

LAYERS = [
    ("e1a", 2, 16), ("e1b", 16, 16), ("e2a", 16, 32), ("e2b", 32, 32), ("e3a", 32, 64), ("e3b", 64, 64),
    ("e3c", 64, 64),
    ("d2a", 96, 32), ("d2b", 32, 32), ("d1a", 48, 16), ("d1b", 16, 16), ("head", 16, 1),
]


def bf16_round(t: torch.Tensor) -> torch.Tensor:
    return t.to(torch.float32).to(torch.bfloat16).to(t.dtype)


class _RoundBF16(torch.autograd.Function):
    """BF16 storage of an activation: rounds the value forward and its gradient backward."""

    @staticmethod
    def forward(ctx, x):
        return bf16_round(x)

    @staticmethod
    def backward(ctx, g):
        return bf16_round(g)


def conv3(x, w, b=None):
    """x [ci][d][h][w], w [co][ci][27] -> [co][d][h][w] (float64)."""
    co, ci = w.shape[0], w.shape[1]
    y = F.conv3d(x.unsqueeze(0), w.reshape(co, ci, 3, 3, 3), b, padding=1)
    return y.squeeze(0)


def pool2(x):
    return F.avg_pool3d(x.unsqueeze(0), 2).squeeze(0)


def up2(x):
    return x.repeat_interleave(2, 1).repeat_interleave(2, 2).repeat_interleave(2, 3)


def unpack(params, device="cpu"):
    """Split a flat parameter vector (layer by layer: weights [co][ci][27], then co biases)
    into float64 leaf tensors {name: (w, b)}."""
    out, n = {}, 0
    for name, ci, co in LAYERS:
        w = params[n:n + co * ci * 27].reshape(co, ci, 27).to(torch.float64).clone().requires_grad_(True)
        n += co * ci * 27
        b = params[n:n + co].to(torch.float64).clone().requires_grad_(True)
        n += co
        out[name] = (w, b)
    return out


def forward(p, x, residual, round_activations=True):
    """p from unpack (weights already BF16-rounded by the caller), x [2][d][h][w],
    residual [d][h][w]. Returns the [1][d][h][w] output."""
    R = _RoundBF16.apply if round_activations else (lambda t: t)

    def layer(name, inp, relu=True):
        y = conv3(inp, *p[name])
        return R(torch.relu(y)) if relu else y

    x = R(x)
    e1a = layer("e1a", x)
    e1b = layer("e1b", e1a)
    p1 = R(pool2(e1b))
    e2a = layer("e2a", p1)
    e2b = layer("e2b", e2a)
    p2 = R(pool2(e2b))
    e3a = layer("e3a", p2)
    e3b = layer("e3b", e3a)
    e3c = layer("e3c", e3b)
    d2a = layer("d2a", torch.cat([up2(e3c), e2b], 0))
    d2b = layer("d2b", d2a)
    d1a = layer("d1a", torch.cat([up2(d2b), e1b], 0))
    d1b = layer("d1b", d1a)
    return layer("head", d1b, relu=False) + residual.unsqueeze(0)


def to_c8(t: torch.Tensor) -> torch.Tensor:
    """[C][D][H][W] -> the kernels' C8 layout [ceil(C/8)][D][H][W][8] (zero-padded)."""
    c = t.shape[0]
    pad = (-c) % 8
    if pad:
        t = torch.cat([t, torch.zeros((pad,) + tuple(t.shape[1:]), dtype=t.dtype, device=t.device)], 0)
    o = t.shape[0] // 8
    return t.reshape((o, 8) + tuple(t.shape[1:])).permute(0, 2, 3, 4, 1).contiguous()


def from_c8(t: torch.Tensor, c: int) -> torch.Tensor:
    """C8 [O][D][H][W][8] -> [c][D][H][W]."""
    o = t.shape[0]
    return t.permute(0, 4, 1, 2, 3).reshape((o * 8,) + tuple(t.shape[1:4]))[:c]
