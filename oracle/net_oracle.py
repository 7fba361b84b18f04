"""CPU oracle of the learned initial guess network (test infrastructure only).

The encoder-decoder of ``flowfpmpp_gb300`` restated with PyTorch's CPU
``conv3d`` in float64, with BF16 rounding applied where the GPU stores BF16:
weights, activations after every ReLU, pooled tensors, the network input,
and (through ``_RoundGrad``) the output adjoint of every convolution, which
the GPU keeps in BF16 as the tensor-core operand of its backward kernels.
Everything else (accumulation, the loss, FP32 gradient buffers) is float64
here, so GPU and oracle agree to accumulation-order and rare BF16 rounding
flips.  Only tests use this module; the product never imports it.

Layouts: the GPU's flat parameter vector (per layer: weights [27][cout][cin]
with tap t = (dk+1)*9 + (dj+1)*3 + (di+1), then biases [cout]); cell fields
are numpy arrays of shape (nx, ny, nz) (x fastest in memory with order='F').
"""
from __future__ import annotations

import numpy as np
import torch
import torch.nn.functional as F

# cin, ca, cout, level, relu -- the layer table of the GPU network
SPEC = [(16, 16, 16, 0, 1), (16, 16, 32, 1, 1), (32, 32, 48, 2, 1), (48, 48, 64, 3, 1),
        (112, 48, 48, 2, 1), (80, 32, 32, 1, 1), (48, 16, 16, 0, 1), (16, 16, 16, 0, 0)]


def param_count() -> int:
    return sum(27 * co * ci + co for ci, _, co, _, _ in SPEC)


def bf(x: torch.Tensor) -> torch.Tensor:
    return x.to(torch.bfloat16).to(torch.float64)


class _RoundGrad(torch.autograd.Function):
    """Identity forward; rounds the incoming gradient to BF16."""

    @staticmethod
    def forward(ctx, x):
        return x.view_as(x)

    @staticmethod
    def backward(ctx, g):
        return bf(g)


def split_params(flat: np.ndarray):
    """Flat FP32 vector -> list of (w[co, ci, 3(dk), 3(dj), 3(di)], b[co]) float64 leaf tensors."""
    out, o = [], 0
    flat = np.asarray(flat, dtype=np.float64)
    for ci, _, co, _, _ in SPEC:
        nw = 27 * co * ci
        w = flat[o:o + nw].reshape(3, 3, 3, co, ci)  # [dk][dj][di][co][ci]
        b = flat[o + nw:o + nw + co]
        o += nw + co
        wt = torch.tensor(np.ascontiguousarray(w.transpose(3, 4, 0, 1, 2)), requires_grad=True)
        out.append((wt, torch.tensor(b, requires_grad=True)))
    return out


def join_grads(params) -> np.ndarray:
    parts = []
    for w, b in params:
        g = w.grad.numpy().transpose(2, 3, 4, 0, 1)  # [dk][dj][di][co][ci]
        parts += [g.reshape(-1), b.grad.numpy()]
    return np.concatenate(parts)


def _cell(a: np.ndarray) -> torch.Tensor:
    """(nx, ny, nz) numpy -> (1, 1, nz, ny, nx) float64 tensor (conv3d's D, H, W = z, y, x)."""
    return torch.tensor(np.ascontiguousarray(np.asarray(a, dtype=np.float64).transpose(2, 1, 0)))[None, None]


def forward(params, fluid, mx, my, mz, rhs):
    """Network output y (1, 1, nz, ny, nx) float64 for the inputs."""
    nx, ny, nz = fluid.shape
    f = _cell((np.asarray(fluid) != 0).astype(np.float64))
    X = torch.zeros(1, 16, nz, ny, nx, dtype=torch.float64)
    X[0, 0] = f[0, 0]
    X[0, 1] = torch.tensor(np.asarray(mx, dtype=np.float64))[None, None, :].expand(nz, ny, nx)
    X[0, 2] = torch.tensor(np.asarray(my, dtype=np.float64))[None, :, None].expand(nz, ny, nx)
    X[0, 3] = torch.tensor(np.asarray(mz, dtype=np.float64))[:, None, None].expand(nz, ny, nx)
    X[0, 4] = f[0, 0] * bf(torch.tensor(np.asarray(rhs, dtype=np.float32).astype(np.float64)).permute(2, 1, 0))
    X = bf(X)

    def conv(l, x):
        w, b = params[l]
        z = F.conv3d(x, bf(w), padding=1) + b[None, :, None, None, None]
        z = _RoundGrad.apply(z)
        return bf(torch.relu(z)) if SPEC[l][4] else z

    def pool(x):
        return bf(F.avg_pool3d(x, 2))

    def up(x):
        return x.repeat_interleave(2, 2).repeat_interleave(2, 3).repeat_interleave(2, 4)

    a0 = conv(0, X)
    a1 = conv(1, pool(a0))
    a2 = conv(2, pool(a1))
    a3 = conv(3, pool(a2))
    d2 = conv(4, torch.cat([a2, up(a3)], 1))
    d1 = conv(5, torch.cat([a1, up(d2)], 1))
    d0 = conv(6, torch.cat([a0, up(d1)], 1))
    y = conv(7, d0)
    return y[:, :1]


def loss(y, fluid, target):
    """1 - cos^2 between y and target over fluid cells, both fluid-mean free."""
    f = _cell((np.asarray(fluid) != 0).astype(np.float64))
    t = _cell(np.asarray(target, dtype=np.float32).astype(np.float64))
    n = f.sum()
    yc = (y - (y * f).sum() / n) * f
    tc = (t - (t * f).sum() / n) * f
    yy, yt, tt = (yc * yc).sum(), (yc * tc).sum(), (tc * tc).sum()
    return 1.0 - yt * yt / (yy * tt)


def output_and_grads(flat_params, fluid, mx, my, mz, rhs, target):
    """(y as (nx, ny, nz) numpy, loss, flat parameter gradient)."""
    params = split_params(flat_params)
    y = forward(params, fluid, mx, my, mz, rhs)
    L = loss(y, fluid, target)
    L.backward()
    return y.detach()[0, 0].numpy().transpose(2, 1, 0), float(L.detach()), join_grads(params)
