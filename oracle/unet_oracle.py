"""unet_oracle.py -- PyTorch CPU restatement of the learned-guess U-Net.

TEST INFRASTRUCTURE ONLY (checker for the library's forward, backward and
Adam kernels).  The network has no counterpart in the reference; this file
states the same computation with torch.nn.functional on the CPU.

Parameter layout (flat FP32 vector, as the library's vfs_unet_get_params):
for each of the ten 3x3x3 convolutions e0a e0b e1a e1b e2a e2b d1a d1b d0a
d0b, W[tap][cin][cout] with tap = 9 kz + 3 ky + kx, then bias[cout]; then the
head's 16 weights and bias.  Decoder convolutions read the concatenation
(upsampled coarser tensor, skip tensor) in that channel order.

`bf16=True` rounds weights, the network input and every activation to BF16
as the library stores them (rounding is treated as the identity in the
backward pass).
"""
from __future__ import annotations

import numpy as np
import torch
import torch.nn.functional as F

LAYERS = [(16, 16), (16, 16), (16, 32), (32, 32), (32, 64), (64, 64), (96, 32), (32, 32), (48, 16), (16, 16)]


def num_params():
    return sum(27 * ci * co + co for ci, co in LAYERS) + 17


def unpack(p):
    """Flat vector -> list of (weight [co][ci][3][3][3], bias) and the head."""
    p = torch.as_tensor(np.asarray(p, np.float32))
    out, off = [], 0
    for ci, co in LAYERS:
        w = p[off:off + 27 * ci * co].reshape(3, 3, 3, ci, co).permute(4, 3, 0, 1, 2).contiguous()
        off += 27 * ci * co
        b = p[off:off + co]
        off += co
        out.append((w, b))
    head = p[off:off + 17]
    return out, head


def _r(x, bf16):
    if not bf16:
        return x
    return x + (x.to(torch.bfloat16).to(torch.float32) - x).detach()


def _up(x):
    return x.repeat_interleave(2, 2).repeat_interleave(2, 3).repeat_interleave(2, 4)


def forward(params, features, bf16=True, requires_grad=False):
    """features: [4][nz][ny][nx] float32 -> (out [nz][ny][nx], leaf tensors)."""
    convs, head = unpack(params)
    leaves = []
    ws = []
    for w, b in convs:
        w = w.clone().requires_grad_(requires_grad)
        b = b.clone().requires_grad_(requires_grad)
        leaves += [w, b]
        ws.append((_r(w, bf16), b))
    head = head.clone().requires_grad_(requires_grad)
    leaves.append(head)
    f = torch.as_tensor(np.asarray(features, np.float32))
    x = torch.zeros((1, 16) + f.shape[1:])
    x[0, :4] = f
    x = _r(x, bf16)

    def conv(i, inp):
        w, b = ws[i]
        return _r(F.relu(F.conv3d(inp, w, b, padding=1)), bf16)

    e0a = conv(0, x)
    e0b = conv(1, e0a)
    p0 = _r(F.avg_pool3d(e0b, 2), bf16)
    e1a = conv(2, p0)
    e1b = conv(3, e1a)
    p1 = _r(F.avg_pool3d(e1b, 2), bf16)
    e2a = conv(4, p1)
    e2b = conv(5, e2a)
    d1a = conv(6, torch.cat([_up(e2b), e1b], 1))
    d1b = conv(7, d1a)
    d0a = conv(8, torch.cat([_up(d1b), e0b], 1))
    d0b = conv(9, d0a)
    out = (d0b[0] * head[:16, None, None, None]).sum(0) + head[16]
    return out, leaves


OFFSETS = [(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1), (1, 1, 0), (1, -1, 0),
           (-1, 1, 0), (-1, -1, 0), (0, 1, 1), (0, 1, -1), (0, -1, 1), (0, -1, -1), (1, 0, 1), (1, 0, -1),
           (-1, 0, 1), (-1, 0, -1)]  # (di, dj, dk) of the 19 operator planes


def residual_loss(out, f2, weight, op, scale):
    """sum w res^2 / sum w over the cells whose 19 neighbours are inside,
    res = f2 - scale * (A out); op: [19][nz][ny][nx] row coefficients."""
    nz, ny, nx = out.shape
    inner = (slice(1, nz - 1), slice(1, ny - 1), slice(1, nx - 1))
    a = torch.zeros((nz - 2, ny - 2, nx - 2))
    for t, (di, dj, dk) in enumerate(OFFSETS):
        a = a + op[t][inner] * out[1 + dk:nz - 1 + dk, 1 + dj:ny - 1 + dj, 1 + di:nx - 1 + di]
    res = f2[inner] - scale * a
    w = weight[inner]
    return (w * res ** 2).sum() / w.sum()


def loss_and_grad(params, features, target, weight, bf16=True, op=None, op_scale=1.0, mse_weight=1.0,
                  res_weight=0.0):
    """Weighted MSE sum(w (out - t)^2) / sum(w) (times mse_weight when a
    residual term is present) plus res_weight times the residual loss, and
    the gradient as a flat vector in the parameter layout."""
    out, leaves = forward(params, features, bf16, requires_grad=True)
    t = torch.as_tensor(np.asarray(target, np.float32))
    w = torch.as_tensor(np.asarray(weight, np.float32))
    loss = (w * (out - t) ** 2).sum() / w.sum().clamp(min=1.0)
    if op is not None:
        f2 = torch.as_tensor(np.asarray(features, np.float32))[2]
        loss = mse_weight * loss + res_weight * residual_loss(out, f2, w, torch.as_tensor(op), op_scale)
    loss.backward()
    g = []
    for q in range(0, len(leaves) - 1, 2):
        wg = leaves[q].grad.permute(2, 3, 4, 1, 0).reshape(-1)  # -> [kz][ky][kx][ci][co]
        g += [wg, leaves[q + 1].grad]
    g.append(leaves[-1].grad)
    return float(loss.detach()), torch.cat(g).numpy()


def adam(p, g, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One bias-corrected Adam step (t counts from 1); returns new p, m, v."""
    p = np.asarray(p, np.float64)
    g = np.asarray(g, np.float64)
    m = b1 * np.asarray(m, np.float64) + (1 - b1) * g
    v = b2 * np.asarray(v, np.float64) + (1 - b2) * g * g
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v
