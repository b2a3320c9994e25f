"""Plain PyTorch FP32 reference (CPU) of the warm-start network, for the
numerics tests of its CUDA kernels.

Same arithmetic model as the kernels: weights and the three hidden
activations rounded to BF16 (round to nearest even), products accumulated in
FP32, biases in FP32, "same" zero-padded 3x3x3 convolutions per frame.  The
rounding is an identity in the backward (the kernels differentiate with
respect to the BF16 weights they use), so autograd of this module gives the
gradient the training kernels approximate (they also round the propagated
gradients to BF16).

Parameter vector: per layer, weights [27][cout][cin] with tap = 9 dz + 3 dy +
dx (offsets -1..1, x fastest), then the biases [cout].
"""
from __future__ import annotations

import numpy as np
import torch
import torch.nn.functional as F

LAYERS = ((16, 24), (24, 24), (24, 24), (24, 1))


def bf16(t: torch.Tensor) -> torch.Tensor:
    return t.to(torch.bfloat16).to(torch.float32)


def _ste(t: torch.Tensor) -> torch.Tensor:
    return t + (bf16(t) - t).detach()


def split(params: np.ndarray, requires_grad: bool = False):
    out, off = [], 0
    for cin, cout in LAYERS:
        nw = 27 * cout * cin
        W = torch.tensor(params[off:off + nw].reshape(27, cout, cin), dtype=torch.float32,
                         requires_grad=requires_grad)
        b = torch.tensor(params[off + nw:off + nw + cout], dtype=torch.float32, requires_grad=requires_grad)
        out.append((W, b))
        off += nw + cout
    return out


def forward(layers, x: torch.Tensor) -> torch.Tensor:
    """x: [F, 16, nz, ny, nx] (BF16 values in FP32) -> [F, nz, ny, nx]"""
    a = x
    for L, (W, b) in enumerate(layers):
        cout, cin = W.shape[1], W.shape[2]
        w = _ste(W).reshape(3, 3, 3, cout, cin).permute(3, 4, 0, 1, 2)
        z = F.conv3d(a, w, bias=b, padding=1)
        a = _ste(torch.relu(z)) if L < 3 else z
    return a[:, 0]


def features_to_input(x0: np.ndarray) -> torch.Tensor:
    """[F][nz][ny][nx][16] feature values (FP32) -> [F, 16, nz, ny, nx]"""
    t = torch.from_numpy(np.ascontiguousarray(x0, dtype=np.float32))
    return t.permute(0, 4, 1, 2, 3).contiguous()


def predict(params: np.ndarray, x0: np.ndarray) -> np.ndarray:
    with torch.no_grad():
        return forward(split(params), features_to_input(x0)).numpy()


def loss_and_grad(params: np.ndarray, x0: np.ndarray, target: np.ndarray, margin: int):
    """mean squared error over voxels >= margin from the crop border, and its
    gradient as a flat vector in the parameter layout"""
    layers = split(params, requires_grad=True)
    out = forward(layers, features_to_input(x0))
    t = torch.from_numpy(np.ascontiguousarray(target, dtype=np.float32))
    m = margin
    nz, ny, nx = out.shape[1:]
    d = (out - t)[:, m:nz - m, m:ny - m, m:nx - m]
    loss = (d * d).mean()
    loss.backward()
    g = np.concatenate([np.concatenate([W.grad.numpy().reshape(-1), b.grad.numpy()]) for W, b in layers])
    return float(loss.detach()), g
