"""Oracle (test infrastructure only): float64 numpy restatement of the warm-start MLP
(48 -> 128 x 4 -> 3, GELU, loss mean(1 - cos)) with the BF16 rounding of the GPU kernels applied to
weights, inputs and inter-layer activations, for gradient checks of the CUDA training kernels."""
from __future__ import annotations

import math

import numpy as np

DIMS = [(48, 128), (128, 128), (128, 128), (128, 128), (128, 3)]


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (round to nearest even), returned as float64."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r.astype(np.uint32)).view(np.float32).astype(np.float64)


def unpack(params: np.ndarray):
    out, o = [], 0
    for i, j in DIMS:
        w = params[o:o + i * j].reshape(j, i)
        o += i * j
        b = params[o:o + j]
        o += j
        out.append((w, b))
    return out


_erf = np.vectorize(math.erf)


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / math.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + _erf(x / math.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)


def forward(params: np.ndarray, feats: np.ndarray) -> np.ndarray:
    """The network's output (n x 3, before normalisation) with the BF16 rounding of the GPU kernels
    (inputs, weights and inter-layer activations), accumulated in float64."""
    layers = unpack(params.astype(np.float64))
    a = bf16(feats)
    for li, (w, b) in enumerate(layers):
        z = a @ bf16(w.astype(np.float32)).T + b
        a = bf16(gelu(z).astype(np.float32)) if li < len(layers) - 1 else z
    return a


def loss_and_grads(params: np.ndarray, feats: np.ndarray, targets: np.ndarray, quantize: bool = True):
    """Mean (1 - cos) loss and its gradient (flat, parameter layout). quantize=False skips the BF16
    rounding (an exactly differentiable network, for finite-difference checks of this code)."""
    q = bf16 if quantize else (lambda a: np.asarray(a, dtype=np.float64))
    layers = unpack(params.astype(np.float64))
    x = q(feats)
    acts, zs = [x], []
    for li, (w, b) in enumerate(layers):
        z = acts[-1] @ (q(w.astype(np.float32)) if quantize else w).T + b
        zs.append(z)
        if li < len(layers) - 1:
            acts.append(q(gelu(z).astype(np.float32)) if quantize else gelu(z))
    y = zs[-1]
    n = len(y)
    ny = np.linalg.norm(y, axis=1, keepdims=True)
    c = np.sum(y * targets, axis=1, keepdims=True) / ny
    loss = float(np.mean(1.0 - c))
    dz = -(targets / ny - y * (c / ny ** 2)) / n
    grads = []
    for li in range(len(layers) - 1, -1, -1):
        w, b = layers[li]
        dzq = q(dz.astype(np.float32)) if quantize else dz
        gw = dzq.T @ acts[li]
        gb = (dzq if li == len(layers) - 1 else dz).sum(axis=0)
        grads.append((gw, gb))
        if li == 0:
            break
        da = dzq @ (q(w.astype(np.float32)) if quantize else w)
        dz = da * gelu_grad(zs[li - 1])
    grads.reverse()
    flat = np.concatenate([np.concatenate([gw.ravel(), gb]) for gw, gb in grads])
    return loss, flat
