"""CPU oracle of the learned sketch's network (TEST INFRASTRUCTURE).

numpy restatement of the MLP that rsvdt_mlp_* runs on the GPU: layers
Z_l = A_l W_l^T + b_l, A_{l+1} = GELU(Z_l) (exact erf form) except after
the last layer, mean-squared-error loss. The GPU stores the weights in
bf16 and multiplies in FP32; `bf16=True` rounds the weights the same way
(round to nearest even) so that gradients can be compared. Flat parameter
layout: for each layer W (out x in, row-major) then b.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf


def bf16_round(x: np.ndarray) -> np.ndarray:
    """float32 -> bf16 -> float32, round to nearest even."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32)


def unpack(params: np.ndarray, widths):
    out, off = [], 0
    for i in range(len(widths) - 1):
        n_in, n_out = widths[i], widths[i + 1]
        W = params[off:off + n_in * n_out].reshape(n_out, n_in)
        off += n_in * n_out
        b = params[off:off + n_out]
        off += n_out
        out.append((W, b))
    return out


def gelu(x):
    return 0.5 * x * (1 + erf(x / np.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2 * np.pi)


def forward(params, widths, X, bf16: bool = True, dtype=np.float32):
    layers = unpack(np.asarray(params, dtype=dtype), widths)
    A = [np.asarray(X, dtype=dtype)]
    Z = []
    for l, (W, b) in enumerate(layers):
        Wm = bf16_round(W).astype(dtype) if bf16 else W
        z = A[-1] @ Wm.T + b
        Z.append(z)
        A.append(gelu(z).astype(dtype) if l + 1 < len(layers) else z)
    return Z, A


def loss_and_grads(params, widths, X, T, bf16: bool = True, dtype=np.float32):
    layers = unpack(np.asarray(params, dtype=dtype), widths)
    Z, A = forward(params, widths, X, bf16, dtype)
    Y = A[-1]
    n = Y.size
    loss = float(np.mean((Y - T) ** 2))
    dZ = (2.0 * (Y - T) / n).astype(dtype)
    grads = []
    for l in range(len(layers) - 1, -1, -1):
        W, _ = layers[l]
        Wm = bf16_round(W).astype(dtype) if bf16 else W
        dW = dZ.T @ A[l]
        db = dZ.sum(axis=0)
        grads.append((dW, db))
        if l == 0:
            break
        dA = dZ @ Wm
        dZ = (dA * gelu_grad(Z[l - 1])).astype(dtype)
    flat = []
    for dW, db in reversed(grads):
        flat.append(dW.reshape(-1))
        flat.append(db)
    return loss, np.concatenate(flat).astype(dtype)
