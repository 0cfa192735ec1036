"""CPU oracle of the warm-start MLP (TEST INFRASTRUCTURE ONLY).

Only tests/ may import this module.  It restates, in numpy float64, the
network the CUDA kernels run (48 -> 64 -> 64 -> 3, ReLU) with the same
roundings to bfloat16 where the kernels store a tensor-core operand: the
features, the three weight matrices, the two hidden activations and the
output gradient.  The backward pass follows the same dataflow as the
kernels (bias gradients as column sums, ReLU masks from the rounded
activations).  It has no counterpart in the reference; it pins the GPU
forward and gradient.
"""
import numpy as np

N_FEAT, N_HID, N_OUT = 48, 64, 3
OFF_W1 = 0
OFF_B1 = OFF_W1 + N_FEAT * N_HID
OFF_W2 = OFF_B1 + N_HID
OFF_B2 = OFF_W2 + N_HID * N_HID
OFF_W3 = OFF_B2 + N_HID
OFF_B3 = OFF_W3 + N_HID * N_OUT
N_PARAMS = OFF_B3 + N_OUT


def bf16(a):
    """Round-to-nearest-even to bfloat16, returned as float32 (finite inputs)."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    r = ((b >> 16) & 1) + 0x7FFF
    return ((b + r) & 0xFFFF0000).astype(np.uint32).view(np.float32).reshape(a.shape)


def bf16_bits(a):
    """bfloat16 bit patterns (uint16) of float values."""
    return (bf16(a).view(np.uint32) >> 16).astype(np.uint16)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[OFF_W1:OFF_B1].reshape(N_FEAT, N_HID), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(N_HID, N_HID),
            p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3].reshape(N_HID, N_OUT), p[OFF_B3:N_PARAMS])


def forward(params, x, keep=False):
    """Prediction (n x 3) for features x (n x 48, float values already
    representable in bf16)."""
    W1, b1, W2, b2, W3, b3 = unpack(params)
    W1, W2, W3 = (bf16(w).astype(np.float64) for w in (W1, W2, W3))
    x = np.asarray(x, dtype=np.float64)
    h1 = bf16(np.maximum(x @ W1 + b1, 0.0)).astype(np.float64)
    h2 = bf16(np.maximum(h1 @ W2 + b2, 0.0)).astype(np.float64)
    y = h2 @ W3 + b3
    if keep:
        return y, (x, h1, h2, W1, W2, W3)
    return y


def loss_and_grad(params, x, t):
    """Mean squared error over the 3n outputs and its gradient, with the
    kernels' roundings of the backward operands."""
    n = x.shape[0]
    y, (x, h1, h2, W1, W2, W3) = forward(params, x, keep=True)
    e = y - np.asarray(t, dtype=np.float64)
    loss = float((e * e).sum() / (3 * n))
    dy = bf16(e * (2.0 / (3 * n))).astype(np.float64)
    g = np.zeros(N_PARAMS, np.float64)
    g[OFF_W3:OFF_B3] = (h2.T @ dy).ravel()
    g[OFF_B3:N_PARAMS] = dy.sum(0)
    dh2 = bf16(np.where(h2 > 0, dy @ W3.T, 0.0)).astype(np.float64)
    g[OFF_W2:OFF_B2] = (h1.T @ dh2).ravel()
    g[OFF_B2:OFF_W3] = dh2.sum(0)
    dh1 = bf16(np.where(h1 > 0, dh2 @ W2.T, 0.0)).astype(np.float64)
    g[OFF_W1:OFF_B1] = (x.T @ dh1).ravel()
    g[OFF_B1:OFF_W2] = dh1.sum(0)
    return loss, g


def loss_exact(params, x, t):
    """The same loss without any bf16 rounding (for finite differences)."""
    W1, b1, W2, b2, W3, b3 = unpack(params)
    x = np.asarray(x, dtype=np.float64)
    h1 = np.maximum(x @ W1 + b1, 0.0)
    h2 = np.maximum(h1 @ W2 + b2, 0.0)
    e = h2 @ W3 + b3 - t
    return float((e * e).sum() / e.size)


def grad_exact(params, x, t):
    """Analytic gradient of loss_exact (float64, no rounding)."""
    W1, b1, W2, b2, W3, b3 = unpack(params)
    x = np.asarray(x, dtype=np.float64)
    z1 = x @ W1 + b1
    h1 = np.maximum(z1, 0.0)
    z2 = h1 @ W2 + b2
    h2 = np.maximum(z2, 0.0)
    e = h2 @ W3 + b3 - t
    dy = 2.0 * e / e.size
    g = np.zeros(N_PARAMS, np.float64)
    g[OFF_W3:OFF_B3] = (h2.T @ dy).ravel()
    g[OFF_B3:N_PARAMS] = dy.sum(0)
    dh2 = (dy @ W3.T) * (z2 > 0)
    g[OFF_W2:OFF_B2] = (h1.T @ dh2).ravel()
    g[OFF_B2:OFF_W3] = dh2.sum(0)
    dh1 = (dh2 @ W2.T) * (z1 > 0)
    g[OFF_W1:OFF_B1] = (x.T @ dh1).ravel()
    g[OFF_B1:OFF_W2] = dh1.sum(0)
    return g
