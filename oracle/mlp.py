"""CPU oracle of the warm-start MLP (TEST INFRASTRUCTURE ONLY).

FP64 numpy forward and backward of the 66 -> 256 -> 256 -> 256 -> 2 GELU
network of ``picca_gb300.learned`` and its MSE loss, and one Adam step. With
``quantize=True`` the inputs, weights, hidden activations and back-propagated
gradients are rounded to bfloat16 at the points where the GPU stores them in
BF16, so the comparison isolates the kernels' arithmetic (FP32 accumulation)
from the storage format. The reference has no counterpart.
"""

import numpy as np
from scipy.special import erf


def bf16(x):
    """Round-to-nearest-even to bfloat16, returned as float64."""
    a = np.asarray(x, dtype=np.float32)
    bits = a.view(np.uint32).astype(np.uint64)
    rounding = ((bits >> 16) & 1) + 0x7FFF
    out = ((bits + rounding) >> 16) << 16
    return out.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2 * np.pi)


def forward(x, weights, quantize=False):
    """weights: list of (W [in, out], b [out]). Returns y and activations."""
    q = bf16 if quantize else (lambda v: np.asarray(v, dtype=np.float64))
    h = q(x)
    acts = {"x": h}
    for layer in range(3):
        w, b = weights[layer]
        z = h @ q(w) + b
        acts[f"z{layer}"] = z
        h = q(gelu(z))
        acts[f"h{layer}"] = h
    w, b = weights[3]
    y = h @ q(w) + b
    return y, acts


def backward(acts, y, target, weights, quantize=False):
    """Gradients of mean((y - t)^2 summed over outputs) for every (W, b)."""
    q = bf16 if quantize else (lambda v: np.asarray(v, dtype=np.float64))
    m = y.shape[0]
    dz = q(2.0 * (y - target) / m)
    grads = [None] * 4
    for layer in (3, 2, 1, 0):
        h_in = acts["x"] if layer == 0 else acts[f"h{layer - 1}"]
        grads[layer] = (h_in.T @ dz, dz.sum(axis=0))
        if layer == 0:
            break
        w, _ = weights[layer]
        dz = q((dz @ q(w).T) * gelu_grad(acts[f"z{layer - 1}"]))
    loss = np.sum((y - target) ** 2) / m
    return grads, loss


def adam(param, grad, m1, m2, step, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.0):
    g = grad + weight_decay * param
    m1 = beta1 * m1 + (1 - beta1) * g
    m2 = beta2 * m2 + (1 - beta2) * g * g
    mh = m1 / (1 - beta1**step)
    vh = m2 / (1 - beta2**step)
    return param - lr * mh / (np.sqrt(vh) + eps), m1, m2
