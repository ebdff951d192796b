"""CPU oracle of the source surrogate's MLP — test infrastructure only, never used by the product.

Forward pass, mean-squared-error loss and its gradients in FP64 numpy, in the flat parameter order
of sbz_surrogate_get_params (per layer W[nout][nin] row-major, then b[nout]); SiLU hidden
activations, identity output.  `bf16_operands=True` rounds the inputs and weights to bfloat16 first,
as the device GEMM reads them, so a comparison isolates the device's BF16 activations and FP32
accumulation.  The surrogate is specified by the build plan (an MLP over (cosmological parameters,
log k, log τ)); the reference has no learned part, so this oracle follows the standard
backpropagation equations, not a reference file.
"""
import numpy as np


def bf16_round(a):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def layer_sizes(nin, width, nhidden, nout):
    return [nin] + [width] * nhidden + [nout]


def unflatten(p, sizes):
    out, o = [], 0
    for a, b in zip(sizes[:-1], sizes[1:]):
        W = np.asarray(p[o:o + a * b], dtype=np.float64).reshape(b, a)
        o += a * b
        bias = np.asarray(p[o:o + b], dtype=np.float64)
        o += b
        out.append((W, bias))
    assert o == len(p)
    return out


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, X, sizes, bf16_operands=False):
    layers = unflatten(p, sizes)
    x = bf16_round(X) if bf16_operands else np.asarray(X, dtype=np.float64)
    xs, zs = [x], []
    for i, (W, b) in enumerate(layers):
        Wd = bf16_round(W) if bf16_operands else W
        z = x @ Wd.T + b
        zs.append(z)
        x = silu(z) if i < len(layers) - 1 else z
        xs.append(x)
    return xs, zs


def loss_and_grad(p, X, Y, sizes, bf16_operands=False):
    """Mean over rows and outputs of (y - t)², and its gradient in flat parameter order."""
    layers = unflatten(p, sizes)
    xs, zs = forward(p, X, sizes, bf16_operands)
    Y = np.asarray(Y, dtype=np.float64)
    n = Y.size
    r = xs[-1] - Y
    loss = float(np.sum(r * r) / n)
    d = 2.0 * r / n  # ∂loss/∂z of the output layer
    grads = []
    for i in range(len(layers) - 1, -1, -1):
        W, _ = layers[i]
        Wd = bf16_round(W) if bf16_operands else W
        grads.append((d.T @ xs[i], d.sum(axis=0)))
        if i > 0:
            d = (d @ Wd) * dsilu(zs[i - 1])
    flat = []
    for gW, gb in reversed(grads):
        flat.append(gW.ravel())
        flat.append(gb)
    return loss, np.concatenate(flat)
