"""CPU oracle of the mean-field extrapolator MLP (test infrastructure only).

Restates the GPU network of macaw_gb300/csrc/mlp.cu in NumPy with the same
rounding points: BF16 copies of the weights in the forward pass, BF16 storage of
the hidden activations, FP32 inputs and outputs, tanh hidden layers, linear
output, mean-squared-error loss.  Used to check the hand-written forward and
backward kernels.
"""
import numpy as np


def bf16(x):
    """Round float32 to bfloat16 (nearest, ties to even) and back to float32."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r.astype(np.uint32)).view(np.float32)


def unflatten(params, widths):
    out, off = [], 0
    for k, n in zip(widths[:-1], widths[1:]):
        W = params[off:off + n * k].reshape(n, k)
        off += n * k
        b = params[off:off + n]
        off += n
        out.append((W, b))
    return out


def forward(params, widths, X):
    layers = unflatten(np.asarray(params, np.float32), widths)
    acts = [np.asarray(X, np.float32)]
    h = acts[0]
    for i, (W, b) in enumerate(layers):
        z = h.astype(np.float64) @ bf16(W).astype(np.float64).T + b
        if i + 1 < len(layers):
            h = bf16(np.tanh(z).astype(np.float32))
        else:
            h = z.astype(np.float32)
        acts.append(h)
    return acts


def loss_and_grad(params, widths, X, T):
    layers = unflatten(np.asarray(params, np.float32), widths)
    acts = forward(params, widths, X)
    Y = acts[-1]
    n = Y.size
    dY = (2.0 * (Y.astype(np.float64) - T) / n)
    loss = float(np.mean((Y.astype(np.float64) - T) ** 2))
    grads = [None] * len(layers)
    g = dY
    for i in range(len(layers) - 1, -1, -1):
        W, _ = layers[i]
        gW = g.T @ acts[i].astype(np.float64)
        gb = g.sum(axis=0)
        grads[i] = (gW, gb)
        if i == 0:
            break
        dh = g @ bf16(W).astype(np.float64)
        h = acts[i].astype(np.float64)
        g = dh * (1.0 - h * h)
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return loss, flat
