"""CPU FP64 reference of the GPU multilayer perceptron's forward and backward
passes (test infrastructure only): the gradient check of mipt_gb300_mlp_*.

Same parameter layout (per layer W_l row-major [out][in], then b_l), ReLU
between layers, linear output, mean squared error over all outputs; the
products read the weights rounded to BF16 (round to nearest, ties to even, on
the upper 16 bits of the FP32 pattern), as the GPU does."""
import numpy as np


def bf16(x):
    b = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params, dims):
    out, o = [], 0
    for i in range(len(dims) - 1):
        n = dims[i] * dims[i + 1]
        W = params[o:o + n].reshape(dims[i + 1], dims[i])
        o += n
        b = params[o:o + dims[i + 1]]
        o += dims[i + 1]
        out.append((W, b))
    return out


def loss_grad(params, dims, x, t):
    layers = unpack(np.asarray(params, np.float32), dims)
    acts = [np.asarray(x, np.float64)]
    for li, (W, b) in enumerate(layers):
        z = acts[-1] @ bf16(W).T + b.astype(np.float64)
        acts.append(np.maximum(z, 0.0) if li + 1 < len(layers) else z)
    y = acts[-1]
    e = y - np.asarray(t, np.float64)
    loss = float(np.mean(e * e))
    dy = 2.0 * e / e.size
    grads = []
    for li in range(len(layers) - 1, -1, -1):
        W, b = layers[li]
        x_in = acts[li]
        gW = dy.T @ x_in
        gb = dy.sum(axis=0)
        grads.append((gW, gb))
        if li > 0:
            dy = (dy @ bf16(W)) * (x_in > 0)
    grads.reverse()
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return loss, flat
