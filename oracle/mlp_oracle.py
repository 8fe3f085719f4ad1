"""CPU oracle (test infrastructure) of the Green-function surrogate network:
2 -> 128 -> 128 -> 128 -> 128 -> 6, SiLU on the hidden layers, weights used as
BF16 (round to nearest even) and everything else in FP64.  Parameter order as in
bem_mlp: W0 (128 x 2), b0, W1 (128 x 128), b1, ..., W4 (6 x 128), b4, W row-major
[out][in].  Only tests and bench.py's report call this module."""
import numpy as np

DIMS = (2, 128, 128, 128, 128, 6)


def bf16(a):
    """Round float32 values to bfloat16 (nearest, ties to even) and back."""
    a = np.asarray(a, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def unpack(params):
    out, o = [], 0
    for l in range(len(DIMS) - 1):
        i, n = DIMS[l], DIMS[l + 1]
        W = params[o:o + n * i].reshape(n, i)
        o += n * i
        b = params[o:o + n]
        o += n
        out.append((W, b))
    return out


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_d(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(params, x, quantize=True, act_bf16=False):
    """x: n x 2 normalised inputs; returns (y, pre-activations, activations).
    quantize=False uses the weights as given (for finite-difference checks);
    act_bf16=True also rounds every hidden activation to BF16, as the tensor-core
    inference (whose MMA operands are BF16) does."""
    a = np.asarray(x, dtype=np.float64)
    zs, acts = [], [a]
    layers = unpack(np.asarray(params, dtype=np.float64))
    for l, (W, b) in enumerate(layers):
        Wq = bf16(W).astype(np.float64) if quantize else W
        z = a @ Wq.T + b
        zs.append(z)
        a = silu(z) if l < len(layers) - 1 else z
        if act_bf16 and l < len(layers) - 1:
            a = bf16(a).astype(np.float64)
        acts.append(a)
    return a, zs, acts


def loss_and_grad(params, x, t, quantize=True):
    """MSE of the normalised outputs and its gradient with respect to the parameters
    (the products use the BF16 weights; the gradient is taken with respect to them)."""
    params = np.asarray(params, dtype=np.float64)
    y, zs, acts = forward(params, x, quantize)
    n = y.size
    loss = float(np.sum((y - t) ** 2) / n)
    dz = 2.0 * (y - t) / n
    layers = unpack(params)
    grads = []
    for l in range(len(layers) - 1, -1, -1):
        W, _ = layers[l]
        Wq = bf16(W).astype(np.float64) if quantize else W
        gW = dz.T @ acts[l]
        gb = dz.sum(axis=0)
        grads.append((gW, gb))
        if l == 0:
            break
        da = dz @ Wq
        dz = da * silu_d(zs[l - 1])
    grads.reverse()
    g = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return loss, g
