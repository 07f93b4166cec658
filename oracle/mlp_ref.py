"""Float64 reference of the cost-model MLP -- TEST INFRASTRUCTURE ONLY.

Checks the library's hand-written forward/backward kernels: same layout
(W1 [128][66], b1, W2 [128][128], b2, W3 [2][128], b3), same bf16 rounding of
the parameters the device computes with, mean squared error over the batch."""
import numpy as np

SHAPES = [(128, 66), (128,), (128, 128), (128,), (2, 128), (2,)]


def bf16_round(x: np.ndarray) -> np.ndarray:
    """float32 -> nearest bf16 (ties to even), returned as float64."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return (b.astype(np.uint32)).view(np.float32).astype(np.float64)


def unpack(params):
    out, o = [], 0
    for s in SHAPES:
        k = int(np.prod(s))
        out.append(params[o:o + k].reshape(s))
        o += k
    return out


def forward(params, x):
    W1, b1, W2, b2, W3, b3 = unpack(bf16_round(params))
    x = np.asarray(x, np.float64)
    z1 = x @ W1.T + b1
    h1 = np.maximum(z1, 0)
    z2 = h1 @ W2.T + b2
    h2 = np.maximum(z2, 0)
    return h2 @ W3.T + b3, (x, h1, h2)


def gradient(params, x, t):
    """Gradient of mean over rows of sum over outputs of (y - t)^2, and the summed squared error."""
    W1, b1, W2, b2, W3, b3 = unpack(bf16_round(params))
    y, (x, h1, h2) = forward(params, x)
    n = x.shape[0]
    e = y - np.asarray(t, np.float64)
    dy = 2 * e / n
    gW3 = dy.T @ h2
    gb3 = dy.sum(0)
    dh2 = (dy @ W3) * (h2 > 0)
    gW2 = dh2.T @ h1
    gb2 = dh2.sum(0)
    dh1 = (dh2 @ W2) * (h1 > 0)
    gW1 = dh1.T @ x
    gb1 = dh1.sum(0)
    g = np.concatenate([a.ravel() for a in (gW1, gb1, gW2, gb2, gW3, gb3)])
    return g, float((e * e).sum())


def forward_bf16_activations(params, x):
    """The tensor-core routing pass: inputs and hidden activations rounded to
    bf16 where they enter a multiply, fp32-or-better accumulation."""
    W1, b1, W2, b2, W3, b3 = unpack(bf16_round(params))
    r = lambda a: bf16_round(np.asarray(a, np.float32))
    h1 = r(np.maximum(r(x) @ W1.T + b1, 0))
    h2 = r(np.maximum(h1 @ W2.T + b2, 0))
    return h2 @ W3.T + b3
