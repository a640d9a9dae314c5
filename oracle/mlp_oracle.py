"""CPU oracle of the randomized route's model (test infrastructure only).

Restates, in float64 numpy, the network the library trains on the GPU
(opentebd-extended_gb300/csrc/mlp.cu): 67 -> 128 (ReLU) -> 128 (ReLU) -> 8, one
parameter vector W1 (128 x 67, row-major), b1, W2 (128 x 128), b2, W3 (8 x 128),
b3; loss = mean squared error over all outputs of all samples.  The library has
no reference counterpart here (the reference keeps chi singular values from a
full ZGESVD), so this oracle pins the kernels by their own mathematics: the
gradient below is the exact derivative of the loss, and tests compare the GPU
gradient with it.
"""
import numpy as np

N_IN, N_H, N_OUT = 67, 128, 8
SHAPES = [(N_H, N_IN), (N_H,), (N_H, N_H), (N_H,), (N_OUT, N_H), (N_OUT,)]
N_PARAMS = sum(int(np.prod(s)) for s in SHAPES)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    out, o = [], 0
    for s in SHAPES:
        n = int(np.prod(s))
        out.append(p[o:o + n].reshape(s))
        o += n
    return out


def forward(p, x):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    x = np.asarray(x, dtype=np.float64)
    h1 = np.maximum(x @ W1.T + b1, 0.0)
    h2 = np.maximum(h1 @ W2.T + b2, 0.0)
    return h2 @ W3.T + b3, (x, h1, h2)


def loss_grad(p, x, t):
    """(loss, gradient) of the mean squared error; the gradient in the order of p."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    y, (x, h1, h2) = forward(p, x)
    t = np.asarray(t, dtype=np.float64)
    n = len(x)
    e = y - t
    loss = float(np.sum(e * e) / (n * N_OUT))
    dy = 2.0 * e / (n * N_OUT)
    gW3, gb3 = dy.T @ h2, dy.sum(0)
    d2 = (dy @ W3) * (h2 > 0)
    gW2, gb2 = d2.T @ h1, d2.sum(0)
    d1 = (d2 @ W2) * (h1 > 0)
    gW1, gb1 = d1.T @ x, d1.sum(0)
    return loss, np.concatenate([g.ravel() for g in (gW1, gb1, gW2, gb2, gW3, gb3)])
