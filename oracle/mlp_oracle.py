"""CPU oracle for the learned warm start's network (test infrastructure only).

A numpy restatement of the GPU network in scwatter_gb300/csrc/mlp.cu, in float64:
    h1 = relu(W1 x + b1), h2 = relu(W2 h1 + b2), y = W3 h2 + b3,
loss = mean((y - t)^2) over all outputs of the batch, and its gradients by hand-written
backpropagation.  The parameter vector layout matches scw_mlp_get_params:
W1 [width][n_in], b1, W2 [width][width], b2, W3 [n_out][width], b3.
The network has no counterpart in the reference; this oracle checks the GPU kernels'
forward pass and gradients.
"""
import numpy as np


def unpack(params, n_in, width, n_out):
    p = np.asarray(params, dtype=np.float64)
    shapes = [(width, n_in), (width,), (width, width), (width,), (n_out, width), (n_out,)]
    out, o = [], 0
    for s in shapes:
        k = int(np.prod(s))
        out.append(p[o:o + k].reshape(s))
        o += k
    return out


def forward(params, X, n_in, width, n_out):
    W1, b1, W2, b2, W3, b3 = unpack(params, n_in, width, n_out)
    X = np.asarray(X, dtype=np.float64)
    h1 = np.maximum(X @ W1.T + b1, 0.0)
    h2 = np.maximum(h1 @ W2.T + b2, 0.0)
    return h2 @ W3.T + b3, (h1, h2)


def loss_and_grad(params, X, T, n_in, width, n_out):
    W1, b1, W2, b2, W3, b3 = unpack(params, n_in, width, n_out)
    X = np.asarray(X, dtype=np.float64)
    Y, (h1, h2) = forward(params, X, n_in, width, n_out)
    d = Y - np.asarray(T, dtype=np.float64)
    loss = float(np.mean(d * d))
    dY = 2.0 * d / d.size
    gW3 = dY.T @ h2
    gb3 = dY.sum(0)
    dh2 = (dY @ W3) * (h2 > 0)
    gW2 = dh2.T @ h1
    gb2 = dh2.sum(0)
    dh1 = (dh2 @ W2) * (h1 > 0)
    gW1 = dh1.T @ X
    gb1 = dh1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g
