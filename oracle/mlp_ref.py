"""CPU restatement (numpy, float64) of the grid pruner's network for checking the CUDA kernels.

Test infrastructure only: the product trains and evaluates the network with its own kernels
(calchem_gb300/csrc/mlp.cu); this module is what their outputs and gradients are compared with.
The network and loss are the ones documented in mlp.cu: h1 = tanh(x W1 + b1),
h2 = tanh(h1 W2 + b2), y = h2 W3 + b3 with 16 inputs, 64 + 64 hidden units and 16 outputs, and the
masked mean squared error L = inv_count * sum mask (y - t)^2.  Parameters are one flat vector
W1 [16][64], b1, W2 [64][64], b2, W3 [64][16], b3.
"""

import numpy as np

N_IN, N_HID, N_OUT = 16, 64, 16
_SIZES = [("W1", (N_IN, N_HID)), ("b1", (N_HID,)), ("W2", (N_HID, N_HID)), ("b2", (N_HID,)),
          ("W3", (N_HID, N_OUT)), ("b3", (N_OUT,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in _SIZES)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    out, o = {}, 0
    for name, shape in _SIZES:
        k = int(np.prod(shape))
        out[name] = p[o:o + k].reshape(shape)
        o += k
    return out


def forward(p, X):
    w = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    h1 = np.tanh(X @ w["W1"] + w["b1"])
    h2 = np.tanh(h1 @ w["W2"] + w["b2"])
    return h2 @ w["W3"] + w["b3"], h1, h2


def loss_grad(p, X, T, M, inv_count):
    """(loss, flat gradient) of the masked mean squared error."""
    w = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    y, h1, h2 = forward(p, X)
    r = y - T
    loss = inv_count * float(np.sum(M * r * r))
    d3 = 2.0 * M * r * inv_count
    d2 = (d3 @ w["W3"].T) * (1.0 - h2 * h2)
    d1 = (d2 @ w["W2"].T) * (1.0 - h1 * h1)
    g = [X.T @ d1, d1.sum(0), h1.T @ d2, d2.sum(0), h2.T @ d3, d3.sum(0)]
    return loss, np.concatenate([a.ravel() for a in g])


def adam_step(p, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    p = p - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    return p, m, v
