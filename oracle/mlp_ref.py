"""CPU oracle of the rank predictor's network -- test infrastructure only.

float64 numpy forward / backward of the 8 -> 64 -> 64 -> 1 ReLU network with the
parameter layout of the GPU kernels: W1[8][64] b1[64] W2[64][64] b2[64] w3[64] b3,
loss = mean squared error, inputs normalised as (x - mean) / std.
"""
import numpy as np

NIN, NH = 8, 64
NPARAMS = NIN * NH + NH + NH * NH + NH + NH + 1


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + NIN * NH].reshape(NIN, NH); o += NIN * NH
    b1 = p[o:o + NH]; o += NH
    W2 = p[o:o + NH * NH].reshape(NH, NH); o += NH * NH
    b2 = p[o:o + NH]; o += NH
    w3 = p[o:o + NH]; o += NH
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


def forward(p, X, mean, std):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    std = np.where(np.asarray(std) > 0, std, 1.0)  # a constant feature is left unscaled
    x = (np.asarray(X, np.float64) - mean) / std
    z1 = x @ W1 + b1
    h1 = np.maximum(z1, 0)
    z2 = h1 @ W2 + b2
    h2 = np.maximum(z2, 0)
    return x, z1, h1, z2, h2, h2 @ w3 + b3


def loss_and_grad(p, X, y, mean, std):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    x, z1, h1, z2, h2, out = forward(p, X, mean, std)
    n = len(y)
    r = out - np.asarray(y, np.float64)
    loss = float((r * r).mean())
    dout = 2.0 * r / n
    dw3 = h2.T @ dout
    db3 = dout.sum()
    dz2 = np.outer(dout, w3) * (z2 > 0)
    dW2 = h1.T @ dz2
    db2 = dz2.sum(0)
    dz1 = (dz2 @ W2.T) * (z1 > 0)
    dW1 = x.T @ dz1
    db1 = dz1.sum(0)
    g = np.concatenate([dW1.ravel(), db1, dW2.ravel(), db2, dw3, [db3]])
    return loss, g
