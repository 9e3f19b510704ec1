"""FP64 NumPy restatement of the library's MLP (test infrastructure only):
forward pass, masked MSE loss and its gradients, in the parameter layout of
pbag_mlp (per layer W [dout][din] row-major, then b [dout]), to check the
library's training kernels."""
import numpy as np


def unpack(params, dims):
    out, o = [], 0
    for din, dout in zip(dims[:-1], dims[1:]):
        W = params[o:o + din * dout].reshape(dout, din)
        o += din * dout
        b = params[o:o + dout]
        o += dout
        out.append((W, b))
    return out


def silu(z):
    return z / (1.0 + np.exp(-z))


def forward(params, dims, X):
    H = np.asarray(X, dtype=np.float64)
    layers = unpack(np.asarray(params, dtype=np.float64), dims)
    Zs, Hs = [], [H]
    for l, (W, b) in enumerate(layers):
        Z = H @ W.T + b
        Zs.append(Z)
        H = Z if l == len(layers) - 1 else silu(Z)
        Hs.append(H)
    return H, Zs, Hs


def loss_and_grads(params, dims, X, T, mask=None):
    Y, Zs, Hs = forward(params, dims, X)
    n, d = Y.shape
    m = np.ones_like(Y) if mask is None else np.asarray(mask, dtype=np.float64)
    E = (Y - T) * m
    loss = (E ** 2).sum() / (n * d)
    dZ = 2.0 * E / (n * d)
    layers = unpack(np.asarray(params, dtype=np.float64), dims)
    grads = [None] * len(layers)
    for l in range(len(layers) - 1, -1, -1):
        W, b = layers[l]
        if l < len(layers) - 1:
            z = Zs[l]
            s = 1.0 / (1.0 + np.exp(-z))
            dZ = dZ * s * (1.0 + z * (1.0 - s))
        gW = dZ.T @ Hs[l]
        gb = dZ.sum(axis=0)
        grads[l] = (gW, gb)
        dZ = dZ @ W
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return loss, flat
