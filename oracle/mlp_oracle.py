"""FP64 restatement of the learned correction's MLP (test infrastructure).

TEST INFRASTRUCTURE ONLY: the checker for the engine's BF16 tensor-core
training and inference kernels (nbody_gb300/csrc/nbg_mlp.cuh,
nbg_learned.cu).  The correction has no counterpart in the reference.

Network 16 -> 64 -> 64 -> 3, GELU in the tanh form
0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))) (Hendrycks & Gimpel 2016)
after both hidden layers.  The three outputs c are coefficients of vectors
built from the sample's features x (the engine's head, apply_head in
nbg_learned.cu): g = c0 u/|u| + c1 Q u/|u| + c2 o, with u = x[0:3],
1/|u| = x[12], Q the symmetric matrix of x[3:9] (xx, yy, zz, xy, xz, yz) and
o = x[13:16].  loss = sum over samples of |g - t|^2, gradients of the mean
loss (sum / count).  Parameter layout (flat, k-major): W1[16][64], b1[64],
W2[64][64], b2[64], W3[64][3], b3[3].
"""
from __future__ import annotations

import numpy as np

IN, H, OUT = 16, 64, 3
OFF_W1 = 0
OFF_B1 = OFF_W1 + IN * H
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H * OUT
N_PARAMS = OFF_B3 + OUT
GC = np.sqrt(2.0 / np.pi)
GA = 0.044715


def unpack(w):
    w = np.asarray(w, dtype=np.float64)
    return (w[OFF_W1:OFF_B1].reshape(IN, H), w[OFF_B1:OFF_W2], w[OFF_W2:OFF_B2].reshape(H, H),
            w[OFF_B2:OFF_W3], w[OFF_W3:OFF_B3].reshape(H, OUT), w[OFF_B3:N_PARAMS])


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(GC * (z + GA * z ** 3)))


def gelu_grad(z):
    t = np.tanh(GC * (z + GA * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * GC * (1.0 + 3.0 * GA * z * z)


def forward(w, x):
    W1, b1, W2, b2, W3, b3 = unpack(w)
    z1 = x @ W1 + b1
    a1 = gelu(z1)
    z2 = a1 @ W2 + b2
    a2 = gelu(z2)
    return a2 @ W3 + b3


def basis(x):
    """[B, 3, 3]: basis[s, i] is the i-th head vector of sample s."""
    x = np.asarray(x, dtype=np.float64)
    uh = x[:, 0:3] * x[:, 12:13]
    xx, yy, zz, xy, xz, yz = (x[:, k] for k in range(3, 9))
    qu = np.stack([xx * uh[:, 0] + xy * uh[:, 1] + xz * uh[:, 2],
                   xy * uh[:, 0] + yy * uh[:, 1] + yz * uh[:, 2],
                   xz * uh[:, 0] + yz * uh[:, 1] + zz * uh[:, 2]], axis=1)
    return np.stack([uh, qu, x[:, 13:16]], axis=1)


def head(x, c):
    """g = sum_i c_i basis_i (the correction in units of m / s^2)."""
    return np.einsum("si,sik->sk", np.asarray(c, dtype=np.float64), basis(x))


def loss_grad(w, x, t):
    """(sum of squared errors, gradient of the mean loss)."""
    x = np.asarray(x, dtype=np.float64)
    t = np.asarray(t, dtype=np.float64)[:, :OUT]
    W1, b1, W2, b2, W3, b3 = unpack(w)
    B = x.shape[0]
    z1 = x @ W1 + b1
    a1 = gelu(z1)
    z2 = a1 @ W2 + b2
    a2 = gelu(z2)
    c = a2 @ W3 + b3
    bs = basis(x)
    e = np.einsum("si,sik->sk", c, bs) - t
    dy = np.einsum("sk,sik->si", 2.0 * e / B, bs)
    g = np.zeros(N_PARAMS)
    g[OFF_W3:OFF_B3] = (a2.T @ dy).ravel()
    g[OFF_B3:N_PARAMS] = dy.sum(axis=0)
    dz2 = (dy @ W3.T) * gelu_grad(z2)
    g[OFF_W2:OFF_B2] = (a1.T @ dz2).ravel()
    g[OFF_B2:OFF_W3] = dz2.sum(axis=0)
    dz1 = (dz2 @ W2.T) * gelu_grad(z1)
    g[OFF_W1:OFF_B1] = (x.T @ dz1).ravel()
    g[OFF_B1:OFF_W2] = dz1.sum(axis=0)
    return float((e * e).sum()), g


def bf16(a):
    """Round to bfloat16 (nearest even), returned as float64."""
    a = np.asarray(a, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)
