"""Float64 reference of the surrogate MLP ensemble (test infrastructure only:
the checker of the GPU's forward and backward kernels, never on the product path).

Architecture per member m: z1 = x W1[m]^T + b1[m], h1 = GELU(z1), z2 = h1 W2[m]^T + b2[m],
h2 = GELU(z2), y = h2 . w3[m] + b3[m]; loss_m = mean_b (y - t)^2. GELU is the tanh
form 0.5 z (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3))) (exact tanh here). Parameters are the flat layout of lmc_mlp_get_params:
W1 [M*H][in], b1 [M*H], W2 [M][H][H], b2 [M*H], w3 [M*H], b3 [M]."""
from __future__ import annotations

import math

import numpy as np

def bf16_round(a: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def bf16_bits_to_float(bits: np.ndarray) -> np.ndarray:
    return (np.asarray(bits, np.uint16).astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def unpack(p: np.ndarray, in_features: int, hidden: int, members: int):
    M, H, K = members, hidden, in_features
    o = 0
    W1 = p[o:o + M * H * K].reshape(M * H, K); o += M * H * K
    b1 = p[o:o + M * H]; o += M * H
    W2 = p[o:o + M * H * H].reshape(M, H, H); o += M * H * H
    b2 = p[o:o + M * H].reshape(M, H); o += M * H
    w3 = p[o:o + M * H].reshape(M, H); o += M * H
    b3 = p[o:o + M]
    return W1, b1, W2, b2, w3, b3


_C = math.sqrt(2.0 / math.pi)


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(_C * (z + 0.044715 * z ** 3)))


def gelu_grad(z):
    t = np.tanh(_C * (z + 0.044715 * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * _C * (1.0 + 3 * 0.044715 * z * z)


def forward_backward(p, x, t, in_features, hidden, members, bf16_weights=True):
    """Loss per member and the flat gradient (float64). With bf16_weights the
    matrices W1 and W2 are rounded to bfloat16 as the GPU's GEMMs read them."""
    p = np.asarray(p, np.float64)
    W1, b1, W2, b2, w3, b3 = unpack(p, in_features, hidden, members)
    if bf16_weights:
        W1, W2 = bf16_round(W1), bf16_round(W2)
    x = np.asarray(x, np.float64)
    B, M, H = x.shape[0], members, hidden
    z1 = x @ W1.T + b1                    # [B][M*H]
    h1 = gelu(z1)
    grads, losses = [], []
    gW1 = np.zeros_like(W1); gb1 = np.zeros_like(b1)
    gW2 = np.zeros_like(W2); gb2 = np.zeros_like(b2)
    gw3 = np.zeros_like(w3); gb3 = np.zeros_like(b3)
    for m in range(M):
        sl = slice(m * H, (m + 1) * H)
        z2 = h1[:, sl] @ W2[m].T + b2[m]
        h2 = gelu(z2)
        y = h2 @ w3[m] + b3[m]
        d = y - t
        losses.append(float(np.mean(d * d)))
        dy = 2.0 * d / B
        gw3[m] = h2.T @ dy
        gb3[m] = dy.sum()
        dz2 = np.outer(dy, w3[m]) * gelu_grad(z2)
        gW2[m] = dz2.T @ h1[:, sl]
        gb2[m] = dz2.sum(0)
        dz1 = (dz2 @ W2[m]) * gelu_grad(z1[:, sl])
        gW1[sl] = dz1.T @ x
        gb1[sl] = dz1.sum(0)
    flat = np.concatenate([gW1.ravel(), gb1.ravel(), gW2.ravel(), gb2.ravel(), gw3.ravel(), gb3.ravel()])
    return np.array(losses), flat


def predict(p, x, in_features, hidden, members, bf16_weights=True):
    """Per-member outputs y [members][B] (float64, standardised label units)."""
    p = np.asarray(p, np.float64)
    W1, b1, W2, b2, w3, b3 = unpack(p, in_features, hidden, members)
    if bf16_weights:
        W1, W2 = bf16_round(W1), bf16_round(W2)
    h1 = gelu(np.asarray(x, np.float64) @ W1.T + b1)
    out = []
    for m in range(members):
        sl = slice(m * hidden, (m + 1) * hidden)
        out.append(gelu(h1[:, sl] @ W2[m].T + b2[m]) @ w3[m] + b3[m])
    return np.array(out)
