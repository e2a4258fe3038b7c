"""CPU restatement of the contention predictor's math (numpy).

TEST INFRASTRUCTURE ONLY: the GPU forward pass, gradients and selection of
ltpg_gb300/csrc/predictor.cu are checked against these functions.  Parameters
use the packed layout of include/ltpg.h (LTPG_PRED_PARAMS floats).  The GPU
feeds BF16 copies of W1, W2, the features and the first hidden layer to the
tensor cores and accumulates in FP32; `bf16=True` rounds the same tensors.
"""
import numpy as np

H, F = 64, 4
W1, B1 = 0, H * F
W2 = B1 + H
B2 = W2 + H * H
W3 = B2 + H
B3 = W3 + H
N_PARAM = B3 + 1


def unpack(p):
    p = np.asarray(p)
    return (p[W1:B1].reshape(H, F), p[B1:W2], p[W2:B2].reshape(H, H), p[B2:W3], p[W3:B3], p[B3])


def bf16(x):
    """Round float32 values to bfloat16 (round to nearest even), back as float32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def forward(p, x, bf=True, dtype=np.float32):
    w1, b1, w2, b2, w3, b3 = unpack(p)
    r = bf16 if bf else (lambda a: np.asarray(a, dtype=dtype))
    xb, w1b, w2b = r(x).astype(dtype), r(w1).astype(dtype), r(w2).astype(dtype)
    z1 = xb @ w1b.T + b1.astype(dtype)
    h1 = np.maximum(z1, 0)
    h1b = r(h1).astype(dtype)
    z2 = h1b @ w2b.T + b2.astype(dtype)
    h2 = np.maximum(z2, 0)
    y = h2 @ w3.astype(dtype) + dtype(b3)
    return y, (xb, w1b, w2b, h1, h1b, h2)


def gradients(p, x, t, bf=True, dtype=np.float32):
    """Gradient of mean((y - t)^2) with respect to the packed parameters."""
    w1, b1, w2, b2, w3, b3 = unpack(p)
    y, (xb, w1b, w2b, h1, h1b, h2) = forward(p, x, bf, dtype)
    n = len(x)
    dy = 2 * (y - np.asarray(t, dtype=dtype)) / n
    g = np.zeros(N_PARAM, dtype=dtype)
    g[W3:B3] = h2.T @ dy
    g[B3] = dy.sum()
    dz2 = np.outer(dy, w3.astype(dtype)) * (h2 > 0)
    g[W2:B2] = (dz2.T @ h1b).ravel()
    g[B2:W3] = dz2.sum(0)
    dz1 = (dz2 @ w2b) * (h1 > 0)
    g[W1:B1] = (dz1.T @ xb).ravel()
    g[B1:W2] = dz1.sum(0)
    return g


def loss(p, x, t, bf=False, dtype=np.float64):
    y, _ = forward(p, x, bf, dtype)
    return float(np.mean((y - t) ** 2))
