"""CPU oracle of the learned-h MLP -- TEST INFRASTRUCTURE ONLY.

numpy restatement of ndspmhd_gb300/csrc/ndsph_mlp.cu: 6 -> 32 -> 32 -> 1,
tanh hidden layers, parameter vector W1[32][6], b1[32], W2[32][32], b2[32],
W3[32], b3.  ``forward_bf16`` emulates the tensor-core inference (BF16
weights, features and activations, FP32 accumulation); ``loss_and_grad``
is the training objective mean((out - y)^2) with BF16-rounded weights and
FP32/FP64 activations, differentiated by hand; ``fd_grad`` checks it by
central finite differences.
"""
import numpy as np

NIN = 6
OFF_W1 = 0
OFF_B1 = OFF_W1 + 32 * NIN
OFF_W2 = OFF_B1 + 32
OFF_B2 = OFF_W2 + 32 * 32
OFF_W3 = OFF_B2 + 32
OFF_B3 = OFF_W3 + 32
NPARAM = OFF_B3 + 1


def bf16(x):
    """Round float32 values to bfloat16 (round to nearest even), as float32."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    b = x.view(np.uint32).astype(np.uint64)
    r = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return r.astype(np.uint32).view(np.float32)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    W1 = p[OFF_W1:OFF_B1].reshape(32, NIN)
    b1 = p[OFF_B1:OFF_W2]
    W2 = p[OFF_W2:OFF_B2].reshape(32, 32)
    b2 = p[OFF_B2:OFF_W3]
    W3 = p[OFF_W3:OFF_B3]
    b3 = p[OFF_B3]
    return W1, b1, W2, b2, W3, b3


def forward_bf16(p, x):
    p32 = np.asarray(p, dtype=np.float32)
    W1, b1, W2, b2, W3, b3 = unpack(p32)
    W1 = bf16(W1).astype(np.float64); W2 = bf16(W2).astype(np.float64); W3 = bf16(W3).astype(np.float64)
    xb = bf16(np.asarray(x, dtype=np.float32)).astype(np.float64)
    h1 = np.tanh(xb @ W1.T + b1)
    h1 = bf16(h1.astype(np.float32)).astype(np.float64)
    h2 = np.tanh(h1 @ W2.T + b2)
    h2 = bf16(h2.astype(np.float32)).astype(np.float64)
    return h2 @ W3 + b3


def loss_and_grad(p, x, y):
    p32 = np.asarray(p, dtype=np.float32)
    W1, b1, W2, b2, W3, b3 = unpack(p32)
    W1 = bf16(W1).astype(np.float64); W2 = bf16(W2).astype(np.float64); W3 = bf16(W3).astype(np.float64)
    xb = bf16(np.asarray(x, dtype=np.float32)).astype(np.float64)
    y = np.asarray(y, dtype=np.float64)
    n = len(y)
    h1 = np.tanh(xb @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    out = h2 @ W3 + b3
    r = out - y
    loss = np.mean(r * r)
    dz3 = 2.0 * r / n
    g = np.zeros(NPARAM)
    g[OFF_W3:OFF_B3] = dz3 @ h2
    g[OFF_B3] = dz3.sum()
    dz2 = (dz3[:, None] * W3[None, :]) * (1 - h2 * h2)
    g[OFF_W2:OFF_B2] = (dz2.T @ h1).ravel()
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    dz1 = (dz2 @ W2) * (1 - h1 * h1)
    g[OFF_W1:OFF_B1] = (dz1.T @ xb).ravel()
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    return loss, g


def loss_only(p, x, y):
    """Loss with the weights taken as given (no BF16 rounding), for finite differences."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    xb = bf16(np.asarray(x, dtype=np.float32)).astype(np.float64)
    h1 = np.tanh(xb @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    out = h2 @ W3 + b3
    return np.mean((out - y) ** 2)


def fd_grad(p, x, y, eps=1e-6, idx=None):
    p = np.asarray(p, dtype=np.float64)
    idx = range(NPARAM) if idx is None else idx
    g = {}
    for q in idx:
        a = p.copy(); a[q] += eps
        b = p.copy(); b[q] -= eps
        g[q] = (loss_only(a, x, y) - loss_only(b, x, y)) / (2 * eps)
    return g
