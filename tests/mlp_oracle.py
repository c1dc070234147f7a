"""CPU oracle of the learned closure's network (test infrastructure).

The 8-32-32-1 tanh MLP of tlbm_gb300/csrc/mlp.cuh in FP64 numpy, with the same BF16 roundings
(weights, inputs and activations) and the same loss, mean of (y - t)^2 / 2.  With
``round_bf16=False`` it is the plain FP64 network, used to check its own gradient by finite
differences.
"""

import numpy as np

IN, HID = 8, 32
OW1 = 0
OB1 = OW1 + HID * IN
OW2 = OB1 + HID
OB2 = OW2 + HID * HID
OW3 = OB2 + HID
OB3 = OW3 + HID
NPARAMS = OB3 + 1


def bf16r(a):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p, round_bf16=True):
    p = np.asarray(p, dtype=np.float64)
    r = bf16r if round_bf16 else (lambda a: np.asarray(a, np.float64))
    # biases are FP32 on the GPU
    f32 = (lambda a: np.asarray(a, np.float32).astype(np.float64)) if round_bf16 else \
        (lambda a: np.asarray(a, np.float64))
    W1 = r(p[OW1:OB1]).reshape(HID, IN)
    b1 = f32(p[OB1:OW2])
    W2 = r(p[OW2:OB2]).reshape(HID, HID)
    b2 = f32(p[OB2:OW3])
    w3 = r(p[OW3:OB3])
    b3 = float(f32(p[OB3:OB3 + 1])[0])
    return W1, b1, W2, b2, w3, b3


def forward_backward(p, X, T, round_bf16=True):
    """Returns (mean loss, gradient[NPARAMS], predictions y)."""
    r = bf16r if round_bf16 else (lambda a: np.asarray(a, np.float64))
    W1, b1, W2, b2, w3, b3 = unpack(p, round_bf16)
    X = np.asarray(X, np.float64).reshape(-1, IN)
    T = np.asarray(T, np.float64).reshape(-1)
    n = len(T)
    x = r(X)
    # act(z) = BF16(tanh(z)) of the FP32 pre-activation (mlp.cuh)
    h1 = r(np.tanh(x @ W1.T + b1))
    h2 = r(np.tanh(h1 @ W2.T + b2))
    y = h2 @ w3 + b3
    dy = y - T
    loss = float(np.mean(0.5 * dy * dy))
    dz2 = dy[:, None] * w3[None, :] * (1.0 - h2 * h2)
    dz1 = (dz2 @ W2) * (1.0 - h1 * h1)
    g = np.empty(NPARAMS)
    g[OW1:OB1] = (dz1.T @ x).reshape(-1) / n
    g[OB1:OW2] = dz1.sum(0) / n
    g[OW2:OB2] = (dz2.T @ h1).reshape(-1) / n
    g[OB2:OW3] = dz2.sum(0) / n
    g[OW3:OB3] = (dy[:, None] * h2).sum(0) / n
    g[OB3] = dy.sum() / n
    return loss, g, y


def init_params(seed=0):
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAMS)
    p[OW1:OB1] = rng.uniform(-1, 1, HID * IN) * np.sqrt(6.0 / (IN + HID))
    p[OW2:OB2] = rng.uniform(-1, 1, HID * HID) * np.sqrt(6.0 / (2 * HID))
    p[OW3:OB3] = rng.uniform(-1, 1, HID) * np.sqrt(6.0 / (HID + 1))
    p[OB1:OW2] = rng.uniform(-0.1, 0.1, HID)
    p[OB2:OW3] = rng.uniform(-0.1, 0.1, HID)
    p[OB3] = 0.05
    return p.astype(np.float32)
