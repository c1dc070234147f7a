"""Parameter vectors of the learned closure's network (layout of include/tlbm.h:
W1[32][8], b1[32], W2[32][32], b2[32], w3[32], b3)."""

from __future__ import annotations

import numpy as np

IN, HID = 8, 32
NPARAMS = HID * IN + HID + HID * HID + HID + HID + 1


def xavier(seed: int = 0) -> np.ndarray:
    """Glorot-uniform weights and small uniform biases, float32."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAMS)
    o = 0
    for fan_in, fan_out in ((IN, HID), (HID, HID), (HID, 1)):
        n = fan_in * fan_out
        p[o:o + n] = rng.uniform(-1, 1, n) * np.sqrt(6.0 / (fan_in + fan_out))
        o += n
        if fan_out > 1:
            p[o:o + fan_out] = rng.uniform(-0.1, 0.1, fan_out)
            o += fan_out
        else:
            p[o] = 0.05
            o += 1
    return p.astype(np.float32)
