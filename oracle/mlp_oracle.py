"""TEST INFRASTRUCTURE (oracle): float64 CPU reference of the p* MLP.

Forward and backward of the 4-64-64-64-1 SiLU network with the parameter
layout of mlh_pstar_* (W1[64][4], b1, W2[64][64], b2, W3[64][64], b3, W4[64],
b4), used to check the GPU's tensor-core forward pass and gradients.  The
weights are rounded to bfloat16 first, as the GPU uses them.
"""
import numpy as np


def bf16(a):
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    # round to nearest even on the 16 dropped bits
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(w, round_weights=True):
    w = np.asarray(w, dtype=np.float64)
    o = 0
    out = {}
    for name, shape in (("W1", (64, 4)), ("b1", (64,)), ("W2", (64, 64)), ("b2", (64,)), ("W3", (64, 64)),
                        ("b3", (64,)), ("W4", (64,)), ("b4", (1,))):
        n = int(np.prod(shape))
        v = w[o:o + n].reshape(shape)
        if round_weights and name in ("W1", "W2", "W3"):
            v = bf16(v)
        out[name] = v
        o += n
    return out


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(w, x):
    p = unpack(w)
    x = bf16(np.asarray(x, dtype=np.float32).reshape(-1, 4))
    z1 = x @ p["W1"].T + p["b1"]
    h1 = silu(z1)
    z2 = h1 @ p["W2"].T + p["b2"]
    h2 = silu(z2)
    z3 = h2 @ p["W3"].T + p["b3"]
    h3 = silu(z3)
    y = h3 @ p["W4"] + p["b4"][0]
    return y, (x, z1, h1, z2, h2, z3, h3)


def loss_and_grad(w, x, t):
    p = unpack(w)
    y, (x, z1, h1, z2, h2, z3, h3) = forward(w, x)
    t = np.asarray(t, dtype=np.float64)
    n = len(t)
    err = y - t
    loss = np.mean(err ** 2)
    dy = 2.0 * err / n
    dW4 = h3.T @ dy
    db4 = np.array([dy.sum()])
    dz3 = np.outer(dy, p["W4"]) * silu_grad(z3)
    dW3 = dz3.T @ h2
    db3 = dz3.sum(0)
    dz2 = (dz3 @ p["W3"]) * silu_grad(z2)
    dW2 = dz2.T @ h1
    db2 = dz2.sum(0)
    dz1 = (dz2 @ p["W2"]) * silu_grad(z1)
    dW1 = dz1.T @ x
    db1 = dz1.sum(0)
    g = np.concatenate([dW1.ravel(), db1, dW2.ravel(), db2, dW3.ravel(), db3, dW4, db4])
    return loss, g


SLICES = {"W1": (0, 256), "b1": (256, 320), "W2": (320, 4416), "b2": (4416, 4480), "W3": (4480, 8576),
          "b3": (8576, 8640), "W4": (8640, 8704), "b4": (8704, 8705)}
