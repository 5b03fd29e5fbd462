"""numpy reference of the learned-guess MLP (6 -> 64 -> 64 -> 1, ReLU) and of the gradient its
tensor-core training kernel computes.

With rounded=True the reference rounds to bfloat16 exactly where the kernel feeds the tensor
cores (weights, inputs, hidden activations, the back-propagated errors of the weight-gradient and
hidden-error products) and accumulates in float64; with rounded=False it is the plain float64
model whose gradient a finite-difference check validates.
"""
import numpy as np

H, K1, NIN = 64, 16, 6
OFF_W1, OFF_B1 = 0, H * K1
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H
NPARAM = OFF_B3 + 1
BLOCKS = {"W1": slice(OFF_W1, OFF_B1), "b1": slice(OFF_B1, OFF_W2), "W2": slice(OFF_W2, OFF_B2),
          "b2": slice(OFF_B2, OFF_W3), "W3": slice(OFF_W3, OFF_B3), "b3": slice(OFF_B3, NPARAM)}


def bf16(a):
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    b = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return b.astype(np.uint32).view(np.float32)


def he_params(rng):
    p = np.zeros(NPARAM, dtype=np.float32)
    w1 = np.zeros((H, K1), dtype=np.float32)
    w1[:, :NIN] = rng.standard_normal((H, NIN)) * np.sqrt(2.0 / NIN)
    p[BLOCKS["W1"]] = w1.ravel()
    p[BLOCKS["W2"]] = (rng.standard_normal(H * H) * np.sqrt(2.0 / H)).astype(np.float32)
    p[BLOCKS["W3"]] = (rng.standard_normal(H) * np.sqrt(1.0 / H)).astype(np.float32)
    p[BLOCKS["b1"]] = rng.standard_normal(H) * 0.1
    p[BLOCKS["b2"]] = rng.standard_normal(H) * 0.1
    p[BLOCKS["b3"]] = 0.05
    return p


def loss_grad(params, x, t, rounded=True):
    """Loss sum((y - t)^2) / (2 n) and its gradient with respect to the parameter vector."""
    r = (lambda a: bf16(a).astype(np.float64)) if rounded else (lambda a: np.asarray(a, dtype=np.float64))
    p = np.asarray(params, dtype=np.float64 if not rounded else np.float32)
    W1 = r(p[BLOCKS["W1"]]).reshape(H, K1)[:, :NIN]
    W2 = r(p[BLOCKS["W2"]]).reshape(H, H)
    W3 = r(p[BLOCKS["W3"]])
    b1, b2 = np.asarray(p[BLOCKS["b1"]], np.float64), np.asarray(p[BLOCKS["b2"]], np.float64)
    b3 = float(p[OFF_B3])
    X = r(x)
    t = np.asarray(t, dtype=np.float64)
    n = len(t)
    z1 = X @ W1.T + b1
    h1 = r(np.maximum(z1, 0.0))
    z2 = h1 @ W2.T + b2
    h2 = r(np.maximum(z2, 0.0))
    y = h2 @ W3 + b3
    d = y - t
    loss = float((d * d).sum() / (2 * n))
    dy = d / n
    dz2 = (z2 > 0) * dy[:, None] * W3[None, :]
    dh1 = r(dz2) @ W2
    dz1 = (z1 > 0) * dh1
    g = np.zeros(NPARAM)
    gw1 = np.zeros((H, K1))
    gw1[:, :NIN] = r(dz1).T @ X
    g[BLOCKS["W1"]] = gw1.ravel()
    g[BLOCKS["b1"]] = dz1.sum(0)
    g[BLOCKS["W2"]] = (r(dz2).T @ h1).ravel()
    g[BLOCKS["b2"]] = dz2.sum(0)
    g[BLOCKS["W3"]] = h2.T @ dy
    g[OFF_B3] = dy.sum()
    return loss, g
