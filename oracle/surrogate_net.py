"""FP64 CPU restatement of the far-field surrogate network -- TEST INFRASTRUCTURE ONLY.

Only tests/ may import this module.  It restates, in numpy, what the GPU
library's surrogate kernels compute (opsec_gpu/csrc/surrogate.cu), so that the
GPU forward pass and the training gradients can be checked against it:

  parameters   one network, FP32 master layout W1[128][16] b1 W2[128][128] b2
               W3[128][128] b3 w4[128] b4, 35336 floats (padded)
  forward      inputs and parameters enter as their BF16 values; z1 = x W1^T + b1,
               a1 = bf16(gelu(z1)), z2 = a1 W2^T + b2, a2 = bf16(gelu(z2)),
               z3 = a2 W3^T + b3, a3 = gelu(z3) (not rounded), out = a3 . w4 + b4;
               gelu is the tanh form 0.5 z (1 + tanh(sqrt(2/pi)(z + 0.044715 z^3)))
  loss         mean squared error; the gradient treats the BF16 roundings as the
               identity (the update is applied to the FP32 master weights)

The reference has no learned component: this restatement pins the GPU network
to its own definition, and `loss_and_grad` is itself checked against finite
differences of `loss` in the CPU tests.
"""
from __future__ import annotations

import numpy as np

IN, HID = 16, 128
OFF = {"W1": 0, "b1": 2048, "W2": 2176, "b2": 18560, "W3": 18688, "b3": 35072, "w4": 35200, "b4": 35328}
NPARAM = 35336
C = np.sqrt(2.0 / np.pi)


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    out = r.view(np.float32).astype(np.float64)
    return np.where(np.isfinite(f), out, f.astype(np.float64))


def unpack(p, rounded=True):
    p = np.asarray(p, dtype=np.float64)
    q = bf16(p) if rounded else p
    return {"W1": q[0:2048].reshape(HID, IN), "b1": q[2048:2176], "W2": q[2176:18560].reshape(HID, HID),
            "b2": q[18560:18688], "W3": q[18688:35072].reshape(HID, HID), "b3": q[35072:35200],
            "w4": q[35200:35328], "b4": q[35328]}


def gelu(z):
    return 0.5 * z * (1 + np.tanh(C * (z + 0.044715 * z ** 3)))


def gelu_grad(z):
    th = np.tanh(C * (z + 0.044715 * z ** 3))
    return 0.5 * (1 + th) + 0.5 * z * (1 - th ** 2) * C * (1 + 3 * 0.044715 * z ** 2)


def forward(p, x, rounded=True):
    w = unpack(p, rounded)
    r = bf16 if rounded else (lambda v: v)
    x = r(x)
    z1 = x @ w["W1"].T + w["b1"]
    a1 = r(gelu(z1))
    z2 = a1 @ w["W2"].T + w["b2"]
    a2 = r(gelu(z2))
    z3 = a2 @ w["W3"].T + w["b3"]
    a3 = gelu(z3)
    out = a3 @ w["w4"] + w["b4"]
    return out, (x, z1, a1, z2, a2, z3, a3, w)


def loss(p, x, y, rounded=True):
    out, _ = forward(p, x, rounded)
    return float(np.mean((out - y) ** 2))


def loss_and_grad(p, x, y, rounded=True):
    out, (x, z1, a1, z2, a2, z3, a3, w) = forward(p, x, rounded)
    n = len(y)
    dout = 2 * (out - y) / n
    g = np.zeros(NPARAM)
    g[OFF["w4"]:OFF["w4"] + HID] = a3.T @ dout
    g[OFF["b4"]] = dout.sum()
    dz3 = np.outer(dout, w["w4"]) * gelu_grad(z3)
    g[OFF["W3"]:OFF["W3"] + HID * HID] = (dz3.T @ a2).ravel()
    g[OFF["b3"]:OFF["b3"] + HID] = dz3.sum(0)
    dz2 = (dz3 @ w["W3"]) * gelu_grad(z2)
    g[OFF["W2"]:OFF["W2"] + HID * HID] = (dz2.T @ a1).ravel()
    g[OFF["b2"]:OFF["b2"] + HID] = dz2.sum(0)
    dz1 = (dz2 @ w["W2"]) * gelu_grad(z1)
    g[OFF["W1"]:OFF["W1"] + HID * IN] = (dz1.T @ x).ravel()
    g[OFF["b1"]:OFF["b1"] + HID] = dz1.sum(0)
    return float(np.mean((out - y) ** 2)), g


def init(seed):
    """Glorot-uniform weights (the first layer over its 12 used inputs), zero biases."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAM)

    def fill(off, nout, nin, used):
        a = np.sqrt(6.0 / (used + nout))
        m = rng.uniform(-a, a, size=(nout, nin))
        m[:, used:] = 0
        p[off:off + nout * nin] = m.ravel()

    fill(OFF["W1"], HID, IN, 12)
    fill(OFF["W2"], HID, HID, HID)
    fill(OFF["W3"], HID, HID, HID)
    fill(OFF["w4"], 1, HID, HID)
    return p.astype(np.float32)
