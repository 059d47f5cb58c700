"""NumPy FP64 restatement of the surrogate MLP (forward, loss, backward).

TEST INFRASTRUCTURE ONLY: the oracle that tests compare
anuga-cuda_gb300/csrc/swgpu_mlp.cu against; never imported by the package.

The network and its rounding points follow the CUDA kernels: features in
FP32, rounded to BF16; weights rounded to BF16; each layer's sum in FP64
(the kernels accumulate in FP32), ReLU, activations rounded to BF16; the
gradient of layer 2's pre-activation is rounded to BF16 where it multiplies
W2 (the kernel feeds it to the tensor cores) and kept unrounded for the
weight and bias gradients.
"""
from __future__ import annotations

import numpy as np

F, H, OUT, NP = 16, 128, 2, 9


def bf16(a):
    """Round float32 values to the nearest BF16 (ties to even), as float64."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unflatten(p):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    out = {}
    for name, shape in (("W1", (F, H)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)),
                        ("W3", (H, OUT)), ("b3", (OUT,))):
        n = int(np.prod(shape))
        out[name] = p[o:o + n].reshape(shape)
        o += n
    return out


def flatten(d):
    return np.concatenate([d[k].ravel() for k in ("W1", "b1", "W2", "b2", "W3", "b3")])


def features(scen, tri, rows, mu, isd):
    """FP32 normalised features of rows (scenario * ntri + triangle)."""
    scen = np.asarray(scen, np.float32)
    tri = np.asarray(tri, np.float32)
    N = tri.shape[0]
    s, k = np.divmod(np.asarray(rows, np.int64), N)
    th = scen[s]
    x, y, z = tri[k, 0], tri[k, 1], tri[k, 2]
    dx, dy = x - th[:, 1], y - th[:, 2]
    r = np.sqrt(dx * dx + dy * dy).astype(np.float32)
    raw = np.zeros((len(rows), F), np.float32)
    raw[:, :NP] = th
    raw[:, 9], raw[:, 10], raw[:, 11], raw[:, 12] = z, x, y, r
    return ((raw - np.asarray(mu, np.float32)) * np.asarray(isd, np.float32)).astype(np.float32)


def forward_backward(params, scen, tri, rows, targets, mu, isd, w_depth=1.0, w_arrival=1.0):
    """(outputs [n][2], loss, flat gradient) of the rows."""
    P = unflatten(params)
    W1, W2, W3 = bf16(P["W1"]), bf16(P["W2"]), bf16(P["W3"])
    b1, b2, b3 = P["b1"].astype(np.float32), P["b2"].astype(np.float32), P["b3"].astype(np.float32)
    x = bf16(features(scen, tri, rows, mu, isd))
    a1 = bf16(np.maximum(x @ W1 + b1, 0.0))
    a2 = bf16(np.maximum(a1 @ W2 + b2, 0.0))
    y = a2 @ W3 + b3
    n = len(rows)
    t = np.asarray(targets, np.float64).reshape(-1, OUT)[np.asarray(rows, np.int64)]
    w = np.array([w_depth, w_arrival])
    e = y - t
    loss = float(np.sum(w * e * e) / n)
    dy = 2.0 * w * e / n
    dz2 = (dy @ W3.T) * (a2 > 0)
    dz1 = (bf16(dz2) @ W2.T) * (a1 > 0)
    g = {"W1": x.T @ dz1, "b1": dz1.sum(0), "W2": a1.T @ dz2, "b2": dz2.sum(0),
         "W3": a2.T @ dy, "b3": dy.sum(0)}
    return y, loss, flatten(g)
