"""NumPy FP64 restatement of the surrogate network (forward, loss, backward).

TEST INFRASTRUCTURE ONLY: the oracle that tests compare
anuga-cuda_gb300/csrc/swgpu_mlp.cu against; never imported by the package.

The network is 16 -> 256 -> 256 -> 256 -> 3 with ReLU after each hidden
layer.  Its rounding points follow the CUDA kernels: features in FP32,
rounded to BF16; weights rounded to BF16, biases read as FP32; each layer's
sum in FP64 (the kernels accumulate in FP32), ReLU, activations rounded to
BF16; the gradient of each hidden layer's pre-activation is rounded to BF16
(the kernels store it in BF16 for the tensor cores), and the weight and
bias gradients are sums of those rounded values.

Loss (mean over the rows): w_d (y0 - t0)^2 + w_a (y1 - t1)^2 +
w_e rho(|y0 - t0| - y2), rho(u) = u (q - [u < 0]) the pinball loss of the
quantile q = 0.9, so that the third output learns that quantile of the first
one's absolute error: |y0 - t0| is held constant in its term (no gradient
flows through it into y0).
"""
from __future__ import annotations

import numpy as np

F, H, OUT, NT, NP = 16, 256, 3, 2, 9
QUANTILE = 0.9
SHAPES = (("W1", (F, H)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, H)),
          ("b3", (H,)), ("W4", (H, OUT)), ("b4", (OUT,)))
NUM_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


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
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = p[o:o + n].reshape(shape)
        o += n
    return out


def flatten(d):
    return np.concatenate([d[k].ravel() for k, _ in SHAPES])


def features(scen, tri, rows, mu, isd):
    """FP32 normalised features of rows (scenario * ntri + triangle): the
    scenario's 9 parameters, the triangle's bed, x, y and distance to the
    inflow (tri [N][4] = x, y, bed, distance), then 3 zeros."""
    scen = np.asarray(scen, np.float32)
    tri = np.asarray(tri, np.float32)
    N = tri.shape[0]
    s, k = np.divmod(np.asarray(rows, np.int64), N)
    raw = np.zeros((len(rows), F), np.float32)
    raw[:, :NP] = scen[s]
    raw[:, 9], raw[:, 10], raw[:, 11], raw[:, 12] = tri[k, 2], tri[k, 0], tri[k, 1], tri[k, 3]
    return ((raw - np.asarray(mu, np.float32)) * np.asarray(isd, np.float32)).astype(np.float32)


def forward(params, x):
    """Outputs [n][3] and the hidden activations of BF16 inputs x [n][16]."""
    P = unflatten(params)
    W = [bf16(P[k]) for k in ("W1", "W2", "W3", "W4")]
    b = [P[k].astype(np.float32).astype(np.float64) for k in ("b1", "b2", "b3", "b4")]
    h1 = bf16(np.maximum(x @ W[0] + b[0], 0.0))
    h2 = bf16(np.maximum(h1 @ W[1] + b[1], 0.0))
    h3 = bf16(np.maximum(h2 @ W[2] + b[2], 0.0))
    y = h3 @ W[3] + b[3]
    return y, (h1, h2, h3), W


def forward_backward(params, scen, tri, rows, targets, mu, isd, w_depth=1.0, w_arrival=1.0,
                     w_error=1.0, frozen_error=None):
    """(outputs [n][3], loss, flat gradient) of the rows.  frozen_error, when
    given, replaces |y0 - t0| in the error term (a finite-difference check
    holds it at its value at the base point, as the gradient does)."""
    x = bf16(features(scen, tri, rows, mu, isd))
    y, (h1, h2, h3), W = forward(params, x)
    n = len(rows)
    t = np.asarray(targets, np.float64).reshape(-1, NT)[np.asarray(rows, np.int64)]
    e0 = y[:, 0] - t[:, 0]
    e1 = y[:, 1] - t[:, 1]
    err = np.abs(e0) if frozen_error is None else np.asarray(frozen_error, np.float64)
    u = err - y[:, 2]
    pin = np.where(u >= 0, QUANTILE * u, (QUANTILE - 1.0) * u)
    loss = float(np.sum(w_depth * e0 * e0 + w_arrival * e1 * e1 + w_error * pin) / n)
    d2 = w_error * np.where(u < 0, 1.0 - QUANTILE, -QUANTILE)
    dy = np.stack([2.0 * w_depth * e0, 2.0 * w_arrival * e1, d2], axis=1) / n
    dz3 = bf16((dy @ W[3].T) * (h3 > 0))
    dz2 = bf16((dz3 @ W[2].T) * (h2 > 0))
    dz1 = bf16((dz2 @ W[1].T) * (h1 > 0))
    g = {"W1": x.T @ dz1, "b1": dz1.sum(0), "W2": h1.T @ dz2, "b2": dz2.sum(0),
         "W3": h2.T @ dz3, "b3": dz3.sum(0), "W4": h3.T @ dy, "b4": dy.sum(0)}
    return y, loss, flatten(g)
