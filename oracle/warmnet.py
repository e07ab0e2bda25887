"""CPU reference of the warm-start network (numpy, FP64).

TEST INFRASTRUCTURE ONLY: the GPU network's forward pass and gradients are
checked against it; the product never imports it.  The network has no
counterpart in the MRFMap reference: it is this project's own learned warm
start (three 3x3x3 convolutions over 8^3 bricks, 4 -> 16 -> 16 -> 1
channels, ReLU between, zeros beyond the brick faces).

``bf16=True`` rounds to bfloat16 at the points where the GPU kernels hold
bfloat16 operands (inputs, weights, stored activations and activation
gradients), so the two agree to accumulation-order differences;
``bf16=False`` is the exact FP64 network used to pin the analytic gradients
against finite differences.
"""
from __future__ import annotations

import numpy as np

C0, C1, C2, C3 = 4, 16, 16, 1
SHAPES = [("W1", (27, C0, C1)), ("b1", (C1,)), ("W2", (27, C1, C2)), ("b2", (C2,)),
          ("W3", (27, C2, C3)), ("b3", (C3,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)
TAPS = [(t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1) for t in range(27)]


def to_bf16(x) -> np.ndarray:
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float64)
    out, o = {}, 0
    for name, shp in SHAPES:
        n = int(np.prod(shp))
        out[name] = p[o:o + n].reshape(shp)
        o += n
    return out


def pack(d) -> np.ndarray:
    return np.concatenate([np.asarray(d[name], np.float64).ravel() for name, _ in SHAPES])


def _shift(X, d):
    """X[b, x+dx, y+dy, z+dz] with zeros outside the brick; X (nb,8,8,8,C)."""
    out = np.zeros_like(X)
    dx, dy, dz = d
    src = [slice(max(0, k), 8 + min(0, k)) for k in (dx, dy, dz)]
    dst = [slice(max(0, -k), 8 + min(0, -k)) for k in (dx, dy, dz)]
    out[:, dst[0], dst[1], dst[2]] = X[:, src[0], src[1], src[2]]
    return out


def conv(X, W):
    """Y[v] = sum_tap X[v + d(tap)] @ W[tap]; X (nb,8,8,8,Ci), W (27,Ci,Co)."""
    Y = np.zeros(X.shape[:4] + (W.shape[2],))
    for t, d in enumerate(TAPS):
        Y += _shift(X, d) @ W[t]
    return Y


def conv_input_grad(dZ, W):
    """dX[u] = sum_tap dZ[u - d(tap)] @ W[tap].T"""
    dX = np.zeros(dZ.shape[:4] + (W.shape[1],))
    for t, d in enumerate(TAPS):
        dX += _shift(dZ, tuple(-k for k in d)) @ W[t].T
    return dX


def conv_weight_grad(X, dZ):
    """dW[tap] = sum_v X[v + d(tap)]^T dZ[v]"""
    ci, co = X.shape[-1], dZ.shape[-1]
    dW = np.zeros((27, ci, co))
    Zf = dZ.reshape(-1, co)
    for t, d in enumerate(TAPS):
        dW[t] = _shift(X, d).reshape(-1, ci).T @ Zf
    return dW


def forward(params, feat, bf16=True):
    """feat (nb, 512, 4) -> (prediction (nb, 512), cache)"""
    r = to_bf16 if bf16 else (lambda a: np.asarray(a, np.float64))
    P = unpack(params)
    nb = feat.shape[0]
    X0 = r(feat).reshape(nb, 8, 8, 8, C0)
    A1 = r(np.maximum(conv(X0, r(P["W1"])) + P["b1"], 0.0))
    A2 = r(np.maximum(conv(A1, r(P["W2"])) + P["b2"], 0.0))
    Y = conv(A2, r(P["W3"]))[..., 0] + P["b3"][0]
    return Y.reshape(nb, 512), dict(X0=X0, A1=A1, A2=A2, P=P)


def gradients(params, feat, target, weight, norm, bf16=True):
    """loss = sum w (y - t)^2 / norm and its gradient (packed like params)."""
    r = to_bf16 if bf16 else (lambda a: np.asarray(a, np.float64))
    Y, c = forward(params, feat, bf16)
    nb = feat.shape[0]
    e = Y - target
    loss = float((weight * e * e).sum() / norm)
    dy = r((2.0 * weight * e / norm).reshape(nb, 8, 8, 8, 1))
    P = c["P"]
    g = {}
    g["W3"] = conv_weight_grad(c["A2"], dy)
    g["b3"] = dy.sum(axis=(0, 1, 2, 3))
    dZ2 = r(conv_input_grad(dy, r(P["W3"])) * (c["A2"] > 0))
    g["W2"] = conv_weight_grad(c["A1"], dZ2)
    g["b2"] = dZ2.sum(axis=(0, 1, 2, 3))
    dZ1 = r(conv_input_grad(dZ2, r(P["W2"])) * (c["A1"] > 0))
    g["W1"] = conv_weight_grad(c["X0"], dZ1)
    g["b1"] = dZ1.sum(axis=(0, 1, 2, 3))
    return loss, pack(g)
