"""FP64 oracle of the learned sizer's MLP (12 -> 64 -> 64 -> 2, ReLU).

TEST INFRASTRUCTURE ONLY: the gradient check of the GPU forward/backward kernels
(pathfinder-cpp_gb300/csrc/pf_sizer.cu) compares against this.  Parameter layout
(float32 vector): W1[64][12] b1[64] W2[64][64] b2[64] W3[2][64] b3[2].  The GPU
forward uses the weights rounded to bf16 (round to nearest even), so does this.
Loss: mean over samples and outputs of the squared error.
"""
from __future__ import annotations

import numpy as np

N_IN, HIDDEN, N_OUT = 12, 64, 2
SHAPES = [("W1", (HIDDEN, N_IN)), ("b1", (HIDDEN,)), ("W2", (HIDDEN, HIDDEN)), ("b2", (HIDDEN,)),
          ("W3", (N_OUT, HIDDEN)), ("b3", (N_OUT,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    b = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def unpack(params: np.ndarray):
    out, o = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = params[o:o + n].reshape(shape)
        o += n
    return out


def pack(d) -> np.ndarray:
    return np.concatenate([np.asarray(d[name], np.float64).reshape(-1) for name, _ in SHAPES])


def forward(params: np.ndarray, x: np.ndarray, round_bf16: bool = True):
    p = unpack(bf16(params) if round_bf16 else params)
    p = {k: v.astype(np.float64) for k, v in p.items()}
    x = x.astype(np.float64)
    z1 = x @ p["W1"].T + p["b1"]
    h1 = np.maximum(z1, 0)
    z2 = h1 @ p["W2"].T + p["b2"]
    h2 = np.maximum(z2, 0)
    y = h2 @ p["W3"].T + p["b3"]
    return y, (x, z1, h1, z2, h2, p)


def loss_and_grad(params: np.ndarray, x: np.ndarray, t: np.ndarray, round_bf16: bool = True):
    y, (x, z1, h1, z2, h2, p) = forward(params, x, round_bf16)
    n = x.shape[0]
    e = y - t.astype(np.float64)
    loss = float((e * e).sum() / (n * N_OUT))
    dy = 2.0 * e / (n * N_OUT)
    g = {"W3": dy.T @ h2, "b3": dy.sum(0)}
    d2 = (dy @ p["W3"]) * (z2 > 0)
    g["W2"] = d2.T @ h1
    g["b2"] = d2.sum(0)
    d1 = (d2 @ p["W2"]) * (z1 > 0)
    g["W1"] = d1.T @ x
    g["b1"] = d1.sum(0)
    return loss, pack(g)


def predict(params: np.ndarray, x: np.ndarray) -> np.ndarray:
    return forward(params, x)[0]
