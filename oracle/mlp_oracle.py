"""CPU oracle of the learned-splitting importance network (test
infrastructure only: the tests compare the engine's GPU kernels with it).

The network: 8 standardised features -> 64 -> 64 -> 64 -> 1 with SiLU hidden
units; the output is the log-odds of the label.  Parameters are one flat
FP32 vector, W1[64][8] b1 W2[64][64] b2 W3[64][64] b3 W4[64] b4, and the
forward pass uses them rounded to BF16 (round to nearest even), as the GPU
kernels store them.  Loss: mean binary cross-entropy with logits.  Computed
in float64 here; the GPU accumulates in FP32.

round_act=True restates the tensor-core kernels' operand rounding: the
standardised inputs, every hidden activation h and silu'(a) are rounded to
BF16 before they enter a product, and so are the deltas d1..d3 of the
backward pass (the weight gradients are d^T h of those BF16 values); the
output delta dz and all sums stay in full precision.
"""
from __future__ import annotations

import numpy as np

F, H = 8, 64
SIZES = [("W1", (H, F)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, H)),
         ("b3", (H,)), ("W4", (H,)), ("b4", (1,))]
NPARAM = sum(int(np.prod(s)) for _, s in SIZES)


def bf16(x: np.ndarray) -> np.ndarray:
    """FP32 -> BF16 (round to nearest even) -> FP32."""
    u = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def unpack(params: np.ndarray) -> dict:
    out, k = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(params[k:k + n], dtype=np.float64).reshape(shape)
        k += n
    return out


def _silu(a):
    return a / (1.0 + np.exp(-a))


def _dsilu(a):
    s = 1.0 / (1.0 + np.exp(-a))
    return s * (1.0 + a * (1.0 - s))


def _r(v, on):
    return bf16(v).astype(np.float64) if on else v


def forward(params: np.ndarray, norm: np.ndarray, x: np.ndarray, keep=False, round_bf16=True,
            round_act=False):
    p = unpack(bf16(params) if round_bf16 else np.asarray(params, np.float64))
    h0 = _r((np.asarray(x, np.float64) - norm[:F]) * norm[F:], round_act)
    a1 = h0 @ p["W1"].T + p["b1"]
    h1 = _r(_silu(a1), round_act)
    a2 = h1 @ p["W2"].T + p["b2"]
    h2 = _r(_silu(a2), round_act)
    a3 = h2 @ p["W3"].T + p["b3"]
    h3 = _r(_silu(a3), round_act)
    z = h3 @ p["W4"] + p["b4"][0]
    if keep:
        return z, (p, h0, a1, h1, a2, h2, a3, h3)
    return z


def loss_grad(params: np.ndarray, norm: np.ndarray, x: np.ndarray, y: np.ndarray,
              round_bf16=True, round_act=False):
    """Mean BCE-with-logits and its gradient w.r.t. the (BF16-rounded)
    parameters, flat in the parameter order."""
    z, (p, h0, a1, h1, a2, h2, a3, h3) = forward(params, norm, x, keep=True,
                                                 round_bf16=round_bf16, round_act=round_act)
    n = len(z)
    y = np.asarray(y, np.float64)
    loss = np.mean(np.maximum(z, 0.0) - y * z + np.log1p(np.exp(-np.abs(z))))
    dz = (1.0 / (1.0 + np.exp(-z)) - y) / n
    g = {"W4": h3.T @ dz, "b4": np.array([dz.sum()])}
    ds = [_r(_dsilu(a), round_act) for a in (a1, a2, a3)]
    d3 = _r(np.outer(dz, p["W4"]) * ds[2], round_act)
    g["W3"], g["b3"] = d3.T @ h2, d3.sum(0)
    d2 = _r((d3 @ p["W3"]) * ds[1], round_act)
    g["W2"], g["b2"] = d2.T @ h1, d2.sum(0)
    d1 = _r((d2 @ p["W2"]) * ds[0], round_act)
    g["W1"], g["b1"] = d1.T @ h0, d1.sum(0)
    flat = np.concatenate([g[name].ravel() for name, _ in SIZES])
    return loss, flat


def init_params(seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    parts = []
    for name, shape in SIZES:
        if name.startswith("W"):
            fan_in = shape[-1] if len(shape) == 2 else H
            parts.append(rng.uniform(-1, 1, size=shape) * np.sqrt(6.0 / fan_in))
        else:
            parts.append(rng.normal(0, 0.1, size=shape))
    return np.concatenate([q.ravel() for q in parts]).astype(np.float32)
