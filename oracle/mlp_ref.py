"""CPU oracle of the learned proposal's network -- TEST INFRASTRUCTURE ONLY.

The reference has no learned component, so this is not a restatement of
reference code: it is the float64 numpy statement of the network that the
CUDA kernels (mdet_gb300/csrc/learned.cu) train, used by the tests to check
the forward pass, the contrastive loss and every gradient -- in float64 with
FP32 activations (the network's definition) and in the form the
tensor-core kernels compute (BF16 GEMM operands: embed_bf16,
loss_and_grad_bf16).

Network: x' = (tnf - mu) * scale; h1 = gelu(x' W1^T + b1) (256);
h2 = gelu(h1 W2^T + b2) (128); z = h2 W3^T + b3 (64).  Weights are read
rounded to BF16 (round to nearest even) wherever a product uses them; the
gradient flows straight through the rounding to the FP32 master weights.
Loss over pairs (a, b) with e = ||z_a - z_b||:
  y * relu(e - m_pos)^2 + (1 - y) * relu(m_neg - e)^2, averaged over pairs.
"""
from __future__ import annotations

import math

import numpy as np

IN, H1, H2, OUT = 136, 256, 128, 64
W1 = 0
B1 = W1 + H1 * IN
W2 = B1 + H1
B2 = W2 + H2 * H1
W3 = B2 + H2
B3 = W3 + OUT * H2
MU = B3 + OUT
SCALE = MU + IN
TAU = SCALE + 1
NPARAM = TAU + 1
NTRAIN = MU

_erf = np.vectorize(math.erf, otypes=[np.float64])


def bf16_round(w: np.ndarray) -> np.ndarray:
    """float32 -> nearest-even BF16 value, returned as float64."""
    u = np.ascontiguousarray(w, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def _gelu(z):
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def _gelu_grad(z):
    return 0.5 * (1.0 + _erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def unpack(p: np.ndarray, rounded: bool = True):
    p = np.asarray(p)
    r = bf16_round if rounded else (lambda a: np.asarray(a, np.float64))
    return {
        "W1": r(p[W1:B1]).reshape(H1, IN), "b1": p[B1:W2].astype(np.float64),
        "W2": r(p[W2:B2]).reshape(H2, H1), "b2": p[B2:W3].astype(np.float64),
        "W3": r(p[W3:B3]).reshape(OUT, H2), "b3": p[B3:MU].astype(np.float64),
        "mu": p[MU:SCALE].astype(np.float64), "scale": float(p[SCALE]),
    }


def forward(p: np.ndarray, tnf: np.ndarray, rounded: bool = True):
    w = unpack(p, rounded)
    x = (np.asarray(tnf, np.float64) - w["mu"]) * w["scale"]
    z1 = x @ w["W1"].T + w["b1"]
    h1 = _gelu(z1)
    z2 = h1 @ w["W2"].T + w["b2"]
    h2 = _gelu(z2)
    z3 = h2 @ w["W3"].T + w["b3"]
    return {"x": x, "z1": z1, "h1": h1, "z2": z2, "h2": h2, "z3": z3, "w": w}


def embed(p: np.ndarray, tnf: np.ndarray) -> np.ndarray:
    return forward(p, tnf)["z3"]


def embed_bf16(p: np.ndarray, tnf: np.ndarray) -> np.ndarray:
    """The inference form: the inputs of every layer (the centred, scaled
    rows and the two hidden activations) rounded to BF16 as well, float64
    sums otherwise."""
    w = unpack(p, True)
    x = bf16_round((np.asarray(tnf, np.float64) - w["mu"]) * w["scale"])
    h1 = bf16_round(_gelu(x @ w["W1"].T + w["b1"]))
    h2 = bf16_round(_gelu(h1 @ w["W2"].T + w["b2"]))
    return h2 @ w["W3"].T + w["b3"]


def loss_and_grad(p: np.ndarray, x: np.ndarray, pairs: np.ndarray, labels: np.ndarray, m_pos: float,
                  m_neg: float, rounded: bool = True):
    """Mean pair loss and its gradient (NTRAIN entries: W1 b1 W2 b2 W3 b3)."""
    pairs = np.asarray(pairs, np.int64).reshape(-1, 2)
    y = np.asarray(labels, np.float64)
    npairs = pairs.shape[0]
    rows = np.concatenate([pairs[:, 0], pairs[:, 1]])
    f = forward(p, np.asarray(x)[rows], rounded)
    w = f["w"]
    z = f["z3"]
    d = z[:npairs] - z[npairs:]
    e = np.sqrt((d * d).sum(1))
    up = np.maximum(e - m_pos, 0.0)
    dn = np.maximum(m_neg - e, 0.0)
    loss = float((y * up * up + (1 - y) * dn * dn).mean())
    dl = (2 * y * up - 2 * (1 - y) * dn) / npairs
    fac = np.where(e > 1e-12, dl / np.maximum(e, 1e-300), 0.0)
    d3 = np.concatenate([fac[:, None] * d, -fac[:, None] * d])
    g = np.zeros(NTRAIN)
    g[W3:B3] = (d3.T @ f["h2"]).ravel()
    g[B3:MU] = d3.sum(0)
    d2 = (d3 @ w["W3"]) * _gelu_grad(f["z2"])
    g[W2:B2] = (d2.T @ f["h1"]).ravel()
    g[B2:W3] = d2.sum(0)
    d1 = (d2 @ w["W2"]) * _gelu_grad(f["z1"])
    g[W1:B1] = (d1.T @ f["x"]).ravel()
    g[B1:W2] = d1.sum(0)
    return loss, g


def loss_and_grad_bf16(p: np.ndarray, x: np.ndarray, pairs: np.ndarray, labels: np.ndarray, m_pos: float,
                       m_neg: float):
    """The same loss and gradient as the tensor-core training pass computes
    them: every GEMM operand rounded to BF16 -- the layer inputs in the
    forward pass (as embed_bf16), and in the backward pass the output
    gradients that meet a weight matrix or an activation (dz3, dz2, dz1) --
    with float64 sums otherwise; the bias gradients sum the unrounded
    output gradients."""
    pairs = np.asarray(pairs, np.int64).reshape(-1, 2)
    y = np.asarray(labels, np.float64)
    npairs = pairs.shape[0]
    rows = np.concatenate([pairs[:, 0], pairs[:, 1]])
    w = unpack(p, True)
    xr = bf16_round((np.asarray(x, np.float64)[rows] - w["mu"]) * w["scale"])
    z1 = xr @ w["W1"].T + w["b1"]
    h1 = bf16_round(_gelu(z1))
    z2 = h1 @ w["W2"].T + w["b2"]
    h2 = bf16_round(_gelu(z2))
    z = h2 @ w["W3"].T + w["b3"]
    d = z[:npairs] - z[npairs:]
    e = np.sqrt((d * d).sum(1))
    up = np.maximum(e - m_pos, 0.0)
    dn = np.maximum(m_neg - e, 0.0)
    loss = float((y * up * up + (1 - y) * dn * dn).mean())
    dl = (2 * y * up - 2 * (1 - y) * dn) / npairs
    fac = np.where(e > 1e-12, dl / np.maximum(e, 1e-300), 0.0)
    d3 = np.concatenate([fac[:, None] * d, -fac[:, None] * d])
    d3r = bf16_round(d3)
    g = np.zeros(NTRAIN)
    g[W3:B3] = (d3r.T @ h2).ravel()
    g[B3:MU] = d3.sum(0)
    d2 = (d3r @ w["W3"]) * _gelu_grad(z2)
    d2r = bf16_round(d2)
    g[W2:B2] = (d2r.T @ h1).ravel()
    g[B2:W3] = d2.sum(0)
    d1 = (d2r @ w["W2"]) * _gelu_grad(z1)
    g[W1:B1] = (bf16_round(d1).T @ xr).ravel()
    g[B1:W2] = d1.sum(0)
    return loss, g
