"""TEST INFRASTRUCTURE ONLY — numpy restatement of the learned troubled-point predictor's network.

The checker of the library's tensor-core kernels (hypercloudcore.jl_gb300/csrc/hcc_learn.cu): forward pass,
weighted binary cross-entropy and its gradient, with the library's rounding points mirrored — the normalised
features, W1, W2, the layer-1 activations and the backpropagated pre-activation gradients dZ2, dZ1 are rounded to
BF16 (round to nearest even) exactly where the kernels stage them as tensor-core operands; every product is
accumulated here in FP64 (the kernels accumulate in FP32 tensor memory), so the two agree to FP32 accumulation
error. The predictor has no counterpart in the reference (its MOOD loop is src/TimeStepping/MOOD.jl:375-405).

Parameter layout (flat, FP32): W1[64][24], b1[64], W2[64][64], b2[64], w3[64], b3; norm = mean[24], inv_std[24].
"""
from __future__ import annotations

import math

import numpy as np

NF, NH = 24, 64
OFF_W1 = 0
OFF_B1 = OFF_W1 + NH * NF
OFF_W2 = OFF_B1 + NH
OFF_B2 = OFF_W2 + NH * NH
OFF_W3 = OFF_B2 + NH
OFF_B3 = OFF_W3 + NH
NPARAMS = OFF_B3 + 1

try:
    from scipy.special import erf as _erf
except ImportError:  # pragma: no cover
    _erf = np.vectorize(math.erf, otypes=[np.float64])


GATE = np.float32(1e-6)


def gated(X) -> np.ndarray:
    """Rows the kernels predict untroubled without the network: every quantity's relative stencil range (features
    0, 6, 12, 18) is at most GATE."""
    X = np.asarray(X, dtype=np.float32)
    return X[:, [0, 6, 12, 18]].max(axis=1) <= GATE


def bf16(x) -> np.ndarray:
    """Round FP32 values to BF16 (round to nearest, ties to even), returned as FP32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    out = (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32)
    return np.where(np.isnan(a), a, out)


# GELU x Phi(x) with Phi replaced by the kernels' odd degree-9 polynomial on [-3.2, 3.2] (held at its end values
# outside); the coefficients are the FP32 constants of the kernels.
ACT_L = np.float32(3.2)
ACT_C = [np.float32(v) for v in (0.397573032, -0.0633290983, 0.00785629494, -0.000559308202, 0.0000167396374)]


def _act_poly(x):
    xc = np.clip(np.asarray(x, dtype=np.float64), -float(ACT_L), float(ACT_L))
    u = xc * xc
    c1, c3, c5, c7, c9 = (float(c) for c in ACT_C)
    P = (((c9 * u + c7) * u + c5) * u + c3) * u + c1
    dP = ((4 * c9 * u + 3 * c7) * u + 2 * c5) * u + c3
    return xc, u, P, dP


def gelu(x):
    xc, u, P, _ = _act_poly(x)
    return np.asarray(x, dtype=np.float64) * (0.5 + xc * P)


def gelu_grad(x):
    x = np.asarray(x, dtype=np.float64)
    xc, u, P, dP = _act_poly(x)
    dphi = np.where(np.abs(x) < float(ACT_L), P + 2.0 * u * dP, 0.0)
    return (0.5 + xc * P) + x * dphi


def normal_cdf(x):
    return 0.5 * (1.0 + _erf(np.asarray(x, dtype=np.float64) / math.sqrt(2.0)))


def softplus(x):
    return np.maximum(x, 0.0) + np.log1p(np.exp(-np.abs(x)))


def unpack(params):
    p = np.asarray(params, dtype=np.float64)
    return (p[OFF_W1:OFF_B1].reshape(NH, NF), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(NH, NH),
            p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3], p[OFF_B3])


def _ident(x):
    return np.asarray(x, dtype=np.float64)


def normalised(norm, X, rnd=bf16):
    n = np.asarray(norm, dtype=np.float32)
    X = np.asarray(X, dtype=np.float32)
    return rnd((X - n[:NF]) * n[NF:])


def forward(params, norm, X, exact=False):
    """Logits and the intermediates of the backward pass. exact=True drops the BF16 rounding (FP64 throughout:
    the form whose gradient a finite-difference check pins)."""
    rnd = _ident if exact else bf16
    W1, b1, W2, b2, w3, b3 = unpack(params)
    xb = normalised(norm, X, rnd).astype(np.float64)
    z1 = xb @ rnd(W1).astype(np.float64).T + b1.astype(np.float64)
    g1 = gelu(z1)
    h1b = rnd(g1 if exact else g1.astype(np.float32)).astype(np.float64)
    z2 = h1b @ rnd(W2).astype(np.float64).T + b2.astype(np.float64)
    h2 = gelu(z2)
    logit = float(b3) + h2 @ w3.astype(np.float64)
    return logit, (xb, z1, h1b, z2, h2)


def loss_grad(params, norm, X, y, pos_weight=1.0, exact=False):
    """(mean weighted BCE, gradient in the flat parameter layout)."""
    rnd = _ident if exact else (lambda v: bf16(np.asarray(v, dtype=np.float32)))
    W1, b1, W2, b2, w3, b3 = unpack(params)
    y = np.asarray(y).astype(bool)
    B = len(y)
    logit, (xb, z1, h1b, z2, h2) = forward(params, norm, X, exact)
    p = 1.0 / (1.0 + np.exp(-logit))
    dz = np.where(y, pos_weight * (p - 1.0), p) / B
    loss = float(np.sum(np.where(y, pos_weight * softplus(-logit), softplus(logit))) / B)
    dz2b = rnd((dz[:, None] * w3.astype(np.float64)[None, :]) * gelu_grad(z2)).astype(np.float64)
    dh1 = dz2b @ rnd(W2).astype(np.float64)
    dz1b = rnd(dh1 * gelu_grad(z1)).astype(np.float64)
    g = np.zeros(NPARAMS, dtype=np.float64)
    g[OFF_W1:OFF_B1] = (dz1b.T @ xb).reshape(-1)
    g[OFF_B1:OFF_W2] = dz1b.sum(axis=0)
    g[OFF_W2:OFF_B2] = (dz2b.T @ h1b).reshape(-1)
    g[OFF_B2:OFF_W3] = dz2b.sum(axis=0)
    g[OFF_W3:OFF_B3] = h2.T @ dz
    g[OFF_B3] = dz.sum()
    return loss, g
