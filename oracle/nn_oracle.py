"""CPU oracle of the learned path guide (torch, float64).  TEST
INFRASTRUCTURE ONLY.

The learned guide has no counterpart in the reference renderer, so its
oracle is this restatement of the network the GPU runs (csrc/nn.cuh,
csrc/nn.cu): input encoding, 64-64-64-64-48 ReLU MLP without biases, the
post-processing into an 8-lobe von Mises-Fisher mixture plus a BSDF
selection probability c = c_lo + (c_hi - c_lo) sigmoid(logit), and the
training loss
    L = -sum_r W_r log(c_r p_bsdf,r + (1 - c_r) q_r(wi_r)) / sum_r W_r
with W = T (the KL divergence) or W = T^2 (the chi-square divergence, the
renderer's default: its gradient is the gradient of the estimator's second
moment up to a positive factor).
Rounding to bfloat16 happens where the GPU rounds (weights, input features,
hidden activations); everything else is float64.  Gradients come from
autograd with the rounding treated as the identity.
"""
from __future__ import annotations

import math

import numpy as np
import torch

LOBES = 8
SHAPES = [(64, 64), (64, 64), (64, 64), (64, 48)]


def split_weights(w: np.ndarray):
    out, off = [], 0
    for i, o in SHAPES:
        out.append(w[off:off + i * o].reshape(i, o))
        off += 64 * 64 if (i, o) == (64, 64) else i * o
    return out


def bf16(x: torch.Tensor) -> torch.Tensor:
    """Round to bfloat16 (nearest even), gradient passes straight through."""
    r = x.to(torch.float32).to(torch.bfloat16).to(x.dtype)
    return x + (r - x).detach()


BLOB_BINS = 6


def one_blob(s: torch.Tensor, wrap: bool) -> torch.Tensor:
    """s in [0, 1] over BLOB_BINS Gaussian bins (sigma = 1 / BLOB_BINS,
    centres (b + 1/2) / BLOB_BINS); wrap: periodic s (an azimuth)."""
    c = (torch.arange(BLOB_BINS, dtype=torch.float64) + 0.5) / BLOB_BINS
    d = (s[:, None] - c[None, :]).abs()
    if wrap:
        d = torch.minimum(d, 1.0 - d)
    z = d * BLOB_BINS
    return torch.exp(-0.5 * z * z)


def features(pos_n: torch.Tensor, n: torch.Tensor, wo: torch.Tensor, encoding: int = 0) -> torch.Tensor:
    """64 inputs.  encoding 0: sin/cos(2^k pi x) for the 3 normalised
    coordinates and 8 octaves (feature j < 48: axis j // 16, octave
    (j // 2) % 8, cos when j is odd), normal, wo, 1, zeros.  encoding 1: the
    same at 6 octaves (j < 36: axis j // 12, octave (j % 12) // 2), then the
    one-blob encodings of the normal's cos theta ((z + 1) / 2) and phi
    (atan2(y, x) / 2 pi + 1/2, periodic) and of wo's, 6 bins each, then 1."""
    B = pos_n.shape[0]
    if encoding == 1:
        f = torch.zeros(B, 64, dtype=torch.float64)
        for j in range(36):
            c, k = j // 12, (j % 12) >> 1
            a = pos_n[:, c] * (2 ** k) * math.pi
            f[:, j] = torch.cos(a) if (j & 1) else torch.sin(a)
        col = 36
        for v in (n, wo):
            f[:, col:col + BLOB_BINS] = one_blob(0.5 * (v[:, 2] + 1.0), False)
            col += BLOB_BINS
            f[:, col:col + BLOB_BINS] = one_blob(torch.atan2(v[:, 1], v[:, 0]) / (2 * math.pi) + 0.5, True)
            col += BLOB_BINS
        f[:, col] = 1.0
        return f
    f = torch.zeros(B, 64, dtype=torch.float64)
    for j in range(48):
        c, k = j >> 4, (j >> 1) & 7
        a = pos_n[:, c] * (2 ** k) * math.pi
        f[:, j] = torch.cos(a) if (j & 1) else torch.sin(a)
    f[:, 48:51] = n
    f[:, 51:54] = wo
    f[:, 54] = 1.0
    return f


def forward_raw(weights: np.ndarray, pos_n, n, wo, encoding: int = 0):
    Ws = [bf16(torch.tensor(w, dtype=torch.float64)) for w in split_weights(weights)]
    x = bf16(features(pos_n, n, wo, encoding))
    for l in range(3):
        x = bf16(torch.relu(x @ Ws[l]))
    return x @ Ws[3]


def postprocess(raw: torch.Tensor, c_lo: float = 0.1, c_hi: float = 0.9):
    mu = raw[:, 0:24].reshape(-1, LOBES, 3)
    mu = mu / mu.norm(dim=2, keepdim=True).clamp_min(1e-20)
    kappa = (torch.nn.functional.softplus(raw[:, 24:32]) + 0.1).clamp(max=5000.0)
    w = torch.softmax(raw[:, 32:40], dim=1)
    c = c_lo + (c_hi - c_lo) * torch.sigmoid(raw[:, 40])
    return mu, kappa, w, c


def vmf_pdf(mu, kappa, wi):
    dot = (mu * wi[:, None, :]).sum(-1)
    norm = kappa / (2 * math.pi * (-torch.expm1(-2 * kappa)))
    return norm * torch.exp(kappa * (dot - 1))


def params41(raw: torch.Tensor) -> torch.Tensor:
    mu, kappa, w, c = postprocess(raw)
    per = torch.cat([mu, kappa[..., None], w[..., None]], dim=2).reshape(-1, 40)
    return torch.cat([per, c[:, None]], dim=1)


def normalise(pos, lo, hi):
    lo = torch.tensor(lo, dtype=torch.float64)
    hi = torch.tensor(hi, dtype=torch.float64)
    return (pos - lo) / (hi - lo).clamp_min(1e-6)


def forward(weights: np.ndarray, lo, hi, inputs: np.ndarray, encoding: int = 0) -> np.ndarray:
    """inputs (n, 9): position, normal, wo -> (n, 41) mixture parameters."""
    x = torch.tensor(inputs, dtype=torch.float64)
    raw = forward_raw(weights, normalise(x[:, 0:3], lo, hi), x[:, 3:6], x[:, 6:9], encoding)
    return params41(raw).numpy()


def loss_and_grad(weights: np.ndarray, lo, hi, records: np.ndarray, divergence: str = "kl",
                  c_lo: float = 0.1, c_hi: float = 0.9, encoding: int = 0):
    """records (n, 16): pos, normal, wo, wi, p_bsdf, T, 0, 0.  divergence
    "kl" weighs a record by T, "chi2" by T^2; c in [c_lo, c_hi]."""
    r = torch.tensor(records, dtype=torch.float64)
    W = torch.tensor(weights, dtype=torch.float64, requires_grad=True)
    Ws, off = [], 0
    for i, o in SHAPES:
        Ws.append(bf16(W[off:off + i * o].reshape(i, o)))
        off += i * o
    x = bf16(features(normalise(r[:, 0:3], lo, hi), r[:, 3:6], r[:, 6:9], encoding))
    for l in range(3):
        x = bf16(torch.relu(x @ Ws[l]))
    raw = x @ Ws[3]
    mu, kappa, w, c = postprocess(raw, c_lo, c_hi)
    wi = r[:, 9:12]
    q = (w * vmf_pdf(mu, kappa, wi)).sum(1)
    m = (c * r[:, 12] + (1 - c) * q).clamp_min(1e-20)
    T = r[:, 13] ** 2 if divergence == "chi2" else r[:, 13]
    T = T / T.sum()
    loss = -(T * torch.log(m)).sum()
    loss.backward()
    return float(loss.detach()), W.grad.numpy()
