"""CPU oracle of the estimator MLP -- TEST INFRASTRUCTURE ONLY.

numpy forward and backward of the network of wukonggpu_gb300/csrc/wk_mlp.cu
(x = [48 features | 32-d embedding] -> 3 x 256 GELU -> 1, mean squared
error), with values rounded to bfloat16 exactly where the GPU path stores
them (inputs, weights, activations, back-propagated pre-activation
gradients, the output gradient) and float32 everywhere else, so that the
GPU gradients can be checked against it.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

N_IN, N_EMB, H = 48, 32, 256
X = N_IN + N_EMB


def bf16(a: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float32."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def unpack(params: np.ndarray, n_ids: int):
    at = 0
    shapes = [(H, X), (H, H), (H, H), (1, H)]
    W = []
    for sh in shapes:
        n = sh[0] * sh[1]
        W.append(params[at:at + n].reshape(sh))
        at += n
    b = []
    for n in (H, H, H, 64):
        b.append(params[at:at + n])
        at += n
    emb = params[at:at + (n_ids + 1) * N_EMB].reshape(n_ids + 1, N_EMB)
    return W, b, emb


def gelu(z):
    return (0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))).astype(np.float32)


def gelu_grad(z):
    return (0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)).astype(np.float32)


def forward_backward(params: np.ndarray, n_ids: int, feats, pids, target):
    """Loss and the gradient of every parameter, in the parameter layout."""
    W, b, emb = unpack(np.asarray(params, np.float32), n_ids)
    Wb = [bf16(w) for w in W]
    M = len(target)
    p = np.clip(np.asarray(pids), 0, n_ids)
    x0 = bf16(np.concatenate([np.asarray(feats, np.float32), emb[p]], axis=1))
    zs, hs = [], [x0]
    h = x0
    for layer in range(3):
        z = (h @ Wb[layer].T + b[layer]).astype(np.float32)
        zs.append(z)
        h = bf16(gelu(z))
        hs.append(h)
    y = (h @ Wb[3].T)[:, 0] + b[3][0]
    d = y - np.asarray(target, np.float32)
    loss = float(np.mean(d * d))
    dy = bf16((2.0 * d / M).astype(np.float32))[:, None]          # [M x 1]
    gW = [None] * 4
    gb = [None] * 4
    gW[3] = (dy.T @ hs[3]).astype(np.float32)
    gb[3] = np.zeros(64, np.float32)
    gb[3][0] = dy.sum()
    dh = (dy @ Wb[3]).astype(np.float32)
    for layer in (2, 1, 0):
        dz = bf16(dh * gelu_grad(zs[layer]))
        gW[layer] = (dz.T @ hs[layer]).astype(np.float32)
        gb[layer] = dz.sum(axis=0).astype(np.float32)
        dh = (dz @ Wb[layer]).astype(np.float32)
    gemb = np.zeros_like(emb)
    np.add.at(gemb, p, dh[:, N_IN:])
    grads = np.concatenate([g.reshape(-1) for g in gW] + [g.reshape(-1) for g in gb] + [gemb.reshape(-1)])
    return loss, grads.astype(np.float32)
