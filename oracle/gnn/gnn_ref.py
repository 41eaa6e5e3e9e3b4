"""Test infrastructure: NumPy restatement of the learned Newton predictor's
network, forward and backward, used as the checker for the GPU kernels.

The reference simulator has no learned predictor; its Newton initial guess
is the previous solution with the devices' state extrapolation (INITPRED,
src/maths/ni/niiter.c:29-367 with PREDICTOR undefined).  The network here
predicts, per circuit node, a correction to the linear (polynomial)
extrapolation of the node voltage to the next timepoint.  It is a
shared-weight message-passing network over the circuit graph:

    H0      = relu(bf(X) bf(Win) + bin)                     X: N x 16
    M_l     = D^-1 A H_l            (mean over graph neighbours, FP32)
    H_l+1   = relu([bf(H_l) | bf(M_l)] bf(W_l) + b_l) + H_l  l = 0, 1, 2
    out     = bf(H3) bf(Wout);  pred = out[:, 0] + bout      Wout: 64 x 16
    loss    = sum_i w_i (pred_i - y_i)^2 / (2 sum_i w_i)

bf() rounds to bfloat16 (round to nearest even) where the GPU kernels feed
a tensor-core product; every product accumulates in FP32.  The backward
pass applies the same rounding to the gradient operands of its products.

Only tests use this module.
"""
from __future__ import annotations

import numpy as np

F_IN = 16
HID = 64
OUT_W = 16
LAYERS = 3

# Arithmetic of the restatement: FP32 with bfloat16 operands (the kernels'
# arithmetic), or, with set_exact(True), FP64 without rounding (for
# finite-difference checks of the backward pass).
DT = np.float32
EXACT = False


def set_exact(on: bool) -> None:
    global DT, EXACT
    EXACT = bool(on)
    DT = np.float64 if on else np.float32


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest even), returned as float32
    (identity in exact mode)."""
    if EXACT:
        return np.asarray(x, dtype=np.float64)
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = (u + 0x7FFF + lsb) & 0xFFFF0000
    out = u.astype(np.uint32).view(np.float32)
    return np.where(np.isnan(a), a, out).astype(np.float32)


def init_params(seed: int = 0) -> dict:
    rng = np.random.default_rng(seed)

    def glorot(fan_in, fan_out):
        s = np.sqrt(2.0 / (fan_in + fan_out))
        return (rng.standard_normal((fan_in, fan_out)) * s).astype(DT)

    p = {"Win": glorot(F_IN, HID), "bin": np.zeros(HID, DT)}
    for l in range(LAYERS):
        p[f"W{l}"] = glorot(2 * HID, HID) * DT(0.5)
        p[f"b{l}"] = np.zeros(HID, DT)
    p["Wout"] = glorot(HID, OUT_W) * DT(0.1)
    p["bout"] = np.zeros(1, DT)
    return p


def mean_agg(H: np.ndarray, ptr: np.ndarray, idx: np.ndarray, dinv: np.ndarray) -> np.ndarray:
    """M[i] = dinv[i] * sum_{j in nbr(i)} H[j], FP32, neighbours in CSR order."""
    N = H.shape[0]
    M = np.zeros_like(H)
    for i in range(N):
        s = np.zeros(H.shape[1], DT)
        for q in range(ptr[i], ptr[i + 1]):
            s += H[idx[q]]
        M[i] = s * dinv[i]
    return M


def mean_agg_t(dM: np.ndarray, ptr: np.ndarray, idx: np.ndarray, dinv: np.ndarray) -> np.ndarray:
    """Adjoint of mean_agg for a symmetric neighbour structure:
    dH[j] = sum_{i in nbr(j)} dinv[i] * dM[i]."""
    N = dM.shape[0]
    dH = np.zeros_like(dM)
    for j in range(N):
        s = np.zeros(dM.shape[1], DT)
        for q in range(ptr[j], ptr[j + 1]):
            i = idx[q]
            s += dM[i] * dinv[i]
        dH[j] = s
    return dH


def forward(p: dict, X: np.ndarray, ptr, idx, dinv) -> tuple[np.ndarray, dict]:
    cache = {}
    Z0 = bf16(X) @ bf16(p["Win"]) + p["bin"]
    H = np.maximum(Z0, 0).astype(DT)
    cache["Z0"], cache["X"] = Z0, X
    for l in range(LAYERS):
        M = mean_agg(H, ptr, idx, dinv)
        U = np.concatenate([bf16(H), bf16(M)], axis=1)
        Z = (U @ bf16(p[f"W{l}"]) + p[f"b{l}"]).astype(DT)
        cache[f"H{l}"], cache[f"U{l}"], cache[f"Z{l + 1}"] = H, U, Z
        H = (np.maximum(Z, 0) + H).astype(DT)
    cache["H3"] = H
    out = (bf16(H) @ bf16(p["Wout"])).astype(DT)
    pred = out[:, 0] + p["bout"][0]
    return pred.astype(DT), cache


def loss_and_grad(p: dict, X, ptr, idx, dinv, y, w) -> tuple[float, dict, np.ndarray]:
    pred, c = forward(p, X, ptr, idx, dinv)
    W = DT(w.sum())
    r = (pred - y).astype(DT)
    loss = float((w * r * r).sum() / (2 * W))
    g = {}
    dpred = (w * r / W).astype(DT)
    dOut = np.zeros((X.shape[0], OUT_W), DT)
    dOut[:, 0] = dpred
    g["bout"] = np.array([dpred.sum()], DT)
    g["Wout"] = (bf16(c["H3"]).T @ bf16(dOut)).astype(DT)
    dH = (bf16(dOut) @ bf16(p["Wout"]).T).astype(DT)
    for l in reversed(range(LAYERS)):
        Z = c[f"Z{l + 1}"]
        dZ = (dH * (Z > 0)).astype(DT)
        g[f"W{l}"] = (c[f"U{l}"].T @ bf16(dZ)).astype(DT)
        g[f"b{l}"] = dZ.sum(axis=0).astype(DT)
        dU = (bf16(dZ) @ bf16(p[f"W{l}"]).T).astype(DT)
        dH = (dH + dU[:, :HID] + mean_agg_t(dU[:, HID:], ptr, idx, dinv)).astype(DT)
    dZ0 = (dH * (c["Z0"] > 0)).astype(DT)
    g["Win"] = (bf16(X).T @ bf16(dZ0)).astype(DT)
    g["bin"] = dZ0.sum(axis=0).astype(DT)
    return loss, g, pred


def adam(p: dict, g: dict, m: dict, v: dict, t: int, lr: float,
         b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8) -> None:
    """Adam on FP32 master weights, in place (step t counts from 1)."""
    for k in p:
        m[k] = (b1 * m[k] + (1 - b1) * g[k]).astype(DT)
        v[k] = (b2 * v[k] + (1 - b2) * g[k] * g[k]).astype(DT)
        mh = m[k] / (1 - b1 ** t)
        vh = v[k] / (1 - b2 ** t)
        p[k] = (p[k] - lr * mh / (np.sqrt(vh) + eps)).astype(DT)
