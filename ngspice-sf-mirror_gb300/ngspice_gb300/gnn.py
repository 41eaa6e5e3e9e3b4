"""Learned Newton predictor: graph, features and training data from circuit
trajectories, and ctypes bindings of the network kernels (gnn.cu).

The network predicts, per circuit node, a correction to the polynomial
(quadratic) extrapolation of the node voltage to the next accepted
timepoint:

    v_lin  = v_n + r1 (v_n - v_{n-1}),      r1 = h_{n+1} / h_n
    v_quad = v_lin + r1 (r1 + 1) r2 (d1 - r2 d2) / (r2 + 1)
    v_next ~ v_quad + VOUT * g * pred,      g = a / (a + QUIET),
    a = |v_n - v_{n-1}| + |v_{n-1} - v_{n-2}|

Node features (16): v_n, (v_n - v_{n-1}) / VSCALE, (v_{n-1} - v_{n-2}) /
VSCALE, r1, r2 = h_n / h_{n-1}, r1 (v_n - v_{n-1}) / VSCALE, log(1 + count)
of the incident MOSFET gate, drain/source, bulk, capacitor, resistor and
source terminals (Circuit.node_graph), a constant 1, the quadratic-
extrapolation increment through the last three points r1 (r1 + 1) r2 (d1 -
r2 d2) / ((r2 + 1) VSCALE) with d1 = v_n - v_{n-1}, d2 = v_{n-1} - v_{n-2},
zeros.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import engine as E

F_IN = 16
VSCALE = 0.05
# unit of the network's correction (the residual after the quadratic
# extrapolation is millivolts; a finer unit keeps BF16 rounding of the output
# well below the convergence tolerance)
VOUT = 0.005
RATIO_MAX = 4.0
QUIET = 1e-4        # V: node activity at which the correction is halved


def lib():
    L = E.lib()
    if not getattr(L, "_gnn_typed", False):
        vp, ip, fp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_float)
        L.ngsf_gnn_param_count.restype = C.c_int
        L.ngsf_gnn_create.restype = vp
        L.ngsf_gnn_create.argtypes = [C.c_int, ip, ip]
        L.ngsf_gnn_destroy.argtypes = [vp]
        L.ngsf_gnn_set_params.argtypes = [vp, fp]
        L.ngsf_gnn_get_params.argtypes = [vp, fp]
        L.ngsf_gnn_forward.argtypes = [vp, fp, fp]
        L.ngsf_gnn_train_step.argtypes = [vp, fp, fp, fp, C.c_float, fp, fp]
        L.ngsf_gnn_gemm_test.argtypes = [fp, fp, fp, C.c_int, C.c_int, C.c_int, C.c_int]
        L._gnn_typed = True
    return L


def _f(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _i(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def param_count() -> int:
    return int(lib().ngsf_gnn_param_count())


def flatten(p: dict) -> np.ndarray:
    """Flat FP32 layout of the kernels: Win, bin, (W_l, b_l) x 3, Wout, bout."""
    parts = [p["Win"].ravel(), p["bin"]]
    for l in range(3):
        parts += [p[f"W{l}"].ravel(), p[f"b{l}"]]
    parts += [p["Wout"].ravel(), p["bout"]]
    return np.concatenate(parts).astype(np.float32)


def unflatten(flat: np.ndarray) -> dict:
    o, p = 0, {}

    def take(name, shape):
        nonlocal o
        n = int(np.prod(shape))
        p[name] = flat[o:o + n].reshape(shape).astype(np.float32)
        o += n
    take("Win", (16, 64))
    take("bin", (64,))
    for l in range(3):
        take(f"W{l}", (128, 64))
        take(f"b{l}", (64,))
    take("Wout", (64, 16))
    take("bout", (1,))
    return p


def gemm_test(A: np.ndarray, B: np.ndarray, splits: int = 1) -> np.ndarray:
    """C = bf16(A) bf16(B)^T on the tensor cores (FP32 result)."""
    A = np.ascontiguousarray(A, np.float32)
    B = np.ascontiguousarray(B, np.float32)
    M, K = A.shape
    N = B.shape[0]
    Cm = np.zeros((M, N), np.float32)
    if lib().ngsf_gnn_gemm_test(_f(A), _f(B), _f(Cm), M, N, K, splits):
        raise E.EngineError(E.last_error())
    return Cm


class Net:
    """The network's device state for one graph (ngsf_gnn_*)."""

    def __init__(self, ptr: np.ndarray, idx: np.ndarray):
        self.ptr = np.ascontiguousarray(ptr, np.int32)
        self.idx = np.ascontiguousarray(idx, np.int32)
        self.n = len(self.ptr) - 1
        h = lib().ngsf_gnn_create(self.n, _i(self.ptr), _i(self.idx))
        if not h:
            raise E.EngineError(E.last_error())
        self._h = C.c_void_p(h)

    def close(self):
        if self._h:
            lib().ngsf_gnn_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, flat: np.ndarray):
        flat = np.ascontiguousarray(flat, np.float32)
        if lib().ngsf_gnn_set_params(self._h, _f(flat)):
            raise E.EngineError(E.last_error())

    def params(self) -> np.ndarray:
        out = np.zeros(param_count(), np.float32)
        if lib().ngsf_gnn_get_params(self._h, _f(out)):
            raise E.EngineError(E.last_error())
        return out

    def forward(self, X: np.ndarray) -> np.ndarray:
        X = np.ascontiguousarray(X, np.float32)
        pred = np.zeros(self.n, np.float32)
        if lib().ngsf_gnn_forward(self._h, _f(X), _f(pred)):
            raise E.EngineError(E.last_error())
        return pred

    def train_step(self, X, y, w, lr: float, want_grads: bool = False):
        X = np.ascontiguousarray(X, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        w = np.ascontiguousarray(w, np.float32)
        loss = np.zeros(1, np.float32)
        g = np.zeros(param_count(), np.float32) if want_grads else None
        if lib().ngsf_gnn_train_step(self._h, _f(X), _f(y), _f(w), float(lr), _f(loss),
                                     _f(g) if g is not None else None):
            raise E.EngineError(E.last_error())
        return float(loss[0]), g


# ---------------------------------------------------------------------------
# circuit graph and features
# ---------------------------------------------------------------------------
def features(v3: np.ndarray, v2: np.ndarray, v1: np.ndarray, h_next: float, h_n: float,
             h_prev: float, stat: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Features at step n for the prediction of n+1, and the linear
    extrapolation (the transient kernel computes the same, predict.cuh).
    v3 = v_n, v2 = v_{n-1}, v1 = v_{n-2} (voltage nodes); stat = the
    log(1 + terminal counts) of Circuit.node_graph()."""
    r1 = min(h_next / h_n, RATIO_MAX) if h_n > 0 else 1.0
    r2 = min(h_n / h_prev, RATIO_MAX) if h_prev > 0 else 1.0
    d1 = v3 - v2
    X = np.zeros((len(v3), F_IN), np.float32)
    X[:, 0] = v3
    X[:, 1] = d1 / VSCALE
    X[:, 2] = (v2 - v1) / VSCALE
    X[:, 3] = r1
    X[:, 4] = r2
    X[:, 5] = r1 * d1 / VSCALE
    X[:, 6:12] = stat
    X[:, 12] = 1.0
    X[:, 13] = r1 * (r1 + 1.0) * r2 * (d1 - r2 * (v2 - v1)) / ((r2 + 1.0) * VSCALE)
    vlin = v3 + r1 * d1
    return X, vlin.astype(np.float64)


def quadratic(X: np.ndarray, vlin: np.ndarray) -> np.ndarray:
    """The quadratic extrapolation the network corrects: the linear one plus
    the quadratic increment (feature 13, in units of VSCALE)."""
    return vlin + VSCALE * X[:, 13].astype(np.float64)


def quadratic_exact(v3, v2, v1, h_next: float, h_n: float, h_prev: float) -> np.ndarray:
    """The parabola through the last three accepted points at the next time,
    in FP64 (the engine's pred_guess arithmetic, ratios capped at 4)."""
    r1 = min(h_next / h_n, RATIO_MAX) if h_n > 0 else 1.0
    r2 = min(h_n / h_prev, RATIO_MAX) if h_prev > 0 else 1.0
    d1, d2 = v3 - v2, v2 - v1
    return v3 + r1 * d1 + r1 * (r1 + 1.0) * r2 * (d1 - r2 * d2) / (r2 + 1.0)


def gate(v3: np.ndarray, v2: np.ndarray, v1: np.ndarray) -> np.ndarray:
    """Weight of the network's correction at each node: a / (a + QUIET)
    with a = |v_n - v_{n-1}| + |v_{n-1} - v_{n-2}| (the transient kernel
    applies the same, predict.cuh)."""
    a = np.abs(v3 - v2) + np.abs(v2 - v1)
    return a / (a + QUIET)


def trajectory_samples(t: np.ndarray, V: np.ndarray, stat: np.ndarray,
                       stride: int = 1) -> list[tuple[np.ndarray, np.ndarray, np.ndarray]]:
    """(X, y, g) training triples from accepted points t[k], V[k, node]:
    y = (v_{n+1} - v_quad) / VOUT, g the correction's gate."""
    out = []
    for n in range(3, len(t) - 1, stride):
        h_next, h_n, h_prev = t[n + 1] - t[n], t[n] - t[n - 1], t[n - 1] - t[n - 2]
        X, vlin = features(V[n], V[n - 1], V[n - 2], h_next, h_n, h_prev, stat)
        y = ((V[n + 1] - quadratic_exact(V[n], V[n - 1], V[n - 2], h_next, h_n, h_prev))
             / VOUT).astype(np.float32)
        out.append((X, y, gate(V[n], V[n - 1], V[n - 2]).astype(np.float32)))
    return out
