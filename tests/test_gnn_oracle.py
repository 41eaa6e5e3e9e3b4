"""CPU: the learned predictor's NumPy restatement (oracle/gnn) — its
backward pass against central finite differences in exact FP64 mode, the
bfloat16 rounding helper, and the graph / feature construction."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle", "gnn"))
import gnn_ref as R  # noqa: E402


def small_graph(n=12, seed=3):
    rng = np.random.default_rng(seed)
    nb = [set() for _ in range(n)]
    for i in range(n):
        for j in rng.choice(n, 3, replace=False):
            if j != i:
                nb[i].add(int(j))
                nb[int(j)].add(i)
    ptr = np.zeros(n + 1, np.int32)
    idx = []
    for i in range(n):
        idx += sorted(nb[i])
        ptr[i + 1] = len(idx)
    deg = np.diff(ptr)
    return ptr, np.array(idx, np.int32), np.where(deg > 0, 1.0 / np.maximum(deg, 1), 0.0)


def test_bf16_rounding_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.1415926, 0.0], np.float32)
    r = R.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                      # tie -> even mantissa
    assert r[2] == np.float32(1.0 + 2 ** -7)
    assert r[3] == -2.5
    assert abs(r[4] - 3.140625) < 1e-7
    assert r[5] == 0.0


def test_backward_matches_finite_differences():
    R.set_exact(True)
    try:
        ptr, idx, dinv = small_graph()
        n = len(ptr) - 1
        rng = np.random.default_rng(0)
        p = R.init_params(1)
        for k in p:                          # biases away from zero: relu kinks rare
            if k.startswith("b"):
                p[k] = rng.standard_normal(p[k].shape) * 0.1
        X = rng.standard_normal((n, R.F_IN))
        y = rng.standard_normal(n)
        w = rng.uniform(0.5, 1.5, n)
        loss, g, _ = R.loss_and_grad(p, X, ptr, idx, dinv, y, w)
        eps = 1e-6
        for k in ["Win", "bin", "W0", "b1", "W2", "Wout", "bout"]:
            flat = p[k].ravel()
            for t in rng.choice(flat.size, min(6, flat.size), replace=False):
                old = flat[t]
                flat[t] = old + eps
                lp, _, _ = R.loss_and_grad(p, X, ptr, idx, dinv, y, w)
                flat[t] = old - eps
                lm, _, _ = R.loss_and_grad(p, X, ptr, idx, dinv, y, w)
                flat[t] = old
                fd = (lp - lm) / (2 * eps)
                an = g[k].ravel()[t]
                assert abs(fd - an) <= 1e-6 + 1e-5 * abs(fd), (k, t, fd, an)
    finally:
        R.set_exact(False)


def test_features_and_targets():
    from ngspice_gb300 import gnn
    t = np.array([0, 1e-12, 2e-12, 3e-12, 4.5e-12, 5e-12])
    V = np.stack([np.full(3, 0.1 * k) for k in range(len(t))])
    stat = np.ones((3, 6), np.float32)
    samples = gnn.trajectory_samples(t, V, stat)
    assert len(samples) == 2
    X, y, g = samples[0]
    assert X.shape == (3, gnn.F_IN)
    assert np.all(g > 0.99)                  # 0.1 V steps: fully active
    assert np.allclose(X[:, 3], 1.5)         # r1 = 1.5p / 1p
    # straight line: the quadratic extrapolation is the linear one,
    # v3 + 1.5 * 0.1 = 0.45; v_next = 0.4 -> y = -0.05 / VOUT
    assert np.allclose(y, (0.4 - 0.45) / gnn.VOUT, atol=1e-4)


def test_node_graph_of_a_compiled_circuit(built_lib):
    """Voltage unknowns, neighbour lists and terminal counts come from the
    compiled circuit (host only, no GPU)."""
    from ngspice_gb300 import engine as E
    text = "\n".join(["* t", "vdd vdd 0 1", "va a 0 0.5",
                      "m1 y a 0 0 nch w=1u l=1u", "m2 y a vdd vdd pch w=1u l=1u",
                      "r1 y z 10", "c1 z 0 1f", ".model nch nmos level=1", ".model pch pmos level=1",
                      ".tran 1p 2p", ".end"])
    c = E.Circuit(text, host_only=True)
    g = c.node_graph()
    names = c.names()
    vn = [names[k] for k in g["vnode"]]
    assert "vdd#branch" not in vn and "va#branch" not in vn
    assert set(vn) == {"vdd", "a", "y", "z"}
    cnt = np.round(np.expm1(g["stat"])).astype(int)
    row = {nm: cnt[i] for i, nm in enumerate(vn)}
    assert row["a"][0] == 2                  # two gates
    assert row["y"][1] == 2 and row["y"][4] == 1
    assert row["vdd"][1] == 1 and row["vdd"][2] == 1 and row["vdd"][5] == 1
    assert row["z"][3] == 1 and row["z"][4] == 1
    ptr, idx = g["gptr"], g["gidx"]
    nb = {vn[i]: {vn[j] for j in idx[ptr[i]:ptr[i + 1]]} for i in range(len(vn))}
    assert "z" in nb["y"] and "y" in nb["z"]          # symmetric
    assert all(vn[i] not in nb[vn[i]] for i in range(len(vn)))
