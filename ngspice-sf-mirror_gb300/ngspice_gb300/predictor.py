"""Learned Newton predictor: trajectories from the plain simulator, training
on the GPU with the network kernels (gnn.cu), and its use by the engine.

    texts = [netlists.random_logic(n_transistors=300, seed=s, tstop="200p")
             for s in range(8)]
    data = collect(texts)                 # plain GPU runs, every node voltage
    params, log = train(data, steps=400)  # tensor-core forward/backward, Adam
    c = engine.Circuit(text); c.set_predictor(2, params); engine.run([c])

A training step feeds one accepted timestep of every training circuit at
once: the circuits' graphs are joined into one block-diagonal graph, and
each step draws a timestep per circuit.
"""
from __future__ import annotations

import numpy as np

from . import engine as E
from . import gnn

# oracle-independent initial weights (Glorot, small decoder)
def init_params(seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)

    def glorot(fi, fo, scale=1.0):
        s = np.sqrt(2.0 / (fi + fo)) * scale
        return (rng.standard_normal((fi, fo)) * s).astype(np.float32)
    p = {"Win": glorot(16, 64), "bin": np.zeros(64, np.float32)}
    for l in range(3):
        p[f"W{l}"] = glorot(128, 64, 0.5)
        p[f"b{l}"] = np.zeros(64, np.float32)
    p["Wout"] = glorot(64, 16, 0.1)
    p["bout"] = np.zeros(1, np.float32)
    return gnn.flatten(p)


def collect(texts: list[str], outcap: int = 4096) -> list[dict]:
    """Run each netlist with the plain simulator (no predictor) and keep
    the accepted points of every voltage node with the node graph."""
    data = []
    circuits = []
    for text in texts:
        host = E.Circuit(text, host_only=True)
        g = host.node_graph()
        names = host.names()
        probes = [names[k] for k in g["vnode"]]
        c = E.Circuit(text, probes=probes, outcap=outcap)
        circuits.append(c)
        data.append({"graph": g, "text": text})
    E.run(circuits)
    for c, d in zip(circuits, data):
        r = c.results()
        if r[E.R_STATUS] != 0:
            raise E.EngineError(f"training run failed with status {r[E.R_STATUS]}")
        t, V = c.points()
        d["t"], d["V"] = t, V
        d["samples"] = gnn.trajectory_samples(t, V, d["graph"]["stat"])
    return data


def _union_graph(graphs: list[dict]) -> tuple[np.ndarray, np.ndarray, list[int]]:
    ptr, idx, offs = [0], [], []
    base = 0
    for g in graphs:
        offs.append(base)
        gp, gi = g["gptr"], g["gidx"]
        for v in range(len(gp) - 1):
            idx.extend((gi[gp[v]:gp[v + 1]] + base).tolist())
            ptr.append(len(idx))
        base += len(gp) - 1
    return np.array(ptr, np.int32), np.array(idx, np.int32), offs


def train(data: list[dict], steps: int = 400, lr: float = 2e-3, seed: int = 0,
          params: np.ndarray | None = None) -> tuple[np.ndarray, list[float]]:
    """Train on the GPU; returns the FP32 parameters and the loss history."""
    rng = np.random.default_rng(seed)
    ptr, idx, offs = _union_graph([d["graph"] for d in data])
    net = gnn.Net(ptr, idx)
    net.set_params(params if params is not None else init_params(seed))
    n = len(ptr) - 1
    losses = []
    for it in range(steps):
        # the correction is applied as g * pred: minimise sum (g p - y)^2 =
        # sum g^2 (p - y / g)^2, i.e. weights g^2 and targets y / g
        X = np.zeros((n, gnn.F_IN), np.float32)
        y = np.zeros(n, np.float32)
        w = np.zeros(n, np.float32)
        for d, o in zip(data, offs):
            Xs, ys, gs = d["samples"][rng.integers(len(d["samples"]))]
            X[o:o + len(ys)] = Xs
            safe = np.maximum(gs, 1e-6)
            y[o:o + len(ys)] = np.where(gs > 1e-6, ys / safe, 0.0)
            w[o:o + len(ys)] = gs * gs
        if not w.sum() > 0:
            continue
        cur_lr = lr * (0.1 ** (it / max(steps, 1)))
        loss, _ = net.train_step(X, y, w, cur_lr)
        losses.append(loss)
    out = net.params()
    net.close()
    return out, losses


def evaluate(texts: list[str], params: np.ndarray | None, kinds=(0, 1, 2)) -> dict:
    """Newton iterations and accepted steps of the same netlists without a
    predictor (0), with the linear guess (1) and with the network (2)."""
    res = {}
    for kind in kinds:
        cs = [E.Circuit(t) for t in texts]
        for c in cs:
            if kind:
                c.set_predictor(kind, params if kind == 2 else None)
        sec = E.run(cs)
        rows = np.array([c.results() for c in cs])
        res[kind] = {
            "seconds": sec,
            "status": rows[:, E.R_STATUS].tolist(),
            "accepted": int(rows[:, E.R_ACCEPTED].sum()),
            "iterations": int(rows[:, E.R_NUMITER].sum()),
            "tran_iterations": int(rows[:, E.R_TRANITER].sum()),
            "guesses": int(rows[:, E.R_GUESSES].sum()),
            "first_iteration": int(rows[:, E.R_GUESS1].sum()),
            "fallbacks": int(rows[:, E.R_FALLBACKS].sum()),
        }
        res[kind]["iterations_per_step"] = res[kind]["tran_iterations"] / max(
            res[kind]["accepted"], 1)
    return res
